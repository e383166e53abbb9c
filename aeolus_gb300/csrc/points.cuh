// Point-set (e.g. icosahedral geodesic) transform: dense real basis product.
//
// Real basis columns, m-major: for each order m the cosine columns
// Pbar_lm cos(m lon) for l = m..L, then (m > 0) the sine columns
// Pbar_lm sin(m lon); (L+1)^2 columns in all, stored column-major
// (point index fastest).  With that basis the reference's complex forms
// (fast_geodesic_sh.py:68-107) become real GEMMs:
//   synthesis  f = B v,  v[cos(l,0)] = Re a_l0, v[cos(l,m)] = 2 Re a_lm,
//                        v[sin(l,m)] = -2 Im a_lm;
//   analysis   c = B^T (w f),  a_lm = c[cos(l,m)] - i c[sin(l,m)].
#pragma once

#include "common.cuh"

namespace aeolus {

__host__ __device__ inline long col_base(int m, int L) { return m == 0 ? 0 : 2 * tri_off(m, L) - (L + 1); }
__host__ __device__ inline long col_cos(int l, int m, int L) { return col_base(m, L) + (l - m); }
__host__ __device__ inline long col_sin(int l, int m, int L) { return col_base(m, L) + (L + 1 - m) + (l - m); }

// V[(b*NF + f) * ncol + col] from Derive columns (one thread per (b, l, m)).
template <class Derive>
__global__ void derive_cols_kernel(int L, int batch, long ncol, double* __restrict__ V, Derive d) {
  constexpr int NF = Derive::NF;
  const long nlm = (long)(L + 1) * (L + 2) / 2;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nlm * batch) return;
  const int b = (int)(idx / nlm);
  long r = idx - (long)b * nlm;
  // r enumerates the m-major triangle: find m with tri_off(m) <= r < tri_off(m+1)
  int m = 0;
  while (tri_off(m + 1, L) <= r) ++m;
  const int l = m + (int)(r - tri_off(m, L));
  double2 v[NF];
  d.column(b, l, m, v);
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    double* col = V + ((long)b * NF + f) * ncol;
    if (m == 0) {
      col[col_cos(l, 0, L)] = v[f].x;
    } else {
      col[col_cos(l, m, L)] = 2.0 * v[f].x;
      col[col_sin(l, m, L)] = -2.0 * v[f].y;
    }
  }
}

// Pointwise op over points.  in: Gr[b * in_b + f * in_f + p];
// out: Out[b * out_b + f * out_f + p] = scale_p * out_f with scale_p = w_p
// (analysis input) or 1 (grid output).
template <class Pw>
__global__ void points_pointwise_kernel(long npts, int batch, const double* __restrict__ Gr, long in_b, long in_f,
                                        double* __restrict__ Out, long out_b, long out_f,
                                        const double* __restrict__ coslat, const double* __restrict__ fgrid,
                                        const double* __restrict__ w, unsigned* status, Pw pw) {
  constexpr int NIN = Pw::NIN, NOUT = Pw::NOUT;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= npts * batch) return;
  const int b = (int)(idx / npts);
  const long p = idx - (long)b * npts;
  double in[NIN], out[NOUT];
#pragma unroll
  for (int f = 0; f < NIN; ++f) in[f] = Gr[(long)b * in_b + (long)f * in_f + p];
  const unsigned bits = pw(coslat[p], fgrid[p], in, out);
  if (status && bits) atomicOr(&status[b], bits);
  const double sc = w ? w[p] : 1.0;
#pragma unroll
  for (int f = 0; f < NOUT; ++f) Out[(long)b * out_b + (long)f * out_f + p] = sc * out[f];
}

// a_lm from real analysis columns; one thread per (b, l, m) of the dense square.
template <class Epi>
__global__ void epilogue_cols_kernel(int L, int batch, long ncol, const double* __restrict__ C, Epi e) {
  constexpr int NF = Epi::NF;
  const long n2 = (long)(L + 1) * (L + 1);
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2 * batch) return;
  const int b = (int)(idx / n2);
  const int r = (int)(idx - (long)b * n2);
  const int l = r / (L + 1), m = r - l * (L + 1);
  if (m > l) {
    e.zero(b, l, m);
    return;
  }
  double2 acc[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    const double* col = C + ((long)b * NF + f) * ncol;
    acc[f] = make_double2(col[col_cos(l, m, L)], m == 0 ? 0.0 : -col[col_sin(l, m, L)]);
  }
  e.finish(b, l, m, acc);
}

// FP64 tiled GEMM: C[j * ldc + i] = sum_k A(i, k) * B[j * ldb + k], with
// A(i, k) = A[k * lda + i] (A_COLMAJOR) or A[i * lda + k].
template <bool A_COLMAJOR>
__global__ void __launch_bounds__(128) dgemm_kernel(long M, long N, long K, const double* __restrict__ A, long lda,
                                                   const double* __restrict__ B, long ldb,
                                                   double* __restrict__ C, long ldc) {
  constexpr int BM = 64, BN = 32, BK = 16;
  __shared__ double sA[BK][BM + 1];
  __shared__ double sB[BK][BN + 1];
  const long i0 = (long)blockIdx.x * BM, j0 = (long)blockIdx.y * BN;
  const int tid = threadIdx.x;
  const int ti = tid % 16, tj = tid / 16;  // 16 x 8 threads, 4 x 4 outputs each
  double acc[4][4] = {};
  for (long k0 = 0; k0 < K; k0 += BK) {
    for (int e = tid; e < BM * BK; e += 128) {
      int ii, kk;
      if (A_COLMAJOR) { ii = e % BM; kk = e / BM; } else { kk = e % BK; ii = e / BK; }
      const long gi = i0 + ii, gk = k0 + kk;
      double v = 0.0;
      if (gi < M && gk < K) v = A_COLMAJOR ? A[gk * lda + gi] : A[gi * lda + gk];
      sA[kk][ii] = v;
    }
    for (int e = tid; e < BN * BK; e += 128) {
      const int kk = e % BK, jj = e / BK;
      const long gj = j0 + jj, gk = k0 + kk;
      sB[kk][jj] = (gj < N && gk < K) ? B[gj * ldb + gk] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[4], bv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = sA[kk][ti + 16 * u];
#pragma unroll
      for (int v = 0; v < 4; ++v) bv[v] = sB[kk][tj + 8 * v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], bv[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const long gi = i0 + ti + 16 * u, gj = j0 + tj + 8 * v;
      if (gi < M && gj < N) C[gj * ldc + gi] = acc[u][v];
    }
}

int points_gemm_synth(const aeolus_plan_impl* p, const double* V, double* out, int ncols, cudaStream_t st);
int points_gemm_analysis(const aeolus_plan_impl* p, const double* W, double* C, int ncols, cudaStream_t st);

}  // namespace aeolus
