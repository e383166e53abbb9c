// Split-precision dense basis products of point-set plans (icosahedral
// geodesic grids) on tcgen05 tensor cores.
//
//   synthesis  out[n][p] = sum_c B[p][c] V[n][c]      (K = real basis columns)
//   analysis   out[n][c] = sum_p B[p][c] W[n][p]      (K = points)
//
// with the same balanced base-256 digits as the Gauss contraction (per-row
// basis exponents, per-column data exponents, 21 digit pairs in 6 MMAs, 6
// level accumulators).  K runs to 16384 (synthesis at l_max 127) or 40962
// (analysis on a level-6 grid), far beyond the depth at which an f32 sum of
// digit products stays exact, so every output tile is contracted in K
// segments of kSegChunks * 16 <= 160: each segment's level sums are exact
// integers below 6 * 160 * 2^14 < 2^24, drained from TMEM into two int64
// running sums per output (exact over at most kMaxPartChunks chunks), and
// the K range of a tile is split into parts whose partial results (one
// rounding each, to FP64) are added by a final pass.  The error is that of the dropped
// digit levels, ~2^-47 of sum_k |b_k| |v_k| per output.
#pragma once

#include "pipeline.cuh"
#include "split.cuh"

namespace aeolus {

constexpr int kDenseSegChunks = kExactChunks;          // 160-deep exact segments
constexpr int kMaxPartChunks = 136 * kDenseSegChunks;  // exact int64 running sums per part

struct DenseDims {
  int M, N;        // output rows (points or basis columns), data columns
  int Mt, Nt;      // 128-row and kNT-column tiles
  int nkc;         // K chunks of 16 (K padded)
  int KP, cpp;     // K parts, chunks per part
};

inline DenseDims dense_dims(int M, int N, int K, int sm_count) {
  DenseDims d;
  d.M = M;
  d.N = N;
  d.Mt = (M + 127) / 128;
  d.Nt = (N + kNT - 1) / kNT;
  d.nkc = (K + kKC - 1) / kKC;
  const int need = (d.nkc + kMaxPartChunks - 1) / kMaxPartChunks;
  const int balance = (8 * sm_count + d.Mt * d.Nt - 1) / (d.Mt * d.Nt);
  d.KP = std::max(1, std::max(need, std::min(16, std::min(balance, d.nkc))));
  d.cpp = (d.nkc + d.KP - 1) / d.KP;
  d.KP = (d.nkc + d.cpp - 1) / d.cpp;  // no empty part
  return d;
}

// Units (M tile, N tile, K part), K part slowest so neighbouring CTAs share
// data tiles.
struct DenseSched {
  static constexpr int kSegChunks = kDenseSegChunks;
  DenseDims d;
  const __nv_bfloat16* A;  // [Mt][nkc] chunks of 128 rows
  const __nv_bfloat16* B;  // [Nt][nkc] chunks of kNT rows
  __host__ __device__ int count() const { return d.Mt * d.Nt * d.KP; }
  int count_host() const { return count(); }
  __device__ TcTile tile(int t) const {
    const int kp = t / (d.Mt * d.Nt), r = t - kp * d.Mt * d.Nt;
    const int nt = r / d.Mt, mt = r - nt * d.Mt;
    const int k0 = kp * d.cpp, k1 = min(d.nkc, k0 + d.cpp);
    return TcTile{A + ((long long)mt * d.nkc + k0) * chunk_elems(128),
                  B + ((long long)nt * d.nkc + k0) * chunk_elems(kNT), k1 - k0};
  }
};

// 2^e as a double for e in the normal range (the callers stay inside it).
__device__ inline double pow2d(int e) { return __longlong_as_double((long long)(e + 1023) << 52); }

// Running sums of one output: with a segment's level sums I_k (|I_k| < 2^24)
// the segment value is T = (I0 2^8 + I1) 2^32 + (I2 2^24 + I3 2^16 + I4 2^8
// + I5); both parts are summed over segments in int64 (below 2^41 and 2^57
// for at most 136 segments) and rounded once to FP64 at the end.
__device__ inline double hr_to_double(long long H, long long R, int e) {
  if (H == 0 && R == 0) return 0.0;
  const double t = fma((double)H, 4294967296.0, (double)R);
  const int e1 = max(-1000, min(1000, e));
  return t * pow2d(e1 / 2) * pow2d(e1 - e1 / 2);
}

struct DenseEpi {
  static constexpr int kWarps = 16, kCols = 4 * kNT / kWarps;
  struct State {
    long long H[kCols], R[kCols];
  };
  DenseDims d;
  const int* eA;   // [Mt*128] row exponents
  const int* eB;   // [Nt*kNT] column exponents
  double* part;    // [KP][Nt*kNT][Mt*128]
  __device__ void seg_begin(State& st) const {
#pragma unroll
    for (int i = 0; i < kCols; ++i) st.H[i] = st.R[i] = 0;
  }
  __device__ void seg_add(State& st, uint32_t tbuf, int q, int c0) const {
    float acc[kCols][kAccs];
    tc_read<kCols>(tbuf, q, c0, acc);
#pragma unroll
    for (int i = 0; i < kCols; ++i) {
      int I[kAccs];
#pragma unroll
      for (int k = 0; k < kAccs; ++k) I[k] = __float2int_rn(acc[i][k]);
      st.H[i] += ((long long)I[0] << 8) + I[1];
      st.R[i] += ((long long)I[2] << 24) + ((long long)I[3] << 16) + ((long long)I[4] << 8) + I[5];
    }
  }
  __device__ void seg_end(int t, const State& st, int row, int c0, int) const {
    const int kp = t / (d.Mt * d.Nt), r = t - kp * d.Mt * d.Nt;
    const int nt = r / d.Mt, mt = r - nt * d.Mt;
    const int m = mt * 128 + row;
    const int ea = eA[m];
    const long long ldp = (long long)d.Mt * 128;
#pragma unroll
    for (int i = 0; i < kCols; ++i) {
      const int n = nt * kNT + c0 + i;
      part[((long long)kp * d.Nt * kNT + n) * ldp + m] = hr_to_double(st.H[i], st.R[i], ea + eB[n] - kOut);
    }
  }
};

// Per-column exponent and digits of a data block X[n * ldx + k] (k < K),
// one CTA per (padded) column; chunk-major tiles of kNT rows.
static __global__ void __launch_bounds__(256) dense_slice_kernel(const double* __restrict__ X, long ldx, int N, int K,
                                                          int nkc, __nv_bfloat16* __restrict__ out,
                                                          int* __restrict__ ecol) {
  __shared__ unsigned long long s_mx[8];
  __shared__ int s_e;
  const int n = blockIdx.x;
  const double* x = X + (long)n * ldx;
  unsigned long long mx = 0ull;
  if (n < N)
    for (int k = threadIdx.x; k < K; k += blockDim.x) mx = max(mx, abs_key(x[k]));
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) s_mx[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m2 = 0ull;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m2 = max(m2, s_mx[w]);
    s_e = n < N ? exponent_for_key(m2) : 0;
    ecol[n] = s_e;
  }
  __syncthreads();
  const int E = s_e;
  __nv_bfloat16* tile = out + (long long)(n / kNT) * nkc * chunk_elems(kNT);
  for (int g = threadIdx.x; g < nkc * kKC / 8; g += blockDim.x) {  // 8 contraction indices per thread
    const int k0 = 8 * g;
    long long Xs[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) Xs[u] = (n < N && k0 + u < K) ? fixed_point(x[k0 + u], E) : 0LL;
    store_digits8(tile, n % kNT, k0, Xs);
  }
}

// out[n * ldo + m] = sum over K parts (FP64, fixed order).
static __global__ void dense_reduce_kernel(const double* __restrict__ part, int KP, int Nt, int Mt, int M, int N,
                                    double* __restrict__ out, long ldo) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)M * N) return;
  const int n = (int)(idx / M), m = (int)(idx - (long)n * M);
  const long long ldp = (long long)Mt * 128, pstride = (long long)Nt * kNT * ldp;
  double v = 0.0;
  for (int kp = 0; kp < KP; ++kp) v += part[kp * pstride + (long long)n * ldp + m];
  out[(long)n * ldo + m] = v;
}

// Scratch of one dense product: data digits, column exponents, partials.
inline size_t dense_scratch_bytes(const DenseDims& d) {
  return align256((size_t)d.Nt * d.nkc * chunk_elems(kNT) * 2) + align256((size_t)d.Nt * kNT * 4) +
         align256((size_t)d.KP * d.Nt * kNT * d.Mt * 128 * 8);
}

// out[n * ldo + m] = sum_k A[m, k] X[n * ldx + k]; A given as digit tiles
// with row exponents (plan tables).
inline int dense_split_gemm(const aeolus_plan_impl* p, const DenseDims& d, const __nv_bfloat16* Adig,
                            const int* eA, const double* X, long ldx, int K, double* out, long ldo, void* scratch,
                            cudaStream_t st, const char* name) {
  char* w = static_cast<char*>(scratch);
  __nv_bfloat16* Bdig = reinterpret_cast<__nv_bfloat16*>(w);
  w += align256((size_t)d.Nt * d.nkc * chunk_elems(kNT) * 2);
  int* eB = reinterpret_cast<int*>(w);
  w += align256((size_t)d.Nt * kNT * 4);
  double* part = reinterpret_cast<double*>(w);
  {
    ProfScope prof("dense_slice", st);
    dense_slice_kernel<<<d.Nt * kNT, 256, 0, st>>>(X, ldx, d.N, K, d.nkc, Bdig, eB);
    AE_LAUNCH("dense_slice_kernel");
  }
  const size_t smt = tc_smem_bytes();
  auto k2 = tc_persistent_kernel<DenseSched, DenseEpi>;
  int s = allow_smem(k2, smt);
  if (s) return s;
  const DenseSched sc{d, Adig, Bdig};
  const DenseEpi ep{d, eA, eB, part};
  {
    ProfScope prof(name, st);
    k2<<<std::max(1, std::min(sc.count_host(), p->sm_count)), tc_threads<DenseEpi>(), smt, st>>>(sc, ep,
                                                                                                 p->split->err);
    AE_LAUNCH("tc_persistent_kernel(dense)");
  }
  const long n = (long)d.M * d.N;
  ProfScope prof("dense_reduce", st);
  dense_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, d.KP, d.Nt, d.Mt, d.M, d.N, out, ldo);
  AE_LAUNCH("dense_reduce_kernel");
  return AEOLUS_OK;
}

inline DenseDims dense_synth_dims(const aeolus_plan_impl* p, int ncols) {
  return dense_dims((int)p->npoints, ncols, p->ncol, p->sm_count);
}
inline DenseDims dense_anal_dims(const aeolus_plan_impl* p, int ncols) {
  return dense_dims(p->ncol, ncols, (int)p->npoints, p->sm_count);
}
inline size_t dense_bytes(const aeolus_plan_impl* p, int ncols) {
  return std::max(dense_scratch_bytes(dense_synth_dims(p, ncols)), dense_scratch_bytes(dense_anal_dims(p, ncols)));
}

}  // namespace aeolus
