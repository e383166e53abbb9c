// Legendre stage of the Gauss transform (FP64 contraction).
//
// Synthesis: F_m(x_j) = sum_{l=m..L} a_lm Pbar_lm(x_j), split by the parity
// of l - m so one pass over the northern rows gives both hemispheres
// (Pbar_lm(-x) = (-1)^(l-m) Pbar_lm(x)).  Analysis: a_lm = sum_j Pbar_lm(x_j)
// G_m(j) over the folded even/odd row sums.  CTAs take the order pair
// (i, L - i) so every CTA contracts the same L + 2 degrees.
//
// Functor contracts (shared with the point-set path):
//   Derive:   NF fields; column(b, l, m, double2 v[NF]) gives the spectral
//             coefficients to synthesise (derived from the caller's input).
//   Epilogue: NF analysed fields; finish(b, l, m, const double2 acc[NF])
//             consumes a_lm for l >= m; zero(b, l, m) handles l < m slots.
#pragma once

#include "common.cuh"

namespace aeolus {

struct LegArgs {
  int L, nlat, nh, batch, bc;
  const double* P;   // synthesis table (row index fastest)
  const double* PT;  // analysis table (degree fastest)
  double2* FG;       // F / G blocks [b][j][nblk][L+1]
  int nblk;
};

inline int n_pairs(int L) { return L / 2 + 1; }

template <class Derive, int CPT>
__device__ __forceinline__ void legendre_synth_body(const LegArgs& a, const Derive& d, int bx, int by) {
  constexpr int NF = Derive::NF;
  extern __shared__ double2 s_a[];
  const int L = a.L, nh = a.nh, ldm = L + 1;
  const int i = bx;
  const int mA = i, mB = L - i;
  const bool two = mB != mA;
  const int KA = L + 1 - mA, KB = two ? L + 1 - mB : 0;
  const int b0 = by * a.bc;
  const int nb = min(a.bc, a.batch - b0);
  const int ncols = nb * NF;
  const int ngroups = (ncols + CPT - 1) / CPT;
  const int ncp = ngroups * CPT;  // padded column count
  double2* sA = s_a;                 // [ncp][KA]
  double2* sB = s_a + (long)ncp * KA;  // [ncp][KB]

  // derived coefficient columns of both orders (zero padding columns)
  for (int idx = threadIdx.x; idx < nb * (KA + KB); idx += blockDim.x) {
    const int bl = idx / (KA + KB);
    const int t = idx - bl * (KA + KB);
    const bool isA = t < KA;
    const int m = isA ? mA : mB;
    const int tt = isA ? t : t - KA;
    const int K = isA ? KA : KB;
    double2 v[NF];
    d.column(b0 + bl, m + tt, m, v);
    double2* dst = isA ? sA : sB;
#pragma unroll
    for (int f = 0; f < NF; ++f) dst[(long)(bl * NF + f) * K + tt] = v[f];
  }
  for (int idx = threadIdx.x; idx < (ncp - ncols) * (KA + KB); idx += blockDim.x) {
    const int c = ncols + idx / (KA + KB);
    const int t = idx % (KA + KB);
    if (t < KA) sA[(long)c * KA + t] = make_double2(0.0, 0.0);
    else sB[(long)c * KB + (t - KA)] = make_double2(0.0, 0.0);
  }
  __syncthreads();

  for (int item = threadIdx.x; item < nh * ngroups; item += blockDim.x) {
    const int jn = item % nh, g = item / nh;
    const int c0 = g * CPT;
    const int jS = a.nlat - 1 - jn;
    for (int pass = 0; pass < (two ? 2 : 1); ++pass) {
      const int m = pass ? mB : mA;
      const int K = pass ? KB : KA;
      const double2* sc = (pass ? sB : sA) + (long)c0 * K;
      const double* Pm = a.P + tri_off(m, L) * nh + jn;
      double2 E[CPT], O[CPT];
#pragma unroll
      for (int q = 0; q < CPT; ++q) E[q] = O[q] = make_double2(0.0, 0.0);
      int t = 0;
      for (; t + 1 < K; t += 2) {
        const double pe = __ldg(Pm + (long)t * nh);
        const double po = __ldg(Pm + (long)(t + 1) * nh);
#pragma unroll
        for (int q = 0; q < CPT; ++q) {
          const double2 ae = sc[(long)q * K + t];
          const double2 ao = sc[(long)q * K + t + 1];
          E[q].x = fma(pe, ae.x, E[q].x);
          E[q].y = fma(pe, ae.y, E[q].y);
          O[q].x = fma(po, ao.x, O[q].x);
          O[q].y = fma(po, ao.y, O[q].y);
        }
      }
      if (t < K) {
        const double pe = __ldg(Pm + (long)t * nh);
#pragma unroll
        for (int q = 0; q < CPT; ++q) {
          const double2 ae = sc[(long)q * K + t];
          E[q].x = fma(pe, ae.x, E[q].x);
          E[q].y = fma(pe, ae.y, E[q].y);
        }
      }
#pragma unroll
      for (int q = 0; q < CPT; ++q) {
        const int c = c0 + q;
        if (c >= ncols) break;
        const int bl = c / NF, f = c - bl * NF;
        const long bb = b0 + bl;
        a.FG[fg_index(bb, m, f, jn, L, a.nblk, a.nlat)] = cadd(E[q], O[q]);
        if (jS != jn) a.FG[fg_index(bb, m, f, jS, L, a.nblk, a.nlat)] = csub(E[q], O[q]);
      }
    }
  }
}

template <class Derive, int CPT>
__global__ void __launch_bounds__(256) legendre_synth_kernel(LegArgs a, Derive d) {
  legendre_synth_body<Derive, CPT>(a, d, blockIdx.x, blockIdx.y);
}

template <class Derive, int CPT>
inline size_t synth_smem_bytes(int L, int bc) {
  const int ncols = bc * Derive::NF;
  const int ncp = (ncols + CPT - 1) / CPT * CPT;
  return (size_t)ncp * (L + 2) * sizeof(double2);
}

template <class Epi>
__device__ __forceinline__ void legendre_analysis_body(const LegArgs& a, const Epi& e, int bx, int by) {
  constexpr int NF = Epi::NF;
  extern __shared__ double2 s_g[];  // [2 orders][nb][NF][2 parities][nh]
  const int L = a.L, nh = a.nh, ldm = L + 1;
  const int i = bx;
  const int mA = i, mB = L - i;
  const bool two = mB != mA;
  const int KA = L + 1 - mA, KB = two ? L + 1 - mB : 0;
  const int b0 = by * a.bc;
  const int nb = min(a.bc, a.batch - b0);
  const long per_order = (long)a.bc * NF * 2 * nh;

  for (int idx = threadIdx.x; idx < (two ? 2 : 1) * nb * NF * nh; idx += blockDim.x) {
    int r = idx;
    const int jn = r % nh; r /= nh;
    const int f = r % NF; r /= NF;
    const int bl = r % nb; r /= nb;
    const int which = r;
    const int m = which ? mB : mA;
    const long bb = b0 + bl;
    const int jS = a.nlat - 1 - jn;
    const double2 gN = a.FG[fg_index(bb, m, f, jn, L, a.nblk, a.nlat)];
    const double2 gS = jS != jn ? a.FG[fg_index(bb, m, f, jS, L, a.nblk, a.nlat)] : make_double2(0.0, 0.0);
    double2* dst = s_g + which * per_order + ((long)(bl * NF + f) * 2) * nh;
    dst[jn] = cadd(gN, gS);
    dst[nh + jn] = csub(gN, gS);
  }
  __syncthreads();

  const int KT = KA + KB;
  for (int item = threadIdx.x; item < nb * KT; item += blockDim.x) {
    const int bl = item / KT;
    const int t0 = item - bl * KT;
    const bool isA = t0 < KA;
    const int m = isA ? mA : mB;
    const int t = isA ? t0 : t0 - KA;
    const int K = isA ? KA : KB;
    const int par = t & 1;
    const double2* sg = s_g + (isA ? 0 : per_order) + ((long)bl * NF * 2 + par) * nh;
    const double* pt = a.PT + tri_off(m, L) * nh + t;
    double2 acc[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) acc[f] = make_double2(0.0, 0.0);
    for (int jn = 0; jn < nh; ++jn) {
      const double p = __ldg(pt + (long)jn * K);
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const double2 g = sg[(long)f * 2 * nh + jn];
        acc[f].x = fma(p, g.x, acc[f].x);
        acc[f].y = fma(p, g.y, acc[f].y);
      }
    }
    e.finish(b0 + bl, m + t, m, acc);
  }
  // slots l < m of the two columns
  for (int idx = threadIdx.x; idx < nb * (mA + (two ? mB : 0)); idx += blockDim.x) {
    const int per = mA + (two ? mB : 0);
    const int bl = idx / per;
    const int r = idx - bl * per;
    if (r < mA) e.zero(b0 + bl, r, mA);
    else e.zero(b0 + bl, r - mA, mB);
  }
}

template <class Epi>
__global__ void __launch_bounds__(256) legendre_analysis_kernel(LegArgs a, Epi e) {
  legendre_analysis_body<Epi>(a, e, blockIdx.x, blockIdx.y);
}

template <class Epi>
inline size_t analysis_smem_bytes(int nh, int bc) {
  return (size_t)2 * bc * Epi::NF * 2 * nh * sizeof(double2);
}

// ------------------------------------------------------------ plain functors
struct DeriveCopy {  // synthesis input: dense [b][L+1][L+1]
  static constexpr int NF = 1;
  const double2* in;
  int L;
  long bstride;
  __device__ void column(int b, int l, int m, double2* v) const {
    v[0] = in[(long)b * bstride + (long)l * (L + 1) + m];
  }
};

struct EpiStore {  // analysis output: dense [b][L+1][L+1]
  static constexpr int NF = 1;
  double2* out;
  int L;
  long bstride;
  __device__ void finish(int b, int l, int m, const double2* acc) const {
    out[(long)b * bstride + (long)l * (L + 1) + m] = acc[0];
  }
  __device__ void zero(int b, int l, int m) const {
    out[(long)b * bstride + (long)l * (L + 1) + m] = make_double2(0.0, 0.0);
  }
};

}  // namespace aeolus
