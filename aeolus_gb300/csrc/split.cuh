// Split-precision (bf16-digit, tcgen05) Legendre stages: data slicing
// kernels, the two tensor-core GEMM kernels and their launch helpers.  The
// digit scheme and exactness argument are described in split.cu.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"
#include "legendre.cuh"
#include "tc.cuh"

namespace aeolus {

constexpr int kSlices = 6;   // base-256 digits per operand (48 bits)
constexpr int kLevels = 6;   // kept levels k = s + t = 2..7 (1-based digits)
constexpr int kAccs = 7;     // TMEM accumulators: the 6-pair top level is split in two
constexpr int kNT = 64;      // data columns per synthesis tile (MMA N)
constexpr int kNTa = 48;     // data columns per analysis tile
constexpr int kTmemCols = 512;
constexpr int kShift = 8 * kSlices;  // X = rint(x 2^(kShift - E))
constexpr int kMaxKp = 128;  // degrees per order (l_max <= 127)

struct SplitTables {
  int L = 0, nlat = 0, nh = 0, NK = 0, Mt = 1;
  __nv_bfloat16* psyn = nullptr;  // synthesis basis digits
  __nv_bfloat16* pana = nullptr;  // analysis basis digits
  int* esyn = nullptr;            // [m][Mt*128] latitude-row exponents
  int* eana = nullptr;            // [m][128] degree-row exponents
  long long* kcum = nullptr;      // [L+2] prefix sums of padded degree counts
  int* err = nullptr;             // sticky device error flag (bounded waits)
  std::vector<long long> h_kcum;
};

int split_build(aeolus_plan_impl* p);

__host__ __device__ inline int kpad(int k) { return (k + 15) / 16 * 16; }

// All conversions below work on IEEE-754 bit patterns with integer
// instructions: GB300's FP64 pipe is ~1/64 of its FP32/INT32 rate, and the
// digit split / recombination touch every element of every contraction.

// |x| as an order-preserving integer key (for the column maxima).
__device__ inline unsigned long long abs_key(double x) {
  return static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7FFFFFFFFFFFFFFFull;
}

// Exponent E with |x| 2^-E < 1/2 for every |x| <= the value whose abs_key
// is k (E = -1000 for zero or subnormal maxima, which then slice to 0).
__device__ inline int exponent_for_key(unsigned long long k) {
  const int ex = static_cast<int>(k >> 52);
  return ex == 0 ? -1000 : ex - 1021;
}

// X = rint(x 2^(48-E)) (round half to even), |X| <= 2^47.
__device__ inline long long fixed_point(double x, int E) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const int ex = static_cast<int>((b >> 52) & 0x7FF);
  if (ex == 0 || E == -1000) return 0;
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);  // |x| = m 2^(ex-1075)
  const int sh = 1075 - kShift + E - ex;                                   // right shift
  unsigned long long q;
  if (sh >= 54) {
    q = 0;
  } else if (sh <= 0) {
    q = m << (-sh);
  } else {
    q = m >> sh;
    const unsigned long long rem = m & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (q & 1ull))) ++q;
  }
  const long long X = static_cast<long long>(q);
  return (b >> 63) ? -X : X;
}

// Balanced base-256 digits of rint(x 2^(48-E)), most significant first.
__device__ inline void digits(double x, int E, float* d) {
  long long X = fixed_point(x, E);
#pragma unroll
  for (int i = kSlices - 1; i >= 1; --i) {
    const long long r = ((X + 128) & 255) - 128;
    d[i] = (float)r;
    X = (X - r) >> 8;
  }
  d[0] = (float)X;
}

// T 2^e as a double (round to nearest even; results below the normal range
// flush to zero), integer instructions only.
__device__ inline double scaled_to_double(long long T, int e) {
  if (T == 0) return 0.0;
  const unsigned long long sign = T < 0 ? (1ull << 63) : 0ull;
  unsigned long long a = T < 0 ? static_cast<unsigned long long>(-T) : static_cast<unsigned long long>(T);
  int msb = 63 - __clzll(static_cast<long long>(a));
  unsigned long long mant;
  if (msb > 52) {
    const int sh = msb - 52;
    const unsigned long long rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    mant = a >> sh;
    if (rem > half || (rem == half && (mant & 1ull))) {
      ++mant;
      if (mant >> 53) {
        mant >>= 1;
        ++msb;
      }
    }
  } else {
    mant = a << (52 - msb);
  }
  const int ex = msb + e + 1023;
  if (ex <= 0) return 0.0;
  return __longlong_as_double(static_cast<long long>(sign | (static_cast<unsigned long long>(ex) << 52) |
                                                     (mant & 0xFFFFFFFFFFFFFull)));
}

// Level recombination: T = sum_k I_k 256^(5-k), k = 0..5 <-> s+t = 2..7,
// the top level held in two accumulators.  |T| < 2^62.
__device__ inline long long combine_levels(const float* acc) {
  long long T = 0;
#pragma unroll
  for (int k = 0; k < kLevels - 1; ++k) T = (T << 8) + __float2int_rn(acc[k]);
  return (T << 8) + ((long long)__float2int_rn(acc[kLevels - 1]) + __float2int_rn(acc[kLevels]));
}

// Accumulator of digit pair (s, t) (0-based): one per level, except the
// top level whose 6 pairs are split 3 + 3 so that each f32 sum stays an
// exact integer for K <= 192 (3 * 192 * 2^14 < 2^24).
__host__ __device__ constexpr int acc_of(int s, int t) {
  return (s + t < kLevels - 1) ? s + t : (s < kSlices / 2 ? kLevels - 1 : kLevels);
}

// Result exponent offset: x y = T 2^(Ex + Ey - kOut).
constexpr int kOut = 2 * kShift - 8 * (kSlices - 1);

// ----------------------------------------------------------- layouts
struct SplitDims {
  int L, nlat, nh, NK, Mt;
  int ncol;     // data columns (members x fields x 2)
  int ntiles;   // ceil(ncol / kNT)
};

// Synthesis data digits, block (m, ntile, slice): kNT x Kpad_m.
__host__ __device__ inline long long dsyn_block(const long long* kcum, const SplitDims& d, int m, int ntile, int s) {
  const int Kp = kpad(d.L + 1 - m);
  return kcum[m] * (long long)d.ntiles * kSlices * kNT + ((long long)ntile * kSlices + s) * kNT * Kp;
}

// Analysis data digits, block (m, ntile, slice): kNTa x NK.
__host__ __device__ inline long long dana_block(const SplitDims& d, int m, int ntile, int s) {
  return (((long long)m * d.ntiles + ntile) * kSlices + s) * kNTa * (long long)d.NK;
}

// ------------------------------------------------- synthesis data slicing
// grid (m, member chunk of `mb` members); columns (b, f, re/im).
template <class Derive>
__global__ void __launch_bounds__(256) split_synth_slice_kernel(SplitDims dm, const long long* __restrict__ kcum,
                                                               int batch, int mb, Derive der,
                                                               __nv_bfloat16* __restrict__ dsyn,
                                                               int* __restrict__ ecol) {
  constexpr int NF = Derive::NF;
  extern __shared__ double s_val[];  // [mb*NF*2][K]
  __shared__ int s_exp[256];
  const int m = blockIdx.x, L = dm.L;
  const int K = L + 1 - m, Kp = kpad(K);
  const int b0 = blockIdx.y * mb;
  const int nb = min(mb, batch - b0);
  const int nc = nb * NF * 2;
  for (int idx = threadIdx.x; idx < nb * K; idx += blockDim.x) {
    const int bl = idx / K, t = idx - bl * K;
    double2 v[NF];
    der.column(b0 + bl, m + t, m, v);
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      s_val[((bl * NF + f) * 2 + 0) * K + t] = v[f].x;
      s_val[((bl * NF + f) * 2 + 1) * K + t] = v[f].y;
    }
  }
  __syncthreads();
  // column exponents (one warp per column)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int c = warp; c < nc; c += nwarp) {
    unsigned long long mx = 0ull;
    for (int t = lane; t < K; t += 32) mx = max(mx, abs_key(s_val[c * K + t]));
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) {
      const int E = exponent_for_key(mx);
      s_exp[c] = E;
      ecol[(long long)m * dm.ntiles * kNT + (long long)b0 * NF * 2 + c] = E;
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < nc * Kp; idx += blockDim.x) {
    const int c = idx / Kp, t = idx - c * Kp;
    const int n = b0 * NF * 2 + c;
    const int tile = n / kNT, nl = n % kNT;
    float d[kSlices];
    digits(t < K ? s_val[c * K + t] : 0.0, s_exp[c], d);
#pragma unroll
    for (int s = 0; s < kSlices; ++s)
      dsyn[dsyn_block(kcum, dm, m, tile, s) + tc::core_index(nl, t, Kp)] = __float2bfloat16(d[s]);
  }
  // zero columns that pad the last tile
  if (blockIdx.y == gridDim.y - 1) {
    const int n0 = batch * NF * 2, n1 = dm.ntiles * kNT;
    for (int idx = threadIdx.x; idx < (n1 - n0) * Kp; idx += blockDim.x) {
      const int n = n0 + idx / Kp, t = idx % Kp;
#pragma unroll
      for (int s = 0; s < kSlices; ++s)
        dsyn[dsyn_block(kcum, dm, m, n / kNT, s) + tc::core_index(n % kNT, t, Kp)] = __float2bfloat16(0.0f);
      if (t == 0) ecol[(long long)m * dm.ntiles * kNT + n] = 0;
    }
  }
}

// ------------------------------------------------- analysis data slicing
// Reads G[b][j][f][m] (F/G blocks of nblk fields), grid (m, member chunk).
template <int NF>
__global__ void __launch_bounds__(256) split_anal_slice_kernel(SplitDims dm, int batch, int mb, int nblk,
                                                              const double2* __restrict__ FG,
                                                              __nv_bfloat16* __restrict__ dana,
                                                              int* __restrict__ ecol) {
  extern __shared__ double s_val[];  // [mb*NF*2][nlat]
  __shared__ int s_exp[256];
  const int m = blockIdx.x, L = dm.L, nlat = dm.nlat, NK = dm.NK;
  const int ldm = L + 1;
  const int b0 = blockIdx.y * mb;
  const int nb = min(mb, batch - b0);
  const int nc = nb * NF * 2;
  for (int idx = threadIdx.x; idx < nb * NF * nlat; idx += blockDim.x) {
    const int j = idx % nlat;
    const int r = idx / nlat;
    const int f = r % NF, bl = r / NF;
    const double2 g = FG[(((long long)(b0 + bl) * nlat + j) * nblk + f) * ldm + m];
    s_val[((bl * NF + f) * 2 + 0) * nlat + j] = g.x;
    s_val[((bl * NF + f) * 2 + 1) * nlat + j] = g.y;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int c = warp; c < nc; c += nwarp) {
    unsigned long long mx = 0ull;
    for (int j = lane; j < nlat; j += 32) mx = max(mx, abs_key(s_val[c * nlat + j]));
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) {
      const int E = exponent_for_key(mx);
      s_exp[c] = E;
      ecol[(long long)m * dm.ntiles * kNTa + (long long)b0 * NF * 2 + c] = E;
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < nc * NK; idx += blockDim.x) {
    const int c = idx / NK, j = idx - c * NK;
    const int n = b0 * NF * 2 + c;
    float d[kSlices];
    digits(j < nlat ? s_val[c * nlat + j] : 0.0, s_exp[c], d);
#pragma unroll
    for (int s = 0; s < kSlices; ++s)
      dana[dana_block(dm, m, n / kNTa, s) + tc::core_index(n % kNTa, j, NK)] = __float2bfloat16(d[s]);
  }
  if (blockIdx.y == gridDim.y - 1) {
    const int n0 = batch * NF * 2, n1 = dm.ntiles * kNTa;
    for (int idx = threadIdx.x; idx < (n1 - n0) * NK; idx += blockDim.x) {
      const int n = n0 + idx / NK, j = idx % NK;
#pragma unroll
      for (int s = 0; s < kSlices; ++s)
        dana[dana_block(dm, m, n / kNTa, s) + tc::core_index(n % kNTa, j, NK)] = __float2bfloat16(0.0f);
      if (j == 0) ecol[(long long)m * dm.ntiles * kNTa + n] = 0;
    }
  }
}

// ---------------------------------------------------- tensor-core GEMM core
// Shared by synthesis and analysis: A = kSlices basis-digit tiles (128 x KK,
// streamed through a double buffer), B = kSlices data-digit tiles (NT x KK,
// resident).  On return accumulator a sits in TMEM columns [a*NT, (a+1)*NT).
// Returns false (and sets *err) if a bounded wait expired.
struct TcSmem {
  __nv_bfloat16* A[2];
  __nv_bfloat16* B;
  uint64_t* bar;  // [0..1] A buffers loaded, [2..3] A buffers free, [4] B loaded, [5] MMAs done
};

template <int NT>
__device__ inline bool tc_levels(const TcSmem& sm, const __nv_bfloat16* gA, long long a_slice_elems,
                                 const __nv_bfloat16* gB, long long b_slice_elems, int KK, uint32_t tmem,
                                 int* err) {
  const uint32_t abytes = 128u * KK * 2u, bbytes = (uint32_t)NT * KK * 2u;
  bool ok = true;
  if (threadIdx.x == 0) {
    int issued[2] = {0, 0}, waited[2] = {0, 0};
    unsigned started = 0u;  // accumulators already holding a partial sum
    bool b_ok = false;
    tc::mbar_expect_tx(&sm.bar[4], kSlices * bbytes);
    for (int t = 0; t < kSlices; ++t)
      tc::bulk_g2s(sm.B + (long long)t * NT * KK, gB + t * b_slice_elems, bbytes, &sm.bar[4]);
    for (int s = 0; s < 2; ++s) {
      tc::mbar_expect_tx(&sm.bar[s], abytes);
      tc::bulk_g2s(sm.A[s], gA + s * a_slice_elems, abytes, &sm.bar[s]);
      issued[s] = 1;
    }
    const uint32_t idesc = tc::idesc_bf16_f32(128, NT);
    const uint32_t sbo = (uint32_t)KK * 16u;
    ok = b_ok = tc::mbar_wait(&sm.bar[4], 0);
    for (int s = 0; s < kSlices && ok; ++s) {
      const int buf = s & 1;
      ok = tc::mbar_wait(&sm.bar[buf], waited[buf] & 1);
      if (!ok) break;
      ++waited[buf];
      for (int t = 0; s + t < kSlices; ++t) {
        const int a = acc_of(s, t);
        const uint32_t dcol = tmem + (uint32_t)a * NT;
        for (int ks = 0; ks < KK / 16; ++ks) {
          const uint64_t da = tc::smem_desc(sm.A[buf] + ks * 128, 128, sbo);
          const uint64_t db = tc::smem_desc(sm.B + (long long)t * NT * KK + ks * 128, 128, sbo);
          tc::mma_bf16(dcol, da, db, idesc, ((started >> a) & 1u) ? 1u : 0u);
          started |= 1u << a;
        }
      }
      if (s + 2 < kSlices) {
        // refill this buffer once the MMAs that read it have completed
        tc::mma_commit(&sm.bar[2 + buf]);
        ok = tc::mbar_wait(&sm.bar[2 + buf], (s >> 1) & 1);
        if (!ok) break;
        tc::mbar_expect_tx(&sm.bar[buf], abytes);
        tc::bulk_g2s(sm.A[buf], gA + (s + 2) * a_slice_elems, abytes, &sm.bar[buf]);
        ++issued[buf];
      }
    }
    tc::mma_commit(&sm.bar[5]);
    if (!ok) {
      // drain copies still in flight (bounded) before the CTA gives up
      atomicExch(err, 1);
      if (!b_ok) tc::mbar_wait(&sm.bar[4], 0);
      for (int b = 0; b < 2; ++b)
        for (; waited[b] < issued[b]; ++waited[b]) tc::mbar_wait(&sm.bar[b], waited[b] & 1);
    }
  }
  __syncthreads();
  const bool done = tc::mbar_wait(&sm.bar[5], 0);
  if (!done && threadIdx.x == 0) atomicExch(err, 2);
  tc::fence_after_sync();
  return __syncthreads_and((done && ok) ? 1 : 0) != 0;
}

// Dynamic shared memory: at least 116 KB so that one CTA holds an SM (each
// CTA takes all 512 TMEM columns; a second resident CTA would only stall in
// tcgen05.alloc).
inline size_t tc_smem_bytes(int KK, int NT) {
  const size_t need = 2 * 128 * (size_t)KK * 2 + (size_t)kSlices * NT * KK * 2 + 1024 + 128;
  return std::max<size_t>(need, 116 * 1024);
}

__device__ inline void tc_carve(char* base, int KK, int NT, TcSmem& sm, uint32_t*& tmem_slot) {
  char* p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(base) + 1023) & ~uintptr_t(1023));
  sm.A[0] = reinterpret_cast<__nv_bfloat16*>(p);
  sm.A[1] = sm.A[0] + 128 * KK;
  sm.B = sm.A[1] + 128 * KK;
  char* q = reinterpret_cast<char*>(sm.B + (long long)kSlices * NT * KK);
  sm.bar = reinterpret_cast<uint64_t*>(q);
  tmem_slot = reinterpret_cast<uint32_t*>(q + 8 * 8);
}

__device__ inline void tc_begin(TcSmem& sm, uint32_t* tmem_slot) {
  if (threadIdx.x == 0) {
    for (int i = 0; i < 6; ++i) tc::mbar_init(&sm.bar[i], 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_alloc(tmem_slot, kTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

__device__ inline void tc_end(uint32_t tmem) {
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_dealloc(tmem, kTmemCols);
}

// The kAccs accumulators of 16 columns starting at c0, for this thread's
// lane (the TMEM lane quadrant of its warp).
template <int NT>
__device__ inline void tc_read16(uint32_t tmem, int c0, float (*acc)[kAccs]) {
  const uint32_t lane_base = (uint32_t)((threadIdx.x >> 5) * 32) << 16;
  uint32_t r[16];
#pragma unroll
  for (int k = 0; k < kAccs; ++k) {
    tc::tmem_ld16(tmem + lane_base + (uint32_t)(k * NT + c0), r);
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i][k] = __uint_as_float(r[i]);
  }
}

// --------------------------------------------------------- synthesis GEMM
// grid (m, latitude tile, data tile), 128 threads.  Writes F blocks.
static __global__ void __launch_bounds__(128, 1) tc_synth_kernel(SplitDims dm, const long long* __restrict__ kcum,
                                                                 const __nv_bfloat16* __restrict__ psyn,
                                                                 const int* __restrict__ esyn,
                                                                 const __nv_bfloat16* __restrict__ dsyn,
                                                                 const int* __restrict__ ecol, int nf, int nblk,
                                                                 double2* __restrict__ F, int* err) {
  extern __shared__ char smem_raw[];
  const int m = blockIdx.x, mt = blockIdx.y, tile = blockIdx.z;
  const int L = dm.L, Kp = kpad(L + 1 - m);
  TcSmem sm;
  uint32_t* tslot;
  tc_carve(smem_raw, Kp, kNT, sm, tslot);
  tc_begin(sm, tslot);
  const uint32_t tmem = *tslot;
  const __nv_bfloat16* gA = psyn + kcum[m] * (long long)dm.Mt * kSlices * 128 + (long long)mt * kSlices * 128 * Kp;
  const __nv_bfloat16* gB = dsyn + dsyn_block(kcum, dm, m, tile, 0);
  const bool ok = tc_levels<kNT>(sm, gA, 128LL * Kp, gB, (long long)kNT * Kp, Kp, tmem, err);
  if (ok) {
    const int j = mt * 128 + threadIdx.x;
    const int Ej = j < dm.nlat ? esyn[m * dm.Mt * 128 + j] : 0;
    const int* ec = ecol + (long long)m * dm.ntiles * kNT + tile * kNT;
    for (int c0 = 0; c0 < kNT; c0 += 16) {
      float acc[16][kAccs];
      tc_read16<kNT>(tmem, c0, acc);
      if (j < dm.nlat) {
#pragma unroll
        for (int i = 0; i < 16; i += 2) {
          const int n = tile * kNT + c0 + i;  // even: real part, n + 1: imaginary part
          if (n >= dm.ncol) break;
          const double re = scaled_to_double(combine_levels(acc[i]), Ej + ec[c0 + i] - kOut);
          const double im = scaled_to_double(combine_levels(acc[i + 1]), Ej + ec[c0 + i + 1] - kOut);
          const int bf = n >> 1;
          const int b = bf / nf, f = bf - b * nf;
          F[(((long long)b * dm.nlat + j) * nblk + f) * (L + 1) + m] = make_double2(re, im);
        }
      }
    }
  }
  tc_end(tmem);
}

// --------------------------------------------------------- analysis GEMM
// grid (m, data tile), 128 threads; lane = degree offset l - m.
template <class Epi>
__global__ void __launch_bounds__(128, 1) tc_anal_kernel(SplitDims dm, const __nv_bfloat16* __restrict__ pana,
                                                         const int* __restrict__ eana,
                                                         const __nv_bfloat16* __restrict__ dana,
                                                         const int* __restrict__ ecol, int batch, Epi epi, int* err) {
  constexpr int NF = Epi::NF;
  static_assert(16 % (2 * NF) == 0, "a 16-column chunk must hold whole members");
  extern __shared__ char smem_raw[];
  const int m = blockIdx.x, tile = blockIdx.y;
  const int L = dm.L, NK = dm.NK, K = L + 1 - m;
  TcSmem sm;
  uint32_t* tslot;
  tc_carve(smem_raw, NK, kNTa, sm, tslot);
  tc_begin(sm, tslot);
  const uint32_t tmem = *tslot;
  const __nv_bfloat16* gA = pana + (long long)m * kSlices * 128 * NK;
  const __nv_bfloat16* gB = dana + dana_block(dm, m, tile, 0);
  const bool ok = tc_levels<kNTa>(sm, gA, 128LL * NK, gB, (long long)kNTa * NK, NK, tmem, err);
  const int t = threadIdx.x;
  if (ok) {
    const int Et = eana[m * 128 + t];
    const int* ec = ecol + (long long)m * dm.ntiles * kNTa + tile * kNTa;
    for (int c0 = 0; c0 < kNTa; c0 += 16) {
      float acc[16][kAccs];
      tc_read16<kNTa>(tmem, c0, acc);
      if (t < K) {
#pragma unroll
        for (int i = 0; i < 16; i += 2 * NF) {
          const int n = tile * kNTa + c0 + i;
          const int b = n / (2 * NF);
          if (b >= batch) break;
          double2 a[NF];
#pragma unroll
          for (int f = 0; f < NF; ++f) {
            a[f].x = scaled_to_double(combine_levels(acc[i + 2 * f]), Et + ec[c0 + i + 2 * f] - kOut);
            a[f].y = scaled_to_double(combine_levels(acc[i + 2 * f + 1]), Et + ec[c0 + i + 2 * f + 1] - kOut);
          }
          epi.finish(b, m + t, m, a);
        }
      }
    }
    // slots l < m of column m for this tile's members
    const int mb0 = tile * kNTa / (2 * NF), mb1 = min(batch, (tile + 1) * kNTa / (2 * NF));
    for (int idx = threadIdx.x; idx < (mb1 - mb0) * m; idx += blockDim.x) epi.zero(mb0 + idx / m, idx % m, m);
  }
  tc_end(tmem);
}

// ------------------------------------------------------------ launchers
inline SplitDims split_dims(const aeolus_plan_impl* p, int ncol, int nt) {
  const SplitTables* t = p->split;
  return SplitDims{t->L, t->nlat, t->nh, t->NK, t->Mt, ncol, (ncol + nt - 1) / nt};
}

inline size_t split_synth_bytes(const aeolus_plan_impl* p, int nf, int batch) {
  const SplitDims d = split_dims(p, batch * nf * 2, kNT);
  return align256((size_t)p->split->h_kcum[d.L + 1] * d.ntiles * kSlices * kNT * 2) +
         align256((size_t)(d.L + 1) * d.ntiles * kNT * 4);
}

inline size_t split_anal_bytes(const aeolus_plan_impl* p, int nf, int batch) {
  const SplitDims d = split_dims(p, batch * nf * 2, kNTa);
  return align256((size_t)(d.L + 1) * d.ntiles * kSlices * kNTa * d.NK * 2) +
         align256((size_t)(d.L + 1) * d.ntiles * kNTa * 4);
}

inline int slice_members(int nf, int K) {
  // members per slicing CTA: staged values within 64 KB and at most 256 columns
  return std::max(1, std::min(256 / (2 * nf), (64 * 1024) / (2 * nf * K * 8)));
}

template <class Derive>
int launch_split_synth(const aeolus_plan_impl* p, const Derive& d, double2* FG, int nblk, int batch, void* scratch,
                       cudaStream_t st) {
  constexpr int NF = Derive::NF;
  const SplitDims dm = split_dims(p, batch * NF * 2, kNT);
  char* w = static_cast<char*>(scratch);
  __nv_bfloat16* dsyn = reinterpret_cast<__nv_bfloat16*>(w);
  w += align256((size_t)p->split->h_kcum[dm.L + 1] * dm.ntiles * kSlices * kNT * 2);
  int* ecol = reinterpret_cast<int*>(w);
  const int mb = slice_members(NF, dm.L + 1);
  const size_t sm1 = (size_t)mb * NF * 2 * (dm.L + 1) * 8;
  auto k1 = split_synth_slice_kernel<Derive>;
  int s = allow_smem(k1, sm1);
  if (s) return s;
  {
    ProfScope prof("split_synth_slice", st);
    k1<<<dim3(dm.L + 1, (batch + mb - 1) / mb), 256, sm1, st>>>(dm, p->split->kcum, batch, mb, d, dsyn, ecol);
    AE_LAUNCH("split_synth_slice_kernel");
  }
  const size_t sm2 = tc_smem_bytes(kpad(dm.L + 1), kNT);
  if ((s = allow_smem(tc_synth_kernel, sm2))) return s;
  ProfScope prof("tc_synth_bf16x6", st);
  tc_synth_kernel<<<dim3(dm.L + 1, dm.Mt, dm.ntiles), 128, sm2, st>>>(dm, p->split->kcum, p->split->psyn,
                                                                      p->split->esyn, dsyn, ecol, NF, nblk, FG,
                                                                      p->split->err);
  AE_LAUNCH("tc_synth_kernel");
  return AEOLUS_OK;
}

template <class Epi>
int launch_split_anal(const aeolus_plan_impl* p, const Epi& e, const double2* FG, int nblk, int batch, void* scratch,
                      cudaStream_t st) {
  constexpr int NF = Epi::NF;
  const SplitDims dm = split_dims(p, batch * NF * 2, kNTa);
  char* w = static_cast<char*>(scratch);
  __nv_bfloat16* dana = reinterpret_cast<__nv_bfloat16*>(w);
  w += align256((size_t)(dm.L + 1) * dm.ntiles * kSlices * kNTa * dm.NK * 2);
  int* ecol = reinterpret_cast<int*>(w);
  const int mb = slice_members(NF, dm.nlat);
  const size_t sm1 = (size_t)mb * NF * 2 * dm.nlat * 8;
  auto k1 = split_anal_slice_kernel<NF>;
  int s = allow_smem(k1, sm1);
  if (s) return s;
  {
    ProfScope prof("split_anal_slice", st);
    k1<<<dim3(dm.L + 1, (batch + mb - 1) / mb), 256, sm1, st>>>(dm, batch, mb, nblk, FG, dana, ecol);
    AE_LAUNCH("split_anal_slice_kernel");
  }
  const size_t sm2 = tc_smem_bytes(dm.NK, kNTa);
  auto k2 = tc_anal_kernel<Epi>;
  if ((s = allow_smem(k2, sm2))) return s;
  ProfScope prof("tc_anal_bf16x6", st);
  k2<<<dim3(dm.L + 1, dm.ntiles), 128, sm2, st>>>(dm, p->split->pana, p->split->eana, dana, ecol, batch, e,
                                                   p->split->err);
  AE_LAUNCH("tc_anal_kernel");
  return AEOLUS_OK;
}

}  // namespace aeolus
