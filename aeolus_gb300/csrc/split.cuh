// Split-precision (bf16-digit, tcgen05) Legendre stages: data slicing
// kernels, the two tensor-core GEMM kernels and their launch helpers.  The
// digit scheme and exactness argument are described in split.cu.
#pragma once

#include <cuda_bf16.h>

#include <type_traits>
#include <utility>

#include "common.cuh"
#include "df.cuh"
#include "fx.cuh"
#include "legendre.cuh"
#include "tc.cuh"

namespace aeolus {

constexpr int kSlices = 6;   // base-256 digits per operand (48 bits)
constexpr int kLevels = 6;   // kept levels k = s + t = 2..7 (1-based digits)
constexpr int kAccs = 6;     // TMEM accumulators, one per kept level
constexpr int kNT = 32;      // data columns per tensor-core tile (one digit slice of the MMA N)
constexpr int kKC = 16;      // contraction depth per pipeline chunk (one MMA K step)
constexpr int kShift = 8 * kSlices;  // X = rint(x 2^(kShift - E))
constexpr int kMaxL = 159;   // l_max <= 159: a synthesis tile (K <= 160) is one exact segment

struct SplitTables {
  int L = 0, nlat = 0, nh = 0, NK = 0, Mt = 1;
  __nv_bfloat16* psyn = nullptr;  // synthesis basis digits
  __nv_bfloat16* pana = nullptr;  // analysis basis digits
  int* esyn = nullptr;            // [m][Mt*128] latitude-row exponents
  int* eana = nullptr;            // [row tile][128] degree-row exponents
  long long* kcum = nullptr;      // [L+2] prefix sums of padded degree counts
  int* err = nullptr;             // sticky device error flag (bounded waits)
  std::vector<long long> h_kcum;
  // point-set plans: dense real basis digits in both operand roles
  __nv_bfloat16* bsyn = nullptr;  // rows = points, K = basis columns
  __nv_bfloat16* bana = nullptr;  // rows = basis columns, K = points
  int* ebsyn = nullptr;           // per point (padded to 128)
  int* ebana = nullptr;           // per basis column (padded to 128)
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

// X = hi 2^p + lo 2^p rounded to an integer (within one unit of
// rint((hi + lo) 2^p)) for 2^p = pa pb and |hi 2^p| < 2^47: the high word's
// multiple of 2^30 from the float magic-number rounding, the rest (|r| <=
// 2^29 and the scaled low word) rounded to 32-bit integers.
__device__ __forceinline__ long long fixed_point_df(float2 v, float pa, float pb) {
  const float th = v.x * pa * pb, tl = v.y * pa * pb;
  const float c15 = 12582912.0f;                             // 1.5 2^23
  const float um = fmaf(th, 9.31322574615478515625e-10f, c15);  // th 2^-30 rounded into the mantissa
  const float r = fmaf(-(um - c15), 1073741824.0f, th);      // th - u 2^30, exact
  const int u = __float_as_int(um) - 0x4B400000;
  return fx_madw(u, 1 << 30, static_cast<long long>(__float2int_rn(r) + __float2int_rn(tl)));
}

// Derives with a double-float column (kColumnDf; column_df(b, l, m, v):
// v[f] a df2 with the lanes re, im).
template <class D, class = void>
struct DeriveHasDf : std::false_type {};
template <class D>
struct DeriveHasDf<D, std::enable_if_t<D::kColumnDf>> : std::true_type {};

// One digit (|r| <= 128) as a bf16, exactly: the magic-number construction
// puts r in the mantissa of 1.5 2^23 (FMA pipe, no integer-to-float
// conversion, which would run on the FP64 pipe for 64-bit operands), and a
// float holding a small integer is its own bf16 upper half.
__device__ __forceinline__ __nv_bfloat16 digit_bf16(int r) {
  const float f = __int_as_float(0x4B400000 + r) - 12582912.0f;
  return __ushort_as_bfloat16(static_cast<unsigned short>(__float_as_uint(f) >> 16));
}

// Balanced base-256 digits of a fixed-point integer X (|X| <= 2^47), most
// significant first.
__device__ inline void digits_from_fixed(long long X, __nv_bfloat16* d) {
#pragma unroll
  for (int i = kSlices - 1; i >= 1; --i) {
    const int r = static_cast<int>(((X + 128) & 255) - 128);
    d[i] = digit_bf16(r);
    X = (X - r) >> 8;
  }
  d[0] = digit_bf16(static_cast<int>(X));
}

// Balanced base-256 digits of rint(x 2^(48-E)), most significant first.
__device__ inline void digits(double x, int E, __nv_bfloat16* d) { digits_from_fixed(fixed_point(x, E), d); }

// Digits of 8 fixed-point values at contraction indices k0..k0+7 (k0 a
// multiple of 8) of data row r of a kNT-row tile: in the core-matrix layout
// those 8 indices are one contiguous 16-byte run per slice, so each slice is
// one vector store.  Defined after tile_elem (below).
__device__ inline void store_digits8(__nv_bfloat16* tile, int r, int k0, const long long* X);

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

// Level recombination on the f32 pipe: every accumulator holds an exact
// integer below 2^24, so acc_k 256^(5-k) is an exact float; their double-
// float sum is T to ~2^-48, and the power-of-two scaling 2^e is applied in
// two exact steps.
__device__ inline float pow2f(int p) { return __int_as_float((p + 127) << 23); }  // p in [-126, 127]

__device__ inline df levels_to_df(const float* acc, int e) {
  // pairwise: three exact two-sums of neighbouring levels, then two Dekker
  // additions (error ~2^-48 of the operands) -- half the dependency depth of
  // a sequential sum, for the latency-bound epilogue warps
  const df p0 = two_sum(acc[0] * pow2f(40), acc[1] * pow2f(32));
  const df p1 = two_sum(acc[2] * pow2f(24), acc[3] * pow2f(16));
  const df p2 = two_sum(acc[4] * pow2f(8), acc[5]);
  const df s = df_add_fast(df_add_fast(p0, p1), p2);
  // s * 2^e, e = e1 + e2 with both factors normal floats
  const int e1 = max(-126, min(127, e)), e2 = max(-126, min(127, e - e1));
  return df{s.hi * pow2f(e1) * pow2f(e2), s.lo * pow2f(e1) * pow2f(e2)};
}

// levels_to_df of two outputs at once (packed two-lane FP32; the same
// operations, so the same results).
__device__ inline void levels_to_df2(const float* a, const float* b, int ea, int eb, df& ra, df& rb) {
  const f2 c40 = f2_splat(pow2f(40)), c32 = f2_splat(pow2f(32)), c24 = f2_splat(pow2f(24));
  const f2 c16 = f2_splat(pow2f(16)), c8 = f2_splat(pow2f(8));
  const df2 p0 = two_sum2(f2_mul(f2_pack(a[0], b[0]), c40), f2_mul(f2_pack(a[1], b[1]), c32));
  const df2 p1 = two_sum2(f2_mul(f2_pack(a[2], b[2]), c24), f2_mul(f2_pack(a[3], b[3]), c16));
  const df2 p2 = two_sum2(f2_mul(f2_pack(a[4], b[4]), c8), f2_pack(a[5], b[5]));
  const df2 s = df2_add_fast(df2_add_fast(p0, p1), p2);
  const int ea1 = max(-126, min(127, ea)), ea2 = max(-126, min(127, ea - ea1));
  const int eb1 = max(-126, min(127, eb)), eb2 = max(-126, min(127, eb - eb1));
  const f2 s1 = f2_pack(pow2f(ea1), pow2f(eb1)), s2 = f2_pack(pow2f(ea2), pow2f(eb2));
  df2_unpack(df2{f2_mul(f2_mul(s.hi, s1), s2), f2_mul(f2_mul(s.lo, s1), s2)}, ra, rb);
}

// Level recombination: T = sum_k I_k 256^(5-k), k = 0..5 <-> s+t = 2..7.
// One K segment (<= 160 deep): |I_0| < 160 * 2^14, so |T| < 2^62.
__device__ inline long long combine_levels(const float* acc) {
  long long T = 0;
#pragma unroll
  for (int k = 0; k < kLevels; ++k) T = (T << 8) + __float2int_rn(acc[k]);
  return T;
}

// Exact-accumulation depth: the deepest level (6 digit pairs) sums at most
// 6 * K * 2^14 in an f32 accumulator, an exact integer while K <= 160.
constexpr int kExactChunks = 10;

// Result exponent offset: x y = T 2^(Ex + Ey - kOut).
constexpr int kOut = 2 * kShift - 8 * (kSlices - 1);

// ----------------------------------------------------------- layouts
// Every operand is stored chunk-major: for each 16-deep K chunk, the
// kSlices digit tiles (rows x 16, core-matrix layout with K = 16) are
// contiguous, so one bulk copy moves a whole pipeline stage.
struct SplitDims {
  int L, nlat, nh, NK, Mt;
  int ncol;     // data columns (members x fields x 2)
  int ntiles;   // ceil(ncol / kNT)
};

__host__ __device__ constexpr long long chunk_elems(int rows) { return (long long)kSlices * rows * kKC; }

// Synthesis basis, tile (m, latitude tile mt): chunks of 128 rows.
__host__ __device__ inline long long psyn_tile(const long long* kcum, int Mt, int m, int mt, int Kp) {
  return kcum[m] * (long long)Mt * kSlices * 128 + (long long)mt * kSlices * 128 * Kp;
}
// Analysis basis, row tile rt: NK/16 chunks of 128 degree rows.  Orders
// with more than 128 degrees (m < L - 127) take a second row tile: row
// tiles 0..L are (m = rt, degrees m..m+127), row tiles L+1.. are
// (m = rt - L - 1, degrees m+128..L).
__host__ __device__ inline long long pana_tile(int NK, int rt) { return (long long)rt * kSlices * 128 * NK; }
__host__ __device__ inline int ana_row_tiles(int L) { return L + 1 + (L > 127 ? L - 127 : 0); }
__host__ __device__ inline void ana_row_tile(int L, int rt, int& m, int& mt) {
  m = rt <= L ? rt : rt - L - 1;
  mt = rt <= L ? 0 : 1;
}
// Synthesis data, tile (m, ntile): Kp/16 chunks of kNT rows.
__host__ __device__ inline long long dsyn_tile(const long long* kcum, const SplitDims& d, int m, int ntile) {
  const int Kp = kpad(d.L + 1 - m);
  return kcum[m] * (long long)d.ntiles * kSlices * kNT + (long long)ntile * kSlices * kNT * Kp;
}
// Analysis data, tile (m, ntile): NK/16 chunks of kNT rows.
__host__ __device__ inline long long dana_tile(const SplitDims& d, int m, int ntile) {
  return ((long long)m * d.ntiles + ntile) * kSlices * kNT * (long long)d.NK;
}
// Element (row r, contraction index k) of slice s inside a tile.
__host__ __device__ inline long long tile_elem(int rows, int s, int r, int k) {
  return (long long)(k / kKC) * chunk_elems(rows) + (long long)s * rows * kKC + tc::core_index(r, k % kKC, kKC);
}

__device__ inline void store_digits8(__nv_bfloat16* tile, int r, int k0, const long long* X) {
  uint32_t w[kSlices][4];
#pragma unroll
  for (int u = 0; u < 8; u += 2) {
    __nv_bfloat16 a[kSlices], b[kSlices];
    digits_from_fixed(X[u], a);
    digits_from_fixed(X[u + 1], b);
#pragma unroll
    for (int s = 0; s < kSlices; ++s)
      w[s][u >> 1] = static_cast<uint32_t>(__bfloat16_as_ushort(a[s])) |
                     (static_cast<uint32_t>(__bfloat16_as_ushort(b[s])) << 16);
  }
  __nv_bfloat16* base = tile + tile_elem(kNT, 0, r, k0);
#pragma unroll
  for (int s = 0; s < kSlices; ++s)
    *reinterpret_cast<uint4*>(base + (long long)s * kNT * kKC) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
}

// ------------------------------------------------- synthesis data slicing
// grid (m, member chunk of `mb` members); columns (b, f, re/im).
template <class Derive>
__device__ __forceinline__ void split_synth_slice_body(const SplitDims& dm, const long long* __restrict__ kcum,
                                                       int batch, int mb, const Derive& der,
                                                       __nv_bfloat16* __restrict__ dsyn, int* __restrict__ ecol,
                                                       int bx, int by, int gy) {
  constexpr int NF = Derive::NF;
  extern __shared__ double s_val[];  // [mb*NF*2][ks]
  __shared__ int s_exp[256];
  const int m = bx, L = dm.L;
  const int K = L + 1 - m, Kp = kpad(K);
  const int ks = K | 1;  // odd row stride: column-strided reads are free of bank conflicts
  const int b0 = by * mb;
  const int nb = min(mb, batch - b0);
  const int nc = nb * NF * 2;
  constexpr bool kDf = DeriveHasDf<Derive>::value;
  float2* s_vdf = reinterpret_cast<float2*>(s_val);  // kDf: (hi, lo) in the same slots
  for (int idx = threadIdx.x; idx < nb * K; idx += blockDim.x) {
    const int bl = idx / K, t = idx - bl * K;
    if constexpr (kDf) {
      df2 v[NF];
      der.column_df(b0 + bl, m + t, m, v);
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        df re, im;
        df2_unpack(v[f], re, im);
        s_vdf[((bl * NF + f) * 2 + 0) * ks + t] = make_float2(re.hi, re.lo);
        s_vdf[((bl * NF + f) * 2 + 1) * ks + t] = make_float2(im.hi, im.lo);
      }
    } else {
      double2 v[NF];
      der.column(b0 + bl, m + t, m, v);
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        s_val[((bl * NF + f) * 2 + 0) * ks + t] = v[f].x;
        s_val[((bl * NF + f) * 2 + 1) * ks + t] = v[f].y;
      }
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int c = warp; c < nc; c += nwarp) {
    int E;
    if constexpr (kDf) {  // from the high words: |hi| < 2^(e - 126) bounds |hi + lo| too
      unsigned mx = 0u;
      for (int t = lane; t < K; t += 32) mx = max(mx, __float_as_uint(s_vdf[c * ks + t].x) & 0x7FFFFFFFu);
      mx = __reduce_max_sync(0xffffffffu, mx);
      E = (mx >> 23) == 0 ? -1000 : static_cast<int>(mx >> 23) - 125;
    } else {
      unsigned long long mx = 0ull;
      for (int t = lane; t < K; t += 32) mx = max(mx, abs_key(s_val[c * ks + t]));
      for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      E = exponent_for_key(mx);
    }
    if (lane == 0) {
      s_exp[c] = E;
      ecol[(long long)m * dm.ntiles * kNT + (long long)b0 * NF * 2 + c] = E;
    }
  }
  __syncthreads();
  // 8 consecutive degrees of one column per thread, columns fastest
  for (int idx = threadIdx.x; idx < nc * (Kp / 8); idx += blockDim.x) {
    const int g = idx / nc, c = idx - g * nc;
    const int n = b0 * NF * 2 + c, t0 = 8 * g, E = s_exp[c];
    long long X[8];
    if constexpr (kDf) {
      float pa, pb;
      fx_pow2_split(kShift - E, pa, pb);
#pragma unroll
      for (int u = 0; u < 8; ++u)
        X[u] = t0 + u < K && E != -1000 ? fixed_point_df(s_vdf[c * ks + t0 + u], pa, pb) : 0LL;
    } else {
#pragma unroll
      for (int u = 0; u < 8; ++u) X[u] = t0 + u < K ? fixed_point(s_val[c * ks + t0 + u], E) : 0LL;
    }
    store_digits8(dsyn + dsyn_tile(kcum, dm, m, n / kNT), n % kNT, t0, X);
  }
  if (by == gy - 1) {  // zero the columns that pad the last tile
    const int n0 = batch * NF * 2, n1 = dm.ntiles * kNT;
    for (int idx = threadIdx.x; idx < (n1 - n0) * Kp; idx += blockDim.x) {
      const int n = n0 + idx / Kp, t = idx % Kp;
      __nv_bfloat16* tile = dsyn + dsyn_tile(kcum, dm, m, n / kNT);
#pragma unroll
      for (int s = 0; s < kSlices; ++s) tile[tile_elem(kNT, s, n % kNT, t)] = __float2bfloat16(0.0f);
      if (t == 0) ecol[(long long)m * dm.ntiles * kNT + n] = 0;
    }
  }
}

// Four CTAs per SM (64 registers) for the FP64 derives; three (85) for the
// double-float ones, whose packed columns spill at 64 registers.
template <class Derive>
__global__ void __launch_bounds__(256, DeriveHasDf<Derive>::value ? 3 : 4) split_synth_slice_kernel(SplitDims dm, const long long* __restrict__ kcum,
                                                               int batch, int mb, Derive der,
                                                               __nv_bfloat16* __restrict__ dsyn,
                                                               int* __restrict__ ecol) {
  pdl_trigger();
  pdl_wait();
  split_synth_slice_body<Derive>(dm, kcum, batch, mb, der, dsyn, ecol, blockIdx.x, blockIdx.y, gridDim.y);
}

// ------------------------------------------------- analysis data slicing
__device__ __forceinline__ void cp_async8(void* sdst, const void* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(tc::smem_u32(sdst)), "l"(gsrc) : "memory");
}

// Reads the packed G words (fx.cuh; two per complex value), grid (m, chunk).
template <int NF>
__device__ __forceinline__ void split_anal_slice_body(const SplitDims& dm, int batch, int mb, int nblk,
                                                      const long long* __restrict__ FG, __nv_bfloat16* __restrict__ dana,
                                                      int* __restrict__ ecol, int bx, int by, int gy) {
  extern __shared__ long long s_wval[];  // [mb*NF*2][ns]
  __shared__ int s_exp[256];
  const int m = bx, L = dm.L, nlat = dm.nlat, NK = dm.NK;
  const int ns = nlat | 1;  // odd row stride: column-strided reads are free of bank conflicts
  const int b0 = by * mb;
  const int nb = min(mb, batch - b0);
  const int nc = nb * NF * 2;
  // the words go straight to shared memory (8-byte cp.async): every load of
  // the CTA is in flight at once instead of one register round trip each
  for (int idx = threadIdx.x; idx < nb * NF * nlat; idx += blockDim.x) {
    const int f = idx % NF;
    const int r = idx / NF;
    const int j = r % nlat, bl = r / nlat;
    const long long* g = FG + 2 * fg_index(b0 + bl, m, f, j, L, nblk, nlat);
    cp_async8(&s_wval[((bl * NF + f) * 2 + 0) * ns + j], g);
    cp_async8(&s_wval[((bl * NF + f) * 2 + 1) * ns + j], g + 1);
  }
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int c = warp; c < nc; c += nwarp) {
    int mx = -100000;
    for (int j = lane; j < nlat; j += 32) mx = max(mx, pk_mag(s_wval[c * ns + j]));
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) {
      const int E = mx == -100000 ? -1000 : mx + 1;  // |x| 2^-E < 1/2
      s_exp[c] = E;
      ecol[(long long)m * dm.ntiles * kNT + (long long)b0 * NF * 2 + c] = E;
    }
  }
  __syncthreads();
  // 8 consecutive latitudes of one column per thread, columns fastest;
  // X = rint(x 2^(48 - E)), |X| <= 2^47
  for (int idx = threadIdx.x; idx < nc * (NK / 8); idx += blockDim.x) {
    const int g = idx / nc, c = idx - g * nc;
    const int n = b0 * NF * 2 + c, j0 = 8 * g, S = s_exp[c] - kShift;
    long long X[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) X[u] = j0 + u < nlat ? pk_align(s_wval[c * ns + j0 + u], S) : 0LL;
    store_digits8(dana + dana_tile(dm, m, n / kNT), n % kNT, j0, X);
  }
  if (by == gy - 1) {
    const int n0 = batch * NF * 2, n1 = dm.ntiles * kNT;
    for (int idx = threadIdx.x; idx < (n1 - n0) * NK; idx += blockDim.x) {
      const int n = n0 + idx / NK, j = idx % NK;
      __nv_bfloat16* tile = dana + dana_tile(dm, m, n / kNT);
#pragma unroll
      for (int s = 0; s < kSlices; ++s) tile[tile_elem(kNT, s, n % kNT, j)] = __float2bfloat16(0.0f);
      if (j == 0) ecol[(long long)m * dm.ntiles * kNT + n] = 0;
    }
  }
}

constexpr int kAnalSliceThreads = 128;  // 8 CTAs per SM: more G loads in flight per SM
template <int NF>
__global__ void __launch_bounds__(kAnalSliceThreads, 8) split_anal_slice_kernel(SplitDims dm, int batch, int mb, int nblk,
                                                              const long long* __restrict__ FG,
                                                              __nv_bfloat16* __restrict__ dana,
                                                              int* __restrict__ ecol) {
  pdl_trigger();
  pdl_wait();
  split_anal_slice_body<NF>(dm, batch, mb, nblk, FG, dana, ecol, blockIdx.x, blockIdx.y, gridDim.y);
}

// ---------------------------------------------------- tensor-core kernels
// Persistent warp-specialised GEMM: one CTA per SM walks a static list of
// output tiles (tile t, t + gridDim.x, ...).  Each tile is a 128 x kNT
// output block contracted over nchunks 16-deep K chunks; every chunk moves
// kSlices basis tiles (128 x 16) and kSlices data tiles (kNT x 16) with two
// TMA bulk copies.
//   warp 0 lane 0   producer: streams chunks through kStages smem stages
//                   (across tile boundaries);
//   warp 1 lane 0   MMA issuer: per chunk 6 MMAs (one per basis digit slice,
//                   N = the data slices it pairs with) carry the 21 digit
//                   pairs into the kAccs level accumulators of one of two
//                   TMEM buffers;
//   warps 2..      Epi::kWarps epilogue warps drain the other TMEM buffer
//                   while the next tile's MMAs run; warp w reads TMEM lane
//                   quadrant w % 4 and the Epi::kCols-column group (w - 2) / 4.
// Barriers: full/empty per stage (TMA bytes / MMA commit), tfull/tempty per
// TMEM buffer (MMA commit / one arrival per epilogue warp).  Every wait is
// bounded: an expired wait sets *err and that role stops; the others then
// time out in turn, copies in flight are waited for and TMEM is freed.
constexpr int kStages = 6;          // smem pipeline depth (30 KB per stage)
constexpr int kTmemBuf = 256;       // column offset of the second accumulator buffer
constexpr int kTmemCols = 512;      // 2 x kAccs * kNT = 448 columns used
constexpr size_t kStageBytesA = chunk_elems(128) * 2;
constexpr size_t kStageBytesB = chunk_elems(kNT) * 2;
constexpr size_t kStageBytes = kStageBytesA + kStageBytesB;

struct TcTile {
  const __nv_bfloat16* A;  // chunk-major basis tile
  const __nv_bfloat16* B;  // chunk-major data tile
  int nchunks;
};

inline size_t tc_smem_bytes() { return 1024 + kStages * kStageBytes + 256; }

struct TcSmem {
  char* stages;
  uint64_t* full;    // [kStages]
  uint64_t* empty;   // [kStages]
  uint64_t* tfull;   // [2]
  uint64_t* tempty;  // [2]
  uint64_t* done;
  uint32_t* tmem_slot;
  __device__ __nv_bfloat16* A(int st) const {
    return reinterpret_cast<__nv_bfloat16*>(stages + (size_t)st * kStageBytes);
  }
  __device__ __nv_bfloat16* B(int st) const {
    return reinterpret_cast<__nv_bfloat16*>(stages + (size_t)st * kStageBytes + kStageBytesA);
  }
};

__device__ inline TcSmem tc_carve(char* base) {
  TcSmem s;
  char* q = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(base) + 1023) & ~uintptr_t(1023));
  s.stages = q;
  q += kStages * kStageBytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(q);
  s.full = bars;
  s.empty = bars + kStages;
  s.tfull = bars + 2 * kStages;
  s.tempty = bars + 2 * kStages + 2;
  s.done = bars + 2 * kStages + 4;
  s.tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 5);
  return s;
}

// The kAccs accumulators of 16 columns starting at c0 for lane `lane` of the
// TMEM quadrant q (the calling warp's own quadrant).
// NC (8 or 16) columns of all kAccs accumulators: every load is issued
// before one wait (one TMEM round trip); the register fences keep every use
// of the loaded values after the wait.
template <int NC>
__device__ inline void tc_read(uint32_t tbuf, int q, int c0, float (*acc)[kAccs]) {
  static_assert(NC == 8 || NC == 16, "8 or 16 columns");
  const uint32_t lane_base = (uint32_t)(q * 32) << 16;
  uint32_t r[kAccs][NC];
#pragma unroll
  for (int k = 0; k < kAccs; ++k) {
    if constexpr (NC == 16) tc::tmem_ld16(tbuf + lane_base + (uint32_t)(k * kNT + c0), r[k]);
    else tc::tmem_ld8(tbuf + lane_base + (uint32_t)(k * kNT + c0), r[k]);
  }
  if constexpr (NC == 16) tc::tmem_wait_ld_dep(r[0]);
  else tc::tmem_wait_ld_dep8(r[0]);
#pragma unroll
  for (int k = 1; k < kAccs; ++k) {
    if constexpr (NC == 16) tc::reg_fence16(r[k]);
    else tc::reg_fence8(r[k]);
  }
#pragma unroll
  for (int k = 0; k < kAccs; ++k)
#pragma unroll
    for (int i = 0; i < NC; ++i) acc[i][k] = __uint_as_float(r[k][i]);
}

template <class Epi>
constexpr int tc_threads() { return 64 + 32 * Epi::kWarps; }

// Epilogues with a Pre type load their per-tile inputs that do not depend on
// the accumulators (prefetch) before waiting for them, so those global
// loads are off the path from "accumulators ready" to "buffer released".
template <class E, class = void>
struct EpiHasPre : std::false_type {};
template <class E>
struct EpiHasPre<E, std::void_t<typename E::Pre>> : std::true_type {};
// K-segmented epilogues may load the same kind of inputs into their State
// (seg_prefetch) before the first segment's wait.
template <class E, class = void>
struct EpiHasSegPrefetch : std::false_type {};
template <class E>
struct EpiHasSegPrefetch<E, std::void_t<decltype(std::declval<const E&>().seg_prefetch(
                                std::declval<typename E::State&>(), 0, 0, 0))>> : std::true_type {};

// Sched: int count() const; TcTile tile(int t) const; kSegChunks (0: one
//        K segment per tile, else K segments of that many chunks).
// Epi:   kWarps (4, 8 or 16 epilogue warps), kCols = 4 kNT / kWarps, and
//        template <class Rel> void run(int t, uint32_t tbuf, int q, int row,
//        int c0, int etid, Rel release) const -- consumes columns
//        [c0, c0 + kCols) of the accumulators of tile t for TMEM lane
//        row = q * 32 + lane (etid = epilogue thread index) and calls
//        release() once they are in registers (the buffer goes back to the
//        MMA warp before the epilogue's math and stores);
//        with K segments instead State, seg_begin(State&), seg_add(State&,
//        tbuf, q, c0) per segment and seg_end(t, State, row, c0, etid).
template <class Sched, class Epi>
__global__ void __launch_bounds__(tc_threads<Epi>(), 1) tc_persistent_kernel(Sched sc, Epi ep, int* err) {
  extern __shared__ char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const TcSmem sm = tc_carve(smem_raw);
  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; ++i) {
      tc::mbar_init(&sm.full[i], 1);
      tc::mbar_init(&sm.empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&sm.tfull[i], 1);
      tc::mbar_init(&sm.tempty[i], Epi::kWarps);
    }
    tc::mbar_init(sm.done, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(sm.tmem_slot, kTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *sm.tmem_slot;
  const int ntiles = sc.count();
  pdl_trigger();
  pdl_wait();  // global memory only from here on

  if (warp == 0) {
    if (lane == 0) {  // ---------------- producer
      bool ok = true;
      uint32_t g = 0;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const TcTile tl = sc.tile(t);
        for (int kc = 0; kc < tl.nchunks; ++kc) {
          const int st = (int)(g % kStages);
          const uint32_t u = g / kStages;
          if (u > 0 && !tc::mbar_wait(&sm.empty[st], (u - 1) & 1)) {
            ok = false;
            break;
          }
          tc::mbar_expect_tx(&sm.full[st], (uint32_t)kStageBytes);
          tc::bulk_g2s(sm.A(st), tl.A + (long long)kc * chunk_elems(128), (uint32_t)kStageBytesA, &sm.full[st]);
          tc::bulk_g2s(sm.B(st), tl.B + (long long)kc * chunk_elems(kNT), (uint32_t)kStageBytesB, &sm.full[st]);
          ++g;
        }
      }
      // no copy may still be in flight when the CTA ends
      for (uint32_t h = g > (uint32_t)kStages ? g - kStages : 0; h < g; ++h)
        if (!tc::mbar_wait(&sm.full[h % kStages], (h / kStages) & 1)) ok = false;
      if (!ok) atomicExch(err, 1);
    }
  } else if (warp == 1) {
    if (lane == 0) {  // ---------------- MMA issuer
      // Digit slices are concatenated along N: the data tile of a stage is
      // the kSlices slices (kNT rows each) back to back, so one MMA per basis
      // slice s multiplies it by data slices 0..5-s (N = (6-s) kNT) and writes
      // levels s..5 at TMEM column s * kNT onwards: 6 MMAs per chunk carry
      // the 21 digit pairs.  Descriptors differ between stages and slices
      // only in the start-address field (stage/slice byte offsets >> 4 added
      // to the descriptors of stage 0, slice 0; smem addresses < 256 KB).
      bool ok = true;
      const uint64_t dA0 = tc::smem_desc(sm.A(0), 128, kKC * 16);
      const uint64_t dB0 = tc::smem_desc(sm.B(0), 128, kKC * 16);
      uint32_t g = 0;
      int i = 0;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const TcTile tl = sc.tile(t);
        // K segments of one tile: each is contracted into a fresh accumulator
        // buffer and drained by the epilogue (one segment unless the
        // schedule bounds the depth of an exact f32 sum)
        const int segc = Sched::kSegChunks > 0 ? Sched::kSegChunks : tl.nchunks;
        for (int k0 = 0; k0 < tl.nchunks && ok; k0 += segc, ++i) {
          const int buf = i & 1;
          const uint32_t ub = (uint32_t)i >> 1;
          if (ub > 0 && !tc::mbar_wait(&sm.tempty[buf], (ub - 1) & 1)) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint32_t dbase = tmem + (uint32_t)(buf * kTmemBuf);
          const int k1 = min(tl.nchunks, k0 + segc);
          for (int kc = k0; kc < k1; ++kc, ++g) {
            const int st = (int)(g % kStages);
            if (!tc::mbar_wait(&sm.full[st], (g / kStages) & 1)) {
              ok = false;
              break;
            }
            tc::fence_after_sync();
            const uint64_t off = (uint64_t)(((size_t)st * kStageBytes) >> 4);
            const uint64_t da0 = dA0 + off, db = dB0 + off;
#pragma unroll
            for (int sl = 0; sl < kSlices; ++sl) {
              const uint64_t da = da0 + (uint64_t)(((size_t)sl * 128 * kKC * 2) >> 4);
              tc::mma_bf16(dbase + (uint32_t)(sl * kNT), da, db, tc::idesc_bf16_f32(128, (kSlices - sl) * kNT),
                           (kc > k0 || sl > 0) ? 1u : 0u);
            }
            tc::mma_commit(&sm.empty[st]);
          }
          if (!ok) break;
          tc::mma_commit(&sm.tfull[buf]);
        }
      }
      // every MMA issued has completed before TMEM is released
      tc::mma_commit(sm.done);
      if (!tc::mbar_wait(sm.done, 0)) ok = false;
      if (!ok) atomicExch(err, 3);
    }
  } else {  // ------------------------ epilogue warps
    const int q = warp & 3;
    const int c0 = ((warp - 2) >> 2) * Epi::kCols;
    const int etid = (warp - 2) * 32 + lane;
    int i = 0;
    bool ok = true;
    // lane 0 waits and the warp follows its verdict, so the warp stays
    // converged for the .sync.aligned TMEM loads
    auto wait_full = [&](int unit) {
      int ready = 0;
      if (lane == 0) ready = tc::mbar_wait(&sm.tfull[unit & 1], ((uint32_t)unit >> 1) & 1) ? 1 : 0;
      ready = __shfl_sync(0xffffffffu, ready, 0);
      if (!ready && lane == 0) atomicExch(err, 2);
      return ready != 0;
    };
    auto release = [&](int unit) {
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&sm.tempty[unit & 1]);
    };
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      if constexpr (Sched::kSegChunks > 0) {
        const int nseg = (sc.tile(t).nchunks + Sched::kSegChunks - 1) / Sched::kSegChunks;
        typename Epi::State es;
        ep.seg_begin(es);
        if constexpr (EpiHasSegPrefetch<Epi>::value) ep.seg_prefetch(es, t, q * 32 + lane, c0);
        for (int sg = 0; sg < nseg; ++sg, ++i) {
          if (!(ok = wait_full(i))) break;
          tc::fence_after_sync();
          ep.seg_add(es, tmem + (uint32_t)((i & 1) * kTmemBuf), q, c0);
          release(i);
        }
        if (ok) ep.seg_end(t, es, q * 32 + lane, c0, etid);
      } else {
        // the epilogue hands the buffer back as soon as its accumulators are
        // in registers, so the next tile's MMAs overlap its math and stores
        const int unit = i;
        if constexpr (EpiHasPre<Epi>::value) {
          const typename Epi::Pre pre = ep.prefetch(t, q * 32 + lane, c0);
          if (!(ok = wait_full(i))) break;
          tc::fence_after_sync();
          ep.run(t, tmem + (uint32_t)((i & 1) * kTmemBuf), q, q * 32 + lane, c0, etid, [&] { release(unit); }, pre);
        } else {
          if (!(ok = wait_full(i))) break;
          tc::fence_after_sync();
          ep.run(t, tmem + (uint32_t)((i & 1) * kTmemBuf), q, q * 32 + lane, c0, etid, [&] { release(unit); });
        }
        ++i;
      }
    }
  }
  // reconverge each warp (lanes 1..31 of warps 0 and 1 wait here for their
  // lane 0) before the CTA barrier and the warp-wide TMEM release
  __syncwarp();
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// --------------------------------------------------------- synthesis GEMM
// Tiles (m, latitude tile, data tile), m-major so tiles of equal depth are
// adjacent (largest depth first: a greedy balance of the static schedule).
struct SynthSched {
  static constexpr int kSegChunks = 0;  // K <= 160: one exact segment per tile
  SplitDims dm;
  const long long* kcum;
  const __nv_bfloat16* psyn;
  const __nv_bfloat16* dsyn;
  __host__ __device__ int count() const { return (dm.L + 1) * dm.Mt * dm.ntiles; }
  int count_host() const { return count(); }
  __device__ TcTile tile(int t) const {
    const int per_m = dm.Mt * dm.ntiles;
    const int m = t / per_m, r = t - m * per_m;
    const int mt = r / dm.ntiles, nt = r - mt * dm.ntiles;
    const int Kp = kpad(dm.L + 1 - m);
    return TcTile{psyn + psyn_tile(kcum, dm.Mt, m, mt, Kp), dsyn + dsyn_tile(kcum, dm, m, nt), Kp / kKC};
  }
};

// Spectra blocks written by the synthesis epilogue for a Derive's NF
// contracted fields: by default field f -> block f.  A Derive may declare
// NBLK blocks, blk(f) and lam_blk(f) >= 0 for fields whose order spectra
// times i m / R (a longitude derivative, diagonal in m) fill a further block.
// Identity placement of NF fields.
template <int NF>
struct SynthOutPlain {
  static constexpr int NBLK = NF;
  static constexpr bool kLam = false;
  __host__ __device__ static constexpr int blk(int f) { return f; }
  __host__ __device__ static constexpr int lam_blk(int) { return -1; }
};
template <class Derive, class = void>
struct SynthOut {
  static constexpr int NBLK = Derive::NF;
  static constexpr bool kLam = false;
  __host__ __device__ static constexpr int blk(int f) { return f; }
  __host__ __device__ static constexpr int lam_blk(int) { return -1; }
  static double ir(const Derive&) { return 0.0; }
};
template <class Derive>
struct SynthOut<Derive, std::void_t<decltype(Derive::NBLK)>> {
  static constexpr int NBLK = Derive::NBLK;
  static constexpr bool kLam = true;
  __host__ __device__ static constexpr int blk(int f) { return Derive::blk(f); }
  __host__ __device__ static constexpr int lam_blk(int f) { return Derive::lam_blk(f); }
  static double ir(const Derive& d) { return d.lam_ir(); }
};

// Writes the F blocks as double-floats (float4 = re.hi, re.lo, im.hi, im.lo per
// complex value); NF contracted fields, placed by Out (SynthOut).
template <int NF, class Out = SynthOutPlain<NF>>
struct SynthEpi {
  static constexpr int kWarps = 16, kCols = 4 * kNT / kWarps;
  SplitDims dm;
  const int* esyn;
  const int* ecol;
  int nblk;
  float4* F;
  float ir_hi = 0.f, ir_lo = 0.f;  // 1 / R as a double-float (Out::kLam)
  struct Pre {
    int e[kCols];  // result exponents of this thread's outputs
  };
  __device__ Pre prefetch(int t, int row, int c0) const {
    const int per_m = dm.Mt * dm.ntiles;
    const int m = t / per_m, r = t - m * per_m;
    const int mt = r / dm.ntiles, tile = r - mt * dm.ntiles;
    const int j = mt * 128 + row;
    const int Ej = j < dm.nlat ? esyn[m * dm.Mt * 128 + j] : 0;
    const int* ec = ecol + (long long)m * dm.ntiles * kNT + tile * kNT + c0;
    Pre p;
#pragma unroll
    for (int i = 0; i < kCols; ++i) p.e[i] = Ej + __ldg(ec + i) - kOut;
    return p;
  }
  template <class Rel>
  __device__ void run(int t, uint32_t tbuf, int q, int row, int c0, int, Rel release, const Pre& pre) const {
    const int per_m = dm.Mt * dm.ntiles;
    const int m = t / per_m, r = t - m * per_m;
    const int mt = r / dm.ntiles, tile = r - mt * dm.ntiles;
    const int j = mt * 128 + row;
    float acc[kCols][kAccs];
    tc_read<kCols>(tbuf, q, c0, acc);
    release();
    if (j >= dm.nlat) return;
    // every recombination first (independent dependency chains that the
    // compiler interleaves), then the stores
    df v[kCols];
#pragma unroll
    for (int i = 0; i < kCols; i += 2) levels_to_df2(acc[i], acc[i + 1], pre.e[i], pre.e[i + 1], v[i], v[i + 1]);
    // F block of (member b, order m, row j): fg_index, with b advanced per column pair
    const long sb = (long)(dm.L + 1) * dm.nlat * nblk;
    float4* Fj = F + ((long)m * dm.nlat + j) * nblk;
    const int k0 = (tile * kNT + c0) >> 1;  // first complex column (member, field) of this thread
    int b = k0 / NF, f = k0 - b * NF;
    df mr = df{0.f, 0.f};
    if constexpr (Out::kLam) {  // m / R on the f32 pipe (m exact as a float; no FP64 instruction)
      const float mf = __int_as_float(0x4B000000 | m) - 8388608.0f;
      const float ph = mf * ir_hi;
      mr = df{ph, fmaf(mf, ir_hi, -ph) + mf * ir_lo};
    }
#pragma unroll
    for (int i = 0; i < kCols; i += 2) {
      if (tile * kNT + c0 + i < dm.ncol) {  // even: real part, odd: imaginary part
        float4* Fb = Fj + (long)b * sb;
        Fb[Out::blk(f)] = make_float4(v[i].hi, v[i].lo, v[i + 1].hi, v[i + 1].lo);
        if constexpr (Out::kLam) {
          // the columns of a warp are one field for all its lanes: no divergence
          const int lb = Out::lam_blk(f);
          if (lb >= 0) {
            const df lre = df_neg(df_mul(v[i + 1], mr)), lim = df_mul(v[i], mr);
            Fb[lb] = make_float4(lre.hi, lre.lo, lim.hi, lim.lo);
          }
        }
      }
      if (++f == NF) {
        f = 0;
        ++b;
      }
    }
  }
};

// --------------------------------------------------------- analysis GEMM
struct AnalSched {
  static constexpr int kSegChunks = kExactChunks;  // K = nlat <= 192: one or two exact segments
  SplitDims dm;
  const __nv_bfloat16* pana;
  const __nv_bfloat16* dana;
  __host__ __device__ int count() const { return ana_row_tiles(dm.L) * dm.ntiles; }
  int count_host() const { return count(); }
  __device__ TcTile tile(int t) const {
    const int rt = t / dm.ntiles, nt = t - rt * dm.ntiles;
    int m, mt;
    ana_row_tile(dm.L, rt, m, mt);
    return TcTile{pana + pana_tile(dm.NK, rt), dana + dana_tile(dm, m, nt), dm.NK / kKC};
  }
};

// Row = degree offset l - m.  Exact 64-bit level recombination summed over
// the (at most two) K segments, FP64 epilogue functor (whole members:
// Epi::finish; else Epi::finish_field).
template <class Epi>
struct AnalEpi {
  static constexpr int kWarps = 16, kCols = 4 * kNT / kWarps;  // FP64 epilogue: 8 columns per warp
  struct State {
    long long T[kCols];
    int e[kCols];  // result exponents of this thread's outputs (loaded before the first wait)
  };
  SplitDims dm;
  const int* eana;
  const int* ecol;
  int batch;
  Epi epi;
  __device__ void seg_begin(State& st) const {
#pragma unroll
    for (int i = 0; i < kCols; ++i) st.T[i] = 0;
  }
  __device__ void seg_prefetch(State& st, int tt, int row, int c0) const {
    const int rt = tt / dm.ntiles, tile = tt - rt * dm.ntiles;
    int m, mt;
    ana_row_tile(dm.L, rt, m, mt);
    const int Et = eana[rt * 128 + row];
    const int* ec = ecol + (long long)m * dm.ntiles * kNT + tile * kNT + c0;
#pragma unroll
    for (int i = 0; i < kCols; ++i) st.e[i] = Et + __ldg(ec + i) - kOut;
  }
  __device__ void seg_add(State& st, uint32_t tbuf, int q, int c0) const {
    float acc[kCols][kAccs];
    tc_read<kCols>(tbuf, q, c0, acc);
#pragma unroll
    for (int i = 0; i < kCols; ++i) st.T[i] += combine_levels(acc[i]);
  }
  __device__ void seg_end(int tt, const State& st, int row, int c0, int etid) const {
    constexpr int NF = Epi::NF;
    constexpr bool kWhole = kCols % (2 * NF) == 0;
    const int rt = tt / dm.ntiles, tile = tt - rt * dm.ntiles;
    int m, mt;
    ana_row_tile(dm.L, rt, m, mt);
    const int K = dm.L + 1 - m;
    const int t = mt * 128 + row;  // degree offset l - m
    if (t < K) {
      if constexpr (kWhole) {
#pragma unroll
        for (int i = 0; i < kCols; i += 2 * NF) {
          const int n = tile * kNT + c0 + i;
          const int b = n / (2 * NF);
          if (b >= batch) break;
          double2 a[NF];
#pragma unroll
          for (int f = 0; f < NF; ++f) {
            a[f].x = scaled_to_double(st.T[i + 2 * f], st.e[i + 2 * f]);
            a[f].y = scaled_to_double(st.T[i + 2 * f + 1], st.e[i + 2 * f + 1]);
          }
          epi.finish(b, m + t, m, a);
        }
      } else {
#pragma unroll
        for (int i = 0; i < kCols; i += 2) {
          const int n = tile * kNT + c0 + i;
          const int bf = n >> 1;
          const int b = bf / NF, f = bf - b * NF;
          if (b >= batch) break;
          double2 a;
          a.x = scaled_to_double(st.T[i], st.e[i]);
          a.y = scaled_to_double(st.T[i + 1], st.e[i + 1]);
          epi.finish_field(b, f, m + t, m, a);
        }
      }
    }
    // slots l < m of column m for the members this tile touches (once per order)
    if (mt == 0) {
      const int mb0 = tile * kNT / (2 * NF), mb1 = min(batch, ((tile + 1) * kNT + 2 * NF - 1) / (2 * NF));
      for (int idx = etid; idx < (mb1 - mb0) * m; idx += 32 * kWarps) epi.zero(mb0 + idx / m, idx % m, m);
    }
  }
};

inline int tc_grid(const aeolus_plan_impl* p, int ntiles) { return std::max(1, std::min(ntiles, p->sm_count)); }

// ------------------------------------------------------------ launchers
inline SplitDims split_dims(const aeolus_plan_impl* p, int ncol) {
  const SplitTables* t = p->split;
  return SplitDims{t->L, t->nlat, t->nh, t->NK, t->Mt, ncol, (ncol + kNT - 1) / kNT};
}

inline size_t split_synth_bytes(const aeolus_plan_impl* p, int nf, int batch) {
  const SplitDims d = split_dims(p, batch * nf * 2);
  return align256((size_t)p->split->h_kcum[d.L + 1] * d.ntiles * kSlices * kNT * 2) +
         align256((size_t)(d.L + 1) * d.ntiles * kNT * 4);
}

inline size_t split_anal_bytes(const aeolus_plan_impl* p, int nf, int batch) {
  const SplitDims d = split_dims(p, batch * nf * 2);
  return align256((size_t)(d.L + 1) * d.ntiles * kSlices * kNT * d.NK * 2) +
         align256((size_t)(d.L + 1) * d.ntiles * kNT * 4);
}

inline int slice_members(int nf, int K, int tuned, int cap_bytes = 64 * 1024) {
  // members per slicing CTA: at most 256 columns (the exponent array) and the
  // staged values within cap_bytes, or the tuned count within 160 KB
  const int cap_cols = std::max(1, 256 / (2 * nf));
  if (tuned > 0) return std::max(1, std::min({tuned, cap_cols, (160 * 1024) / (2 * nf * K * 8)}));
  return std::max(1, std::min(cap_cols, cap_bytes / (2 * nf * K * 8)));
}

// Scratch carving and slicing shapes of the two split stages.
struct SplitParts {
  SplitDims dm;
  __nv_bfloat16* digits;  // data digit planes
  int* ecol;              // per-column exponents
  int mb;                 // members per slicing CTA
  size_t smem;            // slicing kernel dynamic shared memory
  dim3 grid;              // slicing grid
};

template <int NF>
SplitParts split_synth_parts(const aeolus_plan_impl* p, int batch, void* scratch) {
  SplitParts r;
  r.dm = split_dims(p, batch * NF * 2);
  char* w = static_cast<char*>(scratch);
  r.digits = reinterpret_cast<__nv_bfloat16*>(w);
  w += align256((size_t)p->split->h_kcum[r.dm.L + 1] * r.dm.ntiles * kSlices * kNT * 2);
  r.ecol = reinterpret_cast<int*>(w);
  // 32 KB of staged values: four 256-thread CTAs per SM (64 registers each)
  r.mb = slice_members(NF, r.dm.L + 2, p->tune_slice_mb, 32 * 1024);
  r.smem = (size_t)r.mb * NF * 2 * ((r.dm.L + 1) | 1) * 8;
  r.grid = dim3(r.dm.L + 1, (batch + r.mb - 1) / r.mb);
  return r;
}

template <int NF>
SplitParts split_anal_parts(const aeolus_plan_impl* p, int batch, void* scratch) {
  SplitParts r;
  r.dm = split_dims(p, batch * NF * 2);
  char* w = static_cast<char*>(scratch);
  r.digits = reinterpret_cast<__nv_bfloat16*>(w);
  w += align256((size_t)(r.dm.L + 1) * r.dm.ntiles * kSlices * kNT * r.dm.NK * 2);
  r.ecol = reinterpret_cast<int*>(w);
  r.mb = slice_members(NF, r.dm.nlat + 1, p->tune_slice_mb_anal);
  r.smem = (size_t)r.mb * NF * 2 * (r.dm.nlat | 1) * 8;
  r.grid = dim3(r.dm.L + 1, (batch + r.mb - 1) / r.mb);
  return r;
}

template <class Derive>
int launch_split_synth(const aeolus_plan_impl* p, const Derive& d, double2* FG, int nblk, int batch, void* scratch,
                       cudaStream_t st) {
  constexpr int NF = Derive::NF;
  const SplitParts r = split_synth_parts<NF>(p, batch, scratch);
  auto k1 = split_synth_slice_kernel<Derive>;
  int s = allow_smem(k1, r.smem);
  if (s) return s;
  {
    ProfScope prof("split_synth_slice", st);
    launch_pdl(k1, r.grid, dim3(256), r.smem, st, r.dm, p->split->kcum, batch, r.mb, d, r.digits, r.ecol);
    AE_LAUNCH("split_synth_slice_kernel");
  }
  const size_t sm2 = tc_smem_bytes();
  using Out = SynthOut<Derive>;
  using Epi = SynthEpi<NF, Out>;
  auto k2 = tc_persistent_kernel<SynthSched, Epi>;
  if ((s = allow_smem(k2, sm2))) return s;
  const SynthSched sc{r.dm, p->split->kcum, p->split->psyn, r.digits};
  Epi ep{r.dm, p->split->esyn, r.ecol, nblk, reinterpret_cast<float4*>(FG)};
  ep.ir_hi = (float)Out::ir(d);
  ep.ir_lo = (float)(Out::ir(d) - (double)ep.ir_hi);
  ProfScope prof("tc_synth_bf16x6", st);
  launch_pdl(k2, dim3(tc_grid(p, sc.count_host())), dim3(tc_threads<Epi>()), sm2, st, sc, ep, p->split->err);
  AE_LAUNCH("tc_synth_kernel");
  return AEOLUS_OK;
}

template <class Epi>
int launch_split_anal(const aeolus_plan_impl* p, const Epi& e, const double2* FG, int nblk, int batch, void* scratch,
                      cudaStream_t st) {
  constexpr int NF = Epi::NF;
  const SplitParts r = split_anal_parts<NF>(p, batch, scratch);
  auto k1 = split_anal_slice_kernel<NF>;
  int s = allow_smem(k1, r.smem);
  if (s) return s;
  {
    ProfScope prof("split_anal_slice", st);
    launch_pdl(k1, r.grid, dim3(kAnalSliceThreads), r.smem, st, r.dm, batch, r.mb, nblk, reinterpret_cast<const long long*>(FG),
               r.digits, r.ecol);
    AE_LAUNCH("split_anal_slice_kernel");
  }
  const size_t sm2 = tc_smem_bytes();
  auto k2 = tc_persistent_kernel<AnalSched, AnalEpi<Epi>>;
  if ((s = allow_smem(k2, sm2))) return s;
  const AnalSched sc{r.dm, p->split->pana, r.digits};
  const AnalEpi<Epi> ep{r.dm, p->split->eana, r.ecol, batch, e};
  ProfScope prof("tc_anal_bf16x6", st);
  launch_pdl(k2, dim3(tc_grid(p, sc.count_host())), dim3(tc_threads<AnalEpi<Epi>>()), sm2, st, sc, ep, p->split->err);
  AE_LAUNCH("tc_anal_kernel");
  return AEOLUS_OK;
}

}  // namespace aeolus
