// Longitude stage of the split-precision path for half-length transforms
// n = R0 x R1 x R2 (nlon = 2n) with R0 in {1, 3, 5} and R1 R2 = 32 or 64:
// the same arithmetic kinds as row_fx8_body (64-bit fixed-point FFTs,
// double-float products), with
//  * prime-factor (Good-Thomas) transforms: n = R0 x P with R0 and P = R1 R2
//    coprime needs no twiddles between the radix-R0 pass and the P-point
//    transforms, so only the one twiddled pass inside each P-point transform
//    multiplies -- 147 twiddle products per 192-point transform against 273
//    for the 3 x 8 x 8 Cooley-Tukey order;
//  * index maps: spectrum index q sits in block (P^-1 q) mod R0 at position
//    rev(R0^-1 q mod P) (rev: the mixed-radix digit reversal n2 ->
//    R2 (n2 mod R1) + n2 div R1), grid index i in block i mod R0 at position
//    i mod P.  The inverse transform reads the spectrum map and writes the
//    grid map, the forward transform reads the grid map and writes the
//    spectrum map, so the pointwise products stay in place.  Positions inside
//    a block are XOR-swizzled (u ^ (u >> 3) in the low octal digit) so the
//    radix-8 passes and the radix-R0 pass touch 8 distinct 16-byte bank
//    groups per 8-lane phase;
//  * the row's spectra staged once into shared memory by cp.async, each at
//    the slot of the thread that consumes it, while the row constants are
//    formed; block exponents and the real-FFT pre-processing then read
//    shared memory;
//  * phases split so that their item counts fill the 128 threads (pre-
//    processing pairs: n/2 + 1 per field; radix-R0: P per field), and the
//    radix-R0 pass of the forward transform fused into its post-processing
//    (P/2 items per field: the order groups c + jP and P - c + jP);
//  * the pointwise products of functors that provide df_op2 run two grid
//    points at a time on the packed two-lane f32 pipe (fx_to_df2, df2).
// The arithmetic of each butterfly, pre- and post-processing step and
// product is that of row_fx8_body; only the FFT factorisation (and so the
// rounding order) differs.
#pragma once

#include <type_traits>

#include "rows_fx.cuh"

namespace aeolus {

constexpr int pfa_inv_mod(int a, int m) {
  for (int x = 0; x < m; ++x)
    if ((a * x) % m == 1 % m) return x;
  return 0;
}
constexpr int pfa_ceil_log2(int v) {
  int b = 0;
  while ((1 << b) < v) ++b;
  return b;
}

template <int R0_, int R1_, int R2_>
struct PfaShape {
  static constexpr int R0 = R0_, R1 = R1_, R2 = R2_, P = R1 * R2, n = R0 * P, N = 2 * n, fs = n + 1;
  static constexpr int hb = 56 - pfa_ceil_log2(n) < 52 ? 56 - pfa_ceil_log2(n) : 52;  // |FFT input| < 2^hb
  static constexpr int Pinv = pfa_inv_mod(P, R0), R0inv = pfa_inv_mod(R0, P);
  static_assert(R2 == 8 && (R1 == 4 || R1 == 8), "P-point transforms of 4 x 8 or 8 x 8 points");
  static_assert(R0 == 1 || R0 == 3 || R0 == 5, "radix-R0 pass of 1, 3 or 5");
  static __device__ __forceinline__ int sw(int u) { return (u & ~7) | ((u ^ (u >> 3)) & 7); }
  static __device__ __forceinline__ int upos(int q) {
    const int n2 = (R0inv * q) & (P - 1);
    return sw(R2 * (n2 & (R1 - 1)) + n2 / R1);
  }
  static __device__ __forceinline__ int spec(int q) { return R0 == 1 ? upos(q) : ((Pinv * q) % R0) * P + upos(q); }
  static __device__ __forceinline__ int grid(int i) { return R0 == 1 ? sw(i) : (i % R0) * P + sw(i & (P - 1)); }
  static bool matches(const FftInfo& f) { return f.use_fft && f.n == n; }
};
using Pfa192 = PfaShape<3, 8, 8>;  // nlon 384
using Pfa160 = PfaShape<5, 4, 8>;  // nlon 320
using Pfa96 = PfaShape<3, 4, 8>;   // nlon 192
using Pfa64 = PfaShape<1, 8, 8>;   // nlon 128
using Pfa32 = PfaShape<1, 4, 8>;   // nlon 64
constexpr int kPfaThreads = 128;
static_assert(kPfaThreads == kFx8Threads, "the grouped row kernel runs both bodies with one block size");

__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(sdst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;" ::: "memory");
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// df_to_fx of a complex double-float (float4: re.hi, re.lo, im.hi, im.lo),
// the float steps of both parts on the packed two-lane pipe.
__device__ __forceinline__ cfx df_to_fx2(float4 w, f2 pa, f2 pb) {
  const f2 th = f2_mul(f2_mul(f2_pack(w.x, w.z), pa), pb), tl = f2_mul(f2_mul(f2_pack(w.y, w.w), pa), pb);
  const f2 c15 = f2_splat(12582912.0f);  // 1.5 2^23
  const f2 um = f2_fma(th, f2_splat(9.31322574615478515625e-10f), c15);
  const f2 r = f2_fma(f2_neg(f2_sub(um, c15)), f2_splat(1073741824.0f), th);
  float um0, um1, r0, r1, tl0, tl1;
  f2_unpack(um, um0, um1);
  f2_unpack(r, r0, r1);
  f2_unpack(tl, tl0, tl1);
  const int u0 = __float_as_int(um0) - 0x4B400000, u1 = __float_as_int(um1) - 0x4B400000;
  return cfx{fx_madw(u0, 1 << 30, static_cast<long long>(__float2int_rn(r0) + __float2int_rn(tl0))),
             fx_madw(u1, 1 << 30, static_cast<long long>(__float2int_rn(r1) + __float2int_rn(tl1)))};
}

// fx_to_df of two values, the float steps packed.
__device__ __forceinline__ df2 fx_to_df2(long long X0, long long X1, f2 pa, f2 pb) {
  const unsigned l0 = static_cast<unsigned>(X0), h0 = static_cast<unsigned>(X0 >> 32);
  const unsigned l1 = static_cast<unsigned>(X1), h1 = static_cast<unsigned>(X1 >> 32);
  const unsigned a0 = l0 & 0xFFFFFu, b0 = l1 & 0xFFFFFu;
  const unsigned a1 = __funnelshift_r(l0, h0, 20) & 0xFFFFFu, b1 = __funnelshift_r(l1, h1, 20) & 0xFFFFFu;
  const int a2 = static_cast<int>(X0 >> 40), b2 = static_cast<int>(X1 >> 40);
  const f2 f0 = f2_sub(f2_pack(__int_as_float(0x4B000000 | a0), __int_as_float(0x4B000000 | b0)), f2_splat(8388608.0f));
  const f2 f1 = f2_sub(f2_pack(__int_as_float((170u << 23) | a1), __int_as_float((170u << 23) | b1)),
                       f2_splat(8796093022208.0f));
  const f2 fh = f2_sub(f2_pack(__int_as_float((190 << 23) + 0x400000 + a2), __int_as_float((190 << 23) + 0x400000 + b2)),
                       f2_splat(13835058055282163712.0f));
  const f2 s = f2_add(fh, f1);
  const f2 e1 = f2_sub(f1, f2_sub(s, fh));
  const f2 t = f2_add(e1, f0);
  const f2 h = f2_add(s, t);
  const f2 l = f2_sub(t, f2_sub(h, s));
  return df2{f2_mul(f2_mul(h, pa), pb), f2_mul(f2_mul(l, pa), pb)};
}

// Functors with a packed two-point product (df_op2).
template <class Pw, class = void>
struct PwHasPairs : std::false_type {};
template <class Pw>
struct PwHasPairs<Pw, std::void_t<decltype(&Pw::df_op2)>> : std::true_type {};

// One pass over the P-point blocks of NFLD (member row, field) pairs.  PASS1: R1 butterflies
// of radix R2 over R2 consecutive positions, no twiddles; otherwise R2
// butterflies of radix R1 at stride R2 with the twiddles w_P^(a k) before
// the butterfly (inverse, DIT) or after it (forward, DIF).  The inverse runs
// PASS1 then the strided pass, the forward the strided pass then PASS1.
// CONV: the rows still hold double-floats, rounded to the field's fixed-
// point scale (pa pb = 2^-S) as they are loaded.
template <class S, bool INV, bool PASS1, bool CONV, int NFLD, int NPER, int RS>
__device__ __forceinline__ void pfa_pass(cfx* __restrict__ x, const FxW* __restrict__ tw, const FxConst& kc,
                                         const float* sqa, const float* sqb) {
  constexpr int R = PASS1 ? S::R2 : S::R1;        // butterfly radix
  constexpr int NB = PASS1 ? S::R1 : S::R2;       // butterflies per block
  constexpr int TWS = 2 * S::R0;                  // w_P = w_N^(N / P)
#pragma unroll 1
  for (int idx = threadIdx.x; idx < NFLD * S::R0 * NB; idx += kPfaThreads) {
    // f: (member row, field) pair, NPER fields of each row's RS slots
    const int f = idx / (S::R0 * NB), rem = idx - f * (S::R0 * NB), r = rem / NB, k = rem - r * NB;
    cfx* y = x + (NFLD == NPER ? f * S::fs : (f / NPER) * RS + (f % NPER) * S::fs) + r * S::P;
    // swizzled positions, R2 = 8: sw(8k + t) = 8k + (t ^ k), sw(8t + k) = 8t + (k ^ t)
    auto pos = [&](int t) { return PASS1 ? 8 * k + (t ^ k) : 8 * t + (k ^ t); };
    cfx v[R];
    if constexpr (CONV) {
      const f2 pa = f2_splat(sqa[f]), pb = f2_splat(sqb[f]);
#pragma unroll
      for (int t = 0; t < R; ++t) v[t] = df_to_fx2(reinterpret_cast<const float4*>(y)[pos(t)], pa, pb);
    } else {
#pragma unroll
      for (int t = 0; t < R; ++t) v[t] = y[pos(t)];
    }
    if (INV && !PASS1) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = fx_cmul<INV>(v[t], fx_ldw(&tw[TWS * k * t]));
    }
    butterfly_fx<INV, R>(v, kc);
    if (!INV && !PASS1) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = fx_cmul<INV>(v[t], fx_ldw(&tw[TWS * k * t]));
    }
#pragma unroll
    for (int t = 0; t < R; ++t) y[pos(t)] = v[t];
  }
}

// Real-FFT pre-processing of the pair (q, n - q) of one field, in place on
// the spectrum map (as row_fx8_body: z_q = A + P, z_{n-q} = conj(A - P)).
template <class S>
__device__ __forceinline__ void pfa_pre_pair(cfx* z, int q, int L, f2 qa, f2 qb, const FxW* __restrict__ twfx,
                                             const unsigned short* spec) {
  const int qn = S::n - q;
  const int s0 = spec[q], s1 = spec[q == 0 ? 0 : qn];
  const FxW w = fx_ldw(&twfx[q]);
  cfx hq = cfx{0, 0}, hn = cfx{0, 0};
  if (q <= L) {
    hq = df_to_fx2(reinterpret_cast<const float4*>(z)[s0], qa, qb);
    if (q == 0) hq.im = 0;  // Im(F_0) is dropped
  }
  if (q > 0 && qn <= L) hn = df_to_fx2(reinterpret_cast<const float4*>(z)[s1], qa, qb);
  const cfx A = fx_add(hq, fx_conj(hn));
  const cfx B = fx_sub(hq, fx_conj(hn));
  const cfx P = fx_i<true>(fx_cmul<true>(B, w));
  z[s0] = fx_add(A, P);
  if (q > 0 && qn > q) z[s1] = fx_conj(fx_sub(A, P));
}

// Forward post-processing of order q from the spectrum map: the packed G
// word pair of R2 / 2 (as row_fx8_body).
template <class S>
__device__ __forceinline__ void pfa_post(const cfx* Z, int q, int e, const FxW* __restrict__ twfx, longlong2* out,
                                         const unsigned short* spec) {
  const FxW w = fx_ldw(&twfx[q]);
  const cfx zq = Z[spec[q]];
  const cfx zn = fx_conj(Z[spec[q == 0 ? 0 : S::n - q]]);
  const cfx E2 = fx_add(zq, zn);
  const cfx D = fx_sub(zq, zn);
  const cfx O2 = cfx{D.im, -D.re};
  const cfx R2 = fx_add(E2, fx_cmul<false>(O2, w));
  *out = make_longlong2(pk_pack(R2.re, e), pk_pack(R2.im, e));
}

// Member rows per CTA: functors with few fields take several members of
// the same latitude row per CTA, so every phase still has work for the 128
// threads (and the shared memory stays within the 1-row SWE footprint).
template <class Pw>
constexpr int pfa_rows_per_cta() {
  constexpr int NF = Pw::NIN > Pw::NOUT ? Pw::NIN : Pw::NOUT;
  return NF >= 5 ? 1 : NF >= 3 ? 2 : NF == 2 ? 4 : 8;
}

// Per-CTA scalars of a row body (NR member rows of NF fields).
template <int NR, int NF>
struct alignas(16) PfaCtaScratch {
  unsigned bits[NR];
  int in[NR * NF];
  unsigned key[NR * NF], omax[NR * NF];
  float pa[NR * NF], pb[NR * NF], qa[NR * NF], qb[NR * NF];
  RowDf rc;
  df wj;
};

template <class Pw, int IN_MODE, int OUT_MODE, class S>
__device__ __forceinline__ void row_pfa_body(const RowArgs& a, const Pw& pw, const FxW* __restrict__ twfx,
                                             const FxConst& kc, int bx, int by) {
  constexpr int NIN = Pw::NIN, NOUT = Pw::NOUT;
  constexpr int NF = NIN > NOUT ? NIN : NOUT;
  constexpr int NR = pfa_rows_per_cta<Pw>();
  constexpr int NRI = NR * NIN, NRO = NR * NOUT;  // (member row, field) pairs in and out
  constexpr int n = S::n, N = S::N, fs = S::fs, hb = S::hb, P = S::P, R0 = S::R0, T = kPfaThreads;
  constexpr int RS = NF * fs;  // slots of one member row
  constexpr int PSI = (T / NRI) * NRI, QSI = T / NRI;
  static_assert(NRI <= T && NRO <= T, "one thread per (row, field) for the block exponents");
  constexpr bool kPairs = PwHasPairs<Pw>::value;
  // pointwise: slot pairs in rounds of T, and for NR n = 3T/2 the last T/2
  // slots as one single point per thread
  constexpr bool kSplitTail = NR * n - T == T / 2;
  extern __shared__ cfx smem_fx[];
  // After the row buffers, in dynamic shared memory (the grouped row kernel
  // holds every body, and static arrays of all of them would sit in every
  // CTA): the per-CTA scalars and the spectrum and grid maps (S::spec,
  // S::grid), tabulated once per CTA.
  PfaCtaScratch<NR, NF>& sc = *reinterpret_cast<PfaCtaScratch<NR, NF>*>(smem_fx + NR * RS);
  unsigned* s_bits = sc.bits;
  int* s_in = sc.in;        // block exponents (inputs, then outputs)
  unsigned* s_key = sc.key;  // largest |hi| bit key of each input field
  unsigned* s_omax = sc.omax; // largest |hi| bit key of each output field
  float *s_pa = sc.pa, *s_pb = sc.pb, *s_qa = sc.qa, *s_qb = sc.qb;
  RowDf& s_rc = sc.rc;
  df& s_wj = sc.wj;
  unsigned short* s_spec = reinterpret_cast<unsigned short*>(&sc + 1);
  unsigned short* s_grid = s_spec + (S::n + 1);
  const int j = bx, b0 = NR * by, tid = threadIdx.x;
  const int nrow = min(NR, a.batch - b0);  // members of this CTA
  const int L = a.L, ldm = L + 1;
  cfx* buf0 = smem_fx;
  // (member row, field) -> its row buffer
  auto zrow = [&](int row, int f) { return buf0 + row * RS + f * fs; };
  const long sq = (long)a.nblk * a.nlat;
  const long bsi = (long)ldm * a.nlat * a.nblk;  // member stride of the F blocks
  const float4* block = nullptr;
  if (IN_MODE == kInF || OUT_MODE == kOutG)
    block = reinterpret_cast<const float4*>(a.FG) + fg_index(b0, 0, 0, j, L, a.nblk, a.nlat);
  const long sqo = a.G ? (long)a.gblk * a.nlat : sq;
  const long bso = a.G ? (long)ldm * a.nlat * a.gblk : bsi;
  longlong2* oblock = nullptr;
  if (OUT_MODE == kOutG)
    oblock = a.G ? reinterpret_cast<longlong2*>(a.G) + fg_index(b0, 0, 0, j, L, a.gblk, a.nlat)
                 : reinterpret_cast<longlong2*>(const_cast<float4*>(block));
  for (int q = tid; q <= n; q += T) {
    s_spec[q] = static_cast<unsigned short>(S::spec(q));
    if (q < n) s_grid[q] = static_cast<unsigned short>(S::grid(q));
  }
  if (tid < NR) s_bits[tid] = 0u;
  if (tid < NR * NF) {
    s_key[tid] = 0u;
    s_omax[tid] = 0u;
  }
  if (tid == 32) {  // row constants (FP64 work) while the loads fly
    s_rc = pw.df_row(a.coslat[j], a.fgrid ? a.fgrid[j] : 0.0);
    s_wj = (OUT_MODE == kOutG && a.wq) ? df_from_double(a.wq[j]) : df{1.f, 0.f};
  }
  __syncthreads();

  // ---- 1. grid rows of the inputs
  if constexpr (IN_MODE == kInF) {
    // stage F[q][f] at slot spec(q) of field f: thread (row, field) = tid mod
    // NRI, orders tid / NRI + QSI i (fields fastest across the threads:
    // coalesced), four loads in flight per thread; the field's largest |hi|
    // (m = 0: Im dropped) on the way
    if (tid < PSI) {
      const int rf = tid % NRI, row = NR == 1 ? 0 : rf / NIN, f = rf - row * NIN;
      float4* zf = reinterpret_cast<float4*>(zrow(row, f));
      const float4* src = block + row * bsi + f;
      unsigned mx = 0u;
      if (NR == 1 || row < nrow) {
#pragma unroll 1
        for (int q0 = tid / NRI; q0 < ldm; q0 += 4 * QSI) {
          float4 w[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int q = q0 + u * QSI;
            if (q < ldm) w[u] = src[(long)q * sq];  // plain loads: the same blocks may take G later (a.G null)
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int q = q0 + u * QSI;
            if (q < ldm) {
              mx = max(mx, max(__float_as_uint(w[u].x) & 0x7FFFFFFFu, q == 0 ? 0u : __float_as_uint(w[u].z) & 0x7FFFFFFFu));
              zf[s_spec[q]] = w[u];
            }
          }
        }
      }
      if (mx) atomicMax(&s_key[row * NF + f], mx);
    }
    __syncthreads();
    if (tid < NRI) {  // block exponent: |F| < 2^E -> |X| < 2^hb
      const int row = tid / NIN, f = tid - row * NIN, i = row * NF + f;
      const unsigned key = s_key[i];
      const int S0 = (key >> 23) == 0 ? 0 : fkey_exp(key) - hb;
      s_in[i] = S0;
      fx_pow2_split(S0, s_pa[i], s_pb[i]);
      fx_pow2_split(-S0, s_qa[i], s_qb[i]);
    }
    __syncthreads();
#pragma unroll 1
    for (int idx = tid; idx < NRI * (n / 2 + 1); idx += T) {
      const int q = idx / NRI, rf = idx - q * NRI, row = NR == 1 ? 0 : rf / NIN, f = rf - row * NIN;
      pfa_pre_pair<S>(zrow(row, f), q, row < nrow ? L : -1, f2_splat(s_qa[row * NF + f]), f2_splat(s_qb[row * NF + f]),
                      twfx, s_spec);
    }
    __syncthreads();
    if constexpr (R0 > 1) {
#pragma unroll 1
      for (int idx = tid; idx < NRI * P; idx += T) {  // radix-R0 across the blocks (no twiddles)
        const int rf = idx / P, row = NR == 1 ? 0 : rf / NIN, f = rf - row * NIN;
        cfx* z = zrow(row, f) + (idx & (P - 1));
        cfx v[R0];
#pragma unroll
        for (int r = 0; r < R0; ++r) v[r] = z[r * P];
        butterfly_fx<true, R0>(v, kc);
#pragma unroll
        for (int r = 0; r < R0; ++r) z[r * P] = v[r];
      }
      __syncthreads();
    }
    pfa_pass<S, true, true, false, NRI, NIN, RS>(buf0, twfx, kc, nullptr, nullptr);
    __syncthreads();
    pfa_pass<S, true, false, false, NRI, NIN, RS>(buf0, twfx, kc, nullptr, nullptr);
    __syncthreads();
  } else {
#pragma unroll 1
    for (int idx = tid; idx < NRI * N; idx += T) {
      const int rf = idx / N, k = idx - rf * N, row = rf / NIN, f = rf - row * NIN;
      if (row < nrow)
        reinterpret_cast<df*>(zrow(row, f))[2 * s_grid[k >> 1] + (k & 1)] =
            df_of_f64(a.gin[(long)(b0 + row) * a.gin_b + (long)f * a.gin_f + (long)j * N + k]);
    }
    __syncthreads();
  }

  // ---- 2. pointwise products, weighted by the row's quadrature weight; in
  // place (each point is read before it is written, by one thread).  A
  // warp's points in one round lie in one member row (n and N are
  // multiples of 32).
  {
    const RowDf rc = s_rc;
    const df wj = s_wj;
    const bool wq = OUT_MODE == kOutG && a.wq != nullptr;
    unsigned omax[NOUT];
#pragma unroll
    for (int f = 0; f < NOUT; ++f) omax[f] = 0u;
    unsigned bits = 0u;
    int orow = -1;  // member row of omax and bits (NR > 1: flushed when the row changes)
    auto flush = [&]() {
      if (orow < 0) return;
      if (a.status && bits && (NR == 1 || orow < nrow)) atomicOr(&s_bits[orow], bits);
      bits = 0u;
      if constexpr (OUT_MODE == kOutG) {
#pragma unroll
        for (int f = 0; f < NOUT; ++f) {
          unsigned v = omax[f];
          for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
          if ((tid & 31) == 0 && v && (NR == 1 || orow < nrow)) atomicMax(&s_omax[orow * NF + f], v);
          omax[f] = 0u;
        }
      }
    };
    auto at_row = [&](int row) {
      if (NR > 1 && row != orow) {
        flush();
        orow = row;
      }
      if (NR == 1) orow = 0;
    };
    // input scales of a one-row CTA in registers
    float pa1[NIN], pb1[NIN];
    if constexpr (NR == 1 && IN_MODE == kInF) {
#pragma unroll
      for (int f = 0; f < NIN; ++f) {
        pa1[f] = s_pa[f];
        pb1[f] = s_pb[f];
      }
    }
    auto spa = [&](int row, int f) { return NR == 1 ? pa1[f] : s_pa[row * NF + f]; };
    auto spb = [&](int row, int f) { return NR == 1 ? pb1[f] : s_pb[row * NF + f]; };
    auto single = [&](int k) {  // real grid point k of the CTA's rows
      const int row = NR == 1 ? 0 : k / N, kk = k - row * N;
      at_row(row);
      const int slot = 2 * s_grid[kk >> 1] + (kk & 1);
      cfx* zb = zrow(row, 0);
      const long long* xi = reinterpret_cast<const long long*>(zb);
      const df* xd = reinterpret_cast<const df*>(zb);
      df* xo = reinterpret_cast<df*>(zb);
      df in[NIN], out[NOUT];
#pragma unroll
      for (int f = 0; f < NIN; ++f)
        in[f] = IN_MODE == kInF ? fx_to_df(xi[2 * f * fs + slot], spa(row, f), spb(row, f)) : xd[2 * f * fs + slot];
      bits |= pw.df_op(rc, in, out);
#pragma unroll
      for (int f = 0; f < NOUT; ++f) {
        if (wq) out[f] = df_mul(out[f], wj);
        xo[2 * f * fs + slot] = out[f];
        omax[f] = max(omax[f], __float_as_uint(out[f].hi) & 0x7FFFFFFFu);
      }
    };
    if constexpr (kPairs) {
#pragma unroll 1
      for (int i = tid; i < (kSplitTail ? T : NR * n); i += T) {
        const int row = NR == 1 ? 0 : i / n, ii = i - row * n;
        at_row(row);
        const int s = s_grid[ii];
        cfx* zb = zrow(row, 0);
        df2 in[NIN], out[NOUT];
#pragma unroll
        for (int f = 0; f < NIN; ++f) {
          if constexpr (IN_MODE == kInF) {
            const cfx X = zb[f * fs + s];
            in[f] = fx_to_df2(X.re, X.im, f2_splat(spa(row, f)), f2_splat(spb(row, f)));
          } else {
            const float4 w = reinterpret_cast<const float4*>(zb)[f * fs + s];
            in[f] = df2{f2_pack(w.x, w.z), f2_pack(w.y, w.w)};
          }
        }
        bits |= pw.df_op2(rc, in, out);
        const df2 wj2 = df2_pack(wj, wj);
#pragma unroll
        for (int f = 0; f < NOUT; ++f) {
          if (wq) out[f] = df2_mul(out[f], wj2);
          df x0, x1;
          df2_unpack(out[f], x0, x1);
          reinterpret_cast<float4*>(zb)[f * fs + s] = make_float4(x0.hi, x0.lo, x1.hi, x1.lo);
          omax[f] = max(omax[f], max(__float_as_uint(x0.hi) & 0x7FFFFFFFu, __float_as_uint(x1.hi) & 0x7FFFFFFFu));
        }
      }
      if constexpr (kSplitTail) single(2 * T + tid);
    } else {
#pragma unroll 1
      for (int k = tid; k < NR * N; k += T) single(k);
    }
    flush();
  }
  __syncthreads();
  if (a.status && tid < nrow && s_bits[tid]) atomicOr(&a.status[b0 + tid], s_bits[tid]);

  // ---- 3. outputs
  if constexpr (OUT_MODE == kOutGrid) {
#pragma unroll 1
    for (int idx = tid; idx < NRO * N; idx += T) {
      const int rf = idx / N, k = idx - rf * N, row = rf / NOUT, f = rf - row * NOUT;
      if (row < nrow)
        a.gout[(long)(b0 + row) * a.gout_b + (long)f * a.gout_f + (long)j * N + k] =
            f64_of_df(reinterpret_cast<const df*>(zrow(row, f))[2 * s_grid[k >> 1] + (k & 1)]);
    }
  } else {
    if (tid < NRO) {  // output block exponents (|X| < 2^hb)
      const int row = tid / NOUT, f = tid - row * NOUT, i = row * NF + f;
      const unsigned key = s_omax[i];
      const int S0 = (key >> 23) == 0 ? 0 : fkey_exp(key) - hb;
      s_in[i] = S0;
      fx_pow2_split(-S0, s_pa[tid], s_pb[tid]);  // indexed by (row, output field) for the passes
    }
    __syncthreads();
    pfa_pass<S, false, false, true, NRO, NOUT, RS>(buf0, twfx, kc, s_pa, s_pb);
    __syncthreads();
    pfa_pass<S, false, true, false, NRO, NOUT, RS>(buf0, twfx, kc, nullptr, nullptr);
    __syncthreads();
    // radix-R0 across the blocks for the order groups c + jP and P - c + jP
    // (item 0: the self-paired groups 0 and P/2), then the real-FFT
    // post-processing of their 2 R0 orders (partners n - q in the same item)
#pragma unroll 1
    for (int idx = tid; idx < NRO * (P / 2); idx += T) {
      const int c = idx / NRO, rf = idx - c * NRO, row = NR == 1 ? 0 : rf / NOUT, f = rf - row * NOUT;
      const int e = s_in[row * NF + f] - 1;  // R2 / 2 in units of 2^S
      cfx* Z = zrow(row, f);
      const int g1 = c == 0 ? P / 2 : P - c;
      if constexpr (R0 > 1) {
#pragma unroll 1
        for (int g = 0; g < 2; ++g) {
          cfx* z = Z + S::upos(g == 0 ? c : g1);
          cfx v[R0];
#pragma unroll
          for (int r = 0; r < R0; ++r) v[r] = z[r * P];
          butterfly_fx<false, R0>(v, kc);
#pragma unroll
          for (int r = 0; r < R0; ++r) z[r * P] = v[r];
        }
      }
      if (row < nrow) {
        longlong2* ob = oblock + row * bso + f;
#pragma unroll 1
        for (int p = 0; p < 2 * R0; ++p) {
          const int q = (p < R0 ? c : g1) + (p < R0 ? p : p - R0) * P;
          if (q <= L) pfa_post<S>(Z, q, e, twfx, ob + (long)q * sqo, s_spec);
        }
      }
    }
  }
}

template <class Pw, int IN_MODE, int OUT_MODE, class S>
__global__ void __launch_bounds__(kPfaThreads, 6) row_kernel_pfa(RowArgs a, Pw pw, const FxW* __restrict__ twfx,
                                                                 FxConst kc) {
  pdl_trigger();
  pdl_wait();
  row_pfa_body<Pw, IN_MODE, OUT_MODE, S>(a, pw, twfx, kc, blockIdx.x, blockIdx.y);
}

template <class Pw, class S>
constexpr size_t row_pfa_smem_bytes() {
  constexpr int NF = Pw::NIN > Pw::NOUT ? Pw::NIN : Pw::NOUT;
  constexpr int NR = pfa_rows_per_cta<Pw>();
  return (size_t)NR * NF * S::fs * sizeof(cfx) +                           // row buffers
         sizeof(PfaCtaScratch<NR, NF>) +                                   // per-CTA scalars
         ((size_t)(2 * S::n + 1) * sizeof(unsigned short) + 15) / 16 * 16;  // index tables
}
// Grid of a prime-factor row launch: (latitude rows, member groups).
template <class Pw>
inline dim3 row_pfa_grid(int nlat, int batch) {
  constexpr int NR = pfa_rows_per_cta<Pw>();
  return dim3(nlat, (batch + NR - 1) / NR);
}

}  // namespace aeolus
