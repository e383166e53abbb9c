// Longitude stage of the split-precision path: 64-bit fixed-point FFTs
// around double-float pointwise products.
//
// Per (latitude row j, member b), as in row_kernel (rows.cuh):
//   1. the order spectra F_m of every input field arrive as double-floats
//      written by the tensor-core synthesis; each field's row is rounded to
//      integers X at one block exponent S_f chosen from its largest element
//      so that |X| < 2^hb, hb = min(52, 56 - ceil(log2 n));
//   2. the half-length complex inverse FFT (in place, decimation in time,
//      radix 3/5, then 2/4, then 8) runs in
//      exact 64-bit additions and 31-bit-limb twiddle products -- the bound
//      on hb keeps every butterfly below 2^59, and the error is ~2^-(hb+1) of
//      the row's largest input (~2^-49 at n = 192);
//   3. grid values become double-floats for the pointwise products
//      (Pw::df_op), weighted by the quadrature weight of the row;
//   4. each output field is aligned to its own block exponent, forward
//      FFT'd in fixed point (in place, decimation in frequency), and the
//      order spectra G_m are written back as packed words for the analysis
//      slicer.
// The in-place transforms need one row buffer per block (Stockham needs
// two), so twice as many blocks fit an SM; the real-FFT pre- and post-
// processing read and write the digit-reversed positions directly.
// Lengths without a 2/3/5 FFT fall back to a direct double-float DFT.
#pragma once

#include "df.cuh"
#include "fx.cuh"
#include "rows.cuh"

namespace aeolus {

// X 2^S as a double-float for |X| < 2^59 (pa pb = 2^S), on the FMA/ALU
// pipes: X = c2 2^40 + c1 2^20 + c0 with 20-bit limbs, each limb made exact
// by the magic-number construction (the limb placed in the mantissa of a
// float of known exponent, that float's offset subtracted), then summed
// with error-free transformations.
__device__ __forceinline__ df fx_to_df(long long X, float pa, float pb) {
  const unsigned lo = static_cast<unsigned>(X), hi = static_cast<unsigned>(X >> 32);
  const unsigned c0 = lo & 0xFFFFFu;
  const unsigned c1 = __funnelshift_r(lo, hi, 20) & 0xFFFFFu;
  const int c2 = static_cast<int>(X >> 40);
  const float f0 = __int_as_float(0x4B000000 | c0) - 8388608.0f;                    // c0
  const float f1 = __int_as_float((170u << 23) | c1) - 8796093022208.0f;            // c1 2^20
  const float f2 = __int_as_float((190 << 23) + 0x400000 + c2) - 13835058055282163712.0f;  // c2 2^40
  const float s = f2 + f1;
  const float e1 = f1 - (s - f2);  // exact: |f2| >= |f1| or f2 = 0
  const float t = e1 + f0;
  const float h = s + t;
  const float l = t - (h - s);
  return df{h * pa * pb, l * pa * pb};
}

// rint(v 2^-S) for pa pb = 2^-S and |v 2^-S| < 2^52: the high word splits
// into u 2^30 + r (u by the magic-number rounding, r exact by FMA), r and
// the low word are rounded by 32-bit conversions.
__device__ __forceinline__ long long df_to_fx(df v, float pa, float pb) {
  const float th = v.hi * pa * pb, tl = v.lo * pa * pb;
  const float um = fmaf(th, 9.31322574615478515625e-10f, 12582912.0f);  // th 2^-30 + 1.5 2^23
  const int u = __float_as_int(um) - 0x4B400000;
  const float r = fmaf(-(um - 12582912.0f), 1073741824.0f, th);
  const int rl = __float2int_rn(r) + __float2int_rn(tl);
  return fx_madw(u, 1 << 30, static_cast<long long>(rl));
}
// Exponent E with |x| < 2^E for every float whose |bits| <= key.
__device__ __forceinline__ int fkey_exp(unsigned key) { return static_cast<int>(key >> 23) - 126; }
// A double-float as a packed word (52-bit mantissa).
__device__ __forceinline__ long long df_to_pk(df v) {
  const unsigned key = __float_as_uint(v.hi) & 0x7FFFFFFFu;
  if ((key >> 23) == 0) return 0;
  const int S = fkey_exp(key) - kPackMant;
  float pa, pb;
  fx_pow2_split(-S, pa, pb);
  return pk_pack(df_to_fx(v, pa, pb), S);
}

template <bool INV, int R>
__device__ __forceinline__ void butterfly_fx(cfx* v, const FxConst& k) {
  if constexpr (R == 2) {
    const cfx a = v[0], b = v[1];
    v[0] = fx_add(a, b);
    v[1] = fx_sub(a, b);
  } else if constexpr (R == 4) {
    const cfx s02 = fx_add(v[0], v[2]), d02 = fx_sub(v[0], v[2]);
    const cfx s13 = fx_add(v[1], v[3]), d13 = fx_sub(v[1], v[3]);
    const cfx id13 = fx_i<INV>(d13);
    v[0] = fx_add(s02, s13);
    v[2] = fx_sub(s02, s13);
    v[1] = fx_add(d02, id13);
    v[3] = fx_sub(d02, id13);
  } else if constexpr (R == 3) {
    const cfx s = fx_add(v[1], v[2]), d = fx_sub(v[1], v[2]);
    const cfx t = cfx{v[0].re - (s.re >> 1), v[0].im - (s.im >> 1)};
    const cfx id = fx_i<INV>(cfx{fx_mulk(d.re, k.h3), fx_mulk(d.im, k.h3)});
    v[0] = fx_add(v[0], s);
    v[1] = fx_add(t, id);
    v[2] = fx_sub(t, id);
  } else if constexpr (R == 8) {
    // radix-4 transforms of the even and odd inputs, combined with w8^t
    cfx e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    butterfly_fx<INV, 4>(e, k);
    butterfly_fx<INV, 4>(o, k);
    {  // o1 *= (1 +- i)/sqrt2, o3 *= (-1 +- i)/sqrt2 (+: inverse), o2 *= +-i
      const long long s1 = o[1].re + o[1].im, d1 = o[1].re - o[1].im;
      const long long s3 = o[3].re + o[3].im, d3 = o[3].re - o[3].im;
      if (INV) {
        o[1] = cfx{fx_mulk(d1, k.r2), fx_mulk(s1, k.r2)};
        o[3] = cfx{-fx_mulk(s3, k.r2), fx_mulk(d3, k.r2)};
      } else {
        o[1] = cfx{fx_mulk(s1, k.r2), -fx_mulk(d1, k.r2)};
        o[3] = cfx{-fx_mulk(d3, k.r2), -fx_mulk(s3, k.r2)};
      }
      o[2] = fx_i<INV>(o[2]);
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      v[t] = fx_add(e[t], o[t]);
      v[t + 4] = fx_sub(e[t], o[t]);
    }
  } else {  // R == 5
    const cfx a1 = fx_add(v[1], v[4]), a2 = fx_add(v[2], v[3]);
    const cfx b1 = fx_sub(v[1], v[4]), b2 = fx_sub(v[2], v[3]);
    const cfx t1 = cfx{v[0].re + fx_mulk(a1.re, k.c1) + fx_mulk(a2.re, k.c2),
                       v[0].im + fx_mulk(a1.im, k.c1) + fx_mulk(a2.im, k.c2)};
    const cfx t2 = cfx{v[0].re + fx_mulk(a1.re, k.c2) + fx_mulk(a2.re, k.c1),
                       v[0].im + fx_mulk(a1.im, k.c2) + fx_mulk(a2.im, k.c1)};
    const cfx u1 = cfx{fx_mulk(b1.re, k.s1) + fx_mulk(b2.re, k.s2), fx_mulk(b1.im, k.s1) + fx_mulk(b2.im, k.s2)};
    const cfx u2 = cfx{fx_mulk(b1.re, k.s2) - fx_mulk(b2.re, k.s1), fx_mulk(b1.im, k.s2) - fx_mulk(b2.im, k.s1)};
    const cfx iu1 = fx_i<INV>(u1), iu2 = fx_i<INV>(u2);
    v[0] = fx_add(v[0], fx_add(a1, a2));
    v[1] = fx_add(t1, iu1);
    v[4] = fx_sub(t1, iu1);
    v[2] = fx_add(t2, iu2);
    v[3] = fx_sub(t2, iu2);
  }
}

// One in-place stage over sub-transforms of length Ls -> Ls R: the
// butterfly of (group g, offset k) owns elements g Ls R + k + t Ls, t < R.
// DIT (inverse transforms, input in digit-reversed order): twiddles
// w_{Ls R}^{k t} before the butterfly; DIF (forward, output digit-
// reversed): after it.  TW = false for the stage with Ls = 1 (no twiddles).
// CONV: the rows still hold double-float reals (two per complex slot); they
// are rounded to the fixed-point block exponent of their field (scale
// factors pa pb = 2^-S) as they are loaded.
template <bool INV, int R, bool DIT, bool TW, bool CONV>
__device__ __forceinline__ void fft_stage_ip(cfx* __restrict__ x, int nf, int n, int fs, int Ls, unsigned nb_rcp,
                                             unsigned ls_rcp, const FxW* __restrict__ tw, const FxConst& kc,
                                             const float* sqa, const float* sqb) {
  const int nb = n / R, Ns = Ls * R, stride = n / Ns;
  for (int idx = threadIdx.x; idx < nf * nb; idx += blockDim.x) {
    const int f = div_rcp(idx, nb, nb_rcp), jj = idx - f * nb;
    const int g = div_rcp(jj, Ls, ls_rcp), k = jj - g * Ls;
    cfx* y = x + (long)f * fs + g * Ns + k;
    cfx v[R];
    if (CONV) {
      const float pa = sqa[f], pb = sqb[f];
#pragma unroll
      for (int t = 0; t < R; ++t) {
        const float4 w = reinterpret_cast<const float4*>(y)[t * Ls];
        v[t] = cfx{df_to_fx(df{w.x, w.y}, pa, pb), df_to_fx(df{w.z, w.w}, pa, pb)};
      }
    } else {
#pragma unroll
      for (int t = 0; t < R; ++t) v[t] = y[t * Ls];
    }
    if (DIT && TW) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = fx_cmul<INV>(v[t], fx_ldw(&tw[2 * (k * t * stride)]));
    }
    butterfly_fx<INV, R>(v, kc);
    if (!DIT && TW) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = fx_cmul<INV>(v[t], fx_ldw(&tw[2 * (k * t * stride)]));
    }
#pragma unroll
    for (int t = 0; t < R; ++t) y[t * Ls] = v[t];
  }
}

template <bool INV, bool DIT, bool TW, bool CONV>
__device__ __forceinline__ void fft_stage_ip_r(int r, cfx* x, int nf, int n, int fs, int Ls, unsigned nbm,
                                               unsigned lsm, const FxW* __restrict__ tw, const FxConst& kc,
                                               const float* sqa, const float* sqb) {
  switch (r) {
    case 8: fft_stage_ip<INV, 8, DIT, TW, CONV>(x, nf, n, fs, Ls, nbm, lsm, tw, kc, sqa, sqb); break;
    case 4: fft_stage_ip<INV, 4, DIT, TW, CONV>(x, nf, n, fs, Ls, nbm, lsm, tw, kc, sqa, sqb); break;
    case 2: fft_stage_ip<INV, 2, DIT, TW, CONV>(x, nf, n, fs, Ls, nbm, lsm, tw, kc, sqa, sqb); break;
    case 3: fft_stage_ip<INV, 3, DIT, TW, CONV>(x, nf, n, fs, Ls, nbm, lsm, tw, kc, sqa, sqb); break;
    default: fft_stage_ip<INV, 5, DIT, TW, CONV>(x, nf, n, fs, Ls, nbm, lsm, tw, kc, sqa, sqb); break;
  }
}

// In-place transform of nf rows (field stride fs) of length fi.n: inverse
// by decimation in time (digit-reversed input, natural output), forward by
// decimation in frequency (natural input, digit-reversed output; with sqa,
// the input rows are double-floats converted by the first stage).
template <bool INV>
__device__ void fft_ip(cfx* x, int nf, int fs, const FftInfo& fi, const FxW* __restrict__ tw, const FxConst& kc,
                       const float* sqa = nullptr, const float* sqb = nullptr) {
  const int n = fi.n;
  if (INV) {
    int Ls = 1;
    for (int s = 0; s < fi.nfac; ++s) {
      if (s == 0)
        fft_stage_ip_r<INV, true, false, false>(fi.fac[s], x, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw, kc, sqa, sqb);
      else
        fft_stage_ip_r<INV, true, true, false>(fi.fac[s], x, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw, kc, sqa, sqb);
      __syncthreads();
      Ls *= fi.fac[s];
    }
  } else {
    int Ls = n;
    for (int s = fi.nfac - 1; s >= 0; --s) {
      Ls /= fi.fac[s];
      const bool conv = sqa && s == fi.nfac - 1;
      if (s == 0) {
        if (conv)
          fft_stage_ip_r<INV, false, false, true>(fi.fac[s], x, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw, kc, sqa, sqb);
        else
          fft_stage_ip_r<INV, false, false, false>(fi.fac[s], x, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw, kc, sqa, sqb);
      } else {
        if (conv)
          fft_stage_ip_r<INV, false, true, true>(fi.fac[s], x, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw, kc, sqa, sqb);
        else
          fft_stage_ip_r<INV, false, true, false>(fi.fac[s], x, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw, kc, sqa, sqb);
      }
      __syncthreads();
    }
  }
}

// FFT policies of the row body.  FftRuntime dispatches every stage on the
// plan's radix at run time (all radix bodies are compiled in); FftFixed
// compiles exactly the plan's radix sequence, which keeps the kernel small
// enough for the instruction caches.  The host picks FftFixed when the
// plan's factors match.
struct FftRuntime {
  static constexpr bool kFixed = false;  // the plan may fall back to the direct DFT
  template <bool INV>
  static __device__ __forceinline__ void run(cfx* x, int nf, int fs, const FftInfo& fi, const FxW* __restrict__ tw,
                                             const FxConst& kc, const float* sqa = nullptr,
                                             const float* sqb = nullptr) {
    fft_ip<INV>(x, nf, fs, fi, tw, kc, sqa, sqb);
  }
};

template <int... Rs>
struct FftFixed {
  static constexpr bool kFixed = true;  // always an FFT plan: the DFT branches are not compiled
  static constexpr int S = sizeof...(Rs);
  static __host__ __device__ constexpr int radix(int s) {
    constexpr int f[S] = {Rs...};
    return f[s];
  }
  static bool matches(const FftInfo& fi) {
    if (!fi.use_fft || fi.nfac != S) return false;
    for (int s = 0; s < S; ++s)
      if (fi.fac[s] != radix(s)) return false;
    return true;
  }
  template <bool INV, int s>
  static __device__ __forceinline__ void dit(cfx* x, int nf, int n, int fs, int Ls, const FftInfo& fi,
                                             const FxW* __restrict__ tw, const FxConst& kc) {
    if constexpr (s < S) {
      constexpr int R = radix(s);
      fft_stage_ip<INV, R, true, (s > 0), false>(x, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw, kc, nullptr, nullptr);
      __syncthreads();
      dit<INV, s + 1>(x, nf, n, fs, Ls * R, fi, tw, kc);
    }
  }
  template <bool INV, int s, bool CONV>
  static __device__ __forceinline__ void dif(cfx* x, int nf, int n, int fs, int Ls, const FftInfo& fi,
                                             const FxW* __restrict__ tw, const FxConst& kc, const float* sqa,
                                             const float* sqb) {
    if constexpr (s >= 0) {
      constexpr int R = radix(s);
      const int ls = Ls / R;
      fft_stage_ip<INV, R, false, (s > 0), CONV>(x, nf, n, fs, ls, fi.nbm[s], fi.lsm[s], tw, kc, sqa, sqb);
      __syncthreads();
      dif<INV, s - 1, false>(x, nf, n, fs, ls, fi, tw, kc, sqa, sqb);
    }
  }
  template <bool INV>
  static __device__ __forceinline__ void run(cfx* x, int nf, int fs, const FftInfo& fi, const FxW* __restrict__ tw,
                                             const FxConst& kc, const float* sqa = nullptr,
                                             const float* sqb = nullptr) {
    if constexpr (INV) {
      dit<INV, 0>(x, nf, fi.n, fs, 1, fi, tw, kc);
    } else {
      if (sqa)
        dif<INV, S - 1, true>(x, nf, fi.n, fs, fi.n, fi, tw, kc, sqa, sqb);
      else
        dif<INV, S - 1, false>(x, nf, fi.n, fs, fi.n, fi, tw, kc, sqa, sqb);
    }
  }
};

template <class Pw, int IN_MODE, int OUT_MODE, class FFT = FftRuntime>
__device__ __forceinline__ void row_fx_body(const RowArgs& a, const Pw& pw, const FxW* __restrict__ twfx,
                                            const float4* __restrict__ twdf, const FxConst& kc, int bx, int by) {
  constexpr int NIN = Pw::NIN, NOUT = Pw::NOUT;
  constexpr int NF = NIN > NOUT ? NIN : NOUT;
  extern __shared__ cfx smem_fx[];
  __shared__ unsigned s_bits;
  __shared__ int s_in[NF];        // block exponents (inputs, then outputs)
  __shared__ unsigned s_key[NF];   // largest |hi| bit key of each input field
  __shared__ unsigned s_omax[NF];  // largest |hi| bit key of each output field
  __shared__ float s_pa[NF], s_pb[NF], s_qa[NF], s_qb[NF];  // 2^S, 2^-S in two factors
  __shared__ RowDf s_rc;
  __shared__ df s_wj;
  const int j = bx, b = by;
  const int N = a.fft.N, n = a.fft.n, L = a.L;
  const int ldm = L + 1;
  const int ns = n + 1;  // padded field stride of the smem rows (see row_body)
  const bool use_fft = FFT::kFixed || a.fft.use_fft != 0;
  const int hb = min(52, 56 - (32 - __clz(max(n - 1, 1))));  // |fixed-point FFT input| < 2^hb
  cfx* buf0 = smem_fx;                 // the rows (all in-place FFT work)
  cfx* buf1 = smem_fx + (long)NF * ns;  // staged spectra of the direct DFT (allocated only then)
  if (threadIdx.x == 0) s_bits = 0u;
  if (threadIdx.x < NF) {
    s_key[threadIdx.x] = 0u;
    s_omax[threadIdx.x] = 0u;
  }
  if (threadIdx.x == 0) {  // row constants, once per block (FP64 work)
    s_rc = pw.df_row(a.coslat[j], a.fgrid ? a.fgrid[j] : 0.0);
    s_wj = (OUT_MODE == kOutG && a.wq) ? df_from_double(a.wq[j]) : df{1.f, 0.f};
  }
  // this row's order spectra: field f, order q at block[q sq + f]; spectra
  // in: double-floats (float4), spectra out: packed words (two per float4 slot)
  const long sq = (long)a.nblk * a.nlat;
  float4* block = nullptr;
  if (IN_MODE == kInF || OUT_MODE == kOutG)
    block = reinterpret_cast<float4*>(a.FG) + fg_index(b, 0, 0, j, L, a.nblk, a.nlat);
  const long sqo = a.G ? (long)a.gblk * a.nlat : sq;  // output blocks
  float4* oblock = nullptr;
  if (OUT_MODE == kOutG)
    oblock = a.G ? reinterpret_cast<float4*>(a.G) + fg_index(b, 0, 0, j, L, a.gblk, a.nlat) : block;
  __syncthreads();

  // ---- 1. grid rows of the inputs, in buf0
  // in_fx: fixed-point rows X (field stride 2 ns, value X 2^s_in[f]);
  // otherwise double-float rows.
  const bool in_fx = IN_MODE == kInF && use_fft;
  const void* xin = buf0;
  if (IN_MODE == kInF) {
    // largest |hi| of each field's spectra (fields fastest: contiguous reads)
    for (int idx = threadIdx.x; idx < NIN * ldm; idx += blockDim.x) {
      const int q = idx / NIN, f = idx - q * NIN;
      const float4 w = block[(long)q * sq + f];
      const unsigned key = max(__float_as_uint(w.x) & 0x7FFFFFFFu,
                               q == 0 ? 0u : __float_as_uint(w.z) & 0x7FFFFFFFu);  // m = 0: Im dropped
      if (key) atomicMax(&s_key[f], key);
    }
    __syncthreads();
    if (threadIdx.x < NIN) {  // block exponent: |F| < 2^E -> |X| < 2^hb
      const unsigned key = s_key[threadIdx.x];
      const int S = (key >> 23) == 0 ? 0 : fkey_exp(key) - hb;
      s_in[threadIdx.x] = S;
      fx_pow2_split(S, s_pa[threadIdx.x], s_pb[threadIdx.x]);
      fx_pow2_split(-S, s_qa[threadIdx.x], s_qb[threadIdx.x]);
    }
    __syncthreads();
    if (use_fft) {
      // half-length complex input of the real inverse FFT, by pairs (q, n-q):
      //   A = h_q + conj(h_{n-q}), B = h_q - conj(h_{n-q}), P = i conj(e_q) B,
      //   z_q = A + P, z_{n-q} = conj(A - P)   (e_{n-q} = -conj(e_q))
      const int half = n / 2;
      for (int idx = threadIdx.x; idx < NIN * (half + 1); idx += blockDim.x) {
        const int q = idx / NIN, f = idx - q * NIN;
        const float qa = s_qa[f], qb = s_qb[f];
        const int qn = n - q;
        cfx hq = cfx{0, 0}, hn = cfx{0, 0};
        if (q <= L) {
          const float4 w = block[(long)q * sq + f];
          hq = cfx{df_to_fx(df{w.x, w.y}, qa, qb), q == 0 ? 0LL : df_to_fx(df{w.z, w.w}, qa, qb)};
        }
        if (q > 0 && qn <= L) {
          const float4 w = block[(long)qn * sq + f];
          hn = cfx{df_to_fx(df{w.x, w.y}, qa, qb), df_to_fx(df{w.z, w.w}, qa, qb)};
        }
        const cfx A = fx_add(hq, fx_conj(hn));
        const cfx B = fx_sub(hq, fx_conj(hn));
        const cfx P = fx_i<true>(fx_cmul<true>(B, fx_ldw(&twfx[q])));
        cfx* z = buf0 + (long)f * ns;  // digit-reversed positions for the in-place inverse FFT
        z[__ldg(&a.irev[q])] = fx_add(A, P);
        if (q > 0 && qn > q) z[__ldg(&a.irev[qn])] = fx_conj(fx_sub(A, P));
      }
      __syncthreads();
      FFT::template run<true>(buf0, NIN, ns, a.fft, twfx, kc);
    } else {
      // direct DFT in double-float: stage the spectra in buf1
      cdf* Fs = reinterpret_cast<cdf*>(buf1);
      for (int idx = threadIdx.x; idx < NIN * ldm; idx += blockDim.x) {
        const int q = idx / NIN, f = idx - q * NIN;
        float4 w = block[(long)q * sq + f];
        if (q == 0) w.z = w.w = 0.f;
        Fs[(long)f * ns + q] = cdf_from_f4(w);
      }
      __syncthreads();
      df* x0 = reinterpret_cast<df*>(buf0);
      for (int idx = threadIdx.x; idx < NIN * N; idx += blockDim.x) {
        const int f = idx / N, k = idx - f * N;
        const cdf* Ff = Fs + (long)f * ns;
        df acc = df{0.f, 0.f};
        int e = 0;
        for (int m = 1; m <= L; ++m) {
          e += k;
          if (e >= N) e -= N;
          const cdf w = cdf_from_f4(__ldg(&twdf[e]));
          const cdf F = Ff[m];
          acc = df_add_fast(acc, df_add_fast(df_mul(F.re, w.re), df_mul(F.im, w.im)));
        }
        x0[(long)f * 2 * ns + k] = df_add_fast(Ff[0].re, df_scale2(acc, 2.0f));
      }
      __syncthreads();
    }
  } else {
    df* x0 = reinterpret_cast<df*>(buf0);
    for (int idx = threadIdx.x; idx < NIN * N; idx += blockDim.x) {
      const int f = idx / N, k = idx - f * N;
      x0[(long)f * 2 * ns + k] = df_of_f64(a.gin[(long)b * a.gin_b + (long)f * a.gin_f + (long)j * N + k]);
    }
    __syncthreads();
  }

  // ---- 2. pointwise products (double-float), weighted by the row's quadrature
  // weight; in place: the thread of grid point k reads every input at k before
  // it writes the outputs there
  cfx* zout = buf0;
  df* xout = reinterpret_cast<df*>(zout);
  {
    const RowDf rc = s_rc;
    const df wj = s_wj;
    const long long* xi = static_cast<const long long*>(xin);
    const df* xd = static_cast<const df*>(xin);
    unsigned bits = 0u;
    unsigned omax[NOUT];
#pragma unroll
    for (int f = 0; f < NOUT; ++f) omax[f] = 0u;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
      df in[NIN], out[NOUT];
#pragma unroll
      for (int f = 0; f < NIN; ++f)
        in[f] = in_fx ? fx_to_df(xi[(long)f * 2 * ns + k], s_pa[f], s_pb[f]) : xd[(long)f * 2 * ns + k];
      bits |= pw.df_op(rc, in, out);
#pragma unroll
      for (int f = 0; f < NOUT; ++f) {
        if (OUT_MODE == kOutG && a.wq) out[f] = df_mul(out[f], wj);
        xout[(long)f * 2 * ns + k] = out[f];
        omax[f] = max(omax[f], __float_as_uint(out[f].hi) & 0x7FFFFFFFu);
      }
    }
    if (a.status && bits) atomicOr(&s_bits, bits);
    if (OUT_MODE == kOutG && use_fft) {
#pragma unroll
      for (int f = 0; f < NOUT; ++f) {
        unsigned v = omax[f];
        for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
        if ((threadIdx.x & 31) == 0 && v) atomicMax(&s_omax[f], v);
      }
    }
  }
  __syncthreads();
  if (a.status && threadIdx.x == 0 && s_bits) atomicOr(&a.status[b], s_bits);

  // ---- 3. outputs
  if (OUT_MODE == kOutGrid) {
    for (int idx = threadIdx.x; idx < NOUT * N; idx += blockDim.x) {
      const int f = idx / N, k = idx - f * N;
      a.gout[(long)b * a.gout_b + (long)f * a.gout_f + (long)j * N + k] = f64_of_df(xout[(long)f * 2 * ns + k]);
    }
  } else if (use_fft) {
    // output block exponents (|X| < 2^hb)
    if (threadIdx.x < NOUT) {
      const unsigned key = s_omax[threadIdx.x];
      const int S = (key >> 23) == 0 ? 0 : fkey_exp(key) - hb;
      s_in[threadIdx.x] = S;
      fx_pow2_split(-S, s_pa[threadIdx.x], s_pb[threadIdx.x]);
    }
    __syncthreads();
    // rows to fixed point inside the first stage; output in digit-reversed order
    FFT::template run<false>(zout, NOUT, ns, a.fft, twfx, kc, s_pa, s_pb);
    for (int idx = threadIdx.x; idx < NOUT * ldm; idx += blockDim.x) {
      const int q = idx / NOUT, f = idx - q * NOUT;  // fields fastest: contiguous global writes
      const cfx* Zf = zout + (long)f * ns;
      const cfx zq = Zf[__ldg(&a.irev[q])];
      const cfx zn = fx_conj(Zf[__ldg(&a.irev[q == 0 ? 0 : n - q])]);
      const cfx E2 = fx_add(zq, zn);             // 2 E
      const cfx D = fx_sub(zq, zn);
      const cfx O2 = cfx{D.im, -D.re};           // 2 O = -i D
      const cfx R2 = fx_add(E2, fx_cmul<false>(O2, fx_ldw(&twfx[q])));
      const int e = s_in[f] - 1;                 // R2 / 2 in units of 2^S
      reinterpret_cast<longlong2*>(oblock)[(long)q * sqo + f] = make_longlong2(pk_pack(R2.re, e), pk_pack(R2.im, e));
    }
  } else {
    for (int idx = threadIdx.x; idx < NOUT * ldm; idx += blockDim.x) {
      const int q = idx / NOUT, f = idx - q * NOUT;
      const df* x = xout + (long)f * 2 * ns;
      df sr = df{0.f, 0.f}, si = df{0.f, 0.f};
      int e = 0;
      for (int k = 0; k < N; ++k) {
        const cdf w = cdf_from_f4(__ldg(&twdf[e]));
        sr = df_add_fast(sr, df_mul(x[k], w.re));
        si = df_add_fast(si, df_mul(x[k], w.im));
        e += q;
        while (e >= N) e -= N;
      }
      reinterpret_cast<longlong2*>(oblock)[(long)q * sqo + f] = make_longlong2(df_to_pk(sr), df_to_pk(si));
    }
  }
}

// ------------------------------------------------------------------------
// Row stage for the radix sequences (R0, 8, 8), n = 64 R0 (nlon 384 and
// 256), with every length a compile-time constant and kFx8Threads threads.
// The arithmetic and its order are those of row_fx_body (the results are
// bitwise the same); the data movement differs:
//  * complex element i of a field's row lives in slot swz(i), a rotation
//    inside each group of 8 slots (16-byte slots: 8 slots span the 32
//    banks): rotation 3 (i / 24) for R0 = 3, i / 8 for R0 = 2.  With it every
//    8-lane phase of every butterfly pass of the three stages touches 8
//    distinct bank groups (the plain layout had up to 3-way conflicts);
//  * for R0 = 3 the radix-8 stage at sub-length 3 runs its butterflies
//    k-major, which keeps the stage conflict-free and gives whole warps
//    k = 0, whose twiddles are 1 and are skipped (exact: a Q61 twiddle of 1
//    multiplies exactly);
//  * loops over (order, field) pairs stride by a multiple of the field
//    count, so a thread keeps one field: one running maximum per thread
//    instead of a shared atomic per element, block scales in registers;
//  * the digit reversal of the in-place DIT input is arithmetic:
//    natural index q = 64 t0 + 8 t1 + t2 sits at t0 + R0 (t1 + 8 t2).
constexpr int kFx8Threads = 128;

template <int R0>
struct Fx8 {
  static constexpr int n = 64 * R0, N = 2 * n, fs = n + 1;  // fs odd: field-fastest passes spread over banks
  static constexpr int hb = (R0 == 3 ? 56 - 8 : 56 - 7);     // min(52, 56 - ceil(log2 n))
  static __device__ __forceinline__ int swz(int i) {
    return R0 == 3 ? ((i & ~7) | ((i + 3 * (i / 24)) & 7)) : ((i & ~7) | ((i + (i >> 3)) & 7));
  }
  static __device__ __forceinline__ int rev(int q) { return (q >> 6) + R0 * (((q >> 3) & 7) + 8 * (q & 7)); }
};

template <int R0, bool INV, int R, int LS, bool DIT, bool TW, bool CONV, int NFLD>
__device__ __forceinline__ void fx8_stage(cfx* __restrict__ x, const FxW* __restrict__ tw, const FxConst& kc,
                                          const float* sqa, const float* sqb) {
  using Row = Fx8<R0>;
  constexpr int n = Row::n, nb = n / R, NS = LS * R, stride = n / NS, G = nb / LS;
  constexpr bool kmajor = R0 == 3 && LS == R0;
#pragma unroll 1
  for (int idx = threadIdx.x; idx < NFLD * nb; idx += kFx8Threads) {
    int f, g, k;
    if constexpr (kmajor) {
      g = idx % G;
      const int r = idx / G;
      f = r % NFLD;
      k = r / NFLD;
    } else {
      f = idx / nb;
      const int jj = idx - f * nb;
      g = jj / LS;
      k = jj - g * LS;
    }
    cfx* y = x + f * Row::fs;
    const int base = g * NS + k;
    cfx v[R];
    if constexpr (CONV) {
      const float pa = sqa[f], pb = sqb[f];
#pragma unroll
      for (int t = 0; t < R; ++t) {
        const float4 w = reinterpret_cast<const float4*>(y)[Row::swz(base + t * LS)];
        v[t] = cfx{df_to_fx(df{w.x, w.y}, pa, pb), df_to_fx(df{w.z, w.w}, pa, pb)};
      }
    } else {
#pragma unroll
      for (int t = 0; t < R; ++t) v[t] = y[Row::swz(base + t * LS)];
    }
    const bool tw_on = TW && (!kmajor || k != 0);
    if (DIT && tw_on) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = fx_cmul<INV>(v[t], fx_ldw(&tw[2 * (k * t * stride)]));
    }
    butterfly_fx<INV, R>(v, kc);
    if (!DIT && tw_on) {
#pragma unroll
      for (int t = 1; t < R; ++t) v[t] = fx_cmul<INV>(v[t], fx_ldw(&tw[2 * (k * t * stride)]));
    }
#pragma unroll
    for (int t = 0; t < R; ++t) y[Row::swz(base + t * LS)] = v[t];
  }
}

// In-place inverse (DIT, digit-reversed input) or forward (DIF, with the
// double-float rows rounded to fixed point by its first stage) transforms.
template <int R0, bool INV, int NFLD>
__device__ __forceinline__ void fx8_fft(cfx* x, const FxW* __restrict__ tw, const FxConst& kc, const float* sqa,
                                        const float* sqb) {
  if constexpr (INV) {
    fx8_stage<R0, true, R0, 1, true, false, false, NFLD>(x, tw, kc, nullptr, nullptr);
    __syncthreads();
    fx8_stage<R0, true, 8, R0, true, true, false, NFLD>(x, tw, kc, nullptr, nullptr);
    __syncthreads();
    fx8_stage<R0, true, 8, 8 * R0, true, true, false, NFLD>(x, tw, kc, nullptr, nullptr);
    __syncthreads();
  } else {
    fx8_stage<R0, false, 8, 8 * R0, false, true, true, NFLD>(x, tw, kc, sqa, sqb);
    __syncthreads();
    fx8_stage<R0, false, 8, R0, false, true, false, NFLD>(x, tw, kc, nullptr, nullptr);
    __syncthreads();
    fx8_stage<R0, false, R0, 1, false, false, false, NFLD>(x, tw, kc, nullptr, nullptr);
    __syncthreads();
  }
}

template <class Pw, int IN_MODE, int OUT_MODE, int R0>
__device__ __forceinline__ void row_fx8_body(const RowArgs& a, const Pw& pw, const FxW* __restrict__ twfx,
                                             const FxConst& kc, int bx, int by) {
  using Row = Fx8<R0>;
  constexpr int NIN = Pw::NIN, NOUT = Pw::NOUT;
  constexpr int NF = NIN > NOUT ? NIN : NOUT;
  constexpr int n = Row::n, N = Row::N, fs = Row::fs, hb = Row::hb, T = kFx8Threads;
  // (order, field) passes: stride PS, a multiple of the field count
  constexpr int PSI = (T / NIN) * NIN, QSI = T / NIN;
  constexpr int PSO = (T / NOUT) * NOUT, QSO = T / NOUT;
  extern __shared__ cfx smem_fx[];
  __shared__ unsigned s_bits;
  __shared__ int s_in[NF];
  __shared__ unsigned s_key[NF];
  __shared__ unsigned s_omax[NF];
  __shared__ float s_pa[NF], s_pb[NF], s_qa[NF], s_qb[NF];
  __shared__ RowDf s_rc;
  __shared__ df s_wj;
  const int j = bx, b = by, tid = threadIdx.x;
  const int L = a.L, ldm = L + 1;
  cfx* buf0 = smem_fx;
  if (tid == 0) s_bits = 0u;
  if (tid < NF) {
    s_key[tid] = 0u;
    s_omax[tid] = 0u;
  }
  if (tid == 0) {
    s_rc = pw.df_row(a.coslat[j], a.fgrid ? a.fgrid[j] : 0.0);
    s_wj = (OUT_MODE == kOutG && a.wq) ? df_from_double(a.wq[j]) : df{1.f, 0.f};
  }
  const long sq = (long)a.nblk * a.nlat;
  float4* block = nullptr;
  if (IN_MODE == kInF || OUT_MODE == kOutG)
    block = reinterpret_cast<float4*>(a.FG) + fg_index(b, 0, 0, j, L, a.nblk, a.nlat);
  const long sqo = a.G ? (long)a.gblk * a.nlat : sq;
  float4* oblock = nullptr;
  if (OUT_MODE == kOutG)
    oblock = a.G ? reinterpret_cast<float4*>(a.G) + fg_index(b, 0, 0, j, L, a.gblk, a.nlat) : block;
  __syncthreads();

  // ---- 1. grid rows of the inputs, in buf0
  if constexpr (IN_MODE == kInF) {
    if (tid < PSI) {  // largest |hi| of this thread's field over its orders
      const int f = tid % NIN;
      unsigned mx = 0u;
      for (int q = tid / NIN; q < ldm; q += QSI) {
        const float4 w = block[(long)q * sq + f];
        mx = max(mx, max(__float_as_uint(w.x) & 0x7FFFFFFFu, q == 0 ? 0u : __float_as_uint(w.z) & 0x7FFFFFFFu));
      }
      if (mx) atomicMax(&s_key[f], mx);
    }
    __syncthreads();
    if (tid < NIN) {
      const unsigned key = s_key[tid];
      const int S = (key >> 23) == 0 ? 0 : fkey_exp(key) - hb;
      s_in[tid] = S;
      fx_pow2_split(S, s_pa[tid], s_pb[tid]);
      fx_pow2_split(-S, s_qa[tid], s_qb[tid]);
    }
    __syncthreads();
    if (tid < PSI) {
      // half-length complex input of the real inverse FFT, by pairs (q, n-q)
      // (as row_fx_body), written to the digit-reversed slots
      const int f = tid % NIN;
      const float qa = s_qa[f], qb = s_qb[f];
      cfx* z = buf0 + f * fs;
      for (int q = tid / NIN; q <= n / 2; q += QSI) {
        const int qn = n - q;
        cfx hq = cfx{0, 0}, hn = cfx{0, 0};
        if (q <= L) {
          const float4 w = block[(long)q * sq + f];
          hq = cfx{df_to_fx(df{w.x, w.y}, qa, qb), q == 0 ? 0LL : df_to_fx(df{w.z, w.w}, qa, qb)};
        }
        if (q > 0 && qn <= L) {
          const float4 w = block[(long)qn * sq + f];
          hn = cfx{df_to_fx(df{w.x, w.y}, qa, qb), df_to_fx(df{w.z, w.w}, qa, qb)};
        }
        const cfx A = fx_add(hq, fx_conj(hn));
        const cfx B = fx_sub(hq, fx_conj(hn));
        const cfx P = fx_i<true>(fx_cmul<true>(B, fx_ldw(&twfx[q])));
        z[Row::swz(Row::rev(q))] = fx_add(A, P);
        if (q > 0 && qn > q) z[Row::swz(Row::rev(qn))] = fx_conj(fx_sub(A, P));
      }
    }
    __syncthreads();
    fx8_fft<R0, true, NIN>(buf0, twfx, kc, nullptr, nullptr);
  } else {
    df* x0 = reinterpret_cast<df*>(buf0);
    for (int idx = tid; idx < NIN * N; idx += T) {
      const int f = idx / N, k = idx - f * N;
      x0[2 * (f * fs + Row::swz(k >> 1)) + (k & 1)] =
          df_of_f64(a.gin[(long)b * a.gin_b + (long)f * a.gin_f + (long)j * N + k]);
    }
    __syncthreads();
  }

  // ---- 2. pointwise products (double-float), weighted by the row's quadrature
  // weight; in place (each point is read before it is written, by one thread)
  df* xout = reinterpret_cast<df*>(buf0);
  {
    const RowDf rc = s_rc;
    const df wj = s_wj;
    const long long* xi = reinterpret_cast<const long long*>(buf0);
    const df* xd = reinterpret_cast<const df*>(buf0);
    unsigned bits = 0u;
    unsigned omax[NOUT];
#pragma unroll
    for (int f = 0; f < NOUT; ++f) omax[f] = 0u;
    float pa[NIN], pb[NIN];
    if constexpr (IN_MODE == kInF) {
#pragma unroll
      for (int f = 0; f < NIN; ++f) {
        pa[f] = s_pa[f];
        pb[f] = s_pb[f];
      }
    }
#pragma unroll 1
    for (int it = 0; it < N / T; ++it) {
      const int k = tid + it * T;
      const int slot = 2 * Row::swz(k >> 1) + (k & 1);
      df in[NIN], out[NOUT];
#pragma unroll
      for (int f = 0; f < NIN; ++f)
        in[f] = IN_MODE == kInF ? fx_to_df(xi[2 * f * fs + slot], pa[f], pb[f]) : xd[2 * f * fs + slot];
      bits |= pw.df_op(rc, in, out);
#pragma unroll
      for (int f = 0; f < NOUT; ++f) {
        if (OUT_MODE == kOutG && a.wq) out[f] = df_mul(out[f], wj);
        xout[2 * f * fs + slot] = out[f];
        omax[f] = max(omax[f], __float_as_uint(out[f].hi) & 0x7FFFFFFFu);
      }
    }
    if (a.status && bits) atomicOr(&s_bits, bits);
    if (OUT_MODE == kOutG) {
#pragma unroll
      for (int f = 0; f < NOUT; ++f) {
        unsigned v = omax[f];
        for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
        if ((tid & 31) == 0 && v) atomicMax(&s_omax[f], v);
      }
    }
  }
  __syncthreads();
  if (a.status && tid == 0 && s_bits) atomicOr(&a.status[b], s_bits);

  // ---- 3. outputs
  if constexpr (OUT_MODE == kOutGrid) {
    for (int idx = tid; idx < NOUT * N; idx += T) {
      const int f = idx / N, k = idx - f * N;
      a.gout[(long)b * a.gout_b + (long)f * a.gout_f + (long)j * N + k] =
          f64_of_df(xout[2 * (f * fs + Row::swz(k >> 1)) + (k & 1)]);
    }
  } else {
    if (tid < NOUT) {
      const unsigned key = s_omax[tid];
      const int S = (key >> 23) == 0 ? 0 : fkey_exp(key) - hb;
      s_in[tid] = S;
      fx_pow2_split(-S, s_pa[tid], s_pb[tid]);
    }
    __syncthreads();
    fx8_fft<R0, false, NOUT>(buf0, twfx, kc, s_pa, s_pb);
    if (tid < PSO) {
      const int f = tid % NOUT;
      const int e = s_in[f] - 1;  // R2 / 2 in units of 2^S
      const cfx* Zf = buf0 + f * fs;
      for (int q = tid / NOUT; q < ldm; q += QSO) {
        const cfx zq = Zf[Row::swz(Row::rev(q))];
        const cfx zn = fx_conj(Zf[Row::swz(Row::rev(q == 0 ? 0 : n - q))]);
        const cfx E2 = fx_add(zq, zn);
        const cfx D = fx_sub(zq, zn);
        const cfx O2 = cfx{D.im, -D.re};
        const cfx R2 = fx_add(E2, fx_cmul<false>(O2, fx_ldw(&twfx[q])));
        reinterpret_cast<longlong2*>(oblock)[(long)q * sqo + f] = make_longlong2(pk_pack(R2.re, e), pk_pack(R2.im, e));
      }
    }
  }
}

template <class Pw, int IN_MODE, int OUT_MODE, int R0>
__global__ void __launch_bounds__(kFx8Threads, 6) row_kernel_fx8(RowArgs a, Pw pw, const FxW* __restrict__ twfx,
                                                                 FxConst kc) {
  row_fx8_body<Pw, IN_MODE, OUT_MODE, R0>(a, pw, twfx, kc, blockIdx.x, blockIdx.y);
}

template <class Pw>
constexpr size_t row_fx8_smem_bytes(int R0) {
  constexpr int NF = Pw::NIN > Pw::NOUT ? Pw::NIN : Pw::NOUT;
  return (size_t)NF * (64 * R0 + 1) * sizeof(cfx);
}

// Dynamic shared memory of row_kernel_fx: one row buffer for the in-place
// FFTs, a second one for the staged spectra of the direct DFT.
template <class Pw>
inline size_t row_fx_smem_bytes(const FftInfo& f) {
  constexpr int NF = Pw::NIN > Pw::NOUT ? Pw::NIN : Pw::NOUT;
  return (size_t)(f.use_fft ? 1 : 2) * NF * (f.n + 1) * sizeof(cfx);
}

template <class Pw, int IN_MODE, int OUT_MODE, class FFT>
__global__ void __launch_bounds__(256, 3) row_kernel_fx(RowArgs a, Pw pw, const FxW* __restrict__ twfx,
                                                     const float4* __restrict__ twdf, FxConst kc) {
  row_fx_body<Pw, IN_MODE, OUT_MODE, FFT>(a, pw, twfx, twdf, kc, blockIdx.x, blockIdx.y);
}

}  // namespace aeolus
