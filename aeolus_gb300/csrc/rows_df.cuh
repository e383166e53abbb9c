// Longitude stage in double-float arithmetic (split-precision path).
//
// All additions use the Dekker-style df addition (error relative to the
// operands -- the normwise bound that FFT backward stability rests on).
//
// Same structure as row_kernel (rows.cuh): per (latitude row, member) the
// order spectra go through a half-length complex Stockham FFT (radix 2/3/4/5)
// to grid values, the pointwise products are formed, and a forward FFT
// gives the weighted order spectra -- but every operation is a df (f32
// pair) operation, ~2^-48 relative error, on GB300's f32 pipe.  Spectra in
// the F/G blocks hold double-float words (float4 = re.hi, re.lo, im.hi,
// im.lo per complex value) written and read by the tensor-core stages, so
// the row stage touches no f64 arithmetic at all.
#pragma once

#include "df.cuh"
#include "rows.cuh"

namespace aeolus {

template <bool INV, int R>
__device__ __forceinline__ void butterfly_df(cdf* v, const DfConst& k) {
  const float sg = INV ? 1.0f : -1.0f;
  if constexpr (R == 2) {
    const cdf a = v[0], b = v[1];
    v[0] = cdf_addf(a, b);
    v[1] = cdf_subf(a, b);
  } else if constexpr (R == 4) {
    const cdf s02 = cdf_addf(v[0], v[2]), d02 = cdf_subf(v[0], v[2]);
    const cdf s13 = cdf_addf(v[1], v[3]), d13 = cdf_subf(v[1], v[3]);
    const cdf id13 = cdf_scale2(sg, cdf_i(d13));
    v[0] = cdf_addf(s02, s13);
    v[2] = cdf_subf(s02, s13);
    v[1] = cdf_addf(d02, id13);
    v[3] = cdf_subf(d02, id13);
  } else if constexpr (R == 3) {
    const cdf s = cdf_addf(v[1], v[2]), d = cdf_subf(v[1], v[2]);
    const cdf t = cdf_subf(v[0], cdf_scale2(0.5f, s));
    const cdf id = cdf_scale(k.h3, cdf_scale2(sg, cdf_i(d)));
    v[0] = cdf_addf(v[0], s);
    v[1] = cdf_addf(t, id);
    v[2] = cdf_subf(t, id);
  } else {  // R == 5
    const cdf a1 = cdf_addf(v[1], v[4]), a2 = cdf_addf(v[2], v[3]);
    const cdf b1 = cdf_subf(v[1], v[4]), b2 = cdf_subf(v[2], v[3]);
    const cdf t1 = cdf_addf(v[0], cdf_addf(cdf_scale(k.c1, a1), cdf_scale(k.c2, a2)));
    const cdf t2 = cdf_addf(v[0], cdf_addf(cdf_scale(k.c2, a1), cdf_scale(k.c1, a2)));
    const cdf u1 = cdf_addf(cdf_scale(k.s1, b1), cdf_scale(k.s2, b2));
    const cdf u2 = cdf_subf(cdf_scale(k.s2, b1), cdf_scale(k.s1, b2));
    const cdf iu1 = cdf_scale2(sg, cdf_i(u1)), iu2 = cdf_scale2(sg, cdf_i(u2));
    v[0] = cdf_addf(v[0], cdf_addf(a1, a2));
    v[1] = cdf_addf(t1, iu1);
    v[4] = cdf_subf(t1, iu1);
    v[2] = cdf_addf(t2, iu2);
    v[3] = cdf_subf(t2, iu2);
  }
}

template <bool INV, int R>
__device__ __forceinline__ void fft_stage_df(const cdf* __restrict__ src, cdf* __restrict__ dst, int nf, int n, int fs,
                                             int Ls, unsigned nb_rcp, unsigned ls_rcp, const float4* __restrict__ tw,
                                             const DfConst& kc) {
  const int nb = n / R, Ns = Ls * R, stride = n / Ns;
  for (int idx = threadIdx.x; idx < nf * nb; idx += blockDim.x) {
    const int f = div_rcp(idx, nb, nb_rcp), jj = idx - f * nb;
    const int q = div_rcp(jj, Ls, ls_rcp), k = jj - q * Ls;
    const cdf* x = src + (long)f * fs;
    cdf* y = dst + (long)f * fs;
    cdf v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = x[jj + t * nb];
    if (k != 0) {
#pragma unroll
      for (int t = 1; t < R; ++t) {
        cdf w = cdf_from_f4(__ldg(&tw[2 * (k * t * stride)]));
        if (INV) w = cdf_conj(w);
        v[t] = cdf_mulf(v[t], w);
      }
    }
    butterfly_df<INV, R>(v, kc);
    const int base = q * Ns + k;
#pragma unroll
    for (int t = 0; t < R; ++t) y[base + t * Ls] = v[t];
  }
}

template <bool INV>
__device__ cdf* fft_run_df(cdf* src, cdf* dst, int nf, int fs, const FftInfo& fi, const float4* __restrict__ tw,
                           const DfConst& kc) {
  const int n = fi.n;
  int Ls = 1;
  for (int s = 0; s < fi.nfac; ++s) {
    const int r = fi.fac[s];
    switch (r) {
      case 4: fft_stage_df<INV, 4>(src, dst, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw, kc); break;
      case 2: fft_stage_df<INV, 2>(src, dst, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw, kc); break;
      case 3: fft_stage_df<INV, 3>(src, dst, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw, kc); break;
      default: fft_stage_df<INV, 5>(src, dst, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw, kc); break;
    }
    __syncthreads();
    cdf* tmp = src;
    src = dst;
    dst = tmp;
    Ls *= r;
  }
  return src;
}

template <class Pw, int IN_MODE, int OUT_MODE>
__device__ __forceinline__ void row_df_body(const RowArgs& a, const Pw& pw, const float4* __restrict__ twdf,
                                            const DfConst& kc, int bx, int by) {
  constexpr int NIN = Pw::NIN, NOUT = Pw::NOUT;
  constexpr int NF = NIN > NOUT ? NIN : NOUT;
  extern __shared__ cdf smem_df[];
  __shared__ unsigned s_bits;
  const int j = bx, b = by;
  const int N = a.fft.N, n = a.fft.n, L = a.L;
  const int ldm = L + 1;
  const int ns = n + 1;  // padded field stride of the smem rows (see row_body)
  cdf* buf0 = smem_df;
  cdf* buf1 = smem_df + (long)NF * ns;
  if (threadIdx.x == 0) s_bits = 0u;
  // this row's order spectra: field f, order q at block[q * sq + f]
  const long sq = (long)a.nblk * a.nlat;
  float4* block = nullptr;
  if (IN_MODE == kInF || OUT_MODE == kOutG)
    block = reinterpret_cast<float4*>(a.FG) + fg_index(b, 0, 0, j, L, a.nblk, a.nlat);

  // ---- 1. grid rows of the inputs (real df rows, field stride 2n)
  df* xin = reinterpret_cast<df*>(buf0);
  if (IN_MODE == kInF) {
    if (a.fft.use_fft) {
      for (int idx = threadIdx.x; idx < NIN * n; idx += blockDim.x) {
        const int q = idx / NIN, f = idx - q * NIN;  // fields fastest: contiguous global reads
        const float4* Ff = block + f;
        cdf hq = q <= L ? cdf_from_f4(Ff[(long)(q) * sq]) : cdf_zero();
        if (q == 0) hq.im = df{0.f, 0.f};
        const int qn = n - q;
        const cdf hn = (q > 0 && qn <= L) ? cdf_from_f4(Ff[(long)(qn) * sq]) : cdf_zero();
        const cdf A = cdf_addf(hq, cdf_conj(hn));
        const cdf B = cdf_subf(hq, cdf_conj(hn));
        const cdf e = cdf_conj(cdf_from_f4(__ldg(&twdf[q])));
        buf0[(long)f * ns + q] = cdf_addf(A, cdf_i(cdf_mulf(e, B)));
      }
      __syncthreads();
      xin = reinterpret_cast<df*>(fft_run_df<true>(buf0, buf1, NIN, ns, a.fft, twdf, kc));
    } else {
      df* x0 = reinterpret_cast<df*>(buf0);
      for (int idx = threadIdx.x; idx < NIN * N; idx += blockDim.x) {
        const int f = idx / N, k = idx - f * N;
        const float4* Ff = block + f;
        df acc = df{0.f, 0.f};
        int e = 0;
        for (int m = 1; m <= L; ++m) {
          e += k;
          if (e >= N) e -= N;
          const cdf w = cdf_from_f4(__ldg(&twdf[e]));
          const cdf F = cdf_from_f4(Ff[(long)(m) * sq]);
          acc = df_add_fast(acc, df_add_fast(df_mul(F.re, w.re), df_mul(F.im, w.im)));
        }
        x0[(long)f * 2 * ns + k] = df_add_fast(df{Ff[(long)(0) * sq].x, Ff[(long)(0) * sq].y}, df_scale2(acc, 2.0f));
      }
      __syncthreads();
    }
  } else {
    df* x0 = reinterpret_cast<df*>(buf0);
    for (int idx = threadIdx.x; idx < NIN * N; idx += blockDim.x) {
      const int f = idx / N, k = idx - f * N;
      x0[(long)f * 2 * ns + k] = df_from_double(a.gin[(long)b * a.gin_b + (long)f * a.gin_f + (long)j * N + k]);
    }
    __syncthreads();
  }

  // ---- 2. pointwise products
  df* xout = (xin == reinterpret_cast<df*>(buf0)) ? reinterpret_cast<df*>(buf1) : reinterpret_cast<df*>(buf0);
  {
    const RowDf rc = pw.df_row(a.coslat[j], a.fgrid ? a.fgrid[j] : 0.0);
    unsigned bits = 0u;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
      df in[NIN], out[NOUT];
#pragma unroll
      for (int f = 0; f < NIN; ++f) in[f] = xin[(long)f * 2 * ns + k];
      bits |= pw.df_op(rc, in, out);
#pragma unroll
      for (int f = 0; f < NOUT; ++f) xout[(long)f * 2 * ns + k] = out[f];
    }
    if (a.status && bits) atomicOr(&s_bits, bits);
  }
  __syncthreads();
  if (a.status && threadIdx.x == 0 && s_bits) atomicOr(&a.status[b], s_bits);

  // ---- 3. outputs
  if (OUT_MODE == kOutGrid) {
    for (int idx = threadIdx.x; idx < NOUT * N; idx += blockDim.x) {
      const int f = idx / N, k = idx - f * N;
      a.gout[(long)b * a.gout_b + (long)f * a.gout_f + (long)j * N + k] = df_to_double(xout[(long)f * 2 * ns + k]);
    }
  } else {
    const df wj = a.wq ? df_from_double(a.wq[j]) : df{1.f, 0.f};
    if (a.fft.use_fft) {
      cdf* zin = reinterpret_cast<cdf*>(xout);
      cdf* zother = (zin == buf0) ? buf1 : buf0;
      cdf* Z = fft_run_df<false>(zin, zother, NOUT, ns, a.fft, twdf, kc);
      for (int idx = threadIdx.x; idx < NOUT * ldm; idx += blockDim.x) {
        const int q = idx / NOUT, f = idx - q * NOUT;  // fields fastest: contiguous global writes
        const cdf* Zf = Z + (long)f * ns;
        const cdf zq = Zf[q];
        const cdf zn = cdf_conj(Zf[q == 0 ? 0 : n - q]);
        const cdf E = cdf_scale2(0.5f, cdf_addf(zq, zn));
        const cdf D = cdf_subf(zq, zn);
        const cdf O = cdf{df_scale2(D.im, 0.5f), df_scale2(D.re, -0.5f)};  // -(i/2) D
        const cdf R = cdf_scale(wj, cdf_addf(E, cdf_mulf(cdf_from_f4(__ldg(&twdf[q])), O)));
        block[(long)q * sq + f] = make_float4(R.re.hi, R.re.lo, R.im.hi, R.im.lo);
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
        const df gr = df_mul(wj, sr), gi = df_mul(wj, si);
        block[(long)q * sq + f] = make_float4(gr.hi, gr.lo, gi.hi, gi.lo);
      }
    }
  }
}

template <class Pw, int IN_MODE, int OUT_MODE>
__global__ void __launch_bounds__(256) row_kernel_df(RowArgs a, Pw pw, const float4* __restrict__ twdf, DfConst kc) {
  row_df_body<Pw, IN_MODE, OUT_MODE>(a, pw, twdf, kc, blockIdx.x, blockIdx.y);
}

}  // namespace aeolus
