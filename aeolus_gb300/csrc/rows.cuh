// Longitude stage of the Gauss transform, one CTA per (latitude row, member):
//   order spectrum F_m (m <= L) --c2r--> grid row --pointwise--> products
//   --r2c--> weighted order spectrum G_m.
// The real FFTs run as half-length complex mixed-radix (2/3/4/5) Stockham
// FFTs in shared memory; lengths outside that set (odd nlon, nlon/2 with other
// prime factors, or L >= nlon/2) use a direct DFT over the twiddle table.
#pragma once

#include "common.cuh"
#include "df.cuh"

namespace aeolus {

enum { kInF = 0, kInGrid = 1 };
enum { kOutGrid = 0, kOutG = 1 };

struct RowArgs {
  int L, nlat, batch;
  FftInfo fft;
  const int* irev;        // [n] digit-reversed position of index q (fixed-point in-place FFTs)
  const double2* tw;      // [N] exp(-2 pi i q / N)
  const double* coslat;   // [nlat] clamped cos(latitude)
  const double* fgrid;    // [nlat] synthesis of the unit (1,0) mode
  const double* wq;       // [nlat] quadrature weight of a point of row j (NULL: unit weights)
  int unit_weights;       // launch_rows: leave wq NULL (adjoint of synthesis)
  // kInF: spectra F[b][j][nblk][L+1]; kOutG writes G into the same blocks,
  // or (fixed-point rows, G != NULL) into G with gblk fields per block
  double2* FG;
  int nblk;
  double2* G;
  int gblk;
  // kInGrid: grid[b * gin_b + f * gin_f + j * N + k]
  const double* gin;
  long gin_b, gin_f;
  // kOutGrid: out[b * gout_b + f * gout_f + j * N + k]
  double* gout;
  long gout_b, gout_f;
  unsigned* status;       // optional per-member state bits
};

// x / d through the stage's 32-bit reciprocal (exact for x * d < 2^32).
__device__ __forceinline__ int div_rcp(int x, int d, unsigned rcp) {
  return d == 1 ? x : (int)__umulhi((unsigned)x, rcp);
}

// Radix-R butterfly, forward (INV=false, exp(-2 pi i/R)) or inverse.  R is a
// compile-time constant so the R values stay in registers.
template <bool INV, int R>
__device__ __forceinline__ void butterfly(double2* v) {
  const double sg = INV ? 1.0 : -1.0;  // sign of the imaginary exponent
  if constexpr (R == 2) {
    double2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if constexpr (R == 4) {
    double2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    double2 s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
    double2 id13 = cscale(sg, ci(d13));  // sg * i * (v1 - v3)
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, id13);
    v[3] = csub(d02, id13);
  } else if constexpr (R == 3) {
    const double h = 0.86602540378443864676;  // sin(2 pi / 3)
    double2 s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
    double2 t = make_double2(v[0].x - 0.5 * s.x, v[0].y - 0.5 * s.y);
    double2 id = cscale(sg * h, ci(d));
    v[0] = cadd(v[0], s);
    v[1] = cadd(t, id);
    v[2] = csub(t, id);
  } else {  // R == 5
    const double c1 = 0.30901699437494742410, c2 = -0.80901699437494742410;
    const double s1 = 0.95105651629515357212, s2 = 0.58778525229247312917;
    double2 a1 = cadd(v[1], v[4]), a2 = cadd(v[2], v[3]);
    double2 b1 = csub(v[1], v[4]), b2 = csub(v[2], v[3]);
    double2 t1 = make_double2(v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y);
    double2 t2 = make_double2(v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y);
    double2 u1 = make_double2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y);
    double2 u2 = make_double2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y);
    double2 iu1 = cscale(sg, ci(u1)), iu2 = cscale(sg, ci(u2));
    v[0] = cadd(v[0], cadd(a1, a2));
    v[1] = cadd(t1, iu1);
    v[4] = csub(t1, iu1);
    v[2] = cadd(t2, iu2);
    v[3] = csub(t2, iu2);
  }
}

// One Stockham stage of radix R over nf transforms of length n (sub-
// transform length Ls before the stage).
template <bool INV, int R>
__device__ __forceinline__ void fft_stage(const double2* __restrict__ src, double2* __restrict__ dst, int nf, int n,
                                          int fs, int Ls, unsigned nb_rcp, unsigned ls_rcp,
                                          const double2* __restrict__ tw) {
  const int nb = n / R, Ns = Ls * R, stride = n / Ns;
  for (int idx = threadIdx.x; idx < nf * nb; idx += blockDim.x) {
    const int f = div_rcp(idx, nb, nb_rcp), jj = idx - f * nb;
    const int q = div_rcp(jj, Ls, ls_rcp), k = jj - q * Ls;
    const double2* x = src + (long)f * fs;
    double2* y = dst + (long)f * fs;
    double2 v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = x[jj + t * nb];
    if (k != 0) {
#pragma unroll
      for (int t = 1; t < R; ++t) {
        double2 w = __ldg(&tw[2 * (k * t * stride)]);
        if (INV) w.y = -w.y;
        v[t] = cmul(v[t], w);
      }
    }
    butterfly<INV, R>(v);
    const int base = q * Ns + k;
#pragma unroll
    for (int t = 0; t < R; ++t) y[base + t * Ls] = v[t];
  }
}

// nf independent length-n complex FFTs (field stride fs) in shared memory,
// Stockham autosort, ping-pong between src and dst; returns the buffer that
// holds the result.  Ends with __syncthreads().
template <bool INV>
__device__ double2* fft_run(double2* src, double2* dst, int nf, int fs, const FftInfo& fi,
                            const double2* __restrict__ tw) {
  const int n = fi.n;
  int Ls = 1;
  for (int s = 0; s < fi.nfac; ++s) {
    const int r = fi.fac[s];
    switch (r) {
      case 4: fft_stage<INV, 4>(src, dst, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw); break;
      case 2: fft_stage<INV, 2>(src, dst, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw); break;
      case 3: fft_stage<INV, 3>(src, dst, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw); break;
      default: fft_stage<INV, 5>(src, dst, nf, n, fs, Ls, fi.nbm[s], fi.lsm[s], tw); break;
    }
    __syncthreads();
    double2* tmp = src;
    src = dst;
    dst = tmp;
    Ls *= r;
  }
  return src;
}

template <class Pw, int IN_MODE, int OUT_MODE>
__device__ __forceinline__ void row_body(const RowArgs& a, const Pw& pw, int bx, int by) {
  constexpr int NIN = Pw::NIN, NOUT = Pw::NOUT;
  constexpr int NF = NIN > NOUT ? NIN : NOUT;
  extern __shared__ double2 smem[];
  __shared__ unsigned s_bits;
  const int j = bx, b = by;
  const int N = a.fft.N, n = a.fft.n, L = a.L;
  const int ldm = L + 1;
  // smem rows: field stride ns = n + 1 complex values, so accesses that
  // interleave the fields (field-fastest global order) are bank-conflict free
  const int ns = n + 1;
  double2* buf0 = smem;
  double2* buf1 = smem + (long)NF * ns;
  if (threadIdx.x == 0) s_bits = 0u;
  // this row's order spectra: field f, order q at block[q * sq + f]
  const long sq = (long)a.nblk * a.nlat;
  double2* block = nullptr;
  if (IN_MODE == kInF || OUT_MODE == kOutG) block = a.FG + fg_index(b, 0, 0, j, L, a.nblk, a.nlat);

  // ---- 1. grid rows of the NIN input fields (real rows, field stride 2n doubles)
  double* xin = reinterpret_cast<double*>(buf0);
  if (IN_MODE == kInF) {
    if (a.fft.use_fft) {
      // Z_q = (H_q + conj H_{n-q}) + i e^{+2 pi i q/N} (H_q - conj H_{n-q}),
      // H_q = F_q for 1 <= q <= L, H_0 = Re F_0, zero above L.
      for (int idx = threadIdx.x; idx < NIN * n; idx += blockDim.x) {
        const int q = idx / NIN, f = idx - q * NIN;  // fields fastest: contiguous global reads
        const double2* Ff = block + f;
        double2 hq = q <= L ? Ff[(long)(q) * sq] : make_double2(0.0, 0.0);
        if (q == 0) hq.y = 0.0;
        const int qn = n - q;
        double2 hn = (q > 0 && qn <= L) ? Ff[(long)(qn) * sq] : make_double2(0.0, 0.0);
        double2 A = cadd(hq, cconj(hn));
        double2 B = csub(hq, cconj(hn));
        double2 e = cconj(__ldg(&a.tw[q]));
        buf0[(long)f * ns + q] = cadd(A, ci(cmul(e, B)));
      }
      __syncthreads();
      xin = reinterpret_cast<double*>(fft_run<true>(buf0, buf1, NIN, ns, a.fft, a.tw));
    } else {
      // x_k = Re F_0 + 2 sum_{m=1..L} Re(F_m e^{+2 pi i m k/N})
      double* x0 = reinterpret_cast<double*>(buf0);
      for (int idx = threadIdx.x; idx < NIN * N; idx += blockDim.x) {
        const int f = idx / N, k = idx - f * N;
        const double2* Ff = block + f;
        double acc = 0.0;
        int e = 0;
        for (int m = 1; m <= L; ++m) {
          e += k;
          if (e >= N) e -= N;
          double2 w = __ldg(&a.tw[e]);
          double2 F = Ff[(long)(m) * sq];
          acc += F.x * w.x + F.y * w.y;
        }
        x0[(long)f * 2 * ns + k] = Ff[(long)(0) * sq].x + 2.0 * acc;
      }
      __syncthreads();
    }
  } else {
    double* x0 = reinterpret_cast<double*>(buf0);
    for (int idx = threadIdx.x; idx < NIN * N; idx += blockDim.x) {
      const int f = idx / N, k = idx - f * N;
      x0[(long)f * 2 * ns + k] = a.gin[(long)b * a.gin_b + (long)f * a.gin_f + (long)j * N + k];
    }
    __syncthreads();
  }

  // ---- 2. pointwise products into the other buffer
  double* xout = (xin == reinterpret_cast<double*>(buf0)) ? reinterpret_cast<double*>(buf1)
                                                          : reinterpret_cast<double*>(buf0);
  {
    const double c = a.coslat[j];
    const double fg = a.fgrid ? a.fgrid[j] : 0.0;
    unsigned bits = 0u;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
      double in[NIN], out[NOUT];
#pragma unroll
      for (int f = 0; f < NIN; ++f) in[f] = xin[(long)f * 2 * ns + k];
      bits |= pw(c, fg, in, out);
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
      a.gout[(long)b * a.gout_b + (long)f * a.gout_f + (long)j * N + k] = xout[(long)f * 2 * ns + k];
    }
  } else {
    const double wj = a.wq ? a.wq[j] : 1.0;
    if (a.fft.use_fft) {
      double2* zin = reinterpret_cast<double2*>(xout);
      double2* zother = (zin == buf0) ? buf1 : buf0;
      double2* Z = fft_run<false>(zin, zother, NOUT, ns, a.fft, a.tw);
      // R_q = (Z_q + conj Z_{n-q})/2 - (i/2) e^{-2 pi i q/N} (Z_q - conj Z_{n-q})
      for (int idx = threadIdx.x; idx < NOUT * ldm; idx += blockDim.x) {
        const int q = idx / NOUT, f = idx - q * NOUT;  // fields fastest: contiguous global writes
        const double2* Zf = Z + (long)f * ns;
        double2 zq = Zf[q];
        double2 zn = cconj(Zf[q == 0 ? 0 : n - q]);
        double2 E = cscale(0.5, cadd(zq, zn));
        double2 D = csub(zq, zn);
        double2 O = make_double2(0.5 * D.y, -0.5 * D.x);  // -(i/2) D
        double2 R = cadd(E, cmul(__ldg(&a.tw[q]), O));
        block[(long)q * sq + f] = cscale(wj, R);
      }
    } else {
      for (int idx = threadIdx.x; idx < NOUT * ldm; idx += blockDim.x) {
        const int q = idx / NOUT, f = idx - q * NOUT;
        const double* x = xout + (long)f * 2 * ns;
        double sr = 0.0, si = 0.0;
        int e = 0;
        for (int k = 0; k < N; ++k) {
          double2 w = __ldg(&a.tw[e]);
          sr += x[k] * w.x;
          si += x[k] * w.y;
          e += q;
          while (e >= N) e -= N;
        }
        block[(long)q * sq + f] = make_double2(wj * sr, wj * si);
      }
    }
  }
}

template <class Pw, int IN_MODE, int OUT_MODE>
__global__ void __launch_bounds__(256) row_kernel(RowArgs a, Pw pw) {
  row_body<Pw, IN_MODE, OUT_MODE>(a, pw, blockIdx.x, blockIdx.y);
}

template <class Pw>
inline size_t row_smem_bytes(const FftInfo& f) {
  constexpr int NF = Pw::NIN > Pw::NOUT ? Pw::NIN : Pw::NOUT;
  return (size_t)2 * NF * (f.n + 1) * sizeof(double2);
}

// Identity pointwise op for plain synthesis / analysis.
struct PwCopy {
  static constexpr int NIN = 1, NOUT = 1;
  static constexpr bool kIdentity = true;
  __device__ unsigned operator()(double, double, const double* in, double* out) const {
    out[0] = in[0];
    return 0u;
  }
  __device__ RowDf df_row(double c, double) const { return RowDf{df{0.f, 0.f}, df{0.f, 0.f}, (float)c}; }
  __device__ unsigned df_op(const RowDf&, const df* in, df* out) const {
    out[0] = in[0];
    return 0u;
  }
  __device__ unsigned df_op2(const RowDf&, const df2* in, df2* out) const {  // two grid points (packed)
    out[0] = in[0];
    return 0u;
  }
};

}  // namespace aeolus
