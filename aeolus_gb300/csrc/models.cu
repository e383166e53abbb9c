// Operator chains of the BVE and SWE tendencies, RK4, state validation and
// conservation diagnostics.  Each chain is Derive -> synthesis -> Pointwise
// -> analysis -> Epilogue (chains.cuh); the functors below hold the physics.
#include <cmath>

#include "models.cuh"

namespace aeolus {

size_t transform_bytes(const aeolus_plan_impl* p, int op, int batch);  // sht.cu
size_t adjoint_op_bytes(const aeolus_plan_impl* p, int op, int batch);  // adjoint.cu

namespace {

// -------------------------------------------------------------- Jacobian
struct JacDerive {  // a_lam, a_snt, b_lam, b_snt
  static constexpr int NF = 4;
  Spec s;
  const double2* A;
  const double2* B;
  __device__ void column(int b, int l, int m, double2* v) const {
    const long off = (long)b * (s.L + 1) * (s.L + 1);
    const double2* a = A + off;
    const double2* c = B + off;
    const double2 zero = make_double2(0.0, 0.0);
    const int L = s.L;
    v[0] = s.dlam(s.at(a, l, m), m);
    v[1] = cscale(s.ir, s.snt(l >= 1 ? s.at(a, l - 1, m) : zero, l + 1 <= L ? s.at(a, l + 1, m) : zero, l, m));
    v[2] = s.dlam(s.at(c, l, m), m);
    v[3] = cscale(s.ir, s.snt(l >= 1 ? s.at(c, l - 1, m) : zero, l + 1 <= L ? s.at(c, l + 1, m) : zero, l, m));
  }
};

struct TruncEpi {  // 2/3-truncated store
  static constexpr int NF = 1;
  double2* out;
  int L;
  __device__ void finish(int b, int l, int m, const double2* acc) const {
    const int cut = (2 * L) / 3;
    out[((long)b * (L + 1) + l) * (L + 1) + m] = (l > cut || m > cut) ? make_double2(0.0, 0.0) : acc[0];
  }
  __device__ void zero(int b, int l, int m) const {
    out[((long)b * (L + 1) + l) * (L + 1) + m] = make_double2(0.0, 0.0);
  }
};

// ------------------------------------------------------------------ winds
struct WindDerive {  // U = S(psi)/R + (im/R) chi,  V = (im/R) psi - S(chi)/R
  static constexpr int NF = 2;
  Spec s;
  const double2* psi;
  const double2* chi;  // may be null
  __device__ void column(int b, int l, int m, double2* v) const {
    const long off = (long)b * (s.L + 1) * (s.L + 1);
    const double2 zero = make_double2(0.0, 0.0);
    const int L = s.L;
    const double2* p = psi + off;
    double2 U = cscale(s.ir, s.snt(l >= 1 ? s.at(p, l - 1, m) : zero, l + 1 <= L ? s.at(p, l + 1, m) : zero, l, m));
    double2 V = s.dlam(s.at(p, l, m), m);
    if (chi) {
      const double2* c = chi + off;
      U = cadd(U, s.dlam(s.at(c, l, m), m));
      V = csub(V, cscale(s.ir, s.snt(l >= 1 ? s.at(c, l - 1, m) : zero, l + 1 <= L ? s.at(c, l + 1, m) : zero, l, m)));
    }
    v[0] = U;
    v[1] = V;
  }
};

struct WindPw {
  static constexpr int NIN = 2, NOUT = 2;
  static constexpr bool kIdentity = false;
  int nan_guard;  // velocity_from_streamfunction: |cos| < 1e-6 -> 0
  __device__ unsigned operator()(double c, double, const double* in, double* out) const {
    if (nan_guard && c < 1e-6) {
      out[0] = out[1] = 0.0;
    } else {
      out[0] = in[0] / c;
      out[1] = in[1] / c;
    }
    return 0u;
  }
  __device__ RowDf df_row(double c, double) const { return RowDf{df_from_double(1.0 / c), df{0.f, 0.f}, (float)c}; }
  __device__ unsigned df_op(const RowDf& r, const df* in, df* out) const {
    if (nan_guard && r.c < 1e-6f) {
      out[0] = out[1] = df{0.f, 0.f};
    } else {
      out[0] = df_mul(in[0], r.invc);
      out[1] = df_mul(in[1], r.invc);
    }
    return 0u;
  }
};

struct FieldDerive {
  static constexpr int NF = 1;
  const double2* in;
  int L, nf, fi;
  __device__ void column(int b, int l, int m, double2* v) const {
    const long n2 = (long)(L + 1) * (L + 1);
    v[0] = in[((long)b * nf + fi) * n2 + (long)l * (L + 1) + m];
  }
};

// u, v, phi on the state sampling (SWE diagnostics).
struct WindPhiDerive {
  static constexpr int NF = 3;
  Spec s;
  const double2* state;
  __device__ void column(int b, int l, int m, double2* v) const {
    const int L = s.L;
    const long n2 = (long)(L + 1) * (L + 1);
    const double2* z = state + (long)b * 3 * n2;
    const double2* d = z + n2;
    const double2 zero = make_double2(0.0, 0.0);
    const bool lo = l >= 1, hi = l + 1 <= L;
    const double ir = s.ir;
    const double2 psi = s.invlap0(z, l, m), chi = s.invlap0(d, l, m);
    const double2 psi_lo = lo ? s.invlap0(z, l - 1, m) : zero, psi_hi = hi ? s.invlap0(z, l + 1, m) : zero;
    const double2 chi_lo = lo ? s.invlap0(d, l - 1, m) : zero, chi_hi = hi ? s.invlap0(d, l + 1, m) : zero;
    v[0] = cadd(cscale(ir, s.snt(psi_lo, psi_hi, l, m)), s.dlam(chi, m));
    v[1] = csub(s.dlam(psi, m), cscale(ir, s.snt(chi_lo, chi_hi, l, m)));
    v[2] = s.at(z + 2 * n2, l, m);
  }
};

struct WindPhiPw {
  static constexpr int NIN = 3, NOUT = 3;
  static constexpr bool kIdentity = false;
  __device__ unsigned operator()(double c, double, const double* in, double* out) const {
    out[0] = in[0] / c;
    out[1] = in[1] / c;
    out[2] = in[2];
    return 0u;
  }
  __device__ RowDf df_row(double c, double) const { return RowDf{df_from_double(1.0 / c), df{0.f, 0.f}, (float)c}; }
  __device__ unsigned df_op(const RowDf& r, const df* in, df* out) const {
    out[0] = df_mul(in[0], r.invc);
    out[1] = df_mul(in[1], r.invc);
    out[2] = in[2];
    return 0u;
  }
};

// ------------------------------------------------------- reductions
// Deterministic fixed-order block reduction helpers (256 threads).
__device__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

__device__ double block_min(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmin(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

__device__ double block_max(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

// Spectral part of validate_state: non-finite coefficients, monopoles.
__global__ void swe_spectral_check_kernel(int L, const double2* __restrict__ state, unsigned* status) {
  __shared__ double sh[256];
  __shared__ int s_nf;
  const long n2 = (long)(L + 1) * (L + 1);
  const int b = blockIdx.x;
  if (threadIdx.x == 0) s_nf = 0;
  __syncthreads();
  int nf = 0;
  double ss[3] = {0.0, 0.0, 0.0};
  for (int f = 0; f < 3; ++f)
    for (long i = threadIdx.x; i < n2; i += blockDim.x) {
      const double2 v = state[((long)b * 3 + f) * n2 + i];
      if (!(isfinite(v.x) && isfinite(v.y))) nf = 1;
      ss[f] += v.x * v.x + v.y * v.y;
    }
  if (nf) atomicOr(&s_nf, 1);
  unsigned bits = 0u;
  double norm[3];
  for (int f = 0; f < 3; ++f) norm[f] = sqrt(block_sum(ss[f], sh));
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_nf) {
      bits = AEOLUS_STATE_NONFINITE;
    } else {
      for (int f = 0; f < 3; ++f) {
        const double2 a00 = state[((long)b * 3 + f) * n2];
        const double mono = hypot(a00.x, a00.y);
        if (mono > 1e-10 * fmax(norm[f], 1e-30)) bits |= AEOLUS_STATE_MONOPOLE;
      }
    }
    status[b] = bits;
  }
}

// min / max of a grid field per member: mm[b] = (min, max) combined with the
// previous values when `accumulate`.
__global__ void minmax_kernel(long npts, const double* __restrict__ g, double2* mm, int accumulate) {
  __shared__ double sh[256];
  const int b = blockIdx.x;
  double lo = INFINITY, hi = -INFINITY;
  for (long i = threadIdx.x; i < npts; i += blockDim.x) {
    const double v = g[(long)b * npts + i];
    lo = fmin(lo, v);
    hi = fmax(hi, v);
    if (v != v) lo = hi = v;  // propagate NaN
  }
  lo = block_min(lo, sh);
  hi = block_max(hi, sh);
  if (threadIdx.x == 0) {
    if (accumulate) {
      lo = fmin(lo, mm[b].x);
      hi = fmax(hi, mm[b].y);
    }
    mm[b] = make_double2(lo, hi);
  }
}

__global__ void thickness_kernel(int batch, double phi0, const double2* mm, unsigned* status, double* extrema) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  const double lo = phi0 + mm[b].x, hi = phi0 + mm[b].y;
  if (status && !(status[b] & AEOLUS_STATE_NONFINITE) && !(lo > 0.0)) status[b] |= AEOLUS_STATE_THICKNESS;
  if (extrema) {
    extrema[2 * b] = lo;
    extrema[2 * b + 1] = hi;
  }
}

// run/bve/diagnostics.py:52-97, one CTA per member.
__global__ void bve_diag_kernel(int L, double R, double omega, const double2* __restrict__ zeta, double* out) {
  __shared__ double sh[256];
  const int b = blockIdx.x;
  const double2* z = zeta + (long)b * (L + 1) * (L + 1);
  const int cut = (2 * L) / 3;
  const double f10 = 2.0 * omega * kSqrt4PiOver3;
  double Z = 0.0, E = 0.0, Zabs = 0.0, E1 = 0.0, Zhi = 0.0;
  for (int l = threadIdx.x; l <= L; l += blockDim.x) {
    double pl = 0.0, pq = 0.0;
    for (int m = 0; m <= l; ++m) {
      const double2 a = z[(long)l * (L + 1) + m];
      double2 q = a;
      if (l == 1 && m == 0) q.x += f10;
      if (m == 0) {
        pl += a.x * a.x;
        pq += q.x * q.x;
      } else {
        pl += 2.0 * (a.x * a.x + a.y * a.y);
        pq += 2.0 * (q.x * q.x + q.y * q.y);
      }
    }
    const double Zl = 0.5 * R * R * pl;
    const double El = l > 0 ? 0.5 * R * R * R * R * (1.0 / (l * (l + 1.0))) * pl : 0.0;
    Z += Zl;
    E += El;
    Zabs += 0.5 * R * R * pq;
    if (l == 1) E1 = El;
    if (l > cut) Zhi += Zl;
  }
  Z = block_sum(Z, sh);
  E = block_sum(E, sh);
  Zabs = block_sum(Zabs, sh);
  E1 = block_sum(E1, sh);
  Zhi = block_sum(Zhi, sh);
  if (threadIdx.x == 0) {
    double* o = out + 6 * (long)b;
    o[0] = R * R * kSqrt4Pi * z[0].x;
    o[1] = E;
    o[2] = Z;
    o[3] = Zabs;
    o[4] = E1;
    o[5] = Z > 0.0 ? Zhi / Z : 0.0;
  }
}

// run/swe/diagnostics.py:76-173: mass, quadrature energy, L2 norms.
__global__ void swe_invariants_kernel(int L, long npts, int nlon, double R, double phi0, const double2* __restrict__ state,
                                      const double* __restrict__ uvp, const double* __restrict__ wrow,
                                      const double* __restrict__ wpt, double* out) {
  __shared__ double sh[256];
  const int b = blockIdx.x;
  const long n2 = (long)(L + 1) * (L + 1);
  double e = 0.0;
  const double* u = uvp + (long)b * 3 * npts;
  const double* v = u + npts;
  const double* ph = v + npts;
  for (long i = threadIdx.x; i < npts; i += blockDim.x) {
    const double w = (wpt ? wpt[i] : wrow[i / nlon]) * R * R;
    const double Phi = phi0 + ph[i];
    e += w * (0.5 * Phi * (u[i] * u[i] + v[i] * v[i]) + 0.5 * Phi * Phi);
  }
  e = block_sum(e, sh);
  double p[3] = {0.0, 0.0, 0.0};
  for (int f = 0; f < 3; ++f) {
    const double2* a = state + ((long)b * 3 + f) * n2;
    for (long i = threadIdx.x; i < n2; i += blockDim.x) {
      const int l = (int)(i / (L + 1)), m = (int)(i % (L + 1));
      if (m > l) continue;
      const double2 c = a[i];
      p[f] += m == 0 ? c.x * c.x : 2.0 * (c.x * c.x + c.y * c.y);
    }
    p[f] = block_sum(p[f], sh);
  }
  if (threadIdx.x == 0) {
    double* o = out + 5 * (long)b;
    o[0] = R * R * (kFourPi * phi0 + kSqrt4Pi * state[(long)b * 3 * n2 + 2 * n2].x);
    o[1] = e;
    o[2] = sqrt(R * R * p[0]);
    o[3] = sqrt(R * R * p[1]);
    o[4] = sqrt(R * R * p[2]);
  }
}

}  // namespace

size_t op_bytes(const aeolus_plan_impl* p, int op, int batch) {
  switch (op) {
    case AEOLUS_OP_SYNTHESIZE:
    case AEOLUS_OP_ANALYZE:
      return transform_bytes(p, op, batch);
    case AEOLUS_OP_JACOBIAN:
    case AEOLUS_OP_BVE_TENDENCY:
      return full_chain_bytes<4, 1>(p, batch);
    case AEOLUS_OP_WINDS:
      return synth_chain_bytes<2, 2>(p, batch);
    case AEOLUS_OP_SWE_TENDENCY:
      return full_chain_bytes<9, 4>(p, batch) + align256(state_bytes(p, 2, batch));
    case AEOLUS_OP_BVE_RK4:
      return full_chain_bytes<4, 1>(p, batch) + 2 * align256(state_bytes(p, 1, batch));
    case AEOLUS_OP_SWE_RK4:
      return full_chain_bytes<9, 4>(p, batch) + 3 * align256(state_bytes(p, 3, batch)) +
             align256(state_bytes(p, 2, batch));
    case AEOLUS_OP_SWE_VALIDATE:
      return synth_chain_bytes<1, 1>(p, batch) + align256((size_t)batch * p->npoints * 8) +
             align256((size_t)batch * sizeof(double2));
    case AEOLUS_OP_SWE_INVARIANTS:
      return synth_chain_bytes<3, 3>(p, batch) + align256((size_t)batch * 3 * p->npoints * 8);
    default:
      return adjoint_op_bytes(p, op, batch);
  }
}

}  // namespace aeolus

using namespace aeolus;

extern "C" int aeolus_workspace_bytes(aeolus_plan plan, int op, int batch, size_t* bytes) {
  if (!plan_ok(plan) || !bytes) return fail(AEOLUS_ERR_ARG, "aeolus_workspace_bytes: bad arguments");
  if (op < 0 || op > AEOLUS_OP_VECTOR_CURL_DIV) return fail(AEOLUS_ERR_ARG, "aeolus_workspace_bytes: unknown op");
  if (batch < 0) return fail(AEOLUS_ERR_ARG, "aeolus_workspace_bytes: negative batch");
  *bytes = std::max<size_t>(op_bytes(plan, op, std::max(batch, 1)), 256);
  return AEOLUS_OK;
}

#define NEED_WORK(op, who)                                                              \
  do {                                                                                  \
    const size_t _need = op_bytes(plan, op, batch);                                     \
    if (!work || work_bytes < _need)                                                    \
      return fail(AEOLUS_ERR_WORKSPACE, std::string(who) + ": workspace too small (" + \
                                            std::to_string(_need) + " bytes needed)");  \
  } while (0)

extern "C" int aeolus_jacobian(aeolus_plan plan, const double* a, const double* b, double* out, int batch,
                               void* work, size_t work_bytes, void* stream) {
  int s = check_common(plan, "aeolus_jacobian", batch, a, b);
  if (s || batch == 0) return s;
  if (!out) return fail(AEOLUS_ERR_ARG, "aeolus_jacobian: NULL output");
  NEED_WORK(AEOLUS_OP_JACOBIAN, "aeolus_jacobian");
  const Spec sp = make_spec(plan, plan->radius);
  JacDerive d{sp, reinterpret_cast<const double2*>(a), reinterpret_cast<const double2*>(b)};
  TruncEpi e{reinterpret_cast<double2*>(out), plan->lmax};
  return run_full_chain(plan, d, JacPw{}, e, batch, work, nullptr, static_cast<cudaStream_t>(stream));
}

extern "C" int aeolus_winds(aeolus_plan plan, double radius, const double* psi, const double* chi, double* uv,
                            int batch, void* work, size_t work_bytes, void* stream) {
  int s = check_common(plan, "aeolus_winds", batch, psi, uv);
  if (s || batch == 0) return s;
  if (!(radius > 0.0)) return fail(AEOLUS_ERR_ARG, "aeolus_winds: radius must be > 0");
  NEED_WORK(AEOLUS_OP_WINDS, "aeolus_winds");
  const Spec sp = make_spec(plan, radius);
  WindDerive d{sp, reinterpret_cast<const double2*>(psi), reinterpret_cast<const double2*>(chi)};
  WindPw pw{chi == nullptr ? 1 : 0};
  const long np = plan->npoints;
  return run_synth_chain(plan, d, pw, batch, uv, np, np * batch, work, nullptr, static_cast<cudaStream_t>(stream));
}


extern "C" int aeolus_bve_tendency(aeolus_plan plan, const aeolus_bve_params* p, const double* zeta,
                                   const double* forcing, double* tend, int batch, void* work, size_t work_bytes,
                                   void* stream) {
  int s = check_common(plan, "aeolus_bve_tendency", batch, zeta, tend);
  if (s || (s = bve_check(plan, p, "aeolus_bve_tendency")) || batch == 0) return s;
  NEED_WORK(AEOLUS_OP_BVE_TENDENCY, "aeolus_bve_tendency");
  const Spec sp = make_spec(plan, p->radius);
  const double f10 = 2.0 * p->omega * kSqrt4PiOver3;
  BveDerive d{sp, reinterpret_cast<const double2*>(zeta), f10};
  Rk4 rk{0, 0.0, nullptr, nullptr, nullptr, reinterpret_cast<double2*>(tend)};
  BveEpi e{sp, reinterpret_cast<const double2*>(zeta), reinterpret_cast<const double2*>(forcing), p->viscosity, rk};
  return run_full_chain(plan, d, JacPw{}, e, batch, work, nullptr, static_cast<cudaStream_t>(stream));
}

extern "C" int aeolus_swe_tendency(aeolus_plan plan, const aeolus_swe_params* p, const double* state, double* tend,
                                   int batch, void* work, size_t work_bytes, void* stream) {
  int s = check_common(plan, "aeolus_swe_tendency", batch, state, tend);
  if (s || (s = swe_check(p, "aeolus_swe_tendency")) || batch == 0) return s;
  NEED_WORK(AEOLUS_OP_SWE_TENDENCY, "aeolus_swe_tendency");
  const Spec sp = make_spec(plan, p->radius);
  const double f10 = 2.0 * p->omega * kSqrt4PiOver3;
  const double phi0 = p->gravity * p->mean_depth;
  const bool spec_cor = plan->precision == AEOLUS_PREC_SPLIT_BF16;
  const double fp = spec_cor ? 0.0 : f10;
  // split path: the Coriolis spectra are tabulated by the derive stage after the chain scratch
  double2* cor = spec_cor ? reinterpret_cast<double2*>(static_cast<char*>(work) + full_chain_bytes<9, 4>(plan, batch))
                          : nullptr;
  SweDerive d{sp, reinterpret_cast<const double2*>(state), fp, cor, 2.0 * p->omega};
  SwePw pw{fp, phi0, (float)phi0};
  Rk4 rk{0, 0.0, nullptr, nullptr, nullptr, reinterpret_cast<double2*>(tend)};
  SweEpi e{sp, reinterpret_cast<const double2*>(state), phi0, p->nu4, rk, spec_cor ? 2.0 * p->omega : 0.0, cor};
  e.forcing = reinterpret_cast<const double2*>(p->forcing);
  // split path: 7 contracted fields, the two longitude derivatives formed in the synthesis epilogue
  if (spec_cor) return run_full_chain(plan, SweDerive7{d}, pw, e, batch, work, nullptr, static_cast<cudaStream_t>(stream));
  return run_full_chain(plan, d, pw, e, batch, work, nullptr, static_cast<cudaStream_t>(stream));
}

extern "C" int aeolus_bve_rk4(aeolus_plan plan, const aeolus_bve_params* p, double* zeta, int batch, double dt,
                              int nsteps, void* work, size_t work_bytes, void* stream) {
  int s = check_common(plan, "aeolus_bve_rk4", batch, zeta, zeta);
  if (s || (s = bve_check(plan, p, "aeolus_bve_rk4")) || batch == 0 || nsteps <= 0) return s;
  if (!std::isfinite(dt)) return fail(AEOLUS_ERR_ARG, "aeolus_bve_rk4: dt must be finite");
  NEED_WORK(AEOLUS_OP_BVE_RK4, "aeolus_bve_rk4");
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Spec sp = make_spec(plan, p->radius);
  const double f10 = 2.0 * p->omega * kSqrt4PiOver3;
  char* w = static_cast<char*>(work);
  void* chain = w;
  w += full_chain_bytes<4, 1>(plan, batch);
  double2* ystage = reinterpret_cast<double2*>(w);
  w += align256(state_bytes(plan, 1, batch));
  double2* acc = reinterpret_cast<double2*>(w);
  double2* y0 = reinterpret_cast<double2*>(zeta);
  for (int it = 0; it < nsteps; ++it)
    for (int stage = 1; stage <= 4; ++stage) {
      const double2* in = stage == 1 ? y0 : ystage;
      BveDerive d{sp, in, f10};
      Rk4 rk{stage, dt, y0, ystage, acc, nullptr};
      BveEpi e{sp, in, nullptr, p->viscosity, rk};
      if ((s = run_full_chain(plan, d, JacPw{}, e, batch, chain, nullptr, st))) return s;
    }
  return AEOLUS_OK;
}

extern "C" int aeolus_swe_rk4(aeolus_plan plan, const aeolus_swe_params* p, double* state, int batch, double dt,
                              int nsteps, unsigned* status, void* work, size_t work_bytes, void* stream) {
  int s = check_common(plan, "aeolus_swe_rk4", batch, state, state);
  if (s || (s = swe_check(p, "aeolus_swe_rk4")) || batch == 0 || nsteps <= 0) return s;
  if (!std::isfinite(dt)) return fail(AEOLUS_ERR_ARG, "aeolus_swe_rk4: dt must be finite");
  NEED_WORK(AEOLUS_OP_SWE_RK4, "aeolus_swe_rk4");
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Spec sp = make_spec(plan, p->radius);
  const double f10 = 2.0 * p->omega * kSqrt4PiOver3;
  const double phi0 = p->gravity * p->mean_depth;
  char* w = static_cast<char*>(work);
  void* chain = w;
  w += full_chain_bytes<9, 4>(plan, batch);
  // Two stage buffers in turn: the epilogue of a stage reads neighbouring
  // degrees of its input (spectral Coriolis terms) while writing the next
  // stage's input, so the two must not alias.
  double2* stage_buf[2];
  stage_buf[0] = reinterpret_cast<double2*>(w);
  w += align256(state_bytes(plan, 3, batch));
  stage_buf[1] = reinterpret_cast<double2*>(w);
  w += align256(state_bytes(plan, 3, batch));
  double2* acc = reinterpret_cast<double2*>(w);
  w += align256(state_bytes(plan, 3, batch));
  double2* y0 = reinterpret_cast<double2*>(state);
  const bool spec_cor = plan->precision == AEOLUS_PREC_SPLIT_BF16;
  double2* cor = spec_cor ? reinterpret_cast<double2*>(w) : nullptr;  // Coriolis spectra of the stage input
  const double fp = spec_cor ? 0.0 : f10;
  SwePw pw{fp, phi0, (float)phi0};
  for (int it = 0; it < nsteps; ++it)
    for (int stage = 1; stage <= 4; ++stage) {
      const double2* in = stage == 1 ? y0 : stage_buf[stage & 1];        // 2 -> buf0, 3 -> buf1, 4 -> buf0
      double2* next = stage_buf[(stage + 1) & 1];                        // 1 -> buf0, 2 -> buf1, 3 -> buf0
      SweDerive d{sp, in, fp, cor, 2.0 * p->omega};
      Rk4 rk{stage, dt, y0, next, acc, nullptr};
      SweEpi e{sp, in, phi0, p->nu4, rk, spec_cor ? 2.0 * p->omega : 0.0, cor};
      e.forcing = reinterpret_cast<const double2*>(p->forcing);
      s = spec_cor ? run_full_chain(plan, SweDerive7{d}, pw, e, batch, chain, status, st)
                   : run_full_chain(plan, d, pw, e, batch, chain, status, st);
      if (s) return s;
    }
  return AEOLUS_OK;
}

extern "C" int aeolus_swe_validate(aeolus_plan state_plan, aeolus_plan product_plan, const aeolus_swe_params* p,
                                   const double* state, unsigned* status, double* extrema, int batch, void* work,
                                   size_t work_bytes, void* stream) {
  aeolus_plan plan = state_plan;
  int s = check_common(plan, "aeolus_swe_validate", batch, state, state);
  if (s || (s = swe_check(p, "aeolus_swe_validate")) || batch == 0) return s;
  if (product_plan == state_plan) product_plan = nullptr;
  if (product_plan && product_plan->lmax != plan->lmax)
    return fail(AEOLUS_ERR_ARG, "aeolus_swe_validate: product plan truncation differs");
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  size_t need = op_bytes(plan, AEOLUS_OP_SWE_VALIDATE, batch);
  if (product_plan) need = std::max(need, op_bytes(product_plan, AEOLUS_OP_SWE_VALIDATE, batch));
  if (!work || work_bytes < need) return fail(AEOLUS_ERR_WORKSPACE, "aeolus_swe_validate: workspace too small");
  const double2* st2 = reinterpret_cast<const double2*>(state);
  if (status) {
    swe_spectral_check_kernel<<<batch, 256, 0, st>>>(plan->lmax, st2, status);
    AE_LAUNCH("swe_spectral_check_kernel");
  }
  aeolus_plan plans[2] = {plan, product_plan};
  for (int i = 0; i < 2; ++i) {
    aeolus_plan q = plans[i];
    if (!q) continue;
    char* w = static_cast<char*>(work);
    void* chain = w;
    w += synth_chain_bytes<1, 1>(q, batch);
    double* g = reinterpret_cast<double*>(w);
    w += align256((size_t)batch * q->npoints * 8);
    double2* mm = reinterpret_cast<double2*>(static_cast<char*>(work) + need - align256((size_t)batch * sizeof(double2)));
    FieldDerive d{st2, q->lmax, 3, 2};
    if ((s = run_synth_chain(q, d, PwCopy{}, batch, g, q->npoints, q->npoints, chain, nullptr, st))) return s;
    minmax_kernel<<<batch, 256, 0, st>>>(q->npoints, g, mm, i);
    AE_LAUNCH("minmax_kernel");
    if (i == 1 || !product_plan) {
      thickness_kernel<<<(batch + 127) / 128, 128, 0, st>>>(batch, p->gravity * p->mean_depth, mm, status, extrema);
      AE_LAUNCH("thickness_kernel");
    }
  }
  return AEOLUS_OK;
}

extern "C" int aeolus_bve_spectral_diagnostics(int lmax, double radius, double omega, const double* zeta, double* out,
                                               int batch, void* stream) {
  if (lmax < 0 || batch < 0 || !(radius > 0.0)) return fail(AEOLUS_ERR_ARG, "aeolus_bve_spectral_diagnostics: bad arguments");
  if (batch == 0) return AEOLUS_OK;
  if (!zeta || !out) return fail(AEOLUS_ERR_ARG, "aeolus_bve_spectral_diagnostics: NULL array");
  bve_diag_kernel<<<batch, 256, 0, static_cast<cudaStream_t>(stream)>>>(lmax, radius, omega,
                                                                       reinterpret_cast<const double2*>(zeta), out);
  AE_LAUNCH("bve_diag_kernel");
  return AEOLUS_OK;
}

extern "C" int aeolus_swe_invariants(aeolus_plan plan, const aeolus_swe_params* p, const double* state, double* out,
                                     int batch, void* work, size_t work_bytes, void* stream) {
  int s = check_common(plan, "aeolus_swe_invariants", batch, state, out);
  if (s || (s = swe_check(p, "aeolus_swe_invariants")) || batch == 0) return s;
  NEED_WORK(AEOLUS_OP_SWE_INVARIANTS, "aeolus_swe_invariants");
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* w = static_cast<char*>(work);
  void* chain = w;
  w += synth_chain_bytes<3, 3>(plan, batch);
  double* uvp = reinterpret_cast<double*>(w);
  const Spec sp = make_spec(plan, p->radius);
  WindPhiDerive d{sp, reinterpret_cast<const double2*>(state)};
  const long np = plan->npoints;
  if ((s = run_synth_chain(plan, d, WindPhiPw{}, batch, uvp, 3 * np, np, chain, nullptr, st))) return s;
  swe_invariants_kernel<<<batch, 256, 0, st>>>(plan->lmax, np, plan->nlon, p->radius, p->gravity * p->mean_depth,
                                               reinterpret_cast<const double2*>(state), uvp,
                                               plan->kind == kGauss ? plan->wq : nullptr,
                                               plan->kind == kPoints ? plan->wpts : nullptr, out);
  AE_LAUNCH("swe_invariants_kernel");
  return AEOLUS_OK;
}
