// Adjoints (vector-Jacobian products) of the transforms, of the BVE and SWE
// tendencies and of one RK4 step.
//
// Inner products: a spectral array is the real vector of the (Re, Im) parts
// of its m <= l slots; a grid array is the plain real vector of its values.
// With a_lm = sum_j wq_j P_lm(x_j) F_m(f_j) (analysis, F_m the longitude
// DFT) and f = sum_l P_l0 Re a_l0 + 2 Re sum_{m>0} a_lm P_lm e^{i m lon}
// (synthesis, which drops Im a_l0):
//   S^T g = s_m sum_j P_lm(x_j) F_m(g_j)            s_0 = 1 (Im := 0), s_m = 2
//         = s_m A(g / wq)                            (unit-weight analysis)
//   A^T a = wq_j S(h_m a)                            h_0 = 1, h_m = 1/2
// A tendency chain  y -> D y -> S -> P(.) -> A -> E  therefore has the VJP
//   ybar = E_lin^T kbar + D^T s_m A( P'(S D y)^T S(h_m C kbar) )
// which is again one Derive -> synthesis -> pointwise -> analysis chain: the
// derive stage emits the forward fields D y next to the adjoint fields
// h_m C kbar, the pointwise stage applies the transposed Jacobian of the
// grid-point products (the quadrature weights of A^T and S^T cancel into the
// analysis weights), and a spectral kernel applies D^T and the linear terms.
// The adjoint always linearises the FP64-form products (planetary vorticity
// inside eta), on either contraction precision.
#include <cmath>

#include "models.cuh"

namespace aeolus {
namespace {

// kbar = alpha a + beta b (b may be NULL)
struct AdjSrc {
  const double2* a;
  double alpha;
  const double2* b;
  double beta;
  __device__ double2 at(long i) const {
    double2 v = cscale(alpha, a[i]);
    if (b) v = cadd(v, cscale(beta, b[i]));
    return v;
  }
};

// Analysed adjoint fields times s_m, stored dense [b][NF][L+1][L+1].
template <int NFIELDS>
struct EpiStoreAdj {
  static constexpr int NF = NFIELDS;
  double2* out;
  int L;
  __device__ void finish_field(int b, int f, int l, int m, double2 a) const {
    const double2 v = m == 0 ? make_double2(a.x, 0.0) : make_double2(2.0 * a.x, 2.0 * a.y);
    out[(((long)b * NF + f) * (L + 1) + l) * (L + 1) + m] = v;
  }
  __device__ void finish(int b, int l, int m, const double2* acc) const {
#pragma unroll
    for (int f = 0; f < NF; ++f) finish_field(b, f, l, m, acc[f]);
  }
  __device__ void zero(int b, int l, int m) const {
#pragma unroll
    for (int f = 0; f < NF; ++f) out[(((long)b * NF + f) * (L + 1) + l) * (L + 1) + m] = make_double2(0.0, 0.0);
  }
};

// Synthesis input h_m a (the A^T input side).
struct DeriveHalf {
  static constexpr int NF = 1;
  const double2* in;
  int L;
  __device__ void column(int b, int l, int m, double2* v) const {
    v[0] = cscale(m == 0 ? 1.0 : 0.5, in[((long)b * (L + 1) + l) * (L + 1) + m]);
  }
};

__global__ void scale_points_kernel(double* g, long npts, int batch, const double* __restrict__ wrow,
                                    const double* __restrict__ wpt, int nlon) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= npts * batch) return;
  const long p = idx % npts;
  g[idx] *= wpt ? wpt[p] : wrow[p / nlon];
}

// --------------------------------------------------------------- SWE
// Forward fields (SweDerive, 9) followed by h_m C kbar of the four analysed
// product fields: q0 <- kb0, q1 <- kb1, q2 <- -lap kb1, q3 <- kb2
// (physics/shallow_water.py:388-417 with the l = 0 pin and the 2/3 cut).
struct SweAdjDerive {
  static constexpr int NF = 13;
  SweDerive fwd;
  AdjSrc kb;
  __device__ void column(int b, int l, int m, double2* v) const {
    fwd.column(b, l, m, v);
    const int L = fwd.s.L, cut = (2 * L) / 3;
    const long n2 = (long)(L + 1) * (L + 1);
    const long i = (long)b * 3 * n2 + (long)l * (L + 1) + m;
    const bool keep = l > 0 && l <= cut && m <= cut;
    const double2 z0 = make_double2(0.0, 0.0);
    const double h = m == 0 ? 1.0 : 0.5;
    const double2 k0 = keep ? kb.at(i) : z0, k1 = keep ? kb.at(i + n2) : z0, k2 = keep ? kb.at(i + 2 * n2) : z0;
    v[9] = cscale(h, k0);
    v[10] = cscale(h, k1);
    v[11] = cscale(-h * fwd.s.lap(l), k1);
    v[12] = cscale(h, k2);
  }
};

// Transposed Jacobian of the SwePw products at the forward grid values.
// in: U, V, eta_lam, eta_snt, phi_lam, phi_snt, zeta, delta, phi, q0..q3;
// out: the adjoints of the nine synthesised fields.
struct SweAdjPw {
  static constexpr int NIN = 13, NOUT = 9;
  static constexpr bool kIdentity = false;
  double f10;
  __device__ unsigned operator()(double c, double fg, const double* in, double* out) const {
    const double ic = 1.0 / c;
    const double u = in[0] * ic, v = in[1] * ic;
    const double eta_lam = in[2], eta_snt = in[3], phi_lam = in[4], phi_snt = in[5];
    const double zeta = in[6], delta = in[7], phi = in[8];
    const double eta = zeta + f10 * fg;
    const double q0 = in[9], q1 = in[10], q2 = in[11], q3 = in[12];
    const double ub = (-q0 * eta_lam + q1 * eta_snt - q3 * phi_lam) * ic + q2 * u;
    const double vb = (q0 * eta_snt + q1 * eta_lam + q3 * phi_snt) * ic + q2 * v;
    out[0] = ub * ic;
    out[1] = vb * ic;
    out[2] = (-q0 * u + q1 * v) * ic;
    out[3] = (q0 * v + q1 * u) * ic;
    out[4] = -q3 * u * ic;
    out[5] = q3 * v * ic;
    out[6] = -q0 * delta + q1 * (eta + zeta);
    out[7] = -q0 * eta - q3 * phi;
    out[8] = -q3 * delta;
    return 0u;
  }
  __device__ RowDf df_row(double c, double fg) const {
    return RowDf{df_from_double(1.0 / c), df_from_double(f10 * fg), (float)c};
  }
  __device__ unsigned df_op(const RowDf& r, const df* in, df* out) const {
    const df u = df_mul(in[0], r.invc), v = df_mul(in[1], r.invc);
    const df eta_lam = in[2], eta_snt = in[3], phi_lam = in[4], phi_snt = in[5];
    const df zeta = in[6], delta = in[7], phi = in[8];
    const df eta = df_add(zeta, r.fj);
    const df q0 = in[9], q1 = in[10], q2 = in[11], q3 = in[12];
    const df ub = df_add(df_mul(df_add(df_sub(df_mul(q1, eta_snt), df_mul(q0, eta_lam)), df_neg(df_mul(q3, phi_lam))),
                                r.invc),
                         df_mul(q2, u));
    const df vb = df_add(df_mul(df_add(df_add(df_mul(q0, eta_snt), df_mul(q1, eta_lam)), df_mul(q3, phi_snt)), r.invc),
                         df_mul(q2, v));
    out[0] = df_mul(ub, r.invc);
    out[1] = df_mul(vb, r.invc);
    out[2] = df_mul(df_sub(df_mul(q1, v), df_mul(q0, u)), r.invc);
    out[3] = df_mul(df_add(df_mul(q0, v), df_mul(q1, u)), r.invc);
    out[4] = df_neg(df_mul(df_mul(q3, u), r.invc));
    out[5] = df_mul(df_mul(q3, v), r.invc);
    out[6] = df_sub(df_mul(q1, df_add(eta, zeta)), df_mul(q0, delta));
    out[7] = df_neg(df_add(df_mul(q0, eta), df_mul(q3, phi)));
    out[8] = df_neg(df_mul(q3, delta));
    return 0u;
  }
};

// ybar = E_lin^T kbar + D^T vbar (vbar = the nine analysed adjoint fields
// times s_m), one thread per (b, l, m).  g = that VJP; writes g_out = g
// (optional) and acc_out = acc_in + g (acc_in optional).
__global__ void swe_adjoint_finish_kernel(Spec s, double phi0, double nu4, const double2* __restrict__ vbar,
                                          AdjSrc kb, double2* g_out, const double2* acc_in, double2* acc_out,
                                          int batch) {
  const int L = s.L;
  const long n2 = (long)(L + 1) * (L + 1);
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2 * batch) return;
  const int b = (int)(idx / n2);
  const int r = (int)(idx - (long)b * n2);
  const int l = r / (L + 1), m = r - l * (L + 1);
  const long i0 = (long)b * 3 * n2 + r;
  const double2 z0 = make_double2(0.0, 0.0);
  double2 g0 = z0, g1 = z0, g2 = z0;
  if (m <= l) {
    const double2* vb = vbar + (long)b * 9 * n2;
    auto V = [&](int f, int ll) -> double2 { return (ll < 0 || ll > L) ? z0 : vb[f * n2 + (long)ll * (L + 1) + m]; };
    const double ir = s.ir;
    // U = snt(psi)/R + dlam(chi), V = dlam(psi) - snt(chi)/R
    const double2 psib = csub(cscale(ir, s.snt_t(V(0, l - 1), V(0, l + 1), l, m)), s.dlam(V(1, l), m));
    const double2 chib = csub(make_double2(0.0, 0.0),
                              cadd(s.dlam(V(0, l), m), cscale(ir, s.snt_t(V(1, l - 1), V(1, l + 1), l, m))));
    // psi = invlap0(zeta), chi = invlap0(delta) (diagonal, symmetric)
    const double il = l == 0 ? 0.0 : (s.invlap ? s.invlap[l] : 1.0 / s.lap(l));
    g0 = cadd(cadd(cscale(il, psib), csub(cscale(ir, s.snt_t(V(3, l - 1), V(3, l + 1), l, m)), s.dlam(V(2, l), m))),
              V(6, l));
    g1 = cadd(cscale(il, chib), V(7, l));
    g2 = cadd(csub(cscale(ir, s.snt_t(V(5, l - 1), V(5, l + 1), l, m)), s.dlam(V(4, l), m)), V(8, l));
    if (l > 0) {  // linear terms; the l = 0 rows of the tendency are pinned to zero
      const double2 k0 = kb.at(i0), k1 = kb.at(i0 + n2), k2 = kb.at(i0 + 2 * n2);
      const double lap = s.lap(l);
      g1 = csub(g1, cscale(phi0, k2));
      g2 = csub(g2, cscale(lap, k1));
      if (nu4 > 0.0) {
        const double h = nu4 * lap * lap;
        g0 = csub(g0, cscale(h, k0));
        g1 = csub(g1, cscale(h, k1));
        g2 = csub(g2, cscale(h, k2));
      }
    }
  }
  const double2 g[3] = {g0, g1, g2};
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    const long i = i0 + f * n2;
    if (g_out) g_out[i] = g[f];
    acc_out[i] = acc_in ? cadd(acc_in[i], g[f]) : g[f];
  }
}

// --------------------------------------------------------------- BVE
// Forward fields (BveDerive: psi_lam, psi_snt, eta_lam, eta_snt) and
// h_m C (-kbar) of the analysed Jacobian (physics/barotropic.py:150-165).
struct BveAdjDerive {
  static constexpr int NF = 5;
  BveDerive fwd;
  AdjSrc kb;
  __device__ void column(int b, int l, int m, double2* v) const {
    fwd.column(b, l, m, v);
    const int L = fwd.s.L, cut = (2 * L) / 3;
    const long i = ((long)b * (L + 1) + l) * (L + 1) + m;
    const bool keep = l > 0 && l <= cut && m <= cut;
    v[4] = keep ? cscale(m == 0 ? -1.0 : -0.5, kb.at(i)) : make_double2(0.0, 0.0);
  }
};

// J = (in1 in2 - in0 in3) / c^2
struct BveAdjPw {
  static constexpr int NIN = 5, NOUT = 4;
  static constexpr bool kIdentity = false;
  __device__ unsigned operator()(double c, double, const double* in, double* out) const {
    const double q = in[4] / (c * c);
    out[0] = -in[3] * q;
    out[1] = in[2] * q;
    out[2] = in[1] * q;
    out[3] = -in[0] * q;
    return 0u;
  }
  __device__ RowDf df_row(double c, double) const { return RowDf{df_from_double(1.0 / (c * c)), df{0.f, 0.f}, (float)c}; }
  __device__ unsigned df_op(const RowDf& r, const df* in, df* out) const {
    const df q = df_mul(in[4], r.invc);
    out[0] = df_neg(df_mul(in[3], q));
    out[1] = df_mul(in[2], q);
    out[2] = df_mul(in[1], q);
    out[3] = df_neg(df_mul(in[0], q));
    return 0u;
  }
};

__global__ void bve_adjoint_finish_kernel(Spec s, double nu, const double2* __restrict__ vbar, AdjSrc kb,
                                          double2* g_out, const double2* acc_in, double2* acc_out, int batch) {
  const int L = s.L;
  const long n2 = (long)(L + 1) * (L + 1);
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2 * batch) return;
  const int b = (int)(idx / n2);
  const int r = (int)(idx - (long)b * n2);
  const int l = r / (L + 1), m = r - l * (L + 1);
  const double2 z0 = make_double2(0.0, 0.0);
  double2 g = z0;
  if (m <= l) {
    const double2* vb = vbar + (long)b * 4 * n2;
    auto V = [&](int f, int ll) -> double2 { return (ll < 0 || ll > L) ? z0 : vb[f * n2 + (long)ll * (L + 1) + m]; };
    const double ir = s.ir;
    // v0 = dlam(psi), v1 = snt(psi)/R, v2 = dlam(zeta), v3 = snt(zeta + f)/R
    const double2 psib = csub(cscale(ir, s.snt_t(V(1, l - 1), V(1, l + 1), l, m)), s.dlam(V(0, l), m));
    const double il = l == 0 ? 0.0 : (s.invlap ? s.invlap[l] : 1.0 / s.lap(l));
    g = cadd(cscale(il, psib), csub(cscale(ir, s.snt_t(V(3, l - 1), V(3, l + 1), l, m)), s.dlam(V(2, l), m)));
    if (l > 0) g = cadd(g, cscale(nu * s.lap(l), kb.at(idx)));
  }
  if (g_out) g_out[idx] = g;
  acc_out[idx] = acc_in ? cadd(acc_in[idx], g) : g;
}

// ------------------------------------------------------------ helpers
template <int NF>
size_t vbar_bytes(const aeolus_plan_impl* p, int batch) {
  return align256(state_bytes(p, NF, batch));
}

size_t swe_tadj_bytes(const aeolus_plan_impl* p, int batch) {
  return full_chain_bytes<13, 9>(p, batch) + vbar_bytes<9>(p, batch);
}
size_t bve_tadj_bytes(const aeolus_plan_impl* p, int batch) {
  return full_chain_bytes<5, 4>(p, batch) + vbar_bytes<4>(p, batch);
}

// One SWE tendency VJP at `y`: g = (dT/dy)^T kb, g_out / acc as in the finish kernel.
int swe_vjp(const aeolus_plan_impl* plan, const aeolus_swe_params* p, const double2* y, AdjSrc kb, double2* g_out,
            const double2* acc_in, double2* acc_out, int batch, void* work, cudaStream_t st) {
  const Spec sp = make_spec(plan, p->radius);
  const double f10 = 2.0 * p->omega * kSqrt4PiOver3;
  const double phi0 = p->gravity * p->mean_depth;
  char* w = static_cast<char*>(work);
  void* chain = w;
  w += full_chain_bytes<13, 9>(plan, batch);
  double2* vbar = reinterpret_cast<double2*>(w);
  SweAdjDerive d{SweDerive{sp, y, f10}, kb};
  EpiStoreAdj<9> e{vbar, plan->lmax};
  int s = run_full_chain(plan, d, SweAdjPw{f10}, e, batch, chain, nullptr, st);
  if (s) return s;
  const long n = (long)(plan->lmax + 1) * (plan->lmax + 1) * batch;
  {
    ProfScope prof("swe_adjoint_finish", st);
    swe_adjoint_finish_kernel<<<blocks_for(n, 128), 128, 0, st>>>(sp, phi0, p->nu4, vbar, kb, g_out, acc_in, acc_out,
                                                                   batch);
    AE_LAUNCH("swe_adjoint_finish_kernel");
  }
  return AEOLUS_OK;
}

int bve_vjp(const aeolus_plan_impl* plan, const aeolus_bve_params* p, const double2* z, AdjSrc kb, double2* g_out,
            const double2* acc_in, double2* acc_out, int batch, void* work, cudaStream_t st) {
  const Spec sp = make_spec(plan, p->radius);
  const double f10 = 2.0 * p->omega * kSqrt4PiOver3;
  char* w = static_cast<char*>(work);
  void* chain = w;
  w += full_chain_bytes<5, 4>(plan, batch);
  double2* vbar = reinterpret_cast<double2*>(w);
  BveAdjDerive d{BveDerive{sp, z, f10}, kb};
  EpiStoreAdj<4> e{vbar, plan->lmax};
  int s = run_full_chain(plan, d, BveAdjPw{}, e, batch, chain, nullptr, st);
  if (s) return s;
  const long n = (long)(plan->lmax + 1) * (plan->lmax + 1) * batch;
  {
    ProfScope prof("bve_adjoint_finish", st);
    bve_adjoint_finish_kernel<<<blocks_for(n, 128), 128, 0, st>>>(sp, p->viscosity, vbar, kb, g_out, acc_in, acc_out,
                                                                   batch);
    AE_LAUNCH("bve_adjoint_finish_kernel");
  }
  return AEOLUS_OK;
}

}  // namespace

size_t vector_op_bytes(const aeolus_plan_impl* p, int batch);  // vector.cu

size_t adjoint_op_bytes(const aeolus_plan_impl* p, int op, int batch) {
  switch (op) {
    case AEOLUS_OP_SYNTHESIZE_ADJOINT:
      return anal_chain_bytes<1, 1>(p, batch);
    case AEOLUS_OP_ANALYZE_ADJOINT:
      return synth_chain_bytes<1, 1>(p, batch);
    case AEOLUS_OP_BVE_TENDENCY_ADJOINT:
      return bve_tadj_bytes(p, batch);
    case AEOLUS_OP_SWE_TENDENCY_ADJOINT:
      return swe_tadj_bytes(p, batch);
    case AEOLUS_OP_BVE_RK4_ADJOINT:
      return std::max(bve_tadj_bytes(p, batch), full_chain_bytes<4, 1>(p, batch)) +
             7 * align256(state_bytes(p, 1, batch));
    case AEOLUS_OP_SWE_RK4_ADJOINT:
      return std::max(swe_tadj_bytes(p, batch), full_chain_bytes<9, 4>(p, batch)) +
             7 * align256(state_bytes(p, 3, batch)) + align256(state_bytes(p, 2, batch));
    case AEOLUS_OP_VECTOR_CURL_DIV:
      return vector_op_bytes(p, batch);
    default:
      return 0;
  }
}

}  // namespace aeolus

using namespace aeolus;

#define NEED_ADJ_WORK(op, who)                                                          \
  do {                                                                                  \
    const size_t _need = adjoint_op_bytes(plan, op, batch);                             \
    if (!work || work_bytes < _need)                                                    \
      return fail(AEOLUS_ERR_WORKSPACE, std::string(who) + ": workspace too small (" + \
                                            std::to_string(_need) + " bytes needed)");  \
  } while (0)

extern "C" int aeolus_synthesize_adjoint(aeolus_plan plan, const double* grid_bar, double* coeffs_bar, int batch,
                                         void* work, size_t work_bytes, void* stream) {
  int s = check_common(plan, "aeolus_synthesize_adjoint", batch, grid_bar, coeffs_bar);
  if (s || batch == 0) return s;
  NEED_ADJ_WORK(AEOLUS_OP_SYNTHESIZE_ADJOINT, "aeolus_synthesize_adjoint");
  EpiStoreAdj<1> e{reinterpret_cast<double2*>(coeffs_bar), plan->lmax};
  return run_anal_chain(plan, PwCopy{}, e, batch, grid_bar, plan->npoints, plan->npoints, work,
                        static_cast<cudaStream_t>(stream), true);
}

extern "C" int aeolus_analyze_adjoint(aeolus_plan plan, const double* coeffs_bar, double* grid_bar, int batch,
                                      void* work, size_t work_bytes, void* stream) {
  int s = check_common(plan, "aeolus_analyze_adjoint", batch, coeffs_bar, grid_bar);
  if (s || batch == 0) return s;
  NEED_ADJ_WORK(AEOLUS_OP_ANALYZE_ADJOINT, "aeolus_analyze_adjoint");
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  DeriveHalf d{reinterpret_cast<const double2*>(coeffs_bar), plan->lmax};
  if ((s = run_synth_chain(plan, d, PwCopy{}, batch, grid_bar, plan->npoints, plan->npoints, work, nullptr, st)))
    return s;
  const long n = plan->npoints * (long)batch;
  scale_points_kernel<<<blocks_for(n, 256), 256, 0, st>>>(grid_bar, plan->npoints, batch,
                                                          plan->kind == kGauss ? plan->wq : nullptr,
                                                          plan->kind == kGauss ? nullptr : plan->wpts, plan->nlon);
  AE_LAUNCH("scale_points_kernel");
  return AEOLUS_OK;
}

extern "C" int aeolus_swe_tendency_adjoint(aeolus_plan plan, const aeolus_swe_params* p, const double* state,
                                           const double* tend_bar, double* state_bar, int batch, void* work,
                                           size_t work_bytes, void* stream) {
  int s = check_common(plan, "aeolus_swe_tendency_adjoint", batch, state, tend_bar);
  if (s || (s = swe_check(p, "aeolus_swe_tendency_adjoint")) || batch == 0) return s;
  if (!state_bar) return fail(AEOLUS_ERR_ARG, "aeolus_swe_tendency_adjoint: NULL output");
  if (state_bar == tend_bar) return fail(AEOLUS_ERR_ARG, "aeolus_swe_tendency_adjoint: output aliases tend_bar");
  NEED_ADJ_WORK(AEOLUS_OP_SWE_TENDENCY_ADJOINT, "aeolus_swe_tendency_adjoint");
  AdjSrc kb{reinterpret_cast<const double2*>(tend_bar), 1.0, nullptr, 0.0};
  return swe_vjp(plan, p, reinterpret_cast<const double2*>(state), kb, nullptr, nullptr,
                 reinterpret_cast<double2*>(state_bar), batch, work, static_cast<cudaStream_t>(stream));
}

extern "C" int aeolus_bve_tendency_adjoint(aeolus_plan plan, const aeolus_bve_params* p, const double* zeta,
                                           const double* tend_bar, double* zeta_bar, int batch, void* work,
                                           size_t work_bytes, void* stream) {
  int s = check_common(plan, "aeolus_bve_tendency_adjoint", batch, zeta, tend_bar);
  if (s || (s = bve_check(plan, p, "aeolus_bve_tendency_adjoint")) || batch == 0) return s;
  if (!zeta_bar) return fail(AEOLUS_ERR_ARG, "aeolus_bve_tendency_adjoint: NULL output");
  if (zeta_bar == tend_bar) return fail(AEOLUS_ERR_ARG, "aeolus_bve_tendency_adjoint: output aliases tend_bar");
  NEED_ADJ_WORK(AEOLUS_OP_BVE_TENDENCY_ADJOINT, "aeolus_bve_tendency_adjoint");
  AdjSrc kb{reinterpret_cast<const double2*>(tend_bar), 1.0, nullptr, 0.0};
  return bve_vjp(plan, p, reinterpret_cast<const double2*>(zeta), kb, nullptr, nullptr,
                 reinterpret_cast<double2*>(zeta_bar), batch, work, static_cast<cudaStream_t>(stream));
}

// RK4 step adjoint (run/engine.py:406-431 differentiated): with stage inputs
// y1 = y + dt/2 k1, y2 = y + dt/2 k2, y3 = y + dt k3 recomputed by the forward
// chains and ybar' the adjoint of the step's output,
//   g4 = T'(y3)^T (dt/6 ybar')
//   g3 = T'(y2)^T (dt/3 ybar' + dt g4)
//   g2 = T'(y1)^T (dt/3 ybar' + dt/2 g3)
//   g1 = T'(y)^T  (dt/6 ybar' + dt/2 g2)
//   ybar = ybar' + g1 + g2 + g3 + g4.
extern "C" int aeolus_swe_rk4_adjoint(aeolus_plan plan, const aeolus_swe_params* p, const double* state,
                                      double* state_bar, int batch, double dt, void* work, size_t work_bytes,
                                      void* stream) {
  int s = check_common(plan, "aeolus_swe_rk4_adjoint", batch, state, state_bar);
  if (s || (s = swe_check(p, "aeolus_swe_rk4_adjoint")) || batch == 0) return s;
  if (!std::isfinite(dt)) return fail(AEOLUS_ERR_ARG, "aeolus_swe_rk4_adjoint: dt must be finite");
  if (state == state_bar) return fail(AEOLUS_ERR_ARG, "aeolus_swe_rk4_adjoint: state aliases state_bar");
  NEED_ADJ_WORK(AEOLUS_OP_SWE_RK4_ADJOINT, "aeolus_swe_rk4_adjoint");
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Spec sp = make_spec(plan, p->radius);
  const double f10 = 2.0 * p->omega * kSqrt4PiOver3;
  const double phi0 = p->gravity * p->mean_depth;
  char* w = static_cast<char*>(work);
  void* chain = w;
  w += std::max(swe_tadj_bytes(plan, batch), full_chain_bytes<9, 4>(plan, batch));
  const size_t sb = align256(state_bytes(plan, 3, batch));
  double2* buf[7];
  for (int i = 0; i < 7; ++i) buf[i] = reinterpret_cast<double2*>(w + i * sb);
  double2 *y1 = buf[0], *y2 = buf[1], *y3 = buf[2], *kacc = buf[3], *ga = buf[4], *gb = buf[5], *acc = buf[6];
  double2* y0 = const_cast<double2*>(reinterpret_cast<const double2*>(state));  // stages 1-3 never write y0
  double2* yb = reinterpret_cast<double2*>(state_bar);
  // forward stage inputs, with the same functors (and precision form) as aeolus_swe_rk4
  const bool spec_cor = plan->precision == AEOLUS_PREC_SPLIT_BF16;
  double2* cor = spec_cor ? reinterpret_cast<double2*>(w + 7 * sb) : nullptr;
  const double fp = spec_cor ? 0.0 : f10;
  SwePw pw{fp, phi0, (float)phi0};
  double2* next[3] = {y1, y2, y3};
  const double2* in = y0;
  for (int stage = 1; stage <= 3; ++stage) {
    SweDerive d{sp, in, fp, cor, 2.0 * p->omega};
    Rk4 rk{stage, dt, y0, next[stage - 1], kacc, nullptr};
    SweEpi e{sp, in, phi0, p->nu4, rk, spec_cor ? 2.0 * p->omega : 0.0, cor};
    e.forcing = reinterpret_cast<const double2*>(p->forcing);
    if ((s = run_full_chain(plan, d, pw, e, batch, chain, nullptr, st))) return s;
    in = next[stage - 1];
  }
  if ((s = swe_vjp(plan, p, y3, AdjSrc{yb, dt / 6.0, nullptr, 0.0}, ga, yb, acc, batch, chain, st))) return s;
  if ((s = swe_vjp(plan, p, y2, AdjSrc{yb, dt / 3.0, ga, dt}, gb, acc, acc, batch, chain, st))) return s;
  if ((s = swe_vjp(plan, p, y1, AdjSrc{yb, dt / 3.0, gb, dt / 2.0}, ga, acc, acc, batch, chain, st))) return s;
  return swe_vjp(plan, p, y0, AdjSrc{yb, dt / 6.0, ga, dt / 2.0}, nullptr, acc, yb, batch, chain, st);
}

extern "C" int aeolus_bve_rk4_adjoint(aeolus_plan plan, const aeolus_bve_params* p, const double* zeta,
                                      double* zeta_bar, int batch, double dt, void* work, size_t work_bytes,
                                      void* stream) {
  int s = check_common(plan, "aeolus_bve_rk4_adjoint", batch, zeta, zeta_bar);
  if (s || (s = bve_check(plan, p, "aeolus_bve_rk4_adjoint")) || batch == 0) return s;
  if (!std::isfinite(dt)) return fail(AEOLUS_ERR_ARG, "aeolus_bve_rk4_adjoint: dt must be finite");
  if (zeta == zeta_bar) return fail(AEOLUS_ERR_ARG, "aeolus_bve_rk4_adjoint: zeta aliases zeta_bar");
  NEED_ADJ_WORK(AEOLUS_OP_BVE_RK4_ADJOINT, "aeolus_bve_rk4_adjoint");
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Spec sp = make_spec(plan, p->radius);
  const double f10 = 2.0 * p->omega * kSqrt4PiOver3;
  char* w = static_cast<char*>(work);
  void* chain = w;
  w += std::max(bve_tadj_bytes(plan, batch), full_chain_bytes<4, 1>(plan, batch));
  const size_t sb = align256(state_bytes(plan, 1, batch));
  double2* buf[7];
  for (int i = 0; i < 7; ++i) buf[i] = reinterpret_cast<double2*>(w + i * sb);
  double2 *y1 = buf[0], *y2 = buf[1], *y3 = buf[2], *kacc = buf[3], *ga = buf[4], *gb = buf[5], *acc = buf[6];
  double2* y0 = const_cast<double2*>(reinterpret_cast<const double2*>(zeta));
  double2* yb = reinterpret_cast<double2*>(zeta_bar);
  double2* next[3] = {y1, y2, y3};
  const double2* in = y0;
  for (int stage = 1; stage <= 3; ++stage) {
    BveDerive d{sp, in, f10};
    Rk4 rk{stage, dt, y0, next[stage - 1], kacc, nullptr};
    BveEpi e{sp, in, nullptr, p->viscosity, rk};
    if ((s = run_full_chain(plan, d, JacPw{}, e, batch, chain, nullptr, st))) return s;
    in = next[stage - 1];
  }
  if ((s = bve_vjp(plan, p, y3, AdjSrc{yb, dt / 6.0, nullptr, 0.0}, ga, yb, acc, batch, chain, st))) return s;
  if ((s = bve_vjp(plan, p, y2, AdjSrc{yb, dt / 3.0, ga, dt}, gb, acc, acc, batch, chain, st))) return s;
  if ((s = bve_vjp(plan, p, y1, AdjSrc{yb, dt / 3.0, gb, dt / 2.0}, ga, acc, acc, batch, chain, st))) return s;
  return bve_vjp(plan, p, y0, AdjSrc{yb, dt / 6.0, ga, dt / 2.0}, nullptr, acc, yb, batch, chain, st);
}
