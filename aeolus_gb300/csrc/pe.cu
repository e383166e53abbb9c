// Dry hydrostatic primitive-equation tendency in sigma coordinates,
// src/planetary_sandbox/physics/primitive_equations.py:482-753 with the
// column operators of physics/sigma_coordinate.py:164-398, batched over
// levels and members on the library's transforms:
//
//   aeolus_pe_derive    spectral: per level u cos, v cos (from the inverse
//                       Laplacians of zeta, delta), zeta, delta, T, dT/dlambda,
//                       sin(theta) dT/dtheta / R, the same two of eta = zeta + f,
//                       eta; per member the two derivatives of ln p_s
//   (synthesis of all 10 K + 2 fields on the product plan)
//   aeolus_pe_columns   pointwise, one thread per product point and member,
//                       the whole column in registers: G = delta + V.grad ln p_s,
//                       d ln p_s/dt, interface sigma_dot, omega/p, centred
//                       vertical advection of u, v, T; the thermodynamic
//                       integrand, -div(eta V), curl(eta V), kinetic energy, and
//                       the residual vector Z = sigma_dot dV/dsigma + R_d T grad ln p_s
//   (analysis of the 4 K + 1 integrands; weak-form curl/div of Z on the
//   one-degree-extended plan)
//   aeolus_pe_spectral  spectral: 2/3 cuts, Simmons-Burridge geopotential of
//                       the spectral T, -lap(KE + Phi), l = 0 rows of the
//                       momentum tendencies pinned.
#include "models.cuh"

namespace aeolus {
namespace {

constexpr int kPeMaxLevels = 64;
constexpr int kPeLevelFields = 10;  // U, V, zeta, delta, T, T_lam, T_snt, eta_lam, eta_snt, eta
constexpr int kPeOutFields = 4;     // thermodynamic integrand, -div(eta V), curl(eta V), KE

// Lorenz sigma grid, sigma_coordinate.py:43-149: interfaces s[0] = 0 (top)
// .. s[K] = 1 (surface), thickness, interface log ratios beta (beta[0], the
// infinite top entry, is never read) and the Simmons-Burridge alpha.
// The column kernel multiplies by host-computed reciprocals instead of
// dividing (FP64 divides would dominate its FP64 pipe): h2[k] = 1/(2 Dsigma_k)
// and bd[k] = beta_k / Dsigma_k, within an ulp of the reference's quotients.
struct PeSigma {
  int K;
  double s[kPeMaxLevels + 1], dsig[kPeMaxLevels], beta[kPeMaxLevels], alpha[kPeMaxLevels];
  double h2[kPeMaxLevels], bd[kPeMaxLevels];
};

int make_sigma(const double* interfaces, int nlev, PeSigma* g) {
  if (nlev < 1 || nlev > kPeMaxLevels)
    return fail(AEOLUS_ERR_ARG, "nlev must be in [1, " + std::to_string(kPeMaxLevels) + "], got " +
                                    std::to_string(nlev));
  if (!interfaces) return fail(AEOLUS_ERR_ARG, "NULL sigma interfaces");
  if (interfaces[0] != 0.0 || interfaces[nlev] != 1.0)
    return fail(AEOLUS_ERR_ARG, "sigma interfaces must start at exactly 0.0 and end at exactly 1.0");
  g->K = nlev;
  for (int k = 0; k <= nlev; ++k) {
    if (!std::isfinite(interfaces[k]) || (k > 0 && !(interfaces[k] > interfaces[k - 1])))
      return fail(AEOLUS_ERR_ARG, "sigma interfaces must be finite and strictly increasing");
    g->s[k] = interfaces[k];
  }
  for (int k = 0; k < nlev; ++k) {
    g->dsig[k] = g->s[k + 1] - g->s[k];
    g->h2[k] = 1.0 / (2.0 * g->dsig[k]);
  }
  g->beta[0] = 0.0;
  g->bd[0] = 0.0;
  g->alpha[0] = std::log(2.0);
  for (int k = 1; k < nlev; ++k) {
    g->beta[k] = std::log(g->s[k + 1] / g->s[k]);
    g->alpha[k] = 1.0 - (g->s[k] / g->dsig[k]) * g->beta[k];
    g->bd[k] = g->beta[k] / g->dsig[k];
  }
  return AEOLUS_OK;
}

int pe_check(const aeolus_pe_params* prm) {
  if (!prm) return fail(AEOLUS_ERR_ARG, "NULL primitive-equation parameters");
  if (!(std::isfinite(prm->radius) && prm->radius > 0) || !std::isfinite(prm->omega))
    return fail(AEOLUS_ERR_ARG, "primitive equations: bad radius/omega");
  if (!(std::isfinite(prm->r_dry) && prm->r_dry > 0))
    return fail(AEOLUS_ERR_ARG, "r_dry must be finite and > 0, got " + std::to_string(prm->r_dry));
  if (!(std::isfinite(prm->cp_dry) && prm->cp_dry > prm->r_dry))
    return fail(AEOLUS_ERR_ARG, "cp_dry must be finite and > r_dry, got " + std::to_string(prm->cp_dry));
  return AEOLUS_OK;
}

// One thread per (member, l, m): every level's derived spectra.
__global__ void pe_derive_kernel(Spec s, int K, int batch, double f10, const double2* __restrict__ st,
                                 double2* __restrict__ out) {
  const int L = s.L;
  const long n2 = (long)(L + 1) * (L + 1);
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2 * batch) return;
  const int b = (int)(idx / n2);
  const long r = idx - b * n2;
  const int l = (int)(r / (L + 1)), m = (int)(r - (long)l * (L + 1));
  const double2* S = st + (long)b * (3 * K + 1) * n2;
  double2* O = out + (long)b * (kPeLevelFields * K + 2) * n2 + r;
  const double2 zero = make_double2(0.0, 0.0);
  if (m > l) {
    for (int f = 0; f < kPeLevelFields * K + 2; ++f) O[f * n2] = zero;
    return;
  }
  const bool lo = l >= 1 && l - 1 >= m, hi = l + 1 <= L;
  auto val = [&](const double2* a, int ll) { return a[(long)ll * (L + 1) + m]; };
  auto inv = [&](const double2* a, int ll) { return s.invlap0(a, ll, m); };
  auto snt_r = [&](double2 vlo, double2 vhi) { return cscale(s.ir, s.snt(vlo, vhi, l, m)); };
  for (int k = 0; k < K; ++k) {
    const double2* z = S + (long)k * n2;
    const double2* d = S + (long)(K + k) * n2;
    const double2* T = S + (long)(2 * K + k) * n2;
    const double2 psi = inv(z, l), chi = inv(d, l);
    const double2 psi_lo = lo ? inv(z, l - 1) : zero, psi_hi = hi ? inv(z, l + 1) : zero;
    const double2 chi_lo = lo ? inv(d, l - 1) : zero, chi_hi = hi ? inv(d, l + 1) : zero;
    double2 e = val(z, l), e_lo = lo ? val(z, l - 1) : zero, e_hi = hi ? val(z, l + 1) : zero;
    if (m == 0) {  // eta = zeta + f, f = 2 Omega sin(lat): the (1, 0) mode
      if (l == 1) e.x += f10;
      if (l - 1 == 1) e_lo.x += f10;
      if (l + 1 == 1) e_hi.x += f10;
    }
    const double2 Tl = val(T, l);
    double2* o = O + (long)kPeLevelFields * k * n2;
    o[0 * n2] = cadd(snt_r(psi_lo, psi_hi), s.dlam(chi, m));   // u cos
    o[1 * n2] = csub(s.dlam(psi, m), snt_r(chi_lo, chi_hi));   // v cos
    o[2 * n2] = val(z, l);
    o[3 * n2] = val(d, l);
    o[4 * n2] = Tl;
    o[5 * n2] = s.dlam(Tl, m);
    o[6 * n2] = snt_r(lo ? val(T, l - 1) : zero, hi ? val(T, l + 1) : zero);
    o[7 * n2] = s.dlam(e, m);
    o[8 * n2] = snt_r(e_lo, e_hi);
    o[9 * n2] = e;
  }
  const double2* q = S + (long)3 * K * n2;
  O[(long)kPeLevelFields * K * n2] = s.dlam(val(q, l), m);
  O[((long)kPeLevelFields * K + 1) * n2] = snt_r(lo ? val(q, l - 1) : zero, hi ? val(q, l + 1) : zero);
}

// The same spectra for split-precision plans (their synthesis digits carry
// 48 bits) in packed double-float (lanes re, im): the coefficient products
// of the double-float derive table at the plan radius (Spec::dcoef_df: the
// same combinations of C+-, 1/lap and m/R as the SWE derive), the state
// converted by integer operations on its bits, each derived spectrum
// rounded to FP64 by one FP64 addition per word; zeta, delta, T and eta are
// copied in FP64 as they are.
__global__ void __launch_bounds__(128) pe_derive_df_kernel(Spec s, int K, int batch, double f10,
                                                           const double2* __restrict__ st, double2* __restrict__ out) {
  // one thread per (member, level, l, m); "level" K is the pair of ln p_s
  // spectra (the levels are independent, so the loads of all of them fly
  // at once instead of one level after another)
  const int L = s.L;
  const long n2 = (long)(L + 1) * (L + 1);
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2 * (K + 1) * batch) return;
  const long r = idx % n2;
  const int k = (int)((idx / n2) % (K + 1)), b = (int)(idx / (n2 * (K + 1)));
  const int l = (int)(r / (L + 1)), m = (int)(r - (long)l * (L + 1));
  const double2* S = st + (long)b * (3 * K + 1) * n2;
  double2* O = out + (long)b * (kPeLevelFields * K + 2) * n2 + r;
  const int nout = k < K ? kPeLevelFields : 2;
  double2* o = O + (long)kPeLevelFields * k * n2;  // level k's fields, or the two ln p_s ones at k = K
  if (m > l) {
    const double2 zero = make_double2(0.0, 0.0);
    for (int f = 0; f < nout; ++f) o[f * n2] = zero;
    return;
  }
  const bool lo = l >= 1 && l - 1 >= m, hi = l + 1 <= L;
  const float2* c = s.dcoef_df + r * 8;
  auto kc = [&](int i) { return df2_splat(df{c[i].x, c[i].y}); };
  const df2 zero = df2{0ull, 0ull};
  auto cv = [&](const double2* a, int ll) { return df2_of_f64x2(a[(long)ll * (L + 1) + m]); };
  auto cvlo = [&](const double2* a) { return lo ? cv(a, l - 1) : zero; };
  auto cvhi = [&](const double2* a) { return hi ? cv(a, l + 1) : zero; };
  const df2 B1 = kc(3), B2 = kc(4), B3 = kc(5);
  if (k == K) {
    const double2* q = S + (long)3 * K * n2;
    o[0] = f64x2_of_df2(df2_mul(B3, df2_times_i(cv(q, l))));
    o[n2] = f64x2_of_df2(df2_add_fast(df2_mul(B1, cvlo(q)), df2_mul(B2, cvhi(q))));
    return;
  }
  const df2 A1 = kc(0), A2 = kc(1), A3 = kc(2);
  // eta = zeta + f at the (1, 0) mode, in the neighbour slots
  auto add_f = [&](df2 v, bool at) {
    if (!at) return v;
    df re, im;
    df2_unpack(v, re, im);
    return df2_pack(df_add(re, df_of_f64(f10)), im);
  };
  const double2* z = S + (long)k * n2;
  const double2* d = S + (long)(K + k) * n2;
  const double2* T = S + (long)(2 * K + k) * n2;
  const double2 z64 = z[r], d64 = d[r], T64 = T[r];
  const df2 zl = df2_of_f64x2(z64), dl = df2_of_f64x2(d64), Tl = df2_of_f64x2(T64);
  const df2 z_lo = cvlo(z), z_hi = cvhi(z), d_lo = cvlo(d), d_hi = cvhi(d);
  o[0 * n2] = f64x2_of_df2(df2_add_fast(df2_add_fast(df2_mul(A1, z_lo), df2_mul(A2, z_hi)),
                                        df2_mul(A3, df2_times_i(dl))));    // u cos
  o[1 * n2] = f64x2_of_df2(df2_sub_fast(df2_mul(A3, df2_times_i(zl)),
                                        df2_add_fast(df2_mul(A1, d_lo), df2_mul(A2, d_hi))));  // v cos
  o[2 * n2] = z64;
  o[3 * n2] = d64;
  o[4 * n2] = T64;
  o[5 * n2] = f64x2_of_df2(df2_mul(B3, df2_times_i(Tl)));
  o[6 * n2] = f64x2_of_df2(df2_add_fast(df2_mul(B1, cvlo(T)), df2_mul(B2, cvhi(T))));
  o[7 * n2] = f64x2_of_df2(df2_mul(B3, df2_times_i(zl)));  // m = 0 (the only f slot) has B3 = 0
  o[8 * n2] = f64x2_of_df2(df2_add_fast(df2_mul(B1, add_f(z_lo, m == 0 && l == 2)),
                                        df2_mul(B2, add_f(z_hi, m == 0 && l == 0))));
  o[9 * n2] = (m == 0 && l == 1) ? make_double2(z64.x + f10, z64.y) : z64;
}

// One thread per (member, product point): the column in thread-local
// arrays.  The kernel is FP64-bound (84 % FP64-pipe active at 192x384,
// 20 levels); the arrays spill through L1 to L2, which doubles its DRAM
// traffic but not its time: a shared-memory column (occupancy-capped) and a
// two-pass form without arrays (recomputing the FP64 terms) both ran slower.
__global__ void __launch_bounds__(128) pe_columns_kernel(PeSigma sg, long np, int nlon, const double* __restrict__ coslat,
                                                         int batch, double r_dry, double kappa,
                                                         const double* __restrict__ grid, double* __restrict__ prod,
                                                         double* __restrict__ fen) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= np * batch) return;
  const int K = sg.K;
  const int b = (int)(idx / np);
  const long p = idx - b * np;
  const double ic = 1.0 / coslat[nlon > 0 ? p / nlon : p];
  const double* Gd = grid + (long)b * (kPeLevelFields * K + 2) * np + p;
  double* P = prod + (long)b * (kPeOutFields * K + 1) * np + p;
  const double lp_lam = Gd[(long)kPeLevelFields * K * np], lp_snt = Gd[((long)kPeLevelFields * K + 1) * np];
  double u[kPeMaxLevels], v[kPeMaxLevels], T[kPeMaxLevels], G[kPeMaxLevels], A[kPeMaxLevels];
  double part[kPeMaxLevels], sd[kPeMaxLevels + 1];
  double acc = 0.0, total = 0.0;
  for (int k = 0; k < K; ++k) {
    const double* f = Gd + (long)kPeLevelFields * k * np;
    u[k] = f[0] * ic;
    v[k] = f[np] * ic;
    T[k] = f[4 * np];
    A[k] = (u[k] * lp_lam - v[k] * lp_snt) * ic;      // V . grad(ln p_s)
    G[k] = f[3 * np] + A[k];                          // delta + A
    const double w = sg.dsig[k] * G[k];
    acc = k == 0 ? w : acc + w;                       // cumulative thickness-weighted G
    part[k] = acc;
  }
  total = part[K - 1];
  // interface sigma_dot: exact zeros at the top and (total - total) at the surface
  sd[0] = 0.0;
  for (int k = 1; k < K; ++k) sd[k] = sg.s[k] * total - part[k - 1];
  sd[K] = total - total;
  P[(long)kPeOutFields * K * np] = -total;            // d ln p_s / dt
  const double gu = lp_lam * ic, gv = -lp_snt * ic;   // grad(ln p_s)
  auto vadv = [&](const double* X, int k) {
    double a = 0.0;
    bool any = false;
    if (k < K - 1) {
      a = sd[k + 1] * (X[k + 1] - X[k]);
      any = true;
    }
    if (k > 0) {
      const double up = sd[k] * (X[k] - X[k - 1]);
      a = any ? a + up : up;
      any = true;
    }
    return any ? a * sg.h2[k] : 0.0;
  };
  for (int k = 0; k < K; ++k) {
    const double* f = Gd + (long)kPeLevelFields * k * np;
    const double wp = k == 0 ? A[0] - sg.alpha[0] * G[0]
                             : A[k] - sg.bd[k] * part[k - 1] - sg.alpha[k] * G[k];
    const double t_lam = f[5 * np], t_snt = f[6 * np];
    const double e_lam = f[7 * np], e_snt = f[8 * np], eta = f[9 * np];
    const double adv_t = (u[k] * t_lam - v[k] * t_snt) * ic;
    double* o = P + (long)kPeOutFields * k * np;
    o[0] = -adv_t - vadv(T, k) + kappa * T[k] * wp;
    o[np] = -((u[k] * e_lam - v[k] * e_snt) * ic + eta * f[3 * np]);
    o[2 * np] = eta * f[2 * np] + (v[k] * e_lam + u[k] * e_snt) * ic;
    o[3 * np] = 0.5 * (u[k] * u[k] + v[k] * v[k]);
    const double rt = r_dry * T[k];
    double* z = fen + ((long)b * K + k) * 2 * np + p;
    z[0] = vadv(u, k) + rt * gu;
    z[np] = vadv(v, k) + rt * gv;
  }
}

// ---------------------------------------------------------------------------
// The same column in double-float arithmetic, for split-precision plans (the
// rest of their tendency is computed to ~48 bits already): the FP64 grid
// values become double-floats through integer operations on their bits
// (df_of_f64) and the results FP64 with one FP64 addition each (f64_of_df),
// the only FP64 instructions of the kernel (GB300's FP64 pipe is ~1/64 of
// its f32 pipe).  Values below 2^-126 in magnitude are taken as 0, values
// beyond the float range as infinite.
struct PeSigmaDf {
  int K;
  df s[kPeMaxLevels + 1], dsig[kPeMaxLevels], alpha[kPeMaxLevels], h2[kPeMaxLevels], bd[kPeMaxLevels];
};

inline df host_df(double x) {
  const float h = static_cast<float>(x);
  return df{h, static_cast<float>(x - static_cast<double>(h))};
}

PeSigmaDf sigma_df(const PeSigma& g) {
  PeSigmaDf d;
  d.K = g.K;
  for (int k = 0; k <= g.K; ++k) d.s[k] = host_df(g.s[k]);
  for (int k = 0; k < g.K; ++k) {
    d.dsig[k] = host_df(g.dsig[k]);
    d.alpha[k] = host_df(g.alpha[k]);
    d.h2[k] = host_df(g.h2[k]);
    d.bd[k] = host_df(g.bd[k]);
  }
  return d;
}

// 1 / c as a double-float: f32 reciprocal refined by one double-float Newton step.
__device__ __forceinline__ df df_recip(df c) {
  const float r0 = 1.0f / c.hi;
  const df e = df_sub(df{1.0f, 0.0f}, df_mul(c, df{r0, 0.0f}));  // 1 - c r0
  return df_add(df{r0, 0.0f}, df_mul(df{r0, 0.0f}, e));
}

// Two passes over the levels and no per-level arrays (in double-float the
// recomputation is cheap, while thread-local column arrays would make the
// kernel wait on local memory): pass 1 forms the cumulative thickness-weighted
// G for the surface value; pass 2 repeats the same running sum for the
// interface sigma_dot and keeps a three-level window of u, v, T for the
// vertical advection (the same operations in the same order as one pass
// with arrays).
__global__ void __launch_bounds__(128) pe_columns_df_kernel(PeSigmaDf sg, long np, int nlon,
                                                            const double* __restrict__ coslat, int batch, df r_dry,
                                                            df kappa, const double* __restrict__ grid,
                                                            double* __restrict__ prod, double* __restrict__ fen) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= np * batch) return;
  const int K = sg.K;
  const int b = (int)(idx / np);
  const long p = idx - b * np;
  const df ic = df_recip(df_of_f64(coslat[nlon > 0 ? p / nlon : p]));
  const double* Gd = grid + (long)b * (kPeLevelFields * K + 2) * np + p;
  double* P = prod + (long)b * (kPeOutFields * K + 1) * np + p;
  const df lp_lam = df_of_f64(Gd[(long)kPeLevelFields * K * np]), lp_snt = df_of_f64(Gd[((long)kPeLevelFields * K + 1) * np]);
  auto lev = [&](int k) { return Gd + (long)kPeLevelFields * k * np; };
  auto AG = [&](int k, df uk, df vk, df& A, df& G) {
    A = df_mul(df_sub(df_mul(uk, lp_lam), df_mul(vk, lp_snt)), ic);  // V . grad(ln p_s)
    G = df_add(df_of_f64(lev(k)[3 * np]), A);                        // delta + A
  };
  // pass 1: the cumulative thickness-weighted G
  df acc = df{0.f, 0.f};
  for (int k = 0; k < K; ++k) {
    const double* f = lev(k);
    df A, G;
    AG(k, df_mul(df_of_f64(f[0]), ic), df_mul(df_of_f64(f[np]), ic), A, G);
    const df w = df_mul(sg.dsig[k], G);
    acc = k == 0 ? w : df_add(acc, w);
  }
  const df total = acc;
  P[(long)kPeOutFields * K * np] = f64_of_df(df_neg(total));  // d ln p_s / dt
  const df gu = df_mul(lp_lam, ic), gv = df_neg(df_mul(lp_snt, ic));
  const df zero = df{0.f, 0.f};
  // vertical advection of X at level k from (X[k-1], X[k], X[k+1]) with the
  // interface sigma_dot above (sdk) and below (sdk1) the level
  auto vadv = [&](df xm, df x0, df xp, int k, df sdk, df sdk1) {
    df a = zero;
    bool any = false;
    if (k < K - 1) {
      a = df_mul(sdk1, df_sub(xp, x0));
      any = true;
    }
    if (k > 0) {
      const df up = df_mul(sdk, df_sub(x0, xm));
      a = any ? df_add(a, up) : up;
      any = true;
    }
    return any ? df_mul(a, sg.h2[k]) : zero;
  };
  // pass 2
  df um = zero, vm = zero, Tm = zero;
  df u0 = df_mul(df_of_f64(lev(0)[0]), ic), v0 = df_mul(df_of_f64(lev(0)[np]), ic), T0 = df_of_f64(lev(0)[4 * np]);
  df run = zero, part_prev = zero;
  for (int k = 0; k < K; ++k) {
    const double* f = lev(k);
    df up = zero, vp = zero, Tp = zero;
    if (k + 1 < K) {
      const double* g = lev(k + 1);
      up = df_mul(df_of_f64(g[0]), ic);
      vp = df_mul(df_of_f64(g[np]), ic);
      Tp = df_of_f64(g[4 * np]);
    }
    df A, G;
    AG(k, u0, v0, A, G);
    const df w = df_mul(sg.dsig[k], G);
    run = k == 0 ? w : df_add(run, w);
    // interface sigma_dot: exact zeros at the top and (total - total) at the surface
    const df sdk = k == 0 ? zero : df_sub(df_mul(sg.s[k], total), part_prev);
    const df sdk1 = k + 1 == K ? zero : df_sub(df_mul(sg.s[k + 1], total), run);
    const df wp = k == 0 ? df_sub(A, df_mul(sg.alpha[0], G))
                         : df_sub(df_sub(A, df_mul(sg.bd[k], part_prev)), df_mul(sg.alpha[k], G));
    const df t_lam = df_of_f64(f[5 * np]), t_snt = df_of_f64(f[6 * np]);
    const df e_lam = df_of_f64(f[7 * np]), e_snt = df_of_f64(f[8 * np]), eta = df_of_f64(f[9 * np]);
    const df adv_t = df_mul(df_sub(df_mul(u0, t_lam), df_mul(v0, t_snt)), ic);
    double* o = P + (long)kPeOutFields * k * np;
    o[0] = f64_of_df(df_add(df_sub(df_neg(adv_t), vadv(Tm, T0, Tp, k, sdk, sdk1)), df_mul(df_mul(kappa, T0), wp)));
    o[np] = f64_of_df(df_neg(df_add(df_mul(df_sub(df_mul(u0, e_lam), df_mul(v0, e_snt)), ic),
                                    df_mul(eta, df_of_f64(f[3 * np])))));
    o[2 * np] = f64_of_df(df_add(df_mul(eta, df_of_f64(f[2 * np])),
                                 df_mul(df_add(df_mul(v0, e_lam), df_mul(u0, e_snt)), ic)));
    o[3 * np] = f64_of_df(df_scale2(df_add(df_mul(u0, u0), df_mul(v0, v0)), 0.5f));
    const df rt = df_mul(r_dry, T0);
    double* z = fen + ((long)b * K + k) * 2 * np + p;
    z[0] = f64_of_df(df_add(vadv(um, u0, up, k, sdk, sdk1), df_mul(rt, gu)));
    z[np] = f64_of_df(df_add(vadv(vm, v0, vp, k, sdk, sdk1), df_mul(rt, gv)));
    part_prev = run;
    um = u0;
    vm = v0;
    Tm = T0;
    u0 = up;
    v0 = vp;
    T0 = Tp;
  }
}

// One thread per (member, l, m): every level's tendencies.
__global__ void pe_spectral_kernel(PeSigma sg, int L, double R, double r_dry, int batch,
                                   const double2* __restrict__ st, const double2* __restrict__ an,
                                   const double2* __restrict__ cz, const double2* __restrict__ dz,
                                   const double2* __restrict__ phis, double2* __restrict__ out) {
  const int K = sg.K;
  const long n2 = (long)(L + 1) * (L + 1);
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2 * batch) return;
  const int b = (int)(idx / n2);
  const long r = idx - b * n2;
  const int l = (int)(r / (L + 1)), m = (int)(r - (long)l * (L + 1));
  double2* O = out + (long)b * (3 * K + 1) * n2 + r;
  const double2 zero = make_double2(0.0, 0.0);
  if (m > l) {
    for (int f = 0; f < 3 * K + 1; ++f) O[f * n2] = zero;
    return;
  }
  const int cut = (2 * L) / 3;
  const bool keep = l <= cut && m <= cut;
  const double lap = -(double)l * (l + 1.0) / (R * R);
  const double2* A = an + (long)b * (kPeOutFields * K + 1) * n2 + r;
  const double2* T = st + (long)b * (3 * K + 1) * n2 + (long)2 * K * n2 + r;
  // Simmons-Burridge on the spectral T, upward from Phi_s at the surface
  double2 below = phis[r];
  for (int k = K - 1; k >= 0; --k) {
    const double2 Tk = T[(long)k * n2];
    const double2 phi = cadd(below, cscale(r_dry * sg.alpha[k], Tk));
    if (k > 0) below = cadd(below, cscale(r_dry * sg.beta[k], Tk));
    const double2* a = A + (long)kPeOutFields * k * n2;
    const long zk = ((long)b * K + k) * n2 + r;
    const double2 ke = keep ? a[3 * n2] : zero;
    O[(long)(2 * K + k) * n2] = keep ? a[0] : zero;
    O[(long)k * n2] = (l == 0 || !keep) ? zero : csub(a[n2], cz[zk]);
    const double2 dd = keep ? csub(a[2 * n2], dz[zk]) : zero;
    O[(long)(K + k) * n2] = l == 0 ? zero : csub(dd, cscale(lap, cadd(ke, phi)));
  }
  O[(long)3 * K * n2] = keep ? A[(long)kPeOutFields * K * n2] : zero;
}

// One classical RK4 stage update over n complex values, in the reference's
// order of operations (run/engine.py:406-431), with every FP64 product and
// sum rounded separately (no contraction into FMAs), as NumPy/torch do:
//   stage 1: acc = k;           ys = y0 + (dt/2) k
//   stage 2: acc = acc + 2 k;   ys = y0 + (dt/2) k
//   stage 3: acc = acc + 2 k;   ys = y0 + dt k
//   stage 4: out = y0 + (dt/6) (acc + k)
__global__ void rk4_stage_kernel(int stage, double dt, const double2* __restrict__ y0, const double2* __restrict__ k,
                                 double2* __restrict__ ys, double2* __restrict__ acc, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 kk = k[i], y = y0[i];
  if (stage == 4) {
    const double2 a = acc[i];
    const double c = dt / 6.0;
    const double sx = __dadd_rn(a.x, kk.x), sy = __dadd_rn(a.y, kk.y);
    ys[i] = make_double2(__dadd_rn(y.x, __dmul_rn(c, sx)), __dadd_rn(y.y, __dmul_rn(c, sy)));
    return;
  }
  if (stage == 1) {
    acc[i] = kk;
  } else {
    const double2 a = acc[i];
    acc[i] = make_double2(__dadd_rn(a.x, __dmul_rn(2.0, kk.x)), __dadd_rn(a.y, __dmul_rn(2.0, kk.y)));
  }
  const double c = stage == 3 ? dt : 0.5 * dt;
  ys[i] = make_double2(__dadd_rn(y.x, __dmul_rn(c, kk.x)), __dadd_rn(y.y, __dmul_rn(c, kk.y)));
}

}  // namespace
}  // namespace aeolus

using namespace aeolus;

extern "C" int aeolus_rk4_stage(int stage, double dt, const double* y0, const double* k, double* ystage, double* acc,
                                long n, void* stream) {
  if (stage < 1 || stage > 4 || n < 0 || !std::isfinite(dt))
    return fail(AEOLUS_ERR_ARG, "aeolus_rk4_stage: stage must be 1..4, n >= 0, dt finite");
  if (n == 0) return AEOLUS_OK;
  if (!y0 || !k || !ystage || !acc) return fail(AEOLUS_ERR_ARG, "aeolus_rk4_stage: NULL array");
  if (acc == ystage || acc == k) return fail(AEOLUS_ERR_ARG, "aeolus_rk4_stage: acc must not alias ystage or k");
  ProfScope prof("rk4_stage", static_cast<cudaStream_t>(stream));
  rk4_stage_kernel<<<blocks_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      stage, dt, reinterpret_cast<const double2*>(y0), reinterpret_cast<const double2*>(k),
      reinterpret_cast<double2*>(ystage), reinterpret_cast<double2*>(acc), n);
  AE_LAUNCH("rk4_stage_kernel");
  return AEOLUS_OK;
}

extern "C" int aeolus_pe_derive(aeolus_plan plan, const aeolus_pe_params* prm, int nlev, const double* state,
                                double* fields, int batch, void* stream) {
  if (int s = check_common(plan, "aeolus_pe_derive", batch, state, fields)) return s;
  if (int s = pe_check(prm)) return s;
  if (nlev < 1 || nlev > kPeMaxLevels) return fail(AEOLUS_ERR_ARG, "aeolus_pe_derive: bad nlev");
  if (batch == 0) return AEOLUS_OK;
  const long n2 = (long)(plan->lmax + 1) * (plan->lmax + 1);
  ProfScope prof("pe_derive", static_cast<cudaStream_t>(stream));
  const Spec sp = make_spec(plan, prm->radius);
  if (plan->precision == AEOLUS_PREC_SPLIT_BF16 && sp.dcoef_df) {
    pe_derive_df_kernel<<<blocks_for(n2 * (nlev + 1) * batch, 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        sp, nlev, batch, 2.0 * prm->omega * kSqrt4PiOver3, reinterpret_cast<const double2*>(state),
        reinterpret_cast<double2*>(fields));
    AE_LAUNCH("pe_derive_df_kernel");
    return AEOLUS_OK;
  }
  pe_derive_kernel<<<blocks_for(n2 * batch, 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
      sp, nlev, batch, 2.0 * prm->omega * kSqrt4PiOver3, reinterpret_cast<const double2*>(state),
      reinterpret_cast<double2*>(fields));
  AE_LAUNCH("pe_derive_kernel");
  return AEOLUS_OK;
}

extern "C" int aeolus_pe_columns(aeolus_plan plan, const aeolus_pe_params* prm, int nlev, const double* interfaces,
                                 const double* grid, double* prod, double* f_en, int batch, void* stream) {
  if (int s = check_common(plan, "aeolus_pe_columns", batch, grid, prod)) return s;
  if (int s = pe_check(prm)) return s;
  PeSigma sg;
  if (int s = make_sigma(interfaces, nlev, &sg)) return s;
  if (batch > 0 && !f_en) return fail(AEOLUS_ERR_ARG, "aeolus_pe_columns: NULL f_en");
  if (batch == 0) return AEOLUS_OK;
  const long np = plan->npoints;
  const int nlon = plan->kind == kGauss ? plan->nlon : 0;
  ProfScope prof("pe_columns", static_cast<cudaStream_t>(stream));
  if (plan->precision == AEOLUS_PREC_SPLIT_BF16) {  // split plans: the double-float column
    pe_columns_df_kernel<<<blocks_for(np * batch, 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        sigma_df(sg), np, nlon, plan->coslat, batch, host_df(prm->r_dry), host_df(prm->r_dry / prm->cp_dry), grid,
        prod, f_en);
    AE_LAUNCH("pe_columns_df_kernel");
    return AEOLUS_OK;
  }
  pe_columns_kernel<<<blocks_for(np * batch, 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
      sg, np, nlon, plan->coslat, batch, prm->r_dry, prm->r_dry / prm->cp_dry, grid, prod, f_en);
  AE_LAUNCH("pe_columns_kernel");
  return AEOLUS_OK;
}

extern "C" int aeolus_pe_spectral(int lmax, const aeolus_pe_params* prm, int nlev, const double* interfaces,
                                  const double* state, const double* analysed, const double* curl_z,
                                  const double* div_z, const double* phi_s, double* tendency, int batch,
                                  void* stream) {
  if (lmax < 0 || batch < 0) return fail(AEOLUS_ERR_ARG, "aeolus_pe_spectral: bad lmax/batch");
  if (int s = pe_check(prm)) return s;
  PeSigma sg;
  if (int s = make_sigma(interfaces, nlev, &sg)) return s;
  if (batch == 0) return AEOLUS_OK;
  if (!state || !analysed || !curl_z || !div_z || !phi_s || !tendency)
    return fail(AEOLUS_ERR_ARG, "aeolus_pe_spectral: NULL array");
  const long n2 = (long)(lmax + 1) * (lmax + 1);
  ProfScope prof("pe_spectral", static_cast<cudaStream_t>(stream));
  pe_spectral_kernel<<<blocks_for(n2 * batch, 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
      sg, lmax, prm->radius, prm->r_dry, batch, reinterpret_cast<const double2*>(state),
      reinterpret_cast<const double2*>(analysed), reinterpret_cast<const double2*>(curl_z),
      reinterpret_cast<const double2*>(div_z), reinterpret_cast<const double2*>(phi_s),
      reinterpret_cast<double2*>(tendency));
  AE_LAUNCH("pe_spectral_kernel");
  return AEOLUS_OK;
}
