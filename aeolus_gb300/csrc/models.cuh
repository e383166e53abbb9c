// Physics functors shared by the forward model chains (models.cu) and their
// adjoints (adjoint.cu): the spectral context, the BVE and SWE derive /
// pointwise / epilogue functors, RK4 stage bookkeeping and argument checks.
// Everything sits in an unnamed namespace: each translation unit that
// includes this header gets its own copy.
#pragma once

#include <cmath>
#include <string>

#include "chains.cuh"

namespace aeolus {
namespace {

constexpr double kSqrt4PiOver3 = 2.04665341589297697695;  // sqrt(4 pi / 3)
constexpr double kSqrt4Pi = 3.54490770181103205460;       // sqrt(4 pi)
constexpr double kFourPi = 12.56637061435917295384;

struct Spec {  // shared spectral context
  int L;
  double R;
  double ir, ir2;        // 1 / R, 1 / R^2 (no FP64 divides on the device)
  const double* cplus;   // [(L+1)^2], C+[L][:] = 0
  const double* cminus;  // [(L+1)^2]
  const double* invlap;  // [L+1] 1 / lap(l), 0 at l = 0
  const double* xa;      // [(L+1)^2] x-multiplication coefficients (see xmul)
  const double* xb;
  const double* dcoef;   // [(L+1)^2][8] combined SWE derive coefficients (plan radius only)
  const float2* dcoef_df;  // the same as double-floats (hi, lo), or none
  __device__ double lap(int l) const { return -(double)l * (l + 1.0) * ir2; }
  __device__ double2 at(const double2* a, int l, int m) const { return a[(long)l * (L + 1) + m]; }
  // Helmholtz inverse with l = 0 -> 0 (physics/barotropic.py:91); a
  // multiplication by the tabulated reciprocal (within 1 ulp of the divide).
  __device__ double2 invlap0(const double2* a, int l, int m) const {
    const double2 v = at(a, l, m);
    if (!invlap) {
      if (l == 0) return make_double2(0.0, 0.0);
      const double d = lap(l);
      return make_double2(v.x / d, v.y / d);
    }
    const double r = invlap[l];
    return make_double2(v.x * r, v.y * r);
  }
  // (i m / R) v
  __device__ double2 dlam(double2 v, int m) const {
    const double mr = (double)m * ir;
    return make_double2(-mr * v.y, mr * v.x);
  }
  // (x q)_lm, x = cos(colatitude) = sin(latitude):
  //   x Y_lm = a_lm Y_{l+1,m} + b_lm Y_{l-1,m},
  //   a_lm = sqrt(((l+1)^2 - m^2)/((2l+1)(2l+3))), b_lm = sqrt((l^2 - m^2)/((2l-1)(2l+1)))
  // (C+_lm = l a_lm and C-_lm = -(l+1) b_lm of the sin(theta) d/dtheta coupling).
  __device__ double2 xmul(double2 lo, double2 hi, int l, int m) const {
    // a_{l-1,m} = C+_{l-1,m} / (l-1) (a_00 = 1/sqrt(3)),  b_{l+1,m} = -C-_{l+1,m} / (l+2), tabulated
    double2 g = make_double2(0.0, 0.0);
    if (l >= 1 && l - 1 >= m) g = cadd(g, cscale(xa[(long)(l - 1) * (L + 1) + m], lo));
    if (l + 1 <= L) g = cadd(g, cscale(xb[(long)(l + 1) * (L + 1) + m], hi));
    return g;
  }
  // sin(theta) d/dtheta coupling of a column given its values at l-1, l+1
  __device__ double2 snt(double2 lo, double2 hi, int l, int m) const {
    double2 g = make_double2(0.0, 0.0);
    if (l >= 1) g = cadd(g, cscale(cplus[(long)(l - 1) * (L + 1) + m], lo));
    if (l + 1 <= L) g = cadd(g, cscale(cminus[(long)(l + 1) * (L + 1) + m], hi));
    return g;
  }
  // Transpose of snt on degrees [m, L]: (snt^T g)_l = C+_l g_{l+1} + C-_l g_{l-1}
  // (the adjoint coupling of spectral_operators.py:243-270).
  __device__ double2 snt_t(double2 lo, double2 hi, int l, int m) const {
    double2 g = make_double2(0.0, 0.0);
    if (l + 1 <= L) g = cadd(g, cscale(cplus[(long)l * (L + 1) + m], hi));
    if (l >= 1) g = cadd(g, cscale(cminus[(long)l * (L + 1) + m], lo));
    return g;
  }
};

// ------------------------------------------------------------------ BVE
struct BveDerive {  // psi_lam, psi_snt, eta_lam, eta_snt
  static constexpr int NF = 4;
  static constexpr bool kColumnDf = true;  // column_df below
  Spec s;
  const double2* zeta;  // [b][L+1][L+1]
  double f10;           // 2 Omega sqrt(4 pi / 3)
  __device__ void column(int b, int l, int m, double2* v) const {
    const double2* z = zeta + (long)b * (s.L + 1) * (s.L + 1);
    const int L = s.L;
    const double2 zero = make_double2(0.0, 0.0);
    if (s.dcoef) {  // coefficient products tabulated at the plan radius (see SweDerive::column_tab)
      const long r = (long)l * (L + 1) + m;
      const double* c = s.dcoef + r * 8;
      const double A1 = c[0], A2 = c[1], A3 = c[2], B1 = c[3], B2 = c[4], B3 = c[5];
      const bool lo = l >= 1 && l - 1 >= m, hi = l + 1 <= L;
      const double2 zl = z[r];
      double2 z_lo = lo ? z[r - (L + 1)] : zero, z_hi = hi ? z[r + (L + 1)] : zero;
      v[0] = make_double2(-A3 * zl.y, A3 * zl.x);
      v[1] = make_double2(fma(A1, z_lo.x, A2 * z_hi.x), fma(A1, z_lo.y, A2 * z_hi.y));
      v[2] = make_double2(-B3 * zl.y, B3 * zl.x);
      if (m == 0) {
        if (l - 1 == 1) z_lo.x += f10;
        if (l + 1 == 1) z_hi.x += f10;
      }
      v[3] = make_double2(fma(B1, z_lo.x, B2 * z_hi.x), fma(B1, z_lo.y, B2 * z_hi.y));
      return;
    }
    double2 psi = s.invlap0(z, l, m);
    double2 psi_lo = l >= 1 ? s.invlap0(z, l - 1, m) : zero;
    double2 psi_hi = l + 1 <= L ? s.invlap0(z, l + 1, m) : zero;
    double2 eta_lo = l >= 1 ? s.at(z, l - 1, m) : zero;
    double2 eta_hi = l + 1 <= L ? s.at(z, l + 1, m) : zero;
    if (m == 0) {
      if (l - 1 == 1) eta_lo.x += f10;
      if (l + 1 == 1) eta_hi.x += f10;
    }
    v[0] = s.dlam(psi, m);
    v[1] = cscale(s.ir, s.snt(psi_lo, psi_hi, l, m));
    v[2] = s.dlam(s.at(z, l, m), m);
    v[3] = cscale(s.ir, s.snt(eta_lo, eta_hi, l, m));
  }
  // The same fields in double-float arithmetic (lanes re, im) from the
  // double-float coefficient table: the derive of the split path, whose
  // digits carry 48 bits, issues no FP64 instruction.  Without the table
  // (another radius) the FP64 fields, converted.
  __device__ void column_df(int b, int l, int m, df2* v) const {
    if (!s.dcoef_df) {
      double2 w[NF];
      column(b, l, m, w);
#pragma unroll
      for (int f = 0; f < NF; ++f) v[f] = df2_of_f64x2(w[f]);
      return;
    }
    const int L = s.L;
    const long r = (long)l * (L + 1) + m;
    const double2* z = zeta + (long)b * (L + 1) * (L + 1);
    const float2* c = s.dcoef_df + r * 8;
    const df2 zero = df2{0ull, 0ull};
    const bool lo = l >= 1 && l - 1 >= m, hi = l + 1 <= L;
    const df2 izl = df2_times_i(df2_of_f64x2(z[r]));
    df2 z_lo = lo ? df2_of_f64x2(z[r - (L + 1)]) : zero, z_hi = hi ? df2_of_f64x2(z[r + (L + 1)]) : zero;
    auto k = [&](int i) { return df2_splat(df{c[i].x, c[i].y}); };
    v[0] = df2_mul(k(2), izl);
    v[1] = df2_add_fast(df2_mul(k(0), z_lo), df2_mul(k(1), z_hi));
    v[2] = df2_mul(k(5), izl);
    if (m == 0 && (l == 2 || l == 0)) {  // planetary vorticity of the (1, 0) mode in eta
      df re, im;
      df2_unpack(l == 2 ? z_lo : z_hi, re, im);
      re = df_add(re, df_of_f64(f10));
      (l == 2 ? z_lo : z_hi) = df2_pack(re, im);
    }
    v[3] = df2_add_fast(df2_mul(k(3), z_lo), df2_mul(k(4), z_hi));
  }
};

struct JacPw {  // J = (a_snt b_lam - a_lam b_snt) / cos^2
  static constexpr int NIN = 4, NOUT = 1;
  static constexpr bool kIdentity = false;
  __device__ unsigned operator()(double c, double, const double* in, double* out) const {
    out[0] = (in[1] * in[2] - in[0] * in[3]) / (c * c);
    return 0u;
  }
  __device__ RowDf df_row(double c, double) const { return RowDf{df_from_double(1.0 / (c * c)), df{0.f, 0.f}, (float)c}; }
  __device__ unsigned df_op(const RowDf& r, const df* in, df* out) const {
    out[0] = df_mul(df_sub(df_mul(in[1], in[2]), df_mul(in[0], in[3])), r.invc);
    return 0u;
  }
  // df_op at two grid points on the packed two-lane pipe (bitwise df_op)
  __device__ unsigned df_op2(const RowDf& r, const df2* in, df2* out) const {
    out[0] = df2_mul(df2_add(df2_mul(in[1], in[2]), df2_neg(df2_mul(in[0], in[3]))), df2_pack(r.invc, r.invc));
    return 0u;
  }
};

// RK4 stage bookkeeping shared by both models.  mode 0: tendency output;
// modes 1..4: stage s of the classical RK4 (run/engine.py:406-431).
struct Rk4 {
  int mode;
  double dt;
  double2* y0;      // step-start state (updated at stage 4)
  double2* ystage;  // stage input for the next stage
  double2* acc;     // k1 + 2 k2 + 2 k3
  double2* tend;    // mode 0 output
  __device__ void apply(long i, double2 k) const {
    if (mode == 0) {
      tend[i] = k;
    } else if (mode == 1) {
      acc[i] = k;
      ystage[i] = cadd(y0[i], cscale(0.5 * dt, k));
    } else if (mode == 2) {
      acc[i] = cadd(acc[i], cscale(2.0, k));
      ystage[i] = cadd(y0[i], cscale(0.5 * dt, k));
    } else if (mode == 3) {
      acc[i] = cadd(acc[i], cscale(2.0, k));
      ystage[i] = cadd(y0[i], cscale(dt, k));
    } else {
      y0[i] = cadd(y0[i], cscale(dt / 6.0, cadd(acc[i], k)));
    }
  }
  __device__ void zero(long i) const {
    const double2 z = make_double2(0.0, 0.0);
    if (mode == 0) tend[i] = z;
    else if (mode < 4) { acc[i] = z; ystage[i] = z; }
    else y0[i] = z;
  }
};

struct BveEpi {  // -trunc(A J) + nu lap zeta (+ forcing), l = 0 row zero
  static constexpr int NF = 1;
  Spec s;
  const double2* zeta;     // stage input
  const double2* forcing;  // optional
  double nu;
  Rk4 rk;
  __device__ void finish(int b, int l, int m, const double2* acc) const {
    const int L = s.L;
    const int cut = (2 * L) / 3;
    const long i = ((long)b * (L + 1) + l) * (L + 1) + m;
    double2 k = make_double2(0.0, 0.0);
    if (l > 0) {
      double2 J = (l > cut || m > cut) ? make_double2(0.0, 0.0) : acc[0];
      const double lapb = s.lap(l);
      k = cadd(make_double2(-J.x, -J.y), cscale(nu * lapb, zeta[i]));
      if (forcing) k = cadd(k, forcing[i]);
    }
    rk.apply(i, k);
  }
  __device__ void zero(int b, int l, int m) const { rk.zero(((long)b * (s.L + 1) + l) * (s.L + 1) + m); }
};

// ------------------------------------------------------------------ SWE
// Synthesised fields: U, V (= u cos, v cos), eta_lam, eta_snt, phi_lam,
// phi_snt, zeta, delta, phi.
struct SweDerive {
  static constexpr int NF = 9;
  Spec s;
  const double2* state;  // [b][3][L+1][L+1]
  double f10;            // 0 when the Coriolis terms are taken spectrally (SweEpi::coriolis)
  __device__ void column(int b, int l, int m, double2* v) const {
    if (s.dcoef) {
      column_tab(b, l, m, v);
      return;
    }
    const int L = s.L;
    const long n2 = (long)(L + 1) * (L + 1);
    const double2* z = state + (long)b * 3 * n2;
    const double2* d = z + n2;
    const double2* ph = d + n2;
    const double2 zero = make_double2(0.0, 0.0);
    const bool lo = l >= 1, hi = l + 1 <= L;
    const double ir = s.ir;
    // psi, chi (l = 0 zero) at l-1, l, l+1
    const double2 psi = s.invlap0(z, l, m), chi = s.invlap0(d, l, m);
    const double2 psi_lo = lo ? s.invlap0(z, l - 1, m) : zero, psi_hi = hi ? s.invlap0(z, l + 1, m) : zero;
    const double2 chi_lo = lo ? s.invlap0(d, l - 1, m) : zero, chi_hi = hi ? s.invlap0(d, l + 1, m) : zero;
    v[0] = cadd(cscale(ir, s.snt(psi_lo, psi_hi, l, m)), s.dlam(chi, m));
    v[1] = csub(s.dlam(psi, m), cscale(ir, s.snt(chi_lo, chi_hi, l, m)));
    const double2 zl = s.at(z, l, m);
    double2 eta_lo = lo ? s.at(z, l - 1, m) : zero, eta_hi = hi ? s.at(z, l + 1, m) : zero;
    if (m == 0) {
      if (l - 1 == 1) eta_lo.x += f10;
      if (l + 1 == 1) eta_hi.x += f10;
    }
    v[2] = s.dlam(zl, m);
    v[3] = cscale(ir, s.snt(eta_lo, eta_hi, l, m));
    const double2 pl = s.at(ph, l, m);
    v[4] = s.dlam(pl, m);
    v[5] = cscale(ir, s.snt(lo ? s.at(ph, l - 1, m) : zero, hi ? s.at(ph, l + 1, m) : zero, l, m));
    v[6] = zl;
    v[7] = s.at(d, l, m);
    v[8] = pl;
    if (cor) {
      // planetary-vorticity terms of the split path (added by SweEpi), from the
      // fields at hand: zeta_dot += -(2 Omega/a) V - 2 Omega (x delta),
      // curl += 2 Omega (x zeta) - (2 Omega/a) U
      const double wr = two_omega * ir;
      const double2 xz = s.xmul(eta_lo, eta_hi, l, m);
      const double2 xd = s.xmul(lo ? s.at(d, l - 1, m) : zero, hi ? s.at(d, l + 1, m) : zero, l, m);
      double2* c = cor + (long)b * 2 * n2 + (long)l * (L + 1) + m;
      c[0] = make_double2(-(wr * v[1].x + two_omega * xd.x), -(wr * v[1].y + two_omega * xd.y));
      c[n2] = make_double2(two_omega * xz.x - wr * v[0].x, two_omega * xz.y - wr * v[0].y);
    }
  }
  double2* cor = nullptr;   // optional [b][2][L+1][L+1] Coriolis spectra (split path, f10 = 0)
  double two_omega = 0.0;

  // The same fields with the per-(l, m) coefficient products tabulated at the
  // plan radius (Spec::dcoef): U = A1 zeta_{l-1} + A2 zeta_{l+1} + i A3 delta_l,
  // V = i A3 zeta_l - A1 delta_{l-1} - A2 delta_{l+1}, ... -- about half the
  // FP64 operations of the operator-by-operator form (the FP64 pipe is the
  // slow one on GB300).  Neighbour slots outside m..L are not read.
  __device__ void column_tab(int b, int l, int m, double2* v) const {
    const int L = s.L;
    const long n2 = (long)(L + 1) * (L + 1);
    const long r = (long)l * (L + 1) + m;
    const double2* z = state + (long)b * 3 * n2;
    const double2* d = z + n2;
    const double2* ph = d + n2;
    const double* c = s.dcoef + r * 8;
    const double A1 = c[0], A2 = c[1], A3 = c[2], B1 = c[3], B2 = c[4], B3 = c[5];
    const bool lo = l >= 1 && l - 1 >= m, hi = l + 1 <= L;
    const double2 zero = make_double2(0.0, 0.0);
    const double2 zl = z[r], dl = d[r], pl = ph[r];
    double2 z_lo = lo ? z[r - (L + 1)] : zero, z_hi = hi ? z[r + (L + 1)] : zero;
    const double2 d_lo = lo ? d[r - (L + 1)] : zero, d_hi = hi ? d[r + (L + 1)] : zero;
    const double2 p_lo = lo ? ph[r - (L + 1)] : zero, p_hi = hi ? ph[r + (L + 1)] : zero;
    // U, V from psi = zeta / lap, chi = delta / lap (the 1/lap folded into A1..A3)
    const double2 U = make_double2(fma(A1, z_lo.x, fma(A2, z_hi.x, -A3 * dl.y)), fma(A1, z_lo.y, fma(A2, z_hi.y, A3 * dl.x)));
    const double2 V = make_double2(-fma(A1, d_lo.x, fma(A2, d_hi.x, A3 * zl.y)), fma(A3, zl.x, -fma(A1, d_lo.y, A2 * d_hi.y)));
    if (m == 0) {  // planetary vorticity of the (1, 0) mode in eta
      if (l - 1 == 1) z_lo.x += f10;
      if (l + 1 == 1) z_hi.x += f10;
    }
    v[0] = U;
    v[1] = V;
    v[2] = make_double2(-B3 * zl.y, B3 * zl.x);
    v[3] = make_double2(fma(B1, z_lo.x, B2 * z_hi.x), fma(B1, z_lo.y, B2 * z_hi.y));
    v[4] = make_double2(-B3 * pl.y, B3 * pl.x);
    v[5] = make_double2(fma(B1, p_lo.x, B2 * p_hi.x), fma(B1, p_lo.y, B2 * p_hi.y));
    v[6] = zl;
    v[7] = dl;
    v[8] = pl;
    if (cor) {
      const double X1 = c[6], X2 = c[7];
      const double wr = two_omega * s.ir;
      const double2 xz = make_double2(fma(X1, z_lo.x, X2 * z_hi.x), fma(X1, z_lo.y, X2 * z_hi.y));
      const double2 xd = make_double2(fma(X1, d_lo.x, X2 * d_hi.x), fma(X1, d_lo.y, X2 * d_hi.y));
      double2* co = cor + (long)b * 2 * n2 + r;
      co[0] = make_double2(-fma(wr, V.x, two_omega * xd.x), -fma(wr, V.y, two_omega * xd.y));
      co[n2] = make_double2(fma(two_omega, xz.x, -wr * U.x), fma(two_omega, xz.y, -wr * U.y));
    }
  }
};

// Products of physics/shallow_water.py:375-386 (module docstring identities).
struct SwePw {
  static constexpr int NIN = 9, NOUT = 4;
  static constexpr bool kIdentity = false;
  double f10;   // eta = zeta + f10 * fgrid (0: products of the relative vorticity only)
  double phi0;  // positivity check of Phi0 + phi
  float phi0f;  // the same as a float (double-float path)
  __device__ unsigned operator()(double c, double fg, const double* in, double* out) const {
    const double u = in[0] / c, v = in[1] / c;
    const double eta_lam = in[2], eta_snt = in[3], phi_lam = in[4], phi_snt = in[5];
    const double zeta = in[6], delta = in[7], phi = in[8];
    const double eta = zeta + f10 * fg;
    out[0] = -((u * eta_lam - v * eta_snt) / c + eta * delta);
    out[1] = eta * zeta + (v * eta_lam + u * eta_snt) / c;
    out[2] = 0.5 * (u * u + v * v);
    out[3] = -((u * phi_lam - v * phi_snt) / c + phi * delta);
    unsigned bits = 0u;
    if (!(isfinite(out[0]) && isfinite(out[1]) && isfinite(out[2]) && isfinite(out[3]))) bits |= AEOLUS_STATE_NONFINITE;
    if (!(phi0 + phi > 0.0)) bits |= AEOLUS_STATE_THICKNESS;
    return bits;
  }
  __device__ RowDf df_row(double c, double fg) const {
    return RowDf{df_from_double(1.0 / c), df_from_double(f10 * fg), (float)c};
  }
  __device__ unsigned df_op(const RowDf& r, const df* in, df* out) const {
    const df u = df_mul(in[0], r.invc), v = df_mul(in[1], r.invc);
    const df eta_lam = in[2], eta_snt = in[3], phi_lam = in[4], phi_snt = in[5];
    const df zeta = in[6], delta = in[7], phi = in[8];
    // Dekker additions: error relative to the operands, the normwise bound
    // the transforms around these products carry anyway
    const df eta = df_add_fast(zeta, r.fj);
    out[0] = df_neg(df_add_fast(df_mul(df_add_fast(df_mul(u, eta_lam), df_neg(df_mul(v, eta_snt))), r.invc),
                                df_mul(eta, delta)));
    out[1] = df_add_fast(df_mul(eta, zeta), df_mul(df_add_fast(df_mul(v, eta_lam), df_mul(u, eta_snt)), r.invc));
    out[2] = df_scale2(df_add_fast(df_mul(u, u), df_mul(v, v)), 0.5f);
    out[3] = df_neg(df_add_fast(df_mul(df_add_fast(df_mul(u, phi_lam), df_neg(df_mul(v, phi_snt))), r.invc),
                                df_mul(phi, delta)));
    unsigned bits = 0u;
    if (!(isfinite(out[0].hi) && isfinite(out[1].hi) && isfinite(out[2].hi) && isfinite(out[3].hi)))
      bits |= AEOLUS_STATE_NONFINITE;
    if (!(phi0f + phi.hi > 0.0f)) bits |= AEOLUS_STATE_THICKNESS;
    return bits;
  }
  // df_op of two grid points on the packed two-lane f32 pipe (the same
  // operations in the same order, lane by lane).
  __device__ unsigned df_op2(const RowDf& r, const df2* in, df2* out) const {
    const df2 invc = df2_pack(r.invc, r.invc), fj = df2_pack(r.fj, r.fj);
    const df2 u = df2_mul(in[0], invc), v = df2_mul(in[1], invc);
    const df2 eta_lam = in[2], eta_snt = in[3], phi_lam = in[4], phi_snt = in[5];
    const df2 zeta = in[6], delta = in[7], phi = in[8];
    const df2 eta = df2_add_fast(zeta, fj);
    out[0] = df2_neg(df2_add_fast(df2_mul(df2_add_fast(df2_mul(u, eta_lam), df2_neg(df2_mul(v, eta_snt))), invc),
                                  df2_mul(eta, delta)));
    out[1] = df2_add_fast(df2_mul(eta, zeta), df2_mul(df2_add_fast(df2_mul(v, eta_lam), df2_mul(u, eta_snt)), invc));
    out[2] = df2_scale2(df2_add_fast(df2_mul(u, u), df2_mul(v, v)), f2_splat(0.5f));
    out[3] = df2_neg(df2_add_fast(df2_mul(df2_add_fast(df2_mul(u, phi_lam), df2_neg(df2_mul(v, phi_snt))), invc),
                                  df2_mul(phi, delta)));
    bool fin = true;
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      float x0, x1;
      f2_unpack(out[f].hi, x0, x1);
      fin = fin && isfinite(x0) && isfinite(x1);
    }
    float p0, p1;
    f2_unpack(phi.hi, p0, p1);
    unsigned bits = 0u;
    if (!fin) bits |= AEOLUS_STATE_NONFINITE;
    if (!(phi0f + p0 > 0.0f) || !(phi0f + p1 > 0.0f)) bits |= AEOLUS_STATE_THICKNESS;
    return bits;
  }
};

// Split-precision form of the SWE derive: the tensor-core synthesis
// contracts 7 fields [U, V, eta_snt, phi_snt, zeta, delta, phi] and its
// epilogue writes the 9 spectra blocks of SwePw, forming the longitude
// derivatives eta_lam = i m/R zeta and phi_lam = i m/R phi from the zeta
// and phi order spectra (d/dlambda is diagonal in m, so it needs no
// contraction of its own; see SynthOut in split.cuh).
struct SweDerive7 {
  static constexpr int NF = 7;
  static constexpr bool kColumnDf = true;  // column_df below
  static constexpr int NBLK = 9;  // spectra blocks written by the synthesis epilogue
  __host__ __device__ static constexpr int blk(int f) { return f == 0 ? 0 : f == 1 ? 1 : f == 2 ? 3 : f == 3 ? 5 : f + 2; }
  __host__ __device__ static constexpr int lam_blk(int f) { return f == 4 ? 2 : f == 6 ? 4 : -1; }
  SweDerive d9;
  double lam_ir() const { return d9.s.ir; }  // 1 / R of the i m / R factor
  __device__ void column(int b, int l, int m, double2* v) const {
    double2 w[9];
    d9.column(b, l, m, w);
    v[0] = w[0];
    v[1] = w[1];
    v[2] = w[3];
    v[3] = w[5];
    v[4] = w[6];
    v[5] = w[7];
    v[6] = w[8];
  }
  // The same seven fields (and the Coriolis spectra) as SweDerive::column_tab
  // in double-float arithmetic with the lanes (re, im), from the double-
  // float coefficient table: no FP64 instruction but the four additions
  // that round the Coriolis spectra to FP64.  Without the table (another
  // radius) the FP64 fields, converted.
  __device__ void column_df(int b, int l, int m, df2* v) const {
    const Spec& s = d9.s;
    if (!s.dcoef_df) {
      double2 w[NF];
      column(b, l, m, w);
#pragma unroll
      for (int f = 0; f < NF; ++f) v[f] = df2_of_f64x2(w[f]);
      return;
    }
    const int L = s.L;
    const long n2 = (long)(L + 1) * (L + 1);
    const long r = (long)l * (L + 1) + m;
    const double2* z = d9.state + (long)b * 3 * n2;
    const double2* d = z + n2;
    const double2* ph = d + n2;
    const float2* c = s.dcoef_df + r * 8;
    auto k = [&](int i) { return df2_splat(df{c[i].x, c[i].y}); };
    const bool lo = l >= 1 && l - 1 >= m, hi = l + 1 <= L;
    const df2 zero = df2{0ull, 0ull};
    const df2 zl = df2_of_f64x2(z[r]), dl = df2_of_f64x2(d[r]), pl = df2_of_f64x2(ph[r]);
    df2 z_lo = lo ? df2_of_f64x2(z[r - (L + 1)]) : zero, z_hi = hi ? df2_of_f64x2(z[r + (L + 1)]) : zero;
    const df2 d_lo = lo ? df2_of_f64x2(d[r - (L + 1)]) : zero, d_hi = hi ? df2_of_f64x2(d[r + (L + 1)]) : zero;
    const df2 p_lo = lo ? df2_of_f64x2(ph[r - (L + 1)]) : zero, p_hi = hi ? df2_of_f64x2(ph[r + (L + 1)]) : zero;
    // U = A1 zeta_{l-1} + A2 zeta_{l+1} + i A3 delta_l, V = i A3 zeta_l - A1 delta_{l-1} - A2 delta_{l+1}
    const df2 A1 = k(0), A2 = k(1), A3 = k(2);
    const df2 U = df2_add_fast(df2_add_fast(df2_mul(A1, z_lo), df2_mul(A2, z_hi)), df2_mul(A3, df2_times_i(dl)));
    const df2 V = df2_sub_fast(df2_mul(A3, df2_times_i(zl)), df2_add_fast(df2_mul(A1, d_lo), df2_mul(A2, d_hi)));
    if (m == 0 && (l == 2 || l == 0) && d9.f10 != 0.0) {  // planetary vorticity of the (1, 0) mode in eta
      df re, im;
      df2_unpack(l == 2 ? z_lo : z_hi, re, im);
      re = df_add(re, df_of_f64(d9.f10));
      (l == 2 ? z_lo : z_hi) = df2_pack(re, im);
    }
    const df2 B1 = k(3), B2 = k(4);
    v[0] = U;
    v[1] = V;
    v[2] = df2_add_fast(df2_mul(B1, z_lo), df2_mul(B2, z_hi));
    v[3] = df2_add_fast(df2_mul(B1, p_lo), df2_mul(B2, p_hi));
    v[4] = zl;
    v[5] = dl;
    v[6] = pl;
    if (d9.cor) {  // zeta_dot += -(2 Omega/a) V - 2 Omega (x delta), curl += 2 Omega (x zeta) - (2 Omega/a) U
      const df2 X1 = k(6), X2 = k(7);
      const df tw = df_of_f64(d9.two_omega);
      const df2 tw2 = df2_splat(tw), wr2 = df2_splat(df_mul(tw, df_of_f64(s.ir)));
      const df2 xz = df2_add_fast(df2_mul(X1, z_lo), df2_mul(X2, z_hi));
      const df2 xd = df2_add_fast(df2_mul(X1, d_lo), df2_mul(X2, d_hi));
      double2* co = d9.cor + (long)b * 2 * n2 + r;
      co[0] = f64x2_of_df2(df2_neg(df2_add_fast(df2_mul(wr2, V), df2_mul(tw2, xd))));
      co[n2] = f64x2_of_df2(df2_sub_fast(df2_mul(tw2, xz), df2_mul(wr2, U)));
    }
  }
};

// Spectral epilogue of the SWE tendency.  With `coriolis` set (split-
// precision path) the pointwise products carry only the relative vorticity
// and the planetary-vorticity terms are added here exactly:
//   eta u products with eta = zeta + f, f = 2 Omega x, f_snt = -(2 Omega/a) cos^2(lat):
//   zeta_dot += -(2 Omega/a) V - 2 Omega (x delta),  curl += 2 Omega (x zeta) - (2 Omega/a) U
// with U = u cos(lat), V = v cos(lat) the Helmholtz fields of the stage state.
// The Gauss product quadrature is exact for these degree-(L+1) products, so
// this equals the analysed product up to rounding, while the terms that pass
// through the split contraction shrink ~10x (|zeta| << |f|).
struct SweEpi {
  static constexpr int NF = 4;
  Spec s;
  const double2* state;  // stage input [b][3][L+1][L+1]
  double phi0, nu4;
  Rk4 rk;
  double two_omega;      // > 0: add the Coriolis terms spectrally
  const double2* cor = nullptr;  // their spectra tabulated by SweDerive (else computed here)
  const double2* forcing = nullptr;  // constant [3][L+1][L+1] terms (bottom topography), or none
  __device__ void finish(int b, int l, int m, const double2* an_in) const {
    const int L = s.L;
    const int cut = (2 * L) / 3;
    const long n2 = (long)(L + 1) * (L + 1);
    const long base = (long)b * 3 * n2 + (long)l * (L + 1) + m;
    const bool tr = l > cut || m > cut;
    const double2 z0 = make_double2(0.0, 0.0);
    double2 an[4] = {an_in[0], an_in[1], an_in[2], an_in[3]};
    if (two_omega > 0.0 && !tr) {
      if (cor) {  // tabulated by SweDerive for this stage input
        const double2* c = cor + (long)b * 2 * n2 + (long)l * (L + 1) + m;
        an[0] = cadd(an[0], c[0]);
        an[1] = cadd(an[1], c[n2]);
      } else {
        const double2* z = state + (long)b * 3 * n2;
        const double2* d = z + n2;
        const bool lo = l >= 1, hi = l + 1 <= L;
        const double ir = s.ir;
        const double2 psi = s.invlap0(z, l, m), chi = s.invlap0(d, l, m);
        const double2 psi_lo = lo ? s.invlap0(z, l - 1, m) : z0, psi_hi = hi ? s.invlap0(z, l + 1, m) : z0;
        const double2 chi_lo = lo ? s.invlap0(d, l - 1, m) : z0, chi_hi = hi ? s.invlap0(d, l + 1, m) : z0;
        const double2 U = cadd(cscale(ir, s.snt(psi_lo, psi_hi, l, m)), s.dlam(chi, m));
        const double2 V = csub(s.dlam(psi, m), cscale(ir, s.snt(chi_lo, chi_hi, l, m)));
        const double2 xz = s.xmul(lo ? s.at(z, l - 1, m) : z0, hi ? s.at(z, l + 1, m) : z0, l, m);
        const double2 xd = s.xmul(lo ? s.at(d, l - 1, m) : z0, hi ? s.at(d, l + 1, m) : z0, l, m);
        const double wr = two_omega * ir;
        an[0] = csub(an[0], cadd(cscale(wr, V), cscale(two_omega, xd)));
        an[1] = cadd(an[1], csub(cscale(two_omega, xz), cscale(wr, U)));
      }
    }
    const double2 a0 = tr ? z0 : an[0], a1 = tr ? z0 : an[1], a2 = tr ? z0 : an[2], a3 = tr ? z0 : an[3];
    const double2 zs = state[base], ds = state[base + n2], ps = state[base + 2 * n2];
    const double lap = s.lap(l);
    double2 k0 = a0;
    double2 k1 = csub(a1, cscale(lap, cadd(a2, ps)));
    double2 k2 = csub(a3, cscale(phi0, ds));
    const long fo = (long)l * (L + 1) + m;
    if (forcing) {  // -lap(phi_s) joins the divergence tendency before the hyperdiffusion
      k0 = cadd(k0, forcing[fo]);
      k1 = cadd(k1, forcing[n2 + fo]);
    }
    if (nu4 > 0.0) {
      const double h = nu4 * (lap * lap);
      k0 = csub(k0, cscale(h, zs));
      k1 = csub(k1, cscale(h, ds));
      k2 = csub(k2, cscale(h, ps));
    }
    if (forcing) k2 = cadd(k2, forcing[2 * n2 + fo]);  // after it, as -nu4 lap^2 phi_s
    if (l == 0) k0 = k1 = k2 = z0;
    rk.apply(base, k0);
    rk.apply(base + n2, k1);
    rk.apply(base + 2 * n2, k2);
  }
  __device__ void zero(int b, int l, int m) const {
    const long n2 = (long)(s.L + 1) * (s.L + 1);
    const long base = (long)b * 3 * n2 + (long)l * (s.L + 1) + m;
    rk.zero(base);
    rk.zero(base + n2);
    rk.zero(base + 2 * n2);
  }
};

// Synthesis of one field of a stacked state (field index fi of nf).
// The reciprocal table is tabulated with the plan's radius; a call with a
// different radius must not use it.
Spec make_spec(const aeolus_plan_impl* p, double R) {
  return Spec{p->lmax, R, 1.0 / R, 1.0 / (R * R), p->cplus, p->cminus, R == p->radius ? p->invlap : nullptr,
              p->xa, p->xb, R == p->radius ? p->dcoef : nullptr,
              R == p->radius ? reinterpret_cast<const float2*>(p->dcoef_df) : nullptr};
}

// ---------------------------------------------------------- helpers
size_t state_bytes(const aeolus_plan_impl* p, int nf, int batch) {
  return (size_t)batch * nf * (p->lmax + 1) * (p->lmax + 1) * sizeof(double2);
}

int check_common(const aeolus_plan_impl* p, const char* who, int batch, const void* a, const void* b) {
  if (!plan_ok(p)) return fail(AEOLUS_ERR_ARG, std::string(who) + ": invalid plan");
  if (batch < 0) return fail(AEOLUS_ERR_ARG, std::string(who) + ": negative batch");
  if (batch > 0 && (!a || !b)) return fail(AEOLUS_ERR_ARG, std::string(who) + ": NULL array");
  if (batch > 65535) return fail(AEOLUS_ERR_ARG, std::string(who) + ": batch above 65535");
  return AEOLUS_OK;
}

inline int bve_check(aeolus_plan plan, const aeolus_bve_params* p, const char* who) {
  if (!p) return fail(AEOLUS_ERR_ARG, std::string(who) + ": NULL params");
  if (!(p->radius > 0.0) || !std::isfinite(p->omega) || !std::isfinite(p->viscosity))
    return fail(AEOLUS_ERR_ARG, std::string(who) + ": bad parameters");
  (void)plan;
  return AEOLUS_OK;
}

inline int swe_check(const aeolus_swe_params* p, const char* who) {
  if (!p) return fail(AEOLUS_ERR_ARG, std::string(who) + ": NULL params");
  if (!(std::isfinite(p->gravity) && p->gravity > 0))
    return fail(AEOLUS_ERR_ARG, "gravity must be finite and > 0, got " + std::to_string(p->gravity));
  if (!(std::isfinite(p->mean_depth) && p->mean_depth > 0))
    return fail(AEOLUS_ERR_ARG, "mean_depth must be finite and > 0, got " + std::to_string(p->mean_depth));
  if (!(std::isfinite(p->nu4) && p->nu4 >= 0))
    return fail(AEOLUS_ERR_ARG, "hyperdiffusion_nu4 must be finite and >= 0, got " + std::to_string(p->nu4));
  if (!(p->radius > 0.0) || !std::isfinite(p->omega)) return fail(AEOLUS_ERR_ARG, std::string(who) + ": bad radius/omega");
  return AEOLUS_OK;
}
}  // namespace
}  // namespace aeolus
