// Curl and divergence of tangent vector fields by the weak form with
// one-degree-extended analyses (numerics/spectral_operators.py:399-502,
// vector_curl_div_spectral, and :474-492 _vector_analysis_pieces).
//
// Integration by parts on the sphere moves the horizontal derivatives onto
// the basis; with the half-metric analyses a = A(F_east / cos), b =
// A(F_north / cos) on the product points (same points and weights, basis
// extended to degree L+1), the discrete weak form is
//
//   div_lm  = (i m / R) a_lm + (1/R) (S^T b)_lm
//   curl_lm = (i m / R) b_lm - (1/R) (S^T a)_lm
//   (S^T c)_lm = C+_lm c_{l+1,m} + C-_lm c_{l-1,m}
//
// with the unclipped C+ at l = L reading the extended degree, followed by the
// optional 2/3 cut of rows and columns (cut = floor(2L/3)).  One analysis
// chain on the extended plan (the 1/cos metric is its pointwise stage) and
// one spectral kernel.
#include "chains.cuh"

namespace aeolus {
namespace {

struct PwInvCos {  // (F_east, F_north) -> (F_east, F_north) / cos
  static constexpr int NIN = 2, NOUT = 2;
  static constexpr bool kIdentity = false;
  __device__ unsigned operator()(double c, double, const double* in, double* out) const {
    out[0] = in[0] / c;
    out[1] = in[1] / c;
    return 0u;
  }
  __device__ RowDf df_row(double c, double) const { return RowDf{df_from_double(1.0 / c), df{0.f, 0.f}, (float)c}; }
  __device__ unsigned df_op(const RowDf& r, const df* in, df* out) const {
    out[0] = df_mul(in[0], r.invc);
    out[1] = df_mul(in[1], r.invc);
    return 0u;
  }
};

struct EpiStore2 {  // extended analyses: dense [b][2][Le+1][Le+1]
  static constexpr int NF = 2;
  double2* out;
  int Le;
  __device__ long at(int b, int f, int l, int m) const {
    const long n2 = (long)(Le + 1) * (Le + 1);
    return ((long)b * 2 + f) * n2 + (long)l * (Le + 1) + m;
  }
  __device__ void finish(int b, int l, int m, const double2* acc) const {
    out[at(b, 0, l, m)] = acc[0];
    out[at(b, 1, l, m)] = acc[1];
  }
  __device__ void finish_field(int b, int f, int l, int m, double2 a) const { out[at(b, f, l, m)] = a; }
  __device__ void zero(int b, int l, int m) const {
    out[at(b, 0, l, m)] = make_double2(0.0, 0.0);
    out[at(b, 1, l, m)] = make_double2(0.0, 0.0);
  }
};

// C+_lm = l sqrt(((l+1)^2 - m^2) / ((2l+1)(2l+3))), C-_lm = -(l+1) sqrt((l^2 - m^2) / ((2l-1)(2l+1)))
// (spectral_operators.py:135-176), for m <= l; C- is 0 at l = 0.
__device__ inline double c_plus(int l, int m) {
  const double L = l, M = m;
  return L * sqrt(((L + 1.0) * (L + 1.0) - M * M) / ((2.0 * L + 1.0) * (2.0 * L + 3.0)));
}
__device__ inline double c_minus(int l, int m) {
  if (l == 0) return 0.0;
  const double L = l, M = m;
  return -(L + 1.0) * sqrt((L * L - M * M) / ((2.0 * L - 1.0) * (2.0 * L + 1.0)));
}

__global__ void vector_finish_kernel(const double2* __restrict__ ext, int L, int batch, double inv_r, int truncate,
                                     double2* __restrict__ curl, double2* __restrict__ div) {
  const long n2 = (long)(L + 1) * (L + 1);
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2 * batch) return;
  const int b = (int)(idx / n2);
  const int r = (int)(idx - (long)b * n2);
  const int l = r / (L + 1), m = r - l * (L + 1);
  const int Le = L + 1;
  const long ne = (long)(Le + 1) * (Le + 1);
  const int cut = (2 * L) / 3;
  double2 cv = make_double2(0.0, 0.0), dv = make_double2(0.0, 0.0);
  if (m <= l && !(truncate && (l > cut || m > cut))) {
    const double2* a = ext + (long)b * 2 * ne;
    const double2* bb = a + ne;
    const long o = (long)l * (Le + 1) + m;
    const double cp = c_plus(l, m), cm = c_minus(l, m);
    // S^T c at (l, m): C+ c_{l+1,m} (l+1 <= L+1 always) + C- c_{l-1,m}
    const double2 a_up = a[o + (Le + 1)], b_up = bb[o + (Le + 1)];
    const double2 a_dn = l > 0 ? a[o - (Le + 1)] : make_double2(0.0, 0.0);
    const double2 b_dn = l > 0 ? bb[o - (Le + 1)] : make_double2(0.0, 0.0);
    const double2 sta = make_double2(cp * a_up.x + cm * a_dn.x, cp * a_up.y + cm * a_dn.y);
    const double2 stb = make_double2(cp * b_up.x + cm * b_dn.x, cp * b_up.y + cm * b_dn.y);
    const double mr = m * inv_r;  // i m / R times a: (-m a.y, m a.x) / R
    const double2 al = a[o], bl = bb[o];
    dv = make_double2(-mr * al.y + inv_r * stb.x, mr * al.x + inv_r * stb.y);
    cv = make_double2(-mr * bl.y - inv_r * sta.x, mr * bl.x - inv_r * sta.y);
  }
  curl[idx] = cv;
  div[idx] = dv;
}

}  // namespace

size_t vector_op_bytes(const aeolus_plan_impl* p, int batch) {
  const size_t ne = (size_t)(p->lmax + 1) * (p->lmax + 1);
  return anal_chain_bytes<2, 2>(p, batch) + align256((size_t)batch * 2 * ne * sizeof(double2));
}

}  // namespace aeolus

using namespace aeolus;

extern "C" int aeolus_vector_curl_div(aeolus_plan plan_ext, double radius, const double* f_en, double* curl,
                                      double* div, int batch, int truncate, void* work, size_t work_bytes,
                                      void* stream) {
  if (!plan_ok(plan_ext)) return fail(AEOLUS_ERR_ARG, "aeolus_vector_curl_div: invalid plan");
  if (batch < 0 || (batch > 0 && (!f_en || !curl || !div)))
    return fail(AEOLUS_ERR_ARG, "aeolus_vector_curl_div: bad arguments");
  if (!(radius > 0.0) || !std::isfinite(radius))
    return fail(AEOLUS_ERR_ARG, "aeolus_vector_curl_div: radius must be finite and > 0");
  if (plan_ext->lmax < 1)
    return fail(AEOLUS_ERR_ARG, "aeolus_vector_curl_div: the extended plan needs l_max >= 1 (state l_max + 1)");
  if (batch == 0) return AEOLUS_OK;
  const size_t need = vector_op_bytes(plan_ext, batch);
  if (!work || work_bytes < need)
    return fail(AEOLUS_ERR_WORKSPACE,
                "aeolus_vector_curl_div: workspace too small (" + std::to_string(need) + " bytes needed)");
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int Le = plan_ext->lmax, L = Le - 1;
  char* w = static_cast<char*>(work);
  double2* ext = reinterpret_cast<double2*>(w);
  w += align256((size_t)batch * 2 * (Le + 1) * (Le + 1) * sizeof(double2));
  const long np = plan_ext->npoints;
  int s = run_anal_chain(plan_ext, PwInvCos{}, EpiStore2{ext, Le}, batch, f_en, 2 * np, np, w, st);
  if (s) return s;
  const long n = (long)(L + 1) * (L + 1) * batch;
  vector_finish_kernel<<<blocks_for(n, 256), 256, 0, st>>>(ext, L, batch, 1.0 / radius, truncate ? 1 : 0,
                                                            reinterpret_cast<double2*>(curl),
                                                            reinterpret_cast<double2*>(div));
  AE_LAUNCH("vector_finish_kernel");
  return AEOLUS_OK;
}
