// Plan construction: Gauss-Legendre nodes (FP64 Newton on the device),
// normalised associated-Legendre tables, FFT factorisation and twiddles,
// sin(theta) d/dtheta coupling tables; point-set plans build a dense real
// basis on the device.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>

#include "common.cuh"
#include "fx.cuh"

namespace aeolus {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return AEOLUS_OK;
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return AEOLUS_ERR_CUDA;
}

// C+/C- of spectral_operators.py:135-176, same operation order:
//   C+ = l * sqrt(max((l+1)^2 - m^2, 0) / max((2l+1)(2l+3), 1))
//   C- = -(l+1) * sqrt(max(l^2 - m^2, 0) / max((2l-1)(2l+1), 1))
// zero where m > l; C+[L][:] = 0 when clip_top; C-[0][:] = 0.
void sin_theta_tables(int L, std::vector<double>& cp, std::vector<double>& cm, bool clip_top) {
  const int n = L + 1;
  cp.assign((size_t)n * n, 0.0);
  cm.assign((size_t)n * n, 0.0);
  for (int l = 0; l < n; ++l) {
    for (int m = 0; m <= l; ++m) {
      const double lb = l, mb = m;
      double np = (lb + 1.0) * (lb + 1.0) - mb * mb;
      double dp = (2.0 * lb + 1.0) * (2.0 * lb + 3.0);
      cp[(size_t)l * n + m] = lb * std::sqrt(std::fmax(np, 0.0) / std::fmax(dp, 1.0));
      double nm = lb * lb - mb * mb;
      double dm = (2.0 * lb - 1.0) * (2.0 * lb + 1.0);
      cm[(size_t)l * n + m] = -(lb + 1.0) * std::sqrt(std::fmax(nm, 0.0) / std::fmax(dm, 1.0));
    }
  }
  if (clip_top)
    for (int m = 0; m < n; ++m) cp[(size_t)L * n + m] = 0.0;
  for (int m = 0; m < n; ++m) cm[m] = 0.0;
}

namespace {

struct ProfState {
  std::mutex mu;
  bool enabled = false;
  std::vector<cudaEvent_t> pool;
  struct Pending { std::string name; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  struct Stat { long launches = 0; double ms = 0.0; };
  std::vector<std::pair<std::string, Stat>> stats;
};

ProfState& prof() {
  static ProfState s;
  return s;
}

}  // namespace

bool prof_enabled() { return prof().enabled; }

cudaEvent_t prof_event() {
  ProfState& s = prof();
  std::lock_guard<std::mutex> g(s.mu);
  if (!s.pool.empty()) {
    cudaEvent_t e = s.pool.back();
    s.pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void prof_record(const char* name, cudaEvent_t a, cudaEvent_t b) {
  ProfState& s = prof();
  std::lock_guard<std::mutex> g(s.mu);
  s.pending.push_back({name, a, b});
}

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kInvSqrt4Pi = 0.28209479177387814347;  // 1/sqrt(4 pi)

// Gauss-Legendre nodes and weights by Newton's method in colatitude theta.
// P_n is evaluated with Reinsch's modification of the three-term recurrence
// in u = 1 - x = 2 sin^2(theta/2):
//   d_{k+1} = (k d_k - (2k+1) u P_k) / (k+1),  P_{k+1} = P_k + d_{k+1},
// which keeps full relative precision near the pole where x = cos(theta)
// no longer resolves theta.  With q = n (x P_n - P_{n-1}) = n (d_n - u P_n):
//   d/dtheta P_n(cos theta) = q / sin(theta),  w = 2 sin^2(theta) / q^2.
// Nodes are symmetric by construction; the middle node of an odd rule is
// exactly x = 0.  One thread per northern node.
__device__ void legendre_reinsch(int n, double u, double* pn, double* q) {
  double p = 1.0, d = -u;  // P_1 = x = 1 - u, d_1 = P_1 - P_0
  double pk = 1.0 - u;
  if (n == 0) {
    *pn = 1.0;
    *q = 0.0;
    return;
  }
  p = pk;
  for (int k = 1; k < n; ++k) {
    d = (k * d - (2.0 * k + 1.0) * u * p) / (k + 1.0);
    p += d;
  }
  *pn = p;
  *q = n * (d - u * p);
}

__global__ void gauss_nodes_kernel(int n, double* x, double* sth, double* theta, double* w) {
  const int nh = (n + 1) / 2;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nh) return;
  const bool middle = (n & 1) && j == nh - 1;
  double t = middle ? 0.5 * kPi : kPi * (j + 0.75) / (n + 0.5);
  double pn, q;
  if (!middle) {
    // Newton converges quadratically from this guess (~4 steps); once the
    // step is at the rounding level, one more step polishes the node.
    int polish = -1;
    for (int it = 0; it < 32 && polish != 0; ++it) {
      const double sh = sin(0.5 * t);
      legendre_reinsch(n, 2.0 * sh * sh, &pn, &q);
      const double dt = pn * sin(t) / q;
      t -= dt;
      if (polish > 0) --polish;
      else if (polish < 0 && fabs(dt) <= 1e-15 * t) polish = 1;
    }
  }
  const double sv = middle ? 1.0 : sin(t);
  const double xv = middle ? 0.0 : cos(t);
  const double sh = sin(0.5 * t);
  legendre_reinsch(n, middle ? 1.0 : 2.0 * sh * sh, &pn, &q);
  const double wt = 2.0 * sv * sv / (q * q);
  x[j] = xv;
  x[n - 1 - j] = -xv;
  sth[j] = sv;
  sth[n - 1 - j] = sv;
  theta[j] = t;
  theta[n - 1 - j] = kPi - t;
  w[j] = wt;
  w[n - 1 - j] = wt;
}

// Orthonormal P_lm (Condon-Shortley phase) at the northern nodes, by the
// stable normalised recurrence; writes both packed layouts.
__global__ void legendre_table_kernel(int L, int nh, const double* __restrict__ x, const double* __restrict__ sth,
                                      double* __restrict__ P, double* __restrict__ PT) {
  const int jn = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = blockIdx.y;
  if (jn >= nh || m > L) return;
  const double xv = x[jn];
  const double s = sth[jn];
  double pmm = kInvSqrt4Pi;
  for (int k = 1; k <= m; ++k) pmm = -sqrt((2.0 * k + 1.0) / (2.0 * k)) * s * pmm;
  const long base = tri_off(m, L) * nh;
  const int K = L + 1 - m;
  double* prow = P + base;
  double* pcol = PT + base + (long)jn * K;
  prow[jn] = pmm;
  pcol[0] = pmm;
  if (m == L) return;
  double p2 = pmm;
  double p1 = sqrt(2.0 * m + 3.0) * xv * pmm;
  prow[(long)nh + jn] = p1;
  pcol[1] = p1;
  for (int l = m + 2; l <= L; ++l) {
    const double a = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
    const double b = sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
    const double p = a * (xv * p1 - b * p2);
    prow[(long)(l - m) * nh + jn] = p;
    pcol[l - m] = p;
    p2 = p1;
    p1 = p;
  }
}

// coslat (clamped like spherical_backend.py:72,129) and the synthesis of
// the unit (1,0) mode, sqrt(3/(4 pi)) x, per row.
__global__ void row_metrics_kernel(int n, const double* __restrict__ x, const double* __restrict__ sth,
                                   double* coslat, double* fgrid) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double xv = x[j];
  coslat[j] = fmax(sth[j], 1e-8);
  fgrid[j] = sqrt(3.0) * kInvSqrt4Pi * xv;
}

// exp(-2 pi i q / N) with octant reduction for accuracy.
void twiddles(int N, std::vector<double2>& tw) {
  tw.resize(N);
  for (int q = 0; q < N; ++q) {
    // angle = 2 pi q / N, reduced to the first octant by exact integer
    // quadrant arithmetic when 4 | N.
    double c, s;
    if (N % 4 == 0) {
      int quarter = N / 4;
      int k = q / quarter;
      int r = q - k * quarter;
      double ang = 2.0 * kPi * r / N;
      double cr, sr;
      if (2 * r <= quarter) {
        cr = std::cos(ang);
        sr = std::sin(ang);
      } else {  // use complementary angle pi/2 - ang for better accuracy
        double comp = 2.0 * kPi * (quarter - r) / N;
        cr = std::sin(comp);
        sr = std::cos(comp);
      }
      switch (k & 3) {
        case 0: c = cr; s = sr; break;
        case 1: c = -sr; s = cr; break;
        case 2: c = -cr; s = -sr; break;
        default: c = sr; s = -cr; break;
      }
    } else {
      double ang = 2.0 * kPi * q / N;
      c = std::cos(ang);
      s = std::sin(ang);
    }
    tw[q] = make_double2(c, -s);
  }
}

void plan_fft(int N, int L, FftInfo& f, bool radix8) {
  std::memset(&f, 0, sizeof(f));
  f.N = N;
  f.n = (N + 1) / 2;
  f.use_fft = 0;
  if (N % 2 != 0) return;
  int n = N / 2;
  if (L > n - 1) return;  // Nyquist / aliased orders: direct DFT handles them
  // Radix order: odd radices first, then 2 or 4, then 4s (or 8s with
  // radix8).  A stage with sub-transform length 1 touches shared memory at a
  // stride of its radix, which is free of bank conflicts for an odd radix.
  int rem = n, nf = 0, fac[kMaxFactors];
  int c2 = 0;
  while (rem % 2 == 0) { ++c2; rem /= 2; }
  const int odd[2] = {3, 5};
  for (int r : odd)
    while (rem % r == 0 && nf < kMaxFactors) { fac[nf++] = r; rem /= r; }
  const int big = radix8 ? 3 : 2;  // log2 of the main power-of-two radix
  const int lead = c2 % big;        // leading radix 2 or 4
  if (lead > 0 && nf < kMaxFactors) fac[nf++] = 1 << lead;
  for (int i = 0; i < c2 / big && nf < kMaxFactors; ++i) fac[nf++] = 1 << big;
  if (rem != 1 || nf == kMaxFactors || n > kMaxFftHalf) return;
  f.use_fft = 1;
  f.n = n;
  f.nfac = nf;
  auto recip = [](long long d) { return d == 1 ? 0u : (unsigned)(((1LL << 32) + d - 1) / d); };
  long long ls = 1;
  for (int i = 0; i < nf; ++i) {
    f.fac[i] = fac[i];
    f.nbm[i] = recip(n / fac[i]);
    f.lsm[i] = recip(ls);
    ls *= fac[i];
  }
}

template <class T>
int upload(T** dst, const std::vector<T>& src) {
  AE_CUDA(cudaMalloc(dst, src.size() * sizeof(T)));
  AE_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return AEOLUS_OK;
}

int common_tables(aeolus_plan_impl* p) {
  std::vector<double> inv(p->lmax + 1, 0.0);
  for (int l = 1; l <= p->lmax; ++l) inv[l] = 1.0 / (-(double)l * (l + 1.0) / (p->radius * p->radius));
  int s0 = upload(&p->invlap, inv);
  if (s0) return s0;
  std::vector<double> cp, cm, cpt, dummy;
  sin_theta_tables(p->lmax, cp, cm, true);
  sin_theta_tables(p->lmax, cpt, dummy, false);
  int s;
  if ((s = upload(&p->cplus, cp))) return s;
  if ((s = upload(&p->cminus, cm))) return s;
  if ((s = upload(&p->cplus_true, cpt))) return s;
  // x = cos(colatitude) multiplication coefficients: xa_lm = C+_lm / l
  // (xa_00 = 1/sqrt(3)), xb_lm = -C-_lm / (l + 1), from the unclipped C+.
  const int n = p->lmax + 1;
  std::vector<double> xa((size_t)n * n, 0.0), xb((size_t)n * n, 0.0);
  for (int l = 0; l < n; ++l)
    for (int m = 0; m <= l; ++m) {
      xa[(size_t)l * n + m] = l == 0 ? 0.57735026918962576451 : cpt[(size_t)l * n + m] / l;
      xb[(size_t)l * n + m] = -cm[(size_t)l * n + m] / (l + 1.0);
    }
  if ((s = upload(&p->xa, xa))) return s;
  if ((s = upload(&p->xb, xb))) return s;
  // Combined coefficients of the SWE derive stage at the plan radius, per
  // (l, m): 1/R C+_{l-1} / lap(l-1), 1/R C-_{l+1} / lap(l+1), m/R / lap(l),
  // 1/R C+_{l-1}, 1/R C-_{l+1}, m/R, xa_{l-1}, xb_{l+1} (0 where the neighbour
  // degree is outside m..L, and 1/lap(0) = 0).
  std::vector<double> dc((size_t)n * n * 8, 0.0);
  const double ir = 1.0 / p->radius;
  for (int l = 0; l < n; ++l)
    for (int m = 0; m <= l; ++m) {
      double* c = &dc[((size_t)l * n + m) * 8];
      const bool lo = l >= 1 && l - 1 >= m, hi = l + 1 < n;
      const double cpl = lo ? cp[(size_t)(l - 1) * n + m] : 0.0;
      const double cmh = hi ? cm[(size_t)(l + 1) * n + m] : 0.0;
      c[0] = lo ? ir * cpl * inv[l - 1] : 0.0;
      c[1] = hi ? ir * cmh * inv[l + 1] : 0.0;
      c[2] = m * ir * inv[l];
      c[3] = ir * cpl;
      c[4] = ir * cmh;
      c[5] = m * ir;
      c[6] = lo ? xa[(size_t)(l - 1) * n + m] : 0.0;
      c[7] = hi ? xb[(size_t)(l + 1) * n + m] : 0.0;
    }
  if ((s = upload(&p->dcoef, dc))) return s;
  // as double-floats for the derive of the split path (hi = the nearest
  // float, lo = the nearest float to the remainder)
  std::vector<float> dcf(dc.size() * 2);
  for (size_t i = 0; i < dc.size(); ++i) {
    const float h = static_cast<float>(dc[i]);
    dcf[2 * i] = h;
    dcf[2 * i + 1] = static_cast<float>(dc[i] - static_cast<double>(h));
  }
  if ((s = upload(&p->dcoef_df, dcf))) return s;
  return AEOLUS_OK;
}

void free_plan(aeolus_plan_impl* p) {
  double* bufs[] = {p->x, p->wq, p->coslat, p->fgrid, p->P, p->PT, p->basis, p->wpts,
                    p->latp, p->cplus, p->cminus, p->cplus_true, p->invlap, p->xa, p->xb, p->dcoef};
  for (double* b : bufs)
    if (b) cudaFree(b);
  if (p->dcoef_df) cudaFree(p->dcoef_df);
  if (p->tw) cudaFree(p->tw);
  if (p->twdf) cudaFree(p->twdf);
  if (p->twfx) cudaFree(p->twfx);
  if (p->fft_irev) cudaFree(p->fft_irev);
}

}  // namespace

int allow_smem_raw(const void* kern, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  AE_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> g(mu);
  size_t& have = done[{kern, dev}];
  if (have >= bytes) return AEOLUS_OK;
  AE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  have = bytes;
  return AEOLUS_OK;
}


void free_split(aeolus_plan_impl* p);  // split.cu
int build_points_basis(aeolus_plan_impl* p, const double* lat, const double* lon);  // points.cu

}  // namespace aeolus

using namespace aeolus;

extern "C" const char* aeolus_last_error(void) { return g_last_error.c_str(); }

extern "C" int aeolus_version(void) { return 10000; }

extern "C" int aeolus_profile_enable(int enable) {
  ProfState& s = prof();
  std::lock_guard<std::mutex> g(s.mu);
  s.enabled = enable != 0;
  return AEOLUS_OK;
}

extern "C" int aeolus_profile_collect(char* buf, size_t len) {
  ProfState& s = prof();
  std::lock_guard<std::mutex> g(s.mu);
  for (auto& p : s.pending) {
    float ms = 0.0f;
    cudaError_t e = cudaEventSynchronize(p.b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, p.a, p.b);
    if (e != cudaSuccess) return cuda_check(e, "aeolus_profile_collect");
    auto it = s.stats.begin();
    for (; it != s.stats.end(); ++it)
      if (it->first == p.name) break;
    if (it == s.stats.end()) {
      s.stats.push_back({p.name, {}});
      it = s.stats.end() - 1;
    }
    it->second.launches += 1;
    it->second.ms += ms;
    s.pool.push_back(p.a);
    s.pool.push_back(p.b);
  }
  s.pending.clear();
  std::string out;
  for (auto& kv : s.stats) {
    char line[256];
    std::snprintf(line, sizeof(line), "%s %ld %.6f\n", kv.first.c_str(), kv.second.launches, kv.second.ms);
    out += line;
  }
  if (buf && len) {
    std::snprintf(buf, len, "%s", out.c_str());
    if (out.size() + 1 > len) return fail(AEOLUS_ERR_ARG, "aeolus_profile_collect: buffer too small");
  }
  return AEOLUS_OK;
}

extern "C" int aeolus_profile_reset(void) {
  ProfState& s = prof();
  std::lock_guard<std::mutex> g(s.mu);
  for (auto& p : s.pending) {
    cudaEventSynchronize(p.b);
    s.pool.push_back(p.a);
    s.pool.push_back(p.b);
  }
  s.pending.clear();
  s.stats.clear();
  return AEOLUS_OK;
}

extern "C" int aeolus_plan_create_gauss(int nlat, int nlon, int lmax, double radius, int flags,
                                        aeolus_plan* out) {
  (void)flags;
  if (!out) return fail(AEOLUS_ERR_ARG, "aeolus_plan_create_gauss: out is NULL");
  *out = nullptr;
  if (nlat < 2 || nlon < 4)
    return fail(AEOLUS_ERR_ARG, "GaussLatLonGridGeometry needs nlat >= 2 and nlon >= 4, got (" +
                                    std::to_string(nlat) + ", " + std::to_string(nlon) + ")");
  if (lmax < 0 || lmax > 2047) return fail(AEOLUS_ERR_ARG, "lmax must be in [0, 2047]");
  if (!(radius > 0.0) || !std::isfinite(radius)) return fail(AEOLUS_ERR_ARG, "radius must be finite and > 0");
  auto* p = new aeolus_plan_s();
  p->kind = kGauss;
  p->nlat = nlat;
  p->nlon = nlon;
  p->lmax = lmax;
  p->nh = (nlat + 1) / 2;
  p->npoints = (long)nlat * nlon;
  p->radius = radius;
  cudaGetDevice(&p->device);
  cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, p->device);
  plan_fft(nlon, lmax, p->fft, false);
  plan_fft(nlon, lmax, p->fftx, true);
  int s = AEOLUS_OK;
  auto bail = [&](int st) { free_plan(p); delete p; return st; };
  const int L = lmax, nh = p->nh;
  const long ntab = n_coeff(L) * nh;
  struct Tmp {  // node temporaries, freed on every exit path
    double* p = nullptr;
    ~Tmp() { if (p) cudaFree(p); }
  } t_w, t_s, t_t;
  double *&wgl = t_w.p, *&sth = t_s.p, *&theta = t_t.p;
  if ((s = cuda_check(cudaMalloc(&p->x, nlat * sizeof(double)), "cudaMalloc"))) return bail(s);
  if ((s = cuda_check(cudaMalloc(&wgl, nlat * sizeof(double)), "cudaMalloc"))) return bail(s);
  if ((s = cuda_check(cudaMalloc(&sth, nlat * sizeof(double)), "cudaMalloc"))) return bail(s);
  if ((s = cuda_check(cudaMalloc(&theta, nlat * sizeof(double)), "cudaMalloc"))) return bail(s);
  gauss_nodes_kernel<<<(nh + 127) / 128, 128>>>(nlat, p->x, sth, theta, wgl);
  if ((s = cuda_check(cudaGetLastError(), "gauss_nodes_kernel"))) return bail(s);
  p->h_lat.resize(nlat);
  p->h_wgl.resize(nlat);
  std::vector<double> htheta(nlat);
  s = cuda_check(cudaMemcpy(htheta.data(), theta, nlat * sizeof(double), cudaMemcpyDeviceToHost), "nodes");
  if (!s) s = cuda_check(cudaMemcpy(p->h_wgl.data(), wgl, nlat * sizeof(double), cudaMemcpyDeviceToHost), "weights");
  if (s) return bail(s);
  std::vector<double> hwq(nlat);
  for (int j = 0; j < nlat; ++j) {
    p->h_lat[j] = kPi / 2.0 - htheta[j];        // latlon_grid.py:63-64
    hwq[j] = p->h_wgl[j] * (2.0 * kPi / nlon);  // latlon_grid.py:82
  }
  if ((s = upload(&p->wq, hwq))) return bail(s);
  if ((s = cuda_check(cudaMalloc(&p->coslat, nlat * sizeof(double)), "cudaMalloc"))) return bail(s);
  if ((s = cuda_check(cudaMalloc(&p->fgrid, nlat * sizeof(double)), "cudaMalloc"))) return bail(s);
  row_metrics_kernel<<<(nlat + 127) / 128, 128>>>(nlat, p->x, sth, p->coslat, p->fgrid);
  if ((s = cuda_check(cudaGetLastError(), "row_metrics_kernel"))) return bail(s);
  if ((s = cuda_check(cudaMalloc(&p->P, ntab * sizeof(double)), "cudaMalloc P"))) return bail(s);
  if ((s = cuda_check(cudaMalloc(&p->PT, ntab * sizeof(double)), "cudaMalloc PT"))) return bail(s);
  dim3 g((nh + 63) / 64, L + 1);
  legendre_table_kernel<<<g, 64>>>(L, nh, p->x, sth, p->P, p->PT);
  if ((s = cuda_check(cudaGetLastError(), "legendre_table_kernel"))) return bail(s);
  std::vector<double2> tw;
  twiddles(nlon, tw);
  if ((s = cuda_check(cudaMalloc(&p->tw, nlon * sizeof(double2)), "cudaMalloc tw"))) return bail(s);
  {
    std::vector<float4> twf(nlon);
    for (int q = 0; q < nlon; ++q) {
      const float rh = (float)tw[q].x, ih = (float)tw[q].y;
      twf[q] = make_float4(rh, (float)(tw[q].x - (double)rh), ih, (float)(tw[q].y - (double)ih));
    }
    if ((s = cuda_check(cudaMalloc(&p->twdf, nlon * sizeof(float4)), "cudaMalloc twdf"))) return bail(s);
    if ((s = cuda_check(cudaMemcpy(p->twdf, twf.data(), nlon * sizeof(float4), cudaMemcpyHostToDevice), "twdf")))
      return bail(s);
    std::vector<FxW> twx(nlon);
    for (int q = 0; q < nlon; ++q) {
      const FxK c = fx_const(tw[q].x), sn = fx_const(tw[q].y);
      twx[q] = FxW{c.h, c.l, sn.h, sn.l};
    }
    if ((s = cuda_check(cudaMalloc(&p->twfx, nlon * sizeof(FxW)), "cudaMalloc twfx"))) return bail(s);
    if ((s = cuda_check(cudaMemcpy(p->twfx, twx.data(), nlon * sizeof(FxW), cudaMemcpyHostToDevice), "twfx")))
      return bail(s);
    if (p->fftx.use_fft) {
      // digit reversal of the in-place transforms: position t = t0 + R0 (t1 + R1 (...))
      // holds natural index t0 n/R0 + t1 n/(R0 R1) + ...
      const int n = p->fftx.n;
      std::vector<int> irev(n);
      for (int t = 0; t < n; ++t) {
        int rest = n, q = 0, u = t;
        for (int k = 0; k < p->fftx.nfac; ++k) {
          const int r = p->fftx.fac[k];
          rest /= r;
          q += (u % r) * rest;
          u /= r;
        }
        irev[q] = t;
      }
      if ((s = cuda_check(cudaMalloc(&p->fft_irev, n * sizeof(int)), "cudaMalloc irev"))) return bail(s);
      if ((s = cuda_check(cudaMemcpy(p->fft_irev, irev.data(), n * sizeof(int), cudaMemcpyHostToDevice), "irev")))
        return bail(s);
    }
  }
  if ((s = cuda_check(cudaMemcpy(p->tw, tw.data(), nlon * sizeof(double2), cudaMemcpyHostToDevice), "tw")))
    return bail(s);
  if ((s = common_tables(p))) return bail(s);
  if ((s = cuda_check(cudaDeviceSynchronize(), "plan build"))) return bail(s);
  *out = p;
  return AEOLUS_OK;
}

extern "C" int aeolus_plan_create_points(long n, const double* lat, const double* lon, const double* w,
                                         int lmax, double radius, int flags, aeolus_plan* out) {
  (void)flags;
  if (!out) return fail(AEOLUS_ERR_ARG, "aeolus_plan_create_points: out is NULL");
  *out = nullptr;
  if (n < 1 || !lat || !lon) return fail(AEOLUS_ERR_ARG, "point set needs n >= 1 and lat/lon arrays");
  if (lmax < 0 || lmax > 1023) return fail(AEOLUS_ERR_ARG, "lmax must be in [0, 1023]");
  if (!(radius > 0.0) || !std::isfinite(radius)) return fail(AEOLUS_ERR_ARG, "radius must be finite and > 0");
  auto* p = new aeolus_plan_s();
  p->kind = kPoints;
  p->npoints = n;
  p->lmax = lmax;
  p->radius = radius;
  p->ncol = (lmax + 1) * (lmax + 1);
  cudaGetDevice(&p->device);
  cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, p->device);
  auto bail = [&](int st) { free_plan(p); delete p; return st; };
  std::vector<double> hw(n), hlat(lat, lat + n), hcos(n), hf(n);
  for (long i = 0; i < n; ++i) {
    hw[i] = w ? w[i] : 4.0 * kPi / n;  // fast_geodesic_sh.py:35-39
    hcos[i] = std::fmax(std::cos(lat[i]), 1e-8);
    hf[i] = std::sqrt(3.0) * kInvSqrt4Pi * std::sin(lat[i]);
  }
  int s;
  if ((s = upload(&p->wpts, hw))) return bail(s);
  if ((s = upload(&p->latp, hlat))) return bail(s);
  if ((s = upload(&p->coslat, hcos))) return bail(s);
  if ((s = upload(&p->fgrid, hf))) return bail(s);
  if ((s = build_points_basis(p, lat, lon))) return bail(s);
  if ((s = common_tables(p))) return bail(s);
  if ((s = cuda_check(cudaDeviceSynchronize(), "plan build"))) return bail(s);
  *out = p;
  return AEOLUS_OK;
}

extern "C" int aeolus_plan_destroy(aeolus_plan plan) {
  if (!plan) return AEOLUS_OK;
  free_split(plan);
  free_plan(plan);
  delete plan;
  return AEOLUS_OK;
}

extern "C" int aeolus_plan_info(aeolus_plan plan, int* kind, int* nlat, int* nlon, int* lmax, long* npts) {
  if (!plan) return fail(AEOLUS_ERR_ARG, "plan is NULL");
  if (kind) *kind = plan->kind;
  if (nlat) *nlat = plan->nlat;
  if (nlon) *nlon = plan->nlon;
  if (lmax) *lmax = plan->lmax;
  if (npts) *npts = plan->npoints;
  return AEOLUS_OK;
}

extern "C" int aeolus_plan_nodes(aeolus_plan plan, double* lat, double* w_gl) {
  if (!plan) return fail(AEOLUS_ERR_ARG, "plan is NULL");
  if (plan->kind != kGauss) return fail(AEOLUS_ERR_ARG, "aeolus_plan_nodes needs a Gauss plan");
  if (lat) std::memcpy(lat, plan->h_lat.data(), plan->nlat * sizeof(double));
  if (w_gl) std::memcpy(w_gl, plan->h_wgl.data(), plan->nlat * sizeof(double));
  return AEOLUS_OK;
}
