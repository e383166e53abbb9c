// Public transform and spectral-operator entry points.
#include <mutex>

#include "chains.cuh"

namespace aeolus {

// Fixed device scratch of aeolus_synthesize_noalloc: a file-scope array that
// every GPU loading this library holds until process exit.  Host code must
// not pass the symbol itself to a kernel (on the host it is only a stand-in
// for the device object); the device address comes from
// cudaGetSymbolAddress, looked up once per device.
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mu;
constexpr int kMaxDevices = 64;
void* g_noalloc_addr[kMaxDevices] = {};
}  // namespace

namespace {

// Elementwise spectral operators on the dense [b][L+1][L+1] layout,
// numerics/spectral_operators.py:109-334.  One thread per (b, l, m).
__global__ void spectral_op_kernel(int op, int L, double R, const double2* __restrict__ in, double2* __restrict__ out,
                                   int batch) {
  const long n2 = (long)(L + 1) * (L + 1);
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n2 * batch) return;
  const long b = idx / n2;
  const int r = (int)(idx - b * n2);
  const int l = r / (L + 1), m = r - l * (L + 1);
  const double2* a = in + b * n2;
  double2 v = make_double2(0.0, 0.0);
  if (m <= l) {
    const double lb = l;
    const double lap = -lb * (lb + 1.0) / (R * R);
    switch (op) {
      case 0:  // laplacian_coeffs
        v = cscale(lap, a[r]);
        break;
      case 1: {  // inv_laplacian, l = 0 divided by 1/R^2
        const double d = l == 0 ? 1.0 / (R * R) : lap;
        v = make_double2(a[r].x / d, a[r].y / d);
        break;
      }
      case 2:  // Helmholtz inverse, l = 0 -> 0
        if (l > 0) v = make_double2(a[r].x / lap, a[r].y / lap);
        break;
      case 3: {  // d_lambda_coeffs: (i m / R) a
        const double mr = (double)m / R;
        v = make_double2(-mr * a[r].y, mr * a[r].x);
        break;
      }
      case 4:  // sin_theta_d_theta_coeffs
      case 5: {  // adjoint_sin_theta_d_theta_coeffs
        // C+[l,m] = l sqrt(max((l+1)^2-m^2,0)/max((2l+1)(2l+3),1)), 0 at l = L
        // C-[l,m] = -(l+1) sqrt(max(l^2-m^2,0)/max((2l-1)(2l+1),1)), 0 at l = 0
        auto cplus = [&](int ll) -> double {
          if (ll < m || ll >= L) return 0.0;
          const double x = ll, mb = m;
          return x * sqrt(fmax((x + 1.0) * (x + 1.0) - mb * mb, 0.0) / fmax((2.0 * x + 1.0) * (2.0 * x + 3.0), 1.0));
        };
        auto cminus = [&](int ll) -> double {
          if (ll < m || ll == 0) return 0.0;
          const double x = ll, mb = m;
          return -(x + 1.0) * sqrt(fmax(x * x - mb * mb, 0.0) / fmax((2.0 * x - 1.0) * (2.0 * x + 1.0), 1.0));
        };
        double2 g = make_double2(0.0, 0.0);
        if (op == 4) {
          if (l >= 1) g = cadd(g, cscale(cplus(l - 1), a[(l - 1) * (L + 1) + m]));
          if (l + 1 <= L) g = cadd(g, cscale(cminus(l + 1), a[(l + 1) * (L + 1) + m]));
        } else {
          if (l + 1 <= L) g = cadd(g, cscale(cplus(l), a[(l + 1) * (L + 1) + m]));
          if (l >= 1) g = cadd(g, cscale(cminus(l), a[(l - 1) * (L + 1) + m]));
        }
        v = g;
        break;
      }
      case 6: {  // 2/3-rule truncation of rows and columns
        const int cut = (2 * L) / 3;
        if (l <= cut && m <= cut) v = a[r];
        break;
      }
      default:
        break;
    }
  }
  out[b * n2 + r] = v;
}

}  // namespace

size_t transform_bytes(const aeolus_plan_impl* p, int op, int batch) {
  if (op == AEOLUS_OP_SYNTHESIZE) return synth_chain_bytes<1, 1>(p, batch);
  return anal_chain_bytes<1, 1>(p, batch);
}

}  // namespace aeolus

using namespace aeolus;

extern "C" int aeolus_synthesize(aeolus_plan plan, const double* coeffs, double* grid, int batch, void* work,
                                 size_t work_bytes, void* stream) {
  if (!plan_ok(plan)) return fail(AEOLUS_ERR_ARG, "aeolus_synthesize: invalid plan");
  if (batch < 0 || (batch > 0 && (!coeffs || !grid))) return fail(AEOLUS_ERR_ARG, "aeolus_synthesize: bad arguments");
  if (batch == 0) return AEOLUS_OK;
  const size_t need = transform_bytes(plan, AEOLUS_OP_SYNTHESIZE, batch);
  if (!work || work_bytes < need) return fail(AEOLUS_ERR_WORKSPACE, "aeolus_synthesize: workspace too small");
  const int L = plan->lmax;
  DeriveCopy d{reinterpret_cast<const double2*>(coeffs), L, (long)(L + 1) * (L + 1)};
  return run_synth_chain(plan, d, PwCopy{}, batch, grid, plan->npoints, plan->npoints, work, nullptr,
                         static_cast<cudaStream_t>(stream));
}

extern "C" int aeolus_analyze(aeolus_plan plan, const double* grid, double* coeffs, int batch, void* work,
                              size_t work_bytes, void* stream) {
  if (!plan_ok(plan)) return fail(AEOLUS_ERR_ARG, "aeolus_analyze: invalid plan");
  if (batch < 0 || (batch > 0 && (!coeffs || !grid))) return fail(AEOLUS_ERR_ARG, "aeolus_analyze: bad arguments");
  if (batch == 0) return AEOLUS_OK;
  const size_t need = transform_bytes(plan, AEOLUS_OP_ANALYZE, batch);
  if (!work || work_bytes < need) return fail(AEOLUS_ERR_WORKSPACE, "aeolus_analyze: workspace too small");
  const int L = plan->lmax;
  EpiStore e{reinterpret_cast<double2*>(coeffs), L, (long)(L + 1) * (L + 1)};
  return run_anal_chain(plan, PwCopy{}, e, batch, grid, plan->npoints, plan->npoints, work,
                        static_cast<cudaStream_t>(stream));
}

extern "C" int aeolus_synthesize_noalloc(aeolus_plan plan, const double* coeffs, double* grid, int batch,
                                         void* stream) {
  if (!plan_ok(plan)) return fail(AEOLUS_ERR_ARG, "aeolus_synthesize_noalloc: invalid plan");
  if (batch < 0 || (batch > 0 && (!coeffs || !grid)))
    return fail(AEOLUS_ERR_ARG, "aeolus_synthesize_noalloc: bad arguments");
  if (plan->kind != kGauss || plan->precision != AEOLUS_PREC_FP64)
    return fail(AEOLUS_ERR_ARG, "aeolus_synthesize_noalloc: needs a Gauss plan with the FP64 contraction");
  if (batch == 0) return AEOLUS_OK;
  const size_t need = transform_bytes(plan, AEOLUS_OP_SYNTHESIZE, batch);
  if (need > kNoAllocScratchBytes)
    return fail(AEOLUS_ERR_WORKSPACE, "aeolus_synthesize_noalloc: " + std::to_string(batch) +
                                          " fields need " + std::to_string(need) +
                                          " bytes of scratch, above the fixed 16 MiB; split the batch or use "
                                          "aeolus_synthesize with a caller-provided workspace");
  int dev = -1;
  AE_CUDA(cudaGetDevice(&dev));
  if (dev != plan->device)
    return fail(AEOLUS_ERR_ARG, "aeolus_synthesize_noalloc: the current device is not the plan's device");
  if (dev < 0 || dev >= kMaxDevices) return fail(AEOLUS_ERR_ARG, "aeolus_synthesize_noalloc: device ordinal too large");
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void* addr = nullptr;
      AE_CUDA(cudaGetSymbolAddress(&addr, g_noalloc_scratch));
      g_noalloc_addr[dev] = addr;
    }
    scratch = g_noalloc_addr[dev];
  }
  // The synthesis writes every scratch entry it later reads (all orders of
  // every latitude row), so nothing left by an earlier call needs clearing.
  const int L = plan->lmax;
  DeriveCopy d{reinterpret_cast<const double2*>(coeffs), L, (long)(L + 1) * (L + 1)};
  return run_synth_chain(plan, d, PwCopy{}, batch, grid, plan->npoints, plan->npoints, scratch, nullptr,
                         static_cast<cudaStream_t>(stream));
}

extern "C" int aeolus_spectral_op(int op, int lmax, double radius, const double* in, double* out, int batch,
                                  void* stream) {
  if (op < 0 || op > 6) return fail(AEOLUS_ERR_ARG, "aeolus_spectral_op: unknown op " + std::to_string(op));
  if (lmax < 0 || batch < 0 || !(radius > 0.0)) return fail(AEOLUS_ERR_ARG, "aeolus_spectral_op: bad arguments");
  if (batch == 0) return AEOLUS_OK;
  if (!in || !out) return fail(AEOLUS_ERR_ARG, "aeolus_spectral_op: NULL array");
  if ((op == 4 || op == 5) && in == out)
    return fail(AEOLUS_ERR_ARG, "aeolus_spectral_op: sin(theta) d/dtheta coupling cannot run in place");
  const long n = (long)(lmax + 1) * (lmax + 1) * batch;
  spectral_op_kernel<<<blocks_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      op, lmax, radius, reinterpret_cast<const double2*>(in), reinterpret_cast<double2*>(out), batch);
  AE_LAUNCH("spectral_op_kernel");
  return AEOLUS_OK;
}
