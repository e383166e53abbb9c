// Shared definitions of the sm_103a spectral library: the plan object,
// error plumbing, complex helpers and the packed Legendre-table layout.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <utility>
#include <vector>

#include "../../include/aeolus_gb300.h"

namespace aeolus {

struct FxW;  // fx.cuh

// ---------------------------------------------------------------- errors
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);
#define AE_CUDA(call) do { int _s = ::aeolus::cuda_check((call), #call); if (_s) return _s; } while (0)
#define AE_LAUNCH(what) do { int _s = ::aeolus::cuda_check(cudaGetLastError(), what); if (_s) return _s; } while (0)

// ---------------------------------------- programmatic dependent launch
// The split-precision stage kernels are launched with programmatic stream
// serialisation: a kernel's CTAs may be scheduled while the previous kernel
// in the stream drains (each CTA of a kernel triggers its dependents at its
// start), and every such kernel waits (griddepcontrol.wait) for the previous
// grid to complete, with its memory visible, before it touches global memory
// that grid may read or write.  Only the launch and the CTA prologues
// overlap; a kernel launched without the attribute waits for nothing.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// ------------------------------------------------------------- profiling
// Optional per-kernel CUDA-event timing (aeolus_profile_*).  When enabled,
// every library launch is bracketed by two events on its own stream; the
// elapsed times are summed per kernel name at collection.  Disabled by
// default and never on during stream capture.
bool prof_enabled();
void prof_record(const char* name, cudaEvent_t a, cudaEvent_t b);
cudaEvent_t prof_event();

struct ProfScope {
  const char* name = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t a = nullptr;
  ProfScope(const char* n, cudaStream_t s) {
    // no timing events inside a stream capture (they would become graph nodes)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (prof_enabled() && cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
      name = n;
      st = s;
      a = prof_event();
      cudaEventRecord(a, st);
    }
  }
  ~ProfScope() {
    if (a) {
      cudaEvent_t b = prof_event();
      cudaEventRecord(b, st);
      prof_record(name, a, b);
    }
  }
};

// --------------------------------------------------------------- complex
__host__ __device__ inline double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ inline double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline double2 cscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__host__ __device__ inline double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
// i * a
__host__ __device__ inline double2 ci(double2 a) { return make_double2(-a.y, a.x); }

// --------------------------------------------------------------- layout
// Packed m-major triangle: for order m the degrees l = m..L are contiguous.
// F/G blocks (order spectra of the latitude rows) are [member][order m]
// [latitude row][field], fields fastest: a tensor-core epilogue thread owns
// one row and consecutive fields of one member (whole 32-byte sectors per
// store), and the row stage reads / writes all fields of its row per order
// as one contiguous run.
__host__ __device__ inline long fg_index(long b, int m, int f, int j, int L, int nblk, int nlat) {
  return ((b * (L + 1) + m) * (long)nlat + j) * nblk + f;
}

__host__ __device__ inline long tri_off(int m, int L) { return (long)m * (L + 1) - (long)m * (m - 1) / 2; }
__host__ __device__ inline long n_coeff(int L) { return (long)(L + 1) * (L + 2) / 2; }

constexpr int kMaxFactors = 16;

struct FftInfo {
  int N;            // transform length (nlon)
  int n;            // complex half length N/2 (FFT path) or ceil(N/2) (buffer stride)
  int use_fft;      // 1: half-length complex mixed-radix FFT; 0: direct DFT
  int nfac;
  int fac[kMaxFactors];
  // per stage: 32-bit reciprocals ceil(2^32 / d) of the butterfly count n/r
  // and of the sub-transform length Ls (0 when d = 1); x / d = umulhi(x, .)
  // exactly while x * d < 2^32, which n <= kMaxFftHalf guarantees
  unsigned nbm[kMaxFactors];
  unsigned lsm[kMaxFactors];
};
constexpr int kMaxFftHalf = 8192;

// ------------------------------------------------------------------ plan
enum PlanKind { kGauss = 0, kPoints = 1 };

struct SplitTables;  // split-precision operand slices (split.cu)

struct aeolus_plan_impl {
  int kind = kGauss;
  int nlat = 0, nlon = 0, lmax = 0, nh = 0;
  long npoints = 0;
  double radius = 1.0;
  int precision = AEOLUS_PREC_FP64;
  int slices = 0;
  int device = 0;
  int sm_count = 1;  // streaming multiprocessors of `device` (persistent grids)
  // launch shapes chosen by the autotuner (0: built-in heuristics): members
  // per CTA of the FP64 Legendre synthesis / analysis, threads of the row
  // stage, members per CTA of the split-path slicing kernels
  int tune_bc_synth = 0, tune_bc_anal = 0, tune_row_threads = 0, tune_slice_mb = 0, tune_slice_mb_anal = 0;
  FftInfo fft{};   // FP64 row stage (radix 2..5)
  FftInfo fftx{};  // fixed-point row stage (radix 2..5 and 8, in place)
  // device tables (Gauss)
  double* x = nullptr;       // [nlat] cos(colatitude) = sin(latitude)
  double* wq = nullptr;      // [nlat] w_gl * 2 pi / nlon
  double* coslat = nullptr;  // [nlat] or [npoints], max(cos lat, 1e-8)
  double* fgrid = nullptr;   // [nlat] or [npoints]: synthesis of the unit (1,0) mode
  double* P = nullptr;       // [tri_off(m)*nh + (l-m)*nh + jn]  (row jn fastest)
  double* PT = nullptr;      // [tri_off(m)*nh + jn*(L+1-m) + (l-m)] (degree fastest)
  double2* tw = nullptr;     // [nlon] exp(-2 pi i q / nlon)
  float4* twdf = nullptr;    // [nlon] the same twiddles as double-float (re.hi, re.lo, im.hi, im.lo)
  FxW* twfx = nullptr;       // [nlon] the same twiddles as Q61 31-bit limbs (fixed-point rows)
  int* fft_irev = nullptr;   // [fftx.n] position of natural index q in digit-reversed order (in-place FFTs)
  double* invlap = nullptr;  // [L+1] 1 / (-l(l+1)/R^2), 0 at l = 0 (radius of the plan)
  double* xa = nullptr;      // [(L+1)^2] x Y_lm = xa_lm Y_{l+1,m} + xb_lm Y_{l-1,m}
  double* xb = nullptr;      // [(L+1)^2]
  double* dcoef = nullptr;   // [(L+1)^2][8] SWE derive coefficients at the plan radius (see SweDerive)
  float* dcoef_df = nullptr;  // the same as double-floats: [(L+1)^2][8] (hi, lo) float pairs
  // device tables (points)
  double* basis = nullptr;   // [npoints][ncol] real basis (cos / sin columns)
  double* wpts = nullptr;    // [npoints] quadrature weights
  double* latp = nullptr;    // [npoints]
  int ncol = 0;              // (L+1)^2 real columns
  int ld_basis = 0;
  // shared spectral tables
  double* cplus = nullptr;   // [(L+1)*(L+1)] C+[l][m], C+[L][:] = 0
  double* cminus = nullptr;  // [(L+1)*(L+1)] C-[l][m]
  double* cplus_true = nullptr;
  // host copies
  std::vector<double> h_lat, h_wgl;
  SplitTables* split = nullptr;
};

inline bool plan_ok(const aeolus_plan_impl* p) { return p != nullptr && p->lmax >= 0; }

// Spectral tables (host), identical arithmetic to spectral_operators.py:135-176.
void sin_theta_tables(int L, std::vector<double>& cp, std::vector<double>& cm, bool clip_top);

}  // namespace aeolus

struct aeolus_plan_s : aeolus::aeolus_plan_impl {};
