// Launch helpers that chain the three Gauss stages
//   legendre_synth<Derive>  ->  row_kernel<Pointwise>  ->  legendre_analysis<Epilogue>
// and the equivalent point-set chain (points.cu) behind one interface.
#pragma once

#include <algorithm>

#include "common.cuh"
#include "legendre.cuh"
#include "rows.cuh"
#include "rows_fx.cuh"
#include "rows_pfa.cuh"

namespace aeolus {

constexpr int kSynthCPT = 3;

inline int pick_bc(int L, int batch) {
  const long ctas = (long)n_pairs(L) * batch;
  int bc = (int)std::max(1L, std::min(4L, ctas / 608));
  return std::min(bc, std::max(batch, 1));
}

// Raises a kernel's dynamic shared-memory limit once per (kernel, device):
// later calls -- including calls made while a stream is being captured
// into a CUDA graph -- do not touch the function attributes again.
int allow_smem_raw(const void* kern, size_t bytes);  // plan.cu

template <class K>
inline int allow_smem(K kern, size_t bytes) {
  if (bytes <= 48 * 1024) return AEOLUS_OK;
  if (bytes > 227 * 1024) return fail(AEOLUS_ERR_ARG, "shared-memory tile exceeds 227 KB for this size");
  return allow_smem_raw(reinterpret_cast<const void*>(kern), bytes);
}

inline int round_threads(long items, int lo, int hi) {
  long t = (items + 31) / 32 * 32;
  return (int)std::max<long>(lo, std::min<long>(hi, t));
}

// Launch shapes of the three Gauss stages (the autotuner's knobs are the
// plan's tune_* fields; 0 keeps the built-in heuristic).
struct LegCfg {
  int bc;          // members per CTA
  int threads;
  size_t smem;
  dim3 grid;
};

template <class Derive>
LegCfg synth_cfg(const aeolus_plan_impl* p, int batch) {
  const int L = p->lmax;
  int bc = p->tune_bc_synth > 0 ? std::min(p->tune_bc_synth, std::max(batch, 1)) : pick_bc(L, batch);
  while (bc > 1 && synth_smem_bytes<Derive, kSynthCPT>(L, bc) > 200 * 1024) --bc;
  const int ngroups = (bc * Derive::NF + kSynthCPT - 1) / kSynthCPT;
  return LegCfg{bc, round_threads((long)p->nh * ngroups, 64, 256), synth_smem_bytes<Derive, kSynthCPT>(L, bc),
                dim3(n_pairs(L), (batch + bc - 1) / bc)};
}

template <class Epi>
LegCfg analysis_cfg(const aeolus_plan_impl* p, int batch) {
  const int L = p->lmax;
  int bc = p->tune_bc_anal > 0 ? std::min(p->tune_bc_anal, std::max(batch, 1)) : pick_bc(L, batch);
  while (bc > 1 && analysis_smem_bytes<Epi>(p->nh, bc) > 220 * 1024) --bc;
  return LegCfg{bc, round_threads((long)bc * (L + 2), 64, 256), analysis_smem_bytes<Epi>(p->nh, bc),
                dim3(n_pairs(L), (batch + bc - 1) / bc)};
}

inline int row_threads(const aeolus_plan_impl* p) { return p->tune_row_threads > 0 ? p->tune_row_threads : 256; }

template <class Derive>
int launch_synth(const aeolus_plan_impl* p, const Derive& d, double2* FG, int nblk, int batch,
                 cudaStream_t st) {
  const LegCfg c = synth_cfg<Derive>(p, batch);
  LegArgs a{p->lmax, p->nlat, p->nh, batch, c.bc, p->P, p->PT, FG, nblk};
  auto kern = legendre_synth_kernel<Derive, kSynthCPT>;
  int s = allow_smem(kern, c.smem);
  if (s) return s;
  ProfScope prof("legendre_synth_f64", st);
  kern<<<c.grid, c.threads, c.smem, st>>>(a, d);
  AE_LAUNCH("legendre_synth_kernel");
  return AEOLUS_OK;
}

template <class Epi>
int launch_analysis(const aeolus_plan_impl* p, const Epi& e, double2* FG, int nblk, int batch,
                    cudaStream_t st) {
  const LegCfg c = analysis_cfg<Epi>(p, batch);
  LegArgs a{p->lmax, p->nlat, p->nh, batch, c.bc, p->P, p->PT, FG, nblk};
  auto kern = legendre_analysis_kernel<Epi>;
  int s = allow_smem(kern, c.smem);
  if (s) return s;
  ProfScope prof("legendre_analysis_f64", st);
  kern<<<c.grid, c.threads, c.smem, st>>>(a, e);
  AE_LAUNCH("legendre_analysis_kernel");
  return AEOLUS_OK;
}

// Fills the plan-derived fields of a row stage's arguments.
inline void row_args(const aeolus_plan_impl* p, RowArgs& a) {
  a.L = p->lmax;
  a.nlat = p->nlat;
  a.fft = p->fft;
  a.irev = p->fft_irev;
  a.tw = p->tw;
  a.coslat = p->coslat;
  a.fgrid = p->fgrid;
  a.wq = a.unit_weights ? nullptr : p->wq;
}

template <class Pw, int IN_MODE, int OUT_MODE, class FFT>
int launch_rows_fx(const aeolus_plan_impl* p, const Pw& pw, const RowArgs& a, cudaStream_t st) {
  const size_t sm = row_fx_smem_bytes<Pw>(p->fftx);
  auto kern = row_kernel_fx<Pw, IN_MODE, OUT_MODE, FFT>;
  int s = allow_smem(kern, sm);
  if (s) return s;
  ProfScope prof(IN_MODE == kInF ? (OUT_MODE == kOutG ? "rows_fx_c2r_products_r2c" : "rows_fx_c2r") : "rows_fx_r2c",
                 st);
  kern<<<dim3(p->nlat, a.batch), row_threads(p), sm, st>>>(a, pw, p->twfx, p->twdf, fx_consts());
  AE_LAUNCH("row_kernel_fx");
  return AEOLUS_OK;
}

// Fixed radix sequence (R0, 8, 8): compile-time lengths, kFx8Threads threads
// (the plan's row-thread knob does not apply).
template <class Pw, int IN_MODE, int OUT_MODE, int R0>
int launch_rows_fx8(const aeolus_plan_impl* p, const Pw& pw, const RowArgs& a, cudaStream_t st) {
  const size_t sm = row_fx8_smem_bytes<Pw>(R0);
  auto kern = row_kernel_fx8<Pw, IN_MODE, OUT_MODE, R0>;
  int s = allow_smem(kern, sm);
  if (s) return s;
  ProfScope prof(IN_MODE == kInF ? (OUT_MODE == kOutG ? "rows_fx_c2r_products_r2c" : "rows_fx_c2r") : "rows_fx_r2c",
                 st);
  kern<<<dim3(p->nlat, a.batch), kFx8Threads, sm, st>>>(a, pw, p->twfx, fx_consts());
  AE_LAUNCH("row_kernel_fx8");
  return AEOLUS_OK;
}

// nlon = 2 R0 R1 R2: prime-factor transforms (rows_pfa.cuh), kPfaThreads
// threads (the plan's row-thread knob does not apply).
template <class Pw, int IN_MODE, int OUT_MODE, class S>
int launch_rows_pfa(const aeolus_plan_impl* p, const Pw& pw, const RowArgs& a, cudaStream_t st) {
  const size_t sm = row_pfa_smem_bytes<Pw, S>();
  auto kern = row_kernel_pfa<Pw, IN_MODE, OUT_MODE, S>;
  int s = allow_smem(kern, sm);
  if (s) return s;
  ProfScope prof(IN_MODE == kInF ? (OUT_MODE == kOutG ? "rows_fx_c2r_products_r2c" : "rows_fx_c2r") : "rows_fx_r2c",
                 st);
  launch_pdl(kern, row_pfa_grid<Pw>(p->nlat, a.batch), dim3(kPfaThreads), sm, st, a, pw,
             static_cast<const FxW*>(p->twfx), fx_consts());
  AE_LAUNCH("row_kernel_pfa");
  return AEOLUS_OK;
}

// Row-stage body of the split-precision path for a plan: every caller (the
// single-plan chains and the grouped ensemble kernels) picks the same one,
// so a plan's results do not depend on the route.
enum SplitRowKind {
  kRowsRuntime = 0,  // runtime radix sequence (row_fx_body)
  kRowsFx8R2,        // nlon 256: 2 x 8 x 8 Cooley-Tukey (row_fx8_body)
  kRowsPfa192,       // nlon 384: prime-factor 3 x (8 x 8)
  kRowsPfa160,       // nlon 320: 5 x (4 x 8)
  kRowsPfa96,        // nlon 192: 3 x (4 x 8)
  kRowsPfa64,        // nlon 128: 8 x 8
  kRowsPfa32,        // nlon 64: 4 x 8
};
inline int split_row_kind(const aeolus_plan_impl* p) {
  const FftInfo& f = p->fftx;
  if (Pfa192::matches(f)) return kRowsPfa192;
  if (Pfa160::matches(f)) return kRowsPfa160;
  if (Pfa96::matches(f)) return kRowsPfa96;
  if (Pfa64::matches(f)) return kRowsPfa64;
  if (Pfa32::matches(f)) return kRowsPfa32;
  if (FftFixed<2, 8, 8>::matches(f)) return kRowsFx8R2;
  return kRowsRuntime;
}
template <class Pw>
size_t split_row_smem_bytes(const aeolus_plan_impl* p) {
  switch (split_row_kind(p)) {
    case kRowsPfa192: return row_pfa_smem_bytes<Pw, Pfa192>();
    case kRowsPfa160: return row_pfa_smem_bytes<Pw, Pfa160>();
    case kRowsPfa96: return row_pfa_smem_bytes<Pw, Pfa96>();
    case kRowsPfa64: return row_pfa_smem_bytes<Pw, Pfa64>();
    case kRowsPfa32: return row_pfa_smem_bytes<Pw, Pfa32>();
    case kRowsFx8R2: return row_fx8_smem_bytes<Pw>(2);
    default: return row_fx_smem_bytes<Pw>(p->fftx);
  }
}

template <class Pw, int IN_MODE, int OUT_MODE>
int launch_rows(const aeolus_plan_impl* p, const Pw& pw, RowArgs a, cudaStream_t st) {
  row_args(p, a);
  dim3 grid(p->nlat, a.batch);
  const int threads = row_threads(p);
  if (p->precision == AEOLUS_PREC_SPLIT_BF16) {
    // split-precision path: fixed-point FFTs, double-float products; every
    // row stage gets kernels compiled for the common radix sequences
    a.fft = p->fftx;
    switch (split_row_kind(p)) {
      case kRowsPfa192: return launch_rows_pfa<Pw, IN_MODE, OUT_MODE, Pfa192>(p, pw, a, st);
      case kRowsPfa160: return launch_rows_pfa<Pw, IN_MODE, OUT_MODE, Pfa160>(p, pw, a, st);
      case kRowsPfa96: return launch_rows_pfa<Pw, IN_MODE, OUT_MODE, Pfa96>(p, pw, a, st);
      case kRowsPfa64: return launch_rows_pfa<Pw, IN_MODE, OUT_MODE, Pfa64>(p, pw, a, st);
      case kRowsPfa32: return launch_rows_pfa<Pw, IN_MODE, OUT_MODE, Pfa32>(p, pw, a, st);
      case kRowsFx8R2: return launch_rows_fx8<Pw, IN_MODE, OUT_MODE, 2>(p, pw, a, st);
      default: return launch_rows_fx<Pw, IN_MODE, OUT_MODE, FftRuntime>(p, pw, a, st);
    }
  }
  const size_t sm = row_smem_bytes<Pw>(p->fft);
  auto kern = row_kernel<Pw, IN_MODE, OUT_MODE>;
  int s = allow_smem(kern, sm);
  if (s) return s;
  ProfScope prof(IN_MODE == kInF ? (OUT_MODE == kOutG ? "rows_c2r_products_r2c" : "rows_c2r") : "rows_r2c", st);
  kern<<<grid, threads, sm, st>>>(a, pw);
  AE_LAUNCH("row_kernel");
  return AEOLUS_OK;
}

// Bytes of the F/G block area for `nblk` fields per (member, row).
inline size_t fg_bytes(const aeolus_plan_impl* p, int nblk, int batch) {
  return (size_t)batch * p->nlat * nblk * (p->lmax + 1) * sizeof(double2);
}

inline size_t align256(size_t x) { return (x + 255) / 256 * 256; }

}  // namespace aeolus
