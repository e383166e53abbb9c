// Plan-kind independent chains:
//   synth chain : Derive -> synthesis -> Pointwise -> grid fields
//   anal chain  : grid fields -> Pointwise -> weighted analysis -> Epilogue
//   full chain  : Derive -> synthesis -> Pointwise -> analysis -> Epilogue
// On a Gauss plan these are the fused Legendre/row kernels; on a point-set
// plan derive_cols -> basis GEMM -> pointwise -> basis^T GEMM -> epilogue.
#pragma once

#include "pipeline.cuh"
#include "points.cuh"
#include "split.cuh"
#include "dense.cuh"

namespace aeolus {

inline unsigned blocks_for(long n, int t) { return (unsigned)((n + t - 1) / t); }

// ---------------------------------------------------------------- sizes
inline bool split_on(const aeolus_plan_impl* p) {
  return p->kind == kGauss && p->precision == AEOLUS_PREC_SPLIT_BF16 && p->split != nullptr;
}
// point-set plan with split-precision (tensor-core) basis products
inline bool dense_on(const aeolus_plan_impl* p) {
  return p->kind == kPoints && p->precision == AEOLUS_PREC_SPLIT_BF16 && p->split != nullptr;
}
inline size_t dense_extra(const aeolus_plan_impl* p, int ncols) { return dense_on(p) ? dense_bytes(p, ncols) : 0; }

// Basis products of a point-set plan (FP64 GEMM or the split-precision
// tensor-core product), see points.cuh / dense.cuh.
inline int points_synth(const aeolus_plan_impl* p, const double* V, double* out, int ncols, void* scratch,
                        cudaStream_t st) {
  if (!dense_on(p)) return points_gemm_synth(p, V, out, ncols, st);
  return dense_split_gemm(p, dense_synth_dims(p, ncols), p->split->bsyn, p->split->ebsyn, V, p->ncol, p->ncol, out,
                          p->npoints, scratch, st, "tc_dense_synth_bf16x6");
}
inline int points_analysis(const aeolus_plan_impl* p, const double* W, double* C, int ncols, void* scratch,
                           cudaStream_t st) {
  if (!dense_on(p)) return points_gemm_analysis(p, W, C, ncols, st);
  return dense_split_gemm(p, dense_anal_dims(p, ncols), p->split->bana, p->split->ebana, W, p->npoints,
                          (int)p->npoints, C, p->ncol, scratch, st, "tc_dense_anal_bf16x6");
}

template <int NIN, int NOUT>
size_t full_chain_bytes(const aeolus_plan_impl* p, int batch) {
  if (split_on(p))  // F blocks, compact G blocks, slicing scratch
    return align256(fg_bytes(p, NIN > NOUT ? NIN : NOUT, batch)) + align256(fg_bytes(p, NOUT, batch)) +
           std::max(split_synth_bytes(p, NIN, batch), split_anal_bytes(p, NOUT, batch));
  if (p->kind == kGauss) return align256(fg_bytes(p, NIN > NOUT ? NIN : NOUT, batch));
  const size_t nc = p->ncol, np = p->npoints;
  return align256((size_t)batch * NIN * nc * 8) + align256((size_t)batch * NIN * np * 8) +
         align256((size_t)batch * NOUT * np * 8) + align256((size_t)batch * NOUT * nc * 8) +
         dense_extra(p, batch * (NIN > NOUT ? NIN : NOUT));
}

template <int NIN, int NOUT>
size_t synth_chain_bytes(const aeolus_plan_impl* p, int batch) {
  if (split_on(p)) return align256(fg_bytes(p, NIN, batch)) + split_synth_bytes(p, NIN, batch);
  if (p->kind == kGauss) return align256(fg_bytes(p, NIN, batch));
  return align256((size_t)batch * NIN * p->ncol * 8) + align256((size_t)batch * NIN * p->npoints * 8) +
         dense_extra(p, batch * NIN);
}

template <int NIN, int NOUT>
size_t anal_chain_bytes(const aeolus_plan_impl* p, int batch) {
  if (split_on(p)) return align256(fg_bytes(p, NOUT, batch)) + split_anal_bytes(p, NOUT, batch);
  if (p->kind == kGauss) return align256(fg_bytes(p, NOUT, batch));
  return align256((size_t)batch * NOUT * p->npoints * 8) + align256((size_t)batch * NOUT * p->ncol * 8) +
         dense_extra(p, batch * NOUT);
}

// ---------------------------------------------------------------- chains
template <class Derive, class Pw, class Epi>
int run_full_chain(const aeolus_plan_impl* p, const Derive& d, const Pw& pw, const Epi& e, int batch,
                   void* work, unsigned* status, cudaStream_t st) {
  static_assert(SynthOut<Derive>::NBLK == Pw::NIN, "derive/pointwise field count");
  static_assert(Pw::NOUT == Epi::NF, "pointwise/epilogue field count");
  if constexpr (SynthOut<Derive>::kLam) {
    // fields formed by the tensor-core synthesis epilogue: split Gauss plans only
    if (!split_on(p)) return fail(AEOLUS_ERR_ARG, "derived-field synthesis needs a split-precision Gauss plan");
    double2* FG = static_cast<double2*>(work);
    constexpr int NB = Pw::NIN > Pw::NOUT ? Pw::NIN : Pw::NOUT;
    double2* G = reinterpret_cast<double2*>(static_cast<char*>(work) + align256(fg_bytes(p, NB, batch)));
    void* scratch = static_cast<char*>(work) + align256(fg_bytes(p, NB, batch)) + align256(fg_bytes(p, Pw::NOUT, batch));
    int s = launch_split_synth(p, d, FG, NB, batch, scratch, st);
    if (s) return s;
    RowArgs ra{};
    ra.batch = batch;
    ra.FG = FG;
    ra.nblk = NB;
    ra.G = G;
    ra.gblk = Pw::NOUT;
    ra.status = status;
    if ((s = launch_rows<Pw, kInF, kOutG>(p, pw, ra, st))) return s;
    return launch_split_anal(p, e, G, Pw::NOUT, batch, scratch, st);
  } else if (p->kind == kGauss) {
    constexpr int NB = Pw::NIN > Pw::NOUT ? Pw::NIN : Pw::NOUT;
    double2* FG = static_cast<double2*>(work);
    const bool split = split_on(p);
    // split path: the row stage writes G into its own compact blocks (NOUT
    // fields), so the analysis slicer reads only G; FP64 path: G overwrites
    // the row's own F blocks
    double2* G = split ? reinterpret_cast<double2*>(static_cast<char*>(work) + align256(fg_bytes(p, NB, batch)))
                       : nullptr;
    void* scratch = static_cast<char*>(work) + align256(fg_bytes(p, NB, batch)) +
                    (split ? align256(fg_bytes(p, Pw::NOUT, batch)) : 0);
    int s = split ? launch_split_synth(p, d, FG, NB, batch, scratch, st) : launch_synth(p, d, FG, NB, batch, st);
    if (s) return s;
    RowArgs ra{};
    ra.batch = batch;
    ra.FG = FG;
    ra.nblk = NB;
    ra.G = G;
    ra.gblk = Pw::NOUT;
    ra.status = status;
    if ((s = launch_rows<Pw, kInF, kOutG>(p, pw, ra, st))) return s;
    return split ? launch_split_anal(p, e, G, Pw::NOUT, batch, scratch, st)
                 : launch_analysis(p, e, FG, NB, batch, st);
  }
  const long nc = p->ncol, np = p->npoints;
  char* w = static_cast<char*>(work);
  double* V = reinterpret_cast<double*>(w);
  w += align256((size_t)batch * Pw::NIN * nc * 8);
  double* Gr = reinterpret_cast<double*>(w);
  w += align256((size_t)batch * Pw::NIN * np * 8);
  double* Wt = reinterpret_cast<double*>(w);
  w += align256((size_t)batch * Pw::NOUT * np * 8);
  double* C = reinterpret_cast<double*>(w);
  w += align256((size_t)batch * Pw::NOUT * nc * 8);
  void* dscratch = w;
  const long nlm = n_coeff(p->lmax) * batch;
  derive_cols_kernel<Derive><<<blocks_for(nlm, 128), 128, 0, st>>>(p->lmax, batch, nc, V, d);
  AE_LAUNCH("derive_cols_kernel");
  int s = points_synth(p, V, Gr, batch * Pw::NIN, dscratch, st);
  if (s) return s;
  points_pointwise_kernel<Pw><<<blocks_for(np * batch, 128), 128, 0, st>>>(
      np, batch, Gr, (long)Pw::NIN * np, np, Wt, (long)Pw::NOUT * np, np, p->coslat, p->fgrid, p->wpts, status, pw);
  AE_LAUNCH("points_pointwise_kernel");
  if ((s = points_analysis(p, Wt, C, batch * Pw::NOUT, dscratch, st))) return s;
  const long n2 = (long)(p->lmax + 1) * (p->lmax + 1) * batch;
  epilogue_cols_kernel<Epi><<<blocks_for(n2, 128), 128, 0, st>>>(p->lmax, batch, nc, C, e);
  AE_LAUNCH("epilogue_cols_kernel");
  return AEOLUS_OK;
}

// Output grid: out[b * out_b + f * out_f + point].
template <class Derive, class Pw>
int run_synth_chain(const aeolus_plan_impl* p, const Derive& d, const Pw& pw, int batch, double* out, long out_b,
                    long out_f, void* work, unsigned* status, cudaStream_t st) {
  static_assert(Derive::NF == Pw::NIN, "derive/pointwise field count");
  if (p->kind == kGauss) {
    double2* FG = static_cast<double2*>(work);
    void* scratch = static_cast<char*>(work) + align256(fg_bytes(p, Pw::NIN, batch));
    int s = split_on(p) ? launch_split_synth(p, d, FG, Pw::NIN, batch, scratch, st)
                        : launch_synth(p, d, FG, Pw::NIN, batch, st);
    if (s) return s;
    RowArgs ra{};
    ra.batch = batch;
    ra.FG = FG;
    ra.nblk = Pw::NIN;
    ra.gout = out;
    ra.gout_b = out_b;
    ra.gout_f = out_f;
    ra.status = status;
    return launch_rows<Pw, kInF, kOutGrid>(p, pw, ra, st);
  }
  const long nc = p->ncol, np = p->npoints;
  char* w = static_cast<char*>(work);
  double* V = reinterpret_cast<double*>(w);
  w += align256((size_t)batch * Pw::NIN * nc * 8);
  double* Gr = reinterpret_cast<double*>(w);
  w += align256((size_t)batch * Pw::NIN * np * 8);
  void* dscratch = w;
  const long nlm = n_coeff(p->lmax) * batch;
  derive_cols_kernel<Derive><<<blocks_for(nlm, 128), 128, 0, st>>>(p->lmax, batch, nc, V, d);
  AE_LAUNCH("derive_cols_kernel");
  const bool direct = Pw::kIdentity && out_b == np;
  int s = points_synth(p, V, direct ? out : Gr, batch * Pw::NIN, dscratch, st);
  if (s || direct) return s;
  points_pointwise_kernel<Pw><<<blocks_for(np * batch, 128), 128, 0, st>>>(
      np, batch, Gr, (long)Pw::NIN * np, np, out, out_b, out_f, p->coslat, p->fgrid, nullptr, status, pw);
  AE_LAUNCH("points_pointwise_kernel");
  return AEOLUS_OK;
}

// Input grid: in[b * in_b + f * in_f + point].  unit_weights drops the
// quadrature weights (the transpose of synthesis instead of the analysis).
template <class Pw, class Epi>
int run_anal_chain(const aeolus_plan_impl* p, const Pw& pw, const Epi& e, int batch, const double* in, long in_b,
                   long in_f, void* work, cudaStream_t st, bool unit_weights = false) {
  static_assert(Pw::NOUT == Epi::NF, "pointwise/epilogue field count");
  if (p->kind == kGauss) {
    double2* FG = static_cast<double2*>(work);
    RowArgs ra{};
    ra.batch = batch;
    ra.FG = FG;
    ra.nblk = Pw::NOUT;
    ra.gin = in;
    ra.gin_b = in_b;
    ra.gin_f = in_f;
    ra.unit_weights = unit_weights ? 1 : 0;
    int s = launch_rows<Pw, kInGrid, kOutG>(p, pw, ra, st);
    if (s) return s;
    if (split_on(p)) {
      void* scratch = static_cast<char*>(work) + align256(fg_bytes(p, Pw::NOUT, batch));
      return launch_split_anal(p, e, FG, Pw::NOUT, batch, scratch, st);
    }
    return launch_analysis(p, e, FG, Pw::NOUT, batch, st);
  }
  const long nc = p->ncol, np = p->npoints;
  char* w = static_cast<char*>(work);
  double* Wt = reinterpret_cast<double*>(w);
  w += align256((size_t)batch * Pw::NOUT * np * 8);
  double* C = reinterpret_cast<double*>(w);
  w += align256((size_t)batch * Pw::NOUT * nc * 8);
  void* dscratch = w;
  points_pointwise_kernel<Pw><<<blocks_for(np * batch, 128), 128, 0, st>>>(
      np, batch, in, in_b, in_f, Wt, (long)Pw::NOUT * np, np, p->coslat, p->fgrid, unit_weights ? nullptr : p->wpts,
      nullptr, pw);
  AE_LAUNCH("points_pointwise_kernel");
  int s = points_analysis(p, Wt, C, batch * Pw::NOUT, dscratch, st);
  if (s) return s;
  const long n2 = (long)(p->lmax + 1) * (p->lmax + 1) * batch;
  epilogue_cols_kernel<Epi><<<blocks_for(n2, 128), 128, 0, st>>>(p->lmax, batch, nc, C, e);
  AE_LAUNCH("epilogue_cols_kernel");
  return AEOLUS_OK;
}

}  // namespace aeolus
