// Batched uneven ensemble of BVE members: groups of members on Gauss plans
// of different l_max advanced together.  Every RK4 stage launches each stage
// kernel ONCE for all groups (a block-to-group table maps each CTA -- or, in
// the persistent tensor-core kernels, each tile -- to its group), a whole RK4
// step can be captured into a CUDA graph and replayed, and an autotuner times
// candidate launch shapes per group and keeps the fastest.
//
// Reference: the run loop of run/bve/runner.py:211-216 applied to many
// independent states; the reference has no batched or grouped form.
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "models.cuh"

struct aeolus_ensemble_s {
  int ng = 0;
  int model = 0;  // 0: barotropic vorticity, 1: shallow water
  aeolus_plan plan[8] = {};
  int batch[8] = {};
  aeolus_bve_params prm[8] = {};
  aeolus_swe_params sprm[8] = {};
  int split = 0;
  int device = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace aeolus {
namespace {

constexpr int kMaxGroups = 8;

// Per-group block ranges of a grouped launch: CTA b belongs to the group k
// with start[k] <= b < start[k + 1]; inside it, bx = local % gx, by = local / gx.
template <class Arg>
struct Grouped {
  int n;
  int start[kMaxGroups + 1];
  int gx[kMaxGroups];
  int gy[kMaxGroups];
  Arg arg[kMaxGroups];
  __device__ int find(int b) const {
    int k = 0;
    while (k + 1 < n && b >= start[k + 1]) ++k;
    return k;
  }
};

template <class Arg>
void grouped_add(Grouped<Arg>& g, const Arg& a, dim3 grid) {
  const int k = g.n++;
  g.arg[k] = a;
  g.gx[k] = (int)grid.x;
  g.gy[k] = (int)grid.y;
  g.start[k + 1] = g.start[k] + (int)(grid.x * grid.y);
}

template <class Derive>
struct SynthArg {
  LegArgs a;
  Derive d;
};
template <class Epi>
struct AnalArg {
  LegArgs a;
  Epi e;
};
template <class Pw>
struct RowArg {
  RowArgs a;
  Pw pw;
  const FxW* twfx;
  const float4* twdf;
  int kind;  // SplitRowKind of the group's plan (split path)
};
template <class Derive>
struct SliceSynthArg {
  SplitDims dm;
  const long long* kcum;
  int batch, mb;
  Derive d;
  __nv_bfloat16* digits;
  int* ecol;
};
struct SliceAnalArg {
  SplitDims dm;
  int batch, mb, nblk;
  const long long* FG;
  __nv_bfloat16* digits;
  int* ecol;
};

template <class Derive, int CPT>
__global__ void __launch_bounds__(256) g_legendre_synth(Grouped<SynthArg<Derive>> g) {
  const int k = g.find(blockIdx.x);
  const int loc = blockIdx.x - g.start[k];
  legendre_synth_body<Derive, CPT>(g.arg[k].a, g.arg[k].d, loc % g.gx[k], loc / g.gx[k]);
}

template <class Epi>
__global__ void __launch_bounds__(256) g_legendre_analysis(Grouped<AnalArg<Epi>> g) {
  const int k = g.find(blockIdx.x);
  const int loc = blockIdx.x - g.start[k];
  legendre_analysis_body<Epi>(g.arg[k].a, g.arg[k].e, loc % g.gx[k], loc / g.gx[k]);
}

template <class Pw>
__global__ void __launch_bounds__(256) g_rows(Grouped<RowArg<Pw>> g) {
  const int k = g.find(blockIdx.x);
  const int loc = blockIdx.x - g.start[k];
  row_body<Pw, kInF, kOutG>(g.arg[k].a, g.arg[k].pw, loc % g.gx[k], loc / g.gx[k]);
}

// Each group runs the row body its plan's single-plan chains run
// (split_row_kind): the prime-factor and fixed-radix bodies need
// kPfaThreads = kFx8Threads threads, which the launch then uses.
// TH128: the 128-thread launch of groups with fixed row bodies, seven CTAs
// per SM (72 registers; the grouped stage measured 0.391 -> 0.380 ms against
// six); otherwise up to 256 threads (runtime body only), three CTAs per SM.
// The single-plan row kernels stay at six: at seven their own launch is 1 %
// faster but the programmatic-dependent-launch step of the SWE RK4 is 3 %
// slower.
template <class Pw, bool TH128>
__global__ void __launch_bounds__(TH128 ? kPfaThreads : 256, TH128 ? 7 : 3)
    g_rows_fx(Grouped<RowArg<Pw>> g, FxConst kc) {
  pdl_trigger();
  pdl_wait();
  const int k = g.find(blockIdx.x);
  const int loc = blockIdx.x - g.start[k];
  const RowArg<Pw>& r = g.arg[k];
  const int bx = loc % g.gx[k], by = loc / g.gx[k];
  switch (r.kind) {
    case kRowsPfa192: row_pfa_body<Pw, kInF, kOutG, Pfa192>(r.a, r.pw, r.twfx, kc, bx, by); break;
    case kRowsPfa160: row_pfa_body<Pw, kInF, kOutG, Pfa160>(r.a, r.pw, r.twfx, kc, bx, by); break;
    case kRowsPfa96: row_pfa_body<Pw, kInF, kOutG, Pfa96>(r.a, r.pw, r.twfx, kc, bx, by); break;
    case kRowsPfa64: row_pfa_body<Pw, kInF, kOutG, Pfa64>(r.a, r.pw, r.twfx, kc, bx, by); break;
    case kRowsPfa32: row_pfa_body<Pw, kInF, kOutG, Pfa32>(r.a, r.pw, r.twfx, kc, bx, by); break;
    case kRowsFx8R2: row_fx8_body<Pw, kInF, kOutG, 2>(r.a, r.pw, r.twfx, kc, bx, by); break;
    default: row_fx_body<Pw, kInF, kOutG>(r.a, r.pw, r.twfx, r.twdf, kc, bx, by);
  }
}

template <class Derive>
__global__ void __launch_bounds__(256) g_slice_synth(Grouped<SliceSynthArg<Derive>> g) {
  pdl_trigger();
  pdl_wait();
  const int k = g.find(blockIdx.x);
  const int loc = blockIdx.x - g.start[k];
  const SliceSynthArg<Derive>& a = g.arg[k];
  split_synth_slice_body<Derive>(a.dm, a.kcum, a.batch, a.mb, a.d, a.digits, a.ecol, loc % g.gx[k], loc / g.gx[k],
                                 g.gy[k]);
}

template <int NF>
__global__ void __launch_bounds__(256) g_slice_anal(Grouped<SliceAnalArg> g) {
  pdl_trigger();
  pdl_wait();
  const int k = g.find(blockIdx.x);
  const int loc = blockIdx.x - g.start[k];
  const SliceAnalArg& a = g.arg[k];
  split_anal_slice_body<NF>(a.dm, a.batch, a.mb, a.nblk, a.FG, a.digits, a.ecol, loc % g.gx[k], loc / g.gx[k],
                            g.gy[k]);
}

// Persistent tensor-core tiles of all groups in one list.
template <class Sched>
struct GroupedSched {
  static constexpr int kSegChunks = Sched::kSegChunks;
  int n;
  int start[kMaxGroups + 1];
  Sched s[kMaxGroups];
  __device__ int find(int t) const {
    int k = 0;
    while (k + 1 < n && t >= start[k + 1]) ++k;
    return k;
  }
  __device__ int count() const { return start[n]; }
  __device__ TcTile tile(int t) const {
    const int k = find(t);
    return s[k].tile(t - start[k]);
  }
};

template <class Sched, class Epi, bool SEG = (Sched::kSegChunks > 0)>
struct GroupedEpi {
  static constexpr int kWarps = Epi::kWarps, kCols = Epi::kCols;
  GroupedSched<Sched> gs;  // for the tile -> group map
  Epi e[kMaxGroups];
  using Pre = typename Epi::Pre;
  __device__ Pre prefetch(int t, int row, int c0) const {
    const int k = gs.find(t);
    return e[k].prefetch(t - gs.start[k], row, c0);
  }
  template <class Rel>
  __device__ void run(int t, uint32_t tbuf, int q, int row, int c0, int etid, Rel release, const Pre& pre) const {
    const int k = gs.find(t);
    e[k].run(t - gs.start[k], tbuf, q, row, c0, etid, release, pre);
  }
};

// K-segmented epilogues: the per-thread running state is the group-
// independent State of the wrapped epilogue.
template <class Sched, class Epi>
struct GroupedEpi<Sched, Epi, true> {
  static constexpr int kWarps = Epi::kWarps, kCols = Epi::kCols;
  using State = typename Epi::State;
  GroupedSched<Sched> gs;
  Epi e[kMaxGroups];
  __device__ void seg_begin(State& st) const { e[0].seg_begin(st); }
  __device__ void seg_prefetch(State& st, int t, int row, int c0) const {
    const int k = gs.find(t);
    e[k].seg_prefetch(st, t - gs.start[k], row, c0);
  }
  __device__ void seg_add(State& st, uint32_t tbuf, int q, int c0) const { e[0].seg_add(st, tbuf, q, c0); }
  __device__ void seg_end(int t, const State& st, int row, int c0, int etid) const {
    const int k = gs.find(t);
    e[k].seg_end(t - gs.start[k], st, row, c0, etid);
  }
};

// Per-model pieces of a grouped RK4 stage: the functors of the chain and
// the group workspace (chain scratch, stage inputs, RK4 accumulator).
struct BveModel {
  using Derive = BveDerive;
  using SplitDerive = BveDerive;  // the split path's synthesis functor
  static SplitDerive split_derive(const Derive& d) { return d; }
  using Pw = JacPw;
  using Epi = BveEpi;
  static constexpr int NIN = 4, NOUT = 1;
  struct Bufs {
    char* chain;
    double2* ystage;
    double2* acc;
  };
  static size_t bytes(const aeolus_plan_impl* p, int B) {
    return align256(full_chain_bytes<4, 1>(p, B)) + 2 * align256(state_bytes(p, 1, B));
  }
  static Bufs bufs(const aeolus_plan_impl* p, int B, char* base) {
    Bufs b;
    b.chain = base;
    base += align256(full_chain_bytes<4, 1>(p, B));
    b.ystage = reinterpret_cast<double2*>(base);
    base += align256(state_bytes(p, 1, B));
    b.acc = reinterpret_cast<double2*>(base);
    return b;
  }
  // The functors of stage `stage` of group k (BarotropicVorticity.rk4).
  static void make(const aeolus_ensemble_s* E, int k, const Bufs& b, double2* y0, int stage, double dt, Derive& d,
                   Pw& pw, Epi& e) {
    const aeolus_plan_impl* p = E->plan[k];
    const Spec sp = make_spec(p, E->prm[k].radius);
    const double2* in = stage == 1 ? y0 : b.ystage;
    d = BveDerive{sp, in, 2.0 * E->prm[k].omega * kSqrt4PiOver3};
    pw = JacPw{};
    e = BveEpi{sp, in, nullptr, E->prm[k].viscosity, Rk4{stage, dt, y0, b.ystage, b.acc, nullptr}};
  }
};

struct SweModel {
  using Derive = SweDerive;
  // split path: 7 contracted fields, the longitude derivatives formed by the
  // synthesis epilogue (as aeolus_swe_rk4 does)
  using SplitDerive = SweDerive7;
  static SplitDerive split_derive(const Derive& d) { return SweDerive7{d}; }
  using Pw = SwePw;
  using Epi = SweEpi;
  static constexpr int NIN = 9, NOUT = 4;
  struct Bufs {
    char* chain;
    double2* stage[2];
    double2* acc;
    double2* cor;
  };
  static size_t bytes(const aeolus_plan_impl* p, int B) {
    return align256(full_chain_bytes<9, 4>(p, B)) + 3 * align256(state_bytes(p, 3, B)) +
           align256(state_bytes(p, 2, B));
  }
  static Bufs bufs(const aeolus_plan_impl* p, int B, char* base) {
    Bufs b;
    b.chain = base;
    base += align256(full_chain_bytes<9, 4>(p, B));
    for (int i = 0; i < 2; ++i) {
      b.stage[i] = reinterpret_cast<double2*>(base);
      base += align256(state_bytes(p, 3, B));
    }
    b.acc = reinterpret_cast<double2*>(base);
    base += align256(state_bytes(p, 3, B));
    b.cor = reinterpret_cast<double2*>(base);
    return b;
  }
  // The functors of stage `stage` of group k, as in aeolus_swe_rk4: two stage
  // buffers in turn (the epilogue reads neighbouring degrees of its input
  // while writing the next input) and, on the split path, the Coriolis
  // spectra of the stage input added spectrally.
  static void make(const aeolus_ensemble_s* E, int k, const Bufs& b, double2* y0, int stage, double dt, Derive& d,
                   Pw& pw, Epi& e) {
    const aeolus_plan_impl* p = E->plan[k];
    const aeolus_swe_params& q = E->sprm[k];
    const Spec sp = make_spec(p, q.radius);
    const double f10 = 2.0 * q.omega * kSqrt4PiOver3;
    const double phi0 = q.gravity * q.mean_depth;
    const bool spec_cor = p->precision == AEOLUS_PREC_SPLIT_BF16;
    double2* cor = spec_cor ? b.cor : nullptr;
    const double fp = spec_cor ? 0.0 : f10;
    const double2* in = stage == 1 ? y0 : b.stage[stage & 1];
    double2* next = b.stage[(stage + 1) & 1];
    d = SweDerive{sp, in, fp, cor, 2.0 * q.omega};
    pw = SwePw{fp, phi0, (float)phi0};
    e = SweEpi{sp, in, phi0, q.nu4, Rk4{stage, dt, y0, next, b.acc, nullptr}, spec_cor ? 2.0 * q.omega : 0.0, cor};
    e.forcing = reinterpret_cast<const double2*>(q.forcing);
  }
};

size_t group_bytes(const aeolus_ensemble_s* E, int k) {
  return E->model == 1 ? SweModel::bytes(E->plan[k], E->batch[k]) : BveModel::bytes(E->plan[k], E->batch[k]);
}

size_t ens_bytes(const aeolus_ensemble_s* e) {
  size_t n = 0;
  for (int k = 0; k < e->ng; ++k) n += group_bytes(e, k);
  return n;
}

// One RK4 stage of every group: 3 (FP64) or 5 (split) grouped launches.
template <class M>
int ens_stage_m(const aeolus_ensemble_s* E, double2* const* y0, int stage, double dt, char* work, cudaStream_t st) {
  using Derive = typename M::Derive;
  using Pw = typename M::Pw;
  using Epi = typename M::Epi;
  constexpr int NIN = M::NIN, NOUT = M::NOUT, NB = NIN > NOUT ? NIN : NOUT;
  const int ng = E->ng;
  Derive der[kMaxGroups];
  Pw pws[kMaxGroups];
  Epi epi[kMaxGroups];
  char* chain[kMaxGroups];
  char* w = work;
  for (int k = 0; k < ng; ++k) {
    const typename M::Bufs b = M::bufs(E->plan[k], E->batch[k], w);
    w += M::bytes(E->plan[k], E->batch[k]);
    chain[k] = b.chain;
    M::make(E, k, b, y0[k], stage, dt, der[k], pws[k], epi[k]);
  }
  int s;
  // rows (shared by both paths)
  Grouped<RowArg<Pw>> gr{};
  size_t sm_rows = 0;
  int row_thr = 0;
  bool fixed_thr = false;
  for (int k = 0; k < ng; ++k) {
    const aeolus_plan_impl* p = E->plan[k];
    RowArgs ra{};
    ra.batch = E->batch[k];
    ra.FG = reinterpret_cast<double2*>(chain[k]);
    ra.nblk = NB;
    row_args(p, ra);
    if (E->split) ra.fft = p->fftx;
    const int kind = E->split ? split_row_kind(p) : kRowsRuntime;
    const bool pfa = kind >= kRowsPfa192;
    grouped_add(gr, RowArg<Pw>{ra, pws[k], p->twfx, p->twdf, kind},
                pfa ? row_pfa_grid<Pw>(p->nlat, E->batch[k]) : dim3(p->nlat, E->batch[k]));
    sm_rows = std::max(sm_rows, E->split ? split_row_smem_bytes<Pw>(p) : row_smem_bytes<Pw>(p->fft));
    row_thr = std::max(row_thr, row_threads(p));
    if (kind != kRowsRuntime) fixed_thr = true;
  }
  if (fixed_thr) row_thr = kPfaThreads;
  if (!E->split) {
    Grouped<SynthArg<Derive>> gs{};
    Grouped<AnalArg<Epi>> ga{};
    size_t sm_s = 0, sm_a = 0;
    int thr_s = 64, thr_a = 64;
    for (int k = 0; k < ng; ++k) {
      const aeolus_plan_impl* p = E->plan[k];
      double2* FG = reinterpret_cast<double2*>(chain[k]);
      const LegCfg cs = synth_cfg<Derive>(p, E->batch[k]);
      const LegCfg ca = analysis_cfg<Epi>(p, E->batch[k]);
      grouped_add(gs, SynthArg<Derive>{LegArgs{p->lmax, p->nlat, p->nh, E->batch[k], cs.bc, p->P, p->PT, FG, NB},
                                       der[k]},
                  cs.grid);
      grouped_add(ga, AnalArg<Epi>{LegArgs{p->lmax, p->nlat, p->nh, E->batch[k], ca.bc, p->P, p->PT, FG, NB}, epi[k]},
                  ca.grid);
      sm_s = std::max(sm_s, cs.smem);
      sm_a = std::max(sm_a, ca.smem);
      thr_s = std::max(thr_s, cs.threads);
      thr_a = std::max(thr_a, ca.threads);
    }
    auto k1 = g_legendre_synth<Derive, kSynthCPT>;
    auto k2 = g_rows<Pw>;
    auto k3 = g_legendre_analysis<Epi>;
    if ((s = allow_smem(k1, sm_s)) || (s = allow_smem(k2, sm_rows)) || (s = allow_smem(k3, sm_a))) return s;
    {
      ProfScope prof("ens_legendre_synth_f64", st);
      k1<<<gs.start[ng], thr_s, sm_s, st>>>(gs);
      AE_LAUNCH("g_legendre_synth");
    }
    {
      ProfScope prof("ens_rows", st);
      k2<<<gr.start[ng], row_thr, sm_rows, st>>>(gr);
      AE_LAUNCH("g_rows");
    }
    ProfScope prof("ens_legendre_analysis_f64", st);
    k3<<<ga.start[ng], thr_a, sm_a, st>>>(ga);
    AE_LAUNCH("g_legendre_analysis");
    return AEOLUS_OK;
  }
  // split precision
  using SDerive = typename M::SplitDerive;
  constexpr int NS = SDerive::NF;  // contracted fields
  using SEpi = SynthEpi<NS, SynthOut<SDerive>>;
  Grouped<SliceSynthArg<SDerive>> gss{};
  Grouped<SliceAnalArg> gsa{};
  GroupedSched<SynthSched> tsyn{};
  GroupedEpi<SynthSched, SEpi> esyn{};
  GroupedSched<AnalSched> tana{};
  GroupedEpi<AnalSched, AnalEpi<Epi>> eana{};
  size_t sm_ss = 0, sm_sa = 0;
  int sm_count = 1;
  int* err = nullptr;
  for (int k = 0; k < ng; ++k) {
    const aeolus_plan_impl* p = E->plan[k];
    const int B = E->batch[k];
    double2* FG = reinterpret_cast<double2*>(chain[k]);
    void* scratch = chain[k] + align256(fg_bytes(p, NB, B));
    const SplitParts r1 = split_synth_parts<NS>(p, B, scratch);
    const SplitParts r2 = split_anal_parts<NOUT>(p, B, scratch);
    const SDerive sd = M::split_derive(der[k]);
    grouped_add(gss, SliceSynthArg<SDerive>{r1.dm, p->split->kcum, B, r1.mb, sd, r1.digits, r1.ecol}, r1.grid);
    grouped_add(gsa, SliceAnalArg{r2.dm, B, r2.mb, NB, reinterpret_cast<const long long*>(FG), r2.digits, r2.ecol},
                r2.grid);
    sm_ss = std::max(sm_ss, r1.smem);
    sm_sa = std::max(sm_sa, r2.smem);
    const SynthSched sc{r1.dm, p->split->kcum, p->split->psyn, r1.digits};
    tsyn.s[k] = sc;
    tsyn.start[k + 1] = tsyn.start[k] + sc.count_host();
    esyn.e[k] = SEpi{r1.dm, p->split->esyn, r1.ecol, NB, reinterpret_cast<float4*>(FG)};
    esyn.e[k].ir_hi = (float)SynthOut<SDerive>::ir(sd);
    esyn.e[k].ir_lo = (float)(SynthOut<SDerive>::ir(sd) - (double)esyn.e[k].ir_hi);
    const AnalSched sa{r2.dm, p->split->pana, r2.digits};
    tana.s[k] = sa;
    tana.start[k + 1] = tana.start[k] + sa.count_host();
    eana.e[k] = AnalEpi<Epi>{r2.dm, p->split->eana, r2.ecol, B, epi[k]};
    sm_count = std::max(sm_count, p->sm_count);
    err = p->split->err;  // any group's flag: a device error marks every plan's kernels suspect
  }
  tsyn.n = tana.n = ng;
  esyn.gs = tsyn;
  eana.gs = tana;
  auto k1 = g_slice_synth<SDerive>;
  auto k2 = tc_persistent_kernel<GroupedSched<SynthSched>, GroupedEpi<SynthSched, SEpi>>;
  auto k3 = row_thr == kPfaThreads ? g_rows_fx<Pw, true> : g_rows_fx<Pw, false>;
  auto k4 = g_slice_anal<NOUT>;
  auto k5 = tc_persistent_kernel<GroupedSched<AnalSched>, GroupedEpi<AnalSched, AnalEpi<Epi>>>;
  const size_t smt = tc_smem_bytes();
  if ((s = allow_smem(k1, sm_ss)) || (s = allow_smem(k2, smt)) || (s = allow_smem(k3, sm_rows)) ||
      (s = allow_smem(k4, sm_sa)) || (s = allow_smem(k5, smt)))
    return s;
  {
    ProfScope prof("ens_split_synth_slice", st);
    launch_pdl(k1, dim3(gss.start[ng]), dim3(256), sm_ss, st, gss);
    AE_LAUNCH("g_slice_synth");
  }
  {
    ProfScope prof("ens_tc_synth_bf16x6", st);
    launch_pdl(k2, dim3(std::max(1, std::min(tsyn.start[ng], sm_count))),
               dim3(tc_threads<GroupedEpi<SynthSched, SEpi>>()), smt, st, tsyn, esyn, err);
    AE_LAUNCH("tc_persistent_kernel(ensemble synthesis)");
  }
  {
    ProfScope prof("ens_rows_fx", st);
    launch_pdl(k3, dim3(gr.start[ng]), dim3(row_thr), sm_rows, st, gr, fx_consts());
    AE_LAUNCH("g_rows_fx");
  }
  {
    ProfScope prof("ens_split_anal_slice", st);
    launch_pdl(k4, dim3(gsa.start[ng]), dim3(256), sm_sa, st, gsa);
    AE_LAUNCH("g_slice_anal");
  }
  ProfScope prof("ens_tc_anal_bf16x6", st);
  launch_pdl(k5, dim3(std::max(1, std::min(tana.start[ng], sm_count))),
             dim3(tc_threads<GroupedEpi<AnalSched, AnalEpi<Epi>>>()), smt, st, tana, eana, err);
  AE_LAUNCH("tc_persistent_kernel(ensemble analysis)");
  return AEOLUS_OK;
}

int ens_stage(const aeolus_ensemble_s* E, double2* const* y0, int stage, double dt, char* work, cudaStream_t st) {
  return E->model == 1 ? ens_stage_m<SweModel>(E, y0, stage, dt, work, st)
                       : ens_stage_m<BveModel>(E, y0, stage, dt, work, st);
}

int ens_step(const aeolus_ensemble_s* E, double2* const* y0, double dt, char* work, cudaStream_t st) {
  for (int stage = 1; stage <= 4; ++stage) {
    const int s = ens_stage(E, y0, stage, dt, work, st);
    if (s) return s;
  }
  return AEOLUS_OK;
}

bool ens_ok(const aeolus_ensemble_s* e) { return e != nullptr && e->ng > 0 && e->ng <= kMaxGroups; }

void drop_graph(aeolus_ensemble_s* e) {
  if (e->exec) cudaGraphExecDestroy(e->exec);
  if (e->graph) cudaGraphDestroy(e->graph);
  e->exec = nullptr;
  e->graph = nullptr;
}

// Times `reps` RK4 stages (stage 1, which leaves the state untouched) of the
// ensemble on `st`, in ms per stage.
int time_stage(const aeolus_ensemble_s* E, double2* const* y0, char* work, cudaStream_t st, int reps, float* ms) {
  cudaEvent_t a, b;
  AE_CUDA(cudaEventCreate(&a));
  AE_CUDA(cudaEventCreate(&b));
  int s = ens_stage(E, y0, 1, 0.0, work, st);  // warm-up
  if (!s) {
    cudaEventRecord(a, st);
    for (int i = 0; i < reps && !s; ++i) s = ens_stage(E, y0, 1, 0.0, work, st);
    cudaEventRecord(b, st);
  }
  if (!s) s = cuda_check(cudaEventSynchronize(b), "cudaEventSynchronize");
  if (!s) {
    cudaEventElapsedTime(ms, a, b);
    *ms /= reps;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return s;
}

}  // namespace
}  // namespace aeolus

using namespace aeolus;

namespace {

// Shared checks of the two create calls; params_ok(k) validates group k's model parameters.
template <class F>
int ens_create(int model, int ngroups, const aeolus_plan* plans, const int* batch, const char* who, F params_ok,
               aeolus_ensemble* out) {
  if (!out || !plans || !batch || ngroups < 1 || ngroups > kMaxGroups)
    return fail(AEOLUS_ERR_ARG, std::string(who) + ": need 1.." + std::to_string(kMaxGroups) + " groups");
  *out = nullptr;
  int prec = -1, dev = -1;
  for (int k = 0; k < ngroups; ++k) {
    const aeolus_plan_impl* p = plans[k];
    if (!plan_ok(p) || p->kind != kGauss)
      return fail(AEOLUS_ERR_ARG, std::string(who) + ": group " + std::to_string(k) + " needs a Gauss plan");
    if (batch[k] < 1 || batch[k] > 65535)
      return fail(AEOLUS_ERR_ARG, std::string(who) + ": group " + std::to_string(k) + " batch out of range");
    int s = params_ok(k);
    if (s) return s;
    if (prec >= 0 && p->precision != prec)
      return fail(AEOLUS_ERR_ARG, std::string(who) + ": all groups must use the same contraction precision");
    if (dev >= 0 && p->device != dev)
      return fail(AEOLUS_ERR_ARG, std::string(who) + ": all groups must live on one device");
    if (p->precision == AEOLUS_PREC_SPLIT_BF16 && !p->split)
      return fail(AEOLUS_ERR_ARG, std::string(who) + ": split precision without split tables");
    prec = p->precision;
    dev = p->device;
  }
  auto* e = new aeolus_ensemble_s;
  e->ng = ngroups;
  e->model = model;
  for (int k = 0; k < ngroups; ++k) {
    e->plan[k] = plans[k];
    e->batch[k] = batch[k];
  }
  e->split = prec == AEOLUS_PREC_SPLIT_BF16;
  e->device = dev;
  *out = e;
  return AEOLUS_OK;
}

}  // namespace

extern "C" int aeolus_ensemble_create(int ngroups, const aeolus_plan* plans, const int* batch,
                                      const aeolus_bve_params* params, aeolus_ensemble* out) {
  if (!params) return fail(AEOLUS_ERR_ARG, "aeolus_ensemble_create: NULL params");
  int s = ens_create(0, ngroups, plans, batch, "aeolus_ensemble_create",
                     [&](int k) { return bve_check(plans[k], &params[k], "aeolus_ensemble_create"); }, out);
  if (s) return s;
  for (int k = 0; k < ngroups; ++k) (*out)->prm[k] = params[k];
  return AEOLUS_OK;
}

extern "C" int aeolus_ensemble_create_swe(int ngroups, const aeolus_plan* plans, const int* batch,
                                          const aeolus_swe_params* params, aeolus_ensemble* out) {
  if (!params) return fail(AEOLUS_ERR_ARG, "aeolus_ensemble_create_swe: NULL params");
  int s = ens_create(1, ngroups, plans, batch, "aeolus_ensemble_create_swe",
                     [&](int k) { return swe_check(&params[k], "aeolus_ensemble_create_swe"); }, out);
  if (s) return s;
  for (int k = 0; k < ngroups; ++k) (*out)->sprm[k] = params[k];
  return AEOLUS_OK;
}

extern "C" int aeolus_ensemble_destroy(aeolus_ensemble e) {
  if (!e) return AEOLUS_OK;
  drop_graph(e);
  delete e;
  return AEOLUS_OK;
}

extern "C" int aeolus_ensemble_workspace_bytes(aeolus_ensemble e, size_t* bytes) {
  if (!ens_ok(e) || !bytes) return fail(AEOLUS_ERR_ARG, "aeolus_ensemble_workspace_bytes: bad arguments");
  *bytes = std::max<size_t>(ens_bytes(e), 256);
  return AEOLUS_OK;
}

#define ENS_CHECK(who)                                                                                     \
  do {                                                                                                     \
    if (!ens_ok(e) || !zeta) return fail(AEOLUS_ERR_ARG, std::string(who) + ": bad arguments");           \
    for (int k = 0; k < e->ng; ++k)                                                                        \
      if (!zeta[k]) return fail(AEOLUS_ERR_ARG, std::string(who) + ": NULL state of group " + std::to_string(k)); \
    if (!work || work_bytes < ens_bytes(e))                                                                \
      return fail(AEOLUS_ERR_WORKSPACE, std::string(who) + ": workspace too small (" +                    \
                                            std::to_string(ens_bytes(e)) + " bytes needed)");              \
  } while (0)

namespace {

int ens_rk4(aeolus_ensemble e, double* const* zeta, double dt, int nsteps, void* work, size_t work_bytes,
            void* stream, int model, const char* who) {
  ENS_CHECK(who);
  if (e->model != model)
    return fail(AEOLUS_ERR_ARG, std::string(who) + ": the ensemble was created for the other model");
  if (!std::isfinite(dt)) return fail(AEOLUS_ERR_ARG, std::string(who) + ": dt must be finite");
  double2* y[kMaxGroups];
  for (int k = 0; k < e->ng; ++k) y[k] = reinterpret_cast<double2*>(zeta[k]);
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  for (int it = 0; it < nsteps; ++it) {
    const int s = ens_step(e, y, dt, static_cast<char*>(work), st);
    if (s) return s;
  }
  return AEOLUS_OK;
}

}  // namespace

extern "C" int aeolus_ensemble_bve_rk4(aeolus_ensemble e, double* const* zeta, double dt, int nsteps, void* work,
                                       size_t work_bytes, void* stream) {
  return ens_rk4(e, zeta, dt, nsteps, work, work_bytes, stream, 0, "aeolus_ensemble_bve_rk4");
}

extern "C" int aeolus_ensemble_swe_rk4(aeolus_ensemble e, double* const* state, double dt, int nsteps, void* work,
                                       size_t work_bytes, void* stream) {
  return ens_rk4(e, state, dt, nsteps, work, work_bytes, stream, 1, "aeolus_ensemble_swe_rk4");
}

extern "C" int aeolus_ensemble_capture(aeolus_ensemble e, double* const* zeta, double dt, void* work,
                                       size_t work_bytes, void* stream) {
  ENS_CHECK("aeolus_ensemble_capture");
  if (!stream) return fail(AEOLUS_ERR_ARG, "aeolus_ensemble_capture: the legacy default stream cannot be captured");
  if (!std::isfinite(dt)) return fail(AEOLUS_ERR_ARG, "aeolus_ensemble_capture: dt must be finite");
  drop_graph(e);
  double2* y[kMaxGroups];
  for (int k = 0; k < e->ng; ++k) y[k] = reinterpret_cast<double2*>(zeta[k]);
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  // Set every kernel attribute before capturing: a stage-1 pass (which only
  // writes the workspace) runs uncaptured first.
  int s = ens_stage(e, y, 1, dt, static_cast<char*>(work), st);
  if (s) return s;
  AE_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  s = ens_step(e, y, dt, static_cast<char*>(work), st);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(st, &g);
  if (s) {
    if (g) cudaGraphDestroy(g);
    return s;
  }
  if (ce != cudaSuccess) return cuda_check(ce, "cudaStreamEndCapture");
  cudaGraphExec_t x = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&x, g, 0);
  if (ie != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_check(ie, "cudaGraphInstantiate");
  }
  e->graph = g;
  e->exec = x;
  return AEOLUS_OK;
}

extern "C" int aeolus_ensemble_launch(aeolus_ensemble e, int nsteps, void* stream) {
  if (!ens_ok(e) || !e->exec) return fail(AEOLUS_ERR_ARG, "aeolus_ensemble_launch: no captured step");
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  for (int i = 0; i < nsteps; ++i) AE_CUDA(cudaGraphLaunch(e->exec, st));
  return AEOLUS_OK;
}

// Autotuner: per group, candidate members-per-CTA counts of the FP64
// Legendre kernels (or of the split slicing kernels), then the row-stage
// thread count shared by the grouped row launch; each candidate is timed over
// `reps` ensemble stages (stage 1 leaves the states untouched) and the
// fastest kept in the plans.  Results never depend on these shapes.
extern "C" int aeolus_ensemble_autotune(aeolus_ensemble e, double* const* zeta, void* work, size_t work_bytes,
                                        void* stream, char* report, size_t report_len) {
  ENS_CHECK("aeolus_ensemble_autotune");
  drop_graph(e);  // a captured step would keep the old shapes
  double2* y[kMaxGroups];
  for (int k = 0; k < e->ng; ++k) y[k] = reinterpret_cast<double2*>(zeta[k]);
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* w = static_cast<char*>(work);
  const int reps = 3;
  std::string rep;
  char line[256];
  float base = 0.f;
  int s = time_stage(e, y, w, st, reps, &base);
  if (s) return s;
  std::snprintf(line, sizeof(line), "default shapes: %.4f ms per stage\n", base);
  rep += line;
  const int cands[] = {1, 2, 3, 4, 6, 8};
  for (int k = 0; k < e->ng; ++k) {
    aeolus_plan_impl* p = e->plan[k];
    if (!e->split) {
      for (int which = 0; which < 2; ++which) {
        int& knob = which == 0 ? p->tune_bc_synth : p->tune_bc_anal;
        int best_v = knob;
        float best = 1e30f;
        for (int c : cands) {
          if (c > e->batch[k]) break;
          knob = c;
          float ms = 0.f;
          if ((s = time_stage(e, y, w, st, reps, &ms))) return s;
          if (ms < best) {
            best = ms;
            best_v = c;
          }
        }
        knob = best_v;
        std::snprintf(line, sizeof(line), "group %d (l_max %d, %d members): %s members/CTA = %d (%.4f ms)\n", k,
                      p->lmax, e->batch[k], which == 0 ? "synthesis" : "analysis", best_v, best);
        rep += line;
      }
    } else {
      for (int which = 0; which < 2; ++which) {  // synthesis, analysis slicing
        int& knob = which == 0 ? p->tune_slice_mb : p->tune_slice_mb_anal;
        int best_v = knob;
        float best = 1e30f;
        for (int c : cands) {
          knob = c;
          float ms = 0.f;
          if ((s = time_stage(e, y, w, st, reps, &ms))) return s;
          if (ms < best) {
            best = ms;
            best_v = c;
          }
        }
        knob = best_v;
        std::snprintf(line, sizeof(line), "group %d (l_max %d, %d members): %s slicing members/CTA = %d (%.4f ms)\n",
                      k, p->lmax, e->batch[k], which == 0 ? "synthesis" : "analysis", best_v, best);
        rep += line;
      }
    }
  }
  bool fixed_rows = false;  // groups with prime-factor / fixed-radix bodies pin the row stage to their block size
  if (e->split)
    for (int k = 0; k < e->ng; ++k) fixed_rows = fixed_rows || split_row_kind(e->plan[k]) != kRowsRuntime;
  if (fixed_rows) {
    rep += "row stage: 128 threads/CTA (fixed by the prime-factor / fixed-radix row bodies)\n";
  } else {
    const int thr[] = {128, 192, 256};
    int best_v = 256;
    float best = 1e30f;
    for (int t : thr) {
      for (int k = 0; k < e->ng; ++k) e->plan[k]->tune_row_threads = t;
      float ms = 0.f;
      if ((s = time_stage(e, y, w, st, reps, &ms))) return s;
      if (ms < best) {
        best = ms;
        best_v = t;
      }
    }
    for (int k = 0; k < e->ng; ++k) e->plan[k]->tune_row_threads = best_v;
    std::snprintf(line, sizeof(line), "row stage: %d threads/CTA (%.4f ms per stage)\n", best_v, best);
    rep += line;
  }
  if (report && report_len) {
    std::snprintf(report, report_len, "%s", rep.c_str());
  }
  return AEOLUS_OK;
}
