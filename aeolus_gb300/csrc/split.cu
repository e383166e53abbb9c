// Split-precision Legendre contraction on tcgen05 tensor cores.
//
// Both operands of every per-order contraction are cut into balanced
// base-256 digits: with a per-row (basis) or per-column (data) exponent E,
//   X = rint(x * 2^(48-E)) = sum_{s=1..6} d_s 256^(6-s),  |d_s| <= 128,
// so each digit is exact in bf16.  The digit products of level k = s + t
// (k = 2..7, 21 (s,t) pairs) are accumulated in one f32 TMEM accumulator
// per level; every partial sum is an integer below pairs*K*2^14 <= 6*K*2^14
// < 2^24 for K <= 160, so the tensor-core accumulation is exact (analysis
// over 192 latitudes runs two K segments).  The data digit slices sit side
// by side along the MMA's N dimension, so basis slice s meets data slices
// 0..6-s in one MMA whose output columns are the level accumulators s..7.
// The levels are recombined in 64-bit integers, T = sum_k I_k 256^(7-k),
// and one conversion gives the FP64 result T * 2^(E_row + E_col - 56).
// Dropped levels k >= 8 bound the error near 2^-48 of max|P| max|a| per
// term.
//
// Synthesis GEMM (per order m):   F[j, n] = sum_l P_lm(x_j) a[l, n]
//   A = basis digits  (128 latitude rows x Kpad degrees, K-major)
//   B = data digits   (32 data columns x 6 slices x Kpad degrees, K-major)
// Analysis GEMM (per order m):    a[l, n] = sum_j P_lm(x_j) G[j, n]
//   A = basis digits  (128 degree rows x NK latitudes)
//   B = data digits   (32 data columns x 6 slices x NK latitudes)
// Data columns are (member, field, re/im).  Operand chunks stream through a
// 6-stage TMA bulk-copy pipeline of the persistent kernel (split.cuh).
#include <algorithm>
#include <vector>

#include "chains.cuh"
#include "split.cuh"

namespace aeolus {

void free_split(aeolus_plan_impl* p) {
  if (!p->split) return;
  SplitTables* t = p->split;
  if (t->psyn) cudaFree(t->psyn);
  if (t->pana) cudaFree(t->pana);
  if (t->esyn) cudaFree(t->esyn);
  if (t->eana) cudaFree(t->eana);
  if (t->kcum) cudaFree(t->kcum);
  if (t->err) cudaFree(t->err);
  if (t->bsyn) cudaFree(t->bsyn);
  if (t->bana) cudaFree(t->bana);
  if (t->ebsyn) cudaFree(t->ebsyn);
  if (t->ebana) cudaFree(t->ebana);
  delete t;
  p->split = nullptr;
}

namespace {

// Basis digit tables.  Synthesis: one thread per (m, latitude row).
__global__ void split_psyn_kernel(int L, int nlat, int nh, int Mt, const double* __restrict__ P,
                                  const long long* __restrict__ kcum, __nv_bfloat16* __restrict__ out,
                                  int* __restrict__ eout) {
  const int m = blockIdx.y;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (m > L || j >= Mt * 128) return;
  const int K = L + 1 - m, Kp = kpad(K);
  const int mt = j / 128, r = j % 128;
  __nv_bfloat16* blk = out + psyn_tile(kcum, Mt, m, mt, Kp);
  if (j >= nlat) {
    for (int t = 0; t < Kp; ++t)
      for (int s = 0; s < kSlices; ++s) blk[tile_elem(128, s, r, t)] = __float2bfloat16(0.0f);
    eout[m * Mt * 128 + j] = 0;
    return;
  }
  const bool south = j >= nh;
  const int jn = south ? nlat - 1 - j : j;
  const double* Pm = P + tri_off(m, L) * nh + jn;
  unsigned long long mx = 0ull;
  for (int t = 0; t < K; ++t) mx = max(mx, abs_key(Pm[(long)t * nh]));
  const int E = exponent_for_key(mx);
  eout[m * Mt * 128 + j] = E;
  for (int t = 0; t < Kp; ++t) {
    double v = 0.0;
    if (t < K) v = Pm[(long)t * nh] * ((south && (t & 1)) ? -1.0 : 1.0);
    __nv_bfloat16 d[kSlices];
    digits(v, E, d);
    for (int s = 0; s < kSlices; ++s) blk[tile_elem(128, s, r, t)] = d[s];
  }
}

// Analysis: one thread per (row tile, degree row); row tile rt holds
// degrees m + 128 mt + r of order m (ana_row_tile).
__global__ void split_pana_kernel(int L, int nlat, int nh, int NK, const double* __restrict__ P,
                                  __nv_bfloat16* __restrict__ out, int* __restrict__ eout) {
  const int rt = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (rt >= ana_row_tiles(L) || r >= 128) return;
  int m, mt;
  ana_row_tile(L, rt, m, mt);
  const int K = L + 1 - m;
  const int t = mt * 128 + r;  // degree offset l - m
  __nv_bfloat16* blk = out + pana_tile(NK, rt);
  const double* Pm = P + tri_off(m, L) * nh + (long)t * nh;
  unsigned long long mx = 0ull;
  if (t < K)
    for (int jn = 0; jn < nh; ++jn) mx = max(mx, abs_key(Pm[jn]));
  const int E = t < K ? exponent_for_key(mx) : 0;
  eout[rt * 128 + r] = E;
  for (int j = 0; j < NK; ++j) {
    double v = 0.0;
    if (t < K && j < nlat) {
      const bool south = j >= nh;
      v = Pm[south ? nlat - 1 - j : j] * ((south && (t & 1)) ? -1.0 : 1.0);
    }
    __nv_bfloat16 d[kSlices];
    digits(v, E, d);
    for (int s = 0; s < kSlices; ++s) blk[tile_elem(128, s, r, j)] = d[s];
  }
}

// Point-set basis digits, synthesis role (rows = points, K = the ncol real
// columns).  The basis is column-major (point fastest): per-point maxima
// with one thread per point, then the digits over a (point tile, 8-chunk
// group) grid, coalesced along the points.
__global__ void dense_rowmax_kernel(long np, int ncol, const double* __restrict__ B, int* __restrict__ eout) {
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long npad = (np + 127) / 128 * 128;
  if (p >= npad) return;
  unsigned long long mx = 0ull;
  if (p < np)
    for (int c = 0; c < ncol; ++c) mx = max(mx, abs_key(B[(long)c * np + p]));
  eout[p] = p < np ? exponent_for_key(mx) : 0;
}

__global__ void dense_bsyn_kernel(long np, int ncol, int nkc, const double* __restrict__ B,
                                  const int* __restrict__ erow, __nv_bfloat16* __restrict__ out) {
  const long p = (long)blockIdx.x * 128 + threadIdx.x;  // 128 threads = one point tile
  const int E = erow[p];
  __nv_bfloat16* tile = out + (long long)blockIdx.x * nkc * chunk_elems(128);
  const int c0 = blockIdx.y * 8 * kKC, c1 = min(nkc * kKC, c0 + 8 * kKC);
  for (int c = c0; c < c1; ++c) {
    __nv_bfloat16 d[kSlices];
    digits((p < np && c < ncol) ? B[(long)c * np + p] : 0.0, E, d);
    for (int s = 0; s < kSlices; ++s) tile[tile_elem(128, s, threadIdx.x, c)] = d[s];
  }
}

// Analysis role (rows = basis columns, K = points): one CTA per (padded)
// column.
__global__ void __launch_bounds__(256) dense_bana_kernel(long np, int ncol, int nkc, const double* __restrict__ B,
                                                         __nv_bfloat16* __restrict__ out, int* __restrict__ eout) {
  __shared__ unsigned long long s_mx[8];
  __shared__ int s_e;
  const int c = blockIdx.x;
  const double* col = B + (long)c * np;
  unsigned long long mx = 0ull;
  if (c < ncol)
    for (long p = threadIdx.x; p < np; p += blockDim.x) mx = max(mx, abs_key(col[p]));
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) s_mx[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m2 = 0ull;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m2 = max(m2, s_mx[w]);
    s_e = c < ncol ? exponent_for_key(m2) : 0;
    eout[c] = s_e;
  }
  __syncthreads();
  const int E = s_e;
  __nv_bfloat16* tile = out + (long long)(c / 128) * nkc * chunk_elems(128);
  for (long p = threadIdx.x; p < (long)nkc * kKC; p += blockDim.x) {
    __nv_bfloat16 d[kSlices];
    digits((c < ncol && p < np) ? col[p] : 0.0, E, d);
    for (int s = 0; s < kSlices; ++s) tile[tile_elem(128, s, c % 128, (int)p)] = d[s];
  }
}

int split_build_points(aeolus_plan_impl* p) {
  auto* t = new SplitTables();
  p->split = t;
  t->L = p->lmax;
  const long np = p->npoints;
  const int ncol = p->ncol;
  const long mp = (np + 127) / 128, mc = (ncol + 127) / 128;
  const long nkc_s = (ncol + kKC - 1) / kKC, nkc_a = (np + kKC - 1) / kKC;
  AE_CUDA(cudaMalloc(&t->bsyn, (size_t)mp * nkc_s * chunk_elems(128) * sizeof(__nv_bfloat16)));
  AE_CUDA(cudaMalloc(&t->bana, (size_t)mc * nkc_a * chunk_elems(128) * sizeof(__nv_bfloat16)));
  AE_CUDA(cudaMalloc(&t->ebsyn, (size_t)mp * 128 * sizeof(int)));
  AE_CUDA(cudaMalloc(&t->ebana, (size_t)mc * 128 * sizeof(int)));
  AE_CUDA(cudaMalloc(&t->err, sizeof(int)));
  AE_CUDA(cudaMemset(t->err, 0, sizeof(int)));
  dense_rowmax_kernel<<<(unsigned)mp, 128>>>(np, ncol, p->basis, t->ebsyn);
  AE_LAUNCH("dense_rowmax_kernel");
  dense_bsyn_kernel<<<dim3((unsigned)mp, (unsigned)((nkc_s + 7) / 8)), 128>>>(np, ncol, (int)nkc_s, p->basis, t->ebsyn,
                                                                             t->bsyn);
  AE_LAUNCH("dense_bsyn_kernel");
  dense_bana_kernel<<<(unsigned)(mc * 128), 256>>>(np, ncol, (int)nkc_a, p->basis, t->bana, t->ebana);
  AE_LAUNCH("dense_bana_kernel");
  AE_CUDA(cudaDeviceSynchronize());
  return AEOLUS_OK;
}

}  // namespace

int split_build(aeolus_plan_impl* p) {
  if (p->split) return AEOLUS_OK;
  if (p->kind == kPoints) return split_build_points(p);
  const int L = p->lmax;
  if (L > kMaxL) return fail(AEOLUS_ERR_ARG, "split precision supports l_max <= 159 (exact f32 synthesis segments)");
  if (p->nlat > 192) return fail(AEOLUS_ERR_ARG, "split precision supports nlat <= 192 (exact f32 accumulation)");
  auto* t = new SplitTables();
  p->split = t;
  t->L = L;
  t->nlat = p->nlat;
  t->nh = p->nh;
  t->NK = kpad(p->nlat);
  t->Mt = (p->nlat + 127) / 128;
  t->h_kcum.assign(L + 2, 0);
  for (int m = 0; m <= L; ++m) t->h_kcum[m + 1] = t->h_kcum[m] + kpad(L + 1 - m);
  const size_t nsyn = (size_t)t->h_kcum[L + 1] * t->Mt * kSlices * 128;
  const size_t nana = (size_t)ana_row_tiles(L) * kSlices * 128 * t->NK;
  AE_CUDA(cudaMalloc(&t->kcum, (L + 2) * sizeof(long long)));
  AE_CUDA(cudaMemcpy(t->kcum, t->h_kcum.data(), (L + 2) * sizeof(long long), cudaMemcpyHostToDevice));
  AE_CUDA(cudaMalloc(&t->psyn, nsyn * sizeof(__nv_bfloat16)));
  AE_CUDA(cudaMalloc(&t->pana, nana * sizeof(__nv_bfloat16)));
  AE_CUDA(cudaMalloc(&t->esyn, (size_t)(L + 1) * t->Mt * 128 * sizeof(int)));
  AE_CUDA(cudaMalloc(&t->eana, (size_t)ana_row_tiles(L) * 128 * sizeof(int)));
  AE_CUDA(cudaMalloc(&t->err, sizeof(int)));
  AE_CUDA(cudaMemset(t->err, 0, sizeof(int)));
  split_psyn_kernel<<<dim3((t->Mt * 128 + 127) / 128, L + 1), 128>>>(L, p->nlat, p->nh, t->Mt, p->P, t->kcum, t->psyn,
                                                                      t->esyn);
  AE_LAUNCH("split_psyn_kernel");
  split_pana_kernel<<<dim3(1, ana_row_tiles(L)), 128>>>(L, p->nlat, p->nh, t->NK, p->P, t->pana, t->eana);
  AE_LAUNCH("split_pana_kernel");
  AE_CUDA(cudaDeviceSynchronize());
  return AEOLUS_OK;
}

// One thread waits on an mbarrier phase that nothing completes: the bounded
// wait must give up after `limit_ns` and report it.  The phase is then
// completed by the waiter itself, so the kernel leaves nothing pending.
__global__ void mbar_timeout_selftest_kernel(unsigned long long limit_ns, int* timed_out,
                                             unsigned long long* elapsed_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
    const uint64_t t0 = tc::globaltimer_ns();
    const bool ok = tc::mbar_wait(&bar, 0, limit_ns);
    *elapsed_ns = tc::globaltimer_ns() - t0;
    *timed_out = ok ? 0 : 1;
    tc::mbar_arrive(&bar);
  }
}

// The FP64 <-> double-float conversions of the split path on n values:
// out[3i] = hi, out[3i+1] = lo of df_of_f64(x[i]) (as FP64, exactly),
// out[3i+2] = f64_of_df of that double-float.
__global__ void df_convert_selftest_kernel(const double* __restrict__ x, int n, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const df v = df_of_f64(x[i]);
  out[3 * i] = f64_of_f32(v.hi);
  out[3 * i + 1] = f64_of_f32(v.lo);
  out[3 * i + 2] = f64_of_df(v);
}

}  // namespace aeolus

using namespace aeolus;

extern "C" int aeolus_selftest_df_convert(const double* x, int n, double* out, void* stream) {
  if (n < 0 || (n > 0 && (!x || !out))) return fail(AEOLUS_ERR_ARG, "aeolus_selftest_df_convert: bad arguments");
  if (n == 0) return AEOLUS_OK;
  df_convert_selftest_kernel<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(x, n, out);
  AE_LAUNCH("df_convert_selftest_kernel");
  return AEOLUS_OK;
}

extern "C" int aeolus_selftest_wait_timeout(unsigned long long limit_ns, int* timed_out,
                                            unsigned long long* elapsed_ns) {
  if (!timed_out || !elapsed_ns || limit_ns == 0 || limit_ns > 10000000000ull)
    return fail(AEOLUS_ERR_ARG, "aeolus_selftest_wait_timeout: bad arguments (limit in (0, 10 s])");
  int* d_flag = nullptr;
  unsigned long long* d_ns = nullptr;
  AE_CUDA(cudaMalloc(&d_flag, sizeof(int)));
  cudaError_t e = cudaMalloc(&d_ns, sizeof(unsigned long long));
  if (e == cudaSuccess) {
    mbar_timeout_selftest_kernel<<<1, 32>>>(limit_ns, d_flag, d_ns);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(timed_out, d_flag, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(elapsed_ns, d_ns, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  }
  cudaFree(d_flag);
  if (d_ns) cudaFree(d_ns);
  if (e != cudaSuccess) return fail(AEOLUS_ERR_CUDA, std::string("aeolus_selftest_wait_timeout: ") + cudaGetErrorString(e));
  return AEOLUS_OK;
}

extern "C" int aeolus_plan_device_error(aeolus_plan plan, int* flag) {
  if (!plan || !flag) return fail(AEOLUS_ERR_ARG, "aeolus_plan_device_error: bad arguments");
  *flag = 0;
  if (!plan->split) return AEOLUS_OK;
  AE_CUDA(cudaMemcpy(flag, plan->split->err, sizeof(int), cudaMemcpyDeviceToHost));
  return AEOLUS_OK;
}

extern "C" int aeolus_plan_set_precision(aeolus_plan plan, int precision, int slices) {
  if (!plan) return fail(AEOLUS_ERR_ARG, "aeolus_plan_set_precision: plan is NULL");
  if (precision == AEOLUS_PREC_FP64) {
    plan->precision = precision;
    plan->slices = 0;
    return AEOLUS_OK;
  }
  if (precision != AEOLUS_PREC_SPLIT_BF16)
    return fail(AEOLUS_ERR_ARG, "aeolus_plan_set_precision: unknown precision mode");
  if (slices != 0 && slices != kSlices)
    return fail(AEOLUS_ERR_ARG, "aeolus_plan_set_precision: this build uses 6 bf16 slices per operand");
  const int s = split_build(plan);
  if (s) return s;
  plan->precision = precision;
  plan->slices = kSlices;
  return AEOLUS_OK;
}

extern "C" int aeolus_plan_set_tuning(aeolus_plan plan, const int* knobs) {
  if (!plan_ok(plan) || !knobs) return fail(AEOLUS_ERR_ARG, "aeolus_plan_set_tuning: bad arguments");
  if (knobs[0] < 0 || knobs[1] < 0 || knobs[3] < 0 || knobs[4] < 0 || knobs[0] > 64 || knobs[1] > 64 ||
      knobs[3] > 64 || knobs[4] > 64)
    return fail(AEOLUS_ERR_ARG, "aeolus_plan_set_tuning: members per CTA must be in 0..64");
  if (knobs[2] != 0 && (knobs[2] < 64 || knobs[2] > 256 || knobs[2] % 32 != 0))
    return fail(AEOLUS_ERR_ARG, "aeolus_plan_set_tuning: row threads must be 0 or a multiple of 32 in 64..256");
  plan->tune_bc_synth = knobs[0];
  plan->tune_bc_anal = knobs[1];
  plan->tune_row_threads = knobs[2];
  plan->tune_slice_mb = knobs[3];
  plan->tune_slice_mb_anal = knobs[4];
  return AEOLUS_OK;
}

extern "C" int aeolus_plan_get_tuning(aeolus_plan plan, int* knobs) {
  if (!plan_ok(plan) || !knobs) return fail(AEOLUS_ERR_ARG, "aeolus_plan_get_tuning: bad arguments");
  knobs[0] = plan->tune_bc_synth;
  knobs[1] = plan->tune_bc_anal;
  knobs[2] = plan->tune_row_threads;
  knobs[3] = plan->tune_slice_mb;
  knobs[4] = plan->tune_slice_mb_anal;
  return AEOLUS_OK;
}
