// Point-set plan: real basis built on the device (FP64 normalised
// recurrence, one thread per point) and the FP64 basis GEMMs.
#include "points.cuh"

namespace aeolus {

namespace {

constexpr double kInvSqrt4Pi = 0.28209479177387814347;

__global__ void points_basis_kernel(long n, int L, const double* __restrict__ lat, const double* __restrict__ lon,
                                    double* __restrict__ B) {
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const double x = sin(lat[p]);   // cos(colatitude)
  const double s = cos(lat[p]);   // sin(colatitude) >= 0
  const double lam = lon[p];
  double pmm = kInvSqrt4Pi;
  for (int m = 0; m <= L; ++m) {
    if (m > 0) pmm = -sqrt((2.0 * m + 1.0) / (2.0 * m)) * s * pmm;
    double sm, cm;
    sincos(m * lam, &sm, &cm);
    const long cb = col_base(m, L);
    const long sb = cb + (L + 1 - m);
    double p2 = pmm, p1 = 0.0;
    B[(cb + 0) * n + p] = pmm * cm;
    if (m > 0) B[(sb + 0) * n + p] = pmm * sm;
    if (m < L) {
      p1 = sqrt(2.0 * m + 3.0) * x * pmm;
      B[(cb + 1) * n + p] = p1 * cm;
      if (m > 0) B[(sb + 1) * n + p] = p1 * sm;
    }
    for (int l = m + 2; l <= L; ++l) {
      const double a = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
      const double b = sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
      const double pl = a * (x * p1 - b * p2);
      B[(cb + (l - m)) * n + p] = pl * cm;
      if (m > 0) B[(sb + (l - m)) * n + p] = pl * sm;
      p2 = p1;
      p1 = pl;
    }
  }
}

}  // namespace

int build_points_basis(aeolus_plan_impl* p, const double* lat, const double* lon) {
  const long n = p->npoints;
  double *dlat = nullptr, *dlon = nullptr;
  AE_CUDA(cudaMalloc(&dlat, n * sizeof(double)));
  AE_CUDA(cudaMalloc(&dlon, n * sizeof(double)));
  int s = cuda_check(cudaMemcpy(dlat, lat, n * sizeof(double), cudaMemcpyHostToDevice), "lat");
  if (!s) s = cuda_check(cudaMemcpy(dlon, lon, n * sizeof(double), cudaMemcpyHostToDevice), "lon");
  if (!s) s = cuda_check(cudaMalloc(&p->basis, (size_t)n * p->ncol * sizeof(double)), "cudaMalloc basis");
  if (!s) {
    points_basis_kernel<<<(unsigned)((n + 127) / 128), 128>>>(n, p->lmax, dlat, dlon, p->basis);
    s = cuda_check(cudaGetLastError(), "points_basis_kernel");
  }
  if (!s) s = cuda_check(cudaDeviceSynchronize(), "points basis");
  cudaFree(dlat);
  cudaFree(dlon);
  p->ld_basis = (int)n;
  return s;
}

int points_gemm_synth(const aeolus_plan_impl* p, const double* V, double* out, int ncols, cudaStream_t st) {
  const long M = p->npoints, K = p->ncol;
  dim3 grid((unsigned)((M + 63) / 64), (unsigned)((ncols + 31) / 32));
  dgemm_kernel<true><<<grid, 128, 0, st>>>(M, ncols, K, p->basis, M, V, K, out, M);
  AE_LAUNCH("dgemm_kernel(synthesis)");
  return AEOLUS_OK;
}

int points_gemm_analysis(const aeolus_plan_impl* p, const double* W, double* C, int ncols, cudaStream_t st) {
  const long M = p->ncol, K = p->npoints;
  dim3 grid((unsigned)((M + 63) / 64), (unsigned)((ncols + 31) / 32));
  dgemm_kernel<false><<<grid, 128, 0, st>>>(M, ncols, K, p->basis, K, W, K, C, M);
  AE_LAUNCH("dgemm_kernel(analysis)");
  return AEOLUS_OK;
}

}  // namespace aeolus
