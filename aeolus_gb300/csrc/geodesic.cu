// Icosahedral geodesic point set built on the device: midpoint subdivision,
// spherical coordinates, minimum edge length and the barycentric "Voronoi"
// cell areas of src/planetary_sandbox/numerics/geodesic_grid.py:31-266.
//
// Point order.  The reference visits faces in order and, per face, the edges
// (v1 v2), (v2 v3), (v3 v1); an edge's midpoint is appended to the vertex
// list the first time the edge is met (geodesic_grid.py:103-160).  Here every
// face carries, per edge slot s = 3 f + e, the packed slot of the same edge in
// the neighbouring face (adjacency).  The first visit of an edge is the
// smaller of its two slots ("owner"), so the midpoint of slot s gets index
// n_vertices + (number of owner slots below min(s, twin(s))): an exclusive
// prefix sum over owner flags, no hashing or sorting.  Children are numbered
// like the reference's (v1 m12 m31), (v2 m23 m12), (v3 m31 m23),
// (m12 m23 m31), and their adjacency follows from the parent's.
//
// Arithmetic.  Midpoints are normalize((a + b) / 2) with every operation
// rounded separately in the reference's order (x*x + y*y, then + z*z; sqrt;
// divide), so a midpoint is the reference's bit pattern whenever its two
// endpoints are.  Cell areas sum each vertex's face contributions in
// ascending face order, the accumulation order of the reference loop.
#include <cmath>

#include "common.cuh"

namespace aeolus {
namespace {

constexpr int kGeoMaxResolution = 9;          // 2,621,442 points
constexpr int kScanThreads = 1024, kScanItems = 4, kScanTile = kScanThreads * kScanItems;
constexpr int kMaxValence = 6;                // icosahedral meshes: valence 5 or 6

struct IcoSeed {
  double v[12][3];
  int f[20][3];
  int adj[20][3];  // packed slot 3 g + e' of the same edge in the neighbouring face
};

__host__ __device__ inline long geo_points(int r) { return 10L * (1L << (2 * r)) + 2; }
__host__ __device__ inline long geo_faces(int r) { return 20L * (1L << (2 * r)); }

__global__ void geo_seed_kernel(IcoSeed s, double* pts, int* faces, int* adj) {
  const int t = threadIdx.x;
  if (t < 36) pts[t] = s.v[t / 3][t % 3];
  if (t < 60) {
    faces[t] = s.f[t / 3][t % 3];
    adj[t] = s.adj[t / 3][t % 3];
  }
}

__device__ inline int block_sum(int v, int* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) red[w] = v;
  __syncthreads();
  int t = 0;
  if (w == 0) {
    t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  return t;  // valid in thread 0
}

// Exclusive block scan of one value per thread (blockDim.x == kScanThreads).
__device__ inline int block_exclusive_scan(int v, int* red, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int n = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += n;
  }
  if (lane == 31) red[w] = inc;
  __syncthreads();
  if (w == 0) {
    int x = red[lane];
    int xi = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int n = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += n;
    }
    red[lane] = xi - x;  // exclusive warp offsets
    if (lane == 31 && total) *total = xi;
  }
  __syncthreads();
  return red[w] + inc - v;
}

// Owner flag of slot s: its edge is first visited at s (s < twin(s)).
__device__ inline int owner(long s, long nslots, const int* adj) { return s < nslots && s < (long)adj[s]; }

__global__ void __launch_bounds__(kScanThreads) geo_owner_tiles(long nslots, const int* __restrict__ adj,
                                                              int* __restrict__ tile_sums) {
  __shared__ int red[32];
  const long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanItems;
  int c = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) c += owner(base + i, nslots, adj);
  const int t = block_sum(c, red);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = t;
}

// One block: exclusive scan of the tile sums in place (ntiles <= kScanThreads).
__global__ void __launch_bounds__(kScanThreads) geo_scan_tiles(int ntiles, int* tile_sums) {
  __shared__ int red[32];
  const int v = threadIdx.x < ntiles ? tile_sums[threadIdx.x] : 0;
  const int x = block_exclusive_scan(v, red, nullptr);
  if (threadIdx.x < ntiles) tile_sums[threadIdx.x] = x;
}

__global__ void __launch_bounds__(kScanThreads) geo_owner_rank(long nslots, const int* __restrict__ adj,
                                                             const int* __restrict__ tile_off,
                                                             int* __restrict__ rank) {
  __shared__ int red[32];
  const long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanItems;
  int fl[kScanItems], c = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    fl[i] = owner(base + i, nslots, adj);
    c += fl[i];
  }
  int x = block_exclusive_scan(c, red, nullptr) + tile_off[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < nslots) rank[base + i] = x;
    x += fl[i];
  }
}

// g's child-face slot holding the half of g's edge slot e2 that touches
// vertex X (children numbered as in the reference, see the file comment).
__device__ inline int half_slot(const int* F, int g, int e2, int X) {
  const int w0 = F[3 * g + e2];
  const int child = X == w0 ? e2 : (e2 + 1) % 3;
  const int slot = X == w0 ? 0 : 2;
  return 3 * (4 * g + child) + slot;
}

__global__ void geo_subdivide_kernel(int nf, int nv, const int* __restrict__ F, const int* __restrict__ A,
                                     const int* __restrict__ rank, double* __restrict__ pts, int* __restrict__ F2,
                                     int* __restrict__ A2) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int v[3] = {F[3 * f], F[3 * f + 1], F[3 * f + 2]};
  int m[3];
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    const int s = 3 * f + e, t = A[s];
    m[e] = nv + rank[s < t ? s : t];
    if (s < t) {
      const int a = v[e], b = v[(e + 1) % 3];
      const double x = __dmul_rn(__dadd_rn(pts[3 * a + 0], pts[3 * b + 0]), 0.5);
      const double y = __dmul_rn(__dadd_rn(pts[3 * a + 1], pts[3 * b + 1]), 0.5);
      const double z = __dmul_rn(__dadd_rn(pts[3 * a + 2], pts[3 * b + 2]), 0.5);
      const double n = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
      pts[3L * m[e] + 0] = __ddiv_rn(x, n);
      pts[3L * m[e] + 1] = __ddiv_rn(y, n);
      pts[3L * m[e] + 2] = __ddiv_rn(z, n);
    }
  }
  const int c[4][3] = {{v[0], m[0], m[2]}, {v[1], m[1], m[0]}, {v[2], m[2], m[1]}, {m[0], m[1], m[2]}};
  const long cf = 4L * f;
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int j = 0; j < 3; ++j) F2[3 * (cf + k) + j] = c[k][j];
  // interior edges: (m12 m31) | (m31 m12), (m23 m12) | (m12 m23), (m31 m23) | (m23 m31)
  A2[3 * (cf + 0) + 1] = (int)(3 * (cf + 3) + 2);
  A2[3 * (cf + 3) + 2] = (int)(3 * (cf + 0) + 1);
  A2[3 * (cf + 1) + 1] = (int)(3 * (cf + 3) + 0);
  A2[3 * (cf + 3) + 0] = (int)(3 * (cf + 1) + 1);
  A2[3 * (cf + 2) + 1] = (int)(3 * (cf + 3) + 1);
  A2[3 * (cf + 3) + 1] = (int)(3 * (cf + 2) + 1);
  // halves of the parent edges: slot e runs v[e] -> v[e+1]; its half at v[e]
  // is child e slot 0, its half at v[e+1] child e+1 slot 2
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    const int t = A[3 * f + e], g = t / 3, e2 = t - 3 * g;
    A2[3 * (cf + e) + 0] = half_slot(F, g, e2, v[e]);
    A2[3 * (cf + (e + 1) % 3) + 2] = half_slot(F, g, e2, v[(e + 1) % 3]);
  }
}

__global__ void geo_points_kernel(long nv, double radius, double* __restrict__ pts, double* __restrict__ lat,
                                  double* __restrict__ lon, int* __restrict__ cnt) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const double x = radius * pts[3 * i], y = radius * pts[3 * i + 1], z = radius * pts[3 * i + 2];
  pts[3 * i] = x;
  pts[3 * i + 1] = y;
  pts[3 * i + 2] = z;
  lon[i] = atan2(y, x);               // [-pi, pi], cartesian_to_spherical.py
  lat[i] = atan2(z, hypot(x, y));     // geocentric latitude
  cnt[i] = 0;
}

__device__ inline double norm3(double x, double y, double z) {
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
}

__device__ inline double clamped_angle(const double* a, const double* b) {
  const double d = __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
  return acos(fmin(1.0, fmax(-1.0, d)));
}

// Per face: one third of its spherical-triangle area (L'Huilier's excess,
// geodesic_grid.py:212-266), its three edge lengths into the running
// minimum, and its vertex incidences.
__global__ void geo_faces_kernel(long nf, double radius, const double* __restrict__ pts, const int* __restrict__ F,
                                 double* __restrict__ area3, unsigned long long* __restrict__ min_bits,
                                 int* __restrict__ cnt, int* __restrict__ inc, int* __restrict__ err) {
  const long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  double u[3][3], p[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const long v = F[3 * f + k];
#pragma unroll
    for (int j = 0; j < 3; ++j) p[k][j] = pts[3 * v + j];
    const double n = norm3(p[k][0], p[k][1], p[k][2]);
#pragma unroll
    for (int j = 0; j < 3; ++j) u[k][j] = __ddiv_rn(p[k][j], n);
  }
  unsigned long long mb = ~0ull;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int k2 = (k + 1) % 3;
    const double d = norm3(p[k][0] - p[k2][0], p[k][1] - p[k2][1], p[k][2] - p[k2][2]);
    if (d > 0.0) mb = min(mb, (unsigned long long)__double_as_longlong(d));
  }
  if (mb != ~0ull) atomicMin(min_bits, mb);
  const double sa = clamped_angle(u[1], u[2]), sb = clamped_angle(u[0], u[2]), sc = clamped_angle(u[0], u[1]);
  const double s = (sa + sb + sc) / 2.0;
  const double t = sqrt(tan(s / 2.0) * tan((s - sa) / 2.0) * tan((s - sb) / 2.0) * tan((s - sc) / 2.0));
  area3[f] = 4.0 * atan(t) * (radius * radius) / 3.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const long v = F[3 * f + k];
    const int q = atomicAdd(&cnt[v], 1);
    if (q < kMaxValence) inc[kMaxValence * v + q] = (int)f;
    else atomicExch(err, 1);
  }
}

// Per vertex: its incident faces in ascending order, contributions summed in
// that order from zero.
__global__ void geo_areas_kernel(long nv, const double* __restrict__ area3, const int* __restrict__ cnt,
                                 const int* __restrict__ inc, double* __restrict__ areas) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const int n = min(cnt[i], kMaxValence);
  int f[kMaxValence];
  for (int k = 0; k < n; ++k) {
    int x = inc[kMaxValence * i + k], j = k;
    while (j > 0 && f[j - 1] > x) {
      f[j] = f[j - 1];
      --j;
    }
    f[j] = x;
  }
  double acc = 0.0;
  for (int k = 0; k < n; ++k) acc = __dadd_rn(acc, area3[f[k]]);
  areas[i] = acc;
}

__global__ void geo_finish_kernel(const unsigned long long* min_bits, double* min_edge) {
  *min_edge = *min_bits == ~0ull ? 0.0 : __longlong_as_double((long long)*min_bits);
}

IcoSeed make_seed() {
  const double phi = (1.0 + std::sqrt(5.0)) / 2.0;
  const double v0[12][3] = {{-1, phi, 0}, {1, phi, 0}, {-1, -phi, 0}, {1, -phi, 0}, {0, -1, phi}, {0, 1, phi},
                            {0, -1, -phi}, {0, 1, -phi}, {phi, 0, -1}, {phi, 0, 1}, {-phi, 0, -1}, {-phi, 0, 1}};
  const int f0[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                         {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
                         {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
  IcoSeed s{};
  // unit icosahedron (geodesic_grid.py:15-28), rotated 1e-2 rad about x
  // against the polar singularity (:37-38)
  const double c = std::cos(1e-2), sn = std::sin(1e-2), h = std::hypot(1.0, phi);
  for (int i = 0; i < 12; ++i) {
    const double x = v0[i][0] / h, y = v0[i][1] / h, z = v0[i][2] / h;
    // products rounded before the sums (no fused multiply-add on any host)
    volatile double cy = c * y, sz = sn * z, sy = sn * y, cz = c * z;
    s.v[i][0] = x;
    s.v[i][1] = cy - sz;
    s.v[i][2] = sy + cz;
  }
  for (int f = 0; f < 20; ++f)
    for (int e = 0; e < 3; ++e) s.f[f][e] = f0[f][e];
  for (int f = 0; f < 20; ++f)
    for (int e = 0; e < 3; ++e) {
      const int a = f0[f][e], b = f0[f][(e + 1) % 3];
      s.adj[f][e] = -1;
      for (int g = 0; g < 20; ++g)
        for (int e2 = 0; e2 < 3; ++e2) {
          const int a2 = f0[g][e2], b2 = f0[g][(e2 + 1) % 3];
          if (g != f && ((a2 == a && b2 == b) || (a2 == b && b2 == a))) s.adj[f][e] = 3 * g + e2;
        }
    }
  return s;
}

struct GeoWork {
  int *ftmp, *adj0, *adj1, *rank, *tiles, *cnt, *inc, *err;
  double* area3;
  unsigned long long* min_bits;
  size_t bytes;
};

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

GeoWork geo_layout(int r, char* base) {
  const long nf = geo_faces(r), nv = geo_points(r);
  const long nf_prev = r > 0 ? geo_faces(r - 1) : 0;
  GeoWork w{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  w.ftmp = reinterpret_cast<int*>(take(3 * nf * sizeof(int)));
  w.adj0 = reinterpret_cast<int*>(take(3 * nf * sizeof(int)));
  w.adj1 = reinterpret_cast<int*>(take(3 * nf * sizeof(int)));
  w.rank = reinterpret_cast<int*>(take(3 * (nf_prev > 0 ? nf_prev : 1) * sizeof(int)));
  w.tiles = reinterpret_cast<int*>(take(kScanThreads * sizeof(int)));
  w.cnt = reinterpret_cast<int*>(take(nv * sizeof(int)));
  w.inc = reinterpret_cast<int*>(take(kMaxValence * nv * sizeof(int)));
  w.area3 = reinterpret_cast<double*>(take(nf * sizeof(double)));
  w.min_bits = reinterpret_cast<unsigned long long*>(take(sizeof(unsigned long long)));
  w.err = reinterpret_cast<int*>(take(sizeof(int)));
  w.bytes = off;
  return w;
}

}  // namespace
}  // namespace aeolus

using namespace aeolus;

extern "C" int aeolus_geodesic_sizes(int resolution, long* n_points, long* n_faces, size_t* work_bytes) {
  if (resolution < 0 || resolution > kGeoMaxResolution)
    return fail(AEOLUS_ERR_ARG, "geodesic resolution must be in [0, " + std::to_string(kGeoMaxResolution) +
                                    "], got " + std::to_string(resolution));
  if (n_points) *n_points = geo_points(resolution);
  if (n_faces) *n_faces = geo_faces(resolution);
  if (work_bytes) *work_bytes = geo_layout(resolution, nullptr).bytes;
  return AEOLUS_OK;
}

extern "C" int aeolus_geodesic_build(int resolution, double radius, double* points, int* faces, double* lat,
                                     double* lon, double* areas, double* min_edge, int* status, void* work,
                                     size_t work_bytes, void* stream) {
  size_t need = 0;
  if (int s = aeolus_geodesic_sizes(resolution, nullptr, nullptr, &need)) return s;
  if (!(std::isfinite(radius) && radius > 0.0))
    return fail(AEOLUS_ERR_ARG, "geodesic radius must be finite and > 0, got " + std::to_string(radius));
  if (!points || !faces || !lat || !lon || !areas || !min_edge || !status)
    return fail(AEOLUS_ERR_ARG, "geodesic build: null output pointer");
  if (!work || work_bytes < need)
    return fail(AEOLUS_ERR_WORKSPACE, "geodesic build: workspace of " + std::to_string(need) + " bytes needed");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const GeoWork w = geo_layout(resolution, static_cast<char*>(work));
  const int r = resolution;
  // level k's faces live in `faces` when r - k is even, else in ftmp, so
  // the last level lands in the caller's buffer
  auto fbuf = [&](int k) { return ((r - k) & 1) == 0 ? faces : w.ftmp; };
  auto abuf = [&](int k) { return (k & 1) == 0 ? w.adj0 : w.adj1; };
  ProfScope prof("geodesic_build", st);
  geo_seed_kernel<<<1, 64, 0, st>>>(make_seed(), points, fbuf(0), abuf(0));
  AE_LAUNCH("geo_seed_kernel");
  for (int k = 0; k < r; ++k) {
    const long nf = geo_faces(k), nv = geo_points(k), nslots = 3 * nf;
    const int ntiles = (int)((nslots + kScanTile - 1) / kScanTile);
    if (ntiles > kScanThreads) return fail(AEOLUS_ERR_ARG, "geodesic build: scan tile count exceeded");
    geo_owner_tiles<<<ntiles, kScanThreads, 0, st>>>(nslots, abuf(k), w.tiles);
    AE_LAUNCH("geo_owner_tiles");
    geo_scan_tiles<<<1, kScanThreads, 0, st>>>(ntiles, w.tiles);
    AE_LAUNCH("geo_scan_tiles");
    geo_owner_rank<<<ntiles, kScanThreads, 0, st>>>(nslots, abuf(k), w.tiles, w.rank);
    AE_LAUNCH("geo_owner_rank");
    geo_subdivide_kernel<<<(unsigned)((nf + 127) / 128), 128, 0, st>>>((int)nf, (int)nv, fbuf(k), abuf(k), w.rank,
                                                                       points, fbuf(k + 1), abuf(k + 1));
    AE_LAUNCH("geo_subdivide_kernel");
  }
  const long nf = geo_faces(r), nv = geo_points(r);
  AE_CUDA(cudaMemsetAsync(w.min_bits, 0xFF, sizeof(unsigned long long), st));
  AE_CUDA(cudaMemsetAsync(w.err, 0, sizeof(int), st));
  geo_points_kernel<<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(nv, radius, points, lat, lon, w.cnt);
  AE_LAUNCH("geo_points_kernel");
  geo_faces_kernel<<<(unsigned)((nf + 255) / 256), 256, 0, st>>>(nf, radius, points, faces, w.area3, w.min_bits,
                                                                 w.cnt, w.inc, w.err);
  AE_LAUNCH("geo_faces_kernel");
  geo_areas_kernel<<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(nv, w.area3, w.cnt, w.inc, areas);
  AE_LAUNCH("geo_areas_kernel");
  geo_finish_kernel<<<1, 1, 0, st>>>(w.min_bits, min_edge);
  AE_LAUNCH("geo_finish_kernel");
  AE_CUDA(cudaMemcpyAsync(status, w.err, sizeof(int), cudaMemcpyDeviceToDevice, st));
  return AEOLUS_OK;
}
