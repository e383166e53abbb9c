/*
 * aeolus_gb300 -- C ABI of the GB300 (sm_103a) spectral hot path.
 *
 * Spherical-harmonic synthesis/analysis on a Gauss-Legendre grid (per-order
 * Legendre contraction + longitude real FFT) or on an arbitrary point set
 * (dense basis product), and the barotropic-vorticity (BVE) and
 * shallow-water (SWE) tendencies and RK4 steps built on them.
 *
 * Conventions (all citations are paths inside the reference project,
 * planetary_sandbox):
 *  - Spectral arrays use the reference's dense layout: complex128 values
 *    stored as interleaved (re, im) doubles, shape [batch][L+1][L+1],
 *    axis 0 = degree l, axis 1 = order m >= 0 (spectral_operators.py:56-61).
 *    Slots with m > l are ignored on input and written as zero on output.
 *  - SWE state stacks are [batch][3][L+1][L+1] (zeta, delta, phi),
 *    physics/shallow_water.py:106-115.
 *  - Grid arrays are float64 [batch][n_points]; on a Gauss plan the points
 *    are lat-major with rows north -> south (latlon_grid.py:72-76).
 *  - Every data pointer is a DEVICE pointer owned by the caller, except the
 *    host arrays passed to plan creation / returned by aeolus_plan_nodes.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).
 *  - Calls that need scratch take (work, work_bytes); the size comes from
 *    aeolus_workspace_bytes().  Hot-path calls never allocate.
 *  - Status: 0 = ok, nonzero = error; aeolus_last_error() gives the message
 *    for the calling thread.  Invalid arguments are rejected before any
 *    launch (the reference raises ValueError, spherical_backend.py:92-97).
 */
#ifndef AEOLUS_GB300_H
#define AEOLUS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct aeolus_plan_s* aeolus_plan;

enum aeolus_status {
  AEOLUS_OK = 0,
  AEOLUS_ERR_ARG = 1,        /* invalid argument / unsupported shape       */
  AEOLUS_ERR_CUDA = 2,       /* CUDA runtime error                         */
  AEOLUS_ERR_WORKSPACE = 3,  /* work buffer missing or too small           */
  AEOLUS_ERR_STATE = 4       /* state validation failed (see status words) */
};

enum aeolus_precision {
  AEOLUS_PREC_FP64 = 0,        /* plain float64 contraction (the drop-in)   */
  AEOLUS_PREC_SPLIT_BF16 = 1   /* FP64 operands sliced to bf16, tcgen05 MMA */
};

/* Operation ids for aeolus_workspace_bytes. */
enum aeolus_op {
  AEOLUS_OP_SYNTHESIZE = 0,
  AEOLUS_OP_ANALYZE = 1,
  AEOLUS_OP_JACOBIAN = 2,
  AEOLUS_OP_WINDS = 3,
  AEOLUS_OP_BVE_TENDENCY = 4,
  AEOLUS_OP_SWE_TENDENCY = 5,
  AEOLUS_OP_BVE_RK4 = 6,
  AEOLUS_OP_SWE_RK4 = 7,
  AEOLUS_OP_SWE_VALIDATE = 8,
  AEOLUS_OP_SWE_INVARIANTS = 9,
  AEOLUS_OP_SYNTHESIZE_ADJOINT = 10,
  AEOLUS_OP_ANALYZE_ADJOINT = 11,
  AEOLUS_OP_BVE_TENDENCY_ADJOINT = 12,
  AEOLUS_OP_SWE_TENDENCY_ADJOINT = 13,
  AEOLUS_OP_BVE_RK4_ADJOINT = 14,
  AEOLUS_OP_SWE_RK4_ADJOINT = 15,
  AEOLUS_OP_VECTOR_CURL_DIV = 16
};

/* SWE state-check bits (physics/shallow_water.py:494-539). */
enum aeolus_state_bits {
  AEOLUS_STATE_NONFINITE = 1,  /* NaN/Inf coefficient or grid value        */
  AEOLUS_STATE_MONOPOLE = 2,   /* |a00| > 1e-10 * ||field||                 */
  AEOLUS_STATE_THICKNESS = 4   /* min(Phi0 + phi) <= 0 on a sampling        */
};

typedef struct {
  double radius;     /* a [m]                                             */
  double omega;      /* rotation rate [1/s]                               */
  double viscosity;  /* nu [m^2/s], barotropic.py:158                      */
} aeolus_bve_params;

typedef struct {
  double radius;       /* a [m]                                           */
  double omega;        /* [1/s]                                           */
  double gravity;      /* g [m/s^2]                                       */
  double mean_depth;   /* H [m]; Phi0 = g H                               */
  double nu4;          /* hyperdiffusion [m^4/s], shallow_water.py:405-413 */
  const double* forcing;  /* NULL, or a constant DEVICE spectral forcing
                           * [3][L+1][L+1] complex added to every tendency
                           * evaluation: bottom topography's -lap(phi_s) on
                           * delta and -nu4 lap^2 phi_s' on phi
                           * (shallow_water.py:397-413); row l = 0 ignored */
} aeolus_swe_params;

const char* aeolus_last_error(void);
int aeolus_version(void);

/* Per-kernel CUDA-event timing for measurement (no reference counterpart;
 * the reference times whole calls with time.time(), tests/speed_showdown.py).
 * enable != 0 brackets every library launch with events on its stream;
 * collect synchronises the pending events and writes one line per kernel,
 * "name launches total_ms\n", into buf; reset clears the totals.  Keep it
 * disabled during CUDA-graph capture. */
int aeolus_profile_enable(int enable);
int aeolus_profile_collect(char* buf, size_t len);
int aeolus_profile_reset(void);

/* ---- plans ---------------------------------------------------------- */

/* Gauss-Legendre nlat x nlon grid at truncation lmax: nodes/weights by an
 * FP64 Newton iteration on the device, normalised P_lm tables, FFT
 * twiddles.  Replaces GaussLatLonGridGeometry + GaussLatLonSphericalHarmonics
 * (numerics/latlon_grid.py:43-199) and the basis build of
 * PointSetSphericalHarmonics (numerics/fast_geodesic_sh.py:15-66,
 * numerics/cuda/sh_matrix.cu:7-76).  radius only sets operator metrics. */
int aeolus_plan_create_gauss(int nlat, int nlon, int lmax, double radius,
                             int flags, aeolus_plan* out);

/* Arbitrary point set (host arrays, n points): dense real basis built on
 * the device.  Replaces PointSetSphericalHarmonics
 * (numerics/fast_geodesic_sh.py:15-66); w == NULL gives the reference's
 * uniform 4*pi/n default (:35-37). */
int aeolus_plan_create_points(long n, const double* lat, const double* lon,
                              const double* w, int lmax, double radius,
                              int flags, aeolus_plan* out);

int aeolus_plan_destroy(aeolus_plan plan);

/* kind: 0 = Gauss, 1 = points.  Any pointer may be NULL. */
int aeolus_plan_info(aeolus_plan plan, int* kind, int* nlat, int* nlon,
                     int* lmax, long* n_points);

/* Host copies of the Gauss nodes (latitudes [nlat], north -> south) and
 * Gauss-Legendre weights [nlat] (sum 2), latlon_grid.py:59-67. */
int aeolus_plan_nodes(aeolus_plan plan, double* lat, double* w_gl);

/* Contraction precision for later calls on this plan (slices: number of
 * bf16 slices per FP64 operand, 0 = default).  AEOLUS_PREC_SPLIT_BF16 on a
 * Gauss plan needs l_max <= 159 and nlat <= 192 (exact f32 digit sums). */
int aeolus_plan_set_precision(aeolus_plan plan, int precision, int slices);

/* Sticky device error flag of the plan's tensor-core kernels: nonzero when a
 * bounded wait on a copy or MMA completion expired (the kernel then skipped
 * its outputs).  Reading it synchronises the device.  No reference
 * counterpart (the reference has no device-side waits). */
int aeolus_plan_device_error(aeolus_plan plan, int* flag);

/* Self-test of the bounded device-side waits (no reference counterpart): one
 * thread waits on an mbarrier phase that nothing completes, with a wall-time
 * limit of limit_ns (at most 10 s).  *timed_out = 1 when the wait gave up,
 * *elapsed_ns = the wait's duration on the device clock.  Synchronous. */
int aeolus_selftest_wait_timeout(unsigned long long limit_ns, int* timed_out,
                                 unsigned long long* elapsed_ns);

/* Self-test of the FP64 <-> double-float conversions the split path uses
 * in its derive, PE and column kernels (no reference counterpart): for the
 * n FP64 values x (device memory), out (device, 3 n doubles) receives per
 * value hi and lo of its double-float (hi = x truncated to 24 significant
 * bits, lo = the other 29 bits rounded to a float; |x| below 2^-126 gives
 * 0, |x| of 2^128 or more +-infinity) and hi + lo rounded back to FP64.
 * Ordered on `stream`. */
int aeolus_selftest_df_convert(const double* x, int n, double* out, void* stream);

/* Launch shapes of the plan's kernels (no reference counterpart), an array
 * of AEOLUS_TUNING_KNOBS ints: knobs[0] members per CTA of the FP64 Legendre
 * synthesis, knobs[1] of the analysis, knobs[2] threads per CTA of the
 * longitude (row) stage, knobs[3] members per CTA of the split-precision
 * synthesis slicing kernel, knobs[4] of the analysis slicing kernel;
 * 0 = built-in heuristic.  Results do not depend on these shapes (the
 * autotuners set them). */
#define AEOLUS_TUNING_KNOBS 5
int aeolus_plan_set_tuning(aeolus_plan plan, const int* knobs);
int aeolus_plan_get_tuning(aeolus_plan plan, int* knobs);

int aeolus_workspace_bytes(aeolus_plan plan, int op, int batch, size_t* bytes);

/* ---- transforms ------------------------------------------------------ */

/* grid[b] = 2 Re(Y a_b) - Re(Y a_b|m=0), fast_geodesic_sh.py:89-107. */
int aeolus_synthesize(aeolus_plan plan, const double* coeffs, double* grid,
                      int batch, void* work, size_t work_bytes, void* stream);

/* Synthesis that allocates nothing and takes no workspace: same result as
 * aeolus_synthesize on a Gauss plan with the FP64 contraction.  It has no
 * counterpart in the reference.  It serves callers that cannot call
 * cudaMalloc or own a device buffer -- e.g. FFI hosts (Go, Java, plain C)
 * without a device allocator of their own, or code that must not trigger the
 * implicit device synchronisation of cudaMalloc/cudaFree.  Scratch is one
 * fixed 16 MiB device array inside the library, held by every GPU that
 * loads it until process exit; batches needing more scratch are rejected
 * with AEOLUS_ERR_WORKSPACE.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) and must come before any
 * stream capture; that address is kept for the life of the process, so a
 * device reset (cudaDeviceReset) between calls is not supported.  All calls
 * share the array: calls that overlap on the GPU (different streams, or
 * threads without ordering) race on it. */
int aeolus_synthesize_noalloc(aeolus_plan plan, const double* coeffs,
                              double* grid, int batch, void* stream);

/* coeffs[b] = Y^H (w * grid[b]) scattered to the dense layout,
 * fast_geodesic_sh.py:68-87. */
int aeolus_analyze(aeolus_plan plan, const double* grid, double* coeffs,
                   int batch, void* work, size_t work_bytes, void* stream);

/* Curl and divergence of tangent vector fields by the weak form with
 * one-degree-extended analyses, spectral_operators.py:399-492
 * (vector_curl_div_spectral): plan_ext is a plan on the product points with
 * the product weights and l_max = L + 1 (L the state degree); f_en is
 * [batch][2][n_points] (eastward, northward components); curl and div are
 * [batch][L+1][L+1] complex; truncate != 0 applies the 2/3 cut of rows and
 * columns (cut = floor(2L/3)).  Workspace: AEOLUS_OP_VECTOR_CURL_DIV. */
int aeolus_vector_curl_div(aeolus_plan plan_ext, double radius, const double* f_en, double* curl,
                           double* div, int batch, int truncate, void* work, size_t work_bytes,
                           void* stream);

/* ---- dry hydrostatic primitive equations (physics/primitive_equations.py)
 * The tendency of primitive_equations.py:727-753 is five library calls
 * (aeolus_pe_derive -> aeolus_synthesize -> aeolus_pe_columns ->
 * aeolus_analyze + aeolus_vector_curl_div -> aeolus_pe_spectral) on a
 * product plan of degree L and its one-degree-extended plan.  States are
 * [batch][3K+1][L+1][L+1] complex, rows zeta_1..K, delta_1..K, T_1..K,
 * ln p_s (top to bottom, :76-136); sigma interfaces are a HOST array of
 * K + 1 values rising from exactly 0 to exactly 1 (sigma_coordinate.py:43-81);
 * 1 <= K <= 64.  No scratch: the callers own every intermediate. */
typedef struct {
  double radius;  /* m */
  double omega;   /* 1/s */
  double r_dry;   /* J/(kg K), primitive_equations.py:49 */
  double cp_dry;  /* J/(kg K), > r_dry */
} aeolus_pe_params;

/* fields [batch][10K+2][L+1][L+1]: per level u cos(lat), v cos(lat) (from
 * the l=0-zeroed inverse Laplacians of zeta and delta, :266-287), zeta, delta,
 * T, (1/R) dT/dlambda, (1/R) sin(theta) dT/dtheta, the same two of
 * eta = zeta + f, eta; then (1/R) d(ln p_s)/dlambda and
 * (1/R) sin(theta) d(ln p_s)/dtheta (:272-278, :531-548). */
int aeolus_pe_derive(aeolus_plan plan, const aeolus_pe_params* params, int nlev, const double* state,
                     double* fields, int batch, void* stream);

/* Column physics on the product points of `plan` (:482-587, sigma_coordinate.py
 * :212-398): grid = synthesis of the derive fields, [batch][10K+2][n_points];
 * prod [batch][4K+1][n_points] = per level the thermodynamic integrand
 * -V.grad T - sigma_dot dT/dsigma + kappa T omega/p (:615-619), -div(eta V),
 * curl(eta V), |V|^2/2 (:695-711), then d ln p_s/dt; f_en
 * [batch*K][2][n_points] = the residual vector Z = sigma_dot dV/dsigma +
 * R_d T grad(ln p_s) (east, north; :713-716). */
int aeolus_pe_columns(aeolus_plan plan, const aeolus_pe_params* params, int nlev, const double* interfaces,
                      const double* grid, double* prod, double* f_en, int batch, void* stream);

/* tendency [batch][3K+1][L+1][L+1] from the analysed integrands
 * (analysed [batch][4K+1][L+1][L+1]), the untruncated weak-form curl/div of
 * Z (curl_z, div_z [batch*K][L+1][L+1]), the state (for the
 * Simmons-Burridge geopotential of the spectral T, :691-693) and the
 * surface geopotential phi_s [L+1][L+1]: 2/3 cuts, -lap(KE + Phi), l = 0
 * rows of the zeta/delta tendencies zero (:718-724). */
int aeolus_pe_spectral(int lmax, const aeolus_pe_params* params, int nlev, const double* interfaces,
                       const double* state, const double* analysed, const double* curl_z, const double* div_z,
                       const double* phi_s, double* tendency, int batch, void* stream);

/* One classical RK4 stage update of n complex values (y0, k, ystage, acc
 * are [n] complex128 device arrays), the device form of the reference's
 * rk4_step_array (run/engine.py:406-431) for any tendency (the primitive
 * equations' fused RK4 uses it), in the reference's order of operations
 * with every FP64 product and sum rounded separately:
 *   stage 1: acc = k;         ystage = y0 + (dt/2) k
 *   stage 2: acc = acc + 2 k; ystage = y0 + (dt/2) k
 *   stage 3: acc = acc + 2 k; ystage = y0 + dt k
 *   stage 4: ystage = y0 + (dt/6) (acc + k)   (the step's result)
 * acc must not alias ystage or k; ystage may alias y0 at stage 4. */
int aeolus_rk4_stage(int stage, double dt, const double* y0, const double* k, double* ystage, double* acc,
                     long n, void* stream);

/* ---- icosahedral geodesic point set (numerics/geodesic_grid.py) -------- */

/* Point, face and workspace counts of a geodesic point set with
 * `resolution` midpoint subdivisions (0..9): n_points = 10 * 4^r + 2,
 * n_faces = 20 * 4^r.  Host only (no device work). */
int aeolus_geodesic_sizes(int resolution, long* n_points, long* n_faces, size_t* work_bytes);

/* Builds the point set on the device, replacing the host construction of
 * geodesic_grid.py:31-266 (icosahedron rotated 1e-2 rad about x, midpoint
 * subdivision in the reference's point and face order, :103-160;
 * cartesian_to_spherical.py coordinates; min edge length, :162-190;
 * barycentric "Voronoi" areas, one third of each L'Huilier triangle,
 * :212-266).  Outputs (device, caller-owned): points [n_points][3] scaled
 * by radius, faces [n_faces][3] int32, lat / lon [n_points] (lon in
 * [-pi, pi]), areas [n_points] in radius^2 units, min_edge [1], status [1]
 * int32 (nonzero: a vertex had more than 6 incident faces, which a valid
 * subdivision never produces).  Workspace from aeolus_geodesic_sizes. */
int aeolus_geodesic_build(int resolution, double radius, double* points, int* faces, double* lat,
                          double* lon, double* areas, double* min_edge, int* status, void* work,
                          size_t work_bytes, void* stream);

/* ---- spectral operators (numerics/spectral_operators.py) -------------- */

/* op: 0 laplacian (:213-218), 1 inverse laplacian with l=0 -> l=0 * R^2
 * (:275-292), 2 inverse laplacian with l=0 -> 0 (physics/barotropic.py:91,
 * physics/shallow_water.py:277-281), 3 d/dlambda = i m / R (:220-226),
 * 4 sin(theta) d/dtheta coupling (:228-241), 5 its adjoint (:243-270),
 * 6 2/3-rule truncation of rows and columns (:329-334). */
int aeolus_spectral_op(int op, int lmax, double radius, const double* in,
                       double* out, int batch, void* stream);

/* J(a, b) analysed on the plan's grid and 2/3-truncated,
 * spectral_operators.py:590-658 (dealias=True, return_spectral=True). */
int aeolus_jacobian(aeolus_plan plan, const double* a, const double* b,
                    double* out, int batch, void* work, size_t work_bytes,
                    void* stream);

/* Winds on the plan's points from psi, chi: u = (psi_snt + chi_lam)/cos,
 * v = (psi_lam - chi_snt)/cos (physics/shallow_water.py:305-319), written
 * as uv[2][batch][n_points] (uv[0] = u, uv[1] = v); chi == NULL gives
 * velocity_from_streamfunction (spectral_operators.py:517-538). */
int aeolus_winds(aeolus_plan plan, double radius, const double* psi,
                 const double* chi, double* uv, int batch,
                 void* work, size_t work_bytes, void* stream);

/* ---- models ----------------------------------------------------------- */

/* d(zeta)/dt = -J(psi, zeta + f) + nu lap zeta (+ forcing), l = 0 row zero;
 * physics/barotropic.py:120-167.  `plan` is the product-space plan. */
int aeolus_bve_tendency(aeolus_plan plan, const aeolus_bve_params* p,
                        const double* zeta, const double* forcing,
                        double* tend, int batch, void* work,
                        size_t work_bytes, void* stream);

/* SWE tendency of [batch][3][L+1][L+1], physics/shallow_water.py:347-418. */
int aeolus_swe_tendency(aeolus_plan plan, const aeolus_swe_params* p,
                        const double* state, double* tend, int batch,
                        void* work, size_t work_bytes, void* stream);

/* nsteps classical RK4 steps in place (run/bve/runner.py:211-216). */
int aeolus_bve_rk4(aeolus_plan plan, const aeolus_bve_params* p, double* zeta,
                   int batch, double dt, int nsteps, void* work,
                   size_t work_bytes, void* stream);

/* nsteps classical RK4 steps in place (run/engine.py:406-431).  When
 * `status` (device, [batch] uint32) is non-NULL every stage's state is
 * checked on the product grid and offending AEOLUS_STATE_* bits are OR-ed
 * in -- the stage validator of run/swe/runner.py:90-95 without host syncs. */
int aeolus_swe_rk4(aeolus_plan plan, const aeolus_swe_params* p, double* state,
                   int batch, double dt, int nsteps, unsigned* status,
                   void* work, size_t work_bytes, void* stream);

/* validate_state (physics/shallow_water.py:494-539) on the state plan and
 * (when product != state) the product plan: status[b] gets AEOLUS_STATE_*
 * bits, extrema[b] = (min, max) of Phi0 + phi over the samplings
 * (total_geopotential_extrema, :428-454).  Either output may be NULL. */
int aeolus_swe_validate(aeolus_plan state_plan, aeolus_plan product_plan,
                        const aeolus_swe_params* p, const double* state,
                        unsigned* status, double* extrema, int batch,
                        void* work, size_t work_bytes, void* stream);

/* BVE spectral diagnostics, run/bve/diagnostics.py:61-97: out[b][6] =
 * circulation, energy, enstrophy_rel, enstrophy_abs, energy_l1,
 * high_l_enstrophy_frac. */
int aeolus_bve_spectral_diagnostics(int lmax, double radius, double omega,
                                    const double* zeta, double* out,
                                    int batch, void* stream);

/* SWE invariants, run/swe/diagnostics.py:76-173: out[b][5] = total_mass,
 * total_energy (quadrature on the state plan), zeta_l2, delta_l2, phi_l2. */
int aeolus_swe_invariants(aeolus_plan state_plan, const aeolus_swe_params* p,
                          const double* state, double* out, int batch,
                          void* work, size_t work_bytes, void* stream);

/* ---- batched uneven ensembles (BVE and SWE) ------------------------------
 * Groups of members, each group on its own Gauss product-space plan (any
 * l_max; all plans on one device and one contraction precision), advanced
 * together: every RK4 stage launches each stage kernel once for all groups.
 * The reference runs one state per process (run/bve/runner.py:211-216,
 * run/engine.py:406-431); this has no counterpart there.  State pointer g is
 * group g's device state, advanced in place: BVE [batch_g][L_g+1][L_g+1],
 * SWE [batch_g][3][L_g+1][L_g+1].  Capture, launch and autotune serve both
 * models. */
typedef struct aeolus_ensemble_s* aeolus_ensemble;

int aeolus_ensemble_create(int ngroups, const aeolus_plan* plans,
                           const int* batch, const aeolus_bve_params* params,
                           aeolus_ensemble* out);
int aeolus_ensemble_destroy(aeolus_ensemble e);
int aeolus_ensemble_workspace_bytes(aeolus_ensemble e, size_t* bytes);
int aeolus_ensemble_bve_rk4(aeolus_ensemble e, double* const* zeta, double dt,
                            int nsteps, void* work, size_t work_bytes,
                            void* stream);
/* Shallow-water ensemble: per-group SWE parameters; steps as aeolus_swe_rk4
 * does for each group. */
int aeolus_ensemble_create_swe(int ngroups, const aeolus_plan* plans,
                               const int* batch, const aeolus_swe_params* params,
                               aeolus_ensemble* out);
int aeolus_ensemble_swe_rk4(aeolus_ensemble e, double* const* state, double dt,
                            int nsteps, void* work, size_t work_bytes,
                            void* stream);

/* Captures one RK4 step of the ensemble (these zeta pointers, dt and
 * workspace, which must stay valid) into a CUDA graph; `stream` must not be
 * the legacy default stream.  The states are not advanced.  Replay with
 * aeolus_ensemble_launch (nsteps graph launches on `stream`). */
int aeolus_ensemble_capture(aeolus_ensemble e, double* const* zeta,
                            double dt, void* work, size_t work_bytes,
                            void* stream);
int aeolus_ensemble_launch(aeolus_ensemble e, int nsteps, void* stream);

/* Times candidate launch shapes (members per CTA of the Legendre or slicing
 * kernels per group, threads of the row stage) on the ensemble's own states,
 * keeps the fastest in the plans and writes a text report.  States are not
 * advanced; results do not depend on the shapes.  Drops a captured graph. */
int aeolus_ensemble_autotune(aeolus_ensemble e, double* const* zeta,
                             void* work, size_t work_bytes, void* stream,
                             char* report, size_t report_len);

/* ---- adjoints (differentiation) ----------------------------------------
 * The reference differentiates nothing; these are the transposes of the
 * linear maps above and the vector-Jacobian products of the tendencies and
 * RK4 steps, for gradients through the forward model.  Inner products: a
 * spectral array is the real vector of the (Re, Im) parts of its m <= l
 * slots (m > l slots are written as zero), a grid array the real vector of
 * its values.  Each VJP is the exact transpose of the linearisation of the
 * FP64 forward map (planetary vorticity inside the products); on a split-
 * precision plan the contractions run in split precision. */

/* coeffs_bar = S^T grid_bar, S = aeolus_synthesize (a unit-weight analysis:
 * factor 2 on m > 0, Im of m = 0 zero). */
int aeolus_synthesize_adjoint(aeolus_plan plan, const double* grid_bar,
                              double* coeffs_bar, int batch, void* work,
                              size_t work_bytes, void* stream);

/* grid_bar = A^T coeffs_bar, A = aeolus_analyze (a synthesis of the m > 0
 * slots halved, times the quadrature weight of each point). */
int aeolus_analyze_adjoint(aeolus_plan plan, const double* coeffs_bar,
                           double* grid_bar, int batch, void* work,
                           size_t work_bytes, void* stream);

/* zeta_bar = (d tendency / d zeta)^T tend_bar at zeta (aeolus_bve_tendency
 * without forcing; the forcing does not depend on zeta). */
int aeolus_bve_tendency_adjoint(aeolus_plan plan, const aeolus_bve_params* p,
                                const double* zeta, const double* tend_bar,
                                double* zeta_bar, int batch, void* work,
                                size_t work_bytes, void* stream);

/* state_bar = (d tendency / d state)^T tend_bar at state
 * (aeolus_swe_tendency). */
int aeolus_swe_tendency_adjoint(aeolus_plan plan, const aeolus_swe_params* p,
                                const double* state, const double* tend_bar,
                                double* state_bar, int batch, void* work,
                                size_t work_bytes, void* stream);

/* Adjoint of ONE RK4 step taken from `zeta` / `state` (the step's input,
 * unchanged): on entry *_bar holds the adjoint of the step's output, on exit
 * that of its input.  The stage inputs are recomputed from the step input;
 * multi-step gradients checkpoint step inputs on the host side. */
int aeolus_bve_rk4_adjoint(aeolus_plan plan, const aeolus_bve_params* p,
                           const double* zeta, double* zeta_bar, int batch,
                           double dt, void* work, size_t work_bytes,
                           void* stream);
int aeolus_swe_rk4_adjoint(aeolus_plan plan, const aeolus_swe_params* p,
                           const double* state, double* state_bar, int batch,
                           double dt, void* work, size_t work_bytes,
                           void* stream);

#ifdef __cplusplus
}
#endif
#endif /* AEOLUS_GB300_H */
