/*
 * ibem_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the 3D elastic
 * spherical iBEM path.
 *
 * Every entry point replaces one method of the reference's four plugin interfaces
 * (integrator.h:28-34, BEMBuilder.h:27-35, systemSolver.h:28-31, postProcessor.h:27-31)
 * for the Elastic3D family (integratorElastic3D.cpp, BEMBuilderElastic3D.cpp,
 * systemSolverElastic3D.h, postProcessorElastic3D.cpp).  The reference methods take a
 * Config& and fill Eigen matrices; here the caller passes plain pointers:
 *
 *   - "_dev" pointers are device memory owned by the caller (cudaMalloc or any allocator);
 *   - matrices are column-major with an explicit leading dimension (as Eigen's MatrixXd);
 *   - coordinates are row-major (n x 3); connectivity is NE x 4, one-based (BEM.txt);
 *   - `stream` is a cudaStream_t passed as void* (NULL = default stream);
 *   - every call is asynchronous on `stream` unless documented otherwise;
 *   - the return value is an ibem_status; ibem_last_error() gives a message.
 *
 * Per-particle unknown layouts (`layout`): 78 = the reference's [E_ij | E_ijp | E_ijpq]
 * (configElastic3D.cpp:160-195); 24 = orders 0 and 1 only (the same entries, truncated);
 * 60 = order-2 coefficients stored once per symmetric pair p <= q.
 */
#ifndef IBEM_GB300_H
#define IBEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  IBEM_OK = 0,
  IBEM_ERR_ARG = 1,      /* invalid argument (sizes, layout, null pointer) */
  IBEM_ERR_CUDA = 2,     /* a CUDA runtime call or kernel launch failed */
  IBEM_ERR_NOCONV = 3,   /* iterative refinement did not reach the tolerance */
  IBEM_ERR_TIMEOUT = 4,  /* a device-side wait gave up (kernel returned early) */
  IBEM_ERR_SINGULAR = 5, /* a zero pivot was met */
  IBEM_ERR_IO = 6        /* an input file could not be read or parsed */
} ibem_status;

/* Materials: E0, nu0 of the matrix (BEM.txt lines 2-3), E1, nu1 of the particles
 * (position.txt); configElastic3D.cpp:27-30, 56, 118. */
typedef struct {
  double E0, nu0, E1, nu1;
} ibem_material;

/* Message of the last failing call on this host thread. */
const char* ibem_last_error(void);

/* Number of kernels this library has launched since it was loaded (all threads). */
long long ibem_kernel_launches(void);

/* Phase profiler: with profiling on, CUDA events are recorded on the launching stream around
 * each phase (pair blocks, field sums, panels, row exchanges, tensor-core GEMMs, ...);
 * ibem_prof_enable(1) also clears what was recorded.  ibem_prof_report writes a JSON object
 * {"phase": {"launches", "ms", "flops"}} into buf (synchronising the events) and returns its
 * length.  Instrumentation for measurement; no reference counterpart. */
void ibem_prof_enable(int on);
int ibem_prof_report(char* buf, int cap);

/* Number of unknowns per particle of a layout (24, 60, 78), or -1. */
int ibem_layout_size(int layout);

/* ---- integrator (integratorElastic3D.cpp) -------------------------------- */

/* Inclusion <-> inclusion equivalence blocks, all orders of `layout`, self terms
 * included: replaces integratorElastic3D::addFluxEquivalentInclusion,
 * ::addFluxEquivalentFirstOrderInclusion and ::addFluxEquivalentSecondOrderInclusion
 * (integratorElastic3D.cpp:341-682).  Writes the (layout*num)^2 block at
 * A_dev[(col0 + c) * lda + row0 + r]. */
ibem_status ibem_e3d_pair_blocks(const double* centers_dev, const double* radius_dev, int num,
                                 const ibem_material* mat, int layout, double* A_dev,
                                 int64_t lda, int64_t row0, int64_t col0, void* stream);

/* Inclusion -> boundary-node rows: replaces integratorElastic3D::addFieldToBEM
 * (integratorElastic3D.cpp:135-340).  Writes H[(col0 + layout*K + c) * ldh + row0 + 3j + q]
 * for every node j and particle K. */
ibem_status ibem_e3d_node_blocks(const double* nodes_dev, int NN, const double* centers_dev,
                                 const double* radius_dev, int num, const ibem_material* mat,
                                 int layout, double* H_dev, int64_t ldh, int64_t row0,
                                 int64_t col0, void* stream);

/* ---- BEMBuilder (BEMBuilderElastic3D.cpp) -------------------------------- */

/* Classical Q4 BEM matrices with the rigid-body diagonal: replaces
 * BEMBuilderElastic3D::addBEM (BEMBuilderElastic3D.cpp:1355-1509).  H is the 3NN x 3NN
 * block at H_dev[(hcol0 + c) * ldh + hrow0 + r] (overwritten), G the 3NN x 12NE block at
 * G_dev[(gcol0 + c) * ldg + grow0 + r] (overwritten). */
ibem_status ibem_e3d_bem_hg(const double* nodes_dev, int NN, const int* conn_dev, int NE,
                            const ibem_material* mat, double* H_dev, int64_t ldh, int64_t hrow0,
                            int64_t hcol0, double* G_dev, int64_t ldg, int64_t grow0,
                            int64_t gcol0, void* stream);

/* Boundary -> inclusion rows of orders 0..2: replaces
 * BEMBuilderElastic3D::addFluxEquivalentBEM, ::addFluxEquivalentFirstOrderBEM and
 * ::addFluxEquivalentSecondOrderBEM (BEMBuilderElastic3D.cpp:1511-1867).
 * H rows row0 + layout*K + r, boundary columns hcol0 + 3*node + dof, are decremented
 * (H -= DDsu); G rows, columns gcol0 + 12e + k, are overwritten (G = DDst). */
ibem_status ibem_e3d_bem_to_incl(const double* nodes_dev, int NN, const int* conn_dev, int NE,
                                 const double* centers_dev, int num, const ibem_material* mat,
                                 int layout, double* H_dev, int64_t ldh, int64_t hcol0,
                                 double* G_dev, int64_t ldg, int64_t gcol0, int64_t row0,
                                 void* stream);

/* Boundary-condition plan of ApplyBC (BEMBuilderElastic3D.cpp:1920-2051), computed on
 * the host from BC (3NN x 2, row-major) and t_bc (NE x 24, row-major):
 *   ucol[3NN]   column of A taking H column j when the displacement is unknown, else -1
 *   tcol[12NE]  column of A accumulating -G column (12e+i) when the traction is unknown,
 *               else -1 (unknown tractions are shared per (node, dof), first-seen order)
 * Returns IBEM_ERR_ARG if the number of boundary unknowns is not 3NN. Host memory only. */
ibem_status ibem_e3d_bc_plan(int NN, int NE, const int* conn, const double* bc,
                             const double* tbc, int* ucol, int* tcol);

/* ApplyBC on the device from the plan: A (N x N) and b (N) are overwritten.
 * N = 3NN + layout*num; H is N x N, G is N x 12NE. */
ibem_status ibem_e3d_apply_bc(int NN, int NE, int64_t N, const int* ucol_dev,
                              const int* tcol_dev, const double* bc_dev, const double* tbc_dev,
                              const double* H_dev, int64_t ldh, const double* G_dev,
                              int64_t ldg, double* A_dev, int64_t lda, double* b_dev,
                              void* stream);

/* getUTVector (BEMBuilderElastic3D.cpp:2053-2117): X -> U (N) and T (12NE). */
ibem_status ibem_e3d_get_ut(int NN, int NE, int64_t N, const int* ucol_dev, const int* tcol_dev,
                            const double* bc_dev, const double* tbc_dev, const double* X_dev,
                            double* U_dev, double* T_dev, void* stream);

/* Far-field right-hand side (no reference counterpart: the reference is loaded only
 * through the boundary): b[layout*K + r] = (C0 - C1) : C0^-1 : sigma_inf for order-0
 * rows, 0 otherwise.  sig_inf = (xx, xy, xz, yy, yz, zz) in host memory. */
ibem_status ibem_e3d_farfield_rhs(int num, const ibem_material* mat, int layout,
                                  const double* sig_inf, double* b_dev, void* stream);

/* ---- systemSolver (systemSolverElastic3D.h) ------------------------------- */

typedef enum {
  IBEM_SOLVE_FP64 = 0,     /* equilibrated partial-pivot LU in FP64 (plain path) */
  IBEM_SOLVE_MIXED_IR = 1  /* FP32 LU, split-BF16 tensor-core updates, FP64 GMRES-IR */
} ibem_solver_form;

typedef struct {
  /* backward error of the equilibrated system As ys = bs (As = R A C, bs = R b, x = C ys,
   * R and C the row/column max scalings): ||bs - As ys|| / (||As|| ||ys|| + ||bs||), inf-norms */
  double backward_error;
  int iterations;          /* refinement / GMRES iterations (0 for FP64) */
  int info;                /* 0, or the first zero pivot (1-based) */
  double t_factor_ms, t_solve_ms;
} ibem_solve_report;

/* Solve A x = b in place of systemSolverElastic3D::solve (systemSolverElastic3D.h:44-60,
 * X = A.fullPivLu().solve(b)).  A_dev (N x N, column-major, lda) is overwritten by
 * factors (FP64 form) or left intact (mixed form); x_dev receives the solution.
 * Workspace is allocated internally and released before return. Synchronous. */
ibem_status ibem_e3d_solve(ibem_solver_form form, int64_t N, double* A_dev, int64_t lda,
                           const double* b_dev, double* x_dev, double tol,
                           ibem_solve_report* report, void* stream);

/* The trailing-update primitive of the mixed-precision factorisation, exposed for
 * testing and reuse: C (m x n) -= A (m x k) B (k x n), FP32 column-major storage,
 * computed on the tcgen05 tensor cores with each operand split into two BF16 terms
 * (hi*hi + hi*lo + lo*hi, FP32 accumulation).  Allocates its scratch; synchronous.
 * No reference counterpart (the reference's LU is Eigen's, on the CPU). */
ibem_status ibem_gemm_sub_f32(int64_t m, int64_t n, int64_t k, const float* A_dev, int64_t lda,
                              const float* B_dev, int64_t ldb, float* C_dev, int64_t ldc, void* stream);

/* The plain FP64 solve of ibem_e3d_solve for callers that may not allocate device
 * memory; it has no counterpart in the reference.  Meant for code whose device memory
 * belongs to a host framework (a caching allocator or a budget reserved up front, where a
 * raw cudaMalloc can fail or fragment that budget) and for latency-critical loops, where
 * cudaMalloc/cudaFree can stall the device.  The caller owns A_dev (left intact), b_dev
 * and x_dev; the rest of the workspace is one static device array of about 11 MB inside
 * the library, held by every GPU that loads it until the process exits, which limits N
 * to 1024 (larger N returns IBEM_ERR_ARG).  The first call on a device looks the array's
 * address up (setup), so make it before any stream capture.  Every call reuses the same
 * array: calls that overlap on the GPU (from several host threads or streams) race and
 * must be serialised by the caller.  Synchronous; report gets the scaled backward error
 * and info as for ibem_e3d_solve (timings are left 0). */
ibem_status ibem_e3d_solve_noalloc(int64_t N, const double* A_dev, int64_t lda, const double* b_dev,
                                   double* x_dev, ibem_solve_report* report, void* stream);

/* ---- postProcessor (postProcessorElastic3D.cpp) -------------------------- */

/* Stress at sample points: replaces postProcessorElastic3D::getFlux
 * (postProcessorElastic3D.cpp:224-587): boundary part from U and T
 * (post_stress_BEM, :224-365; skipped when NE == 0, in which case sig_inf, host
 * memory, is the remote stress) plus the sum over all particles of the
 * eigenstrain fields, less the local eigenstrain inside a particle, through C0.
 * E_dev holds layout*num coefficients; stress_dev is nump x 6 (xx xy xz yy yz zz). */
ibem_status ibem_e3d_field(const double* points_dev, int nump, const double* centers_dev,
                           const double* radius_dev, int num, const ibem_material* mat,
                           int layout, const double* E_dev, const double* nodes_dev, int NN,
                           const int* conn_dev, int NE, const double* U_dev,
                           const double* T_dev, const double* sig_inf, double* stress_dev,
                           void* stream);

/* ibem_e3d_field with a precision choice (no counterpart in the reference, which has one
 * precision).  IBEM_SOLVE_FP64 is ibem_e3d_field.  IBEM_SOLVE_MIXED_IR runs the sphere
 * sums of the 24-unknown layout in double-float arithmetic (pairs of FP32 numbers, about
 * 48 significant bits; agrees with the FP64 sums to ~1e-12 of the strain), which GB300
 * executes several times faster than FP64; the 60/78 layouts and the boundary part stay
 * FP64.  ibem_e3d_run_host / ibem_e3d_run_dir use the form given to them here too. */
ibem_status ibem_e3d_field_form(ibem_solver_form form, const double* points_dev, int nump,
                                const double* centers_dev, const double* radius_dev, int num,
                                const ibem_material* mat, int layout, const double* E_dev,
                                const double* nodes_dev, int NN, const int* conn_dev, int NE,
                                const double* U_dev, const double* T_dev, const double* sig_inf,
                                double* stress_dev, void* stream);

/* ---- whole pipeline on host buffers --------------------------------------- */

/* One call per input case with host arrays, for FFI callers: assembly, ApplyBC,
 * solve, getUTVector and stresses, with all host<->device copies inside.
 * Outputs (host): X (N), stress (nump x 6).  N = 3NN + layout*num. Synchronous. */
ibem_status ibem_e3d_run_host(int layout, ibem_solver_form form, const ibem_material* mat,
                              int NN, const double* nodes, int NE, const int* conn,
                              const double* bc, const double* tbc, int num,
                              const double* centers, const double* radius, int nump,
                              const double* points, const double* sig_inf, double tol,
                              double* X, double* stress, ibem_solve_report* report);

/* Same, reading position.txt, BEM.txt, postprocess.txt (and farfield.txt when the
 * case has no boundary) from `dir` as configElastic3D::setUp does
 * (configElastic3D.cpp:32-197, configElastic3D.h:76-129) and writing stress.txt
 * there as postProcessorElastic3D::getFlux does (:578-585). */
ibem_status ibem_e3d_run_dir(const char* dir, int layout, ibem_solver_form form, double tol,
                             ibem_solve_report* report);

#ifdef __cplusplus
}
#endif

#endif /* IBEM_GB300_H */
