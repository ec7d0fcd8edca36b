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
  IBEM_ERR_NOCONV = 3,   /* iterative refinement did not reach the tolerance (x holds the iterate reached) */
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
  IBEM_SOLVE_MIXED_IR = 1, /* FP32 LU, split-BF16 tensor-core updates, FP64 GMRES-IR */
  IBEM_SOLVE_GMRES_BJ = 2  /* no factorisation: FP64 refinement of FP32-product GMRES,
                            * block-Jacobi preconditioned (ibem_e3d_solve_bj) */
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

/* The block-Jacobi form (IBEM_SOLVE_GMRES_BJ), another form of systemSolverElastic3D::solve
 * for the small far-field systems whose LU is bound by launch latency: A is equilibrated
 * (As = R A C) and copied to FP32, the block x block diagonal blocks of As (block = unknowns
 * per particle, 1..80) are inverted in FP64 and kept in FP32, and iterative refinement runs
 * FP64 residuals bs - As ys, each followed by a GMRES(60) correction with the FP32 copy
 * (products accumulated in FP64), right-preconditioned by the block inverses, until the
 * scaled backward error (as in ibem_solve_report) is <= tol.  A_dev is left intact.
 * report->iterations counts the Arnoldi steps.  Synchronous. */
ibem_status ibem_e3d_solve_bj(int64_t N, int block, const double* A_dev, int64_t lda,
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
 * to 1024 (larger N returns IBEM_ERR_ARG).  The first call on a device sets that device
 * up (launch shapes), so make it before any stream capture; every call looks the array's
 * device address up again (no allocation).  Every call reuses the same array: calls that
 * overlap on the GPU (from several host threads or streams) race and must be serialised
 * by the caller.  The call waits for its stream before it returns (it reads the solve's
 * status back); report gets the scaled backward error and info as for ibem_e3d_solve
 * (timings are left 0). */
/* Self-test of the bounded device-side waits (no reference counterpart; the reference
 * has no device code).  which = 0: one CTA waits, with the panel kernel's flag wait, for a
 * flag that nothing sets; which = 1: one thread waits, with the tensor-core GEMM's mbarrier
 * wait, on a barrier nobody arrives at.  Each wait gives up after `limit` polls
 * (1 .. 2^22, the production limit), raises the kernel's error flag and returns, so the
 * call returns IBEM_ERR_TIMEOUT and the context stays usable.  Synchronous. */
ibem_status ibem_selftest_bounded_wait(int which, long long limit, void* stream);

ibem_status ibem_e3d_solve_noalloc(int64_t N, const double* A_dev, int64_t lda, const double* b_dev,
                                   double* x_dev, ibem_solve_report* report, void* stream);

/* ---- matrix-free solves, batches of realisations (layout 24) --------------- */

/* Several independent microstructures ("realisations", "segments") whose particles are
 * concatenated: particles seg_begin[s] .. seg_begin[s+1]-1 form realisation s and interact
 * only with each other; unknowns of particle p are entries 24p .. 24p+23 of b and x (the
 * layout-24 order of a single-realisation system).  No reference counterpart: the
 * reference solves one microstructure per run (systemSolverElastic3D.h:44-60) with
 * the matrix stored.  A batch of ellipsoids (axes_dev and quats_dev set, radius_dev their
 * longest semi-axes) is solved by ibem_e3d_batch_dense_solve with layout 24 (the
 * matrix-free products take spheres only); ibem_e3d_effective_modulus* uses the ellipsoid
 * volumes. */
typedef struct {
  int nseg;
  const int* seg_begin;          /* host, nseg + 1 offsets, seg_begin[0] = 0 */
  const double* centers_dev;     /* seg_begin[nseg] x 3, row-major */
  const double* radius_dev;      /* seg_begin[nseg] */
  const ibem_material* mats;     /* host, one per realisation */
  const double* axes_dev;        /* ellipsoids: seg_begin[nseg] x 3 semi-axes, or NULL (spheres) */
  const double* quats_dev;       /* ellipsoids: seg_begin[nseg] x 4 unit quaternions (w, x, y, z) */
} ibem_e3d_batch;

typedef enum {
  IBEM_PRECOND_BLOCK_JACOBI = 0, /* inverse of each particle's own 24 x 24 block */
  IBEM_PRECOND_LEARNED = 1,      /* block-Jacobi + GNN-weighted Neumann blocks on the kNN graph */
  IBEM_PRECOND_NEUMANN = 2       /* the same blocks with every weight 1 (no network) */
} ibem_precond;

typedef struct {
  int restart;        /* Krylov basis size of the FP32 GMRES (0 = 50) */
  int max_cycles;     /* GMRES restarts per refinement step (0 = 20) */
  int max_outer;      /* FP64 refinement steps (0 = 8) */
  double tol;         /* target rel_residual (0 = 1e-10) */
  double inner_tol;   /* residual reduction asked of each FP32 GMRES solve (0 = 1e-5) */
  int stepwise;       /* 0: the Arnoldi steps of each GMRES cycle run as one launch of a
                       * captured CUDA graph (a device-side while loop: no host round trip
                       * per step); 1: each step launched from the host, which reads the
                       * count of still-active realisations after it */
} ibem_mf_options;

typedef struct {
  double rel_residual;   /* ||Dr (b - A x)||_2 / ||Dr b||_2, FP64, Dr the row scaling
                          * a_s^order / mu0 that makes every entry O(1) */
  int outer;             /* FP64 residual evaluations / refinement steps */
  int inner;             /* Arnoldi steps (FP32 matrix-free products) */
  double t_setup_ms, t_solve_ms;
} ibem_mf_report;

/* y = A x for the sphere systems of a batch (the matrix ibem_e3d_pair_blocks would
 * assemble for each realisation, layout 24), without storing A: every 24 x 24 pair block is
 * evaluated inside the product, on the scaled system (x and y are converted on the way in
 * and out).  precision 64: the product that decides the solver's convergence (in
 * batches whose largest realisation has 1,280 particles or more, FP64 for the sources within
 * 4 of their radii of a warp's 32 targets and double-float beyond: measured within 1e-15
 * norm-wise of every pair in FP64; FP64 throughout below that);
 * 65: every pair in FP64; 48: double-float (FP32 pairs, ~48 bits, several times faster on
 * GB300); 32: FP32, about 1e-6 relative, in the tile shape the autotuner picks for the
 * solver (ibem_e3d_mf_tile_shape).  x_dev, y_dev: 24 * seg_begin[nseg] doubles. */
ibem_status ibem_e3d_mf_matvec(const ibem_e3d_batch* batch, int precision, const double* x_dev,
                               double* y_dev, void* stream);

/* Solve A x = b for every realisation of a batch without storing A (a form of
 * systemSolverElastic3D::solve, systemSolverElastic3D.h:44-60, for boundary-free far-field
 * cases): iterative refinement in which each correction is an FP32 restarted GMRES on the
 * scaled system with matrix-free FP32 products, right-preconditioned by `pc`
 * (IBEM_PRECOND_LEARNED needs gnn_params_dev from ibem_gnn_train); residuals that drive a
 * correction are double-float matrix-free products and the residual that decides
 * convergence (and rel_residual) is the FP64 matrix-free product.  reports: host array of nseg.  Workspace is allocated internally.
 * Synchronous.  IBEM_ERR_NOCONV if a realisation misses opt->tol. */
ibem_status ibem_e3d_mf_solve(const ibem_e3d_batch* batch, const double* b_dev, double* x_dev,
                              ibem_precond pc, const float* gnn_params_dev,
                              const ibem_mf_options* opt, ibem_mf_report* reports, void* stream);

/* The same for quadratic eigenstrain (layout 60: orders 0, 1 and 2, 60 unknowns per sphere,
 * integratorElastic3D.cpp:341-682) or layout 24: every 60 x 60 pair block is evaluated
 * inside the products from the same generated code as ibem_e3d_pair_blocks(layout 60), in
 * FP32 for the GMRES products and in FP64 for the refinement residuals (both of them; there
 * is no double-float form of layout 60).  Layout 60 takes IBEM_PRECOND_BLOCK_JACOBI only (the
 * realisation's own 60 x 60 block, the same for all its spheres in the scaled system).
 * b_dev, x_dev: layout * seg_begin[nseg] doubles. */
ibem_status ibem_e3d_mf_solve_layout(const ibem_e3d_batch* batch, int layout, const double* b_dev,
                                     double* x_dev, ibem_precond pc, const float* gnn_params_dev,
                                     const ibem_mf_options* opt, ibem_mf_report* reports, void* stream);

/* ibem_e3d_mf_matvec for layout 24 or 60 (layout 60: precision 32 or FP64 for 48, 64, 65). */
ibem_status ibem_e3d_mf_matvec_layout(const ibem_e3d_batch* batch, int layout, int precision,
                                      const double* x_dev, double* y_dev, void* stream);

/* Launch shape the autotuner picks for this batch's products: source slices per target tile
 * of the FP32 product and of the double-float / FP64 products.  The first call for a shape
 * class (log2 buckets of the tile count and of the largest realisation) times the
 * candidates once; the result is cached for the process and used by ibem_e3d_mf_solve.
 * No reference counterpart.  Synchronous. */
ibem_status ibem_e3d_mf_tuning(const ibem_e3d_batch* batch, int* slices_fp32, int* slices_wide,
                               void* stream);

/* The FP32 product's tile shape the same autotuner picks (it times every candidate of the
 * shape class once): targets per CTA (64, 128 or 256), launch form (0: one CTA per (tile,
 * source slice); 1: persistent CTAs, as many as fit on the GPU, over the (tile, slice)
 * items sorted by decreasing cost) and source slices.  No reference counterpart.
 * Synchronous. */
ibem_status ibem_e3d_mf_tile_shape(const ibem_e3d_batch* batch, int* targets_per_cta, int* persistent,
                                   int* slices, void* stream);

/* Far-field right-hand sides of a batch (ibem_e3d_farfield_rhs per realisation, layout 24). */
ibem_status ibem_e3d_batch_farfield_rhs(const ibem_e3d_batch* batch, const double* sig_inf,
                                        double* b_dev, void* stream);

/* The same for any layout (24, 60, 78): realisation s occupies entries
 * layout * seg_begin[s] .. layout * seg_begin[s+1] - 1 of b_dev. */
ibem_status ibem_e3d_batch_farfield_rhs_layout(const ibem_e3d_batch* batch, int layout,
                                               const double* sig_inf, double* b_dev, void* stream);

/* Dense solves of the realisations of a batch, one after another on the stream, for the
 * layouts the matrix-free products do not cover (quadratic eigenstrain, layouts 60 and 78):
 * per realisation its pair blocks (ibem_e3d_pair_blocks) into one N x N matrix sized for
 * the largest realisation and allocated once, then ibem_e3d_solve(form, tol) (the mixed
 * form: FP32 LU with split-BF16 tensor-core updates, FP64 GMRES-IR; IBEM_SOLVE_GMRES_BJ:
 * ibem_e3d_solve_bj with one block per particle).  b_dev, x_dev: layout *
 * seg_begin[nseg] doubles.  reports: host array of nseg (may be NULL).  Synchronous.
 * The reference solves one microstructure per run (systemSolverElastic3D.h:44-60). */
ibem_status ibem_e3d_batch_dense_solve(const ibem_e3d_batch* batch, int layout,
                                       ibem_solver_form form, const double* b_dev, double* x_dev,
                                       double tol, ibem_solve_report* reports, void* stream);

/* Effective response of each realisation under the remote stress sig_inf (host, xx xy xz yy
 * yz zz) from its solution x: mean strain <e> = C0^-1 : sig_inf + sum_p (V_p / volume) E_p
 * (the eigenstrain's order-0 part, whose volume average over a sphere is E_p), written to
 * mean_strain (host nseg x 6, may be NULL), and E_eff = sig_inf[5] / <e_33> to e_eff (host
 * nseg).  volume: host nseg, each realisation's cell volume.  Synchronous. */
ibem_status ibem_e3d_effective_modulus(const ibem_e3d_batch* batch, const double* x_dev,
                                       const double* volume, const double* sig_inf,
                                       double* mean_strain, double* e_eff, void* stream);

/* The same for solutions of any layout: a layout-60/78 particle's eigenstrain
 * E_ij + E_ijk x_k + E_ijkl x_k x_l averages to E_ij + (a^2 / 5) sum_k E_ijkk over its sphere. */
ibem_status ibem_e3d_effective_modulus_layout(const ibem_e3d_batch* batch, int layout,
                                              const double* x_dev, const double* volume,
                                              const double* sig_inf, double* mean_strain,
                                              double* e_eff, void* stream);

/* The boundary-free far-field pipeline of one microstructure on host buffers, for FFI
 * callers (the matrix-free counterpart of ibem_e3d_run_host, layout 24): copies in,
 * far-field right-hand side, ibem_e3d_mf_solve with `pc` (gnn_params: host array of
 * ibem_gnn_param_count() floats, needed for IBEM_PRECOND_LEARNED), stresses at the points
 * (ibem_e3d_field_form, double-float sphere sums) and copies out.  X: 24*num; stress:
 * nump x 6.  Synchronous. */
ibem_status ibem_e3d_run_host_mf(const ibem_material* mat, int num, const double* centers,
                                 const double* radius, int nump, const double* points,
                                 const double* sig_inf, ibem_precond pc, const float* gnn_params,
                                 const ibem_mf_options* opt, double* X, double* stress,
                                 ibem_mf_report* report);

/* ---- binary side-car of a case directory (no reference counterpart) --------- */
/* case.ibemb holds what position.txt, BEM.txt, postprocess.txt (configElastic3D.cpp:32-197,
 * configElastic3D.h:76-129) and farfield.txt hold, in binary (layout in host/sidecar.cpp);
 * ibem_e3d_run_dir, ibem_e3d_case_sizes and ibem_e3d_read_case use it in place of the text
 * files when it is at least as new as each of them.  All host-only and synchronous. */

/* Parse the text files of `dir` and write dir/case.ibemb. */
ibem_status ibem_e3d_sidecar_from_txt(const char* dir);

/* Write a side-car at `path` from host arrays (the layouts of ibem_e3d_run_host;
 * sig_inf may be NULL for a bounded case). */
ibem_status ibem_e3d_sidecar_write(const char* path, const ibem_material* mat, int NN,
                                   const double* nodes, int NE, const int* conn, const double* bc,
                                   const double* tbc, int num, const double* centers,
                                   const double* radius, int nump, const double* points,
                                   const double* sig_inf);

/* sizes[6] = NN, NE, num, nump, has_farfield, read_from_side_car. */
ibem_status ibem_e3d_case_sizes(const char* dir, int64_t* sizes);

/* The inputs of `dir` into host arrays sized by ibem_e3d_case_sizes (arrays of empty blocks
 * may be NULL; sig_inf gets zeros when the case has a boundary). */
ibem_status ibem_e3d_read_case(const char* dir, ibem_material* mat, double* nodes, int* conn,
                               double* bc, double* tbc, double* centers, double* radius,
                               double* points, double* sig_inf);

/* ---- microstructure generator (no reference counterpart) -------------------- */
/* The reference reads centres and radii from position.txt (configElastic3D.cpp:106-128);
 * this makes seeded far-field microstructures without text files. */
typedef enum {
  IBEM_GEN_RSA = 0, /* random sequential addition, every sphere inside the cube */
  IBEM_GEN_MC = 1   /* hard-sphere Monte Carlo from a lattice with box compression, centres in
                     * the cube; reaches volume fractions at which addition jams (30%) */
} ibem_gen_method;

typedef struct {
  int num;            /* spheres */
  double r0;          /* radius scale: radius_k = r0 * U[rlo, rhi] */
  double rlo, rhi;
  double vf;          /* volume fraction: cube side L = (sum of sphere volumes / vf)^(1/3) */
  double gap;         /* centre distance >= r_i + r_j + gap * max(r_i, r_j) */
  int method;         /* ibem_gen_method */
  uint64_t seed;      /* the same seed gives the same microstructure on every platform */
  int64_t max_tries;  /* RSA: candidate centres before giving up (0 = 2e8) */
  int sweeps;         /* MC: sweeps after the target side is reached (0 = 100) */
} ibem_gen_params;

/* Host arrays: centers num x 3 (row-major), radius num; side (may be NULL) gets L.  Runs on
 * the host only.  IBEM_ERR_ARG with a message when the packing cannot be reached. */
ibem_status ibem_e3d_generate_spheres(const ibem_gen_params* p, double* centers, double* radius,
                                      double* side);

/* Seeded ellipsoid microstructures: semi-axes a1, a2 = a1 U[a2lo, a2hi], a3 = a1 U[a3lo, a3hi]
 * (a3 is then the shortest only if a3hi <= a2lo), orientations uniform on SO(3) (Haar,
 * quaternions from three uniforms), cube side L = (sum of volumes / vf)^(1/3).  Two
 * ellipsoids are kept apart by testing them with every semi-axis inflated by gap * a3 / 2
 * (Perram-Wertheim contact function).  method IBEM_GEN_RSA: random sequential addition of
 * centres inside [a1, L - a1]^3 (jams near 20% for the default shapes); IBEM_GEN_MC:
 * hard-ellipsoid Monte Carlo (translations and rotations) with box compression, centres in
 * [0, L]^3, orientations moved from their Haar draws.  Host outputs: centers n x 3, axes
 * n x 3 (a1 a2 a3 along the principal axes), quats n x 4 (w, x, y, z), side (may be NULL).
 * Host only. */
typedef struct {
  int num;
  double a1;
  double a2lo, a2hi, a3lo, a3hi;
  double vf;
  double gap;
  uint64_t seed;
  int64_t max_tries;  /* RSA: candidate centres before giving up (0 = 2e8) */
  int method;         /* ibem_gen_method */
  int sweeps;         /* MC: sweeps after the target side is reached (0 = 50) */
} ibem_ell_gen_params;

ibem_status ibem_e3d_generate_ellipsoids(const ibem_ell_gen_params* p, double* centers, double* axes,
                                         double* quats, double* side);

/* ---- learned preconditioner (no reference counterpart) --------------------- */
/* On the graph of each particle's 16 nearest neighbours (edges e = (i <- j)), with B the
 * block-Jacobi inverses and As the scaled pair blocks, the Neumann series of As^-1 gives
 *   C_e = -B_i As_ij B_j            (first-order term of (As^-1)_ij)
 *   T_e =  B_i As_ij B_j As_ji B_i   (second-order term of (As^-1)_ii from j).
 * The preconditioner is block-sparse on that graph:
 *   (P v)_i = (B_i + sum_e w_e T_e) v_i + sum_e alpha_e C_e v_j,
 * and a message-passing network predicts the two weights (w_e, alpha_e) of every edge.
 * Inputs: node features (dim 10: semi-axes / radius, orientation quaternion, E1/(10 E0),
 * nu0, nu1) and edge features (dim 7: offset / a_i, distance / a_i, a_j / a_i, gap / a_i,
 * (2 a_i / distance)^3).  Network: h = relu(W_in x + b); 3 layers of
 * m_e = relu(W_m [h_i, h_j, f_e] + b), h_i += relu(W_u [h_i, mean_e m_e] + b);
 * (w_e, alpha_e) = W_o2 relu(W_o1 [h_i, h_j, f_e] + b) + b_o2.  Hidden width 64.
 * Parameters: one flat FP32 array of ibem_gnn_param_count() values (W row-major
 * fan-in x fan-out, each followed by its bias, in the order above). */
int64_t ibem_gnn_param_count(void);

/* Seeded initialisation (uniform +-1/sqrt(fan_in); output layer zero, so that the untrained
 * network gives w = alpha = 0, i.e. block-Jacobi). */
ibem_status ibem_gnn_init_params(float* params_dev, uint64_t seed, void* stream);

/* Graph, features and training projections of a batch.  nbr_dev: num*16 ints (-1 when a
 * realisation has fewer than 17 particles); node_feat_dev num*10; edge_feat_dev num*16*7.
 * With nrhs > 0 pairs (r_hat, e_hat) of the scaled system (e_hat = As^-1 r_hat, FP64,
 * nrhs x N each): z_dev (nrhs x N) = B r - e, and u_dev (nrhs x num*16 x 2 x 24) holds
 * (T_e r_i, C_e r_j) for every edge, all divided by sqrt(sum ||e||^2), so that the
 * training loss is the relative squared error of P r against e:
 *   L = sum_q sum_i || z_qi + sum_e (w_e u_qe0 + alpha_e u_qe1) ||^2. */
ibem_status ibem_gnn_prepare(const ibem_e3d_batch* batch, int nrhs, const double* r_hat_dev,
                             const double* e_hat_dev, int* nbr_dev, float* node_feat_dev,
                             float* edge_feat_dev, float* z_dev, float* u_dev, void* stream);

/* Loss L (host) and its gradient with respect to the parameters (grad_dev, overwritten). */
ibem_status ibem_gnn_loss_grad(int num, const int* nbr_dev, const float* node_feat_dev,
                               const float* edge_feat_dev, int nrhs, const float* z_dev,
                               const float* u_dev, const float* params_dev, double* loss,
                               float* grad_dev, void* stream);

/* Edge weights (w_e, alpha_e) of the network, num*16 x 2 (forward pass only). */
ibem_status ibem_gnn_edge_weights(int num, const int* nbr_dev, const float* node_feat_dev,
                                  const float* edge_feat_dev, const float* params_dev, float* w_dev,
                                  void* stream);

/* One AdamW step (decoupled weight decay, bias-corrected moments; step counts from 1). */
ibem_status ibem_gnn_adamw(int64_t n, float* params_dev, const float* grad_dev, float* m_dev,
                           float* v_dev, int step, float lr, float beta1, float beta2, float eps,
                           float weight_decay, void* stream);

/* Full-batch training: prepare, then `steps` AdamW steps (betas 0.9/0.999, eps 1e-8);
 * loss_hist (host, steps + 1) gets the loss before every step and after the last.  Synchronous. */
ibem_status ibem_gnn_train(const ibem_e3d_batch* batch, int nrhs, const double* r_hat_dev,
                           const double* e_hat_dev, float* params_dev, int steps, float lr,
                           float weight_decay, double* loss_hist, void* stream);

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
 * 48 significant bits) for spheres within 12 radii of a warp's points and in FP32 beyond
 * (agrees with the FP64 sums to ~1e-9 of the strain), which GB300 executes several times
 * faster than FP64; the 60/78 layouts and the boundary part stay FP64.
 * ibem_e3d_run_host / ibem_e3d_run_dir use the form given to them here too. */
ibem_status ibem_e3d_field_form(ibem_solver_form form, const double* points_dev, int nump,
                                const double* centers_dev, const double* radius_dev, int num,
                                const ibem_material* mat, int layout, const double* E_dev,
                                const double* nodes_dev, int NN, const int* conn_dev, int NE,
                                const double* U_dev, const double* T_dev, const double* sig_inf,
                                double* stress_dev, void* stream);

/* Grid service: ibem_e3d_field_form at the cell centres of an n[0] x n[1] x n[2] grid over
 * the box [lo, hi] (host arrays of 3), generated on the device instead of read from a
 * point list (postprocess.txt of a grid, configElastic3D.h:116-129): point (i, j, k) =
 * lo + ((i, j, k) + 1/2) (hi - lo) / n, x fastest; stress_dev: n[0] n[1] n[2] x 6. */
ibem_status ibem_e3d_field_grid(ibem_solver_form form, const double* lo, const double* hi,
                                const int* n, const double* centers_dev, const double* radius_dev,
                                int num, const ibem_material* mat, int layout, const double* E_dev,
                                const double* nodes_dev, int NN, const int* conn_dev, int NE,
                                const double* U_dev, const double* T_dev, const double* sig_inf,
                                double* stress_dev, void* stream);

/* ---- ellipsoidal inclusions (layout 24, boundary-free cases) ---------------- */

/* No reference counterpart: the reference's elastic integrator treats spheres only
 * (integratorElastic3DHelper.cpp:41-664).  An ellipsoid h has a centre (centers_dev, n x 3),
 * semi-axes a1, a2, a3 (axes_dev, n x 3) along its principal axes, and an orientation
 * (quats_dev, n x 4: unit quaternion w, x, y, z taking the principal frame to the global
 * one; normalised on use).  Unknowns per particle: the 24 of layout 24 (E_ij, E_ijp) in
 * global coordinates about the centre.  For a1 = a2 = a3 every result equals the sphere
 * entry point's.  Device pointers; up to 65535 ellipsoids per call. */

/* Pair blocks of the equivalent-inclusion rows (the ellipsoid counterpart of
 * ibem_e3d_pair_blocks with layout 24; integratorElastic3D.cpp:341-567): the (24 num)^2
 * block at A[row0.., col0..] (column-major, lda), FP64. */
ibem_status ibem_e3d_ell_pair_blocks(const double* centers_dev, const double* axes_dev, const double* quats_dev,
                                     int num, const ibem_material* mat, double* A_dev, int64_t lda, int64_t row0,
                                     int64_t col0, void* stream);

/* Stresses at sample points under the remote stress sig_inf (host, 6) from the layout-24
 * eigenstrain E_dev (postProcessorElastic3D.cpp:367-522 with ellipsoids): stress_dev is
 * overwritten (nump x 6, xx xy xz yy yz zz).  form IBEM_SOLVE_FP64: FP64 throughout;
 * IBEM_SOLVE_MIXED_IR: an ellipsoid farther than 14 of its longest semi-axes from all 32
 * points of a warp is evaluated in FP32, the others in FP64. */
ibem_status ibem_e3d_ell_field(ibem_solver_form form, const double* points_dev, int nump, const double* centers_dev,
                               const double* axes_dev, const double* quats_dev, int num, const ibem_material* mat,
                               const double* E_dev, const double* sig_inf, double* stress_dev, void* stream);

/* Whole boundary-free ellipsoid pipeline on host arrays (pair blocks, far-field right-hand
 * side, dense solve in `form` (IBEM_SOLVE_FP64 or IBEM_SOLVE_MIXED_IR), stresses), all
 * copies inside: X (24 num) and stress (nump x 6) are host outputs.  Synchronous. */
ibem_status ibem_e3d_run_host_ell(ibem_solver_form form, const ibem_material* mat, int num, const double* centers,
                                  const double* axes, const double* quats, int nump, const double* points,
                                  const double* sig_inf, double tol, double* X, double* stress,
                                  ibem_solve_report* report);

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
