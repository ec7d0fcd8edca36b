// extern "C" entry points of libibem_gb300.so (declared in include/ibem_gb300.h).
#include <cuda_runtime.h>

#include <cstdint>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ibem_internal.h"
#include "solver.h"

namespace ibem {

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};

int count_launch() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return 0;
}
void add_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches_so_far() { return g_launches.load(); }

ibem_status fail(ibem_status st, const std::string& msg) {
  g_last_error = msg;
  return st;
}

ibem_status cuda_fail(cudaError_t e, const char* where) {
  g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return IBEM_ERR_CUDA;
}

static bool valid_layout(int layout) { return layout == 24 || layout == 60 || layout == 78; }

static SphLaunch sph(const double* cen, const double* rad, int num, const ibem_material* m) {
  SphLaunch p;
  p.cen = cen;
  p.rad = rad;
  p.num = num;
  p.E0 = m->E0;
  p.nu0 = m->nu0;
  p.E1 = m->E1;
  p.nu1 = m->nu1;
  return p;
}

namespace {

// A boundary columns from the ApplyBC plan (BEMBuilderElastic3D.cpp:1957-2018)
__global__ void k_bc_ucols(int64_t N, int n3, const int* __restrict__ ucol, const double* __restrict__ H,
                           int64_t ldh, double* __restrict__ A, int64_t lda) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= N) return;
  for (int j = blockIdx.y; j < n3; j += gridDim.y) {
    const int c = ucol[j];
    if (c >= 0) A[(int64_t)c * lda + i] = H[(int64_t)j * ldh + i];
  }
}
__global__ void k_bc_tcols(int64_t N, int nt, const int* __restrict__ tcol, const double* __restrict__ G,
                           int64_t ldg, double* __restrict__ A, int64_t lda) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (i >= N || k >= nt) return;
  const int c = tcol[k];
  if (c >= 0) atomicAdd(A + (int64_t)c * lda + i, -G[(int64_t)k * ldg + i]);
}
// b = - sum_{u prescribed} H(:,j) u_j + sum_{t prescribed} t_k G(:,k)   (:1967-1995)
__global__ void k_bc_rhs(int64_t N, int n3, int nt, const double* __restrict__ bc, const double* __restrict__ tbc,
                         const double* __restrict__ H, int64_t ldh, const double* __restrict__ G, int64_t ldg,
                         double* __restrict__ b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= N) return;
  double s = 0;
  for (int j = 0; j < n3; ++j)
    if (bc[2 * j] == 0) s -= H[(int64_t)j * ldh + i] * bc[2 * j + 1];
  for (int k = 0; k < nt; ++k) {
    const int e = k / 12, ii = k % 12;
    if (tbc[24 * e + ii] == 1) s += tbc[24 * e + 12 + ii] * G[(int64_t)k * ldg + i];
  }
  b[i] = s;
}
__global__ void k_get_ut(int n3, int64_t N, int nt, const int* __restrict__ ucol, const int* __restrict__ tcol,
                         const double* __restrict__ bc, const double* __restrict__ tbc, const double* __restrict__ X,
                         double* __restrict__ U, double* __restrict__ T) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < N) {
    if (i < n3) U[i] = (ucol[i] >= 0) ? X[ucol[i]] : bc[2 * i + 1];
    else U[i] = X[i];
  }
  if (i < nt) {
    const int e = (int)(i / 12), ii = (int)(i % 12);
    T[i] = (tcol[i] >= 0) ? X[tcol[i]] : tbc[24 * e + 12 + ii];
  }
}
struct FarRhs {
  double v[6];
};
__global__ void k_farfield(int num, int nu, FarRhs f, double* __restrict__ b) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)num * nu) return;
  const int r = (int)(t % nu);
  b[t] = r < 6 ? f.v[r] : 0.0;
}
__global__ void k_fill6(int nump, FarRhs f, double* __restrict__ s) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < (int64_t)nump * 6) s[t] = f.v[t % 6];
}

struct GridSpec {
  double lo[3], span[3];
  int n[3];
};
// cell-centred grid points, x fastest: lo + ((i, j, k) + 1/2) / n * (hi - lo), the order of
// operations of cases.cell_grid
__global__ void k_grid_points(int64_t nump, GridSpec g, double* __restrict__ pts) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nump) return;
  const int64_t idx[3] = {t % g.n[0], (t / g.n[0]) % g.n[1], t / ((int64_t)g.n[0] * g.n[1])};
#pragma unroll
  for (int d = 0; d < 3; ++d)  // rounded operation by operation (no fused multiply-add): a host grid matches
    pts[3 * t + d] = __dadd_rn(g.lo[d], __dmul_rn(__ddiv_rn((double)idx[d] + 0.5, (double)g.n[d]), g.span[d]));
}
}  // namespace
}  // namespace ibem

using namespace ibem;


extern "C" {

const char* ibem_last_error(void) { return g_last_error.c_str(); }

long long ibem_kernel_launches(void) { return g_launches.load(); }

int ibem_layout_size(int layout) { return valid_layout(layout) ? layout : -1; }

ibem_status ibem_e3d_pair_blocks(const double* centers_dev, const double* radius_dev, int num,
                                 const ibem_material* mat, int layout, double* A_dev, int64_t lda,
                                 int64_t row0, int64_t col0, void* stream) {
  if (!mat || !valid_layout(layout) || num < 0 || (num && (!centers_dev || !radius_dev || !A_dev)))
    return fail(IBEM_ERR_ARG, "pair_blocks: bad arguments");
  if (num > 65535) return fail(IBEM_ERR_ARG, "pair_blocks: at most 65535 particles per call");
  if (lda < row0 + (int64_t)layout * num) return fail(IBEM_ERR_ARG, "pair_blocks: lda too small");
  if (num == 0) return IBEM_OK;
  SphLaunch p = sph(centers_dev, radius_dev, num, mat);
  cudaStream_t st = as_stream(stream);
  if (layout == 24) return launch_pair24(p, A_dev, lda, row0, col0, st);
  if (layout == 60) return launch_pair60(p, A_dev, lda, row0, col0, st);
  return launch_pair78(p, A_dev, lda, row0, col0, st);
}

ibem_status ibem_e3d_node_blocks(const double* nodes_dev, int NN, const double* centers_dev,
                                 const double* radius_dev, int num, const ibem_material* mat,
                                 int layout, double* H_dev, int64_t ldh, int64_t row0,
                                 int64_t col0, void* stream) {
  if (!mat || !valid_layout(layout) || NN < 0 || num < 0) return fail(IBEM_ERR_ARG, "node_blocks: bad arguments");
  if (num > 65535) return fail(IBEM_ERR_ARG, "node_blocks: at most 65535 particles per call");
  if (ldh < row0 + 3 * (int64_t)NN) return fail(IBEM_ERR_ARG, "node_blocks: ldh too small");
  if (NN == 0 || num == 0) return IBEM_OK;
  SphLaunch p = sph(centers_dev, radius_dev, num, mat);
  cudaStream_t st = as_stream(stream);
  if (layout == 24) return launch_node24(p, nodes_dev, NN, H_dev, ldh, row0, col0, st);
  if (layout == 60) return launch_node60(p, nodes_dev, NN, H_dev, ldh, row0, col0, st);
  return launch_node78(p, nodes_dev, NN, H_dev, ldh, row0, col0, st);
}

ibem_status ibem_e3d_bem_hg(const double* nodes_dev, int NN, const int* conn_dev, int NE,
                            const ibem_material* mat, double* H_dev, int64_t ldh, int64_t hrow0,
                            int64_t hcol0, double* G_dev, int64_t ldg, int64_t grow0,
                            int64_t gcol0, void* stream) {
  if (!mat || NN <= 0 || NE <= 0 || !nodes_dev || !conn_dev || !H_dev || !G_dev)
    return fail(IBEM_ERR_ARG, "bem_hg: bad arguments");
  if (NE > 65535) return fail(IBEM_ERR_ARG, "bem_hg: at most 65535 elements");
  if (ldh < hrow0 + 3 * (int64_t)NN || ldg < grow0 + 3 * (int64_t)NN) return fail(IBEM_ERR_ARG, "bem_hg: ld too small");
  return bem_hg(nodes_dev, NN, conn_dev, NE, *mat, H_dev, ldh, hrow0, hcol0, G_dev, ldg, grow0, gcol0,
                as_stream(stream));
}

ibem_status ibem_e3d_bem_to_incl(const double* nodes_dev, int NN, const int* conn_dev, int NE,
                                 const double* centers_dev, int num, const ibem_material* mat,
                                 int layout, double* H_dev, int64_t ldh, int64_t hcol0,
                                 double* G_dev, int64_t ldg, int64_t gcol0, int64_t row0,
                                 void* stream) {
  if (!mat || !valid_layout(layout) || NN <= 0 || NE <= 0 || num < 0)
    return fail(IBEM_ERR_ARG, "bem_to_incl: bad arguments");
  if (NE > 65535) return fail(IBEM_ERR_ARG, "bem_to_incl: at most 65535 elements");
  if (ldh < row0 + (int64_t)layout * num || ldg < row0 + (int64_t)layout * num)
    return fail(IBEM_ERR_ARG, "bem_to_incl: ld too small");
  if (num == 0) return IBEM_OK;
  return bem_to_incl(nodes_dev, NN, conn_dev, NE, centers_dev, num, *mat, layout, H_dev, ldh, hcol0, G_dev, ldg,
                     gcol0, row0, as_stream(stream));
}

ibem_status ibem_e3d_bc_plan(int NN, int NE, const int* conn, const double* bc, const double* tbc,
                             int* ucol, int* tcol) {
  if (NN < 0 || NE < 0 || (NN && (!bc || !ucol)) || (NE && (!conn || !tbc || !tcol)))
    return fail(IBEM_ERR_ARG, "bc_plan: bad arguments");
  const int n3 = 3 * NN;
  int t = 0;
  for (int j = 0; j < n3; ++j) {
    if (bc[2 * j] != 0 && bc[2 * j] != 1) return fail(IBEM_ERR_ARG, "bc_plan: displacement flag not 0/1");
    ucol[j] = (bc[2 * j] == 1) ? t++ : -1;
  }
  std::vector<int> key((size_t)n3, -1);
  for (int e = 0; e < NE; ++e)
    for (int i = 0; i < 12; ++i) {
      const double f = tbc[24 * e + i];
      tcol[12 * e + i] = -1;
      if (f == 1) continue;
      if (f != 0) return fail(IBEM_ERR_ARG, "bc_plan: traction flag not 0/1");
      const int node = conn[4 * e + i / 3];
      if (node < 1 || node > NN) return fail(IBEM_ERR_ARG, "bc_plan: connectivity out of range");
      const int kk = 3 * (node - 1) + i % 3;
      if (key[kk] < 0) key[kk] = t++;
      tcol[12 * e + i] = key[kk];
    }
  if (t != n3) {
    char buf[160];
    std::snprintf(buf, sizeof buf, "bc_plan: %d boundary unknowns for %d boundary equations", t, n3);
    return fail(IBEM_ERR_ARG, buf);
  }
  return IBEM_OK;
}

ibem_status ibem_e3d_apply_bc(int NN, int NE, int64_t N, const int* ucol_dev, const int* tcol_dev,
                              const double* bc_dev, const double* tbc_dev, const double* H_dev,
                              int64_t ldh, const double* G_dev, int64_t ldg, double* A_dev,
                              int64_t lda, double* b_dev, void* stream) {
  const int n3 = 3 * NN, nt = 12 * NE;
  if (NN <= 0 || NE <= 0 || N < n3 || lda < N || ldh < N || ldg < N)
    return fail(IBEM_ERR_ARG, "apply_bc: bad sizes");
  if (n3 > 65535 || nt > 65535 * 4) return fail(IBEM_ERR_ARG, "apply_bc: boundary too large for one call");
  cudaStream_t st = as_stream(stream);
  IBEM_CUDA(cudaMemset2DAsync(A_dev, lda * sizeof(double), 0, N * sizeof(double), n3, st));
  const unsigned gx = (unsigned)((N + 255) / 256);
  ::ibem::count_launch(), k_bc_ucols<<<dim3(gx, std::min(n3, 65535)), 256, 0, st>>>(N, n3, ucol_dev, H_dev, ldh, A_dev, lda);
  for (int k0 = 0; k0 < nt; k0 += 65535) {
    const int cnt = std::min(65535, nt - k0);
    ::ibem::count_launch(), k_bc_tcols<<<dim3(gx, cnt), 256, 0, st>>>(N, cnt, tcol_dev + k0, G_dev + (int64_t)k0 * ldg, ldg, A_dev, lda);
  }
  ::ibem::count_launch(), k_bc_rhs<<<gx, 256, 0, st>>>(N, n3, nt, bc_dev, tbc_dev, H_dev, ldh, G_dev, ldg, b_dev);
  if (N > n3)
    IBEM_CUDA(cudaMemcpy2DAsync(A_dev + (int64_t)n3 * lda, lda * sizeof(double), H_dev + (int64_t)n3 * ldh,
                                ldh * sizeof(double), N * sizeof(double), N - n3, cudaMemcpyDeviceToDevice, st));
  IBEM_LAUNCH_CHECK("apply_bc");
  return IBEM_OK;
}

ibem_status ibem_e3d_get_ut(int NN, int NE, int64_t N, const int* ucol_dev, const int* tcol_dev,
                            const double* bc_dev, const double* tbc_dev, const double* X_dev,
                            double* U_dev, double* T_dev, void* stream) {
  if (NN < 0 || NE < 0 || N < 3 * (int64_t)NN) return fail(IBEM_ERR_ARG, "get_ut: bad sizes");
  const int64_t n = std::max<int64_t>(N, 12 * (int64_t)NE);
  ::ibem::count_launch(), k_get_ut<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(3 * NN, N, 12 * NE, ucol_dev, tcol_dev,
                                                                       bc_dev, tbc_dev, X_dev, U_dev, T_dev);
  IBEM_LAUNCH_CHECK("get_ut");
  return IBEM_OK;
}

ibem_status ibem_e3d_farfield_rhs(int num, const ibem_material* mat, int layout,
                                  const double* sig_inf, double* b_dev, void* stream) {
  if (!mat || !sig_inf || !valid_layout(layout) || num < 0) return fail(IBEM_ERR_ARG, "farfield_rhs: bad arguments");
  // eps = C0^-1 : sigma (isotropic compliance), rhs_ij = (C0 - C1) : eps  for i <= j
  const double S[3][3] = {{sig_inf[0], sig_inf[1], sig_inf[2]},
                          {sig_inf[1], sig_inf[3], sig_inf[4]},
                          {sig_inf[2], sig_inf[4], sig_inf[5]}};
  const double tr = S[0][0] + S[1][1] + S[2][2];
  double eps[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) eps[i][j] = ((1 + mat->nu0) * S[i][j] - mat->nu0 * tr * (i == j)) / mat->E0;
  const double mu0 = mat->E0 / (2 * (1 + mat->nu0)), mu1 = mat->E1 / (2 * (1 + mat->nu1));
  const double l0 = 2 * mu0 * mat->nu0 / (1 - 2 * mat->nu0), l1 = 2 * mu1 * mat->nu1 / (1 - 2 * mat->nu1);
  const double etr = eps[0][0] + eps[1][1] + eps[2][2];
  FarRhs f;
  int r = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j, ++r) f.v[r] = (l0 - l1) * etr * (i == j) + 2 * (mu0 - mu1) * eps[i][j];
  if (num == 0) return IBEM_OK;
  const int64_t n = (int64_t)num * layout;
  ::ibem::count_launch(), k_farfield<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(num, layout, f, b_dev);
  IBEM_LAUNCH_CHECK("farfield_rhs");
  return IBEM_OK;
}

ibem_status ibem_e3d_solve(ibem_solver_form form, int64_t N, double* A_dev, int64_t lda,
                           const double* b_dev, double* x_dev, double tol,
                           ibem_solve_report* report, void* stream) {
  if (form == IBEM_SOLVE_GMRES_BJ) return fail(IBEM_ERR_ARG, "solve: the block-Jacobi form is ibem_e3d_solve_bj");
  return solve_dense(form, N, A_dev, lda, b_dev, x_dev, tol, report, as_stream(stream));
}

ibem_status ibem_e3d_solve_bj(int64_t N, int block, const double* A_dev, int64_t lda, const double* b_dev,
                              double* x_dev, double tol, ibem_solve_report* report, void* stream) {
  // the block-Jacobi form reads A and never writes it
  return solve_dense(IBEM_SOLVE_GMRES_BJ, N, const_cast<double*>(A_dev), lda, b_dev, x_dev, tol, report,
                     as_stream(stream), block);
}

ibem_status ibem_gemm_sub_f32(int64_t m, int64_t n, int64_t k, const float* A_dev, int64_t lda,
                              const float* B_dev, int64_t ldb, float* C_dev, int64_t ldc, void* stream) {
  if (m < 0 || n < 0 || k < 0 || lda < m || ldb < k || ldc < m) return fail(IBEM_ERR_ARG, "gemm_sub_f32: bad sizes");
  if (m == 0 || n == 0 || k == 0) return IBEM_OK;
  cudaStream_t st = as_stream(stream);
  const size_t ws_bytes = gemm_tc_workspace_bytes(m, n);
  void* ws = nullptr;
  int* err = nullptr;
  IBEM_CUDA(cudaMalloc(&ws, ws_bytes));
  cudaError_t ce = cudaMalloc(&err, sizeof(int));
  if (ce != cudaSuccess) { cudaFree(ws); return cuda_fail(ce, "gemm_sub_f32"); }
  ibem_status s = IBEM_OK;
  ce = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (ce != cudaSuccess) s = cuda_fail(ce, "gemm_sub_f32");
  if (!s) s = gemm_sub_f32_tc(m, n, k, A_dev, lda, B_dev, ldb, C_dev, ldc, ws, ws_bytes, err, st);
  int herr = 0;
  if (!s) {
    ce = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) s = cuda_fail(ce, "gemm_sub_f32");
    else if (herr) s = fail(IBEM_ERR_TIMEOUT, "gemm_sub_f32: a device-side wait gave up");
  }
  cudaFree(ws);
  cudaFree(err);
  return s;
}

ibem_status ibem_selftest_bounded_wait(int which, long long limit, void* stream) {
  if (which == 0) return selftest_flag_wait(limit, as_stream(stream));
  if (which == 1) return selftest_mbar_wait(limit, as_stream(stream));
  return fail(IBEM_ERR_ARG, "selftest_bounded_wait: which must be 0 (panel flag) or 1 (GEMM mbarrier)");
}

ibem_status ibem_e3d_solve_noalloc(int64_t N, const double* A_dev, int64_t lda, const double* b_dev,
                                   double* x_dev, ibem_solve_report* report, void* stream) {
  return solve_fp64_noalloc(N, A_dev, lda, b_dev, x_dev, report, as_stream(stream));
}

ibem_status ibem_e3d_field_form(ibem_solver_form form, const double* points_dev, int nump,
                                const double* centers_dev, const double* radius_dev, int num,
                                const ibem_material* mat, int layout, const double* E_dev,
                                const double* nodes_dev, int NN, const int* conn_dev, int NE,
                                const double* U_dev, const double* T_dev, const double* sig_inf,
                                double* stress_dev, void* stream) {
  if (!mat || !valid_layout(layout) || nump < 0 || num < 0) return fail(IBEM_ERR_ARG, "field: bad arguments");
  if (form != IBEM_SOLVE_FP64 && form != IBEM_SOLVE_MIXED_IR) return fail(IBEM_ERR_ARG, "field: unknown form");
  if (nump == 0) return IBEM_OK;
  cudaStream_t st = as_stream(stream);
  if (NE > 0) {
    ibem_status s = bem_post(points_dev, nump, nodes_dev, NN, conn_dev, NE, *mat, U_dev, T_dev, stress_dev, st,
                             form == IBEM_SOLVE_MIXED_IR);
    if (s) return s;
  } else {
    FarRhs f;
    for (int i = 0; i < 6; ++i) f.v[i] = sig_inf ? sig_inf[i] : 0.0;
    ::ibem::count_launch(), k_fill6<<<(unsigned)(((int64_t)nump * 6 + 255) / 256), 256, 0, st>>>(nump, f, stress_dev);
    IBEM_LAUNCH_CHECK("field init");
  }
  if (num == 0) return IBEM_OK;
  SphLaunch p = sph(centers_dev, radius_dev, num, mat);
  if (layout == 24)
    return form == IBEM_SOLVE_MIXED_IR ? launch_field24_df(p, points_dev, nump, E_dev, stress_dev, st)
                                       : launch_field24(p, points_dev, nump, E_dev, stress_dev, st);
  if (layout == 60) return launch_field60(p, points_dev, nump, E_dev, stress_dev, st);
  return launch_field78(p, points_dev, nump, E_dev, stress_dev, st);
}

ibem_status ibem_e3d_field_grid(ibem_solver_form form, const double* lo, const double* hi, const int* n,
                                const double* centers_dev, const double* radius_dev, int num,
                                const ibem_material* mat, int layout, const double* E_dev,
                                const double* nodes_dev, int NN, const int* conn_dev, int NE,
                                const double* U_dev, const double* T_dev, const double* sig_inf,
                                double* stress_dev, void* stream) {
  if (!lo || !hi || !n || n[0] < 0 || n[1] < 0 || n[2] < 0) return fail(IBEM_ERR_ARG, "field_grid: bad grid");
  const int64_t nump = (int64_t)n[0] * n[1] * n[2];
  if (nump > INT32_MAX) return fail(IBEM_ERR_ARG, "field_grid: more than 2^31 - 1 points");
  if (nump == 0) return IBEM_OK;
  cudaStream_t st = as_stream(stream);
  double* pts = nullptr;
  IBEM_CUDA(cudaMallocAsync((void**)&pts, sizeof(double) * 3 * nump, st));
  GridSpec g;
  for (int d = 0; d < 3; ++d) g.lo[d] = lo[d], g.span[d] = hi[d] - lo[d], g.n[d] = n[d];
  ::ibem::count_launch(), k_grid_points<<<(unsigned)((nump + 255) / 256), 256, 0, st>>>(nump, g, pts);
  ibem_status s = IBEM_OK;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) s = cuda_fail(e, "field_grid");
  if (!s)
    s = ibem_e3d_field_form(form, pts, (int)nump, centers_dev, radius_dev, num, mat, layout, E_dev, nodes_dev, NN,
                            conn_dev, NE, U_dev, T_dev, sig_inf, stress_dev, stream);
  cudaFreeAsync(pts, st);
  return s;
}

ibem_status ibem_e3d_field(const double* points_dev, int nump, const double* centers_dev,
                           const double* radius_dev, int num, const ibem_material* mat,
                           int layout, const double* E_dev, const double* nodes_dev, int NN,
                           const int* conn_dev, int NE, const double* U_dev,
                           const double* T_dev, const double* sig_inf, double* stress_dev,
                           void* stream) {
  return ibem_e3d_field_form(IBEM_SOLVE_FP64, points_dev, nump, centers_dev, radius_dev, num, mat, layout, E_dev,
                             nodes_dev, NN, conn_dev, NE, U_dev, T_dev, sig_inf, stress_dev, stream);
}

}  // extern "C"
