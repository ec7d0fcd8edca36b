// Internal interface of the dense solver (solver.cu) and its tensor-core GEMM (gemm_tc.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ibem_internal.h"

namespace ibem {

// C (m x n, ldc) -= A (m x k, lda) B (k x n, ldb), FP32 storage, column-major, computed on
// the tensor cores with each operand split into two BF16 terms (hi + lo) and the three
// products hi*hi + hi*lo + lo*hi accumulated in FP32.
// `ws` is scratch of at least gemm_tc_workspace_bytes(max m, max n) bytes (the BF16 splits);
// `err` a device int raised if a bounded device-side wait gave up.
ibem_status gemm_sub_f32_tc(int64_t m, int64_t n, int64_t k, const float* A, int64_t lda, const float* B,
                            int64_t ldb, float* C, int64_t ldc, void* ws, size_t ws_bytes, int* err,
                            cudaStream_t st);
size_t gemm_tc_workspace_bytes(int64_t max_m, int64_t max_n);

// block: diagonal block size of the IBEM_SOLVE_GMRES_BJ form (1..80; unknowns per particle);
// ws32: optional FP32 workspace of that form, ((N + 3) / 4 * 4) x N floats (allocated and
// freed inside when null).
ibem_status solve_dense(ibem_solver_form form, int64_t N, double* A, int64_t lda, const double* b, double* x,
                        double tol, ibem_solve_report* rep, cudaStream_t st, int block = 0,
                        float* ws32 = nullptr);

// Allocation-free FP64 solve for N <= 1024 (workspace in a static device array).
ibem_status solve_fp64_noalloc(int64_t N, const double* A, int64_t lda, const double* b, double* x,
                               ibem_solve_report* rep, cudaStream_t st);

// Self-tests of the bounded device-side waits (a wait on a flag / an mbarrier that nothing
// completes, given up after `limit` polls): IBEM_ERR_TIMEOUT when the wait gave up.
ibem_status selftest_flag_wait(long long limit, cudaStream_t st);
ibem_status selftest_mbar_wait(long long limit, cudaStream_t st);

}  // namespace ibem
