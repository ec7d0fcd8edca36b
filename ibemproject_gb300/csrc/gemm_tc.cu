// Tensor-core GEMM of the mixed-precision factorisation (filled in by the tcgen05 kernel).
#include "solver.h"

namespace ibem {

ibem_status gemm_sub_f32_tc(int64_t m, int64_t n, int64_t k, const float* A, int64_t lda, const float* B,
                            int64_t ldb, float* C, int64_t ldc, cudaStream_t st) {
  (void)m; (void)n; (void)k; (void)A; (void)lda; (void)B; (void)ldb; (void)C; (void)ldc; (void)st;
  return fail(IBEM_ERR_ARG, "tensor-core GEMM not built");
}

}  // namespace ibem
