// Internal declarations shared by the translation units of libibem_gb300.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/ibem_gb300.h"

namespace ibem {

// Record a failure message for ibem_last_error() and return `st`.
ibem_status fail(ibem_status st, const std::string& msg);
ibem_status cuda_fail(cudaError_t e, const char* where);

#define IBEM_CUDA(call)                                        \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return ::ibem::cuda_fail(e_, #call); \
  } while (0)

#define IBEM_LAUNCH_CHECK(where)                                \
  do {                                                          \
    cudaError_t e_ = cudaGetLastError();                        \
    if (e_ != cudaSuccess) return ::ibem::cuda_fail(e_, where); \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Counts kernel launches of this library (read through ibem_kernel_launches); every
// launch site is written `::ibem::count_launch(), kernel<<<...>>>(...)`.
int count_launch();
// Adds n launches to the count (kernels that ran as nodes of a replayed CUDA graph; n < 0
// takes back launches counted while a graph was captured, when nothing ran).
void add_launches(long long n);
long long launches_so_far();

// ---- sphere kernels (sphere24.cu / sphere60.cu / sphere78.cu) ----
struct SphLaunch {
  const double* cen;
  const double* rad;
  int num;
  double E0, nu0, E1, nu1;
};
ibem_status launch_pair24(const SphLaunch& p, double* A, int64_t lda, int64_t row0, int64_t col0, cudaStream_t st);
ibem_status launch_pair60(const SphLaunch& p, double* A, int64_t lda, int64_t row0, int64_t col0, cudaStream_t st);
ibem_status launch_pair78(const SphLaunch& p, double* A, int64_t lda, int64_t row0, int64_t col0, cudaStream_t st);
ibem_status launch_node24(const SphLaunch& p, const double* nodes, int NN, double* H, int64_t ldh, int64_t row0, int64_t col0, cudaStream_t st);
ibem_status launch_node60(const SphLaunch& p, const double* nodes, int NN, double* H, int64_t ldh, int64_t row0, int64_t col0, cudaStream_t st);
ibem_status launch_node78(const SphLaunch& p, const double* nodes, int NN, double* H, int64_t ldh, int64_t row0, int64_t col0, cudaStream_t st);
// particle part of the stress at points; sbase (nump x 6) holds the boundary or
// remote stress on entry and the total stress on exit
ibem_status launch_field24(const SphLaunch& p, const double* pts, int nump, const double* E, double* stress, cudaStream_t st);
ibem_status launch_field24_df(const SphLaunch& p, const double* pts, int nump, const double* E, double* stress,
                              cudaStream_t st);
ibem_status launch_field60(const SphLaunch& p, const double* pts, int nump, const double* E, double* stress, cudaStream_t st);
ibem_status launch_field78(const SphLaunch& p, const double* pts, int nump, const double* E, double* stress, cudaStream_t st);

// ---- boundary kernels (bem.cu) ----
ibem_status bem_hg(const double* nodes, int NN, const int* conn, int NE, const ibem_material& m,
                   double* H, int64_t ldh, int64_t hrow0, int64_t hcol0, double* G, int64_t ldg,
                   int64_t grow0, int64_t gcol0, cudaStream_t st);
ibem_status bem_to_incl(const double* nodes, int NN, const int* conn, int NE, const double* cen,
                        int num, const ibem_material& m, int layout, double* H, int64_t ldh,
                        int64_t hcol0, double* G, int64_t ldg, int64_t gcol0, int64_t row0,
                        cudaStream_t st);
ibem_status bem_post(const double* pts, int nump, const double* nodes, int NN, const int* conn,
                     int NE, const ibem_material& m, const double* U, const double* T,
                     double* stress, cudaStream_t st, bool mixed = false);

}  // namespace ibem
