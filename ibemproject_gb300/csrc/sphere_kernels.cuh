// Sphere interaction kernels, instantiated once per unknown layout by sphere24.cu,
// sphere60.cu and sphere78.cu (each defines IBEM_NU and includes its generated header).
//
// pair blocks (integratorElastic3D.cpp:341-682): one thread per (s, h) particle pair,
//   threads of a warp take 32 consecutive s for one h, so the geometry of h is a
//   broadcast load and every thread writes its own column-major block.  One kernel per
//   column group of the generated code keeps the straight-line code (and its register
//   allocation) per launch small; the self term of s == h is added by a second pass.
// node blocks (integratorElastic3D.cpp:135-340): one thread per (node, particle).
// field sums (postProcessorElastic3D.cpp:367-522): one thread per sample point; the
//   block stages particle geometry and eigenstrain coefficients in shared memory in
//   chunks and every thread sweeps all particles of the chunk.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gen_sphere_common.cuh"
#include "ibem_internal.h"

namespace ibem {

struct StoreSink {
  double* A;
  int64_t lda;
  __device__ __forceinline__ void operator()(int r, int c, double v) const { A[c * lda + r] = v; }
};
struct AddSink {
  double* A;
  int64_t lda;
  __device__ __forceinline__ void operator()(int r, int c, double v) const { A[c * lda + r] += v; }
};

constexpr int kPairThreads = 128;
constexpr int kFieldThreads = 128;
constexpr int kFieldChunk = 64;

}  // namespace ibem

// One pair-block kernel for the generated sub-block function FN.
#define IBEM_PAIR_KERNEL(KNAME, FN, NU)                                                        \
  __global__ void __launch_bounds__(ibem::kPairThreads)                                        \
      KNAME(const double* __restrict__ cen, const double* __restrict__ rad, int num, SphMat mc, \
            double* __restrict__ A, int64_t lda) {                                            \
    const int s = blockIdx.x * blockDim.x + threadIdx.x;                                       \
    const int h = blockIdx.y;                                                                  \
    if (s >= num) return;                                                                      \
    const double x0 = cen[3 * s] - cen[3 * h];                                                 \
    const double x1 = cen[3 * s + 1] - cen[3 * h + 1];                                         \
    const double x2 = cen[3 * s + 2] - cen[3 * h + 2];                                         \
    ibem::StoreSink sink{A + (int64_t)(NU) * h * lda + (int64_t)(NU) * s, lda};              \
    FN(x0, x1, x2, rad[h], mc, sink);                                                          \
  }

#define IBEM_SELF_KERNEL(KNAME, FN, NU)                                              \
  __global__ void KNAME(int num, SphMat mc, double* __restrict__ A, int64_t lda) {   \
    const int s = blockIdx.x * blockDim.x + threadIdx.x;                             \
    if (s >= num) return;                                                            \
    ibem::AddSink sink{A + (int64_t)(NU) * s * lda + (int64_t)(NU) * s, lda};        \
    FN(mc, sink);                                                                    \
  }

#define IBEM_NODE_KERNEL(KNAME, FN, NU)                                                       \
  __global__ void __launch_bounds__(ibem::kPairThreads)                                       \
      KNAME(const double* __restrict__ nodes, int NN, const double* __restrict__ cen,         \
            const double* __restrict__ rad, SphMat mc, double* __restrict__ H, int64_t ldh) { \
    const int j = blockIdx.x * blockDim.x + threadIdx.x;                                      \
    const int K = blockIdx.y;                                                                 \
    if (j >= NN) return;                                                                      \
    const double x0 = nodes[3 * j] - cen[3 * K];                                              \
    const double x1 = nodes[3 * j + 1] - cen[3 * K + 1];                                      \
    const double x2 = nodes[3 * j + 2] - cen[3 * K + 2];                                      \
    ibem::StoreSink sink{H + (int64_t)(NU) * K * ldh + 3 * (int64_t)j, ldh};                 \
    FN(x0, x1, x2, rad[K], mc, sink);                                                         \
  }

// Local eigenstrain polynomial at x (relative to the centre) of unknown row r (i<=j):
// E_r + sum_p E_rp x_p + sum_{p<=q} map[p][q] E_rpq x_p x_q  (postprocessor :409-433).
template <int NU>
__device__ __forceinline__ double local_eigenstrain(const double* __restrict__ E, int r, double x0,
                                                    double x1, double x2) {
  const double x[3] = {x0, x1, x2};
  double v = E[r];
#pragma unroll
  for (int p = 0; p < 3; ++p) v += E[6 + 3 * r + p] * x[p];
  if (NU == 78) {
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = p; q < 3; ++q) v += (p == q ? 1.0 : 2.0) * E[24 + 9 * r + 3 * p + q] * x[p] * x[q];
  } else if (NU == 60) {
    int t = 0;
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = p; q < 3; ++q, ++t) v += (p == q ? 1.0 : 2.0) * E[24 + 6 * r + t] * x[p] * x[q];
  }
  return v;
}

#define IBEM_FIELD_KERNEL(KNAME, FN, NU)                                                         \
  __global__ void __launch_bounds__(ibem::kFieldThreads)                                         \
      KNAME(const double* __restrict__ pts, int nump, const double* __restrict__ cen,            \
            const double* __restrict__ rad, int num, SphMat mc, const double* __restrict__ E,    \
            double* __restrict__ stress) {                                                       \
    __shared__ double sc[ibem::kFieldChunk * 3];                                                 \
    __shared__ double sr[ibem::kFieldChunk];                                                     \
    __shared__ double sE[ibem::kFieldChunk * (NU)];                                              \
    const int s = blockIdx.x * blockDim.x + threadIdx.x;                                         \
    const bool act = s < nump;                                                                   \
    double p0 = 0, p1 = 0, p2 = 0;                                                               \
    if (act) { p0 = pts[3 * s]; p1 = pts[3 * s + 1]; p2 = pts[3 * s + 2]; }                      \
    double e[6] = {0, 0, 0, 0, 0, 0};                                                            \
    int inside = -1;                                                                             \
    for (int h0 = 0; h0 < num; h0 += ibem::kFieldChunk) {                                        \
      const int nh = min(ibem::kFieldChunk, num - h0);                                           \
      __syncthreads();                                                                           \
      for (int i = threadIdx.x; i < nh * 3; i += blockDim.x) sc[i] = cen[3 * (int64_t)h0 + i];   \
      for (int i = threadIdx.x; i < nh; i += blockDim.x) sr[i] = rad[h0 + i];                    \
      for (int i = threadIdx.x; i < nh * (NU); i += blockDim.x)                                  \
        sE[i] = E[(int64_t)(NU) * h0 + i];                                                       \
      __syncthreads();                                                                           \
      if (act) {                                                                                 \
        for (int hh = 0; hh < nh; ++hh) {                                                        \
          const double x0 = p0 - sc[3 * hh], x1 = p1 - sc[3 * hh + 1], x2 = p2 - sc[3 * hh + 2]; \
          const double a = sr[hh];                                                               \
          if (x0 * x0 + x1 * x1 + x2 * x2 - a * a <= 0) inside = h0 + hh;                        \
          FN(x0, x1, x2, a, mc, sE + (NU) * hh, e);                                              \
        }                                                                                        \
      }                                                                                          \
    }                                                                                            \
    if (!act) return;                                                                            \
    if (inside >= 0) {                                                                           \
      const double* Ei = E + (int64_t)(NU) * inside;                                             \
      const double x0 = p0 - cen[3 * inside], x1 = p1 - cen[3 * inside + 1],                     \
                   x2 = p2 - cen[3 * inside + 2];                                                \
      for (int r = 0; r < 6; ++r) e[r] -= local_eigenstrain<NU>(Ei, r, x0, x1, x2);              \
    }                                                                                            \
    /* s = C0 : e with e stored once per symmetric pair (map = 2 off the diagonal) */            \
    const double tr = e[0] + e[3] + e[5];                                                        \
    double* o = stress + 6 * (int64_t)s;                                                         \
    o[0] += mc.lam0 * tr + 2.0 * mc.mu0 * e[0];                                                  \
    o[1] += 2.0 * mc.mu0 * e[1];                                                                 \
    o[2] += 2.0 * mc.mu0 * e[2];                                                                 \
    o[3] += mc.lam0 * tr + 2.0 * mc.mu0 * e[3];                                                  \
    o[4] += 2.0 * mc.mu0 * e[4];                                                                 \
    o[5] += mc.lam0 * tr + 2.0 * mc.mu0 * e[5];                                                  \
  }
