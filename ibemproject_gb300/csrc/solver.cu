// Dense solve of the iBEM system (replaces systemSolverElastic3D::_solve,
// systemSolverElastic3D.h:44-60, X = A.fullPivLu().solve(b)).
//
// Both forms first equilibrate A (row, then column max scaling): the raw iBEM matrix
// spans ~47 decades, which partial pivoting alone cannot handle (full pivoting can).
//
//   IBEM_SOLVE_FP64      LU with partial pivoting of the scaled matrix in FP64.
//   IBEM_SOLVE_MIXED_IR  LU with partial pivoting in FP32 (trailing updates on the tensor
//                        cores with the split-BF16 "x3" scheme, FP32 accumulation), then
//                        FP64 GMRES iterative refinement preconditioned by the FP32 factors;
//                        FP64 is used for the residual b - A x and the GMRES arithmetic.
//
// LU structure: recursive on column halves (Toledo), so most flops sit in a few large
// GEMMs.  Leaves are panels of <= 32 columns factorised by one cooperative kernel that
// keeps the panel rows in shared memory across all SMs and needs one grid barrier per
// column: every CTA publishes its best pivot candidate row (and the current diagonal row
// if it owns it), then all CTAs pick the same pivot and swap/scale/update locally.
// The grid barrier is a bounded spin: after kSpinLimit polls it raises an error flag and
// every CTA returns, so a fault can end the kernel but never hang it.
#include <cooperative_groups.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "ibem_internal.h"
#include "prof.h"
#include "solver.h"

namespace ibem {
namespace {

constexpr int kPanelThreads = 256;
constexpr int kLeaf = 32;                   // panel width of the recursion leaves
constexpr long long kSpinLimit = 1LL << 22; // polls before a barrier gives up

// ---------------------------------------------------------------- utilities
template <typename T>
__global__ void k_fill(T* p, int64_t n, T v) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

// row max |a_ij| (threads over rows: coalesced along columns)
__global__ void k_rowmax(int64_t n, const double* __restrict__ A, int64_t lda, double* __restrict__ r) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double m = 0;
  for (int64_t j = 0; j < n; ++j) m = fmax(m, fabs(A[j * lda + i]));
  r[i] = m > 0 ? 1.0 / m : 1.0;
}

// column max |r_i a_ij| -> c_j (one block per column)
__global__ void k_colmax(int64_t n, const double* __restrict__ A, int64_t lda, const double* __restrict__ r,
                         double* __restrict__ c) {
  __shared__ double sm[256];
  const int64_t j = blockIdx.x;
  double m = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(r[i] * A[j * lda + i]));
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) c[j] = sm[0] > 0 ? 1.0 / sm[0] : 1.0;
}

// W = R A C in precision T (column-major, ldw)
template <typename T>
__global__ void k_scale_copy(int64_t n, const double* __restrict__ A, int64_t lda, const double* __restrict__ r,
                             const double* __restrict__ c, T* __restrict__ W, int64_t ldw) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t j = blockIdx.y;
  if (i >= n) return;
  W[j * ldw + i] = (T)(r[i] * A[j * lda + i] * c[j]);
}

// ---------------------------------------------------------------- panel error flag
// Sticky error flag shared by the CTAs of the panel kernel: set when a spin gives up.
struct GridSync {
  int err;
};

// ---------------------------------------------------------------- panel kernel
// Factorises the m x nb panel (nb <= kLeaf) at P with partial pivoting.  Rows are split
// evenly over the CTAs and live in dynamic shared memory.  Per column j, every CTA writes
// one record in rec[j & 1][cta] = {|best|, its global row, that row's values and, in the
// CTA that owns row j, row j's values} and adds 1 to the arrival counter cnt[j & 1]; one
// thread per CTA waits (bounded) until the counter reaches base[j & 1] + (j / 2 + 1) * ncta,
// the value after every CTA of this launch has arrived for column j.  The counters only
// grow; the host passes the bases they had at launch.  Every CTA then reads all records
// (L2 loads), picks the same pivot (largest |a|, ties to the smallest row), swaps and
// updates its own rows.  Double buffering by column parity is enough: a CTA overwrites a
// record two columns later only after every CTA has arrived for the next column, which
// each does only after reading the current records.
// ipiv[j] receives the absolute pivot row of column j; info the first zero pivot.
constexpr int kRec = 2 * kLeaf + 4;  // record length in elements of T

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add_u32(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename T>
__global__ void __launch_bounds__(kPanelThreads) k_panel(T* __restrict__ P, int64_t lda, int m, int nb,
                                                         int rows_per, T* rec, unsigned* cnt, unsigned base0,
                                                         unsigned base1, int* __restrict__ ipiv, int kglob,
                                                         int* __restrict__ info, GridSync* gs) {
  extern __shared__ unsigned char smem_raw[];
  T* sp = reinterpret_cast<T*>(smem_raw);  // rows_per x kLeaf, row-major
  __shared__ T s_pr[kLeaf];                 // pivot row
  __shared__ T s_jr[kLeaf];                 // row j
  __shared__ T s_bv[kPanelThreads / 32];
  __shared__ int s_bi[kPanelThreads / 32];
  __shared__ int s_src[kPanelThreads / 32];
  __shared__ int s_piv, s_sel, s_fail;
  const int cta = blockIdx.x, ncta = gridDim.x;
  const int r0 = cta * rows_per;
  const int nr = max(0, min(rows_per, m - r0));
  for (int idx = threadIdx.x; idx < nr * nb; idx += blockDim.x) {
    const int rr = idx % nr, cc = idx / nr;
    sp[rr * kLeaf + cc] = P[(int64_t)cc * lda + r0 + rr];
  }
  if (threadIdx.x == 0) s_fail = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = 0; j < nb; ++j) {
    const int buf = j & 1;
    // (a) local candidate: max |a_ij| over rows >= j owned here (first max wins)
    T best = -1;
    int bi = -1;
    for (int rr = threadIdx.x; rr < nr; rr += blockDim.x) {
      const int gr = r0 + rr;
      if (gr < j) continue;
      const T v = fabs(sp[rr * kLeaf + j]);
      if (v > best) { best = v; bi = gr; }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const T ov = __shfl_down_sync(0xffffffffu, best, off);
      const int oi = __shfl_down_sync(0xffffffffu, bi, off);
      if (ov > best || (ov == best && oi >= 0 && (bi < 0 || oi < bi))) { best = ov; bi = oi; }
    }
    if (lane == 0) { s_bv[warp] = best; s_bi[warp] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
      T b = -1;
      int i = -1;
      for (int w = 0; w < kPanelThreads / 32; ++w)
        if (s_bv[w] > b || (s_bv[w] == b && s_bi[w] >= 0 && (i < 0 || s_bi[w] < i))) { b = s_bv[w]; i = s_bi[w]; }
      s_piv = i;
      T* rc = rec + ((int64_t)buf * ncta + cta) * kRec;
      rc[0] = b;
      rc[1] = (T)i;
    }
    __syncthreads();
    {
      T* rc = rec + ((int64_t)buf * ncta + cta) * kRec;
      const int i = s_piv;
      if (threadIdx.x < nb) {
        rc[4 + threadIdx.x] = (i >= 0) ? sp[(i - r0) * kLeaf + threadIdx.x] : (T)0;
        if (j >= r0 && j < r0 + nr) rc[4 + kLeaf + threadIdx.x] = sp[(j - r0) * kLeaf + threadIdx.x];
      }
      __threadfence();
    }
    __syncthreads();
    // (b) arrive, wait for every CTA, then read all records and pick the pivot in parallel
    if (threadIdx.x == 0) {
      red_release_add_u32(cnt + buf, 1u);
      const unsigned target = (buf ? base1 : base0) + (unsigned)(j / 2 + 1) * (unsigned)ncta;
      long long it = 0;
      while ((int)(ld_acquire_u32(cnt + buf) - target) < 0) {
        if (++it > kSpinLimit || *reinterpret_cast<volatile int*>(&gs->err) != 0) {
          atomicExch(&gs->err, 1);
          s_fail = 1;
          break;
        }
      }
    }
    __syncthreads();
    if (s_fail) return;  // uniform: read after the barrier by every thread
    T v = -1;
    int ci = -1, src = -1;
    if (threadIdx.x < ncta) {
      const T* rc = rec + ((int64_t)buf * ncta + threadIdx.x) * kRec;
      ci = (int)__ldcg(rc + 1);
      v = ci >= 0 ? __ldcg(rc) : (T)-1;
      src = threadIdx.x;
    }
    for (int off = 16; off > 0; off >>= 1) {
      const T ov = __shfl_down_sync(0xffffffffu, v, off);
      const int oi = __shfl_down_sync(0xffffffffu, ci, off);
      const int os = __shfl_down_sync(0xffffffffu, src, off);
      if (oi >= 0 && (ci < 0 || ov > v || (ov == v && oi < ci))) { v = ov; ci = oi; src = os; }
    }
    if (lane == 0) { s_bv[warp] = v; s_bi[warp] = ci; s_src[warp] = src; }
    __syncthreads();
    if (threadIdx.x == 0) {
      T b = -1;
      int i = -1, sr = -1;
      for (int w = 0; w < kPanelThreads / 32; ++w)
        if (s_bi[w] >= 0 && (i < 0 || s_bv[w] > b || (s_bv[w] == b && s_bi[w] < i))) {
          b = s_bv[w];
          i = s_bi[w];
          sr = s_src[w];
        }
      s_piv = i;
      s_sel = sr;
      if (cta == 0) {
        ipiv[j] = kglob + i;
        if (b == 0 && *info == 0) *info = kglob + j + 1;
      }
    }
    __syncthreads();
    const int piv = s_piv;
    if (threadIdx.x < nb) {
      // pivot row from the winning record, row j from its owner's record
      const int owner = j / rows_per;
      s_pr[threadIdx.x] = __ldcg(rec + ((int64_t)buf * ncta + s_sel) * kRec + 4 + threadIdx.x);
      s_jr[threadIdx.x] = __ldcg(rec + ((int64_t)buf * ncta + owner) * kRec + 4 + kLeaf + threadIdx.x);
    }
    __syncthreads();
    // (c) swap rows j and piv where they live
    if (piv != j) {
      if (piv >= r0 && piv < r0 + nr && threadIdx.x < nb) sp[(piv - r0) * kLeaf + threadIdx.x] = s_jr[threadIdx.x];
      if (j >= r0 && j < r0 + nr && threadIdx.x < nb) sp[(j - r0) * kLeaf + threadIdx.x] = s_pr[threadIdx.x];
    }
    __syncthreads();
    // (d) scale and rank-1 update of rows below j
    const T pjj = s_pr[j];
    if (pjj != (T)0) {
      for (int rr = threadIdx.x; rr < nr; rr += blockDim.x) {
        if (r0 + rr <= j) continue;
        T* row = sp + rr * kLeaf;
        const T l = row[j] / pjj;
        row[j] = l;
        for (int k = j + 1; k < nb; ++k) row[k] -= l * s_pr[k];
      }
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < nr * nb; idx += blockDim.x) {
    const int rr = idx % nr, cc = idx / nr;
    P[(int64_t)cc * lda + r0 + rr] = sp[rr * kLeaf + cc];
  }
}

// apply the panel's row exchanges (rows k0+j <-> ipiv[j], j ascending) to every column
// outside the panel [k0, k0+nb): thread t takes column t (t < k0) or t + nb
template <typename T>
__global__ void k_laswp(T* __restrict__ A, int64_t lda, int64_t k0, const int* __restrict__ ipiv, int nb,
                        int64_t ncols) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= ncols) return;
  const int64_t c = t < k0 ? t : t + nb;
  T* col = A + c * lda;
  for (int j = 0; j < nb; ++j) {
    const int64_t p = ipiv[j];
    const int64_t q = k0 + j;
    if (p != q) { const T tv = col[q]; col[q] = col[p]; col[p] = tv; }
  }
}

// small triangular solve: B (n1 x n2) <- L^-1 B, L unit lower n1 x n1 (n1 <= 64);
// one CTA per 64 columns of B, L and the B columns staged in shared memory, one thread
// per column
template <typename T>
__global__ void __launch_bounds__(64) k_trsm_small(const T* __restrict__ L, int64_t ldl, int n1, T* __restrict__ B,
                                                   int64_t ldb, int64_t n2) {
  extern __shared__ unsigned char trsm_smem[];
  T* sL = reinterpret_cast<T*>(trsm_smem);  // [k][i] = L(i, k), 64 x 65
  T* sB = sL + 64 * 65;                      // [i][c] = B(i, c0 + c), 64 x 65
  const int64_t c0 = blockIdx.x * (int64_t)64;
  for (int idx = threadIdx.x; idx < n1 * n1; idx += blockDim.x) {
    const int i = idx % n1, k = idx / n1;
    sL[k * 65 + i] = L[(int64_t)k * ldl + i];
  }
  for (int idx = threadIdx.x; idx < n1 * 64; idx += blockDim.x) {
    const int i = idx % n1, c = idx / n1;
    sB[i * 65 + c] = (c0 + c < n2) ? B[(c0 + c) * ldb + i] : (T)0;
  }
  __syncthreads();
  const int c = threadIdx.x;
  for (int i = 0; i < n1; ++i) {
    const T xi = sB[i * 65 + c];
    for (int k = i + 1; k < n1; ++k) sB[k * 65 + c] -= sL[i * 65 + k] * xi;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < n1 * 64; idx += blockDim.x) {
    const int i = idx % n1, cc = idx / n1;
    if (c0 + cc < n2) B[(c0 + cc) * ldb + i] = sB[i * 65 + cc];
  }
}

// Same solve with the triangle size fixed at compile time: the column lives in registers,
// the loops are fully unrolled (no dependent shared-memory round trips).
template <typename T, int NB>
__global__ void __launch_bounds__(128) k_trsm_small_fixed(const T* __restrict__ L, int64_t ldl, T* __restrict__ B,
                                                          int64_t ldb, int64_t n2) {
  __shared__ T sL[NB * NB];  // [i][k] = L(k, i) for k > i
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int k = idx % NB, i = idx / NB;
    sL[i * NB + k] = L[(int64_t)i * ldl + k];
  }
  __syncthreads();
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= n2) return;
  T* b = B + c * ldb;
  T x[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) x[i] = b[i];
#pragma unroll
  for (int i = 0; i < NB; ++i)
#pragma unroll
    for (int k = i + 1; k < NB; ++k) x[k] -= sL[i * NB + k] * x[i];
#pragma unroll
  for (int i = 0; i < NB; ++i) b[i] = x[i];
}

// ---------------------------------------------------------------- SIMT GEMM  C -= A B
// 64x64 tile, 256 threads, 4x4 outputs per thread, k-step 16.
template <typename T>
__global__ void __launch_bounds__(256) k_gemm_sub(int64_t m, int64_t n, int64_t k, const T* __restrict__ A,
                                                  int64_t lda, const T* __restrict__ B, int64_t ldb,
                                                  T* __restrict__ C, int64_t ldc) {
  __shared__ T sA[16][64 + 1];
  __shared__ T sB[16][64 + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int64_t i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0;
  for (int64_t kk = 0; kk < k; kk += 16) {
    for (int idx = threadIdx.x; idx < 16 * 64; idx += 256) {
      const int r = idx % 64, c = idx / 64;
      const int64_t gi = i0 + r, gk = kk + c;
      sA[c][r] = (gi < m && gk < k) ? A[gk * lda + gi] : (T)0;
      const int rk = idx % 16, cj = idx / 16;
      const int64_t gk2 = kk + rk, gj = j0 + cj;
      sB[rk][cj] = (gk2 < k && gj < n) ? B[gj * ldb + gk2] : (T)0;
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      T av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) av[a] = sA[t][tx + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) bv[b] = sB[t][ty + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] += av[a] * bv[b];
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int64_t gi = i0 + tx + 16 * a, gj = j0 + ty + 16 * b;
      if (gi < m && gj < n) C[gj * ldc + gi] -= acc[a][b];
    }
}

// ---------------------------------------------------------------- vectors
// y[i] = b[i] - sum_j A[i,j] x[j] over a column chunk; partial sums summed by k_sum_parts
__global__ void k_gemv_part(int64_t n, const double* __restrict__ A, int64_t lda, const double* __restrict__ x,
                            int64_t chunk, double* __restrict__ part) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
  if (i >= n) return;
  double s0 = 0, s1 = 0;
  int64_t j = j0;
  for (; j + 1 < j1; j += 2) {
    s0 += A[j * lda + i] * x[j];
    s1 += A[(j + 1) * lda + i] * x[j + 1];
  }
  if (j < j1) s0 += A[j * lda + i] * x[j];
  part[blockIdx.y * n + i] = s0 + s1;
}
__global__ void k_residual(int64_t n, int nparts, const double* __restrict__ part, const double* __restrict__ b,
                           double* __restrict__ r) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
  for (int p = 0; p < nparts; ++p) s += part[p * n + i];
  r[i] = b[i] - s;
}

// Blocked substitution with the factors in precision T (vectors FP64), one launch per
// kTrsvB-row block.  Every CTA loads the diagonal block and the block's right-hand side,
// solves the small triangle in shared memory (the same arithmetic in every CTA), CTA 0
// stores the solved block to `out`, and each CTA applies the block column to its share of
// the remaining rows of `y`.  `y` rows of the block are only read and other rows only
// written within a launch, so CTAs never race.
constexpr int kTrsvB = 128;
template <typename T, bool LOWER>
__global__ void __launch_bounds__(256) k_trsv_block(const T* __restrict__ F, int64_t ldf, int64_t N, int64_t k0,
                                                    int nb, double* __restrict__ y, double* __restrict__ out) {
  extern __shared__ unsigned char trsv_smem[];
  T* sF = reinterpret_cast<T*>(trsv_smem);  // [c][r] = F(k0 + r, k0 + c), kTrsvB x (kTrsvB + 1)
  // arithmetic in T: FP32 factors give an FP32 solve (the preconditioner of the mixed form)
  T* sy = reinterpret_cast<T*>(trsv_smem + sizeof(T) * kTrsvB * (kTrsvB + 1) + 16);
  for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
    const int r = idx % nb, c = idx / nb;
    sF[c * (kTrsvB + 1) + r] = F[(k0 + c) * ldf + k0 + r];
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    // the small triangle in one warp: lane owns rows lane, lane+32, lane+64, lane+96;
    // the solved value of row j is broadcast with a shuffle (no block barriers)
    const int lane = threadIdx.x;
    T v[kTrsvB / 32];
#pragma unroll
    for (int q = 0; q < kTrsvB / 32; ++q) {
      const int r = lane + 32 * q;
      v[q] = r < nb ? (T)y[k0 + r] : (T)0;
    }
    if (LOWER) {
#pragma unroll
      for (int q = 0; q < kTrsvB / 32; ++q)
        for (int jj = 0; jj < 32; ++jj) {
          const int j = 32 * q + jj;
          if (j >= nb) break;
          const T xj = __shfl_sync(0xffffffffu, v[q], jj);
#pragma unroll
          for (int q2 = 0; q2 < kTrsvB / 32; ++q2) {
            const int r = lane + 32 * q2;
            if (r > j && r < nb) v[q2] -= sF[j * (kTrsvB + 1) + r] * xj;
          }
        }
    } else {
#pragma unroll
      for (int q = kTrsvB / 32 - 1; q >= 0; --q)
        for (int jj = 31; jj >= 0; --jj) {
          const int j = 32 * q + jj;
          if (j >= nb) continue;
          if (lane == jj) v[q] /= sF[j * (kTrsvB + 1) + j];
          const T xj = __shfl_sync(0xffffffffu, v[q], jj);
#pragma unroll
          for (int q2 = 0; q2 < kTrsvB / 32; ++q2) {
            const int r = lane + 32 * q2;
            if (r < j) v[q2] -= sF[j * (kTrsvB + 1) + r] * xj;
          }
        }
    }
#pragma unroll
    for (int q = 0; q < kTrsvB / 32; ++q) {
      const int r = lane + 32 * q;
      if (r < nb) sy[r] = v[q];
    }
  }
  __syncthreads();
  if (blockIdx.x == 0)
    for (int r = threadIdx.x; r < nb; r += blockDim.x) out[k0 + r] = (double)sy[r];
  // block column applied to this CTA's rows: 4 independent partial sums keep loads in flight
  const int64_t r0 = LOWER ? k0 + nb : 0, r1 = LOWER ? N : k0;
  const int64_t r = r0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r < r1) {
    T a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    const T* col = F + k0 * ldf + r;
    int c = 0;
    for (; c + 3 < nb; c += 4) {
      a0 += col[(int64_t)c * ldf] * sy[c];
      a1 += col[(int64_t)(c + 1) * ldf] * sy[c + 1];
      a2 += col[(int64_t)(c + 2) * ldf] * sy[c + 2];
      a3 += col[(int64_t)(c + 3) * ldf] * sy[c + 3];
    }
    for (; c < nb; ++c) a0 += col[(int64_t)c * ldf] * sy[c];
    y[r] -= (double)((a0 + a1) + (a2 + a3));
  }
}

template <typename T>
cudaError_t set_solver_smem_attrs() {
  cudaError_t e = cudaFuncSetAttribute((const void*)k_trsm_small<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(2 * 64 * 65 * sizeof(T)));
  const int tb = (int)(sizeof(T) * kTrsvB * (kTrsvB + 1) + 16 + sizeof(double) * kTrsvB);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k_trsv_block<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tb);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k_trsv_block<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tb);
  return e;
}

// out[i] = y[perm[i]]  (P y with P the row permutation of the factorisation)
__global__ void k_gather(int64_t n, const int* __restrict__ perm, const double* __restrict__ y,
                         double* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = y[perm[i]];
}

__global__ void k_vmul(int64_t n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = a[i] * b[i];
}

}  // namespace

// =====================================================================================
template <typename T>
struct LuWork {
  T* cand = nullptr;         // panel records [2][ncta][kRec]
  unsigned* cnt = nullptr;   // panel arrival counters [2] (only grow)
  unsigned arrived[2] = {0, 0};  // host copy of the counters' values after the last launch
  int* ipiv_dev = nullptr;  // N entries (global, absolute row of each exchange)
  int* perm = nullptr;      // N entries: row i of P A is row perm[i] of A
  double* tmp = nullptr;    // N-vector scratch of lu_apply
  int* info = nullptr;
  GridSync* gs = nullptr;
  int ncta = 0;
  int rows_cap = 0;
  void* gemm_ws = nullptr;   // BF16 split workspace of the tensor-core GEMM (FP32 LU only)
  size_t gemm_ws_bytes = 0;
  int* gemm_err = nullptr;   // raised by the tensor-core GEMM's bounded waits
};

template <typename T>
static ibem_status panel(T* A, int64_t lda, int64_t k0, int64_t m, int nb, LuWork<T>& w, cudaStream_t st) {
  // rows per CTA so that every CTA fits its rows in shared memory
  int ncta = w.ncta;
  int rows_per = (int)((m + ncta - 1) / ncta);
  if (rows_per > w.rows_cap) return fail(IBEM_ERR_ARG, "panel too tall for shared memory");
  if (rows_per < 1) rows_per = 1;
  ncta = (int)((m + rows_per - 1) / rows_per);
  size_t smem = (size_t)rows_per * kLeaf * sizeof(T);
  T* P = A + k0 * lda + k0;
  int mm = (int)m;
  int* ip = w.ipiv_dev + k0;
  int kg = (int)k0;
  unsigned b0 = w.arrived[0], b1 = w.arrived[1];
  void* args[] = {&P, &lda, &mm, &nb, &rows_per, &w.cand, &w.cnt, &b0, &b1, &ip, &kg, &w.info, &w.gs};
  ProfScope ps(PROF_PANEL, st);
  count_launch();
  IBEM_CUDA(cudaLaunchCooperativeKernel((void*)k_panel<T>, dim3(ncta), dim3(kPanelThreads), args, smem, st));
  w.arrived[0] += (unsigned)ncta * (unsigned)((nb + 1) / 2);
  w.arrived[1] += (unsigned)ncta * (unsigned)(nb / 2);
  return IBEM_OK;
}

template <typename T>
static ibem_status gemm_sub(int64_t m, int64_t n, int64_t k, const T* A, int64_t lda, const T* B, int64_t ldb,
                            T* C, int64_t ldc, LuWork<T>& w, cudaStream_t st);

template <>
ibem_status gemm_sub<double>(int64_t m, int64_t n, int64_t k, const double* A, int64_t lda, const double* B,
                             int64_t ldb, double* C, int64_t ldc, LuWork<double>& w, cudaStream_t st) {
  (void)w;
  if (m <= 0 || n <= 0 || k <= 0) return IBEM_OK;
  ProfScope ps(PROF_GEMM_SIMT, st, 2.0 * m * n * k);
  dim3 grid((unsigned)((m + 63) / 64), (unsigned)((n + 63) / 64));
  ::ibem::count_launch(), k_gemm_sub<double><<<grid, 256, 0, st>>>(m, n, k, A, lda, B, ldb, C, ldc);
  IBEM_LAUNCH_CHECK("gemm f64");
  return IBEM_OK;
}

template <>
ibem_status gemm_sub<float>(int64_t m, int64_t n, int64_t k, const float* A, int64_t lda, const float* B,
                            int64_t ldb, float* C, int64_t ldc, LuWork<float>& w, cudaStream_t st) {
  if (m <= 0 || n <= 0 || k <= 0) return IBEM_OK;
  // tensor cores for every update large enough to fill 128 x 256 tiles; small ones on CUDA cores
  if (w.gemm_ws && m >= 128 && n >= 128 && k >= 32)
    return gemm_sub_f32_tc(m, n, k, A, lda, B, ldb, C, ldc, w.gemm_ws, w.gemm_ws_bytes, w.gemm_err, st);
  ProfScope ps(PROF_GEMM_SIMT, st, 2.0 * m * n * k);
  dim3 grid((unsigned)((m + 63) / 64), (unsigned)((n + 63) / 64));
  ::ibem::count_launch(), k_gemm_sub<float><<<grid, 256, 0, st>>>(m, n, k, A, lda, B, ldb, C, ldc);
  IBEM_LAUNCH_CHECK("gemm f32");
  return IBEM_OK;
}

// B (n1 x n2) <- L^-1 B with L the unit-lower n1 x n1 block at L (recursive)
template <typename T>
static ibem_status trsm(const T* L, int64_t ldl, int64_t n1, T* B, int64_t ldb, int64_t n2, LuWork<T>& w,
                        cudaStream_t st) {
  if (n1 <= 0 || n2 <= 0) return IBEM_OK;
  if (n1 <= 64) {
    ProfScope ps(PROF_TRSM_SMALL, st);
    if (n1 == 32)
      ::ibem::count_launch(), k_trsm_small_fixed<T, 32><<<(unsigned)((n2 + 127) / 128), 128, 0, st>>>(L, ldl, B, ldb, n2);
    else if (n1 == 64 && sizeof(T) == sizeof(float))
      ::ibem::count_launch(), k_trsm_small_fixed<T, 64><<<(unsigned)((n2 + 127) / 128), 128, 0, st>>>(L, ldl, B, ldb, n2);
    else
      ::ibem::count_launch(), k_trsm_small<T><<<(unsigned)((n2 + 63) / 64), 64, 2 * 64 * 65 * sizeof(T), st>>>(
          L, ldl, (int)n1, B, ldb, n2);
    IBEM_LAUNCH_CHECK("trsm_small");
    return IBEM_OK;
  }
  const int64_t h = std::max<int64_t>(kLeaf, (n1 / 2) / kLeaf * kLeaf);
  ibem_status s = trsm(L, ldl, h, B, ldb, n2, w, st);
  if (s) return s;
  s = gemm_sub<T>(n1 - h, n2, h, L + h, ldl, B, ldb, B + h, ldb, w, st);
  if (s) return s;
  return trsm(L + h * ldl + h, ldl, n1 - h, B + h, ldb, n2, w, st);
}

// recursive LU of the m x n column block starting at (k0, k0) of A (m = N - k0).
template <typename T>
static ibem_status lu_rec(T* A, int64_t lda, int64_t N, int64_t k0, int64_t n, LuWork<T>& w, cudaStream_t st) {
  const int64_t m = N - k0;
  if (n <= kLeaf) {
    ibem_status s = panel(A, lda, k0, m, (int)n, w, st);
    if (s) return s;
    // exchanges of this panel on the columns to its left and right (within [0, N))
    ProfScope ps(PROF_LASWP, st);
    const int64_t ncols = N - n;  // every column outside the panel
    if (ncols > 0)
      ::ibem::count_launch(), k_laswp<T><<<(unsigned)((ncols + 127) / 128), 128, 0, st>>>(A, lda, k0, w.ipiv_dev + k0,
                                                                                           (int)n, ncols);
    IBEM_LAUNCH_CHECK("laswp");
    return IBEM_OK;
  }
  const int64_t n1 = std::max<int64_t>(kLeaf, (n / 2) / kLeaf * kLeaf), n2 = n - n1;
  // left half (its exchanges are applied to every column, including the right half)
  ibem_status s = lu_rec(A, lda, N, k0, n1, w, st);
  if (s) return s;
  T* A11 = A + k0 * lda + k0;
  T* A12 = A + (k0 + n1) * lda + k0;
  T* A21 = A + k0 * lda + k0 + n1;
  T* A22 = A + (k0 + n1) * lda + k0 + n1;
  s = trsm(A11, lda, n1, A12, lda, n2, w, st);
  if (s) return s;
  s = gemm_sub<T>(m - n1, n2, n1, A21, lda, A12, lda, A22, lda, w, st);
  if (s) return s;
  return lu_rec(A, lda, N, k0 + n1, n2, w, st);
}

template <typename T>
static ibem_status lu_alloc(LuWork<T>& w, int64_t N) {
  int dev = 0, nsm = 0, smem_optin = 0;
  IBEM_CUDA(cudaGetDevice(&dev));
  IBEM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  IBEM_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const int static_smem = 2 * kLeaf * (int)sizeof(T) + 64;
  int dyn_cap = std::min(smem_optin - static_smem - 1024, 200 * 1024);
  w.rows_cap = dyn_cap / (kLeaf * (int)sizeof(T));
  IBEM_CUDA(cudaFuncSetAttribute((const void*)k_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_cap));
  IBEM_CUDA(set_solver_smem_attrs<T>());
  int per_sm = 0;
  IBEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_panel<T>, kPanelThreads,
                                                          (size_t)w.rows_cap * kLeaf * sizeof(T)));
  if (per_sm < 1) return fail(IBEM_ERR_CUDA, "panel kernel cannot be resident");
  w.ncta = std::min(nsm, kPanelThreads);  // one CTA per SM (co-resident for the cooperative launch);
                                          // the candidate argmax uses one thread per CTA
  if ((int64_t)w.ncta * w.rows_cap < N) return fail(IBEM_ERR_ARG, "matrix too large for the panel kernel");
  IBEM_CUDA(cudaMalloc(&w.cand, sizeof(T) * 2 * (size_t)w.ncta * kRec));
  IBEM_CUDA(cudaMalloc(&w.cnt, sizeof(unsigned) * 2));
  IBEM_CUDA(cudaMemset(w.cnt, 0, sizeof(unsigned) * 2));
  IBEM_CUDA(cudaMalloc(&w.ipiv_dev, sizeof(int) * (size_t)N));
  IBEM_CUDA(cudaMalloc(&w.perm, sizeof(int) * (size_t)N));
  IBEM_CUDA(cudaMalloc(&w.tmp, sizeof(double) * (size_t)N));
  IBEM_CUDA(cudaMalloc(&w.info, sizeof(int)));
  IBEM_CUDA(cudaMalloc(&w.gs, sizeof(GridSync)));
  IBEM_CUDA(cudaMemset(w.info, 0, sizeof(int)));
  IBEM_CUDA(cudaMemset(w.gs, 0, sizeof(GridSync)));
  if (sizeof(T) == sizeof(float)) {
    w.gemm_ws_bytes = gemm_tc_workspace_bytes(N, N / 2 + 2 * kLeaf);
    IBEM_CUDA(cudaMalloc(&w.gemm_ws, w.gemm_ws_bytes));
    IBEM_CUDA(cudaMalloc(&w.gemm_err, sizeof(int)));
    IBEM_CUDA(cudaMemset(w.gemm_err, 0, sizeof(int)));
  }
  return IBEM_OK;
}

template <typename T>
static void lu_free(LuWork<T>& w) {
  cudaFree(w.cand);
  cudaFree(w.cnt);
  cudaFree(w.ipiv_dev);
  cudaFree(w.perm);
  cudaFree(w.tmp);
  cudaFree(w.info);
  cudaFree(w.gs);
  cudaFree(w.gemm_ws);
  cudaFree(w.gemm_err);
  w = LuWork<T>();
}

// Solve with the factors F (precision T): y <- U^-1 L^-1 P y (y FP64, in place; tmp N-vector)
template <typename T>
static ibem_status lu_apply(const T* F, int64_t ldf, int64_t N, const int* perm, double* tmp, double* y,
                            cudaStream_t st) {
  ProfScope ps(PROF_TRSV, st, 2.0 * N * N);
  ::ibem::count_launch(), k_gather<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(N, perm, y, tmp);
  const size_t smem = sizeof(T) * kTrsvB * (kTrsvB + 1) + 16 + sizeof(double) * kTrsvB;
  // forward: unit lower, right-hand side and updates in tmp, solved blocks to y
  for (int64_t k0 = 0; k0 < N; k0 += kTrsvB) {
    const int b = (int)std::min<int64_t>(kTrsvB, N - k0);
    const int64_t rows = N - k0 - b;
    const unsigned grid = (unsigned)std::max<int64_t>(1, (rows + 255) / 256);
    ::ibem::count_launch(), k_trsv_block<T, true><<<grid, 256, smem, st>>>(F, ldf, N, k0, b, tmp, y);
  }
  // backward: upper, right-hand side and updates in y, solved blocks to tmp
  for (int64_t k0 = ((N - 1) / kTrsvB) * kTrsvB; k0 >= 0; k0 -= kTrsvB) {
    const int b = (int)std::min<int64_t>(kTrsvB, N - k0);
    const unsigned grid = (unsigned)std::max<int64_t>(1, (k0 + 255) / 256);
    ::ibem::count_launch(), k_trsv_block<T, false><<<grid, 256, smem, st>>>(F, ldf, N, k0, b, y, tmp);
  }
  IBEM_CUDA(cudaMemcpyAsync(y, tmp, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
  IBEM_LAUNCH_CHECK("lu_apply");
  return IBEM_OK;
}

// r = b - A x  (FP64)
static ibem_status residual(int64_t N, const double* A, int64_t lda, const double* x, const double* b, double* r,
                            double* part, int nparts, cudaStream_t st) {
  const int64_t chunk = (N + nparts - 1) / nparts;
  dim3 grid((unsigned)((N + 255) / 256), (unsigned)nparts);
  ::ibem::count_launch(), k_gemv_part<<<grid, 256, 0, st>>>(N, A, lda, x, chunk, part);
  ::ibem::count_launch(), k_residual<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(N, nparts, part, b, r);
  IBEM_LAUNCH_CHECK("residual");
  return IBEM_OK;
}


// ------------------------------------------------------------------ device vectors
namespace {
__global__ void k_dot_many(int64_t n, int nv, const double* __restrict__ V, int64_t ldv, const double* __restrict__ w,
                           double* __restrict__ out) {
  // out[j] += sum_i V[i,j] w[i]  (grid-stride over rows, one atomic per block and vector)
  __shared__ double red[256];
  for (int j = 0; j < nv; ++j) {
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      s += V[j * ldv + i] * w[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int t = blockDim.x / 2; t > 0; t >>= 1) {
      if (threadIdx.x < t) red[threadIdx.x] += red[threadIdx.x + t];
      __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(out + j, red[0]);
    __syncthreads();
  }
}
// w -= V h (h on device, nv entries); y = alpha x
__global__ void k_sub_Vh(int64_t n, int nv, const double* __restrict__ V, int64_t ldv, const double* __restrict__ h,
                         double* __restrict__ w) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
  for (int j = 0; j < nv; ++j) s += V[j * ldv + i] * h[j];
  w[i] -= s;
}
__global__ void k_axpby(int64_t n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i] + b * y[i];
}
}  // namespace

static double host_absmax(const std::vector<double>& v) {
  double m = 0;
  for (double x : v) m = std::max(m, std::fabs(x));
  return m;
}

struct SolveCtx {
  int64_t N;
  cudaStream_t st;
  double *r = nullptr, *c = nullptr, *part = nullptr, *rs = nullptr;
  int nparts = 16;
  ibem_status alloc(int64_t n, cudaStream_t s) {
    N = n;
    st = s;
    IBEM_CUDA(cudaMalloc(&r, sizeof(double) * N));
    IBEM_CUDA(cudaMalloc(&c, sizeof(double) * N));
    IBEM_CUDA(cudaMalloc(&rs, sizeof(double) * N));
    IBEM_CUDA(cudaMalloc(&part, sizeof(double) * N * nparts));
    return IBEM_OK;
  }
  ~SolveCtx() {
    cudaFree(r);
    cudaFree(c);
    cudaFree(part);
    cudaFree(rs);
  }
};

static ibem_status vec_to_host(const double* d, int64_t n, std::vector<double>& h, cudaStream_t st) {
  h.resize(n);
  IBEM_CUDA(cudaMemcpyAsync(h.data(), d, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  IBEM_CUDA(cudaStreamSynchronize(st));
  return IBEM_OK;
}

namespace {
// row sums of |R A C| (the inf-norm of the equilibrated matrix)
__global__ void k_scaled_rowsum(int64_t n, const double* __restrict__ A, int64_t lda, const double* __restrict__ r,
                                const double* __restrict__ c, double* __restrict__ rs) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
  for (int64_t j = 0; j < n; ++j) s += fabs(A[j * lda + i]) * c[j];
  rs[i] = s * r[i];
}
// y = r .* (A (c .* v)) via the partial-sum GEMV; tmp is an N-vector
__global__ void k_scale_rows_of_parts(int64_t n, int nparts, const double* __restrict__ part,
                                      const double* __restrict__ r, double* __restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
  for (int p = 0; p < nparts; ++p) s += part[p * n + i];
  y[i] = r[i] * s;
}
}  // namespace

// y = As v with As = R A C (FP64; tmp is N-vector scratch)
static ibem_status scaled_matvec(SolveCtx& cx, const double* A, int64_t lda, const double* v, double* tmp,
                                 double* y) {
  const int64_t N = cx.N;
  ProfScope ps(PROF_MATVEC, cx.st, 2.0 * N * N);
  const unsigned nb = (unsigned)((N + 255) / 256);
  ::ibem::count_launch(), k_vmul<<<nb, 256, 0, cx.st>>>(N, cx.c, v, tmp);
  const int64_t chunk = (N + cx.nparts - 1) / cx.nparts;
  ::ibem::count_launch(), k_gemv_part<<<dim3(nb, (unsigned)cx.nparts), 256, 0, cx.st>>>(N, A, lda, tmp, chunk, cx.part);
  ::ibem::count_launch(), k_scale_rows_of_parts<<<nb, 256, 0, cx.st>>>(N, cx.nparts, cx.part, cx.r, y);
  IBEM_LAUNCH_CHECK("scaled_matvec");
  return IBEM_OK;
}

// scaled backward error of ys for As ys = bs: ||bs - As ys|| / (||As|| ||ys|| + ||bs||)  (inf-norms)
static ibem_status scaled_backward_error(SolveCtx& cx, const double* A, int64_t lda, const double* ys,
                                         const double* bs, double* rvec, double* tmp, double as_norm, double& be) {
  ibem_status s = scaled_matvec(cx, A, lda, ys, tmp, rvec);
  if (s) return s;
  ::ibem::count_launch(), k_axpby<<<(unsigned)((cx.N + 255) / 256), 256, 0, cx.st>>>(cx.N, 1.0, bs, -1.0, rvec);  // rvec = bs - As ys
  std::vector<double> hr, hy, hb;
  if ((s = vec_to_host(rvec, cx.N, hr, cx.st))) return s;
  if ((s = vec_to_host(ys, cx.N, hy, cx.st))) return s;
  if ((s = vec_to_host(bs, cx.N, hb, cx.st))) return s;
  be = host_absmax(hr) / (as_norm * host_absmax(hy) + host_absmax(hb));
  return IBEM_OK;
}

template <typename T>
static ibem_status factor(SolveCtx& cx, const double* A, int64_t lda, T*& W, LuWork<T>& w, int& info) {
  const int64_t N = cx.N;
  IBEM_CUDA(cudaMalloc(&W, sizeof(T) * (size_t)N * N));
  {
    ProfScope ps(PROF_EQUIL, cx.st);
    ::ibem::count_launch(), k_rowmax<<<(unsigned)((N + 255) / 256), 256, 0, cx.st>>>(N, A, lda, cx.r);
    ::ibem::count_launch(), k_colmax<<<(unsigned)N, 256, 0, cx.st>>>(N, A, lda, cx.r, cx.c);
    dim3 g((unsigned)((N + 255) / 256), (unsigned)N);
    ::ibem::count_launch(), k_scale_copy<T><<<g, 256, 0, cx.st>>>(N, A, lda, cx.r, cx.c, W, N);
    IBEM_LAUNCH_CHECK("equilibrate");
  }
  ibem_status s = lu_alloc(w, N);
  if (s) return s;
  s = lu_rec<T>(W, N, N, 0, N, w, cx.st);
  if (s) return s;
  // row permutation from the sequence of exchanges (LAPACK ipiv semantics)
  {
    std::vector<int> ip((size_t)N), perm((size_t)N);
    IBEM_CUDA(cudaMemcpyAsync(ip.data(), w.ipiv_dev, sizeof(int) * N, cudaMemcpyDeviceToHost, cx.st));
    IBEM_CUDA(cudaStreamSynchronize(cx.st));
    for (int64_t i = 0; i < N; ++i) perm[i] = (int)i;
    for (int64_t i = 0; i < N; ++i) {
      const int p = ip[i];
      if (p < 0 || p >= N) return fail(IBEM_ERR_CUDA, "factorisation produced an invalid pivot");
      std::swap(perm[i], perm[p]);
    }
    IBEM_CUDA(cudaMemcpyAsync(w.perm, perm.data(), sizeof(int) * N, cudaMemcpyHostToDevice, cx.st));
    IBEM_CUDA(cudaStreamSynchronize(cx.st));
  }
  int hinfo = 0, herr = 0;
  GridSync hgs;
  IBEM_CUDA(cudaMemcpyAsync(&hinfo, w.info, sizeof(int), cudaMemcpyDeviceToHost, cx.st));
  IBEM_CUDA(cudaMemcpyAsync(&hgs, w.gs, sizeof(GridSync), cudaMemcpyDeviceToHost, cx.st));
  if (w.gemm_err) IBEM_CUDA(cudaMemcpyAsync(&herr, w.gemm_err, sizeof(int), cudaMemcpyDeviceToHost, cx.st));
  IBEM_CUDA(cudaStreamSynchronize(cx.st));
  if (hgs.err) return fail(IBEM_ERR_TIMEOUT, "panel grid barrier gave up");
  if (herr) return fail(IBEM_ERR_TIMEOUT, "tensor-core GEMM wait gave up");
  info = hinfo;
  return IBEM_OK;
}

ibem_status solve_dense(ibem_solver_form form, int64_t N, double* A, int64_t lda, const double* b, double* x,
                        double tol, ibem_solve_report* rep, cudaStream_t st) {
  if (N <= 0 || !A || !b || !x || lda < N) return fail(IBEM_ERR_ARG, "solve: bad sizes or pointers");
  if (form != IBEM_SOLVE_FP64 && form != IBEM_SOLVE_MIXED_IR) return fail(IBEM_ERR_ARG, "unknown solver form");
  SolveCtx cx;
  ibem_status s = cx.alloc(N, st);
  if (s) return s;
  // Everything below works on the equilibrated system  As ys = bs,  As = R A C,
  // bs = R b, x = C ys: errors are measured row-relative, so the small boundary rows of
  // the iBEM matrix weigh as much as the inclusion rows.
  double *bs = nullptr, *ys = nullptr, *rvec = nullptr, *tmp = nullptr;
  IBEM_CUDA(cudaMalloc(&bs, sizeof(double) * N));
  IBEM_CUDA(cudaMalloc(&ys, sizeof(double) * N));
  IBEM_CUDA(cudaMalloc(&rvec, sizeof(double) * N));
  IBEM_CUDA(cudaMalloc(&tmp, sizeof(double) * N));
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  ibem_solve_report R{};
  const unsigned nb = (unsigned)((N + 255) / 256);
  cudaEventRecord(e0, st);
  double as_norm = 0;
  auto finish_norm = [&]() -> ibem_status {
    ::ibem::count_launch(), k_scaled_rowsum<<<nb, 256, 0, st>>>(N, A, lda, cx.r, cx.c, cx.rs);
    IBEM_LAUNCH_CHECK("scaled_rowsum");
    std::vector<double> h;
    ibem_status q = vec_to_host(cx.rs, N, h, st);
    as_norm = host_absmax(h);
    return q;
  };
  if (form == IBEM_SOLVE_FP64) {
    double* W = nullptr;
    LuWork<double> w;
    int info = 0;
    s = factor<double>(cx, A, lda, W, w, info);
    cudaEventRecord(e1, st);
    if (!s && info) { R.info = info; s = fail(IBEM_ERR_SINGULAR, "zero pivot in the FP64 factorisation"); }
    if (!s) {
      ::ibem::count_launch(), k_vmul<<<nb, 256, 0, st>>>(N, cx.r, b, bs);
      IBEM_CUDA(cudaMemcpyAsync(ys, bs, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
      s = lu_apply<double>(W, N, N, w.perm, w.tmp, ys, st);
    }
    cudaEventRecord(e2, st);
    if (!s) s = finish_norm();
    if (!s) s = scaled_backward_error(cx, A, lda, ys, bs, rvec, tmp, as_norm, R.backward_error);
    lu_free(w);
    cudaFree(W);
  } else {
    float* W = nullptr;
    LuWork<float> w;
    int info = 0;
    s = factor<float>(cx, A, lda, W, w, info);
    cudaEventRecord(e1, st);
    if (!s && info) { R.info = info; s = fail(IBEM_ERR_SINGULAR, "zero pivot in the FP32 factorisation"); }
    // GMRES(m) on As d = rs, right-preconditioned by the FP32 factors of As, all in FP64
    const int m = 30, max_outer = 20;
    double *V = nullptr, *Z = nullptr, *hd = nullptr;
    if (!s) {
      cudaError_t ce = cudaMalloc(&V, sizeof(double) * (size_t)N * (m + 1));
      if (ce == cudaSuccess) ce = cudaMalloc(&Z, sizeof(double) * (size_t)N * m);
      if (ce == cudaSuccess) ce = cudaMalloc(&hd, sizeof(double) * (m + 1) * 2);
      if (ce != cudaSuccess) s = cuda_fail(ce, "gmres workspace");
    }
    if (!s) {
      ::ibem::count_launch(), k_vmul<<<nb, 256, 0, st>>>(N, cx.r, b, bs);
      IBEM_CUDA(cudaMemcpyAsync(ys, bs, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
      s = lu_apply<float>(W, N, N, w.perm, w.tmp, ys, st);
    }
    if (!s) s = finish_norm();
    int iters = 0;
    for (int outer = 0; !s && outer < max_outer; ++outer) {
      double be = 0;
      if ((s = scaled_backward_error(cx, A, lda, ys, bs, rvec, tmp, as_norm, be))) break;
      R.backward_error = be;
      if (be <= tol) break;
      // rvec holds rs = bs - As ys
      IBEM_CUDA(cudaMemsetAsync(hd, 0, sizeof(double), st));
      ::ibem::count_launch(), k_dot_many<<<256, 256, 0, st>>>(N, 1, rvec, N, rvec, hd);
      double b2 = 0;
      IBEM_CUDA(cudaMemcpyAsync(&b2, hd, sizeof(double), cudaMemcpyDeviceToHost, st));
      IBEM_CUDA(cudaStreamSynchronize(st));
      const double beta = std::sqrt(std::max(b2, 0.0));
      if (beta == 0) break;
      ::ibem::count_launch(), k_axpby<<<nb, 256, 0, st>>>(N, 1.0 / beta, rvec, 0.0, V);
      std::vector<double> H((m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0);
      g[0] = beta;
      int k = 0;
      for (; k < m; ++k) {
        double* vk = V + (size_t)k * N;
        double* zk = Z + (size_t)k * N;
        double* wv = V + (size_t)(k + 1) * N;
        IBEM_CUDA(cudaMemcpyAsync(zk, vk, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        if ((s = lu_apply<float>(W, N, N, w.perm, w.tmp, zk, st))) break;
        if ((s = scaled_matvec(cx, A, lda, zk, tmp, wv))) break;
        // classical Gram-Schmidt, twice
        std::vector<double> hk(k + 1, 0.0), h2(k + 1);
        for (int pass = 0; pass < 2; ++pass) {
          IBEM_CUDA(cudaMemsetAsync(hd, 0, sizeof(double) * (k + 1), st));
          ::ibem::count_launch(), k_dot_many<<<256, 256, 0, st>>>(N, k + 1, V, N, wv, hd);
          ::ibem::count_launch(), k_sub_Vh<<<nb, 256, 0, st>>>(N, k + 1, V, N, hd, wv);
          IBEM_CUDA(cudaMemcpyAsync(h2.data(), hd, sizeof(double) * (k + 1), cudaMemcpyDeviceToHost, st));
          IBEM_CUDA(cudaStreamSynchronize(st));
          for (int i = 0; i <= k; ++i) hk[i] += h2[i];
        }
        IBEM_CUDA(cudaMemsetAsync(hd, 0, sizeof(double), st));
        ::ibem::count_launch(), k_dot_many<<<256, 256, 0, st>>>(N, 1, wv, N, wv, hd);
        double nrm2 = 0;
        IBEM_CUDA(cudaMemcpyAsync(&nrm2, hd, sizeof(double), cudaMemcpyDeviceToHost, st));
        IBEM_CUDA(cudaStreamSynchronize(st));
        const double hn = std::sqrt(std::max(nrm2, 0.0));
        if (hn > 0) ::ibem::count_launch(), k_axpby<<<nb, 256, 0, st>>>(N, 1.0 / hn, wv, 0.0, wv);
        for (int i = 0; i <= k; ++i) H[i * m + k] = hk[i];
        H[(k + 1) * m + k] = hn;
        for (int i = 0; i < k; ++i) {  // previous Givens rotations
          const double t = cs[i] * H[i * m + k] + sn[i] * H[(i + 1) * m + k];
          H[(i + 1) * m + k] = -sn[i] * H[i * m + k] + cs[i] * H[(i + 1) * m + k];
          H[i * m + k] = t;
        }
        const double den = std::hypot(H[k * m + k], H[(k + 1) * m + k]);
        cs[k] = den > 0 ? H[k * m + k] / den : 1.0;
        sn[k] = den > 0 ? H[(k + 1) * m + k] / den : 0.0;
        H[k * m + k] = den;
        H[(k + 1) * m + k] = 0;
        g[k + 1] = -sn[k] * g[k];
        g[k] = cs[k] * g[k];
        ++iters;
        // stop the inner cycle once the scaled residual estimate is well below tol
        if (std::fabs(g[k + 1]) <= 1e-2 * tol * (as_norm + 1.0) || hn == 0) { ++k; break; }
      }
      if (s) break;
      std::vector<double> yv(k, 0.0);
      for (int i = k - 1; i >= 0; --i) {
        double t = g[i];
        for (int j2 = i + 1; j2 < k; ++j2) t -= H[i * m + j2] * yv[j2];
        yv[i] = t / H[i * m + i];
      }
      IBEM_CUDA(cudaMemcpyAsync(hd, yv.data(), sizeof(double) * k, cudaMemcpyHostToDevice, st));
      ::ibem::count_launch(), k_axpby<<<nb, 256, 0, st>>>(N, -1.0, ys, 0.0, ys);  // ys = -ys
      ::ibem::count_launch(), k_sub_Vh<<<nb, 256, 0, st>>>(N, k, Z, N, hd, ys);    // ys = -ys - Z y
      ::ibem::count_launch(), k_axpby<<<nb, 256, 0, st>>>(N, -1.0, ys, 0.0, ys);  // ys = ys + Z y
      IBEM_LAUNCH_CHECK("gmres update");
    }
    cudaEventRecord(e2, st);
    if (!s) {
      double be = 0;
      s = scaled_backward_error(cx, A, lda, ys, bs, rvec, tmp, as_norm, be);
      R.backward_error = be;
      if (!s && be > tol) s = fail(IBEM_ERR_NOCONV, "GMRES-IR did not reach the tolerance");
    }
    R.iterations = iters;
    cudaFree(V);
    cudaFree(Z);
    cudaFree(hd);
    lu_free(w);
    cudaFree(W);
  }
  if (!s) ::ibem::count_launch(), k_vmul<<<nb, 256, 0, st>>>(N, cx.c, ys, x);  // x = C ys
  cudaStreamSynchronize(st);
  float t1 = 0, t2 = 0;
  cudaEventElapsedTime(&t1, e0, e1);
  cudaEventElapsedTime(&t2, e1, e2);
  R.t_factor_ms = t1;
  R.t_solve_ms = t2;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  cudaFree(bs);
  cudaFree(ys);
  cudaFree(rvec);
  cudaFree(tmp);
  if (rep) *rep = R;
  return s;
}


// ===================================================================================
// Allocation-free FP64 solve for small systems (no counterpart in the reference).
//
// For callers that must not allocate device memory: applications whose device memory is
// owned by a host framework (a caching allocator or a fixed budget reserved up front),
// where a raw cudaMalloc can fail or fragment that budget, and latency-critical loops,
// where cudaMalloc/cudaFree may synchronise the device.  The caller passes A, b and x;
// every other buffer of the solve (the factor copy, scalings, pivots, permutation, the
// panel kernel's candidate rows and grid barrier, residual scratch) lives in one
// file-scope static __device__ array of kNoAllocBytes, so N is limited to kNoAllocMaxN.
// The array is held by every GPU that loads the library until the process exits.
// Its device address is looked up once per device, on that device's first call
// (cudaGetSymbolAddress); make that first call before any stream capture.  All calls
// share the array and it keeps the last call's contents: calls that overlap on the GPU
// (other host threads, other streams) race and must be serialised by the caller.
// ===================================================================================
namespace {
constexpr int64_t kNoAllocMaxN = 1024;
constexpr int kNoAllocMaxCta = 256;   // panel kernel CTAs (>= SMs of one GPU)
constexpr int kNoAllocParts = 16;
constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kNaW = 0;                                                           // N x N factor copy
constexpr size_t kNaVec = align256(sizeof(double) * kNoAllocMaxN * kNoAllocMaxN);    // 6 N-vectors
constexpr size_t kNaPerm = kNaVec + 6 * align256(sizeof(double) * kNoAllocMaxN);     // perm, ipiv
constexpr size_t kNaCand = kNaPerm + 2 * align256(sizeof(int) * kNoAllocMaxN);
constexpr size_t kNaSeq = kNaCand + align256(sizeof(double) * 2 * kNoAllocMaxCta * kRec);  // panel records
constexpr size_t kNaGs = kNaSeq + align256(sizeof(unsigned) * 2);                            // panel counters
constexpr size_t kNaInfo = kNaGs + align256(sizeof(GridSync));
constexpr size_t kNaPart = kNaInfo + align256(sizeof(int));
constexpr size_t kNaRed = kNaPart + align256(sizeof(double) * kNoAllocParts * kNoAllocMaxN);
constexpr size_t kNoAllocBytes = kNaRed + align256(sizeof(double) * 4);

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_base[kNoAllocMaxDevices] = {};
int g_noalloc_ncta[kNoAllocMaxDevices] = {};
int g_noalloc_rows_cap[kNoAllocMaxDevices] = {};

// row exchanges (LAPACK ipiv) -> gather permutation, one thread (N <= kNoAllocMaxN)
__global__ void k_ipiv_to_perm(int64_t n, const int* __restrict__ ipiv, int* __restrict__ perm) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int64_t i = 0; i < n; ++i) perm[i] = (int)i;
  for (int64_t i = 0; i < n; ++i) {
    int p = ipiv[i];
    if (p < 0 || p >= n) p = (int)i;  // never index outside (a bad pivot shows in info)
    const int t = perm[i];
    perm[i] = perm[p];
    perm[p] = t;
  }
}

// out[0..3] = max|a|, max|b|, max|c|, max|d| over n entries (one block)
__global__ void k_absmax4(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                          const double* __restrict__ c, const double* __restrict__ d, double* __restrict__ out) {
  __shared__ double red[4][256];
  double m[4] = {0, 0, 0, 0};
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    m[0] = fmax(m[0], fabs(a[i]));
    m[1] = fmax(m[1], fabs(b[i]));
    m[2] = fmax(m[2], fabs(c[i]));
    m[3] = fmax(m[3], fabs(d[i]));
  }
  for (int q = 0; q < 4; ++q) red[q][threadIdx.x] = m[q];
  __syncthreads();
  for (int t = blockDim.x / 2; t > 0; t >>= 1) {
    if (threadIdx.x < t)
      for (int q = 0; q < 4; ++q) red[q][threadIdx.x] = fmax(red[q][threadIdx.x], red[q][threadIdx.x + t]);
    __syncthreads();
  }
  if (threadIdx.x < 4) out[threadIdx.x] = red[threadIdx.x][0];
}
}  // namespace

static ibem_status noalloc_setup(int dev, unsigned char** base, int* ncta, int* rows_cap) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(IBEM_ERR_ARG, "solve_noalloc: device index out of range");
  if (!g_noalloc_base[dev]) {
    void* p = nullptr;
    IBEM_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    int nsm = 0, smem_optin = 0;
    IBEM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    IBEM_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (nsm > kNoAllocMaxCta) return fail(IBEM_ERR_ARG, "solve_noalloc: more SMs than the static panel scratch holds");
    const int static_smem = 2 * kLeaf * (int)sizeof(double) + 64;
    const int dyn_cap = std::min(smem_optin - static_smem - 1024, 200 * 1024);
    IBEM_CUDA(cudaFuncSetAttribute((const void*)k_panel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   dyn_cap));
    IBEM_CUDA(set_solver_smem_attrs<double>());
    int per_sm = 0;
    const int cap = dyn_cap / (kLeaf * (int)sizeof(double));
    IBEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_panel<double>, kPanelThreads,
                                                            (size_t)cap * kLeaf * sizeof(double)));
    if (per_sm < 1) return fail(IBEM_ERR_CUDA, "solve_noalloc: panel kernel cannot be resident");
    g_noalloc_ncta[dev] = std::min(nsm, kPanelThreads);
    g_noalloc_rows_cap[dev] = cap;
    g_noalloc_base[dev] = static_cast<unsigned char*>(p);
  }
  *base = g_noalloc_base[dev];
  *ncta = g_noalloc_ncta[dev];
  *rows_cap = g_noalloc_rows_cap[dev];
  return IBEM_OK;
}

ibem_status solve_fp64_noalloc(int64_t N, const double* A, int64_t lda, const double* b, double* x,
                               ibem_solve_report* rep, cudaStream_t st) {
  if (N <= 0 || N > kNoAllocMaxN) {
    char buf[128];
    std::snprintf(buf, sizeof buf, "solve_noalloc: N = %lld outside 1..%lld (the static workspace limit)",
                  (long long)N, (long long)kNoAllocMaxN);
    return fail(IBEM_ERR_ARG, buf);
  }
  if (!A || !b || !x || lda < N) return fail(IBEM_ERR_ARG, "solve_noalloc: bad pointers or lda");
  int dev = 0;
  IBEM_CUDA(cudaGetDevice(&dev));
  unsigned char* base = nullptr;
  int ncta = 0, rows_cap = 0;
  ibem_status s = noalloc_setup(dev, &base, &ncta, &rows_cap);
  if (s) return s;
  double* W = reinterpret_cast<double*>(base + kNaW);
  double* vec[6];
  for (int i = 0; i < 6; ++i) vec[i] = reinterpret_cast<double*>(base + kNaVec + i * align256(sizeof(double) * kNoAllocMaxN));
  double *r = vec[0], *c = vec[1], *bs = vec[2], *ys = vec[3], *tmp = vec[4], *rv = vec[5];
  int* perm = reinterpret_cast<int*>(base + kNaPerm);
  int* ipiv = reinterpret_cast<int*>(base + kNaPerm + align256(sizeof(int) * kNoAllocMaxN));
  GridSync* gs = reinterpret_cast<GridSync*>(base + kNaGs);
  int* info = reinterpret_cast<int*>(base + kNaInfo);
  double* part = reinterpret_cast<double*>(base + kNaPart);
  double* red = reinterpret_cast<double*>(base + kNaRed);
  // the previous call's contents are still there: clear what must start at zero
  IBEM_CUDA(cudaMemsetAsync(gs, 0, sizeof(GridSync), st));
  IBEM_CUDA(cudaMemsetAsync(info, 0, sizeof(int), st));
  unsigned* cntf = reinterpret_cast<unsigned*>(base + kNaSeq);
  IBEM_CUDA(cudaMemsetAsync(cntf, 0, sizeof(unsigned) * 2, st));
  const unsigned nb = (unsigned)((N + 255) / 256);
  ::ibem::count_launch(), k_rowmax<<<nb, 256, 0, st>>>(N, A, lda, r);
  ::ibem::count_launch(), k_colmax<<<(unsigned)N, 256, 0, st>>>(N, A, lda, r, c);
  ::ibem::count_launch(), k_scale_copy<double><<<dim3(nb, (unsigned)N), 256, 0, st>>>(N, A, lda, r, c, W, N);
  IBEM_LAUNCH_CHECK("solve_noalloc: equilibrate");
  LuWork<double> w;
  w.cand = reinterpret_cast<double*>(base + kNaCand);
  w.cnt = cntf;
  w.ipiv_dev = ipiv;
  w.perm = perm;
  w.tmp = tmp;
  w.info = info;
  w.gs = gs;
  w.ncta = ncta;
  w.rows_cap = rows_cap;
  if ((s = lu_rec<double>(W, N, N, 0, N, w, st))) return s;
  ::ibem::count_launch(), k_ipiv_to_perm<<<1, 1, 0, st>>>(N, ipiv, perm);
  ::ibem::count_launch(), k_vmul<<<nb, 256, 0, st>>>(N, r, b, bs);
  IBEM_CUDA(cudaMemcpyAsync(ys, bs, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
  if ((s = lu_apply<double>(W, N, N, perm, tmp, ys, st))) return s;
  ::ibem::count_launch(), k_vmul<<<nb, 256, 0, st>>>(N, c, ys, x);
  // scaled backward error, reduced on the device
  ::ibem::count_launch(), k_vmul<<<nb, 256, 0, st>>>(N, c, ys, tmp);
  const int64_t chunk = (N + kNoAllocParts - 1) / kNoAllocParts;
  ::ibem::count_launch(), k_gemv_part<<<dim3(nb, kNoAllocParts), 256, 0, st>>>(N, A, lda, tmp, chunk, part);
  ::ibem::count_launch(), k_scale_rows_of_parts<<<nb, 256, 0, st>>>(N, kNoAllocParts, part, r, rv);
  ::ibem::count_launch(), k_axpby<<<nb, 256, 0, st>>>(N, 1.0, bs, -1.0, rv);
  ::ibem::count_launch(), k_scaled_rowsum<<<nb, 256, 0, st>>>(N, A, lda, r, c, tmp);
  ::ibem::count_launch(), k_absmax4<<<1, 256, 0, st>>>(N, rv, ys, bs, tmp, red);
  IBEM_LAUNCH_CHECK("solve_noalloc");
  double h[4] = {0, 0, 0, 0};
  int hinfo = 0;
  GridSync hgs{};
  IBEM_CUDA(cudaMemcpyAsync(h, red, sizeof h, cudaMemcpyDeviceToHost, st));
  IBEM_CUDA(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st));
  IBEM_CUDA(cudaMemcpyAsync(&hgs, gs, sizeof(GridSync), cudaMemcpyDeviceToHost, st));
  IBEM_CUDA(cudaStreamSynchronize(st));
  if (rep) {
    ibem_solve_report R{};
    R.backward_error = h[0] / (h[3] * h[1] + h[2]);
    R.info = hinfo;
    *rep = R;
  }
  if (hgs.err) return fail(IBEM_ERR_TIMEOUT, "solve_noalloc: panel grid barrier gave up");
  if (hinfo) return fail(IBEM_ERR_SINGULAR, "solve_noalloc: zero pivot");
  return IBEM_OK;
}

}  // namespace ibem
