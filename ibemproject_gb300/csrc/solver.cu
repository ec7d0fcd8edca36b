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
//   IBEM_SOLVE_GMRES_BJ  no factorisation: iterative refinement whose corrections are GMRES
//                        solves with an FP32 copy of the scaled matrix (products accumulated
//                        in FP64), right-preconditioned by the inverses of its diagonal
//                        blocks (one block per particle); FP64 residuals decide convergence.
//                        Far cheaper than a factorisation for the small, well-conditioned
//                        systems of far-field microstructures (a few thousand to 30,000
//                        unknowns), whose LU is bound by launch latency.
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
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "ibem_internal.h"
#include "prof.h"
#include "solver.h"

namespace ibem {
namespace {

constexpr int kPanelThreads = 256;
constexpr int kLeaf = 32;                   // panel width of the recursion leaves
constexpr int kLdS = kLeaf + 1;             // shared-memory row stride of panel rows (no bank conflicts)
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

// row max over a column chunk (grid.y = chunk): coalesced along columns, N x chunks threads
__global__ void k_rowmax_part(int64_t n, const double* __restrict__ A, int64_t lda, int64_t chunk,
                              double* __restrict__ part) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
  if (i >= n) return;
  double m = 0;
  for (int64_t j = j0; j < j1; ++j) m = fmax(m, fabs(A[j * lda + i]));
  part[blockIdx.y * n + i] = m;
}
__global__ void k_rowmax_fin(int64_t n, int nparts, const double* __restrict__ part, double* __restrict__ r) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double m = 0;
  for (int p = 0; p < nparts; ++p) m = fmax(m, part[p * n + i]);
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
  if (i >= n) return;
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y) W[j * ldw + i] = (T)(r[i] * A[j * lda + i] * c[j]);
}

// ---------------------------------------------------------------- panel error flag
// Sticky error flag shared by the CTAs of the panel kernel: set when a spin gives up.
struct GridSync {
  int err;
};

// ---------------------------------------------------------------- panel kernel
// Factorises the m x nb panel (nb <= kLeaf) at P with tournament pivoting (communication-
// avoiding LU, Grigori-Demmel-Xiang): rows are split evenly over the CTAs and staged in
// shared memory.
//  1. Every CTA runs partial-pivoting elimination on its own rows and publishes the
//     original values of the (up to nb) rows it picked as pivots: cand[cta], flag f0[cta].
//  2. The leader of every group of F consecutive CTAs waits for its members, runs the same
//     elimination on their candidates and publishes its nb winners: lcand[g], flag f1[g].
//  3. CTA 0 waits for every group, eliminates their winners and so fixes the nb pivot rows
//     and the factored top block (L11 below the diagonal, U11 on and above it).  It turns
//     the pivot order into LAPACK row exchanges (ipiv) and a short list of the rows >= nb
//     that receive one of the original top rows, and releases the broadcast flag fb.
//  4. Every CTA writes its rows of the factored panel: the top rows from the broadcast, the
//     others as L = A_row U11^-1 from the row's original values (its own or, for a row
//     that received one of the top rows, that row's original values from the broadcast).
// Each wait is one polling thread, bounded by kSpinLimit; a wait that gives up sets the
// sticky gs->err and the CTA returns.  Flags hold the tag of the launch (unique and
// increasing within a factorisation), so they are never cleared between launches.
// Pivots: largest |a| to 14 bits, ties to the smallest row, so the result is deterministic.
constexpr int kCaluMinRows = 256;   // fewest rows a CTA takes before fewer CTAs are used

__device__ __forceinline__ int ld_acquire_s32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_s32(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename T>
struct CaluBufs {
  T* cand;     // [ncta][kLeaf][kLeaf] original values of each CTA's pivot rows (row-major)
  int* cidx;   // [ncta][kLeaf] their panel rows (-1: none)
  T* lcand;    // [groups][kLeaf][kLeaf] group winners
  int* lidx;   // [groups][kLeaf]
  T* top;      // [kLeaf][kLeaf] factored top block
  T* orig;     // [kLeaf][kLeaf] original values of the panel's first nb rows
  int* meta;   // [0, kLeaf) ipiv (panel-local), [kLeaf, 2 kLeaf) displaced rows,
               // [2 kLeaf, 3 kLeaf) their source rows, [3 kLeaf] count,
               // [3 kLeaf + 1, 4 kLeaf + 1) the pivot rows in order (panel-local; a record)
  int* flags;  // [0, kCaluMaxCta) f0, [kCaluMaxCta, 2 kCaluMaxCta) f1, [2 kCaluMaxCta] fb
};
constexpr int kCaluMaxCta = 256;
constexpr int kMetaLen = 4 * kLeaf + 1;

constexpr int kPanelRmax = 4;  // rows per thread at most (1024 rows per elimination)

// Partial-pivoting elimination of the rows held in registers: thread t holds rows
// q = t + kPanelThreads i (i < R) in a[i][*]; live[i] marks rows that exist and are not yet
// pivots.  Picks k pivots: s_sel[j] = q of pivot j (-1 when the rows ran out) and
// s_top[j][*] = that row as it stood at step j (multipliers left of j, U from j on).
// Before step j every live row is stored rotated by j: a[c] = column (c + j) mod kLeaf, so
// column j is a[0], the columns still to update are a[1 .. kLeaf-1-j] and the multipliers
// of steps 0 .. j-1 sit in a[kLeaf-j .. kLeaf-1].  One step rotates by one more (update and
// shift fused), which keeps every register index static while the column loop stays
// rolled (small code: the loop runs from the instruction cache).  The pivot's reciprocal
// scales the column, as LAPACK's getf2 does.  Two CTA barriers per column; every thread
// folds the warp winners in the same order, so all agree on the pivot.
__device__ __forceinline__ float calu_rcp(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double calu_rcp(double x) { return __drcp_rn(x); }

// Pivot search key of row q (< 1024) with |a| = av: the top 22 bits of the FP32 |a| above
// the inverted row index, so one unsigned max picks the largest |a| (to 14 bits, about
// 6e-5 relative) with ties to the smallest row; 0 is "no row".
__device__ __forceinline__ unsigned calu_key(float av, int q) {
  return (((__float_as_uint(av) >> 9) + 1u) << 10) | (unsigned)(1023 - q);
}

template <typename T, int R>
__device__ __forceinline__ void calu_elim(T (&a)[R][kLeaf], bool (&live)[R], int k, T* s_top, T* s_pr, int* s_sel,
                                          unsigned* s_key) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int nw = kPanelThreads / 32;
#pragma unroll 1
  for (int j = 0; j < k; ++j) {
    unsigned key = 0;
#pragma unroll
    for (int i = 0; i < R; ++i)
      if (live[i]) key = max(key, calu_key((float)fabs(a[i][0]), tid + kPanelThreads * i));
    key = __reduce_max_sync(0xffffffffu, key);
    if (lane == 0) s_key[warp] = key;
    __syncthreads();
#pragma unroll
    for (int w = 0; w < nw; ++w) key = max(key, s_key[w]);
    if (key == 0) {  // uniform: no rows left for this and later pivots
      if (tid == 0)
        for (int jj = j; jj < k; ++jj) s_sel[jj] = -1;
      break;
    }
    const int bq = 1023 - (int)(key & 1023u);
    // the owner thread alone publishes the pivot row: un-rotated into s_top[j] (the
    // factored block) and rotated into s_pr (the update's operand, static offsets, zero
    // where a[] holds multipliers)
    if (tid == bq % kPanelThreads) {
      const int oi = bq / kPanelThreads;
#pragma unroll
      for (int c = 0; c < kLeaf; ++c) {
        T v = a[0][c];
#pragma unroll
        for (int i = 1; i < R; ++i) v = oi == i ? a[i][c] : v;  // selects, not an indexed read
        s_top[j * kLdS + ((c + j) & (kLeaf - 1))] = v;
        s_pr[c] = (c + j < kLeaf) ? v : (T)0;
      }
#pragma unroll
      for (int i = 0; i < R; ++i) live[i] = live[i] && oi != i;
      s_sel[j] = bq;
    }
    __syncthreads();
    T pr[kLeaf];
#pragma unroll
    for (int c = 0; c < kLeaf; ++c) pr[c] = s_pr[c];
    const T rp = pr[0] != (T)0 ? calu_rcp(pr[0]) : (T)0;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      if (live[i]) {
        const T l = a[i][0] * rp;
#pragma unroll
        for (int c = 1; c < kLeaf; ++c) a[i][c - 1] = a[i][c] - l * pr[c];
        a[i][kLeaf - 1] = l;
      }
    }
  }
  __syncthreads();
}

// one polling thread per flag: threads t < n wait for flags[t] == tag (bounded by limit polls)
__device__ __forceinline__ void calu_wait(const int* flags, int n, int tag, GridSync* gs, int* s_fail,
                                          long long limit = kSpinLimit) {
  if ((int)threadIdx.x < n) {
    long long it = 0;
    while (ld_acquire_s32(flags + threadIdx.x) != tag) {
      if (++it > limit || *reinterpret_cast<volatile int*>(&gs->err) != 0) {
        atomicExch(&gs->err, 1);
        *s_fail = 1;
        break;
      }
    }
  }
  __syncthreads();
}

template <typename T, int R>
__global__ void __launch_bounds__(kPanelThreads, 1) k_panel(T* __restrict__ P, int64_t lda, int m, int nb, int rows_per,
                                                         int F, CaluBufs<T> cb, int tag, int* __restrict__ ipiv,
                                                         int kglob, int* __restrict__ info, GridSync* gs) {
  __shared__ T s_top[kLeaf * kLdS];                // pivot rows of the current elimination
  __shared__ __align__(16) T s_pr[kLeaf * kLeaf];  // rotated pivot row; in step 4 the rotated rows of U11
  __shared__ __align__(16) unsigned s_key[kPanelThreads / 32];
  __shared__ int s_sel[kLeaf];
  __shared__ int s_meta[kMetaLen];
  __shared__ int s_work[3 * kLeaf];
  __shared__ T s_rinv[kLeaf];
  __shared__ int s_fail;
  const int cta = blockIdx.x, ncta = gridDim.x, tid = threadIdx.x;
  const int G = (ncta + F - 1) / F;
  const int r0 = cta * rows_per;
  const int nr = max(0, min(rows_per, m - r0));
  int* f0 = cb.flags;
  int* f1 = cb.flags + kCaluMaxCta;
  int* fb = cb.flags + 2 * kCaluMaxCta;
  if (tid == 0) s_fail = 0;
  T a[R][kLeaf];
  bool live[R];
  // ---- 1. local elimination of this CTA's rows
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int q = tid + kPanelThreads * i;
    live[i] = q < nr;
#pragma unroll
    for (int c = 0; c < kLeaf; ++c) a[i][c] = (live[i] && c < nb) ? P[(int64_t)c * lda + r0 + q] : (T)0;
  }
  const int kl = min(nr, nb);
  calu_elim<T, R>(a, live, kl, s_top, s_pr, s_sel, s_key);
  {
    T* cv = cb.cand + (size_t)cta * kLeaf * kLeaf;
    for (int idx = tid; idx < kLeaf * nb; idx += kPanelThreads) {
      const int i = idx / nb, c = idx % nb;
      if (i < kl) cv[i * kLeaf + c] = P[(int64_t)c * lda + r0 + s_sel[i]];
    }
    if (tid < kLeaf) cb.cidx[cta * kLeaf + tid] = tid < kl ? r0 + s_sel[tid] : -1;
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release_s32(f0 + cta, tag);
  }
  // ---- 2. group leaders: nb winners among the members' candidates
  if (cta % F == 0) {
    const int g = cta / F, gsz = min(F, ncta - cta);
    calu_wait(f0 + cta, gsz, tag, gs, &s_fail);
    if (s_fail) return;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int q = tid + kPanelThreads * i;
      const int slot = cta * kLeaf + q;  // member cta + q / kLeaf, candidate q % kLeaf
      live[i] = q < gsz * kLeaf && __ldcg(cb.cidx + slot) >= 0;
#pragma unroll
      for (int c = 0; c < kLeaf; ++c) a[i][c] = (live[i] && c < nb) ? __ldcg(cb.cand + (size_t)slot * kLeaf + c) : (T)0;
    }
    calu_elim<T, R>(a, live, nb, s_top, s_pr, s_sel, s_key);
    T* lv = cb.lcand + (size_t)g * kLeaf * kLeaf;
    // the nb winners only: s_sel[j] for j >= nb is not set by this elimination (ragged
    // last panel, nb < kLeaf)
    for (int idx = tid; idx < nb * nb; idx += kPanelThreads) {
      const int j = idx / nb, c = idx % nb;
      const int q = s_sel[j];
      if (q >= 0) lv[j * kLeaf + c] = __ldcg(cb.cand + (size_t)(cta * kLeaf + q) * kLeaf + c);
    }
    if (tid < kLeaf) {
      const int q = tid < nb ? s_sel[tid] : -1;
      cb.lidx[g * kLeaf + tid] = q >= 0 ? __ldcg(cb.cidx + cta * kLeaf + q) : -1;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release_s32(f1 + g, tag);
  }
  // ---- 3. root: the nb pivots, the factored top block and the row exchanges
  if (cta == 0) {
    calu_wait(f1, G, tag, gs, &s_fail);
    if (s_fail) return;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int q = tid + kPanelThreads * i;
      live[i] = q < G * kLeaf && __ldcg(cb.lidx + q) >= 0;
#pragma unroll
      for (int c = 0; c < kLeaf; ++c) a[i][c] = (live[i] && c < nb) ? __ldcg(cb.lcand + (size_t)q * kLeaf + c) : (T)0;
    }
    calu_elim<T, R>(a, live, nb, s_top, s_pr, s_sel, s_key);
    for (int idx = tid; idx < nb * nb; idx += kPanelThreads) {
      const int j = idx / nb, c = idx % nb;
      cb.top[j * kLeaf + c] = s_top[j * kLdS + c];
      cb.orig[j * kLeaf + c] = P[(int64_t)c * lda + j];
    }
    if (tid == 0) {
      // pivot order -> sequential row exchanges; track where the original top rows go
      int* loc = s_work;  // shared scratch: thread 0 only
      int* content = s_work + kLeaf;
      int* slot = s_work + 2 * kLeaf;
      for (int s = 0; s < nb; ++s) { loc[s] = s; content[s] = s; slot[s] = -1; }
      int nd = 0;
      for (int j = 0; j < nb; ++j) {
        const int w = __ldcg(cb.lidx + s_sel[j]);
        if (s_top[j * kLdS + j] == (T)0 && *info == 0) *info = kglob + j + 1;
        const int p = w < nb ? loc[w] : w;
        s_meta[j] = p;
        s_meta[3 * kLeaf + 1 + j] = w;
        const int c = content[j];
        if (p != j) {
          if (p < nb) {
            content[p] = c;
            loc[c] = p;
          } else {
            const int sl = w >= nb ? nd++ : slot[w];
            s_meta[kLeaf + sl] = p;
            s_meta[2 * kLeaf + sl] = c;
            slot[c] = sl;
            loc[c] = p;
          }
          content[j] = w;
          if (w < nb) loc[w] = j;
        }
        ipiv[j] = kglob + p;
      }
      s_meta[3 * kLeaf] = nd;
    }
    __syncthreads();
    for (int i = tid; i < kMetaLen; i += kPanelThreads) cb.meta[i] = s_meta[i];
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release_s32(fb, tag);
  }
  // ---- 4. every CTA: its rows of the factored panel
  calu_wait(fb, 1, tag, gs, &s_fail);
  if (s_fail) return;
  for (int idx = tid; idx < kLeaf * kLeaf; idx += kPanelThreads) {
    const int i = idx / kLeaf, c = idx % kLeaf;  // s_pr[i][c] = U11[i][i + c], zero past the block
    s_pr[idx] = (i < nb && i + c < nb) ? __ldcg(cb.top + i * kLeaf + i + c) : (T)0;
  }
  if (tid < kMetaLen) s_meta[tid] = __ldcg(cb.meta + tid);
  if (tid < nb) {
    const T u = __ldcg(cb.top + tid * kLeaf + tid);
    s_rinv[tid] = u != (T)0 ? calu_rcp(u) : (T)0;
  }
  __syncthreads();
  const int nd = s_meta[3 * kLeaf];
  for (int rr = tid; rr < nr; rr += kPanelThreads) {
    const int r = r0 + rr;
    if (r < nb) {
#pragma unroll
      for (int c = 0; c < kLeaf; ++c)
        if (c < nb) P[(int64_t)c * lda + r] = __ldcg(cb.top + r * kLeaf + c);
      continue;
    }
    int src = -1;
    for (int t = 0; t < nd; ++t)
      if (s_meta[kLeaf + t] == r) src = s_meta[2 * kLeaf + t];
    T x[kLeaf];
#pragma unroll
    for (int c = 0; c < kLeaf; ++c)
      x[c] = c < nb ? (src < 0 ? P[(int64_t)c * lda + r] : __ldcg(cb.orig + src * kLeaf + c)) : (T)0;
    // x U11 = original row, right-looking with the same rotation as the elimination:
    // before step kk, x[c] holds column (c + kk) mod kLeaf; the solved value enters at the end
#pragma unroll 1
    for (int kk = 0; kk < nb; ++kk) {
      const T xk = x[0] * s_rinv[kk];
      const T* ur = s_pr + kk * kLeaf;  // U11[kk][kk + c], zero past the block
#pragma unroll
      for (int c = 1; c < kLeaf; ++c) x[c - 1] = x[c] - xk * ur[c];
      x[kLeaf - 1] = xk;
    }
    // after nb steps column c sits in x[(c - nb) mod kLeaf]
#pragma unroll
    for (int c = 0; c < kLeaf; ++c) {
      const int col = (c + nb) & (kLeaf - 1);
      if (col < nb) P[(int64_t)col * lda + r] = x[c];
    }
  }
}

constexpr size_t calu_a256(size_t v) { return (v + 255) / 256 * 256; }
// bytes of the panel kernel's buffers for up to ncta CTAs
template <typename T>
constexpr size_t calu_bytes(int ncta) {
  return 2 * calu_a256(sizeof(T) * (size_t)ncta * kLeaf * kLeaf) + 2 * calu_a256(sizeof(int) * (size_t)ncta * kLeaf) +
         2 * calu_a256(sizeof(T) * kLeaf * kLeaf) + calu_a256(sizeof(int) * kMetaLen) +
         calu_a256(sizeof(int) * (2 * kCaluMaxCta + 1));
}
template <typename T>
CaluBufs<T> calu_carve(unsigned char* base, int ncta) {
  CaluBufs<T> b;
  size_t o = 0;
  auto take = [&](size_t bytes) { unsigned char* q = base + o; o += calu_a256(bytes); return q; };
  b.cand = reinterpret_cast<T*>(take(sizeof(T) * (size_t)ncta * kLeaf * kLeaf));
  b.lcand = reinterpret_cast<T*>(take(sizeof(T) * (size_t)ncta * kLeaf * kLeaf));
  b.cidx = reinterpret_cast<int*>(take(sizeof(int) * (size_t)ncta * kLeaf));
  b.lidx = reinterpret_cast<int*>(take(sizeof(int) * (size_t)ncta * kLeaf));
  b.top = reinterpret_cast<T*>(take(sizeof(T) * kLeaf * kLeaf));
  b.orig = reinterpret_cast<T*>(take(sizeof(T) * kLeaf * kLeaf));
  b.meta = reinterpret_cast<int*>(take(sizeof(int) * kMetaLen));
  b.flags = reinterpret_cast<int*>(take(sizeof(int) * (2 * kCaluMaxCta + 1)));
  return b;
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

// Same solve with the triangle size fixed at compile time: 128 columns per CTA are staged
// through shared memory with coalesced loads and stores, each thread solves one column in
// registers with fully unrolled loops.
constexpr int kTrsmCols = 128;
template <typename T, int NB>
__global__ void __launch_bounds__(kTrsmCols) k_trsm_small_fixed(const T* __restrict__ L, int64_t ldl,
                                                                T* __restrict__ B, int64_t ldb, int64_t n2) {
  extern __shared__ __align__(16) unsigned char trsm_smem[];
  T* sL = reinterpret_cast<T*>(trsm_smem);   // [i][k] = L(k, i) for k > i
  T* sB = sL + NB * NB;                      // [r][cc], stride kTrsmCols + 1
  const int64_t c0 = blockIdx.x * (int64_t)kTrsmCols;
  for (int idx = threadIdx.x; idx < NB * NB; idx += kTrsmCols) {
    const int k = idx % NB, i = idx / NB;
    sL[i * NB + k] = L[(int64_t)i * ldl + k];
  }
  // loads in batches of 16 per thread, each batch issued before its shared-memory stores
#pragma unroll 1
  for (int q0 = 0; q0 < NB; q0 += 16) {
    T v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int idx = threadIdx.x + (q0 + q) * kTrsmCols, r = idx % NB, cc = idx / NB;
      v[q] = c0 + cc < n2 ? B[(c0 + cc) * ldb + r] : (T)0;
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int idx = threadIdx.x + (q0 + q) * kTrsmCols, r = idx % NB, cc = idx / NB;
      sB[r * (kTrsmCols + 1) + cc] = v[q];
    }
  }
  __syncthreads();
  T x[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) x[i] = sB[i * (kTrsmCols + 1) + threadIdx.x];
#pragma unroll
  for (int i = 0; i < NB; ++i)
#pragma unroll
    for (int k = i + 1; k < NB; ++k) x[k] -= sL[i * NB + k] * x[i];
#pragma unroll
  for (int i = 0; i < NB; ++i) sB[i * (kTrsmCols + 1) + threadIdx.x] = x[i];
  __syncthreads();
#pragma unroll 4
  for (int q = 0; q < NB; ++q) {
    const int idx = threadIdx.x + q * kTrsmCols, r = idx % NB, cc = idx / NB;
    if (c0 + cc < n2) B[(c0 + cc) * ldb + r] = sB[r * (kTrsmCols + 1) + cc];
  }
}
template <typename T, int NB>
constexpr size_t trsm_fixed_smem() {
  return sizeof(T) * (NB * NB + NB * (kTrsmCols + 1));
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
  // all sixteen loads of C before any store: independent, so they overlap
  T cv[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int64_t gi = i0 + tx + 16 * a, gj = j0 + ty + 16 * b;
      cv[a][b] = (gi < m && gj < n) ? C[gj * ldc + gi] : (T)0;
    }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int64_t gi = i0 + tx + 16 * a, gj = j0 + ty + 16 * b;
      if (gi < m && gj < n) C[gj * ldc + gi] = cv[a][b] - acc[a][b];
    }
}

// Small-k variant (k <= kSmallK): the whole A (64 x k) and B (k x 64) panels are staged in
// shared memory with one barrier, instead of k / 16 load-barrier-compute rounds; this is
// the shape of every SIMT update in the recursive factorisation (k = 32 .. 96).
constexpr int kSmallK = 128;
template <typename T>
__global__ void __launch_bounds__(256) k_gemm_sub_smallk(int64_t m, int64_t n, int k, const T* __restrict__ A,
                                                         int64_t lda, const T* __restrict__ B, int64_t ldb,
                                                         T* __restrict__ C, int64_t ldc) {
  extern __shared__ __align__(16) unsigned char gs_smem[];
  T* sA = reinterpret_cast<T*>(gs_smem);  // [kk][r], stride 65
  T* sB = sA + kSmallK * 65;              // [kk][c], stride 65
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int64_t i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
#pragma unroll 8
  for (int idx = threadIdx.x; idx < 64 * k; idx += 256) {
    const int r = idx % 64, kk = idx / 64;
    const int64_t gi = i0 + r;
    sA[kk * 65 + r] = gi < m ? A[kk * lda + gi] : (T)0;
    const int rk = idx % k, cj = idx / k;
    const int64_t gj = j0 + cj;
    sB[rk * 65 + cj] = gj < n ? B[gj * ldb + rk] : (T)0;
  }
  __syncthreads();
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0;
#pragma unroll 4
  for (int t = 0; t < k; ++t) {
    T av[4], bv[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) av[a] = sA[t * 65 + tx + 16 * a];
#pragma unroll
    for (int b = 0; b < 4; ++b) bv[b] = sB[t * 65 + ty + 16 * b];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] += av[a] * bv[b];
  }
  T cv[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int64_t gi = i0 + tx + 16 * a, gj = j0 + ty + 16 * b;
      cv[a][b] = (gi < m && gj < n) ? C[gj * ldc + gi] : (T)0;
    }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int64_t gi = i0 + tx + 16 * a, gj = j0 + ty + 16 * b;
      if (gi < m && gj < n) C[gj * ldc + gi] = cv[a][b] - acc[a][b];
    }
}
template <typename T>
constexpr size_t gemm_smallk_smem() {
  return sizeof(T) * 2 * kSmallK * 65;
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

// partial row sums of |A_ij| c_j over a column chunk (finished by k_scale_rows_of_parts)
__global__ void k_abs_rowsum_part(int64_t n, const double* __restrict__ A, int64_t lda, const double* __restrict__ c,
                                  int64_t chunk, double* __restrict__ part) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
  if (i >= n) return;
  double s = 0;
  for (int64_t j = j0; j < j1; ++j) s += fabs(A[j * lda + i]) * c[j];
  part[blockIdx.y * n + i] = s;
}

// Column-chunk reductions over a column-major matrix with 16-byte loads: thread t covers the
// kV = 16 / sizeof(T) consecutive rows kV t .. kV t + kV - 1, eight columns per iteration,
// FP64 accumulation; grid.y = chunk.  MODE 0: part = sum_j A_ij x_j; 1: part = max_j |A_ij|
// (x unused); 2: part = sum_j |A_ij| x_j.  The caller checks that A is 16-byte aligned and
// lda a multiple of kV; rows past a partial last vector are read one by one.
template <typename T>
__device__ __forceinline__ double vget(const float4& a, int v) {
  return v == 0 ? a.x : v == 1 ? a.y : v == 2 ? a.z : a.w;
}
template <typename T>
__device__ __forceinline__ double vget(const double2& a, int v) {
  return v == 0 ? a.x : a.y;
}
template <int MODE>
__device__ __forceinline__ void vacc(double& s, double a, double x) {
  if (MODE == 0) {
    s += a * x;
  } else if (MODE == 1) {  // max |a| on the bit patterns: integer instructions, not the FP64 pipe
    const long long m = max(__double_as_longlong(s), __double_as_longlong(a) & 0x7fffffffffffffffLL);
    s = __longlong_as_double(m);
  } else {
    s += fabs(a) * x;
  }
}
template <typename T, int MODE>
__global__ void __launch_bounds__(256) k_colreduce_v(int64_t n, const T* __restrict__ A, int64_t lda,
                                                     const double* __restrict__ x, int64_t chunk,
                                                     double* __restrict__ part) {
  constexpr int kV = 16 / sizeof(T);
  using VT = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  const int64_t i0 = kV * (blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
  if (i0 >= n) return;
  const int64_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
  double s[kV];
#pragma unroll
  for (int v = 0; v < kV; ++v) s[v] = 0.0;
  if (i0 + kV <= n) {
    int64_t j = j0;
    for (; j + 7 < j1; j += 8) {
      VT a[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) a[u] = *reinterpret_cast<const VT*>(A + (j + u) * lda + i0);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const double xv = MODE == 1 ? 0.0 : x[j + u];
#pragma unroll
        for (int v = 0; v < kV; ++v) vacc<MODE>(s[v], vget<T>(a[u], v), xv);
      }
    }
    for (; j < j1; ++j) {
      const VT a = *reinterpret_cast<const VT*>(A + j * lda + i0);
      const double xv = MODE == 1 ? 0.0 : x[j];
#pragma unroll
      for (int v = 0; v < kV; ++v) vacc<MODE>(s[v], vget<T>(a, v), xv);
    }
  } else {
#pragma unroll
    for (int v = 0; v < kV; ++v)
      if (i0 + v < n)
        for (int64_t j = j0; j < j1; ++j) vacc<MODE>(s[v], (double)A[j * lda + i0 + v], MODE == 1 ? 0.0 : x[j]);
  }
#pragma unroll
  for (int v = 0; v < kV; ++v)
    if (i0 + v < n) part[blockIdx.y * n + i0 + v] = s[v];
}

// ---------------------------------------------------------------- triangular solves
// Substitution with the factors in precision T (vectors FP64), blocks of kTrsvB rows.
// After the factorisation, k_trsv_inv writes the inverse of every diagonal block of L
// (unit lower) and U (upper) to dinv.  One cooperative launch of k_trsv_persist then solves
// the whole triangle: CTA c takes blocks c, c + G, c + 2G, ... in dependency order and,
// for block i, accumulates F_ij x_j over the solved blocks j (waiting on flags[j] == tag,
// bounded), forms r_i = rhs_i - sum, applies the inverse diagonal block (x_i = D_i^-1 r_i),
// stores x_i and releases flags[i] = tag.  Tags grow by one per launch, so the flags are
// never cleared.  Deadlock-free because all CTAs are co-resident and every CTA meets its
// blocks in increasing dependency order.
constexpr int kTrsvB = 128;
constexpr int kTrsvThreads = 256;   // 8 warps: warp w covers columns 16w..16w+15 of a tile

// inverse of the diagonal block blockIdx.x of L (blockIdx.y = 0, unit lower) or U (= 1),
// column-major kTrsvB x kTrsvB with explicit zeros; rows/columns past N are identity
template <typename T>
__global__ void __launch_bounds__(kTrsvB) k_trsv_inv(const T* __restrict__ F, int64_t ldf, int64_t N,
                                                     T* __restrict__ dinv) {
  extern __shared__ unsigned char inv_smem[];
  T* X = reinterpret_cast<T*>(inv_smem);          // X[c * (kTrsvB + 1) + r]
  T* tcol = X + kTrsvB * (kTrsvB + 1);            // kTrsvB scratch
  const int blk = blockIdx.x, upper = blockIdx.y;
  const int64_t k0 = (int64_t)blk * kTrsvB;
  const int nb = (int)(N - k0 < kTrsvB ? N - k0 : kTrsvB);
  const int r = threadIdx.x;
  for (int c = 0; c < kTrsvB; ++c) {
    T v;
    if (r < nb && c < nb) v = F[(k0 + c) * ldf + k0 + r];
    else v = (r == c) ? (T)1 : (T)0;
    if (!upper && r <= c) v = (r == c) ? (T)1 : (T)0;   // unit lower: ignore U's part
    if (upper && r > c) v = 0;                           // upper: ignore L's part
    X[c * (kTrsvB + 1) + r] = v;
  }
  __syncthreads();
  if (!upper) {
    // right to left: X[r][j] = -(L[r][j] + sum_{j<k<r} X[r][k] L[k][j]),  r > j
    for (int j = kTrsvB - 2; j >= 0; --j) {
      T t = 0;
      if (r > j) {
        t = X[j * (kTrsvB + 1) + r];
        for (int k = j + 1; k < r; ++k) t += X[k * (kTrsvB + 1) + r] * X[j * (kTrsvB + 1) + k];
      }
      __syncthreads();
      if (r > j) X[j * (kTrsvB + 1) + r] = -t;
      __syncthreads();
    }
  } else {
    // left to right: X[j][j] = 1 / U[j][j];  X[r][j] = -X[j][j] sum_{r<=k<j} X[r][k] U[k][j],  r < j
    for (int j = 0; j < kTrsvB; ++j) {
      const T djj = (T)1 / X[j * (kTrsvB + 1) + j];
      T t = 0;
      if (r < j)
        for (int k = r; k < j; ++k) t += X[k * (kTrsvB + 1) + r] * X[j * (kTrsvB + 1) + k];
      tcol[r] = t;
      __syncthreads();
      if (r < j) X[j * (kTrsvB + 1) + r] = -djj * tcol[r];
      if (r == j) X[j * (kTrsvB + 1) + j] = djj;
      __syncthreads();
    }
  }
  T* out = dinv + (size_t)(2 * blk + upper) * kTrsvB * kTrsvB;
  for (int c = 0; c < kTrsvB; ++c) out[c * kTrsvB + r] = X[c * (kTrsvB + 1) + r];
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// rows 4 * lane .. 4 * lane + 3 of column c of a tile starting at row i0 (nbi valid rows)
template <typename T, bool VEC>
__device__ __forceinline__ void trsv_load4(const T* col, int lane, int nbi, T v[4]) {
  const int r = 4 * lane;
  if (VEC && r + 3 < nbi) {
    if (sizeof(T) == 4) {
      const float4 q = __ldg(reinterpret_cast<const float4*>(col + r));
      v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
      const double2 q0 = __ldg(reinterpret_cast<const double2*>(col + r));
      const double2 q1 = __ldg(reinterpret_cast<const double2*>(col + r + 2));
      v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
    }
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = (r + q < nbi) ? col[r + q] : (T)0;
  }
}

template <typename T, bool LOWER, bool VEC>
__global__ void __launch_bounds__(kTrsvThreads) k_trsv_persist(const T* __restrict__ F, int64_t ldf, int64_t N,
                                                               int nblk, const T* __restrict__ dinv,
                                                               const double* __restrict__ rhs, double* x,
                                                               int* flags, int tag, GridSync* gs) {
  extern __shared__ __align__(16) unsigned char ps_smem[];
  T* sD = reinterpret_cast<T*>(ps_smem);                 // inverse diagonal block, kTrsvB^2
  T* s_red = sD + kTrsvB * kTrsvB;                       // [8][kTrsvB] partial sums
  __shared__ T s_x[kTrsvB];
  __shared__ T s_r[kTrsvB];
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) s_fail = 0;
  for (int t = blockIdx.x; t < nblk; t += gridDim.x) {
    const int bi = LOWER ? t : nblk - 1 - t;
    const int64_t i0 = (int64_t)bi * kTrsvB;
    const int nbi = (int)(N - i0 < kTrsvB ? N - i0 : kTrsvB);
    // stage D_i^-1 in shared memory while the tiles stream
    {
      const char* g = reinterpret_cast<const char*>(dinv + (size_t)(2 * bi + (LOWER ? 0 : 1)) * kTrsvB * kTrsvB);
      char* sm = reinterpret_cast<char*>(sD);
      for (int o = tid * 16; o < (int)(sizeof(T) * kTrsvB * kTrsvB); o += kTrsvThreads * 16) cp_async16(sm + o, g + o);
    }
    T acc[4] = {0, 0, 0, 0};
    const int ntiles = LOWER ? bi : nblk - 1 - bi;
    for (int s = 0; s < ntiles; ++s) {
      const int bj = LOWER ? s : nblk - 1 - s;
      const int64_t j0 = (int64_t)bj * kTrsvB;
      const int nbj = (int)(N - j0 < kTrsvB ? N - j0 : kTrsvB);
      // the tile does not depend on x_j: issue its loads first
      T v[16][4];
#pragma unroll
      for (int cc = 0; cc < 16; ++cc) {
        const int c = warp * 16 + cc;
        if (c < nbj) trsv_load4<T, VEC>(F + (j0 + c) * ldf + i0, lane, nbi, v[cc]);
        else v[cc][0] = v[cc][1] = v[cc][2] = v[cc][3] = 0;
      }
      if (tid == 0) {
        long long it = 0;
        while (ld_acquire_s32(flags + bj) != tag) {
          if (++it > kSpinLimit || *reinterpret_cast<volatile int*>(&gs->err) != 0) {
            atomicExch(&gs->err, 1);
            s_fail = 1;
            break;
          }
        }
      }
      __syncthreads();
      if (s_fail) { cp_async_wait_all(); return; }
      if (tid < kTrsvB) s_x[tid] = tid < nbj ? (T)__ldcg(x + j0 + tid) : (T)0;
      __syncthreads();
#pragma unroll
      for (int cc = 0; cc < 16; ++cc) {
        const T xc = s_x[warp * 16 + cc];
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] += v[cc][q] * xc;
      }
    }
    // r_i = rhs_i - sum over the eight warps
#pragma unroll
    for (int q = 0; q < 4; ++q) s_red[warp * kTrsvB + 4 * lane + q] = acc[q];
    cp_async_wait_all();
    __syncthreads();
    if (tid < kTrsvB) {
      T sum = 0;
#pragma unroll
      for (int w = 0; w < kTrsvThreads / 32; ++w) sum += s_red[w * kTrsvB + tid];
      s_r[tid] = tid < nbi ? (T)rhs[i0 + tid] - sum : (T)0;
    }
    __syncthreads();
    // x_i = D_i^-1 r_i
    T acc2[4] = {0, 0, 0, 0};
#pragma unroll
    for (int cc = 0; cc < 16; ++cc) {
      const int c = warp * 16 + cc;
      const T rc = s_r[c];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc2[q] += sD[c * kTrsvB + 4 * lane + q] * rc;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) s_red[warp * kTrsvB + 4 * lane + q] = acc2[q];
    __syncthreads();
    if (tid < nbi) {
      T sum = 0;
#pragma unroll
      for (int w = 0; w < kTrsvThreads / 32; ++w) sum += s_red[w * kTrsvB + tid];
      x[i0 + tid] = (double)sum;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release_s32(flags + bi, tag);
  }
}

template <typename T>
size_t trsv_persist_smem() {
  return sizeof(T) * kTrsvB * kTrsvB + sizeof(T) * 8 * kTrsvB;
}

template <typename T>
cudaError_t set_solver_smem_attrs() {
  cudaError_t e = cudaFuncSetAttribute((const void*)k_trsm_small<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(2 * 64 * 65 * sizeof(T)));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k_gemm_sub_smallk<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)gemm_smallk_smem<T>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k_trsm_small_fixed<T, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)trsm_fixed_smem<T, 32>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k_trsm_small_fixed<T, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)trsm_fixed_smem<T, 64>());
  const int inv = (int)(sizeof(T) * (kTrsvB * (kTrsvB + 1) + kTrsvB));
  const int ps = (int)trsv_persist_smem<T>();
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k_trsv_inv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, inv);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k_trsv_persist<T, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k_trsv_persist<T, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k_trsv_persist<T, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k_trsv_persist<T, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, ps);
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
  CaluBufs<T> cb{};          // buffers of the panel kernel (one allocation at cb_mem)
  void* cb_mem = nullptr;
  int* ipiv_dev = nullptr;  // N entries (global, absolute row of each exchange)
  int* perm = nullptr;      // N entries: row i of P A is row perm[i] of A
  double* tmp = nullptr;    // N-vector scratch of lu_apply
  int* info = nullptr;
  GridSync* gs = nullptr;
  int ncta = 0;
  T* dinv = nullptr;         // inverses of the diagonal blocks of L and U, [nblk][2][kTrsvB^2]
  int* tflags = nullptr;     // per-block release flags of the triangular solves
  int ttag = 0;              // tag of the last triangular-solve launch
  int trsv_grid = 0;         // co-resident CTAs of the persistent triangular solve
  void* gemm_ws = nullptr;   // BF16 split workspace of the tensor-core GEMM (FP32 LU only)
  size_t gemm_ws_bytes = 0;
  int* gemm_err = nullptr;   // raised by the tensor-core GEMM's bounded waits
};

template <typename T>
static ibem_status panel(T* A, int64_t lda, int64_t k0, int64_t m, int nb, LuWork<T>& w, cudaStream_t st) {
  // CTAs: at most one per SM, at least kCaluMinRows rows each; the tree's fan-in F ~ sqrt
  int ncta = (int)std::max<int64_t>(1, std::min<int64_t>(w.ncta, (m + kCaluMinRows - 1) / kCaluMinRows));
  int rows_per = (int)((m + ncta - 1) / ncta);
  ncta = (int)((m + rows_per - 1) / rows_per);
  int F = 1;
  while (F * F < ncta) ++F;
  const int G = (ncta + F - 1) / F;
  // rows of the largest elimination (own rows, a group's or the root's candidates)
  const int rows = std::max(rows_per, std::max(F, G) * kLeaf);
  if (rows > kPanelThreads * kPanelRmax || ncta > kCaluMaxCta)
    return fail(IBEM_ERR_ARG, "panel too tall for the panel kernel");
  const void* fn = rows <= kPanelThreads       ? (const void*)k_panel<T, 1>
                   : rows <= 2 * kPanelThreads ? (const void*)k_panel<T, 2>
                                               : (const void*)k_panel<T, 4>;
  T* P = A + k0 * lda + k0;
  int mm = (int)m;
  int* ip = w.ipiv_dev + k0;
  int kg = (int)k0;
  int tag = (int)k0 + 1;   // unique within the factorisation; the flags start at zero
  void* args[] = {&P, &lda, &mm, &nb, &rows_per, &F, &w.cb, &tag, &ip, &kg, &w.info, &w.gs};
  ProfScope ps(PROF_PANEL, st);
  count_launch();
  IBEM_CUDA(cudaLaunchCooperativeKernel(fn, dim3(ncta), dim3(kPanelThreads), args, 0, st));
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
  if (k <= kSmallK)
    ::ibem::count_launch(), k_gemm_sub_smallk<double><<<grid, 256, gemm_smallk_smem<double>(), st>>>(m, n, (int)k, A, lda, B,
                                                                                         ldb, C, ldc);
  else
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
  if (k <= kSmallK)
    ::ibem::count_launch(), k_gemm_sub_smallk<float><<<grid, 256, gemm_smallk_smem<float>(), st>>>(m, n, (int)k, A, lda, B,
                                                                                         ldb, C, ldc);
  else
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
      ::ibem::count_launch(), k_trsm_small_fixed<T, 32><<<(unsigned)((n2 + kTrsmCols - 1) / kTrsmCols), kTrsmCols,
                                                          trsm_fixed_smem<T, 32>(), st>>>(L, ldl, B, ldb, n2);
    else if (n1 == 64 && sizeof(T) == sizeof(float))
      ::ibem::count_launch(), k_trsm_small_fixed<T, 64><<<(unsigned)((n2 + kTrsmCols - 1) / kTrsmCols), kTrsmCols,
                                                          trsm_fixed_smem<T, 64>(), st>>>(L, ldl, B, ldb, n2);
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
  int dev = 0, nsm = 0;
  IBEM_CUDA(cudaGetDevice(&dev));
  IBEM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  IBEM_CUDA(set_solver_smem_attrs<T>());
  int per_sm = 0;
  IBEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_panel<T, kPanelRmax>, kPanelThreads, 0));
  if (per_sm < 1) return fail(IBEM_ERR_CUDA, "panel kernel cannot be resident");
  w.ncta = std::min(nsm, kCaluMaxCta);  // at most one CTA per SM (co-resident for the cooperative launch)
  if ((int64_t)w.ncta * kPanelThreads * kPanelRmax < N) return fail(IBEM_ERR_ARG, "matrix too large for the panel kernel");
  IBEM_CUDA(cudaMalloc(&w.cb_mem, calu_bytes<T>(w.ncta)));
  IBEM_CUDA(cudaMemset(w.cb_mem, 0, calu_bytes<T>(w.ncta)));
  w.cb = calu_carve<T>(static_cast<unsigned char*>(w.cb_mem), w.ncta);
  IBEM_CUDA(cudaMalloc(&w.ipiv_dev, sizeof(int) * (size_t)N));
  IBEM_CUDA(cudaMalloc(&w.perm, sizeof(int) * (size_t)N));
  IBEM_CUDA(cudaMalloc(&w.tmp, sizeof(double) * (size_t)N));
  IBEM_CUDA(cudaMalloc(&w.info, sizeof(int)));
  IBEM_CUDA(cudaMalloc(&w.gs, sizeof(GridSync)));
  {
    const int64_t nblk = (N + kTrsvB - 1) / kTrsvB;
    IBEM_CUDA(cudaMalloc(&w.dinv, sizeof(T) * 2 * (size_t)nblk * kTrsvB * kTrsvB));
    IBEM_CUDA(cudaMalloc(&w.tflags, sizeof(int) * (size_t)nblk));
    IBEM_CUDA(cudaMemset(w.tflags, 0, sizeof(int) * (size_t)nblk));
    int per = 0;
    IBEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_trsv_persist<T, true, true>, kTrsvThreads,
                                                            trsv_persist_smem<T>()));
    if (per < 1) return fail(IBEM_ERR_CUDA, "triangular-solve kernel cannot be resident");
    w.trsv_grid = per * nsm;
  }
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
  cudaFree(w.cb_mem);
  cudaFree(w.ipiv_dev);
  cudaFree(w.perm);
  cudaFree(w.tmp);
  cudaFree(w.info);
  cudaFree(w.gs);
  cudaFree(w.dinv);
  cudaFree(w.tflags);
  cudaFree(w.gemm_ws);
  cudaFree(w.gemm_err);
  w = LuWork<T>();
}

// Inverses of the diagonal blocks of the factors (after the factorisation, before any solve)
template <typename T>
static ibem_status trsv_prepare(const T* F, int64_t ldf, int64_t N, LuWork<T>& w, cudaStream_t st) {
  const unsigned nblk = (unsigned)((N + kTrsvB - 1) / kTrsvB);
  ProfScope ps(PROF_TRSV, st);
  const size_t smem = sizeof(T) * (kTrsvB * (kTrsvB + 1) + kTrsvB);
  ::ibem::count_launch(), k_trsv_inv<T><<<dim3(nblk, 2), kTrsvB, smem, st>>>(F, ldf, N, w.dinv);
  IBEM_LAUNCH_CHECK("trsv_prepare");
  return IBEM_OK;
}

template <typename T, bool LOWER>
static ibem_status trsv_launch(const T* F, int64_t ldf, int64_t N, LuWork<T>& w, const double* rhs, double* xo,
                               cudaStream_t st) {
  int nblk = (int)((N + kTrsvB - 1) / kTrsvB);
  const bool vec = (ldf % (int64_t)(16 / sizeof(T)) == 0) && (reinterpret_cast<uintptr_t>(F) % 16 == 0);
  const unsigned grid = (unsigned)std::min(nblk, w.trsv_grid);
  int tag = ++w.ttag;
  void* args[] = {&F, &ldf, &N, &nblk, &w.dinv, &rhs, &xo, &w.tflags, &tag, &w.gs};
  const void* fn = vec ? (const void*)k_trsv_persist<T, LOWER, true> : (const void*)k_trsv_persist<T, LOWER, false>;
  ::ibem::count_launch();
  IBEM_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kTrsvThreads), args, trsv_persist_smem<T>(), st));
  return IBEM_OK;
}

// Solve with the factors F (precision T): y <- U^-1 L^-1 P y (y FP64, in place; w.tmp N-vector).
// A wait that gave up sets the sticky flag w.gs->err, read by the caller (sticky_err).
template <typename T>
static ibem_status lu_apply(const T* F, int64_t ldf, int64_t N, LuWork<T>& w, double* y, cudaStream_t st) {
  ProfScope ps(PROF_TRSV, st, 2.0 * N * N);
  ::ibem::count_launch(), k_gather<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(N, w.perm, y, w.tmp);
  ibem_status s = trsv_launch<T, true>(F, ldf, N, w, w.tmp, y, st);    // forward: L z = P y
  if (!s) s = trsv_launch<T, false>(F, ldf, N, w, y, w.tmp, st);      // backward: U x = z
  if (s) return s;
  IBEM_CUDA(cudaMemcpyAsync(y, w.tmp, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
  IBEM_LAUNCH_CHECK("lu_apply");
  return IBEM_OK;
}

template <typename T>
static ibem_status sticky_err(const LuWork<T>& w, cudaStream_t st) {
  GridSync hgs{};
  IBEM_CUDA(cudaMemcpyAsync(&hgs, w.gs, sizeof(GridSync), cudaMemcpyDeviceToHost, st));
  IBEM_CUDA(cudaStreamSynchronize(st));
  if (hgs.err) return fail(IBEM_ERR_TIMEOUT, "a bounded wait of the panel or triangular-solve kernel gave up");
  return IBEM_OK;
}

// r = b - A x  (FP64)
// part (nparts x N) = column-chunk reductions of A (MODE as k_colreduce_v) with 16-byte
// loads when A and lda allow them, else one element per load (dot products only).
template <int MODE, typename T>
static ibem_status colreduce(int64_t N, const T* A, int64_t lda, const double* x, int nparts, double* part,
                             cudaStream_t st) {
  constexpr int kV = 16 / sizeof(T);
  const int64_t chunk = (N + nparts - 1) / nparts;
  if (reinterpret_cast<uintptr_t>(A) % 16 == 0 && lda % kV == 0) {
    const int64_t rows = (N + kV - 1) / kV;
    ::ibem::count_launch(), k_colreduce_v<T, MODE><<<dim3((unsigned)((rows + 255) / 256), (unsigned)nparts), 256, 0,
                                                    st>>>(N, A, lda, x, chunk, part);
  } else {
    static_assert(sizeof(T) == 8, "the one-element-per-load fallback reads FP64 matrices");
    const dim3 grid((unsigned)((N + 255) / 256), (unsigned)nparts);
    if constexpr (MODE == 0)
      ::ibem::count_launch(), k_gemv_part<<<grid, 256, 0, st>>>(N, A, lda, x, chunk, part);
    else if constexpr (MODE == 1)
      ::ibem::count_launch(), k_rowmax_part<<<grid, 256, 0, st>>>(N, A, lda, chunk, part);
    else
      ::ibem::count_launch(), k_abs_rowsum_part<<<grid, 256, 0, st>>>(N, A, lda, x, chunk, part);
  }
  IBEM_LAUNCH_CHECK("column reduction");
  return IBEM_OK;
}

static ibem_status residual(int64_t N, const double* A, int64_t lda, const double* x, const double* b, double* r,
                            double* part, int nparts, cudaStream_t st) {
  if (ibem_status q = colreduce<0>(N, A, lda, x, nparts, part, st)) return q;
  ::ibem::count_launch(), k_residual<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(N, nparts, part, b, r);
  IBEM_LAUNCH_CHECK("residual");
  return IBEM_OK;
}


// ------------------------------------------------------------------ device vectors
namespace {
__global__ void __launch_bounds__(256) k_dot_many(int64_t n, int nv, const double* __restrict__ V, int64_t ldv,
                                                  const double* __restrict__ w, double* __restrict__ out) {
  // out[j] += sum_i V[i,j] w[i]: grid-stride over rows, eight vectors per pass accumulated
  // in registers, warp shuffles, one shared-memory step and one atomic per block and vector
  __shared__ double red[8][8];  // [warp][vector]; 256 threads
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j0 = 0; j0 < nv; j0 += 8) {
    const int nj = min(8, nv - j0);
    double s[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) s[u] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      const double wi = w[i];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (u < nj) s[u] += V[(j0 + u) * ldv + i] * wi;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      double v = s[u];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][u] = v;
    }
    __syncthreads();
    if (threadIdx.x < nj) {
      double t = 0;
      for (int q = 0; q < 8; ++q) t += red[q][threadIdx.x];
      atomicAdd(out + j0 + threadIdx.x, t);
    }
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
  y[i] = (r ? r[i] : 1.0) * s;
}

// y-parts of the FP32 scaled matrix times an FP32 vector: float4 loads of four rows, eight
// columns per iteration summed in FP32, those partial sums added in FP64 (GB300 runs FP64 at
// a small fraction of its FP32 rate, so FP64 multiply-adds would bound this product).
// Requires ldw % 4 == 0 and W 16-byte aligned.
// ABS: row sums of |W| instead (x unused), for the norm of the backward error.
template <bool ABS>
__global__ void __launch_bounds__(256) k_gemv_f32acc(int64_t n, const float* __restrict__ W, int64_t ldw,
                                                     const float* __restrict__ x, int64_t chunk,
                                                     double* __restrict__ part) {
  const int64_t i0 = 4 * (blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
  if (i0 >= n) return;
  const int64_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  int64_t j = j0;
  for (; j + 7 < j1; j += 8) {
    float4 a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) a[u] = *reinterpret_cast<const float4*>(W + (j + u) * ldw + i0);
    float t0 = 0.f, t1 = 0.f, t2 = 0.f, t3 = 0.f;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      if (ABS) {
        t0 += fabsf(a[u].x), t1 += fabsf(a[u].y), t2 += fabsf(a[u].z), t3 += fabsf(a[u].w);
      } else {
        const float xv = x[j + u];
        t0 = fmaf(a[u].x, xv, t0);
        t1 = fmaf(a[u].y, xv, t1);
        t2 = fmaf(a[u].z, xv, t2);
        t3 = fmaf(a[u].w, xv, t3);
      }
    }
    s[0] += t0, s[1] += t1, s[2] += t2, s[3] += t3;
  }
  float t0 = 0.f, t1 = 0.f, t2 = 0.f, t3 = 0.f;
  for (; j < j1; ++j) {
    const float4 a = *reinterpret_cast<const float4*>(W + j * ldw + i0);
    if (ABS) {
      t0 += fabsf(a.x), t1 += fabsf(a.y), t2 += fabsf(a.z), t3 += fabsf(a.w);
    } else {
      const float xv = x[j];
      t0 = fmaf(a.x, xv, t0);
      t1 = fmaf(a.y, xv, t1);
      t2 = fmaf(a.z, xv, t2);
      t3 = fmaf(a.w, xv, t3);
    }
  }
  s[0] += t0, s[1] += t1, s[2] += t2, s[3] += t3;
#pragma unroll
  for (int v = 0; v < 4; ++v)
    if (i0 + v < n) part[blockIdx.y * n + i0 + v] = s[v];
}
__global__ void k_d2f(int64_t n, const double* __restrict__ x, float* __restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = (float)x[i];
}

// Inverse of diagonal block blockIdx.x (rows and columns g0 .. g0 + nb - 1, g0 = block *
// blockIdx.x, nb = min(block, n - g0)) of As = R A C: Gauss-Jordan elimination in place with
// partial pivoting, FP64 in dynamic shared memory (block x (block + 1) doubles, block <=
// kBjMax), written in FP32, column-major, to P + blockIdx.x * block^2.  A zero pivot raises
// *info (the block's first row + 1).
constexpr int kBjMax = 80;
constexpr int kBjThreads = 256;
constexpr int kBjApplyThreads = 96;   // >= kBjMax, whole warps
inline size_t bj_smem(int block) { return sizeof(double) * (size_t)block * (block + 1); }
__global__ void __launch_bounds__(kBjThreads) k_bj_invert(int64_t n, int block, const double* __restrict__ A,
                                                          int64_t lda, const double* __restrict__ r,
                                                          const double* __restrict__ c, float* __restrict__ P,
                                                          int* __restrict__ info) {
  extern __shared__ double bj_mem[];
  __shared__ double col[kBjMax];
  __shared__ int piv[kBjMax];
  __shared__ int sp;
  const int ld = block + 1;
  auto M = [&](int i) { return bj_mem + (size_t)i * ld; };   // row i
  const int64_t g0 = (int64_t)block * blockIdx.x;
  const int nb = (int)min((int64_t)block, n - g0);
  const int t = threadIdx.x;
  for (int e = t; e < nb * nb; e += kBjThreads) {
    const int i = e % nb, j = e / nb;
    M(i)[j] = r[g0 + i] * A[(g0 + j) * lda + g0 + i] * c[g0 + j];
  }
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    if (t < 32) {  // pivot: largest |M(i)[k]|, i >= k
      double best = -1.0;
      int bi = k;
      for (int i = k + t; i < nb; i += 32) {
        const double v = fabs(M(i)[k]);
        if (v > best) best = v, bi = i;
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, o);
        const int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) best = ob, bi = oi;
      }
      if (t == 0) sp = bi, piv[k] = bi;
    }
    __syncthreads();
    const int p = sp;
    if (p != k)
      for (int j = t; j < nb; j += kBjThreads) {
        const double v = M(k)[j];
        M(k)[j] = M(p)[j];
        M(p)[j] = v;
      }
    __syncthreads();
    const double d = M(k)[k];
    if (d == 0.0) {
      if (t == 0) atomicCAS(info, 0, (int)g0 + 1);
      return;
    }
    for (int i = t; i < nb; i += kBjThreads) col[i] = M(i)[k];
    __syncthreads();
    if (t == 0) M(k)[k] = 1.0;
    __syncthreads();
    for (int j = t; j < nb; j += kBjThreads) M(k)[j] /= d;
    __syncthreads();
    for (int e = t; e < nb * nb; e += kBjThreads) {
      const int i = e % nb, j = e / nb;
      if (i != k) M(i)[j] = (j == k ? 0.0 : M(i)[j]) - col[i] * M(k)[j];
    }
    __syncthreads();
  }
  // undo the row exchanges as column exchanges of the inverse, last first
  for (int k = nb - 1; k >= 0; --k) {
    const int p = piv[k];
    if (p != k)
      for (int i = t; i < nb; i += kBjThreads) {
        const double v = M(i)[k];
        M(i)[k] = M(i)[p];
        M(i)[p] = v;
      }
    __syncthreads();
  }
  float* out = P + (int64_t)blockIdx.x * block * block;
  for (int e = t; e < nb * nb; e += kBjThreads) out[e] = (float)M(e % nb)[e / nb];
}

// z = P v blockwise (one CTA per diagonal block, thread i = row i of the block)
__global__ void __launch_bounds__(kBjApplyThreads) k_bj_apply(int64_t n, int block, const float* __restrict__ P,
                                                     const double* __restrict__ v, double* __restrict__ z) {
  __shared__ double sv[kBjMax];
  const int64_t g0 = (int64_t)block * blockIdx.x;
  const int nb = (int)min((int64_t)block, n - g0);
  const int i = threadIdx.x;
  if (i < nb) sv[i] = v[g0 + i];
  __syncthreads();
  if (i >= nb) return;
  const float* Pb = P + (int64_t)blockIdx.x * block * block;
  double s = 0;
  for (int j = 0; j < nb; ++j) s += (double)Pb[j * nb + i] * sv[j];
  z[g0 + i] = s;
}
}  // namespace

// y = As v with As = R A C (FP64; tmp is N-vector scratch)
static ibem_status scaled_matvec(SolveCtx& cx, const double* A, int64_t lda, const double* v, double* tmp,
                                 double* y) {
  const int64_t N = cx.N;
  ProfScope ps(PROF_MATVEC, cx.st, 2.0 * N * N);
  const unsigned nb = (unsigned)((N + 255) / 256);
  ::ibem::count_launch(), k_vmul<<<nb, 256, 0, cx.st>>>(N, cx.c, v, tmp);
  if (ibem_status q = colreduce<0>(N, A, lda, tmp, cx.nparts, cx.part, cx.st)) return q;
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

// Row scaling r (1 / row max) and column scaling c (1 / column max of R A): As = R A C.
static ibem_status equilibrate(SolveCtx& cx, const double* A, int64_t lda) {
  const int64_t N = cx.N;
  const unsigned nb = (unsigned)((N + 255) / 256);
  if (ibem_status q = colreduce<1>(N, A, lda, (const double*)nullptr, cx.nparts, cx.part, cx.st)) return q;
  ::ibem::count_launch(), k_rowmax_fin<<<nb, 256, 0, cx.st>>>(N, cx.nparts, cx.part, cx.r);
  ::ibem::count_launch(), k_colmax<<<(unsigned)N, 256, 0, cx.st>>>(N, A, lda, cx.r, cx.c);
  IBEM_LAUNCH_CHECK("equilibrate");
  return IBEM_OK;
}

template <typename T>
static ibem_status factor(SolveCtx& cx, const double* A, int64_t lda, T*& W, LuWork<T>& w, int& info) {
  const int64_t N = cx.N;
  IBEM_CUDA(cudaMalloc(&W, sizeof(T) * (size_t)N * N));
  {
    ProfScope ps(PROF_EQUIL, cx.st);
    if (ibem_status q = equilibrate(cx, A, lda)) return q;
    dim3 g((unsigned)((N + 255) / 256), (unsigned)std::min<int64_t>(N, 65535));
    ::ibem::count_launch(), k_scale_copy<T><<<g, 256, 0, cx.st>>>(N, A, lda, cx.r, cx.c, W, N);
    IBEM_LAUNCH_CHECK("equilibrate");
  }
  ibem_status s = lu_alloc(w, N);
  if (s) return s;
  s = lu_rec<T>(W, N, N, 0, N, w, cx.st);
  if (!s) s = trsv_prepare<T>(W, N, N, w, cx.st);
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
  if (hgs.err) return fail(IBEM_ERR_TIMEOUT, "a bounded wait of the panel kernel gave up");
  if (herr) return fail(IBEM_ERR_TIMEOUT, "tensor-core GEMM wait gave up");
  info = hinfo;
  return IBEM_OK;
}

// One restart cycle of right-preconditioned GMRES on As d = rvec with FP64 vectors (V: N x
// (m + 1), Z: N x m, hd: m + 1 doubles of device scratch): prec(v, z) writes z = M^-1 v and
// op(z, w) writes w = As z.  Classical Gram-Schmidt applied twice, Givens rotations on the
// host.  Stops after m steps or once the residual estimate |g_k+1| <= max(stop_abs,
// stop_rel * beta); adds the correction Z y to ys.  steps: Arnoldi steps taken; est: the
// final residual estimate; beta: ||rvec|| (0: nothing to do).
template <class Prec, class Op>
static ibem_status gmres_cycle(int64_t N, int m, const double* rvec, double* V, double* Z, double* hd, double* ys,
                               double stop_abs, double stop_rel, Prec&& prec, Op&& op, int& steps, double& est,
                               double& beta, cudaStream_t st) {
  const unsigned nb = (unsigned)((N + 255) / 256);
  steps = 0;
  IBEM_CUDA(cudaMemsetAsync(hd, 0, sizeof(double), st));
  ::ibem::count_launch(), k_dot_many<<<256, 256, 0, st>>>(N, 1, rvec, N, rvec, hd);
  double b2 = 0;
  IBEM_CUDA(cudaMemcpyAsync(&b2, hd, sizeof(double), cudaMemcpyDeviceToHost, st));
  IBEM_CUDA(cudaStreamSynchronize(st));
  beta = std::sqrt(std::max(b2, 0.0));
  est = beta;
  if (beta == 0) return IBEM_OK;
  const double stop = std::max(stop_abs, stop_rel * beta);
  ::ibem::count_launch(), k_axpby<<<nb, 256, 0, st>>>(N, 1.0 / beta, rvec, 0.0, V);
  std::vector<double> H((m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0);
  g[0] = beta;
  int k = 0;
  ibem_status s = IBEM_OK;
  for (; k < m; ++k) {
    double* vk = V + (size_t)k * N;
    double* zk = Z + (size_t)k * N;
    double* wv = V + (size_t)(k + 1) * N;
    if ((s = prec(vk, zk))) return s;
    if ((s = op(zk, wv))) return s;
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
    ++steps;
    est = std::fabs(g[k + 1]);
    if (est <= stop || hn == 0) { ++k; break; }
  }
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
  return IBEM_OK;
}

ibem_status solve_dense(ibem_solver_form form, int64_t N, double* A, int64_t lda, const double* b, double* x,
                        double tol, ibem_solve_report* rep, cudaStream_t st, int block, float* ws32) {
  if (N <= 0 || !A || !b || !x || lda < N) return fail(IBEM_ERR_ARG, "solve: bad sizes or pointers");
  if (form != IBEM_SOLVE_FP64 && form != IBEM_SOLVE_MIXED_IR && form != IBEM_SOLVE_GMRES_BJ)
    return fail(IBEM_ERR_ARG, "unknown solver form");
  if (form == IBEM_SOLVE_GMRES_BJ && (block < 1 || block > kBjMax))
    return fail(IBEM_ERR_ARG, "block-Jacobi form: block size must be 1.." + std::to_string(kBjMax));
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
    if (ibem_status q = colreduce<2>(N, (const double*)A, lda, cx.c, cx.nparts, cx.part, st)) return q;
    ::ibem::count_launch(), k_scale_rows_of_parts<<<nb, 256, 0, st>>>(N, cx.nparts, cx.part, cx.r, cx.rs);
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
      s = lu_apply<double>(W, N, N, w, ys, st);
      if (!s) s = sticky_err(w, st);
    }
    cudaEventRecord(e2, st);
    if (!s) s = finish_norm();
    if (!s) s = scaled_backward_error(cx, A, lda, ys, bs, rvec, tmp, as_norm, R.backward_error);
    lu_free(w);
    cudaFree(W);
  } else if (form == IBEM_SOLVE_GMRES_BJ) {
    // As32 = FP32 copy of the scaled matrix, P = FP32 inverses of its block x block diagonal
    // blocks; refinement: FP64 residual rs = bs - As ys, GMRES with As32 products (FP64
    // accumulation) right-preconditioned by P reduces it by kInner, ys += correction.
    constexpr int m = 60, max_outer = 30;
    constexpr double kInner = 1e-6;  // about what an FP32 operator can resolve
    const int64_t nblk = (N + block - 1) / block;
    const int64_t ldw = (N + 3) / 4 * 4;   // float4 columns
    float *W = nullptr, *P = nullptr, *zf = nullptr;
    double *V = nullptr, *Z = nullptr, *hd = nullptr;
    int* info_dev = nullptr;
    cudaError_t ce = ws32 ? cudaSuccess : cudaMalloc(&W, sizeof(float) * (size_t)ldw * N);
    float* const Wown = W;
    if (ws32) W = ws32;
    if (ce == cudaSuccess) ce = cudaMalloc(&P, sizeof(float) * (size_t)nblk * block * block);
    if (ce == cudaSuccess) ce = cudaMalloc(&zf, sizeof(float) * (size_t)N);
    if (ce == cudaSuccess) ce = cudaMalloc(&V, sizeof(double) * (size_t)N * (m + 1));
    if (ce == cudaSuccess) ce = cudaMalloc(&Z, sizeof(double) * (size_t)N * m);
    if (ce == cudaSuccess) ce = cudaMalloc(&hd, sizeof(double) * (m + 1) * 2);
    if (ce == cudaSuccess) ce = cudaMalloc(&info_dev, sizeof(int));
    if (ce == cudaSuccess) ce = cudaMemsetAsync(info_dev, 0, sizeof(int), st);
    if (ce != cudaSuccess) s = cuda_fail(ce, "block-Jacobi workspace");
    if (!s) {
      ProfScope ps(PROF_EQUIL, st);
      s = equilibrate(cx, A, lda);
      if (!s) {
        dim3 g((unsigned)((N + 255) / 256), (unsigned)std::min<int64_t>(N, 65535));
        ::ibem::count_launch(), k_scale_copy<float><<<g, 256, 0, st>>>(N, A, lda, cx.r, cx.c, W, ldw);
        if (bj_smem(block) > 48 * 1024)
          cudaFuncSetAttribute(k_bj_invert, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bj_smem(block));
        ::ibem::count_launch(), k_bj_invert<<<(unsigned)nblk, kBjThreads, bj_smem(block), st>>>(N, block, A, lda, cx.r,
                                                                                               cx.c, P, info_dev);
        ::ibem::count_launch(), k_vmul<<<nb, 256, 0, st>>>(N, cx.r, b, bs);
        IBEM_LAUNCH_CHECK("block-Jacobi setup");
      }
    }
    int hinfo = 0;
    if (!s) {
      ce = cudaMemcpyAsync(&hinfo, info_dev, sizeof(int), cudaMemcpyDeviceToHost, st);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
      if (ce != cudaSuccess) s = cuda_fail(ce, "block-Jacobi setup");
      if (!s && hinfo) {
        R.info = hinfo;
        s = fail(IBEM_ERR_SINGULAR, "singular diagonal block in the block-Jacobi form");
      }
    }
    cudaEventRecord(e1, st);
    if (!s) {  // ||As||_inf from the FP32 copy: a denominator of the backward error, FP32 sums are ample
      const int64_t chunk = (N + cx.nparts - 1) / cx.nparts;
      ::ibem::count_launch(), k_gemv_f32acc<true><<<dim3((unsigned)((N + 1023) / 1024), (unsigned)cx.nparts), 256, 0,
                                                     st>>>(N, W, ldw, nullptr, chunk, cx.part);
      ::ibem::count_launch(), k_scale_rows_of_parts<<<nb, 256, 0, st>>>(N, cx.nparts, cx.part, nullptr, cx.rs);
      std::vector<double> h;
      s = vec_to_host(cx.rs, N, h, st);
      as_norm = host_absmax(h);
    }
    if (!s) IBEM_CUDA(cudaMemsetAsync(ys, 0, sizeof(double) * N, st));
    auto prec = [&](const double* v, double* z) -> ibem_status {
      ::ibem::count_launch(), k_bj_apply<<<(unsigned)nblk, kBjApplyThreads, 0, st>>>(N, block, P, v, z);
      IBEM_LAUNCH_CHECK("block-Jacobi apply");
      return IBEM_OK;
    };
    auto op32 = [&](const double* z, double* wv) -> ibem_status {
      ProfScope ps(PROF_MATVEC, st, 2.0 * N * N);
      const int64_t chunk = (N + cx.nparts - 1) / cx.nparts;
      ::ibem::count_launch(), k_d2f<<<nb, 256, 0, st>>>(N, z, zf);
      ::ibem::count_launch(), k_gemv_f32acc<false><<<dim3((unsigned)((N + 1023) / 1024), (unsigned)cx.nparts), 256, 0,
                                                      st>>>(N, W, ldw, zf, chunk, cx.part);
      ::ibem::count_launch(), k_scale_rows_of_parts<<<nb, 256, 0, st>>>(N, cx.nparts, cx.part, nullptr, wv);
      IBEM_LAUNCH_CHECK("FP32 product");
      return IBEM_OK;
    };
    int iters = 0;
    for (int outer = 0; !s && outer < max_outer; ++outer) {
      double be = 0;
      if ((s = scaled_backward_error(cx, A, lda, ys, bs, rvec, tmp, as_norm, be))) break;
      R.backward_error = be;
      if (be <= tol) break;
      int steps = 0;
      double est = 0, beta = 0;
      s = gmres_cycle(N, m, rvec, V, Z, hd, ys, 0.0, kInner, prec, op32, steps, est, beta, st);
      iters += steps;
      if (s || beta == 0) break;
    }
    cudaEventRecord(e2, st);
    if (!s && R.backward_error > tol) s = fail(IBEM_ERR_NOCONV, "block-Jacobi GMRES did not reach the tolerance");
    R.iterations = iters;
    cudaFree(Wown);
    cudaFree(P);
    cudaFree(zf);
    cudaFree(V);
    cudaFree(Z);
    cudaFree(hd);
    cudaFree(info_dev);
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
      s = lu_apply<float>(W, N, N, w, ys, st);
    }
    if (!s) s = finish_norm();
    int iters = 0;
    for (int outer = 0; !s && outer < max_outer; ++outer) {
      if ((s = sticky_err(w, st))) break;
      double be = 0;
      if ((s = scaled_backward_error(cx, A, lda, ys, bs, rvec, tmp, as_norm, be))) break;
      R.backward_error = be;
      if (be <= tol) break;
      // rvec holds rs = bs - As ys
      int steps = 0;
      double est = 0, beta = 0;
      s = gmres_cycle(
          N, m, rvec, V, Z, hd, ys, 1e-2 * tol * (as_norm + 1.0), 0.0,
          [&](const double* v, double* z) -> ibem_status {
            IBEM_CUDA(cudaMemcpyAsync(z, v, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
            return lu_apply<float>(W, N, N, w, z, st);
          },
          [&](const double* z, double* wv) { return scaled_matvec(cx, A, lda, z, tmp, wv); }, steps, est, beta, st);
      iters += steps;
      if (s || beta == 0) break;
    }
    cudaEventRecord(e2, st);
    if (!s) s = sticky_err(w, st);
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
  // x = C ys; also when the tolerance was missed, so that the caller gets the iterate reached
  if (!s || s == IBEM_ERR_NOCONV) ::ibem::count_launch(), k_vmul<<<nb, 256, 0, st>>>(N, cx.c, ys, x);
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
// The first call on a device sets that device up (launch shapes from occupancy
// queries); make that first call before any stream capture.  The array's device
// address is looked up on every call (cudaGetSymbolAddress, which allocates nothing),
// so it stays valid after the module is reloaded.  The call waits for its stream before
// it returns, because it reads the solve's status back to the host.  All calls share
// the array and it keeps the last call's contents: calls that overlap on the GPU (other
// host threads, other streams) race and must be serialised by the caller.
// ===================================================================================
namespace {
constexpr int64_t kNoAllocMaxN = 1024;
constexpr int kNoAllocParts = 16;
constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kNaW = 0;                                                           // N x N factor copy
constexpr size_t kNaVec = align256(sizeof(double) * kNoAllocMaxN * kNoAllocMaxN);    // 6 N-vectors
constexpr size_t kNaPerm = kNaVec + 6 * align256(sizeof(double) * kNoAllocMaxN);     // perm, ipiv
constexpr size_t kNaCand = kNaPerm + 2 * align256(sizeof(int) * kNoAllocMaxN);
constexpr int kNoAllocCaluCta = (int)((kNoAllocMaxN + kCaluMinRows - 1) / kCaluMinRows);  // panel CTAs at most
constexpr size_t kNaGs = kNaCand + calu_bytes<double>(kNoAllocCaluCta);                    // panel buffers
constexpr size_t kNaInfo = kNaGs + align256(sizeof(GridSync));
constexpr size_t kNaPart = kNaInfo + align256(sizeof(int));
constexpr size_t kNaRed = kNaPart + align256(sizeof(double) * kNoAllocParts * kNoAllocMaxN);
constexpr int kNoAllocBlk = (int)((kNoAllocMaxN + kTrsvB - 1) / kTrsvB);                   // triangular-solve blocks
constexpr size_t kNaDinv = kNaRed + align256(sizeof(double) * 4);
constexpr size_t kNaTflags = kNaDinv + align256(sizeof(double) * 2 * kNoAllocBlk * kTrsvB * kTrsvB);
constexpr size_t kNoAllocBytes = kNaTflags + align256(sizeof(int) * kNoAllocBlk);

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
bool g_noalloc_ready[kNoAllocMaxDevices] = {};
int g_noalloc_ncta[kNoAllocMaxDevices] = {};
int g_noalloc_trsv_grid[kNoAllocMaxDevices] = {};

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

static ibem_status noalloc_setup(int dev, unsigned char** base, int* ncta, int* trsv_grid) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(IBEM_ERR_ARG, "solve_noalloc: device index out of range");
  void* p = nullptr;
  IBEM_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  if (!p) return fail(IBEM_ERR_CUDA, "solve_noalloc: no device address for the static workspace");
  if (!g_noalloc_ready[dev]) {
    int nsm = 0;
    IBEM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    IBEM_CUDA(set_solver_smem_attrs<double>());
    int per_sm = 0;
    IBEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_panel<double, kPanelRmax>, kPanelThreads, 0));
    if (per_sm < 1) return fail(IBEM_ERR_CUDA, "solve_noalloc: panel kernel cannot be resident");
    int per_tr = 0;
    IBEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_tr, k_trsv_persist<double, true, true>, kTrsvThreads,
                                                            trsv_persist_smem<double>()));
    if (per_tr < 1) return fail(IBEM_ERR_CUDA, "solve_noalloc: triangular-solve kernel cannot be resident");
    g_noalloc_trsv_grid[dev] = per_tr * nsm;
    g_noalloc_ncta[dev] = std::min(nsm, kCaluMaxCta);
    g_noalloc_ready[dev] = true;
  }
  *base = static_cast<unsigned char*>(p);
  *ncta = g_noalloc_ncta[dev];
  *trsv_grid = g_noalloc_trsv_grid[dev];
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
  int ncta = 0, trsv_grid = 0;
  ibem_status s = noalloc_setup(dev, &base, &ncta, &trsv_grid);
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
  IBEM_CUDA(cudaMemsetAsync(base + kNaCand, 0, calu_bytes<double>(kNoAllocCaluCta), st));
  const unsigned nb = (unsigned)((N + 255) / 256);
  ::ibem::count_launch(), k_rowmax<<<nb, 256, 0, st>>>(N, A, lda, r);
  ::ibem::count_launch(), k_colmax<<<(unsigned)N, 256, 0, st>>>(N, A, lda, r, c);
  ::ibem::count_launch(), k_scale_copy<double><<<dim3(nb, (unsigned)N), 256, 0, st>>>(N, A, lda, r, c, W, N);
  IBEM_LAUNCH_CHECK("solve_noalloc: equilibrate");
  LuWork<double> w;
  w.cb = calu_carve<double>(base + kNaCand, kNoAllocCaluCta);
  w.ipiv_dev = ipiv;
  w.perm = perm;
  w.tmp = tmp;
  w.info = info;
  w.gs = gs;
  w.ncta = std::min(ncta, kNoAllocCaluCta);
  w.dinv = reinterpret_cast<double*>(base + kNaDinv);
  w.tflags = reinterpret_cast<int*>(base + kNaTflags);
  w.trsv_grid = trsv_grid;
  IBEM_CUDA(cudaMemsetAsync(w.tflags, 0, sizeof(int) * kNoAllocBlk, st));
  if ((s = lu_rec<double>(W, N, N, 0, N, w, st))) return s;
  if ((s = trsv_prepare<double>(W, N, N, w, st))) return s;
  ::ibem::count_launch(), k_ipiv_to_perm<<<1, 1, 0, st>>>(N, ipiv, perm);
  ::ibem::count_launch(), k_vmul<<<nb, 256, 0, st>>>(N, r, b, bs);
  IBEM_CUDA(cudaMemcpyAsync(ys, bs, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
  if ((s = lu_apply<double>(W, N, N, w, ys, st))) return s;
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
  if (hgs.err) return fail(IBEM_ERR_TIMEOUT, "solve_noalloc: a bounded wait of the panel or triangular-solve kernel gave up");
  if (hinfo) return fail(IBEM_ERR_SINGULAR, "solve_noalloc: zero pivot");
  return IBEM_OK;
}

// ===================================================================================
// Self-test of the panel kernel's bounded flag wait: one CTA waits, with the same
// calu_wait, for a flag that nothing sets.  The wait must give up after `limit` polls,
// raise the sticky error flag and return, so the host sees IBEM_ERR_TIMEOUT and the
// context stays usable.
// ===================================================================================
namespace {
__global__ void k_selftest_flag_wait(const int* flags, GridSync* gs, long long limit, int* s_out) {
  __shared__ int s_fail;
  if (threadIdx.x == 0) s_fail = 0;
  __syncthreads();
  calu_wait(flags, 1, 1, gs, &s_fail, limit);
  if (threadIdx.x == 0) *s_out = s_fail;
}
}  // namespace

ibem_status selftest_flag_wait(long long limit, cudaStream_t st) {
  if (limit < 1 || limit > kSpinLimit) return fail(IBEM_ERR_ARG, "selftest_flag_wait: limit outside 1..2^22 polls");
  int* d = nullptr;   // [0] the flag nothing sets, [1] GridSync, [2] the CTA's failure record
  IBEM_CUDA(cudaMalloc(&d, 4 * sizeof(int)));
  ibem_status s = IBEM_OK;
  int h[4] = {0, 0, 0, 0};
  cudaError_t ce = cudaMemsetAsync(d, 0, 4 * sizeof(int), st);
  if (ce == cudaSuccess) {
    ::ibem::count_launch(), k_selftest_flag_wait<<<1, 32, 0, st>>>(d, reinterpret_cast<GridSync*>(d + 1), limit, d + 2);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess) s = cuda_fail(ce, "selftest_flag_wait");
  cudaFree(d);
  if (s) return s;
  if (h[1] && h[2]) return fail(IBEM_ERR_TIMEOUT, "selftest_flag_wait: the bounded wait gave up (expected)");
  return IBEM_OK;
}

}  // namespace ibem
