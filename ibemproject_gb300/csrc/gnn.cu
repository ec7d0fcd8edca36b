// Learned neighbour-coupled preconditioner of the matrix-free solver (no reference
// counterpart).
//
// With B_i the block-Jacobi inverses and As = D + O split into its diagonal and
// off-diagonal blocks, the Neumann series As^-1 = B - B O B + B O B O B - ... gives, on the
// graph of each particle's 16 nearest neighbours j (edges e = (i <- j)),
//   C_e = -B_i As_ij B_j           (first-order term of (As^-1)_ij)
//   T_e =  B_i As_ij B_j As_ji B_i  (second-order term of (As^-1)_ii from neighbour j).
// The preconditioner is block-sparse on that graph:
//   (P v)_i = (B_i + sum_e w_e T_e) v_i + sum_e alpha_e C_e v_j,
// with two weights per edge predicted by a message-passing network from the local geometry
// (w = alpha = 0: block-Jacobi; w = alpha = 1: the truncated series; trained weights absorb
// the higher-order terms and the neighbours left out).
//
// Kernels: k_knn (brute force within a realisation, one warp per particle), k_features, k_edge_corr (one CTA of
// 64 threads per edge: eight threads evaluate the two FP32 pair blocks into shared memory,
// all 64 form the four 24 x 24 products), the network's dense layers as one tiled FP32 GEMM
// kernel (k_gemm, 64 x 64 tiles, optional transposes, bias, ReLU, atomic split-K for the
// weight gradients) with gather / scatter / mean kernels around it, the loss and its
// gradient with respect to the edge weights (k_loss), and AdamW (k_adamw).  Training runs
// these in a host loop (ibem_gnn_train) on one batch of realisations.  Inference (the edge
// weights of a solve) uses a split form of the first edge layers: per-node products and
// one fused kernel per layer (forward_fast).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "mf.h"
#include "prof.h"

namespace ibem {
namespace {

inline unsigned nb(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// ---------------------------------------------------------------- parameter layout
constexpr int kH = kGnnHidden, kEin = 2 * kGnnHidden + kGnnEdgeF, kUin = 2 * kGnnHidden;
struct Layout {
  int64_t w_in, b_in, w_m[kGnnLayers], b_m[kGnnLayers], w_u[kGnnLayers], b_u[kGnnLayers], w_o1, b_o1, w_o2, b_o2,
      total;
  Layout() {
    int64_t o = 0;
    auto take = [&](int64_t n) { const int64_t r = o; o += n; return r; };
    w_in = take((int64_t)kGnnNodeF * kH);
    b_in = take(kH);
    for (int l = 0; l < kGnnLayers; ++l) {
      w_m[l] = take((int64_t)kEin * kH);
      b_m[l] = take(kH);
      w_u[l] = take((int64_t)kUin * kH);
      b_u[l] = take(kH);
    }
    w_o1 = take((int64_t)kEin * kH);
    b_o1 = take(kH);
    w_o2 = take((int64_t)kH * kGnnOut);
    b_o2 = take(kGnnOut);
    total = o;
  }
};

// ---------------------------------------------------------------- graph and features
// k nearest neighbours of p within its realisation: distance^2 in FP64, ties to the
// lower index.  One warp per particle: every lane keeps a sorted list of the best 16 of its
// own share of the candidates (q = first + lane, + 32, ...), then 16 rounds of a warp-wide
// minimum over the lanes' list heads pick the result in order.
__global__ void k_knn(int num, const int* __restrict__ seg_of, const int* __restrict__ seg_begin,
                      const double* __restrict__ cen, int* __restrict__ nbr) {
  const int p = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (p >= num) return;  // uniform per warp
  const int sg = seg_of[p];
  const int b0 = seg_begin[sg], b1 = seg_begin[sg + 1];
  const double px = cen[3 * (int64_t)p], py = cen[3 * (int64_t)p + 1], pz = cen[3 * (int64_t)p + 2];
  double bd[kKnn];
  int bi[kKnn];
#pragma unroll
  for (int j = 0; j < kKnn; ++j) {
    bd[j] = INFINITY;
    bi[j] = -1;
  }
  for (int q = b0 + lane; q < b1; q += 32) {
    if (q == p) continue;
    const double dx = cen[3 * (int64_t)q] - px, dy = cen[3 * (int64_t)q + 1] - py, dz = cen[3 * (int64_t)q + 2] - pz;
    const double d2 = dx * dx + dy * dy + dz * dz;
    if (!(d2 < bd[kKnn - 1])) continue;  // later q of this lane: an equal distance loses
    double cd = d2;
    int ci = q;
#pragma unroll
    for (int j = 0; j < kKnn; ++j) {  // insert (cd, ci), shifting larger entries down
      if (cd < bd[j]) {
        const double td = bd[j];
        const int ti = bi[j];
        bd[j] = cd;
        bi[j] = ci;
        cd = td;
        ci = ti;
      }
    }
  }
  int mine = -1;
#pragma unroll 1
  for (int r = 0; r < kKnn; ++r) {
    double wd = bd[0];
    int wi = bi[0];
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const double od = __shfl_xor_sync(0xffffffffu, wd, off);
      const int oi = __shfl_xor_sync(0xffffffffu, wi, off);
      if (od < wd || (od == wd && (unsigned)oi < (unsigned)wi)) {
        wd = od;
        wi = oi;
      }
    }
    if (lane == r) mine = wi;
    if (wi >= 0 && bi[0] == wi) {  // candidates are unique across lanes: one lane pops
#pragma unroll
      for (int j = 0; j < kKnn - 1; ++j) {
        bd[j] = bd[j + 1];
        bi[j] = bi[j + 1];
      }
      bd[kKnn - 1] = INFINITY;
      bi[kKnn - 1] = -1;
    }
  }
  if (lane < kKnn) nbr[(int64_t)kKnn * p + lane] = mine;
}

struct MatFeat {
  float e_ratio, nu0, nu1;
};

__global__ void k_features(int num, const int* __restrict__ seg_of, const MatFeat* __restrict__ mf,
                           const double* __restrict__ cen, const double* __restrict__ rad, const int* __restrict__ nbr,
                           float* __restrict__ xn, float* __restrict__ ef) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)num * kKnn) return;
  const int i = (int)(t / kKnn), slot = (int)(t % kKnn);
  if (slot == 0) {
    const MatFeat m = mf[seg_of[i]];
    const float v[kGnnNodeF] = {1.f, 1.f, 1.f, 1.f, 0.f, 0.f, 0.f, m.e_ratio, m.nu0, m.nu1};
    for (int k = 0; k < kGnnNodeF; ++k) xn[(int64_t)kGnnNodeF * i + k] = v[k];
  }
  const int j = nbr[t];
  float* o = ef + t * kGnnEdgeF;
  if (j < 0) {
    for (int k = 0; k < kGnnEdgeF; ++k) o[k] = 0.f;
    return;
  }
  const double ai = rad[i], ia = 1.0 / ai;
  const double d0 = (cen[3 * (int64_t)j] - cen[3 * (int64_t)i]) * ia;
  const double d1 = (cen[3 * (int64_t)j + 1] - cen[3 * (int64_t)i + 1]) * ia;
  const double d2 = (cen[3 * (int64_t)j + 2] - cen[3 * (int64_t)i + 2]) * ia;
  const double dist = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
  const double ratio = rad[j] * ia;
  const double q = 2.0 / dist;
  o[0] = (float)d0;
  o[1] = (float)d1;
  o[2] = (float)d2;
  o[3] = (float)dist;
  o[4] = (float)ratio;
  o[5] = (float)(dist - 1.0 - ratio);
  o[6] = (float)(q * q * q);
}

// ---------------------------------------------------------------- edge corrections
struct SmemSink {
  float* M;
  float scale;
  __device__ __forceinline__ void operator()(int r, int c, float v) const { M[r * kMfNu + c] = v * scale; }
};

// C = sc * A B for 24 x 24 row-major matrices in shared memory; 64 threads, each a 3 x 3
// register tile (rows 3 (t / 8) .., columns 3 (t % 8) ..): 6 shared loads per 9 FMAs
__device__ __forceinline__ void mm24(const float* A, const float* B, float* C, float sc) {
  const int tr = 3 * (threadIdx.x >> 3), tc = 3 * (threadIdx.x & 7);
  float acc[3][3] = {};
#pragma unroll 4
  for (int k = 0; k < kMfNu; ++k) {
    float a[3], b[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) a[i] = A[(tr + i) * kMfNu + k];
#pragma unroll
    for (int j = 0; j < 3; ++j) b[j] = B[k * kMfNu + tc + j];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[(tr + i) * kMfNu + tc + j] = sc * acc[i][j];
}

__global__ void __launch_bounds__(64)
    k_edge_corr(int num, const int* __restrict__ nbr, const int* __restrict__ seg_of, const SphMatF* __restrict__ mats,
                const double* __restrict__ cen, const double* __restrict__ rad, const float* __restrict__ B,
                const float* __restrict__ wa, float* __restrict__ D, float* __restrict__ Q, int nrhs,
                const float* __restrict__ rq, int64_t N, float* __restrict__ u) {
  __shared__ float Aij[kMfNu * kMfNu], Aji[kMfNu * kMfNu], Bi[kMfNu * kMfNu], Bj[kMfNu * kMfNu];
  __shared__ float T1[kMfNu * kMfNu], T2[kMfNu * kMfNu];
  const int64_t e = blockIdx.x;
  const int64_t E = (int64_t)num * kKnn;
  const int i = (int)(e / kKnn);
  const int j = nbr[e];
  if (j < 0) {  // no neighbour in this slot
    if (u)
      for (int t = threadIdx.x; t < nrhs * 2 * kMfNu; t += blockDim.x)
        u[((int64_t)(t / (2 * kMfNu)) * E + e) * 2 * kMfNu + t % (2 * kMfNu)] = 0.f;
    return;
  }
  const float* bi = B + (int64_t)kMfNu * kMfNu * i;
  const float* bj = B + (int64_t)kMfNu * kMfNu * j;
  for (int k = threadIdx.x; k < kMfNu * kMfNu; k += blockDim.x) {
    Bi[k] = bi[k];
    Bj[k] = bj[k];
  }
  if (threadIdx.x < 8) {  // 8 generators: 4 sub-blocks (column order x row order) of each block
    const SphMatF mc = mats[seg_of[i]];
    const bool ij = threadIdx.x < 4;  // As_ij: target i, source j; As_ji: target j, source i
    const int fn = threadIdx.x & 3;
    const int tgt = ij ? i : j, src = ij ? j : i;
    const double ia = 1.0 / rad[src];
    const float x0 = (float)((cen[3 * (int64_t)tgt] - cen[3 * (int64_t)src]) * ia);
    const float x1 = (float)((cen[3 * (int64_t)tgt + 1] - cen[3 * (int64_t)src + 1]) * ia);
    const float x2 = (float)((cen[3 * (int64_t)tgt + 2] - cen[3 * (int64_t)src + 2]) * ia);
    float* M = ij ? Aij : Aji;
    SmemSink sk{M, fn >= 2 ? (float)(rad[tgt] * ia) : 1.f};   // rows of order 1 carry a_tgt / a_src
    if (fn == 0) sph_block24f_c0_r0(x0, x1, x2, 1.f, mc, sk);
    else if (fn == 1) sph_block24f_c1_r0(x0, x1, x2, 1.f, mc, sk);
    else if (fn == 2) sph_block24f_c0_r1(x0, x1, x2, 1.f, mc, sk);
    else sph_block24f_c1_r1(x0, x1, x2, 1.f, mc, sk);
  }
  __syncthreads();
  mm24(Aji, Bi, T1, 1.f);    // As_ji B_i
  mm24(Aij, Bj, T2, 1.f);    // As_ij B_j
  __syncthreads();
  mm24(Bi, T2, Aij, -1.f);   // C = -B_i As_ij B_j        (As_ij no longer needed)
  __syncthreads();
  mm24(Aij, T1, T2, -1.f);   // T = -C As_ji B_i
  __syncthreads();
  if (wa) {
    const float we = wa[2 * e], ae = wa[2 * e + 1];
    if (D) {
      float* di = D + (int64_t)kMfNu * kMfNu * i;
      for (int k = threadIdx.x; k < kMfNu * kMfNu; k += blockDim.x) atomicAdd(di + k, we * T2[k]);
    }
    if (Q) {
      float* qe = Q + (int64_t)kMfNu * kMfNu * e;
      for (int k = threadIdx.x; k < kMfNu * kMfNu; k += blockDim.x) qe[k] = ae * Aij[k];
    }
  }
  if (u && rq) {
    for (int t = threadIdx.x; t < nrhs * 2 * kMfNu; t += blockDim.x) {
      const int q = t / (2 * kMfNu), part = (t / kMfNu) & 1, r = t % kMfNu;
      const float* rv = rq + (int64_t)q * N + (int64_t)kMfNu * (part ? j : i);
      const float* M = part ? Aij : T2;
      float s = 0.f;
#pragma unroll
      for (int c = 0; c < kMfNu; ++c) s = fmaf(M[r * kMfNu + c], rv[c], s);
      u[((int64_t)q * E + e) * 2 * kMfNu + part * kMfNu + r] = s;
    }
  }
}

// z = (B r - e) * scale, r and e FP64 -> FP32 (one thread per row)
__global__ void k_sample_z(int num, const float* __restrict__ B, const double* __restrict__ r,
                           const double* __restrict__ e, const double* __restrict__ scale, float* __restrict__ z,
                           float* __restrict__ rf) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)num * kMfNu) return;
  const int64_t p = t / kMfNu;
  const float* row = B + t * kMfNu;
  const double* rv = r + p * kMfNu;
  double s = 0;
  for (int c = 0; c < kMfNu; ++c) s += (double)row[c] * rv[c];
  const double k = *scale;
  z[t] = (float)((s - e[t]) * k);
  rf[t] = (float)(r[t] * k);
}

__global__ void k_sumsq(int64_t n, const double* __restrict__ x, double* __restrict__ out) {
  double s = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += x[i] * x[i];
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}
__global__ void k_rsqrt_inplace(double* x) { *x = *x > 0 ? 1.0 / sqrt(*x) : 0.0; }

// ---------------------------------------------------------------- dense layers
// C (M x N, ldc) = op(A) op(B) [+ bias] [relu], op(A)(m,k) = TA ? A[k*lda+m] : A[m*lda+k],
// op(B)(k,n) = TB ? B[n*ldb+k] : B[k*ldb+n].  mode 0: store, 1: atomic add (split-K over z).
constexpr int kGT = 64, kGK = 16;
template <bool TA, bool TB>
__global__ void __launch_bounds__(256)
    k_gemm(int M, int N, int K, const float* __restrict__ A, int lda, const float* __restrict__ B, int ldb,
           float* __restrict__ C, int ldc, const float* __restrict__ bias, int relu, int mode) {
  __shared__ float As[kGK][kGT + 1], Bs[kGK][kGT + 1];
  const int m0 = blockIdx.y * kGT, n0 = blockIdx.x * kGT;
  const int kper = (K + gridDim.z - 1) / gridDim.z;
  const int kb = blockIdx.z * kper, ke = min(K, kb + kper);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4] = {};
  for (int k0 = kb; k0 < ke; k0 += kGK) {
    for (int t = threadIdx.x; t < kGK * kGT; t += 256) {
      int kk, mm;
      if (TA) { mm = t % kGT; kk = t / kGT; } else { kk = t % kGK; mm = t / kGK; }
      const int gm = m0 + mm, gk = k0 + kk;
      float v = 0.f;
      if (gm < M && gk < ke) v = TA ? A[(int64_t)gk * lda + gm] : A[(int64_t)gm * lda + gk];
      As[kk][mm] = v;
    }
    for (int t = threadIdx.x; t < kGK * kGT; t += 256) {
      int kk, nn;
      if (TB) { kk = t % kGK; nn = t / kGK; } else { nn = t % kGT; kk = t / kGT; }
      const int gn = n0 + nn, gk = k0 + kk;
      float v = 0.f;
      if (gn < N && gk < ke) v = TB ? B[(int64_t)gn * ldb + gk] : B[(int64_t)gk * ldb + gn];
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      float v = acc[i][j];
      if (mode == 1) {
        atomicAdd(C + (int64_t)gm * ldc + gn, v);
      } else {
        if (bias) v += bias[gn];
        if (relu) v = fmaxf(v, 0.f);
        C[(int64_t)gm * ldc + gn] = v;
      }
    }
  }
}

// db[n] += sum_m dZ[m][n]
__global__ void k_colsum(int M, int N, const float* __restrict__ dZ, float* __restrict__ db) {
  const int n = threadIdx.x % 64 + blockIdx.y * 64;
  if (n >= N) return;
  float s = 0.f;
  for (int m = blockIdx.x * 4 + threadIdx.x / 64; m < M; m += gridDim.x * 4) s += dZ[(int64_t)m * N + n];
  atomicAdd(db + n, s);
}

// Ein[e] = [H[i], H[j], ef[e]] (zeros for a missing neighbour)
__global__ void k_gather_edges(int64_t E, const int* __restrict__ nbr, const float* __restrict__ H,
                               const float* __restrict__ ef, float* __restrict__ Ein) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= E * kEin) return;
  const int64_t e = t / kEin;
  const int c = (int)(t % kEin);
  const int j = nbr[e];
  const int i = (int)(e / kKnn);
  float v = 0.f;
  if (j >= 0) {
    if (c < kH) v = H[(int64_t)i * kH + c];
    else if (c < 2 * kH) v = H[(int64_t)j * kH + c - kH];
    else v = ef[e * kGnnEdgeF + c - 2 * kH];
  }
  Ein[t] = v;
}

// dH[i] += dEin[e][0:H], dH[j] += dEin[e][H:2H]
__global__ void k_scatter_edges(int64_t E, const int* __restrict__ nbr, const float* __restrict__ dEin,
                                float* __restrict__ dH) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= E * 2 * kH) return;
  const int64_t e = t / (2 * kH);
  const int c = (int)(t % (2 * kH));
  const int j = nbr[e];
  if (j < 0) return;
  const int i = (int)(e / kKnn);
  const float v = dEin[e * kEin + c];
  if (c < kH) atomicAdd(dH + (int64_t)i * kH + c, v);
  else atomicAdd(dH + (int64_t)j * kH + c - kH, v);
}

// Uin[i] = [H[i], mean over valid edges of M[e]]
__global__ void k_mean_concat(int num, const int* __restrict__ nbr, const float* __restrict__ H,
                              const float* __restrict__ Mm, float* __restrict__ Uin) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)num * kH) return;
  const int i = (int)(t / kH), c = (int)(t % kH);
  float s = 0.f;
  int deg = 0;
  for (int k = 0; k < kKnn; ++k)
    if (nbr[(int64_t)i * kKnn + k] >= 0) {
      s += Mm[((int64_t)i * kKnn + k) * kH + c];
      ++deg;
    }
  Uin[(int64_t)i * kUin + c] = H[t];
  Uin[(int64_t)i * kUin + kH + c] = deg ? s / deg : 0.f;
}

// dM[e] = dUin[i][H + c] / deg_i * (M[e] > 0), 0 for a missing neighbour
__global__ void k_mean_bwd(int num, const int* __restrict__ nbr, const float* __restrict__ dUin,
                           const float* __restrict__ Mm, float* __restrict__ dM) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)num * kKnn * kH) return;
  const int64_t e = t / kH;
  const int c = (int)(t % kH);
  const int i = (int)(e / kKnn);
  int deg = 0;
  for (int k = 0; k < kKnn; ++k) deg += nbr[(int64_t)i * kKnn + k] >= 0;
  float v = 0.f;
  if (nbr[e] >= 0 && Mm[t] > 0.f) v = dUin[(int64_t)i * kUin + kH + c] / deg;
  dM[t] = v;
}

// H1 = H0 + U ; dZ = dY * (Y > 0) ; dH = dHn + dUin[:, :H]
__global__ void k_add(int64_t n, const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ c) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < n) c[t] = a[t] + b[t];
}
__global__ void k_relu_mask(int64_t n, const float* __restrict__ dY, const float* __restrict__ Y, float* __restrict__ dZ) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < n) dZ[t] = Y[t] > 0.f ? dY[t] : 0.f;
}
__global__ void k_add_left(int num, const float* __restrict__ dHn, const float* __restrict__ dUin, float* __restrict__ dH) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)num * kH) return;
  dH[t] = dHn[t] + dUin[(t / kH) * kUin + t % kH];
}
// out[e][k] = O1[e] . w_o2[:, k] + b_o2[k] (0 for a missing neighbour)
__global__ void k_out(int64_t E, const int* __restrict__ nbr, const float* __restrict__ O1, const float* __restrict__ w2,
                      const float* __restrict__ b2, float* __restrict__ w) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= E * kGnnOut) return;
  const int64_t e = t / kGnnOut;
  const int k = (int)(t % kGnnOut);
  if (nbr[e] < 0) {
    w[t] = 0.f;
    return;
  }
  float s = b2[k];
  for (int c = 0; c < kH; ++c) s = fmaf(O1[e * kH + c], w2[c * kGnnOut + k], s);
  w[t] = s;
}
// dO1[e][c] = sum_k dout[e][k] w_o2[c][k] * (O1 > 0)
__global__ void k_out_bwd(int64_t E, const float* __restrict__ O1, const float* __restrict__ w2,
                          const float* __restrict__ dw, float* __restrict__ dO1) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= E * kH) return;
  const int64_t e = t / kH;
  const int c = (int)(t % kH);
  float d = 0.f;
  for (int k = 0; k < kGnnOut; ++k) d = fmaf(dw[e * kGnnOut + k], w2[c * kGnnOut + k], d);
  dO1[t] = O1[t] > 0.f ? d : 0.f;
}

// Loss L = sum_q sum_i ||z_qi + sum_e (w_e u_qe + alpha_e v_qe)||^2 and its gradient with
// respect to (w_e, alpha_e); one warp per particle, lanes over the 24 rows
__global__ void k_loss(int num, int nrhs, const int* __restrict__ nbr, const float* __restrict__ wa,
                       const float* __restrict__ z, const float* __restrict__ u, double* __restrict__ loss,
                       float* __restrict__ dw) {
  const int i = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (i >= num) return;
  const int64_t E = (int64_t)num * kKnn;
  float we[kKnn], ae[kKnn], gw[kKnn], ga[kKnn];
#pragma unroll
  for (int k = 0; k < kKnn; ++k) {
    const bool v = nbr[(int64_t)i * kKnn + k] >= 0;
    we[k] = v ? wa[2 * ((int64_t)i * kKnn + k)] : 0.f;
    ae[k] = v ? wa[2 * ((int64_t)i * kKnn + k) + 1] : 0.f;
    gw[k] = ga[k] = 0.f;
  }
  double ls = 0;
  for (int q = 0; q < nrhs; ++q) {
    float qv = 0.f;
    float uk[kKnn], vk[kKnn];
    if (lane < kMfNu) {
      qv = z[(int64_t)q * num * kMfNu + (int64_t)i * kMfNu + lane];
#pragma unroll
      for (int k = 0; k < kKnn; ++k) {
        const float* ue = u + ((int64_t)q * E + (int64_t)i * kKnn + k) * 2 * kMfNu;
        uk[k] = ue[lane];
        vk[k] = ue[kMfNu + lane];
        qv = fmaf(we[k], uk[k], fmaf(ae[k], vk[k], qv));
      }
    } else {
#pragma unroll
      for (int k = 0; k < kKnn; ++k) uk[k] = vk[k] = 0.f;
    }
    ls += (double)qv * qv;
#pragma unroll
    for (int k = 0; k < kKnn; ++k) {
      gw[k] = fmaf(2.f * qv, uk[k], gw[k]);
      ga[k] = fmaf(2.f * qv, vk[k], ga[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < kKnn; ++k)
    for (int o = 16; o; o >>= 1) {
      gw[k] += __shfl_xor_sync(0xffffffffu, gw[k], o);
      ga[k] += __shfl_xor_sync(0xffffffffu, ga[k], o);
    }
  for (int o = 16; o; o >>= 1) ls += __shfl_xor_sync(0xffffffffu, ls, o);
  if (lane == 0) {
    atomicAdd(loss, ls);
#pragma unroll
    for (int k = 0; k < kKnn; ++k) {
      const bool v = nbr[(int64_t)i * kKnn + k] >= 0;
      dw[2 * ((int64_t)i * kKnn + k)] = v ? gw[k] : 0.f;
      dw[2 * ((int64_t)i * kKnn + k) + 1] = v ? ga[k] : 0.f;
    }
  }
}

__global__ void k_adamw(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                        float* __restrict__ v, float lr, float b1, float b2, float eps, float wd, float c1, float c2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / c1, vh = vi / c2;
  p[i] = p[i] - lr * wd * p[i] - lr * mh / (sqrtf(vh) + eps);
}

// ---------------------------------------------------------------- inference pass
// The first layer of every edge MLP splits: [h_i, h_j, f_e] W = (H W_top)_i + (H W_mid)_j
// + f_e W_bot, so the two 64 x 64 products run once per node (P, Q) and the edge work is a
// 7-term dot product per channel, fused with the ReLU and the mean (messages) or with the
// output layer (edge weights).  Same arithmetic as the training pass up to rounding.

// Uin[i] = [H[i], mean over valid edges of relu(P[i] + Q[j] + f_e W_bot + b)]
__global__ void k_msg_mean(int num, const int* __restrict__ nbr, const float* __restrict__ H,
                           const float* __restrict__ P, const float* __restrict__ Q, const float* __restrict__ ef,
                           const float* __restrict__ Wb, const float* __restrict__ bias, float* __restrict__ Uin) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)num * kH) return;
  const int i = (int)(t / kH), c = (int)(t % kH);
  float w[kGnnEdgeF];
#pragma unroll
  for (int k = 0; k < kGnnEdgeF; ++k) w[k] = Wb[k * kH + c];
  const float pc = P[t] + bias[c];
  float s = 0.f;
  int deg = 0;
  for (int k = 0; k < kKnn; ++k) {
    const int64_t e = (int64_t)i * kKnn + k;
    const int j = nbr[e];
    if (j < 0) continue;
    float m = pc + Q[(int64_t)j * kH + c];
#pragma unroll
    for (int q = 0; q < kGnnEdgeF; ++q) m = fmaf(ef[e * kGnnEdgeF + q], w[q], m);
    s += fmaxf(m, 0.f);
    ++deg;
  }
  Uin[(int64_t)i * kUin + c] = H[t];
  Uin[(int64_t)i * kUin + kH + c] = deg ? s / deg : 0.f;
}

// w_e = relu(P[i] + Q[j] + f_e W_bot + b1) W_o2 + b_o2 (0 for a missing neighbour); one warp
// per edge, lanes over channel pairs
__global__ void k_edge_out(int64_t E, const int* __restrict__ nbr, const float* __restrict__ P,
                           const float* __restrict__ Q, const float* __restrict__ ef, const float* __restrict__ Wb,
                           const float* __restrict__ b1, const float* __restrict__ w2, const float* __restrict__ b2,
                           float* __restrict__ out) {
  const int64_t e = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (e >= E) return;
  const int j = nbr[e];
  if (j < 0) {
    if (lane < kGnnOut) out[e * kGnnOut + lane] = 0.f;
    return;
  }
  const int64_t i = e / kKnn;
  float acc[kGnnOut] = {};
#pragma unroll
  for (int h = 0; h < kH / 32; ++h) {
    const int c = lane + 32 * h;
    float m = P[i * kH + c] + Q[(int64_t)j * kH + c] + b1[c];
#pragma unroll
    for (int q = 0; q < kGnnEdgeF; ++q) m = fmaf(ef[e * kGnnEdgeF + q], Wb[q * kH + c], m);
    m = fmaxf(m, 0.f);
#pragma unroll
    for (int k = 0; k < kGnnOut; ++k) acc[k] = fmaf(m, w2[c * kGnnOut + k], acc[k]);
  }
#pragma unroll
  for (int k = 0; k < kGnnOut; ++k)
    for (int o = 16; o; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
  if (lane < kGnnOut) out[e * kGnnOut + lane] = (lane == 0 ? acc[0] : acc[1]) + b2[lane];
}

// ---------------------------------------------------------------- network driver
struct Net {
  int num;
  int64_t E;
  cudaStream_t st;
  Layout L;
  std::vector<void*> mem;
  float *H[kGnnLayers + 1], *Ein[kGnnLayers], *Mm[kGnnLayers], *Uin[kGnnLayers], *Upd[kGnnLayers];
  float *Oin, *O1, *w;
  // backward
  float *dw, *dO1, *dEin, *dH, *dHn, *dUpd, *dUin, *dM;
  ~Net() {
    for (void* p : mem) free_async(p, st);
  }
  ibem_status buf(float*& p, int64_t n) {
    IBEM_CUDA(alloc_async((void**)&p, sizeof(float) * std::max<int64_t>(n, 1), st));
    mem.push_back(p);
    return IBEM_OK;
  }
  ibem_status alloc(bool backward) {
    ibem_status s = IBEM_OK;
    for (int l = 0; l <= kGnnLayers && !s; ++l) s = buf(H[l], (int64_t)num * kH);
    for (int l = 0; l < kGnnLayers && !s; ++l) {
      if (!s) s = buf(Ein[l], E * kEin);
      if (!s) s = buf(Mm[l], E * kH);
      if (!s) s = buf(Uin[l], (int64_t)num * kUin);
      if (!s) s = buf(Upd[l], (int64_t)num * kH);
    }
    if (!s) s = buf(Oin, E * kEin);
    if (!s) s = buf(O1, E * kH);
    if (!s) s = buf(w, E * kGnnOut);
    if (backward) {
      if (!s) s = buf(dw, E * kGnnOut);
      if (!s) s = buf(dO1, E * kH);
      if (!s) s = buf(dEin, E * kEin);
      if (!s) s = buf(dH, (int64_t)num * kH);
      if (!s) s = buf(dHn, (int64_t)num * kH);
      if (!s) s = buf(dUpd, (int64_t)num * kH);
      if (!s) s = buf(dUin, (int64_t)num * kUin);
      if (!s) s = buf(dM, E * kH);
    }
    return s;
  }
  void gemm(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
            const float* bias, int relu) {
    dim3 g((N + kGT - 1) / kGT, (M + kGT - 1) / kGT, 1);
    ::ibem::count_launch(), k_gemm<false, false><<<g, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, relu, 0);
  }
  // dX = dZ W^T  (dZ: M x N, W: K x N row-major) -> M x K
  void gemm_dx(int M, int N, int K, const float* dZ, const float* W, float* dX) {
    dim3 g((K + kGT - 1) / kGT, (M + kGT - 1) / kGT, 1);
    ::ibem::count_launch(), k_gemm<false, true><<<g, 256, 0, st>>>(M, K, N, dZ, N, W, N, dX, K, nullptr, 0, 0);
  }
  // gW += X^T dZ (X: M x K, dZ: M x N) -> K x N, split over M
  void gemm_dw(int M, int N, int K, const float* X, const float* dZ, float* gW, float* gb) {
    const int splits = std::max(1, std::min(256, M / 512));
    dim3 g((N + kGT - 1) / kGT, (K + kGT - 1) / kGT, splits);
    ::ibem::count_launch(), k_gemm<true, false><<<g, 256, 0, st>>>(K, N, M, X, K, dZ, N, gW, N, nullptr, 0, 1);
    ::ibem::count_launch(), k_colsum<<<dim3(std::max(1, std::min(512, M / 64)), (N + 63) / 64), 256, 0, st>>>(M, N, dZ, gb);
  }
  ibem_status forward(const int* nbr, const float* xn, const float* ef, const float* P) {
    gemm(num, kH, kGnnNodeF, xn, kGnnNodeF, P + L.w_in, kH, H[0], kH, P + L.b_in, 1);
    for (int l = 0; l < kGnnLayers; ++l) {
      ::ibem::count_launch(), k_gather_edges<<<nb(E * kEin), 256, 0, st>>>(E, nbr, H[l], ef, Ein[l]);
      gemm((int)E, kH, kEin, Ein[l], kEin, P + L.w_m[l], kH, Mm[l], kH, P + L.b_m[l], 1);
      ::ibem::count_launch(), k_mean_concat<<<nb((int64_t)num * kH), 256, 0, st>>>(num, nbr, H[l], Mm[l], Uin[l]);
      gemm(num, kH, kUin, Uin[l], kUin, P + L.w_u[l], kH, Upd[l], kH, P + L.b_u[l], 1);
      ::ibem::count_launch(), k_add<<<nb((int64_t)num * kH), 256, 0, st>>>((int64_t)num * kH, H[l], Upd[l], H[l + 1]);
    }
    ::ibem::count_launch(), k_gather_edges<<<nb(E * kEin), 256, 0, st>>>(E, nbr, H[kGnnLayers], ef, Oin);
    gemm((int)E, kH, kEin, Oin, kEin, P + L.w_o1, kH, O1, kH, P + L.b_o1, 1);
    ::ibem::count_launch(), k_out<<<nb(E * kGnnOut), 256, 0, st>>>(E, nbr, O1, P + L.w_o2, P + L.b_o2, w);
    IBEM_LAUNCH_CHECK("gnn forward");
    return IBEM_OK;
  }
  // gradient of the parameters from dw (set by the loss); G zeroed here
  ibem_status backward(const int* nbr, const float* xn, const float* P, float* G) {
    IBEM_CUDA(cudaMemsetAsync(G, 0, sizeof(float) * L.total, st));
    // out = O1 w_o2 + b_o2 (dw is 0 on missing neighbours)
    gemm_dw((int)E, kGnnOut, kH, O1, dw, G + L.w_o2, G + L.b_o2);
    ::ibem::count_launch(), k_out_bwd<<<nb(E * kH), 256, 0, st>>>(E, O1, P + L.w_o2, dw, dO1);
    gemm_dw((int)E, kH, kEin, Oin, dO1, G + L.w_o1, G + L.b_o1);
    gemm_dx((int)E, kH, kEin, dO1, P + L.w_o1, dEin);
    IBEM_CUDA(cudaMemsetAsync(dH, 0, sizeof(float) * (int64_t)num * kH, st));
    ::ibem::count_launch(), k_scatter_edges<<<nb(E * 2 * kH), 256, 0, st>>>(E, nbr, dEin, dH);
    for (int l = kGnnLayers - 1; l >= 0; --l) {
      // dH holds dL/dH[l+1]
      ::ibem::count_launch(), k_relu_mask<<<nb((int64_t)num * kH), 256, 0, st>>>((int64_t)num * kH, dH, Upd[l], dUpd);
      gemm_dw(num, kH, kUin, Uin[l], dUpd, G + L.w_u[l], G + L.b_u[l]);
      gemm_dx(num, kH, kUin, dUpd, P + L.w_u[l], dUin);
      ::ibem::count_launch(), k_add_left<<<nb((int64_t)num * kH), 256, 0, st>>>(num, dH, dUin, dHn);
      ::ibem::count_launch(), k_mean_bwd<<<nb(E * kH), 256, 0, st>>>(num, nbr, dUin, Mm[l], dM);
      gemm_dw((int)E, kH, kEin, Ein[l], dM, G + L.w_m[l], G + L.b_m[l]);
      gemm_dx((int)E, kH, kEin, dM, P + L.w_m[l], dEin);
      ::ibem::count_launch(), k_scatter_edges<<<nb(E * 2 * kH), 256, 0, st>>>(E, nbr, dEin, dHn);
      std::swap(dH, dHn);
    }
    ::ibem::count_launch(), k_relu_mask<<<nb((int64_t)num * kH), 256, 0, st>>>((int64_t)num * kH, dH, H[0], dUpd);
    gemm_dw(num, kH, kGnnNodeF, xn, dUpd, G + L.w_in, G + L.b_in);
    IBEM_LAUNCH_CHECK("gnn backward");
    return IBEM_OK;
  }
};

// Inference pass of the network (edge weights only), with the split first layers above.
ibem_status forward_fast(int num, const int* nbr, const float* xn, const float* ef, const float* Pm, float* w,
                         cudaStream_t st) {
  static_assert(kGnnOut == 2, "k_edge_out writes two outputs per edge");
  const Layout L;
  const int64_t E = (int64_t)num * kKnn;
  float *H = nullptr, *H2 = nullptr, *P = nullptr, *Q = nullptr, *Uin = nullptr, *Upd = nullptr;
  const size_t nh = sizeof(float) * (size_t)num * kH;
  cudaError_t e = alloc_async((void**)&H, nh, st);
  if (e == cudaSuccess) e = alloc_async((void**)&H2, nh, st);
  if (e == cudaSuccess) e = alloc_async((void**)&P, nh, st);
  if (e == cudaSuccess) e = alloc_async((void**)&Q, nh, st);
  if (e == cudaSuccess) e = alloc_async((void**)&Upd, nh, st);
  if (e == cudaSuccess) e = alloc_async((void**)&Uin, 2 * nh, st);
  ibem_status s = e == cudaSuccess ? IBEM_OK : cuda_fail(e, "gnn forward");
  Net g;  // launch helpers only (no buffers)
  g.num = num;
  g.E = E;
  g.st = st;
  if (!s) {
    g.gemm(num, kH, kGnnNodeF, xn, kGnnNodeF, Pm + L.w_in, kH, H, kH, Pm + L.b_in, 1);
    for (int l = 0; l < kGnnLayers; ++l) {
      const float* W = Pm + L.w_m[l];
      g.gemm(num, kH, kH, H, kH, W, kH, P, kH, nullptr, 0);                 // rows 0..63: h_i
      g.gemm(num, kH, kH, H, kH, W + kH * kH, kH, Q, kH, nullptr, 0);       // rows 64..127: h_j
      ::ibem::count_launch(), k_msg_mean<<<nb((int64_t)num * kH), 256, 0, st>>>(num, nbr, H, P, Q, ef, W + 2 * kH * kH,
                                                                                Pm + L.b_m[l], Uin);
      g.gemm(num, kH, kUin, Uin, kUin, Pm + L.w_u[l], kH, Upd, kH, Pm + L.b_u[l], 1);
      ::ibem::count_launch(), k_add<<<nb((int64_t)num * kH), 256, 0, st>>>((int64_t)num * kH, H, Upd, H2);
      std::swap(H, H2);
    }
    const float* W = Pm + L.w_o1;
    g.gemm(num, kH, kH, H, kH, W, kH, P, kH, nullptr, 0);
    g.gemm(num, kH, kH, H, kH, W + kH * kH, kH, Q, kH, nullptr, 0);
    ::ibem::count_launch(), k_edge_out<<<nb(E * 32, 256), 256, 0, st>>>(E, nbr, P, Q, ef, W + 2 * kH * kH, Pm + L.b_o1,
                                                                          Pm + L.w_o2, Pm + L.b_o2, w);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) s = cuda_fail(le, "gnn forward");
  }
  free_async(H, st);
  free_async(H2, st);
  free_async(P, st);
  free_async(Q, st);
  free_async(Upd, st);
  free_async(Uin, st);
  return s;
}

ibem_status loss_grad(Net& net, const int* nbr, const float* xn, const float* ef, int nrhs, const float* z,
                      const float* u, const float* P, double* loss_dev, float* G) {
  ibem_status s = net.forward(nbr, xn, ef, P);
  if (s) return s;
  IBEM_CUDA(cudaMemsetAsync(loss_dev, 0, sizeof(double), net.st));
  ::ibem::count_launch(), k_loss<<<nb(net.num, 4), 128, 0, net.st>>>(net.num, nrhs, nbr, net.w, z, u, loss_dev, net.dw);
  IBEM_LAUNCH_CHECK("gnn loss");
  if (G) s = net.backward(nbr, xn, P, G);
  return s;
}

struct Prepared {
  cudaStream_t st = nullptr;
  std::vector<void*> mem;
  int* nbr = nullptr;
  float *xn = nullptr, *ef = nullptr, *z = nullptr, *u = nullptr, *B = nullptr;
  ~Prepared() {
    for (void* p : mem) free_async(p, st);
  }
  template <class T>
  ibem_status buf(T*& p, int64_t n) {
    IBEM_CUDA(alloc_async((void**)&p, sizeof(T) * std::max<int64_t>(n, 1), st));
    mem.push_back(p);
    return IBEM_OK;
  }
};

}  // namespace

int64_t gnn_param_count() { return Layout().total; }

ibem_status gnn_knn(const MfBatch& b, int* nbr, cudaStream_t st) {
  ProfScope ps(PROF_KNN, st);
  ::ibem::count_launch(), k_knn<<<nb((int64_t)b.num * 32, 128), 128, 0, st>>>(b.num, b.seg_of, b.seg_begin, b.cen, nbr);
  IBEM_LAUNCH_CHECK("knn");
  return IBEM_OK;
}

ibem_status gnn_features(const MfBatch& b, const int* nbr, float* xn, float* ef, cudaStream_t st) {
  std::vector<MatFeat> h(b.nseg);
  for (int s = 0; s < b.nseg; ++s) {
    const ibem_material& m = b.mats_h[s];
    h[s] = {(float)(m.E1 / (10.0 * m.E0)), (float)m.nu0, (float)m.nu1};
  }
  MatFeat* d = nullptr;
  IBEM_CUDA(alloc_async((void**)&d, sizeof(MatFeat) * b.nseg, st));
  IBEM_CUDA(cudaMemcpyAsync(d, h.data(), sizeof(MatFeat) * b.nseg, cudaMemcpyHostToDevice, st));
  ::ibem::count_launch(), k_features<<<nb((int64_t)b.num * kKnn), 256, 0, st>>>(b.num, b.seg_of, d, b.cen, b.rad, nbr, xn, ef);
  const cudaError_t e = cudaStreamSynchronize(st);   // the host array h is read by the copy above
  free_async(d, st);
  if (e != cudaSuccess) return cuda_fail(e, "gnn features");
  IBEM_LAUNCH_CHECK("gnn features");
  return IBEM_OK;
}

ibem_status gnn_edge_corrections(const MfBatch& b, const int* nbr, const float* B, const float* wa, float* D, float* Q,
                                 int nrhs, const float* r, float* u, cudaStream_t st) {
  const int64_t E = (int64_t)b.num * kKnn;
  ProfScope ps(PROF_EDGE, st);
  ::ibem::count_launch(), k_edge_corr<<<(unsigned)E, 64, 0, st>>>(b.num, nbr, b.seg_of, b.matf, b.cen, b.rad, B, wa, D,
                                                                  Q, nrhs, r, b.N, u);
  IBEM_LAUNCH_CHECK("edge corrections");
  return IBEM_OK;
}

ibem_status gnn_forward_weights(int num, const int* nbr, const float* xn, const float* ef, const float* params, float* w,
                                cudaStream_t st) {  // w: num * kKnn x kGnnOut
  ProfScope ps(PROF_GNN_FWD, st);
  return forward_fast(num, nbr, xn, ef, params, w, st);
}

__global__ void k_fill1(int64_t n, float* __restrict__ p) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = 1.f;
}

ibem_status mf_neighbour_precond(const MfBatch& b, const float* params, MfPrecond& pc, cudaStream_t st) {
  Prepared pr;
  pr.st = st;
  const int64_t E = (int64_t)b.num * kKnn;
  IBEM_CUDA(alloc_async((void**)&pc.nbr, sizeof(int) * E, st));
  IBEM_CUDA(alloc_async((void**)&pc.Q, sizeof(float) * E * kMfNu * kMfNu, st));
  pr.nbr = pc.nbr;
  float* wa = nullptr;
  ibem_status s = pr.buf(wa, E * kGnnOut);
  if (!s) s = pr.buf(pr.B, (int64_t)b.num * kMfNu * kMfNu);
  if (!s) s = gnn_knn(b, pc.nbr, st);
  if (!s && params) {
    if (!s) s = pr.buf(pr.xn, (int64_t)b.num * kGnnNodeF);
    if (!s) s = pr.buf(pr.ef, E * kGnnEdgeF);
    if (!s) s = gnn_features(b, pc.nbr, pr.xn, pr.ef, st);
    if (!s) s = gnn_forward_weights(b.num, pc.nbr, pr.xn, pr.ef, params, wa, st);
  } else if (!s) {
    ::ibem::count_launch(), k_fill1<<<nb(E * kGnnOut), 256, 0, st>>>(E * kGnnOut, wa);
  }
  if (!s) IBEM_CUDA(cudaMemcpyAsync(pr.B, pc.D, sizeof(float) * b.num * kMfNu * kMfNu, cudaMemcpyDeviceToDevice, st));
  if (!s) s = gnn_edge_corrections(b, pc.nbr, pr.B, wa, pc.D, pc.Q, 0, nullptr, nullptr, st);
  return s;
}

namespace {
ibem_status prepare(const MfBatch& b, int nrhs, const double* r, const double* e, Prepared& pr, int* nbr_out,
                    float* xn_out, float* ef_out, float* z_out, float* u_out, cudaStream_t st) {
  const int64_t E = (int64_t)b.num * kKnn;
  ibem_status s = IBEM_OK;
  pr.nbr = nbr_out;
  pr.xn = xn_out;
  pr.ef = ef_out;
  pr.z = z_out;
  pr.u = u_out;
  if (!pr.nbr) s = pr.buf(pr.nbr, E);
  if (!s && !pr.xn) s = pr.buf(pr.xn, (int64_t)b.num * kGnnNodeF);
  if (!s && !pr.ef) s = pr.buf(pr.ef, E * kGnnEdgeF);
  if (!s && nrhs > 0 && !pr.z) s = pr.buf(pr.z, (int64_t)nrhs * b.N);
  if (!s && nrhs > 0 && !pr.u) s = pr.buf(pr.u, (int64_t)nrhs * E * 2 * kMfNu);
  if (!s) s = pr.buf(pr.B, (int64_t)b.num * kMfNu * kMfNu);
  if (!s) s = gnn_knn(b, pr.nbr, st);
  if (!s) s = gnn_features(b, pr.nbr, pr.xn, pr.ef, st);
  if (!s && nrhs > 0) {
    s = mf_block_jacobi(b, pr.B, st);
    double* sc = nullptr;
    float* rf = nullptr;
    if (!s) s = pr.buf(sc, 1);
    if (!s) s = pr.buf(rf, (int64_t)nrhs * b.N);
    if (!s) {
      IBEM_CUDA(cudaMemsetAsync(sc, 0, sizeof(double), st));
      ::ibem::count_launch(), k_sumsq<<<256, 256, 0, st>>>((int64_t)nrhs * b.N, e, sc);
      ::ibem::count_launch(), k_rsqrt_inplace<<<1, 1, 0, st>>>(sc);
      for (int q = 0; q < nrhs; ++q)
        ::ibem::count_launch(), k_sample_z<<<nb(b.N), 256, 0, st>>>(b.num, pr.B, r + (int64_t)q * b.N, e + (int64_t)q * b.N,
                                                                     sc, pr.z + (int64_t)q * b.N, rf + (int64_t)q * b.N);
      IBEM_LAUNCH_CHECK("gnn samples");
      s = gnn_edge_corrections(b, pr.nbr, pr.B, nullptr, nullptr, nullptr, nrhs, rf, pr.u, st);
    }
  }
  if (!s) IBEM_CUDA(cudaStreamSynchronize(st));
  return s;
}
}  // namespace

}  // namespace ibem

// ------------------------------------------------------------------ C ABI
using namespace ibem;

extern "C" int64_t ibem_gnn_param_count(void) { return gnn_param_count(); }

extern "C" ibem_status ibem_gnn_init_params(float* params_dev, uint64_t seed, void* stream) {
  if (!params_dev) return fail(IBEM_ERR_ARG, "gnn_init_params: null");
  const Layout L;
  std::vector<float> h(L.total, 0.f);
  std::mt19937_64 rng(seed);
  auto fill = [&](int64_t off, int64_t fan_in, int64_t n) {
    const double a = 1.0 / std::sqrt((double)fan_in);
    std::uniform_real_distribution<double> U(-a, a);
    for (int64_t i = 0; i < n; ++i) h[off + i] = (float)U(rng);
  };
  fill(L.w_in, kGnnNodeF, (int64_t)kGnnNodeF * kH);
  fill(L.b_in, kGnnNodeF, kH);
  for (int l = 0; l < kGnnLayers; ++l) {
    fill(L.w_m[l], kEin, (int64_t)kEin * kH);
    fill(L.b_m[l], kEin, kH);
    fill(L.w_u[l], kUin, (int64_t)kUin * kH);
    fill(L.b_u[l], kUin, kH);
  }
  fill(L.w_o1, kEin, (int64_t)kEin * kH);
  fill(L.b_o1, kEin, kH);
  // output layer zero: the untrained network gives w = 0, i.e. block-Jacobi
  cudaStream_t st = as_stream(stream);
  IBEM_CUDA(cudaMemcpyAsync(params_dev, h.data(), sizeof(float) * L.total, cudaMemcpyHostToDevice, st));
  IBEM_CUDA(cudaStreamSynchronize(st));
  return IBEM_OK;
}

extern "C" ibem_status ibem_gnn_prepare(const ibem_e3d_batch* batch, int nrhs, const double* r_hat_dev,
                                        const double* e_hat_dev, int* nbr_dev, float* node_feat_dev,
                                        float* edge_feat_dev, float* z_dev, float* u_dev, void* stream) {
  if (batch && batch->axes_dev) return fail(IBEM_ERR_ARG, "matrix-free products and the learned preconditioner take spheres; solve ellipsoid batches with ibem_e3d_batch_dense_solve");
  if (!batch || !nbr_dev || !node_feat_dev || !edge_feat_dev || nrhs < 0) return fail(IBEM_ERR_ARG, "gnn_prepare: bad arguments");
  if (nrhs > 0 && (!r_hat_dev || !e_hat_dev || !z_dev || !u_dev)) return fail(IBEM_ERR_ARG, "gnn_prepare: samples");
  cudaStream_t st = as_stream(stream);
  MfBatch b;
  ibem_status s = mf_batch_init(b, *batch, st);
  if (!s) {
    Prepared pr;
    pr.st = st;
    // the caller's buffers are used in place (prepare allocates only what is missing)
    s = prepare(b, nrhs, r_hat_dev, e_hat_dev, pr, nbr_dev, node_feat_dev, edge_feat_dev, z_dev, u_dev, st);
  }
  mf_batch_free(b);
  return s;
}

extern "C" ibem_status ibem_gnn_loss_grad(int num, const int* nbr_dev, const float* node_feat_dev,
                                          const float* edge_feat_dev, int nrhs, const float* z_dev, const float* u_dev,
                                          const float* params_dev, double* loss, float* grad_dev, void* stream) {
  if (num <= 0 || !nbr_dev || !node_feat_dev || !edge_feat_dev || nrhs <= 0 || !z_dev || !u_dev || !params_dev || !loss)
    return fail(IBEM_ERR_ARG, "gnn_loss_grad: bad arguments");
  Net net;
  net.num = num;
  net.E = (int64_t)num * kKnn;
  net.st = as_stream(stream);
  ibem_status s = net.alloc(true);
  double* ld = nullptr;
  if (!s) {
    const cudaError_t e = cudaMalloc(&ld, sizeof(double));
    if (e != cudaSuccess) s = cuda_fail(e, "gnn_loss_grad");
  }
  if (!s) s = loss_grad(net, nbr_dev, node_feat_dev, edge_feat_dev, nrhs, z_dev, u_dev, params_dev, ld, grad_dev);
  if (!s) {
    cudaMemcpyAsync(loss, ld, sizeof(double), cudaMemcpyDeviceToHost, net.st);
    const cudaError_t e = cudaStreamSynchronize(net.st);
    if (e != cudaSuccess) s = cuda_fail(e, "gnn_loss_grad");
  }
  cudaFree(ld);
  return s;
}

extern "C" ibem_status ibem_gnn_edge_weights(int num, const int* nbr_dev, const float* node_feat_dev,
                                             const float* edge_feat_dev, const float* params_dev, float* w_dev,
                                             void* stream) {
  if (num <= 0 || !nbr_dev || !node_feat_dev || !edge_feat_dev || !params_dev || !w_dev)
    return fail(IBEM_ERR_ARG, "gnn_edge_weights: bad arguments");
  return gnn_forward_weights(num, nbr_dev, node_feat_dev, edge_feat_dev, params_dev, w_dev, as_stream(stream));
}

extern "C" ibem_status ibem_gnn_adamw(int64_t n, float* params_dev, const float* grad_dev, float* m_dev, float* v_dev,
                                      int step, float lr, float beta1, float beta2, float eps, float weight_decay,
                                      void* stream) {
  if (n <= 0 || !params_dev || !grad_dev || !m_dev || !v_dev || step < 1) return fail(IBEM_ERR_ARG, "gnn_adamw: bad arguments");
  const float c1 = 1.f - std::pow(beta1, (float)step), c2 = 1.f - std::pow(beta2, (float)step);
  ::ibem::count_launch(), k_adamw<<<nb(n), 256, 0, as_stream(stream)>>>(n, params_dev, grad_dev, m_dev, v_dev, lr, beta1,
                                                                       beta2, eps, weight_decay, c1, c2);
  IBEM_LAUNCH_CHECK("adamw");
  return IBEM_OK;
}

extern "C" ibem_status ibem_gnn_train(const ibem_e3d_batch* batch, int nrhs, const double* r_hat_dev,
                                      const double* e_hat_dev, float* params_dev, int steps, float lr,
                                      float weight_decay, double* loss_hist, void* stream) {
  if (batch && batch->axes_dev) return fail(IBEM_ERR_ARG, "matrix-free products and the learned preconditioner take spheres; solve ellipsoid batches with ibem_e3d_batch_dense_solve");
  if (!batch || nrhs <= 0 || !r_hat_dev || !e_hat_dev || !params_dev || steps < 0 || !loss_hist)
    return fail(IBEM_ERR_ARG, "gnn_train: bad arguments");
  cudaStream_t st = as_stream(stream);
  MfBatch b;
  ibem_status s = mf_batch_init(b, *batch, st);
  if (s) return s;
  {
    Prepared pr;
    pr.st = st;
    s = prepare(b, nrhs, r_hat_dev, e_hat_dev, pr, nullptr, nullptr, nullptr, nullptr, nullptr, st);
    Net net;
    net.num = b.num;
    net.E = (int64_t)b.num * kKnn;
    net.st = st;
    if (!s) s = net.alloc(true);
    const int64_t np = net.L.total;
    float *G = nullptr, *M1 = nullptr, *M2 = nullptr;
    double* ld = nullptr;
    if (!s) s = pr.buf(G, np);
    if (!s) s = pr.buf(M1, np);
    if (!s) s = pr.buf(M2, np);
    if (!s) s = pr.buf(ld, 1);
    if (!s) {
      cudaMemsetAsync(M1, 0, sizeof(float) * np, st);
      cudaMemsetAsync(M2, 0, sizeof(float) * np, st);
    }
    for (int it = 0; it <= steps && !s; ++it) {
      s = loss_grad(net, pr.nbr, pr.xn, pr.ef, nrhs, pr.z, pr.u, params_dev, ld, it < steps ? G : nullptr);
      if (s) break;
      cudaMemcpyAsync(loss_hist + it, ld, sizeof(double), cudaMemcpyDeviceToHost, st);
      if (it < steps) s = ibem_gnn_adamw(np, params_dev, G, M1, M2, it + 1, lr, 0.9f, 0.999f, 1e-8f, weight_decay, stream);
    }
    if (!s) {
      const cudaError_t e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) s = cuda_fail(e, "gnn_train");
    }
  }
  mf_batch_free(b);
  return s;
}
