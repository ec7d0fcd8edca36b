// Matrix-free solves of the layout-24 sphere systems, one realisation or a batch of them.
//
// The pair blocks that ibem_e3d_pair_blocks stores (integratorElastic3D.cpp:341-567,
// orders 0 and 1) are never formed: their products with the coefficients are evaluated
// as the contracted strain and its gradient (mf_contract.cuh):
//   k_mf_apply_f32  As x in FP32 on the scaled system (mf.h), the GMRES operator;
//   k_mf_apply_f64  As x in FP64, the refinement residual Dr b - As xs; for the residual
//                   that decides convergence it takes only the source chunks near each
//                   warp's targets and k_mf_apply_df the far ones (both visit particles in
//                   the Morton order of their centres, so warps and chunks are compact).
// One thread per target particle s, 128 consecutive targets of one realisation per CTA;
// the CTA's source particles h (a slice of the realisation, gridDim.y slices) are staged
// through shared memory in chunks with their coefficients, and every thread sums the
// pair products in registers.  Slices add their partial sums atomically.
//
// Solver: iterative refinement x += Dc d; each correction d solves As d = Dr r with a
// restarted FP32 GMRES right-preconditioned by a block-sparse P (block-Jacobi, Neumann or
// learned); the residual that drives the next correction is a double-float product
// (k_mf_apply_df, ~48 bits) and the one that decides convergence the split product.  All
// realisations of a batch run in lock step (per-realisation Arnoldi: segmented dot
// products, Hessenberg updates and Givens rotations on the device, one thread per
// realisation), stopping each realisation on its own residual estimate.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <map>
#include <mutex>
#include <thread>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gen_sphere24.cuh"
#include "mf.h"
#include "dfnum.cuh"
#include "mf_contract.cuh"
#include "prof.h"
#include "solver.h"

namespace ibem {
namespace {

constexpr int kMfThreads = 128;
constexpr int kMfChunk = 32;
constexpr double kMfFarRadii = 4.0;   // near / far split of the deciding residual
constexpr int kMfSplitMin = 1280;     // smallest realisation (particles) that uses the split
constexpr int kMfSkipMin = 5000;      // from here the far pass skips near sources (256-thread CTAs)

// sink of a generated block: acc[r] += v * x[c] (r, c compile-time constants after inlining)
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
template <class T>
struct MvSink {
  T (&acc)[kMfNu];
  const T* __restrict__ xs;
  __device__ __forceinline__ void operator()(int r, int c, T v) const { acc[r] = fma_t(v, xs[c], acc[r]); }
};

// One work item of the FP32 product: the TT targets of a tile against source slice `slice`
// of `nslice` of its realisation (TT = blockDim.x, the tile shape the autotuner picks).
template <int TT>
__device__ __forceinline__ void mf_f32_item(const MfTile t, int slice, int nslice, const int* __restrict__ seg_begin,
                                            const int* __restrict__ mask, int mask_on,
                                            const float4* __restrict__ gh, const float4* __restrict__ gl,
                                            const SphMatF* __restrict__ mats, const float* __restrict__ x,
                                            float* __restrict__ y, float4* sgh, float4* sgl, float* sx) {
  if (mask && mask[t.seg] != mask_on) return;  // realisation left out of this product
  const int hb0 = seg_begin[t.seg], he0 = seg_begin[t.seg + 1];
  const int per = (he0 - hb0 + nslice - 1) / nslice;
  const int hb = hb0 + slice * per, he = min(he0, hb + per);
  if (hb >= he) return;
  const int s = t.s0 + threadIdx.x;
  const bool act = threadIdx.x < t.ns;
  const SphMatF mc = mats[t.seg];
  const float4 ph = act ? gh[s] : make_float4(0.f, 0.f, 0.f, 1.f);
  const float4 pl = act ? gl[s] : make_float4(0.f, 0.f, 0.f, 1.f);
  float acc[kMfNu];
#pragma unroll
  for (int r = 0; r < kMfNu; ++r) acc[r] = 0.f;
  for (int h0 = hb; h0 < he; h0 += kMfChunk) {
    const int nh = min(kMfChunk, he - h0);
    __syncthreads();
    for (int i = threadIdx.x; i < nh; i += TT) {
      sgh[i] = gh[h0 + i];
      sgl[i] = gl[h0 + i];
    }
    for (int i = threadIdx.x; i < nh * kMfNu; i += TT) sx[i] = x[(int64_t)kMfNu * h0 + i];
    __syncthreads();
    if (!act) continue;
#pragma unroll 1
    for (int hh = 0; hh < nh; ++hh) {
      const float4 qh = sgh[hh], ql = sgl[hh];
      const float ia = ql.w;
      // offset from the source centre in units of its radius (hi/lo parts keep ~48 bits)
      const float x0 = ((ph.x - qh.x) + (pl.x - ql.x)) * ia;
      const float x1 = ((ph.y - qh.y) + (pl.y - ql.y)) * ia;
      const float x2 = ((ph.z - qh.z) + (pl.z - ql.z)) * ia;
      sph_pair_apply24<float, true>(x0, x1, x2, 1.f, 0.f, 0.f, mc.tn1, mc.tn2, sx + kMfNu * hh, ph.w * ia, acc);
    }
  }
  if (!act) return;
  float yv[kMfNu];
  sph_pair_map24<float>(acc, mc.kmu, mc.klam, yv);
  if (s >= hb && s < he) {  // the slice holding the target adds its self term (C0 / mu0)
    MvSink<float> sk{yv, x + (int64_t)kMfNu * s};
    sph_self24f(mc, sk);
  }
  float* o = y + (int64_t)kMfNu * s;
#pragma unroll
  for (int r = 0; r < kMfNu; ++r) atomicAdd(o + r, yv[r]);
}

// one CTA per (tile, slice): grid (ntiles, nslice)
template <int TT>
__global__ void __launch_bounds__(TT)
    k_mf_apply_f32(const MfTile* __restrict__ tiles, const int* __restrict__ seg_begin,
                   const int* __restrict__ mask, int mask_on,
                   const float4* __restrict__ gh, const float4* __restrict__ gl,
                   const SphMatF* __restrict__ mats, const float* __restrict__ x, float* __restrict__ y) {
  __shared__ float4 sgh[kMfChunk], sgl[kMfChunk];
  __shared__ float sx[kMfChunk * kMfNu];
  mf_f32_item<TT>(tiles[blockIdx.x], blockIdx.y, gridDim.y, seg_begin, mask, mask_on, gh, gl, mats, x, y, sgh, sgl,
                  sx);
}

// persistent form: as many CTAs as fit on the GPU at once walk a work list of (tile,
// slice) pairs sorted by decreasing cost (sources x targets), CTA c taking items c,
// c + gridDim.x, ... (the longest first, so that the realisations of a ragged batch finish
// together)
template <int TT>
__global__ void __launch_bounds__(TT)
    k_mf_apply_f32_persist(const MfTile* __restrict__ tiles, const int2* __restrict__ work, int nwork, int nslice,
                           const int* __restrict__ seg_begin, const int* __restrict__ mask, int mask_on,
                           const float4* __restrict__ gh, const float4* __restrict__ gl,
                           const SphMatF* __restrict__ mats, const float* __restrict__ x, float* __restrict__ y) {
  __shared__ float4 sgh[kMfChunk], sgl[kMfChunk];
  __shared__ float sx[kMfChunk * kMfNu];
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const int2 it = work[w];
    mf_f32_item<TT>(tiles[it.x], it.y, nslice, seg_begin, mask, mask_on, gh, gl, mats, x, y, sgh, sgl, sx);
  }
}

// FP64 product of the scaled system (the refinement residual): the same evaluation as the
// FP32 kernel in double precision, offsets from FP64 centres.
// Split products (the deciding residual): particles are visited in the Morton order of
// their centres within each realisation (perm: position -> particle), so the 32 targets of a
// warp form a compact cluster.  mode 0: every pair; 1: only the sources near the warp's
// targets (within kMfFarRadii of their radius of the targets' bounding box), and the self
// term; 2 and 3: only the far sources, no self term.  The test is per (warp, source) and
// warp-uniform.  The double-float pair code is longer than the instruction cache: warps of
// an SM that run it at different places each fetch their own instructions, and issue fell
// to half when the far pass let every warp skip its own near sources.  So the far pass
// keeps them together: mode 2 (two 128-thread CTAs per SM) evaluates every source of the
// chunk, a warp's near ones against zero coefficients, so every CTA does the same work;
// mode 3 (one 256-thread CTA per SM) skips them, the barrier at each chunk realigning the
// warps of the SM.
__device__ __forceinline__ void warp_box(bool act, double x, double y, double z, double* lo, double* hi) {
  double v[3] = {x, y, z};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double a = act ? v[d] : 1e300, b = act ? v[d] : -1e300;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a = fmin(a, __shfl_xor_sync(0xffffffffu, a, o));
      b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    lo[d] = a;
    hi[d] = b;
  }
}

// whether a source sphere (c, r) lies beyond kMfFarRadii of its radius from the box of the
// warp's targets: the same for every lane; rounded operations without contraction, so that
// the FP64 and double-float kernels of a split product classify every pair the same way
__device__ __forceinline__ bool source_is_far(const double* wlo, const double* whi, double cx, double cy, double cz,
                                              double r) {
  const double c[3] = {cx, cy, cz};
  double d2 = 0.0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double g = fmax(0.0, fmax(__dadd_rn(wlo[d], -c[d]), __dadd_rn(c[d], -whi[d])));
    d2 = __dadd_rn(d2, __dmul_rn(g, g));
  }
  const double lim = __dmul_rn(kMfFarRadii, r);
  return d2 > __dmul_rn(lim, lim);
}
// The sources of one CTA (blockIdx.y of gridDim.y slices), in chunks of kMfChunk: chunk j
// starts at first + j * step and ends at end at the latest.  The full product (mode 0) takes
// a contiguous range of the realisation; the split ones take every gridDim.y-th chunk from
// blockIdx.y.  In Morton order the near sources of a tile sit in a few neighbouring chunks:
// dealt out in turn, every CTA gets about the average share of them.
struct MfSlice {
  int first, step, end;
  __device__ __forceinline__ bool holds(int p) const {
    return p >= first && p < end && (p - first) % step < kMfChunk;
  }
};
__device__ __forceinline__ MfSlice mf_slice(int hb0, int he0, int mode) {
  const int k = blockIdx.y, ns = gridDim.y;
  if (mode) return {hb0 + kMfChunk * k, kMfChunk * ns, he0};
  const int per = (he0 - hb0 + ns - 1) / ns;
  const int hb = hb0 + k * per;
  return {hb, kMfChunk, min(he0, hb + per)};
}

// Sources of the chunk at h0 (nh of them) that this warp evaluates, as a bit mask (bit i:
// source h0 + i); the same for every lane.  Lane i classifies source i.  Evaluating the
// selected sources in turn keeps the warps of a CTA at the same place in the long
// straight-line pair code (instruction fetches shared), which skipping inside the loop
// would not.
__device__ __forceinline__ unsigned chunk_mask(int mode, bool warp_on, const double* wlo, const double* whi, int h0,
                                               int nh, const int* __restrict__ perm, const double* __restrict__ cen,
                                               const double* __restrict__ rad) {
  const int lane = threadIdx.x & 31;
  bool take = lane < nh;
  if (mode && take) {
    const int h = perm[h0 + lane];
    take = source_is_far(wlo, whi, cen[3 * (int64_t)h], cen[3 * (int64_t)h + 1], cen[3 * (int64_t)h + 2], rad[h]) ==
           (mode >= 2);
  }
  const unsigned m = __ballot_sync(0xffffffffu, take);
  return warp_on ? m : 0u;
}

__global__ void __launch_bounds__(kMfThreads)
    k_mf_apply_f64(const MfTile* __restrict__ tiles, const int* __restrict__ seg_begin,
                   const int* __restrict__ mask, int mask_on,
                   const double* __restrict__ cen, const double* __restrict__ rad,
                   const SphMat* __restrict__ mats, const double* __restrict__ x, double* __restrict__ y,
                   const int* __restrict__ perm, int mode) {
  __shared__ double sc[kMfChunk * 4];
  __shared__ double sx[kMfChunk * kMfNu];
  const MfTile t = tiles[blockIdx.x];
  if (mask && mask[t.seg] != mask_on) return;  // realisation left out of this product
  const MfSlice sl = mf_slice(seg_begin[t.seg], seg_begin[t.seg + 1], mode);
  if (sl.first >= sl.end) return;
  const int pos = t.s0 + threadIdx.x;
  const bool act = threadIdx.x < t.ns;
  const int s = act ? perm[pos] : 0;
  const SphMat mc = mats[t.seg];   // moduli divided by mu0 (scaled system)
  double p0 = 0, p1 = 0, p2 = 0, as = 1;
  if (act) {
    p0 = cen[3 * (int64_t)s];
    p1 = cen[3 * (int64_t)s + 1];
    p2 = cen[3 * (int64_t)s + 2];
    as = rad[s];
  }
  double wlo[3], whi[3];
  warp_box(act, p0, p1, p2, wlo, whi);
  double acc[kMfNu];
#pragma unroll
  for (int r = 0; r < kMfNu; ++r) acc[r] = 0.0;
  const bool warp_on = __any_sync(0xffffffffu, act);
  for (int h0 = sl.first; h0 < sl.end; h0 += sl.step) {
    const int nh = min(kMfChunk, sl.end - h0);
    // mode 1: the sources near the warp's targets; 2: the far ones; 0: all
    unsigned m = chunk_mask(mode, warp_on, wlo, whi, h0, nh, perm, cen, rad);
    if (!__syncthreads_or(m != 0u)) continue;   // no warp of the CTA needs this chunk
    for (int i = threadIdx.x; i < nh; i += blockDim.x) {
      const int h = perm[h0 + i];
      sc[4 * i] = cen[3 * (int64_t)h];
      sc[4 * i + 1] = cen[3 * (int64_t)h + 1];
      sc[4 * i + 2] = cen[3 * (int64_t)h + 2];
      sc[4 * i + 3] = 1.0 / rad[h];
    }
    for (int i = threadIdx.x; i < nh * kMfNu; i += blockDim.x)
      sx[i] = x[(int64_t)kMfNu * perm[h0 + i / kMfNu] + i % kMfNu];
    __syncthreads();
    if (!act) continue;
#pragma unroll 1
    for (; m; m &= m - 1u) {
      const int hh = __ffs(m) - 1;
      const double ia = sc[4 * hh + 3];
      const double x0 = (p0 - sc[4 * hh]) * ia, x1 = (p1 - sc[4 * hh + 1]) * ia, x2 = (p2 - sc[4 * hh + 2]) * ia;
      sph_pair_apply24<double, true>(x0, x1, x2, 1.0, 0.0, 0.0, mc.tn1, mc.tn2, sx + kMfNu * hh, as * ia, acc);
    }
  }
  if (!act) return;
  double yv[kMfNu];
  sph_pair_map24<double>(acc, mc.kmu, mc.klam, yv);
  if (sl.holds(pos) && mode < 2) {
    MvSink<double> sk{yv, x + (int64_t)kMfNu * s};
    sph_self24(mc, sk);
  }
  double* o = y + (int64_t)kMfNu * s;
#pragma unroll
  for (int r = 0; r < kMfNu; ++r) atomicAdd(o + r, yv[r]);
}

// The scaled product in double-float arithmetic (~48 bits): the residual that drives a
// refinement step (the final residual, which decides convergence, is the FP64 kernel's).
// Centres, inverse radii and coefficients are staged as double-float pairs.
struct DfSink {
  DF (&acc)[kMfNu];
  const double* __restrict__ xs;
  __device__ __forceinline__ void operator()(int r, int c, double v) const { acc[r] += DF(v) * DF(xs[c]); }
};

template <int TT>
__global__ void __launch_bounds__(TT)
    k_mf_apply_df(const MfTile* __restrict__ tiles, const int* __restrict__ seg_begin,
                   const int* __restrict__ mask, int mask_on,
                  const double* __restrict__ cen, const double* __restrict__ rad,
                  const SphMat* __restrict__ mats, const double* __restrict__ x, double* __restrict__ y,
                  const int* __restrict__ perm, int mode) {
  __shared__ DF sc[kMfChunk * 4];
  __shared__ DF sx[kMfChunk * kMfNu];
  __shared__ DF szero[kMfNu];   // the coefficients of a skipped source in mode 2
  if (threadIdx.x < kMfNu) szero[threadIdx.x] = DF();
  const MfTile t = tiles[blockIdx.x];
  if (mask && mask[t.seg] != mask_on) return;  // realisation left out of this product
  const MfSlice sl = mf_slice(seg_begin[t.seg], seg_begin[t.seg + 1], mode);
  if (sl.first >= sl.end) return;
  const int pos = t.s0 + threadIdx.x;
  const bool act = threadIdx.x < t.ns;
  const int s = act ? perm[pos] : 0;
  const SphMat mc = mats[t.seg];   // moduli divided by mu0 (scaled system)
  DF p0, p1, p2, as(1.0);
  double q0 = 0, q1 = 0, q2 = 0;
  if (act) {
    q0 = cen[3 * (int64_t)s];
    q1 = cen[3 * (int64_t)s + 1];
    q2 = cen[3 * (int64_t)s + 2];
    p0 = DF(q0);
    p1 = DF(q1);
    p2 = DF(q2);
    as = DF(rad[s]);
  }
  double wlo[3], whi[3];
  warp_box(act, q0, q1, q2, wlo, whi);
  const DF tn1(mc.tn1), tn2(mc.tn2);
  DF acc[kMfNu];
  const bool warp_on = __any_sync(0xffffffffu, act);
  for (int h0 = sl.first; h0 < sl.end; h0 += sl.step) {
    const int nh = min(kMfChunk, sl.end - h0);
    unsigned m = chunk_mask(mode, warp_on, wlo, whi, h0, nh, perm, cen, rad);
    if (!__syncthreads_or(m != 0u)) continue;   // no warp of the CTA needs this chunk
    for (int i = threadIdx.x; i < nh; i += blockDim.x) {
      const int h = perm[h0 + i];
      sc[4 * i] = DF(cen[3 * (int64_t)h]);
      sc[4 * i + 1] = DF(cen[3 * (int64_t)h + 1]);
      sc[4 * i + 2] = DF(cen[3 * (int64_t)h + 2]);
      sc[4 * i + 3] = DF(1.0 / rad[h]);
    }
    for (int i = threadIdx.x; i < nh * kMfNu; i += blockDim.x)
      sx[i] = DF(x[(int64_t)kMfNu * perm[h0 + i / kMfNu] + i % kMfNu]);
    __syncthreads();
    if (!act) continue;
    const unsigned all = nh >= 32 ? 0xffffffffu : (1u << nh) - 1u;
#pragma unroll 1
    for (unsigned k = mode == 2 ? all : m; k; k &= k - 1u) {
      const int hh = __ffs(k) - 1;
      const DF* xs = (m >> hh) & 1u ? sx + kMfNu * hh : szero;
      const DF ia = sc[4 * hh + 3];
      const DF x0 = (p0 - sc[4 * hh]) * ia, x1 = (p1 - sc[4 * hh + 1]) * ia, x2 = (p2 - sc[4 * hh + 2]) * ia;
      sph_pair_apply24<DF, true>(x0, x1, x2, DF(1.0), DF(), DF(), tn1, tn2, xs, as * ia, acc);
    }
  }
  if (!act) return;
  DF yv[kMfNu];
  sph_pair_map24<DF>(acc, DF(mc.kmu), DF(mc.klam), yv);
  if (sl.holds(pos) && mode < 2) {
    DfSink sk{yv, x + (int64_t)kMfNu * s};
    sph_self24(mc, sk);
  }
  double* o = y + (int64_t)kMfNu * s;
#pragma unroll
  for (int r = 0; r < kMfNu; ++r) atomicAdd(o + r, df_value(yv[r]));
}

// Geometry in the FP32 layout, scalings, segment of every particle.
__global__ void k_mf_prep(int nu, int num, const double* __restrict__ cen, const double* __restrict__ rad,
                          const int* __restrict__ seg_of, const SphMat* __restrict__ mats, float4* __restrict__ gh,
                          float4* __restrict__ gl, double* __restrict__ dr, double* __restrict__ dc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= num) return;
  float hi[3], lo[3];
  for (int k = 0; k < 3; ++k) {
    const double c = cen[3 * (int64_t)p + k];
    hi[k] = (float)c;
    lo[k] = (float)(c - (double)hi[k]);
  }
  const double a = rad[p];
  gh[p] = make_float4(hi[0], hi[1], hi[2], (float)a);
  gl[p] = make_float4(lo[0], lo[1], lo[2], (float)(1.0 / a));
  const double imu = 1.0 / mats[seg_of[p]].mu0;
  // rows / columns of eigenstrain order o (0: 6, 1: 18, 2: 36 unknowns): a^o / mu0, a^-o
  for (int r = 0; r < nu; ++r) {
    const int o = r < 6 ? 0 : (r < 24 ? 1 : 2);
    const double ao = o == 0 ? 1.0 : (o == 1 ? a : a * a);
    dr[(int64_t)nu * p + r] = ao * imu;
    dc[(int64_t)nu * p + r] = 1.0 / ao;
  }
}

// Scaled diagonal block (FP64, x = 0, unit sphere, moduli / mu0) inverted by Gauss-Jordan
// with partial pivoting; one CTA of 32 threads per realisation: in the scaled system a
// sphere's own block depends on the materials only, so every sphere of a realisation shares
// it (k_bcast_blocks copies it to each).
__global__ void __launch_bounds__(32) k_block_jacobi(const SphMat* __restrict__ mats, float* __restrict__ P) {
  __shared__ double M[kMfNu][2 * kMfNu + 1];
  const int p = blockIdx.x;   // realisation
  const int t = threadIdx.x;
  for (int i = t; i < kMfNu * 2 * kMfNu; i += 32) {
    const int r = i / (2 * kMfNu), c = i % (2 * kMfNu);
    M[r][c] = (c >= kMfNu && c - kMfNu == r) ? 1.0 : 0.0;
  }
  __syncthreads();
  if (t == 0) {
    SphMat mc = mats[p];
    const double s = 1.0 / mc.mu0;
    mc.kmu *= s;
    mc.klam *= s;
    mc.lam0 *= s;
    mc.mu0 = 1.0;
    struct Put {
      double (*M)[2 * kMfNu + 1];
      __device__ void operator()(int r, int c, double v) const { M[r][c] += v; }
    } put{M};
    sph_block24_c0_r0(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_block24_c1_r0(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_block24_c0_r1(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_block24_c1_r1(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_self24(mc, put);
  }
  __syncthreads();
  __shared__ int piv;
  __shared__ double f[kMfNu];
  for (int k = 0; k < kMfNu; ++k) {
    if (t == 0) {
      int best = k;
      for (int r = k + 1; r < kMfNu; ++r)
        if (fabs(M[r][k]) > fabs(M[best][k])) best = r;
      piv = best;
    }
    __syncthreads();
    const int pr = piv;
    if (pr != k)
      for (int c = t; c < 2 * kMfNu; c += 32) {
        const double v = M[k][c];
        M[k][c] = M[pr][c];
        M[pr][c] = v;
      }
    __syncthreads();
    const double d = M[k][k];
    const double id = d != 0.0 ? 1.0 / d : 0.0;
    __syncthreads();
    for (int c = t; c < 2 * kMfNu; c += 32) M[k][c] *= id;
    if (t < kMfNu) f[t] = M[t][k];  // column k of the other rows (row k is being scaled, unused)
    __syncthreads();
    for (int i = t; i < kMfNu * 2 * kMfNu; i += 32) {
      const int r = i / (2 * kMfNu), c = i % (2 * kMfNu);
      if (r != k) M[r][c] -= f[r] * M[k][c];
    }
    __syncthreads();
  }
  float* o = P + (int64_t)kMfNu * kMfNu * p;
  for (int i = t; i < kMfNu * kMfNu; i += 32) o[i] = (float)M[i / kMfNu][kMfNu + i % kMfNu];
}

// P[p] = Pseg[seg_of[p]] (24 x 24 blocks, float4 copies)
__global__ void k_bcast_blocks(int num, const int* __restrict__ seg_of, const float* __restrict__ Pseg,
                               float* __restrict__ P) {
  constexpr int kQ = kMfNu * kMfNu / 4;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)num * kQ) return;
  const int64_t p = t / kQ;
  const int q = (int)(t % kQ);
  reinterpret_cast<float4*>(P)[t] = reinterpret_cast<const float4*>(Pseg)[(int64_t)seg_of[p] * kQ + q];
}

// z = P v for the block-sparse preconditioner: z_p = D_p v_p + sum_slot Q_(p,slot) v_nbr;
// one thread per row (24 x 24 row-major blocks, float4 loads)
__device__ __forceinline__ float dot24(const float* __restrict__ a, const float* __restrict__ b) {
  const float4* x = reinterpret_cast<const float4*>(a);
  const float4* y = reinterpret_cast<const float4*>(b);
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kMfNu / 4; ++c) {
    const float4 u = x[c], v = y[c];
    s = fmaf(u.x, v.x, fmaf(u.y, v.y, fmaf(u.z, v.z, fmaf(u.w, v.w, s))));
  }
  return s;
}
// kdev (graph-captured Arnoldi steps): v is column *kdev of a basis with column stride vstride
__global__ void k_precond_apply(int num, const float* __restrict__ D, const float* __restrict__ Q,
                                const int* __restrict__ nbr, const float* __restrict__ v, float* __restrict__ z,
                                const int* __restrict__ kdev = nullptr, int64_t vstride = 0) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)num * kMfNu) return;
  if (kdev) v += (int64_t)(*kdev) * vstride;
  const int64_t p = t / kMfNu;
  const int r = (int)(t % kMfNu);
  float s = dot24(D + t * kMfNu, v + p * kMfNu);
  if (Q) {
    for (int k = 0; k < kKnn; ++k) {
      const int j = nbr[p * kKnn + k];
      if (j >= 0) s += dot24(Q + ((p * kKnn + k) * kMfNu + r) * kMfNu, v + (int64_t)j * kMfNu);
    }
  }
  z[t] = s;
}

// out[seg * ldo + j] += sum over the segment's rows of V_j[row] * w[row], j < nv (+ *kdev).
// grid (nseg, splits); a CTA of 256 threads holds up to 8 rows per thread in registers.
constexpr int kDotRows = 8, kDotThreads = 256;
template <class TV>
__global__ void __launch_bounds__(kDotThreads)
    k_seg_dots(int nu, const int* __restrict__ seg_begin, int nv, const TV* __restrict__ V, int64_t ldv,
               const TV* __restrict__ w, double* __restrict__ out, int ldo, const int* __restrict__ kdev = nullptr) {
  if (kdev) nv += *kdev;
  const int seg = blockIdx.x;
  const int64_t r0 = (int64_t)nu * seg_begin[seg], r1 = (int64_t)nu * seg_begin[seg + 1];
  const int64_t base = r0 + (int64_t)blockIdx.y * kDotThreads * kDotRows;
  if (base >= r1) return;
  TV wr[kDotRows];
#pragma unroll
  for (int i = 0; i < kDotRows; ++i) {
    const int64_t r = base + threadIdx.x + (int64_t)i * kDotThreads;
    wr[i] = r < r1 ? w[r] : TV(0);
  }
  __shared__ double red[kDotThreads / 32];
  for (int j = 0; j < nv; ++j) {
    const TV* vj = V + (int64_t)j * ldv;
    double s = 0;
#pragma unroll
    for (int i = 0; i < kDotRows; ++i) {
      const int64_t r = base + threadIdx.x + (int64_t)i * kDotThreads;
      if (r < r1) s += (double)vj[r] * (double)wr[i];
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0;
      for (int k = 0; k < kDotThreads / 32; ++k) tot += red[k];
      atomicAdd(out + (int64_t)seg * ldo + j, tot);
    }
    __syncthreads();
  }
}

// w[row] -= sum_j h[seg(row) * ldh + j] V_j[row], j < nv (+ *kdev)
__global__ void k_seg_sub(int nu, int64_t N, const int* __restrict__ seg_of, int nv, const float* __restrict__ V, int64_t ldv,
                          const double* __restrict__ h, int ldh, float* __restrict__ w,
                          const int* __restrict__ kdev = nullptr) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= N) return;
  if (kdev) nv += *kdev;
  const double* hs = h + (int64_t)seg_of[r / nu] * ldh;
  float s = w[r];
  for (int j = 0; j < nv; ++j) s -= (float)hs[j] * V[(int64_t)j * ldv + r];
  w[r] = s;
}

// y[row] (+)= scale[seg(row)] * x[row] (FP32 <- FP64 / FP32); with kdev, y is column
// *kdev + 1 of a basis with column stride ystride
template <class TX, class TY>
__global__ void k_seg_scale(int nu, int64_t N, const int* __restrict__ seg_of, const double* __restrict__ scale,
                            const TX* __restrict__ x, TY* __restrict__ y, int add, const int* __restrict__ kdev = nullptr,
                            int64_t ystride = 0) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= N) return;
  if (kdev) y += (int64_t)(*kdev + 1) * ystride;
  const double v = scale[seg_of[r / nu]] * (double)x[r];
  y[r] = add ? (TY)((double)y[r] + v) : (TY)v;
}

// Per-realisation Arnoldi bookkeeping after step k (one thread per realisation):
// H(:,k) = d1 + d2 (two Gram-Schmidt passes), H(k+1,k) = sqrt(n2), previous Givens
// rotations, the new one, g; inv = 1 / H(k+1,k) for normalising the new basis vector.
struct Krylov {
  double* H;      // nseg x (m+1) x m, row-major per realisation
  double* g;      // nseg x (m+1)
  double* cs;     // nseg x m
  double* sn;
  double* beta;   // nseg
  double* inv;    // nseg
  int* kc;        // nseg: Arnoldi columns accepted in this cycle
  int* active;    // nseg: 1 while the cycle continues for the realisation
  double* d1;     // nseg x (m+1) dot products, pass 1
  double* d2;     // pass 2
  double* n2;     // nseg
  double* yv;     // nseg x m
  double* thr;    // nseg: |g| target of the current GMRES solve (inner_tol * first beta)
  double* est;    // nseg: latest Arnoldi estimate of the GMRES residual norm
  int* nsteps;    // nseg: Arnoldi steps taken while active (reported)
  int* nactive;   // 1
};

__global__ void k_arnoldi_update(int nseg, int m, int k, Krylov K, const int* __restrict__ kdev = nullptr) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  if (kdev) k = *kdev;
  if (!K.active[s]) {
    K.inv[s] = 0.0;
    return;
  }
  double* H = K.H + (int64_t)s * (m + 1) * m;
  double* g = K.g + (int64_t)s * (m + 1);
  double* cs = K.cs + (int64_t)s * m;
  double* sn = K.sn + (int64_t)s * m;
  for (int i = 0; i <= k; ++i) H[i * m + k] = K.d1[(int64_t)s * (m + 1) + i] + K.d2[(int64_t)s * (m + 1) + i];
  // ||w|| after the two Gram-Schmidt passes
  const double hn = sqrt(fmax(K.n2[s], 0.0));
  H[(k + 1) * m + k] = hn;
  for (int i = 0; i < k; ++i) {
    const double a = H[i * m + k], b = H[(i + 1) * m + k];
    H[i * m + k] = cs[i] * a + sn[i] * b;
    H[(i + 1) * m + k] = -sn[i] * a + cs[i] * b;
  }
  const double a = H[k * m + k], b = H[(k + 1) * m + k];
  const double den = hypot(a, b);
  cs[k] = den > 0 ? a / den : 1.0;
  sn[k] = den > 0 ? b / den : 0.0;
  H[k * m + k] = den;
  H[(k + 1) * m + k] = 0.0;
  g[k + 1] = -sn[k] * g[k];
  g[k] = cs[k] * g[k];
  K.kc[s] = k + 1;
  K.nsteps[s] += 1;
  K.est[s] = fabs(g[k + 1]);
  K.inv[s] = hn > 0 ? 1.0 / hn : 0.0;
  if (fabs(g[k + 1]) <= K.thr[s] || hn == 0.0 || k + 1 == m) {
    K.active[s] = 0;
    K.inv[s] = 0.0;
  } else {
    atomicAdd(K.nactive, 1);
  }
}

// y = H(0:kc, 0:kc)^-1 g(0:kc) per realisation (zeros beyond kc)
__global__ void k_hess_solve(int nseg, int m, Krylov K) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const double* H = K.H + (int64_t)s * (m + 1) * m;
  const double* g = K.g + (int64_t)s * (m + 1);
  double* y = K.yv + (int64_t)s * m;
  const int kc = K.kc[s];
  for (int i = m - 1; i >= kc; --i) y[i] = 0.0;
  for (int i = kc - 1; i >= 0; --i) {
    double t = g[i];
    for (int j = i + 1; j < kc; ++j) t -= H[i * m + j] * y[j];
    y[i] = H[i * m + i] != 0.0 ? t / H[i * m + i] : 0.0;
  }
}

// start of a GMRES cycle: beta = sqrt(n2), g = (beta, 0, ...); on the first cycle of a
// solve thr = inner_tol[s] * beta; active while beta > thr and the realisation is not done
__global__ void k_cycle_start(int nseg, int m, Krylov K, const int* __restrict__ done, int first,
                              const double* __restrict__ inner_tol) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const double b = sqrt(fmax(K.n2[s], 0.0));
  K.beta[s] = b;
  if (first) K.thr[s] = inner_tol[s] * b;
  K.est[s] = b;
  double* g = K.g + (int64_t)s * (m + 1);
  for (int i = 0; i <= m; ++i) g[i] = 0.0;
  g[0] = b;
  const int a = (b > K.thr[s] && b > 0.0 && !done[s]) ? 1 : 0;
  K.active[s] = a;
  K.kc[s] = 0;
  K.inv[s] = a ? 1.0 / b : 0.0;
  if (a) atomicAdd(K.nactive, 1);
}

// x[row] += sum_j y[seg][j] V_j[row], j < nv (+ *kdev)
__global__ void k_seg_combine(int nu, int64_t N, const int* __restrict__ seg_of, int nv, const float* __restrict__ V,
                              int64_t ldv, const double* __restrict__ y, int ldy, float* __restrict__ x,
                              const int* __restrict__ kdev = nullptr) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= N) return;
  if (kdev) nv += *kdev;
  const double* ys = y + (int64_t)seg_of[r / nu] * ldy;
  double s = 0;
  for (int j = 0; j < nv; ++j) s += ys[j] * (double)V[(int64_t)j * ldv + r];
  x[r] += (float)s;
}

// end of a graph-captured Arnoldi step: k += 1; the cycle's while loop goes on while
// k < m and some realisation is still active
__global__ void k_step_ctl(int* __restrict__ kdev, const int* __restrict__ nactive, int m,
                           cudaGraphConditionalHandle h) {
  const int k = *kdev + 1;
  *kdev = k;
  cudaGraphSetConditional(h, (k < m && *nactive > 0) ? 1u : 0u);
}

// steps taken by a captured cycle, added up for the launch count
__global__ void k_add_steps(const int* __restrict__ kdev, int* __restrict__ total) { *total += *kdev; }

template <class T>
__global__ void k_fill(T* p, int64_t n, T v) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}
__global__ void k_mul(int64_t n, const double* __restrict__ a, const double* __restrict__ x, double* __restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = a[i] * x[i];
}
__global__ void k_div_to_f32(int64_t n, const double* __restrict__ x, const double* __restrict__ d, float* __restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = (float)(x[i] / d[i]);
}
__global__ void k_f32_div(int64_t n, const float* __restrict__ x, const double* __restrict__ d, double* __restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = (double)x[i] / d[i];
}
// out = a - b (FP64)
__global__ void k_sub64(int64_t n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}
// out = a - b (FP64) on the rows of realisations with done == 0
__global__ void k_sub64_masked(int nu, int64_t n, const int* __restrict__ seg_of, const int* __restrict__ done,
                               const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n && !done[seg_of[i / nu]]) out[i] = a[i] - b[i];
}
// y = x / d (FP64)
__global__ void k_div64(int64_t n, const double* __restrict__ x, const double* __restrict__ d, double* __restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] / d[i];
}
__global__ void k_to_f32(int64_t n, const double* __restrict__ x, float* __restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = (float)x[i];
}
// y += x (FP32)
__global__ void k_add_f32(int64_t n, const float* __restrict__ x, float* __restrict__ y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] += x[i];
}
// xs += d (FP64 += FP32)
__global__ void k_acc_f32(int64_t n, const float* __restrict__ d, double* __restrict__ xs) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) xs[i] += (double)d[i];
}
// out = a - b (FP32)
__global__ void k_sub_f32(int64_t n, const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}
// mean order-0 eigenstrain weighted by volume: out[seg*6 + r] += V_p E_p[r]
// Volume integral of each particle's eigenstrain polynomial, summed per realisation.  Over a
// sphere of radius a the linear terms average to zero and x_k x_l averages to a^2/5 delta_kl,
// so the order-2 coefficients E_ijkk (diagonal (k, k) slots: 0, 3, 5 of the six p <= q of
// layout 60; 0, 4, 8 of the nine (p, q) of layout 78) add a^2/5 each.
__global__ void k_vol_eigen(int num, int nu, const int* __restrict__ seg_of, const double* __restrict__ rad,
                            const double* __restrict__ axes, const double* __restrict__ x, double* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= num) return;
  const double a = rad[p];
  // particle volume (an ellipsoid's linear eigenstrain averages to its uniform part)
  const double vp = 4.0 / 3.0 * 3.141592653589793 *
                    (axes ? axes[3 * (int64_t)p] * axes[3 * (int64_t)p + 1] * axes[3 * (int64_t)p + 2] : a * a * a);
  const double q = a * a / 5.0;
  const double* e = x + (int64_t)nu * p;
  for (int r = 0; r < 6; ++r) {
    double v = e[r];
    if (nu == 60) v += q * (e[24 + 6 * r] + e[24 + 6 * r + 3] + e[24 + 6 * r + 5]);
    if (nu == 78) v += q * (e[24 + 9 * r] + e[24 + 9 * r + 4] + e[24 + 9 * r + 8]);
    atomicAdd(out + 6 * seg_of[p] + r, vp * v);
  }
}

inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// ------------------------------------------------------------------ batch set-up
ibem_status mf_batch_init(MfBatch& b, const ibem_e3d_batch& in, cudaStream_t st, int layout) {
  if (layout != 24 && layout != 60) return fail(IBEM_ERR_ARG, "mf: layout 24 or 60");
  b.nu = layout;
  if (in.nseg <= 0 || !in.seg_begin || !in.centers_dev || !in.radius_dev || !in.mats)
    return fail(IBEM_ERR_ARG, "mf: bad batch");
  b.st = st;
  b.nseg = in.nseg;
  b.seg_begin_h.assign(in.seg_begin, in.seg_begin + in.nseg + 1);
  b.mats_h.assign(in.mats, in.mats + in.nseg);
  if (b.seg_begin_h[0] != 0) return fail(IBEM_ERR_ARG, "mf: seg_begin[0] must be 0");
  b.max_seg = 0;
  for (int s = 0; s < in.nseg; ++s) {
    const int n = b.seg_begin_h[s + 1] - b.seg_begin_h[s];
    if (n < 1) return fail(IBEM_ERR_ARG, "mf: every realisation needs at least one particle");
    b.max_seg = std::max(b.max_seg, n);
  }
  b.num = b.seg_begin_h[in.nseg];
  b.N = (int64_t)b.nu * b.num;
  b.cen = in.centers_dev;
  b.rad = in.radius_dev;
  b.axes = in.axes_dev;
  std::vector<int> seg_of(b.num);
  std::vector<MfTile> tiles;
  for (int s = 0; s < in.nseg; ++s) {
    for (int p = b.seg_begin_h[s]; p < b.seg_begin_h[s + 1]; ++p) seg_of[p] = s;
    for (int p = b.seg_begin_h[s]; p < b.seg_begin_h[s + 1]; p += kMfThreads)
      tiles.push_back({s, p, std::min(kMfThreads, b.seg_begin_h[s + 1] - p), 0});
  }
  b.ntiles = (int)tiles.size();
  std::vector<MfTile> tiles_s[3];
  for (int k = 0; k < 3; ++k) {
    const int tt = 64 << k;
    for (int s = 0; s < in.nseg; ++s)
      for (int p = b.seg_begin_h[s]; p < b.seg_begin_h[s + 1]; p += tt)
        tiles_s[k].push_back({s, p, std::min(tt, b.seg_begin_h[s + 1] - p), 0});
    b.ntiles_s[k] = (int)tiles_s[k].size();
  }
  // slices of the source range: about 4 CTAs per SM in total, at least 32 sources per slice
  int dev = 0, nsm = 0;
  IBEM_CUDA(cudaGetDevice(&dev));
  IBEM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int want = std::max(1, nsm) * 4;
  b.hsplit = std::max(1, std::min((want + b.ntiles - 1) / b.ntiles, (b.max_seg + 31) / 32));
  b.hsplit_wide = b.hsplit;
  std::vector<SphMat> md(in.nseg), ms(in.nseg);
  std::vector<SphMatF> mf(in.nseg);
  for (int s = 0; s < in.nseg; ++s) {
    const ibem_material& m = in.mats[s];
    md[s] = sph_mat_init(m.E0, m.nu0, m.E1, m.nu1);
    mf[s] = sph_matf_init(md[s]);
    ms[s] = md[s];  // scaled: moduli / mu0
    const double k = 1.0 / md[s].mu0;
    ms[s].kmu *= k;
    ms[s].klam *= k;
    ms[s].lam0 *= k;
    ms[s].twomu0 *= k;
    ms[s].mu0 = 1.0;
  }
  IBEM_CUDA(alloc_async((void**)&b.seg_begin, sizeof(int) * (in.nseg + 1), st));
  IBEM_CUDA(alloc_async((void**)&b.seg_of, sizeof(int) * b.num, st));
  IBEM_CUDA(alloc_async((void**)&b.gh, sizeof(float4) * b.num, st));
  IBEM_CUDA(alloc_async((void**)&b.gl, sizeof(float4) * b.num, st));
  IBEM_CUDA(alloc_async((void**)&b.matd, sizeof(SphMat) * in.nseg, st));
  IBEM_CUDA(alloc_async((void**)&b.matf, sizeof(SphMatF) * in.nseg, st));
  IBEM_CUDA(alloc_async((void**)&b.mats, sizeof(SphMat) * in.nseg, st));
  IBEM_CUDA(alloc_async((void**)&b.dr, sizeof(double) * b.N, st));
  IBEM_CUDA(alloc_async((void**)&b.dc, sizeof(double) * b.N, st));
  IBEM_CUDA(alloc_async((void**)&b.tiles, sizeof(MfTile) * b.ntiles, st));
  for (int k = 0; k < 3; ++k) IBEM_CUDA(alloc_async((void**)&b.tiles_s[k], sizeof(MfTile) * b.ntiles_s[k], st));
  // Morton order of the centres within each realisation (10 bits per axis of its bounding box)
  std::vector<int> perm(b.num);
  {
    std::vector<double> ch(3 * (size_t)b.num);
    IBEM_CUDA(cudaMemcpyAsync(ch.data(), in.centers_dev, sizeof(double) * ch.size(), cudaMemcpyDeviceToHost, st));
    IBEM_CUDA(cudaStreamSynchronize(st));
    auto spread = [](uint32_t v) {
      v &= 0x3ffu;
      v = (v | (v << 16)) & 0x030000ffu;
      v = (v | (v << 8)) & 0x0300f00fu;
      v = (v | (v << 4)) & 0x030c30c3u;
      v = (v | (v << 2)) & 0x09249249u;
      return v;
    };
    std::vector<std::pair<uint32_t, int>> key;
    for (int s = 0; s < in.nseg; ++s) {
      const int p0 = b.seg_begin_h[s], p1 = b.seg_begin_h[s + 1];
      double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
      for (int p = p0; p < p1; ++p)
        for (int d = 0; d < 3; ++d) {
          lo[d] = std::min(lo[d], ch[3 * (size_t)p + d]);
          hi[d] = std::max(hi[d], ch[3 * (size_t)p + d]);
        }
      key.clear();
      for (int p = p0; p < p1; ++p) {
        uint32_t q[3];
        for (int d = 0; d < 3; ++d) {
          const double w = hi[d] > lo[d] ? (ch[3 * (size_t)p + d] - lo[d]) / (hi[d] - lo[d]) : 0.0;
          q[d] = (uint32_t)std::min(1023.0, std::max(0.0, std::floor(w * 1024.0)));
        }
        key.push_back({spread(q[0]) | (spread(q[1]) << 1) | (spread(q[2]) << 2), p});
      }
      std::sort(key.begin(), key.end());
      for (int i = 0; i < p1 - p0; ++i) perm[p0 + i] = key[i].second;
    }
  }
  IBEM_CUDA(alloc_async((void**)&b.perm, sizeof(int) * b.num, st));
  IBEM_CUDA(cudaMemcpyAsync(b.perm, perm.data(), sizeof(int) * b.num, cudaMemcpyHostToDevice, st));
  IBEM_CUDA(cudaMemcpyAsync(b.seg_begin, b.seg_begin_h.data(), sizeof(int) * (in.nseg + 1), cudaMemcpyHostToDevice, st));
  IBEM_CUDA(cudaMemcpyAsync(b.seg_of, seg_of.data(), sizeof(int) * b.num, cudaMemcpyHostToDevice, st));
  IBEM_CUDA(cudaMemcpyAsync(b.matd, md.data(), sizeof(SphMat) * in.nseg, cudaMemcpyHostToDevice, st));
  IBEM_CUDA(cudaMemcpyAsync(b.matf, mf.data(), sizeof(SphMatF) * in.nseg, cudaMemcpyHostToDevice, st));
  IBEM_CUDA(cudaMemcpyAsync(b.mats, ms.data(), sizeof(SphMat) * in.nseg, cudaMemcpyHostToDevice, st));
  IBEM_CUDA(cudaMemcpyAsync(b.tiles, tiles.data(), sizeof(MfTile) * b.ntiles, cudaMemcpyHostToDevice, st));
  for (int k = 0; k < 3; ++k)
    IBEM_CUDA(cudaMemcpyAsync(b.tiles_s[k], tiles_s[k].data(), sizeof(MfTile) * b.ntiles_s[k], cudaMemcpyHostToDevice,
                              st));
  b.tshape = 1;   // 128 targets per CTA until the autotuner says otherwise
  ::ibem::count_launch(), k_mf_prep<<<nblk(b.num), 256, 0, st>>>(b.nu, b.num, b.cen, b.rad, b.seg_of, b.matd, b.gh, b.gl,
                                                                 b.dr, b.dc);
  IBEM_LAUNCH_CHECK("mf prep");
  // the host vectors above must outlive the copies
  IBEM_CUDA(cudaStreamSynchronize(st));
  return IBEM_OK;
}

void mf_batch_free(MfBatch& b) {
  const cudaStream_t st = b.st;
  free_async(b.seg_begin, st);
  free_async(b.seg_of, st);
  free_async(b.gh, st);
  free_async(b.gl, st);
  free_async(b.matd, st);
  free_async(b.matf, st);
  free_async(b.mats, st);
  free_async(b.dr, st);
  free_async(b.dc, st);
  free_async(b.tiles, st);
  for (int k = 0; k < 3; ++k) free_async(b.tiles_s[k], st);
  free_async(b.work, st);
  free_async(b.perm, st);
  b = MfBatch();
}

ibem_status mf_set_f32_shape(MfBatch& b, int tshape, int hsplit, int persist, cudaStream_t st) {
  b.tshape = tshape;
  b.hsplit = hsplit;
  b.persist = persist;
  if (!persist) return IBEM_OK;
  // work list: every (tile, slice) with sources, by decreasing targets x sources
  std::vector<MfTile> tiles(b.ntiles_s[tshape]);
  {
    // tiles of this shape, rebuilt on the host from the segment table (as at batch init)
    const int tt = 64 << tshape;
    int n = 0;
    for (int s = 0; s < b.nseg; ++s)
      for (int p = b.seg_begin_h[s]; p < b.seg_begin_h[s + 1]; p += tt)
        tiles[n++] = {s, p, std::min(tt, b.seg_begin_h[s + 1] - p), 0};
  }
  std::vector<std::pair<int64_t, int2>> items;
  for (int t = 0; t < (int)tiles.size(); ++t) {
    const int hb0 = b.seg_begin_h[tiles[t].seg], he0 = b.seg_begin_h[tiles[t].seg + 1];
    const int per = (he0 - hb0 + hsplit - 1) / hsplit;
    for (int j = 0; j < hsplit; ++j) {
      const int len = std::min(he0, hb0 + (j + 1) * per) - (hb0 + j * per);
      if (len > 0) items.push_back({(int64_t)len * tiles[t].ns, make_int2(t, j)});
    }
  }
  std::stable_sort(items.begin(), items.end(), [](const auto& a, const auto& c) { return a.first > c.first; });
  std::vector<int2> w(items.size());
  for (size_t i = 0; i < items.size(); ++i) w[i] = items[i].second;
  free_async(b.work, st);
  b.work = nullptr;
  b.nwork = (int)w.size();
  IBEM_CUDA(alloc_async((void**)&b.work, sizeof(int2) * std::max<size_t>(1, w.size()), st));
  IBEM_CUDA(cudaMemcpyAsync(b.work, w.data(), sizeof(int2) * w.size(), cudaMemcpyHostToDevice, st));
  IBEM_CUDA(cudaStreamSynchronize(st));   // w must outlive the copy
  int dev = 0, sms = 0, per_sm = 0;
  IBEM_CUDA(cudaGetDevice(&dev));
  IBEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int tt = 64 << tshape;
  cudaError_t e = tshape == 0   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mf_apply_f32_persist<64>, tt, 0)
                  : tshape == 1 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mf_apply_f32_persist<128>, tt, 0)
                                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mf_apply_f32_persist<256>, tt, 0);
  if (e != cudaSuccess) return cuda_fail(e, "mf persistent occupancy");
  b.persist_ctas = std::max(1, std::min(b.nwork, std::max(1, per_sm) * sms));
  return IBEM_OK;
}

// ------------------------------------------------------------------ autotuner
// The products' launch shape is (target tiles) x (source slices); the slice count trades
// parallelism and tail effects against the atomic adds of the partial sums.  For the FP32
// product (the GMRES operator, launched once per Arnoldi step) the tuner also picks the
// tile shape (64, 128 or 256 targets per CTA) and the launch form: one CTA per (tile,
// slice), or persistent CTAs (as many as fit on the GPU) over a list of (tile, slice) items
// sorted by decreasing cost.  For a shape class (log2 buckets of the tile count and of the
// largest realisation, and the number of SMs) every candidate is run once to warm up and
// once timed with CUDA events (inputs of zeros: the same work as any input); the fastest is
// kept for the process.  The double-float / FP64 kernels (~255 registers) keep 128-target
// tiles and get their own slice count.
namespace {
struct TuneKey {
  int tiles_b, seg_b, sms;
  bool operator<(const TuneKey& o) const {
    return tiles_b != o.tiles_b ? tiles_b < o.tiles_b : seg_b != o.seg_b ? seg_b < o.seg_b : sms < o.sms;
  }
};
struct TuneVal {
  int hsplit, hsplit_wide, tshape, persist;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune;

int log2_bucket(int v) {
  int b = 0;
  while ((1 << b) < v) ++b;
  return b;
}
// slice counts that give 1, 2, 4 and 8 CTAs per SM in total (at least 32 sources a slice)
std::vector<int> slice_candidates(int ntiles, int max_seg, int sms) {
  const int cap = std::max(1, (max_seg + 31) / 32);
  std::vector<int> cand;
  for (int per_sm : {1, 2, 4, 8}) {
    const int h = std::max(1, std::min(cap, (sms * per_sm + ntiles - 1) / ntiles));
    if (std::find(cand.begin(), cand.end(), h) == cand.end()) cand.push_back(h);
  }
  return cand;
}
}  // namespace

ibem_status mf_tune(MfBatch& b, cudaStream_t st) {
  int dev = 0, sms = 0;
  IBEM_CUDA(cudaGetDevice(&dev));
  IBEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const TuneKey key{log2_bucket(b.ntiles), log2_bucket(b.max_seg), sms * 100 + b.nu};
  const int cap = std::max(1, (b.max_seg + 31) / 32);
  // IBEM_MF_F32_SHAPE="shape,persistent,slices" fixes the FP32 product's launch (tests and
  // measurements of every shape); the wide products keep the batch's initial slice count
  if (const char* f = b.nu == 24 ? std::getenv("IBEM_MF_F32_SHAPE") : nullptr) {
    int ts = 1, pers = 0, h = 1;
    if (std::sscanf(f, "%d,%d,%d", &ts, &pers, &h) == 3 && ts >= 0 && ts < 3 && (pers == 0 || pers == 1) && h >= 1)
      return mf_set_f32_shape(b, ts, std::min(h, cap), pers, st);
    return fail(IBEM_ERR_ARG, "IBEM_MF_F32_SHAPE: expected shape (0-2),persistent (0/1),slices (>= 1)");
  }
  {
    bool hit = false;
    TuneVal v{};
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tune.find(key);
      if (it != g_tune.end()) {
        hit = true;
        v = it->second;
      }
    }
    if (hit) {
      b.hsplit_wide = std::min(v.hsplit_wide, cap);
      return mf_set_f32_shape(b, v.tshape, std::min(v.hsplit, cap), v.persist, st);
    }
  }
  float* xf = nullptr;
  float* yf = nullptr;
  double* xd = nullptr;
  double* yd = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ibem_status s = IBEM_OK;
  {
    cudaError_t e = alloc_async((void**)&xf, sizeof(float) * b.N, st);
    if (e == cudaSuccess) e = alloc_async((void**)&yf, sizeof(float) * b.N, st);
    if (e == cudaSuccess) e = alloc_async((void**)&xd, sizeof(double) * b.N, st);
    if (e == cudaSuccess) e = alloc_async((void**)&yd, sizeof(double) * b.N, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(xf, 0, sizeof(float) * b.N, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(xd, 0, sizeof(double) * b.N, st);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) s = cuda_fail(e, "mf tune");
  }
  // runs the product twice (warm-up, then timed) and returns the timed milliseconds
  auto time_it = [&](bool wide, float& ms) -> ibem_status {
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0, st);
      ibem_status r = wide ? mf_apply_df(b, xd, yd, st) : mf_apply_f32(b, xf, yf, st);
      cudaEventRecord(e1, st);
      if (r) return r;
    }
    const cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) return cuda_fail(e, "mf tune");
    cudaEventElapsedTime(&ms, e0, e1);
    return IBEM_OK;
  };
  TuneVal best{b.hsplit, b.hsplit_wide, b.tshape, 0};
  float best_ms = 1e30f;
  for (int ts = 0; ts < 3 && !s; ++ts)
    for (int h : slice_candidates(b.ntiles_s[ts], b.max_seg, sms)) {
      if (b.nu == 60 && ts != 1) break;   // the layout-60 products have 128-target tiles only
      for (int pers = 0; pers < (b.nu == 60 ? 1 : 2) && !s; ++pers) {
        if ((s = mf_set_f32_shape(b, ts, h, pers, st))) break;
        float ms = 0.f;
        if ((s = time_it(false, ms))) break;
        if (ms < best_ms) {
          best_ms = ms;
          best.tshape = ts;
          best.hsplit = h;
          best.persist = pers;
        }
      }
      if (s) break;
    }
  best_ms = 1e30f;
  for (int h : slice_candidates(b.ntiles, b.max_seg, sms)) {
    if (s) break;
    b.hsplit_wide = h;
    float ms = 0.f;
    if ((s = time_it(true, ms))) break;
    if (ms < best_ms) {
      best_ms = ms;
      best.hsplit_wide = h;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  free_async(xf, st);
  free_async(yf, st);
  free_async(xd, st);
  free_async(yd, st);
  if (s) return s;
  b.hsplit_wide = best.hsplit_wide;
  if ((s = mf_set_f32_shape(b, best.tshape, best.hsplit, best.persist, st))) return s;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = best;
  return IBEM_OK;
}

template <int TT>
void launch_f32(const MfBatch& b, const float* x, float* y, cudaStream_t st, const int* mask, int mask_on) {
  const MfTile* tiles = b.tiles_s[TT == 64 ? 0 : (TT == 128 ? 1 : 2)];
  if (b.persist)
    ::ibem::count_launch(), k_mf_apply_f32_persist<TT><<<b.persist_ctas, TT, 0, st>>>(
        tiles, b.work, b.nwork, b.hsplit, b.seg_begin, mask, mask_on, b.gh, b.gl, b.matf, x, y);
  else
    ::ibem::count_launch(), k_mf_apply_f32<TT><<<dim3(b.ntiles_s[TT == 64 ? 0 : (TT == 128 ? 1 : 2)], b.hsplit), TT, 0,
                                                 st>>>(tiles, b.seg_begin, mask, mask_on, b.gh, b.gl, b.matf, x, y);
}

ibem_status mf_apply_f32(const MfBatch& b, const float* x, float* y, cudaStream_t st, const int* mask, int mask_on) {
  ProfScope ps(PROF_MF_F32, st, 0.0);
  IBEM_CUDA(cudaMemsetAsync(y, 0, sizeof(float) * b.N, st));
  if (b.nu == 60) return mf60_apply_f32(b, x, y, st, mask, mask_on);
  if (b.tshape == 0) launch_f32<64>(b, x, y, st, mask, mask_on);
  else if (b.tshape == 2) launch_f32<256>(b, x, y, st, mask, mask_on);
  else launch_f32<128>(b, x, y, st, mask, mask_on);
  IBEM_LAUNCH_CHECK("mf apply f32");
  return IBEM_OK;
}

ibem_status mf_apply_f64(const MfBatch& b, const double* x, double* y, cudaStream_t st, const int* mask, int mask_on) {
  ProfScope ps(PROF_MF_F64, st, 0.0);
  IBEM_CUDA(cudaMemsetAsync(y, 0, sizeof(double) * b.N, st));
  if (b.nu == 60) return mf60_apply_f64(b, x, y, st, mask, mask_on);
  // near sources in FP64, far sources (beyond kMfFarRadii of their radius from the box of
  // the warp's targets) in double-float: their contributions are at most kMfFarRadii^-3 of a
  // touching one, so the double-float rounding (~2^-44 per operation, times 4^-3) is ~1e-15
  // of the largest term, the level of the FP64 rounding of the near pairs (measured: split
  // against all pairs in FP64 6.6e-16 relative, 5.2e-16 with 8 radii, 1.7e-14 for
  // double-float everywhere).  In realisations below kMfSplitMin particles most (warp,
  // source) pairs are near, and one FP64 launch over every pair is faster than the two passes
  const bool split = b.max_seg >= kMfSplitMin;
  ::ibem::count_launch(), k_mf_apply_f64<<<dim3(b.ntiles, b.hsplit_wide), kMfThreads, 0, st>>>(
      b.tiles, b.seg_begin, mask, mask_on, b.cen, b.rad, b.mats, x, y, b.perm, split ? 1 : 0);
  if (split && b.max_seg < kMfSkipMin)
    ::ibem::count_launch(), k_mf_apply_df<kMfThreads><<<dim3(b.ntiles, b.hsplit_wide), kMfThreads, 0, st>>>(
        b.tiles, b.seg_begin, mask, mask_on, b.cen, b.rad, b.mats, x, y, b.perm, 2);
  else if (split)   // the same number of warps per SM, one CTA of 256 targets (tiles_s[2])
    ::ibem::count_launch(),
        k_mf_apply_df<2 * kMfThreads><<<dim3(b.ntiles_s[2], std::min((b.max_seg + 31) / 32, 2 * b.hsplit_wide)),
                                         2 * kMfThreads, 0, st>>>(b.tiles_s[2], b.seg_begin, mask, mask_on, b.cen,
                                                                  b.rad, b.mats, x, y, b.perm, 3);
  IBEM_LAUNCH_CHECK("mf apply f64");
  return IBEM_OK;
}

ibem_status mf_apply_f64_all(const MfBatch& b, const double* x, double* y, cudaStream_t st) {
  ProfScope ps(PROF_MF_F64, st, 0.0);
  IBEM_CUDA(cudaMemsetAsync(y, 0, sizeof(double) * b.N, st));
  if (b.nu == 60) return mf60_apply_f64(b, x, y, st, nullptr, 1);
  ::ibem::count_launch(), k_mf_apply_f64<<<dim3(b.ntiles, b.hsplit_wide), kMfThreads, 0, st>>>(
      b.tiles, b.seg_begin, nullptr, 1, b.cen, b.rad, b.mats, x, y, b.perm, 0);
  IBEM_LAUNCH_CHECK("mf apply f64 (all pairs)");
  return IBEM_OK;
}

ibem_status mf_apply_df(const MfBatch& b, const double* x, double* y, cudaStream_t st, const int* mask, int mask_on) {
  ProfScope ps(PROF_MF_DF, st, 0.0);
  IBEM_CUDA(cudaMemsetAsync(y, 0, sizeof(double) * b.N, st));
  if (b.nu == 60) return mf60_apply_f64(b, x, y, st, mask, mask_on);   // no double-float form of layout 60
  ::ibem::count_launch(), k_mf_apply_df<kMfThreads><<<dim3(b.ntiles, b.hsplit_wide), kMfThreads, 0, st>>>(
      b.tiles, b.seg_begin, mask, mask_on, b.cen, b.rad, b.mats, x, y, b.perm, 0);
  IBEM_LAUNCH_CHECK("mf apply df");
  return IBEM_OK;
}

ibem_status mf_block_jacobi(const MfBatch& b, float* P, cudaStream_t st) {
  float* Pseg = nullptr;
  IBEM_CUDA(alloc_async((void**)&Pseg, sizeof(float) * kMfNu * kMfNu * (size_t)b.nseg, st));
  ::ibem::count_launch(), k_block_jacobi<<<b.nseg, 32, 0, st>>>(b.matd, Pseg);
  ::ibem::count_launch(), k_bcast_blocks<<<nblk((int64_t)b.num * kMfNu * kMfNu / 4), 256, 0, st>>>(b.num, b.seg_of, Pseg, P);
  free_async(Pseg, st);
  IBEM_LAUNCH_CHECK("block jacobi");
  return IBEM_OK;
}


// ------------------------------------------------------------------ solver
namespace {

struct MfSolver {
  const MfBatch& b;
  cudaStream_t st;
  int m;
  int64_t N;
  float* V = nullptr;    // (m+1) x N Krylov basis
  float* z = nullptr;    // N
  float* w = nullptr;    // N   new Arnoldi vector before normalisation (and scratch)
  float* d = nullptr;    // N   correction of the current refinement step
  float* rin = nullptr;  // N   right-hand side of the current GMRES solve
  float* r32 = nullptr;  // N   residual of a restarted cycle
  int* done = nullptr;   // nseg
  double* tolv = nullptr;  // nseg: residual reduction asked of this GMRES solve
  int* kdev = nullptr;     // Arnoldi step index of the graph-captured cycle
  int* steps_dev = nullptr;  // Arnoldi steps run by the captured cycles (launch count)
  Krylov K{};
  void* kmem = nullptr;
  int splits = 1;
  // one GMRES cycle's Arnoldi steps as a CUDA graph: a while node whose body is one step
  // (captured once per solver; the buffers it uses live as long as the solver)
  bool use_graph = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long step_kernels = 0;   // kernels in one captured step
  const MfPrecond* graph_pc = nullptr;
  MfSolver(const MfBatch& bb, cudaStream_t s, int mm, bool graphs) : b(bb), st(s), m(mm), N(bb.N), use_graph(graphs) {
    splits = (int)((b.nu * (int64_t)b.max_seg + kDotThreads * kDotRows - 1) / (kDotThreads * kDotRows));
  }
  ~MfSolver() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    free_async(V, st);
    free_async(z, st);
    free_async(w, st);
    free_async(d, st);
    free_async(rin, st);
    free_async(r32, st);
    free_async(done, st);
    free_async(tolv, st);
    free_async(kmem, st);
  }
  ibem_status alloc() {
    IBEM_CUDA(alloc_async((void**)&V, sizeof(float) * N * (m + 1), st));
    IBEM_CUDA(alloc_async((void**)&z, sizeof(float) * N, st));
    IBEM_CUDA(alloc_async((void**)&w, sizeof(float) * N, st));
    IBEM_CUDA(alloc_async((void**)&d, sizeof(float) * N, st));
    IBEM_CUDA(alloc_async((void**)&rin, sizeof(float) * N, st));
    IBEM_CUDA(alloc_async((void**)&r32, sizeof(float) * N, st));
    IBEM_CUDA(alloc_async((void**)&done, sizeof(int) * b.nseg, st));
    IBEM_CUDA(alloc_async((void**)&tolv, sizeof(double) * b.nseg, st));
    const size_t S = b.nseg;
    const size_t nd = S * ((size_t)(m + 1) * m + (m + 1) + 2 * (size_t)m + 5 + 2 * (size_t)(m + 1) + m);
    const size_t ni = 3 * S + 3;
    IBEM_CUDA(alloc_async((void**)&kmem, nd * sizeof(double) + sizeof(int) * ni, st));
    double* p = (double*)kmem;
    K.H = p; p += S * (m + 1) * m;
    K.g = p; p += S * (m + 1);
    K.cs = p; p += S * m;
    K.sn = p; p += S * m;
    K.beta = p; p += S;
    K.inv = p; p += S;
    K.n2 = p; p += S;
    K.thr = p; p += S;
    K.est = p; p += S;
    K.d1 = p; p += S * (m + 1);
    K.d2 = p; p += S * (m + 1);
    K.yv = p; p += S * m;
    int* ip = (int*)p;
    K.kc = ip; ip += S;
    K.active = ip; ip += S;
    K.nsteps = ip; ip += S;
    K.nactive = ip; ip += 1;
    kdev = ip; ip += 1;
    steps_dev = ip;
    IBEM_CUDA(cudaMemsetAsync(kmem, 0, nd * sizeof(double) + sizeof(int) * ni, st));
    return IBEM_OK;
  }
  template <class T>
  ibem_status seg_norm2(const T* v, double* n2, cudaStream_t s) {
    IBEM_CUDA(cudaMemsetAsync(n2, 0, sizeof(double) * b.nseg, s));
    ::ibem::count_launch(), k_seg_dots<T><<<dim3(b.nseg, splits), kDotThreads, 0, s>>>(b.nu, b.seg_begin, 1, v, 0, v, n2, 1);
    IBEM_LAUNCH_CHECK("seg norm");
    return IBEM_OK;
  }
  template <class T>
  ibem_status seg_norm2(const T* v, double* n2) { return seg_norm2(v, n2, st); }
  int read_nactive(ibem_status& s) {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, K.nactive, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = cuda_fail(e, "gmres: read active count");
    return h;
  }
  // z = P v (layout 24: the block-sparse preconditioner; layout 60: the realisation's
  // block-Jacobi block, P.D holding one 60 x 60 block per realisation)
  ibem_status precond(const MfPrecond& P, const float* v, float* z, const int* kd, int64_t vstride, cudaStream_t s) {
    if (b.nu == 60) return mf60_precond_apply(b, P.D, v, z, kd, vstride, s);
    ::ibem::count_launch(), k_precond_apply<<<nblk(N), 256, 0, s>>>(b.num, P.D, P.Q, P.nbr, v, z, kd, vstride);
    IBEM_LAUNCH_CHECK("preconditioner");
    return IBEM_OK;
  }
  // Arnoldi step k on stream s: w = As P v_k, two Gram-Schmidt passes against v_0..v_k,
  // the per-realisation Hessenberg update, v_(k+1) = w / ||w||.  With kd (graph capture) the
  // kernels read k from *kd instead.
  ibem_status arnoldi_step(const MfPrecond& P, int k, const int* kd, cudaStream_t s) {
    const int S = b.nseg;
    const float* vk = kd ? V : V + (int64_t)k * N;
    const int nv = kd ? 1 : k + 1;   // k_seg_dots / k_seg_sub add *kd
    ibem_status r = precond(P, vk, z, kd, kd ? N : 0, s);
    if (r) return r;
    r = mf_apply_f32(b, z, w, s, K.active, 1);   // converged realisations sit out
    if (r) return r;
    ProfScope pg(PROF_GMRES_OTHER, s);
    IBEM_CUDA(cudaMemsetAsync(K.d1, 0, sizeof(double) * 2 * (size_t)S * (m + 1), s));
    ::ibem::count_launch(), k_seg_dots<float><<<dim3(S, splits), kDotThreads, 0, s>>>(b.nu, b.seg_begin, nv, V, N, w, K.d1, m + 1, kd);
    ::ibem::count_launch(), k_seg_sub<<<nblk(N), 256, 0, s>>>(b.nu, N, b.seg_of, nv, V, N, K.d1, m + 1, w, kd);
    ::ibem::count_launch(), k_seg_dots<float><<<dim3(S, splits), kDotThreads, 0, s>>>(b.nu, b.seg_begin, nv, V, N, w, K.d2, m + 1, kd);
    ::ibem::count_launch(), k_seg_sub<<<nblk(N), 256, 0, s>>>(b.nu, N, b.seg_of, nv, V, N, K.d2, m + 1, w, kd);
    if ((r = seg_norm2(w, K.n2, s))) return r;
    IBEM_CUDA(cudaMemsetAsync(K.nactive, 0, sizeof(int), s));
    ::ibem::count_launch(), k_arnoldi_update<<<nblk(S, 128), 128, 0, s>>>(S, m, k, K, kd);
    float* vnext = kd ? V : V + (int64_t)(k + 1) * N;
    ::ibem::count_launch(), k_seg_scale<float, float><<<nblk(N), 256, 0, s>>>(b.nu, N, b.seg_of, K.inv, w, vnext, 0, kd,
                                                                               kd ? N : 0);
    IBEM_LAUNCH_CHECK("arnoldi step");
    return IBEM_OK;
  }
  // The cycle graph: while (k < m and a realisation is active) { Arnoldi step *kdev; k += 1 }.
  // Captured on a private stream (capture only records; the graph runs on st).
  ibem_status build_graph(const MfPrecond& P) {
    cudaStream_t cs = nullptr;
    cudaGraphConditionalHandle h;
    cudaGraphNodeParams cp{};
    cudaGraphNode_t node;
    IBEM_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaError_t e = cudaGraphCreate(&graph, 0);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) {
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp);
    }
    ibem_status r = IBEM_OK;
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(cs, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                            cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      const long long before = launches_so_far();
      r = arnoldi_step(P, 0, kdev, cs);
      if (!r) ::ibem::count_launch(), k_step_ctl<<<1, 1, 0, cs>>>(kdev, K.nactive, m, h);
      step_kernels = launches_so_far() - before;
      add_launches(-step_kernels);   // captured, not run
      cudaGraph_t body = nullptr;
      const cudaError_t e2 = cudaStreamEndCapture(cs, &body);
      if (e2 != cudaSuccess && !r) e = e2;
    }
    if (e == cudaSuccess && !r) e = cudaGraphInstantiate(&exec, graph, 0);
    cudaStreamDestroy(cs);
    if (r) return r;
    if (e != cudaSuccess) return cuda_fail(e, "gmres: cycle graph");
    graph_pc = &P;
    return IBEM_OK;
  }
  // FP32 GMRES(m) with restarts on As d = rin, right-preconditioned by P; d overwritten.
  // Realisations flagged in `done` take no step.  Stops each realisation once
  // ||rin - As d|| <= inner_tol ||rin|| (Arnoldi estimate).
  ibem_status gmres(const MfPrecond& P, int max_cycles) {
    const int S = b.nseg;
    ibem_status s = IBEM_OK;
    // the phase profiler records events, which a graph's while loop cannot hold
    const bool graphed = use_graph && !prof_on();
    if (graphed && (!exec || graph_pc != &P) && (s = build_graph(P))) return s;
    IBEM_CUDA(cudaMemsetAsync(d, 0, sizeof(float) * N, st));
    for (int cyc = 0; cyc < max_cycles && !s; ++cyc) {
      const float* r = rin;
      if (cyc > 0) {  // residual of the restarted cycle, rin - As d
        if ((s = mf_apply_f32(b, d, w, st, done, 0))) break;
        ::ibem::count_launch(), k_sub_f32<<<nblk(N), 256, 0, st>>>(N, rin, w, r32);
        r = r32;
      }
      if ((s = seg_norm2(r, K.n2))) break;
      IBEM_CUDA(cudaMemsetAsync(K.nactive, 0, sizeof(int), st));
      ::ibem::count_launch(), k_cycle_start<<<nblk(S, 128), 128, 0, st>>>(S, m, K, done, cyc == 0, tolv);
      ::ibem::count_launch(), k_seg_scale<float, float><<<nblk(N), 256, 0, st>>>(b.nu, N, b.seg_of, K.inv, r, V, 0);
      IBEM_LAUNCH_CHECK("gmres cycle start");
      const int na = read_nactive(s);
      if (s || na == 0) break;
      int k = 0;
      if (graphed) {
        IBEM_CUDA(cudaMemsetAsync(kdev, 0, sizeof(int), st));
        IBEM_CUDA(cudaGraphLaunch(exec, st));
        ::ibem::count_launch(), k_add_steps<<<1, 1, 0, st>>>(kdev, steps_dev);
        IBEM_LAUNCH_CHECK("gmres cycle graph");
      } else {
        while (k < m) {
          if ((s = arnoldi_step(P, k, nullptr, st))) break;
          ++k;
          if (read_nactive(s) == 0 || s) break;
        }
      }
      if (s) break;
      // d += P V y
      ::ibem::count_launch(), k_hess_solve<<<nblk(S, 128), 128, 0, st>>>(S, m, K);
      IBEM_CUDA(cudaMemsetAsync(w, 0, sizeof(float) * N, st));
      ::ibem::count_launch(), k_seg_combine<<<nblk(N), 256, 0, st>>>(b.nu, N, b.seg_of, graphed ? 0 : k, V, N, K.yv, m, w,
                                                                    graphed ? kdev : nullptr);
      if ((s = precond(P, w, z, nullptr, 0, st))) break;
      ::ibem::count_launch(), k_add_f32<<<nblk(N), 256, 0, st>>>(N, z, d);
      IBEM_LAUNCH_CHECK("gmres update");
    }
    return s;
  }
  // kernels the captured cycles ran (read once, when the solve has synchronised)
  long long graph_launches() {
    if (!exec) return 0;
    int h = 0;
    if (cudaMemcpy(&h, steps_dev, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
    return (long long)h * step_kernels;
  }
};

}  // namespace

ibem_status mf_solve(const MfBatch& b, const double* bvec, double* x, const MfPrecond& P, const ibem_mf_options& o,
                     ibem_mf_report* rep, cudaStream_t st) {
  const int S = b.nseg;
  const int64_t N = b.N;
  MfSolver g(b, st, o.restart, o.stepwise == 0);
  ibem_status s = g.alloc();
  double *xs = nullptr, *rs = nullptr, *y = nullptr, *bs = nullptr, *bn2 = nullptr;
  if (!s) {
    cudaError_t e = alloc_async((void**)&xs, sizeof(double) * N, st);
    if (e == cudaSuccess) e = alloc_async((void**)&rs, sizeof(double) * N, st);
    if (e == cudaSuccess) e = alloc_async((void**)&y, sizeof(double) * N, st);
    if (e == cudaSuccess) e = alloc_async((void**)&bs, sizeof(double) * N, st);
    if (e == cudaSuccess) e = alloc_async((void**)&bn2, sizeof(double) * 2 * S, st);
    if (e != cudaSuccess) s = cuda_fail(e, "mf solve workspace");
  }
  std::vector<double> hb(S), hr(S), htol(S);
  std::vector<int> hdone(S, 0), outer_of(S, 0);
  if (!s) {
    cudaMemsetAsync(xs, 0, sizeof(double) * N, st);
    ::ibem::count_launch(), k_mul<<<nblk(N), 256, 0, st>>>(N, b.dr, bvec, bs);  // bs = Dr b
    cudaMemcpyAsync(rs, bs, sizeof(double) * N, cudaMemcpyDeviceToDevice, st);  // rs = bs (x = 0)
    s = g.seg_norm2(rs, bn2);
    if (!s) {
      cudaMemcpyAsync(hb.data(), bn2, sizeof(double) * S, cudaMemcpyDeviceToHost, st);
      const cudaError_t e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) s = cuda_fail(e, "mf solve: rhs norms");
    }
  }
  // rs holds the residual of the current iterate; `exact` says whether it came from the
  // FP64 product (or x = 0).  A double-float residual drives the next correction; once it
  // shows every realisation within tol, the FP64 residual of the same iterate decides.
  bool exact = true;
  auto read_rel = [&]() -> ibem_status {
    ibem_status r = g.seg_norm2(rs, bn2 + S);
    if (r) return r;
    cudaMemcpyAsync(hr.data(), bn2 + S, sizeof(double) * S, cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "mf solve: residual norms");
    return IBEM_OK;
  };
  auto fp64_residual = [&]() -> ibem_status {
    ibem_status r = mf_apply_f64(b, xs, y, st);   // As xs in FP64
    if (r) return r;
    ::ibem::count_launch(), k_sub64<<<nblk(N), 256, 0, st>>>(N, bs, y, rs);   // rs = bs - As xs
    IBEM_LAUNCH_CHECK("mf residual");
    exact = true;
    return read_rel();
  };
  int outer = 0;
  hr = hb;
  while (!s) {
    bool all = true;
    for (int i = 0; i < S; ++i) all = all && (hb[i] > 0 ? std::sqrt(hr[i] / hb[i]) : 0.0) <= o.tol;
    if (!exact && (all || outer >= o.max_outer)) {
      if ((s = fp64_residual())) break;
      all = true;
      for (int i = 0; i < S; ++i) all = all && (hb[i] > 0 ? std::sqrt(hr[i] / hb[i]) : 0.0) <= o.tol;
    }
    for (int i = 0; i < S; ++i) {
      const double rel = hb[i] > 0 ? std::sqrt(hr[i] / hb[i]) : 0.0;
      rep[i].rel_residual = rel;
      hdone[i] = rel <= o.tol ? 1 : 0;
    }
    if (all || outer >= o.max_outer) break;
    for (int i = 0; i < S; ++i)
      if (!hdone[i]) outer_of[i] = outer + 1;
    cudaMemcpyAsync(g.done, hdone.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st);
    // reduction asked of each realisation's GMRES: inner_tol, or deeper when that is what
    // brings the next residual within tol (never below the ~1e-6 the FP32 products allow)
    for (int i = 0; i < S; ++i)
      htol[i] = std::max(1e-6, std::min(o.inner_tol, rep[i].rel_residual > 0 ? 0.1 * o.tol / rep[i].rel_residual : o.inner_tol));
    cudaMemcpyAsync(g.tolv, htol.data(), sizeof(double) * S, cudaMemcpyHostToDevice, st);
    // FP32 correction of the scaled system, then the double-float residual of the new iterate
    ::ibem::count_launch(), k_to_f32<<<nblk(N), 256, 0, st>>>(N, rs, g.rin);
    if ((s = g.gmres(P, o.max_cycles))) break;
    ::ibem::count_launch(), k_acc_f32<<<nblk(N), 256, 0, st>>>(N, g.d, xs);
    ++outer;
    // expected residual of every realisation still running: its previous residual times the
    // reduction its GMRES reached (Arnoldi estimate over the first beta), but no better than
    // the FP32 products allow (~1e-6 of the correction).  When all are expected to meet tol,
    // go straight to the deciding FP64 residual; otherwise a double-float one.
    std::vector<double> est(S), thr(S);
    cudaMemcpyAsync(est.data(), g.K.est, sizeof(double) * S, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(thr.data(), g.K.thr, sizeof(double) * S, cudaMemcpyDeviceToHost, st);
    {
      const cudaError_t e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) { s = cuda_fail(e, "mf solve: GMRES estimates"); break; }
    }
    bool expect = true;
    for (int i = 0; i < S; ++i) {
      if (hdone[i]) continue;
      const double beta0 = thr[i] > 0 ? thr[i] / htol[i] : 0.0;
      const double red = beta0 > 0 ? std::max(est[i] / beta0, 1e-6) : 1.0;
      expect = expect && rep[i].rel_residual * red <= 0.5 * o.tol;
    }
    if (expect) {
      if ((s = fp64_residual())) break;
      continue;
    }
    if ((s = mf_apply_df(b, xs, y, st, g.done, 0))) break;   // done realisations keep their residual
    ::ibem::count_launch(), k_sub64_masked<<<nblk(N), 256, 0, st>>>(b.nu, N, b.seg_of, g.done, bs, y, rs);
    IBEM_LAUNCH_CHECK("mf refinement");
    exact = false;
    if ((s = read_rel())) break;
  }
  if (!s) {
    ::ibem::count_launch(), k_mul<<<nblk(N), 256, 0, st>>>(N, b.dc, xs, x);
    std::vector<int> steps(S);
    cudaMemcpyAsync(steps.data(), g.K.nsteps, sizeof(int) * S, cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = cuda_fail(e, "mf solve: finish");
    for (int i = 0; i < S; ++i) {
      rep[i].outer = outer_of[i];
      rep[i].inner = steps[i];
    }
    if (!s) add_launches(g.graph_launches());
    for (int i = 0; i < S && !s; ++i)
      if (!(rep[i].rel_residual <= o.tol)) s = fail(IBEM_ERR_NOCONV, "mf solve: a realisation missed the tolerance");
  }
  free_async(xs, st);
  free_async(rs, st);
  free_async(y, st);
  free_async(bs, st);
  free_async(bn2, st);
  return s;
}

}  // namespace ibem

// ------------------------------------------------------------------ C ABI
using namespace ibem;

extern "C" ibem_status ibem_e3d_mf_matvec(const ibem_e3d_batch* batch, int precision, const double* x_dev,
                                          double* y_dev, void* stream) {
  return ibem_e3d_mf_matvec_layout(batch, 24, precision, x_dev, y_dev, stream);
}

extern "C" ibem_status ibem_e3d_mf_matvec_layout(const ibem_e3d_batch* batch, int layout, int precision,
                                                 const double* x_dev, double* y_dev, void* stream) {
  if (batch && batch->axes_dev) return fail(IBEM_ERR_ARG, "matrix-free products and the learned preconditioner take spheres; solve ellipsoid batches with ibem_e3d_batch_dense_solve");
  if (!batch || !x_dev || !y_dev || (precision != 32 && precision != 48 && precision != 64 && precision != 65))
    return fail(IBEM_ERR_ARG, "mf_matvec: bad arguments");
  if (layout != 24 && layout != 60) return fail(IBEM_ERR_ARG, "mf_matvec: layout 24 or 60");
  cudaStream_t st = as_stream(stream);
  MfBatch b;
  ibem_status s = mf_batch_init(b, *batch, st, layout);
  if (!s) {
    if (precision != 32) {
      double *xs = nullptr, *ys = nullptr;
      cudaError_t e = alloc_async((void**)&xs, sizeof(double) * b.N, st);
      if (e == cudaSuccess) e = alloc_async((void**)&ys, sizeof(double) * b.N, st);
      if (e != cudaSuccess) s = cuda_fail(e, "mf_matvec workspace");
      if (!s) {
        ::ibem::count_launch(), k_div64<<<nblk(b.N), 256, 0, st>>>(b.N, x_dev, b.dc, xs);  // xs = x / Dc
        s = precision == 64 ? mf_apply_f64(b, xs, ys, st)
                            : precision == 65 ? mf_apply_f64_all(b, xs, ys, st) : mf_apply_df(b, xs, ys, st);
        if (!s) ::ibem::count_launch(), k_div64<<<nblk(b.N), 256, 0, st>>>(b.N, ys, b.dr, y_dev);  // y = ys / Dr
      }
      if (!s) {
        const cudaError_t e2 = cudaStreamSynchronize(st);
        if (e2 != cudaSuccess) s = cuda_fail(e2, "mf_matvec");
      }
      free_async(xs, st);
      free_async(ys, st);
    } else {
      float *xf = nullptr, *yf = nullptr;
      s = mf_tune(b, st);   // the tile shape the solver's GMRES uses
      cudaError_t e = s ? cudaSuccess : alloc_async((void**)&xf, sizeof(float) * b.N, st);
      if (e == cudaSuccess && !s) e = alloc_async((void**)&yf, sizeof(float) * b.N, st);
      if (e != cudaSuccess) s = cuda_fail(e, "mf_matvec workspace");
      if (!s) {
        ::ibem::count_launch(), k_div_to_f32<<<nblk(b.N), 256, 0, st>>>(b.N, x_dev, b.dc, xf);  // xs = x / Dc
        s = mf_apply_f32(b, xf, yf, st);
        if (!s) ::ibem::count_launch(), k_f32_div<<<nblk(b.N), 256, 0, st>>>(b.N, yf, b.dr, y_dev);  // y = ys / Dr
      }
      if (!s) {
        const cudaError_t e2 = cudaStreamSynchronize(st);
        if (e2 != cudaSuccess) s = cuda_fail(e2, "mf_matvec");
      }
      free_async(xf, st);
      free_async(yf, st);
    }
  }
  if (!s) {
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = cuda_fail(e, "mf_matvec");
  }
  mf_batch_free(b);
  return s;
}

extern "C" ibem_status ibem_e3d_mf_solve(const ibem_e3d_batch* batch, const double* b_dev, double* x_dev,
                                         ibem_precond pc, const float* gnn_params_dev, const ibem_mf_options* opt,
                                         ibem_mf_report* reports, void* stream) {
  return ibem_e3d_mf_solve_layout(batch, 24, b_dev, x_dev, pc, gnn_params_dev, opt, reports, stream);
}

extern "C" ibem_status ibem_e3d_mf_solve_layout(const ibem_e3d_batch* batch, int layout, const double* b_dev,
                                                double* x_dev, ibem_precond pc, const float* gnn_params_dev,
                                                const ibem_mf_options* opt, ibem_mf_report* reports, void* stream) {
  if (layout != 24 && layout != 60) return fail(IBEM_ERR_ARG, "mf_solve: layout 24 or 60");
  if (layout == 60 && pc != IBEM_PRECOND_BLOCK_JACOBI)
    return fail(IBEM_ERR_ARG, "mf_solve: layout 60 takes the block-Jacobi preconditioner");
  if (batch && batch->axes_dev) return fail(IBEM_ERR_ARG, "matrix-free products and the learned preconditioner take spheres; solve ellipsoid batches with ibem_e3d_batch_dense_solve");
  if (!batch || !b_dev || !x_dev || !reports) return fail(IBEM_ERR_ARG, "mf_solve: bad arguments");
  if (pc != IBEM_PRECOND_BLOCK_JACOBI && pc != IBEM_PRECOND_LEARNED && pc != IBEM_PRECOND_NEUMANN)
    return fail(IBEM_ERR_ARG, "mf_solve: preconditioner");
  if (pc == IBEM_PRECOND_LEARNED && !gnn_params_dev) return fail(IBEM_ERR_ARG, "mf_solve: learned form needs parameters");
  ibem_mf_options o{};
  if (opt) o = *opt;
  if (o.restart <= 0) o.restart = 50;
  if (o.max_cycles <= 0) o.max_cycles = 20;
  if (o.max_outer <= 0) o.max_outer = 8;
  if (o.tol <= 0) o.tol = 1e-10;
  if (o.inner_tol <= 0) o.inner_tol = 1e-5;
  if (o.restart > 200) return fail(IBEM_ERR_ARG, "mf_solve: restart > 200");
  cudaStream_t st = as_stream(stream);
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  for (auto& e : ev) IBEM_CUDA(cudaEventCreate(&e));
  IBEM_CUDA(cudaEventRecord(ev[0], st));
  MfBatch b;
  ibem_status s = mf_batch_init(b, *batch, st, layout);
  if (!s) s = mf_tune(b, st);
  MfPrecond P;
  if (!s) {
    // layout 24: one 24 x 24 block per particle (the learned and Neumann forms change them);
    // layout 60: one 60 x 60 block per realisation
    const size_t nblocks = layout == 60 ? (size_t)b.nseg : (size_t)b.num;
    const cudaError_t e = alloc_async((void**)&P.D, sizeof(float) * layout * layout * nblocks, st);
    if (e != cudaSuccess) s = cuda_fail(e, "mf_solve: preconditioner blocks");
  }
  {
    ProfScope pp(PROF_PRECOND, st);
    if (!s) s = layout == 60 ? mf60_block_jacobi(b, P.D, st) : mf_block_jacobi(b, P.D, st);
    if (!s && pc != IBEM_PRECOND_BLOCK_JACOBI)
      s = mf_neighbour_precond(b, pc == IBEM_PRECOND_LEARNED ? gnn_params_dev : nullptr, P, st);
  }
  cudaEventRecord(ev[1], st);
  for (int i = 0; i < batch->nseg; ++i) reports[i] = ibem_mf_report{};
  if (!s) s = mf_solve(b, b_dev, x_dev, P, o, reports, st);
  cudaEventRecord(ev[2], st);
  float t_set = 0.f, t_sol = 0.f;
  if (cudaEventSynchronize(ev[2]) == cudaSuccess) {
    cudaEventElapsedTime(&t_set, ev[0], ev[1]);
    cudaEventElapsedTime(&t_sol, ev[1], ev[2]);
  }
  for (auto& e : ev) cudaEventDestroy(e);
  for (int i = 0; i < batch->nseg; ++i) {
    reports[i].t_setup_ms = t_set;
    reports[i].t_solve_ms = t_sol;
  }
  free_async(P.D, st);
  free_async(P.Q, st);
  free_async(P.nbr, st);
  mf_batch_free(b);
  return s;
}

extern "C" ibem_status ibem_e3d_batch_farfield_rhs_layout(const ibem_e3d_batch* batch, int layout,
                                                          const double* sig_inf, double* b_dev, void* stream) {
  const int nu = ibem_layout_size(layout);
  if (!batch || !batch->seg_begin || !batch->mats || !sig_inf || !b_dev || nu < 0)
    return fail(IBEM_ERR_ARG, "batch_farfield_rhs: bad arguments");
  for (int s = 0; s < batch->nseg; ++s) {
    const int p0 = batch->seg_begin[s], n = batch->seg_begin[s + 1] - p0;
    const ibem_status r = ibem_e3d_farfield_rhs(n, &batch->mats[s], layout, sig_inf, b_dev + (int64_t)nu * p0, stream);
    if (r) return r;
  }
  return IBEM_OK;
}

extern "C" ibem_status ibem_e3d_batch_farfield_rhs(const ibem_e3d_batch* batch, const double* sig_inf, double* b_dev,
                                                   void* stream) {
  return ibem_e3d_batch_farfield_rhs_layout(batch, 24, sig_inf, b_dev, stream);
}

extern "C" ibem_status ibem_e3d_batch_dense_solve(const ibem_e3d_batch* batch, int layout, ibem_solver_form form,
                                                  const double* b_dev, double* x_dev, double tol,
                                                  ibem_solve_report* reports, void* stream) {
  const int nu = ibem_layout_size(layout);
  if (!batch || !batch->seg_begin || !batch->mats || !batch->centers_dev || !batch->radius_dev || !b_dev || !x_dev ||
      nu < 0 || batch->nseg < 0 || batch->seg_begin[0] != 0)
    return fail(IBEM_ERR_ARG, "batch_dense_solve: bad arguments");
  int64_t nmax = 0;
  for (int s = 0; s < batch->nseg; ++s) {
    const int n = batch->seg_begin[s + 1] - batch->seg_begin[s];
    if (n < 0) return fail(IBEM_ERR_ARG, "batch_dense_solve: seg_begin must not decrease");
    nmax = std::max<int64_t>(nmax, (int64_t)nu * n);
  }
  if (form != IBEM_SOLVE_FP64 && form != IBEM_SOLVE_MIXED_IR && form != IBEM_SOLVE_GMRES_BJ)
    return fail(IBEM_ERR_ARG, "batch_dense_solve: unknown solver form");
  if (batch->axes_dev && (layout != 24 || !batch->quats_dev))
    return fail(IBEM_ERR_ARG, "batch_dense_solve: ellipsoids take layout 24 and need quaternions");
  cudaStream_t st = as_stream(stream);
  // Workers: each owns a stream, the largest realisation's N x N matrix and (block-Jacobi
  // form) its FP32 copy, and takes the next unsolved realisation until none is left.  The
  // block-Jacobi form runs several workers at once, so that one realisation's
  // latency-bound steps (host-driven GMRES, small kernels) overlap another's products; the
  // factorising forms run one worker (their panel kernel needs every SM to itself).  As many
  // workers as fit in a quarter of the free device memory, at most kDenseWorkers.
  constexpr int kDenseWorkers = 4;
  const size_t per_worker = sizeof(double) * nmax * nmax +
                            (form == IBEM_SOLVE_GMRES_BJ ? sizeof(float) * ((nmax + 3) / 4 * 4) * nmax : 0);
  int nwork = 1;
  if (form == IBEM_SOLVE_GMRES_BJ && per_worker > 0) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
      nwork = (int)std::max<size_t>(1, std::min<size_t>({(size_t)kDenseWorkers, (size_t)batch->nseg,
                                                         free_b / 4 / per_worker}));
  }
  // b_dev is written on the caller's stream: let it land before the workers read it
  cudaError_t e0 = cudaStreamSynchronize(st);
  if (e0 != cudaSuccess) return cuda_fail(e0, "batch_dense_solve");
  int dev = 0;
  cudaGetDevice(&dev);
  std::atomic<int> next{0};
  std::atomic<bool> failed{false};
  std::mutex err_mu;
  ibem_status first = IBEM_OK;
  std::string first_msg;
  auto worker = [&](bool own_stream) {
    cudaSetDevice(dev);
    cudaStream_t ws = st;
    ibem_status s = IBEM_OK;
    if (own_stream) {
      const cudaError_t e = cudaStreamCreateWithFlags(&ws, cudaStreamNonBlocking);
      if (e != cudaSuccess) s = cuda_fail(e, "batch_dense_solve: stream");
    }
    double* A = nullptr;
    float* W = nullptr;
    if (!s && nmax) {
      cudaError_t e = alloc_async((void**)&A, sizeof(double) * nmax * nmax, ws);
      if (e == cudaSuccess && form == IBEM_SOLVE_GMRES_BJ)
        e = alloc_async((void**)&W, sizeof(float) * ((nmax + 3) / 4 * 4) * nmax, ws);
      if (e != cudaSuccess) s = cuda_fail(e, "batch_dense_solve: matrix");
    }
    while (!s && !failed.load()) {
      const int i = next.fetch_add(1);
      if (i >= batch->nseg) break;
      const int p0 = batch->seg_begin[i], n = batch->seg_begin[i + 1] - p0;
      const int64_t N = (int64_t)nu * n, off = (int64_t)nu * p0;
      ibem_solve_report rep{};
      if (n) {
        s = batch->axes_dev
                ? ibem_e3d_ell_pair_blocks(batch->centers_dev + 3 * (int64_t)p0, batch->axes_dev + 3 * (int64_t)p0,
                                           batch->quats_dev + 4 * (int64_t)p0, n, &batch->mats[i], A, N, 0, 0, ws)
                : ibem_e3d_pair_blocks(batch->centers_dev + 3 * (int64_t)p0, batch->radius_dev + p0, n,
                                       &batch->mats[i], layout, A, N, 0, 0, ws);
        if (!s) s = solve_dense(form, N, A, N, b_dev + off, x_dev + off, tol, &rep, ws, nu, W);
      }
      if (reports) reports[i] = rep;
    }
    free_async(A, ws);
    free_async(W, ws);
    cudaStreamSynchronize(ws);
    if (own_stream && ws) cudaStreamDestroy(ws);
    if (s) {
      failed.store(true);
      std::lock_guard<std::mutex> l(err_mu);
      if (!first) first = s, first_msg = ibem_last_error();
    }
  };
  if (nwork == 1) {
    worker(false);
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < nwork; ++t) pool.emplace_back(worker, true);
    for (auto& t : pool) t.join();
  }
  return first ? fail(first, first_msg) : IBEM_OK;
}

extern "C" ibem_status ibem_e3d_effective_modulus(const ibem_e3d_batch* batch, const double* x_dev,
                                                  const double* volume, const double* sig_inf, double* mean_strain,
                                                  double* e_eff, void* stream) {
  return ibem_e3d_effective_modulus_layout(batch, 24, x_dev, volume, sig_inf, mean_strain, e_eff, stream);
}

extern "C" ibem_status ibem_e3d_effective_modulus_layout(const ibem_e3d_batch* batch, int layout, const double* x_dev,
                                                         const double* volume, const double* sig_inf,
                                                         double* mean_strain, double* e_eff, void* stream) {
  const int nu = ibem_layout_size(layout);
  if (!batch || !x_dev || !volume || !sig_inf || !e_eff || nu < 0)
    return fail(IBEM_ERR_ARG, "effective_modulus: bad arguments");
  if (batch->axes_dev && layout != 24) return fail(IBEM_ERR_ARG, "effective_modulus: ellipsoids take layout 24");
  cudaStream_t st = as_stream(stream);
  MfBatch b;
  ibem_status s = mf_batch_init(b, *batch, st);
  double* acc = nullptr;
  const int S = batch->nseg;
  std::vector<double> h(6 * (size_t)S);
  if (!s) {
    cudaError_t e = alloc_async((void**)&acc, sizeof(double) * 6 * S, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(acc, 0, sizeof(double) * 6 * S, st);
    if (e != cudaSuccess) s = cuda_fail(e, "effective_modulus");
  }
  if (!s) {
    ::ibem::count_launch(), k_vol_eigen<<<nblk(b.num), 256, 0, st>>>(b.num, nu, b.seg_of, b.rad, b.axes, x_dev, acc);
    cudaMemcpyAsync(h.data(), acc, sizeof(double) * 6 * S, cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = cuda_fail(e, "effective_modulus");
  }
  if (!s) {
    for (int i = 0; i < S; ++i) {
      const ibem_material& m = batch->mats[i];
      const double tr = sig_inf[0] + sig_inf[3] + sig_inf[5];
      double eps[6];
      for (int r = 0; r < 6; ++r) {
        const bool diag = (r == 0 || r == 3 || r == 5);
        eps[r] = ((1 + m.nu0) * sig_inf[r] - (diag ? m.nu0 * tr : 0.0)) / m.E0 + h[6 * i + r] / volume[i];
      }
      if (mean_strain)
        for (int r = 0; r < 6; ++r) mean_strain[6 * i + r] = eps[r];
      e_eff[i] = eps[5] != 0 ? sig_inf[5] / eps[5] : 0.0;
    }
  }
  free_async(acc, st);
  mf_batch_free(b);
  return s;
}

// Host buffers in, host buffers out, copied straight between the caller's (pageable) arrays
// and the device: on a Grace host the GPU reads and writes pageable memory at full link speed
// (12.6 MB of stresses: 0.08 ms, the same as from pinned memory), and a pinned staging copy
// would cost a host memcpy (0.74 ms for the same stresses).  The points, needed only by the
// stress sums, go on a second stream ahead of the solve.  Output arrays whose pages are not
// yet mapped (a fresh allocation) would be faulted in by the device copy at a far lower rate:
// a helper thread writes one byte of every page while the device solves.
extern "C" ibem_status ibem_e3d_run_host_mf(const ibem_material* mat, int num, const double* centers,
                                            const double* radius, int nump, const double* points,
                                            const double* sig_inf, ibem_precond pc, const float* gnn_params,
                                            const ibem_mf_options* opt, double* X, double* stress,
                                            ibem_mf_report* report) {
  if (!mat || num <= 0 || !centers || !radius || nump < 0 || (nump > 0 && !points) || !sig_inf || !X ||
      (nump > 0 && !stress) || !report)
    return fail(IBEM_ERR_ARG, "run_host_mf: bad arguments");
  if (pc == IBEM_PRECOND_LEARNED && !gnn_params) return fail(IBEM_ERR_ARG, "run_host_mf: learned form needs parameters");
  const int64_t N = (int64_t)kMfNu * num;
  const int64_t np = gnn_param_count();
  const size_t pts_bytes = sizeof(double) * 3 * (size_t)nump, str_bytes = sizeof(double) * 6 * (size_t)nump;
  double *cen = nullptr, *rad = nullptr, *pts = nullptr, *b = nullptr, *x = nullptr, *S = nullptr;
  float* prm = nullptr;
  cudaStream_t st = nullptr, st2 = nullptr;
  cudaEvent_t ev = nullptr;
  ibem_status s = IBEM_OK;
  {
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = alloc_async((void**)&cen, sizeof(double) * 3 * num, st);
    if (e == cudaSuccess) e = alloc_async((void**)&rad, sizeof(double) * num, st);
    if (e == cudaSuccess) e = alloc_async((void**)&pts, sizeof(double) * 3 * std::max(nump, 1), st);
    if (e == cudaSuccess) e = alloc_async((void**)&b, sizeof(double) * N, st);
    if (e == cudaSuccess) e = alloc_async((void**)&x, sizeof(double) * N, st);
    if (e == cudaSuccess) e = alloc_async((void**)&S, sizeof(double) * 6 * std::max(nump, 1), st);
    if (e == cudaSuccess && gnn_params) e = alloc_async((void**)&prm, sizeof(float) * np, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cen, centers, sizeof(double) * 3 * num, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rad, radius, sizeof(double) * num, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && gnn_params) e = cudaMemcpyAsync(prm, gnn_params, sizeof(float) * np, cudaMemcpyHostToDevice, st);
    // pts is allocated on st: st2 waits for that before it copies into it
    if (e == cudaSuccess) e = cudaEventRecord(ev, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st2, ev, 0);
    if (e == cudaSuccess && nump > 0) e = cudaMemcpyAsync(pts, points, pts_bytes, cudaMemcpyHostToDevice, st2);
    if (e == cudaSuccess) e = cudaEventRecord(ev, st2);
    if (e != cudaSuccess) s = cuda_fail(e, "run_host_mf: set-up");
  }
  std::thread toucher;
  if (!s)
    toucher = std::thread([=]() {
      const size_t step = 4096;   // no larger than any page size
      auto touch = [step](double* p, size_t bytes) {
        for (size_t o = 0; o < bytes; o += step) reinterpret_cast<volatile char*>(p)[o] = 0;
      };
      touch(X, sizeof(double) * (size_t)N);
      if (nump > 0) touch(stress, str_bytes);
    });
  const int seg[2] = {0, num};
  const ibem_e3d_batch bt{1, seg, cen, rad, mat};
  if (!s) s = ibem_e3d_farfield_rhs(num, mat, kMfNu, sig_inf, b, st);
  if (!s) s = ibem_e3d_mf_solve(&bt, b, x, pc, prm, opt, report, st);
  if (!s && nump > 0) {
    const cudaError_t e = cudaStreamWaitEvent(st, ev, 0);
    if (e != cudaSuccess) s = cuda_fail(e, "run_host_mf: points");
  }
  if (!s && nump > 0)
    s = ibem_e3d_field_form(IBEM_SOLVE_MIXED_IR, pts, nump, cen, rad, num, mat, kMfNu, x, nullptr, 0, nullptr, 0,
                            nullptr, nullptr, sig_inf, S, st);
  if (toucher.joinable()) toucher.join();
  if (!s) {
    cudaError_t e = cudaMemcpyAsync(X, x, sizeof(double) * N, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && nump > 0) e = cudaMemcpyAsync(stress, S, str_bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = cuda_fail(e, "run_host_mf: results");
  }
  if (st2) cudaStreamSynchronize(st2);
  if (st) cudaStreamSynchronize(st);
  free_async(cen, st);
  free_async(rad, st);
  free_async(pts, st);
  free_async(b, st);
  free_async(x, st);
  free_async(S, st);
  free_async(prm, st);
  if (ev) cudaEventDestroy(ev);
  if (st2) cudaStreamDestroy(st2);
  if (st) cudaStreamDestroy(st);
  return s;
}

extern "C" ibem_status ibem_e3d_mf_tuning(const ibem_e3d_batch* batch, int* slices_fp32, int* slices_wide,
                                          void* stream) {
  if (batch && batch->axes_dev) return fail(IBEM_ERR_ARG, "matrix-free products and the learned preconditioner take spheres; solve ellipsoid batches with ibem_e3d_batch_dense_solve");
  if (!batch || !slices_fp32 || !slices_wide) return fail(IBEM_ERR_ARG, "mf_tuning: bad arguments");
  cudaStream_t st = as_stream(stream);
  MfBatch b;
  ibem_status s = mf_batch_init(b, *batch, st);
  if (!s) s = mf_tune(b, st);
  if (!s) {
    *slices_fp32 = b.hsplit;
    *slices_wide = b.hsplit_wide;
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = cuda_fail(e, "mf_tuning");
  }
  mf_batch_free(b);
  return s;
}

extern "C" ibem_status ibem_e3d_mf_tile_shape(const ibem_e3d_batch* batch, int* targets_per_cta, int* persistent,
                                              int* slices, void* stream) {
  if (batch && batch->axes_dev) return fail(IBEM_ERR_ARG, "matrix-free products and the learned preconditioner take spheres; solve ellipsoid batches with ibem_e3d_batch_dense_solve");
  if (!batch || !targets_per_cta || !persistent || !slices) return fail(IBEM_ERR_ARG, "mf_tile_shape: bad arguments");
  cudaStream_t st = as_stream(stream);
  MfBatch b;
  ibem_status s = mf_batch_init(b, *batch, st);
  if (!s) s = mf_tune(b, st);
  if (!s) {
    *targets_per_cta = 64 << b.tshape;
    *persistent = b.persist;
    *slices = b.hsplit;
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = cuda_fail(e, "mf_tile_shape");
  }
  mf_batch_free(b);
  return s;
}
