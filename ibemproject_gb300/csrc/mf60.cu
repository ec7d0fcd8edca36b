// Matrix-free products of the layout-60 sphere systems (eigenstrain orders 0, 1 and 2):
// the pair blocks that ibem_e3d_pair_blocks(layout 60) assembles (integratorElastic3D.cpp:
// 341-682: ...EquivalentInclusion, ...FirstOrderInclusion, ...SecondOrderInclusion) are
// evaluated inside the product from the generated straight-line code (gen_sphere60*.cuh),
// so a batch of quadratic realisations is solved without storing its matrices.
//
// Scaled system As = Dr A Dc with Dr = a_s^order / mu0 (rows of target s), Dc = a_h^-order
// (columns of source h): in coordinates x' = (c_s - c_h) / a_h and with the moduli divided by
// mu0 a block is the unit-sphere block times (a_s / a_h)^(row order).  The kernels stage the
// sources' coefficients already multiplied by a_h^-(row order) and multiply the sums by
// a_s^(row order) once, then add the self term C0 / mu0.
//
// One thread per target particle, 128 consecutive targets of one realisation per CTA, source
// slices over gridDim.y; one kernel per row order (6, 18 and 36 rows) and group of columns
// (the generated sub-blocks, the largest split into groups of 6 columns), so that its sums
// and the straight-line code's values stay in registers: FP32 (the GMRES operator) and FP64
// (the refinement residuals).
#include <cuda_runtime.h>

#include <type_traits>

#include "gen_sphere60.cuh"
#include "gen_sphere60_f32.cuh"
#include "mf.h"
#include "prof.h"

namespace ibem {
namespace {

constexpr int kNu = 60;
constexpr int kT = 128;      // targets per CTA
constexpr int kChunk = 16;   // sources staged per chunk

template <int RO>
struct Rows;
template <>
struct Rows<0> {
  static constexpr int off = 0, n = 6;
};
template <>
struct Rows<1> {
  static constexpr int off = 6, n = 18;
};
template <>
struct Rows<2> {
  static constexpr int off = 24, n = 36;
};

__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }

// acc[r - off] += v * xs[c] for the rows of order RO (the generated functions of one row
// order emit only those rows; the self function emits all of them, the others are skipped)
template <class T, int RO>
struct RowSink {
  T* acc;
  const T* __restrict__ xs;
  __device__ __forceinline__ void operator()(int r, int c, T v) const {
    if (r >= Rows<RO>::off && r < Rows<RO>::off + Rows<RO>::n) acc[r - Rows<RO>::off] = fma_t(v, xs[c], acc[r - Rows<RO>::off]);
  }
};

template <class T>
__device__ __forceinline__ T powi(T v, int n) {
  return n == 0 ? T(1) : (n == 1 ? v : v * v);
}

// The generated FP32 sub-blocks one launch evaluates: row order RO, group F (RO 0: F -1,
// all columns; RO 1: F 0 the order-0 and order-1 columns, F 1..6 the order-2 columns of pair
// F - 1; RO 2: F 0 the order-0 columns, F 1..3 the order-1 columns of pairs 2(F-1),
// 2(F-1)+1, F 4..9 the order-2 columns of pair F - 4).  The launch with F <= 0 adds the
// self term.  (FP64: whole column orders, F = CO; splitting them repeats the shared
// intermediates on the FP64 pipe, which costs more than the spills it saves.)
template <class T, int RO, int F, class Sink, class M>
__device__ __forceinline__ void blk(T x0, T x1, T x2, const M& mc, Sink& sk) {
  const T one = T(1);
  if constexpr (std::is_same<T, double>::value) {
    if constexpr (RO == 0) {
      sph_block60_c0_r0(x0, x1, x2, one, mc, sk);
      sph_block60_c1_r0(x0, x1, x2, one, mc, sk);
      sph_block60_c2_r0(x0, x1, x2, one, mc, sk);
    } else if constexpr (RO == 1) {
      if constexpr (F == 0) sph_block60_c0_r1(x0, x1, x2, one, mc, sk);
      else if constexpr (F == 1) sph_block60_c1_r1(x0, x1, x2, one, mc, sk);
      else sph_block60_c2_r1(x0, x1, x2, one, mc, sk);
    } else {
      if constexpr (F == 0) sph_block60_c0_r2(x0, x1, x2, one, mc, sk);
      else if constexpr (F == 1) sph_block60_c1_r2(x0, x1, x2, one, mc, sk);
      else sph_block60_c2_r2(x0, x1, x2, one, mc, sk);
    }
    return;
  } else {
#define IBEM_B(NM) sph_block60f##NM(x0, x1, x2, one, mc, sk)
#define IBEM_BM(NM) sph_block60fm##NM(x0, x1, x2, one, mc, sk)
  if constexpr (RO == 0) {
    IBEM_BM(_c0_r0);
    IBEM_BM(_c1_r0);
    IBEM_BM(_c2_r0);
  } else if constexpr (RO == 1) {
    if constexpr (F == 0) {
      IBEM_BM(_c0_r1);
      IBEM_BM(_c1_r1);
    } else if constexpr (F == 1) IBEM_B(_c2g0_r1);
    else if constexpr (F == 2) IBEM_B(_c2g1_r1);
    else if constexpr (F == 3) IBEM_B(_c2g2_r1);
    else if constexpr (F == 4) IBEM_B(_c2g3_r1);
    else if constexpr (F == 5) IBEM_B(_c2g4_r1);
    else IBEM_B(_c2g5_r1);
  } else {
    if constexpr (F == 0) IBEM_BM(_c0_r2);
    else if constexpr (F == 1) IBEM_B(_c1g0_r2);
    else if constexpr (F == 2) IBEM_B(_c1g1_r2);
    else if constexpr (F == 3) IBEM_B(_c1g2_r2);
    else if constexpr (F == 4) IBEM_B(_c2g0_r2);
    else if constexpr (F == 5) IBEM_B(_c2g1_r2);
    else if constexpr (F == 6) IBEM_B(_c2g2_r2);
    else if constexpr (F == 7) IBEM_B(_c2g3_r2);
    else if constexpr (F == 8) IBEM_B(_c2g4_r2);
    else IBEM_B(_c2g5_r2);
  }
#undef IBEM_B
#undef IBEM_BM
  }
}

template <int RO, int F>
__global__ void __launch_bounds__(kT)
    k_mf60_f32(const MfTile* __restrict__ tiles, const int* __restrict__ seg_begin, const int* __restrict__ mask,
               int mask_on, const float4* __restrict__ gh, const float4* __restrict__ gl,
               const SphMatF* __restrict__ mats, const float* __restrict__ x, float* __restrict__ y) {
  constexpr int NR = Rows<RO>::n;
  __shared__ float4 sgh[kChunk], sgl[kChunk];
  __shared__ float sx[kChunk * kNu];
  const MfTile t = tiles[blockIdx.x];
  if (mask && mask[t.seg] != mask_on) return;
  const int hb0 = seg_begin[t.seg], he0 = seg_begin[t.seg + 1];
  const int per = (he0 - hb0 + gridDim.y - 1) / gridDim.y;
  const int hb = hb0 + blockIdx.y * per, he = min(he0, hb + per);
  if (hb >= he) return;
  const int s = t.s0 + threadIdx.x;
  const bool act = threadIdx.x < t.ns;
  const SphMatF mc = mats[t.seg];
  const float4 ph = act ? gh[s] : make_float4(0.f, 0.f, 0.f, 1.f);
  const float4 pl = act ? gl[s] : make_float4(0.f, 0.f, 0.f, 1.f);
  float acc[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) acc[r] = 0.f;
  for (int h0 = hb; h0 < he; h0 += kChunk) {
    const int nh = min(kChunk, he - h0);
    __syncthreads();
    for (int i = threadIdx.x; i < nh; i += kT) {
      sgh[i] = gh[h0 + i];
      sgl[i] = gl[h0 + i];
    }
    for (int i = threadIdx.x; i < nh * kNu; i += kT)
      sx[i] = x[(int64_t)kNu * h0 + i] * powi(gl[h0 + i / kNu].w, RO);   // times a_h^-RO
    __syncthreads();
    if (!act) continue;
#pragma unroll 1
    for (int hh = 0; hh < nh; ++hh) {
      const float4 qh = sgh[hh], ql = sgl[hh];
      const float ia = ql.w;
      const float x0 = ((ph.x - qh.x) + (pl.x - ql.x)) * ia;
      const float x1 = ((ph.y - qh.y) + (pl.y - ql.y)) * ia;
      const float x2 = ((ph.z - qh.z) + (pl.z - ql.z)) * ia;
      RowSink<float, RO> sk{acc, sx + kNu * hh};
      blk<float, RO, F>(x0, x1, x2, mc, sk);
    }
  }
  if (!act) return;
  const float f = powi(ph.w, RO);   // a_s^RO
#pragma unroll
  for (int r = 0; r < NR; ++r) acc[r] *= f;
  if (F <= 0 && s >= hb && s < he) {   // the slice holding the target adds its self term (C0 / mu0)
    RowSink<float, RO> sk{acc, x + (int64_t)kNu * s};
    sph_self60f(mc, sk);
  }
  float* o = y + (int64_t)kNu * s + Rows<RO>::off;
#pragma unroll
  for (int r = 0; r < NR; ++r) atomicAdd(o + r, acc[r]);
}

template <int RO, int F>
__global__ void __launch_bounds__(kT)
    k_mf60_f64(const MfTile* __restrict__ tiles, const int* __restrict__ seg_begin, const int* __restrict__ mask,
               int mask_on, const double* __restrict__ cen, const double* __restrict__ rad,
               const SphMat* __restrict__ mats, const double* __restrict__ x, double* __restrict__ y) {
  constexpr int NR = Rows<RO>::n;
  __shared__ double sc[kChunk * 4];
  __shared__ double sx[kChunk * kNu];
  const MfTile t = tiles[blockIdx.x];
  if (mask && mask[t.seg] != mask_on) return;
  const int hb0 = seg_begin[t.seg], he0 = seg_begin[t.seg + 1];
  const int per = (he0 - hb0 + gridDim.y - 1) / gridDim.y;
  const int hb = hb0 + blockIdx.y * per, he = min(he0, hb + per);
  if (hb >= he) return;
  const int s = t.s0 + threadIdx.x;
  const bool act = threadIdx.x < t.ns;
  const SphMat mc = mats[t.seg];
  double p0 = 0.0, p1 = 0.0, p2 = 0.0, as = 1.0;
  if (act) {
    p0 = cen[3 * (int64_t)s];
    p1 = cen[3 * (int64_t)s + 1];
    p2 = cen[3 * (int64_t)s + 2];
    as = rad[s];
  }
  double acc[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) acc[r] = 0.0;
  for (int h0 = hb; h0 < he; h0 += kChunk) {
    const int nh = min(kChunk, he - h0);
    __syncthreads();
    for (int i = threadIdx.x; i < nh; i += kT) {
      sc[4 * i] = cen[3 * (int64_t)(h0 + i)];
      sc[4 * i + 1] = cen[3 * (int64_t)(h0 + i) + 1];
      sc[4 * i + 2] = cen[3 * (int64_t)(h0 + i) + 2];
      sc[4 * i + 3] = 1.0 / rad[h0 + i];
    }
    for (int i = threadIdx.x; i < nh * kNu; i += kT)
      sx[i] = x[(int64_t)kNu * h0 + i] * powi(1.0 / rad[h0 + i / kNu], RO);
    __syncthreads();
    if (!act) continue;
#pragma unroll 1
    for (int hh = 0; hh < nh; ++hh) {
      const double ia = sc[4 * hh + 3];
      const double x0 = (p0 - sc[4 * hh]) * ia, x1 = (p1 - sc[4 * hh + 1]) * ia, x2 = (p2 - sc[4 * hh + 2]) * ia;
      RowSink<double, RO> sk{acc, sx + kNu * hh};
      blk<double, RO, F>(x0, x1, x2, mc, sk);
    }
  }
  if (!act) return;
  const double f = powi(as, RO);
#pragma unroll
  for (int r = 0; r < NR; ++r) acc[r] *= f;
  if (F <= 0 && s >= hb && s < he) {
    RowSink<double, RO> sk{acc, x + (int64_t)kNu * s};
    sph_self60(mc, sk);
  }
  double* o = y + (int64_t)kNu * s + Rows<RO>::off;
#pragma unroll
  for (int r = 0; r < NR; ++r) atomicAdd(o + r, acc[r]);
}

// Scaled diagonal block of a realisation (unit sphere at x = 0 plus C0, moduli / mu0) inverted
// by Gauss-Jordan with partial pivoting in FP64: one CTA of 64 threads per realisation, the
// 60 x 120 augmented matrix in dynamic shared memory (57.6 KB).
constexpr int kBjThreads = 64;
constexpr size_t kBjSmem = sizeof(double) * kNu * (2 * kNu + 1);
__global__ void __launch_bounds__(kBjThreads) k_block_jacobi60(const SphMat* __restrict__ mats, float* __restrict__ P) {
  extern __shared__ double smem[];
  double (*M)[2 * kNu + 1] = reinterpret_cast<double (*)[2 * kNu + 1]>(smem);
  __shared__ int piv;
  __shared__ double f[kNu];
  const int p = blockIdx.x;
  const int t = threadIdx.x;
  for (int i = t; i < kNu * 2 * kNu; i += kBjThreads) {
    const int r = i / (2 * kNu), c = i % (2 * kNu);
    M[r][c] = (c >= kNu && c - kNu == r) ? 1.0 : 0.0;
  }
  __syncthreads();
  if (t == 0) {
    SphMat mc = mats[p];
    struct Put {
      double (*M)[2 * kNu + 1];
      __device__ void operator()(int r, int c, double v) const { M[r][c] += v; }
    } put{M};
    sph_block60_c0_r0(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_block60_c1_r0(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_block60_c2_r0(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_block60_c0_r1(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_block60_c1_r1(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_block60_c2_r1(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_block60_c0_r2(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_block60_c1_r2(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_block60_c2_r2(0.0, 0.0, 0.0, 1.0, mc, put);
    sph_self60(mc, put);
  }
  __syncthreads();
  for (int k = 0; k < kNu; ++k) {
    if (t == 0) {
      int best = k;
      for (int r = k + 1; r < kNu; ++r)
        if (fabs(M[r][k]) > fabs(M[best][k])) best = r;
      piv = best;
    }
    __syncthreads();
    const int pr = piv;
    if (pr != k)
      for (int c = t; c < 2 * kNu; c += kBjThreads) {
        const double v = M[k][c];
        M[k][c] = M[pr][c];
        M[pr][c] = v;
      }
    __syncthreads();
    const double d = M[k][k];
    const double id = d != 0.0 ? 1.0 / d : 0.0;
    __syncthreads();
    for (int c = t; c < 2 * kNu; c += kBjThreads) M[k][c] *= id;
    for (int r = t; r < kNu; r += kBjThreads) f[r] = M[r][k];
    __syncthreads();
    for (int i = t; i < kNu * 2 * kNu; i += kBjThreads) {
      const int r = i / (2 * kNu), c = i % (2 * kNu);
      if (r != k) M[r][c] -= f[r] * M[k][c];
    }
    __syncthreads();
  }
  float* o = P + (int64_t)kNu * kNu * p;
  for (int i = t; i < kNu * kNu; i += kBjThreads) o[i] = (float)M[i / kNu][kNu + i % kNu];
}

// z = P v with the realisation's block (Pseg[seg], 60 x 60 row-major); kdev: v is column
// *kdev of a basis with column stride vstride (graph-captured Arnoldi steps)
__global__ void k_precond_apply60(int num, const int* __restrict__ seg_of, const float* __restrict__ Pseg,
                                  const float* __restrict__ v, float* __restrict__ z, const int* __restrict__ kdev,
                                  int64_t vstride) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)num * kNu) return;
  if (kdev) v += (int64_t)(*kdev) * vstride;
  const int64_t p = t / kNu;
  const int r = (int)(t % kNu);
  const float* row = Pseg + (int64_t)seg_of[p] * kNu * kNu + (int64_t)r * kNu;
  const float* vp = v + p * kNu;
  float s = 0.f;
#pragma unroll 4
  for (int c = 0; c < kNu; ++c) s = fmaf(row[c], vp[c], s);
  z[t] = s;
}

}  // namespace

// FP32: 18 launches (row order 0; row order 1 in 7 column groups; row order 2 in 10)
#define IBEM_MF60_ALL(K, ...)                                                                            \
  K(0, -1, __VA_ARGS__); K(1, 0, __VA_ARGS__); K(1, 1, __VA_ARGS__); K(1, 2, __VA_ARGS__); K(1, 3, __VA_ARGS__); \
  K(1, 4, __VA_ARGS__); K(1, 5, __VA_ARGS__); K(1, 6, __VA_ARGS__); K(2, 0, __VA_ARGS__); K(2, 1, __VA_ARGS__); \
  K(2, 2, __VA_ARGS__); K(2, 3, __VA_ARGS__); K(2, 4, __VA_ARGS__); K(2, 5, __VA_ARGS__); K(2, 6, __VA_ARGS__); \
  K(2, 7, __VA_ARGS__); K(2, 8, __VA_ARGS__); K(2, 9, __VA_ARGS__)

ibem_status mf60_apply_f32(const MfBatch& b, const float* x, float* y, cudaStream_t st, const int* mask,
                           int mask_on) {
  const dim3 grid(b.ntiles_s[1], b.hsplit);
#define IBEM_MF60_F32(RO, F, unused)                                                                           \
  ::ibem::count_launch(), k_mf60_f32<RO, F><<<grid, kT, 0, st>>>(b.tiles_s[1], b.seg_begin, mask, mask_on, b.gh, \
                                                                  b.gl, b.matf, x, y)
  IBEM_MF60_ALL(IBEM_MF60_F32, 0);
#undef IBEM_MF60_F32
  IBEM_LAUNCH_CHECK("mf60 apply f32");
  return IBEM_OK;
}

// FP64: 7 launches (row order 0; row orders 1 and 2 one column order at a time)
ibem_status mf60_apply_f64(const MfBatch& b, const double* x, double* y, cudaStream_t st, const int* mask,
                           int mask_on) {
  const dim3 grid(b.ntiles_s[1], b.hsplit_wide);
#define IBEM_MF60_F64(RO, F)                                                                                     \
  ::ibem::count_launch(), k_mf60_f64<RO, F><<<grid, kT, 0, st>>>(b.tiles_s[1], b.seg_begin, mask, mask_on, b.cen, \
                                                                  b.rad, b.mats, x, y)
  IBEM_MF60_F64(0, -1);
  IBEM_MF60_F64(1, 0);
  IBEM_MF60_F64(1, 1);
  IBEM_MF60_F64(1, 2);
  IBEM_MF60_F64(2, 0);
  IBEM_MF60_F64(2, 1);
  IBEM_MF60_F64(2, 2);
#undef IBEM_MF60_F64
  IBEM_LAUNCH_CHECK("mf60 apply f64");
  return IBEM_OK;
}
#undef IBEM_MF60_ALL

ibem_status mf60_block_jacobi(const MfBatch& b, float* Pseg, cudaStream_t st) {
  IBEM_CUDA(cudaFuncSetAttribute(k_block_jacobi60, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBjSmem));
  ::ibem::count_launch(), k_block_jacobi60<<<b.nseg, kBjThreads, kBjSmem, st>>>(b.mats, Pseg);
  IBEM_LAUNCH_CHECK("mf60 block jacobi");
  return IBEM_OK;
}

ibem_status mf60_precond_apply(const MfBatch& b, const float* Pseg, const float* v, float* z, const int* kdev,
                               int64_t vstride, cudaStream_t st) {
  const int64_t n = (int64_t)b.num * kNu;
  ::ibem::count_launch(), k_precond_apply60<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(b.num, b.seg_of, Pseg, v, z,
                                                                                       kdev, vstride);
  IBEM_LAUNCH_CHECK("mf60 preconditioner");
  return IBEM_OK;
}

}  // namespace ibem
