// Sphere kernels for the 24-unknown layout (eigenstrain orders 0 and 1).
#include "field_contract.cuh"
#include "gen_sphere24.cuh"
#include "prof.h"
#include "sphere_kernels.cuh"

#include <cub/device/device_radix_sort.cuh>

IBEM_PAIR_KERNEL(pair24_c0_r0, sph_block24_c0_r0, 24)
IBEM_PAIR_KERNEL(pair24_c0_r1, sph_block24_c0_r1, 24)
IBEM_PAIR_KERNEL(pair24_c1_r0, sph_block24_c1_r0, 24)
IBEM_PAIR_KERNEL(pair24_c1_r1, sph_block24_c1_r1, 24)
IBEM_SELF_KERNEL(self24, sph_self24, 24)
IBEM_NODE_KERNEL(node24, sph_node24, 24)
IBEM_FIELD_KERNEL(field24, sph_field24_contracted, 24)

// Field sum of the mixed form: the same contraction in double-float arithmetic
// (field_contract.cuh), split by distance.  Points are processed in Morton order (a stable
// radix sort of 30-bit keys inside the point cloud's bounding box), so the 32 points of a
// warp form a compact cluster; a sphere that lies beyond kFarRadii radii from all 32 of them
// is summed in FP32 (sph_field24_f32), every other one in double-float.  Two kernels, one
// code path each (a single loop over both paths stalled on instruction fetch, and the
// double-float path's registers limited the FP32 path's occupancy):
//   field24_far   every (warp, sphere) pair: the distance test, the FP32 sum of the far
//                 spheres (Kahan-compensated per chunk of 64 spheres, then added to
//                 double-float accumulators: as accurate as a double-float sum of every
//                 term, at 4 instead of ~10 FP32 adds), and per (warp, chunk) a 64-bit
//                 mask of the near spheres;
//   field24_near  per warp, the spheres of its masks in double-float (compensated dot
//                 products; each warp stages one sphere's constants at a time in its own
//                 shared slot: no block barriers), then the inside test, the local
//                 eigenstrain and C0 in FP64.
// Per-sphere double-float constants (SphDF, scaled coordinates) are made once per call.
__global__ void k_sph_df(int num, const double* __restrict__ cen, const double* __restrict__ rad,
                         const double* __restrict__ E, ibem::SphDF* __restrict__ out) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h < num) out[h] = ibem::sph_df_make(cen + 3 * (int64_t)h, rad[h], E + 24 * (int64_t)h);
}

__global__ void __launch_bounds__(ibem::kFieldThreads)
    field24_far(const double* __restrict__ pts, const int* __restrict__ order, int nump,
                const ibem::SphDF* __restrict__ sph, int num, float tn1, float tn2,
                unsigned long long* __restrict__ nmask, int nchunk, ibem::dfloat* __restrict__ accbuf) {
  static_assert(sizeof(ibem::SphDF) == 18 * sizeof(float4), "SphDF is copied as 18 float4");
  static_assert(ibem::kFieldChunk == 64, "the near-sphere mask of a chunk is 64 bits");
  __shared__ __align__(16) ibem::SphDF ss[ibem::kFieldChunk];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = t < nump;
  const bool warp_act = (t & ~31) < nump;
  const int s = act ? order[t] : 0;
  ibem::dfloat pd[3] = {};
  if (act)
    for (int k = 0; k < 3; ++k) pd[k] = ibem::df_make(pts[3 * (int64_t)s + k]);
  const float far2 = ibem::kFarRadii * ibem::kFarRadii;
  ibem::dfloat acc[6] = {};
  for (int h0 = 0, c = 0; h0 < num; h0 += ibem::kFieldChunk, ++c) {
    const int nh = min(ibem::kFieldChunk, num - h0);
    __syncthreads();
    {
      const float4* src = reinterpret_cast<const float4*>(sph + h0);
      float4* dst = reinterpret_cast<float4*>(ss);
      for (int i = threadIdx.x; i < nh * 18; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    unsigned long long near = 0;
    float sum[6] = {}, comp[6] = {};   // Kahan sums of the chunk's far spheres
#pragma unroll 1
    for (int hh = 0; hh < nh; ++hh) {
      const ibem::SphDF& sp = ss[hh];
      const float dx = (pd[0].hi - sp.c[0].hi) * sp.ia.hi, dy = (pd[1].hi - sp.c[1].hi) * sp.ia.hi,
                  dz = (pd[2].hi - sp.c[2].hi) * sp.ia.hi;
      const bool far = !act || dx * dx + dy * dy + dz * dz > far2;
      if (__all_sync(0xffffffffu, far)) {
        if (act) {
          float r[6];
          ibem::sph_field24_f32(pd, sp, tn1, tn2, r);
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            const float y = r[k] - comp[k], u = sum[k] + y;
            comp[k] = (u - sum[k]) - y;
            sum[k] = u;
          }
        }
      } else {
        near |= 1ull << hh;
      }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      ibem::df_add_f(acc[k], sum[k]);
      ibem::df_add_f(acc[k], -comp[k]);
    }
    if (warp_act && (threadIdx.x & 31) == 0) nmask[(int64_t)(t >> 5) * nchunk + c] = near;
  }
  if (act)
#pragma unroll
    for (int k = 0; k < 6; ++k) accbuf[6 * (int64_t)t + k] = acc[k];
}

__global__ void __launch_bounds__(ibem::kFieldThreads)
    field24_near(const double* __restrict__ pts, const int* __restrict__ order, int nump,
                 const double* __restrict__ cen, const ibem::SphDF* __restrict__ sph, SphMat mc,
                 const double* __restrict__ E, const unsigned long long* __restrict__ nmask, int nchunk,
                 const ibem::dfloat* __restrict__ accbuf, double* __restrict__ stress) {
  __shared__ __align__(16) ibem::SphDF ss[ibem::kFieldThreads / 32];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if ((t & ~31) >= nump) return;   // whole warp past the end (no block barriers below)
  const bool act = t < nump;
  const int s = act ? order[t] : 0;
  double p0 = 0, p1 = 0, p2 = 0;
  if (act) { p0 = pts[3 * (int64_t)s]; p1 = pts[3 * (int64_t)s + 1]; p2 = pts[3 * (int64_t)s + 2]; }
  const ibem::dfloat pd[3] = {ibem::df_make(p0), ibem::df_make(p1), ibem::df_make(p2)};
  const ibem::dfloat tn1 = ibem::df_make(mc.tn1), tn2 = ibem::df_make(mc.tn2);
  ibem::dacc acc[6] = {};
  if (act)
#pragma unroll
    for (int k = 0; k < 6; ++k) acc[k] = ibem::dacc_of(accbuf[6 * (int64_t)t + k]);
  ibem::SphDF& sp = ss[threadIdx.x >> 5];
  const unsigned long long* wm = nmask + (int64_t)(t >> 5) * nchunk;
  int inside = -1;
#pragma unroll 1
  for (int c = 0; c < nchunk; ++c) {
    unsigned long long near = wm[c];
#pragma unroll 1
    while (near) {
      const int h = c * ibem::kFieldChunk + __ffsll((long long)near) - 1;
      near &= near - 1;
      __syncwarp();
      if (lane < 18) reinterpret_cast<float4*>(&sp)[lane] = reinterpret_cast<const float4*>(sph + h)[lane];
      __syncwarp();
      if (act && ibem::sph_field24_df(pd, sp, tn1, tn2, acc)) inside = h;
    }
  }
  if (!act) return;
  double e[6];
  for (int r = 0; r < 6; ++r) e[r] = mc.kd * ((double)acc[r].s + (double)acc[r].c);
  if (inside >= 0) {
    const double* Ei = E + 24 * (int64_t)inside;
    const double x0 = p0 - cen[3 * inside], x1 = p1 - cen[3 * inside + 1], x2 = p2 - cen[3 * inside + 2];
    for (int r = 0; r < 6; ++r) e[r] -= local_eigenstrain<24>(Ei, r, x0, x1, x2);
  }
  const double tr = e[0] + e[3] + e[5];
  double* o = stress + 6 * (int64_t)s;
  o[0] += mc.lam0 * tr + 2.0 * mc.mu0 * e[0];
  o[1] += 2.0 * mc.mu0 * e[1];
  o[2] += 2.0 * mc.mu0 * e[2];
  o[3] += mc.lam0 * tr + 2.0 * mc.mu0 * e[3];
  o[4] += 2.0 * mc.mu0 * e[4];
  o[5] += mc.lam0 * tr + 2.0 * mc.mu0 * e[5];
}

// Bounding box of the points (FP64 min / max, atomics on the ordered integer image).
__device__ __forceinline__ unsigned long long ord_key(double v) {
  const unsigned long long b = __double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_val(unsigned long long k) {
  return __longlong_as_double((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k);
}
__global__ void k_bbox(int n, const double* __restrict__ pts, unsigned long long* __restrict__ box) {
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int k = 0; k < 3; ++k) {
      const unsigned long long o = ord_key(pts[3 * (int64_t)i + k]);
      lo[k] = o < lo[k] ? o : lo[k];
      hi[k] = o > hi[k] ? o : hi[k];
    }
  for (int k = 0; k < 3; ++k) {  // warp minimum / maximum first: one atomic per warp
    for (int off = 16; off; off >>= 1) {
      const unsigned long long ol = __shfl_xor_sync(0xffffffffu, lo[k], off);
      const unsigned long long oh = __shfl_xor_sync(0xffffffffu, hi[k], off);
      lo[k] = ol < lo[k] ? ol : lo[k];
      hi[k] = oh > hi[k] ? oh : hi[k];
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(box + k, lo[k]);
      atomicMax(box + 3 + k, hi[k]);
    }
  }
}
__device__ __forceinline__ unsigned spread3(unsigned v) {  // 10 bits -> every third bit
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
__global__ void k_morton(int n, const double* __restrict__ pts, const unsigned long long* __restrict__ box,
                         unsigned* __restrict__ key, int* __restrict__ idx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned q[3];
  for (int k = 0; k < 3; ++k) {
    const double lo = ord_val(box[k]), hi = ord_val(box[3 + k]);
    const double span = hi > lo ? hi - lo : 1.0;
    const double f = (pts[3 * (int64_t)i + k] - lo) / span;
    q[k] = (unsigned)min(1023.0, max(0.0, f * 1024.0));
  }
  key[i] = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
  idx[i] = i;
}

namespace ibem {

ibem_status launch_pair24(const SphLaunch& p, double* A, int64_t lda, int64_t row0, int64_t col0,
                          cudaStream_t st) {
  SphMat mc = sph_mat_init(p.E0, p.nu0, p.E1, p.nu1);
  ProfScope ps(PROF_PAIR, st);
  double* base = A + col0 * lda + row0;
  dim3 grid((p.num + kPairThreads - 1) / kPairThreads, p.num);
  ::ibem::count_launch(), pair24_c0_r0<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), pair24_c0_r1<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), pair24_c1_r0<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), pair24_c1_r1<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), self24<<<(p.num + 127) / 128, 128, 0, st>>>(p.num, mc, base, lda);
  IBEM_LAUNCH_CHECK("pair24");
  return IBEM_OK;
}

ibem_status launch_node24(const SphLaunch& p, const double* nodes, int NN, double* H, int64_t ldh,
                          int64_t row0, int64_t col0, cudaStream_t st) {
  SphMat mc = sph_mat_init(p.E0, p.nu0, p.E1, p.nu1);
  dim3 grid((NN + kPairThreads - 1) / kPairThreads, p.num);
  ::ibem::count_launch(), node24<<<grid, kPairThreads, 0, st>>>(nodes, NN, p.cen, p.rad, mc, H + col0 * ldh + row0, ldh);
  IBEM_LAUNCH_CHECK("node24");
  return IBEM_OK;
}

ibem_status launch_field24(const SphLaunch& p, const double* pts, int nump, const double* E,
                           double* stress, cudaStream_t st) {
  SphMat mc = sph_mat_init(p.E0, p.nu0, p.E1, p.nu1);
  ProfScope ps(PROF_FIELD, st);
  ::ibem::count_launch(), field24<<<(nump + kFieldThreads - 1) / kFieldThreads, kFieldThreads, 0, st>>>(
      pts, nump, p.cen, p.rad, p.num, mc, E, stress);
  IBEM_LAUNCH_CHECK("field24");
  return IBEM_OK;
}

ibem_status launch_field24_df(const SphLaunch& p, const double* pts, int nump, const double* E,
                              double* stress, cudaStream_t st) {
  if (nump <= 0) return IBEM_OK;
  SphMat mc = sph_mat_init(p.E0, p.nu0, p.E1, p.nu1);
  ProfScope ps(PROF_FIELD, st);
  // stream-ordered scratch: Morton keys and indices, sort workspace, sphere constants, the
  // near masks (one 64-bit word per warp and chunk of spheres) and the far sums
  const unsigned nb = (unsigned)((nump + 255) / 256);
  size_t sort_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, (const unsigned*)nullptr, (unsigned*)nullptr,
                                  (const int*)nullptr, (int*)nullptr, nump, 0, 30, st);
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const int nchunk = (p.num + kFieldChunk - 1) / kFieldChunk;
  const int64_t nwarp = (nump + 31) / 32;
  const size_t n4 = up((size_t)nump * 4);
  const size_t nsph = up((size_t)p.num * sizeof(SphDF));
  const size_t nmsk = up((size_t)nwarp * (size_t)nchunk * 8);
  const size_t nacc = up((size_t)nump * 6 * sizeof(dfloat));
  const size_t bytes = 256 + 4 * n4 + nsph + nmsk + nacc + sort_bytes;
  char* buf = nullptr;
  IBEM_CUDA(cudaMallocAsync((void**)&buf, bytes, st));
  unsigned long long* box = reinterpret_cast<unsigned long long*>(buf);
  char* q = buf + 256;
  unsigned* k0 = reinterpret_cast<unsigned*>(q);
  unsigned* k1 = reinterpret_cast<unsigned*>(q + n4);
  int* i0 = reinterpret_cast<int*>(q + 2 * n4);
  int* i1 = reinterpret_cast<int*>(q + 3 * n4);
  q += 4 * n4;
  SphDF* sph = reinterpret_cast<SphDF*>(q);
  q += nsph;
  unsigned long long* nmask = reinterpret_cast<unsigned long long*>(q);
  q += nmsk;
  dfloat* accbuf = reinterpret_cast<dfloat*>(q);
  q += nacc;
  void* tmp = q;
  ibem_status s = IBEM_OK;
  // box = (min, min, min, max, max, max) starts at (all ones, zeros) in the ordered-integer image
  cudaError_t e = cudaMemsetAsync(box, 0xff, 3 * sizeof(unsigned long long), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(box + 3, 0, 3 * sizeof(unsigned long long), st);
  if (e == cudaSuccess) {
    ::ibem::count_launch(), k_bbox<<<min(nb, 304u), 256, 0, st>>>(nump, pts, box);
    ::ibem::count_launch(), k_morton<<<nb, 256, 0, st>>>(nump, pts, box, k0, i0);
    if (p.num > 0) ::ibem::count_launch(), k_sph_df<<<(p.num + 127) / 128, 128, 0, st>>>(p.num, p.cen, p.rad, E, sph);
    e = cub::DeviceRadixSort::SortPairs(tmp, sort_bytes, k0, k1, i0, i1, nump, 0, 30, st);
  }
  if (e == cudaSuccess) {
    const unsigned grid = (unsigned)((nump + kFieldThreads - 1) / kFieldThreads);
    ::ibem::count_launch(), field24_far<<<grid, kFieldThreads, 0, st>>>(
        pts, i1, nump, sph, p.num, (float)mc.tn1, (float)mc.tn2, nmask, nchunk, accbuf);
    ::ibem::count_launch(), field24_near<<<grid, kFieldThreads, 0, st>>>(pts, i1, nump, p.cen, sph, mc, E, nmask,
                                                                        nchunk, accbuf, stress);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) s = cuda_fail(e, "field24_df");
  cudaFreeAsync(buf, st);
  return s;
}

}  // namespace ibem
