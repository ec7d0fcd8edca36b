// Ellipsoidal inclusions on the GPU: pair blocks of the equivalent-inclusion system and
// stress sums at sample points, layout 24 (eigenstrain orders 0 and 1), boundary-free
// cases under a remote stress.  The evaluation itself is ellipsoid.cuh (host/device).
//
// No reference counterpart: the reference's elastic integrator handles spheres only
// (integratorElastic3DHelper.cpp:41-664); the block and sum definitions are its
// integratorElastic3D.cpp:341-567 and postProcessorElastic3D.cpp:367-470 with the
// sphere's potentials replaced by the ellipsoid's.
//
// pair blocks: one thread per (target s, source h); a warp takes 32 consecutive targets of
//   one source, so the source's geometry is a broadcast load.  Each thread forms its 24 x 24
//   block in FP64 (the FP64 pipe bounds the kernel); the warp then writes the blocks one
//   column at a time through shared memory, so that every store instruction covers
//   consecutive rows (the 32 blocks of a warp are 768 consecutive rows of each column).
// stress sums: one thread per sample point and source slice (blockIdx.y; enough slices
//   to fill the GPU when there are few points), sources staged through shared memory in
//   chunks; the mixed form evaluates a source in FP32 (coordinates scaled by its longest
//   semi-axis) when it lies beyond kEllFarAxes of those axes from all 32 points of the
//   warp and in FP64 otherwise, the FP64 form in FP64 throughout.  The slices' partial sums
//   are added in slice order by a second kernel (no atomics: the same stresses on every run).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "ellipsoid.cuh"
#include "ibem_internal.h"
#include "prof.h"
#include "solver.h"

namespace ibem {
namespace {

constexpr int kEllPairThreads = 64;
constexpr int kEllFieldThreads = 128;
constexpr int kEllChunk = 32;
constexpr float kEllFarAxes = 14.0f;

__global__ void k_ell_rot(int num, const double* __restrict__ quat, double* __restrict__ Q) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h < num) ell::quat_to_rot(quat + 4 * (int64_t)h, Q + 9 * (int64_t)h);
}

__global__ void __launch_bounds__(kEllPairThreads) k_ell_pair24(const double* __restrict__ cen,
                                                                const double* __restrict__ axes,
                                                                const double* __restrict__ Qall, int num, SphMat mc,
                                                                double* __restrict__ A, int64_t lda) {
  __shared__ double stage[kEllPairThreads / 32][32 * 24];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int h = blockIdx.y;
  const int s0 = s - lane;
  if (s0 >= num) return;   // whole warp past the end
  const int nact = min(32, num - s0);
  const bool act = s < num;
  double blk[576];
  if (act) {
    double d[3], Q[9], a[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      d[i] = cen[3 * (int64_t)s + i] - cen[3 * (int64_t)h + i];
      a[i] = axes[3 * (int64_t)h + i];
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) Q[i] = Qall[9 * (int64_t)h + i];
    ell::ell_block24<double>(d, Q, a, mc, s == h, blk);
  }
  double* base = A + 24 * (int64_t)h * lda + 24 * (int64_t)s0;
  for (int c = 0; c < 24; ++c) {
    if (act)
#pragma unroll 4
      for (int r = 0; r < 24; ++r) stage[warp][lane * 24 + r] = blk[r * 24 + c];
    __syncwarp();
    for (int i = lane; i < 24 * nact; i += 32) base[(int64_t)c * lda + i] = stage[warp][i];
    __syncwarp();
  }
}

struct EllRec {
  double c[3], a[3], Q[9], E[24];
};

// Partial strain sums of the ellipsoids of one source slice (blockIdx.y) at every point:
// part[(slice * nump + t) * 6 + k], and the last ellipsoid of the slice that holds the point
// (or -1) in inside_part[slice * nump + t].
__global__ void __launch_bounds__(kEllFieldThreads) k_ell_field24(const double* __restrict__ pts, int nump,
                                                                  const double* __restrict__ cen,
                                                                  const double* __restrict__ axes,
                                                                  const double* __restrict__ Qall, int num, SphMat mc,
                                                                  const double* __restrict__ E, int mixed,
                                                                  double* __restrict__ part,
                                                                  int* __restrict__ inside_part) {
  __shared__ EllRec sr[kEllChunk];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = t < nump;
  const int per = (num + gridDim.y - 1) / gridDim.y;
  const int hb = blockIdx.y * per, he = min(num, hb + per);
  double p[3] = {0, 0, 0};
  if (act)
#pragma unroll
    for (int i = 0; i < 3; ++i) p[i] = pts[3 * (int64_t)t + i];
  double e[6] = {0, 0, 0, 0, 0, 0};
  int inside = -1;
  for (int h0 = hb; h0 < he; h0 += kEllChunk) {
    const int nh = min(kEllChunk, he - h0);
    __syncthreads();
    for (int i = threadIdx.x; i < nh * 39; i += blockDim.x) {
      const int hh = i / 39, f = i % 39;
      const int64_t hg = h0 + hh;
      double v;
      if (f < 3) v = cen[3 * hg + f];
      else if (f < 6) v = axes[3 * hg + f - 3];
      else if (f < 15) v = Qall[9 * hg + f - 6];
      else v = E[24 * hg + f - 15];
      reinterpret_cast<double*>(&sr[hh])[f] = v;
    }
    __syncthreads();
#pragma unroll 1
    for (int hh = 0; hh < nh; ++hh) {
      const EllRec& r = sr[hh];
      const double d[3] = {p[0] - r.c[0], p[1] - r.c[1], p[2] - r.c[2]};
      const double amax = fmax(r.a[0], fmax(r.a[1], r.a[2]));
      const double dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      const bool far = !act || dd > (double)(kEllFarAxes * kEllFarAxes) * amax * amax;
      if (mixed && __all_sync(0xffffffffu, far)) {
        if (act) {
          const float is = (float)(1.0 / amax);
          float df[3], af[3], Qf[9], Ef[24], ef[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            df[i] = (float)d[i] * is;
            af[i] = (float)r.a[i] * is;
          }
#pragma unroll
          for (int i = 0; i < 9; ++i) Qf[i] = (float)r.Q[i];
#pragma unroll
          for (int i = 0; i < 24; ++i) Ef[i] = (float)(i < 6 ? r.E[i] : r.E[i] * amax);
          ell::ell_strain24<float>(df, Qf, af, mc, Ef, ef);
#pragma unroll
          for (int i = 0; i < 6; ++i) e[i] += (double)ef[i];
        }
      } else if (act) {
        if (ell::ell_strain24<double>(d, r.Q, r.a, mc, r.E, e)) inside = h0 + hh;
      }
    }
  }
  if (!act) return;
  const int64_t o = (int64_t)blockIdx.y * nump + t;
#pragma unroll
  for (int k = 0; k < 6; ++k) part[6 * o + k] = e[k];
  inside_part[o] = inside;
}

// Sum of the slices in slice order (the same on every run), the local eigenstrain of the
// last ellipsoid holding the point (postProcessorElastic3D.cpp:383-433), stress += C0 : e.
__global__ void k_ell_field_reduce(int nump, int nsl, const double* __restrict__ part,
                                   const int* __restrict__ inside_part, const double* __restrict__ pts,
                                   const double* __restrict__ cen, const double* __restrict__ E, SphMat mc,
                                   double* __restrict__ stress) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nump) return;
  double e[6] = {0, 0, 0, 0, 0, 0};
  int inside = -1;
  for (int sl = 0; sl < nsl; ++sl) {
    const int64_t o = (int64_t)sl * nump + t;
#pragma unroll
    for (int k = 0; k < 6; ++k) e[k] += part[6 * o + k];
    inside = max(inside, inside_part[o]);
  }
  if (inside >= 0) {
    const double* Ei = E + 24 * (int64_t)inside;
    const double d[3] = {pts[3 * (int64_t)t] - cen[3 * (int64_t)inside],
                         pts[3 * (int64_t)t + 1] - cen[3 * (int64_t)inside + 1],
                         pts[3 * (int64_t)t + 2] - cen[3 * (int64_t)inside + 2]};
    for (int r = 0; r < 6; ++r) e[r] -= Ei[r] + Ei[6 + 3 * r] * d[0] + Ei[7 + 3 * r] * d[1] + Ei[8 + 3 * r] * d[2];
  }
  const double tr = e[0] + e[3] + e[5];
  double* o = stress + 6 * (int64_t)t;
  o[0] += mc.lam0 * tr + 2.0 * mc.mu0 * e[0];
  o[1] += 2.0 * mc.mu0 * e[1];
  o[2] += 2.0 * mc.mu0 * e[2];
  o[3] += mc.lam0 * tr + 2.0 * mc.mu0 * e[3];
  o[4] += 2.0 * mc.mu0 * e[4];
  o[5] += mc.lam0 * tr + 2.0 * mc.mu0 * e[5];
}

__global__ void k_ell_fill6(int nump, double s0, double s1, double s2, double s3, double s4, double s5,
                            double* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 6 * (int64_t)nump) return;
  const int k = (int)(i % 6);
  out[i] = k == 0 ? s0 : k == 1 ? s1 : k == 2 ? s2 : k == 3 ? s3 : k == 4 ? s4 : s5;
}

ibem_status check_geometry(const double* c, const double* a, const double* q, int num, const char* who) {
  if (num < 0 || (num && (!c || !a || !q))) return fail(IBEM_ERR_ARG, std::string(who) + ": bad arguments");
  if (num > 65535) return fail(IBEM_ERR_ARG, std::string(who) + ": at most 65535 ellipsoids per call");
  return IBEM_OK;
}

}  // namespace

ibem_status ell_rotations(const double* quat, int num, double* Q, cudaStream_t st) {
  if (num <= 0) return IBEM_OK;
  ::ibem::count_launch(), k_ell_rot<<<(num + 127) / 128, 128, 0, st>>>(num, quat, Q);
  IBEM_LAUNCH_CHECK("ell rotations");
  return IBEM_OK;
}

}  // namespace ibem

using namespace ibem;

extern "C" {

ibem_status ibem_e3d_ell_pair_blocks(const double* centers_dev, const double* axes_dev, const double* quats_dev,
                                     int num, const ibem_material* mat, double* A_dev, int64_t lda, int64_t row0,
                                     int64_t col0, void* stream) {
  ibem_status s = check_geometry(centers_dev, axes_dev, quats_dev, num, "ell_pair_blocks");
  if (s) return s;
  if (!mat || (num && !A_dev) || row0 < 0 || col0 < 0) return fail(IBEM_ERR_ARG, "ell_pair_blocks: bad arguments");
  if (lda < row0 + 24 * (int64_t)num) return fail(IBEM_ERR_ARG, "ell_pair_blocks: lda too small");
  if (num == 0) return IBEM_OK;
  cudaStream_t st = as_stream(stream);
  double* Q = nullptr;
  IBEM_CUDA(cudaMallocAsync((void**)&Q, sizeof(double) * 9 * (size_t)num, st));
  s = ell_rotations(quats_dev, num, Q, st);
  if (!s) {
    const SphMat mc = sph_mat_init(mat->E0, mat->nu0, mat->E1, mat->nu1);
    ProfScope ps(PROF_PAIR, st);
    dim3 grid((unsigned)((num + kEllPairThreads - 1) / kEllPairThreads), (unsigned)num);
    ::ibem::count_launch(), k_ell_pair24<<<grid, kEllPairThreads, 0, st>>>(centers_dev, axes_dev, Q, num, mc,
                                                                           A_dev + col0 * lda + row0, lda);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) s = cuda_fail(e, "ell_pair_blocks");
  }
  cudaFreeAsync(Q, st);
  return s;
}

ibem_status ibem_e3d_ell_field(ibem_solver_form form, const double* points_dev, int nump, const double* centers_dev,
                               const double* axes_dev, const double* quats_dev, int num, const ibem_material* mat,
                               const double* E_dev, const double* sig_inf, double* stress_dev, void* stream) {
  ibem_status s = check_geometry(centers_dev, axes_dev, quats_dev, num, "ell_field");
  if (s) return s;
  if (!mat || nump < 0 || (nump && (!points_dev || !stress_dev)) || (num && !E_dev))
    return fail(IBEM_ERR_ARG, "ell_field: bad arguments");
  if (form != IBEM_SOLVE_FP64 && form != IBEM_SOLVE_MIXED_IR) return fail(IBEM_ERR_ARG, "ell_field: unknown form");
  if (nump == 0) return IBEM_OK;
  cudaStream_t st = as_stream(stream);
  double sg[6] = {0, 0, 0, 0, 0, 0};
  if (sig_inf)
    for (int i = 0; i < 6; ++i) sg[i] = sig_inf[i];
  ::ibem::count_launch(), k_ell_fill6<<<(unsigned)((6 * (int64_t)nump + 255) / 256), 256, 0, st>>>(
      nump, sg[0], sg[1], sg[2], sg[3], sg[4], sg[5], stress_dev);
  IBEM_LAUNCH_CHECK("ell_field init");
  if (num == 0) return IBEM_OK;
  double* Q = nullptr;
  IBEM_CUDA(cudaMallocAsync((void**)&Q, sizeof(double) * 9 * (size_t)num, st));
  s = ell_rotations(quats_dev, num, Q, st);
  if (!s) {
    const SphMat mc = sph_mat_init(mat->E0, mat->nu0, mat->E1, mat->nu1);
    ProfScope ps(PROF_FIELD, st);
    // source slices: about 8 CTAs per SM in total, at least one chunk of sources per slice
    int dev = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int gx = (nump + kEllFieldThreads - 1) / kEllFieldThreads;
    const int nsl = std::max(1, std::min((8 * nsm + gx - 1) / gx, (num + kEllChunk - 1) / kEllChunk));
    double* part = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&part, (sizeof(double) * 6 + sizeof(int)) * (size_t)nsl * nump, st);
    if (e == cudaSuccess) {
      int* inside = reinterpret_cast<int*>(part + 6 * (size_t)nsl * nump);
      ::ibem::count_launch(), k_ell_field24<<<dim3((unsigned)gx, (unsigned)nsl), kEllFieldThreads, 0, st>>>(
          points_dev, nump, centers_dev, axes_dev, Q, num, mc, E_dev, form == IBEM_SOLVE_MIXED_IR ? 1 : 0, part,
          inside);
      ::ibem::count_launch(), k_ell_field_reduce<<<(unsigned)((nump + 255) / 256), 256, 0, st>>>(
          nump, nsl, part, inside, points_dev, centers_dev, E_dev, mc, stress_dev);
      e = cudaGetLastError();
      cudaFreeAsync(part, st);
    }
    if (e != cudaSuccess) s = cuda_fail(e, "ell_field");
  }
  cudaFreeAsync(Q, st);
  return s;
}

ibem_status ibem_e3d_run_host_ell(ibem_solver_form form, const ibem_material* mat, int num, const double* centers,
                                  const double* axes, const double* quats, int nump, const double* points,
                                  const double* sig_inf, double tol, double* X, double* stress,
                                  ibem_solve_report* report) {
  if (!mat || !sig_inf || num <= 0 || nump < 0 || !centers || !axes || !quats || !X || (nump && (!points || !stress)))
    return fail(IBEM_ERR_ARG, "run_host_ell: bad arguments");
  if (form != IBEM_SOLVE_FP64 && form != IBEM_SOLVE_MIXED_IR) return fail(IBEM_ERR_ARG, "run_host_ell: unknown form");
  const int64_t N = 24 * (int64_t)num;
  cudaStream_t st = nullptr;
  IBEM_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  double *A = nullptr, *g = nullptr;
  const size_t geo = (size_t)num * 10 + (size_t)nump * 9 + 2 * (size_t)N;
  ibem_status s = IBEM_OK;
  cudaError_t e = cudaMalloc((void**)&A, sizeof(double) * (size_t)N * (size_t)N);
  if (e == cudaSuccess) e = cudaMalloc((void**)&g, sizeof(double) * geo);
  if (e != cudaSuccess) s = cuda_fail(e, "run_host_ell: device memory");
  double *c = g, *a = g + 3 * (size_t)num, *q = g + 6 * (size_t)num, *p = g + 10 * (size_t)num;
  double *S = p + 3 * (size_t)nump, *b = S + 6 * (size_t)nump, *x = b + N;
  ibem_solve_report rep{};
  if (!s) {
    e = cudaMemcpyAsync(c, centers, sizeof(double) * 3 * num, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(a, axes, sizeof(double) * 3 * num, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(q, quats, sizeof(double) * 4 * num, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nump)
      e = cudaMemcpyAsync(p, points, sizeof(double) * 3 * nump, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) s = cuda_fail(e, "run_host_ell: upload");
  }
  if (!s) s = ibem_e3d_ell_pair_blocks(c, a, q, num, mat, A, N, 0, 0, st);
  if (!s) s = ibem_e3d_farfield_rhs(num, mat, 24, sig_inf, b, st);
  if (!s) s = solve_dense(form, N, A, N, b, x, tol, &rep, st);
  if (!s && nump) s = ibem_e3d_ell_field(form, p, nump, c, a, q, num, mat, x, sig_inf, S, st);
  if (!s) {
    e = cudaMemcpyAsync(X, x, sizeof(double) * N, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && nump) e = cudaMemcpyAsync(stress, S, sizeof(double) * 6 * nump, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = cuda_fail(e, "run_host_ell: download");
  }
  if (report) *report = rep;
  cudaFree(A);
  cudaFree(g);
  cudaStreamDestroy(st);
  return s;
}

}  // extern "C"
