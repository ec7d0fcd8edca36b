// Sphere kernels for the 24-unknown layout (eigenstrain orders 0 and 1).
#include "field_contract.cuh"
#include "gen_sphere24.cuh"
#include "prof.h"
#include "sphere_kernels.cuh"

IBEM_PAIR_KERNEL(pair24_c0_r0, sph_block24_c0_r0, 24)
IBEM_PAIR_KERNEL(pair24_c0_r1, sph_block24_c0_r1, 24)
IBEM_PAIR_KERNEL(pair24_c1_r0, sph_block24_c1_r0, 24)
IBEM_PAIR_KERNEL(pair24_c1_r1, sph_block24_c1_r1, 24)
IBEM_SELF_KERNEL(self24, sph_self24, 24)
IBEM_NODE_KERNEL(node24, sph_node24, 24)
IBEM_FIELD_KERNEL(field24, sph_field24_contracted, 24)

// Field sum of the mixed form: the same contraction in double-float arithmetic
// (field_contract.cuh).  The loading threads turn each chunk of spheres into SphDF
// constants (scaled coordinates); every thread keeps its point and its six strain sums in
// double-float, and the inside test, the local eigenstrain and C0 run in FP64 at the end.
__global__ void __launch_bounds__(ibem::kFieldThreads)
    field24_df(const double* __restrict__ pts, int nump, const double* __restrict__ cen,
               const double* __restrict__ rad, int num, SphMat mc, const double* __restrict__ E,
               double* __restrict__ stress) {
  __shared__ ibem::SphDF ss[ibem::kFieldChunk];
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = s < nump;
  double p0 = 0, p1 = 0, p2 = 0;
  if (act) { p0 = pts[3 * s]; p1 = pts[3 * s + 1]; p2 = pts[3 * s + 2]; }
  const ibem::dfloat pd[3] = {ibem::df_make(p0), ibem::df_make(p1), ibem::df_make(p2)};
  const ibem::dfloat tn1 = ibem::df_make(mc.tn1), tn2 = ibem::df_make(mc.tn2);
  ibem::dfloat acc[6] = {};
  int inside = -1;
  for (int h0 = 0; h0 < num; h0 += ibem::kFieldChunk) {
    const int nh = min(ibem::kFieldChunk, num - h0);
    __syncthreads();
    for (int i = threadIdx.x; i < nh; i += blockDim.x)
      ss[i] = ibem::sph_df_make(cen + 3 * (int64_t)(h0 + i), rad[h0 + i], E + 24 * (int64_t)(h0 + i));
    __syncthreads();
    if (act)
      for (int hh = 0; hh < nh; ++hh)
        if (ibem::sph_field24_df(pd, ss[hh], tn1, tn2, acc)) inside = h0 + hh;
  }
  if (!act) return;
  double e[6];
  for (int r = 0; r < 6; ++r) e[r] = mc.kd * ibem::df_double(acc[r]);
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
  SphMat mc = sph_mat_init(p.E0, p.nu0, p.E1, p.nu1);
  ProfScope ps(PROF_FIELD, st);
  ::ibem::count_launch(), field24_df<<<(nump + kFieldThreads - 1) / kFieldThreads, kFieldThreads, 0, st>>>(
      pts, nump, p.cen, p.rad, p.num, mc, E, stress);
  IBEM_LAUNCH_CHECK("field24_df");
  return IBEM_OK;
}

}  // namespace ibem
