// Sphere kernels for the 60-unknown layout (eigenstrain orders 0, 1 and 2, order 2 stored for p <= q ).
#include "gen_sphere60.cuh"
#include "prof.h"
#include "sphere_kernels.cuh"

#define IBEM_PAIRS_60(C) \
  IBEM_PAIR_KERNEL(pair60_c##C##_r0, sph_block60_c##C##_r0, 60) \
  IBEM_PAIR_KERNEL(pair60_c##C##_r1, sph_block60_c##C##_r1, 60) \
  IBEM_PAIR_KERNEL(pair60_c##C##_r2, sph_block60_c##C##_r2, 60)
IBEM_PAIRS_60(0)
IBEM_PAIRS_60(1)
IBEM_PAIRS_60(2)
IBEM_SELF_KERNEL(self60, sph_self60, 60)
IBEM_NODE_KERNEL(node60, sph_node60, 60)
IBEM_FIELD_KERNEL(field60, sph_field60, 60)

namespace ibem {

ibem_status launch_pair60(const SphLaunch& p, double* A, int64_t lda, int64_t row0, int64_t col0,
                          cudaStream_t st) {
  SphMat mc = sph_mat_init(p.E0, p.nu0, p.E1, p.nu1);
  ProfScope ps(PROF_PAIR, st);
  double* base = A + col0 * lda + row0;
  dim3 grid((p.num + kPairThreads - 1) / kPairThreads, p.num);
  ::ibem::count_launch(), pair60_c0_r0<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), pair60_c0_r1<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), pair60_c0_r2<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), pair60_c1_r0<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), pair60_c1_r1<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), pair60_c1_r2<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), pair60_c2_r0<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), pair60_c2_r1<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), pair60_c2_r2<<<grid, kPairThreads, 0, st>>>(p.cen, p.rad, p.num, mc, base, lda);
  ::ibem::count_launch(), self60<<<(p.num + 127) / 128, 128, 0, st>>>(p.num, mc, base, lda);
  IBEM_LAUNCH_CHECK("pair60");
  return IBEM_OK;
}

ibem_status launch_node60(const SphLaunch& p, const double* nodes, int NN, double* H, int64_t ldh,
                          int64_t row0, int64_t col0, cudaStream_t st) {
  SphMat mc = sph_mat_init(p.E0, p.nu0, p.E1, p.nu1);
  dim3 grid((NN + kPairThreads - 1) / kPairThreads, p.num);
  ::ibem::count_launch(), node60<<<grid, kPairThreads, 0, st>>>(nodes, NN, p.cen, p.rad, mc, H + col0 * ldh + row0, ldh);
  IBEM_LAUNCH_CHECK("node60");
  return IBEM_OK;
}

ibem_status launch_field60(const SphLaunch& p, const double* pts, int nump, const double* E,
                           double* stress, cudaStream_t st) {
  SphMat mc = sph_mat_init(p.E0, p.nu0, p.E1, p.nu1);
  ProfScope ps(PROF_FIELD, st);
  ::ibem::count_launch(), field60<<<(nump + kFieldThreads - 1) / kFieldThreads, kFieldThreads, 0, st>>>(
      pts, nump, p.cen, p.rad, p.num, mc, E, stress);
  IBEM_LAUNCH_CHECK("field60");
  return IBEM_OK;
}

}  // namespace ibem
