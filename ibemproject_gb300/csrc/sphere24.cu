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

}  // namespace ibem
