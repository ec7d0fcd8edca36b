// Host build of the ellipsoid evaluator (ibemproject_gb300/csrc/ellipsoid.cuh), for
// checking it against the oracle and against closed forms without a GPU (compiled by
// tests/test_ellipsoid_host.py with the host compiler).
#include <string.h>

#include "ellipsoid.cuh"

using namespace ibem::ell;

extern "C" int he_block24(const double* d, const double* quat, const double* a, double E0, double nu0,
                          double E1, double nu1, int self, double* out) {
  double Q[9];
  quat_to_rot(quat, Q);
  SphMat mc = sph_mat_init(E0, nu0, E1, nu1);
  ell_block24<double>(d, Q, a, mc, self != 0, out);
  return 0;
}

extern "C" int he_strain24(const double* d, const double* quat, const double* a, double E0, double nu0,
                           double E1, double nu1, const double* E, double* e) {
  double Q[9];
  quat_to_rot(quat, Q);
  SphMat mc = sph_mat_init(E0, nu0, E1, nu1);
  return ell_strain24<double>(d, Q, a, mc, E, e) ? 1 : 0;
}

extern "C" int he_block24_f32(const double* d, const double* quat, const double* a, double E0, double nu0,
                              double E1, double nu1, int self, double* out) {
  float Q[9], qf[4], df[3], af[3], o[576];
  for (int i = 0; i < 4; ++i) qf[i] = (float)quat[i];
  for (int i = 0; i < 3; ++i) { df[i] = (float)d[i]; af[i] = (float)a[i]; }
  quat_to_rot(qf, Q);
  SphMat mc = sph_mat_init(E0, nu0, E1, nu1);
  ell_block24<float>(df, Q, af, mc, self != 0, o);
  for (int i = 0; i < 576; ++i) out[i] = o[i];
  return 0;
}

// I_k(lambda) for |k| <= 3 at x_m = a_m^2 + lambda, in midx order (20 values)
extern "C" void he_ik(const double* x, double* out) { carlson_ik<double>(x, out); }

extern "C" double he_lambda(const double* y, const double* a2) { return ell_lambda<double>(y, a2); }

// potentials and their derivatives at a point: out[0..N) phi_1 jet, then 3 phi_p, 6 phi_pq
// (order-4 jets, N = 35 each)
extern "C" int he_potentials(const double* d, const double* quat, const double* a, double* out) {
  double Q[9];
  quat_to_rot(quat, Q);
  EllPot<double, 4> P;
  ell_potentials<double, 4>(d, Q, a, P);
  const int N = Jet<double, 4>::N;
  memcpy(out, P.f0.c, sizeof(double) * N);
  for (int p = 0; p < 3; ++p) memcpy(out + N * (1 + p), P.f1[p].c, sizeof(double) * N);
  for (int p = 0; p < 6; ++p) memcpy(out + N * (4 + p), P.f2[p].c, sizeof(double) * N);
  return P.inside ? 1 : 0;
}

// D tensor (digit order strain i, j, eigenstrain k, l [, p] [, r]) with the factor
// 1 / (8 pi (1 - nu)), as orc_D / orc_ell_D_quad lay it out
extern "C" int he_D(int order, int nder, const double* d, const double* quat, const double* a, double nu,
                    double* out) {
  double Q[9];
  quat_to_rot(quat, Q);
  EllPot<double, 4> pot;
  ell_potentials<double, 4>(d, Q, a, pot);
  EllDer<double, 4> P;
  ell_derivs(pot, P);
  const int total = 4 + order + nder;
  int lim = 1;
  for (int t = 0; t < total; ++t) lim *= 3;
  const double kd = 1.0 / (8 * IBEM_PI * (1 - nu));
  for (int f = 0; f < lim; ++f) {
    int dig[8], g = f;
    for (int t = total - 1; t >= 0; --t) { dig[t] = g % 3; g /= 3; }
    const int rho = order ? dig[4] : -1;
    out[f] = kd * Dsum(P, nu, rho, dig[0], dig[1], dig[2], dig[3], dig + 4 + order, nder);
  }
  return lim;
}

extern "C" void he_rot(const double* quat, double* Q) { quat_to_rot(quat, Q); }
