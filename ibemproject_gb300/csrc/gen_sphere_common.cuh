// GENERATED by ibemproject_gb300/codegen.py -- do not edit by hand.
// Material constants and qualifiers shared by the generated sphere code.
#pragma once
#include <math.h>
#ifndef IBEM_HD
#ifdef __CUDACC__
#define IBEM_HD __host__ __device__
#define IBEM_INLINE __forceinline__
#else
#define IBEM_HD
#define IBEM_INLINE inline
#endif
#endif
#ifndef IBEM_PI
#define IBEM_PI 3.141592653589793
#endif

// Material constants folded for the generated code (filled by sph_mat_init).
struct SphMat {
  double kmu, klam;   // -2 dmu c, -dlam c   with c = 1 / (8 pi (1 - nu0))
  double tn1, tn2;    // 1 - nu0, 2 nu0
  double kd;          // c (field sums use D itself)
  double g1, g2;      // 1 / (8 pi mu0), 1 / (16 pi mu0 (1 - nu0))
  double twomu0, lam0, mu0;
  double dlam, dmu;
};

// Kelvin-solution constants of the boundary kernels.
struct BemMat {
  double kA, kB;      // 1 / (4 pi mu0), 1 / (16 pi mu0 (1 - nu0))
  double lam0, mu0;
  double dlam, dmu;   // (C0 - C1) contrast
};

IBEM_HD inline BemMat bem_mat_init(double E0, double nu0, double E1, double nu1) {
  BemMat m;
  const double mu0 = E0 / (2.0 * (1.0 + nu0));
  const double mu1 = E1 / (2.0 * (1.0 + nu1));
  m.lam0 = 2.0 * mu0 * nu0 / (1.0 - 2.0 * nu0);
  m.mu0 = mu0;
  m.kA = 1.0 / (4.0 * IBEM_PI * mu0);
  m.kB = 1.0 / (16.0 * IBEM_PI * mu0 * (1.0 - nu0));
  m.dlam = m.lam0 - 2.0 * mu1 * nu1 / (1.0 - 2.0 * nu1);
  m.dmu = mu0 - mu1;
  return m;
}

IBEM_HD inline SphMat sph_mat_init(double E0, double nu0, double E1, double nu1) {
  SphMat m;
  const double mu0 = E0 / (2.0 * (1.0 + nu0));
  const double mu1 = E1 / (2.0 * (1.0 + nu1));
  const double lam0 = 2.0 * mu0 * nu0 / (1.0 - 2.0 * nu0);
  const double lam1 = 2.0 * mu1 * nu1 / (1.0 - 2.0 * nu1);
  const double c = 1.0 / (8.0 * IBEM_PI * (1.0 - nu0));
  m.dlam = lam0 - lam1;
  m.dmu = mu0 - mu1;
  m.kmu = -2.0 * m.dmu * c;
  m.klam = -m.dlam * c;
  m.tn1 = 1.0 - nu0;
  m.tn2 = 2.0 * nu0;
  m.kd = c;
  m.g1 = 1.0 / (8.0 * IBEM_PI * mu0);
  m.g2 = 1.0 / (16.0 * IBEM_PI * mu0 * (1.0 - nu0));
  m.twomu0 = 2.0 * mu0;
  m.lam0 = lam0;
  m.mu0 = mu0;
  return m;
}
