// Stress of the boundary part of the post-processor (postProcessorElastic3D.cpp:32-114,
// get_for_stress_BEM_post) contracted with the boundary values before any tensor is formed:
// at a Gauss point y with unit normal n, displacement u and traction t, and x = y - p for the
// sample point p,
//   sigma_kl(p) = sum_n Dsu[kl][n] u_n + Dst[kl][n] t_n
// where Dsu, Dst are the Kelvin stress kernels of bem_stress_post (gen_bem.cuh: the
// derivatives of G_ij = A d_ij / R - B R_,ij, A = 1 / (4 pi mu0), B = 1 / (16 pi mu0 (1 - nu0)),
// integratorElastic3DHelper.cpp:2559-2593).  Being isotropic, linear in (n u) and in t, the
// contraction is a combination of seven tensors in x, n, u and three in x, t:
//   sigma = [cu0 (n.u) / R^3 + cu1 (x.n)(x.u) / R^5 + ct0 (x.t) / R^3] d
//         + [cu1 (n.u) / R^5 + cu3 (x.n)(x.u) / R^7 + ct1 (x.t) / R^5] x x
//         + cu4 / R^3 (n u + u n) + cu5 / R^5 [(x.u)(n x + x n) + (x.n)(u x + x u)]
//         + ct2 / R^3 (t x + x t)
// with the material coefficients below (matched exactly, symbolically in A, B, lambda0, mu0,
// against the generated kernels by ibemproject_gb300/bem_contract_derivation.py; the host
// tests compare the two to 1e-13).
// About 115 FP64 operations per (point, Gauss point) against ~700 for forming Dsu and Dst.
#pragma once
#include "gen_sphere_common.cuh"

struct BemPostCoef {
  double cu0, cu1, cu3, cu4, cu5, ct0, ct1, ct2;
};

IBEM_HD inline BemPostCoef bem_post_coef(const BemMat& m) {
  const double A = m.kA, B = m.kB, l = m.lam0, u = m.mu0;
  BemPostCoef c;
  c.cu0 = -4.0 * A * l * u + 8.0 * B * l * u + 4.0 * B * u * u;
  c.cu1 = 6.0 * A * l * u - 12.0 * B * l * u - 12.0 * B * u * u;
  c.cu3 = 60.0 * B * u * u;
  c.cu4 = -2.0 * A * u * u + 4.0 * B * u * u;
  c.cu5 = 3.0 * A * u * u - 12.0 * B * u * u;
  c.ct0 = A * l - 2.0 * B * l - 2.0 * B * u;
  c.ct1 = 6.0 * B * u;
  c.ct2 = A * u - 2.0 * B * u;
  return c;
}

// s[6] (xx xy xz yy yz zz) = sigma at the sample point from one Gauss point
IBEM_HD IBEM_INLINE void bem_post_contracted(double x0, double x1, double x2, double n0, double n1, double n2,
                                             double u0, double u1, double u2, double t0, double t1, double t2,
                                             const BemPostCoef& c, double* s) {
  const double r2 = x0 * x0 + x1 * x1 + x2 * x2;
  const double ir2 = 1.0 / r2;
#ifdef __CUDA_ARCH__
  const double ir = rsqrt(r2);
#else
  const double ir = 1.0 / sqrt(r2);
#endif
  const double ir3 = ir * ir2, ir5 = ir3 * ir2, ir7 = ir5 * ir2;
  const double xn = x0 * n0 + x1 * n1 + x2 * n2, xu = x0 * u0 + x1 * u1 + x2 * u2;
  const double nu = n0 * u0 + n1 * u1 + n2 * u2, xt = x0 * t0 + x1 * t1 + x2 * t2;
  const double xnxu = xn * xu;
  const double a = (c.cu0 * nu + c.ct0 * xt) * ir3 + c.cu1 * xnxu * ir5;
  const double b = (c.cu1 * nu + c.ct1 * xt) * ir5 + c.cu3 * xnxu * ir7;
  const double cc = c.cu4 * ir3, d = c.cu5 * xu * ir5, e = c.cu5 * xn * ir5, f = c.ct2 * ir3;
  const double x[3] = {x0, x1, x2}, n[3] = {n0, n1, n2}, u[3] = {u0, u1, u2}, t[3] = {t0, t1, t2};
  // w_k = d n_k + e u_k + f t_k multiplies x_l (and symmetrically)
  double w[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) w[k] = d * n[k] + e * u[k] + f * t[k];
  const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const int k = pi[q], l = pj[q];
    double v = b * x[k] * x[l] + cc * (n[k] * u[l] + n[l] * u[k]) + w[k] * x[l] + w[l] * x[k];
    if (k == l) v += a;
    s[q] = v;
  }
}
