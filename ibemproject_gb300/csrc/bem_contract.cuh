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
#ifdef __CUDA_ARCH__
  const double ir = rsqrt(r2);
#else
  const double ir = 1.0 / sqrt(r2);
#endif
  const double ir2 = ir * ir;   // no separate FP64 division
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

// ---------------------------------------------------------------------------------------
// The same contraction in double-float arithmetic (dfloat.cuh: ~48 bits on the FP32 pipe,
// which GB300 runs at 64x its FP64 rate), for the mixed form's stresses.  Everything that
// depends on the Gauss point only is converted once per call into a BemPostDF record,
// including n.u and n_k u_l + n_l u_k times their material coefficients; per (point, Gauss
// point) pair the kernel forms x, the powers of 1/R and four dot products, and adds the six
// components, weighted by the quadrature weight, to compensated sums (dacc).
#include "dfloat.cuh"

namespace ibem {

struct BemPostDF {
  dfloat y[3], n[3], u[3], t[3];
  dfloat w;        // quadrature weight x Jacobian
  dfloat nu0, nu1; // cu0 (n.u), cu1 (n.u)
  dfloat nuk[6];   // cu4 (n_k u_l + n_l u_k), pairs xx xy xz yy yz zz
  dfloat pad;      // 176 bytes: 11 float4
};

struct BemPostCoefDF {
  dfloat cu1, cu3, cu5, ct0, ct1, ct2;
};

IBEM_HD inline BemPostCoefDF bem_post_coef_df(const BemPostCoef& c) {
  return {df_make(c.cu1), df_make(c.cu3), df_make(c.cu5), df_make(c.ct0), df_make(c.ct1), df_make(c.ct2)};
}

// r: y, n, w, u, t of one Gauss point (the FP64 quadrature-table record layout: y 0-2, n 3-5,
// w 6, u 7-9, t 10-12)
IBEM_HD inline BemPostDF bem_post_df_record(const double* r, const BemPostCoef& c) {
  BemPostDF o;
  for (int k = 0; k < 3; ++k) {
    o.y[k] = df_make(r[k]);
    o.n[k] = df_make(r[3 + k]);
    o.u[k] = df_make(r[7 + k]);
    o.t[k] = df_make(r[10 + k]);
  }
  o.w = df_make(r[6]);
  const double nu = r[3] * r[7] + r[4] * r[8] + r[5] * r[9];
  o.nu0 = df_make(c.cu0 * nu);
  o.nu1 = df_make(c.cu1 * nu);
  const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
  for (int q = 0; q < 6; ++q)
    o.nuk[q] = df_make(c.cu4 * (r[3 + pi[q]] * r[7 + pj[q]] + r[3 + pj[q]] * r[7 + pi[q]]));
  o.pad = dfloat{0.0f, 0.0f};
  return o;
}

// acc[6] += w sigma (compensated sums) for the sample point p (double-float)
IBEM_HD IBEM_INLINE void bem_post_contracted_df(const dfloat* p, const BemPostDF& g, const BemPostCoefDF& c,
                                                dacc* acc) {
  dfloat x[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) x[k] = g.y[k] - p[k];
  const dfloat r2 = dot3(x, x);
  // 1 / R: FP32 estimate, one double-float Newton step
  float y0;
#ifdef __CUDA_ARCH__
  y0 = rsqrtf(r2.hi);
#else
  y0 = 1.0f / std::sqrt(r2.hi);
#endif
  const dfloat yd{y0, 0.0f};
  const dfloat ir = yd + yd * ((dfloat{1.0f, 0.0f} - r2 * (yd * yd)) * 0.5f);
  const dfloat ir2 = ir * ir;
  const dfloat W3 = g.w * (ir * ir2), W5 = W3 * ir2, W7 = W5 * ir2;
  const dfloat xn = dot3(x, g.n), xu = dot3(x, g.u), xt = dot3(x, g.t);
  const dfloat xnxu = xn * xu;
  dacc aa = dacc_of(g.nu0);
  dacc_fma(aa, c.ct0, xt);
  dacc ab = dacc_of(g.nu1);
  dacc_fma(ab, c.ct1, xt);
  dacc a = dacc_prod(W3, dacc_val(aa));
  dacc_fma(a, W5 * c.cu1, xnxu);
  dacc b = dacc_prod(W5, dacc_val(ab));
  dacc_fma(b, W7 * c.cu3, xnxu);
  const dfloat av = dacc_val(a), bv = dacc_val(b);
  const dfloat d = (W5 * c.cu5) * xu, e = (W5 * c.cu5) * xn, f = W3 * c.ct2;
  dfloat w[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    dacc s = dacc_prod(d, g.n[k]);
    dacc_fma(s, e, g.u[k]);
    dacc_fma(s, f, g.t[k]);
    w[k] = dacc_val(s);
  }
  const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const int k = pi[q], l = pj[q];
    dacc& o = acc[q];
    dacc_fma(o, bv * x[k], x[l]);
    dacc_fma(o, W3, g.nuk[q]);
    dacc_fma(o, w[k], x[l]);
    dacc_fma(o, w[l], x[k]);
    if (k == l) dacc_add(o, av);
  }
}

}  // namespace ibem
