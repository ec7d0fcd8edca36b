// Product of one 24 x 24 sphere pair block with a coefficient vector, without forming the
// block (the matrix-free solver's inner loop).
//
// Rows of order 0 of the pair block (integratorElastic3D.cpp:341-454) are, for every source
// column, map[m][n] (kmu D_ij + klam d_ij Tr D) with D the Eshelby-type tensor without its
// 1 / (8 pi (1 - nu)) factor (integratorElastic3DHelper.cpp:2394-2442); rows of order 1
// (:455-567) are the same with one more derivative in the target position x_r (D_41, D_51).
// Summed against the source's coefficients x_h, the order-0 rows are therefore
//   y_ij = kmu r_ij + klam d_ij (r_00 + r_11 + r_22),   r = e / c,
// with e the strain that the source's eigenstrain x_h produces at the target centre (the
// post-processor's sum, postProcessorElastic3D.cpp:407-470, contracted with the eigenstrain
// before any tensor is formed: field_contract.cuh), and the order-1 rows are the same
// combination of the gradient d r_ij / d x_r.  Both come from one evaluation of the
// contracted strain in dual numbers carrying the three partial derivatives in x: about
// 1,000 operations per pair instead of the ~6,000 of the generated block and its 576
// multiply-adds.
#pragma once
#include "gen_sphere_common.cuh"

namespace ibem {

// value and gradient in x (forward-mode dual number)
template <class R>
struct D3 {
  R v, g0, g1, g2;
};
template <class R>
__device__ __forceinline__ D3<R> operator+(const D3<R>& a, const D3<R>& b) {
  return {a.v + b.v, a.g0 + b.g0, a.g1 + b.g1, a.g2 + b.g2};
}
template <class R>
__device__ __forceinline__ D3<R> operator-(const D3<R>& a, const D3<R>& b) {
  return {a.v - b.v, a.g0 - b.g0, a.g1 - b.g1, a.g2 - b.g2};
}
template <class R>
__device__ __forceinline__ D3<R> operator*(const D3<R>& a, const D3<R>& b) {
  return {a.v * b.v, a.v * b.g0 + a.g0 * b.v, a.v * b.g1 + a.g1 * b.v, a.v * b.g2 + a.g2 * b.v};
}
template <class R>
__device__ __forceinline__ D3<R> operator*(R s, const D3<R>& a) {
  return {s * a.v, s * a.g0, s * a.g1, s * a.g2};
}
template <class R>
__device__ __forceinline__ D3<R> operator+(const D3<R>& a, R s) {
  return {a.v + s, a.g0, a.g1, a.g2};
}
template <class R>
__device__ __forceinline__ D3<R> cst(R s) {
  return {s, R(0), R(0), R(0)};
}
__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrt_t(double x) { return rsqrt(x); }

// y[24] += the pair block (target at offset x from a source of radius a) times xs[24],
// kmu, klam, tn1 = 1 - nu0, tn2 = 2 nu0 as in SphMat; row_scale multiplies the order-1 rows.
template <class R>
__device__ __forceinline__ void sph_pair_apply24(R x0, R x1, R x2, R a, R kmu, R klam, R tn1, R tn2,
                                                 const R* __restrict__ Eu, R row_scale, R (&y)[24]) {
  using T = D3<R>;
  const T x[3] = {{x0, R(1), R(0), R(0)}, {x1, R(0), R(1), R(0)}, {x2, R(0), R(0), R(1)}};
  const R a2 = a * a;
  const T r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
  const bool outside = r2.v - a2 > R(0);
  const R ext = outside ? R(1) : R(0);
  // rho^2 = a^2 + lambda = |x|^2 outside, a^2 inside (lambda = 0, integratorElastic3DHelper.cpp:51-54)
  const T rho2 = outside ? r2 : cst(a2);
  const R irv = rsqrt_t(rho2.v);
  const R dir = R(-0.5) * irv * irv * irv;
  const T ir = {irv, dir * rho2.g0, dir * rho2.g1, dir * rho2.g2};
  const T irho2 = ir * ir;
  const T j0 = (R(4.0 * IBEM_PI) * a * a2) * ir;
  const T p1 = j0 * irho2, p2 = p1 * irho2, p3 = p2 * irho2, p4 = p3 * irho2, p5 = p4 * irho2;
  const T J1 = R(1.0 / 3.0) * p1, J2 = R(1.0 / 5.0) * p2, J3 = R(1.0 / 7.0) * p3, J4 = R(1.0 / 9.0) * p4,
          J5 = R(1.0 / 11.0) * p5;
  const T V0_1 = R(-1) * J1, V0_2 = (R(5) * ext) * J2, V0_3 = (R(-35) * ext) * J3;
  const T V1_1 = R(-1) * J2, V1_2 = (R(7) * ext) * J3, V1_3 = (R(-63) * ext) * J4;
  const T V2_1 = R(-1) * J3, V2_2 = (R(9) * ext) * J4, V2_3 = (R(-99) * ext) * J5;
  const T Ps2 = V0_1 - a2 * V1_1, Ps3 = V0_2 - a2 * V1_2, Ps4 = V0_3 - a2 * V1_3;
  const T Q2 = V1_1 - a2 * V2_1, Q3 = V1_2 - a2 * V2_2, Q4 = V1_3 - a2 * V2_3;
  const T Ph1 = V0_1, Ph2 = V0_2;
  // coefficients as full tensors symmetric in the first two indices (absorbs map[m][n])
  R E[3][3], F[3][3][3];
  {
    const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      E[pi[t]][pj[t]] = E[pj[t]][pi[t]] = Eu[t];
#pragma unroll
      for (int p = 0; p < 3; ++p) F[pi[t]][pj[t]][p] = F[pj[t]][pi[t]][p] = Eu[6 + 3 * t + p];
    }
  }
  T Ex[3], Ep[3][3], Epx[3], Gx[3][3], s[3];
  R v[3], w[3], g[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) Ex[i] = E[i][0] * x[0] + E[i][1] * x[1] + E[i][2] * x[2];
#pragma unroll
  for (int m = 0; m < 3; ++m)
#pragma unroll
    for (int n = m; n < 3; ++n) Ep[m][n] = Ep[n][m] = F[m][n][0] * x[0] + F[m][n][1] * x[1] + F[m][n][2] * x[2];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    v[n] = F[0][n][0] + F[1][n][1] + F[2][n][2];
    w[n] = F[0][0][n] + F[1][1][n] + F[2][2][n];
    Epx[n] = Ep[n][0] * x[0] + Ep[n][1] * x[1] + Ep[n][2] * x[2];
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) Gx[i][j] = F[j][0][i] * x[0] + F[j][1][i] * x[1] + F[j][2][i] * x[2];
    s[i] = Gx[i][0] * x[0] + Gx[i][1] * x[1] + Gx[i][2] * x[2];
    g[i] = F[0][0][i] + F[1][1][i] + F[2][2][i];
  }
  const T q = Ex[0] * x[0] + Ex[1] * x[1] + Ex[2] * x[2];
  const R tE = E[0][0] + E[1][1] + E[2][2];
  const T qp = Epx[0] * x[0] + Epx[1] * x[1] + Epx[2] * x[2];
  const T tEp = Ep[0][0] + Ep[1][1] + Ep[2][2];
  const T vx = v[0] * x[0] + v[1] * x[1] + v[2] * x[2];
  const T wx = w[0] * x[0] + w[1] * x[1] + w[2] * x[2];
  const T A = Ps4 * q + tE * Ps3 - (tn2 * tE) * Ph2 + a2 * (Q4 * qp + Q3 * (tEp + R(2) * vx) - tn2 * (wx * V1_2));
  const T B = Ps3 * q + tE * Ps2 - (tn2 * tE) * Ph1 + a2 * (Q3 * qp + Q2 * (tEp + R(2) * vx) - tn2 * (wx * V1_1));
  const T cE = R(2) * Ps3 - (R(2) * tn1) * Ph2;
  const T cEp = a2 * (R(2) * Q3 - (R(2) * tn1) * V1_2), cv = a2 * (R(2) * Q2 - (R(2) * tn1) * V1_1);
  const T cs = a2 * Q3, cg = a2 * Q2, cw = (-a2 * tn2) * V1_1;
  T W[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) W[i] = cE * Ex[i] + cEp * Epx[i] + v[i] * cv + cs * s[i] + g[i] * cg + w[i] * cw;
  const T C0 = R(2) * Ps2 - (R(4) * tn1) * Ph1;
  const T C1 = a2 * (R(2) * Q2 - (R(4) * tn1) * V1_1);
  const T C2 = a2 * (R(2) * Q2 - (R(2) * tn1) * V1_1);
  const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
  T r[6];
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const int i = pi[t], j = pj[t];
    r[t] = A * x[i] * x[j] + W[i] * x[j] + W[j] * x[i] + E[i][j] * C0 + C1 * Ep[i][j] + C2 * (Gx[i][j] + Gx[j][i]);
    if (i == j) r[t] = r[t] + B;
  }
  const T tr = r[0] + r[3] + r[5];
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const bool d = (t == 0 || t == 3 || t == 5);
    const T o = d ? kmu * r[t] + klam * tr : kmu * r[t];
    y[t] += o.v;
    y[6 + 3 * t] += row_scale * o.g0;
    y[6 + 3 * t + 1] += row_scale * o.g1;
    y[6 + 3 * t + 2] += row_scale * o.g2;
  }
}

}  // namespace ibem
