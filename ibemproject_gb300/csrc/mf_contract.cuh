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
// combination of the gradient d r_ij / d x_r.  Every coefficient of the contraction is a
// radial function F(u), u = |x|^2 / 2, times a polynomial in x; its gradient is F'(u) x
// plus F times the polynomial's gradient, and F' is the next rung of the same u-derivative
// ladder (V_n^(k) = -J_{n+1}^(k-1), J_m' = -(2m+3) J_{m+1} outside, 0 inside), so
//   d_k r_ij = Ru_ij x_k + P_ijk,
// Ru the contraction with every radial coefficient replaced by its u-derivative and P the
// polynomial part (written out below).  About 750 operations per pair, against ~6,000 for
// the generated block and its 576 multiply-adds.
#pragma once
#include "gen_sphere_common.cuh"

namespace ibem {

IBEM_HD IBEM_INLINE float rsqrt_t(float x) {
#ifdef __CUDA_ARCH__
  return rsqrtf(x);
#else
  return 1.0f / sqrtf(x);
#endif
}
IBEM_HD IBEM_INLINE double rsqrt_t(double x) {
#ifdef __CUDA_ARCH__
  return rsqrt(x);
#else
  return 1.0 / sqrt(x);
#endif
}

// y[24] += the pair block (target at offset x from a source of radius a) times Eu[24];
// kmu, klam, tn1 = 1 - nu0, tn2 = 2 nu0 as in SphMat; row_scale multiplies the order-1 rows.
// With RAW, y instead accumulates the contraction itself (r_t in y[t], row_scale * d_k r_t in
// y[6 + 3t + k]) and the caller applies the same kmu / klam map once after the sum over
// sources (sph_pair_map24): the map is linear and the same for every source of a target.
template <class R, bool RAW = false>
IBEM_HD IBEM_INLINE void sph_pair_apply24(R x0, R x1, R x2, R a, R kmu, R klam, R tn1, R tn2,
                                          const R* __restrict__ Eu, R row_scale, R (&y)[24]) {
  const R x[3] = {x0, x1, x2};
  const R a2 = a * a;
  const R r2 = x0 * x0 + x1 * x1 + x2 * x2;
  const bool outside = r2 - a2 > R(0);
  const R ext = outside ? R(1) : R(0);
  // rho^2 = a^2 + lambda: |x|^2 outside, a^2 inside (lambda = 0, integratorElastic3DHelper.cpp:51-54)
  const R ir = rsqrt_t(outside ? r2 : a2);
  const R irho2 = ir * ir;
  const R p1 = R(4.0 * IBEM_PI) * a * a2 * ir * irho2;
  const R p2 = p1 * irho2, p3 = p2 * irho2, p4 = p3 * irho2, p5 = p4 * irho2, p6 = p5 * irho2;
  const R J1 = p1 * R(1.0 / 3.0), J2 = p2 * R(1.0 / 5.0), J3 = p3 * R(1.0 / 7.0), J4 = p4 * R(1.0 / 9.0),
          J5 = p5 * R(1.0 / 11.0), J6 = p6 * R(1.0 / 13.0);
  // u-derivative ladders of V_0, V_1, V_2 (first to fourth derivative)
  const R V0_1 = -J1, V0_2 = R(5) * ext * J2, V0_3 = R(-35) * ext * J3, V0_4 = R(315) * ext * J4;
  const R V1_1 = -J2, V1_2 = R(7) * ext * J3, V1_3 = R(-63) * ext * J4, V1_4 = R(693) * ext * J5;
  const R V2_1 = -J3, V2_2 = R(9) * ext * J4, V2_3 = R(-99) * ext * J5, V2_4 = R(1287) * ext * J6;
  const R Ps2 = V0_1 - a2 * V1_1, Ps3 = V0_2 - a2 * V1_2, Ps4 = V0_3 - a2 * V1_3, Ps5 = V0_4 - a2 * V1_4;
  const R Q2 = V1_1 - a2 * V2_1, Q3 = V1_2 - a2 * V2_2, Q4 = V1_3 - a2 * V2_3, Q5 = V1_4 - a2 * V2_4;
  const R Ph1 = V0_1, Ph2 = V0_2, Ph3 = V0_3;
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
  // polynomial quantities: Ex = E x, Ep = F.x, Epx = Ep x, Gx[i][j] = (G^i x)_j = F_jli x_l,
  // s_i = x.G^i.x, v_n = F_mnm, w_n = F_mmn (= g_n = tr G^n)
  R Ex[3], Ep[3][3], Epx[3], Gx[3][3], s[3], v[3], w[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) Ex[i] = E[i][0] * x0 + E[i][1] * x1 + E[i][2] * x2;
#pragma unroll
  for (int m = 0; m < 3; ++m)
#pragma unroll
    for (int n = m; n < 3; ++n) Ep[m][n] = Ep[n][m] = F[m][n][0] * x0 + F[m][n][1] * x1 + F[m][n][2] * x2;
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    v[n] = F[0][n][0] + F[1][n][1] + F[2][n][2];
    w[n] = F[0][0][n] + F[1][1][n] + F[2][2][n];
    Epx[n] = Ep[n][0] * x0 + Ep[n][1] * x1 + Ep[n][2] * x2;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) Gx[i][j] = F[j][0][i] * x0 + F[j][1][i] * x1 + F[j][2][i] * x2;
    s[i] = Gx[i][0] * x0 + Gx[i][1] * x1 + Gx[i][2] * x2;
  }
  const R q = Ex[0] * x0 + Ex[1] * x1 + Ex[2] * x2;
  const R tE = E[0][0] + E[1][1] + E[2][2];
  const R qp = Epx[0] * x0 + Epx[1] * x1 + Epx[2] * x2;
  const R tEp = Ep[0][0] + Ep[1][1] + Ep[2][2];
  const R vx = v[0] * x0 + v[1] * x1 + v[2] * x2;
  const R wx = w[0] * x0 + w[1] * x1 + w[2] * x2;
  const R t2v = tEp + R(2) * vx;
  // scalar coefficients and their u-derivatives (B_u = A)
  const R A = Ps4 * q + Ps3 * tE - tn2 * tE * Ph2 + a2 * (Q4 * qp + Q3 * t2v - tn2 * wx * V1_2);
  const R Au = Ps5 * q + Ps4 * tE - tn2 * tE * Ph3 + a2 * (Q5 * qp + Q4 * t2v - tn2 * wx * V1_3);
  const R B = Ps3 * q + Ps2 * tE - tn2 * tE * Ph1 + a2 * (Q3 * qp + Q2 * t2v - tn2 * wx * V1_1);
  const R cE = R(2) * Ps3 - R(2) * tn1 * Ph2, cEu = R(2) * Ps4 - R(2) * tn1 * Ph3;
  const R cEp = a2 * (R(2) * Q3 - R(2) * tn1 * V1_2), cEpu = a2 * (R(2) * Q4 - R(2) * tn1 * V1_3);
  const R cv = a2 * (R(2) * Q2 - R(2) * tn1 * V1_1), cvu = cEp;
  const R cs = a2 * Q3, csu = a2 * Q4;
  const R cg = a2 * Q2, cgu = cs;
  const R cw = -a2 * tn2 * V1_1, cwu = -a2 * tn2 * V1_2;
  const R C0 = R(2) * Ps2 - R(4) * tn1 * Ph1, C0u = R(2) * Ps3 - R(4) * tn1 * Ph2;
  const R C1 = a2 * (R(2) * Q2 - R(4) * tn1 * V1_1), C1u = a2 * (R(2) * Q3 - R(4) * tn1 * V1_2);
  const R C2 = cv, C2u = cEp;
  R W[3], Wu[3], dA[3], dB[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    W[i] = cE * Ex[i] + cEp * Epx[i] + cv * v[i] + cs * s[i] + (cg + cw) * w[i];
    Wu[i] = cEu * Ex[i] + cEpu * Epx[i] + cvu * v[i] + csu * s[i] + (cgu + cwu) * w[i];
    // polynomial parts of d_k A and d_k B: dq = 2 Ex, dqp = 2 Epx + s, dtEp = w, dvx = v, dwx = w
    const R dqp = R(2) * Epx[i] + s[i], dt2v = w[i] + R(2) * v[i];
    dA[i] = R(2) * Ps4 * Ex[i] + a2 * (Q4 * dqp + Q3 * dt2v - tn2 * V1_2 * w[i]);
    dB[i] = R(2) * Ps3 * Ex[i] + a2 * (Q3 * dqp + Q2 * dt2v - tn2 * V1_1 * w[i]);
  }
  const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
  R r[6], g[6][3];
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const int i = pi[t], j = pj[t];
    const R H = Gx[i][j] + Gx[j][i];
    const R xij = x[i] * x[j];
    r[t] = A * xij + W[i] * x[j] + W[j] * x[i] + C0 * E[i][j] + C1 * Ep[i][j] + C2 * H;
    R Ru = Au * xij + Wu[i] * x[j] + Wu[j] * x[i] + C0u * E[i][j] + C1u * Ep[i][j] + C2u * H;
    if (i == j) {
      r[t] += B;
      Ru += A;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      // d_k W_i = Wu_i x_k + cE E_ik + cEp (Ep_ik + Gx_ki) + 2 cs Gx_ik
      const R dWi = cE * E[i][k] + cEp * (Ep[i][k] + Gx[k][i]) + R(2) * cs * Gx[i][k];
      const R dWj = cE * E[j][k] + cEp * (Ep[j][k] + Gx[k][j]) + R(2) * cs * Gx[j][k];
      R P = dA[k] * xij + dWi * x[j] + dWj * x[i] + C1 * F[i][j][k] + C2 * (F[j][k][i] + F[i][k][j]);
      if (i == j) P += dB[k];
      if (i == k) P += A * x[j] + W[j];
      if (j == k) P += A * x[i] + W[i];
      g[t][k] = Ru * x[k] + P;
    }
  }
  if (RAW) {
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      y[t] += r[t];
#pragma unroll
      for (int k = 0; k < 3; ++k) y[6 + 3 * t + k] += row_scale * g[t][k];
    }
    return;
  }
  const R tr = r[0] + r[3] + r[5];
  const R dtr[3] = {g[0][0] + g[3][0] + g[5][0], g[0][1] + g[3][1] + g[5][1], g[0][2] + g[3][2] + g[5][2]};
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const bool d = (t == 0 || t == 3 || t == 5);
    y[t] += d ? kmu * r[t] + klam * tr : kmu * r[t];
#pragma unroll
    for (int k = 0; k < 3; ++k) y[6 + 3 * t + k] += row_scale * (d ? kmu * g[t][k] + klam * dtr[k] : kmu * g[t][k]);
  }
}

// y = the kmu / klam map of a raw accumulation (sph_pair_apply24<R, true>)
template <class R>
IBEM_HD IBEM_INLINE void sph_pair_map24(const R (&acc)[24], R kmu, R klam, R (&y)[24]) {
  const R tr = acc[0] + acc[3] + acc[5];
  R dtr[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) dtr[k] = acc[6 + k] + acc[6 + 9 + k] + acc[6 + 15 + k];
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const bool d = (t == 0 || t == 3 || t == 5);
    y[t] = d ? kmu * acc[t] + klam * tr : kmu * acc[t];
#pragma unroll
    for (int k = 0; k < 3; ++k) y[6 + 3 * t + k] = d ? kmu * acc[6 + 3 * t + k] + klam * dtr[k] : kmu * acc[6 + 3 * t + k];
  }
}

}  // namespace ibem
