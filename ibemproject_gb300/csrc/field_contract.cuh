// Strain at a field point from one sphere with a linear Taylor eigenstrain (24 unknowns),
// contracted with the eigenstrain before any tensor is formed.
//
// postProcessorElastic3D.cpp:407-470 forms e_ij = sum_cols D_ijmn(..)·map·E_col with the
// Eshelby-type tensors of integratorElastic3DHelper.cpp:2394-2442 (D_40, D_50).  Writing
// E_mn (order 0) and F_mnp (order 1) as full tensors symmetric in (m, n) absorbs map[m][n],
// and every derivative of the sphere potentials is a radial pattern:
//   d_ij F = F2 x_i x_j + F1 d_ij,   d_ijk F = F3 x_i x_j x_k + F2 (d_ij x_k + 2 more),
//   d_ijkl F = F4 xxxx + F3 (6 d xx) + F2 (3 d d),   Fk = k-th derivative of F in u = |x|^2/2.
// With psi = Psi0, phi = V0, psi_p = a^2 x_p Q, phi_p = a^2 x_p V1 the contraction gives
//   e_ij = c { T(Psi, E)_ij - 2 nu trE phi_,ij - 2 (1-nu) [M_ij + M_ji]
//            + a^2 [ T(Q, E')_ij + 2 (Q3 (v.x) x_i x_j + Q2 (v_i x_j + v_j x_i + d_ij v.x))
//                    + Q3 (s_i x_j + s_j x_i) + Q2 (g_i x_j + g_j x_i + 2 (G^j x)_i + 2 (G^i x)_j) ]
//            - 2 nu a^2 [ (w.x)(V1'' x_i x_j + V1' d_ij) + V1' (w_i x_j + w_j x_i) ]
//            - 2 (1-nu) a^2 [ P_ij + P_ji ] },   c = 1 / (8 pi (1 - nu))
// with T(G, E)_ij = G4 q x_i x_j + G3 (d_ij q + 2 (Ex)_i x_j + 2 x_i (Ex)_j + trE x_i x_j)
//                   + G2 (d_ij trE + 2 E_ij),  q = x.E.x,
//      M_ij = Phi2 (Ex)_i x_j + Phi1 E_ij,  E'_mn = sum_p F_mnp x_p,  v_n = sum_m F_mnm,
//      w_p = sum_m F_mmp,  G^i_mn = F_mni,  s_i = x.G^i.x,  g_i = tr G^i,
//      P_ij = V1'' (E'x)_i x_j + V1' (E'_ij + v_i x_j + (G^j x)_i).
// Collecting like terms, per (point, sphere) pair:
//   e_ij / c = A x_i x_j + B d_ij + W_i x_j + W_j x_i + C0 E_ij + C1 E'_ij + C2 ((G^i x)_j + (G^j x)_i)
// with scalar A, B, C0..C2 and vector W computed once (about 260 FP64 operations per pair).
// Inside the sphere (lambda = 0) the u-derivatives of J vanish, exactly as the reference.
#pragma once
#include "gen_sphere_common.cuh"

IBEM_HD IBEM_INLINE void sph_field24_contracted(const double x0, const double x1, const double x2, const double a,
                                                const SphMat& mc, const double* __restrict__ Eu,
                                                double* __restrict__ e) {
  const double x[3] = {x0, x1, x2};
  const double a2 = a * a;
  const double r2 = x0 * x0 + x1 * x1 + x2 * x2;
  const double lam = r2 - a2;
  const double ext = lam > 0.0 ? 1.0 : 0.0;
  const double rho2 = lam > 0.0 ? a2 + lam : a2;
  // J_m = 4 pi a^3 / ((2m+1) rho^(2m+1)), m = 1..5
#ifdef __CUDA_ARCH__
  const double ir = rsqrt(rho2);
#else
  const double ir = 1.0 / sqrt(rho2);
#endif
  const double irho2 = ir * ir;
  const double j0 = 4.0 * IBEM_PI * a * a2 * ir;
  const double p1 = j0 * irho2, p2 = p1 * irho2, p3 = p2 * irho2, p4 = p3 * irho2, p5 = p4 * irho2;
  const double J1 = p1 * (1.0 / 3.0), J2 = p2 * (1.0 / 5.0), J3 = p3 * (1.0 / 7.0), J4 = p4 * (1.0 / 9.0),
               J5 = p5 * (1.0 / 11.0);
  // u-derivative ladders: V_n^(k) = -J_{n+1}^(k-1), J_m^(k) = (-1)^k (2m+3)..(2m+2k+1) J_{m+k} (outside)
  const double V0_1 = -J1, V0_2 = 5.0 * ext * J2, V0_3 = -35.0 * ext * J3;
  const double V1_1 = -J2, V1_2 = 7.0 * ext * J3, V1_3 = -63.0 * ext * J4;
  const double V2_1 = -J3, V2_2 = 9.0 * ext * J4, V2_3 = -99.0 * ext * J5;
  // 2nd..4th u-derivatives of Psi0 and Q; 1st and 2nd of phi = V0
  const double Ps2 = V0_1 - a2 * V1_1, Ps3 = V0_2 - a2 * V1_2, Ps4 = V0_3 - a2 * V1_3;
  const double Q2 = V1_1 - a2 * V2_1, Q3 = V1_2 - a2 * V2_2, Q4 = V1_3 - a2 * V2_3;
  const double Ph1 = V0_1, Ph2 = V0_2;
  // eigenstrain tensors (symmetric in the first two indices)
  double E[3][3], F[3][3][3];
  {
    const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      E[pi[t]][pj[t]] = E[pj[t]][pi[t]] = Eu[t];
#pragma unroll
      for (int p = 0; p < 3; ++p) F[pi[t]][pj[t]][p] = F[pj[t]][pi[t]][p] = Eu[6 + 3 * t + p];
    }
  }
  double Ex[3], Ep[3][3], Epx[3], v[3], w[3], Gx[3][3], s[3], g[3];  // Gx[i][j] = (G^i x)_j
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
    g[i] = F[0][0][i] + F[1][1][i] + F[2][2][i];
  }
  const double q = Ex[0] * x0 + Ex[1] * x1 + Ex[2] * x2;
  const double tE = E[0][0] + E[1][1] + E[2][2];
  const double qp = Epx[0] * x0 + Epx[1] * x1 + Epx[2] * x2;
  const double tEp = Ep[0][0] + Ep[1][1] + Ep[2][2];
  const double vx = v[0] * x0 + v[1] * x1 + v[2] * x2;
  const double wx = w[0] * x0 + w[1] * x1 + w[2] * x2;
  const double nu2 = mc.tn2, nu1m = mc.tn1;  // 2 nu, 1 - nu
  const double A = Ps4 * q + Ps3 * tE - nu2 * tE * Ph2 + a2 * (Q4 * qp + Q3 * (tEp + 2.0 * vx) - nu2 * wx * V1_2);
  const double B = Ps3 * q + Ps2 * tE - nu2 * tE * Ph1 + a2 * (Q3 * qp + Q2 * (tEp + 2.0 * vx) - nu2 * wx * V1_1);
  const double cE = 2.0 * Ps3 - 2.0 * nu1m * Ph2;
  const double cEp = a2 * (2.0 * Q3 - 2.0 * nu1m * V1_2), cv = a2 * (2.0 * Q2 - 2.0 * nu1m * V1_1);
  const double cs = a2 * Q3, cg = a2 * Q2, cw = -a2 * nu2 * V1_1;
  double W[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) W[i] = cE * Ex[i] + cEp * Epx[i] + cv * v[i] + cs * s[i] + cg * g[i] + cw * w[i];
  const double C0 = 2.0 * Ps2 - 4.0 * nu1m * Ph1;
  const double C1 = a2 * (2.0 * Q2 - 4.0 * nu1m * V1_1);
  const double C2 = a2 * (2.0 * Q2 - 2.0 * nu1m * V1_1);
  const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const int i = pi[t], j = pj[t];
    double r = A * x[i] * x[j] + W[i] * x[j] + W[j] * x[i] + C0 * E[i][j] + C1 * Ep[i][j] + C2 * (Gx[i][j] + Gx[j][i]);
    if (i == j) r += B;
    e[t] += mc.kd * r;
  }
}

// ----------------------------------------------------------------------------------------
// The same contraction in double-float arithmetic (dfloat.cuh), for the mixed-precision
// form.  The strain of an inclusion depends on x / a only: with x' = x / a, a' = 1 and the
// order-1 eigenstrain scaled to F' = a F, every term above is unchanged (E' = F'.x' = F.x,
// and the coefficients of each power of x scale with the matching power of a), so the sums
// run on O(1) quantities that stay well inside the FP32 exponent range for any sphere size.
#include "dfloat.cuh"

namespace ibem {

// per-sphere constants of the double-float sum (scaled coordinates)
struct SphDF {
  dfloat c[3];   // centre
  dfloat ia;     // 1 / a
  dfloat E[6];   // order-0 eigenstrain, storage order of the 24 unknowns
  dfloat F[18];  // a * order-1 eigenstrain, F[3 t + p] for the symmetric pair t and p
  dfloat v[3];   // v_n = sum_m F_mnm
  dfloat w[3];   // w_p = sum_m F_mmp (also the trace vector g of the derivation)
  dfloat tE;     // trace of E
  float pad[2];  // 288 bytes: 18 float4
};

IBEM_HD inline SphDF sph_df_make(const double* cen, double a, const double* Eu) {
  SphDF s;
  const double ia = 1.0 / a;
  for (int i = 0; i < 3; ++i) s.c[i] = df_make(cen[i]);
  s.ia = df_make(ia);
  const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
  double F[3][3][3];
  for (int t = 0; t < 6; ++t) {
    s.E[t] = df_make(Eu[t]);
    for (int p = 0; p < 3; ++p) {
      F[pi[t]][pj[t]][p] = F[pj[t]][pi[t]][p] = a * Eu[6 + 3 * t + p];
      s.F[3 * t + p] = df_make(a * Eu[6 + 3 * t + p]);
    }
  }
  for (int n = 0; n < 3; ++n) {
    s.v[n] = df_make(F[0][n][0] + F[1][n][1] + F[2][n][2]);
    s.w[n] = df_make(F[0][0][n] + F[1][1][n] + F[2][2][n]);
  }
  s.tE = df_make(Eu[0] + Eu[3] + Eu[5]);
  return s;
}

// e[6] += strain / c at the point p (double-float, point already converted), each e[t] a
// compensated sum over the spheres; returns whether the point lies inside or on the sphere.
// The caller multiplies by c = 1 / (8 pi (1 - nu)) once, after the sum.
IBEM_HD IBEM_INLINE bool sph_field24_df(const dfloat* p, const SphDF& sp, dfloat tn1, dfloat tn2, dacc* e) {
  dfloat x[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) x[i] = (p[i] - sp.c[i]) * sp.ia;
  const dfloat r2 = dot3(x, x);
  const bool ext = r2.hi > 1.0f || (r2.hi == 1.0f && r2.lo > 0.0f);
  const float fe = ext ? 1.0f : 0.0f;
  const dfloat rho2 = ext ? r2 : dfloat{1.0f, 0.0f};
  // ir = rho2^-1/2: FP32 estimate, one double-float Newton step
  float y0;
#ifdef __CUDA_ARCH__
  y0 = rsqrtf(rho2.hi);
#else
  y0 = 1.0f / std::sqrt(rho2.hi);
#endif
  const dfloat yd{y0, 0.0f};
  const dfloat t = dfloat{1.0f, 0.0f} - rho2 * (yd * yd);
  const dfloat ir = yd + yd * (t * 0.5f);
  const dfloat irho2 = ir * ir;
  const dfloat four_pi = df_make(4.0 * IBEM_PI);
  const dfloat j0 = four_pi * ir;
  const dfloat p1 = j0 * irho2, p2 = p1 * irho2, p3 = p2 * irho2, p4 = p3 * irho2, p5 = p4 * irho2;
  const dfloat J1 = p1 * df_make(1.0 / 3.0), J2 = p2 * df_make(1.0 / 5.0), J3 = p3 * df_make(1.0 / 7.0),
               J4 = p4 * df_make(1.0 / 9.0), J5 = p5 * df_make(1.0 / 11.0);
  const dfloat V0_1 = -J1, V0_2 = J2 * (5.0f * fe), V0_3 = J3 * (-35.0f * fe);
  const dfloat V1_1 = -J2, V1_2 = J3 * (7.0f * fe), V1_3 = J4 * (-63.0f * fe);
  const dfloat V2_1 = -J3, V2_2 = J4 * (9.0f * fe), V2_3 = J5 * (-99.0f * fe);
  const dfloat Ps2 = V0_1 - V1_1, Ps3 = V0_2 - V1_2, Ps4 = V0_3 - V1_3;
  const dfloat Q2 = V1_1 - V2_1, Q3 = V1_2 - V2_2, Q4 = V1_3 - V2_3;
  const dfloat Ph1 = V0_1, Ph2 = V0_2;
  // E x, E' = F'.x (symmetric), E' x, G^i x, s_i = x.G^i.x
  const int ti[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};  // (m, n) -> symmetric pair
  dfloat Ex[3], Ep[6], Epx[3], Gx[3][3], s[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const dfloat u[3] = {sp.E[ti[i][0]], sp.E[ti[i][1]], sp.E[ti[i][2]]};
    Ex[i] = dot3(u, x);
  }
#pragma unroll
  for (int t2 = 0; t2 < 6; ++t2) Ep[t2] = dot3(sp.F + 3 * t2, x);
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const dfloat u[3] = {Ep[ti[n][0]], Ep[ti[n][1]], Ep[ti[n][2]]};
    Epx[n] = dot3(u, x);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const dfloat u[3] = {sp.F[3 * ti[j][0] + i], sp.F[3 * ti[j][1] + i], sp.F[3 * ti[j][2] + i]};
      Gx[i][j] = dot3(u, x);
    }
    s[i] = dot3(Gx[i], x);
  }
  const dfloat q = dot3(Ex, x), qp = dot3(Epx, x), vx = dot3(sp.v, x), wx = dot3(sp.w, x);
  const dfloat tE = sp.tE;
  dacc ta = dacc_of(Ep[0]);
  dacc_add(ta, Ep[3]);
  dacc_add(ta, Ep[5]);
  dacc_add(ta, vx * 2.0f);
  const dfloat tv = dacc_val(ta);
  const dfloat Ph2t = Ph2 * tn2, Ph1t = Ph1 * tn2, V12t = V1_2 * tn2, V11t = V1_1 * tn2;
  dacc aA = dacc_prod(Ps4, q);
  dacc_fma(aA, Ps3 - Ph2t, tE);
  dacc_fma(aA, Q4, qp);
  dacc_fma(aA, Q3, tv);
  dacc_fma(aA, -V12t, wx);
  const dfloat A = dacc_val(aA);
  dacc aB = dacc_prod(Ps3, q);
  dacc_fma(aB, Ps2 - Ph1t, tE);
  dacc_fma(aB, Q3, qp);
  dacc_fma(aB, Q2, tv);
  dacc_fma(aB, -V11t, wx);
  const dfloat B = dacc_val(aB);
  const dfloat tn1x2 = tn1 * 2.0f, tn1x4 = tn1 * 4.0f;
  dacc c;
  c = dacc_of(Ps3 * 2.0f); dacc_fma(c, -tn1x2, Ph2); const dfloat cE = dacc_val(c);
  c = dacc_of(Q3 * 2.0f); dacc_fma(c, -tn1x2, V1_2); const dfloat cEp = dacc_val(c);
  c = dacc_of(Q2 * 2.0f); dacc_fma(c, -tn1x2, V1_1); const dfloat cv = dacc_val(c);
  const dfloat cs = Q3, cgw = Q2 - V11t;  // g == w: the two terms share a coefficient
  c = dacc_of(Ps2 * 2.0f); dacc_fma(c, -tn1x4, Ph1); const dfloat C0 = dacc_val(c);
  c = dacc_of(Q2 * 2.0f); dacc_fma(c, -tn1x4, V1_1); const dfloat C1 = dacc_val(c);
  const dfloat C2 = cv;   // 2 Q2 - 2 tn1 V1_1
  dfloat W[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    dacc w = dacc_prod(cE, Ex[i]);
    dacc_fma(w, cEp, Epx[i]);
    dacc_fma(w, cv, sp.v[i]);
    dacc_fma(w, cs, s[i]);
    dacc_fma(w, cgw, sp.w[i]);
    W[i] = dacc_val(w);
  }
  dfloat Ax[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) Ax[i] = A * x[i];
  const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int t2 = 0; t2 < 6; ++t2) {
    const int i = pi[t2], j = pj[t2];
    dacc& o = e[t2];
    dacc_fma(o, Ax[i], x[j]);
    if (i == j) {
      dacc_fma(o, W[i] * 2.0f, x[i]);
      dacc_add(o, B);
      dacc_fma(o, C2 * 2.0f, Gx[i][i]);
    } else {
      dacc_fma(o, W[i], x[j]);
      dacc_fma(o, W[j], x[i]);
      dacc_fma(o, C2, Gx[i][j]);
      dacc_fma(o, C2, Gx[j][i]);
    }
    dacc_fma(o, C0, sp.E[t2]);
    dacc_fma(o, C1, Ep[t2]);
  }
  return !ext;
}

// The same contraction in FP32 for far pairs of the mixed form's split sum: a sphere whose
// centre lies beyond kFarRadii of its radius from every point of a warp contributes at most
// (1/kFarRadii)^3 of a near sphere, so its FP32 rounding (a few 1e-7 of the contribution,
// unbiased) stays near 1e-9 of the strain when summed over all far spheres.  The random-sign
// errors add in squares, so the nearest far shell dominates and the summed error grows as
// kFarRadii^-1.5: stresses of the 2,000-sphere, 64^3-point workload from its solution, against
// FP64 sums, 3.2e-9 at 14 radii, 4.2e-9 at 12, 5.5e-9 at 10 (the solution target is 1e-8).
// Coordinates scaled by 1/a as above; the sphere's constants are the high parts of its SphDF.
constexpr float kFarRadii = 12.0f;

IBEM_HD IBEM_INLINE void sph_field24_f32(const dfloat* p, const SphDF& sp, float tn1, float tn2, float* e) {
  float x[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) x[i] = ((p[i].hi - sp.c[i].hi) + (p[i].lo - sp.c[i].lo)) * sp.ia.hi;
  const float r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
  // outside by construction (far pair): rho^2 = |x|^2
  float ir;
#ifdef __CUDA_ARCH__
  ir = rsqrtf(r2);
#else
  ir = 1.0f / std::sqrt(r2);
#endif
  ir = ir * (1.5f - 0.5f * r2 * ir * ir);  // one Newton step
  const float irho2 = ir * ir;
  const float p1 = 4.0f * 3.14159265358979f * ir * irho2, p2 = p1 * irho2, p3 = p2 * irho2, p4 = p3 * irho2,
              p5 = p4 * irho2;
  const float J1 = p1 * (1.0f / 3.0f), J2 = p2 * 0.2f, J3 = p3 * (1.0f / 7.0f), J4 = p4 * (1.0f / 9.0f),
              J5 = p5 * (1.0f / 11.0f);
  const float V0_1 = -J1, V0_2 = 5.0f * J2, V0_3 = -35.0f * J3;
  const float V1_1 = -J2, V1_2 = 7.0f * J3, V1_3 = -63.0f * J4;
  const float V2_1 = -J3, V2_2 = 9.0f * J4, V2_3 = -99.0f * J5;
  const float Ps2 = V0_1 - V1_1, Ps3 = V0_2 - V1_2, Ps4 = V0_3 - V1_3;
  const float Q2 = V1_1 - V2_1, Q3 = V1_2 - V2_2, Q4 = V1_3 - V2_3;
  const float Ph1 = V0_1, Ph2 = V0_2;
  const int ti[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  float Ex[3], Ep[6], Epx[3], Gx[3][3], s[3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    Ex[i] = sp.E[ti[i][0]].hi * x[0] + sp.E[ti[i][1]].hi * x[1] + sp.E[ti[i][2]].hi * x[2];
#pragma unroll
  for (int t = 0; t < 6; ++t) Ep[t] = sp.F[3 * t].hi * x[0] + sp.F[3 * t + 1].hi * x[1] + sp.F[3 * t + 2].hi * x[2];
#pragma unroll
  for (int n = 0; n < 3; ++n) Epx[n] = Ep[ti[n][0]] * x[0] + Ep[ti[n][1]] * x[1] + Ep[ti[n][2]] * x[2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j)
      Gx[i][j] = sp.F[3 * ti[j][0] + i].hi * x[0] + sp.F[3 * ti[j][1] + i].hi * x[1] + sp.F[3 * ti[j][2] + i].hi * x[2];
    s[i] = Gx[i][0] * x[0] + Gx[i][1] * x[1] + Gx[i][2] * x[2];
  }
  const float q = Ex[0] * x[0] + Ex[1] * x[1] + Ex[2] * x[2];
  const float qp = Epx[0] * x[0] + Epx[1] * x[1] + Epx[2] * x[2];
  const float tEp = Ep[0] + Ep[3] + Ep[5];
  const float vx = sp.v[0].hi * x[0] + sp.v[1].hi * x[1] + sp.v[2].hi * x[2];
  const float wx = sp.w[0].hi * x[0] + sp.w[1].hi * x[1] + sp.w[2].hi * x[2];
  const float tE = sp.tE.hi;
  const float tv = tEp + 2.0f * vx;
  const float A = Ps4 * q + Ps3 * tE - tE * Ph2 * tn2 + (Q4 * qp + Q3 * tv - wx * V1_2 * tn2);
  const float B = Ps3 * q + Ps2 * tE - tE * Ph1 * tn2 + (Q3 * qp + Q2 * tv - wx * V1_1 * tn2);
  const float cE = 2.0f * Ps3 - 2.0f * tn1 * Ph2;
  const float cEp = 2.0f * Q3 - 2.0f * tn1 * V1_2, cv = 2.0f * Q2 - 2.0f * tn1 * V1_1;
  const float cs = Q3, cgw = Q2 - tn2 * V1_1;
  float W[3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    W[i] = cE * Ex[i] + cEp * Epx[i] + cv * sp.v[i].hi + cs * s[i] + cgw * sp.w[i].hi;
  const float C0 = 2.0f * Ps2 - 4.0f * tn1 * Ph1;
  const float C1 = 2.0f * Q2 - 4.0f * tn1 * V1_1;
  const float C2 = 2.0f * Q2 - 2.0f * tn1 * V1_1;
  const int pi[6] = {0, 0, 0, 1, 1, 2}, pj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const int i = pi[t], j = pj[t];
    float r = A * x[i] * x[j] + W[i] * x[j] + W[j] * x[i] + C0 * sp.E[t].hi + C1 * Ep[t] + C2 * (Gx[i][j] + Gx[j][i]);
    if (i == j) r += B;
    e[t] = r;
  }
}

// a += b (double-float plus FP32, error-free sum of the high parts)
IBEM_HD IBEM_INLINE void df_add_f(dfloat& a, float b) {
  const dfloat s = df_two_sum(a.hi, b);
  a = df_fast_two_sum(s.hi, s.lo + a.lo);
}

}  // namespace ibem
