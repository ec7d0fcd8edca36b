// Exterior and interior Eshelby fields of an ellipsoidal inclusion with a linear
// (Taylor order 0 + 1) eigenstrain, host and device, in any real type T (double, float).
//
// The reference's spherical integrator (integratorElastic3DHelper.cpp:41-664, 2394-2554)
// writes the disturbance strain of an inclusion as derivatives of two potentials of its
// eigenstrain density rho,
//     phi_rho(x) = int rho(x') / |x - x'| dV',   psi_rho(x) = int rho(x') |x - x'| dV',
//     D_ijkl = [psi_,klij - 2 nu d_kl phi_,ij - (1 - nu)(d_il phi_,kj + d_jl phi_,ki
//               + d_ik phi_,lj + d_jk phi_,li)] / (8 pi (1 - nu))          (:2394-2554)
// with rho = 1 (uniform part) or x'_p (linear part).  The same tensor is evaluated here
// for an ellipsoid sum_m y_m^2 / a_m^2 <= 1 in its principal frame y = Q^T (x - c):
//
//  * psi from phi: psi_rho,k = x_k phi_rho - phi_{rho x'_k}, so only Newtonian potentials
//    of the densities 1, y'_m and y'_m y'_n are needed;
//  * those are Ferrers / Dyson integrals over the confocal parameter s >= lambda,
//        phi_1     = C int U ds / Delta
//        phi_m     = C a_m^2 y_m int U t_m ds / Delta
//        phi_mn    = C [ a_m^2/4 d_mn int U^2 ds/Delta + a_m^2 a_n^2 y_m y_n int U t_m t_n ds/Delta
//                        - a_m^2 a_n^2/4 d_mn int U^2 t_n ds/Delta ]
//    with C = pi a1 a2 a3, t_m = 1 / (a_m^2 + s), U = 1 - sum y_m^2 t_m,
//    Delta = sqrt(prod (a_m^2 + s)); lambda = 0 inside, else the largest root of the cubic
//    sum y_m^2 / (a_m^2 + lambda) = 1 (obtained from x'_m rho_n = -a_m^2/(2(n+1)) d'_m of
//    (1 - |y'|_a^2)^(n+1) and integration by parts);
//  * expanding U, every potential is a polynomial in y times the integrals
//        I_k(lambda) = int_lambda^inf prod_m t_m^(k_m) ds / Delta,   |k| <= 3;
//  * I_k are third-order parameter derivatives of Carlson's R_F (I_0 = 2 R_F(a^2 + lambda)),
//    evaluated by Carlson's duplication algorithm (B. C. Carlson, "Numerical computation
//    of real or complex elliptic integrals", Numer. Algorithms 10, 1995) run in truncated
//    Taylor arithmetic in the three arguments -- exact in the sphere and spheroid limits,
//    where partial-fraction recurrences between the I_k break down;
//  * derivatives in x come from truncated multivariate Taylor series ("jets") in the
//    global displacement h of the target point: lambda(x + h) by Newton iteration on jets,
//    I_k(lambda0 + delta) from the closed-form lambda-derivatives dI_k/dlambda = -prod
//    x_m^-(k_m + 1/2), then products with the polynomial factors.
// For a1 = a2 = a3 everything reduces to the sphere formulas of the reference.
#pragma once
#include <math.h>

#include "gen_sphere_common.cuh"

namespace ibem {
namespace ell {

// ------------------------------------------------------------------ number types
// The evaluator runs in double or float.  Scalar functions and the unit roundoff by type:
IBEM_HD inline double vsqrt(double x) { return sqrt(x); }
IBEM_HD inline float vsqrt(float x) { return sqrtf(x); }
IBEM_HD inline double vfabs(double x) { return fabs(x); }
IBEM_HD inline float vfabs(float x) { return fabsf(x); }
template <typename T>
IBEM_HD inline T vfmax(T a, T b) { return a > b ? a : b; }
template <typename T>
struct NumTraits;
template <>
struct NumTraits<double> {
  static constexpr double eps = 1.1102230246251565e-16;
  static constexpr double carlson_q = 379.82022430228585;   // (3 eps)^(-1/6)
};
template <>
struct NumTraits<float> {
  static constexpr double eps = 5.9604645e-08;
  static constexpr double carlson_q = 13.322930834122156;
};

// ------------------------------------------------------------------ jets
// Monomials h1^a h2^b h3^c of total degree d <= K in graded order; inside one degree a
// descending, then b descending.
IBEM_HD constexpr int nmono(int K) { return (K + 1) * (K + 2) * (K + 3) / 6; }
IBEM_HD constexpr int midx(int a, int b, int c) {
  return (a + b + c) * (a + b + c + 1) * (a + b + c + 2) / 6 + (b + c) * (b + c + 1) / 2 + c;
}

template <typename T, int K>
struct Jet {
  static constexpr int N = nmono(K);
  T c[N];
};

template <typename T, int K>
IBEM_HD IBEM_INLINE void jzero(Jet<T, K>& o) {
#pragma unroll
  for (int i = 0; i < Jet<T, K>::N; ++i) o.c[i] = T(0);
}

// Product tables: the (alpha, beta) decompositions of every output monomial gamma,
// grouped by gamma; `last` marks the final term of a group.  AMAX bounds the degree of alpha:
// K for general products, 2 when the left operand is a quadratic polynomial (the squared
// offsets l_m^2, whose coefficients of degree 3 and more are zero; 155 instead of 210 terms
// at order 4).  Built at compile time (the unrolled products below index their operands with
// its entries as constants).
template <int K, int AMAX>
IBEM_HD constexpr int multab_count() {
  int n = 0;
  for (int d = 0; d <= K; ++d)
    for (int g1 = d; g1 >= 0; --g1)
      for (int g2 = d - g1; g2 >= 0; --g2)
        for (int a1 = 0; a1 <= g1; ++a1)
          for (int a2 = 0; a2 <= g2; ++a2)
            for (int a3 = 0; a3 <= d - g1 - g2; ++a3)
              if (a1 + a2 + a3 <= AMAX) ++n;
  return n;
}

template <int K, int AMAX = K>
struct MulTab {
  static constexpr int NT = multab_count<K, AMAX>();
  unsigned char a[NT], b[NT], g[NT], last[NT];
};

template <int K, int AMAX = K>
IBEM_HD constexpr MulTab<K, AMAX> make_multab() {
  MulTab<K, AMAX> t{};
  int n = 0;
  for (int d = 0; d <= K; ++d)
    for (int g1 = d; g1 >= 0; --g1)
      for (int g2 = d - g1; g2 >= 0; --g2) {
        const int g3 = d - g1 - g2;
        for (int a1 = 0; a1 <= g1; ++a1)
          for (int a2 = 0; a2 <= g2; ++a2)
            for (int a3 = 0; a3 <= g3; ++a3) {
              if (a1 + a2 + a3 > AMAX) continue;
              t.a[n] = (unsigned char)midx(a1, a2, a3);
              t.b[n] = (unsigned char)midx(g1 - a1, g2 - a2, g3 - a3);
              t.g[n] = (unsigned char)midx(g1, g2, g3);
              t.last[n] = 0;
              ++n;
            }
        t.last[n - 1] = 1;
      }
  return t;
}

// Shift tables: for every monomial gamma (midx order) the index of gamma - e_i (255: none).
template <int K>
struct ShiftTab {
  unsigned char s[nmono(K)][3];
};

template <int K>
constexpr ShiftTab<K> make_shifttab() {
  ShiftTab<K> t{};
  for (int d = 0; d <= K; ++d)
    for (int g1 = d; g1 >= 0; --g1)
      for (int g2 = d - g1; g2 >= 0; --g2) {
        const int g3 = d - g1 - g2, id = midx(g1, g2, g3);
        t.s[id][0] = (unsigned char)(g1 > 0 ? midx(g1 - 1, g2, g3) : 255);
        t.s[id][1] = (unsigned char)(g2 > 0 ? midx(g1, g2 - 1, g3) : 255);
        t.s[id][2] = (unsigned char)(g3 > 0 ? midx(g1, g2, g3 - 1) : 255);
      }
  return t;
}

constexpr ShiftTab<3> kShiftTab3 = make_shifttab<3>();
constexpr ShiftTab<4> kShiftTab4 = make_shifttab<4>();
#ifdef __CUDACC__
static __constant__ ShiftTab<3> kShiftTab3Dev = make_shifttab<3>();
static __constant__ ShiftTab<4> kShiftTab4Dev = make_shifttab<4>();
#endif

template <int K>
IBEM_HD IBEM_INLINE const ShiftTab<K>& shifttab() {
#ifdef __CUDA_ARCH__
  if constexpr (K == 3) return kShiftTab3Dev; else return kShiftTab4Dev;
#else
  if constexpr (K == 3) return kShiftTab3; else return kShiftTab4;
#endif
}

// o = w_old * o + w * a * b  (o must not alias a or b).  One out-of-line copy per type and
// order, fully unrolled over the product table (a compile-time constant): both operands are
// read once into registers and every term indexes them with constant indices, instead of
// two loads per term from the caller's local memory.
#ifdef __CUDACC__
#define IBEM_NOINLINE __noinline__
#else
#define IBEM_NOINLINE __attribute__((noinline))
#endif
template <typename T, int K, int AMAX = K>
IBEM_HD IBEM_NOINLINE void jmul_acc_ptr(T keep, T w, const T* __restrict__ a, const T* __restrict__ b,
                                        T* __restrict__ o) {
  static_assert(K == 3 || K == 4, "jets of order 3 or 4");
  constexpr MulTab<K, AMAX> tb = make_multab<K, AMAX>();
  constexpr int N = nmono(K), NA = nmono(AMAX);
  T av[NA], bv[N];
#pragma unroll
  for (int i = 0; i < NA; ++i) av[i] = a[i];
#pragma unroll
  for (int i = 0; i < N; ++i) bv[i] = b[i];
  T acc = T(0);
#pragma unroll
  for (int t = 0; t < MulTab<K, AMAX>::NT; ++t) {
    acc += av[tb.a[t]] * bv[tb.b[t]];
    if (tb.last[t]) {
      o[tb.g[t]] = keep * o[tb.g[t]] + w * acc;
      acc = T(0);
    }
  }
}
template <typename T, int K>
IBEM_HD IBEM_INLINE void jmul_acc(T keep, T w, const Jet<T, K>& a, const Jet<T, K>& b, Jet<T, K>& o) {
  jmul_acc_ptr<T, K>(keep, w, a.c, b.c, o.c);
}

// o = a * b (o must not alias a or b)
template <typename T, int K>
IBEM_HD IBEM_INLINE void jmul(const Jet<T, K>& a, const Jet<T, K>& b, Jet<T, K>& o) {
  jzero(o);
  jmul_acc(T(1), T(1), a, b, o);
}

// o += w * a * b
template <typename T, int K>
IBEM_HD IBEM_INLINE void jfma(T w, const Jet<T, K>& a, const Jet<T, K>& b, Jet<T, K>& o) {
  jmul_acc(T(1), w, a, b, o);
}

// the same with a quadratic left operand (coefficients of degree 3 and more zero)
template <typename T, int K>
IBEM_HD IBEM_INLINE void jfma_q(T w, const Jet<T, K>& a, const Jet<T, K>& b, Jet<T, K>& o) {
  jmul_acc_ptr<T, K, 2>(T(1), w, a.c, b.c, o.c);
}
template <typename T, int K>
IBEM_HD IBEM_INLINE void jmul_q(const Jet<T, K>& a, const Jet<T, K>& b, Jet<T, K>& o) {
  jzero(o);
  jmul_acc_ptr<T, K, 2>(T(1), T(1), a.c, b.c, o.c);
}

// o = (l0 + l1 h1 + l2 h2 + l3 h3) * a   (o must not alias a)
template <typename T, int K>
IBEM_HD inline void jmul_lin(T l0, T l1, T l2, T l3, const Jet<T, K>& a, Jet<T, K>& o) {
  const ShiftTab<K>& sh = shifttab<K>();
#pragma unroll 1
  for (int g = 0; g < Jet<T, K>::N; ++g) {
    T v = l0 * a.c[g];
    if (sh.s[g][0] != 255) v += l1 * a.c[sh.s[g][0]];
    if (sh.s[g][1] != 255) v += l2 * a.c[sh.s[g][1]];
    if (sh.s[g][2] != 255) v += l3 * a.c[sh.s[g][2]];
    o.c[g] = v;
  }
}

// o += w * a
template <typename T, int K>
IBEM_HD IBEM_INLINE void jaxpy(T w, const Jet<T, K>& a, Jet<T, K>& o) {
#pragma unroll
  for (int i = 0; i < Jet<T, K>::N; ++i) o.c[i] += w * a.c[i];
}

// f(a) for a jet a with constant term a0 and f given by its Taylor coefficients at a0:
// o = sum_n f_n (a - a0)^n, f_n = f^(n)(a0)/n!
template <typename T, int K>
IBEM_HD IBEM_INLINE void jcompose(const Jet<T, K>& a, const T* f, Jet<T, K>& o) {
  Jet<T, K> u = a, p, t;
  u.c[0] = T(0);
  jzero(o);
  o.c[0] = f[0];
  p = u;
#pragma unroll
  for (int n = 1; n <= K; ++n) {
    jaxpy(f[n], p, o);
    if (n < K) {
      jmul(p, u, t);
      p = t;
    }
  }
}

// a^q for q in {1/2, -1/2, -1} (a0 > 0): f_0 = a0^q from sqrt / reciprocal, then the
// Taylor coefficients f_n = f_(n-1) (q - n + 1) / (n a0)
template <typename T, int K>
IBEM_HD IBEM_INLINE void jpow(const Jet<T, K>& a, int twice_q, Jet<T, K>& o) {
  T f[K + 1];
  const T a0 = a.c[0], ia = T(1) / a0, q = T(twice_q) / T(2);
  f[0] = twice_q == 1 ? vsqrt(a0) : (twice_q == -1 ? T(1) / vsqrt(a0) : ia);
#pragma unroll
  for (int n = 1; n <= K; ++n) f[n] = f[n - 1] * (q - T(n - 1)) / T(n) * ia;
  jcompose(a, f, o);
}

// ------------------------------------------------------------------ Carlson R_F jets
// I_k(lambda) for all |k| <= 3 at x_m = a_m^2 + lambda: third-order Taylor coefficients of
// 2 R_F(x1, x2, x3) in its arguments (duplication algorithm, Carlson 1995), scaled by
// d/dx_m of int prod (x + tau)^-(k_m + 1/2) = -(k_m + 1/2) I_{k + e_m}:
//     I_k = 2 c_k(R_F) prod_m w(k_m),  w = 1, -2, 8/3, -16/5.
// Output ik[midx(k1, k2, k3)] (20 values).
template <typename T>
IBEM_HD inline void carlson_ik(const T x[3], T* ik) {
  using J = Jet<T, 3>;
  J X[3], A, A0;
#pragma unroll 1
  for (int m = 0; m < 3; ++m) {
    jzero(X[m]);
    X[m].c[0] = x[m];
  }
  X[0].c[midx(1, 0, 0)] = T(1);
  X[1].c[midx(0, 1, 0)] = T(1);
  X[2].c[midx(0, 0, 1)] = T(1);
#pragma unroll 1
  for (int i = 0; i < J::N; ++i) A0.c[i] = (X[0].c[i] + X[1].c[i] + X[2].c[i]) / T(3);
  A = A0;
  // iteration count from the values (Carlson 1995, eq. 2.2-2.4 with r the unit roundoff)
  // (3 r)^(-1/6) max |A0 - x_m|
  const T Qv = T(NumTraits<T>::carlson_q) *
               vfmax(vfabs(A0.c[0] - x[0]), vfmax(vfabs(A0.c[0] - x[1]), vfabs(A0.c[0] - x[2])));
  T pow4 = T(1);
  J s[3], lam, t;
#pragma unroll 1
  // Carlson's criterion bounds the error of the value; the third parameter derivatives are
  // 4^-3 smaller per unit of deviation, so the loop runs until the criterion holds with a
  // margin of 4^3 (three more halvings of the relative spread's square root)
  for (int it = 0; it < 40 && T(64.0) * pow4 * Qv >= vfabs(A.c[0]); ++it) {
#pragma unroll 1
    for (int m = 0; m < 3; ++m) jpow(X[m], 1, s[m]);
    jmul(s[0], s[1], lam);
    jfma(T(1), s[0], s[2], lam);
    jfma(T(1), s[1], s[2], lam);
#pragma unroll 1
    for (int i = 0; i < J::N; ++i) {
      A.c[i] = (A.c[i] + lam.c[i]) * T(0.25);
#pragma unroll 1
      for (int m = 0; m < 3; ++m) X[m].c[i] = (X[m].c[i] + lam.c[i]) * T(0.25);
    }
    pow4 *= T(0.25);
  }
  // X = (A0 - x) / (4^m A), Y likewise, Z = -X - Y
  J invA, Xs, Ys, Zs;
  jpow(A, -2, invA);
  J d0 = A0, d1 = A0;
  d0.c[0] -= x[0];
  d0.c[midx(1, 0, 0)] -= T(1);
  d1.c[0] -= x[1];
  d1.c[midx(0, 1, 0)] -= T(1);
  jmul(d0, invA, Xs);
  jmul(d1, invA, Ys);
#pragma unroll 1
  for (int i = 0; i < J::N; ++i) {
    Xs.c[i] *= pow4;
    Ys.c[i] *= pow4;
    Zs.c[i] = -Xs.c[i] - Ys.c[i];
  }
  J E2, E3, E22, E23;
  jmul(Xs, Ys, E2);
  jmul(Zs, Zs, t);
#pragma unroll 1
  for (int i = 0; i < J::N; ++i) E2.c[i] -= t.c[i];
  jmul(Xs, Ys, t);
  jmul(t, Zs, E3);
  jmul(E2, E2, E22);
  jmul(E2, E3, E23);
  J ser;
#pragma unroll 1
  for (int i = 0; i < J::N; ++i)
    ser.c[i] = -E2.c[i] / T(10) + E3.c[i] / T(14) + E22.c[i] / T(24) - T(3) * E23.c[i] / T(44);
  ser.c[0] += T(1);
  J rsA, rf;
  jpow(A, -1, rsA);
  jmul(rsA, ser, rf);
  const T w[4] = {T(1), T(-2), T(8.0 / 3.0), T(-16.0 / 5.0)};
#pragma unroll 1
  for (int k1 = 0; k1 <= 3; ++k1)
#pragma unroll 1
    for (int k2 = 0; k2 <= 3 - k1; ++k2)
#pragma unroll 1
      for (int k3 = 0; k3 <= 3 - k1 - k2; ++k3)
        ik[midx(k1, k2, k3)] = T(2) * rf.c[midx(k1, k2, k3)] * w[k1] * w[k2] * w[k3];
}

// ------------------------------------------------------------------ lambda
// Largest root of sum y_m^2 / (a2_m + lambda) = 1 for an exterior point (the cubic
// prod (a2 + lambda) - sum y_m^2 prod_{n != m} (a2_n + lambda) = 0), by Newton on the
// convex decreasing rational form from the left, where each step stays below the root;
// 0 for a point inside or on the surface.
template <typename T>
IBEM_HD inline T ell_lambda(const T y[3], const T a2[3]) {
  const T q = y[0] * y[0] / a2[0] + y[1] * y[1] / a2[1] + y[2] * y[2] / a2[2];
  if (q <= T(1)) return T(0);
  const T r2 = y[0] * y[0] + y[1] * y[1] + y[2] * y[2];
  const T amax = vfmax(a2[0], vfmax(a2[1], a2[2]));
  T lam = vfmax(T(0), r2 - amax);
#pragma unroll 1
  for (int it = 0; it < 100; ++it) {
    T f = T(-1), df = T(0);
#pragma unroll 1
    for (int m = 0; m < 3; ++m) {
      const T t = T(1) / (a2[m] + lam);
      f += y[m] * y[m] * t;
      df -= y[m] * y[m] * t * t;
    }
    const T step = -f / df;
    lam += step;
    if (!(step > T(4.0 * NumTraits<T>::eps) * lam)) break;
  }
  return lam;
}

// ------------------------------------------------------------------ potentials
// Jets (order K in the global displacement h of the evaluation point) of the Newtonian
// potentials of the densities 1, x'_p and x'_p x'_q (global components, relative to the
// centre), for an ellipsoid with semi-axes a and rotation Q (Q[3 i + m]: global component
// i of principal axis m), at the point c + d.
template <typename T, int K>
struct EllPot {
  Jet<T, K> f0;      // phi_1
  Jet<T, K> f1[3];   // phi_{x'_p}
  Jet<T, K> f2[6];   // phi_{x'_p x'_q}, pairs 00 01 02 11 12 22
  T d[3];            // x - c
  bool inside;
};

IBEM_HD constexpr int sym_pair(int p, int q) {
  return p <= q ? (p == 0 ? q : (p == 1 ? 2 + q : 5)) : (q == 0 ? p : (q == 1 ? 2 + p : 5));
}

template <typename T, int K>
IBEM_HD inline void ell_potentials(const T d[3], const T Q[9], const T a[3], EllPot<T, K>& P) {
  using J = Jet<T, K>;
  T y[3], a2[3];
#pragma unroll 1
  for (int m = 0; m < 3; ++m) {
    y[m] = Q[m] * d[0] + Q[3 + m] * d[1] + Q[6 + m] * d[2];
    a2[m] = a[m] * a[m];
    P.d[m] = d[m];
  }
  const T lam0 = ell_lambda(y, a2);
  const T qin = y[0] * y[0] / a2[0] + y[1] * y[1] / a2[1] + y[2] * y[2] / a2[2];
  P.inside = qin <= T(1);
  T x[3];
#pragma unroll 1
  for (int m = 0; m < 3; ++m) x[m] = a2[m] + lam0;
  // l_m(h) = y_m + (Q^T h)_m and sq_m = l_m^2
  J sq[3];
#pragma unroll 1
  for (int m = 0; m < 3; ++m) {
    jzero(sq[m]);
    const T l1 = Q[m], l2 = Q[3 + m], l3 = Q[6 + m];
    sq[m].c[0] = y[m] * y[m];
    if (K >= 1) {
      sq[m].c[midx(1, 0, 0)] = T(2) * y[m] * l1;
      sq[m].c[midx(0, 1, 0)] = T(2) * y[m] * l2;
      sq[m].c[midx(0, 0, 1)] = T(2) * y[m] * l3;
    }
    if (K >= 2) {
      sq[m].c[midx(2, 0, 0)] = l1 * l1;
      sq[m].c[midx(0, 2, 0)] = l2 * l2;
      sq[m].c[midx(0, 0, 2)] = l3 * l3;
      sq[m].c[midx(1, 1, 0)] = T(2) * l1 * l2;
      sq[m].c[midx(1, 0, 1)] = T(2) * l1 * l3;
      sq[m].c[midx(0, 1, 1)] = T(2) * l2 * l3;
    }
  }
  // powers of delta(h) = lambda(c + d + h) - lambda0 (zero inside)
  J dp[K + 1];
#pragma unroll 1
  for (int n = 0; n <= K; ++n) jzero(dp[n]);
  dp[0].c[0] = T(1);
  if (!P.inside) {
    T gp = T(0);
#pragma unroll 1
    for (int m = 0; m < 3; ++m) gp -= y[m] * y[m] / (x[m] * x[m]);
    J del, G, inv, t;
    jzero(del);
#pragma unroll 1
    for (int it = 0; it < K; ++it) {
      dp[1] = del;
#pragma unroll 1
      for (int n = 2; n <= K && it > 0; ++n) jmul(dp[n - 1], del, dp[n]);   // del = 0 on the first pass
      jzero(G);
      G.c[0] = T(-1);
#pragma unroll 1
      for (int m = 0; m < 3; ++m) {
        jzero(inv);
        T xm = T(1) / x[m], s = xm;
#pragma unroll 1
        for (int n = 0; n <= K; ++n) {
          jaxpy(s, dp[n], inv);
          s *= -xm;
        }
        jfma_q(T(1), sq[m], inv, G);
      }
      G.c[0] = T(0);   // lambda0 is the root: the constant term vanishes (to rounding)
      jaxpy(-T(1) / gp, G, del);
    }
    dp[1] = del;
#pragma unroll 1
    for (int n = 2; n <= K; ++n) jmul(dp[n - 1], del, dp[n]);
  }
  // I_k(lambda0) and their jets
  T ik[20];
  carlson_ik(x, ik);
  // 1 / x_m, 1 / sqrt(x_m) for the lambda-derivatives
  T ix[3], rx[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    ix[m] = T(1) / x[m];
    rx[m] = vsqrt(ix[m]);
  }
  J I[20];
#pragma unroll 1
  for (int k1 = 0; k1 <= 3; ++k1)
#pragma unroll 1
    for (int k2 = 0; k2 <= 3 - k1; ++k2)
#pragma unroll 1
      for (int k3 = 0; k3 <= 3 - k1 - k2; ++k3) {
        const int id = midx(k1, k2, k3);
        J& o = I[id];
        jzero(o);
        o.c[0] = ik[id];
        if (!P.inside) {
          // dI/dlambda = -f(lambda), f(lambda0 + delta) = f0 prod_m (1 + delta/x_m)^-(k_m + 1/2)
          const int kk[3] = {k1, k2, k3};
          T b[K + 1];
          b[0] = T(1);
#pragma unroll
          for (int n = 1; n <= K; ++n) b[n] = T(0);
          T f0 = T(1);
#pragma unroll 1
          for (int m = 0; m < 3; ++m) {
            const T qm = T(kk[m]) + T(0.5);
            f0 *= rx[m];
            for (int j = 0; j < kk[m]; ++j) f0 *= ix[m];
            T bm[K + 1], coef = T(1);
            bm[0] = T(1);
#pragma unroll
            for (int n = 1; n <= K; ++n) {
              coef *= (-qm - T(n - 1)) / T(n) * ix[m];
              bm[n] = coef;
            }
#pragma unroll
            for (int n = K; n >= 1; --n) {
              T s = T(0);
#pragma unroll
              for (int j = 0; j <= n; ++j) s += b[j] * bm[n - j];
              b[n] = s;
            }
          }
#pragma unroll 1
          for (int n = 0; n < K; ++n) jaxpy(-f0 * b[n] / T(n + 1), dp[n + 1], o);
        }
      }
  // the six products sq_m sq_n (pairs 00 01 02 11 12 22)
  J sq2[6];
#pragma unroll 1
  for (int m = 0; m < 3; ++m)
#pragma unroll 1
    for (int n = m; n < 3; ++n) jmul_q(sq[m], sq[n], sq2[sym_pair(m, n)]);
  // F1_j = int U prod t^j ds/Delta = I_j - sum_m sq_m I_{j+e_m}
  // F2_j = int U^2 prod t^j ds/Delta = I_j - 2 sum_m sq_m I_{j+e_m} + sum_{m,n} sq_m sq_n I_{j+e_m+e_n}
  const T C = T(IBEM_PI) * a[0] * a[1] * a[2];
  J t;
  auto e = [](int m, int k1, int k2, int k3) { return midx(k1 + (m == 0), k2 + (m == 1), k3 + (m == 2)); };
  // phi_1 = C F1_0
  J F;
  F = I[0];
#pragma unroll 1
  for (int m = 0; m < 3; ++m) jfma_q(-T(1), sq[m], I[e(m, 0, 0, 0)], F);
#pragma unroll 1
  for (int i = 0; i < J::N; ++i) P.f0.c[i] = C * F.c[i];
  // phi_{y'_m} = C a_m^2 l_m F1_{e_m}, rotated to global densities
  J p1[3];
#pragma unroll 1
  for (int m = 0; m < 3; ++m) {
    const int km[3] = {m == 0, m == 1, m == 2};
    F = I[midx(km[0], km[1], km[2])];
#pragma unroll 1
    for (int n = 0; n < 3; ++n) jfma_q(-T(1), sq[n], I[e(n, km[0], km[1], km[2])], F);
    jmul_lin(C * a2[m] * y[m], C * a2[m] * Q[m], C * a2[m] * Q[3 + m], C * a2[m] * Q[6 + m], F, p1[m]);
  }
#pragma unroll 1
  for (int p = 0; p < 3; ++p) {
    jzero(P.f1[p]);
#pragma unroll 1
    for (int m = 0; m < 3; ++m) jaxpy(Q[3 * p + m], p1[m], P.f1[p]);
  }
  // phi_{y'_m y'_n}
  J F20;   // F2_0
  F20 = I[0];
#pragma unroll 1
  for (int m = 0; m < 3; ++m) jfma_q(-T(2), sq[m], I[e(m, 0, 0, 0)], F20);
#pragma unroll 1
  for (int m = 0; m < 3; ++m)
#pragma unroll 1
    for (int n = m; n < 3; ++n)
      jfma(m == n ? T(1) : T(2), sq2[sym_pair(m, n)], I[midx((m == 0) + (n == 0), (m == 1) + (n == 1), (m == 2) + (n == 2))],
           F20);
  J p2[6];
#pragma unroll 1
  for (int m = 0; m < 3; ++m)
#pragma unroll 1
    for (int n = m; n < 3; ++n) {
      const int km[3] = {(m == 0) + (n == 0), (m == 1) + (n == 1), (m == 2) + (n == 2)};
      // F1_{e_m + e_n}, times a_m^2 a_n^2 l_m l_n
      F = I[midx(km[0], km[1], km[2])];
#pragma unroll 1
      for (int r = 0; r < 3; ++r) jfma_q(-T(1), sq[r], I[e(r, km[0], km[1], km[2])], F);
      jmul_lin(y[m], Q[m], Q[3 + m], Q[6 + m], F, t);
      J& o = p2[sym_pair(m, n)];
      jmul_lin(C * a2[m] * a2[n] * y[n], C * a2[m] * a2[n] * Q[n], C * a2[m] * a2[n] * Q[3 + n],
               C * a2[m] * a2[n] * Q[6 + n], t, o);
      if (m == n) {
        // + C a_m^2/4 F2_0 - C a_m^4/4 F2_{e_m}
        jaxpy(C * a2[m] / T(4), F20, o);
        const int em[3] = {m == 0, m == 1, m == 2};
        F = I[midx(em[0], em[1], em[2])];
#pragma unroll 1
        for (int r = 0; r < 3; ++r) jfma_q(-T(2), sq[r], I[e(r, em[0], em[1], em[2])], F);
#pragma unroll 1
        for (int r = 0; r < 3; ++r)
#pragma unroll 1
          for (int s = r; s < 3; ++s)
            jfma(r == s ? T(1) : T(2), sq2[sym_pair(r, s)],
                 I[midx(em[0] + (r == 0) + (s == 0), em[1] + (r == 1) + (s == 1), em[2] + (r == 2) + (s == 2))], F);
        jaxpy(-C * a2[m] * a2[m] / T(4), F, o);
      }
    }
  // global densities x'_p x'_q = sum_mn Q_pm Q_qn y'_m y'_n
#pragma unroll 1
  for (int p = 0; p < 3; ++p)
#pragma unroll 1
    for (int q = p; q < 3; ++q) {
      J& o = P.f2[sym_pair(p, q)];
      jzero(o);
#pragma unroll 1
      for (int m = 0; m < 3; ++m)
#pragma unroll 1
        for (int n = 0; n < 3; ++n) jaxpy(Q[3 * p + m] * Q[3 * q + n], p2[sym_pair(m, n)], o);
    }
}

// ------------------------------------------------------------------ derivatives
// Derivative tables of one evaluation: phi[r][midx(alpha)] = d^alpha phi_rho for |alpha| <= K
// and psi[r][midx(beta)] = d^beta psi_rho for 4 <= |beta| <= K + 1, with r = 0 the uniform
// density and r = 1 + p the density x'_p.  d^beta psi = d^(beta - e_k) (x_k phi_rho -
// phi_{rho x'_k}) for any k with beta_k > 0; d^alpha (h_k f) = alpha! c_(alpha - e_k)(f).
template <typename T, int K>
struct EllDer {
  T phi[4][nmono(K)];
  T psi[4][nmono(K + 1)];
  bool inside;
};

IBEM_HD IBEM_INLINE int fact_small(int n) { return n <= 1 ? 1 : (n == 2 ? 2 : (n == 3 ? 6 : (n == 4 ? 24 : 120))); }

template <typename T, int K>
IBEM_HD inline void ell_derivs(const EllPot<T, K>& P, EllDer<T, K>& D) {
  D.inside = P.inside;
#pragma unroll 1
  for (int r = 0; r < 4; ++r) {
    const Jet<T, K>& f = r == 0 ? P.f0 : P.f1[r - 1];
#pragma unroll 1
    for (int a1 = 0; a1 <= K; ++a1)
#pragma unroll 1
      for (int a2 = 0; a2 <= K - a1; ++a2)
#pragma unroll 1
        for (int a3 = 0; a3 <= K - a1 - a2; ++a3) {
          const int id = midx(a1, a2, a3);
          D.phi[r][id] = T(fact_small(a1) * fact_small(a2) * fact_small(a3)) * f.c[id];
        }
#pragma unroll 1
    for (int b1 = 0; b1 <= K + 1; ++b1)
#pragma unroll 1
      for (int b2 = 0; b2 <= K + 1 - b1; ++b2)
#pragma unroll 1
        for (int b3 = 0; b3 <= K + 1 - b1 - b2; ++b3) {
          const int deg = b1 + b2 + b3;
          if (deg < 4) continue;
          const int k = b1 > 0 ? 0 : (b2 > 0 ? 1 : 2);
          const int a[3] = {b1 - (k == 0), b2 - (k == 1), b3 - (k == 2)};
          const Jet<T, K>& g = r == 0 ? P.f1[k] : P.f2[sym_pair(r - 1, k)];
          const int ia = midx(a[0], a[1], a[2]);
          const T af = T(fact_small(a[0]) * fact_small(a[1]) * fact_small(a[2]));
          T v = P.d[k] * f.c[ia] - g.c[ia];
          if (a[k] > 0) v += f.c[midx(a[0] - (k == 0), a[1] - (k == 1), a[2] - (k == 2))];
          D.psi[r][midx(b1, b2, b3)] = af * v;
        }
  }
}

// D(i,j,k,l [,p]; R) of the reference (strain ij, eigenstrain kl of density rho = -1
// (uniform) or p), without the factor 1 / (8 pi (1 - nu)):
//   psi_,klijR - 2 nu d_kl phi_,ijR - (1 - nu)(d_il phi_,kjR + d_jl phi_,kiR + d_ik phi_,ljR + d_jk phi_,liR)
template <typename T, int K>
IBEM_HD inline T Dsum(const EllDer<T, K>& D, T nu, int rho, int i, int j, int k, int l, const int* R, int nR) {
  const int r = rho + 1;
  int c[3] = {0, 0, 0};
  for (int s = 0; s < nR; ++s) ++c[R[s]];
  int cp[3] = {c[0], c[1], c[2]};
  ++cp[k];
  ++cp[l];
  ++cp[i];
  ++cp[j];
  T v = D.psi[r][midx(cp[0], cp[1], cp[2])];
  auto ph = [&](int x1, int x2) {
    int q[3] = {c[0], c[1], c[2]};
    ++q[x1];
    ++q[x2];
    return D.phi[r][midx(q[0], q[1], q[2])];
  };
  if (k == l) v -= T(2) * nu * ph(i, j);
  T s4 = T(0);
  if (i == l) s4 += ph(k, j);
  if (j == l) s4 += ph(k, i);
  if (i == k) s4 += ph(l, j);
  if (j == k) s4 += ph(l, i);
  return v - (T(1) - nu) * s4;
}

// ------------------------------------------------------------------ blocks and sums
// layout-24 unknown u: order 0 (u < 6): symmetric pair t = u; order 1: t = (u - 6) / 3,
// moment p = (u - 6) % 3.  Pairs t: 00 01 02 11 12 22.
IBEM_HD constexpr int pair_i(int t) { return t < 3 ? 0 : (t < 5 ? 1 : 2); }
IBEM_HD constexpr int pair_j(int t) { return t < 3 ? t : (t < 5 ? t - 2 : 2); }

// One (s, h) block of the layout-24 equivalent-inclusion system for an ellipsoidal source
// h (integratorElastic3D.cpp:341-567 with the sphere's potentials replaced): rows (s, ij[,r]),
// columns (h, mn[,p]):
//   map[m][n] (-sum_kl (C0 - C1)_ijkl D(k,l,m,n[,p]; [r]) + [self] C0_ijmn delta),
// d = centre of s - centre of h.  out[row * 24 + col].
// The evaluation runs in coordinates scaled by the source's longest semi-axis s, where every
// quantity is O(1); the tensor is scale-free except for one factor s per column of order 1
// and 1/s per row of order 1.
template <typename T>
IBEM_HD inline void ell_block24(const T d[3], const T Q[9], const T a[3], const SphMat& mc, bool self, T* out) {
  const T sc = vfmax(a[0], vfmax(a[1], a[2])), isc = T(1) / sc;
  EllDer<T, 4> P;
  {
    T ds[3], as[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      ds[i] = d[i] * isc;
      as[i] = a[i] * isc;
    }
    EllPot<T, 4> pot;
    ell_potentials<T, 4>(ds, Q, as, pot);
    ell_derivs(pot, P);
  }
  const T nu = T(mc.tn2) / T(2);
  const T kd = T(mc.kd);
  // Dt[r][rho][t][u] = D(pair t, pair u [, rho]; R) with r = 0: no collocation derivative,
  // 1 + R: the derivative R; rho = 0 uniform, 1 + p linear.  576 values, one Dsum each.
  T Dt[4][4][6][6];
#pragma unroll 1
  for (int r = 0; r < 4; ++r) {
    const int R[1] = {r - 1};
#pragma unroll 1
    for (int rho = 0; rho < 4; ++rho)
#pragma unroll 1
      for (int t = 0; t < 6; ++t)
#pragma unroll 1
        for (int u = 0; u < 6; ++u)
          Dt[r][rho][t][u] = Dsum(P, nu, rho - 1, pair_i(t), pair_j(t), pair_i(u), pair_j(u), R, r > 0 ? 1 : 0);
  }
#pragma unroll 1
  for (int rr = 0; rr < 24; ++rr) {
    const int ro = rr < 6 ? 0 : 1;
    const int rt = ro ? (rr - 6) / 3 : rr;
    const int r = ro ? 1 + (rr - 6) % 3 : 0;
    const int i = pair_i(rt), j = pair_j(rt);
#pragma unroll 1
    for (int cc = 0; cc < 24; ++cc) {
      const int co = cc < 6 ? 0 : 1;
      const int ct = co ? (cc - 6) / 3 : cc;
      const int rho = co ? 1 + (cc - 6) % 3 : 0;
      const int m = pair_i(ct), n = pair_j(ct);
      // sum_kl (C0 - C1)_ijkl D_kl = dlam d_ij D_kk + 2 dmu D_ij
      T acc = T(2) * T(mc.dmu) * Dt[r][rho][rt][ct];
      if (i == j) acc += T(mc.dlam) * (Dt[r][rho][0][ct] + Dt[r][rho][3][ct] + Dt[r][rho][5][ct]);
      T v = -kd * acc * (co == ro ? T(1) : (co ? sc : isc));
      if (self && ro == co && (ro == 0 || r == rho)) {
        // C0_ijmn
        T c0 = T(mc.mu0) * (T((i == m) * (j == n)) + T((i == n) * (j == m)));
        if (i == j && m == n) c0 += T(mc.lam0);
        v += c0;
      }
      out[rr * 24 + cc] = (m == n ? T(1) : T(2)) * v;
    }
  }
}

// Strain (6: xx xy xz yy yz zz) at c + d due to the layout-24 eigenstrain E of an
// ellipsoidal source (postProcessorElastic3D.cpp:367-470 with the ellipsoid's potentials),
// accumulated into e.  Returns true if the point lies inside (or on) the ellipsoid.
// Coordinates scaled by the longest semi-axis s; the order-1 coefficients (of x'_p) carry
// the factor s back.
template <typename T>
IBEM_HD inline bool ell_strain24(const T d[3], const T Q[9], const T a[3], const SphMat& mc, const T* E, T* e) {
  const T sc = vfmax(a[0], vfmax(a[1], a[2])), isc = T(1) / sc;
  EllDer<T, 3> P;
  {
    T ds[3], as[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      ds[i] = d[i] * isc;
      as[i] = a[i] * isc;
    }
    EllPot<T, 3> pot;
    ell_potentials<T, 3>(ds, Q, as, pot);
    ell_derivs(pot, P);
  }
  const T nu = T(mc.tn2) / T(2);
  const T kd = T(mc.kd);
  for (int rt = 0; rt < 6; ++rt) {
    const int i = pair_i(rt), j = pair_j(rt);
    T s = T(0);
    for (int cc = 0; cc < 24; ++cc) {
      const int co = cc < 6 ? 0 : 1;
      const int ct = co ? (cc - 6) / 3 : cc;
      const int rho = co ? (cc - 6) % 3 : -1;
      const int m = pair_i(ct), n = pair_j(ct);
      s += (m == n ? T(1) : T(2)) * Dsum(P, nu, rho, i, j, m, n, nullptr, 0) * (co ? sc * E[cc] : E[cc]);
    }
    e[rt] += kd * s;
  }
  return P.inside;
}

// Rotation matrix (Q[3 i + m]: global component i of principal axis m) of a unit quaternion
// (w, x, y, z); the quaternion is normalised first.
template <typename T>
IBEM_HD inline void quat_to_rot(const T* q, T* Q) {
  const T n = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  const T w = q[0] / n, x = q[1] / n, y = q[2] / n, z = q[3] / n;
  Q[0] = T(1) - T(2) * (y * y + z * z);
  Q[1] = T(2) * (x * y - w * z);
  Q[2] = T(2) * (x * z + w * y);
  Q[3] = T(2) * (x * y + w * z);
  Q[4] = T(1) - T(2) * (x * x + z * z);
  Q[5] = T(2) * (y * z - w * x);
  Q[6] = T(2) * (x * z - w * y);
  Q[7] = T(2) * (y * z + w * x);
  Q[8] = T(1) - T(2) * (x * x + y * y);
}

}  // namespace ell
}  // namespace ibem
