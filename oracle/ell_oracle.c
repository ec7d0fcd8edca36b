/*
 * ell_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle) for ellipsoidal inclusions.
 *
 * The reference has no elastic ellipsoid code; its spherical integrator
 * (integratorElastic3DHelper.cpp:2394-2554) defines the interaction tensor
 *     D_ijkl[rho] = [psi_,klij - 2 nu d_kl phi_,ij - (1 - nu)(d_il phi_,kj + d_jl phi_,ki
 *                   + d_ik phi_,lj + d_jk phi_,li)] / (8 pi (1 - nu))
 * from phi = int rho / |x - x'| and psi = int rho |x - x'| over the inclusion.  This file
 * evaluates the same tensor for an ellipsoid by a route that shares nothing with the
 * CUDA library's (Ferrers / Dyson potentials, Carlson R_F in Taylor arithmetic):
 *
 *  orc_ell_D_quad   exterior points: the kernel derivatives d^alpha |z| and d^alpha 1/|z|
 *                   (z = x - x') integrated over the ellipsoid by tensor-product Gauss
 *                   rules in mapped spherical coordinates (x' = c + Q diag(a) u, |u| <= 1:
 *                   Gauss-Legendre in the radius and in cos(theta), the trapezoid rule in
 *                   the azimuth).  Differentiation under the integral is exact outside the
 *                   body; accuracy is set by the rule and by the distance to the body.
 *  orc_ell_I        I_k(lambda) = int_lambda^inf prod (a_m^2 + s)^-(k_m + 1/2) ds by Gauss-
 *                   Legendre quadrature after s = lambda + c (1/u^2 - 1) (a smooth integrand
 *                   on [0, 1]), for checking the library's Carlson-based values.
 *  orc_carlson_rf / orc_carlson_rd   plain Carlson R_F and R_D (duplication algorithm,
 *                   B. C. Carlson, Numer. Algorithms 10 (1995) 13-26), scalar.
 *  orc_ell_lambda   largest root of the cubic sum y_m^2 / (a_m^2 + lambda) = 1 by bisection.
 *
 * Layout of orc_ell_D_quad's output: the same digit order as orc_D (ibem_oracle.c):
 * (strain i, strain j, eigenstrain k, eigenstrain l [, moment p] [, derivative r]),
 * 3^(4 + order + nder) values, the moment taken about the centre in global coordinates.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.141592653589793

/* Gauss-Legendre nodes and weights on [-1, 1] (Newton on P_n, Golub-Welsch not needed) */
static void gauss_legendre(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    double z = cos(ORC_PI * (i + 0.75) / (n + 0.5)), pp = 0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; ++j) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1);
      double z1 = z;
      z = z1 - p1 / pp;
      if (fabs(z - z1) < 1e-16) break;
    }
    x[i] = z;
    w[i] = 2 / ((1 - z * z) * pp * pp);
  }
}

/* d^alpha r^s at z (derivatives in x, z = x - x'), alpha given by counts */
static double dpow_c(const double* z, double r, double s, int c0, int c1, int c2) {
  int c[3] = {c0, c1, c2};
  int i = c[0] > 0 ? 0 : (c[1] > 0 ? 1 : (c[2] > 0 ? 2 : -1));
  if (i < 0) return pow(r, s);
  /* d_i r^s = s z_i r^(s-2); the remaining alpha - e_i derivatives by Leibniz */
  c[i] -= 1;
  double v = z[i] * dpow_c(z, r, s - 2, c[0], c[1], c[2]);
  if (c[i] > 0) {
    int ci = c[i];
    c[i] -= 1;
    v += ci * dpow_c(z, r, s - 2, c[0], c[1], c[2]);
  }
  return s * v;
}

/* multi-index <-> flat id over counts with |alpha| <= 6: id = c0 * 49 + c1 * 7 + c2 */
#define AID(c0, c1, c2) ((c0) * 49 + (c1) * 7 + (c2))
#define NAID (7 * 49)

static int idx_counts(const int* idx, int n) {
  int c[3] = {0, 0, 0};
  for (int s = 0; s < n; ++s) c[idx[s]]++;
  return AID(c[0], c[1], c[2]);
}

int orc_ell_D_quad(int order, int nder, const double* x, const double* a, const double* Q, double nu,
                   int nr, int nt, int np, double* out) {
  /* integrated kernel derivatives: Phi[rho][alpha] (1/r, |alpha| <= 2 + nder) and
   * Psi[rho][alpha] (r, |alpha| <= 4 + nder), rho = 0: 1, rho = 1 + p: x'_p */
  const int mphi = 2 + nder, mpsi = 4 + nder;
  double* acc = (double*)calloc((size_t)2 * 4 * NAID, sizeof(double));
  double* Phi = acc;
  double* Psi = acc + 4 * NAID;
  double *xr = malloc(sizeof(double) * nr), *wr = malloc(sizeof(double) * nr);
  double *xt = malloc(sizeof(double) * nt), *wt = malloc(sizeof(double) * nt);
  gauss_legendre(nr, xr, wr);
  gauss_legendre(nt, xt, wt);
  const double vol = a[0] * a[1] * a[2];
  for (int ir = 0; ir < nr; ++ir) {
    const double rho = 0.5 * (xr[ir] + 1), wrho = 0.5 * wr[ir] * rho * rho;
    for (int it = 0; it < nt; ++it) {
      const double ct = xt[it], st = sqrt(fmax(0.0, 1 - ct * ct));
      for (int ip = 0; ip < np; ++ip) {
        const double ph = 2 * ORC_PI * (ip + 0.5) / np;
        const double u[3] = {rho * st * cos(ph), rho * st * sin(ph), rho * ct};
        const double w = vol * wrho * wt[it] * (2 * ORC_PI / np);
        double xp[3], z[3];
        for (int i = 0; i < 3; ++i) {
          xp[i] = Q[3 * i] * a[0] * u[0] + Q[3 * i + 1] * a[1] * u[1] + Q[3 * i + 2] * a[2] * u[2];
          z[i] = x[i] - xp[i];
        }
        const double r = sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
        const double dens[4] = {w, w * xp[0], w * xp[1], w * xp[2]};
        const int nrho = order == 0 ? 1 : 4;
        for (int c0 = 0; c0 <= mpsi; ++c0)
          for (int c1 = 0; c0 + c1 <= mpsi; ++c1)
            for (int c2 = 0; c0 + c1 + c2 <= mpsi; ++c2) {
              const int n = c0 + c1 + c2;
              if (n >= 4) {
                const double v = dpow_c(z, r, 1.0, c0, c1, c2);
                for (int q = 0; q < nrho; ++q) Psi[q * NAID + AID(c0, c1, c2)] += dens[q] * v;
              }
              if (n >= 2 && n <= mphi) {
                const double v = dpow_c(z, r, -1.0, c0, c1, c2);
                for (int q = 0; q < nrho; ++q) Phi[q * NAID + AID(c0, c1, c2)] += dens[q] * v;
              }
            }
      }
    }
  }
  free(xr); free(wr); free(xt); free(wt);
  const int total = 4 + order + nder;
  int lim = 1;
  for (int t = 0; t < total; ++t) lim *= 3;
  const double kd = 1.0 / (8 * ORC_PI * (1 - nu));
  for (int f = 0; f < lim; ++f) {
    int dig[8], g = f;
    for (int t = total - 1; t >= 0; --t) { dig[t] = g % 3; g /= 3; }
    const int i = dig[0], j = dig[1], k = dig[2], l = dig[3];
    const int q = order ? 1 + dig[4] : 0;
    const int* R = dig + 4 + order;
    int id[8], n = 0;
    id[n++] = k; id[n++] = l; id[n++] = i; id[n++] = j;
    for (int s = 0; s < nder; ++s) id[n++] = R[s];
    double v = Psi[q * NAID + idx_counts(id, n)];
#define PH(x1, x2) (id[0] = (x1), id[1] = (x2), Phi[q * NAID + idx_counts(id, 2 + nder)])
    for (int s = 0; s < nder; ++s) id[2 + s] = R[s];
    if (k == l) v -= 2 * nu * PH(i, j);
    double s4 = 0;
    if (i == l) s4 += PH(k, j);
    if (j == l) s4 += PH(k, i);
    if (i == k) s4 += PH(l, j);
    if (j == k) s4 += PH(l, i);
#undef PH
    out[f] = kd * (v - (1 - nu) * s4);
  }
  free(acc);
  return lim;
}

/* I_k(lambda) by quadrature: s = lambda + c (1/u^2 - 1), c = a_min^2 + lambda, so that
 * I_k = 2 c int_0^1 u^(2|k|) prod_m (c + d_m u^2)^-(k_m + 1/2) du, d_m = a_m^2 - a_min^2. */
double orc_ell_I(const int* k, const double* a, double lambda, int n) {
  double amin2 = fmin(a[0] * a[0], fmin(a[1] * a[1], a[2] * a[2]));
  const double c = amin2 + lambda;
  double* x = malloc(sizeof(double) * n);
  double* w = malloc(sizeof(double) * n);
  gauss_legendre(n, x, w);
  const int kk = k[0] + k[1] + k[2];
  double s = 0;
  for (int i = 0; i < n; ++i) {
    const double u = 0.5 * (x[i] + 1);
    double f = pow(u, 2 * kk);
    for (int m = 0; m < 3; ++m) f *= pow(c + (a[m] * a[m] - amin2) * u * u, -(k[m] + 0.5));
    s += 0.5 * w[i] * f;
  }
  free(x);
  free(w);
  return 2 * c * s;
}

/* Carlson R_F (duplication, Carlson 1995 section 2) */
double orc_carlson_rf(double x, double y, double z) {
  const double r = 1e-16;
  double A0 = (x + y + z) / 3, A = A0;
  double Q = pow(3 * r, -1.0 / 6.0) * fmax(fabs(A0 - x), fmax(fabs(A0 - y), fabs(A0 - z)));
  double xm = x, ym = y, zm = z, p4 = 1;
  while (p4 * Q >= fabs(A)) {
    double lam = sqrt(xm) * sqrt(ym) + sqrt(xm) * sqrt(zm) + sqrt(ym) * sqrt(zm);
    A = (A + lam) / 4; xm = (xm + lam) / 4; ym = (ym + lam) / 4; zm = (zm + lam) / 4;
    p4 /= 4;
  }
  double X = p4 * (A0 - x) / A, Y = p4 * (A0 - y) / A, Z = -X - Y;
  double E2 = X * Y - Z * Z, E3 = X * Y * Z;
  return (1 - E2 / 10 + E3 / 14 + E2 * E2 / 24 - 3 * E2 * E3 / 44) / sqrt(A);
}

/* Carlson R_D (duplication, Carlson 1995 section 4) */
double orc_carlson_rd(double x, double y, double z) {
  const double r = 1e-16;
  double A0 = (x + y + 3 * z) / 5, A = A0;
  double Q = pow(r / 4, -1.0 / 6.0) * fmax(fabs(A0 - x), fmax(fabs(A0 - y), fabs(A0 - z)));
  double xm = x, ym = y, zm = z, p4 = 1, sum = 0;
  while (p4 * Q >= fabs(A)) {
    double lam = sqrt(xm) * sqrt(ym) + sqrt(xm) * sqrt(zm) + sqrt(ym) * sqrt(zm);
    sum += p4 / (sqrt(zm) * (zm + lam));
    A = (A + lam) / 4; xm = (xm + lam) / 4; ym = (ym + lam) / 4; zm = (zm + lam) / 4;
    p4 /= 4;
  }
  double X = p4 * (A0 - x) / A, Y = p4 * (A0 - y) / A, Z = -(X + Y) / 3;
  double E2 = X * Y - 6 * Z * Z, E3 = (3 * X * Y - 8 * Z * Z) * Z, E4 = 3 * (X * Y - Z * Z) * Z * Z,
         E5 = X * Y * Z * Z * Z;
  double ser = 1 - 3 * E2 / 14 + E3 / 6 + 9 * E2 * E2 / 88 - 3 * E4 / 22 - 9 * E2 * E3 / 52 + 3 * E5 / 26;
  return p4 * pow(A, -1.5) * ser + 3 * sum;
}

/* largest root of sum y_m^2 / (a_m^2 + lambda) = 1 (0 inside), by bisection */
double orc_ell_lambda(const double* y, const double* a) {
  double q = 0, r2 = 0;
  for (int m = 0; m < 3; ++m) { q += y[m] * y[m] / (a[m] * a[m]); r2 += y[m] * y[m]; }
  if (q <= 1) return 0;
  double lo = 0, hi = r2;
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi), f = -1;
    for (int m = 0; m < 3; ++m) f += y[m] * y[m] / (a[m] * a[m] + mid);
    if (f > 0) lo = mid; else hi = mid;
  }
  return 0.5 * (lo + hi);
}
