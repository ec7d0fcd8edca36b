/*
 * ibem_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C CPU restatement of the reference's 3D elastic spherical iBEM path
 * (huoxingshu1/iBEMProject, namespace Elastic3DSpherical).  It is the checker for
 * the CUDA library and the CPU baseline timed beside it; the product never links,
 * loads or calls it.  Every function cites the reference file:line it follows.
 *
 * How the potentials are evaluated.  The reference hand-expands every derivative of
 * the sphere potentials (integratorElastic3DHelper.cpp:41-664).  All of them are
 * exact derivatives of a few base forms built from the sphere integrals
 *     J_m = I_m0(lambda) = 4 pi a^3 / ((2m+1) (a^2+lambda)^(m+1/2))     (:41-45)
 * with lambda = |x|^2 - a^2 outside the sphere and 0 inside (:137-140), whose
 * x-derivative is  dJ_m/dx_p = -(2m+3) x_p J_{m+1}  outside and 0 inside (:47-104).
 * This file keeps those base forms and differentiates them with a generic Leibniz
 * recursion at concrete indices, instead of restating each expanded formula:
 *     V_n        = (J_n - |x|^2 J_{n+1}) / 2,  V_n,p = -x_p J_{n+1}      (:169-244)
 *     phi,I      = V_0,I                                                (:279-313)
 *     psi,i      = x_i (V_0 - a^2 V_1)                                  (:429-462)
 *     phi_p      = a^2 x_p V_1                                          (:266-353)
 *     psi_p,i    = a^2 [ d_ip Q + x_p x_i W1 ],  Q,j = x_j W1,  W1 = V_1 - a^2 V_2   (:464-527)
 *     phi_pq,i   = a^2 [ a^2 (x_p x_q V_2),i - d_pq x_i W1 ]            (:355-426)
 *     psi_pq,i   = a^4 [ (d_pi x_q + d_qi x_p) P + x_p x_q x_i W2 ] - a^2 d_pq x_i S,
 *                  P,j = x_j W2, S,j = x_j U,  W2 = V_2 - a^2 V_3,
 *                  U = V_1 - 2 a^2 V_2 + a^4 V_3                        (:529-750)
 * The Kelvin solution (:2559-2593) is differentiated the same way from |x| and 1/|x|.
 *
 * Layout conventions follow the reference: unknowns per particle ordered
 * [E_ij (i<=j) | E_ijp | E_ijpq] (configElastic3D.cpp:160-195), column-major
 * matrices, boundary unknowns first (3 per node), 12 traction values per element.
 * Three per-particle layouts are supported: 78 (the reference's), 24 (orders 0/1
 * only: the same entries, truncated) and 60 (order-2 eigenstrain stored once per
 * symmetric pair p<=q; columns of (p,q) and (q,p) summed, rows r<=z kept).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.141592653589793 /* GlobalConstant.h:26 */

typedef struct {
  double E0, nu0, E1, nu1;
} orc_mat;

/* ------------------------------------------------------------------------ */
/* Materials: Constitutive / Constitutive1 (integratorElastic3DHelper.cpp:2376-2389) */
typedef struct {
  double mu0, nu0, mu1, nu1, lam0, lam1;
} Mat;

static Mat mat_from(const orc_mat* m) {
  Mat r;
  r.nu0 = m->nu0;
  r.nu1 = m->nu1;
  r.mu0 = m->E0 / (2.0 * (1.0 + m->nu0)); /* configElastic3D.cpp:56 */
  r.mu1 = m->E1 / (2.0 * (1.0 + m->nu1)); /* configElastic3D.cpp:118 */
  r.lam0 = 2.0 * r.mu0 * r.nu0 / (1 - 2 * r.nu0);
  r.lam1 = 2.0 * r.mu1 * r.nu1 / (1 - 2 * r.nu1);
  return r;
}
static inline int dl(int i, int j) { return i == j; }
static double C0(const Mat* M, int i, int j, int k, int l) {
  return M->lam0 * dl(i, j) * dl(k, l) + M->mu0 * (dl(i, k) * dl(j, l) + dl(i, l) * dl(j, k));
}
static double C1(const Mat* M, int i, int j, int k, int l) {
  return M->lam1 * dl(i, j) * dl(k, l) + M->mu1 * (dl(i, k) * dl(j, l) + dl(i, l) * dl(j, k));
}
static const int MAPF[3][3] = {{1, 2, 2}, {0, 1, 2}, {0, 0, 1}}; /* GlobalConstant.h:28 */

/* ------------------------------------------------------------------------ */
/* Sphere potentials and their derivatives at concrete indices.             */
typedef struct {
  double x[3];
  double a, a2, r2, rho2; /* rho2 = a^2 + lambda */
  int ext;                /* lambda > 0 */
} Ctx;

static void ctx_init(Ctx* c, const double* x, double a) {
  c->x[0] = x[0];
  c->x[1] = x[1];
  c->x[2] = x[2];
  c->a = a;
  c->a2 = a * a;
  c->r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
  double lam = c->r2 - c->a2;
  c->ext = lam > 0;
  if (!c->ext) lam = 0;
  c->rho2 = c->a2 + lam;
}

/* remove entry t from idx[0..k-1] into out */
static void drop(const int* idx, int k, int t, int* out) {
  int n = 0;
  for (int s = 0; s < k; ++s)
    if (s != t) out[n++] = idx[s];
}

/* d^k J_m (I_n0..I_n4, integratorElastic3DHelper.cpp:41-104) */
static double dJ(const Ctx* c, int m, const int* idx, int k) {
  if (k == 0) return 4 * ORC_PI * c->a * c->a2 / ((2 * m + 1) * pow(c->rho2, m + 0.5));
  if (!c->ext) return 0.0;
  /* d_{i0} J_m = -(2m+3) x_{i0} J_{m+1}; then Leibniz over the remaining indices */
  int rest[16], r2[16];
  const int i0 = idx[0];
  memcpy(rest, idx + 1, sizeof(int) * (k - 1));
  double v = c->x[i0] * dJ(c, m + 1, rest, k - 1);
  for (int t = 0; t < k - 1; ++t)
    if (rest[t] == i0) {
      drop(rest, k - 1, t, r2);
      v += dJ(c, m + 1, r2, k - 2);
    }
  return -(2 * m + 3) * v;
}

/* d^k V_n (V_n0..V_n5, :169-244) */
static double dV(const Ctx* c, int n, const int* idx, int k) {
  if (k == 0) return 0.5 * (dJ(c, n, idx, 0) - c->r2 * dJ(c, n + 1, idx, 0));
  int rest[16], r2[16];
  const int i0 = idx[0];
  memcpy(rest, idx + 1, sizeof(int) * (k - 1));
  double v = c->x[i0] * dJ(c, n + 1, rest, k - 1);
  for (int t = 0; t < k - 1; ++t)
    if (rest[t] == i0) {
      drop(rest, k - 1, t, r2);
      v += dJ(c, n + 1, r2, k - 2);
    }
  return -v;
}

/* linear combination sum_t coef[t] V_{n0+t} */
typedef struct {
  int n0, cnt;
  double coef[3];
} Lin;

static double dLin(const Ctx* c, const Lin* L, const int* idx, int k) {
  double v = 0;
  for (int t = 0; t < L->cnt; ++t)
    if (L->coef[t] != 0) v += L->coef[t] * dV(c, L->n0 + t, idx, k);
  return v;
}

/* d^k [ x_{xf[0]} ... x_{xf[nx-1]} F ],  F = L (prim == 0) or the primitive P of L
 * with P,j = x_j L (prim == 1; only derivatives of order >= 1 of P are defined). */
static double dXLin(const Ctx* c, const int* xf, int nx, const Lin* L, int prim,
                    const int* idx, int k) {
  if (nx == 0) {
    if (!prim) return dLin(c, L, idx, k);
    if (k == 0) return NAN;
    int j0 = idx[0];
    return dXLin(c, &j0, 1, L, 0, idx + 1, k - 1);
  }
  const int c0 = xf[0];
  double v = c->x[c0] * dXLin(c, xf + 1, nx - 1, L, prim, idx, k);
  int r2[16];
  for (int t = 0; t < k; ++t)
    if (idx[t] == c0) {
      drop(idx, k, t, r2);
      v += dXLin(c, xf + 1, nx - 1, L, prim, r2, k - 1);
    }
  return v;
}

/* The six potential families.  order = eigenstrain polynomial order of the source
 * (0: uniform, 1: linear weight x'_p, 2: quadratic weight x'_p x'_q). */
static double d_phi(const Ctx* c, int order, int p, int q, const int* idx, int k) {
  const double a2 = c->a2;
  if (order == 0) {
    Lin V0 = {0, 1, {1, 0, 0}};
    return dLin(c, &V0, idx, k); /* Phi_0x = V_n x with n = 0 (:279-313) */
  }
  if (order == 1) {
    Lin V1 = {1, 1, {1, 0, 0}};
    return a2 * dXLin(c, &p, 1, &V1, 0, idx, k); /* Phi_1x (:266, :316-353) */
  }
  /* Phi_2x (:355-426), defined for k >= 1 */
  Lin V2 = {2, 1, {1, 0, 0}};
  Lin W1 = {1, 2, {1, -a2, 0}};
  int pq[2] = {p, q};
  double v = a2 * dXLin(c, pq, 2, &V2, 0, idx, k);
  if (p == q) v -= dXLin(c, idx, 1, &W1, 0, idx + 1, k - 1);
  return a2 * v;
}

static double d_psi(const Ctx* c, int order, int p, int q, const int* idx, int k) {
  const double a2 = c->a2;
  const int i0 = idx[0];
  if (order == 0) {
    Lin W0 = {0, 2, {1, -a2, 0}}; /* Psi_0x (:429-462) */
    return dXLin(c, &i0, 1, &W0, 0, idx + 1, k - 1);
  }
  if (order == 1) {
    Lin W1 = {1, 2, {1, -a2, 0}}; /* Psi_1x (:464-527) */
    int pi[2] = {p, i0};
    double v = dXLin(c, pi, 2, &W1, 0, idx + 1, k - 1);
    if (p == i0) v += dXLin(c, NULL, 0, &W1, 1, idx + 1, k - 1);
    return a2 * v;
  }
  Lin W2 = {2, 2, {1, -a2, 0}}; /* Psi_2x (:529-750) */
  Lin U = {1, 3, {1, -2 * a2, a2 * a2}};
  int pqi[3] = {p, q, i0};
  double v = dXLin(c, pqi, 3, &W2, 0, idx + 1, k - 1);
  if (p == i0) v += dXLin(c, &q, 1, &W2, 1, idx + 1, k - 1);
  if (q == i0) v += dXLin(c, &p, 1, &W2, 1, idx + 1, k - 1);
  v *= a2 * a2;
  if (p == q) v -= a2 * dXLin(c, &i0, 1, &U, 1, idx + 1, k - 1);
  return v;
}

/* D_{order,nder}(i,j,k,l,P,R): D_40..D_62 (integratorElastic3DHelper.cpp:2394-2554).
 * (i,j) strain indices, (k,l) eigenstrain indices, P the order moment indices,
 * R the nder collocation-derivative indices. */
static double D_tensor(const Ctx* c, double nu, int order, const int* P, int i, int j, int k,
                       int l, const int* R, int nder) {
  int p = order >= 1 ? P[0] : 0, q = order >= 2 ? P[1] : 0;
  int idx[12], n;
  double psi, t;
  n = 0;
  idx[n++] = k; idx[n++] = l; idx[n++] = i; idx[n++] = j;
  for (int s = 0; s < nder; ++s) idx[n++] = R[s];
  psi = d_psi(c, order, p, q, idx, n);
#define PHI2(a_, b_) (idx[0] = (a_), idx[1] = (b_), d_phi(c, order, p, q, idx, 2 + nder))
  for (int s = 0; s < nder; ++s) idx[2 + s] = R[s];
  t = psi;
  if (k == l) t -= 2 * nu * PHI2(i, j);
  double s4 = 0;
  if (i == l) s4 += PHI2(k, j);
  if (j == l) s4 += PHI2(k, i);
  if (i == k) s4 += PHI2(l, j);
  if (j == k) s4 += PHI2(l, i);
#undef PHI2
  t -= (1 - nu) * s4;
  return t / (8 * ORC_PI * (1 - nu));
}

/* IGreen_01/11/21 (:2604-2624): volume integral of the Kelvin derivative G_ij,l. */
static double IGreen(const Ctx* c, const Mat* M, int order, int i, int j, const int* P, int l) {
  int p = order >= 1 ? P[0] : 0, q = order >= 2 ? P[1] : 0;
  int idx[3];
  double v = 0;
  if (i == j) { idx[0] = l; v += 0.5 * d_phi(c, order, p, q, idx, 1); }
  if (i == l) { idx[0] = j; v += 0.5 * d_phi(c, order, p, q, idx, 1); }
  v /= (4 * ORC_PI * M->mu0);
  idx[0] = i; idx[1] = j; idx[2] = l;
  v -= d_psi(c, order, p, q, idx, 3) / (16 * ORC_PI * M->mu0 * (1 - M->nu0));
  return v;
}

/* ------------------------------------------------------------------------ */
/* Kelvin fundamental solution and its derivatives (:754-995, :2559-2593).
 * G_ij = d_ij/(4 pi mu0 R) - R_,ij / (16 pi mu0 (1-nu0)). */
static double dPow(const double* x, double r, double s, const int* idx, int k) {
  if (k == 0) return pow(r, s);
  int rest[16], r2[16];
  const int i0 = idx[0];
  memcpy(rest, idx + 1, sizeof(int) * (k - 1));
  double v = x[i0] * dPow(x, r, s - 2, rest, k - 1);
  for (int t = 0; t < k - 1; ++t)
    if (rest[t] == i0) {
      drop(rest, k - 1, t, r2);
      v += dPow(x, r, s - 2, r2, k - 2);
    }
  return s * v;
}

/* d/dx_K G_ij with K = idx[0..k-1]  (Green .. Green_04) */
static double dGreen(const double* x, const Mat* M, int i, int j, const int* K, int k) {
  double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  int idx[16];
  double v = 0;
  if (i == j) v += dPow(x, r, -1.0, K, k) / (4 * ORC_PI * M->mu0);
  idx[0] = i;
  idx[1] = j;
  memcpy(idx + 2, K, sizeof(int) * k);
  v -= dPow(x, r, 1.0, idx, k + 2) / (16 * ORC_PI * M->mu0 * (1 - M->nu0));
  return v;
}

/* ------------------------------------------------------------------------ */
/* Per-particle unknown layouts (configElastic3D.cpp:160-195 for 78).         */
typedef struct {
  int order, i, j, p, q;
  double mult; /* column multiplier (2 for compact p<q) */
} Unk;

static int layout_units(int layout, Unk* u) {
  int n = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j) { Unk t = {0, i, j, 0, 0, 1}; u[n++] = t; }
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j)
      for (int p = 0; p < 3; ++p) { Unk t = {1, i, j, p, 0, 1}; u[n++] = t; }
  if (layout == 24) return n;
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j)
      for (int p = 0; p < 3; ++p)
        for (int q = (layout == 60 ? p : 0); q < 3; ++q) {
          Unk t = {2, i, j, p, q, (layout == 60 && p != q) ? 2.0 : 1.0};
          u[n++] = t;
        }
  return n;
}

int orc_layout_size(int layout) {
  Unk u[78];
  if (layout != 24 && layout != 60 && layout != 78) return -1;
  return layout_units(layout, u);
}

/* ------------------------------------------------------------------------ */
/* Function-level values for pinning against the reference (ref_harness kat). */
int orc_D(int order, int nder, const double* x, double a, const orc_mat* m, double* out) {
  Mat M = mat_from(m);
  Ctx c;
  ctx_init(&c, x, a);
  int total = 4 + order + nder, n = 0;
  int lim = 1;
  for (int t = 0; t < total; ++t) lim *= 3;
  for (int f = 0; f < lim; ++f) {
    int dig[12], g = f;
    for (int t = total - 1; t >= 0; --t) { dig[t] = g % 3; g /= 3; }
    out[n++] = D_tensor(&c, M.nu0, order, dig + 4, dig[0], dig[1], dig[2], dig[3], dig + 4 + order, nder);
  }
  return n;
}

int orc_IGreen(int order, const double* x, double a, const orc_mat* m, double* out) {
  Mat M = mat_from(m);
  Ctx c;
  ctx_init(&c, x, a);
  int n = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int l = 0; l < 3; ++l) {
        if (order == 0) { out[n++] = IGreen(&c, &M, 0, i, j, NULL, l); continue; }
        for (int p = 0; p < 3; ++p) {
          if (order == 1) { int P[1] = {p}; out[n++] = IGreen(&c, &M, 1, i, j, P, l); continue; }
          for (int q = 0; q < 3; ++q) { int P[2] = {p, q}; out[n++] = IGreen(&c, &M, 2, i, j, P, l); }
        }
      }
  return n;
}

int orc_Green(int nder, const double* x, const orc_mat* m, double* out) {
  Mat M = mat_from(m);
  int total = 2 + nder, lim = 1, n = 0;
  for (int t = 0; t < total; ++t) lim *= 3;
  for (int f = 0; f < lim; ++f) {
    int dig[8], g = f;
    for (int t = total - 1; t >= 0; --t) { dig[t] = g % 3; g /= 3; }
    out[n++] = dGreen(x, &M, dig[0], dig[1], dig + 2, nder);
  }
  return n;
}

/* ------------------------------------------------------------------------ */
/* Inclusion <-> inclusion blocks: integratorElastic3D.cpp:341-682.
 * Row (s, ro, ij, R), column (h, co, mn, P):
 *   fac(ro) * map[m][n] * mult * ( -sum_kl (C0-C1)_ijkl D_{co,ro}(k,l,m,n,P,R) )
 *   + [s==h] map[m][n] * C0_ijmn * delta(P,R)        (self term, :392-397,509-523,634-650)
 * fac = 1 for rows of order 0/1 and 0.5 for order 2 (:616,627,645).
 * Writes the (nu*num)^2 block at A[row0 + ..., col0 + ...] (column-major, lda). */
static void entry_block(const Ctx* c, const Mat* M, const Unk* U, int nu, int same, double* blk) {
  /* blk[r * nu + col] for one (s,h) pair */
  for (int rr = 0; rr < nu; ++rr) {
    const Unk* ru = &U[rr];
    int R[2] = {ru->p, ru->q};
    double fac = ru->order == 2 ? 0.5 : 1.0;
    for (int cc = 0; cc < nu; ++cc) {
      const Unk* cu = &U[cc];
      int P[2] = {cu->p, cu->q};
      double acc = 0;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) {
          double dc = C0(M, ru->i, ru->j, k, l) - C1(M, ru->i, ru->j, k, l);
          if (dc == 0) continue;
          acc -= fac * dc * D_tensor(c, M->nu0, cu->order, P, k, l, cu->i, cu->j, R, ru->order);
        }
      acc *= cu->mult;
      if (same && ru->order == cu->order) {
        int match = 1;
        if (ru->order >= 1 && ru->p != cu->p) match = 0;
        if (ru->order == 2 && ru->q != cu->q) match = 0;
        if (match) acc += C0(M, ru->i, ru->j, cu->i, cu->j);
      }
      blk[rr * nu + cc] = MAPF[cu->i][cu->j] * acc;
    }
  }
}

int orc_pair_blocks(int num, const double* centers, const double* radius, const orc_mat* m,
                    int layout, double* A, int64_t lda, int64_t row0, int64_t col0) {
  Unk U[78];
  int nu = orc_layout_size(layout);
  if (nu < 0) return -1;
  layout_units(layout, U);
  Mat M = mat_from(m);
#pragma omp parallel for schedule(dynamic, 1)
  for (int s = 0; s < num; ++s) {
    double* blk = (double*)malloc(sizeof(double) * nu * nu);
    for (int h = 0; h < num; ++h) {
      double x[3] = {centers[3 * s] - centers[3 * h], centers[3 * s + 1] - centers[3 * h + 1],
                     centers[3 * s + 2] - centers[3 * h + 2]};
      Ctx c;
      ctx_init(&c, x, radius[h]);
      entry_block(&c, &M, U, nu, s == h, blk);
      for (int rr = 0; rr < nu; ++rr)
        for (int cc = 0; cc < nu; ++cc)
          A[(col0 + (int64_t)nu * h + cc) * lda + row0 + (int64_t)nu * s + rr] = blk[rr * nu + cc];
    }
    free(blk);
  }
  return 0;
}

/* Inclusion -> boundary node rows: get_addu/1/2 + addFieldToBEM
 * (integratorElastic3D.cpp:30-133, 135-340):
 *   HMAT(3j+q, col0 + nu*K + c) = + map[m][n] * mult * sum_{jj,ll} C0(jj,ll,m,n) IGreen(x_j - x_K)  */
int orc_node_blocks(int NN, const double* nodes, int num, const double* centers,
                    const double* radius, const orc_mat* m, int layout, double* H, int64_t ldh,
                    int64_t row0, int64_t col0) {
  Unk U[78];
  int nu = orc_layout_size(layout);
  if (nu < 0) return -1;
  layout_units(layout, U);
  Mat M = mat_from(m);
#pragma omp parallel for schedule(dynamic, 1)
  for (int K = 0; K < num; ++K)
    for (int j = 0; j < NN; ++j) {
      double x[3] = {nodes[3 * j] - centers[3 * K], nodes[3 * j + 1] - centers[3 * K + 1],
                     nodes[3 * j + 2] - centers[3 * K + 2]};
      Ctx c;
      ctx_init(&c, x, radius[K]);
      for (int cc = 0; cc < nu; ++cc) {
        const Unk* cu = &U[cc];
        int P[2] = {cu->p, cu->q};
        for (int q = 0; q < 3; ++q) {
          double dd = 0;
          for (int jj = 0; jj < 3; ++jj)
            for (int ll = 0; ll < 3; ++ll) {
              double cv = C0(&M, jj, ll, cu->i, cu->j);
              if (cv != 0) dd -= MAPF[cu->i][cu->j] * cv * IGreen(&c, &M, cu->order, q, jj, P, ll);
            }
          H[(col0 + (int64_t)nu * K + cc) * ldh + row0 + 3 * j + q] = -dd * cu->mult;
        }
      }
    }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Q4 boundary elements: BEMElasticHelper3D.cpp:29-321 and Integ3/addBEM
 * (BEMBuilderElastic3D.cpp:1169-1509).  8-point Gauss-Legendre rule (:1204-1222). */
static const double GP8[8] = {0.960289856497536,  -0.960289856497536, 0.796666477413627,
                              -0.796666477413627, 0.525532409916329,  -0.525532409916329,
                              0.183434642495650,  -0.183434642495650};
static const double GW8[8] = {0.101228536290376, 0.101228536290376, 0.222381034453374,
                              0.222381034453374, 0.313706645877887, 0.313706645877887,
                              0.362683783378362, 0.362683783378362};

static void q4_shape(double xi, double et, double* N) { /* Serendip_func :199-224 */
  N[0] = 0.25 * (1 - xi) * (1 - et);
  N[1] = 0.25 * (1 + xi) * (1 - et);
  N[2] = 0.25 * (1 + xi) * (1 + et);
  N[3] = 0.25 * (1 - xi) * (1 + et);
}

static void q4_normal_jac(double xi, double et, const double* el, double* jac, double* nv) {
  /* Normal_Jac :226-267 ; el = 4 x 3 row-major corner coordinates */
  double dxi[4] = {-0.25 * (1 - et), 0.25 * (1 - et), 0.25 * (1 + et), -0.25 * (1 + et)};
  double det[4] = {-0.25 * (1 - xi), -0.25 * (1 + xi), 0.25 * (1 + xi), 0.25 * (1 - xi)};
  double vx[3], ve[3];
  for (int i = 0; i < 3; ++i) {
    vx[i] = dxi[0] * el[i] + dxi[1] * el[3 + i] + dxi[2] * el[6 + i] + dxi[3] * el[9 + i];
    ve[i] = det[0] * el[i] + det[1] * el[3 + i] + det[2] * el[6 + i] + det[3] * el[9 + i];
  }
  nv[0] = vx[1] * ve[2] - ve[1] * vx[2];
  nv[1] = vx[2] * ve[0] - vx[0] * ve[2];
  nv[2] = vx[0] * ve[1] - vx[1] * ve[0];
  *jac = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
  nv[0] /= *jac;
  nv[1] /= *jac;
  nv[2] /= *jac;
}

/* Trans_Tri + Triangle_Coord (:29-191): degenerate map of a Gauss point of the
 * unit square onto one of the two triangles that split the element at corner l_pi. */
static void tri_map(int ntr, int l_pi, double xb, double eb, double* xi, double* et, double* jb) {
  static const int tab[2][4][3] = {{{1, 2, 0}, {2, 3, 1}, {0, 1, 2}, {0, 1, 3}},
                                   {{2, 3, 0}, {3, 0, 1}, {3, 0, 2}, {1, 2, 3}}};
  static const int xsii[8] = {-1, 1, 1, -1, 0, 1, 0, -1};
  static const int etai[8] = {-1, -1, 1, 1, -1, 0, 1, 0};
  double cx[3], ce[3];
  for (int n = 0; n < 3; ++n) {
    cx[n] = xsii[tab[ntr][l_pi][n]];
    ce[n] = etai[tab[ntr][l_pi][n]];
  }
  double Nb[3] = {0.25 * (1 + xb) * (1 - eb), 0.25 * (1 + xb) * (1 + eb), 0.5 * (1 - xb)};
  double dNx[3] = {0.25 * (1 - eb), 0.25 * (1 + eb), -0.5};
  double dNe[3] = {-0.25 * (1 + xb), 0.25 * (1 + xb), 0};
  *xi = 0;
  *et = 0;
  for (int n = 0; n < 3; ++n) {
    *xi += Nb[n] * cx[n];
    *et += Nb[n] * ce[n];
  }
  double J00 = 0, J01 = 0, J10 = 0, J11 = 0;
  for (int n = 0; n < 3; ++n) {
    J00 += dNx[n] * cx[n];
    J01 += dNx[n] * ce[n];
    J10 += dNe[n] * cx[n];
    J11 += dNe[n] * ce[n];
  }
  *jb = J00 * J11 - J01 * J10;
}

static void kelvin_UT(const double* dxr, double r, const Mat* M, const double* nv, double U[3][3],
                      double T[3][3]) {
  /* UK / TK (BEMElasticHelper3D.cpp:269-321) */
  double G = M->mu0, nu = M->nu0;
  double c = 1 / (16 * ORC_PI * G * (1 - nu)), conr = c / r, c1 = 3 - 4 * nu;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) U[i][j] = conr * ((i == j ? c1 : 0) + dxr[i] * dxr[j]);
  double c3 = 1 - 2 * nu, c2 = 1 / (8 * ORC_PI * (1 - nu));
  double cth = nv[0] * dxr[0] + nv[1] * dxr[1] + nv[2] * dxr[2], cr = c2 / (r * r);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      if (i == j)
        T[i][j] = -cr * (c3 + 3 * dxr[i] * dxr[i]) * cth;
      else
        T[i][j] = -cr * (3 * dxr[i] * dxr[j] * cth - c3 * (nv[j] * dxr[i] - nv[i] * dxr[j]));
    }
}

/* Classical BEM H and G (addBEM :1355-1509): G is 3NN x 12NE written into
 * G[(gcol0 + 12e + k) * ldg + grow0 + row]; H is 3NN x 3NN at H[(hcol0 + c) * ldh + hrow0 + r].
 * conn is NE x 4, 1-based node numbers (as in BEM.txt). */
int orc_bem_hg(int NN, const double* nodes, int NE, const int* conn, const orc_mat* m, double* H,
               int64_t ldh, int64_t hrow0, int64_t hcol0, double* G, int64_t ldg, int64_t grow0,
               int64_t gcol0) {
  Mat M = mat_from(m);
  int n3 = 3 * NN;
  for (int c = 0; c < n3; ++c)
    for (int r = 0; r < n3; ++r) H[(hcol0 + c) * ldh + hrow0 + r] = 0;
  /* element-wise accumulation; the per-element dTe scatter into node columns */
  double* dT = (double*)malloc(sizeof(double) * (size_t)n3 * 12 * NE);
#pragma omp parallel for schedule(dynamic, 4)
  for (int e = 0; e < NE; ++e) {
    double el[12];
    int sc[4];
    for (int j = 0; j < 4; ++j) {
      sc[j] = conn[4 * e + j];
      for (int k = 0; k < 3; ++k) el[3 * j + k] = nodes[3 * (sc[j] - 1) + k];
    }
    double* dTe = dT + (size_t)e * n3 * 12;
    for (int i = 0; i < NN; ++i) {
      double dU[3][12], dTl[3][12];
      memset(dU, 0, sizeof dU);
      memset(dTl, 0, sizeof dTl);
      int l_pi = -1;
      for (int n = 0; n < 4; ++n)
        if (sc[n] == i + 1) l_pi = n;
      const double* xP = nodes + 3 * i;
      int ntri = (l_pi < 0) ? 1 : 2;
      for (int ntr = 0; ntr < ntri; ++ntr)
        for (int mq = 0; mq < 8; ++mq)
          for (int kq = 0; kq < 8; ++kq) {
            double W = GW8[mq] * GW8[kq], xi, et, jb = 1, N[4], jac, nv[3], gc[3];
            if (l_pi < 0) {
              xi = GP8[mq];
              et = GP8[kq];
            } else {
              tri_map(ntr, l_pi, GP8[mq], GP8[kq], &xi, &et, &jb);
            }
            q4_shape(xi, et, N);
            q4_normal_jac(xi, et, el, &jac, nv);
            jac *= jb;
            for (int d = 0; d < 3; ++d)
              gc[d] = N[0] * el[d] + N[1] * el[3 + d] + N[2] * el[6 + d] + N[3] * el[9 + d];
            double dx[3] = {gc[0] - xP[0], gc[1] - xP[1], gc[2] - xP[2]};
            double r = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
            double dxr[3] = {dx[0] / r, dx[1] / r, dx[2] / r};
            double U[3][3], T[3][3];
            kelvin_UT(dxr, r, &M, nv, U, T);
            for (int ii = 0; ii < 3; ++ii)
              for (int jj = 0; jj < 3; ++jj)
                for (int n = 0; n < 4; ++n) {
                  dU[ii][3 * n + jj] += N[n] * U[ii][jj] * jac * W;
                  if (l_pi < 0 || sc[n] != i + 1) dTl[ii][3 * n + jj] += N[n] * T[ii][jj] * jac * W;
                }
          }
      for (int ii = 0; ii < 3; ++ii)
        for (int k = 0; k < 12; ++k) {
          G[(gcol0 + 12 * e + k) * ldg + grow0 + 3 * i + ii] = dU[ii][k];
          dTe[(size_t)(3 * i + ii) * 12 + k] = dTl[ii][k];
        }
    }
  }
  /* scatter in element order (the reference accumulates under omp critical) */
  for (int e = 0; e < NE; ++e)
    for (int j = 0; j < 4; ++j) {
      int p = 3 * (conn[4 * e + j] - 1);
      for (int k = 0; k < 3; ++k)
        for (int r = 0; r < n3; ++r)
          H[(hcol0 + p + k) * ldh + hrow0 + r] += dT[((size_t)e * n3 + r) * 12 + 3 * j + k];
    }
  free(dT);
  /* rigid-body diagonal (:1478-1501) */
  for (int i = 0; i < NN; ++i)
    for (int r = 3 * i; r < 3 * i + 3; ++r) {
      double s[3] = {0, 0, 0};
      for (int c = 0; c < n3; ++c) s[c % 3] += H[(hcol0 + c) * ldh + hrow0 + r];
      for (int l = 0; l < 3; ++l) H[(hcol0 + 3 * i + l) * ldh + hrow0 + r] = -s[l];
    }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Stress (or its nder-th gradient) at a point from unit boundary displacement and
 * traction at a Gauss point: get_for_stress_BEM / 1 / 2 (BEMBuilderElastic3D.cpp:
 * 780-980, 429-672, 37-322) with the contrast (dlam, dmu); the post-processing
 * variant (postProcessorElastic3D.cpp:32-114) is dlam = lam0, dmu = mu0, nder = 0.
 * Rows t = (k<=l) x W (W the nder derivative indices, last fastest); Dsu/Dst [t][n]. */
/* All derivatives of 1/R (orders 0..kmax_i) and R (orders 0..kmax_r) at x, stored as
 * full 3^k tensors (index digits, first index slowest). */
typedef struct {
  double* inv[7];
  double* len[9];
  double buf[3 * 2187 + 3 * 729];
} GCache;

static void gcache_fill(GCache* g, const double* x, int kmax_i, int kmax_r) {
  double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  double* p = g->buf;
  int idx[12];
  for (int k = 0; k <= kmax_i; ++k) {
    int lim = 1;
    for (int t = 0; t < k; ++t) lim *= 3;
    g->inv[k] = p;
    for (int f = 0; f < lim; ++f) {
      int q = f;
      for (int t = k - 1; t >= 0; --t) { idx[t] = q % 3; q /= 3; }
      p[f] = dPow(x, r, -1.0, idx, k);
    }
    p += lim;
  }
  for (int k = 0; k <= kmax_r; ++k) {
    int lim = 1;
    for (int t = 0; t < k; ++t) lim *= 3;
    g->len[k] = p;
    for (int f = 0; f < lim; ++f) {
      int q = f;
      for (int t = k - 1; t >= 0; --t) { idx[t] = q % 3; q /= 3; }
      p[f] = dPow(x, r, 1.0, idx, k);
    }
    p += lim;
  }
}

static inline int flat(const int* idx, int k) {
  int f = 0;
  for (int t = 0; t < k; ++t) f = 3 * f + idx[t];
  return f;
}

/* d_K G_ij from the cache (same formula as dGreen) */
static double dGreenC(const GCache* g, const Mat* M, int i, int j, const int* K, int k) {
  int idx[12];
  double v = 0;
  if (i == j) v += g->inv[k][flat(K, k)] / (4 * ORC_PI * M->mu0);
  idx[0] = i;
  idx[1] = j;
  memcpy(idx + 2, K, sizeof(int) * k);
  v -= g->len[k + 2][flat(idx, k + 2)] / (16 * ORC_PI * M->mu0 * (1 - M->nu0));
  return v;
}

static void stress_kernel(const double* x, const Mat* M, double dlam, double dmu, int nder,
                          const double* nv, double* Dsu, double* Dst) {
  GCache gc;
  gcache_fill(&gc, x, 2 + nder, 4 + nder);
#define dGreen(x_, M_, i_, j_, K_, k_) dGreenC(&gc, M_, i_, j_, K_, k_)

  int nW = nder == 0 ? 1 : (nder == 1 ? 3 : 9);
  double su = (nder % 2 == 0) ? 1.0 : -1.0; /* Dsu sign */
  double st = -su;                          /* Dst sign */
  int t = 0;
  for (int k = 0; k < 3; ++k)
    for (int l = k; l < 3; ++l)
      for (int w = 0; w < nW; ++w) {
        int W[2] = {nder == 2 ? w / 3 : w, w % 3};
        for (int n = 0; n < 3; ++n) {
          int K[4];
          /* TG1[n][W] = sum_i d_{i W} G_{n i} */
          double tg1 = 0;
          for (int i = 0; i < 3; ++i) {
            K[0] = i; K[1] = W[0]; K[2] = W[1];
            tg1 += dGreen(x, M, n, i, K, 1 + nder);
          }
          double dst = dlam * dl(k, l) * tg1;
          K[0] = l; K[1] = W[0]; K[2] = W[1];
          dst += dmu * dGreen(x, M, n, k, K, 1 + nder);
          K[0] = k;
          dst += dmu * dGreen(x, M, n, l, K, 1 + nder);
          Dst[t * 3 + n] = st * dst;
          double dsu = 0;
          for (int mm = 0; mm < 3; ++mm) {
            /* sgm[m][n][W] = sum_i lam0 d_mn TG[i][i][W] + mu0 (G_mi,niW + G_ni,miW) */
            double sg = 0;
            for (int i = 0; i < 3; ++i) {
              if (mm == n)
                for (int ll = 0; ll < 3; ++ll) {
                  int K3[4] = {ll, i, W[0], W[1]};
                  sg += M->lam0 * dGreen(x, M, ll, i, K3, 2 + nder);
                }
              int Ka[4] = {n, i, W[0], W[1]}, Kb[4] = {mm, i, W[0], W[1]};
              sg += M->mu0 * dGreen(x, M, mm, i, Ka, 2 + nder) + M->mu0 * dGreen(x, M, n, i, Kb, 2 + nder);
            }
            double tgkl = 0, tglk = 0;
            if (mm == n)
              for (int ll = 0; ll < 3; ++ll) {
                int Ka[4] = {ll, l, W[0], W[1]}, Kb[4] = {ll, k, W[0], W[1]};
                tgkl += dGreen(x, M, ll, k, Ka, 2 + nder);
                tglk += dGreen(x, M, ll, l, Kb, 2 + nder);
              }
            int K1[4] = {n, l, W[0], W[1]}, K2[4] = {n, k, W[0], W[1]};
            int K3[4] = {mm, l, W[0], W[1]}, K4[4] = {mm, k, W[0], W[1]};
            double g4 = M->mu0 * (dGreen(x, M, mm, k, K1, 2 + nder) + dGreen(x, M, mm, l, K2, 2 + nder) +
                                  dGreen(x, M, n, k, K3, 2 + nder) + dGreen(x, M, n, l, K4, 2 + nder));
            dsu += (dlam * dl(k, l) * sg + dmu * (M->lam0 * dl(mm, n) * (tgkl + tglk) + g4)) * nv[mm];
          }
          Dsu[t * 3 + n] = su * dsu;
        }
        ++t;
      }
#undef dGreen
}

/* Integ3_stress{,1,2} (:982-1167, 674-778, 324-427): regular 8x8 quadrature over one
 * element of the stress kernel at `point`; DDsu/DDst [row][12] accumulated. */
static void integ_stress(const double* el, const double* point, const Mat* M, double dlam,
                         double dmu, int nder, double* DDsu, double* DDst) {
  int nrow = 6 * (nder == 0 ? 1 : (nder == 1 ? 3 : 9));
  double* Dsu = (double*)malloc(sizeof(double) * nrow * 3 * 2);
  double* Dst = Dsu + nrow * 3;
  for (int mq = 0; mq < 8; ++mq)
    for (int kq = 0; kq < 8; ++kq) {
      double xi = GP8[mq], et = GP8[kq], W = GW8[mq] * GW8[kq], N[4], jac, nv[3], gc[3];
      q4_shape(xi, et, N);
      q4_normal_jac(xi, et, el, &jac, nv);
      for (int d = 0; d < 3; ++d)
        gc[d] = N[0] * el[d] + N[1] * el[3 + d] + N[2] * el[6 + d] + N[3] * el[9 + d];
      double x[3] = {gc[0] - point[0], gc[1] - point[1], gc[2] - point[2]};
      stress_kernel(x, M, dlam, dmu, nder, nv, Dsu, Dst);
      for (int r = 0; r < nrow; ++r)
        for (int a = 0; a < 4; ++a)
          for (int n = 0; n < 3; ++n) {
            DDsu[r * 12 + 3 * a + n] += Dsu[r * 3 + n] * N[a] * W * jac;
            DDst[r * 12 + 3 * a + n] += Dst[r * 3 + n] * N[a] * W * jac;
          }
    }
  free(Dsu);
}

/* Boundary -> inclusion rows: addFluxEquivalent{,FirstOrder,SecondOrder}BEM
 * (:1511-1867).  For every particle K and element e:
 *   H(row0 + nu*K + r, hcol0 + node dofs) -= fac * DDsu   (scatter-add)
 *   G(row0 + nu*K + r, gcol0 + 12e + k)    = fac * DDst
 * fac = 0.5 for order-2 rows.  Row r follows the layout (order-2 compact rows keep w<=z). */
int orc_bem_to_incl(int NN, const double* nodes, int NE, const int* conn, int num,
                    const double* centers, const orc_mat* m, int layout, double* H, int64_t ldh,
                    int64_t hcol0, double* G, int64_t ldg, int64_t gcol0, int64_t row0) {
  Unk U[78];
  int nu = orc_layout_size(layout);
  if (nu < 0) return -1;
  layout_units(layout, U);
  Mat M = mat_from(m);
  double dlam = M.lam0 - M.lam1, dmu = M.mu0 - M.mu1;
  /* map each layout row to (order, row within the Integ3_stress order block) */
  int rord[78], ridx[78];
  for (int r = 0; r < nu; ++r) {
    int pr = 0; /* (i<=j) pair index */
    for (int i = 0; i < 3; ++i)
      for (int j = i; j < 3; ++j, ++pr)
        if (i == U[r].i && j == U[r].j) goto found;
  found:
    rord[r] = U[r].order;
    ridx[r] = U[r].order == 0 ? pr : (U[r].order == 1 ? pr * 3 + U[r].p : pr * 9 + 3 * U[r].p + U[r].q);
  }
  int maxo = layout == 24 ? 1 : 2;
#pragma omp parallel for schedule(dynamic, 1)
  for (int K = 0; K < num; ++K) {
    double* DD[3][2];
    for (int o = 0; o <= maxo; ++o) {
      int nrow = 6 * (o == 0 ? 1 : (o == 1 ? 3 : 9));
      DD[o][0] = (double*)malloc(sizeof(double) * nrow * 12);
      DD[o][1] = (double*)malloc(sizeof(double) * nrow * 12);
    }
    for (int e = 0; e < NE; ++e) {
      double el[12];
      for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 3; ++k) el[3 * j + k] = nodes[3 * (conn[4 * e + j] - 1) + k];
      for (int o = 0; o <= maxo; ++o) {
        int nrow = 6 * (o == 0 ? 1 : (o == 1 ? 3 : 9));
        memset(DD[o][0], 0, sizeof(double) * nrow * 12);
        memset(DD[o][1], 0, sizeof(double) * nrow * 12);
        integ_stress(el, centers + 3 * K, &M, dlam, dmu, o, DD[o][0], DD[o][1]);
      }
      for (int r = 0; r < nu; ++r) {
        double fac = rord[r] == 2 ? 0.5 : 1.0;
        const double* su = DD[rord[r]][0] + ridx[r] * 12;
        const double* st = DD[rord[r]][1] + ridx[r] * 12;
        int64_t row = row0 + (int64_t)nu * K + r;
        for (int j = 0; j < 4; ++j) {
          int p = 3 * (conn[4 * e + j] - 1);
          for (int k = 0; k < 3; ++k) H[(hcol0 + p + k) * ldh + row] -= fac * su[3 * j + k];
        }
        for (int k = 0; k < 12; ++k) G[(gcol0 + 12 * e + k) * ldg + row] = fac * st[k];
      }
    }
    for (int o = 0; o <= maxo; ++o) {
      free(DD[o][0]);
      free(DD[o][1]);
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* ApplyBC (BEMBuilderElastic3D.cpp:1920-2051).  Traction unknowns are shared per
 * (node, dof) in first-seen order over (e, i); the reference keys them by the double
 * node + 0.1*(dof+1) (:1999-2000), this uses the integer pair.  tcol[12*NE] receives
 * the column of every traction value that is unknown (-1 when prescribed).
 * H is N x N (first 3NN columns boundary, rest inclusion), G is N x 12NE.
 * Returns the number of boundary unknown columns (must equal 3NN). */
int orc_apply_bc(int NN, int NE, const int* conn, const double* bc /* 3NN x 2 row-major */,
                 const double* tbc /* NE x 24 row-major */, int64_t N, const double* H,
                 int64_t ldh, const double* G, int64_t ldg, double* A, int64_t lda, double* b,
                 int* tcol) {
  int n3 = 3 * NN, t = 0;
  int* key = (int*)malloc(sizeof(int) * (size_t)n3);
  for (int i = 0; i < n3; ++i) key[i] = -1;
  for (int64_t i = 0; i < N; ++i) b[i] = 0;
  for (int j = 0; j < n3; ++j)
    if (bc[2 * j] == 1) {
      for (int64_t i = 0; i < N; ++i) A[(int64_t)t * lda + i] = H[(int64_t)j * ldh + i];
      ++t;
    }
  for (int j = 0; j < n3; ++j)
    if (bc[2 * j] == 0)
      for (int64_t i = 0; i < N; ++i) b[i] -= H[(int64_t)j * ldh + i] * bc[2 * j + 1];
  for (int e = 0; e < NE; ++e)
    for (int i = 0; i < 12; ++i) {
      int64_t gc = (int64_t)(12 * e + i) * ldg;
      tcol[12 * e + i] = -1;
      if (tbc[24 * e + i] == 1) {
        for (int64_t r = 0; r < N; ++r) b[r] += tbc[24 * e + 12 + i] * G[gc + r];
      } else if (tbc[24 * e + i] == 0) {
        int kk = 3 * (conn[4 * e + i / 3] - 1) + i % 3;
        if (key[kk] < 0) {
          key[kk] = t;
          for (int64_t r = 0; r < N; ++r) A[(int64_t)t * lda + r] = -G[gc + r];
          ++t;
        } else {
          int cc = key[kk];
          for (int64_t r = 0; r < N; ++r) A[(int64_t)cc * lda + r] -= G[gc + r];
        }
        tcol[12 * e + i] = key[kk];
      }
    }
  for (int64_t j = n3; j < N; ++j)
    for (int64_t i = 0; i < N; ++i) A[j * lda + i] = H[j * ldh + i];
  free(key);
  return t;
}

/* getUTVector (:2053-2117) */
void orc_get_ut(int NN, int NE, int64_t N, const double* bc, const double* tbc, const int* tcol,
                const double* X, double* Uv, double* Tv) {
  int t = 0, m = 0;
  for (int i = 0; i < 3 * NN; ++i) Uv[i] = (bc[2 * i] == 0) ? bc[2 * i + 1] : X[t++];
  for (int64_t i = 3 * NN; i < N; ++i) Uv[i] = X[i];
  for (int e = 0; e < NE; ++e)
    for (int i = 0; i < 12; ++i) {
      if (tbc[24 * e + i] == 1) Tv[m++] = tbc[24 * e + 12 + i];
      else if (tbc[24 * e + i] == 0) Tv[m++] = X[tcol[12 * e + i]];
    }
}

/* ------------------------------------------------------------------------ */
/* Dense solve, full pivoting: the algorithm of Eigen's FullPivLU used by
 * systemSolverElastic3D.h:55 (largest |a_ij| of the trailing block as pivot, row and
 * column exchanges, unit-lower L).  A (N x N, column-major) is overwritten. */
int orc_solve_fullpiv(int64_t N, double* A, int64_t lda, const double* b, double* x) {
  int64_t* rp = (int64_t*)malloc(sizeof(int64_t) * N);
  int64_t* cp = (int64_t*)malloc(sizeof(int64_t) * N);
  double* y = (double*)malloc(sizeof(double) * N);
  for (int64_t k = 0; k < N; ++k) { rp[k] = k; cp[k] = k; }
  for (int64_t k = 0; k < N; ++k) {
    double best = -1;
    int64_t bi = k, bj = k;
#pragma omp parallel
    {
      double lb = -1;
      int64_t li = k, lj = k;
#pragma omp for nowait
      for (int64_t j = k; j < N; ++j)
        for (int64_t i = k; i < N; ++i) {
          double v = fabs(A[j * lda + i]);
          if (v > lb) { lb = v; li = i; lj = j; }
        }
#pragma omp critical
      if (lb > best || (lb == best && (lj < bj || (lj == bj && li < bi)))) { best = lb; bi = li; bj = lj; }
    }
    if (best == 0) { free(rp); free(cp); free(y); return 1; }
    if (bi != k) {
      for (int64_t j = 0; j < N; ++j) { double t = A[j * lda + k]; A[j * lda + k] = A[j * lda + bi]; A[j * lda + bi] = t; }
      int64_t t = rp[k]; rp[k] = rp[bi]; rp[bi] = t;
    }
    if (bj != k) {
      for (int64_t i = 0; i < N; ++i) { double t = A[k * lda + i]; A[k * lda + i] = A[bj * lda + i]; A[bj * lda + i] = t; }
      int64_t t = cp[k]; cp[k] = cp[bj]; cp[bj] = t;
    }
    double piv = A[k * lda + k];
    for (int64_t i = k + 1; i < N; ++i) A[k * lda + i] /= piv;
#pragma omp parallel for schedule(static)
    for (int64_t j = k + 1; j < N; ++j) {
      double u = A[j * lda + k];
      if (u == 0) continue;
      double* cj = A + j * lda;
      const double* ck = A + k * lda;
      for (int64_t i = k + 1; i < N; ++i) cj[i] -= ck[i] * u;
    }
  }
  for (int64_t i = 0; i < N; ++i) y[i] = b[rp[i]];
  for (int64_t k = 0; k < N; ++k)
    for (int64_t i = k + 1; i < N; ++i) y[i] -= A[k * lda + i] * y[k];
  for (int64_t k = N - 1; k >= 0; --k) {
    y[k] /= A[k * lda + k];
    for (int64_t i = 0; i < k; ++i) y[i] -= A[k * lda + i] * y[k];
  }
  for (int64_t i = 0; i < N; ++i) x[cp[i]] = y[i];
  free(rp); free(cp); free(y);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Post-processing: post_stress_BEM + postprocessor (postProcessorElastic3D.cpp:224-522).
 *   boundary part  s_pb = GSTe U + GSUe T   (skipped when NE == 0)
 *   particle part  e_p  = sum_h D_{order,0}(x_p - x_h) map mult E  - local eigenstrain
 *                  s_p  = C0 : e_p
 * With NE == 0 the far field sigma_inf (6: xx xy xz yy yz zz) replaces s_pb.
 * E holds nu*num eigenstrain coefficients; Ub (3NN) and Tb (12NE) the boundary values.
 * Output stress[nump][6] in the order xx xy xz yy yz zz (getFlux :578-585). */
int orc_post(int nump, const double* pts, int num, const double* centers, const double* radius,
             const orc_mat* m, int layout, const double* E, int NN, const double* nodes, int NE,
             const int* conn, const double* Ub, const double* Tb, const double* sig_inf,
             double* stress) {
  Unk U[78];
  int nu = orc_layout_size(layout);
  if (nu < 0) return -1;
  layout_units(layout, U);
  Mat M = mat_from(m);
  static const int PI_[6] = {0, 0, 0, 1, 1, 2}, PJ_[6] = {0, 1, 2, 1, 2, 2};
#pragma omp parallel for schedule(dynamic, 1)
  for (int s = 0; s < nump; ++s) {
    const double* xp = pts + 3 * s;
    double spb[6] = {0, 0, 0, 0, 0, 0};
    if (NE > 0) {
      double DDsu[72], DDst[72];
      for (int e = 0; e < NE; ++e) {
        double el[12];
        for (int j = 0; j < 4; ++j)
          for (int k = 0; k < 3; ++k) el[3 * j + k] = nodes[3 * (conn[4 * e + j] - 1) + k];
        memset(DDsu, 0, sizeof DDsu);
        memset(DDst, 0, sizeof DDst);
        integ_stress(el, xp, &M, M.lam0, M.mu0, 0, DDsu, DDst);
        for (int r = 0; r < 6; ++r) {
          for (int j = 0; j < 4; ++j) {
            int p = 3 * (conn[4 * e + j] - 1);
            for (int k = 0; k < 3; ++k) spb[r] += DDsu[r * 12 + 3 * j + k] * Ub[p + k];
          }
          for (int k = 0; k < 12; ++k) spb[r] += DDst[r * 12 + k] * Tb[12 * e + k];
        }
      }
    } else if (sig_inf) {
      for (int r = 0; r < 6; ++r) spb[r] = sig_inf[r];
    }
    /* inside test: the last particle containing the point wins (:383-390) */
    int in = -1;
    for (int h = 0; h < num; ++h) {
      double dx = xp[0] - centers[3 * h], dy = xp[1] - centers[3 * h + 1], dz = xp[2] - centers[3 * h + 2];
      if (dx * dx + dy * dy + dz * dz - radius[h] * radius[h] <= 0) in = h;
    }
    double ep[6] = {0, 0, 0, 0, 0, 0};
    for (int h = 0; h < num; ++h) {
      double x[3] = {xp[0] - centers[3 * h], xp[1] - centers[3 * h + 1], xp[2] - centers[3 * h + 2]};
      Ctx c;
      ctx_init(&c, x, radius[h]);
      for (int r = 0; r < 6; ++r)
        for (int cc = 0; cc < nu; ++cc) {
          const Unk* cu = &U[cc];
          int P[2] = {cu->p, cu->q};
          ep[r] += D_tensor(&c, M.nu0, cu->order, P, PI_[r], PJ_[r], cu->i, cu->j, NULL, 0) *
                   MAPF[cu->i][cu->j] * cu->mult * E[(int64_t)nu * h + cc];
        }
    }
    if (in >= 0) {
      double x[3] = {xp[0] - centers[3 * in], xp[1] - centers[3 * in + 1], xp[2] - centers[3 * in + 2]};
      for (int cc = 0; cc < nu; ++cc) {
        const Unk* cu = &U[cc];
        int r = 0;
        for (int i = 0; i < 3; ++i)
          for (int j = i; j < 3; ++j, ++r)
            if (i == cu->i && j == cu->j) goto got;
      got:;
        double v = E[(int64_t)nu * in + cc];
        if (cu->order == 1) v *= x[cu->p];
        if (cu->order == 2) {
          /* reference: sum_{k<=l} map[k][l] E_ijkl x_k x_l (:424-432) */
          if (layout == 78 && cu->p > cu->q) continue;
          v *= MAPF[cu->p][cu->q] * x[cu->p] * x[cu->q];
        }
        ep[r] -= v;
      }
    }
    for (int r = 0; r < 6; ++r) {
      double sp = 0;
      for (int q = 0; q < 6; ++q) sp += C0(&M, PI_[r], PJ_[r], PI_[q], PJ_[q]) * MAPF[PI_[q]][PJ_[q]] * ep[q];
      stress[6 * s + r] = sp + spb[r];
    }
  }
  return 0;
}

/* Far-field right-hand side (no reference counterpart: the reference loads only through
 * the boundary).  Uniform applied strain eps = C0^-1 : sigma_inf enters the equivalence
 * rows of order 0 as (C0 - C1) : eps; rows of order >= 1 get 0 (a uniform field has no
 * gradient). b has nu*num entries. */
int orc_farfield_rhs(int num, const orc_mat* m, int layout, const double* sig_inf, double* b) {
  Unk U[78];
  int nu = orc_layout_size(layout);
  if (nu < 0) return -1;
  layout_units(layout, U);
  Mat M = mat_from(m);
  /* isotropic compliance: eps = (1+nu)/E sigma - nu/E tr(sigma) I */
  double S[3][3] = {{sig_inf[0], sig_inf[1], sig_inf[2]},
                    {sig_inf[1], sig_inf[3], sig_inf[4]},
                    {sig_inf[2], sig_inf[4], sig_inf[5]}};
  double tr = S[0][0] + S[1][1] + S[2][2];
  double eps[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) eps[i][j] = ((1 + m->nu0) * S[i][j] - m->nu0 * tr * (i == j)) / m->E0;
  for (int h = 0; h < num; ++h)
    for (int r = 0; r < nu; ++r) {
      double v = 0;
      if (U[r].order == 0)
        for (int k = 0; k < 3; ++k)
          for (int l = 0; l < 3; ++l)
            v += (C0(&M, U[r].i, U[r].j, k, l) - C1(&M, U[r].i, U[r].j, k, l)) * eps[k][l];
      b[(int64_t)nu * h + r] = v;
    }
  return 0;
}

/* Stress kernel at one Gauss point (for checking the CUDA code function by function);
 * dlam/dmu = (C0 - C1) contrast, or (lam0, mu0) for the post-processing variant. */
int orc_stress_kernel(const double* x, const double* nv, const orc_mat* m, double dlam,
                      double dmu, int nder, double* Dsu, double* Dst) {
  Mat M = mat_from(m);
  stress_kernel(x, &M, dlam, dmu, nder, nv, Dsu, Dst);
  return 0;
}
