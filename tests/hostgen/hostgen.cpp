// Host build of the generated sphere code, for checking the generator against the
// oracle without a GPU (compiled by tests/test_codegen_host.py with the host compiler).
#include <string.h>
#include "gen_sphere24.cuh"
#include "gen_sphere60.cuh"
#include "gen_sphere60_f32.cuh"
#include "gen_sphere78.cuh"

namespace {
struct ArrSink {
  double* out;
  int nu;
  void operator()(int r, int c, double v) { out[r * nu + c] += v; }
};
}  // namespace

extern "C" int hg_pair_block(int layout, const double* x, double a, double E0, double nu0,
                             double E1, double nu1, int self, double* out) {
  SphMat mc = sph_mat_init(E0, nu0, E1, nu1);
  int nu = layout;
  memset(out, 0, sizeof(double) * nu * nu);
  ArrSink s{out, nu};
  if (layout == 24) {
    sph_block24_c0_r0(x[0], x[1], x[2], a, mc, s); sph_block24_c0_r1(x[0], x[1], x[2], a, mc, s);
    sph_block24_c1_r0(x[0], x[1], x[2], a, mc, s); sph_block24_c1_r1(x[0], x[1], x[2], a, mc, s);
    if (self) sph_self24(mc, s);
  } else if (layout == 78) {
    sph_block78_c0_r0(x[0], x[1], x[2], a, mc, s); sph_block78_c0_r1(x[0], x[1], x[2], a, mc, s);
    sph_block78_c0_r2(x[0], x[1], x[2], a, mc, s); sph_block78_c1_r0(x[0], x[1], x[2], a, mc, s);
    sph_block78_c1_r1(x[0], x[1], x[2], a, mc, s); sph_block78_c1_r2(x[0], x[1], x[2], a, mc, s);
    sph_block78_c2_r0(x[0], x[1], x[2], a, mc, s); sph_block78_c2_r1(x[0], x[1], x[2], a, mc, s);
    sph_block78_c2_r2(x[0], x[1], x[2], a, mc, s);
    if (self) sph_self78(mc, s);
  } else if (layout == 60) {
    sph_block60_c0_r0(x[0], x[1], x[2], a, mc, s); sph_block60_c0_r1(x[0], x[1], x[2], a, mc, s);
    sph_block60_c0_r2(x[0], x[1], x[2], a, mc, s); sph_block60_c1_r0(x[0], x[1], x[2], a, mc, s);
    sph_block60_c1_r1(x[0], x[1], x[2], a, mc, s); sph_block60_c1_r2(x[0], x[1], x[2], a, mc, s);
    sph_block60_c2_r0(x[0], x[1], x[2], a, mc, s); sph_block60_c2_r1(x[0], x[1], x[2], a, mc, s);
    sph_block60_c2_r2(x[0], x[1], x[2], a, mc, s);
    if (self) sph_self60(mc, s);
  } else {
    return -1;
  }
  return 0;
}

extern "C" int hg_node(int layout, const double* x, double a, double E0, double nu0, double E1,
                       double nu1, double* out /* 3 x layout */) {
  SphMat mc = sph_mat_init(E0, nu0, E1, nu1);
  memset(out, 0, sizeof(double) * 3 * layout);
  ArrSink s{out, layout};
  if (layout == 24) sph_node24(x[0], x[1], x[2], a, mc, s);
  else if (layout == 78) sph_node78(x[0], x[1], x[2], a, mc, s);
  else if (layout == 60) sph_node60(x[0], x[1], x[2], a, mc, s);
  else return -1;
  return 0;
}

extern "C" int hg_field(int layout, const double* x, double a, double E0, double nu0, double E1,
                        double nu1, const double* E, double* e /* 6, accumulated */) {
  SphMat mc = sph_mat_init(E0, nu0, E1, nu1);
  if (layout == 24) sph_field24(x[0], x[1], x[2], a, mc, E, e);
  else if (layout == 78) sph_field78(x[0], x[1], x[2], a, mc, E, e);
  else if (layout == 60) sph_field60(x[0], x[1], x[2], a, mc, E, e);
  else return -1;
  return 0;
}

#include "gen_bem.cuh"
#include "bem_contract.cuh"

// Dsu/Dst of all rows of one order (rows (k<=l) x W, W last), dofs fastest.
extern "C" int hg_bem_stress(int order, const double* x, const double* nv, double E0, double nu0,
                             double E1, double nu1, double dlam, double dmu, double* Dsu,
                             double* Dst) {
  BemMat bm = bem_mat_init(E0, nu0, E1, nu1);
  double su[18], st[18];
  int nW = order == 0 ? 1 : (order == 1 ? 3 : 9);
#define CALL(fn)                                                                  \
  fn(x[0], x[1], x[2], nv[0], nv[1], nv[2], bm, dlam, dmu, su, st);               \
  for (int t = 0; t < 6; ++t) {                                                   \
    Dsu[(t * nW + w) * 3 + n] = su[t * 3 + n];                                    \
    Dst[(t * nW + w) * 3 + n] = st[t * 3 + n];                                    \
  }
  for (int w = 0; w < nW; ++w)
    for (int n = 0; n < 3; ++n) {
      if (order == 0) {
        if (n == 0) { CALL(bem_stress_o0_w_n0) } else if (n == 1) { CALL(bem_stress_o0_w_n1) } else { CALL(bem_stress_o0_w_n2) }
      } else if (order == 1) {
        switch (w * 3 + n) {
          case 0: { CALL(bem_stress_o1_w0_n0) } break; case 1: { CALL(bem_stress_o1_w0_n1) } break;
          case 2: { CALL(bem_stress_o1_w0_n2) } break; case 3: { CALL(bem_stress_o1_w1_n0) } break;
          case 4: { CALL(bem_stress_o1_w1_n1) } break; case 5: { CALL(bem_stress_o1_w1_n2) } break;
          case 6: { CALL(bem_stress_o1_w2_n0) } break; case 7: { CALL(bem_stress_o1_w2_n1) } break;
          case 8: { CALL(bem_stress_o1_w2_n2) } break;
        }
      } else {
        switch (w * 3 + n) {
#define C2(W, N, WS) case W * 3 + N: { CALL(bem_stress_o2_w##WS##_n##N) } break;
          C2(0, 0, 00) C2(0, 1, 00) C2(0, 2, 00) C2(1, 0, 01) C2(1, 1, 01) C2(1, 2, 01)
          C2(2, 0, 02) C2(2, 1, 02) C2(2, 2, 02) C2(3, 0, 10) C2(3, 1, 10) C2(3, 2, 10)
          C2(4, 0, 11) C2(4, 1, 11) C2(4, 2, 11) C2(5, 0, 12) C2(5, 1, 12) C2(5, 2, 12)
          C2(6, 0, 20) C2(6, 1, 20) C2(6, 2, 20) C2(7, 0, 21) C2(7, 1, 21) C2(7, 2, 21)
          C2(8, 0, 22) C2(8, 1, 22) C2(8, 2, 22)
#undef C2
        }
      }
    }
#undef CALL
  return 0;
}

extern "C" int hg_bem_stress_post(const double* x, const double* nv, double E0, double nu0,
                                  double E1, double nu1, double* Dsu, double* Dst) {
  BemMat bm = bem_mat_init(E0, nu0, E1, nu1);
  bem_stress_post(x[0], x[1], x[2], nv[0], nv[1], nv[2], bm, bm.lam0, bm.mu0, Dsu, Dst);
  return 0;
}

// the same stress contracted with boundary values u and t (bem_contract.cuh), and the
// generated kernels contracted with them afterwards
extern "C" int hg_bem_post_pair(const double* x, const double* nv, const double* u, const double* t, double E0,
                                double nu0, double E1, double nu1, double* s_contracted, double* s_generated) {
  BemMat bm = bem_mat_init(E0, nu0, E1, nu1);
  double Dsu[18], Dst[18];
  bem_stress_post(x[0], x[1], x[2], nv[0], nv[1], nv[2], bm, bm.lam0, bm.mu0, Dsu, Dst);
  for (int q = 0; q < 6; ++q) {
    s_generated[q] = 0.0;
    for (int n = 0; n < 3; ++n) s_generated[q] += Dsu[3 * q + n] * u[n] + Dst[3 * q + n] * t[n];
  }
  bem_post_contracted(x[0], x[1], x[2], nv[0], nv[1], nv[2], u[0], u[1], u[2], t[0], t[1], t[2], bem_post_coef(bm),
                      s_contracted);
  return 0;
}

// the mixed form's double-float contraction of one Gauss point record r (y, n, w, u, t) at
// the sample point p, and the FP64 contraction times the weight
extern "C" int hg_bem_post_pair_df(const double* p, const double* r, double E0, double nu0, double E1, double nu1,
                                   double* s_df, double* s_fp64) {
  BemMat bm = bem_mat_init(E0, nu0, E1, nu1);
  const BemPostCoef cf = bem_post_coef(bm);
  const ibem::BemPostDF g = ibem::bem_post_df_record(r, cf);
  const ibem::dfloat pd[3] = {ibem::df_make(p[0]), ibem::df_make(p[1]), ibem::df_make(p[2])};
  ibem::dacc acc[6] = {};
  ibem::bem_post_contracted_df(pd, g, ibem::bem_post_coef_df(cf), acc);
  double s[6];
  bem_post_contracted(r[0] - p[0], r[1] - p[1], r[2] - p[2], r[3], r[4], r[5], r[7], r[8], r[9], r[10], r[11], r[12], cf,
                      s);
  for (int q = 0; q < 6; ++q) {
    s_df[q] = (double)acc[q].s + (double)acc[q].c;
    s_fp64[q] = r[6] * s[q];
  }
  return 0;
}

#include "field_contract.cuh"

extern "C" int hg_field24c(const double* x, double a, double E0, double nu0, double E1, double nu1,
                           const double* E, double* e) {
  SphMat mc = sph_mat_init(E0, nu0, E1, nu1);
  sph_field24_contracted(x[0], x[1], x[2], a, mc, E, e);
  return 0;
}

// the double-float form of the same contraction: point p, sphere centre cen, radius a;
// returns the strain (times the material constant) in e
extern "C" int hg_field24df(const double* p, const double* cen, double a, double E0, double nu0, double E1,
                            double nu1, const double* E, double* e) {
  SphMat mc = sph_mat_init(E0, nu0, E1, nu1);
  const ibem::SphDF sp = ibem::sph_df_make(cen, a, E);
  const ibem::dfloat pd[3] = {ibem::df_make(p[0]), ibem::df_make(p[1]), ibem::df_make(p[2])};
  ibem::dacc acc[6] = {};
  ibem::sph_field24_df(pd, sp, ibem::df_make(mc.tn1), ibem::df_make(mc.tn2), acc);
  for (int t = 0; t < 6; ++t) e[t] = mc.kd * ((double)acc[t].s + (double)acc[t].c);
  return 0;
}

#include "mf_contract.cuh"

// The layout-60 pair block at offset x of a unit source sphere: out64 from the FP64 functions
// (all nine sub-blocks), out32 from the FP32 column groups the matrix-free solver calls
// (moduli / mu0, multiplied back by mu0 here); out[r * 60 + c]
struct Put60 {
  double* M;
  double scale;
  template <class T>
  void operator()(int r, int c, T v) { M[r * 60 + c] += scale * (double)v; }
};
extern "C" int hg_block60_groups(const double* x, double E0, double nu0, double E1, double nu1, double* out64,
                                 double* out32) {
  SphMat mc = sph_mat_init(E0, nu0, E1, nu1);
  const SphMatF mf = sph_matf_init(mc);
  for (int i = 0; i < 3600; ++i) out64[i] = out32[i] = 0.0;
  Put60 p64{out64, 1.0}, p32{out32, mc.mu0};
  const double a = 1.0;
  sph_block60_c0_r0(x[0], x[1], x[2], a, mc, p64); sph_block60_c1_r0(x[0], x[1], x[2], a, mc, p64);
  sph_block60_c2_r0(x[0], x[1], x[2], a, mc, p64); sph_block60_c0_r1(x[0], x[1], x[2], a, mc, p64);
  sph_block60_c1_r1(x[0], x[1], x[2], a, mc, p64); sph_block60_c2_r1(x[0], x[1], x[2], a, mc, p64);
  sph_block60_c0_r2(x[0], x[1], x[2], a, mc, p64); sph_block60_c1_r2(x[0], x[1], x[2], a, mc, p64);
  sph_block60_c2_r2(x[0], x[1], x[2], a, mc, p64);
  const float f0 = (float)x[0], f1 = (float)x[1], f2 = (float)x[2], one = 1.0f;
  sph_block60fm_c0_r0(f0, f1, f2, one, mf, p32); sph_block60fm_c1_r0(f0, f1, f2, one, mf, p32);
  sph_block60fm_c2_r0(f0, f1, f2, one, mf, p32); sph_block60fm_c0_r1(f0, f1, f2, one, mf, p32);
  sph_block60fm_c1_r1(f0, f1, f2, one, mf, p32);
  sph_block60f_c2g0_r1(f0, f1, f2, one, mf, p32); sph_block60f_c2g1_r1(f0, f1, f2, one, mf, p32);
  sph_block60f_c2g2_r1(f0, f1, f2, one, mf, p32); sph_block60f_c2g3_r1(f0, f1, f2, one, mf, p32);
  sph_block60f_c2g4_r1(f0, f1, f2, one, mf, p32); sph_block60f_c2g5_r1(f0, f1, f2, one, mf, p32);
  sph_block60fm_c0_r2(f0, f1, f2, one, mf, p32);
  sph_block60f_c1g0_r2(f0, f1, f2, one, mf, p32); sph_block60f_c1g1_r2(f0, f1, f2, one, mf, p32);
  sph_block60f_c1g2_r2(f0, f1, f2, one, mf, p32);
  sph_block60f_c2g0_r2(f0, f1, f2, one, mf, p32); sph_block60f_c2g1_r2(f0, f1, f2, one, mf, p32);
  sph_block60f_c2g2_r2(f0, f1, f2, one, mf, p32); sph_block60f_c2g3_r2(f0, f1, f2, one, mf, p32);
  sph_block60f_c2g4_r2(f0, f1, f2, one, mf, p32); sph_block60f_c2g5_r2(f0, f1, f2, one, mf, p32);
  return 0;
}

// Product of one layout-24 pair block with a coefficient vector as the matrix-free solver
// evaluates it (contracted strain and its gradient), in FP64 or FP32.
extern "C" int hg_pair_apply24(int fp32, const double* x, double a, double E0, double nu0, double E1,
                               double nu1, const double* coef, double* out /* 24 */) {
  SphMat mc = sph_mat_init(E0, nu0, E1, nu1);
  if (fp32) {
    float y[24] = {0}, cf[24];
    for (int i = 0; i < 24; ++i) cf[i] = (float)coef[i];
    ibem::sph_pair_apply24<float>((float)x[0], (float)x[1], (float)x[2], (float)a, (float)mc.kmu, (float)mc.klam,
                                  (float)mc.tn1, (float)mc.tn2, cf, 1.0f, y);
    for (int i = 0; i < 24; ++i) out[i] = y[i];
  } else {
    double y[24] = {0};
    ibem::sph_pair_apply24<double>(x[0], x[1], x[2], a, mc.kmu, mc.klam, mc.tn1, mc.tn2, coef, 1.0, y);
    for (int i = 0; i < 24; ++i) out[i] = y[i];
  }
  return 0;
}

// the FP32 far-pair form of the contraction (field_contract.cuh: sph_field24_f32)
extern "C" int hg_field24f32(const double* p, const double* cen, double a, double E0, double nu0, double E1,
                             double nu1, const double* E, double* e) {
  SphMat mc = sph_mat_init(E0, nu0, E1, nu1);
  const ibem::SphDF sp = ibem::sph_df_make(cen, a, E);
  const ibem::dfloat pd[3] = {ibem::df_make(p[0]), ibem::df_make(p[1]), ibem::df_make(p[2])};
  float r[6];
  ibem::sph_field24_f32(pd, sp, (float)mc.tn1, (float)mc.tn2, r);
  for (int t = 0; t < 6; ++t) e[t] = mc.kd * (double)r[t];
  return 0;
}
