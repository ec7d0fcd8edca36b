// Test infrastructure only: a driver that links the reference's own elastic-3D
// translation units (compiled from their sources in place, never copied) and
// dumps every intermediate of the 3D spherical iBEM pipeline as .npy files.
//
// It calls the four plugin interfaces in the order of the reference services:
//   iBEMSystemService.h:58-67   addBEM, addFieldToBEM, inclusion 0/1/2, BEM->incl 0/1/2
//   systemSolverService.h:41-45 ApplyBC, solve (Eigen fullPivLu), getUTVector
//   postprocessService.h:40-43  getField, getFlux
// Nothing in the product links, loads or runs this file or its binary.
//
// Usage:
//   ibem_ref run <workdir> [--no-solve] [--no-post] [--no-matrices]
//       reads position.txt / BEM.txt / postprocess.txt from <workdir> (the reference
//       opens them by fixed relative names, configElastic3D.h:54-56), writes
//       HMAT.npy GMAT.npy A.npy b.npy X.npy U.npy T.npy stress.npy timings.txt there
//       (--no-matrices: no HMAT / GMAT / A, which are N x N and N x 12NE doubles).
//   ibem_ref kat <workdir>
//       reads kat_in.npy (rows: x0 x1 x2 a) and kat_mat.npy (E0 nu0 E1 nu1) and
//       writes the reference's D_xy / IGreen / Green values to kat_*.npy.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <unistd.h>

#include "configElastic3D.h"
#include "integratorElastic3D.h"
#include "BEMBuilderElastic3D.h"
#include "postProcessorElastic3D.h"
#include "systemSolverElastic3D.h"
#include "integratorElastic3DHelper.h"

using namespace Elastic3DSpherical;

static void write_npy(const std::string& path, const double* data,
                      const std::vector<long>& shape, bool fortran) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { std::perror(path.c_str()); std::exit(2); }
  std::string shp = "(";
  for (size_t i = 0; i < shape.size(); ++i) {
    shp += std::to_string(shape[i]);
    shp += (shape.size() == 1 || i + 1 < shape.size()) ? "," : "";
    if (i + 1 < shape.size()) shp += " ";
  }
  shp += ")";
  std::string hdr = std::string("{'descr': '<f8', 'fortran_order': ") +
                    (fortran ? "True" : "False") + ", 'shape': " + shp + ", }";
  size_t total = 10 + hdr.size() + 1;
  size_t pad = (64 - total % 64) % 64;
  hdr.append(pad, ' ');
  hdr.push_back('\n');
  unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  std::fwrite(magic, 1, 8, f);
  unsigned short hl = (unsigned short)hdr.size();
  std::fwrite(&hl, 2, 1, f);
  std::fwrite(hdr.data(), 1, hdr.size(), f);
  long n = 1;
  for (long s : shape) n *= s;
  std::fwrite(data, sizeof(double), (size_t)n, f);
  std::fclose(f);
}

static std::vector<double> read_npy(const std::string& path, std::vector<long>& shape) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) { std::perror(path.c_str()); std::exit(2); }
  unsigned char magic[8];
  if (std::fread(magic, 1, 8, f) != 8) std::exit(2);
  unsigned short hl = 0;
  if (std::fread(&hl, 2, 1, f) != 1) std::exit(2);
  std::string hdr(hl, ' ');
  if (std::fread(&hdr[0], 1, hl, f) != hl) std::exit(2);
  if (hdr.find("'<f8'") == std::string::npos || hdr.find("True") != std::string::npos) {
    std::fprintf(stderr, "%s: need C-order float64\n", path.c_str());
    std::exit(2);
  }
  size_t p = hdr.find('(');
  size_t q = hdr.find(')');
  std::string dims = hdr.substr(p + 1, q - p - 1);
  shape.clear();
  long n = 1;
  for (char* tok = std::strtok(&dims[0], ", "); tok; tok = std::strtok(nullptr, ", ")) {
    shape.push_back(std::atol(tok));
    n *= shape.back();
  }
  std::vector<double> v((size_t)n);
  if (std::fread(v.data(), sizeof(double), (size_t)n, f) != (size_t)n) std::exit(2);
  std::fclose(f);
  return v;
}

static double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

static void dump_mat(const std::string& name, const MatrixXd& m) {
  write_npy(name, m.data(), {(long)m.rows(), (long)m.cols()}, true);
}
static void dump_vec(const std::string& name, const VectorXd& v) {
  write_npy(name, v.data(), {(long)v.size()}, false);
}

static int cmd_run(const char* dir, bool solve, bool post, bool matrices) {
  if (chdir(dir) != 0) { std::perror(dir); return 2; }
  configElastic3D cfg;
  FILE* tf = std::fopen("timings.txt", "w");
  double t0 = now_s();
  cfg.setUp();
  double t1 = now_s();
  std::fprintf(tf, "preprocess %.6f\n", t1 - t0);

  BEMBuilderElastic3D bem;
  integratorElastic3D integ;
  BEMBuilder& B = bem;
  integrator& I = integ;
  struct Stage { const char* name; double t; };
  auto timed = [&](const char* name, auto&& fn) {
    double a = now_s();
    fn();
    double b = now_s();
    std::fprintf(tf, "%s %.6f\n", name, b - a);
    std::fflush(tf);
  };
  timed("addBEM", [&] { B.addBEM(cfg); });
  timed("addFieldToBEM", [&] { I.addFieldToBEM(cfg); });
  timed("addFluxEquivalentInclusion", [&] { I.addFluxEquivalentInclusion(cfg); });
  timed("addFluxEquivalentFirstOrderInclusion", [&] { I.addFluxEquivalentFirstOrderInclusion(cfg); });
  timed("addFluxEquivalentSecondOrderInclusion", [&] { I.addFluxEquivalentSecondOrderInclusion(cfg); });
  timed("addFluxEquivalentBEM", [&] { B.addFluxEquivalentBEM(cfg); });
  timed("addFluxEquivalentFirstOrderBEM", [&] { B.addFluxEquivalentFirstOrderBEM(cfg); });
  timed("addFluxEquivalentSecondOrderBEM", [&] { B.addFluxEquivalentSecondOrderBEM(cfg); });
  if (matrices) {
    dump_mat("HMAT.npy", cfg.HMAT);
    dump_mat("GMAT.npy", cfg.GMAT);
  }
  timed("ApplyBC", [&] { B.ApplyBC(cfg); });
  if (matrices) dump_mat("A.npy", cfg.A);
  dump_vec("b.npy", cfg.b);
  if (solve) {
    systemSolverElastic3D solver;
    systemSolver& S = solver;
    timed("solve", [&] { S.solve(cfg); });
    dump_vec("X.npy", cfg.X);
    timed("getUTVector", [&] { B.getUTVector(cfg); });
    dump_vec("U.npy", cfg.U);
    dump_vec("T.npy", cfg.T);
    if (post) {
      postProcessorElastic3D pp;
      postProcessor& P = pp;
      timed("getField", [&] { P.getField(cfg); });
      timed("getFlux", [&] { P.getFlux(cfg); });
      std::vector<double> s((size_t)cfg.nump * 6);
      for (int i = 0; i < cfg.nump; ++i)
        for (int j = 0; j < 6; ++j) s[(size_t)i * 6 + j] = cfg.s_pt[i][j];
      write_npy("stress.npy", s.data(), {(long)cfg.nump, 6}, false);
    }
  }
  std::fclose(tf);
  return 0;
}

// Reference function values at a list of (x, a) rows, for pinning the oracle's
// restatement function by function.  Index loops follow the argument order of the
// reference signatures (integratorElastic3DHelper.h).
static int cmd_kat(const char* dir) {
  if (chdir(dir) != 0) { std::perror(dir); return 2; }
  std::vector<long> sh, shm;
  std::vector<double> in = read_npy("kat_in.npy", sh);
  std::vector<double> mat = read_npy("kat_mat.npy", shm);
  long npts = sh[0];
  mu_0 = mat[0] / (2.0 * (1.0 + mat[1]));
  nu0 = mat[1];
  mu_1 = mat[2] / (2.0 * (1.0 + mat[3]));
  nu1 = mat[3];
  // The D_xy functions take (s, h, radius, x_o, x_p): x = x_p(s) - x_o(h), a = radius(h).
  MatrixXd xo = MatrixXd::Zero(1, 3);
  MatrixXd xp(1, 3);
  VectorXd rad(1);
  std::vector<double> d40, d50, d60, d41, d51, d61, d42, d52, d62, ig0, ig1, ig2, g1, g2, g3, g4;
  for (long t = 0; t < npts; ++t) {
    double x[3] = {in[t * 4 + 0], in[t * 4 + 1], in[t * 4 + 2]};
    xp(0, 0) = x[0]; xp(0, 1) = x[1]; xp(0, 2) = x[2];
    rad(0) = in[t * 4 + 3];
    double a = rad(0);
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j)
    for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l) {
      d40.push_back(D_40(i, j, k, l, 0, 0, rad, xo, xp));
      for (int r = 0; r < 3; ++r) {
        d50.push_back(D_50(i, j, k, l, r, 0, 0, rad, xo, xp));
        d41.push_back(D_41(i, j, k, l, r, 0, 0, rad, xo, xp));
        for (int z = 0; z < 3; ++z) {
          d60.push_back(D_60(i, j, k, l, r, z, 0, 0, rad, xo, xp));
          d51.push_back(D_51(i, j, k, l, r, z, 0, 0, rad, xo, xp));
          d42.push_back(D_42(i, j, k, l, r, z, 0, 0, rad, xo, xp));
          for (int w = 0; w < 3; ++w) {
            d61.push_back(D_61(i, j, k, l, r, z, w, 0, 0, rad, xo, xp));
            d52.push_back(D_52(i, j, k, l, r, z, w, 0, 0, rad, xo, xp));
            for (int v = 0; v < 3; ++v)
              d62.push_back(D_62(i, j, k, l, r, z, w, v, 0, 0, rad, xo, xp));
          }
        }
      }
    }
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) for (int l = 0; l < 3; ++l) {
      ig0.push_back(IGreen_01(x, a, i, j, l));
      for (int p = 0; p < 3; ++p) {
        ig1.push_back(IGreen_11(x, a, i, j, p, l));
        for (int q = 0; q < 3; ++q) ig2.push_back(IGreen_21(x, a, i, j, p, q, l));
      }
    }
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) for (int k = 0; k < 3; ++k) {
      g1.push_back(Green_01(x, i, j, k));
      for (int l = 0; l < 3; ++l) {
        g2.push_back(Green_02(x, i, j, k, l));
        for (int s = 0; s < 3; ++s) {
          g3.push_back(Green_03(x, i, j, k, l, s));
          for (int u = 0; u < 3; ++u) g4.push_back(Green_04(x, i, j, k, l, s, u));
        }
      }
    }
  }
  auto w = [&](const char* name, std::vector<double>& v, int rank) {
    std::vector<long> shape{npts};
    for (int r = 0; r < rank; ++r) shape.push_back(3);
    write_npy(name, v.data(), shape, false);
  };
  w("kat_D40.npy", d40, 4); w("kat_D50.npy", d50, 5); w("kat_D60.npy", d60, 6);
  w("kat_D41.npy", d41, 5); w("kat_D51.npy", d51, 6); w("kat_D61.npy", d61, 7);
  w("kat_D42.npy", d42, 6); w("kat_D52.npy", d52, 7); w("kat_D62.npy", d62, 8);
  w("kat_IG0.npy", ig0, 3); w("kat_IG1.npy", ig1, 4); w("kat_IG2.npy", ig2, 5);
  w("kat_G1.npy", g1, 3); w("kat_G2.npy", g2, 4); w("kat_G3.npy", g3, 5); w("kat_G4.npy", g4, 6);
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 3 && std::strcmp(argv[1], "run") == 0) {
    bool solve = true, post = true, matrices = true;
    for (int i = 3; i < argc; ++i) {
      if (std::strcmp(argv[i], "--no-solve") == 0) solve = false;
      if (std::strcmp(argv[i], "--no-post") == 0) post = false;
      if (std::strcmp(argv[i], "--no-matrices") == 0) matrices = false;
    }
    return cmd_run(argv[2], solve, post, matrices);
  }
  if (argc >= 3 && std::strcmp(argv[1], "kat") == 0) return cmd_kat(argv[2]);
  std::fprintf(stderr, "usage: ibem_ref run <dir> [--no-solve] [--no-post] [--no-matrices] | kat <dir>\n");
  return 2;
}
