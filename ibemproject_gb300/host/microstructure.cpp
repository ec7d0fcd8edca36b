// Seeded sphere microstructures for boundary-free far-field cases: the C ABI entry point
// ibem_e3d_generate_spheres.  The reference reads centres and radii from position.txt
// (configElastic3D.cpp:106-128) and ships no generator; this one makes the inputs of the
// far-field workloads (thousands of spheres, hundreds of realisations) without text files.
//
// Two methods:
//   RSA  random sequential addition: draw a centre uniformly in the box that keeps every
//        sphere inside the cube, keep it when it clears every placed sphere, repeat;
//        fast up to about 20% volume fraction, jams below 30% in small cubes.
//   MC   hard-sphere Monte Carlo with box compression: spheres start on a simple cubic
//        lattice in a cube large enough for the largest pair, every sweep moves each sphere
//        by a random step (reflected at the faces, rejected if it would come closer than the
//        minimum distance to a neighbour), then the cube and all centres are scaled down toward
//        the target side as far as the closest pair allows; once the target is reached,
//        further sweeps randomise the configuration.  Centres stay in [0, L]^3 (spheres may
//        reach across the faces: the cube is a window of an unbounded particle cloud).
// Pairs must keep a centre distance of at least r_i + r_j + gap * max(r_i, r_j).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ibem_gb300.h"
#include "../csrc/ibem_internal.h"

namespace {

// xoshiro256** seeded through splitmix64 (Blackman & Vigna, public-domain generators): the
// same stream on every platform, so a seed names one microstructure.
struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    for (uint64_t& v : s) {
      seed += 0x9e3779b97f4a7c15ULL;
      uint64_t z = seed;
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
      v = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
};

inline double min_dist(double ri, double rj, double gap) { return ri + rj + gap * std::max(ri, rj); }
}  // namespace

namespace ibem {
void ell_quat_to_rot_host(const double* q, double* Q);
}

namespace {

// Uniform cell grid over [0, L]^3 with cells no smaller than `h`, one vector of sphere
// indices per cell.
struct Cells {
  int n = 1;
  double inv = 0.0;
  std::vector<std::vector<int>> cell;
  std::vector<int> where;

  void build(double L, double h, const std::vector<double>& c, int count) {
    n = std::max(1, std::min(128, (int)std::floor(L / h)));
    inv = n / L;
    cell.assign((size_t)n * n * n, {});
    where.assign(c.size() / 3, -1);
    for (int k = 0; k < count; ++k) insert(k, &c[3 * k]);
  }
  int index(const double* x) const {
    int i[3];
    for (int d = 0; d < 3; ++d) i[d] = std::min(n - 1, std::max(0, (int)(x[d] * inv)));
    return (i[2] * n + i[1]) * n + i[0];
  }
  void insert(int k, const double* x) {
    const int id = index(x);
    cell[id].push_back(k);
    where[k] = id;
  }
  void remove(int k) {
    std::vector<int>& v = cell[where[k]];
    const auto it = std::find(v.begin(), v.end(), k);
    *it = v.back();
    v.pop_back();
    where[k] = -1;
  }
  // Calls f(j) for every sphere j in the 27 cells around x.
  template <class F>
  bool any_near(const double* x, F&& f) const {
    int i[3];
    for (int d = 0; d < 3; ++d) i[d] = std::min(n - 1, std::max(0, (int)(x[d] * inv)));
    for (int z = std::max(0, i[2] - 1); z <= std::min(n - 1, i[2] + 1); ++z)
      for (int y = std::max(0, i[1] - 1); y <= std::min(n - 1, i[1] + 1); ++y)
        for (int w = std::max(0, i[0] - 1); w <= std::min(n - 1, i[0] + 1); ++w)
          for (int j : cell[(z * n + y) * n + w])
            if (f(j)) return true;
    return false;
  }
};

bool clashes(const Cells& g, const std::vector<double>& c, const std::vector<double>& r, const double* x, double rx,
             int self, double gap) {
  return g.any_near(x, [&](int j) {
    if (j == self) return false;
    const double dx = x[0] - c[3 * j], dy = x[1] - c[3 * j + 1], dz = x[2] - c[3 * j + 2];
    const double m = min_dist(rx, r[j], gap);
    return dx * dx + dy * dy + dz * dz < m * m;
  });
}

ibem_status rsa(const ibem_gen_params& p, double L, std::vector<double>& c, const std::vector<double>& r) {
  const int num = p.num;
  const double rmax = p.r0 * p.rhi, lo = rmax, hi = L - rmax;
  if (hi <= lo) return ibem::fail(IBEM_ERR_ARG, "generate_spheres: cube smaller than one sphere");
  Rng rng(p.seed);
  Cells g;
  g.build(L, min_dist(rmax, rmax, p.gap), c, 0);
  const int64_t cap = p.max_tries > 0 ? p.max_tries : 200000000LL;
  int64_t tries = 0;
  for (int k = 0; k < num; ++k) {
    double x[3];
    do {
      if (++tries > cap)
        return ibem::fail(IBEM_ERR_ARG, "generate_spheres: random sequential addition stalled at " +
                                            std::to_string(k) + " of " + std::to_string(num) + " spheres");
      for (double& v : x) v = rng.uniform(lo, hi);
    } while (clashes(g, c, r, x, r[k], -1, p.gap));
    std::memcpy(&c[3 * k], x, sizeof x);
    g.insert(k, x);
  }
  return IBEM_OK;
}

ibem_status mc(const ibem_gen_params& p, double L, std::vector<double>& c, const std::vector<double>& r) {
  const int num = p.num;
  const double rmax = *std::max_element(r.begin(), r.end());
  const double h = min_dist(rmax, rmax, p.gap);
  Rng rng(p.seed ^ 0x5bd1e995ULL);
  // simple cubic start, spacing that clears the largest pair, sites in random order
  int m = 1;
  while ((int64_t)m * m * m < num) ++m;
  const double s0 = h * (1.0 + 1e-9);
  double Lc = std::max(L, m > 1 ? s0 * (m - 1) : L);
  const double step0 = m > 1 ? Lc / (m - 1) : 0.0;
  std::vector<int> site((size_t)m * m * m);
  for (size_t i = 0; i < site.size(); ++i) site[i] = (int)i;
  for (size_t i = site.size() - 1; i > 0; --i) std::swap(site[i], site[rng.next() % (i + 1)]);
  for (int k = 0; k < num; ++k) {
    const int q = site[k];
    c[3 * k] = step0 * (q % m);
    c[3 * k + 1] = step0 * ((q / m) % m);
    c[3 * k + 2] = step0 * (q / (m * m));
    if (m == 1)
      for (int d = 0; d < 3; ++d) c[3 * k + d] = 0.5 * L;
  }
  // Cells of side >= h / kMinScale: a pair in non-adjacent cells is at least h / kMinScale
  // apart, so after one shrink by a factor >= kMinScale it still clears h, the largest
  // minimum distance; the closest pairs, which limit the shrink, are all in adjacent cells.
  constexpr double kMinScale = 0.9;
  const double hc = h / kMinScale;
  Cells g;
  double delta = 0.5 * h;
  const int settle = p.sweeps > 0 ? p.sweeps : 100;
  int after = 0, stalled = 0;
  for (int sweep = 0; sweep < 100000; ++sweep) {
    g.build(Lc, hc, c, num);
    int accepted = 0;
    for (int t = 0; t < num; ++t) {
      const int k = (int)(rng.next() % (uint64_t)num);
      double x[3];
      for (int d = 0; d < 3; ++d) {  // steps that cross a face are reflected back into the cube
        x[d] = c[3 * k + d] + rng.uniform(-delta, delta);
        if (x[d] < 0.0) x[d] = -x[d];
        if (x[d] > Lc) x[d] = 2.0 * Lc - x[d];
        x[d] = std::min(std::max(x[d], 0.0), Lc);
      }
      if (clashes(g, c, r, x, r[k], k, p.gap)) continue;
      g.remove(k);
      std::memcpy(&c[3 * k], x, sizeof x);
      g.insert(k, x);
      ++accepted;
    }
    // keep about a third of the moves accepted
    const double acc = (double)accepted / num;
    delta *= acc > 0.35 ? 1.1 : 0.9;
    delta = std::min(std::max(delta, 1e-6 * h), 0.5 * h);
    if (Lc <= L) {
      if (++after >= settle) return IBEM_OK;
      continue;
    }
    // largest admissible shrink: the closest pair (relative to its minimum distance) may
    // close half of its remaining room
    double f = 0.0;
    for (int k = 0; k < num; ++k)
      g.any_near(&c[3 * k], [&](int j) {
        if (j <= k) return false;
        const double dx = c[3 * k] - c[3 * j], dy = c[3 * k + 1] - c[3 * j + 1], dz = c[3 * k + 2] - c[3 * j + 2];
        f = std::max(f, min_dist(r[k], r[j], p.gap) / std::sqrt(dx * dx + dy * dy + dz * dz));
        return false;
      });
    const double scale = std::max({L / Lc, kMinScale, 0.5 * (1.0 + f)});
    stalled = scale > 1.0 - 1e-7 ? stalled + 1 : 0;
    if (stalled > 2000) break;  // jammed: the closest pairs no longer open up
    if (scale < 1.0) {
      for (double& v : c) v *= scale;
      Lc = std::max(L, Lc * scale);
    }
  }
  return ibem::fail(IBEM_ERR_ARG, "generate_spheres: compression did not reach the volume fraction");
}

// ---------------------------------------------------------------- ellipsoids
// Perram-Wertheim contact function of two ellipsoids x^T M_A x <= 1 and x^T M_B x <= 1
// (M = Q diag(a^-2) Q^T) whose centres differ by r:
//   F(lam) = lam (1 - lam) r^T [(1 - lam) M_A^-1 + lam M_B^-1]^-1 r,  0 <= lam <= 1;
// F is concave and the bodies are disjoint exactly when max F > 1 (J. W. Perram and
// M. S. Wertheim, J. Comput. Phys. 58 (1985) 409).  Scaling r by s scales F by s^2.
struct Ell {
  double P[9];   // M^-1 = Q diag(a^2) Q^T
  double rb;     // bounding radius (longest semi-axis)
  double ri;     // inscribed radius (shortest semi-axis)
};

Ell make_ell(const double* a, const double* q, double inflate) {
  Ell e;
  double Q[9];
  ibem::ell_quat_to_rot_host(q, Q);
  double s[3];
  for (int m = 0; m < 3; ++m) s[m] = (a[m] + inflate) * (a[m] + inflate);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double v = 0.0;
      for (int m = 0; m < 3; ++m) v += Q[3 * i + m] * s[m] * Q[3 * j + m];
      e.P[3 * i + j] = v;
    }
  e.rb = std::max(a[0], std::max(a[1], a[2])) + inflate;
  e.ri = std::min(a[0], std::min(a[1], a[2])) + inflate;
  return e;
}

double pw_value(const Ell& A, const Ell& B, const double* r, double lam) {
  double G[9];
  for (int i = 0; i < 9; ++i) G[i] = (1.0 - lam) * A.P[i] + lam * B.P[i];
  // r^T G^-1 r by Cramer's rule (G symmetric positive definite)
  const double c00 = G[4] * G[8] - G[5] * G[7], c01 = G[5] * G[6] - G[3] * G[8], c02 = G[3] * G[7] - G[4] * G[6];
  const double det = G[0] * c00 + G[1] * c01 + G[2] * c02;
  const double c11 = G[0] * G[8] - G[2] * G[6], c12 = G[2] * G[3] - G[0] * G[5], c22 = G[0] * G[4] - G[1] * G[3];
  const double q = r[0] * r[0] * c00 + r[1] * r[1] * c11 + r[2] * r[2] * c22 +
                   2.0 * (r[0] * r[1] * c01 + r[0] * r[2] * c02 + r[1] * r[2] * c12);
  return lam * (1.0 - lam) * q / det;
}

// max_lam F by golden-section search (F is concave on [0, 1])
double pw_max(const Ell& A, const Ell& B, const double* r) {
  const double g = 0.6180339887498949;
  double lo = 0.0, hi = 1.0, x1 = hi - g * (hi - lo), x2 = lo + g * (hi - lo);
  double f1 = pw_value(A, B, r, x1), f2 = pw_value(A, B, r, x2);
  for (int it = 0; it < 40; ++it) {
    if (f1 < f2) { lo = x1; x1 = x2; f1 = f2; x2 = lo + g * (hi - lo); f2 = pw_value(A, B, r, x2); }
    else { hi = x2; x2 = x1; f2 = f1; x1 = hi - g * (hi - lo); f1 = pw_value(A, B, r, x1); }
  }
  return std::max(f1, f2);
}

// true when the (inflated) ellipsoids overlap
bool ell_overlap(const Ell& A, const Ell& B, const double* r) {
  const double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  if (d2 >= (A.rb + B.rb) * (A.rb + B.rb)) return false;
  if (d2 < (A.ri + B.ri) * (A.ri + B.ri)) return true;
  return pw_max(A, B, r) <= 1.0;
}

// Haar-uniform unit quaternion (w, x, y, z) from three uniforms (K. Shoemake, Graphics Gems III, 1992)
void uniform_quat(Rng& g, double* q) {
  const double u1 = g.uniform(), u2 = 2.0 * M_PI * g.uniform(), u3 = 2.0 * M_PI * g.uniform();
  const double s1 = std::sqrt(1.0 - u1), s2 = std::sqrt(u1);
  q[0] = s2 * std::cos(u3);
  q[1] = s1 * std::sin(u2);
  q[2] = s1 * std::cos(u2);
  q[3] = s2 * std::sin(u3);
}

}  // namespace

namespace ibem {
void ell_quat_to_rot_host(const double* q, double* Q) {
  const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  const double w = q[0] / n, x = q[1] / n, y = q[2] / n, z = q[3] / n;
  Q[0] = 1 - 2 * (y * y + z * z); Q[1] = 2 * (x * y - w * z); Q[2] = 2 * (x * z + w * y);
  Q[3] = 2 * (x * y + w * z); Q[4] = 1 - 2 * (x * x + z * z); Q[5] = 2 * (y * z - w * x);
  Q[6] = 2 * (x * z - w * y); Q[7] = 2 * (y * z + w * x); Q[8] = 1 - 2 * (x * x + y * y);
}
}  // namespace ibem

namespace {

// random sequential addition inside [a1, L - a1]^3
ibem_status ell_rsa(const ibem_ell_gen_params& p, double L, double rbmax, const std::vector<Ell>& e,
                    std::vector<double>& c) {
  const int num = p.num;
  const double lo = p.a1, hi = L - p.a1;
  if (hi <= lo) return ibem::fail(IBEM_ERR_ARG, "generate_ellipsoids: cube smaller than one ellipsoid");
  Rng rng(p.seed + 0x632be59bd9b4e019ULL);
  Cells g;
  g.build(L, 2.0 * rbmax, c, 0);
  const int64_t cap = p.max_tries > 0 ? p.max_tries : 200000000LL;
  int64_t tries = 0;
  for (int k = 0; k < num; ++k) {
    double x[3];
    bool bad;
    do {
      if (++tries > cap)
        return ibem::fail(IBEM_ERR_ARG, "generate_ellipsoids: random sequential addition stalled at " +
                                            std::to_string(k) + " of " + std::to_string(num));
      for (double& v : x) v = rng.uniform(lo, hi);
      bad = g.any_near(x, [&](int j) {
        const double r[3] = {c[3 * j] - x[0], c[3 * j + 1] - x[1], c[3 * j + 2] - x[2]};
        return ell_overlap(e[k], e[j], r);
      });
    } while (bad);
    std::memcpy(&c[3 * k], x, sizeof x);
    g.insert(k, x);
  }
  return IBEM_OK;
}

// q <- q * (rotation by a small random angle about a uniform axis), normalised
void jiggle_quat(Rng& g, double maxang, const double* q, double* out) {
  double ax[3], n2;
  do {
    for (double& v : ax) v = g.uniform(-1.0, 1.0);
    n2 = ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2];
  } while (n2 > 1.0 || n2 < 1e-12);
  const double ang = g.uniform(-maxang, maxang), sh = std::sin(0.5 * ang) / std::sqrt(n2);
  const double r[4] = {std::cos(0.5 * ang), ax[0] * sh, ax[1] * sh, ax[2] * sh};
  double o[4] = {q[0] * r[0] - q[1] * r[1] - q[2] * r[2] - q[3] * r[3],
                 q[0] * r[1] + q[1] * r[0] + q[2] * r[3] - q[3] * r[2],
                 q[0] * r[2] - q[1] * r[3] + q[2] * r[0] + q[3] * r[1],
                 q[0] * r[3] + q[1] * r[2] - q[2] * r[1] + q[3] * r[0]};
  const double n = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2] + o[3] * o[3]);
  for (int i = 0; i < 4; ++i) out[i] = o[i] / n;
}

// Hard-ellipsoid Monte Carlo with box compression (the ellipsoid counterpart of `mc` above):
// a simple cubic start that clears the largest bounding spheres, sweeps of random
// translations (reflected at the faces) and small rotations rejected on overlap, and after
// each sweep a uniform scaling of the centres toward the target side as far as the closest
// pair allows (scaling a pair's offset by s scales its contact function by s^2, so the pair
// touches at s = F_max^-1/2; the scale closes half of the remaining room).  Centres stay in
// [0, L]^3; orientations change with the moves.
ibem_status ell_mc(const ibem_ell_gen_params& p, double L, double rbmax, const std::vector<double>& a,
                   std::vector<double>& q, std::vector<Ell>& e, std::vector<double>& c) {
  const int num = p.num;
  Rng rng(p.seed ^ 0x5bd1e995ULL);
  int m = 1;
  while ((int64_t)m * m * m < num) ++m;
  const double s0 = 2.0 * rbmax * (1.0 + 1e-9);
  double Lc = std::max(L, m > 1 ? s0 * (m - 1) : L);
  const double step0 = m > 1 ? Lc / (m - 1) : 0.0;
  std::vector<int> site((size_t)m * m * m);
  for (size_t i = 0; i < site.size(); ++i) site[i] = (int)i;
  for (size_t i = site.size() - 1; i > 0; --i) std::swap(site[i], site[rng.next() % (i + 1)]);
  for (int k = 0; k < num; ++k) {
    const int t = site[k];
    c[3 * k] = step0 * (t % m);
    c[3 * k + 1] = step0 * ((t / m) % m);
    c[3 * k + 2] = step0 * (t / (m * m));
    if (m == 1)
      for (int d = 0; d < 3; ++d) c[3 * k + d] = 0.5 * L;
  }
  constexpr double kMinScale = 0.9;
  const double h = 2.0 * rbmax;
  const double hc = h / kMinScale;
  const double infl = 0.5 * p.gap;
  Cells g;
  double delta = 0.25 * h, rot = 0.3;
  const int settle = p.sweeps > 0 ? p.sweeps : 50;
  int after = 0, stalled = 0;
  for (int sweep = 0; sweep < 20000; ++sweep) {
    g.build(Lc, hc, c, num);
    int accepted = 0;
    for (int t = 0; t < num; ++t) {
      const int k = (int)(rng.next() % (uint64_t)num);
      double x[3], qn[4];
      for (int d = 0; d < 3; ++d) {
        x[d] = c[3 * k + d] + rng.uniform(-delta, delta);
        if (x[d] < 0.0) x[d] = -x[d];
        if (x[d] > Lc) x[d] = 2.0 * Lc - x[d];
        x[d] = std::min(std::max(x[d], 0.0), Lc);
      }
      jiggle_quat(rng, rot, &q[4 * k], qn);
      const Ell en = make_ell(&a[3 * k], qn, infl * a[3 * k + 2]);
      const bool bad = g.any_near(x, [&](int j) {
        if (j == k) return false;
        const double r[3] = {c[3 * j] - x[0], c[3 * j + 1] - x[1], c[3 * j + 2] - x[2]};
        return ell_overlap(en, e[j], r);
      });
      if (bad) continue;
      g.remove(k);
      std::memcpy(&c[3 * k], x, sizeof x);
      std::memcpy(&q[4 * k], qn, sizeof qn);
      e[k] = en;
      g.insert(k, x);
      ++accepted;
    }
    const double acc = (double)accepted / num;
    delta *= acc > 0.35 ? 1.1 : 0.9;
    delta = std::min(std::max(delta, 1e-6 * h), 0.5 * h);
    rot = std::min(std::max(rot * (acc > 0.35 ? 1.1 : 0.9), 1e-4), 1.0);
    if (Lc <= L) {
      if (++after >= settle) return IBEM_OK;
      continue;
    }
    // largest admissible shrink from the closest pair (bounding spheres overlapping)
    double f = 0.0;
    for (int k = 0; k < num; ++k)
      g.any_near(&c[3 * k], [&](int j) {
        if (j <= k) return false;
        const double r[3] = {c[3 * j] - c[3 * k], c[3 * j + 1] - c[3 * k + 1], c[3 * j + 2] - c[3 * k + 2]};
        const double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        if (d2 >= (e[k].rb + e[j].rb) * (e[k].rb + e[j].rb)) {
          f = std::max(f, (e[k].rb + e[j].rb) / std::sqrt(d2));
          return false;
        }
        f = std::max(f, 1.0 / std::sqrt(pw_max(e[k], e[j], r)));
        return false;
      });
    const double scale = std::max({L / Lc, kMinScale, 0.5 * (1.0 + f)});
    stalled = scale > 1.0 - 1e-7 ? stalled + 1 : 0;
    if (stalled > 500) break;
    if (scale < 1.0) {
      for (double& v : c) v *= scale;
      Lc = std::max(L, Lc * scale);
    }
  }
  return ibem::fail(IBEM_ERR_ARG, "generate_ellipsoids: compression did not reach the volume fraction");
}

}  // namespace

extern "C" ibem_status ibem_e3d_generate_ellipsoids(const ibem_ell_gen_params* p, double* centers, double* axes,
                                                    double* quats, double* side) {
  if (!p || p->num < 1 || !centers || !axes || !quats || !(p->a1 > 0) || !(p->a2lo > 0) || p->a2hi < p->a2lo ||
      !(p->a3lo > 0) || p->a3hi < p->a3lo || p->a2hi > 1 || p->a3hi > 1 || !(p->vf > 0 && p->vf < 0.5) ||
      p->gap < 0 || (p->method != IBEM_GEN_RSA && p->method != IBEM_GEN_MC))
    return ibem::fail(IBEM_ERR_ARG, "generate_ellipsoids: bad parameters");
  const int num = p->num;
  Rng rs(p->seed);
  std::vector<double> a(3 * (size_t)num), q(4 * (size_t)num), c(3 * (size_t)num, 0.0);
  double vol = 0.0;
  for (int k = 0; k < num; ++k) {
    a[3 * k] = p->a1;
    a[3 * k + 1] = p->a1 * rs.uniform(p->a2lo, p->a2hi);
    a[3 * k + 2] = p->a1 * rs.uniform(p->a3lo, p->a3hi);
    uniform_quat(rs, &q[4 * k]);
    vol += 4.0 / 3.0 * M_PI * a[3 * k] * a[3 * k + 1] * a[3 * k + 2];
  }
  const double L = std::cbrt(vol / p->vf);
  // surfaces kept apart by inflating every semi-axis by gap * a3 / 2 during the tests
  std::vector<Ell> e(num);
  double rbmax = 0.0;
  for (int k = 0; k < num; ++k) {
    e[k] = make_ell(&a[3 * k], &q[4 * k], 0.5 * p->gap * a[3 * k + 2]);
    rbmax = std::max(rbmax, e[k].rb);
  }
  ibem_status st = p->method == IBEM_GEN_MC ? ell_mc(*p, L, rbmax, a, q, e, c) : ell_rsa(*p, L, rbmax, e, c);
  if (st) return st;
  std::memcpy(centers, c.data(), sizeof(double) * c.size());
  std::memcpy(axes, a.data(), sizeof(double) * a.size());
  std::memcpy(quats, q.data(), sizeof(double) * q.size());
  if (side) *side = L;
  return IBEM_OK;
}

extern "C" ibem_status ibem_e3d_generate_spheres(const ibem_gen_params* p, double* centers, double* radius,
                                                 double* side) {
  if (!p || p->num < 1 || !centers || !radius || !(p->r0 > 0) || !(p->rlo > 0) || p->rhi < p->rlo ||
      !(p->vf > 0 && p->vf < 0.6) || p->gap < 0 || (p->method != IBEM_GEN_RSA && p->method != IBEM_GEN_MC))
    return ibem::fail(IBEM_ERR_ARG, "generate_spheres: bad parameters");
  const int num = p->num;
  std::vector<double> r(num), c(3 * (size_t)num, 0.0);
  Rng rr(p->seed);
  for (double& v : r) v = p->r0 * rr.uniform(p->rlo, p->rhi);
  double vol = 0.0;
  for (double v : r) vol += 4.0 / 3.0 * M_PI * v * v * v;
  const double L = std::cbrt(vol / p->vf);
  Rng rc(p->seed + 0x632be59bd9b4e019ULL);
  ibem_gen_params q = *p;
  q.seed = rc.next();
  const ibem_status s = p->method == IBEM_GEN_RSA ? rsa(q, L, c, r) : mc(q, L, c, r);
  if (s) return s;
  std::memcpy(centers, c.data(), sizeof(double) * c.size());
  std::memcpy(radius, r.data(), sizeof(double) * r.size());
  if (side) *side = L;
  return IBEM_OK;
}
