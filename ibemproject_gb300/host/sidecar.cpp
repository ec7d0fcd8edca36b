// Binary side-car of a case directory: one file, case.ibemb, that holds what position.txt,
// BEM.txt, postprocess.txt (configElastic3D.cpp:32-197, configElastic3D.h:76-129) and
// farfield.txt hold, so that large cases (tens of thousands of spheres, 64^3 sample points)
// load without parsing text.  No reference counterpart: the reference reads the text files
// on every run.
//
// Layout (every number in the byte order of the machine that wrote it; the marker lets a
// reader of the other byte order fail instead of misreading):
//   char    magic[8] = "IBEMCAS1"
//   uint32  0x01020304 (byte-order marker), uint32 0 (reserved)
//   double  E0, nu0, E1, nu1
//   int64   NN, NE, num, nump, has_farfield
//   double  nodes[3 NN]     (BEM.txt node block, row-major)
//   int32   conn[4 NE]      (one-based, as in BEM.txt)
//   double  bc[6 NN]        (3 NN rows of flag, value)
//   double  tbc[24 NE]      (12 flags, 12 values per element)
//   double  centers[3 num], radius[num]
//   double  points[3 nump]
//   double  sig_inf[6]      (only when has_farfield = 1)
// A directory's side-car is used in place of its text files when it is at least as new as
// each of them (configElastic3D_gb300::setUp).
#include <cstdint>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <string>
#include <vector>

#include "ibem_plugins.h"

#include "../csrc/ibem_internal.h"

namespace ibem_gb300 {

namespace {

constexpr char kMagic[8] = {'I', 'B', 'E', 'M', 'C', 'A', 'S', '1'};
constexpr uint32_t kOrder = 0x01020304u;
const char* const kSidecar = "case.ibemb";

std::string join(const std::string& dir, const std::string& f) { return dir.empty() ? f : dir + "/" + f; }

template <class T>
void put(std::ofstream& f, const T* p, size_t n) {
  if (n) f.write(reinterpret_cast<const char*>(p), (std::streamsize)(sizeof(T) * n));
}
template <class T>
void get(std::ifstream& f, T* p, size_t n, const std::string& path) {
  if (n && !f.read(reinterpret_cast<char*>(p), (std::streamsize)(sizeof(T) * n)))
    throw ibem_error(IBEM_ERR_IO, path + ": truncated");
}

// The text inputs of a directory that exist (the side-car must be at least as new as each).
bool sidecar_fresh(const configElastic3D_gb300& c) {
  namespace fs = std::filesystem;
  std::error_code ec;
  const fs::path sc = join(c.dir, kSidecar);
  if (!fs::exists(sc, ec)) return false;
  const auto t = fs::last_write_time(sc, ec);
  if (ec) return false;
  for (const std::string& f : {c.particleInput, c.bemInput, c.postProcessInput, std::string("farfield.txt")}) {
    const fs::path p = join(c.dir, f);
    if (fs::exists(p, ec) && fs::last_write_time(p, ec) > t) return false;
  }
  return true;
}

}  // namespace

void write_sidecar(const std::string& path, const configElastic3D_gb300& c) {
  std::ofstream f(path, std::ios::out | std::ios::binary | std::ios::trunc);
  if (!f) throw ibem_error(IBEM_ERR_IO, "cannot write " + path);
  const uint32_t hdr[2] = {kOrder, 0u};
  const double mat[4] = {c.EE, c.XNU, c.E1, c.nu1};
  const int64_t has_ff = c.sig_inf.size() == 6 ? 1 : 0;
  const int64_t sizes[5] = {c.NN, c.NE, c.num, c.nump, has_ff};
  put(f, kMagic, 8);
  put(f, hdr, 2);
  put(f, mat, 4);
  put(f, sizes, 5);
  put(f, c.NODES.data(), 3 * (size_t)c.NN);
  std::vector<int32_t> conn(c.NConnect.begin(), c.NConnect.end());
  put(f, conn.data(), 4 * (size_t)c.NE);
  put(f, c.BC.data(), 6 * (size_t)c.NN);
  put(f, c.t_bc.data(), 24 * (size_t)c.NE);
  put(f, c.eigen_point.data(), 3 * (size_t)c.num);
  put(f, c.radius.data(), (size_t)c.num);
  put(f, c.x_p.data(), 3 * (size_t)c.nump);
  if (has_ff) put(f, c.sig_inf.data(), 6);
  if (!f) throw ibem_error(IBEM_ERR_IO, "write failed: " + path);
}

void read_sidecar(const std::string& path, configElastic3D_gb300& c) {
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) throw ibem_error(IBEM_ERR_IO, "cannot open " + path);
  char magic[8];
  uint32_t hdr[2];
  double mat[4];
  int64_t sizes[5];
  get(f, magic, 8, path);
  if (std::memcmp(magic, kMagic, 8) != 0) throw ibem_error(IBEM_ERR_IO, path + ": not a case side-car");
  get(f, hdr, 2, path);
  if (hdr[0] != kOrder) throw ibem_error(IBEM_ERR_IO, path + ": written with another byte order");
  get(f, mat, 4, path);
  get(f, sizes, 5, path);
  for (int i = 0; i < 4; ++i)
    if (sizes[i] < 0 || sizes[i] > (int64_t)1 << 31) throw ibem_error(IBEM_ERR_IO, path + ": bad sizes");
  c.EE = mat[0];
  c.XNU = mat[1];
  c.E1 = mat[2];
  c.nu1 = mat[3];
  c.NN = (int)sizes[0];
  c.NE = (int)sizes[1];
  c.num = (int)sizes[2];
  c.nump = (int)sizes[3];
  c.NODES.assign(3 * (size_t)c.NN, 0.0);
  get(f, c.NODES.data(), c.NODES.size(), path);
  std::vector<int32_t> conn(4 * (size_t)c.NE);
  get(f, conn.data(), conn.size(), path);
  c.NConnect.assign(conn.begin(), conn.end());
  c.BC.assign(6 * (size_t)c.NN, 0.0);
  get(f, c.BC.data(), c.BC.size(), path);
  c.t_bc.assign(24 * (size_t)c.NE, 0.0);
  get(f, c.t_bc.data(), c.t_bc.size(), path);
  c.eigen_point.assign(3 * (size_t)c.num, 0.0);
  get(f, c.eigen_point.data(), c.eigen_point.size(), path);
  c.radius.assign((size_t)c.num, 0.0);
  get(f, c.radius.data(), c.radius.size(), path);
  c.x_p.assign(3 * (size_t)c.nump, 0.0);
  get(f, c.x_p.data(), c.x_p.size(), path);
  c.sig_inf.clear();
  if (sizes[4] == 1) {
    c.sig_inf.assign(6, 0.0);
    get(f, c.sig_inf.data(), 6, path);
  }
}

void configElastic3D_gb300::setUp() {
  if (use_sidecar && sidecar_fresh(*this)) {
    read_sidecar(join(dir, kSidecar), *this);
    from_sidecar = true;
    return;
  }
  Config::setUp();
  from_sidecar = false;
}

}  // namespace ibem_gb300

using namespace ibem_gb300;

namespace {

template <class F>
ibem_status guarded(F&& f) {
  try {
    f();
    return IBEM_OK;
  } catch (const ibem_error& e) {
    ibem::fail(e.status, e.what());
    return e.status;
  } catch (const std::exception& e) {
    ibem::fail(IBEM_ERR_IO, e.what());
    return IBEM_ERR_IO;
  }
}

}  // namespace

extern "C" ibem_status ibem_e3d_sidecar_from_txt(const char* dir) {
  if (!dir) return ibem::fail(IBEM_ERR_ARG, "sidecar_from_txt: null directory");
  return guarded([&] {
    configElastic3D_gb300 c;
    c.dir = dir;
    c.use_sidecar = false;
    c.setUp();
    write_sidecar(join(c.dir, kSidecar), c);
  });
}

extern "C" ibem_status ibem_e3d_sidecar_write(const char* path, const ibem_material* mat, int NN, const double* nodes,
                                              int NE, const int* conn, const double* bc, const double* tbc, int num,
                                              const double* centers, const double* radius, int nump,
                                              const double* points, const double* sig_inf) {
  if (!path || !mat || NN < 0 || NE < 0 || num < 0 || nump < 0 || (NN && (!nodes || !bc)) || (NE && (!conn || !tbc)) ||
      (num && (!centers || !radius)) || (nump && !points))
    return ibem::fail(IBEM_ERR_ARG, "sidecar_write: bad arguments");
  return guarded([&] {
    configElastic3D_gb300 c;
    c.EE = mat->E0;
    c.XNU = mat->nu0;
    c.E1 = mat->E1;
    c.nu1 = mat->nu1;
    c.NN = NN;
    c.NE = NE;
    c.num = num;
    c.nump = nump;
    if (NN) c.NODES.assign(nodes, nodes + 3 * (size_t)NN), c.BC.assign(bc, bc + 6 * (size_t)NN);
    if (NE) c.NConnect.assign(conn, conn + 4 * (size_t)NE), c.t_bc.assign(tbc, tbc + 24 * (size_t)NE);
    if (num) c.eigen_point.assign(centers, centers + 3 * (size_t)num), c.radius.assign(radius, radius + num);
    if (nump) c.x_p.assign(points, points + 3 * (size_t)nump);
    if (sig_inf) c.sig_inf.assign(sig_inf, sig_inf + 6);
    write_sidecar(path, c);
  });
}

extern "C" ibem_status ibem_e3d_case_sizes(const char* dir, int64_t* sizes) {
  if (!dir || !sizes) return ibem::fail(IBEM_ERR_ARG, "case_sizes: bad arguments");
  return guarded([&] {
    configElastic3D_gb300 c;
    c.dir = dir;
    c.setUp();
    sizes[0] = c.NN;
    sizes[1] = c.NE;
    sizes[2] = c.num;
    sizes[3] = c.nump;
    sizes[4] = c.sig_inf.size() == 6 ? 1 : 0;
    sizes[5] = c.from_sidecar ? 1 : 0;
  });
}

extern "C" ibem_status ibem_e3d_read_case(const char* dir, ibem_material* mat, double* nodes, int* conn, double* bc,
                                          double* tbc, double* centers, double* radius, double* points,
                                          double* sig_inf) {
  if (!dir || !mat) return ibem::fail(IBEM_ERR_ARG, "read_case: bad arguments");
  return guarded([&] {
    configElastic3D_gb300 c;
    c.dir = dir;
    c.setUp();
    *mat = c.material();
    auto out = [](const auto& v, auto* p) {
      if (!v.empty()) {
        if (!p) throw ibem_error(IBEM_ERR_ARG, "read_case: missing output array");
        std::memcpy(p, v.data(), sizeof(v[0]) * v.size());
      }
    };
    out(c.NODES, nodes);
    out(c.NConnect, conn);
    out(c.BC, bc);
    out(c.t_bc, tbc);
    out(c.eigen_point, centers);
    out(c.radius, radius);
    out(c.x_p, points);
    if (sig_inf) {
      for (int i = 0; i < 6; ++i) sig_inf[i] = c.sig_inf.size() == 6 ? c.sig_inf[i] : 0.0;
    }
  });
}
