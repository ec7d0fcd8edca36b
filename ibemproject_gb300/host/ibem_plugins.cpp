// Implementation of the host-side plugins (see ibem_plugins.h) and of the whole-pipeline
// C ABI entry points ibem_e3d_run_host / ibem_e3d_run_dir.
#include "ibem_plugins.h"

#include "../csrc/ibem_internal.h"

#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>

namespace ibem_gb300 {

static void check(ibem_status s, const char* where) {
  if (s != IBEM_OK) throw ibem_error(s, std::string(where) + ": " + ibem_last_error());
}
static void check_cuda(cudaError_t e, const char* where) {
  if (e != cudaSuccess) throw ibem_error(IBEM_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

template <typename T>
void DeviceArray<T>::alloc(size_t count) {
  reset();
  if (count == 0) return;
  check_cuda(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
  n = count;
}
template <typename T>
void DeviceArray<T>::upload(const std::vector<T>& h, cudaStream_t st) {
  alloc(h.size());
  if (!h.empty()) check_cuda(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st), "upload");
}
template <typename T>
void DeviceArray<T>::download(std::vector<T>& h, cudaStream_t st) const {
  h.resize(n);
  if (n) check_cuda(cudaMemcpyAsync(h.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost, st), "download");
  check_cuda(cudaStreamSynchronize(st), "download sync");
}
template struct DeviceArray<double>;
template struct DeviceArray<int>;

static configElastic3D_gb300& as_e3d(Config& c) {
  // the reference uses dynamic_cast<configElastic3D&> and throws std::bad_cast
  return dynamic_cast<configElastic3D_gb300&>(c);
}

// ------------------------------------------------------------------ input files
static std::string path_of(const configElastic3D_gb300& c, const std::string& f) {
  return c.dir.empty() ? f : c.dir + "/" + f;
}

static std::ifstream open_in(const std::string& p) {
  std::ifstream f(p, std::ios::in | std::ios::binary);
  if (!f) throw ibem_error(IBEM_ERR_IO, "cannot open " + p);
  return f;
}

void configElastic3D_gb300::Readparticle_num() {  // configElastic3D.h:76-82
  std::ifstream f = open_in(path_of(*this, particleInput));
  if (!(f >> num)) throw ibem_error(IBEM_ERR_IO, "position.txt: particle count");
}

void configElastic3D_gb300::Readpartical_info() {  // configElastic3D.cpp:106-128
  std::ifstream f = open_in(path_of(*this, particleInput));
  f >> num >> E1 >> nu1;
  eigen_point.assign(3 * (size_t)num, 0.0);
  radius.assign(num, 0.0);
  for (int k = 0; k < num; ++k)
    if (!(f >> eigen_point[3 * k] >> eigen_point[3 * k + 1] >> eigen_point[3 * k + 2] >> radius[k]))
      throw ibem_error(IBEM_ERR_IO, "position.txt: truncated particle list");
}

static std::string strip_cr(std::string s) {
  while (!s.empty() && (s.back() == '\r' || s.back() == '\n')) s.pop_back();
  return s;
}

void configElastic3D_gb300::ReadBEM_num() {  // configElastic3D.h:86-112
  std::ifstream f = open_in(path_of(*this, bemInput));
  std::string t;
  std::getline(f, t);
  std::getline(f, t);
  EE = std::stod(strip_cr(t));
  std::getline(f, t);
  XNU = std::stod(strip_cr(t));
  std::getline(f, t);
  NN = std::stoi(strip_cr(t));
  std::getline(f, t);
  NE = std::stoi(strip_cr(t));
}

void configElastic3D_gb300::ReadBEM_info() {  // configElastic3D.cpp:32-105
  std::ifstream f = open_in(path_of(*this, bemInput));
  std::string t;
  for (int i = 0; i < 5; ++i) std::getline(f, t);
  NODES.assign(3 * (size_t)NN, 0.0);
  NConnect.assign(4 * (size_t)NE, 0);
  BC.assign(6 * (size_t)NN, 0.0);
  t_bc.assign(24 * (size_t)NE, 0.0);
  bool ok = true;
  for (auto& v : NODES) ok = ok && (f >> v);
  for (auto& v : NConnect) ok = ok && (f >> v);
  for (auto& v : BC) ok = ok && (f >> v);
  for (auto& v : t_bc) ok = ok && (f >> v);
  if (!ok) throw ibem_error(IBEM_ERR_IO, "BEM.txt: truncated");
  // boundary-free cases carry their remote stress in farfield.txt (no reference counterpart)
  std::ifstream ff(path_of(*this, "farfield.txt"));
  sig_inf.clear();
  if (ff) {
    sig_inf.assign(6, 0.0);
    for (auto& v : sig_inf) ff >> v;
  }
}

void configElastic3D_gb300::ReadPostProcess_info() {  // configElastic3D.h:116-129
  std::ifstream f = open_in(path_of(*this, postProcessInput));
  f >> nump;
  x_p.assign(3 * (size_t)nump, 0.0);
  for (auto& v : x_p)
    if (!(f >> v)) throw ibem_error(IBEM_ERR_IO, "postprocess.txt: truncated");
}

void configElastic3D_gb300::upload() {
  if (!stream) check_cuda(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
  if (ibem_layout_size(layout) < 0) throw ibem_error(IBEM_ERR_ARG, "unsupported layout");
  d_nodes.upload(NODES, stream);
  d_conn.upload(NConnect, stream);
  d_bc.upload(BC, stream);
  d_tbc.upload(t_bc, stream);
  d_cen.upload(eigen_point, stream);
  d_rad.upload(radius, stream);
  d_pts.upload(x_p, stream);
  const int64_t N = n_unknowns();
  HMAT.alloc((size_t)N * N);
  check_cuda(cudaMemsetAsync(HMAT.p, 0, sizeof(double) * (size_t)N * N, stream), "HMAT zero");
  if (NE > 0) {
    GMAT.alloc((size_t)N * 12 * NE);
    check_cuda(cudaMemsetAsync(GMAT.p, 0, sizeof(double) * GMAT.n, stream), "GMAT zero");
  }
  b.alloc(N);
  X.alloc(N);
}

// ------------------------------------------------------------------ integrator
void integratorElastic3D_gb300::addFieldToBEM(Config& c_) {
  auto& c = as_e3d(c_);
  if (c.NE == 0) return;
  const ibem_material m = c.material();
  const int64_t N = c.n_unknowns();
  check(ibem_e3d_node_blocks(c.d_nodes.p, c.NN, c.d_cen.p, c.d_rad.p, c.num, &m, c.layout, c.HMAT.p, N, 0,
                             3 * (int64_t)c.NN, c.stream),
        "addFieldToBEM");
}
void integratorElastic3D_gb300::addFluxEquivalentInclusion(Config& c_) {
  auto& c = as_e3d(c_);
  const ibem_material m = c.material();
  const int64_t N = c.n_unknowns(), o = 3 * (int64_t)c.NN;
  check(ibem_e3d_pair_blocks(c.d_cen.p, c.d_rad.p, c.num, &m, c.layout, c.HMAT.p, N, o, o, c.stream),
        "addFluxEquivalentInclusion");
}
void integratorElastic3D_gb300::addFluxEquivalentFirstOrderInclusion(Config& c_) { (void)as_e3d(c_); }
void integratorElastic3D_gb300::addFluxEquivalentSecondOrderInclusion(Config& c_) { (void)as_e3d(c_); }

// ------------------------------------------------------------------ BEM builder
void BEMBuilderElastic3D_gb300::addBEM(Config& c_) {
  auto& c = as_e3d(c_);
  if (c.NE == 0) return;
  const ibem_material m = c.material();
  const int64_t N = c.n_unknowns();
  check(ibem_e3d_bem_hg(c.d_nodes.p, c.NN, c.d_conn.p, c.NE, &m, c.HMAT.p, N, 0, 0, c.GMAT.p, N, 0, 0, c.stream),
        "addBEM");
}
void BEMBuilderElastic3D_gb300::addFluxEquivalentBEM(Config& c_) {
  auto& c = as_e3d(c_);
  if (c.NE == 0) return;
  const ibem_material m = c.material();
  const int64_t N = c.n_unknowns();
  check(ibem_e3d_bem_to_incl(c.d_nodes.p, c.NN, c.d_conn.p, c.NE, c.d_cen.p, c.num, &m, c.layout, c.HMAT.p, N, 0,
                             c.GMAT.p, N, 0, 3 * (int64_t)c.NN, c.stream),
        "addFluxEquivalentBEM");
}
void BEMBuilderElastic3D_gb300::addFluxEquivalentFirstOrderBEM(Config& c_) { (void)as_e3d(c_); }
void BEMBuilderElastic3D_gb300::addFluxEquivalentSecondOrderBEM(Config& c_) { (void)as_e3d(c_); }

void BEMBuilderElastic3D_gb300::ApplyBC(Config& c_) {
  auto& c = as_e3d(c_);
  const int64_t N = c.n_unknowns();
  if (c.NE == 0) {
    // no boundary: the equivalence rows are the whole system, loaded by the remote stress
    if (c.sig_inf.size() != 6) throw ibem_error(IBEM_ERR_ARG, "boundary-free case without a far-field stress");
    const ibem_material m = c.material();
    check(ibem_e3d_farfield_rhs(c.num, &m, c.layout, c.sig_inf.data(), c.b.p, c.stream), "ApplyBC");
    std::swap(c.A.p, c.HMAT.p);
    std::swap(c.A.n, c.HMAT.n);
    c.a_is_hmat = true;
    return;
  }
  c.ucol.assign(3 * (size_t)c.NN, -1);
  c.tcol.assign(12 * (size_t)c.NE, -1);
  check(ibem_e3d_bc_plan(c.NN, c.NE, c.NConnect.data(), c.BC.data(), c.t_bc.data(), c.ucol.data(), c.tcol.data()),
        "ApplyBC plan");
  c.d_ucol.upload(c.ucol, c.stream);
  c.d_tcol.upload(c.tcol, c.stream);
  c.A.alloc((size_t)N * N);
  check(ibem_e3d_apply_bc(c.NN, c.NE, N, c.d_ucol.p, c.d_tcol.p, c.d_bc.p, c.d_tbc.p, c.HMAT.p, N, c.GMAT.p, N, c.A.p,
                          N, c.b.p, c.stream),
        "ApplyBC");
  check_cuda(cudaStreamSynchronize(c.stream), "ApplyBC sync");
  // the reference releases HMAT and GMAT here (BEMBuilderElastic3D.cpp:2033-2034)
  c.HMAT.reset();
  c.GMAT.reset();
}

void BEMBuilderElastic3D_gb300::getUTVector(Config& c_) {
  auto& c = as_e3d(c_);
  const int64_t N = c.n_unknowns();
  c.U.alloc(N);
  if (c.NE == 0) {
    check_cuda(cudaMemcpyAsync(c.U.p, c.X.p, sizeof(double) * N, cudaMemcpyDeviceToDevice, c.stream), "getUTVector");
    return;
  }
  c.T.alloc(12 * (size_t)c.NE);
  check(ibem_e3d_get_ut(c.NN, c.NE, N, c.d_ucol.p, c.d_tcol.p, c.d_bc.p, c.d_tbc.p, c.X.p, c.U.p, c.T.p, c.stream),
        "getUTVector");
}

// ------------------------------------------------------------------ solver
void systemSolverElastic3D_gb300::solve(Config& c_) {
  auto& c = as_e3d(c_);
  const int64_t N = c.n_unknowns();
  check(ibem_e3d_solve(c.form, N, c.A.p, N, c.b.p, c.X.p, c.tol, &c.report, c.stream), "solve");
}

// ------------------------------------------------------------------ post-processor
void postProcessorElastic3D_gb300::getFlux(Config& c_) {
  auto& c = as_e3d(c_);
  const ibem_material m = c.material();
  c.stress.alloc(6 * (size_t)c.nump);
  const double* E = c.U.p + 3 * (int64_t)c.NN;
  check(ibem_e3d_field_form(c.form, c.d_pts.p, c.nump, c.d_cen.p, c.d_rad.p, c.num, &m, c.layout, E, c.d_nodes.p,
                            c.NN, c.d_conn.p, c.NE, c.U.p, c.T.p, c.sig_inf.empty() ? nullptr : c.sig_inf.data(),
                            c.stress.p, c.stream),
        "getFlux");
  c.stress.download(c.s_pt, c.stream);
  if (!write_file) return;
  std::ofstream f(path_of(c, "stress.txt"));  // postProcessorElastic3D.cpp:578-585
  if (!f) throw ibem_error(IBEM_ERR_IO, "cannot write stress.txt");
  for (int k = 0; k < c.nump; ++k) {
    for (int i = 0; i < 6; ++i) f << std::scientific << c.s_pt[6 * (size_t)k + i] << (i < 5 ? " " : "");
    f << "\n";
  }
}

// ------------------------------------------------------------------ registry / runner
std::shared_ptr<integrator> getIntegrator(const std::string& t) {
  if (t == "integratorElastic3D_gb300") return std::make_shared<integratorElastic3D_gb300>();
  return nullptr;
}
std::shared_ptr<BEMBuilder> getBEMBuilder(const std::string& t) {
  if (t == "BEMBuilderElastic3D_gb300") return std::make_shared<BEMBuilderElastic3D_gb300>();
  return nullptr;
}
std::shared_ptr<systemSolver> getSystemSolver(const std::string& t) {
  if (t == "systemSolverElastic3D_gb300") return std::make_shared<systemSolverElastic3D_gb300>();
  return nullptr;
}
std::shared_ptr<postProcessor> getPostProcessor(const std::string& t) {
  if (t == "postProcessorElastic3D_gb300") return std::make_shared<postProcessorElastic3D_gb300>();
  return nullptr;
}

void run_services(configElastic3D_gb300& cfg, bool read_files, bool write_stress) {
  // preprocessService (preprocessService.h:35-37)
  if (read_files) cfg.setUp();
  cfg.upload();
  {  // iBEMSystemService::run (iBEMSystemService.h:58-67)
    auto B = getBEMBuilder(cfg.getbembuilder());
    auto I = getIntegrator(cfg.getintegrator());
    B->addBEM(cfg);
    I->addFieldToBEM(cfg);
    I->addFluxEquivalentInclusion(cfg);
    I->addFluxEquivalentFirstOrderInclusion(cfg);
    I->addFluxEquivalentSecondOrderInclusion(cfg);
    B->addFluxEquivalentBEM(cfg);
    B->addFluxEquivalentFirstOrderBEM(cfg);
    B->addFluxEquivalentSecondOrderBEM(cfg);
  }
  {  // systemSolverService::run (systemSolverService.h:41-45)
    auto B = getBEMBuilder(cfg.getbembuilder());
    auto S = getSystemSolver(cfg.getsystemsolver());
    B->ApplyBC(cfg);
    S->solve(cfg);
    B->getUTVector(cfg);
  }
  {  // postprocessService::run (postprocessService.h:40-43)
    auto P = getPostProcessor(cfg.getpostprocessor());
    auto* pp = dynamic_cast<postProcessorElastic3D_gb300*>(P.get());
    if (pp) pp->write_file = write_stress;
    P->getField(cfg);
    P->getFlux(cfg);
  }
}

}  // namespace ibem_gb300

using namespace ibem_gb300;

extern "C" ibem_status ibem_e3d_run_host(int layout, ibem_solver_form form, const ibem_material* mat, int NN,
                                         const double* nodes, int NE, const int* conn, const double* bc,
                                         const double* tbc, int num, const double* centers, const double* radius,
                                         int nump, const double* points, const double* sig_inf, double tol,
                                         double* X, double* stress, ibem_solve_report* report) {
  try {
    if (!mat || NN < 0 || NE < 0 || num < 0 || nump < 0) throw ibem_error(IBEM_ERR_ARG, "run_host: bad sizes");
    configElastic3D_gb300 c;
    c.layout = layout;
    c.form = form;
    c.tol = tol;
    c.NN = NN;
    c.NE = NE;
    c.num = num;
    c.nump = nump;
    c.EE = mat->E0;
    c.XNU = mat->nu0;
    c.E1 = mat->E1;
    c.nu1 = mat->nu1;
    c.NODES.assign(nodes, nodes + 3 * (size_t)NN);
    c.NConnect.assign(conn, conn + 4 * (size_t)NE);
    c.BC.assign(bc, bc + 6 * (size_t)NN);
    c.t_bc.assign(tbc, tbc + 24 * (size_t)NE);
    c.eigen_point.assign(centers, centers + 3 * (size_t)num);
    c.radius.assign(radius, radius + num);
    c.x_p.assign(points, points + 3 * (size_t)nump);
    if (sig_inf) c.sig_inf.assign(sig_inf, sig_inf + 6);
    run_services(c, false, false);
    std::vector<double> hx;
    c.X.download(hx, c.stream);
    if (X) std::memcpy(X, hx.data(), sizeof(double) * hx.size());
    if (stress) std::memcpy(stress, c.s_pt.data(), sizeof(double) * c.s_pt.size());
    if (report) *report = c.report;
    cudaStreamDestroy(c.stream);
    return IBEM_OK;
  } catch (const ibem_error& e) {
    ibem::fail(e.status, e.what());
    return e.status;
  } catch (const std::exception& e) {
    ibem::fail(IBEM_ERR_ARG, e.what());
    return IBEM_ERR_ARG;
  }
}

extern "C" ibem_status ibem_e3d_run_dir(const char* dir, int layout, ibem_solver_form form, double tol,
                                        ibem_solve_report* report) {
  try {
    if (!dir) throw ibem_error(IBEM_ERR_ARG, "run_dir: null directory");
    configElastic3D_gb300 c;
    c.dir = dir;
    c.layout = layout;
    c.form = form;
    c.tol = tol;
    run_services(c, true, true);
    if (report) *report = c.report;
    cudaStreamDestroy(c.stream);
    return IBEM_OK;
  } catch (const ibem_error& e) {
    ibem::fail(e.status, e.what());
    return e.status;
  } catch (const std::exception& e) {
    ibem::fail(IBEM_ERR_IO, e.what());
    return IBEM_ERR_IO;
  }
}
