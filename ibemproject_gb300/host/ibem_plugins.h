// Host-side mirror of the reference's plugin architecture for the 3D elastic family,
// backed by the sm_103a kernels of libibem_gb300.so.
//
//   reference                                   here
//   Config (Config.h:31-55)                     ibem_gb300::Config
//   configElastic3D (configElastic3D.h:41-148)  ibem_gb300::configElastic3D_gb300
//   integrator / integratorElastic3D            ibem_gb300::integrator / integratorElastic3D_gb300
//   BEMBuilder / BEMBuilderElastic3D            ibem_gb300::BEMBuilder / BEMBuilderElastic3D_gb300
//   systemSolver / systemSolverElastic3D        ibem_gb300::systemSolver / systemSolverElastic3D_gb300
//   postProcessor / postProcessorElastic3D      ibem_gb300::postProcessor / postProcessorElastic3D_gb300
//   classFinder.h getIntegrator(...) etc.       ibem_gb300::getIntegrator(...) etc.
//   ibemRunner::run (ibemRunner.cpp:37-133)     ibem_gb300::run_services
//
// Method names, call order and the meaning of every matrix follow the reference; the
// matrices live in device memory (column-major, as Eigen's MatrixXd) and only the
// stresses come back to the host (s_pt), as getFlux leaves them in the reference.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ibem_gb300.h"

namespace ibem_gb300 {

// Raised by every plugin method on failure (the reference's methods return void and
// only throw std::bad_cast; here a failed kernel or bad input is reported too).
struct ibem_error : std::runtime_error {
  ibem_status status;
  ibem_error(ibem_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

template <typename T>
struct DeviceArray {
  T* p = nullptr;
  size_t n = 0;
  DeviceArray() = default;
  DeviceArray(const DeviceArray&) = delete;
  DeviceArray& operator=(const DeviceArray&) = delete;
  ~DeviceArray() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count);
  void upload(const std::vector<T>& h, cudaStream_t st);
  void download(std::vector<T>& h, cudaStream_t st) const;
};

class Config {
 public:
  virtual ~Config() = default;
  virtual void setUp() {
    Readparticle_num();
    Readpartical_info();
    ReadBEM_num();
    ReadBEM_info();
    ReadPostProcess_info();
  }
  virtual void Readparticle_num() {}
  virtual void Readpartical_info() {}
  virtual void ReadBEM_num() {}
  virtual void ReadBEM_info() {}
  virtual void ReadPostProcess_info() {}
  virtual std::string getbembuilder() { return " "; }
  virtual std::string getintegrator() { return " "; }
  virtual std::string getpostprocessor() { return " "; }
  virtual std::string getsystemsolver() { return " "; }
};

class configElastic3D_gb300 : public Config {
 public:
  // inputs (host, row-major)
  std::string dir = ".";
  std::string particleInput = "position.txt", bemInput = "BEM.txt", postProcessInput = "postprocess.txt";
  int NN = 0, NE = 0, num = 0, nump = 0;
  double EE = 0, XNU = 0, E1 = 0, nu1 = 0;
  std::vector<double> NODES, BC, t_bc, eigen_point, radius, x_p, sig_inf;
  std::vector<int> NConnect;
  // options (no reference counterpart: the reference always uses 78 and fullPivLu)
  int layout = 78;
  ibem_solver_form form = IBEM_SOLVE_FP64;
  double tol = 1e-12;

  // device state
  cudaStream_t stream = nullptr;
  DeviceArray<double> d_nodes, d_bc, d_tbc, d_cen, d_rad, d_pts;
  DeviceArray<int> d_conn, d_ucol, d_tcol;
  DeviceArray<double> HMAT, GMAT, A, b, X, U, T, stress;
  std::vector<int> ucol, tcol;
  bool a_is_hmat = false;  // boundary-free case: the system matrix is HMAT itself
  ibem_solve_report report{};
  std::vector<double> s_pt;  // nump x 6 stresses (getFlux)

  int64_t n_unknowns() const { return 3 * (int64_t)NN + (int64_t)layout * num; }
  ibem_material material() const { return ibem_material{EE, XNU, E1, nu1}; }

  // the text inputs, or the directory's binary side-car case.ibemb when it is at least as
  // new as each of them (host/sidecar.cpp)
  void setUp() override;
  bool use_sidecar = true;
  bool from_sidecar = false;
  void Readparticle_num() override;
  void Readpartical_info() override;
  void ReadBEM_num() override;
  void ReadBEM_info() override;
  void ReadPostProcess_info() override;
  // copies inputs to the device and allocates HMAT/GMAT (the reference allocates them in
  // ReadBEM_info, configElastic3D.cpp:95-101)
  void upload();

  std::string getbembuilder() override { return "BEMBuilderElastic3D_gb300"; }
  std::string getintegrator() override { return "integratorElastic3D_gb300"; }
  std::string getsystemsolver() override { return "systemSolverElastic3D_gb300"; }
  std::string getpostprocessor() override { return "postProcessorElastic3D_gb300"; }
};

class integrator {
 public:
  virtual ~integrator() = default;
  virtual void addFieldToBEM(Config&) = 0;
  virtual void addFluxEquivalentInclusion(Config&) = 0;
  virtual void addFluxEquivalentFirstOrderInclusion(Config&) = 0;
  virtual void addFluxEquivalentSecondOrderInclusion(Config&) = 0;
};

class BEMBuilder {
 public:
  virtual ~BEMBuilder() = default;
  virtual void addBEM(Config&) = 0;
  virtual void addFluxEquivalentBEM(Config&) = 0;
  virtual void addFluxEquivalentFirstOrderBEM(Config&) = 0;
  virtual void addFluxEquivalentSecondOrderBEM(Config&) = 0;
  virtual void ApplyBC(Config&) = 0;
  virtual void getUTVector(Config&) = 0;
};

class systemSolver {
 public:
  virtual ~systemSolver() = default;
  virtual void solve(Config&) = 0;
};

class postProcessor {
 public:
  virtual ~postProcessor() = default;
  virtual void getFlux(Config&) = 0;
  virtual void getField(Config&) = 0;
};

class integratorElastic3D_gb300 : public integrator {
 public:
  void addFieldToBEM(Config&) override;
  // all orders of the layout are written by the first call (one kernel family covers the
  // three reference methods); the first/second-order calls only validate the config
  void addFluxEquivalentInclusion(Config&) override;
  void addFluxEquivalentFirstOrderInclusion(Config&) override;
  void addFluxEquivalentSecondOrderInclusion(Config&) override;
};

class BEMBuilderElastic3D_gb300 : public BEMBuilder {
 public:
  void addBEM(Config&) override;
  void addFluxEquivalentBEM(Config&) override;  // all orders, see integratorElastic3D_gb300
  void addFluxEquivalentFirstOrderBEM(Config&) override;
  void addFluxEquivalentSecondOrderBEM(Config&) override;
  void ApplyBC(Config&) override;
  void getUTVector(Config&) override;
};

class systemSolverElastic3D_gb300 : public systemSolver {
 public:
  void solve(Config&) override;
};

class postProcessorElastic3D_gb300 : public postProcessor {
 public:
  void getFlux(Config&) override;
  void getField(Config&) override {}  // empty in the reference (postProcessorElastic3D.cpp:590-592)
  bool write_file = true;             // stress.txt in config.dir
};

std::shared_ptr<integrator> getIntegrator(const std::string& type);
std::shared_ptr<BEMBuilder> getBEMBuilder(const std::string& type);
std::shared_ptr<systemSolver> getSystemSolver(const std::string& type);
std::shared_ptr<postProcessor> getPostProcessor(const std::string& type);

// preprocess -> iBEMSystem -> systemSolver -> postprocess, each service with fresh plugin
// objects from the registry (serviceWrapper.h:41-47), in the reference's order.
void run_services(configElastic3D_gb300& cfg, bool read_files, bool write_stress);

}  // namespace ibem_gb300
