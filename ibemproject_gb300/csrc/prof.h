// Phase profiler of libibem_gb300.so: CUDA events recorded on the launching stream around
// each instrumented phase while profiling is enabled (ibem_prof_enable); read back with
// ibem_prof_report.  Disabled, a Scope costs one branch.
#pragma once
#include <cuda_runtime.h>

namespace ibem {

enum ProfCat {
  PROF_PAIR = 0, PROF_FIELD, PROF_BEM, PROF_EQUIL, PROF_PANEL, PROF_LASWP, PROF_TRSM_SMALL,
  PROF_GEMM_TC, PROF_GEMM_SPLIT, PROF_GEMM_SIMT, PROF_TRSV, PROF_MATVEC, PROF_GMRES_OTHER, PROF_MF_F32,
  PROF_MF_F64, PROF_PRECOND, PROF_MF_DF, PROF_GNN_FWD, PROF_EDGE, PROF_KNN, PROF_NCAT
};

bool prof_on();
void prof_push(int cat, cudaEvent_t a, cudaEvent_t b, double flops);
cudaEvent_t prof_event();

struct ProfScope {
  int cat;
  cudaStream_t st;
  double flops;
  cudaEvent_t a = nullptr;
  ProfScope(int c, cudaStream_t s, double f = 0) : cat(c), st(s), flops(f) {
    if (prof_on()) {
      a = prof_event();
      cudaEventRecord(a, st);
    }
  }
  ~ProfScope() {
    if (a) {
      cudaEvent_t b = prof_event();
      cudaEventRecord(b, st);
      prof_push(cat, a, b, flops);
    }
  }
};

}  // namespace ibem
