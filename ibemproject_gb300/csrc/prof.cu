// Phase profiler (see prof.h).
#include <algorithm>
#include <atomic>
#include <cstring>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "ibem_internal.h"
#include "prof.h"

namespace ibem {
namespace {
const char* kNames[PROF_NCAT] = {"pair_blocks", "field", "bem", "equilibrate", "panel", "laswp", "trsm_small",
                                 "gemm_tc", "gemm_split", "gemm_simt", "trsv", "matvec", "gmres_other",
                                 "mf_f32", "mf_f64", "precond_setup", "mf_df",
                                 "gnn_forward", "edge_blocks", "knn"};
std::atomic<bool> g_on{false};
std::mutex g_mu;
struct Rec {
  int cat;
  cudaEvent_t a, b;
  double flops;
};
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;
}  // namespace

bool prof_on() { return g_on.load(std::memory_order_relaxed); }

cudaEvent_t prof_event() {
  std::lock_guard<std::mutex> l(g_mu);
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void prof_push(int cat, cudaEvent_t a, cudaEvent_t b, double flops) {
  std::lock_guard<std::mutex> l(g_mu);
  g_recs.push_back({cat, a, b, flops});
}

}  // namespace ibem

using namespace ibem;

extern "C" void ibem_prof_enable(int on) {
  std::lock_guard<std::mutex> l(g_mu);
  for (auto& r : g_recs) {
    g_pool.push_back(r.a);
    g_pool.push_back(r.b);
  }
  g_recs.clear();
  g_on.store(on != 0);
}

// JSON object {"phase": {"launches": n, "ms": t, "flops": f}, ...} of everything recorded
// since the last ibem_prof_enable; synchronises the recorded events.  Returns the length
// written (truncated to cap - 1).
extern "C" int ibem_prof_report(char* buf, int cap) {
  std::lock_guard<std::mutex> l(g_mu);
  double ms[PROF_NCAT] = {0}, fl[PROF_NCAT] = {0};
  long long n[PROF_NCAT] = {0};
  for (auto& r : g_recs) {
    cudaEventSynchronize(r.b);
    float t = 0;
    if (cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
      ms[r.cat] += t;
      fl[r.cat] += r.flops;
      n[r.cat] += 1;
    }
  }
  std::string s = "{";
  bool first = true;
  for (int c = 0; c < PROF_NCAT; ++c) {
    if (!n[c]) continue;
    char tmp[160];
    std::snprintf(tmp, sizeof tmp, "%s\"%s\": {\"launches\": %lld, \"ms\": %.4f, \"flops\": %.6e}", first ? "" : ", ",
                  kNames[c], n[c], ms[c], fl[c]);
    s += tmp;
    first = false;
  }
  s += "}";
  if (buf && cap > 0) {
    const int k = (int)std::min<size_t>(s.size(), (size_t)cap - 1);
    std::memcpy(buf, s.data(), k);
    buf[k] = 0;
  }
  return (int)s.size();
}
