// Per-kernel CUDA-event timing of the entry points (rs_*_profile): when active, every launch
// (or phase; begin/end pairs may nest) is bracketed by two events on the launching stream;
// averages per name.
#pragma once
#include <cuda_runtime.h>

#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "common.hpp"

namespace rsg {

struct Profiler {
  bool active = false;
  struct Rec {
    std::string name;
    cudaEvent_t a, b;
  };
  std::vector<Rec> recs;
  std::vector<std::pair<std::string, cudaEvent_t>> open;  // begun, not yet ended

  void start() {
    clear();
    active = true;
  }
  void begin(cudaStream_t s, const char *name) {
    if (!active) return;
    cudaEvent_t e;
    RSG_CUDA("launch", cudaEventCreate(&e));
    RSG_CUDA("launch", cudaEventRecord(e, s));
    open.push_back({name, e});
  }
  void end(cudaStream_t s) {
    if (!active || open.empty()) return;
    cudaEvent_t e;
    RSG_CUDA("launch", cudaEventCreate(&e));
    RSG_CUDA("launch", cudaEventRecord(e, s));
    recs.push_back({open.back().first, open.back().second, e});
    open.pop_back();
  }
  void stop(cudaStream_t s) {
    active = false;
    RSG_CUDA("launch", cudaStreamSynchronize(s));
  }
  // Average milliseconds per kernel name over `reps` repetitions, in first-seen order.
  void report(char *names, int names_len, double *ms, int max_k, int *n_k, int reps) {
    std::vector<std::string> order;
    std::map<std::string, double> tot;
    for (auto &r : recs) {
      float t = 0.f;
      RSG_CUDA("launch", cudaEventElapsedTime(&t, r.a, r.b));
      if (!tot.count(r.name)) order.push_back(r.name);
      tot[r.name] += t;
    }
    int k = 0, off = 0;
    for (auto &n : order) {
      if (k >= max_k || off + (int)n.size() + 1 > names_len) break;
      std::memcpy(names + off, n.c_str(), n.size() + 1);
      off += (int)n.size() + 1;
      ms[k++] = tot[n] / (reps > 0 ? reps : 1);
    }
    if (off < names_len) names[off] = 0;
    *n_k = k;
    clear();
  }
  void clear() {
    for (auto &r : recs) cudaEventDestroy(r.a), cudaEventDestroy(r.b);
    recs.clear();
    for (auto &p : open) cudaEventDestroy(p.second);
    open.clear();
  }
  ~Profiler() { clear(); }
};

}  // namespace rsg
