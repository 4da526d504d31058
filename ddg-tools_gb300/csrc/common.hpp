// Shared host-side plumbing of librsgpu: status/error reporting, the context, device buffers.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <thread>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "rsgpu.h"

namespace rsg {

// Bytes the library copied host -> device and device -> host (process-wide; rs_copy_counters).
inline std::atomic<uint64_t> g_h2d_bytes{0}, g_d2h_bytes{0};

// cudaMemcpyAsync of a host <-> device copy, counted.
inline cudaError_t copy_async(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
  if (kind == cudaMemcpyHostToDevice) g_h2d_bytes += bytes;
  else if (kind == cudaMemcpyDeviceToHost) g_d2h_bytes += bytes;
  return cudaMemcpyAsync(dst, src, bytes, kind, s);
}


// An error carrying the RsError kind, the operation word and a detail string
// (RsError::Gpu { operation, detail }, RS/src/gpu/cuda.rs:19-24).
struct Error : std::runtime_error {
  int code;
  std::string kind, operation;
  Error(int c, std::string k, std::string op, const std::string &detail)
      : std::runtime_error(detail), code(c), kind(std::move(k)), operation(std::move(op)) {}
};

[[noreturn]] inline void fail(int code, const char *kind, const char *op, const std::string &d) {
  throw Error(code, kind, op, d);
}

inline void cuda_check(cudaError_t e, const char *op, const char *what) {
  if (e != cudaSuccess)
    fail(RS_GPU, "Gpu", op, std::string(what) + ": " + cudaGetErrorString(e));
}
#define RSG_CUDA(op, call) ::rsg::cuda_check((call), op, #call)

void set_last_error(const Error &e);
void set_last_error_other(int code, const char *what);

// Runs `f`, converting exceptions into a status and the thread's last error.
template <class F>
int guard(F &&f) {
  try {
    f();
    return RS_OK;
  } catch (const Error &e) {
    set_last_error(e);
    return e.code;
  } catch (const std::bad_alloc &) {
    set_last_error_other(RS_INTERNAL, "host allocation failed");
    return RS_INTERNAL;
  } catch (const std::exception &e) {
    set_last_error_other(RS_INTERNAL, e.what());
    return RS_INTERNAL;
  }
}

// A typed device allocation owned by one object (freed on destruction).
template <class T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t count) { alloc(count); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr, o.n = 0; }
  DevBuf &operator=(DevBuf &&o) noexcept {
    if (this != &o) {
      release();
      p = o.p, n = o.n, o.p = nullptr, o.n = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count) {
    release();
    n = count;
    if (count) RSG_CUDA("upload", cudaMalloc(&p, count * sizeof(T)));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr, n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
  void upload(const T *h, size_t count, cudaStream_t s) {
    if (count != n) alloc(count);
    if (count) RSG_CUDA("upload", rsg::copy_async(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void upload(const std::vector<T> &v, cudaStream_t s) { upload(v.data(), v.size(), s); }
  void download(T *h, size_t count, cudaStream_t s) const {
    if (count) RSG_CUDA("product", rsg::copy_async(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
  }
};

}  // namespace rsg

struct rs_ctx {
  // Owners: the caller's handle plus every object built on the context (trees, operators,
  // solvers, flows); the last release destroys it, so handles may be freed in any order.
  std::atomic<int> refs{1};
  int device = 0;
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  int cc_major = 0, cc_minor = 0;
  std::string name;
  std::atomic<int64_t> launches{0};  // kernel launches (host threads may build concurrently)
  // Pinned staging buffer for host <-> device copies of the entry points with host arrays.
  void *pinned = nullptr;
  size_t pinned_bytes = 0;
  void *staging(size_t bytes);
  void use() const;  // makes the context's device current for the calling thread
};

namespace rsg {
rs_ctx *ctx_retain(rs_ctx *ctx);

// f(begin, end) over [0, n) in contiguous chunks on up to 16 host threads (the host set-up
// loops of the trees and blocks). Results that depend on the chunking must not be produced.
template <class Fn>
void parallel_for(size_t n, Fn f, size_t min_chunk = 4096) {
  size_t hw = std::thread::hardware_concurrency();
  size_t t = std::min<size_t>(std::min<size_t>(hw ? hw : 1, 16), (n + min_chunk - 1) / min_chunk);
  if (t <= 1) {
    f((size_t)0, n);
    return;
  }
  std::vector<std::thread> pool;
  for (size_t i = 1; i < t; ++i) pool.emplace_back([&, i] { f(n * i / t, n * (i + 1) / t); });
  f((size_t)0, n / t);
  for (auto &th : pool) th.join();
}
void ctx_release(rs_ctx *ctx);
}  // namespace rsg

// Counts one kernel launch of `ctx` and checks the launch status.
#define RSG_LAUNCHED(ctx, what)                                   \
  do {                                                            \
    (ctx)->launches++;                                            \
    ::rsg::cuda_check(cudaGetLastError(), "launch", what);        \
  } while (0)
