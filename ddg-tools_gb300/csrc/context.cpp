// Context, device queries and the thread-local last error of the C ABI.
// Replaces GpuContext / device selection of RS/src/gpu/mod.rs:36-127 and cuda.rs:100-178.
#include "common.hpp"

namespace rsg {

namespace {
thread_local std::string t_detail, t_operation, t_kind;
}

void set_last_error(const Error &e) {
  t_detail = e.what();
  t_operation = e.operation;
  t_kind = e.kind;
}

void set_last_error_other(int code, const char *what) {
  t_detail = what;
  t_operation = "internal";
  t_kind = code == RS_GPU ? "Gpu" : "Internal";
}

const char *last_detail() { return t_detail.c_str(); }
const char *last_operation() { return t_operation.c_str(); }
const char *last_kind() { return t_kind.c_str(); }

}  // namespace rsg

void *rs_ctx::staging(size_t bytes) {
  if (bytes > pinned_bytes) {
    if (pinned) cudaFreeHost(pinned);
    pinned = nullptr;
    pinned_bytes = 0;
    size_t want = bytes + bytes / 4;
    RSG_CUDA("upload", cudaMallocHost(&pinned, want));
    pinned_bytes = want;
  }
  return pinned;
}

void rs_ctx::use() const { RSG_CUDA("context", cudaSetDevice(device)); }

rs_ctx *rsg::ctx_retain(rs_ctx *ctx) {
  ctx->refs.fetch_add(1);
  return ctx;
}

void rsg::ctx_release(rs_ctx *ctx) {
  if (!ctx || ctx->refs.fetch_sub(1) != 1) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) {
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
  }
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  delete ctx;
}

extern "C" {

const char *rs_last_error(void) { return rsg::last_detail(); }
const char *rs_last_error_operation(void) { return rsg::last_operation(); }
const char *rs_last_error_kind(void) { return rsg::last_kind(); }

int rs_device_info(int ordinal, char *name, int name_len, int *cc_major, int *cc_minor,
                   uint64_t *memory_bytes) {
  return rsg::guard([&] {
    int n = 0;
    RSG_CUDA("context", cudaGetDeviceCount(&n));
    if (ordinal < 0 || ordinal >= n)
      rsg::fail(RS_INVALID_OPTION, "InvalidOption", "context", "cuda_ordinal " + std::to_string(ordinal) +
                " is not below the device count " + std::to_string(n));
    cudaDeviceProp p;
    RSG_CUDA("context", cudaGetDeviceProperties(&p, ordinal));
    if (name && name_len > 0) {
      std::strncpy(name, p.name, (size_t)name_len - 1);
      name[name_len - 1] = 0;
    }
    *cc_major = p.major, *cc_minor = p.minor;
    *memory_bytes = (uint64_t)p.totalGlobalMem;
  });
}

int rs_device_count(int *count) {
  return rsg::guard([&] {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) {
      cudaGetLastError();
      n = 0;
    } else {
      RSG_CUDA("context", e);
    }
    *count = n;
  });
}

int rs_ctx_create(int ordinal, rs_ctx **out) {
  *out = nullptr;
  return rsg::guard([&] {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
      cudaGetLastError();
      rsg::fail(RS_GPU, "Gpu", "context", "no CUDA device is available");
    }
    if (ordinal < 0 || ordinal >= n)
      rsg::fail(RS_GPU, "Gpu", "context", "device ordinal " + std::to_string(ordinal) + " of " +
                                              std::to_string(n) + " devices");
    auto *c = new rs_ctx();
    c->device = ordinal;
    try {
      c->use();
      cudaDeviceProp prop;
      RSG_CUDA("context", cudaGetDeviceProperties(&prop, ordinal));
      c->name = prop.name;
      c->sm_count = prop.multiProcessorCount;
      c->cc_major = prop.major;
      c->cc_minor = prop.minor;
      if (prop.major < 10)
        rsg::fail(RS_GPU, "Gpu", "context",
                  "librsgpu is built for sm_103a (GB300); device is sm_" +
                      std::to_string(prop.major) + std::to_string(prop.minor));
      RSG_CUDA("context", cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    } catch (...) {
      delete c;
      throw;
    }
    *out = c;
  });
}

void rs_ctx_free(rs_ctx *ctx) { rsg::ctx_release(ctx); }

int rs_ctx_stream(rs_ctx *ctx, void **stream) {
  return rsg::guard([&] { *stream = (void *)ctx->stream; });
}

int rs_copy_counters(uint64_t *h2d_bytes, uint64_t *d2h_bytes) {
  return rsg::guard([&] {
    if (h2d_bytes) *h2d_bytes = rsg::g_h2d_bytes.load();
    if (d2h_bytes) *d2h_bytes = rsg::g_d2h_bytes.load();
  });
}

int rs_ctx_synchronize(rs_ctx *ctx) {
  return rsg::guard([&] {
    ctx->use();
    RSG_CUDA("product", cudaStreamSynchronize(ctx->stream));
  });
}

int rs_ctx_info(rs_ctx *ctx, char *name, int name_len, int *sm_count, int *cc_major,
                int *cc_minor) {
  return rsg::guard([&] {
    if (name && name_len > 0) {
      std::strncpy(name, ctx->name.c_str(), (size_t)name_len - 1);
      name[name_len - 1] = 0;
    }
    if (sm_count) *sm_count = ctx->sm_count;
    if (cc_major) *cc_major = ctx->cc_major;
    if (cc_minor) *cc_minor = ctx->cc_minor;
  });
}

int rs_ctx_launch_count(rs_ctx *ctx, int64_t *count) {
  return rsg::guard([&] { *count = ctx->launches; });
}

}  // extern "C"
