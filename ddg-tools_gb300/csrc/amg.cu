// Device V-cycle of the smoothed-aggregation multigrid (see amg.hpp). Vectors hold C
// interleaved columns per row (x[row * C + c]); every kernel is one thread per row.
#include "amg.hpp"

namespace rsg {

namespace {

inline unsigned nblk(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// y = A x (accumulate: y += A x); C columns per row, a compile-time width so that the
// accumulators stay in registers.
template <bool ACC, int C>
__global__ void spmv_c_kernel(int n, const int *__restrict__ ap, const int *__restrict__ ac,
                              const double *__restrict__ av, const double *__restrict__ x,
                              double *__restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc[C];
#pragma unroll
  for (int c = 0; c < C; ++c) acc[c] = ACC ? y[(size_t)i * C + c] : 0.0;
  for (int p = ap[i]; p < ap[i + 1]; ++p) {
    double a = av[p];
    const double *xr = x + (size_t)ac[p] * C;
#pragma unroll
    for (int c = 0; c < C; ++c) acc[c] = fma(a, xr[c], acc[c]);
  }
#pragma unroll
  for (int c = 0; c < C; ++c) y[(size_t)i * C + c] = acc[c];
}

// out = x + dinv (b - A x); x = null means x = 0 (out = dinv b).
template <int C>
__global__ void jacobi_kernel(int n, const int *__restrict__ ap, const int *__restrict__ ac,
                              const double *__restrict__ av, const double *__restrict__ dinv,
                              const double *__restrict__ b, const double *__restrict__ x,
                              double *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc[C];
#pragma unroll
  for (int c = 0; c < C; ++c) acc[c] = b[(size_t)i * C + c];
  if (x)
    for (int p = ap[i]; p < ap[i + 1]; ++p) {
      double a = av[p];
      const double *xr = x + (size_t)ac[p] * C;
#pragma unroll
      for (int c = 0; c < C; ++c) acc[c] = fma(-a, xr[c], acc[c]);
    }
  double d = dinv[i];
#pragma unroll
  for (int c = 0; c < C; ++c) out[(size_t)i * C + c] = (x ? x[(size_t)i * C + c] : 0.0) + d * acc[c];
}

template <int C>
__global__ void residual_kernel(int n, const int *__restrict__ ap, const int *__restrict__ ac,
                                const double *__restrict__ av, const double *__restrict__ b,
                                const double *__restrict__ x, double *__restrict__ r) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc[C];
#pragma unroll
  for (int c = 0; c < C; ++c) acc[c] = b[(size_t)i * C + c];
  for (int p = ap[i]; p < ap[i + 1]; ++p) {
    double a = av[p];
    const double *xr = x + (size_t)ac[p] * C;
#pragma unroll
    for (int c = 0; c < C; ++c) acc[c] = fma(-a, xr[c], acc[c]);
  }
#pragma unroll
  for (int c = 0; c < C; ++c) r[(size_t)i * C + c] = acc[c];
}

__global__ void dense_solve_kernel(int n, const double *__restrict__ inv, const double *__restrict__ b,
                                   int C, double *__restrict__ x) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * C) return;
  int i = t / C, c = t % C;
  double acc = 0.0;
  for (int j = 0; j < n; ++j) acc = fma(inv[(size_t)i * n + j], b[(size_t)j * C + c], acc);
  x[(size_t)i * C + c] = acc;
}

constexpr int kDotBlocks = 120;  // fixed split of the column dot products (deterministic)

// part[b][c] = sum over rows i of block b's range of a[i][c] * w[i][c]
__global__ void col_dots_partial(int n, int C, const double *__restrict__ a, const double *__restrict__ w,
                                 double *part) {
  __shared__ double sh[12][128];
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
  for (int c = 0; c < C; ++c) {
    double acc = 0.0;
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) acc = fma(a[(size_t)i * C + c], w[(size_t)i * C + c], acc);
    sh[c][threadIdx.x] = acc;
  }
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st)
      for (int c = 0; c < C; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < C; ++c) part[(size_t)blockIdx.x * C + c] = sh[c][0];
}

// Scalars of one CG step, per column: slot layout s[0..C) = r.z, s[C..2C) = step length alpha
// (mode 0: alpha = rz / (p.q) from the partial sums; a non-positive curvature stops the column),
// mode 1: beta = rz_new / rz into s[2C..3C) and rz = rz_new.
__global__ void cg_scalars(int C, const double *part, double *s, int mode) {
  int c = threadIdx.x;
  if (c >= C) return;
  double t = 0.0;
  for (int b = 0; b < kDotBlocks; ++b) t += part[(size_t)b * C + c];
  if (mode == 0) {
    s[C + c] = (t > 0.0 && s[c] > 0.0) ? s[c] / t : 0.0;
  } else if (mode == 1) {
    s[2 * C + c] = s[c] > 0.0 ? t / s[c] : 0.0;
    s[c] = t;
  } else {
    s[c] = t;
  }
}

// x += alpha p, r -= alpha q (per column)
__global__ void cg_update(int n, int C, const double *__restrict__ s, const double *__restrict__ p,
                          const double *__restrict__ q, double *__restrict__ x, double *__restrict__ r) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)n * C) return;
  const double a = s[C + t % C];
  x[t] = fma(a, p[t], x[t]);
  r[t] = fma(-a, q[t], r[t]);
}

// p = z + beta p
__global__ void cg_direction(int n, int C, const double *__restrict__ s, const double *__restrict__ z,
                             double *__restrict__ p) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)n * C) return;
  p[t] = fma(s[2 * C + t % C], p[t], z[t]);
}

template <class T>
void up(DevBuf<T> &d, const std::vector<T> &v, cudaStream_t s) {
  d.alloc(std::max<size_t>(v.size(), 1));
  if (!v.empty()) d.upload(v.data(), v.size(), s);
}

}  // namespace

void AmgDevice::upload(const AmgHost &h, cudaStream_t s) {
  for (auto &gr : graphs)
    if (gr.exec) cudaGraphExecDestroy(gr.exec);
  graphs.clear();
  size_t nl = h.A.size();
  L.clear();
  L.resize(nl);
  for (size_t l = 0; l < nl; ++l) {
    Level &v = L[l];
    v.n = h.A[l].n;
    up(v.ap, h.A[l].ptr, s), up(v.ac, h.A[l].col, s), up(v.av, h.A[l].val, s);
    up(v.dinv, h.dinv[l], s);
    if (l + 1 < nl) {
      up(v.pp, h.P[l].ptr, s), up(v.pc, h.P[l].col, s), up(v.pv, h.P[l].val, s);
      up(v.rp, h.R[l].ptr, s), up(v.rc, h.R[l].col, s), up(v.rv, h.R[l].val, s);
    }
  }
  up(cinv, h.coarse_inv, s);
  C = 0;
}

void AmgDevice::reserve(int C_) {
  if (C_ > 12) fail(RS_INTERNAL, "Internal", "preconditioner", "at most 12 multigrid columns");
  if (C >= 12) return;
  // buffers for the widest batch at once: graphs captured for a width keep their pointers
  C = 12;
  for (auto &v : L) {
    size_t m = (size_t)v.n * C;
    v.x.alloc(m), v.b.alloc(m), v.r.alloc(m), v.t.alloc(m);
  }
}

template <int CC>
void AmgDevice::spmv0_t(rs_ctx *ctx, const double *x, double *y) {
  Level &v = L[0];
  spmv_c_kernel<false, CC><<<nblk(v.n, 128), 128, 0, ctx->stream>>>(v.n, v.ap.p, v.ac.p, v.av.p, x, y);
  RSG_LAUNCHED(ctx, "amg_spmv");
}

template <int CC>
void AmgDevice::vcycle_t(rs_ctx *ctx, const double *b, double *x) {
  cudaStream_t s = ctx->stream;
  const int nl = (int)L.size();
  // down: level l solves A_l x_l = b_l (b_0 = b), x_l starts at 0
  const double *bl = b;
  for (int l = 0; l < nl - 1; ++l) {
    Level &v = L[l];
    double *xl = (l == 0) ? x : v.x.p;
    const unsigned g = nblk(v.n, 128);
    // pre-smoothing from x = 0
    jacobi_kernel<CC><<<g, 128, 0, s>>>(v.n, v.ap.p, v.ac.p, v.av.p, v.dinv.p, bl, nullptr, v.t.p);
    RSG_LAUNCHED(ctx, "amg_jacobi");
    const double *cur = v.t.p;
    double *nxt = xl;
    for (int k = 1; k < sweeps; ++k) {
      jacobi_kernel<CC><<<g, 128, 0, s>>>(v.n, v.ap.p, v.ac.p, v.av.p, v.dinv.p, bl, cur, nxt);
      RSG_LAUNCHED(ctx, "amg_jacobi");
      std::swap(cur, *(const double **)&nxt);
    }
    if (cur != xl)
      RSG_CUDA("preconditioner", cudaMemcpyAsync(xl, cur, (size_t)v.n * CC * sizeof(double), cudaMemcpyDeviceToDevice, s));
    residual_kernel<CC><<<g, 128, 0, s>>>(v.n, v.ap.p, v.ac.p, v.av.p, bl, xl, v.r.p);
    RSG_LAUNCHED(ctx, "amg_residual");
    Level &w = L[l + 1];
    spmv_c_kernel<false, CC><<<nblk(w.n, 128), 128, 0, s>>>(w.n, v.rp.p, v.rc.p, v.rv.p, v.r.p, w.b.p);
    RSG_LAUNCHED(ctx, "amg_restrict");
    bl = w.b.p;
  }
  // coarsest
  {
    Level &v = L[nl - 1];
    double *xl = (nl == 1) ? x : v.x.p;
    dense_solve_kernel<<<nblk((size_t)v.n * CC, 128), 128, 0, s>>>(v.n, cinv.p, bl, CC, xl);
    RSG_LAUNCHED(ctx, "amg_coarse");
  }
  // up: x_l += P x_{l+1}, post-smoothing
  for (int l = nl - 2; l >= 0; --l) {
    Level &v = L[l];
    double *xl = (l == 0) ? x : v.x.p;
    const double *xc = L[l + 1].x.p;
    spmv_c_kernel<true, CC><<<nblk(v.n, 128), 128, 0, s>>>(v.n, v.pp.p, v.pc.p, v.pv.p, xc, xl);
    RSG_LAUNCHED(ctx, "amg_prolong");
    const double *blv = (l == 0) ? b : v.b.p;
    const unsigned g = nblk(v.n, 128);
    for (int k = 0; k < sweeps; ++k) {
      jacobi_kernel<CC><<<g, 128, 0, s>>>(v.n, v.ap.p, v.ac.p, v.av.p, v.dinv.p, blv, xl, v.t.p);
      RSG_LAUNCHED(ctx, "amg_jacobi");
      RSG_CUDA("preconditioner", cudaMemcpyAsync(xl, v.t.p, (size_t)v.n * CC * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
  }
}

#define RSG_AMG_WIDTH(CALL)                                                              \
  switch (C_) {                                                                          \
    case 3: CALL(3); break;                                                              \
    case 6: CALL(6); break;                                                              \
    case 9: CALL(9); break;                                                              \
    case 12: CALL(12); break;                                                            \
    default: fail(RS_INTERNAL, "Internal", "preconditioner", "multigrid width 3, 6, 9 or 12"); \
  }

void AmgDevice::spmv0(rs_ctx *ctx, const double *x, double *y, int C_) {
#define RSG_CALL(W) spmv0_t<W>(ctx, x, y)
  RSG_AMG_WIDTH(RSG_CALL)
#undef RSG_CALL
}

void AmgDevice::vcycle(rs_ctx *ctx, const double *b, double *x, int C_) {
  reserve(C_);
#define RSG_CALL(W) vcycle_t<W>(ctx, b, x)
  RSG_AMG_WIDTH(RSG_CALL)
#undef RSG_CALL
}

void AmgDevice::pcg_body(rs_ctx *ctx, const double *b, double *x, int C_, int iters) {
  cudaStream_t s = ctx->stream;
  const int n = L[0].n;
  const size_t m = (size_t)n * C_;
  const unsigned g = nblk(m, 256);
  auto dots = [&](const double *a, const double *w, int mode) {
    col_dots_partial<<<kDotBlocks, 128, 0, s>>>(n, C_, a, w, cg_part.p);
    RSG_LAUNCHED(ctx, "cg_dots");
    cg_scalars<<<1, 32, 0, s>>>(C_, cg_part.p, cg_s.p, mode);
    RSG_LAUNCHED(ctx, "cg_scalars");
  };
  // x = 0, r = b, z = M r, p = z, rz = r.z
  RSG_CUDA("preconditioner", cudaMemsetAsync(x, 0, m * sizeof(double), s));
  RSG_CUDA("preconditioner", cudaMemcpyAsync(cg_r.p, b, m * sizeof(double), cudaMemcpyDeviceToDevice, s));
  vcycle(ctx, cg_r.p, cg_z.p, C_);
  RSG_CUDA("preconditioner", cudaMemcpyAsync(cg_p.p, cg_z.p, m * sizeof(double), cudaMemcpyDeviceToDevice, s));
  dots(cg_r.p, cg_z.p, 2);
  for (int it = 0; it < iters; ++it) {
    spmv0(ctx, cg_p.p, cg_q.p, C_);
    dots(cg_p.p, cg_q.p, 0);
    cg_update<<<g, 256, 0, s>>>(n, C_, cg_s.p, cg_p.p, cg_q.p, x, cg_r.p);
    RSG_LAUNCHED(ctx, "cg_update");
    if (it + 1 == iters) break;
    vcycle(ctx, cg_r.p, cg_z.p, C_);
    dots(cg_r.p, cg_z.p, 1);
    cg_direction<<<g, 256, 0, s>>>(n, C_, cg_s.p, cg_z.p, cg_p.p);
    RSG_LAUNCHED(ctx, "cg_direction");
  }
}

// The conjugate-gradient solve is a few hundred small launches (levels x sweeps x steps) with
// all scalars on the device, so it is captured once per (b, x, width, steps) into a CUDA graph
// and replayed: the buffers it touches are allocated for the widest batch before the first
// capture and never move.
void AmgDevice::pcg(rs_ctx *ctx, const double *b, double *x, int C_, int iters) {
  reserve(C_);
  const size_t m = (size_t)L[0].n * 12;
  if (cg_r.n < m) cg_r.alloc(m), cg_z.alloc(m), cg_p.alloc(m), cg_q.alloc(m);
  if (cg_part.n < (size_t)kDotBlocks * 12) cg_part.alloc((size_t)kDotBlocks * 12), cg_s.alloc(36);
  cudaStream_t s = ctx->stream;
  for (auto &gr : graphs)
    if (gr.b == b && gr.x == x && gr.C == C_ && gr.iters == iters) {
      RSG_CUDA("preconditioner", cudaGraphLaunch(gr.exec, s));
      ctx->launches += gr.launches;
      return;
    }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  RSG_CUDA("preconditioner", cudaStreamIsCapturing(s, &cs));
  if (cs != cudaStreamCaptureStatusNone) {  // the caller is capturing already: record inline
    pcg_body(ctx, b, x, C_, iters);
    return;
  }
  Graph gr;
  gr.b = b, gr.x = x, gr.C = C_, gr.iters = iters;
  const int64_t l0 = ctx->launches;
  RSG_CUDA("preconditioner", cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  try {
    pcg_body(ctx, b, x, C_, iters);
  } catch (...) {
    cudaGraph_t dummy = nullptr;
    cudaStreamEndCapture(s, &dummy);
    if (dummy) cudaGraphDestroy(dummy);
    throw;
  }
  cudaGraph_t graph = nullptr;
  RSG_CUDA("preconditioner", cudaStreamEndCapture(s, &graph));
  gr.launches = ctx->launches - l0;
  ctx->launches = l0;
  cudaError_t e = cudaGraphInstantiate(&gr.exec, graph, 0);
  cudaGraphDestroy(graph);
  RSG_CUDA("preconditioner", e);
  graphs.push_back(gr);
  RSG_CUDA("preconditioner", cudaGraphLaunch(gr.exec, s));
  ctx->launches += gr.launches;
}

AmgDevice::~AmgDevice() {
  for (auto &gr : graphs)
    if (gr.exec) cudaGraphExecDestroy(gr.exec);
}

}  // namespace rsg
