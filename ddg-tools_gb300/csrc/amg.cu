// Device V-cycle of the smoothed-aggregation multigrid (see amg.hpp). Vectors hold C
// interleaved columns per row (x[row * C + c]); every kernel is one thread per row.
#include "amg.hpp"

namespace rsg {

namespace {

inline unsigned nblk(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// Sparse rows are split over groups of TPR consecutive lanes (TPR a power of two, at most
// 32): lane `sub` of a group takes the nonzeros sub, sub + TPR, ... of its row, and the group
// combines its partial sums by a butterfly of shuffles (every lane ends with the same sum).
// A group shares one row, so a group leaves a kernel early as a whole and its shuffles name
// only its own lanes.
template <int TPR>
__device__ __forceinline__ unsigned group_mask() {
  if constexpr (TPR == 32) return 0xffffffffu;
  else return ((1u << TPR) - 1u) << ((threadIdx.x & 31u) & ~(unsigned)(TPR - 1));
}

// acc[c] = sum over the nonzeros p of row i of a_p x[col_p][c]
template <int TPR, int C>
__device__ __forceinline__ void row_product(int i, int sub, const int *__restrict__ ap, const int *__restrict__ ac,
                                            const mgreal *__restrict__ av, const mgreal *__restrict__ x,
                                            mgreal (&acc)[C]) {
#pragma unroll
  for (int c = 0; c < C; ++c) acc[c] = 0.0;
  const int p1 = ap[i + 1];
  for (int p = ap[i] + sub; p < p1; p += TPR) {
    const mgreal a = av[p];
    const mgreal *xr = x + (size_t)ac[p] * C;
#pragma unroll
    for (int c = 0; c < C; ++c) acc[c] = fma(a, xr[c], acc[c]);
  }
  if constexpr (TPR > 1) {
    const unsigned mask = group_mask<TPR>();
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1)
#pragma unroll
      for (int c = 0; c < C; ++c) acc[c] += __shfl_xor_sync(mask, acc[c], o, TPR);
  }
}

// y = A x (accumulate: y += A x); C columns per row, a compile-time width so that the
// accumulators stay in registers.
// With t_out (and ACC false) also t_out = dinv y: the first Jacobi sweep from x = 0 of the level
// whose right-hand side y is (a restriction that starts the next level's pre-smoothing).
template <int TPR, bool ACC, int C>
__global__ void spmv_c_kernel(int n, const int *__restrict__ ap, const int *__restrict__ ac,
                              const mgreal *__restrict__ av, const mgreal *__restrict__ x,
                              mgreal *__restrict__ y, const mgreal *__restrict__ dinv, mgreal *__restrict__ t_out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / TPR, sub = t % TPR;
  if (i >= n) return;
  mgreal acc[C];
  row_product<TPR, C>(i, sub, ap, ac, av, x, acc);
  if (sub != 0) return;
#pragma unroll
  for (int c = 0; c < C; ++c) y[(size_t)i * C + c] = ACC ? y[(size_t)i * C + c] + acc[c] : acc[c];
  if (!ACC && t_out) {
    const mgreal d = dinv[i];
#pragma unroll
    for (int c = 0; c < C; ++c) t_out[(size_t)i * C + c] = d * acc[c];
  }
}

// out = x + dinv (b - A x)
template <int TPR, int C>
__global__ void jacobi_kernel(int n, const int *__restrict__ ap, const int *__restrict__ ac,
                              const mgreal *__restrict__ av, const mgreal *__restrict__ dinv,
                              const mgreal *__restrict__ b, const mgreal *__restrict__ x,
                              mgreal *__restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / TPR, sub = t % TPR;
  if (i >= n) return;
  mgreal acc[C];
  row_product<TPR, C>(i, sub, ap, ac, av, x, acc);
  if (sub != 0) return;
  const mgreal d = dinv[i];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const size_t k = (size_t)i * C + c;
    out[k] = fma(d, b[k] - acc[c], x[k]);
  }
}

// out = dinv b (the first Jacobi step from x = 0)
template <int C>
__global__ void jacobi0_kernel(int n, const mgreal *__restrict__ dinv, const mgreal *__restrict__ b,
                               mgreal *__restrict__ out) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)n * C) return;
  out[t] = dinv[t / C] * b[t];
}

// r = b - A x
template <int TPR, int C>
__global__ void residual_kernel(int n, const int *__restrict__ ap, const int *__restrict__ ac,
                                const mgreal *__restrict__ av, const mgreal *__restrict__ b,
                                const mgreal *__restrict__ x, mgreal *__restrict__ r) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / TPR, sub = t % TPR;
  if (i >= n) return;
  mgreal acc[C];
  row_product<TPR, C>(i, sub, ap, ac, av, x, acc);
  if (sub != 0) return;
#pragma unroll
  for (int c = 0; c < C; ++c) r[(size_t)i * C + c] = b[(size_t)i * C + c] - acc[c];
}

// x = inv b on the coarsest level (dense n x n inverse), one warp per row
template <int C>
__global__ void dense_solve_kernel(int n, const mgreal *__restrict__ inv, const mgreal *__restrict__ b,
                                   mgreal *__restrict__ x) {
  const int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (i >= n) return;
  mgreal acc[C];
#pragma unroll
  for (int c = 0; c < C; ++c) acc[c] = 0.0;
  for (int j = lane; j < n; j += 32) {
    const mgreal a = inv[(size_t)i * n + j];
#pragma unroll
    for (int c = 0; c < C; ++c) acc[c] = fma(a, b[(size_t)j * C + c], acc[c]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int c = 0; c < C; ++c) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  if (lane == 0)
#pragma unroll
    for (int c = 0; c < C; ++c) x[(size_t)i * C + c] = acc[c];
}

constexpr int kDotBlocks = 304;  // fixed split of the column dot products (deterministic)

// Column dot products a.w of one CG step and the scalars that follow from them. Each block
// writes its partial sums; the last block to finish (a ticket counter) adds the partials in
// block order and updates the scalars, then resets the counter for the next launch. Slot
// layout s[0..C) = r.z, s[C..2C) = step length alpha, s[2C..3C) = beta. Mode 0: alpha =
// rz / (p.q) (a non-positive curvature stops the column); mode 1: beta = rz_new / rz and
// rz = rz_new; mode 2: rz = the sum.
template <int C>
__global__ void __launch_bounds__(128) cg_dots_kernel(int n, const mgreal *__restrict__ a, const mgreal *__restrict__ w,
                                                      double *part, unsigned *ticket, double *s, int mode) {
  __shared__ double sh[C][128];
  __shared__ bool last;
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
  float acc[C];
#pragma unroll
  for (int c = 0; c < C; ++c) acc[c] = 0.f;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x)
#pragma unroll
    for (int c = 0; c < C; ++c) acc[c] = fmaf(a[(size_t)i * C + c], w[(size_t)i * C + c], acc[c]);
#pragma unroll
  for (int c = 0; c < C; ++c) sh[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st)
#pragma unroll
      for (int c = 0; c < C; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < C; ++c) part[(size_t)blockIdx.x * C + c] = sh[c][0];
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the last block: the partials strided over its threads, then the same tree
  double tp[C];
#pragma unroll
  for (int c = 0; c < C; ++c) tp[c] = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
#pragma unroll
    for (int c = 0; c < C; ++c) tp[c] += __ldcg(part + (size_t)b * C + c);
#pragma unroll
  for (int c = 0; c < C; ++c) sh[c][threadIdx.x] = tp[c];
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st)
#pragma unroll
      for (int c = 0; c < C; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + st];
    __syncthreads();
  }
  const int c = threadIdx.x;
  if (c < C) {
    const double t = sh[c][0];
    if (mode == 0) {
      s[C + c] = (t > 0.0 && s[c] > 0.0) ? s[c] / t : 0.0;
    } else if (mode == 1) {
      s[2 * C + c] = s[c] > 0.0 ? t / s[c] : 0.0;
      s[c] = t;
    } else {
      s[c] = t;
    }
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

// x += alpha p, r -= alpha q (per column)
// With t0: also t0 = dinv r (the next V-cycle's first sweep on level 0).
__global__ void cg_update(int n, int C, const double *__restrict__ s, const mgreal *__restrict__ p,
                          const mgreal *__restrict__ q, mgreal *__restrict__ x, mgreal *__restrict__ r,
                          const mgreal *__restrict__ dinv, mgreal *__restrict__ t0) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)n * C) return;
  const mgreal a = (mgreal)s[C + t % C];
  x[t] = fma(a, p[t], x[t]);
  const mgreal rn = fma(-a, q[t], r[t]);
  r[t] = rn;
  if (t0) t0[t] = dinv[t / C] * rn;
}

// p = z + beta p
__global__ void cg_direction(int n, int C, const double *__restrict__ s, const mgreal *__restrict__ z,
                             mgreal *__restrict__ p) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)n * C) return;
  p[t] = fma((mgreal)s[2 * C + t % C], p[t], z[t]);
}

template <class T>
void up(DevBuf<T> &d, const std::vector<T> &v, cudaStream_t s) {
  d.alloc(std::max<size_t>(v.size(), 1));
  if (!v.empty()) d.upload(v.data(), v.size(), s);
}

// the FP64 setup's values rounded to the multigrid type
void up(DevBuf<mgreal> &d, const std::vector<double> &v, cudaStream_t s) {
  std::vector<mgreal> w(v.begin(), v.end());
  up(d, w, s);
}

// lanes per row: the smallest power of two (at most 32) that leaves each lane about four nonzeros
int lanes_per_row(const Csr &A) {
  const double mean = A.n > 0 ? (double)A.ptr[A.n] / A.n : 0.0;
  int t = 1;
  while (t < 32 && 4 * t < mean) t *= 2;
  return t;
}

#define RSG_TPR(T, CALL)        \
  switch (T) {                  \
    case 1: CALL(1); break;     \
    case 2: CALL(2); break;     \
    case 4: CALL(4); break;     \
    case 8: CALL(8); break;     \
    case 16: CALL(16); break;   \
    default: CALL(32); break;   \
  }

template <bool ACC, int C>
void spmv_launch(int tpr, int n, const int *ap, const int *ac, const mgreal *av, const mgreal *x, mgreal *y,
                 cudaStream_t s, const mgreal *dinv = nullptr, mgreal *t_out = nullptr) {
  const unsigned g = nblk((size_t)n * tpr, 128);
#define RSG_CALL(T) spmv_c_kernel<T, ACC, C><<<g, 128, 0, s>>>(n, ap, ac, av, x, y, dinv, t_out)
  RSG_TPR(tpr, RSG_CALL)
#undef RSG_CALL
}

template <int C>
void jacobi_launch(int tpr, int n, const int *ap, const int *ac, const mgreal *av, const mgreal *dinv,
                   const mgreal *b, const mgreal *x, mgreal *out, cudaStream_t s) {
  const unsigned g = nblk((size_t)n * tpr, 128);
#define RSG_CALL(T) jacobi_kernel<T, C><<<g, 128, 0, s>>>(n, ap, ac, av, dinv, b, x, out)
  RSG_TPR(tpr, RSG_CALL)
#undef RSG_CALL
}

template <int C>
void residual_launch(int tpr, int n, const int *ap, const int *ac, const mgreal *av, const mgreal *b,
                     const mgreal *x, mgreal *r, cudaStream_t s) {
  const unsigned g = nblk((size_t)n * tpr, 128);
#define RSG_CALL(T) residual_kernel<T, C><<<g, 128, 0, s>>>(n, ap, ac, av, b, x, r)
  RSG_TPR(tpr, RSG_CALL)
#undef RSG_CALL
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
    v.tpr_a = lanes_per_row(h.A[l]);
    if (l + 1 < nl) {
      up(v.pp, h.P[l].ptr, s), up(v.pc, h.P[l].col, s), up(v.pv, h.P[l].val, s);
      up(v.rp, h.R[l].ptr, s), up(v.rc, h.R[l].col, s), up(v.rv, h.R[l].val, s);
      v.tpr_p = lanes_per_row(h.P[l]), v.tpr_r = lanes_per_row(h.R[l]);
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
void AmgDevice::spmv0_t(rs_ctx *ctx, const mgreal *x, mgreal *y) {
  Level &v = L[0];
  spmv_launch<false, CC>(v.tpr_a, v.n, v.ap.p, v.ac.p, v.av.p, x, y, ctx->stream);
  RSG_LAUNCHED(ctx, "amg_spmv");
}

template <int CC>
void AmgDevice::vcycle_t(rs_ctx *ctx, const mgreal *b, mgreal *x, bool pre0) {
  cudaStream_t s = ctx->stream;
  const int nl = (int)L.size();
  // `count` Jacobi sweeps that alternate between x_l and the level's scratch t, starting from
  // t (from_t) or x_l; a sweep count that ends in t is followed by a copy
  auto smooth = [&](Level &v, const mgreal *bl, mgreal *xl, bool from_t, int count) {
    mgreal *cur = from_t ? v.t.p : xl, *other = from_t ? xl : v.t.p;
    for (int k = 0; k < count; ++k) {
      jacobi_launch<CC>(v.tpr_a, v.n, v.ap.p, v.ac.p, v.av.p, v.dinv.p, bl, cur, other, s);
      RSG_LAUNCHED(ctx, "amg_jacobi");
      std::swap(cur, other);
    }
    if (cur != xl)
      RSG_CUDA("preconditioner", cudaMemcpyAsync(xl, cur, (size_t)v.n * CC * sizeof(mgreal), cudaMemcpyDeviceToDevice, s));
  };
  // down: level l solves A_l x_l = b_l (b_0 = b), x_l starts at 0. Pre-smoothing: the first
  // sweep from x = 0 is dinv b, written where the remaining sweeps end in x_l (t for an even
  // sweep count); below level 0 the restriction that forms b_l writes it, on level 0 the caller
  // may have (pre0)
  const bool odd = (sweeps - 1) % 2 == 1;
  const mgreal *bl = b;
  for (int l = 0; l < nl - 1; ++l) {
    Level &v = L[l];
    mgreal *xl = (l == 0) ? x : v.x.p;
    if (l == 0 && !pre0) {
      jacobi0_kernel<CC><<<nblk((size_t)v.n * CC, 256), 256, 0, s>>>(v.n, v.dinv.p, bl, odd ? v.t.p : xl);
      RSG_LAUNCHED(ctx, "amg_jacobi");
    }
    smooth(v, bl, xl, odd, sweeps - 1);
    residual_launch<CC>(v.tpr_a, v.n, v.ap.p, v.ac.p, v.av.p, bl, xl, v.r.p, s);
    RSG_LAUNCHED(ctx, "amg_residual");
    Level &w = L[l + 1];
    const bool coarsest = l + 1 == nl - 1;  // solved densely, no sweep
    spmv_launch<false, CC>(v.tpr_r, w.n, v.rp.p, v.rc.p, v.rv.p, v.r.p, w.b.p, s, coarsest ? nullptr : w.dinv.p,
                           coarsest ? nullptr : (odd ? w.t.p : w.x.p));
    RSG_LAUNCHED(ctx, "amg_restrict");
    bl = w.b.p;
  }
  // coarsest
  {
    Level &v = L[nl - 1];
    mgreal *xl = (nl == 1) ? x : v.x.p;
    dense_solve_kernel<CC><<<nblk((size_t)v.n * 32, 128), 128, 0, s>>>(v.n, cinv.p, bl, xl);
    RSG_LAUNCHED(ctx, "amg_coarse");
  }
  // up: x_l += P x_{l+1}, post-smoothing
  for (int l = nl - 2; l >= 0; --l) {
    Level &v = L[l];
    mgreal *xl = (l == 0) ? x : v.x.p;
    spmv_launch<true, CC>(v.tpr_p, v.n, v.pp.p, v.pc.p, v.pv.p, L[l + 1].x.p, xl, s);
    RSG_LAUNCHED(ctx, "amg_prolong");
    smooth(v, (l == 0) ? b : v.b.p, xl, false, sweeps);
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

void AmgDevice::spmv0(rs_ctx *ctx, const mgreal *x, mgreal *y, int C_) {
#define RSG_CALL(W) spmv0_t<W>(ctx, x, y)
  RSG_AMG_WIDTH(RSG_CALL)
#undef RSG_CALL
}

void AmgDevice::vcycle(rs_ctx *ctx, const mgreal *b, mgreal *x, int C_, bool pre0) {
  reserve(C_);
#define RSG_CALL(W) vcycle_t<W>(ctx, b, x, pre0)
  RSG_AMG_WIDTH(RSG_CALL)
#undef RSG_CALL
}

void AmgDevice::pcg_body(rs_ctx *ctx, const mgreal *b, mgreal *x, int C_, int iters) {
  cudaStream_t s = ctx->stream;
  const int n = L[0].n;
  const size_t m = (size_t)n * C_;
  const unsigned g = nblk(m, 256);
  auto dots = [&](const mgreal *a, const mgreal *w, int mode) {
#define RSG_CALL(W) cg_dots_kernel<W><<<kDotBlocks, 128, 0, s>>>(n, a, w, cg_part.p, cg_ticket.p, cg_s.p, mode)
    RSG_AMG_WIDTH(RSG_CALL)
#undef RSG_CALL
    RSG_LAUNCHED(ctx, "cg_dots");
  };
  // x = 0, r = b, z = M r, p = z, rz = r.z
  RSG_CUDA("preconditioner", cudaMemsetAsync(x, 0, m * sizeof(mgreal), s));
  RSG_CUDA("preconditioner", cudaMemcpyAsync(cg_r.p, b, m * sizeof(mgreal), cudaMemcpyDeviceToDevice, s));
  vcycle(ctx, cg_r.p, cg_z.p, C_);
  RSG_CUDA("preconditioner", cudaMemcpyAsync(cg_p.p, cg_z.p, m * sizeof(mgreal), cudaMemcpyDeviceToDevice, s));
  dots(cg_r.p, cg_z.p, 2);
  for (int it = 0; it < iters; ++it) {
    spmv0(ctx, cg_p.p, cg_q.p, C_);
    dots(cg_p.p, cg_q.p, 0);
    // the update also writes the next V-cycle's first level-0 sweep (none after the last step)
    const bool more = it + 1 < iters;
    const bool odd = (sweeps - 1) % 2 == 1;
    cg_update<<<g, 256, 0, s>>>(n, C_, cg_s.p, cg_p.p, cg_q.p, x, cg_r.p, L[0].dinv.p,
                                more ? (odd ? L[0].t.p : cg_z.p) : nullptr);
    RSG_LAUNCHED(ctx, "cg_update");
    if (!more) break;
    vcycle(ctx, cg_r.p, cg_z.p, C_, true);
    dots(cg_r.p, cg_z.p, 1);
    cg_direction<<<g, 256, 0, s>>>(n, C_, cg_s.p, cg_z.p, cg_p.p);
    RSG_LAUNCHED(ctx, "cg_direction");
  }
}

// The conjugate-gradient solve is a few hundred small launches (levels x sweeps x steps) with
// all scalars on the device, so it is captured once per (b, x, width, steps) into a CUDA graph
// and replayed: the buffers it touches are allocated for the widest batch before the first
// capture and never move.
void AmgDevice::pcg(rs_ctx *ctx, const mgreal *b, mgreal *x, int C_, int iters) {
  reserve(C_);
  const size_t m = (size_t)L[0].n * 12;
  if (cg_r.n < m) cg_r.alloc(m), cg_z.alloc(m), cg_p.alloc(m), cg_q.alloc(m);
  if (cg_part.n < (size_t)kDotBlocks * 12) {
    cg_part.alloc((size_t)kDotBlocks * 12), cg_s.alloc(36), cg_ticket.alloc(1);
    RSG_CUDA("preconditioner", cudaMemsetAsync(cg_ticket.p, 0, sizeof(unsigned), ctx->stream));
  }
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
