// Device V-cycle of the smoothed-aggregation multigrid (see amg.hpp). Vectors hold C
// interleaved columns per row (x[row * C + c]); every kernel is one thread per row.
#include "amg.hpp"

namespace rsg {

namespace {

inline unsigned nblk(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// y = A x (accumulate: y += A x)
template <bool ACC>
__global__ void spmv_c_kernel(int n, const int *__restrict__ ap, const int *__restrict__ ac,
                              const double *__restrict__ av, const double *__restrict__ x, int C,
                              double *__restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc[12];
  for (int c = 0; c < C; ++c) acc[c] = ACC ? y[(size_t)i * C + c] : 0.0;
  for (int p = ap[i]; p < ap[i + 1]; ++p) {
    double a = av[p];
    const double *xr = x + (size_t)ac[p] * C;
    for (int c = 0; c < C; ++c) acc[c] = fma(a, xr[c], acc[c]);
  }
  for (int c = 0; c < C; ++c) y[(size_t)i * C + c] = acc[c];
}

// out = x + dinv (b - A x); x = null means x = 0 (out = dinv b). Also r = b - A x if r != null.
__global__ void jacobi_kernel(int n, const int *__restrict__ ap, const int *__restrict__ ac,
                              const double *__restrict__ av, const double *__restrict__ dinv,
                              const double *__restrict__ b, const double *__restrict__ x, int C,
                              double *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc[12];
  for (int c = 0; c < C; ++c) acc[c] = b[(size_t)i * C + c];
  if (x)
    for (int p = ap[i]; p < ap[i + 1]; ++p) {
      double a = av[p];
      const double *xr = x + (size_t)ac[p] * C;
      for (int c = 0; c < C; ++c) acc[c] = fma(-a, xr[c], acc[c]);
    }
  double d = dinv[i];
  for (int c = 0; c < C; ++c) out[(size_t)i * C + c] = (x ? x[(size_t)i * C + c] : 0.0) + d * acc[c];
}

__global__ void residual_kernel(int n, const int *__restrict__ ap, const int *__restrict__ ac,
                                const double *__restrict__ av, const double *__restrict__ b,
                                const double *__restrict__ x, int C, double *__restrict__ r) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc[12];
  for (int c = 0; c < C; ++c) acc[c] = b[(size_t)i * C + c];
  for (int p = ap[i]; p < ap[i + 1]; ++p) {
    double a = av[p];
    const double *xr = x + (size_t)ac[p] * C;
    for (int c = 0; c < C; ++c) acc[c] = fma(-a, xr[c], acc[c]);
  }
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

template <class T>
void up(DevBuf<T> &d, const std::vector<T> &v, cudaStream_t s) {
  d.alloc(std::max<size_t>(v.size(), 1));
  if (!v.empty()) d.upload(v.data(), v.size(), s);
}

}  // namespace

void AmgDevice::upload(const AmgHost &h, cudaStream_t s) {
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
  if (C_ <= C) return;
  if (C_ > 12) fail(RS_INTERNAL, "Internal", "preconditioner", "at most 12 multigrid columns");
  C = C_;
  for (auto &v : L) {
    size_t m = (size_t)v.n * C;
    v.x.alloc(m), v.b.alloc(m), v.r.alloc(m), v.t.alloc(m);
  }
}

void AmgDevice::spmv0(rs_ctx *ctx, const double *x, double *y, int C_) {
  Level &v = L[0];
  spmv_c_kernel<false><<<nblk(v.n, 128), 128, 0, ctx->stream>>>(v.n, v.ap.p, v.ac.p, v.av.p, x, C_, y);
  RSG_LAUNCHED(ctx, "amg_spmv");
}

void AmgDevice::vcycle(rs_ctx *ctx, const double *b, double *x, int C_) {
  reserve(C_);
  cudaStream_t s = ctx->stream;
  const int nl = (int)L.size();
  // down: level l solves A_l x_l = b_l (b_0 = b), x_l starts at 0
  const double *bl = b;
  for (int l = 0; l < nl - 1; ++l) {
    Level &v = L[l];
    double *xl = (l == 0) ? x : v.x.p;
    const unsigned g = nblk(v.n, 128);
    // pre-smoothing from x = 0
    jacobi_kernel<<<g, 128, 0, s>>>(v.n, v.ap.p, v.ac.p, v.av.p, v.dinv.p, bl, nullptr, C_, v.t.p);
    RSG_LAUNCHED(ctx, "amg_jacobi");
    const double *cur = v.t.p;
    double *nxt = xl;
    for (int k = 1; k < sweeps; ++k) {
      jacobi_kernel<<<g, 128, 0, s>>>(v.n, v.ap.p, v.ac.p, v.av.p, v.dinv.p, bl, cur, C_, nxt);
      RSG_LAUNCHED(ctx, "amg_jacobi");
      std::swap(cur, *(const double **)&nxt);
    }
    if (cur != xl)
      RSG_CUDA("preconditioner", cudaMemcpyAsync(xl, cur, (size_t)v.n * C_ * sizeof(double), cudaMemcpyDeviceToDevice, s));
    residual_kernel<<<g, 128, 0, s>>>(v.n, v.ap.p, v.ac.p, v.av.p, bl, xl, C_, v.r.p);
    RSG_LAUNCHED(ctx, "amg_residual");
    Level &w = L[l + 1];
    spmv_c_kernel<false><<<nblk(w.n, 128), 128, 0, s>>>(w.n, v.rp.p, v.rc.p, v.rv.p, v.r.p, C_, w.b.p);
    RSG_LAUNCHED(ctx, "amg_restrict");
    bl = w.b.p;
  }
  // coarsest
  {
    Level &v = L[nl - 1];
    double *xl = (nl == 1) ? x : v.x.p;
    dense_solve_kernel<<<nblk((size_t)v.n * C_, 128), 128, 0, s>>>(v.n, cinv.p, bl, C_, xl);
    RSG_LAUNCHED(ctx, "amg_coarse");
  }
  // up: x_l += P x_{l+1}, post-smoothing
  for (int l = nl - 2; l >= 0; --l) {
    Level &v = L[l];
    double *xl = (l == 0) ? x : v.x.p;
    const double *xc = (l + 1 == nl - 1 && nl == 1) ? x : L[l + 1].x.p;
    spmv_c_kernel<true><<<nblk(v.n, 128), 128, 0, s>>>(v.n, v.pp.p, v.pc.p, v.pv.p, xc, C_, xl);
    RSG_LAUNCHED(ctx, "amg_prolong");
    const double *blv = (l == 0) ? b : v.b.p;
    const unsigned g = nblk(v.n, 128);
    for (int k = 0; k < sweeps; ++k) {
      jacobi_kernel<<<g, 128, 0, s>>>(v.n, v.ap.p, v.ac.p, v.av.p, v.dinv.p, blv, xl, C_, v.t.p);
      RSG_LAUNCHED(ctx, "amg_jacobi");
      RSG_CUDA("preconditioner", cudaMemcpyAsync(xl, v.t.p, (size_t)v.n * C_ * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
  }
}

}  // namespace rsg
