// Device-resident restarted GMRES (see krylov.hpp). The vectors never leave the device; per
// Arnoldi step the host receives the j+2 Hessenberg entries of every right-hand side (one small
// copy) and runs the Givens rotations and the stop test, as GmresRun::after_arnoldi does
// (RS/src/solve/gmres.rs:454-513).
#include "krylov.hpp"
#include "profile.hpp"

#include <chrono>
#include <cmath>

namespace rsg {

namespace {

constexpr int RB = 256;  // reduction blocks of the dot products (fixed: deterministic sums)

inline unsigned nb_(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// Partial sums of v_i . w over a fixed row split: block b owns rows [b c, (b+1) c).
constexpr int kDotVecs = 8;  // vectors per pass over w

// out[i] = v_i . w (sqrt of it with `root`) for i < nvec, v_i = vs[i] (or v1 when given, nvec =
// 1). Each block takes a fixed row range and up to kDotVecs vectors per pass over it (w read
// once per pass), reduces by warp shuffles and then over the warps in order, and writes its
// partials; the last block to finish (a ticket counter, reset by that block) adds the
// partials of every vector in block order, a warp per vector. Deterministic: the grid, the
// row ranges and every reduction order are fixed.
__global__ void __launch_bounds__(256) dots_kernel(const double *const *vs, const double *v1, int nvec,
                                                   const double *__restrict__ w, size_t n, double *part,
                                                   unsigned *ticket, double *out, int root) {
  __shared__ double sh[8][kDotVecs];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const size_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const size_t r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
  for (int i0 = 0; i0 < nvec; i0 += kDotVecs) {
    const double *vp[kDotVecs];
    double acc[kDotVecs];
#pragma unroll
    for (int j = 0; j < kDotVecs; ++j) {
      vp[j] = (i0 + j < nvec) ? (v1 ? v1 : vs[i0 + j]) : nullptr;
      acc[j] = 0.0;
    }
    for (size_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      const double wr = w[r];
#pragma unroll
      for (int j = 0; j < kDotVecs; ++j)
        if (vp[j]) acc[j] = fma(vp[j][r], wr, acc[j]);
    }
#pragma unroll
    for (int j = 0; j < kDotVecs; ++j) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
      if (lane == 0) sh[wid][j] = acc[j];
    }
    __syncthreads();
    if ((int)threadIdx.x < kDotVecs && i0 + (int)threadIdx.x < nvec) {
      double t = 0.0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k][threadIdx.x];
      part[(size_t)blockIdx.x * nvec + i0 + threadIdx.x] = t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int i = wid; i < nvec; i += (int)(blockDim.x >> 5)) {
    double t = 0.0;
    for (unsigned b = lane; b < gridDim.x; b += 32) t += __ldcg(part + (size_t)b * nvec + i);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) out[i] = root ? sqrt(t) : t;
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

// w -= sum_i h_i v_i (sign = -1) or x += sum_i h_i v_i (sign = +1).
__global__ void axpy_many_kernel(const double *const *vs, int nvec, const double *__restrict__ h,
                                 double sign, double *w, size_t n) {
  __shared__ double hs[64];
  __shared__ const double *vp[64];
  if (threadIdx.x < nvec) hs[threadIdx.x] = h[threadIdx.x], vp[threadIdx.x] = vs[threadIdx.x];
  __syncthreads();
  for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < n; r += (size_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int i = 0; i < nvec; ++i) acc = fma(hs[i], vp[i][r], acc);
    w[r] = fma(sign, acc, w[r]);
  }
}

__global__ void scale_kernel(const double *x, const double *s_dev, double s_host, double *y, size_t n) {
  double s = s_dev ? 1.0 / *s_dev : s_host;
  for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < n; r += (size_t)gridDim.x * blockDim.x)
    y[r] = x[r] * s;
}

__global__ void sub_kernel(const double *a, const double *b, double *y, size_t n) {
  for (size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x; r < n; r += (size_t)gridDim.x * blockDim.x)
    y[r] = a[r] - b[r];
}


}  // namespace

void dev_dots(rs_ctx *ctx, const double *const *vs, int nvec, const double *w, size_t n,
              double *out_dev, const double *v1, bool root) {
  static thread_local DevBuf<double> partial;
  static thread_local DevBuf<unsigned> ticket;
  if (nvec < 1 || nvec > 64) fail(RS_INTERNAL, "Internal", "gmres", "1 to 64 vectors per dot-product launch");
  if (partial.n < (size_t)RB * 64) {
    partial.alloc((size_t)RB * 64), ticket.alloc(1);
    RSG_CUDA("gmres", cudaMemsetAsync(ticket.p, 0, sizeof(unsigned), ctx->stream));
  }
  dots_kernel<<<RB, 256, 0, ctx->stream>>>(vs, v1, nvec, w, n, partial.p, ticket.p, out_dev, root ? 1 : 0);
  RSG_LAUNCHED(ctx, "dots");
}

namespace {

// Per right-hand side: the device basis, the host Hessenberg / Givens state.
struct Rhs {
  DevBuf<double> V, Z, w, r, h;           // V: (m+1) n, Z: m n, h: 2 (m+2) scratch
  DevBuf<const double *> vptr, zptr;  // pointer tables for the multi-vector kernels
  std::vector<double> H, cs, sn, g, hcol;
  double bnorm = 0, beta = 0;
  int j = 0;
  bool done = false, active = false;
  GmresReport rep;
};

}  // namespace

void gmres_batch(rs_ctx *ctx, const Operator &A, const Operator *P, int nb, const double *b,
                 double *x, const GmresOptions &opt, std::vector<GmresReport> &reports,
                 const Operator *A_true) {
  const Operator &At = A_true ? *A_true : A;
  using clk = std::chrono::steady_clock;
  auto t0 = clk::now();
  if (opt.restart < 1 || opt.restart > 63 || opt.max_iterations < 1 || !(opt.tolerance > 0.0 && opt.tolerance < 1.0))
    fail(RS_INVALID_OPTION, "InvalidOption", "gmres",
         "restart in 1..63, max_iterations >= 1, tolerance in (0, 1)");
  const size_t n = A.n;
  const int m = (int)std::min<size_t>((size_t)opt.restart, std::max<size_t>(n, 1));
  cudaStream_t s = ctx->stream;
  std::vector<Rhs> R(nb);
  DevBuf<double> xbuf((size_t)nb * n), ybuf((size_t)nb * n);  // batched operator in/out
  DevBuf<double> norm2(1);
  // one norm: dots of w with itself, then sqrt
  auto norm_dev = [&](Rhs &, const double *v, double *out) { dev_dots(ctx, nullptr, 1, v, n, out, v, true); };
  auto host_value = [&](const double *dev) {
    double v;
    RSG_CUDA("gmres", rsg::copy_async(&v, dev, sizeof(double), cudaMemcpyDeviceToHost, s));
    RSG_CUDA("gmres", cudaStreamSynchronize(s));
    return v;
  };
  RSG_CUDA("gmres", cudaMemsetAsync(x, 0, (size_t)nb * n * sizeof(double), s));
  for (int q = 0; q < nb; ++q) {
    Rhs &Q = R[q];
    Q.V.alloc((size_t)(m + 1) * n);
    Q.Z.alloc((size_t)m * n);
    Q.w.alloc(n);
    Q.r.alloc(n);
    Q.h.alloc(2 * (size_t)(m + 2) + 2);
    Q.vptr.alloc(m + 1), Q.zptr.alloc(m);
    std::vector<const double *> vp(m + 1), zp(m);
    for (int i = 0; i <= m; ++i) vp[i] = Q.V.p + (size_t)i * n;
    for (int i = 0; i < m; ++i) zp[i] = Q.Z.p + (size_t)i * n;
    RSG_CUDA("gmres", rsg::copy_async(Q.vptr.p, vp.data(), vp.size() * sizeof(void *), cudaMemcpyHostToDevice, s));
    RSG_CUDA("gmres", rsg::copy_async(Q.zptr.p, zp.data(), zp.size() * sizeof(void *), cudaMemcpyHostToDevice, s));
    norm_dev(Q, b + (size_t)q * n, Q.h.p);
    Q.bnorm = host_value(Q.h.p);
    Q.H.assign((size_t)(m + 1) * m, 0.0);
    Q.cs.assign(m, 0.0), Q.sn.assign(m, 0.0), Q.g.assign(m + 1, 0.0);
    if (Q.bnorm == 0.0) {
      Q.done = true;
      Q.rep.converged = true;
    } else if (!std::isfinite(Q.bnorm)) {
      fail(RS_SOLVER_DIVERGED, "SolverDiverged", "gmres", "non-finite right-hand side");
    }
  }
  // the explicit residual r = b - A x of every active solve (x = 0 in the first cycle)
  auto cycle_start = [&](bool first) {
    std::vector<int> act;
    for (int q = 0; q < nb; ++q)
      if (!R[q].done) act.push_back(q);
    if (act.empty()) return;
    if (!first) {
      for (size_t i = 0; i < act.size(); ++i)
        RSG_CUDA("gmres", cudaMemcpyAsync(xbuf.p + i * n, x + (size_t)act[i] * n, n * sizeof(double),
                                          cudaMemcpyDeviceToDevice, s));
      At.apply((int)act.size(), xbuf.p, ybuf.p);
    }
    for (size_t i = 0; i < act.size(); ++i) {
      Rhs &Q = R[act[i]];
      if (!first) {
        Q.rep.operator_applications++;
        sub_kernel<<<nb_(n, 256), 256, 0, s>>>(b + (size_t)act[i] * n, ybuf.p + i * n, Q.r.p, n);
        RSG_LAUNCHED(ctx, "sub");
      } else {
        RSG_CUDA("gmres", cudaMemcpyAsync(Q.r.p, b + (size_t)act[i] * n, n * sizeof(double),
                                          cudaMemcpyDeviceToDevice, s));
      }
      norm_dev(Q, Q.r.p, Q.h.p);
    }
    for (size_t i = 0; i < act.size(); ++i) {
      Rhs &Q = R[act[i]];
      double beta = host_value(Q.h.p);
      double rel = beta / Q.bnorm;
      Q.rep.cycle_residuals.push_back(rel);
      Q.rep.relative_residual = rel;
      if (!std::isfinite(rel)) {
        Q.done = true;
        continue;
      }
      if (rel <= opt.tolerance) {
        Q.rep.converged = true;
        Q.done = true;
        continue;
      }
      if (Q.rep.iterations >= opt.max_iterations) {
        Q.done = true;
        continue;
      }
      Q.rep.cycles++;
      Q.beta = beta;
      std::fill(Q.g.begin(), Q.g.end(), 0.0);
      Q.g[0] = beta;
      Q.j = 0;
      scale_kernel<<<nb_(n, 256), 256, 0, s>>>(Q.r.p, nullptr, 1.0 / beta, Q.V.p, n);
      RSG_LAUNCHED(ctx, "scale");
    }
  };
  cycle_start(true);
  for (;;) {
    std::vector<int> act;
    for (int q = 0; q < nb; ++q)
      if (!R[q].done) act.push_back(q);
    if (act.empty()) break;
    const int na = (int)act.size();
    // z_j = P^-1 v_j, w = A z_j (batched over the active solves)
    for (int i = 0; i < na; ++i) {
      Rhs &Q = R[act[i]];
      RSG_CUDA("gmres", cudaMemcpyAsync(xbuf.p + (size_t)i * n, Q.V.p + (size_t)Q.j * n, n * sizeof(double),
                                        cudaMemcpyDeviceToDevice, s));
    }
    if (P) {
      P->apply(na, xbuf.p, ybuf.p);
      for (int i = 0; i < na; ++i) {
        Rhs &Q = R[act[i]];
        Q.rep.preconditioner_applications++;
        RSG_CUDA("gmres", cudaMemcpyAsync(Q.Z.p + (size_t)Q.j * n, ybuf.p + (size_t)i * n, n * sizeof(double),
                                          cudaMemcpyDeviceToDevice, s));
      }
      std::swap(xbuf.p, ybuf.p);  // z in xbuf; A z lands in ybuf as in the plain branch
      A.apply(na, xbuf.p, ybuf.p);
    } else {
      for (int i = 0; i < na; ++i) {
        Rhs &Q = R[act[i]];
        RSG_CUDA("gmres", cudaMemcpyAsync(Q.Z.p + (size_t)Q.j * n, xbuf.p + (size_t)i * n, n * sizeof(double),
                                          cudaMemcpyDeviceToDevice, s));
      }
      A.apply(na, xbuf.p, ybuf.p);
    }
    // classical Gram-Schmidt, twice; h = h1 + h2, then |w|
    if (opt.prof) opt.prof->begin(s, "gmres_orthogonalize");
    for (int i = 0; i < na; ++i) {
      Rhs &Q = R[act[i]];
      Q.rep.operator_applications++;
      const int k = Q.j + 1;
      double *w = Q.w.p;
      RSG_CUDA("gmres", cudaMemcpyAsync(w, ybuf.p + (size_t)i * n, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      double *h1 = Q.h.p, *h2 = Q.h.p + (m + 2);
      dev_dots(ctx, Q.vptr.p, k, w, n, h1);
      axpy_many_kernel<<<nb_(n, 256), 256, 0, s>>>(Q.vptr.p, k, h1, -1.0, w, n);
      RSG_LAUNCHED(ctx, "axpy_many");
      dev_dots(ctx, Q.vptr.p, k, w, n, h2);
      axpy_many_kernel<<<nb_(n, 256), 256, 0, s>>>(Q.vptr.p, k, h2, -1.0, w, n);
      RSG_LAUNCHED(ctx, "axpy_many");
      norm_dev(Q, w, Q.h.p + 2 * (m + 2));
    }
    if (opt.prof) opt.prof->end(s);
    std::vector<double> hh((size_t)na * (2 * (m + 2) + 1));
    for (int i = 0; i < na; ++i)
      RSG_CUDA("gmres", rsg::copy_async(hh.data() + (size_t)i * (2 * (m + 2) + 1), R[act[i]].h.p,
                                        (2 * (m + 2) + 1) * sizeof(double), cudaMemcpyDeviceToHost, s));
    RSG_CUDA("gmres", cudaStreamSynchronize(s));
    bool any_end = false;
    for (int i = 0; i < na; ++i) {
      Rhs &Q = R[act[i]];
      const double *hv = hh.data() + (size_t)i * (2 * (m + 2) + 1);
      const int j = Q.j;
      std::vector<double> col(j + 2);
      for (int t = 0; t <= j; ++t) col[t] = hv[t] + hv[(m + 2) + t];
      const double hn = hv[2 * (m + 2)];
      col[j + 1] = hn;
      for (int t = 0; t < j; ++t) {  // previous rotations
        double a = Q.cs[t] * col[t] + Q.sn[t] * col[t + 1];
        col[t + 1] = -Q.sn[t] * col[t] + Q.cs[t] * col[t + 1];
        col[t] = a;
      }
      double den = std::hypot(col[j], col[j + 1]);
      if (den == 0.0) Q.cs[j] = 1.0, Q.sn[j] = 0.0;
      else Q.cs[j] = col[j] / den, Q.sn[j] = col[j + 1] / den;
      col[j] = den;
      col[j + 1] = 0.0;
      Q.g[j + 1] = -Q.sn[j] * Q.g[j];
      Q.g[j] *= Q.cs[j];
      for (int t = 0; t <= j; ++t) Q.H[(size_t)t * m + j] = col[t];
      Q.rep.iterations++;
      double est = std::fabs(Q.g[j + 1]) / Q.bnorm;
      Q.rep.history.push_back(est);
      // a cycle ends when the Givens estimate is at half the tolerance: the explicit residual
      // of the FP32 operator sits a little above the estimate, and stopping at the tolerance
      // itself gives a run of short restarts near the target
      bool end = hn == 0.0 || !std::isfinite(hn) || est <= 0.5 * opt.tolerance ||
                 Q.rep.iterations >= opt.max_iterations || j + 1 >= m;
      if (!end) {
        scale_kernel<<<nb_(n, 256), 256, 0, s>>>(Q.w.p, nullptr, 1.0 / hn, Q.V.p + (size_t)(j + 1) * n, n);
        RSG_LAUNCHED(ctx, "scale");
        Q.j = j + 1;
        continue;
      }
      // back substitution H y = g, x += Z y (cycle_end, gmres.rs:515-541)
      int kk = j + 1;
      std::vector<double> y(kk);
      for (int t = kk - 1; t >= 0; --t) {
        double sum = Q.g[t];
        for (int l = t + 1; l < kk; ++l) sum -= Q.H[(size_t)t * m + l] * y[l];
        double d = Q.H[(size_t)t * m + t];
        y[t] = d != 0.0 ? sum / d : 0.0;
      }
      RSG_CUDA("gmres", rsg::copy_async(Q.h.p, y.data(), kk * sizeof(double), cudaMemcpyHostToDevice, s));
      axpy_many_kernel<<<nb_(n, 256), 256, 0, s>>>(Q.zptr.p, kk, Q.h.p, 1.0, x + (size_t)act[i] * n, n);
      RSG_LAUNCHED(ctx, "axpy_many");
      RSG_CUDA("gmres", cudaStreamSynchronize(s));  // y lives on the host stack
      Q.active = false;
      Q.j = -1;  // cycle ended
      any_end = true;
    }
    if (any_end) {
      // solves whose cycle ended restart (explicit residual); the others continue
      std::vector<bool> restart(nb, false);
      for (int q = 0; q < nb; ++q)
        if (!R[q].done && R[q].j == -1) restart[q] = true;
      // run cycle_start only for the restarting solves
      std::vector<bool> saved(nb);
      for (int q = 0; q < nb; ++q) {
        saved[q] = R[q].done;
        if (!restart[q]) R[q].done = true;
      }
      cycle_start(false);
      for (int q = 0; q < nb; ++q)
        if (!restart[q]) R[q].done = saved[q];
    }
  }
  double secs = std::chrono::duration<double>(clk::now() - t0).count();
  reports.assign(nb, GmresReport());
  for (int q = 0; q < nb; ++q) R[q].rep.seconds = secs, reports[q] = R[q].rep;
  for (int q = 0; q < nb; ++q) {
    if (!R[q].rep.converged && !(R[q].rep.relative_residual <= 0.1))
      fail(RS_SOLVER_DIVERGED, "SolverDiverged", "gmres",
           "true relative residual " + std::to_string(R[q].rep.relative_residual));
  }
}

double dev_norm(rs_ctx *ctx, const double *w, size_t n) {
  DevBuf<double> out(1);
  dev_dots(ctx, nullptr, 1, w, n, out.p, w, false);
  double v;
  RSG_CUDA("gmres", rsg::copy_async(&v, out.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  RSG_CUDA("gmres", cudaStreamSynchronize(ctx->stream));
  return std::sqrt(v);
}

}  // namespace rsg
