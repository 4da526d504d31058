// The dense last resort of the recovery chain on the device (see dense.hpp): the exact metric
// assembled column by column from products with unit vectors, bordered by the barycenter rows,
// equilibrated, and factored by a right-looking LU with partial pivoting in FP64 (one pivot
// kernel and one rank-1 update per column; at most 6,003 columns, so the factor takes a few
// hundred milliseconds, a last resort after two GMRES runs failed).
#include <cmath>

#include "dense.hpp"

namespace rsg {
namespace {

inline unsigned nblk(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// Three stacked 3V vectors: vector q has a one in axis a at vertex v0 + 3 q + a (if < nv).
__global__ void unit_columns_kernel(int nv, int v0, double *x) {
  const size_t nd = 3 * (size_t)nv, t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= 3 * nd) return;
  const int q = (int)(t / nd);
  const size_t i = t - (size_t)q * nd;
  const int w = (int)(i / 3), a = (int)(i % 3);
  x[t] = (w == v0 + 3 * q + a) ? 1.0 : 0.0;
}

// K[w, v] = (A e_v)_w for the nine columns v = v0 + 3 q + a of one product.
__global__ void scatter_columns_kernel(int nv, int n, int v0, const double *y, double *K) {
  const size_t nd = 3 * (size_t)nv, t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= 9 * (size_t)nv) return;
  const int qa = (int)(t / nv), w = (int)(t % nv);
  const int q = qa / 3, a = qa % 3, v = v0 + qa;
  if (v >= nv) return;
  K[w + (size_t)v * n] = y[(size_t)q * nd + 3 * (size_t)w + a];
}

// The border: K[V + g, v] = K[v, V + g] = c_v for the group g of v.
__global__ void border_kernel(int nv, int n, const uint32_t *group, const double *c, double *K) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const size_t r = (size_t)nv + group[v];
  K[r + (size_t)v * n] = c[v];
  K[v + r * n] = c[v];
}

// equilibration (dense.rs:289-307): 1/sqrt(K_jj) for the primal unknowns (1 if K_jj <= 0 or
// not finite); a border row r gets 1/|row r after the primal scaling| (1 if zero). One block
// per border row after the primal ones.
__global__ void equilibrate_primal_kernel(int nv, int n, const double *K, double *d) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nv) return;
  const double x = K[j + (size_t)j * n];
  d[j] = (x > 0.0 && isfinite(x)) ? 1.0 / sqrt(x) : 1.0;
}
__global__ void equilibrate_rows_kernel(int nv, int n, const double *K, double *d) {
  const int r = nv + blockIdx.x;
  __shared__ double part[32];
  double s = 0.0;
  for (int j = threadIdx.x; j < nv; j += blockDim.x) {
    const double x = K[r + (size_t)j * n] * d[j];
    s += x * x;
  }
  for (int m = 16; m >= 1; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
    d[r] = t > 0.0 ? 1.0 / sqrt(t) : 1.0;
  }
}

__global__ void scale_kernel(int n, const double *K, const double *d, double *LU) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)n * n) return;
  const int i = (int)(t % n), j = (int)(t / n);
  LU[t] = d[i] * K[t] * d[j];
}

// Column k: the pivot row p = argmax_{i >= k} |A[i, k]| (lowest index on ties), rows k and p
// interchanged across all columns, then the multipliers A[i, k] / A[k, k] below the diagonal.
__global__ void __launch_bounds__(1024) lu_pivot_kernel(int n, int k, double *A, int *perm) {
  __shared__ double bv[32];
  __shared__ int bi[32];
  __shared__ int p_s;
  double best = -1.0;
  int arg = n;
  for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
    const double x = fabs(A[i + (size_t)k * n]);
    if (x > best) best = x, arg = i;  // ascending i per thread: the first maximum
  }
  for (int m = 16; m >= 1; m >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, m);
    const int oa = __shfl_xor_sync(0xffffffffu, arg, m);
    if (ob > best || (ob == best && oa < arg)) best = ob, arg = oa;
  }
  if ((threadIdx.x & 31) == 0) bv[threadIdx.x >> 5] = best, bi[threadIdx.x >> 5] = arg;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = bv[0];
    int a = bi[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      if (bv[w] > b || (bv[w] == b && bi[w] < a)) b = bv[w], a = bi[w];
    p_s = a < n ? a : k;
    perm[k] = p_s;
  }
  __syncthreads();
  const int p = p_s;
  if (p != k)
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      const double t = A[k + (size_t)j * n];
      A[k + (size_t)j * n] = A[p + (size_t)j * n];
      A[p + (size_t)j * n] = t;
    }
  __syncthreads();
  const double akk = A[k + (size_t)k * n];
  if (akk != 0.0)
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[i + (size_t)k * n] /= akk;
}

// The trailing update A[i, j] -= A[i, k] A[k, j] for i, j > k: threads over i (coalesced in
// the column-major layout), blocks over 64 columns.
__global__ void lu_update_kernel(int n, int k, double *A) {
  const int i = k + 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j0 = k + 1 + blockIdx.y * 64, j1 = min(n, j0 + 64);
  const double l = A[i + (size_t)k * n];
  if (l == 0.0) return;
  for (int j = j0; j < j1; ++j) A[i + (size_t)j * n] -= l * A[k + (size_t)j * n];
}

// out[0] = min |u_ii|, out[1] = max |u_ii|, out[2] = 1 if a pivot is not finite (one block).
__global__ void pivot_range_kernel(int n, const double *A, double *out) {
  __shared__ double lo_s[32], hi_s[32];
  __shared__ int bad_s[32];
  double lo = INFINITY, hi = 0.0;
  int bad = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double u = fabs(A[i + (size_t)i * n]);
    if (!isfinite(u)) bad = 1;
    else lo = fmin(lo, u), hi = fmax(hi, u);
  }
  for (int m = 16; m >= 1; m >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, m));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, m));
    bad |= __shfl_xor_sync(0xffffffffu, bad, m);
  }
  if ((threadIdx.x & 31) == 0) lo_s[threadIdx.x >> 5] = lo, hi_s[threadIdx.x >> 5] = hi, bad_s[threadIdx.x >> 5] = bad;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) lo = fmin(lo, lo_s[w]), hi = fmax(hi, hi_s[w]), bad |= bad_s[w];
    out[0] = lo, out[1] = hi, out[2] = bad;
  }
}

// B = D R (the refinement's right-hand side in the column layout).
__global__ void scale_rows_kernel(size_t m, int n, const double *R, const double *d, double *B) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t < m) B[t] = d[t % n] * R[t];
}

// The columns b_m of B (n x m, column-major): b_m[i] = d_i rhs_q[i] of axis a (m = 3 q + a).
__global__ void gather_rhs_kernel(int nv, int n, int nb, const double *rhs, size_t ld, const double *d,
                                  double *B) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)3 * nb * n) return;
  const int m = (int)(t / n), i = (int)(t % n), q = m / 3, a = m % 3;
  const size_t nd = 3 * (size_t)nv;
  const double r = i < nv ? rhs[q * ld + 3 * (size_t)i + a] : rhs[q * ld + nd + 3 * (size_t)(i - nv) + a];
  B[t] = d[i] * r;
}

// One column per block: b <- (P^T L U)^-1 b (the interchanges in order, then the unit lower
// and the upper triangle), then b_i <- d_i b_i.
__global__ void __launch_bounds__(1024) lu_solve_kernel(int n, const double *A, const int *perm, const double *d,
                                                        double *B) {
  double *b = B + (size_t)blockIdx.x * n;
  if (threadIdx.x == 0)
    for (int k = 0; k < n; ++k) {
      const int p = perm[k];
      if (p != k) {
        const double t = b[k];
        b[k] = b[p], b[p] = t;
      }
    }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    const double bk = b[k];
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) b[i] -= A[i + (size_t)k * n] * bk;
    __syncthreads();
  }
  for (int k = n - 1; k >= 0; --k) {
    if (threadIdx.x == 0) b[k] /= A[k + (size_t)k * n];
    __syncthreads();
    const double bk = b[k];
    for (int i = threadIdx.x; i < k; i += blockDim.x) b[i] -= A[i + (size_t)k * n] * bk;
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) b[i] *= d[i];
}

// sol_q (+)= the columns of B back in the [x (3V); l (3G)] layout.
__global__ void scatter_sol_kernel(int nv, int n, int nb, const double *B, size_t ld, double *sol, int add) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)3 * nb * n) return;
  const int m = (int)(t / n), i = (int)(t % n), q = m / 3, a = m % 3;
  const size_t nd = 3 * (size_t)nv;
  double &o = i < nv ? sol[q * ld + 3 * (size_t)i + a] : sol[q * ld + nd + 3 * (size_t)(i - nv) + a];
  o = add ? o + B[t] : B[t];
}

// r = rhs - A' sol per axis column with the unscaled K: R[m][i] = rhs_q[i, a] - sum_j K[i, j]
// sol_q[j, a]; thread per (row i, column m).
__global__ void residual_kernel(int nv, int n, int nb, const double *K, const double *rhs, const double *sol,
                                size_t ld, double *R) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)3 * nb * n) return;
  const int m = (int)(t / n), i = (int)(t % n), q = m / 3, a = m % 3;
  const size_t nd = 3 * (size_t)nv;
  auto at = [&](const double *v, int j) {
    return j < nv ? v[q * ld + 3 * (size_t)j + a] : v[q * ld + nd + 3 * (size_t)(j - nv) + a];
  };
  double s = 0.0;
  for (int j = 0; j < n; ++j) s += K[i + (size_t)j * n] * at(sol, j);
  R[t] = at(rhs, i) - s;
}

// rel[q] = |R_q| / |rhs_q| over the three axis columns of vector q (one block per vector).
__global__ void rel_kernel(int nv, int n, const double *R, const double *rhs, size_t ld, double *rel) {
  const int q = blockIdx.x;
  __shared__ double sr[32], sb[32];
  double r2 = 0.0, b2 = 0.0;
  for (int t = threadIdx.x; t < 3 * n; t += blockDim.x) {
    const double x = R[(size_t)q * 3 * n + t];
    r2 += x * x;
  }
  for (size_t i = threadIdx.x; i < ld; i += blockDim.x) {
    const double x = rhs[q * ld + i];
    b2 += x * x;
  }
  for (int m = 16; m >= 1; m >>= 1) {
    r2 += __shfl_xor_sync(0xffffffffu, r2, m);
    b2 += __shfl_xor_sync(0xffffffffu, b2, m);
  }
  if ((threadIdx.x & 31) == 0) sr[threadIdx.x >> 5] = r2, sb[threadIdx.x >> 5] = b2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a += sr[w], b += sb[w];
    rel[q] = b > 0.0 ? sqrt(a / b) : sqrt(a);
  }
}

}  // namespace

void DenseSaddleDev::build(rs_ctx *c, int nv_, int G_, const uint32_t *group_dev, const double *c_dev,
                           const std::function<void(int, const double *, double *)> &metric) {
  ctx = c, nv = nv_, G = G_, n = nv + G;
  cudaStream_t s = ctx->stream;
  const size_t nn = (size_t)n * n, nd = 3 * (size_t)nv;
  K.alloc(nn), LU.alloc(nn), d.alloc(n), perm.alloc(n), X.alloc(3 * nd), Y.alloc(3 * nd), piv.alloc(3);
  RSG_CUDA("solver", cudaMemsetAsync(K.p, 0, nn * sizeof(double), s));
  for (int v0 = 0; v0 < nv; v0 += 9) {
    unit_columns_kernel<<<nblk(3 * nd, 256), 256, 0, s>>>(nv, v0, X.p);
    RSG_LAUNCHED(ctx, "dense_units");
    metric(3, X.p, Y.p);
    scatter_columns_kernel<<<nblk(9 * (size_t)nv, 256), 256, 0, s>>>(nv, n, v0, Y.p, K.p);
    RSG_LAUNCHED(ctx, "dense_columns");
  }
  border_kernel<<<nblk(nv, 256), 256, 0, s>>>(nv, n, group_dev, c_dev, K.p);
  RSG_LAUNCHED(ctx, "dense_border");
  equilibrate_primal_kernel<<<nblk(nv, 256), 256, 0, s>>>(nv, n, K.p, d.p);
  RSG_LAUNCHED(ctx, "dense_equilibrate");
  equilibrate_rows_kernel<<<G, 256, 0, s>>>(nv, n, K.p, d.p);
  RSG_LAUNCHED(ctx, "dense_equilibrate");
  scale_kernel<<<nblk(nn, 256), 256, 0, s>>>(n, K.p, d.p, LU.p);
  RSG_LAUNCHED(ctx, "dense_scale");
  for (int k = 0; k < n; ++k) {
    lu_pivot_kernel<<<1, 1024, 0, s>>>(n, k, LU.p, perm.p);
    RSG_LAUNCHED(ctx, "dense_lu_pivot");
    const int m = n - k - 1;
    if (m > 0) {
      lu_update_kernel<<<dim3(nblk(m, 256), nblk(m, 64)), 256, 0, s>>>(n, k, LU.p);
      RSG_LAUNCHED(ctx, "dense_lu_update");
    }
  }
  pivot_range_kernel<<<1, 1024, 0, s>>>(n, LU.p, piv.p);
  RSG_LAUNCHED(ctx, "dense_lu_pivots");
  double pr[3] = {0.0, 0.0, 0.0};
  RSG_CUDA("solver", copy_async(pr, piv.p, sizeof(pr), cudaMemcpyDeviceToHost, s));
  RSG_CUDA("solver", cudaStreamSynchronize(s));
  // Lu::new (dense.rs:82-97): a non-finite pivot, or an equilibrated pivot ratio at most
  // PIVOT_TOLERANCE (1e-13), is a singular saddle
  pivot_ratio = (pr[1] > 0.0) ? pr[0] / pr[1] : 0.0;
  if (pr[2] != 0.0 || !(pivot_ratio > 1e-13))
    fail(RS_SINGULAR, "SingularSaddle", "solver",
         "dense LU pivot ratio " + std::to_string(pivot_ratio) + " at or below 1e-13");
}

void DenseSaddleDev::solve(int nb, const double *rhs, double *sol, double *rel) {
  cudaStream_t s = ctx->stream;
  const size_t ld = 3 * (size_t)nv + 3 * (size_t)G, m = (size_t)3 * nb * n;
  if (B.n < m) B.alloc(m), R.alloc(m);
  DevBuf<double> reld(nb);
  gather_rhs_kernel<<<nblk(m, 256), 256, 0, s>>>(nv, n, nb, rhs, ld, d.p, B.p);
  RSG_LAUNCHED(ctx, "dense_rhs");
  lu_solve_kernel<<<3 * nb, 1024, 0, s>>>(n, LU.p, perm.p, d.p, B.p);
  RSG_LAUNCHED(ctx, "dense_lu_solve");
  scatter_sol_kernel<<<nblk(m, 256), 256, 0, s>>>(nv, n, nb, B.p, ld, sol, 0);
  RSG_LAUNCHED(ctx, "dense_sol");
  // one step of iterative refinement: sol += A'^-1 (rhs - A' sol)
  residual_kernel<<<nblk(m, 256), 256, 0, s>>>(nv, n, nb, K.p, rhs, sol, ld, R.p);
  RSG_LAUNCHED(ctx, "dense_residual");
  scale_rows_kernel<<<nblk(m, 256), 256, 0, s>>>(m, n, R.p, d.p, B.p);
  RSG_LAUNCHED(ctx, "dense_rhs");
  lu_solve_kernel<<<3 * nb, 1024, 0, s>>>(n, LU.p, perm.p, d.p, B.p);
  RSG_LAUNCHED(ctx, "dense_lu_solve");
  scatter_sol_kernel<<<nblk(m, 256), 256, 0, s>>>(nv, n, nb, B.p, ld, sol, 1);
  RSG_LAUNCHED(ctx, "dense_sol");
  residual_kernel<<<nblk(m, 256), 256, 0, s>>>(nv, n, nb, K.p, rhs, sol, ld, R.p);
  RSG_LAUNCHED(ctx, "dense_residual");
  rel_kernel<<<nb, 256, 0, s>>>(nv, n, R.p, rhs, ld, reld.p);
  RSG_LAUNCHED(ctx, "dense_residual");
  RSG_CUDA("solver", copy_async(rel, reld.p, nb * sizeof(double), cudaMemcpyDeviceToHost, s));
  RSG_CUDA("solver", cudaStreamSynchronize(s));
}

}  // namespace rsg
