// The hierarchical saddle solver of one step on the GPU (HierarchicalSaddle =
// GmresSaddle<HierarchicalOperator, SparsePreconditioner>, RS/src/solve/iterative.rs:126-575,
// RS/src/solve/precond.rs, RS/src/solve/gmres.rs) and the constrained direction
// (SchurComplement, RS/src/solve/schur.rs), behind rs_solver_* of include/rsgpu.h.
//
//   A' [x; l] = [ w (B~ + c_lo B~0) x + C_Q^T l ; C_Q x ]                       (operator)
//   P^-1 = L'^-1 + L'^-1 blockdiag((s L^V_{2-s} - K) x I3, 0) L'^-1             (augmented form)
//   L' = [[K x I3, C_Q^T], [C_Q, 0]],  K = W + eps M
//
// C_Q holds the barycenter rows (global or per component: c_v = a_v / A_group per axis). The
// reference factors L' by a sparse LDL^T; here L'^-1 is applied as: mu = 1_g^T r - eps A_g b
// per group and axis (exact: 1^T K = eps m^T), y = MG(K, r - c mu) by smoothed-aggregation
// multigrid V-cycles, then y is shifted by a constant per group so that C_Q y = b holds
// exactly. The preconditioner is a fixed linear map (fixed V-cycles), so plain right
// preconditioning applies; GMRES stores the preconditioned vectors anyway (flexible form).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <future>
#include <memory>
#include <optional>
#include <numeric>
#include <string>
#include <vector>

#include "amg.hpp"
#include "common.hpp"
#include "hmat.hpp"
#include "host_tree.hpp"
#include "krylov.hpp"
#include "learned.hpp"
#include "dense.hpp"
#include "profile.hpp"

namespace rsg {

namespace {

inline unsigned nblk(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }
constexpr int GB = 128;  // reduction blocks of the group sums

// The end of a group-sum launch: the block's K partials are in part; the last block to finish
// (a ticket counter, reset by that block) adds every entry's partials in block order, a warp
// per entry with the lanes strided over the blocks, and writes out.
__device__ __forceinline__ void finish_group_sums(const double *part, int K, unsigned *ticket, double *out) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const int lane = threadIdx.x & 31;
  for (int i = threadIdx.x >> 5; i < K; i += (int)(blockDim.x >> 5)) {
    double t = 0.0;
    for (unsigned b = lane; b < gridDim.x; b += 32) t += __ldcg(part + (size_t)b * K + i);
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) out[i] = t;
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

// part[b][q][3 g + k] = sum over the block's vertices v of group g of wgt_v x_q[3 v + k]
// (wgt = null: weight 1). x has leading dimension ld; G groups.
__global__ void group_sums_partial(const double *__restrict__ x, size_t ld, int nb, int nv,
                                   const uint32_t *__restrict__ group, const double *__restrict__ wgt,
                                   int G, double *part, unsigned *ticket, double *out) {
  extern __shared__ double sh[];  // 3 G nb per block
  const int K = 3 * G * nb;
  for (int i = threadIdx.x; i < K; i += blockDim.x) sh[i] = 0.0;
  __syncthreads();
  const size_t chunk = (nv + gridDim.x - 1) / gridDim.x;
  const size_t v0 = blockIdx.x * chunk, v1 = min((size_t)nv, v0 + chunk);
  // each thread accumulates privately over a strided subset, then a fixed-order tree
  for (int q = 0; q < nb; ++q)
    for (int g = 0; g < G; ++g)
      for (int k = 0; k < 3; ++k) {
        double acc = 0.0;
        for (size_t v = v0 + threadIdx.x; v < v1; v += blockDim.x)
          if ((int)group[v] == g) acc += (wgt ? wgt[v] : 1.0) * x[q * ld + 3 * v + k];
        // warp tree then lane-0 adds in warp order
        for (int m = 16; m >= 1; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
        __shared__ double wsum[32];
        if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
          double t = 0.0;
          for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[w];
          sh[(q * G + g) * 3 + k] = t;
        }
        __syncthreads();
      }
  for (int i = threadIdx.x; i < K; i += blockDim.x) part[(size_t)blockIdx.x * K + i] = sh[i];
  finish_group_sums(part, K, ticket, out);
}


// Operator tail: y_pos += c_v l_{g(v)} and y_mult = C_Q x (from the group sums `cx`).
__global__ void cq_apply_kernel(const double *__restrict__ x, double *__restrict__ y, size_t ld,
                                int nb, int nv, const uint32_t *__restrict__ group,
                                const double *__restrict__ c, int G, const double *__restrict__ cx) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  size_t nd = 3 * (size_t)nv;
  if (t >= (size_t)nb * (nd + 3 * G)) return;
  int q = (int)(t / (nd + 3 * G));
  size_t i = t % (nd + 3 * G);
  if (i < nd) {
    size_t v = i / 3;
    int k = (int)(i % 3);
    y[q * ld + i] += c[v] * x[q * ld + nd + 3 * group[v] + k];
  } else {
    y[q * ld + i] = cx[(size_t)q * 3 * G + (i - nd)];
  }
}

// mu = 1_g^T r - eps A_g b (per vector, group, axis), from the group sums s1 = 1_g^T r.
__global__ void mu_kernel(const double *__restrict__ s1, const double *__restrict__ r, size_t ld,
                          size_t nd, int nb, int G, const double *__restrict__ eps_area, double *mu) {
  int t = threadIdx.x + blockIdx.x * blockDim.x;
  if (t >= nb * 3 * G) return;
  int q = t / (3 * G), i = t % (3 * G), g = i / 3;
  mu[t] = s1[t] - eps_area[g] * r[q * ld + nd + i];
}

// AMG layout [v][3 nb] <- r_q[3 v + k] - c_v mu_{q, g(v), k}
__global__ void to_mg_kernel(const double *__restrict__ r, size_t ld, int nb, int nv,
                             const uint32_t *__restrict__ group, const double *__restrict__ c,
                             const double *__restrict__ mu, int G, mgreal *__restrict__ out) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)nv * 3 * nb) return;
  size_t v = t / (3 * nb);
  int col = (int)(t % (3 * nb)), q = col / 3, k = col % 3;
  double sub = mu ? c[v] * mu[(size_t)q * 3 * G + 3 * group[v] + k] : 0.0;
  out[t] = (mgreal)(r[q * ld + 3 * v + k] - sub);
}

// y_q[3 v + k] = yy[v][3 q + k] + shift_{q, g(v), k}, y_q[nd + 3 g + k] = mu (multipliers).
__global__ void from_mg_kernel(const mgreal *__restrict__ yy, double *__restrict__ y, size_t ld,
                               int nb, int nv, const uint32_t *__restrict__ group, int G,
                               const double *__restrict__ shift, const double *__restrict__ mu,
                               const double *__restrict__ add) {
  size_t nd = 3 * (size_t)nv;
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)nb * (nd + 3 * G)) return;
  int q = (int)(t / (nd + 3 * G));
  size_t i = t % (nd + 3 * G);
  double val;
  if (i < nd) {
    size_t v = i / 3;
    int k = (int)(i % 3);
    val = (double)yy[v * 3 * nb + 3 * q + k] + shift[(size_t)q * 3 * G + 3 * group[v] + k];
  } else {
    val = mu[(size_t)q * 3 * G + (i - nd)];
  }
  y[q * ld + i] = add ? val + add[q * ld + i] : val;
}

// shift = b - C_Q y' per vector, group, axis (from the weighted group sums of y').
__global__ void shift_kernel(const double *__restrict__ cy, const double *__restrict__ r, size_t ld,
                             size_t nd, int nb, int G, double *shift) {
  int t = threadIdx.x + blockIdx.x * blockDim.x;
  if (t >= nb * 3 * G) return;
  int q = t / (3 * G), i = t % (3 * G);
  shift[t] = r[q * ld + nd + i] - cy[t];
}

// ---- the coarse space (CoarseSpace, RS/src/solve/coarse.rs:101-327): columns 3 k + a are the
// translations of free component slot k along axis a, scaled by 1/sqrt(|members|); the last
// n_rows columns are the multipliers of the positional rows that touch a free component.

// t[q][j] = (Z^T x_q)_j from the slot sums gs[q][3 k + a] (slot n_free collects the vertices
// of fixed components) and the multiplier entries of x.
__global__ void coarse_zt_kernel(const double *__restrict__ gs, int gstride, const double *__restrict__ x,
                                 size_t ld, size_t nd, int nb, int nfree, const double *__restrict__ scale,
                                 const int *__restrict__ rows, int nrows, double *__restrict__ t) {
  const int cm = 3 * nfree + nrows;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb * cm) return;
  int q = i / cm, j = i % cm;
  t[i] = j < 3 * nfree ? scale[j / 3] * gs[(size_t)q * gstride + j] : x[q * ld + nd + rows[j - 3 * nfree]];
}

// out[q][i] = sum_j E+[i][j] t[q][j]; with sub, out = sub - that
__global__ void coarse_esolve_kernel(const double *__restrict__ epinv, const double *__restrict__ t, int nb, int cm,
                                     const double *__restrict__ sub, double *__restrict__ out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb * cm) return;
  int q = k / cm, i = k % cm;
  double s = 0.0;
  for (int j = 0; j < cm; ++j) s += epinv[i * cm + j] * t[q * cm + j];
  out[k] = sub ? sub[k] - s : s;
}

// rp_q = r_q - (A'Z) yc_q
__global__ void coarse_sub_kernel(const double *__restrict__ r, double *__restrict__ rp, size_t ld, size_t n, int nb,
                                  const double *__restrict__ az, const double *__restrict__ yc, int cm) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)nb * n) return;
  int q = (int)(t / n);
  size_t i = t % n;
  double s = r[q * ld + i];
  for (int j = 0; j < cm; ++j) s -= az[(size_t)j * n + i] * yc[q * cm + j];
  rp[q * ld + i] = s;
}

// part[b][q][j] = the chunk b partial of (A'Z)_j . z_q (fixed chunks, fixed order in a chunk)
constexpr int kCoarseChunks = 128;
__global__ void coarse_azt_partial(const double *__restrict__ az, const double *__restrict__ z, size_t ld, size_t n,
                                   int nb, int cm, double *__restrict__ part) {
  const int b = blockIdx.x, qj = blockIdx.y, q = qj / cm, j = qj % cm;
  const size_t chunk = (n + kCoarseChunks - 1) / kCoarseChunks, i0 = b * chunk, i1 = min(n, i0 + chunk);
  double s = 0.0;
  for (size_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) s += az[(size_t)j * n + i] * z[q * ld + i];
  __shared__ double ws[8];
  for (int m = 16; m >= 1; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
    part[(size_t)b * nb * cm + qj] = t;
  }
}
__global__ void coarse_azt_finish(const double *__restrict__ part, int nbcm, double *__restrict__ out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nbcm) return;
  double s = 0.0;
  for (int b = 0; b < kCoarseChunks; ++b) s += part[(size_t)b * nbcm + k];
  out[k] = s;
}

// z_q += Z c_q
__global__ void coarse_addz_kernel(double *__restrict__ z, size_t ld, size_t nd, size_t n, int nb,
                                   const uint32_t *__restrict__ slot_of_vertex, int nfree,
                                   const double *__restrict__ scale, const int *__restrict__ rowcol,
                                   const double *__restrict__ c, int cm) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)nb * n) return;
  int q = (int)(t / n);
  size_t i = t % n;
  if (i < nd) {
    const uint32_t k = slot_of_vertex[i / 3];
    if ((int)k < nfree) z[q * ld + i] += scale[k] * c[q * cm + 3 * k + (int)(i % 3)];
  } else {
    const int j = rowcol[i - nd];
    if (j >= 0) z[q * ld + i] += c[q * cm + j];
  }
}

// Symmetric eigendecomposition (m x m, row-major) by cyclic Jacobi rotations: the coarse matrix
// has 3 columns per free component and one per multiplier row.
void jacobi_eigen(int m, std::vector<double> a, std::vector<double> &lam, std::vector<double> &u) {
  u.assign((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) u[(size_t)i * m + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        const double x = a[(size_t)i * m + j] * a[(size_t)i * m + j];
        tot += x;
        if (i != j) off += x;
      }
    if (!(off > 1e-30 * tot)) break;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) {
        const double apq = a[(size_t)p * m + q];
        if (apq == 0.0) continue;
        const double th = 0.5 * (a[(size_t)q * m + q] - a[(size_t)p * m + p]) / apq;
        const double t = (th >= 0.0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < m; ++k) {
          const double akp = a[(size_t)k * m + p], akq = a[(size_t)k * m + q];
          a[(size_t)k * m + p] = c * akp - sn * akq, a[(size_t)k * m + q] = sn * akp + c * akq;
        }
        for (int k = 0; k < m; ++k) {
          const double apk = a[(size_t)p * m + k], aqk = a[(size_t)q * m + k];
          a[(size_t)p * m + k] = c * apk - sn * aqk, a[(size_t)q * m + k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < m; ++k) {
          const double ukp = u[(size_t)k * m + p], ukq = u[(size_t)k * m + q];
          u[(size_t)k * m + p] = c * ukp - sn * ukq, u[(size_t)k * m + q] = sn * ukp + c * ukq;
        }
      }
  }
  lam.resize(m);
  for (int i = 0; i < m; ++i) lam[i] = a[(size_t)i * m + i];
}

// Planar symbol ratio 4 I(sigma) I(2 - s) of W^-1 L_{2-s} W^-1 B, I(t) = pi Gamma(1-t) /
// (t 4^t Gamma(1+t)) (fractional_symbol_ratio, RS/src/solve/precond.rs:548-568).
double symbol_ratio(double s) {
  auto I = [](double t) { return M_PI * std::tgamma(1.0 - t) / (t * std::pow(4.0, t) * std::tgamma(1.0 + t)); };
  return 4.0 * I(s - 1.0) * I(2.0 - s);
}

}  // namespace

}  // namespace rsg

using namespace rsg;

struct rs_solver {
  rs_ctx *ctx = nullptr;
  int nv = 0, nf = 0, G = 1;
  size_t nd = 0, n = 0;
  rs_metric *metric = nullptr;
  rs_vfrac *vfrac = nullptr;
  double w_hi = 1.0, w_lo = 1.0, frac_scale = 1.0, eps = 0.0;
  bool use_prec = true;
  int vcycles = 1;
  double build_times[6] = {0, 0, 0, 0, 0, 0};
  Profiler prof;
  // learned preconditioner (optional): z = learned(r, P_cheap^-1 r), plain solver as fallback
  rs_learned *lmodel = nullptr;
  rs_lgraph *lgraph = nullptr;
  int l_cheap = 2, l_cap = 0;
  int64_t l_solves = 0, l_fallbacks = 0;
  DevBuf<double> lbuf;
  Operator lprec;
  GmresOptions gopt;
  FaceGeom geom;
  std::vector<double> vmass;
  std::vector<uint32_t> group_h;
  AmgDevice amg;
  DevBuf<uint32_t> group;
  DevBuf<double> c, eps_area, part, s1, mu, cy, shift, tmp, tmp2;
  DevBuf<unsigned> gs_ticket;  // blocks done in the current group-sum launch (0 between launches)
  DevBuf<mgreal> mg_in, mg_out;  // right-hand sides and solutions on the multigrid layout
  std::vector<GmresReport> last;
  Operator op, prec;
  // the Arnoldi steps on the inner operator (plain near-field sums, also in the preconditioner's
  // vertex product), every cycle-start residual and the convergence test on op
  bool inner_plain = true;
  Operator op_inner;
  // the coarse space (coarse.rs): cm columns, 0 when every component is fixed by rows of its own
  int cm = 0, c_nfree = 0;
  std::vector<int> c_rows_h;                // multiplier rows touching a free component
  DevBuf<uint32_t> c_slot;                  // per vertex: free slot of its component, n_free if fixed
  DevBuf<double> c_scale, c_az, c_epinv;    // per slot 1/sqrt(|members|); A'Z (n x cm); E+ (cm x cm)
  DevBuf<int> c_rows, c_rowcol;             // the rows; per multiplier row its column or -1
  DevBuf<double> c_t, c_yc, c_t2, c_part, c_rp;
  double c_conditioning = 0.0;
  int c_dropped = 0;
  // the dense last resort (at most kDenseMaxVertices vertices): the surface kept on the host for
  // the exact metric, and the factor once built
  std::vector<uint32_t> faces_h;
  std::vector<double> pos_h;
  double alpha = 6.0, beta = 12.0;
  int leaf_size = 8, leaf_pairs = 64;
  std::unique_ptr<DenseSaddleDev> dense;

  cudaStream_t st() const { return ctx->stream; }

  // group sums (weighted by c or not) of nb vectors into out [nb][3G]
  void group_sums(const double *x, size_t ld, int nb, const double *wgt, double *out) {
    group_sums_by(x, ld, nb, wgt, group.p, G, out);
  }
  void group_sums_by(const double *x, size_t ld, int nb, const double *wgt, const uint32_t *grp, int ng,
                     double *out) {
    int K = 3 * ng * nb;
    if (part.n < (size_t)GB * K) part.alloc((size_t)GB * K);
    group_sums_partial<<<GB, 256, (size_t)K * sizeof(double), st()>>>(x, ld, nb, nv, grp, wgt, ng, part.p,
                                                                      gs_ticket.p, out);
    RSG_LAUNCHED(ctx, "group_sums");
  }

  // t = Z^T x for nb vectors (ld n) into t [nb][cm]
  void coarse_zt(int nb, const double *x, double *t) {
    const int ng = c_nfree + 1;
    group_sums_by(x, n, nb, nullptr, c_slot.p, ng, c_part.p);
    coarse_zt_kernel<<<nblk((size_t)nb * cm, 128), 128, 0, st()>>>(c_part.p, 3 * ng, x, n, nd, nb, c_nfree,
                                                                  c_scale.p, c_rows.p, (int)c_rows_h.size(), t);
    RSG_LAUNCHED(ctx, "coarse_zt");
  }

  // the balancing preconditioner around the fine one (CoarseSpace::apply_many, coarse.rs:296-327):
  // yc = E+ Z^T r, z = P^-1 (r - A'Z yc), z += Z (yc - E+ (A'Z)^T z)
  void apply_prec_coarse(int nb, const double *r, double *z, int steps) {
    const size_t nbcm = (size_t)nb * cm;
    if (c_t.n < nbcm) c_t.alloc(nbcm), c_yc.alloc(nbcm), c_t2.alloc(nbcm);
    if (c_rp.n < (size_t)nb * n) c_rp.alloc((size_t)nb * n);
    coarse_zt(nb, r, c_t.p);
    coarse_esolve_kernel<<<nblk(nbcm, 128), 128, 0, st()>>>(c_epinv.p, c_t.p, nb, cm, nullptr, c_yc.p);
    RSG_LAUNCHED(ctx, "coarse_esolve");
    coarse_sub_kernel<<<nblk((size_t)nb * n, 256), 256, 0, st()>>>(r, c_rp.p, n, n, nb, c_az.p, c_yc.p, cm);
    RSG_LAUNCHED(ctx, "coarse_sub");
    apply_prec_fine(nb, c_rp.p, z, steps);
    coarse_azt_partial<<<dim3(kCoarseChunks, (unsigned)nbcm), 256, 0, st()>>>(c_az.p, z, n, n, nb, cm, c_part.p);
    RSG_LAUNCHED(ctx, "coarse_azt");
    coarse_azt_finish<<<nblk(nbcm, 128), 128, 0, st()>>>(c_part.p, (int)nbcm, c_t.p);
    RSG_LAUNCHED(ctx, "coarse_azt_finish");
    coarse_esolve_kernel<<<nblk(nbcm, 128), 128, 0, st()>>>(c_epinv.p, c_t.p, nb, cm, c_yc.p, c_t2.p);
    RSG_LAUNCHED(ctx, "coarse_esolve");
    coarse_addz_kernel<<<nblk((size_t)nb * n, 256), 256, 0, st()>>>(z, n, nd, n, nb, c_slot.p, c_nfree, c_scale.p,
                                                                    c_rowcol.p, c_t2.p, cm);
    RSG_LAUNCHED(ctx, "coarse_addz");
  }

  void reserve(int nb) {
    size_t K = (size_t)3 * G * nb;
    if (s1.n < K) s1.alloc(K), mu.alloc(K), cy.alloc(K), shift.alloc(K);
    size_t m = (size_t)nv * 3 * nb;
    if (mg_in.n < m) mg_in.alloc(m), mg_out.alloc(m);
    if (tmp.n < (size_t)nb * n) tmp.alloc((size_t)nb * n), tmp2.alloc((size_t)nb * n);
  }

  // A' x
  // plain: the inner operator of the Arnoldi steps (the near field in plain FP32 sums)
  void apply_op(int nb, const double *x, double *y, bool plain = false) {
    reserve(nb);
    prof.begin(st(), "operator");
    metric_apply_strided(metric, w_hi, w_lo, nb, x, n, y, n, plain);
    group_sums(x, n, nb, c.p, cy.p);
    size_t tot = (size_t)nb * n;
    cq_apply_kernel<<<nblk(tot, 256), 256, 0, st()>>>(x, y, n, nb, nv, group.p, c.p, G, cy.p);
    RSG_LAUNCHED(ctx, "cq_apply");
    prof.end(st());
  }

  // y = L'^-1 r (+ add) by `steps` multigrid-preconditioned CG steps (0: the solver's setting)
  void lsolve(int nb, const double *r, double *y, const double *add, int steps = 0) {
    group_sums(r, n, nb, nullptr, s1.p);
    mu_kernel<<<nblk(3 * G * nb, 128), 128, 0, st()>>>(s1.p, r, n, nd, nb, G, eps_area.p, mu.p);
    RSG_LAUNCHED(ctx, "mu");
    size_t m = (size_t)nv * 3 * nb;
    to_mg_kernel<<<nblk(m, 256), 256, 0, st()>>>(r, n, nb, nv, group.p, c.p, mu.p, G, mg_in.p);
    RSG_LAUNCHED(ctx, "to_mg");
    prof.begin(st(), "precondition_multigrid_cg");
    amg.pcg(ctx, mg_in.p, mg_out.p, 3 * nb, steps > 0 ? steps : vcycles);
    prof.end(st());
    // shift: C_Q y = b
    pos_copy_weighted(nb);
    shift_kernel<<<nblk(3 * G * nb, 128), 128, 0, st()>>>(cy.p, r, n, nd, nb, G, shift.p);
    RSG_LAUNCHED(ctx, "shift");
    size_t tot = (size_t)nb * n;
    from_mg_kernel<<<nblk(tot, 256), 256, 0, st()>>>(mg_out.p, y, n, nb, nv, group.p, G, shift.p, mu.p, add);
    RSG_LAUNCHED(ctx, "from_mg");
  }

  // helpers on the multigrid layout
  void axpby(size_t m, const double *b, double *y);
  void add_into(size_t m, const double *x, double *y);
  void pos_copy_weighted(int nb);

  // z = P^-1 r for the augmented preconditioner of precond.rs:1026-1079,
  //   P^-1 = X + X (s L^V - K^) X,  X = L'^-1,  K^ = blockdiag(K x I3, 0),
  // applied in the equivalent form X (s L^V + C^) X with C^ = [[0, C_Q^T], [C_Q, 0]]: from
  // X L' X = X and L' = K^ + C^, X - X K^ X = X C^ X. The two agree for an exact X; for the
  // multigrid X~ = K^-1 (I - E) the first form leaves X~ E, an order -2 error term that
  // outgrows the order -2s main term at high frequencies (the iteration count then grows
  // with the mesh), while the second form only perturbs the main term by (I - E) factors.
  void apply_prec(int nb, const double *r, double *z, int steps = 0) {
    if (cm > 0) apply_prec_coarse(nb, r, z, steps);
    else apply_prec_fine(nb, r, z, steps);
  }
  void apply_prec_fine(int nb, const double *r, double *z, int steps = 0) {
    reserve(nb);
    prof.begin(st(), "precondition");
    double *y = tmp.p, *v = tmp2.p;
    lsolve(nb, r, y, nullptr, steps);
    prof.begin(st(), "precondition_fractional");
    vfrac_apply_strided(vfrac, frac_scale, nb, y, n, v, n, inner_plain);
    prof.end(st());
    group_sums(y, n, nb, c.p, cy.p);
    size_t tot = (size_t)nb * n;
    cq_apply_kernel<<<nblk(tot, 256), 256, 0, st()>>>(y, v, n, nb, nv, group.p, c.p, G, cy.p);
    RSG_LAUNCHED(ctx, "cq_apply");
    lsolve(nb, v, z, nullptr, steps);
    prof.end(st());
  }

  // the learned preconditioner: y = P^-1 r with l_cheap CG steps, then the network's correction
  void apply_learned(int nb, const double *r, double *z) {
    if (lbuf.n < (size_t)nb * n) lbuf.alloc((size_t)nb * n);
    apply_prec(nb, r, lbuf.p, l_cheap);
    prof.begin(st(), "precondition_learned");
    learned_apply(lmodel, lgraph, nb, r, lbuf.p, n, n, z);
    prof.end(st());
  }

  // GMRES with the learned preconditioner when one is set (capped at l_cap iterations), the
  // plain preconditioner otherwise or when the learned solve does not converge
  void solve(int nb, const double *b, double *x, const GmresOptions &o) {
    if (lmodel && use_prec) {
      GmresOptions ol = o;
      if (l_cap > 0) ol.max_iterations = l_cap;
      l_solves++;
      bool ok = true;
      try {
        gmres_batch(ctx, inner_plain ? op_inner : op, &lprec, nb, b, x, ol, last, inner_plain ? &op : nullptr);
        for (auto &r : last) ok = ok && r.converged;
      } catch (const Error &e) {
        if (e.code != RS_SOLVER_DIVERGED) throw;
        ok = false;
      }
      if (ok) return;
      l_fallbacks++;
    }
    gmres_batch(ctx, inner_plain ? op_inner : op, use_prec ? &prec : nullptr, nb, b, x, o, last,
                inner_plain ? &op : nullptr);
  }
};

namespace rsg {
namespace {

__global__ void axpby_kernel(size_t m, const double *b, double *y) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < m) y[i] = b[i] - y[i];
}
__global__ void add_kernel(size_t m, const double *x, double *y) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < m) y[i] += x[i];
}
// cy[q][3g + k] = sum_{v in g} c_v yy[v][3q + k]  (weighted group sums on the multigrid layout)
__global__ void mg_group_partial(const mgreal *__restrict__ yy, int nb, int nv,
                                 const uint32_t *__restrict__ group, const double *__restrict__ c,
                                 int G, double *part, unsigned *ticket, double *out) {
  const int K = 3 * G * nb;
  const size_t chunk = (nv + gridDim.x - 1) / gridDim.x;
  const size_t v0 = blockIdx.x * chunk, v1 = min((size_t)nv, v0 + chunk);
  __shared__ double wsum[32];
  for (int i = 0; i < K; ++i) {
    int q = i / (3 * G), g = (i % (3 * G)) / 3, k = i % 3;
    double acc = 0.0;
    for (size_t v = v0 + threadIdx.x; v < v1; v += blockDim.x)
      if ((int)group[v] == g) acc += c[v] * (double)yy[v * 3 * nb + 3 * q + k];
    for (int m = 16; m >= 1; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[w];
      part[(size_t)blockIdx.x * K + i] = t;
    }
    __syncthreads();
  }
  finish_group_sums(part, K, ticket, out);
}

}  // namespace
}  // namespace rsg

void rs_solver::axpby(size_t m, const double *b, double *y) {
  axpby_kernel<<<nblk(m, 256), 256, 0, st()>>>(m, b, y);
  RSG_LAUNCHED(ctx, "axpby");
}
void rs_solver::add_into(size_t m, const double *x, double *y) {
  add_kernel<<<nblk(m, 256), 256, 0, st()>>>(m, x, y);
  RSG_LAUNCHED(ctx, "add");
}
void rs_solver::pos_copy_weighted(int nb) {
  int K = 3 * G * nb;
  if (part.n < (size_t)GB * K) part.alloc((size_t)GB * K);
  mg_group_partial<<<GB, 256, 0, st()>>>(mg_out.p, nb, nv, group.p, c.p, G, part.p, gs_ticket.p, cy.p);
  RSG_LAUNCHED(ctx, "mg_group");
}

namespace rsg {
namespace {

// cotan stiffness W (RS/src/geometry.rs:217-249), scalar |V| x |V|, plus eps M on the diagonal.
Csr laplacian_block(int nv, int nf, const uint32_t *faces, const double *pos, const std::vector<double> &mass,
                    double eps_rel, bool clamp, double &eps_out) {
  // cotangent half-weights per face corner c (the edge opposite it: t[c+1], t[c+2])
  std::vector<double> hc(3 * (size_t)nf);
  parallel_for((size_t)nf, [&](size_t f0, size_t f1) {
    for (size_t f = f0; f < f1; ++f) {
      const uint32_t *t = faces + 3 * f;
      for (int c = 0; c < 3; ++c) {
        const double *p = pos + 3 * (size_t)t[c];
        const double *p1 = pos + 3 * (size_t)t[(c + 1) % 3];
        const double *p2 = pos + 3 * (size_t)t[(c + 2) % 3];
        double u[3] = {p1[0] - p[0], p1[1] - p[1], p1[2] - p[2]};
        double w[3] = {p2[0] - p[0], p2[1] - p[1], p2[2] - p[2]};
        double cr[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
        double cot = (u[0] * w[0] + u[1] * w[1] + u[2] * w[2]) /
                     std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        hc[3 * f + c] = 0.5 * cot;
      }
    }
  });
  // vertex -> incident faces, ascending
  std::vector<uint32_t> ioff((size_t)nv + 1, 0), inc(3 * (size_t)nf);
  for (size_t e = 0; e < 3 * (size_t)nf; ++e) ioff[faces[e] + 1]++;
  for (int v = 0; v < nv; ++v) ioff[v + 1] += ioff[v];
  {
    std::vector<uint32_t> fill(ioff.begin(), ioff.end() - 1);
    for (size_t f = 0; f < (size_t)nf; ++f)
      for (int c = 0; c < 3; ++c) inc[fill[faces[3 * f + c]]++] = (uint32_t)f;
  }
  // row i: the terms (i, b, -h), (i, i, h) of every face corner whose opposite edge touches i,
  // in face, corner, slot order; sorted by column (stable), equal columns added in that order
  auto row = [&](int i, std::vector<std::pair<int, double>> &r) {
    r.clear();
    for (uint32_t e = ioff[i]; e < ioff[i + 1]; ++e) {
      const uint32_t f = inc[e], *t = faces + 3 * (size_t)f;
      for (int c = 0; c < 3; ++c) {
        const int a = (int)t[(c + 1) % 3], b = (int)t[(c + 2) % 3];
        const double h = hc[3 * (size_t)f + c];
        if (a == i) r.push_back({b, -h});
        if (b == i) r.push_back({a, -h});
        if (a == i) r.push_back({i, h});
        if (b == i) r.push_back({i, h});
      }
    }
    std::stable_sort(r.begin(), r.end(), [](const auto &x, const auto &y) { return x.first < y.first; });
  };
  Csr K;
  K.n = K.m = nv;
  K.ptr.assign(nv + 1, 0);
  parallel_for((size_t)nv, [&](size_t v0, size_t v1) {
    std::vector<std::pair<int, double>> r;
    for (size_t i = v0; i < v1; ++i) {
      row((int)i, r);
      int cnt = 0;
      for (size_t p = 0; p < r.size(); ++p) cnt += (p == 0 || r[p].first != r[p - 1].first);
      K.ptr[i + 1] = cnt;
    }
  });
  for (int i = 0; i < nv; ++i) K.ptr[i + 1] += K.ptr[i];
  K.col.resize(K.ptr[nv]);
  K.val.resize(K.ptr[nv]);
  parallel_for((size_t)nv, [&](size_t v0, size_t v1) {
    std::vector<std::pair<int, double>> r;
    for (size_t i = v0; i < v1; ++i) {
      row((int)i, r);
      int o = K.ptr[i];
      for (size_t p = 0; p < r.size();) {
        size_t q = p;
        double v = 0.0;
        while (q < r.size() && r[q].first == r[p].first) v += r[q++].second;
        K.col[o] = r[p].first, K.val[o] = v, ++o;
        p = q;
      }
    }
  });
  double trw = 0.0, trm = 0.0;
  for (int i = 0; i < nv; ++i) trm += mass[i];
  for (int i = 0; i < nv; ++i) {
    int dp = -1;
    for (int p = K.ptr[i]; p < K.ptr[i + 1]; ++p)
      if (K.col[p] == i) dp = p;
    if (clamp)  // a positive off-diagonal is a negative edge weight: drop the edge
      for (int p = K.ptr[i]; p < K.ptr[i + 1]; ++p)
        if (K.col[p] != i && K.val[p] > 0.0) K.val[dp] += K.val[p], K.val[p] = 0.0;
    trw += K.val[dp];
  }
  double eps = eps_rel * trw / trm;  // preconditioner_epsilon (RS/src/solve/dense.rs:529-533)
  for (int i = 0; i < nv; ++i)
    for (int p = K.ptr[i]; p < K.ptr[i + 1]; ++p)
      if (K.col[p] == i) K.val[p] += eps * mass[i];
  eps_out = eps;
  return K;
}

std::vector<uint32_t> vertex_components(int nv, int nf, const uint32_t *faces, int &nc) {
  std::vector<uint32_t> par(nv);
  std::iota(par.begin(), par.end(), 0u);
  auto find = [&](uint32_t x) {
    while (par[x] != x) x = par[x] = par[par[x]];
    return x;
  };
  for (int f = 0; f < nf; ++f)
    for (int c = 1; c < 3; ++c) {
      uint32_t a = find(faces[3 * f]), b = find(faces[3 * f + c]);
      if (a != b) par[std::max(a, b)] = std::min(a, b);
    }
  // number components by lowest face index (the crate's component order)
  std::vector<int64_t> id(nv, -1);
  std::vector<uint32_t> comp(nv);
  nc = 0;
  for (int f = 0; f < nf; ++f) {
    uint32_t r = find(faces[3 * f]);
    if (id[r] < 0) id[r] = nc++;
  }
  for (int v = 0; v < nv; ++v) comp[v] = (uint32_t)id[find(v)];
  return comp;
}

}  // namespace
}  // namespace rsg

extern "C" {

int rs_solver_build(rs_ctx *ctx, int nv, int nf, const uint32_t *faces, const double *positions_host,
                    double alpha, double beta, const rs_solver_options *o, rs_solver **out) {
  *out = nullptr;
  return guard([&] {
    rs_solver_options def = rs_solver_options_default();
    if (!o) o = &def;
    validate_topology(nv, nf, faces);
    validate_positions(nv, nf, faces, positions_host);
    if (!(o->tp_weight > 0.0 && std::isfinite(o->tp_weight)))
      fail(RS_INVALID_OPTION, "InvalidOption", "solver", "tp_weight must be finite and positive");
    ctx->use();
    using clk = std::chrono::steady_clock;
    auto t_all = clk::now(), t_ph = t_all;
    auto lap = [&](double &slot) {
      auto now = clk::now();
      slot = std::chrono::duration<double>(now - t_ph).count();
      t_ph = now;
    };
    auto S = std::make_unique<rs_solver>();
    S->ctx = ctx;
    S->nv = nv, S->nf = nf, S->nd = 3 * (size_t)nv;
    S->geom = face_geometry(nf, faces, positions_host);
    S->alpha = alpha, S->beta = beta, S->leaf_size = o->leaf_size, S->leaf_pairs = o->leaf_pairs;
    if (nv <= kDenseMaxVertices) {
      S->faces_h.assign(faces, faces + 3 * (size_t)nf);
      S->pos_h.assign(positions_host, positions_host + 3 * (size_t)nv);
    }
    S->vmass.assign(nv, 0.0);
    for (int f = 0; f < nf; ++f)
      for (int c = 0; c < 3; ++c) S->vmass[faces[3 * f + c]] += S->geom.area[f] / 3.0;
    // positional rows: barycenters (global or per component)
    int ncomp = 0;
    std::vector<uint32_t> comp = vertex_components(nv, nf, faces, ncomp);
    bool per_comp = o->barycenter_per_component != 0;
    S->G = per_comp ? ncomp : 1;
    S->group_h.assign(nv, 0);
    if (per_comp) S->group_h = comp;
    std::vector<double> garea(S->G, 0.0), ch(nv);
    for (int v = 0; v < nv; ++v) garea[S->group_h[v]] += S->vmass[v];
    for (int v = 0; v < nv; ++v) ch[v] = S->vmass[v] / garea[S->group_h[v]];
    S->n = S->nd + 3 * (size_t)S->G;
    bool multi = !per_comp && ncomp > 1;  // translations_fixed_per_component (precond.rs:96-124)
    auto secs = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); };
    // Three independent parts run side by side: the metric's face tree and blocks (this
    // thread), the vertex fractional tree, and the Laplacian block with its multigrid set-up
    // (host only). A worker keeps the caller's trust in the face list.
    const bool trusted = topology_trusted();
    const double sexp = (beta - 2.0) / alpha;
    double eps = 0.0, t_lap = 0.0, t_amg = 0.0, t_vf = 0.0;
    auto amg_task = std::async(std::launch::async, [&, trusted] {
      std::optional<TrustedTopology> tt;
      if (trusted) tt.emplace();
      auto t0 = clk::now();
      Csr K = laplacian_block(nv, nf, faces, positions_host, S->vmass, multi ? o->eps_multi_rel : o->eps_rel,
                              o->clamp_laplacian != 0, eps);
      auto t1 = clk::now();
      AmgHost h = amg_setup(K, 300, 12, per_comp && ncomp > 1 ? &comp : nullptr);
      t_lap = secs(t0, t1), t_amg = secs(t1, clk::now());
      return h;
    });
    std::unique_ptr<rs_vfrac, void (*)(rs_vfrac *)> vf(nullptr, rs_vfrac_free);
    auto vf_task = std::async(std::launch::async, [&, trusted] {
      std::optional<TrustedTopology> tt;
      if (trusted) tt.emplace();
      auto t0 = clk::now();
      rs_vfrac *v = nullptr;
      int rc = rs_vfrac_build(ctx, nv, positions_host, S->vmass.data(), 2.0 - sexp, o->chi, o->leaf_size,
                              o->leaf_pairs, &v);
      vf.reset(v);
      t_vf = secs(t0, clk::now());
      return std::make_pair(rc, rc ? std::string(rs_last_error()) : std::string());
    });
    auto t_m0 = clk::now();
    std::unique_ptr<rs_metric, void (*)(rs_metric *)> m(nullptr, rs_metric_free);
    rs_metric *mp = nullptr;
    int rc_m = rs_metric_build(ctx, nv, nf, faces, positions_host, alpha, beta, o->chi, o->leaf_size,
                               o->leaf_pairs, &mp);
    m.reset(mp);
    std::string err_m = rc_m ? rs_last_error() : "";
    S->build_times[0] = secs(t_m0, clk::now());
    auto [rc_v, err_v] = vf_task.get();
    AmgHost amg_h = amg_task.get();
    if (rc_m) fail(rc_m, "Gpu", "solver", "metric: " + err_m);
    if (rc_v) fail(rc_v, "Gpu", "solver", "fractional tree: " + err_v);
    S->build_times[1] = t_vf, S->build_times[2] = t_lap, S->build_times[3] = t_amg;
    t_ph = clk::now();
    S->eps = eps;
    std::vector<double> ea(S->G);
    for (int g = 0; g < S->G; ++g) ea[g] = eps * garea[g];
    cudaStream_t s = ctx->stream;
    S->group.upload(S->group_h, s);
    S->gs_ticket.alloc(1);
    RSG_CUDA("solver", cudaMemsetAsync(S->gs_ticket.p, 0, sizeof(unsigned), s));
    S->c.upload(ch, s);
    S->eps_area.upload(ea, s);
    S->w_hi = o->tp_weight;
    S->w_lo = o->tp_weight * (o->low_order ? 1.0 : 0.0);
    S->frac_scale = 1.0 / (o->tp_weight * symbol_ratio(sexp));  // FractionalScale::Symbol
    S->amg.upload(amg_h, s);
    S->vcycles = std::max(1, o->vcycles);
    S->use_prec = o->preconditioner != 0;
    S->gopt.restart = o->restart;
    S->gopt.tolerance = o->tolerance;
    S->gopt.max_iterations = o->max_iterations;
    rs_solver *P = S.get();
    S->op.n = S->n;
    S->op.apply = [P](int nb, const double *x, double *y) { P->apply_op(nb, x, y); };
    S->op_inner.n = S->n;
    S->op_inner.apply = [P](int nb, const double *x, double *y) { P->apply_op(nb, x, y, true); };
    S->inner_plain = o->inner_plain != 0;
    S->prec.n = S->n;
    S->prec.apply = [P](int nb, const double *x, double *y) { P->apply_prec(nb, x, y); };
    S->lprec.n = S->n;
    S->lprec.apply = [P](int nb, const double *x, double *y) { P->apply_learned(nb, x, y); };
    // the coarse space (CoarseSpace::free_components and build, RS/src/solve/coarse.rs:63-247):
    // with one global barycenter group on several components no component is fixed by rows of
    // its own, so every component is free and the group's three rows touch them; columns are
    // the scaled translations of every component and the three multipliers
    // the operator's products below need the metric (still owned by m and vf here)
    S->metric = m.get(), S->vfrac = vf.get();
    const int nfree = ncomp, cmm = 3 * ncomp + 3;
    if (o->coarse && S->use_prec && !per_comp && ncomp > 1 && (double)S->n * cmm <= (double)(1 << 25)) {
      const size_t n = S->n;
      S->c_nfree = nfree;
      S->c_rows_h = {0, 1, 2};
      std::vector<double> members(nfree, 0.0), scale(nfree);
      for (int v = 0; v < nv; ++v) members[comp[v]] += 1.0;
      for (int k = 0; k < nfree; ++k) scale[k] = 1.0 / std::sqrt(members[k]);
      S->c_slot.upload(comp, s);
      S->c_scale.upload(scale, s);
      S->c_rows.upload(S->c_rows_h, s);
      std::vector<int> rowcol = {3 * nfree, 3 * nfree + 1, 3 * nfree + 2};
      S->c_rowcol.upload(rowcol, s);
      S->c_az.alloc(n * cmm);
      // A'Z of the translation columns, four per product
      std::vector<double> zc(n * 3 * nfree, 0.0);
      for (int v = 0; v < nv; ++v)
        for (int a = 0; a < 3; ++a) zc[(size_t)(3 * comp[v] + a) * n + 3 * v + a] = scale[comp[v]];
      DevBuf<double> zd;
      zd.upload(zc, s);
      for (int j0 = 0; j0 < 3 * nfree; j0 += 4)
        S->apply_op(std::min(4, 3 * nfree - j0), zd.p + (size_t)j0 * n, S->c_az.p + (size_t)j0 * n);
      // A' e_(nd + r) = [C_Q^T e_r; 0]: c_v on axis r
      std::vector<double> mc(n * 3, 0.0);
      for (int r = 0; r < 3; ++r)
        for (int v = 0; v < nv; ++v) mc[(size_t)r * n + 3 * v + r] = ch[v];
      RSG_CUDA("solver", rsg::copy_async(S->c_az.p + (size_t)3 * nfree * n, mc.data(), mc.size() * sizeof(double),
                                         cudaMemcpyHostToDevice, s));
      S->c_part.alloc(std::max<size_t>((size_t)kCoarseChunks * 4 * cmm, (size_t)3 * (nfree + 1) * std::max(4, cmm)));
      S->c_t.alloc((size_t)4 * cmm), S->c_yc.alloc((size_t)4 * cmm), S->c_t2.alloc((size_t)4 * cmm);
      S->c_rp.alloc((size_t)4 * n);
      // E = Z^T A'Z, symmetrized, and its pseudo-inverse (eigenvalues at or below 1e-12 of the
      // largest dropped)
      S->cm = cmm;
      DevBuf<double> et((size_t)cmm * cmm);
      S->coarse_zt(cmm, S->c_az.p, et.p);
      std::vector<double> e((size_t)cmm * cmm);
      et.download(e.data(), e.size(), s);
      RSG_CUDA("solver", cudaStreamSynchronize(s));
      for (int i = 0; i < cmm; ++i)
        for (int j = 0; j < i; ++j) {
          const double v = 0.5 * (e[(size_t)i * cmm + j] + e[(size_t)j * cmm + i]);
          e[(size_t)i * cmm + j] = e[(size_t)j * cmm + i] = v;
        }
      std::vector<double> lam, u;
      jacobi_eigen(cmm, e, lam, u);
      double lmax = 0.0;
      for (double l : lam) lmax = std::max(lmax, std::fabs(l));
      std::vector<double> pinv((size_t)cmm * cmm, 0.0);
      double lmin = INFINITY;
      for (int k = 0; k < cmm; ++k) {
        const double l = lam[k];
        if (std::isnan(l) || std::fabs(l) <= 1e-12 * lmax) {
          ++S->c_dropped;
          continue;
        }
        lmin = std::min(lmin, std::fabs(l));
        for (int i = 0; i < cmm; ++i)
          for (int j = 0; j < cmm; ++j) pinv[(size_t)i * cmm + j] += u[(size_t)i * cmm + k] / l * u[(size_t)j * cmm + k];
      }
      S->c_conditioning = lmax > 0.0 ? lmin / lmax : 0.0;
      S->c_epinv.upload(pinv, s);
    }
    RSG_CUDA("solver", cudaStreamSynchronize(s));
    lap(S->build_times[4]);
    S->build_times[5] = std::chrono::duration<double>(clk::now() - t_all).count();
    S->metric = m.release(), S->vfrac = vf.release();
    ctx_retain(ctx);
    *out = S.release();
  });
}

void rs_solver_free(rs_solver *S) {
  if (!S) return;
  rs_ctx *ctx = S->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  rs_metric_free(S->metric);
  rs_vfrac_free(S->vfrac);
  delete S;
  ctx_release(ctx);
}

int rs_solver_profile(rs_solver *S, int nb, const double *rhs, char *names, int names_len, double *ms,
                      int max_kernels, int *n_kernels) {
  return guard([&] {
    S->ctx->use();
    if (nb < 1 || nb > 4) fail(RS_INVALID_OPTION, "InvalidOption", "solver", "1 to 4 right-hand sides per batch");
    size_t tot = (size_t)nb * S->n;
    DevBuf<double> a(tot), b(tot);
    a.upload(rhs, tot, S->st());
    GmresOptions o = S->gopt;
    o.prof = &S->prof;
    S->prof.start();
    S->prof.begin(S->st(), "solve");
    S->solve(nb, a.p, b.p, o);
    S->prof.end(S->st());
    S->prof.stop(S->st());
    S->prof.report(names, names_len, ms, max_kernels, n_kernels, 1);
  });
}

int rs_solver_multigrid_levels(rs_solver *S, int64_t *out, int max_levels, int *n_levels) {
  return guard([&] {
    int n = (int)S->amg.L.size();
    for (int l = 0; l < n && l < max_levels; ++l) {
      out[2 * l] = S->amg.L[l].n;
      out[2 * l + 1] = (int64_t)S->amg.L[l].av.n;
    }
    *n_levels = n;
  });
}

int rs_solver_set_gmres(rs_solver *S, int restart, int max_iterations, double tolerance) {
  return guard([&] {
    if (restart < 1 || restart > 63 || max_iterations < 1 || !(tolerance > 0.0 && tolerance < 1.0))
      fail(RS_INVALID_OPTION, "InvalidOption", "solver", "restart in 1..63, max_iterations >= 1, tolerance in (0, 1)");
    S->gopt.restart = restart, S->gopt.max_iterations = max_iterations, S->gopt.tolerance = tolerance;
  });
}

int rs_solver_set_learned(rs_solver *S, rs_learned *model, rs_lgraph *graph, int cheap_steps,
                          int max_iterations) {
  return guard([&] {
    if (model && !graph) fail(RS_INVALID_OPTION, "InvalidOption", "solver", "a learned model needs its surface graph");
    if (model && (cheap_steps < 1 || max_iterations < 0))
      fail(RS_INVALID_OPTION, "InvalidOption", "solver", "cheap_steps >= 1, max_iterations >= 0");
    S->lmodel = model, S->lgraph = graph;
    S->l_cheap = cheap_steps, S->l_cap = max_iterations;
  });
}

int rs_solver_learned_counts(rs_solver *S, int64_t *solves, int64_t *fallbacks) {
  return guard([&] {
    *solves = S->l_solves;
    *fallbacks = S->l_fallbacks;
  });
}

int rs_solver_build_times(rs_solver *S, double *out6) {
  return guard([&] { std::copy(S->build_times, S->build_times + 6, out6); });
}

int rs_solver_dims(rs_solver *S, int64_t *n_dofs, int64_t *n_constraints) {
  return guard([&] {
    *n_dofs = (int64_t)S->nd;
    *n_constraints = (int64_t)(S->n - S->nd);
  });
}

int rs_solver_apply_device(rs_solver *S, int nb, const double *x_dev, double *y_dev) {
  return guard([&] {
    S->ctx->use();
    S->apply_op(nb, x_dev, y_dev);
  });
}

int rs_solver_precondition_device(rs_solver *S, int nb, const double *r_dev, double *z_dev) {
  return guard([&] {
    S->ctx->use();
    S->apply_prec(nb, r_dev, z_dev);
  });
}

int rs_solver_dense_solve_many_device(rs_solver *S, int nb, const double *rhs_dev, double *sol_dev,
                                      double *report) {
  return guard([&] {
    S->ctx->use();
    if (nb < 1 || nb > 4) fail(RS_INVALID_OPTION, "InvalidOption", "solver", "1 to 4 right-hand sides per batch");
    if (S->nv > kDenseMaxVertices)
      fail(RS_INVALID_OPTION, "InvalidOption", "solver",
           "the dense last resort takes at most " + std::to_string(kDenseMaxVertices) + " vertices");
    auto t0 = std::chrono::steady_clock::now();
    if (!S->dense) {
      // the exact metric: the block cluster tree at chi = 0 holds every pair in near blocks
      rs_metric *m0 = nullptr;
      int rc = rs_metric_build(S->ctx, S->nv, S->nf, S->faces_h.data(), S->pos_h.data(), S->alpha, S->beta, 0.0,
                               S->leaf_size, S->leaf_pairs, &m0);
      if (rc) fail(rc, "Gpu", "solver", std::string("dense metric: ") + rs_last_error());
      std::unique_ptr<rs_metric, void (*)(rs_metric *)> own(m0, rs_metric_free);
      auto D = std::make_unique<DenseSaddleDev>();
      const double wh = S->w_hi, wl = S->w_lo;
      const size_t nd = S->nd;
      D->build(S->ctx, S->nv, S->G, S->group.p, S->c.p, [&](int k, const double *x, double *y) {
        metric_apply_strided(m0, wh, wl, k, x, nd, y, nd);
      });
      S->dense = std::move(D);
    }
    std::vector<double> rel(nb);
    S->dense->solve(nb, rhs_dev, sol_dev, rel.data());
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    S->last.assign(nb, GmresReport());
    for (int q = 0; q < nb; ++q) {
      S->last[q].iterations = 0, S->last[q].relative_residual = rel[q];
      S->last[q].converged = true, S->last[q].seconds = secs / nb, S->last[q].cycles = 0;
      if (report) {
        report[5 * q + 0] = 0.0;
        report[5 * q + 1] = rel[q];
        report[5 * q + 2] = 1.0;
        report[5 * q + 3] = secs / nb;
        report[5 * q + 4] = 0.0;
      }
    }
  });
}

int rs_solver_dense_pivot_ratio(rs_solver *S, double *ratio) {
  return guard([&] { *ratio = S->dense ? S->dense->pivot_ratio : 0.0; });
}

int rs_solver_solve_many_device(rs_solver *S, int nb, const double *rhs_dev, double *sol_dev,
                                double *report) {
  return guard([&] {
    S->ctx->use();
    if (nb < 1 || nb > 4) fail(RS_INVALID_OPTION, "InvalidOption", "solver", "1 to 4 right-hand sides per batch");
    S->solve(nb, rhs_dev, sol_dev, S->gopt);
    if (report)
      for (int q = 0; q < nb; ++q) {
        report[5 * q + 0] = S->last[q].iterations;
        report[5 * q + 1] = S->last[q].relative_residual;
        report[5 * q + 2] = S->last[q].converged ? 1.0 : 0.0;
        report[5 * q + 3] = S->last[q].seconds;
        report[5 * q + 4] = S->last[q].cycles;
      }
  });
}

// Host-buffer variants: vectors of length n = 3V + k_Q, stacked.
static void host_roundtrip(rs_solver *S, int nb, const double *in, double *out,
                           const std::function<void(const double *, double *)> &f) {
  size_t tot = (size_t)nb * S->n;
  DevBuf<double> a(tot), b(tot);
  a.upload(in, tot, S->st());
  f(a.p, b.p);
  b.download(out, tot, S->st());
  RSG_CUDA("solver", cudaStreamSynchronize(S->st()));
}

int rs_solver_apply(rs_solver *S, int nb, const double *x, double *y) {
  return guard([&] {
    S->ctx->use();
    host_roundtrip(S, nb, x, y, [&](const double *a, double *b) { S->apply_op(nb, a, b); });
  });
}

int rs_solver_precondition(rs_solver *S, int nb, const double *r, double *z) {
  return guard([&] {
    S->ctx->use();
    host_roundtrip(S, nb, r, z, [&](const double *a, double *b) { S->apply_prec(nb, a, b); });
  });
}

int rs_solver_solve_many(rs_solver *S, int nb, const double *rhs, double *sol, double *report) {
  return guard([&] {
    S->ctx->use();
    if (nb < 1 || nb > 4) fail(RS_INVALID_OPTION, "InvalidOption", "solver", "1 to 4 right-hand sides per batch");
    host_roundtrip(S, nb, rhs, sol, [&](const double *a, double *b) {
      S->solve(nb, a, b, S->gopt);
    });
    if (report)
      for (int q = 0; q < nb; ++q) {
        report[5 * q + 0] = S->last[q].iterations;
        report[5 * q + 1] = S->last[q].relative_residual;
        report[5 * q + 2] = S->last[q].converged ? 1.0 : 0.0;
        report[5 * q + 3] = S->last[q].seconds;
        report[5 * q + 4] = S->last[q].cycles;
      }
  });
}

int rs_solver_history(rs_solver *S, int q, double *estimates, int max_iter, int *n_iter,
                      double *cycle_residuals, int max_cycles, int *n_cycles) {
  return guard([&] {
    if (q < 0 || q >= (int)S->last.size())
      fail(RS_INVALID_OPTION, "InvalidOption", "solver", "no such right-hand side in the last solve");
    const GmresReport &r = S->last[q];
    int a = (int)std::min<size_t>(r.history.size(), (size_t)std::max(max_iter, 0));
    int b = (int)std::min<size_t>(r.cycle_residuals.size(), (size_t)std::max(max_cycles, 0));
    if (estimates) std::copy(r.history.begin(), r.history.begin() + a, estimates);
    if (cycle_residuals) std::copy(r.cycle_residuals.begin(), r.cycle_residuals.begin() + b, cycle_residuals);
    if (n_iter) *n_iter = (int)r.history.size();
    if (n_cycles) *n_cycles = (int)r.cycle_residuals.size();
  });
}

rs_solver_options rs_solver_options_default(void) {
  rs_solver_options o;
  o.chi = 0.5;
  o.leaf_size = 8;
  o.leaf_pairs = 64;
  o.restart = 30;
  o.tolerance = 1e-6;
  o.max_iterations = 200;
  o.tp_weight = 1.0;
  o.low_order = 1;
  o.eps_rel = 1e-10;
  o.eps_multi_rel = 1e-4;
  o.barycenter_per_component = 0;
  o.vcycles = 6;
  o.preconditioner = 1;
  o.clamp_laplacian = 0;
  o.coarse = 1;
  o.inner_plain = 1;
  return o;
}

}  // extern "C"
