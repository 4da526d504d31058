// Smoothed-aggregation algebraic multigrid for the preconditioner's Laplacian block
// K = W + eps M (RS/src/solve/precond.rs:157-460 factors L' by a sparse LDL^T on the CPU; this
// library solves it with multigrid V-cycles on the device instead, see saddle.cu).
#pragma once
#include <cstdint>
#include <vector>

#include "common.hpp"

namespace rsg {

// Storage and arithmetic type of the device hierarchy and its conjugate-gradient vectors: FP32.
// The multigrid solve is a preconditioner inside flexible FP64 GMRES, so its rounding only
// perturbs the preconditioner; GB300 runs FP32 at many times its FP64 rate. Dot products
// are added up in FP64 across blocks.
using mgreal = float;

struct Csr {
  int n = 0, m = 0;  // rows, columns
  std::vector<int> ptr, col;
  std::vector<double> val;
};

// Host setup: strength (|a_ij| >= 0.08 sqrt(a_ii a_jj)), greedy aggregation, the tentative
// prolongator of the constant near-null space, one damped-Jacobi smoothing step
// (omega = 4 / (3 rho(D^-1 A))), Galerkin coarse operators, down to at most `coarse_max` rows;
// the coarsest operator is inverted densely after adding z z^T (z its null vector).
struct AmgHost {
  std::vector<Csr> A, P, R;  // A[l] n_l x n_l, P[l] n_l x n_{l+1}, R[l] = P[l]^T
  std::vector<std::vector<double>> dinv;  // damped inverse diagonals of A[l]
  std::vector<double> coarse_inv;         // dense n_L x n_L
};
// groups (optional, one label per row): rows that form separate near-null blocks (the
// components of a surface whose barycenters are held one by one); the coarsest level is then
// regularised along the constant of every group instead of the global constant only.
AmgHost amg_setup(const Csr &A, int coarse_max = 300, int max_levels = 12,
                  const std::vector<uint32_t> *groups = nullptr);

// The hierarchy on the device and its V-cycle for C interleaved columns per row
// (x[row * C + c]): pre- and post-smoothing by `sweeps` damped Jacobi steps, dense coarse solve.
// Each sparse product gives a row to a group of 1-32 lanes sized to the matrix's mean row length
// (the coarse operators of smoothed aggregation have 40-70 nonzeros per row on a few hundred
// rows, where one thread per row would leave the GPU idle behind long serial loops).
struct AmgDevice {
  struct Level {
    int n = 0;
    int tpr_a = 1, tpr_r = 1, tpr_p = 1;  // lanes per row of A, R (rows of level l+1) and P
    DevBuf<int> ap, ac, pp, pc, rp, rc;
    DevBuf<mgreal> av, pv, rv, dinv;
    DevBuf<mgreal> x, b, r, t;  // C columns each
  };
  std::vector<Level> L;
  DevBuf<mgreal> cinv;
  int C = 0, sweeps = 2;
  void upload(const AmgHost &h, cudaStream_t s);
  void reserve(int C_);
  // x = V-cycle(b) on level 0; b and x are n_0 x C device arrays (x overwritten).
  // pre0: the first Jacobi sweep of level 0 (dinv b) is already in place.
  void vcycle(rs_ctx *ctx, const mgreal *b, mgreal *x, int C_, bool pre0 = false);
  // y = A_0 x for C columns.
  void spmv0(rs_ctx *ctx, const mgreal *x, mgreal *y, int C_);
  // x ~ A_0^-1 b by `iters` steps of conjugate gradients per column, preconditioned by one
  // V-cycle each (x_0 = 0; iters = 1 is the V-cycle with the optimal step length). The
  // scalars stay on the device (no host synchronization); a fixed number of steps makes it a
  // nonlinear map of b, which flexible GMRES (the stored preconditioned vectors) allows.
  void pcg(rs_ctx *ctx, const mgreal *b, mgreal *x, int C_, int iters);
  DevBuf<mgreal> cg_r, cg_z, cg_p, cg_q;  // n_0 x C each
  DevBuf<double> cg_part, cg_s;           // per-block partial sums; scalars
  DevBuf<unsigned> cg_ticket;  // blocks done in the current dot-product launch (0 between launches)
  struct Graph {
    const mgreal *b = nullptr;
    mgreal *x = nullptr;
    int C = 0, iters = 0;
    int64_t launches = 0;
    cudaGraphExec_t exec = nullptr;
  };
  std::vector<Graph> graphs;  // captured conjugate-gradient solves
  AmgDevice() = default;
  AmgDevice(const AmgDevice &) = delete;
  AmgDevice &operator=(const AmgDevice &) = delete;
  ~AmgDevice();

 private:
  template <int CC>
  void vcycle_t(rs_ctx *ctx, const mgreal *b, mgreal *x, bool pre0);
  template <int CC>
  void spmv0_t(rs_ctx *ctx, const mgreal *x, mgreal *y);
  void pcg_body(rs_ctx *ctx, const mgreal *b, mgreal *x, int C_, int iters);
};

}  // namespace rsg
