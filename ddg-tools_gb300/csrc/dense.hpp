// The dense last resort of the recovery chain (DenseSaddle, RS/src/solve/dense.rs:282-470;
// RobustHierarchical::escalate, RS/src/step/direction.rs:238-300) on the device.
#pragma once
#include <functional>

#include "common.hpp"

namespace rsg {

// The crate's limit: a failed GMRES solve falls back to a dense LU for at most this many
// vertices (DENSE_FALLBACK_MAX_VERTICES, direction.rs:238).
constexpr int kDenseMaxVertices = 6000;

// A' = [[A (x) I3, C_Q^T], [C_Q, 0]] with positional rows C_Q = C_1 (x) I3 (one row of C_1 per
// barycenter group g: c_v for the vertices v of g), factored per axis as the (V + G) square
// K = [[A, C_1^T], [C_1, 0]] (DenseSaddle::factor_scalar, dense.rs:345-366): equilibrated as
// D K D (equilibration, dense.rs:289-307) and factored by LU with partial pivoting in FP64.
struct DenseSaddleDev {
  rs_ctx *ctx = nullptr;
  int nv = 0, G = 0, n = 0;
  double pivot_ratio = 0.0;
  DevBuf<double> K;   // n x n, column-major, unscaled (the operator of the refinement residual)
  DevBuf<double> LU;  // the factor of D K D, in place
  DevBuf<double> d;   // D
  DevBuf<int> perm;   // row interchanges in order (perm[k]: the row swapped with k)
  DevBuf<double> X, Y, B, R, piv;

  // metric(nb, x, y): y = A x per axis for nb <= 3 stacked 3V vectors on the device
  void build(rs_ctx *c, int nv_, int G_, const uint32_t *group_dev, const double *c_dev,
             const std::function<void(int nb, const double *x, double *y)> &metric);
  // sol = A'^-1 rhs for nb stacked [a (3V); b (3G)] vectors on the device, with one step of
  // iterative refinement (DenseSaddle::solve_full, dense.rs:451-473); rel[q] = the relative
  // residual |rhs - A' sol| / |rhs| of vector q.
  void solve(int nb, const double *rhs, double *sol, double *rel);
};

}  // namespace rsg
