// Device-resident restarted GMRES (RS/src/solve/gmres.rs) and its FP64 vector kernels.
#pragma once
#include <functional>
#include <string>
#include <vector>

#include "common.hpp"

namespace rsg {

// y = A x for nb stacked device vectors of length n (x: nb*n, y: nb*n), on the context stream.
struct Operator {
  size_t n = 0;
  std::function<void(int nb, const double *x, double *y)> apply;
};

struct Profiler;
struct GmresOptions {  // GmresOptions (RS/src/solve/gmres.rs:135-190)
  int restart = 30;
  double tolerance = 1e-6;
  int max_iterations = 200;
  Profiler *prof = nullptr;  // phase timing (orthogonalization) when active
};

struct GmresReport {  // GmresReport (gmres.rs:200-225)
  int iterations = 0, cycles = 0;
  bool converged = false;
  double relative_residual = 0.0;
  std::vector<double> cycle_residuals, history;
  int operator_applications = 0, preconditioner_applications = 0;
  double seconds = 0.0;
};

// Right-preconditioned restarted GMRES on A P^-1 (P may be null: identity) for nb right-hand
// sides in lock step (gmres_batch, gmres.rs:592-715): x0 = 0, Arnoldi with classical
// Gram-Schmidt applied twice (FP64, fixed-order reductions), Givens rotations on the host, the
// explicit residual at every cycle start and end. The preconditioned basis vectors are stored
// (flexible form), so a preconditioner that varies between applications is allowed.
// b, x: nb*n device vectors. Throws RS_SOLVER_DIVERGED when a solve ends above a true relative
// residual of 0.1 (DIVERGENCE_THRESHOLD, gmres.rs:196).
// A_true (optional): the operator of the explicit residuals (every cycle start, and so the
// convergence test), when the Arnoldi steps use a cheaper approximation A of it. Each cycle
// then corrects the previous cycles' approximation error, as iterative refinement does, and the
// reported residuals are those of A_true.
void gmres_batch(rs_ctx *ctx, const Operator &A, const Operator *P, int nb, const double *b,
                 double *x, const GmresOptions &opt, std::vector<GmresReport> &reports,
                 const Operator *A_true = nullptr);

// FP64 helpers (deterministic: fixed grid, fixed reduction trees).
// out[i] = v_i . w for v_i = vs[i], or for the single vector v1 when given (nvec = 1); root:
// out = sqrt of it
void dev_dots(rs_ctx *ctx, const double *const *vs, int nvec, const double *w, size_t n,
              double *out_dev, const double *v1 = nullptr, bool root = false);
double dev_norm(rs_ctx *ctx, const double *w, size_t n);

}  // namespace rsg
