// The learned preconditioner correction (no crate counterpart): a per-vertex network with
// one-ring message passing that maps a residual r and a cheap plain-preconditioned vector
// y = P_cheap^-1 r (with the surface's positions, normals and dual areas) to
// z = y + s_y N(features), an approximation of A'^-1 r for flexible GMRES. Three layers,
// hidden width 64 (configurable at creation), SiLU; weights kept in FP32 for training and
// used as BF16 in every forward pass (FP32 accumulation). Training kernels (forward with
// stored activations, backward, Adam) and inference kernels are hand-written here.
#pragma once
#include <cstdint>

#include "common.hpp"

struct rs_learned;
struct rs_lgraph;

namespace rsg {

// z_q = y_q + rms(y_q) N(features(r_q, y_q)) on the position rows (3V, interleaved) of nb
// vectors with leading dimension ld; the other rows of z are copied from y.
void learned_apply(rs_learned *model, rs_lgraph *graph, int nb, const double *r, const double *y,
                   size_t ld, size_t rows, double *z);

}  // namespace rsg
