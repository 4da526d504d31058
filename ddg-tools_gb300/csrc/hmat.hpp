// Internal entry points of the hierarchical products (hmat.cu) for the saddle solver.
#pragma once
#include <cstddef>

#include "rsgpu.h"

namespace rsg {

// ys = (w_hi B~ + w_lo B~0) xs for nb device vectors with leading dimensions ldx, ldy (>= 3V).
// plain: the near field summed in plain FP32 instead of error-free sums (an inner operator:
// about 1e-6 relative to a smooth product instead of 1e-10 of input-dependent noise).
void metric_apply_strided(rs_metric *M, double w_hi, double w_lo, int nb, const double *xs,
                          size_t ldx, double *ys, size_t ldy, bool plain = false);
// ys = scale L^V xs.
void vfrac_apply_strided(rs_vfrac *V, double scale, int nb, const double *xs, size_t ldx,
                         double *ys, size_t ldy, bool plain = false);

}  // namespace rsg
