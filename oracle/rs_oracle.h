/*
 * FP64 CPU oracle of the Repulsive-Surfaces hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain restatement, in C++ and double precision, of the algorithms of the
 * `ddg-repulsive-surfaces` crate (m1el/ddg-tools) that the GPU library accelerates.
 * It is used by the tests (as the checker), by `__graft_entry__.smoke()` and by the
 * CPU-baseline leg of `bench.py`. The product library (`librsgpu.so`) never links,
 * loads or calls it.
 *
 * Every function states the reference file:line it follows (paths relative to the
 * reference project; `RS/` = crates/ddg-repulsive-surfaces/, `RC/` =
 * crates/ddg-repulsive-curves/).
 *
 * Parity pins: the Lean-oracle golden fixtures (lean/oracle/fixtures/rs/NAME.in and .out, tasks
 * energy/df/metric/precond/saddle) and the authors' C++ program dumps
 * (RS/tests/fixtures/reference/NAME.*) -- see tests/test_oracle_fixtures.py.
 *
 * Conventions: all arrays are flat, row-major, caller-owned. Positions are V x 3 doubles,
 * faces F x 3 uint32. Every entry point returns 0 on success or a nonzero status; the
 * message of the last failure is returned by rso_last_error().
 */
#ifndef RS_ORACLE_H
#define RS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (shared meaning with include/rsgpu.h). */
enum {
  RSO_OK = 0,
  RSO_INVALID_EXPONENTS = 1,
  RSO_INVALID_OPTION = 2,
  RSO_POSITION_COUNT = 3,
  RSO_NONFINITE_POSITION = 4,
  RSO_DEGENERATE_FACE = 5,
  RSO_NONFINITE_ENERGY = 6,
  RSO_TOPOLOGY = 7,
  RSO_SOLVER_DIVERGED = 8,
  RSO_SINGULAR = 9,
  RSO_INTERNAL = 99
};

const char *rso_last_error(void);
/* Sets the number of OpenMP-style worker threads the oracle may use (1 = sequential).
 * Results do not depend on it (every reduction has a fixed order). */
void rso_set_threads(int n);

/* Exponent validation (RS/src/kernel.rs:50-76). */
int rso_exponents_check(double alpha, double beta);

/* Per-face area, unit normal, barycenter (RS/src/geometry.rs:33-39).
 * out_area[F], out_normal[F*3], out_bary[F*3]. */
int rso_face_geometry(int nv, const double *pos, int nf, const uint32_t *faces,
                      double *out_area, double *out_normal, double *out_bary);

/* Exact all-pairs energy and differential (RS/src/energy/exact.rs:87-161).
 * dE may be NULL (value only, exact.rs:61-78). face_partials7 (F*7: d_area, d_bary[3],
 * d_normal[3]) may be NULL. */
int rso_exact_energy(int nv, const double *pos, int nf, const uint32_t *faces, double alpha,
                     double beta, double *energy, double *dE, double *face_partials7);

/* ---- Barnes-Hut evaluator (RS/src/energy/barnes_hut.rs) ---- */
typedef struct rso_bh rso_bh;

/* BhTree::build (barnes_hut.rs:156-195): validates positions, builds the face BVH
 * (RC/src/spatial/bvh.rs:126-220) and the interaction lists (barnes_hut.rs:743-808). */
int rso_bh_build(int nv, const double *pos, int nf, const uint32_t *faces, double theta,
                 int leaf_size, rso_bh **out);
void rso_bh_free(rso_bh *h);
/* BhTree::refit (barnes_hut.rs:204-229). */
int rso_bh_refit(rso_bh *h, const double *pos);

/* Sizes: n_nodes, n_leaves, n_lumped, n_exact, n_partner_slots, pairs_exact. */
int rso_bh_sizes(const rso_bh *h, int64_t *out6);
/* Tree topology: node_start/end/right [n_nodes], order [F], leaves [n_leaves]. */
int rso_bh_tree(const rso_bh *h, uint32_t *start, uint32_t *end, uint32_t *right,
                uint32_t *order, uint32_t *leaves);
/* Build-time cluster geometry per node: bbox lo/hi [n_nodes*6], radius [n_nodes];
 * current aggregates: area [n_nodes], centroid [n_nodes*3], projector [n_nodes*6]. */
int rso_bh_clusters(const rso_bh *h, double *bbox6, double *radius, double *area,
                    double *centroid, double *projector);
/* Interaction lists in CSR form (barnes_hut.rs:61-81). Offsets have n_leaves+1 entries. */
int rso_bh_lists(const rso_bh *h, int64_t *lumped_off, uint32_t *lumped, int64_t *exact_off,
                 uint32_t *exact);

/* BhTree::energy (barnes_hut.rs:366-375, 583-614). */
int rso_bh_energy(const rso_bh *h, double alpha, double beta, double *energy);
/* BhTree::energy_and_differential (barnes_hut.rs:387-412, 478-579). dE [V*3] and
 * face_partials7 [F*7] (by face) may each be NULL. */
int rso_bh_energy_and_differential(const rso_bh *h, double alpha, double beta,
                                   double *energy, double *dE, double *face_partials7);

/* Pull-back of per-face partials to the vertices (RS/src/geometry.rs:87-188). */
int rso_pull_back(int nv, const double *pos, int nf, const uint32_t *faces,
                  const double *face_partials7, double *dE);

/* ---- hierarchical metric (RS/src/metric/hierarchical.rs, RS/src/spatial/block_tree.rs) ---- */
typedef struct rso_metric rso_metric;
/* FaceMetricTree::build (hierarchical.rs:302-363): face tree (leaf_size), block cluster tree
 * of h_hi = rho^-2s and h_lo = (nu_S^2 + nu_T^2)/2 rho^-4 rho^-2s (chi, leaf_pairs), H~ a. */
int rso_metric_build(int nv, const double *pos, int nf, const uint32_t *faces, double alpha,
                     double beta, double chi, int leaf_size, int leaf_pairs, rso_metric **out);
void rso_metric_free(rso_metric *h);
const char *rso_metric_last_error(void);
/* far blocks, near blocks, near entries, depth, nodes */
int rso_metric_stats(const rso_metric *h, int64_t *out5);
int rso_metric_blocks(const rso_metric *h, int64_t *far_ptr, uint32_t *far_col, double *far_coef,
                      int64_t *near_ptr, uint32_t *near_col);
int rso_metric_ha(const rso_metric *h, double *ha2);
/* y = (w_hi B~ + w_lo B~0) x for nb interleaved 3V vectors (hierarchical.rs:521-812). */
int rso_metric_apply(const rso_metric *h, double w_hi, double w_lo, int nb, const double *xs,
                     double *ys);

typedef struct rso_vfrac rso_vfrac;
/* VertexFractionalTree::build (hierarchical.rs:1017-1084): vertex BVH with dual-area masses,
 * kernel |f_v - f_w|^-(2 tau + 2). */
int rso_vfrac_build(int nv, const double *pos, const double *mass, double tau, double chi,
                    int leaf_size, int leaf_pairs, rso_vfrac **out);
void rso_vfrac_free(rso_vfrac *h);
int rso_vfrac_stats(const rso_vfrac *h, int64_t *out5);
/* y = L^V_tau x = 2 (a . H~a . x - a . H~(a . x)) per axis (hierarchical.rs:1313-1345). */
int rso_vfrac_apply(const rso_vfrac *h, int nb, const double *xs, double *ys);

/* first_contact of a mesh moving against itself, start + t velocity on [0, tau_end]
 * (RS/src/ccd.rs:762-884; no obstacles), with the exempt band of the start positions when
 * use_band (first_contact_with_band, ccd.rs:781-884). gap, max_iterations and close_factor are
 * CcdOptions (ccd.rs:86-111); reference_length 0 takes the mean edge length of start.
 * out7: contact found (0/1), windows, candidate pairs tested, close pairs, touching pairs,
 * exempt pairs, band vertices. */
int rso_ccd_first_contact(int nv, const double *start, int nf, const uint32_t *faces,
                          const double *velocity, double tau_end, double gap, double reference_length,
                          int max_iterations, double close_factor, int use_band, double *tau_max,
                          int64_t *out7);
/* intersecting_pairs (ccd.rs:1229-1279): sorted (f, g) pairs, up to cap written to out. */
int rso_ccd_intersecting_pairs(int nv, const double *pos, int nf, const uint32_t *faces, int64_t cap,
                               uint32_t *out, int64_t *n);
const char *rso_ccd_last_error(void);
/* The smallest vertex-triangle / edge-edge distance over the pairs CCD constrains. */
int rso_ccd_min_distance(int nv, const double *pos, int nf, const uint32_t *faces, double *out);

#ifdef __cplusplus
}
#endif
#endif
