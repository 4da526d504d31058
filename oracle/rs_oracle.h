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

/* ---- constraints, saddle, preconditioner, GMRES and the step (rs_oracle_solve.cpp) ---- */

/* A list of constraints (RS/src/constraints/mod.rs:36-110): kind 0 barycenter, 1 pins, 2 area,
 * 3 volume; comp = component or -1 (barycenter: every component separately when per_component,
 * else one global group; area/volume: the whole mesh). n_target[i] doubles of `target` (in
 * order) give the targets (0: the current value); n_pin[i] vertices of `pin` are pinned. */
typedef struct rso_constraints {
  int n;
  const int *kind;
  const int *comp;
  const int *n_target;
  const double *target;
  const int *n_pin;
  const uint32_t *pin;
  int per_component;
} rso_constraints;

/* Options of the hierarchical saddle solver (HierarchicalOptions, RS/src/solve/iterative.rs:348-395;
 * PreconditionerOptions, RS/src/solve/precond.rs:466-583; GmresOptions, gmres.rs:135-190). */
typedef struct rso_solver_options {
  double chi;
  int leaf_size, leaf_pairs;
  double tp_weight;
  int low_order;
  double eps_rel, eps_multi_rel;
  int preconditioner; /* 1 the augmented vertex-pair preconditioner, 0 none */
  int coarse;         /* the coarse correction for components without own positional rows */
  int restart, max_iterations;
  double tolerance;
} rso_solver_options;
rso_solver_options rso_solver_options_default(void);

/* Options of one step (FlowOptions, RS/src/step/options.rs:290-382). energy_theta < 0: the
 * exact energy, else Barnes-Hut lists at that opening angle. backend 0: dense saddle (LU),
 * 1: hierarchical (the solver options). start_rule 0 absolute start_value, 1 start_value mean
 * edge lengths for the farthest vertex, 2 reference 2/|x|, 3 grow previous_tau by start_value
 * (without one: first_rule with first_value). max_halvings < 0: unbounded. l0 = 0: the mean edge
 * length of the positions. */
typedef struct rso_step_options {
  double energy_theta;
  int leaf_size;
  int backend;
  rso_solver_options solver;
  int start_rule;
  double start_value;
  int first_rule;
  double first_value;
  double previous_tau;
  double armijo_c;
  int max_halvings;
  double tau_min_rel;
  int newton_fixed, newton_max;
  int guard_projection;
  double l0;
} rso_step_options;
rso_step_options rso_step_options_default(void);

const char *rso_solve_last_error(void);

/* ConstraintSet::new / values / jacobian (constraints/mod.rs:191-604): rows in order, their
 * kind (0..3), whether positional, Phi, the dense Jacobian (n_rows x 3V, may be NULL), the
 * component of every vertex and the number of components. */
int rso_constraint_rows(int nv, const double *pos, int nf, const uint32_t *faces, const rso_constraints *c,
                        int max_rows, int *n_rows, int *kind, int *positional, double *phi, double *jac,
                        uint32_t *vcomp, int *n_comp);

/* The dense nested saddle (RS/src/solve/dense.rs, schur.rs:101-356) with A = w_TP (B + c_lo B0)
 * and the exact energy gradient g: the direction x, S = -C_N Z (kn x kn), Phi_N, the Newton
 * correction h and <g, x>. */
int rso_dense_saddle(int nv, const double *pos, int nf, const uint32_t *faces, double alpha, double beta,
                     double tp_weight, int low_order, const rso_constraints *c, int max_rows, int *kq, int *kn,
                     double *g, double *x, double *S, double *phin, double *h, double *gx);

/* The dense face-pair preconditioner (RS/src/solve/dense.rs:527-600): eps, L_{2-s} (V x V),
 * L' ((3V+kQ)^2) and z = P^-1 [r; 0] (3V). */
int rso_dense_precond(int nv, const double *pos, int nf, const uint32_t *faces, double alpha, double beta,
                      double eps_rel, const rso_constraints *c, const double *r, double *eps, double *lfr, double *lp,
                      double *z, int *kq);

#define RSO_STEP_REPORT_LEN 28
/* One step (Session::step_inner, RS/src/step/session.rs:749-1100). report: 0 F0, 1 F after the
 * projection, 2 F at the accepted trial, 3 tau (0 stuck), 4 tau0, 5 accepted, 6 halvings,
 * 7 slope <g,x>, 8 |x|_2, 9 |x|_inf, 10 l0, 11 Newton rounds, 12 projection status (0 converged,
 * 1 max rounds, 2 not improving, 3 blocked), 13 |g|_2, 14 rows, 15 blocked projections,
 * 16..22 seconds (objective build, energy, solver build, solves, line search, projection, total),
 * 23 operator products, 24 GMRES iterations, 25 worst true relative residual, 26 solves,
 * 27 preconditioner applications. trials: (tau, energy, outcome) with outcome 0 accepted,
 * 1 armijo-failed, 2 non-finite, 3 projection blocked. */
int rso_step(int nv, const double *pos, int nf, const uint32_t *faces, double alpha, double beta,
             const rso_constraints *c, const rso_step_options *o, double *pos_out, double *x_out, double *g_out,
             double *report, double *trials, int max_trials, int *n_trials, double *phi_before, double *phi_after,
             int max_rows);

/* The hierarchical saddle solver alone (hierarchical_saddle_with, iterative.rs:487-575): A' and
 * P^-1 on vectors [x (3V); l (k_Q)], GMRES solves (report 5 per rhs: iterations, true relative
 * residual, converged, seconds, cycles). info: eps, multi (0/1), fractional scale, coarse
 * dimension, build seconds (metric, fractional tree, Laplacian factor, coarse space). */
typedef struct rso_hsolver rso_hsolver;
int rso_hsolver_build(int nv, const double *pos, int nf, const uint32_t *faces, double alpha, double beta,
                      const rso_solver_options *o, const rso_constraints *c, rso_hsolver **out);
void rso_hsolver_free(rso_hsolver *h);
int rso_hsolver_dims(rso_hsolver *h, int64_t *n_dofs, int64_t *n_constraints);
int rso_hsolver_set_gmres(rso_hsolver *h, int restart, int max_iterations, double tolerance);
int rso_hsolver_apply(rso_hsolver *h, int nb, const double *xs, double *ys);
int rso_hsolver_precondition(rso_hsolver *h, int nb, const double *rs, double *zs);
int rso_hsolver_solve(rso_hsolver *h, int nb, const double *rhs, double *sol, double *report5);
int rso_hsolver_info(rso_hsolver *h, double *out8);

#ifdef __cplusplus
}
#endif
#endif
