/*
 * librsgpu -- GB300 (sm_103a) implementation of the data-parallel core of the
 * Repulsive-Surfaces flow (crate `ddg-repulsive-surfaces` of m1el/ddg-tools).
 *
 * A plain C ABI: opaque handles, plain pointers and sizes, int status codes. It is the
 * boundary a host in any language binds (the reference's Rust crate would bind it with
 * `extern "C"` declarations). Each entry point names the reference
 * interface it replaces (paths relative to the reference project; RS/ =
 * crates/ddg-repulsive-surfaces/).
 *
 * Conventions
 *  - Positions are V x 3 doubles (x, y, z per vertex); faces are F x 3 uint32 vertex ids;
 *    per-vertex vectors are interleaved `3 v + axis`, like the crate's `&[[f64; 3]]`.
 *  - `*_host` pointers are caller-owned host memory; `*_dev` pointers are device memory of
 *    the context's device (for example from cudaMalloc or a torch tensor).
 *  - All work is issued on the context's own CUDA stream (rs_ctx_stream); entry points with
 *    host outputs synchronise it before returning, `*_device` entry points do not.
 *  - Every function returns RS_OK (0) or an error status; rs_last_error() describes the last
 *    failure of the calling thread as the reference's `RsError::Gpu { operation, detail }`
 *    (RS/src/gpu/cuda.rs:19-24) or the matching `RsError` kind.
 *  - There is no CPU fallback: without a usable CUDA device every call fails with RS_GPU.
 */
#ifndef RSGPU_H
#define RSGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. Each maps to one `RsError` variant of RS/src/error.rs. */
enum rs_status {
  RS_OK = 0,
  RS_INVALID_EXPONENTS = 1,  /* RsError::InvalidExponents (RS/src/error.rs:110) */
  RS_INVALID_OPTION = 2,     /* RsError::InvalidOption (:119) */
  RS_POSITION_COUNT = 3,     /* RsError::PositionCountMismatch (:83) */
  RS_NONFINITE_POSITION = 4, /* RsError::NonFinitePosition (:90) */
  RS_DEGENERATE_FACE = 5,    /* RsError::DegenerateFace (:95) */
  RS_NONFINITE_ENERGY = 6,   /* RsError::NonFiniteEnergy (:104) */
  RS_TOPOLOGY = 7,           /* NoFaces / VertexOutOfRange / RepeatedVertex / DuplicateFace /
                                NonManifoldEdge / NonManifoldVertex / UnreferencedVertex */
  RS_SOLVER_DIVERGED = 8,    /* RsError::SolverDiverged (:174) */
  RS_SINGULAR = 9,           /* RsError::SingularSaddle (:169) */
  RS_GPU = 10,               /* RsError::Gpu (:218) */
  RS_CANCELLED = 11,         /* RsError::Cancelled: a step stopped by rs_flow_cancel */
  RS_INTERNAL = 99
};

typedef struct rs_ctx rs_ctx; /* GpuContext (RS/src/gpu/mod.rs:36-127) */
typedef struct rs_bh rs_bh;   /* BhTree + DeviceBh (RS/src/energy/barnes_hut.rs:114-127) */

/* ---------------------------------------------------------------- errors and devices */

/* The last failure of the calling thread: `operation` is a short word ("context",
 * "upload", "launch", "product", "surface", "energy", ...), `detail` free text; `kind` is
 * the RsError variant name ("Gpu", "DegenerateFace", ...). Strings stay valid until the
 * thread's next failing call. Replaces RsError::Gpu { operation, detail } (cuda.rs:19-24). */
const char *rs_last_error(void);
const char *rs_last_error_operation(void);
const char *rs_last_error_kind(void);

/* Number of CUDA devices (gpu::device_count, RS/src/gpu/mod.rs:89-100). */
int rs_device_count(int *count);
/* Name, compute capability and memory of device `ordinal`, without creating a context
 * (gpu::devices, RS/src/gpu/mod.rs:89-100, as gpu_info lists them:
 * crates/ddg-py/src/repulsive_surfaces.rs:1899-1938). */
int rs_device_info(int ordinal, char *name, int name_len, int *cc_major, int *cc_minor,
                   uint64_t *memory_bytes);

/* A context on device `ordinal` with its own non-blocking stream
 * (GpuContext::new, RS/src/gpu/mod.rs:102-127; cuda.rs:100-119). */
int rs_ctx_create(int ordinal, rs_ctx **out);
/* Releases the caller's handle. Objects built on the context (rs_bh, rs_metric, rs_vfrac,
 * rs_solver, rs_flow) hold it too, so handles may be freed in any order. */
void rs_ctx_free(rs_ctx *ctx);
/* The context's cudaStream_t, for callers that time or order work around it. */
int rs_ctx_stream(rs_ctx *ctx, void **stream);
int rs_ctx_synchronize(rs_ctx *ctx);
/* Device name and SM count (gpu_info, crates/ddg-py/src/python/repulsive_surfaces.rs:687-691). */
int rs_ctx_info(rs_ctx *ctx, char *name, int name_len, int *sm_count, int *cc_major,
                int *cc_minor);
/* Kernel launches issued by this context since creation (all entry points). */
int rs_ctx_launch_count(rs_ctx *ctx, int64_t *count);
/* Bytes the library has copied host -> device and device -> host since the process started
 * (all contexts). No counterpart in the crate. */
int rs_copy_counters(uint64_t *h2d_bytes, uint64_t *d2h_bytes);

/* ---------------------------------------------------------------- surface validation */

/* Surface::new topology checks (RS/src/surface.rs:132-330) followed by
 * Surface::validate_positions (surface.rs:513-541): no faces, vertex out of range, repeated
 * vertex, duplicate face, non-manifold edge or vertex, unreferenced vertex, position count,
 * non-finite position, degenerate face. Host-side, no device work. */
int rs_surface_validate(int nv, int nf, const uint32_t *faces, const double *positions_host);

/* The face BVH alone, built on the host exactly as rs_bh_build builds it (FaceTree::build,
 * RS/src/spatial/mod.rs:175-221; split rule RC/src/spatial/bvh.rs:126-220). No device work.
 * Arrays have room for `capacity` nodes (at most 2 nf - 1 are needed); box6 is lo xyz, hi xyz
 * per node at the given positions; radius the farthest box corner from the node centroid. */
int rs_face_tree_build(int nv, int nf, const uint32_t *faces, const double *positions_host,
                       int leaf_size, int capacity, uint32_t *start, uint32_t *end,
                       uint32_t *right, uint32_t *order, double *box6, double *radius,
                       int *n_nodes);

/* ---------------------------------------------------------------- Barnes-Hut energy */

/* BhTree::build + attach_gpu (RS/src/energy/barnes_hut.rs:156-195, 265-307): validates
 * the surface, builds the face BVH (leaf size `leaf_size`, split rule of
 * RC/src/spatial/bvh.rs:126-220) at `positions_host`, uploads it, and builds the frozen
 * interaction lists for the opening angle `theta` ON THE DEVICE (barnes_hut.rs:743-808). */
int rs_bh_build(rs_ctx *ctx, int nv, int nf, const uint32_t *faces,
                const double *positions_host, double theta, int leaf_size, rs_bh **out);

/* BhTree::attach_gpu with the tree and lists built by the caller (the crate's own host
 * build): node ranges/right children [n_nodes], the element order [nf], and the CSR
 * lists per leaf (leaves in increasing node index; offsets have n_leaves+1 entries).
 * `positions_host` sets the current positions (as rs_bh_refit). */
int rs_bh_attach(rs_ctx *ctx, int nv, int nf, const uint32_t *faces,
                 const double *positions_host, int n_nodes, const uint32_t *node_start,
                 const uint32_t *node_end, const uint32_t *node_right, const uint32_t *order,
                 const int64_t *lumped_off, const uint32_t *lumped, const int64_t *exact_off,
                 const uint32_t *exact, rs_bh **out);
void rs_bh_free(rs_bh *bh);

/* BhTree::refit (barnes_hut.rs:204-229): new positions, same topology, boxes and lists. */
int rs_bh_refit(rs_bh *bh, const double *positions_host);
int rs_bh_refit_device(rs_bh *bh, const double *positions_dev);

/* BhTree::try_energy (barnes_hut.rs:350-360): the energy on the frozen lists. */
int rs_bh_energy(rs_bh *bh, double alpha, double beta, double *energy);

/* BhTree::energy_and_differential (barnes_hut.rs:387-412): energy and dE/df_v, V x 3.
 * NonFiniteEnergy names the culprit pair (faces[2]) when not finite. */
int rs_bh_energy_and_differential(rs_bh *bh, double alpha, double beta, double *energy,
                                  double *differential_host);

/* Device-resident variant: energy (one double) and differential (V x 3 doubles) written to
 * device memory on the context stream, without synchronising. */
int rs_bh_energy_and_differential_device(rs_bh *bh, double alpha, double beta,
                                         double *energy_dev, double *differential_dev);

/* BhTree::try_face_partials (barnes_hut.rs:421-471): per-face (d_area, d_bary[3],
 * d_normal[3]) by face index, F x 7. */
int rs_bh_face_partials(rs_bh *bh, double alpha, double beta, double *energy,
                        double *partials7_host);

/* Counts of InteractionLists (barnes_hut.rs:94-107) and the tree:
 * out[0..7] = n_nodes, n_leaves, n_lumped, n_exact, n_partner_slots, pairs_exact,
 *             lumped_interactions (sum over lumped entries of the leaf's face count). */
int rs_bh_sizes(rs_bh *bh, int64_t *out7);
// Seconds spent in the phases of rs_bh_build: geometry, tree, topology, list counts, list
// fill, list finish, refit. No crate counterpart (diagnostics).
int rs_bh_build_times(rs_bh *bh, double *out7);
/* The tree and lists (for parity checks): arrays sized by rs_bh_sizes. */
int rs_bh_export(rs_bh *bh, uint32_t *node_start, uint32_t *node_end, uint32_t *node_right,
                 uint32_t *order, int64_t *lumped_off, uint32_t *lumped, int64_t *exact_off,
                 uint32_t *exact);
/* Culprit pair of the last non-finite evaluation (faces[2]), or -1,-1. */
int rs_bh_culprit(rs_bh *bh, int64_t *faces2);

/* Average device time (ms) of each kernel of the last `rs_bh_profile` run: runs the
 * energy+differential `reps` times with CUDA events around every launch and returns up to
 * `max_kernels` (name, ms) pairs; names are NUL-separated in `names` (size names_len). */
int rs_bh_profile(rs_bh *bh, double alpha, double beta, int reps, char *names, int names_len,
                  double *ms, int max_kernels, int *n_kernels);

/* ---------------------------------------------------------------- Hs metric (H-matrix) */

typedef struct rs_metric rs_metric; /* FaceMetricTree + GpuFaceMetric (RS/src/metric/hierarchical.rs:279-812) */
typedef struct rs_vfrac rs_vfrac;   /* VertexFractionalTree + GpuVertexFractional (hierarchical.rs:998-1346) */

/* FaceMetricTree::build / build_on_gpu (hierarchical.rs:302-468): face BVH (leaf_size <= 8),
 * block cluster tree of h_hi = rho^-2s and h_lo = (nu_S^2 + nu_T^2)/2 rho^-4 rho^-2s with
 * separation chi and leaf_pairs (ClusterTreeOptions, hierarchical.rs:63-108; defaults 0.5,
 * 8, 64), far coefficients, and the far part of H~a. The near field is evaluated in every
 * product on the device, not stored. */
int rs_metric_build(rs_ctx *ctx, int nv, int nf, const uint32_t *faces,
                    const double *positions_host, double alpha, double beta, double chi,
                    int leaf_size, int leaf_pairs, rs_metric **out);
void rs_metric_free(rs_metric *m);
/* GpuFaceMetric::apply_batch (RS/src/gpu/mod.rs:318-341, hierarchical.rs:540-622):
 * ys = (w_hi B~ + w_lo B~0) xs for nb interleaved 3V vectors (stacked). */
int rs_metric_apply(rs_metric *m, double w_hi, double w_lo, int nb, const double *xs_host,
                    double *ys_host);
int rs_metric_apply_device(rs_metric *m, double w_hi, double w_lo, int nb, const double *xs_dev,
                           double *ys_dev);
/* rs_metric_apply_device without device allocation. No counterpart in the reference: the
 * crate's products allocate on the host heap only. Same result as rs_metric_apply_device;
 * the per-call scratch (at most 64 MiB per device: InvalidOption above that, e.g. three
 * vectors on 80,000 faces) lives in one file-scope device array, so it serves callers that
 * must not allocate while the product runs (a host whose device memory is held by its own
 * pool after set-up; a latency-critical stream, as cudaMalloc/cudaFree can synchronize the
 * device). The 64 MiB are a file-scope device array: they stay resident on every device
 * where the library's metric kernels are loaded, whether or not this call is ever made (with
 * CUDA_MODULE_LOADING=LAZY, the CUDA default, from the first metric build or product on that
 * device). Calls that overlap in time race on the shared scratch, and a call also shares the
 * metric's arrival counters with the other products of the same rs_metric: serialize them
 * with each other and with every product on that metric. The first call on a device looks up
 * the scratch address; make that call outside any stream capture. */
int rs_metric_apply_device_noalloc(rs_metric *m, double w_hi, double w_lo, int nb,
                                   const double *xs_dev, double *ys_dev);
/* BctStats (far blocks, near blocks, near entries, depth, nodes). */
int rs_metric_stats(rs_metric *m, int64_t *out5);
// Seconds spent in the phases of rs_metric_build: geometry, tree, projectors, blocks, face
// records, work items, far coefficients, device part. No crate counterpart (diagnostics).
int rs_metric_build_times(rs_metric *m, double *out8);
/* The blocks grouped by row node: far_ptr [nodes+1], far_col, near_ptr [nodes+1], near_col. */
int rs_metric_blocks(rs_metric *m, uint32_t *far_ptr, uint32_t *far_col, uint32_t *near_ptr,
                     uint32_t *near_col);
/* Per-kernel average device time of `reps` products of nb vectors (as rs_bh_profile). */
int rs_metric_profile(rs_metric *m, double w_hi, double w_lo, int nb, int reps, char *names,
                      int names_len, double *ms, int max_kernels, int *n_kernels);

/* VertexFractionalTree::build / build_on_gpu (hierarchical.rs:1017-1151): vertex BVH with
 * masses `mass_host` (dual areas), kernel |f_v - f_w|^-(2 tau + 2). */
int rs_vfrac_build(rs_ctx *ctx, int nv, const double *positions_host, const double *mass_host,
                   double tau, double chi, int leaf_size, int leaf_pairs, rs_vfrac **out);
void rs_vfrac_free(rs_vfrac *v);
/* GpuVertexFractional::apply_batch (RS/src/gpu/mod.rs:361-371): ys = L^V_tau xs. */
int rs_vfrac_apply(rs_vfrac *v, int nb, const double *xs_host, double *ys_host);
int rs_vfrac_apply_device(rs_vfrac *v, int nb, const double *xs_dev, double *ys_dev);
int rs_vfrac_stats(rs_vfrac *v, int64_t *out5);

/* ---------------------------------------------------------------- saddle solve */

typedef struct rs_solver rs_solver; /* HierarchicalSaddle (RS/src/solve/iterative.rs:426-575) */

/* Options of the hierarchical saddle solver (HierarchicalOptions, iterative.rs:348-395;
 * PreconditionerOptions, RS/src/solve/precond.rs:466-583; GmresOptions, gmres.rs:135-190). */
typedef struct rs_solver_options {
  double chi;            /* block cluster tree separation (0.5) */
  int leaf_size;         /* BVH leaf size, <= 8 (8) */
  int leaf_pairs;        /* near-block size limit (64) */
  int restart;           /* GMRES restart (30) */
  double tolerance;      /* true relative residual (1e-6) */
  int max_iterations;    /* GMRES iterations over all cycles (200) */
  double tp_weight;      /* w_TP (1) */
  int low_order;         /* keep B0 (1) */
  double eps_rel;        /* eps_rel of eps = eps_rel tr W / tr M (1e-10) */
  double eps_multi_rel;  /* eps when a global barycenter spans several components (1e-4) */
  int barycenter_per_component; /* 1: one barycenter group per component, 0: global (0) */
  int vcycles;           /* conjugate-gradient steps, each preconditioned by one multigrid
                            V-cycle, per L' solve (6) */
  int preconditioner;    /* 1: the fractional preconditioner, 0: none */
  int clamp_laplacian;   /* 1: edges with negative cotan weight dropped from the
                            preconditioner's Laplacian (an M-matrix for multigrid), 0: cotan */
  int coarse;            /* the coarse (deflation) correction on the translations of components
                            that no positional row of their own fixes: a global barycenter on
                            several components (PreconditionerOptions::coarse, CoarseSpace,
                            RS/src/solve/coarse.rs; 1) */
  int inner_plain;       /* 1: the Arnoldi steps apply an inner operator whose near fields (of the
                            metric, and of the preconditioner's vertex product) are summed in plain
                            FP32; every cycle-start residual, and so the convergence test and the
                            reported residual, uses the full operator. 0: the full operator
                            throughout. No counterpart in the crate (1) */
} rs_solver_options;

rs_solver_options rs_solver_options_default(void);

/* hierarchical_saddle_with (iterative.rs:487-575) for a surface and positions: the metric
 * operator A' = [w (B~ + c_lo B~0) + C_Q^T ; C_Q] with barycenter rows C_Q, and the augmented
 * fractional preconditioner L'^-1 + L'^-1 ((s L^V_{2-s} - K) x I3) L'^-1 (L'^-1 applied by
 * multigrid V-cycles on the device instead of the reference's sparse LDL^T). */
int rs_solver_build(rs_ctx *ctx, int nv, int nf, const uint32_t *faces,
                    const double *positions_host, double alpha, double beta,
                    const rs_solver_options *opts, rs_solver **out);
void rs_solver_free(rs_solver *s);
/* n_dofs = 3V, n_constraints = k_Q (3 per barycenter group). Vectors are [x (3V); l (k_Q)]. */
int rs_solver_dims(rs_solver *s, int64_t *n_dofs, int64_t *n_constraints);
/* Host seconds of rs_solver_build by phase: [metric tree and upload, vertex fractional tree,
 * Laplacian block, multigrid set-up, multigrid upload, total]. No counterpart in the crate. */
int rs_solver_build_times(rs_solver *s, double *out6);
/* Changes the GMRES settings of later solves (GmresOptions, RS/src/solve/gmres.rs:135-190). */
int rs_solver_set_gmres(rs_solver *s, int restart, int max_iterations, double tolerance);
/* Rows and nonzeros of every multigrid level of the preconditioner's Laplacian block, finest
 * first: out[2 l] = rows, out[2 l + 1] = nonzeros (the coarsest level is inverted densely).
 * No counterpart in the crate. */
int rs_solver_multigrid_levels(rs_solver *s, int64_t *out, int max_levels, int *n_levels);
/* Solves nb host right-hand sides once with phase timing (CUDA events on the context's
 * stream) and reports the milliseconds spent per phase for that solve: solve, operator,
 * precondition, precondition_multigrid_cg, precondition_fractional, gmres_orthogonalize.
 * Names are NUL-separated in `names`. No counterpart in the crate. */
int rs_solver_profile(rs_solver *s, int nb, const double *rhs_host, char *names, int names_len,
                      double *ms, int max_kernels, int *n_kernels);
/* LinearOperator::apply_batch (gmres.rs:32-52): ys = A' xs for nb stacked vectors. */
int rs_solver_apply(rs_solver *s, int nb, const double *xs_host, double *ys_host);
int rs_solver_apply_device(rs_solver *s, int nb, const double *xs_dev, double *ys_dev);
/* Preconditioner::apply_batch (gmres.rs:55-75): zs = P^-1 rs. */
int rs_solver_precondition(rs_solver *s, int nb, const double *rs_host, double *zs_host);
int rs_solver_precondition_device(rs_solver *s, int nb, const double *rs_dev, double *zs_dev);
/* SaddleSolver::solve_many (RS/src/solve/mod.rs:107-130): right-preconditioned GMRES on the
 * device for nb (1..4) right-hand sides [a; b] at once; report (5 per rhs): iterations, true
 * relative residual, converged, seconds, cycles. SolverDiverged above 0.1 (gmres.rs:196). */
int rs_solver_solve_many(rs_solver *s, int nb, const double *rhs_host, double *sol_host,
                         double *report);
/* The convergence history of right-hand side q of the last solve (GmresReport::history and the
 * explicit residual of every cycle start, RS/src/solve/gmres.rs:200-225): up to max_iter
 * estimated relative residuals per Arnoldi step and up to max_cycles explicit ones. No
 * counterpart call in the crate, where the report is a returned struct. */
int rs_solver_history(rs_solver *s, int q, double *estimates, int max_iter, int *n_iter,
                      double *cycle_residuals, int max_cycles, int *n_cycles);
int rs_solver_solve_many_device(rs_solver *s, int nb, const double *rhs_dev, double *sol_dev,
                                double *report);

/* The last stage of the recovery chain (RobustHierarchical::escalate, RS/src/step/
 * direction.rs:238-300; DenseSaddle, RS/src/solve/dense.rs:282-470): A' with the exact metric
 * (every face pair, chi = 0) assembled densely on the device, equilibrated and factored by LU
 * with partial pivoting in FP64, per axis ((V + G) square with the barycenter rows); nb (1..4)
 * right-hand sides solved with one step of iterative refinement. The factor is built on the
 * first call and kept. Report as rs_solver_solve_many (iterations 0, relative residual on the
 * dense operator, converged 1). InvalidOption above RS_DENSE_FALLBACK_MAX_VERTICES vertices;
 * SingularSaddle when the equilibrated pivot ratio is at most 1e-13 (PIVOT_TOLERANCE). */
#define RS_DENSE_FALLBACK_MAX_VERTICES 6000 /* DENSE_FALLBACK_MAX_VERTICES, direction.rs:238 */
int rs_solver_dense_solve_many_device(rs_solver *s, int nb, const double *rhs_dev, double *sol_dev,
                                      double *report);
/* min |u_ii| / max |u_ii| of the equilibrated dense factor (0 before the first dense solve). */
int rs_solver_dense_pivot_ratio(rs_solver *s, double *ratio);

/* ---------------------------------------------------------------- one Hs step */

typedef struct rs_flow rs_flow; /* Session (RS/src/step/session.rs:371-1369), step_inner's
                                   energy / solve / line-search / projection parts */

typedef struct rs_flow_options {
  double alpha, beta;        /* exponents (6, 12) */
  double theta;              /* Barnes-Hut opening (BhOptions, 0.5) */
  int leaf_size;             /* (8) */
  rs_solver_options solver;  /* FLOW_GMRES defaults: restart 60, tolerance 1e-3 */
  int hold_area;             /* hold the initial total area (a Schur row) */
  int hold_volume;           /* hold the initial volume (a Schur row) */
  double armijo_c;           /* ArmijoRule::Standard c (1e-2) */
  int max_halvings;          /* line-search halvings before a step is refused (30) */
  int newton_max;            /* NewtonSteps::UntilTolerance max (5) */
  int ccd;                   /* cap the first trial by continuous collision detection (0) */
  double ccd_gap;            /* CcdOptions: gap relative to the initial mean edge length (0.05), */
  int ccd_max_iterations;    /* advances per pair and window (100), */
  double ccd_close_factor;   /* closing fraction of pairs closer than the gap (0.5) */
  /* StartRule (RS/src/step/options.rs:60-107; session.rs:1604-1615): 3 GrowPrevious (the last
   * accepted tau times start_value; the first step uses first_rule with first_value), 0 Absolute
   * (tau = start_value), 1 MaxDisplacement (the farthest vertex moves start_value initial mean
   * edge lengths), 2 Reference (tau = 2 / |x|). Default: 3, 2.0, first 1, 1.0. */
  int start_rule;
  double start_value;
  int first_rule;
  double first_value;
  double tau_min_rel;        /* the search stops below tau_min_rel l0 / |x|_inf (1e-12) */
  int newton_fixed;          /* 1: NewtonSteps::Fixed(newton_max), 0: UntilTolerance (0) */
  double newton_tolerance;   /* a held row is met within newton_tolerance |target| (1e-8,
                                NONLINEAR_TOLERANCE, RS/src/constraints/mod.rs:147) */
  double area_target;        /* NaN: the initial total area */
  double volume_target;      /* NaN: the initial volume */
  int guard_projection;      /* keep an Armijo trial only if its projection is admissible (1) */
  /* The recovery chain of a diverged solve (RobustHierarchical, direction.rs:269-379): the
   * solves are repeated with restart 60 and retry_max_iterations GMRES iterations (0: the
   * crate's max(4 solver.max_iterations, 800)), then, if dense_fallback is set and the mesh has
   * at most RS_DENSE_FALLBACK_MAX_VERTICES vertices, by the dense LU (1). */
  int retry_max_iterations;
  int dense_fallback;
} rs_flow_options;

rs_flow_options rs_flow_options_default(void);

/* Session::new (session.rs:371): the surface, its positions and the options; the initial
 * barycenter (always held), area and volume become the targets. */
int rs_flow_create(rs_ctx *ctx, int nv, int nf, const uint32_t *faces,
                   const double *positions_host, const rs_flow_options *opts, rs_flow **out);
void rs_flow_free(rs_flow *f);

/* ---------------------------------------------------------------- learned preconditioner
 * No counterpart in the crate. A per-vertex network with one-ring message passing (three
 * layers, hidden width 64, SiLU; BF16 weights, FP32 accumulation) maps a residual r and the
 * cheap plain-preconditioned y = P_cheap^-1 r, with the surface's positions, normals and dual
 * areas, to z = y + rms(y) N(.), an approximation of A'^-1 r for flexible GMRES. The plain
 * preconditioner stays the fallback: a learned solve that does not reach the tolerance within
 * its iteration cap is repeated with the plain one. */
typedef struct rs_learned rs_learned; /* the network: parameters, Adam state, activations */
typedef struct rs_lgraph rs_lgraph;   /* a surface: one-ring adjacency and static features */
int rs_learned_create(rs_ctx *ctx, uint64_t seed, rs_learned **out);
void rs_learned_free(rs_learned *m);
int rs_learned_parameter_count(rs_learned *m, int64_t *count);
int rs_learned_get_parameters(rs_learned *m, float *host);
int rs_learned_set_parameters(rs_learned *m, const float *host);
/* The accumulated gradient (cleared by rs_learned_adam_step and rs_learned_set_parameters). */
int rs_learned_get_gradient(rs_learned *m, float *host);
int rs_lgraph_create(rs_ctx *ctx, int nv, int nf, const uint32_t *faces, const double *positions_host,
                     rs_lgraph **out);
void rs_lgraph_free(rs_lgraph *g);
/* z = y + rms(y) N(features(r, y)) for nb stacked 3V vectors on the device. */
int rs_learned_apply_device(rs_learned *m, rs_lgraph *g, int nb, const double *r_dev,
                            const double *y_dev, double *z_dev);
/* One training sample (3V device vectors): the loss |z - zt|^2 / max(|zt|^2, |y|^2) and its gradient,
 * added to the accumulated gradient. */
int rs_learned_loss_and_gradient_device(rs_learned *m, rs_lgraph *g, const double *r_dev,
                                        const double *y_dev, const double *zt_dev, double *loss);
/* Adam on the accumulated gradient (clipped to [-clip, clip] per parameter when clip > 0),
 * which it then clears. */
int rs_learned_adam_step(rs_learned *m, double lr, double clip);
/* Sets (model != NULL) or clears the learned preconditioner of a solver: cheap_steps CG steps
 * for y, GMRES capped at max_iterations (0: the solver's cap) before the plain fallback. */
int rs_solver_set_learned(rs_solver *s, rs_learned *model, rs_lgraph *graph, int cheap_steps,
                          int max_iterations);
/* Learned solves and how many of them fell back to the plain preconditioner. */
int rs_solver_learned_counts(rs_solver *s, int64_t *solves, int64_t *fallbacks);

/* ---- Continuous collision detection (RS/src/ccd.rs) ---------------------------------- */

typedef struct rs_ccd rs_ccd;
/* CcdOptions (RS/src/ccd.rs:86-111): gap relative to the reference length (0.05), the
 * reference length (0: the mean edge length of the start positions), advances per pair and
 * window (100), the fraction of its initial distance a pair closer than the gap may close to
 * (0.5). The broad-phase leaf size is 8. */
typedef struct rs_ccd_options {
  double gap;
  double reference_length;
  int max_iterations;
  double close_factor;
} rs_ccd_options;
rs_ccd_options rs_ccd_options_default(void);
/* The surface's topology (faces, its sorted edge list) on the device, for repeated queries. */
int rs_ccd_create(rs_ctx *ctx, int nv, int nf, const uint32_t *faces, rs_ccd **out);
void rs_ccd_free(rs_ccd *c);
/* first_contact (RS/src/ccd.rs:762-884) of the mesh moving as start + t velocity (host arrays,
 * V x 3) on [0, tau_end], against itself: the largest tau_max <= tau_end that keeps every
 * vertex-triangle pair (vertex not in the triangle) and every edge-edge pair without a common
 * vertex at distance >= gap (pairs closer at t = 0: >= close_factor times their distance;
 * touching pairs unconstrained). With a band set (rs_ccd_set_band) a pair whose two elements
 * both have a vertex in the band is exempt (first_contact_with_band, ccd.rs:781-884). No
 * obstacles. tau_max is bitwise the crate's. report7 (may be NULL): contact found (0/1),
 * windows, candidate pairs tested, close pairs, touching pairs, exempt pairs, distance
 * evaluations (the last depends on the order pairs are met and is not the crate's count). */
int rs_ccd_first_contact(rs_ccd *c, const double *start, const double *velocity, double tau_end,
                         const rs_ccd_options *o, double *tau_max, int64_t *report7);
/* IntersectionBand::new (ccd.rs:1292-1319) of `positions` (V x 3, host), kept for the following
 * rs_ccd_first_contact calls: the vertices of the intersecting faces widened by one ring. NULL
 * positions clear it. n_pairs: intersecting face pairs; n_vertices: band vertices (0: the mesh
 * is embedded and nothing is exempt). */
int rs_ccd_set_band(rs_ccd *c, const double *positions, int64_t *n_pairs, int64_t *n_vertices);
/* intersecting_pairs (ccd.rs:1229-1279): the face pairs (f, g), f < g, that intersect, sorted;
 * up to cap pairs are written to out (2 per pair), *n is their number. */
int rs_ccd_intersecting_pairs(rs_ccd *c, const double *positions, int64_t cap, uint32_t *out, int64_t *n);
/* Wall seconds of the last rs_ccd_first_contact. No counterpart in the crate. */
int rs_ccd_last_seconds(rs_ccd *c, double *seconds);

#define RS_FLOW_REPORT_LEN 30
/* Session::step (session.rs:724-747): one step. report[RS_FLOW_REPORT_LEN]:
 *  0 energy before, 1 energy after the projection (on the step's lists; the energy before
 *  when refused), 2 accepted tau (0: refused), 3 halvings,
 *  4..6 GMRES iterations of the solves (area row, volume row, direction),
 *  7 worst true relative residual, 8 seconds of the step, 9 tree and lists, 10 energy,
 *  11 solver build, 12 solves, 13 line search, 14 projection, 15 accepted (1/0),
 *  16 slope g.x, 17 relative nonlinear-constraint residual after the projection,
 *  18 fallbacks: solves repeated with restart 60 and the larger iteration cap after GMRES
 *     ended above the divergence threshold (RobustHierarchical, direction.rs:269-379),
 *  19 learned-preconditioner solves, 20 of them repeated with the plain preconditioner,
 *  21 gradient norm |dE|_2 over the 3V coordinates (StepReport::gradient_norm, session.rs:161-162),
 *  22 the first trial's step size (tau0, after the collision cap), 23 |x|_inf, the largest
 *     coordinate of the direction,
 *  24 Newton rounds of the projection, 25 projection status (0 converged: every held row within
 *     1e-12 relative, or no held rows; 1 the rounds were used up: ProjectionStatus::MaxRounds,
 *     solve/schur.rs:450-461), 26 energy at the accepted trial, before the projection,
 *  27 tau_max of the collision detection (NaN when it is off), 28 its seconds.
 * With ccd on, the first trial is min(tau0, 2/3 tau_max) when the motion x -> x - t d meets a
 * contact before tau0 (session.rs:927-955; reference length the initial mean edge length),
 * with the exempt band of the step's start positions. The projection guard is not applied. */
int rs_flow_step(rs_flow *f, double *report);
/* The current positions (V x 3). */
int rs_flow_positions(rs_flow *f, double *positions_host);
/* The energy, differential and constrained direction at the current positions, without a line
 * search (Objective::evaluate and SchurComplement::with_direction, RS/src/step/objective.rs:
 * 151-249, RS/src/solve/schur.rs:101-126, as step_inner computes them, session.rs:771-860).
 * report as rs_flow_step's entries 0, 4..12, 16, 18, 21, 23; the positions do not change. */
int rs_flow_direction(rs_flow *f, double *report);
/* The direction x (f <- f - tau x) and the differential g (V x 3 each) of the last
 * rs_flow_step or rs_flow_direction (StepReport's direction and gradient, session.rs:1255-1262). */
int rs_flow_last_direction(rs_flow *f, double *x_host, double *g_host);
/* The saddle solutions of the last rs_flow_step or rs_flow_direction: the k Schur columns
 * Z_r = A'^-1 [C_N^T e_r; 0] of the held rows (area first, then volume), then
 * y = A'^-1 [g; 0], each n = 3V + k_Q entries [x; multipliers] (SchurComplement::z and the
 * direction's solve, RS/src/solve/schur.rs:101-126). sol_host NULL: only *n_held and *n. No
 * counterpart call in the crate (a diagnostic, for checking the solves against an FP64 operator). */
int rs_flow_last_solutions(rs_flow *f, double *sol_host, int *n_held, int64_t *n);
/* The line-search trials of the last step (StepReport::trials, session.rs:1262): up to
 * max_trials triples (tau, energy, outcome: 0 accepted, 1 Armijo failed, 2 non-finite,
 * 3 projection blocked); *n_trials is their number. */
int rs_flow_last_trials(rs_flow *f, double *out3, int max_trials, int *n_trials);
/* Uses (model != NULL) or stops using a learned preconditioner in the following steps (see
 * rs_solver_set_learned); the model must outlive its use. No counterpart in the crate. */
int rs_flow_set_learned(rs_flow *f, rs_learned *model, int cheap_steps, int max_iterations);
/* Asks the running step (between line-search trials) and every later step to stop with
 * RS_CANCELLED; the positions stay those of the last completed step (Session's cancel flag,
 * session.rs:989-998). Safe from any thread; never waits. rs_flow_cancel(f, 0) clears it. */
int rs_flow_cancel(rs_flow *f, int cancel);

#ifdef __cplusplus
}
#endif
#endif
