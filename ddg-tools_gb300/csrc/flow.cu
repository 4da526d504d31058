// One Hs descent step of the repulsive-surface flow on the GPU (Session::step_inner,
// RS/src/step/session.rs:749-1200, without remeshing; with rs_flow_options.ccd the first trial is
// capped by continuous collision detection), behind rs_flow_* of include/rsgpu.h.
//
//   1. Barnes-Hut energy F and differential g (rs_bh_*; objective.rs:151-249)
//   2. the saddle solver of the step (rs_solver_*; direction.rs:426-484)
//   3. the Schur complement of the nonlinear rows (total area, volume) and the direction
//      x = y - Z N^-1 C_N y with Z = A'^-1 C_N^T, y = A'^-1 g: one batch of k + 1 solves
//      (SchurComplement::with_direction, RS/src/solve/schur.rs:101-347)
//   4. Armijo backtracking on the frozen-list energy F(f - tau x) <= F - c tau g.x from the
//      start rule's tau (default: the farthest vertex moves one initial mean edge length, then
//      twice the last accepted tau; StartRule, RS/src/step/options.rs:74-107), a trial kept
//      only if its projection is admissible (the projection guard, session.rs:1481-1552)
//   5. projection (project, RS/src/solve/schur.rs:499-575): the barycenter groups translated to
//      their targets, then Newton rounds f <- f - Z N^-1 Phi_N with the step's Z and N, each
//      kept only while it lowers max |Phi_r| / tol_r (NewtonSteps default: until tolerance, at
//      most 5); a stuck step projects the unmoved positions.
// Host-side vectors (positions, constraint rows) are FP64 and O(V); the rest is on the device.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <future>
#include <memory>
#include <numeric>
#include <optional>
#include <string>
#include <thread>
#include <vector>

#include "common.hpp"
#include "host_tree.hpp"
#include "krylov.hpp"

using namespace rsg;

namespace {

using clk = std::chrono::steady_clock;
double since(clk::time_point t) { return std::chrono::duration<double>(clk::now() - t).count(); }

double total_area(int nf, const uint32_t *f, const double *p) {
  double s = 0.0;
  for (int i = 0; i < nf; ++i) {
    const double *a = p + 3 * (size_t)f[3 * i], *b = p + 3 * (size_t)f[3 * i + 1], *c = p + 3 * (size_t)f[3 * i + 2];
    double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double n0 = u[1] * w[2] - u[2] * w[1], n1 = u[2] * w[0] - u[0] * w[2], n2 = u[0] * w[1] - u[1] * w[0];
    s += 0.5 * std::sqrt(n0 * n0 + n1 * n1 + n2 * n2);
  }
  return s;
}

double total_volume(int nf, const uint32_t *f, const double *p) {  // constraints/mod.rs:473-483
  double s = 0.0;
  for (int i = 0; i < nf; ++i) {
    const double *a = p + 3 * (size_t)f[3 * i], *b = p + 3 * (size_t)f[3 * i + 1], *c = p + 3 * (size_t)f[3 * i + 2];
    double x0 = b[1] * c[2] - b[2] * c[1], x1 = b[2] * c[0] - b[0] * c[2], x2 = b[0] * c[1] - b[1] * c[0];
    s += (a[0] * x0 + a[1] * x1 + a[2] * x2) / 6.0;
  }
  return s;
}

// area gradient sum_{S ni v} 1/2 N_S x e_opp(v) (constraints/mod.rs:606-623)
void area_gradient(int nv, int nf, const uint32_t *f, const double *p, double *g) {
  std::fill(g, g + 3 * (size_t)nv, 0.0);
  for (int i = 0; i < nf; ++i) {
    const uint32_t *t = f + 3 * (size_t)i;
    const double *q[3] = {p + 3 * (size_t)t[0], p + 3 * (size_t)t[1], p + 3 * (size_t)t[2]};
    double u[3], w[3], n[3];
    for (int k = 0; k < 3; ++k) u[k] = q[1][k] - q[0][k], w[k] = q[2][k] - q[0][k];
    n[0] = u[1] * w[2] - u[2] * w[1], n[1] = u[2] * w[0] - u[0] * w[2], n[2] = u[0] * w[1] - u[1] * w[0];
    double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; ++k) n[k] /= len;
    for (int c = 0; c < 3; ++c) {
      const double *a = q[(c + 1) % 3], *b = q[(c + 2) % 3];
      double e[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
      double x[3] = {n[1] * e[2] - n[2] * e[1], n[2] * e[0] - n[0] * e[2], n[0] * e[1] - n[1] * e[0]};
      for (int k = 0; k < 3; ++k) g[3 * (size_t)t[c] + k] += 0.5 * x[k];
    }
  }
}

// volume gradient 1/6 sum_{S ni v} f_j x f_k (constraints/mod.rs:627-645)
void volume_gradient(int nv, int nf, const uint32_t *f, const double *p, double *g) {
  std::fill(g, g + 3 * (size_t)nv, 0.0);
  for (int i = 0; i < nf; ++i) {
    const uint32_t *t = f + 3 * (size_t)i;
    for (int c = 0; c < 3; ++c) {
      const double *a = p + 3 * (size_t)t[(c + 1) % 3], *b = p + 3 * (size_t)t[(c + 2) % 3];
      double x[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
      for (int k = 0; k < 3; ++k) g[3 * (size_t)t[c] + k] += x[k] / 6.0;
    }
  }
}

double mean_edge_length(int nf, const uint32_t *f, const double *p) {
  std::vector<std::pair<uint32_t, uint32_t>> e;
  e.reserve(3 * (size_t)nf);
  for (int i = 0; i < nf; ++i)
    for (int c = 0; c < 3; ++c) {
      uint32_t a = f[3 * i + c], b = f[3 * i + (c + 1) % 3];
      e.push_back({std::min(a, b), std::max(a, b)});
    }
  std::sort(e.begin(), e.end());
  e.erase(std::unique(e.begin(), e.end()), e.end());
  double s = 0.0;
  for (auto [a, b] : e) {
    const double *x = p + 3 * (size_t)a, *y = p + 3 * (size_t)b;
    s += std::sqrt((x[0] - y[0]) * (x[0] - y[0]) + (x[1] - y[1]) * (x[1] - y[1]) + (x[2] - y[2]) * (x[2] - y[2]));
  }
  return s / (double)e.size();
}

template <class T>
struct Owned {
  T *p = nullptr;
  void (*del)(T *) = nullptr;
  ~Owned() {
    if (p) del(p);
  }
};

void check(int rc, const char *what) {
  if (rc != 0) fail(rc, rs_last_error_kind(), what, rs_last_error());
}

}  // namespace

struct rs_flow {
  rs_ctx *ctx = nullptr;
  int nv = 0, nf = 0;
  std::vector<uint32_t> faces;
  std::vector<double> pos;
  rs_flow_options o;
  double l0 = 0.0, last_tau = 0.0, area_t = 0.0, vol_t = 0.0;
  int groups = 1;                // barycenter groups: one global, or one per component
  std::vector<uint32_t> group;   // group of every vertex
  std::vector<double> bary0;     // target barycenter of every group (3 per group)
  std::vector<double> last_x, last_g, trials;  // the last direction, differential, trials
  std::vector<double> last_sol;  // the last step's saddle solutions: Z columns, then y (n each)
  int last_k = 0;
  int64_t last_n = 0;
  rs_learned *lmodel = nullptr;
  int l_cheap = 2, l_cap = 0;
  int iteration = 0;
  rs_ccd *ccd = nullptr;  // the surface's topology for the collision cap (ccd on)
  std::atomic<int> cancel{0};  // set by rs_flow_cancel from any thread
  ~rs_flow() { rs_ccd_free(ccd); }
};

namespace {
void group_barycenters(const rs_flow *F, const double *p, std::vector<double> &out);
}

extern "C" {

rs_flow_options rs_flow_options_default(void) {
  rs_flow_options o;
  o.alpha = 6.0;
  o.beta = 12.0;
  o.theta = 0.5;
  o.leaf_size = 8;
  o.solver = rs_solver_options_default();
  o.solver.tolerance = 1e-3;  // FLOW_GMRES (RS/src/solve/iterative.rs:341-346)
  o.solver.restart = 60;
  o.hold_area = 0;
  o.hold_volume = 0;
  o.armijo_c = 1e-2;
  o.max_halvings = 30;
  o.newton_max = 5;
  o.ccd = 0;
  o.ccd_gap = 0.05;
  o.ccd_max_iterations = 100;
  o.ccd_close_factor = 0.5;
  o.start_rule = 3;  // StartRule::GrowPrevious { factor: 2, first: MaxDisplacement { lengths: 1 } }
  o.start_value = 2.0;
  o.first_rule = 1;
  o.first_value = 1.0;
  o.tau_min_rel = 1e-12;
  o.newton_fixed = 0;
  o.newton_tolerance = 1e-8;  // NONLINEAR_TOLERANCE (RS/src/constraints/mod.rs:147)
  o.area_target = NAN;
  o.volume_target = NAN;
  o.guard_projection = 1;
  o.retry_max_iterations = 0;
  o.dense_fallback = 1;
  return o;
}

int rs_flow_create(rs_ctx *ctx, int nv, int nf, const uint32_t *faces, const double *positions_host,
                   const rs_flow_options *o, rs_flow **out) {
  *out = nullptr;
  return guard([&] {
    validate_topology(nv, nf, faces);
    validate_positions(nv, nf, faces, positions_host);
    auto F = std::make_unique<rs_flow>();
    F->ctx = ctx;
    F->nv = nv, F->nf = nf;
    F->faces.assign(faces, faces + 3 * (size_t)nf);
    F->pos.assign(positions_host, positions_host + 3 * (size_t)nv);
    F->o = o ? *o : rs_flow_options_default();
    const rs_flow_options &o = F->o;
    if (!(o.start_rule >= 0 && o.start_rule <= 3 && o.first_rule >= 0 && o.first_rule <= 2))
      fail(RS_INVALID_OPTION, "InvalidOption", "flow", "start_rule in 0..3, first_rule in 0..2");
    if (!(o.start_value > 0.0 && std::isfinite(o.start_value)) ||
        (o.start_rule == 3 && !(o.first_rule == 2 || (o.first_value > 0.0 && std::isfinite(o.first_value)))))
      fail(RS_INVALID_OPTION, "InvalidOption", "flow", "start values must be finite and positive");
    if (!(o.tau_min_rel > 0.0 && std::isfinite(o.tau_min_rel)) || !(o.newton_tolerance > 0.0) || o.newton_max < 0)
      fail(RS_INVALID_OPTION, "InvalidOption", "flow", "tau_min_rel, newton_tolerance > 0, newton_max >= 0");
    F->l0 = mean_edge_length(nf, faces, positions_host);
    F->area_t = std::isnan(o.area_target) ? total_area(nf, faces, positions_host) : o.area_target;
    F->vol_t = std::isnan(o.volume_target) ? total_volume(nf, faces, positions_host) : o.volume_target;
    // barycenter groups numbered as the solver's positional rows: one global group, or one per
    // component, components numbered by their lowest face (RS/src/surface.rs:349-402)
    F->group.assign(nv, 0u);
    if (o.solver.barycenter_per_component) {
      std::vector<uint32_t> par(nv);
      std::iota(par.begin(), par.end(), 0u);
      auto find = [&](uint32_t v) {
        while (par[v] != v) v = par[v] = par[par[v]];
        return v;
      };
      for (int i = 0; i < nf; ++i)
        for (int c = 1; c < 3; ++c) {
          uint32_t a = find(faces[3 * i]), b = find(faces[3 * i + c]);
          if (a != b) par[std::max(a, b)] = std::min(a, b);
        }
      std::vector<int64_t> id(nv, -1);
      int nc = 0;
      for (int i = 0; i < nf; ++i)
        if (id[find(faces[3 * i])] < 0) id[find(faces[3 * i])] = nc++;
      for (int v = 0; v < nv; ++v) F->group[v] = (uint32_t)id[find(v)];
      F->groups = nc;
    }
    F->bary0.assign(3 * (size_t)F->groups, 0.0);
    std::vector<double> b;
    group_barycenters(F.get(), positions_host, b);
    for (int g = 0; g < F->groups; ++g)
      for (int kk = 0; kk < 3; ++kk) F->bary0[3 * (size_t)g + kk] = b[4 * (size_t)g + kk];
    if (F->o.ccd) check(rs_ccd_create(ctx, nv, nf, faces, &F->ccd), "flow (ccd)");
    ctx_retain(ctx);
    *out = F.release();
  });
}

void rs_flow_free(rs_flow *F) {
  if (!F) return;
  rs_ctx *ctx = F->ctx;
  delete F;
  ctx_release(ctx);
}

int rs_flow_set_learned(rs_flow *F, rs_learned *model, int cheap_steps, int max_iterations) {
  return guard([&] {
    if (model && (cheap_steps < 1 || max_iterations < 0))
      fail(RS_INVALID_OPTION, "InvalidOption", "flow", "cheap_steps >= 1, max_iterations >= 0");
    F->lmodel = model, F->l_cheap = cheap_steps, F->l_cap = max_iterations;
  });
}

int rs_flow_cancel(rs_flow *F, int cancel) {
  return guard([&] { F->cancel.store(cancel ? 1 : 0); });
}

int rs_flow_positions(rs_flow *F, double *positions_host) {
  return guard([&] { std::memcpy(positions_host, F->pos.data(), F->pos.size() * sizeof(double)); });
}

}  // extern "C"

namespace {

// The Schur complement of the held rows (SchurComplement::factor / solve_n, RS/src/solve/schur.rs:
// 190-292): N = C_N Z symmetrized, equilibrated to unit diagonal, Cholesky with diagonal pivoting
// (largest remaining pivot first, ties by row order); a row whose pivot is at or below 1e-10 is
// dropped for the step.
struct SchurN {
  int k = 0;
  std::vector<double> d, l;
  std::vector<int> kept;
  void factor(const std::vector<double> &N, int k_) {
    k = k_;
    auto nn = [&](int i, int j) { return 0.5 * (N[(size_t)i * k + j] + N[(size_t)j * k + i]); };
    d.assign(k, 0.0);
    for (int i = 0; i < k; ++i) {
      double nii = nn(i, i);
      d[i] = nii > 0.0 && std::isfinite(nii) ? 1.0 / std::sqrt(nii) : 0.0;
    }
    std::vector<double> w((size_t)k * k);
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < k; ++j) w[(size_t)i * k + j] = nn(i, j) * d[i] * d[j];
    std::vector<int> rem;
    for (int i = 0; i < k; ++i)
      if (d[i] > 0.0) rem.push_back(i);
    std::vector<std::vector<double>> cols;
    kept.clear();
    while (!rem.empty()) {
      size_t pos = 0;
      for (size_t a = 1; a < rem.size(); ++a)
        if (!(w[(size_t)rem[pos] * k + rem[pos]] >= w[(size_t)rem[a] * k + rem[a]])) pos = a;
      const int p = rem[pos];
      const double piv = w[(size_t)p * k + p];
      if (!(piv > 1e-10)) break;
      rem.erase(rem.begin() + pos);
      const double sq = std::sqrt(piv);
      std::vector<double> col(k, 0.0);
      col[p] = sq;
      for (int i : rem) col[i] = w[(size_t)i * k + p] / sq;
      for (int i : rem)
        for (int j : rem) w[(size_t)i * k + j] -= col[i] * col[j];
      kept.push_back(p);
      cols.push_back(col);
    }
    const int m = (int)kept.size();
    l.assign((size_t)m * m, 0.0);
    for (int b = 0; b < m; ++b)
      for (int a = 0; a < m; ++a) l[(size_t)a * m + b] = cols[b][kept[a]];
  }
  std::vector<double> solve(const std::vector<double> &v) const {
    const int m = (int)kept.size();
    std::vector<double> y(m);
    for (int a = 0; a < m; ++a) y[a] = d[kept[a]] * v[kept[a]];
    for (int a = 0; a < m; ++a) {
      double t = y[a];
      for (int b = 0; b < a; ++b) t -= l[(size_t)a * m + b] * y[b];
      y[a] = t / l[(size_t)a * m + a];
    }
    for (int a = m - 1; a >= 0; --a) {
      double t = y[a];
      for (int b = a + 1; b < m; ++b) t -= l[(size_t)b * m + a] * y[b];
      y[a] = t / l[(size_t)a * m + a];
    }
    std::vector<double> out(k, 0.0);
    for (int a = 0; a < m; ++a) out[kept[a]] = d[kept[a]] * y[a];
    return out;
  }
};

// Barycenter of every group (global: one group) with the vertex areas of p.
void group_barycenters(const rs_flow *F, const double *p, std::vector<double> &out) {
  std::vector<double> va(F->nv, 0.0);
  for (int i = 0; i < F->nf; ++i) {
    const uint32_t *t = F->faces.data() + 3 * (size_t)i;
    const double *a = p + 3 * (size_t)t[0], *b = p + 3 * (size_t)t[1], *c = p + 3 * (size_t)t[2];
    double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double n0 = u[1] * w[2] - u[2] * w[1], n1 = u[2] * w[0] - u[0] * w[2], n2 = u[0] * w[1] - u[1] * w[0];
    double ar = 0.5 * std::sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    for (int k = 0; k < 3; ++k) va[t[k]] += ar / 3.0;
  }
  out.assign(4 * (size_t)F->groups, 0.0);
  for (int v = 0; v < F->nv; ++v) {
    double *o = &out[4 * (size_t)F->group[v]];
    for (int k = 0; k < 3; ++k) o[k] += va[v] * p[3 * (size_t)v + k];
    o[3] += va[v];
  }
  for (int g = 0; g < F->groups; ++g)
    for (int k = 0; k < 3; ++k) out[4 * (size_t)g + k] /= out[4 * (size_t)g + 3];
}

// The positional projection: every barycenter group translated to its target
// (ConstraintSet::project_positional without pins, RS/src/constraints/mod.rs:657-740).
void project_positional(const rs_flow *F, std::vector<double> &p) {
  std::vector<double> b;
  group_barycenters(F, p.data(), b);
  for (int v = 0; v < F->nv; ++v) {
    const int g = (int)F->group[v];
    for (int k = 0; k < 3; ++k) p[3 * (size_t)v + k] -= b[4 * (size_t)g + k] - F->bary0[3 * (size_t)g + k];
  }
}

}  // namespace

namespace {

// One step, or (direction_only) its energy, differential and direction at the current positions.
void flow_step(rs_flow *F, double *report, bool direction_only) {
  TrustedTopology trusted;  // validated by rs_flow_create; the face list never changes
  if (F->cancel.load()) fail(RS_CANCELLED, "Cancelled", "flow", "the step was cancelled");
  auto t_step = clk::now();
  rs_ctx *ctx = F->ctx;
  ctx->use();
  cudaStream_t s = ctx->stream;
  const int nv = F->nv, nf = F->nf;
  const uint32_t *faces = F->faces.data();
  const size_t nd = 3 * (size_t)nv;
  const rs_flow_options &o = F->o;
  double rep[RS_FLOW_REPORT_LEN] = {0};
  F->trials.clear();
  // 1. trees: the BH tree and lists here, the solver's set-up (mostly host work: block trees,
  // far coefficients, multigrid hierarchy) on a second host thread at the same time; both
  // enqueue on the context's stream, on disjoint buffers
  auto t = clk::now();
  Owned<rs_bh> bh;
  bh.del = rs_bh_free;
  Owned<rs_solver> sv;
  sv.del = rs_solver_free;
  Owned<rs_lgraph> lg;
  lg.del = rs_lgraph_free;
  int w_code = 0;
  std::string w_kind, w_op, w_msg;
  double t_solver = 0.0;
  // one face BVH for the Barnes-Hut lists and the metric's block cluster tree (when both ask
  // for the same leaf size), built here while the solver's other parts (vertex tree,
  // Laplacian, multigrid) start on the worker; the metric's build waits for it
  FaceGeom g_sh;
  Tree t_sh;
  const bool share = o.leaf_size == o.solver.leaf_size;
  std::promise<void> tree_ready;
  std::shared_future<void> tree_fut = tree_ready.get_future().share();
  std::thread worker([&] {
    TrustedTopology trusted_here;
    std::optional<SharedFaceTree> sh;
    if (share) sh.emplace(g_sh, t_sh, faces, F->pos.data(), nf, o.leaf_size, &tree_fut);
    auto t0 = clk::now();
    int c = rs_solver_build(ctx, nv, nf, faces, F->pos.data(), o.alpha, o.beta, &o.solver, &sv.p);
    if (c == 0 && F->lmodel) {
      c = rs_lgraph_create(ctx, nv, nf, faces, F->pos.data(), &lg.p);
      if (c == 0) c = rs_solver_set_learned(sv.p, F->lmodel, lg.p, F->l_cheap, F->l_cap);
    }
    if (c != 0) w_code = c, w_kind = rs_last_error_kind(), w_op = rs_last_error_operation(), w_msg = rs_last_error();
    t_solver = since(t0);
  });
  int b_code = 0;
  try {
    if (share) {
      g_sh = face_geometry(nf, faces, F->pos.data());
      t_sh = build_face_tree(nf, faces, F->pos.data(), g_sh, o.leaf_size);
    }
    tree_ready.set_value();
  } catch (...) {
    tree_ready.set_exception(std::current_exception());
    worker.join();
    throw;
  }
  {
    std::optional<SharedFaceTree> sh_main;
    if (share) sh_main.emplace(g_sh, t_sh, faces, F->pos.data(), nf, o.leaf_size, nullptr);
    b_code = rs_bh_build(ctx, nv, nf, faces, F->pos.data(), o.theta, o.leaf_size, &bh.p);
  }
  rep[9] = since(t);
  worker.join();
  check(b_code, "flow (tree)");
  if (w_code != 0) fail(w_code, w_kind.c_str(), w_op.c_str(), w_msg);
  rep[11] = t_solver;
  int64_t ndof = 0, nq = 0;
  check(rs_solver_dims(sv.p, &ndof, &nq), "flow");
  const size_t n = nd + (size_t)nq;
  // the held rows: total area (kind 0), volume (kind 1), with their targets
  std::vector<int> rows;
  if (o.hold_area) rows.push_back(0);
  if (o.hold_volume) rows.push_back(1);
  const int k = (int)rows.size();
  const int nb = k + 1;
  auto row_value = [&](int r, const double *p) { return r == 0 ? total_area(nf, faces, p) : total_volume(nf, faces, p); };
  auto row_target = [&](int r) { return r == 0 ? F->area_t : F->vol_t; };
  // ConstraintSet::tolerance (constraints/mod.rs:435-442)
  auto row_tol = [&](int r) {
    double tg = std::fabs(row_target(r));
    return tg > 0.0 ? o.newton_tolerance * tg : o.newton_tolerance;
  };
  DevBuf<double> rhs((size_t)nb * n), sol((size_t)nb * n), e_dev(1);
  RSG_CUDA("flow", cudaMemsetAsync(rhs.p, 0, (size_t)nb * n * sizeof(double), s));
  t = clk::now();
  check(rs_bh_energy_and_differential_device(bh.p, o.alpha, o.beta, e_dev.p, rhs.p + (size_t)k * n), "flow (energy)");
  double E0 = 0.0;
  e_dev.download(&E0, 1, s);
  std::vector<double> g(nd);
  RSG_CUDA("flow", rsg::copy_async(g.data(), rhs.p + (size_t)k * n, nd * sizeof(double), cudaMemcpyDeviceToHost, s));
  RSG_CUDA("flow", cudaStreamSynchronize(s));
  rep[10] = since(t);
  if (!std::isfinite(E0)) fail(RS_NONFINITE_ENERGY, "NonFiniteEnergy", "flow", "non-finite energy");
  double gsq = 0.0;
  for (double x : g) {
    if (!std::isfinite(x)) fail(RS_NONFINITE_ENERGY, "NonFiniteEnergy", "flow", "non-finite differential");
    gsq += x * x;
  }
  rep[21] = std::sqrt(gsq);
  // C_N rows
  std::vector<std::vector<double>> cn(k, std::vector<double>(nd));
  for (int i = 0; i < k; ++i) {
    if (rows[i] == 0) area_gradient(nv, nf, faces, F->pos.data(), cn[i].data());
    else volume_gradient(nv, nf, faces, F->pos.data(), cn[i].data());
    RSG_CUDA("flow", rsg::copy_async(rhs.p + (size_t)i * n, cn[i].data(), nd * sizeof(double), cudaMemcpyHostToDevice, s));
  }
  // 3. one batch: Z columns and y
  t = clk::now();
  double srep[20] = {0};
  int code = rs_solver_solve_many_device(sv.p, nb, rhs.p, sol.p, srep);
  if (code == RS_SOLVER_DIVERGED) {
    // the crate's recovery (RobustHierarchical::escalate, direction.rs:269-379): repeat the
    // solves with restart 60 and at least four times the iteration cap (800 or more), then by
    // the dense LU of the exact metric for at most 6000 vertices
    const rs_solver_options &so = o.solver;
    const int it = o.retry_max_iterations > 0 ? o.retry_max_iterations : std::max(4 * so.max_iterations, 800);
    check(rs_solver_set_gmres(sv.p, 60, it, so.tolerance), "flow (solve)");
    rep[18] += 1.0;
    code = rs_solver_solve_many_device(sv.p, nb, rhs.p, sol.p, srep);
    if (code == RS_SOLVER_DIVERGED && o.dense_fallback && nv <= RS_DENSE_FALLBACK_MAX_VERTICES) {
      rep[18] += 1.0;
      code = rs_solver_dense_solve_many_device(sv.p, nb, rhs.p, sol.p, srep);
    }
  }
  check(code, "flow (solve)");
  rep[12] = since(t);
  std::vector<double> hs((size_t)nb * n);
  sol.download(hs.data(), hs.size(), s);
  RSG_CUDA("flow", cudaStreamSynchronize(s));
  // GMRES iterations per right-hand side: the held rows (area, volume), then the direction
  double worst = 0.0;
  for (int q = 0; q < nb; ++q) worst = std::max(worst, srep[5 * q + 1]);
  for (int i = 0; i < k; ++i) rep[4 + rows[i]] = srep[5 * i];
  rep[6] = srep[5 * k];
  rep[7] = worst;
  const double *y = hs.data() + (size_t)k * n;
  // N = C_N Z (k x k) and the direction x = y - Z N^-1 C_N y (schur.rs:320-344)
  std::vector<double> N((size_t)k * k), cy(k), x(nd);
  for (int i = 0; i < k; ++i) {
    for (int j = 0; j < k; ++j) {
      double sum = 0.0;
      const double *z = hs.data() + (size_t)j * n;
      for (size_t r = 0; r < nd; ++r) sum += cn[i][r] * z[r];
      N[(size_t)i * k + j] = sum;
    }
    double sum = 0.0;
    for (size_t r = 0; r < nd; ++r) sum += cn[i][r] * y[r];
    cy[i] = sum;
  }
  SchurN schur;
  schur.factor(N, k);
  std::vector<double> c = schur.solve(cy);
  double slope = 0.0, xinf = 0.0, xsq = 0.0, maxdisp = 0.0;
  for (size_t r = 0; r < nd; ++r) {
    double v = y[r];
    for (int j = 0; j < k; ++j) v -= hs[(size_t)j * n + r] * c[j];
    x[r] = v;
    slope += g[r] * v;
    xsq += v * v;
    xinf = std::max(xinf, std::fabs(v));
  }
  for (int v = 0; v < nv; ++v)
    maxdisp = std::max(maxdisp, std::sqrt(x[3 * v] * x[3 * v] + x[3 * v + 1] * x[3 * v + 1] + x[3 * v + 2] * x[3 * v + 2]));
  const double xnorm = std::sqrt(xsq);
  rep[16] = slope;
  rep[23] = xinf;
  rep[0] = E0;
  F->last_x = x, F->last_g = g;
  F->last_sol = hs, F->last_k = k, F->last_n = (int64_t)n;
  if (direction_only) {
    rep[1] = E0, rep[26] = E0;
    rep[8] = since(t_step);
    if (report) std::memcpy(report, rep, sizeof(rep));
    return;
  }
  // 4. Armijo backtracking on the frozen lists; start_tau (session.rs:1604-1615)
  t = clk::now();
  auto start = [&](int rule, double val) {
    return rule == 0 ? val : rule == 1 ? val * F->l0 / maxdisp : 2.0 / xnorm;
  };
  double tau = o.start_rule == 3 ? (F->last_tau > 0.0 ? o.start_value * F->last_tau : start(o.first_rule, o.first_value))
                                 : start(o.start_rule, o.start_value);
  // the collision cap (session.rs:927-955): the largest safe time of x - t d, two thirds of it
  rep[27] = NAN;
  if (F->ccd && std::isfinite(tau) && tau > 0.0) {
    auto tc = clk::now();
    std::vector<double> vel(nd);
    for (size_t r = 0; r < nd; ++r) vel[r] = -x[r];
    rs_ccd_options co = rs_ccd_options_default();
    co.gap = o.ccd_gap, co.reference_length = F->l0;
    co.max_iterations = o.ccd_max_iterations, co.close_factor = o.ccd_close_factor;
    double tmax = 0.0;
    int64_t cr[7] = {0, 0, 0, 0, 0, 0, 0}, band_pairs = 0, band_vertices = 0;
    // the faces that intersect at the start of the step exempt their neighbourhood
    // (IntersectionBand, session.rs:917-928); empty for an embedded mesh
    check(rs_ccd_set_band(F->ccd, F->pos.data(), &band_pairs, &band_vertices), "flow (ccd)");
    check(rs_ccd_first_contact(F->ccd, F->pos.data(), vel.data(), tau, &co, &tmax, cr), "flow (ccd)");
    if (cr[0]) tau = std::min(tau, 2.0 / 3.0 * tmax);
    rep[27] = tmax;
    rep[28] = since(tc);
  }
  rep[22] = tau;
  const double tau_min = o.tau_min_rel * F->l0 / xinf;
  // the projection (project, RS/src/solve/schur.rs:499-575): barycenters exactly, then Newton
  // rounds f <- f - Z N^-1 Phi_N with the step's Z and N, each followed by the positional
  // projection and kept only while it lowers max |Phi_r| / tol_r over the kept rows
  auto phis = [&](const double *p) {
    std::vector<double> ph(k);
    for (int i = 0; i < k; ++i) ph[i] = row_value(rows[i], p) - row_target(rows[i]);
    return ph;
  };
  auto measure = [&](const std::vector<double> &ph, bool all_rows) {
    double m = 0.0;
    for (int i = 0; i < k; ++i) {
      if (!all_rows && std::find(schur.kept.begin(), schur.kept.end(), i) == schur.kept.end()) continue;
      double v = std::fabs(ph[i]) / row_tol(rows[i]);
      m = (std::isnan(v) || std::isnan(m)) ? NAN : std::max(m, v);
    }
    return m;
  };
  struct Proj {
    std::vector<double> p;
    int rounds = 0, status = 0;  // 0 converged, 1 max rounds, 2 not improving, 3 blocked
  };
  auto project = [&](const std::vector<double> &moved) {
    Proj pr;
    pr.p = moved;
    project_positional(F, pr.p);
    std::vector<double> ph = phis(pr.p.data());
    double m = measure(ph, false);
    bool stopped = false;
    const bool until = !o.newton_fixed;
    while (pr.rounds < o.newton_max && !schur.kept.empty()) {
      if (until && m <= 1.0) break;
      std::vector<double> cc = schur.solve(ph);
      std::vector<double> trial = pr.p;
      for (size_t r = 0; r < nd; ++r) {
        double h = 0.0;
        for (int j = 0; j < k; ++j) h += hs[(size_t)j * n + r] * cc[j];
        trial[r] -= h;
      }
      project_positional(F, trial);
      std::vector<double> pt = phis(trial.data());
      double mt = measure(pt, false);
      if (!(mt < m)) {
        stopped = true;
        break;
      }
      pr.p.swap(trial), ph = pt, m = mt;
      ++pr.rounds;
    }
    pr.status = (m <= 1.0 || schur.kept.empty()) ? 0 : stopped ? 2 : 1;
    return pr;
  };
  auto energy_at = [&](const std::vector<double> &p) {
    for (double v : p)
      if (!std::isfinite(v)) return (double)NAN;
    double e = NAN;
    if (rs_bh_refit(bh.p, p.data()) != RS_OK || rs_bh_energy(bh.p, o.alpha, o.beta, &e) != RS_OK) return (double)NAN;
    return e;
  };
  // the projection guard (session.rs:1481-1552, without collision detection): the projection
  // must give a finite F and leave the held rows no further from their targets than the start
  const double base_measure = measure(phis(F->pos.data()), true);
  auto admissible = [&](const Proj &pr, double e_after) {
    return std::isfinite(e_after) && (!o.guard_projection || measure(phis(pr.p.data()), true) <= std::max(base_measure, 1.0));
  };
  // half the projection's motion, halved while F is not finite (limit, session.rs:1554-1602)
  auto limit = [&](const std::vector<double> &moved, Proj &pr, double &e_after) {
    double frac = 0.5;
    std::vector<double> target = pr.p, q(nd);
    bool chosen = false;
    for (int it = 0; it < 12 && frac > 0.0; ++it) {
      for (size_t r = 0; r < nd; ++r) q[r] = moved[r] + frac * (target[r] - moved[r]);
      double e = energy_at(q);
      if (std::isfinite(e)) {
        pr.p = q, e_after = e, chosen = true;
        break;
      }
      frac *= 0.5;
    }
    if (!chosen) pr.p = moved, e_after = energy_at(moved);
    pr.status = 3;
  };
  std::vector<double> trial(nd);
  double E_trial = E0, E_after = NAN;
  bool accepted = false;
  int halvings = 0, blocked = 0, base_contact = -1;
  Proj proj;
  double t_proj = 0.0;
  if (slope > 0.0 && std::isfinite(tau) && tau > 0.0) {
    for (;;) {
      if (!(tau >= tau_min) || (o.max_halvings >= 0 && halvings > o.max_halvings)) break;
      if (F->cancel.load()) fail(RS_CANCELLED, "Cancelled", "flow", "the step was cancelled");
      for (size_t r = 0; r < nd; ++r) trial[r] = F->pos[r] - tau * x[r];
      const double Et = energy_at(trial);
      const bool ok = std::isfinite(Et) && Et <= E0 - o.armijo_c * tau * slope;
      double outcome = !std::isfinite(Et) ? 2.0 : ok ? 0.0 : 1.0;
      if (ok) {
        auto tp = clk::now();
        Proj pr = project(trial);
        double ea = energy_at(pr.p);
        if (admissible(pr, ea) || !o.guard_projection) {
          t_proj += since(tp);
          F->trials.insert(F->trials.end(), {tau, Et, 0.0});
          accepted = true, proj = pr, E_trial = Et, E_after = ea;
          break;
        }
        ++blocked;
        if (!std::isfinite(ea)) {
          if (base_contact < 0) {
            Proj pb = project(F->pos);
            double eb = energy_at(pb.p);
            base_contact = (!admissible(pb, eb) && !std::isfinite(eb)) ? 1 : 0;
          }
          if (base_contact == 1) {
            limit(trial, pr, ea);
            t_proj += since(tp);
            F->trials.insert(F->trials.end(), {tau, Et, 0.0});
            accepted = true, proj = pr, E_trial = Et, E_after = ea;
            break;
          }
        }
        t_proj += since(tp);
        outcome = 3.0;
      }
      F->trials.insert(F->trials.end(), {tau, std::isfinite(Et) ? Et : NAN, outcome});
      tau *= 0.5;
      ++halvings;
    }
  }
  rep[13] = since(t) - t_proj;
  // 5. the projection of a stuck step: the unmoved positions (session.rs:1073-1090)
  t = clk::now();
  if (!accepted) {
    proj = project(F->pos);
    E_after = energy_at(proj.p);
    if (!admissible(proj, E_after) && o.guard_projection) {
      ++blocked;
      limit(F->pos, proj, E_after);
    }
  }
  if (!std::isfinite(E_after)) fail(RS_NONFINITE_ENERGY, "NonFiniteEnergy", "flow", "non-finite energy after the projection");
  double cres = 0.0;
  for (int i = 0; i < k; ++i) {
    double val = row_value(rows[i], proj.p.data()), tgt = row_target(rows[i]);
    cres = std::max(cres, std::fabs(val - tgt) / std::max(1.0, std::fabs(tgt)));
  }
  F->pos = proj.p;
  if (accepted) F->last_tau = tau;
  F->iteration++;
  rep[14] = since(t) + t_proj;
  if (F->lmodel) {
    int64_t ls = 0, lf = 0;
    check(rs_solver_learned_counts(sv.p, &ls, &lf), "flow");
    rep[19] = (double)ls, rep[20] = (double)lf;
  }
  rep[1] = E_after;
  rep[2] = accepted ? tau : 0.0;
  rep[3] = halvings;
  rep[15] = accepted ? 1.0 : 0.0;
  rep[17] = cres;
  rep[24] = proj.rounds;
  rep[25] = proj.status;
  rep[26] = E_trial;
  rep[29] = blocked;
  rep[8] = since(t_step);
  if (report) std::memcpy(report, rep, sizeof(rep));
}

}  // namespace

extern "C" {

int rs_flow_step(rs_flow *F, double *report) {
  return guard([&] { flow_step(F, report, false); });
}

int rs_flow_direction(rs_flow *F, double *report) {
  return guard([&] { flow_step(F, report, true); });
}

int rs_flow_last_direction(rs_flow *F, double *x_host, double *g_host) {
  return guard([&] {
    if (F->last_x.empty()) fail(RS_INVALID_OPTION, "InvalidOption", "flow", "no step or direction computed yet");
    if (x_host) std::memcpy(x_host, F->last_x.data(), F->last_x.size() * sizeof(double));
    if (g_host) std::memcpy(g_host, F->last_g.data(), F->last_g.size() * sizeof(double));
  });
}

int rs_flow_last_solutions(rs_flow *F, double *sol_host, int *n_held, int64_t *n) {
  return guard([&] {
    if (F->last_sol.empty()) fail(RS_INVALID_OPTION, "InvalidOption", "flow", "no step or direction computed yet");
    if (n_held) *n_held = F->last_k;
    if (n) *n = F->last_n;
    if (sol_host) std::memcpy(sol_host, F->last_sol.data(), F->last_sol.size() * sizeof(double));
  });
}

int rs_flow_last_trials(rs_flow *F, double *out3, int max_trials, int *n_trials) {
  return guard([&] {
    const int nt = (int)(F->trials.size() / 3);
    if (n_trials) *n_trials = nt;
    if (out3) std::memcpy(out3, F->trials.data(), 3 * (size_t)std::min(nt, max_trials) * sizeof(double));
  });
}

}  // extern "C"
