// One Hs descent step of the repulsive-surface flow on the GPU (Session::step_inner,
// RS/src/step/session.rs:749-1200, without remeshing and collision detection), behind rs_flow_*
// of include/rsgpu.h.
//
//   1. Barnes-Hut energy F and differential g (rs_bh_*; objective.rs:151-249)
//   2. the saddle solver of the step (rs_solver_*; direction.rs:426-484)
//   3. the Schur complement of the nonlinear rows (total area, volume) and the direction
//      x = y - Z N^-1 C_N y with Z = A'^-1 C_N^T, y = A'^-1 g: one batch of k + 1 solves
//      (SchurComplement::with_direction, RS/src/solve/schur.rs:101-347)
//   4. Armijo backtracking on the frozen-list energy F(f - tau x) <= F - c tau g.x, first
//      tau moving the farthest vertex by one initial mean edge length, then twice the last
//      accepted tau (StartRule default, RS/src/step/options.rs:74-83)
//   5. projection: Newton rounds f <- f - Z N^-1 Phi_N with the step's Z and N
//      (SchurComplement::correction, schur.rs:350-356; NewtonSteps default: until tolerance,
//      at most 5), then the barycenter translated back to its target.
// Host-side vectors (positions, constraint rows) are FP64 and O(V); the rest is on the device.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <future>
#include <memory>
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

void barycenter(int nv, int nf, const uint32_t *f, const double *p, double out[3]) {
  std::vector<double> va(nv, 0.0);
  for (int i = 0; i < nf; ++i) {
    const double *a = p + 3 * (size_t)f[3 * i], *b = p + 3 * (size_t)f[3 * i + 1], *c = p + 3 * (size_t)f[3 * i + 2];
    double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double n0 = u[1] * w[2] - u[2] * w[1], n1 = u[2] * w[0] - u[0] * w[2], n2 = u[0] * w[1] - u[1] * w[0];
    double ar = 0.5 * std::sqrt(n0 * n0 + n1 * n1 + n2 * n2) / 3.0;
    for (int c2 = 0; c2 < 3; ++c2) va[f[3 * i + c2]] += ar;
  }
  double s[3] = {0, 0, 0}, tot = 0.0;
  for (int v = 0; v < nv; ++v) {
    for (int k = 0; k < 3; ++k) s[k] += va[v] * p[3 * (size_t)v + k];
    tot += va[v];
  }
  for (int k = 0; k < 3; ++k) out[k] = s[k] / tot;
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
  double l0 = 0.0, last_tau = 0.0, area0 = 0.0, vol0 = 0.0, bary0[3] = {0, 0, 0};
  rs_learned *lmodel = nullptr;
  int l_cheap = 2, l_cap = 0;
  int iteration = 0;
  rs_ccd *ccd = nullptr;  // the surface's topology for the collision cap (ccd on)
  std::atomic<int> cancel{0};  // set by rs_flow_cancel from any thread
  ~rs_flow() { rs_ccd_free(ccd); }
};

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
    F->l0 = mean_edge_length(nf, faces, positions_host);
    F->area0 = total_area(nf, faces, positions_host);
    F->vol0 = total_volume(nf, faces, positions_host);
    barycenter(nv, nf, faces, positions_host, F->bary0);
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

int rs_flow_step(rs_flow *F, double *report) {
  return guard([&] {
    TrustedTopology trusted;  // validated by rs_flow_create; the face list never changes
    if (F->cancel.load()) fail(RS_CANCELLED, "Cancelled", "flow", "the step was cancelled");
    auto t_step = clk::now();
    rs_ctx *ctx = F->ctx;
    ctx->use();
    cudaStream_t s = ctx->stream;
    const int nv = F->nv, nf = F->nf;
    const uint32_t *faces = F->faces.data();
    const size_t nd = 3 * (size_t)nv;
    double rep[RS_FLOW_REPORT_LEN] = {0};
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
    const bool share = F->o.leaf_size == F->o.solver.leaf_size;
    std::promise<void> tree_ready;
    std::shared_future<void> tree_fut = tree_ready.get_future().share();
    std::thread worker([&] {
      TrustedTopology trusted_here;
      std::optional<SharedFaceTree> sh;
      if (share) sh.emplace(g_sh, t_sh, faces, F->pos.data(), nf, F->o.leaf_size, &tree_fut);
      auto t0 = clk::now();
      int c = rs_solver_build(ctx, nv, nf, faces, F->pos.data(), F->o.alpha, F->o.beta, &F->o.solver, &sv.p);
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
        t_sh = build_face_tree(nf, faces, F->pos.data(), g_sh, F->o.leaf_size);
      }
      tree_ready.set_value();
    } catch (...) {
      tree_ready.set_exception(std::current_exception());
      worker.join();
      throw;
    }
    {
      std::optional<SharedFaceTree> sh_main;
      if (share) sh_main.emplace(g_sh, t_sh, faces, F->pos.data(), nf, F->o.leaf_size, nullptr);
      b_code = rs_bh_build(ctx, nv, nf, faces, F->pos.data(), F->o.theta, F->o.leaf_size, &bh.p);
    }
    rep[9] = since(t);
    worker.join();
    check(b_code, "flow (tree)");
    if (w_code != 0) fail(w_code, w_kind.c_str(), w_op.c_str(), w_msg);
    rep[11] = t_solver;
    int64_t ndof = 0, nq = 0;
    check(rs_solver_dims(sv.p, &ndof, &nq), "flow");
    const size_t n = nd + (size_t)nq;
    // nonlinear rows
    std::vector<int> rows;
    if (F->o.hold_area) rows.push_back(0);
    if (F->o.hold_volume) rows.push_back(1);
    const int k = (int)rows.size();
    const int nb = k + 1;
    DevBuf<double> rhs((size_t)nb * n), sol((size_t)nb * n), e_dev(1);
    RSG_CUDA("flow", cudaMemsetAsync(rhs.p, 0, (size_t)nb * n * sizeof(double), s));
    t = clk::now();
    check(rs_bh_energy_and_differential_device(bh.p, F->o.alpha, F->o.beta, e_dev.p, rhs.p + (size_t)k * n),
          "flow (energy)");
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
      // solves with restart 60 and at least four times the iteration cap (800 or more)
      const rs_solver_options &so = F->o.solver;
      check(rs_solver_set_gmres(sv.p, 60, std::max(4 * so.max_iterations, 800), so.tolerance),
            "flow (solve)");
      rep[18] += 1.0;
      code = rs_solver_solve_many_device(sv.p, nb, rhs.p, sol.p, srep);
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
    // N = C_N Z (k x k), equilibrated, pivoted Cholesky with drop (schur.rs:230-289)
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
    std::vector<double> Ns = N;  // symmetrized
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < k; ++j) Ns[(size_t)i * k + j] = 0.5 * (N[(size_t)i * k + j] + N[(size_t)j * k + i]);
    auto solve_n = [&](const std::vector<double> &rhs_) {
      // equilibrated Cholesky of the kept rows (drop pivots <= 1e-10)
      std::vector<double> d(k), L((size_t)k * k, 0.0), sol_(k, 0.0);
      std::vector<int> kept;
      for (int i = 0; i < k; ++i) d[i] = Ns[(size_t)i * k + i] > 0 ? 1.0 / std::sqrt(Ns[(size_t)i * k + i]) : 0.0;
      for (int i = 0; i < k; ++i) {
        double piv = Ns[(size_t)i * k + i] * d[i] * d[i];
        for (size_t a = 0; a < kept.size(); ++a) piv -= L[(size_t)i * k + kept[a]] * L[(size_t)i * k + kept[a]];
        if (!(piv > 1e-10)) continue;
        double l = std::sqrt(piv);
        L[(size_t)i * k + i] = l;
        for (int j = i + 1; j < k; ++j) {
          double v = Ns[(size_t)j * k + i] * d[i] * d[j];
          for (size_t a = 0; a < kept.size(); ++a) v -= L[(size_t)j * k + kept[a]] * L[(size_t)i * k + kept[a]];
          L[(size_t)j * k + i] = v / l;
        }
        kept.push_back(i);
      }
      std::vector<double> w(k, 0.0);
      for (int i : kept) {
        double v = rhs_[i] * d[i];
        for (int j : kept)
          if (j < i) v -= L[(size_t)i * k + j] * w[j];
        w[i] = v / L[(size_t)i * k + i];
      }
      for (auto it = kept.rbegin(); it != kept.rend(); ++it) {
        int i = *it;
        double v = w[i];
        for (int j : kept)
          if (j > i) v -= L[(size_t)j * k + i] * sol_[j];
        sol_[i] = v / L[(size_t)i * k + i];
      }
      for (int i = 0; i < k; ++i) sol_[i] *= d[i];
      return sol_;
    };
    std::vector<double> c = solve_n(cy);
    double slope = 0.0, xinf = 0.0, maxdisp = 0.0;
    for (size_t r = 0; r < nd; ++r) {
      double v = y[r];
      for (int j = 0; j < k; ++j) v -= hs[(size_t)j * n + r] * c[j];
      x[r] = v;
      slope += g[r] * v;
      xinf = std::max(xinf, std::fabs(v));
    }
    for (int v = 0; v < nv; ++v)
      maxdisp = std::max(maxdisp, std::sqrt(x[3 * v] * x[3 * v] + x[3 * v + 1] * x[3 * v + 1] + x[3 * v + 2] * x[3 * v + 2]));
    rep[16] = slope;
    // 4. Armijo backtracking on the frozen lists
    t = clk::now();
    double tau = F->last_tau > 0.0 ? 2.0 * F->last_tau : F->l0 / maxdisp;
    // the collision cap (session.rs:927-955): the largest safe time of x - t d, two thirds of it
    rep[27] = NAN;
    if (F->ccd && std::isfinite(tau) && tau > 0.0) {
      auto tc = clk::now();
      std::vector<double> vel(nd);
      for (size_t r = 0; r < nd; ++r) vel[r] = -x[r];
      rs_ccd_options co = rs_ccd_options_default();
      co.gap = F->o.ccd_gap, co.reference_length = F->l0;
      co.max_iterations = F->o.ccd_max_iterations, co.close_factor = F->o.ccd_close_factor;
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
    rep[23] = xinf;
    const double tau_min = 1e-12 * F->l0 / xinf;
    std::vector<double> trial(nd);
    double E1 = E0;
    bool accepted = false;
    int halvings = 0;
    while (halvings <= F->o.max_halvings && tau >= tau_min) {
      if (F->cancel.load()) fail(RS_CANCELLED, "Cancelled", "flow", "the step was cancelled");
      for (size_t r = 0; r < nd; ++r) trial[r] = F->pos[r] - tau * x[r];
      bool ok = true;
      for (double v : trial) ok = ok && std::isfinite(v);
      double Et = NAN;
      if (ok && rs_bh_refit(bh.p, trial.data()) == RS_OK && rs_bh_energy(bh.p, F->o.alpha, F->o.beta, &Et) == RS_OK &&
          std::isfinite(Et) && Et <= E0 - F->o.armijo_c * tau * slope) {
        E1 = Et;
        accepted = true;
        break;
      }
      tau *= 0.5;
      ++halvings;
    }
    rep[13] = since(t);
    // 5. projection
    t = clk::now();
    double cres = 0.0;
    int newton_rounds = 0;
    bool proj_converged = true;
    if (accepted) {
      proj_converged = k == 0;
      for (int round = 0; round < F->o.newton_max && k > 0; ++round) {
        std::vector<double> phi(k);
        double worst_rel = 0.0;
        for (int i = 0; i < k; ++i) {
          double val = rows[i] == 0 ? total_area(nf, faces, trial.data()) : total_volume(nf, faces, trial.data());
          double tgt = rows[i] == 0 ? F->area0 : F->vol0;
          phi[i] = val - tgt;
          worst_rel = std::max(worst_rel, std::fabs(phi[i]) / std::max(1.0, std::fabs(tgt)));
        }
        if (worst_rel <= 1e-12) {
          proj_converged = true;
          break;
        }
        ++newton_rounds;
        std::vector<double> cc = solve_n(phi);
        for (size_t r = 0; r < nd; ++r) {
          double h = 0.0;
          for (int j = 0; j < k; ++j) h += hs[(size_t)j * n + r] * cc[j];
          trial[r] -= h;
        }
      }
      double b[3];
      barycenter(nv, nf, faces, trial.data(), b);
      for (int v = 0; v < nv; ++v)
        for (int kk = 0; kk < 3; ++kk) trial[3 * (size_t)v + kk] += F->bary0[kk] - b[kk];
      for (int i = 0; i < k; ++i) {
        double val = rows[i] == 0 ? total_area(nf, faces, trial.data()) : total_volume(nf, faces, trial.data());
        double tgt = rows[i] == 0 ? F->area0 : F->vol0;
        cres = std::max(cres, std::fabs(val - tgt) / std::max(1.0, std::fabs(tgt)));
      }
      if (cres <= 1e-12) proj_converged = true;
      // F after the projection, on the same lists (StepReport::energy_after, session.rs:155-156)
      double Ea = NAN;
      check(rs_bh_refit(bh.p, trial.data()), "flow (energy)");
      check(rs_bh_energy(bh.p, F->o.alpha, F->o.beta, &Ea), "flow (energy)");
      if (!std::isfinite(Ea)) fail(RS_NONFINITE_ENERGY, "NonFiniteEnergy", "flow", "non-finite energy after the projection");
      rep[26] = E1;
      E1 = Ea;
      F->pos = trial;
      F->last_tau = tau;
      F->iteration++;
    }
    rep[14] = since(t);
    if (F->lmodel) {
      int64_t ls = 0, lf = 0;
      check(rs_solver_learned_counts(sv.p, &ls, &lf), "flow");
      rep[19] = (double)ls, rep[20] = (double)lf;
    }
    if (!accepted) rep[26] = E0;
    rep[0] = E0;
    rep[1] = E1;
    rep[2] = accepted ? tau : 0.0;
    rep[3] = halvings;
    rep[15] = accepted ? 1.0 : 0.0;
    rep[17] = cres;
    rep[24] = newton_rounds;
    rep[25] = proj_converged ? 0.0 : 1.0;
    rep[8] = since(t_step);
    if (report) std::memcpy(report, rep, sizeof(rep));
  });
}

}  // extern "C"
