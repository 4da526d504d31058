// FP64 oracle of the direction solve and the descent step -- TEST INFRASTRUCTURE ONLY (see
// rs_oracle.h). A plain restatement, in C++ and double precision, of:
//
//   * the constraint set: barycenter, pin, area and volume rows, their values, Jacobians,
//     tolerances and the positional projection (RS/src/constraints/mod.rs:185-764);
//   * the dense saddle with the Schur complement of the nonlinear rows, its direction and the
//     Newton correction (RS/src/solve/dense.rs, RS/src/solve/schur.rs:101-356);
//   * the dense fractional preconditioner over face pairs (RS/src/solve/dense.rs:527-600,
//     RS/src/metric/dense.rs:453-467);
//   * the hierarchical saddle operator A' (RS/src/solve/iterative.rs:126-338), the augmented
//     sparse preconditioner with the symbol scale (RS/src/solve/precond.rs:466-564,1003-1079),
//     the coarse (deflation) correction (RS/src/solve/coarse.rs:101-328) and right-preconditioned
//     restarted GMRES with modified Gram-Schmidt and Givens rotations
//     (RS/src/solve/gmres.rs:227-590);
//   * one descent step: energy and differential, direction, Armijo backtracking, projection with
//     its safeguard (RS/src/step/session.rs:749-1100,1458-1615; RS/src/solve/schur.rs:450-575).
//
// Where the crate calls the faer library (0.24.4 in Cargo.lock) for its sparse LDL^T of L' and
// its dense factorizations, this file has its own: a sparse LDL^T in a nested-dissection order
// (the up-looking algorithm of T. A. Davis, "Algorithm 849: a concise sparse Cholesky
// factorization package", ACM TOMS 31(4), 2005), dense LU with partial pivoting, and Jacobi
// eigenvalue iteration for the coarse matrix. They compute the same mathematical objects;
// results agree with the crate's to rounding.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "rs_oracle.h"
#include "rso_internal.hpp"

namespace rso {
namespace {

thread_local std::string g_serr;

using clk = std::chrono::steady_clock;
double since(clk::time_point t) { return std::chrono::duration<double>(clk::now() - t).count(); }

[[noreturn]] void fail(int code, const std::string &m) { throw Error(code, m); }

void check_c(int rc, const char *what) {
  if (rc != 0) {
    std::string m = rso_last_error();
    if (m.empty()) m = rso_metric_last_error();
    fail(rc, std::string(what) + ": " + m);
  }
}

// ------------------------------------------------------------------ topology

// Face components seeded in face order, so that components are numbered by their smallest
// face (RS/src/surface.rs:349-402); vertices take the component of their faces.
struct Topo {
  int nv = 0, nf = 0, ncomp = 0;
  std::vector<tri> faces;
  std::vector<uint32_t> fcomp, vcomp;
};

Topo make_topo(int nv, int nf, const uint32_t *f) {
  Topo t;
  t.nv = nv, t.nf = nf;
  t.faces.resize(nf);
  for (int i = 0; i < nf; ++i) t.faces[i] = {f[3 * i], f[3 * i + 1], f[3 * i + 2]};
  std::vector<uint32_t> parent(nv);
  std::iota(parent.begin(), parent.end(), 0u);
  auto find = [&](uint32_t x) {
    while (parent[x] != x) x = parent[x] = parent[parent[x]];
    return x;
  };
  for (const tri &tr : t.faces)
    for (int c = 1; c < 3; ++c) {
      uint32_t a = find(tr[0]), b = find(tr[c]);
      if (a != b) parent[std::max(a, b)] = std::min(a, b);
    }
  std::vector<int64_t> id(nv, -1);
  t.fcomp.resize(nf);
  t.vcomp.assign(nv, 0);
  for (int i = 0; i < nf; ++i) {
    uint32_t r = find(t.faces[i][0]);
    if (id[r] < 0) id[r] = t.ncomp++;
    t.fcomp[i] = (uint32_t)id[r];
  }
  for (int v = 0; v < nv; ++v) t.vcomp[v] = id[find(v)] < 0 ? 0u : (uint32_t)id[find(v)];
  return t;
}

std::vector<v3> to_v3(int nv, const double *p) {
  std::vector<v3> out(nv);
  for (int v = 0; v < nv; ++v) out[v] = {p[3 * v], p[3 * v + 1], p[3 * v + 2]};
  return out;
}

// Per-face areas and vertex areas a_v = sum over incident faces of a_S / 3
// (RS/src/constraints/mod.rs:487-500; RS/src/geometry.rs:194-203).
void areas_of(const Topo &t, const std::vector<v3> &pos, std::vector<double> &fa, std::vector<double> &va) {
  fa.resize(t.nf);
  va.assign(t.nv, 0.0);
  for (int i = 0; i < t.nf; ++i) {
    double a;
    v3 n, x;
    face_quantities(corners(pos, t.faces[i]), a, n, x);
    fa[i] = a;
  }
  for (int i = 0; i < t.nf; ++i)
    for (uint32_t v : t.faces[i]) va[v] += fa[i] / 3.0;
}

// Mean edge length over the unique edges (RS/src/geometry.rs:249-256).
double mean_edge_length(const Topo &t, const std::vector<v3> &pos) {
  std::vector<std::pair<uint32_t, uint32_t>> e;
  e.reserve(3 * (size_t)t.nf);
  for (const tri &tr : t.faces)
    for (int c = 0; c < 3; ++c) {
      uint32_t a = tr[c], b = tr[(c + 1) % 3];
      e.push_back({std::min(a, b), std::max(a, b)});
    }
  std::sort(e.begin(), e.end());
  e.erase(std::unique(e.begin(), e.end()), e.end());
  double s = 0.0;
  for (auto [a, b] : e) s += norm(sub(pos[a], pos[b]));
  return s / (double)e.size();
}

// ------------------------------------------------------------------ constraint set

constexpr double NONLINEAR_TOLERANCE = 1e-8;  // constraints/mod.rs:147
constexpr double POSITIONAL_TOLERANCE = 1e-14;  // constraints/mod.rs:152
constexpr int POSITIONAL_MAX_ROUNDS = 100;  // constraints/mod.rs:155

enum RowKind { BARY = 0, PIN = 1, AREA = 2, VOLUME = 3 };

struct Row {
  int kind;
  int comp;   // barycenter, area, volume: component or -1 (all)
  int axis;   // barycenter, pin
  uint32_t vertex;
  double target;
};

struct SparseRow {
  std::vector<uint32_t> idx;
  std::vector<double> val;
};

// ConstraintSet::new, values, jacobian, tolerance, project_positional
// (RS/src/constraints/mod.rs:185-335, 435-764). Rows keep the crate's order: constraints in the
// given order, a barycenter as three rows (axis fastest) per group, a pin as three rows.
struct ConstraintSet {
  const Topo *t = nullptr;
  std::vector<Row> rows;

  bool in_comp(int v, int c) const { return c < 0 || (int)t->vcomp[v] == c; }

  v3 barycenter(const std::vector<double> &va, const std::vector<v3> &pos, int c) const {
    v3 s{{0, 0, 0}};
    double tot = 0.0;
    for (int v = 0; v < t->nv; ++v)
      if (in_comp(v, c)) {
        for (int k = 0; k < 3; ++k) s[k] += va[v] * pos[v][k];
        tot += va[v];
      }
    return scale(s, 1.0 / tot);
  }
  double area_of(const std::vector<double> &fa, int c) const {
    double s = 0.0;
    for (int i = 0; i < t->nf; ++i)
      if (c < 0 || (int)t->fcomp[i] == c) s += fa[i];
    return s;
  }
  double volume_of(const std::vector<v3> &pos, int c) const {  // constraints/mod.rs:474-485
    double s = 0.0;
    for (int i = 0; i < t->nf; ++i)
      if (c < 0 || (int)t->fcomp[i] == c) {
        auto p = corners(pos, t->faces[i]);
        s += dot(p[0], cross(p[1], p[2])) / 6.0;
      }
    return s;
  }

  bool positional(int r) const { return rows[r].kind == BARY || rows[r].kind == PIN; }
  std::vector<int> positional_rows() const {
    std::vector<int> o;
    for (int r = 0; r < (int)rows.size(); ++r)
      if (positional(r)) o.push_back(r);
    return o;
  }
  std::vector<int> nonlinear_rows() const {
    std::vector<int> o;
    for (int r = 0; r < (int)rows.size(); ++r)
      if (!positional(r)) o.push_back(r);
    return o;
  }
  double tolerance(int r) const {  // constraints/mod.rs:435-442
    double tg = std::fabs(rows[r].target);
    return tg > 0.0 ? NONLINEAR_TOLERANCE * tg : NONLINEAR_TOLERANCE;
  }

  std::vector<double> values(const std::vector<v3> &pos) const {  // constraints/mod.rs:519-553
    std::vector<double> fa, va;
    areas_of(*t, pos, fa, va);
    std::vector<double> out(rows.size());
    for (size_t r = 0; r < rows.size(); ++r) {
      const Row &w = rows[r];
      double value = 0.0;
      switch (w.kind) {
        case BARY: value = barycenter(va, pos, w.comp)[w.axis]; break;
        case PIN: value = pos[w.vertex][w.axis]; break;
        case AREA: value = area_of(fa, w.comp); break;
        default: value = volume_of(pos, w.comp); break;
      }
      out[r] = value - w.target;
    }
    return out;
  }

  // area gradient sum_{S ni v} 1/2 N_S x e_opp(v) (constraints/mod.rs:606-623)
  std::vector<v3> area_gradient(const std::vector<v3> &pos, int c) const {
    std::vector<v3> g(t->nv, v3{{0, 0, 0}});
    for (int i = 0; i < t->nf; ++i) {
      if (!(c < 0 || (int)t->fcomp[i] == c)) continue;
      auto p = corners(pos, t->faces[i]);
      double a;
      v3 n, x;
      face_quantities(p, a, n, x);
      for (int k = 0; k < 3; ++k) {
        v3 e = sub(p[(k + 2) % 3], p[(k + 1) % 3]);
        g[t->faces[i][k]] = add(g[t->faces[i][k]], scale(cross(n, e), 0.5));
      }
    }
    return g;
  }
  // volume gradient 1/6 sum_{S ni v} f_j x f_k (constraints/mod.rs:627-645)
  std::vector<v3> volume_gradient(const std::vector<v3> &pos, int c) const {
    std::vector<v3> g(t->nv, v3{{0, 0, 0}});
    for (int i = 0; i < t->nf; ++i) {
      if (!(c < 0 || (int)t->fcomp[i] == c)) continue;
      auto p = corners(pos, t->faces[i]);
      for (int k = 0; k < 3; ++k)
        g[t->faces[i][k]] = add(g[t->faces[i][k]], scale(cross(p[(k + 1) % 3], p[(k + 2) % 3]), 1.0 / 6.0));
    }
    return g;
  }

  // The Jacobian rows, sparse over the 3V columns 3 v + axis; barycenter weights frozen at pos
  // (constraints/mod.rs:556-604).
  std::vector<SparseRow> jacobian(const std::vector<v3> &pos, const std::vector<int> &which) const {
    std::vector<double> fa, va;
    areas_of(*t, pos, fa, va);
    std::vector<SparseRow> out;
    for (int r : which) {
      const Row &w = rows[r];
      SparseRow s;
      if (w.kind == BARY) {
        double tot = 0.0;
        for (int v = 0; v < t->nv; ++v)
          if (in_comp(v, w.comp)) tot += va[v];
        for (int v = 0; v < t->nv; ++v)
          if (in_comp(v, w.comp)) s.idx.push_back(3 * v + w.axis), s.val.push_back(va[v] / tot);
      } else if (w.kind == PIN) {
        s.idx.push_back(3 * w.vertex + w.axis), s.val.push_back(1.0);
      } else {
        std::vector<v3> g = w.kind == AREA ? area_gradient(pos, w.comp) : volume_gradient(pos, w.comp);
        for (int v = 0; v < t->nv; ++v)
          for (int k = 0; k < 3; ++k)
            if (g[v][k] != 0.0) s.idx.push_back(3 * v + k), s.val.push_back(g[v][k]);
      }
      out.push_back(std::move(s));
    }
    return out;
  }

  // One translation of every barycenter group, then every pin reset (constraints/mod.rs:707-740).
  void translate_and_reset(std::vector<v3> &pos) const {
    size_t r = 0;
    while (r < rows.size()) {
      if (rows[r].kind == BARY && rows[r].axis == 0) {
        std::vector<double> fa, va;
        areas_of(*t, pos, fa, va);
        v3 b = barycenter(va, pos, rows[r].comp);
        v3 d = {b[0] - rows[r].target, b[1] - rows[r + 1].target, b[2] - rows[r + 2].target};
        for (int v = 0; v < t->nv; ++v)
          if (in_comp(v, rows[r].comp))
            for (int k = 0; k < 3; ++k) pos[v][k] -= d[k];
        r += 3;
        continue;
      }
      ++r;
    }
    for (const Row &w : rows)
      if (w.kind == PIN) pos[w.vertex][w.axis] = w.target;
  }

  // constraints/mod.rs:657-704: rounds while a barycenter group holds a pinned vertex.
  void project_positional(std::vector<v3> &pos) const {
    std::vector<char> pinned(t->nv, 0);
    for (const Row &w : rows)
      if (w.kind == PIN) pinned[w.vertex] = 1;
    std::vector<size_t> mixed;
    for (size_t r = 0; r < rows.size(); ++r)
      if (rows[r].kind == BARY && rows[r].axis == 0)
        for (int v = 0; v < t->nv; ++v)
          if (pinned[v] && in_comp(v, rows[r].comp)) {
            mixed.push_back(r);
            break;
          }
    for (int round = 0; round < POSITIONAL_MAX_ROUNDS; ++round) {
      translate_and_reset(pos);
      if (mixed.empty()) return;
      double sc = 1.0;
      for (const v3 &p : pos)
        for (double x : p) sc = std::max(sc, std::fabs(x));
      std::vector<double> fa, va;
      areas_of(*t, pos, fa, va);
      double worst = 0.0;
      for (size_t r : mixed) {
        v3 b = barycenter(va, pos, rows[r].comp);
        for (int k = 0; k < 3; ++k) worst = std::max(worst, std::fabs(b[k] - rows[r + k].target));
      }
      if (!(worst > POSITIONAL_TOLERANCE * sc)) return;
    }
  }
};

// ConstraintSet::new (constraints/mod.rs:191-333) from the C description.
ConstraintSet make_constraints(const Topo &t, const std::vector<v3> &pos, const rso_constraints *c) {
  ConstraintSet s;
  s.t = &t;
  if (!c) return s;
  std::vector<double> fa, va;
  areas_of(t, pos, fa, va);
  size_t toff = 0, poff = 0;
  for (int i = 0; i < c->n; ++i) {
    const int kind = c->kind[i], comp = c->comp[i], nt = c->n_target[i];
    const double *tg = nt > 0 ? c->target + toff : nullptr;
    toff += nt;
    if (comp >= t.ncomp)
      fail(RSO_INVALID_OPTION, "ConstraintOutOfRange: component " + std::to_string(comp) + ", " +
                                   std::to_string(t.ncomp) + " components");
    if (kind == BARY) {
      std::vector<int> groups;
      if (comp >= 0) groups.push_back(comp);
      else if (c->per_component)
        for (int k = 0; k < t.ncomp; ++k) groups.push_back(k);
      else groups.push_back(-1);
      for (int g : groups) {
        v3 cur = s.barycenter(va, pos, g);
        for (int a = 0; a < 3; ++a) s.rows.push_back({BARY, g, a, 0u, tg ? tg[a] : cur[a]});
      }
    } else if (kind == PIN) {
      const int np = c->n_pin[i];
      const uint32_t *pv = c->pin + poff;
      poff += np;
      for (int k = 0; k < np; ++k) {
        if ((int)pv[k] >= t.nv)
          fail(RSO_INVALID_OPTION, "ConstraintOutOfRange: pinned vertex " + std::to_string(pv[k]));
        for (int a = 0; a < 3; ++a) s.rows.push_back({PIN, -1, a, pv[k], tg ? tg[3 * k + a] : pos[pv[k]][a]});
      }
    } else if (kind == AREA) {
      s.rows.push_back({AREA, comp, 0, 0u, tg ? tg[0] : s.area_of(fa, comp)});
    } else if (kind == VOLUME) {
      // the volume needs consistently oriented components: no edge traversed in the same
      // direction by two faces (VolumeNeedsOrientation, constraints/mod.rs:287-296)
      std::vector<std::pair<uint64_t, int>> dir;
      for (int f = 0; f < t.nf; ++f)
        if (comp < 0 || (int)t.fcomp[f] == comp)
          for (int k = 0; k < 3; ++k)
            dir.push_back({((uint64_t)t.faces[f][k] << 32) | t.faces[f][(k + 1) % 3], f});
      std::sort(dir.begin(), dir.end());
      for (size_t a = 1; a < dir.size(); ++a)
        if (dir[a].first == dir[a - 1].first)
          fail(RSO_INVALID_OPTION, "NonOrientable: component " + std::to_string(t.fcomp[dir[a].second]) +
                                       " is not consistently oriented: faces " + std::to_string(dir[a - 1].second) +
                                       " and " + std::to_string(dir[a].second) + " traverse an edge the same way");
      s.rows.push_back({VOLUME, comp, 0, 0u, tg ? tg[0] : s.volume_of(pos, comp)});
    } else {
      fail(RSO_INVALID_OPTION, "unknown constraint kind " + std::to_string(kind));
    }
  }
  // Every component's translations must be fixed by a barycenter or a pin
  // (TranslationNotFixed, constraints/mod.rs:335-345).
  for (int k = 0; k < t.ncomp; ++k) {
    bool fixed = false;
    for (const Row &w : s.rows)
      if ((w.kind == BARY && (w.comp < 0 || w.comp == k)) || (w.kind == PIN && (int)t.vcomp[w.vertex] == k))
        fixed = true;
    if (!fixed) fail(RSO_SINGULAR, "TranslationNotFixed: component " + std::to_string(k));
  }
  return s;
}

// ------------------------------------------------------------------ dense linear algebra

// LU with partial pivoting of a row-major n x n matrix; fails on a zero pivot.
struct DenseLu {
  int n = 0;
  std::vector<double> a;
  std::vector<int> piv;
  void factor(int n_, std::vector<double> m) {
    n = n_, a = std::move(m), piv.resize(n);
    for (int k = 0; k < n; ++k) {
      int p = k;
      for (int i = k + 1; i < n; ++i)
        if (std::fabs(a[(size_t)i * n + k]) > std::fabs(a[(size_t)p * n + k])) p = i;
      if (!(std::fabs(a[(size_t)p * n + k]) > 0.0)) fail(RSO_SINGULAR, "SingularSaddle: the saddle matrix is singular");
      piv[k] = p;
      if (p != k)
        for (int j = 0; j < n; ++j) std::swap(a[(size_t)k * n + j], a[(size_t)p * n + j]);
      const double d = a[(size_t)k * n + k];
      for (int i = k + 1; i < n; ++i) {
        double l = a[(size_t)i * n + k] / d;
        a[(size_t)i * n + k] = l;
        if (l != 0.0)
          for (int j = k + 1; j < n; ++j) a[(size_t)i * n + j] -= l * a[(size_t)k * n + j];
      }
    }
  }
  std::vector<double> solve(std::vector<double> b) const {
    for (int k = 0; k < n; ++k) std::swap(b[k], b[piv[k]]);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < i; ++j) b[i] -= a[(size_t)i * n + j] * b[j];
    for (int i = n - 1; i >= 0; --i) {
      for (int j = i + 1; j < n; ++j) b[i] -= a[(size_t)i * n + j] * b[j];
      b[i] /= a[(size_t)i * n + i];
    }
    return b;
  }
};

// Symmetric eigendecomposition by cyclic Jacobi rotations (m x m, row-major); the coarse
// matrix is small (3 per free component plus its rows).
void jacobi_eigen(int m, std::vector<double> a, std::vector<double> &lam, std::vector<double> &u) {
  u.assign((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) u[(size_t)i * m + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        double x = a[(size_t)i * m + j] * a[(size_t)i * m + j];
        tot += x;
        if (i != j) off += x;
      }
    if (!(off > 1e-30 * tot)) break;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) {
        double apq = a[(size_t)p * m + q];
        if (apq == 0.0) continue;
        double app = a[(size_t)p * m + p], aqq = a[(size_t)q * m + q];
        double th = 0.5 * (aqq - app) / apq;
        double tt = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        double c = 1.0 / std::sqrt(tt * tt + 1.0), s = tt * c;
        for (int k = 0; k < m; ++k) {
          double akp = a[(size_t)k * m + p], akq = a[(size_t)k * m + q];
          a[(size_t)k * m + p] = c * akp - s * akq;
          a[(size_t)k * m + q] = s * akp + c * akq;
        }
        for (int k = 0; k < m; ++k) {
          double apk = a[(size_t)p * m + k], aqk = a[(size_t)q * m + k];
          a[(size_t)p * m + k] = c * apk - s * aqk;
          a[(size_t)q * m + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < m; ++k) {
          double ukp = u[(size_t)k * m + p], ukq = u[(size_t)k * m + q];
          u[(size_t)k * m + p] = c * ukp - s * ukq;
          u[(size_t)k * m + q] = s * ukp + c * ukq;
        }
      }
  }
  lam.resize(m);
  for (int i = 0; i < m; ++i) lam[i] = a[(size_t)i * m + i];
}

// ------------------------------------------------------------------ sparse LDL^T

// Symmetric sparse matrix by rows (full pattern, both triangles).
struct Csr {
  int n = 0;
  std::vector<int64_t> ptr;
  std::vector<int> col;
  std::vector<double> val;
};

// A symmetric positive definite matrix factored as P K P^T = L D L^T. The order is a nested
// dissection of the mesh by coordinate bisection (separators last); the factorization is the
// up-looking LDL^T of Davis (ACM TOMS 31(4), 2005): the pattern of row k of L is the set of
// elimination-tree paths from the nonzeros of row k of the matrix.
struct SparseLdl {
  int n = 0;
  std::vector<int> perm, iperm;  // perm[new] = old
  std::vector<int64_t> lp;
  std::vector<int> li;
  std::vector<double> lx, d;

  static void dissect(const Csr &a, const std::vector<v3> &xyz, std::vector<int> &ids, std::vector<int> &mark,
                      int stamp_base, std::vector<int> &out) {
    if (ids.size() <= 64) {
      out.insert(out.end(), ids.begin(), ids.end());
      return;
    }
    v3 lo = xyz[ids[0]], hi = xyz[ids[0]];
    for (int v : ids)
      for (int k = 0; k < 3; ++k) lo[k] = std::min(lo[k], xyz[v][k]), hi[k] = std::max(hi[k], xyz[v][k]);
    int ax = 0;
    for (int k = 1; k < 3; ++k)
      if (hi[k] - lo[k] > hi[ax] - lo[ax]) ax = k;
    std::vector<int> sorted = ids;
    size_t mid = sorted.size() / 2;
    std::nth_element(sorted.begin(), sorted.begin() + mid, sorted.end(), [&](int p, int q) {
      return xyz[p][ax] < xyz[q][ax] || (xyz[p][ax] == xyz[q][ax] && p < q);
    });
    // side: 1 left, 2 right (marks are local to this call through the stamp)
    const int left = stamp_base + 1, right = stamp_base + 2;
    for (size_t i = 0; i < sorted.size(); ++i) mark[sorted[i]] = i < mid ? left : right;
    std::vector<int> L, R, S;
    for (int v : sorted) {
      if (mark[v] != left) continue;
      bool sep = false;
      for (int64_t p = a.ptr[v]; p < a.ptr[v + 1] && !sep; ++p) sep = mark[a.col[p]] == right;
      (sep ? S : L).push_back(v);
    }
    for (int v : sorted)
      if (mark[v] == right) R.push_back(v);
    for (int v : ids) mark[v] = 0;
    if (L.empty() || R.empty()) {  // no progress: take the set as it is
      out.insert(out.end(), ids.begin(), ids.end());
      return;
    }
    dissect(a, xyz, L, mark, stamp_base + 2, out);
    dissect(a, xyz, R, mark, stamp_base + 2, out);
    out.insert(out.end(), S.begin(), S.end());
  }

  void factor(const Csr &a, const std::vector<v3> &xyz) {
    n = a.n;
    std::vector<int> ids(n), mark(n, 0);
    std::iota(ids.begin(), ids.end(), 0);
    perm.clear();
    perm.reserve(n);
    dissect(a, xyz, ids, mark, 0, perm);
    iperm.assign(n, 0);
    for (int i = 0; i < n; ++i) iperm[perm[i]] = i;
    // upper triangle of the permuted matrix by columns = lower entries of each permuted row
    std::vector<std::vector<std::pair<int, double>>> up(n);
    for (int i = 0; i < n; ++i) {
      const int r = perm[i];
      for (int64_t p = a.ptr[r]; p < a.ptr[r + 1]; ++p) {
        int j = iperm[a.col[p]];
        if (j <= i) up[i].push_back({j, a.val[p]});
      }
    }
    // symbolic: elimination tree and column counts (ldl_symbolic)
    std::vector<int> parent(n, -1), flag(n, -1), lnz(n, 0);
    for (int k = 0; k < n; ++k) {
      flag[k] = k;
      for (auto [i0, x] : up[k]) {
        (void)x;
        for (int i = i0; i < k && flag[i] != k; i = parent[i]) {
          if (parent[i] == -1) parent[i] = k;
          ++lnz[i];
          flag[i] = k;
        }
      }
    }
    lp.assign(n + 1, 0);
    for (int k = 0; k < n; ++k) lp[k + 1] = lp[k] + lnz[k];
    li.assign(lp[n], 0);
    lx.assign(lp[n], 0.0);
    d.assign(n, 0.0);
    // numeric (ldl_numeric)
    std::vector<double> y(n, 0.0);
    std::vector<int> pattern(n), fill(n, 0);
    std::fill(flag.begin(), flag.end(), -1);
    for (int k = 0; k < n; ++k) {
      int top = n;
      flag[k] = k;
      for (auto [i0, x] : up[k]) {
        y[i0] += x;
        int len = 0;
        for (int i = i0; flag[i] != k; i = parent[i]) {
          pattern[len++] = i;
          flag[i] = k;
        }
        while (len > 0) pattern[--top] = pattern[--len];
      }
      d[k] = y[k];
      y[k] = 0.0;
      for (; top < n; ++top) {
        const int i = pattern[top];
        const double yi = y[i];
        y[i] = 0.0;
        const int64_t p2 = lp[i] + fill[i];
        for (int64_t p = lp[i]; p < p2; ++p) y[li[p]] -= lx[p] * yi;
        const double l = yi / d[i];
        d[k] -= l * yi;
        li[p2] = k;
        lx[p2] = l;
        ++fill[i];
      }
      if (!(d[k] > 0.0)) fail(RSO_SINGULAR, "SingularSaddle: zero pivot in the Laplacian block");
    }
  }

  // x (n x m, row-major, natural order) <- K^-1 x
  void solve(double *x, int m) const {
    std::vector<double> w((size_t)n * m);
    for (int i = 0; i < n; ++i)
      for (int c = 0; c < m; ++c) w[(size_t)i * m + c] = x[(size_t)perm[i] * m + c];
    for (int j = 0; j < n; ++j) {
      const double *wj = &w[(size_t)j * m];
      for (int64_t p = lp[j]; p < lp[j + 1]; ++p) {
        double *wi = &w[(size_t)li[p] * m];
        for (int c = 0; c < m; ++c) wi[c] -= lx[p] * wj[c];
      }
    }
    for (int j = 0; j < n; ++j)
      for (int c = 0; c < m; ++c) w[(size_t)j * m + c] /= d[j];
    for (int j = n - 1; j >= 0; --j) {
      double *wj = &w[(size_t)j * m];
      for (int64_t p = lp[j]; p < lp[j + 1]; ++p) {
        const double *wi = &w[(size_t)li[p] * m];
        for (int c = 0; c < m; ++c) wj[c] -= lx[p] * wi[c];
      }
    }
    for (int i = 0; i < n; ++i)
      for (int c = 0; c < m; ++c) x[(size_t)perm[i] * m + c] = w[(size_t)i * m + c];
  }
};

// ------------------------------------------------------------------ saddle solvers

// The positional rows as C_1 (x) I_3: every barycenter group and pinned vertex is one row of
// the scalar C_1 (per_axis_rows, RS/src/solve/precond.rs:82-116); C_Q row 3 g + axis.
struct PositionalRows {
  int k1 = 0;
  std::vector<std::vector<std::pair<int, double>>> c1;  // k1 rows over vertices
  std::vector<int> comps;  // touched components per row (one per row here)
};

PositionalRows positional_of(const ConstraintSet &set, const std::vector<v3> &pos) {
  PositionalRows pr;
  std::vector<int> q = set.positional_rows();
  std::vector<SparseRow> j = set.jacobian(pos, q);
  for (size_t r = 0; r < q.size(); r += 3) {
    std::vector<std::pair<int, double>> row;
    for (size_t p = 0; p < j[r].idx.size(); ++p) row.push_back({(int)(j[r].idx[p] / 3), j[r].val[p]});
    pr.c1.push_back(row);
  }
  pr.k1 = (int)pr.c1.size();
  return pr;
}

// A saddle solver of A' = [[A (x) I3, C_Q^T], [C_Q, 0]] (SaddleSolver, RS/src/solve/mod.rs:107-130).
struct Saddle {
  int nd = 0, nq = 0;
  virtual ~Saddle() = default;
  int dim() const { return nd + nq; }
  // solutions of A' [x; l] = rhs for nb full right-hand sides (stacked), with per-solve
  // reports (iterations, true relative residual, converged, seconds, cycles)
  virtual void solve_many(int nb, const double *rhs, double *sol, double *rep5) = 0;
};

// DenseSaddle: A' assembled and factored by LU (RS/src/solve/dense.rs).
struct DenseSaddle : Saddle {
  DenseLu lu;
  void build(const std::vector<double> &a, int nv, const std::vector<SparseRow> &cq) {
    nd = 3 * nv, nq = (int)cq.size();
    const int n = nd + nq;
    std::vector<double> m((size_t)n * n, 0.0);
    for (int v = 0; v < nv; ++v)
      for (int w = 0; w < nv; ++w)
        for (int k = 0; k < 3; ++k) m[(size_t)(3 * v + k) * n + 3 * w + k] = a[(size_t)v * nv + w];
    for (int r = 0; r < nq; ++r)
      for (size_t p = 0; p < cq[r].idx.size(); ++p) {
        m[(size_t)(nd + r) * n + cq[r].idx[p]] += cq[r].val[p];
        m[(size_t)cq[r].idx[p] * n + nd + r] += cq[r].val[p];
      }
    lu.factor(n, std::move(m));
  }
  void solve_many(int nb, const double *rhs, double *sol, double *rep5) override {
    const int n = dim();
    for (int q = 0; q < nb; ++q) {
      std::vector<double> b(rhs + (size_t)q * n, rhs + (size_t)(q + 1) * n);
      std::vector<double> x = lu.solve(b);
      std::copy(x.begin(), x.end(), sol + (size_t)q * n);
      if (rep5) rep5[5 * q] = 0, rep5[5 * q + 1] = 0, rep5[5 * q + 2] = 1, rep5[5 * q + 3] = 0, rep5[5 * q + 4] = 0;
    }
  }
};

// The dense metric A (V x V) of w_TP (B + c_lo B0): the chi = 0 product applied to unit vectors.
std::vector<double> dense_metric(int nv, const double *pos, int nf, const uint32_t *faces, double alpha,
                                 double beta, double w_tp, double c_lo) {
  rso_metric *m = nullptr;
  check_c(rso_metric_build(nv, pos, nf, faces, alpha, beta, 0.0, 8, 64, &m), "dense metric");
  std::unique_ptr<rso_metric, void (*)(rso_metric *)> hold(m, rso_metric_free);
  std::vector<double> xs((size_t)nv * 3 * nv, 0.0), ys((size_t)nv * 3 * nv);
  for (int v = 0; v < nv; ++v) xs[(size_t)v * 3 * nv + 3 * v] = 1.0;
  check_c(rso_metric_apply(m, w_tp, w_tp * c_lo, nv, xs.data(), ys.data()), "dense metric");
  std::vector<double> a((size_t)nv * nv);
  for (int v = 0; v < nv; ++v)
    for (int w = 0; w < nv; ++w) a[(size_t)w * nv + v] = ys[(size_t)v * 3 * nv + 3 * w];
  return a;
}

// The cotan stiffness W (RS/src/geometry.rs:221-245) plus eps M, by rows.
Csr laplacian_block(const Topo &t, const std::vector<v3> &pos, const std::vector<double> &mass, double eps_rel,
                    double &eps_out) {
  std::vector<std::vector<std::pair<int, double>>> rows(t.nv);
  for (const tri &tr : t.faces) {
    auto p = corners(pos, tr);
    for (int c = 0; c < 3; ++c) {
      uint32_t a = tr[(c + 1) % 3], b = tr[(c + 2) % 3];
      v3 u = sub(p[(c + 1) % 3], p[c]), w = sub(p[(c + 2) % 3], p[c]);
      double h = 0.5 * (dot(u, w) / norm(cross(u, w)));
      rows[a].push_back({(int)b, -h});
      rows[b].push_back({(int)a, -h});
      rows[a].push_back({(int)a, h});
      rows[b].push_back({(int)b, h});
    }
  }
  Csr k;
  k.n = t.nv;
  k.ptr.assign(t.nv + 1, 0);
  double trw = 0.0, trm = 0.0;
  for (int v = 0; v < t.nv; ++v) {
    auto &r = rows[v];
    std::sort(r.begin(), r.end(), [](auto &x, auto &y) { return x.first < y.first; });
    std::vector<std::pair<int, double>> merged;
    for (auto &e : r) {
      if (!merged.empty() && merged.back().first == e.first) merged.back().second += e.second;
      else merged.push_back(e);
    }
    r.swap(merged);
    for (auto &e : r)
      if (e.first == v) trw += e.second;
    trm += mass[v];
  }
  const double eps = eps_rel * trw / trm;  // preconditioner_epsilon (RS/src/solve/dense.rs:529-533)
  eps_out = eps;
  for (int v = 0; v < t.nv; ++v) {
    for (auto &e : rows[v]) {
      k.col.push_back(e.first);
      k.val.push_back(e.first == v ? e.second + eps * mass[v] : e.second);
    }
    k.ptr[v + 1] = (int64_t)k.col.size();
  }
  return k;
}

// L' = [[K (x) I3, C_Q^T], [C_Q, 0]] with C_Q = C_1 (x) I3, solved per axis through the Schur
// complement of the multipliers: y = K^-1 (r - C_1^T l), l from S_1 l = C_1 K^-1 r - b with
// S_1 = C_1 K^-1 C_1^T. This is the block elimination of the crate's factor order "Laplacian
// block, then the multipliers" (LaplacianSaddle, RS/src/solve/precond.rs:157-460).
struct LaplacianSaddle {
  int nv = 0, k1 = 0;
  Csr K;
  SparseLdl ldl;
  PositionalRows pr;
  std::vector<double> Y;  // K^-1 C_1^T, nv x k1
  DenseLu s1;
  void build(const Csr &k, const std::vector<v3> &xyz, const PositionalRows &p) {
    K = k, nv = k.n, pr = p, k1 = p.k1;
    ldl.factor(K, xyz);
    Y.assign((size_t)nv * k1, 0.0);
    for (int g = 0; g < k1; ++g)
      for (auto [v, w] : pr.c1[g]) Y[(size_t)v * k1 + g] += w;
    if (k1 > 0) ldl.solve(Y.data(), k1);
    std::vector<double> s((size_t)k1 * k1, 0.0);
    for (int g = 0; g < k1; ++g)
      for (int h = 0; h < k1; ++h) {
        double acc = 0.0;
        for (auto [v, w] : pr.c1[g]) acc += w * Y[(size_t)v * k1 + h];
        s[(size_t)g * k1 + h] = acc;
      }
    if (k1 > 0) s1.factor(k1, s);
  }
  // z = L'^-1 r for full vectors (3V + 3 k1)
  void solve(const double *r, double *z) const {
    const size_t nd = 3 * (size_t)nv;
    std::vector<double> u(r, r + nd);
    ldl.solve(u.data(), 3);
    for (int a = 0; a < 3; ++a) {
      if (k1 == 0) break;
      std::vector<double> rhs(k1);
      for (int g = 0; g < k1; ++g) {
        double acc = 0.0;
        for (auto [v, w] : pr.c1[g]) acc += w * u[3 * (size_t)v + a];
        rhs[g] = acc - r[nd + 3 * g + a];
      }
      std::vector<double> lam = s1.solve(rhs);
      for (int v = 0; v < nv; ++v) {
        double acc = 0.0;
        for (int g = 0; g < k1; ++g) acc += Y[(size_t)v * k1 + g] * lam[g];
        u[3 * (size_t)v + a] -= acc;
      }
      for (int g = 0; g < k1; ++g) z[nd + 3 * g + a] = lam[g];
    }
    std::copy(u.begin(), u.end(), z);
  }
};

// Gagliardo constant I(t) = pi Gamma(1-t) / (t 4^t Gamma(1+t)) and the planar symbol ratio
// 4 I(sigma) I(2 - s) of W^-1 L_{2-s} W^-1 B (fractional_symbol_ratio, precond.rs:540-564).
double gagliardo(double t) { return M_PI * std::tgamma(1.0 - t) / (t * std::pow(4.0, t) * std::tgamma(1.0 + t)); }
double symbol_ratio(double alpha, double beta) {
  const double s = (beta - 2.0) / alpha;
  return 4.0 * gagliardo(s - 1.0) * gagliardo(2.0 - s);
}

// The hierarchical saddle solver: A' by the block cluster tree (HierarchicalOperator,
// iterative.rs:126-338), the augmented vertex-pair preconditioner with the symbol scale
// (SparsePreconditioner, precond.rs:1003-1079), the coarse correction when a component's
// translations are not fixed by rows of its own (coarse.rs), right-preconditioned GMRES.
struct HSaddle : Saddle {
  const Topo *t = nullptr;
  rso_solver_options o{};
  rso_metric *metric = nullptr;
  rso_vfrac *vfrac = nullptr;
  std::vector<SparseRow> cq;
  LaplacianSaddle lps;
  double frac_scale = 1.0, eps = 0.0;
  bool multi = false;
  // coarse space
  int cm = 0;
  std::vector<int> c_slot, c_axis, c_row;  // per column: translation (slot, axis) or row (-1)
  std::vector<double> c_scale;
  std::vector<std::vector<uint32_t>> members;
  std::vector<double> az, epinv;  // dim x cm (column-major), cm x cm
  double seconds_build[4] = {0, 0, 0, 0};
  int64_t op_apps = 0, prec_apps = 0;

  ~HSaddle() override {
    if (metric) rso_metric_free(metric);
    if (vfrac) rso_vfrac_free(vfrac);
  }

  void apply(int nb, const double *xs, double *ys) {
    const int n = dim();
    std::vector<double> xp((size_t)nb * nd), yp((size_t)nb * nd);
    for (int q = 0; q < nb; ++q) std::copy(xs + (size_t)q * n, xs + (size_t)q * n + nd, xp.data() + (size_t)q * nd);
    check_c(rso_metric_apply(metric, o.tp_weight, o.tp_weight * (o.low_order ? 1.0 : 0.0), nb, xp.data(), yp.data()),
            "operator");
    for (int q = 0; q < nb; ++q) {
      const double *x = xs + (size_t)q * n;
      double *y = ys + (size_t)q * n;
      std::copy(yp.data() + (size_t)q * nd, yp.data() + (size_t)(q + 1) * nd, y);
      for (int r = 0; r < nq; ++r) {
        double acc = 0.0;
        for (size_t p = 0; p < cq[r].idx.size(); ++p) {
          y[cq[r].idx[p]] += cq[r].val[p] * x[nd + r];
          acc += cq[r].val[p] * x[cq[r].idx[p]];
        }
        y[nd + r] = acc;
      }
    }
    op_apps += nb;
  }

  void fine(int nb, const double *rs, double *zs) {
    const int n = dim();
    std::vector<double> ys((size_t)nb * n), vs((size_t)nb * n, 0.0);
    for (int q = 0; q < nb; ++q) lps.solve(rs + (size_t)q * n, ys.data() + (size_t)q * n);
    std::vector<double> yp((size_t)nb * nd), vp((size_t)nb * nd);
    for (int q = 0; q < nb; ++q) std::copy(ys.data() + (size_t)q * n, ys.data() + (size_t)q * n + nd, yp.data() + (size_t)q * nd);
    check_c(rso_vfrac_apply(vfrac, nb, yp.data(), vp.data()), "preconditioner");
    for (int q = 0; q < nb; ++q) {
      double *v = vs.data() + (size_t)q * n;
      const double *y = ys.data() + (size_t)q * n;
      for (int i = 0; i < nd; ++i) v[i] = frac_scale * vp[(size_t)q * nd + i];
      // v = s L y - (K (x) I3) y
      for (int j = 0; j < lps.nv; ++j) {
        double acc[3] = {0, 0, 0};
        for (int64_t p = lps.K.ptr[j]; p < lps.K.ptr[j + 1]; ++p) {
          const int i = lps.K.col[p];
          for (int a = 0; a < 3; ++a) acc[a] += lps.K.val[p] * y[3 * (size_t)i + a];
        }
        for (int a = 0; a < 3; ++a) v[3 * (size_t)j + a] -= acc[a];
      }
      lps.solve(v, zs + (size_t)q * n);
      for (int i = 0; i < n; ++i) zs[(size_t)q * n + i] += y[i];
    }
  }

  std::vector<double> zt(const double *r) const {
    std::vector<double> out(cm, 0.0);
    for (int j = 0; j < cm; ++j) {
      if (c_row[j] >= 0) {
        out[j] = r[nd + c_row[j]];
      } else {
        double s = 0.0;
        for (uint32_t v : members[c_slot[j]]) s += r[3 * (size_t)v + c_axis[j]];
        out[j] = c_scale[j] * s;
      }
    }
    return out;
  }
  std::vector<double> e_solve(const std::vector<double> &tv) const {
    std::vector<double> out(cm, 0.0);
    for (int i = 0; i < cm; ++i) {
      double s = 0.0;
      for (int j = 0; j < cm; ++j) s += epinv[(size_t)i * cm + j] * tv[j];
      out[i] = s;
    }
    return out;
  }

  void precondition(int nb, const double *rs, double *zs) {
    prec_apps += nb;
    if (o.preconditioner == 0) {
      std::copy(rs, rs + (size_t)nb * dim(), zs);
      return;
    }
    if (cm == 0) return fine(nb, rs, zs);
    // the balancing preconditioner around the fine one (CoarseSpace::apply_many, coarse.rs:296-327)
    const int n = dim();
    std::vector<double> rp(rs, rs + (size_t)nb * n);
    std::vector<std::vector<double>> ycs(nb);
    for (int q = 0; q < nb; ++q) {
      ycs[q] = e_solve(zt(rs + (size_t)q * n));
      for (int j = 0; j < cm; ++j)
        if (ycs[q][j] != 0.0)
          for (int i = 0; i < n; ++i) rp[(size_t)q * n + i] -= ycs[q][j] * az[(size_t)j * n + i];
    }
    fine(nb, rp.data(), zs);
    for (int q = 0; q < nb; ++q) {
      double *z = zs + (size_t)q * n;
      std::vector<double> azt(cm);
      for (int j = 0; j < cm; ++j) {
        double s = 0.0;
        for (int i = 0; i < n; ++i) s += az[(size_t)j * n + i] * z[i];
        azt[j] = s;
      }
      std::vector<double> t2 = e_solve(azt);
      for (int j = 0; j < cm; ++j) {
        double c = ycs[q][j] - t2[j];
        if (c_row[j] >= 0) z[nd + c_row[j]] += c;
        else
          for (uint32_t v : members[c_slot[j]]) z[3 * (size_t)v + c_axis[j]] += c_scale[j] * c;
      }
    }
  }

  // CoarseSpace::free_components and build (coarse.rs:63-247)
  void build_coarse() {
    const int nc = t->ncomp;
    std::vector<char> fixed(nc, 0);
    std::vector<std::vector<int>> touched(nq);
    for (int r = 0; r < nq; ++r) {
      std::vector<int> cs;
      for (uint32_t i : cq[r].idx) cs.push_back((int)t->vcomp[i / 3]);
      std::sort(cs.begin(), cs.end());
      cs.erase(std::unique(cs.begin(), cs.end()), cs.end());
      if (cs.size() == 1) fixed[cs[0]] = 1;
      touched[r] = cs;
    }
    std::vector<int> freec, rows;
    for (int k = 0; k < nc; ++k)
      if (!fixed[k]) freec.push_back(k);
    if (freec.empty()) return;
    for (int r = 0; r < nq; ++r)
      for (int k : touched[r])
        if (!fixed[k]) {
          rows.push_back(r);
          break;
        }
    const int n = dim();
    cm = 3 * (int)freec.size() + (int)rows.size();
    std::vector<int> slot_of(nc, -1);
    for (size_t k = 0; k < freec.size(); ++k) slot_of[freec[k]] = (int)k;
    members.assign(freec.size(), {});
    for (int v = 0; v < t->nv; ++v)
      if (slot_of[t->vcomp[v]] >= 0) members[slot_of[t->vcomp[v]]].push_back(v);
    // A 1_c, three components per product
    std::vector<std::vector<double>> a1(freec.size());
    for (size_t c0 = 0; c0 < freec.size(); c0 += 3) {
      std::vector<double> x(n, 0.0), y(n);
      for (size_t a = 0; a < 3 && c0 + a < freec.size(); ++a)
        for (uint32_t v : members[c0 + a]) x[3 * (size_t)v + a] = 1.0;
      apply(1, x.data(), y.data());
      for (size_t a = 0; a < 3 && c0 + a < freec.size(); ++a) {
        a1[c0 + a].resize(t->nv);
        for (int v = 0; v < t->nv; ++v) a1[c0 + a][v] = y[3 * (size_t)v + a];
      }
    }
    c_slot.clear(), c_axis.clear(), c_row.clear(), c_scale.clear();
    for (size_t k = 0; k < freec.size(); ++k)
      for (int a = 0; a < 3; ++a)
        c_slot.push_back((int)k), c_axis.push_back(a), c_row.push_back(-1),
            c_scale.push_back(1.0 / std::sqrt((double)members[k].size()));
    for (int r : rows) c_slot.push_back(-1), c_axis.push_back(0), c_row.push_back(r), c_scale.push_back(1.0);
    az.assign((size_t)n * cm, 0.0);
    for (int j = 0; j < cm; ++j) {
      double *out = &az[(size_t)j * n];
      if (c_row[j] < 0) {
        const int sl = c_slot[j], ax = c_axis[j];
        const double sc = c_scale[j];
        for (int v = 0; v < t->nv; ++v) out[3 * (size_t)v + ax] = sc * a1[sl][v];
        std::vector<double> zc(nd, 0.0);
        for (uint32_t v : members[sl]) zc[3 * (size_t)v + ax] = sc;
        for (int r = 0; r < nq; ++r) {
          double acc = 0.0;
          for (size_t p = 0; p < cq[r].idx.size(); ++p) acc += cq[r].val[p] * zc[cq[r].idx[p]];
          out[nd + r] = acc;
        }
      } else {
        const SparseRow &row = cq[c_row[j]];
        for (size_t p = 0; p < row.idx.size(); ++p) out[row.idx[p]] = row.val[p];
      }
    }
    std::vector<double> e((size_t)cm * cm);
    for (int j = 0; j < cm; ++j) {
      std::vector<double> tv = zt(&az[(size_t)j * n]);
      for (int i = 0; i < cm; ++i) e[(size_t)i * cm + j] = tv[i];
    }
    for (int j = 0; j < cm; ++j)
      for (int i = 0; i < j; ++i) {
        double s = 0.5 * (e[(size_t)i * cm + j] + e[(size_t)j * cm + i]);
        e[(size_t)i * cm + j] = e[(size_t)j * cm + i] = s;
      }
    std::vector<double> lam, u;
    jacobi_eigen(cm, e, lam, u);
    double lmax = 0.0;
    for (double l : lam) lmax = std::max(lmax, std::fabs(l));
    epinv.assign((size_t)cm * cm, 0.0);
    for (int k = 0; k < cm; ++k) {
      const double l = lam[k];
      if (std::isnan(l) || std::fabs(l) <= 1e-12 * lmax) continue;
      for (int i = 0; i < cm; ++i) {
        const double ui = u[(size_t)i * cm + k] / l;
        for (int jj = 0; jj < cm; ++jj) epinv[(size_t)i * cm + jj] += ui * u[(size_t)jj * cm + k];
      }
    }
  }

  void build(int nv, const double *pos, int nf, const uint32_t *faces, double alpha, double beta,
             const rso_solver_options &opts, const ConstraintSet &set, const std::vector<v3> &P) {
    t = set.t, o = opts;
    nd = 3 * nv;
    std::vector<int> q = set.positional_rows();
    cq = set.jacobian(P, q);
    nq = (int)cq.size();
    auto t0 = clk::now();
    check_c(rso_metric_build(nv, pos, nf, faces, alpha, beta, o.chi, o.leaf_size, o.leaf_pairs, &metric), "metric");
    seconds_build[0] = since(t0);
    if (!o.preconditioner) return;  // the operator alone
    t0 = clk::now();
    std::vector<double> fa, va;
    areas_of(*t, P, fa, va);
    const double s = (beta - 2.0) / alpha;
    check_c(rso_vfrac_build(nv, pos, va.data(), 2.0 - s, o.chi, o.leaf_size, o.leaf_pairs, &vfrac), "fractional tree");
    seconds_build[1] = since(t0);
    t0 = clk::now();
    PositionalRows pr = positional_of(set, P);
    // eps: eps_rel when every component has a positional row of its own, else eps_multi_rel
    // (translations_fixed_per_component, precond.rs:118-146)
    std::vector<char> fixed(t->ncomp, 0);
    for (const auto &row : pr.c1) {
      int comp = -1;
      bool single = true;
      for (auto [v, w] : row) {
        (void)w;
        if (comp < 0) comp = (int)t->vcomp[v];
        else if (comp != (int)t->vcomp[v]) single = false;
      }
      if (single && comp >= 0) fixed[comp] = 1;
    }
    multi = false;
    for (char f : fixed) multi = multi || !f;
    Csr K = laplacian_block(*t, P, va, multi ? o.eps_multi_rel : o.eps_rel, eps);
    lps.build(K, P, pr);
    frac_scale = 1.0 / symbol_ratio(alpha, beta);
    if (o.tp_weight > 0.0) frac_scale /= o.tp_weight;  // with_metric_weight (precond.rs:896-905)
    seconds_build[2] = since(t0);
    t0 = clk::now();
    if (o.preconditioner && o.coarse) build_coarse();
    seconds_build[3] = since(t0);
  }

  // ----- GMRES (GmresRun, RS/src/solve/gmres.rs:334-590), right preconditioning
  static constexpr size_t CHUNK = 4096;
  static double dot_(const double *a, const double *b, size_t n) {
    double tot = 0.0;
    for (size_t c = 0; c < n; c += CHUNK) {
      double s = 0.0;
      const size_t e = std::min(n, c + CHUNK);
      for (size_t i = c; i < e; ++i) s += a[i] * b[i];
      tot += s;
    }
    return tot;
  }
  // w -= h v, then (w . next) over the same chunks
  static double axpy_dot(double *w, double h, const double *v, const double *next, size_t n) {
    double tot = 0.0;
    for (size_t c = 0; c < n; c += CHUNK) {
      const size_t e = std::min(n, c + CHUNK);
      for (size_t i = c; i < e; ++i) w[i] -= h * v[i];
      if (next) {
        double s = 0.0;
        for (size_t i = c; i < e; ++i) s += w[i] * next[i];
        tot += s;
      }
    }
    return tot;
  }

  void gmres(const double *b, double *x, double *rep5) {
    auto t0 = clk::now();
    const size_t n = dim();
    const int mres = std::min<int>(o.restart, (int)std::max<size_t>(n, 1));
    std::fill(x, x + n, 0.0);
    const double bnorm = std::sqrt(dot_(b, b, n));
    int iterations = 0, cycles = 0;
    bool converged = false;
    double true_rel = 0.0;
    if (bnorm == 0.0) {
      rep5[0] = 0, rep5[1] = 0, rep5[2] = 1, rep5[3] = since(t0), rep5[4] = 0;
      return;
    }
    std::vector<std::vector<double>> basis;
    std::vector<std::vector<double>> h;
    std::vector<double> cs(mres), sn(mres), g(mres + 1), r(n), w(n), z(n), u(n);
    for (;;) {
      // explicit residual r = b - A x (x = 0 in the first cycle)
      if (cycles > 0) {
        std::vector<double> full(n);
        apply(1, x, full.data());
        for (size_t i = 0; i < n; ++i) r[i] = b[i] - full[i];
      } else {
        std::copy(b, b + n, r.begin());
      }
      const double beta = std::sqrt(dot_(r.data(), r.data(), n));
      true_rel = beta / bnorm;
      if (!std::isfinite(true_rel)) break;
      if (true_rel <= o.tolerance) {
        converged = true;
        break;
      }
      if (iterations >= o.max_iterations) break;
      ++cycles;
      basis.assign(1, std::vector<double>(n));
      for (size_t i = 0; i < n; ++i) basis[0][i] = r[i] / beta;
      h.clear();
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int j = 0, k = 0;
      for (;;) {
        precondition(1, basis[j].data(), z.data());
        apply(1, z.data(), w.data());
        std::vector<double> col(j + 2, 0.0);
        double hij = dot_(w.data(), basis[0].data(), n);
        for (int i = 0; i <= j; ++i) {
          col[i] = hij;
          hij = axpy_dot(w.data(), col[i], basis[i].data(), i < j ? basis[i + 1].data() : nullptr, n);
        }
        const double hn = std::sqrt(dot_(w.data(), w.data(), n));
        col[j + 1] = hn;
        for (int i = 0; i < j; ++i) {
          double tt = cs[i] * col[i] + sn[i] * col[i + 1];
          col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1];
          col[i] = tt;
        }
        const double denom = std::hypot(col[j], col[j + 1]);
        if (denom == 0.0) cs[j] = 1.0, sn[j] = 0.0;
        else cs[j] = col[j] / denom, sn[j] = col[j + 1] / denom;
        col[j] = denom;
        col[j + 1] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] *= cs[j];
        h.push_back(col);
        ++iterations;
        const double est = std::fabs(g[j + 1]) / bnorm;
        if (hn == 0.0 || !std::isfinite(hn) || est <= o.tolerance || iterations >= o.max_iterations || j + 1 >= mres) {
          k = j + 1;
          break;
        }
        basis.push_back(std::vector<double>(n));
        for (size_t i = 0; i < n; ++i) basis[j + 1][i] = w[i] / hn;
        ++j;
      }
      // back substitution and the update x += P^-1 (V y)
      std::vector<double> y(k, 0.0);
      for (int i = k - 1; i >= 0; --i) {
        double s = g[i];
        for (int l = i + 1; l < k; ++l) s -= h[l][i] * y[l];
        y[i] = h[i][i] != 0.0 ? s / h[i][i] : 0.0;
      }
      std::fill(u.begin(), u.end(), 0.0);
      for (int l = 0; l < k; ++l)
        for (size_t i = 0; i < n; ++i) u[i] += y[l] * basis[l][i];
      precondition(1, u.data(), z.data());
      for (size_t i = 0; i < n; ++i) x[i] += z[i];
    }
    rep5[0] = iterations, rep5[1] = true_rel, rep5[2] = converged ? 1 : 0, rep5[3] = since(t0), rep5[4] = cycles;
    if (!converged && !(true_rel <= 1e-1))  // DIVERGENCE_THRESHOLD (gmres.rs:196)
      fail(RSO_SOLVER_DIVERGED, "SolverDiverged: true relative residual " + std::to_string(true_rel));
  }

  void solve_many(int nb, const double *rhs, double *sol, double *rep5) override {
    const int n = dim();
    double tmp[5];
    for (int q = 0; q < nb; ++q) gmres(rhs + (size_t)q * n, sol + (size_t)q * n, rep5 ? rep5 + 5 * q : tmp);
  }
};

// ------------------------------------------------------------------ Schur complement

constexpr double SCHUR_DROP_TOLERANCE = 1e-10;  // schur.rs:33

// SchurComplement (RS/src/solve/schur.rs:37-356): Z = A'^-1 C_N^T (position block), S = -C_N Z,
// N = -(S + S^T)/2 equilibrated and factored by Cholesky with diagonal pivoting and row drop.
struct Schur {
  int nd = 0, k = 0;
  std::vector<SparseRow> c;
  std::vector<std::vector<double>> z;
  std::vector<double> s, l, d;
  std::vector<int> kept;

  void from_solutions(int nd_, std::vector<SparseRow> c_, std::vector<std::vector<double>> z_) {
    nd = nd_, c = std::move(c_), z = std::move(z_), k = (int)c.size();
    s.assign((size_t)k * k, 0.0);
    for (int r = 0; r < k; ++r)
      for (int q = 0; q < k; ++q) {
        double acc = 0.0;
        for (size_t p = 0; p < c[r].idx.size(); ++p) acc += c[r].val[p] * z[q][c[r].idx[p]];
        s[(size_t)r * k + q] = -acc;
      }
    factor();
  }
  void factor() {  // schur.rs:190-264
    auto nn = [&](int i, int j) { return -0.5 * (s[(size_t)i * k + j] + s[(size_t)j * k + i]); };
    d.assign(k, 1.0);
    for (int i = 0; i < k; ++i) {
      double nii = nn(i, i);
      d[i] = nii > 0.0 && std::isfinite(nii) ? 1.0 / std::sqrt(nii) : 0.0;
    }
    std::vector<double> w((size_t)k * k);
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < k; ++j) w[(size_t)i * k + j] = nn(i, j) * d[i] * d[j];
    std::vector<int> remaining;
    for (int i = 0; i < k; ++i)
      if (d[i] > 0.0) remaining.push_back(i);
    std::vector<std::vector<double>> lcols;
    kept.clear();
    while (!remaining.empty()) {
      size_t pos = 0;
      for (size_t a = 1; a < remaining.size(); ++a)
        if (!(w[(size_t)remaining[pos] * k + remaining[pos]] >= w[(size_t)remaining[a] * k + remaining[a]])) pos = a;
      const int p = remaining[pos];
      const double piv = w[(size_t)p * k + p];
      if (!(piv > SCHUR_DROP_TOLERANCE)) break;
      remaining.erase(remaining.begin() + pos);
      const double sq = std::sqrt(piv);
      std::vector<double> col(k, 0.0);
      col[p] = sq;
      for (int i : remaining) col[i] = w[(size_t)i * k + p] / sq;
      for (int i : remaining)
        for (int j : remaining) w[(size_t)i * k + j] -= col[i] * col[j];
      kept.push_back(p);
      lcols.push_back(col);
    }
    const int m = (int)kept.size();
    l.assign((size_t)m * m, 0.0);
    for (int b = 0; b < m; ++b)
      for (int a = 0; a < m; ++a) l[(size_t)a * m + b] = lcols[b][kept[a]];
  }
  std::vector<double> solve_n(const std::vector<double> &v) const {  // schur.rs:268-292
    const int m = (int)kept.size();
    std::vector<double> y(m);
    for (int a = 0; a < m; ++a) y[a] = d[kept[a]] * v[kept[a]];
    for (int a = 0; a < m; ++a) {
      double sum = y[a];
      for (int b = 0; b < a; ++b) sum -= l[(size_t)a * m + b] * y[b];
      y[a] = sum / l[(size_t)a * m + a];
    }
    for (int a = m - 1; a >= 0; --a) {
      double sum = y[a];
      for (int b = a + 1; b < m; ++b) sum -= l[(size_t)b * m + a] * y[b];
      y[a] = sum / l[(size_t)a * m + a];
    }
    std::vector<double> out(k, 0.0);
    for (int a = 0; a < m; ++a) out[kept[a]] = d[kept[a]] * y[a];
    return out;
  }
  std::vector<double> combine(const std::vector<double> &cv) const {
    std::vector<double> out(nd, 0.0);
    for (int r = 0; r < k; ++r)
      if (cv[r] != 0.0)
        for (int i = 0; i < nd; ++i) out[i] += cv[r] * z[r][i];
    return out;
  }
  std::vector<double> apply_c(const std::vector<double> &v) const {
    std::vector<double> out(k, 0.0);
    for (int r = 0; r < k; ++r) {
      double acc = 0.0;
      for (size_t p = 0; p < c[r].idx.size(); ++p) acc += c[r].val[p] * v[c[r].idx[p]];
      out[r] = acc;
    }
    return out;
  }
  std::vector<double> direction_from(const std::vector<double> &y) const {  // schur.rs:320-344
    std::vector<double> cvec = solve_n(apply_c(y));
    std::vector<double> zc = combine(cvec);
    std::vector<double> x(nd);
    for (int i = 0; i < nd; ++i) x[i] = y[i] - zc[i];
    return x;
  }
  std::vector<double> correction(const std::vector<double> &phi) const { return combine(solve_n(phi)); }
};

// SchurComplement::with_direction (schur.rs:101-126): the k Schur columns and y = A'^-1 g as one
// batch of k + 1 solves.
Schur schur_with_direction(Saddle &sv, const std::vector<SparseRow> &cn, const std::vector<double> &g,
                           std::vector<double> &x, std::vector<double> *rep) {
  const int nd = sv.nd, n = sv.dim(), k = (int)cn.size(), nb = k + 1;
  std::vector<double> rhs((size_t)nb * n, 0.0), sol((size_t)nb * n), rep5(5 * nb);
  for (int r = 0; r < k; ++r)
    for (size_t p = 0; p < cn[r].idx.size(); ++p) rhs[(size_t)r * n + cn[r].idx[p]] = cn[r].val[p];
  std::copy(g.begin(), g.end(), rhs.begin() + (size_t)k * n);
  sv.solve_many(nb, rhs.data(), sol.data(), rep5.data());
  std::vector<std::vector<double>> z(k);
  for (int r = 0; r < k; ++r) z[r].assign(sol.begin() + (size_t)r * n, sol.begin() + (size_t)r * n + nd);
  Schur s;
  s.from_solutions(nd, cn, std::move(z));
  std::vector<double> y(sol.begin() + (size_t)k * n, sol.begin() + (size_t)k * n + nd);
  x = s.direction_from(y);
  if (rep) *rep = rep5;
  return s;
}

// ------------------------------------------------------------------ the step

// The objective: the exact energy, or Barnes-Hut on lists frozen at the step's start
// (Objective::build/evaluate, RS/src/step/objective.rs:71-249).
struct Objective {
  int nv = 0, nf = 0;
  const uint32_t *faces = nullptr;
  double alpha = 6, beta = 12;
  rso_bh *bh = nullptr;
  ~Objective() {
    if (bh) rso_bh_free(bh);
  }
  void build(int nv_, int nf_, const uint32_t *f, const double *pos, const rso_step_options &o, double a, double b) {
    nv = nv_, nf = nf_, faces = f, alpha = a, beta = b;
    if (o.energy_theta >= 0.0) check_c(rso_bh_build(nv, pos, nf, faces, o.energy_theta, o.leaf_size, &bh), "objective");
  }
  double value_and_gradient(const double *pos, double *g) {
    double e = 0.0;
    if (bh) check_c(rso_bh_energy_and_differential(bh, alpha, beta, &e, g, nullptr), "energy");
    else check_c(rso_exact_energy(nv, pos, nf, faces, alpha, beta, &e, g, nullptr), "energy");
    return e;
  }
  // value only; geometric failures become NaN (session.rs:1466-1479)
  double value(const std::vector<v3> &p) {
    std::vector<double> flat(3 * (size_t)nv);
    for (int v = 0; v < nv; ++v)
      for (int k = 0; k < 3; ++k) flat[3 * (size_t)v + k] = p[v][k];
    for (double x : flat)
      if (!std::isfinite(x)) return NAN;
    double e = NAN;
    int rc = bh ? (rso_bh_refit(bh, flat.data()) == 0 ? rso_bh_energy(bh, alpha, beta, &e) : 1)
                : rso_exact_energy(nv, flat.data(), nf, faces, alpha, beta, &e, nullptr, nullptr);
    if (rc != 0) return NAN;
    return e;
  }
};

struct StepOut {
  double f0 = 0, slope = 0, xnorm = 0, xinf = 0, l0 = 0, tau0 = 0, tau = 0, energy_trial = 0, energy_after = 0, gnorm = 0;
  int accepted = 0, halvings = 0, rounds = 0, status = 0, blocked = 0;
  std::vector<double> trials;  // tau, energy, outcome per trial
  std::vector<double> phi_before, phi_after, x, g;
  std::vector<v3> pos;
  std::vector<double> solve_rep;
  double seconds[7] = {0, 0, 0, 0, 0, 0, 0};
  int64_t operator_apps = 0, prec_apps = 0;
};

struct ProjectionResult {
  std::vector<v3> pos;
  std::vector<double> phi;
  int rounds = 0, status = 0;  // 0 converged, 1 max rounds, 2 not improving, 3 blocked
};

// project (RS/src/solve/schur.rs:499-575)
ProjectionResult project(const ConstraintSet &set, const Schur *schur, const std::vector<int> &nrows,
                         const std::vector<v3> &positions, int newton_fixed, int newton_max) {
  ProjectionResult out;
  std::vector<v3> pos = positions;
  set.project_positional(pos);
  std::vector<int> kept;
  if (schur) {
    kept = schur->kept;
    std::sort(kept.begin(), kept.end());
  }
  std::vector<double> tol;
  for (int r : nrows) tol.push_back(set.tolerance(r));
  auto measure = [&](const std::vector<double> &phi) {
    double m = 0.0;
    for (int i : kept) {
      double v = std::fabs(phi[nrows[i]]) / tol[i];
      if (std::isnan(v) || std::isnan(m)) m = NAN;
      else m = std::max(m, v);
    }
    return m;
  };
  std::vector<double> phi = set.values(pos);
  double m = measure(phi);
  int rounds = 0;
  const int cap = newton_max;
  const bool until = !newton_fixed;
  bool stopped = false;
  if (schur) {
    while (rounds < cap && !kept.empty()) {
      if (until && m <= 1.0) break;
      std::vector<double> phin;
      for (int r : nrows) phin.push_back(phi[r]);
      std::vector<double> h = schur->correction(phin);
      std::vector<v3> trial = pos;
      for (int v = 0; v < set.t->nv; ++v)
        for (int k = 0; k < 3; ++k) trial[v][k] -= h[3 * (size_t)v + k];
      set.project_positional(trial);
      std::vector<double> phit = set.values(trial);
      double mt = measure(phit);
      if (!(mt < m)) {
        stopped = true;
        break;
      }
      pos = trial, phi = phit, m = mt;
      ++rounds;
    }
  }
  out.status = (m <= 1.0 || kept.empty()) ? 0 : stopped ? 2 : 1;
  out.pos = pos, out.phi = phi, out.rounds = rounds;
  return out;
}

StepOut run_step(int nv, const double *pos_in, int nf, const uint32_t *faces, double alpha, double beta,
                 const rso_constraints *cons, const rso_step_options &o) {
  auto t_step = clk::now();
  StepOut out;
  Topo t = make_topo(nv, nf, faces);
  std::vector<v3> P = to_v3(nv, pos_in);
  validate_positions(nv, P, t.faces);
  ConstraintSet set = make_constraints(t, P, cons);
  const size_t nd = 3 * (size_t)nv;
  // 1. objective, F and dF
  auto t0 = clk::now();
  Objective obj;
  obj.build(nv, nf, faces, pos_in, o, alpha, beta);
  out.seconds[0] = since(t0);
  t0 = clk::now();
  out.g.assign(nd, 0.0);
  out.f0 = obj.value_and_gradient(pos_in, out.g.data());
  out.seconds[1] = since(t0);
  if (!std::isfinite(out.f0)) fail(RSO_NONFINITE_ENERGY, "NonFiniteEnergy at the start of the step");
  double gsq = 0.0;
  for (double x : out.g) gsq += x * x;
  out.gnorm = std::sqrt(gsq);
  // 2. the solver and the direction
  t0 = clk::now();
  std::vector<int> qrows = set.positional_rows(), nrows = set.nonlinear_rows();
  std::vector<SparseRow> cq = set.jacobian(P, qrows), cn = set.jacobian(P, nrows);
  std::unique_ptr<Saddle> solver;
  if (o.backend == 0) {
    auto ds = std::make_unique<DenseSaddle>();
    std::vector<double> a = dense_metric(nv, pos_in, nf, faces, alpha, beta, o.solver.tp_weight,
                                         o.solver.low_order ? 1.0 : 0.0);
    ds->build(a, nv, cq);
    solver = std::move(ds);
  } else {
    auto hs = std::make_unique<HSaddle>();
    hs->build(nv, pos_in, nf, faces, alpha, beta, o.solver, set, P);
    solver = std::move(hs);
  }
  out.seconds[2] = since(t0);
  t0 = clk::now();
  std::vector<double> x;
  Schur schur = schur_with_direction(*solver, cn, out.g, x, &out.solve_rep);
  out.seconds[3] = since(t0);
  out.x = x;
  double slope = 0.0, xinf = 0.0, xsq = 0.0, maxdisp = 0.0;
  for (size_t i = 0; i < nd; ++i) slope += out.g[i] * x[i], xinf = std::max(xinf, std::fabs(x[i])), xsq += x[i] * x[i];
  for (int v = 0; v < nv; ++v)
    maxdisp = std::max(maxdisp, std::sqrt(x[3 * v] * x[3 * v] + x[3 * v + 1] * x[3 * v + 1] + x[3 * v + 2] * x[3 * v + 2]));
  out.slope = slope, out.xinf = xinf, out.xnorm = std::sqrt(xsq);
  out.l0 = o.l0 > 0.0 ? o.l0 : mean_edge_length(t, P);
  // 3. line search (session.rs:936-1067), start_tau (session.rs:1604-1615)
  t0 = clk::now();
  auto start = [&](int rule, double val) {
    return rule == 0 ? val : rule == 1 ? val * out.l0 / maxdisp : 2.0 / out.xnorm;
  };
  const double tau0 = o.start_rule == 3 ? (o.previous_tau > 0.0 ? o.start_value * o.previous_tau
                                                                 : start(o.first_rule, o.first_value))
                                        : start(o.start_rule, o.start_value);
  out.tau0 = tau0;
  const double tau_min = o.tau_min_rel * out.l0 / xinf;
  // the projection guard's base measure (session.rs:965, 1458-1464): all Schur rows
  auto guard_measure = [&](const std::vector<double> &phi) {
    double m = 0.0;
    for (int r : nrows) {
      double v = std::fabs(phi[r]) / set.tolerance(r);
      if (std::isnan(v) || std::isnan(m)) m = NAN;
      else m = std::max(m, v);
    }
    return m;
  };
  const double base_measure = guard_measure(set.values(P));
  const Schur *sp = nrows.empty() ? nullptr : &schur;
  bool accepted = false;
  ProjectionResult proj;
  double e_after = NAN;
  double t_proj = 0.0;
  int base_contact = -1;
  auto check_proj = [&](const std::vector<v3> &moved, ProjectionResult &pr, double &ea) {
    pr = project(set, sp, nrows, moved, o.newton_fixed, o.newton_max);
    ea = obj.value(pr.pos);
    const bool finite = std::isfinite(ea);
    const double m_after = guard_measure(pr.phi);
    const bool admissible = finite && (!o.guard_projection || m_after <= std::max(base_measure, 1.0));
    return std::make_pair(admissible, !finite);
  };
  // limit (session.rs:1554-1602) without collision detection: half the projection's motion,
  // halved while F is not finite
  auto limit = [&](const std::vector<v3> &moved, ProjectionResult &pr, double &ea) {
    double frac = 0.5;
    bool chosen = false;
    std::vector<v3> target = pr.pos;
    for (int it = 0; it < 12 && frac > 0.0; ++it) {
      std::vector<v3> p(moved.size());
      for (size_t v = 0; v < moved.size(); ++v)
        for (int k = 0; k < 3; ++k) p[v][k] = moved[v][k] + frac * (target[v][k] - moved[v][k]);
      double e = obj.value(p);
      if (std::isfinite(e)) {
        pr.pos = p, ea = e, chosen = true;
        break;
      }
      frac *= 0.5;
    }
    if (!chosen) pr.pos = moved, ea = obj.value(moved);
    pr.phi = set.values(pr.pos);
    pr.status = 3;
  };
  int halvings = 0;
  if (slope > 0.0 && std::isfinite(tau0) && tau0 > 0.0) {
    double tau = tau0;
    for (;;) {
      if (!(tau >= tau_min) || (o.max_halvings >= 0 && halvings > o.max_halvings)) break;
      std::vector<v3> trial(nv);
      for (int v = 0; v < nv; ++v)
        for (int k = 0; k < 3; ++k) trial[v][k] = P[v][k] - tau * x[3 * (size_t)v + k];
      const double ft = obj.value(trial);
      const bool ok = std::isfinite(ft) && ft <= out.f0 - o.armijo_c * tau * slope;
      double outcome = !std::isfinite(ft) ? 2.0 : ok ? 0.0 : 1.0;  // accepted 0, armijo-failed 1, non-finite 2
      if (ok) {
        auto tp = clk::now();
        ProjectionResult pr;
        double ea;
        auto [admissible, contact] = check_proj(trial, pr, ea);
        if (admissible || !o.guard_projection) {
          t_proj += since(tp);
          out.trials.insert(out.trials.end(), {tau, ft, 0.0});
          accepted = true, proj = pr, e_after = ea, out.tau = tau, out.energy_trial = ft;
          break;
        }
        ++out.blocked;
        if (contact) {
          if (base_contact < 0) {
            ProjectionResult pb;
            double eb;
            auto [adm_b, con_b] = check_proj(P, pb, eb);
            base_contact = (!adm_b && con_b) ? 1 : 0;
          }
          if (base_contact == 1) {
            limit(trial, pr, ea);
            t_proj += since(tp);
            out.trials.insert(out.trials.end(), {tau, ft, 0.0});
            accepted = true, proj = pr, e_after = ea, out.tau = tau, out.energy_trial = ft;
            break;
          }
        }
        t_proj += since(tp);
        outcome = 3.0;  // projection blocked
      }
      out.trials.insert(out.trials.end(), {tau, std::isfinite(ft) ? ft : NAN, outcome});
      tau *= 0.5;
      ++halvings;
    }
  }
  out.halvings = halvings;
  out.seconds[4] = since(t0) - t_proj;
  // 4. projection of the accepted trial, or of the unmoved positions
  t0 = clk::now();
  if (accepted) {
    out.accepted = 1;
    std::vector<v3> trial(nv);
    for (int v = 0; v < nv; ++v)
      for (int k = 0; k < 3; ++k) trial[v][k] = P[v][k] - out.tau * x[3 * (size_t)v + k];
    out.phi_before = set.values(trial);
  } else {
    out.tau = 0.0, out.energy_trial = out.f0;
    out.phi_before = set.values(P);
    auto [adm, con] = check_proj(P, proj, e_after);
    (void)con;
    if (!adm && o.guard_projection) {
      ++out.blocked;
      limit(P, proj, e_after);
    }
  }
  out.seconds[5] = since(t0) + t_proj;
  out.pos = proj.pos, out.phi_after = proj.phi, out.rounds = proj.rounds, out.status = proj.status;
  out.energy_after = e_after;
  out.seconds[6] = since(t_step);
  if (auto *hs = dynamic_cast<HSaddle *>(solver.get())) out.operator_apps = hs->op_apps, out.prec_apps = hs->prec_apps;
  return out;
}

template <class F>
int sguard(F &&f) {
  try {
    f();
    return RSO_OK;
  } catch (const Error &e) {
    g_serr = e.what();
    return e.code;
  } catch (const std::exception &e) {
    g_serr = e.what();
    return RSO_INTERNAL;
  }
}

}  // namespace
}  // namespace rso

using namespace rso;

struct rso_hsolver {
  Topo topo;
  ConstraintSet set;
  HSaddle s;
};

extern "C" {

const char *rso_solve_last_error(void) { return g_serr.c_str(); }

rso_solver_options rso_solver_options_default(void) {
  rso_solver_options o;
  o.chi = 0.5;
  o.leaf_size = 8;
  o.leaf_pairs = 64;
  o.tp_weight = 1.0;
  o.low_order = 1;
  o.eps_rel = 1e-10;
  o.eps_multi_rel = 1e-4;
  o.preconditioner = 1;
  o.coarse = 1;
  o.restart = 30;
  o.max_iterations = 200;
  o.tolerance = 1e-6;
  return o;
}

rso_step_options rso_step_options_default(void) {
  rso_step_options o;
  o.energy_theta = -1.0;
  o.leaf_size = 8;
  o.backend = 0;
  o.solver = rso_solver_options_default();
  o.start_rule = 3;
  o.start_value = 2.0;
  o.first_rule = 1;
  o.first_value = 1.0;
  o.previous_tau = 0.0;
  o.armijo_c = 1e-2;
  o.max_halvings = -1;
  o.tau_min_rel = 1e-12;
  o.newton_fixed = 0;
  o.newton_max = 5;
  o.guard_projection = 1;
  o.l0 = 0.0;
  return o;
}

int rso_constraint_rows(int nv, const double *pos, int nf, const uint32_t *faces, const rso_constraints *c,
                        int max_rows, int *n_rows, int *kind, int *positional, double *phi, double *jac,
                        uint32_t *vcomp, int *n_comp) {
  return sguard([&] {
    Topo t = make_topo(nv, nf, faces);
    std::vector<v3> P = to_v3(nv, pos);
    validate_positions(nv, P, t.faces);
    ConstraintSet set = make_constraints(t, P, c);
    const int nr = (int)set.rows.size();
    *n_rows = nr;
    if (n_comp) *n_comp = t.ncomp;
    if (vcomp) std::copy(t.vcomp.begin(), t.vcomp.end(), vcomp);
    if (nr > max_rows) fail(RSO_INVALID_OPTION, "more rows than max_rows");
    std::vector<double> ph = set.values(P);
    std::vector<int> all(nr);
    std::iota(all.begin(), all.end(), 0);
    std::vector<SparseRow> j = set.jacobian(P, all);
    for (int r = 0; r < nr; ++r) {
      kind[r] = set.rows[r].kind;
      positional[r] = set.positional(r);
      phi[r] = ph[r];
      if (jac) {
        std::fill(jac + (size_t)r * 3 * nv, jac + (size_t)(r + 1) * 3 * nv, 0.0);
        for (size_t p = 0; p < j[r].idx.size(); ++p) jac[(size_t)r * 3 * nv + j[r].idx[p]] += j[r].val[p];
      }
    }
  });
}

int rso_dense_saddle(int nv, const double *pos, int nf, const uint32_t *faces, double alpha, double beta,
                     double tp_weight, int low_order, const rso_constraints *c, int max_rows, int *kq, int *kn,
                     double *g, double *x, double *S, double *phin, double *h, double *gx) {
  return sguard([&] {
    Topo t = make_topo(nv, nf, faces);
    std::vector<v3> P = to_v3(nv, pos);
    validate_positions(nv, P, t.faces);
    ConstraintSet set = make_constraints(t, P, c);
    std::vector<int> q = set.positional_rows(), nl = set.nonlinear_rows();
    *kq = (int)q.size(), *kn = (int)nl.size();
    if ((int)nl.size() > max_rows) fail(RSO_INVALID_OPTION, "more rows than max_rows");
    double e;
    std::vector<double> gg(3 * (size_t)nv);
    check_c(rso_exact_energy(nv, pos, nf, faces, alpha, beta, &e, gg.data(), nullptr), "energy");
    DenseSaddle ds;
    ds.build(dense_metric(nv, pos, nf, faces, alpha, beta, tp_weight, low_order ? 1.0 : 0.0), nv, set.jacobian(P, q));
    std::vector<double> xx;
    Schur s = schur_with_direction(ds, set.jacobian(P, nl), gg, xx, nullptr);
    std::vector<double> ph = set.values(P), pn;
    for (int r : nl) pn.push_back(ph[r]);
    std::vector<double> hh = s.correction(pn);
    double gxs = 0.0;
    for (size_t i = 0; i < gg.size(); ++i) gxs += gg[i] * xx[i];
    std::copy(gg.begin(), gg.end(), g);
    std::copy(xx.begin(), xx.end(), x);
    std::copy(s.s.begin(), s.s.end(), S);
    std::copy(pn.begin(), pn.end(), phin);
    std::copy(hh.begin(), hh.end(), h);
    *gx = gxs;
  });
}

int rso_dense_precond(int nv, const double *pos, int nf, const uint32_t *faces, double alpha, double beta,
                      double eps_rel, const rso_constraints *c, const double *r, double *eps, double *lfr, double *lp,
                      double *z, int *kq) {
  return sguard([&] {
    Topo t = make_topo(nv, nf, faces);
    std::vector<v3> P = to_v3(nv, pos);
    validate_positions(nv, P, t.faces);
    ConstraintSet set = make_constraints(t, P, c);
    std::vector<int> q = set.positional_rows();
    std::vector<SparseRow> cq = set.jacobian(P, q);
    const int nq = (int)cq.size(), nd = 3 * nv, n = nd + nq;
    *kq = nq;
    // L_{2-s} over face pairs, kernel rho^-(2 tau + 2), tau = 2 - s, in the kernel-matrix form
    // 2 Mavg^T (diag(K 1) - K) Mavg with K_ST = a_S a_T rho_ST^-(2 tau + 2), S != T
    // (fractional_operator, RS/src/metric/dense.rs:453-467)
    FaceGeometry fg = face_geometry(P, t.faces);
    const double s = (beta - 2.0) / alpha, tau = 2.0 - s, ex = -(2.0 * tau + 2.0) / 2.0;
    std::vector<double> kk((size_t)nf * nf, 0.0), k1(nf, 0.0);
    for (int a = 0; a < nf; ++a)
      for (int b = 0; b < nf; ++b) {
        if (a == b) continue;
        v3 d = sub(fg.barycenters[a], fg.barycenters[b]);
        double w = fg.areas[a] * fg.areas[b] * std::pow(dot(d, d), ex);
        kk[(size_t)a * nf + b] = w;
        k1[a] += w;
      }
    std::vector<double> L((size_t)nv * nv, 0.0);
    for (int a = 0; a < nf; ++a)
      for (int b = 0; b < nf; ++b) {
        double m = (a == b ? k1[a] : 0.0) - kk[(size_t)a * nf + b];
        if (m == 0.0) continue;
        for (uint32_t va : t.faces[a])
          for (uint32_t vb : t.faces[b]) L[(size_t)va * nv + vb] += 2.0 * m / 9.0;
      }
    std::copy(L.begin(), L.end(), lfr);
    // L' dense
    std::vector<double> fa, va;
    areas_of(t, P, fa, va);
    Csr K = laplacian_block(t, P, va, eps_rel, *eps);
    std::vector<double> m((size_t)n * n, 0.0);
    for (int v = 0; v < nv; ++v)
      for (int64_t p = K.ptr[v]; p < K.ptr[v + 1]; ++p)
        for (int k = 0; k < 3; ++k) m[(size_t)(3 * v + k) * n + 3 * K.col[p] + k] = K.val[p];
    for (int rr = 0; rr < nq; ++rr)
      for (size_t p = 0; p < cq[rr].idx.size(); ++p) {
        m[(size_t)(nd + rr) * n + cq[rr].idx[p]] += cq[rr].val[p];
        m[(size_t)cq[rr].idx[p] * n + nd + rr] += cq[rr].val[p];
      }
    std::copy(m.begin(), m.end(), lp);
    DenseLu lu;
    lu.factor(n, m);
    // P^-1 r = L'^-1 blockdiag(L (x) I3, 0) L'^-1 r (the congruence form of the dense
    // preconditioner, RS/src/solve/dense.rs:535-600)
    std::vector<double> rv(n, 0.0);
    std::copy(r, r + nd, rv.begin());
    std::vector<double> p1 = lu.solve(rv), v2(n, 0.0);
    for (int i = 0; i < nv; ++i)
      for (int k = 0; k < 3; ++k) {
        double acc = 0.0;
        for (int j = 0; j < nv; ++j) acc += L[(size_t)i * nv + j] * p1[3 * (size_t)j + k];
        v2[3 * (size_t)i + k] = acc;
      }
    std::vector<double> zz = lu.solve(v2);
    std::copy(zz.begin(), zz.begin() + nd, z);
  });
}

int rso_step(int nv, const double *pos, int nf, const uint32_t *faces, double alpha, double beta,
             const rso_constraints *c, const rso_step_options *o, double *pos_out, double *x_out, double *g_out,
             double *report, double *trials, int max_trials, int *n_trials, double *phi_before, double *phi_after,
             int max_rows) {
  return sguard([&] {
    rso_step_options opts = o ? *o : rso_step_options_default();
    StepOut s = run_step(nv, pos, nf, faces, alpha, beta, c, opts);
    if (pos_out)
      for (int v = 0; v < nv; ++v)
        for (int k = 0; k < 3; ++k) pos_out[3 * (size_t)v + k] = s.pos[v][k];
    if (x_out) std::copy(s.x.begin(), s.x.end(), x_out);
    if (g_out) std::copy(s.g.begin(), s.g.end(), g_out);
    const int nt = (int)s.trials.size() / 3;
    if (n_trials) *n_trials = nt;
    if (trials) std::copy(s.trials.begin(), s.trials.begin() + 3 * std::min(nt, max_trials), trials);
    const int nr = (int)s.phi_after.size();
    if (nr > max_rows && (phi_before || phi_after)) fail(RSO_INVALID_OPTION, "more rows than max_rows");
    if (phi_before) std::copy(s.phi_before.begin(), s.phi_before.end(), phi_before);
    if (phi_after) std::copy(s.phi_after.begin(), s.phi_after.end(), phi_after);
    if (report) {
      double r[RSO_STEP_REPORT_LEN] = {0};
      r[0] = s.f0, r[1] = s.energy_after, r[2] = s.energy_trial, r[3] = s.tau, r[4] = s.tau0, r[5] = s.accepted;
      r[6] = s.halvings, r[7] = s.slope, r[8] = s.xnorm, r[9] = s.xinf, r[10] = s.l0, r[11] = s.rounds;
      r[12] = s.status, r[13] = s.gnorm, r[14] = nr, r[15] = s.blocked;
      for (int i = 0; i < 7; ++i) r[16 + i] = s.seconds[i];
      r[23] = (double)s.operator_apps;
      double worst = 0.0;
      int its = 0;
      for (size_t q = 0; q + 4 < s.solve_rep.size(); q += 5) its += (int)s.solve_rep[q], worst = std::max(worst, s.solve_rep[q + 1]);
      r[24] = its, r[25] = worst, r[26] = (double)s.solve_rep.size() / 5, r[27] = (double)s.prec_apps;
      std::copy(r, r + RSO_STEP_REPORT_LEN, report);
    }
  });
}

int rso_hsolver_build(int nv, const double *pos, int nf, const uint32_t *faces, double alpha, double beta,
                      const rso_solver_options *o, const rso_constraints *c, rso_hsolver **out) {
  *out = nullptr;
  return sguard([&] {
    auto h = std::make_unique<rso_hsolver>();
    h->topo = make_topo(nv, nf, faces);
    std::vector<v3> P = to_v3(nv, pos);
    validate_positions(nv, P, h->topo.faces);
    h->set = make_constraints(h->topo, P, c);
    h->set.t = &h->topo;
    h->s.build(nv, pos, nf, faces, alpha, beta, o ? *o : rso_solver_options_default(), h->set, P);
    *out = h.release();
  });
}

void rso_hsolver_free(rso_hsolver *h) { delete h; }

int rso_hsolver_dims(rso_hsolver *h, int64_t *n_dofs, int64_t *n_constraints) {
  *n_dofs = h->s.nd, *n_constraints = h->s.nq;
  return RSO_OK;
}

int rso_hsolver_set_gmres(rso_hsolver *h, int restart, int max_iterations, double tolerance) {
  h->s.o.restart = restart, h->s.o.max_iterations = max_iterations, h->s.o.tolerance = tolerance;
  return RSO_OK;
}

int rso_hsolver_apply(rso_hsolver *h, int nb, const double *xs, double *ys) {
  return sguard([&] { h->s.apply(nb, xs, ys); });
}

int rso_hsolver_precondition(rso_hsolver *h, int nb, const double *rs, double *zs) {
  return sguard([&] { h->s.precondition(nb, rs, zs); });
}

int rso_hsolver_solve(rso_hsolver *h, int nb, const double *rhs, double *sol, double *report5) {
  return sguard([&] { h->s.solve_many(nb, rhs, sol, report5); });
}

int rso_hsolver_info(rso_hsolver *h, double *out8) {
  out8[0] = h->s.eps, out8[1] = h->s.multi, out8[2] = h->s.frac_scale, out8[3] = h->s.cm;
  for (int i = 0; i < 4; ++i) out8[4 + i] = h->s.seconds_build[i];
  return RSO_OK;
}

}  // extern "C"
