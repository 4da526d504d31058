// FP64 CPU oracle of the Repulsive-Surfaces energy path -- TEST INFRASTRUCTURE ONLY.
// A restatement of the reference algorithms; see rs_oracle.h for the contract.
#include "rs_oracle.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <memory>
#include <thread>

#include "rso_internal.hpp"

namespace rso {

static thread_local std::string g_last_error;
static int g_threads = 1;

int threads() { return g_threads; }

// Static partition of [0, n) over the worker threads; each index is handled once and every
// caller writes disjoint outputs, so results never depend on the thread count.
void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)> &body) {
  int t = std::max(1, g_threads);
  if (t == 1 || n < 64) {
    body(0, n);
    return;
  }
  std::vector<std::thread> pool;
  std::atomic<int64_t> next{0};
  const int64_t chunk = std::max<int64_t>(16, n / (8 * t));
  for (int i = 0; i < t; ++i)
    pool.emplace_back([&] {
      for (;;) {
        int64_t s = next.fetch_add(chunk);
        if (s >= n) break;
        body(s, std::min(n, s + chunk));
      }
    });
  for (auto &th : pool) th.join();
}

// ---------------------------------------------------------------- kernel (RS/src/kernel.rs)

static int as_small_int(double x, double max) {  // kernel.rs:36-38
  return (x == std::trunc(x) && x > 0.0 && x <= max) ? (int)x : -1;
}

Exponents Exponents::make(double alpha, double beta) {  // kernel.rs:50-76
  if (!std::isfinite(alpha) || !std::isfinite(beta))
    throw Error(RSO_INVALID_EXPONENTS, "both exponents must be finite");
  if (alpha <= 1.0) throw Error(RSO_INVALID_EXPONENTS, "alpha must be greater than 1");
  if (beta <= alpha + 2.0)
    throw Error(RSO_INVALID_EXPONENTS,
                "beta must be greater than alpha + 2 (s = (beta - 2)/alpha > 1)");
  if (beta >= 2.0 * alpha + 2.0)
    throw Error(RSO_INVALID_EXPONENTS,
                "beta must be smaller than 2 alpha + 2 (s = (beta - 2)/alpha < 2)");
  Exponents e;
  e.alpha = alpha;
  e.beta = beta;
  e.alpha_int = as_small_int(alpha, 64.0);
  e.beta_int = as_small_int(beta, 128.0);
  return e;
}

double ipow(double x, uint32_t n) {  // kernel.rs:180-193
  double acc = 1.0;
  while (n > 0) {
    if (n & 1) acc *= x;
    n >>= 1;
    if (n > 0) x *= x;
  }
  return acc;
}

void Exponents::nu_powers(double nu, double &pa, double &sp) const {  // kernel.rs:144-152
  double a = std::fabs(nu);
  double p1 = alpha_int >= 0 ? ipow(a, (uint32_t)(alpha_int - 1)) : std::pow(a, alpha - 1.0);
  pa = p1 * a;
  sp = std::copysign(p1, nu);
}

double Exponents::r_power(double r2) const {  // kernel.rs:155-162
  if (beta_int >= 0) {
    uint32_t k = (uint32_t)beta_int;
    if (k % 2 == 0) return 1.0 / ipow(r2, k / 2);
    return 1.0 / (ipow(r2, k / 2) * std::sqrt(r2));
  }
  return std::pow(r2, -0.5 * beta);
}

double kernel_of_v(const Exponents &e, v3 v, v3 n) {  // kernel.rs:206-210
  double pa, sp;
  e.nu_powers(dot(n, v), pa, sp);
  return pa * e.r_power(dot(v, v));
}

KernelEval kernel_with_gradient_of_v(const Exponents &e, v3 v, v3 n) {  // kernel.rs:238-250
  double r2 = dot(v, v);
  double rb = e.r_power(r2);
  double pa, sp1;
  e.nu_powers(dot(n, v), pa, sp1);
  double value = pa * rb;
  double c_n = e.alpha * sp1 * rb;
  KernelEval k;
  k.value = value;
  k.d_v = axpy(scale(n, c_n), -e.beta * value / r2, v);
  k.d_n = scale(v, c_n);
  return k;
}

void pair_terms(const Exponents &e, v3 v, v3 n_s, v3 n_t, double &k_st, double &k_ts, v3 &dv_st,
                v3 &dv_ts, v3 &dn_st) {  // kernel.rs:256-275
  double r2 = dot(v, v);
  double rb = e.r_power(r2);
  double pa_s, sp_s, pa_t, sp_t;
  e.nu_powers(dot(n_s, v), pa_s, sp_s);
  e.nu_powers(-dot(n_t, v), pa_t, sp_t);
  k_st = pa_s * rb;
  k_ts = pa_t * rb;
  double c_s = e.alpha * sp_s * rb;
  double c_t = e.alpha * sp_t * rb;
  double inv_r2 = 1.0 / r2;
  dv_st = axpy(scale(n_s, c_s), -e.beta * k_st * inv_r2, v);
  dv_ts = axpy(scale(n_t, c_t), e.beta * k_ts * inv_r2, v);
  dn_st = scale(v, c_s);
}

// ---------------------------------------------------------------- geometry (RS/src/geometry.rs)

void face_quantities(const std::array<v3, 3> &p, double &a, v3 &n, v3 &x) {  // geometry.rs:33-39
  v3 nn = cross(sub(p[1], p[0]), sub(p[2], p[0]));
  double len = norm(nn);
  x = scale(add(add(p[0], p[1]), p[2]), 1.0 / 3.0);
  a = 0.5 * len;
  n = scale(nn, 1.0 / len);
}

static std::array<v3, 3> opposite_edges(const std::array<v3, 3> &p) {  // geometry.rs:43-45
  return {sub(p[2], p[1]), sub(p[0], p[2]), sub(p[1], p[0])};
}

std::array<v3, 3> face_pull_back(const std::array<v3, 3> &p, double d_area, v3 d_bary,
                                 v3 d_normal) {  // geometry.rs:87-110
  v3 n = cross(sub(p[1], p[0]), sub(p[2], p[0]));
  double len = norm(n);
  v3 nrm = scale(n, 1.0 / len);
  auto e = opposite_edges(p);
  v3 xb = scale(d_bary, 1.0 / 3.0);
  double inv_2a = 1.0 / len;
  std::array<v3, 3> out;
  for (int c = 0; c < 3; ++c) {
    v3 ga = scale(cross(nrm, e[c]), 0.5 * d_area);
    v3 gn = scale(nrm, dot(cross(e[c], nrm), d_normal) * inv_2a);
    out[c] = add(add(ga, xb), gn);
  }
  return out;
}

std::array<v3, 3> corners(const std::vector<v3> &pos, const tri &t) {
  return {pos[t[0]], pos[t[1]], pos[t[2]]};
}

void validate_positions(int nv, const std::vector<v3> &pos, const std::vector<tri> &faces) {
  if ((int)pos.size() != nv) throw Error(RSO_POSITION_COUNT, "position count mismatch");
  for (int v = 0; v < nv; ++v)
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(pos[v][k]))
        throw Error(RSO_NONFINITE_POSITION, "vertex " + std::to_string(v) + " is not finite");
  for (size_t f = 0; f < faces.size(); ++f) {
    for (int c = 0; c < 3; ++c)
      if ((int)faces[f][c] >= nv) throw Error(RSO_TOPOLOGY, "vertex out of range");
    double a;
    v3 n, x;
    face_quantities(corners(pos, faces[f]), a, n, x);
    bool ok = a > 0.0 && std::isfinite(a) && std::isfinite(n[0]) && std::isfinite(n[1]) &&
              std::isfinite(n[2]);
    if (!ok)
      throw Error(RSO_DEGENERATE_FACE, "face " + std::to_string(f) + " has zero area");
  }
}

FaceGeometry face_geometry(const std::vector<v3> &pos, const std::vector<tri> &faces) {
  FaceGeometry g;
  size_t nf = faces.size();
  g.areas.resize(nf);
  g.normals.resize(nf);
  g.barycenters.resize(nf);
  for (size_t f = 0; f < nf; ++f)
    face_quantities(corners(pos, faces[f]), g.areas[f], g.normals[f], g.barycenters[f]);
  return g;
}

std::vector<v3> pull_back(int nv, const std::vector<v3> &pos, const std::vector<tri> &faces,
                          const std::vector<double> &da, const std::vector<v3> &dx,
                          const std::vector<v3> &dn) {  // geometry.rs:172-188
  std::vector<v3> out(nv, v3{0, 0, 0});
  for (size_t f = 0; f < faces.size(); ++f) {
    auto g = face_pull_back(corners(pos, faces[f]), da[f], dx[f], dn[f]);
    for (int c = 0; c < 3; ++c) out[faces[f][c]] = add(out[faces[f][c]], g[c]);
  }
  return out;
}

// ---------------------------------------------------------------- BVH (RC/src/spatial/bvh.rs)

// f64::total_cmp (used by the split sort, bvh.rs:165-169) as a key order.
static inline int64_t total_key(double x) {
  int64_t b;
  std::memcpy(&b, &x, 8);
  return b ^ (int64_t)(((uint64_t)(b >> 63)) >> 1);
}

Bvh Bvh::build(const std::vector<Element> &el, int leaf_size, double min_fraction) {
  // bvh.rs:126-220: top down, axis = depth mod 3, elements sorted by that coordinate (ties by
  // index), split minimising diam^2(prefix) + diam^2(suffix) with >= ceil(f n) per side,
  // nodes in pre-order, left child = i + 1.
  if (leaf_size <= 0) throw Error(RSO_INVALID_OPTION, "leaf_size must be at least 1");
  if (el.empty()) throw Error(RSO_INVALID_OPTION, "at least 1 element");
  size_t n = el.size();
  Bvh b;
  b.leaf_size = leaf_size;
  b.order.resize(n);
  for (size_t i = 0; i < n; ++i) b.order[i] = (uint32_t)i;
  struct Item {
    size_t start, end, depth;
    uint32_t patch;
  };
  std::vector<Item> stack{{0, n, 0, UINT32_MAX}};
  std::vector<Aabb> suffix;
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    uint32_t id = (uint32_t)b.nodes.size();
    if (it.patch != UINT32_MAX) b.nodes[it.patch].right = id;
    Node nd;
    nd.start = (uint32_t)it.start;
    nd.end = (uint32_t)it.end;
    b.nodes.push_back(nd);
    size_t cnt = it.end - it.start;
    if (cnt <= (size_t)leaf_size) continue;
    int axis = (int)(it.depth % 3);
    uint32_t *sl = b.order.data() + it.start;
    std::sort(sl, sl + cnt, [&](uint32_t a, uint32_t c) {
      int64_t ka = total_key(el[a].point[axis]), kc = total_key(el[c].point[axis]);
      if (ka != kc) return ka < kc;
      return a < c;
    });
    suffix.assign(cnt, Aabb());
    Aabb acc;
    for (size_t k = cnt; k-- > 0;) {
      acc = acc.uni(el[sl[k]].bounds);
      suffix[k] = acc;
    }
    Aabb prefix;
    double best_cost = INFINITY;
    size_t best_k = cnt / 2;
    size_t lo = (size_t)std::ceil(min_fraction * (double)cnt);
    lo = std::min(std::max<size_t>(lo, 1), cnt / 2);
    for (size_t k = 1; k <= cnt - lo; ++k) {
      prefix = prefix.uni(el[sl[k - 1]].bounds);
      if (k < lo) continue;
      double cost = prefix.diameter_sq() + suffix[k].diameter_sq();
      if (cost < best_cost) best_cost = cost, best_k = k;
    }
    size_t split = it.start + best_k;
    stack.push_back({split, it.end, it.depth + 1, id});
    stack.push_back({it.start, split, it.depth + 1, UINT32_MAX});
  }
  b.refit(el);
  return b;
}

void Bvh::refit(const std::vector<Element> &el) {  // bvh.rs:226-260 (+ summarize 314-330)
  if (el.size() != order.size()) throw Error(RSO_INVALID_OPTION, "element count changed");
  for (size_t i = nodes.size(); i-- > 0;) {
    Node &nd = nodes[i];
    if (nd.leaf()) {
      Aabb bb;
      double mass = 0;
      v3 mom{0, 0, 0};
      for (uint32_t p = nd.start; p < nd.end; ++p) {
        const Element &e = el[order[p]];
        bb = bb.uni(e.bounds);
        mass += e.mass;
        for (int k = 0; k < 3; ++k) mom[k] += e.mass * e.point[k];
      }
      nd.bbox = bb, nd.mass = mass, nd.moment = mom;
    } else {
      const Node &l = nodes[i + 1], &r = nodes[nd.right];
      v3 mom = l.moment;
      for (int k = 0; k < 3; ++k) mom[k] += r.moment[k];
      nd.bbox = l.bbox.uni(r.bbox);
      nd.mass = l.mass + r.mass;
      nd.moment = mom;
    }
  }
}

double box_distance_sq(const Aabb &a, const Aabb &b) {  // RS/src/spatial/mod.rs:131-138
  double d2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    double d = fmax_(fmax_(a.lo[k], b.lo[k]) - fmin_(a.hi[k], b.hi[k]), 0.0);
    d2 += d * d;
  }
  return d2;
}

double farthest_corner_distance(const Aabb &b, v3 x) {  // RS/src/spatial/mod.rs:143-150
  double r2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    double d = fmax_(b.hi[k] - x[k], x[k] - b.lo[k]);
    r2 += d * d;
  }
  return std::sqrt(r2);
}

bool bh_admissible(const Cluster &leaf, const Cluster &c, double theta) {  // mod.rs:160-163
  double h = fmax_(leaf.radius, c.radius);
  return h * h < theta * theta * box_distance_sq(leaf.bbox, c.bbox);
}

std::vector<Element> face_elements(const std::vector<v3> &pos, const std::vector<tri> &faces,
                                   const FaceGeometry &g) {  // RS/src/spatial/mod.rs:56-76
  std::vector<Element> out(faces.size());
  for (size_t f = 0; f < faces.size(); ++f) {
    Aabb b;
    for (int c = 0; c < 3; ++c) b.grow(pos[faces[f][c]]);
    out[f] = {g.barycenters[f], b, g.areas[f]};
  }
  return out;
}

std::vector<std::array<double, 6>> FaceTree::projectors(const FaceGeometry &g) const {
  // RS/src/spatial/mod.rs:268-290 via Bvh::fold_up (RC/src/spatial/bvh.rs:265-284)
  size_t nn = bvh.nodes.size();
  std::vector<std::array<double, 7>> s(nn);
  for (size_t i = nn; i-- > 0;) {
    const Node &nd = bvh.nodes[i];
    std::array<double, 7> acc{};
    if (nd.leaf()) {
      for (uint32_t p = nd.start; p < nd.end; ++p) {
        uint32_t f = bvh.order[p];
        double a = g.areas[f];
        v3 n = g.normals[f];
        acc[0] += a;
        acc[1] += a * n[0] * n[0];
        acc[2] += a * n[0] * n[1];
        acc[3] += a * n[0] * n[2];
        acc[4] += a * n[1] * n[1];
        acc[5] += a * n[1] * n[2];
        acc[6] += a * n[2] * n[2];
      }
    } else {
      for (int k = 0; k < 7; ++k) acc[k] = s[i + 1][k] + s[nd.right][k];
    }
    s[i] = acc;
  }
  std::vector<std::array<double, 6>> out(nn);
  for (size_t i = 0; i < nn; ++i)
    for (int k = 0; k < 6; ++k) out[i][k] = s[i][k + 1] / s[i][0];
  return out;
}

FaceTree FaceTree::build(const std::vector<v3> &pos, const std::vector<tri> &faces,
                         const FaceGeometry &g, int leaf_size) {  // spatial/mod.rs:175-221
  FaceTree t;
  t.bvh = Bvh::build(face_elements(pos, faces, g), leaf_size);
  size_t nn = t.bvh.nodes.size();
  t.leaf_ordinal.assign(nn, UINT32_MAX);
  t.leaf_of_face.assign(faces.size(), 0);
  for (size_t n = 0; n < nn; ++n) {
    const Node &nd = t.bvh.nodes[n];
    if (nd.leaf()) {
      t.leaf_ordinal[n] = (uint32_t)t.leaves.size();
      t.leaves.push_back((uint32_t)n);
      for (uint32_t p = nd.start; p < nd.end; ++p) t.leaf_of_face[t.bvh.order[p]] = (uint32_t)n;
    }
  }
  auto pr = t.projectors(g);
  t.clusters.resize(nn);
  for (size_t n = 0; n < nn; ++n) {
    const Node &nd = t.bvh.nodes[n];
    v3 c = nd.centroid();
    t.clusters[n] = {nd.mass, c, pr[n], nd.bbox, farthest_corner_distance(nd.bbox, c)};
  }
  return t;
}

void FaceTree::refit(const std::vector<v3> &pos, const std::vector<tri> &faces,
                     const FaceGeometry &g) {  // spatial/mod.rs:241-265
  bvh.refit(face_elements(pos, faces, g));
  auto pr = projectors(g);
  for (size_t n = 0; n < clusters.size(); ++n) {
    clusters[n].area = bvh.nodes[n].mass;
    clusters[n].centroid = bvh.nodes[n].centroid();
    clusters[n].projector = pr[n];
  }
}

}  // namespace rso

// ================================================================ Barnes-Hut
using namespace rso;

namespace {

struct Lists {  // RS/src/energy/barnes_hut.rs:61-81
  std::vector<size_t> lumped_off, exact_off, partner_off, lumped_t_off, exact_t_off;
  std::vector<uint32_t> lumped, exact, lumped_t, exact_t;
  uint64_t pairs_exact = 0;
};

struct Packed {
  v3 x, n;
  double a;
};

template <class Key>
static void transpose(const std::vector<uint32_t> &entries, size_t m, Key key,
                      std::vector<size_t> &off, std::vector<uint32_t> &idx) {
  // barnes_hut.rs:811-827
  off.assign(m + 1, 0);
  for (uint32_t x : entries) off[key(x) + 1] += 1;
  for (size_t i = 0; i < m; ++i) off[i + 1] += off[i];
  std::vector<size_t> fill = off;
  idx.assign(entries.size(), 0);
  for (size_t k = 0; k < entries.size(); ++k) idx[fill[key(entries[k])]++] = (uint32_t)k;
}

static Lists build_lists(const FaceTree &tree, double theta) {  // barnes_hut.rs:743-808
  const auto &leaves = tree.leaves;
  size_t nl = leaves.size(), nn = tree.bvh.nodes.size();
  std::vector<std::vector<uint32_t>> lum(nl), ex(nl);
  parallel_for((int64_t)nl, [&](int64_t b, int64_t e) {
    std::vector<size_t> stack;
    for (int64_t k = b; k < e; ++k) {
      const Cluster &cl = tree.clusters[leaves[k]];
      stack.clear();
      stack.push_back(0);
      while (!stack.empty()) {
        size_t c = stack.back();
        stack.pop_back();
        if (bh_admissible(cl, tree.clusters[c], theta))
          lum[k].push_back((uint32_t)c);
        else if (tree.bvh.nodes[c].leaf())
          ex[k].push_back((uint32_t)c);
        else {
          stack.push_back(tree.bvh.nodes[c].right);
          stack.push_back(c + 1);
        }
      }
    }
  });
  Lists L;
  L.lumped_off.push_back(0);
  L.exact_off.push_back(0);
  size_t poff = 0;
  for (size_t k = 0; k < nl; ++k) {
    const Node &ln = tree.bvh.nodes[leaves[k]];
    uint64_t ns = ln.end - ln.start;
    for (uint32_t c : ex[k]) {
      const Node &cn = tree.bvh.nodes[c];
      uint64_t nc = cn.end - cn.start;
      L.partner_off.push_back(poff);
      poff += nc;
      L.pairs_exact += (c == leaves[k]) ? ns * (ns - 1) : ns * nc;
    }
    L.lumped.insert(L.lumped.end(), lum[k].begin(), lum[k].end());
    L.exact.insert(L.exact.end(), ex[k].begin(), ex[k].end());
    L.lumped_off.push_back(L.lumped.size());
    L.exact_off.push_back(L.exact.size());
  }
  L.partner_off.push_back(poff);
  transpose(L.lumped, nn, [](uint32_t n) { return (size_t)n; }, L.lumped_t_off, L.lumped_t);
  transpose(L.exact, nl, [&](uint32_t n) { return (size_t)tree.leaf_ordinal[n]; }, L.exact_t_off,
            L.exact_t);
  return L;
}

struct LeafOut {  // barnes_hut.rs:728-736
  double energy = 0;
  std::vector<std::array<double, 7>> own;  // (d_a, d_x[3], d_n[3])
  std::vector<std::array<double, 4>> node;     // (b, u[3])
  std::vector<std::array<double, 4>> partner;  // (d_a, d_x[3])
};

}  // namespace

struct rso_bh {
  double theta;
  int leaf_size;
  int nv;
  std::vector<tri> faces;
  std::vector<v3> positions;
  FaceGeometry geom;
  FaceTree tree;
  Lists lists;
  std::vector<Packed> packed;

  void pack() {  // barnes_hut.rs:137-147
    packed.resize(tree.bvh.order.size());
    for (size_t p = 0; p < packed.size(); ++p) {
      uint32_t f = tree.bvh.order[p];
      packed[p] = {geom.barycenters[f], geom.normals[f], geom.areas[f]};
    }
  }

  double leaf_energy(size_t k, const Exponents &e) const {  // barnes_hut.rs:583-614
    const Node &ln = tree.bvh.nodes[tree.leaves[k]];
    double energy = 0.0;
    for (size_t q = lists.lumped_off[k]; q < lists.lumped_off[k + 1]; ++q) {
      const Cluster &cl = tree.clusters[lists.lumped[q]];
      double b = 0.0;
      for (uint32_t p = ln.start; p < ln.end; ++p) {
        const Packed &fs = packed[p];
        b += fs.a * kernel_of_v(e, sub(fs.x, cl.centroid), fs.n);
      }
      energy += b * cl.area;
    }
    for (size_t q = lists.exact_off[k]; q < lists.exact_off[k + 1]; ++q) {
      const Node &cn = tree.bvh.nodes[lists.exact[q]];
      for (uint32_t ps = ln.start; ps < ln.end; ++ps) {
        const Packed &fs = packed[ps];
        double row = 0.0;
        for (uint32_t pt = cn.start; pt < cn.end; ++pt) {
          if (pt == ps) continue;
          const Packed &ft = packed[pt];
          row += ft.a * kernel_of_v(e, sub(fs.x, ft.x), fs.n);
        }
        energy += fs.a * row;
      }
    }
    return energy;
  }

  LeafOut leaf_with_gradient(size_t k, const Exponents &e) const {  // barnes_hut.rs:627-689
    const Node &ln = tree.bvh.nodes[tree.leaves[k]];
    size_t ns = ln.end - ln.start;
    LeafOut out;
    out.own.assign(ns, std::array<double, 7>{});
    for (size_t q = lists.lumped_off[k]; q < lists.lumped_off[k + 1]; ++q) {
      const Cluster &cl = tree.clusters[lists.lumped[q]];
      double ac = cl.area, b = 0.0;
      v3 u{0, 0, 0};
      for (size_t i = 0; i < ns; ++i) {
        const Packed &fs = packed[ln.start + i];
        double a_s = fs.a;
        KernelEval kv = kernel_with_gradient_of_v(e, sub(fs.x, cl.centroid), fs.n);
        b += a_s * kv.value;
        auto &o = out.own[i];
        o[0] += kv.value * ac;
        v3 ox = axpy({o[1], o[2], o[3]}, a_s * ac, kv.d_v);
        v3 on = axpy({o[4], o[5], o[6]}, a_s * ac, kv.d_n);
        o[1] = ox[0], o[2] = ox[1], o[3] = ox[2], o[4] = on[0], o[5] = on[1], o[6] = on[2];
        u = axpy(u, -a_s, kv.d_v);
      }
      out.energy += b * ac;
      out.node.push_back({b, u[0], u[1], u[2]});
    }
    for (size_t q = lists.exact_off[k]; q < lists.exact_off[k + 1]; ++q) {
      const Node &cn = tree.bvh.nodes[lists.exact[q]];
      size_t base = out.partner.size();
      out.partner.resize(base + (cn.end - cn.start), std::array<double, 4>{});
      for (size_t i = 0; i < ns; ++i) {
        uint32_t ps = ln.start + (uint32_t)i;
        const Packed &fs = packed[ps];
        double a_s = fs.a, row = 0.0;
        v3 dx{0, 0, 0}, dn{0, 0, 0};
        for (uint32_t pt = cn.start; pt < cn.end; ++pt) {
          if (pt == ps) continue;
          const Packed &ft = packed[pt];
          double a_t = ft.a;
          KernelEval kv = kernel_with_gradient_of_v(e, sub(fs.x, ft.x), fs.n);
          row += a_t * kv.value;
          dx = axpy(dx, a_t, kv.d_v);
          dn = axpy(dn, a_t, kv.d_n);
          auto &p = out.partner[base + (pt - cn.start)];
          p[0] += a_s * kv.value;
          v3 px = axpy({p[1], p[2], p[3]}, -a_s * a_t, kv.d_v);
          p[1] = px[0], p[2] = px[1], p[3] = px[2];
        }
        out.energy += a_s * row;
        auto &o = out.own[i];
        o[0] += row;
        v3 ox = axpy({o[1], o[2], o[3]}, a_s, dx);
        v3 on = axpy({o[4], o[5], o[6]}, a_s, dn);
        o[1] = ox[0], o[2] = ox[1], o[3] = ox[2], o[4] = on[0], o[5] = on[1], o[6] = on[2];
      }
    }
    return out;
  }

  double energy(const Exponents &e) const {  // barnes_hut.rs:366-375
    size_t nl = tree.leaves.size();
    std::vector<double> per(nl);
    parallel_for((int64_t)nl, [&](int64_t b, int64_t en) {
      for (int64_t k = b; k < en; ++k) per[k] = leaf_energy((size_t)k, e);
    });
    double s = 0.0;
    for (double x : per) s += x;
    return s;
  }

  // barnes_hut.rs:478-579; out7 by face.
  double face_partials(const Exponents &e, std::vector<std::array<double, 7>> &out7) const {
    const auto &leaves = tree.leaves;
    size_t nl = leaves.size(), nn = tree.clusters.size(), nf = faces.size();
    std::vector<LeafOut> outs(nl);
    parallel_for((int64_t)nl, [&](int64_t b, int64_t en) {
      for (int64_t k = b; k < en; ++k) outs[k] = leaf_with_gradient((size_t)k, e);
    });
    double energy = 0.0;
    for (auto &o : outs) energy += o.energy;
    std::vector<std::array<double, 4>> node_terms, partner;
    node_terms.reserve(lists.lumped.size());
    partner.reserve(lists.partner_off.back());
    for (auto &o : outs) {
      node_terms.insert(node_terms.end(), o.node.begin(), o.node.end());
      partner.insert(partner.end(), o.partner.begin(), o.partner.end());
    }
    // 2. node sums over the transposed lumped lists
    std::vector<std::array<double, 4>> sums(nn);
    for (size_t n = 0; n < nn; ++n) {
      double b = 0.0;
      v3 u{0, 0, 0};
      for (size_t q = lists.lumped_t_off[n]; q < lists.lumped_t_off[n + 1]; ++q) {
        const auto &t = node_terms[lists.lumped_t[q]];
        b += t[0];
        u = axpy(u, 1.0, {t[1], t[2], t[3]});
      }
      sums[n] = {b, u[0], u[1], u[2]};
    }
    // 3. downward pass (pre-order)
    std::vector<double> beta(nn, 0.0);
    std::vector<v3> ubig(nn, v3{0, 0, 0});
    if (nn > 0) beta[0] = sums[0][0], ubig[0] = {sums[0][1], sums[0][2], sums[0][3]};
    for (size_t n = 0; n < nn; ++n) {
      const Node &nd = tree.bvh.nodes[n];
      if (nd.leaf()) continue;
      size_t kids[2] = {n + 1, nd.right};
      for (size_t c : kids) {
        v3 shift = sub(tree.clusters[c].centroid, tree.clusters[n].centroid);
        beta[c] = beta[n] + dot(ubig[n], shift) + sums[c][0];
        ubig[c] = axpy(ubig[n], 1.0, {sums[c][1], sums[c][2], sums[c][3]});
      }
    }
    // 4. per leaf: own + partner + cluster
    out7.assign(nf, std::array<double, 7>{});
    parallel_for((int64_t)nl, [&](int64_t b, int64_t en) {
      for (int64_t kc = b; kc < en; ++kc) {
        uint32_t c = leaves[kc];
        const Node &cn = tree.bvh.nodes[c];
        std::vector<std::array<double, 7>> res = outs[kc].own;
        for (size_t q = lists.exact_t_off[kc]; q < lists.exact_t_off[kc + 1]; ++q) {
          size_t off = lists.partner_off[lists.exact_t[q]];
          for (size_t t = 0; t < res.size(); ++t) {
            const auto &p = partner[off + t];
            res[t][0] += p[0];
            v3 rx = axpy({res[t][1], res[t][2], res[t][3]}, 1.0, {p[1], p[2], p[3]});
            res[t][1] = rx[0], res[t][2] = rx[1], res[t][3] = rx[2];
          }
        }
        v3 xc = tree.clusters[c].centroid;
        for (size_t t = 0; t < res.size(); ++t) {
          uint32_t f = tree.bvh.order[cn.start + t];
          double a = geom.areas[f];
          v3 x = geom.barycenters[f];
          res[t][0] += beta[c] + dot(ubig[c], sub(x, xc));
          v3 rx = axpy({res[t][1], res[t][2], res[t][3]}, a, ubig[c]);
          res[t][1] = rx[0], res[t][2] = rx[1], res[t][3] = rx[2];
          out7[f] = res[t];
        }
      }
    });
    return energy;
  }
};

// ================================================================ C ABI

template <class F>
static int guard(F &&f) {
  try {
    f();
    return RSO_OK;
  } catch (const Error &e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return RSO_INTERNAL;
  }
}

static std::vector<v3> to_v3(const double *p, int n) {
  std::vector<v3> out(n);
  for (int i = 0; i < n; ++i) out[i] = {p[3 * i], p[3 * i + 1], p[3 * i + 2]};
  return out;
}
static std::vector<tri> to_tri(const uint32_t *f, int n) {
  std::vector<tri> out(n);
  for (int i = 0; i < n; ++i) out[i] = {f[3 * i], f[3 * i + 1], f[3 * i + 2]};
  return out;
}

// The first ordered pair whose term or gradient is non-finite (exact.rs:165-186 /
// barnes_hut.rs:693-724) is reported in the message.
static void non_finite(const char *what) {
  throw Error(RSO_NONFINITE_ENERGY, std::string("non-finite ") + what);
}

extern "C" {

const char *rso_last_error(void) { return g_last_error.c_str(); }
void rso_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

int rso_exponents_check(double alpha, double beta) {
  return guard([&] { Exponents::make(alpha, beta); });
}

int rso_face_geometry(int nv, const double *pos, int nf, const uint32_t *faces,
                      double *out_area, double *out_normal, double *out_bary) {
  return guard([&] {
    auto P = to_v3(pos, nv);
    auto T = to_tri(faces, nf);
    validate_positions(nv, P, T);
    FaceGeometry g = face_geometry(P, T);
    for (int f = 0; f < nf; ++f) {
      out_area[f] = g.areas[f];
      for (int k = 0; k < 3; ++k)
        out_normal[3 * f + k] = g.normals[f][k], out_bary[3 * f + k] = g.barycenters[f][k];
    }
  });
}

int rso_exact_energy(int nv, const double *pos, int nf, const uint32_t *faces, double alpha,
                     double beta, double *energy, double *dE, double *fp7) {
  return guard([&] {
    Exponents e = Exponents::make(alpha, beta);
    auto P = to_v3(pos, nv);
    auto T = to_tri(faces, nf);
    validate_positions(nv, P, T);
    FaceGeometry g = face_geometry(P, T);
    if (!dE && !fp7) {  // exact.rs:61-78, value only
      std::vector<double> rows(nf);
      parallel_for(nf, [&](int64_t b, int64_t en) {
        for (int64_t s = b; s < en; ++s) {
          double acc = 0.0;
          for (int t = 0; t < nf; ++t)
            if (t != s)
              acc += g.areas[t] * kernel_of_v(e, sub(g.barycenters[s], g.barycenters[t]),
                                              g.normals[s]);
          rows[s] = g.areas[s] * acc;
        }
      });
      double s = 0.0;
      for (double r : rows) s += r;
      *energy = s;
      return;
    }
    // exact.rs:87-134
    std::vector<double> da(nf), en(nf);
    std::vector<v3> dx(nf), dn(nf);
    parallel_for(nf, [&](int64_t b, int64_t end) {
      for (int64_t s = b; s < end; ++s) {
        v3 xs = g.barycenters[s], ns = g.normals[s];
        double a_s = g.areas[s], e_row = 0.0, d_a = 0.0;
        v3 d_x{0, 0, 0}, d_n{0, 0, 0};
        for (int t = 0; t < nf; ++t) {
          if (t == s) continue;
          double a_t = g.areas[t], k_st, k_ts;
          v3 dv_st, dv_ts, dn_st;
          pair_terms(e, sub(xs, g.barycenters[t]), ns, g.normals[t], k_st, k_ts, dv_st, dv_ts,
                     dn_st);
          e_row += a_t * k_st;
          d_a += a_t * (k_st + k_ts);
          d_x = axpy(d_x, a_t, sub(dv_st, dv_ts));
          d_n = axpy(d_n, a_t, dn_st);
        }
        en[s] = a_s * e_row;
        da[s] = d_a;
        dx[s] = scale(d_x, a_s);
        dn[s] = scale(d_n, a_s);
      }
    });
    double E = 0.0;
    for (double x : en) E += x;
    std::vector<v3> G = pull_back(nv, P, T, da, dx, dn);
    bool finite = std::isfinite(E);
    for (auto &v : G)
      for (double x : v) finite = finite && std::isfinite(x);
    if (!finite) non_finite("exact energy (coincident barycenters)");
    *energy = E;
    if (dE)
      for (int v = 0; v < nv; ++v)
        for (int k = 0; k < 3; ++k) dE[3 * v + k] = G[v][k];
    if (fp7)
      for (int f = 0; f < nf; ++f) {
        fp7[7 * f] = da[f];
        for (int k = 0; k < 3; ++k) fp7[7 * f + 1 + k] = dx[f][k], fp7[7 * f + 4 + k] = dn[f][k];
      }
  });
}

int rso_bh_build(int nv, const double *pos, int nf, const uint32_t *faces, double theta,
                 int leaf_size, rso_bh **out) {
  *out = nullptr;
  return guard([&] {
    if (!(std::isfinite(theta) && theta >= 0.0))
      throw Error(RSO_INVALID_OPTION, "theta must be finite and non-negative");
    if (leaf_size < 1) throw Error(RSO_INVALID_OPTION, "leaf_size must be at least 1");
    auto h = std::make_unique<rso_bh>();
    h->theta = theta;
    h->leaf_size = leaf_size;
    h->nv = nv;
    h->positions = to_v3(pos, nv);
    h->faces = to_tri(faces, nf);
    validate_positions(nv, h->positions, h->faces);
    h->geom = face_geometry(h->positions, h->faces);
    h->tree = FaceTree::build(h->positions, h->faces, h->geom, leaf_size);
    h->lists = build_lists(h->tree, theta);
    h->pack();
    *out = h.release();
  });
}

void rso_bh_free(rso_bh *h) { delete h; }

int rso_bh_refit(rso_bh *h, const double *pos) {
  return guard([&] {  // barnes_hut.rs:204-229
    auto P = to_v3(pos, h->nv);
    for (int v = 0; v < h->nv; ++v)
      for (int k = 0; k < 3; ++k)
        if (!std::isfinite(P[v][k])) throw Error(RSO_NONFINITE_POSITION, "non-finite position");
    h->positions = P;
    h->geom = face_geometry(P, h->faces);
    h->pack();
    h->tree.refit(P, h->faces, h->geom);
  });
}

int rso_bh_sizes(const rso_bh *h, int64_t *o) {
  return guard([&] {
    o[0] = (int64_t)h->tree.bvh.nodes.size();
    o[1] = (int64_t)h->tree.leaves.size();
    o[2] = (int64_t)h->lists.lumped.size();
    o[3] = (int64_t)h->lists.exact.size();
    o[4] = (int64_t)h->lists.partner_off.back();
    o[5] = (int64_t)h->lists.pairs_exact;
  });
}

int rso_bh_tree(const rso_bh *h, uint32_t *start, uint32_t *end, uint32_t *right, uint32_t *order,
                uint32_t *leaves) {
  return guard([&] {
    const auto &N = h->tree.bvh.nodes;
    for (size_t i = 0; i < N.size(); ++i) start[i] = N[i].start, end[i] = N[i].end, right[i] = N[i].right;
    std::copy(h->tree.bvh.order.begin(), h->tree.bvh.order.end(), order);
    std::copy(h->tree.leaves.begin(), h->tree.leaves.end(), leaves);
  });
}

int rso_bh_clusters(const rso_bh *h, double *bbox6, double *radius, double *area, double *centroid,
                    double *projector) {
  return guard([&] {
    const auto &C = h->tree.clusters;
    for (size_t i = 0; i < C.size(); ++i) {
      for (int k = 0; k < 3; ++k) {
        bbox6[6 * i + k] = C[i].bbox.lo[k];
        bbox6[6 * i + 3 + k] = C[i].bbox.hi[k];
        centroid[3 * i + k] = C[i].centroid[k];
      }
      for (int k = 0; k < 6; ++k) projector[6 * i + k] = C[i].projector[k];
      radius[i] = C[i].radius;
      area[i] = C[i].area;
    }
  });
}

int rso_bh_lists(const rso_bh *h, int64_t *lumped_off, uint32_t *lumped, int64_t *exact_off,
                 uint32_t *exact) {
  return guard([&] {
    const Lists &L = h->lists;
    for (size_t i = 0; i < L.lumped_off.size(); ++i) lumped_off[i] = (int64_t)L.lumped_off[i];
    for (size_t i = 0; i < L.exact_off.size(); ++i) exact_off[i] = (int64_t)L.exact_off[i];
    std::copy(L.lumped.begin(), L.lumped.end(), lumped);
    std::copy(L.exact.begin(), L.exact.end(), exact);
  });
}

int rso_bh_energy(const rso_bh *h, double alpha, double beta, double *energy) {
  return guard([&] { *energy = h->energy(Exponents::make(alpha, beta)); });
}

int rso_bh_energy_and_differential(const rso_bh *h, double alpha, double beta, double *energy,
                                   double *dE, double *fp7) {
  return guard([&] {  // barnes_hut.rs:387-412
    Exponents e = Exponents::make(alpha, beta);
    std::vector<std::array<double, 7>> o7;
    double E = h->face_partials(e, o7);
    size_t nf = h->faces.size();
    std::vector<double> da(nf);
    std::vector<v3> dx(nf), dn(nf);
    for (size_t f = 0; f < nf; ++f) {
      da[f] = o7[f][0];
      dx[f] = {o7[f][1], o7[f][2], o7[f][3]};
      dn[f] = {o7[f][4], o7[f][5], o7[f][6]};
    }
    std::vector<v3> G = pull_back(h->nv, h->positions, h->faces, da, dx, dn);
    bool finite = std::isfinite(E);
    for (auto &v : G)
      for (double x : v) finite = finite && std::isfinite(x);
    if (!finite) non_finite("Barnes-Hut energy (coincident barycenters)");
    *energy = E;
    if (dE)
      for (int v = 0; v < h->nv; ++v)
        for (int k = 0; k < 3; ++k) dE[3 * v + k] = G[v][k];
    if (fp7)
      for (size_t f = 0; f < nf; ++f)
        for (int k = 0; k < 7; ++k) fp7[7 * f + k] = o7[f][k];
  });
}

int rso_pull_back(int nv, const double *pos, int nf, const uint32_t *faces, const double *fp7,
                  double *dE) {
  return guard([&] {
    auto P = to_v3(pos, nv);
    auto T = to_tri(faces, nf);
    std::vector<double> da(nf);
    std::vector<v3> dx(nf), dn(nf);
    for (int f = 0; f < nf; ++f) {
      da[f] = fp7[7 * f];
      dx[f] = {fp7[7 * f + 1], fp7[7 * f + 2], fp7[7 * f + 3]};
      dn[f] = {fp7[7 * f + 4], fp7[7 * f + 5], fp7[7 * f + 6]};
    }
    auto G = pull_back(nv, P, T, da, dx, dn);
    for (int v = 0; v < nv; ++v)
      for (int k = 0; k < 3; ++k) dE[3 * v + k] = G[v][k];
  });
}

}  // extern "C"
