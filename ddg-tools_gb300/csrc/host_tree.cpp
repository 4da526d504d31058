// Surface validation, FP64 face geometry and the face BVH build (host C++).
//
// The BVH follows the split rule of RC/src/spatial/bvh.rs:126-220 (axis = depth mod 3,
// elements ordered by that coordinate with ties by index, split minimising the sum of the
// squared box diameters of the two sides with at least ceil(n/4) elements per side, leaf size
// L, nodes in pre-order). Instead of sorting every node's slice, the build keeps the elements
// presorted along each axis and partitions the three orders stably at every split, so a level
// costs O(n). The resulting tree (node ranges, right children, element order) is the crate's,
// bit for bit: the order inside a leaf is the parent's sort, i.e. the leaf's elements along the
// parent's axis.
//
// Compiled with -ffp-contract=off: every box, mass and centroid is computed with the same
// roundings as the reference.
#include "host_tree.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <future>
#include <numeric>
#include <string>
#include <thread>

#include "common.hpp"

namespace rsg {

static std::string s(size_t x) { return std::to_string(x); }

namespace {
thread_local bool g_topology_trusted = false;
thread_local const SharedFaceTree *g_shared_tree = nullptr;
}

SharedFaceTree::SharedFaceTree(const FaceGeom &g, const Tree &t, const uint32_t *faces_, const double *pos_, int nf_,
                               int leaf_size_, const std::shared_future<void> *ready_)
    : geom(g), tree(t), faces(faces_), pos(pos_), nf(nf_), leaf_size(leaf_size_), ready(ready_),
      prev(g_shared_tree) {
  g_shared_tree = this;
}
SharedFaceTree::~SharedFaceTree() { g_shared_tree = prev; }
const SharedFaceTree *shared_face_tree(const uint32_t *faces, const double *pos, int nf, int leaf_size) {
  for (const SharedFaceTree *s = g_shared_tree; s; s = s->prev)
    if (s->faces == faces && s->pos == pos && s->nf == nf && s->leaf_size == leaf_size) {
      if (s->ready) s->ready->get();
      return s;
    }
  return nullptr;
}

TrustedTopology::TrustedTopology() : prev(g_topology_trusted) { g_topology_trusted = true; }
TrustedTopology::~TrustedTopology() { g_topology_trusted = prev; }
bool topology_trusted() { return g_topology_trusted; }

void validate_topology(int nv, int nf, const uint32_t *faces) {
  if (g_topology_trusted) return;
  if (nf <= 0) fail(RS_TOPOLOGY, "NoFaces", "surface", "the face list is empty");
  if (nv < 0) fail(RS_TOPOLOGY, "TooLarge", "surface", "negative vertex count");
  for (int f = 0; f < nf; ++f) {  // surface.rs:144-161
    const uint32_t *t = faces + 3 * (size_t)f;
    for (int k = 0; k < 3; ++k)
      if (t[k] >= (uint32_t)nv)
        fail(RS_TOPOLOGY, "VertexOutOfRange", "surface",
             "face " + s(f) + " = (" + s(t[0]) + ", " + s(t[1]) + ", " + s(t[2]) + "), " +
                 s(nv) + " vertices");
    if (t[0] == t[1] || t[1] == t[2] || t[0] == t[2])
      fail(RS_TOPOLOGY, "RepeatedVertex", "surface", "face " + s(f) + " repeats a vertex");
  }
  {  // duplicates, surface.rs:163-196
    std::vector<std::pair<std::array<uint32_t, 3>, uint32_t>> keys((size_t)nf);
    for (int f = 0; f < nf; ++f) {
      std::array<uint32_t, 3> k{faces[3 * f], faces[3 * f + 1], faces[3 * f + 2]};
      std::sort(k.begin(), k.end());
      keys[f] = {k, (uint32_t)f};
    }
    std::sort(keys.begin(), keys.end());
    int64_t best_second = -1, best_first = -1;
    for (size_t i = 0; i < keys.size();) {
      size_t j = i + 1;
      while (j < keys.size() && keys[j].first == keys[i].first) ++j;
      if (j - i > 1 && (best_second < 0 || keys[i + 1].second < best_second))
        best_first = keys[i].second, best_second = keys[i + 1].second;
      i = j;
    }
    if (best_second >= 0)
      fail(RS_TOPOLOGY, "DuplicateFace", "surface",
           "faces " + s(best_first) + " and " + s(best_second) + " have the same vertices");
  }
  // edges, surface.rs:197-230
  struct Half {
    uint32_t a, b, f;
    uint8_t k;
  };
  std::vector<Half> half(3 * (size_t)nf);
  for (int f = 0; f < nf; ++f)
    for (int k = 0; k < 3; ++k) {
      uint32_t a = faces[3 * f + k], b = faces[3 * f + (k + 1) % 3];
      half[3 * f + k] = {std::min(a, b), std::max(a, b), (uint32_t)f, (uint8_t)k};
    }
  std::sort(half.begin(), half.end(), [](const Half &x, const Half &y) {
    if (x.a != y.a) return x.a < y.a;
    if (x.b != y.b) return x.b < y.b;
    if (x.f != y.f) return x.f < y.f;
    return x.k < y.k;
  });
  const uint32_t NONE = UINT32_MAX;
  std::vector<std::array<uint32_t, 2>> edge_faces;
  std::vector<std::array<uint32_t, 3>> face_edges((size_t)nf, {NONE, NONE, NONE});
  for (size_t i = 0; i < half.size();) {
    size_t j = i + 1;
    while (j < half.size() && half[j].a == half[i].a && half[j].b == half[i].b) ++j;
    if (j - i > 2)
      fail(RS_TOPOLOGY, "NonManifoldEdge", "surface",
           "edge (" + s(half[i].a) + ", " + s(half[i].b) + ") is shared by " + s(j - i) + " faces");
    uint32_t e = (uint32_t)edge_faces.size();
    edge_faces.push_back({half[i].f, j - i == 2 ? half[i + 1].f : NONE});
    for (size_t h = i; h < j; ++h) face_edges[half[h].f][half[h].k] = e;
    i = j;
  }
  // fans, surface.rs:233-346: the faces around a vertex must form one edge-connected fan.
  std::vector<uint32_t> ptr((size_t)nv + 1, 0), inc(3 * (size_t)nf);
  for (int f = 0; f < nf; ++f)
    for (int k = 0; k < 3; ++k) ptr[faces[3 * f + k] + 1]++;
  for (int v = 0; v < nv; ++v) ptr[v + 1] += ptr[v];
  {
    std::vector<uint32_t> fill(ptr.begin(), ptr.end() - 1);
    for (int f = 0; f < nf; ++f)
      for (int k = 0; k < 3; ++k) inc[fill[faces[3 * f + k]]++] = (uint32_t)f;
  }
  int64_t unref = -1, nonman = -1;
  std::vector<uint32_t> comp;
  for (int v = 0; v < nv; ++v) {
    uint32_t b = ptr[v], e = ptr[v + 1];
    if (b == e) {
      if (unref < 0) unref = v;
      continue;
    }
    // union-find over the incident faces joined by the two edges of each face at v
    size_t m = e - b;
    comp.resize(m);
    std::iota(comp.begin(), comp.end(), 0u);
    auto find = [&](uint32_t x) {
      while (comp[x] != x) x = comp[x] = comp[comp[x]];
      return x;
    };
    for (size_t i = 0; i < m; ++i) {
      uint32_t f = inc[b + i];
      const uint32_t *t = faces + 3 * (size_t)f;
      for (int k = 0; k < 3; ++k) {
        if (t[k] != (uint32_t)v && t[(k + 1) % 3] != (uint32_t)v) continue;
        auto ef = edge_faces[face_edges[f][k]];
        uint32_t g = ef[0] == f ? ef[1] : ef[0];
        if (g == NONE) continue;
        for (size_t j = 0; j < m; ++j)
          if (inc[b + j] == g) {
            uint32_t ra = find((uint32_t)i), rb = find((uint32_t)j);
            if (ra != rb) comp[ra] = rb;
          }
      }
    }
    size_t fans = 0;
    for (size_t i = 0; i < m; ++i) fans += find((uint32_t)i) == i;
    if (fans > 1 && nonman < 0) nonman = v;
  }
  if (nonman >= 0)
    fail(RS_TOPOLOGY, "NonManifoldVertex", "surface",
         "vertex " + s(nonman) + " has more than one fan of faces");
  if (unref >= 0)
    fail(RS_TOPOLOGY, "UnreferencedVertex", "surface", "vertex " + s(unref));
}

static inline void face_q(const double *p0, const double *p1, const double *p2, double &a,
                          double n[3], double x[3]) {
  // geometry.rs:33-39: n = (p1-p0) x (p2-p0), a = |n|/2, N = n/|n|, X = (p0+p1+p2) * (1/3)
  double u[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
  double w[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
  double c[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
  double len = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  const double third = 1.0 / 3.0;
  for (int k = 0; k < 3; ++k) x[k] = ((p0[k] + p1[k]) + p2[k]) * third;
  a = 0.5 * len;
  double il = 1.0 / len;
  for (int k = 0; k < 3; ++k) n[k] = c[k] * il;
}

void validate_positions(int nv, int nf, const uint32_t *faces, const double *pos) {
  for (int v = 0; v < nv; ++v)
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(pos[3 * v + k]))
        fail(RS_NONFINITE_POSITION, "NonFinitePosition", "surface", "vertex " + s(v));
  for (int f = 0; f < nf; ++f) {
    const uint32_t *t = faces + 3 * (size_t)f;
    double a, n[3], x[3];
    face_q(pos + 3 * (size_t)t[0], pos + 3 * (size_t)t[1], pos + 3 * (size_t)t[2], a, n, x);
    bool ok = a > 0.0 && std::isfinite(a) && std::isfinite(n[0]) && std::isfinite(n[1]) &&
              std::isfinite(n[2]);
    if (!ok) fail(RS_DEGENERATE_FACE, "DegenerateFace", "surface", "face " + s(f) + " has zero area");
  }
}

FaceGeom face_geometry(int nf, const uint32_t *faces, const double *pos) {
  FaceGeom g;
  g.area.resize(nf);
  g.normal.resize(3 * (size_t)nf);
  g.bary.resize(3 * (size_t)nf);
  for (int f = 0; f < nf; ++f) {
    const uint32_t *t = faces + 3 * (size_t)f;
    face_q(pos + 3 * (size_t)t[0], pos + 3 * (size_t)t[1], pos + 3 * (size_t)t[2], g.area[f],
           &g.normal[3 * (size_t)f], &g.bary[3 * (size_t)f]);
  }
  return g;
}

// ---------------------------------------------------------------- BVH

namespace {

struct Box {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  void join(const double *b) {  // Aabb::union (RC/src/spatial/aabb.rs:45-52): fmin/fmax
    for (int k = 0; k < 3; ++k) lo[k] = std::fmin(lo[k], b[k]), hi[k] = std::fmax(hi[k], b[3 + k]);
  }
  double diam2() const {  // Aabb::diameter_sq (aabb.rs:66-77)
    if (lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]) return 0.0;
    double s = 0.0;
    for (int k = 0; k < 3; ++k) {
      double w = hi[k] - lo[k];
      s += w * w;
    }
    return s;
  }
};

// Total order of f64::total_cmp as an integer key.
inline int64_t tkey(double x) {
  int64_t b;
  std::memcpy(&b, &x, 8);
  return b ^ (int64_t)(((uint64_t)(b >> 63)) >> 1);
}

// Indices 0..n-1 ordered by (key, index): a stable least-significant-digit radix sort of the
// keys made unsigned (sign bit flipped), 8 bits per pass, starting from index order; passes
// whose digit is the same for every key are skipped.
std::vector<uint32_t> sort_by_key(const std::vector<int64_t> &key) {
  const size_t n = key.size();
  std::vector<uint64_t> k0(n), k1(n);
  std::vector<uint32_t> i0(n), i1(n);
  std::vector<size_t> hist(8 * 256, 0);
  for (size_t i = 0; i < n; ++i) {
    const uint64_t u = (uint64_t)key[i] ^ (1ull << 63);
    k0[i] = u, i0[i] = (uint32_t)i;
    for (int d = 0; d < 8; ++d) hist[256 * d + ((u >> (8 * d)) & 255u)]++;
  }
  for (int d = 0; d < 8; ++d) {
    size_t *h = hist.data() + 256 * d;
    if (*std::max_element(h, h + 256) == n) continue;
    size_t off = 0;
    for (int b = 0; b < 256; ++b) {
      const size_t c = h[b];
      h[b] = off;
      off += c;
    }
    for (size_t i = 0; i < n; ++i) {
      const size_t o = h[(k0[i] >> (8 * d)) & 255u]++;
      k1[o] = k0[i], i1[o] = i0[i];
    }
    k0.swap(k1), i0.swap(i1);
  }
  return i0;
}

}  // namespace

namespace {

// The split recursion of build_tree over one subtree: nodes in pre-order relative to the
// subtree (right = index of the right child within the subtree, 0 for a leaf). Subtrees of
// the top levels run as concurrent tasks; their ranges of the presorted orders, of `tmp` and
// of `order` are disjoint, and the element flags are per element, so nothing is shared.
struct SplitCtx {
  const double *ebox;
  int leaf_size;
  size_t n;
  std::vector<uint32_t> *srt;  // [3]
  std::vector<uint8_t> *left_flag;
  std::vector<uint32_t> *tmp;
  std::vector<uint32_t> *order;
};

struct LocalNodes {
  std::vector<uint32_t> start, end, right;
};

void split_range(const SplitCtx &c, size_t start, size_t end, size_t depth, LocalNodes &out, int par_depth) {
  const uint32_t id = (uint32_t)out.start.size();
  out.start.push_back((uint32_t)start);
  out.end.push_back((uint32_t)end);
  out.right.push_back(0);
  const size_t cnt = end - start;
  if (cnt <= (size_t)c.leaf_size) {
    // A leaf keeps its parent's sort (axis (depth-1) mod 3); a root leaf is unsorted.
    if (depth == 0)
      for (size_t i = 0; i < c.n; ++i) (*c.order)[i] = (uint32_t)i;
    else
      std::copy(c.srt[(depth - 1) % 3].begin() + start, c.srt[(depth - 1) % 3].begin() + end,
                c.order->begin() + start);
    return;
  }
  const int axis = (int)(depth % 3);
  const uint32_t *sl = c.srt[axis].data() + start;
  std::vector<Box> suffix(cnt);
  Box acc;
  for (size_t k = cnt; k-- > 0;) {
    acc.join(c.ebox + 6 * (size_t)sl[k]);
    suffix[k] = acc;
  }
  Box prefix;
  double best_cost = INFINITY;
  size_t best_k = cnt / 2;
  size_t lo = (size_t)std::ceil(0.25 * (double)cnt);
  lo = std::min(std::max<size_t>(lo, 1), cnt / 2);
  for (size_t k = 1; k <= cnt - lo; ++k) {
    prefix.join(c.ebox + 6 * (size_t)sl[k - 1]);
    if (k < lo) continue;
    double cost = prefix.diam2() + suffix[k].diam2();
    if (cost < best_cost) best_cost = cost, best_k = k;
  }
  for (size_t k = 0; k < cnt; ++k) (*c.left_flag)[sl[k]] = k < best_k;
  uint32_t *tmp = c.tmp->data() + start;
  for (int b = 0; b < 3; ++b) {
    if (b == axis) continue;
    uint32_t *o = c.srt[b].data() + start;
    size_t nl = 0, nr = best_k;
    for (size_t k = 0; k < cnt; ++k) {
      uint32_t e = o[k];
      tmp[(*c.left_flag)[e] ? nl++ : nr++] = e;
    }
    std::copy(tmp, tmp + cnt, o);
  }
  const size_t split = start + best_k;
  auto append = [&](const LocalNodes &sub) {
    const uint32_t off = (uint32_t)out.start.size();
    for (size_t i = 0; i < sub.start.size(); ++i) {
      out.start.push_back(sub.start[i]);
      out.end.push_back(sub.end[i]);
      out.right.push_back(sub.right[i] ? sub.right[i] + off : 0);
    }
  };
  if (par_depth > 0 && cnt > 4096) {
    LocalNodes left, right;
    auto fut = std::async(std::launch::async, [&] { split_range(c, start, split, depth + 1, left, par_depth - 1); });
    split_range(c, split, end, depth + 1, right, par_depth - 1);
    fut.get();
    append(left);
    out.right[id] = (uint32_t)out.start.size();
    append(right);
  } else {
    split_range(c, start, split, depth + 1, out, 0);
    out.right[id] = (uint32_t)out.start.size();
    split_range(c, split, end, depth + 1, out, 0);
  }
}

}  // namespace

Tree build_tree(size_t n, const double *pts, const double *ebox, const double *mass,
                int leaf_size) {
  if (leaf_size < 1) fail(RS_INVALID_OPTION, "InvalidOption", "tree", "leaf_size must be at least 1");
  if (n == 0) fail(RS_INVALID_OPTION, "InvalidOption", "tree", "at least 1 element");
  Tree T;
  T.order.resize(n);
  // Presorted orders per axis (one thread per axis), partitioned stably at every split.
  std::vector<uint32_t> srt[3];
  {
    auto presort = [&](int a) {
      std::vector<int64_t> key(n);
      for (size_t i = 0; i < n; ++i) key[i] = tkey(pts[3 * i + a]);
      srt[a] = sort_by_key(key);
    };
    if (n > 65536) {
      auto f1 = std::async(std::launch::async, presort, 1);
      auto f2 = std::async(std::launch::async, presort, 2);
      presort(0);
      f1.get(), f2.get();
    } else {
      for (int a = 0; a < 3; ++a) presort(a);
    }
  }
  std::vector<uint8_t> left_flag(n, 0);
  std::vector<uint32_t> tmp(n);
  SplitCtx c{ebox, leaf_size, n, srt, &left_flag, &tmp, &T.order};
  LocalNodes nodes;
  const int par_depth = std::thread::hardware_concurrency() > 1 ? 4 : 0;  // up to 16 subtrees
  split_range(c, 0, n, 0, nodes, par_depth);
  T.start = std::move(nodes.start);
  T.end = std::move(nodes.end);
  T.right = std::move(nodes.right);
  // Node data as Bvh::refit (bvh.rs:226-260, summarize 314-330).
  size_t nn = T.start.size();
  T.box.resize(6 * nn);
  T.mass.resize(nn);
  T.centroid.resize(3 * nn);
  T.radius.resize(nn);
  std::vector<double> mom(3 * nn);
  for (size_t i = nn; i-- > 0;) {
    Box bb;
    double m = 0, mo[3] = {0, 0, 0};
    if (T.right[i] == 0) {
      for (uint32_t p = T.start[i]; p < T.end[i]; ++p) {
        uint32_t e = T.order[p];
        bb.join(ebox + 6 * (size_t)e);
        m += mass[e];
        for (int k = 0; k < 3; ++k) mo[k] += mass[e] * pts[3 * (size_t)e + k];
      }
    } else {
      size_t l = i + 1, r = T.right[i];
      bb.join(&T.box[6 * l]);
      bb.join(&T.box[6 * r]);
      m = T.mass[l] + T.mass[r];
      for (int k = 0; k < 3; ++k) mo[k] = mom[3 * l + k] + mom[3 * r + k];
    }
    for (int k = 0; k < 3; ++k) T.box[6 * i + k] = bb.lo[k], T.box[6 * i + 3 + k] = bb.hi[k];
    T.mass[i] = m;
    for (int k = 0; k < 3; ++k) mom[3 * i + k] = mo[k];
  }
  T.leaf_ordinal.assign(nn, UINT32_MAX);
  for (size_t i = 0; i < nn; ++i) {
    double r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      double c = mom[3 * i + k] / T.mass[i];  // Node::centroid (bvh.rs:83-90)
      T.centroid[3 * i + k] = c;
      double d = std::fmax(T.box[6 * i + 3 + k] - c, c - T.box[6 * i + k]);
      r2 += d * d;
    }
    T.radius[i] = std::sqrt(r2);
    if (T.right[i] == 0) {
      T.leaf_ordinal[i] = (uint32_t)T.leaves.size();
      T.leaves.push_back((uint32_t)i);
    }
  }
  return T;
}

Tree build_face_tree(int nf, const uint32_t *faces, const double *pos, const FaceGeom &g,
                     int leaf_size) {
  std::vector<double> ebox(6 * (size_t)nf);
  for (int f = 0; f < nf; ++f) {
    Box b;
    for (int c = 0; c < 3; ++c) {
      const double *p = pos + 3 * (size_t)faces[3 * f + c];
      double pb[6] = {p[0], p[1], p[2], p[0], p[1], p[2]};
      b.join(pb);
    }
    for (int k = 0; k < 3; ++k) ebox[6 * f + k] = b.lo[k], ebox[6 * f + 3 + k] = b.hi[k];
  }
  return build_tree((size_t)nf, g.bary.data(), ebox.data(), g.area.data(), leaf_size);
}

}  // namespace rsg

extern "C" int rs_surface_validate(int nv, int nf, const uint32_t *faces, const double *positions_host) {
  return rsg::guard([&] {
    rsg::validate_topology(nv, nf, faces);
    rsg::validate_positions(nv, nf, faces, positions_host);
  });
}

extern "C" int rs_face_tree_build(int nv, int nf, const uint32_t *faces, const double *positions_host,
                                  int leaf_size, int capacity, uint32_t *start, uint32_t *end,
                                  uint32_t *right, uint32_t *order, double *box6, double *radius,
                                  int *n_nodes) {
  return rsg::guard([&] {
    rsg::validate_topology(nv, nf, faces);
    rsg::validate_positions(nv, nf, faces, positions_host);
    rsg::FaceGeom g = rsg::face_geometry(nf, faces, positions_host);
    rsg::Tree T = rsg::build_face_tree(nf, faces, positions_host, g, leaf_size);
    int nn = (int)T.n_nodes();
    *n_nodes = nn;
    if (nn > capacity)
      rsg::fail(RS_INVALID_OPTION, "InvalidOption", "tree",
                "capacity " + std::to_string(capacity) + " < " + std::to_string(nn) + " nodes");
    std::copy(T.start.begin(), T.start.end(), start);
    std::copy(T.end.begin(), T.end.end(), end);
    std::copy(T.right.begin(), T.right.end(), right);
    std::copy(T.order.begin(), T.order.end(), order);
    std::copy(T.box.begin(), T.box.end(), box6);
    std::copy(T.radius.begin(), T.radius.end(), radius);
  });
}
