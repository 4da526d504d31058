// FP64 oracle of the hierarchical (block cluster tree) metric products -- TEST INFRASTRUCTURE
// ONLY. Restates RS/src/spatial/block_tree.rs (BlockTree::build_impl 129-413, multiply_core
// 536-613, leaf_rows 647-690), RS/src/metric/hierarchical.rs (separated 116-123, FaceKernels
// 183-236, FaceMetricTree::from_parts/product 323-363, 696-812, VertexKernel 967-996,
// VertexFractionalTree::build/product 1017-1084, 1313-1345) and RS/src/metric/mod.rs
// (df_coefficients 120-131).
#include <algorithm>
#include <cstring>
#include <memory>

#include "rs_oracle.h"
#include "rso_internal.hpp"

using namespace rso;

namespace {

template <class F>
int guard2(F &&f, std::string &err) {
  try {
    f();
    return RSO_OK;
  } catch (const Error &e) {
    err = e.what();
    return e.code;
  } catch (const std::exception &e) {
    err = e.what();
    return RSO_INTERNAL;
  }
}
thread_local std::string g_err;

// separated (hierarchical.rs:116-123): chi > 0, d2 > 0 and max(r)^2 <= chi^2 d2.
bool separated(double ra, const Aabb &ba, double rb, const Aabb &bb, double chi) {
  if (!(chi > 0.0)) return false;
  double d2 = box_distance_sq(ba, bb);
  double h = fmax_(ra, rb);
  return d2 > 0.0 && h * h <= chi * chi * d2;
}

// A kernel of the block tree: admissibility, far coefficients (per node pair), near entries
// (per element pair), N values each.
struct KernelIface {
  int N;
  std::function<bool(size_t, size_t)> admissible;
  std::function<void(size_t, size_t, double *)> far;
  std::function<void(size_t, size_t, double *)> near;
};

// One row of one near block with stored kernel values: out_r += sum over the block's columns
// of k[kmap[c]] psi[c], in column order (the element itself skipped), with the row's CC sums
// held in registers; N <= 2 kernels per entry, km[c] = (kmap[c] != 0).
template <int CC>
static inline void near_run(const double *&stored, int N, const unsigned char *km, const double *xb, uint32_t cb,
                            bool self, uint32_t self_col, double *o) {
  double acc[CC];
  for (int c = 0; c < CC; ++c) acc[c] = o[c];
  for (uint32_t cc = 0; cc < cb; ++cc) {
    const double *kv = stored;
    stored += N;
    if (self && cc == self_col) continue;
    const double *x = xb + (size_t)cc * CC;
    const double k0 = kv[0], k1 = N == 2 ? kv[1] : kv[0];
    for (int c = 0; c < CC; ++c) acc[c] += (km[c] ? k1 : k0) * x[c];
  }
  for (int c = 0; c < CC; ++c) o[c] = acc[c];
}

struct BlockTree {  // block_tree.rs:61-91
  int N = 1;
  // The near-field values, stored once per build as the crate stores its dense near blocks
  // (block_tree.rs:372-415), in the order the product visits them: per leaf, per block of its
  // chain, row-major over (row, column), N values each; near_off[li] starts leaf li.
  std::vector<double> near_val;
  std::vector<size_t> near_off;
  std::vector<uint32_t> start, end, right, order, position, leaves, chain_ptr, chain;
  std::vector<size_t> far_ptr, near_ptr;
  std::vector<uint32_t> far_col, near_col;
  std::vector<double> far_coef;  // N per far block
  size_t n_adm = 0, n_near_blocks = 0, near_entries = 0, depth = 0;
  const KernelIface *k = nullptr;

  static void group_by_row(const std::vector<std::pair<uint32_t, uint32_t>> &pairs, size_t n,
                           std::vector<size_t> &ptr, std::vector<uint32_t> &col) {
    ptr.assign(n + 1, 0);  // block_tree.rs:741-756
    for (auto &p : pairs) ptr[p.first + 1]++;
    for (size_t i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
    std::vector<size_t> fill(ptr.begin(), ptr.end() - 1);
    col.assign(pairs.size(), 0);
    for (auto &p : pairs) col[fill[p.first]++] = p.second;
  }

  void build(const Bvh &bvh, const KernelIface &kern, size_t leaf_pairs) {
    k = &kern;
    N = kern.N;
    size_t nn = bvh.nodes.size(), n = bvh.order.size();
    start.resize(nn), end.resize(nn), right.resize(nn);
    for (size_t i = 0; i < nn; ++i)
      start[i] = bvh.nodes[i].start, end[i] = bvh.nodes[i].end, right[i] = bvh.nodes[i].right;
    order = bvh.order;
    position.assign(n, 0);
    for (size_t p = 0; p < n; ++p) position[order[p]] = (uint32_t)p;
    auto is_leaf = [&](size_t a) { return right[a] == 0; };
    auto len = [&](size_t a) { return (size_t)(end[a] - start[a]); };
    std::vector<std::pair<uint32_t, uint32_t>> adm, nearb, level{{0, 0}}, next;
    depth = 0;
    while (!level.empty()) {  // block_tree.rs:170-202
      ++depth;
      next.clear();
      for (auto [a, b] : level) {
        if (a != b && kern.admissible(a, b))
          adm.push_back({a, b});
        else if ((is_leaf(a) && is_leaf(b)) || len(a) * len(b) <= leaf_pairs)
          nearb.push_back({a, b});
        else {
          uint32_t ka[2], kb[2];
          int na = is_leaf(a) ? 1 : 2, nb = is_leaf(b) ? 1 : 2;
          ka[0] = is_leaf(a) ? a : a + 1, ka[1] = right[a];
          kb[0] = is_leaf(b) ? b : b + 1, kb[1] = right[b];
          for (int i = 0; i < na; ++i)
            for (int j = 0; j < nb; ++j) next.push_back({ka[i], kb[j]});
        }
      }
      level.swap(next);
    }
    group_by_row(adm, nn, far_ptr, far_col);
    far_coef.assign(far_col.size() * N, 0.0);
    for (size_t a = 0; a < nn; ++a)
      for (size_t p = far_ptr[a]; p < far_ptr[a + 1]; ++p) kern.far(a, far_col[p], &far_coef[p * N]);
    group_by_row(nearb, nn, near_ptr, near_col);
    n_adm = adm.size();
    n_near_blocks = nearb.size();
    near_entries = 0;
    for (auto [a, b] : nearb) near_entries += a == b ? len(a) * (len(a) - 1) : len(a) * len(b);
    // leaves and their chains root -> leaf (block_tree.rs:349-372)
    std::vector<uint32_t> parent(nn, UINT32_MAX);
    for (size_t i = 0; i < nn; ++i)
      if (!is_leaf(i)) parent[i + 1] = (uint32_t)i, parent[right[i]] = (uint32_t)i;
    leaves.clear();
    chain_ptr.assign(1, 0);
    chain.clear();
    for (size_t a = 0; a < nn; ++a)
      if (is_leaf(a)) {
        leaves.push_back((uint32_t)a);
        size_t s = chain.size();
        uint32_t x = (uint32_t)a;
        for (;;) {
          chain.push_back(x);
          if (x == 0) break;
          x = parent[x];
        }
        std::reverse(chain.begin() + s, chain.end());
        chain_ptr.push_back(chain.size());
      }
  }

  // Evaluates every near entry once (the kernels at (min, max) index, so the values equal the
  // on-demand ones bit for bit).
  void store_near() {
    const size_t nl = leaves.size();
    near_off.assign(nl + 1, 0);
    for (size_t li = 0; li < nl; ++li) {
      uint32_t l = leaves[li];
      size_t rows = end[l] - start[l], cnt = 0;
      for (size_t ci = chain_ptr[li]; ci < chain_ptr[li + 1]; ++ci) {
        uint32_t a = chain[ci];
        for (size_t q = near_ptr[a]; q < near_ptr[a + 1]; ++q) cnt += rows * (end[near_col[q]] - start[near_col[q]]);
      }
      near_off[li + 1] = near_off[li] + cnt * N;
    }
    near_val.assign(near_off[nl], 0.0);
    parallel_for((int64_t)nl, [&](int64_t lb, int64_t le) {
      for (int64_t li = lb; li < le; ++li) {
        uint32_t l = leaves[li];
        uint32_t s = start[l];
        size_t rows = end[l] - s;
        double *o = &near_val[near_off[li]];
        for (size_t ci = chain_ptr[li]; ci < chain_ptr[li + 1]; ++ci) {
          uint32_t a = chain[ci];
          size_t r0 = s - start[a];
          for (size_t q = near_ptr[a]; q < near_ptr[a + 1]; ++q) {
            uint32_t b = near_col[q];
            uint32_t sb = start[b], cb = end[b] - start[b];
            for (size_t r = 0; r < rows; ++r)
              for (uint32_t cc = 0; cc < cb; ++cc, o += N)
                if (!(a == b && cc == r0 + r)) k->near(order[s + r], order[sb + cc], o);
          }
        }
      }
    });
  }

  // multiply_core (block_tree.rs:536-613) with channel c on kernel kmap[c]; psi/out in BVH
  // order, C channels per element.
  void multiply_core(const std::vector<int> &kmap, const std::vector<double> &psi,
                     std::vector<double> &out) const {
    size_t C = kmap.size(), nn = start.size(), n = order.size();
    std::vector<double> up(nn * C, 0.0), acc(nn * C, 0.0);
    for (size_t a = nn; a-- > 0;) {
      double *u = &up[a * C];
      if (right[a] == 0) {
        for (uint32_t p = start[a]; p < end[a]; ++p)
          for (size_t c = 0; c < C; ++c) u[c] += 1.0 * psi[p * C + c];  // weight 1
      } else {
        for (size_t c = 0; c < C; ++c) u[c] = up[(a + 1) * C + c] + up[right[a] * C + c];
      }
    }
    // far blocks per row node (independent rows: the same sums in the same order per node)
    parallel_for((int64_t)nn, [&](int64_t ab, int64_t ae) {
      for (int64_t a = ab; a < ae; ++a) {
        double *f = &acc[a * C];
        for (size_t p = far_ptr[a]; p < far_ptr[a + 1]; ++p) {
          const double *kc = &far_coef[p * N];
          const double *u = &up[far_col[p] * C];
          for (size_t c = 0; c < C; ++c) f[c] += kc[kmap[c]] * u[c];
        }
      }
    });
    for (size_t a = 0; a < nn; ++a)
      if (right[a] != 0)
        for (size_t ch : {a + 1, (size_t)right[a]})
          for (size_t c = 0; c < C; ++c) acc[ch * C + c] += acc[a * C + c];
    out.assign(n * C, 0.0);
    std::vector<double> kv(N);
    std::vector<unsigned char> km(C);
    for (size_t c = 0; c < C; ++c) km[c] = kmap[c] != 0;
    parallel_for((int64_t)leaves.size(), [&](int64_t lb, int64_t le) {
      std::vector<double> kvv(N);
      for (int64_t li = lb; li < le; ++li) {
        uint32_t l = leaves[li];
        uint32_t s = start[l];
        size_t rows = end[l] - s;
        for (size_t r = 0; r < rows; ++r)
          for (size_t c = 0; c < C; ++c) out[(s + r) * C + c] = 1.0 * acc[l * C + c];
        const double *stored = near_val.empty() ? nullptr : &near_val[near_off[li]];
        for (size_t ci = chain_ptr[li]; ci < chain_ptr[li + 1]; ++ci) {
          uint32_t a = chain[ci];
          size_t r0 = s - start[a];
          for (size_t q = near_ptr[a]; q < near_ptr[a + 1]; ++q) {
            uint32_t b = near_col[q];
            uint32_t sb = start[b], cb = end[b] - start[b];
            for (size_t r = 0; r < rows; ++r) {
              size_t i = order[s + r];
              double *o = &out[(s + r) * C];
              if (stored && N <= 2 && (C == 12 || C == 3 || C == 1)) {
                const bool self = a == b;
                const uint32_t sc = (uint32_t)(r0 + r);
                const double *xb = &psi[(size_t)sb * C];
                if (C == 12) near_run<12>(stored, N, km.data(), xb, cb, self, sc, o);
                else if (C == 3) near_run<3>(stored, N, km.data(), xb, cb, self, sc, o);
                else near_run<1>(stored, N, km.data(), xb, cb, self, sc, o);
                continue;
              }
              for (uint32_t cc = 0; cc < cb; ++cc) {
                const double *kv = stored;
                if (stored) stored += N;
                if (a == b && cc == r0 + r) continue;  // the element itself
                if (!kv) {
                  k->near(i, order[sb + cc], kvv.data());
                  kv = kvv.data();
                }
                const double *x = &psi[(sb + cc) * C];
                if (N == 2) {  // the selection written as a blend, so that the loop vectorises
                  const double k0 = kv[0], k1 = kv[1];
                  for (size_t c = 0; c < C; ++c) o[c] += (km[c] ? k1 : k0) * x[c];
                } else {
                  for (size_t c = 0; c < C; ++c) o[c] += kv[kmap[c]] * x[c];
                }
              }
            }
          }
        }
      }
    });
  }

  // multiply (block_tree.rs:472-482): original element order in and out.
  std::vector<double> multiply(const std::vector<int> &kmap, const std::vector<double> &psi) const {
    size_t C = kmap.size(), n = order.size();
    std::vector<double> pp(n * C), out, res(n * C);
    for (size_t p = 0; p < n; ++p)
      for (size_t c = 0; c < C; ++c) pp[p * C + c] = psi[order[p] * C + c];
    multiply_core(kmap, pp, out);
    for (size_t i = 0; i < n; ++i)
      for (size_t c = 0; c < C; ++c) res[i * C + c] = out[position[i] * C + c];
    return res;
  }
};

// df_coefficients (RS/src/metric/mod.rs:120-131): g_c = (n/|n|^2) x e_opp(c).
std::array<v3, 3> df_coefficients(const std::array<v3, 3> &p) {
  v3 n = cross(sub(p[1], p[0]), sub(p[2], p[0]));
  double len = norm(n);
  v3 w = scale(n, 1.0 / (len * len));
  std::array<v3, 3> e = {sub(p[2], p[1]), sub(p[0], p[2]), sub(p[1], p[0])};
  return {cross(w, e[0]), cross(w, e[1]), cross(w, e[2])};
}

}  // namespace

// ---------------------------------------------------------------- FaceMetricTree

struct rso_metric {
  int nv = 0, nf = 0;
  std::vector<tri> faces;
  std::vector<v3> pos;
  FaceGeometry g;
  std::vector<std::array<v3, 3>> df;
  FaceTree tree;
  KernelIface kern;
  BlockTree bct;
  std::vector<double> ha_perm;  // 2 per BVH position
  std::vector<std::vector<std::pair<uint32_t, int>>> inc;
  double neg_s = 0;
};

extern "C" {

int rso_metric_build(int nv, const double *pos, int nf, const uint32_t *faces, double alpha,
                     double beta, double chi, int leaf_size, int leaf_pairs, rso_metric **out) {
  *out = nullptr;
  return guard2([&] {
    Exponents e = Exponents::make(alpha, beta);
    if (!(std::isfinite(chi) && chi >= 0.0)) throw Error(RSO_INVALID_OPTION, "chi must be >= 0");
    auto h = std::make_unique<rso_metric>();
    h->nv = nv, h->nf = nf;
    for (int i = 0; i < nv; ++i) h->pos.push_back({pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]});
    for (int f = 0; f < nf; ++f) h->faces.push_back({faces[3 * f], faces[3 * f + 1], faces[3 * f + 2]});
    validate_positions(nv, h->pos, h->faces);
    h->g = face_geometry(h->pos, h->faces);
    for (int f = 0; f < nf; ++f) h->df.push_back(df_coefficients(corners(h->pos, h->faces[f])));
    h->tree = FaceTree::build(h->pos, h->faces, h->g, leaf_size);
    h->neg_s = -e.s();
    rso_metric *H = h.get();
    auto hi_lo = [H](v3 d, double qa, double qb, double *o) {  // hierarchical.rs:185-189
      double r2 = dot(d, d);
      double hi = std::pow(r2, H->neg_s);
      o[0] = hi;
      o[1] = 0.5 * (qa + qb) / (r2 * r2) * hi;
    };
    h->kern.N = 2;
    h->kern.admissible = [H, chi](size_t a, size_t b) {
      const Cluster &ca = H->tree.clusters[a], &cb = H->tree.clusters[b];
      return separated(ca.radius, ca.bbox, cb.radius, cb.bbox, chi);
    };
    h->kern.far = [H, hi_lo](size_t a, size_t b, double *o) {  // hierarchical.rs:210-220
      if (a > b) std::swap(a, b);
      const Cluster &ca = H->tree.clusters[a], &cb = H->tree.clusters[b];
      v3 d = sub(ca.centroid, cb.centroid);
      hi_lo(d, ca.projector_quadratic_form(d), cb.projector_quadratic_form(d), o);
    };
    h->kern.near = [H, hi_lo](size_t i, size_t j, double *o) {  // hierarchical.rs:224-231
      size_t a = std::min(i, j), b = std::max(i, j);
      v3 d = sub(H->g.barycenters[a], H->g.barycenters[b]);
      double ns = dot(H->g.normals[a], d), nt = dot(H->g.normals[b], d);
      hi_lo(d, ns * ns, nt * nt, o);
    };
    h->bct.build(h->tree.bvh, h->kern, (size_t)leaf_pairs);
    h->bct.store_near();
    std::vector<double> psi(2 * (size_t)nf);
    for (int f = 0; f < nf; ++f) psi[2 * f] = psi[2 * f + 1] = h->g.areas[f];
    std::vector<double> ha = h->bct.multiply({0, 1}, psi);
    for (int f = 0; f < nf; ++f)
      if (!(std::isfinite(ha[2 * f]) && std::isfinite(ha[2 * f + 1])))
        throw Error(RSO_NONFINITE_ENERGY, "coincident barycenters");
    h->ha_perm.resize(2 * (size_t)nf);
    for (int p = 0; p < nf; ++p) {
      uint32_t s = h->bct.order[p];
      h->ha_perm[2 * p] = ha[2 * s], h->ha_perm[2 * p + 1] = ha[2 * s + 1];
    }
    h->inc.assign(nv, {});
    for (int f = 0; f < nf; ++f)
      for (int c = 0; c < 3; ++c) h->inc[h->faces[f][c]].push_back({(uint32_t)f, c});
    *out = h.release();
  }, g_err);
}

void rso_metric_free(rso_metric *h) { delete h; }

const char *rso_metric_last_error(void) { return g_err.c_str(); }

// Counts: far blocks, near blocks, near entries (off-diagonal), depth, nodes.
int rso_metric_stats(const rso_metric *h, int64_t *o5) {
  return guard2([&] {
    o5[0] = (int64_t)h->bct.n_adm;
    o5[1] = (int64_t)h->bct.n_near_blocks;
    o5[2] = (int64_t)h->bct.near_entries;
    o5[3] = (int64_t)h->bct.depth;
    o5[4] = (int64_t)h->bct.start.size();
  }, g_err);
}

// The blocks grouped by row node: far_ptr [nodes+1], far_col, near_ptr [nodes+1], near_col.
int rso_metric_blocks(const rso_metric *h, int64_t *far_ptr, uint32_t *far_col, double *far_coef,
                      int64_t *near_ptr, uint32_t *near_col) {
  return guard2([&] {
    const BlockTree &B = h->bct;
    for (size_t i = 0; i < B.far_ptr.size(); ++i) far_ptr[i] = (int64_t)B.far_ptr[i];
    for (size_t i = 0; i < B.near_ptr.size(); ++i) near_ptr[i] = (int64_t)B.near_ptr[i];
    std::copy(B.far_col.begin(), B.far_col.end(), far_col);
    std::copy(B.near_col.begin(), B.near_col.end(), near_col);
    std::copy(B.far_coef.begin(), B.far_coef.end(), far_coef);
  }, g_err);
}

// H~ a per face in original order, 2 per face (FaceMetricTree::kernel_times_areas).
int rso_metric_ha(const rso_metric *h, double *ha) {
  return guard2([&] {
    for (int p = 0; p < h->nf; ++p) {
      uint32_t s = h->bct.order[p];
      ha[2 * s] = h->ha_perm[2 * p], ha[2 * s + 1] = h->ha_perm[2 * p + 1];
    }
  }, g_err);
}

// FaceMetricTree::apply (hierarchical.rs:521-531, product 696-812) for nb vectors one by one.
int rso_metric_apply(const rso_metric *h, double w_hi, double w_lo, int nb, const double *xs,
                     double *ys) {
  return guard2([&] {
    const bool hi = w_hi != 0.0, lo = w_lo != 0.0;
    const size_t nf = h->nf, n3 = 3 * (size_t)h->nv;
    const size_t C = (hi ? 9 : 0) + (lo ? 3 : 0), off = hi ? 9 : 0;
    std::vector<int> kmap;
    for (size_t c = 0; c < C; ++c) kmap.push_back(c < off ? 0 : 1);
    const auto &order = h->bct.order;
    for (int q = 0; q < nb; ++q) {
      const double *x = xs + q * n3;
      double *y = ys + q * n3;
      if (C == 0) {
        std::fill(y, y + n3, 0.0);
        continue;
      }
      std::vector<double> m(nf * C, 0.0), psi(nf * C), hx, z(nf * C);
      for (size_t p = 0; p < nf; ++p) {
        uint32_t s = order[p];
        const tri &t = h->faces[s];
        double *o = &m[p * C];
        if (hi) {
          const auto &g = h->df[s];
          for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) {
              double xc = x[3 * (size_t)t[c] + k];
              for (int r = 0; r < 3; ++r) o[3 * k + r] += xc * g[c][r];
            }
        }
        if (lo)
          for (int k = 0; k < 3; ++k)
            o[off + k] = (x[3 * (size_t)t[0] + k] + x[3 * (size_t)t[1] + k] + x[3 * (size_t)t[2] + k]) / 3.0;
        double a = h->g.areas[s];
        for (size_t c = 0; c < C; ++c) psi[p * C + c] = m[p * C + c] * a;
      }
      h->bct.multiply_core(kmap, psi, hx);
      for (size_t p = 0; p < nf; ++p)
        for (size_t c = 0; c < C; ++c) {
          double w = c < off ? w_hi : w_lo;
          int kern = c < off ? 0 : 1;
          z[p * C + c] = w * (h->ha_perm[2 * p + kern] * m[p * C + c] - hx[p * C + c]) + 0.0 * m[p * C + c];
        }
      for (int v = 0; v < h->nv; ++v) {
        double acc[3] = {0, 0, 0};
        for (auto [s, c] : h->inc[v]) {
          double a = h->g.areas[s];
          const double *zs = &z[h->bct.position[s] * C];
          if (hi) {
            const v3 &g = h->df[s][c];
            for (int k = 0; k < 3; ++k)
              acc[k] += a * (g[0] * zs[3 * k] + g[1] * zs[3 * k + 1] + g[2] * zs[3 * k + 2]);
          }
          if (lo)
            for (int k = 0; k < 3; ++k) acc[k] += a / 3.0 * zs[off + k];
        }
        for (int k = 0; k < 3; ++k) y[3 * v + k] = 2.0 * acc[k];
      }
    }
  }, g_err);
}

// ---------------------------------------------------------------- VertexFractionalTree

struct rso_vfrac {
  int nv = 0;
  std::vector<v3> pos;
  std::vector<double> mass, ha;
  Bvh bvh;
  std::vector<v3> centroid;
  std::vector<Aabb> bbox;
  std::vector<double> radius;
  KernelIface kern;
  BlockTree bct;
  double expo = 0;
};

int rso_vfrac_build(int nv, const double *pos, const double *mass, double tau, double chi,
                    int leaf_size, int leaf_pairs, rso_vfrac **out) {
  *out = nullptr;
  return guard2([&] {  // hierarchical.rs:1017-1084
    if (!std::isfinite(tau) || nv == 0) throw Error(RSO_INVALID_OPTION, "bad tau or empty");
    auto h = std::make_unique<rso_vfrac>();
    h->nv = nv;
    std::vector<Element> el(nv);
    for (int i = 0; i < nv; ++i) {
      h->pos.push_back({pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]});
      if (!(std::isfinite(mass[i]) && mass[i] > 0)) throw Error(RSO_INVALID_OPTION, "mass");
      h->mass.push_back(mass[i]);
      Aabb b;
      b.grow(h->pos[i]);
      el[i] = {h->pos[i], b, mass[i]};
    }
    h->bvh = Bvh::build(el, leaf_size);
    for (auto &nd : h->bvh.nodes) {
      v3 c = nd.centroid();
      h->centroid.push_back(c);
      h->bbox.push_back(nd.bbox);
      h->radius.push_back(farthest_corner_distance(nd.bbox, c));
    }
    h->expo = -(tau + 1.0);
    rso_vfrac *H = h.get();
    h->kern.N = 1;
    h->kern.admissible = [H, chi](size_t a, size_t b) {
      return separated(H->radius[a], H->bbox[a], H->radius[b], H->bbox[b], chi);
    };
    h->kern.far = [H](size_t a, size_t b, double *o) {
      if (a > b) std::swap(a, b);
      v3 d = sub(H->centroid[a], H->centroid[b]);
      o[0] = std::pow(dot(d, d), H->expo);
    };
    h->kern.near = [H](size_t i, size_t j, double *o) {
      size_t a = std::min(i, j), b = std::max(i, j);
      v3 d = sub(H->pos[a], H->pos[b]);
      o[0] = std::pow(dot(d, d), H->expo);
    };
    h->bct.build(h->bvh, h->kern, (size_t)leaf_pairs);
    h->bct.store_near();
    h->ha = h->bct.multiply({0}, h->mass);
    for (int v = 0; v < nv; ++v)
      if (!std::isfinite(h->ha[v])) throw Error(RSO_INVALID_OPTION, "coincident vertices");
    *out = h.release();
  }, g_err);
}

void rso_vfrac_free(rso_vfrac *h) { delete h; }

int rso_vfrac_stats(const rso_vfrac *h, int64_t *o5) {
  return guard2([&] {
    o5[0] = (int64_t)h->bct.n_adm;
    o5[1] = (int64_t)h->bct.n_near_blocks;
    o5[2] = (int64_t)h->bct.near_entries;
    o5[3] = (int64_t)h->bct.depth;
    o5[4] = (int64_t)h->bct.start.size();
  }, g_err);
}

// y = 2 (a ha x - a H~(a x)) per axis (hierarchical.rs:1313-1345), nb vectors one by one.
int rso_vfrac_apply(const rso_vfrac *h, int nb, const double *xs, double *ys) {
  return guard2([&] {
    size_t nv = h->nv, n3 = 3 * nv;
    for (int q = 0; q < nb; ++q) {
      const double *x = xs + q * n3;
      double *y = ys + q * n3;
      std::vector<double> psi(n3), hx;
      for (size_t p = 0; p < nv; ++p) {
        uint32_t v = h->bct.order[p];
        for (int k = 0; k < 3; ++k) psi[3 * p + k] = h->mass[v] * x[3 * v + k];
      }
      h->bct.multiply_core({0, 0, 0}, psi, hx);
      for (size_t v = 0; v < nv; ++v) {
        double a = h->mass[v];
        const double *hh = &hx[3 * (size_t)h->bct.position[v]];
        for (int k = 0; k < 3; ++k) y[3 * v + k] = 2.0 * a * (h->ha[v] * x[3 * v + k] - hh[k]);
      }
    }
  }, g_err);
}

}  // extern "C"
