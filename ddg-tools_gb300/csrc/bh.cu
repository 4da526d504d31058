// Barnes-Hut tangent-point energy and exact adjoint gradient on the GPU
// (RS/src/energy/barnes_hut.rs, RS/src/kernel.rs, RS/src/geometry.rs), behind the C ABI
// rs_bh_* of include/rsgpu.h.
//
// Per step:   host BVH build (host_tree.cpp) -> device list build (lists_count/lists_fill,
//             radix-sorted transposes).
// Per energy: refit (FP64 face geometry + bottom-up node aggregates, packs FP32 offsets)
//             -> bh_pair (the pair kernel, warp per target leaf)
//             -> node_sums -> downward (per-leaf chain walk) -> final (own + partner +
//             cluster) -> pull_back (per-vertex gather) -> energy reduction (FP64).
// Every reduction has a fixed order (gathers over the transposed lists, fixed shuffle
// trees), so results are bitwise reproducible run to run.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <memory>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

#include "bh_kernels.cuh"
#include "common.hpp"
#include "host_tree.hpp"
#include "profile.hpp"

namespace rsg {

constexpr int kMaxDepth = 96;  // DFS stack bound of the list traversal (checked on the host)

// ------------------------------------------------------------------ refit

// The node centroid in FP64 and as a float pair (hi + lo) for the pair kernel.
__device__ __forceinline__ void store_centroid(const BhDev &d, uint32_t n, double x, double y,
                                               double z, double A) {
  d.ncA[n] = make_double4(x, y, z, A);
  float hx = (float)x, hy = (float)y, hz = (float)z;
  d.nch[n] = make_float4(hx, hy, hz, (float)A);
  d.ncl[n] = make_float4((float)(x - (double)hx), (float)(y - (double)hy), (float)(z - (double)hz), 0.f);
}

// L2-coherent load of a node record written by another thread of the same launch.
__device__ __forceinline__ double4 ldcg4(const double4 *p) {
  const double2 *q = reinterpret_cast<const double2 *>(p);
  double2 a = __ldcg(q), b = __ldcg(q + 1);
  return make_double4(a.x, a.y, b.x, b.y);
}

// One thread per leaf: FP64 face geometry of the leaf's faces (face_quantities,
// RS/src/geometry.rs:33-39), the leaf's area and moment (Bvh::refit order, bvh.rs:226-260),
// the packed FP32 face records relative to the leaf centroid, then the parents bottom-up: the
// second child to arrive at a parent computes it (left + right), so every node is written once
// with the crate's summation order.
__global__ void refit_kernel(BhDev d, const double *__restrict__ pos) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.n_leaves) return;
  uint32_t leaf = d.leaves[k];
  uint32_t s0 = d.node_start[leaf], s1 = d.node_end[leaf];
  double A = 0.0, M0 = 0.0, M1 = 0.0, M2 = 0.0;
  double xb[8][3], ar[8], nr[8][3];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    uint32_t p = s0 + i;
    if (p >= s1) break;
    uint32_t f = d.order[p];
    const double *p0 = pos + 3 * (size_t)d.faces[3 * f];
    const double *p1 = pos + 3 * (size_t)d.faces[3 * f + 1];
    const double *p2 = pos + 3 * (size_t)d.faces[3 * f + 2];
    double u0 = __dsub_rn(p1[0], p0[0]), u1 = __dsub_rn(p1[1], p0[1]), u2 = __dsub_rn(p1[2], p0[2]);
    double w0 = __dsub_rn(p2[0], p0[0]), w1 = __dsub_rn(p2[1], p0[1]), w2 = __dsub_rn(p2[2], p0[2]);
    double c0 = __dsub_rn(__dmul_rn(u1, w2), __dmul_rn(u2, w1));
    double c1 = __dsub_rn(__dmul_rn(u2, w0), __dmul_rn(u0, w2));
    double c2 = __dsub_rn(__dmul_rn(u0, w1), __dmul_rn(u1, w0));
    double len = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(c0, c0), __dmul_rn(c1, c1)), __dmul_rn(c2, c2)));
    const double third = 1.0 / 3.0;
    double x0 = __dmul_rn(__dadd_rn(__dadd_rn(p0[0], p1[0]), p2[0]), third);
    double x1 = __dmul_rn(__dadd_rn(__dadd_rn(p0[1], p1[1]), p2[1]), third);
    double x2 = __dmul_rn(__dadd_rn(__dadd_rn(p0[2], p1[2]), p2[2]), third);
    double a = __dmul_rn(0.5, len);
    double il = __drcp_rn(len);
    nr[i][0] = __dmul_rn(c0, il);
    nr[i][1] = __dmul_rn(c1, il);
    nr[i][2] = __dmul_rn(c2, il);
    xb[i][0] = x0, xb[i][1] = x1, xb[i][2] = x2, ar[i] = a;
    A = __dadd_rn(A, a);
    M0 = __dadd_rn(M0, __dmul_rn(a, x0));
    M1 = __dadd_rn(M1, __dmul_rn(a, x1));
    M2 = __dadd_rn(M2, __dmul_rn(a, x2));
  }
  double cx = __ddiv_rn(M0, A), cy = __ddiv_rn(M1, A), cz = __ddiv_rn(M2, A);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    uint32_t p = s0 + i;
    if (p >= s1) break;
    double o0 = xb[i][0] - cx, o1 = xb[i][1] - cy, o2 = xb[i][2] - cz;
    float h0 = (float)o0, h1 = (float)o1, h2 = (float)o2;
    // alpha = N . (X - X_leaf) as a float pair: hi in fnl.w, lo in fol.w
    double alpha = nr[i][0] * o0 + nr[i][1] * o1 + nr[i][2] * o2;
    float al = (float)alpha;
    d.fxa[p] = make_float4(h0, h1, h2, (float)ar[i]);
    d.fol[p] = make_float4((float)(o0 - (double)h0), (float)(o1 - (double)h1), (float)(o2 - (double)h2),
                           (float)(alpha - (double)al));
    float n0 = (float)nr[i][0], n1 = (float)nr[i][1], n2 = (float)nr[i][2];
    d.fnn[p] = make_float4(n0, n1, n2, 0.f);
    d.fnl[p] = make_float4((float)(nr[i][0] - (double)n0), (float)(nr[i][1] - (double)n1),
                           (float)(nr[i][2] - (double)n2), al);
  }
  d.nmom[leaf] = make_double4(M0, M1, M2, A);
  store_centroid(d, leaf, cx, cy, cz, A);
  uint32_t n = leaf;
  while (n != 0) {
    uint32_t par = d.node_parent[n];
    __threadfence();
    unsigned old = atomicAdd(&d.refit_count[par], 1u);
    if ((old & 1u) == 0u) return;  // first child here: the sibling completes the parent
    __threadfence();
    double4 l = ldcg4(&d.nmom[par + 1]);
    double4 r = ldcg4(&d.nmom[d.node_right[par]]);
    double4 m = make_double4(__dadd_rn(l.x, r.x), __dadd_rn(l.y, r.y), __dadd_rn(l.z, r.z),
                             __dadd_rn(l.w, r.w));
    d.nmom[par] = m;
    store_centroid(d, par, __ddiv_rn(m.x, m.w), __ddiv_rn(m.y, m.w), __ddiv_rn(m.z, m.w), m.w);
    n = par;
  }
}

// ------------------------------------------------------------------ interaction lists

struct ListsDev {
  const double *box;     // 6 per node (build positions)
  const double *radius;  // per node
  double theta2;
};

// bh_admissible (RS/src/spatial/mod.rs:131-163): max(r_l, r_c)^2 < theta^2 d_box^2, in FP64
// without contraction so the lists match the crate's bit for bit.
__device__ __forceinline__ bool admissible(const ListsDev &L, const double *lb, double lr,
                                           uint32_t c) {
  const double *cb = L.box + 6 * (size_t)c;
  double d2 = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double dd = fmax(__dsub_rn(fmax(lb[k], cb[k]), fmin(lb[3 + k], cb[3 + k])), 0.0);
    d2 = __dadd_rn(d2, __dmul_rn(dd, dd));
  }
  double h = fmax(lr, L.radius[c]);
  return __dmul_rn(h, h) < __dmul_rn(L.theta2, d2);
}

// The lists of a leaf: a depth-first traversal from the root, left child first
// (barnes_hut.rs:752-766): an admissible node is lumped, an inadmissible leaf is exact, any
// other node is opened. The traversal is cut into ordered segments so that it runs in
// parallel: lists_top_kernel walks the tree down to depth kTopDepth and records, in traversal
// order, the entries met there and the depth-kTopDepth nodes it has to open (subtree roots);
// lists_seg_kernel runs the traversal of each segment, counting (FILL=false) or writing at the
// segment's offsets (FILL=true): one thread per slot for the single entries, one thread per
// subtree from a compact work list for the rest (so that the warps that walk subtrees are full;
// most segments are single entries); lists_scan_kernel turns a leaf's segment counts into
// offsets. The concatenated segments are the sequential traversal's lists, entry for entry.
constexpr int kTopDepth = 5;
constexpr int kSegs = 64;  // at most one segment per node of depth <= kTopDepth: 63
constexpr uint32_t kSegNode = 0x3fffffffu;

struct LeafBox {
  double lb[6], lr;
  uint32_t leaf, ns;
};
__device__ __forceinline__ LeafBox leaf_box(const BhDev &d, const ListsDev &L, uint32_t k) {
  LeafBox b;
  b.leaf = d.leaves[k];
#pragma unroll
  for (int i = 0; i < 6; ++i) b.lb[i] = L.box[6 * (size_t)b.leaf + i];
  b.lr = L.radius[b.leaf];
  b.ns = d.node_end[b.leaf] - d.node_start[b.leaf];
  return b;
}

// seg[k][i] = node | kind << 30 (0 lumped node, 1 exact leaf, 2 opened node of depth
// kTopDepth: its subtree's traversal), nseg[k] of them; the kind-2 slots k kSegs + i are also
// appended to the work list `heavy` (in any order: each slot's results have their own place)
__global__ void lists_top_kernel(BhDev d, ListsDev L, uint32_t *seg, uint32_t *nseg, uint32_t *heavy,
                                 uint32_t *n_heavy, unsigned int *overflow) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (uint32_t)d.n_leaves) return;
  const LeafBox B = leaf_box(d, L, k);
  uint32_t st[2 * kTopDepth + 4];
  int sd[2 * kTopDepth + 4];
  int sp = 0, n = 0;
  st[sp] = 0, sd[sp++] = 0;
  uint32_t *out = seg + (size_t)k * kSegs;
  while (sp > 0) {
    --sp;
    const uint32_t c = st[sp];
    const int dep = sd[sp];
    uint32_t code;
    if (admissible(L, B.lb, B.lr, c)) {
      code = c;
    } else if (d.node_right[c] == 0) {
      code = c | (1u << 30);
    } else if (dep == kTopDepth) {
      code = c | (2u << 30);
    } else {
      st[sp] = d.node_right[c], sd[sp++] = dep + 1;
      st[sp] = c + 1, sd[sp++] = dep + 1;
      continue;
    }
    if (n == kSegs) {
      atomicExch(overflow, 1u);
      break;
    }
    if ((code >> 30) == 2u) heavy[atomicAdd(n_heavy, 1u)] = k * kSegs + (uint32_t)n;
    out[n++] = code;
  }
  nseg[k] = (uint32_t)n;
}

// HEAVY = false: one thread per slot, the single-entry segments (kinds 0, 1); HEAVY = true:
// one thread per work-list entry, the subtree traversals (kind 2).
template <bool FILL, bool HEAVY>
__global__ void lists_seg_kernel(BhDev d, ListsDev L, const uint32_t *seg, const uint32_t *nseg,
                                 const uint32_t *heavy, const uint32_t *n_heavy, uint32_t *s_lum, uint32_t *s_ex,
                                 uint32_t *s_par, unsigned long long *s_pr, uint32_t *lumped, uint32_t *exact,
                                 uint32_t *partner_off, const uint32_t *partner_base, unsigned int *overflow) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (HEAVY) {
    if (t >= *n_heavy) return;
    t = heavy[t];
  }
  const uint32_t k = (uint32_t)(t / kSegs), i = (uint32_t)(t % kSegs);
  if (k >= (uint32_t)d.n_leaves || i >= nseg[k]) return;
  if (HEAVY != ((seg[t] >> 30) == 2u)) return;
  const LeafBox B = leaf_box(d, L, k);
  uint32_t nl = 0, ne = 0, np = 0;
  unsigned long long pr = 0;
  const uint32_t lo = FILL ? d.lumped_off[k] + s_lum[t] : 0, eo = FILL ? d.exact_off[k] + s_ex[t] : 0;
  const uint32_t pb = FILL ? partner_base[k] + s_par[t] : 0;
  auto lump = [&](uint32_t c) {
    if (FILL) lumped[lo + nl] = c;
    ++nl;
  };
  auto exact_leaf = [&](uint32_t c) {
    const uint32_t nc = d.node_end[c] - d.node_start[c];
    if (FILL) {
      exact[eo + ne] = c;
      partner_off[eo + ne] = pb + np;
    }
    ++ne;
    np += nc;
    pr += (c == B.leaf) ? (unsigned long long)B.ns * (B.ns - 1) : (unsigned long long)B.ns * nc;
  };
  const uint32_t code = seg[t], c0 = code & kSegNode, kind = code >> 30;
  if (kind == 0) {
    lump(c0);
  } else if (kind == 1) {
    exact_leaf(c0);
  } else {
    uint32_t stack[kMaxDepth];
    int sp = 0;
    stack[sp++] = d.node_right[c0];  // c0 was tested (inadmissible, not a leaf): open it
    stack[sp++] = c0 + 1;
    while (sp > 0) {
      const uint32_t c = stack[--sp];
      if (admissible(L, B.lb, B.lr, c)) {
        lump(c);
      } else if (d.node_right[c] == 0) {
        exact_leaf(c);
      } else {
        if (sp + 2 > kMaxDepth) {
          atomicExch(overflow, 1u);
          break;
        }
        stack[sp++] = d.node_right[c];
        stack[sp++] = c + 1;
      }
    }
  }
  if (!FILL) s_lum[t] = nl, s_ex[t] = ne, s_par[t] = np, s_pr[t] = pr;
}

// One warp per leaf: the segment counts become exclusive offsets within the leaf (in place),
// the leaf's totals go to the per-leaf arrays (pairs: exact element pairs; lum_inter: lumped
// nodes x the leaf's faces).
__global__ void lists_scan_kernel(BhDev d, const uint32_t *nseg, uint32_t *s_lum, uint32_t *s_ex, uint32_t *s_par,
                                  const unsigned long long *s_pr, uint32_t *cnt_lum, uint32_t *cnt_ex,
                                  uint32_t *cnt_partner, unsigned long long *pairs, unsigned long long *lum_inter) {
  const uint32_t k = (uint32_t)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= (uint32_t)d.n_leaves) return;
  static_assert(kSegs == 64, "two segments per lane");
  const uint32_t n = nseg[k];
  const size_t b = (size_t)k * kSegs + 2 * lane;
  const bool v0 = 2u * lane < n, v1 = 2u * lane + 1 < n;
  uint32_t *arr[3] = {s_lum, s_ex, s_par};
  uint32_t tot[3];
  for (int a = 0; a < 3; ++a) {
    const uint32_t x0 = v0 ? arr[a][b] : 0u, x1 = v1 ? arr[a][b + 1] : 0u;
    uint32_t inc = x0 + x1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    const uint32_t exc = inc - (x0 + x1);
    if (v0) arr[a][b] = exc;
    if (v1) arr[a][b + 1] = exc + x0;
    tot[a] = __shfl_sync(0xffffffffu, inc, 31);
  }
  unsigned long long p = (v0 ? s_pr[b] : 0ull) + (v1 ? s_pr[b + 1] : 0ull);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
  if (lane == 0) {
    const uint32_t leaf = d.leaves[k], ns = d.node_end[leaf] - d.node_start[leaf];
    cnt_lum[k] = tot[0], cnt_ex[k] = tot[1], cnt_partner[k] = tot[2];
    pairs[k] = p;
    lum_inter[k] = (unsigned long long)tot[0] * ns;
  }
}

__global__ void iota_kernel(uint32_t *v, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = i;
}

__global__ void leaf_key_kernel(const uint32_t *exact, const uint32_t *leaf_ordinal_of_node,
                                uint32_t *key, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) key[i] = leaf_ordinal_of_node[exact[i]];
}

// Group boundaries of sorted keys -> CSR offsets (off[k] = first index with key >= k).
__global__ void offsets_from_sorted(const uint32_t *key, uint32_t n, uint32_t m, uint32_t *off) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  uint32_t prev = (i == 0) ? 0 : key[i - 1] + 1;
  uint32_t cur = (i == n) ? m : key[i];
  for (uint32_t k = prev; k <= cur; ++k) off[k] = i;
}

// ------------------------------------------------------------------ the pair kernel

// Error-free product and sum (Dekker/Knuth with FMA): a*b = p + e, a+b = s + t exactly.
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
  p = a * b;
  e = fmaf(a, b, -p);
}
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &t) {
  s = a + b;
  float bv = s - a;
  t = (a - (s - bv)) + (b - bv);
}

// N . o for a unit normal and an offset both held as float pairs (hi + lo), compensated
// (the Dot2 scheme of Ogita, Rump and Oishi, 2005): the sum of the three products carries its
// rounding errors, which matters because it nearly cancels for a smooth surface.
// The result is left unrounded as u + lo.
__device__ __forceinline__ void dot2(float nx, float ny, float nz, float lx, float ly, float lz,
                                     float ox, float oy, float oz, float px, float py, float pz,
                                     float &u, float &lo) {
  float p0, e0, p1, e1, p2, e2, s, t0, t1;
  two_prod(nx, ox, p0, e0);
  two_prod(ny, oy, p1, e1);
  two_prod(nz, oz, p2, e2);
  two_sum(p0, p1, s, t0);
  two_sum(s, p2, u, t1);
  lo = ((e0 + e1) + (e2 + t0)) + t1;
  lo += (nx * px + ny * py + nz * pz) + (lx * ox + ly * oy + lz * oz);
}

// X_L - X_C from two centroids held as float pairs, as a float pair (h + l) per axis.
__device__ __forceinline__ void pair_diff(const float4 &ah, const float4 &al, const float4 &bh,
                                          const float4 &bl, float (&h)[3], float (&l)[3]) {
  float t0, t1, t2;
  two_sum(ah.x, -bh.x, h[0], t0);
  two_sum(ah.y, -bh.y, h[1], t1);
  two_sum(ah.z, -bh.z, h[2], t2);
  l[0] = t0 + (al.x - bl.x);
  l[1] = t1 + (al.y - bl.y);
  l[2] = t2 + (al.z - bl.z);
}

// Per-warp staging of the pair kernel in shared memory (one batch of up to kBatch sources).
constexpr int kBatch = 64;
struct PairStage {
  // lumped: per node entry, X_L - X_C rounded to FP32 (xyz) and A_C (w);
  // exact: per source face T, y_T = X_T - X_L as a float pair: hi (xyz) with a_T (w), lo (xyz)
  // with T's slot in the target leaf when C = L, else -1 (w, integer bits)
  float4 src_hi[kBatch], src_lo[kBatch];
  uint32_t src_slot[kBatch];            // exact: partner slot of each staged face
  float4 ent_h[32], ent_l[32];          // exact: X_L - X_C of each entry as a float pair
  uint32_t ent_cs[32], ent_po[32], ent_first[32];
  uint8_t fmap[256];                    // exact: entry of every face of the chunk
  float4 red[264];                      // per (target slot s, source e): the terms summed over s;
                                        // ns (8 G + 1) <= 264 for every leaf size ns <= 8
};

// The pair kernel. One warp per work item: a slice of one target leaf's lumped and exact
// lists (leaf size <= 8; long lists are split so that no warp carries a whole-mesh leaf).
// Lanes are (group g, target face s) = g ns + s for the leaf's ns faces and G = min(8, 32/ns)
// groups, so that 24-32 lanes work whatever the leaf size. Sources go through shared memory in
// batches of 8 G: lumped nodes (one per entry) and the faces of exact leaves (flattened over
// up to 32 entries at a time); group g takes sources g, g + G, ... The per-source terms
// (node terms b = sum_S a_S K, u = -sum_S a_S dK/dv, and the exact partner terms) are summed
// over s from shared memory in fixed order; own partials and the energy go through Kahan
// accumulators and are written per work item (leaf_with_gradient, barnes_hut.rs:627-689;
// value only: leaf_energy, barnes_hut.rs:583-614).
//
// Lumped nodes are admissible, so |v| is at least the node's size over theta and
// nu = alpha_S + N_S.(X_L - X_C) keeps FP32 relative precision in plain arithmetic. Exact
// pairs are near: on a smooth surface nu is ~|v|^2 kappa, far below |v|, plain FP32 loses it,
// and the differential (large terms that cancel around every vertex) inherits the loss. So
// nu = alpha_S - N_S.y_T with y_T = X_T - X_L held as a float pair and a compensated dot
// product, and v = X_S - X_T is summed with its rounding error (leaf offsets can be large next
// to |v| in a stretched leaf). alpha_S = N_S.(X_S - X_L) is a float pair from the FP64 refit.
template <bool GRAD, bool FAST>
__global__ void __launch_bounds__(128, 6) bh_pair_kernel(BhDev d, Pow pw) {
  __shared__ PairStage stage[4];
  PairStage &st = stage[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned int w = 0;
    if (lane == 0) w = atomicAdd(d.ticket, 1u);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= (unsigned)d.n_items) return;
    const uint32_t item = d.schedule[w];
    const uint4 it = d.items[item];  // lumped [x, y), exact [z, w) entry ranges
    const uint32_t k = d.item_leaf[item];
    const uint32_t leaf = d.leaves[k];
    const uint32_t s0 = d.node_start[leaf];
    const int ns = (int)(d.node_end[leaf] - s0);
    const int G = min(8, 32 / ns), B = 8 * G, RS = B + 1;
    const int g = lane / ns, s = lane - g * ns;
    const bool act = g < G;
    const float4 xs = act ? d.fxa[s0 + s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 nS = act ? d.fnn[s0 + s] : make_float4(0.f, 0.f, 1.f, 0.f);
    const float4 nL = act ? d.fnl[s0 + s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 xsl = act ? d.fol[s0 + s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 cLh = d.nch[leaf], cLl = d.ncl[leaf];
    const float a_s = xs.w;
    Kahan e_acc, da_acc, dx0, dx1, dx2, dn0, dn1, dn2;

    // ---- lumped nodes
    const uint32_t llo = it.x, lhi = it.y;
    for (uint32_t base = llo; base < lhi; base += B) {
      const int cnt = (int)min((uint32_t)B, lhi - base);
      __syncwarp();
      for (int e = lane; e < cnt; e += 32) {
        const uint32_t c = d.lumped[base + e];
        const float4 ch = d.nch[c], cl = d.ncl[c];
        float h[3], l[3];
        pair_diff(cLh, cLl, ch, cl, h, l);
        st.src_hi[e] = make_float4(h[0] + l[0], h[1] + l[1], h[2] + l[2], ch.w);
      }
      __syncwarp();
      float bda = 0.f, be = 0.f, bx0 = 0.f, bx1 = 0.f, bx2 = 0.f, bn0 = 0.f, bn1 = 0.f, bn2 = 0.f;
#pragma unroll 2
      for (int i = 0; i < 8; ++i) {
        const int e = g + G * i;
        if (!act || e >= cnt) continue;
        const float4 nd = st.src_hi[e];
        const float v0 = xs.x + nd.x, v1 = xs.y + nd.y, v2 = xs.z + nd.z;
        const float u = fmaf(nS.z, nd.z, fmaf(nS.y, nd.y, nS.x * nd.x));
        const float nu = nL.w + (u + xsl.w);
        const float r2 = v0 * v0 + v1 * v1 + v2 * v2;
        const float ir2 = __fdividef(1.f, r2);
        float K, cn;
        kernel_k<FAST>(pw, nu, r2, ir2, K, cn);
        const float Ac = nd.w;
        be += a_s * K * Ac;
        if (GRAD) {
          const float gg = pw.beta * K * ir2;
          const float dv0 = cn * nS.x - gg * v0, dv1 = cn * nS.y - gg * v1, dv2 = cn * nS.z - gg * v2;
          bda += K * Ac;
          const float aa = a_s * Ac;
          bx0 += aa * dv0, bx1 += aa * dv1, bx2 += aa * dv2;
          const float ac = aa * cn;
          bn0 += ac * v0, bn1 += ac * v1, bn2 += ac * v2;
          st.red[s * RS + e] = make_float4(a_s * K, -a_s * dv0, -a_s * dv1, -a_s * dv2);
        }
      }
      e_acc.add(be);
      if (GRAD) {
        da_acc.add(bda);
        dx0.add(bx0), dx1.add(bx1), dx2.add(bx2);
        dn0.add(bn0), dn1.add(bn1), dn2.add(bn2);
        __syncwarp();
        for (int e = lane; e < cnt; e += 32) {
          float4 t = st.red[e];
          for (int r = 1; r < ns; ++r) {
            const float4 q = st.red[r * RS + e];
            t.x += q.x, t.y += q.y, t.z += q.z, t.w += q.w;
          }
          d.node_term[base + e] = t;
        }
      }
    }

    // ---- exact leaves, up to 32 entries at a time, their faces flattened
    const uint32_t elo = it.z, ehi = it.w;
    for (uint32_t cb = elo; cb < ehi; cb += 32) {
      const int ncnt = (int)min(32u, ehi - cb);
      __syncwarp();
      uint32_t nc = 0;
      if (lane < ncnt) {
        const uint32_t q = cb + lane;
        const uint32_t c = d.exact[q];
        const uint32_t cs = d.node_start[c];
        nc = d.node_end[c] - cs;
        float h[3], l[3];
        pair_diff(cLh, cLl, d.nch[c], d.ncl[c], h, l);  // X_L - X_C
        st.ent_h[lane] = make_float4(h[0], h[1], h[2], 0.f);
        st.ent_l[lane] = make_float4(l[0], l[1], l[2], __int_as_float(c == leaf ? 1 : 0));
        st.ent_cs[lane] = cs;
        st.ent_po[lane] = d.partner_off[q];
      }
      uint32_t incl = nc;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      const int FT = (int)__shfl_sync(0xffffffffu, incl, 31);
      if (lane < ncnt) {
        st.ent_first[lane] = incl - nc;
        for (uint32_t t = 0; t < nc; ++t) st.fmap[incl - nc + t] = (uint8_t)lane;
      }
      for (int fb = 0; fb < FT; fb += B) {
        const int cnt = min(B, FT - fb);
        __syncwarp();
        for (int f = lane; f < cnt; f += 32) {
          const int i = st.fmap[fb + f];
          const uint32_t t = (uint32_t)(fb + f) - st.ent_first[i];
          const uint32_t p = st.ent_cs[i] + t;
          const float4 xt = d.fxa[p], xl = d.fol[p];
          const float4 hh = st.ent_h[i], ll = st.ent_l[i];
          // y_T = x_T - (X_L - X_C) as a float pair
          float y0, y1, y2, e0, e1, e2;
          two_sum(xt.x, -hh.x, y0, e0);
          two_sum(xt.y, -hh.y, y1, e1);
          two_sum(xt.z, -hh.z, y2, e2);
          st.src_hi[f] = make_float4(y0, y1, y2, xt.w);
          st.src_lo[f] = make_float4(e0 + (xl.x - ll.x), e1 + (xl.y - ll.y), e2 + (xl.z - ll.z),
                                     __int_as_float(__float_as_int(ll.w) ? (int)t : -1));
          st.src_slot[f] = st.ent_po[i] + t;
        }
        __syncwarp();
        float row = 0.f, rx0 = 0.f, rx1 = 0.f, rx2 = 0.f, rn0 = 0.f, rn1 = 0.f, rn2 = 0.f;
#pragma unroll 2
        for (int i = 0; i < 8; ++i) {
          const int f = g + G * i;
          if (!act || f >= cnt) continue;
          const float4 yh = st.src_hi[f], yl = st.src_lo[f];
          const float a_t = yh.w;
          float K = 0.f, cn = 0.f, gg = 0.f, v0 = 0.f, v1 = 0.f, v2 = 0.f;
          if (__float_as_int(yl.w) != s) {
            float w0, w1, w2, e0, e1, e2;
            two_sum(xs.x, -yh.x, w0, e0);
            two_sum(xs.y, -yh.y, w1, e1);
            two_sum(xs.z, -yh.z, w2, e2);
            v0 = w0 + (e0 + (xsl.x - yl.x));
            v1 = w1 + (e1 + (xsl.y - yl.y));
            v2 = w2 + (e2 + (xsl.z - yl.z));
            const float r2 = v0 * v0 + v1 * v1 + v2 * v2;
            const float ir2 = __fdividef(1.f, r2);
            float ph, pl, sh, se;
            dot2(nS.x, nS.y, nS.z, nL.x, nL.y, nL.z, yh.x, yh.y, yh.z, yl.x, yl.y, yl.z, ph, pl);
            two_sum(nL.w, -ph, sh, se);
            const float nu = sh + (se + (xsl.w - pl));
            kernel_k<FAST>(pw, nu, r2, ir2, K, cn);
            gg = pw.beta * K * ir2;
          }
          row += a_t * K;
          if (GRAD) {
            const float dv0 = cn * nS.x - gg * v0, dv1 = cn * nS.y - gg * v1, dv2 = cn * nS.z - gg * v2;
            rx0 += a_t * dv0, rx1 += a_t * dv1, rx2 += a_t * dv2;
            const float tc = a_t * cn;
            rn0 += tc * v0, rn1 += tc * v1, rn2 += tc * v2;
            const float aa = -a_s * a_t;
            st.red[s * RS + f] = make_float4(a_s * K, aa * dv0, aa * dv1, aa * dv2);
          }
        }
        e_acc.add(a_s * row);
        if (GRAD) {
          da_acc.add(row);
          dx0.add(a_s * rx0), dx1.add(a_s * rx1), dx2.add(a_s * rx2);
          dn0.add(a_s * rn0), dn1.add(a_s * rn1), dn2.add(a_s * rn2);
          __syncwarp();
          for (int f = lane; f < cnt; f += 32) {
            float4 t = st.red[f];
            for (int r = 1; r < ns; ++r) {
              const float4 q = st.red[r * RS + f];
              t.x += q.x, t.y += q.y, t.z += q.z, t.w += q.w;
            }
            d.partner[st.src_slot[f]] = t;
          }
        }
      }
    }

    // ---- own partials summed over the groups in order; lanes 0..7 write the item's slots
    if (GRAD) {
      __syncwarp();
      if (act) {
        st.red[2 * (g * 8 + s)] = make_float4(da_acc.value(), dx0.value(), dx1.value(), dx2.value());
        st.red[2 * (g * 8 + s) + 1] = make_float4(dn0.value(), dn1.value(), dn2.value(), 0.f);
      }
      __syncwarp();
      if (lane < 8) {
        float4 o0 = make_float4(0.f, 0.f, 0.f, 0.f), o1 = o0;
        if (lane < ns) {
          o0 = st.red[2 * lane], o1 = st.red[2 * lane + 1];
          for (int r = 1; r < G; ++r) {
            const float4 p0 = st.red[2 * (r * 8 + lane)], p1 = st.red[2 * (r * 8 + lane) + 1];
            o0.x += p0.x, o0.y += p0.y, o0.z += p0.z, o0.w += p0.w;
            o1.x += p1.x, o1.y += p1.y, o1.z += p1.z;
          }
        }
        d.own[16 * (size_t)item + 2 * lane] = o0;
        d.own[16 * (size_t)item + 2 * lane + 1] = o1;
      }
    }
    double e = (double)e_acc.s - (double)e_acc.c;
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) e += __shfl_xor_sync(0xffffffffu, e, m);
    if (lane == 0) d.item_energy[item] = e;
  }
}

// b_C, u_C per node over the transposed lumped lists (barnes_hut.rs:505-520): one warp per
// node, lanes strided over the entries (Kahan), then a fixed shuffle tree.
// Node terms summed per chunk of a node's transposed lumped list (one warp per chunk), then
// per node over its chunks in order.
__global__ void node_partial_kernel(BhDev d) {
  int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (w >= d.n_nchunks) return;
  const uint4 ch = d.nchunk[w];
  Kahan b, u0, u1, u2;
  for (uint32_t e = ch.y + lane; e < ch.z; e += 32) {
    float4 t = d.node_term[d.lumped_t[e]];
    b.add(t.x), u0.add(t.y), u1.add(t.z), u2.add(t.w);
  }
  float r0 = b.value(), r1 = u0.value(), r2 = u1.value(), r3 = u2.value();
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    r0 += __shfl_xor_sync(0xffffffffu, r0, m);
    r1 += __shfl_xor_sync(0xffffffffu, r1, m);
    r2 += __shfl_xor_sync(0xffffffffu, r2, m);
    r3 += __shfl_xor_sync(0xffffffffu, r3, m);
  }
  if (lane == 0) d.npart[w] = make_float4(r0, r1, r2, r3);
}

__global__ void node_sums_kernel(BhDev d) {
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= d.n_nodes) return;
  float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
  for (uint32_t c = d.nchunk_off[n]; c < d.nchunk_off[n + 1]; ++c) {
    const float4 p = d.npart[c];
    s.x += p.x, s.y += p.y, s.z += p.z, s.w += p.w;
  }
  d.node_sum[n] = s;
}

// Downward pass per leaf along its root -> leaf chain (barnes_hut.rs:521-538), in FP64 (about
// 20 steps per leaf): beta_c = beta_p + U_p.(X_c - X_p) + b_c, U_c = U_p + u_c.
__global__ void downward_kernel(BhDev d) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.n_leaves) return;
  uint32_t c0 = d.chain_off[k], c1 = d.chain_off[k + 1];
  uint32_t p = d.chain[c0];
  float4 s = d.node_sum[p];
  double beta = s.x, U0 = s.y, U1 = s.z, U2 = s.w;
  double4 xp = d.ncA[p];
  for (uint32_t i = c0 + 1; i < c1; ++i) {
    uint32_t c = d.chain[i];
    double4 xc = d.ncA[c];
    float4 sc = d.node_sum[c];
    beta = beta + (U0 * (xc.x - xp.x) + U1 * (xc.y - xp.y) + U2 * (xc.z - xp.z)) + (double)sc.x;
    U0 += sc.y, U1 += sc.z, U2 += sc.w;
    xp = xc;
  }
  d.leaf_bu[k] = make_float4((float)beta, (float)U0, (float)U1, (float)U2);
}

// Partner sums per chunk of a leaf's transposed exact list (one warp per chunk): lanes stride
// over the chunk's entries, each summing the leaf's (<= 8) partner slots of an entry into
// 8 x 4 registers; a transposing reduce over the 32 lanes leaves lane 4 t + c with component c
// of face t, written to the chunk's 32 partial sums.
__global__ void final_partial_kernel(BhDev d) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= d.n_fchunks) return;
  const uint4 ch = d.fchunk[w];
  const uint32_t leaf = d.leaves[ch.x];
  const uint32_t ns = d.node_end[leaf] - d.node_start[leaf];
  float acc[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) acc[i] = 0.f;
  for (uint32_t e = ch.y + lane; e < ch.z; e += 32) {
    const float4 *pp = d.partner + d.partner_off[d.exact_t[e]];
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if ((uint32_t)t < ns) {
        float4 v = pp[t];
        acc[4 * t] += v.x, acc[4 * t + 1] += v.y, acc[4 * t + 2] += v.z, acc[4 * t + 3] += v.w;
      }
  }
  // 32 -> 16 -> 8 -> 4 -> 2 -> 1 values per lane; lane L ends with the sum of acc[L]
  float r16[16], r8[8], r4[4], r2[2];
  const bool b4 = (lane >> 4) & 1, b3 = (lane >> 3) & 1, b2 = (lane >> 2) & 1, b1 = (lane >> 1) & 1,
             b0 = lane & 1;
#pragma unroll
  for (int i = 0; i < 16; ++i)
    r16[i] = (b4 ? acc[16 + i] : acc[i]) + __shfl_xor_sync(0xffffffffu, b4 ? acc[i] : acc[16 + i], 16);
#pragma unroll
  for (int i = 0; i < 8; ++i)
    r8[i] = (b3 ? r16[8 + i] : r16[i]) + __shfl_xor_sync(0xffffffffu, b3 ? r16[i] : r16[8 + i], 8);
#pragma unroll
  for (int i = 0; i < 4; ++i)
    r4[i] = (b2 ? r8[4 + i] : r8[i]) + __shfl_xor_sync(0xffffffffu, b2 ? r8[i] : r8[4 + i], 4);
#pragma unroll
  for (int i = 0; i < 2; ++i)
    r2[i] = (b1 ? r4[2 + i] : r4[i]) + __shfl_xor_sync(0xffffffffu, b1 ? r4[i] : r4[2 + i], 2);
  d.fpart[32 * (size_t)w + lane] = (b0 ? r2[1] : r2[0]) + __shfl_xor_sync(0xffffffffu, b0 ? r2[0] : r2[1], 1);
}

// Per leaf (one warp, lane 4 t + c = component c of face t): own + partner (the leaf's chunks in
// order) + cluster part (barnes_hut.rs:539-567), written by face id.
__global__ void final_kernel(BhDev d) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (k >= d.n_leaves) return;
  const uint32_t leaf = d.leaves[k];
  const uint32_t s0 = d.node_start[leaf];
  const uint32_t ns = d.node_end[leaf] - s0;
  const uint32_t t = lane >> 2, c = lane & 3;
  if (t >= ns) return;
  float part = 0.f;
  for (uint32_t ch = d.fchunk_off[k]; ch < d.fchunk_off[k + 1]; ++ch) part += d.fpart[32 * (size_t)ch + lane];
  const uint32_t p = s0 + t;
  const float *ow = reinterpret_cast<const float *>(d.own);
  float own = 0.f, ownn = 0.f;
  for (uint32_t i = d.item_off[k]; i < d.item_off[k + 1]; ++i) {  // 64 floats per item
    own += ow[64 * (size_t)i + 8 * t + c];
    ownn += ow[64 * (size_t)i + 8 * t + 4 + c];
  }
  const float4 bu = d.leaf_bu[k];
  const float4 xa = d.fxa[p];  // offset X_T - X_leaf and a_T
  float cl;
  if (c == 0) cl = bu.x + (bu.y * xa.x + bu.z * xa.y + bu.w * xa.z);
  else cl = xa.w * (c == 1 ? bu.y : (c == 2 ? bu.z : bu.w));
  const uint32_t f = d.order[p];
  float *out = reinterpret_cast<float *>(d.partials);
  out[8 * (size_t)f + c] = (own + part) + cl;
  out[8 * (size_t)f + 4 + c] = ownn;
}

// Pull-back to the vertices (face_pull_back, RS/src/geometry.rs:87-110, summed over the
// incident faces in increasing face order, geometry.rs:172-188), in FP64: the face terms
// around a vertex cancel to a small differential, so this O(F) step keeps FP64.
__global__ void pull_back_kernel(BhDev d, const double *__restrict__ pos, double *__restrict__ dE) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= d.n_vertices) return;
  double g0 = 0.0, g1 = 0.0, g2 = 0.0;
  const float *pa_ = reinterpret_cast<const float *>(d.partials);
  for (uint32_t e = d.inc_off[v]; e < d.inc_off[v + 1]; ++e) {
    uint32_t fc = d.inc[e];
    uint32_t f = fc >> 2, c = fc & 3;
    const uint32_t *t = d.faces + 3 * (size_t)f;
    const double *p0 = pos + 3 * (size_t)t[0];
    const double *p1 = pos + 3 * (size_t)t[1];
    const double *p2 = pos + 3 * (size_t)t[2];
    double u0 = p1[0] - p0[0], u1 = p1[1] - p0[1], u2 = p1[2] - p0[2];
    double w0 = p2[0] - p0[0], w1 = p2[1] - p0[1], w2 = p2[2] - p0[2];
    double n0 = u1 * w2 - u2 * w1, n1 = u2 * w0 - u0 * w2, n2 = u0 * w1 - u1 * w0;
    double len = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    double il = 1.0 / len;
    n0 *= il, n1 *= il, n2 *= il;
    // edge opposite corner c: e_jk = p2 - p1, e_ki = p0 - p2, e_ij = p1 - p0
    const double *pa = c == 0 ? p1 : (c == 1 ? p2 : p0);
    const double *pb = c == 0 ? p2 : (c == 1 ? p0 : p1);
    double e0 = pb[0] - pa[0], e1 = pb[1] - pa[1], e2 = pb[2] - pa[2];
    const float *q = pa_ + 8 * (size_t)f;
    double ha = 0.5 * (double)q[0];
    double c0 = n1 * e2 - n2 * e1, c1 = n2 * e0 - n0 * e2, c2 = n0 * e1 - n1 * e0;  // N x e
    double dotn = -(c0 * (double)q[4] + c1 * (double)q[5] + c2 * (double)q[6]) * il;
    const double third = 1.0 / 3.0;
    g0 += ha * c0 + (double)q[1] * third + n0 * dotn;
    g1 += ha * c1 + (double)q[2] * third + n1 * dotn;
    g2 += ha * c2 + (double)q[3] * third + n2 * dotn;
  }
  dE[3 * v] = g0, dE[3 * v + 1] = g1, dE[3 * v + 2] = g2;
}

// Energy over the leaves in FP64: fixed strided partial sums, then a fixed tree.
__global__ void energy_reduce_kernel(const double *leaf_energy, int n, double *out) {
  __shared__ double sh[1024];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += leaf_energy[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int m = blockDim.x / 2; m > 0; m >>= 1) {
    if ((int)threadIdx.x < m) sh[threadIdx.x] += sh[threadIdx.x + m];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// First exact pair in leaf, list, s, t order whose FP32 term is non-finite (culprit_pair,
// barnes_hut.rs:693-724): the smallest (entry << 8 | s << 4 | t) rank.
template <bool FAST>
__global__ void culprit_kernel(BhDev d, Pow pw, unsigned long long *best) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.n_leaves) return;
  uint32_t leaf = d.leaves[k];
  uint32_t s0 = d.node_start[leaf], s1 = d.node_end[leaf];
  double4 cL = d.ncA[leaf];
  for (uint32_t q = d.exact_off[k]; q < d.exact_off[k + 1]; ++q) {
    uint32_t c = d.exact[q], cs = d.node_start[c], ce = d.node_end[c];
    double4 cC = d.ncA[c];
    float d0 = (float)(cL.x - cC.x), d1 = (float)(cL.y - cC.y), d2 = (float)(cL.z - cC.z);
    for (uint32_t ps = s0; ps < s1; ++ps)
      for (uint32_t pt = cs; pt < ce; ++pt) {
        if (ps == pt) continue;
        float4 xs = d.fxa[ps], xt = d.fxa[pt], n = d.fnn[ps];
        float v0 = (xs.x - xt.x) + d0, v1 = (xs.y - xt.y) + d1, v2 = (xs.z - xt.z) + d2;
        float r2 = v0 * v0 + v1 * v1 + v2 * v2, ir2 = 1.f / r2, K, cn;
        kernel_k<FAST>(pw, n.x * v0 + n.y * v1 + n.z * v2, r2, ir2, K, cn);
        float term = K * xs.w * xt.w;
        if (!isfinite(term) || !isfinite(cn) || !isfinite(ir2)) {
          unsigned long long rank =
              ((unsigned long long)q << 8) | ((ps - s0) << 4) | (unsigned long long)(pt - cs);
          atomicMin(best, rank);
          return;
        }
      }
  }
}

}  // namespace rsg

// ====================================================================== host driver

using namespace rsg;

struct rs_bh {
  rs_ctx *ctx = nullptr;
  int nv = 0, nf = 0, leaf_size = 8;
  // build phases in seconds: geometry, tree, topology, list counts, list fill, list finish
  // (transposes, chunks, schedule), refit
  double build_times[7] = {0, 0, 0, 0, 0, 0, 0};
  double theta = 0.5;
  Tree tree;
  std::vector<uint32_t> faces_h;
  uint64_t pairs_exact = 0, lumped_inter = 0;
  size_t n_lumped = 0, n_exact = 0, n_partner = 0;
  int64_t culprit[2] = {-1, -1};
  // device topology
  DevBuf<uint32_t> faces, order, node_start, node_end, node_right, node_parent, leaves,
      leaf_of_pos, schedule, chain_off, chain, inc_off, inc, leaf_ordinal, item_leaf, item_off;
  DevBuf<uint4> items;
  size_t n_items = 0;
  DevBuf<double> box, radius;
  DevBuf<uint32_t> lumped_off, lumped, exact_off, exact, partner_off, lumped_t_off, lumped_t,
      exact_t_off, exact_t;
  DevBuf<uint4> fchunk, nchunk;
  DevBuf<uint32_t> fchunk_off, nchunk_off;
  DevBuf<float> fpart;
  DevBuf<float4> npart;
  size_t n_fchunks = 0, n_nchunks = 0;
  // per evaluation
  DevBuf<double> pos;
  DevBuf<float4> fxa, fnn, fol, fnl, own, node_term, partner, node_sum, leaf_bu, partials;
  DevBuf<double4> ncA, nmom;
  DevBuf<float4> nch, ncl;
  DevBuf<uint32_t> refit_count;
  DevBuf<double> item_energy, energy, dE;
  DevBuf<unsigned int> ticket;
  DevBuf<unsigned long long> culprit_key;
  bool positions_current = false;
  Profiler prof;

  BhDev dev() const {
    BhDev d;
    d.faces = faces.p, d.order = order.p, d.node_start = node_start.p, d.node_end = node_end.p;
    d.node_right = node_right.p, d.node_parent = node_parent.p, d.leaves = leaves.p;
    d.leaf_of_pos = leaf_of_pos.p, d.schedule = schedule.p, d.chain_off = chain_off.p;
    d.items = items.p, d.item_leaf = item_leaf.p, d.item_off = item_off.p, d.n_items = (int)n_items;
    d.fol = fol.p, d.fnl = fnl.p;
    d.chain = chain.p, d.inc_off = inc_off.p, d.inc = inc.p;
    d.lumped_off = lumped_off.p, d.lumped = lumped.p, d.exact_off = exact_off.p, d.exact = exact.p;
    d.partner_off = partner_off.p, d.lumped_t_off = lumped_t_off.p, d.lumped_t = lumped_t.p;
    d.exact_t_off = exact_t_off.p, d.exact_t = exact_t.p;
    d.fchunk = fchunk.p, d.nchunk = nchunk.p, d.fchunk_off = fchunk_off.p, d.nchunk_off = nchunk_off.p;
    d.fpart = fpart.p, d.npart = npart.p;
    d.n_fchunks = (int)n_fchunks, d.n_nchunks = (int)n_nchunks;
    d.n_vertices = nv, d.n_faces = nf, d.n_nodes = (int)tree.n_nodes();
    d.n_leaves = (int)tree.leaves.size();
    d.fxa = fxa.p, d.fnn = fnn.p, d.ncA = ncA.p, d.nmom = nmom.p, d.refit_count = refit_count.p;
    d.nch = nch.p, d.ncl = ncl.p;
    d.own = own.p, d.node_term = node_term.p, d.partner = partner.p, d.node_sum = node_sum.p;
    d.leaf_bu = leaf_bu.p, d.partials = partials.p, d.item_energy = item_energy.p;
    d.ticket = ticket.p;
    return d;
  }
  cudaStream_t st() const { return ctx->stream; }
};

namespace {

inline unsigned blocks(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

template <class T>
void upload_vec(DevBuf<T> &b, const std::vector<T> &v, cudaStream_t s) {
  b.alloc(v.size());
  b.upload(v.data(), v.size(), s);
}

Pow make_pow(double alpha, double beta) {
  // Exponents::new (RS/src/kernel.rs:50-76)
  if (!std::isfinite(alpha) || !std::isfinite(beta))
    fail(RS_INVALID_EXPONENTS, "InvalidExponents", "energy", "both exponents must be finite");
  if (alpha <= 1.0) fail(RS_INVALID_EXPONENTS, "InvalidExponents", "energy", "alpha must be greater than 1");
  if (beta <= alpha + 2.0)
    fail(RS_INVALID_EXPONENTS, "InvalidExponents", "energy",
         "beta must be greater than alpha + 2 (s = (beta - 2)/alpha > 1)");
  if (beta >= 2.0 * alpha + 2.0)
    fail(RS_INVALID_EXPONENTS, "InvalidExponents", "energy",
         "beta must be smaller than 2 alpha + 2 (s = (beta - 2)/alpha < 2)");
  Pow p;
  p.alpha = (float)alpha;
  p.beta = (float)beta;
  p.a_int = (alpha == std::trunc(alpha) && alpha >= 2 && alpha <= 64) ? (int)alpha : -1;
  double ab = beta - alpha;
  p.ab_int = (ab == std::trunc(ab) && ab >= 0 && ab <= 128) ? (int)ab : -1;
  return p;
}

bool is_fast(double alpha, double beta) { return alpha == 6.0 && beta == 12.0; }

// Topology arrays common to rs_bh_build and rs_bh_attach: parents, leaf chains, leaf of
// every position, vertex incidence.
void upload_topology(rs_bh *h) {
  cudaStream_t s = h->st();
  const Tree &T = h->tree;
  size_t nn = T.n_nodes(), nl = T.leaves.size();
  std::vector<uint32_t> parent(nn, 0);
  for (size_t i = 0; i < nn; ++i)
    if (T.right[i]) parent[i + 1] = (uint32_t)i, parent[T.right[i]] = (uint32_t)i;
  std::vector<uint32_t> leaf_of_pos(h->nf), coff(nl + 1, 0), chain;
  size_t max_depth = 0;
  for (size_t k = 0; k < nl; ++k) {
    uint32_t l = T.leaves[k];
    for (uint32_t p = T.start[l]; p < T.end[l]; ++p) leaf_of_pos[p] = (uint32_t)k;
    size_t b = chain.size();
    uint32_t a = l;
    for (;;) {
      chain.push_back(a);
      if (a == 0) break;
      a = parent[a];
    }
    std::reverse(chain.begin() + b, chain.end());
    max_depth = std::max(max_depth, chain.size() - b);
    coff[k + 1] = (uint32_t)chain.size();
  }
  if (max_depth + 2 >= (size_t)kMaxDepth)
    fail(RS_INVALID_OPTION, "InvalidOption", "upload",
         "tree depth " + std::to_string(max_depth) + " exceeds the traversal stack");
  if (h->leaf_size > 8)
    fail(RS_INVALID_OPTION, "InvalidOption", "upload", "the GPU path needs leaf_size <= 8");
  for (size_t k = 0; k < nl; ++k) {
    uint32_t l = T.leaves[k];
    if (T.end[l] - T.start[l] > 8)
      fail(RS_INVALID_OPTION, "InvalidOption", "upload", "a leaf holds more than 8 faces");
  }
  // vertex -> (face, corner), faces ascending
  std::vector<uint32_t> ioff((size_t)h->nv + 1, 0), inc(3 * (size_t)h->nf);
  for (int f = 0; f < h->nf; ++f)
    for (int c = 0; c < 3; ++c) ioff[h->faces_h[3 * f + c] + 1]++;
  for (int v = 0; v < h->nv; ++v) ioff[v + 1] += ioff[v];
  {
    std::vector<uint32_t> fill(ioff.begin(), ioff.end() - 1);
    for (int f = 0; f < h->nf; ++f)
      for (int c = 0; c < 3; ++c) inc[fill[h->faces_h[3 * f + c]]++] = ((uint32_t)f << 2) | c;
  }
  upload_vec(h->faces, h->faces_h, s);
  upload_vec(h->order, T.order, s);
  upload_vec(h->node_start, T.start, s);
  upload_vec(h->node_end, T.end, s);
  upload_vec(h->node_right, T.right, s);
  upload_vec(h->node_parent, parent, s);
  upload_vec(h->leaves, T.leaves, s);
  upload_vec(h->leaf_of_pos, leaf_of_pos, s);
  upload_vec(h->chain_off, coff, s);
  upload_vec(h->chain, chain, s);
  upload_vec(h->inc_off, ioff, s);
  upload_vec(h->inc, inc, s);
  upload_vec(h->leaf_ordinal, T.leaf_ordinal, s);
  h->fxa.alloc(h->nf);
  h->fnn.alloc(h->nf);
  h->fol.alloc(h->nf);
  h->fnl.alloc(h->nf);
  h->partials.alloc(2 * (size_t)h->nf);
  h->ncA.alloc(nn);
  h->nmom.alloc(nn);
  h->nch.alloc(nn);
  h->ncl.alloc(nn);
  h->node_sum.alloc(nn);
  h->refit_count.alloc(nn);
  RSG_CUDA("upload", cudaMemsetAsync(h->refit_count.p, 0, nn * sizeof(uint32_t), s));
  h->leaf_bu.alloc(nl);
  h->energy.alloc(1);
  h->dE.alloc(3 * (size_t)h->nv);
  h->pos.alloc(3 * (size_t)h->nv);
  h->ticket.alloc(1);
  h->culprit_key.alloc(1);
}

// Transposes of the lists (barnes_hut.rs:798-806, 811-827) by a stable radix sort of
// (key, entry) pairs, and the processing schedule.
void finish_lists(rs_bh *h, const std::vector<uint32_t> &lo, const std::vector<uint32_t> &eo) {
  cudaStream_t s = h->st();
  size_t nn = h->tree.n_nodes(), nl = h->tree.leaves.size();
  auto transpose = [&](const uint32_t *keys_in, size_t n, size_t m, DevBuf<uint32_t> &off,
                       DevBuf<uint32_t> &idx, const char *what) {
    off.alloc(m + 1);
    idx.alloc(std::max<size_t>(n, 1));
    if (n == 0) {
      RSG_CUDA("upload", cudaMemsetAsync(off.p, 0, (m + 1) * sizeof(uint32_t), s));
      return;
    }
    DevBuf<uint32_t> vals(n), keys_out(n);
    iota_kernel<<<blocks(n, 256), 256, 0, s>>>(vals.p, (uint32_t)n);
    RSG_LAUNCHED(h->ctx, "iota");
    size_t tmp_bytes = 0;
    int bits = 1;
    while ((size_t(1) << bits) < m + 1) ++bits;
    RSG_CUDA("upload", cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys_in, keys_out.p, vals.p,
                                                  idx.p, (int)n, 0, bits, s));
    DevBuf<unsigned char> tmp(tmp_bytes);
    RSG_CUDA("upload", cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, keys_in, keys_out.p, vals.p,
                                                  idx.p, (int)n, 0, bits, s));
    offsets_from_sorted<<<blocks(n + 1, 256), 256, 0, s>>>(keys_out.p, (uint32_t)n, (uint32_t)m, off.p);
    RSG_LAUNCHED(h->ctx, what);
    RSG_CUDA("upload", cudaStreamSynchronize(s));
  };
  transpose(h->lumped.p, h->n_lumped, nn, h->lumped_t_off, h->lumped_t, "lumped_t");
  {
    DevBuf<uint32_t> key(std::max<size_t>(h->n_exact, 1));
    if (h->n_exact) {
      leaf_key_kernel<<<blocks(h->n_exact, 256), 256, 0, s>>>(h->exact.p, h->leaf_ordinal.p, key.p,
                                                             (uint32_t)h->n_exact);
      RSG_LAUNCHED(h->ctx, "leaf_key");
    }
    transpose(key.p, h->n_exact, nl, h->exact_t_off, h->exact_t, "exact_t");
  }
  // Chunks of the transposed lists: at most 256 exact entries (partner slots of a leaf) or 1024
  // lumped entries (node terms of a node) per warp; every leaf / node has at least one chunk.
  {
    std::vector<uint32_t> et(nl + 1), lt(nn + 1);
    h->exact_t_off.download(et.data(), nl + 1, s);
    h->lumped_t_off.download(lt.data(), nn + 1, s);
    RSG_CUDA("upload", cudaStreamSynchronize(s));
    auto chunks = [](const std::vector<uint32_t> &off, size_t m, uint32_t len, std::vector<uint4> &ch,
                     std::vector<uint32_t> &choff) {
      choff.assign(m + 1, 0);
      for (size_t k = 0; k < m; ++k) {
        uint32_t x = off[k];
        do {
          uint32_t y = std::min(off[k + 1], x + len);
          ch.push_back(make_uint4((uint32_t)k, x, y, 0));
          x = y;
        } while (x < off[k + 1]);
        choff[k + 1] = (uint32_t)ch.size();
      }
    };
    std::vector<uint4> fc, nc;
    std::vector<uint32_t> fco, nco;
    chunks(et, nl, 256, fc, fco);
    chunks(lt, nn, 1024, nc, nco);
    h->n_fchunks = fc.size(), h->n_nchunks = nc.size();
    upload_vec(h->fchunk, fc, s), upload_vec(h->fchunk_off, fco, s);
    upload_vec(h->nchunk, nc, s), upload_vec(h->nchunk_off, nco, s);
    h->fpart.alloc(32 * fc.size());
    h->npart.alloc(nc.size());
  }
  // Work items: every leaf's lumped and exact ranges split into slices of at most ~512
  // lumped / ~128 exact entries (a few leaves of a degenerate tree open every other leaf);
  // warps take them from an atomic ticket, most work first.
  std::vector<uint4> it;
  std::vector<uint32_t> it_leaf, it_off(nl + 1, 0);
  std::vector<uint64_t> cost;
  for (size_t k = 0; k < nl; ++k) {
    uint32_t l0 = lo[k], l1 = lo[k + 1], e0 = eo[k], e1 = eo[k + 1];
    uint32_t nl_ = l1 - l0, ne = e1 - e0;
    uint32_t n = std::max<uint32_t>(1, std::max((nl_ + 511) / 512, (ne + 127) / 128));
    uint32_t leaf = h->tree.leaves[k];
    uint64_t ns = h->tree.end[leaf] - h->tree.start[leaf];
    for (uint32_t i = 0; i < n; ++i) {
      uint32_t a0 = l0 + (uint32_t)((uint64_t)nl_ * i / n), a1 = l0 + (uint32_t)((uint64_t)nl_ * (i + 1) / n);
      uint32_t b0 = e0 + (uint32_t)((uint64_t)ne * i / n), b1 = e0 + (uint32_t)((uint64_t)ne * (i + 1) / n);
      it.push_back(make_uint4(a0, a1, b0, b1));
      it_leaf.push_back((uint32_t)k);
      cost.push_back(ns * ((uint64_t)(a1 - a0) + 8ull * (b1 - b0)));
    }
    it_off[k + 1] = (uint32_t)it.size();
  }
  h->n_items = it.size();
  std::vector<uint32_t> sched(it.size());
  std::iota(sched.begin(), sched.end(), 0u);
  std::stable_sort(sched.begin(), sched.end(), [&](uint32_t a, uint32_t b) { return cost[a] > cost[b]; });
  upload_vec(h->schedule, sched, s);
  upload_vec(h->items, it, s);
  upload_vec(h->item_leaf, it_leaf, s);
  upload_vec(h->item_off, it_off, s);
  h->own.alloc(16 * it.size());
  h->item_energy.alloc(it.size());
  h->node_term.alloc(std::max<size_t>(h->n_lumped, 1));
  h->partner.alloc(std::max<size_t>(h->n_partner, 1));
  RSG_CUDA("upload", cudaStreamSynchronize(s));
}

void build_lists_device(rs_bh *h) {
  using clk = std::chrono::steady_clock;
  auto t_ph = clk::now();
  auto lap = [&] {
    const auto now = clk::now();
    const double d = std::chrono::duration<double>(now - t_ph).count();
    t_ph = now;
    return d;
  };
  cudaStream_t s = h->st();
  const Tree &T = h->tree;
  size_t nl = T.leaves.size();
  upload_vec(h->box, T.box, s);
  upload_vec(h->radius, T.radius, s);
  ListsDev L{h->box.p, h->radius.p, h->theta * h->theta};
  DevBuf<uint32_t> c_lum(nl), c_ex(nl), c_par(nl);
  DevBuf<unsigned long long> pairs(nl), linter(nl);
  DevBuf<unsigned int> overflow(1);
  RSG_CUDA("upload", cudaMemsetAsync(overflow.p, 0, sizeof(unsigned), s));
  BhDev d = h->dev();
  const size_t nsl = nl * (size_t)kSegs;
  DevBuf<uint32_t> seg(nsl), nseg(nl), s_lum(nsl), s_ex(nsl), s_par(nsl), heavy(nsl), n_heavy(1);
  DevBuf<unsigned long long> s_pr(nsl);
  RSG_CUDA("upload", cudaMemsetAsync(n_heavy.p, 0, sizeof(uint32_t), s));
  lists_top_kernel<<<blocks(nl, 128), 128, 0, s>>>(d, L, seg.p, nseg.p, heavy.p, n_heavy.p, overflow.p);
  RSG_LAUNCHED(h->ctx, "lists_top");
  auto seg_pass = [&](auto fill, uint32_t *lum, uint32_t *ex, uint32_t *po, const uint32_t *pbase) {
    constexpr bool F = decltype(fill)::value;
    lists_seg_kernel<F, false><<<blocks(nsl, 128), 128, 0, s>>>(d, L, seg.p, nseg.p, heavy.p, n_heavy.p, s_lum.p,
                                                                s_ex.p, s_par.p, s_pr.p, lum, ex, po, pbase, overflow.p);
    RSG_LAUNCHED(h->ctx, F ? "lists_fill" : "lists_count");
    lists_seg_kernel<F, true><<<blocks(nsl, 128), 128, 0, s>>>(d, L, seg.p, nseg.p, heavy.p, n_heavy.p, s_lum.p,
                                                               s_ex.p, s_par.p, s_pr.p, lum, ex, po, pbase, overflow.p);
    RSG_LAUNCHED(h->ctx, F ? "lists_fill" : "lists_count");
  };
  seg_pass(std::false_type{}, nullptr, nullptr, nullptr, nullptr);
  lists_scan_kernel<<<blocks(nl * 32, 128), 128, 0, s>>>(d, nseg.p, s_lum.p, s_ex.p, s_par.p, s_pr.p, c_lum.p, c_ex.p,
                                                          c_par.p, pairs.p, linter.p);
  RSG_LAUNCHED(h->ctx, "lists_scan");
  std::vector<uint32_t> hl(nl), he(nl), hp(nl);
  std::vector<unsigned long long> hpr(nl), hli(nl);
  unsigned ovf = 0;
  c_lum.download(hl.data(), nl, s);
  c_ex.download(he.data(), nl, s);
  c_par.download(hp.data(), nl, s);
  pairs.download(hpr.data(), nl, s);
  linter.download(hli.data(), nl, s);
  overflow.download(&ovf, 1, s);
  RSG_CUDA("upload", cudaStreamSynchronize(s));
  h->build_times[3] = lap();
  if (ovf) fail(RS_INTERNAL, "Internal", "upload", "traversal stack overflow");
  std::vector<uint32_t> lo(nl + 1, 0), eo(nl + 1, 0), pb(nl, 0);
  uint64_t tl = 0, te = 0, tp = 0;
  h->pairs_exact = 0;
  h->lumped_inter = 0;
  for (size_t k = 0; k < nl; ++k) {
    pb[k] = (uint32_t)tp;
    tl += hl[k], te += he[k], tp += hp[k];
    if (tl > 0xffffffffull || tp > 0xffffffffull)
      fail(RS_INVALID_OPTION, "InvalidOption", "upload", "interaction lists exceed 2^32 entries");
    lo[k + 1] = (uint32_t)tl, eo[k + 1] = (uint32_t)te;
    h->pairs_exact += hpr[k];
    h->lumped_inter += hli[k];
  }
  h->n_lumped = tl, h->n_exact = te, h->n_partner = tp;
  upload_vec(h->lumped_off, lo, s);
  upload_vec(h->exact_off, eo, s);
  DevBuf<uint32_t> pbase;
  upload_vec(pbase, pb, s);
  h->lumped.alloc(std::max<size_t>(tl, 1));
  h->exact.alloc(std::max<size_t>(te, 1));
  h->partner_off.alloc(te + 1);
  d = h->dev();
  seg_pass(std::true_type{}, h->lumped.p, h->exact.p, h->partner_off.p, pbase.p);
  uint32_t tp32 = (uint32_t)tp;
  RSG_CUDA("upload", rsg::copy_async(h->partner_off.p + te, &tp32, sizeof(uint32_t),
                                     cudaMemcpyHostToDevice, s));
  RSG_CUDA("upload", cudaStreamSynchronize(s));
  h->build_times[4] = lap();
  finish_lists(h, lo, eo);
  h->build_times[5] = lap();
}

void refit_device(rs_bh *h) {
  BhDev d = h->dev();
  size_t nl = h->tree.leaves.size();
  refit_kernel<<<blocks(nl, 128), 128, 0, h->st()>>>(d, h->pos.p);
  RSG_LAUNCHED(h->ctx, "refit");
  h->positions_current = true;
}

void check_positions_host(rs_bh *h, const double *pos) {
  // BhTree::refit (barnes_hut.rs:204-229): counts and finiteness; degenerate faces make the
  // energy non-finite instead.
  for (int v = 0; v < h->nv; ++v)
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(pos[3 * v + k]))
        fail(RS_NONFINITE_POSITION, "NonFinitePosition", "energy", "vertex " + std::to_string(v));
}

// Resident 256-thread blocks per SM of the pair kernel (a persistent grid: one wave).
int pair_blocks_per_sm(bool grad, bool fast) {
  static int cache[4] = {0, 0, 0, 0};
  int &c = cache[(grad ? 2 : 0) + (fast ? 1 : 0)];
  if (c == 0) {
    const void *fn = grad ? (fast ? (const void *)bh_pair_kernel<true, true> : (const void *)bh_pair_kernel<true, false>)
                          : (fast ? (const void *)bh_pair_kernel<false, true> : (const void *)bh_pair_kernel<false, false>);
    int b = 0;
    RSG_CUDA("launch", cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, 128, 0));
    c = b > 0 ? b : 1;
  }
  return c;
}

// The pair kernel and the gradient passes on the context stream (no synchronisation).
void evaluate(rs_bh *h, const Pow &pw, bool fast, bool grad, double *energy_dev, double *dE_dev) {
  if (!h->positions_current) fail(RS_INVALID_OPTION, "InvalidOption", "energy", "no positions");
  cudaStream_t s = h->st();
  BhDev d = h->dev();
  size_t nl = h->tree.leaves.size(), nn = h->tree.n_nodes();
  Profiler &P = h->prof;
  RSG_CUDA("launch", cudaMemsetAsync(h->ticket.p, 0, sizeof(unsigned), s));
  unsigned grid = (unsigned)std::min<size_t>((size_t)h->ctx->sm_count * pair_blocks_per_sm(grad, fast),
                                             blocks(h->n_items, 4));
  P.begin(s, grad ? "bh_pair_grad" : "bh_pair_value");
  if (grad) {
    if (fast) bh_pair_kernel<true, true><<<grid, 128, 0, s>>>(d, pw);
    else bh_pair_kernel<true, false><<<grid, 128, 0, s>>>(d, pw);
  } else {
    if (fast) bh_pair_kernel<false, true><<<grid, 128, 0, s>>>(d, pw);
    else bh_pair_kernel<false, false><<<grid, 128, 0, s>>>(d, pw);
  }
  RSG_LAUNCHED(h->ctx, "bh_pair");
  P.end(s);
  if (grad) {
    P.begin(s, "node_sums");
    node_partial_kernel<<<blocks((size_t)h->n_nchunks * 32, 256), 256, 0, s>>>(d);
    RSG_LAUNCHED(h->ctx, "node_sums");
    node_sums_kernel<<<blocks(nn, 256), 256, 0, s>>>(d);
    RSG_LAUNCHED(h->ctx, "node_sums");
    P.end(s);
    P.begin(s, "downward");
    downward_kernel<<<blocks(nl, 128), 128, 0, s>>>(d);
    RSG_LAUNCHED(h->ctx, "downward");
    P.end(s);
    P.begin(s, "final");
    final_partial_kernel<<<blocks((size_t)h->n_fchunks * 32, 256), 256, 0, s>>>(d);
    RSG_LAUNCHED(h->ctx, "final");
    final_kernel<<<blocks(nl * 32, 256), 256, 0, s>>>(d);
    RSG_LAUNCHED(h->ctx, "final");
    P.end(s);
    if (dE_dev) {
      P.begin(s, "pull_back");
      pull_back_kernel<<<blocks(h->nv, 256), 256, 0, s>>>(d, h->pos.p, dE_dev);
      RSG_LAUNCHED(h->ctx, "pull_back");
      P.end(s);
    }
  }
  P.begin(s, "energy_reduce");
  energy_reduce_kernel<<<1, 1024, 0, s>>>(h->item_energy.p, (int)h->n_items, energy_dev);
  RSG_LAUNCHED(h->ctx, "energy_reduce");
  P.end(s);
}

void find_culprit(rs_bh *h, const Pow &pw, bool fast) {
  cudaStream_t s = h->st();
  unsigned long long init = ~0ull, rank = ~0ull;
  RSG_CUDA("product", rsg::copy_async(h->culprit_key.p, &init, sizeof(init), cudaMemcpyHostToDevice, s));
  size_t nl = h->tree.leaves.size();
  if (fast) culprit_kernel<true><<<blocks(nl, 128), 128, 0, s>>>(h->dev(), pw, h->culprit_key.p);
  else culprit_kernel<false><<<blocks(nl, 128), 128, 0, s>>>(h->dev(), pw, h->culprit_key.p);
  RSG_LAUNCHED(h->ctx, "culprit");
  h->culprit_key.download(&rank, 1, s);
  RSG_CUDA("product", cudaStreamSynchronize(s));
  h->culprit[0] = h->culprit[1] = -1;
  if (rank == ~0ull) return;
  uint32_t q = (uint32_t)(rank >> 8), ds = (rank >> 4) & 15, dt = rank & 15;
  std::vector<uint32_t> eo(nl + 1);
  uint32_t c = 0;
  h->exact_off.download(eo.data(), nl + 1, s);
  RSG_CUDA("product", rsg::copy_async(&c, h->exact.p + q, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  RSG_CUDA("product", cudaStreamSynchronize(s));
  size_t k = (size_t)(std::upper_bound(eo.begin(), eo.end(), q) - eo.begin()) - 1;
  const Tree &T = h->tree;
  uint32_t leaf = T.leaves[k];
  uint32_t fs = T.order[T.start[leaf] + ds], ft = T.order[T.start[c] + dt];
  h->culprit[0] = std::min(fs, ft);
  h->culprit[1] = std::max(fs, ft);
}

}  // namespace

extern "C" {

int rs_bh_build(rs_ctx *ctx, int nv, int nf, const uint32_t *faces, const double *positions_host,
                double theta, int leaf_size, rs_bh **out) {
  *out = nullptr;
  return guard([&] {
    if (!(std::isfinite(theta) && theta >= 0.0))
      fail(RS_INVALID_OPTION, "InvalidOption", "energy", "theta must be finite and non-negative");
    if (leaf_size < 1) fail(RS_INVALID_OPTION, "InvalidOption", "energy", "leaf_size must be at least 1");
    validate_topology(nv, nf, faces);
    validate_positions(nv, nf, faces, positions_host);
    ctx->use();
    auto h = std::make_unique<rs_bh>();
    h->ctx = ctx;
    h->nv = nv, h->nf = nf, h->theta = theta, h->leaf_size = leaf_size;
    h->faces_h.assign(faces, faces + 3 * (size_t)nf);
    using clk = std::chrono::steady_clock;
    auto t_ph = clk::now();
    auto lap = [&](int slot) {
      const auto now = clk::now();
      h->build_times[slot] = std::chrono::duration<double>(now - t_ph).count();
      t_ph = now;
    };
    const SharedFaceTree *sh = shared_face_tree(faces, positions_host, nf, leaf_size);
    if (!sh) {
      FaceGeom g = face_geometry(nf, faces, positions_host);
      lap(0);
      h->tree = build_face_tree(nf, faces, positions_host, g, leaf_size);
    } else {
      lap(0);
      h->tree = sh->tree;
    }
    lap(1);
    upload_topology(h.get());
    lap(2);
    build_lists_device(h.get());
    t_ph = clk::now();
    h->pos.upload(positions_host, 3 * (size_t)nv, h->st());
    refit_device(h.get());
    RSG_CUDA("upload", cudaStreamSynchronize(h->st()));
    lap(6);
    ctx_retain(ctx);
    *out = h.release();
  });
}

int rs_bh_attach(rs_ctx *ctx, int nv, int nf, const uint32_t *faces, const double *positions_host,
                 int n_nodes, const uint32_t *node_start, const uint32_t *node_end,
                 const uint32_t *node_right, const uint32_t *order, const int64_t *lumped_off,
                 const uint32_t *lumped, const int64_t *exact_off, const uint32_t *exact,
                 rs_bh **out) {
  *out = nullptr;
  return guard([&] {
    validate_topology(nv, nf, faces);
    validate_positions(nv, nf, faces, positions_host);
    if (n_nodes < 1) fail(RS_INVALID_OPTION, "InvalidOption", "upload", "empty tree");
    ctx->use();
    auto h = std::make_unique<rs_bh>();
    h->ctx = ctx;
    h->nv = nv, h->nf = nf;
    h->faces_h.assign(faces, faces + 3 * (size_t)nf);
    Tree &T = h->tree;
    T.start.assign(node_start, node_start + n_nodes);
    T.end.assign(node_end, node_end + n_nodes);
    T.right.assign(node_right, node_right + n_nodes);
    T.order.assign(order, order + nf);
    T.leaf_ordinal.assign(n_nodes, UINT32_MAX);
    int max_leaf = 0;
    for (int i = 0; i < n_nodes; ++i) {
      if (T.right[i] && (T.right[i] <= (uint32_t)i || T.right[i] >= (uint32_t)n_nodes))
        fail(RS_INVALID_OPTION, "InvalidOption", "upload", "bad right child");
      if (T.end[i] < T.start[i] || T.end[i] > (uint32_t)nf)
        fail(RS_INVALID_OPTION, "InvalidOption", "upload", "bad node range");
      if (T.right[i] == 0) {
        T.leaf_ordinal[i] = (uint32_t)T.leaves.size();
        T.leaves.push_back((uint32_t)i);
        max_leaf = std::max<int>(max_leaf, (int)(T.end[i] - T.start[i]));
      }
    }
    h->leaf_size = max_leaf;
    size_t nl = T.leaves.size();
    upload_topology(h.get());
    // lists from the caller
    cudaStream_t s = h->st();
    std::vector<uint32_t> lo(nl + 1), eo(nl + 1);
    for (size_t k = 0; k <= nl; ++k) lo[k] = (uint32_t)lumped_off[k], eo[k] = (uint32_t)exact_off[k];
    h->n_lumped = lo[nl], h->n_exact = eo[nl];
    std::vector<uint32_t> poff(h->n_exact + 1, 0);
    h->pairs_exact = 0, h->lumped_inter = 0;
    uint64_t p = 0;
    for (size_t k = 0; k < nl; ++k) {
      uint32_t l = T.leaves[k];
      uint64_t ns = T.end[l] - T.start[l];
      for (uint32_t q = eo[k]; q < eo[k + 1]; ++q) {
        uint32_t c = exact[q];
        if (c >= (uint32_t)n_nodes || T.right[c] != 0)
          fail(RS_INVALID_OPTION, "InvalidOption", "upload", "exact entry is not a leaf");
        uint64_t nc = T.end[c] - T.start[c];
        poff[q] = (uint32_t)p;
        p += nc;
        h->pairs_exact += (c == l) ? ns * (ns - 1) : ns * nc;
      }
      for (uint32_t q = lo[k]; q < lo[k + 1]; ++q)
        if (lumped[q] >= (uint32_t)n_nodes)
          fail(RS_INVALID_OPTION, "InvalidOption", "upload", "lumped entry out of range");
      h->lumped_inter += (uint64_t)(lo[k + 1] - lo[k]) * ns;
    }
    poff[h->n_exact] = (uint32_t)p;
    h->n_partner = p;
    upload_vec(h->lumped_off, lo, s);
    upload_vec(h->exact_off, eo, s);
    h->lumped.alloc(std::max<size_t>(h->n_lumped, 1));
    if (h->n_lumped) h->lumped.upload(lumped, h->n_lumped, s);
    h->exact.alloc(std::max<size_t>(h->n_exact, 1));
    if (h->n_exact) h->exact.upload(exact, h->n_exact, s);
    upload_vec(h->partner_off, poff, s);
    finish_lists(h.get(), lo, eo);
    h->pos.upload(positions_host, 3 * (size_t)nv, s);
    refit_device(h.get());
    RSG_CUDA("upload", cudaStreamSynchronize(s));
    ctx_retain(ctx);
    *out = h.release();
  });
}

void rs_bh_free(rs_bh *bh) {
  if (!bh) return;
  rs_ctx *ctx = bh->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  delete bh;
  ctx_release(ctx);
}

int rs_bh_refit(rs_bh *h, const double *positions_host) {
  return guard([&] {
    check_positions_host(h, positions_host);
    h->ctx->use();
    h->pos.upload(positions_host, 3 * (size_t)h->nv, h->st());
    refit_device(h);
  });
}

int rs_bh_refit_device(rs_bh *h, const double *positions_dev) {
  return guard([&] {
    h->ctx->use();
    RSG_CUDA("upload", cudaMemcpyAsync(h->pos.p, positions_dev, 3 * (size_t)h->nv * sizeof(double),
                                       cudaMemcpyDeviceToDevice, h->st()));
    refit_device(h);
  });
}

int rs_bh_energy(rs_bh *h, double alpha, double beta, double *energy) {
  return guard([&] {
    Pow pw = make_pow(alpha, beta);
    h->ctx->use();
    evaluate(h, pw, is_fast(alpha, beta), false, h->energy.p, nullptr);
    h->energy.download(energy, 1, h->st());
    RSG_CUDA("product", cudaStreamSynchronize(h->st()));
  });
}

static void eval_host(rs_bh *h, double alpha, double beta, double *energy, double *dE_host,
                      double *p7_host) {
  Pow pw = make_pow(alpha, beta);
  bool fast = is_fast(alpha, beta);
  h->ctx->use();
  evaluate(h, pw, fast, true, h->energy.p, h->dE.p);
  cudaStream_t s = h->st();
  double E = 0;
  h->energy.download(&E, 1, s);
  size_t nd = 3 * (size_t)h->nv;
  double *stage = (double *)h->ctx->staging(nd * sizeof(double) + 8 * sizeof(float) * (size_t)h->nf);
  h->dE.download(stage, nd, s);
  float *p7 = (float *)(stage + nd);
  if (p7_host) h->partials.download((float4 *)p7, 2 * (size_t)h->nf, s);
  RSG_CUDA("product", cudaStreamSynchronize(s));
  bool finite = std::isfinite(E);
  for (size_t i = 0; i < nd && finite; ++i) finite = std::isfinite(stage[i]);
  if (!finite) {
    find_culprit(h, pw, fast);
    fail(RS_NONFINITE_ENERGY, "NonFiniteEnergy", "energy",
         "faces (" + std::to_string(h->culprit[0]) + ", " + std::to_string(h->culprit[1]) +
             ") have the same barycenter or a non-finite term");
  }
  *energy = E;
  if (dE_host) std::memcpy(dE_host, stage, nd * sizeof(double));
  if (p7_host)
    for (int f = 0; f < h->nf; ++f)
      for (int c = 0; c < 7; ++c) p7_host[7 * (size_t)f + c] = (double)p7[8 * (size_t)f + c];
}

int rs_bh_energy_and_differential(rs_bh *h, double alpha, double beta, double *energy,
                                  double *differential_host) {
  return guard([&] { eval_host(h, alpha, beta, energy, differential_host, nullptr); });
}

int rs_bh_face_partials(rs_bh *h, double alpha, double beta, double *energy, double *p7) {
  return guard([&] { eval_host(h, alpha, beta, energy, nullptr, p7); });
}

int rs_bh_energy_and_differential_device(rs_bh *h, double alpha, double beta, double *energy_dev,
                                         double *differential_dev) {
  return guard([&] {
    Pow pw = make_pow(alpha, beta);
    h->ctx->use();
    evaluate(h, pw, is_fast(alpha, beta), true, energy_dev, differential_dev);
  });
}

int rs_bh_build_times(rs_bh *h, double *out7) {
  return guard([&] { std::copy(h->build_times, h->build_times + 7, out7); });
}

int rs_bh_sizes(rs_bh *h, int64_t *o) {
  return guard([&] {
    o[0] = (int64_t)h->tree.n_nodes();
    o[1] = (int64_t)h->tree.leaves.size();
    o[2] = (int64_t)h->n_lumped;
    o[3] = (int64_t)h->n_exact;
    o[4] = (int64_t)h->n_partner;
    o[5] = (int64_t)h->pairs_exact;
    o[6] = (int64_t)h->lumped_inter;
  });
}

int rs_bh_export(rs_bh *h, uint32_t *node_start, uint32_t *node_end, uint32_t *node_right,
                 uint32_t *order, int64_t *lumped_off, uint32_t *lumped, int64_t *exact_off,
                 uint32_t *exact) {
  return guard([&] {
    const Tree &T = h->tree;
    std::copy(T.start.begin(), T.start.end(), node_start);
    std::copy(T.end.begin(), T.end.end(), node_end);
    std::copy(T.right.begin(), T.right.end(), node_right);
    std::copy(T.order.begin(), T.order.end(), order);
    size_t nl = T.leaves.size();
    std::vector<uint32_t> lo(nl + 1), eo(nl + 1);
    cudaStream_t s = h->st();
    h->lumped_off.download(lo.data(), nl + 1, s);
    h->exact_off.download(eo.data(), nl + 1, s);
    if (h->n_lumped) h->lumped.download(lumped, h->n_lumped, s);
    if (h->n_exact) h->exact.download(exact, h->n_exact, s);
    RSG_CUDA("product", cudaStreamSynchronize(s));
    for (size_t k = 0; k <= nl; ++k) lumped_off[k] = lo[k], exact_off[k] = eo[k];
  });
}

int rs_bh_culprit(rs_bh *h, int64_t *faces2) {
  return guard([&] { faces2[0] = h->culprit[0], faces2[1] = h->culprit[1]; });
}

int rs_bh_profile(rs_bh *h, double alpha, double beta, int reps, char *names, int names_len,
                  double *ms, int max_kernels, int *n_kernels) {
  return guard([&] {
    Pow pw = make_pow(alpha, beta);
    bool fast = is_fast(alpha, beta);
    h->ctx->use();
    h->prof.start();
    for (int r = 0; r < reps; ++r) evaluate(h, pw, fast, true, h->energy.p, h->dE.p);
    h->prof.stop(h->st());
    h->prof.report(names, names_len, ms, max_kernels, n_kernels, reps);
  });
}

}  // extern "C"
