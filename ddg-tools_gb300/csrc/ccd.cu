// Continuous collision detection of a mesh moving against itself, on the GPU: first_contact of
// RS/src/ccd.rs:762-884 (no obstacles, no exempt band) with its windows (ccd.rs:887-1045), the
// conservative advancement (ccd.rs:529-592) and the distances of RC/src/ccd.rs:237-319.
//
// This file is compiled with -fmad=false: every FP64 operation rounds as the reference's host
// code does (Rust never contracts a multiply-add), so tau_max is bitwise the reference's.
//
// Per window [lo, hi]:
//   1. swept boxes: per vertex the hull of its positions at lo and hi; per face and per edge the
//      union of its vertices' boxes, inflated by h = gap/2 (1 + 1e-6);
//   2. a box tree per primitive kind, as the reference builds it: boxes sorted along a Morton
//      curve of their centres, blocks of 8 united, blocks merged pairwise up to one root;
//   3. one thread per query (a vertex against the face tree, an edge against the edge tree)
//      walks the tree and runs the narrow phase on every element whose own box overlaps the
//      query box (so the candidate pairs are exactly those of the reference, whatever the
//      tree's shape), keeping the earliest contact in one global atomic minimum.
// A pair's contact time does not depend on the horizon it is given (see advance()), so the
// global minimum used as horizon only skips pairs that cannot lower the result.
#include <cub/cub.cuh>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "common.hpp"

namespace rsg {
namespace {

struct DBox {
  double lo[3], hi[3];
};

__device__ __forceinline__ double3 at3(double3 p, double3 u, double t) {
  return make_double3(p.x + t * u.x, p.y + t * u.y, p.z + t * u.z);
}
__device__ __forceinline__ double3 sub3(double3 a, double3 b) { return make_double3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ double3 add3(double3 a, double3 b) { return make_double3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ double3 scale3(double3 a, double s) { return make_double3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double dot3(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double3 cross3(double3 a, double3 b) {
  return make_double3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double norm3(double3 a) { return sqrt(dot3(a, a)); }
// f64::clamp(0, 1): a NaN stays NaN
__device__ __forceinline__ double clamp01(double x) {
  if (x < 0.0) x = 0.0;
  if (x > 1.0) x = 1.0;
  return x;
}

__device__ double point_segment_distance(double3 p, double3 a, double3 b) {  // RC/src/ccd.rs:237-247
  const double3 ab = sub3(b, a), ap = sub3(p, a);
  const double e = dot3(ab, ab);
  const double t = e > 0.0 ? clamp01(dot3(ap, ab) / e) : 0.0;
  return norm3(sub3(ap, scale3(ab, t)));
}

__device__ double segment_segment_distance(double3 p1, double3 q1, double3 p2, double3 q2) {  // ccd.rs:266-291
  double best = fmin(fmin(fmin(point_segment_distance(p1, p2, q2), point_segment_distance(q1, p2, q2)),
                          point_segment_distance(p2, p1, q1)),
                     point_segment_distance(q2, p1, q1));
  const double3 d1 = sub3(q1, p1), d2 = sub3(q2, p2);
  const double a = dot3(d1, d1), e = dot3(d2, d2);
  const double3 n = cross3(d1, d2);
  const double nn = dot3(n, n);
  if (a > 0.0 && e > 0.0 && nn > 0.0) {
    const double3 r = sub3(p1, p2);
    const double b = dot3(d1, d2), c = dot3(d1, r), f = dot3(d2, r);
    double s = clamp01(dot3(cross3(sub3(p2, p1), d2), n) / nn);
    const double t = clamp01((b * s + f) / e);
    s = clamp01((b * t - c) / a);
    best = fmin(best, norm3(sub3(add3(p1, scale3(d1, s)), add3(p2, scale3(d2, t)))));
  }
  return best;
}

__device__ double point_triangle_distance(double3 p, double3 a, double3 b, double3 c) {  // ccd.rs:298-319
  const double edges =
      fmin(fmin(point_segment_distance(p, a, b), point_segment_distance(p, b, c)), point_segment_distance(p, c, a));
  const double3 ab = sub3(b, a), ac = sub3(c, a);
  const double3 n = cross3(ab, ac);
  const double nn = dot3(n, n);
  if (nn <= 0.0) return edges;
  const double3 ap = sub3(p, a);
  const double v = dot3(cross3(ap, ac), n) / nn;
  const double w = dot3(cross3(ab, ap), n) / nn;
  if (v >= 0.0 && w >= 0.0 && v + w <= 1.0) return fmin(edges, fabs(dot3(ap, n)) / sqrt(nn));
  return edges;
}

// ---- static queries (RS/src/ccd.rs:1153-1191) ----

__device__ __forceinline__ double orient(double3 a, double3 b, double3 c, double3 d) {
  return dot3(cross3(sub3(b, a), sub3(c, a)), sub3(d, a));
}

__device__ bool segment_meets_triangle(double3 p, double3 q, double3 a, double3 b, double3 c) {  // ccd.rs:1158-1186
  const double d1 = orient(a, b, c, p), d2 = orient(a, b, c, q);
  if ((d1 > 0.0 && d2 > 0.0) || (d1 < 0.0 && d2 < 0.0)) return false;
  const double n = norm3(cross3(sub3(b, a), sub3(c, a)));
  const double len = fmax(fmax(fmax(norm3(sub3(q, p)), norm3(sub3(b, a))), norm3(sub3(c, a))), norm3(sub3(c, b)));
  const double flat = 1e-12 * n * len;
  if (fabs(d1) <= flat && fabs(d2) <= flat) {
    const double eps = 1e-14 * (norm3(sub3(b, a)) + norm3(sub3(c, a)));
    return point_triangle_distance(p, a, b, c) <= eps || point_triangle_distance(q, a, b, c) <= eps ||
           segment_segment_distance(p, q, a, b) <= eps || segment_segment_distance(p, q, b, c) <= eps ||
           segment_segment_distance(p, q, c, a) <= eps;
  }
  const double s1 = orient(p, q, a, b), s2 = orient(p, q, b, c), s3 = orient(p, q, c, a);
  return (s1 >= 0.0 && s2 >= 0.0 && s3 >= 0.0) || (s1 <= 0.0 && s2 <= 0.0 && s3 <= 0.0);
}

struct Tally {
  unsigned long long pairs = 0, close = 0, touching = 0, evals = 0;
};

// Conservative advancement of one pair on [lo, hz] (advance, RS/src/ccd.rs:529-592); returns
// the contact time or -1 for none. When a step would pass hz with the cheap bound, the
// reference retries with the refined bound l' and takes min(l, l'); that step is at least as
// long, so it passes hz too and the pair has no contact before hz. The retry is therefore
// left out: the result is the same. Every iterate that stays below hz is the reference's, so
// a contact time below the horizon does not depend on the horizon.
template <class Dist>
__device__ double advance(const Dist &dist, double l, double gap_abs, int max_iterations, double close_factor,
                          double lo, double hz, Tally &tally) {
  const double d0 = dist(0.0);
  tally.pairs += 1;
  tally.evals += 1;
  if (lo == 0.0) {
    if (d0 <= 1e-12 * gap_abs) {
      tally.touching += 1;
      return -1.0;
    }
    if (d0 < gap_abs) tally.close += 1;
  } else if (d0 <= 1e-12 * gap_abs) {
    return -1.0;
  }
  const double target = d0 > gap_abs ? gap_abs : close_factor * d0;
  const double slack = 1e-9 * d0;
  double tau = lo;
  double d = d0;
  if (lo != 0.0) {
    d = dist(lo);
    tally.evals += 1;
  }
  for (int it = 0; it < max_iterations; ++it) {
    if (isnan(d) || d - target <= slack) return tau;
    const double next = tau + (d - target) / l;
    if (next >= hz || isnan(next)) return -1.0;
    tau = next;
    d = dist(tau);
    tally.evals += 1;
  }
  return tau;
}

__device__ __forceinline__ bool overlaps(const DBox &a, const DBox &b) {  // ccd.rs:258-261
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (!(a.lo[k] <= b.hi[k] && b.lo[k] <= a.hi[k])) return false;
  return true;
}

__device__ __forceinline__ DBox inflate(DBox b, double h) {
#pragma unroll
  for (int k = 0; k < 3; ++k) b.lo[k] = b.lo[k] - h, b.hi[k] = b.hi[k] + h;
  return b;
}

__device__ __forceinline__ DBox unite(DBox a, const DBox &b) {
#pragma unroll
  for (int k = 0; k < 3; ++k) a.lo[k] = fmin(a.lo[k], b.lo[k]), a.hi[k] = fmax(a.hi[k], b.hi[k]);
  return a;
}

__global__ void speed_kernel(int nv, const double3 *vel, double *speed) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < nv) speed[v] = norm3(vel[v]);
}

// hull of the positions at lo and hi (Aabb::empty grown by both points)
__global__ void vbox_kernel(int nv, const double3 *start, const double3 *vel, double lo, double hi, DBox *vbox) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const double3 a = at3(start[v], vel[v], lo), b = at3(start[v], vel[v], hi);
  DBox r;
  r.lo[0] = fmin(fmin(INFINITY, a.x), b.x), r.hi[0] = fmax(fmax(-INFINITY, a.x), b.x);
  r.lo[1] = fmin(fmin(INFINITY, a.y), b.y), r.hi[1] = fmax(fmax(-INFINITY, a.y), b.y);
  r.lo[2] = fmin(fmin(INFINITY, a.z), b.z), r.hi[2] = fmax(fmax(-INFINITY, a.z), b.z);
  vbox[v] = r;
}

// Inflated primitive boxes and 30-bit Morton keys of their centres (the order only shapes the
// tree; it does not change the candidate pairs).
template <int K>
__global__ void prim_box_kernel(int n, const uint32_t *verts, const DBox *vbox, double h, double3 blo,
                                double3 bscale, DBox *box, uint32_t *key, uint32_t *idx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  DBox b = vbox[verts[K * i]];
#pragma unroll
  for (int k = 1; k < K; ++k) b = unite(b, vbox[verts[K * i + k]]);
  b = inflate(b, h);
  box[i] = b;
  auto q = [](double c, double l, double s) {
    double x = (c - l) * s;
    x = x < 0.0 ? 0.0 : (x > 1023.0 ? 1023.0 : x);
    uint32_t u = (uint32_t)x;
    u = (u | (u << 16)) & 0x030000FFu;
    u = (u | (u << 8)) & 0x0300F00Fu;
    u = (u | (u << 4)) & 0x030C30C3u;
    u = (u | (u << 2)) & 0x09249249u;
    return u;
  };
  key[i] = q(0.5 * (b.lo[0] + b.hi[0]), blo.x, bscale.x) | (q(0.5 * (b.lo[1] + b.hi[1]), blo.y, bscale.y) << 1) |
           (q(0.5 * (b.lo[2] + b.hi[2]), blo.z, bscale.z) << 2);
  idx[i] = (uint32_t)i;
}

__global__ void gather_boxes_kernel(int n, const uint32_t *order, const DBox *box, DBox *sbox) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) sbox[i] = box[order[i]];
}

// Node boxes of the walk in FP32, rounded outward: a node box contains the FP64 union of its
// elements' boxes, so the walk visits every leaf block the FP64 tree would (it may visit more;
// the element test below is exact).
struct FBox {
  float lo[3], hi[3];
};

__device__ __forceinline__ FBox outward(const DBox &b) {
  FBox r;
#pragma unroll
  for (int k = 0; k < 3; ++k) r.lo[k] = __double2float_rd(b.lo[k]), r.hi[k] = __double2float_ru(b.hi[k]);
  return r;
}

__device__ __forceinline__ bool overlaps_f(const FBox &a, const FBox &b) {
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (!(a.lo[k] <= b.hi[k] && b.lo[k] <= a.hi[k])) return false;
  return true;
}

// level 0: unions of blocks of 8 sorted element boxes (FP64, then rounded outward)
__global__ void level0_kernel(int n_out, const DBox *in, int n_in, FBox *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_out) return;
  DBox r;
  for (int k = 0; k < 3; ++k) r.lo[k] = INFINITY, r.hi[k] = -INFINITY;
  const int b = i * 8, e = min(b + 8, n_in);
  for (int j = b; j < e; ++j) r = unite(r, in[j]);
  out[i] = outward(r);
}

// level k: unions of pairs of level k - 1 (min / max of floats are exact)
__global__ void level_kernel(int n_out, const FBox *in, int n_in, FBox *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_out) return;
  FBox r = in[2 * i];
  if (2 * i + 1 < n_in) {
    const FBox &o = in[2 * i + 1];
#pragma unroll
    for (int k = 0; k < 3; ++k) r.lo[k] = fminf(r.lo[k], o.lo[k]), r.hi[k] = fmaxf(r.hi[k], o.hi[k]);
  }
  out[i] = r;
}

struct Tree {
  const DBox *sbox;      // sorted element boxes (FP64, the exact test)
  const uint32_t *order; // sorted position -> element
  const FBox *levels;    // all levels, level 0 first
  const int *lvl_off;    // offset of each level in `levels`
  const int *lvl_len;
  int n, n_levels, leaf;
};

constexpr int kStack = 64;

// Calls f(element) for every element whose FP64 box overlaps q (query, ccd.rs:359-389).
// Returns false if the stack would overflow (not reachable: a depth-first walk of a tree of
// n_levels <= 62 levels holds at most n_levels + 1 entries).
template <class F>
__device__ bool query(const Tree &t, const DBox &q, F &&f) {
  const FBox qf = outward(q);
  int2 stack[kStack];
  int sp = 0;
  stack[sp++] = make_int2(t.n_levels - 1, 0);
  while (sp > 0) {
    const int2 e = stack[--sp];
    if (!overlaps_f(t.levels[t.lvl_off[e.x] + e.y], qf)) continue;
    if (e.x == 0) {
      const int b = e.y * t.leaf, end = min(b + t.leaf, t.n);
      for (int pos = b; pos < end; ++pos)
        if (overlaps(t.sbox[pos], q)) f(t.order[pos]);
    } else {
      if (sp + 2 > kStack) return false;
      stack[sp++] = make_int2(e.x - 1, 2 * e.y);
      if (2 * e.y + 1 < t.lvl_len[e.x - 1]) stack[sp++] = make_int2(e.x - 1, 2 * e.y + 1);
    }
  }
  return true;
}

struct Params {
  const double3 *start, *vel;
  const double *speed;
  const uint32_t *faces;  // 3 per face
  const uint32_t *edges;  // 2 per edge
  const DBox *vbox;
  const DBox *ebox;       // inflated, element order
  const DBox *fbox;       // face boxes, element order (the band's face-face walk)
  const uint8_t *band;    // exempt band per vertex, or null
  int nv, ne, nf, max_iterations;
  double gap_abs, close_factor, h, lo, hi;
  unsigned long long *best;   // bits of the earliest contact time (+inf: none)
  unsigned long long *tally;  // pairs, close, touching, evaluations, exempt
  int *overflow;
};

constexpr double kMargin = 1.0 + 1e-12;  // ccd.rs:498-499

__device__ __forceinline__ double horizon(const Params &P) {
  const double b = __longlong_as_double((long long)*(volatile unsigned long long *)P.best);
  return fmin(b, P.hi);
}

__device__ void flush_tally(const Params &P, const Tally &t) {
  unsigned long long v[4] = {t.pairs, t.close, t.touching, t.evals};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    unsigned long long x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(P.tally + k, x);
  }
}

// Broad phase, one thread per query: KIND 0 a vertex against the face tree (the vertex not in
// the face, ccd.rs:937-985), KIND 1 an edge against the edge tree (partners e2 > e without a
// common vertex, ccd.rs:987-1038). FILL 0 counts each query's candidates; FILL 1 writes them
// as (query, element) from the query's offset, in the walk's order.
// KIND 2 (the band): a face against the face tree of the static hulls, partners g > f
// (intersecting_pairs, ccd.rs:1229-1279); the intersection test runs per pair afterwards.
// A pair whose two elements both have a vertex in the band is exempt (ccd.rs:947-950,
// 1001-1004): it is not a candidate, and it is counted in `counters[1]`.
// Candidates are appended as (query, element) to `pairs`: each thread buffers up to 16 and
// reserves room for them with one atomic add on `counters[0]`; pairs beyond `cap` are not
// written (the caller grows the list and walks again). The order of the list depends on the
// atomics; nothing computed from it does (a minimum, and sums of counts).
constexpr int kAppend = 16;

template <int KIND>
__global__ void __launch_bounds__(128) walk_kernel(Params P, Tree t, unsigned long long *counters, uint2 *pairs,
                                                   unsigned long long cap) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int nq = KIND == 0 ? P.nv : (KIND == 1 ? P.ne : P.nf);
  if (q >= nq) return;
  const DBox qb = KIND == 0 ? inflate(P.vbox[q], P.h) : (KIND == 1 ? P.ebox[q] : P.fbox[q]);
  uint32_t a = 0, b = 0;
  if (KIND == 1) a = P.edges[2 * q], b = P.edges[2 * q + 1];
  const bool qband = P.band && (KIND == 0 ? P.band[q] : (KIND == 1 ? (P.band[a] || P.band[b]) : false));
  uint32_t buf[kAppend];
  int nb = 0;
  uint32_t exempt = 0;
  auto flush = [&]() {
    const unsigned long long base = atomicAdd(counters, (unsigned long long)nb);
    for (int i = 0; i < nb; ++i)
      if (base + i < cap) pairs[base + i] = make_uint2((uint32_t)q, buf[i]);
    nb = 0;
  };
  const bool ok = query(t, qb, [&](uint32_t el) {
    if (KIND == 0) {
      const uint32_t fa = P.faces[3 * el], fb = P.faces[3 * el + 1], fc = P.faces[3 * el + 2];
      if (fa == (uint32_t)q || fb == (uint32_t)q || fc == (uint32_t)q) return;
      if (qband && (P.band[fa] || P.band[fb] || P.band[fc])) {
        ++exempt;
        return;
      }
    } else if (KIND == 1) {
      if (el <= (uint32_t)q) return;
      const uint32_t c = P.edges[2 * el], d = P.edges[2 * el + 1];
      if (c == a || c == b || d == a || d == b) return;
      if (qband && (P.band[c] || P.band[d])) {
        ++exempt;
        return;
      }
    } else {
      if (el <= (uint32_t)q) return;
    }
    buf[nb++] = el;
    if (nb == kAppend) flush();
  });
  if (nb) flush();
  if (!ok) atomicExch(P.overflow, 1);
  if (exempt) atomicAdd(counters + 1, (unsigned long long)exempt);
}

// The intersection test of one candidate face pair (f, g), f < g (ccd.rs:1247-1270): faces
// without a common vertex that meet, or faces with one common vertex whose opposite edge meets
// the other face; faces that share an edge are not tested.
__global__ void isect_kernel(Params P, const uint2 *pairs, unsigned long long n, uint8_t *hit) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t f = pairs[i].x, g = pairs[i].y;
  uint32_t A[3] = {P.faces[3 * f], P.faces[3 * f + 1], P.faces[3 * f + 2]};
  uint32_t B[3] = {P.faces[3 * g], P.faces[3 * g + 1], P.faces[3 * g + 2]};
  int common[3], nc = 0;
  for (int k = 0; k < 3; ++k)
    if (B[0] == A[k] || B[1] == A[k] || B[2] == A[k]) common[nc++] = k;
  const double3 a0 = P.start[A[0]], a1 = P.start[A[1]], a2 = P.start[A[2]];
  const double3 b0 = P.start[B[0]], b1 = P.start[B[1]], b2 = P.start[B[2]];
  bool h = false;
  if (nc == 0) {
    // triangles_intersect (ccd.rs:1188-1191): each edge of one against the other, in order
    const double3 ta[3] = {a0, a1, a2}, tb[3] = {b0, b1, b2};
    for (int k = 0; k < 3 && !h; ++k) h = segment_meets_triangle(ta[k], ta[(k + 1) % 3], b0, b1, b2);
    for (int k = 0; k < 3 && !h; ++k) h = segment_meets_triangle(tb[k], tb[(k + 1) % 3], a0, a1, a2);
  } else if (nc == 1) {
    const int k = common[0];
    int j = 0;
    while (B[j] != A[k]) ++j;
    h = segment_meets_triangle(P.start[A[(k + 1) % 3]], P.start[A[(k + 2) % 3]], b0, b1, b2) ||
        segment_meets_triangle(P.start[B[(j + 1) % 3]], P.start[B[(j + 2) % 3]], a0, a1, a2);
  }
  hit[i] = h ? 1 : 0;
}

// IntersectionBand::new (ccd.rs:1292-1319): the vertices of the intersecting faces (core) ...
__global__ void core_kernel(Params P, const uint2 *pairs, const uint8_t *hit, unsigned long long n, uint8_t *core,
                            unsigned long long *n_hits) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !hit[i]) return;
  const uint32_t f = pairs[i].x, g = pairs[i].y;
  for (int k = 0; k < 3; ++k) core[P.faces[3 * f + k]] = 1, core[P.faces[3 * g + k]] = 1;
  atomicAdd(n_hits, 1ull);
}

// ... widened by one ring: both ends of every edge with an end in the core
__global__ void ring_kernel(Params P, const uint8_t *core, uint8_t *band) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.ne) return;
  const uint32_t a = P.edges[2 * e], b = P.edges[2 * e + 1];
  if (core[a] || core[b]) band[a] = 1, band[b] = 1;
}

__global__ void count_flags_kernel(int n, const uint8_t *flag, unsigned long long *count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool f = i < n && flag[i];
  const unsigned m = __ballot_sync(0xffffffffu, f);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
}

// Narrow phase, one thread per candidate pair: the lanes of a warp evaluate their distances
// together. KIND 0: (vertex, face); KIND 1: (edge, edge).
template <int KIND>
__global__ void __launch_bounds__(128) narrow_kernel(Params P, const uint2 *pairs, unsigned long long n) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  Tally tally;
  if (i < n) {
    const uint2 pr = pairs[i];
    double r;
    if (KIND == 0) {
      const uint32_t v = pr.x, f = pr.y;
      const uint32_t a = P.faces[3 * f], b = P.faces[3 * f + 1], c = P.faces[3 * f + 2];
      const double3 p = P.start[v], u = P.vel[v];
      const double3 ta = at3(P.start[a], P.vel[a], 0.0), tb = at3(P.start[b], P.vel[b], 0.0),
                    tc = at3(P.start[c], P.vel[c], 0.0);
      const double3 ua = P.vel[a], ub = P.vel[b], uc = P.vel[c];
      const double lc = (P.speed[v] + fmax(fmax(P.speed[a], P.speed[b]), P.speed[c])) * kMargin;
      auto dist = [&](double t) {
        return point_triangle_distance(at3(p, u, t), at3(ta, ua, t), at3(tb, ub, t), at3(tc, uc, t));
      };
      r = advance(dist, lc, P.gap_abs, P.max_iterations, P.close_factor, P.lo, horizon(P), tally);
    } else {
      const uint32_t a = P.edges[2 * pr.x], b = P.edges[2 * pr.x + 1];
      const uint32_t c = P.edges[2 * pr.y], d = P.edges[2 * pr.y + 1];
      const double3 pa = P.start[a], pb = P.start[b], ua = P.vel[a], ub = P.vel[b];
      const double3 pc = P.start[c], pd = P.start[d], uc = P.vel[c], ud = P.vel[d];
      const double lc = (fmax(P.speed[a], P.speed[b]) + fmax(P.speed[c], P.speed[d])) * kMargin;
      auto dist = [&](double t) {
        return segment_segment_distance(at3(pa, ua, t), at3(pb, ub, t), at3(pc, uc, t), at3(pd, ud, t));
      };
      r = advance(dist, lc, P.gap_abs, P.max_iterations, P.close_factor, P.lo, horizon(P), tally);
    }
    if (r >= 0.0) atomicMin(P.best, (unsigned long long)__double_as_longlong(r));
  }
  flush_tally(P, tally);
}

// best = +inf (no contact), the five counters = 0
__global__ void reset_kernel(unsigned long long *best, unsigned long long *tally) {
  if (threadIdx.x == 0) *best = 0x7FF0000000000000ull;
  if (threadIdx.x < 5) tally[threadIdx.x] = 0;
}

inline unsigned blocks(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// A box tree's device storage, rebuilt per window.
struct TreeBufs {
  int n = 0;
  DevBuf<DBox> box, sbox;
  DevBuf<FBox> levels;
  DevBuf<uint32_t> key, key_sorted, idx, order;
  DevBuf<int> lvl_off, lvl_len;
  std::vector<int> off, len;
  void init(int n_, cudaStream_t s) {
    n = n_;
    box.alloc(n), sbox.alloc(n), key.alloc(n), key_sorted.alloc(n), idx.alloc(n), order.alloc(n);
    off.clear(), len.clear();
    int total = 0, m = (n + 7) / 8;
    for (;;) {
      off.push_back(total), len.push_back(m);
      total += m;
      if (m <= 1) break;
      m = (m + 1) / 2;
    }
    if (off.size() > 62) fail(RS_INTERNAL, "Internal", "ccd", "box tree deeper than 62 levels");
    levels.alloc(total);
    lvl_off.upload(off, s), lvl_len.upload(len, s);
  }
  Tree view() const {
    return Tree{sbox.p, order.p, levels.p, lvl_off.p, lvl_len.p, n, (int)off.size(), 8};
  }
};

}  // namespace
}  // namespace rsg

using namespace rsg;

struct rs_ccd {
  rs_ctx *ctx = nullptr;
  int nv = 0, nf = 0, ne = 0;
  std::vector<uint32_t> edges_h;  // sorted (min, max) pairs: the Surface's edge order
  DevBuf<uint32_t> faces, edges;
  DevBuf<double3> start, vel;
  DevBuf<double> speed;
  DevBuf<DBox> vbox;
  TreeBufs ft, et;
  DevBuf<unsigned long long> counters;  // appended candidates, exempt pairs (one walk)
  DevBuf<uint2> pairs;                // candidate pairs of a window (or of the band's walk)
  DevBuf<uint8_t> hit, core, band;    // the band: intersection flags per candidate, per vertex
  bool has_band = false;
  DevBuf<unsigned char> cub_tmp;
  DevBuf<unsigned long long> scratch;  // best, 5 tally counters, overflow flag, band hits
  double last_seconds = 0.0;
};

namespace {

// The element boxes of one kind, sorted along the Morton curve, and the tree levels over them.
void build_tree(rs_ccd *c, TreeBufs &T, int kind, double h, double3 gl, double3 gs, cudaStream_t s) {
  rs_ctx *ctx = c->ctx;
  const int n = T.n;
  if (kind == 0)
    prim_box_kernel<3><<<blocks(n, 256), 256, 0, s>>>(n, c->faces.p, c->vbox.p, h, gl, gs, T.box.p, T.key.p, T.idx.p);
  else
    prim_box_kernel<2><<<blocks(n, 256), 256, 0, s>>>(n, c->edges.p, c->vbox.p, h, gl, gs, T.box.p, T.key.p, T.idx.p);
  RSG_LAUNCHED(ctx, "ccd primitive boxes");
  size_t tb = c->cub_tmp.n;
  RSG_CUDA("ccd", cub::DeviceRadixSort::SortPairs(c->cub_tmp.p, tb, T.key.p, T.key_sorted.p, T.idx.p, T.order.p, n,
                                                  0, 30, s));
  ctx->launches++;
  gather_boxes_kernel<<<blocks(n, 256), 256, 0, s>>>(n, T.order.p, T.box.p, T.sbox.p);
  RSG_LAUNCHED(ctx, "ccd gather");
  level0_kernel<<<blocks(T.len[0], 128), 128, 0, s>>>(T.len[0], T.sbox.p, n, T.levels.p);
  RSG_LAUNCHED(ctx, "ccd tree level");
  for (size_t k = 1; k < T.off.size(); ++k) {
    level_kernel<<<blocks(T.len[k], 128), 128, 0, s>>>(T.len[k], T.levels.p + T.off[k - 1], T.len[k - 1],
                                                       T.levels.p + T.off[k]);
    RSG_LAUNCHED(ctx, "ccd tree level");
  }
}

// The Morton grid over the start positions widened by `ext` (any grid gives the same pairs).
void morton_grid(const double *start, int nv, double ext, double3 &gl, double3 &gs) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int v = 0; v < nv; ++v)
    for (int k = 0; k < 3; ++k) lo[k] = std::fmin(lo[k], start[3 * (size_t)v + k]), hi[k] = std::fmax(hi[k], start[3 * (size_t)v + k]);
  double l3[3], s3[3];
  for (int k = 0; k < 3; ++k) {
    l3[k] = lo[k] - ext;
    const double w = (hi[k] + ext) - l3[k];
    s3[k] = w > 0.0 ? 1023.0 / w : 0.0;
  }
  gl = make_double3(l3[0], l3[1], l3[2]);
  gs = make_double3(s3[0], s3[1], s3[2]);
}

// Candidate pairs of one kind, appended at c->pairs + base by one walk (walked again into a
// larger list when they did not fit). Returns their number; adds the exempt pairs to *exempt.
template <int KIND>
unsigned long long collect(rs_ccd *c, const Params &P, const Tree &t, int nq, unsigned long long base,
                           bool grow_keep, cudaStream_t s, int64_t *exempt = nullptr) {
  rs_ctx *ctx = c->ctx;
  for (int attempt = 0; attempt < 2; ++attempt) {
    const unsigned long long cap = c->pairs.n > base ? c->pairs.n - base : 0;
    RSG_CUDA("ccd", cudaMemsetAsync(c->counters.p, 0, c->counters.bytes(), s));
    walk_kernel<KIND><<<blocks(nq, 128), 128, 0, s>>>(P, t, c->counters.p, cap ? c->pairs.p + base : nullptr, cap);
    RSG_LAUNCHED(ctx, "ccd walk");
    unsigned long long got[2] = {0, 0};
    RSG_CUDA("ccd", rsg::copy_async(got, c->counters.p, sizeof(got), cudaMemcpyDeviceToHost, s));
    RSG_CUDA("ccd", cudaStreamSynchronize(s));
    if (got[0] <= cap) {
      if (exempt) *exempt += (int64_t)got[1];
      return got[0];
    }
    DevBuf<uint2> bigger((size_t)((base + got[0]) * 5 / 4 + 1024));
    if (grow_keep && base)
      RSG_CUDA("ccd", cudaMemcpyAsync(bigger.p, c->pairs.p, base * sizeof(uint2), cudaMemcpyDeviceToDevice, s));
    c->pairs = std::move(bigger);
  }
  fail(RS_INTERNAL, "Internal", "ccd", "candidate list did not fit after growing");
}

Params make_params(rs_ccd *c, double gap_abs, double close_factor, int max_iterations, double h, double lo,
                   double hi, const uint8_t *band) {
  Params P;
  P.start = c->start.p, P.vel = c->vel.p, P.speed = c->speed.p, P.faces = c->faces.p, P.edges = c->edges.p;
  P.vbox = c->vbox.p, P.ebox = c->et.box.p, P.fbox = c->ft.box.p, P.band = band;
  P.nv = c->nv, P.ne = c->ne, P.nf = c->nf, P.max_iterations = max_iterations;
  P.gap_abs = gap_abs, P.close_factor = close_factor, P.h = h, P.lo = lo, P.hi = hi;
  P.best = c->scratch.p, P.tally = c->scratch.p + 1;
  P.overflow = reinterpret_cast<int *>(c->scratch.p + 6);
  return P;
}

void check_overflow(rs_ccd *c, cudaStream_t s) {
  int ov = 0;
  RSG_CUDA("ccd", rsg::copy_async(&ov, c->scratch.p + 6, sizeof(int), cudaMemcpyDeviceToHost, s));
  RSG_CUDA("ccd", cudaStreamSynchronize(s));
  if (ov) fail(RS_INTERNAL, "Internal", "ccd", "box tree stack overflow");
}

void check_positions(const double *x, size_t n, const char *what) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(x[i])) fail(RS_INVALID_OPTION, "InvalidOption", "ccd", std::string(what) + " must be finite");
}

// The candidate face pairs of the static hulls of `positions` (uploaded into c->start) and
// their intersection flags (c->hit); returns the number of candidates.
unsigned long long face_pairs(rs_ccd *c, const double *positions, cudaStream_t s) {
  rs_ctx *ctx = c->ctx;
  c->start.upload(reinterpret_cast<const double3 *>(positions), c->nv, s);
  RSG_CUDA("ccd", cudaMemsetAsync(c->vel.p, 0, c->vel.bytes(), s));
  RSG_CUDA("ccd", cudaMemsetAsync(c->scratch.p, 0, c->scratch.bytes(), s));
  vbox_kernel<<<blocks(c->nv, 256), 256, 0, s>>>(c->nv, c->start.p, c->vel.p, 0.0, 0.0, c->vbox.p);
  RSG_LAUNCHED(ctx, "ccd boxes");
  double3 gl, gs;
  morton_grid(positions, c->nv, 0.0, gl, gs);
  build_tree(c, c->ft, 0, 0.0, gl, gs, s);
  const Params P = make_params(c, 0.0, 0.0, 1, 0.0, 0.0, 0.0, nullptr);
  const unsigned long long n = collect<2>(c, P, c->ft.view(), c->nf, 0, false, s);
  if (n > c->hit.n) c->hit.alloc((size_t)(n * 5 / 4 + 1024));
  if (n) {
    isect_kernel<<<blocks((long long)n, 128), 128, 0, s>>>(P, c->pairs.p, n, c->hit.p);
    RSG_LAUNCHED(ctx, "ccd intersection test");
  }
  check_overflow(c, s);
  return n;
}

}  // namespace

extern "C" {

rs_ccd_options rs_ccd_options_default(void) {
  rs_ccd_options o;
  o.gap = 0.05;
  o.reference_length = 0.0;
  o.max_iterations = 100;
  o.close_factor = 0.5;
  return o;
}

int rs_ccd_create(rs_ctx *ctx, int nv, int nf, const uint32_t *faces, rs_ccd **out) {
  *out = nullptr;
  return guard([&] {
    if (nv <= 0 || nf <= 0) fail(RS_INVALID_OPTION, "InvalidOption", "ccd", "a surface has vertices and faces");
    ctx->use();
    cudaStream_t s = ctx->stream;
    auto c = std::make_unique<rs_ccd>();
    c->ctx = ctx;
    c->nv = nv, c->nf = nf;
    std::vector<std::pair<uint32_t, uint32_t>> e;
    e.reserve(3 * (size_t)nf);
    for (int f = 0; f < nf; ++f)
      for (int k = 0; k < 3; ++k) {
        const uint32_t a = faces[3 * f + k], b = faces[3 * f + (k + 1) % 3];
        if (a >= (uint32_t)nv || b >= (uint32_t)nv)
          fail(RS_INVALID_OPTION, "InvalidOption", "ccd", "face index out of range");
        e.push_back({std::min(a, b), std::max(a, b)});
      }
    std::sort(e.begin(), e.end());
    e.erase(std::unique(e.begin(), e.end()), e.end());
    c->ne = (int)e.size();
    c->edges_h.resize(2 * e.size());
    for (size_t i = 0; i < e.size(); ++i) c->edges_h[2 * i] = e[i].first, c->edges_h[2 * i + 1] = e[i].second;
    c->faces.upload(faces, 3 * (size_t)nf, s);
    c->edges.upload(c->edges_h, s);
    c->start.alloc(nv), c->vel.alloc(nv), c->speed.alloc(nv), c->vbox.alloc(nv);
    c->core.alloc(nv), c->band.alloc(nv);
    c->ft.init(nf, s), c->et.init(c->ne, s);
    size_t t1 = 0, t2 = 0, t3 = 0;
    RSG_CUDA("ccd", cub::DeviceRadixSort::SortPairs(nullptr, t1, c->ft.key.p, c->ft.key_sorted.p, c->ft.idx.p,
                                                    c->ft.order.p, nf, 0, 30, s));
    RSG_CUDA("ccd", cub::DeviceRadixSort::SortPairs(nullptr, t2, c->et.key.p, c->et.key_sorted.p, c->et.idx.p,
                                                    c->et.order.p, c->ne, 0, 30, s));
    c->counters.alloc(2);
    c->pairs.alloc((size_t)8 * (nv + c->ne));  // grown on demand
    c->cub_tmp.alloc(std::max<size_t>(std::max(std::max(t1, t2), t3), 16));
    c->scratch.alloc(8);
    RSG_CUDA("ccd", cudaStreamSynchronize(s));
    ctx_retain(ctx);
    *out = c.release();
  });
}

void rs_ccd_free(rs_ccd *c) {
  if (!c) return;
  rs_ctx *ctx = c->ctx;
  delete c;
  ctx_release(ctx);
}

int rs_ccd_intersecting_pairs(rs_ccd *c, const double *positions, int64_t cap, uint32_t *out, int64_t *n) {
  return guard([&] {
    check_positions(positions, 3 * (size_t)c->nv, "positions");
    rs_ctx *ctx = c->ctx;
    ctx->use();
    cudaStream_t s = ctx->stream;
    const unsigned long long m = face_pairs(c, positions, s);
    std::vector<uint2> pr(m);
    std::vector<uint8_t> hit(m);
    if (m) {
      c->pairs.download(pr.data(), m, s);
      c->hit.download(hit.data(), m, s);
    }
    RSG_CUDA("ccd", cudaStreamSynchronize(s));
    std::vector<std::pair<uint32_t, uint32_t>> res;
    for (size_t i = 0; i < m; ++i)
      if (hit[i]) res.push_back({pr[i].x, pr[i].y});
    std::sort(res.begin(), res.end());
    *n = (int64_t)res.size();
    for (size_t i = 0; i < res.size() && (int64_t)i < cap; ++i) out[2 * i] = res[i].first, out[2 * i + 1] = res[i].second;
  });
}

int rs_ccd_set_band(rs_ccd *c, const double *positions, int64_t *n_pairs, int64_t *n_vertices) {
  return guard([&] {
    c->has_band = false;
    if (!positions) {
      if (n_pairs) *n_pairs = 0;
      if (n_vertices) *n_vertices = 0;
      return;
    }
    check_positions(positions, 3 * (size_t)c->nv, "positions");
    rs_ctx *ctx = c->ctx;
    ctx->use();
    cudaStream_t s = ctx->stream;
    const unsigned long long m = face_pairs(c, positions, s);
    RSG_CUDA("ccd", cudaMemsetAsync(c->core.p, 0, c->core.bytes(), s));
    RSG_CUDA("ccd", cudaMemsetAsync(c->scratch.p, 0, c->scratch.bytes(), s));
    unsigned long long *hits = c->scratch.p + 7, *count = c->scratch.p + 5;
    const Params P = make_params(c, 0.0, 0.0, 1, 0.0, 0.0, 0.0, nullptr);
    if (m) {
      core_kernel<<<blocks((long long)m, 128), 128, 0, s>>>(P, c->pairs.p, c->hit.p, m, c->core.p, hits);
      RSG_LAUNCHED(ctx, "ccd band");
    }
    RSG_CUDA("ccd", cudaMemcpyAsync(c->band.p, c->core.p, c->core.bytes(), cudaMemcpyDeviceToDevice, s));
    ring_kernel<<<blocks(c->ne, 256), 256, 0, s>>>(P, c->core.p, c->band.p);
    RSG_LAUNCHED(ctx, "ccd band");
    count_flags_kernel<<<blocks(c->nv, 256), 256, 0, s>>>(c->nv, c->band.p, count);
    RSG_LAUNCHED(ctx, "ccd band");
    unsigned long long res[8];
    c->scratch.download(res, 8, s);
    RSG_CUDA("ccd", cudaStreamSynchronize(s));
    c->has_band = res[5] > 0;  // an empty band is no band (ccd.rs:790-792)
    if (n_pairs) *n_pairs = (int64_t)res[7];
    if (n_vertices) *n_vertices = (int64_t)res[5];
  });
}

int rs_ccd_first_contact(rs_ccd *c, const double *start, const double *velocity, double tau_end,
                         const rs_ccd_options *opts, double *tau_max, int64_t *report7) {
  return guard([&] {
    auto t_begin = std::chrono::steady_clock::now();
    const rs_ccd_options o = opts ? *opts : rs_ccd_options_default();
    // CcdOptions::validate (ccd.rs:126-153) and first_contact's checks (ccd.rs:820-835)
    if (!(std::isfinite(o.gap) && o.gap > 0.0))
      fail(RS_INVALID_OPTION, "InvalidOption", "ccd", "ccd.gap must be finite and positive");
    if (!(std::isfinite(o.reference_length) && o.reference_length >= 0.0))
      fail(RS_INVALID_OPTION, "InvalidOption", "ccd",
           "ccd.reference_length must be finite and positive (0: the mean edge length of start)");
    if (o.max_iterations < 1) fail(RS_INVALID_OPTION, "InvalidOption", "ccd", "ccd.max_iterations must be at least 1");
    if (!(o.close_factor >= 0.0 && o.close_factor < 1.0))
      fail(RS_INVALID_OPTION, "InvalidOption", "ccd", "ccd.close_factor must be in [0, 1)");
    if (!(std::isfinite(tau_end) && tau_end >= 0.0))
      fail(RS_INVALID_OPTION, "InvalidOption", "ccd", "tau_end must be finite and non-negative");
    const int nv = c->nv;
    check_positions(start, 3 * (size_t)nv, "positions");
    for (size_t i = 0; i < 3 * (size_t)nv; ++i)
      if (!std::isfinite(velocity[i]))
        fail(RS_INVALID_OPTION, "InvalidOption", "ccd", "velocity must have finite components");
    rs_ctx *ctx = c->ctx;
    ctx->use();
    cudaStream_t s = ctx->stream;
    // host scalars, in the reference's order: the mean edge length over the sorted edges and
    // the largest speed
    double sum = 0.0;
    for (int i = 0; i < c->ne; ++i) {
      const double *x = start + 3 * (size_t)c->edges_h[2 * i], *y = start + 3 * (size_t)c->edges_h[2 * i + 1];
      const double d0 = x[0] - y[0], d1 = x[1] - y[1], d2 = x[2] - y[2];
      sum += std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    }
    const double mel = sum / (double)c->ne;
    const double ell = o.reference_length > 0.0 ? o.reference_length : mel;
    const double gap_abs = o.gap * ell;
    double vmax = 0.0;
    for (int v = 0; v < nv; ++v) {
      const double *u = velocity + 3 * (size_t)v;
      vmax = std::fmax(vmax, std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]));
    }
    const double t1 = vmax > 0.0 ? mel / vmax : INFINITY;
    c->start.upload(reinterpret_cast<const double3 *>(start), nv, s);
    c->vel.upload(reinterpret_cast<const double3 *>(velocity), nv, s);
    speed_kernel<<<blocks(nv, 256), 256, 0, s>>>(nv, c->vel.p, c->speed.p);
    RSG_LAUNCHED(ctx, "ccd speed");
    const double h = 0.5 * gap_abs * (1.0 + 1e-6);
    RSG_CUDA("ccd", cudaMemsetAsync(c->scratch.p, 0, c->scratch.bytes(), s));
    const uint8_t *band = c->has_band ? c->band.p : nullptr;
    int64_t windows = 0, pairs_total = 0, close = 0, touching = 0, exempt = 0, evals = 0, contact = 0;
    double tau = tau_end, lo = 0.0, hi = std::fmin(t1, tau_end);
    const unsigned long long kInf = 0x7FF0000000000000ull;
    for (;;) {
      if (vmax == 0.0) hi = 0.0;
      windows += 1;
      const Params P = make_params(c, gap_abs, o.close_factor, o.max_iterations, h, lo, hi, band);
      reset_kernel<<<1, 32, 0, s>>>(P.best, P.tally);
      RSG_LAUNCHED(ctx, "ccd reset");
      vbox_kernel<<<blocks(nv, 256), 256, 0, s>>>(nv, c->start.p, c->vel.p, lo, hi, c->vbox.p);
      RSG_LAUNCHED(ctx, "ccd boxes");
      double3 gl, gs;
      morton_grid(start, nv, vmax * hi + h, gl, gs);
      build_tree(c, c->ft, 0, h, gl, gs, s);
      build_tree(c, c->et, 1, h, gl, gs, s);
      // broad phase: the candidate pairs of both kinds, vertex-face first
      int64_t exempt_w = 0;
      const unsigned long long n_vt = collect<0>(c, P, c->ft.view(), nv, 0, false, s, &exempt_w);
      const unsigned long long n_ee = collect<1>(c, P, c->et.view(), c->ne, n_vt, true, s, &exempt_w);
      // narrow phase, one thread per candidate pair
      if (n_vt) {
        narrow_kernel<0><<<blocks((long long)n_vt, 128), 128, 0, s>>>(P, c->pairs.p, n_vt);
        RSG_LAUNCHED(ctx, "ccd vertex-triangle");
      }
      if (n_ee) {
        narrow_kernel<1><<<blocks((long long)n_ee, 128), 128, 0, s>>>(P, c->pairs.p + n_vt, n_ee);
        RSG_LAUNCHED(ctx, "ccd edge-edge");
      }
      unsigned long long res[8];
      c->scratch.download(res, 8, s);
      RSG_CUDA("ccd", cudaStreamSynchronize(s));
      if (reinterpret_cast<int *>(res + 6)[0]) fail(RS_INTERNAL, "Internal", "ccd", "box tree stack overflow");
      pairs_total += (int64_t)res[1];
      evals += (int64_t)res[4];
      if (lo == 0.0) close = (int64_t)res[2], touching = (int64_t)res[3], exempt = exempt_w;
      if (res[0] != kInf) {
        double b;
        std::memcpy(&b, &res[0], sizeof(b));
        tau = b;
        contact = 1;
        break;
      }
      if (hi >= tau_end || vmax == 0.0) break;
      lo = hi;
      hi = std::fmin(std::fmax(2.0 * hi, hi + t1), tau_end);
      if (hi <= lo) break;
    }
    *tau_max = tau;
    if (report7) {
      report7[0] = contact, report7[1] = windows, report7[2] = pairs_total, report7[3] = close;
      report7[4] = touching, report7[5] = exempt, report7[6] = evals;
    }
    c->last_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_begin).count();
  });
}

int rs_ccd_last_seconds(rs_ccd *c, double *seconds) {
  return guard([&] { *seconds = c->last_seconds; });
}

}  // extern "C"
