// Continuous collision detection of a mesh moving against itself -- TEST INFRASTRUCTURE ONLY
// (see rs_oracle.h). Restates first_contact of RS/src/ccd.rs:762-884 without obstacles and
// without an exempt band, its window pass (ccd.rs:887-1045), the conservative advancement
// (ccd.rs:529-592), the Lipschitz bound (ccd.rs:480-496) and the distances of
// RC/src/ccd.rs:237-319, operation for operation (built with -ffp-contract=off).
//
// The broad phase here finds every pair whose inflated swept boxes overlap by an x sweep with
// the exact overlap test. The reference reaches the same set through its box trees: the tree
// query tests every element box against the query box (ccd.rs:359-389), so the tree only
// prunes.
//
// The reference also passes each pair a horizon, the earliest contact its query has found so
// far. A pair's result does not depend on it: the advancement reaches its contact time through
// the same iterates whatever the horizon. A horizon at or below that time ends it with "none"
// first. The horizon only drops pairs that cannot lower the minimum, so tau_max, the window
// count and the candidate, close and touching counts here equal the reference's. Each pair
// runs against the full window.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "rs_oracle.h"
#include "rso_internal.hpp"

namespace rso {
namespace {

struct Box {
  v3 lo, hi;
};

inline v3 at(v3 p, v3 u, double t) { return {p[0] + t * u[0], p[1] + t * u[1], p[2] + t * u[2]}; }

// f64::clamp(0, 1): a NaN stays NaN.
inline double clamp01(double x) {
  if (x < 0.0) x = 0.0;
  if (x > 1.0) x = 1.0;
  return x;
}

double point_segment_distance(v3 p, v3 a, v3 b) {  // RC/src/ccd.rs:237-247
  const v3 ab = sub(b, a), ap = sub(p, a);
  const double e = dot(ab, ab);
  const double t = e > 0.0 ? clamp01(dot(ap, ab) / e) : 0.0;
  return norm(sub(ap, scale(ab, t)));
}

double segment_segment_distance(v3 p1, v3 q1, v3 p2, v3 q2) {  // RC/src/ccd.rs:266-291
  double best = fmin_(fmin_(fmin_(point_segment_distance(p1, p2, q2), point_segment_distance(q1, p2, q2)),
                            point_segment_distance(p2, p1, q1)),
                      point_segment_distance(q2, p1, q1));
  const v3 d1 = sub(q1, p1), d2 = sub(q2, p2);
  const double a = dot(d1, d1), e = dot(d2, d2);
  const v3 n = cross(d1, d2);
  const double nn = dot(n, n);
  if (a > 0.0 && e > 0.0 && nn > 0.0) {
    const v3 r = sub(p1, p2);
    const double b = dot(d1, d2), c = dot(d1, r), f = dot(d2, r);
    double s = clamp01(dot(cross(sub(p2, p1), d2), n) / nn);
    const double t = clamp01((b * s + f) / e);
    s = clamp01((b * t - c) / a);
    const v3 c1 = add(p1, scale(d1, s)), c2 = add(p2, scale(d2, t));
    best = fmin_(best, norm(sub(c1, c2)));
  }
  return best;
}

double point_triangle_distance(v3 p, v3 a, v3 b, v3 c) {  // RC/src/ccd.rs:298-319
  const double edges =
      fmin_(fmin_(point_segment_distance(p, a, b), point_segment_distance(p, b, c)), point_segment_distance(p, c, a));
  const v3 ab = sub(b, a), ac = sub(c, a);
  const v3 n = cross(ab, ac);
  const double nn = dot(n, n);
  if (nn <= 0.0) return edges;
  const v3 ap = sub(p, a);
  const double v = dot(cross(ap, ac), n) / nn;
  const double w = dot(cross(ab, ap), n) / nn;
  if (v >= 0.0 && w >= 0.0 && v + w <= 1.0) {
    const double h = std::fabs(dot(ap, n)) / std::sqrt(nn);
    return fmin_(edges, h);
  }
  return edges;
}

// max |u_a - c| + max |u_b - c| for the better of c = 0 and the mean corner velocity,
// times 1 + 1e-12 (ccd.rs:480-496).
double lipschitz(const std::vector<v3> &ua, const std::vector<v3> &ub) {
  const double n = (double)(ua.size() + ub.size());
  v3 mean{0.0, 0.0, 0.0};
  for (const v3 &v : ua) mean = add(mean, v);
  for (const v3 &v : ub) mean = add(mean, v);
  mean = scale(mean, 1.0 / n);
  auto l_of = [&](v3 c) {
    double la = 0.0, lb = 0.0;
    for (const v3 &v : ua) la = fmax_(la, norm(sub(v, c)));
    for (const v3 &v : ub) lb = fmax_(lb, norm(sub(v, c)));
    return la + lb;
  };
  return fmin_(l_of({0.0, 0.0, 0.0}), l_of(mean)) * (1.0 + 1e-12);
}

constexpr double kMargin = 1.0 + 1e-12;  // ccd.rs:498-499

struct Tally {
  int64_t pairs = 0, close = 0, touching = 0, exempt = 0;
};

// Conservative advancement of one pair on [lo, hi] (ccd.rs:529-592); NaN for "none".
template <class Dist, class LRefined>
double advance(const Dist &dist, double l_cheap, const LRefined &l_refined, double gap_abs, int max_iterations,
               double close_factor, double lo, double hi, Tally &tally) {
  const double d0 = dist(0.0);
  tally.pairs += 1;
  if (lo == 0.0) {
    if (d0 <= 1e-12 * gap_abs) {
      tally.touching += 1;
      return NAN;
    }
    if (d0 < gap_abs) tally.close += 1;
  } else if (d0 <= 1e-12 * gap_abs) {
    return NAN;
  }
  const double target = d0 > gap_abs ? gap_abs : close_factor * d0;
  const double slack = 1e-9 * d0;
  double l = l_cheap;
  bool refined = false;
  double tau = lo;
  double d = lo == 0.0 ? d0 : dist(lo);
  for (int it = 0; it < max_iterations; ++it) {
    if (std::isnan(d) || d - target <= slack) return tau;
    double next = tau + (d - target) / l;
    if (next >= hi && !refined) {
      l = fmin_(l, l_refined());
      refined = true;
      next = tau + (d - target) / l;
    }
    if (next >= hi || std::isnan(next)) return NAN;
    tau = next;
    d = dist(tau);
  }
  return tau;
}

double mean_edge_length(const std::vector<std::pair<uint32_t, uint32_t>> &edges, const std::vector<v3> &p) {
  double sum = 0.0;  // RS/src/geometry.rs:249-256, edges in Surface order (sorted (min, max))
  for (auto [a, b] : edges) sum += norm(sub(p[a], p[b]));
  return sum / (double)edges.size();
}

bool overlaps(const Box &a, const Box &b) {  // ccd.rs:258-261
  for (int k = 0; k < 3; ++k)
    if (!(a.lo[k] <= b.hi[k] && b.lo[k] <= a.hi[k])) return false;
  return true;
}

Box inflate(const Box &b, double h) {  // ccd.rs:251-256
  return {{b.lo[0] - h, b.lo[1] - h, b.lo[2] - h}, {b.hi[0] + h, b.hi[1] + h, b.hi[2] + h}};
}

Box unite(const Box &a, const Box &b) {  // Aabb::union, RC/src/spatial/aabb.rs:45-52
  Box r = a;
  for (int k = 0; k < 3; ++k) r.lo[k] = fmin_(r.lo[k], b.lo[k]), r.hi[k] = fmax_(r.hi[k], b.hi[k]);
  return r;
}

struct Result {
  double tau = NAN;  // NaN: no contact in the window
  Tally tally;
};

// All pairs of one window (ccd.rs:887-1045 without obstacles and band).
Result window(const std::vector<tri> &faces, const std::vector<std::pair<uint32_t, uint32_t>> &edges,
              const std::vector<v3> &start, const std::vector<v3> &vel, const std::vector<double> &speed,
              double gap_abs, int max_iterations, double close_factor, double lo, double hi,
              const uint8_t *band) {
  const size_t nv = start.size(), nf = faces.size(), ne = edges.size();
  const double h = 0.5 * gap_abs * (1.0 + 1e-6);
  std::vector<Box> vbox(nv), fbox(nf), ebox(ne);
  for (size_t v = 0; v < nv; ++v) {
    // hull of the positions at both ends: Aabb::empty grown by each point
    const v3 a = at(start[v], vel[v], lo), b = at(start[v], vel[v], hi);
    Box bx{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
    for (int k = 0; k < 3; ++k) {
      bx.lo[k] = fmin_(fmin_(bx.lo[k], a[k]), b[k]);
      bx.hi[k] = fmax_(fmax_(bx.hi[k], a[k]), b[k]);
    }
    vbox[v] = bx;
  }
  for (size_t f = 0; f < nf; ++f)
    fbox[f] = inflate(unite(unite(vbox[faces[f][0]], vbox[faces[f][1]]), vbox[faces[f][2]]), h);
  for (size_t e = 0; e < ne; ++e) ebox[e] = inflate(unite(vbox[edges[e].first], vbox[edges[e].second]), h);

  // Broad phase by an x sweep: the element boxes sorted by lo.x; a query scans the elements
  // with lo.x in [q.lo.x - W, q.hi.x], W the widest element box in x (padded against rounding),
  // which every box overlapping q satisfies; the exact overlap test then decides, so the
  // candidates are those of an enumeration of all pairs. Queries run on the oracle's threads;
  // their results combine by a minimum and integer sums, which do not depend on the order.
  struct Sweep {
    std::vector<uint32_t> ord;
    std::vector<double> key;
    double w = 0.0;
  };
  auto make_sweep = [](const std::vector<Box> &b) {
    Sweep sw;
    sw.ord.resize(b.size());
    for (size_t i = 0; i < b.size(); ++i) sw.ord[i] = (uint32_t)i, sw.w = fmax_(sw.w, b[i].hi[0] - b[i].lo[0]);
    std::sort(sw.ord.begin(), sw.ord.end(), [&](uint32_t x, uint32_t y) {
      return b[x].lo[0] < b[y].lo[0] || (b[x].lo[0] == b[y].lo[0] && x < y);
    });
    sw.key.resize(b.size());
    for (size_t i = 0; i < b.size(); ++i) sw.key[i] = b[sw.ord[i]].lo[0];
    sw.w = sw.w * 1.000001 + 1e-300;
    return sw;
  };
  const Sweep fs = make_sweep(fbox), es = make_sweep(ebox);
  auto range = [](const Sweep &sw, const Box &q) {
    const double from = q.lo[0] - sw.w - std::fabs(q.lo[0]) * 1e-12;
    const size_t b = std::lower_bound(sw.key.begin(), sw.key.end(), from) - sw.key.begin();
    const size_t e = std::upper_bound(sw.key.begin(), sw.key.end(), q.hi[0]) - sw.key.begin();
    return std::make_pair(b, e);
  };
  Result out;
  std::mutex mu;
  auto merge = [&](const Result &r) {
    std::lock_guard<std::mutex> lock(mu);
    if (!std::isnan(r.tau) && (std::isnan(out.tau) || r.tau < out.tau)) out.tau = r.tau;
    out.tally.pairs += r.tally.pairs, out.tally.close += r.tally.close;
    out.tally.touching += r.tally.touching, out.tally.exempt += r.tally.exempt;
  };
  auto offer = [](Result &r, double t) {
    if (!std::isnan(t) && (std::isnan(r.tau) || t < r.tau)) r.tau = t;
  };
  // vertex against triangle
  parallel_for((int64_t)nv, [&](int64_t v0, int64_t v1) {
    Result loc;
    for (uint32_t v = (uint32_t)v0; v < (uint32_t)v1; ++v) {
      const Box q = inflate(vbox[v], h);
      const auto [rb, re] = range(fs, q);
      for (size_t k = rb; k < re; ++k) {
        const uint32_t f = fs.ord[k];
        if (!overlaps(fbox[f], q)) continue;
        const tri &t = faces[f];
        if (t[0] == v || t[1] == v || t[2] == v) continue;
        if (band && band[v] && (band[t[0]] || band[t[1]] || band[t[2]])) {  // ccd.rs:947-950
          loc.tally.exempt += 1;
          continue;
        }
        const v3 p = start[v], u = vel[v];
        const v3 tp[3] = {at(start[t[0]], vel[t[0]], 0.0), at(start[t[1]], vel[t[1]], 0.0),
                          at(start[t[2]], vel[t[2]], 0.0)};
        const v3 tu[3] = {vel[t[0]], vel[t[1]], vel[t[2]]};
        const double tri_speed = fmax_(fmax_(speed[t[0]], speed[t[1]]), speed[t[2]]);
        const double lc = (speed[v] + tri_speed) * kMargin;
        auto dist = [&](double tt) {
          return point_triangle_distance(at(p, u, tt), at(tp[0], tu[0], tt), at(tp[1], tu[1], tt),
                                         at(tp[2], tu[2], tt));
        };
        auto lref = [&] { return lipschitz({u}, {tu[0], tu[1], tu[2]}); };
        offer(loc, advance(dist, lc, lref, gap_abs, max_iterations, close_factor, lo, hi, loc.tally));
      }
    }
    merge(loc);
  });
  // edge against edge, e2 > e, no common vertex
  parallel_for((int64_t)ne, [&](int64_t e0, int64_t e1) {
    Result loc;
    for (uint32_t e = (uint32_t)e0; e < (uint32_t)e1; ++e) {
      const Box q = ebox[e];
      const uint32_t a = edges[e].first, b = edges[e].second;
      const auto [rb, re] = range(es, q);
      for (size_t k = rb; k < re; ++k) {
        const uint32_t e2 = es.ord[k];
        if (e2 <= e || !overlaps(ebox[e2], q)) continue;
        const uint32_t c = edges[e2].first, d = edges[e2].second;
        if (c == a || c == b || d == a || d == b) continue;
        if (band && (band[a] || band[b]) && (band[c] || band[d])) {  // ccd.rs:1001-1004
          loc.tally.exempt += 1;
          continue;
        }
        const v3 pp[2] = {start[a], start[b]}, uu[2] = {vel[a], vel[b]};
        const v3 qq[2] = {start[c], start[d]}, ww[2] = {vel[c], vel[d]};
        const double lc = (fmax_(speed[a], speed[b]) + fmax_(speed[c], speed[d])) * kMargin;
        auto dist = [&](double tt) {
          return segment_segment_distance(at(pp[0], uu[0], tt), at(pp[1], uu[1], tt), at(qq[0], ww[0], tt),
                                          at(qq[1], ww[1], tt));
        };
        auto lref = [&] { return lipschitz({uu[0], uu[1]}, {ww[0], ww[1]}); };
        offer(loc, advance(dist, lc, lref, gap_abs, max_iterations, close_factor, lo, hi, loc.tally));
      }
    }
    merge(loc);
  });
  return out;
}

// ---- static queries (ccd.rs:1153-1215) ----

double orient(v3 a, v3 b, v3 c, v3 d) { return dot(cross(sub(b, a), sub(c, a)), sub(d, a)); }

bool segment_meets_triangle(v3 p, v3 q, const v3 (&t)[3]) {  // ccd.rs:1158-1186
  const v3 a = t[0], b = t[1], c = t[2];
  const double d1 = orient(a, b, c, p), d2 = orient(a, b, c, q);
  if ((d1 > 0.0 && d2 > 0.0) || (d1 < 0.0 && d2 < 0.0)) return false;
  const double n = norm(cross(sub(b, a), sub(c, a)));
  const double len = fmax_(fmax_(fmax_(norm(sub(q, p)), norm(sub(b, a))), norm(sub(c, a))), norm(sub(c, b)));
  const double flat = 1e-12 * n * len;
  if (std::fabs(d1) <= flat && std::fabs(d2) <= flat) {
    const double eps = 1e-14 * (norm(sub(b, a)) + norm(sub(c, a)));
    return point_triangle_distance(p, a, b, c) <= eps || point_triangle_distance(q, a, b, c) <= eps ||
           segment_segment_distance(p, q, a, b) <= eps || segment_segment_distance(p, q, b, c) <= eps ||
           segment_segment_distance(p, q, c, a) <= eps;
  }
  const double s1 = orient(p, q, a, b), s2 = orient(p, q, b, c), s3 = orient(p, q, c, a);
  return (s1 >= 0.0 && s2 >= 0.0 && s3 >= 0.0) || (s1 <= 0.0 && s2 <= 0.0 && s3 <= 0.0);
}

bool triangles_intersect(const v3 (&t1)[3], const v3 (&t2)[3]) {  // ccd.rs:1188-1191
  for (int k = 0; k < 3; ++k)
    if (segment_meets_triangle(t1[k], t1[(k + 1) % 3], t2)) return true;
  for (int k = 0; k < 3; ++k)
    if (segment_meets_triangle(t2[k], t2[(k + 1) % 3], t1)) return true;
  return false;
}

// intersecting_pairs (ccd.rs:1229-1279): pairs f < g whose corner hulls overlap and that
// intersect (no common vertex), or whose one common vertex's opposite edge meets the other
// face; sorted. The candidate set is that of the reference's box tree (every element box is
// tested), enumerated by brute force.
std::vector<std::pair<uint32_t, uint32_t>> intersecting_pairs(const std::vector<tri> &faces,
                                                              const std::vector<v3> &p) {
  const size_t nf = faces.size();
  std::vector<Box> box(nf);
  for (size_t f = 0; f < nf; ++f) {
    Box b{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
    for (int c = 0; c < 3; ++c)
      for (int k = 0; k < 3; ++k)
        b.lo[k] = fmin_(b.lo[k], p[faces[f][c]][k]), b.hi[k] = fmax_(b.hi[k], p[faces[f][c]][k]);
    box[f] = b;
  }
  std::vector<std::pair<uint32_t, uint32_t>> out;
  for (uint32_t f = 0; f < nf; ++f)
    for (uint32_t g = f + 1; g < nf; ++g) {
      if (!overlaps(box[g], box[f])) continue;
      const tri &a = faces[f], &b = faces[g];
      int common[3], n_common = 0;
      for (int i = 0; i < 3; ++i)
        if (b[0] == a[i] || b[1] == a[i] || b[2] == a[i]) common[n_common++] = i;
      const v3 tf[3] = {p[a[0]], p[a[1]], p[a[2]]}, tg[3] = {p[b[0]], p[b[1]], p[b[2]]};
      bool hit = false;
      if (n_common == 0) {
        hit = triangles_intersect(tf, tg);
      } else if (n_common == 1) {
        const int i = common[0];
        int j = 0;
        while (b[j] != a[i]) ++j;
        hit = segment_meets_triangle(p[a[(i + 1) % 3]], p[a[(i + 2) % 3]], tg) ||
              segment_meets_triangle(p[b[(j + 1) % 3]], p[b[(j + 2) % 3]], tf);
      }
      if (hit) out.push_back({f, g});
    }
  return out;
}

// IntersectionBand::new (ccd.rs:1292-1319): the vertices of the intersecting faces, widened by
// one ring over the edges.
std::vector<uint8_t> intersection_band(const std::vector<tri> &faces,
                                       const std::vector<std::pair<uint32_t, uint32_t>> &edges,
                                       const std::vector<std::pair<uint32_t, uint32_t>> &pairs, size_t nv) {
  std::vector<uint8_t> core(nv, 0);
  for (auto [f, g] : pairs)
    for (uint32_t fid : {f, g})
      for (int c = 0; c < 3; ++c) core[faces[fid][c]] = 1;
  std::vector<uint8_t> band = core;
  if (!pairs.empty())
    for (auto [a, b] : edges)
      if (core[a] || core[b]) band[a] = band[b] = 1;
  return band;
}

}  // namespace
}  // namespace rso

using namespace rso;

static thread_local std::string g_ccd_err;

static int rso_fail(int code, const char *message) {
  g_ccd_err = message;
  return code;
}

extern "C" const char *rso_ccd_last_error(void) { return g_ccd_err.c_str(); }

// first_contact_with_band (ccd.rs:781-884) when use_band: the band of the start positions
// (IntersectionBand::new; empty for an embedded mesh, which changes nothing).
// out7: contact, windows, pairs tested, close pairs, touching pairs, exempt pairs, band vertices.
extern "C" int rso_ccd_first_contact(int nv, const double *start, int nf, const uint32_t *faces,
                                     const double *velocity, double tau_end, double gap, double reference_length,
                                     int max_iterations, double close_factor, int use_band, double *tau_max,
                                     int64_t *out7) {
  // CcdOptions::validate (ccd.rs:126-153) and first_contact's own checks (ccd.rs:820-835)
  if (!(std::isfinite(gap) && gap > 0.0)) return rso_fail(1, "ccd.gap must be finite and positive");
  if (!(std::isfinite(reference_length) && reference_length >= 0.0))
    return rso_fail(1, "ccd.reference_length must be finite and positive (0: the mean edge length)");
  if (max_iterations < 1) return rso_fail(1, "ccd.max_iterations must be at least 1");
  if (!(close_factor >= 0.0 && close_factor < 1.0)) return rso_fail(1, "ccd.close_factor must be in [0, 1)");
  if (!(std::isfinite(tau_end) && tau_end >= 0.0)) return rso_fail(1, "tau_end must be finite and non-negative");
  std::vector<v3> p(nv), u(nv);
  std::vector<double> speed(nv);
  for (int v = 0; v < nv; ++v) {
    p[v] = {start[3 * v], start[3 * v + 1], start[3 * v + 2]};
    u[v] = {velocity[3 * v], velocity[3 * v + 1], velocity[3 * v + 2]};
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(u[v][k])) return rso_fail(1, "velocity must have finite components");
    speed[v] = norm(u[v]);
  }
  std::vector<tri> F(nf);
  std::vector<std::pair<uint32_t, uint32_t>> edges;
  for (int f = 0; f < nf; ++f) {
    F[f] = {faces[3 * f], faces[3 * f + 1], faces[3 * f + 2]};
    for (int k = 0; k < 3; ++k) {
      const uint32_t a = F[f][k], b = F[f][(k + 1) % 3];
      if (a >= (uint32_t)nv || b >= (uint32_t)nv) return rso_fail(1, "face index out of range");
      edges.push_back({std::min(a, b), std::max(a, b)});
    }
  }
  std::sort(edges.begin(), edges.end());
  edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
  if (edges.empty()) return rso_fail(1, "a surface has edges");
  std::vector<uint8_t> band;
  int64_t band_vertices = 0;
  if (use_band) {
    band = intersection_band(F, edges, intersecting_pairs(F, p), (size_t)nv);
    for (uint8_t b : band) band_vertices += b;
    if (band_vertices == 0) band.clear();  // an empty band is no band (ccd.rs:790-792)
  }
  const double mel = mean_edge_length(edges, p);
  const double ell = reference_length > 0.0 ? reference_length : mel;
  const double gap_abs = gap * ell;
  double vmax = 0.0;
  for (int v = 0; v < nv; ++v) vmax = fmax_(vmax, norm(u[v]));
  const double t1 = vmax > 0.0 ? mel / vmax : INFINITY;
  double lo = 0.0, hi = fmin_(t1, tau_end);
  int64_t windows = 0, pairs = 0, close = 0, touching = 0, exempt = 0;
  double tau = tau_end;
  int64_t contact = 0;
  for (;;) {
    if (vmax == 0.0) hi = 0.0;
    windows += 1;
    const Result r = window(F, edges, p, u, speed, gap_abs, max_iterations, close_factor, lo, hi,
                            band.empty() ? nullptr : band.data());
    pairs += r.tally.pairs;
    if (lo == 0.0) close = r.tally.close, touching = r.tally.touching, exempt = r.tally.exempt;
    if (!std::isnan(r.tau)) {
      tau = r.tau;
      contact = 1;
      break;
    }
    if (hi >= tau_end || vmax == 0.0) break;
    lo = hi;
    hi = fmin_(fmax_(2.0 * hi, hi + t1), tau_end);
    if (hi <= lo) break;
  }
  *tau_max = tau;
  out7[0] = contact, out7[1] = windows, out7[2] = pairs, out7[3] = close, out7[4] = touching;
  out7[5] = exempt, out7[6] = band_vertices;
  return 0;
}

// intersecting_pairs (ccd.rs:1229-1279) of the positions, sorted; out holds up to cap pairs.
extern "C" int rso_ccd_intersecting_pairs(int nv, const double *pos, int nf, const uint32_t *faces, int64_t cap,
                                          uint32_t *out, int64_t *n) {
  std::vector<v3> p(nv);
  for (int v = 0; v < nv; ++v) p[v] = {pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]};
  std::vector<tri> F(nf);
  for (int f = 0; f < nf; ++f) {
    F[f] = {faces[3 * f], faces[3 * f + 1], faces[3 * f + 2]};
    for (int k = 0; k < 3; ++k)
      if (F[f][k] >= (uint32_t)nv) return rso_fail(1, "face index out of range");
  }
  const auto pairs = intersecting_pairs(F, p);
  *n = (int64_t)pairs.size();
  for (size_t i = 0; i < pairs.size() && (int64_t)i < cap; ++i) out[2 * i] = pairs[i].first, out[2 * i + 1] = pairs[i].second;
  return 0;
}

// The smallest distance over the pairs CCD constrains (vertex-triangle with the vertex not in
// the triangle, edge-edge without a common vertex), by brute force: the check of the tests'
// sampled motions.
extern "C" int rso_ccd_min_distance(int nv, const double *pos, int nf, const uint32_t *faces, double *out) {
  std::vector<v3> p(nv);
  for (int v = 0; v < nv; ++v) p[v] = {pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]};
  std::vector<std::pair<uint32_t, uint32_t>> edges;
  for (int f = 0; f < nf; ++f)
    for (int k = 0; k < 3; ++k) {
      const uint32_t a = faces[3 * f + k], b = faces[3 * f + (k + 1) % 3];
      if (a >= (uint32_t)nv || b >= (uint32_t)nv) return rso_fail(1, "face index out of range");
      edges.push_back({std::min(a, b), std::max(a, b)});
    }
  std::sort(edges.begin(), edges.end());
  edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
  double best = INFINITY;
  for (int v = 0; v < nv; ++v)
    for (int f = 0; f < nf; ++f) {
      const uint32_t a = faces[3 * f], b = faces[3 * f + 1], c = faces[3 * f + 2];
      if (a == (uint32_t)v || b == (uint32_t)v || c == (uint32_t)v) continue;
      best = fmin_(best, point_triangle_distance(p[v], p[a], p[b], p[c]));
    }
  for (size_t e = 0; e < edges.size(); ++e)
    for (size_t e2 = e + 1; e2 < edges.size(); ++e2) {
      const auto [a, b] = edges[e];
      const auto [c, d] = edges[e2];
      if (c == a || c == b || d == a || d == b) continue;
      best = fmin_(best, segment_segment_distance(p[a], p[b], p[c], p[d]));
    }
  *out = best;
  return 0;
}
