// Internal C++ types of the FP64 oracle -- TEST INFRASTRUCTURE ONLY (see rs_oracle.h).
//
// Vector helpers follow RC/src/kernel.rs:12-52 operation for operation (no FMA contraction:
// the recipe compiles with -ffp-contract=off, as Rust does not contract).
#pragma once
#include <array>
#include <cmath>
#include <cstdint>
#include <functional>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

namespace rso {

using v3 = std::array<double, 3>;
using tri = std::array<uint32_t, 3>;

inline v3 add(v3 a, v3 b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
inline v3 sub(v3 a, v3 b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
inline v3 scale(v3 a, double s) { return {a[0] * s, a[1] * s, a[2] * s}; }
inline v3 axpy(v3 a, double s, v3 b) { return {a[0] + s * b[0], a[1] + s * b[1], a[2] + s * b[2]}; }
inline double dot(v3 a, v3 b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline v3 cross(v3 a, v3 b) {
  return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
inline double norm(v3 a) { return std::sqrt(dot(a, a)); }

// Rust's f64::min / f64::max ignore a NaN argument, like fmin / fmax.
inline double fmin_(double a, double b) { return std::fmin(a, b); }
inline double fmax_(double a, double b) { return std::fmax(a, b); }

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// ---- exponents and the kernel (RS/src/kernel.rs) ----
struct Exponents {
  double alpha = 6, beta = 12;
  int alpha_int = 6, beta_int = 12;  // -1 when not a small integer
  static Exponents make(double alpha, double beta);  // validates (kernel.rs:50-76)
  double s() const { return (beta - 2.0) / alpha; }
  // (|nu|^alpha, sign(nu)|nu|^(alpha-1))  (kernel.rs:144-152)
  void nu_powers(double nu, double &pa, double &sp) const;
  // r^(-beta) from r^2  (kernel.rs:155-162)
  double r_power(double r2) const;
};

double ipow(double x, uint32_t n);  // kernel.rs:180-193

struct KernelEval {
  double value;
  v3 d_v, d_n;
};
double kernel_of_v(const Exponents &e, v3 v, v3 n);               // kernel.rs:206-210
KernelEval kernel_with_gradient_of_v(const Exponents &e, v3 v, v3 n);  // kernel.rs:238-250
// kernel.rs:256-275
void pair_terms(const Exponents &e, v3 v, v3 ns, v3 nt, double &k_st, double &k_ts, v3 &dv_st,
                v3 &dv_ts, v3 &dn_st);

// ---- geometry (RS/src/geometry.rs) ----
struct FaceGeometry {
  std::vector<double> areas;
  std::vector<v3> normals, barycenters;
};
void face_quantities(const std::array<v3, 3> &p, double &a, v3 &n, v3 &x);  // geometry.rs:33-39
std::array<v3, 3> face_pull_back(const std::array<v3, 3> &p, double d_area, v3 d_bary,
                                 v3 d_normal);  // geometry.rs:87-110
std::array<v3, 3> corners(const std::vector<v3> &pos, const tri &t);
// Surface::validate_positions (RS/src/surface.rs:513-541)
void validate_positions(int nv, const std::vector<v3> &pos, const std::vector<tri> &faces);
FaceGeometry face_geometry(const std::vector<v3> &pos, const std::vector<tri> &faces);
std::vector<v3> pull_back(int nv, const std::vector<v3> &pos, const std::vector<tri> &faces,
                          const std::vector<double> &da, const std::vector<v3> &dx,
                          const std::vector<v3> &dn);  // geometry.rs:172-188

// ---- axis-aligned boxes and the BVH (RC/src/spatial/{aabb,bvh}.rs) ----
struct Aabb {
  v3 lo{{INFINITY, INFINITY, INFINITY}}, hi{{-INFINITY, -INFINITY, -INFINITY}};
  bool empty() const { return lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]; }
  void grow(v3 p) {
    for (int k = 0; k < 3; ++k) lo[k] = fmin_(lo[k], p[k]), hi[k] = fmax_(hi[k], p[k]);
  }
  Aabb uni(const Aabb &o) const {
    Aabb r = *this;
    for (int k = 0; k < 3; ++k) r.lo[k] = fmin_(r.lo[k], o.lo[k]), r.hi[k] = fmax_(r.hi[k], o.hi[k]);
    return r;
  }
  double diameter_sq() const {
    if (empty()) return 0.0;
    double s = 0.0;
    for (int k = 0; k < 3; ++k) {
      double w = hi[k] - lo[k];
      s += w * w;
    }
    return s;
  }
};

struct Element {
  v3 point;
  Aabb bounds;
  double mass;
};

struct Node {
  Aabb bbox;
  double mass = 0;
  v3 moment{{0, 0, 0}};
  uint32_t start = 0, end = 0, right = 0;
  bool leaf() const { return right == 0; }
  v3 centroid() const { return {moment[0] / mass, moment[1] / mass, moment[2] / mass}; }
};

struct Bvh {
  std::vector<Node> nodes;
  std::vector<uint32_t> order;
  int leaf_size = 8;
  static Bvh build(const std::vector<Element> &el, int leaf_size, double min_fraction = 0.25);
  void refit(const std::vector<Element> &el);
};

double box_distance_sq(const Aabb &a, const Aabb &b);      // RS/src/spatial/mod.rs:131-138
double farthest_corner_distance(const Aabb &b, v3 x);       // RS/src/spatial/mod.rs:143-150

struct Cluster {
  double area;
  v3 centroid;
  std::array<double, 6> projector;
  Aabb bbox;
  double radius;
  double projector_quadratic_form(v3 v) const {  // RS/src/spatial/mod.rs:102-109
    const auto &p = projector;
    return p[0] * v[0] * v[0] + p[3] * v[1] * v[1] + p[5] * v[2] * v[2] +
           2.0 * (p[1] * v[0] * v[1] + p[2] * v[0] * v[2] + p[4] * v[1] * v[2]);
  }
};

bool bh_admissible(const Cluster &leaf, const Cluster &c, double theta);  // spatial/mod.rs:160-163

// FaceTree (RS/src/spatial/mod.rs:167-297)
struct FaceTree {
  Bvh bvh;
  std::vector<Cluster> clusters;
  std::vector<uint32_t> leaves, leaf_ordinal, leaf_of_face;
  static FaceTree build(const std::vector<v3> &pos, const std::vector<tri> &faces,
                        const FaceGeometry &g, int leaf_size);
  void refit(const std::vector<v3> &pos, const std::vector<tri> &faces, const FaceGeometry &g);
  std::vector<std::array<double, 6>> projectors(const FaceGeometry &g) const;
};
std::vector<Element> face_elements(const std::vector<v3> &pos, const std::vector<tri> &faces,
                                   const FaceGeometry &g);

void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)> &body);
int threads();

}  // namespace rso
