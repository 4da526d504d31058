// Device code of the Barnes-Hut tangent-point energy and its exact adjoint gradient
// (RS/src/energy/barnes_hut.rs; kernel RS/src/kernel.rs). See bh.cu for the host driver.
//
// Data layout in HBM (per evaluation, BVH order = the order of the tree's `order` array, so a
// leaf's faces are contiguous):
//   fxa[p] : float4 (X_S - X_leaf (xyz, FP32 offset from the leaf centroid), a_S)
//   fnn[p] : float4 (N_S (xyz), 0)
//   ncA[n] : double4 (X_n (xyz), A_n) cluster centroid and area of every node, FP64
//   nch[n], ncl[n] : the same centroid as a float pair (hi + lo) and the area in FP32
// A pair's separation is (X_L - X_C) formed from the float pairs ((hi_L - hi_C) + (lo_L - lo_C),
// exact to FP32 rounding of the result), plus the difference of the two FP32 offsets. This
// keeps v = X_S - X_T at FP32 precision relative to |v| (not to |X|), which the near-field
// terms (r^-12 nu^6) need, without FP64 work in the pair kernel.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rsg {

struct BhDev {
  // chunks of the transposed lists (long lists of degenerate leaves / big nodes are split):
  // fchunk = (leaf ordinal, exact_t begin, end, -), fchunk_off per leaf; nchunk likewise for
  // the transposed lumped list per node; fpart / npart hold the chunks' partial sums
  const uint4 *fchunk, *nchunk;
  const uint32_t *fchunk_off, *nchunk_off;
  float *fpart;
  float4 *npart;
  int n_fchunks, n_nchunks;
  // topology (fixed per step)
  const uint32_t *faces;       // 3F, original face order
  const uint32_t *order;       // F: BVH position -> face
  const uint32_t *node_start;  // N
  const uint32_t *node_end;    // N
  const uint32_t *node_right;  // N
  const uint32_t *node_parent; // N (root: 0)
  const uint32_t *leaves;      // L: node id of each leaf
  const uint32_t *leaf_of_pos; // F: leaf ordinal of each BVH position
  const uint32_t *schedule;    // work items, most work first
  const uint4 *items;          // per work item: lumped [x, y), exact [z, w) entry ranges
  const uint32_t *item_leaf;   // per work item: its leaf ordinal
  const uint32_t *item_off;    // L + 1: the work items of each leaf (leaf-major numbering)
  int n_items;
  const uint32_t *chain_off;   // L + 1: root -> leaf chains
  const uint32_t *chain;
  const uint32_t *inc_off;     // V + 1: vertex -> incident (face << 2 | corner), faces ascending
  const uint32_t *inc;
  // interaction lists (CSR per leaf ordinal) and their transposes
  const uint32_t *lumped_off, *lumped, *exact_off, *exact, *partner_off;
  const uint32_t *lumped_t_off, *lumped_t, *exact_t_off, *exact_t;
  int n_vertices, n_faces, n_nodes, n_leaves;
  // per-evaluation state
  float4 *fxa, *fnn;
  float4 *fol;      // per position: lo part of the offset (xyz) -- offset = fxa.xyz + fol.xyz
  float4 *fnl;      // per position: lo part of the normal (xyz), alpha_S = N_S.(X_S - X_leaf) (w)
  double4 *ncA;     // node centroid (xyz) and area (w)
  float4 *nch;      // node centroid as a float pair: hi (xyz) and area (w) ...
  float4 *ncl;      // ... and lo (xyz): X = hi + lo to ~48 bits, no FP64 in the pair kernel
  double4 *nmom;    // node first moment (xyz) and area (w), for the bottom-up refit
  uint32_t *refit_count;
  // outputs and scratch
  float4 *own;       // 16 per work item (2 per leaf face slot): (d_a, d_x), (d_n, 0)
  float4 *node_term; // per lumped entry: (b, u)
  float4 *partner;   // per partner slot: (d_a, d_x)
  float4 *node_sum;  // per node: (b_C, u_C)
  float4 *leaf_bu;   // per leaf: (beta, U) of the downward pass
  float4 *partials;  // 2 per face (by face id): (d_a, d_x), (d_n, 0)
  double *item_energy;
  unsigned int *ticket;
};

// Exponents of K = |N.v|^alpha |v|^-beta in the forms the kernels evaluate:
// K = q^(alpha/2) r2^((alpha-beta)/2), q = nu^2 / r2 in [0, 1]; c_n = alpha nu q^(alpha/2-1) r2^((alpha-beta)/2-1).
struct Pow {
  float alpha, beta;
  int a_int;   // alpha as an integer, or -1
  int ab_int;  // beta - alpha as an integer, or -1
};

// q^(alpha/2 - 1): (alpha - 2)/2 = h, integer or half-integer for integer alpha.
__device__ __forceinline__ float pow_q1(const Pow &p, float q) {
  if (p.a_int >= 2) {
    int m = p.a_int - 2;  // q^(m/2)
    float acc = 1.f, x = q;
    int k = m >> 1;
    while (k) {
      if (k & 1) acc *= x;
      x *= x;
      k >>= 1;
    }
    if (m & 1) acc *= sqrtf(q);
    return acc;
  }
  return q > 0.f ? powf(q, 0.5f * p.alpha - 1.f) : 0.f;
}

// r2^((alpha-beta)/2) = ir2^((beta-alpha)/2)
__device__ __forceinline__ float pow_r(const Pow &p, float r2, float ir2) {
  if (p.ab_int >= 0) {
    int m = p.ab_int;
    float acc = 1.f, x = ir2;
    int k = m >> 1;
    while (k) {
      if (k & 1) acc *= x;
      x *= x;
      k >>= 1;
    }
    if (m & 1) acc *= rsqrtf(r2);
    return acc;
  }
  return powf(r2, 0.5f * (p.alpha - p.beta));
}

// K and c_n for (alpha, beta) = (6, 12) (FAST) or the general exponents.
template <bool FAST>
__device__ __forceinline__ void kernel_k(const Pow &p, float nu, float r2, float ir2, float &K,
                                         float &cn) {
  float q = nu * nu * ir2;
  if (FAST) {
    float q2 = q * q;
    float i3 = ir2 * ir2 * ir2;
    float t = q2 * i3;  // nu^4 r^-10 .. scaled: q^2 ir2^3
    K = t * q;
    cn = 6.f * nu * t * ir2;
  } else {
    float a1 = pow_q1(p, q);
    float b = pow_r(p, r2, ir2);
    float t = a1 * b;
    K = t * q;
    cn = (nu == 0.f) ? 0.f : p.alpha * nu * t * ir2;
  }
}

// Kahan-compensated FP32 accumulator.
struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ float value() const { return s - c; }
};

}  // namespace rsg
