// Hierarchical (block cluster tree) products on the GPU: the Hs metric B~ + B~0 over face
// pairs (FaceMetricTree, RS/src/metric/hierarchical.rs:279-812) and the vertex-pair fractional
// operator L^V_{2-s} of the preconditioner (VertexFractionalTree, hierarchical.rs:998-1346),
// behind rs_metric_* / rs_vfrac_* of include/rsgpu.h.
//
// Both are kernel-matrix forms L u = 2 M^T diag(a) (diag(H~a) M u - H~(a M u)) with a block
// cluster tree H~: rank-one far blocks (cluster data) and exact near blocks. The near entries
// are NOT stored: every product evaluates them from the element records (FP32 offsets from the
// leaf centroid, normals) while it streams the columns, which costs less than reading a stored
// near field from HBM (0.3 G entries x 2 kernels at 204,800 faces).
//
// Per product (C channels per element: 9 gradient + 3 average per input vector for faces, 3
// per vector for vertices):
//   prologue    m = M x per element (FP32), element-major [n][C]
//   upward      up[node] = sum_{q in node} a_q m_q, bottom-up (the second child to arrive adds)
//   far         farx[node] = sum_{b in far(node)} h(node, b) up[b]            (warp per node)
//   rows        per leaf (warp): near sums over the chain's near blocks with H~a accumulated
//               in the same loop, far sums along the chain, z = H~a m - H~(a m)
//   epilogue    y = 2 M^T diag(a) W z (faces: per-vertex gather; vertices: y = 2 a z)
// H~a is formed with the same operations as H~(a m) for m = 1, so L 1 = 0 exactly (the
// reference's null-space property, hierarchical.rs:13-16).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

#include <cub/device/device_scan.cuh>

#include "block_tree.hpp"
#include "common.hpp"
#include "host_tree.hpp"
#include "hmat.hpp"
#include "profile.hpp"

namespace rsg {

constexpr int FACE = 0, VERTEX = 1;
// Which of the two kernels a channel uses: FACE_CH (vector q owns channels 12q..12q+11, the
// last three of them the averages, kernel 1), VERTEX_CH (kernel 0 throughout), ONES (channel
// c uses kernel c: the two-channel pass that forms the far part of H~a).
constexpr int FACE_CH = 0, VERTEX_CH = 1, ONES = 2;
template <int SEL>
__device__ __forceinline__ bool uses_k1(int c) {
  return SEL == FACE_CH ? (c % 12) >= 9 : (SEL == ONES ? c == 1 : false);
}

struct HDev {
  const uint32_t *start, *end, *right, *parent, *leaves, *chain_off, *chain;
  const uint32_t *far_ptr, *far_col;
  const uint4 *far_items;       // per far work item: node, block range [y, z) (at most kFarChunk), -
  const uint32_t *far_item_off; // per node: its far items [far_item_off[a], far_item_off[a + 1])
  float2 *fpart;                // per far item: C channel partial sums (float pairs)
  const float4 *far_coef;    // per far block: (k_0, k_1) as float pairs (k_0 hi, k_0 lo, k_1 hi, k_1 lo)
  const float4 *xh;          // per BVH position: position hi (xyz), weight a (w)
  const float4 *xl;          // per BVH position: position lo (xyz): X = hi + lo to ~48 bits
  const float4 *nrm;         // per BVH position: normal (faces only)
  const double2 *leaf_farA;  // per leaf: far sums of psi = a (k_0, k_1) along its chain, the far part of H~a
  double *leafsum;           // per leaf: C channel far sums along its chain
  const uint32_t *colidx;    // near columns of every leaf's chain, flattened, leaf by leaf
  const uint4 *items;        // per work item: leaf ordinal, column-range begin / end, weight base
  const void *wts;           // near weights per item: rows x (columns padded to 32), see NearW
  const uint32_t *item_off;  // per leaf: its work items [item_off[k], item_off[k + 1])
  double *up;                // per node: C channel sums of a m (FP64)
  float2 *up2;               // the same sums as float pairs (hi, lo), read by the far sums
  double *farx;              // per node: C channel far sums (FP64)
  float2 *part;              // per work item: 8 rows x C near sums as float pairs
  uint32_t *count;           // per node: arrival counter of the upward pass
  const float2 *m;           // [n][C] channel values as float pairs (hi, lo)
  float2 *z;                 // [n][C] results as float pairs
  int n_nodes, n_leaves, n_el, n_items, n_far_items, C;
  float neg_s;               // kernel exponent e applied to r^2: r2^e
  int pw_mode, pw_k;         // e = pw_k / pw_mode for pw_mode 2 or 3 (exact roots), else powf
};

// Error-free sum (Knuth): a + b = s + t exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &t) {
  s = a + b;
  const float bv = s - a;
  t = (a - (s - bv)) + (b - bv);
}

// (h, l) += (oh, ol) for float pairs.
// Layout of the channel values m: per element, C channels as float pairs (hi, lo), stored by
// channel pairs as (hi_2i, hi_2i+1, lo_2i, lo_2i+1) so that the near field reads the hi parts
// (and the lo parts) of two channels as one packed operand.
__device__ __forceinline__ int m_hi(int c) { return (c >> 1) * 4 + (c & 1); }
__device__ __forceinline__ float2 m_get(const float2 *row, int c) {
  const float *f = reinterpret_cast<const float *>(row);
  return make_float2(f[m_hi(c)], f[m_hi(c) + 2]);
}
__device__ __forceinline__ void m_set(float2 *row, int c, float2 v) {
  float *f = reinterpret_cast<float *>(row);
  f[m_hi(c)] = v.x, f[m_hi(c) + 2] = v.y;
}

// Two FP32 values in one 64-bit register (first in the low half) and the packed FP32 pair
// arithmetic of sm_100 and later (each half rounded to nearest, as the scalar operations).
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f2_pack(float a, float b) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float2 f2_unpack(f32x2 v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
__device__ __forceinline__ f32x2 f2_add(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
constexpr f32x2 kF2Sign = 0x8000000080000000ull;  // both halves' sign bits

// v as a float pair: hi = v rounded to FP32, lo = the rest rounded
__device__ __forceinline__ float2 to_pair(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}

__device__ __forceinline__ void pair_add(float &h, float &l, float oh, float ol) {
  float s, t;
  two_sum(h, oh, s, t);
  h = s;
  l = (l + ol) + t;
}

__device__ __forceinline__ float ipow(float x, int n) {
  float r = 1.f;
  for (; n > 0; --n) r *= x;
  return r;
}

// r2^e. For e = k/3 or k/2 (the exponents of integer alpha, beta) the power is an integer
// power times a correctly rounded root: a few roundings, independent of the size of
// log r2 (exp2(e log2 r2) loses accuracy in proportion to it).
__device__ __forceinline__ float r2pow(const HDev &d, float r2, float ir2) {
  if (d.pw_mode == 3 || d.pw_mode == 2) {
    const int q = d.pw_mode, k = d.pw_k;
    const int a = (k >= 0) ? k / q : -((-k + q - 1) / q);  // floor(k / q)
    const int b = k - q * a;                                // 0 .. q-1
    float base = a >= 0 ? ipow(r2, a) : ipow(ir2, -a);
    if (b) {
      const float root = q == 3 ? cbrtf(r2) : sqrtf(r2);
      base *= b == 1 ? root : root * root;
    }
    return base;
  }
  return powf(r2, d.neg_s);
}

// The near kernel values of an element pair (hierarchical.rs:185-189, 224-231 and 987-991):
// faces: [r2^-s, (nu_p^2 + nu_q^2)/2 r2^-2 r2^-s]; vertices: [r2^e].
template <int KIND>
__device__ __forceinline__ void near_kernel(const HDev &d, float d0, float d1, float d2,
                                            const float4 &np, const float4 &nq, float &k0, float &k1) {
  const float r2 = d0 * d0 + d1 * d1 + d2 * d2;
  const float ir2 = __frcp_rn(r2);
  const float h = r2pow(d, r2, ir2);
  k0 = h;
  if (KIND == FACE) {
    const float a = np.x * d0 + np.y * d1 + np.z * d2;
    const float b = nq.x * d0 + nq.y * d1 + nq.z * d2;
    k1 = 0.5f * (a * a + b * b) * ir2 * ir2 * h;
  } else {
    k1 = h;
  }
}

// Bottom-up channel sums in FP64: one warp per leaf (lanes over the channels) sums its
// elements in registers, then climbs; at every parent the second child to arrive adds
// left + right (fixed order, no waiting). The far field is FP64 end to end (upward, far sums, chain push-down): its sums
// cancel against m_p H~a for a smooth input just as the near sums do, and at O(nodes) and
// O(far blocks) work the FP64 rate costs little.
template <int CC>
__global__ void hm_upward_kernel(HDev d) {
  // one warp per leaf, lane l holding channels l, l + 32, ...
  constexpr int NPL = (CC + 31) / 32;
  const int k = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= d.n_leaves) return;
  const uint32_t leaf = d.leaves[k];
  double u[NPL];
#pragma unroll
  for (int i = 0; i < NPL; ++i) u[i] = 0.0;
  for (uint32_t p = d.start[leaf]; p < d.end[leaf]; ++p) {
    const double a = d.xh[p].w;
    const float2 *mp = d.m + (size_t)p * CC;
#pragma unroll
    for (int i = 0; i < NPL; ++i) {
      const int c = lane + 32 * i;
      if (c < CC) {
        const float2 v = m_get(mp, c);
        u[i] = fma(a, (double)v.x + (double)v.y, u[i]);
      }
    }
  }
  double *o = d.up + (size_t)leaf * CC;
  float2 *o2 = d.up2 + (size_t)leaf * CC;
#pragma unroll
  for (int i = 0; i < NPL; ++i)
    if (lane + 32 * i < CC) o[lane + 32 * i] = u[i], o2[lane + 32 * i] = to_pair(u[i]);
  uint32_t n = leaf;
  while (n != 0) {
    const uint32_t par = d.parent[n];
    __threadfence();  // this warp's sums of n, before the arrival is counted
    __syncwarp();
    unsigned old = 0u;
    if (lane == 0) old = atomicAdd(&d.count[par], 1u);
    old = __shfl_sync(0xffffffffu, old, 0);
    if ((old & 1u) == 0u) return;  // first child to arrive: the sibling's warp adds
    __threadfence();
    const double *l = d.up + (size_t)(par + 1) * CC;
    const double *r = d.up + (size_t)d.right[par] * CC;
    double *op = d.up + (size_t)par * CC;
    float2 *op2 = d.up2 + (size_t)par * CC;
#pragma unroll
    for (int i = 0; i < NPL; ++i) {
      const int c = lane + 32 * i;
      if (c < CC) {
        const double v = __ldcg(l + c) + __ldcg(r + c);
        op[c] = v, op2[c] = to_pair(v);
      }
    }
    n = par;
  }
}

// farx[a][c] = sum over the far blocks (a, b) of h(a, b)[kernel(c)] up[b][c] (block_tree.rs:
// 564-578) in double-float arithmetic: the coefficients and the node sums are float pairs
// (about 48 bits), each product is formed exactly to that width (FMA) and added by error-free
// transformations; the result is handed on in FP64. GB300 issues FP32 at many times its FP64
// rate. One warp per (node, group of at most twelve channels): lane = sub CG + c holds channel
// c of the group and takes the node's far blocks sub, sub + 2, ... (sub = 0, 1); the two
// partial sums are then added. The operations do not depend on the channel count, so the pass
// over psi = a (two channels) and a product pass add the same terms in the same order.
__device__ __forceinline__ void df_fma(float &ah, float &al, float kh, float kl, float uh, float ul) {
  const float ph = kh * uh;
  float pe = fmaf(kh, uh, -ph);
  pe = fmaf(kh, ul, pe);
  pe = fmaf(kl, uh, pe);
  float sh, se;
  two_sum(ah, ph, sh, se);
  se += al + pe;
  ah = sh + se;
  al = se - (ah - sh);
}

template <int SEL, int CC>
__global__ void hm_far_kernel(HDev d) {
  constexpr int CG = CC < 12 ? CC : 12;
  static_assert(CC % CG == 0 && 2 * CG <= 32, "channel groups");
  constexpr int NG = CC / CG;
  const int wg = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int w = wg / NG, grp = wg - w * NG;
  if (w >= d.n_far_items) return;
  const uint4 it = d.far_items[w];
  const int lane = threadIdx.x & 31, sub = lane / CG, c = lane - sub * CG;
  const int ch = grp * CG + c;
  float ah = 0.f, al = 0.f;
  if (sub < 2) {
    const bool k1 = uses_k1<SEL>(ch);
    uint32_t q = it.y + sub;
    // four of the lane's blocks at a time: loads first, then the additions in order
    for (; q + 6 < it.z; q += 8) {
      float4 kk[4];
      float2 u[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        kk[i] = d.far_coef[q + 2 * i];
        u[i] = d.up2[(size_t)d.far_col[q + 2 * i] * CC + ch];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
        df_fma(ah, al, k1 ? kk[i].z : kk[i].x, k1 ? kk[i].w : kk[i].y, u[i].x, u[i].y);
    }
    for (; q < it.z; q += 2) {
      const float4 k = d.far_coef[q];
      const float2 u = d.up2[(size_t)d.far_col[q] * CC + ch];
      df_fma(ah, al, k1 ? k.z : k.x, k1 ? k.w : k.y, u.x, u.y);
    }
  }
  const float oh = __shfl_down_sync(0xffffffffu, ah, CG), ol = __shfl_down_sync(0xffffffffu, al, CG);
  pair_add(ah, al, oh, ol);
  if (sub == 0) d.fpart[(size_t)w * CC + ch] = make_float2(ah, al);
}

// farx[a][c]: the node's item partials added in item order as float pairs, handed on in FP64
// (zero for a node without far blocks); one thread per (node, channel)
template <int CC>
__global__ void hm_far_final_kernel(HDev d) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)d.n_nodes * CC) return;
  const size_t a = t / CC;
  const int c = (int)(t - a * CC);
  float h = 0.f, l = 0.f;
  for (uint32_t i = d.far_item_off[a]; i < d.far_item_off[a + 1]; ++i) {
    const float2 v = d.fpart[(size_t)i * CC + c];
    pair_add(h, l, v.x, v.y);
  }
  d.farx[t] = (double)h + (double)l;
}

// Far coefficients (k_0, k_1) of every far block, FP64, as float pairs (hi, lo): d the centroid
// difference of the pair (lower node index first), h = r2^e, and for faces
// k_1 = (q_lo(d) + q_hi(d)) / 2 / r2^2 h with q the node's area-weighted projector form
// (proj = null: vertices, k_1 = k_0). One warp per far work item, lanes over its blocks.
__global__ void hm_far_coef_kernel(const uint4 *__restrict__ items, int n_items, const uint32_t *__restrict__ far_col,
                                   const double *__restrict__ cen, const double *__restrict__ proj, double e,
                                   float4 *__restrict__ coef) {
  const int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (w >= n_items) return;
  const uint4 it = items[w];
  const uint32_t a = it.x;
  auto qf = [&](uint32_t n, const double *d) {
    const double *p = proj + 6 * (size_t)n;
    return p[0] * d[0] * d[0] + p[3] * d[1] * d[1] + p[5] * d[2] * d[2] +
           2.0 * (p[1] * d[0] * d[1] + p[2] * d[0] * d[2] + p[4] * d[1] * d[2]);
  };
  for (uint32_t q = it.y + lane; q < it.z; q += 32) {
    const uint32_t b = far_col[q], lo = min(a, b), hi = max(a, b);
    const double d[3] = {cen[3 * (size_t)lo] - cen[3 * (size_t)hi], cen[3 * (size_t)lo + 1] - cen[3 * (size_t)hi + 1],
                         cen[3 * (size_t)lo + 2] - cen[3 * (size_t)hi + 2]};
    const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double h = pow(r2, e);
    const double h1 = proj ? 0.5 * (qf(lo, d) + qf(hi, d)) / (r2 * r2) * h : h;
    const float2 k0 = to_pair(h), k1 = to_pair(h1);
    coef[q] = make_float4(k0.x, k0.y, k1.x, k1.y);
  }
}

// Near weights of an element pair as the rows kernel applies them: faces (w_0, w_1) =
// a_q (k_0, k_1), vertices w_0 = a_q k_0; zero on the diagonal (q = p). Stored per work item
// as [row][column], rows padded to a multiple of 32 columns so that each 32-column slice
// starts on a 128-byte boundary.
template <int KIND>
using NearW = typename std::conditional<KIND == FACE, float2, float>::type;
constexpr int kTileW = 36;          // shared-memory row stride of a weight tile (bank spread)
constexpr uint32_t kFarChunk = 64;  // far blocks per far work item

template <int KIND>
__global__ void hm_weights_kernel(HDev d, size_t total) {
  // one warp per (item, row); lanes strided over the item's columns
  const size_t wr = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wr >= (size_t)d.n_items * 8) return;
  const uint32_t w = (uint32_t)(wr >> 3), r = (uint32_t)(wr & 7);
  const uint4 it = d.items[w];
  const uint32_t leaf = d.leaves[it.x];
  const uint32_t s0 = d.start[leaf], ns = d.end[leaf] - s0;
  if (r >= ns) return;
  const uint32_t p = s0 + r, ncol = it.z - it.y, npad = (ncol + 31) & ~31u;
  const float4 ph = d.xh[p], pl = d.xl[p];
  const float4 np = KIND == FACE ? d.nrm[p] : make_float4(0.f, 0.f, 0.f, 0.f);
  NearW<KIND> *out = reinterpret_cast<NearW<KIND> *>(const_cast<void *>(d.wts)) + it.w + (size_t)r * npad;
  for (uint32_t k = lane; k < npad; k += 32) {
    float w0 = 0.f, w1 = 0.f;
    if (k < ncol) {
      const uint32_t q = d.colidx[it.y + k];
      if (q != p) {
        const float4 qh = d.xh[q], ql = d.xl[q];
        const float d0 = (ph.x - qh.x) + (pl.x - ql.x);
        const float d1 = (ph.y - qh.y) + (pl.y - ql.y);
        const float d2 = (ph.z - qh.z) + (pl.z - ql.z);
        float k0, k1;
        near_kernel<KIND>(d, d0, d1, d2, np, KIND == FACE ? d.nrm[q] : np, k0, k1);
        w0 = k0 * qh.w, w1 = k1 * qh.w;
      }
    }
    if constexpr (KIND == FACE) out[k] = make_float2(w0, w1);
    else out[k] = w0;
  }
  (void)total;
}

// One tile of a work item in shared memory: the channel values of 32 columns (per channel
// pair the 16 bytes (hi, hi, lo, lo) of the paired layout), channel pair major (consecutive columns in consecutive 16-byte slots, so that the lanes of a
// load phase reading up to 8 columns meet no bank twice), and the near weights of up to
// 8 rows x 32 columns.
template <int KIND, int CC>
struct alignas(16) RowsTile {
  float4 m[CC / 2][32];
  NearW<KIND> w[8][kTileW];
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Near sums of one work item (a slice of the flattened near columns of a leaf's root-to-leaf
// chain) in difference form: sum_q w_pq (m_p - m_q) for channels [c0, c0 + CC) of the row's
// element p. One warp per item; the leaf's ns rows (3 to 8) each take G = 32 / ns lanes
// (lane = r G + j), lane j of a row taking every G-th column, so that small leaves keep the
// warp busy. The weights w_pq were evaluated once per set-up (hm_weights_kernel) and are
// applied to the CC channels. m_p - m_q is formed exactly from the float pairs (their hi
// parts share a grid), each product w (m_p - m_q) is split exactly too, and the terms are
// summed as float pairs: the high parts by error-free additions (two_sum), whose errors gather
// with the low parts in a second float. (Kahan summation would leave an error of eps times
// each lane's partial sum, a first-order quantity.) The G partial sums of a row are then added
// in lane order as float pairs (through shared memory). The columns of an item pass through
// shared memory in tiles of 32 (channel values and the weights of the tile, copied by cp.async
// while the previous tile is being used). For a smooth input the terms are first-order
// quantities that cancel to a second-order result, and the output stage (M^T, a discrete
// divergence) cancels once more, so plain FP32 sums of H~a m and H~(a m) would lose about
// four digits.
template <int KIND, int CC, bool PLAIN>
__global__ void __launch_bounds__(128, 5) hm_rows_kernel(HDev d, int c0) {
  static_assert(CC <= 12 && CC % 2 == 0, "at most twelve channels per pass");
  using WT = NearW<KIND>;
  constexpr int kChunkW = 16 / (int)sizeof(WT);   // weights per 16-byte copy
  constexpr int kChunksRow = 32 / kChunkW;         // copies per 32-column weight row
  // per warp: two tiles (double buffer filled by cp.async); the lane-sum table of the end
  // reuses the warp's tiles
  __shared__ RowsTile<KIND, CC> tiles[4][2];
  static_assert(sizeof(tiles[0]) >= 32 * CC * sizeof(float2), "reduction table fits a warp's tiles");
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= d.n_items) return;
  const uint4 it = d.items[w];  // leaf ordinal, flat column range [y, z), weight base
  const uint32_t leaf = d.leaves[it.x];
  const uint32_t s0 = d.start[leaf], ns = d.end[leaf] - s0;
  const int G = 32 / (int)ns;
  const int r = lane / G, j = lane - r * G;
  const bool act = (uint32_t)r < ns;
  const uint32_t p = s0 + (act ? r : 0);
  const int C = d.C;
  // channel pairs c2: hi parts mh, lo parts ml of the row, sums (ks, kc)
  f32x2 mh[CC / 2], ml[CC / 2], ks[CC / 2], kc[CC / 2];
  {
    const ulonglong2 *mp = reinterpret_cast<const ulonglong2 *>(d.m + (size_t)p * C + c0);
#pragma unroll
    for (int c2 = 0; c2 < CC / 2; ++c2) {
      const ulonglong2 v = mp[c2];
      mh[c2] = v.x, ml[c2] = v.y, ks[c2] = 0ull, kc[c2] = 0ull;
    }
  }
  const uint32_t ncol = it.z - it.y, ntiles = (ncol + 31) / 32, npad = ntiles * 32;
  const WT *wg = reinterpret_cast<const WT *>(d.wts) + it.w;
  // lane l copies the channel values of column t0 + l and its share of the weight rows
  auto stage = [&](int buf, uint32_t t0) {
    RowsTile<KIND, CC> &tl = tiles[wib][buf];
    if ((uint32_t)lane < ncol - t0) {
      const uint32_t q = d.colidx[it.y + t0 + lane];
      const float4 *mq = reinterpret_cast<const float4 *>(d.m + (size_t)q * C + c0);
#pragma unroll
      for (int c2 = 0; c2 < CC / 2; ++c2) cp_async16(&tl.m[c2][lane], mq + c2);
    }
#pragma unroll
    for (int i = 0; i < 8 * kChunksRow / 32; ++i) {
      const int id = lane + 32 * i, row = id / kChunksRow, ch = id - row * kChunksRow;
      if ((uint32_t)row < ns) cp_async16(&tl.w[row][ch * kChunkW], wg + (size_t)row * npad + t0 + ch * kChunkW);
    }
    cp_async_commit();
  };
  if (ntiles > 0) stage(0, 0);
  for (uint32_t ti = 0; ti < ntiles; ++ti) {
    const int buf = ti & 1;
    if (ti + 1 < ntiles) {
      stage(buf ^ 1, (ti + 1) * 32);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncwarp();
    const uint32_t t0 = ti * 32, nt = min(32u, ncol - t0);
    const RowsTile<KIND, CC> &tl = tiles[wib][buf];
    // lane j of a row takes the item's columns j, j + G, ... (in order): here the local
    // indices k with (t0 + k) = j mod G
    if (act)
      for (uint32_t k = ((uint32_t)j + (uint32_t)G - t0 % (uint32_t)G) % (uint32_t)G; k < nt; k += G) {
        // packed weights of the channel pairs: (w0, w0), (w0, w1) (the pair of channels 8, 9),
        // (w1, w1), and their negatives
        f32x2 W[3];
        if constexpr (KIND == FACE) {
          const f32x2 ww = *reinterpret_cast<const f32x2 *>(&tl.w[r][k]);
          const float2 wf = f2_unpack(ww);
          W[0] = f2_pack(wf.x, wf.x), W[1] = ww, W[2] = f2_pack(wf.y, wf.y);
        } else {
          const float w0 = tl.w[r][k];
          W[0] = W[1] = W[2] = f2_pack(w0, w0);
        }
#pragma unroll
        for (int c2 = 0; c2 < CC / 2; ++c2) {
          const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(&tl.m[c2][k]);  // (hi pair, lo pair)
          const int wi = KIND == FACE ? (2 * c2 + 1 < 9 ? 0 : (2 * c2 >= 9 ? 2 : 1)) : 0;
          if constexpr (PLAIN) {
            // the inner operator: w (m_p - m_q) from the same exact differences, summed in plain
            // FP32 (no error-free transformations)
            const f32x2 t = f2_add(f2_sub(mh[c2], v.x), f2_sub(ml[c2], v.y));
            ks[c2] = f2_fma(W[wi], t, ks[c2]);
            continue;
          }
          const f32x2 w = W[wi], wn = W[wi] ^ kF2Sign;
          // w (m_p - m_q) = pr + pe + w dl up to eps^2 terms: dh = mh_p - mh_q is exact (the
          // hi parts share a grid), dl = ml_p - ml_q, w dh = pr + pe (FMA), so no rounding that
          // depends on the input reaches the sum above eps^2. npr = -pr (exact); the
          // error-free sum ks + pr = s + err: bb = s - ks, err = (ks - (s - bb)) + (pr - bb).
          const f32x2 dh = f2_sub(mh[c2], v.x);
          const f32x2 dl = f2_sub(ml[c2], v.y);
          const f32x2 npr = f2_mul(wn, dh);
          const f32x2 lo = f2_fma(w, dl, f2_fma(w, dh, npr));
          const f32x2 sn = f2_sub(ks[c2], npr);
          const f32x2 bb = f2_sub(sn, ks[c2]);
          const f32x2 err = f2_sub(f2_sub(ks[c2], f2_sub(sn, bb)), f2_add(npr, bb));
          ks[c2] = sn;
          kc[c2] = f2_add(kc[c2], f2_add(err, lo));
        }
      }
    __syncwarp();
  }
  // the G lanes of a row: partial sums (s, t) added in lane order as float pairs
  float2(*red)[CC] = reinterpret_cast<float2(*)[CC]>(&tiles[wib][0]);
#pragma unroll
  for (int c2 = 0; c2 < CC / 2; ++c2) {
    const float2 s2 = f2_unpack(ks[c2]), k2 = f2_unpack(kc[c2]);
    red[lane][2 * c2] = make_float2(s2.x, k2.x), red[lane][2 * c2 + 1] = make_float2(s2.y, k2.y);
  }
  __syncwarp();
  if (!act || j != 0) return;
  float2 *o = d.part + ((size_t)w * 8 + r) * C + c0;
#pragma unroll
  for (int c = 0; c < CC; ++c) {
    float h = red[lane][c].x, l = red[lane][c].y;
    for (int g = 1; g < G; ++g) pair_add(h, l, red[lane + g][c].x, red[lane + g][c].y);
    o[c] = make_float2(h, l);
  }
}

// Per (leaf, channel): the far sums along the leaf's chain (root to leaf), FP64, shared by the
// leaf's rows. With psi = a (CC = 2, ONES) the same sums give the far part of H~a per leaf.
template <int CC>
__global__ void hm_chain_sum_kernel(HDev d, const double *__restrict__ src, double *__restrict__ dst) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)d.n_leaves * CC) return;
  const int k = (int)(t / CC), c = (int)(t % CC);
  double s = 0.0;
  for (uint32_t ci = d.chain_off[k]; ci < d.chain_off[k + 1]; ++ci) s += src[(size_t)d.chain[ci] * CC + c];
  dst[t] = s;
}

// Per (row, channel): z = near + (m_p H~a_far - H~(a m)_far), the near sums of the leaf's
// items (in item order, as float pairs) plus the leaf's chain sums of the far field (FP64,
// hm_chain_sum_kernel). The far part of H~a was summed with the same operations from psi = a,
// so m = 1 gives z = 0 exactly.
template <int SEL, int CC>
__global__ void hm_epilogue_kernel(HDev d) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t row = t / CC;
  const int c = (int)(t - row * CC);
  const uint32_t k = (uint32_t)(row >> 3), r = (uint32_t)(row & 7);
  if (k >= (uint32_t)d.n_leaves) return;
  const uint32_t leaf = d.leaves[k];
  const uint32_t s0 = d.start[leaf];
  if (r >= d.end[leaf] - s0) return;
  const uint32_t p = s0 + r;
  float nh = 0.f, nl = 0.f;
  for (uint32_t i = d.item_off[k]; i < d.item_off[k + 1]; ++i) {
    const float2 v = d.part[((size_t)i * 8 + r) * CC + c];
    pair_add(nh, nl, v.x, v.y);
  }
  const double2 fa = d.leaf_farA[k];
  const float2 mv = m_get(d.m + (size_t)p * CC, c);
  const double far = ((double)mv.x + (double)mv.y) * (uses_k1<SEL>(c) ? fa.y : fa.x) - d.leafsum[(size_t)k * CC + c];
  const double zz = ((double)nh + (double)nl) + far;
  const float zh = (float)zz;
  d.z[(size_t)p * CC + c] = make_float2(zh, (float)(zz - (double)zh));
}

// ------------------------------------------------------------------ face prologue / epilogue

struct FaceOps {
  const uint32_t *faces;   // 3F original order
  const uint32_t *order;   // BVH position -> face
  const uint32_t *position;  // face -> BVH position
  // FP64 both: the gradient rows of a face sum to zero and the area-weighted rows around a
  // vertex sum to zero, and a smooth input leaves only what survives those cancellations
  const double *g;         // 9 per face (original order): g_c (df_coefficients, mod.rs:120-131)
  const double *area;      // per face
  const uint32_t *inc_off, *inc;  // vertex -> (face << 2 | corner), faces ascending
  int nv, nf;
};

// Channel values as float pairs on a common grid per channel: hi = k Q with Q = 2^(e - 22) for
// the channel's largest magnitude 2^e <= max < 2^(e+1), so |k| < 2^24 and the difference of two
// hi values is exact in FP32; lo = v - hi (|lo| <= Q / 2) rounded to FP32. The near field then
// forms m_p - m_q with two plain subtractions. Only the exponent of the largest magnitude
// matters: qmax holds, per channel, the largest high word (sign, exponent, leading mantissa
// bits) of |v| among the channel's values, shifted into the high half of a 64-bit word (the
// bit pattern of a non-negative double, ordered like the integers). Q is a power of two, so
// v / Q is the exact product v 2^(22 - e).
__device__ __forceinline__ double pow2(int k) {  // 2^k, from the bits when it is a normal number
  return (k >= -1022 && k <= 1023) ? __longlong_as_double((long long)(k + 1023) << 52) : ldexp(1.0, k);
}
__device__ __forceinline__ float2 split_q(double v, unsigned long long qbits) {
  const unsigned hw = (unsigned)(qbits >> 32);
  if (hw == 0u) return make_float2(0.f, 0.f);
  const int ef = (int)((hw >> 20) & 0x7ffu);
  const int e = ef ? ef - 1023 : ilogb(__longlong_as_double((long long)qbits));
  const double hi = rint(v * pow2(22 - e)) * pow2(e - 22);
  return make_float2((float)hi, (float)(v - hi));
}

// pass 0: the channels' largest magnitudes (a warp maximum of the high words, then one atomic
// per warp and channel; every lane of the warp takes part, `act` false contributing 0);
// pass 1: the split values
__device__ __forceinline__ void emit(float2 *mp, int c, double v, unsigned long long *qmax, int pass, bool act) {
  if (pass == 0) {
    unsigned a = act ? (unsigned)((unsigned long long)__double_as_longlong(fabs(v)) >> 32) : 0u;
    a = __reduce_max_sync(0xffffffffu, a);
    if ((threadIdx.x & 31) == 0 && a != 0u) atomicMax(qmax + c, (unsigned long long)a << 32);
  } else if (act) {
    m_set(mp, c, split_q(v, qmax[c]));
  }
}

// m per face in BVH order (FaceMetricTree::product, hierarchical.rs:711-746), in FP64 and
// stored as float pairs; vector q owns channels 12q + (3k + r) = sum_c x[3 t_c + k] g_c[r]
// (gradient) and 12q + 9 + k = (x_0 + x_1 + x_2)/3 for axis k (average; the division by 3 is
// a product with the rounded 1/3, within an FP64 unit of the quotient, far below the float
// pairs' resolution).
__global__ void face_m_kernel(FaceOps o, const double *__restrict__ xs, size_t ldx, int nb, int C,
                              float2 *m, unsigned long long *qmax, int pass) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = p < o.nf;  // the whole warp runs the loops (warp maxima in pass 0)
  const uint32_t f = act ? o.order[p] : 0;
  const uint32_t *t = o.faces + 3 * (size_t)f;
  const double *g = o.g + 9 * (size_t)f;
  float2 *mp = m + (size_t)(act ? p : 0) * C;
  for (int q = 0; q < nb; ++q) {
    const double *x = xs + q * ldx;
    for (int k = 0; k < 3; ++k) {
      const double x0 = x[3 * (size_t)t[0] + k], x1 = x[3 * (size_t)t[1] + k], x2 = x[3 * (size_t)t[2] + k];
      for (int r = 0; r < 3; ++r)
        emit(mp, 12 * q + 3 * k + r, x0 * g[r] + x1 * g[3 + r] + x2 * g[6 + r], qmax, pass, act);
      emit(mp, 12 * q + 9 + k, ((x0 + x1) + x2) * (1.0 / 3.0), qmax, pass, act);
    }
  }
  if (pass == 1 && act)
    for (int c = 12 * nb; c < C; ++c) m_set(mp, c, make_float2(0.f, 0.f));
}

// y_v = 2 sum_{S ni v} a_S (w_hi g_c . z_hi + w_lo z_lo / 3) in FP64 (hierarchical.rs:779-811).
__global__ void face_gather_kernel(FaceOps o, const float2 *__restrict__ z, int nb, int C,
                                   double w_hi, double w_lo, double *__restrict__ ys, size_t ldy) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= o.nv) return;
  for (int q = 0; q < nb; ++q) {
    double acc0 = 0.0, acc1 = 0.0, acc2 = 0.0;
    for (uint32_t e = o.inc_off[v]; e < o.inc_off[v + 1]; ++e) {
      uint32_t fc = o.inc[e], f = fc >> 2, c = fc & 3;
      double a = o.area[f];
      const double *g = o.g + 9 * (size_t)f + 3 * c;
      const float2 *zs = z + (size_t)o.position[f] * C + 12 * q;
      double acc[3];
      for (int k = 0; k < 3; ++k) {
        const float2 *zh = zs + 3 * k;
        double hi = g[0] * ((double)zh[0].x + zh[0].y) + g[1] * ((double)zh[1].x + zh[1].y) +
                    g[2] * ((double)zh[2].x + zh[2].y);
        double lo = (double)zs[9 + k].x + zs[9 + k].y;
        acc[k] = a * (w_hi * hi + w_lo * (1.0 / 3.0) * lo);
      }
      acc0 += acc[0], acc1 += acc[1], acc2 += acc[2];
    }
    double *y = ys + q * ldy + 3 * (size_t)v;
    y[0] = 2.0 * acc0, y[1] = 2.0 * acc1, y[2] = 2.0 * acc2;
  }
}

// ------------------------------------------------------------------ vertex prologue / epilogue

// psi channels of the vertex operator: m = x per axis (psi = a x in the upward sums), vector q
// at channels 4q + k (4q + 3 is padding).
__global__ void vertex_m_kernel(const uint32_t *order, const double *__restrict__ xs, size_t ldx,
                                int nv, int nb, int C, float2 *m, unsigned long long *qmax, int pass) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = p < nv;  // the whole warp runs the loops (warp maxima in pass 0)
  const uint32_t v = act ? order[p] : 0;
  float2 *mp = m + (size_t)(act ? p : 0) * C;
  if (pass == 1 && act)
    for (int c = 0; c < C; ++c) m_set(mp, c, make_float2(0.f, 0.f));
  for (int q = 0; q < nb; ++q)
    for (int k = 0; k < 3; ++k) emit(mp, 4 * q + k, xs[q * ldx + 3 * (size_t)v + k], qmax, pass, act);
}

// y = 2 a (H~a x - H~(a x)) = 2 a z (hierarchical.rs:1330-1343).
__global__ void vertex_out_kernel(const uint32_t *order, const float4 *el, const float2 *z, int nv,
                                  int nb, int C, double scale, double *__restrict__ ys, size_t ldy) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nv) return;
  uint32_t v = order[p];
  double a = el[p].w;
  for (int q = 0; q < nb; ++q)
    for (int k = 0; k < 3; ++k) {
      const float2 zz = z[(size_t)p * C + 4 * q + k];
      ys[q * ldy + 3 * (size_t)v + k] = scale * 2.0 * a * ((double)zz.x + zz.y);
    }
}

// Element records: positions as float pairs (hi + lo), weights, normals; FP64 in.
__global__ void hm_pack_kernel(const double *pts, const double *wt, const double *nrm64,
                               const uint32_t *order, int n, float4 *xh, float4 *xl, float4 *nrm) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  uint32_t e = order[p];
  const double *x = pts + 3 * (size_t)e;
  float h0 = (float)x[0], h1 = (float)x[1], h2 = (float)x[2];
  xh[p] = make_float4(h0, h1, h2, (float)wt[e]);
  xl[p] = make_float4((float)(x[0] - (double)h0), (float)(x[1] - (double)h1), (float)(x[2] - (double)h2), 0.f);
  if (nrm) nrm[p] = make_float4((float)nrm64[3 * (size_t)e], (float)nrm64[3 * (size_t)e + 1],
                                (float)nrm64[3 * (size_t)e + 2], 0.f);
}

// ---- the near columns and work items of every leaf, built on the device from the block lists

// per leaf k: the length of its root-to-leaf chain, the near columns of the chain's blocks and
// the number of work items (at most item_cols columns each, at least one)
__global__ void near_count_kernel(uint32_t nl, const uint32_t *__restrict__ leaves, const uint32_t *__restrict__ parent,
                                  const uint32_t *__restrict__ start, const uint32_t *__restrict__ end,
                                  const uint32_t *__restrict__ near_ptr, const uint32_t *__restrict__ near_col,
                                  uint32_t item_cols, uint32_t *depth, unsigned long long *cols, uint32_t *nitems) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nl) return;
  uint32_t dep = 1;
  unsigned long long c = 0;
  for (uint32_t a = leaves[k];; a = parent[a]) {
    for (uint32_t q = near_ptr[a]; q < near_ptr[a + 1]; ++q) {
      const uint32_t b = near_col[q];
      c += end[b] - start[b];
    }
    if (a == 0) break;
    ++dep;
  }
  depth[k] = dep, cols[k] = c;
  nitems[k] = (uint32_t)max(1ull, (c + item_cols - 1) / item_cols);
}

// per leaf k at its scanned offsets: the chain (root first), the near columns in chain, block and
// element order, and the work items (leaf, column range [y, z), weight base filled later)
__global__ void near_fill_kernel(uint32_t nl, const uint32_t *__restrict__ leaves, const uint32_t *__restrict__ parent,
                                 const uint32_t *__restrict__ start, const uint32_t *__restrict__ end,
                                 const uint32_t *__restrict__ near_ptr, const uint32_t *__restrict__ near_col,
                                 uint32_t item_cols, const uint32_t *__restrict__ coff,
                                 const unsigned long long *__restrict__ ncol, const uint32_t *__restrict__ ioff,
                                 uint32_t *chain, uint32_t *cols, uint4 *items) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nl) return;
  const uint32_t depth = coff[k + 1] - coff[k];
  uint32_t *ch = chain + coff[k];
  uint32_t a = leaves[k];
  for (uint32_t i = depth; i-- > 0; a = parent[a]) ch[i] = a;
  uint32_t x = (uint32_t)ncol[k];
  for (uint32_t i = 0; i < depth; ++i) {
    const uint32_t n = ch[i];
    for (uint32_t q = near_ptr[n]; q < near_ptr[n + 1]; ++q) {
      const uint32_t b = near_col[q];
      for (uint32_t e = start[b]; e < end[b]; ++e) cols[x++] = e;
    }
  }
  const uint32_t c_end = (uint32_t)ncol[k + 1];
  uint32_t y0 = (uint32_t)ncol[k];
  for (uint32_t it = ioff[k]; it < ioff[k + 1]; ++it) {
    const uint32_t y1 = min(c_end, y0 + item_cols);
    items[it] = make_uint4(k, y0, y1, 0u);
    y0 = y1;
  }
}

// the weight count of every work item: its rows times its columns padded to 32
__global__ void item_weights_kernel(uint32_t n_items, const uint4 *__restrict__ items, const uint32_t *__restrict__ leaves,
                                    const uint32_t *__restrict__ start, const uint32_t *__restrict__ end,
                                    unsigned long long *w) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_items) return;
  const uint4 it = items[i];
  const uint32_t leaf = leaves[it.x];
  w[i] = (unsigned long long)(end[leaf] - start[leaf]) * ((it.z - it.y + 31) & ~31u);
}
__global__ void item_base_kernel(uint32_t n_items, const unsigned long long *__restrict__ base, uint4 *items) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_items) items[i].w = (uint32_t)base[i];
}

// far work items: node a's far blocks cut into runs of at most kFarChunk
__global__ void far_count_kernel(uint32_t nn, const uint32_t *__restrict__ far_ptr, uint32_t *cnt) {
  const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a < nn) cnt[a] = (far_ptr[a + 1] - far_ptr[a] + kFarChunk - 1) / kFarChunk;
}
__global__ void far_fill_kernel(uint32_t nn, const uint32_t *__restrict__ far_ptr, const uint32_t *__restrict__ off,
                                uint4 *items) {
  const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nn) return;
  const uint32_t q1 = far_ptr[a + 1];
  uint32_t j = off[a];
  for (uint32_t q0 = far_ptr[a]; q0 < q1; q0 += kFarChunk) items[j++] = make_uint4(a, q0, min(q0 + kFarChunk, q1), 0u);
}

// m = 1 in both channels of the paired layout: hi parts (1, 1), lo parts (0, 0)
__global__ void ones_kernel(size_t n_el, float2 *m) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n_el) m[2 * i] = make_float2(1.f, 1.f), m[2 * i + 1] = make_float2(0.f, 0.f);
}

}  // namespace rsg

// ====================================================================== host side

using namespace rsg;

namespace {

inline unsigned nblk(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

template <class T>
void up_vec(DevBuf<T> &b, const std::vector<T> &v, cudaStream_t s) {
  b.alloc(std::max<size_t>(v.size(), 1));
  if (!v.empty()) b.upload(v.data(), v.size(), s);
}

// The block cluster tree on the device with its per-step data (both operators).
struct HMat {
  rs_ctx *ctx = nullptr;
  int kind = FACE;
  Tree tree;
  Blocks blocks;
  size_t n_el = 0, n_items = 0;
  double neg_s = 0;
  DevBuf<uint32_t> start, end, right, parent, leaves, chain_off, chain, item_off;
  DevBuf<uint32_t> count, far_item_off;
  DevBuf<uint4> far_items;
  size_t n_far_items = 0;
  DevBuf<float2> fpart;
  DevBuf<uint32_t> colidx;
  DevBuf<uint4> items;
  DevBuf<unsigned char> wts;  // near weights (NearW per entry), see hm_weights_kernel
  size_t n_wts = 0;
  DevBuf<float4> far_coef;
  DevBuf<double2> leaf_farA;
  DevBuf<double> leafsum;
  DevBuf<float4> xh, xl, nrm;
  DevBuf<double> up, farx;
  DevBuf<float2> up2;
  DevBuf<float2> part, m, z;
  DevBuf<unsigned long long> qmax;  // per channel: largest |m| (see split_q)
  int pw_mode = 0, pw_k = 0;
  bool plain_rows = false;  // the near field of the next product in plain FP32 sums (inner operator)
  Profiler prof;
  double setup_times[3] = {0, 0, 0};  // seconds: work items, far coefficients, device part

  HDev dev(int C_) const {
    HDev d;
    d.start = start.p, d.end = end.p, d.right = right.p, d.parent = parent.p, d.leaves = leaves.p;
    d.chain_off = chain_off.p, d.chain = chain.p;
    d.far_ptr = blocks.far_ptr.p, d.far_col = blocks.far_col.p, d.far_coef = far_coef.p;
    d.far_items = far_items.p, d.far_item_off = far_item_off.p, d.fpart = fpart.p;
    d.n_far_items = (int)n_far_items;
    d.xh = xh.p, d.xl = xl.p, d.nrm = nrm.p, d.leaf_farA = leaf_farA.p;
    d.colidx = colidx.p, d.items = items.p, d.item_off = item_off.p, d.wts = wts.p;
    d.up = up.p, d.up2 = up2.p, d.farx = farx.p, d.part = part.p, d.count = count.p, d.leafsum = leafsum.p;
    d.m = m.p, d.z = z.p;
    d.n_nodes = (int)tree.n_nodes(), d.n_leaves = (int)tree.leaves.size(), d.n_el = (int)n_el;
    d.n_items = (int)n_items;
    d.C = C_;
    d.neg_s = (float)neg_s;
    d.pw_mode = pw_mode, d.pw_k = pw_k;
    return d;
  }
  cudaStream_t st() const { return ctx->stream; }

  // Channel scratch for C channels.
  void reserve(int C_) {
    size_t nn = tree.n_nodes();
    if ((size_t)C_ * nn > up.n) up.alloc((size_t)C_ * nn), up2.alloc((size_t)C_ * nn), farx.alloc((size_t)C_ * nn);
    if ((size_t)C_ * n_far_items > fpart.n) fpart.alloc(std::max<size_t>((size_t)C_ * n_far_items, 1));
    if ((size_t)C_ * tree.leaves.size() > leafsum.n) leafsum.alloc((size_t)C_ * tree.leaves.size());
    if ((size_t)C_ * n_el > m.n) m.alloc((size_t)C_ * n_el), z.alloc((size_t)C_ * n_el);
    if (n_items * 8 * (size_t)C_ > part.n) part.alloc(std::max<size_t>(n_items * 8 * (size_t)C_, 1));
  }

  // The exponent r2^e as an integer power times a cube or square root when 3e or 2e is an
  // integer (integer alpha, beta), else powf.
  void set_exponent(double e) {
    neg_s = e;
    pw_mode = 0, pw_k = 0;
    for (int q : {1, 2, 3}) {
      double k = e * q;
      if (std::fabs(k - std::round(k)) < 1e-12 && std::fabs(k) <= 64) {
        pw_mode = q == 1 ? 3 : q, pw_k = (int)std::round(k) * (q == 1 ? 3 : 1);
        break;
      }
    }
  }

  template <int SEL, int CC>
  void upward_far(const HDev &d) {
    size_t nn = tree.n_nodes(), nl = tree.leaves.size();
    cudaStream_t s = st();
    prof.begin(s, kind == FACE ? "metric_upward" : "vfrac_upward");
    hm_upward_kernel<CC><<<nblk(nl * 32, 128), 128, 0, s>>>(d);
    RSG_LAUNCHED(ctx, "hm_upward");
    prof.end(s);
    prof.begin(s, kind == FACE ? "metric_far" : "vfrac_far");
    if (n_far_items > 0) {  // chi = 0 (all near) has none
      hm_far_kernel<SEL, CC><<<nblk(n_far_items * (CC < 12 ? 1 : CC / 12) * 32, 256), 256, 0, s>>>(d);
      RSG_LAUNCHED(ctx, "hm_far");
    }
    hm_far_final_kernel<CC><<<nblk(nn * CC, 256), 256, 0, s>>>(d);
    RSG_LAUNCHED(ctx, "hm_far_final");
    if (SEL != ONES) {
      hm_chain_sum_kernel<CC><<<nblk(nl * CC, 256), 256, 0, s>>>(d, d.farx, d.leafsum);
      RSG_LAUNCHED(ctx, "hm_chain_sum");
    }
    prof.end(s);
  }

  // Uploads the tree, the near column ranges split into work items, the element records and
  // the far coefficients; computes the far part of H~a. pts/wt/nrm64 are per element
  // (original order), FP64.
  void setup(const double *pts, const double *wt, const double *nrm64, const double *proj6) {
    using clk = std::chrono::steady_clock;
    auto t_ph = clk::now();
    auto lap = [&](double &slot) {
      const auto now = clk::now();
      slot = std::chrono::duration<double>(now - t_ph).count();
      t_ph = now;
    };
    cudaStream_t s = st();
    const Tree &T = tree;
    size_t nn = T.n_nodes(), nl = T.leaves.size();
    std::vector<uint32_t> parent_h(nn, 0);
    const uint32_t kItemCols = 512;
    for (size_t i = 0; i < nn; ++i)
      if (T.right[i]) parent_h[i + 1] = (uint32_t)i, parent_h[T.right[i]] = (uint32_t)i;
    for (size_t k = 0; k < nl; ++k)
      if (T.end[T.leaves[k]] - T.start[T.leaves[k]] > 8)
        fail(RS_INVALID_OPTION, "InvalidOption", "upload", "the GPU path needs leaf_size <= 8");
    up_vec(start, T.start, s), up_vec(end, T.end, s), up_vec(right, T.right, s);
    up_vec(parent, parent_h, s), up_vec(leaves, T.leaves, s);
    // per leaf: its root-to-leaf chain and the near columns of the chain (chain order, block
    // order, element order), flattened and cut into items of at most kItemCols columns: counts,
    // exclusive scans (one extra zero entry gives the totals), then the fill at the offsets
    DevBuf<unsigned char> tmp;
    auto scan = [&](auto *in, auto *out, size_t m) {
      size_t bytes = 0;
      RSG_CUDA("upload", cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, (int)m, s));
      if (bytes > tmp.n) tmp.alloc(bytes);
      RSG_CUDA("upload", cub::DeviceScan::ExclusiveSum(tmp.p, bytes, in, out, (int)m, s));
    };
    {
      DevBuf<uint32_t> dep(nl + 1), nit(nl + 1);
      DevBuf<unsigned long long> cnt(nl + 1), ncol(nl + 1);
      RSG_CUDA("upload", cudaMemsetAsync(dep.p + nl, 0, sizeof(uint32_t), s));
      RSG_CUDA("upload", cudaMemsetAsync(nit.p + nl, 0, sizeof(uint32_t), s));
      RSG_CUDA("upload", cudaMemsetAsync(cnt.p + nl, 0, sizeof(unsigned long long), s));
      near_count_kernel<<<nblk(nl, 128), 128, 0, s>>>((uint32_t)nl, leaves.p, parent.p, start.p, end.p,
                                                      blocks.near_ptr.p, blocks.near_col.p, kItemCols, dep.p, cnt.p,
                                                      nit.p);
      RSG_LAUNCHED(ctx, "hm_near_count");
      chain_off.alloc(nl + 1), item_off.alloc(nl + 1);
      scan(dep.p, chain_off.p, nl + 1), scan(cnt.p, ncol.p, nl + 1), scan(nit.p, item_off.p, nl + 1);
      uint32_t n_chain = 0, n_it = 0;
      unsigned long long n_col = 0;
      RSG_CUDA("upload", copy_async(&n_chain, chain_off.p + nl, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
      RSG_CUDA("upload", copy_async(&n_col, ncol.p + nl, sizeof(n_col), cudaMemcpyDeviceToHost, s));
      RSG_CUDA("upload", copy_async(&n_it, item_off.p + nl, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
      RSG_CUDA("upload", cudaStreamSynchronize(s));
      if (n_col > UINT32_MAX) fail(RS_INVALID_OPTION, "InvalidOption", "upload", "near field too large");
      chain.alloc(std::max<uint32_t>(n_chain, 1)), colidx.alloc(std::max<size_t>(n_col, 1)), items.alloc(n_it);
      near_fill_kernel<<<nblk(nl, 128), 128, 0, s>>>((uint32_t)nl, leaves.p, parent.p, start.p, end.p,
                                                     blocks.near_ptr.p, blocks.near_col.p, kItemCols, chain_off.p,
                                                     ncol.p, item_off.p, chain.p, colidx.p, items.p);
      RSG_LAUNCHED(ctx, "hm_near_fill");
      n_items = n_it;
    }
    lap(setup_times[0]);
    // weight base of every item: its rows times its columns padded to 32
    {
      DevBuf<unsigned long long> w(n_items + 1), base(n_items + 1);
      RSG_CUDA("upload", cudaMemsetAsync(w.p + n_items, 0, sizeof(unsigned long long), s));
      item_weights_kernel<<<nblk(n_items, 256), 256, 0, s>>>((uint32_t)n_items, items.p, leaves.p, start.p, end.p,
                                                              w.p);
      RSG_LAUNCHED(ctx, "hm_item_weights");
      scan(w.p, base.p, n_items + 1);
      unsigned long long tot = 0;
      RSG_CUDA("upload", copy_async(&tot, base.p + n_items, sizeof(tot), cudaMemcpyDeviceToHost, s));
      RSG_CUDA("upload", cudaStreamSynchronize(s));
      if (tot > UINT32_MAX) fail(RS_INVALID_OPTION, "InvalidOption", "upload", "near field too large");
      n_wts = tot;
      item_base_kernel<<<nblk(n_items, 256), 256, 0, s>>>((uint32_t)n_items, base.p, items.p);
      RSG_LAUNCHED(ctx, "hm_item_weights");
    }
    // far work items
    {
      DevBuf<uint32_t> cnt(nn + 1);
      RSG_CUDA("upload", cudaMemsetAsync(cnt.p + nn, 0, sizeof(uint32_t), s));
      far_count_kernel<<<nblk(nn, 256), 256, 0, s>>>((uint32_t)nn, blocks.far_ptr.p, cnt.p);
      RSG_LAUNCHED(ctx, "hm_far_items");
      far_item_off.alloc(nn + 1);
      scan(cnt.p, far_item_off.p, nn + 1);
      uint32_t nfi = 0;
      RSG_CUDA("upload", copy_async(&nfi, far_item_off.p + nn, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
      RSG_CUDA("upload", cudaStreamSynchronize(s));
      n_far_items = nfi;
      far_items.alloc(std::max<size_t>(n_far_items, 1));
      far_fill_kernel<<<nblk(nn, 256), 256, 0, s>>>((uint32_t)nn, blocks.far_ptr.p, far_item_off.p, far_items.p);
      RSG_LAUNCHED(ctx, "hm_far_items");
    }
    count.alloc(nn);
    RSG_CUDA("upload", cudaMemsetAsync(count.p, 0, nn * sizeof(uint32_t), s));
    // far coefficients (kernel.far, hierarchical.rs:210-220 / 980-984) in FP64 on the device
    // from the node centroids (and, for faces, the node projectors)
    {
      DevBuf<double> cen, pj;
      cen.upload(T.centroid.data(), 3 * nn, s);
      if (kind == FACE) pj.upload(proj6, 6 * nn, s);
      far_coef.alloc(std::max<size_t>(blocks.n_far, 1));
      if (n_far_items > 0) {
        hm_far_coef_kernel<<<nblk(n_far_items * 32, 256), 256, 0, s>>>(
            far_items.p, (int)n_far_items, blocks.far_col.p, cen.p, kind == FACE ? pj.p : nullptr, neg_s, far_coef.p);
        RSG_LAUNCHED(ctx, "hm_far_coef");
      }
      RSG_CUDA("upload", cudaStreamSynchronize(s));  // before the staging buffers go
    }
    lap(setup_times[1]);
    // element records
    DevBuf<double> dp, dw, dn;
    dp.upload(pts, 3 * n_el, s);
    dw.upload(wt, n_el, s);
    if (nrm64) dn.upload(nrm64, 3 * n_el, s);
    DevBuf<uint32_t> ord;
    ord.upload(T.order.data(), T.order.size(), s);
    xh.alloc(n_el), xl.alloc(n_el);
    if (kind == FACE) nrm.alloc(n_el);
    hm_pack_kernel<<<nblk(n_el, 256), 256, 0, s>>>(dp.p, dw.p, nrm64 ? dn.p : nullptr, ord.p, (int)n_el,
                                                   xh.p, xl.p, kind == FACE ? nrm.p : nullptr);
    RSG_LAUNCHED(ctx, "hm_pack");
    // near weights of every work item, evaluated once; the product passes read them
    wts.alloc(std::max<size_t>(n_wts * (kind == FACE ? sizeof(float2) : sizeof(float)), 16));
    {
      const HDev dw0 = dev(0);
      const unsigned g = nblk(n_items * 8 * 32, 256);
      if (kind == FACE) hm_weights_kernel<FACE><<<g, 256, 0, s>>>(dw0, n_wts);
      else hm_weights_kernel<VERTEX><<<g, 256, 0, s>>>(dw0, n_wts);
      RSG_LAUNCHED(ctx, "hm_weights");
    }
    // far part of H~a: upward over psi = a (m = 1, 2 channels) and far sums per node
    reserve(4);
    // m = 1 in both channels: hi parts (1, 1), lo parts (0, 0) in the paired layout
    DevBuf<float2> mm(2 * n_el);
    ones_kernel<<<nblk(n_el, 256), 256, 0, s>>>(n_el, mm.p);
    RSG_LAUNCHED(ctx, "hm_ones");
    HDev d = dev(2);
    d.m = mm.p;
    upward_far<ONES, 2>(d);
    leaf_farA.alloc(std::max<size_t>(nl, 1));
    hm_chain_sum_kernel<2><<<nblk(nl * 2, 256), 256, 0, s>>>(d, farx.p, reinterpret_cast<double *>(leaf_farA.p));
    RSG_LAUNCHED(ctx, "hm_chain_sum");
    RSG_CUDA("upload", cudaStreamSynchronize(s));
    lap(setup_times[2]);
  }

  // z for the C-channel m already in `m` (faces: C = 12 nb, vertices: C = 4 nb).
  template <int K, int CC>
  void product_cc(int nb) {
    cudaStream_t s = st();
    HDev d = dev(CC);
    constexpr int SEL = K == FACE ? FACE_CH : VERTEX_CH;
    upward_far<SEL, CC>(d);
    prof.begin(s, K == FACE ? "metric_rows" : "vfrac_rows");
    if constexpr (K == FACE) {
      for (int q = 0; q < nb; ++q) {  // one vector (12 channels) per pass
        if (plain_rows) hm_rows_kernel<K, 12, true><<<nblk(n_items * 32, 128), 128, 0, s>>>(d, 12 * q);
        else hm_rows_kernel<K, 12, false><<<nblk(n_items * 32, 128), 128, 0, s>>>(d, 12 * q);
        RSG_LAUNCHED(ctx, "hm_rows");
      }
    } else {
      if (plain_rows) hm_rows_kernel<K, CC, true><<<nblk(n_items * 32, 128), 128, 0, s>>>(d, 0);
      else hm_rows_kernel<K, CC, false><<<nblk(n_items * 32, 128), 128, 0, s>>>(d, 0);
      RSG_LAUNCHED(ctx, "hm_rows");
    }
    prof.end(s);
    prof.begin(s, K == FACE ? "metric_epilogue" : "vfrac_epilogue");
    epilogue<SEL, CC>(d);
    prof.end(s);
  }

  // z from the near partial sums and the far chain sums (one thread per row and channel)
  template <int SEL, int CC>
  void epilogue(const HDev &d) {
    hm_epilogue_kernel<SEL, CC><<<nblk(tree.leaves.size() * 8 * CC, 256), 256, 0, st()>>>(d);
    RSG_LAUNCHED(ctx, "hm_epilogue");
  }

  void product(int nb) {
    if (kind == FACE) {
      if (nb == 1) product_cc<FACE, 12>(1);
      else if (nb == 2) product_cc<FACE, 24>(2);
      else if (nb == 3) product_cc<FACE, 36>(3);
      else fail(RS_INTERNAL, "Internal", "product", "unsupported channel count");
    } else {
      if (nb == 1) product_cc<VERTEX, 4>(1);
      else if (nb == 2) product_cc<VERTEX, 8>(2);
      else if (nb == 3) product_cc<VERTEX, 12>(3);
      else fail(RS_INTERNAL, "Internal", "product", "unsupported channel count");
    }
  }

  void build_common(rs_ctx *c, Tree &&t, double chi, int leaf_pairs) {
    ctx = c;
    tree = std::move(t);
    if (!(std::isfinite(chi) && chi >= 0.0))
      fail(RS_INVALID_OPTION, "InvalidOption", "upload", "chi must be a finite number >= 0");
    if (leaf_pairs < 0) fail(RS_INVALID_OPTION, "InvalidOption", "upload", "leaf_pairs must be >= 0");
    blocks = classify_blocks_device(tree, chi, (size_t)leaf_pairs);
  }
};

void check_exponents(double alpha, double beta) {
  if (!std::isfinite(alpha) || !std::isfinite(beta) || alpha <= 1.0 || beta <= alpha + 2.0 ||
      beta >= 2.0 * alpha + 2.0)
    fail(RS_INVALID_EXPONENTS, "InvalidExponents", "metric",
         "exponents must satisfy alpha > 1 and alpha + 2 < beta < 2 alpha + 2");
}

}  // namespace

struct rs_metric {
  HMat h;
  int nv = 0, nf = 0;
  // build phases in seconds: geometry, tree, projectors, blocks, face records, work items,
  // far coefficients, device part (uploads, element records, weights, far part of H~a)
  double build_times[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  FaceGeom geom;
  DevBuf<uint32_t> faces, order, position, inc_off, inc;
  DevBuf<double> g, area;
  DevBuf<double> xbuf, ybuf;
  FaceOps ops() const {
    FaceOps o;
    o.faces = faces.p, o.order = order.p, o.position = position.p, o.g = g.p, o.area = area.p;
    o.inc_off = inc_off.p, o.inc = inc.p, o.nv = nv, o.nf = nf;
    return o;
  }
};

struct rs_vfrac {
  HMat h;
  int nv = 0;
  DevBuf<uint32_t> order;
  DevBuf<double> xbuf, ybuf;
};

namespace {

// FaceMetricTree::from_parts / build (hierarchical.rs:302-363): df coefficients, projectors,
// blocks, element records.
void metric_setup(rs_metric *M, rs_ctx *ctx, int nv, int nf, const uint32_t *faces,
                  const double *pos, double alpha, double beta, double chi, int leaf_size,
                  int leaf_pairs) {
  check_exponents(alpha, beta);
  validate_topology(nv, nf, faces);
  validate_positions(nv, nf, faces, pos);
  ctx->use();
  using clk = std::chrono::steady_clock;
  auto t_ph = clk::now();
  auto lap = [&](int slot) {
    const auto now = clk::now();
    M->build_times[slot] = std::chrono::duration<double>(now - t_ph).count();
    t_ph = now;
  };
  M->nv = nv, M->nf = nf;
  const SharedFaceTree *sh = shared_face_tree(faces, pos, nf, leaf_size);
  M->geom = sh ? sh->geom : face_geometry(nf, faces, pos);
  lap(0);
  Tree T = sh ? sh->tree : build_face_tree(nf, faces, pos, M->geom, leaf_size);
  lap(1);
  M->h.kind = FACE;
  M->h.n_el = nf;
  M->h.set_exponent(-(beta - 2.0) / alpha);
  // projectors P = sum a N N^T / A per node (RS/src/spatial/mod.rs:268-290), bottom-up
  size_t nn = T.n_nodes();
  std::vector<double> ps(7 * nn, 0.0), proj(6 * nn);
  for (size_t i = nn; i-- > 0;) {
    double *o = &ps[7 * i];
    if (T.right[i] == 0) {
      for (uint32_t p = T.start[i]; p < T.end[i]; ++p) {
        uint32_t f = T.order[p];
        double a = M->geom.area[f];
        const double *n = &M->geom.normal[3 * (size_t)f];
        o[0] += a, o[1] += a * n[0] * n[0], o[2] += a * n[0] * n[1], o[3] += a * n[0] * n[2];
        o[4] += a * n[1] * n[1], o[5] += a * n[1] * n[2], o[6] += a * n[2] * n[2];
      }
    } else {
      for (int k = 0; k < 7; ++k) o[k] = ps[7 * (i + 1) + k] + ps[7 * (size_t)T.right[i] + k];
    }
    for (int k = 0; k < 6; ++k) proj[6 * i + k] = o[k + 1] / o[0];
  }
  lap(2);
  M->h.build_common(ctx, std::move(T), chi, leaf_pairs);
  lap(3);
  cudaStream_t s = M->h.st();
  // df coefficients (RS/src/metric/mod.rs:120-131) in FP64
  std::vector<double> gh(9 * (size_t)nf), ah(nf);
  for (int f = 0; f < nf; ++f) {
    const double *p0 = pos + 3 * (size_t)faces[3 * f], *p1 = pos + 3 * (size_t)faces[3 * f + 1],
                 *p2 = pos + 3 * (size_t)faces[3 * f + 2];
    double u[3], w[3], n[3];
    for (int k = 0; k < 3; ++k) u[k] = p1[k] - p0[k], w[k] = p2[k] - p0[k];
    n[0] = u[1] * w[2] - u[2] * w[1], n[1] = u[2] * w[0] - u[0] * w[2], n[2] = u[0] * w[1] - u[1] * w[0];
    double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    double sc = 1.0 / (len * len);
    double ww[3] = {n[0] * sc, n[1] * sc, n[2] * sc};
    const double *pa[3] = {p1, p2, p0}, *pb[3] = {p2, p0, p1};
    for (int c = 0; c < 3; ++c) {
      double e[3] = {pb[c][0] - pa[c][0], pb[c][1] - pa[c][1], pb[c][2] - pa[c][2]};
      gh[9 * f + 3 * c + 0] = ww[1] * e[2] - ww[2] * e[1];
      gh[9 * f + 3 * c + 1] = ww[2] * e[0] - ww[0] * e[2];
      gh[9 * f + 3 * c + 2] = ww[0] * e[1] - ww[1] * e[0];
    }
    ah[f] = M->geom.area[f];
  }
  std::vector<uint32_t> fh(faces, faces + 3 * (size_t)nf), posn(nf);
  for (int p = 0; p < nf; ++p) posn[M->h.tree.order[p]] = (uint32_t)p;
  std::vector<uint32_t> ioff((size_t)nv + 1, 0), inc(3 * (size_t)nf);
  for (int f = 0; f < nf; ++f)
    for (int c = 0; c < 3; ++c) ioff[faces[3 * f + c] + 1]++;
  for (int v = 0; v < nv; ++v) ioff[v + 1] += ioff[v];
  {
    std::vector<uint32_t> fill(ioff.begin(), ioff.end() - 1);
    for (int f = 0; f < nf; ++f)
      for (int c = 0; c < 3; ++c) inc[fill[faces[3 * f + c]]++] = ((uint32_t)f << 2) | c;
  }
  up_vec(M->faces, fh, s), up_vec(M->order, M->h.tree.order, s), up_vec(M->position, posn, s);
  up_vec(M->g, gh, s), up_vec(M->area, ah, s), up_vec(M->inc_off, ioff, s), up_vec(M->inc, inc, s);
  lap(4);
  M->h.setup(M->geom.bary.data(), M->geom.area.data(), M->geom.normal.data(), proj.data());
  for (int i = 0; i < 3; ++i) M->build_times[5 + i] = M->h.setup_times[i];
}

}  // namespace

// FaceMetricTree::apply_batch (hierarchical.rs:540-622) on device vectors with leading
// dimensions ldx, ldy (>= 3V): groups of <= 3 vectors per tree pass.
void rsg::metric_apply_strided(rs_metric *M, double w_hi, double w_lo, int nb, const double *xs,
                               size_t ldx, double *ys, size_t ldy, bool plain) {
  if (!(std::isfinite(w_hi) && std::isfinite(w_lo)))
    fail(RS_INVALID_OPTION, "InvalidOption", "product", "finite weights");
  cudaStream_t s = M->h.st();
  M->h.plain_rows = plain;
  for (int q0 = 0; q0 < nb; q0 += 3) {
    int k = std::min(3, nb - q0);
    int CC = 12 * k;
    M->h.reserve(CC);
    M->h.prof.begin(s, "metric_m");
    if (M->h.qmax.n < 64) M->h.qmax.alloc(64);
    RSG_CUDA("product", cudaMemsetAsync(M->h.qmax.p, 0, CC * sizeof(unsigned long long), s));
    for (int pass = 0; pass < 2; ++pass) {
      face_m_kernel<<<nblk(M->nf, 256), 256, 0, s>>>(M->ops(), xs + q0 * ldx, ldx, k, CC, M->h.m.p, M->h.qmax.p, pass);
      RSG_LAUNCHED(M->h.ctx, "face_m");
    }
    M->h.prof.end(s);
    M->h.product(k);
    M->h.prof.begin(s, "metric_gather");
    face_gather_kernel<<<nblk(M->nv, 128), 128, 0, s>>>(M->ops(), M->h.z.p, k, CC, w_hi, w_lo,
                                                        ys + q0 * ldy, ldy);
    RSG_LAUNCHED(M->h.ctx, "face_gather");
    M->h.prof.end(s);
  }
}

// VertexFractionalTree::apply_batch (hierarchical.rs:1274-1345) scaled by `scale`.
void rsg::vfrac_apply_strided(rs_vfrac *V, double scale, int nb, const double *xs, size_t ldx,
                              double *ys, size_t ldy, bool plain) {
  cudaStream_t s = V->h.st();
  V->h.plain_rows = plain;
  for (int q0 = 0; q0 < nb; q0 += 3) {
    int k = std::min(3, nb - q0);
    int CC = 4 * k;  // 3 k channels padded to a multiple of 4
    V->h.reserve(CC);
    if (V->h.qmax.n < 64) V->h.qmax.alloc(64);
    RSG_CUDA("product", cudaMemsetAsync(V->h.qmax.p, 0, CC * sizeof(unsigned long long), s));
    for (int pass = 0; pass < 2; ++pass) {
      vertex_m_kernel<<<nblk(V->nv, 256), 256, 0, s>>>(V->order.p, xs + q0 * ldx, ldx, V->nv, k, CC, V->h.m.p,
                                                       V->h.qmax.p, pass);
      RSG_LAUNCHED(V->h.ctx, "vertex_m");
    }
    V->h.product(k);
    vertex_out_kernel<<<nblk(V->nv, 256), 256, 0, s>>>(V->order.p, V->h.xh.p, V->h.z.p, V->nv, k, CC,
                                                       scale, ys + q0 * ldy, ldy);
    RSG_LAUNCHED(V->h.ctx, "vertex_out");
  }
}

namespace {

template <class F>
void host_io(rs_ctx *ctx, DevBuf<double> &xb, DevBuf<double> &yb, size_t n, const double *xh,
             double *yh, F &&apply) {
  cudaStream_t s = ctx->stream;
  if (xb.n < n) xb.alloc(n), yb.alloc(n);
  double *stage = (double *)ctx->staging(n * sizeof(double));
  std::memcpy(stage, xh, n * sizeof(double));
  RSG_CUDA("upload", rsg::copy_async(xb.p, stage, n * sizeof(double), cudaMemcpyHostToDevice, s));
  apply(xb.p, yb.p);
  RSG_CUDA("product", rsg::copy_async(stage, yb.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  RSG_CUDA("product", cudaStreamSynchronize(s));
  std::memcpy(yh, stage, n * sizeof(double));
}

}  // namespace

extern "C" {

int rs_metric_build(rs_ctx *ctx, int nv, int nf, const uint32_t *faces, const double *positions_host,
                    double alpha, double beta, double chi, int leaf_size, int leaf_pairs,
                    rs_metric **out) {
  *out = nullptr;
  return guard([&] {
    auto M = std::make_unique<rs_metric>();
    metric_setup(M.get(), ctx, nv, nf, faces, positions_host, alpha, beta, chi, leaf_size, leaf_pairs);
    ctx_retain(ctx);
    *out = M.release();
  });
}

void rs_metric_free(rs_metric *M) {
  if (!M) return;
  rs_ctx *ctx = M->h.ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  delete M;
  ctx_release(ctx);
}

int rs_metric_apply(rs_metric *M, double w_hi, double w_lo, int nb, const double *xs_host,
                    double *ys_host) {
  return guard([&] {
    M->h.ctx->use();
    size_t n = (size_t)nb * 3 * M->nv;
    host_io(M->h.ctx, M->xbuf, M->ybuf, n, xs_host, ys_host,
            [&](const double *x, double *y) { metric_apply_strided(M, w_hi, w_lo, nb, x, 3 * (size_t)M->nv, y, 3 * (size_t)M->nv); });
  });
}

int rs_metric_apply_device(rs_metric *M, double w_hi, double w_lo, int nb, const double *xs_dev,
                           double *ys_dev) {
  return guard([&] {
    M->h.ctx->use();
    metric_apply_strided(M, w_hi, w_lo, nb, xs_dev, 3 * (size_t)M->nv, ys_dev, 3 * (size_t)M->nv);
  });
}

int rs_metric_build_times(rs_metric *M, double *out8) {
  return guard([&] { std::copy(M->build_times, M->build_times + 8, out8); });
}

int rs_metric_stats(rs_metric *M, int64_t *o) {
  return guard([&] {
    o[0] = (int64_t)M->h.blocks.n_far;
    o[1] = (int64_t)M->h.blocks.n_near;
    o[2] = (int64_t)M->h.blocks.near_entries;
    o[3] = (int64_t)M->h.blocks.depth;
    o[4] = (int64_t)M->h.tree.n_nodes();
  });
}

int rs_metric_blocks(rs_metric *M, uint32_t *far_ptr, uint32_t *far_col, uint32_t *near_ptr,
                     uint32_t *near_col) {
  return guard([&] {
    std::vector<uint32_t> fp, fc, np, nc;
    M->h.blocks.download(fp, fc, np, nc);
    std::copy(fp.begin(), fp.end(), far_ptr);
    std::copy(fc.begin(), fc.end(), far_col);
    std::copy(np.begin(), np.end(), near_ptr);
    std::copy(nc.begin(), nc.end(), near_col);
  });
}

int rs_metric_profile(rs_metric *M, double w_hi, double w_lo, int nb, int reps, char *names,
                      int names_len, double *ms, int max_kernels, int *n_kernels) {
  return guard([&] {
    M->h.ctx->use();
    size_t n = (size_t)nb * 3 * M->nv;
    if (M->xbuf.n < n) M->xbuf.alloc(n), M->ybuf.alloc(n);
    RSG_CUDA("product", cudaMemsetAsync(M->xbuf.p, 0, n * sizeof(double), M->h.st()));
    M->h.prof.start();
    for (int r = 0; r < reps; ++r)
      metric_apply_strided(M, w_hi, w_lo, nb, M->xbuf.p, 3 * (size_t)M->nv, M->ybuf.p, 3 * (size_t)M->nv);
    M->h.prof.stop(M->h.st());
    M->h.prof.report(names, names_len, ms, max_kernels, n_kernels, reps);
  });
}

int rs_vfrac_build(rs_ctx *ctx, int nv, const double *positions_host, const double *mass_host,
                   double tau, double chi, int leaf_size, int leaf_pairs, rs_vfrac **out) {
  *out = nullptr;
  return guard([&] {
    if (!std::isfinite(tau) || nv <= 0)
      fail(RS_INVALID_OPTION, "InvalidOption", "upload", "a finite order and at least one vertex");
    for (int v = 0; v < nv; ++v)
      if (!(std::isfinite(mass_host[v]) && mass_host[v] > 0.0))
        fail(RS_INVALID_OPTION, "InvalidOption", "upload", "positive finite vertex areas");
    ctx->use();
    auto V = std::make_unique<rs_vfrac>();
    V->nv = nv;
    // vertex elements: point f_v, box of the point, mass a_v (hierarchical.rs:1041-1058)
    std::vector<double> ebox(6 * (size_t)nv);
    for (int v = 0; v < nv; ++v)
      for (int k = 0; k < 3; ++k) ebox[6 * v + k] = ebox[6 * v + 3 + k] = positions_host[3 * v + k];
    Tree T = build_tree((size_t)nv, positions_host, ebox.data(), mass_host, leaf_size);
    V->h.kind = VERTEX;
    V->h.n_el = nv;
    V->h.set_exponent(-(tau + 1.0));
    V->h.build_common(ctx, std::move(T), chi, leaf_pairs);
    up_vec(V->order, V->h.tree.order, V->h.st());
    V->h.setup(positions_host, mass_host, nullptr, nullptr);
    ctx_retain(ctx);
    *out = V.release();
  });
}

void rs_vfrac_free(rs_vfrac *V) {
  if (!V) return;
  rs_ctx *ctx = V->h.ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  delete V;
  ctx_release(ctx);
}

int rs_vfrac_apply(rs_vfrac *V, int nb, const double *xs_host, double *ys_host) {
  return guard([&] {
    V->h.ctx->use();
    size_t n = (size_t)nb * 3 * V->nv;
    host_io(V->h.ctx, V->xbuf, V->ybuf, n, xs_host, ys_host,
            [&](const double *x, double *y) { vfrac_apply_strided(V, 1.0, nb, x, 3 * (size_t)V->nv, y, 3 * (size_t)V->nv); });
  });
}

int rs_vfrac_apply_device(rs_vfrac *V, int nb, const double *xs_dev, double *ys_dev) {
  return guard([&] {
    V->h.ctx->use();
    vfrac_apply_strided(V, 1.0, nb, xs_dev, 3 * (size_t)V->nv, ys_dev, 3 * (size_t)V->nv);
  });
}

int rs_vfrac_stats(rs_vfrac *V, int64_t *o) {
  return guard([&] {
    o[0] = (int64_t)V->h.blocks.n_far;
    o[1] = (int64_t)V->h.blocks.n_near;
    o[2] = (int64_t)V->h.blocks.near_entries;
    o[3] = (int64_t)V->h.blocks.depth;
    o[4] = (int64_t)V->h.tree.n_nodes();
  });
}

}  // extern "C"

// ====================================================================== no-allocation product
//
// rs_metric_apply_device_noalloc: the metric product of rs_metric_apply_device with its
// per-call scratch (channel values, results, near partial sums, node sums) carved from one
// file-scope device array instead of buffers that the first call of a size allocates. It is
// for callers that must not allocate while the product runs: a host whose device memory is
// entirely reserved by its own pool after set-up, and a caller on a latency-critical stream,
// since cudaMalloc and cudaFree can synchronize the whole device.
//
// Limits: the scratch is kNoAllocScratchBytes per device, shared by every call in the process,
// so calls that overlap in time (two host threads, or two streams in flight) race on it and
// must be serialized by the caller; a call also uses the metric's own arrival counters (the
// upward pass), so it must not overlap any other product on the same rs_metric either. The
// array is resident on every device where this file's kernels are loaded (from the first
// metric build or product there, with lazy module loading), whether or not this entry point
// is ever called. The first call on a device looks up the array's address
// (cudaGetSymbolAddress, with that device current); when that call is made inside a stream
// capture the lookup should have been done before it, by one earlier call.

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB
constexpr int kNoAllocMaxDevices = 64;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

unsigned char *noalloc_scratch(int device) {
  static std::mutex mu;
  static unsigned char *addr[kNoAllocMaxDevices] = {};
  if (device < 0 || device >= kNoAllocMaxDevices)
    fail(RS_INVALID_OPTION, "InvalidOption", "product", "device ordinal out of range for the no-alloc scratch");
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[device]) {
    void *p = nullptr;
    RSG_CUDA("product", cudaGetSymbolAddress(&p, g_noalloc_scratch));
    addr[device] = static_cast<unsigned char *>(p);
  }
  return addr[device];
}

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Scratch bytes of one tree pass with C channels (the layout carved below).
size_t noalloc_bytes(const HMat &h, int C) {
  size_t nn = h.tree.n_nodes();
  return 2 * align256(nn * C * sizeof(double)) + align256(nn * C * sizeof(float2)) +
         2 * align256(h.n_el * C * sizeof(float2)) +
         align256(std::max<size_t>(h.n_items, 1) * 8 * C * sizeof(float2)) +
         align256(h.tree.leaves.size() * C * sizeof(double)) +
         align256(std::max<size_t>(h.n_far_items, 1) * C * sizeof(float2)) + align256(64 * sizeof(unsigned long long));
}

HDev noalloc_dev(const HMat &h, int C, unsigned char *base) {
  HDev d = h.dev(C);
  size_t nn = h.tree.n_nodes(), off = 0;
  auto take = [&](size_t bytes) {
    unsigned char *p = base + off;
    off += align256(bytes);
    return p;
  };
  d.up = reinterpret_cast<double *>(take(nn * C * sizeof(double)));
  d.up2 = reinterpret_cast<float2 *>(take(nn * C * sizeof(float2)));
  d.farx = reinterpret_cast<double *>(take(nn * C * sizeof(double)));
  d.m = reinterpret_cast<const float2 *>(take(h.n_el * C * sizeof(float2)));
  d.z = reinterpret_cast<float2 *>(take(h.n_el * C * sizeof(float2)));
  d.part = reinterpret_cast<float2 *>(take(std::max<size_t>(h.n_items, 1) * 8 * C * sizeof(float2)));
  d.leafsum = reinterpret_cast<double *>(take(h.tree.leaves.size() * C * sizeof(double)));
  d.fpart = reinterpret_cast<float2 *>(take(std::max<size_t>(h.n_far_items, 1) * C * sizeof(float2)));
  return d;
}

// the per-channel magnitudes of the no-alloc product, after the buffers of noalloc_dev
unsigned long long *noalloc_qmax(const HMat &h, int C, unsigned char *base) {
  return reinterpret_cast<unsigned long long *>(base + noalloc_bytes(h, C) - align256(64 * sizeof(unsigned long long)));
}

// The face product of one group of k <= 3 vectors on the given scratch (the kernels and order
// of HMat::product_cc and metric_apply_strided).
template <int CC>
void noalloc_face_group(rs_metric *M, const HDev &d, unsigned long long *qmax, int k, const double *xs, size_t ldx,
                        double w_hi, double w_lo, double *ys, size_t ldy) {
  HMat &h = M->h;
  cudaStream_t s = h.st();
  float2 *m = const_cast<float2 *>(d.m);
  RSG_CUDA("product", cudaMemsetAsync(qmax, 0, CC * sizeof(unsigned long long), s));
  for (int pass = 0; pass < 2; ++pass) {
    face_m_kernel<<<nblk(M->nf, 256), 256, 0, s>>>(M->ops(), xs, ldx, k, CC, m, qmax, pass);
    RSG_LAUNCHED(h.ctx, "face_m");
  }
  h.upward_far<FACE_CH, CC>(d);
  for (int q = 0; q < k; ++q) {
    hm_rows_kernel<FACE, 12, false><<<nblk(h.n_items * 32, 128), 128, 0, s>>>(d, 12 * q);
    RSG_LAUNCHED(h.ctx, "hm_rows");
  }
  h.epilogue<FACE_CH, CC>(d);
  face_gather_kernel<<<nblk(M->nv, 128), 128, 0, s>>>(M->ops(), d.z, k, CC, w_hi, w_lo, ys, ldy);
  RSG_LAUNCHED(h.ctx, "face_gather");
}

}  // namespace

extern "C" int rs_metric_apply_device_noalloc(rs_metric *M, double w_hi, double w_lo, int nb,
                                              const double *xs_dev, double *ys_dev) {
  return guard([&] {
    if (nb < 1) fail(RS_INVALID_OPTION, "InvalidOption", "product", "at least one vector");
    if (!(std::isfinite(w_hi) && std::isfinite(w_lo)))
      fail(RS_INVALID_OPTION, "InvalidOption", "product", "finite weights");
    const int Cmax = 12 * std::min(3, nb);
    const size_t need = noalloc_bytes(M->h, Cmax);
    if (need > kNoAllocScratchBytes)
      fail(RS_INVALID_OPTION, "InvalidOption", "product",
           "the no-alloc product of " + std::to_string(std::min(3, nb)) + " vector(s) on this mesh needs " +
               std::to_string(need >> 20) + " MiB of scratch, above its 64 MiB; use rs_metric_apply_device");
    M->h.ctx->use();
    unsigned char *base = noalloc_scratch(M->h.ctx->device);
    const size_t ld = 3 * (size_t)M->nv;
    for (int q0 = 0; q0 < nb; q0 += 3) {
      const int k = std::min(3, nb - q0);
      HDev d = noalloc_dev(M->h, 12 * k, base);
      unsigned long long *qm = noalloc_qmax(M->h, 12 * k, base);
      if (k == 1) noalloc_face_group<12>(M, d, qm, 1, xs_dev + q0 * ld, ld, w_hi, w_lo, ys_dev + q0 * ld, ld);
      else if (k == 2) noalloc_face_group<24>(M, d, qm, 2, xs_dev + q0 * ld, ld, w_hi, w_lo, ys_dev + q0 * ld, ld);
      else noalloc_face_group<36>(M, d, qm, 3, xs_dev + q0 * ld, ld, w_hi, w_lo, ys_dev + q0 * ld, ld);
    }
  });
}
