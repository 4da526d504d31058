// Learned preconditioner correction (see learned.hpp): graph, features, the three message-
// passing layers (forward, backward), Adam, and the C ABI rs_learned_* / rs_lgraph_*.
//
// Layer l: h_l[v] = act(W_l,self h_{l-1}[v] + W_l,nb mean_{u in N(v)} h_{l-1}[u] + b_l), with
// act = SiLU for the two hidden layers and the identity for the output layer (3 channels).
// The layers' products (forward, input gradient, weight gradient) run on the tensor cores
// (mma.sync, BF16 operands, FP32 accumulation).
// Features h_0[v] (13): position (centred, divided by the RMS radius), unit vertex normal,
// dual area / mean, r_v / rms(r), y_v / rms(y). Every reduction is a fixed-order two-stage
// sum, so training and inference are deterministic.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <random>
#include <vector>

#include "host_tree.hpp"
#include "learned.hpp"

namespace rsg {

constexpr int kIn = 13;      // input features
constexpr int kOut = 3;      // output channels
constexpr int kChunks = 120; // fixed split of the reductions over vertices

namespace {

inline unsigned nblk(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

__device__ __forceinline__ float silu(float x) { return x / (1.f + __expf(-x)); }
__device__ __forceinline__ float silu_grad(float x) {
  const float s = 1.f / (1.f + __expf(-x));
  return s * (1.f + x * (1.f - s));
}

// partial[b] = sum of x[i]^2 over block b's share of [0, n) for two vectors (stride ld)
__global__ void rms_partial(const double *__restrict__ a, const double *__restrict__ b, size_t n,
                            double *partial) {
  __shared__ double sa[256], sb[256];
  const size_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const size_t i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
  double xa = 0.0, xb = 0.0;
  for (size_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    xa = fma(a[i], a[i], xa);
    if (b) xb = fma(b[i], b[i], xb);
  }
  sa[threadIdx.x] = xa, sb[threadIdx.x] = xb;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sa[threadIdx.x] += sa[threadIdx.x + s], sb[threadIdx.x] += sb[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[2 * blockIdx.x] = sa[0], partial[2 * blockIdx.x + 1] = sb[0];
}

// scales = (rms(a), rms(b)) (1 for a zero vector), also the plain sums of squares
__global__ void rms_final(const double *partial, int nb, size_t n, double *scales) {
  if (threadIdx.x != 0) return;
  double sa = 0.0, sb = 0.0;
  for (int i = 0; i < nb; ++i) sa += partial[2 * i], sb += partial[2 * i + 1];
  const double ra = sqrt(sa / (double)n), rb = sqrt(sb / (double)n);
  scales[0] = ra > 0.0 ? ra : 1.0;
  scales[1] = rb > 0.0 ? rb : 1.0;
  scales[2] = sa, scales[3] = sb;
}

__global__ void features_kernel(int nv, const float *__restrict__ stat7, const double *__restrict__ r,
                                const double *__restrict__ y, const double *__restrict__ scales,
                                float *__restrict__ X) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  float *x = X + (size_t)v * kIn;
  for (int k = 0; k < 7; ++k) x[k] = stat7[(size_t)v * 7 + k];
  const double ir = 1.0 / scales[0], iy = 1.0 / scales[1];
  for (int k = 0; k < 3; ++k) {
    x[7 + k] = (float)(r[3 * (size_t)v + k] * ir);
    x[10 + k] = (float)(y[3 * (size_t)v + k] * iy);
  }
}

// out[v][c] = mean over the one-ring of in[u][c]
__global__ void ring_mean(int nv, int W, const uint32_t *__restrict__ off, const uint32_t *__restrict__ idx,
                          const float *__restrict__ in, float *__restrict__ out) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)nv * W) return;
  const int v = (int)(t / W), c = (int)(t % W);
  const uint32_t a = off[v], b = off[v + 1];
  float s = 0.f;
  for (uint32_t p = a; p < b; ++p) s += in[(size_t)idx[p] * W + c];
  out[t] = b > a ? s / (float)(b - a) : 0.f;
}

// dh[u][c] += sum over v in N(u) of dnb[v][c] / deg(v)   (transpose of ring_mean; the mesh
// one-ring is symmetric)
__global__ void ring_mean_bwd(int nv, int W, const uint32_t *__restrict__ off, const uint32_t *__restrict__ idx,
                              const float *__restrict__ dnb, float *__restrict__ dh) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)nv * W) return;
  const int u = (int)(t / W), c = (int)(t % W);
  float s = 0.f;
  for (uint32_t p = off[u]; p < off[u + 1]; ++p) {
    const uint32_t v = idx[p];
    const uint32_t dv = off[v + 1] - off[v];
    s += dnb[(size_t)v * W + c] / (float)dv;
  }
  dh[t] += s;
}

// ---- the three products of a layer on the tensor cores: mma.sync m16n8k16 with BF16 operands
// and FP32 accumulation. The BF16 weights enter exactly; FP32 activations and gradients are split
// into BF16 parts whose products with a BF16 factor are exact in FP32: three parts (h + m + l)
// carry all 24 significand bits of an FP32 value (the remainders x - h and x - h - m are exact
// FP32 numbers of at most 16 and 8 significant bits). So the forward layer and the input
// gradient equal the FP32 products up to the order of the FP32 additions; the weight gradient
// (two FP32 factors) keeps the three leading products of two-part splits (relative 2^-16).

__device__ __forceinline__ uint32_t bf16x2(float e0, float e1) {
  __nv_bfloat162 t = __floats2bfloat162_rn(e0, e1);  // e0 in the low half
  return *reinterpret_cast<uint32_t *>(&t);
}
__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ void split3(float x, float &h, float &m, float &l) {
  h = bf16_round(x);
  const float r = x - h;
  m = bf16_round(r);
  l = r - m;
}
__device__ __forceinline__ void split2(float x, float &h, float &l) {
  h = bf16_round(x);
  l = x - h;
}

// d += a b for one m16n8k16 tile: a (16 x 16, row-major fragment), b (16 x 8, column-major)
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// The A fragment of a 16 x 16 tile whose element (row, col) is at(row, col): lane (g, t) holds
// rows g and g + 8, columns 2t, 2t + 1, 2t + 8, 2t + 9.
template <class F>
__device__ __forceinline__ void load_a(F at, int g, int t, float (&e)[8]) {
  e[0] = at(g, 2 * t), e[1] = at(g, 2 * t + 1), e[2] = at(g + 8, 2 * t), e[3] = at(g + 8, 2 * t + 1);
  e[4] = at(g, 2 * t + 8), e[5] = at(g, 2 * t + 9), e[6] = at(g + 8, 2 * t + 8), e[7] = at(g + 8, 2 * t + 9);
}
__device__ __forceinline__ void pack_a(const float (&e)[8], uint32_t (&a)[4]) {
  a[0] = bf16x2(e[0], e[1]), a[1] = bf16x2(e[2], e[3]), a[2] = bf16x2(e[4], e[5]), a[3] = bf16x2(e[6], e[7]);
}

// One layer, out[v][o] = act(b[o] + sum_i Ws[o][i] xs[v][i] + sum_i Wn[o][i] xn[v][i]): a warp
// per 16 vertices, all outputs; the weights (zero-padded to K = 16k, N = 8k) in shared memory.
template <int IN, int OUT, bool ACT>
__global__ void __launch_bounds__(128) dense_fwd(int nv, const __nv_bfloat16 *__restrict__ ws,
                                                 const __nv_bfloat16 *__restrict__ wn,
                                                 const __nv_bfloat16 *__restrict__ bias, const float *__restrict__ xs,
                                                 const float *__restrict__ xn, float *__restrict__ pre,
                                                 float *__restrict__ out) {
  constexpr int KP = (IN + 15) / 16 * 16, NP = (OUT + 7) / 8 * 8, NT = NP / 8, KS = KP + 8;
  __shared__ __align__(16) __nv_bfloat16 sw[2][NP][KS];
  __shared__ float sb[NP];
  for (int q = threadIdx.x; q < 2 * NP * KS; q += blockDim.x) {
    const int part = q / (NP * KS), n = (q / KS) % NP, k = q % KS;
    sw[part][n][k] = (n < OUT && k < IN) ? (part ? wn : ws)[n * IN + k] : __float2bfloat16(0.f);
  }
  for (int q = threadIdx.x; q < NP; q += blockDim.x) sb[q] = q < OUT ? __bfloat162float(bias[q]) : 0.f;
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int v0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 16;
  if (v0 >= nv) return;
  float acc[NT][4];
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) {
    const int n0 = nt * 8 + 2 * t;
    acc[nt][0] = sb[n0], acc[nt][1] = sb[n0 + 1], acc[nt][2] = sb[n0], acc[nt][3] = sb[n0 + 1];
  }
#pragma unroll
  for (int part = 0; part < 2; ++part) {
    const float *X = part ? xn : xs;
#pragma unroll
    for (int k0 = 0; k0 < KP; k0 += 16) {
      float e[8], h[8], m[8], l[8];
      load_a([&](int r, int c) { return (v0 + r < nv && k0 + c < IN) ? X[(size_t)(v0 + r) * IN + k0 + c] : 0.f; }, g,
             t, e);
#pragma unroll
      for (int i = 0; i < 8; ++i) split3(e[i], h[i], m[i], l[i]);
      uint32_t ah[4], am[4], al[4];
      pack_a(h, ah), pack_a(m, am), pack_a(l, al);
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const __nv_bfloat16 *wr = &sw[part][nt * 8 + g][k0 + 2 * t];
        const uint32_t b0 = *reinterpret_cast<const uint32_t *>(wr), b1 = *reinterpret_cast<const uint32_t *>(wr + 8);
        mma_bf16(acc[nt], ah, b0, b1);
        mma_bf16(acc[nt], am, b0, b1);
        mma_bf16(acc[nt], al, b0, b1);
      }
    }
  }
#pragma unroll
  for (int nt = 0; nt < NT; ++nt)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int v = v0 + g + (i >= 2 ? 8 : 0), n = nt * 8 + 2 * t + (i & 1);
      if (v < nv && n < OUT) {
        if (pre) pre[(size_t)v * OUT + n] = acc[nt][i];
        out[(size_t)v * OUT + n] = ACT ? silu(acc[nt][i]) : acc[nt][i];
      }
    }
}

// Input gradients din_self[v][i] = sum_o Ws[o][i] dpre[v][o] and din_nb likewise with Wn: a
// warp per 16 vertices; K = OUT, N = IN, the transposed weights in shared memory.
template <int IN, int OUT>
__global__ void __launch_bounds__(128) dense_bwd_in(int nv, const __nv_bfloat16 *__restrict__ ws,
                                                    const __nv_bfloat16 *__restrict__ wn,
                                                    const float *__restrict__ dpre, float *__restrict__ dself,
                                                    float *__restrict__ dnb) {
  constexpr int KP = (OUT + 15) / 16 * 16, NP = (IN + 7) / 8 * 8, NT = NP / 8, KS = KP + 8;
  __shared__ __align__(16) __nv_bfloat16 sw[2][NP][KS];  // sw[part][i][o] = W[o][i]
  for (int q = threadIdx.x; q < 2 * NP * KS; q += blockDim.x) {
    const int part = q / (NP * KS), i = (q / KS) % NP, o = q % KS;
    sw[part][i][o] = (i < IN && o < OUT) ? (part ? wn : ws)[o * IN + i] : __float2bfloat16(0.f);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int v0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 16;
  if (v0 >= nv) return;
  float acc[2][NT][4];
#pragma unroll
  for (int part = 0; part < 2; ++part)
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) acc[part][nt][0] = acc[part][nt][1] = acc[part][nt][2] = acc[part][nt][3] = 0.f;
#pragma unroll
  for (int k0 = 0; k0 < KP; k0 += 16) {
    float e[8], h[8], m[8], l[8];
    load_a([&](int r, int c) { return (v0 + r < nv && k0 + c < OUT) ? dpre[(size_t)(v0 + r) * OUT + k0 + c] : 0.f; },
           g, t, e);
#pragma unroll
    for (int i = 0; i < 8; ++i) split3(e[i], h[i], m[i], l[i]);
    uint32_t ah[4], am[4], al[4];
    pack_a(h, ah), pack_a(m, am), pack_a(l, al);
#pragma unroll
    for (int part = 0; part < 2; ++part)
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const __nv_bfloat16 *wr = &sw[part][nt * 8 + g][k0 + 2 * t];
        const uint32_t b0 = *reinterpret_cast<const uint32_t *>(wr), b1 = *reinterpret_cast<const uint32_t *>(wr + 8);
        mma_bf16(acc[part][nt], ah, b0, b1);
        mma_bf16(acc[part][nt], am, b0, b1);
        mma_bf16(acc[part][nt], al, b0, b1);
      }
  }
#pragma unroll
  for (int part = 0; part < 2; ++part)
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int v = v0 + g + (i >= 2 ? 8 : 0), n = nt * 8 + 2 * t + (i & 1);
        if (v < nv && n < IN) (part ? dnb : dself)[(size_t)v * IN + n] = acc[part][nt][i];
      }
}

// Weight and bias gradients of one layer per vertex chunk c (fixed split, grid = chunks):
// partial[c] = dpre^T [xs | 1 | xn] over the chunk's vertices, K = vertices. Warp w takes the
// output rows 16 (w mod MT) .. and the self (with the bias column at index IN) or the
// neighbour part. Layout of partial[c]: self [o][i], neighbour [o][i], bias [o].
template <int IN, int OUT>
__global__ void dense_bwd_w(int nv, const float *__restrict__ xs, const float *__restrict__ xn,
                            const float *__restrict__ dpre, float *__restrict__ partial) {
  constexpr int MT = (OUT + 15) / 16, NS = (IN + 1 + 7) / 8, NN = (IN + 7) / 8;
  constexpr int NTM = NS > NN ? NS : NN;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, warp = threadIdx.x >> 5;
  const int mt = warp % MT, part = warp / MT;
  const int NT = part ? NN : NS;
  const float *X = part ? xn : xs;
  const int chunk = (nv + gridDim.x - 1) / gridDim.x;
  const int c0 = blockIdx.x * chunk, c1 = min(nv, c0 + chunk);
  const int o0 = mt * 16 + g, o1 = o0 + 8;
  float acc[NTM][4];
#pragma unroll
  for (int nt = 0; nt < NTM; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
  for (int k0 = c0; k0 < c1; k0 += 16) {
    float e[8], h[8], l[8];
    load_a([&](int r, int c) { return (mt * 16 + r < OUT && k0 + c < c1) ? dpre[(size_t)(k0 + c) * OUT + mt * 16 + r] : 0.f; },
           g, t, e);
#pragma unroll
    for (int i = 0; i < 8; ++i) split2(e[i], h[i], l[i]);
    uint32_t ah[4], al[4];
    pack_a(h, ah), pack_a(l, al);
    auto bx = [&](int v, int i) -> float {
      if (v >= c1) return 0.f;
      if (i < IN) return X[(size_t)v * IN + i];
      return (part == 0 && i == IN) ? 1.f : 0.f;
    };
#pragma unroll
    for (int nt = 0; nt < NTM; ++nt) {
      if (nt >= NT) break;
      const int n = nt * 8 + g;
      float f[4] = {bx(k0 + 2 * t, n), bx(k0 + 2 * t + 1, n), bx(k0 + 2 * t + 8, n), bx(k0 + 2 * t + 9, n)};
      float fh[4], fl[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) split2(f[i], fh[i], fl[i]);
      const uint32_t bh0 = bf16x2(fh[0], fh[1]), bh1 = bf16x2(fh[2], fh[3]);
      const uint32_t bl0 = bf16x2(fl[0], fl[1]), bl1 = bf16x2(fl[2], fl[3]);
      mma_bf16(acc[nt], ah, bh0, bh1);
      mma_bf16(acc[nt], ah, bl0, bl1);
      mma_bf16(acc[nt], al, bh0, bh1);
    }
  }
  const size_t P = 2 * (size_t)OUT * IN + OUT;
  float *pc = partial + (size_t)blockIdx.x * P;
#pragma unroll
  for (int nt = 0; nt < NTM; ++nt) {
    if (nt >= NT) break;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int o = i >= 2 ? o1 : o0, n = nt * 8 + 2 * t + (i & 1);
      if (o >= OUT) continue;
      if (n < IN) pc[(part ? (size_t)OUT * IN : 0) + (size_t)o * IN + n] = acc[nt][i];
      else if (part == 0 && n == IN) pc[2 * (size_t)OUT * IN + o] = acc[nt][i];
    }
  }
}

// z = y + rms(y) o on the position rows; rows >= 3V of the vector are copied from y
__global__ void output_kernel(int nv, size_t rows, const float *__restrict__ o, const double *__restrict__ y,
                              const double *__restrict__ scales, double *__restrict__ z) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= rows) return;
  z[t] = t < 3 * (size_t)nv ? y[t] + scales[1] * (double)o[t] : y[t];
}

// loss partials and dL/do for L = sum |z - zt|^2 / max(sum |zt|^2, sum |y|^2), z = y + s o
// (s = rms(y)); the larger of the two norms keeps residuals whose solution is far smaller than
// the cheap preconditioner's answer (rough residuals) from dominating the training
__global__ void loss_kernel(int nv, const float *__restrict__ o, const double *__restrict__ y,
                            const double *__restrict__ zt, const double *__restrict__ scales,
                            const double *__restrict__ zz, float *__restrict__ dO, double *partial) {
  __shared__ double sh[256];
  const size_t n = 3 * (size_t)nv;
  const size_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const size_t i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
  const double s = scales[1], d0 = fmax(zz[0], scales[3]), den = d0 > 0.0 ? d0 : 1.0;
  double acc = 0.0;
  for (size_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const double e = y[i] + s * (double)o[i] - zt[i];
    acc = fma(e, e, acc);
    dO[i] = (float)(2.0 * s * e / den);
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0] / den;
}

template <bool ACT>
__global__ void dpre_kernel(size_t n, const float *__restrict__ dout, const float *__restrict__ pre,
                            float *__restrict__ dpre) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  dpre[t] = ACT ? dout[t] * silu_grad(pre[t]) : dout[t];
}

// grad[k] += sum over chunks of partial[c][k] (fixed order)
__global__ void grad_reduce(int nchunks, size_t P, const float *__restrict__ partial, float *__restrict__ grad) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= P) return;
  float s = 0.f;
  for (int c = 0; c < nchunks; ++c) s += partial[(size_t)c * P + k];
  grad[k] += s;
}

__global__ void adam_kernel(size_t P, float *__restrict__ w, float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, __nv_bfloat16 *__restrict__ wb, float lr, float b1, float b2,
                            float eps, float c1, float c2, float clip) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= P) return;
  float gk = fminf(fmaxf(g[k], -clip), clip);
  m[k] = b1 * m[k] + (1.f - b1) * gk;
  v[k] = b2 * v[k] + (1.f - b2) * gk * gk;
  w[k] -= lr * (m[k] / c1) / (sqrtf(v[k] / c2) + eps);
  g[k] = 0.f;
  wb[k] = __float2bfloat16(w[k]);
}

__global__ void to_bf16(size_t P, const float *__restrict__ w, __nv_bfloat16 *__restrict__ wb) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k < P) wb[k] = __float2bfloat16(w[k]);
}

}  // namespace

}  // namespace rsg

using namespace rsg;

// Parameter layout (floats): W1s[H][13] W1n[H][13] b1[H] W2s[H][H] W2n[H][H] b2[H] W3s[3][H]
// W3n[3][H] b3[3]; H = 64.
struct rs_learned {
  static constexpr int H = 64;
  rs_ctx *ctx = nullptr;
  size_t P = 0;
  size_t o1s, o1n, o1b, o2s, o2n, o2b, o3s, o3n, o3b;
  DevBuf<float> w, g, m, v, partial;
  DevBuf<__nv_bfloat16> wb;
  int64_t steps = 0;
  int cap_v = 0;
  DevBuf<float> X, nX, pre1, h1, nh1, pre2, h2, nh2, o, dO, dpre, dh, dself, dnb;
  DevBuf<double> red, scales, zz;
  rs_learned() {
    const size_t H_ = H;
    o1s = 0, o1n = o1s + H_ * kIn, o1b = o1n + H_ * kIn;
    o2s = o1b + H_, o2n = o2s + H_ * H_, o2b = o2n + H_ * H_;
    o3s = o2b + H_, o3n = o3s + kOut * H_, o3b = o3n + kOut * H_;
    P = o3b + kOut;
  }
  void reserve(int nv) {
    if (nv <= cap_v) return;
    cap_v = nv;
    size_t n = (size_t)nv;
    X.alloc(n * kIn), nX.alloc(n * kIn);
    pre1.alloc(n * H), h1.alloc(n * H), nh1.alloc(n * H), pre2.alloc(n * H), h2.alloc(n * H), nh2.alloc(n * H);
    o.alloc(n * kOut), dO.alloc(n * kOut);
    dpre.alloc(n * H), dh.alloc(n * H), dself.alloc(n * H), dnb.alloc(n * H);
  }
};

struct rs_lgraph {
  rs_ctx *ctx = nullptr;
  int nv = 0;
  DevBuf<uint32_t> off, idx;
  DevBuf<float> stat7;
};

namespace rsg {
namespace {

// Forward pass of vector (r, y) on the graph; keeps the activations in the model buffers.
void forward(rs_learned *M, rs_lgraph *G, const double *r, const double *y, bool keep) {
  rs_ctx *ctx = M->ctx;
  cudaStream_t s = ctx->stream;
  const int nv = G->nv, H = rs_learned::H;
  M->reserve(nv);
  if (M->red.n < 2 * kChunks) M->red.alloc(2 * kChunks), M->scales.alloc(4), M->zz.alloc(4);
  const size_t n3 = 3 * (size_t)nv;
  rms_partial<<<kChunks, 256, 0, s>>>(r, y, n3, M->red.p);
  RSG_LAUNCHED(ctx, "learned_rms");
  rms_final<<<1, 32, 0, s>>>(M->red.p, kChunks, n3, M->scales.p);
  RSG_LAUNCHED(ctx, "learned_rms");
  features_kernel<<<nblk(nv, 128), 128, 0, s>>>(nv, G->stat7.p, r, y, M->scales.p, M->X.p);
  RSG_LAUNCHED(ctx, "learned_features");
  const __nv_bfloat16 *wb = M->wb.p;
  auto mean = [&](int W, const float *in, float *out) {
    ring_mean<<<nblk((size_t)nv * W, 256), 256, 0, s>>>(nv, W, G->off.p, G->idx.p, in, out);
    RSG_LAUNCHED(ctx, "learned_mean");
  };
  mean(kIn, M->X.p, M->nX.p);
  dense_fwd<kIn, 64, true><<<nblk(nv, 64), 128, 0, s>>>(nv, wb + M->o1s, wb + M->o1n, wb + M->o1b, M->X.p,
                                                               M->nX.p, keep ? M->pre1.p : nullptr, M->h1.p);
  RSG_LAUNCHED(ctx, "learned_dense");
  mean(H, M->h1.p, M->nh1.p);
  dense_fwd<64, 64, true><<<nblk(nv, 64), 128, 0, s>>>(nv, wb + M->o2s, wb + M->o2n, wb + M->o2b, M->h1.p,
                                                              M->nh1.p, keep ? M->pre2.p : nullptr, M->h2.p);
  RSG_LAUNCHED(ctx, "learned_dense");
  mean(H, M->h2.p, M->nh2.p);
  dense_fwd<64, kOut, false><<<nblk(nv, 64), 128, 0, s>>>(nv, wb + M->o3s, wb + M->o3n, wb + M->o3b,
                                                                   M->h2.p, M->nh2.p, nullptr, M->o.p);
  RSG_LAUNCHED(ctx, "learned_dense");
}

template <int IN, int OUT>
void layer_grad(rs_learned *M, int nv, const float *xs, const float *xn, size_t ows) {
  rs_ctx *ctx = M->ctx;
  cudaStream_t s = ctx->stream;
  const int nch = std::max(1, std::min(kChunks, (nv + 255) / 256));
  const size_t P = 2 * (size_t)OUT * IN + OUT;
  if (M->partial.n < (size_t)kChunks * P) M->partial.alloc((size_t)kChunks * P);
  dense_bwd_w<IN, OUT><<<nch, 64 * ((OUT + 15) / 16), 0, s>>>(nv, xs, xn, M->dpre.p, M->partial.p);
  RSG_LAUNCHED(ctx, "learned_bwd_w");
  // the layer's parameters are contiguous: self, nb, bias
  grad_reduce<<<nblk(P, 256), 256, 0, s>>>(nch, P, M->partial.p, M->g.p + ows);
  RSG_LAUNCHED(ctx, "learned_grad_reduce");
}

}  // namespace

void learned_apply(rs_learned *M, rs_lgraph *G, int nb, const double *r, const double *y, size_t ld,
                   size_t rows, double *z) {
  for (int q = 0; q < nb; ++q) {
    forward(M, G, r + q * ld, y + q * ld, false);
    output_kernel<<<nblk(rows, 256), 256, 0, M->ctx->stream>>>(G->nv, rows, M->o.p, y + q * ld, M->scales.p,
                                                               z + q * ld);
    RSG_LAUNCHED(M->ctx, "learned_output");
  }
}

}  // namespace rsg

extern "C" {

int rs_learned_create(rs_ctx *ctx, uint64_t seed, rs_learned **out) {
  *out = nullptr;
  return guard([&] {
    ctx->use();
    auto M = std::make_unique<rs_learned>();
    M->ctx = ctx;
    std::vector<float> w(M->P, 0.f);
    std::mt19937_64 rng(seed);
    auto init = [&](size_t off, int fan_out, int fan_in) {
      std::normal_distribution<double> nd(0.0, std::sqrt(1.0 / (2.0 * fan_in)));
      for (size_t i = 0; i < (size_t)fan_out * fan_in; ++i) w[off + i] = (float)nd(rng);
    };
    const int H = rs_learned::H;
    init(M->o1s, H, kIn), init(M->o1n, H, kIn), init(M->o2s, H, H), init(M->o2n, H, H);
    init(M->o3s, kOut, H), init(M->o3n, kOut, H);
    for (size_t i = M->o3s; i < M->P; ++i) w[i] *= 0.01f;  // start near z = y
    cudaStream_t s = ctx->stream;
    M->w.upload(w, s);
    M->g.alloc(M->P), M->m.alloc(M->P), M->v.alloc(M->P), M->wb.alloc(M->P);
    RSG_CUDA("upload", cudaMemsetAsync(M->g.p, 0, M->P * sizeof(float), s));
    RSG_CUDA("upload", cudaMemsetAsync(M->m.p, 0, M->P * sizeof(float), s));
    RSG_CUDA("upload", cudaMemsetAsync(M->v.p, 0, M->P * sizeof(float), s));
    to_bf16<<<nblk(M->P, 256), 256, 0, s>>>(M->P, M->w.p, M->wb.p);
    RSG_LAUNCHED(ctx, "learned_bf16");
    RSG_CUDA("upload", cudaStreamSynchronize(s));
    ctx_retain(ctx);
    *out = M.release();
  });
}

void rs_learned_free(rs_learned *M) {
  if (!M) return;
  rs_ctx *ctx = M->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  delete M;
  ctx_release(ctx);
}

int rs_learned_parameter_count(rs_learned *M, int64_t *count) {
  return guard([&] { *count = (int64_t)M->P; });
}

int rs_learned_get_parameters(rs_learned *M, float *host) {
  return guard([&] {
    M->ctx->use();
    M->w.download(host, M->P, M->ctx->stream);
    RSG_CUDA("product", cudaStreamSynchronize(M->ctx->stream));
  });
}

int rs_learned_get_gradient(rs_learned *M, float *host) {
  return guard([&] {
    M->ctx->use();
    M->g.download(host, M->P, M->ctx->stream);
    RSG_CUDA("product", cudaStreamSynchronize(M->ctx->stream));
  });
}

int rs_learned_set_parameters(rs_learned *M, const float *host) {
  return guard([&] {
    M->ctx->use();
    for (size_t i = 0; i < M->P; ++i)
      if (!std::isfinite(host[i])) fail(RS_INVALID_OPTION, "InvalidOption", "upload", "finite parameters");
    cudaStream_t s = M->ctx->stream;
    RSG_CUDA("upload", rsg::copy_async(M->w.p, host, M->P * sizeof(float), cudaMemcpyHostToDevice, s));
    RSG_CUDA("upload", cudaMemsetAsync(M->m.p, 0, M->P * sizeof(float), s));
    RSG_CUDA("upload", cudaMemsetAsync(M->v.p, 0, M->P * sizeof(float), s));
    RSG_CUDA("upload", cudaMemsetAsync(M->g.p, 0, M->P * sizeof(float), s));
    to_bf16<<<nblk(M->P, 256), 256, 0, s>>>(M->P, M->w.p, M->wb.p);
    RSG_LAUNCHED(M->ctx, "learned_bf16");
    M->steps = 0;
    RSG_CUDA("upload", cudaStreamSynchronize(s));
  });
}

int rs_lgraph_create(rs_ctx *ctx, int nv, int nf, const uint32_t *faces, const double *positions_host,
                     rs_lgraph **out) {
  *out = nullptr;
  return guard([&] {
    validate_topology(nv, nf, faces);
    validate_positions(nv, nf, faces, positions_host);
    ctx->use();
    auto G = std::make_unique<rs_lgraph>();
    G->ctx = ctx;
    G->nv = nv;
    // one-ring adjacency (sorted, unique) from the faces
    std::vector<std::vector<uint32_t>> nb(nv);
    for (int f = 0; f < nf; ++f)
      for (int c = 0; c < 3; ++c) {
        uint32_t a = faces[3 * f + c], b = faces[3 * f + (c + 1) % 3];
        nb[a].push_back(b), nb[b].push_back(a);
      }
    std::vector<uint32_t> off(nv + 1, 0), idx;
    for (int v = 0; v < nv; ++v) {
      auto &l = nb[v];
      std::sort(l.begin(), l.end());
      l.erase(std::unique(l.begin(), l.end()), l.end());
      off[v + 1] = off[v] + (uint32_t)l.size();
      idx.insert(idx.end(), l.begin(), l.end());
    }
    // static features: centred / RMS-radius positions, unit area-weighted normals, dual area
    FaceGeom g = face_geometry(nf, faces, positions_host);
    std::vector<double> nrm(3 * (size_t)nv, 0.0), area(nv, 0.0);
    double cen[3] = {0, 0, 0};
    for (int v = 0; v < nv; ++v)
      for (int k = 0; k < 3; ++k) cen[k] += positions_host[3 * (size_t)v + k] / nv;
    double r2 = 0.0;
    for (int v = 0; v < nv; ++v)
      for (int k = 0; k < 3; ++k) r2 += std::pow(positions_host[3 * (size_t)v + k] - cen[k], 2) / nv;
    const double R = r2 > 0.0 ? std::sqrt(r2) : 1.0;
    for (int f = 0; f < nf; ++f)
      for (int c = 0; c < 3; ++c) {
        uint32_t v = faces[3 * f + c];
        area[v] += g.area[f] / 3.0;
        for (int k = 0; k < 3; ++k) nrm[3 * (size_t)v + k] += g.area[f] * g.normal[3 * (size_t)f + k];
      }
    double amean = 0.0;
    for (int v = 0; v < nv; ++v) amean += area[v] / nv;
    std::vector<float> st(7 * (size_t)nv);
    for (int v = 0; v < nv; ++v) {
      double nn = std::sqrt(nrm[3 * (size_t)v] * nrm[3 * (size_t)v] + nrm[3 * (size_t)v + 1] * nrm[3 * (size_t)v + 1] +
                            nrm[3 * (size_t)v + 2] * nrm[3 * (size_t)v + 2]);
      for (int k = 0; k < 3; ++k) {
        st[7 * (size_t)v + k] = (float)((positions_host[3 * (size_t)v + k] - cen[k]) / R);
        st[7 * (size_t)v + 3 + k] = (float)(nn > 0.0 ? nrm[3 * (size_t)v + k] / nn : 0.0);
      }
      st[7 * (size_t)v + 6] = (float)(area[v] / amean);
    }
    cudaStream_t s = ctx->stream;
    G->off.upload(off, s), G->idx.upload(idx, s), G->stat7.upload(st, s);
    RSG_CUDA("upload", cudaStreamSynchronize(s));
    ctx_retain(ctx);
    *out = G.release();
  });
}

void rs_lgraph_free(rs_lgraph *G) {
  if (!G) return;
  rs_ctx *ctx = G->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  delete G;
  ctx_release(ctx);
}

int rs_learned_apply_device(rs_learned *M, rs_lgraph *G, int nb, const double *r_dev, const double *y_dev,
                            double *z_dev) {
  return guard([&] {
    M->ctx->use();
    if (nb < 1) fail(RS_INVALID_OPTION, "InvalidOption", "product", "at least one vector");
    learned_apply(M, G, nb, r_dev, y_dev, 3 * (size_t)G->nv, 3 * (size_t)G->nv, z_dev);
  });
}

int rs_learned_loss_and_gradient_device(rs_learned *M, rs_lgraph *G, const double *r_dev, const double *y_dev,
                                        const double *zt_dev, double *loss) {
  return guard([&] {
    M->ctx->use();
    rs_ctx *ctx = M->ctx;
    cudaStream_t s = ctx->stream;
    const int nv = G->nv, H = rs_learned::H;
    const size_t n3 = 3 * (size_t)nv;
    forward(M, G, r_dev, y_dev, true);
    // |zt|^2, then the loss and dL/do
    rms_partial<<<kChunks, 256, 0, s>>>(zt_dev, nullptr, n3, M->red.p);
    RSG_LAUNCHED(ctx, "learned_rms");
    rms_final<<<1, 32, 0, s>>>(M->red.p, kChunks, n3, M->zz.p);  // zz[2] = sum of zt^2
    RSG_LAUNCHED(ctx, "learned_rms");
    DevBuf<double> lpart(kChunks);
    loss_kernel<<<kChunks, 256, 0, s>>>(nv, M->o.p, y_dev, zt_dev, M->scales.p, M->zz.p + 2, M->dO.p, lpart.p);
    RSG_LAUNCHED(ctx, "learned_loss");
    // layer 3 (linear): dpre = dO
    M->reserve(nv);
    RSG_CUDA("product", cudaMemcpyAsync(M->dpre.p, M->dO.p, n3 * sizeof(float), cudaMemcpyDeviceToDevice, s));
    layer_grad<64, kOut>(M, nv, M->h2.p, M->nh2.p, M->o3s);
    const __nv_bfloat16 *wb = M->wb.p;
    dense_bwd_in<64, kOut><<<nblk(nv, 64), 128, 0, s>>>(nv, wb + M->o3s, wb + M->o3n, M->dpre.p,
                                                                      M->dself.p, M->dnb.p);
    RSG_LAUNCHED(ctx, "learned_bwd_in");
    // dh2 = dself + mean^T(dnb)
    RSG_CUDA("product", cudaMemcpyAsync(M->dh.p, M->dself.p, (size_t)nv * H * sizeof(float), cudaMemcpyDeviceToDevice, s));
    ring_mean_bwd<<<nblk((size_t)nv * H, 256), 256, 0, s>>>(nv, H, G->off.p, G->idx.p, M->dnb.p, M->dh.p);
    RSG_LAUNCHED(ctx, "learned_mean_bwd");
    // layer 2
    dpre_kernel<true><<<nblk((size_t)nv * H, 256), 256, 0, s>>>((size_t)nv * H, M->dh.p, M->pre2.p, M->dpre.p);
    RSG_LAUNCHED(ctx, "learned_dpre");
    layer_grad<64, 64>(M, nv, M->h1.p, M->nh1.p, M->o2s);
    dense_bwd_in<64, 64><<<nblk(nv, 64), 128, 0, s>>>(nv, wb + M->o2s, wb + M->o2n, M->dpre.p,
                                                                    M->dself.p, M->dnb.p);
    RSG_LAUNCHED(ctx, "learned_bwd_in");
    RSG_CUDA("product", cudaMemcpyAsync(M->dh.p, M->dself.p, (size_t)nv * H * sizeof(float), cudaMemcpyDeviceToDevice, s));
    ring_mean_bwd<<<nblk((size_t)nv * H, 256), 256, 0, s>>>(nv, H, G->off.p, G->idx.p, M->dnb.p, M->dh.p);
    RSG_LAUNCHED(ctx, "learned_mean_bwd");
    // layer 1
    dpre_kernel<true><<<nblk((size_t)nv * H, 256), 256, 0, s>>>((size_t)nv * H, M->dh.p, M->pre1.p, M->dpre.p);
    RSG_LAUNCHED(ctx, "learned_dpre");
    layer_grad<kIn, 64>(M, nv, M->X.p, M->nX.p, M->o1s);
    std::vector<double> lp(kChunks);
    lpart.download(lp.data(), kChunks, s);
    RSG_CUDA("product", cudaStreamSynchronize(s));
    double L = 0.0;
    for (double x : lp) L += x;
    *loss = L;
  });
}

int rs_learned_adam_step(rs_learned *M, double lr, double clip) {
  return guard([&] {
    M->ctx->use();
    if (!(lr > 0.0 && std::isfinite(lr))) fail(RS_INVALID_OPTION, "InvalidOption", "product", "positive learning rate");
    M->steps++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)M->steps), c2 = 1.f - std::pow(b2, (float)M->steps);
    adam_kernel<<<nblk(M->P, 256), 256, 0, M->ctx->stream>>>(M->P, M->w.p, M->g.p, M->m.p, M->v.p, M->wb.p,
                                                             (float)lr, b1, b2, 1e-8f, c1, c2,
                                                             clip > 0.0 ? (float)clip : 1e30f);
    RSG_LAUNCHED(M->ctx, "learned_adam");
  });
}

}  // extern "C"
