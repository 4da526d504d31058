// Learned preconditioner correction (see learned.hpp): graph, features, the three message-
// passing layers (forward, backward), Adam, and the C ABI rs_learned_* / rs_lgraph_*.
//
// Layer l: h_l[v] = act(W_l,self h_{l-1}[v] + W_l,nb mean_{u in N(v)} h_{l-1}[u] + b_l), with
// act = SiLU for the two hidden layers and the identity for the output layer (3 channels).
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

// One layer: thread (v, o) of VPB vertices per block; weights (BF16 -> float) in shared memory.
template <int IN, int OUT, bool ACT>
__global__ void dense_fwd(int nv, const __nv_bfloat16 *__restrict__ ws, const __nv_bfloat16 *__restrict__ wn,
                          const __nv_bfloat16 *__restrict__ bias, const float *__restrict__ xs,
                          const float *__restrict__ xn, float *__restrict__ pre, float *__restrict__ out) {
  __shared__ float sw[2 * OUT * IN + OUT];
  for (int i = threadIdx.x; i < OUT * IN; i += blockDim.x) {
    sw[i] = __bfloat162float(ws[i]);
    sw[OUT * IN + i] = __bfloat162float(wn[i]);
  }
  for (int i = threadIdx.x; i < OUT; i += blockDim.x) sw[2 * OUT * IN + i] = __bfloat162float(bias[i]);
  __syncthreads();
  constexpr int VPB = 256 / OUT;
  const int o = threadIdx.x % OUT, vl = threadIdx.x / OUT;
  const int v = blockIdx.x * VPB + vl;
  if (vl >= VPB || v >= nv) return;
  const float *a = xs + (size_t)v * IN, *b = xn + (size_t)v * IN;
  const float *wa = sw + o * IN, *wb = sw + OUT * IN + o * IN;
  float acc = sw[2 * OUT * IN + o];
#pragma unroll 8
  for (int i = 0; i < IN; ++i) acc = fmaf(wa[i], a[i], fmaf(wb[i], b[i], acc));
  if (pre) pre[(size_t)v * OUT + o] = acc;
  out[(size_t)v * OUT + o] = ACT ? silu(acc) : acc;
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

// Weight gradients of one layer, per vertex chunk: grid (kChunks, OUT), block 2 IN threads;
// partial[c][o][i] (self, then nb at OUT IN + ...), bias at 2 OUT IN + o.
template <int IN, int OUT>
__global__ void dense_bwd_w(int nv, const float *__restrict__ xs, const float *__restrict__ xn,
                            const float *__restrict__ dpre, float *__restrict__ partial) {
  const int c = blockIdx.x, o = blockIdx.y, i = threadIdx.x;
  const int chunk = (nv + gridDim.x - 1) / gridDim.x;
  const int v0 = c * chunk, v1 = min(nv, v0 + chunk);
  const bool self = i < IN;
  const int ii = self ? i : i - IN;
  if (ii >= IN) return;
  const float *x = self ? xs : xn;
  float acc = 0.f, accb = 0.f;
  for (int v = v0; v < v1; ++v) {
    const float d = dpre[(size_t)v * OUT + o];
    acc = fmaf(d, x[(size_t)v * IN + ii], acc);
    accb += d;
  }
  const size_t P = 2 * (size_t)OUT * IN + OUT;
  float *pc = partial + (size_t)c * P;
  pc[(self ? 0 : (size_t)OUT * IN) + (size_t)o * IN + ii] = acc;
  if (i == 0) pc[2 * (size_t)OUT * IN + o] = accb;
}

// grad[k] += sum over chunks of partial[c][k] (fixed order)
__global__ void grad_reduce(int nchunks, size_t P, const float *__restrict__ partial, float *__restrict__ grad) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= P) return;
  float s = 0.f;
  for (int c = 0; c < nchunks; ++c) s += partial[(size_t)c * P + k];
  grad[k] += s;
}

// din_self[v][i] = sum_o Ws[o][i] dpre[v][o]; din_nb likewise with Wn
template <int IN, int OUT>
__global__ void dense_bwd_in(int nv, const __nv_bfloat16 *__restrict__ ws, const __nv_bfloat16 *__restrict__ wn,
                             const float *__restrict__ dpre, float *__restrict__ dself, float *__restrict__ dnb) {
  __shared__ float sw[2 * OUT * IN];
  for (int i = threadIdx.x; i < OUT * IN; i += blockDim.x) {
    sw[i] = __bfloat162float(ws[i]);
    sw[OUT * IN + i] = __bfloat162float(wn[i]);
  }
  __syncthreads();
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)nv * IN) return;
  const int v = (int)(t / IN), i = (int)(t % IN);
  const float *d = dpre + (size_t)v * OUT;
  float a = 0.f, b = 0.f;
  for (int o = 0; o < OUT; ++o) {
    a = fmaf(sw[o * IN + i], d[o], a);
    b = fmaf(sw[OUT * IN + o * IN + i], d[o], b);
  }
  dself[t] = a;
  dnb[t] = b;
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
  dense_fwd<kIn, 64, true><<<nblk(nv, 256 / 64), 256, 0, s>>>(nv, wb + M->o1s, wb + M->o1n, wb + M->o1b, M->X.p,
                                                               M->nX.p, keep ? M->pre1.p : nullptr, M->h1.p);
  RSG_LAUNCHED(ctx, "learned_dense");
  mean(H, M->h1.p, M->nh1.p);
  dense_fwd<64, 64, true><<<nblk(nv, 256 / 64), 256, 0, s>>>(nv, wb + M->o2s, wb + M->o2n, wb + M->o2b, M->h1.p,
                                                              M->nh1.p, keep ? M->pre2.p : nullptr, M->h2.p);
  RSG_LAUNCHED(ctx, "learned_dense");
  mean(H, M->h2.p, M->nh2.p);
  dense_fwd<64, kOut, false><<<nblk(nv, 256 / kOut), 256, 0, s>>>(nv, wb + M->o3s, wb + M->o3n, wb + M->o3b,
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
  dense_bwd_w<IN, OUT><<<dim3(nch, OUT), 2 * IN, 0, s>>>(nv, xs, xn, M->dpre.p, M->partial.p);
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
    dense_bwd_in<64, kOut><<<nblk((size_t)nv * H, 256), 256, 0, s>>>(nv, wb + M->o3s, wb + M->o3n, M->dpre.p,
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
    dense_bwd_in<64, 64><<<nblk((size_t)nv * H, 256), 256, 0, s>>>(nv, wb + M->o2s, wb + M->o2n, M->dpre.p,
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
