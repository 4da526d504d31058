// Block classification on the device (see block_tree.hpp): the level-by-level pass of
// classify_blocks with every level's pairs classified in parallel and compacted in order by
// exclusive scans, then the CSR grouping by a stable radix sort on the row node (pairs of a row
// keep their level order). The blocks are those of the host classification, in the same order.
// It runs on a stream of its own with stream-ordered allocations, so that it neither waits for
// nor holds up other work on the context's stream.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_reduce.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <vector>

#include "block_tree.hpp"
#include "common.hpp"

namespace rsg {

namespace {

inline unsigned nblk(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

struct NodeRecD {
  double box[6];  // min xyz, max xyz
  double radius;
  uint32_t right;  // 0 for a leaf
  uint32_t len;    // elements
};

__device__ __forceinline__ double dmx(double a, double b) { return a < b ? b : a; }
__device__ __forceinline__ double dmn(double a, double b) { return b < a ? b : a; }

// separated (RS/src/metric/hierarchical.rs:116-123) with the host's operations, rounded one by
// one (no contraction), so that both sides classify every pair alike
__device__ __forceinline__ bool separated_d(const NodeRecD &A, const NodeRecD &B, double chi) {
  if (!(chi > 0.0)) return false;
  double d2 = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double d = dmx(__dsub_rn(dmx(A.box[k], B.box[k]), dmn(A.box[3 + k], B.box[3 + k])), 0.0);
    d2 = __dadd_rn(d2, __dmul_rn(d, d));
  }
  const double h = dmx(A.radius, B.radius);
  return d2 > 0.0 && __dmul_rn(h, h) <= __dmul_rn(__dmul_rn(chi, chi), d2);
}

// per pair: far / near flags and the number of children of a split pair
__global__ void classify_kernel(const uint2 *__restrict__ pairs, uint32_t n, const NodeRecD *__restrict__ rec,
                                double chi, unsigned long long leaf_pairs, uint32_t *__restrict__ f_far,
                                uint32_t *__restrict__ f_near, uint32_t *__restrict__ f_kids) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint2 pr = pairs[i];
  const NodeRecD &A = rec[pr.x], &C = rec[pr.y];
  const bool la = A.right == 0, lc = C.right == 0;
  const bool far_ = pr.x != pr.y && separated_d(A, C, chi);
  const bool near_ = !far_ && ((la && lc) || (unsigned long long)A.len * C.len <= leaf_pairs);
  f_far[i] = far_, f_near[i] = near_;
  f_kids[i] = (far_ || near_) ? 0u : ((la || lc) ? 2u : 4u);
}

// every pair to its place: far and near pairs at their scanned offsets, a split pair's children
// (x, y) for x < na, y < nc in order at its child offset
__global__ void scatter_kernel(const uint2 *__restrict__ pairs, uint32_t n, const NodeRecD *__restrict__ rec,
                               const uint32_t *__restrict__ f_far, const uint32_t *__restrict__ o_far,
                               const uint32_t *__restrict__ f_near, const uint32_t *__restrict__ o_near,
                               const uint32_t *__restrict__ o_kids, uint2 *__restrict__ far_out,
                               uint2 *__restrict__ near_out, uint2 *__restrict__ next) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint2 pr = pairs[i];
  if (f_far[i]) {
    far_out[o_far[i]] = pr;
    return;
  }
  if (f_near[i]) {
    near_out[o_near[i]] = pr;
    return;
  }
  const NodeRecD &A = rec[pr.x], &C = rec[pr.y];
  const bool la = A.right == 0, lc = C.right == 0;
  const uint32_t a0 = la ? pr.x : pr.x + 1, a1 = A.right, c0 = lc ? pr.y : pr.y + 1, c1 = C.right;
  uint2 *o = next + o_kids[i];
  o[0] = make_uint2(a0, c0);
  if (la) {
    o[1] = make_uint2(a0, c1);
  } else if (lc) {
    o[1] = make_uint2(a1, c0);
  } else {
    o[1] = make_uint2(a0, c1), o[2] = make_uint2(a1, c0), o[3] = make_uint2(a1, c1);
  }
}

// tot = {far, near, kids} of a level: the last exclusive offset plus the last flag
__global__ void totals_kernel(uint32_t n, const uint32_t *f_far, const uint32_t *o_far, const uint32_t *f_near,
                              const uint32_t *o_near, const uint32_t *f_kids, const uint32_t *o_kids, uint32_t *tot) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  tot[0] = o_far[n - 1] + f_far[n - 1];
  tot[1] = o_near[n - 1] + f_near[n - 1];
  tot[2] = o_kids[n - 1] + f_kids[n - 1];
}

__global__ void split_pairs_kernel(const uint2 *__restrict__ p, uint32_t n, uint32_t *__restrict__ row,
                                   uint32_t *__restrict__ col) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) row[i] = p[i].x, col[i] = p[i].y;
}

// CSR offsets of rows sorted ascending: ptr[r] = first index with row >= r
__global__ void row_offsets_kernel(const uint32_t *__restrict__ row, uint32_t n, uint32_t nrows,
                                   uint32_t *__restrict__ ptr) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  const uint32_t prev = (i == 0) ? 0 : row[i - 1] + 1;
  const uint32_t cur = (i == n) ? nrows : row[i];
  for (uint32_t r = prev; r <= cur; ++r) ptr[r] = i;
}

// A device array on the classification's stream (stream-ordered allocation and release).
template <class T>
struct AsyncBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaStream_t s;
  explicit AsyncBuf(cudaStream_t st) : s(st) {}
  ~AsyncBuf() {
    if (p) cudaFreeAsync(p, s);
  }
  AsyncBuf(const AsyncBuf &) = delete;
  AsyncBuf &operator=(const AsyncBuf &) = delete;
  void alloc(size_t m) {
    if (p) cudaFreeAsync(p, s);
    p = nullptr, n = 0;
    RSG_CUDA("upload", cudaMallocAsync((void **)&p, std::max<size_t>(m, 1) * sizeof(T), s));
    n = m;
  }
  // grow to at least m elements, keeping the first `keep`
  void reserve(size_t m, size_t keep) {
    if (m <= n) return;
    T *q = nullptr;
    const size_t cap = std::max(m, 2 * n);
    RSG_CUDA("upload", cudaMallocAsync((void **)&q, cap * sizeof(T), s));
    if (keep) RSG_CUDA("upload", cudaMemcpyAsync(q, p, keep * sizeof(T), cudaMemcpyDeviceToDevice, s));
    if (p) cudaFreeAsync(p, s);
    p = q, n = cap;
  }
};

struct StreamGuard {
  cudaStream_t s = nullptr;
  StreamGuard() { RSG_CUDA("upload", cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
  ~StreamGuard() {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
};

// the CSR (ptr, col) of `m` pairs grouped by row, level order kept, into device buffers
void group_device(const AsyncBuf<uint2> &pairs, size_t m, uint32_t nn, cudaStream_t s, DevBuf<uint32_t> &ptr,
                  DevBuf<uint32_t> &col) {
  ptr.alloc((size_t)nn + 1);
  col.alloc(std::max<size_t>(m, 1));
  if (m == 0) {
    RSG_CUDA("upload", cudaMemsetAsync(ptr.p, 0, ((size_t)nn + 1) * sizeof(uint32_t), s));
    return;
  }
  AsyncBuf<uint32_t> r0(s), c0(s), r1(s);
  r0.alloc(m), c0.alloc(m), r1.alloc(m);
  split_pairs_kernel<<<nblk(m, 256), 256, 0, s>>>(pairs.p, (uint32_t)m, r0.p, c0.p);
  RSG_CUDA("upload", cudaGetLastError());
  int bits = 1;
  while (bits < 32 && (1ull << bits) < nn) ++bits;
  size_t tmp_bytes = 0;
  RSG_CUDA("upload", cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, r0.p, r1.p, c0.p, col.p, (int)m, 0, bits, s));
  AsyncBuf<unsigned char> tmp(s);
  tmp.alloc(tmp_bytes);
  RSG_CUDA("upload", cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, r0.p, r1.p, c0.p, col.p, (int)m, 0, bits, s));
  row_offsets_kernel<<<nblk(m + 1, 256), 256, 0, s>>>(r1.p, (uint32_t)m, nn, ptr.p);
  RSG_CUDA("upload", cudaGetLastError());
}

// element pairs of the blocks of row node a (integer sums): far |a||c|, near |a||c| (|a|(|a|-1)
// on the diagonal)
__global__ void block_pairs_kernel(uint32_t nn, const NodeRecD *__restrict__ rec, const uint32_t *far_ptr,
                                   const uint32_t *far_col, const uint32_t *near_ptr, const uint32_t *near_col,
                                   unsigned long long *fp, unsigned long long *ne) {
  const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nn) return;
  const unsigned long long la = rec[a].len;
  unsigned long long f = 0, e = 0;
  for (uint32_t q = far_ptr[a]; q < far_ptr[a + 1]; ++q) f += la * rec[far_col[q]].len;
  for (uint32_t q = near_ptr[a]; q < near_ptr[a + 1]; ++q) {
    const uint32_t c = near_col[q];
    e += c == a ? la * (la - 1) : la * rec[c].len;
  }
  fp[a] = f, ne[a] = e;
}

}  // namespace

void Blocks::download(std::vector<uint32_t> &fp, std::vector<uint32_t> &fc, std::vector<uint32_t> &np,
                      std::vector<uint32_t> &nc) const {
  fp.resize(far_ptr.n), fc.resize(n_far), np.resize(near_ptr.n), nc.resize(n_near);
  RSG_CUDA("blocks", cudaMemcpy(fp.data(), far_ptr.p, far_ptr.n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  RSG_CUDA("blocks", cudaMemcpy(np.data(), near_ptr.p, near_ptr.n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  if (n_far) RSG_CUDA("blocks", cudaMemcpy(fc.data(), far_col.p, n_far * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  if (n_near) RSG_CUDA("blocks", cudaMemcpy(nc.data(), near_col.p, n_near * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  g_d2h_bytes += (fp.size() + fc.size() + np.size() + nc.size()) * sizeof(uint32_t);
}

Blocks classify_blocks_device(const Tree &T, double chi, size_t leaf_pairs) {
  const size_t nn = T.n_nodes();
  Blocks B;
  StreamGuard sg;
  const cudaStream_t s = sg.s;
  std::vector<NodeRecD> rec_h(nn);
  parallel_for(nn, [&](size_t a0, size_t a1) {
    for (size_t a = a0; a < a1; ++a) {
      NodeRecD &r = rec_h[a];
      for (int k = 0; k < 6; ++k) r.box[k] = T.box[6 * a + k];
      r.radius = T.radius[a], r.right = T.right[a], r.len = T.end[a] - T.start[a];
    }
  });
  AsyncBuf<NodeRecD> rec(s);
  rec.alloc(nn);
  RSG_CUDA("upload", copy_async(rec.p, rec_h.data(), nn * sizeof(NodeRecD), cudaMemcpyHostToDevice, s));
  AsyncBuf<uint2> cur(s), nxt(s), far_l(s), near_l(s);
  AsyncBuf<uint32_t> f_far(s), f_near(s), f_kids(s), o_far(s), o_near(s), o_kids(s), tot(s);
  AsyncBuf<unsigned char> scan_tmp(s);
  tot.alloc(3);
  cur.alloc(1);
  const uint2 root = make_uint2(0u, 0u);
  RSG_CUDA("upload", copy_async(cur.p, &root, sizeof(uint2), cudaMemcpyHostToDevice, s));
  size_t n = 1, n_far = 0, n_near = 0;
  auto scan = [&](const uint32_t *in, uint32_t *out, size_t m) {
    size_t bytes = 0;
    RSG_CUDA("upload", cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, (int)m, s));
    if (bytes > scan_tmp.n) scan_tmp.alloc(bytes);
    RSG_CUDA("upload", cub::DeviceScan::ExclusiveSum(scan_tmp.p, bytes, in, out, (int)m, s));
  };
  while (n > 0) {
    ++B.depth;
    if (n > f_far.n) {
      f_far.alloc(n), f_near.alloc(n), f_kids.alloc(n), o_far.alloc(n), o_near.alloc(n), o_kids.alloc(n);
    }
    classify_kernel<<<nblk(n, 256), 256, 0, s>>>(cur.p, (uint32_t)n, rec.p, chi, (unsigned long long)leaf_pairs,
                                                 f_far.p, f_near.p, f_kids.p);
    RSG_CUDA("upload", cudaGetLastError());
    scan(f_far.p, o_far.p, n), scan(f_near.p, o_near.p, n), scan(f_kids.p, o_kids.p, n);
    totals_kernel<<<1, 32, 0, s>>>((uint32_t)n, f_far.p, o_far.p, f_near.p, o_near.p, f_kids.p, o_kids.p, tot.p);
    uint32_t t[3];
    RSG_CUDA("upload", copy_async(t, tot.p, sizeof(t), cudaMemcpyDeviceToHost, s));
    RSG_CUDA("upload", cudaStreamSynchronize(s));
    far_l.reserve(n_far + t[0], n_far);
    near_l.reserve(n_near + t[1], n_near);
    nxt.alloc(t[2]);
    scatter_kernel<<<nblk(n, 256), 256, 0, s>>>(cur.p, (uint32_t)n, rec.p, f_far.p, o_far.p, f_near.p, o_near.p,
                                                o_kids.p, far_l.p + n_far, near_l.p + n_near, nxt.p);
    RSG_CUDA("upload", cudaGetLastError());
    n_far += t[0], n_near += t[1];
    std::swap(cur.p, nxt.p), std::swap(cur.n, nxt.n);
    n = t[2];
  }
  if (n_far > UINT32_MAX || n_near > UINT32_MAX)
    fail(RS_INVALID_OPTION, "InvalidOption", "upload", "block lists exceed 2^32 entries");
  group_device(far_l, n_far, (uint32_t)nn, s, B.far_ptr, B.far_col);
  group_device(near_l, n_near, (uint32_t)nn, s, B.near_ptr, B.near_col);
  B.n_far = n_far, B.n_near = n_near;
  // element pairs of the blocks (integer sums, any order)
  {
    AsyncBuf<unsigned long long> fp(s), ne(s), sums(s);
    fp.alloc(nn), ne.alloc(nn), sums.alloc(2);
    block_pairs_kernel<<<nblk(nn, 256), 256, 0, s>>>((uint32_t)nn, rec.p, B.far_ptr.p, B.far_col.p, B.near_ptr.p,
                                                     B.near_col.p, fp.p, ne.p);
    RSG_CUDA("upload", cudaGetLastError());
    size_t bytes = 0;
    RSG_CUDA("upload", cub::DeviceReduce::Sum(nullptr, bytes, fp.p, sums.p, (int)nn, s));
    if (bytes > scan_tmp.n) scan_tmp.alloc(bytes);
    RSG_CUDA("upload", cub::DeviceReduce::Sum(scan_tmp.p, bytes, fp.p, sums.p, (int)nn, s));
    RSG_CUDA("upload", cub::DeviceReduce::Sum(scan_tmp.p, bytes, ne.p, sums.p + 1, (int)nn, s));
    unsigned long long h[2] = {0, 0};
    RSG_CUDA("upload", copy_async(h, sums.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    RSG_CUDA("upload", cudaStreamSynchronize(s));
    B.far_pairs = h[0], B.near_entries = h[1];
  }
  return B;
}

}  // namespace rsg
