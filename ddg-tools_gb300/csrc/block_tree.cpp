// Block classification of the block cluster tree (see block_tree.hpp). Each level's pairs
// are classified by worker threads in contiguous chunks whose outputs are concatenated in
// chunk order, so the blocks come out in exactly the sequential level order.
#include "block_tree.hpp"

#include <algorithm>
#include <cmath>
#include <thread>

namespace rsg {

namespace {

// box_distance_sq (RS/src/spatial/mod.rs:131-138) and separated (hierarchical.rs:116-123).
inline bool separated(const Tree &T, uint32_t a, uint32_t b, double chi) {
  if (!(chi > 0.0)) return false;
  const double *ba = &T.box[6 * (size_t)a], *bb = &T.box[6 * (size_t)b];
  double d2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    double d = std::fmax(std::fmax(ba[k], bb[k]) - std::fmin(ba[3 + k], bb[3 + k]), 0.0);
    d2 += d * d;
  }
  double h = std::fmax(T.radius[a], T.radius[b]);
  return d2 > 0.0 && h * h <= chi * chi * d2;
}

struct Out {
  std::vector<std::pair<uint32_t, uint32_t>> far, near, next;
};

void group(const std::vector<std::pair<uint32_t, uint32_t>> &pairs, size_t n,
           std::vector<uint32_t> &ptr, std::vector<uint32_t> &col) {
  ptr.assign(n + 1, 0);
  for (auto &p : pairs) ptr[p.first + 1]++;
  for (size_t i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
  std::vector<uint32_t> fill(ptr.begin(), ptr.end() - 1);
  col.resize(pairs.size());
  for (auto &p : pairs) col[fill[p.first]++] = p.second;
}

}  // namespace

Blocks classify_blocks(const Tree &T, double chi, size_t leaf_pairs, int threads) {
  const size_t nn = T.n_nodes();
  auto leaf = [&](uint32_t a) { return T.right[a] == 0; };
  auto len = [&](uint32_t a) { return (size_t)(T.end[a] - T.start[a]); };
  int nt = threads > 0 ? threads : (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::pair<uint32_t, uint32_t>> far, near, level{{0, 0}};
  Blocks B;
  auto classify = [&](size_t b, size_t e, Out &o) {
    for (size_t i = b; i < e; ++i) {
      auto [a, c] = level[i];
      if (a != c && separated(T, a, c, chi))
        o.far.push_back({a, c});
      else if ((leaf(a) && leaf(c)) || len(a) * len(c) <= leaf_pairs)
        o.near.push_back({a, c});
      else {
        uint32_t ka[2] = {leaf(a) ? a : a + 1, T.right[a]};
        uint32_t kc[2] = {leaf(c) ? c : c + 1, T.right[c]};
        int na = leaf(a) ? 1 : 2, nc = leaf(c) ? 1 : 2;
        for (int x = 0; x < na; ++x)
          for (int y = 0; y < nc; ++y) o.next.push_back({ka[x], kc[y]});
      }
    }
  };
  while (!level.empty()) {
    ++B.depth;
    size_t n = level.size();
    int parts = (n < 4096) ? 1 : nt;
    std::vector<Out> outs(parts);
    if (parts == 1) {
      classify(0, n, outs[0]);
    } else {
      std::vector<std::thread> pool;
      for (int t = 0; t < parts; ++t)
        pool.emplace_back([&, t] { classify(n * t / parts, n * (t + 1) / parts, outs[t]); });
      for (auto &th : pool) th.join();
    }
    std::vector<std::pair<uint32_t, uint32_t>> next;
    for (auto &o : outs) {
      far.insert(far.end(), o.far.begin(), o.far.end());
      near.insert(near.end(), o.near.begin(), o.near.end());
      next.insert(next.end(), o.next.begin(), o.next.end());
    }
    level.swap(next);
  }
  for (auto [a, c] : near) B.near_entries += a == c ? len(a) * (len(a) - 1) : len(a) * len(c);
  for (auto [a, c] : far) B.far_pairs += len(a) * len(c);
  group(far, nn, B.far_ptr, B.far_col);
  group(near, nn, B.near_ptr, B.near_col);
  return B;
}

}  // namespace rsg
