// Block classification of the block cluster tree (see block_tree.hpp). Level by level, worker
// threads classify contiguous slices of the level's pairs; the slices' outputs are kept in
// slice order (never concatenated), so the blocks come out in exactly the sequential level
// order. The CSR grouping by row node is split by row ranges: each worker owns a range of rows
// and reads the slices in order, so every row keeps its level order too.
#include "block_tree.hpp"

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>

namespace rsg {

namespace {

// box_distance_sq (RS/src/spatial/mod.rs:131-138) and separated (hierarchical.rs:116-123).
// The boxes and radii are finite, so plain comparisons give fmax / fmin's values (a zero's
// sign aside, which the squares remove).
inline double mx(double a, double b) { return a < b ? b : a; }
inline double mn(double a, double b) { return b < a ? b : a; }
inline bool separated(const Tree &T, uint32_t a, uint32_t b, double chi) {
  if (!(chi > 0.0)) return false;
  const double *ba = &T.box[6 * (size_t)a], *bb = &T.box[6 * (size_t)b];
  double d2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    double d = mx(mx(ba[k], bb[k]) - mn(ba[3 + k], bb[3 + k]), 0.0);
    d2 += d * d;
  }
  double h = mx(T.radius[a], T.radius[b]);
  return d2 > 0.0 && h * h <= chi * chi * d2;
}

using Pair = std::pair<uint32_t, uint32_t>;

// Workers that live for one classification: run(parts, f) calls f(0 .. parts-1), part 0 on
// the calling thread, and returns when all parts are done.
class Workers {
 public:
  explicit Workers(int n) : n_(n) {
    for (int i = 1; i < n; ++i) th_.emplace_back([this, i] { loop(i); });
  }
  ~Workers() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto &t : th_) t.join();
  }
  void run(int parts, const std::function<void(int)> &f) {
    parts = std::min(parts, n_);
    if (parts <= 1) {
      f(0);
      return;
    }
    {
      std::lock_guard<std::mutex> g(m_);
      job_ = &f, parts_ = parts, pending_ = parts - 1, ++gen_;
    }
    cv_.notify_all();
    f(0);
    std::unique_lock<std::mutex> g(m_);
    done_.wait(g, [this] { return pending_ == 0; });
  }

 private:
  void loop(int i) {
    uint64_t seen = 0;
    for (;;) {
      const std::function<void(int)> *f;
      int parts;
      {
        std::unique_lock<std::mutex> g(m_);
        cv_.wait(g, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_, f = job_, parts = parts_;
      }
      if (i < parts) {
        (*f)(i);
        std::lock_guard<std::mutex> g(m_);
        if (--pending_ == 0) done_.notify_one();
      }
    }
  }
  int n_;
  std::vector<std::thread> th_;
  std::mutex m_;
  std::condition_variable cv_, done_;
  const std::function<void(int)> *job_ = nullptr;
  int parts_ = 0, pending_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// Slices of one sequence: element i of the whole lies in slice s with off[s] <= i < off[s+1].
struct Slices {
  std::vector<std::vector<Pair>> v;
  std::vector<size_t> off{0};
  void add(std::vector<Pair> &&s) {
    off.push_back(off.back() + s.size());
    v.push_back(std::move(s));
  }
  size_t size() const { return off.back(); }
  // calls f(pair) for the elements [b, e) in order
  template <class F>
  void each(size_t b, size_t e, F f) const {
    size_t s = std::upper_bound(off.begin(), off.end(), b) - off.begin() - 1;
    for (size_t i = b; i < e; ++s)
      for (size_t j = i - off[s]; j < v[s].size() && i < e; ++j, ++i) f(v[s][j]);
  }
};

// CSR by row (pair.first) of the levels' pairs in order: counts per row range, then each
// worker fills its rows (a range balanced by entries) from all slices in order.
void group(const std::vector<Slices> &levels, size_t n, Workers &W, int nt, std::vector<uint32_t> &ptr,
           std::vector<uint32_t> &col) {
  ptr.assign(n + 1, 0);
  W.run(nt, [&](int t) {
    const size_t r0 = n * t / nt, r1 = n * (t + 1) / nt;
    for (const Slices &L : levels)
      for (const auto &s : L.v)
        for (const Pair &p : s)
          if (p.first >= r0 && p.first < r1) ptr[p.first + 1]++;
  });
  for (size_t i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
  col.resize(ptr[n]);
  // row ranges balanced by entries
  std::vector<size_t> cut(nt + 1, n);
  cut[0] = 0;
  for (int t = 1; t < nt; ++t)
    cut[t] = std::lower_bound(ptr.begin(), ptr.end(), (uint32_t)((uint64_t)ptr[n] * t / nt)) - ptr.begin();
  for (int t = 1; t <= nt; ++t) cut[t] = std::max(cut[t], cut[t - 1]);
  W.run(nt, [&](int t) {
    const size_t r0 = cut[t], r1 = cut[t + 1];
    if (r0 >= r1) return;
    std::vector<uint32_t> fill(ptr.begin() + r0, ptr.begin() + r1);
    for (const Slices &L : levels)
      for (const auto &s : L.v)
        for (const Pair &p : s)
          if (p.first >= r0 && p.first < r1) col[fill[p.first - r0]++] = p.second;
  });
}

}  // namespace

Blocks classify_blocks(const Tree &T, double chi, size_t leaf_pairs, int threads) {
  const size_t nn = T.n_nodes();
  auto leaf = [&](uint32_t a) { return T.right[a] == 0; };
  auto len = [&](uint32_t a) { return (size_t)(T.end[a] - T.start[a]); };
  const int nt = threads > 0 ? threads : (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  Workers W(nt);
  Blocks B;
  std::vector<Slices> far, near;
  Slices level;
  level.add({{0, 0}});
  while (level.size() > 0) {
    ++B.depth;
    const size_t n = level.size();
    const int parts = (n < 4096) ? 1 : nt;
    std::vector<std::vector<Pair>> of(parts), on(parts), ox(parts);
    W.run(parts, [&](int t) {
      std::vector<Pair> &fa = of[t], &ne = on[t], &nx = ox[t];
      level.each(n * t / parts, n * (t + 1) / parts, [&](const Pair &pr) {
        const uint32_t a = pr.first, c = pr.second;
        if (a != c && separated(T, a, c, chi))
          fa.push_back(pr);
        else if ((leaf(a) && leaf(c)) || len(a) * len(c) <= leaf_pairs)
          ne.push_back(pr);
        else {
          uint32_t ka[2] = {leaf(a) ? a : a + 1, T.right[a]};
          uint32_t kc[2] = {leaf(c) ? c : c + 1, T.right[c]};
          int na = leaf(a) ? 1 : 2, nc = leaf(c) ? 1 : 2;
          for (int x = 0; x < na; ++x)
            for (int y = 0; y < nc; ++y) nx.push_back({ka[x], kc[y]});
        }
      });
    });
    Slices fl, nl, next;
    for (int t = 0; t < parts; ++t) {
      fl.add(std::move(of[t]));
      nl.add(std::move(on[t]));
      next.add(std::move(ox[t]));
    }
    far.push_back(std::move(fl));
    near.push_back(std::move(nl));
    level = std::move(next);
  }
  for (const Slices &L : near)
    for (const auto &s : L.v)
      for (auto [a, c] : s) B.near_entries += a == c ? len(a) * (len(a) - 1) : len(a) * len(c);
  for (const Slices &L : far)
    for (const auto &s : L.v)
      for (auto [a, c] : s) B.far_pairs += len(a) * len(c);
  group(far, nn, W, nt, B.far_ptr, B.far_col);
  group(near, nn, W, nt, B.near_ptr, B.near_col);
  return B;
}

}  // namespace rsg
