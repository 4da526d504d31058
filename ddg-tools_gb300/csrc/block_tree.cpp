// Block classification of the block cluster tree (see block_tree.hpp). Level by level, worker
// threads classify contiguous slices of the level's pairs; the slices' outputs are kept in
// slice order (never concatenated), so the blocks come out in exactly the sequential level
// order. The CSR grouping by row node is a parallel stable counting sort of that sequence, so
// every row keeps its level order too.
#include "block_tree.hpp"

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>

namespace rsg {

namespace {

// What the classification reads of a node, in one cache line.
struct alignas(64) NodeRec {
  double box[6];  // min xyz, max xyz
  double radius;
  uint32_t right;  // 0 for a leaf
  uint32_t len;    // elements
};

// box_distance_sq (RS/src/spatial/mod.rs:131-138) and separated (hierarchical.rs:116-123).
// The boxes and radii are finite, so plain comparisons give fmax / fmin's values (a zero's
// sign aside, which the squares remove).
inline double mx(double a, double b) { return a < b ? b : a; }
inline double mn(double a, double b) { return b < a ? b : a; }
inline bool separated(const NodeRec &A, const NodeRec &B, double chi) {
  if (!(chi > 0.0)) return false;
  double d2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    double d = mx(mx(A.box[k], B.box[k]) - mn(A.box[3 + k], B.box[3 + k]), 0.0);
    d2 += d * d;
  }
  double h = mx(A.radius, B.radius);
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
  // calls f(pair) for the elements [b, e) in order, and ahead(pair) for the element kAhead
  // positions further on within the same slice (to prefetch what f will read)
  template <class F, class A>
  void each(size_t b, size_t e, F f, A ahead) const {
    constexpr size_t kAhead = 16;
    size_t s = std::upper_bound(off.begin(), off.end(), b) - off.begin() - 1;
    for (size_t i = b; i < e; ++s) {
      const std::vector<Pair> &x = v[s];
      for (size_t j = i - off[s]; j < x.size() && i < e; ++j, ++i) {
        if (j + kAhead < x.size()) ahead(x[j + kAhead]);
        f(x[j]);
      }
    }
  }
};

// CSR by row (pair.first) of the levels' pairs in order, a stable counting sort: the ordered
// sequence of all slices is cut into nt contiguous parts; each part counts its rows, every
// part's write offset per row follows from the counts (row start + the counts of the parts
// before it), and each part scatters its pairs in order. `weight(pair)` is summed on the way.
template <class Wt>
void group(const std::vector<Slices> &levels, size_t n, Workers &W, int nt, std::vector<uint32_t> &ptr,
           std::vector<uint32_t> &col, Wt weight, uint64_t &total) {
  std::vector<const std::vector<Pair> *> sl;
  std::vector<size_t> off{0};
  for (const Slices &L : levels)
    for (const auto &s : L.v) sl.push_back(&s), off.push_back(off.back() + s.size());
  const size_t m = off.back();
  auto range = [&](int t, auto f) {  // f(pair) over part t in order
    const size_t b = m * t / nt, e = m * (t + 1) / nt;
    size_t s = std::upper_bound(off.begin(), off.end(), b) - off.begin() - 1;
    for (size_t i = b; i < e; ++s)
      for (size_t j = i - off[s]; j < sl[s]->size() && i < e; ++j, ++i) f((*sl[s])[j]);
  };
  std::vector<std::vector<uint32_t>> cnt(nt);
  std::vector<uint64_t> tot(nt, 0);
  W.run(nt, [&](int t) {
    std::vector<uint32_t> &c = cnt[t];
    c.assign(n, 0);
    uint64_t w = 0;
    range(t, [&](const Pair &p) { ++c[p.first], w += weight(p); });
    tot[t] = w;
  });
  total = 0;
  for (uint64_t w : tot) total += w;
  ptr.assign(n + 1, 0);
  W.run(nt, [&](int t) {  // rows split over the workers: row sums, then per-part offsets
    for (size_t r = n * t / nt; r < n * (t + 1) / nt; ++r) {
      uint32_t sum = 0;
      for (int k = 0; k < nt; ++k) sum += cnt[k][r];
      ptr[r + 1] = sum;
    }
  });
  for (size_t r = 0; r < n; ++r) ptr[r + 1] += ptr[r];
  W.run(nt, [&](int t) {
    for (size_t r = n * t / nt; r < n * (t + 1) / nt; ++r) {
      uint32_t o = ptr[r];
      for (int k = 0; k < nt; ++k) {
        const uint32_t c = cnt[k][r];
        cnt[k][r] = o;
        o += c;
      }
    }
  });
  col.resize(ptr[n]);
  W.run(nt, [&](int t) {
    std::vector<uint32_t> &o = cnt[t];
    range(t, [&](const Pair &p) { col[o[p.first]++] = p.second; });
  });
}

}  // namespace

Blocks classify_blocks(const Tree &T, double chi, size_t leaf_pairs, int threads) {
  const size_t nn = T.n_nodes();
  auto len = [&](uint32_t a) { return (size_t)(T.end[a] - T.start[a]); };
  const int nt = threads > 0 ? threads : (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  Workers W(nt);
  std::vector<NodeRec> rec(nn);
  W.run(nt, [&](int t) {
    for (size_t a = nn * t / nt; a < nn * (t + 1) / nt; ++a) {
      NodeRec &r = rec[a];
      for (int k = 0; k < 6; ++k) r.box[k] = T.box[6 * a + k];
      r.radius = T.radius[a], r.right = T.right[a], r.len = T.end[a] - T.start[a];
    }
  });
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
      // branch-free: every pair's far and near entries and its (up to four) children are
      // written at the current ends and the ends advance by the pair's class; the buffers hold
      // the worst case (one far or near entry, four children per pair)
      const size_t b = n * t / parts, e = n * (t + 1) / parts;
      std::vector<Pair> &fa = of[t], &ne = on[t], &nx = ox[t];
      fa.resize(e - b), ne.resize(e - b), nx.resize(4 * (e - b));
      Pair *pf = fa.data(), *pn = ne.data(), *px = nx.data();
      level.each(b, e, [&](const Pair &pr) {
        const uint32_t a = pr.first, c = pr.second;
        const NodeRec &A = rec[a], &Cn = rec[c];
        const bool la = A.right == 0, lc = Cn.right == 0;
        const bool far_ = a != c && separated(A, Cn, chi);
        const bool near_ = !far_ && ((la && lc) || (size_t)A.len * Cn.len <= leaf_pairs);
        const bool split = !far_ && !near_;
        *pf = pr, pf += far_;
        *pn = pr, pn += near_;
        // children (x, y) for x < na, y < nc in order; na = 1 or nc = 1 gives two of them
        const uint32_t a0 = la ? a : a + 1, a1 = A.right, c0 = lc ? c : c + 1, c1 = Cn.right;
        px[0] = {a0, c0};
        px[1] = lc ? Pair{a1, c0} : Pair{a0, c1};
        px[2] = {a1, c0};
        px[3] = {a1, c1};
        px += split ? (la || lc ? 2 : 4) : 0;
      }, [&](const Pair &pr) {
        __builtin_prefetch(&rec[pr.first]);
        __builtin_prefetch(&rec[pr.second]);
      });
      fa.resize(pf - fa.data()), ne.resize(pn - ne.data()), nx.resize(px - nx.data());
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
  uint64_t fp = 0, ne = 0;
  group(far, nn, W, nt, B.far_ptr, B.far_col, [&](const Pair &p) { return (uint64_t)len(p.first) * len(p.second); }, fp);
  group(near, nn, W, nt, B.near_ptr, B.near_col, [&](const Pair &p) {
    return p.first == p.second ? (uint64_t)len(p.first) * (len(p.first) - 1) : (uint64_t)len(p.first) * len(p.second);
  }, ne);
  B.far_pairs = fp, B.near_entries = ne;
  return B;
}

}  // namespace rsg
