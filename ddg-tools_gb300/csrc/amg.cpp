// Host setup of the smoothed-aggregation multigrid hierarchy (see amg.hpp).
#include <algorithm>
#include <cmath>
#include <numeric>

#include "amg.hpp"

namespace rsg {

namespace {

Csr transpose(const Csr &A) {
  Csr T;
  T.n = A.m, T.m = A.n;
  T.ptr.assign(T.n + 1, 0);
  for (int c : A.col) T.ptr[c + 1]++;
  for (int i = 0; i < T.n; ++i) T.ptr[i + 1] += T.ptr[i];
  T.col.resize(A.col.size());
  T.val.resize(A.val.size());
  std::vector<int> fill(T.ptr.begin(), T.ptr.end() - 1);
  for (int i = 0; i < A.n; ++i)
    for (int p = A.ptr[i]; p < A.ptr[i + 1]; ++p) {
      int q = fill[A.col[p]]++;
      T.col[q] = i;
      T.val[q] = A.val[p];
    }
  return T;
}

// C = A B (Gustavson, columns sorted), rows in parallel: a pass that counts each row's
// columns, then a pass that fills the rows at their prefix offsets. Every row is formed
// exactly as a sequential pass would form it.
Csr spgemm(const Csr &A, const Csr &B) {
  Csr C;
  C.n = A.n, C.m = B.m;
  C.ptr.assign(C.n + 1, 0);
  parallel_for((size_t)A.n, [&](size_t i0, size_t i1) {
    std::vector<int> mark(B.m, -1);
    for (size_t i = i0; i < i1; ++i) {
      int cnt = 0;
      for (int p = A.ptr[i]; p < A.ptr[i + 1]; ++p) {
        const int k = A.col[p];
        for (int q = B.ptr[k]; q < B.ptr[k + 1]; ++q)
          if (mark[B.col[q]] != (int)i) mark[B.col[q]] = (int)i, ++cnt;
      }
      C.ptr[i + 1] = cnt;
    }
  }, 2048);
  for (int i = 0; i < C.n; ++i) C.ptr[i + 1] += C.ptr[i];
  C.col.resize(C.ptr[C.n]);
  C.val.resize(C.ptr[C.n]);
  parallel_for((size_t)A.n, [&](size_t i0, size_t i1) {
    std::vector<double> acc(B.m, 0.0);
    std::vector<int> mark(B.m, -1), cols;
    for (size_t i = i0; i < i1; ++i) {
      cols.clear();
      for (int p = A.ptr[i]; p < A.ptr[i + 1]; ++p) {
        const int k = A.col[p];
        const double a = A.val[p];
        for (int q = B.ptr[k]; q < B.ptr[k + 1]; ++q) {
          const int j = B.col[q];
          if (mark[j] != (int)i) mark[j] = (int)i, acc[j] = 0.0, cols.push_back(j);
          acc[j] += a * B.val[q];
        }
      }
      std::sort(cols.begin(), cols.end());
      int o = C.ptr[i];
      for (int j : cols) C.col[o] = j, C.val[o] = acc[j], ++o;
    }
  }, 2048);
  return C;
}

std::vector<double> diag(const Csr &A) {
  std::vector<double> d(A.n, 0.0);
  for (int i = 0; i < A.n; ++i)
    for (int p = A.ptr[i]; p < A.ptr[i + 1]; ++p)
      if (A.col[p] == i) d[i] += A.val[p];
  return d;
}

// An upper bound of rho(D^-1 A) (Gershgorin: max_i sum_j |a_ij| / a_ii). A power-iteration
// estimate approaches rho from below, and a damping weight built on an underestimate lets
// the Jacobi sweeps amplify the highest modes of a large mesh.
double spectral_radius(const Csr &A, const std::vector<double> &d) {
  double rho = 0.0;
  for (int i = 0; i < A.n; ++i) {
    double s = 0.0;
    for (int p = A.ptr[i]; p < A.ptr[i + 1]; ++p) s += std::fabs(A.val[p]);
    rho = std::max(rho, s / d[i]);
  }
  return rho > 0.0 ? rho : 1.0;
}

// Aggregates of the strength graph: seeds whose strong neighbourhood is free, then attach
// leftovers to a neighbouring aggregate, then group whatever remains.
std::vector<int> aggregate(const Csr &A, const std::vector<double> &d, int &n_agg) {
  const double theta = 0.08;
  // strong[p]: entry p of A is a strong connection (off the diagonal); computed in parallel,
  // read in A's column order by the sequential greedy passes
  std::vector<unsigned char> strong(A.col.size(), 0);
  parallel_for((size_t)A.n, [&](size_t i0, size_t i1) {
    for (size_t i = i0; i < i1; ++i)
      for (int p = A.ptr[i]; p < A.ptr[i + 1]; ++p) {
        const int j = A.col[p];
        strong[p] = j != (int)i && std::fabs(A.val[p]) >= theta * std::sqrt(std::fabs(d[i] * d[j]));
      }
  });
  std::vector<int> agg(A.n, -1);
  n_agg = 0;
  for (int i = 0; i < A.n; ++i) {
    if (agg[i] != -1) continue;
    bool free_ = true, any = false;
    for (int p = A.ptr[i]; p < A.ptr[i + 1]; ++p)
      if (strong[p]) free_ = free_ && agg[A.col[p]] == -1, any = true;
    if (!free_ || !any) continue;
    agg[i] = n_agg;
    for (int p = A.ptr[i]; p < A.ptr[i + 1]; ++p)
      if (strong[p]) agg[A.col[p]] = n_agg;
    ++n_agg;
  }
  std::vector<int> first = agg;
  for (int i = 0; i < A.n; ++i) {
    if (agg[i] != -1) continue;
    for (int p = A.ptr[i]; p < A.ptr[i + 1]; ++p)
      if (strong[p] && first[A.col[p]] != -1) {
        agg[i] = first[A.col[p]];
        break;
      }
  }
  for (int i = 0; i < A.n; ++i) {
    if (agg[i] != -1) continue;
    agg[i] = n_agg;
    for (int p = A.ptr[i]; p < A.ptr[i + 1]; ++p)
      if (strong[p] && agg[A.col[p]] == -1) agg[A.col[p]] = n_agg;
    ++n_agg;
  }
  return agg;
}

// Dense Cholesky inverse of an SPD matrix (row-major, n x n).
std::vector<double> dense_inverse(std::vector<double> a, int n) {
  for (int k = 0; k < n; ++k) {
    double s = a[(size_t)k * n + k];
    for (int p = 0; p < k; ++p) s -= a[(size_t)k * n + p] * a[(size_t)k * n + p];
    if (!(s > 0.0)) fail(RS_SINGULAR, "SingularSaddle", "preconditioner", "coarse multigrid operator is not positive definite");
    double l = std::sqrt(s);
    a[(size_t)k * n + k] = l;
    for (int i = k + 1; i < n; ++i) {
      double t = a[(size_t)i * n + k];
      for (int p = 0; p < k; ++p) t -= a[(size_t)i * n + p] * a[(size_t)k * n + p];
      a[(size_t)i * n + k] = t / l;
    }
  }
  std::vector<double> inv((size_t)n * n, 0.0), col(n);
  for (int c = 0; c < n; ++c) {
    for (int i = 0; i < n; ++i) {  // L y = e_c
      double t = (i == c) ? 1.0 : 0.0;
      for (int p = 0; p < i; ++p) t -= a[(size_t)i * n + p] * col[p];
      col[i] = t / a[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {  // L^T x = y
      double t = col[i];
      for (int p = i + 1; p < n; ++p) t -= a[(size_t)p * n + i] * col[p];
      col[i] = t / a[(size_t)i * n + i];
    }
    for (int i = 0; i < n; ++i) inv[(size_t)i * n + c] = col[i];
  }
  return inv;
}

}  // namespace

AmgHost amg_setup(const Csr &A0, int coarse_max, int max_levels, const std::vector<uint32_t> *groups) {
  AmgHost H;
  H.A.push_back(A0);
  std::vector<double> z(A0.n, 1.0);  // near-null vector (constants)
  // the group of every node (aggregates never join unconnected rows, so an aggregate lies in
  // one group when the groups are connected components)
  std::vector<uint32_t> gid = groups ? *groups : std::vector<uint32_t>(A0.n, 0u);
  while ((int)H.A.size() < max_levels && H.A.back().n > coarse_max) {
    const Csr &A = H.A.back();
    std::vector<double> d = diag(A);
    for (double &x : d)
      if (!(x > 0.0)) fail(RS_SINGULAR, "SingularSaddle", "preconditioner", "non-positive Laplacian diagonal");
    int na = 0;
    std::vector<int> agg = aggregate(A, d, na);
    if (na >= A.n) break;
    // tentative prolongator interpolating z exactly
    std::vector<double> zn(na, 0.0);
    for (int i = 0; i < A.n; ++i) zn[agg[i]] += z[i] * z[i];
    for (double &x : zn) x = std::sqrt(x);
    Csr Pt;
    Pt.n = A.n, Pt.m = na;
    Pt.ptr.resize(A.n + 1);
    for (int i = 0; i < A.n; ++i) {
      Pt.ptr[i] = i;
      Pt.col.push_back(agg[i]);
      Pt.val.push_back(zn[agg[i]] > 0.0 ? z[i] / zn[agg[i]] : 0.0);
    }
    Pt.ptr[A.n] = A.n;
    // P = (I - omega D^-1 A) Pt
    double rho = spectral_radius(A, d);
    double omega = 4.0 / (3.0 * rho);
    Csr AP = spgemm(A, Pt);
    Csr P;
    P.n = A.n, P.m = na;
    P.ptr.assign(A.n + 1, 0);
    // merge the Pt row (one entry) with the -omega/d_i AP row: the row has AP's columns plus
    // Pt's when AP lacks it
    parallel_for((size_t)A.n, [&](size_t i0, size_t i1) {
      for (size_t i = i0; i < i1; ++i) {
        const int pc = Pt.col[i];
        const int *b = AP.col.data() + AP.ptr[i], *e = AP.col.data() + AP.ptr[i + 1];
        P.ptr[i + 1] = (int)(e - b) + (std::binary_search(b, e, pc) ? 0 : 1);
      }
    });
    for (int i = 0; i < A.n; ++i) P.ptr[i + 1] += P.ptr[i];
    P.col.resize(P.ptr[A.n]);
    P.val.resize(P.ptr[A.n]);
    parallel_for((size_t)A.n, [&](size_t i0, size_t i1) {
      for (size_t i = i0; i < i1; ++i) {
        const int pc = Pt.col[i];
        const double pv = Pt.val[i];
        int o = P.ptr[i];
        bool done = false;
        for (int q = AP.ptr[i]; q < AP.ptr[i + 1]; ++q) {
          const int j = AP.col[q];
          double v = -omega / d[i] * AP.val[q];
          if (!done && pc < j) P.col[o] = pc, P.val[o] = pv, ++o, done = true;
          if (j == pc) v += pv, done = true;
          P.col[o] = j, P.val[o] = v, ++o;
        }
        if (!done) P.col[o] = pc, P.val[o] = pv;
      }
    });
    Csr R = transpose(P);
    Csr Ac = spgemm(R, spgemm(A, P));
    std::vector<double> dinv(A.n);
    for (int i = 0; i < A.n; ++i) dinv[i] = 4.0 / (3.0 * rho * d[i]);  // damped Jacobi
    H.dinv.push_back(dinv);
    H.P.push_back(P);
    H.R.push_back(R);
    // (A refers into H.A: read it before the push_back below)
    std::vector<uint32_t> gc(na, 0u);
    for (int i = 0; i < A.n; ++i) gc[agg[i]] = gid[i];
    gid.swap(gc);
    H.A.push_back(Ac);
    z = zn;
  }
  // coarsest level: dense inverse of A_L + (tr A_L / n) sum_g zhat_g zhat_g^T, the constant of
  // every group g regularised (one group: the global constant)
  const Csr &Ac = H.A.back();
  int n = Ac.n;
  {
    std::vector<double> d = diag(Ac);
    double rho = n > 0 ? spectral_radius(Ac, d) : 1.0;
    std::vector<double> dinv(n);
    for (int i = 0; i < n; ++i) dinv[i] = 4.0 / (3.0 * rho * d[i]);
    H.dinv.push_back(dinv);
  }
  std::vector<double> dense((size_t)n * n, 0.0);
  double tr = 0.0;
  for (int i = 0; i < n; ++i)
    for (int p = Ac.ptr[i]; p < Ac.ptr[i + 1]; ++p) {
      dense[(size_t)i * n + Ac.col[p]] += Ac.val[p];
      if (Ac.col[p] == i) tr += Ac.val[p];
    }
  uint32_t ng = 0;
  for (uint32_t g : gid) ng = std::max(ng, g + 1);
  std::vector<double> zz(ng, 0.0);
  for (int i = 0; i < n; ++i) zz[gid[i]] += z[i] * z[i];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      if (gid[i] == gid[j]) dense[(size_t)i * n + j] += (tr / std::max(n, 1)) / std::max(zz[gid[i]], 1e-300) * z[i] * z[j];
  H.coarse_inv = dense_inverse(dense, n);
  return H;
}

}  // namespace rsg
