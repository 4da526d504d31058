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

// C = A B (Gustavson, rows in order, columns sorted).
Csr spgemm(const Csr &A, const Csr &B) {
  Csr C;
  C.n = A.n, C.m = B.m;
  C.ptr.assign(C.n + 1, 0);
  std::vector<double> acc(B.m, 0.0);
  std::vector<int> mark(B.m, -1), cols;
  for (int i = 0; i < A.n; ++i) {
    cols.clear();
    for (int p = A.ptr[i]; p < A.ptr[i + 1]; ++p) {
      int k = A.col[p];
      double a = A.val[p];
      for (int q = B.ptr[k]; q < B.ptr[k + 1]; ++q) {
        int j = B.col[q];
        if (mark[j] != i) mark[j] = i, acc[j] = 0.0, cols.push_back(j);
        acc[j] += a * B.val[q];
      }
    }
    std::sort(cols.begin(), cols.end());
    for (int j : cols) C.col.push_back(j), C.val.push_back(acc[j]);
    C.ptr[i + 1] = (int)C.col.size();
  }
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
  std::vector<std::vector<int>> S(A.n);
  for (int i = 0; i < A.n; ++i)
    for (int p = A.ptr[i]; p < A.ptr[i + 1]; ++p) {
      int j = A.col[p];
      if (j != i && std::fabs(A.val[p]) >= theta * std::sqrt(std::fabs(d[i] * d[j]))) S[i].push_back(j);
    }
  std::vector<int> agg(A.n, -1);
  n_agg = 0;
  for (int i = 0; i < A.n; ++i) {
    if (agg[i] != -1) continue;
    bool free_ = true;
    for (int j : S[i]) free_ = free_ && agg[j] == -1;
    if (!free_ || S[i].empty()) continue;
    agg[i] = n_agg;
    for (int j : S[i]) agg[j] = n_agg;
    ++n_agg;
  }
  std::vector<int> first = agg;
  for (int i = 0; i < A.n; ++i) {
    if (agg[i] != -1) continue;
    for (int j : S[i])
      if (first[j] != -1) {
        agg[i] = first[j];
        break;
      }
  }
  for (int i = 0; i < A.n; ++i) {
    if (agg[i] != -1) continue;
    agg[i] = n_agg;
    for (int j : S[i])
      if (agg[j] == -1) agg[j] = n_agg;
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

AmgHost amg_setup(const Csr &A0, int coarse_max, int max_levels) {
  AmgHost H;
  H.A.push_back(A0);
  std::vector<double> z(A0.n, 1.0);  // near-null vector (constants)
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
    for (int i = 0; i < A.n; ++i) {
      // merge Pt row (one entry) with -omega/d_i AP row
      int pc = Pt.col[i];
      double pv = Pt.val[i];
      bool done = false;
      for (int q = AP.ptr[i]; q < AP.ptr[i + 1]; ++q) {
        int j = AP.col[q];
        double v = -omega / d[i] * AP.val[q];
        if (!done && pc < j) P.col.push_back(pc), P.val.push_back(pv), done = true;
        if (j == pc) v += pv, done = true;
        P.col.push_back(j), P.val.push_back(v);
      }
      if (!done) P.col.push_back(pc), P.val.push_back(pv);
      P.ptr[i + 1] = (int)P.col.size();
    }
    Csr R = transpose(P);
    Csr Ac = spgemm(R, spgemm(A, P));
    std::vector<double> dinv(A.n);
    for (int i = 0; i < A.n; ++i) dinv[i] = 4.0 / (3.0 * rho * d[i]);  // damped Jacobi
    H.dinv.push_back(dinv);
    H.P.push_back(P);
    H.R.push_back(R);
    H.A.push_back(Ac);
    z = zn;
  }
  // coarsest level: dense inverse of A_L + (tr A_L / n) zhat zhat^T
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
  double zz = 0.0;
  for (double v : z) zz += v * v;
  double sc = (tr / std::max(n, 1)) / std::max(zz, 1e-300);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) dense[(size_t)i * n + j] += sc * z[i] * z[j];
  H.coarse_inv = dense_inverse(dense, n);
  return H;
}

}  // namespace rsg
