// CPU restatement of the block-preconditioned GMRES(m) linear solve that replaces the
// AMGCL call of the reference's implicit solver (src/CoefficientMatrix.cpp:210-325 of
// joel-ho/BES).  TEST INFRASTRUCTURE ONLY: it is the checker for the library's GPU
// solver and the linear solve of the patched reference build; nothing in the product links it.
//
// The system is the reference's 5x5-block matrix (one block row per cell, the diagonal
// block plus one block per face neighbour).  Two preconditioners:
//   * block Jacobi: M = blockdiag(A_ii), applied as inv(A_ii) per cell;
//   * block ILU(0): the incomplete factorisation restricted to A's block pattern, computed
//     row by row in a caller-given cell order (IKJ variant).  The GPU processes the same
//     order colour by colour, which is the same sequence of row operations.
// GMRES is right preconditioned, restarted every m iterations, x0 = 0, classical
// Gram-Schmidt with a second (re-orthogonalisation) pass only where the first one cancelled
// most of the new vector (see kReorthTheta2), Givens rotations, and the stopping test
// |g_{j+1}| <= tol*|b| of AMGCL's gmres.hpp:163,214 (tol is relative, which is what the
// reference's LINEAR_SOLVER_ABS_TOL key really sets).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace besla {

constexpr int NB = 5;             // block size: 5 conserved variables
constexpr int NB2 = NB * NB;
// Second Gram-Schmidt pass when |w - V h|^2 <= kReorthTheta2 |w|^2, i.e. when the first pass
// cancelled 3/4 or more of |w| (two or more leading bits).
constexpr double kReorthTheta2 = 1.0 / 16.0;

// Block CSR: block row i owns blocks [row[i], row[i+1]); col[k] is the block column.
struct BlockCsr {
  int64_t n = 0;
  std::vector<int64_t> row;
  std::vector<int64_t> col;
  std::vector<double> val;  // row-major 5x5 per block
  std::vector<int64_t> diag;  // index of the diagonal block of each row
};

inline void mat5_inverse(const double* a, double* inv) {
  // Gauss-Jordan elimination with partial pivoting on a 5x5 block.
  double m[NB][2 * NB];
  for (int i = 0; i < NB; ++i)
    for (int j = 0; j < NB; ++j) {
      m[i][j] = a[i * NB + j];
      m[i][NB + j] = (i == j) ? 1.0 : 0.0;
    }
  for (int c = 0; c < NB; ++c) {
    int p = c;
    for (int r = c + 1; r < NB; ++r)
      if (std::fabs(m[r][c]) > std::fabs(m[p][c])) p = r;
    if (p != c)
      for (int j = 0; j < 2 * NB; ++j) std::swap(m[p][j], m[c][j]);
    const double piv = 1.0 / m[c][c];
    for (int j = 0; j < 2 * NB; ++j) m[c][j] *= piv;
    for (int r = 0; r < NB; ++r) {
      if (r == c) continue;
      const double f = m[r][c];
      if (f == 0.0) continue;
      for (int j = 0; j < 2 * NB; ++j) m[r][j] -= f * m[c][j];
    }
  }
  for (int i = 0; i < NB; ++i)
    for (int j = 0; j < NB; ++j) inv[i * NB + j] = m[i][NB + j];
}

inline void mat5_mul(const double* a, const double* b, double* c) {
  for (int i = 0; i < NB; ++i)
    for (int j = 0; j < NB; ++j) {
      double s = 0.0;
      for (int k = 0; k < NB; ++k) s += a[i * NB + k] * b[k * NB + j];
      c[i * NB + j] = s;
    }
}

inline void mat5_vec(const double* a, const double* x, double* y) {
  for (int i = 0; i < NB; ++i) {
    double s = 0.0;
    for (int k = 0; k < NB; ++k) s += a[i * NB + k] * x[k];
    y[i] = s;
  }
}

inline void bcsr_spmv(const BlockCsr& A, const double* x, double* y) {
  for (int64_t i = 0; i < A.n; ++i) {
    double acc[NB] = {0, 0, 0, 0, 0};
    for (int64_t k = A.row[i]; k < A.row[i + 1]; ++k) {
      double t[NB];
      mat5_vec(&A.val[k * NB2], &x[A.col[k] * NB], t);
      for (int r = 0; r < NB; ++r) acc[r] += t[r];
    }
    for (int r = 0; r < NB; ++r) y[i * NB + r] = acc[r];
  }
}

struct Preconditioner {
  int kind = 0;  // 0 block Jacobi, 1 block ILU(0)
  int64_t n = 0;
  std::vector<double> dinv;      // inverse of the (factorised) diagonal blocks
  BlockCsr lu;                   // ILU(0) factors in A's pattern (unit-lower L, U)
  std::vector<int64_t> order;    // factorisation order (position -> cell)
  std::vector<int64_t> pos;      // cell -> position

  void setup_jacobi(const BlockCsr& A) {
    kind = 0;
    n = A.n;
    dinv.assign(n * NB2, 0.0);
    for (int64_t i = 0; i < n; ++i) mat5_inverse(&A.val[A.diag[i] * NB2], &dinv[i * NB2]);
  }

  // IKJ block ILU(0) in the given order: for row i (in order), for each block (i,j) with
  // pos[j] < pos[i] taken in increasing pos[j]: L_ij = A_ij * inv(U_jj); then for every
  // block (i,k) of row i with pos[k] > pos[j] that also exists in row j: A_ik -= L_ij*U_jk.
  std::vector<int64_t> dom;       // optional subdomain id per cell: couplings between
                                  // subdomains are dropped (block Jacobi over subdomains)
  bool same(int64_t a, int64_t b) const { return dom.empty() || dom[a] == dom[b]; }

  void setup_ilu0(const BlockCsr& A, const std::vector<int64_t>& ord) {
    kind = 1;
    n = A.n;
    lu = A;
    order = ord;
    pos.assign(n, 0);
    for (int64_t p = 0; p < n; ++p) pos[order[p]] = p;
    dinv.assign(n * NB2, 0.0);
    std::vector<int64_t> lookup(n, -1);
    for (int64_t p = 0; p < n; ++p) {
      const int64_t i = order[p];
      const int64_t b0 = lu.row[i], b1 = lu.row[i + 1];
      for (int64_t k = b0; k < b1; ++k) lookup[lu.col[k]] = k;
      // lower blocks sorted by factorisation position
      std::vector<int64_t> lower;
      for (int64_t k = b0; k < b1; ++k)
        if (pos[lu.col[k]] < p && same(i, lu.col[k])) lower.push_back(k);
      for (size_t a = 1; a < lower.size(); ++a)
        for (size_t b = a; b > 0 && pos[lu.col[lower[b]]] < pos[lu.col[lower[b - 1]]]; --b)
          std::swap(lower[b], lower[b - 1]);
      for (int64_t kl : lower) {
        const int64_t j = lu.col[kl];
        double lij[NB2];
        mat5_mul(&lu.val[kl * NB2], &dinv[j * NB2], lij);
        std::memcpy(&lu.val[kl * NB2], lij, sizeof(lij));
        for (int64_t kj = lu.row[j]; kj < lu.row[j + 1]; ++kj) {
          const int64_t c = lu.col[kj];
          if (pos[c] <= pos[j] || !same(j, c)) continue;  // only U part of row j
          const int64_t ki = lookup[c];
          if (ki < 0) continue;  // outside the pattern of row i: dropped (zero fill)
          double t[NB2];
          mat5_mul(lij, &lu.val[kj * NB2], t);
          for (int q = 0; q < NB2; ++q) lu.val[ki * NB2 + q] -= t[q];
        }
      }
      mat5_inverse(&lu.val[lu.diag[i] * NB2], &dinv[i * NB2]);
      for (int64_t k = b0; k < b1; ++k) lookup[lu.col[k]] = -1;
    }
  }

  // z = M^{-1} r
  void apply(const double* r, double* z) const {
    if (kind == 0) {
      for (int64_t i = 0; i < n; ++i) mat5_vec(&dinv[i * NB2], &r[i * NB], &z[i * NB]);
      return;
    }
    // forward: y_i = r_i - sum_{pos j < pos i} L_ij y_j (unit lower)
    std::vector<double> y(n * NB);
    for (int64_t p = 0; p < n; ++p) {
      const int64_t i = order[p];
      double acc[NB];
      for (int q = 0; q < NB; ++q) acc[q] = r[i * NB + q];
      for (int64_t k = lu.row[i]; k < lu.row[i + 1]; ++k) {
        const int64_t j = lu.col[k];
        if (pos[j] >= p || !same(i, j)) continue;
        double t[NB];
        mat5_vec(&lu.val[k * NB2], &y[j * NB], t);
        for (int q = 0; q < NB; ++q) acc[q] -= t[q];
      }
      for (int q = 0; q < NB; ++q) y[i * NB + q] = acc[q];
    }
    // backward: z_i = inv(U_ii) (y_i - sum_{pos j > pos i} U_ij z_j)
    for (int64_t p = n - 1; p >= 0; --p) {
      const int64_t i = order[p];
      double acc[NB];
      for (int q = 0; q < NB; ++q) acc[q] = y[i * NB + q];
      for (int64_t k = lu.row[i]; k < lu.row[i + 1]; ++k) {
        const int64_t j = lu.col[k];
        if (pos[j] <= p || !same(i, j)) continue;
        double t[NB];
        mat5_vec(&lu.val[k * NB2], &z[j * NB], t);
        for (int q = 0; q < NB; ++q) acc[q] -= t[q];
      }
      mat5_vec(&dinv[i * NB2], acc, &z[i * NB]);
    }
  }
};

inline double dot(const double* a, const double* b, int64_t n) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

struct GmresResult {
  int iterations = 0;
  double rel_residual = 0.0;
};

// Right-preconditioned restarted GMRES, x0 = 0.
inline GmresResult gmres(const BlockCsr& A, const Preconditioner& M, const double* b,
                         double* x, int restart, int maxiter, double tol) {
  const int64_t N = A.n * NB;
  std::vector<double> V((int64_t)(restart + 1) * N), Z(N), W(N), r(N);
  std::vector<double> H((restart + 1) * restart), cs(restart), sn(restart), g(restart + 1);
  for (int64_t q = 0; q < N; ++q) x[q] = 0.0;
  const double norm_b = std::sqrt(dot(b, b, N));
  GmresResult res;
  if (norm_b == 0.0) return res;
  const double eps = tol * norm_b;
  int iter = 0;
  double norm_r = norm_b;
  for (int64_t q = 0; q < N; ++q) r[q] = b[q];
  while (true) {
    double beta = std::sqrt(dot(r.data(), r.data(), N));
    norm_r = beta;
    if (beta < eps || iter >= maxiter) break;
    for (int64_t q = 0; q < N; ++q) V[q] = r[q] / beta;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    for (; j < restart && iter < maxiter; ++j, ++iter) {
      M.apply(&V[(int64_t)j * N], Z.data());
      bcsr_spmv(A, Z.data(), W.data());
      // classical Gram-Schmidt: h = V^T w, w -= V h; the norm of the result follows from
      // Pythagoras, |w - V h|^2 = |w|^2 - |h|^2, unless that estimate shows that more than
      // 1 - sqrt(kReorthTheta2) of |w| cancelled, in which case a second pass orthogonalises
      // again and the norm comes from the second pass's own Pythagoras step
      std::vector<double> h(j + 1), h2(j + 1, 0.0);
      for (int i = 0; i <= j; ++i) h[i] = dot(&V[(int64_t)i * N], W.data(), N);
      const double nw2 = dot(W.data(), W.data(), N);
      double s1 = 0.0;
      for (int i = 0; i <= j; ++i) s1 += h[i] * h[i];
      const double est = nw2 - s1;
      const bool reorth = !(est > kReorthTheta2 * nw2);
      for (int i = 0; i <= j; ++i) {
        const double* vi = &V[(int64_t)i * N];
        for (int64_t q = 0; q < N; ++q) W[q] -= h[i] * vi[q];
      }
      double hn = 0.0;
      if (reorth) {
        for (int i = 0; i <= j; ++i) h2[i] = dot(&V[(int64_t)i * N], W.data(), N);
        const double nw2b = dot(W.data(), W.data(), N);
        double s2 = 0.0;
        for (int i = 0; i <= j; ++i) s2 += h2[i] * h2[i];
        for (int i = 0; i <= j; ++i) {
          const double* vi = &V[(int64_t)i * N];
          for (int64_t q = 0; q < N; ++q) W[q] -= h2[i] * vi[q];
        }
        const double e2 = nw2b - s2;
        hn = e2 > 0.0 ? std::sqrt(e2) : 0.0;
      } else {
        hn = std::sqrt(est);
      }
      for (int i = 0; i <= j; ++i) H[i * restart + j] = h[i] + h2[i];
      H[(j + 1) * restart + j] = hn;
      if (hn != 0.0) {
        const double inv = 1.0 / hn;
        for (int64_t q = 0; q < N; ++q) V[(int64_t)(j + 1) * N + q] = W[q] * inv;
      }
      for (int i = 0; i < j; ++i) {
        const double t = cs[i] * H[i * restart + j] + sn[i] * H[(i + 1) * restart + j];
        H[(i + 1) * restart + j] = -sn[i] * H[i * restart + j] + cs[i] * H[(i + 1) * restart + j];
        H[i * restart + j] = t;
      }
      const double a = H[j * restart + j], c = H[(j + 1) * restart + j];
      const double d = std::sqrt(a * a + c * c);
      cs[j] = (d == 0.0) ? 1.0 : a / d;
      sn[j] = (d == 0.0) ? 0.0 : c / d;
      H[j * restart + j] = d;
      H[(j + 1) * restart + j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      if (std::fabs(g[j + 1]) <= eps) {
        ++j;
        ++iter;
        break;
      }
    }
    // back substitution y = H^{-1} g, x += M^{-1} (V y)
    std::vector<double> y(j);
    for (int i = j - 1; i >= 0; --i) {
      double s = g[i];
      for (int k = i + 1; k < j; ++k) s -= H[i * restart + k] * y[k];
      y[i] = s / H[i * restart + i];
    }
    std::fill(W.begin(), W.end(), 0.0);
    for (int i = 0; i < j; ++i) {
      const double* vi = &V[(int64_t)i * N];
      for (int64_t q = 0; q < N; ++q) W[q] += y[i] * vi[q];
    }
    M.apply(W.data(), Z.data());
    for (int64_t q = 0; q < N; ++q) x[q] += Z[q];
    // true residual for the restart / final report
    bcsr_spmv(A, x, W.data());
    for (int64_t q = 0; q < N; ++q) r[q] = b[q] - W[q];
    norm_r = std::sqrt(dot(r.data(), r.data(), N));
    if (norm_r <= eps || iter >= maxiter) break;
  }
  res.iterations = iter;
  res.rel_residual = norm_r / norm_b;
  return res;
}

}  // namespace besla
