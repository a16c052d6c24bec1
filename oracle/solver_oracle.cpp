/*
 * TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
 *
 * CPU restatement ("oracle") of the linear solve the reference runs after each
 * assembly: belos_linear_solver::execute (src/fem/ls/belos_linear_solver_factory.hpp:
 * 103-218) with the shipped settings (sim/fluid_mc/P0/setup.txt:10-16: Flexible GMRES,
 * ILU, relative residual 1e-9, 200 vectors per cycle, 5 restarts, maxiters -1 = rows - 1,
 * level of fill 1).  Used only by tests/ and bench.py's CPU-baseline leg as the checker.
 *
 * PARITY UNPINNED: Trilinos (Belos, Ifpack, Epetra) is absent here.  Restated from the
 * published algorithms of Trilinos 12.x:
 *   - Ifpack "ILU" (Ifpack_ILU over Ifpack_IlukGraph): scalar ILU(k) on the matrix
 *     graph.  Symbolic: a row starts with the matrix's columns at level 0; for each of
 *     its columns k < i in ascending order, every column j > k of row k's upper part gets
 *     level lev(i,k) + lev(k,j) + 1 and is kept (or lowered) when that is <= k_fill.
 *     Numeric: row-oriented (ikj) Gaussian elimination restricted to the pattern, unit L,
 *     no pivoting, no diagonal perturbation (athresh 0, rthresh 1, relax 0).  With one
 *     rank the additive Schwarz wrapper (overlap 1, belos_linear_solver_factory.hpp:
 *     143-151) is the plain factorisation.
 *   - Belos BlockGmresSolMgr with "Flexible Gmres" and block size 1: right
 *     preconditioning, x0 = 0 (belos_linear_solver_factory.hpp:119-121), Arnoldi on
 *     A M^-1 with two classical Gram-Schmidt passes per step, Givens rotations for the
 *     least-squares problem, x += Z y at the end of a cycle (Z = M^-1 V).  A step
 *     converges when the implicit residual |g_{j+1}| <= tol ||r0|| (r0 = b); the cycle
 *     then ends and the explicit residual ||b - A x|| <= tol ||b|| confirms it, else the
 *     solve restarts.  Iterations count Arnoldi steps over all cycles (getNumIters).
 *   - The returned ARE/RRE are ||b - A x|| and ||b - A x|| / ||b||
 *     (belos_linear_solver_factory.hpp:206-214).
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>

namespace {

struct Iluk {
  std::vector<int64_t> rp;
  std::vector<int32_t> col;
  std::vector<int> lev;
  std::vector<int64_t> diag;
  std::vector<double> val;
};

// Ifpack_IlukGraph restated (see the header).
bool iluk_symbolic(int64_t n, const int64_t* rp, const int32_t* col, int fill, Iluk& F) {
  F.rp.assign(n + 1, 0);
  F.col.clear();
  F.lev.clear();
  F.diag.assign(n, -1);
  for (int64_t i = 0; i < n; ++i) {
    std::map<int32_t, int> row;
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p) row[col[p]] = 0;
    row.emplace((int32_t)i, 0);  // the diagonal is part of every row's graph
    for (auto it = row.begin(); it != row.end() && it->first < i; ++it) {
      const int32_t k = it->first;
      const int lik = it->second;
      for (int64_t q = F.diag[k] + 1; q < F.rp[k + 1]; ++q) {
        const int l = lik + F.lev[q] + 1;
        if (l > fill) continue;
        auto f = row.find(F.col[q]);
        if (f == row.end()) row.emplace(F.col[q], l);
        else if (l < f->second) f->second = l;
      }
    }
    for (const auto& e : row) {
      if (e.first == i) F.diag[i] = (int64_t)F.col.size();
      F.col.push_back(e.first);
      F.lev.push_back(e.second);
    }
    F.rp[i + 1] = (int64_t)F.col.size();
  }
  return true;
}

// Row-oriented ILU on the symbolic pattern; returns the first zero pivot row or -1.
int64_t iluk_numeric(int64_t n, const int64_t* rp, const int32_t* col, const double* a, Iluk& F) {
  F.val.assign(F.col.size(), 0.0);
  std::vector<int64_t> pos(n, -1);
  for (int64_t i = 0; i < n; ++i) {
    for (int64_t p = F.rp[i]; p < F.rp[i + 1]; ++p) pos[F.col[p]] = p;
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p) F.val[pos[col[p]]] += a[p];
    for (int64_t p = F.rp[i]; p < F.diag[i]; ++p) {
      const int32_t k = F.col[p];
      const double lik = F.val[p] / F.val[F.diag[k]];
      F.val[p] = lik;
      for (int64_t q = F.diag[k] + 1; q < F.rp[k + 1]; ++q) {
        const int64_t t = pos[F.col[q]];
        if (t >= 0) F.val[t] -= lik * F.val[q];
      }
    }
    for (int64_t p = F.rp[i]; p < F.rp[i + 1]; ++p) pos[F.col[p]] = -1;
    if (F.val[F.diag[i]] == 0.0) return i;
  }
  return -1;
}

void ilu_apply(const Iluk& F, int64_t n, const double* v, double* z) {
  for (int64_t i = 0; i < n; ++i) {
    double s = v[i];
    for (int64_t p = F.rp[i]; p < F.diag[i]; ++p) s -= F.val[p] * z[F.col[p]];
    z[i] = s;
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    double s = z[i];
    for (int64_t p = F.diag[i] + 1; p < F.rp[i + 1]; ++p) s -= F.val[p] * z[F.col[p]];
    z[i] = s / F.val[F.diag[i]];
  }
}

void spmv(int64_t n, const int64_t* rp, const int32_t* col, const double* a, const double* x, double* y) {
  for (int64_t i = 0; i < n; ++i) {
    double s = 0.0;
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p) s += a[p] * x[col[p]];
    y[i] = s;
  }
}

double dot(int64_t n, const double* x, const double* y) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += x[i] * y[i];
  return s;
}

}  // namespace

extern "C" {

// ILU(fill) of a CSR matrix.  With f_rp null only *nnz_out is set; otherwise f_rp
// (n + 1), f_col and f_val (*nnz_out) receive the factor: unit L strictly below the
// diagonal, U on and above it.  Returns 0, or 1 + the row of the first zero pivot.
int64_t gor_iluk(int64_t n, const int64_t* rp, const int32_t* col, const double* a, int32_t fill,
                 int64_t* nnz_out, int64_t* f_rp, int32_t* f_col, double* f_val) {
  Iluk F;
  iluk_symbolic(n, rp, col, fill, F);
  *nnz_out = (int64_t)F.col.size();
  if (!f_rp) return 0;
  const int64_t bad = iluk_numeric(n, rp, col, a, F);
  std::memcpy(f_rp, F.rp.data(), sizeof(int64_t) * (n + 1));
  std::memcpy(f_col, F.col.data(), sizeof(int32_t) * F.col.size());
  std::memcpy(f_val, F.val.data(), sizeof(double) * F.val.size());
  return bad < 0 ? 0 : bad + 1;
}

// Flexible GMRES with right ILU(fill) preconditioning (precond 0: none); see the header.
// out[0] = iterations, out[1] = ||b - A x||, out[2] = relative, out[3] = converged,
// out[4] = cycles.  Returns 0, or 1 + the first zero-pivot row.
int64_t gor_fgmres(int64_t n, const int64_t* rp, const int32_t* col, const double* a, const double* b,
                   int32_t fill, int32_t precond, double tol, int32_t m, int32_t maxrestarts, int64_t maxiters,
                   double* x, double* out) {
  Iluk F;
  if (precond) {
    iluk_symbolic(n, rp, col, fill, F);
    const int64_t bad = iluk_numeric(n, rp, col, a, F);
    if (bad >= 0) return bad + 1;
  }
  if (maxiters < 0) maxiters = n - 1;
  for (int64_t i = 0; i < n; ++i) x[i] = 0.0;
  const double bnorm = std::sqrt(dot(n, b, b));
  std::vector<double> r(b, b + n), w(n);
  std::vector<std::vector<double>> V, Z;
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m), h(m + 1), h2(m + 1);
  int64_t iters = 0;
  int cycles = 0;
  bool converged = bnorm == 0.0;
  double beta = bnorm;
  while (!converged && cycles <= maxrestarts && iters < maxiters && beta > 0.0) {
    ++cycles;
    V.assign(1, std::vector<double>(n));
    Z.clear();
    for (int64_t i = 0; i < n; ++i) V[0][i] = r[i] / beta;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    bool est_conv = false;
    for (; j < m && iters < maxiters; ++j) {
      Z.emplace_back(n);
      if (precond) ilu_apply(F, n, V[j].data(), Z[j].data());
      else Z[j] = V[j];
      spmv(n, rp, col, a, Z[j].data(), w.data());
      for (int c = 0; c <= j; ++c) h[c] = 0.0;
      for (int pass = 0; pass < 2; ++pass) {
        for (int c = 0; c <= j; ++c) h2[c] = dot(n, V[c].data(), w.data());
        for (int64_t i = 0; i < n; ++i) {
          double s = 0.0;
          for (int c = 0; c <= j; ++c) s += V[c][i] * h2[c];
          w[i] -= s;
        }
        for (int c = 0; c <= j; ++c) h[c] += h2[c];
      }
      const double hn = std::sqrt(dot(n, w.data(), w.data()));
      h[j + 1] = hn;
      V.emplace_back(n);
      if (hn > 0.0)
        for (int64_t i = 0; i < n; ++i) V[j + 1][i] = w[i] / hn;
      for (int c = 0; c < j; ++c) {
        const double t = cs[c] * h[c] + sn[c] * h[c + 1];
        h[c + 1] = -sn[c] * h[c] + cs[c] * h[c + 1];
        h[c] = t;
      }
      const double d = std::hypot(h[j], h[j + 1]);
      cs[j] = d > 0.0 ? h[j] / d : 1.0;
      sn[j] = d > 0.0 ? h[j + 1] / d : 0.0;
      h[j] = d;
      h[j + 1] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      for (int c = 0; c <= j; ++c) H[(size_t)c * m + j] = h[c];
      ++iters;
      if (std::fabs(g[j + 1]) <= tol * bnorm || hn == 0.0) {
        est_conv = true;
        ++j;
        break;
      }
    }
    for (int c = j - 1; c >= 0; --c) {
      double s = g[c];
      for (int t = c + 1; t < j; ++t) s -= H[(size_t)c * m + t] * y[t];
      y[c] = s / H[(size_t)c * m + c];
    }
    for (int64_t i = 0; i < n; ++i) {
      double s = 0.0;
      for (int c = 0; c < j; ++c) s += Z[c][i] * y[c];
      x[i] += s;
    }
    spmv(n, rp, col, a, x, w.data());
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - w[i];
    beta = std::sqrt(dot(n, r.data(), r.data()));
    if (est_conv && beta <= tol * bnorm) converged = true;
  }
  spmv(n, rp, col, a, x, w.data());
  for (int64_t i = 0; i < n; ++i) r[i] = b[i] - w[i];
  const double res = std::sqrt(dot(n, r.data(), r.data()));
  out[0] = (double)iters;
  out[1] = res;
  out[2] = bnorm > 0.0 ? res / bnorm : 0.0;
  out[3] = converged ? 1.0 : 0.0;
  out[4] = (double)cycles;
  return 0;
}

}  // extern "C"
