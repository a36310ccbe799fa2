// ORACLE (test infrastructure only) -- built-in sparse solvers.
// Restates src/linearSolvers/linear_solvers.f90: csrsolve :40-91,
// GaussSeidel :96-201, dpcg :206-359, iccg :364-545, bicgstab :548-786,
// pmgmres_ilu :789-1077, atx_cr :1079, ax_cr :1173, ilu_cr :1267,
// lus_cr :1386, mult_givens :1479.  All arrays are 1-based raw pointers
// (element 0 unused).  The L1 sums are plain left-to-right loops, which is
// what gfortran's SUM intrinsic computes without -ffast-math.
#include <cmath>
#include <vector>

#include "oracle.hpp"

namespace orc {

static inline double l1(int n, const double* r) {
  double s = 0.0;
  for (int i = 1; i <= n; ++i) s += std::fabs(r[i]);
  return s;
}
static inline double dotp(int n, const double* a, const double* b) {
  double s = 0.0;
  for (int i = 1; i <= n; ++i) s += a[i] * b[i];
  return s;
}
static inline double factor_of(int n, const double* a, const int* diag, const double* fi) {
  double s = 0.0;
  for (int i = 1; i <= n; ++i) s += std::fabs(a[diag[i]] * fi[i]);
  return s + kSmall;
}

void gauss_seidel(int n, int nnz, const int* ia, const int* ja, const double* a, const int* diag, double* fi,
                  const double* rhs, double& resor, int itr_max, double tol_abs, double tol_rel, double* res,
                  SolveInfo& si) {
  (void)nnz;
  int itr_used = 0;
  double factor = 0.0, res0 = 0.0, resl = 0.0;
  for (int l = 1; l <= itr_max; ++l) {
    for (int i = 1; i <= n; ++i) {
      res[i] = rhs[i];
      for (int k = ia[i]; k <= ia[i + 1] - 1; ++k) res[i] = res[i] - a[k] * fi[ja[k]];
      fi[i] = fi[i] + res[i] / (a[diag[i]] + kSmall);
    }
    if (l == 1) {
      res0 = l1(n, res);
      if (res0 < tol_abs) {  // linear_solvers.f90:158-162 (resor is left unset there)
        si.itr_used = 0; si.res0 = res0; si.resl = res0; si.early = 1;
        return;
      }
    }
    resl = l1(n, res);
    itr_used = itr_used + 1;
    if (l == 1) {
      factor = factor_of(n, a, diag, fi);
      resor = res0 / factor;
    }
    double rsm = resl / (res0 + kSmall);
    if (rsm < tol_rel || resl < tol_abs) break;
  }
  si.itr_used = itr_used; si.res0 = res0; si.resl = resl; si.factor = factor; si.resor = resor;
}

void dpcg(int n, int nnz, const int* ia, const int* ja, const double* a, const int* diag, double* fi,
          const double* rhs, double& resor, int itr_max, double tol_abs, double tol_rel, double* res, double* pk,
          double* zk, SolveInfo& si) {
  (void)nnz;
  double factor = 0.0;
  for (int i = 1; i <= n; ++i) { pk[i] = 0.0; zk[i] = 0.0; res[i] = 0.0; }
  for (int i = 1; i <= n; ++i) {
    res[i] = rhs[i];
    for (int k = ia[i]; k <= ia[i + 1] - 1; ++k) res[i] = res[i] - a[k] * fi[ja[k]];
  }
  double res0 = l1(n, res);
  if (res0 < tol_abs) { si.itr_used = 0; si.res0 = res0; si.resl = res0; si.early = 1; return; }
  double s0 = kS0, resl = 0.0;
  int itr_used = 0;
  for (int l = 1; l <= itr_max; ++l) {
    for (int i = 1; i <= n; ++i) zk[i] = res[i] / a[diag[i]];
    double sk = dotp(n, res, zk);
    double bet = sk / s0;
    for (int i = 1; i <= n; ++i) pk[i] = zk[i] + bet * pk[i];
    for (int i = 1; i <= n; ++i) {
      zk[i] = 0.0;
      for (int k = ia[i]; k <= ia[i + 1] - 1; ++k) zk[i] = zk[i] + a[k] * pk[ja[k]];
    }
    double pkapk = dotp(n, pk, zk);
    double alf = sk / pkapk;
    for (int i = 1; i <= n; ++i) fi[i] = fi[i] + alf * pk[i];
    for (int i = 1; i <= n; ++i) res[i] = res[i] - alf * zk[i];
    resl = l1(n, res);
    s0 = sk;
    itr_used = itr_used + 1;
    if (l == 1) {
      factor = factor_of(n, a, diag, fi);
      resor = res0 / factor;
    }
    double rsm = resl / (res0 + kSmall);
    if (rsm < tol_rel || resl < tol_abs) break;
  }
  si.itr_used = itr_used; si.res0 = res0; si.resl = resl; si.factor = factor; si.resor = resor;
}

// DIC recurrence, linear_solvers.f90:439-445
void dic_setup(int n, const int* ia, const int* ja, const double* a, const int* diag, double* d) {
  for (int i = 1; i <= n; ++i) {
    d[i] = a[diag[i]];
    for (int k = ia[i]; k <= diag[i] - 1; ++k) d[i] = d[i] - (a[k] * a[k]) * d[ja[k]];
    d[i] = 1.0 / d[i];
  }
}

// DILU recurrence with the transpose search, linear_solvers.f90:613-624
void dilu_setup(int n, const int* ia, const int* ja, const double* a, const int* diag, double* d) {
  for (int i = 1; i <= n; ++i) {
    d[i] = a[diag[i]];
    for (int k = ia[i]; k <= diag[i] - 1; ++k) {
      int l;
      for (l = diag[ja[k]]; l <= ia[ja[k] + 1] - 1; ++l)
        if (ja[l] == i) break;
      d[i] = d[i] - a[k] * d[ja[k]] * a[l];
    }
    d[i] = 1.0 / d[i];
  }
}

// forward sweep, z/(d+small) scaling and backward sweep shared by iccg
// (:458-475) and bicgstab (:650-672, :705-725)
void diag_precond_apply(int n, const int* ia, const int* ja, const double* a, const int* diag, const double* d,
                        const double* r, double* z) {
  for (int i = 1; i <= n; ++i) {
    z[i] = r[i];
    for (int k = ia[i]; k <= diag[i] - 1; ++k) z[i] = z[i] - a[k] * z[ja[k]];
    z[i] = z[i] * d[i];
  }
  for (int i = 1; i <= n; ++i) z[i] = z[i] / (d[i] + kSmall);
  for (int i = n; i >= 1; --i) {
    for (int k = diag[i] + 1; k <= ia[i + 1] - 1; ++k) z[i] = z[i] - a[k] * z[ja[k]];
    z[i] = z[i] * d[i];
  }
}

void iccg(int n, int nnz, const int* ia, const int* ja, const double* a, const int* diag, double* fi,
          const double* rhs, double& resor, int itr_max, double tol_abs, double tol_rel, double* res, double* pk,
          double* zk, double* d, SolveInfo& si) {
  (void)nnz;
  double factor = 0.0;
  for (int i = 1; i <= n; ++i) { pk[i] = 0.0; zk[i] = 0.0; d[i] = 0.0; res[i] = 0.0; }
  for (int i = 1; i <= n; ++i) {
    res[i] = rhs[i];
    for (int k = ia[i]; k <= ia[i + 1] - 1; ++k) res[i] = res[i] - a[k] * fi[ja[k]];
  }
  double res0 = l1(n, res);
  if (res0 < tol_abs) { si.itr_used = 0; si.res0 = res0; si.resl = res0; si.early = 1; return; }
  dic_setup(n, ia, ja, a, diag, d);
  double s0 = kS0, resl = 0.0;
  int itr_used = 0;
  for (int l = 1; l <= itr_max; ++l) {
    diag_precond_apply(n, ia, ja, a, diag, d, res, zk);
    double sk = dotp(n, res, zk);
    double bet = sk / s0;
    for (int i = 1; i <= n; ++i) pk[i] = zk[i] + bet * pk[i];
    for (int i = 1; i <= n; ++i) {
      zk[i] = 0.0;
      for (int k = ia[i]; k <= ia[i + 1] - 1; ++k) zk[i] = zk[i] + a[k] * pk[ja[k]];
    }
    double pkapk = dotp(n, pk, zk);
    double alf = sk / pkapk;
    for (int i = 1; i <= n; ++i) fi[i] = fi[i] + alf * pk[i];
    for (int i = 1; i <= n; ++i) res[i] = res[i] - alf * zk[i];
    resl = l1(n, res);
    s0 = sk;
    itr_used = itr_used + 1;
    if (l == 1) {
      factor = factor_of(n, a, diag, fi);
      resor = res0 / factor;
    }
    double rsm = resl / (res0 + kSmall);
    if (rsm < tol_rel || resl < tol_abs) break;
  }
  si.itr_used = itr_used; si.res0 = res0; si.resl = resl; si.factor = factor; si.resor = resor;
}

void bicgstab(int n, int nnz, const int* ia, const int* ja, const double* a, const int* diag, double* fi,
              const double* rhs, double& resor, int itr_max, double tol_abs, double tol_rel, double* res,
              double* reso, double* pk, double* uk, double* zk, double* vk, double* d, SolveInfo& si) {
  (void)nnz;
  for (int i = 1; i <= n; ++i) {
    res[i] = rhs[i];
    for (int k = ia[i]; k <= ia[i + 1] - 1; ++k) res[i] = res[i] - a[k] * fi[ja[k]];
  }
  double res0 = l1(n, res);
  if (res0 < tol_abs) { si.itr_used = 0; si.res0 = res0; si.resl = res0; si.early = 1; return; }
  dilu_setup(n, ia, ja, a, diag, d);
  for (int i = 1; i <= n; ++i) { reso[i] = res[i]; pk[i] = 0.0; uk[i] = 0.0; zk[i] = 0.0; vk[i] = 0.0; }
  double factor = 0.0;
  double alf = 1.0, beto = 1.0, gam = 1.0, resl = 0.0;
  int itr_used = 0;
  for (int l = 1; l <= itr_max; ++l) {
    double bet = dotp(n, res, reso);
    double om = bet * gam / (alf * beto + kSmall);
    beto = bet;
    for (int i = 1; i <= n; ++i) pk[i] = res[i] + om * (pk[i] - alf * uk[i]);
    diag_precond_apply(n, ia, ja, a, diag, d, pk, zk);
    for (int i = 1; i <= n; ++i) {
      uk[i] = 0.0;
      for (int k = ia[i]; k <= ia[i + 1] - 1; ++k) uk[i] = uk[i] + a[k] * zk[ja[k]];
    }
    double ukreso = dotp(n, uk, reso);
    gam = bet / ukreso;
    for (int i = 1; i <= n; ++i) fi[i] = fi[i] + gam * zk[i];
    for (int i = 1; i <= n; ++i) res[i] = res[i] - gam * uk[i];
    diag_precond_apply(n, ia, ja, a, diag, d, res, zk);
    for (int i = 1; i <= n; ++i) {
      vk[i] = 0.0;
      for (int k = ia[i]; k <= ia[i + 1] - 1; ++k) vk[i] = vk[i] + a[k] * zk[ja[k]];
    }
    alf = dotp(n, vk, res) / (dotp(n, vk, vk) + kSmall);
    for (int i = 1; i <= n; ++i) fi[i] = fi[i] + alf * zk[i];
    for (int i = 1; i <= n; ++i) res[i] = res[i] - alf * vk[i];
    resl = l1(n, res);
    itr_used = itr_used + 1;
    if (l == 1) {
      factor = factor_of(n, a, diag, fi);
      resor = res0 / factor;
    }
    double rsm = resl / (res0 + kSmall);
    if (rsm < tol_rel || resl < tol_abs) break;
  }
  si.itr_used = itr_used; si.res0 = res0; si.resl = resl; si.factor = factor; si.resor = resor;
}

// ax_cr, linear_solvers.f90:1173-1265: w(i) = 0 + dot_product(a(k1:k2), x(ja(k1:k2)))
void ax_cr(int n, const int* ia, const int* ja, const double* a, const double* x, double* w) {
  for (int i = 1; i <= n; ++i) w[i] = 0.0;
  for (int i = 1; i <= n; ++i) {
    double s = 0.0;
    for (int k = ia[i]; k <= ia[i + 1] - 1; ++k) s += a[k] * x[ja[k]];
    w[i] = w[i] + s;
  }
}

// atx_cr, linear_solvers.f90:1079-1171 (scatter form of A^T x)
void atx_cr(int n, const int* ia, const int* ja, const double* a, const double* x, double* w) {
  for (int i = 1; i <= n; ++i) w[i] = 0.0;
  for (int i = 1; i <= n; ++i)
    for (int k = ia[i]; k <= ia[i + 1] - 1; ++k) w[ja[k]] = w[ja[k]] + a[k] * x[i];
}

// ilu_cr, linear_solvers.f90:1267-1385.  Returns FC_ERR_ZERO_PIVOT (-8) or
// FC_ERR_BAD_INPUT (-1) where the reference stops the program.
int ilu_cr(int n, const int* ia, const int* ja, const double* a, int* ua, double* l) {
  const int nz = ia[n + 1] - 1;
  for (int k = 1; k <= nz; ++k) l[k] = a[k];
  std::vector<int> iw(n + 1, -1);
  for (int i = 1; i <= n; ++i) {
    for (int k = 1; k <= n; ++k) iw[k] = -1;
    for (int k = ia[i]; k <= ia[i + 1] - 1; ++k) iw[ja[k]] = k;
    int j, jrow = 0;
    for (j = ia[i]; j <= ia[i + 1] - 1; ++j) {
      jrow = ja[j];
      if (i <= jrow) break;
      double tl = l[j] * l[ua[jrow]];
      l[j] = tl;
      for (int jj = ua[jrow] + 1; jj <= ia[jrow + 1] - 1; ++jj) {
        int jw = iw[ja[jj]];
        if (jw != -1) l[jw] = l[jw] - tl * l[jj];
      }
    }
    ua[i] = j;
    if (jrow != i) return -1;
    if (l[j] == 0.0) return -8;
    l[j] = 1.0 / l[j];
  }
  for (int i = 1; i <= n; ++i) l[ua[i]] = 1.0 / l[ua[i]];
  return 0;
}

// lus_cr, linear_solvers.f90:1386-1478
void lus_cr(int n, const int* ia, const int* ja, const double* l, const int* ua, const double* r, double* z) {
  std::vector<double> w(n + 1);
  for (int i = 1; i <= n; ++i) w[i] = r[i];
  for (int i = 2; i <= n; ++i)
    for (int j = ia[i]; j <= ua[i] - 1; ++j) w[i] = w[i] - l[j] * w[ja[j]];
  for (int i = n; i >= 1; --i) {
    for (int j = ua[i] + 1; j <= ia[i + 1] - 1; ++j) w[i] = w[i] - l[j] * w[ja[j]];
    w[i] = w[i] / l[ua[i]];
  }
  for (int i = 1; i <= n; ++i) z[i] = w[i];
}

static inline void mult_givens(double c, double s, int k, double* g) {
  double g1 = c * g[k] - s * g[k + 1];
  double g2 = s * g[k] + c * g[k + 1];
  g[k] = g1;
  g[k + 1] = g2;
}

// pmgmres_ilu, linear_solvers.f90:789-1077 (stopping test kept as written:
// resl/resor <= rho_tol with rho_tol = resor*tol_rel).
int pmgmres_ilu(int n, int nz_num, const int* ia, const int* ja, const double* a, int* ua, double* x,
                const double* rhs, double& resor, int itr_max, int mr, double tol_abs, double tol_rel,
                SolveInfo& si) {
  const double delta = 1.0e-03;
  int itr_used = 0;
  double rho_tol = 0.0, resl = 0.0;
  int k_copy = 0;
  std::vector<double> r(n + 1), l(nz_num + 2), v((size_t)(n + 1) * (mr + 2));
  auto V = [&](int i, int j) -> double& { return v[(size_t)j * (n + 1) + i]; };
  std::vector<double> c(mr + 2), g(mr + 2), s(mr + 2), y(mr + 2), h((size_t)(mr + 2) * (mr + 1));
  auto H = [&](int i, int j) -> double& { return h[(size_t)j * (mr + 2) + i]; };
  int st = ilu_cr(n, ia, ja, a, ua, l.data());
  if (st != 0) return st;
  std::vector<double> tmp(n + 1);
  for (int itr = 1; itr <= itr_max; ++itr) {
    ax_cr(n, ia, ja, a, x, r.data());
    for (int i = 1; i <= n; ++i) r[i] = rhs[i] - r[i];
    if (itr == 1) {
      resor = l1(n, r.data());
      rho_tol = resor * tol_rel;
    }
    double rho = std::sqrt(dotp(n, r.data(), r.data()));
    lus_cr(n, ia, ja, l.data(), ua, r.data(), r.data());
    for (int i = 1; i <= n; ++i) V(i, 1) = r[i] / rho;
    g[1] = rho;
    for (int i = 2; i <= mr + 1; ++i) g[i] = 0.0;
    for (int j = 1; j <= mr; ++j)
      for (int i = 1; i <= mr + 1; ++i) H(i, j) = 0.0;
    int k;
    for (k = 1; k <= mr; ++k) {
      k_copy = k;
      for (int i = 1; i <= n; ++i) tmp[i] = V(i, k);
      std::vector<double> w(n + 1);
      ax_cr(n, ia, ja, a, tmp.data(), w.data());
      lus_cr(n, ia, ja, l.data(), ua, w.data(), w.data());
      for (int i = 1; i <= n; ++i) V(i, k + 1) = w[i];
      double av = 0.0;
      for (int i = 1; i <= n; ++i) av += V(i, k + 1) * V(i, k + 1);
      av = std::sqrt(av);
      for (int j = 1; j <= k; ++j) {
        double hs = 0.0;
        for (int i = 1; i <= n; ++i) hs += V(i, k + 1) * V(i, j);
        H(j, k) = hs;
        for (int i = 1; i <= n; ++i) V(i, k + 1) = V(i, k + 1) - V(i, j) * H(j, k);
      }
      double hn = 0.0;
      for (int i = 1; i <= n; ++i) hn += V(i, k + 1) * V(i, k + 1);
      H(k + 1, k) = std::sqrt(hn);
      if ((av + delta * H(k + 1, k)) == av) {
        for (int j = 1; j <= k; ++j) {
          double htmp = 0.0;
          for (int i = 1; i <= n; ++i) htmp += V(i, k + 1) * V(i, j);
          H(j, k) = H(j, k) + htmp;
          for (int i = 1; i <= n; ++i) V(i, k + 1) = V(i, k + 1) - htmp * V(i, j);
        }
        hn = 0.0;
        for (int i = 1; i <= n; ++i) hn += V(i, k + 1) * V(i, k + 1);
        H(k + 1, k) = std::sqrt(hn);
      }
      if (H(k + 1, k) != 0.0)
        for (int i = 1; i <= n; ++i) V(i, k + 1) = V(i, k + 1) / H(k + 1, k);
      if (1 < k) {
        for (int i = 1; i <= k + 1; ++i) y[i] = H(i, k);
        for (int j = 1; j <= k - 1; ++j) mult_givens(c[j], s[j], j, y.data());
        for (int i = 1; i <= k + 1; ++i) H(i, k) = y[i];
      }
      double mu = std::sqrt(H(k, k) * H(k, k) + H(k + 1, k) * H(k + 1, k));
      c[k] = H(k, k) / mu;
      s[k] = -H(k + 1, k) / mu;
      H(k, k) = c[k] * H(k, k) - s[k] * H(k + 1, k);
      H(k + 1, k) = 0.0;
      mult_givens(c[k], s[k], k, g.data());
      resl = std::fabs(g[k + 1]);
      itr_used = itr_used + 1;
      if (resl / resor <= rho_tol || resl <= tol_abs) break;
    }
    k = k_copy - 1;
    y[k + 1] = g[k + 1] / H(k + 1, k + 1);
    for (int i = k; i >= 1; --i) {
      double sdot = 0.0;
      for (int q = i + 1; q <= k + 1; ++q) sdot += H(i, q) * y[q];
      y[i] = (g[i] - sdot) / H(i, i);
    }
    for (int i = 1; i <= n; ++i) {
      double sdot = 0.0;
      for (int q = 1; q <= k + 1; ++q) sdot += V(i, q) * y[q];
      x[i] = x[i] + sdot;
    }
    if (resl / resor <= rho_tol || resl <= tol_abs) break;
  }
  si.itr_used = itr_used; si.resl = resl; si.resor = resor; si.res0 = resor;
  return 0;
}

// csrsolve dispatch on the case's global matrix, linear_solvers.f90:40-91
int csrsolve(Case& c, const std::string& solver, std::vector<double>& fi, const std::vector<double>& rhs,
             double& res0, int itr_max, double tol_abs, double tol_rel, SolveInfo& si) {
  const int n = c.numCells;
  if (solver == "gauss-seidel") {
    gauss_seidel(n, c.nnz, c.ia.data(), c.ja.data(), c.a.data(), c.diag.data(), fi.data(), rhs.data(), res0, itr_max,
                 tol_abs, tol_rel, c.res.data(), si);
  } else if (solver == "dpcg") {
    dpcg(n, c.nnz, c.ia.data(), c.ja.data(), c.a.data(), c.diag.data(), fi.data(), rhs.data(), res0, itr_max, tol_abs,
         tol_rel, c.res.data(), c.pk.data(), c.zk.data(), si);
  } else if (solver == "iccg") {
    iccg(n, c.nnz, c.ia.data(), c.ja.data(), c.a.data(), c.diag.data(), fi.data(), rhs.data(), res0, itr_max, tol_abs,
         tol_rel, c.res.data(), c.pk.data(), c.zk.data(), c.d.data(), si);
  } else if (solver == "bicgstab") {
    bicgstab(n, c.nnz, c.ia.data(), c.ja.data(), c.a.data(), c.diag.data(), fi.data(), rhs.data(), res0, itr_max,
             tol_abs, tol_rel, c.res.data(), c.reso.data(), c.pk.data(), c.uk.data(), c.zk.data(), c.vk.data(),
             c.d.data(), si);
  } else if (solver == "pmgmres") {
    std::vector<int> ua(c.diag);
    return pmgmres_ilu(n, c.nnz, c.ia.data(), c.ja.data(), c.a.data(), ua.data(), fi.data(), rhs.data(), res0,
                       itr_max, 4, tol_abs, tol_rel, si);
  } else {
    return -1;
  }
  return 0;
}

}  // namespace orc
