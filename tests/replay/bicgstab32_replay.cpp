// CPU replay of the FP32 inner solve of the mixed-precision BiCGStab: the
// reference's DILU-BiCGStab (linear_solvers.f90:548-786) with the matrix,
// the preconditioner and every Krylov vector in FP32 and the dots and L1
// norms accumulated in FP64, the precision split of the device kernel
// k_bicgstab<float> / k_bicgstab_batch<float>.  Vector updates use FMA where
// the device's expressions contract to one (p = r + om (p - alf u), x += g z,
// r -= g u); the triangular sweeps and the row products accumulate with FMA
// in the row's entry order, as the device does.  Test infrastructure only.
//
// bicgstab32(n, ia, ja, a, diag, x, b, itr_max, tol_rel, stall_window,
// hist): 1-based CSR (ia(n+1), ja(nnz), diag(n)); a (FP32 values), b (FP32
// right-hand side), x (FP32, in: start, out: solution); stops on
// resl/(res0+small) < tol_rel, after itr_max iterations, or (stall_window
// > 0, the device's rule for the inner solves) once resl has gone
// stall_window iterations without falling below half of its last recorded
// value; hist[l-1] receives resl after iteration l, hist[itr_max] receives
// res0.  Returns the iterations used.
#include <cmath>
#include <vector>

namespace {
const double kSmall = static_cast<double>(1e-20f);  // parameters.f90 small, a default-real literal
const float kSmallF = 1e-20f;
}

extern "C" int bicgstab32(int n, const int* ia, const int* ja, const float* a, const int* diag, float* x,
                          const float* b, int itr_max, double tol_rel, int stall_window, double* hist) {
  auto A = [&](int k) { return a[k - 1]; };
  auto JA = [&](int k) { return ja[k - 1]; };
  std::vector<float> res(n + 1), reso(n + 1), pk(n + 1, 0.f), uk(n + 1, 0.f), zk(n + 1, 0.f), vk(n + 1, 0.f),
      d(n + 1), f(n + 1);
  double res0 = 0.0;
  for (int i = 1; i <= n; ++i) {
    float s = b[i - 1];
    for (int k = ia[i - 1]; k < ia[i]; ++k) s = std::fma(-A(k), x[JA(k) - 1], s);
    res[i] = s;
    res0 += std::fabs((double)s);
  }
  hist[itr_max] = res0;
  // DILU factors (linear_solvers.f90:613-624), FP32, no contraction
  for (int i = 1; i <= n; ++i) {
    float di = A(diag[i - 1]);
    for (int k = ia[i - 1]; k < diag[i - 1]; ++k) {
      const int j = JA(k);
      int l = diag[j - 1];
      for (; l < ia[j]; ++l)
        if (JA(l) == i) break;
      const volatile float t = A(k) * d[j];
      di = di - t * A(l);
    }
    d[i] = 1.0f / di;
    f[i] = 1.0f / (d[i] + kSmallF);
  }
  auto apply = [&](const std::vector<float>& q) {
    for (int i = 1; i <= n; ++i) {
      float s = q[i];
      for (int k = ia[i - 1]; k < diag[i - 1]; ++k) s = std::fma(-A(k), zk[JA(k)], s);
      zk[i] = s * d[i];
    }
    for (int i = n; i >= 1; --i) {
      float s = zk[i] * f[i];
      for (int k = diag[i - 1] + 1; k < ia[i]; ++k) s = std::fma(-A(k), zk[JA(k)], s);
      zk[i] = s * d[i];
    }
  };
  auto matvec = [&](std::vector<float>& out) {
    for (int i = 1; i <= n; ++i) {
      float s = 0.f;
      for (int k = ia[i - 1]; k < ia[i]; ++k) s = std::fma(A(k), zk[JA(k)], s);
      out[i] = s;
    }
  };
  double betn = 0.0;
  for (int i = 1; i <= n; ++i) { reso[i] = res[i]; betn += (double)res[i] * (double)res[i]; }
  double alf = 1.0, beto = 1.0, gam = 1.0;
  int used = 0;
  double stall_ref = res0;
  int stall_at = 0;
  for (int l = 1; l <= itr_max; ++l) {
    const double bet = betn;
    const double om = bet * gam / (alf * beto + kSmall);
    beto = bet;
    const float omF = (float)om, alfF = (float)alf;
    for (int i = 1; i <= n; ++i) pk[i] = std::fma(omF, std::fma(-alfF, uk[i], pk[i]), res[i]);
    apply(pk);
    matvec(uk);
    double ur = 0.0;
    for (int i = 1; i <= n; ++i) ur += (double)uk[i] * (double)reso[i];
    gam = bet / ur;
    const float gF = (float)gam;
    for (int i = 1; i <= n; ++i) {
      x[i - 1] = std::fma(gF, zk[i], x[i - 1]);
      res[i] = std::fma(-gF, uk[i], res[i]);
    }
    apply(res);
    matvec(vk);
    double vr0 = 0.0, vr1 = 0.0;
    for (int i = 1; i <= n; ++i) {
      vr0 += (double)vk[i] * (double)res[i];
      vr1 += (double)vk[i] * (double)vk[i];
    }
    alf = vr0 / (vr1 + kSmall);
    const float aF = (float)alf;
    double resl = 0.0;
    betn = 0.0;
    for (int i = 1; i <= n; ++i) {
      x[i - 1] = std::fma(aF, zk[i], x[i - 1]);
      res[i] = std::fma(-aF, vk[i], res[i]);
      resl += std::fabs((double)res[i]);
      betn += (double)res[i] * (double)reso[i];
    }
    hist[l - 1] = resl;
    used = l;
    if (resl / (res0 + kSmall) < tol_rel) break;
    if (stall_window > 0) {
      if (resl < 0.5 * stall_ref) { stall_ref = resl; stall_at = l; }
      else if (l - stall_at >= stall_window) break;
    }
  }
  return used;
}
