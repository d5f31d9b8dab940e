// CPU check of the adjoint's log-conformation product (vebi_adjoint_logconf.cuh, test only).
//
// logconf_vjp chains three four-direction Jacobians backwards; the reference here is the full
// nine-direction forward mode through the whole update (logconf_eval over DualN<9>), contracted
// with the same adjoint seed, and central differences of the FP64 update itself.  Prints the
// largest relative differences (by kind of conformation: general, diagonal, at rest, eigenvalues
// within 1e-7); exits non-zero when one is above its bound.  The two products apply the chain rule
// in different orders, so they differ by rounding amplified by the update's own conditioning:
// the eigenvector turn a21 / (a11 - a22) and the factor 1 / (L2 - L1 + 1e-10).
#include <cmath>
#include <cstdio>
#include <random>

#include "vebi_adjoint_logconf.cuh"

using namespace vebi;

struct Case { double tau[4], G[4], dt, e1; };

static void full9(const Case& c, const double tb[4], double taub[4], double Gb[4], double& e1b) {
  typedef DualN<9> D9;
  D9 tau[4], G[4], out[4];
  for (int q = 0; q < 4; ++q) {
    tau[q] = D9(c.tau[q]);
    tau[q].d[q] = 1.0;
    G[q] = D9(c.G[q]);
    G[q].d[4 + q] = 1.0;
  }
  D9 e(c.e1);
  e.d[8] = 1.0;
  logconf_eval(tau, G, c.dt, e, out);
  for (int q = 0; q < 4; ++q) {
    taub[q] = 0.0;
    Gb[q] = 0.0;
    for (int r = 0; r < 4; ++r) {
      taub[q] += out[r].d[q] * tb[r];
      Gb[q] += out[r].d[4 + q] * tb[r];
    }
  }
  e1b = 0.0;
  for (int r = 0; r < 4; ++r) e1b += out[r].d[8] * tb[r];
}

static double J(const Case& c, const double tb[4]) {
  double out[4];
  logconf_eval(c.tau, c.G, c.dt, c.e1, out);
  double s = 0.0;
  for (int r = 0; r < 4; ++r) s += out[r] * tb[r];
  return s;
}

static double rel(const double* a, const double* b, int n) {
  double num = 0.0, den = 0.0;
  for (int q = 0; q < n; ++q) {
    num = std::fmax(num, std::fabs(a[q] - b[q]));
    den = std::fmax(den, std::fmax(std::fabs(a[q]), std::fabs(b[q])));
  }
  return den > 0.0 ? num / den : 0.0;
}

int main() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(-1.0, 1.0), L(0.2, 5.0);
  double worst_chain = 0.0, worst_fd = 0.0, worst_value = 0.0, by_kind[4] = {0.0, 0.0, 0.0, 0.0};
  int n_cases = 0;
  for (int k = 0; k < 4000; ++k) {
    Case c;
    const int kind = k % 4;  // 0 general, 1 diagonal (a21 == 0), 2 at rest (A = I), 3 close eigenvalues
    double l1 = L(rng), l2 = L(rng), th = 3.14159 * U(rng);
    if (kind == 2) l1 = l2 = 1.0;
    if (kind == 3) l2 = l1 * (1.0 + 1.0e-7 * U(rng));
    const double cs = std::cos(th), sn = std::sin(th);
    double a11 = cs * cs * l1 + sn * sn * l2, a22 = sn * sn * l1 + cs * cs * l2, a12 = cs * sn * (l1 - l2);
    if (kind == 1 || kind == 2) a12 = 0.0;
    c.tau[0] = a11 - 1.0;
    c.tau[1] = a12;
    c.tau[2] = a12;
    c.tau[3] = a22 - 1.0;
    for (int q = 0; q < 4; ++q) c.G[q] = 3.0 * U(rng);
    c.dt = 1.0e-3 * (1.0 + 9.0 * (0.5 + 0.5 * U(rng)));
    c.e1 = std::exp(-c.dt / (0.1 + 2.0 * (0.5 + 0.5 * U(rng))));
    double tb[4];
    for (int r = 0; r < 4; ++r) tb[r] = U(rng);
    double ta[4], ga[4], ea, tr[4], gr[4], er;
    logconf_vjp(c.tau, c.G, c.dt, c.e1, tb, ta, ga, ea);
    full9(c, tb, tr, gr, er);
    double all_a[9], all_r[9];
    for (int q = 0; q < 4; ++q) { all_a[q] = ta[q]; all_a[4 + q] = ga[q]; all_r[q] = tr[q]; all_r[4 + q] = gr[q]; }
    all_a[8] = ea;
    all_r[8] = er;
    worst_chain = std::fmax(worst_chain, rel(all_a, all_r, 9));
    by_kind[kind] = std::fmax(by_kind[kind], rel(all_a, all_r, 9));
    // the dual values are the FP64 update's, bit for bit
    {
      typedef DualN<9> D9;
      D9 t9[4], g9[4], o9[4];
      for (int q = 0; q < 4; ++q) { t9[q] = D9(c.tau[q]); g9[q] = D9(c.G[q]); }
      logconf_eval(t9, g9, c.dt, D9(c.e1), o9);
      double o[4];
      logconf_eval(c.tau, c.G, c.dt, c.e1, o);
      for (int r = 0; r < 4; ++r) worst_value = std::fmax(worst_value, o9[r].v == o[r] ? 0.0 : 1.0);
    }
    // central differences of the FP64 update, away from the branches (general cases only)
    if (kind == 0) {
      double fd[9];
      const double h = 1.0e-6;
      for (int q = 0; q < 9; ++q) {
        Case p = c, m = c;
        if (q < 4) { p.tau[q] += h; m.tau[q] -= h; }
        else if (q < 8) { p.G[q - 4] += h; m.G[q - 4] -= h; }
        else { p.e1 += h; m.e1 -= h; }
        fd[q] = (J(p, tb) - J(m, tb)) / (2.0 * h);
      }
      worst_fd = std::fmax(worst_fd, rel(all_a, fd, 9));
    }
    ++n_cases;
  }
  std::printf("cases %d  chained vs nine-direction: %.3e (general %.2e, diagonal %.2e, at rest %.2e, close "
              "eigenvalues %.2e)  vs central differences: %.3e  values differ: %.0f\n",
              n_cases, worst_chain, by_kind[0], by_kind[1], by_kind[2], by_kind[3], worst_fd, worst_value);
  return (worst_chain <= 1.0e-10 && by_kind[0] <= 1.0e-11 && worst_fd <= 1.0e-5 && worst_value == 0.0) ? 0 : 1;
}
