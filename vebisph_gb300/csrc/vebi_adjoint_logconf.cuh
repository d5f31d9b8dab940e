// vebi_adjoint_logconf.cuh -- the log-conformation update of one particle written once over a
// scalar type, so that the adjoint evaluates its derivatives in forward mode.
//
// The update is k_logconf's arithmetic (constitutive_eqn_evolve, predictor_mod.F90:141-251,
// with calc_eigens :253-290 and the Oldroyd-B relaxation :292-331), operation for operation, in
// four parts:
//   logconf_first  A = tau + I -> eigen-decomposition (L, R) -> Psi0 = R log(L) R^T
//   logconf_rate   the rate 2B + Om Psi0 - Psi0 Om from the velocity gradient G (linear in G)
//   logconf_exp    Psi = Psi0 + dt rate -> eigen-decomposition -> R' exp(L') R'^T
//   logconf_relax  the relaxation A e1 + (1 - e1) I and tau = A - I
// logconf_eval composes them.  Over DualN<N> each part carries N directional derivatives; the
// branches (the eigenvalue clamp, a21 == 0) follow the values, as the step takes them.
//
// logconf_vjp is the adjoint's product (tau-bar, G-bar, e1-bar) = J^T out-bar.  It needs no
// nine-direction pass through the whole update: it takes Psi's Jacobian over the stress planes
// and the exponential's over the entries of Psi in forward mode (four directions each), the
// rate's over the entries of G as the rates of the four unit G (the rate is linear in G), and
// chains them backwards; the relaxation's derivatives are written out.  logconf_eval<DualN<9>>
// (all nine inputs through the whole update) gives the same products and is kept for checking it.
//
// Everything here is __host__ __device__ so that the products can be checked on the CPU.
#pragma once
#include <cuda_runtime.h>

#include <cmath>

#define VEBI_HD __host__ __device__ __forceinline__

namespace vebi {

template <int N>
struct DualN {
  double v;
  double d[N];
  VEBI_HD DualN() {}
  VEBI_HD DualN(double x) : v(x) {
#pragma unroll
    for (int q = 0; q < N; ++q) d[q] = 0.0;
  }
};
template <int N>
VEBI_HD DualN<N> operator+(const DualN<N>& a, const DualN<N>& b) {
  DualN<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] + b.d[q];
  return r;
}
template <int N>
VEBI_HD DualN<N> operator-(const DualN<N>& a, const DualN<N>& b) {
  DualN<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] - b.d[q];
  return r;
}
template <int N>
VEBI_HD DualN<N> operator-(const DualN<N>& a) {
  DualN<N> r;
  r.v = -a.v;
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = -a.d[q];
  return r;
}
template <int N>
VEBI_HD DualN<N> operator*(const DualN<N>& a, const DualN<N>& b) {
  DualN<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] * b.v + a.v * b.d[q];
  return r;
}
template <int N>
VEBI_HD DualN<N> operator/(const DualN<N>& a, const DualN<N>& b) {
  DualN<N> r;
  r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = (a.d[q] - r.v * b.d[q]) * ib;
  return r;
}
template <int N>
VEBI_HD DualN<N> operator+(const DualN<N>& a, double b) {
  DualN<N> r = a;
  r.v = a.v + b;
  return r;
}
template <int N>
VEBI_HD DualN<N> operator+(double a, const DualN<N>& b) {
  return b + a;
}
template <int N>
VEBI_HD DualN<N> operator-(const DualN<N>& a, double b) {
  DualN<N> r = a;
  r.v = a.v - b;
  return r;
}
template <int N>
VEBI_HD DualN<N> operator-(double a, const DualN<N>& b) {
  return -(b - a);
}
template <int N>
VEBI_HD DualN<N> operator*(const DualN<N>& a, double b) {
  DualN<N> r;
  r.v = a.v * b;
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] * b;
  return r;
}
template <int N>
VEBI_HD DualN<N> operator*(double a, const DualN<N>& b) {
  return b * a;
}
template <int N>
VEBI_HD DualN<N> operator/(const DualN<N>& a, double b) {
  DualN<N> r;
  r.v = a.v / b;
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] / b;
  return r;
}
template <int N>
VEBI_HD DualN<N> dsqrt(const DualN<N>& a) {
  DualN<N> r;
  r.v = sqrt(a.v);
  const double f = r.v > 0.0 ? 0.5 / r.v : 0.0;
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] * f;
  return r;
}
template <int N>
VEBI_HD DualN<N> dlog(const DualN<N>& a) {
  DualN<N> r;
  r.v = log(a.v);
  const double f = 1.0 / a.v;
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] * f;
  return r;
}
template <int N>
VEBI_HD DualN<N> dexp(const DualN<N>& a) {
  DualN<N> r;
  r.v = exp(a.v);
#pragma unroll
  for (int q = 0; q < N; ++q) r.d[q] = a.d[q] * r.v;
  return r;
}
VEBI_HD double val(double a) { return a; }
template <int N>
VEBI_HD double val(const DualN<N>& a) {
  return a.v;
}
VEBI_HD double dsqrt(double a) { return sqrt(a); }
VEBI_HD double dlog(double a) { return log(a); }
VEBI_HD double dexp(double a) { return exp(a); }

template <class T>
struct M2T {
  T a11, a12, a21, a22;
};
template <class T>
VEBI_HD M2T<T> mmT(const M2T<T>& A, const M2T<T>& B) {
  return M2T<T>{A.a11 * B.a11 + A.a12 * B.a21, A.a11 * B.a12 + A.a12 * B.a22,
                A.a21 * B.a11 + A.a22 * B.a21, A.a21 * B.a12 + A.a22 * B.a22};
}
template <class T>
VEBI_HD M2T<T> trT(const M2T<T>& A) {
  return M2T<T>{A.a11, A.a21, A.a12, A.a22};
}

// The a21 == 0 branch below sets R = I, the limit of the general branch as a21 -> 0 (for
// a11 != a22 the eigenvector of L1 = a11 turns by a21 / (a11 - a22)).  Its values are those of
// the continuous map A -> R f(Lambda) R^T, but a literal derivative of the branch would drop
// that turn; the dual carrier adds it to R's off-diagonal entries.
VEBI_HD void diag_branch_turn(M2T<double>&, const M2T<double>&) {}
template <int N>
VEBI_HD void diag_branch_turn(M2T<DualN<N>>& R, const M2T<DualN<N>>& A) {
  const double gap = A.a11.v - A.a22.v;
  if (gap == 0.0) return;
#pragma unroll
  for (int q = 0; q < N; ++q) {
    const double ds = A.a21.d[q] / gap;
    R.a21.d[q] = ds;
    R.a12.d[q] = -ds;
  }
}

template <class T>
VEBI_HD void eigensT(const M2T<T>& A, T& L1, T& L2, M2T<T>& R) {
  T trc = A.a11 + A.a22;
  T det = A.a11 * A.a22 - A.a21 * A.a12;
  T tmp = 0.25 * trc * trc - det;
  if (val(tmp) <= 2.220446049250313e-16) tmp = T(0.0);
  T sq = dsqrt(tmp);
  L1 = 0.5 * trc + sq;
  L2 = 0.5 * trc - sq;
  if (val(A.a21) != 0.0) {
    T r11 = L1 - A.a22, r21 = A.a21;
    T nrm = dsqrt(r11 * r11 + r21 * r21);
    r11 = r11 / nrm;
    r21 = r21 / nrm;
    R = M2T<T>{r11, -r21, r21, r11};
  } else {
    L1 = A.a11;
    L2 = A.a22;
    R = M2T<T>{T(1.0), T(0.0), T(0.0), T(1.0)};
    diag_branch_turn(R, A);
  }
}

// tau = (t11, t21, t12, t22) planes 0..3 -> eigen-decomposition of A = tau + I and Psi0 = log A
template <class T>
VEBI_HD void logconf_first(const T tau[4], M2T<T>& R, T& L1, T& L2, M2T<T>& Psi0) {
  M2T<T> A{tau[0] / 1.0 + 1.0, tau[2] / 1.0 + 0.0, tau[1] / 1.0 + 0.0, tau[3] / 1.0 + 1.0};
  A = M2T<T>{A.a11 / 1.0, A.a12 / 1.0, A.a21 / 1.0, A.a22 / 1.0};
  eigensT(A, L1, L2, R);
  const T z = T(0.0);
  M2T<T> D{dlog(L1), z, z, dlog(L2)};
  Psi0 = mmT(R, mmT(D, trT(R)));
}

// G = (du/dx, du/dy, dv/dx, dv/dy) -> the rate 2B + Om Psi0 - Psi0 Om (linear in G)
template <class T>
VEBI_HD M2T<T> logconf_rate(const M2T<T>& R, const T& L1, const T& L2, const M2T<T>& Psi0, const T G[4]) {
  const T z = T(0.0);
  M2T<T> Gm{G[0], G[1], G[2], G[3]};
  M2T<T> tm = mmT(trT(R), mmT(Gm, R));
  T tmp1 = (L2 * tm.a12 + L1 * tm.a21) / (L2 - L1 + 1e-10);
  tm.a12 = z;
  tm.a21 = z;
  M2T<T> B = mmT(R, mmT(tm, trT(R)));
  M2T<T> W{z, tmp1, -tmp1, z};
  M2T<T> Om = mmT(R, mmT(W, trT(R)));
  M2T<T> OP = mmT(Om, Psi0), PO = mmT(Psi0, Om);
  return M2T<T>{2.0 * B.a11 + OP.a11 - PO.a11, 2.0 * B.a12 + OP.a12 - PO.a12, 2.0 * B.a21 + OP.a21 - PO.a21,
                2.0 * B.a22 + OP.a22 - PO.a22};
}

// Psi -> exp(Psi) through its eigen-decomposition
template <class T>
VEBI_HD M2T<T> logconf_exp(const M2T<T>& Psi) {
  T L1, L2;
  M2T<T> R;
  eigensT(Psi, L1, L2, R);
  L1 = dexp(L1);
  L2 = dexp(L2);
  const T z = T(0.0);
  M2T<T> E2{L1, z, z, L2};
  return mmT(R, mmT(E2, trT(R)));
}

// the relaxation with factor e1 = exp(-dt/Wi) and tau = A - I, out as tau
template <class T>
VEBI_HD void logconf_relax(M2T<T> A, const T& e1, T out[4]) {
  const T e2 = (1.0 - e1) / 1.0;
  A = M2T<T>{A.a11 * e1 + e2 * 1.0, A.a12 * e1 + e2 * 0.0, A.a21 * e1 + e2 * 0.0, A.a22 * e1 + e2 * 1.0};
  out[0] = 1.0 * (1.0 * A.a11 - 1.0);
  out[2] = 1.0 * (1.0 * A.a12 - 0.0);
  out[1] = 1.0 * (1.0 * A.a21 - 0.0);
  out[3] = 1.0 * (1.0 * A.a22 - 1.0);
}

// tau = (t11, t21, t12, t22) planes 0..3, G = (du/dx, du/dy, dv/dx, dv/dy); out as tau
template <class T>
VEBI_HD void logconf_eval(const T tau[4], const T G[4], double dt, const T& e1, T out[4]) {
  M2T<T> R, Psi0;
  T L1, L2;
  logconf_first(tau, R, L1, L2, Psi0);
  M2T<T> t6 = logconf_rate(R, L1, L2, Psi0, G);
  M2T<T> Psi{Psi0.a11 + dt * t6.a11, Psi0.a12 + dt * t6.a12, Psi0.a21 + dt * t6.a21, Psi0.a22 + dt * t6.a22};
  logconf_relax(logconf_exp(Psi), e1, out);
}

// (taub, Gb, e1b) = J^T tb for out = logconf_eval(tau, G, dt, e1); tb, taub in tau's plane order
VEBI_HD void logconf_vjp(const double tau[4], const double G[4], double dt, double e1, const double tb[4],
                         double taub[4], double Gb[4], double& e1b) {
  typedef DualN<4> D4;
  // Psi and its derivatives over the four stress planes (G held)
  D4 tA[4], GA[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    tA[q] = D4(tau[q]);
    tA[q].d[q] = 1.0;
    GA[q] = D4(G[q]);
  }
  M2T<D4> R, Psi0;
  D4 L1, L2;
  logconf_first(tA, R, L1, L2, Psi0);
  M2T<D4> t6 = logconf_rate(R, L1, L2, Psi0, GA);
  M2T<D4> Psi{Psi0.a11 + dt * t6.a11, Psi0.a12 + dt * t6.a12, Psi0.a21 + dt * t6.a21, Psi0.a22 + dt * t6.a22};
  // the rate's derivatives over the four entries of G, at the same R, L, Psi0: the rate is
  // linear in G, so they are the rate of each unit G
  const M2T<double> Rv{R.a11.v, R.a12.v, R.a21.v, R.a22.v};
  const M2T<double> P0v{Psi0.a11.v, Psi0.a12.v, Psi0.a21.v, Psi0.a22.v};
  double rG[4][4];  // [q][p]: d rate_p / d G_q, p over (a11, a12, a21, a22)
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const double Gq[4] = {q == 0 ? 1.0 : 0.0, q == 1 ? 1.0 : 0.0, q == 2 ? 1.0 : 0.0, q == 3 ? 1.0 : 0.0};
    const M2T<double> r = logconf_rate(Rv, L1.v, L2.v, P0v, Gq);
    rG[q][0] = r.a11;
    rG[q][1] = r.a12;
    rG[q][2] = r.a21;
    rG[q][3] = r.a22;
  }
  // exp(Psi) and its derivatives over the entries of Psi (a11, a12, a21, a22)
  M2T<D4> PB{D4(Psi.a11.v), D4(Psi.a12.v), D4(Psi.a21.v), D4(Psi.a22.v)};
  PB.a11.d[0] = 1.0;
  PB.a12.d[1] = 1.0;
  PB.a21.d[2] = 1.0;
  PB.a22.d[3] = 1.0;
  M2T<D4> Ax = logconf_exp(PB);
  // backwards: out = e1 (Ax - I) in the planes (a11, a21, a12, a22)
  const double b11 = tb[0] * e1, b21 = tb[1] * e1, b12 = tb[2] * e1, b22 = tb[3] * e1;
  e1b = tb[0] * (Ax.a11.v - 1.0) + tb[1] * Ax.a21.v + tb[2] * Ax.a12.v + tb[3] * (Ax.a22.v - 1.0);
  double pb[4];  // Psi-bar over (a11, a12, a21, a22)
#pragma unroll
  for (int p = 0; p < 4; ++p) pb[p] = b11 * Ax.a11.d[p] + b12 * Ax.a12.d[p] + b21 * Ax.a21.d[p] + b22 * Ax.a22.d[p];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    taub[q] = pb[0] * Psi.a11.d[q] + pb[1] * Psi.a12.d[q] + pb[2] * Psi.a21.d[q] + pb[3] * Psi.a22.d[q];
    Gb[q] = dt * (pb[0] * rG[q][0] + pb[1] * rG[q][1] + pb[2] * rG[q][2] + pb[3] * rG[q][3]);
  }
}

}  // namespace vebi

#undef VEBI_HD
