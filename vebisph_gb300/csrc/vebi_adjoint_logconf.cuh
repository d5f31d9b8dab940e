// vebi_adjoint_logconf.cuh -- the log-conformation update of one particle written once over a
// scalar type, so that the adjoint evaluates its Jacobian in forward mode.
//
// logconf_eval<double> is k_logconf's arithmetic (constitutive_eqn_evolve, predictor_mod.F90:
// 141-251, with calc_eigens :253-290 and the Oldroyd-B relaxation :292-331) operation for
// operation; logconf_eval<Dual9> carries nine directional derivatives along: the four stress
// planes, the four velocity-gradient entries and the relaxation factor e1 = exp(-dt/Wi).  The
// branches (the eigenvalue clamp, a21 == 0) follow the values, as the step takes them.
#pragma once
#include <cuda_runtime.h>

namespace vebi {

constexpr int NDUAL = 9;

struct Dual9 {
  double v;
  double d[NDUAL];
  __device__ Dual9() {}
  __device__ Dual9(double x) : v(x) {
#pragma unroll
    for (int q = 0; q < NDUAL; ++q) d[q] = 0.0;
  }
};
__device__ __forceinline__ Dual9 operator+(const Dual9& a, const Dual9& b) {
  Dual9 r;
  r.v = a.v + b.v;
#pragma unroll
  for (int q = 0; q < NDUAL; ++q) r.d[q] = a.d[q] + b.d[q];
  return r;
}
__device__ __forceinline__ Dual9 operator-(const Dual9& a, const Dual9& b) {
  Dual9 r;
  r.v = a.v - b.v;
#pragma unroll
  for (int q = 0; q < NDUAL; ++q) r.d[q] = a.d[q] - b.d[q];
  return r;
}
__device__ __forceinline__ Dual9 operator-(const Dual9& a) {
  Dual9 r;
  r.v = -a.v;
#pragma unroll
  for (int q = 0; q < NDUAL; ++q) r.d[q] = -a.d[q];
  return r;
}
__device__ __forceinline__ Dual9 operator*(const Dual9& a, const Dual9& b) {
  Dual9 r;
  r.v = a.v * b.v;
#pragma unroll
  for (int q = 0; q < NDUAL; ++q) r.d[q] = a.d[q] * b.v + a.v * b.d[q];
  return r;
}
__device__ __forceinline__ Dual9 operator/(const Dual9& a, const Dual9& b) {
  Dual9 r;
  r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int q = 0; q < NDUAL; ++q) r.d[q] = (a.d[q] - r.v * b.d[q]) * ib;
  return r;
}
__device__ __forceinline__ Dual9 operator+(const Dual9& a, double b) { Dual9 r = a; r.v = a.v + b; return r; }
__device__ __forceinline__ Dual9 operator+(double a, const Dual9& b) { return b + a; }
__device__ __forceinline__ Dual9 operator-(const Dual9& a, double b) { Dual9 r = a; r.v = a.v - b; return r; }
__device__ __forceinline__ Dual9 operator-(double a, const Dual9& b) { return -(b - a); }
__device__ __forceinline__ Dual9 operator*(const Dual9& a, double b) {
  Dual9 r;
  r.v = a.v * b;
#pragma unroll
  for (int q = 0; q < NDUAL; ++q) r.d[q] = a.d[q] * b;
  return r;
}
__device__ __forceinline__ Dual9 operator*(double a, const Dual9& b) { return b * a; }
__device__ __forceinline__ Dual9 operator/(const Dual9& a, double b) {
  Dual9 r;
  r.v = a.v / b;
#pragma unroll
  for (int q = 0; q < NDUAL; ++q) r.d[q] = a.d[q] / b;
  return r;
}
__device__ __forceinline__ Dual9 dsqrt(const Dual9& a) {
  Dual9 r;
  r.v = sqrt(a.v);
  const double f = r.v > 0.0 ? 0.5 / r.v : 0.0;
#pragma unroll
  for (int q = 0; q < NDUAL; ++q) r.d[q] = a.d[q] * f;
  return r;
}
__device__ __forceinline__ Dual9 dlog(const Dual9& a) {
  Dual9 r;
  r.v = log(a.v);
  const double f = 1.0 / a.v;
#pragma unroll
  for (int q = 0; q < NDUAL; ++q) r.d[q] = a.d[q] * f;
  return r;
}
__device__ __forceinline__ Dual9 dexp(const Dual9& a) {
  Dual9 r;
  r.v = exp(a.v);
#pragma unroll
  for (int q = 0; q < NDUAL; ++q) r.d[q] = a.d[q] * r.v;
  return r;
}
__device__ __forceinline__ double val(double a) { return a; }
__device__ __forceinline__ double val(const Dual9& a) { return a.v; }
__device__ __forceinline__ double dsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ double dlog(double a) { return log(a); }
__device__ __forceinline__ double dexp(double a) { return exp(a); }

template <class T>
struct M2T {
  T a11, a12, a21, a22;
};
template <class T>
__device__ __forceinline__ M2T<T> mmT(const M2T<T>& A, const M2T<T>& B) {
  return M2T<T>{A.a11 * B.a11 + A.a12 * B.a21, A.a11 * B.a12 + A.a12 * B.a22,
                A.a21 * B.a11 + A.a22 * B.a21, A.a21 * B.a12 + A.a22 * B.a22};
}
template <class T>
__device__ __forceinline__ M2T<T> trT(const M2T<T>& A) {
  return M2T<T>{A.a11, A.a21, A.a12, A.a22};
}

// The a21 == 0 branch below sets R = I, the limit of the general branch as a21 -> 0 (for
// a11 != a22 the eigenvector of L1 = a11 turns by a21 / (a11 - a22)).  Its values are those of
// the continuous map A -> R f(Lambda) R^T, but a literal derivative of the branch would drop
// that turn; the dual carrier adds it to R's off-diagonal entries.
__device__ __forceinline__ void diag_branch_turn(M2T<double>&, const M2T<double>&) {}
__device__ __forceinline__ void diag_branch_turn(M2T<Dual9>& R, const M2T<Dual9>& A) {
  const double gap = A.a11.v - A.a22.v;
  if (gap == 0.0) return;
#pragma unroll
  for (int q = 0; q < NDUAL; ++q) {
    const double ds = A.a21.d[q] / gap;
    R.a21.d[q] = ds;
    R.a12.d[q] = -ds;
  }
}

template <class T>
__device__ __forceinline__ void eigensT(const M2T<T>& A, T& L1, T& L2, M2T<T>& R) {
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

// tau = (t11, t21, t12, t22) planes 0..3, G = (du/dx, du/dy, dv/dx, dv/dy); out as tau
template <class T>
__device__ void logconf_eval(const T tau[4], const T G[4], double dt, const T& e1, T out[4]) {
  M2T<T> A{tau[0] / 1.0 + 1.0, tau[2] / 1.0 + 0.0, tau[1] / 1.0 + 0.0, tau[3] / 1.0 + 1.0};
  A = M2T<T>{A.a11 / 1.0, A.a12 / 1.0, A.a21 / 1.0, A.a22 / 1.0};
  T L1, L2;
  M2T<T> R;
  eigensT(A, L1, L2, R);
  const T z = T(0.0);
  M2T<T> D{dlog(L1), z, z, dlog(L2)};
  M2T<T> Psi0 = mmT(R, mmT(D, trT(R)));
  M2T<T> Gm{G[0], G[1], G[2], G[3]};
  M2T<T> tm = mmT(trT(R), mmT(Gm, R));
  T tmp1 = (L2 * tm.a12 + L1 * tm.a21) / (L2 - L1 + 1e-10);
  tm.a12 = z;
  tm.a21 = z;
  M2T<T> B = mmT(R, mmT(tm, trT(R)));
  M2T<T> W{z, tmp1, -tmp1, z};
  M2T<T> Om = mmT(R, mmT(W, trT(R)));
  M2T<T> OP = mmT(Om, Psi0), PO = mmT(Psi0, Om);
  M2T<T> t6{2.0 * B.a11 + OP.a11 - PO.a11, 2.0 * B.a12 + OP.a12 - PO.a12, 2.0 * B.a21 + OP.a21 - PO.a21,
            2.0 * B.a22 + OP.a22 - PO.a22};
  M2T<T> Psi{Psi0.a11 + dt * t6.a11, Psi0.a12 + dt * t6.a12, Psi0.a21 + dt * t6.a21, Psi0.a22 + dt * t6.a22};
  eigensT(Psi, L1, L2, R);
  L1 = dexp(L1);
  L2 = dexp(L2);
  M2T<T> E2{L1, z, z, L2};
  A = mmT(R, mmT(E2, trT(R)));
  const T e2 = (1.0 - e1) / 1.0;
  A = M2T<T>{A.a11 * e1 + e2 * 1.0, A.a12 * e1 + e2 * 0.0, A.a21 * e1 + e2 * 0.0, A.a22 * e1 + e2 * 1.0};
  out[0] = 1.0 * (1.0 * A.a11 - 1.0);
  out[2] = 1.0 * (1.0 * A.a12 - 0.0);
  out[1] = 1.0 * (1.0 * A.a21 - 0.0);
  out[3] = 1.0 * (1.0 * A.a22 - 1.0);
}

}  // namespace vebi
