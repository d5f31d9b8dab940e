// vebi_oracle.cpp -- CPU oracle for the vebisph time step (TEST INFRASTRUCTURE ONLY).
//
// This file restates, in C++17 FP64, the reference's time step `div_free`
// (source/base/div_free.F90:22-124) and every routine it calls, so that the GPU library
// can be checked against it on the same inputs.  It is the checker, never the product:
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
//
// PARITY STATUS: parity with the Fortran binary is UNPINNED.  The reference is Fortran 90
// + OpenMP, no Fortran compiler exists where this is built, and the reference ships no tests
// or golden vectors.  This restatement is pinned instead by analytic known-answer tests
// (tests/test_oracle_kat.py) and by the shipped case deck (tests/golden/).
//
// Restatement rules:
//  * loop orders, neighbour order (C,E,NE,SE,W,NW,SW,N,S), mirror order (global `imp`
//    counter), constants, and expression association follow the Fortran source;
//  * compiled with -ffp-contract=off (no FMA), matching gfortran's x86-64 default;
//  * integer powers q**4, q**5 are expanded as gfortran's powi does: x4=(x*x)*(x*x),
//    x5=(x*x)*(x*(x*x));
//  * default-real (single precision) literals that are not exactly representable are
//    promoted from float, as Fortran does (`0.01*h*h` in kernel_calculation.F90:36);
//  * reductions are summed in fixed chunks of 4096 in index order, then the chunk
//    partials in order: deterministic and independent of the OpenMP thread count
//    (the reference's OpenMP reductions are not);
//  * the data races of the reference (put_in_bin.F90:34-47 counters,
//    new_fick_shift.F90:32-36 `maxU = temp` under reduction(max)) are given their
//    intended meaning (a count; a maximum).
//
// Indexing: 0-based.  Particle i here is particle i+1 of the reference.  Integer codes
// (vrelation, b_periodic_parent) keep the reference's 1-based patch numbers.
//
// Tangent-linear model.  The step is written once over the scalar type of its fields
// (OracleT<R>): OracleT<double> is the restatement; OracleT<Tan> runs the same code over
// forward-mode dual numbers (orc_tlm_*), giving the FP64 tangent-linear model of the step with
// the geometry (positions, dt, pair lists, weights, PPE matrix) of the unperturbed trajectory.
// It is the reference gradient the GPU adjoint is checked against.  orc_geometry records and
// replays r* and dt of an FP64 run, so that central differences see the same map.

#include "../include/vebi.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double PI = 3.14159265358979323846;  // common_parameter.F90:12
constexpr int CHUNK = 4096;

inline double pw2(double x) { return x * x; }
inline double pw4(double x) { double x2 = x * x; return x2 * x2; }
inline double pw5(double x) { double x2 = x * x; double x3 = x * x2; return x2 * x3; }

// ---------------------------------------------------------------------- field scalar types
// The step is written once over the scalar type R of the particle fields (u, theta, tau, P and
// everything computed from them).  R = double is the restatement itself.  R = Tan carries one
// directional derivative along (forward mode), which turns the same code into the FP64
// tangent-linear model of the step: positions, dt, pair lists, kernel weights, correction
// matrices and the PPE matrix stay plain doubles computed from the values, so the geometry of
// every step is that of the unperturbed trajectory and only the fields are differentiated.
struct Tan {
  double v = 0.0, d = 0.0;
  Tan() = default;
  Tan(double x) : v(x), d(0.0) {}  // NOLINT: a constant carries no derivative
  Tan(double x, double y) : v(x), d(y) {}
};
inline Tan operator+(const Tan& a, const Tan& b) { return Tan(a.v + b.v, a.d + b.d); }
inline Tan operator-(const Tan& a, const Tan& b) { return Tan(a.v - b.v, a.d - b.d); }
inline Tan operator-(const Tan& a) { return Tan(-a.v, -a.d); }
inline Tan operator*(const Tan& a, const Tan& b) { return Tan(a.v * b.v, a.d * b.v + a.v * b.d); }
inline Tan operator/(const Tan& a, const Tan& b) {
  double q = a.v / b.v;
  return Tan(q, (a.d - q * b.d) / b.v);
}
inline Tan operator+(const Tan& a, double b) { return Tan(a.v + b, a.d); }
inline Tan operator+(double a, const Tan& b) { return Tan(a + b.v, b.d); }
inline Tan operator-(const Tan& a, double b) { return Tan(a.v - b, a.d); }
inline Tan operator-(double a, const Tan& b) { return Tan(a - b.v, -b.d); }
inline Tan operator*(const Tan& a, double b) { return Tan(a.v * b, a.d * b); }
inline Tan operator*(double a, const Tan& b) { return Tan(a * b.v, a * b.d); }
inline Tan operator/(const Tan& a, double b) { return Tan(a.v / b, a.d / b); }
inline Tan operator/(double a, const Tan& b) {
  double q = a / b.v;
  return Tan(q, -q * b.d / b.v);
}
inline Tan& operator+=(Tan& a, const Tan& b) { a = a + b; return a; }
// branches follow the values, as the step takes them
inline bool operator<(const Tan& a, const Tan& b) { return a.v < b.v; }
inline bool operator>(const Tan& a, const Tan& b) { return a.v > b.v; }
inline bool operator<=(const Tan& a, const Tan& b) { return a.v <= b.v; }
inline bool operator>=(const Tan& a, const Tan& b) { return a.v >= b.v; }
inline bool operator==(const Tan& a, const Tan& b) { return a.v == b.v; }
inline bool operator!=(const Tan& a, const Tan& b) { return a.v != b.v; }

inline double val(double x) { return x; }
inline double val(const Tan& x) { return x.v; }
inline double Sqrt(double x) { return std::sqrt(x); }
inline double Exp(double x) { return std::exp(x); }
inline double Log(double x) { return std::log(x); }
// d sqrt at 0 is taken as 0: the only zero argument is the clamped eigen discriminant, a constant
inline Tan Sqrt(const Tan& x) {
  double s = std::sqrt(x.v);
  return Tan(s, s > 0.0 ? 0.5 * x.d / s : 0.0);
}
inline Tan Exp(const Tan& x) {
  double e = std::exp(x.v);
  return Tan(e, e * x.d);
}
inline Tan Log(const Tan& x) { return Tan(std::log(x.v), x.d / x.v); }

template <class T>
struct M2T { T a11, a12, a21, a22; };  // 2x2 matrix, Fortran (row,col)
using M2 = M2T<double>;
template <class A, class B>
inline auto mm(const M2T<A>& X, const M2T<B>& Y) {  // matmul, inner index ascending
  M2T<decltype(A() * B())> C;
  C.a11 = X.a11 * Y.a11 + X.a12 * Y.a21;
  C.a12 = X.a11 * Y.a12 + X.a12 * Y.a22;
  C.a21 = X.a21 * Y.a11 + X.a22 * Y.a21;
  C.a22 = X.a21 * Y.a12 + X.a22 * Y.a22;
  return C;
}
template <class T>
inline M2T<T> tr(const M2T<T>& A) { return M2T<T>{A.a11, A.a21, A.a12, A.a22}; }

template <class F>
auto chunk_sum(int64_t n0, int64_t n1, F f) {
  using S = decltype(f(n0) + 0.0);
  int64_t n = n1 - n0;
  if (n <= 0) return S(0.0);
  int64_t nch = (n + CHUNK - 1) / CHUNK;
  std::vector<S> part(nch);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nch; ++c) {
    S s = 0.0;
    int64_t a = n0 + c * CHUNK, b = std::min(n1, a + CHUNK);
    for (int64_t i = a; i < b; ++i) s += f(i);
    part[c] = s;
  }
  S s = 0.0;
  for (int64_t c = 0; c < nch; ++c) s += part[c];
  return s;
}

template <class R>
struct OracleT {
  vebi_params P{};
  // constants set by getdata (input.F90:164-172)
  double h = 0, h2 = 0, sup_size = 0, sup_size_2 = 0, uno_sup_size = 0, ad_7 = 0, ad_7h = 0,
         eta2 = 0, dx = 0, dv = 0;
  double x_mint = 0, x_maxt = 0, y_mint = 0, y_maxt = 0;
  int ncx = 0, ncy = 0, nct = 0;
  int npfb = 0, nbS = 0, np = 0, nmirror = 0, cap = 0, mcap = 0, nplink = 75;
  int nb = 0, ncirc = 0;
  double b_corner_angle[VEBI_MAX_PATCHES]{};
  double dt = 0, umax = 0, time = 0;
  int LS_iters = 0;
  double LS_residual = 0;
  int n_inbin = 0, n_escapees = 0, error = 0, warnings = 0;
  double ppe_rhs_mean = 0, rms_u = 0;
  double circle_fx = 0, circle_fy = 0;     // force of the fluid on the circles (diagnostic)
  std::vector<R> circ_s1, circ_s2;         // circle-mirror share of the predictor sums
  int maxneighbours = 0;
  double t_solve_ms = 0.0, t_step_ms = 0.0;  // per-step wall times (CPU baseline)
  static double wtime() {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
  }

  // particle fields (R) and geometry (double), capacity cap = npfb + mirror capacity
  std::vector<double> rx, ry, conc, div_r;
  std::vector<R> ux, uy, theta, p, tau[4], trace_conf, a_out, vort;
  std::vector<int> n_surf;
  std::vector<uint8_t> inbin;
  std::vector<int> irelation, vrelation;
  std::vector<double> dP_mp;
  // step temporaries kept for inspection
  std::vector<double> r0x, r0y, rsx, rsy;  // r0, and r* used for neighbours
  std::vector<R> u0x, u0y;                 // u0
  std::vector<int> cellpart, ist, ipl, ncell;
  std::vector<int> ij_count, ij_link;  // ij_link[k*npfb+i]
  std::vector<double> wGx, wGy, wL, kgcm[4];
  std::vector<R> grad[6];              // du/dx,du/dy,dv/dx,dv/dy,dth/dx,dth/dy over np
  std::vector<double> ushx, ushy, drx, dry, gradCx, gradCy;
  std::vector<R> ustx, usty, thst;     // u*, theta* after the predictor (+ mirror u*)
  std::vector<R> ppe_B;
  std::vector<double> ppe_diag, ppe_val;
  std::vector<int> ppe_col;
  std::vector<R> gpx, gpy;
  std::vector<double> surf_nx, surf_ny, ppe_smooth;
  // geometry record/replay: r* (after binning) and dt of each step, so that a rerun from
  // perturbed fields sees the recorded geometry (the map the tangent-linear model differentiates)
  int geo_mode = 0;  // 0 off, 1 record, 2 replay
  size_t geo_step = 0;
  std::vector<std::vector<double>> geo_rx, geo_ry;
  std::vector<double> geo_dt;

  // ------------------------------------------------------------------ geometry helpers
  // bound_dist (mirror_boundaries_mod.F90:447-462): signed distance of a point to patch ib
  double bound_dist_xy(double x, double y, int ib) const {
    int ibp1 = (ib + 1) % nb;
    double p_dist = P.b_edge[ib][1] * x - P.b_edge[ib][0] * y +
                    P.b_node[ibp1][0] * P.b_node[ib][1] - P.b_node[ibp1][1] * P.b_node[ib][0];
    p_dist = -1.0 * p_dist /
             std::sqrt(P.b_edge[ib][0] * P.b_edge[ib][0] + P.b_edge[ib][1] * P.b_edge[ib][1]);
    return p_dist;
  }
  double bound_dist(int i, int ib) const { return bound_dist_xy(rx[i], ry[i], ib); }
  // bound_norm (:464-474)
  void bound_norm(int ib, double& n1, double& n2) const {
    double tmp1 =
        std::sqrt(P.b_edge[ib][0] * P.b_edge[ib][0] + P.b_edge[ib][1] * P.b_edge[ib][1]);
    n1 = -1.0 * P.b_edge[ib][1] / tmp1;
    n2 = P.b_edge[ib][0] / tmp1;
  }
  // position_along_patch (:476-491), with the module globals perp_dist, norm_be passed in
  double position_along_patch_xy(double x, double y, int ib, double perp, double n1,
                                 double n2) const {
    if (std::fabs(P.b_edge[ib][0]) > std::fabs(P.b_edge[ib][1]))
      return (x - P.b_node[ib][0] - perp * n1) / P.b_edge[ib][0];
    return (y - P.b_node[ib][1] - perp * n2) / P.b_edge[ib][1];
  }
  // angle_between_patches (:493-507)
  M2 angle_between_patches(int a, int b) const {
    double ta = P.b_edge[a][0] * P.b_edge[b][0] + P.b_edge[a][1] * P.b_edge[b][1];
    double na = P.b_edge[a][0] * P.b_edge[a][0] + P.b_edge[a][1] * P.b_edge[a][1];
    double nbb = P.b_edge[b][0] * P.b_edge[b][0] + P.b_edge[b][1] * P.b_edge[b][1];
    double t = ta / std::sqrt(na * nbb);
    t = std::acos(t) - PI;
    return M2{std::cos(t), -std::sin(t), std::sin(t), std::cos(t)};
  }

  // ------------------------------------------------------------------ kernels (sphtools.F90)
  // fac (sphtools.F90:11-44): derivative of the quintic spline
  double fac(double qq) const {
    int isel = (int)std::floor(qq);
    if (isel == 0) {
      double q3 = 3.0 - qq, q2 = 2.0 - qq, q1 = 1.0 - qq;
      return ad_7h * (-5.0 * pw4(q3) + 30.0 * pw4(q2) - 75.0 * pw4(q1));
    } else if (isel == 1) {
      double q3 = 3.0 - qq, q2 = 2.0 - qq;
      return ad_7h * (-5.0 * pw4(q3) + 30.0 * pw4(q2));
    } else if (isel == 2) {
      double q3 = 3.0 - qq;
      return ad_7h * (-5.0 * pw4(q3));
    }
    return 0.0;
  }
  // Wab (sphtools.F90:46-76): quintic spline
  double Wab(double qq) const {
    int isel = (int)std::floor(qq);
    if (isel == 0) {
      double q3 = 3.0 - qq, q2 = 2.0 - qq, q1 = 1.0 - qq;
      return ad_7 * (pw5(q3) - 6.0 * pw5(q2) + 15.0 * pw5(q1));
    } else if (isel == 1) {
      double q3 = 3.0 - qq, q2 = 2.0 - qq;
      return ad_7 * (pw5(q3) - 6.0 * pw5(q2));
    } else if (isel == 2) {
      return ad_7 * pw5(3.0 - qq);
    }
    return 0.0;
  }

  // ------------------------------------------------------------------ setup
  int create(const vebi_params* prm) {
    P = *prm;
    nb = P.nb_patches;
    ncirc = P.nb_circles;
    npfb = P.npfb;
    nbS = P.nbS;
    nplink = P.nplink > 0 ? P.nplink : 75;
    if (P.itermax <= 0) P.itermax = 1000;
    if (P.tol <= 0) P.tol = 1.0e-8;
    if (npfb <= 0 || nbS < 0 || nbS > npfb || nb < 0 || nb > VEBI_MAX_PATCHES || ncirc < 0 ||
        ncirc > VEBI_MAX_CIRCLES)
      return VEBI_ERR_ARG;
    dx = P.dx;
    dv = P.dv;
    h = P.h;
    // input.F90:164-172
    h2 = h * h;
    sup_size = 3.0 * h;
    sup_size_2 = 9.0 * h2;
    uno_sup_size = 1.0 / (3.0 * h);
    ad_7 = 7.0 / 478.0 / PI / h / h;
    ad_7h = ad_7 / h;
    eta2 = h * h * 1.0e-10;
    // check_boundaries (input.F90:182-273): checks 1-3 and the corner angles
    {
      int n_fail = 0;
      for (int i = 0; i < nb; ++i) {
        int j = (i == nb - 1) ? 0 : i + 1;
        double t1 = P.b_node[i][0] + P.b_edge[i][0] - P.b_node[j][0];
        double t2 = P.b_node[i][1] + P.b_edge[i][1] - P.b_node[j][1];
        if (std::sqrt(t1 * t1 + t2 * t2) > 1.0e-10) ++n_fail;
      }
      double s1 = 0.0, s2 = 0.0;
      for (int i = 0; i < nb; ++i) { s1 += P.b_edge[i][0]; s2 += P.b_edge[i][1]; }
      if (nb > 0 && std::sqrt(s1 * s1 + s2 * s2) > 1.0e-10) ++n_fail;
      for (int i = 0; i < nb; ++i) {
        if (P.b_type[i] == 2) {
          int pp = P.b_periodic_parent[i] - 1;
          if (pp < 0 || pp >= nb) { ++n_fail; continue; }
          double t1 = P.b_edge[i][0] + P.b_edge[pp][0], t2 = P.b_edge[i][1] + P.b_edge[pp][1];
          if (std::fabs(std::sqrt(t1 * t1 + t2 * t2)) > 1.0e-10) ++n_fail;
        }
      }
      if (n_fail) return VEBI_ERR_BOUNDARY;
      for (int i = 0; i < nb; ++i) {
        int ibm1 = (i + nb - 1) % nb, ibp1 = (i + 1) % nb;
        double p_dist = P.b_edge[ibm1][1] * P.b_node[ibp1][0] - P.b_edge[ibm1][0] * P.b_node[ibp1][1] +
                        P.b_node[i][0] * P.b_node[ibm1][1] - P.b_node[i][1] * P.b_node[ibm1][0];
        p_dist = -1.0 * p_dist /
                 std::sqrt(P.b_edge[ibm1][0] * P.b_edge[ibm1][0] + P.b_edge[ibm1][1] * P.b_edge[ibm1][1]);
        double tmp1 = std::sqrt(P.b_edge[i][0] * P.b_edge[i][0] + P.b_edge[i][1] * P.b_edge[i][1]);
        if (p_dist <= 0.0 && std::fabs(p_dist) > std::fabs(tmp1)) p_dist = -tmp1;
        else if (p_dist > 0.0 && std::fabs(p_dist) > std::fabs(tmp1)) p_dist = tmp1;
        b_corner_angle[i] = std::asin(p_dist / tmp1);
      }
    }
    // padded box (sph2D_incom.F90:64-67)
    if (P.x_mint == 0.0 && P.x_maxt == 0.0 && P.y_mint == 0.0 && P.y_maxt == 0.0) {
      double xb_min = 1e300, xb_max = -1e300, yb_min = 1e300, yb_max = -1e300;
      for (int i = 0; i < nb; ++i) {
        xb_min = std::min(xb_min, P.b_node[i][0]); xb_max = std::max(xb_max, P.b_node[i][0]);
        yb_min = std::min(yb_min, P.b_node[i][1]); yb_max = std::max(yb_max, P.b_node[i][1]);
      }
      P.x_mint = xb_min - sup_size * 1.5; P.x_maxt = xb_max + sup_size * 1.5;
      P.y_mint = yb_min - sup_size * 1.5; P.y_maxt = yb_max + sup_size * 1.5;
    }
    x_mint = P.x_mint; x_maxt = P.x_maxt; y_mint = P.y_mint; y_maxt = P.y_maxt;
    // cell_generator (cell_griddin.F90:13-24)
    ncx = (int)((x_maxt - x_mint) * uno_sup_size) + 1;
    ncy = (int)((y_maxt - y_mint) * uno_sup_size) + 1;
    nct = ncx * ncy;
    // mirror capacity: create_mirror_particles' estimate (mirror_boundaries_mod.F90:53-54)
    mcap = P.nmirror_cap > 0 ? P.nmirror_cap : (npfb <= 500 ? 10 * npfb : 2 * npfb);
    cap = npfb + mcap;
    auto zd = [&](std::vector<double>& v) { v.assign(cap, 0.0); };
    auto zr = [&](std::vector<R>& v) { v.assign(cap, R(0.0)); };
    zd(rx); zd(ry); zr(ux); zr(uy); zr(theta); zr(p); for (auto& t : tau) zr(t);
    trace_conf.assign(cap, R(2.0));  // input.F90:111
    zr(a_out); zr(vort); zd(conc); zd(div_r); zd(dP_mp);
    n_surf.assign(cap, 0);
    inbin.assign(cap, 0);
    irelation.assign(cap, 0);
    vrelation.assign(cap, 0);
    return VEBI_OK;
  }

  int set_state(const double* r, const double* u, const double* tp, const double* th,
                const double* tc, const uint8_t* ib, int ld) {
    if (ld < npfb) return VEBI_ERR_ARG;
    for (int i = 0; i < npfb; ++i) {
      rx[i] = r[i]; ry[i] = r[ld + i];
      ux[i] = u[i]; uy[i] = u[ld + i];
      theta[i] = th ? th[i] : 0.0;
      for (int c = 0; c < 4; ++c) tau[c][i] = tp ? tp[(int64_t)c * ld + i] : 0.0;
      trace_conf[i] = tc ? tc[i] : 2.0;
      inbin[i] = ib ? (ib[i] ? 1 : 0) : 0;
      n_surf[i] = P.i_open_domain ? 1 : 0;  // input.F90:148-153
    }
    np = npfb;
    return VEBI_OK;
  }
  // tangent-linear model only: the direction of the fields' perturbation (any pointer may be null)
  int set_tangent(const double* du, const double* dtp, const double* dth, int ld) {
    if constexpr (std::is_same<R, Tan>::value) {
      if (ld < npfb) return VEBI_ERR_ARG;
      for (int i = 0; i < npfb; ++i) {
        ux[i].d = du ? du[i] : 0.0;
        uy[i].d = du ? du[ld + i] : 0.0;
        theta[i].d = dth ? dth[i] : 0.0;
        for (int c = 0; c < 4; ++c) tau[c][i].d = dtp ? dtp[(int64_t)c * ld + i] : 0.0;
      }
      return VEBI_OK;
    } else {
      (void)du; (void)dtp; (void)dth; (void)ld;
      return VEBI_ERR_ARG;
    }
  }

  // ------------------------------------------------------------------ set_time_step
  // div_free.F90:126-146
  void set_time_step() {
    umax = 1.0e-10;
    for (int i = nbS; i < npfb; ++i) {
      double u_abs = std::sqrt(val(ux[i]) * val(ux[i]) + val(uy[i]) * val(uy[i]));
      if (u_abs > umax) umax = u_abs;
    }
    double dt_CFL = P.dt_coef_cfl * h / umax;
    double dt_visc = P.dt_coef_visc * h * h * std::min(std::sqrt(P.Ra / P.Pr), std::sqrt(P.Ra * P.Pr));
    dt = std::min(dt_CFL, dt_visc);
  }

  // ------------------------------------------------------------------ put_in_bin
  // put_in_bin.F90:1-56
  int put_in_bin(double xmn, double xmx, double ymn, double ymx) {
    for (int i = nbS; i < npfb; ++i) {
      if (!inbin[i]) {
        if (rx[i] < xmn || rx[i] > xmx || ry[i] < ymn || ry[i] > ymx) inbin[i] = 1;
        if (std::isnan(rx[i]) || std::isnan(ry[i])) inbin[i] = 1;
      }
    }
    n_inbin = 0;
    for (int i = nbS; i < npfb; ++i) {
      if (inbin[i]) {
        rx[i] = 2.0 * xmn - xmx;
        ry[i] = 2.0 * ymn - ymx;
        ux[i] = 0.0; uy[i] = 0.0;
        ++n_inbin;
      }
    }
    if (n_inbin == npfb - nbS) return VEBI_ERR_ALL_IN_BIN;
    return VEBI_OK;
  }

  // ------------------------------------------------------------------ mirrors
  // replace_escapees (mirror_boundaries_mod.F90:336-407)
  void replace_escapees() {
    n_escapees = 0;
    for (int ib = 0; ib < ncirc; ++ib) {
      for (int i = nbS; i < npfb; ++i) {
        double ric1 = rx[i] - P.c_centre[ib][0], ric2 = ry[i] - P.c_centre[ib][1];
        double rad = std::sqrt(ric1 * ric1 + ric2 * ric2);
        if (rad < std::fabs(P.c_radius[ib]) && P.c_radius[ib] > 0.0) {
          rx[i] = rx[i] + (ric1 / rad) * 2.0 * (P.c_radius[ib] - rad);
          ry[i] = ry[i] + (ric2 / rad) * 2.0 * (P.c_radius[ib] - rad);
          ++n_escapees;
        }
        if (rad > std::fabs(P.c_radius[ib]) && P.c_radius[ib] < 0.0) {
          rx[i] = rx[i] - (ric1 / rad) * 2.0 * (rad + P.c_radius[ib]);
          ry[i] = ry[i] - (ric2 / rad) * 2.0 * (rad + P.c_radius[ib]);
          ++n_escapees;
        }
      }
    }
    for (int ib = 0; ib < nb; ++ib) {
      if (P.b_type[ib] == 0) continue;
      if (P.b_type[ib] == 1 || P.b_type[ib] == 2) {
        double n1, n2;
        bound_norm(ib, n1, n2);
        int ibp = P.b_periodic_parent[ib] - 1;
        for (int i = nbS; i < npfb; ++i) {
          if (inbin[i]) continue;
          double perp = bound_dist(i, ib);
          if (perp > 0.0) continue;
          if (std::fabs(perp) > sup_size + 1.0e-10) continue;
          double tmp = position_along_patch_xy(rx[i], ry[i], ib, perp, n1, n2);
          if (P.b_type[ib] == 1) {
            if (tmp < 0.0 || tmp > 1.0) continue;
            rx[i] = rx[i] - 2.0 * perp * n1;
            ry[i] = ry[i] - 2.0 * perp * n2;
            ++n_escapees;
          } else {
            double pn1, pn2;
            bound_norm(ibp, pn1, pn2);
            double t1 = -1.0 * tmp * P.b_edge[ibp][0] - perp * pn1;
            double t2 = -1.0 * tmp * P.b_edge[ibp][1] - perp * pn2;
            rx[i] = P.b_node[ibp][0] + P.b_edge[ibp][0] + t1;
            ry[i] = P.b_node[ibp][1] + P.b_edge[ibp][1] + t2;
            ++n_escapees;
          }
          r0x[i] = rx[i] - val(ux[i]) * dt;
          r0y[i] = ry[i] - val(uy[i]) * dt;
          u0x[i] = ux[i];
          u0y[i] = uy[i];
        }
      }
    }
  }

  int push_mirror(int parent, int vrel) {
    if (nmirror >= mcap) { error = VEBI_ERR_MIRROR_CAPACITY; return -1; }
    int k = npfb + nmirror;
    ++nmirror;
    irelation[k] = parent;
    vrelation[k] = vrel;
    return k;
  }

  // create_mirror_particles (mirror_boundaries_mod.F90:18-334)
  int create_mirror_particles() {
    replace_escapees();
    // create_boundary_boxes (:409-445)
    std::vector<std::vector<int>> b_nb(nb), bc_nb(nb);
    std::vector<std::vector<double>> b_pos1(nb), b_pos2(nb);
    for (int ib = 0; ib < nb; ++ib) {
      if (P.b_type[ib] == 0) continue;
      double n1, n2;
      bound_norm(ib, n1, n2);
      for (int i = 0; i < npfb; ++i) {
        double perp = bound_dist(i, ib);
        if (std::fabs(perp) > sup_size + 1.0e-10) continue;
        double tmp = position_along_patch_xy(rx[i], ry[i], ib, perp, n1, n2);
        if (tmp < 0.0 || tmp > 1.0) continue;
        b_nb[ib].push_back(i);
        b_pos1[ib].push_back(tmp);
        b_pos2[ib].push_back(perp);
      }
      for (int i = nbS; i < npfb; ++i) {
        double d = std::sqrt(pw2(rx[i] - P.b_node[ib][0]) + pw2(ry[i] - P.b_node[ib][1]));
        if (d > sup_size + 1.0e-10) continue;
        bc_nb[ib].push_back(i);
      }
    }
    nmirror = 0;
    const double* bf = P.body_force;
    auto dP = [&](int k, int i) { return bf[0] * (rx[k] - rx[i]) + bf[1] * (ry[k] - ry[i]); };
    // STEP 5a: circles (:61-96)
    if (ncirc != 0) {
      for (int i = nbS; i < npfb; ++i) {
        for (int ib = 0; ib < ncirc; ++ib) {
          double Rc = P.c_radius[ib];
          double c_dir = Rc / std::fabs(Rc);
          double ric1 = rx[i] - P.c_centre[ib][0], ric2 = ry[i] - P.c_centre[ib][1];
          double rad = std::sqrt(ric1 * ric1 + ric2 * ric2);
          if (c_dir > 0.0) {
            if (rad <= Rc + sup_size) {
              ric1 = ric1 / rad; ric2 = ric2 / rad;
              int k = push_mirror(i, 999 + ib + 1);
              if (k < 0) return error;
              rx[k] = rx[i] - ric1 * 2.0 * (rad - Rc);
              ry[k] = ry[i] - ric2 * 2.0 * (rad - Rc);
              double t1 = ric2, t2 = -ric1;
              ux[k] = 2.0 * P.c_vel[ib][0] + 2.0 * t1 * Rc * P.c_omega[ib] - 1.0 * ux[i];
              uy[k] = 2.0 * P.c_vel[ib][1] + 2.0 * t2 * Rc * P.c_omega[ib] - 1.0 * uy[i];
              theta[k] = 2.0 * P.c_thermal[ib] - 1.0 * theta[i];
              dP_mp[k] = dP(k, i);
            }
          } else if (c_dir < 0.0) {
            if (rad >= std::fabs(Rc) - sup_size) {
              ric1 = ric1 / rad; ric2 = ric2 / rad;
              int k = push_mirror(i, 999 + ib + 1);
              if (k < 0) return error;
              rx[k] = rx[i] + ric1 * 2.0 * (std::fabs(Rc) - rad);
              ry[k] = ry[i] + ric2 * 2.0 * (std::fabs(Rc) - rad);
              double t1 = ric2, t2 = -ric1;
              ux[k] = 2.0 * P.c_vel[ib][0] + 2.0 * t1 * std::fabs(Rc) * P.c_omega[ib] - 1.0 * ux[i];
              uy[k] = 2.0 * P.c_vel[ib][1] + 2.0 * t2 * std::fabs(Rc) * P.c_omega[ib] - 1.0 * uy[i];
              theta[k] = 2.0 * P.c_thermal[ib] - 1.0 * theta[i];
              dP_mp[k] = dP(k, i);
            }
          }
        }
      }
    }
    // STEP 5: patches (:99-188)
    for (int ib = 0; ib < nb; ++ib) {
      int ibp1 = (ib + 1) % nb;
      if (P.b_type[ib] == 0) continue;
      if (P.b_type[ib] == 1) {
        double n1, n2;
        bound_norm(ib, n1, n2);
        for (size_t j = 0; j < b_nb[ib].size(); ++j) {
          int i = b_nb[ib][j];
          double bp1 = b_pos1[ib][j], bp2 = b_pos2[ib][j];
          if (bp2 <= 1.0e-10) continue;
          if (b_corner_angle[ib] < 0.0) {
            double ta = 0.5 * (PI + b_corner_angle[ib]);
            double m_be = std::sqrt(P.b_edge[ib][0] * P.b_edge[ib][0] + P.b_edge[ib][1] * P.b_edge[ib][1]);
            if (bp2 + 0.1 * dx >= bp1 * std::tan(ta) * m_be) continue;
          }
          if (b_corner_angle[ibp1] < 0.0) {
            double ta = 0.5 * (PI + b_corner_angle[ibp1]);
            double m_be = std::sqrt(P.b_edge[ib][0] * P.b_edge[ib][0] + P.b_edge[ib][1] * P.b_edge[ib][1]);
            if (bp2 >= (1.0 - bp1) * std::tan(ta) * m_be) continue;
          }
          int k = push_mirror(i, ib + 1);
          if (k < 0) return error;
          rx[k] = rx[i] - 2.0 * bp2 * n1;
          ry[k] = ry[i] - 2.0 * bp2 * n2;
          double t1 = n2, t2 = -n1;
          ux[k] = 2.0 * P.b_vel[ib] * t1 - ux[i];
          uy[k] = 2.0 * P.b_vel[ib] * t2 - uy[i];
          theta[k] = 2.0 * P.b_thermal[ib] - theta[i];
          dP_mp[k] = dP(k, i);
        }
      }
      if (P.b_type[ib] == 2) {
        int ibp = P.b_periodic_parent[ib] - 1;
        double n1, n2;
        bound_norm(ib, n1, n2);
        for (size_t j = 0; j < b_nb[ibp].size(); ++j) {
          int i = b_nb[ibp][j];
          double bp1 = b_pos1[ibp][j], bp2 = b_pos2[ibp][j];
          if (bp2 <= 0.0) continue;
          int k = push_mirror(i, ib + 1);
          if (k < 0) return error;
          double t1 = -1.0 * bp1 * P.b_edge[ib][0] - bp2 * n1;
          double t2 = -1.0 * bp1 * P.b_edge[ib][1] - bp2 * n2;
          rx[k] = P.b_node[ib][0] + P.b_edge[ib][0] + t1;
          ry[k] = P.b_node[ib][1] + P.b_edge[ib][1] + t2;
          ux[k] = ux[i]; uy[k] = uy[i];
          theta[k] = theta[i];
          dP_mp[k] = 0.0;
        }
      }
    }
    // mirrors of moving solid particles copy their parent's velocity/temperature (:191-206)
    for (int j = npfb; j < npfb + nmirror; ++j) {
      int i = irelation[j];
      double tmp = val(ux[i] * ux[i] + uy[i] * uy[i]);
      if (i < nbS && tmp != 0.0) { ux[j] = ux[i]; uy[j] = uy[i]; }
    }
    for (int j = npfb; j < npfb + nmirror; ++j) {
      int i = irelation[j];
      double tmp = val(theta[i] * theta[i]);
      if (i < nbS && tmp != 0.0) theta[j] = theta[i];
    }
    // STEP 6: corners (:209-324)
    for (int ib = 0; ib < nb; ++ib) {
      int ibm1 = (ib + nb - 1) % nb;
      if (P.b_type[ib] == 0 || P.b_type[ibm1] == 0) continue;
      double tmp = P.b_edge[ibm1][0] * P.b_edge[ib][1] - P.b_edge[ibm1][1] * P.b_edge[ib][0];
      if (std::fabs(tmp) < 1e-10) continue;
      if (P.b_type[ib] == 1 && P.b_type[ibm1] == 1) {
        if (b_corner_angle[ib] <= 0.0) continue;
        for (int i : bc_nb[ib]) {
          double tb1 = rx[i] - P.b_node[ib][0], tb2 = ry[i] - P.b_node[ib][1];
          int k = push_mirror(i, -(ib + 1));
          if (k < 0) return error;
          rx[k] = rx[i] - 2.0 * tb1;
          ry[k] = ry[i] - 2.0 * tb2;
          double n1, n2;
          bound_norm(ib, n1, n2);
          // `tmp` still holds the edge cross product (mirror_boundaries_mod.F90:216,242)
          ux[k] = 2.0 * tmp * n2 - ux[i];
          uy[k] = 2.0 * tmp * (-n1) - uy[i];
          bound_norm(ibm1, n1, n2);
          ux[k] = ux[k] + 2.0 * tmp * n2;
          uy[k] = uy[k] + 2.0 * tmp * (-n1);
          theta[k] = theta[i] + 2.0 * P.b_thermal[ib];
          dP_mp[k] = dP(k, i);
        }
      }
      if (P.b_type[ib] == 2 && P.b_type[ibm1] == 2) {
        int ibp = P.b_periodic_parent[ib] - 1;
        for (int i : bc_nb[ibp]) {
          int k = push_mirror(i, -(ib + 1));
          if (k < 0) return error;
          double tb1 = P.b_node[ib][0] - P.b_node[ibp][0], tb2 = P.b_node[ib][1] - P.b_node[ibp][1];
          rx[k] = rx[i] + tb1;
          ry[k] = ry[i] + tb2;
          ux[k] = ux[i]; uy[k] = uy[i];
          theta[k] = theta[i];
          dP_mp[k] = 0.0;
        }
      }
      if (P.b_type[ib] != P.b_type[ibm1]) {
        if (P.b_type[ib] == 1 || P.b_type[ibm1] == 1) {
          int ibb = (P.b_type[ibm1] == 1) ? ibm1 : ib;
          int imp_temp = nmirror;
          for (int j = npfb; j < npfb + imp_temp; ++j) {
            double perp = bound_dist(j, ibb);
            if (perp > sup_size + 1.0e-10) continue;
            if (perp < 1.0e-10) continue;
            double n1, n2;
            bound_norm(ibb, n1, n2);
            double t = position_along_patch_xy(rx[j], ry[j], ibb, perp, n1, n2);
            if ((t < 0.0 && ibb == ib) || (t > 1.0 && ibb == ibm1)) {
              int i = irelation[j];
              int k = push_mirror(i, -(ib + 1));
              if (k < 0) return error;
              rx[k] = rx[j] - 2.0 * perp * n1;
              ry[k] = ry[j] - 2.0 * perp * n2;
              double t1 = n2, t2 = -n1;
              ux[k] = 2.0 * P.b_vel[ibb] * t1 - ux[j];
              uy[k] = 2.0 * P.b_vel[ibb] * t2 - uy[j];
              theta[k] = 2.0 * P.b_thermal[ibb] - theta[j];
              dP_mp[k] = dP_mp[j];
              dP_mp[k] = dP_mp[k] + (bf[0] * (rx[k] - rx[j]) + bf[1] * (ry[k] - ry[j]));
            }
          }
        }
      }
    }
    np = npfb + nmirror;
    for (int j = npfb; j < np; ++j) inbin[j] = 0;
    return VEBI_OK;
  }

  // mirror_velocities (mirror_boundaries_mod.F90:509-584)
  void mirror_velocities() {
    for (int j = npfb; j < np; ++j) {
      int i = irelation[j];
      int vr = vrelation[j];
      if (vr > 999) {
        int ib = vr - 999 - 1;
        ux[j] = -ux[i]; uy[j] = -uy[i];
        double r1 = 0.5 * (rx[i] - rx[j]), r2 = 0.5 * (ry[i] - ry[j]);
        double tmp = std::sqrt(r1 * r1 + r2 * r2);
        double t1 = r2 / tmp, t2 = -r1 / tmp;
        ux[j] = 2.0 * P.c_vel[ib][0] + 2.0 * t1 * P.c_radius[ib] * P.c_omega[ib] - 1.0 * ux[i];
        uy[j] = 2.0 * P.c_vel[ib][1] + 2.0 * t2 * P.c_radius[ib] * P.c_omega[ib] - 1.0 * uy[i];
      }
      if (vr > 0 && vr < 999) {
        int ib = vr - 1;
        if (std::abs(P.b_type[ib]) == 1) {
          double r1 = 0.5 * (rx[i] - rx[j]), r2 = 0.5 * (ry[i] - ry[j]);
          double tmp = std::sqrt(r1 * r1 + r2 * r2);
          double t1 = r2 / tmp, t2 = -r1 / tmp;
          ux[j] = 2.0 * P.b_vel[ib] * t1 - ux[i];
          uy[j] = 2.0 * P.b_vel[ib] * t2 - uy[i];
        } else if (P.b_type[ib] == 2) {
          ux[j] = ux[i]; uy[j] = uy[i];
        }
      }
      if (vr < 0 && vr > -npfb) {
        int ib = -vr - 1;
        int ibm1 = (ib + nb - 1) % nb;
        if (P.b_type[ib] == 1 && P.b_type[ibm1] == 1) {
          ux[j] = ux[i]; uy[j] = uy[i];
          if (P.b_vel[ib] != 0.0) {
            double n1, n2; bound_norm(ib, n1, n2);
            double tmp = P.b_vel[ib];
            ux[j] = 2.0 * tmp * n2 - ux[i];
            uy[j] = 2.0 * tmp * (-n1) - uy[i];
          }
          if (P.b_vel[ibm1] != 0.0) {
            double n1, n2; bound_norm(ibm1, n1, n2);
            double tmp = P.b_vel[ibm1];
            ux[j] = ux[j] + 2.0 * tmp * n2;
            uy[j] = uy[j] + 2.0 * tmp * (-n1);
          }
        } else if (P.b_type[ib] == 2 && P.b_type[ibm1] == 2) {
          ux[j] = ux[i]; uy[j] = uy[i];
        } else if ((P.b_type[ib] == 1 && P.b_type[ibm1] == 2) ||
                   (P.b_type[ib] == 2 && P.b_type[ibm1] == 1)) {
          double tmp, t1, t2;
          if (P.b_vel[ib] != 0.0) {
            double n1, n2; bound_norm(ib, n1, n2); t1 = n2; t2 = -n1; tmp = P.b_vel[ib];
          } else if (P.b_vel[ibm1] != 0.0) {
            double n1, n2; bound_norm(ibm1, n1, n2); t1 = n2; t2 = -n1; tmp = P.b_vel[ibm1];
          } else {
            tmp = 0.0; t1 = 0.0; t2 = 0.0;
          }
          ux[j] = 2.0 * tmp * t1 - ux[i];
          uy[j] = 2.0 * tmp * t2 - uy[i];
        }
      }
    }
    for (int j = npfb; j < np; ++j) {
      int i = irelation[j];
      double tmp = val(ux[i] * ux[i] + uy[i] * uy[i]);
      if (i < nbS && tmp != 0.0) { ux[j] = ux[i]; uy[j] = uy[i]; }
    }
  }

  // mirror_polymeric_stress (mirror_boundaries_mod.F90:586-653)
  void mirror_polymeric_stress() {
    auto reflect = [&](int i, int j, double n1, double n2) {
      double nt1 = -n2, nt2 = n1;
      M2 Q{1.0 * n1 + 0.0 * n2, 1.0 * nt1 + 0.0 * nt2, 0.0 * n1 + 1.0 * n2, 0.0 * nt1 + 1.0 * nt2};
      M2 QT = tr(Q);
      M2T<R> T{tau[0][i], tau[2][i], tau[1][i], tau[3][i]};
      M2T<R> t = mm(QT, mm(T, Q));
      t.a11 = -t.a11; t.a12 = -t.a12;
      M2T<R> o = mm(Q, mm(t, QT));
      tau[0][j] = o.a11; tau[1][j] = o.a21; tau[2][j] = o.a12; tau[3][j] = o.a22;
    };
#pragma omp parallel for schedule(static)
    for (int j = npfb; j < np; ++j) {
      int i = irelation[j];
      int vr = vrelation[j];
      if (vr > 999) {
        double r1 = rx[i] - rx[j], r2 = ry[i] - ry[j];
        double nn = std::sqrt(r1 * r1 + r2 * r2);
        reflect(i, j, r1 / nn, r2 / nn);
      }
      if (vr > 0 && vr < 999) {
        int ib = vr - 1;
        if (P.b_type[ib] == 1) {
          double r1 = rx[i] - rx[j], r2 = ry[i] - ry[j];
          double nn = std::sqrt(r1 * r1 + r2 * r2);
          reflect(i, j, r1 / nn, r2 / nn);
        } else if (P.b_type[ib] == 2 || P.b_type[ib] == 4) {
          for (int c = 0; c < 4; ++c) tau[c][j] = tau[c][i];
        } else if (P.b_type[ib] == 3) {
          for (int c = 0; c < 4; ++c) tau[c][j] = R(0.0);
        }
      }
      if (vr < 0 && vr > -npfb) {
        int ib = -vr - 1;
        int ibm1 = (ib + nb - 1) % nb;
        if (P.b_type[ib] == 1 && P.b_type[ibm1] == 1) {
          for (int c = 0; c < 4; ++c) tau[c][j] = -tau[c][i];
        } else if (P.b_type[ib] == 2 && P.b_type[ibm1] == 2) {
          for (int c = 0; c < 4; ++c) tau[c][j] = tau[c][i];
        } else if ((P.b_type[ib] == 1 && P.b_type[ibm1] == 2) ||
                   (P.b_type[ib] == 2 && P.b_type[ibm1] == 1)) {
          double n1, n2;
          if (P.b_type[ib] == 1) bound_norm(ib, n1, n2);
          else bound_norm(ibm1, n1, n2);
          reflect(i, j, n1, n2);
        }
      }
    }
  }

  // ------------------------------------------------------------------ neighbours
  // divide (neighbour_finding_mod.F90:56-127): serial counting sort into cells
  int divide() {
    ncell.assign(nct + 1, 0);
    cellpart.assign(np, -1);
    int nc_max = 0;
    for (int k = 0; k < np; ++k) {
      if (inbin[k]) continue;
      double ddx = rx[k] - x_mint, ddy = ry[k] - y_mint;
      int icell = (int)(ddx * uno_sup_size) + 1;
      int jcell = (int)(ddy * uno_sup_size) + 1;
      int ii = icell + (jcell - 1) * ncx;  // 1-based cell
      if (ii > nct || ii < 1) return VEBI_ERR_OUT_OF_DOMAIN;
      ncell[ii - 1] += 1;
      nc_max = std::max(nc_max, ncell[ii - 1]);
      if (nc_max > nplink) return VEBI_ERR_CELL_CAPACITY;
      cellpart[k] = ii - 1;
    }
    ist.assign(nct + 1, 0);
    for (int c = 0; c < nct; ++c) { ist[c + 1] = ist[c] + ncell[c]; ncell[c] = 0; }
    ipl.assign(std::max(ist[nct], 1), 0);
    for (int k = 0; k < np; ++k) {
      if (inbin[k]) continue;
      int c = cellpart[k];
      ipl[ist[c] + ncell[c]] = k;
      ncell[c] += 1;
    }
    return VEBI_OK;
  }

  // neighboring_list_parallel + neighbour_particle_cell (neighbour_finding_mod.F90:261-365)
  int neighbour_list() {
    ij_count.assign(npfb, 0);
    ij_link.assign((size_t)nplink * npfb, 0);
    int overflow = 0;
#pragma omp parallel for schedule(static) reduction(| : overflow)
    for (int i = 0; i < npfb; ++i) {
      if (inbin[i]) continue;
      int ic = cellpart[i] + 1;  // 1-based as the reference
      int icx = ic % ncx;        // the reference's column formula (last column -> 0)
      int icy = ic / ncx + 1;
      auto scan = [&](int jc) {  // jc 1-based
        if (jc < 1 || jc > nct) return;  // the reference's nc(jc)==0 for these
        int c = jc - 1;
        if (ncell[c] == 0) return;
        for (int jj = ist[c]; jj < ist[c + 1]; ++jj) {
          int j = ipl[jj];
          double r1 = rx[i] - rx[j], r2 = ry[i] - ry[j];
          double rr2 = r1 * r1 + r2 * r2;
          if (rr2 > 0.0 && rr2 <= sup_size_2) {
            int k = ij_count[i];
            if (k >= nplink) { overflow = 1; continue; }
            ij_link[(size_t)k * npfb + i] = j;
            ij_count[i] = k + 1;
          }
        }
      };
      scan(ic);
      if (icx + 1 <= ncx) {
        scan(ic + 1);
        if (icy + 1 <= ncy) scan(ic + ncx + 1);
        if (icy - 1 >= 1) scan(ic - ncx + 1);
      }
      if (icx - 1 >= 1) {
        scan(ic - 1);
        if (icy + 1 <= ncy) scan(ic + ncx - 1);
        if (icy - 1 >= 1) scan(ic - ncx - 1);
      }
      if (icy + 1 <= ncy) scan(ic + ncx);
      if (icy - 1 >= 1) scan(ic - ncx);
    }
    if (overflow) return VEBI_ERR_NEIGH_CAPACITY;
    maxneighbours = 0;
    for (int i = 0; i < npfb; ++i) maxneighbours = std::max(maxneighbours, ij_count[i]);
    return VEBI_OK;
  }

  inline int L(int k, int i) const { return ij_link[(size_t)k * npfb + i]; }
  inline size_t E(int k, int i) const { return (size_t)k * npfb + i; }

  // ------------------------------------------------------------------ kernel_calculation
  // kernel_calculation.F90:2-75 (KGC=1)
  void kernel_calculation() {
    size_t n = (size_t)std::max(maxneighbours, 1) * npfb;
    wGx.assign(n, 0.0); wGy.assign(n, 0.0); wL.assign(n, 0.0);
    for (auto& k : kgcm) k.assign(npfb, 0.0);
    const double eta_small = (double)0.01f * h * h;  // default-real literal 0.01
    const double oneoverh = 1.0 / h;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npfb; ++i) {
      double k11 = 0, k12 = 0, k21 = 0, k22 = 0;
      for (int k = 0; k < ij_count[i]; ++k) {
        int j = L(k, i);
        double r1 = rx[i] - rx[j], r2 = ry[i] - ry[j];
        double rr2 = r1 * r1 + r2 * r2;
        double rad = std::sqrt(rr2);
        double qq = rad * oneoverh;
        double f = fac(qq);
        double m = std::max(rad, eta2);
        double g1 = r1 * f / m, g2 = r2 * f / m;
        double w1 = g1 * dv, w2 = g2 * dv;
        wGx[E(k, i)] = w1; wGy[E(k, i)] = w2;
        wL[E(k, i)] = 2.0 * (r1 * w1 + r2 * w2) / (rr2 + eta_small);
        k11 = k11 - dv * g1 * r1;
        k12 = k12 - dv * g2 * r1;
        k21 = k21 - dv * g1 * r2;
        k22 = k22 - dv * g2 * r2;
      }
      double temp = 1.0 / ((k11 * k22 - k12 * k21) + 1.0e-15);
      double temp2 = k11;
      kgcm[0][i] = temp * k22;        // (1,1)
      kgcm[2][i] = -temp * k12;       // (1,2)
      kgcm[1][i] = -temp * k21;       // (2,1)
      kgcm[3][i] = temp * temp2;      // (2,2)
    }
  }
  inline M2 K(int i) const { return M2{kgcm[0][i], kgcm[2][i], kgcm[1][i], kgcm[3][i]}; }

  // ------------------------------------------------------------------ free surface
  // locate_free_surf_part, calc_part_dist_vars, smooth_normals (freesurf_mod.F90:17-137)
  void locate_free_surf_part() {
    std::vector<double> beta_div_r;
    if (P.i_open_domain == 1) {
      surf_nx.assign(npfb, 0.0); surf_ny.assign(npfb, 0.0);
      beta_div_r.assign(npfb, 0.0);
#pragma omp parallel for schedule(static)
      for (int i = 0; i < npfb; ++i) {
        double ct = 0, dr = 0, s1 = 0, s2 = 0;
        for (int k = 0; k < ij_count[i]; ++k) {
          int j = L(k, i);
          double r1 = rx[i] - rx[j], r2 = ry[i] - ry[j];
          double rad = std::sqrt(r1 * r1 + r2 * r2);
          double qq = rad / h;
          ct = ct + Wab(qq);
          dr = dr - (r1 * wGx[E(k, i)] + r2 * wGy[E(k, i)]);
          s1 = s1 - wGx[E(k, i)];
          s2 = s2 - wGy[E(k, i)];
        }
        conc[i] = ct * dv; div_r[i] = dr; surf_nx[i] = s1; surf_ny[i] = s2;
      }
      double w0 = Wab(0.0);
      for (int i = 0; i < npfb; ++i) {
        conc[i] = conc[i] + dv * w0;
        surf_nx[i] = surf_nx[i] * h; surf_ny[i] = surf_ny[i] * h;
      }
      for (int i = 0; i < npfb; ++i) {
        beta_div_r[i] = 1.4 + 0.5 * std::max(conc[i] - 1.0, -0.2);
        n_surf[i] = (div_r[i] > beta_div_r[i]) ? 0 : 1;
      }
    } else {
      for (int i = 0; i < cap; ++i) n_surf[i] = 0;
    }
    for (int i = npfb; i < np; ++i) n_surf[i] = n_surf[irelation[i]];
    if (P.i_open_domain == 1) {
      std::vector<double> t1(npfb), t2(npfb);
      double w0 = Wab(0.0);
#pragma omp parallel for schedule(static)
      for (int i = 0; i < npfb; ++i) {
        double a = 0, b = 0;
        for (int k = 0; k < ij_count[i]; ++k) {
          int j = L(k, i);
          if (j >= npfb) continue;
          double r1 = rx[i] - rx[j], r2 = ry[i] - ry[j];
          double rad = std::sqrt(r1 * r1 + r2 * r2);
          double w = Wab(rad / h);
          a = a + w * surf_nx[j];
          b = b + w * surf_ny[j];
        }
        t1[i] = a * dv + surf_nx[i] * w0 * dv;
        t2[i] = b * dv + surf_ny[i] * w0 * dv;
      }
      surf_nx = t1; surf_ny = t2;
      ppe_smooth.assign(npfb, 1.0);
      for (int i = 0; i < npfb; ++i) {
        if (div_r[i] > 1.2 * beta_div_r[i]) continue;
        if (n_surf[i] == 1) ppe_smooth[i] = 0.0;
        else ppe_smooth[i] = 0.5 * (1.0 - std::cos((div_r[i] - beta_div_r[i]) * PI / (0.2 * beta_div_r[i])));
      }
    }
  }

  // ------------------------------------------------------------------ shifting
  // new_fick_shift + shifting_forces (new_fick_shift.F90:15-92,117-210), Akinci off
  void new_fick_shift() {
    gradCx.assign(npfb, 0.0); gradCy.assign(npfb, 0.0);
    const double nt = 4.0, Rt = 0.25;
    const double Wab1 = Wab(dx / h);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npfb; ++i) {
      double f1 = 0, f2 = 0, t1 = 0, t2 = 0;
      for (int k = 0; k < ij_count[i]; ++k) {
        int j = L(k, i);
        double r1 = rx[i] - rx[j], r2 = ry[i] - ry[j];
        double rad = std::sqrt(r1 * r1 + r2 * r2);
        double qq = rad / h;
        double fab = Rt * std::pow(Wab(qq) / Wab1, nt);
        f1 = f1 + wGx[E(k, i)];
        f2 = f2 + wGy[E(k, i)];
        t1 = t1 + wGx[E(k, i)] * fab;
        t2 = t2 + wGy[E(k, i)] * fab;
      }
      gradCx[i] = f1 + t1;
      gradCy[i] = f2 + t2;
    }
    drx.assign(npfb, 0.0); dry.assign(npfb, 0.0);
    double maxU = 1.0e-10;
    for (int i = 0; i < npfb; ++i)
      maxU = std::max(maxU, std::sqrt(val(ux[i]) * val(ux[i]) + val(uy[i]) * val(uy[i])));
#pragma omp parallel for schedule(static)
    for (int i = nbS; i < npfb; ++i) {
      double D;
      if (P.i_shift_coeff == 1) {
        double absU = std::sqrt(val(ux[i]) * val(ux[i]) + val(uy[i]) * val(uy[i]));
        double temp = (double)0.2f * std::exp(-absU / ((double)0.2f * maxU));
        D = 4.0 * h * dt * (absU + temp * maxU);
      } else {
        D = 0.25 * h * h;
      }
      double d1, d2;
      if (n_surf[i] == 1 && P.i_open_domain == 1) {
        double temp = std::sqrt(surf_nx[i] * surf_nx[i] + surf_ny[i] * surf_ny[i]);
        double sn1 = surf_nx[i] / std::max(temp, (double)1e-8f);
        double sn2 = surf_ny[i] / std::max(temp, (double)1e-8f);
        double st1 = -sn2, st2 = sn1;
        double dCds = st1 * gradCx[i] + st2 * gradCy[i];
        d1 = -D * dCds * st1;
        d2 = -D * dCds * st2;
      } else {
        d1 = -D * gradCx[i];
        d2 = -D * gradCy[i];
      }
      double temp = std::sqrt(d1 * d1 + d2 * d2);
      if (temp > 0.1 * h) {
        d1 = 0.1 * h * d1 / temp;
        d2 = 0.1 * h * d2 / temp;
      }
      drx[i] = d1; dry[i] = d2;
    }
  }

  // ------------------------------------------------------------------ gradients
  // grad_operator (gradient_calculation.F90:50-147) for u, v, theta in one pass
  void grad_operators() {
    for (auto& g : grad) g.assign(np, R(0.0));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npfb; ++i) {
      R a[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      for (int k = 0; k < ij_count[i]; ++k) {
        int j = L(k, i);
        double w1 = wGx[E(k, i)], w2 = wGy[E(k, i)];
        R du = ux[j] - ux[i], dvv = uy[j] - uy[i], dth = theta[j] - theta[i];
        a[0] = a[0] + du * w1; a[1] = a[1] + du * w2;
        a[2] = a[2] + dvv * w1; a[3] = a[3] + dvv * w2;
        a[4] = a[4] + dth * w1; a[5] = a[5] + dth * w2;
      }
      M2 Kc = K(i);
      for (int f = 0; f < 3; ++f) {
        grad[2 * f][i] = Kc.a11 * a[2 * f] + Kc.a12 * a[2 * f + 1];
        grad[2 * f + 1][i] = Kc.a21 * a[2 * f] + Kc.a22 * a[2 * f + 1];
      }
    }
    // mirror transfer (gradient_calculation.F90:96-145)
#pragma omp parallel for schedule(static)
    for (int j = npfb; j < np; ++j) {
      int i = irelation[j];
      int vr = vrelation[j];
      for (int f = 0; f < 3; ++f) {
        R g1 = grad[2 * f][i], g2 = grad[2 * f + 1][i];
        R o1 = 0.0, o2 = 0.0;
        bool set = false;
        auto reflect = [&](double r1, double r2, bool normal_zero) {
          double nn = std::sqrt(r1 * r1 + r2 * r2);
          double q11 = r1 / nn, q21 = r2 / nn, q12 = -q21, q22 = q11;
          R b1 = q11 * g1 + q12 * g2, b2 = q21 * g1 + q22 * g2;
          if (normal_zero) b1 = 0.0; else b2 = -b2;
          o1 = q11 * b1 + q21 * b2;
          o2 = q12 * b1 + q22 * b2;
          set = true;
        };
        if (vr == 999) reflect(rx[i] - rx[j], ry[i] - ry[j], false);  // never true (circles are 999+ib)
        if (vr > 0 && vr < 999) {
          int ib = vr - 1;
          if (P.b_type[ib] == 2) {
            int ibp = P.b_periodic_parent[ib] - 1;
            M2 Q = angle_between_patches(ib, ibp);
            o1 = Q.a11 * g1 + Q.a12 * g2; o2 = Q.a21 * g1 + Q.a22 * g2; set = true;
          } else if (P.b_type[ib] == 3) {
            o1 = g1; o2 = g2; set = true;
          } else if (P.b_type[ib] == 1) {
            reflect(rx[i] - rx[j], ry[i] - ry[j], false);
          } else if (P.b_type[ib] == 4) {
            reflect(rx[i] - rx[j], ry[i] - ry[j], true);
          }
        } else if (vr < 0 && vr > -npfb) {
          int ib = -vr - 1;
          int ibm1 = (ib + nb - 1) % nb;
          if (P.b_type[ib] == 1 && P.b_type[ibm1] == 1) { o1 = -g1; o2 = -g2; set = true; }
          else if (P.b_type[ib] == 2 && P.b_type[ibm1] == 2) { o1 = g1; o2 = g2; set = true; }
          else if ((P.b_type[ib] == 1 && P.b_type[ibm1] == 2) || (P.b_type[ib] == 2 && P.b_type[ibm1] == 1)) {
            double r1 = 0, r2 = 0;
            if (P.b_type[ib] == 1) { r1 = -1.0 * P.b_edge[ib][1]; r2 = P.b_edge[ib][0]; }
            else if (P.b_type[ibm1] == 1) { r1 = -1.0 * P.b_edge[ibm1][1]; r2 = P.b_edge[ibm1][0]; }
            reflect(r1, r2, false);
          }
        }
        if (set) { grad[2 * f][j] = o1; grad[2 * f + 1][j] = o2; }
      }
    }
  }

  // ------------------------------------------------------------------ log-conformation
  // calc_eigens (predictor_mod.F90:253-290), over the field type
  template <class T>
  static void calc_eigens(const M2T<T>& A, T& L1, T& L2, M2T<T>& Q) {
    T trc = A.a11 + A.a22;
    T det = A.a11 * A.a22 - A.a21 * A.a12;
    T tmp = 0.25 * trc * trc - det;
    if (tmp <= 2.220446049250313e-16) tmp = 0.0;
    L1 = 0.5 * trc + Sqrt(tmp);
    L2 = 0.5 * trc - Sqrt(tmp);
    if (A.a21 != 0.0) {
      T r11 = L1 - A.a22, r21 = A.a21;
      T nrm = Sqrt(r11 * r11 + r21 * r21);
      r11 = r11 / nrm; r21 = r21 / nrm;
      Q = M2T<T>{r11, -r21, r21, r11};
    } else {
      L1 = A.a11; L2 = A.a22;
      Q = M2T<T>{1.0, 0.0, 0.0, 1.0};
      diagonal_turn(A, Q);
    }
  }
  // The a21 == 0 branch returns Q = I, the limit of the general branch as a21 -> 0, where the
  // eigenvector of L1 = a11 turns by a21 / (a11 - a22) (first order in a21, for a11 != a22).
  // The derivative of the map A -> Q f(Lambda) Q^T keeps that turn; the branch's own constant
  // Q would drop it.  The tangent carries it on Q's off-diagonal entries.
  static void diagonal_turn(const M2T<double>&, M2T<double>&) {}
  static void diagonal_turn(const M2T<Tan>& A, M2T<Tan>& Q) {
    double gap = A.a11.v - A.a22.v;
    if (gap == 0.0) return;
    Q.a21.d = A.a21.d / gap;
    Q.a12.d = -Q.a21.d;
  }
  // constitutive_eqn_evolve (predictor_mod.F90:141-251), Lagrangian, const_mod=2: the update
  // of one particle's stress t (planes t11, t21, t12, t22) and conformation trace under the
  // velocity gradient g (du/dx, du/dy, dv/dx, dv/dy) over dt
  template <class T>
  static void logconf_particle(T t[4], T& trace, const T g[4], double dtl, double Wi, double eps_PTT) {
    using MR = M2T<T>;
    // steps 1-2
    MR A{t[0] / 1.0 + 1.0, t[2] / 1.0 + 0.0, t[1] / 1.0 + 0.0, t[3] / 1.0 + 1.0};
    A = MR{A.a11 / 1.0, A.a12 / 1.0, A.a21 / 1.0, A.a22 / 1.0};
    T L1, L2; MR Q;
    calc_eigens(A, L1, L2, Q);
    // step 3
    MR D{Log(L1), 0.0, 0.0, Log(L2)};
    MR Psi0 = mm(Q, mm(D, tr(Q)));
    // step 5
    MR G{g[0], g[1], g[2], g[3]};  // G(a,b) = du_a/dx_b
    MR tm = mm(tr(Q), mm(G, Q));
    T tmp1 = (L2 * tm.a12 + L1 * tm.a21) / (L2 - L1 + 1e-10);
    tm.a12 = 0.0; tm.a21 = 0.0;
    MR B = mm(Q, mm(tm, tr(Q)));
    MR W{0.0, tmp1, -tmp1, 0.0};
    MR Om = mm(Q, mm(W, tr(Q)));
    // step 6
    MR OP = mm(Om, Psi0), PO = mm(Psi0, Om);
    MR t6{2.0 * B.a11 + OP.a11 - PO.a11, 2.0 * B.a12 + OP.a12 - PO.a12,
          2.0 * B.a21 + OP.a21 - PO.a21, 2.0 * B.a22 + OP.a22 - PO.a22};
    MR Psi{Psi0.a11 + dtl * t6.a11, Psi0.a12 + dtl * t6.a12, Psi0.a21 + dtl * t6.a21,
           Psi0.a22 + dtl * t6.a22};
    // step 7
    calc_eigens(Psi, L1, L2, Q);
    L1 = Exp(L1); L2 = Exp(L2);
    MR E2{L1, 0.0, 0.0, L2};
    A = mm(Q, mm(E2, tr(Q)));
    // step 8: f_relaxation_integrate (:318-331) with the old trace
    T alpha_R = 1.0 + eps_PTT * (trace - 2.0);
    T e1 = Exp(-(alpha_R * 1.0 * dtl / Wi));
    T e2 = (1.0 - e1) / 1.0;
    A = MR{A.a11 * e1 + e2 * 1.0, A.a12 * e1 + e2 * 0.0, A.a21 * e1 + e2 * 0.0, A.a22 * e1 + e2 * 1.0};
    // step 9
    trace = A.a11 + A.a22;
    t[0] = 1.0 * (1.0 * A.a11 - 1.0);
    t[2] = 1.0 * (1.0 * A.a12 - 0.0);
    t[1] = 1.0 * (1.0 * A.a21 - 0.0);
    t[3] = 1.0 * (1.0 * A.a22 - 1.0);
  }
  void constitutive_eqn_evolve() {
    const double eps_PTT = P.ve_nonlinearity;
    const double Wi = P.El * std::sqrt(P.Ra / P.Pr);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npfb; ++i) {
      R t[4] = {tau[0][i], tau[1][i], tau[2][i], tau[3][i]};
      const R g[4] = {grad[0][i], grad[1][i], grad[2][i], grad[3][i]};
      R trace = trace_conf[i];
      logconf_particle(t, trace, g, dt, Wi, eps_PTT);
      for (int q = 0; q < 4; ++q) tau[q][i] = t[q];
      trace_conf[i] = trace;
      a_out[i] = trace_conf[i];
    }
    mirror_polymeric_stress();
  }

  // ------------------------------------------------------------------ prediction_step
  // predictor_mod.F90:27-139
  void prediction_step() {
    grad_operators();
    if (P.const_mod != 1) constitutive_eqn_evolve();
    const double cs = P.beta * std::sqrt(P.Pr / P.Ra);
    const double cp = (1.0 - P.beta) * P.Pr / (P.Ra * P.El);
    const double ct = 1.0 / std::sqrt(P.Ra * P.Pr);
    std::vector<R> rh1(npfb), rh2(npfb), rht(npfb);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npfb; ++i) {
      R s1 = 0.0, s2 = 0.0, st = 0.0;
      M2 Kc = K(i);
      for (int k = 0; k < ij_count[i]; ++k) {
        int j = L(k, i);
        R u1 = ux[i] - ux[j], u2 = uy[i] - uy[j];
        double w1 = wGx[E(k, i)], w2 = wGy[E(k, i)], wl = wL[E(k, i)];
        if (P.const_mod == 1) {
          s1 = s1 + cs * u1 * wl;
          s2 = s2 + cs * u2 * wl;
        } else {
          R T11 = tau[0][j] - tau[0][i], T21 = tau[1][j] - tau[1][i];
          R T12 = tau[2][j] - tau[2][i], T22 = tau[3][j] - tau[3][i];
          double kw1 = Kc.a11 * w1 + Kc.a12 * w2, kw2 = Kc.a21 * w1 + Kc.a22 * w2;
          R tw1 = T11 * kw1 + T12 * kw2, tw2 = T21 * kw1 + T22 * kw2;
          s1 = s1 + cp * tw1 + cs * u1 * wl;
          s2 = s2 + cp * tw2 + cs * u2 * wl;
        }
        R thij = theta[i] - theta[j];
        st = st + ct * thij * wl;
      }
      rh1[i] = s1; rh2[i] = s2; rht[i] = st;
    }
    // the circle mirrors' share of the same sums (the drag diagnostic; no reference counterpart)
    circ_s1.assign(npfb, R(0.0)); circ_s2.assign(npfb, R(0.0));
    if (P.nb_circles > 0) {
#pragma omp parallel for schedule(static)
      for (int i = nbS; i < npfb; ++i) {
        R s1 = 0.0, s2 = 0.0;
        M2 Kc = K(i);
        for (int k = 0; k < ij_count[i]; ++k) {
          int j = L(k, i);
          if (j < npfb || vrelation[j] <= 999) continue;
          R u1 = ux[i] - ux[j], u2 = uy[i] - uy[j];
          double w1 = wGx[E(k, i)], w2 = wGy[E(k, i)], wl = wL[E(k, i)];
          if (P.const_mod == 1) {
            s1 = s1 + cs * u1 * wl;
            s2 = s2 + cs * u2 * wl;
          } else {
            R T11 = tau[0][j] - tau[0][i], T21 = tau[1][j] - tau[1][i];
            R T12 = tau[2][j] - tau[2][i], T22 = tau[3][j] - tau[3][i];
            double kw1 = Kc.a11 * w1 + Kc.a12 * w2, kw2 = Kc.a21 * w1 + Kc.a22 * w2;
            s1 = s1 + cp * (T11 * kw1 + T12 * kw2) + cs * u1 * wl;
            s2 = s2 + cp * (T21 * kw1 + T22 * kw2) + cs * u2 * wl;
          }
        }
        circ_s1[i] = s1; circ_s2[i] = s2;
      }
    }
    for (int i = 0; i < npfb; ++i) rh2[i] = rh2[i] + theta[i];  // buoyancy (:111-119)
    for (int i = nbS; i < npfb; ++i) {
      ux[i] = ux[i] + rh1[i] * dt;
      uy[i] = uy[i] + rh2[i] * dt;
    }
    for (int i = nbS; i < npfb; ++i) theta[i] = theta[i] + rht[i] * dt;
  }

  // ------------------------------------------------------------------ PPE
  void sparse_atime(const std::vector<double>& x, std::vector<double>& b) const {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npfb; ++i) {
      double bb = ppe_diag[i] * x[i];
      for (int k = 0; k < ij_count[i]; ++k) bb = bb + ppe_val[E(k, i)] * x[ppe_col[E(k, i)]];
      b[i] = bb;
    }
  }
  double vtime(const std::vector<double>& a, const std::vector<double>& b) const {
    return chunk_sum(0, npfb, [&](int64_t i) { return a[i] * b[i]; });
  }
  void remove_dc(std::vector<double>& a) const {
    double tmp = chunk_sum(0, npfb, [&](int64_t i) { return a[i]; });
    tmp = tmp / (double)npfb;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npfb; ++i) a[i] = a[i] - tmp;
  }

  // SPARSE_PBICGSTAB_nonull (linear_solver.F90:275-425) and SPARSE_PBICGSTAB (:82-227)
  void bicgstab(std::vector<double>& x, const std::vector<double>& B, bool nonull) {
    const int n = npfb;
    const double tol = P.tol;
    const int itermax = P.itermax;
    std::vector<double> r(n), r_bar(n), v(n, 0.0), AX(n), pp(n, 0.0), p_inv(n, 0.0), s(n, 0.0),
        s_inv(n, 0.0), t(n, 0.0), M(n);
    double rho0 = 1.0, alpha = 1.0, omega = 1.0, rho = 0.0, temp = 0.0, beta = 0.0;
    if (nonull) for (int i = 0; i < n; ++i) M[i] = 1.0;
    else for (int i = 0; i < n; ++i) M[i] = ppe_diag[i];  // sparse_make_preconditioner
    sparse_atime(x, AX);
    for (int i = 0; i < n; ++i) { r[i] = B[i] - AX[i]; r_bar[i] = r[i]; }
    // the open-domain solver's small-norm threshold is the integer expression 10-6 (= 4)
    const double small = nonull ? 1.0e-6 : 4.0;
    int iter = 1;
    double n2r0 = 1.0, n2s0 = 1.0, n2r = 0, n2s = 0, n2t = 0;
    LS_residual = 0.0;
    bool done = false;
    while (iter <= itermax) {
      rho = vtime(r_bar, r);
      if (rho == 0.0) { warnings |= VEBI_WARN_BICGSTAB_BREAKDOWN; done = true; break; }
      if (iter == 1) {
        for (int i = 0; i < n; ++i) pp[i] = r[i];
      } else {
        beta = rho / (rho0 + 1.0e-15) * alpha / (omega + 1.0e-15);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) pp[i] = r[i] + beta * (pp[i] - omega * v[i]);
      }
      if (nonull) remove_dc(pp);
#pragma omp parallel for schedule(static)
      for (int i = 0; i < n; ++i) p_inv[i] = pp[i] / (M[i] + 1.0e-15);
      sparse_atime(p_inv, v);
      temp = vtime(r_bar, v);
      alpha = rho / (temp + 1.0e-15);
#pragma omp parallel for schedule(static)
      for (int i = 0; i < n; ++i) s[i] = r[i] - alpha * v[i];
      n2s = vtime(s, s);
      if (iter == 1) n2s0 = (n2s <= small) ? 1.0 : n2s;
      if (n2s <= tol * tol * n2s0) {
        for (int i = 0; i < n; ++i) x[i] = x[i] + alpha * p_inv[i];
        LS_residual = std::sqrt(n2s / n2s0);
        done = true;
        break;
      }
      if (nonull) remove_dc(s);
#pragma omp parallel for schedule(static)
      for (int i = 0; i < n; ++i) s_inv[i] = s[i] / (M[i] + 1.0e-15);
      sparse_atime(s_inv, t);
      temp = vtime(t, s);
      n2t = vtime(t, t);
      omega = temp / (n2t + 1.0e-15);
#pragma omp parallel for schedule(static)
      for (int i = 0; i < n; ++i) {
        x[i] = x[i] + alpha * p_inv[i] + omega * s_inv[i];
        r[i] = s[i] - omega * t[i];
      }
      n2r = vtime(r, r);
      if (iter == 1) n2r0 = (n2r <= small) ? 1.0 : n2r;
      LS_residual = std::sqrt(n2r / n2r0);
      if (n2r <= tol * tol * n2r0) { done = true; break; }
      iter = iter + 1;
      rho0 = rho;
    }
    if (!done) warnings |= VEBI_WARN_MAXITER;
    LS_iters = iter;
  }

  // The PPE solve over the field type.  With R = Tan the system is solved twice on the same
  // matrix: the values (the step's own solve, which sets LS_iters and LS_residual) and then the
  // derivatives, A dP = dB, from a zero start.  dB is scaled to unit RMS for that solve and the
  // result scaled back, since the solver's rule that a first residual norm <= 1e-6 makes the
  // tolerance absolute would otherwise stop a small tangent after one iteration.
  int tangent_iters = 0;
  void solve_system(std::vector<R>& x, const std::vector<R>& B) {
    const bool nonull = P.i_open_domain == 0;
    if constexpr (std::is_same<R, double>::value) {
      bicgstab(x, B, nonull);
    } else {
      std::vector<double> xv(npfb), bv(npfb), xd(npfb, 0.0), bd(npfb);
      for (int i = 0; i < npfb; ++i) { xv[i] = x[i].v; bv[i] = B[i].v; bd[i] = B[i].d; }
      bicgstab(xv, bv, nonull);
      const int it = LS_iters;
      const double res = LS_residual;
      const int warn = warnings;
      double ms = chunk_sum(0, npfb, [&](int64_t i) { return bd[i] * bd[i]; }) / (double)npfb;
      tangent_iters = 0;
      if (ms > 0.0) {
        const double rms = std::sqrt(ms);
        for (auto& v : bd) v = v / rms;
        bicgstab(xd, bd, nonull);
        tangent_iters = LS_iters;
        for (auto& v : xd) v = v * rms;
      }
      LS_iters = it; LS_residual = res; warnings = warn;
      for (int i = 0; i < npfb; ++i) x[i] = Tan(xv[i], xd[i]);
    }
  }

  // ppe_solve_in_house_simple_dirichlet (ppe_solve_in_house_simple_dirichlet.F90:1-158)
  void ppe_solve() {
    ppe_B.assign(npfb, R(0.0));
    const double dtl = dt;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npfb; ++i) {
      R fb = 0.0;
      M2 Kc = K(i);
      for (int k = 0; k < ij_count[i]; ++k) {
        int j = L(k, i);
        R u1 = ux[i] - ux[j], u2 = uy[i] - uy[j];
        double w1 = wGx[E(k, i)], w2 = wGy[E(k, i)];
        double kw1 = Kc.a11 * w1 + Kc.a12 * w2, kw2 = Kc.a21 * w1 + Kc.a22 * w2;
        fb = fb - (u1 * kw1 + u2 * kw2);
      }
      ppe_B[i] = fb / dtl;
    }
    ppe_rhs_mean = 0.0;
    if (P.i_open_domain == 0) {
      R temp = chunk_sum(0, npfb, [&](int64_t i) { return ppe_B[i]; });
      temp = temp / (double)npfb;
      ppe_rhs_mean = val(temp);
      for (int i = 0; i < npfb; ++i) ppe_B[i] = ppe_B[i] - temp;
    }
    // assembly: one ELL slot per neighbour; duplicate parent columns accumulate into the
    // last slot written for that column, earlier duplicates keep 0 (ppe...:72-121)
    size_t n = (size_t)std::max(maxneighbours, 1) * npfb;
    ppe_val.assign(n, 0.0);
    ppe_col.assign(n, 0);
    ppe_diag.assign(npfb, 0.0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npfb; ++i) {
      const int cnt = ij_count[i];
      bool any_mirror = false;
      for (int k = 0; k < cnt; ++k) {
        int j = L(k, i);
        ppe_col[E(k, i)] = (j < npfb) ? j : irelation[j];
        any_mirror |= (j >= npfb);
      }
      // without mirror neighbours every column is distinct, so slot k is its own last slot
      auto last_slot = [&](int k, int c) {
        if (!any_mirror) return k;
        for (int kk = cnt - 1; kk >= 0; --kk)
          if (ppe_col[E(kk, i)] == c) return kk;
        return k;
      };
      double Adiag = 0.0;
      for (int k = 0; k < cnt; ++k) {
        int j = L(k, i);
        double temp = -wL[E(k, i)];
        Adiag = Adiag - temp;
        if (j >= npfb) {
          int ij = irelation[j];
          if (i != ij) {
            int nt = last_slot(k, ij);
            ppe_val[E(nt, i)] = ppe_val[E(nt, i)] + temp;
          } else {
            Adiag = Adiag + temp;
          }
          ppe_B[i] = ppe_B[i] - dP_mp[j] * temp;
        } else {
          int nt = last_slot(k, j);
          ppe_val[E(nt, i)] = ppe_val[E(nt, i)] + temp;
        }
      }
      if (n_surf[i] != 0) Adiag = 1.0e30;
      ppe_diag[i] = 0.0 + Adiag;
    }
    if (P.i_open_domain == 1) {
      for (int i = 0; i < npfb; ++i) {
        if (n_surf[i] == 1) continue;
        if (ppe_smooth[i] == 1.0) continue;
        ppe_B[i] = ppe_B[i] * ppe_smooth[i];
        for (int k = 0; k < ij_count[i]; ++k) ppe_val[E(k, i)] = ppe_val[E(k, i)] * ppe_smooth[i];
      }
    }
    std::vector<R> x(npfb, R(0.0));
    if (P.ppe_warm_start)  // opt-in: start from the previous step's P (the reference uses 0)
      for (int i = 0; i < npfb; ++i) x[i] = p[i];
    mark(10);
    double t0 = wtime();
    solve_system(x, ppe_B);
    t_solve_ms = (wtime() - t0) * 1e3;
    mark(9);
    for (int i = 0; i < npfb; ++i) p[i] = x[i];
  }

  // calc_pressure_gradient (gradient_calculation.F90:16-48)
  void calc_pressure_gradient() {
    for (int j = npfb; j < np; ++j) p[j] = p[irelation[j]] + dP_mp[j];
    gpx.assign(npfb, R(0.0)); gpy.assign(npfb, R(0.0));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npfb; ++i) {
      R a = 0.0, b = 0.0;
      for (int k = 0; k < ij_count[i]; ++k) {
        int j = L(k, i);
        R temp = p[j] - p[i];
        a = a + temp * wGx[E(k, i)];
        b = b + temp * wGy[E(k, i)];
      }
      M2 Kc = K(i);
      gpx[i] = Kc.a11 * a + Kc.a12 * b;
      gpy[i] = Kc.a21 * a + Kc.a22 * b;
    }
    // force of the fluid on the circles: per fluid particle, dv x (circle-mirror share of the
    // pressure gradient - circle-mirror share of the viscous/polymeric sums)
    circle_fx = circle_fy = 0.0;
    if (P.nb_circles > 0) {
      std::vector<R> fx(npfb, R(0.0)), fy(npfb, R(0.0));
#pragma omp parallel for schedule(static)
      for (int i = nbS; i < npfb; ++i) {
        if (inbin[i]) continue;
        R a = 0.0, b = 0.0;
        for (int k = 0; k < ij_count[i]; ++k) {
          int j = L(k, i);
          if (j < npfb || vrelation[j] <= 999) continue;
          R temp = p[j] - p[i];
          a = a + temp * wGx[E(k, i)];
          b = b + temp * wGy[E(k, i)];
        }
        M2 Kc = K(i);
        fx[i] = P.dv * ((Kc.a11 * a + Kc.a12 * b) - circ_s1[i]);
        fy[i] = P.dv * ((Kc.a21 * a + Kc.a22 * b) - circ_s2[i]);
      }
      circle_fx = val(chunk_sum(0, npfb, [&](int64_t i) { return fx[i]; }));
      circle_fy = val(chunk_sum(0, npfb, [&](int64_t i) { return fy[i]; }));
    }
  }

  // correct_velocity (correct_velocity.F90:13-70): remove the velocity component of particles
  // closing on a wall mirror closer than dx.  The reference indexes b_type(vrelation(j)) also for
  // circle mirrors (vrelation = 999+ib, out of range); here a circle mirror is not a wall.
  void correct_velocity() {
    std::vector<int> close(npfb, -1);
    for (int i = nbS; i < npfb; ++i) {
      double r_min2 = dx * dx;
      for (int k = 0; k < ij_count[i]; ++k) {
        int j = L(k, i);
        if (j < npfb) continue;
        double a = rx[i] - rx[j], b = ry[i] - ry[j];
        double d2 = a * a + b * b;
        if (!(d2 < r_min2)) continue;
        int vr = vrelation[j];
        if (vr > 0 && vr < 999 && P.b_type[vr - 1] == 1) { r_min2 = d2; close[i] = j; }
        if (vr == -1 || vr < -2) { r_min2 = d2; close[i] = j; }
      }
    }
    for (int i = nbS; i < npfb; ++i) {
      int j = close[i];
      if (j < 0) continue;
      double n1 = rx[i] - rx[j], n2 = ry[i] - ry[j];
      double t = std::sqrt(n1 * n1 + n2 * n2);
      n1 = n1 / t; n2 = n2 / t;
      R u1 = ux[i] - ux[j], u2 = uy[i] - uy[j];
      R un = u1 * n1 + u2 * n2;
      if (un <= 0.0) { ux[i] = ux[i] - un * n1; uy[i] = uy[i] - un * n2; }
    }
  }

  // secondary_properties (div_free.F90:148-192), only when asked
  void secondary_properties() {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npfb; ++i) {
      R vt = 0.0;
      for (int k = 0; k < ij_count[i]; ++k) {
        int j = L(k, i);
        R tmp = (uy[i] - uy[j]) * wGx[E(k, i)] - (ux[i] - ux[j]) * wGy[E(k, i)];
        vt = vt - tmp;
      }
      vort[i] = vt;
    }
    double s = val(chunk_sum(0, npfb, [&](int64_t i) { return ux[i] * ux[i] + uy[i] * uy[i]; }));
    rms_u = std::sqrt(s / (double)npfb);
  }

  // ------------------------------------------------------------------ div_free
  int step(double xmn, double ymn, double xmx, double ymx, int secondary) {
    double t0 = wtime();
    int st = step_body(xmn, ymn, xmx, ymx, secondary);
    t_step_ms = (wtime() - t0) * 1e3;
    return st;
  }
  double stage_t[VEBI_NSTAGES] = {};
  double tmark = 0.0;
  int tstage = -1;
  void mark(int s) {  // per-stage wall time, same stage numbering as the GPU library
    double t = wtime();
    if (tstage >= 0 && tstage < VEBI_NSTAGES) stage_t[tstage] += (t - tmark) * 1e3;
    tstage = s;
    tmark = t;
  }
  int step_body(double xmn, double ymn, double xmx, double ymx, int secondary) {
    for (auto& v : stage_t) v = 0.0;
    tstage = -1;
    mark(0);
    int st = step_stages(xmn, ymn, xmx, ymx, secondary);
    mark(-1);
    return st;
  }
  int step_stages(double xmn, double ymn, double xmx, double ymx, int secondary) {
    error = 0; warnings = 0; n_escapees = 0;
    // STEP 1 (div_free.F90:39-41)
    r0x.assign(2 * npfb, 0.0); r0y.assign(2 * npfb, 0.0);
    u0x.assign(2 * npfb, R(0.0)); u0y.assign(2 * npfb, R(0.0));
    for (int i = 0; i < npfb; ++i) { u0x[i] = ux[i]; u0y[i] = uy[i]; r0x[i] = rx[i]; r0y[i] = ry[i]; }
    // STEP 2
    set_time_step();
    const bool replay = geo_mode == 2 && geo_step < geo_dt.size();
    if (replay) dt = geo_dt[geo_step];
    // STEP 3
    for (int i = nbS; i < npfb; ++i) {
      rx[i] = r0x[i] + val(u0x[i]) * dt;
      ry[i] = r0y[i] + val(u0y[i]) * dt;
    }
    if (replay) {
      std::copy(geo_rx[geo_step].begin(), geo_rx[geo_step].end(), rx.begin());
      std::copy(geo_ry[geo_step].begin(), geo_ry[geo_step].end(), ry.begin());
    }
    // STEP 4
    int st = put_in_bin(xmn, xmx, ymn, ymx);
    if (st) return st;
    if (geo_mode == 1) {
      geo_rx.emplace_back(rx.begin(), rx.begin() + npfb);
      geo_ry.emplace_back(ry.begin(), ry.begin() + npfb);
      geo_dt.push_back(dt);
    }
    if (geo_mode != 0) ++geo_step;
    mark(1);
    st = create_mirror_particles();
    if (st) return st;
    if (n_escapees) warnings |= VEBI_WARN_ESCAPEES;
    rsx.assign(rx.begin(), rx.begin() + np); rsy.assign(ry.begin(), ry.begin() + np);
    mark(2);
    st = divide();
    if (st) return st;
    mark(3);
    st = neighbour_list();
    if (st) return st;
    mark(4);
    kernel_calculation();
    locate_free_surf_part();
    mark(5);
    // STEP 5
    ushx.assign(npfb, 0.0); ushy.assign(npfb, 0.0);
    new_fick_shift();
    for (int i = 0; i < npfb; ++i) { ushx[i] = drx[i] / dt; ushy[i] = dry[i] / dt; }
    for (int i = 0; i < nbS; ++i) { ushx[i] = -val(ux[i]); ushy[i] = -val(uy[i]); }
    // STEP 7
    mark(8);
    prediction_step();
    // STEP 8
    mirror_velocities();
    mark(9);
    ustx.assign(ux.begin(), ux.begin() + np); usty.assign(uy.begin(), uy.begin() + np);
    thst.assign(theta.begin(), theta.begin() + npfb);
    ppe_solve();
    // STEP 9
    mark(11);
    calc_pressure_gradient();
    for (int i = nbS; i < npfb; ++i) {
      ux[i] = ux[i] + dt * (P.body_force[0] - gpx[i]);
      uy[i] = uy[i] + dt * (P.body_force[1] - gpy[i]);
      if (ij_count[i] <= 3) {
        ux[i] = u0x[i] + dt * P.body_force[0];
        uy[i] = u0y[i] + dt * P.body_force[1];
      }
    }
    // STEP 10 (off in the reference: the call is commented out, div_free.F90:105)
    if (P.correct_velocity) correct_velocity();
    // STEP 11
    mark(13);
    if (secondary) secondary_properties();
    mark(12);
    // STEP 12
    for (int i = nbS; i < npfb; ++i) {
      rx[i] = r0x[i] + val(0.5 * (ux[i] + u0x[i])) * dt + ushx[i] * dt;
      ry[i] = r0y[i] + val(0.5 * (uy[i] + u0y[i])) * dt + ushy[i] * dt;
    }
    time += dt;
    return VEBI_OK;
  }

  void fill_stats(vebi_step_stats* s) const {
    std::memset(s, 0, sizeof(*s));
    s->dt = dt; s->LS_residual = LS_residual; s->umax = umax;
    double mu = 0, mv = 0, mp = 0;
    for (int i = 0; i < npfb; ++i) {
      mu = std::max(mu, std::fabs(val(ux[i]))); mv = std::max(mv, std::fabs(val(uy[i])));
      mp = std::max(mp, std::fabs(val(p[i])));
    }
    s->max_abs_u = mu; s->max_abs_v = mv; s->max_abs_p = mp;
    s->rms_u = rms_u; s->ppe_rhs_mean = ppe_rhs_mean;
    s->circle_force[0] = circle_fx; s->circle_force[1] = circle_fy;
    s->LS_iters = LS_iters; s->n_inbin = n_inbin; s->np = np; s->npfb = npfb;
    s->nmirror = nmirror; s->maxneighbours = maxneighbours; s->n_escapees = n_escapees;
    s->error = error; s->warnings = warnings;
    for (int q = 0; q < VEBI_NSTAGES; ++q) s->stage_ms[q] = stage_t[q];
    s->stage_ms[10] = t_solve_ms;   // PPE solve
    s->stage_ms[14] = t_step_ms;    // whole step
    s->LS_iters_total = LS_iters; s->nsteps = 1;
  }

  // ------------------------------------------------------------------ inspection
  struct View { const void* p; int64_t esz, n; };
  static View view_of(const std::vector<double>& v, int64_t n) { return View{v.data(), 8, n}; }
  static View view_of(const std::vector<Tan>&, int64_t) { return View{nullptr, 0, -1}; }
  View view(const std::string& nm) const {
    auto D = [](const auto& v, int64_t n) { return view_of(v, n); };
    auto I = [](const std::vector<int>& v, int64_t n) { return View{v.data(), 4, n}; };
    int64_t ell = (int64_t)std::max(maxneighbours, 1) * npfb;
    if (nm == "rx") return D(rx, np);
    if (nm == "ry") return D(ry, np);
    if (nm == "ux") return D(ux, np);
    if (nm == "uy") return D(uy, np);
    if (nm == "theta") return D(theta, np);
    if (nm == "p") return D(p, np);
    if (nm == "tau11") return D(tau[0], np);
    if (nm == "tau21") return D(tau[1], np);
    if (nm == "tau12") return D(tau[2], np);
    if (nm == "tau22") return D(tau[3], np);
    if (nm == "trace_conf") return D(trace_conf, npfb);
    if (nm == "a_out") return D(a_out, npfb);
    if (nm == "vort") return D(vort, npfb);
    if (nm == "n_surf") return I(n_surf, np);
    if (nm == "irelation") return View{irelation.data() + npfb, 4, nmirror};
    if (nm == "vrelation") return View{vrelation.data() + npfb, 4, nmirror};
    if (nm == "dP_mp") return View{dP_mp.data() + npfb, 8, nmirror};
    if (nm == "rsx") return D(rsx, (int64_t)rsx.size());
    if (nm == "rsy") return D(rsy, (int64_t)rsy.size());
    if (nm == "cellpart") return I(cellpart, (int64_t)cellpart.size());
    if (nm == "ist") return I(ist, (int64_t)ist.size());
    if (nm == "ip") return I(ipl, ist.empty() ? 0 : ist.back());
    if (nm == "ij_count") return I(ij_count, npfb);
    if (nm == "ij_link") return I(ij_link, ell);
    if (nm == "w_Gx") return D(wGx, ell);
    if (nm == "w_Gy") return D(wGy, ell);
    if (nm == "w_L") return D(wL, ell);
    if (nm == "kgcm11") return D(kgcm[0], npfb);
    if (nm == "kgcm21") return D(kgcm[1], npfb);
    if (nm == "kgcm12") return D(kgcm[2], npfb);
    if (nm == "kgcm22") return D(kgcm[3], npfb);
    if (nm == "gradu_x") return D(grad[0], np);
    if (nm == "gradu_y") return D(grad[1], np);
    if (nm == "gradv_x") return D(grad[2], np);
    if (nm == "gradv_y") return D(grad[3], np);
    if (nm == "gradth_x") return D(grad[4], np);
    if (nm == "gradth_y") return D(grad[5], np);
    if (nm == "gradC_x") return D(gradCx, npfb);
    if (nm == "gradC_y") return D(gradCy, npfb);
    if (nm == "ushift_x") return D(ushx, npfb);
    if (nm == "ushift_y") return D(ushy, npfb);
    if (nm == "ustar_x") return D(ustx, (int64_t)ustx.size());
    if (nm == "ustar_y") return D(usty, (int64_t)usty.size());
    if (nm == "theta_star") return D(thst, (int64_t)thst.size());
    if (nm == "ppe_B") return D(ppe_B, npfb);
    if (nm == "ppe_diag") return D(ppe_diag, npfb);
    if (nm == "ppe_val") return D(ppe_val, ell);
    if (nm == "ppe_col") return I(ppe_col, ell);
    if (nm == "grad_px") return D(gpx, npfb);
    if (nm == "grad_py") return D(gpy, npfb);
    if (nm == "conc") return D(conc, npfb);
    if (nm == "div_r") return D(div_r, npfb);
    return View{nullptr, 0, -1};
  }
  // the fields of the tangent-linear model, by name, with their lengths
  const std::vector<R>* field(const std::string& nm, int64_t* n) const {
    *n = np;
    if (nm == "ux") return &ux;
    if (nm == "uy") return &uy;
    if (nm == "theta") return &theta;
    if (nm == "p") return &p;
    if (nm == "tau11") return &tau[0];
    if (nm == "tau21") return &tau[1];
    if (nm == "tau12") return &tau[2];
    if (nm == "tau22") return &tau[3];
    *n = npfb;
    if (nm == "trace_conf") return &trace_conf;
    if (nm == "ppe_B") return &ppe_B;
    return nullptr;
  }
};

using Oracle = OracleT<double>;
using OracleTan = OracleT<Tan>;

}  // namespace

extern "C" {

void* orc_create(const vebi_params* p, int* status) {
  auto* o = new Oracle();
  int st = o->create(p);
  if (status) *status = st;
  if (st) { delete o; return nullptr; }
  return o;
}
int orc_destroy(void* h) { delete static_cast<Oracle*>(h); return 0; }
int orc_set_state(void* h, const double* r, const double* u, const double* tp, const double* th,
                  const double* tc, const uint8_t* ib, int ld) {
  return static_cast<Oracle*>(h)->set_state(r, u, tp, th, tc, ib, ld);
}
int orc_step(void* h, double xmn, double ymn, double xmx, double ymx, int secondary,
             vebi_step_stats* st) {
  auto* o = static_cast<Oracle*>(h);
  int s = o->step(xmn, ymn, xmx, ymx, secondary);
  if (st) { o->fill_stats(st); st->error = s; }
  return s;
}
// geometry record/replay of an FP64 oracle: 1 starts a record (clearing the last), 2 replays
// the record from its first step, 0 turns both off and drops the record
int orc_geometry(void* h, int mode) {
  auto* o = static_cast<Oracle*>(h);
  if (mode < 0 || mode > 2) return VEBI_ERR_ARG;
  if (mode != 2) { o->geo_rx.clear(); o->geo_ry.clear(); o->geo_dt.clear(); }
  o->geo_mode = mode;
  o->geo_step = 0;
  return 0;
}

// ---- FP64 tangent-linear model of the step (the oracle over forward-mode dual numbers)
void* orc_tlm_create(const vebi_params* p, int* status) {
  auto* o = new OracleTan();
  int st = o->create(p);
  if (status) *status = st;
  if (st) { delete o; return nullptr; }
  return o;
}
int orc_tlm_destroy(void* h) { delete static_cast<OracleTan*>(h); return 0; }
int orc_tlm_set_state(void* h, const double* r, const double* u, const double* tp, const double* th,
                      const double* tc, const uint8_t* ib, int ld) {
  return static_cast<OracleTan*>(h)->set_state(r, u, tp, th, tc, ib, ld);
}
int orc_tlm_set_tangent(void* h, const double* du, const double* dtp, const double* dth, int ld) {
  return static_cast<OracleTan*>(h)->set_tangent(du, dtp, dth, ld);
}
int orc_tlm_step(void* h, double xmn, double ymn, double xmx, double ymx, vebi_step_stats* st,
                 int* tangent_iters) {
  auto* o = static_cast<OracleTan*>(h);
  int s = o->step(xmn, ymn, xmx, ymx, 0);
  if (st) { o->fill_stats(st); st->error = s; }
  if (tangent_iters) *tangent_iters = o->tangent_iters;
  return s;
}
int orc_tlm_size(void* h, const char* name, int64_t* n) {
  return static_cast<OracleTan*>(h)->field(name, n) ? 0 : VEBI_ERR_ARG;
}
int orc_tlm_get(void* h, const char* name, double* value, double* tangent, int64_t n) {
  int64_t m = 0;
  const auto* f = static_cast<OracleTan*>(h)->field(name, &m);
  if (!f || n < m) return VEBI_ERR_ARG;
  for (int64_t i = 0; i < m; ++i) {
    if (value) value[i] = (*f)[i].v;
    if (tangent) tangent[i] = (*f)[i].d;
  }
  return 0;
}
int orc_tlm_box(void* h, double* box4) {
  auto* o = static_cast<OracleTan*>(h);
  box4[0] = o->x_mint; box4[1] = o->x_maxt; box4[2] = o->y_mint; box4[3] = o->y_maxt;
  return 0;
}
int orc_tlm_set_itermax(void* h, int itermax) {
  static_cast<OracleTan*>(h)->P.itermax = itermax;
  return 0;
}

int orc_set_itermax(void* h, int itermax) {
  static_cast<Oracle*>(h)->P.itermax = itermax;
  return 0;
}
int orc_box(void* h, double* box4, int* ncxy) {
  auto* o = static_cast<Oracle*>(h);
  box4[0] = o->x_mint; box4[1] = o->x_maxt; box4[2] = o->y_mint; box4[3] = o->y_maxt;
  ncxy[0] = o->ncx; ncxy[1] = o->ncy;
  return 0;
}
int orc_size(void* h, const char* name, int64_t* esz, int64_t* n) {
  auto v = static_cast<Oracle*>(h)->view(name);
  if (v.n < 0) return VEBI_ERR_ARG;
  *esz = v.esz; *n = v.n;
  return 0;
}
int orc_get(void* h, const char* name, void* out, int64_t bytes) {
  auto v = static_cast<Oracle*>(h)->view(name);
  if (v.n < 0 || bytes < v.n * v.esz) return VEBI_ERR_ARG;
  if (v.n > 0) std::memcpy(out, v.p, (size_t)(v.n * v.esz));
  return 0;
}
double orc_kernel_w(void* h, double q) { return static_cast<Oracle*>(h)->Wab(q); }
double orc_kernel_fac(void* h, double q) { return static_cast<Oracle*>(h)->fac(q); }
int orc_eigens(const double* A4, double* L2, double* R4) {
  M2 A{A4[0], A4[1], A4[2], A4[3]}, Q;
  Oracle::calc_eigens(A, L2[0], L2[1], Q);
  R4[0] = Q.a11; R4[1] = Q.a12; R4[2] = Q.a21; R4[3] = Q.a22;
  return 0;
}
// one particle's log-conformation update (test of the constitutive law): tau4 (t11, t21, t12,
// t22) and trace updated in place under the velocity gradient g4 (du/dx, du/dy, dv/dx, dv/dy)
int orc_logconf_particle(double* tau4, double* trace, const double* g4, double dt, double Wi, double eps_ptt,
                         int nsteps) {
  for (int s = 0; s < nsteps; ++s) Oracle::logconf_particle(tau4, *trace, g4, dt, Wi, eps_ptt);
  return 0;
}
int orc_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
