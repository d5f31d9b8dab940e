// vebi_sph.cu -- per-pair SPH operators and per-particle updates of the step.
//
//  kernel_calculation (weights, Bonet-Lok kgcm)   kernel_calculation.F90:2-75
//  locate_free_surf_part, calc_part_dist_vars,
//  smooth_normals (open domain)                   freesurf_mod.F90:17-137
//  new_fick_shift + shifting_forces               new_fick_shift.F90:15-92,117-210
//  grad_operator (u, v, theta in one pass)        gradient_calculation.F90:50-94
//  constitutive_eqn_evolve, calc_eigens,
//  f_strain_*, f_relaxation_integrate             predictor_mod.F90:141-331
//  prediction_step pair loop and updates          predictor_mod.F90:27-139
//  calc_pressure_gradient + velocity update +
//  final advection                                gradient_calculation.F90:16-48, div_free.F90:94-117
//  secondary_properties                           div_free.F90:148-192
//
// One thread per particle walks that particle's ELL row k = 0..ij_count-1 in the reference's
// order with the reference's association, so every per-particle sum is the reference's sum.
#include "vebi_ctx.cuh"

namespace vebi {

#define ELL(k, i) ((size_t)(k) * c.npfb + (i))

// ---------------------------------------------------------------------- kernel_calculation
__global__ void k_weights(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const double xi = d.rx[i], yi = d.ry[i], dv = c.dv;
  double k11 = 0.0, k12 = 0.0, k21 = 0.0, k22 = 0.0;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    int j = d.ij_link[ELL(k, i)];
    double r1 = xi - d.rx[j], r2 = yi - d.ry[j];
    double rr2 = r1 * r1 + r2 * r2;
    double rad = sqrt(rr2);
    double qq = rad * c.oneoverh;
    double f = fac(c, qq);
    double m = fmax(rad, c.eta2);
    double g1 = r1 * f / m, g2 = r2 * f / m;
    double w1 = g1 * dv, w2 = g2 * dv;
    d.wGx[ELL(k, i)] = w1;
    d.wGy[ELL(k, i)] = w2;
    d.wL[ELL(k, i)] = 2.0 * (r1 * w1 + r2 * w2) / (rr2 + c.eta_small);
    k11 = k11 - dv * g1 * r1;
    k12 = k12 - dv * g2 * r1;
    k21 = k21 - dv * g1 * r2;
    k22 = k22 - dv * g2 * r2;
  }
  double temp = 1.0 / ((k11 * k22 - k12 * k21) + 1.0e-15);
  d.kgcm[0][i] = temp * k22;
  d.kgcm[2][i] = -temp * k12;
  d.kgcm[1][i] = -temp * k21;
  d.kgcm[3][i] = temp * k11;
}

// ---------------------------------------------------------------------- free surface (open)
__global__ void k_part_dist_vars(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const double xi = d.rx[i], yi = d.ry[i];
  double ct = 0, dr = 0, s1 = 0, s2 = 0;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    int j = d.ij_link[ELL(k, i)];
    double r1 = xi - d.rx[j], r2 = yi - d.ry[j];
    double rad = sqrt(r1 * r1 + r2 * r2);
    ct = ct + wab(c, rad / c.h);
    double w1 = d.wGx[ELL(k, i)], w2 = d.wGy[ELL(k, i)];
    dr = dr - (r1 * w1 + r2 * w2);
    s1 = s1 - w1;
    s2 = s2 - w2;
  }
  double w0 = wab(c, 0.0);
  double conc = ct * c.dv;
  conc = conc + c.dv * w0;
  d.conc[i] = conc;
  d.div_r[i] = dr;
  d.surf_nx[i] = s1 * c.h;
  d.surf_ny[i] = s2 * c.h;
  double bdr = 1.4 + 0.5 * fmax(conc - 1.0, -0.2);
  d.beta_div_r[i] = bdr;
  d.n_surf[i] = (dr > bdr) ? 0 : 1;
}

__global__ void k_nsurf_mirrors(Consts c, Dev d) {
  const int nm = d.s->nmirror;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nm; m += gridDim.x * blockDim.x) {
    int j = c.npfb + m;
    d.n_surf[j] = d.n_surf[d.irel[j]];
  }
}

// smooth_normals (Shepard filter) + ppe_smooth; the filtered normals go to gradCx/gradCy
// scratch first and are copied back after (the reference uses a temporary array too)
__global__ void k_smooth_normals(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const double xi = d.rx[i], yi = d.ry[i];
  double a = 0, b = 0;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    int j = d.ij_link[ELL(k, i)];
    if (j >= c.npfb) continue;
    double r1 = xi - d.rx[j], r2 = yi - d.ry[j];
    double rad = sqrt(r1 * r1 + r2 * r2);
    double w = wab(c, rad / c.h);
    a = a + w * d.surf_nx[j];
    b = b + w * d.surf_ny[j];
  }
  double w0 = wab(c, 0.0);
  d.gradCx[i] = a * c.dv + d.surf_nx[i] * w0 * c.dv;
  d.gradCy[i] = b * c.dv + d.surf_ny[i] * w0 * c.dv;
  double ps = 1.0;
  double dr = d.div_r[i], bdr = d.beta_div_r[i];
  if (!(dr > 1.2 * bdr)) {
    if (d.n_surf[i] == 1) ps = 0.0;
    else ps = 0.5 * (1.0 - cos((dr - bdr) * PI / (0.2 * bdr)));
  }
  d.ppe_smooth[i] = ps;
}

__global__ void k_copy_normals(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  d.surf_nx[i] = d.gradCx[i];
  d.surf_ny[i] = d.gradCy[i];
}

// ---------------------------------------------------------------------- shifting
__global__ void k_shift(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const double xi = d.rx[i], yi = d.ry[i];
  double f1 = 0, f2 = 0, t1 = 0, t2 = 0;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    int j = d.ij_link[ELL(k, i)];
    double r1 = xi - d.rx[j], r2 = yi - d.ry[j];
    double rad = sqrt(r1 * r1 + r2 * r2);
    double qq = rad / c.h;
    // Rt*(Wab/Wab1)**nt with nt = 4.0 (new_fick_shift.F90:135-148); the reference calls pow
    double fab = 0.25 * pw4(wab(c, qq) / c.wab1);
    double w1 = d.wGx[ELL(k, i)], w2 = d.wGy[ELL(k, i)];
    f1 = f1 + w1;
    f2 = f2 + w2;
    t1 = t1 + w1 * fab;
    t2 = t2 + w2 * fab;
  }
  double gx = f1 + t1, gy = f2 + t2;
  d.gradCx[i] = gx;
  d.gradCy[i] = gy;
  const double dt = d.s->dt;
  double d1 = 0.0, d2 = 0.0;
  if (i >= c.nbS) {
    double D;
    if (c.shift_coeff == 1) {
      double maxU = bits_to_double(d.s->maxU_bits);
      double absU = sqrt(d.ux[i] * d.ux[i] + d.uy[i] * d.uy[i]);
      double temp = (double)0.2f * exp(-absU / ((double)0.2f * maxU));
      D = 4.0 * c.h * dt * (absU + temp * maxU);
    } else {
      D = 0.25 * c.h * c.h;
    }
    if (d.n_surf[i] == 1 && c.open_domain == 1) {
      double temp = sqrt(d.surf_nx[i] * d.surf_nx[i] + d.surf_ny[i] * d.surf_ny[i]);
      double sn1 = d.surf_nx[i] / fmax(temp, (double)1e-8f);
      double sn2 = d.surf_ny[i] / fmax(temp, (double)1e-8f);
      double st1 = -sn2, st2 = sn1;
      double dCds = st1 * gx + st2 * gy;
      d1 = -D * dCds * st1;
      d2 = -D * dCds * st2;
    } else {
      d1 = -D * gx;
      d2 = -D * gy;
    }
    double temp = sqrt(d1 * d1 + d2 * d2);
    if (temp > 0.1 * c.h) {
      d1 = 0.1 * c.h * d1 / temp;
      d2 = 0.1 * c.h * d2 / temp;
    }
  }
  // ushift = dr_fs/dt; solid boundary particles get -u (div_free.F90:65-78)
  if (i < c.nbS) {
    d.ushx[i] = -d.ux[i];
    d.ushy[i] = -d.uy[i];
  } else {
    d.ushx[i] = d1 / dt;
    d.ushy[i] = d2 / dt;
  }
}

// ---------------------------------------------------------------------- gradients
__global__ void k_gradients(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const double ui = d.ux[i], vi = d.uy[i], ti = d.th[i];
  double a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    int j = d.ij_link[ELL(k, i)];
    double w1 = d.wGx[ELL(k, i)], w2 = d.wGy[ELL(k, i)];
    double du = d.ux[j] - ui, dvv = d.uy[j] - vi, dth = d.th[j] - ti;
    a0 = a0 + du * w1;
    a1 = a1 + du * w2;
    a2 = a2 + dvv * w1;
    a3 = a3 + dvv * w2;
    a4 = a4 + dth * w1;
    a5 = a5 + dth * w2;
  }
  const double K11 = d.kgcm[0][i], K21 = d.kgcm[1][i], K12 = d.kgcm[2][i], K22 = d.kgcm[3][i];
  d.grad[0][i] = K11 * a0 + K12 * a1;
  d.grad[1][i] = K21 * a0 + K22 * a1;
  d.grad[2][i] = K11 * a2 + K12 * a3;
  d.grad[3][i] = K21 * a2 + K22 * a3;
  d.grad[4][i] = K11 * a4 + K12 * a5;
  d.grad[5][i] = K21 * a4 + K22 * a5;
}

// ---------------------------------------------------------------------- log-conformation
struct M2 { double a11, a12, a21, a22; };
__device__ __forceinline__ M2 mm(const M2& A, const M2& B) {
  return M2{A.a11 * B.a11 + A.a12 * B.a21, A.a11 * B.a12 + A.a12 * B.a22,
            A.a21 * B.a11 + A.a22 * B.a21, A.a21 * B.a12 + A.a22 * B.a22};
}
__device__ __forceinline__ M2 tr(const M2& A) { return M2{A.a11, A.a21, A.a12, A.a22}; }

// calc_eigens (predictor_mod.F90:253-290): closed-form symmetric 2x2 eigen-decomposition
__device__ __forceinline__ void calc_eigens(const M2& A, double& L1, double& L2, M2& R) {
  double trc = A.a11 + A.a22;
  double det = A.a11 * A.a22 - A.a21 * A.a12;
  double tmp = 0.25 * trc * trc - det;
  if (tmp <= 2.220446049250313e-16) tmp = 0.0;  // epsilon(1d0)
  L1 = 0.5 * trc + sqrt(tmp);
  L2 = 0.5 * trc - sqrt(tmp);
  if (A.a21 != 0.0) {
    double r11 = L1 - A.a22, r21 = A.a21;
    double nrm = sqrt(r11 * r11 + r21 * r21);
    r11 = r11 / nrm;
    r21 = r21 / nrm;
    R = M2{r11, -r21, r21, r11};
  } else {
    L1 = A.a11;
    L2 = A.a22;
    R = M2{1.0, 0.0, 0.0, 1.0};
  }
}

__global__ void k_logconf(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const double dt = d.s->dt;
  // steps 1-2: A = f_strain_backward(tau) = (tau/1 + I)/1
  M2 A{d.tau[0][i] / 1.0 + 1.0, d.tau[2][i] / 1.0 + 0.0, d.tau[1][i] / 1.0 + 0.0, d.tau[3][i] / 1.0 + 1.0};
  A = M2{A.a11 / 1.0, A.a12 / 1.0, A.a21 / 1.0, A.a22 / 1.0};
  double L1, L2;
  M2 R;
  calc_eigens(A, L1, L2, R);
  {  // diagnostic: particles within reach of the 1/(L2 - L1 + 1e-10) pole of step 5
    const unsigned am = __activemask();
    const unsigned near = __ballot_sync(am, fabs(L2 - L1) < 1.0e-7);
    if ((threadIdx.x & 31) == __ffs(am) - 1 && near) {
      atomicAdd(&d.s->n_near_pole, __popc(near));
      atomicAdd(&d.s->n_near_pole_total, __popc(near));
    }
  }
  // step 3: Psi = R log(Lambda) R^T
  M2 D{log(L1), 0.0, 0.0, log(L2)};
  M2 Psi0 = mm(R, mm(D, tr(R)));
  // step 5: B and Omega from R^T grad(u) R
  M2 G{d.grad[0][i], d.grad[1][i], d.grad[2][i], d.grad[3][i]};
  M2 tm = mm(tr(R), mm(G, R));
  double tmp1 = (L2 * tm.a12 + L1 * tm.a21) / (L2 - L1 + 1e-10);
  tm.a12 = 0.0;
  tm.a21 = 0.0;
  M2 B = mm(R, mm(tm, tr(R)));
  M2 W{0.0, tmp1, -tmp1, 0.0};
  M2 Om = mm(R, mm(W, tr(R)));
  // step 6: Psi += dt (2B + Omega Psi - Psi Omega)
  M2 OP = mm(Om, Psi0), PO = mm(Psi0, Om);
  M2 t6{2.0 * B.a11 + OP.a11 - PO.a11, 2.0 * B.a12 + OP.a12 - PO.a12, 2.0 * B.a21 + OP.a21 - PO.a21,
        2.0 * B.a22 + OP.a22 - PO.a22};
  M2 Psi{Psi0.a11 + dt * t6.a11, Psi0.a12 + dt * t6.a12, Psi0.a21 + dt * t6.a21, Psi0.a22 + dt * t6.a22};
  // step 7: A = R exp(Lambda) R^T
  calc_eigens(Psi, L1, L2, R);
  L1 = exp(L1);
  L2 = exp(L2);
  M2 E2{L1, 0.0, 0.0, L2};
  A = mm(R, mm(E2, tr(R)));
  // step 8: analytic PTT relaxation with the previous trace
  double alpha_R = 1.0 + c.eps_ptt * (d.trace_conf[i] - 2.0);
  double e1 = exp(-(alpha_R * 1.0 * dt / c.Wi));
  double e2 = (1.0 - e1) / 1.0;
  A = M2{A.a11 * e1 + e2 * 1.0, A.a12 * e1 + e2 * 0.0, A.a21 * e1 + e2 * 0.0, A.a22 * e1 + e2 * 1.0};
  // step 9
  double trc = A.a11 + A.a22;
  d.trace_conf[i] = trc;
  d.a_out[i] = trc;
  d.tau[0][i] = 1.0 * (1.0 * A.a11 - 1.0);
  d.tau[2][i] = 1.0 * (1.0 * A.a12 - 0.0);
  d.tau[1][i] = 1.0 * (1.0 * A.a21 - 0.0);
  d.tau[3][i] = 1.0 * (1.0 * A.a22 - 1.0);
}

// ---------------------------------------------------------------------- predictor
// rhs pair loop + buoyancy; u*, theta* written to the second buffers (walls copied)
__global__ void k_predictor(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const double ui = d.ux[i], vi = d.uy[i], ti = d.th[i];
  const double K11 = d.kgcm[0][i], K21 = d.kgcm[1][i], K12 = d.kgcm[2][i], K22 = d.kgcm[3][i];
  double Ti11 = 0, Ti21 = 0, Ti12 = 0, Ti22 = 0;
  const bool ve = c.const_mod != 1;
  if (ve) { Ti11 = d.tau[0][i]; Ti21 = d.tau[1][i]; Ti12 = d.tau[2][i]; Ti22 = d.tau[3][i]; }
  const double cs = c.coeff_solvent, cp = c.coeff_polymeric, ct = c.coeff_theta;
  double s1 = 0, s2 = 0, st = 0;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    int j = d.ij_link[ELL(k, i)];
    double u1 = ui - d.ux[j], u2 = vi - d.uy[j];
    double wl = d.wL[ELL(k, i)];
    if (ve) {
      double w1 = d.wGx[ELL(k, i)], w2 = d.wGy[ELL(k, i)];
      double T11 = d.tau[0][j] - Ti11, T21 = d.tau[1][j] - Ti21;
      double T12 = d.tau[2][j] - Ti12, T22 = d.tau[3][j] - Ti22;
      double kw1 = K11 * w1 + K12 * w2, kw2 = K21 * w1 + K22 * w2;
      double tw1 = T11 * kw1 + T12 * kw2, tw2 = T21 * kw1 + T22 * kw2;
      s1 = s1 + cp * tw1 + cs * u1 * wl;
      s2 = s2 + cp * tw2 + cs * u2 * wl;
    } else {
      s1 = s1 + cs * u1 * wl;
      s2 = s2 + cs * u2 * wl;
    }
    double thij = ti - d.th[j];
    st = st + ct * thij * wl;
  }
  s2 = s2 + ti;  // buoyancy (predictor_mod.F90:111-119)
  const double dt = d.s->dt;
  if (i >= c.nbS) {
    d.ux2[i] = ui + s1 * dt;
    d.uy2[i] = vi + s2 * dt;
    d.th2[i] = ti + st * dt;
  } else {
    d.ux2[i] = ui;
    d.uy2[i] = vi;
    d.th2[i] = ti;
  }
}

__device__ __forceinline__ void pgrad_one(const Consts& c, const Dev& d, int i, double& mu, double& mv,
                                          double& mp) {
  const double pi_ = d.p[i];
  double a = 0, b = 0;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    int j = d.ij_link[ELL(k, i)];
    double temp = d.p[j] - pi_;
    a = a + temp * d.wGx[ELL(k, i)];
    b = b + temp * d.wGy[ELL(k, i)];
  }
  const double K11 = d.kgcm[0][i], K21 = d.kgcm[1][i], K12 = d.kgcm[2][i], K22 = d.kgcm[3][i];
  double gx = K11 * a + K12 * b, gy = K21 * a + K22 * b;
  d.gpx[i] = gx;
  d.gpy[i] = gy;
  const double dt = d.s->dt;
  double ux = d.ux2[i], uy = d.uy2[i], x = d.rx[i], y = d.ry[i];
  if (i >= c.nbS) {
    ux = ux + dt * (c.bf[0] - gx);
    uy = uy + dt * (c.bf[1] - gy);
    if (cnt <= 3) {
      ux = d.u0x[i] + dt * c.bf[0];
      uy = d.u0y[i] + dt * c.bf[1];
    }
    if (!c.correct_velocity) {  // else k_advect_final moves the particles after the correction
      x = d.r0x[i] + 0.5 * (ux + d.u0x[i]) * dt + d.ushx[i] * dt;
      y = d.r0y[i] + 0.5 * (uy + d.u0y[i]) * dt + d.ushy[i] * dt;
    }
  }
  d.ux[i] = ux;
  d.uy[i] = uy;
  d.rx[i] = x;
  d.ry[i] = y;
  mu = fabs(ux);
  mv = fabs(uy);
  mp = fabs(pi_);
}

// ---------------------------------------------------------------------- pressure gradient
// grad P, velocity update (div_free.F90:96-101), final advection (:111-117): reads u* (ux2)
// and writes u^{n+1} and r^{n+1} in place (no kernel of this launch reads neighbours' u or r).
__global__ void k_pgrad_final(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double mu = -1.0, mv = -1.0, mp = -1.0;
  if (i < c.npfb) pgrad_one(c, d, i, mu, mv, mp);
  // divergence guard (opt-in) on the new velocity (false for NaN too)
  if (c.u_limit > 0.0 && i < c.npfb && !(mu <= c.u_limit && mv <= c.u_limit)) set_error(d.s, VEBI_ERR_DIVERGED);
  warp_max_pos(&d.s->absu_bits, mu);
  warp_max_pos(&d.s->absv_bits, mv);
  warp_max_pos(&d.s->absp_bits, mp);
}


// correct_velocity (correct_velocity.F90:13-70), behind a switch: the reference has the call
// commented out (div_free.F90:105).  Particles closer than dx to a wall (or wall-wall corner)
// mirror lose the velocity component towards it.  A circle mirror (vrelation = 999+ib) is not
// treated as a wall: the reference indexes b_type out of range there.
__global__ void k_correct_velocity(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < c.nbS || i >= c.npfb) return;
  const double xi = d.rx[i], yi = d.ry[i];
  double r_min2 = c.dx * c.dx;
  int close = -1;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    int j = d.ij_link[ELL(k, i)];
    if (j < c.npfb) continue;
    double a = xi - d.rx[j], b = yi - d.ry[j];
    double d2 = a * a + b * b;
    if (!(d2 < r_min2)) continue;
    int vr = d.vrel[j];
    if (vr > 0 && vr < 999 && c.b_type[vr - 1] == 1) { r_min2 = d2; close = j; }
    if (vr == -1 || vr < -2) { r_min2 = d2; close = j; }
  }
  if (close < 0) return;
  double n1 = xi - d.rx[close], n2 = yi - d.ry[close];
  double t = sqrt(n1 * n1 + n2 * n2);
  n1 = n1 / t;
  n2 = n2 / t;
  double u1 = d.ux[i] - d.ux2[close], u2 = d.uy[i] - d.uy2[close];
  double un = u1 * n1 + u2 * n2;
  if (un <= 0.0) {
    d.ux[i] = d.ux[i] - un * n1;
    d.uy[i] = d.uy[i] - un * n2;
  }
}

// final advection after correct_velocity (div_free.F90:111-117)
__global__ void k_advect_final(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < c.nbS || i >= c.npfb) return;
  const double dt = d.s->dt;
  d.rx[i] = d.r0x[i] + 0.5 * (d.ux[i] + d.u0x[i]) * dt + d.ushx[i] * dt;
  d.ry[i] = d.r0y[i] + 0.5 * (d.uy[i] + d.u0y[i]) * dt + d.ushy[i] * dt;
}

// secondary_properties: vorticity from final fluid u and mirror u* (div_free.F90:160-183)
template <typename W>
__global__ void k_secondary(Consts c, Dev d, const double* __restrict__ uxn, const double* __restrict__ uyn,
                            const double* __restrict__ uxm, const double* __restrict__ uym,
                            const W* __restrict__ wgx, const W* __restrict__ wgy) {
  __shared__ double sh[TPB / 32 + 1];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0;
  if (i < c.npfb) {
    const double ui = uxn[i], vi = uyn[i];
    double vt = 0.0;
    const int cnt = d.ij_count[i];
    for (int k = 0; k < cnt; ++k) {
      int j = d.ij_link[ELL(k, i)];
      double uj = j < c.npfb ? uxn[j] : uxm[j], vj = j < c.npfb ? uyn[j] : uym[j];
      double tmp = (vi - vj) * (double)wgx[ELL(k, i)] - (ui - uj) * (double)wgy[ELL(k, i)];
      vt = vt - tmp;
    }
    d.vort[i] = vt;
    e = ui * ui + vi * vi;
  }
  double bs = block_sum<TPB>(e, sh);
  if (threadIdx.x == 0) d.partials[blockIdx.x] = bs;
}

__global__ void k_secondary_final(Consts c, Dev d, int nblk) {
  __shared__ double sh[TPB / 32 + 1];
  double s = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += d.partials[b];
  s = block_sum<TPB>(s, sh);
  if (threadIdx.x == 0) d.s->rms_u = sqrt(s / (double)c.npfb);
}

// Force of the fluid on the circles (the cylinder's drag and lift), as the step's own pair
// terms see it: for every fluid particle, the circle mirrors' (vrelation > 999) share of the
// viscous and polymeric sums of prediction_step (predictor_mod.F90:27-139) and of the pressure
// gradient of calc_pressure_gradient (gradient_calculation.F90:16-48), times dv; the circles
// feel the opposite.  Evaluated after the step from the values those stages read: the
// start-of-step fluid velocity u0, the mirrors' creation-time velocity (ux/uy at npfb..), the
// updated tau and the new pressure.  A diagnostic of this library; the reference has none.
// A circle mirror lies at radius 2R - rad of a source at rad (inside the support band), so a
// particle that has one as a neighbour (distance <= sup) is within sup of the circle: the
// mirror stages' candidate list (every particle within sup plus a margin of a boundary, in
// ascending index) holds all of them, and the kernel walks that list alone.
constexpr int CF_BLOCKS = 256;

template <class W>
__global__ void k_circle_force(Consts c, Dev d, const W* __restrict__ wgx, const W* __restrict__ wgy,
                               const W* __restrict__ wl_, const W* __restrict__ k11, const W* __restrict__ k21,
                               const W* __restrict__ k12, const W* __restrict__ k22) {
  __shared__ double sh[TPB / 32 + 1];
  const int ncand = d.s->n_cand;
  double fx = 0.0, fy = 0.0;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < ncand; q += gridDim.x * blockDim.x) {
    const int i = d.cand[q];
    if (i < c.nbS || i >= c.npfb || d.inbin[i]) continue;
    const bool ve = c.const_mod != 1;
    const double ui = d.u0x[i], vi = d.u0y[i], pi_ = d.p[i];
    const double K11 = (double)k11[i], K21 = (double)k21[i], K12 = (double)k12[i], K22 = (double)k22[i];
    double Ti11 = 0, Ti21 = 0, Ti12 = 0, Ti22 = 0;
    if (ve) { Ti11 = d.tau[0][i]; Ti21 = d.tau[1][i]; Ti12 = d.tau[2][i]; Ti22 = d.tau[3][i]; }
    const double cs = c.coeff_solvent, cp = c.coeff_polymeric;
    double s1 = 0, s2 = 0, a = 0, b = 0;
    const int cnt = d.ij_count[i];
    for (int k = 0; k < cnt; ++k) {
      int j = d.ij_link[ELL(k, i)];
      if (j < c.npfb || d.vrel[j] <= 999) continue;
      double w1 = (double)wgx[ELL(k, i)], w2 = (double)wgy[ELL(k, i)], wl = (double)wl_[ELL(k, i)];
      double u1 = ui - d.ux[j], u2 = vi - d.uy[j];
      if (ve) {
        double T11 = d.tau[0][j] - Ti11, T21 = d.tau[1][j] - Ti21;
        double T12 = d.tau[2][j] - Ti12, T22 = d.tau[3][j] - Ti22;
        double kw1 = K11 * w1 + K12 * w2, kw2 = K21 * w1 + K22 * w2;
        s1 = s1 + cp * (T11 * kw1 + T12 * kw2) + cs * u1 * wl;
        s2 = s2 + cp * (T21 * kw1 + T22 * kw2) + cs * u2 * wl;
      } else {
        s1 = s1 + cs * u1 * wl;
        s2 = s2 + cs * u2 * wl;
      }
      double temp = d.p[j] - pi_;
      a = a + temp * w1;
      b = b + temp * w2;
    }
    const double gx = K11 * a + K12 * b, gy = K21 * a + K22 * b;
    fx += c.dv * (gx - s1);
    fy += c.dv * (gy - s2);
  }
  double bx = block_sum<TPB>(fx, sh);
  double by = block_sum<TPB>(fy, sh);
  if (threadIdx.x == 0) {
    d.partials[blockIdx.x] = bx;
    d.partials[gridDim.x + blockIdx.x] = by;
  }
}

__global__ void k_circle_force_final(Dev d, int nblk) {
  __shared__ double sh[TPB / 32 + 1];
  double sx = 0.0, sy = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    sx += d.partials[b];
    sy += d.partials[nblk + b];
  }
  sx = block_sum<TPB>(sx, sh);
  sy = block_sum<TPB>(sy, sh);
  if (threadIdx.x == 0) {
    d.s->circle_fx = sx;
    d.s->circle_fy = sy;
  }
}

void launch_prep_weights32(Ctx& x);
void launch_shift32(Ctx& x);
void launch_gradients32(Ctx& x);
void launch_predictor32(Ctx& x);
void launch_pgrad_final32(Ctx& x);

void launch_weights_surface_shift(Ctx& x) {
  const Consts& c = x.c;
  int g = grid_for(c.npfb);
  const bool mixed = x.precision == VEBI_PREC_MIXED;
  if (mixed) launch_prep_weights32(x);
  // FP64 weights: the FP64 step, and the free-surface operators of an open domain
  if (!mixed || c.open_domain == 1) VEBI_LAUNCH(x, k_weights, g, TPB, c, x.d);
  if (c.open_domain == 1) {
    VEBI_LAUNCH(x, k_part_dist_vars, g, TPB, c, x.d);
    VEBI_LAUNCH(x, k_nsurf_mirrors, x.gs_blocks, TPB, c, x.d);
    VEBI_LAUNCH(x, k_smooth_normals, g, TPB, c, x.d);
    VEBI_LAUNCH(x, k_copy_normals, g, TPB, c, x.d);
  } else {
    cudaMemsetAsync(x.d.n_surf, 0, sizeof(int) * (size_t)c.cap, x.st);
  }
  stage_mark(x, 5);
  if (mixed && c.open_domain == 0) launch_shift32(x);
  else VEBI_LAUNCH(x, k_shift, g, TPB, c, x.d);
}

void launch_grad_mirrors(Ctx& x);
void launch_mirror_stress(Ctx& x);
void launch_mirror_velocities(Ctx& x);
void launch_mirror_pressure(Ctx& x);

void launch_predictor(Ctx& x) {
  const Consts& c = x.c;
  int g = grid_for(c.npfb);
  const bool mixed = x.precision == VEBI_PREC_MIXED;
  stage_mark(x, 6);
  if (mixed) launch_gradients32(x);
  else VEBI_LAUNCH(x, k_gradients, g, TPB, c, x.d);
  launch_grad_mirrors(x);
  stage_mark(x, 7);
  if (c.const_mod != 1) {
    VEBI_LAUNCH(x, k_logconf, g, TPB, c, x.d);
    launch_mirror_stress(x);
  }
  stage_mark(x, 8);
  if (mixed) launch_predictor32(x);
  else VEBI_LAUNCH(x, k_predictor, g, TPB, c, x.d);
  launch_mirror_velocities(x);
  // theta* replaces theta for walls and fluid; u* stays in ux2/uy2 for the PPE and the update
  cudaMemcpyAsync(x.d.th, x.d.th2, sizeof(double) * (size_t)c.npfb, cudaMemcpyDeviceToDevice, x.st);
}

void launch_final(Ctx& x, int secondary) {
  const Consts& c = x.c;
  int g = grid_for(c.npfb);
  stage_mark(x, 11);
  launch_mirror_pressure(x);
  // keep r* (fluid and mirrors) readable after the step: the update below overwrites r
  cudaMemcpyAsync(x.d.rx2, x.d.rx, sizeof(double) * (size_t)c.cap, cudaMemcpyDeviceToDevice, x.st);
  cudaMemcpyAsync(x.d.ry2, x.d.ry, sizeof(double) * (size_t)c.cap, cudaMemcpyDeviceToDevice, x.st);
  const bool mixed = x.precision == VEBI_PREC_MIXED;
  if (mixed) launch_pgrad_final32(x);
  else VEBI_LAUNCH(x, k_pgrad_final, g, TPB, c, x.d);
  if (c.correct_velocity) {
    VEBI_LAUNCH(x, k_correct_velocity, g, TPB, c, x.d);
    VEBI_LAUNCH(x, k_advect_final, g, TPB, c, x.d);
  }
  if (c.ncirc > 0) {
    if (mixed)
      VEBI_LAUNCH(x, k_circle_force<float>, CF_BLOCKS, TPB, c, x.d, x.d.wGx32, x.d.wGy32, x.d.wL32, x.d.kgcm32[0],
                  x.d.kgcm32[1], x.d.kgcm32[2], x.d.kgcm32[3]);
    else
      VEBI_LAUNCH(x, k_circle_force<double>, CF_BLOCKS, TPB, c, x.d, x.d.wGx, x.d.wGy, x.d.wL, x.d.kgcm[0], x.d.kgcm[1],
                  x.d.kgcm[2], x.d.kgcm[3]);
    VEBI_LAUNCH(x, k_circle_force_final, 1, TPB, x.d, CF_BLOCKS);
  }
  if (secondary) {
    stage_mark(x, 13);
    if (mixed) VEBI_LAUNCH(x, k_secondary<float>, g, TPB, c, x.d, x.d.ux, x.d.uy, x.d.ux2, x.d.uy2, x.d.wGx32, x.d.wGy32);
    else VEBI_LAUNCH(x, k_secondary<double>, g, TPB, c, x.d, x.d.ux, x.d.uy, x.d.ux2, x.d.uy2, x.d.wGx, x.d.wGy);
    VEBI_LAUNCH(x, k_secondary_final, 1, TPB, c, x.d, g);
  }
}

}  // namespace vebi
