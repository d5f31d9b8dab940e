// vebi_sph32.cu -- the SPH pair operators of the mixed-precision step (VEBI_PREC_MIXED).
//
// Same operators and loop orders as vebi_sph.cu, with the pair sums in FP32 and FP32
// accumulation.  Two rules keep FP32 from losing the signal to cancellation:
//  * pair offsets r_i - r_j come from FP32 offsets to each particle's cell origin plus the
//    (small integer) cell difference times the cell size, so no large coordinate is ever
//    subtracted in FP32;
//  * neighbour differences of a field (u_i - u_j, tau_j - tau_i, theta_i - theta_j,
//    P_j - P_i) are taken in FP64 and rounded once, then multiplied in FP32.
// The updates of u, theta and the positions stay FP64, and so do the log-conformation
// eigen-step (k_logconf) and the PPE refinement.  The PPE matrix is assembled in FP64 from the
// FP32 Morris weights, so the FP32 solver's matrix and the FP64 residual's matrix agree.
#include <initializer_list>

#include "vebi_ctx.cuh"

namespace vebi {

#define ELL(k, i) ((size_t)(k) * c.npfb + (i))

__device__ __forceinline__ float pw4f(float x) { float x2 = x * x; return x2 * x2; }
__device__ __forceinline__ float pw5f(float x) { float x2 = x * x; return x2 * (x * x2); }

__device__ __forceinline__ float fac32(const Consts& c, float qq) {
  const float a = (float)c.ad_7h;
  if (qq < 1.0f) {
    float q3 = 3.0f - qq, q2 = 2.0f - qq, q1 = 1.0f - qq;
    return a * (-5.0f * pw4f(q3) + 30.0f * pw4f(q2) - 75.0f * pw4f(q1));
  } else if (qq < 2.0f) {
    float q3 = 3.0f - qq, q2 = 2.0f - qq;
    return a * (-5.0f * pw4f(q3) + 30.0f * pw4f(q2));
  } else if (qq < 3.0f) {
    return a * (-5.0f * pw4f(3.0f - qq));
  }
  return 0.0f;
}

__device__ __forceinline__ float wab32(const Consts& c, float qq) {
  const float a = (float)c.ad_7;
  if (qq < 1.0f) {
    float q3 = 3.0f - qq, q2 = 2.0f - qq, q1 = 1.0f - qq;
    return a * (pw5f(q3) - 6.0f * pw5f(q2) + 15.0f * pw5f(q1));
  } else if (qq < 2.0f) {
    float q3 = 3.0f - qq, q2 = 2.0f - qq;
    return a * (pw5f(q3) - 6.0f * pw5f(q2));
  } else if (qq < 3.0f) {
    return a * pw5f(3.0f - qq);
  }
  return 0.0f;
}

__device__ __forceinline__ void pair_offset(const Consts& c, const float4& a, const float4& b, float& r1,
                                            float& r2) {
  const float S = (float)c.cell_size;
  r1 = (a.x - b.x) + (a.z - b.z) * S;
  r2 = (a.y - b.y) + (a.w - b.w) * S;
}

// kernel_calculation in FP32 (kernel_calculation.F90:22-71)
__global__ void k_weights32(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const float4 pi = d.pk[i];
  const float dv = (float)c.dv, oneoverh = (float)c.oneoverh, eta2 = (float)c.eta2, etas = (float)c.eta_small;
  float k11 = 0.f, k12 = 0.f, k21 = 0.f, k22 = 0.f;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    int j = d.ij_link[ELL(k, i)];
    float r1, r2;
    pair_offset(c, pi, d.pk[j], r1, r2);
    float rr2 = fmaf(r1, r1, r2 * r2);
    float rad = sqrtf(rr2);
    float f = fac32(c, rad * oneoverh);
    float inv = f / fmaxf(rad, eta2);
    float g1 = r1 * inv, g2 = r2 * inv;
    float w1 = g1 * dv, w2 = g2 * dv;
    d.wGx32[ELL(k, i)] = w1;
    d.wGy32[ELL(k, i)] = w2;
    d.wL32[ELL(k, i)] = 2.0f * fmaf(r1, w1, r2 * w2) / (rr2 + etas);
    k11 = fmaf(-dv * g1, r1, k11);
    k12 = fmaf(-dv * g2, r1, k12);
    k21 = fmaf(-dv * g1, r2, k21);
    k22 = fmaf(-dv * g2, r2, k22);
  }
  float temp = 1.0f / ((k11 * k22 - k12 * k21) + 1.0e-15f);
  d.kgcm32[0][i] = temp * k22;
  d.kgcm32[2][i] = -temp * k12;
  d.kgcm32[1][i] = -temp * k21;
  d.kgcm32[3][i] = temp * k11;
}

// new_fick_shift + shifting_forces in FP32 (new_fick_shift.F90:15-92,117-210), closed domain
__global__ void k_shift32(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const float4 pi = d.pk[i];
  const float oneoverh = (float)c.oneoverh, iw1 = (float)(1.0 / c.wab1);
  float f1 = 0.f, f2 = 0.f, t1 = 0.f, t2 = 0.f;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    int j = d.ij_link[ELL(k, i)];
    float r1, r2;
    pair_offset(c, pi, d.pk[j], r1, r2);
    float rad = sqrtf(fmaf(r1, r1, r2 * r2));
    float fab = 0.25f * pw4f(wab32(c, rad * oneoverh) * iw1);
    float w1 = d.wGx32[ELL(k, i)], w2 = d.wGy32[ELL(k, i)];
    f1 += w1;
    f2 += w2;
    t1 = fmaf(w1, fab, t1);
    t2 = fmaf(w2, fab, t2);
  }
  float gx = f1 + t1, gy = f2 + t2;
  d.gradCx[i] = gx;
  d.gradCy[i] = gy;
  const double dt = d.s->dt;
  if (i < c.nbS) {
    d.ushx[i] = -d.ux[i];
    d.ushy[i] = -d.uy[i];
    return;
  }
  float D;
  if (c.shift_coeff == 1) {
    double maxU = bits_to_double(d.s->maxU_bits);
    double absU = sqrt(d.ux[i] * d.ux[i] + d.uy[i] * d.uy[i]);
    double temp = (double)0.2f * exp(-absU / ((double)0.2f * maxU));
    D = (float)(4.0 * c.h * dt * (absU + temp * maxU));
  } else {
    D = (float)(0.25 * c.h * c.h);
  }
  float d1 = -D * gx, d2 = -D * gy;
  float temp = sqrtf(fmaf(d1, d1, d2 * d2));
  const float lim = (float)(0.1 * c.h);
  if (temp > lim) {
    d1 = lim * d1 / temp;
    d2 = lim * d2 / temp;
  }
  d.ushx[i] = (double)d1 / dt;
  d.ushy[i] = (double)d2 / dt;
}

// grad_operator for u, v, theta in FP32 (gradient_calculation.F90:50-94)
// FP64 fields of all np particles (fluid, walls, mirrors) as FP32 (hi, lo) pairs
struct SplitArgs {
  const double* src[4];
  float2* dst[4];
  int nf;
};

__global__ void k_split_fields(Dev d, SplitArgs a) {
  const int np = d.s->np;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x)
    for (int f = 0; f < a.nf; ++f) {
      const double v = a.src[f][i];
      const float h = narrow(v);  // (float)v, (float)(v - (double)h) on the integer pipe
      a.dst[f][i] = make_float2(h, narrow(v - widen(h)));
    }
}

// f_j - f_i of two split values, in FP32
__device__ __forceinline__ float dhl(float2 fj, float2 fi) { return (fj.x - fi.x) + (fj.y - fi.y); }

__global__ void k_gradients32(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const float2 ui = d.hl_u[0][i], vi = d.hl_u[1][i], ti = d.hl_th[i];
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f, a4 = 0.f, a5 = 0.f;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    int j = d.ij_link[ELL(k, i)];
    float w1 = d.wGx32[ELL(k, i)], w2 = d.wGy32[ELL(k, i)];
    float du = dhl(d.hl_u[0][j], ui), dvv = dhl(d.hl_u[1][j], vi), dth = dhl(d.hl_th[j], ti);
    a0 = fmaf(du, w1, a0);
    a1 = fmaf(du, w2, a1);
    a2 = fmaf(dvv, w1, a2);
    a3 = fmaf(dvv, w2, a3);
    a4 = fmaf(dth, w1, a4);
    a5 = fmaf(dth, w2, a5);
  }
  const float K11 = d.kgcm32[0][i], K21 = d.kgcm32[1][i], K12 = d.kgcm32[2][i], K22 = d.kgcm32[3][i];
  d.grad[0][i] = (double)fmaf(K11, a0, K12 * a1);
  d.grad[1][i] = (double)fmaf(K21, a0, K22 * a1);
  d.grad[2][i] = (double)fmaf(K11, a2, K12 * a3);
  d.grad[3][i] = (double)fmaf(K21, a2, K22 * a3);
  d.grad[4][i] = (double)fmaf(K11, a4, K12 * a5);
  d.grad[5][i] = (double)fmaf(K21, a4, K22 * a5);
}

// prediction_step pair loop in FP32 (predictor_mod.F90:79-133); u*, theta* updated in FP64
__global__ void k_predictor32(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const double ui = d.ux[i], vi = d.uy[i], ti = d.th[i];
  const float2 hu = d.hl_u[0][i], hv = d.hl_u[1][i], ht = d.hl_th[i];
  const float K11 = d.kgcm32[0][i], K21 = d.kgcm32[1][i], K12 = d.kgcm32[2][i], K22 = d.kgcm32[3][i];
  const bool ve = c.const_mod != 1;
  float2 Ti11 = make_float2(0.f, 0.f), Ti21 = Ti11, Ti12 = Ti11, Ti22 = Ti11;
  if (ve) { Ti11 = d.hl_tau[0][i]; Ti21 = d.hl_tau[1][i]; Ti12 = d.hl_tau[2][i]; Ti22 = d.hl_tau[3][i]; }
  const float cs = (float)c.coeff_solvent, cp = (float)c.coeff_polymeric, ct = (float)c.coeff_theta;
  float s1 = 0.f, s2 = 0.f, st = 0.f;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    int j = d.ij_link[ELL(k, i)];
    float u1 = dhl(hu, d.hl_u[0][j]), u2 = dhl(hv, d.hl_u[1][j]);
    float wl = d.wL32[ELL(k, i)];
    if (ve) {
      float w1 = d.wGx32[ELL(k, i)], w2 = d.wGy32[ELL(k, i)];
      float T11 = dhl(d.hl_tau[0][j], Ti11), T21 = dhl(d.hl_tau[1][j], Ti21);
      float T12 = dhl(d.hl_tau[2][j], Ti12), T22 = dhl(d.hl_tau[3][j], Ti22);
      float kw1 = fmaf(K11, w1, K12 * w2), kw2 = fmaf(K21, w1, K22 * w2);
      float tw1 = fmaf(T11, kw1, T12 * kw2), tw2 = fmaf(T21, kw1, T22 * kw2);
      s1 = fmaf(cp, tw1, fmaf(cs * u1, wl, s1));
      s2 = fmaf(cp, tw2, fmaf(cs * u2, wl, s2));
    } else {
      s1 = fmaf(cs * u1, wl, s1);
      s2 = fmaf(cs * u2, wl, s2);
    }
    float thij = dhl(ht, d.hl_th[j]);
    st = fmaf(ct * thij, wl, st);
  }
  const double dt = d.s->dt;
  const double r2 = (double)s2 + ti;  // buoyancy (predictor_mod.F90:111-119)
  if (i >= c.nbS) {
    d.ux2[i] = ui + (double)s1 * dt;
    d.uy2[i] = vi + r2 * dt;
    d.th2[i] = ti + (double)st * dt;
  } else {
    d.ux2[i] = ui;
    d.uy2[i] = vi;
    d.th2[i] = ti;
  }
}

// PPE right-hand side in FP32 sums (ppe_solve_in_house_simple_dirichlet.F90:27-43)
__global__ void k_ppe_rhs32(Consts c, Dev d) {
  __shared__ double sh[TPB / 32 + 1];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double b = 0.0;
  if (i < c.npfb) {
    const float2 ui = d.hl_us[0][i], vi = d.hl_us[1][i];
    const float K11 = d.kgcm32[0][i], K21 = d.kgcm32[1][i], K12 = d.kgcm32[2][i], K22 = d.kgcm32[3][i];
    float fb = 0.f;
    const int cnt = d.ij_count[i];
    for (int k = 0; k < cnt; ++k) {
      int j = d.ij_link[ELL(k, i)];
      float u1 = dhl(ui, d.hl_us[0][j]), u2 = dhl(vi, d.hl_us[1][j]);
      float w1 = d.wGx32[ELL(k, i)], w2 = d.wGy32[ELL(k, i)];
      float kw1 = fmaf(K11, w1, K12 * w2), kw2 = fmaf(K21, w1, K22 * w2);
      fb = fb - fmaf(u1, kw1, u2 * kw2);
    }
    b = (double)fb / d.s->dt;
    d.ppe_B[i] = b;
  }
  double bs = block_sum<TPB>(b, sh);
  if (threadIdx.x == 0) d.partials[blockIdx.x] = bs;
}

// calc_pressure_gradient in FP32 sums + FP64 velocity update and advection
__global__ void k_pgrad_final32(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double mu = -1.0, mv = -1.0, mp = -1.0;
  if (i < c.npfb) {
    const double pi_ = d.p[i];
    const float2 hp = d.hl_p[i];
    float a = 0.f, b = 0.f;
    const int cnt = d.ij_count[i];
    for (int k = 0; k < cnt; ++k) {
      int j = d.ij_link[ELL(k, i)];
      float temp = dhl(d.hl_p[j], hp);
      a = fmaf(temp, d.wGx32[ELL(k, i)], a);
      b = fmaf(temp, d.wGy32[ELL(k, i)], b);
    }
    const float K11 = d.kgcm32[0][i], K21 = d.kgcm32[1][i], K12 = d.kgcm32[2][i], K22 = d.kgcm32[3][i];
    double gx = (double)fmaf(K11, a, K12 * b), gy = (double)fmaf(K21, a, K22 * b);
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
      if (!c.correct_velocity) {
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
  // divergence guard (opt-in) on the new velocity (false for NaN too)
  if (c.u_limit > 0.0 && i < c.npfb && !(mu <= c.u_limit && mv <= c.u_limit)) set_error(d.s, VEBI_ERR_DIVERGED);
  warp_max_pos(&d.s->absu_bits, mu);
  warp_max_pos(&d.s->absv_bits, mv);
  warp_max_pos(&d.s->absp_bits, mp);
}

// the cell-relative offsets d.pk are written by the neighbour search (vebi_cells.cu)
void launch_prep_weights32(Ctx& x) { VEBI_LAUNCH(x, k_weights32, grid_for(x.c.npfb), TPB, x.c, x.d); }
void launch_shift32(Ctx& x) { VEBI_LAUNCH(x, k_shift32, grid_for(x.c.npfb), TPB, x.c, x.d); }
static void split(Ctx& x, std::initializer_list<const double*> src, std::initializer_list<float2*> dst) {
  SplitArgs a{};
  int f = 0;
  for (const double* p : src) a.src[f++] = p;
  a.nf = f;
  f = 0;
  for (float2* p : dst) a.dst[f++] = p;
  VEBI_LAUNCH(x, k_split_fields, x.gs_blocks, TPB, x.d, a);
}

void launch_gradients32(Ctx& x) {
  split(x, {x.d.ux, x.d.uy, x.d.th}, {x.d.hl_u[0], x.d.hl_u[1], x.d.hl_th});  // also read by the predictor
  VEBI_LAUNCH(x, k_gradients32, grid_for(x.c.npfb), TPB, x.c, x.d);
}
void launch_predictor32(Ctx& x) {
  if (x.c.const_mod != 1)  // tau after the log-conformation update and the mirror stresses
    split(x, {x.d.tau[0], x.d.tau[1], x.d.tau[2], x.d.tau[3]}, {x.d.hl_tau[0], x.d.hl_tau[1], x.d.hl_tau[2], x.d.hl_tau[3]});
  VEBI_LAUNCH(x, k_predictor32, grid_for(x.c.npfb), TPB, x.c, x.d);
}
void launch_ppe_rhs32(Ctx& x) {
  split(x, {x.d.ux2, x.d.uy2}, {x.d.hl_us[0], x.d.hl_us[1]});  // u* with the mirrors' u*
  VEBI_LAUNCH(x, k_ppe_rhs32, grid_for(x.c.npfb), TPB, x.c, x.d);
}
void launch_pgrad_final32(Ctx& x) {
  split(x, {x.d.p}, {x.d.hl_p});  // P with the mirrors' P
  VEBI_LAUNCH(x, k_pgrad_final32, grid_for(x.c.npfb), TPB, x.c, x.d);
}

}  // namespace vebi
