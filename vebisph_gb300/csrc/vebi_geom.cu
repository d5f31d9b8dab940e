// vebi_geom.cu -- time step bound, advection, bin, escapees and mirror particles.
//
//  set_time_step        div_free.F90:126-146
//  advection r*=r+dt u  div_free.F90:47-53
//  put_in_bin           put_in_bin.F90:1-56
//  replace_escapees     mirror_boundaries_mod.F90:336-407
//  create_mirror_particles (+create_boundary_boxes)  mirror_boundaries_mod.F90:18-334,409-445
//  mirror_velocities    mirror_boundaries_mod.F90:509-584
//  mirror_polymeric_stress                 mirror_boundaries_mod.F90:586-653
//  grad_operator mirror transfer           gradient_calculation.F90:96-145
//
// The reference builds mirrors serially with one global counter `imp`, patch after patch,
// then corner after corner; wall-periodic corners scan the mirrors made so far.  Here every
// such stage is an order-preserving stream compaction (count / scan / emit) over the
// candidate particles, so mirror k here is mirror k of the reference.
#include "vebi_ctx.cuh"

namespace vebi {

// ------------------------------------------------------------------------------- step start
__global__ void k_step_reset(Scal* s, int npfb, int nbS) {
  // a failed step (device status, or every liquid particle binned) stays recorded; later
  // steps of this state skip the PPE solve
  if (!s->first_error) {
    if (s->error) s->first_error = s->error;
    else if (npfb > nbS && s->n_inbin == npfb - nbS) s->first_error = VEBI_ERR_ALL_IN_BIN;
  }
  s->umax_bits = (unsigned long long)__double_as_longlong(1.0e-10);
  s->maxU_bits = (unsigned long long)__double_as_longlong(1.0e-10);
  s->absu_bits = s->absv_bits = s->absp_bits = 0ull;
  s->nmirror = 0;
  s->np = npfb;
  s->n_inbin = 0;
  s->n_escapees = 0;
  s->maxneigh = 0;
  s->ls_iters = 0;
  s->warnings = 0;
  s->error = 0;
  s->rhs_mean = 0.0;
  s->ls_residual = 0.0;
  s->rms_u = 0.0;
  s->bar_count = 0;
  s->refine_iters = 0;
  s->mg_fail = 0;
  s->n_near_pole = 0;
}

// STEP 1-2: keep r0,u0 and reduce max|u| over the fluid (set_time_step)
__global__ void k_save_umax(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double um = -1.0;
  if (i < c.npfb) {
    double ux = d.ux[i], uy = d.uy[i];
    d.r0x[i] = d.rx[i];
    d.r0y[i] = d.ry[i];
    d.u0x[i] = ux;
    d.u0y[i] = uy;
    if (i >= c.nbS) {
      um = sqrt(ux * ux + uy * uy);
      // divergence guard (opt-in): a non-finite or runaway velocity fails the step
      if (c.u_limit > 0.0 && !(um <= c.u_limit)) set_error(d.s, VEBI_ERR_DIVERGED);
    }
  }
  warp_max_pos(&d.s->umax_bits, um);
}

__device__ __forceinline__ double step_dt(const Consts& c, const Scal* s) {
  double umax = bits_to_double(s->umax_bits);
  double dt_cfl = c.dt_coef_cfl * c.h / umax;
  return fmin(dt_cfl, c.dt_visc);
}

// STEP 3-4: advect, bin, replace escapees; per particle, in the reference's order
__device__ __forceinline__ double advect_bin_one(const Consts& c, const Dev& d, int i, double dt);

__global__ void k_advect_bin(Consts c, Dev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  Scal* s = d.s;
  const double dt = step_dt(c, s);
  if (i == 0) s->dt = dt;
  double um = -1.0;
  if (i < c.nbS) {  // walls do not move; they still enter the maximum of new_fick_shift
    um = sqrt(d.ux[i] * d.ux[i] + d.uy[i] * d.uy[i]);
  } else if (i < c.npfb) {
    um = advect_bin_one(c, d, i, dt);
  }
  warp_max_pos(&s->maxU_bits, um);
}

// one fluid particle: advection, put_in_bin, replace_escapees; returns |u| after binning
__device__ __forceinline__ double advect_bin_one(const Consts& c, const Dev& d, int i, double dt) {
  Scal* s = d.s;
  double x = d.r0x[i] + d.u0x[i] * dt;
  double y = d.r0y[i] + d.u0y[i] * dt;
  double ux = d.ux[i], uy = d.uy[i];
  // put_in_bin
  bool ib = d.inbin[i] != 0;
  if (!ib) {
    if (x < c.x_mint || x > c.x_maxt || y < c.y_mint || y > c.y_maxt) ib = true;
    if (isnan(x) || isnan(y)) ib = true;
  }
  if (ib) {
    x = 2.0 * c.x_mint - c.x_maxt;
    y = 2.0 * c.y_mint - c.y_maxt;
    ux = 0.0;
    uy = 0.0;
    atomicAdd(&s->n_inbin, 1);
    d.inbin[i] = 1;
    d.ux[i] = 0.0;
    d.uy[i] = 0.0;
  }
  // replace_escapees: circles (no bin test in the reference), then walls / periodic patches
  int nesc = 0;
  bool touched = false;
  // FP32 prefilters (margin near_band): a particle clearly away from a circle or a patch skips
  // the FP64 tests, which would find nothing to do for it
  const float band = c.near_band;
  for (int ic = 0; ic < c.ncirc; ++ic) {
    double R = c.c_radius[ic];
    {  // from the current position: an earlier circle may have moved the particle
      const float d1 = (float)x - (float)c.c_centre[ic][0], d2 = (float)y - (float)c.c_centre[ic][1];
      const float q = fmaf(d1, d1, d2 * d2), Rf = (float)fabs(R);
      if (R > 0.0 && q > (Rf + band) * (Rf + band)) continue;              // clearly outside
      if (R < 0.0 && Rf > band && q < (Rf - band) * (Rf - band)) continue;  // clearly inside
    }
    double ric1 = x - c.c_centre[ic][0], ric2 = y - c.c_centre[ic][1];
    double rad = sqrt(ric1 * ric1 + ric2 * ric2);
    if (rad < fabs(R) && R > 0.0) {
      x = x + (ric1 / rad) * 2.0 * (R - rad);
      y = y + (ric2 / rad) * 2.0 * (R - rad);
      ++nesc;
    }
    if (rad > fabs(R) && R < 0.0) {
      x = x - (ric1 / rad) * 2.0 * (rad + R);
      y = y - (ric2 / rad) * 2.0 * (rad + R);
      ++nesc;
    }
  }
  double r0x = 0.0, r0y = 0.0;
  for (int p = 0; p < c.nb; ++p) {
    if (c.b_type[p] != 1 && c.b_type[p] != 2) continue;
    if (ib) continue;
    {
      const float pf = fmaf(c.bl_a[p], (float)x, fmaf(c.bl_b[p], (float)y, c.bl_c[p]));
      if (pf > band || pf < -band) continue;  // clearly inside, or clearly beyond the support
    }
    double perp = bound_dist(c, x, y, p);
    if (perp > 0.0) continue;
    if (fabs(perp) > c.sup_size + 1.0e-10) continue;
    double n1, n2;
    bound_norm(c, p, n1, n2);
    double tmp = pos_along(c, x, y, p, perp, n1, n2);
    if (c.b_type[p] == 1) {
      if (tmp < 0.0 || tmp > 1.0) continue;
      x = x - 2.0 * perp * n1;
      y = y - 2.0 * perp * n2;
    } else {
      int pp = c.b_pp[p];
      double pn1, pn2;
      bound_norm(c, pp, pn1, pn2);
      double t1 = -1.0 * tmp * c.b_edge[pp][0] - perp * pn1;
      double t2 = -1.0 * tmp * c.b_edge[pp][1] - perp * pn2;
      x = c.b_node[pp][0] + c.b_edge[pp][0] + t1;
      y = c.b_node[pp][1] + c.b_edge[pp][1] + t2;
    }
    ++nesc;
    r0x = x - ux * dt;
    r0y = y - uy * dt;
    touched = true;
  }
  if (touched) {
    d.r0x[i] = r0x;
    d.r0y[i] = r0y;
    d.u0x[i] = ux;
    d.u0y[i] = uy;
  }
  if (nesc) atomicAdd(&s->n_escapees, nesc);
  d.rx[i] = x;
  d.ry[i] = y;
  return sqrt(ux * ux + uy * uy);
}

// ------------------------------------------------------------------------------- mirrors
enum SelKind { SEL_CIRCLES = 0, SEL_WALL, SEL_PERIODIC, SEL_CORNER_WW, SEL_CORNER_PP, SEL_CORNER_WP };

struct SelArgs {
  int kind;
  int ib;      // patch (0-based)
  int n0;      // first item
  int n1;      // end item (static kinds)
  int cand;    // 1: the items are the candidate list (particles 0..npfb near a boundary), from n0
};

// near-patch test of create_boundary_boxes: |perp| <= sup+1e-10 and 0<=tmp<=1
__device__ __forceinline__ bool near_patch(const Consts& c, double x, double y, int ib, double& tmp,
                                           double& perp) {
  perp = bound_dist(c, x, y, ib);
  if (fabs(perp) > c.sup_size + 1.0e-10) return false;
  double n1, n2;
  bound_norm(c, ib, n1, n2);
  tmp = pos_along(c, x, y, ib, perp, n1, n2);
  if (tmp < 0.0 || tmp > 1.0) return false;
  return true;
}
__device__ __forceinline__ bool near_corner(const Consts& c, double x, double y, int ib) {
  double a = x - c.b_node[ib][0], b = y - c.b_node[ib][1];
  double dd = sqrt(a * a + b * b);
  return !(dd > c.sup_size + 1.0e-10);
}

__device__ __forceinline__ int sel_end(const Consts& c, const Dev& d, const SelArgs& a) {
  return a.kind == SEL_CORNER_WP ? c.npfb + d.s->imp_temp : a.n1;
}

// number of mirrors item `it` creates in this stage
__device__ int sel_count(const Consts& c, const Dev& d, const SelArgs& a, int it) {
  const double x = d.rx[it], y = d.ry[it];
  switch (a.kind) {
    case SEL_CIRCLES: {
      int n = 0;
      for (int ic = 0; ic < c.ncirc; ++ic) {
        double R = c.c_radius[ic];
        double cdir = R / fabs(R);
        double r1 = x - c.c_centre[ic][0], r2 = y - c.c_centre[ic][1];
        double rad = sqrt(r1 * r1 + r2 * r2);
        if (cdir > 0.0) { if (rad <= R + c.sup_size) ++n; }
        else if (cdir < 0.0) { if (rad >= fabs(R) - c.sup_size) ++n; }
      }
      return n;
    }
    case SEL_WALL: {
      double bp1, bp2;
      if (!near_patch(c, x, y, a.ib, bp1, bp2)) return 0;
      if (bp2 <= 1.0e-10) return 0;
      int ibp1 = (a.ib + 1) % c.nb;
      double mbe = c.b_elen[a.ib];
      if (c.b_corner_angle[a.ib] < 0.0) {
        double ta = 0.5 * (PI + c.b_corner_angle[a.ib]);
        if (bp2 + 0.1 * c.dx >= bp1 * tan(ta) * mbe) return 0;
      }
      if (c.b_corner_angle[ibp1] < 0.0) {
        double ta = 0.5 * (PI + c.b_corner_angle[ibp1]);
        if (bp2 >= (1.0 - bp1) * tan(ta) * mbe) return 0;
      }
      return 1;
    }
    case SEL_PERIODIC: {
      double bp1, bp2;
      if (!near_patch(c, x, y, c.b_pp[a.ib], bp1, bp2)) return 0;
      return bp2 <= 0.0 ? 0 : 1;
    }
    case SEL_CORNER_WW:
      return near_corner(c, x, y, a.ib) ? 1 : 0;
    case SEL_CORNER_PP:
      return near_corner(c, x, y, c.b_pp[a.ib]) ? 1 : 0;
    case SEL_CORNER_WP: {
      int ibm1 = (a.ib + c.nb - 1) % c.nb;
      int ibb = (c.b_type[ibm1] == 1) ? ibm1 : a.ib;
      double perp = bound_dist(c, x, y, ibb);
      if (perp > c.sup_size + 1.0e-10) return 0;
      if (perp < 1.0e-10) return 0;
      double n1, n2;
      bound_norm(c, ibb, n1, n2);
      double t = pos_along(c, x, y, ibb, perp, n1, n2);
      return ((t < 0.0 && ibb == a.ib) || (t > 1.0 && ibb == ibm1)) ? 1 : 0;
    }
  }
  return 0;
}

__device__ __forceinline__ double dPf(const Consts& c, double xk, double yk, double xi, double yi) {
  return c.bf[0] * (xk - xi) + c.bf[1] * (yk - yi);
}

// write the mirrors of item `it` starting at mirror slot `slot` (0-based mirror number)
__device__ void sel_emit(const Consts& c, const Dev& d, const SelArgs& a, int it, int slot) {
  const double x = d.rx[it], y = d.ry[it];
  auto put = [&](int parent, int vrel, double mx, double my, double mu, double mv, double mth,
                 double dp) -> void {
    if (slot >= c.mcap) { set_error(d.s, VEBI_ERR_MIRROR_CAPACITY); return; }
    int k = c.npfb + slot;
    d.irel[k] = parent;
    d.vrel[k] = vrel;
    d.rx[k] = mx;
    d.ry[k] = my;
    d.ux[k] = mu;
    d.uy[k] = mv;
    d.th[k] = mth;
    d.dP_mp[k] = dp;
    d.inbin[k] = 0;
    ++slot;
  };
  switch (a.kind) {
    case SEL_CIRCLES: {
      for (int ic = 0; ic < c.ncirc; ++ic) {
        double R = c.c_radius[ic];
        double cdir = R / fabs(R);
        double r1 = x - c.c_centre[ic][0], r2 = y - c.c_centre[ic][1];
        double rad = sqrt(r1 * r1 + r2 * r2);
        bool make = false;
        double mx = 0, my = 0, Ra = 0;
        if (cdir > 0.0) {
          if (rad <= R + c.sup_size) {
            r1 = r1 / rad; r2 = r2 / rad;
            mx = x - r1 * 2.0 * (rad - R);
            my = y - r2 * 2.0 * (rad - R);
            Ra = R;
            make = true;
          }
        } else if (cdir < 0.0) {
          if (rad >= fabs(R) - c.sup_size) {
            r1 = r1 / rad; r2 = r2 / rad;
            mx = x + r1 * 2.0 * (fabs(R) - rad);
            my = y + r2 * 2.0 * (fabs(R) - rad);
            Ra = fabs(R);
            make = true;
          }
        }
        if (make) {
          double t1 = r2, t2 = -r1;
          double mu = 2.0 * c.c_vel[ic][0] + 2.0 * t1 * Ra * c.c_omega[ic] - 1.0 * d.ux[it];
          double mv = 2.0 * c.c_vel[ic][1] + 2.0 * t2 * Ra * c.c_omega[ic] - 1.0 * d.uy[it];
          double mth = 2.0 * c.c_thermal[ic] - 1.0 * d.th[it];
          put(it, 999 + ic + 1, mx, my, mu, mv, mth, dPf(c, mx, my, x, y));
        }
      }
      break;
    }
    case SEL_WALL: {
      double bp1, bp2;
      near_patch(c, x, y, a.ib, bp1, bp2);
      double n1, n2;
      bound_norm(c, a.ib, n1, n2);
      double mx = x - 2.0 * bp2 * n1, my = y - 2.0 * bp2 * n2;
      double t1 = n2, t2 = -n1;
      put(it, a.ib + 1, mx, my, 2.0 * c.b_vel[a.ib] * t1 - d.ux[it], 2.0 * c.b_vel[a.ib] * t2 - d.uy[it],
          2.0 * c.b_thermal[a.ib] - d.th[it], dPf(c, mx, my, x, y));
      break;
    }
    case SEL_PERIODIC: {
      double bp1, bp2;
      near_patch(c, x, y, c.b_pp[a.ib], bp1, bp2);
      double n1, n2;
      bound_norm(c, a.ib, n1, n2);
      double t1 = -1.0 * bp1 * c.b_edge[a.ib][0] - bp2 * n1;
      double t2 = -1.0 * bp1 * c.b_edge[a.ib][1] - bp2 * n2;
      double mx = c.b_node[a.ib][0] + c.b_edge[a.ib][0] + t1;
      double my = c.b_node[a.ib][1] + c.b_edge[a.ib][1] + t2;
      put(it, a.ib + 1, mx, my, d.ux[it], d.uy[it], d.th[it], 0.0);
      break;
    }
    case SEL_CORNER_WW: {
      int ib = a.ib, ibm1 = (ib + c.nb - 1) % c.nb;
      // `tmp` of the reference still holds the edge cross product (mirror_..:216,242)
      double tmp = c.b_edge[ibm1][0] * c.b_edge[ib][1] - c.b_edge[ibm1][1] * c.b_edge[ib][0];
      double tb1 = x - c.b_node[ib][0], tb2 = y - c.b_node[ib][1];
      double mx = x - 2.0 * tb1, my = y - 2.0 * tb2;
      double n1, n2;
      bound_norm(c, ib, n1, n2);
      double mu = 2.0 * tmp * n2 - d.ux[it];
      double mv = 2.0 * tmp * (-n1) - d.uy[it];
      bound_norm(c, ibm1, n1, n2);
      mu = mu + 2.0 * tmp * n2;
      mv = mv + 2.0 * tmp * (-n1);
      put(it, -(ib + 1), mx, my, mu, mv, d.th[it] + 2.0 * c.b_thermal[ib], dPf(c, mx, my, x, y));
      break;
    }
    case SEL_CORNER_PP: {
      int ib = a.ib, ibp = c.b_pp[ib];
      double tb1 = c.b_node[ib][0] - c.b_node[ibp][0], tb2 = c.b_node[ib][1] - c.b_node[ibp][1];
      put(it, -(ib + 1), x + tb1, y + tb2, d.ux[it], d.uy[it], d.th[it], 0.0);
      break;
    }
    case SEL_CORNER_WP: {
      int ib = a.ib, ibm1 = (ib + c.nb - 1) % c.nb;
      int ibb = (c.b_type[ibm1] == 1) ? ibm1 : ib;
      double perp = bound_dist(c, x, y, ibb);
      double n1, n2;
      bound_norm(c, ibb, n1, n2);
      double mx = x - 2.0 * perp * n1, my = y - 2.0 * perp * n2;
      double t1 = n2, t2 = -n1;
      double dp = d.dP_mp[it];
      dp = dp + (c.bf[0] * (mx - x) + c.bf[1] * (my - y));
      put(d.irel[it], -(ib + 1), mx, my, 2.0 * c.b_vel[ibb] * t1 - d.ux[it], 2.0 * c.b_vel[ibb] * t2 - d.uy[it],
          2.0 * c.b_thermal[ibb] - d.th[it], dp);
      break;
    }
  }
}

// per-block item counts
// item q of a stage: a particle or mirror index, or -1 past the end.  In candidate mode the
// items are the ascending candidate list, and those below n0 count nothing, so every stage
// still visits its items in ascending index order.
__device__ __forceinline__ int sel_item(const Consts& c, const Dev& d, const SelArgs& a, int q, int n1) {
  if (a.cand) {
    if (q >= d.s->n_cand) return -1;
    const int it = d.cand[q];
    return it >= a.n0 ? it : -1;
  }
  const int it = a.n0 + q;
  return it < n1 ? it : -1;
}

__global__ void k_sel_count(Consts c, Dev d, SelArgs a) {
  __shared__ int sh[TPB / 32];
  const int n1 = sel_end(c, d, a);
  int base = blockIdx.x * SEL_CH + threadIdx.x * SEL_IPT;
  int cnt = 0;
  for (int q = 0; q < SEL_IPT; ++q) {
    int it = sel_item(c, d, a, base + q, n1);
    if (it >= 0) cnt += sel_count(c, d, a, it);
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < TPB / 32; ++w) t += sh[w];
    d.sel_blk[blockIdx.x] = t;
  }
}

// exclusive scan of the block counts (one block), and the stage's base mirror number
__global__ void k_sel_scan(Dev d, int nblk, int mcap) {
  __shared__ int sh[1024];
  const int T = blockDim.x;
  int per = (nblk + T - 1) / T;
  int b0 = threadIdx.x * per, b1 = min(nblk, b0 + per);
  int loc = 0;
  for (int b = b0; b < b1; ++b) loc += d.sel_blk[b];
  sh[threadIdx.x] = loc;
  __syncthreads();
  for (int o = 1; o < T; o <<= 1) {
    int v = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += v;
    __syncthreads();
  }
  int run = sh[threadIdx.x] - loc;  // exclusive prefix of this thread's range
  for (int b = b0; b < b1; ++b) {
    int v = d.sel_blk[b];
    d.sel_blk[b] = run;
    run += v;
  }
  if (threadIdx.x == T - 1) {
    int total = sh[T - 1];
    Scal* s = d.s;
    s->sel_base = s->nmirror;
    s->sel_total = total;
    long long nm = (long long)s->nmirror + total;
    if (nm > mcap) { set_error(s, VEBI_ERR_MIRROR_CAPACITY); nm = mcap; }
    s->nmirror = (int)nm;
  }
}

// emit in item order: block offset + ordered prefix inside the block
__global__ void k_sel_emit(Consts c, Dev d, SelArgs a) {
  __shared__ int sh[TPB / 32 + 1];
  const int n1 = sel_end(c, d, a);
  int base = blockIdx.x * SEL_CH + threadIdx.x * SEL_IPT;
  int cnts[SEL_IPT], items[SEL_IPT];
  int tot = 0;
  for (int q = 0; q < SEL_IPT; ++q) {
    items[q] = sel_item(c, d, a, base + q, n1);
    cnts[q] = items[q] >= 0 ? sel_count(c, d, a, items[q]) : 0;
    tot += cnts[q];
  }
  // block exclusive scan of tot in thread order
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = tot;
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += v;
  }
  if (lane == 31) sh[w] = inc;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int q = 0; q < TPB / 32; ++q) { int v = sh[q]; sh[q] = run; run += v; }
  }
  __syncthreads();
  int slot = d.s->sel_base + d.sel_blk[blockIdx.x] + sh[w] + inc - tot;
  for (int q = 0; q < SEL_IPT; ++q) {
    if (cnts[q]) {
      sel_emit(c, d, a, items[q], slot);
      slot += cnts[q];
    }
  }
}

// The candidates of the mirror stages: particles 0..npfb within the support of a boundary line
// or a circle.  Every item any stage over particles can select is one: a wall or periodic
// image needs |perp| <= sup + 1e-10 to that patch's line, a corner image a node distance within
// the same bound (the node is on both lines), a circle image rad within R + sup (or |R| - sup).
// The test runs in FP32 with a margin of dx/10 plus 4e-6 of the box's extent, far above its
// rounding error, so the list is a superset of every stage's selection; the stages then apply
// their own FP64 tests.
struct NearTab {
  float a[VEBI_MAX_PATCHES], b[VEBI_MAX_PATCHES], c0[VEBI_MAX_PATCHES];  // perp = a x + b y + c0
  float cx[VEBI_MAX_CIRCLES], cy[VEBI_MAX_CIRCLES], lo2[VEBI_MAX_CIRCLES], hi2[VEBI_MAX_CIRCLES];
  float band;
  int np, nc;
};

__device__ void near_table(const Consts& c, NearTab& t) {
  const double m = c.near_band;
  if (threadIdx.x == 0) {
    int k = 0;
    for (int ib = 0; ib < c.nb; ++ib) {
      if (c.b_type[ib] == 0) continue;
      t.a[k] = c.bl_a[ib];
      t.b[k] = c.bl_b[ib];
      t.c0[k] = c.bl_c[ib];
      ++k;
    }
    t.np = k;
    for (int ic = 0; ic < c.ncirc; ++ic) {
      const double R = c.c_radius[ic];
      t.cx[ic] = (float)c.c_centre[ic][0];
      t.cy[ic] = (float)c.c_centre[ic][1];
      if (R > 0.0) { t.lo2[ic] = -1.0f; t.hi2[ic] = (float)((R + m) * (R + m)); }
      else { const double l = fmax(fabs(R) - m, 0.0); t.lo2[ic] = (float)(l * l); t.hi2[ic] = 3.0e38f; }
    }
    t.nc = c.ncirc;
    t.band = (float)m;
  }
  __syncthreads();
}

__device__ __forceinline__ bool near_boundary(const NearTab& t, double xd, double yd) {
  const float x = (float)xd, y = (float)yd;
  for (int k = 0; k < t.np; ++k)
    if (fabsf(fmaf(t.a[k], x, fmaf(t.b[k], y, t.c0[k]))) <= t.band) return true;
  for (int ic = 0; ic < t.nc; ++ic) {
    const float r1 = x - t.cx[ic], r2 = y - t.cy[ic];
    const float q = fmaf(r1, r1, r2 * r2);
    if (t.lo2[ic] < 0.0f ? q <= t.hi2[ic] : q >= t.lo2[ic]) return true;
  }
  return false;
}

__global__ void k_cand_count(Consts c, Dev d) {
  __shared__ int sh[TPB / 32];
  __shared__ NearTab t;
  near_table(c, t);
  const int base = blockIdx.x * SEL_CH + threadIdx.x * SEL_IPT;
  int cnt = 0;
  for (int q = 0; q < SEL_IPT; ++q) {
    const int it = base + q;
    if (it < c.npfb && near_boundary(t, d.rx[it], d.ry[it])) ++cnt;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int tt = 0;
    for (int w = 0; w < TPB / 32; ++w) tt += sh[w];
    d.cand_blk[blockIdx.x] = tt;
  }
}

__global__ void k_cand_scan(Dev d, int nblk) {
  __shared__ int sh[1024];
  const int T = blockDim.x;
  const int per = (nblk + T - 1) / T;
  const int b0 = threadIdx.x * per, b1 = min(nblk, b0 + per);
  int loc = 0;
  for (int b = b0; b < b1; ++b) loc += d.cand_blk[b];
  sh[threadIdx.x] = loc;
  __syncthreads();
  for (int o = 1; o < T; o <<= 1) {
    int v = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += v;
    __syncthreads();
  }
  int run = sh[threadIdx.x] - loc;
  for (int b = b0; b < b1; ++b) {
    int v = d.cand_blk[b];
    d.cand_blk[b] = run;
    run += v;
  }
  if (threadIdx.x == T - 1) d.s->n_cand = sh[T - 1];
}

__global__ void k_cand_emit(Consts c, Dev d) {
  __shared__ int sh[TPB / 32 + 1];
  __shared__ NearTab t;
  near_table(c, t);
  const int base = blockIdx.x * SEL_CH + threadIdx.x * SEL_IPT;
  bool f[SEL_IPT];
  int tot = 0;
  for (int q = 0; q < SEL_IPT; ++q) {
    const int it = base + q;
    f[q] = it < c.npfb && near_boundary(t, d.rx[it], d.ry[it]);
    tot += f[q] ? 1 : 0;
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = tot;
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += v;
  }
  if (lane == 31) sh[w] = inc;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int q = 0; q < TPB / 32; ++q) { int v = sh[q]; sh[q] = run; run += v; }
  }
  __syncthreads();
  int slot = d.cand_blk[blockIdx.x] + sh[w] + inc - tot;
  for (int q = 0; q < SEL_IPT; ++q)
    if (f[q]) d.cand[slot++] = base + q;
}

__global__ void k_snapshot_imp(Scal* s) { s->imp_temp = s->nmirror; }

// mirrors of moving solid particles copy their parent's u and theta (mirror_..:191-206)
__global__ void k_solid_fixup(Consts c, Dev d) {
  const int nm = d.s->nmirror;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nm; m += gridDim.x * blockDim.x) {
    int j = c.npfb + m, i = d.irel[j];
    if (i < c.nbS) {
      double tmp = d.ux[i] * d.ux[i] + d.uy[i] * d.uy[i];
      if (tmp != 0.0) { d.ux[j] = d.ux[i]; d.uy[j] = d.uy[i]; }
      double tt = d.th[i] * d.th[i];
      if (tt != 0.0) d.th[j] = d.th[i];
    }
  }
}

__global__ void k_set_np(Consts c, Scal* s) { s->np = c.npfb + s->nmirror; }

static void run_stage(Ctx& x, int kind, int ib, int n0, int n1_static, int n_items_bound) {
  // stages over particles (their items end at npfb) walk the candidate list instead
  const int cand = n1_static == x.c.npfb ? 1 : 0;
  SelArgs a{kind, ib, n0, n1_static, cand};
  if (cand) n_items_bound = x.c.npfb;  // the list can hold every particle, walls included
  int nblk = (n_items_bound + SEL_CH - 1) / SEL_CH;
  if (nblk < 1) nblk = 1;
  VEBI_LAUNCH(x, k_sel_count, nblk, TPB, x.c, x.d, a);
  VEBI_LAUNCH(x, k_sel_scan, 1, 1024, x.d, nblk, x.c.mcap);
  VEBI_LAUNCH(x, k_sel_emit, nblk, TPB, x.c, x.d, a);
}

void launch_advect_bin(Ctx& x) {
  const Consts& c = x.c;
  VEBI_LAUNCH(x, k_step_reset, 1, 1, x.d.s, c.npfb, c.nbS);
  VEBI_LAUNCH(x, k_save_umax, grid_for(c.npfb), TPB, c, x.d);
  VEBI_LAUNCH(x, k_advect_bin, grid_for(c.npfb), TPB, c, x.d);
}

// create_mirror_particles (mirror_boundaries_mod.F90:18-334)
void launch_mirrors(Ctx& x) {
  const Consts& c = x.c;
  {  // the candidate list of the stages over particles, in ascending index
    const int nblk = (c.npfb + SEL_CH - 1) / SEL_CH;
    VEBI_LAUNCH(x, k_cand_count, nblk, TPB, c, x.d);
    VEBI_LAUNCH(x, k_cand_scan, 1, 1024, x.d, nblk);
    VEBI_LAUNCH(x, k_cand_emit, nblk, TPB, c, x.d);
  }
  if (c.ncirc > 0) run_stage(x, SEL_CIRCLES, 0, c.nbS, c.npfb, c.npfb - c.nbS);
  for (int ib = 0; ib < c.nb; ++ib) {
    if (c.b_type[ib] == 1) run_stage(x, SEL_WALL, ib, 0, c.npfb, c.npfb);
    if (c.b_type[ib] == 2) run_stage(x, SEL_PERIODIC, ib, 0, c.npfb, c.npfb);
  }
  VEBI_LAUNCH(x, k_solid_fixup, x.gs_blocks, TPB, c, x.d);
  for (int ib = 0; ib < c.nb; ++ib) {
    int ibm1 = (ib + c.nb - 1) % c.nb;
    if (c.b_type[ib] == 0 || c.b_type[ibm1] == 0) continue;
    double tmp = c.b_edge[ibm1][0] * c.b_edge[ib][1] - c.b_edge[ibm1][1] * c.b_edge[ib][0];
    if (fabs(tmp) < 1e-10) continue;
    if (c.b_type[ib] == 1 && c.b_type[ibm1] == 1) {
      if (!(c.b_corner_angle[ib] <= 0.0)) run_stage(x, SEL_CORNER_WW, ib, c.nbS, c.npfb, c.npfb - c.nbS);
    }
    if (c.b_type[ib] == 2 && c.b_type[ibm1] == 2) run_stage(x, SEL_CORNER_PP, ib, c.nbS, c.npfb, c.npfb - c.nbS);
    if (c.b_type[ib] != c.b_type[ibm1] && (c.b_type[ib] == 1 || c.b_type[ibm1] == 1)) {
      VEBI_LAUNCH(x, k_snapshot_imp, 1, 1, x.d.s);
      run_stage(x, SEL_CORNER_WP, ib, c.npfb, 0, c.mcap);
    }
  }
  VEBI_LAUNCH(x, k_set_np, 1, 1, c, x.d.s);
}

// ------------------------------------------------------------------------------- mirror fields
// mirror_velocities (mirror_boundaries_mod.F90:509-584): u* of mirrors from their parents' u*
// (the predictor's output ux2/uy2), then solid-parent copies.
__global__ void k_mirror_velocities(Consts c, Dev d) {
  const int nm = d.s->nmirror;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nm; m += gridDim.x * blockDim.x) {
    int j = c.npfb + m, i = d.irel[j], vr = d.vrel[j];
    double ui = d.ux2[i], vi = d.uy2[i];
    double uj = d.ux[j], vj = d.uy[j];  // creation-time value (kept if no branch applies)
    if (vr > 999) {
      int ib = vr - 999 - 1;
      double r1 = 0.5 * (d.rx[i] - d.rx[j]), r2 = 0.5 * (d.ry[i] - d.ry[j]);
      double tmp = sqrt(r1 * r1 + r2 * r2);
      double t1 = r2 / tmp, t2 = -r1 / tmp;
      uj = 2.0 * c.c_vel[ib][0] + 2.0 * t1 * c.c_radius[ib] * c.c_omega[ib] - 1.0 * ui;
      vj = 2.0 * c.c_vel[ib][1] + 2.0 * t2 * c.c_radius[ib] * c.c_omega[ib] - 1.0 * vi;
    }
    if (vr > 0 && vr < 999) {
      int ib = vr - 1;
      if (abs(c.b_type[ib]) == 1) {
        double r1 = 0.5 * (d.rx[i] - d.rx[j]), r2 = 0.5 * (d.ry[i] - d.ry[j]);
        double tmp = sqrt(r1 * r1 + r2 * r2);
        double t1 = r2 / tmp, t2 = -r1 / tmp;
        uj = 2.0 * c.b_vel[ib] * t1 - ui;
        vj = 2.0 * c.b_vel[ib] * t2 - vi;
      } else if (c.b_type[ib] == 2) {
        uj = ui;
        vj = vi;
      }
    }
    if (vr < 0 && vr > -c.npfb) {
      int ib = -vr - 1, ibm1 = (ib + c.nb - 1) % c.nb;
      if (c.b_type[ib] == 1 && c.b_type[ibm1] == 1) {
        uj = ui; vj = vi;
        if (c.b_vel[ib] != 0.0) {
          double n1, n2; bound_norm(c, ib, n1, n2);
          double tmp = c.b_vel[ib];
          uj = 2.0 * tmp * n2 - ui;
          vj = 2.0 * tmp * (-n1) - vi;
        }
        if (c.b_vel[ibm1] != 0.0) {
          double n1, n2; bound_norm(c, ibm1, n1, n2);
          double tmp = c.b_vel[ibm1];
          uj = uj + 2.0 * tmp * n2;
          vj = vj + 2.0 * tmp * (-n1);
        }
      } else if (c.b_type[ib] == 2 && c.b_type[ibm1] == 2) {
        uj = ui; vj = vi;
      } else if ((c.b_type[ib] == 1 && c.b_type[ibm1] == 2) || (c.b_type[ib] == 2 && c.b_type[ibm1] == 1)) {
        double tmp = 0.0, t1 = 0.0, t2 = 0.0;
        if (c.b_vel[ib] != 0.0) {
          double n1, n2; bound_norm(c, ib, n1, n2); t1 = n2; t2 = -n1; tmp = c.b_vel[ib];
        } else if (c.b_vel[ibm1] != 0.0) {
          double n1, n2; bound_norm(c, ibm1, n1, n2); t1 = n2; t2 = -n1; tmp = c.b_vel[ibm1];
        }
        uj = 2.0 * tmp * t1 - ui;
        vj = 2.0 * tmp * t2 - vi;
      }
    }
    if (i < c.nbS) {
      double tmp = ui * ui + vi * vi;
      if (tmp != 0.0) { uj = ui; vj = vi; }
    }
    d.ux2[j] = uj;
    d.uy2[j] = vj;
  }
}

// mirror_polymeric_stress (mirror_boundaries_mod.F90:586-653)
__device__ __forceinline__ void reflect_tau(const Dev& d, int i, int j, double n1, double n2) {
  double nt1 = -n2, nt2 = n1;
  double q11 = 1.0 * n1 + 0.0 * n2, q12 = 1.0 * nt1 + 0.0 * nt2;
  double q21 = 0.0 * n1 + 1.0 * n2, q22 = 0.0 * nt1 + 1.0 * nt2;
  double T11 = d.tau[0][i], T21 = d.tau[1][i], T12 = d.tau[2][i], T22 = d.tau[3][i];
  // tmp = Q^T (T Q)
  double a11 = T11 * q11 + T12 * q21, a12 = T11 * q12 + T12 * q22;
  double a21 = T21 * q11 + T22 * q21, a22 = T21 * q12 + T22 * q22;
  double m11 = q11 * a11 + q21 * a21, m12 = q11 * a12 + q21 * a22;
  double m21 = q12 * a11 + q22 * a21, m22 = q12 * a12 + q22 * a22;
  m11 = -m11;
  m12 = -m12;
  // Q (tmp Q^T)
  double b11 = m11 * q11 + m12 * q12, b12 = m11 * q21 + m12 * q22;
  double b21 = m21 * q11 + m22 * q12, b22 = m21 * q21 + m22 * q22;
  d.tau[0][j] = q11 * b11 + q12 * b21;
  d.tau[2][j] = q11 * b12 + q12 * b22;
  d.tau[1][j] = q21 * b11 + q22 * b21;
  d.tau[3][j] = q21 * b12 + q22 * b22;
}

__global__ void k_mirror_stress(Consts c, Dev d) {
  const int nm = d.s->nmirror;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nm; m += gridDim.x * blockDim.x) {
    int j = c.npfb + m, i = d.irel[j], vr = d.vrel[j];
    if (vr > 999) {
      double r1 = d.rx[i] - d.rx[j], r2 = d.ry[i] - d.ry[j];
      double nn = sqrt(r1 * r1 + r2 * r2);
      reflect_tau(d, i, j, r1 / nn, r2 / nn);
    }
    if (vr > 0 && vr < 999) {
      int ib = vr - 1;
      if (c.b_type[ib] == 1) {
        double r1 = d.rx[i] - d.rx[j], r2 = d.ry[i] - d.ry[j];
        double nn = sqrt(r1 * r1 + r2 * r2);
        reflect_tau(d, i, j, r1 / nn, r2 / nn);
      } else if (c.b_type[ib] == 2 || c.b_type[ib] == 4) {
        for (int q = 0; q < 4; ++q) d.tau[q][j] = d.tau[q][i];
      } else if (c.b_type[ib] == 3) {
        for (int q = 0; q < 4; ++q) d.tau[q][j] = 0.0;
      }
    }
    if (vr < 0 && vr > -c.npfb) {
      int ib = -vr - 1, ibm1 = (ib + c.nb - 1) % c.nb;
      if (c.b_type[ib] == 1 && c.b_type[ibm1] == 1) {
        for (int q = 0; q < 4; ++q) d.tau[q][j] = -d.tau[q][i];
      } else if (c.b_type[ib] == 2 && c.b_type[ibm1] == 2) {
        for (int q = 0; q < 4; ++q) d.tau[q][j] = d.tau[q][i];
      } else if ((c.b_type[ib] == 1 && c.b_type[ibm1] == 2) || (c.b_type[ib] == 2 && c.b_type[ibm1] == 1)) {
        double n1, n2;
        if (c.b_type[ib] == 1) bound_norm(c, ib, n1, n2);
        else bound_norm(c, ibm1, n1, n2);
        reflect_tau(d, i, j, n1, n2);
      }
    }
  }
}

// grad_operator mirror transfer for the three gradients (gradient_calculation.F90:96-145).
// Circle mirrors keep 0: the reference tests vrelation == 999 while circles carry 999+ib.
__global__ void k_grad_mirrors(Consts c, Dev d) {
  const int nm = d.s->nmirror;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nm; m += gridDim.x * blockDim.x) {
    int j = c.npfb + m, i = d.irel[j], vr = d.vrel[j];
    int mode = 0;  // 0 none, 1 reflect, 2 reflect normal-zero, 3 copy, 4 negate, 5 rotate
    double r1 = 0, r2 = 0;
    if (vr > 0 && vr < 999) {
      int ib = vr - 1;
      if (c.b_type[ib] == 2) mode = 5;
      else if (c.b_type[ib] == 3) mode = 3;
      else if (c.b_type[ib] == 1) { mode = 1; r1 = d.rx[i] - d.rx[j]; r2 = d.ry[i] - d.ry[j]; }
      else if (c.b_type[ib] == 4) { mode = 2; r1 = d.rx[i] - d.rx[j]; r2 = d.ry[i] - d.ry[j]; }
    } else if (vr < 0 && vr > -c.npfb) {
      int ib = -vr - 1, ibm1 = (ib + c.nb - 1) % c.nb;
      if (c.b_type[ib] == 1 && c.b_type[ibm1] == 1) mode = 4;
      else if (c.b_type[ib] == 2 && c.b_type[ibm1] == 2) mode = 3;
      else if ((c.b_type[ib] == 1 && c.b_type[ibm1] == 2) || (c.b_type[ib] == 2 && c.b_type[ibm1] == 1)) {
        mode = 1;
        if (c.b_type[ib] == 1) { r1 = -1.0 * c.b_edge[ib][1]; r2 = c.b_edge[ib][0]; }
        else { r1 = -1.0 * c.b_edge[ibm1][1]; r2 = c.b_edge[ibm1][0]; }
      }
    }
    if (mode == 0) {  // no branch of the reference applies: the gradient stays 0
      for (int f = 0; f < 6; ++f) d.grad[f][j] = 0.0;
      continue;
    }
    for (int f = 0; f < 3; ++f) {
      double g1 = d.grad[2 * f][i], g2 = d.grad[2 * f + 1][i], o1, o2;
      if (mode == 3) { o1 = g1; o2 = g2; }
      else if (mode == 4) { o1 = -g1; o2 = -g2; }
      else if (mode == 5) {
        const double* Q = c.b_rot[vr - 1];
        o1 = Q[0] * g1 + Q[1] * g2;
        o2 = Q[2] * g1 + Q[3] * g2;
      } else {
        double nn = sqrt(r1 * r1 + r2 * r2);
        double q11 = r1 / nn, q21 = r2 / nn, q12 = -q21, q22 = q11;
        double b1 = q11 * g1 + q12 * g2, b2 = q21 * g1 + q22 * g2;
        if (mode == 2) b1 = 0.0; else b2 = -b2;
        o1 = q11 * b1 + q21 * b2;
        o2 = q12 * b1 + q22 * b2;
      }
      d.grad[2 * f][j] = o1;
      d.grad[2 * f + 1][j] = o2;
    }
  }
}

// mirror pressure P_j = P_parent + dP_mp (gradient_calculation.F90:26-30)
__global__ void k_mirror_pressure(Consts c, Dev d) {
  const int nm = d.s->nmirror;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nm; m += gridDim.x * blockDim.x) {
    int j = c.npfb + m;
    d.p[j] = d.p[d.irel[j]] + d.dP_mp[j];
  }
}

void launch_mirror_velocities(Ctx& x) { VEBI_LAUNCH(x, k_mirror_velocities, x.gs_blocks, TPB, x.c, x.d); }
void launch_mirror_stress(Ctx& x) { VEBI_LAUNCH(x, k_mirror_stress, x.gs_blocks, TPB, x.c, x.d); }
void launch_grad_mirrors(Ctx& x) { VEBI_LAUNCH(x, k_grad_mirrors, x.gs_blocks, TPB, x.c, x.d); }
void launch_mirror_pressure(Ctx& x) { VEBI_LAUNCH(x, k_mirror_pressure, x.gs_blocks, TPB, x.c, x.d); }

}  // namespace vebi
