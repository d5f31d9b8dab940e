// vebi_adjoint.cu -- reverse mode (vector-Jacobian products) of the step over a window of steps.
//
// The differentiated map.  One step takes the fields (u, theta, tau) of state n to state n+1.
// Inside the window the geometry of every step is that of a recorded base trajectory: the
// advected positions r* at which mirrors, the pair list, the kernel weights, the correction
// matrices and the PPE matrix are built, and dt.  The step's fields then go through the SPH
// operators, the log-conformation update and the PPE exactly as in the forward step
// (vebi_adjoint_replay runs that map, so finite differences see the same function).  The
// position update of the fields' next step is not differentiated.
//
// Reverse sweep.  The record run keeps the geometry (r*, dt) and the pressure of every step and
// the fields every K steps.  The reverse sweep walks the checkpoints backwards: it restores one,
// replays its K steps forward -- taking each step's pressure from the record instead of solving
// the PPE again -- while copying into a tape what the step's VJP needs (pair list and weights,
// correction matrices, PPE matrix, velocity gradients, tau before and after, per-mirror
// transfer coefficients), then runs the VJP kernels from the last of those steps to the first.
// The VJP of one step, in reverse order of the forward stages:
//   final update      u^{n+1} = u* + dt (f - grad P)            (u0 + dt f for cnt <= 3)
//   pressure gradient grad P_i = K_i sum_k (P_j - P_i) gradW_ik, mirrors P_m = P_parent + dP
//   PPE               A P = B: the transposed BiCGSTAB on A^T (built per step, ELL), zero-mean
//   right-hand side   b_i = -(1/dt) sum_k (u*_i - u*_j).(K_i gradW_ik), mean removed
//   predictor         u* = u + dt (cp (tau_j - tau_i).(K_i gradW) + cs (u_i - u_j) wL) + buoyancy,
//                     theta* = theta + dt ct sum (theta_i - theta_j) wL
//   log-conformation  per particle, three small forward-mode Jacobians chained backwards
//                     (vebi_adjoint_logconf.cuh)
//   gradients         grad u_i = K_i sum_k (u_j - u_i) gradW_ik
// and the mirror transfers (creation values, mirror velocities, mirror stress, mirror pressure)
// through their linear parts.  The j-side of every pair sum is gathered, not scattered: a
// transposed pair list per step (entries sorted by row and slot) gives each particle or mirror
// its incoming pairs in a fixed order, and a mirror-by-parent list moves mirror adjoints to the
// parents, so the reverse sweep is deterministic.
//
// Supported: closed domains with wall (b_type 1) and periodic (b_type 2) patches and their
// corners, circles, Newtonian or Oldroyd-B (ve_nonlinearity = 0), FP64 or mixed-precision
// contexts.  In a mixed context the window runs the mixed step (FP32 weights and correction
// matrices, FP32 pair sums); the tape widens the step's FP32 weights and correction matrices to
// FP64, so the VJP, in FP64, is that of the mixed map with the weights it used, exact up to the
// FP32 rounding of its pair sums; the transposed solve runs the context's mixed solver (FP64
// recurrences, FP32 SpMV) on an FP32 copy of A^T.  The adjoint also returns dJ/dWi
// (El = Wi sqrt(Pr/Ra) with Ra, Pr, beta fixed): Wi enters the polymeric coefficient
// (1-beta)/(Re Wi) and the relaxation factor exp(-dt/Wi).
//
// The reference has no adjoint; this file is this library's own.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "vebi_adjoint_logconf.cuh"
#include "vebi_ctx.cuh"
#include "vebi_solver.cuh"

namespace vebi {

void vebi_set_error_text(const std::string& msg);
void launch_bicgstab_on(Ctx& x, const BiArgs& a, bool nonull);
void launch_ppe_mg(Ctx& x);
void launch_ppe_mixed_solve(Ctx& x);

namespace {

constexpr int SLOT_BITS = 7;  // transposed-pair entries: row * 128 + slot
constexpr int MCO = 20;       // per-mirror coefficients: cu, ctheta, cv, (pad), tau map 4x4
constexpr int ATB = 1024;     // scan block

// ------------------------------------------------------------------------- device helpers
struct Tape {
  int nm = 0, kmax = 0;
  double dt = 0.0;
  int *cnt = nullptr, *link = nullptr, *pcol = nullptr, *irel = nullptr;  // irel: mirror m at m
  double *wgx = nullptr, *wgy = nullptr, *wl = nullptr, *pval = nullptr, *pdiag = nullptr;
  double* kg[4] = {};
  double* G[4] = {};
  double* tau0[4] = {};
  double* tau1[4] = {};  // after the step, particles and mirrors (cap entries)
  double* mco = nullptr;
};

struct Trans {  // incoming pairs per target (particles 0..npfb, mirrors npfb..np), mirrors per parent
  int *tptr, *tent, *tfill;
  int *mptr, *ment, *mfill;
  int *acnt, *acol, *afill, *aptr, *aent;
  double* aval;
  int capT;
  int* scan_tot;
  int* flag;  // [0]: a transposed PPE column over capacity
};

__device__ __forceinline__ void reflect_map(const double T[4], double n1, double n2, double out[4]) {
  // mirror_polymeric_stress's wall reflection (mirror_boundaries_mod.F90:586-653), linear in T
  double nt1 = -n2, nt2 = n1;
  double q11 = 1.0 * n1 + 0.0 * n2, q12 = 1.0 * nt1 + 0.0 * nt2;
  double q21 = 0.0 * n1 + 1.0 * n2, q22 = 0.0 * nt1 + 1.0 * nt2;
  double T11 = T[0], T21 = T[1], T12 = T[2], T22 = T[3];
  double a11 = T11 * q11 + T12 * q21, a12 = T11 * q12 + T12 * q22;
  double a21 = T21 * q11 + T22 * q21, a22 = T21 * q12 + T22 * q22;
  double m11 = q11 * a11 + q21 * a21, m12 = q11 * a12 + q21 * a22;
  double m21 = q12 * a11 + q22 * a21, m22 = q12 * a12 + q22 * a22;
  m11 = -m11;
  m12 = -m12;
  double b11 = m11 * q11 + m12 * q12, b12 = m11 * q21 + m12 * q22;
  double b21 = m21 * q11 + m22 * q12, b22 = m21 * q21 + m22 * q22;
  out[0] = q11 * b11 + q12 * b21;
  out[2] = q11 * b12 + q12 * b22;
  out[1] = q21 * b11 + q22 * b21;
  out[3] = q21 * b12 + q22 * b22;
}

// the linear part of k_mirror_stress for mirror j of parent i: out = map(T)
__device__ void tau_map(const Consts& c, int vr, double pr1, double pr2, const double T[4], double out[4]) {
  for (int q = 0; q < 4; ++q) out[q] = 0.0;
  if (vr > 999) {  // circle: reflection about the radial direction
    double nn = sqrt(pr1 * pr1 + pr2 * pr2);
    reflect_map(T, pr1 / nn, pr2 / nn, out);
  }
  if (vr > 0 && vr < 999) {
    int ib = vr - 1;
    if (c.b_type[ib] == 1) {
      double nn = sqrt(pr1 * pr1 + pr2 * pr2);
      reflect_map(T, pr1 / nn, pr2 / nn, out);
    } else if (c.b_type[ib] == 2 || c.b_type[ib] == 4) {
      for (int q = 0; q < 4; ++q) out[q] = T[q];
    }
  } else if (vr < 0 && vr > -c.npfb) {
    int ib = -vr - 1, ibm1 = (ib + c.nb - 1) % c.nb;
    if (c.b_type[ib] == 1 && c.b_type[ibm1] == 1) {
      for (int q = 0; q < 4; ++q) out[q] = -T[q];
    } else if (c.b_type[ib] == 2 && c.b_type[ibm1] == 2) {
      for (int q = 0; q < 4; ++q) out[q] = T[q];
    } else if ((c.b_type[ib] == 1 && c.b_type[ibm1] == 2) || (c.b_type[ib] == 2 && c.b_type[ibm1] == 1)) {
      double n1, n2;
      if (c.b_type[ib] == 1) bound_norm(c, ib, n1, n2);
      else bound_norm(c, ibm1, n1, n2);
      reflect_map(T, n1, n2, out);
    }
  }
}

// Per-mirror coefficients of the step just run: the creation values' and the mirror
// velocities' factor on the parent's value (sel_emit / k_mirror_velocities: 2 b - x is -1 for
// walls and circles, copies +1, a wall-periodic corner mirror -1 of its periodic image), and
// the stress map.
// geo = the step's r* (parent positions at the mirror stages); mirrors keep theirs in d.rx.
__global__ void k_adj_mirror_coefs(Consts c, Dev d, const double* __restrict__ geo, double* __restrict__ mco,
                                   int* __restrict__ irel_out) {
  const int nm = d.s->nmirror;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nm; m += gridDim.x * blockDim.x) {
    const int j = c.npfb + m, i = d.irel[j], vr = d.vrel[j];
    double cu = 0.0, cth = 0.0, cv = 0.0;
    if (vr > 999) {  // circle: 2 c_vel + rotation - u, 2 c_thermal - theta
      cu = -1.0;
      cth = -1.0;
      cv = -1.0;
    } else if (vr > 0 && vr < 999) {
      const int ib = vr - 1;
      if (c.b_type[ib] == 1) { cu = -1.0; cth = -1.0; cv = -1.0; }
      else if (c.b_type[ib] == 2) { cu = 1.0; cth = 1.0; cv = 1.0; }
    } else if (vr < 0 && vr > -c.npfb) {
      const int ib = -vr - 1, ibm1 = (ib + c.nb - 1) % c.nb;
      if (c.b_type[ib] == 1 && c.b_type[ibm1] == 1) { cu = -1.0; cth = 1.0; cv = c.b_vel[ib] != 0.0 ? -1.0 : 1.0; }
      else if (c.b_type[ib] == 2 && c.b_type[ibm1] == 2) { cu = 1.0; cth = 1.0; cv = 1.0; }
      else { cu = -1.0; cth = -1.0; cv = -1.0; }
    }
    if (i < c.nbS) {
      const double ui = d.ux2[i], vi = d.uy2[i];
      if (ui * ui + vi * vi != 0.0) cv = 1.0;
    }
    double* o = mco + (size_t)m * MCO;
    o[0] = cu;
    o[1] = cth;
    o[2] = cv;
    o[3] = 0.0;
    const double pr1 = geo[i] - d.rx[j], pr2 = geo[(size_t)c.npfb + i] - d.ry[j];
    for (int r = 0; r < 4; ++r) {
      double e[4] = {0.0, 0.0, 0.0, 0.0}, out[4];
      e[r] = 1.0;
      tau_map(c, vr, pr1, pr2, e, out);
      for (int q = 0; q < 4; ++q) o[4 + q * 4 + r] = out[q];  // row q (output), column r (input)
    }
    irel_out[m] = i;
  }
}

// a mixed-precision step's FP32 weights and correction matrices, widened into tape slot t
__global__ void k_adj_widen(Dev d, Tape t, long long ell, int n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < ell; e += stride) {
    t.wgx[e] = (double)d.wGx32[e];
    t.wgy[e] = (double)d.wGy32[e];
    t.wl[e] = (double)d.wL32[e];
  }
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    for (int q = 0; q < 4; ++q) t.kg[q][i] = (double)d.kgcm32[q][i];
}

// A^T for the mixed solver: its values in FP32 and its FP64 row sums (diagonal first, then the
// slots in order, as the forward assembly sums A's), for the SpMV's difference form
__global__ void k_adj_at32(int n, const int* __restrict__ acnt, const double* __restrict__ aval,
                           const double* __restrict__ pdiag, float* __restrict__ aval32,
                           double* __restrict__ arow) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double rs = pdiag[i];
  const int cnt = acnt[i];
  for (int k = 0; k < cnt; ++k) {
    const double v = aval[(size_t)k * n + i];
    rs += v;
    aval32[(size_t)k * n + i] = (float)v;
  }
  arow[i] = rs;
}

// ------------------------------------------------------------------ counting-sort transposes
__global__ void k_adj_count_pairs(int npfb, const int* __restrict__ cnt, const int* __restrict__ link,
                                  int* __restrict__ tcnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npfb) return;
  const int n = cnt[i];
  for (int k = 0; k < n; ++k) atomicAdd(&tcnt[link[(size_t)k * npfb + i]], 1);
}
__global__ void k_adj_fill_pairs(int npfb, const int* __restrict__ cnt, const int* __restrict__ link,
                                 const int* __restrict__ tptr, int* __restrict__ tfill, int* __restrict__ tent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npfb) return;
  const int n = cnt[i];
  for (int k = 0; k < n; ++k) {
    const int j = link[(size_t)k * npfb + i];
    const int pos = atomicAdd(&tfill[j], 1);
    tent[tptr[j] + pos] = (i << SLOT_BITS) | k;
  }
}
__global__ void k_adj_count_mirrors(int nm, const int* __restrict__ irel, int* __restrict__ mcnt) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < nm) atomicAdd(&mcnt[irel[m]], 1);
}
__global__ void k_adj_fill_mirrors(int nm, const int* __restrict__ irel, const int* __restrict__ mptr,
                                   int* __restrict__ mfill, int* __restrict__ ment) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nm) return;
  const int p = irel[m];
  ment[mptr[p] + atomicAdd(&mfill[p], 1)] = m;
}
// PPE columns: nonzero slots only (one per row and column: the assembly accumulates duplicates
// into the last slot and leaves the others 0)
__global__ void k_adj_count_cols(int npfb, const int* __restrict__ cnt, const int* __restrict__ pcol,
                                 const double* __restrict__ pval, int* __restrict__ acnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npfb) return;
  const int n = cnt[i];
  for (int k = 0; k < n; ++k) {
    const size_t e = (size_t)k * npfb + i;
    if (pval[e] != 0.0) atomicAdd(&acnt[pcol[e]], 1);
  }
}
__global__ void k_adj_fill_cols(int npfb, const int* __restrict__ cnt, const int* __restrict__ pcol,
                                const double* __restrict__ pval, const int* __restrict__ aptr,
                                int* __restrict__ afill, int* __restrict__ aent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npfb) return;
  const int n = cnt[i];
  for (int k = 0; k < n; ++k) {
    const size_t e = (size_t)k * npfb + i;
    if (pval[e] == 0.0) continue;
    const int col = pcol[e];
    aent[aptr[col] + atomicAdd(&afill[col], 1)] = (i << SLOT_BITS) | k;
  }
}
// Sort every segment ascending.  One warp per segment: each lane holds up to R of its entries
// in registers, every entry's rank is the number of entries below it (the entries of a segment
// are distinct: (row, slot) codes or mirror indices), and each entry is stored at its rank.
// Segments of up to 64 entries (nearly all) take R = 2, up to 256 R = 8; a longer one (none with
// nplink <= 128) is sorted by one lane.
template <int R>
__device__ __forceinline__ void warp_rank_sort(int* __restrict__ ent, int a, int len, int lane) {
  int v[R], rk[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int e = lane + 32 * q;
    v[q] = e < len ? ent[a + e] : 0x7fffffff;
    rk[q] = 0;
  }
#pragma unroll
  for (int q2 = 0; q2 < R; ++q2) {
    if (32 * q2 >= len) break;
    for (int src = 0; src < 32; ++src) {
      const int o = __shfl_sync(0xffffffffu, v[q2], src);
#pragma unroll
      for (int q = 0; q < R; ++q) rk[q] += (o < v[q]) ? 1 : 0;
    }
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int e = lane + 32 * q;
    if (e < len) ent[a + rk[q]] = v[q];
  }
  __syncwarp();
}
__global__ void k_adj_sort_segments(int n, const int* __restrict__ ptr, int* __restrict__ ent) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < n; s += nw) {
    const int a = ptr[s], len = ptr[s + 1] - a;
    if (len <= 1) continue;
    if (len <= 64) {
      warp_rank_sort<2>(ent, a, len, lane);
    } else if (len <= 256) {
      warp_rank_sort<8>(ent, a, len, lane);
    } else {
      if (lane == 0) {
        for (int q = a + 1; q < a + len; ++q) {
          const int v = ent[q];
          int r = q - 1;
          while (r >= a && ent[r] > v) {
            ent[r + 1] = ent[r];
            --r;
          }
          ent[r + 1] = v;
        }
      }
      __syncwarp();
    }
  }
}
static int sort_grid(int segments) {
  const long long warps = segments > 0 ? segments : 1;
  const long long g = (warps * 32 + TPB - 1) / TPB;
  return (int)(g < 4096 ? g : 4096);
}
// A^T in the ELL layout of the step's solver: row c of A^T lists (i, A_ic) in ascending i
__global__ void k_adj_write_at(int npfb, int capT, const int* __restrict__ aptr, const int* __restrict__ aent,
                               const double* __restrict__ pval, int* __restrict__ acnt, int* __restrict__ acol,
                               double* __restrict__ aval, int* __restrict__ flag) {
  const int cidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (cidx >= npfb) return;
  const int a = aptr[cidx], n = aptr[cidx + 1] - a;
  if (n > capT) {
    atomicExch(flag, 1);
    acnt[cidx] = 0;
    return;
  }
  for (int q = 0; q < n; ++q) {
    const int e = aent[a + q];
    const int i = e >> SLOT_BITS, k = e & ((1 << SLOT_BITS) - 1);
    acol[(size_t)q * npfb + cidx] = i;
    aval[(size_t)q * npfb + cidx] = pval[(size_t)k * npfb + i];
  }
  acnt[cidx] = n;
}

// exclusive scan of n ints (in place into ptr[0..n], ptr[n] = total), three passes
__global__ void k_adj_scan_blocks(int n, const int* __restrict__ v, int* __restrict__ tot) {
  __shared__ int sh[32];
  const int b0 = blockIdx.x * ATB;
  int loc = 0;
  for (int q = threadIdx.x; q < ATB; q += blockDim.x)
    if (b0 + q < n) loc += v[b0 + q];
  for (int o = 16; o; o >>= 1) loc += __shfl_down_sync(0xffffffffu, loc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = loc;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
    tot[blockIdx.x] = t;
  }
}
__global__ void k_adj_scan_totals(int nb, int* __restrict__ tot) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int run = 0;
  for (int b = 0; b < nb; ++b) {
    const int t = tot[b];
    tot[b] = run;
    run += t;
  }
  tot[nb] = run;
}
__global__ void k_adj_scan_apply(int n, const int* __restrict__ v, const int* __restrict__ tot,
                                 int* __restrict__ ptr) {
  // one block per ATB entries: thread 0 scans the block's entries serially from its offset
  __shared__ int sh[ATB];
  const int b0 = blockIdx.x * ATB;
  for (int q = threadIdx.x; q < ATB; q += blockDim.x) sh[q] = b0 + q < n ? v[b0 + q] : 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = tot[blockIdx.x];
    for (int q = 0; q < ATB; ++q) {
      const int t = sh[q];
      sh[q] = run;
      run += t;
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < ATB; q += blockDim.x)
    if (b0 + q < n) ptr[b0 + q] = sh[q];
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) ptr[n] = tot[gridDim.x];
}

// ------------------------------------------------------------------------------ VJP stages
struct AdjVec {
  double *Ru, *Rv, *Rth, *Rtau[4];  // adjoint of state n+1 (npfb)
  double *Nu, *Nv, *Nth, *Ntau[4];  // adjoint of state n (npfb), accumulated
  double *aus, *avs, *aP, *abx, *aby, *lam, *q;  // work (cap or npfb)
  double *s1, *s2, *st, *at[4], *Gb[4];           // work (npfb; at: cap)
  double *mu, *mv, *mth, *mt[4];                  // mirror-side values (mcap)
  double* part;                                   // block partials
};

// final update and pressure gradient, own-row part
__global__ void k_adj_final(Consts c, Tape t, AdjVec a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const int cnt = t.cnt[i];
  const double ru = a.Ru[i], rv = a.Rv[i];
  double us = 0.0, vs = 0.0, gx = 0.0, gy = 0.0;
  if (i >= c.nbS) {
    if (cnt <= 3) {
      a.Nu[i] += ru;
      a.Nv[i] += rv;
    } else {
      us = ru;
      vs = rv;
      gx = -t.dt * ru;
      gy = -t.dt * rv;
    }
  } else {
    us = ru;
    vs = rv;
  }
  a.aus[i] = us;
  a.avs[i] = vs;
  const double K11 = t.kg[0][i], K21 = t.kg[1][i], K12 = t.kg[2][i], K22 = t.kg[3][i];
  const double a1 = K11 * gx + K21 * gy, a2 = K12 * gx + K22 * gy;
  a.abx[i] = a1;
  a.aby[i] = a2;
  double own = 0.0;
  for (int k = 0; k < cnt; ++k) {
    const size_t e = (size_t)k * c.npfb + i;
    own -= a1 * t.wgx[e] + a2 * t.wgy[e];
  }
  a.aP[i] = own;
}

// P-bar of every particle and mirror: own part + incoming pairs
__global__ void k_adj_gather_P(Consts c, Tape t, Trans T, AdjVec a, int np) {
  const int cc = blockIdx.x * blockDim.x + threadIdx.x;
  if (cc >= np) return;
  double acc = cc < c.npfb ? a.aP[cc] : 0.0;
  for (int q = T.tptr[cc]; q < T.tptr[cc + 1]; ++q) {
    const int en = T.tent[q];
    const int i = en >> SLOT_BITS, k = en & ((1 << SLOT_BITS) - 1);
    const size_t e = (size_t)k * c.npfb + i;
    acc += a.abx[i] * t.wgx[e] + a.aby[i] * t.wgy[e];
  }
  a.aP[cc] = acc;
}

// mirror values to parents: dst[p] += sum over p's mirrors of coef(m) * src[mirror]
// (src indexed by mirror number, or by particle index npfb + m when src_global)
__global__ void k_adj_push(Consts c, Trans T, const double* __restrict__ mco, int which, const double* src,
                           int src_global, double* dst, const double* src2, double* dst2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.npfb) return;
  double acc = 0.0, acc2 = 0.0;
  for (int q = T.mptr[p]; q < T.mptr[p + 1]; ++q) {
    const int m = T.ment[q];
    const double f = which < 0 ? 1.0 : mco[(size_t)m * MCO + which];
    const size_t s = src_global ? (size_t)c.npfb + m : (size_t)m;
    acc += f * src[s];
    if (src2) acc2 += f * src2[s];
  }
  dst[p] += acc;
  if (dst2) dst2[p] += acc2;
}

// stress adjoint of the mirrors to their parents through the transposed stress map
__global__ void k_adj_push_tau(Consts c, Trans T, const double* __restrict__ mco, AdjVec a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.npfb) return;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int q = T.mptr[p]; q < T.mptr[p + 1]; ++q) {
    const int m = T.ment[q];
    const double* M = mco + (size_t)m * MCO + 4;
    for (int r = 0; r < 4; ++r) {
      double s = 0.0;
      for (int o = 0; o < 4; ++o) s += M[o * 4 + r] * a.mt[o][m];
      acc[r] += s;
    }
  }
  for (int r = 0; r < 4; ++r) a.at[r][p] += acc[r];
}

// deterministic sum of v[0..n) into part[blockIdx] then into out (one block)
__global__ void k_adj_block_sum(int n, const double* __restrict__ v, double* __restrict__ part) {
  __shared__ double sh[TPB / 32 + 1];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double x = i < n ? v[i] : 0.0;
  x = block_sum<TPB>(x, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = x;
}
__global__ void k_adj_final_sum(int nb, const double* __restrict__ part, double* __restrict__ out) {
  __shared__ double sh[TPB / 32 + 1];
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[b];
  s = block_sum<TPB>(s, sh);
  if (threadIdx.x == 0) *out = s;
}
__global__ void k_adj_sub_mean(int n, const double* __restrict__ sum, const double* __restrict__ v,
                               double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = v[i] - *sum / (double)n;
}
__global__ void k_adj_block_sumsq(int n, const double* __restrict__ v, double* __restrict__ part) {
  __shared__ double sh[TPB / 32 + 1];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double x = i < n ? v[i] * v[i] : 0.0;
  x = block_sum<TPB>(x, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = x;
}
// v *= 1/rms (dir > 0) or rms (dir < 0), rms = sqrt(sumsq/n); a zero vector stays zero
__global__ void k_adj_scale(int n, const double* __restrict__ sumsq, double* __restrict__ v, int dir) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double rms = sqrt(*sumsq / (double)n);
  v[i] = rms > 0.0 ? (dir > 0 ? v[i] / rms : v[i] * rms) : 0.0;
}

// right-hand side: q_i = b-bar_i / dt and the own-row part of u*-bar
__global__ void k_adj_rhs_rows(Consts c, Tape t, AdjVec a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const double q = -a.lam[i] / t.dt;  // b_i = -(1/dt) sum (u*_i - u*_j).kw: d b_i / d u*_j = +kw/dt
  a.q[i] = q;
  const double K11 = t.kg[0][i], K21 = t.kg[1][i], K12 = t.kg[2][i], K22 = t.kg[3][i];
  double s1 = 0.0, s2 = 0.0;
  const int cnt = t.cnt[i];
  for (int k = 0; k < cnt; ++k) {
    const size_t e = (size_t)k * c.npfb + i;
    const double w1 = t.wgx[e], w2 = t.wgy[e];
    s1 += K11 * w1 + K12 * w2;
    s2 += K21 * w1 + K22 * w2;
  }
  a.aus[i] += q * s1;  // d b_i / d u*_i = -(1/dt) sum kw
  a.avs[i] += q * s2;
}
__global__ void k_adj_gather_us(Consts c, Tape t, Trans T, AdjVec a, int np) {
  const int cc = blockIdx.x * blockDim.x + threadIdx.x;
  if (cc >= np) return;
  double gu = 0.0, gv = 0.0;
  for (int q = T.tptr[cc]; q < T.tptr[cc + 1]; ++q) {
    const int en = T.tent[q];
    const int i = en >> SLOT_BITS, k = en & ((1 << SLOT_BITS) - 1);
    const size_t e = (size_t)k * c.npfb + i;
    const double w1 = t.wgx[e], w2 = t.wgy[e];
    const double qi = a.q[i];
    gu -= qi * (t.kg[0][i] * w1 + t.kg[2][i] * w2);
    gv -= qi * (t.kg[1][i] * w1 + t.kg[3][i] * w2);
  }
  if (cc < c.npfb) {
    a.aus[cc] += gu;
    a.avs[cc] += gv;
  } else {
    a.aus[cc] = gu;
    a.avs[cc] = gv;
  }
}

// predictor, own-row part; dJ/dcp of this step into part
__global__ void k_adj_pred_rows(Consts c, Tape t, AdjVec a, int ve) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < c.npfb) {
    const double us = a.aus[i], vs = a.avs[i], ths = a.Rth[i];
    a.Nu[i] += us;
    a.Nv[i] += vs;
    a.Nth[i] += ths;
    double s1 = 0.0, s2 = 0.0, st = 0.0;
    if (i >= c.nbS) {
      s1 = t.dt * us;
      s2 = t.dt * vs;
      st = t.dt * ths;
      a.Nth[i] += s2;  // buoyancy: s2 += theta_i
    }
    a.s1[i] = s1;
    a.s2[i] = s2;
    a.st[i] = st;
    const double cs = c.coeff_solvent, cp = c.coeff_polymeric, ct = c.coeff_theta;
    const double K11 = t.kg[0][i], K21 = t.kg[1][i], K12 = t.kg[2][i], K22 = t.kg[3][i];
    double swl = 0.0, o0 = 0.0, o1 = 0.0, o2 = 0.0, o3 = 0.0;
    const int cnt = t.cnt[i];
    for (int k = 0; k < cnt; ++k) {
      const size_t e = (size_t)k * c.npfb + i;
      swl += t.wl[e];
      if (ve) {
        const double w1 = t.wgx[e], w2 = t.wgy[e];
        const double kw1 = K11 * w1 + K12 * w2, kw2 = K21 * w1 + K22 * w2;
        o0 -= cp * kw1 * s1;
        o2 -= cp * kw2 * s1;
        o1 -= cp * kw1 * s2;
        o3 -= cp * kw2 * s2;
      }
    }
    a.Nu[i] += cs * s1 * swl;
    a.Nv[i] += cs * s2 * swl;
    a.Nth[i] += ct * st * swl;
    a.at[0][i] = o0;
    a.at[1][i] = o1;
    a.at[2][i] = o2;
    a.at[3][i] = o3;
  }
}
__global__ void k_adj_gather_pred(Consts c, Tape t, Trans T, AdjVec a, int np, int ve) {
  const int cc = blockIdx.x * blockDim.x + threadIdx.x;
  if (cc >= np) return;
  const double cs = c.coeff_solvent, cp = c.coeff_polymeric, ct = c.coeff_theta;
  double gu = 0.0, gv = 0.0, gth = 0.0, g0 = 0.0, g1 = 0.0, g2 = 0.0, g3 = 0.0;
  for (int q = T.tptr[cc]; q < T.tptr[cc + 1]; ++q) {
    const int en = T.tent[q];
    const int i = en >> SLOT_BITS, k = en & ((1 << SLOT_BITS) - 1);
    const size_t e = (size_t)k * c.npfb + i;
    const double wl = t.wl[e], s1 = a.s1[i], s2 = a.s2[i];
    gu -= cs * wl * s1;
    gv -= cs * wl * s2;
    gth -= ct * wl * a.st[i];
    if (ve) {
      const double w1 = t.wgx[e], w2 = t.wgy[e];
      const double kw1 = t.kg[0][i] * w1 + t.kg[2][i] * w2, kw2 = t.kg[1][i] * w1 + t.kg[3][i] * w2;
      g0 += cp * kw1 * s1;
      g2 += cp * kw2 * s1;
      g1 += cp * kw1 * s2;
      g3 += cp * kw2 * s2;
    }
  }
  if (cc < c.npfb) {
    a.Nu[cc] += gu;
    a.Nv[cc] += gv;
    a.Nth[cc] += gth;
    a.at[0][cc] += g0;
    a.at[1][cc] += g1;
    a.at[2][cc] += g2;
    a.at[3][cc] += g3;
  } else {
    const int m = cc - c.npfb;
    a.mu[m] = gu;
    a.mv[m] = gv;
    a.mth[m] = gth;
    a.mt[0][m] = g0;
    a.mt[1][m] = g1;
    a.mt[2][m] = g2;
    a.mt[3][m] = g3;
  }
}

// dJ/dcp of this step into part: the polymeric pair sum is bilinear in cp and tau, so
// cp dJ/dcp = sum over particles and mirrors of tau . tau-bar (its own-row and gathered parts,
// before the mirrors' share moves to the parents), with no second pass over the pairs.
// A grid-stride loop over np; one partial per block (grid <= npfb / TPB + 1 blocks).
__global__ void k_adj_dcp(Consts c, Tape t, AdjVec a, int np, double inv_cp) {
  __shared__ double sh[TPB / 32 + 1];
  double acc = 0.0;
  for (int cc = blockIdx.x * blockDim.x + threadIdx.x; cc < np; cc += gridDim.x * blockDim.x) {
    if (cc < c.npfb) {
      for (int q = 0; q < 4; ++q) acc += t.tau1[q][cc] * a.at[q][cc];
    } else {
      const int m = cc - c.npfb;
      for (int q = 0; q < 4; ++q) acc += t.tau1[q][cc] * a.mt[q][m];
    }
  }
  acc = block_sum<TPB>(acc, sh);
  if (threadIdx.x == 0) a.part[blockIdx.x] = acc * inv_cp;
}

// log-conformation: (tau-bar^n, G-bar) = J^T tau-bar^{n+1}; dJ/de1 of this step into part
__global__ void k_adj_logconf(Consts c, Tape t, AdjVec a, double e1, int ve) {
  __shared__ double sh[TPB / 32 + 1];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double de1 = 0.0;
  if (i < c.npfb) {
    double tb[4];
    for (int q = 0; q < 4; ++q) tb[q] = a.Rtau[q][i] + a.at[q][i];
    if (ve) {
      double tau[4], G[4], taub[4], Gb[4], e1b;
      for (int q = 0; q < 4; ++q) {
        tau[q] = t.tau0[q][i];
        G[q] = t.G[q][i];
      }
      logconf_vjp(tau, G, t.dt, e1, tb, taub, Gb, e1b);
      for (int q = 0; q < 4; ++q) {
        a.Ntau[q][i] += taub[q];
        a.Gb[q][i] = Gb[q];
      }
      de1 += e1b;
    } else {  // Newtonian: tau is carried unchanged
      for (int q = 0; q < 4; ++q) {
        a.Ntau[q][i] += tb[q];
        a.Gb[q][i] = 0.0;
      }
    }
  }
  de1 = block_sum<TPB>(de1, sh);
  if (threadIdx.x == 0) a.part[blockIdx.x] = de1;
}

// velocity gradients: own-row part; the per-row factors a0..a3 go to s1, s2, st, q
__global__ void k_adj_grad_rows(Consts c, Tape t, AdjVec a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const double K11 = t.kg[0][i], K21 = t.kg[1][i], K12 = t.kg[2][i], K22 = t.kg[3][i];
  const double G0 = a.Gb[0][i], G1 = a.Gb[1][i], G2 = a.Gb[2][i], G3 = a.Gb[3][i];
  const double a0 = K11 * G0 + K21 * G1, a1 = K12 * G0 + K22 * G1;
  const double a2 = K11 * G2 + K21 * G3, a3 = K12 * G2 + K22 * G3;
  a.s1[i] = a0;
  a.s2[i] = a1;
  a.st[i] = a2;
  a.q[i] = a3;
  double su = 0.0, sv = 0.0;
  const int cnt = t.cnt[i];
  for (int k = 0; k < cnt; ++k) {
    const size_t e = (size_t)k * c.npfb + i;
    const double w1 = t.wgx[e], w2 = t.wgy[e];
    su += a0 * w1 + a1 * w2;
    sv += a2 * w1 + a3 * w2;
  }
  a.Nu[i] -= su;
  a.Nv[i] -= sv;
}
__global__ void k_adj_gather_grad(Consts c, Tape t, Trans T, AdjVec a, int np) {
  const int cc = blockIdx.x * blockDim.x + threadIdx.x;
  if (cc >= np) return;
  double gu = 0.0, gv = 0.0;
  for (int q = T.tptr[cc]; q < T.tptr[cc + 1]; ++q) {
    const int en = T.tent[q];
    const int i = en >> SLOT_BITS, k = en & ((1 << SLOT_BITS) - 1);
    const size_t e = (size_t)k * c.npfb + i;
    const double w1 = t.wgx[e], w2 = t.wgy[e];
    gu += a.s1[i] * w1 + a.s2[i] * w2;
    gv += a.st[i] * w1 + a.q[i] * w2;
  }
  if (cc < c.npfb) {
    a.Nu[cc] += gu;
    a.Nv[cc] += gv;
  } else {
    a.mu[cc - c.npfb] = gu;
    a.mv[cc - c.npfb] = gv;
  }
}

// the value e1 of the step's relaxation (k_logconf, Oldroyd-B: alpha_R = 1)
double relax_e1(const Consts& c, double dt) { return exp(-(1.0 * 1.0 * dt / c.Wi)); }

}  // namespace

// ----------------------------------------------------------------------------- host side
struct Adjoint {
  Ctx* x = nullptr;
  int max_steps = 0, K = 1, nsteps = 0, nseg = 0;
  size_t n = 0, cap = 0, mcap = 0, kp = 0;
  double* geo = nullptr;    // per step: r* x, r* y (npfb each), dt
  double* pres = nullptr;   // per step: the pressure P (npfb)
  double* ckpt = nullptr;   // per checkpoint: u, v, theta, tau x4, trace, r x, r y (npfb each)
  uint8_t* ckpt_inbin = nullptr;
  std::vector<Tape> tape;   // K slots
  Trans T{};
  AdjVec a{};
  double* sums = nullptr;   // per step: dJ/dcp, dJ/de1
  float* aval32 = nullptr;  // mixed contexts: A^T in FP32 (same slots as Trans::aval)
  double* arow = nullptr;   // mixed contexts: A^T's row sums
  double* tmp1 = nullptr;
  std::vector<void*> allocs;
  int ls_iters_total = 0;
};

static int afail(int code, const std::string& msg) {
  vebi_set_error_text(msg);
  return code;
}

template <class T>
static T* aalloc(Adjoint& A, size_t count, cudaError_t& err) {
  void* p = nullptr;
  if (err == cudaSuccess) err = cudaMalloc(&p, sizeof(T) * (count ? count : 1));
  if (err == cudaSuccess) A.allocs.push_back(p);
  return (T*)p;
}

static constexpr int CK_PLANES = 10;

int adjoint_check_scope(const Ctx& x) {
  const Consts& c = x.c;
  if (c.open_domain) return afail(VEBI_ERR_ARG, "adjoint: closed domains only");
  for (int p = 0; p < c.nb; ++p)
    if (c.b_type[p] != 1 && c.b_type[p] != 2) return afail(VEBI_ERR_ARG, "adjoint: wall and periodic patches only");
  if (c.const_mod != 1 && c.eps_ptt != 0.0) return afail(VEBI_ERR_ARG, "adjoint: Oldroyd-B (ve_nonlinearity = 0) only");
  if (c.correct_velocity) return afail(VEBI_ERR_ARG, "adjoint: correct_velocity is not supported");
  if (c.warm_start) return afail(VEBI_ERR_ARG, "adjoint: the PPE warm start is not supported");
  if (x.precision != VEBI_PREC_FP64 && x.precision != VEBI_PREC_MIXED)
    return afail(VEBI_ERR_ARG, "adjoint: FP64 or mixed-precision contexts only");
  if (c.npfb >= (1 << (31 - SLOT_BITS))) return afail(VEBI_ERR_ARG, "adjoint: too many particles");
  if (c.nplink > (1 << SLOT_BITS)) return afail(VEBI_ERR_ARG, "adjoint: nplink above 128");
  return VEBI_OK;
}

int adjoint_create(Ctx& x, int max_steps, int K, Adjoint** out) {
  if (max_steps < 1 || K < 1) return afail(VEBI_ERR_ARG, "adjoint: max_steps and checkpoint_every must be >= 1");
  int st = adjoint_check_scope(x);
  if (st) return st;
  Adjoint* A = new Adjoint();
  A->x = &x;
  A->max_steps = max_steps;
  A->K = K < max_steps ? K : max_steps;
  const Consts& c = x.c;
  A->n = (size_t)c.npfb;
  A->cap = (size_t)c.cap;
  A->mcap = (size_t)(c.cap - c.npfb);
  A->kp = (size_t)c.nplink;
  const size_t n = A->n, cap = A->cap, mcap = A->mcap, kp = A->kp;
  const int nck = (max_steps + A->K - 1) / A->K;
  cudaError_t err = cudaSuccess;
  A->geo = aalloc<double>(*A, (size_t)max_steps * (2 * n + 1), err);
  A->pres = aalloc<double>(*A, (size_t)max_steps * n, err);
  A->ckpt = aalloc<double>(*A, (size_t)nck * CK_PLANES * n, err);
  A->ckpt_inbin = aalloc<uint8_t>(*A, (size_t)nck * n, err);
  A->tape.resize(A->K);
  for (auto& t : A->tape) {
    t.cnt = aalloc<int>(*A, n, err);
    t.link = aalloc<int>(*A, kp * n, err);
    t.pcol = aalloc<int>(*A, kp * n, err);
    t.irel = aalloc<int>(*A, mcap, err);
    t.wgx = aalloc<double>(*A, kp * n, err);
    t.wgy = aalloc<double>(*A, kp * n, err);
    t.wl = aalloc<double>(*A, kp * n, err);
    t.pval = aalloc<double>(*A, kp * n, err);
    t.pdiag = aalloc<double>(*A, n, err);
    for (int q = 0; q < 4; ++q) {
      t.kg[q] = aalloc<double>(*A, n, err);
      t.G[q] = aalloc<double>(*A, n, err);
      t.tau0[q] = aalloc<double>(*A, n, err);
      t.tau1[q] = aalloc<double>(*A, cap, err);
    }
    t.mco = aalloc<double>(*A, mcap * MCO, err);
  }
  Trans& T = A->T;
  T.capT = 2 * (int)kp;
  T.tptr = aalloc<int>(*A, cap + 1, err);
  T.tent = aalloc<int>(*A, kp * n, err);
  T.tfill = aalloc<int>(*A, cap, err);
  T.mptr = aalloc<int>(*A, n + 1, err);
  T.ment = aalloc<int>(*A, mcap, err);
  T.mfill = aalloc<int>(*A, n, err);
  T.acnt = aalloc<int>(*A, n, err);
  T.afill = aalloc<int>(*A, n, err);
  T.aptr = aalloc<int>(*A, n + 1, err);
  T.aent = aalloc<int>(*A, kp * n, err);
  T.acol = aalloc<int>(*A, (size_t)T.capT * n, err);
  T.aval = aalloc<double>(*A, (size_t)T.capT * n, err);
  T.scan_tot = aalloc<int>(*A, cap / ATB + 2, err);
  T.flag = aalloc<int>(*A, 1, err);
  AdjVec& a = A->a;
  a.Ru = aalloc<double>(*A, n, err);
  a.Rv = aalloc<double>(*A, n, err);
  a.Rth = aalloc<double>(*A, n, err);
  a.Nu = aalloc<double>(*A, n, err);
  a.Nv = aalloc<double>(*A, n, err);
  a.Nth = aalloc<double>(*A, n, err);
  for (int q = 0; q < 4; ++q) {
    a.Rtau[q] = aalloc<double>(*A, n, err);
    a.Ntau[q] = aalloc<double>(*A, n, err);
    a.at[q] = aalloc<double>(*A, n, err);
    a.Gb[q] = aalloc<double>(*A, n, err);
    a.mt[q] = aalloc<double>(*A, mcap, err);
  }
  a.aus = aalloc<double>(*A, cap, err);
  a.avs = aalloc<double>(*A, cap, err);
  a.aP = aalloc<double>(*A, cap, err);
  a.abx = aalloc<double>(*A, n, err);
  a.aby = aalloc<double>(*A, n, err);
  a.lam = aalloc<double>(*A, n, err);
  a.q = aalloc<double>(*A, n, err);
  a.s1 = aalloc<double>(*A, n, err);
  a.s2 = aalloc<double>(*A, n, err);
  a.st = aalloc<double>(*A, n, err);
  a.mu = aalloc<double>(*A, mcap, err);
  a.mv = aalloc<double>(*A, mcap, err);
  a.mth = aalloc<double>(*A, mcap, err);
  a.part = aalloc<double>(*A, n / TPB + 2, err);
  A->sums = aalloc<double>(*A, 2 * (size_t)max_steps + 2, err);
  if (x.precision == VEBI_PREC_MIXED) {
    A->aval32 = aalloc<float>(*A, (size_t)T.capT * n, err);
    A->arow = aalloc<double>(*A, n, err);
  }
  A->tmp1 = aalloc<double>(*A, 4, err);
  if (err != cudaSuccess) {
    for (void* p : A->allocs) cudaFree(p);
    delete A;
    cudaGetLastError();
    return afail(VEBI_ERR_CUDA, std::string("adjoint: device allocation failed: ") + cudaGetErrorString(err));
  }
  *out = A;
  return VEBI_OK;
}

void adjoint_destroy(Adjoint* A) {
  if (!A) return;
  if (A->x) cudaStreamSynchronize(A->x->st);
  for (void* p : A->allocs) cudaFree(p);
  delete A;
}

static void save_state(Adjoint& A, int ck) {
  Ctx& x = *A.x;
  const size_t n = A.n, B = sizeof(double) * n;
  double* base = A.ckpt + (size_t)ck * CK_PLANES * n;
  const double* src[CK_PLANES] = {x.d.ux, x.d.uy, x.d.th, x.d.tau[0], x.d.tau[1], x.d.tau[2], x.d.tau[3],
                                  x.d.trace_conf, x.d.rx, x.d.ry};
  for (int q = 0; q < CK_PLANES; ++q) cudaMemcpyAsync(base + q * n, src[q], B, cudaMemcpyDeviceToDevice, x.st);
  cudaMemcpyAsync(A.ckpt_inbin + (size_t)ck * n, x.d.inbin, n, cudaMemcpyDeviceToDevice, x.st);
}
static void load_state(Adjoint& A, int ck) {
  Ctx& x = *A.x;
  const size_t n = A.n, B = sizeof(double) * n;
  const double* base = A.ckpt + (size_t)ck * CK_PLANES * n;
  double* dst[CK_PLANES] = {x.d.ux, x.d.uy, x.d.th, x.d.tau[0], x.d.tau[1], x.d.tau[2], x.d.tau[3],
                            x.d.trace_conf, x.d.rx, x.d.ry};
  for (int q = 0; q < CK_PLANES; ++q) cudaMemcpyAsync(dst[q], base + q * n, B, cudaMemcpyDeviceToDevice, x.st);
  cudaMemcpyAsync(x.d.inbin, A.ckpt_inbin + (size_t)ck * n, n, cudaMemcpyDeviceToDevice, x.st);
}

int adjoint_record(Adjoint& A, int nsteps, vebi_step_stats* last) {
  Ctx& x = *A.x;
  if (nsteps < 1 || nsteps > A.max_steps) return afail(VEBI_ERR_ARG, "adjoint: nsteps outside 1..max_steps");
  if (!x.have_state) return afail(VEBI_ERR_ARG, "adjoint: no state uploaded");
  A.nsteps = 0;
  A.nseg = (nsteps + A.K - 1) / A.K;
  for (int s = 0; s < nsteps; ++s) {
    if (s % A.K == 0) save_state(A, s / A.K);
    x.rec_geo = A.geo + (size_t)s * (2 * A.n + 1);
    const int st = run_one_step(x, last);
    x.rec_geo = nullptr;
    if (st) return st;
    cudaMemcpyAsync(A.pres + (size_t)s * A.n, x.d.p, sizeof(double) * A.n, cudaMemcpyDeviceToDevice, x.st);
  }
  A.nsteps = nsteps;
  return VEBI_OK;
}

int adjoint_replay(Adjoint& A, int nsteps, vebi_step_stats* last) {
  Ctx& x = *A.x;
  if (nsteps < 1 || nsteps > A.nsteps) return afail(VEBI_ERR_ARG, "adjoint: nsteps outside the recorded window");
  for (int s = 0; s < nsteps; ++s) {
    x.rep_geo = A.geo + (size_t)s * (2 * A.n + 1);
    const int st = run_one_step(x, last);
    x.rep_geo = nullptr;
    if (st) return st;
  }
  return VEBI_OK;
}

int adjoint_restore(Adjoint& A, int step) {
  if (step < 0 || step >= A.nsteps || step % A.K) return afail(VEBI_ERR_ARG, "adjoint: not a checkpointed step");
  load_state(A, step / A.K);
  cudaStreamSynchronize(A.x->st);
  return VEBI_OK;
}

// replay step s from the context's current fields and copy what its VJP needs into slot t
static int tape_step(Adjoint& A, int s, Tape& t) {
  Ctx& x = *A.x;
  const size_t n = A.n, B = sizeof(double) * n;
  for (int q = 0; q < 4; ++q) cudaMemcpyAsync(t.tau0[q], x.d.tau[q], B, cudaMemcpyDeviceToDevice, x.st);
  vebi_step_stats st{};
  const double* geo = A.geo + (size_t)s * (2 * A.n + 1);
  x.rep_geo = geo;
  x.rep_p = A.pres + (size_t)s * n;
  int rc = run_one_step(x, &st);
  x.rep_geo = nullptr;
  x.rep_p = nullptr;
  if (rc) return rc;
  t.nm = st.nmirror;
  t.kmax = st.maxneighbours < (int)A.kp ? st.maxneighbours : (int)A.kp;
  t.dt = st.dt;
  const size_t ell = (size_t)t.kmax * n;
  cudaMemcpyAsync(t.cnt, x.d.ij_count, sizeof(int) * n, cudaMemcpyDeviceToDevice, x.st);
  cudaMemcpyAsync(t.link, x.d.ij_link, sizeof(int) * ell, cudaMemcpyDeviceToDevice, x.st);
  cudaMemcpyAsync(t.pcol, x.d.ppe_col, sizeof(int) * ell, cudaMemcpyDeviceToDevice, x.st);
  const bool mixed = x.precision == VEBI_PREC_MIXED;
  if (mixed) {  // the FP32 weights and correction matrices the step used (the FP64 ones are not computed)
    const long long ecount = (long long)ell;
    const int g = grid_for(ecount > (long long)n ? ecount : (long long)n);
    k_adj_widen<<<g < 4096 ? g : 4096, TPB, 0, x.st>>>(x.d, t, ecount, (int)n);
    x.launches++;
  } else {
    cudaMemcpyAsync(t.wgx, x.d.wGx, sizeof(double) * ell, cudaMemcpyDeviceToDevice, x.st);
    cudaMemcpyAsync(t.wgy, x.d.wGy, sizeof(double) * ell, cudaMemcpyDeviceToDevice, x.st);
    cudaMemcpyAsync(t.wl, x.d.wL, sizeof(double) * ell, cudaMemcpyDeviceToDevice, x.st);
  }
  // the PPE matrix is FP64 in both contexts (a mixed step assembles it from its FP32 weights)
  cudaMemcpyAsync(t.pval, x.d.ppe_val, sizeof(double) * ell, cudaMemcpyDeviceToDevice, x.st);
  cudaMemcpyAsync(t.pdiag, x.d.ppe_diag, B, cudaMemcpyDeviceToDevice, x.st);
  const size_t np = n + (size_t)t.nm;
  for (int q = 0; q < 4; ++q) {
    if (!mixed) cudaMemcpyAsync(t.kg[q], x.d.kgcm[q], B, cudaMemcpyDeviceToDevice, x.st);
    cudaMemcpyAsync(t.G[q], x.d.grad[q], B, cudaMemcpyDeviceToDevice, x.st);
    cudaMemcpyAsync(t.tau1[q], x.d.tau[q], sizeof(double) * np, cudaMemcpyDeviceToDevice, x.st);
  }
  if (t.nm > 0) {
    k_adj_mirror_coefs<<<grid_for(t.nm), TPB, 0, x.st>>>(x.c, x.d, geo, t.mco, t.irel);
    x.launches++;
  }
  return VEBI_OK;
}

static void scan_into(Ctx& x, int len, const int* v, int* ptr, int* tot) {
  const int nb = (len + ATB - 1) / ATB > 0 ? (len + ATB - 1) / ATB : 1;
  k_adj_scan_blocks<<<nb, TPB, 0, x.st>>>(len, v, tot);
  k_adj_scan_totals<<<1, 32, 0, x.st>>>(nb, tot);
  k_adj_scan_apply<<<nb, TPB, 0, x.st>>>(len, v, tot, ptr);
  x.launches += 3;
}

// the transposed pair list, the mirrors of every parent and A^T of slot t
static void build_transposes(Adjoint& A, const Tape& t) {
  Ctx& x = *A.x;
  Trans& T = A.T;
  const int n = (int)A.n, np = n + t.nm;
  cudaMemsetAsync(T.tfill, 0, sizeof(int) * np, x.st);
  k_adj_count_pairs<<<grid_for(n), TPB, 0, x.st>>>(n, t.cnt, t.link, T.tfill);
  scan_into(x, np, T.tfill, T.tptr, T.scan_tot);
  cudaMemsetAsync(T.tfill, 0, sizeof(int) * np, x.st);
  k_adj_fill_pairs<<<grid_for(n), TPB, 0, x.st>>>(n, t.cnt, t.link, T.tptr, T.tfill, T.tent);
  k_adj_sort_segments<<<sort_grid(np), TPB, 0, x.st>>>(np, T.tptr, T.tent);
  cudaMemsetAsync(T.mfill, 0, sizeof(int) * n, x.st);
  if (t.nm > 0) k_adj_count_mirrors<<<grid_for(t.nm), TPB, 0, x.st>>>(t.nm, t.irel, T.mfill);
  scan_into(x, n, T.mfill, T.mptr, T.scan_tot);
  cudaMemsetAsync(T.mfill, 0, sizeof(int) * n, x.st);
  if (t.nm > 0) k_adj_fill_mirrors<<<grid_for(t.nm), TPB, 0, x.st>>>(t.nm, t.irel, T.mptr, T.mfill, T.ment);
  k_adj_sort_segments<<<sort_grid(n), TPB, 0, x.st>>>(n, T.mptr, T.ment);
  cudaMemsetAsync(T.afill, 0, sizeof(int) * n, x.st);
  k_adj_count_cols<<<grid_for(n), TPB, 0, x.st>>>(n, t.cnt, t.pcol, t.pval, T.afill);
  scan_into(x, n, T.afill, T.aptr, T.scan_tot);
  cudaMemsetAsync(T.afill, 0, sizeof(int) * n, x.st);
  k_adj_fill_cols<<<grid_for(n), TPB, 0, x.st>>>(n, t.cnt, t.pcol, t.pval, T.aptr, T.afill, T.aent);
  k_adj_sort_segments<<<sort_grid(n), TPB, 0, x.st>>>(n, T.aptr, T.aent);
  k_adj_write_at<<<grid_for(n), TPB, 0, x.st>>>(n, T.capT, T.aptr, T.aent, t.pval, T.acnt, T.acol, T.aval, T.flag);
  x.launches += 10 + (t.nm > 0 ? 2 : 0);
}

// mean of v[0..n) removed into out
static void project_mean(Adjoint& A, const double* v, double* out) {
  Ctx& x = *A.x;
  const int n = (int)A.n, g = grid_for(n);
  k_adj_block_sum<<<g, TPB, 0, x.st>>>(n, v, A.a.part);
  k_adj_final_sum<<<1, TPB, 0, x.st>>>(g, A.a.part, A.tmp1);
  k_adj_sub_mean<<<g, TPB, 0, x.st>>>(n, A.tmp1, v, out);
  x.launches += 3;
}

// one step of the reverse sweep: R (adjoint of state s+1) -> R (adjoint of state s)
static int vjp_step(Adjoint& A, int s, const Tape& t) {
  Ctx& x = *A.x;
  const Consts& c = x.c;
  AdjVec& a = A.a;
  Trans& T = A.T;
  const int n = (int)A.n, np = n + t.nm, g = grid_for(n), gp = grid_for(np);
  const int ve = c.const_mod != 1 ? 1 : 0;
  const size_t B = sizeof(double) * (size_t)n;
  cudaMemsetAsync(T.flag, 0, sizeof(int), x.st);
  build_transposes(A, t);
  cudaMemsetAsync(a.Nu, 0, B, x.st);
  cudaMemsetAsync(a.Nv, 0, B, x.st);
  cudaMemsetAsync(a.Nth, 0, B, x.st);
  for (int q = 0; q < 4; ++q) cudaMemsetAsync(a.Ntau[q], 0, B, x.st);
  // final update and pressure gradient
  k_adj_final<<<g, TPB, 0, x.st>>>(c, t, a);
  k_adj_gather_P<<<gp, TPB, 0, x.st>>>(c, t, T, a, np);
  k_adj_push<<<g, TPB, 0, x.st>>>(c, T, t.mco, -1, a.aP, 1, a.aP, nullptr, nullptr);
  // PPE: A^T lambda = P-bar with its mean removed (P has zero mean)
  project_mean(A, a.aP, a.aP);
  // The solver's convergence test turns absolute below a first residual norm of 1e-6 (the
  // reference's rule for its pressure); adjoint right-hand sides can be any size, so the
  // system is solved for the right-hand side scaled to unit RMS and lambda is scaled back.
  k_adj_block_sumsq<<<g, TPB, 0, x.st>>>(n, a.aP, a.part);
  k_adj_final_sum<<<1, TPB, 0, x.st>>>(g, a.part, A.tmp1 + 1);
  k_adj_scale<<<g, TPB, 0, x.st>>>(n, A.tmp1 + 1, a.aP, 1);
  x.launches += 6;
  if (x.precision == VEBI_PREC_MIXED) {
    // the context's own mixed solver (FP64 recurrences, FP32 SpMV in the difference form, with
    // or without its multigrid) on A^T: FP32 values and FP64 row sums of A^T first
    k_adj_at32<<<g, TPB, 0, x.st>>>(n, T.acnt, T.aval, t.pdiag, A.aval32, A.arow);
    x.launches++;
    Dev keep = x.d;
    x.d.ppe_col = T.acol;
    x.d.ppe_val = T.aval;
    x.d.ppe_val32 = A.aval32;
    x.d.rowsum = A.arow;
    x.d.ij_count = T.acnt;
    x.d.ppe_diag = t.pdiag;
    x.d.ppe_B = a.aP;
    x.d.p = a.lam;
    launch_ppe_mixed_solve(x);
    x.d = keep;
  } else if (c.precond) {
    // the context's multigrid on A^T: the same set-up and solver read the transposed arrays
    // (piecewise-constant aggregation: the Galerkin levels of A^T are those of A transposed)
    Dev keep = x.d;
    x.d.ppe_col = T.acol;
    x.d.ppe_val = T.aval;
    x.d.ij_count = T.acnt;
    x.d.ppe_diag = t.pdiag;
    x.d.ppe_B = a.aP;
    x.d.p = a.lam;
    launch_ppe_mg(x);
    x.d = keep;
  } else {
    const Dev& d = x.d;
    BiArgs b{d.bx, d.br, d.brb, d.bv, d.bp, d.bpi, d.bs, d.bsi, d.bt, d.bM, d.partials, a.lam,
             a.aP, t.pdiag, T.aval, T.acol, T.acnt, d.s, (long long)n, n, c.itermax, c.tol, 0};
    launch_bicgstab_on(x, b, true);
  }
  k_adj_scale<<<g, TPB, 0, x.st>>>(n, A.tmp1 + 1, a.lam, -1);
  x.launches++;
  project_mean(A, a.lam, a.lam);
  // right-hand side (mean removal's adjoint is the projection above)
  k_adj_rhs_rows<<<g, TPB, 0, x.st>>>(c, t, a);
  k_adj_gather_us<<<gp, TPB, 0, x.st>>>(c, t, T, a, np);
  k_adj_push<<<g, TPB, 0, x.st>>>(c, T, t.mco, 2, a.aus, 1, a.aus, a.avs, a.avs);
  // predictor
  k_adj_pred_rows<<<g, TPB, 0, x.st>>>(c, t, a, ve);
  k_adj_gather_pred<<<gp, TPB, 0, x.st>>>(c, t, T, a, np, ve);
  if (ve) {
    const double inv_cp = c.coeff_polymeric != 0.0 ? 1.0 / c.coeff_polymeric : 0.0;
    k_adj_dcp<<<g, TPB, 0, x.st>>>(c, t, a, np, inv_cp);
    k_adj_final_sum<<<1, TPB, 0, x.st>>>(g, a.part, A.sums + 2 * (size_t)s);
    x.launches += 2;
  }
  k_adj_push<<<g, TPB, 0, x.st>>>(c, T, t.mco, 0, a.mu, 0, a.Nu, a.mv, a.Nv);
  k_adj_push<<<g, TPB, 0, x.st>>>(c, T, t.mco, 1, a.mth, 0, a.Nth, nullptr, nullptr);
  if (ve) k_adj_push_tau<<<g, TPB, 0, x.st>>>(c, T, t.mco, a);
  // log-conformation
  k_adj_logconf<<<g, TPB, 0, x.st>>>(c, t, a, relax_e1(c, t.dt), ve);
  k_adj_final_sum<<<1, TPB, 0, x.st>>>(g, a.part, A.sums + 2 * (size_t)s + 1);
  // velocity gradients
  if (ve) {
    k_adj_grad_rows<<<g, TPB, 0, x.st>>>(c, t, a);
    k_adj_gather_grad<<<gp, TPB, 0, x.st>>>(c, t, T, a, np);
    k_adj_push<<<g, TPB, 0, x.st>>>(c, T, t.mco, 0, a.mu, 0, a.Nu, a.mv, a.Nv);
  }
  x.launches += 11;
  // state adjoint of step s
  std::swap(a.Ru, a.Nu);
  std::swap(a.Rv, a.Nv);
  std::swap(a.Rth, a.Nth);
  for (int q = 0; q < 4; ++q) std::swap(a.Rtau[q], a.Ntau[q]);
  int flag = 0;
  cudaError_t e = cudaMemcpyAsync(&flag, T.flag, sizeof(int), cudaMemcpyDeviceToHost, x.st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(x.st);
  if (e != cudaSuccess) return afail(VEBI_ERR_CUDA, std::string("adjoint: ") + cudaGetErrorString(e));
  if (flag) return afail(VEBI_ERR_NEIGH_CAPACITY, "adjoint: a column of A^T holds more than 2*nplink entries");
  int err = 0, its = 0;
  cudaMemcpy(&err, &x.d.s->error, sizeof(int), cudaMemcpyDeviceToHost);
  cudaMemcpy(&its, &x.d.s->ls_iters, sizeof(int), cudaMemcpyDeviceToHost);
  if (err) return afail(err, "adjoint: device error in the transposed solve");
  A.ls_iters_total += its;
  return VEBI_OK;
}

int adjoint_reverse(Adjoint& A, const double* seed_u, const double* seed_theta, const double* seed_tau, int ld,
                    double* grad_u, double* grad_theta, double* grad_tau, double* grad_wi, int* ls_iters) {
  Ctx& x = *A.x;
  if (A.nsteps < 1) return afail(VEBI_ERR_ARG, "adjoint: record a window first");
  const size_t n = A.n, B = sizeof(double) * n;
  if (ld < (int)n) return afail(VEBI_ERR_ARG, "adjoint: ld < npfb");
  AdjVec& a = A.a;
  cudaMemsetAsync(a.Ru, 0, B, x.st);
  cudaMemsetAsync(a.Rv, 0, B, x.st);
  cudaMemsetAsync(a.Rth, 0, B, x.st);
  for (int q = 0; q < 4; ++q) cudaMemsetAsync(a.Rtau[q], 0, B, x.st);
  if (seed_u) {
    cudaMemcpyAsync(a.Ru, seed_u, B, cudaMemcpyHostToDevice, x.st);
    cudaMemcpyAsync(a.Rv, seed_u + ld, B, cudaMemcpyHostToDevice, x.st);
  }
  if (seed_theta) cudaMemcpyAsync(a.Rth, seed_theta, B, cudaMemcpyHostToDevice, x.st);
  if (seed_tau)
    for (int q = 0; q < 4; ++q) cudaMemcpyAsync(a.Rtau[q], seed_tau + (size_t)q * ld, B, cudaMemcpyHostToDevice, x.st);
  cudaMemsetAsync(A.sums, 0, sizeof(double) * 2 * (size_t)A.nsteps, x.st);
  A.ls_iters_total = 0;
  for (int seg = A.nseg - 1; seg >= 0; --seg) {
    const int s0 = seg * A.K, s1 = std::min(A.nsteps, s0 + A.K);
    load_state(A, seg);
    for (int s = s0; s < s1; ++s) {
      const int rc = tape_step(A, s, A.tape[s - s0]);
      if (rc) return rc;
    }
    for (int s = s1 - 1; s >= s0; --s) {
      const int rc = vjp_step(A, s, A.tape[s - s0]);
      if (rc) return rc;
    }
  }
  // outputs
  if (grad_u) {
    cudaMemcpyAsync(grad_u, a.Ru, B, cudaMemcpyDeviceToHost, x.st);
    cudaMemcpyAsync(grad_u + ld, a.Rv, B, cudaMemcpyDeviceToHost, x.st);
  }
  if (grad_theta) cudaMemcpyAsync(grad_theta, a.Rth, B, cudaMemcpyDeviceToHost, x.st);
  if (grad_tau)
    for (int q = 0; q < 4; ++q) cudaMemcpyAsync(grad_tau + (size_t)q * ld, a.Rtau[q], B, cudaMemcpyDeviceToHost, x.st);
  std::vector<double> sums(2 * (size_t)A.nsteps), dts(A.nsteps);
  cudaMemcpyAsync(sums.data(), A.sums, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost, x.st);
  for (int s = 0; s < A.nsteps; ++s)
    cudaMemcpyAsync(&dts[s], A.geo + (size_t)s * (2 * n + 1) + 2 * n, sizeof(double), cudaMemcpyDeviceToHost, x.st);
  cudaError_t e = cudaStreamSynchronize(x.st);
  if (e != cudaSuccess) return afail(VEBI_ERR_CUDA, std::string("adjoint: ") + cudaGetErrorString(e));
  if (grad_wi) {
    const Consts& c = x.c;
    double g = 0.0;
    if (c.const_mod != 1) {
      for (int s = 0; s < A.nsteps; ++s) {
        const double e1 = relax_e1(c, dts[s]);
        g += sums[2 * s] * (-c.coeff_polymeric / c.Wi) + sums[2 * s + 1] * (e1 * dts[s] / (c.Wi * c.Wi));
      }
    }
    *grad_wi = g;
  }
  if (ls_iters) *ls_iters = A.ls_iters_total;
  return VEBI_OK;
}

}  // namespace vebi

// ------------------------------------------------------------------------------- C entry points
struct vebi_adjoint {
  vebi::Adjoint* a;
};

extern "C" {

int vebi_adjoint_create(vebi_ctx* ctx, int32_t max_steps, int32_t checkpoint_every, vebi_adjoint** out) {
  vebi::Ctx* x = vebi::ctx_of(ctx);
  if (!x || !out) return vebi::afail(VEBI_ERR_ARG, "adjoint: null context or output");
  vebi::Adjoint* A = nullptr;
  const int st = vebi::adjoint_create(*x, max_steps, checkpoint_every, &A);
  if (st) return st;
  *out = new vebi_adjoint{A};
  return VEBI_OK;
}

int vebi_adjoint_record(vebi_adjoint* a, int32_t nsteps, vebi_step_stats* last) {
  if (!a) return vebi::afail(VEBI_ERR_ARG, "adjoint: null handle");
  return vebi::adjoint_record(*a->a, nsteps, last);
}

int vebi_adjoint_replay(vebi_adjoint* a, int32_t nsteps, vebi_step_stats* last) {
  if (!a) return vebi::afail(VEBI_ERR_ARG, "adjoint: null handle");
  return vebi::adjoint_replay(*a->a, nsteps, last);
}

int vebi_adjoint_restore(vebi_adjoint* a, int32_t step) {
  if (!a) return vebi::afail(VEBI_ERR_ARG, "adjoint: null handle");
  return vebi::adjoint_restore(*a->a, step);
}

int vebi_adjoint_reverse(vebi_adjoint* a, const double* seed_u, const double* seed_theta, const double* seed_tau,
                         int32_t ld, double* grad_u, double* grad_theta, double* grad_tau, double* grad_wi,
                         int32_t* ls_iters) {
  if (!a) return vebi::afail(VEBI_ERR_ARG, "adjoint: null handle");
  return vebi::adjoint_reverse(*a->a, seed_u, seed_theta, seed_tau, ld, grad_u, grad_theta, grad_tau, grad_wi,
                               ls_iters);
}

int vebi_adjoint_destroy(vebi_adjoint* a) {
  if (!a) return VEBI_OK;
  vebi::adjoint_destroy(a->a);
  delete a;
  return VEBI_OK;
}

}  // extern "C"
