// vebi_common.cuh -- shared device structures and helpers of the GB300 step library.
//
// The whole library is compiled with --fmad=false: every expression below is evaluated as
// written, one IEEE binary64 operation at a time, as gfortran evaluates the reference on
// x86-64.  Where a kernel wants fused multiply-adds for speed it calls fma() explicitly.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vebi.h"

namespace vebi {

constexpr double PI = 3.14159265358979323846;  // common_parameter.F90:12
constexpr int TPB = 256;                         // threads per block of per-particle kernels

// ---------------------------------------------------------------------------------------------
// Run constants, passed by value to every kernel (lives in the kernel-parameter bank).
struct Consts {
  // kernel constants of getdata (input.F90:164-172)
  double h, dx, dv, sup_size, sup_size_2, uno_sup_size, ad_7, ad_7h, eta2, eta_small, oneoverh;
  double x_mint, x_maxt, y_mint, y_maxt;           // padded box (sph2D_incom.F90:64-67)
  double Ra, Pr, El, beta, eps_ptt, Wi;
  double bf[2];
  double dt_coef_cfl, dt_coef_visc, dt_visc;
  double coeff_solvent, coeff_polymeric, coeff_theta;
  double wab1;                                      // Wab(dx/h) of shifting_forces
  double cell_size;                                 // 1/uno_sup_size: edge of a cell
  double tol;
  // boundary framework (IBOUND)
  double b_node[VEBI_MAX_PATCHES][2], b_edge[VEBI_MAX_PATCHES][2];
  double b_vel[VEBI_MAX_PATCHES], b_thermal[VEBI_MAX_PATCHES];
  double b_elen[VEBI_MAX_PATCHES];                  // sqrt(dot(b_edge,b_edge))
  // FP32 prefilters: bound_dist ~ bl_a x + bl_b y + bl_c; near_band = sup + dx/10 + 4e-6 x the
  // box extent, a margin far above the FP32 rounding of that expression
  float bl_a[VEBI_MAX_PATCHES], bl_b[VEBI_MAX_PATCHES], bl_c[VEBI_MAX_PATCHES];
  float near_band;
  double b_corner_angle[VEBI_MAX_PATCHES];          // check_boundaries (input.F90:246-270)
  double b_rot[VEBI_MAX_PATCHES][4];                // angle_between_patches(ib, parent), row-major
  double c_centre[VEBI_MAX_CIRCLES][2], c_radius[VEBI_MAX_CIRCLES], c_omega[VEBI_MAX_CIRCLES];
  double c_vel[VEBI_MAX_CIRCLES][2], c_thermal[VEBI_MAX_CIRCLES];
  int b_type[VEBI_MAX_PATCHES], b_pp[VEBI_MAX_PATCHES];  // b_pp: 0-based parent patch
  int nb, ncirc;
  int ncx, ncy, nct;
  int npfb, nbS, cap, mcap, nplink;
  int open_domain, shift_coeff, const_mod, itermax;
  int correct_velocity;                             // run correct_velocity (off in the reference)
  int warm_start;                                   // PPE starts from the previous P (opt-in)
  int precond;                                      // 1: multigrid-preconditioned PPE (opt-in)
  double u_limit;                                   // > 0: velocity bound of the divergence guard
};

// Scalars that change during a step; they live in device memory so no step needs a host sync.
struct Scal {
  double dt;
  unsigned long long umax_bits;      // max |u| over fluid (set_time_step), as ordered bits
  unsigned long long maxU_bits;      // max |u| over 1..npfb after binning (new_fick_shift)
  unsigned long long absu_bits, absv_bits, absp_bits;  // TIME-file maxima
  double rhs_mean;
  double ls_residual;
  double rms_u;
  double circle_fx, circle_fy;       // force of the fluid on the circles (k_circle_force)
  int nmirror;                       // mirror counter `imp`
  int np;
  int n_inbin;
  int n_escapees;
  int maxneigh;
  int ls_iters;
  int warnings;
  int error;
  int sel_base;                      // mirror offset of the current ordered-select stage
  int n_cand;                        // particles in cand (candidates of the mirror stages)
  int sel_total;
  int imp_temp;                      // mirror count snapshot for wall-periodic corners
  int bar_count;                     // grid barrier state of the PPE kernel
  unsigned int bar_gen;
  int refine_iters;
  int ls_iters_total;                // summed over the steps of one vebi_run_steps call
  int first_error;                   // first failing status since the last upload (sticky)
  int mg_fail;                       // multigrid set-up overflowed a coarse row: solve without it
  int n_near_pole;                   // particles whose conformation eigenvalues are < 1e-7 apart
  int n_near_pole_total;             // the same summed over the steps of one vebi_run_steps call
};

// multigrid preconditioner (opt-in): coarse-row capacity, coarsest size, level cap, levels run
// by one block, coarsest sweeps, Jacobi damping, coarse-correction scaling
constexpr int MG_SLOTS = 24;
constexpr int MG_ROW_SLOTS = 16;
constexpr int MG_COARSEST = 32;
constexpr int MG_MAX_LEVELS = 12;
constexpr int MG_BLOCK_ROWS = 2048;
constexpr int MG_SWEEPS = 16;
constexpr double MG_OMEGA = 0.9;
constexpr double MG_GAMMA = 1.8;

// One coarse level of the multigrid preconditioner: the cell grid (level 1) or a 2x2
// agglomeration of the level below, as a gx x gy grid of aggregates; its Galerkin matrix in
// ELL form (off-diagonal slots [t][c], stride n) with the diagonal apart; work vectors.
struct MgLevel {
  int n, gx, gy;
  int* cnt;
  int* col;
  double *val, *diag, *dinv;
  double *x, *b, *r;
};

// Device arrays of one context.  Particle fields have capacity cap = npfb + mcap and are
// indexed 0..np-1 with mirrors at npfb..np-1.  Pair arrays are ELL [k][i], stride npfb.
struct Dev {
  Scal* s;
  double *rx, *ry, *ux, *uy, *th;            // current buffers
  double *rx2, *ry2, *ux2, *uy2, *th2;       // second buffers (double buffering)
  double *r0x, *r0y, *u0x, *u0y;
  double *p;
  double *tau[4];                            // (1,1),(2,1),(1,2),(2,2)
  double *trace_conf, *a_out, *vort;
  int *n_surf;
  uint8_t* inbin;
  int *irel, *vrel;                          // indexed by particle (only mirrors meaningful)
  double* dP_mp;
  // cells
  int *cellpart, *cell_cnt, *cell_start, *cell_fill, *ip;
  int *scan_part;
  // ordered select scratch
  int* sel_blk;
  int *cand, *cand_blk;                      // particles near a boundary or circle, ascending
  // pairs
  int *ij_count, *ij_link;
  double *wGx, *wGy, *wL;
  double *kgcm[4];                           // (1,1),(2,1),(1,2),(2,2)
  double *grad[6];                           // du/dx du/dy dv/dx dv/dy dth/dx dth/dy (np)
  double *gradCx, *gradCy, *ushx, *ushy;
  // open domain
  double *conc, *div_r, *surf_nx, *surf_ny, *ppe_smooth, *beta_div_r;
  // PPE
  double *ppe_B, *ppe_diag, *ppe_val;
  int* ppe_col;
  double *bx, *br, *brb, *bv, *bp, *bpi, *bs, *bsi, *bt, *bM;  // BiCGSTAB vectors
  double* partials;                          // block partial sums
  double* red;                               // small reduction scratch
  double *gpx, *gpy;
  // mixed precision
  float* ppe_val32;                          // FP32 off-diagonal values
  double* rowsum;                            // FP64 row sums of the PPE matrix
  float2 *pi2, *si2;                         // p_inv, s_inv as FP32 (hi, lo) pairs
  // mixed precision: particle fields (fluid, walls and mirrors) as FP32 (hi, lo) pairs, so a
  // pair difference f_j - f_i = (hi_j - hi_i) + (lo_j - lo_i) is formed in FP32 arithmetic
  // with the accuracy of the FP64 difference rounded to FP32
  float2 *hl_u[2], *hl_th, *hl_tau[4], *hl_us[2], *hl_p;
  float4* pk;                                // FP32 offset to the cell origin + cell coords
  float4* pko;                               // the same offsets in cell-list (ip) order, with the
                                             // particle index (bits of .z); .w unused
  float *wGx32, *wGy32, *wL32;               // FP32 pair weights (ELL)
  float* kgcm32[4];
};

// ---------------------------------------------------------------------------------------------
// small helpers
__device__ __forceinline__ double pw4(double x) { double x2 = x * x; return x2 * x2; }
__device__ __forceinline__ double pw5(double x) { double x2 = x * x; double x3 = x * x2; return x2 * x3; }

// quintic spline derivative `fac` (sphtools.F90:11-44)
__device__ __forceinline__ double fac(const Consts& c, double qq) {
  int isel = (int)floor(qq);
  if (isel == 0) {
    double q3 = 3.0 - qq, q2 = 2.0 - qq, q1 = 1.0 - qq;
    return c.ad_7h * (-5.0 * pw4(q3) + 30.0 * pw4(q2) - 75.0 * pw4(q1));
  } else if (isel == 1) {
    double q3 = 3.0 - qq, q2 = 2.0 - qq;
    return c.ad_7h * (-5.0 * pw4(q3) + 30.0 * pw4(q2));
  } else if (isel == 2) {
    double q3 = 3.0 - qq;
    return c.ad_7h * (-5.0 * pw4(q3));
  }
  return 0.0;
}
// quintic spline `Wab` (sphtools.F90:46-76)
__device__ __forceinline__ double wab(const Consts& c, double qq) {
  int isel = (int)floor(qq);
  if (isel == 0) {
    double q3 = 3.0 - qq, q2 = 2.0 - qq, q1 = 1.0 - qq;
    return c.ad_7 * (pw5(q3) - 6.0 * pw5(q2) + 15.0 * pw5(q1));
  } else if (isel == 1) {
    double q3 = 3.0 - qq, q2 = 2.0 - qq;
    return c.ad_7 * (pw5(q3) - 6.0 * pw5(q2));
  } else if (isel == 2) {
    return c.ad_7 * pw5(3.0 - qq);
  }
  return 0.0;
}

// signed distance of a point to patch ib (bound_dist, mirror_boundaries_mod.F90:447-462)
__device__ __forceinline__ double bound_dist(const Consts& c, double x, double y, int ib) {
  int ibp1 = (ib + 1) % c.nb;
  double p = c.b_edge[ib][1] * x - c.b_edge[ib][0] * y + c.b_node[ibp1][0] * c.b_node[ib][1] -
             c.b_node[ibp1][1] * c.b_node[ib][0];
  return -1.0 * p / c.b_elen[ib];
}
// unit normal of patch ib (bound_norm, :464-474)
__device__ __forceinline__ void bound_norm(const Consts& c, int ib, double& n1, double& n2) {
  n1 = -1.0 * c.b_edge[ib][1] / c.b_elen[ib];
  n2 = c.b_edge[ib][0] / c.b_elen[ib];
}
// position along patch ib given perp_dist and norm_be (position_along_patch, :476-491)
__device__ __forceinline__ double pos_along(const Consts& c, double x, double y, int ib, double perp,
                                            double n1, double n2) {
  if (fabs(c.b_edge[ib][0]) > fabs(c.b_edge[ib][1])) return (x - c.b_node[ib][0] - perp * n1) / c.b_edge[ib][0];
  return (y - c.b_node[ib][1] - perp * n2) / c.b_edge[ib][1];
}

// order-preserving max of non-negative doubles through their bit patterns
__device__ __forceinline__ void atomic_max_pos(unsigned long long* a, double v) {
  if (!(v >= 0.0)) return;  // NaN never wins
  atomicMax(a, (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ double bits_to_double(unsigned long long b) { return __longlong_as_double((long long)b); }

// the same maximum with one atomic per warp; every lane of the warp must call it
__device__ __forceinline__ void warp_max_pos(unsigned long long* a, double v) {
  unsigned long long b = (v >= 0.0) ? (unsigned long long)__double_as_longlong(v) : 0ull;
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long q = __shfl_xor_sync(0xffffffffu, b, o);
    b = q > b ? q : b;
  }
  if ((threadIdx.x & 31) == 0 && b) atomicMax(a, b);
}

__device__ __forceinline__ void set_error(Scal* s, int code) { atomicCAS(&s->error, 0, code); }

// deterministic block sum: fixed shuffle tree, warps combined in order by warp 0
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < NT / 32; ++i) r += sh[i];
    sh[NT / 32] = r;
  }
  __syncthreads();
  return sh[NT / 32];
}

// ---------------------------------------------------------------------------------------------
// FP32 <-> FP64 conversions on the integer pipe.  This GPU runs conversions on its FP64 pipe
// (2 lanes per clock per SM): measured, an FP32-to-FP64 conversion costs as much as an FP64
// add and an FP64-to-FP32 conversion about twice that.  Both are rebuilt here from the IEEE 754
// binary32/binary64 encodings for the normal range, bit for bit the results of the hardware
// conversions (round to nearest even), which handle the rest (zeros, subnormals, infinities,
// NaNs, results outside the binary32 normal range).  vebi_test_conversions checks them against
// the hardware on every class of input.
__device__ __forceinline__ double widen(float f) {  // == (double)f
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e - 1u < 254u) {  // normal binary32: rebias the exponent (+896), shift the mantissa by 29
    const unsigned long long b = ((unsigned long long)(u >> 31) << 63) | ((unsigned long long)(e + 896u) << 52) |
                                 ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)b);
  }
  return (double)f;
}

__device__ __forceinline__ float narrow(double d) {  // == (float)d
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if (e - 897u < 254u) {  // a binary32 normal exponent (a round-up may carry into infinity)
    const unsigned long long m = b & 0x000fffffffffffffull;
    unsigned r = ((e - 896u) << 23) | (unsigned)(m >> 29);
    const unsigned low = (unsigned)(m & 0x1fffffffull), half = 0x10000000u;
    r += (low > half || (low == half && (r & 1u))) ? 1u : 0u;  // the carry propagates into the exponent
    return __uint_as_float((unsigned)(b >> 63) << 31 | r);
  }
  return (float)d;
}

// ---------------------------------------------------------------------------------------------
// host side: per-context bookkeeping shared between translation units
struct Ctx;
void launch_advect_bin(Ctx& x);
void launch_mirrors(Ctx& x);
void launch_cells_neighbours(Ctx& x);
void launch_weights_surface_shift(Ctx& x);
void launch_predictor(Ctx& x);
void launch_ppe(Ctx& x);
void launch_final(Ctx& x, int secondary);

}  // namespace vebi
