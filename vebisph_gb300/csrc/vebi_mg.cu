// vebi_mg.cu -- opt-in multigrid preconditioner of the PPE BiCGSTAB (VEBI_PRECOND_MULTIGRID).
// No counterpart in the reference, which solves closed domains unpreconditioned
// (SPARSE_PBICGSTAB_nonull, linear_solver.F90:275-425, M = 1 at :318) and open domains with
// Jacobi (SPARSE_PBICGSTAB, :82-227).
//
// Hierarchy.  Level 1 aggregates the particles by the cell they sit in: the cell grid of
// cell_griddin.F90:13-24, whose cell lists the neighbour search built this step.  Each further
// level agglomerates 2x2 aggregates of the level below, until at most MG_COARSEST remain.
// Interpolation is piecewise constant, so a coarse matrix is the Galerkin product R A P: the
// sum of the couplings between two aggregates.  Coarse matrices are ELL with at most MG_SLOTS
// off-diagonal slots per row (the 3x3 neighbourhood plus partners across periodic boundaries);
// a row that needs more sets mg_fail, and that step solves without the preconditioner.
//
// V-cycle, one per preconditioning step: one damped Jacobi sweep (MG_OMEGA) from zero, the
// residual, restriction (the sum over each aggregate), the coarser levels, prolongation scaled
// by MG_GAMMA (over-correction for piecewise-constant interpolation) and, on the coarse levels,
// one post-smoothing sweep; the particle level is pre-smoothed only (two particle-level
// products per V-cycle cost more than the iterations they save).  The coarsest level takes
// MG_SWEEPS Jacobi sweeps.  Levels of at most MG_BLOCK_ROWS rows run in
// block 0 alone with block barriers.  Every sum runs in a fixed order.
//
// Solver.  BiCGSTAB with right preconditioning, in the persistent cooperative kernel of the
// unpreconditioned solver: the same recurrences, residual test and, for closed domains, mean
// removal.  The preconditioned directions are made mean-free, so the solution keeps the zero
// mean of the reference's iterates.  The V-cycle reads only its own rows of the vector it is
// applied to, so it needs no barrier before it.
#include "vebi_solver.cuh"

namespace vebi {

#define ELL(k, i) ((size_t)(k) * c.npfb + (i))

// ---------------------------------------------------------------- set-up (every step)
// add v to column `col` of a row's slot table of capacity CAP; false when the table is full
template <int CAP = MG_SLOTS>
__device__ __forceinline__ bool slot_add(int* tc, double* tv, int& m, int col, double v) {
  int t = 0;
  while (t < m && tc[t] != col) ++t;
  if (t == m) {
    if (m == CAP) return false;
    tc[m] = col;
    tv[m] = 0.0;
    ++m;
  }
  tv[t] += v;
  return true;
}

__device__ __forceinline__ void slot_store(const MgLevel& L, int row, const int* tc, const double* tv, int m,
                                           double dg) {
  for (int t = 0; t < m; ++t) {
    L.col[(size_t)t * L.n + row] = tc[t];
    L.val[(size_t)t * L.n + row] = tv[t];
  }
  L.cnt[row] = m;
  L.diag[row] = dg;
  L.dinv[row] = dg != 0.0 ? 1.0 / dg : 0.0;
}

// Level 1 in two passes.  Rows: one thread per PPE row sums the row by the cell of each
// column (its own cell first, with the diagonal) into MG_ROW_SLOTS (cell, value) pairs,
// [t][i] layout.  Cells: one thread per cell merges its particles' pairs in ascending particle
// order.  val32 (mixed precision) replaces the FP64 values when given.
//
// A row's columns lie in the 3x3 cells around its own, except the parents of mirrors across
// periodic boundaries.  The nine cells own + dy*ncx + dx are summed in shared memory by direct
// index (the key difference alone picks the slot: nine distinct keys, nine distinct slots);
// any other cell goes to a short searched list.  Each cell's sum runs in slot order, as a
// searched table's would; the pairs come out own cell first, then the 3x3 in key order, then
// the list.
//
// The same sums also go out by direction for the output pass of the V-cycle: rv9[k][i] for the
// eight directions q = 0..8 without the own cell (k = q, or q - 1 past it), zero where the row
// has no column, and rx[i] = (first list slot) | (pair count << 8) | (used directions << 16).
// The output pass then computes every gather address from the row's own cell, without a
// dependent load of the pair's cell.  With val32 (mixed precision) the direction values are
// FP32, rv9 read as float [8][npfb].
__global__ void __launch_bounds__(TPB) k_mg_rows(Consts c, Dev d, const float* __restrict__ val32,
                                                 int* __restrict__ ragg, double* __restrict__ rval,
                                                 int* __restrict__ rcnt, double* __restrict__ rv9,
                                                 int* __restrict__ rx) {
  __shared__ double nb9[9][TPB];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  const int own = d.cellpart[i];
  if (own < 0) {  // a binned particle belongs to no cell
    rcnt[i] = 0;
    rx[i] = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (val32) ((float*)rv9)[(size_t)k * c.npfb + i] = 0.f;
      else rv9[(size_t)k * c.npfb + i] = 0.0;
    }
    return;
  }
  double* acc = &nb9[0][threadIdx.x];  // slot q at acc[q * TPB]
#pragma unroll
  for (int q = 0; q < 9; ++q) acc[q * TPB] = 0.0;
  acc[4 * TPB] = d.ppe_diag[i];
  unsigned used = 1u << 4;
  int tc[MG_ROW_SLOTS - 9];
  double tv[MG_ROW_SLOTS - 9];
  int m = 0;
  bool ok = true;
  const int ncx = c.ncx;
  const int cnt = d.ij_count[i];
  for (int k = 0; k < cnt; ++k) {
    const int a = d.cellpart[d.ppe_col[ELL(k, i)]];
    const double v = val32 ? widen(val32[ELL(k, i)]) : d.ppe_val[ELL(k, i)];
    if (a < 0) continue;
    const int del = a - own;
    const int r = del + ncx + 1;  // row dy=-1 at 0..2, dy=0 at ncx..ncx+2, dy=+1 at 2ncx..2ncx+2
    int q = -1;
    if (r >= 0 && r <= 2) q = r;
    else if (r >= ncx && r <= ncx + 2) q = 3 + r - ncx;
    else if (r >= 2 * ncx && r <= 2 * ncx + 2) q = 6 + r - 2 * ncx;
    if (q >= 0) {
      acc[q * TPB] += v;
      used |= 1u << q;
    } else {
      ok &= slot_add<MG_ROW_SLOTS - 9>(tc, tv, m, a, v);
    }
  }
  int t = 0;
  ragg[i] = own;
  rval[i] = acc[4 * TPB];
  ++t;
  unsigned used8 = 0;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    if (q == 4) continue;
    const int k = q < 4 ? q : q - 1;
    const bool u = (used & (1u << q)) != 0;
    if (val32) ((float*)rv9)[(size_t)k * c.npfb + i] = u ? narrow(acc[q * TPB]) : 0.f;
    else rv9[(size_t)k * c.npfb + i] = u ? acc[q * TPB] : 0.0;
    if (!u) continue;
    used8 |= 1u << k;
    ragg[(size_t)t * c.npfb + i] = own + (q / 3 - 1) * ncx + (q % 3 - 1);
    rval[(size_t)t * c.npfb + i] = acc[q * TPB];
    ++t;
  }
  const int t_list = t;
  for (int e = 0; e < m; ++e, ++t) {
    ragg[(size_t)t * c.npfb + i] = tc[e];
    rval[(size_t)t * c.npfb + i] = tv[e];
  }
  rcnt[i] = t;
  rx[i] = t_list | (t << 8) | (int)(used8 << 16);
  if (!ok) d.s->mg_fail = 1;
}

__global__ void k_mg_level1(Consts c, Dev d, MgLevel L, const int* __restrict__ ragg,
                            const double* __restrict__ rval, const int* __restrict__ rcnt) {
  const int cc = blockIdx.x * blockDim.x + threadIdx.x;
  if (cc >= L.n) return;
  int tc[MG_SLOTS];
  double tv[MG_SLOTS];
  int m = 0;
  double dg = 0.0;
  bool ok = true;
  const int s0 = d.cell_start[cc], ne = d.cell_cnt[cc];
  for (int q = 0; q < ne; ++q) {
    const int i = d.ip[s0 + q];
    if (i >= c.npfb) break;  // mirrors follow the particles in a sorted cell list
    const int mi = rcnt[i];
    for (int t = 0; t < mi; ++t) {
      const int a = ragg[(size_t)t * c.npfb + i];
      const double v = rval[(size_t)t * c.npfb + i];
      if (a == cc) dg += v;
      else ok &= slot_add(tc, tv, m, a, v);
    }
  }
  slot_store(L, cc, tc, tv, m, dg);
  if (!ok) d.s->mg_fail = 1;
}

// level l+1 from level l: one thread per coarse row sums its (up to) 2x2 child rows
__global__ void k_mg_coarsen(MgLevel F, MgLevel G, Scal* s) {
  const int C = blockIdx.x * blockDim.x + threadIdx.x;
  if (C >= G.n) return;
  const int X = C % G.gx, Y = C / G.gx;
  int tc[MG_SLOTS];
  double tv[MG_SLOTS];
  int m = 0;
  double dg = 0.0;
  bool ok = true;
  for (int q = 0; q < 4; ++q) {
    const int fx = 2 * X + (q & 1), fy = 2 * Y + (q >> 1);
    if (fx >= F.gx || fy >= F.gy) continue;
    const int f = fx + fy * F.gx;
    dg += F.diag[f];
    const int cnt = F.cnt[f];
    for (int t = 0; t < cnt; ++t) {
      const int cf = F.col[(size_t)t * F.n + f];
      const int a = (cf % F.gx) / 2 + ((cf / F.gx) / 2) * G.gx;
      const double v = F.val[(size_t)t * F.n + f];
      if (a == C) dg += v;
      else ok &= slot_add(tc, tv, m, a, v);
    }
  }
  slot_store(G, C, tc, tv, m, dg);
  if (!ok) s->mg_fail = 1;
}

// The coarsest level's dense inverse, for a direct coarse solve in the V-cycle: Gauss-Jordan
// with partial pivoting in one 32 x 32 block, thread (ty, tx) owning row ty and columns tx and
// tx + 32 of [M | I] (at most MG_COARSEST = 32 rows).  A closed domain's coarse matrix is
// singular (its rows sum to zero: the constant is in its null space), so it is inverted as
// M + alpha 1 1^T with alpha = mean |diag| / n, which moves that eigenvalue to mean |diag| and
// leaves the mean-free solution of M x = b unchanged.  *ok = 0 (a zero pivot, or a level too
// large) makes the V-cycle fall back to Jacobi sweeps.
__global__ void __launch_bounds__(1024) k_mg_coarse_inverse(MgLevel K, double* inv, int* ok, int closed) {
  __shared__ double M[MG_COARSEST][2 * MG_COARSEST + 1];
  __shared__ double fcol[MG_COARSEST];
  __shared__ int piv_row;
  __shared__ double alpha_s;
  const int n = K.n, tx = threadIdx.x, ty = threadIdx.y;
  if (n > MG_COARSEST || n < 1) {
    if (tx == 0 && ty == 0) *ok = 0;
    return;
  }
  if (ty == 0) {  // alpha from the warp of row-owners
    double ad = tx < n ? fabs(K.diag[tx]) : 0.0;
    for (int o = 16; o > 0; o >>= 1) ad += __shfl_xor_sync(0xffffffffu, ad, o);
    if (tx == 0) alpha_s = closed ? ad / ((double)n * (double)n) : 0.0;
  }
  __syncthreads();
  const int r = ty;
  if (r < n)
    for (int c = tx; c < 2 * n; c += 32) M[r][c] = c < n ? alpha_s : (c - n == r ? 1.0 : 0.0);
  __syncthreads();
  if (r < n && tx == 0) {
    M[r][r] += K.diag[r];
    const int m = K.cnt[r];
    for (int t = 0; t < m; ++t) M[r][K.col[(size_t)t * K.n + r]] += K.val[(size_t)t * K.n + r];
  }
  __syncthreads();
  bool good = true;
  for (int k = 0; k < n; ++k) {
    if (ty == 0) {  // argmax of |M[i][k]| over i >= k, ties to the lower row
      double v = (tx >= k && tx < n) ? fabs(M[tx][k]) : -1.0;
      int p = tx;
      for (int o = 16; o > 0; o >>= 1) {
        const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const int p2 = __shfl_xor_sync(0xffffffffu, p, o);
        if (v2 > v || (v2 == v && p2 < p)) { v = v2; p = p2; }
      }
      if (tx == 0) piv_row = v > 0.0 ? p : -1;
    }
    __syncthreads();
    const int p = piv_row;
    if (p < 0) { good = false; break; }
    if (ty == 0 && p != k)
      for (int c = tx; c < 2 * n; c += 32) { const double t = M[k][c]; M[k][c] = M[p][c]; M[p][c] = t; }
    __syncthreads();
    const double piv = M[k][k];
    __syncthreads();
    if (ty == 0)
      for (int c = tx; c < 2 * n; c += 32) M[k][c] /= piv;
    if (tx == 0 && r < n) fcol[r] = M[r][k];
    __syncthreads();
    if (r < n && r != k) {
      const double f = fcol[r];
      for (int c = tx; c < 2 * n; c += 32) M[r][c] = fma(-f, M[k][c], M[r][c]);
    }
    __syncthreads();
  }
  if (good && r < n)
    for (int c = tx; c < n; c += 32) inv[(size_t)r * n + c] = M[r][n + c];
  if (tx == 0 && ty == 0) *ok = good ? 1 : 0;
}

// The row's A P g in direct form, vown g_own + sum_c (A P)_ic g_c, from its direction table:
// the eight neighbour cells' values and gathers are all issued at once, their addresses computed
// from the row's own cell (`own`, with g[own] = gc, vown = (A P) at the own cell); unused
// directions gather g[own] and add nothing.  The sum runs in the pair order of k_mg_rows (the
// 3x3 in key order, then the row's searched list).  Direct form, as the FP64 row product sums
// A_ik x_k: nine FMAs on the FP64 pipe (2 lanes per clock per SM here) where the difference
// form took seventeen operations.
__device__ __forceinline__ double ap_stencil(const double* __restrict__ rv9, const int* __restrict__ ragg,
                                             const double* __restrict__ rval, int rx, size_t i, size_t n,
                                             const double* g, int own, int ncx, double gc, double vown) {
  const unsigned used = ((unsigned)rx >> 16) & 0xffu;
  double v8[8], g8[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int q = k < 4 ? k : k + 1;
    const int off = (q / 3 - 1) * ncx + (q % 3 - 1);
    v8[k] = __ldg(rv9 + (size_t)k * n + i);
    g8[k] = g[(used >> k) & 1u ? own + off : own];
  }
  double ap = vown * gc;
#pragma unroll
  for (int k = 0; k < 8; ++k)
    if ((used >> k) & 1u) ap = fma(v8[k], g8[k], ap);
  const int t0 = rx & 0xff, m = (rx >> 8) & 0xff;
  for (int t = t0; t < m; ++t) {
    const size_t e = (size_t)t * n + i;
    ap = fma(__ldg(rval + e), g[__ldg(ragg + e)], ap);
  }
  return ap;
}

// ---------------------------------------------------------------- V-cycle
struct MgArgs {
  BiArgs b;                  // the unpreconditioned solver's arguments
  const MgLevel* lv;         // coarse levels, finest first
  int nl;                    // number of coarse levels (>= 1)
  int tail;                  // first level handled by block 0 alone
  const int *agg, *cstart, *ccnt, *ip;  // fine aggregate (cell) of each row; cell lists
  double *z, *fr, *dinv0, *rsum;        // fine work vectors, 1/diag, row sums
  // A P by fine row (k_mg_rows): (cell, sum of the row's values in that cell) pairs, own cell
  // first, and the same by 3x3 direction with the packed word; A times the V-cycle's output
  const int *ragg, *rx;
  const double *rval, *rv9;
  int ncx;
  double* w;
  const double* kinv;        // the coarsest level's dense inverse, if *kinv_ok
  const int* kinv_ok;
  float* g32;                // mixed precision: the level-1 solution rounded to FP32, else null
};

// (A x)_c on a coarse level; x may have been written by other blocks in this launch
__device__ __forceinline__ double lv_Ax(const MgLevel& L, const double* x, int c) {
  double y = __ldg(L.diag + c) * x[c];
  const int m = __ldg(L.cnt + c);
  for (int t = 0; t < m; ++t) y = fma(__ldg(L.val + (size_t)t * L.n + c), x[__ldg(L.col + (size_t)t * L.n + c)], y);
  return y;
}

__device__ __forceinline__ void lv_residual(const MgLevel& L, int i0, int st) {
  for (int c = i0; c < L.n; c += st) L.r[c] = L.b[c] - lv_Ax(L, L.x, c);
}

// restriction of F's residual into G's right-hand side, and G's first sweep from zero
__device__ __forceinline__ void lv_restrict(const MgLevel& F, const MgLevel& G, int i0, int st) {
  for (int C = i0; C < G.n; C += st) {
    const int X = C % G.gx, Y = C / G.gx;
    double b = 0.0;
    for (int q = 0; q < 4; ++q) {
      const int fx = 2 * X + (q & 1), fy = 2 * Y + (q >> 1);
      if (fx < F.gx && fy < F.gy) b += F.r[fx + fy * F.gx];
    }
    G.b[C] = b;
    G.x[C] = MG_OMEGA * __ldg(G.dinv + C) * b;
  }
}

__device__ __forceinline__ void lv_prolong(const MgLevel& F, const double* gsol, int ggx, int i0, int st) {
  for (int c = i0; c < F.n; c += st) {
    const int X = (c % F.gx) >> 1, Y = (c / F.gx) >> 1;
    F.x[c] = fma(MG_GAMMA, gsol[X + Y * ggx], F.x[c]);
  }
}

// one damped Jacobi sweep of x into r, and into x32 rounded to FP32 when given
__device__ __forceinline__ void lv_smooth(const MgLevel& L, int i0, int st, float* x32 = nullptr) {
  for (int c = i0; c < L.n; c += st) {
    const double v = fma(MG_OMEGA * __ldg(L.dinv + c), L.b[c] - lv_Ax(L, L.x, c), L.x[c]);
    L.r[c] = v;
    if (x32) x32[c] = narrow(v);
  }
}

// The grid-wide levels fuse each pair of phases, so a level costs one grid barrier on the way
// down and one on the way up; both give the same bits as the two phases in sequence.
//
// Down: F's residual and its restriction into G.  Four consecutive lanes take the four children
// of one coarse row; their residuals are summed by shuffles in child order, as lv_restrict sums
// F.r.  The loop bound is warp-uniform (the shuffles need every lane).
__device__ __forceinline__ void lv_residual_restrict(const MgLevel& F, const MgLevel& G, int i0, int st) {
  const int lane = threadIdx.x & 31;
  const int total = 4 * G.n;
  for (int t0 = i0 - lane; t0 < total; t0 += st) {
    const int t = t0 + lane;
    const int C = t >> 2, q = t & 3;
    double r = 0.0;
    int ok = 0;
    if (t < total) {
      const int X = C % G.gx, Y = C / G.gx;
      const int fx = 2 * X + (q & 1), fy = 2 * Y + (q >> 1);
      if (fx < F.gx && fy < F.gy) {
        const int f = fx + fy * F.gx;
        r = F.b[f] - lv_Ax(F, F.x, f);
        ok = 1;
      }
    }
    const double r1 = __shfl_down_sync(0xffffffffu, r, 1);
    const double r2 = __shfl_down_sync(0xffffffffu, r, 2);
    const double r3 = __shfl_down_sync(0xffffffffu, r, 3);
    const int okm = ok | (__shfl_down_sync(0xffffffffu, ok, 1) << 1) | (__shfl_down_sync(0xffffffffu, ok, 2) << 2) |
                    (__shfl_down_sync(0xffffffffu, ok, 3) << 3);
    if (q == 0 && t < total) {
      double b = 0.0;
      if (okm & 1) b += r;
      if (okm & 2) b += r1;
      if (okm & 4) b += r2;
      if (okm & 8) b += r3;
      G.b[C] = b;
      G.x[C] = MG_OMEGA * __ldg(G.dinv + C) * b;
    }
  }
}

// Up: prolongation of G's solution into F and F's smoothing sweep.  Each row forms the
// prolonged x of itself and of its columns from F.x and gsol (neither written in this phase) and
// writes the smoothed value into r (and x32 rounded to FP32 when given); F.x itself is left
// as it was, which nothing reads afterwards.
__device__ __forceinline__ void lv_prolong_smooth(const MgLevel& F, const double* gsol, int ggx, int i0, int st,
                                                  float* x32 = nullptr) {
  for (int c = i0; c < F.n; c += st) {
    auto xp = [&](int k) {
      const int X = (k % F.gx) >> 1, Y = (k / F.gx) >> 1;
      return fma(MG_GAMMA, gsol[X + Y * ggx], F.x[k]);
    };
    const double xc = xp(c);
    double y = __ldg(F.diag + c) * xc;
    const int m = __ldg(F.cnt + c);
    for (int t = 0; t < m; ++t) y = fma(__ldg(F.val + (size_t)t * F.n + c), xp(__ldg(F.col + (size_t)t * F.n + c)), y);
    const double v = fma(MG_OMEGA * __ldg(F.dinv + c), F.b[c] - y, xc);
    F.r[c] = v;
    if (x32) x32[c] = narrow(v);
  }
}

// the solution of level l after the upward pass: post-smoothed into r, or x on the coarsest
__device__ __forceinline__ const double* lv_sol(const MgArgs& a, int l) {
  return l == a.nl - 1 ? a.lv[l].x : a.lv[l].r;
}

// levels tail..nl-1 by block 0 alone
__device__ void mg_block_levels(const MgArgs& a) {
  const int i0 = threadIdx.x, st = blockDim.x;
  for (int l = a.tail; l + 1 < a.nl; ++l) {
    const MgLevel F = a.lv[l], G = a.lv[l + 1];
    lv_residual(F, i0, st);
    __syncthreads();
    lv_restrict(F, G, i0, st);
    __syncthreads();
  }
  const MgLevel K = a.lv[a.nl - 1];
  if (a.kinv_ok && *a.kinv_ok) {  // direct solve with the dense inverse
    for (int r = i0; r < K.n; r += st) {
      double v = 0.0;
      for (int c = 0; c < K.n; ++c) v = fma(__ldg(a.kinv + (size_t)r * K.n + c), K.b[c], v);
      K.x[r] = v;
    }
    __syncthreads();
  } else {
    for (int sw = 0; sw < MG_SWEEPS; ++sw) {
      lv_smooth(K, i0, st);
      __syncthreads();
      for (int c = i0; c < K.n; c += st) K.x[c] = K.r[c];
      __syncthreads();
    }
  }
  if (a.g32 && a.nl == 1) {  // level 1 is the coarsest
    for (int c = i0; c < K.n; c += st) a.g32[c] = narrow(K.x[c]);
    __syncthreads();
  }
  for (int l = a.nl - 2; l >= a.tail; --l) {
    const MgLevel F = a.lv[l];
    lv_prolong(F, lv_sol(a, l + 1), a.lv[l + 1].gx, i0, st);
    __syncthreads();
    lv_smooth(F, i0, st, l == 0 ? a.g32 : nullptr);
    __syncthreads();
  }
}

// out = M^-1 q by one V-cycle; the last loop also writes the block partial of sum(out) into
// slot.  q needs only its own rows complete (the calling thread wrote them).
// q -= qshift first (the closed domain's mean removal), stored back.  As in the solvers, the
// vector passes load each row's operands one row ahead (rows_ahead).
__device__ bool mg_vcycle(const MgArgs& a, double* q, double qshift, double* out, double* slot, double* sh,
                          int tid, int stride) {
  const int n = a.b.n;
  Scal* s = a.b.sc;
  double* z = a.z;
  rows_ahead(
      tid, stride, n, [&](int i) { return make_double2(q[i], a.dinv0[i]); },
      [&](int i, const double2& o) {
        const double qi = o.x - qshift;
        q[i] = qi;
        z[i] = MG_OMEGA * o.y * qi;
      });
  if (!grid_sync(s)) return false;
  for (int i = tid; i < n; i += stride) a.fr[i] = q[i] - spmv_row(a.b, z, i);
  if (!grid_sync(s)) return false;
  {  // restriction to the cells (level 1)
    const MgLevel L1 = a.lv[0];
    for (int cc = tid; cc < L1.n; cc += stride) {
      const int s0 = __ldg(a.cstart + cc), ne = __ldg(a.ccnt + cc);
      double b = 0.0;
      for (int k = 0; k < ne; ++k) {
        const int i = __ldg(a.ip + s0 + k);
        if (i >= n) break;
        b += a.fr[i];
      }
      L1.b[cc] = b;
      L1.x[cc] = MG_OMEGA * __ldg(L1.dinv + cc) * b;
    }
  }
  if (!grid_sync(s)) return false;
  for (int l = 0; l < a.tail; ++l) {
    lv_residual_restrict(a.lv[l], a.lv[l + 1], tid, stride);
    if (!grid_sync(s)) return false;
  }
  if (blockIdx.x == 0) mg_block_levels(a);
  if (!grid_sync(s)) return false;
  for (int l = a.tail - 1; l >= 0; --l) {
    lv_prolong_smooth(a.lv[l], lv_sol(a, l + 1), a.lv[l + 1].gx, tid, stride);
    if (!grid_sync(s)) return false;
  }
  // prolongation to the particles (the particle level is pre-smoothed only), and
  // w = A out = A z + gamma (A P) g1 with A z = q - fr from the fine residual and (A P) g1 in
  // direct form over the row's cells (ap_stencil).
  // Software-pipelined: a row's streamed operands are loaded one pass ahead, together with the
  // gathers of the row before, so each pass waits for one round trip to memory, not two.
  const double* g1 = lv_sol(a, 0);
  double acc = 0.0;
  struct Row {
    int c, rx;
    double z, q, fr, vown;
  };
  auto load_row = [&](int i) {
    Row r;
    r.c = __ldg(a.agg + i);
    r.rx = __ldg(a.rx + i);
    r.z = z[i];
    r.q = q[i];
    r.fr = a.fr[i];
    r.vown = __ldg(a.rval + i);  // slot 0: the row's own cell
    return r;
  };
  Row cur{};
  if (tid < n) cur = load_row(tid);
  for (int i = tid; i < n; i += stride) {
    const Row r = cur;
    if (i + stride < n) cur = load_row(i + stride);
    double o = r.z;
    double w = r.q - r.fr;
    if (r.c >= 0) {
      const double gc = g1[r.c];
      o = fma(MG_GAMMA, gc, o);
      w = fma(MG_GAMMA, ap_stencil(a.rv9, a.ragg, a.rval, r.rx, i, n, g1, r.c, a.ncx, gc, r.vown), w);
    }
    out[i] = o;
    a.w[i] = w;
    acc += o;
  }
  write_partials(acc, 0.0, 1, slot, sh);
  return true;
}

// ---------------------------------------------------------------- preconditioned BiCGSTAB
template <bool NONULL>
__global__ void __launch_bounds__(TPB, 4) k_bicgstab_mg(MgArgs m) {
  __shared__ double sh[64];
  __shared__ double shv[4];
  const BiArgs& a = m.b;
  const int n = a.n;
  const int nb = gridDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  Scal* s = a.sc;
  if (*((volatile int*)&s->first_error)) return;  // this state already failed a step
  const bool use_mg = *((volatile int*)&s->mg_fail) == 0;
  double* part = a.part;
  const double rinv1 = 1.0 / (1.0 + 1.0e-15);
  const double small = NONULL ? 1.0e-6 : 4.0;  // open solver: the integer expression 10-6
  double red[4];
  double acc = 0.0;
  // out = M^-1 (q - qshift) with q -= qshift stored back (q: own rows complete), and the
  // block partial of sum(out) into slot
  auto precond = [&](double* q, double qshift, double* out, double* slot) -> bool {
    if (use_mg) return mg_vcycle(m, q, qshift, out, slot, sh, tid, stride);
    double sum = 0.0;
    for (int i = tid; i < n; i += stride) {
      const double qi = q[i] - qshift;
      q[i] = qi;
      const double o = NONULL ? qi * rinv1 : qi * a.rinvM[i];
      out[i] = o;
      sum += o;
    }
    write_partials(sum, 0.0, 1, slot, sh);
    return true;
  };
  for (int i = tid; i < n; i += stride) {  // 1/diag and row sums of the fine matrix
    const double dg = __ldg(a.diag + i);
    double rs = dg;
    const int cnt = __ldg(a.cnt + i);
    for (int k = 0; k < cnt; ++k) rs += __ldg(a.val + (size_t)k * a.stride + i);
    m.dinv0[i] = dg != 0.0 ? 1.0 / dg : 0.0;
    m.rsum[i] = rs;
    if (!NONULL) a.rinvM[i] = 1.0 / (dg + 1.0e-15);
  }
  if (a.warm) {  // x0 = P of the previous step
    for (int i = tid; i < n; i += stride) {
      double xi = a.P[i];
      a.x[i] = xi;
      a.pinv[i] = xi;
    }
    if (!grid_sync(s)) return;
  }
  for (int i = tid; i < n; i += stride) {
    double bi = a.B[i];
    if (a.warm) bi = bi - spmv_row(a, a.pinv, i);
    else a.x[i] = 0.0;
    a.r[i] = bi;
    a.rb[i] = bi;
    a.v[i] = 0.0;
    a.p[i] = 0.0;
    acc = fma(bi, bi, acc);
  }
  write_partials(acc, 0.0, 1, part + 10 * (size_t)nb, sh);
  if (!grid_sync(s)) return;
  reduce_partials(part + 10 * (size_t)nb, nb, 1, red, shv);
  double rho = red[0], alpha = 1.0, omega = 1.0;
  double beta = 0.0;  // for iteration 2 on, derived with the previous iteration's last reduction
  const double dn = (double)n;
  double n2r0 = 1.0, n2s0 = 1.0, resid = 0.0;
  int iter = 1, warn = 0;
  bool done = false;
  while (iter <= a.itermax) {
    if (rho == 0.0) { warn |= VEBI_WARN_BICGSTAB_BREAKDOWN; done = true; break; }
    acc = 0.0;
    // the vector passes load each row's operands one row ahead (rows_ahead)
    rows_ahead(
        tid, stride, n, [&](int i) { return make_double3(a.r[i], a.v[i], a.p[i]); },
        [&](int i, const double3& o) {
          const double ni = (iter == 1) ? o.x : fma(beta, fma(-omega, o.y, o.z), o.x);
          a.p[i] = ni;
          acc += ni;
        });
    double mean = 0.0;
    if (NONULL) {
      write_partials(acc, 0.0, 1, part, sh);
      if (!grid_sync(s)) return;
      reduce_partials(part, nb, 1, red, shv, [=](double* v) { v[0] = v[0] / dn; });
      mean = red[0];
    }
    // p_hat = M^-1 (p - mean), made mean-free (closed domains) through mp
    if (!precond(a.p, mean, a.pinv, part + 1 * (size_t)nb)) return;
    if (!grid_sync(s)) return;
    reduce_partials(part + 1 * (size_t)nb, nb, 1, red, shv, [=](double* v) { v[0] = NONULL ? v[0] / dn : 0.0; });
    const double mp = red[0];
    // v = A (p_hat - mp) ; (r_bar, v)
    acc = 0.0;
    if (use_mg) {
      rows_ahead(
          tid, stride, n, [&](int i) { return make_double3(m.w[i], m.rsum[i], a.rb[i]); },
          [&](int i, const double3& o) {
            const double vi = fma(-mp, o.y, o.x);
            a.v[i] = vi;
            acc = fma(o.z, vi, acc);
          });
    } else {
      for (int i = tid; i < n; i += stride) {
        double vi = fma(-mp, m.rsum[i], spmv_row(a, a.pinv, i));
        a.v[i] = vi;
        acc = fma(a.rb[i], vi, acc);
      }
    }
    write_partials(acc, 0.0, 1, part + 2 * (size_t)nb, sh);
    if (!grid_sync(s)) return;
    reduce_partials(part + 2 * (size_t)nb, nb, 1, red, shv, [=](double* v) { v[0] = rho / (v[0] + 1.0e-15); });
    alpha = red[0];
    double a2 = 0.0;
    acc = 0.0;
    rows_ahead(
        tid, stride, n, [&](int i) { return make_double2(a.v[i], a.r[i]); },
        [&](int i, const double2& o) {
          const double si = fma(-alpha, o.x, o.y);
          a.s[i] = si;
          acc = fma(si, si, acc);
          a2 += si;
        });
    write_partials(acc, a2, 2, part + 4 * (size_t)nb, sh);
    if (!grid_sync(s)) return;
    reduce_partials(part + 4 * (size_t)nb, nb, 2, red, shv, [=](double* v) { v[1] = v[1] / dn; });
    const double n2s = red[0];
    const double mean_s = red[1];
    if (iter == 1) n2s0 = (n2s <= small) ? 1.0 : n2s;
    if (n2s <= a.tol * a.tol * n2s0) {
      for (int i = tid; i < n; i += stride) a.x[i] = fma(alpha, a.pinv[i] - mp, a.x[i]);
      resid = sqrt(n2s / n2s0);
      done = true;
      break;
    }
    if (!precond(a.s, NONULL ? mean_s : 0.0, a.sinv, part + 3 * (size_t)nb)) return;
    if (!grid_sync(s)) return;
    reduce_partials(part + 3 * (size_t)nb, nb, 1, red, shv, [=](double* v) { v[0] = NONULL ? v[0] / dn : 0.0; });
    const double ms = red[0];
    // t = A (s_hat - ms) ; (t, s) ; |t|^2
    acc = 0.0;
    a2 = 0.0;
    if (use_mg) {
      rows_ahead(
          tid, stride, n, [&](int i) { return make_double3(m.w[i], m.rsum[i], a.s[i]); },
          [&](int i, const double3& o) {
            const double ti = fma(-ms, o.y, o.x);
            a.t[i] = ti;
            acc = fma(ti, o.z, acc);
            a2 = fma(ti, ti, a2);
          });
    } else {
      for (int i = tid; i < n; i += stride) {
        double ti = fma(-ms, m.rsum[i], spmv_row(a, a.sinv, i));
        a.t[i] = ti;
        acc = fma(ti, a.s[i], acc);
        a2 = fma(ti, ti, a2);
      }
    }
    write_partials(acc, a2, 2, part + 6 * (size_t)nb, sh);
    if (!grid_sync(s)) return;
    reduce_partials(part + 6 * (size_t)nb, nb, 2, red, shv, [](double* v) { v[0] = v[0] / (v[1] + 1.0e-15); });
    omega = red[0];
    acc = 0.0;
    a2 = 0.0;
    // x += alpha (p_hat - mp) + omega (s_hat - ms), with the two mean shifts folded into one
    const double xshift = fma(alpha, mp, omega * ms);
    struct XRow {
      double s, p, x, t, sv, rb;
    };
    rows_ahead(
        tid, stride, n, [&](int i) { return XRow{a.sinv[i], a.pinv[i], a.x[i], a.t[i], a.s[i], a.rb[i]}; },
        [&](int i, const XRow& o) {
          a.x[i] = fma(omega, o.s, fma(alpha, o.p, o.x - xshift));
          const double ri = fma(-omega, o.t, o.sv);
          a.r[i] = ri;
          acc = fma(ri, ri, acc);
          a2 = fma(o.rb, ri, a2);
        });
    write_partials(acc, a2, 2, part + 8 * (size_t)nb, sh);
    if (!grid_sync(s)) return;
    // v[2] = the relative residual, v[3] = the next iteration's beta from the new rho v[1]
    reduce_partials(part + 8 * (size_t)nb, nb, 2, red, shv, [=](double* v) {
      const double r0 = iter == 1 ? ((v[0] <= small) ? 1.0 : v[0]) : n2r0;
      v[2] = sqrt(v[0] / r0);
      v[3] = v[1] / (rho + 1.0e-15) * alpha / (omega + 1.0e-15);
    });
    const double n2r = red[0];
    if (iter == 1) n2r0 = (n2r <= small) ? 1.0 : n2r;
    resid = red[2];
    if (n2r <= a.tol * a.tol * n2r0) { done = true; break; }
    iter = iter + 1;
    rho = red[1];
    beta = red[3];
  }
  if (!done) warn |= VEBI_WARN_MAXITER;
  for (int i = tid; i < n; i += stride) a.P[i] = a.x[i];
  if (tid == 0) {
    s->ls_iters = iter;
    s->ls_iters_total += iter;
    s->ls_residual = resid;
    atomicOr(&s->warnings, warn);
  }
}

// ---------------------------------------------------------------- mixed precision
// The mixed-precision solver (FP64 recurrences, FP32 difference-form SpMV) with the same
// V-cycle, whose particle level runs in FP32: the smoothing vector and the fine residual are
// FP32 and the fine products use the FP32 values in difference form.  The coarse levels are the
// FP64 ones of the FP64 solver.  The preconditioner need not be exact: its rounding changes the
// iteration count, not the residual test the solve stops on.
struct MgMxArgs {
  MxArgs b;
  const MgLevel* lv;
  int nl, tail;
  const int *agg, *cstart, *ccnt, *ip;
  float *z, *fr, *dinv0;
  const int *ragg, *rx;  // A P by fine row, as in MgArgs, with FP32 direction values
  const double* rval;
  const float* rv9;
  int ncx;
  float* w;                // A times the V-cycle's output, FP32
  const double* kinv;      // the coarsest level's dense inverse, if *kinv_ok
  const int* kinv_ok;
  float* g32;              // the level-1 solution rounded to FP32
  float* rs32;             // the row sums rounded to FP32
  float* q32;              // the V-cycle's input (after mean removal) rounded to FP32
  const double* diag;      // the PPE matrix's FP64 diagonal
};

// sum_k A_ik (z_col - z_i) + rowsum_i z_i in FP32 (one FP32 vector; rs32 = FP32 row sums)
__device__ __forceinline__ float spmv_diff32s(const MxArgs& a, const float* rs32, const float* z, int i) {
  const int cnt = __ldg(a.cnt + i);
  const float* vp = a.val32 + i;
  const int* cp = a.col + i;
  const long long st = a.stride;
  const float zi = __ldca(z + i);
  float b0 = 0.f, b1 = 0.f, b2 = 0.f, b3 = 0.f;
  int k = 0;
  for (; k + 3 < cnt; k += 4) {
    const int c0 = __ldg(cp), c1 = __ldg(cp + st), c2 = __ldg(cp + 2 * st), c3 = __ldg(cp + 3 * st);
    const float v0 = __ldg(vp), v1 = __ldg(vp + st), v2 = __ldg(vp + 2 * st), v3 = __ldg(vp + 3 * st);
    b0 = fmaf(v0, __ldca(z + c0) - zi, b0);
    b1 = fmaf(v1, __ldca(z + c1) - zi, b1);
    b2 = fmaf(v2, __ldca(z + c2) - zi, b2);
    b3 = fmaf(v3, __ldca(z + c3) - zi, b3);
    cp += 4 * st;
    vp += 4 * st;
  }
  for (; k < cnt; ++k) {
    b0 = fmaf(__ldg(vp), __ldca(z + __ldg(cp)) - zi, b0);
    cp += st;
    vp += st;
  }
  return fmaf(rs32[i], zi, (b0 + b1) + (b2 + b3));
}

// The row's A P g1 in FP32: rowsum_i g_own + sum_c (A P)_ic (g_c - g_own) from the FP32 direction
// table and the FP32 level-1 solution g, in the pair order of k_mg_rows; the searched list (rare:
// periodic partners, mirror parents outside the 3x3) from the FP64 pairs rounded to FP32.
__device__ __forceinline__ float ap_stencil32(const float* __restrict__ rv9, const int* __restrict__ ragg,
                                              const double* __restrict__ rval, int rx, size_t i, size_t n,
                                              const float* g, int own, int ncx, float gc, float rs) {
  const unsigned used = ((unsigned)rx >> 16) & 0xffu;
  float v8[8], g8[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int q = k < 4 ? k : k + 1;
    const int off = (q / 3 - 1) * ncx + (q % 3 - 1);
    v8[k] = __ldg(rv9 + (size_t)k * n + i);
    g8[k] = g[(used >> k) & 1u ? own + off : own];
  }
  float ap = rs * gc;
#pragma unroll
  for (int k = 0; k < 8; ++k)
    if ((used >> k) & 1u) ap = fmaf(v8[k], g8[k] - gc, ap);
  const int t0 = rx & 0xff, m = (rx >> 8) & 0xff;
  for (int t = t0; t < m; ++t) {
    const size_t e = (size_t)t * n + i;
    ap = fmaf((float)__ldg(rval + e), g[__ldg(ragg + e)] - gc, ap);
  }
  return ap;
}

// out = M^-1 q in FP64 (the preconditioned direction); block partial of sum(out) into slot.
// The vector passes load each row's operands one row ahead (rows_ahead), so a pass's loads are
// in flight before the previous row's stores: the compiler cannot move a load above a store
// to another array it may alias.
__device__ bool mg_vcycle_mixed(const MgMxArgs& a, double* q, double qshift, double* out, double* slot,
                                double* sh, int tid, int stride) {
  const int n = a.b.n;
  Scal* s = a.b.sc;
  float* z = a.z;
  // q -= qshift (the closed domain's mean removal), its FP32 rounding q32, and z = omega D^-1 q
  float* q32 = a.q32;
  struct QRow {
    double q;
    float d;
  };
  rows_ahead(
      tid, stride, n, [&](int i) { return QRow{q[i], a.dinv0[i]}; },
      [&](int i, const QRow& o) {
        const double qi = o.q - qshift;
        const float fi = narrow(qi);
        q[i] = qi;
        q32[i] = fi;
        z[i] = (float)MG_OMEGA * o.d * fi;
      });
  if (!grid_sync(s)) return false;
  for (int i = tid; i < n; i += stride) a.fr[i] = q32[i] - spmv_diff32s(a.b, a.rs32, z, i);
  if (!grid_sync(s)) return false;
  {
    const MgLevel L1 = a.lv[0];
    for (int cc = tid; cc < L1.n; cc += stride) {
      const int s0 = __ldg(a.cstart + cc), ne = __ldg(a.ccnt + cc);
      float b32 = 0.f;  // the cell's residuals summed in FP32, in cell-list order
      for (int k = 0; k < ne; ++k) {
        const int i = __ldg(a.ip + s0 + k);
        if (i >= n) break;
        b32 += a.fr[i];
      }
      const double b = widen(b32);
      L1.b[cc] = b;
      L1.x[cc] = MG_OMEGA * __ldg(L1.dinv + cc) * b;
    }
  }
  if (!grid_sync(s)) return false;
  MgArgs c{};  // the coarse-level view shared with the FP64 V-cycle
  c.lv = a.lv;
  c.nl = a.nl;
  c.tail = a.tail;
  c.kinv = a.kinv;
  c.kinv_ok = a.kinv_ok;
  c.g32 = a.g32;
  for (int l = 0; l < a.tail; ++l) {
    lv_residual_restrict(a.lv[l], a.lv[l + 1], tid, stride);
    if (!grid_sync(s)) return false;
  }
  if (blockIdx.x == 0) mg_block_levels(c);
  if (!grid_sync(s)) return false;
  for (int l = a.tail - 1; l >= 0; --l) {
    lv_prolong_smooth(a.lv[l], lv_sol(c, l + 1), a.lv[l + 1].gx, tid, stride, l == 0 ? a.g32 : nullptr);
    if (!grid_sync(s)) return false;
  }
  // prolongation to the particles (pre-smoothed only) from the FP32 level-1 solution g, and
  // w = A out, both in FP32 (the precision of this solver's products): A z = q32 - fr, plus
  // gamma (A P) g in difference form with the FP32 row sums.  The output is stored as FP64 and
  // summed in FP64 (the mean removal).  This GPU issues FP64 at 1/64 of the FP32 rate, so the
  // pass keeps to FP32 arithmetic; streamed operands are loaded one pass ahead of the gathers.
  const float* g32 = a.g32;
  const float gam = (float)MG_GAMMA;
  double acc = 0.0;
  struct Row {
    int c, rx;
    float z, fr, rs, q;
  };
  auto load_row = [&](int i) {
    Row r;
    r.c = __ldg(a.agg + i);
    r.rx = __ldg(a.rx + i);
    r.z = z[i];
    r.fr = a.fr[i];
    r.rs = a.rs32[i];
    r.q = q32[i];
    return r;
  };
  Row cur{};
  if (tid < n) cur = load_row(tid);
  for (int i = tid; i < n; i += stride) {
    const Row r = cur;
    if (i + stride < n) cur = load_row(i + stride);
    float oi = r.z;
    float wi = r.q - r.fr;
    if (r.c >= 0) {
      const float gc = g32[r.c];
      oi = fmaf(gam, gc, oi);
      wi = fmaf(gam, ap_stencil32(a.rv9, a.ragg, a.rval, r.rx, i, n, g32, r.c, a.ncx, gc, r.rs), wi);
    }
    const double od = widen(oi);
    out[i] = od;
    a.w[i] = wi;
    acc += od;
  }
  write_partials(acc, 0.0, 1, slot, sh);
  return true;
}

// Blocks per SM the mixed kernel is compiled for: its register budget is 65536 / (TPB x this)
#ifndef VEBI_MIXED_MG_BLOCKS_PER_SM
#define VEBI_MIXED_MG_BLOCKS_PER_SM 4
#endif

template <bool NONULL>
__global__ void __launch_bounds__(TPB, VEBI_MIXED_MG_BLOCKS_PER_SM) k_bicgstab_mixed_mg(MgMxArgs m) {
  __shared__ double sh[64];
  __shared__ double shv[4];
  const MxArgs& a = m.b;
  const int n = a.n;
  const int nb = gridDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  Scal* s = a.sc;
  if (*((volatile int*)&s->first_error)) return;  // this state already failed a step
  const bool use_mg = *((volatile int*)&s->mg_fail) == 0;
  double* part = a.part;
  const double rinv1 = 1.0 / (1.0 + 1.0e-15);
  const double small = NONULL ? 1.0e-6 : 4.0;
  double red[4];
  double acc = 0.0;
  // out = M^-1 (q - qshift), with q -= qshift stored back; block partial of sum(out) into slot
  // With the multigrid the preconditioned directions are FP64 (pi, si read as double: same
  // size as the (hi, lo) pairs the unpreconditioned products gather)
  double* const pd = reinterpret_cast<double*>(a.pi);
  double* const sd = reinterpret_cast<double*>(a.si);
  auto precond = [&](double* q, double qshift, float2* out, double* slot) -> bool {
    if (use_mg) return mg_vcycle_mixed(m, q, qshift, reinterpret_cast<double*>(out), slot, sh, tid, stride);
    double sum = 0.0;
    for (int i = tid; i < n; i += stride) {
      const double qi = q[i] - qshift;
      q[i] = qi;
      const double o = NONULL ? qi * rinv1 : qi * a.rinvM[i];
      out[i] = split2(o);
      sum += o;
    }
    write_partials(sum, 0.0, 1, slot, sh);
    return true;
  };
  for (int i = tid; i < n; i += stride) {
    // the particle level's Jacobi sweep, in FP32: 1/diag of the assembled matrix
    const float dg = narrow(__ldg(m.diag + i));
    m.dinv0[i] = dg != 0.f ? 1.0f / dg : 0.f;
    m.rs32[i] = narrow(__ldg(a.rs + i));
  }
  if (a.warm) {
    for (int i = tid; i < n; i += stride) {
      double xi = a.P[i];
      a.x[i] = xi;
      a.pi[i] = split2(xi);
    }
    if (!grid_sync(s)) return;
  }
  for (int i = tid; i < n; i += stride) {
    double bi = a.B[i];
    if (a.warm) bi = bi - spmv_diff32(a, a.pi, i);
    else a.x[i] = 0.0;
    a.r[i] = bi;
    a.rb[i] = bi;
    a.v[i] = 0.0;
    a.p[i] = 0.0;
    acc = fma(bi, bi, acc);
  }
  write_partials(acc, 0.0, 1, part + 10 * (size_t)nb, sh);
  if (!grid_sync(s)) return;
  reduce_partials(part + 10 * (size_t)nb, nb, 1, red, shv);
  double rho = red[0], alpha = 1.0, omega = 1.0;
  double beta = 0.0;  // for iteration 2 on, derived with the previous iteration's last reduction
  const double dn = (double)n;
  double n2r0 = 1.0, n2s0 = 1.0, resid = 0.0;
  int iter = 1, warn = 0;
  bool done = false;
  while (iter <= a.itermax) {
    if (rho == 0.0) { warn |= VEBI_WARN_BICGSTAB_BREAKDOWN; done = true; break; }
    acc = 0.0;
    // The vector passes load each row's operands one row ahead (rows_ahead)
    rows_ahead(
        tid, stride, n, [&](int i) { return make_double3(a.r[i], a.v[i], a.p[i]); },
        [&](int i, const double3& o) {
          const double ni = (iter == 1) ? o.x : fma(beta, fma(-omega, o.y, o.z), o.x);
          a.p[i] = ni;
          acc += ni;
        });
    double mean = 0.0;
    if (NONULL) {
      write_partials(acc, 0.0, 1, part, sh);
      if (!grid_sync(s)) return;
      reduce_partials(part, nb, 1, red, shv, [=](double* v) { v[0] = v[0] / dn; });
      mean = red[0];
    }
    if (!precond(a.p, mean, a.pi, part + 1 * (size_t)nb)) return;
    if (!grid_sync(s)) return;
    reduce_partials(part + 1 * (size_t)nb, nb, 1, red, shv, [=](double* v) { v[0] = NONULL ? v[0] / dn : 0.0; });
    const double mp = red[0];
    acc = 0.0;
    if (use_mg) {
      rows_ahead(
          tid, stride, n, [&](int i) { return make_double3(widen(m.w[i]), __ldg(a.rs + i), a.rb[i]); },
          [&](int i, const double3& o) {
            const double vi = fma(-mp, o.y, o.x);
            a.v[i] = vi;
            acc = fma(o.z, vi, acc);
          });
    } else {
      for (int i = tid; i < n; i += stride) {
        double vi = fma(-mp, __ldg(a.rs + i), spmv_diff32(a, a.pi, i));
        a.v[i] = vi;
        acc = fma(a.rb[i], vi, acc);
      }
    }
    write_partials(acc, 0.0, 1, part + 2 * (size_t)nb, sh);
    if (!grid_sync(s)) return;
    reduce_partials(part + 2 * (size_t)nb, nb, 1, red, shv, [=](double* v) { v[0] = rho / (v[0] + 1.0e-15); });
    alpha = red[0];
    double a2 = 0.0;
    acc = 0.0;
    rows_ahead(
        tid, stride, n, [&](int i) { return make_double2(a.v[i], a.r[i]); },
        [&](int i, const double2& o) {
          const double si = fma(-alpha, o.x, o.y);
          a.s[i] = si;
          acc = fma(si, si, acc);
          a2 += si;
        });
    write_partials(acc, a2, 2, part + 4 * (size_t)nb, sh);
    if (!grid_sync(s)) return;
    reduce_partials(part + 4 * (size_t)nb, nb, 2, red, shv, [=](double* v) { v[1] = v[1] / dn; });
    const double n2s = red[0];
    const double mean_s = red[1];
    if (iter == 1) n2s0 = (n2s <= small) ? 1.0 : n2s;
    if (n2s <= a.tol * a.tol * n2s0) {
      for (int i = tid; i < n; i += stride)
        a.x[i] = fma(alpha, (use_mg ? pd[i] : join2(a.pi[i])) - mp, a.x[i]);
      resid = sqrt(n2s / n2s0);
      done = true;
      break;
    }
    if (!precond(a.s, NONULL ? mean_s : 0.0, a.si, part + 3 * (size_t)nb)) return;
    if (!grid_sync(s)) return;
    reduce_partials(part + 3 * (size_t)nb, nb, 1, red, shv, [=](double* v) { v[0] = NONULL ? v[0] / dn : 0.0; });
    const double ms = red[0];
    acc = 0.0;
    a2 = 0.0;
    if (use_mg) {
      rows_ahead(
          tid, stride, n, [&](int i) { return make_double3(widen(m.w[i]), __ldg(a.rs + i), a.s[i]); },
          [&](int i, const double3& o) {
            const double ti = fma(-ms, o.y, o.x);
            a.t[i] = ti;
            acc = fma(ti, o.z, acc);
            a2 = fma(ti, ti, a2);
          });
    } else {
      for (int i = tid; i < n; i += stride) {
        double ti = fma(-ms, __ldg(a.rs + i), spmv_diff32(a, a.si, i));
        a.t[i] = ti;
        acc = fma(ti, a.s[i], acc);
        a2 = fma(ti, ti, a2);
      }
    }
    write_partials(acc, a2, 2, part + 6 * (size_t)nb, sh);
    if (!grid_sync(s)) return;
    reduce_partials(part + 6 * (size_t)nb, nb, 2, red, shv, [](double* v) { v[0] = v[0] / (v[1] + 1.0e-15); });
    omega = red[0];
    acc = 0.0;
    a2 = 0.0;
    // x += alpha (p_hat - mp) + omega (s_hat - ms), with the two mean shifts folded into one
    const double xshift = fma(alpha, mp, omega * ms);
    struct XRow {
      double p, s, x, t, sv, rb;
    };
    auto xr_update = [&](int i, const XRow& o) {
      a.x[i] = fma(omega, o.s, fma(alpha, o.p, o.x - xshift));
      const double ri = fma(-omega, o.t, o.sv);
      a.r[i] = ri;
      acc = fma(ri, ri, acc);
      a2 = fma(o.rb, ri, a2);
    };
    // the preconditioned directions: FP64 with the multigrid, else (hi, lo) pairs
    if (use_mg) {
      rows_ahead(
          tid, stride, n, [&](int i) { return XRow{pd[i], sd[i], a.x[i], a.t[i], a.s[i], a.rb[i]}; }, xr_update);
    } else {
      rows_ahead(
          tid, stride, n,
          [&](int i) { return XRow{join2(a.pi[i]), join2(a.si[i]), a.x[i], a.t[i], a.s[i], a.rb[i]}; }, xr_update);
    }
    write_partials(acc, a2, 2, part + 8 * (size_t)nb, sh);
    if (!grid_sync(s)) return;
    // v[2] = the relative residual, v[3] = the next iteration's beta from the new rho v[1]
    reduce_partials(part + 8 * (size_t)nb, nb, 2, red, shv, [=](double* v) {
      const double r0 = iter == 1 ? ((v[0] <= small) ? 1.0 : v[0]) : n2r0;
      v[2] = sqrt(v[0] / r0);
      v[3] = v[1] / (rho + 1.0e-15) * alpha / (omega + 1.0e-15);
    });
    const double n2r = red[0];
    if (iter == 1) n2r0 = (n2r <= small) ? 1.0 : n2r;
    resid = red[2];
    if (n2r <= a.tol * a.tol * n2r0) { done = true; break; }
    iter = iter + 1;
    rho = red[1];
    beta = red[3];
  }
  if (!done) warn |= VEBI_WARN_MAXITER;
  for (int i = tid; i < n; i += stride) a.P[i] = a.x[i];
  if (tid == 0) {
    s->ls_iters = iter;
    s->ls_iters_total += iter;
    s->ls_residual = resid;
    atomicOr(&s->warnings, warn);
  }
}

// ---------------------------------------------------------------- host side
// co-resident blocks of the FP64 (mixed = false) or the mixed multigrid solver
int ppe_mg_blocks(int nsm, bool mixed) {
  int per = 1 << 20;
  int o[2] = {0, 0};
  if (mixed) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o[0], k_bicgstab_mixed_mg<true>, TPB, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o[1], k_bicgstab_mixed_mg<false>, TPB, 0);
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o[0], k_bicgstab_mg<true>, TPB, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o[1], k_bicgstab_mg<false>, TPB, 0);
  }
  for (int q = 0; q < 2; ++q) per = o[q] < per ? o[q] : per;
  if (per < 1) per = 1;
  return per * nsm;
}

// coarse level sizes for a gx x gy cell grid: halve until at most MG_COARSEST aggregates
std::vector<int> mg_level_dims(int gx, int gy) {
  std::vector<int> dims;
  for (int l = 0; l < MG_MAX_LEVELS; ++l) {
    dims.push_back(gx);
    dims.push_back(gy);
    if ((long long)gx * gy <= MG_COARSEST || (gx <= 1 && gy <= 1)) break;
    gx = (gx + 1) / 2;
    gy = (gy + 1) / 2;
  }
  return dims;
}

// the coarse matrices of this step, and the first level small enough for one block
static int mg_setup(Ctx& x) {
  const Consts& c = x.c;
  const int nl = (int)x.mg.size();
  const float* v32 = x.precision == VEBI_PREC_MIXED ? x.d.ppe_val32 : nullptr;
  VEBI_LAUNCH(x, k_mg_rows, grid_for(c.npfb), TPB, c, x.d, v32, x.mg_ragg, x.mg_rval, x.mg_rcnt, x.mg_rv9,
              x.mg_rx);
  VEBI_LAUNCH(x, k_mg_level1, grid_for(x.mg[0].n), TPB, c, x.d, x.mg[0], x.mg_ragg, x.mg_rval, x.mg_rcnt);
  for (int l = 0; l + 1 < nl; ++l)
    VEBI_LAUNCH(x, k_mg_coarsen, grid_for(x.mg[l + 1].n), TPB, x.mg[l], x.mg[l + 1], x.d.s);
  VEBI_LAUNCH(x, k_mg_coarse_inverse, 1, dim3(32, 32), x.mg[nl - 1], x.mg_kinv, x.mg_kinv_ok,
              c.open_domain == 0 ? 1 : 0);
  int tail = nl - 1;
  for (int l = 0; l < nl; ++l)
    if (x.mg[l].n <= x.mg_block_rows) { tail = l; break; }
  return tail;
}

void launch_ppe_mg_mixed(Ctx& x) {
  const Consts& c = x.c;
  const Dev& d = x.d;
  const int tail = mg_setup(x);
  int nblk = x.mg_blocks_mixed;
  const long long rows_per_block = (long long)TPB * (x.solver_rows_per_thread > 0 ? x.solver_rows_per_thread : 1);
  long long need = (c.npfb + rows_per_block - 1) / rows_per_block;
  if (need < nblk) nblk = (int)(need < 1 ? 1 : need);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblk);
  cfg.blockDim = dim3(TPB);
  cfg.stream = x.st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MgMxArgs m{MxArgs{d.bx, d.br, d.brb, d.bv, d.bp, d.bs, d.bt, d.bM, d.partials, d.p, d.pi2, d.si2, d.ppe_B,
                    d.rowsum, d.ppe_val32, d.ppe_col, d.ij_count, d.s, (long long)c.npfb, c.npfb, c.itermax, c.tol,
                    c.warm_start},
             x.d_mg, (int)x.mg.size(), tail, d.cellpart, d.cell_start, d.cell_cnt, d.ip, (float*)x.mg_z,
             (float*)x.mg_fr, (float*)x.mg_dinv0, x.mg_ragg, x.mg_rx, x.mg_rval, (const float*)x.mg_rv9, c.ncx,
             (float*)x.mg_w, x.mg_kinv, x.mg_kinv_ok, x.mg_g32, (float*)x.mg_rsum, x.mg_q32, d.ppe_diag};
  if (c.open_domain == 0) cudaLaunchKernelEx(&cfg, k_bicgstab_mixed_mg<true>, m);
  else cudaLaunchKernelEx(&cfg, k_bicgstab_mixed_mg<false>, m);
  x.launches++;
}

void launch_ppe_mg(Ctx& x) {
  const Consts& c = x.c;
  const Dev& d = x.d;
  const int nl = (int)x.mg.size();
  const int tail = mg_setup(x);
  int nblk = x.mg_blocks;
  const long long rows_per_block = (long long)TPB * (x.solver_rows_per_thread > 0 ? x.solver_rows_per_thread : 1);
  long long need = (c.npfb + rows_per_block - 1) / rows_per_block;
  if (need < nblk) nblk = (int)(need < 1 ? 1 : need);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblk);
  cfg.blockDim = dim3(TPB);
  cfg.stream = x.st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MgArgs m{BiArgs{d.bx, d.br, d.brb, d.bv, d.bp, d.bpi, d.bs, d.bsi, d.bt, d.bM, d.partials, d.p, d.ppe_B,
                  d.ppe_diag, d.ppe_val, d.ppe_col, d.ij_count, d.s, (long long)c.npfb, c.npfb, c.itermax, c.tol,
                  c.warm_start},
           x.d_mg, nl, tail, d.cellpart, d.cell_start, d.cell_cnt, d.ip, x.mg_z, x.mg_fr, x.mg_dinv0, x.mg_rsum,
           x.mg_ragg, x.mg_rx, x.mg_rval, x.mg_rv9, c.ncx, x.mg_w, x.mg_kinv, x.mg_kinv_ok};
  if (c.open_domain == 0) cudaLaunchKernelEx(&cfg, k_bicgstab_mg<true>, m);
  else cudaLaunchKernelEx(&cfg, k_bicgstab_mg<false>, m);
  x.launches++;
}

}  // namespace vebi

#ifdef VEBI_BARRIER_TIMESTAMPS
// diagnostic build only: the multigrid solvers' barrier timestamps (see vebi_solver.cuh)
extern "C" int vebi_barrier_timestamps_reset(void) {
  unsigned int z = 0;
  static unsigned int zb[vebi::BAR_ALL_BLOCKS];
  cudaError_t e = cudaMemcpyToSymbol(vebi::g_bar_blk_n, zb, sizeof(zb));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(vebi::g_bar_n, &z, sizeof(z));
  return (int)e;
}
// every block's arrival at BAR_ALL_N barriers from BAR_ALL_FIRST on ([q][block]), and its SM
extern "C" int vebi_barrier_arrivals_read(unsigned long long* arr, unsigned int* smid) {
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess)
    e = cudaMemcpyFromSymbol(arr, vebi::g_bar_all, sizeof(unsigned long long) * vebi::BAR_ALL_N * vebi::BAR_ALL_BLOCKS);
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(smid, vebi::g_bar_smid, sizeof(unsigned int) * vebi::BAR_ALL_BLOCKS);
  return (int)e;
}
extern "C" int vebi_barrier_timestamps_read(unsigned long long* ts, unsigned int* n) {
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(n, vebi::g_bar_n, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(ts, vebi::g_bar_ts, sizeof(unsigned long long) * 2 * vebi::BAR_TS_MAX);
  return (int)e;
}
#endif
