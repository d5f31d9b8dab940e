// vebi_solver.cuh -- building blocks of the persistent cooperative PPE solvers: the bounded
// grid barrier, the deterministic block-partial reductions, the solver arguments and the
// FP64 ELL row product (sparse_atime, linear_solver.F90:254-273).
#pragma once
#include "vebi_ctx.cuh"

namespace vebi {

constexpr unsigned long long SPIN_LIMIT = 1ull << 25;  // ~2-4 s of __nanosleep(64) polls

#ifdef VEBI_BARRIER_TIMESTAMPS
// Diagnostic build only (vebisph_gb300/barrier_profile.py): block 0 records the global timer
// when it arrives at and leaves every grid barrier, so the time of each solver phase and of the
// wait for the slowest block can be read back.  Each translation unit has its own copy; the
// solvers of vebi_mg.cu export theirs.
constexpr int BAR_TS_MAX = 16384;
static __device__ unsigned long long g_bar_ts[2][BAR_TS_MAX];
static __device__ unsigned int g_bar_n;
// every block's arrival time at the barriers BAR_ALL_FIRST .. BAR_ALL_FIRST + BAR_ALL_N - 1 of
// the solve (one iteration and more), and the SM each block runs on
constexpr int BAR_ALL_FIRST = 200, BAR_ALL_N = 64, BAR_ALL_BLOCKS = 2048;
static __device__ unsigned int g_bar_blk_n[BAR_ALL_BLOCKS];
static __device__ unsigned long long g_bar_all[BAR_ALL_N][BAR_ALL_BLOCKS];
static __device__ unsigned int g_bar_smid[BAR_ALL_BLOCKS];
__device__ __forceinline__ unsigned long long bar_clock() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
#endif

// bounded grid-wide barrier for a co-resident (cooperative) grid; false on error/timeout.
// A block that polls more than `limit` times records VEBI_ERR_TIMEOUT and returns false, and so
// does every block that arrives or polls after the error is recorded.
__device__ __forceinline__ bool grid_sync_bounded(Scal* s, unsigned long long limit) {
#ifdef VEBI_BARRIER_TIMESTAMPS
  const unsigned long long ts_arrive = bar_clock();
#endif
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* vgen = &s->bar_gen;
    volatile int* verr = &s->error;
    unsigned int g = *vgen;
    __threadfence();
    unsigned int arrived = atomicAdd((unsigned int*)&s->bar_count, 1u) + 1u;
    if (arrived == gridDim.x) {
      atomicExch((unsigned int*)&s->bar_count, 0u);
      __threadfence();
      atomicAdd((unsigned int*)&s->bar_gen, 1u);
    } else {
      unsigned long long spins = 0;
      while (*vgen == g) {
        if (*verr != 0) break;
        if (++spins > limit) {
          atomicCAS((int*)&s->error, 0, VEBI_ERR_TIMEOUT);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
#ifdef VEBI_BARRIER_TIMESTAMPS
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const unsigned int q = g_bar_n++;
    if (q < BAR_TS_MAX) {
      g_bar_ts[0][q] = ts_arrive;
      g_bar_ts[1][q] = bar_clock();
    }
  }
  if (threadIdx.x == 0 && blockIdx.x < BAR_ALL_BLOCKS) {
    const unsigned int q = g_bar_blk_n[blockIdx.x]++;
    if (q >= BAR_ALL_FIRST && q < BAR_ALL_FIRST + BAR_ALL_N) g_bar_all[q - BAR_ALL_FIRST][blockIdx.x] = ts_arrive;
    if (q == 0) {
      unsigned int sm;
      asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
      g_bar_smid[blockIdx.x] = sm;
    }
  }
#endif
  return *((volatile int*)&s->error) == 0;
}

__device__ __forceinline__ bool grid_sync(Scal* s) { return grid_sync_bounded(s, SPIN_LIMIT); }

// Sum of the block partials of `slot` in a fixed order; identical in every block.  `post`,
// run by thread 0 alone on the nval sums in v[0..3] before they are shared, derives the
// iteration's scalars (its divisions and square roots) in place: this GPU issues FP64 at 1/64
// of the FP32 rate, so uniform FP64 work is done once per block rather than once per warp.
struct NoPost {
  __device__ void operator()(double*) const {}
};
template <class Post = NoPost>
__device__ __forceinline__ void reduce_partials(const double* part, int nb, int nval, double* out, double* shv,
                                                Post post = Post()) {
  if (threadIdx.x < 32) {
    for (int q = 0; q < nval; ++q) {
      double v = 0.0;
      for (int b = threadIdx.x; b < nb; b += 32) v += __ldcg(part + (size_t)q * nb + b);
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (threadIdx.x == 0) shv[q] = v;
    }
    if (threadIdx.x == 0) post(shv);
  }
  __syncthreads();
  for (int q = 0; q < 4; ++q) out[q] = shv[q];
  __syncthreads();
}

// A vector pass over the rows tid, tid + stride, ... with each row's operands loaded one row
// ahead: load(i) returns row i's operands, body(i, ops) does the arithmetic and the stores.
// The next row's loads are issued before the current row's arithmetic, so a warp waiting for
// the FP64 pipe (2 lanes per clock per SM on this GPU) already has its next loads in flight.
// Rows are visited in the same order as a plain loop, so sums come out bit for bit the same.
template <class Load, class Body>
__device__ __forceinline__ void rows_ahead(int tid, int stride, int n, Load load, Body body) {
  if (tid >= n) return;
  auto cur = load(tid);
  for (int i = tid; i < n; i += stride) {
    auto nxt = cur;
    if (i + stride < n) nxt = load(i + stride);
    body(i, cur);
    cur = nxt;
  }
}

// block partial of one or two values into part[q*nb + blockIdx.x]
__device__ __forceinline__ void write_partials(double a, double b, int nval, double* part, double* sh) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    if (nval > 1) b += __shfl_down_sync(0xffffffffu, b, o);
  }
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sh[w] = a; sh[32 + w] = b; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sa = 0.0, sb = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      sa += sh[q];
      if (nval > 1) sb += sh[32 + q];
    }
    part[blockIdx.x] = sa;
    if (nval > 1) part[gridDim.x + blockIdx.x] = sb;
  }
  __syncthreads();
}

// Solver arguments: only what the loop touches (keeps the kernel's register footprint small).
struct BiArgs {
  double *x, *r, *rb, *v, *p, *pinv, *s, *sinv, *t, *rinvM, *part, *P;
  const double *B, *diag, *val;
  const int *col, *cnt;
  Scal* sc;
  long long stride;
  int n, itermax;
  double tol;
  int warm;
};

// y_i = A_ii x_i + sum_k A_ik x_col(ik)  (sparse_atime, linear_solver.F90:254-273).  Four
// interleaved accumulators keep four independent load chains (column -> x) in flight per thread.
// x was written inside this kernel by other blocks: the grid barrier's release/acquire fences
// (gpu scope, followed by a CTA barrier) make those writes visible to the L1-cached loads
// (ld.global.ca) that follow, as in a cooperative-groups grid sync; neighbouring rows share most
// of their columns, so the gathers mostly hit L1.
__device__ __forceinline__ double spmv_row(const BiArgs& a, const double* xv, int i) {
  const int cnt = __ldg(a.cnt + i);
  const double* vp = a.val + i;
  const int* cp = a.col + i;
  const long long st = a.stride;
  double b0 = __ldg(a.diag + i) * __ldca(xv + i), b1 = 0.0, b2 = 0.0, b3 = 0.0;
  int k = 0;
  for (; k + 3 < cnt; k += 4) {
    const int c0 = __ldg(cp), c1 = __ldg(cp + st), c2 = __ldg(cp + 2 * st), c3 = __ldg(cp + 3 * st);
    const double v0 = __ldg(vp), v1 = __ldg(vp + st), v2 = __ldg(vp + 2 * st), v3 = __ldg(vp + 3 * st);
    b0 = fma(v0, __ldca(xv + c0), b0);
    b1 = fma(v1, __ldca(xv + c1), b1);
    b2 = fma(v2, __ldca(xv + c2), b2);
    b3 = fma(v3, __ldca(xv + c3), b3);
    cp += 4 * st;
    vp += 4 * st;
  }
  for (; k < cnt; ++k) {
    b0 = fma(__ldg(vp), __ldca(xv + __ldg(cp)), b0);
    cp += st;
    vp += st;
  }
  return (b0 + b1) + (b2 + b3);
}

// ---- mixed precision: FP64 recurrences, FP32 difference-form SpMV (see vebi_ppe.cu)
struct MxArgs {
  double *x, *r, *rb, *v, *p, *s, *t, *rinvM, *part, *P;
  float2 *pi, *si;                     // p_inv, s_inv as (hi, lo)
  const double *B, *rs;                // right-hand side, FP64 row sums
  const float* val32;
  const int *col, *cnt;
  Scal* sc;
  long long stride;
  int n, itermax;
  double tol;
  int warm;
};

// (hi, lo) FP32 pair of a double and back; conversions on the integer pipe (widen, narrow)
__device__ __forceinline__ float2 split2(double v) {
  const float h = narrow(v);
  return make_float2(h, narrow(v - widen(h)));
}
__device__ __forceinline__ double join2(float2 q) { return widen(q.x) + widen(q.y); }

__device__ __forceinline__ double spmv_diff32(const MxArgs& a, const float2* xv, int i) {
  const int cnt = __ldg(a.cnt + i);
  const float* vp = a.val32 + i;
  const int* cp = a.col + i;
  const long long st = a.stride;
  const float2 xi = __ldca(xv + i);
  float b0 = 0.0f, b1 = 0.0f, b2 = 0.0f, b3 = 0.0f;
  int k = 0;
  for (; k + 3 < cnt; k += 4) {
    const int c0 = __ldg(cp), c1 = __ldg(cp + st), c2 = __ldg(cp + 2 * st), c3 = __ldg(cp + 3 * st);
    const float v0 = __ldg(vp), v1 = __ldg(vp + st), v2 = __ldg(vp + 2 * st), v3 = __ldg(vp + 3 * st);
    const float2 x0 = __ldca(xv + c0), x1 = __ldca(xv + c1), x2 = __ldca(xv + c2), x3 = __ldca(xv + c3);
    b0 = fmaf(v0, (x0.x - xi.x) + (x0.y - xi.y), b0);
    b1 = fmaf(v1, (x1.x - xi.x) + (x1.y - xi.y), b1);
    b2 = fmaf(v2, (x2.x - xi.x) + (x2.y - xi.y), b2);
    b3 = fmaf(v3, (x3.x - xi.x) + (x3.y - xi.y), b3);
    cp += 4 * st;
    vp += 4 * st;
  }
  for (; k < cnt; ++k) {
    const float2 x0 = __ldca(xv + __ldg(cp));
    b0 = fmaf(__ldg(vp), (x0.x - xi.x) + (x0.y - xi.y), b0);
    cp += st;
    vp += st;
  }
  return fma(__ldg(a.rs + i), join2(xi), widen((b0 + b1) + (b2 + b3)));
}

}  // namespace vebi
