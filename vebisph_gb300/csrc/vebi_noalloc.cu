// vebi_noalloc.cu -- a pressure-Poisson solve that allocates nothing.
//
// Some callers cannot call cudaMalloc: a host framework whose own allocator owns all device
// memory (raw allocations are forbidden or invisible to its accounting), or a real-time time
// loop that must not allocate once it runs.  For them vebi_ppe_solve_noalloc runs the same
// BiCGSTAB as the time step on an ELL matrix and right-hand side the caller already holds in
// device memory, and keeps its Krylov vectors, block partial sums and barrier state in the
// file-scope array below instead of in allocated buffers.
//
// Limits and rules of the shared array:
//  * at most VEBI_NOALLOC_MAX_ROWS rows (65536); larger systems are rejected with VEBI_ERR_ARG;
//  * the array is ~4.3 MB and every GPU that loads this library holds it until the process exits;
//  * all calls on a device share it and it keeps the last call's contents: each call clears the
//    part that must start at zero (barrier counters, error word) before its kernel runs, and
//    calls that overlap on the GPU (two streams, or two host threads) race on it;
//  * the first call on a device looks up the array's device address (cudaGetSymbolAddress) with
//    that device current; make that first call before any stream capture begins.
//
// Errors: with iters_out or residual_out given, the call waits for the solve and returns its
// device-side status (VEBI_ERR_TIMEOUT if a grid barrier gave up).  With both NULL the call only
// enqueues the work and returns launch errors; a device-side failure then shows in the output,
// which the kernel fills with NaN.
#include <mutex>
#include <string>

#include "vebi_ctx.cuh"

namespace vebi {

namespace {

constexpr int NA_VECS = 8;              // r, r_bar, v, p, p_inv, s, s_inv, t
constexpr int NA_MAX_BLOCKS = 2048;     // co-resident blocks the solver may use
constexpr int NA_SLOTS = 12;            // partial-sum slots (as in the step's solver)
constexpr size_t NA_CTRL = 32;          // doubles reserved for control words (256 B)
constexpr size_t NA_DOUBLES =
    NA_CTRL + (size_t)NA_VECS * VEBI_NOALLOC_MAX_ROWS + (size_t)NA_SLOTS * NA_MAX_BLOCKS;

// The scratch.  Host code must not take its address directly: in host code this name is a
// host-side stand-in, not a device address.  Host code uses the address from
// cudaGetSymbolAddress (g_dev_addr below); device code may name it directly.
static __device__ __align__(256) double g_noalloc_scratch[NA_DOUBLES];

struct NaCtrl {  // lives in the first NA_CTRL doubles of the scratch
  unsigned int bar_count;
  unsigned int bar_gen;
  int error;
  int iters;
  int warnings;
  int pad;
  double residual;
};

struct NaArgs {
  const int* cnt;
  const int* col;
  const double* val;
  const double* diag;
  const double* rhs;
  double* x;
  long long stride;
  int n;
  int closed;
  int itermax;
  double tol;
  double* scratch;  // device address of g_noalloc_scratch
};

constexpr unsigned long long NA_SPIN_LIMIT = 1ull << 25;

__device__ __forceinline__ bool na_sync(NaCtrl* c) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* vgen = &c->bar_gen;
    volatile int* verr = &c->error;
    unsigned int g = *vgen;
    __threadfence();
    unsigned int arrived = atomicAdd(&c->bar_count, 1u) + 1u;
    if (arrived == gridDim.x) {
      atomicExch(&c->bar_count, 0u);
      __threadfence();
      atomicAdd(&c->bar_gen, 1u);
    } else {
      unsigned long long spins = 0;
      while (*vgen == g) {
        if (*verr != 0) break;
        if (++spins > NA_SPIN_LIMIT) {
          atomicCAS(&c->error, 0, VEBI_ERR_TIMEOUT);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *((volatile int*)&c->error) == 0;
}

// A block that leaves the solve on an error (a barrier that timed out, or saw another block's
// timeout) fills its rows of x with NaN, so a failed solve cannot pass for a result even when
// the caller reads nothing back.  Every block reaches the barrier that failed or returns from
// it with the error, and the blocks' rows (i = tid, tid + stride, ...) cover 0..n-1.
__device__ __forceinline__ void na_fail_rows(double* x, int n, int tid, int stride) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  for (int i = tid; i < n; i += stride) x[i] = nan;
}

__device__ __forceinline__ void na_partials(double a, double b, int nval, double* part, double* sh) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sh[w] = a; sh[32 + w] = b; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sa = 0.0, sb = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { sa += sh[q]; sb += sh[32 + q]; }
    part[blockIdx.x] = sa;
    if (nval > 1) part[gridDim.x + blockIdx.x] = sb;
  }
  __syncthreads();
}

__device__ __forceinline__ void na_reduce(const double* part, int nb, int nval, double* out, double* shv) {
  if (threadIdx.x < 32) {
    for (int q = 0; q < nval; ++q) {
      double v = 0.0;
      for (int b = threadIdx.x; b < nb; b += 32) v += __ldcg(part + (size_t)q * nb + b);
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (threadIdx.x == 0) shv[q] = v;
    }
  }
  __syncthreads();
  for (int q = 0; q < nval; ++q) out[q] = shv[q];
  __syncthreads();
}

__device__ __forceinline__ double na_spmv(const NaArgs& a, const double* xv, int i) {
  double bb = a.diag[i] * __ldcg(xv + i);
  const int cnt = a.cnt[i];
  for (int k = 0; k < cnt; ++k) {
    size_t e = (size_t)k * a.stride + i;
    bb = fma(a.val[e], __ldcg(xv + a.col[e]), bb);
  }
  return bb;
}

// SPARSE_PBICGSTAB_nonull / SPARSE_PBICGSTAB (linear_solver.F90:275-425 / 82-227) with x0 = 0
template <bool NONULL>
__global__ void __launch_bounds__(TPB) k_na_bicgstab(NaArgs a) {
  __shared__ double sh[64];
  __shared__ double shv[4];
  NaCtrl* ctl = reinterpret_cast<NaCtrl*>(a.scratch);
  const size_t N = VEBI_NOALLOC_MAX_ROWS;
  double* base = a.scratch + NA_CTRL;
  double *r = base, *rb = base + N, *v = base + 2 * N, *p = base + 3 * N, *pinv = base + 4 * N;
  double *sv = base + 5 * N, *sinv = base + 6 * N, *t = base + 7 * N;
  double* part = base + (size_t)NA_VECS * N;
  const int n = a.n, nb = gridDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  double* x = a.x;
  const double small = NONULL ? 1.0e-6 : 4.0;
  auto den = [&](int i) -> double { return NONULL ? (1.0 + 1.0e-15) : (a.diag[i] + 1.0e-15); };
  double red[4];
  double acc = 0.0;
  for (int i = tid; i < n; i += stride) {
    double bi = a.rhs[i];
    x[i] = 0.0;
    r[i] = bi;
    rb[i] = bi;
    v[i] = 0.0;
    p[i] = 0.0;
    acc += bi * bi;
  }
  na_partials(acc, 0.0, 1, part + 10 * (size_t)nb, sh);
  if (!na_sync(ctl)) { na_fail_rows(x, n, tid, stride); return; }
  na_reduce(part + 10 * (size_t)nb, nb, 1, red, shv);
  double rho = red[0], rho0 = 1.0, alpha = 1.0, omega = 1.0, n2r0 = 1.0, n2s0 = 1.0, resid = 0.0;
  int iter = 1, warn = 0;
  bool done = false;
  while (iter <= a.itermax) {
    if (rho == 0.0) { warn |= VEBI_WARN_BICGSTAB_BREAKDOWN; done = true; break; }
    double beta = rho / (rho0 + 1.0e-15) * alpha / (omega + 1.0e-15);
    acc = 0.0;
    for (int i = tid; i < n; i += stride) {
      double pi = (iter == 1) ? r[i] : r[i] + beta * (p[i] - omega * v[i]);
      p[i] = pi;
      acc += pi;
    }
    if (NONULL) {
      na_partials(acc, 0.0, 1, part, sh);
      if (!na_sync(ctl)) { na_fail_rows(x, n, tid, stride); return; }
      na_reduce(part, nb, 1, red, shv);
      const double mean = red[0] / (double)n;
      for (int i = tid; i < n; i += stride) {
        double pi = p[i] - mean;
        p[i] = pi;
        pinv[i] = pi / den(i);
      }
    } else {
      for (int i = tid; i < n; i += stride) pinv[i] = p[i] / den(i);
    }
    if (!na_sync(ctl)) { na_fail_rows(x, n, tid, stride); return; }
    acc = 0.0;
    for (int i = tid; i < n; i += stride) {
      double vi = na_spmv(a, pinv, i);
      v[i] = vi;
      acc += rb[i] * vi;
    }
    na_partials(acc, 0.0, 1, part + 2 * (size_t)nb, sh);
    if (!na_sync(ctl)) { na_fail_rows(x, n, tid, stride); return; }
    na_reduce(part + 2 * (size_t)nb, nb, 1, red, shv);
    alpha = rho / (red[0] + 1.0e-15);
    double a2 = 0.0;
    acc = 0.0;
    for (int i = tid; i < n; i += stride) {
      double si = r[i] - alpha * v[i];
      sv[i] = si;
      acc += si * si;
      a2 += si;
    }
    na_partials(acc, a2, 2, part + 4 * (size_t)nb, sh);
    if (!na_sync(ctl)) { na_fail_rows(x, n, tid, stride); return; }
    na_reduce(part + 4 * (size_t)nb, nb, 2, red, shv);
    const double n2s = red[0], mean_s = red[1] / (double)n;
    if (iter == 1) n2s0 = (n2s <= small) ? 1.0 : n2s;
    if (n2s <= a.tol * a.tol * n2s0) {
      for (int i = tid; i < n; i += stride) x[i] = x[i] + alpha * pinv[i];
      resid = sqrt(n2s / n2s0);
      done = true;
      break;
    }
    for (int i = tid; i < n; i += stride) {
      double si = sv[i];
      if (NONULL) { si = si - mean_s; sv[i] = si; }
      sinv[i] = si / den(i);
    }
    if (!na_sync(ctl)) { na_fail_rows(x, n, tid, stride); return; }
    acc = 0.0;
    a2 = 0.0;
    for (int i = tid; i < n; i += stride) {
      double ti = na_spmv(a, sinv, i);
      t[i] = ti;
      acc += ti * sv[i];
      a2 += ti * ti;
    }
    na_partials(acc, a2, 2, part + 6 * (size_t)nb, sh);
    if (!na_sync(ctl)) { na_fail_rows(x, n, tid, stride); return; }
    na_reduce(part + 6 * (size_t)nb, nb, 2, red, shv);
    omega = red[0] / (red[1] + 1.0e-15);
    acc = 0.0;
    a2 = 0.0;
    for (int i = tid; i < n; i += stride) {
      x[i] = x[i] + alpha * pinv[i] + omega * sinv[i];
      double ri = sv[i] - omega * t[i];
      r[i] = ri;
      acc += ri * ri;
      a2 += rb[i] * ri;
    }
    na_partials(acc, a2, 2, part + 8 * (size_t)nb, sh);
    if (!na_sync(ctl)) { na_fail_rows(x, n, tid, stride); return; }
    na_reduce(part + 8 * (size_t)nb, nb, 2, red, shv);
    const double n2r = red[0];
    if (iter == 1) n2r0 = (n2r <= small) ? 1.0 : n2r;
    resid = sqrt(n2r / n2r0);
    if (n2r <= a.tol * a.tol * n2r0) { done = true; break; }
    iter = iter + 1;
    rho0 = rho;
    rho = red[1];
  }
  if (!done) warn |= VEBI_WARN_MAXITER;
  if (tid == 0) {
    ctl->iters = iter;
    ctl->residual = resid;
    ctl->warnings = warn;
  }
}

// per-device set-up: the scratch's device address, looked up with that device current
constexpr int NA_MAX_DEVICES = 64;
std::mutex g_mu;
double* g_dev_addr[NA_MAX_DEVICES] = {};
int g_blocks[NA_MAX_DEVICES] = {};

}  // namespace
}  // namespace vebi

extern "C" void vebi_set_last_error_internal(const char* msg);

namespace vebi {
namespace {

int na_fail(int code, const std::string& m) {
  vebi_set_last_error_internal(m.c_str());
  return code;
}

}  // namespace
}  // namespace vebi

using namespace vebi;

extern "C" int vebi_ppe_solve_noalloc(const int32_t* ij_count, const int32_t* ppe_col, const double* ppe_val,
                                      const double* ppe_diag, const double* rhs, double* x, int32_t n,
                                      int64_t ell_stride, int32_t closed_domain, double tol, int32_t itermax,
                                      void* stream, int32_t* iters_out, double* residual_out) {
  if (!ij_count || !ppe_col || !ppe_val || !ppe_diag || !rhs || !x)
    return na_fail(VEBI_ERR_ARG, "vebi_ppe_solve_noalloc: null array");
  if (n < 1 || n > VEBI_NOALLOC_MAX_ROWS)
    return na_fail(VEBI_ERR_ARG, "vebi_ppe_solve_noalloc: n must be in 1..VEBI_NOALLOC_MAX_ROWS (65536)");
  if (ell_stride < n) return na_fail(VEBI_ERR_ARG, "vebi_ppe_solve_noalloc: ell_stride < n");
  if (!(tol > 0.0) || itermax < 1) return na_fail(VEBI_ERR_ARG, "vebi_ppe_solve_noalloc: bad tol/itermax");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES)
    return na_fail(VEBI_ERR_NO_DEVICE, "vebi_ppe_solve_noalloc: no current CUDA device");
  double* addr = nullptr;
  int blocks = 0;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_dev_addr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return na_fail(VEBI_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      int nsm = 0, per = 0, per2 = 0;
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_na_bicgstab<true>, TPB, 0);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, k_na_bicgstab<false>, TPB, 0);
      per = per < per2 ? per : per2;
      long long b = (long long)(per < 1 ? 1 : per) * (nsm < 1 ? 1 : nsm);
      g_blocks[dev] = (int)(b > NA_MAX_BLOCKS ? NA_MAX_BLOCKS : b);
      g_dev_addr[dev] = static_cast<double*>(p);
    }
    addr = g_dev_addr[dev];
    blocks = g_blocks[dev];
  }
  long long need = ((long long)n + TPB - 1) / TPB;
  if (need < blocks) blocks = (int)need;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (iters_out || residual_out) {
    // the read-back waits for the stream, which a stream being captured cannot do
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t ce = cudaStreamIsCapturing(st, &cs);
    if (ce != cudaSuccess) return na_fail(VEBI_ERR_CUDA, std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(ce));
    if (cs != cudaStreamCaptureStatusNone)
      return na_fail(VEBI_ERR_ARG, "vebi_ppe_solve_noalloc: iters_out and residual_out must be NULL while the "
                                   "stream is being captured (the read-back waits for the stream)");
  }
  // clear the control words; the vectors are initialised by the kernel itself
  cudaError_t e = cudaMemsetAsync(addr, 0, NA_CTRL * sizeof(double), st);
  if (e != cudaSuccess) return na_fail(VEBI_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  NaArgs a{ij_count, ppe_col, ppe_val, ppe_diag, rhs, x, (long long)ell_stride, n, closed_domain ? 1 : 0,
           itermax, tol, addr};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(TPB);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = closed_domain ? cudaLaunchKernelEx(&cfg, k_na_bicgstab<true>, a) : cudaLaunchKernelEx(&cfg, k_na_bicgstab<false>, a);
  if (e != cudaSuccess) return na_fail(VEBI_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  if (iters_out || residual_out) {
    NaCtrl ctl;
    e = cudaMemcpyAsync(&ctl, addr, sizeof(NaCtrl), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return na_fail(VEBI_ERR_CUDA, std::string("read-back: ") + cudaGetErrorString(e));
    if (iters_out) *iters_out = ctl.iters;
    if (residual_out) *residual_out = ctl.residual;
    if (ctl.error) return na_fail(ctl.error, "vebi_ppe_solve_noalloc: device-side error");
  }
  return VEBI_OK;
}
