// vebi_ppe.cu -- pressure Poisson equation: right-hand side, assembly and BiCGSTAB.
//
//  ppe_solve_in_house_simple_dirichlet   ppe_solve_in_house_simple_dirichlet.F90:1-158
//  SPARSE_PBICGSTAB_nonull (closed)       linear_solver.F90:275-425
//  SPARSE_PBICGSTAB (open, Jacobi)        linear_solver.F90:82-227
//  sparse_atime, vtime, norm, remove_dc, inverseM
//
// Matrix layout.  The reference stores the Laplacian in Numerical Recipes row-indexed form:
// A(1:n) the diagonal, then one off-diagonal slot per neighbour of each row, in neighbour
// order (ppe...:60-121).  Here the same slots live in ELL form, ppe_col/ppe_val[k][i],
// k < ij_count(i), beside ppe_diag[i]; slot k of row i is NR slot ia(i)+k-1.  A mirror
// neighbour maps to its parent's column; duplicate columns accumulate into the last slot
// written for that column and leave 0 in the earlier ones, as the reference does.
//
// Solver.  One persistent cooperative kernel runs the whole BiCGSTAB loop.  Every global
// reduction is a block partial written to `partials` followed by a bounded grid barrier, after
// which every block sums the partials in the same fixed order, so all blocks hold identical
// scalars and take identical branches.  Seven barriers per iteration (closed domain):
//   p-update+sum(p) | p-=mean, p_inv | v=A p_inv, (r_bar,v) | s, |s|^2, sum(s) |
//   s-=mean, s_inv | t=A s_inv, (t,s), |t|^2 | x,r update, |r|^2, (r_bar,r)
// The barrier spins are bounded: on timeout the kernel records VEBI_ERR_TIMEOUT and returns.
#include "vebi_solver.cuh"

namespace vebi {

#define ELL(k, i) ((size_t)(k) * c.npfb + (i))

// ---------------------------------------------------------------------- right-hand side
__global__ void k_ppe_rhs(Consts c, Dev d) {
  __shared__ double sh[TPB / 32 + 1];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double b = 0.0;
  if (i < c.npfb) {
    const double ui = d.ux2[i], vi = d.uy2[i];  // u* (predictor output, mirrors included)
    const double K11 = d.kgcm[0][i], K21 = d.kgcm[1][i], K12 = d.kgcm[2][i], K22 = d.kgcm[3][i];
    double fb = 0.0;
    const int cnt = d.ij_count[i];
    for (int k = 0; k < cnt; ++k) {
      int j = d.ij_link[ELL(k, i)];
      double u1 = ui - d.ux2[j], u2 = vi - d.uy2[j];
      double w1 = d.wGx[ELL(k, i)], w2 = d.wGy[ELL(k, i)];
      double kw1 = K11 * w1 + K12 * w2, kw2 = K21 * w1 + K22 * w2;
      fb = fb - (u1 * kw1 + u2 * kw2);
    }
    b = fb / d.s->dt;
    d.ppe_B[i] = b;
  }
  double bs = block_sum<TPB>(b, sh);
  if (threadIdx.x == 0) d.partials[blockIdx.x] = bs;
}

__global__ void k_ppe_mean(Consts c, Dev d, int nblk) {
  __shared__ double sh[TPB / 32 + 1];
  double s = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += d.partials[b];
  s = block_sum<TPB>(s, sh);
  if (threadIdx.x == 0) d.s->rhs_mean = (c.open_domain == 0) ? s / (double)c.npfb : 0.0;
}

// ---------------------------------------------------------------------- assembly
// Rows without a mirror neighbour (all but a thin layer along the boundaries) hold distinct
// columns, so one pass writes each slot once with the same value (0 + temp) the general path
// accumulates; the first mirror neighbour sends the row to the general path, which starts over.
// The mixed step (wL32 given) also writes the FP32 off-diagonal values and the FP64 row sums
// diag + sum_k A_ik, in slot order, that its difference-form SpMV reads.  Its solvers read no
// FP64 off-diagonal value, so a mixed row without mirrors, smoothing or a free-surface
// condition takes a single FP32 pass: the FP32 values directly (0 + (-w) rounded to FP32 is -w,
// +0 for a zero weight), the diagonal sum_k w_k by compensated FP32 summation (TwoSum, Knuth;
// exact unless the sum needs more than 48 bits) widened to FP64 once, and the row sum diag +
// sum_k A_ik, which is exactly 0 for such a row.  This GPU issues FP64 at 1/64 of the FP32 rate,
// and the FP64 form of this pass was bound by it.  keep64 (the adjoint's recompute of a
// recorded step, which tapes the FP64 matrix) takes the FP64 form.
__device__ __forceinline__ double plus_zero(double x) {  // 0.0 + x without the FP64 pipe
  const long long b = __double_as_longlong(x);
  return __longlong_as_double(b == (long long)0x8000000000000000ull ? 0ll : b);
}

__global__ void k_ppe_assemble(Consts c, Dev d, const float* __restrict__ wL32, int keep64) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.npfb) return;
  double B = d.ppe_B[i];
  if (c.open_domain == 0) B = B - d.s->rhs_mean;
  const int cnt = d.ij_count[i];
  const bool smooth = c.open_domain == 1 && d.n_surf[i] != 1 && d.ppe_smooth[i] != 1.0;
  bool w64 = wL32 == nullptr || keep64 || smooth || d.n_surf[i] != 0;
  bool any_mirror = false;
  double Adiag = 0.0;
  if (!w64) {  // mixed, FP32 pass, four slots at a time with their loads ahead of their stores
    float hs = 0.f, hc = 0.f;
    for (int k0 = 0; k0 < cnt && !any_mirror; k0 += 4) {
      int j4[4];
      float w4[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const bool in = k0 + u < cnt;
        j4[u] = in ? d.ij_link[ELL(k0 + u, i)] : 0;
        w4[u] = in ? wL32[ELL(k0 + u, i)] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (k0 + u >= cnt) break;
        const int j = j4[u];
        const float w = w4[u];
        any_mirror |= j >= c.npfb;  // such a row starts over in the general path below
        const float t = hs + w, bp = t - hs;
        hc += (hs - (t - bp)) + (w - bp);
        hs = t;
        d.ppe_col[ELL(k0 + u, i)] = j;
        d.ppe_val32[ELL(k0 + u, i)] = w == 0.f ? 0.f : -w;
      }
    }
    if (!any_mirror) {
      d.ppe_diag[i] = widen(hs) + widen(hc);
      d.ppe_B[i] = B;
      d.rowsum[i] = 0.0;
      if (c.open_domain == 1) d.bM[i] = 1.0 / (d.ppe_diag[i] + 1.0e-15);
      return;
    }
  } else {  // FP64 pass, four slots at a time as above
    for (int k0 = 0; k0 < cnt && !any_mirror; k0 += 4) {
      int j4[4];
      double t4[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const bool in = k0 + u < cnt;
        j4[u] = in ? d.ij_link[ELL(k0 + u, i)] : 0;
        t4[u] = in ? (wL32 ? -widen(wL32[ELL(k0 + u, i)]) : -d.wL[ELL(k0 + u, i)]) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (k0 + u >= cnt) break;
        any_mirror |= j4[u] >= c.npfb;  // such a row starts over in the general path below
        Adiag = Adiag - t4[u];
        d.ppe_col[ELL(k0 + u, i)] = j4[u];
        d.ppe_val[ELL(k0 + u, i)] = plus_zero(t4[u]);
      }
    }
  }
  if (any_mirror) {
    for (int k = 0; k < cnt; ++k) {
      int j = d.ij_link[ELL(k, i)];
      d.ppe_col[ELL(k, i)] = j >= c.npfb ? d.irel[j] : j;
      d.ppe_val[ELL(k, i)] = 0.0;
    }
    Adiag = 0.0;
    for (int k = 0; k < cnt; ++k) {
      int j = d.ij_link[ELL(k, i)];
      // the mixed step assembles in FP64 from its FP32 Morris weights
      double temp = wL32 ? -(double)wL32[ELL(k, i)] : -d.wL[ELL(k, i)];
      Adiag = Adiag - temp;
      int colk = j;
      bool self = false;
      if (j >= c.npfb) {
        colk = d.irel[j];
        if (colk == i) self = true;
        B = B - d.dP_mp[j] * temp;
      }
      if (self) {
        Adiag = Adiag + temp;
      } else {
        int nt = k;  // last slot holding this column
        for (int kk = cnt - 1; kk >= 0; --kk)
          if (d.ppe_col[ELL(kk, i)] == colk) { nt = kk; break; }
        d.ppe_val[ELL(nt, i)] = d.ppe_val[ELL(nt, i)] + temp;
      }
    }
  }
  if (d.n_surf[i] != 0) Adiag = 1.0e30;
  const double diag = 0.0 + Adiag;
  d.ppe_diag[i] = diag;
  if (smooth) {
    const double ps = d.ppe_smooth[i];
    B = B * ps;
    for (int k = 0; k < cnt; ++k) d.ppe_val[ELL(k, i)] = d.ppe_val[ELL(k, i)] * ps;
  }
  d.ppe_B[i] = B;
  if (wL32) {
    double rs = diag;
    for (int k = 0; k < cnt; ++k) {
      const double v = d.ppe_val[ELL(k, i)];
      rs += v;
      d.ppe_val32[ELL(k, i)] = (float)v;
    }
    d.rowsum[i] = rs;
    if (c.open_domain == 1) d.bM[i] = 1.0 / (diag + 1.0e-15);
  }
}

// ---------------------------------------------------------------------- BiCGSTAB
// SPARSE_PBICGSTAB_nonull (NONULL) / SPARSE_PBICGSTAB with x0 = 0.  The recurrences are the
// reference's; the arithmetic uses fused multiply-adds and multiplies by 1/(M+1e-15) instead
// of dividing by it (inverseM), which changes results by rounding only.
template <bool NONULL>
__global__ void __launch_bounds__(TPB, 5) k_bicgstab(BiArgs a) {
  __shared__ double sh[64];
  __shared__ double shv[4];
  const int n = a.n;
  const int nb = gridDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  Scal* s = a.sc;
  if (*((volatile int*)&s->first_error)) return;  // this state already failed a step
  double* part = a.part;
  const double rinv1 = 1.0 / (1.0 + 1.0e-15);
  const double small = NONULL ? 1.0e-6 : 4.0;  // open solver: the integer expression 10-6
  double red[4];
  double acc = 0.0;
  if (a.warm) {  // x0 = P of the previous step: r0 = B - A x0 (the SpMV reads x through pinv)
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
    if (!NONULL) a.rinvM[i] = 1.0 / (__ldg(a.diag + i) + 1.0e-15);
    acc = fma(bi, bi, acc);
  }
  // slot 10 for the initial reduction: slot 0 is rewritten before every block has read it
  write_partials(acc, 0.0, 1, part + 10 * (size_t)nb, sh);
  if (!grid_sync(s)) return;
  reduce_partials(part + 10 * (size_t)nb, nb, 1, red, shv);
  double rho = red[0], alpha = 1.0, omega = 1.0;
  double n2r0 = 1.0, n2s0 = 1.0, resid = 0.0;
  double beta = 0.0;  // for iteration 2 on, derived with the previous iteration's last reduction
  int iter = 1, warn = 0;
  bool done = false;
  const double dn = (double)n;
  while (iter <= a.itermax) {
    if (rho == 0.0) { warn |= VEBI_WARN_BICGSTAB_BREAKDOWN; done = true; break; }
    // p = r + beta (p - omega v).  The vector passes load each row's operands one row ahead
    // (rows_ahead), so a row's loads are in flight before the previous row's stores: the
    // compiler cannot move a load of one array above a store to another that may alias it.
    acc = 0.0;
    rows_ahead(
        tid, stride, n, [&](int i) { return make_double3(a.r[i], a.v[i], a.p[i]); },
        [&](int i, const double3& o) {
          const double pi = (iter == 1) ? o.x : fma(beta, fma(-omega, o.y, o.z), o.x);
          a.p[i] = pi;
          acc += pi;
        });
    double* slot = part;
    if (NONULL) {
      write_partials(acc, 0.0, 1, slot, sh);
      if (!grid_sync(s)) return;
      reduce_partials(slot, nb, 1, red, shv, [=](double* v) { v[0] = v[0] / dn; });
      const double mean = red[0];
      rows_ahead(
          tid, stride, n, [&](int i) { return a.p[i]; },
          [&](int i, double p) {
            const double pi = p - mean;
            a.p[i] = pi;
            a.pinv[i] = pi * rinv1;
          });
    } else {
      rows_ahead(
          tid, stride, n, [&](int i) { return make_double2(a.p[i], a.rinvM[i]); },
          [&](int i, const double2& o) { a.pinv[i] = o.x * o.y; });
    }
    if (!grid_sync(s)) return;
    // v = A p_inv ; (r_bar, v)
    acc = 0.0;
    for (int i = tid; i < n; i += stride) {
      double vi = spmv_row(a, a.pinv, i);
      a.v[i] = vi;
      acc = fma(a.rb[i], vi, acc);
    }
    slot = part + 2 * (size_t)nb;
    write_partials(acc, 0.0, 1, slot, sh);
    if (!grid_sync(s)) return;
    reduce_partials(slot, nb, 1, red, shv, [=](double* v) { v[0] = rho / (v[0] + 1.0e-15); });
    alpha = red[0];
    // s = r - alpha v ; |s|^2 ; sum(s)
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
    slot = part + 4 * (size_t)nb;
    write_partials(acc, a2, 2, slot, sh);
    if (!grid_sync(s)) return;
    reduce_partials(slot, nb, 2, red, shv, [=](double* v) { v[1] = v[1] / dn; });
    const double n2s = red[0];
    const double mean_s = red[1];
    if (iter == 1) n2s0 = (n2s <= small) ? 1.0 : n2s;
    if (n2s <= a.tol * a.tol * n2s0) {
      for (int i = tid; i < n; i += stride) a.x[i] = fma(alpha, a.pinv[i], a.x[i]);
      resid = sqrt(n2s / n2s0);
      done = true;
      break;
    }
    // s -= mean (closed) ; s_inv
    rows_ahead(
        tid, stride, n, [&](int i) { return make_double2(a.s[i], NONULL ? rinv1 : a.rinvM[i]); },
        [&](int i, const double2& o) {
          double si = o.x;
          if (NONULL) { si = si - mean_s; a.s[i] = si; }
          a.sinv[i] = si * o.y;
        });
    if (!grid_sync(s)) return;
    // t = A s_inv ; (t, s) ; |t|^2
    acc = 0.0;
    a2 = 0.0;
    for (int i = tid; i < n; i += stride) {
      double ti = spmv_row(a, a.sinv, i);
      a.t[i] = ti;
      acc = fma(ti, a.s[i], acc);
      a2 = fma(ti, ti, a2);
    }
    slot = part + 6 * (size_t)nb;
    write_partials(acc, a2, 2, slot, sh);
    if (!grid_sync(s)) return;
    reduce_partials(slot, nb, 2, red, shv, [](double* v) { v[0] = v[0] / (v[1] + 1.0e-15); });
    omega = red[0];
    // x, r update ; |r|^2 ; (r_bar, r) for the next rho
    acc = 0.0;
    a2 = 0.0;
    struct XRow {
      double s, p, x, t, sv, rb;
    };
    rows_ahead(
        tid, stride, n, [&](int i) { return XRow{a.sinv[i], a.pinv[i], a.x[i], a.t[i], a.s[i], a.rb[i]}; },
        [&](int i, const XRow& o) {
          a.x[i] = fma(omega, o.s, fma(alpha, o.p, o.x));
          const double ri = fma(-omega, o.t, o.sv);
          a.r[i] = ri;
          acc = fma(ri, ri, acc);
          a2 = fma(o.rb, ri, a2);
        });
    slot = part + 8 * (size_t)nb;
    write_partials(acc, a2, 2, slot, sh);
    if (!grid_sync(s)) return;
    // v[2] = the relative residual, v[3] = the next iteration's beta from the new rho v[1]
    reduce_partials(slot, nb, 2, red, shv, [=](double* v) {
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

int ppe_solver_blocks(int device, int nsm) {
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_bicgstab<true>, TPB, 0);
  int per2 = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, k_bicgstab<false>, TPB, 0);
  per = per < per2 ? per : per2;
  if (per < 1) per = 1;
  (void)device;
  return per * nsm;
}

void launch_ppe_mixed_solve(Ctx& x);
void launch_ppe_mg(Ctx& x);
void launch_ppe_rhs32(Ctx& x);

void launch_ppe(Ctx& x) {
  const Consts& c = x.c;
  int g = grid_for(c.npfb);
  stage_mark(x, 9);
  const bool mixed = x.precision == VEBI_PREC_MIXED;
  if (mixed) launch_ppe_rhs32(x);
  else VEBI_LAUNCH(x, k_ppe_rhs, g, TPB, c, x.d);
  VEBI_LAUNCH(x, k_ppe_mean, 1, TPB, c, x.d, g);
  VEBI_LAUNCH(x, k_ppe_assemble, g, TPB, c, x.d, mixed ? (const float*)x.d.wL32 : (const float*)nullptr,
              x.rep_p != nullptr ? 1 : 0);
  stage_mark(x, 10);
  if (x.rep_p) {  // a recorded step recomputed by the adjoint: its solution is known
    cudaMemcpyAsync(x.d.p, x.rep_p, sizeof(double) * (size_t)c.npfb, cudaMemcpyDeviceToDevice, x.st);
    return;
  }
  if (x.precision == VEBI_PREC_MIXED) {
    launch_ppe_mixed_solve(x);
    return;
  }
  if (c.precond) {
    launch_ppe_mg(x);
    return;
  }
  // persistent cooperative launch: all blocks co-resident, so the grid barrier is safe
  int nblk = x.coop_blocks;
  const long long rows_per_block = (long long)TPB * (x.solver_rows_per_thread > 0 ? x.solver_rows_per_thread : 1);
  long long need = (c.npfb + rows_per_block - 1) / rows_per_block;
  if (need < nblk) nblk = (int)(need < 1 ? 1 : need);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblk);
  cfg.blockDim = dim3(TPB);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = x.st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const Dev& d = x.d;
  BiArgs a{d.bx, d.br, d.brb, d.bv, d.bp, d.bpi, d.bs, d.bsi, d.bt, d.bM, d.partials, d.p,
           d.ppe_B, d.ppe_diag, d.ppe_val, d.ppe_col, d.ij_count, d.s, (long long)c.npfb, c.npfb, c.itermax, c.tol,
           c.warm_start};
  if (c.open_domain == 0) cudaLaunchKernelEx(&cfg, k_bicgstab<true>, a);
  else cudaLaunchKernelEx(&cfg, k_bicgstab<false>, a);
  x.launches++;
}

// The persistent FP64 BiCGSTAB on a caller's system (the adjoint's transposed PPE): the same
// grid and kernels as the step's solve, other arrays.
void launch_bicgstab_on(Ctx& x, const BiArgs& a, bool nonull) {
  int nblk = x.coop_blocks;
  const long long need = (a.n + TPB - 1) / TPB;
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
  if (nonull) cudaLaunchKernelEx(&cfg, k_bicgstab<true>, a);
  else cudaLaunchKernelEx(&cfg, k_bicgstab<false>, a);
  x.launches++;
}

}  // namespace vebi

// =====================================================================================
// Mixed precision PPE (VEBI_PREC_MIXED): the BiCGSTAB of the FP64 step with an FP32 SpMV.
//
// FP32 Krylov recurrences cannot solve this system at scale: the attainable relative residual
// of a Krylov method is ~ eps * cond(A), and the Laplacian of a 4M-particle domain has
// cond ~ 1e7, so FP32 (eps 6e-8) stalls near 1 (an FP32 inner solver inside FP64 refinement
// diverged on the 4M cylinder).  The recurrences, dot products and the solution therefore stay
// FP64, and the SpMV -- the bytes and the FP64 instructions of the solve -- runs in FP32 in the
// Laplacian's difference form
//     y_i = rowsum_i * x_i + sum_k A_ik (x_col(ik) - x_i),       rowsum_i = A_ii + sum_k A_ik,
// with rowsum in FP64 (0 up to rounding except Dirichlet rows) and the sum in FP32.  The
// vectors the SpMV gathers (p_inv, s_inv) are kept as FP32 hi/lo pairs (x = hi + lo), so
// x_j - x_i = (hi_j - hi_i) + (lo_j - lo_i) keeps FP32 accuracy relative to the difference
// instead of to |x|.  Per off-diagonal slot the solve reads 8 B (FP32 value + column) instead
// of 12 B, and performs no FP64 operation in the SpMV.
namespace vebi {

template <bool NONULL>
__global__ void __launch_bounds__(TPB, 5) k_bicgstab_mixed(MxArgs a) {
  __shared__ double sh[64];
  __shared__ double shv[4];
  const int n = a.n;
  const int nb = gridDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  Scal* s = a.sc;
  if (*((volatile int*)&s->first_error)) return;  // this state already failed a step
  double* part = a.part;
  const double rinv1 = 1.0 / (1.0 + 1.0e-15);
  const double small = NONULL ? 1.0e-6 : 4.0;
  double red[4];
  double acc = 0.0;
  if (a.warm) {  // x0 = P of the previous step
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
  double n2r0 = 1.0, n2s0 = 1.0, resid = 0.0;
  double beta = 0.0;  // for iteration 2 on, derived with the previous iteration's last reduction
  int iter = 1, warn = 0;
  bool done = false;
  const double dn = (double)n;
  while (iter <= a.itermax) {
    if (rho == 0.0) { warn |= VEBI_WARN_BICGSTAB_BREAKDOWN; done = true; break; }
    acc = 0.0;
    // vector passes: each row's operands loaded one row ahead (rows_ahead)
    rows_ahead(
        tid, stride, n, [&](int i) { return make_double3(a.r[i], a.v[i], a.p[i]); },
        [&](int i, const double3& o) {
          const double pi = (iter == 1) ? o.x : fma(beta, fma(-omega, o.y, o.z), o.x);
          a.p[i] = pi;
          acc += pi;
        });
    double mean = 0.0;
    if (NONULL) {
      write_partials(acc, 0.0, 1, part, sh);
      if (!grid_sync(s)) return;
      reduce_partials(part, nb, 1, red, shv, [=](double* v) { v[0] = v[0] / dn; });
      mean = red[0];
    }
    rows_ahead(
        tid, stride, n, [&](int i) { return make_double2(a.p[i], NONULL ? rinv1 : a.rinvM[i]); },
        [&](int i, const double2& o) {
          double pi = o.x;
          if (NONULL) { pi = pi - mean; a.p[i] = pi; }
          a.pi[i] = split2(pi * o.y);
        });
    if (!grid_sync(s)) return;
    acc = 0.0;
    for (int i = tid; i < n; i += stride) {
      double vi = spmv_diff32(a, a.pi, i);
      a.v[i] = vi;
      acc = fma(a.rb[i], vi, acc);
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
      for (int i = tid; i < n; i += stride) a.x[i] = fma(alpha, join2(a.pi[i]), a.x[i]);
      resid = sqrt(n2s / n2s0);
      done = true;
      break;
    }
    rows_ahead(
        tid, stride, n, [&](int i) { return make_double2(a.s[i], NONULL ? rinv1 : a.rinvM[i]); },
        [&](int i, const double2& o) {
          double si = o.x;
          if (NONULL) { si = si - mean_s; a.s[i] = si; }
          a.si[i] = split2(si * o.y);
        });
    if (!grid_sync(s)) return;
    acc = 0.0;
    a2 = 0.0;
    for (int i = tid; i < n; i += stride) {
      double ti = spmv_diff32(a, a.si, i);
      a.t[i] = ti;
      acc = fma(ti, a.s[i], acc);
      a2 = fma(ti, ti, a2);
    }
    write_partials(acc, a2, 2, part + 6 * (size_t)nb, sh);
    if (!grid_sync(s)) return;
    reduce_partials(part + 6 * (size_t)nb, nb, 2, red, shv, [](double* v) { v[0] = v[0] / (v[1] + 1.0e-15); });
    omega = red[0];
    acc = 0.0;
    a2 = 0.0;
    struct XRow {
      float2 s, p;
      double x, t, sv, rb;
    };
    rows_ahead(
        tid, stride, n, [&](int i) { return XRow{a.si[i], a.pi[i], a.x[i], a.t[i], a.s[i], a.rb[i]}; },
        [&](int i, const XRow& o) {
          a.x[i] = fma(omega, join2(o.s), fma(alpha, join2(o.p), o.x));
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

int ppe_mixed_blocks(int nsm) {
  int per = 0, per2 = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_bicgstab_mixed<true>, TPB, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, k_bicgstab_mixed<false>, TPB, 0);
  per = per < per2 ? per : per2;
  if (per < 1) per = 1;
  return per * nsm;
}

void launch_ppe_mg_mixed(Ctx& x);

void launch_ppe_mixed_solve(Ctx& x) {
  const Consts& c = x.c;
  if (c.precond) {
    launch_ppe_mg_mixed(x);
    return;
  }
  int nblk = x.coop_blocks_mixed;
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
  const Dev& d = x.d;
  MxArgs a{d.bx, d.br, d.brb, d.bv, d.bp, d.bs, d.bt, d.bM, d.partials, d.p, d.pi2, d.si2, d.ppe_B, d.rowsum,
           d.ppe_val32, d.ppe_col, d.ij_count, d.s, (long long)c.npfb, c.npfb, c.itermax, c.tol, c.warm_start};
  if (c.open_domain == 0) cudaLaunchKernelEx(&cfg, k_bicgstab_mixed<true>, a);
  else cudaLaunchKernelEx(&cfg, k_bicgstab_mixed<false>, a);
  x.launches++;
}

}  // namespace vebi

// ---- failure-detection check of the bounded grid barrier ---------------------------------
// Block 0 never arrives at the barrier, so every other block polls until `limit`, records
// VEBI_ERR_TIMEOUT in the status word and returns: the wait ends by its own limit and the host
// reads the status, with the context still usable.  The solvers use the same barrier with the
// long SPIN_LIMIT.
namespace vebi {
__global__ void k_barrier_timeout_check(Scal* s, unsigned long long limit) {
  if (blockIdx.x == 0) return;
  grid_sync_bounded(s, limit);
}
}  // namespace vebi

extern "C" void vebi_set_last_error_internal(const char* msg);

extern "C" int vebi_test_barrier_timeout(int32_t blocks, int64_t spin_limit, int32_t* status_out, double* ms_out) {
  using namespace vebi;
  if (blocks < 2 || blocks > 64 || spin_limit < 1 || spin_limit > (1ll << 22) || !status_out) {
    vebi_set_last_error_internal("vebi_test_barrier_timeout: blocks in 2..64, spin_limit in 1..2^22, status_out");
    return VEBI_ERR_ARG;
  }
  Scal* s = nullptr;
  cudaError_t e = cudaMalloc(&s, sizeof(Scal));
  if (e != cudaSuccess) { vebi_set_last_error_internal(cudaGetErrorString(e)); return VEBI_ERR_CUDA; }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  e = cudaMemset(s, 0, sizeof(Scal));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(32);
  cfg.stream = 0;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (e == cudaSuccess) e = cudaEventRecord(e0, 0);
  if (e == cudaSuccess) e = cudaLaunchKernelEx(&cfg, k_barrier_timeout_check, s, (unsigned long long)spin_limit);
  if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
  int status = -1;
  if (e == cudaSuccess) e = cudaMemcpy(&status, &s->error, sizeof(int), cudaMemcpyDeviceToHost);
  float ms = 0.f;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(s);
  if (e != cudaSuccess) { vebi_set_last_error_internal(cudaGetErrorString(e)); return VEBI_ERR_CUDA; }
  *status_out = status;
  if (ms_out) *ms_out = ms;
  return VEBI_OK;
}

// Check of the integer-pipe conversions (vebi_common.cuh: widen, narrow) against the hardware
// conversions: every thread draws one 64-bit and one 32-bit pattern from a SplitMix64 stream
// and, in turn, covers random patterns of every class, doubles whose exponent lies around the
// binary32 range (including exact halfway cases and the largest binary32 values), and exact
// zeros; results are compared bit for bit (NaN against NaN).
namespace vebi {
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__global__ void k_conversion_check(long long n, unsigned long long seed, unsigned int* bad) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    unsigned long long b = splitmix64(seed ^ (unsigned long long)t * 0x632be59bd9b4e019ull);
    const unsigned long long r2 = splitmix64(b);
    switch (t & 7) {
      case 0: case 1: break;  // any 64-bit pattern
      case 2: case 3: {       // exponent 880..1167 around the binary32 range
        const unsigned long long e = 880 + (r2 % 288);
        b = (b & 0x800fffffffffffffull) | (e << 52);
        break;
      }
      case 4: {  // exact halfway between two binary32 values (low 29 bits 0x10000000)
        const unsigned long long e = 890 + (r2 % 270);
        b = (b & 0x800fffffe0000000ull) | (e << 52) | 0x10000000ull;
        break;
      }
      case 5: {  // at and next to the largest binary32 magnitudes, and the smallest normals
        const unsigned long long e = (r2 & 1) ? 1150 : 897;
        b = (b & 0x8000000000000000ull) | (e << 52) | (0x000fffffe0000000ull + (r2 >> 1) % 0x40000000ull);
        break;
      }
      case 6: b &= 0x8000000000000000ull; break;  // signed zeros
      default: b = (b & 0x800fffffffffffffull) | ((unsigned long long)(r2 % 2048) << 52); break;
    }
    const double d = __longlong_as_double((long long)b);
    const float fh = (float)d, fs = narrow(d);
    const bool okn = (fh != fh) ? (fs != fs) : __float_as_uint(fh) == __float_as_uint(fs);
    const float f = __uint_as_float((unsigned)r2 ^ (unsigned)(b >> 32));
    const double dh = (double)f, ds = widen(f);
    const bool okw = (dh != dh) ? (ds != ds) : __double_as_longlong(dh) == __double_as_longlong(ds);
    if (!okn) atomicAdd(bad, 1u);
    if (!okw) atomicAdd(bad + 1, 1u);
  }
}
}  // namespace vebi

extern "C" int vebi_test_conversions(int64_t n, uint64_t seed, int64_t* bad_narrow, int64_t* bad_widen) {
  using namespace vebi;
  if (n < 1 || n > (1ll << 32) || !bad_narrow || !bad_widen) {
    vebi_set_last_error_internal("vebi_test_conversions: n in 1..2^32, bad_narrow, bad_widen");
    return VEBI_ERR_ARG;
  }
  unsigned int* bad = nullptr;
  cudaError_t e = cudaMalloc(&bad, 2 * sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemset(bad, 0, 2 * sizeof(unsigned int));
  if (e == cudaSuccess) {
    k_conversion_check<<<1024, 256>>>((long long)n, (unsigned long long)seed, bad);
    e = cudaGetLastError();
  }
  unsigned int h[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, bad, sizeof(h), cudaMemcpyDeviceToHost);
  if (bad) cudaFree(bad);
  if (e != cudaSuccess) { vebi_set_last_error_internal(cudaGetErrorString(e)); return VEBI_ERR_CUDA; }
  *bad_narrow = h[0];
  *bad_widen = h[1];
  return VEBI_OK;
}
