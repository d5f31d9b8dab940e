// vebi_api.cu -- the C-ABI of include/vebi.h: context set-up, state transfer, the step
// orchestration (div_free, div_free.F90:22-124) and the inspection entry points.
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "vebi_ctx.cuh"

namespace vebi {

int ppe_solver_blocks(int device, int nsm);
int ppe_mixed_blocks(int nsm);
int ppe_mg_blocks(int nsm, bool mixed);
std::vector<int> mg_level_dims(int gx, int gy);
void dump_free(Ctx& x);
int dump_async(Ctx& x);
int dump_write(Ctx& x, const vebi_dump_info* info, const char* part, const char* restart);
int dump_wait(Ctx& x);

static thread_local std::string g_err;

static double bits_to_double_host(unsigned long long b) {
  double v;
  std::memcpy(&v, &b, sizeof(v));
  return v;
}

static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

void vebi_set_error_text(const std::string& msg) { g_err = msg; }

#define CUDA_TRY(expr)                                                              \
  do {                                                                              \
    cudaError_t e_ = (expr);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return fail(VEBI_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// host copy of the quintic spline (sphtools.F90:46-76) for the shifting constant Wab(dx/h)
static double host_wab(double ad_7, double qq) {
  auto p5 = [](double x) { double x2 = x * x; double x3 = x * x2; return x2 * x3; };
  int isel = (int)std::floor(qq);
  if (isel == 0) return ad_7 * (p5(3.0 - qq) - 6.0 * p5(2.0 - qq) + 15.0 * p5(1.0 - qq));
  if (isel == 1) return ad_7 * (p5(3.0 - qq) - 6.0 * p5(2.0 - qq));
  if (isel == 2) return ad_7 * p5(3.0 - qq);
  return 0.0;
}

template <class T>
static int dalloc(Ctx& x, T** p, size_t n) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) return fail(VEBI_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  x.allocs.push_back((void*)*p);
  cudaMemset(*p, 0, n * sizeof(T));
  return VEBI_OK;
}

// check_boundaries (input.F90:182-273) and the run constants (input.F90:164-172)
static int build_consts(Ctx& x) {
  const vebi_params& P = x.prm;
  Consts& c = x.c;
  std::memset(&c, 0, sizeof(c));
  if (P.npfb <= 0 || P.nbS < 0 || P.nbS > P.npfb) return fail(VEBI_ERR_ARG, "npfb/nbS out of range");
  if (P.nb_patches < 0 || P.nb_patches > VEBI_MAX_PATCHES) return fail(VEBI_ERR_ARG, "nb_patches out of range");
  if (P.nb_circles < 0 || P.nb_circles > VEBI_MAX_CIRCLES) return fail(VEBI_ERR_ARG, "nb_circles out of range");
  if (!(P.h > 0.0) || !(P.dv > 0.0)) return fail(VEBI_ERR_ARG, "h and dv must be positive");
  const int nb = P.nb_patches;
  c.nb = nb;
  c.ncirc = P.nb_circles;
  c.h = P.h;
  c.dx = P.dx;
  c.dv = P.dv;
  c.sup_size = 3.0 * c.h;
  c.sup_size_2 = 9.0 * (c.h * c.h);
  c.uno_sup_size = 1.0 / (3.0 * c.h);
  c.ad_7 = 7.0 / 478.0 / PI / c.h / c.h;
  c.ad_7h = c.ad_7 / c.h;
  c.eta2 = c.h * c.h * 1.0e-10;
  c.eta_small = (double)0.01f * c.h * c.h;  // default-real literal (kernel_calculation.F90:36)
  c.oneoverh = 1.0 / c.h;
  c.Ra = P.Ra;
  c.Pr = P.Pr;
  c.El = P.El;
  c.beta = P.beta;
  c.eps_ptt = P.ve_nonlinearity;
  c.Wi = P.El * std::sqrt(P.Ra / P.Pr);
  c.bf[0] = P.body_force[0];
  c.bf[1] = P.body_force[1];
  c.dt_coef_cfl = P.dt_coef_cfl;
  c.dt_coef_visc = P.dt_coef_visc;
  c.dt_visc = P.dt_coef_visc * c.h * c.h * std::fmin(std::sqrt(P.Ra / P.Pr), std::sqrt(P.Ra * P.Pr));
  c.coeff_solvent = P.beta * std::sqrt(P.Pr / P.Ra);
  c.coeff_polymeric = (1.0 - P.beta) * P.Pr / (P.Ra * P.El);
  c.coeff_theta = 1.0 / std::sqrt(P.Ra * P.Pr);
  c.wab1 = host_wab(c.ad_7, c.dx / c.h);
  c.cell_size = 1.0 / c.uno_sup_size;
  c.tol = P.tol > 0 ? P.tol : 1.0e-8;
  c.itermax = P.itermax > 0 ? P.itermax : 1000;
  c.nplink = P.nplink > 0 ? P.nplink : 75;
  if (c.nplink > 96) return fail(VEBI_ERR_ARG, "nplink above 96 is not supported");
  c.open_domain = P.i_open_domain;
  c.shift_coeff = P.i_shift_coeff;
  c.const_mod = P.const_mod == 1 ? 1 : 2;
  c.correct_velocity = P.correct_velocity ? 1 : 0;
  c.warm_start = P.ppe_warm_start ? 1 : 0;
  c.precond = P.ppe_precond == VEBI_PRECOND_MULTIGRID ? 1 : 0;
  c.npfb = P.npfb;
  c.nbS = P.nbS;
  for (int i = 0; i < nb; ++i) {
    for (int q = 0; q < 2; ++q) { c.b_node[i][q] = P.b_node[i][q]; c.b_edge[i][q] = P.b_edge[i][q]; }
    c.b_vel[i] = P.b_vel[i];
    c.b_thermal[i] = P.b_thermal[i];
    c.b_type[i] = P.b_type[i];
    c.b_pp[i] = P.b_periodic_parent[i] - 1;
    c.b_elen[i] = std::sqrt(P.b_edge[i][0] * P.b_edge[i][0] + P.b_edge[i][1] * P.b_edge[i][1]);
  }
  for (int i = 0; i < c.ncirc; ++i) {
    c.c_centre[i][0] = P.c_centre[i][0];
    c.c_centre[i][1] = P.c_centre[i][1];
    c.c_radius[i] = P.c_radius[i];
    c.c_omega[i] = P.c_omega[i];
    c.c_vel[i][0] = P.c_vel[i][0];
    c.c_vel[i][1] = P.c_vel[i][1];
    c.c_thermal[i] = P.c_thermal[i];
  }
  // checks 1-3 of check_boundaries
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
  if (n_fail) return fail(VEBI_ERR_BOUNDARY, "check_boundaries failed");
  // check 4: corner angles; rotation matrices of periodic pairs (angle_between_patches)
  for (int i = 0; i < nb; ++i) {
    int ibm1 = (i + nb - 1) % nb, ibp1 = (i + 1) % nb;
    double p_dist = P.b_edge[ibm1][1] * P.b_node[ibp1][0] - P.b_edge[ibm1][0] * P.b_node[ibp1][1] +
                    P.b_node[i][0] * P.b_node[ibm1][1] - P.b_node[i][1] * P.b_node[ibm1][0];
    p_dist = -1.0 * p_dist / std::sqrt(P.b_edge[ibm1][0] * P.b_edge[ibm1][0] + P.b_edge[ibm1][1] * P.b_edge[ibm1][1]);
    double tmp1 = std::sqrt(P.b_edge[i][0] * P.b_edge[i][0] + P.b_edge[i][1] * P.b_edge[i][1]);
    if (p_dist <= 0.0 && std::fabs(p_dist) > std::fabs(tmp1)) p_dist = -tmp1;
    else if (p_dist > 0.0 && std::fabs(p_dist) > std::fabs(tmp1)) p_dist = tmp1;
    c.b_corner_angle[i] = std::asin(p_dist / tmp1);
    if (P.b_type[i] == 2) {
      int b = P.b_periodic_parent[i] - 1;
      double ta = P.b_edge[i][0] * P.b_edge[b][0] + P.b_edge[i][1] * P.b_edge[b][1];
      double na = P.b_edge[i][0] * P.b_edge[i][0] + P.b_edge[i][1] * P.b_edge[i][1];
      double nbb = P.b_edge[b][0] * P.b_edge[b][0] + P.b_edge[b][1] * P.b_edge[b][1];
      double t = ta / std::sqrt(na * nbb);
      t = std::acos(t) - PI;
      c.b_rot[i][0] = std::cos(t);
      c.b_rot[i][1] = -std::sin(t);
      c.b_rot[i][2] = std::sin(t);
      c.b_rot[i][3] = std::cos(t);
    }
  }
  // padded box (sph2D_incom.F90:64-67) and cell grid (cell_griddin.F90:13-24)
  double xmn = P.x_mint, xmx = P.x_maxt, ymn = P.y_mint, ymx = P.y_maxt;
  if (xmn == 0.0 && xmx == 0.0 && ymn == 0.0 && ymx == 0.0) {
    double xb_min = 1e300, xb_max = -1e300, yb_min = 1e300, yb_max = -1e300;
    for (int i = 0; i < nb; ++i) {
      xb_min = std::fmin(xb_min, P.b_node[i][0]); xb_max = std::fmax(xb_max, P.b_node[i][0]);
      yb_min = std::fmin(yb_min, P.b_node[i][1]); yb_max = std::fmax(yb_max, P.b_node[i][1]);
    }
    xmn = xb_min - c.sup_size * 1.5; xmx = xb_max + c.sup_size * 1.5;
    ymn = yb_min - c.sup_size * 1.5; ymx = yb_max + c.sup_size * 1.5;
  }
  c.x_mint = xmn; c.x_maxt = xmx; c.y_mint = ymn; c.y_maxt = ymx;
  double fx = (xmx - xmn) * c.uno_sup_size, fy = (ymx - ymn) * c.uno_sup_size;
  if (!(fx >= 0.0 && fy >= 0.0 && fx < 1.0e8 && fy < 1.0e8)) return fail(VEBI_ERR_ARG, "bad domain box");
  c.ncx = (int)fx + 1;
  c.ncy = (int)fy + 1;
  long long nct = (long long)c.ncx * c.ncy;
  if (nct > 400000000LL) return fail(VEBI_ERR_ARG, "cell grid too large");
  c.nct = (int)nct;
  // mirror capacity: create_mirror_particles' estimate (mirror_boundaries_mod.F90:53-54)
  c.mcap = P.nmirror_cap > 0 ? P.nmirror_cap : (P.npfb <= 500 ? 10 * P.npfb : 2 * P.npfb);
  for (int i = 0; i < nb; ++i) {  // FP32 line table of the prefilters (bound_dist's expression)
    const int ip1 = (i + 1) % nb;
    const double inv = -1.0 / c.b_elen[i];
    c.bl_a[i] = (float)(c.b_edge[i][1] * inv);
    c.bl_b[i] = (float)(-c.b_edge[i][0] * inv);
    c.bl_c[i] = (float)((c.b_node[ip1][0] * c.b_node[i][1] - c.b_node[ip1][1] * c.b_node[i][0]) * inv);
  }
  {
    const double ext = std::fmax(std::fmax(std::fabs(c.x_mint), std::fabs(c.x_maxt)),
                                 std::fmax(std::fabs(c.y_mint), std::fabs(c.y_maxt)));
    c.near_band = (float)(c.sup_size + 0.1 * c.dx + 4.0e-6 * ext);
  }
  c.cap = c.npfb + c.mcap;
  return VEBI_OK;
}

static int allocate_all(Ctx& x) {
  Consts& c = x.c;
  Dev& d = x.d;
  const size_t cap = (size_t)c.cap, n = (size_t)c.npfb, E = (size_t)c.nplink * n;
  int st = 0;
#define A_(p, cnt) if ((st = dalloc(x, &(p), (cnt)))) return st
  A_(d.s, 1);
  A_(d.rx, cap); A_(d.ry, cap); A_(d.ux, cap); A_(d.uy, cap); A_(d.th, cap);
  A_(d.rx2, cap); A_(d.ry2, cap); A_(d.ux2, cap); A_(d.uy2, cap); A_(d.th2, cap);
  A_(d.r0x, n); A_(d.r0y, n); A_(d.u0x, n); A_(d.u0y, n);
  A_(d.p, cap);
  for (int q = 0; q < 4; ++q) A_(d.tau[q], cap);
  A_(d.trace_conf, n); A_(d.a_out, n); A_(d.vort, n);
  A_(d.n_surf, cap); A_(d.inbin, cap);
  A_(d.irel, cap); A_(d.vrel, cap); A_(d.dP_mp, cap);
  A_(d.cellpart, cap); A_(d.cell_fill, cap); A_(d.ip, cap);
  A_(d.cell_cnt, (size_t)c.nct); A_(d.cell_start, (size_t)c.nct + 1);
  A_(d.scan_part, (size_t)c.nct / 1024 + 2);
  size_t sel_items = (size_t)(c.npfb > c.mcap ? c.npfb : c.mcap);
  A_(d.sel_blk, sel_items / SEL_CH + 2);
  A_(d.cand, n); A_(d.cand_blk, n / SEL_CH + 2);
  A_(d.pk, cap); A_(d.pko, cap);
  A_(d.ij_count, n); A_(d.ij_link, E);
  A_(d.wGx, E); A_(d.wGy, E); A_(d.wL, E);
  for (int q = 0; q < 4; ++q) A_(d.kgcm[q], n);
  for (int q = 0; q < 6; ++q) A_(d.grad[q], cap);
  A_(d.gradCx, n); A_(d.gradCy, n); A_(d.ushx, n); A_(d.ushy, n);
  if (c.open_domain == 1) {
    A_(d.conc, n); A_(d.div_r, n); A_(d.surf_nx, n); A_(d.surf_ny, n); A_(d.ppe_smooth, n);
    A_(d.beta_div_r, n);
  }
  A_(d.ppe_B, n); A_(d.ppe_diag, n); A_(d.ppe_val, E); A_(d.ppe_col, E);
  A_(d.bx, n); A_(d.br, n); A_(d.brb, n); A_(d.bv, n); A_(d.bp, n); A_(d.bpi, n);
  A_(d.bs, n); A_(d.bsi, n); A_(d.bt, n); A_(d.bM, n);
  size_t np_part = (size_t)grid_for(c.npfb);
  // block partials of the persistent solvers: 12 slots of one value per block
  int part_blocks = x.coop_blocks;
  if (x.coop_blocks_mixed > part_blocks) part_blocks = x.coop_blocks_mixed;
  if (x.mg_blocks > part_blocks) part_blocks = x.mg_blocks;
  if (x.mg_blocks_mixed > part_blocks) part_blocks = x.mg_blocks_mixed;
  size_t coop_part = (size_t)part_blocks * 12;
  A_(d.partials, (2 * np_part > coop_part ? 2 * np_part : coop_part) + 64);
  A_(d.gpx, n); A_(d.gpy, n);
  if (x.precision == VEBI_PREC_MIXED) {
    A_(d.ppe_val32, E); A_(d.rowsum, n); A_(d.pi2, n); A_(d.si2, n);
    A_(d.hl_u[0], cap); A_(d.hl_u[1], cap); A_(d.hl_th, cap); A_(d.hl_us[0], cap); A_(d.hl_us[1], cap);
    A_(d.hl_p, cap);
    for (int q = 0; q < 4; ++q) A_(d.hl_tau[q], cap);
    A_(d.wGx32, E); A_(d.wGy32, E); A_(d.wL32, E);
    for (int q = 0; q < 4; ++q) A_(d.kgcm32[q], n);
  }
  if (c.precond) {  // multigrid levels on the cell grid
    std::vector<int> dims = mg_level_dims(c.ncx, c.ncy);
    for (size_t l = 0; l + 1 < dims.size(); l += 2) {
      MgLevel L{};
      L.gx = dims[l];
      L.gy = dims[l + 1];
      L.n = L.gx * L.gy;
      const size_t ln = (size_t)L.n;
      A_(L.cnt, ln); A_(L.col, ln * MG_SLOTS); A_(L.val, ln * MG_SLOTS);
      A_(L.diag, ln); A_(L.dinv, ln); A_(L.x, ln); A_(L.b, ln); A_(L.r, ln);
      x.mg.push_back(L);
    }
    A_(x.d_mg, x.mg.size());
    cudaMemcpy(x.d_mg, x.mg.data(), sizeof(MgLevel) * x.mg.size(), cudaMemcpyHostToDevice);
    A_(x.mg_z, n); A_(x.mg_fr, n); A_(x.mg_dinv0, n); A_(x.mg_rsum, n); A_(x.mg_w, n);
    A_(x.mg_ragg, n * MG_ROW_SLOTS); A_(x.mg_rval, n * MG_ROW_SLOTS); A_(x.mg_rcnt, n);
    A_(x.mg_rv9, n * 8); A_(x.mg_rx, n); A_(x.mg_g32, (size_t)x.mg[0].n); A_(x.mg_q32, n);
    A_(x.mg_kinv, (size_t)MG_COARSEST * MG_COARSEST); A_(x.mg_kinv_ok, 1);
  }
#undef A_
  return VEBI_OK;
}

}  // namespace vebi

using namespace vebi;

struct vebi_ctx {
  Ctx x;
};

namespace vebi {
Ctx* ctx_of(vebi_ctx* h) { return h ? &h->x : nullptr; }
}  // namespace vebi

extern "C" {

const char* vebi_version(void) {
  return "vebisph-gb300 step library for sm_103a: the div_free step in FP64 (the reference's arithmetic) or mixed "
         "precision, persistent BiCGSTAB with an optional multigrid preconditioner, batches, output files";
}

const char* vebi_last_error(void) { return g_err.c_str(); }

// error text of entry points defined in other translation units
void vebi_set_last_error_internal(const char* msg) { g_err = msg ? msg : ""; }

int vebi_create(const vebi_params* params, vebi_ctx** out) {
  if (!params || !out) return fail(VEBI_ERR_ARG, "null argument");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(VEBI_ERR_NO_DEVICE, "no CUDA device");
  auto* h = new vebi_ctx();
  Ctx& x = h->x;
  x.prm = *params;
  x.precision = params->precision;
  int st = build_consts(x);
  if (st) { delete h; return st; }
  cudaGetDevice(&x.device);
  cudaDeviceGetAttribute(&x.nsm, cudaDevAttrMultiProcessorCount, x.device);
  x.coop_blocks = ppe_solver_blocks(x.device, x.nsm);
  x.coop_blocks_mixed = ppe_mixed_blocks(x.nsm);
  x.gs_blocks = x.nsm * 8;
  x.mg_blocks = ppe_mg_blocks(x.nsm, false);
  x.mg_blocks_mixed = ppe_mg_blocks(x.nsm, true);
  if (cudaStreamCreateWithFlags(&x.st, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return fail(VEBI_ERR_CUDA, "cudaStreamCreate failed");
  }
  for (int i = 0; i <= VEBI_NSTAGES; ++i) cudaEventCreate(&x.ev[i]);
  st = allocate_all(x);
  if (st) { vebi_destroy(h); return st; }
  // trace of the conformation tensor starts at 2 (input.F90:111)
  std::vector<double> two((size_t)x.c.npfb, 2.0);
  cudaMemcpy(x.d.trace_conf, two.data(), two.size() * sizeof(double), cudaMemcpyHostToDevice);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { vebi_destroy(h); return fail(VEBI_ERR_CUDA, cudaGetErrorString(e)); }
  *out = h;
  return VEBI_OK;
}

int vebi_upload_state(vebi_ctx* h, const double* r, const double* u, const double* tau_p, const double* theta,
                      const double* trace_conf, const uint8_t* inbin, int32_t ld) {
  if (!h || !r || !u) return fail(VEBI_ERR_ARG, "null argument");
  Ctx& x = h->x;
  const int n = x.c.npfb;
  if (ld < n) return fail(VEBI_ERR_ARG, "ld < npfb");
  const size_t B = sizeof(double) * (size_t)n;
  Dev& d = x.d;
  CUDA_TRY(cudaMemcpyAsync(d.rx, r, B, cudaMemcpyHostToDevice, x.st));
  CUDA_TRY(cudaMemcpyAsync(d.ry, r + ld, B, cudaMemcpyHostToDevice, x.st));
  CUDA_TRY(cudaMemcpyAsync(d.ux, u, B, cudaMemcpyHostToDevice, x.st));
  CUDA_TRY(cudaMemcpyAsync(d.uy, u + ld, B, cudaMemcpyHostToDevice, x.st));
  if (theta) CUDA_TRY(cudaMemcpyAsync(d.th, theta, B, cudaMemcpyHostToDevice, x.st));
  else CUDA_TRY(cudaMemsetAsync(d.th, 0, B, x.st));
  for (int q = 0; q < 4; ++q) {
    if (tau_p) CUDA_TRY(cudaMemcpyAsync(d.tau[q], tau_p + (size_t)q * ld, B, cudaMemcpyHostToDevice, x.st));
    else CUDA_TRY(cudaMemsetAsync(d.tau[q], 0, B, x.st));
  }
  if (trace_conf) CUDA_TRY(cudaMemcpyAsync(d.trace_conf, trace_conf, B, cudaMemcpyHostToDevice, x.st));
  if (inbin) CUDA_TRY(cudaMemcpyAsync(d.inbin, inbin, (size_t)n, cudaMemcpyHostToDevice, x.st));
  else CUDA_TRY(cudaMemsetAsync(d.inbin, 0, (size_t)n, x.st));
  // a new state starts with no recorded failure
  CUDA_TRY(cudaMemsetAsync(&d.s->first_error, 0, sizeof(int), x.st));
  CUDA_TRY(cudaMemsetAsync(&d.s->error, 0, sizeof(int), x.st));
  CUDA_TRY(cudaMemsetAsync(&d.s->n_inbin, 0, sizeof(int), x.st));
  x.have_state = true;
  return VEBI_OK;
}

static int finish_step(Ctx& x, vebi_step_stats* stats, bool sync) {
  Scal s;
  CUDA_TRY(cudaMemcpyAsync(&s, x.d.s, sizeof(Scal), cudaMemcpyDeviceToHost, x.st));
  if (sync) CUDA_TRY(cudaStreamSynchronize(x.st));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(VEBI_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  vebi_step_stats o;
  std::memset(&o, 0, sizeof(o));
  o.dt = s.dt;
  o.LS_residual = s.ls_residual;
  o.umax = bits_to_double_host(s.umax_bits);
  o.max_abs_u = bits_to_double_host(s.absu_bits);
  o.max_abs_v = bits_to_double_host(s.absv_bits);
  o.max_abs_p = bits_to_double_host(s.absp_bits);
  o.rms_u = s.rms_u;
  o.circle_force[0] = s.circle_fx;
  o.circle_force[1] = s.circle_fy;
  o.ppe_rhs_mean = s.rhs_mean;
  o.LS_iters = s.ls_iters;
  o.n_inbin = s.n_inbin;
  o.np = s.np;
  o.npfb = x.c.npfb;
  o.nmirror = s.nmirror;
  o.maxneighbours = s.maxneigh;
  o.n_escapees = s.n_escapees;
  o.error = s.error ? s.error : s.first_error;
  o.warnings = s.warnings | (s.n_escapees ? VEBI_WARN_ESCAPEES : 0);
  o.gpu_launches = x.launches;
  o.refine_iters = s.refine_iters;
  o.LS_iters_total = s.ls_iters_total;
  o.n_near_pole = s.n_near_pole;
  o.n_near_pole_total = s.n_near_pole_total;
  o.nsteps = 1;
  if (x.timing && sync) {
    int prev = -1;
    for (int q = 0; q <= VEBI_NSTAGES; ++q) {
      bool used = q == VEBI_NSTAGES || x.ev_used[q];
      if (!used) continue;
      if (prev >= 0) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, x.ev[prev], x.ev[q]);
        o.stage_ms[prev] = ms;
      }
      prev = q;
    }
  }
  x.last = o;
  if (stats) *stats = o;
  if (s.error) return fail(s.error, "device-side error in the step");
  if (s.first_error) return fail(s.first_error, "an earlier step of this state failed");
  if (s.n_inbin == x.c.npfb - x.c.nbS && x.c.npfb > x.c.nbS) return fail(VEBI_ERR_ALL_IN_BIN, "all liquid particles are in the bin");
  return VEBI_OK;
}

static void enqueue_step(Ctx& x, int secondary) {
  for (int q = 0; q < VEBI_NSTAGES; ++q) x.ev_used[q] = false;
  stage_mark(x, 0);
  launch_advect_bin(x);
  if (x.rec_geo || x.rep_geo) {
    const size_t B = sizeof(double) * (size_t)x.c.npfb;
    const size_t n = (size_t)x.c.npfb;
    if (x.rep_geo) {
      cudaMemcpyAsync(x.d.rx, x.rep_geo, B, cudaMemcpyDeviceToDevice, x.st);
      cudaMemcpyAsync(x.d.ry, x.rep_geo + n, B, cudaMemcpyDeviceToDevice, x.st);
      cudaMemcpyAsync(&x.d.s->dt, x.rep_geo + 2 * n, sizeof(double), cudaMemcpyDeviceToDevice, x.st);
    }
    if (x.rec_geo) {
      cudaMemcpyAsync(x.rec_geo, x.d.rx, B, cudaMemcpyDeviceToDevice, x.st);
      cudaMemcpyAsync(x.rec_geo + n, x.d.ry, B, cudaMemcpyDeviceToDevice, x.st);
      cudaMemcpyAsync(x.rec_geo + 2 * n, &x.d.s->dt, sizeof(double), cudaMemcpyDeviceToDevice, x.st);
    }
  }
  stage_mark(x, 1);
  launch_mirrors(x);
  stage_mark(x, 2);
  launch_cells_neighbours(x);
  stage_mark(x, 4);
  launch_weights_surface_shift(x);
  launch_predictor(x);
  launch_ppe(x);
  launch_final(x, secondary);
}

// Capture one step (without the dump-time diagnostic) into a CUDA graph, once per context and
// timing mode; later steps replay it with one launch.  Every kernel argument of a step is the
// same from step to step (counts live in device memory), so one capture serves all steps.
// If capture is not possible the step is launched kernel by kernel instead.
static bool graph_ready(Ctx& x) {
  const int m = x.timing ? 1 : 0;
  if (x.graph[m]) return true;
  if (x.graph_failed[m]) return false;
  cudaGraph_t g = nullptr;
  x.launches = 0;
  for (int q = 0; q < VEBI_NSTAGES; ++q) x.ev_used[q] = false;
  if (cudaStreamBeginCapture(x.st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    x.graph_failed[m] = true;
    return false;
  }
  x.capturing = true;
  enqueue_step(x, 0);
  if (x.timing) cudaEventRecordWithFlags(x.ev[VEBI_NSTAGES], x.st, cudaEventRecordExternal);
  x.capturing = false;
  cudaError_t e = cudaStreamEndCapture(x.st, &g);
  cudaGraphExec_t ge = nullptr;
  if (e == cudaSuccess && g) e = cudaGraphInstantiate(&ge, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess || !ge) {
    cudaGetLastError();
    x.graph_failed[m] = true;
    return false;
  }
  x.graph[m] = ge;
  x.graph_launches[m] = x.launches;
  for (int q = 0; q < VEBI_NSTAGES; ++q) x.graph_used[m][q] = x.ev_used[q];
  return true;
}

// enqueue one step: the captured graph when possible, else kernel by kernel
static void launch_step(Ctx& x, int secondary) {
  if (!secondary && graph_ready(x)) {
    const int m = x.timing ? 1 : 0;
    cudaGraphLaunch(x.graph[m], x.st);
    x.launches += x.graph_launches[m];
    for (int q = 0; q < VEBI_NSTAGES; ++q) x.ev_used[q] = x.graph_used[m][q];
    return;
  }
  enqueue_step(x, secondary);
  if (x.timing && !x.capturing) cudaEventRecord(x.ev[VEBI_NSTAGES], x.st);
}

int vebi_step(vebi_ctx* h, double x_mint, double y_mint, double x_maxt, double y_maxt, int32_t secondary,
              vebi_step_stats* stats) {
  if (!h) return fail(VEBI_ERR_ARG, "null context");
  Ctx& x = h->x;
  if (!x.have_state) return fail(VEBI_ERR_ARG, "no state uploaded");
  if (x_mint != x.c.x_mint || x_maxt != x.c.x_maxt || y_mint != x.c.y_mint || y_maxt != x.c.y_maxt)
    return fail(VEBI_ERR_ARG, "domain box differs from the one the context was created with");
  x.launches = 0;
  launch_step(x, secondary);
  return finish_step(x, stats, true);
}

int vebi_run_steps(vebi_ctx* h, double x_mint, double y_mint, double x_maxt, double y_maxt, int32_t nsteps,
                   double* ms, vebi_step_stats* last) {
  if (!h || nsteps < 0) return fail(VEBI_ERR_ARG, "bad argument");
  Ctx& x = h->x;
  if (!x.have_state) return fail(VEBI_ERR_ARG, "no state uploaded");
  if (x_mint != x.c.x_mint || x_maxt != x.c.x_maxt || y_mint != x.c.y_mint || y_maxt != x.c.y_maxt)
    return fail(VEBI_ERR_ARG, "domain box differs from the one the context was created with");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double acc[VEBI_NSTAGES] = {};
  x.launches = 0;
  cudaMemsetAsync(&x.d.s->ls_iters_total, 0, sizeof(int), x.st);
  cudaMemsetAsync(&x.d.s->n_near_pole_total, 0, sizeof(int), x.st);
  cudaEventRecord(e0, x.st);
  for (int s = 0; s < nsteps; ++s) {
    launch_step(x, 0);
    if (x.timing) {
      // read this step's stage events before the next step records them again
      cudaEventSynchronize(x.ev[VEBI_NSTAGES]);
      int prev = -1;
      for (int q = 0; q <= VEBI_NSTAGES; ++q) {
        bool u = q == VEBI_NSTAGES || x.ev_used[q];
        if (!u) continue;
        if (prev >= 0) {
          float m = 0.f;
          cudaEventElapsedTime(&m, x.ev[prev], x.ev[q]);
          acc[prev] += m;
        }
        prev = q;
      }
    }
  }
  cudaEventRecord(e1, x.st);
  bool timing = x.timing;
  x.timing = false;  // the stage sums are already collected
  int st = finish_step(x, last, true);
  x.timing = timing;
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  if (ms) *ms = t;
  if (last) {
    last->nsteps = nsteps;
    for (int q = 0; q < VEBI_NSTAGES; ++q) last->stage_ms[q] = timing ? acc[q] : 0.0;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return st;
}

// Wait for a stream by polling, for up to a second, before falling back to a blocking
// synchronize: the copies of a download take ~2 ms, and a blocking wait can return tens of ms
// late (measured on the Grace host) when the waiting thread is not woken promptly.
static cudaError_t wait_stream_polling(cudaStream_t st) {
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    const cudaError_t e = cudaStreamQuery(st);
    if (e != cudaErrorNotReady) return e;
    if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(1)) return cudaStreamSynchronize(st);
  }
}

int vebi_download_state(vebi_ctx* h, double* r, double* u, double* tau_p, double* theta, double* p, double* vort,
                        double* a_out, double* trace_conf, int32_t* n_surf, uint8_t* inbin, int32_t ld) {
  if (!h) return fail(VEBI_ERR_ARG, "null context");
  Ctx& x = h->x;
  const int n = x.c.npfb;
  if (ld < n) return fail(VEBI_ERR_ARG, "ld < npfb");
  const size_t B = sizeof(double) * (size_t)n;
  Dev& d = x.d;
  if (r) {
    CUDA_TRY(cudaMemcpyAsync(r, d.rx, B, cudaMemcpyDeviceToHost, x.st));
    CUDA_TRY(cudaMemcpyAsync(r + ld, d.ry, B, cudaMemcpyDeviceToHost, x.st));
  }
  if (u) {
    CUDA_TRY(cudaMemcpyAsync(u, d.ux, B, cudaMemcpyDeviceToHost, x.st));
    CUDA_TRY(cudaMemcpyAsync(u + ld, d.uy, B, cudaMemcpyDeviceToHost, x.st));
  }
  if (tau_p)
    for (int q = 0; q < 4; ++q) CUDA_TRY(cudaMemcpyAsync(tau_p + (size_t)q * ld, d.tau[q], B, cudaMemcpyDeviceToHost, x.st));
  if (theta) CUDA_TRY(cudaMemcpyAsync(theta, d.th, B, cudaMemcpyDeviceToHost, x.st));
  if (p) CUDA_TRY(cudaMemcpyAsync(p, d.p, B, cudaMemcpyDeviceToHost, x.st));
  if (vort) CUDA_TRY(cudaMemcpyAsync(vort, d.vort, B, cudaMemcpyDeviceToHost, x.st));
  if (a_out) CUDA_TRY(cudaMemcpyAsync(a_out, d.a_out, B, cudaMemcpyDeviceToHost, x.st));
  if (trace_conf) CUDA_TRY(cudaMemcpyAsync(trace_conf, d.trace_conf, B, cudaMemcpyDeviceToHost, x.st));
  if (n_surf) CUDA_TRY(cudaMemcpyAsync(n_surf, d.n_surf, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, x.st));
  if (inbin) CUDA_TRY(cudaMemcpyAsync(inbin, d.inbin, (size_t)n, cudaMemcpyDeviceToHost, x.st));
  CUDA_TRY(wait_stream_polling(x.st));
  return VEBI_OK;
}

int vebi_destroy(vebi_ctx* h) {
  if (!h) return VEBI_OK;
  Ctx& x = h->x;
  if (x.st) cudaStreamSynchronize(x.st);
  dump_free(x);
  for (auto& g : x.graph)
    if (g) cudaGraphExecDestroy(g);
  for (void* p : x.allocs) cudaFree(p);
  x.allocs.clear();
  for (int i = 0; i <= VEBI_NSTAGES; ++i)
    if (x.ev[i]) cudaEventDestroy(x.ev[i]);
  if (x.st) cudaStreamDestroy(x.st);
  delete h;
  return VEBI_OK;
}

int vebi_pin_host(void* ptr, int64_t bytes) {
  if (!ptr || bytes <= 0) return fail(VEBI_ERR_ARG, "bad argument");
  CUDA_TRY(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault));
  return VEBI_OK;
}

int vebi_unpin_host(void* ptr) {
  if (!ptr) return fail(VEBI_ERR_ARG, "null pointer");
  CUDA_TRY(cudaHostUnregister(ptr));
  return VEBI_OK;
}

int vebi_set_solver_grid(vebi_ctx* h, int32_t rows_per_thread) {
  if (!h || rows_per_thread < 1) return fail(VEBI_ERR_ARG, "bad argument");
  Ctx& x = h->x;
  if (x.solver_rows_per_thread == rows_per_thread) return VEBI_OK;
  cudaStreamSynchronize(x.st);
  x.solver_rows_per_thread = rows_per_thread;
  ++x.grid_gen;
  for (int m = 0; m < 2; ++m) {  // the captured steps hold the old grid
    if (x.graph[m]) cudaGraphExecDestroy(x.graph[m]);
    x.graph[m] = nullptr;
    x.graph_failed[m] = false;
  }
  return VEBI_OK;
}

int vebi_set_coarse_block_rows(vebi_ctx* h, int32_t rows) {
  if (!h || rows < 0) return fail(VEBI_ERR_ARG, "bad argument");
  Ctx& x = h->x;
  if (x.mg_block_rows == rows) return VEBI_OK;
  cudaStreamSynchronize(x.st);
  x.mg_block_rows = rows;
  ++x.grid_gen;
  for (int m = 0; m < 2; ++m) {  // the captured steps hold the old launch arguments
    if (x.graph[m]) cudaGraphExecDestroy(x.graph[m]);
    x.graph[m] = nullptr;
    x.graph_failed[m] = false;
  }
  return VEBI_OK;
}

int vebi_set_weissenberg(vebi_ctx* h, double wi) {
  if (!h || !(wi > 0.0)) return fail(VEBI_ERR_ARG, "bad argument");
  Ctx& x = h->x;
  cudaStreamSynchronize(x.st);
  vebi_params& P = x.prm;
  P.El = wi / std::sqrt(P.Ra / P.Pr);
  x.c.El = P.El;
  x.c.Wi = P.El * std::sqrt(P.Ra / P.Pr);
  x.c.coeff_polymeric = (1.0 - P.beta) * P.Pr / (P.Ra * P.El);
  ++x.grid_gen;
  for (int m = 0; m < 2; ++m) {  // the captured steps hold the old constants
    if (x.graph[m]) cudaGraphExecDestroy(x.graph[m]);
    x.graph[m] = nullptr;
    x.graph_failed[m] = false;
  }
  return VEBI_OK;
}

int vebi_set_velocity_limit(vebi_ctx* h, double u_limit) {
  if (!h || !(u_limit >= 0.0) || !std::isfinite(u_limit)) return fail(VEBI_ERR_ARG, "bad argument");
  Ctx& x = h->x;
  if (x.c.u_limit == u_limit) return VEBI_OK;
  cudaStreamSynchronize(x.st);
  x.c.u_limit = u_limit;
  ++x.grid_gen;
  for (int m = 0; m < 2; ++m) {  // the captured steps hold the old constants
    if (x.graph[m]) cudaGraphExecDestroy(x.graph[m]);
    x.graph[m] = nullptr;
    x.graph_failed[m] = false;
  }
  return VEBI_OK;
}

int vebi_dump_async(vebi_ctx* h) {
  if (!h) return fail(VEBI_ERR_ARG, "null context");
  if (!h->x.have_state) return fail(VEBI_ERR_ARG, "no state uploaded");
  int st = dump_async(h->x);
  if (st == VEBI_ERR_CUDA) return fail(st, "dump staging failed");
  return st;
}

int vebi_dump_write(vebi_ctx* h, const vebi_dump_info* info, const char* part_path, const char* restart_path) {
  if (!h || !info) return fail(VEBI_ERR_ARG, "null argument");
  return dump_write(h->x, info, part_path, restart_path);
}

int vebi_dump_wait(vebi_ctx* h) {
  if (!h) return fail(VEBI_ERR_ARG, "null context");
  return dump_wait(h->x);
}

int vebi_set_timing(vebi_ctx* h, int32_t on) {
  if (!h) return fail(VEBI_ERR_ARG, "null context");
  h->x.timing = on != 0;
  return VEBI_OK;
}

// ------------------------------------------------------------------ batches
// A batch is a set of independent contexts (one per simulation, each with its own sizes,
// parameters and device arrays).  One batch step is one launch of a CUDA graph whose
// independent branches are the instances' captured steps, so the instances' kernels overlap
// on the GPU with no host work between them; each instance's solver converges on its own.
struct vebi_batch {
  std::vector<vebi_ctx*> ctx;
  cudaGraphExec_t graph = nullptr;
  bool graph_failed = false;
  std::vector<int> launches;  // kernels in each instance's captured step
  std::vector<int> gen;  // grid_gen of each instance when the batch graph was captured
};

static void batch_drop_graph(vebi_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_failed = false;
}

// capture every instance's step into a child graph of one batch graph
static bool batch_graph_ready(vebi_batch* b) {
  const int n = (int)b->ctx.size();
  if (b->graph) {
    bool stale = false;
    for (int i = 0; i < n; ++i) stale |= b->gen[i] != b->ctx[i]->x.grid_gen;
    if (!stale) return true;
    batch_drop_graph(b);
  }
  if (b->graph_failed) return false;
  cudaGraph_t bg = nullptr;
  if (cudaGraphCreate(&bg, 0) != cudaSuccess) {
    cudaGetLastError();
    b->graph_failed = true;
    return false;
  }
  std::vector<int> launches(n, 0);
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < n && e == cudaSuccess; ++i) {
    Ctx& x = b->ctx[i]->x;
    const bool timing = x.timing;
    x.timing = false;
    x.launches = 0;
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(x.st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      x.capturing = true;
      enqueue_step(x, 0);
      x.capturing = false;
      e = cudaStreamEndCapture(x.st, &g);
    }
    x.timing = timing;
    cudaGraphNode_t node;
    if (e == cudaSuccess && g) e = cudaGraphAddChildGraphNode(&node, bg, nullptr, 0, g);
    if (g) cudaGraphDestroy(g);
    launches[i] = x.launches;
  }
  cudaGraphExec_t ge = nullptr;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, bg, 0);
  cudaGraphDestroy(bg);
  if (e != cudaSuccess || !ge) {
    cudaGetLastError();
    b->graph_failed = true;
    return false;
  }
  b->graph = ge;
  b->launches = launches;
  b->gen.resize(n);
  for (int i = 0; i < n; ++i) b->gen[i] = b->ctx[i]->x.grid_gen;
  return true;
}

int vebi_batch_create(const vebi_params* params, int32_t n, vebi_batch** out) {
  if (!params || !out || n < 1) return fail(VEBI_ERR_ARG, "bad argument");
  *out = nullptr;
  auto* b = new vebi_batch();
  for (int i = 0; i < n; ++i) {
    vebi_ctx* c = nullptr;
    int st = vebi_create(params + i, &c);
    if (st) {
      std::string m = g_err;
      vebi_batch_destroy(b);
      return fail(st, "batch instance " + std::to_string(i) + ": " + m);
    }
    b->ctx.push_back(c);
  }
  *out = b;
  return VEBI_OK;
}

int vebi_batch_get(vebi_batch* b, int32_t i, vebi_ctx** ctx) {
  if (!b || !ctx || i < 0 || i >= (int)b->ctx.size()) return fail(VEBI_ERR_ARG, "bad argument");
  *ctx = b->ctx[i];
  return VEBI_OK;
}

int vebi_batch_step(vebi_batch* b, int32_t nsteps, double* ms, vebi_step_stats* stats) {
  if (!b || nsteps < 0) return fail(VEBI_ERR_ARG, "bad argument");
  const int n = (int)b->ctx.size();
  for (int i = 0; i < n; ++i) {
    Ctx& x = b->ctx[i]->x;
    if (!x.have_state) return fail(VEBI_ERR_ARG, "batch instance without state");
  }
  const bool graph = batch_graph_ready(b);
  cudaStream_t s0 = b->ctx[0]->x.st;
  // every instance's pending work (uploads) is ordered before the batch; the whole batch
  // runs on instance 0's stream when it is one graph, else on the instances' own streams
  std::vector<cudaEvent_t> ev(n);
  for (int i = 0; i < n; ++i) cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
  for (int i = 0; i < n; ++i) {
    Ctx& x = b->ctx[i]->x;
    x.launches = 0;
    cudaMemsetAsync(&x.d.s->ls_iters_total, 0, sizeof(int), x.st);
    if (i) {
      cudaEventRecord(ev[i], x.st);
      cudaStreamWaitEvent(s0, ev[i], 0);
    }
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s0);
  if (graph) {
    for (int s = 0; s < nsteps; ++s) cudaGraphLaunch(b->graph, s0);
  } else {
    for (int i = 1; i < n; ++i) cudaStreamWaitEvent(b->ctx[i]->x.st, e0, 0);
    for (int s = 0; s < nsteps; ++s)
      for (int i = 0; i < n; ++i) {
        Ctx& x = b->ctx[i]->x;
        const bool timing = x.timing;
        x.timing = false;
        launch_step(x, 0);
        x.timing = timing;
      }
    for (int i = 1; i < n; ++i) {
      cudaEventRecord(ev[i], b->ctx[i]->x.st);
      cudaStreamWaitEvent(s0, ev[i], 0);
    }
  }
  cudaEventRecord(e1, s0);
  cudaError_t se = cudaStreamSynchronize(s0);
  int st = VEBI_OK;
  if (se != cudaSuccess) st = fail(VEBI_ERR_CUDA, std::string("batch step: ") + cudaGetErrorString(se));
  int n_failed = 0, first_failed = -1;
  for (int i = 0; i < n && st == VEBI_OK; ++i) {
    Ctx& x = b->ctx[i]->x;
    const bool timing = x.timing;
    x.timing = false;
    vebi_step_stats o;
    int si = finish_step(x, &o, true);
    x.timing = timing;
    o.nsteps = nsteps;
    o.gpu_launches = graph ? b->launches[i] * nsteps : x.launches;
    if (si && !o.error) o.error = si;  // a failure seen only on the host (all liquid binned)
    if (stats) stats[i] = o;
    if (si == VEBI_ERR_CUDA) st = si;
    else if (si) {
      ++n_failed;
      if (first_failed < 0) first_failed = i;
    }
  }
  if (st == VEBI_OK && n_failed)
    g_err = std::to_string(n_failed) + " instance(s) failed, first " + std::to_string(first_failed) +
            " (status in stats[i].error)";
  else if (st == VEBI_OK)
    g_err.clear();
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  if (ms) *ms = t;
  for (int i = 0; i < n; ++i) cudaEventDestroy(ev[i]);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return st;
}

int vebi_batch_destroy(vebi_batch* b) {
  if (!b) return VEBI_OK;
  batch_drop_graph(b);
  for (auto* c : b->ctx) vebi_destroy(c);
  delete b;
  return VEBI_OK;
}

// ------------------------------------------------------------------ inspection
struct DView { const void* p; int64_t esz, n; };

static DView dview(Ctx& x, const std::string& nm) {
  Dev& d = x.d;
  const Consts& c = x.c;
  Scal s;
  cudaMemcpy(&s, d.s, sizeof(Scal), cudaMemcpyDeviceToHost);
  const int64_t np = s.np, n = c.npfb, nm_ = s.nmirror;
  const int64_t ell = (int64_t)(s.maxneigh > 0 ? s.maxneigh : 1) * n;
  auto D = [](const double* p, int64_t k) { return DView{p, 8, k}; };
  auto I = [](const int* p, int64_t k) { return DView{p, 4, k}; };
  if (nm == "rx") return D(d.rx, n);
  if (nm == "ry") return D(d.ry, n);
  if (nm == "ux") return D(d.ux, n);
  if (nm == "uy") return D(d.uy, n);
  if (nm == "theta") return D(d.th, n);
  if (nm == "p") return D(d.p, np);
  if (nm == "tau11") return D(d.tau[0], np);
  if (nm == "tau21") return D(d.tau[1], np);
  if (nm == "tau12") return D(d.tau[2], np);
  if (nm == "tau22") return D(d.tau[3], np);
  if (nm == "trace_conf") return D(d.trace_conf, n);
  if (nm == "a_out") return D(d.a_out, n);
  if (nm == "vort") return D(d.vort, n);
  if (nm == "n_surf") return I(d.n_surf, np);
  if (nm == "irelation") return I(d.irel + n, nm_);
  if (nm == "vrelation") return I(d.vrel + n, nm_);
  if (nm == "dP_mp") return D(d.dP_mp + n, nm_);
  if (nm == "rsx") return D(d.rx2, np);
  if (nm == "rsy") return D(d.ry2, np);
  if (nm == "cellpart") return I(d.cellpart, np);
  if (nm == "ist") return I(d.cell_start, (int64_t)c.nct + 1);
  if (nm == "cell_cnt") return I(d.cell_cnt, (int64_t)c.nct);
  if (nm == "ij_count") return I(d.ij_count, n);
  if (nm == "ij_link") return I(d.ij_link, ell);
  if (nm == "w_Gx") return D(d.wGx, ell);
  if (nm == "w_Gy") return D(d.wGy, ell);
  if (nm == "w_L") return D(d.wL, ell);
  if (nm == "w_L32" && d.wL32) return DView{d.wL32, 4, ell};
  if (nm == "w_Gx32" && d.wGx32) return DView{d.wGx32, 4, ell};
  if (nm == "kgcm11") return D(d.kgcm[0], n);
  if (nm == "kgcm21") return D(d.kgcm[1], n);
  if (nm == "kgcm12") return D(d.kgcm[2], n);
  if (nm == "kgcm22") return D(d.kgcm[3], n);
  if (nm == "gradu_x") return D(d.grad[0], np);
  if (nm == "gradu_y") return D(d.grad[1], np);
  if (nm == "gradv_x") return D(d.grad[2], np);
  if (nm == "gradv_y") return D(d.grad[3], np);
  if (nm == "gradth_x") return D(d.grad[4], np);
  if (nm == "gradth_y") return D(d.grad[5], np);
  if (nm == "gradC_x") return D(d.gradCx, n);
  if (nm == "gradC_y") return D(d.gradCy, n);
  if (nm == "ushift_x") return D(d.ushx, n);
  if (nm == "ushift_y") return D(d.ushy, n);
  if (nm == "ustar_x") return D(d.ux2, np);
  if (nm == "ustar_y") return D(d.uy2, np);
  if (nm == "theta_star") return D(d.th, n);  // theta* is the step's final theta
  if (nm == "ppe_B") return D(d.ppe_B, n);
  if (nm == "ppe_diag") return D(d.ppe_diag, n);
  // FP64 off-diagonal values: a mixed step writes them only for rows with mirrors or smoothing
  // (and all rows while the adjoint tapes it); its solvers read ppe_val32 and rowsum
  if (nm == "ppe_val") return D(d.ppe_val, ell);
  if (nm == "ppe_col") return I(d.ppe_col, ell);
  if (nm == "grad_px") return D(d.gpx, n);
  if (nm == "grad_py") return D(d.gpy, n);
  if (nm == "conc" && d.conc) return D(d.conc, n);
  if (nm == "div_r" && d.div_r) return D(d.div_r, n);
  if (nm == "mg_pairs" && x.mg_rcnt) return I(x.mg_rcnt, n);  // (cell, value) pairs of each row of A P
  return DView{nullptr, 0, -1};
}

int vebi_debug_size(vebi_ctx* h, const char* name, int64_t* esz, int64_t* count) {
  if (!h || !name || !esz || !count) return fail(VEBI_ERR_ARG, "null argument");
  cudaStreamSynchronize(h->x.st);
  DView v = dview(h->x, name);
  if (v.n < 0) return fail(VEBI_ERR_ARG, std::string("unknown field ") + name);
  *esz = v.esz;
  *count = v.n;
  return VEBI_OK;
}

int vebi_debug_get(vebi_ctx* h, const char* name, void* out, int64_t bytes) {
  if (!h || !name || !out) return fail(VEBI_ERR_ARG, "null argument");
  cudaStreamSynchronize(h->x.st);
  DView v = dview(h->x, name);
  if (v.n < 0) return fail(VEBI_ERR_ARG, std::string("unknown field ") + name);
  if (bytes < v.n * v.esz) return fail(VEBI_ERR_ARG, "buffer too small");
  if (v.n > 0) CUDA_TRY(cudaMemcpy(out, v.p, (size_t)(v.n * v.esz), cudaMemcpyDeviceToHost));
  return VEBI_OK;
}

}  // extern "C"

namespace vebi {
int run_one_step(Ctx& x, vebi_step_stats* stats) {
  x.launches = 0;
  enqueue_step(x, 0);
  if (x.timing) cudaEventRecord(x.ev[VEBI_NSTAGES], x.st);
  return finish_step(x, stats, true);
}
}  // namespace vebi
