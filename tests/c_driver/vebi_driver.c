/* A host driver in plain C over the C-ABI of include/vebi.h, the loop a Fortran driver runs
 * through its bind(C) module (sph2D_incom.F90:90-125): create, upload, step, log the TIME and
 * LS records (output.F90:84-85) with the list-directed formatter, dump PART and TEMP_REC.dat
 * (output.F90:40-77), download, destroy.  No Python, no PyTorch.
 *
 * usage: vebi_driver INPUT NSTEPS OUTDIR
 *   INPUT: the vebi_params struct, then r(npfb,2), u(npfb,2), tau_p(npfb,2,2), theta(npfb),
 *          trace_conf(npfb) as float64 Fortran planes (leading dimension npfb), inbin(npfb) as u8.
 *   writes OUTDIR/TIME, OUTDIR/LS, OUTDIR/PART1, OUTDIR/TEMP_REC.dat and OUTDIR/state.bin
 *   (r, u, tau_p, theta, p after the last step, float64 planes). */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "vebi.h"

static void die(const char* what, int st) {
  fprintf(stderr, "%s: status %d: %s\n", what, st, vebi_last_error());
  exit(1);
}

static FILE* open_in(const char* dir, const char* name, const char* mode) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s", dir, name);
  FILE* f = fopen(path, mode);
  if (!f) {
    fprintf(stderr, "cannot open %s\n", path);
    exit(1);
  }
  return f;
}

int main(int argc, char** argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: %s INPUT NSTEPS OUTDIR\n", argv[0]);
    return 2;
  }
  const int nsteps = atoi(argv[2]);
  const char* out = argv[3];
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 2;
  vebi_params prm;
  if (fread(&prm, sizeof prm, 1, f) != 1) return 2;
  const size_t n = (size_t)prm.npfb;
  double* r = malloc(sizeof(double) * 2 * n);
  double* u = malloc(sizeof(double) * 2 * n);
  double* tau = malloc(sizeof(double) * 4 * n);
  double* th = malloc(sizeof(double) * n);
  double* tc = malloc(sizeof(double) * n);
  double* p = malloc(sizeof(double) * n);
  uint8_t* inbin = malloc(n);
  if (fread(r, sizeof(double), 2 * n, f) != 2 * n || fread(u, sizeof(double), 2 * n, f) != 2 * n ||
      fread(tau, sizeof(double), 4 * n, f) != 4 * n || fread(th, sizeof(double), n, f) != n ||
      fread(tc, sizeof(double), n, f) != n || fread(inbin, 1, n, f) != n)
    return 2;
  fclose(f);

  vebi_ctx* ctx = NULL;
  int st = vebi_create(&prm, &ctx);
  if (st) die("vebi_create", st);
  st = vebi_upload_state(ctx, r, u, tau, th, tc, inbin, (int32_t)n);
  if (st) die("vebi_upload_state", st);

  FILE* ftime = open_in(out, "TIME", "w");
  FILE* fls = open_in(out, "LS", "w");
  double time = 0.0;
  char rec[1024];
  vebi_step_stats s;
  for (int it = 1; it <= nsteps; ++it) {
    st = vebi_step(ctx, prm.x_mint, prm.y_mint, prm.x_maxt, prm.y_maxt, it == nsteps, &s);
    if (st) die("vebi_step", st);
    time += s.dt;
    /* write(92,*) time,dt,npfb-n_inbin,max|u|,max|v|,max|P| ; write(93,*) LS_iters,LS_residual */
    const double tr[5] = {time, s.dt, s.max_abs_u, s.max_abs_v, s.max_abs_p};
    const int32_t ti[1] = {s.npfb - s.n_inbin};
    const double t92[5] = {tr[0], tr[1], tr[2], tr[3], tr[4]};
    if (vebi_format_list("rrirrr", t92, ti, rec, sizeof rec) < 0) return 3;
    fputs(rec, ftime);
    const double lr[1] = {s.LS_residual};
    const int32_t li[1] = {s.LS_iters};
    if (vebi_format_list("ir", lr, li, rec, sizeof rec) < 0) return 3;
    fputs(rec, fls);
  }
  fclose(ftime);
  fclose(fls);

  st = vebi_dump_async(ctx);
  if (st) die("vebi_dump_async", st);
  vebi_dump_info info;
  memset(&info, 0, sizeof info);
  info.time = time;
  info.dt = s.dt;
  info.xb_min = prm.x_mint;
  info.xb_max = prm.x_maxt;
  info.yb_min = prm.y_mint;
  info.yb_max = prm.y_maxt;
  info.dx = prm.dx;
  info.dv = prm.dv;
  info.itime = nsteps;
  info.n_dump = 1;
  char part[4096], rest[4096];
  snprintf(part, sizeof part, "%s/PART1", out);
  snprintf(rest, sizeof rest, "%s/TEMP_REC.dat", out);
  st = vebi_dump_write(ctx, &info, part, rest);
  if (st) die("vebi_dump_write", st);

  st = vebi_download_state(ctx, r, u, tau, th, p, NULL, NULL, NULL, NULL, NULL, (int32_t)n);
  if (st) die("vebi_download_state", st);
  FILE* fo = open_in(out, "state.bin", "wb");
  fwrite(r, sizeof(double), 2 * n, fo);
  fwrite(u, sizeof(double), 2 * n, fo);
  fwrite(tau, sizeof(double), 4 * n, fo);
  fwrite(th, sizeof(double), n, fo);
  fwrite(p, sizeof(double), n, fo);
  fclose(fo);
  vebi_destroy(ctx);
  free(r);
  free(u);
  free(tau);
  free(th);
  free(tc);
  free(p);
  free(inbin);
  printf("ok %d steps, LS_iters %d\n", nsteps, s.LS_iters);
  return 0;
}
