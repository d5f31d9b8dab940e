// vebi_output.cu -- the reference's output files from the GPU state (output.F90:18-85):
// PART dumps and the TEMP_REC.dat restart record, plus the list-directed record formatter the
// per-step TIME / LS / TIME_OUT lines use (output.F90:56,84-85).
//
// Staging.  vebi_dump_async snapshots the fields on the context's stream (device-to-device,
// right after the step) and copies the snapshot to pinned host memory on a stream of its own,
// so the copies overlap the next steps.  vebi_dump_write waits for those copies and writes the
// files, on the calling thread or on a background host thread (VEBI_DUMP_BACKGROUND), with the
// formatting split over host threads.
//
// Format.  The reference writes with list-directed output compiled by gfortran (Makefile:
// FC := gfortran): an integer(4) item is a blank and an I11 field; a real(8) item is a blank
// and a 25-wide G field with 17 significant digits and a 3-digit exponent -- F form
// (17 - k decimals, k digits before the point, then 5 blanks) for 0.1 <= |x| < 1e17 after
// rounding and for zero (16 decimals), E form with one digit before the point otherwise.  The
// formatter reproduces the reference's own list-directed files byte for byte
// (source/gen/IPART, IBOUND; tests/test_output_format.py).
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "vebi_ctx.cuh"

namespace vebi {

void vebi_set_error_text(const std::string& msg);

// ---------------------------------------------------------------- list-directed items
// one real(8) item: 26 characters (a blank separator and the 25-wide field)
static int fmt_real8(double v, char* o) {
  char num[48];
  int len = 0;
  if (std::isnan(v)) {
    len = std::snprintf(num, sizeof(num), "NaN");
  } else if (std::isinf(v)) {
    len = std::snprintf(num, sizeof(num), v < 0 ? "-Infinity" : "Infinity");
  } else if (v == 0.0) {
    len = std::snprintf(num, sizeof(num), "%s0.0000000000000000     ", std::signbit(v) ? "-" : "");
  } else {
    char e[40];
    // d.dddddddddddddddde+XX, correctly rounded to 17 significant digits (as printf's %.16e)
    const auto res = std::to_chars(e, e + sizeof(e) - 1, std::fabs(v), std::chars_format::scientific, 16);
    *res.ptr = '\0';
    char dig[17];
    dig[0] = e[0];
    std::memcpy(dig + 1, e + 2, 16);
    const int ex = std::atoi(e + 19);  // decimal exponent of the rounded value
    const int k = ex + 1;              // digits before the point in F form
    char* p = num;
    if (v < 0) *p++ = '-';
    if (k >= 0 && k <= 17) {  // F form: 17 significant digits, then 5 blanks
      if (k == 0) {
        *p++ = '0';
        *p++ = '.';
        std::memcpy(p, dig, 17);
        p += 17;
      } else {
        std::memcpy(p, dig, k);
        p += k;
        *p++ = '.';
        std::memcpy(p, dig + k, 17 - k);
        p += 17 - k;
      }
      std::memcpy(p, "     ", 5);
      p += 5;
    } else {  // E form, one digit before the point, 3-digit exponent
      *p++ = dig[0];
      *p++ = '.';
      std::memcpy(p, dig + 1, 16);
      p += 16;
      p += std::snprintf(p, 8, "E%c%03d", ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
    }
    len = (int)(p - num);
  }
  const int w = len > 25 ? len : 25;
  o[0] = ' ';
  std::memset(o + 1, ' ', (size_t)(w - len));
  std::memcpy(o + 1 + (w - len), num, (size_t)len);
  return 1 + w;
}

// one integer(4) item: 12 characters (a blank separator and I11)
static int fmt_int4(int v, char* o) {
  char t[24];
  const int len = (int)(std::to_chars(t, t + sizeof(t), v).ptr - t);
  const int w = len > 11 ? len : 11;
  o[0] = ' ';
  std::memset(o + 1, ' ', (size_t)(w - len));
  std::memcpy(o + 1 + (w - len), t, (size_t)len);
  return 1 + w;
}

// a record of kinds ('r' real(8), 'i' integer(4)) into o, with the newline; returns its length
static int fmt_record(const char* kinds, const double* r, const int32_t* iv, char* o) {
  int n = 0;
  for (const char* k = kinds; *k; ++k) n += *k == 'r' ? fmt_real8(*r++, o + n) : fmt_int4(*iv++, o + n);
  o[n++] = '\n';
  return n;
}

// ---------------------------------------------------------------- dump staging
// planes of the snapshot, in this order
enum { F_RX, F_RY, F_UX, F_UY, F_TH, F_P, F_CONC, F_AOUT, F_VORT, F_T11, F_T21, F_T12, F_T22, NF };

struct DumpState {
  cudaStream_t st = nullptr;
  cudaEvent_t ev_snap = nullptr, ev_done = nullptr;
  double* d_snap = nullptr;   // NF planes of npfb
  int* d_nsurf = nullptr;
  uint8_t* d_inbin = nullptr;
  double* h_snap = nullptr;   // pinned copies
  int* h_nsurf = nullptr;
  uint8_t* h_inbin = nullptr;
  Scal* h_scal = nullptr;
  int n = 0;
  bool pending = false;       // copies enqueued and not yet written
  std::thread writer;
  int writer_status = VEBI_OK;
  std::string writer_error;
};

void dump_free(Ctx& x) {
  DumpState* D = x.dump;
  if (!D) return;
  if (D->writer.joinable()) D->writer.join();
  if (D->st) cudaStreamSynchronize(D->st);
  cudaFree(D->d_snap);
  cudaFree(D->d_nsurf);
  cudaFree(D->d_inbin);
  cudaFreeHost(D->h_snap);
  cudaFreeHost(D->h_nsurf);
  cudaFreeHost(D->h_inbin);
  cudaFreeHost(D->h_scal);
  if (D->ev_snap) cudaEventDestroy(D->ev_snap);
  if (D->ev_done) cudaEventDestroy(D->ev_done);
  if (D->st) cudaStreamDestroy(D->st);
  delete D;
  x.dump = nullptr;
}

static int dump_alloc(Ctx& x) {
  if (x.dump) return VEBI_OK;
  auto* D = new DumpState();
  x.dump = D;
  const size_t n = (size_t)x.c.npfb;
  D->n = x.c.npfb;
  bool ok = cudaStreamCreateWithFlags(&D->st, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&D->ev_snap, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&D->ev_done, cudaEventDisableTiming) == cudaSuccess &&
            cudaMalloc((void**)&D->d_snap, sizeof(double) * n * NF) == cudaSuccess &&
            cudaMalloc((void**)&D->d_nsurf, sizeof(int) * n) == cudaSuccess &&
            cudaMalloc((void**)&D->d_inbin, n) == cudaSuccess &&
            cudaMallocHost((void**)&D->h_snap, sizeof(double) * n * NF) == cudaSuccess &&
            cudaMallocHost((void**)&D->h_nsurf, sizeof(int) * n) == cudaSuccess &&
            cudaMallocHost((void**)&D->h_inbin, n) == cudaSuccess &&
            cudaMallocHost((void**)&D->h_scal, sizeof(Scal)) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    dump_free(x);
    return VEBI_ERR_CUDA;
  }
  return VEBI_OK;
}

static int dump_join(Ctx& x) {
  DumpState* D = x.dump;
  if (!D || !D->writer.joinable()) return VEBI_OK;
  D->writer.join();
  if (D->writer_status) vebi_set_error_text(D->writer_error);
  return D->writer_status;
}

int dump_async(Ctx& x) {
  int st = dump_join(x);  // the staging buffers are free again
  if (st) return st;
  if ((st = dump_alloc(x))) return st;
  DumpState* D = x.dump;
  const size_t n = (size_t)x.c.npfb, B = sizeof(double) * n;
  const Dev& d = x.d;
  const double* src[NF] = {d.rx, d.ry, d.ux, d.uy, d.th, d.p, d.conc, d.a_out, d.vort,
                           d.tau[0], d.tau[1], d.tau[2], d.tau[3]};
  // the previous dump's host copies must finish before the snapshot is overwritten
  cudaStreamWaitEvent(x.st, D->ev_done, 0);
  for (int f = 0; f < NF; ++f) {
    if (src[f]) cudaMemcpyAsync(D->d_snap + f * n, src[f], B, cudaMemcpyDeviceToDevice, x.st);
    else cudaMemsetAsync(D->d_snap + f * n, 0, B, x.st);  // conc outside an open domain
  }
  cudaMemcpyAsync(D->d_nsurf, d.n_surf, sizeof(int) * n, cudaMemcpyDeviceToDevice, x.st);
  cudaMemcpyAsync(D->d_inbin, d.inbin, n, cudaMemcpyDeviceToDevice, x.st);
  cudaEventRecord(D->ev_snap, x.st);
  // the host copies run on the dump stream, overlapping the following steps
  cudaStreamWaitEvent(D->st, D->ev_snap, 0);
  cudaMemcpyAsync(D->h_scal, d.s, sizeof(Scal), cudaMemcpyDeviceToHost, x.st);
  cudaMemcpyAsync(D->h_snap, D->d_snap, B * NF, cudaMemcpyDeviceToHost, D->st);
  cudaMemcpyAsync(D->h_nsurf, D->d_nsurf, sizeof(int) * n, cudaMemcpyDeviceToHost, D->st);
  cudaMemcpyAsync(D->h_inbin, D->d_inbin, n, cudaMemcpyDeviceToHost, D->st);
  cudaEventRecord(D->ev_done, D->st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return VEBI_ERR_CUDA;
  D->pending = true;
  return VEBI_OK;
}

// format rows [0, n) with `line(i, buf)` over host threads and write them in order
template <class Line>
static bool write_rows(FILE* f, int n, int max_line, Line line) {
  const int nt = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), 32));
  const int chunk = 1 << 16;
  std::vector<std::string> out((size_t)nt);
  bool ok = true;
  for (int base = 0; base < n && ok; base += chunk * nt) {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
      th.emplace_back([&, t]() {
        const int a = base + t * chunk, b = std::min(n, a + chunk);
        std::string& s = out[(size_t)t];
        s.clear();
        if (a >= b) return;
        s.resize((size_t)(b - a) * (size_t)max_line);
        size_t m = 0;
        for (int i = a; i < b; ++i) m += (size_t)line(i, &s[m]);
        s.resize(m);
      });
    }
    for (auto& t : th) t.join();
    for (int t = 0; t < nt; ++t)
      if (!out[(size_t)t].empty() && std::fwrite(out[(size_t)t].data(), 1, out[(size_t)t].size(), f) != out[(size_t)t].size())
        ok = false;
  }
  return ok;
}

static int write_files(Ctx& x, vebi_dump_info info, std::string part, std::string restart, std::string* err) {
  DumpState* D = x.dump;
  if (cudaEventSynchronize(D->ev_done) != cudaSuccess) {
    *err = "dump copies failed";
    return VEBI_ERR_CUDA;
  }
  const int n = D->n;
  const double* S = D->h_snap;
  auto F = [&](int f, int i) { return S[(size_t)f * n + i]; };
  const bool ve = x.c.const_mod != 1;
  if (!part.empty()) {  // output.F90:40-51 (output_mirrors is .false., div_free.F90:36)
    FILE* f = std::fopen(part.c_str(), "w");
    if (!f) {
      *err = "cannot open " + part;
      return VEBI_ERR_ARG;
    }
    bool ok = write_rows(f, n, 14 * 26 + 2, [&](int i, char* o) -> int {
      if (D->h_inbin[i]) return 0;
      double r[13] = {F(F_RX, i), F(F_RY, i), F(F_UX, i), F(F_UY, i), F(F_TH, i), F(F_P, i), F(F_CONC, i),
                      F(F_AOUT, i), F(F_VORT, i), F(F_T11, i), F(F_T12, i), F(F_T22, i), 0.0};
      const int32_t iv[1] = {D->h_nsurf[i]};
      return fmt_record(ve ? "rrrrrrrrirrrr" : "rrrrrrrrir", r, iv, o);
    });
    ok &= std::fclose(f) == 0;
    if (!ok) {
      *err = "write failed: " + part;
      return VEBI_ERR_ARG;
    }
  }
  if (!restart.empty()) {  // output.F90:59-77
    FILE* f = std::fopen(restart.c_str(), "w");
    if (!f) {
      *err = "cannot open " + restart;
      return VEBI_ERR_ARG;
    }
    const Scal& s = *D->h_scal;
    char buf[512];
    int m;
    {
      const double r[1] = {info.time};
      const int32_t iv[2] = {info.itime, info.n_dump};
      m = fmt_record("iri", r, iv, buf);
      std::fwrite(buf, 1, (size_t)m, f);
    }
    {
      const int32_t iv[4] = {s.np - s.n_inbin, x.c.npfb - s.n_inbin, x.c.nbS, info.np_inflow};
      m = fmt_record("iiii", nullptr, iv, buf);
      std::fwrite(buf, 1, (size_t)m, f);
    }
    {
      const double r[6] = {info.xb_min, info.xb_max, info.yb_min, info.yb_max, info.dx, info.av_conc};
      m = fmt_record("rrrrrr", r, nullptr, buf);
      std::fwrite(buf, 1, (size_t)m, f);
    }
    const bool no_theta = (info.flags & VEBI_DUMP_RESTART_READABLE) != 0;
    bool ok = write_rows(f, n, 16 * 26, [&](int i, char* o) -> int {
      if (D->h_inbin[i]) return 0;
      const int32_t iv[1] = {D->h_nsurf[i]};
      int k;
      if (no_theta) {  // the layout input.F90:123-126 reads back
        const double r[6] = {F(F_RX, i), F(F_RY, i), F(F_UX, i), F(F_UY, i), F(F_P, i), info.dv};
        k = fmt_record("rrrrrri", r, iv, o);
      } else {
        const double r[7] = {F(F_RX, i), F(F_RY, i), F(F_UX, i), F(F_UY, i), F(F_TH, i), F(F_P, i), info.dv};
        k = fmt_record("rrrrrrri", r, iv, o);
      }
      if (ve) {
        const double t[4] = {F(F_T11, i), F(F_T12, i), F(F_T21, i), F(F_T22, i)};
        k += fmt_record("rrrr", t, nullptr, o + k);
      }
      return k;
    });
    ok &= std::fclose(f) == 0;
    if (!ok) {
      *err = "write failed: " + restart;
      return VEBI_ERR_ARG;
    }
  }
  return VEBI_OK;
}

int dump_write(Ctx& x, const vebi_dump_info* info, const char* part, const char* restart) {
  int st = dump_join(x);
  if (st) return st;
  DumpState* D = x.dump;
  if (!D || !D->pending) {
    vebi_set_error_text("no dump staged: call vebi_dump_async after a step first");
    return VEBI_ERR_ARG;
  }
  D->pending = false;
  const vebi_dump_info inf = *info;
  std::string ps = part ? part : "", rs = restart ? restart : "";
  if (inf.flags & VEBI_DUMP_BACKGROUND) {
    D->writer_status = VEBI_OK;
    D->writer = std::thread([&x, D, inf, ps, rs]() { D->writer_status = write_files(x, inf, ps, rs, &D->writer_error); });
    return VEBI_OK;
  }
  std::string err;
  st = write_files(x, inf, ps, rs, &err);
  if (st) vebi_set_error_text(err);
  return st;
}

int dump_wait(Ctx& x) { return dump_join(x); }

}  // namespace vebi

extern "C" int64_t vebi_format_list(const char* kinds, const double* reals, const int32_t* ints, char* out,
                                    int64_t cap) {
  if (!kinds || !out) return -1;
  int64_t need = 1;
  for (const char* k = kinds; *k; ++k) {
    if (*k != 'r' && *k != 'i') return -1;
    need += *k == 'r' ? 26 : 12;
  }
  if (cap < need + 1) return -1;
  std::vector<char> tmp((size_t)need + 64);
  const int n = vebi::fmt_record(kinds, reals, ints, tmp.data());
  if (n + 1 > cap) return -1;
  std::memcpy(out, tmp.data(), (size_t)n);
  out[n] = '\0';
  return n;
}
