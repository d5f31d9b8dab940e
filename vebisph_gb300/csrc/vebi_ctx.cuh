// vebi_ctx.cuh -- host-side context of one simulation (opaque vebi_ctx of include/vebi.h).
#pragma once

#include <cstdio>
#include <string>
#include <vector>

#include "vebi_common.cuh"

namespace vebi {

struct DumpState;

struct Ctx {
  vebi_params prm{};
  Consts c{};
  Dev d{};
  cudaStream_t st = nullptr;
  int device = 0;
  int nsm = 0;
  int launches = 0;
  bool timing = false;
  cudaEvent_t ev[VEBI_NSTAGES + 1]{};
  bool ev_used[VEBI_NSTAGES]{};
  cudaEvent_t* ev_run = nullptr;   // per-step stage events of vebi_run_steps (timing on)
  int ev_run_step = -1;            // step whose events stage_mark records, -1 = use ev[]
  bool capturing = false;          // enqueue_step is being captured into a CUDA graph
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // one step: [0] plain, [1] with stage events
  bool graph_failed[2] = {false, false};
  int graph_launches[2] = {0, 0};
  bool graph_used[2][VEBI_NSTAGES] = {};
  int coop_blocks = 0;       // persistent PPE grid (co-resident blocks)
  int coop_blocks_mixed = 0; // same for the mixed-precision solver
  int solver_rows_per_thread = 1;  // batch tuning: rows per solver thread
  int mg_block_rows = MG_BLOCK_ROWS;  // batch tuning: coarse levels of at most this many rows run in one block
  int grid_gen = 0;                // bumped when a launch shape changes (captured graphs are stale)
  int gs_blocks = 0;         // grid of grid-stride kernels over dynamic counts
  int sel_max_blocks = 0;    // blocks of the ordered-select kernels
  int precision = VEBI_PREC_FP64;
  bool have_state = false;
  // multigrid-preconditioned PPE (opt-in)
  std::vector<MgLevel> mg;         // coarse levels, finest first
  MgLevel* d_mg = nullptr;         // device copy of the level descriptors
  int mg_blocks = 0;               // co-resident blocks of the preconditioned solver (FP64)
  int mg_blocks_mixed = 0;         // the same for the mixed-precision kernel
  double *mg_z = nullptr, *mg_fr = nullptr, *mg_dinv0 = nullptr, *mg_rsum = nullptr, *mg_w = nullptr;
  int *mg_ragg = nullptr, *mg_rcnt = nullptr;  // per-row (cell, value) pairs of the level-1 build
  double* mg_kinv = nullptr;       // dense inverse of the coarsest level
  int* mg_kinv_ok = nullptr;
  double* mg_rval = nullptr;
  // the same rows by 3x3 direction for the V-cycle's output pass: values [8][n] (own cell
  // excluded, zero where unused) and a packed word per row (list start | count << 8 | used << 16)
  double* mg_rv9 = nullptr;
  int* mg_rx = nullptr;
  float* mg_g32 = nullptr;         // mixed precision: the level-1 solution rounded to FP32
  float* mg_q32 = nullptr;         // mixed precision: the V-cycle's input rounded to FP32
  std::vector<void*> allocs;
  DumpState* dump = nullptr;       // output staging (vebi_output.cu), made at the first dump
  // adjoint window (vebi_adjoint.cu): right after advection a step records its geometry --
  // the advected positions r* (x plane, y plane, npfb each) and dt -- into rec_geo, or takes
  // them from rep_geo instead of its own, so that it replays a recorded step's geometry
  double* rec_geo = nullptr;
  const double* rep_geo = nullptr;
  // adjoint: when set, the step takes its pressure (npfb values) from rep_p instead of solving
  // the PPE; the reverse sweep's recompute of a recorded step, whose solution is known
  const double* rep_p = nullptr;
  vebi_step_stats last{};
};

// one step kernel by kernel (no graph), with the adjoint hooks above; the step's status
int run_one_step(Ctx& x, vebi_step_stats* stats);
// the context behind a handle (nullptr for a null handle)
Ctx* ctx_of(vebi_ctx* h);

// kernel launch with launch accounting and an immediate launch-error check
#define VEBI_LAUNCH(x, kern, grid, block, ...)                         \
  do {                                                                 \
    kern<<<(grid), (block), 0, (x).st>>>(__VA_ARGS__);                 \
    (x).launches++;                                                    \
  } while (0)

inline int grid_for(long long n, int tpb = TPB) {
  long long g = (n + tpb - 1) / tpb;
  if (g < 1) g = 1;
  return (int)g;
}

// stage timers: record the start event of stage `s` (ends at the next recorded stage)
inline void stage_mark(Ctx& x, int s) {
  if (!x.timing) return;
  if (x.capturing) cudaEventRecordWithFlags(x.ev[s], x.st, cudaEventRecordExternal);
  else if (x.ev_run_step >= 0) cudaEventRecord(x.ev_run[(size_t)x.ev_run_step * (VEBI_NSTAGES + 1) + s], x.st);
  else cudaEventRecord(x.ev[s], x.st);
  x.ev_used[s] = true;
}

// ordered-select items per block
constexpr int SEL_IPT = 8;
constexpr int SEL_CH = TPB * SEL_IPT;

}  // namespace vebi
