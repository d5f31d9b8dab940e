"""Host-side mirror of the reference's time step over the C-ABI (include/vebi.h).

The Fortran driver calls `div_free(x_mint,y_mint,x_maxt,y_maxt)` once per step
(source/base/sph2D_incom.F90:97) on state held in module globals; `StepSolver` holds the
same state on the GPU and exposes the same call.  Every computation runs in the CUDA
library; this module only moves host arrays and reads results.  It raises when the
library is missing -- there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .cases import Case

# intermediate arrays of the last step exposed by vebi_debug_get
DEBUG_FIELDS = (
    "rx", "ry", "ux", "uy", "theta", "p", "tau11", "tau21", "tau12", "tau22", "trace_conf", "a_out",
    "vort", "n_surf", "irelation", "vrelation", "dP_mp", "rsx", "rsy", "cellpart", "ist", "cell_cnt",
    "ij_count", "ij_link", "w_Gx", "w_Gy", "w_L", "kgcm11", "kgcm21", "kgcm12", "kgcm22", "gradu_x",
    "gradu_y", "gradv_x", "gradv_y", "gradth_x", "gradth_y", "gradC_x", "gradC_y", "ushift_x",
    "ushift_y", "ustar_x", "ustar_y", "theta_star", "ppe_B", "ppe_diag", "ppe_val", "ppe_col",
    "grad_px", "grad_py", "conc", "div_r",
)


class VebiError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {abi.STATUS_NAMES.get(status, status)} {detail}".strip())


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


class StepSolver:
    """One GPU context holding one simulation's particle state.

    `handle` wraps a context owned elsewhere (an instance of a BatchSolver) instead of
    creating one."""

    def __init__(self, case: Case, precision: int = abi.PREC_FP64, timing: bool = False, handle=None):
        self.lib = abi.load_library()
        self.case = case
        self.params = case.params(precision)
        self.x_mint, self.x_maxt, self.y_mint, self.y_maxt = (
            self.params.x_mint, self.params.x_maxt, self.params.y_mint, self.params.y_maxt)
        self.owned = handle is None
        if handle is None:
            h = C.c_void_p()
            self._check(self.lib.vebi_create(C.byref(self.params), C.byref(h)), "vebi_create")
        else:
            h = handle
        self.h = h
        if timing:
            self.lib.vebi_set_timing(self.h, 1)
        f = case.fortran_planes()
        self.upload(f["r"], f["u"], f["tau"], f["theta"], f["trace_conf"], f["inbin"], f["ld"])

    def _check(self, st: int, where: str):
        if st:
            raise VebiError(st, where, self.lib.vebi_last_error().decode())

    # -- state transfer ---------------------------------------------------------------
    def upload(self, r, u, tau, theta, trace_conf, inbin, ld: int):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (r, u, tau, theta, trace_conf)]
        ib = np.ascontiguousarray(inbin, dtype=np.uint8)
        self._check(self.lib.vebi_upload_state(self.h, *[_dp(a) for a in arrs],
                                               ib.ctypes.data_as(C.POINTER(C.c_uint8)), ld),
                    "vebi_upload_state")

    def download(self, ld: int | None = None) -> dict:
        n = self.case.npfb
        ld = ld or n
        out = dict(r=np.zeros((2, ld)), u=np.zeros((2, ld)), tau=np.zeros((4, ld)), theta=np.zeros(ld),
                   p=np.zeros(ld), vort=np.zeros(ld), a_out=np.zeros(ld), trace_conf=np.zeros(ld),
                   n_surf=np.zeros(ld, np.int32), inbin=np.zeros(ld, np.uint8))
        self._check(self.lib.vebi_download_state(
            self.h, _dp(out["r"]), _dp(out["u"]), _dp(out["tau"]), _dp(out["theta"]), _dp(out["p"]),
            _dp(out["vort"]), _dp(out["a_out"]), _dp(out["trace_conf"]),
            out["n_surf"].ctypes.data_as(C.POINTER(C.c_int32)),
            out["inbin"].ctypes.data_as(C.POINTER(C.c_uint8)), ld), "vebi_download_state")
        return out

    # -- the step ---------------------------------------------------------------------
    def div_free(self, x_mint, y_mint, x_maxt, y_maxt, secondary: bool = False) -> dict:
        """The reference's call signature (div_free.F90:22)."""
        s = abi.VebiStepStats()
        st = self.lib.vebi_step(self.h, x_mint, y_mint, x_maxt, y_maxt, int(secondary), C.byref(s))
        d = s.as_dict()
        d["status"] = st
        self._check(st, "vebi_step")
        return d

    def step(self, secondary: bool = False) -> dict:
        return self.div_free(self.x_mint, self.y_mint, self.x_maxt, self.y_maxt, secondary)

    def run_steps(self, n: int) -> tuple[float, dict]:
        ms = C.c_double(0.0)
        s = abi.VebiStepStats()
        self._check(self.lib.vebi_run_steps(self.h, self.x_mint, self.y_mint, self.x_maxt, self.y_maxt, n,
                                            C.byref(ms), C.byref(s)), "vebi_run_steps")
        return ms.value, s.as_dict()

    # -- inspection -------------------------------------------------------------------
    def get(self, name: str) -> np.ndarray:
        esz, n = C.c_int64(), C.c_int64()
        self._check(self.lib.vebi_debug_size(self.h, name.encode(), C.byref(esz), C.byref(n)), name)
        out = np.empty(n.value, np.float64 if esz.value == 8 else np.int32)
        self._check(self.lib.vebi_debug_get(self.h, name.encode(), out.ctypes.data_as(C.c_void_p), out.nbytes),
                    name)
        return out

    def set_solver_grid(self, rows_per_thread: int):
        self._check(self.lib.vebi_set_solver_grid(self.h, int(rows_per_thread)), "vebi_set_solver_grid")

    def set_coarse_block_rows(self, rows: int):
        self._check(self.lib.vebi_set_coarse_block_rows(self.h, int(rows)), "vebi_set_coarse_block_rows")

    # -- output files (output.F90) ------------------------------------------------------
    def dump_async(self):
        """Snapshot the fields after the last step; the host copies overlap later steps."""
        self._check(self.lib.vebi_dump_async(self.h), "vebi_dump_async")

    def dump_write(self, part_path=None, restart_path=None, *, time=0.0, dt=0.0, itime=0, n_dump=0,
                   background=False, restart_readable=False, av_conc=0.0):
        """Write the staged snapshot as a PART dump and/or a TEMP_REC.dat restart record."""
        c = self.case
        info = abi.VebiDumpInfo(time=time, dt=dt, xb_min=self.x_mint, xb_max=self.x_maxt, yb_min=self.y_mint,
                                yb_max=self.y_maxt, dx=c.dx, av_conc=av_conc, dv=c.dv, itime=itime,
                                n_dump=n_dump, np_inflow=0,
                                flags=(abi.DUMP_BACKGROUND if background else 0) |
                                      (abi.DUMP_RESTART_READABLE if restart_readable else 0))
        enc = lambda p: None if p is None else str(p).encode()  # noqa: E731
        self._check(self.lib.vebi_dump_write(self.h, C.byref(info), enc(part_path), enc(restart_path)),
                    "vebi_dump_write")

    def dump_wait(self):
        self._check(self.lib.vebi_dump_wait(self.h), "vebi_dump_wait")

    def close(self):
        if getattr(self, "h", None):
            if self.owned:
                self.lib.vebi_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


    def set_weissenberg(self, wi: float):
        self._check(self.lib.vebi_set_weissenberg(self.h, wi), "vebi_set_weissenberg")

    def set_velocity_limit(self, u_limit: float):
        """Opt-in divergence guard: steps with a non-finite or |u| > u_limit velocity fail
        with VEBI_ERR_DIVERGED (0 turns it off)."""
        self._check(self.lib.vebi_set_velocity_limit(self.h, u_limit), "vebi_set_velocity_limit")


class Adjoint:
    """Reverse mode of a StepSolver's steps over a window (vebi_adjoint_*).

    record(n) runs n ordinary steps from the solver's state and keeps their geometry (advected
    positions, dt) and the fields every `checkpoint_every` steps; replay(n) runs the
    differentiated map -- the same steps with the recorded geometry -- from the solver's current
    fields; reverse(...) returns dJ/d(state before the window) from dJ/d(state after it).
    The solver may be FP64 or mixed-precision: a mixed window runs the mixed step, and its
    reverse sweep differentiates the mixed map in FP64 with the FP32 weights the steps used."""

    def __init__(self, solver: StepSolver, max_steps: int, checkpoint_every: int = 20):
        self.solver = solver
        self.lib = solver.lib
        h = C.c_void_p()
        solver._check(self.lib.vebi_adjoint_create(solver.h, max_steps, checkpoint_every, C.byref(h)),
                      "vebi_adjoint_create")
        self.h = h

    def record(self, nsteps: int) -> dict:
        s = abi.VebiStepStats()
        self.solver._check(self.lib.vebi_adjoint_record(self.h, nsteps, C.byref(s)), "vebi_adjoint_record")
        return s.as_dict()

    def replay(self, nsteps: int) -> dict:
        s = abi.VebiStepStats()
        self.solver._check(self.lib.vebi_adjoint_replay(self.h, nsteps, C.byref(s)), "vebi_adjoint_replay")
        return s.as_dict()

    def restore(self, step: int = 0):
        self.solver._check(self.lib.vebi_adjoint_restore(self.h, step), "vebi_adjoint_restore")

    def reverse(self, seed_u=None, seed_theta=None, seed_tau=None) -> dict:
        """Seeds: dJ/du (2, n), dJ/dtheta (n,), dJ/dtau (4, n) of the state after the window;
        returns the same of the state before it, dJ/dWi and the transposed solves' iterations."""
        n = self.solver.case.npfb

        def arr(a, shape):
            return None if a is None else np.ascontiguousarray(np.broadcast_to(a, shape), dtype=np.float64)

        su, sth, sta = arr(seed_u, (2, n)), arr(seed_theta, (n,)), arr(seed_tau, (4, n))
        gu, gth, gta = np.zeros((2, n)), np.zeros(n), np.zeros((4, n))
        gwi = C.c_double(0.0)
        its = C.c_int32(0)
        self.solver._check(self.lib.vebi_adjoint_reverse(self.h, _dp(su), _dp(sth), _dp(sta), n, _dp(gu), _dp(gth),
                                                         _dp(gta), C.byref(gwi), C.byref(its)),
                           "vebi_adjoint_reverse")
        return dict(u=gu, theta=gth, tau=gta, wi=gwi.value, ls_iters=its.value)

    def close(self):
        if getattr(self, "h", None):
            self.lib.vebi_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchSolver:
    """Independent simulations of uneven sizes advanced together (vebi_batch_*): every batch
    step replays each instance's captured step graph on its own stream; one wait per call."""

    def __init__(self, cases_list, precision: int = abi.PREC_MIXED):
        self.lib = abi.load_library()
        n = len(cases_list)
        arr = (abi.VebiParams * n)(*[c.params(precision) for c in cases_list])
        h = C.c_void_p()
        st = self.lib.vebi_batch_create(arr, n, C.byref(h))
        if st:
            raise VebiError(st, "vebi_batch_create", self.lib.vebi_last_error().decode())
        self.h = h
        self.instances = []
        for i, c in enumerate(cases_list):
            ch = C.c_void_p()
            self.lib.vebi_batch_get(self.h, i, C.byref(ch))
            self.instances.append(StepSolver(c, precision, handle=ch))
        self.n_fluid = sum(c.n_fluid for c in cases_list)

    def step(self, nsteps: int = 1):
        """Advance every instance by nsteps; returns (device ms, per-instance stats)."""
        n = len(self.instances)
        stats = (abi.VebiStepStats * n)()
        ms = C.c_double(0.0)
        st = self.lib.vebi_batch_step(self.h, int(nsteps), C.byref(ms), stats)
        if st:
            raise VebiError(st, "vebi_batch_step", self.lib.vebi_last_error().decode())
        # instances that failed carry their status in stats[i]["error"]; the others went on
        return ms.value, [stats[i].as_dict() for i in range(n)]

    def set_solver_grid(self, rows_per_thread: int):
        for inst in self.instances:
            inst.set_solver_grid(rows_per_thread)

    def set_coarse_block_rows(self, rows: int):
        for inst in self.instances:
            inst.set_coarse_block_rows(rows)

    def autotune(self, candidates=(1, 2, 4, 8), coarse_candidates=(2048,)) -> dict:
        """Pick the batch's solver tiles by measurement: the rows each solver thread owns (so
        the rows per block and the blocks per instance) and, with the multigrid preconditioner,
        the size up to which coarse levels run in one block.  Every pair of candidates costs one
        step to capture the graphs and one timed step (real steps of the simulations).  The rows
        per thread set the solver's block count and so the order of its block-partial sums
        (results move by rounding); the coarse-level size leaves results unchanged."""
        times = {}
        for r in candidates:
            for cb in coarse_candidates:
                self.set_solver_grid(r)
                self.set_coarse_block_rows(cb)
                self.step(1)
                ms, _ = self.step(1)
                times[(r, cb)] = ms
        best = min(times, key=times.get)
        self.set_solver_grid(best[0])
        self.set_coarse_block_rows(best[1])
        return {"rows_per_thread": best[0], "coarse_block_rows": best[1],
                "ms_per_candidate": {f"{r},{cb}": v for (r, cb), v in times.items()}}

    def close(self):
        if getattr(self, "h", None):
            for inst in self.instances:
                inst.h = None
            self.lib.vebi_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
