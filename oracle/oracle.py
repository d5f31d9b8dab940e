"""ctypes wrapper of the CPU oracle (test infrastructure only).

Mirrors the GPU solver's host API (vebisph_gb300.solver.StepSolver) so parity tests can
drive both the same way: create from a Case, upload, step, read fields and intermediates.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from vebisph_gb300 import abi
from . import build as _build

_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(_build.build()))
        vp = C.c_void_p
        P = C.POINTER
        lib.orc_create.argtypes = [P(abi.VebiParams), P(C.c_int)]
        lib.orc_create.restype = vp
        lib.orc_destroy.argtypes = [vp]
        lib.orc_set_state.argtypes = [vp, P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_double),
                                      P(C.c_double), P(C.c_uint8), C.c_int]
        lib.orc_step.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                 P(abi.VebiStepStats)]
        lib.orc_box.argtypes = [vp, P(C.c_double), P(C.c_int)]
        lib.orc_set_itermax.argtypes = [vp, C.c_int]
        lib.orc_size.argtypes = [vp, C.c_char_p, P(C.c_int64), P(C.c_int64)]
        lib.orc_get.argtypes = [vp, C.c_char_p, vp, C.c_int64]
        lib.orc_kernel_w.argtypes = [vp, C.c_double]
        lib.orc_kernel_w.restype = C.c_double
        lib.orc_kernel_fac.argtypes = [vp, C.c_double]
        lib.orc_kernel_fac.restype = C.c_double
        lib.orc_eigens.argtypes = [P(C.c_double), P(C.c_double), P(C.c_double)]
        lib.orc_threads.restype = C.c_int
        lib.orc_geometry.argtypes = [vp, C.c_int]
        lib.orc_tlm_create.argtypes = [P(abi.VebiParams), P(C.c_int)]
        lib.orc_tlm_create.restype = vp
        lib.orc_tlm_destroy.argtypes = [vp]
        lib.orc_tlm_set_state.argtypes = lib.orc_set_state.argtypes
        lib.orc_tlm_set_tangent.argtypes = [vp, P(C.c_double), P(C.c_double), P(C.c_double), C.c_int]
        lib.orc_tlm_step.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double,
                                     P(abi.VebiStepStats), P(C.c_int)]
        lib.orc_tlm_size.argtypes = [vp, C.c_char_p, P(C.c_int64)]
        lib.orc_tlm_get.argtypes = [vp, C.c_char_p, P(C.c_double), P(C.c_double), C.c_int64]
        lib.orc_tlm_set_itermax.argtypes = [vp, C.c_int]
        lib.orc_tlm_box.argtypes = [vp, P(C.c_double)]
        lib.orc_logconf_particle.argtypes = [P(C.c_double), P(C.c_double), P(C.c_double), C.c_double,
                                             C.c_double, C.c_double, C.c_int]
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


class OracleSolver:
    """One oracle context holding a Case's state."""

    def __init__(self, case, precision: int = abi.PREC_FP64):
        self.lib = load()
        self.case = case
        self.params = case.params(precision)
        st = C.c_int(0)
        self.h = self.lib.orc_create(C.byref(self.params), C.byref(st))
        if not self.h:
            raise RuntimeError(f"oracle create failed: {abi.STATUS_NAMES.get(st.value, st.value)}")
        box = (C.c_double * 4)()
        nc = (C.c_int * 2)()
        self.lib.orc_box(self.h, box, nc)
        self.x_mint, self.x_maxt, self.y_mint, self.y_maxt = list(box)
        self.ncx, self.ncy = list(nc)
        f = case.fortran_planes()
        self.upload(f["r"], f["u"], f["tau"], f["theta"], f["trace_conf"], f["inbin"], f["ld"])

    def upload(self, r, u, tau, theta, trace_conf, inbin, ld):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (r, u, tau, theta, trace_conf)]
        ib = np.ascontiguousarray(inbin, dtype=np.uint8)
        st = self.lib.orc_set_state(self.h, *[_dp(a) for a in arrs],
                                    ib.ctypes.data_as(C.POINTER(C.c_uint8)), ld)
        if st:
            raise RuntimeError(f"oracle set_state: {abi.STATUS_NAMES.get(st, st)}")

    def step(self, secondary: bool = False) -> dict:
        s = abi.VebiStepStats()
        st = self.lib.orc_step(self.h, self.x_mint, self.y_mint, self.x_maxt, self.y_maxt,
                               int(secondary), C.byref(s))
        d = s.as_dict()
        d["status"] = st
        if st:
            raise RuntimeError(f"oracle step: {abi.STATUS_NAMES.get(st, st)}")
        return d

    def get(self, name: str) -> np.ndarray:
        esz, n = C.c_int64(), C.c_int64()
        if self.lib.orc_size(self.h, name.encode(), C.byref(esz), C.byref(n)):
            raise KeyError(name)
        dt = np.float64 if esz.value == 8 else np.int32
        out = np.empty(n.value, dt)
        self.lib.orc_get(self.h, name.encode(), out.ctypes.data_as(C.c_void_p), out.nbytes)
        return out

    def set_itermax(self, itermax: int):
        self.lib.orc_set_itermax(self.h, int(itermax))

    def record_geometry(self):
        """Keep r* (after binning) and dt of every following step."""
        self.lib.orc_geometry(self.h, 1)

    def replay_geometry(self):
        """Following steps take r* and dt from the record, from its first step on, so that a
        rerun from perturbed fields is the map the tangent-linear model differentiates."""
        self.lib.orc_geometry(self.h, 2)

    def state(self) -> dict:
        """The step's state in the host's Fortran planes (fluid and wall particles)."""
        n = self.case.npfb
        r = np.stack([self.get("rx")[:n], self.get("ry")[:n]])
        u = np.stack([self.get("ux")[:n], self.get("uy")[:n]])
        tau = np.stack([self.get(f"tau{c}")[:n] for c in ("11", "21", "12", "22")])
        return dict(r=r, u=u, tau=tau, theta=self.get("theta")[:n].copy(),
                    trace_conf=self.get("trace_conf")[:n].copy(), p=self.get("p")[:n].copy())

    def W(self, q: float) -> float:
        return self.lib.orc_kernel_w(self.h, q)

    def fac(self, q: float) -> float:
        return self.lib.orc_kernel_fac(self.h, q)

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TangentLinear:
    """FP64 tangent-linear model of the step: the oracle run over forward-mode dual numbers.

    Each field (u, theta, tau, and all computed from them) carries its derivative along one
    direction; positions, dt, pair lists, weights and the PPE matrix are those of the
    unperturbed trajectory, so n steps give d(state after)/d(state before) . direction of the
    map with the geometry held at the base trajectory's."""

    def __init__(self, case, state: dict | None = None):
        self.lib = load()
        self.case = case
        self.params = case.params(abi.PREC_FP64)
        st = C.c_int(0)
        self.h = self.lib.orc_tlm_create(C.byref(self.params), C.byref(st))
        if not self.h:
            raise RuntimeError(f"oracle create failed: {abi.STATUS_NAMES.get(st.value, st.value)}")
        box = (C.c_double * 4)()
        self.lib.orc_tlm_box(self.h, box)
        self.box = tuple(box)  # x_mint, x_maxt, y_mint, y_maxt
        f = case.fortran_planes()
        self.ld = f["ld"]
        s = state or {}
        self.upload(s.get("r", f["r"]), s.get("u", f["u"]), s.get("tau", f["tau"]),
                    s.get("theta", f["theta"]), s.get("trace_conf", f["trace_conf"]), f["inbin"], f["ld"])
        self.tangent_iters = 0

    def upload(self, r, u, tau, theta, trace_conf, inbin, ld):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (r, u, tau, theta, trace_conf)]
        ib = np.ascontiguousarray(inbin, dtype=np.uint8)
        st = self.lib.orc_tlm_set_state(self.h, *[_dp(a) for a in arrs],
                                        ib.ctypes.data_as(C.POINTER(C.c_uint8)), ld)
        if st:
            raise RuntimeError(f"oracle set_state: {abi.STATUS_NAMES.get(st, st)}")

    def set_direction(self, du=None, dtau=None, dtheta=None):
        """The perturbation's direction, in the host's planes; a missing field is not perturbed."""
        n, ld = self.case.npfb, self.ld

        def planes(a, k):
            if a is None:
                return None
            out = np.zeros((k, ld)) if k > 1 else np.zeros(ld)
            out[..., :n] = a
            return np.ascontiguousarray(out)

        du, dtau, dtheta = planes(du, 2), planes(dtau, 4), planes(dtheta, 1)
        st = self.lib.orc_tlm_set_tangent(self.h, _dp(du), _dp(dtau), _dp(dtheta), ld)
        if st:
            raise RuntimeError(f"oracle set_tangent: {abi.STATUS_NAMES.get(st, st)}")

    def step(self) -> dict:
        s = abi.VebiStepStats()
        it = C.c_int(0)
        x0, x1, y0, y1 = self.box
        st = self.lib.orc_tlm_step(self.h, x0, y0, x1, y1, C.byref(s), C.byref(it))
        if st:
            raise RuntimeError(f"oracle step: {abi.STATUS_NAMES.get(st, st)}")
        self.tangent_iters = it.value
        d = s.as_dict()
        d["tangent_iters"] = it.value
        return d

    def get(self, name: str):
        """(value, derivative) of a field over all particles and mirrors."""
        n = C.c_int64()
        if self.lib.orc_tlm_size(self.h, name.encode(), C.byref(n)):
            raise KeyError(name)
        v, d = np.empty(n.value), np.empty(n.value)
        self.lib.orc_tlm_get(self.h, name.encode(), _dp(v), _dp(d), n.value)
        return v, d

    def close(self):
        if self.h:
            self.lib.orc_tlm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def logconf_particle(tau, grad_u, dt, Wi, eps_ptt=0.0, nsteps=1, trace=None):
    """nsteps of one particle's log-conformation update (constitutive_eqn_evolve) under a fixed
    velocity gradient: tau = (t11, t21, t12, t22), grad_u = (du/dx, du/dy, dv/dx, dv/dy).
    Returns the stress and the conformation trace after them."""
    lib = load()
    t = np.ascontiguousarray(np.asarray(tau, float).ravel().copy())
    g = np.ascontiguousarray(np.asarray(grad_u, float).ravel())
    tr = C.c_double(2.0 + t[0] + t[3] if trace is None else float(trace))
    lib.orc_logconf_particle(_dp(t), C.byref(tr), _dp(g), float(dt), float(Wi), float(eps_ptt), int(nsteps))
    return t, tr.value


def eigens(A):
    """calc_eigens on a 2x2 matrix given as [[a11,a12],[a21,a22]]."""
    lib = load()
    a = np.ascontiguousarray(np.asarray(A, float).ravel())
    L = np.zeros(2)
    R = np.zeros(4)
    lib.orc_eigens(_dp(a), _dp(L), _dp(R))
    return L, R.reshape(2, 2)


def threads() -> int:
    return load().orc_threads()
