"""Field-by-field comparison of one GPU step against one oracle step (helpers for tests)."""
from __future__ import annotations

import numpy as np

EXACT_INT = ("irelation", "vrelation", "ij_count", "cellpart")
EXACT_ELL = ("ij_link", "w_Gx", "w_Gy", "w_L", "ppe_col", "ppe_val")

# relative tolerances (to the field's max magnitude) after one FP64 step from the same input
TOL = {
    "dP_mp": 0.0, "kgcm11": 0.0, "kgcm21": 0.0, "kgcm12": 0.0, "kgcm22": 0.0, "ppe_diag": 0.0,
    "gradu_x": 1e-13, "gradu_y": 1e-13, "gradv_x": 1e-13, "gradv_y": 1e-13,
    "gradth_x": 1e-13, "gradth_y": 1e-13,
    "gradC_x": 1e-13, "gradC_y": 1e-13, "ushift_x": 1e-13, "ushift_y": 1e-13,
    "tau11": 1e-11, "tau21": 1e-11, "tau12": 1e-11, "tau22": 1e-11, "trace_conf": 1e-13,
    "ustar_x": 1e-12, "ustar_y": 1e-12, "theta_star": 1e-13,
    "ppe_B": 1e-10,
    "p": 1e-5, "grad_px": 1e-5, "grad_py": 1e-5,
    "ux": 1e-6, "uy": 1e-6,
}


def relerr(a, b, scale=None):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    if not b.size:
        return 0.0
    if scale is None:
        scale = float(np.abs(b).max())
    return float(np.abs(a - b).max()) / max(scale, 1e-300)


def partner(name: str):
    """The other component of a vector field (x<->y): errors are relative to the vector's size,
    since one component can be pure rounding noise (e.g. d/dx on an x-periodic lattice)."""
    for a, b in (("_x", "_y"), ("_y", "_x")):
        if name.endswith(a):
            return name[: -len(a)] + b
    if name in ("ux", "uy"):
        return "uy" if name == "ux" else "ux"
    if name in ("grad_px", "grad_py"):
        return "grad_py" if name == "grad_px" else "grad_px"
    return None


def compare_step(gpu, ref, case) -> dict:
    """Return {field: (error, tolerance)}; integer/ELL fields report 0 when identical."""
    n = case.npfb
    out = {}
    cnt_g, cnt_o = gpu.get("ij_count"), ref.get("ij_count")
    out["ij_count"] = (0.0 if np.array_equal(cnt_g, cnt_o) else 1.0, 0.0)
    for name in EXACT_INT:
        if name == "ij_count":
            continue
        a, b = gpu.get(name), ref.get(name)
        out[name] = (0.0 if (a.shape == b.shape and np.array_equal(a, b)) else 1.0, 0.0)
    # r* (positions after advection/bin/escapees, plus mirrors) must be bit-identical
    for name in ("rsx", "rsy"):
        a, b = gpu.get(name), ref.get(name)
        out[name] = (0.0 if (a.shape == b.shape and np.array_equal(a, b)) else relerr(a, b) + 1e-300, 0.0)
    kmax = int(max(cnt_o.max(), 1))
    mask = np.arange(kmax)[:, None] < cnt_o[None, :]
    for name in EXACT_ELL:
        a = gpu.get(name).reshape(-1, n)[:kmax]
        b = ref.get(name).reshape(-1, n)[:kmax]
        if a.shape != b.shape:
            out[name] = (1.0, 0.0)
            continue
        same = np.array_equal(a[mask], b[mask])
        out[name] = (0.0 if same else relerr(a[mask], b[mask]) + 1e-300, 0.0)
    for name, tol in TOL.items():
        a, b = gpu.get(name), ref.get(name)
        m = min(len(a), len(b))
        if name in ("ux", "uy", "p"):
            m = n
        if len(a) < m or len(b) < m:
            out[name] = (1.0, tol)
            continue
        scale = float(np.abs(b[:m]).max()) if m else 0.0
        pn = partner(name)
        if pn is not None:
            bp = ref.get(pn)[:m]
            scale = max(scale, float(np.abs(bp).max()) if m else 0.0)
        out[name] = (relerr(a[:m], b[:m], scale), tol)
    return out


def failures(report: dict) -> dict:
    return {k: v for k, v in report.items() if not (v[0] <= v[1])}
