"""Case decks for the step: readers of the reference's text inputs and synthetic generators.

* `read_deck` parses INDAT / IBOUND / IPART as getdata does (source/base/input.F90:18-145).
* `rayleigh_benard_deck` restates the case generator's case 4 (source/gen/datclass.F90:280-352)
  including its wall-particle rules (make_boundary_particles, datclass.F90:746-815) and its
  accumulated-sum lattice, so it reproduces the deck shipped with the reference bit for bit.
* `poiseuille`, `cylinder`, `cavity` build the seeded synthetic workloads: jittered square
  lattices (U(-0.01dx, 0.01dx) per coordinate), walls and circles placed by the same
  make_boundary_particles rules, h = 1.3 dx as in every generator case (datclass.F90:237).

All arrays are float64; particle order is walls first (1..nbS), fluid after, as in the
reference.  Fields are returned particle-major (N, m); `fortran_planes` converts to the
column-major planes the C-ABI takes.
"""
from __future__ import annotations

import dataclasses
import math
import pathlib

import numpy as np

from . import abi

PI = 3.14159265358979323846


@dataclasses.dataclass
class Case:
    name: str
    r: np.ndarray            # (N, 2)
    u: np.ndarray            # (N, 2)
    theta: np.ndarray        # (N,)
    npfb: int
    nbS: int
    h: float
    dx: float
    dv: float
    Ra: float
    Pr: float
    El: float
    beta: float
    body_force: tuple
    ve_nonlinearity: float = 0.0
    alpha_evss: float = 0.0
    dt_coef_cfl: float = 0.4
    dt_coef_visc: float = 0.2
    i_open_domain: int = 0
    i_shift_coeff: int = 0
    const_mod: int = 2
    tmax: float = 100.0
    dt_out: float = 0.1
    b_node: np.ndarray = None        # (nb, 2)
    b_edge: np.ndarray = None        # (nb, 2)
    b_type: np.ndarray = None        # (nb,)
    b_vel: np.ndarray = None
    b_thermal: np.ndarray = None
    b_periodic_parent: np.ndarray = None  # 1-based patch numbers
    c_centre: np.ndarray = None      # (nc, 2)
    c_radius: np.ndarray = None
    c_omega: np.ndarray = None
    c_vel: np.ndarray = None
    c_thermal: np.ndarray = None
    tau: np.ndarray = None           # (N, 4) planes (1,1),(2,1),(1,2),(2,2)
    trace_conf: np.ndarray = None    # (N,)
    tol: float = 1.0e-8
    itermax: int = 1000
    nplink: int = 75
    nmirror_cap: int = 0
    correct_velocity: int = 0
    ppe_warm_start: int = 0
    ppe_precond: int = 0

    def __post_init__(self):
        n = self.npfb
        if self.tau is None:
            self.tau = np.zeros((n, 4))
        if self.trace_conf is None:
            self.trace_conf = np.full(n, 2.0)   # input.F90:111
        if self.c_centre is None:
            self.c_centre = np.zeros((0, 2))
            self.c_radius = np.zeros(0)
            self.c_omega = np.zeros(0)
            self.c_vel = np.zeros((0, 2))
            self.c_thermal = np.zeros(0)

    @property
    def nb_patches(self) -> int:
        return len(self.b_type)

    @property
    def nb_circles(self) -> int:
        return len(self.c_radius)

    @property
    def n_fluid(self) -> int:
        return self.npfb - self.nbS

    def box(self):
        """Padded box of the driver (sph2D_incom.F90:64-67): x_mint, x_maxt, y_mint, y_maxt."""
        sup = 3.0 * self.h
        return (float(self.b_node[:, 0].min()) - sup * 1.5, float(self.b_node[:, 0].max()) + sup * 1.5,
                float(self.b_node[:, 1].min()) - sup * 1.5, float(self.b_node[:, 1].max()) + sup * 1.5)

    def params(self, precision: int = abi.PREC_FP64) -> abi.VebiParams:
        p = abi.VebiParams()
        for k in ("h", "dx", "dv", "Ra", "Pr", "El", "beta", "ve_nonlinearity", "alpha_evss",
                  "dt_coef_cfl", "dt_coef_visc", "tol"):
            setattr(p, k, float(getattr(self, k)))
        p.body_force[0], p.body_force[1] = float(self.body_force[0]), float(self.body_force[1])
        p.x_mint, p.x_maxt, p.y_mint, p.y_maxt = self.box()
        nb = self.nb_patches
        if nb > abi.MAX_PATCHES or self.nb_circles > abi.MAX_CIRCLES:
            raise ValueError("too many patches or circles")
        for i in range(nb):
            p.b_node[i][0], p.b_node[i][1] = self.b_node[i]
            p.b_edge[i][0], p.b_edge[i][1] = self.b_edge[i]
            p.b_vel[i] = self.b_vel[i]
            p.b_thermal[i] = self.b_thermal[i]
            p.b_type[i] = int(self.b_type[i])
            p.b_periodic_parent[i] = int(self.b_periodic_parent[i])
        for i in range(self.nb_circles):
            p.c_centre[i][0], p.c_centre[i][1] = self.c_centre[i]
            p.c_radius[i] = self.c_radius[i]
            p.c_omega[i] = self.c_omega[i]
            p.c_vel[i][0], p.c_vel[i][1] = self.c_vel[i]
            p.c_thermal[i] = self.c_thermal[i]
        p.nb_patches = nb
        p.nb_circles = self.nb_circles
        p.i_open_domain = self.i_open_domain
        p.i_shift_coeff = self.i_shift_coeff
        p.npfb = self.npfb
        p.nbS = self.nbS
        p.const_mod = self.const_mod
        p.itermax = self.itermax
        p.nplink = self.nplink
        p.nmirror_cap = self.nmirror_cap
        p.precision = precision
        p.correct_velocity = self.correct_velocity
        p.ppe_warm_start = self.ppe_warm_start
        p.ppe_precond = self.ppe_precond
        return p

    def fortran_planes(self, ld: int | None = None) -> dict:
        """Host arrays in the reference's column-major layout with leading dimension ld."""
        n = self.npfb
        ld = ld or n

        def planes(a, m):
            out = np.zeros((m, ld))
            out[:, :n] = np.asarray(a).reshape(n, m).T
            return out

        return dict(r=planes(self.r, 2), u=planes(self.u, 2), tau=planes(self.tau, 4),
                    theta=planes(self.theta, 1)[0], trace_conf=planes(self.trace_conf, 1)[0],
                    inbin=np.zeros(ld, np.uint8), ld=ld)


# ----------------------------------------------------------------------------- walls
def make_boundary_edge_vectors(b_node):
    """datclass.F90:730-744."""
    nb = len(b_node)
    return np.array([b_node[(i + 1) % nb] - b_node[i] for i in range(nb)])


def make_boundary_particles(b_node, b_edge, b_type, b_vel, b_thermal, dx,
                            c_centre=(), c_radius=(), c_omega=(), c_vel=(), c_thermal=()):
    """Circle then wall particles as in make_boundary_particles (datclass.F90:746-815).

    Positions along a wall are b_node + tmp*b_edge with tmp accumulated by repeated
    addition of dx/|edge|, exactly as the Fortran loop does."""
    xs, ys, us, vs, ths = [], [], [], [], []
    for ib in range(len(c_radius)):
        R = abs(float(c_radius[ib]))
        tmp = 2.0 * R * PI
        nround = math.ceil(tmp / dx)
        for iround in range(1, nround + 1):
            tmp2 = iround * 2.0 * PI / nround
            xs.append(c_centre[ib][0] + R * math.cos(tmp2))
            ys.append(c_centre[ib][1] + R * math.sin(tmp2))
            us.append(c_vel[ib][0] + c_omega[ib] * R * math.sin(tmp2))
            vs.append(c_vel[ib][1] - c_omega[ib] * R * math.cos(tmp2))
            ths.append(float(c_thermal[ib]))
    nb = len(b_type)
    for ib in range(nb):
        ibm1 = (ib + nb - 1) % nb
        if abs(b_type[ib]) == 1:
            e0, e1 = float(b_edge[ib][0]), float(b_edge[ib][1])
            m_be = math.sqrt(e0 * e0 + e1 * e1)
            x, y = float(b_node[ib][0]), float(b_node[ib][1])
            tmp = 0.0
            while tmp < 1.0 - 1.0e-10:
                xs.append(x)
                ys.append(y)
                u0 = b_vel[ib] * e0 / m_be
                v0 = b_vel[ib] * e1 / m_be
                if abs(b_type[ibm1]) == 1 and b_vel[ibm1] != 0.0 and tmp == 0.0:
                    pm = math.sqrt(b_edge[ibm1][0] ** 2 + b_edge[ibm1][1] ** 2)
                    u0 = b_vel[ibm1] * b_edge[ibm1][0] / pm
                    v0 = b_vel[ibm1] * b_edge[ibm1][1] / pm
                us.append(u0)
                vs.append(v0)
                ths.append(float(b_thermal[ib]))
                tmp = tmp + dx / m_be
                x = b_node[ib][0] + tmp * e0
                y = b_node[ib][1] + tmp * e1
        elif abs(b_type[ibm1]) == 1:
            xs.append(float(b_node[ib][0]))
            ys.append(float(b_node[ib][1]))
            pm = math.sqrt(b_edge[ibm1][0] ** 2 + b_edge[ibm1][1] ** 2)
            us.append(b_vel[ibm1] * b_edge[ibm1][0] / pm)
            vs.append(b_vel[ibm1] * b_edge[ibm1][1] / pm)
            ths.append(float(b_thermal[ibm1]))
    return (np.array(xs, float), np.array(ys, float), np.array(us, float), np.array(vs, float),
            np.array(ths, float))


def _channel_boundaries(x0, x1, y0, y1):
    """Four patches: bottom wall, right periodic, top wall, left periodic (datclass case 3/4).
    Walls carry parent 0 (IBOUND lists a parent only for periodic patches)."""
    b_node = np.array([[x0, y0], [x1, y0], [x1, y1], [x0, y1]], float)
    return dict(b_node=b_node, b_edge=make_boundary_edge_vectors(b_node),
                b_type=np.array([1, 2, 1, 2]), b_periodic_parent=np.array([0, 4, 0, 2]))


# ----------------------------------------------------------------------------- decks
def rayleigh_benard_deck() -> Case:
    """Restatement of datclass case 4 (datclass.F90:280-352) as written to INDAT/IBOUND/IPART.

    Values pass through the same text formats as the written deck: INDAT floats with
    F18.10 (datclass.F90:662-682), IPART/IBOUND list-directed (full precision)."""
    xl = yl = 1.0
    dx = yl / 100.0
    h = 1.3 * dx
    bd = _channel_boundaries(0.0, xl, 0.0, yl)
    b_vel = np.array([-0.0, 0.0, 0.0, 0.0])
    b_thermal = np.array([1.0, 0.0, -1.0, 0.0])
    xs, ys, us, vs, ths = make_boundary_particles(bd["b_node"], bd["b_edge"], bd["b_type"], b_vel,
                                                  b_thermal, dx)
    nbS = len(xs)
    fx, fy, ft = [], [], []
    x = 0.0 + 0.5 * dx
    while x < xl:
        y = 0.0 + dx
        while y < yl - 0.5 * dx:
            fx.append(x)
            fy.append(y)
            ft.append(1.0 if y <= 0.5 * yl + 0.25 * yl * math.sin(2.0 * PI * x) else -1.0)
            y = y + dx
        x = x + dx
    r = np.stack([np.concatenate([xs, fx]), np.concatenate([ys, fy])], 1)
    u = np.stack([np.concatenate([us, np.zeros(len(fx))]), np.concatenate([vs, np.zeros(len(fx))])], 1)
    theta = np.concatenate([ths, ft])
    f18 = lambda v: float(f"{v:18.10f}")  # noqa: E731  (INDAT round trip)
    return Case(name="rayleigh_benard_10102", r=r, u=u, theta=theta, npfb=len(r), nbS=nbS,
                h=f18(h), dx=f18(dx), dv=dx * dx, Ra=1.0e4, Pr=1.0, El=1.0e-4, beta=0.9,
                body_force=(0.0, 0.0), ve_nonlinearity=0.1, alpha_evss=0.0,
                b_vel=b_vel, b_thermal=b_thermal, dt_out=f18(float(np.float32(0.1))), **bd)


def read_deck(directory) -> Case:
    """getdata (input.F90:12-180) for a non-restart deck: INDAT, IBOUND, IPART."""
    d = pathlib.Path(directory)
    ind = [ln.split() for ln in (d / "INDAT").read_text().splitlines() if ln.strip()]
    num = lambda s: float(s.replace("D", "E").replace("d", "e"))  # noqa: E731
    i_restart = ind[0][0].upper().startswith(("T", ".T"))
    if i_restart:
        raise ValueError("restart decks (TEMP_REC) are not read by this reader")
    vals = dict(
        i_open_domain=int(ind[1][0]), tmax=num(ind[2][0]), i_shift_coeff=int(ind[3][0]),
        np=int(ind[4][0]), npfb=int(ind[5][0]), nbS=int(ind[6][0]), dt_out=num(ind[7][0]),
        h=num(ind[8][0]), dx=num(ind[9][0]), body_force=(num(ind[11][0]), num(ind[11][1])),
        Ra=num(ind[12][0]), Pr=num(ind[13][0]), El=num(ind[14][0]), beta=num(ind[15][0]),
        dt_coef_cfl=num(ind[16][0]), dt_coef_visc=num(ind[16][1]),
        ve_nonlinearity=num(ind[17][0]), alpha_evss=num(ind[18][0]))
    # IBOUND: one record per line, trailing comment text after the numbers
    lines = [ln for ln in (d / "IBOUND").read_text().splitlines() if ln.strip()]
    li = 0

    def line_nums(k):
        nonlocal li
        parts = lines[li].split()
        li += 1
        return [num(x) for x in parts[:k]]

    nb = int(line_nums(1)[0])
    b_node, b_edge, b_type, b_vel, b_th, b_pp = [], [], [], [], [], []
    for _ in range(nb):
        b_node.append(line_nums(2))
        b_edge.append(line_nums(2))
        t = int(line_nums(1)[0])
        b_type.append(t)
        b_vel.append(line_nums(1)[0])
        b_th.append(line_nums(1)[0])
        b_pp.append(int(line_nums(1)[0]) if t == 2 else 0)
        if t == 3:
            line_nums(1)
    ncirc = int(line_nums(1)[0])
    cc, cr, co, cv, ct = [], [], [], [], []
    for _ in range(ncirc):
        cc.append(line_nums(2))
        cr.append(line_nums(1)[0])
        co.append(line_nums(1)[0])
        cv.append(line_nums(2))
        ct.append(line_nums(1)[0])
    ip = np.loadtxt(d / "IPART", ndmin=2)
    npfb = vals["npfb"]
    ip = ip[:npfb]
    dv = float(ip[-1, 5])  # the reference keeps the last particle's dv (input.F90:140)
    return Case(
        name=d.name, r=ip[:, 0:2].copy(), u=ip[:, 2:4].copy(), theta=ip[:, 4].copy(), npfb=npfb,
        nbS=vals["nbS"], h=vals["h"], dx=vals["dx"], dv=dv, Ra=vals["Ra"], Pr=vals["Pr"],
        El=vals["El"], beta=vals["beta"], body_force=vals["body_force"],
        ve_nonlinearity=vals["ve_nonlinearity"], alpha_evss=vals["alpha_evss"],
        dt_coef_cfl=vals["dt_coef_cfl"], dt_coef_visc=vals["dt_coef_visc"],
        i_open_domain=vals["i_open_domain"], i_shift_coeff=vals["i_shift_coeff"],
        tmax=vals["tmax"], dt_out=vals["dt_out"],
        b_node=np.array(b_node), b_edge=np.array(b_edge), b_type=np.array(b_type),
        b_vel=np.array(b_vel), b_thermal=np.array(b_th), b_periodic_parent=np.array(b_pp),
        c_centre=np.array(cc).reshape(-1, 2), c_radius=np.array(cr), c_omega=np.array(co),
        c_vel=np.array(cv).reshape(-1, 2), c_thermal=np.array(ct))


# ----------------------------------------------------------------------------- synthetic
def _jitter(rng, n, dx):
    return rng.uniform(-0.01 * dx, 0.01 * dx, size=(n, 2))


def poiseuille(n: int = 40, seed: int = 0, Re: float = 0.1, Wi: float = 1.0, beta: float = 0.1,
               const_mod: int = 2) -> Case:
    """Planar Poiseuille flow of an Oldroyd-B fluid in the unit square, periodic in x,
    no-slip walls at y=0,1; an n x n cell-centred jittered lattice.  Pr=1, Ra=Re^2,
    El=Wi/Re, body force 8/Re gives unit centreline velocity (total viscosity 1/Re)."""
    dx = 1.0 / n
    h = 1.3 * dx
    bd = _channel_boundaries(0.0, 1.0, 0.0, 1.0)
    b_vel = np.zeros(4)
    b_th = np.zeros(4)
    xs, ys, us, vs, ths = make_boundary_particles(bd["b_node"], bd["b_edge"], bd["b_type"], b_vel, b_th, dx)
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")  # x outer, y inner
    fr = np.stack([(ii.ravel() + 0.5) * dx, (jj.ravel() + 0.5) * dx], 1)
    fr += _jitter(np.random.default_rng(seed), len(fr), dx)
    r = np.concatenate([np.stack([xs, ys], 1), fr])
    u = np.concatenate([np.stack([us, vs], 1), np.zeros_like(fr)])
    theta = np.concatenate([ths, np.zeros(len(fr))])
    Pr = 1.0
    Ra = Re * Re * Pr
    return Case(name=f"poiseuille_{n}x{n}", r=r, u=u, theta=theta, npfb=len(r), nbS=len(xs), h=h, dx=dx,
                dv=dx * dx, Ra=Ra, Pr=Pr, El=Wi / Re, beta=beta, body_force=(8.0 / Re, 0.0),
                ve_nonlinearity=0.0, const_mod=const_mod, b_vel=b_vel, b_thermal=b_th, **bd)


def cylinder(n_fluid_target: float = 4.0e6, Wi: float = 0.6, seed: int = 0, Re: float = 0.01,
             beta: float = 0.59, R: float = 1.0, length: float = 30.0, height: float = 4.0,
             U: float = 1.0, dx: float | None = None) -> Case:
    """Confined flow past a cylinder: channel length x height (30R x 4R, blockage 0.5),
    cylinder of radius R on the centreline (an empty circle, c_radius=+R), walls at
    y=+-height/2, periodic in x, jittered lattice outside r > R + 0.25dx (datclass case 5
    rule, datclass.F90:422).  Oldroyd-B, Pr=1, Ra=Re^2, El=Wi/Re.  The body force
    12 U/(Re H^2) drives a mean velocity U; u starts on the parabolic channel profile."""
    H = height
    if dx is None:
        area = length * H - PI * R * R
        dx = H / round(H / math.sqrt(area / n_fluid_target))
    h = 1.3 * dx
    bd = _channel_boundaries(-0.5 * length, 0.5 * length, -0.5 * H, 0.5 * H)
    b_vel = np.zeros(4)
    b_th = np.zeros(4)
    cc = np.array([[0.0, 0.0]])
    cr = np.array([R])
    xs, ys, us, vs, ths = make_boundary_particles(bd["b_node"], bd["b_edge"], bd["b_type"], b_vel, b_th, dx,
                                                  cc, cr, [0.0], [[0.0, 0.0]], [0.0])
    nx = int(round(length / dx))
    ny = int(round(H / dx))
    ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    x = -0.5 * length + (ii.ravel() + 0.5) * dx
    y = -0.5 * H + (jj.ravel() + 0.5) * dx
    keep = x * x + y * y > (R + 0.25 * dx) ** 2
    fr = np.stack([x[keep], y[keep]], 1)
    fr += _jitter(np.random.default_rng(seed), len(fr), dx)
    fu = np.zeros_like(fr)
    fu[:, 0] = 1.5 * U * (1.0 - (2.0 * fr[:, 1] / H) ** 2)
    r = np.concatenate([np.stack([xs, ys], 1), fr])
    u = np.concatenate([np.stack([us, vs], 1), fu])
    theta = np.zeros(len(r))
    Pr = 1.0
    Ra = Re * Re * Pr
    return Case(name=f"cylinder_{len(fr)}_Wi{Wi}", r=r, u=u, theta=theta, npfb=len(r), nbS=len(xs), h=h,
                dx=dx, dv=dx * dx, Ra=Ra, Pr=Pr, El=Wi / Re, beta=beta,
                body_force=(12.0 * U / (Re * H * H), 0.0), ve_nonlinearity=0.0, b_vel=b_vel, b_thermal=b_th,
                c_centre=cc, c_radius=cr, c_omega=np.zeros(1), c_vel=np.zeros((1, 2)),
                c_thermal=np.zeros(1), **bd)


def cavity(n: int = 1024, seed: int = 0, Ra: float = 1.0e5, Pr: float = 1.0, Wi: float = 0.5,
           beta: float = 0.5, amp: float = 1.0e-3, corr: float = 0.05, n_bumps: int = 64) -> Case:
    """Differentially heated square cavity: all four walls no-slip (b_type 1), left/right
    walls at theta = +-1/2, top/bottom walls at theta = 0 (the reference has no adiabatic
    wall).  theta0 = linear wall-to-wall profile plus a seeded sum of Gaussian bumps
    (amplitude amp, correlation length corr)."""
    dx = 1.0 / n
    h = 1.3 * dx
    b_node = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])
    b_edge = make_boundary_edge_vectors(b_node)
    b_type = np.array([1, 1, 1, 1])
    b_vel = np.zeros(4)
    b_th = np.array([0.0, -0.5, 0.0, 0.5])
    xs, ys, us, vs, ths = make_boundary_particles(b_node, b_edge, b_type, b_vel, b_th, dx)
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    fr = np.stack([(ii.ravel() + 0.5) * dx, (jj.ravel() + 0.5) * dx], 1)
    rng = np.random.default_rng(seed)
    fr += _jitter(rng, len(fr), dx)
    th = 0.5 - fr[:, 0]
    centres = rng.uniform(0, 1, size=(n_bumps, 2))
    signs = rng.normal(size=n_bumps)
    pert = np.zeros(len(fr))
    for c, s in zip(centres, signs):
        pert += s * np.exp(-((fr[:, 0] - c[0]) ** 2 + (fr[:, 1] - c[1]) ** 2) / (2 * corr * corr))
    pert *= amp / max(np.abs(pert).max(), 1e-300)
    r = np.concatenate([np.stack([xs, ys], 1), fr])
    u = np.concatenate([np.stack([us, vs], 1), np.zeros_like(fr)])
    theta = np.concatenate([ths, th + pert])
    Re = math.sqrt(Ra / Pr)
    return Case(name=f"cavity_{n}x{n}", r=r, u=u, theta=theta, npfb=len(r), nbS=len(xs), h=h, dx=dx,
                dv=dx * dx, Ra=Ra, Pr=Pr, El=Wi / Re, beta=beta, body_force=(0.0, 0.0),
                ve_nonlinearity=0.0, b_node=b_node, b_edge=b_edge, b_type=b_type, b_vel=b_vel,
                b_thermal=b_th, b_periodic_parent=np.zeros(4, int))


def free_surface_periodic(n: int = 75, seed: int | None = None) -> Case:
    """Open-domain case: datclass case 8 "FREE SURFACE PERIODIC" (datclass.F90:561-631) --
    a 2x2 box, wall at y=0, periodic in x, no boundary on top (b_type 0), fluid filling
    y < 1, i_open_domain=1, shift_coeff=1, PTT with ve_nonlinearity=400, beta=0.1, Ra=1e3,
    Pr=10, El=1, dx = 2/n.  seed=None gives the unjittered lattice of the generator."""
    xl = yl = 2.0
    dx = yl / n
    h = 1.3 * dx
    b_node = np.array([[0.0, 0.0], [xl, 0.0], [xl, yl], [0.0, yl]])
    b_edge = make_boundary_edge_vectors(b_node)
    b_type = np.array([1, 2, 0, 2])
    b_vel = np.array([-0.0, 0.0, 0.0, 0.0])
    b_th = np.array([1.0, 0.0, -1.0, 0.0])
    xs, ys, us, vs, ths = make_boundary_particles(b_node, b_edge, b_type, b_vel, b_th, dx)
    fx, fy, ft = [], [], []
    x = 0.0 + 0.5 * dx
    while x < xl:
        y = 0.0 + dx
        while y < 0.5 * yl:
            fx.append(x)
            fy.append(y)
            ft.append(1.0 if y <= 0.125 * yl + 0.0625 * yl * math.sin(2.0 * PI * x) else -1.0)
            y = y + dx
        x = x + dx
    fr = np.stack([fx, fy], 1)
    if seed is not None:
        fr += _jitter(np.random.default_rng(seed), len(fr), dx)
    r = np.concatenate([np.stack([xs, ys], 1), fr])
    u = np.zeros_like(r)
    theta = np.concatenate([ths, ft])
    return Case(name=f"free_surface_periodic_{n}", r=r, u=u, theta=theta, npfb=len(r), nbS=len(xs), h=h, dx=dx,
                dv=dx * dx, Ra=1000.0, Pr=10.0, El=1.0, beta=0.1, body_force=(0.0, 0.0), ve_nonlinearity=400.0,
                i_open_domain=1, i_shift_coeff=1, b_node=b_node, b_edge=b_edge, b_type=b_type, b_vel=b_vel,
                b_thermal=b_th, b_periodic_parent=np.array([0, 4, 0, 2]))


def dam_break(m: int = 40, seed: int | None = None) -> Case:
    """Open-domain case: datclass case 1 "2 d dam break" (datclass.F90:47-117) -- a unit box
    with four no-slip walls, a water column x <= h0, y <= 2 h0 (h0 = 0.25) in the lower-left
    corner, gravity body force (0, -1), i_open_domain=1, shift_coeff=0, Newtonian (beta=1,
    El=0: const_mod 1), Ra=1e4, Pr=1, dx = h0/m (the generator's m = 40).  seed=None gives the
    unjittered lattice of the generator."""
    xl = yl = 1.0
    h0 = 0.25
    dx = h0 / m
    h = 1.3 * dx
    b_node = np.array([[0.0, 0.0], [xl, 0.0], [xl, yl], [0.0, yl]])
    b_edge = make_boundary_edge_vectors(b_node)
    b_type = np.array([1, 1, 1, 1])
    b_vel = np.zeros(4)
    b_th = np.zeros(4)
    xs, ys, us, vs, ths = make_boundary_particles(b_node, b_edge, b_type, b_vel, b_th, dx)
    fx, fy = [], []
    x = 0.0 + dx * 0.5
    while x < xl - 0.5 * dx:
        y = 0.0 + dx * 0.5
        while y < yl - 0.5 * dx:
            if x <= h0 and y <= 2.0 * h0:
                fx.append(x)
                fy.append(y)
            y = y + dx
        x = x + dx
    fr = np.stack([fx, fy], 1)
    if seed is not None:
        fr += _jitter(np.random.default_rng(seed), len(fr), dx)
    r = np.concatenate([np.stack([xs, ys], 1), fr])
    u = np.zeros_like(r)
    theta = np.concatenate([ths, np.zeros(len(fr))])
    return Case(name=f"dam_break_{m}", r=r, u=u, theta=theta, npfb=len(r), nbS=len(xs), h=h, dx=dx, dv=dx * dx,
                Ra=1.0e4, Pr=1.0, El=0.0, beta=1.0, body_force=(0.0, -1.0), ve_nonlinearity=100.0,
                i_open_domain=1, i_shift_coeff=0, const_mod=1, b_node=b_node, b_edge=b_edge, b_type=b_type,
                b_vel=b_vel, b_thermal=b_th, b_periodic_parent=np.array([3, 4, 1, 2]))


def by_name(name: str, **kw) -> Case:
    table = {
        "poiseuille_40": lambda: poiseuille(40, **kw),
        "poiseuille_1m": lambda: poiseuille(1000, **kw),
        "cylinder_4m": lambda: cylinder(4.0e6, **kw),
        "cavity_1m": lambda: cavity(1024, **kw),
        "rb_deck": rayleigh_benard_deck,
    }
    return table[name]()


def batch_sweep(n: int = 512, seed: int = 0, lo: float = 4.0e3, hi: float = 2.56e5):
    """The batched parameter sweep: n instances with fluid counts log-uniform in [lo, hi],
    Wi ~ U[0.1, 4.0], beta ~ U[0.1, 0.9] (seeded), alternating Poiseuille channel and cylinder
    geometry."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(lo), np.log(hi), size=n))
    wis = rng.uniform(0.1, 4.0, size=n)
    betas = rng.uniform(0.1, 0.9, size=n)
    out = []
    for k in range(n):
        if k % 2 == 0:
            m = max(8, int(round(math.sqrt(counts[k]))))
            out.append(poiseuille(m, seed=seed + k, Wi=float(wis[k]), beta=float(betas[k])))
        else:
            out.append(cylinder(float(counts[k]), Wi=float(wis[k]), beta=float(betas[k]), seed=seed + k))
    return out


def read_restart(path, const_mod: int = 2, theta: bool = True) -> dict:
    """Read a TEMP_REC.dat restart record (output.F90:59-77; reader input.F90:119-136).

    theta=True reads the particle lines as the reference writes them (theta included,
    output.F90:70); theta=False reads the opt-in layout without theta that the reference's
    reader expects (input.F90:123-126)."""
    with open(path) as f:
        head = [f.readline().split() for _ in range(3)]
        rest = f.read().split()
    itime, time, n_dump = int(head[0][0]), float(head[0][1]), int(head[0][2])
    np_, npfb, nbS, np_inflow = (int(v) for v in head[1][:4])
    box = [float(v) for v in head[2][:6]]
    per = (8 if theta else 7) + (4 if const_mod != 1 else 0)
    a = np.array(rest[: len(rest) - np_inflow], dtype=object).reshape(-1, per)
    f64 = lambda col: np.array([float(v) for v in a[:, col]])  # noqa: E731
    out = dict(itime=itime, time=time, n_dump=n_dump, np=np_, npfb=npfb, nbS=nbS, np_inflow=np_inflow,
               xb_min=box[0], xb_max=box[1], yb_min=box[2], yb_max=box[3], dx=box[4], av_conc=box[5])
    k = 0
    out["r"] = np.stack([f64(0), f64(1)], 1)
    out["u"] = np.stack([f64(2), f64(3)], 1)
    k = 4
    if theta:
        out["theta"] = f64(4)
        k = 5
    out["p"] = f64(k)
    out["dv"] = f64(k + 1)
    out["n_surf"] = np.array([int(v) for v in a[:, k + 2]])
    if const_mod != 1:  # tau_p(i,1,1), (1,2), (2,1), (2,2)
        out["tau"] = np.stack([f64(k + 3 + q) for q in range(4)], 1)
    return out
