"""Host-side case set-up: meshes, velocity grids and parameters.

These play the part of the reference host's input handling (Creat_Mesh's
mesh file, Quadrature_Para.dat, control.in) for the planar-Couette
workloads; the solver itself only sees the arrays they produce.
"""
import math
from dataclasses import dataclass, field

import numpy as np

from . import hyb_types as T


def grid_nc(n, vdown, vup, rule=0):
    """Uniform Newton-Cotes velocity grid of n nodes on [vdown, vup].

    rule 0: composite Simpson 1/3 with a closing Simpson 3/8 panel when the
    interval count is odd (exact for cubics on every node count).
    rule 1: the reference's end/even/odd = 1/4/2 pattern times dv/3
    (Hybrid2D/src/GKUA_DETFP.f90:419-444), which is a valid Simpson rule
    only for an odd node count.
    """
    dv = (vup - vdown) / (n - 1)
    v = vdown + dv * np.arange(n, dtype=np.float64)
    w = np.zeros(n)
    if rule == 1:
        kk = np.arange(1, n + 1)
        c = np.where((kk == 1) | (kk == n), 1.0, np.where(kk % 2 == 0, 4.0, 2.0))
        return v, dv / 3.0 * c
    iv = n - 1
    simpson = iv if iv % 2 == 0 else iv - 3
    if simpson < 0:
        w[:] = dv / 2.0
        return v, w
    for p in range(0, simpson, 2):
        w[p] += dv / 3.0
        w[p + 1] += 4.0 * dv / 3.0
        w[p + 2] += dv / 3.0
    if simpson != iv:
        p = simpson
        w[p:p + 4] += np.array([3.0, 9.0, 9.0, 3.0]) * dv / 8.0
    return v, w


def grid_gl(dv, n, vdown, kgln, single_literals=True):
    """Composite Gauss-Legendre grid (GKUA_lisansudu.f90:94-196).

    The reference's node and weight table are REAL(4) literals
    (GKUA_lisansudu.f90:305-351); single_literals rounds the rule to float32
    the same way.  Returns nodes and full weights FBAV*w.
    """
    a, h = np.polynomial.legendre.leggauss(kgln)
    if single_literals:
        a = np.sign(a) * np.abs(a).astype(np.float32).astype(np.float64)
        h = h.astype(np.float32).astype(np.float64)
    v, w = [], []
    for iv in range(n):
        va, vb = vdown + iv * dv, vdown + (iv + 1) * dv
        vapb, vbma = (va + vb) / 2.0, (vb - va) / 2.0
        v.extend(vapb + vbma * a)
        w.extend(vbma * h)
    return np.array(v), np.array(w)


def half_range_hermite(n, m=600, vcut=12.0):
    """Nodes and weights of the n-point Gauss rule for integral_0^inf
    exp(-v^2) g(v) dv (the reference's "modified (half-range)
    Gauss-Hermite" rule, GKUA_lisansudu.f90:364-440, which tabulates n = 7, 8
    and 16).  Computed here from the weight function: the recurrence
    coefficients of its orthogonal polynomials by the discretised Stieltjes
    procedure on an m-point Gauss-Legendre discretisation of [0, vcut]
    (exp(-vcut^2) is below double precision), then the Golub-Welsch
    eigenvalue problem of the Jacobi matrix."""
    x, h = np.polynomial.legendre.leggauss(m)
    x = 0.5 * vcut * (x + 1.0)
    w = 0.5 * vcut * h * np.exp(-x * x)
    alpha, beta = np.zeros(n), np.zeros(n)
    p_prev, p = np.zeros(m), np.ones(m)
    norm_prev = 1.0
    for k in range(n):
        norm = np.sum(w * p * p)
        alpha[k] = np.sum(w * x * p * p) / norm
        beta[k] = norm if k == 0 else norm / norm_prev
        p_prev, p = p, (x - alpha[k]) * p - (beta[k] if k > 0 else 0.0) * p_prev
        norm_prev = norm
    J = np.diag(alpha) + np.diag(np.sqrt(beta[1:]), 1) + np.diag(np.sqrt(beta[1:]), -1)
    nodes, vec = np.linalg.eigh(J)
    weights = beta[0] * vec[0, :] ** 2
    return nodes, weights


def grid_gh(n2):
    """Gauss-Hermite velocity grid of n2 = 2n nodes (lisanv with
    Quadrature_Mode = GKUA_GH, GKUA_lisansudu.f90:102-115): the half-range
    nodes mirrored to negative velocities.  The returned weights are the
    ones the moments use, H exp(v^2) (IntegralGaussHermite,
    GKUA_DETFP.f90:174-201)."""
    if n2 % 2:
        raise ValueError("a Gauss-Hermite grid has an even node count")
    a, h = half_range_hermite(n2 // 2)
    v = np.concatenate([-a[::-1], a])
    w = np.concatenate([h[::-1], h]) * np.exp(v * v)
    return v, w


@dataclass
class Case:
    """One planar-Couette problem: everything hyb_create needs."""
    name: str
    ncx: int                 # cells in x
    ncy: int                 # cells in y
    nvx: int
    nvy: int
    vmax: float
    kn: float
    uw: float                # plate speed: bottom -uw, top +uw (units sqrt(2RT0))
    t_bottom: float = 1.0
    t_top: float = 1.0
    t_pert: float = 0.0      # T_w(x) = T(1 + t_pert sin(2 pi x / Lx)) on both plates
    lx: float = 1.0
    ly: float = 1.0
    dt: float = 1.0e3
    scheme: int = T.HYB_SCHEME_NND
    precision: int = T.HYB_PREC_FP64
    omega: float = 0.5       # viscosity exponent (hard sphere)
    pr: float = 2.0 / 3.0
    gamma: float = 5.0 / 3.0
    nc_rule: int = 1         # the reference NewtonCotes pattern (GKUA_DETFP.f90:419-444)
    quadrature: str = "nc"   # "nc": Newton-Cotes on [-vmax, vmax]; "gh": Gauss-Hermite (vmax unused)
    stretch: float = 0.0     # >0: tanh clustering of the y nodes towards both plates
    sweep_order: int = T.HYB_SWEEP_REFERENCE   # order of the kinetic implicit step
    mass_pin: int = 0        # 1: hold the total mass of f at its initial value
    # boundary kind of faces 1..4 (x low, y low, x high, y high); the Couette
    # channel is periodic in x with plates at the y faces.  Walls on the x
    # faces are at rest at t_bottom (face 1) and t_top (face 3)
    bcs: tuple = (T.HYB_BC_PERIODIC, T.HYB_BC_WALL, T.HYB_BC_PERIODIC, T.HYB_BC_WALL)
    extra: dict = field(default_factory=dict)

    # ---- derived arrays -------------------------------------------------
    @property
    def nx(self):
        return self.ncx + 1

    @property
    def ny(self):
        return self.ncy + 1

    @property
    def cells(self):
        return self.ncx * self.ncy

    @property
    def nv(self):
        return self.nvx * self.nvy

    def nodes(self):
        xs = np.linspace(0.0, self.lx, self.nx)
        eta = np.linspace(0.0, 1.0, self.ny)
        if self.stretch > 0.0:
            ys = self.ly * 0.5 * (1.0 + np.tanh(self.stretch * (2.0 * eta - 1.0)) / np.tanh(self.stretch))
        else:
            ys = self.ly * eta
        X, Y = np.meshgrid(xs, ys, indexing="ij")      # (nx, ny)
        return np.asfortranarray(X), np.asfortranarray(Y)

    def walls(self):
        """wall_u / wall_v / wall_t per face (faces 2 and 4 are the plates)."""
        xc = (np.arange(self.ncx) + 0.5) * self.lx / self.ncx
        pert = 1.0 + self.t_pert * np.sin(2.0 * math.pi * xc / self.lx)
        u = [None] * 4
        v = [None] * 4
        t = [None] * 4
        u[1] = np.full(self.ncx, -self.uw)
        u[3] = np.full(self.ncx, self.uw)
        v[1] = np.zeros(self.ncx)
        v[3] = np.zeros(self.ncx)
        t[1] = self.t_bottom * pert
        t[3] = self.t_top * pert
        for f, tw in ((0, self.t_bottom), (2, self.t_top)):
            u[f] = np.zeros(self.ncy)
            v[f] = np.zeros(self.ncy)
            t[f] = np.full(self.ncy, tw)
        return u, v, t

    def vgrid(self):
        if self.quadrature == "gh":
            vi, wi = grid_gh(self.nvx)
            vj, wj = grid_gh(self.nvy)
            return vi, wi, vj, wj
        vi, wi = grid_nc(self.nvx, -self.vmax, self.vmax, self.nc_rule)
        vj, wj = grid_nc(self.nvy, -self.vmax, self.vmax, self.nc_rule)
        return vi, wi, vj, wj

    def params(self):
        cfc = math.sqrt(math.pi) / (2.0 * self.kn)
        ma = math.sqrt(2.0 / self.gamma)
        p = T.HybParams()
        p.dt = self.dt
        p.cfc = cfc
        p.cpr = (1.0 - self.pr) / (5.0 / 2.0)
        p.x1s = 1.0 - self.omega
        p.r00 = 1.0
        p.t00 = 1.0
        p.scheme = self.scheme
        p.precision = self.precision
        p.gamma = self.gamma
        p.ma = ma
        p.pr = self.pr
        p.re = cfc * ma * math.sqrt(2.0 * self.gamma)
        p.omega_ns = self.omega
        p.device = 0
        p.sweep_order = self.sweep_order
        p.mass_pin = self.mass_pin
        return p

    def c_structs(self):
        """(mesh, vgrid, params, keepalive) ready for hyb_create/orc_create."""
        X, Y = self.nodes()
        x = np.ascontiguousarray(X.ravel(order="F"))
        y = np.ascontiguousarray(Y.ravel(order="F"))
        u, v, t = self.walls()
        vi, wi, vj, wj = self.vgrid()
        keep = [x, y, vi, wi, vj, wj]
        m = T.HybMesh()
        m.nx, m.ny = self.nx, self.ny
        m.x, m.y = T.dptr(x), T.dptr(y)
        bcs = list(self.bcs)
        for f in range(4):
            m.bc[f] = bcs[f]
            if bcs[f] == T.HYB_BC_WALL:
                arrs = [np.ascontiguousarray(a[f], dtype=np.float64) for a in (u, v, t)]
                keep.extend(arrs)
                m.wall_u[f], m.wall_v[f], m.wall_t[f] = (T.dptr(a) for a in arrs)
        g = T.HybVgrid()
        g.nvi, g.nvj = self.nvx, self.nvy
        g.vi, g.vj, g.wi, g.wj = T.dptr(vi), T.dptr(vj), T.dptr(wi), T.dptr(wj)
        return m, g, self.params(), keep


def couette_small(**kw):
    """Plain Couette, FP64, CPU-runnable: 4x64 cells, 32^2 NC on [-5,5],
    Kn=0.1, plates at +-0.2, T_w = 1."""
    args = dict(name="couette-4x64-nv32-kn0.1", ncx=4, ncy=64, nvx=32, nvy=32,
                vmax=5.0, kn=0.1, uw=0.2)
    args.update(kw)
    return Case(**args)


def couette_large(**kw):
    """Single large Couette: 128x512 cells, 64^2 on [-6,6], Kn=0.01,
    plates at +-0.5, T_w = 1.0 / 1.2, FP32 distribution."""
    args = dict(name="couette-128x512-nv64-kn0.01", ncx=128, ncy=512, nvx=64, nvy=64,
                vmax=6.0, kn=0.01, uw=0.5, t_bottom=1.0, t_top=1.2,
                precision=T.HYB_PREC_MIXED)
    args.update(kw)
    return Case(**args)


def couette_sine(**kw):
    """512x512 Couette with T_w = 1 + 0.1 sin(2 pi x), 48^2 on [-5,5],
    Kn=0.005, plates at +-0.3."""
    args = dict(name="couette-512x512-nv48-kn0.005-sine", ncx=512, ncy=512, nvx=48, nvy=48,
                vmax=5.0, kn=0.005, uw=0.3, t_pert=0.1, precision=T.HYB_PREC_MIXED)
    args.update(kw)
    return Case(**args)


def batch_manifest(n=256, seed=20261203):
    """Seeded instance list of the batched-Couette workload."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        ncy = int(rng.choice([32, 64, 128, 256]))
        nv = int(rng.choice([24, 32, 48, 64]))
        kn = float(10 ** rng.uniform(-3.0, 1.0))
        uw = float(rng.uniform(0.05, 0.8))
        tr = float(rng.uniform(0.8, 1.5))
        out.append(dict(name=f"batch-{k}", ncx=4, ncy=ncy, nvx=nv, nvy=nv, vmax=5.0 if nv < 48 else 6.0,
                        kn=kn, uw=uw, t_bottom=1.0, t_top=tr))
    return out
