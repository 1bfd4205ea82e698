"""Shared LBM-PSM parity cases: the same synthetic inputs drive the CPU oracle
(oracle/) and the GPU library, step by step, in the call order of the
reference fixes (lbm-psm post_force, then lbm-psm-bc post_force).

Most cases use lattice units (dx = 1, dt = 1): rho = 1, nu = (tau-1/2)/3,
lc = Nlc - 1 and Re = u_lb*lc/nu, which makes every unit factor 1 up to
rounding.  The cases with ``phys`` set run in SI units, as the reference's
own decks do (benchmark/in.lbmpsm_1:8-40: lc 0.0005 m, rho 1000 kg/m^3,
nu 1e-4 m^2/s, Re 0.1): lattice spacing lc/(Nlc-1), a non-zero box origin,
particle sizes, positions, velocities (m/s) and spins (rad/s) in physical
units, so that every unit factor of UnitConversion is exercised.  Particles
are placed by a seeded random sequential addition and moved by a prescribed
velocity each step, x += v*dt_move (the DEM integration is the host's job
and is not part of the path).
"""
from __future__ import annotations

import os
import sys
from dataclasses import dataclass, field

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "lammps-lbm-psm_gb300"))

BC_NAMES = {0: "none", 1: "shear", 2: "xFlow", 3: "channel", 4: "channel-velIn-pressOut", 5: "closedBox"}


@dataclass
class Case:
    name: str
    dim: int
    n: tuple            # interior node counts per axis (periodic) / node counts incl. walls
    periodic: tuple
    tau: float
    F: tuple            # lattice-unit body force
    bc: int
    steps: int
    u_lb: float = 0.01
    Nlc: int = 9
    nparts: int = 0
    diam: tuple = (6.0, 6.0)
    centres: list = field(default_factory=list)  # explicit centres (lattice units)
    vel: float = 0.0    # particle speed scale (lattice units per step)
    spin: float = 0.0
    seed: int = 0
    min_gap: float = 0.0
    cutghost: float = 0.0
    boxlo: tuple = (0.0, 0.0, 0.0)
    phys: dict = None     # SI units: lc, rho, nu, Re (F is then Fext in N/m^3)
    dt_move: float = 1.0  # time per step of the prescribed motion (SI cases: the DEM dt)

    @property
    def dx(self) -> float:
        """Lattice spacing lc/(Nlc-1) (exactly 1.0 for the lattice-unit cases)."""
        lc = self.phys["lc"] if self.phys else float(self.Nlc - 1)
        return lc / (self.Nlc - 1)

    def params(self) -> dict:
        if self.phys:
            lc, rho, nu, Re = (self.phys[k] for k in ("lc", "rho", "nu", "Re"))
        else:
            lc = float(self.Nlc - 1)
            rho = 1.0
            nu = (self.tau - 0.5) / 3.0
            Re = self.u_lb * lc / nu
        dx = self.dx
        prd = []
        for d in range(3):
            if d >= self.dim:
                prd.append(dx)
            else:
                # periodic: n nodes span n*dx; walls: n nodes span (n-1)*dx
                prd.append(self.n[d] * dx if self.periodic[d] else (self.n[d] - 1) * dx)
        # lattice units: volumeForceFactor is 1, so Fext = F_lbm
        return dict(dimension=self.dim, boxlo=self.boxlo, prd=tuple(prd), periodic=self.periodic,
                    nevery=1, Nlc=self.Nlc, lc=lc, rho=rho, nu=nu, Re=Re, tau=self.tau,
                    Fext=self.F)


def rsa(rng, n, diam_range, box_lo, box_hi, dim, min_gap=0.0, max_tries=200000):
    """Seeded random sequential addition of non-overlapping spheres/discs."""
    cs, rs = [], []
    tries = 0
    while len(cs) < n and tries < max_tries:
        tries += 1
        d = rng.uniform(*diam_range)
        r = d / 2
        c = rng.uniform(box_lo, box_hi)
        if dim == 2:
            c[2] = 0.0
        ok = True
        for c2, r2 in zip(cs, rs):
            if np.linalg.norm((c - c2)[:dim]) < r + r2 + min_gap:
                ok = False
                break
        if ok:
            cs.append(c)
            rs.append(r)
    return np.array(cs).reshape(-1, 3), np.array(rs)


def initial_particles(case: Case):
    rng = np.random.default_rng(case.seed)
    p = case.params()
    lo = np.array(case.boxlo, float)
    hi = lo + np.array(p["prd"])
    if case.centres:
        x = np.array(case.centres, float).reshape(-1, 3)
        r = np.full(len(x), case.diam[0] / 2)
    else:
        margin = np.zeros(3)
        for d in range(case.dim):
            if not case.periodic[d]:
                margin[d] = case.diam[1] / 2 + 2.0 * case.dx
        x, r = rsa(rng, case.nparts, case.diam, lo + margin, hi - margin, case.dim, case.min_gap)
    n = len(x)
    v = rng.normal(0.0, 1.0, (n, 3)) * case.vel
    w = rng.normal(0.0, 1.0, (n, 3)) * case.spin
    if case.dim == 2:
        v[:, 2] = 0.0
        w[:, :2] = 0.0
    for d in range(case.dim):
        if not case.periodic[d]:
            v[:, d] = 0.0
    tag = np.arange(1, n + 1, dtype=np.int32)
    return tag, x, v, w, r


def advance(case: Case, x, v):
    """Prescribed motion: x += v, wrapped into the box along periodic axes."""
    p = case.params()
    x = x + v * case.dt_move
    for d in range(case.dim):
        if case.periodic[d]:
            lo = case.boxlo[d]
            x[:, d] = lo + np.mod(x[:, d] - lo, p["prd"][d])
    return x


def cutghost(case: Case) -> float:
    return case.cutghost if case.cutghost > 0 else case.diam[1] / 2 + 3.0 * case.dx


def phys_dt(Nlc, lc, nu, Re, tau, nevery=1, rho=None):
    """The DEM timestep fix_LBM_PSM::init sets, phys_time(1)/nevery
    (src/fix_LBM_PSM.cpp:120, src/LBM_PSM_unitConversion.cpp:22-31)."""
    nu_lb = (tau - 0.5) * (1.0 / 3.0)
    Uc = Re * nu / lc
    u_lb = Re * nu_lb / (Nlc - 1)
    dt_d = (1.0 / (Nlc - 1)) * u_lb / 1.0
    return (1.0 * dt_d * (lc / Uc)) / nevery


# the reference's benchmark deck units (benchmark/in.lbmpsm_1:8-40), Nlc 11
PHYS_DECK = dict(lc=0.0005, rho=1000.0, nu=1e-4, Re=0.1)
# an air-like 2-D channel in SI units
PHYS_AIR = dict(lc=0.002, rho=1.2, nu=1.5e-5, Re=1.0)

CASES = {
    # C1 at reduced size: D2Q9 periodic, tau 0.65, Guo force, one fixed disc of D=16
    "c1_disc_2d": Case("c1_disc_2d", 2, (64, 64, 1), (1, 1, 1), 0.65, (1e-6, 0.0, 0.0), 0, 120,
                       Nlc=17, diam=(16.0, 16.0), centres=[[32.0, 32.0, 0.0]]),
    # C2 at reduced size: D3Q19 periodic, tau 0.7, one fixed sphere D=8 at the centre
    "c2_sphere_3d": Case("c2_sphere_3d", 3, (24, 24, 24), (1, 1, 1), 0.7, (1e-6, 0.0, 0.0), 0, 60,
                         Nlc=9, diam=(8.0, 8.0), centres=[[12.0, 12.0, 12.0]]),
    # C3 in miniature: y walls with Zou-He shear, moving/spinning spheres crossing x/z seams
    "shear_3d": Case("shear_3d", 3, (20, 16, 20), (1, 0, 1), 0.65, (0.0, 0.0, 0.0), 1, 40,
                     nparts=6, diam=(5.0, 7.0), vel=0.05, spin=0.01, seed=3, min_gap=0.5),
    # dense periodic packing: overlapping boxes, 3-particle nodes, seams, ghosts of ghosts
    "dense_periodic_3d": Case("dense_periodic_3d", 3, (14, 14, 14), (1, 1, 1), 0.8,
                              (2e-6, -1e-6, 5e-7), 0, 25, nparts=9, diam=(4.0, 6.0), vel=0.08,
                              spin=0.02, seed=11, min_gap=-1.0),
    # C4-like small box with an off-centre sphere
    "box_small_3d": Case("box_small_3d", 3, (16, 16, 16), (1, 1, 1), 0.9, (1e-5, 0.0, 0.0), 0, 30,
                         Nlc=9, diam=(8.0, 8.0), centres=[[6.3, 9.7, 8.1]]),
    # every 3-D keyword of fix lbm-psm-bc on a walled box
    "xflow_3d": Case("xflow_3d", 3, (12, 10, 10), (0, 0, 0), 0.7, (0.0, 0.0, 0.0), 2, 20,
                     nparts=1, diam=(4.0, 4.0), seed=5),
    "channel_3d": Case("channel_3d", 3, (12, 10, 12), (1, 0, 1), 0.7, (1e-5, 0.0, 0.0), 3, 20,
                       nparts=2, diam=(4.0, 4.0), seed=6, vel=0.03),
    "velin_pressout_3d": Case("velin_pressout_3d", 3, (12, 10, 10), (0, 0, 0), 0.7,
                              (0.0, 0.0, 0.0), 4, 20, nparts=1, diam=(4.0, 4.0), seed=7),
    "closedbox_3d": Case("closedbox_3d", 3, (10, 10, 10), (0, 0, 0), 0.7, (1e-5, 2e-6, 0.0), 5, 20,
                         nparts=1, diam=(4.0, 4.0), seed=8, spin=0.01),
    # a non-periodic axis without any BC fix (Stokes-drag deck layout p f p)
    "pfp_nobc_3d": Case("pfp_nobc_3d", 3, (14, 12, 14), (1, 0, 1), 0.7, (0.0, 0.0, 0.0), 0, 25,
                        nparts=1, diam=(6.0, 6.0), seed=9, vel=0.04),
    # 2-D keywords
    "shear_2d": Case("shear_2d", 2, (40, 24, 1), (1, 0, 1), 0.7, (0.0, 0.0, 0.0), 1, 50, nparts=4,
                     diam=(4.0, 8.0), seed=12, vel=0.05, spin=0.01),
    "xflow_2d": Case("xflow_2d", 2, (40, 24, 1), (0, 0, 1), 0.7, (0.0, 0.0, 0.0), 2, 50, nparts=2,
                     diam=(4.0, 6.0), seed=13),
    "channel_2d": Case("channel_2d", 2, (40, 24, 1), (1, 0, 1), 0.7, (1e-5, 0.0, 0.0), 3, 50,
                       nparts=3, diam=(4.0, 6.0), seed=14, vel=0.02),
    "velin_pressout_2d": Case("velin_pressout_2d", 2, (40, 24, 1), (0, 0, 1), 0.7,
                              (0.0, 0.0, 0.0), 4, 50, nparts=2, diam=(4.0, 6.0), seed=15),
    "closedbox_2d": Case("closedbox_2d", 2, (24, 24, 1), (0, 0, 1), 0.7, (1e-5, -1e-5, 0.0), 5, 50,
                         nparts=2, diam=(4.0, 6.0), seed=16, spin=0.01),
    "dense_periodic_2d": Case("dense_periodic_2d", 2, (30, 30, 1), (1, 1, 1), 0.6,
                              (1e-6, 1e-6, 0.0), 0, 40, nparts=10, diam=(4.0, 8.0), vel=0.1,
                              spin=0.02, seed=17, min_gap=-1.5),
    # SI units of the benchmark deck: dx = 5e-5 m, shear walls in y, origin off
    # zero, Fext in N/m^3 (F_lbm ~ 1e-6), spheres of 0.3-0.4 mm moving at ~1 m/s
    # (~0.03 lattice units per step) and spinning at ~6000 rad/s, crossing x/z seams
    "phys_shear_3d": Case("phys_shear_3d", 3, (24, 20, 24), (1, 0, 1), 0.7, (1.8e4, 0.0, -9e3),
                          1, 30, Nlc=11, nparts=4, diam=(3e-4, 4e-4), vel=1.0, spin=6000.0,
                          seed=21, min_gap=2.5e-5, boxlo=(-3.7e-4, 1.3e-4, 2.05e-3),
                          phys=PHYS_DECK, dt_move=phys_dt(11, **PHYS_DECK, tau=0.7)),
    # SI units in 2-D: channel walls, z origin ignored (origin[2] = 0 in 2-D)
    "phys_channel_2d": Case("phys_channel_2d", 2, (40, 24, 1), (1, 0, 1), 0.8, (3.5e-3, 1e-3, 0.0),
                            3, 40, Nlc=9, nparts=3, diam=(1e-3, 2e-3), vel=0.018, spin=24.0,
                            seed=22, min_gap=1e-4, boxlo=(0.31, -0.07, 0.5), phys=PHYS_AIR,
                            dt_move=phys_dt(9, **PHYS_AIR, tau=0.8)),
}

# cases whose particle boxes never reach a periodic seam: the whole state is
# bit-identical to the reference; seam cases differ only where the reference
# collides halo nodes with ghost-image data rounded differently from the twin
SEAM_FREE = {"c1_disc_2d", "c2_sphere_3d", "box_small_3d", "xflow_3d", "velin_pressout_3d",
             "closedbox_3d", "xflow_2d", "velin_pressout_2d", "closedbox_2d"}


def images(case: Case, tag, x, v, w, r, make_ghosts):
    """Particle images (locals then ghosts) for one step."""
    p = case.params()
    return make_ghosts(case.dim, p["boxlo"], p["prd"], p["periodic"], cutghost(case), tag, x, v, w, r)


def run(case: Case, backend, make_ghosts, steps=None, record_every=1):
    """Drive ``backend`` (an object with step(tag,x,v,w,r)->(fh,th,S) and
    apply_bc()) through the case; returns per-step outputs."""
    tag, x, v, w, r = initial_particles(case)
    steps = case.steps if steps is None else steps
    out = []
    for s in range(steps):
        g = images(case, tag, x, v, w, r, make_ghosts)
        fh, th, S = backend.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        if case.bc:
            backend.apply_bc()
        if s % record_every == 0 or s == steps - 1:
            out.append((s, g["tag"].copy(), fh.copy(), th.copy(), S.copy()))
        x = advance(case, x, v)
    return out


def oracle_make_ghosts(dim, boxlo, prd, periodic, cut, tag, x, v, w, r):
    import pyoracle
    return pyoracle.make_ghosts(dim, boxlo, prd, periodic, cut, tag, x, v, w, r)


def product_make_ghosts(dim, boxlo, prd, periodic, cut, tag, x, v, w, r):
    from lbmpsm.host import Domain, ghost_images
    lo = tuple(boxlo)
    hi = tuple(l + p for l, p in zip(lo, prd))
    a = ghost_images(Domain(dim, lo, hi, tuple(periodic)), cut, tag, x, v, w, r)
    return dict(tag=a.tag, x=a.x, v=a.v, omega=a.omega, radius=a.radius, owner=a.owner,
                swap=a.swap, nlocal=a.nlocal)


class OracleBackend:
    def __init__(self, case: Case, kind="restatement"):
        import pyoracle
        prm = case.params()
        prm["bc_type"] = case.bc
        self.sim = pyoracle.Sim(kind, **prm)

    def step(self, tag, x, v, w, r):
        return self.sim.step(tag, x, v, w, r)

    def apply_bc(self):
        self.sim.apply_bc()


class GpuBackend:
    def __init__(self, case: Case, storage="fp64", **kw):
        import lbmpsm
        self.lat = lbmpsm.Lattice(**case.params(), storage=storage, **kw)
        if case.bc:
            self.lat.set_bc(case.bc)

    def step(self, tag, x, v, w, r):
        return self.lat.step(tag, x, v, w, r)

    def apply_bc(self):
        self.lat.apply_bc()


def rel_err(a, b, floor=1e-300):
    """Max |a-b| relative to the largest |b| of the same quantity row-wise."""
    a = np.asarray(a, float); b = np.asarray(b, float)
    scale = np.maximum(np.abs(b).max(axis=-1, keepdims=True), floor)
    return float((np.abs(a - b) / scale).max()) if a.size else 0.0
