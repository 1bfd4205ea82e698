"""`fix lbm-psm every 5` in SI units, through the host fix classes, against the
oracle's restatement of the fix (pyoracle.FixOracle).

Two decks, each run for 23 DEM timesteps (coupling steps at 0, 5, 10, 15, 20):

* the fluidised-bed example's fix line (examples/fluidisedBed-3D/in.lbmpsm:32-41):
  `every 5 Nlc 6 lc 0.0125 rho 100 nu 0.005 Re 0.1 tau 0.65 Fext -981 0 0`
  with `lbm-psm-bc channel-velIn-pressOut`, walls on every side
  (`boundary f f f`), box origin off zero;
* the benchmark deck's units (benchmark/in.lbmpsm_1:8-40: Nlc 11, lc 0.0005,
  rho 1000, nu 1e-4, Re 0.1, tau 0.7) with `boundary p f p`, shear walls and
  spheres that cross the periodic x and z seams (ghost images, reverse
  communication).

Checked on every timestep: the force and torque the fix leaves on the owned
atoms (coupling steps: the step's F/T with the ghosts' rows summed in;
steps in between: the stored F/T of the local images re-applied,
src/fix_LBM_PSM.cpp:181-196) within 1e-12 relative, and the DEM timestep the
fix sets, phys_time(1)/nevery (src/fix_LBM_PSM.cpp:120), bit for bit.  The
spheres move by a prescribed velocity, x += v*dt, the same on both sides.
"""
import numpy as np
import pytest

import cases
import pyoracle
from lbmpsm.host import Domain, FixLbmPsm, FixLbmPsmBC, ghost_images

pytestmark = pytest.mark.gpu

STEPS = 23
TOL = 1e-12

DECKS = {
    "fluidised_bed_fff": dict(
        fix="every 5 Nlc 6 lc 0.0125 rho 100 nu 0.005 Re 0.1 tau 0.65 Fext -981.0 0.0 0.0",
        bc="channel-velIn-pressOut", periodic=(0, 0, 0), nodes=(20, 12, 12),
        boxlo=(0.0, -0.015, -0.015), nparts=3, diam=(0.009, 0.0125), speed=1.0, spin=100.0,
        seed=41),
    "benchmark_units_pfp": dict(
        fix="every 5 Nlc 11 lc 0.0005 rho 1000.0 nu 0.0001 Re 0.1 tau 0.7",
        bc="shear", periodic=(1, 0, 1), nodes=(22, 18, 22),
        boxlo=(-2.5e-4, 1.0e-4, 3.0e-4), nparts=4, diam=(3e-4, 4e-4), speed=1.5, spin=5000.0,
        seed=42),
}


def _setup(deck):
    args = ["1", "all", "lbm-psm", *deck["fix"].split()]
    fix = FixLbmPsm(args)
    p = fix.params
    dx = p["lc"] / (p["Nlc"] - 1)
    lo = np.array(deck["boxlo"])
    n = np.array(deck["nodes"])
    per = deck["periodic"]
    prd = np.array([n[d] * dx if per[d] else (n[d] - 1) * dx for d in range(3)])
    dom = Domain(3, tuple(lo), tuple(lo + prd), per)
    pyoracle_params = dict(dimension=3, boxlo=tuple(lo), prd=tuple(dom.prd), periodic=per,
                           nevery=fix.nevery, Nlc=p["Nlc"], lc=p["lc"], rho=p["rho"], nu=p["nu"],
                           Re=p["Re"], tau=p["tau"], Fext=p["Fext"],
                           bc_type=FixLbmPsmBC.KEYWORDS.index(deck["bc"]) + 1)
    rng = np.random.default_rng(deck["seed"])
    margin = np.array([0.0 if per[d] else deck["diam"][1] / 2 + 2 * dx for d in range(3)])
    x, r = cases.rsa(rng, deck["nparts"], deck["diam"], lo + margin, lo + prd - margin, 3,
                     min_gap=dx)
    m = len(x)
    v = rng.normal(0.0, deck["speed"], (m, 3))
    w = rng.normal(0.0, deck["spin"], (m, 3))
    for d in range(3):
        if not per[d]:
            v[:, d] *= 0.2  # slower towards the walls
    return fix, dom, pyoracle_params, np.arange(1, m + 1, dtype=np.int32), x, v, w, r, dx


@pytest.mark.parametrize("name", list(DECKS))
def test_every_5_host_fix_against_oracle_fix(name):
    deck = DECKS[name]
    fix, dom, oprm, tag, x, v, w, r, dx = _setup(deck)
    bc = FixLbmPsmBC(["2", "all", "lbm-psm-bc", deck["bc"]], fix)
    dt = fix.init(dom)
    bc.init()
    orc = pyoracle.FixOracle(**oprm)
    dt_o = orc.init()
    assert fix.nevery == 5
    assert dt == dt_o  # update->dt = phys_time(1)/nevery, bit for bit
    cut = deck["diam"][1] / 2 + 3 * dx
    crossed = False
    for t in range(STEPS):
        a = ghost_images(dom, cut, tag, x, v, w, r)
        g = pyoracle.make_ghosts(3, dom.boxlo, dom.prd, dom.periodic, cut, tag, x, v, w, r)
        assert np.array_equal(a.tag, g["tag"]) and np.array_equal(a.x, g["x"])
        crossed = crossed or len(a.tag) > len(tag)
        a.f[:] = 0.0
        a.torque[:] = 0.0
        fo = np.zeros((len(g["tag"]), 3))
        to = np.zeros((len(g["tag"]), 3))
        fix.post_force(t, a)
        bc.post_force(t)
        orc.post_force(t, g, fo, to)
        orc.apply_bc(t)
        nl = len(tag)
        sF = np.abs(fo[:nl]).max()
        sT = max(np.abs(to[:nl]).max(), r.max() * sF)
        assert sF > 0, t
        assert np.abs(a.f[:nl] - fo[:nl]).max() <= TOL * sF, t
        assert np.abs(a.torque[:nl] - to[:nl]).max() <= TOL * sT, t
        # prescribed motion over the DEM timestep, wrapped along periodic axes
        x = x + v * dt
        for d in range(3):
            if dom.periodic[d]:
                x[:, d] = dom.boxlo[d] + np.mod(x[:, d] - dom.boxlo[d], dom.prd[d])
    assert crossed or not any(deck["periodic"])
    orc.close()
    fix.lattice.close()
