"""The C++ host side against the Python mirror of the fixes (lbmpsm.host).

The standalone driver (lammps-lbm-psm_gb300/lbmpsm_driver, built on the C++
fix classes of lammps-lbm-psm_gb300/host) runs a deck -- sheared suspension
with y walls (fix lbm-psm-bc shear), spheres moved by their hydrodynamic
force and torque (explicit DEM update), VTI output and restart writes -- and
the same call sequence is run through the Python classes.  Both hosts call
the same library with the same arrays, so the per-step forces and torques of
the owned atoms must agree bit for bit and the VTI and restart files byte
for byte.
"""
import math
import os
import subprocess

import numpy as np
import pytest

import cases
import lbmpsm  # noqa: F401
from lbmpsm.host import (Domain, FixLbmPsm, FixLbmPsmBC, FixLbmPsmRestart, FixLbmPsmVTI,
                         ghost_images, restart_file_name)

pytestmark = pytest.mark.gpu

DRIVER = os.path.join(cases.ROOT, "lammps-lbm-psm_gb300", "lbmpsm_driver")
CUT = 6.5


def _fix_args(nevery):
    return ["1", "all", "lbm-psm", "every", str(nevery), "Nlc", "9", "lc", "8.0", "rho", "1.0",
            "nu", repr(0.15 / 3), "Re", repr(0.01 * 8 / (0.15 / 3)), "tau", "0.65"]


BC = ["2", "all", "lbm-psm-bc", "shear"]
VTI = ["3", "all", "lbm-psm-vti", "every", "5", "binary", "1", "useDouble", "0"]
RST = ["4", "all", "lbm-psm-restart", "every", "10", "write", "1", "read", "0"]
BOX = (0.0, 20.0, 0.0, 15.0, 0.0, 20.0)


def _atoms():
    rng = np.random.default_rng(33)
    x, r = cases.rsa(rng, 5, (4.0, 6.0), np.array([0.0, 3.5, 0.0]), np.array([20.0, 11.5, 20.0]),
                     3, min_gap=1.0)
    n = len(x)
    v = rng.normal(0, 0.01, (n, 3))
    w = rng.normal(0, 0.005, (n, 3))
    dens = np.full(n, 2.5)
    return np.arange(1, n + 1), x, v, w, r, dens


def _dem(dom, dt, dens, x, v, w, r, f, t):
    """The driver's explicit update, same operations in the same order."""
    pi = 3.14159265358979323846
    for i in range(len(x)):
        m = dens[i] * 4.0 / 3.0 * pi * r[i] * r[i] * r[i]
        inertia = 0.4 * m * r[i] * r[i]
        for c in range(3):
            v[i, c] += dt * f[i, c] / m
            w[i, c] += dt * t[i, c] / inertia
            xc = x[i, c] + dt * v[i, c]
            if dom.periodic[c]:
                lo, L = dom.boxlo[c], dom.prd[c]
                xc = lo + math.fmod(math.fmod(xc - lo, L) + L, L)
            x[i, c] = xc


@pytest.mark.parametrize("nevery,STEPS", [(1, 12), (5, 23)])
def test_cpp_host_equals_python_host(tmp_path, nevery, STEPS):
    """every 1, and every 5 as in the reference's fluidised-bed example
    (examples/fluidisedBed-3D/in.lbmpsm:32): the four timesteps between
    coupling steps re-apply the stored forces (src/fix_LBM_PSM.cpp:183-196)
    and the DEM timestep is phys_time(1)/5 (src/fix_LBM_PSM.cpp:120)."""
    if not os.path.exists(DRIVER):
        pytest.skip("lbmpsm_driver not built")
    FIX = _fix_args(nevery)
    tag, x, v, w, r, dens = _atoms()
    cdir = tmp_path / "cpp"
    pdir = tmp_path / "py"
    cdir.mkdir()
    pdir.mkdir()
    with open(cdir / "atoms.txt", "w") as fh:
        for i in range(len(tag)):
            vals = [*x[i], *v[i], *w[i], r[i], dens[i]]
            fh.write(str(int(tag[i])) + " " + " ".join(repr(float(a)) for a in vals) + "\n")
    deck = ["dimension 3", "boundary p f p", "box " + " ".join(repr(b) for b in BOX),
            "atoms atoms.txt", f"cutghost {CUT!r}", "storage fp64", "fix " + " ".join(FIX),
            "fix " + " ".join(BC), "fix " + " ".join(VTI), "fix " + " ".join(RST), "dem nve",
            "output forces.txt", f"run {STEPS}"]
    (cdir / "deck.in").write_text("\n".join(deck) + "\n")
    res = subprocess.run([DRIVER, "deck.in"], cwd=cdir, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    cpp = {}
    step = None
    for line in (cdir / "forces.txt").read_text().splitlines():
        if line.startswith("step"):
            step = int(line.split()[1])
            cpp[step] = []
        else:
            cpp[step].append([float(s) for s in line.split()])

    # the same sequence through the Python classes
    dom = Domain(3, (BOX[0], BOX[2], BOX[4]), (BOX[1], BOX[3], BOX[5]), (1, 0, 1))
    fix = FixLbmPsm(FIX)
    bc = FixLbmPsmBC(BC, fix)
    vti = FixLbmPsmVTI(VTI, fix, folder=str(pdir / "flow_field_output_data"))
    rst = FixLbmPsmRestart(RST, fix, rank=0, folder=str(pdir))
    dt = fix.init(dom)
    bc.init()
    rst.init()
    vti.init()
    x, v, w = x.copy(), v.copy(), w.copy()
    for t in range(STEPS):
        a = ghost_images(dom, CUT, tag, x, v, w, r)
        vti.pre_force(t)
        rst.pre_force(t)
        vti.before_lbm_step(t)
        fix.post_force(t, a)
        bc.post_force(t)
        nl = a.nlocal
        py = np.concatenate([tag[:, None], a.f[:nl], a.torque[:nl]], axis=1)
        assert np.array_equal(np.array(cpp[t]), py), t
        assert np.abs(py[:, 1:4]).max() > 0  # the stored forces on the steps in between
        _dem(dom, dt, dens, x, v, w, r, a.f[:nl], a.torque[:nl])

    cv = sorted(os.listdir(cdir / "flow_field_output_data"))
    pv = sorted(os.listdir(pdir / "flow_field_output_data"))
    # every 5 steps: one piece and one master file each
    assert cv == pv and len(cv) == 2 * len(range(0, STEPS, 5))
    for name in cv:
        assert (cdir / "flow_field_output_data" / name).read_bytes() == \
            (pdir / "flow_field_output_data" / name).read_bytes(), name
    rname = restart_file_name(0)
    assert (cdir / rname).read_bytes() == (pdir / rname).read_bytes()
