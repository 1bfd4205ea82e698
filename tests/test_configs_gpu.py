"""The parity configurations at their full sizes.

* C1: D2Q9 256 x 256 periodic, tau 0.65, Guo force (1e-6, 0), one fixed disc
  of diameter 16 at the centre, plain FP64, 5000 steps: the GPU path against
  the CPU oracle after all 5000 steps (populations bit for bit -- no particle
  crosses a seam -- and the drag within 1e-12 relative).
* C2: D3Q19 128^3 periodic, tau 0.7, Guo force (1e-6, 0, 0), one fixed
  sphere of diameter 16 at the centre, 10^4 steps: FP64 against the oracle on
  the first steps, then FP32 and FP16 storage against FP64 after 10^4 steps on
  drag and on the velocity field.  Bounds: FP32 1e-3 relative drag (the
  target the FP32 path is built to), FP16 5e-2 (FP16 keeps 11 significant
  bits of the scaled deviations).
"""
import numpy as np
import pytest

import cases
import lbmpsm

pytestmark = pytest.mark.gpu

C1 = cases.Case("c1_full", 2, (256, 256, 1), (1, 1, 1), 0.65, (1e-6, 0.0, 0.0), 0, 5000,
                Nlc=17, diam=(16.0, 16.0), centres=[[128.0, 128.0, 0.0]])
C2 = cases.Case("c2_full", 3, (128, 128, 128), (1, 1, 1), 0.7, (1e-6, 0.0, 0.0), 0, 10000,
                Nlc=17, diam=(16.0, 16.0), centres=[[64.0, 64.0, 64.0]])


def _images(case):
    tag, x, v, w, r = cases.initial_particles(case)
    return cases.images(case, tag, x, v, w, r, cases.product_make_ghosts), len(tag)


def test_c1_full_size_5000_steps_bit_exact():
    g, nloc = _images(C1)
    gpu = lbmpsm.Lattice(**C1.params(), storage="fp64")
    orc = cases.OracleBackend(C1)
    fg = gpu.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
    gpu.run_fixed(C1.steps - 2)
    fg = gpu.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
    fo = None
    for _ in range(C1.steps):
        fo = orc.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
    drag_o = fo[0][:nloc]
    assert np.abs(drag_o).max() > 0
    assert np.abs(fg[0][:nloc] - drag_o).max() <= 1e-12 * np.abs(drag_o).max()
    m = gpu.stored_mask()
    assert np.array_equal(gpu.populations()[m], orc.sim.populations()[m])


def test_c2_full_size_oracle_parity_first_steps():
    g, nloc = _images(C2)
    gpu = lbmpsm.Lattice(**C2.params(), storage="fp64")
    orc = cases.OracleBackend(C2)
    for _ in range(3):
        a = gpu.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        b = orc.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
    assert np.abs(a[0] - b[0]).max() <= 1e-12 * np.abs(b[0]).max()
    ids_g, eps_g, _ = gpu.particle_table()
    ids_o, eps_o, _, _ = orc.sim.pdata()
    m = gpu.stored_mask()
    assert np.array_equal(ids_g[m], ids_o[m]) and np.array_equal(eps_g[m], eps_o[m])
    assert np.array_equal(gpu.populations()[m], orc.sim.populations()[m])


def _c2_run(storage):
    g, nloc = _images(C2)
    lat = lbmpsm.Lattice(**C2.params(), storage=storage)
    lat.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
    lat.run_fixed(C2.steps - 2)
    lat.request_macro()
    fh, th, _ = lat.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
    u = lat.export_fields(1.0, 1.0, 1.0)[2]
    mass, _ = lat.check()
    return fh[:nloc], u, mass


def test_c2_full_size_low_precision_against_fp64():
    f64, u64, m64 = _c2_run("fp64")
    assert f64[0, 0] > 0  # drag along the body force
    for storage, tol in (("fp32", 1e-3), ("fp16", 5e-2)):
        f, u, m = _c2_run(storage)
        drag = np.abs(f - f64).max() / np.abs(f64).max()
        vel = np.linalg.norm(u - u64) / np.linalg.norm(u64)
        assert drag <= tol, (storage, drag)
        assert vel <= tol, (storage, vel)
        assert abs(m - m64) <= tol * m64, (storage, m, m64)
