"""GPU parity: the CUDA path through the C-ABI against the CPU oracle.

FP64 storage keeps the reference arithmetic:
  * the particle table (ids, solid fractions, node velocities) must be
    bit-identical on every node the device stores;
  * populations must be bit-identical in cases whose particles stay away
    from periodic seams, and within 1e-13 absolute (populations are O(0.1))
    where the reference collides halo nodes with ghost-image coordinates
    that round differently from the interior twin;
  * per-image force, torque and stresslet within 1e-12 relative (the device
    sums node contributions in a fixed tree order, the reference
    sequentially); torque and stresslet relative to r_max*|F|_max.
FP32 / FP16 / BF16 storage: drag and torque within the tolerances stated below
against the FP64 device path.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

TOL_FTS = 1e-12
TOL_POP_SEAM = 1e-13


def fts_scales(fh, th, S, radius):
    # torque and stresslet are lever arm x force: their rounding scales with
    # the largest radius (in the case's own units) times the largest force
    sF = max(np.abs(fh).max(), 1e-300)
    rmax = float(np.max(radius))
    sT = max(np.abs(th).max(), rmax * sF)
    sS = max(np.abs(S).max(), rmax * sF)
    return sF, sT, sS


def compare_fts(a, b, radius):
    fa, ta, Sa = a
    fb, tb, Sb = b
    sF, sT, sS = fts_scales(fb, tb, Sb, radius)
    return max(np.abs(fa - fb).max() / sF, np.abs(ta - tb).max() / sT,
               np.abs(Sa - Sb).max() / sS)


def stored(gpu_lat):
    return gpu_lat.stored_mask()


@pytest.mark.parametrize("name", list(cases.CASES))
def test_fp64_step_by_step_against_oracle(name):
    case = cases.CASES[name]
    gpu = cases.GpuBackend(case, "fp64")
    orc = cases.OracleBackend(case, "restatement")
    tag, x, v, w, r = cases.initial_particles(case)
    worst = 0.0
    for s in range(case.steps):
        g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
        a = gpu.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        b = orc.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        if case.bc:
            gpu.apply_bc()
            orc.apply_bc()
        if len(g["tag"]):
            err = compare_fts(a, b, g["radius"])
            worst = max(worst, err)
            assert err <= TOL_FTS, (s, err)
        x = cases.advance(case, x, v)
    mask = stored(gpu.lat)
    ids_g, eps_g, us_g = gpu.lat.particle_table()
    ids_o, eps_o, us_o, _ = orc.sim.pdata()
    assert np.array_equal(ids_g[mask], ids_o[mask])
    assert np.array_equal(eps_g[mask], eps_o[mask])
    assert np.array_equal(us_g[mask], us_o[mask])
    fg = gpu.lat.populations()[mask]
    fo = orc.sim.populations()[mask]
    if name in cases.SEAM_FREE:
        assert np.array_equal(fg, fo), np.abs(fg - fo).max()
    else:
        assert np.abs(fg - fo).max() <= TOL_POP_SEAM, np.abs(fg - fo).max()


@pytest.fixture(scope="module")
def golden():
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_cases.npz"))


@pytest.mark.parametrize("name", ["c1_disc_2d", "c2_sphere_3d", "shear_3d", "dense_periodic_3d",
                                  "closedbox_3d", "xflow_2d", "phys_shear_3d", "phys_channel_2d"])
def test_fp64_against_reference_golden(name, golden):
    """Direct check against fixtures generated by the reference's own code."""
    case = cases.CASES[name]
    gpu = cases.GpuBackend(case, "fp64")
    rec = cases.run(case, gpu, cases.product_make_ghosts, record_every=5)
    fts = np.concatenate([np.concatenate([fh, th, S], axis=1) for _, _, fh, th, S in rec])
    ref = golden[f"{name}/fts"]
    assert fts.shape == ref.shape
    r = np.max(golden[f"{name}/r0"])
    sF = np.abs(ref[:, :3]).max()
    assert np.abs(fts[:, :3] - ref[:, :3]).max() <= TOL_FTS * sF
    assert np.abs(fts[:, 3:] - ref[:, 3:]).max() <= TOL_FTS * r * sF * 10
    f = gpu.lat.populations().reshape(-1, gpu.lat.q)
    np.testing.assert_allclose(f[golden[f"{name}/sample"]], golden[f"{name}/fpop"], rtol=1e-12, atol=0)


def _drag_run(case, storage, steps):
    gpu = cases.GpuBackend(case, storage)
    tag, x, v, w, r = cases.initial_particles(case)
    out = None
    for _ in range(steps):
        g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
        out = gpu.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        if case.bc:
            gpu.apply_bc()
        x = cases.advance(case, x, v)
    return out, gpu


@pytest.mark.parametrize("name,storage,tol", [
    ("c2_sphere_3d", "fp32", 1e-3), ("c1_disc_2d", "fp32", 1e-3), ("shear_3d", "fp32", 1e-3),
    ("closedbox_3d", "fp32", 1e-3), ("c2_sphere_3d", "fp16", 1e-1), ("shear_3d", "fp16", 1e-1),
    ("c2_sphere_3d", "bf16", 2e-1), ("shear_3d", "bf16", 2e-1),
])
def test_low_precision_storage_against_fp64(name, storage, tol):
    case = cases.CASES[name]
    ref, _ = _drag_run(case, "fp64", case.steps)
    got, lat = _drag_run(case, storage, case.steps)
    nl = len(cases.initial_particles(case)[0])
    F64, F = ref[0][:nl], got[0][:nl]
    rel = np.abs(F - F64).max() / np.abs(F64).max()
    assert rel <= tol, rel
    mass, mom = lat.lat.check()
    assert np.isfinite(mass)


@pytest.mark.parametrize("dim,seed", [(3, 0), (3, 1), (2, 2)])
def test_map_random_particles_bit_exact(dim, seed):
    """Many particles of random radius (0.3-9 lattice units, tiny ones exercise
    rM < 0) at random positions, mapped twice with motion in between: the
    particle table must equal the oracle's bit for bit on every stored node."""
    rng = np.random.default_rng(seed)
    n = 120 if dim == 3 else 60
    L = 40.0
    prd = (L, L, L if dim == 3 else 1.0)
    nu = 0.2 / 3
    params = dict(dimension=dim, boxlo=(0.0, 0.0, 0.0), prd=prd, periodic=(1, 1, 1), nevery=1,
                  Nlc=9, lc=8.0, rho=1.0, nu=nu, Re=0.01 * 8 / nu, tau=0.7, Fext=(0.0, 0.0, 0.0))
    import lbmpsm
    import pyoracle
    gpu = lbmpsm.Lattice(**params, storage="fp64")
    orc = pyoracle.Sim("restatement", **params)
    x = rng.uniform(0, L, (n, 3))
    if dim == 2:
        x[:, 2] = 0.0
    r = rng.uniform(0.3, 9.0, n)
    v = rng.normal(0, 1e-3, (n, 3)); w = rng.normal(0, 1e-3, (n, 3))
    tag = np.arange(1, n + 1)
    for _ in range(2):
        g = cases.product_make_ghosts(dim, (0.0, 0.0, 0.0), prd, (1, 1, 1), 12.0, tag, x, v, w, r)
        gpu.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        orc.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        x = x + rng.normal(0, 0.3, (n, 3)) * (np.arange(3) < dim)
        x[:, :dim] = np.mod(x[:, :dim], L)
    m = gpu.stored_mask()
    a = gpu.particle_table()
    b = orc.pdata()
    for k in range(3):
        assert np.array_equal(a[k][m], b[k][m]), k


@pytest.mark.parametrize("name", ["dense_periodic_3d", "dense_periodic_2d", "shear_3d"])
def test_fp32_table_is_the_fp64_table_rounded(name):
    """The FP32-storage map keeps only FP32 records (the collide kernel's
    input); they must hold the same particles in the same slots as the FP64
    table, with solid fractions equal to the FP32 roundings of the FP64 ones
    and node velocities equal to those roundings (images without spin) or
    within FP32 rounding of them (spinning images form the velocity in FP32).
    Dense packings: three particles at one node, dropped entries, slots
    cleared and refilled as particles move."""
    import lbmpsm
    case = cases.CASES[name]
    tag, x, v, w, r = cases.initial_particles(case)
    lats = {s: lbmpsm.Lattice(**case.params(), storage=s) for s in ("fp64", "fp32")}
    for lat in lats.values():
        if case.bc:
            lat.set_bc(case.bc)
    m = lats["fp64"].stored_mask()
    for step in range(min(case.steps, 12)):
        g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
        for lat in lats.values():
            lat.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
            if case.bc:
                lat.apply_bc()
        ids64, eps64, us64 = lats["fp64"].particle_table()
        ids32, eps32, us32 = lats["fp32"].particle_table()
        assert np.array_equal(ids32[m], ids64[m]), (name, step)
        assert np.array_equal(eps32[m], eps64[m].astype(np.float32).astype(np.float64)), (name, step)
        scale = max(np.abs(us64).max(), 1e-30)
        assert np.abs(us32[m] - us64[m]).max() <= 1e-6 * scale, (name, step)
        x = cases.advance(case, x, v)
