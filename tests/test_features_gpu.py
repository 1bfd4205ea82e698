"""GPU behaviour around the coupling step: graph replay, field export,
state read/write, the global check, capacity growth and edge inputs.
Failures are injected on the host (bad inputs, NaN populations); no test
faults, traps or hangs the GPU."""
import numpy as np
import pytest

import cases
import lbmpsm

pytestmark = pytest.mark.gpu


def _lat(case, storage="fp64", **kw):
    lat = lbmpsm.Lattice(**case.params(), storage=storage, **kw)
    if case.bc:
        lat.set_bc(case.bc)
    return lat


@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_graph_replay_equals_eager_steps(storage):
    case = cases.CASES["shear_3d"]
    tag, x, v, w, r = cases.initial_particles(case)
    g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
    a = _lat(case, storage)
    b = _lat(case, storage)
    a.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"]); a.apply_bc()
    b.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"]); b.apply_bc()
    for _ in range(7):
        out_a = a.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"]); a.apply_bc()
    b.run_fixed(7)
    out_b = b.read_forces(len(g["tag"]))
    for u, v_ in zip(out_a, out_b):
        assert np.array_equal(u, v_)
    assert np.array_equal(a.populations(), b.populations())
    assert a.steps == b.steps == 8


def test_export_fields_match_oracle():
    case = cases.CASES["channel_2d"]
    lat = _lat(case)
    orc = cases.OracleBackend(case)
    tag, x, v, w, r = cases.initial_particles(case)
    s0 = lat.export_fields(1.0, 1000.0, 3.0)  # before any step: rho = 1, u = 0
    o0 = orc.sim.export_fields(1.0, 1000.0, 3.0)
    for p, q in zip(s0, o0):
        assert np.array_equal(p, q)
    for s in range(6):
        g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
        if s == 5:
            lat.request_macro()
        lat.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"]); lat.apply_bc()
        orc.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"]); orc.apply_bc()
        x = cases.advance(case, x, v)
    got = lat.export_fields(1.0, 1000.0, 3.0)
    exp = orc.sim.export_fields(1.0, 1000.0, 3.0)
    for p, q in zip(got, exp):
        assert np.array_equal(p, q)
    f32 = lat.export_fields(1.0, 1000.0, 3.0, as_double=False)
    assert f32[0].dtype == np.float32 and np.allclose(f32[1], exp[1], rtol=1e-6)


@pytest.mark.parametrize("storage", ["fp64", "fp32", "fp16", "bf16"])
def test_populations_roundtrip_and_mass_check(storage):
    case = cases.CASES["box_small_3d"]
    lat = _lat(case, storage)
    f0 = lat.populations()
    rng = np.random.default_rng(1)
    f1 = f0 * (1 + 1e-3 * rng.standard_normal(f0.shape))
    lat.set_populations(f1)
    back = lat.populations()
    m = lat.stored_mask()
    tol = {"fp64": 0.0, "fp32": 1e-8, "fp16": 1e-5, "bf16": 1e-5}[storage]
    assert np.abs(back[m] - f1[m]).max() <= tol
    mass0, _ = lat.check()
    for _ in range(5):
        lat.step([], np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 3)), [])
    mass1, _ = lat.check()
    assert abs(mass1 - mass0) <= {"fp64": 1e-9, "fp32": 1e-3, "fp16": 1e-1, "bf16": 1e-1}[storage] * 1e-3 * mass0


def test_nonfinite_population_is_reported():
    case = cases.CASES["box_small_3d"]
    lat = _lat(case)
    f = lat.populations()
    f[5, 5, 5, 3] = np.nan
    lat.set_populations(f)
    with pytest.raises(lbmpsm.LbmPsmError) as e:
        lat.check()
    assert e.value.code == lbmpsm.ERR_NUMERIC


def test_nonfinite_particle_input_rejected_on_host():
    case = cases.CASES["box_small_3d"]
    lat = _lat(case)
    with pytest.raises(lbmpsm.LbmPsmError) as e:
        lat.step([1], [[np.nan, 1.0, 1.0]], [[0, 0, 0]], [[0, 0, 0]], [2.0])
    assert e.value.code == lbmpsm.ERR_NUMERIC


def test_capacity_grows_for_many_images():
    case = cases.CASES["dense_periodic_3d"]
    lat = _lat(case, max_images=4)
    orc = cases.OracleBackend(case)
    tag, x, v, w, r = cases.initial_particles(case)
    g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
    assert len(g["tag"]) > 4
    a = lat.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
    b = orc.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
    assert np.abs(a[0] - b[0]).max() <= 1e-12 * np.abs(b[0]).max()


def test_particles_outside_the_lattice_give_zero_force():
    case = cases.CASES["box_small_3d"]
    lat = _lat(case)
    fh, th, S = lat.step([7, 8], [[-50.0, 3.0, 3.0], [3.0, 3.0, 400.0]], np.zeros((2, 3)),
                         np.zeros((2, 3)), [2.0, 3.0])
    assert not fh.any() and not th.any() and not S.any()


def test_step_device_matches_host_step():
    torch = pytest.importorskip("torch")
    case = cases.CASES["shear_3d"]
    tag, x, v, w, r = cases.initial_particles(case)
    g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
    n = len(g["tag"])
    a = _lat(case, max_radius=float(np.max(r)))
    b = _lat(case, max_radius=float(np.max(r)))
    ha = a.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
    dev = torch.device("cuda", 0)
    t = torch.as_tensor(g["tag"], dtype=torch.int32, device=dev)
    X = torch.as_tensor(g["x"], device=dev); V = torch.as_tensor(g["v"], device=dev)
    W = torch.as_tensor(g["omega"], device=dev); R = torch.as_tensor(g["radius"], device=dev)
    fh = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    th = torch.zeros_like(fh); S = torch.zeros((n, 6), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    b.step_device(n, t.data_ptr(), X.data_ptr(), V.data_ptr(), W.data_ptr(), R.data_ptr(),
                  fh.data_ptr(), th.data_ptr(), S.data_ptr())
    b.synchronize()
    assert np.array_equal(fh.cpu().numpy(), ha[0])
    assert np.array_equal(S.cpu().numpy(), ha[2])


def test_replayed_device_steps_take_each_calls_arrays():
    """lbmpsm_step_device replays a captured graph once the image count has
    held; every call's own input and output arrays must be the ones used.
    Every step passes freshly allocated device buffers of moving, spinning
    images; each step must equal the host-pointer step of the same images bit
    for bit, in the caller's output buffers and in the handle's own."""
    torch = pytest.importorskip("torch")
    case = cases.CASES["shear_3d"]
    tag, x, v, w, r = cases.initial_particles(case)
    a = _lat(case, max_radius=float(np.max(r)) + 0.5)
    b = _lat(case, max_radius=float(np.max(r)) + 0.5)
    dev = torch.device("cuda", 0)
    sets = []
    for s in range(14):  # a ghost image leaves after step 3: the graph is captured anew
        g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
        sets.append(g)
        x = cases.advance(case, x, v)
    assert len({len(g["tag"]) for g in sets}) > 1
    for s, g in enumerate(sets):
        n = len(g["tag"])
        ha = a.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        a.apply_bc()
        bb = {"out": [torch.full((n, 3), np.nan, dtype=torch.float64, device=dev),
                      torch.full((n, 3), np.nan, dtype=torch.float64, device=dev),
                      torch.full((n, 6), np.nan, dtype=torch.float64, device=dev)]}
        for key in ("tag", "x", "v", "omega", "radius"):
            bb[key] = torch.as_tensor(np.asarray(g[key], np.int32 if key == "tag" else np.float64),
                                      device=dev)
        torch.cuda.synchronize()
        b.step_device(n, bb["tag"].data_ptr(), bb["x"].data_ptr(), bb["v"].data_ptr(),
                      bb["omega"].data_ptr(), bb["radius"].data_ptr(),
                      *[o.data_ptr() for o in bb["out"]])
        b.apply_bc()
        b.synchronize()
        for got, exp in zip(bb["out"], ha):
            assert np.array_equal(got.cpu().numpy(), exp), s
        for got, exp in zip(b.read_forces(n), ha):
            assert np.array_equal(got, exp), s
    m = a.stored_mask()
    assert np.array_equal(a.populations()[m], b.populations()[m])


def test_fix_classes_drive_the_library(tmp_path):
    """The host mirror of the fixes runs the reference call order and writes VTI files."""
    from lbmpsm.host import Atoms, Domain, FixLbmPsm, FixLbmPsmBC, FixLbmPsmVTI, ghost_images
    dom = Domain(3, (0.0, 0.0, 0.0), (16.0, 15.0, 16.0), (1, 0, 1))
    nu = 0.2 / 3
    args = f"1 all lbm-psm every 1 Nlc 9 lc 8.0 rho 1.0 nu {nu!r} Re {0.01 * 8 / nu!r} tau 0.7".split()
    fix = FixLbmPsm(args)
    bcf = FixLbmPsmBC("2 all lbm-psm-bc shear".split(), fix)
    vti = FixLbmPsmVTI("3 all lbm-psm-vti every 2 binary 1".split(), fix, folder=str(tmp_path / "out"))
    dt = fix.init(dom)
    assert abs(dt - 1.0) < 1e-12
    bcf.init()
    vti.init()
    x = np.array([[8.0, 7.5, 8.0]])
    for step in range(1, 5):
        vti.pre_force(step)
        at = ghost_images(dom, 6.0, [1], x, np.zeros((1, 3)), np.zeros((1, 3)), [3.0])
        vti.before_lbm_step(step)
        fix.post_force(step, at)
        bcf.post_force(step)
        assert np.isfinite(at.f).all()
    files = sorted(p.name for p in (tmp_path / "out").iterdir())
    assert "flow_field.00000000.pvti" in files and "flow_field.00000000_rank0.vti" in files
    assert "flow_field.00000002_rank0.vti" in files and "flow_field.00000004_rank0.vti" in files
    assert "flow_field.00000003_rank0.vti" not in files


@pytest.mark.parametrize("name", ["dense_periodic_3d", "c2_sphere_3d", "dense_periodic_2d"])
def test_fp16_step_is_the_fp32_step_rounded(name):
    """FP16 storage runs the FP32 collision on deviations kept scaled by 2^12
    (the scale folded into the equilibrium weights): from one state, an FP16
    step must give the FP32 step's populations rounded to FP16, bit for bit,
    and the same forces.  Both lattices see the same images from the start,
    so that their two-slot tables share the same history."""
    case = cases.CASES[name]
    tag, x, v, w, r = cases.initial_particles(case)
    a = _lat(case, "fp16")
    b = _lat(case, "fp32")
    wq = b.populations().reshape(-1, b.q)[0].copy()  # at rest: f_q = w_q
    for _ in range(6):
        g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
        a.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        b.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        x = cases.advance(case, x, v)
    b.set_populations(a.populations())
    g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
    fa = a.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
    fb = b.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
    for p, q in zip(fa, fb):
        assert np.array_equal(p, q)
    pa, pb = a.populations(), b.populations()
    dev32 = (pb - wq).astype(np.float32)  # exact: the FP32 deviations
    assert np.array_equal((pb - wq), dev32.astype(np.float64))
    dev16 = (dev32 * np.float32(4096.0)).astype(np.float16).astype(np.float64) / 4096.0
    assert np.count_nonzero(pa != wq) > 0  # a developed state, not rest
    assert np.array_equal(pa, wq + dev16)


@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_host_steps_in_place_equal_staged_steps(storage, monkeypatch):
    """Host-pointer steps on a device that reads pageable host memory take
    the caller's arrays in place (gather kernel and reduction over
    NVLink-C2C); LBMPSM_HOST_STAGING=1 stages them through pinned copies.
    Both give the same forces and populations bit for bit, through the
    eager first steps and the replayed graphs, with the image count
    changing on the way; a non-finite position is still rejected."""
    case = cases.CASES["shear_3d"]
    tag, x, v, w, r = cases.initial_particles(case)
    a = _lat(case, storage)
    monkeypatch.setenv("LBMPSM_HOST_STAGING", "1")
    b = _lat(case, storage)
    monkeypatch.delenv("LBMPSM_HOST_STAGING")
    assert not b.host_direct
    buf = np.empty(12 * 64)  # one output array for every step of a (out=)
    for _ in range(9):
        g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
        assert 12 * len(g["tag"]) <= buf.size
        fa = a.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"], out=buf); a.apply_bc()
        fb = b.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"]); b.apply_bc()
        for p, q in zip(fa, fb):
            assert np.array_equal(p, q)
        x = cases.advance(case, x, v)
    assert np.array_equal(a.populations(), b.populations())
    # non-finite input: rejected on the host before any device work
    g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
    bad = np.array(g["x"], dtype=np.float64)
    bad[0, 0] = np.nan
    with pytest.raises(lbmpsm.LbmPsmError):
        a.step(g["tag"], bad, g["v"], g["omega"], g["radius"])
    with pytest.raises(ValueError):
        a.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"], out=np.empty(3))
