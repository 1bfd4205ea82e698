"""The collide autotuner (lbmpsm_options.collide_tuning, lbmpsm_info.collide_*).

Every candidate launch shape of the FP32/FP16 collide kernel -- the row
pipeline with 2, 3, 4 or 5 shared-memory stages, forced one at a time through
LBMPSM_PIPE_STAGES -- must give bit-identical populations and forces over a
run with moving particles and Zou-He walls, so the shape the tuner picks
changes speed only; the direct kernel (the fallback for long rows) agrees to
FP32 rounding.  The tuner runs at the start of the second step
(once the particle table is filled), must time every candidate that fits and
report the fastest as its choice; the default shape is taken untimed.
"""
import numpy as np
import pytest

import cases
import lbmpsm

pytestmark = pytest.mark.gpu


def _run(case, storage, steps, **kw):
    lat = lbmpsm.Lattice(**case.params(), storage=storage, **kw)
    if case.bc:
        lat.set_bc(case.bc)
    tag, x, v, w, r = cases.initial_particles(case)
    out = []
    for _ in range(steps):
        g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
        out.append(lat.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"]))
        if case.bc:
            lat.apply_bc()
        x = cases.advance(case, x, v)
    return lat, out


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("name", ["shear_3d", "shear_2d"])
def test_every_launch_shape_gives_the_same_results(name, storage, monkeypatch):
    case = cases.CASES[name]
    ref_pop = ref_out = None
    for stages in ("3", "2", "4", "5", "0"):
        monkeypatch.setenv("LBMPSM_PIPE_STAGES", stages)
        lat, out = _run(case, storage, 12)
        info = lat.get_info()
        assert info.collide_stages == int(stages), (stages, info.collide_stages)
        assert (info.collide_blocks > 0) == (stages != "0")
        pop = lat.populations()[lat.stored_mask()]
        if ref_pop is None:
            ref_pop, ref_out = pop, out
            continue
        if stages == "0":
            # the direct kernel (rows longer than a staged block) is not a
            # tuner candidate: the same node arithmetic inlined elsewhere may
            # contract multiply-adds differently, FP32 rounding apart
            scale = np.abs(ref_pop).max()
            tol = 1e-5 if storage == "fp32" else 1e-3
            assert np.abs(pop - ref_pop).max() <= tol * scale, (name, storage)
            continue
        assert np.array_equal(pop, ref_pop), (name, storage, stages)
        for a, b in zip(out, ref_out):
            for u, w in zip(a, b):
                assert np.array_equal(u, w), (name, storage, stages)
    monkeypatch.delenv("LBMPSM_PIPE_STAGES")
    lat, out = _run(case, storage, 12)
    assert np.array_equal(lat.populations()[lat.stored_mask()], ref_pop)


def test_tuner_times_the_candidates_and_keeps_the_fastest(monkeypatch):
    monkeypatch.delenv("LBMPSM_PIPE_STAGES", raising=False)
    case = cases.CASES["shear_3d"]
    lat, _ = _run(case, "fp32", 1)
    assert all(t == -1.0 for t in lat.get_info().collide_tune_ms)  # not before the 2nd step
    lat, _ = _run(case, "fp32", 3)
    info = lat.get_info()
    ms = list(info.collide_tune_ms)
    shapes = [3, 2, 4, 5]
    timed = [(t, s) for t, s in zip(ms, shapes) if t >= 0]
    assert len(timed) >= 2 and all(t > 0 for t, _ in timed)
    # the kept shape is one with the least time (ties keep the earlier candidate)
    assert ms[shapes.index(info.collide_stages)] == min(t for t, _ in timed)
    fixed = lbmpsm.Lattice(**case.params(), storage="fp32", collide_tuning="default")
    finfo = fixed.get_info()
    assert finfo.collide_stages == 3 and all(t == -1.0 for t in finfo.collide_tune_ms)
    f64 = lbmpsm.Lattice(**case.params(), storage="fp64").get_info()
    assert f64.collide_stages == -1
