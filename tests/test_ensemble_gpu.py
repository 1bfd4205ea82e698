"""Batched ensembles (lbmpsm_create_batch / lbmpsm_step_batch).

An ensemble of boxes with different tau, body force, origin and particles
must evolve exactly like the same boxes run as separate lattices: the same
kernels run on each box's planes with that box's parameters.  Checked bit
for bit on the per-image force / torque / stresslet of every step and on
each box's populations and particle table at the end, in FP64, FP32 and
FP16 and BF16 storage.
"""
import numpy as np
import pytest

import cases
import lbmpsm

pytestmark = pytest.mark.gpu

EDGE = 20


def _boxes():
    out = []
    for b, (tau, fx, lo) in enumerate([(0.7, 1e-6, 0.0), (0.9, 5e-6, 3.0), (0.62, 0.0, -2.5)]):
        nu = (tau - 0.5) / 3.0
        out.append(dict(dimension=3, boxlo=(lo, 2 * lo, -lo), prd=(float(EDGE),) * 3,
                        periodic=(1, 1, 1), Nlc=9, lc=8.0, rho=1.0, nu=nu, Re=0.01 * 8 / nu,
                        tau=tau, Fext=(fx, 0.3 * fx, 0.0)))
    return out


def _particles(b, box):
    rng = np.random.default_rng(100 + b)
    lo = np.array(box["boxlo"])
    x, r = cases.rsa(rng, 3 + b, (4.0, 7.0), lo, lo + EDGE, 3, min_gap=0.5)
    n = len(x)
    v = rng.normal(0, 0.02, (n, 3))
    w = rng.normal(0, 0.01, (n, 3)) if b == 1 else np.zeros((n, 3))
    return np.arange(1, n + 1, dtype=np.int32), x, v, w, r


def _images(box, tag, x, v, w, r):
    return cases.product_make_ghosts(3, box["boxlo"], box["prd"], box["periodic"], 7.0, tag, x, v,
                                     w, r)


@pytest.mark.parametrize("storage", ["fp64", "fp32", "fp16", "bf16"])
def test_ensemble_equals_separate_lattices(storage):
    boxes = _boxes()
    ens = lbmpsm.Ensemble(boxes, storage=storage)
    singles = [lbmpsm.Lattice(**b, storage=storage) for b in boxes]
    parts = [_particles(b, box) for b, box in enumerate(boxes)]
    for step in range(12):
        imgs = [_images(box, *pp) for box, pp in zip(boxes, parts)]
        out_s = [lat.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
                 for lat, g in zip(singles, imgs)]
        cat = {k: np.concatenate([g[k] for g in imgs]) for k in ("tag", "x", "v", "omega", "radius")}
        bidx = np.concatenate([np.full(len(g["tag"]), b, np.int32) for b, g in enumerate(imgs)])
        out_e = ens.step(bidx, cat["tag"], cat["x"], cat["v"], cat["omega"], cat["radius"])
        k = 0
        for b, g in enumerate(imgs):
            m = len(g["tag"])
            for a, s in zip(out_e, out_s[b]):
                assert np.array_equal(a[k:k + m], s), (storage, step, b)
            k += m
        # particles move and wrap within their own box
        for b, box in enumerate(boxes):
            tag, x, v, w, r = parts[b]
            lo = np.array(box["boxlo"])
            x = lo + np.mod(x + v - lo, EDGE)
            parts[b] = (tag, x, v, w, r)
    for b, lat in enumerate(singles):
        ens.select_box(b)
        m = lat.stored_mask()
        assert np.array_equal(ens.populations()[m], lat.populations()[m]), (storage, b)
        for a, s in zip(ens.particle_table(), lat.particle_table()):
            assert np.array_equal(a[m], s[m]), (storage, b)
    mass_e, _ = ens.check()
    assert np.isclose(mass_e, sum(lat.check()[0] for lat in singles), rtol=1e-12)


def test_ensemble_rejects_mixed_geometry_and_boundary_conditions():
    boxes = _boxes()
    boxes[1] = dict(boxes[1], prd=(float(EDGE), float(EDGE), float(EDGE + 4)))
    with pytest.raises(lbmpsm.LbmPsmError) as e:
        lbmpsm.Ensemble(boxes)
    assert e.value.code == lbmpsm.ERR_ARG and "box 1" in str(e.value)
    ens = lbmpsm.Ensemble(_boxes())
    with pytest.raises(lbmpsm.LbmPsmError) as e:
        ens.set_bc("shear")
    assert e.value.code == lbmpsm.ERR_STATE
    with pytest.raises(lbmpsm.LbmPsmError):
        ens.select_box(3)


def test_group_of_ensembles_of_different_sizes_equals_separate_runs():
    """Boxes of two sizes (an ensemble of 20^3 boxes, one of 16^3 boxes), a
    plain lattice and a sheared lattice (Zou-He faces) stepped as one group --
    one graph launch per step -- give the same populations and forces as each
    advanced on its own."""
    def make(edge, seed):
        boxes = []
        for b, tau in enumerate((0.7, 0.85)):
            nu = (tau - 0.5) / 3.0
            boxes.append(dict(dimension=3, prd=(float(edge),) * 3, periodic=(1, 1, 1), Nlc=9,
                              lc=8.0, rho=1.0, nu=nu, Re=0.01 * 8 / nu, tau=tau,
                              Fext=(2e-6 * (b + 1), 0.0, 0.0)))
        imgs, bidx = [], []
        for b, box in enumerate(boxes):
            rng = np.random.default_rng(seed + b)
            x, r = cases.rsa(rng, 2, (4.0, 6.0), np.zeros(3), np.full(3, float(edge)), 3,
                             min_gap=0.5)
            n = len(x)
            g = cases.product_make_ghosts(3, (0.0, 0.0, 0.0), box["prd"], (1, 1, 1), 6.0,
                                          np.arange(1, n + 1), x, np.zeros((n, 3)),
                                          np.zeros((n, 3)), r)
            imgs.append(g)
            bidx.append(np.full(len(g["tag"]), b, np.int32))
        cat = {k: np.concatenate([g[k] for g in imgs]) for k in ("tag", "x", "v", "omega", "radius")}
        return boxes, np.concatenate(bidx), cat

    def setup():
        members, nimg = [], []
        for edge, seed in ((20, 7), (16, 9)):
            boxes, bidx, cat = make(edge, seed)
            ens = lbmpsm.Ensemble(boxes, storage="fp32")
            ens.step(bidx, cat["tag"], cat["x"], cat["v"], cat["omega"], cat["radius"])
            members.append(ens)
            nimg.append(len(cat["tag"]))
        case = cases.CASES["c2_sphere_3d"]
        lat = lbmpsm.Lattice(**case.params(), storage="fp32")
        tag, x, v, w, r = cases.initial_particles(case)
        g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
        lat.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        members.append(lat)
        nimg.append(len(g["tag"]))
        case = cases.CASES["shear_3d"]
        lat = lbmpsm.Lattice(**case.params(), storage="fp32")
        lat.set_bc(case.bc)
        tag, x, v, w, r = cases.initial_particles(case)
        g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
        lat.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        lat.apply_bc()
        members.append(lat)
        nimg.append(len(g["tag"]))
        return members, nimg

    solo, nimg = setup()
    for m in solo:
        m.run_fixed(9)
    grouped, _ = setup()
    grp = lbmpsm.Group(grouped)
    grp.run_fixed(4)
    grp.run_fixed(5)
    grp.close()
    for a, b, n in zip(solo, grouped, nimg):
        assert a.steps == b.steps == 10
        fa, fb = a.read_forces(n), b.read_forces(n)
        assert np.abs(fa[0]).max() > 0
        for u, w in zip(fa, fb):
            assert np.array_equal(u, w)
        nb = getattr(a, "nbox", 1)
        for box in range(nb):
            if nb > 1:
                a.select_box(box)
                b.select_box(box)
            m = a.stored_mask()
            assert np.array_equal(a.populations()[m], b.populations()[m])
    # members at different step parities are rejected
    odd, _ = setup()
    odd[0].run_fixed(1)
    grp = lbmpsm.Group(odd)
    with pytest.raises(lbmpsm.LbmPsmError) as e:
        grp.run_fixed(1)
    assert e.value.code == lbmpsm.ERR_STATE
    grp.close()


def _periodic_members(storage, edges=((24, 2), (16, 3), (10, 2)), seed=40):
    """Ensembles of fully periodic boxes of several edges, every box with a
    body force and spheres; the first step through the host call."""
    members, nimg, specs = [], [], []
    for e_i, (edge, nbox) in enumerate(edges):
        boxes, imgs, bidx = [], [], []
        for b in range(nbox):
            tau = 0.62 + 0.11 * b + 0.05 * e_i
            nu = (tau - 0.5) / 3.0
            boxes.append(dict(dimension=3, boxlo=(0.5 * b, -0.25 * e_i, 0.0),
                              prd=(float(edge),) * 3, periodic=(1, 1, 1), Nlc=9, lc=8.0,
                              rho=1.0, nu=nu, Re=0.01 * 8 / nu, tau=tau,
                              Fext=(1e-6 * (1 + b), 5e-7 * e_i, 0.0)))
            rng = np.random.default_rng(seed + 10 * e_i + b)
            lo = np.array(boxes[-1]["boxlo"])
            x, r = cases.rsa(rng, 1 + b, (3.0, 4.5), lo, lo + edge, 3, min_gap=0.5)
            n = len(x)
            v = rng.normal(0, 0.01, (n, 3))
            g = cases.product_make_ghosts(3, tuple(lo), boxes[-1]["prd"], (1, 1, 1), 5.5,
                                          np.arange(1, n + 1), x, v, np.zeros((n, 3)), r)
            imgs.append(g)
            bidx.append(np.full(len(g["tag"]), b, np.int32))
        cat = {k: np.concatenate([g[k] for g in imgs]) for k in ("tag", "x", "v", "omega", "radius")}
        bi = np.concatenate(bidx)
        ens = lbmpsm.Ensemble(boxes, storage=storage)
        ens.step(bi, cat["tag"], cat["x"], cat["v"], cat["omega"], cat["radius"])
        members.append(ens)
        nimg.append(len(cat["tag"]))
        specs.append((boxes, imgs))
    return members, nimg, specs


@pytest.mark.parametrize("storage", ["fp64", "fp32", "fp16", "bf16"])
def test_one_collide_launch_for_boxes_of_every_size(storage, monkeypatch):
    """Periodic ensembles of edges 24, 16 and 10 (the row pipeline packs one,
    two and three x-rows per tile) stepped as one group whose collide is a
    single launch for all boxes: the same forces and populations, bit for
    bit, as each ensemble stepped on its own and as the group with one
    collide launch per member."""
    solo, nimg, _ = _periodic_members(storage)
    for m in solo:
        m.run_fixed(7)
    monkeypatch.setenv("LBMPSM_GROUP_FUSE", "0")
    sep, _, _ = _periodic_members(storage)
    g0 = lbmpsm.Group(sep)
    g0.run_fixed(7)
    assert g0.collide_launches == len(sep)
    g0.close()
    monkeypatch.delenv("LBMPSM_GROUP_FUSE")
    fused, _, _ = _periodic_members(storage)
    grp = lbmpsm.Group(fused)
    assert grp.collide_launches == -1
    grp.run_fixed(3)
    assert grp.collide_launches == 1
    grp.run_fixed(4)
    grp.close()
    for a, b, c, n in zip(solo, sep, fused, nimg):
        assert a.steps == b.steps == c.steps == 8
        fa = a.read_forces(n)
        assert np.abs(fa[0]).max() > 0
        for u, v_, w in zip(fa, b.read_forces(n), c.read_forces(n)):
            assert np.array_equal(u, w) and np.array_equal(v_, w), storage
        for box in range(a.nbox):
            for e in (a, b, c):
                e.select_box(box)
            m = a.stored_mask()
            pa = a.populations()[m]
            assert np.array_equal(pa, b.populations()[m]), (storage, box)
            assert np.array_equal(pa, c.populations()[m]), (storage, box)


def test_fused_group_fp64_against_oracle_per_box(monkeypatch):
    """The batched workload against the CPU oracle: boxes of three edges, each
    with its own tau, body force, origin and spheres, stepped as one fused
    group in FP64; every box's per-image force, torque and stresslet within
    1e-12 of a separate oracle lattice of that box, and its populations
    within 1e-13 (spheres that cross a periodic seam are collided by the
    reference on halo twins whose coordinates round differently)."""
    import pyoracle
    from test_parity_gpu import compare_fts
    monkeypatch.setenv("LBMPSM_GROUP_FUSE", "1")  # the one-launch plan, whatever the tuner would pick
    edges = ((14, 2), (12, 1), (10, 2))
    members, nimg, specs = _periodic_members("fp64", edges=edges, seed=60)
    steps = 9
    grp = lbmpsm.Group(members)
    grp.run_fixed(steps - 1)
    assert grp.collide_launches == 1
    grp.close()
    for ens, n, (boxes, imgs) in zip(members, nimg, specs):
        out = ens.read_forces(n)
        k = 0
        for b, (box, g) in enumerate(zip(boxes, imgs)):
            orc = pyoracle.Sim("restatement", **box, bc_type=0)
            a = (g["tag"], g["x"], g["v"], g["omega"], g["radius"])
            for _ in range(steps):
                fo = orc.step(*a)
            m = len(g["tag"])
            got = tuple(o[k:k + m] for o in out)
            k += m
            assert compare_fts(got, fo, g["radius"]) <= 1e-12, (b, box["prd"])
            ens.select_box(b)
            mask = ens.stored_mask()
            fg = ens.populations()[mask]
            fr = orc.populations()[mask]
            assert np.abs(fg - fr).max() <= 1e-13, (b, box["prd"])
            orc.close()


def test_group_tuner_keeps_the_results(monkeypatch):
    """The group's tuner times both collide plans on live steps of the first
    run of at least 8 steps and keeps the faster; the results stay those of
    the members' own steps, bit for bit."""
    monkeypatch.delenv("LBMPSM_GROUP_FUSE", raising=False)
    solo, nimg, _ = _periodic_members("fp32", seed=80)
    for m in solo:
        m.run_fixed(11)
    grouped, _, _ = _periodic_members("fp32", seed=80)
    grp = lbmpsm.Group(grouped)
    grp.run_fixed(11)
    per_member, one = grp.tune_ms
    assert per_member > 0 and one > 0
    assert grp.collide_launches == (1 if one <= per_member else len(grouped))
    grp.close()
    for a, b, n in zip(solo, grouped, nimg):
        assert a.steps == b.steps == 12
        for u, w in zip(a.read_forces(n), b.read_forces(n)):
            assert np.array_equal(u, w)
        for box in range(a.nbox):
            a.select_box(box)
            b.select_box(box)
            m = a.stored_mask()
            assert np.array_equal(a.populations()[m], b.populations()[m])
