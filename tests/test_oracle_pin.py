"""Pins the CPU oracle (plain-C restatement, oracle/lbmpsm_oracle.c):
  * bit-identical to the reference's own sources built here
    (oracle/_ref/libref_oracle.so) on every parity case, full state;
  * equal to the committed golden fixtures generated from the reference
    (tests/golden/reference_cases.npz) to 1e-12 relative;
  * known answers of the reference formulas and conservation properties.
"""
import os

import numpy as np
import pytest

import cases
import pyoracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_cases.npz")
have_ref = os.path.exists(pyoracle.REFERENCE_SO)


def _full_state(sim):
    f = sim.populations()
    ids, eps, us, F = sim.pdata()
    rho, u = sim.macro()
    return dict(f=f, ids=ids, eps=eps, us=us, F=F, rho=rho, u=u)


@pytest.mark.skipif(not have_ref, reason="reference sources not present (oracle/_ref not built)")
@pytest.mark.parametrize("name", list(cases.CASES))
def test_restatement_bit_identical_to_reference(name):
    case = cases.CASES[name]
    a = cases.OracleBackend(case, "restatement")
    b = cases.OracleBackend(case, "reference")
    ra = cases.run(case, a, cases.oracle_make_ghosts)
    rb = cases.run(case, b, cases.oracle_make_ghosts)
    for (sa, ta, fa, tha, Sa), (sb, tb, fb, thb, Sb) in zip(ra, rb):
        assert np.array_equal(ta, tb)
        assert np.array_equal(fa, fb) and np.array_equal(tha, thb) and np.array_equal(Sa, Sb), sa
    sa_, sb_ = _full_state(a.sim), _full_state(b.sim)
    for k in sa_:
        assert np.array_equal(sa_[k], sb_[k]), k
    ea = a.sim.export_fields(1.0, 1000.0, 2.5)
    eb = b.sim.export_fields(1.0, 1000.0, 2.5)
    for x, y in zip(ea, eb):
        assert np.array_equal(x, y)


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("name", list(cases.CASES))
def test_restatement_matches_golden(name, golden):
    case = cases.CASES[name]
    tag, x, v, w, r = cases.initial_particles(case)
    assert np.array_equal(x, golden[f"{name}/x0"]) and np.array_equal(r, golden[f"{name}/r0"])
    be = cases.OracleBackend(case, "restatement")
    rec = cases.run(case, be, cases.oracle_make_ghosts, record_every=5)
    assert [s for s, *_ in rec] == list(golden[f"{name}/steps"])
    fts = np.concatenate([np.concatenate([fh, th, S], axis=1) for _, _, fh, th, S in rec])
    tags = np.concatenate([t for _, t, *_ in rec])
    assert np.array_equal(tags, golden[f"{name}/tags"])
    ref = golden[f"{name}/fts"]
    for blk in (slice(0, 3), slice(3, 6), slice(6, 12)):
        assert cases.rel_err(fts[:, blk], ref[:, blk]) <= 1e-12
    f = be.sim.populations().reshape(-1, be.sim.q)
    np.testing.assert_allclose(f[golden[f"{name}/sample"]], golden[f"{name}/fpop"], rtol=1e-12, atol=0)
    ids, eps, us, _ = be.sim.pdata()
    occ = golden[f"{name}/occ"]
    assert np.array_equal(ids.reshape(-1, 2)[occ], golden[f"{name}/ids"])
    np.testing.assert_allclose(eps.reshape(-1, 2)[occ], golden[f"{name}/eps"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(us.reshape(-1, 6)[occ], golden[f"{name}/us"], rtol=1e-12, atol=1e-18)


def _sim(**kw):
    base = dict(dimension=3, prd=(8.0, 8.0, 8.0), periodic=(1, 1, 1), Nlc=9, lc=8.0,
                nu=0.2 / 3.0, Re=0.01 * 8 / (0.2 / 3.0), tau=0.7)
    base.update(kw)
    return pyoracle.Sim("restatement", **base)


def test_initial_state_is_rest_equilibrium():
    s = _sim()
    f = s.populations()
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    assert np.array_equal(f, np.broadcast_to(w, f.shape))
    rho, u = s.macro()
    assert np.all(rho == 1.0) and np.all(u == 0.0)


def test_solid_fraction_known_answers():
    """calcSolidFraction: full node inside, empty outside, and the exact
    sub-cell count of a node on the surface (1000 sub-cells in 3-D)."""
    s = _sim(prd=(16.0, 16.0, 16.0), lc=8.0)
    s.map([1], [[8.0, 8.0, 8.0]], [[0, 0, 0]], [[0, 0, 0]], [3.0])
    ids, eps, us, _ = s.pdata()
    # lattice-local centre is x + 1: node (9,9,9) is the centre, inside
    assert ids[9, 9, 9, 0] == 1 and eps[9, 9, 9, 0] == 1.0
    assert ids[9, 9, 1, 0] == 0 and eps[9, 9, 1, 0] == 0.0
    # node at distance exactly r along x: half the sub-cell centres lie inside
    # (planar approximation), counted exactly by the 10^3 sampling
    e = eps[12, 9, 9, 0]
    assert 0.4 < e < 0.6 and (e * 1000) == round(e * 1000)


def test_2d_solid_fraction_uses_dz_minus_one():
    """In 2-D the reference's node-centre distance keeps dz = 0 - (z/dx + 1) = -1
    for atoms at z = 0, which shifts its early-out tests; the oracle keeps it."""
    s = _sim(dimension=2, prd=(32.0, 32.0, 1.0), periodic=(1, 1, 1))
    r = 8.0
    # a node at in-plane distance 8.68 from the centre: partially covered
    # (8.68 < r + sqrt(2)/2) but sqrt(8.68^2 + 1) > r + sqrt(2.1)/2 -> 0
    s.map([1], [[16.0, 16.0, 0.0]], [[0, 0, 0]], [[0, 0, 0]], [r])
    ids, eps, _, _ = s.pdata()
    xl = 17.0
    for i in range(s.shape[0]):
        for j in range(s.shape[1]):
            d = np.hypot(i - xl, j - xl)
            if 8.62 < d < 8.7:
                assert eps[i, j, 0, 0] == 0.0


def test_periodic_fluid_conserves_mass_and_momentum():
    s = _sim(prd=(10.0, 10.0, 10.0))
    rng = np.random.default_rng(0)
    f = s.populations()
    f = f * (1.0 + 1e-3 * rng.standard_normal(f.shape))
    s.set_populations(f)
    ex = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0])
    inner = (slice(1, -1),) * 3
    m0 = s.populations()[inner].sum()
    p0 = (s.populations()[inner] * ex).sum()
    for _ in range(20):
        s.collide_stream()
    f1 = s.populations()[inner]
    assert abs(f1.sum() - m0) < 1e-12 * m0
    assert abs((f1 * ex).sum() - p0) < 1e-12 * m0


def test_guo_force_adds_momentum_per_step():
    """With a uniform body force F and no particles, total momentum grows by
    exactly N*F per step (Guo forcing, src/LBM_PSM_dynamics.h:89-116)."""
    F = 1e-5
    s = _sim(prd=(6.0, 6.0, 6.0), Fext=(F, 0.0, 0.0))
    ex = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0])
    inner = (slice(1, -1),) * 3
    vff = 1.0  # lattice units
    p = []
    for _ in range(4):
        s.collide_stream()
        p.append((s.populations()[inner] * ex).sum())
    d = np.diff(p)
    assert np.allclose(d, 216 * F * s.info.F_lbm[0] / F, rtol=1e-9)


def test_make_ghosts_matches_product_host_restatement():
    """The product's numpy ghost generator equals the oracle's on random atoms."""
    from lbmpsm.host import Domain, ghost_images, reverse_comm
    rng = np.random.default_rng(5)
    for dim, per in ((3, (1, 1, 1)), (3, (1, 0, 1)), (2, (1, 1, 1)), (2, (0, 1, 1))):
        n = 40
        lo = np.array([-2.0, 1.0, 0.5]); prd = np.array([10.0, 12.0, 9.0])
        if dim == 2:
            prd[2] = 1.0
        x = lo + rng.uniform(0, 1, (n, 3)) * prd
        if dim == 2:
            x[:, 2] = 0.0
        v = rng.normal(size=(n, 3)); w = rng.normal(size=(n, 3)); r = rng.uniform(0.5, 2, n)
        tag = np.arange(1, n + 1)
        g1 = pyoracle.make_ghosts(dim, lo, prd, per, 2.5, tag, x, v, w, r)
        g2 = ghost_images(Domain(dim, tuple(lo), tuple(lo + prd), per), 2.5, tag, x, v, w, r)
        for k in ("tag", "x", "v", "omega", "radius", "owner", "swap"):
            assert np.array_equal(g1[k], getattr(g2, k)), k
        vals = rng.normal(size=(len(g1["tag"]), 6))
        a = pyoracle.reverse_comm(vals, g1["owner"], g1["swap"], n)
        b = reverse_comm(vals, g2.owner, g2.swap, n)
        assert np.array_equal(a, b)


def test_reference_error_conditions():
    with pytest.raises(ValueError):  # tau <= 0.5
        _sim(tau=0.5)
    with pytest.raises(ValueError):  # Ma > 0.3
        _sim(Re=1e6)
    with pytest.raises(ValueError):  # domain not a multiple of dx
        _sim(prd=(8.5, 8.0, 8.0))
