"""lbmpsm_export_fields_static: the field export that allocates nothing.

A host program that keeps nearly all of HBM in its own pool allocator, or
that runs other streams on the GPU which cudaFree's device-wide wait would
stall, cannot let the library allocate in the middle of a run.  For those
callers the library exports the VTI fields through one fixed device array
instead of a per-call cudaMalloc.  These tests call that entry point through
the C ABI and hold it to the allocating lbmpsm_export_fields: both launch the
same kernel, so the outputs must be identical (the tolerance of the export
tests, which compare bit for bit).

The file is named to be collected last; each test builds its own lattices so
that it passes alone in a fresh process and after every other test.
"""
import ctypes as C

import numpy as np
import pytest

import cases
import lbmpsm

pytestmark = pytest.mark.gpu

MAX_BYTES = 64 * 1024 * 1024  # LBMPSM_EXPORT_STATIC_MAX_BYTES


def _npts(lat):
    nx, ny, nz = lat.local
    return (nx - 2) * (ny - 2) * ((nz - 2) if lat.dimension == 3 else 1)


def export_static(lat, B0, rho0, u0, as_double=True, fields=("solid", "rho", "u")):
    """Call lbmpsm_export_fields_static directly through the C ABI."""
    lib = lbmpsm.load()
    n = _npts(lat)
    dt = np.float64 if as_double else np.float32
    out = {"solid": np.full(n, np.nan, dt), "rho": np.full(n, np.nan, dt),
           "u": np.full((n, 3), np.nan, dt)}
    ptr = {k: (out[k].ctypes.data if k in fields else None) for k in out}
    code = lib.lbmpsm_export_fields_static(lat.h, int(as_double), C.c_double(B0),
                                           C.c_double(rho0), C.c_double(u0), ptr["solid"],
                                           ptr["rho"], ptr["u"])
    return code, out


def _advance(lat, case, state, steps, macro):
    tag, x, v, w, r = state
    for s in range(steps):
        g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
        if macro and s == steps - 1:
            lat.request_macro()
        lat.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        if case.bc:
            lat.apply_bc()
        x = cases.advance(case, x, v)
    return tag, x, v, w, r


@pytest.mark.parametrize("name", ["c2_sphere_3d", "channel_2d"])
def test_two_calls_in_a_row_equal_the_allocating_export(name):
    case = cases.CASES[name]
    lat = lbmpsm.Lattice(**case.params(), storage="fp64")
    if case.bc:
        lat.set_bc(case.bc)
    state = _advance(lat, case, cases.initial_particles(case), 4, macro=True)

    # first call: every field, double output
    code, got = export_static(lat, 1.0, 1000.0, 3.0, as_double=True)
    assert code == lbmpsm.OK, lat.lib.lbmpsm_last_error(lat.h)
    exp = lat.export_fields(1.0, 1000.0, 3.0, as_double=True)
    for k, e in zip(("solid", "rho", "u"), exp):
        assert np.array_equal(got[k], e), k
    assert np.any(exp[0] > 0) and np.any(exp[2] != 0)  # particles and flow present

    # second call straight after: the state has moved on and the request is
    # smaller (float, rho and u only), so it lands on the first call's bytes
    _advance(lat, case, state, 3, macro=True)
    code, got2 = export_static(lat, 2.0, 1.0, 0.5, as_double=False, fields=("rho", "u"))
    assert code == lbmpsm.OK, lat.lib.lbmpsm_last_error(lat.h)
    exp2 = lat.export_fields(2.0, 1.0, 0.5, as_double=False)
    assert np.array_equal(got2["rho"], exp2[1])
    assert np.array_equal(got2["u"], exp2[2])
    assert np.all(np.isnan(got2["solid"]))  # not requested, not written


def test_requests_beyond_the_fixed_array_are_rejected():
    # 1400 x 1400 nodes: all five double components need 78.4 MB > 64 MiB,
    # the float export 39.2 MB fits
    prd = (1400.0, 1400.0, 1.0)
    nu = 0.15 / 3
    lat = lbmpsm.Lattice(dimension=2, prd=prd, periodic=(1, 1, 1), Nlc=13, lc=12.0, nu=nu,
                         Re=0.01 * 12 / nu, tau=0.65, storage="fp32")
    n = _npts(lat)
    assert 40 * n > MAX_BYTES >= 20 * n
    code, _ = export_static(lat, 1.0, 1.0, 1.0, as_double=True)
    assert code == lbmpsm.ERR_CAPACITY
    msg = lat.lib.lbmpsm_last_error(lat.h).decode()
    assert "lbmpsm_export_fields_static" in msg and str(MAX_BYTES) in msg
    # the handle stays usable: the float export fits and equals the allocating one
    lat.step([], np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 3)), [])
    code, got = export_static(lat, 1.0, 1.0, 1.0, as_double=False)
    assert code == lbmpsm.OK, lat.lib.lbmpsm_last_error(lat.h)
    exp = lat.export_fields(1.0, 1.0, 1.0, as_double=False)
    for k, e in zip(("solid", "rho", "u"), exp):
        assert np.array_equal(got[k], e), k


def test_selected_box_of_an_ensemble_equals_the_allocating_export():
    # three periodic boxes of one geometry but different tau, force and
    # particles; each selected box (the last ones especially, whose planes
    # sit furthest from the start of the allocation) must export its own
    # fields, as lbmpsm_export_fields does
    edge = 16
    boxes, parts = [], []
    for b, (tau, fx) in enumerate([(0.7, 1e-6), (0.9, 6e-6), (0.62, 3e-6)]):
        nu = (tau - 0.5) / 3.0
        boxes.append(dict(dimension=3, boxlo=(0.0, 0.0, 0.0), prd=(float(edge),) * 3,
                          periodic=(1, 1, 1), Nlc=9, lc=8.0, rho=1.0, nu=nu, Re=0.01 * 8 / nu,
                          tau=tau, Fext=(fx, 0.0, 0.0)))
        rng = np.random.default_rng(300 + b)
        x, r = cases.rsa(rng, 1 + b, (4.0, 6.0), np.zeros(3) + 3.0, np.zeros(3) + edge - 3.0, 3,
                         min_gap=0.5)
        parts.append((np.arange(1, len(x) + 1, dtype=np.int32), x, r))
    ens = lbmpsm.Ensemble(boxes, storage="fp64")
    cols = {k: [] for k in ("box", "tag", "x", "r")}
    for b, (tag, x, r) in enumerate(parts):
        cols["box"].append(np.full(len(tag), b, np.int32))
        cols["tag"].append(tag)
        cols["x"].append(x)
        cols["r"].append(r)
    c = {k: np.concatenate(v) for k, v in cols.items()}
    z = np.zeros_like(c["x"])
    for s in range(6):
        if s == 5:
            ens.request_macro()
        ens.step(c["box"], c["tag"], c["x"], z, z, c["r"])
    seen = []
    for b in (2, 1, 0):
        ens.select_box(b)
        code, got = export_static(ens, 1.0, 1000.0, 3.0, as_double=True)
        assert code == lbmpsm.OK, ens.lib.lbmpsm_last_error(ens.h)
        exp = ens.export_fields(1.0, 1000.0, 3.0, as_double=True)
        for k, e in zip(("solid", "rho", "u"), exp):
            assert np.array_equal(got[k], e), (b, k)
        seen.append(got["u"].copy())
    # the boxes differ (tau, force, particles), so box selection is visible
    assert not np.array_equal(seen[0], seen[2])
