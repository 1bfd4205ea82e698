"""Adjoint and tangent sweeps of the time-averaged drag (lbmpsm_adjoint_drag,
lbmpsm_tangent_drag) through the C ABI.

Small cases, against the numpy restatement (oracle/adjoint_oracle.py, itself
pinned to the C oracle's finite differences by test_adjoint_oracle.py):
  * J to 1e-12 relative of the C oracle's steps (of the numpy forward for the
    Noble-Torczynski weighting, which the reference lacks), and the per-step
    drag and the final populations equal to plain lbmpsm_step calls;
  * dJ/dtau, dJ/dFext and dJ/dx per image row to 1e-9 relative;
  * the tangent to 1e-9 of the restatement's tangent and of the adjoint
    gradient projected on the same direction;
  * gradients bit-identical for every checkpoint spacing.
Covered: one sphere (3-D), two spheres across periodic seams moving and
spinning in place with Noble-Torczynski weighting, two discs (2-D).

The sensitivity configuration at full size (D3Q19 96^3 periodic, tau 0.7,
Fext (1e-6, 0, 0), 8 fixed spheres of diameter 12 by seeded random
sequential addition, J = x-drag averaged over steps 1000-2000, checkpoints
every 100 steps): dJ/dtau and dJ/dFx within 1e-4 relative of central finite
differences of lbmpsm_step runs (tau +- 1e-4 with nu moved along, Fx +- 1e-10),
the tangent within 1e-8 of the adjoint along tau, Fext and three centre
coordinates, the centre gradient within 5e-3 of central differences at
h = 1e-4 (their gap is the second-order response to the 1/1000 jumps of the
sub-cell counts; the first-order agreement is the restatement's test), and
the adjoint call at most 4x the wall time of the same steps run forward.

A thin torch.autograd.Function over the C ABI (harness only) returns the
same gradient through torch.autograd.grad.
"""
import time

import numpy as np
import pytest

import cases
import lbmpsm

pytestmark = pytest.mark.gpu

ao = pytest.importorskip("adjoint_oracle")

KEYS = ("tag", "x", "v", "omega", "radius")


def _imgs(case, parts, make_ghosts=cases.product_make_ghosts):
    tag, x, v, w, r = parts
    g = cases.images(case, tag, x, v, w, r, make_ghosts)
    return {k: g[k] for k in KEYS}, g


def _args(im):
    return [im[k] for k in KEYS]


def _rel(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


SMALL = dict(
    one_sphere=(cases.Case("adj1", 3, (20, 20, 20), (1, 1, 1), 0.7, (1e-5, 0.0, 0.0), 0, 40,
                           Nlc=9, diam=(8.0, 8.0), centres=[[9.3137, 10.6291, 8.8463]]),
                40, 20, 40, "reference", (1.0, 0.0, 0.0), 1e-4),
    seams_nt=(cases.Case("adj2", 3, (18, 16, 18), (1, 1, 1), 0.8, (4e-6, -2e-6, 1e-6), 0, 30,
                         Nlc=7, nparts=2, diam=(5.0, 7.0), vel=0.01, spin=0.004, seed=21,
                         min_gap=2.5),
              30, 6, 25, "noble-torczynski", (0.6, 0.8, 0.0), 1e-4),
    discs_2d=(cases.Case("adj3", 2, (48, 40, 1), (1, 1, 1), 0.65, (1e-5, 2e-6, 0.0), 0, 50,
                         Nlc=9, nparts=2, diam=(7.0, 9.0), seed=5, min_gap=3.0),
              50, 10, 50, "reference", (1.0, 0.0, 0.0), 2e-3),
)
# (case, nsteps, t0, t1, weighting, direction, centre step): a disc's perimeter
# holds ~100x fewer sub-cell centres per unit shift than a sphere's surface,
# so the 2-D case moves its discs further to see solid-fraction changes


@pytest.fixture(scope="module", params=list(SMALL))
def small(request):
    case, T, t0, t1, weighting, d, h = SMALL[request.param]
    parts = cases.initial_particles(case)
    im, g = _imgs(case, parts)
    P = ao.Problem(case.params(), im, T, t0, t1, direction=d, centre_step=h,
                   weighting=1 if weighting == "noble-torczynski" else 0)
    A = P.adjoint()
    gx = P.centre_gradient(A["sigma"])
    return request.param, case, T, t0, t1, weighting, d, h, im, P, A, gx


def test_adjoint_against_the_restatement(small):
    name, case, T, t0, t1, weighting, d, h, im, P, A, gx = small
    lat = lbmpsm.Lattice(**case.params(), storage="fp64", weighting=weighting)
    R = lat.adjoint_drag(*_args(im), T, t0, t1, direction=d, checkpoint_every=7, centre_step=h)
    if weighting == "reference":
        Jo = ao.oracle_J(case.params(), im, T, t0, t1, direction=d)
        assert abs(R["J"] - Jo) <= 1e-12 * abs(Jo), (name, R["J"], Jo)
    assert abs(R["J"] - A["J"]) <= 1e-12 * abs(A["J"]), (name, R["J"], A["J"])
    assert abs(R["dtau"] - A["dtau"]) <= 1e-9 * abs(A["dtau"]), (name, R["dtau"], A["dtau"])
    assert _rel(R["dFext"], A["dF"]) <= 1e-9, (name, R["dFext"], A["dF"])
    assert np.abs(gx).max() > 0
    assert _rel(R["dx"], gx) <= 1e-9, (name, R["dx"], gx)
    # the forward pass is the plain step sequence
    ref = lbmpsm.Lattice(**case.params(), storage="fp64", weighting=weighting)
    drag = [float((ref.step(*_args(im))[0] @ np.asarray(d)).sum()) for _ in range(T)]
    assert _rel(R["drag"], drag) <= 1e-13
    m = lat.stored_mask()
    assert np.array_equal(lat.populations()[m], ref.populations()[m])
    assert lat.steps == ref.steps == T


def test_tangent_against_the_restatement_and_the_adjoint(small):
    name, case, T, t0, t1, weighting, d, h, im, P, A, gx = small
    n = len(im["tag"])
    dx = np.tile((1.0, -0.5, 0.25), (n, 1))
    dF = (0.3, -1.0, 0.5)
    lat = lbmpsm.Lattice(**case.params(), storage="fp64", weighting=weighting)
    R = lat.adjoint_drag(*_args(im), T, t0, t1, direction=d, centre_step=h)
    for kw, num in ((dict(dtau=1.0), dict(dtau=1.0)), (dict(dFext=dF), dict(dF=dF)),
                    (dict(dx=dx), dict(dx_img=dx))):
        lt = lbmpsm.Lattice(**case.params(), storage="fp64", weighting=weighting)
        J, dJ = lt.tangent_drag(*_args(im), T, t0, t1, direction=d, centre_step=h, **kw)
        _, dJo = P.tangent(**num)
        adj = (R["dtau"] * kw.get("dtau", 0.0) + float(np.dot(R["dFext"], kw.get("dFext", (0, 0, 0))))
               + float((R["dx"] * kw["dx"]).sum() if "dx" in kw else 0.0))
        assert abs(J - R["J"]) <= 1e-14 * abs(R["J"])
        assert abs(dJ - dJo) <= 1e-9 * abs(dJo), (name, kw.keys(), dJ, dJo)
        assert abs(dJ - adj) <= 1e-9 * abs(adj), (name, kw.keys(), dJ, adj)


def test_checkpoint_spacing_does_not_change_the_gradient():
    case, T, t0, t1, weighting, d, h = SMALL["one_sphere"]
    im, _ = _imgs(case, cases.initial_particles(case))
    out = []
    for K in (1, 7, 40, 100):
        lat = lbmpsm.Lattice(**case.params(), storage="fp64")
        out.append(lat.adjoint_drag(*_args(im), T, t0, t1, checkpoint_every=K))
    for R in out[1:]:
        for k in ("J", "dtau"):
            assert R[k] == out[0][k]
        for k in ("dFext", "dx", "drag"):
            assert np.array_equal(R[k], out[0][k])


def test_rejected_configurations():
    case, T, t0, t1, weighting, d, h = SMALL["one_sphere"]
    im, _ = _imgs(case, cases.initial_particles(case))
    lat = lbmpsm.Lattice(**case.params(), storage="fp32")
    with pytest.raises(lbmpsm.LbmPsmError) as e:
        lat.adjoint_drag(*_args(im), T, t0, t1)
    assert e.value.code == lbmpsm.ERR_STATE
    lat = lbmpsm.Lattice(**case.params(), storage="fp64")
    for bad in ((T, 0, 5), (T, 5, 3), (T, 5, T + 1), (0, 1, 1)):
        with pytest.raises(lbmpsm.LbmPsmError) as e:
            lat.adjoint_drag(*_args(im), *bad)
        assert e.value.code == lbmpsm.ERR_ARG
    lat.set_bc("shear")
    with pytest.raises(lbmpsm.LbmPsmError) as e:
        lat.tangent_drag(*_args(im), T, t0, t1, dtau=1.0)
    assert e.value.code == lbmpsm.ERR_STATE
    walled = cases.CASES["channel_3d"]
    lat = lbmpsm.Lattice(**walled.params(), storage="fp64")
    with pytest.raises(lbmpsm.LbmPsmError) as e:
        lat.adjoint_drag(*_args(im), T, t0, t1)
    assert e.value.code == lbmpsm.ERR_STATE and "periodic" in str(e.value)
    assert lat.steps == 0  # nothing ran


# ------------------------------------------------------------------ full size
C5 = cases.Case("c5", 3, (96, 96, 96), (1, 1, 1), 0.7, (1e-6, 0.0, 0.0), 0, 2000, Nlc=13,
                nparts=8, diam=(12.0, 12.0), seed=2024, min_gap=2.0)
C5_T, C5_T0, C5_T1, C5_K = 2000, 1000, 2000, 100


def _c5_params(tau=0.7, Fx=1e-6):
    c = cases.Case("c5", 3, (96, 96, 96), (1, 1, 1), tau, (Fx, 0.0, 0.0), 0, 2000, Nlc=13)
    return c.params()


def _c5_J(im, **kw):
    lat = lbmpsm.Lattice(**_c5_params(**kw), storage="fp64")
    J = 0.0
    for t in range(1, C5_T + 1):
        fh = lat.step(*_args(im))[0]
        if t >= C5_T0:
            J += float(fh[:, 0].sum())
    return J / (C5_T1 - C5_T0 + 1)


def _owner_rows(g, rows):
    """ghost rows summed into their owners (reverse communication), local rows"""
    from lbmpsm.host import reverse_comm
    return reverse_comm(rows, g["owner"], g["swap"], g["nlocal"])[:g["nlocal"]]


def _c5_fd_centres(parts, h):
    """Central differences of J over every centre coordinate: the 48
    configurations (one coordinate moved by +h or -h) as the boxes of one
    ensemble, each box's J from its own images' forces."""
    tag, x, v, w, r = parts
    prm = C5.params()
    boxes, cols = [], {k: [] for k in ("box",) + KEYS}
    for p_ in range(len(tag)):
        for a in range(3):
            for sgn in (1, -1):
                xs = x.copy()
                xs[p_, a] += sgn * h
                ims, _ = _imgs(C5, (tag, xs, v, w, r))
                cols["box"].append(np.full(len(ims["tag"]), len(boxes), np.int32))
                for k in KEYS:
                    cols[k].append(ims[k])
                boxes.append(prm)
    cat = {k: np.concatenate(a_) for k, a_ in cols.items()}
    ens = lbmpsm.Ensemble(boxes, storage="fp64")
    J = np.zeros(len(boxes))
    for t in range(1, C5_T + 1):
        fh = ens.step(cat["box"], *[cat[k] for k in KEYS])[0]
        if t >= C5_T0:
            J += np.bincount(cat["box"], weights=fh[:, 0], minlength=len(boxes))
    ens.close()
    J /= (C5_T1 - C5_T0 + 1)
    return ((J[0::2] - J[1::2]) / (2 * h)).reshape(len(tag), 3)


def test_full_size_sensitivities():
    parts = cases.initial_particles(C5)
    assert len(parts[0]) == 8
    im, g = _imgs(C5, parts)
    lat = lbmpsm.Lattice(**C5.params(), storage="fp64")
    t = time.perf_counter()
    R = lat.adjoint_drag(*_args(im), C5_T, C5_T0, C5_T1, checkpoint_every=C5_K)
    t_adj = time.perf_counter() - t
    fwd = lbmpsm.Lattice(**C5.params(), storage="fp64")
    fwd.step(*_args(im))
    fwd.synchronize()
    t = time.perf_counter()
    fwd.run_fixed(C5_T - 1)
    fwd.synchronize()
    t_fwd = (time.perf_counter() - t) * C5_T / (C5_T - 1)
    assert t_adj <= 4.0 * t_fwd, (t_adj, t_fwd)

    J0 = _c5_J(im)
    assert abs(R["J"] - J0) <= 1e-12 * abs(J0)
    h = 1e-4
    fd_tau = (_c5_J(im, tau=0.7 + h) - _c5_J(im, tau=0.7 - h)) / (2 * h)
    assert abs(R["dtau"] - fd_tau) <= 1e-4 * abs(fd_tau), (R["dtau"], fd_tau)
    hF = 1e-10
    fd_F = (_c5_J(im, Fx=1e-6 + hF) - _c5_J(im, Fx=1e-6 - hF)) / (2 * hF)
    assert abs(R["dFext"][0] - fd_F) <= 1e-4 * abs(fd_F), (R["dFext"][0], fd_F)

    grad = _owner_rows(g, R["dx"])
    tag, x, v, w, r = parts
    # all 24 centre coordinates against central differences at h; the 48
    # perturbed configurations run together as one batched ensemble of boxes
    fd = _c5_fd_centres(parts, h)
    err = np.abs(grad - fd)
    scale = np.abs(fd).max()
    # J is a staircase in the centres (a node's solid fraction changes by
    # 1/1000 when a sub-cell centre crosses the surface): the adjoint's centre
    # derivative is the first-order response to the count changes a central
    # difference at h sees, so they differ by the second-order response to
    # those changes.  Measured at h = 1e-4: max 7.4e-4 and median 1.8e-4 of
    # the largest component; per component up to 2.3e-2 where a component is
    # fifty times below the largest.
    assert err.max() <= 2e-3 * scale, (err.max() / scale, err / scale)
    big = np.abs(fd) >= 0.1 * scale
    assert np.all(err[big] <= 5e-3 * np.abs(fd[big])), (err / np.abs(fd))
    for p_, a in ((0, 0), (3, 1), (6, 2)):
        # tangent along the same coordinate (every image of the particle moves)
        dx = np.zeros((len(im["tag"]), 3))
        dx[im["tag"] == tag[p_], a] = 1.0
        lt = lbmpsm.Lattice(**C5.params(), storage="fp64")
        _, dJ = lt.tangent_drag(*_args(im), C5_T, C5_T0, C5_T1, dx=dx)
        assert abs(dJ - grad[p_, a]) <= 1e-8 * abs(grad[p_, a]), (p_, a, dJ, grad[p_, a])
    for kw, ref in ((dict(dtau=1.0), R["dtau"]), (dict(dFext=(1.0, 0.0, 0.0)), R["dFext"][0])):
        lt = lbmpsm.Lattice(**C5.params(), storage="fp64")
        _, dJ = lt.tangent_drag(*_args(im), C5_T, C5_T0, C5_T1, **kw)
        assert abs(dJ - ref) <= 1e-8 * abs(ref), (kw, dJ, ref)


def test_torch_autograd_binding():
    torch = pytest.importorskip("torch")

    class TimeAveragedDrag(torch.autograd.Function):
        """J(tau, Fext, centres) through the C ABI; backward = the adjoint."""

        @staticmethod
        def forward(ctx, tau, fext, x, case, parts):
            prm = case.params()
            prm.update(tau=float(tau), nu=(float(tau) - 0.5) / 3.0,
                       Fext=tuple(float(f) for f in fext))
            prm["Re"] = case.u_lb * prm["lc"] / prm["nu"]
            tag, _, v, w, r = parts
            im, g = _imgs(case, (tag, x.detach().cpu().numpy(), v, w, r))
            lat = lbmpsm.Lattice(**prm, storage="fp64")
            R = lat.adjoint_drag(*_args(im), 40, 20, 40, checkpoint_every=10)
            ctx.grads = (R["dtau"], R["dFext"], _owner_rows(g, R["dx"]))
            return torch.tensor(R["J"], dtype=torch.float64)

        @staticmethod
        def backward(ctx, gJ):
            dtau, dF, dx = ctx.grads
            return (gJ * torch.tensor(dtau, dtype=torch.float64),
                    gJ * torch.tensor(dF, dtype=torch.float64),
                    gJ * torch.tensor(dx, dtype=torch.float64), None, None)

    case, T, t0, t1, weighting, d, h = SMALL["one_sphere"]
    parts = cases.initial_particles(case)
    tau = torch.tensor(0.7, dtype=torch.float64, requires_grad=True)
    fext = torch.tensor(case.F, dtype=torch.float64, requires_grad=True)
    x = torch.tensor(parts[1], dtype=torch.float64, requires_grad=True)
    J = TimeAveragedDrag.apply(tau, fext, x, case, parts)
    gt, gF, gx = torch.autograd.grad(J, (tau, fext, x))
    im, g = _imgs(case, parts)
    R = lbmpsm.Lattice(**case.params(), storage="fp64").adjoint_drag(*_args(im), T, t0, t1)
    assert float(J.detach()) == R["J"]
    assert float(gt) == R["dtau"]
    assert np.array_equal(gF.numpy(), R["dFext"])
    assert np.array_equal(gx.numpy(), _owner_rows(g, R["dx"]))
