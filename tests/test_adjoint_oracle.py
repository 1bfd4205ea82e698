"""The numpy restatement of the adjoint and tangent sweeps (oracle/adjoint_oracle.py)
pinned against the C oracle, on the CPU.

* its forward J equals the objective of the C oracle's own steps (map +
  collide + reduce) to 1e-12 relative: the closed-form step is the
  reference's step up to rounding;
* dJ/dtau and dJ/dFext equal central finite differences of the C oracle's J
  (tau +- 1e-4 with nu moved along so the unit factors stay 1; Fext +- 1e-9)
  to 1e-6 and 1e-4 relative (the cross-stream force components are small:
  their differences carry round-off of J);
* the centre gradient equals the derivative of J along the solid-fraction
  jumps of a +-h move, taken with those jumps scaled by s = 1e-3 (J is
  linear in them to that order) to 1e-4 relative; with the full jumps (s = 1,
  the plain finite difference) it differs by ~5e-4 relative here, the
  second-order response to the 1/1000 jumps of the sub-cell count, so the
  plain finite difference is held to 3e-3;
* the tangent along tau, Fext and a centre equals the adjoint gradient
  projected on that direction to 1e-10.
"""
import numpy as np
import pytest

import cases

ao = pytest.importorskip("adjoint_oracle")

T, T0, T1 = 40, 20, 40


def _case(tau=0.7, F=(1e-5, 0.0, 0.0), centres=((9.3137, 10.6291, 8.8463),)):
    return cases.Case("adj", 3, (20, 20, 20), (1, 1, 1), tau, F, 0, T, Nlc=9, diam=(8.0, 8.0),
                      centres=[list(c) for c in centres])


def _images(case, x=None):
    tag, x0, v, w, r = cases.initial_particles(case)
    x = x0 if x is None else x
    g = cases.images(case, tag, x, v, w, r, cases.oracle_make_ghosts)
    return {k: g[k] for k in ("tag", "x", "v", "omega", "radius")}, (tag, x0, v, w, r)


@pytest.fixture(scope="module")
def problem():
    case = _case()
    im, parts = _images(case)
    P = ao.Problem(case.params(), im, T, T0, T1)
    A = P.adjoint()
    return case, im, parts, P, A, P.centre_gradient(A["sigma"])


def test_forward_matches_the_c_oracle(problem):
    case, im, _, P, A, _ = problem
    Jo = ao.oracle_J(case.params(), im, T, T0, T1)
    assert abs(A["J"] - Jo) <= 1e-12 * abs(Jo)
    assert abs(P.forward() - Jo) <= 1e-12 * abs(Jo)


def test_tau_and_force_gradients_against_finite_differences(problem):
    case, im, _, P, A, _ = problem
    h = 1e-4
    fd = (ao.oracle_J(_case(tau=0.7 + h).params(), im, T, T0, T1) -
          ao.oracle_J(_case(tau=0.7 - h).params(), im, T, T0, T1)) / (2 * h)
    assert abs(A["dtau"] - fd) <= 1e-6 * abs(fd), (A["dtau"], fd)
    hF = 1e-9
    for a in range(3):
        Fp = [1e-5, 0.0, 0.0]
        Fm = [1e-5, 0.0, 0.0]
        Fp[a] += hF
        Fm[a] -= hF
        fd = (ao.oracle_J(_case(F=tuple(Fp)).params(), im, T, T0, T1) -
              ao.oracle_J(_case(F=tuple(Fm)).params(), im, T, T0, T1)) / (2 * hF)
        assert abs(A["dF"][a] - fd) <= 1e-4 * abs(fd), (a, A["dF"][a], fd)


def test_centre_gradient_against_linearised_and_plain_differences(problem):
    case, im, parts, P, A, gx = problem
    tag, x, v, w, r = parts
    h = P.h
    prm = case.params()
    for a in range(3):
        xp = x.copy()
        xm = x.copy()
        xp[0, a] += h
        xm[0, a] -= h
        ip, _ = _images(case, xp)
        imm, _ = _images(case, xm)
        Pp = ao.Problem(prm, ip, T, T0, T1)
        Pm = ao.Problem(prm, imm, T, T0, T1)
        assert np.array_equal(Pp.table[0], P.table[0]) and np.array_equal(Pm.table[0], P.table[0])
        e0 = P.table[1]
        Dp, Dm = Pp.table[1] - e0, Pm.table[1] - e0
        assert np.count_nonzero(Dp) and np.count_nonzero(Dm)
        s = 1e-3

        def J_with(eps):
            Q = ao.Problem(prm, im, T, T0, T1)
            Q.B = np.where(Q.table[0] > 0, eps, 0.0)
            return Q.forward()

        lin = (J_with(e0 + s * Dp) - J_with(e0 + s * Dm)) / (2 * h * s)
        adj = gx[:, a].sum()
        assert abs(adj - lin) <= 1e-4 * abs(lin), (a, adj, lin)
        fd = (ao.oracle_J(prm, ip, T, T0, T1) - ao.oracle_J(prm, imm, T, T0, T1)) / (2 * h)
        assert abs(adj - fd) <= 3e-3 * abs(fd), (a, adj, fd)


def test_tangent_equals_adjoint(problem):
    case, im, parts, P, A, gx = problem
    _, dJ = P.tangent(dtau=1.0)
    assert abs(dJ - A["dtau"]) <= 1e-10 * abs(A["dtau"])
    _, dJ = P.tangent(dF=(0.3, -1.0, 0.5))
    ref = float(np.dot(A["dF"], (0.3, -1.0, 0.5)))
    assert abs(dJ - ref) <= 1e-10 * abs(ref)
    dx = np.zeros((len(im["tag"]), 3))
    dx[:, :] = (1.0, -0.5, 0.25)  # every image of the particle moves alike
    _, dJ = P.tangent(dx_img=dx)
    ref = float((gx * dx).sum())
    assert abs(dJ - ref) <= 1e-10 * abs(ref)
