"""Discrete adjoint and tangent of the FP64 collide-stream-PSM step, restated
in numpy (TEST INFRASTRUCTURE ONLY: the tests use it as the checker of the
library's adjoint and tangent sweeps; nothing in the product imports it).

The reference has no adjoint; what is differentiated is its forward step on
a fully periodic lattice with particles held in place:

* the particle table is set by ExchangeParticleData::setParticlesOnLattice
  (src/LBM_PSM_exchangeParticleData.cpp:24-112), taken here from the C
  oracle's map (``pyoracle.Sim.map``), and stays constant from step to step;
* one step is compute_macro_values + collisionAndStream
  (src/LBM_PSM_BGK_dynamics.cpp:48-109, src/LBM_PSM_BGK_dynamics.h:40-114)
  with feq / F_iq (src/LBM_PSM_dynamics.h:43-116), written in the closed form
  C_q = (1-w) f_q + (w - Bt) feq_q(rho,u) + sum_s B_s feq_q(rho,us_s) + (1-w/2) g_q(u)
  which equals the reference's per-direction update in exact arithmetic
  (Bt = B_1 + B_2, w = 1/tau, g_q the unscaled Guo term);
* the slot force of a node is -B_s sum_q Omega_s,q e_q (add_Fhyd,
  src/LBM_PSM_lattice.cpp:355-363) = B_s (m + (1-w) F/2 - rho us_s), and an
  image's hydrodynamic force sums the slot of its tag over its reduction box
  (calculateHydrodynamicInteractions, src/LBM_PSM_exchangeParticleData.cpp:172-244).

Objective: J = forceFactor/M * sum_{t=t0..t1} sum_images d . F_image(t) with
M = t1 - t0 + 1 and d a fixed direction (the time-averaged total drag along d).

Parameters: tau and the lattice body force F (unit factors held fixed), and
the particle centres.  The solid fraction of a node is a count of sub-cell
centres (calcSolidFraction, :116-169), piecewise constant in the centre; the
centre derivative is defined through the central difference of that count,
D eps = (eps(x + h e_a) - eps(x - h e_a)) / (2h), the same quantity a central
finite difference of J with step h sees to first order.
"""
from __future__ import annotations

import numpy as np

import pyoracle

D2Q9_E = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [-1, 0, 0], [0, -1, 0], [1, 1, 0],
                   [-1, 1, 0], [-1, -1, 0], [1, -1, 0]], dtype=np.int64)
D2Q9_W = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
# velocity order of src/LBM_PSM_lattice.h:198-209
D3Q19_E = np.array(
    list(zip([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0],
             [0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1],
             [0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1])), dtype=np.int64)
D3Q19_W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def velocity_set(dim):
    return (D2Q9_E, D2Q9_W) if dim == 2 else (D3Q19_E, D3Q19_W)


def solid_fraction(dim, node, xl, r):
    """calcSolidFraction (src/LBM_PSM_exchangeParticleData.cpp:116-169) of one
    node, same operations in the same order (FP64)."""
    slices = 10
    width = 1.0 / float(slices)
    fraction = 1.0 / float(slices ** 3 if dim == 3 else slices ** 2)
    h = np.sqrt(3.1) / 2.0 if dim == 3 else np.sqrt(2.1) / 2.0
    dx = float(node[0]) - xl[0]
    dy = float(node[1]) - xl[1]
    dz = float(node[2]) - xl[2]
    dist = dx * dx + dy * dy + dz * dz
    rP = r + h
    if dist > rP * rP:
        return 0.0
    rM = r - h
    if dist < rM * rM:
        return 1.0
    rSq = r * r
    delta = -0.5 + (np.arange(slices, dtype=np.float64) + 0.5) * width
    sx = (dx + delta) ** 2
    sy = (dy + delta) ** 2
    if dim == 2:
        n = int(np.count_nonzero(sx[:, None] + sy[None, :] < rSq))
    else:
        sz = (dz + delta) ** 2
        n = int(np.count_nonzero((sx[:, None, None] + sy[None, :, None]) + sz[None, None, :] < rSq))
    return fraction * float(n)


class Problem:
    """One fully periodic lattice, a fixed set of particle images and an
    objective window; holds the constant particle table and the per-node
    data the sweeps need (interior nodes only, arrays indexed [x, y, z])."""

    def __init__(self, params, images, nsteps, t0, t1, direction=(1.0, 0.0, 0.0),
                 centre_step=1e-4, weighting=0):
        if any(not p for p in params.get("periodic", (1, 1, 1))[: params.get("dimension", 3)]):
            raise ValueError("the adjoint restatement covers fully periodic lattices")
        self.params = dict(params)
        self.images = {k: np.array(images[k]) for k in ("tag", "x", "v", "omega", "radius")}
        self.images["x"] = self.images["x"].reshape(-1, 3)
        self.images["v"] = self.images["v"].reshape(-1, 3)
        self.images["omega"] = self.images["omega"].reshape(-1, 3)
        self.T, self.t0, self.t1 = int(nsteps), int(t0), int(t1)
        self.d = np.asarray(direction, dtype=np.float64)
        self.h = float(centre_step)
        self.weighting = int(weighting)
        sim = pyoracle.Sim(**self.params)
        self.sim = sim
        info = sim.info
        self.dim = params.get("dimension", 3)
        self.E, self.W = velocity_set(self.dim)
        self.Q = len(self.W)
        self.L = sim.shape
        self.dx = info.dx
        self.Uc, self.u_lb, self.tc, self.dt_d = info.Uc, info.u_lb, info.tc, info.dt_d
        self.forceFactor = info.forceFactor
        self.F = np.array([info.F_lbm[0], info.F_lbm[1], info.F_lbm[2]])
        self.tau = float(params.get("tau", 0.7))
        self.origin = np.array(params.get("boxlo", (0.0, 0.0, 0.0)), dtype=np.float64)
        if self.dim == 2:
            self.origin[2] = 0.0
        self.sl = (slice(1, -1), slice(1, -1), slice(1, -1) if self.dim == 3 else slice(0, 1))
        self.f0 = np.moveaxis(sim.populations()[self.sl], -1, 0).copy()
        self.table = self._table(self.images)
        self.shape = self.f0.shape[1:]
        self._entries()

    # ---------------------------------------------------------------- table
    def _table(self, im):
        sim = pyoracle.Sim(**self.params)
        sim.map(im["tag"], im["x"], im["v"], im["omega"], im["radius"])
        ids, eps, us, _ = sim.pdata()
        sim.close()
        return ids[self.sl].copy(), eps[self.sl].copy(), us[self.sl].copy()

    def local_centre(self, x):
        # src/LBM_PSM_exchangeParticleData.cpp:31-37 on one rank
        g = (np.asarray(x, dtype=np.float64) - self.origin) / self.dx
        return g - ((0 - (0.0 * 2.0 * 1.0)) - 1)

    def _zone(self, xl, r, reduce):
        z = []
        for d in range(3):
            a = int(xl[d] - r) - 2
            b = int(xl[d] + r) + 2
            if reduce:
                lo, hi = 1, self.L[d] - 1
                if d == 2 and self.dim == 2:
                    a, b = 0, 1
                else:
                    a, b = min(max(a, lo), hi), min(max(b, lo), hi)
            else:
                a, b = min(max(a, 0), self.L[d]), min(max(b, 0), self.L[d])
                if d == 2 and self.dim == 2:
                    a, b = 0, 1
            z.append((a, b))
        return z

    def _interior(self, i, j, k):
        """halo-frame node -> interior index, or None"""
        if not (1 <= i <= self.L[0] - 2 and 1 <= j <= self.L[1] - 2):
            return None
        if self.dim == 3:
            if not 1 <= k <= self.L[2] - 2:
                return None
            return (i - 1, j - 1, k - 1)
        return (i - 1, j - 1, 0)

    def node_velocity(self, i_img, node):
        im = self.images
        uT = im["v"][i_img] / self.Uc * self.u_lb
        om = im["omega"][i_img] * self.tc * self.dt_d
        xl = self.local_centre(im["x"][i_img])
        dx, dy, dz = node[0] - xl[0], node[1] - xl[1], node[2] - xl[2]
        return np.array([uT[0] + om[1] * dz - om[2] * dy, uT[1] + om[2] * dx - om[0] * dz,
                         uT[2] + om[0] * dy - om[1] * dx])

    def _entries(self):
        """Per node and slot: tag, solid velocity, count weight (number of
        images of that tag whose reduction box holds the node) and, in the
        surface shell of a particle, the slot an entering particle takes."""
        ids, eps, us = self.table
        X = self.shape
        self.tag = ids.astype(np.int64).copy()
        self.us = us.reshape(X + (2, 3)).copy()
        self.eps = eps.copy()
        self.cw = np.zeros(X + (2,), dtype=np.int64)
        self.band = np.zeros(X, dtype=bool)
        im = self.images
        h0 = np.sqrt(3.1) / 2.0 if self.dim == 3 else np.sqrt(2.1) / 2.0
        hl = self.h / self.dx
        seen = {}
        for i in range(len(im["tag"])):
            t = int(im["tag"][i])
            xl = self.local_centre(im["x"][i])
            r = im["radius"][i] / self.dx
            lo2, hi2 = (r - h0 - 2 * hl) ** 2, (r + h0 + 2 * hl) ** 2
            zone = self._zone(xl, r, reduce=False)
            for a in range(*zone[0]):
                for b in range(*zone[1]):
                    for c in range(*zone[2]):
                        n = self._interior(a, b, c)
                        if n is None:
                            continue
                        dist = (a - xl[0]) ** 2 + (b - xl[1]) ** 2 + (c - xl[2]) ** 2
                        if not lo2 <= dist <= hi2:
                            continue
                        self.band[n] = True
                        key = (n, t)
                        if key in seen:
                            raise ValueError("two images of one particle share a surface node")
                        seen[key] = i
                        if t in (self.tag[n][0], self.tag[n][1]) and eps_slot(self, n, t) > 0:
                            continue
                        # an entering particle takes the first empty slot
                        for s in range(2):
                            if self.tag[n][s] == 0:
                                self.tag[n][s] = t
                                self.us[n][s] = self.node_velocity(i, (a, b, c))
                                self.eps[n][s] = 0.0
                                break
                            if self.tag[n][s] == t:
                                break
                        else:
                            raise ValueError("a surface node of three particles")
        for i in range(len(im["tag"])):
            t = int(im["tag"][i])
            xl = self.local_centre(im["x"][i])
            r = im["radius"][i] / self.dx
            zone = self._zone(xl, r, reduce=True)
            for a in range(*zone[0]):
                for b in range(*zone[1]):
                    for c in range(*zone[2]):
                        n = self._interior(a, b, c)
                        if n is None:
                            continue
                        if self.tag[n][0] == t:
                            self.cw[n][0] += 1
                        elif self.tag[n][1] == t:
                            self.cw[n][1] += 1
        # weights B and their derivatives
        occ = ids > 0
        e = np.where(occ, eps, 0.0)
        tm = self.tau - 0.5
        if self.weighting == 1:
            b = e * tm / ((1.0 - e) + tm)
            db_de = tm * (1.0 + tm) / ((1.0 - e) + tm) ** 2
            db_dtau = e * (1.0 - e) / ((1.0 - e) + tm) ** 2
        else:
            b = e
            db_de = np.ones_like(e)
            db_dtau = np.zeros_like(e)
        # an entering particle (eps 0) has b = 0 and db/deps = db_de(0)
        sb = b.sum(axis=-1)
        ren = sb > 1.0
        B = np.where(ren[..., None], b / np.where(ren, sb, 1.0)[..., None], b)
        # dB_r/db_k
        J = np.zeros(X + (2, 2))
        for r_ in range(2):
            for k in range(2):
                J[..., r_, k] = np.where(ren, ((r_ == k) * sb - b[..., r_]) / np.where(ren, sb, 1.0) ** 2,
                                         float(r_ == k))
        self.B = B
        self.dB_deps = J * db_de[..., None, :]
        self.dB_dtau = np.einsum("...rk,...k->...r", J, db_dtau)

    # ------------------------------------------------------------- dynamics
    def _macro(self, f):
        E = self.E.astype(np.float64)
        rho = f.sum(axis=0)
        m = np.einsum("q...,qa->a...", f, E)
        return rho, m

    def _pieces(self, f, omega, F):
        E = self.E.astype(np.float64)
        W = self.W
        rho, m = self._macro(f)
        j = m + (F * 0.5)[:, None, None, None]
        u = j / rho
        eu = np.einsum("qa,a...->q...", E, u)
        usq = (u * u).sum(axis=0)
        Wb = W[:, None, None, None]
        feq = rho * Wb * (1.0 + 3.0 * eu + 4.5 * eu * eu - 1.5 * usq)
        eF = E @ F
        emuF = (E[:, :, None, None, None] - u[None]).transpose(0, 1, 2, 3, 4)
        g = Wb * (3.0 * np.einsum("qa...,a->q...", emuF, F) + 9.0 * eu * eF[:, None, None, None])
        fs = []
        for s in range(2):
            vs = np.moveaxis(self.us[..., s, :], -1, 0)
            evs = np.einsum("qa,a...->q...", E, vs)
            fs.append(rho * Wb * (1.0 + 3.0 * evs + 4.5 * evs * evs - 1.5 * (vs * vs).sum(axis=0)))
        return rho, m, j, u, eu, feq, g, fs

    def collide(self, f, omega, F):
        rho, m, j, u, eu, feq, g, fs = self._pieces(f, omega, F)
        B = self.B
        Bt = B.sum(axis=-1)
        C = (1.0 - omega) * f + (omega - Bt) * feq + B[..., 0] * fs[0] + B[..., 1] * fs[1] \
            + (1.0 - 0.5 * omega) * g
        drag = 0.0
        for s in range(2):
            vs = np.moveaxis(self.us[..., s, :], -1, 0)
            Fs = B[..., s] * (np.einsum("a,a...->...", self.d, m) + (1.0 - omega) * (self.d @ F) * 0.5
                              - rho * np.einsum("a,a...->...", self.d, vs))
            drag = drag + (self.cw[..., s] * Fs).sum()
        return C, drag

    def stream(self, C):
        out = np.empty_like(C)
        for q in range(self.Q):
            out[q] = np.roll(C[q], shift=tuple(self.E[q]), axis=(0, 1, 2))
        return out

    def pull(self, lam):
        out = np.empty_like(lam)
        for q in range(self.Q):
            out[q] = np.roll(lam[q], shift=tuple(-self.E[q]), axis=(0, 1, 2))
        return out

    def weight(self, t):
        M = self.t1 - self.t0 + 1
        return self.forceFactor / M if self.t0 <= t <= self.t1 else 0.0

    def forward(self, tau=None, F=None, keep=False):
        omega = 1.0 / (self.tau if tau is None else tau)
        F = self.F if F is None else np.asarray(F, dtype=np.float64)
        f = self.f0.copy()
        J = 0.0
        states = []
        for t in range(1, self.T + 1):
            if keep:
                states.append(f)
            C, drag = self.collide(f, omega, F)
            J += self.weight(t) * drag
            f = self.stream(C)
        return (J, states) if keep else J

    # -------------------------------------------------------------- adjoint
    def adjoint(self):
        """Reverse sweep: dJ/dtau, dJ/dF (lattice units) and, per node and
        slot, sigma = sum_t dJ/dB_s(t)."""
        J, states = self.forward(keep=True)
        omega = 1.0 / self.tau
        F = self.F
        E = self.E.astype(np.float64)
        W = self.W
        Wb = W[:, None, None, None]
        d = self.d
        B = self.B
        Bt = B.sum(axis=-1)
        gp = 1.0 - 0.5 * omega
        lam = np.zeros_like(self.f0)
        g_omega = 0.0
        g_tauB = 0.0
        g_F = np.zeros(3)
        sigma = np.zeros(self.shape + (2,))
        for t in range(self.T, 0, -1):
            f = states[t - 1]
            mu = self.pull(lam)
            c = self.weight(t)
            rho, m, j, u, eu, feq, g, fs = self._pieces(f, omega, F)
            usq = (u * u).sum(axis=0)
            # d feq_p / d rho (at fixed j) and d feq_p / d j_a
            dfeq_drho = Wb * (1.0 - 4.5 * eu * eu + 1.5 * usq)
            A_rho = (mu * dfeq_drho).sum(axis=0)
            A_j = np.stack([(mu * Wb * (3.0 * E[:, a, None, None, None] + 9.0 * eu * E[:, a, None, None, None]
                                          - 3.0 * u[a])).sum(axis=0) for a in range(3)])
            eF = E @ F
            A_u = gp * np.stack([(mu * Wb * (-3.0 * F[a] + 9.0 * E[:, a, None, None, None]
                                             * eF[:, None, None, None])).sum(axis=0) for a in range(3)])
            A_F = gp * np.stack([(mu * Wb * (3.0 * (E[:, a, None, None, None] - u[a])
                                             + 9.0 * eu * E[:, a, None, None, None])).sum(axis=0)
                                 for a in range(3)])
            A_s = [(mu * fs[s]).sum(axis=0) / rho for s in range(2)]
            ej = np.einsum("qa,a...->q...", E, A_j)
            eAu = np.einsum("qa,a...->q...", E, A_u)
            uAu = (A_u * u).sum(axis=0)
            new = (1.0 - omega) * mu + (omega - Bt) * (A_rho + ej) + B[..., 0] * A_s[0] \
                + B[..., 1] * A_s[1] + (eAu - uAu) / rho
            dm = np.einsum("a,a...->...", d, m)
            smf = (mu * feq).sum(axis=0)
            for s in range(2):
                vs = np.moveaxis(self.us[..., s, :], -1, 0)
                dvs = np.einsum("a,a...->...", d, vs)
                k = c * self.cw[..., s]
                new = new + k * B[..., s] * (np.einsum("a,qa->q", d, E)[:, None, None, None] - dvs)
                beta = (mu * fs[s]).sum(axis=0) - smf + k * (dm + (1.0 - omega) * (d @ F) * 0.5 - rho * dvs)
                sigma[..., s] += beta
                g_tauB += (beta * self.dB_dtau[..., s]).sum()
                g_omega += (k * B[..., s] * (-(d @ F) * 0.5)).sum()
                g_F += (k * B[..., s]).sum() * (1.0 - omega) * d * 0.5
            g_omega += (smf - (mu * f).sum(axis=0) - 0.5 * (mu * g).sum(axis=0)).sum()
            g_F += ((omega - Bt) * A_j * 0.5 + A_F + A_u / (2.0 * rho)).reshape(3, -1).sum(axis=1)
            lam = new
        dtau = -omega * omega * g_omega + g_tauB
        return dict(J=J, dtau=dtau, dF=g_F, sigma=sigma)

    # ---------------------------------------------------- centre derivative
    def eps_difference(self, i_img, axis):
        """(eps(x + h e_a) - eps(x - h e_a)) / (2h) over the map box of one
        image, as {interior node: value} (nodes where it is non-zero)."""
        im = self.images
        r = im["radius"][i_img] / self.dx
        out = {}
        xp = im["x"][i_img].copy()
        xm = im["x"][i_img].copy()
        xp[axis] += self.h
        xm[axis] -= self.h
        xlp, xlm = self.local_centre(xp), self.local_centre(xm)
        zone = self._zone(self.local_centre(im["x"][i_img]), r, reduce=False)
        for a in range(*zone[0]):
            for b in range(*zone[1]):
                for c in range(*zone[2]):
                    n = self._interior(a, b, c)
                    if n is None or not self.band[n]:
                        continue
                    de = solid_fraction(self.dim, (a, b, c), xlp, r) - \
                        solid_fraction(self.dim, (a, b, c), xlm, r)
                    if de != 0.0:
                        out[n] = de / (2.0 * self.h)
        return out

    def centre_gradient(self, sigma):
        """dJ/dx for every image row (ghost rows are summed into their owner
        by the caller, like forces)."""
        im = self.images
        out = np.zeros((len(im["tag"]), 3))
        for i in range(len(im["tag"])):
            t = int(im["tag"][i])
            for a in range(3):
                for n, de in self.eps_difference(i, a).items():
                    s = 0 if self.tag[n][0] == t else (1 if self.tag[n][1] == t else -1)
                    if s < 0:
                        continue
                    out[i, a] += de * float(np.dot(sigma[n], self.dB_deps[n][:, s]))
        return out

    def eps_dot(self, dx_img):
        """Solid-fraction tangent per node and slot for centre velocities
        dx_img (one row per image)."""
        im = self.images
        out = np.zeros(self.shape + (2,))
        for i in range(len(im["tag"])):
            t = int(im["tag"][i])
            for a in range(3):
                if dx_img[i, a] == 0.0:
                    continue
                for n, de in self.eps_difference(i, a).items():
                    s = 0 if self.tag[n][0] == t else (1 if self.tag[n][1] == t else -1)
                    if s >= 0:
                        out[n][s] += dx_img[i, a] * de
        return out

    # -------------------------------------------------------------- tangent
    def tangent(self, dtau=0.0, dF=(0.0, 0.0, 0.0), dx_img=None):
        """Forward-mode sweep: dJ along (dtau, dF, dx_img)."""
        omega = 1.0 / self.tau
        domega = -omega * omega * dtau
        F = self.F
        dF = np.asarray(dF, dtype=np.float64)
        E = self.E.astype(np.float64)
        W = self.W
        Wb = W[:, None, None, None]
        d = self.d
        B = self.B
        Bt = B.sum(axis=-1)
        gp = 1.0 - 0.5 * omega
        edot = self.eps_dot(dx_img) if dx_img is not None else np.zeros(self.shape + (2,))
        dB = np.einsum("...rk,...k->...r", self.dB_deps, edot) + self.dB_dtau * dtau
        dBt = dB.sum(axis=-1)
        f = self.f0.copy()
        fd = np.zeros_like(f)
        J = 0.0
        dJ = 0.0
        eF = E @ F
        edF = E @ dF
        for t in range(1, self.T + 1):
            c = self.weight(t)
            rho, m, j, u, eu, feq, g, fs = self._pieces(f, omega, F)
            usq = (u * u).sum(axis=0)
            rhod = fd.sum(axis=0)
            md = np.einsum("q...,qa->a...", fd, E)
            jd = md + (dF * 0.5)[:, None, None, None]
            ud = (jd - u * rhod) / rho
            feqd = Wb * (rhod * (1.0 - 4.5 * eu * eu + 1.5 * usq)
                         + np.einsum("qa...,a...->q...",
                                     3.0 * E[:, :, None, None, None] + 9.0 * eu[:, None] * E[:, :, None, None, None]
                                     - 3.0 * u[None], jd))
            gd = Wb * (np.einsum("qa...,a...->q...",
                                 -3.0 * F[None, :, None, None, None]
                                 + 9.0 * E[:, :, None, None, None] * eF[:, None, None, None, None], ud)
                       + np.einsum("qa...,a->q...",
                                   3.0 * (E[:, :, None, None, None] - u[None])
                                   + 9.0 * eu[:, None] * E[:, :, None, None, None], dF))
            Cd = (1.0 - omega) * fd - domega * f + (domega - dBt) * feq + (omega - Bt) * feqd \
                - 0.5 * domega * g + gp * gd
            dm = np.einsum("a,a...->...", d, m)
            dmd = np.einsum("a,a...->...", d, md)
            drag = 0.0
            for s in range(2):
                vs = np.moveaxis(self.us[..., s, :], -1, 0)
                dvs = np.einsum("a,a...->...", d, vs)
                Cd = Cd + dB[..., s] * fs[s] + B[..., s] * fs[s] * (rhod / rho)
                k = c * self.cw[..., s]
                base = dm + (1.0 - omega) * (d @ F) * 0.5 - rho * dvs
                dJ += (k * (dB[..., s] * base + B[..., s] * (dmd - domega * (d @ F) * 0.5
                                                              + (1.0 - omega) * (d @ dF) * 0.5
                                                              - rhod * dvs))).sum()
                drag += (self.cw[..., s] * B[..., s] * base).sum()
            J += c * drag
            C = (1.0 - omega) * f + (omega - Bt) * feq + B[..., 0] * fs[0] + B[..., 1] * fs[1] + gp * g
            f = self.stream(C)
            fd = self.stream(Cd)
        return J, dJ


def eps_slot(p, n, t):
    ids, eps, _ = p.table
    if ids[n][0] == t:
        return eps[n][0]
    if ids[n][1] == t:
        return eps[n][1]
    return 0.0


def oracle_J(params, images, nsteps, t0, t1, direction=(1.0, 0.0, 0.0), kind="restatement"):
    """The objective from the C oracle's own steps (map + collide + reduce)."""
    sim = pyoracle.Sim(kind, **params)
    d = np.asarray(direction, dtype=np.float64)
    M = t1 - t0 + 1
    J = 0.0
    for t in range(1, nsteps + 1):
        fh, _, _ = sim.step(images["tag"], images["x"], images["v"], images["omega"], images["radius"])
        if t0 <= t <= t1:
            J += float((fh @ d).sum()) / M
    sim.close()
    return J
