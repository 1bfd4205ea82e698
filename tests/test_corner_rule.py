"""The shell-node corner rule of the particle map, restated in numpy FP32
(the device code is built without contraction, so each FP32 operation rounds
as here): a node between the early-out radii whose far sub-cell corner is
inside gets the full count, one whose nearest possible sub-cell is outside
gets 0.  Every node the rule decides must carry that count in the
reference's FP64 sub-cell loop (src/LBM_PSM_exchangeParticleData.cpp:144-168);
the GPU map tests check the kernel itself bit for bit against the oracle."""
import numpy as np

F32 = np.float32
U = F32(2.0 ** -24)
DELTA = np.array([-0.5 + (i + 0.5) * 0.1 for i in range(10)])  # the reference's offsets


def exact_count(dx, dy, dz, r, dim):
    rsq = r * r
    X, Y, Z = (dx + DELTA) ** 2, (dy + DELTA) ** 2, (dz + DELTA) ** 2
    if dim == 2:
        return int(np.sum((X[:, None] + Y[None, :]) < rsq))
    return int(np.sum(((X[:, None, None] + Y[None, :, None]) + Z[None, None, :]) < rsq))


def corner_count(dim, dxf, dyf, dzf, rsqf):
    """The device rule (particles.cu corner_count), operation for operation."""
    ax, ay = abs(dxf), abs(dyf)
    az = abs(dzf) if dim == 3 else F32(0)
    ea, eb, ec = ax + F32(2), ay + F32(2), az + F32(2)
    m = F32(16) * U * (ea * ea + eb * eb + (ec * ec if dim == 3 else F32(0)) + rsqf)
    fx, fy, fz = ax + F32(0.45), ay + F32(0.45), az + F32(0.45)
    far = fx * fx + fy * fy + (fz * fz if dim == 3 else F32(0))
    if far < rsqf - m:
        return 1000 if dim == 3 else 100
    nx, ny, nz = (max(a - F32(0.45), F32(0)) for a in (ax, ay, az))
    near = nx * nx + ny * ny + (nz * nz if dim == 3 else F32(0))
    if near > rsqf + m:
        return 0
    return -1


def test_corner_rule_agrees_with_the_reference_count():
    rng = np.random.default_rng(2026)
    half = {2: np.sqrt(2.1) / 2.0, 3: np.sqrt(3.1) / 2.0}
    decided = {2: 0, 3: 0}
    shell = {2: 0, 3: 0}
    for trial in range(6000):
        dim = 3 if trial % 3 else 2
        r = rng.uniform(0.3, 12.0)
        xl = rng.uniform(-40.0, 300.0, 3)
        d = rng.normal(size=3)
        if dim == 2:
            d[2] = 0.0
        d /= np.linalg.norm(d)
        node = np.round(xl + d * (r + rng.uniform(-half[dim], half[dim]))).astype(int)
        if dim == 2:
            node[2] = 0
            xl[2] = 0.0
        dx, dy, dz = node - xl
        if trial % 2:
            # the node's farthest or nearest sub-cell centre a hair from the
            # surface: only the margin keeps the FP32 rule from deciding it
            sums = [(dx + DELTA) ** 2, (dy + DELTA) ** 2,
                    (dz + DELTA) ** 2 if dim == 3 else np.zeros(1)]
            pick = max if trial % 4 == 1 else min
            s2 = pick(sums[0]) + pick(sums[1]) + pick(sums[2])
            r = float(np.sqrt(s2)) * (1.0 + 1e-12 * rng.integers(-1, 2))
            if r < 0.3:
                continue
        dist = dx * dx + dy * dy + dz * dz
        rp, rm = r + half[dim], r - half[dim]
        if dist > rp * rp or dist < rm * rm:
            continue  # decided by the reference's own early-outs
        shell[dim] += 1
        xi = np.floor(xl).astype(int)
        xf = (xl - xi).astype(F32)  # xl = xi + xf exactly, as the map splits it
        dxf, dyf, dzf = (F32(node[k] - xi[k]) - xf[k] for k in range(3))
        c = corner_count(dim, dxf, dyf, dzf, F32(r * r))
        if c < 0:
            continue
        decided[dim] += 1
        assert c == exact_count(dx, dy, dz, r, dim), (dim, r, xl, node, c)
    for dim in (2, 3):
        assert shell[dim] > 500 and decided[dim] > 0.05 * shell[dim], (dim, shell, decided)
