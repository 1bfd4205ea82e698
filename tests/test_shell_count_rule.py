"""The shell-node sub-cell count of the particle map (sf_shell), restated in
numpy FP32 operation for operation (the device code is built without
contraction): the FP32 filter with its margin M, whole slabs decided at
once, rows wholly inside or outside, crossing rows counted by rank among the
sorted c-terms, and the FP64 recount of a row with a c-term inside the
margin band.  The count must equal the reference's FP64 loop
(src/LBM_PSM_exchangeParticleData.cpp:144-168) on every node of the
reference's shell band; the GPU map tests check the kernel itself."""
import numpy as np

F32 = np.float32
U = F32(2.0 ** -24)
DELTA = np.array([-0.5 + (i + 0.5) * 0.1 for i in range(10)])  # the reference's offsets
OFFC = DELTA.astype(F32)                                         # their FP32 roundings
SUB = np.array([F32(-0.45) + F32(0.1) * F32(k) for k in range(10)], dtype=F32)  # sub_offset
BIG = F32(3.0e38)


def exact_count(d, r, dim):
    rsq = r * r
    X, Y, Z = ((d[k] + DELTA) ** 2 for k in range(3))
    if dim == 2:
        return int(np.sum((X[:, None] + Y[None, :]) < rsq))
    return int(np.sum(((X[:, None, None] + Y[None, :, None]) + Z[None, None, :]) < rsq))


def exact_row(D, rsq, pa, pb, ia, ib, dc, tlo, thi):
    """The row (ia on axis pa, ib on axis pb) recounted: FP32 filter, FP64
    reference expression inside the band (particles.cu exact_row_count)."""
    n = 0
    for c in range(10):
        t = dc + OFFC[c]
        sc = t * t
        if sc < tlo:
            n += 1
        elif sc <= thi:
            idx = [None, None, None]
            idx[pa], idx[pb] = ia, ib
            idx[3 - pa - pb] = c
            t0, t1, t2 = (D[k] + DELTA[idx[k]] for k in range(3))
            if t0 * t0 + t1 * t1 + t2 * t2 < rsq:
                n += 1
    return n


def shell_count(dim, dxf, dyf, dzf, rsqf, D, r):
    rsq = r * r
    if dim == 2:
        ea, eb = abs(dxf) + F32(2), abs(dyf) + F32(2)
        m = F32(16) * U * (ea * ea + eb * eb + rsqf)
        lo, hi = rsqf - m, rsqf + m
        n, amb = 0, 0
        for a in range(10):
            ta = dxf + SUB[a]
            sa = ta * ta
            for b in range(10):
                tb = dyf + OFFC[b]
                t = sa + tb * tb
                n += int(t < lo)
                amb += int(lo <= t <= hi)
        return exact_count(D, r, 2) if amb else n
    ax, ay, az = abs(dxf), abs(dyf), abs(dzf)
    da, db, dc, pa, pb = dxf, dyf, dzf, 0, 1
    if ax <= ay and ax <= az:
        da, db, dc, pa, pb = dyf, dzf, dxf, 1, 2
    elif ay <= ax and ay <= az:
        da, db, dc, pa, pb = dxf, dzf, dyf, 0, 2
    if abs(db) > abs(da):  # the outer role takes the larger offset
        da, db, pa, pb = db, da, pb, pa
    ea, eb, ec = abs(da) + F32(2), abs(db) + F32(2), abs(dc) + F32(2)
    m = F32(16) * U * (ea * ea + eb * eb + ec * ec + rsqf)
    lo, hi = rsqf - m, rsqf + m
    sc = np.sort(np.array([(dc + OFFC[c]) * (dc + OFFC[c]) for c in range(10)], dtype=F32))
    srt = np.concatenate([sc, np.full(6, BIG, dtype=F32)])
    lo_in, hi_out = lo - sc[9], hi - sc[0]
    sb = np.array([(db + SUB[b]) * (db + SUB[b]) for b in range(10)], dtype=F32)
    n = 0
    for a in range(10):
        ta = da + SUB[a]
        sa = ta * ta
        if sa + sb.max() < lo_in:  # the whole slab inside
            n += 100
            continue
        if sa + sb.min() > hi_out:  # the whole slab outside
            continue
        for b in range(10):
            sv = sa + sb[b]
            if sv < lo_in:
                n += 10
            elif sv <= hi_out:  # a crossing row
                tlo, thi = lo - sv, hi - sv
                r = int(np.sum(srt < tlo))
                n += exact_row(D, rsq, pa, pb, a, b, dc, tlo, thi) if srt[r] <= thi else r
    return n


def test_shell_count_equals_the_reference_count():
    rng = np.random.default_rng(77)
    half = {2: np.sqrt(2.1) / 2.0, 3: np.sqrt(3.1) / 2.0}
    seen = {2: 0, 3: 0}
    for trial in range(4000):
        dim = 3 if trial % 4 < 2 else 2
        r = rng.uniform(0.3, 10.0)
        xl = rng.uniform(-30.0, 200.0, 3)
        d = rng.normal(size=3)
        if dim == 2:
            d[2] = 0.0
        d /= np.linalg.norm(d)
        node = np.round(xl + d * (r + rng.uniform(-half[dim], half[dim]))).astype(int)
        if dim == 2:
            node[2] = 0
            xl[2] = 0.0
        D = node - xl
        if trial % 4 in (1, 3):
            # a sub-cell centre on the surface: the FP32 margin band must
            # send its row (its node in 2-D) to the FP64 recount
            i = rng.integers(0, 10, 3)
            s2 = (D[0] + DELTA[i[0]]) ** 2 + (D[1] + DELTA[i[1]]) ** 2
            if dim == 3:
                s2 += (D[2] + DELTA[i[2]]) ** 2
            # exactly on it, or a hair inside or outside (below FP32 resolution)
            r = float(np.sqrt(s2)) * (1.0 + 1e-12 * rng.integers(-1, 2))
            if r < 0.3:
                continue
        dist = D @ D
        if dist > (r + half[dim]) ** 2 or dist < (r - half[dim]) ** 2:
            continue  # the reference's early-outs decide it
        seen[dim] += 1
        xi = np.floor(xl).astype(int)
        xf = (xl - xi).astype(F32)
        dxf, dyf, dzf = (F32(node[k] - xi[k]) - xf[k] for k in range(3))
        got = shell_count(dim, dxf, dyf, dzf, F32(r * r), D, r)
        assert got == exact_count(D, r, dim), (dim, r, xl, node, got)
    assert seen[2] > 1000 and seen[3] > 1000, seen
