"""The row segments of the particle map's classification and of the FP32
reduction, restated in numpy FP32 (the device code is built without
contraction, so each FP32 operation rounds as here).  Both kernels visit, in
each x-row of an image box, only the nodes between

    xa = xi + ceil(xf - h),  xb = xi + floor(xf + h) + 1,
    h = sqrt(rP^2 * 1.0001 + 0.01 - dy^2 - dz^2) + 0.01   (FP32)

and treat every other node as beyond the early-out radius rP.  That is exact
when the segment holds every node that classify_node's FP32 test does not put
beyond rP for certain (d32 <= rP^2 + m): those are the only nodes whose code
can be non-zero, and the only ones that can hold the image's tag after the
map (an eps > 0 from this image means the FP64 distance is at most rP).  The
GPU map and force tests check the kernels themselves against the oracle."""
import numpy as np

F32 = np.float32
U = F32(2.0 ** -24)


def small_int(k):
    return F32(k)  # exact for |k| < 2^24, as small_int_to_float on the device


def beyond_rp(dxf, dyf, dzf, rp2f):
    """classify_node's first test (particles.cu beyond_rP_f), operation for operation."""
    d32 = (dxf * dxf + dyf * dyf) + dzf * dzf
    ad = (abs(dxf) + abs(dyf)) + abs(dzf)
    m = (F32(16) * U) * ((((F32(5) * d32) + (F32(2) * ad)) + F32(1)) + rp2f)
    return d32 > rp2f + m


def segment(xi0, xf0, dyf, dzf, rp2f):
    """The x-range [xa, xb) of one row (None when the row misses rP)."""
    rem0 = rp2f * F32(1.0001) + F32(0.01)
    rem = (rem0 - dyf * dyf) - dzf * dzf
    if rem < F32(0):
        return None
    h = np.sqrt(rem, dtype=F32) + F32(0.01)
    xa = xi0 + int(np.ceil(xf0 - h))
    xb = xi0 + int(np.floor(xf0 + h)) + 1
    return xa, xb


def check_image(rng, r, dim):
    """Every node of the image's box outside its rows' segments is beyond rP."""
    xl = rng.uniform(-40.0, 40.0, 3)
    if dim == 2:
        xl[2] = rng.choice([0.0, 1.0])  # the single z layer's offset
    xi = np.floor(xl).astype(np.int64)
    xf = (xl - xi).astype(F32)  # the FP32 rounding of the exact fraction, as im.xf
    rp = r + (np.sqrt(3.1) / 2.0 if dim == 3 else np.sqrt(2.1) / 2.0)
    rp2f = F32(rp * rp)
    lo = np.floor(xl - r).astype(np.int64) - 2
    hi = np.floor(xl + r).astype(np.int64) + 3
    kz = [int(xi[2])] if dim == 2 else range(lo[2], hi[2])
    inside = missed = 0
    for k in kz:
        dzf = small_int(k - xi[2]) - xf[2]
        for j in range(lo[1], hi[1]):
            dyf = small_int(j - xi[1]) - xf[1]
            seg = segment(int(xi[0]), xf[0], dyf, dzf, rp2f)
            for i in range(lo[0], hi[0]):
                dxf = small_int(i - xi[0]) - xf[0]
                if beyond_rp(dxf, dyf, dzf, rp2f):
                    continue
                inside += 1
                if seg is None or not (seg[0] <= i < seg[1]):
                    missed += 1
    return inside, missed


def test_segments_hold_every_node_within_rp_3d():
    rng = np.random.default_rng(11)
    total = 0
    for r in list(rng.uniform(0.3, 3.0, 40)) + list(rng.uniform(3.0, 12.0, 20)):
        inside, missed = check_image(rng, float(r), 3)
        assert missed == 0
        total += inside
    assert total > 10000


def test_segments_hold_every_node_within_rp_2d():
    rng = np.random.default_rng(12)
    for r in list(rng.uniform(0.3, 4.0, 60)) + list(rng.uniform(4.0, 20.0, 20)):
        inside, missed = check_image(rng, float(r), 2)
        assert missed == 0


class _Fixed:
    """A stand-in generator that places the centre at (c, c, c)."""

    def __init__(self, c):
        self.c = c

    def uniform(self, a, b, n):
        return np.full(n, self.c)

    def choice(self, options):
        return options[0]


def test_segments_at_integer_and_half_integer_centres():
    """Centres on and next to node planes, where segment ends meet nodes."""
    for frac in (0.0, 0.5, 1.0 - 2.0 ** -20, 2.0 ** -20):
        for r in (0.5, 1.0, 2.0, 3.5, 6.0, 6.5, 9.0):
            inside, missed = check_image(_Fixed(7.0 + frac), r, 3)
            assert missed == 0 and inside > 0
