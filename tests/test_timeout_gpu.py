"""The bounded device-side wait of the FP32 / FP16 collide pipeline.

Every wait in collide_pipe_kernel has an iteration limit; when the consumer
warps give up on a stage they record STATUS_TIMEOUT, the producer warp lets
the bulk loads it issued land and the block returns, and the host reports
LBMPSM_ERR_TIMEOUT.  The test hook LBMPSM_TEST_FULL_WAIT_LIMIT=-1 (read when
a handle is created) gives the consumers' stage wait no polls at all, so the
first stage "times out" at once on every block -- the expiry path runs
without any wait running long and without a fault.  A handle created
afterwards without the hook steps normally.
"""
import numpy as np
import pytest

import cases
import lbmpsm

pytestmark = pytest.mark.gpu


def _first_images(case):
    tag, x, v, w, r = cases.initial_particles(case)
    return cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
def test_stage_wait_expiry_is_reported_and_a_fresh_handle_steps(storage, monkeypatch):
    case = cases.CASES["c2_sphere_3d"]
    g = _first_images(case)
    a = (g["tag"], g["x"], g["v"], g["omega"], g["radius"])
    monkeypatch.delenv("LBMPSM_PIPE_STAGES", raising=False)
    monkeypatch.setenv("LBMPSM_TEST_FULL_WAIT_LIMIT", "-1")
    lat = lbmpsm.Lattice(**case.params(), storage=storage, collide_tuning="default")
    monkeypatch.delenv("LBMPSM_TEST_FULL_WAIT_LIMIT")
    assert lat.get_info().collide_stages > 0  # the row pipeline, not the direct kernel
    with pytest.raises(lbmpsm.LbmPsmError) as e:
        lat.step(*a)
    assert e.value.code == lbmpsm.ERR_TIMEOUT
    assert "bounded device-side wait" in str(e.value)
    # the context is usable: the status word was reset and the handle closes
    lat.synchronize()
    lat.close()

    fresh = lbmpsm.Lattice(**case.params(), storage=storage, collide_tuning="default")
    ref = lbmpsm.Lattice(**case.params(), storage=storage, collide_tuning="default")
    for _ in range(3):
        out = fresh.step(*a)
        exp = ref.step(*a)
        for o, x in zip(out, exp):
            assert np.all(np.isfinite(o))
            assert np.array_equal(o, x)
    assert abs(out[0][0, 0]) > 0.0
    mass, _ = fresh.check()
    assert np.isfinite(mass)
    fresh.close()
    ref.close()
