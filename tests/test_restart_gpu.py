"""Restart files interoperate between the CPU reference path and the GPU
library (`fix lbm-psm-restart`, src/fix_LBM_PSM_writeReadRestart.cpp).

A restart holds the post-stream populations only, so a run restarted from a
file starts with an empty particle table on either side.  Both directions
are checked bit for bit (FP64 storage, cases without periodic-seam
crossings): a file the GPU wrote and a file the oracle wrote (the raw
f_curr, stale periodic halo included) are read by a fresh GPU lattice and a
fresh oracle, which then run on identically.
"""
import numpy as np
import pytest

import cases
from lbmpsm import host

pytestmark = pytest.mark.gpu


def _run(backend, case, state, steps):
    tag, x, v, w, r = state
    for _ in range(steps):
        g = cases.images(case, tag, x, v, w, r, cases.product_make_ghosts)
        backend.step(g["tag"], g["x"], g["v"], g["omega"], g["radius"])
        if case.bc:
            backend.apply_bc()
        x = cases.advance(case, x, v)
    return tag, x, v, w, r


def _restarted_pair(case, path):
    gpu = cases.GpuBackend(case, "fp64")
    fix = type("F", (), {"lattice": gpu.lat})()
    rs = host.FixLbmPsmRestart(["rs", "all", "lbm-psm-restart", "every", "1", "write", "0",
                                "read", "1"], fix, folder=str(path))
    rs.init()
    orc = cases.OracleBackend(case)
    orc.sim.set_populations(host.read_restart(str(path / host.restart_file_name(0))).reshape(
        orc.sim.shape + (orc.sim.q,)))
    return gpu, orc


@pytest.mark.parametrize("name", ["c2_sphere_3d", "closedbox_3d"])
def test_restart_written_by_gpu_and_by_oracle(name, tmp_path):
    case = cases.CASES[name]
    state0 = cases.initial_particles(case)
    for writer in ("gpu", "oracle"):
        d = tmp_path / writer
        d.mkdir()
        if writer == "gpu":
            a = cases.GpuBackend(case, "fp64")
            state = _run(a, case, state0, 7)
            fix = type("F", (), {"lattice": a.lat})()
            host.FixLbmPsmRestart(["rs", "all", "lbm-psm-restart", "every", "7", "write", "1",
                                   "read", "0"], fix, folder=str(d)).pre_force(7)
        else:
            a = cases.OracleBackend(case)
            state = _run(a, case, state0, 7)
            host.write_restart(str(d / host.restart_file_name(0)), a.sim.populations())
        gpu, orc = _restarted_pair(case, d)
        _run(gpu, case, state, 6)
        _run(orc, case, state, 6)
        m = gpu.lat.stored_mask()
        assert np.array_equal(gpu.lat.populations()[m], orc.sim.populations()[m]), writer
