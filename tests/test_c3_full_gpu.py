"""The benchmarked workload at full size against the CPU oracle.

D3Q19 256^3, x and z periodic, Zou-He shear walls in y (+-0.01), tau 0.65,
2000 spheres of diameter 12 by the benchmark's seeded random sequential
addition (2281 images with the periodic ghosts), moving on the benchmark's
closed loops.  Two coupling steps: the first with the spheres where the
placement put them (an empty table), the second with every sphere moved to
its next position (slots set, kept and cleared).

* FP64 storage: after each step the device's particle table is bit-identical
  to the oracle's setParticlesOnLattice result on every stored node
  (src/LBM_PSM_exchangeParticleData.cpp:24-169), and the per-image force,
  torque and stresslet agree within 1e-12 relative
  (src/LBM_PSM_exchangeParticleData.cpp:172-244).
* FP32 storage (the benchmarked path, with its FP32 solid-fraction filters,
  whole-slab shortcuts and crossing-row ranks): the same slot ids on every
  node, and the FP32 records equal the FP32 roundings of the oracle's solid
  fractions and node velocities.
"""
import os
import sys

import numpy as np
import pytest

import cases
import pyoracle

pytestmark = pytest.mark.gpu

sys.path.insert(0, cases.ROOT)
import bench  # noqa: E402

TOL_FTS = 1e-12


@pytest.fixture(scope="module")
def workload():
    g, nloc = bench.images()
    xs, vs = bench.moving_image_sets(g, nloc)
    a = dict(tag=np.asarray(g.tag, np.int32), omega=np.zeros((len(g.tag), 3)),
             radius=np.asarray(g.radius))
    steps = [dict(a, x=xs[k], v=vs[k]) for k in range(2)]
    prm = bench.workload_params()
    orc = pyoracle.Sim("restatement", **prm, bc_type=1)
    orc.set_threads(os.cpu_count() or 1)
    out, tables = [], []
    for s in steps:
        out.append(orc.step(s["tag"], s["x"], s["v"], s["omega"], s["radius"], bc=True))
        ids, eps, us, _ = orc.pdata()
        tables.append((ids, eps, us))
    orc.close()
    return prm, steps, out, tables, nloc


def _lattice(prm, storage, n):
    import lbmpsm
    lat = lbmpsm.Lattice(**prm, storage=storage, max_images=n, max_radius=bench.DIAM / 2)
    lat.set_bc("shear")
    return lat


def test_c3_full_size_fp64_map_and_forces_against_oracle(workload):
    from test_parity_gpu import compare_fts
    prm, steps, out, tables, nloc = workload
    lat = _lattice(prm, "fp64", len(steps[0]["tag"]))
    m = lat.stored_mask()
    for k, s in enumerate(steps):
        got = lat.step(s["tag"], s["x"], s["v"], s["omega"], s["radius"])
        lat.apply_bc()
        err = compare_fts(got, out[k], s["radius"])
        assert err <= TOL_FTS, (k, err)
        ids_g, eps_g, us_g = lat.particle_table()
        ids_o, eps_o, us_o = tables[k]
        assert np.array_equal(ids_g[m], ids_o[m]), k
        assert np.array_equal(eps_g[m], eps_o[m]), k
        assert np.array_equal(us_g[m], us_o[m]), k
        occ = (ids_o[m] > 0).sum()
        assert occ > 2000 * 500, occ  # the spheres' nodes are all in the table
    lat.close()


def test_c3_full_size_fp32_map_against_oracle(workload):
    prm, steps, out, tables, nloc = workload
    lat = _lattice(prm, "fp32", len(steps[0]["tag"]))
    m = lat.stored_mask()
    for k, s in enumerate(steps):
        got = lat.step(s["tag"], s["x"], s["v"], s["omega"], s["radius"])
        lat.apply_bc()
        ids_g, eps_g, us_g = lat.particle_table()
        ids_o, eps_o, us_o = tables[k]
        assert np.array_equal(ids_g[m], ids_o[m]), k
        # the FP32 records: eps and the (non-spinning) node velocity rounded once
        assert np.array_equal(eps_g[m], eps_o[m].astype(np.float32).astype(np.float64)), k
        assert np.array_equal(us_g[m], us_o[m].astype(np.float32).astype(np.float64)), k
        # FP32 collision: drag of the locals within the FP32 bound of the FP64 oracle
        F, F64 = got[0][:nloc], out[k][0][:nloc]
        assert np.abs(F - F64).max() <= 1e-3 * np.abs(F64).max(), k
    lat.close()
