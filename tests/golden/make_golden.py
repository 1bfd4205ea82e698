"""Generate the golden fixtures of the LBM-PSM parity cases from the reference
itself: the reference's own unmodified src/LBM_PSM_*.cpp built with stub
LAMMPS/MPI headers (oracle/_ref/libref_oracle.so, see oracle/Makefile).

    make -C oracle ref && python tests/golden/make_golden.py

Writes tests/golden/reference_cases.npz.  For every case of tests/cases.py it
stores the per-image force / torque / stresslet at sampled steps, and of the
final state the nonzero particle-table entries, the mass/momentum sums and
the populations of a fixed sample of nodes (all in the reference layout).
The reference sources are needed only here; the fixtures travel with the
repository.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import cases  # noqa: E402
import pyoracle  # noqa: E402

OUT = os.path.join(HERE, "reference_cases.npz")
RECORD_EVERY = 5
NODE_SAMPLE = 64


def stored_mask(case, shape):
    """Nodes a single-GPU lattice stores: all but the halo planes of periodic axes."""
    m = np.ones(shape, dtype=bool)
    for d in range(case.dim):
        if case.periodic[d]:
            idx = [slice(None)] * 3
            idx[d] = 0
            m[tuple(idx)] = False
            idx[d] = shape[d] - 1
            m[tuple(idx)] = False
    return m


def summarize(case, sim):
    f = sim.populations()
    ids, eps, us, _ = sim.pdata()
    mask = stored_mask(case, sim.shape)
    e = np.array([[1, 0, 0]])
    ex = np.array([[0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0],
                   [0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1],
                   [0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1]]) if case.dim == 3 else \
        np.array([[0, 1, 0, -1, 0, 1, -1, -1, 1], [0, 0, 1, 0, -1, 1, 1, -1, -1], [0] * 9])
    fs = f[mask]
    sums = np.array([fs.sum(), (fs * ex[0]).sum(), (fs * ex[1]).sum(), (fs * ex[2]).sum()])
    flat = np.flatnonzero(mask.reshape(-1))
    rng = np.random.default_rng(1234)
    sample = np.sort(rng.choice(flat, size=min(NODE_SAMPLE, len(flat)), replace=False))
    fpop = f.reshape(-1, sim.q)[sample]
    occ = np.flatnonzero((ids.reshape(-1, 2) != 0).any(axis=1))
    occ = occ[mask.reshape(-1)[occ]]
    del e
    return dict(sums=sums, sample=sample, fpop=fpop, occ=occ, ids=ids.reshape(-1, 2)[occ],
                eps=eps.reshape(-1, 2)[occ], us=us.reshape(-1, 6)[occ])


def main():
    pyoracle.build(reference=True)
    data = {}
    for name, case in cases.CASES.items():
        be = cases.OracleBackend(case, kind="reference")
        rec = cases.run(case, be, cases.oracle_make_ghosts, record_every=RECORD_EVERY)
        steps = np.array([r[0] for r in rec])
        counts = np.array([len(r[1]) for r in rec])
        tags = np.concatenate([r[1] for r in rec])
        fts = np.concatenate([np.concatenate([r[2], r[3], r[4]], axis=1) for r in rec])
        tag, x, v, w, rad = cases.initial_particles(case)
        data[f"{name}/steps"] = steps
        data[f"{name}/counts"] = counts
        data[f"{name}/tags"] = tags
        data[f"{name}/fts"] = fts
        data[f"{name}/x0"] = x
        data[f"{name}/r0"] = rad
        for k, val in summarize(case, be.sim).items():
            data[f"{name}/{k}"] = val
        print(f"{name:20s} steps={case.steps} images/step={counts.max()} "
              f"occupied={len(data[f'{name}/occ'])} |F|={np.abs(fts[:, :3]).max():.3e}")
    np.savez_compressed(OUT, **data)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
