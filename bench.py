#!/usr/bin/env python3
"""LBM-PSM coupling-step throughput on GB300: D3Q19 PSM MLUPS and % of the
HBM roofline, FP32 storage against the plain FP64 path.

Workload (the sheared dense suspension): D3Q19 256^3 lattice, x and z
periodic, Zou-He moving walls in y (top +0.01, bottom -0.01 lattice units,
`fix lbm-psm-bc shear`), tau = 0.65, 2000 spheres of diameter 12 lattice
units placed by seeded random sequential addition (solid fraction ~0.108).
Synthetic data: no dataset is involved.  One "step" is one LBM coupling
step: particle map, fused collide + stream, per-particle force/torque/
stresslet reduction, and the wall boundary condition.  The spheres move on
every step (each on its own seeded closed loop of radius 0.1 lattice units,
their ghost images with them), so every step maps new sub-cell positions,
as the host DEM's motion would make it do.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line on rank 0.  `value` is measured with the images'
positions resident in HBM (one set per step of the loops) and handed to
lbmpsm_step_device each step, which the library replays as a CUDA graph;
`e2e` runs the same steps through the host-pointer C-ABI call, also one graph
per step: on GB300 the gather kernel reads the caller's image arrays and the
reduction writes the forces into the caller's arrays over NVLink-C2C
(pageable host memory through the host page tables, no staging copies);
`e2e_staged` is the same call with LBMPSM_HOST_STAGING=1 (images copied into
pinned memory and up, forces copied back).  The lattice (1.27 GB in FP32) is ~10x larger than L2, so no L2 flush
is needed between steps.  `--impl reference` times the CPU oracle (the
reference algorithm restated in C, FP64, all host cores) on the same
workload.  `--workload ensemble` and `--workload adjoint` time the batched
boxes and the drag sensitivities.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "lammps-lbm-psm_gb300")
sys.path.insert(0, PKG)

EDGE = 256
NSPHERES = 2000
DIAM = 12.0
TAU = 0.65
U_WALL = 0.01
SEED = 20261203
METRIC = "D3Q19 PSM MLUPS & % HBM roofline, FP32 vs FP64 at fixed drag error, 1 GB300"
REF_MAX_STEPS = 20
BYTES_PER_NODE = {"fp64": 2 * 19 * 8, "fp32": 2 * 19 * 4, "fp16": 2 * 19 * 2, "bf16": 2 * 19 * 2}


def workload_params(edge=None):
    edge = edge or EDGE
    lc = DIAM
    nu = (TAU - 0.5) / 3.0
    Re = U_WALL * lc / nu
    # x, z periodic: edge nodes span edge*dx; y walls: edge nodes span (edge-1)*dx
    return dict(dimension=3, boxlo=(0.0, 0.0, 0.0), prd=(float(edge), float(edge - 1), float(edge)),
                periodic=(1, 0, 1), nevery=1, Nlc=int(DIAM) + 1, lc=lc, rho=1.0, nu=nu, Re=Re,
                tau=TAU, Fext=(0.0, 0.0, 0.0))


def rsa_spheres(edge=None, n=None, d=DIAM, seed=SEED):
    """Seeded random sequential addition, minimum image in the periodic x, z."""
    edge = edge or EDGE
    n = NSPHERES if n is None else n
    rng = np.random.default_rng(seed)
    L = np.array([edge, edge - 1.0, edge])
    r = d / 2
    acc = np.zeros((n, 3))
    k = 0
    tries = 0
    while k < n:
        tries += 1
        if tries > 200 * n:
            raise RuntimeError("random sequential addition did not converge")
        c = np.array([rng.uniform(0, L[0]), rng.uniform(r + 1.0, L[1] - r - 1.0), rng.uniform(0, L[2])])
        if k:
            dlt = acc[:k] - c
            for ax in (0, 2):
                dlt[:, ax] -= L[ax] * np.round(dlt[:, ax] / L[ax])
            if np.min(np.einsum("ij,ij->i", dlt, dlt)) < d * d:
                continue
        acc[k] = c
        k += 1
    return acc, np.full(n, r)


def images(edge=None, nspheres=None):
    from lbmpsm.host import Domain, ghost_images
    edge = edge or EDGE
    x, r = rsa_spheres(edge, nspheres)
    n = len(x)
    prm = workload_params(edge)
    lo = prm["boxlo"]
    hi = tuple(a + b for a, b in zip(lo, prm["prd"]))
    dom = Domain(3, lo, hi, prm["periodic"])
    return ghost_images(dom, DIAM / 2 + 3.0, np.arange(1, n + 1), x, np.zeros((n, 3)), np.zeros((n, 3)), r), n


MOVE_SETS = 32      # the images' positions repeat after this many steps
MOVE_AMP = 0.1      # lattice units: each sphere walks a closed loop of this radius
MOVE_SEED = 20261205


def suspension_workload(edge, nspheres):
    """The suspension workload's description, the same for both arms."""
    return (f"sheared suspension: D3Q19 {edge}^3, y Zou-He shear walls +-0.01, tau 0.65, "
            f"{nspheres} spheres D=12 (seeded RSA, phi~0.108 at 256^3) moving on seeded closed "
            f"loops (new positions every step)")


def moving_image_sets(g, nloc, nsets=MOVE_SETS, amp=MOVE_AMP, seed=MOVE_SEED):
    """Positions and velocities of the images for nsets consecutive steps: every
    sphere moves on its own seeded closed loop (an ellipse of radius `amp`
    lattice units in a random plane, one turn per nsets steps, top speed
    2*pi*amp/nsets ~ 0.02 lattice units per step), its ghost images with it,
    so that the map sees new sub-cell positions on every step.  Returns
    x[nsets, n, 3] and v[nsets, n, 3] (v = displacement per step)."""
    rng = np.random.default_rng(seed)
    n = len(g.tag)
    a = rng.normal(size=(nloc, 3))
    b = rng.normal(size=(nloc, 3))
    a /= np.linalg.norm(a, axis=1, keepdims=True)
    b -= a * np.einsum("ij,ij->i", a, b)[:, None]
    b /= np.linalg.norm(b, axis=1, keepdims=True)
    phase = rng.uniform(0.0, 2 * np.pi, nloc)
    # the local atom each image was copied from (ghosts of ghosts resolved)
    src = np.asarray(g.owner).copy()
    for _ in range(4):
        src = np.where(src >= nloc, np.asarray(g.owner)[src], src)
    t = 2 * np.pi * np.arange(nsets + 1)[:, None] / nsets + phase[None, :]
    d = amp * (np.cos(t)[..., None] * a[None] + np.sin(t)[..., None] * b[None])  # (nsets+1, nloc, 3)
    d -= d[0][None]  # the first set is the RSA placement itself
    x = np.asarray(g.x)[None] + d[:nsets, src]
    v = (d[1:] - d[:-1])[:, src]
    return np.ascontiguousarray(x), np.ascontiguousarray(v)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms; only the
    samples that arrive inside the marked timed window are summarised."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[tuple[float, str]] = []
        self.window = (0.0, 0.0)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.monotonic()
            while not self.lines and time.monotonic() - t0 < 3.0:  # sampler is running
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))

    def mark(self, start: float, end: float):
        self.window = (start, end)

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.06)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t0, t1 = self.window
        for ts, ln in self.lines:
            if not (t0 <= ts <= t1 + 0.06):
                continue
            p = [s.strip() for s in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, val in zip(names, p[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(storage="fp32"):
    """Per-launch DRAM traffic of the collide kernel at the bench size, from
    the committed ncu summary of that storage
    (profiles/collide_{f32,f16,bf16}_d3q19_256.md), else None."""
    tag = {"fp32": "f32", "fp16": "f16", "bf16": "bf16"}[storage]
    path = os.path.join(ROOT, "profiles", f"collide_{tag}_d3q19_256.md")
    try:
        for ln in open(path):
            if ln.startswith("traffic_bytes_per_launch:"):
                return float(ln.split(":")[1])
    except OSError:
        pass
    return None


class MovingImages:
    """The images of the suspension workload on the device, one position and
    velocity set per step of the closed loops (moving_image_sets), uploaded
    once; step k hands set k % MOVE_SETS to lbmpsm_step_device, so that every
    step maps images that have moved."""

    def __init__(self, g, nloc, device):
        import torch
        xs, vs = moving_image_sets(g, nloc)
        self.n = len(g.tag)
        self.nsets = len(xs)
        dev = torch.device("cuda", device)
        self.tag = torch.as_tensor(np.asarray(g.tag, np.int32), device=dev)
        self.x = torch.as_tensor(xs, device=dev)
        self.v = torch.as_tensor(vs, device=dev)
        self.omega = torch.zeros((self.n, 3), dtype=torch.float64, device=dev)
        self.radius = torch.as_tensor(np.asarray(g.radius, np.float64), device=dev)
        self.host = (np.asarray(g.tag, np.int32), xs, vs, np.zeros((self.n, 3)),
                     np.asarray(g.radius, np.float64))
        self.host_out = None  # F/T/S of the host steps, one array reused
        torch.cuda.synchronize(dev)

    def step(self, lat, k, bc=True):
        j = k % self.nsets
        lat.step_device(self.n, self.tag.data_ptr(), self.x[j].data_ptr(), self.v[j].data_ptr(),
                        self.omega.data_ptr(), self.radius.data_ptr())
        if bc:
            lat.apply_bc()

    def host_step(self, lat, k):
        """The same step through the host-pointer call, into one output array
        that every step reuses (as a host program's force arrays)."""
        t, xs, vs, w, r = self.host
        j = k % self.nsets
        if self.host_out is None:
            self.host_out = np.empty(12 * len(t))
        out = lat.step(t, xs[j], vs[j], w, r, out=self.host_out)
        lat.apply_bc()
        return out


def run_ours(args, rank=0, world=1):
    import torch

    import lbmpsm

    device = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    edge = args.edge
    g, nloc = images(edge, args.nspheres)
    n = len(g.tag)
    prm = workload_params(edge)
    nodes = edge * edge * edge
    mov = MovingImages(g, nloc, device)

    def make(storage):
        lat = lbmpsm.Lattice(**prm, storage=storage, device=device, max_images=n,
                             max_radius=DIAM / 2 + MOVE_AMP)
        lat.set_bc("shear")
        return lat

    def ev_time(lat, fn):
        s = torch.cuda.ExternalStream(lat.stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        lat.synchronize()
        torch.cuda.synchronize()
        e0.record(s)
        fn()
        e1.record(s)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3

    K, W = args.steps, args.warmup

    def moving(lt, k0, steps):
        def go():
            for k in range(k0, k0 + steps):
                mov.step(lt, k)
        return go

    # FP32 storage: the headline path.  The first step goes through the host
    # call (images up, map, autotuner pending); then W untimed and K timed
    # device steps, the images moving every step
    lat = make(args.storage)
    mov.host_step(lat, 0)
    with ClockSampler(device) as clk:
        moving(lat, 1, W)()
        lat.synchronize()
        if world > 1:
            torch.distributed.barrier()
        t_a = time.monotonic()
        t_val = ev_time(lat, moving(lat, 1 + W, K))
        clk.mark(t_a, time.monotonic())
    t_val = max_over_ranks(t_val, world)
    info = lat.get_info()  # the collide autotuner ran at the second step
    launch = {"stages": int(info.collide_stages), "blocks": int(info.collide_blocks),
              "tuner_ms_per_step_pair": dict(zip(["3", "2", "4", "5"],
                                                 [round(float(t), 4) for t in info.collide_tune_ms]))}

    # end to end: host arrays through lbmpsm_step, copies every step; W
    # untimed steps first (the library captures its host-step graph once the
    # image count has held for two calls)
    k0 = 1 + W + K
    for k in range(k0, k0 + max(W, 3)):
        mov.host_step(lat, k)
    lat.synchronize()
    k0 += max(W, 3)
    t0 = time.perf_counter()
    for k in range(k0, k0 + K):
        mov.host_step(lat, k)
    lat.synchronize()
    t_e2e = max_over_ranks(time.perf_counter() - t0, world)
    e2e_direct = bool(lat.host_direct)

    # the same through pinned staging copies (the path without C2C access)
    os.environ["LBMPSM_HOST_STAGING"] = "1"
    try:
        stg = make(args.storage)
    finally:
        del os.environ["LBMPSM_HOST_STAGING"]
    assert not stg.host_direct
    for k in range(0, 1 + max(W, 3)):
        mov.host_step(stg, k)
    stg.synchronize()
    t0 = time.perf_counter()
    for k in range(1 + max(W, 3), 1 + max(W, 3) + K):
        mov.host_step(stg, k)
    stg.synchronize()
    t_stg = max_over_ranks(time.perf_counter() - t0, world)
    stg.close()

    # the collide-stream kernel alone: lattice-only steps (no images, so the
    # step launches only the collide kernel; the particle table stays in place)
    def lattice_only(lt, steps):
        def go():
            for _ in range(steps):
                lt.step_device(0, None, None, None, None, None)
        return go
    t_kernel = ev_time(lat, lattice_only(lat, K)) / K
    lat.close()

    # plain FP64 path on the same moving workload
    fp64 = None
    if not args.no_fp64:
        lat64 = make("fp64")
        mov.host_step(lat64, 0)
        K64 = max(3, K // 8)
        moving(lat64, 1, 2)()
        t64 = ev_time(lat64, moving(lat64, 3, K64))
        t64_kernel = ev_time(lat64, lattice_only(lat64, 3)) / 3
        lat64.close()
        fp64 = (nodes * K64 / t64 / 1e6, t64_kernel)

    accuracy = None
    if not args.no_accuracy and not args.no_fp64:
        accuracy = developed_accuracy(args, make, mov, nloc, g)

    mlups = whole_job_mlups(nodes, K, world, t_val)
    peak, peak_kind = measured_peak_gbs()
    achieved = BYTES_PER_NODE[args.storage] * nodes / t_kernel / 1e9
    traffic = profile_traffic(args.storage)
    # map: prep, scan, fill, sort, classify, shell, apply; collide; reduce; bc
    launches_per_step = 10
    out = {
        "metric": METRIC,
        "value": round(mlups, 1),
        "unit": "MLUPS",
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": round(t_val / K * 1e3, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",  # FP32 collision arithmetic (FP32 or FP16 storage)
        "data": "synthetic",
        "config": {
            "workload": suspension_workload(edge, nloc) + f", {args.storage.upper()} storage, "
                                                          "FP64 F/T/S",
            "nodes": nodes, "particles": nloc, "images": n, "storage": args.storage,
            "motion": f"every sphere on its own closed loop of radius {MOVE_AMP} lattice units, "
                      f"period {MOVE_SETS} steps (top speed ~0.02 lattice units per step); "
                      "positions uploaded once, handed to lbmpsm_step_device each step",
            "l2": "lattice 1.27 GB > 129 MB L2: no flush needed",
            "parallelism": f"replicas x{world}",
        },
        "e2e": {"value": round(whole_job_mlups(nodes, K, world, t_e2e), 1), "unit": "MLUPS",
                "h2d_bytes_per_step": int(n * (4 + 10 * 8)),
                "d2h_bytes_per_step": int(n * 12 * 8 + 4),  # F/T/S + the status word
                "transfer": ("read and written by the step's kernels over NVLink-C2C (pageable "
                             "host memory through the host page tables)" if e2e_direct else
                             "pinned staging copies")},
        "e2e_staged": {"value": round(whole_job_mlups(nodes, K, world, t_stg), 1), "unit": "MLUPS",
                       "transfer": "images copied into pinned memory and up, forces copied back "
                                   "(LBMPSM_HOST_STAGING=1)"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "kernel": f"collide_pipe_kernel<D3Q19,{ {'fp32': 'float', 'fp16': '__half', 'bf16': '__nv_bfloat16'}[args.storage]}> "
                               "(warp-specialised row pipeline, A-A even/odd)",
                     "algorithmic_bytes_per_node": BYTES_PER_NODE[args.storage],
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "step_hbm_frac": round(BYTES_PER_NODE[args.storage] * nodes / (t_val / K) / 1e9 / peak, 4),
        "fp64_plain": None if fp64 is None else {
            "value": round(fp64[0], 1), "unit": "MLUPS", "kernel_ms": round(fp64[1] * 1e3, 3),
            "hbm_frac": round(BYTES_PER_NODE["fp64"] * nodes / fp64[1] / 1e9 / peak, 4)},
        "fp32_over_fp64": None if fp64 is None else round(mlups / world / fp64[0], 2),
        "drag_rel_err_fp32_vs_fp64": None if accuracy is None else accuracy["suspension"]["fp32"]["drag"],
        "accuracy_vs_fp64": accuracy,
        "kernel_ms": round(t_kernel * 1e3, 4),
        "collide_launch": launch,
        "gpu_launches": launches_per_step * K,
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args.cpu_steps, single_core=True)
    return out


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def developed_accuracy(args, make, mov, nloc, g):
    """FP32 (and FP16, BF16) storage against the plain FP64 path at developed
    states, every run from rest with the same inputs:
      * the suspension itself after args.acc_steps coupling steps (default
        2000, about 0.7 viscous times D^2/nu of a sphere) with the images
        moving every step: drag, torque and stresslet of the 2000 spheres
        (ghost rows summed into their owners), velocity field, mass drift;
      * the single-sphere configuration (D3Q19 128^3 periodic, tau 0.7,
        Fext (1e-6, 0, 0), sphere of diameter 16 at the centre) after
        args.acc_c2_steps steps (default 10^4): drag and velocity field.
    Errors: max |x - x64| / max |x64| over particles (F, T, S) or nodes (u),
    and the L2 norm ratio for u."""
    import lbmpsm
    from lbmpsm.host import reverse_comm

    storages = ["fp32", "fp16"] + (["bf16"] if "bf16" in lbmpsm.STORAGE else [])
    res = {}

    def susp(storage):
        lt = make(storage)
        mass0 = lt.check()[0]
        mov.host_step(lt, 0)
        for k in range(1, args.acc_steps - 1):
            mov.step(lt, k)
        lt.request_macro()
        mov.host_step(lt, args.acc_steps - 1)
        parts = lt.read_forces(len(g.tag))
        fts = [reverse_comm(a, g.owner, g.swap, nloc)[:nloc] for a in parts]
        u = lt.export_fields(1.0, 1.0, 1.0, as_double=True)[2]
        m = lt.check()[0]
        lt.close()
        return fts, u, (m - mass0) / mass0

    (F64, T64, S64), u64, d64 = susp("fp64")
    block = {"steps": args.acc_steps, "mass_drift_fp64": float(d64)}
    for st in storages:
        (F, T, S), u, d = susp(st)
        block[st] = {"drag": _rel(F, F64), "torque": _rel(T, T64), "stresslet": _rel(S, S64),
                     "velocity_l2": float(np.linalg.norm(u - u64) / np.linalg.norm(u64)),
                     "velocity_max": _rel(u, u64), "mass_drift": float(d)}
    res["suspension"] = block

    # the single-sphere configuration at 10^4 steps
    nu = (0.7 - 0.5) / 3.0
    c2 = dict(dimension=3, boxlo=(0.0, 0.0, 0.0), prd=(128.0,) * 3, periodic=(1, 1, 1), nevery=1,
              Nlc=17, lc=16.0, rho=1.0, nu=nu, Re=0.01 * 16 / nu, tau=0.7, Fext=(1e-6, 0.0, 0.0))
    one = [np.array([1], np.int32), np.array([[64.0, 64.0, 64.0]]), np.zeros((1, 3)),
           np.zeros((1, 3)), np.array([8.0])]

    def sphere(storage):
        lt = lbmpsm.Lattice(**c2, storage=storage)
        lt.step(*one)
        lt.run_fixed(args.acc_c2_steps - 2)
        lt.request_macro()
        fh = lt.step(*one)[0]
        u = lt.export_fields(1.0, 1.0, 1.0, as_double=True)[2]
        lt.close()
        return fh, u

    F64, u64 = sphere("fp64")
    block = {"steps": args.acc_c2_steps, "config": "D3Q19 128^3 periodic, tau 0.7, Fext (1e-6,0,0), "
             "one fixed sphere D=16 at the centre", "drag_fp64": float(F64[0, 0])}
    for st in storages:
        F, u = sphere(st)
        block[st] = {"drag": float(abs(F[0, 0] - F64[0, 0]) / abs(F64[0, 0])),
                     "velocity_l2": float(np.linalg.norm(u - u64) / np.linalg.norm(u64)),
                     "velocity_max": _rel(u, u64)}
    res["single_sphere"] = block
    res["vs"] = ("the plain FP64 GPU path (bit-identical to the CPU oracle's table and within "
                 "1e-12 of its forces on the parity cases and on this workload's first steps)")
    return res


def max_over_ranks(t, world):
    """The largest of the ranks' times (a CUDA tensor over NCCL, a host
    tensor over gloo)."""
    if world <= 1:
        return t
    import torch
    dev = "cuda" if torch.distributed.get_backend() == "nccl" else "cpu"
    v = torch.tensor([t], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(v, op=torch.distributed.ReduceOp.MAX)
    return float(v.item())


def whole_job_mlups(nodes, steps, world, seconds):
    """MLUPS of the whole job: every replica advances its own lattice of
    `nodes` nodes by `steps` steps; `seconds` is the slowest rank's time."""
    return nodes * steps * world / seconds / 1e6


def cpu_baseline(steps, threads=None, single_core=False):
    """The CPU oracle (FP64, the reference's layout and arithmetic) on the same
    workload, all host cores, a bounded number of coupling steps; with
    single_core, also one step on one thread."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liblbmpsm_oracle.so"], check=True)
    threads = threads or os.cpu_count()
    g, nloc = images()
    xs, vs = moving_image_sets(g, nloc)  # the GPU arm's moving images, step by step
    prm = workload_params()
    prm["bc_type"] = 1
    sim = pyoracle.Sim("restatement", **prm)
    sim.set_threads(threads)
    sim.step(g.tag, xs[0], vs[0], g.omega, g.radius, bc=True)  # warm-up (first touch)
    t0 = time.perf_counter()
    for k in range(1, steps + 1):
        j = k % len(xs)
        sim.step(g.tag, xs[j], vs[j], g.omega, g.radius, bc=True)
    dt = time.perf_counter() - t0
    nodes = EDGE ** 3
    out = {"value": round(nodes * steps / dt / 1e6, 3), "unit": "MLUPS", "cores": threads,
           "kind": "port",
           "sample": f"{steps} full coupling steps of the same 256^3 / 2000-sphere workload, "
                     f"spheres moving on the same loops (after 1 warm-up step), FP64, OpenMP "
                     f"over {threads} threads",
           "seconds": round(dt, 2)}
    if single_core:
        sim.set_threads(1)
        t0 = time.perf_counter()
        j = (steps + 1) % len(xs)
        sim.step(g.tag, xs[j], vs[j], g.omega, g.radius, bc=True)
        d1 = time.perf_counter() - t0
        out["single_core"] = {"value": round(nodes / d1 / 1e6, 3), "unit": "MLUPS", "cores": 1,
                              "sample": "1 full coupling step, one thread", "seconds": round(d1, 2)}
    sim.close()
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return None
    # a full 256^3 coupling step takes ~1.3 s on 16 Grace cores: time at most
    # REF_MAX_STEPS of them so that the run ends within a minute or so
    steps = min(max(1, args.steps), REF_MAX_STEPS)
    cb = cpu_baseline(steps)
    nodes = EDGE ** 3
    return {
        "metric": METRIC, "value": cb["value"], "unit": "MLUPS", "n_gpus": world,
        "steps": steps, "warmup": 1,
        "ms_per_step": round(cb["seconds"] / steps * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "impl": "reference",
        "config": {"workload": suspension_workload(EDGE, NSPHERES) + ", FP64 (the reference's "
                                                                      "arithmetic)",
                   "nodes": nodes, "particles": NSPHERES,
                   "motion": f"the same closed loops as the GPU arm (radius {MOVE_AMP}, period "
                             f"{MOVE_SETS} steps)",
                   "parallelism": f"{cb['cores']} host threads"},
        "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": cb["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------- ensemble
ENS_BOXES = 512
ENS_EDGES = (32, 48, 64, 80, 96)
ENS_SEED = 20261204
ENS_LC = 12.0  # lattice units: Nlc = 13, lc = 12 gives dx = 1 in every box


def ensemble_spec(nbox=ENS_BOXES, seed=ENS_SEED):
    """The batched-ensemble workload: per box an edge from ENS_EDGES, tau in
    U[0.6, 1.0], a body force along x in U[1e-7, 1e-5] (lattice units) and
    1-40 fixed spheres of diameter U[8, 14] placed by seeded random
    sequential addition with the periodic minimum image (a box takes as many
    of its drawn spheres as fit within the try budget)."""
    rng = np.random.default_rng(seed)
    spec = []
    for _ in range(nbox):
        e = int(rng.choice(ENS_EDGES))
        tau = float(rng.uniform(0.6, 1.0))
        fx = float(rng.uniform(1e-7, 1e-5))
        want = int(rng.integers(1, 41))
        xs = np.zeros((want, 3))
        rs = np.zeros(want)
        k = tries = 0
        while k < want and tries < 400 * want:
            tries += 1
            d = rng.uniform(8.0, 14.0)
            c = rng.uniform(0.0, e, 3)
            if k:
                dl = xs[:k] - c
                dl -= e * np.round(dl / e)
                if np.any(np.einsum("ij,ij->i", dl, dl) < (d / 2 + rs[:k]) ** 2):
                    continue
            xs[k] = c
            rs[k] = d / 2
            k += 1
        spec.append(dict(edge=e, tau=tau, fx=fx, x=xs[:k].copy(), r=rs[:k].copy()))
    return spec


def ensemble_box_params(e, tau, fx):
    nu = (tau - 0.5) / 3.0
    return dict(dimension=3, boxlo=(0.0, 0.0, 0.0), prd=(float(e),) * 3, periodic=(1, 1, 1),
                Nlc=int(ENS_LC) + 1, lc=ENS_LC, rho=1.0, nu=nu, Re=U_WALL * ENS_LC / nu, tau=tau,
                Fext=(fx, 0.0, 0.0))


def ensemble_images(boxes):
    """Per-box periodic images, concatenated with the box of each image."""
    from lbmpsm.host import Domain, ghost_images
    cols = {k: [] for k in ("box", "tag", "x", "v", "omega", "radius")}
    nloc = []
    for b, sb in enumerate(boxes):
        e = sb["edge"]
        n = len(sb["r"])
        dom = Domain(3, (0.0, 0.0, 0.0), (float(e),) * 3, (1, 1, 1))
        g = ghost_images(dom, 7.0 + 3.0, np.arange(1, n + 1), sb["x"], np.zeros((n, 3)),
                         np.zeros((n, 3)), sb["r"])
        cols["box"].append(np.full(len(g.tag), b, np.int32))
        for k, a in (("tag", g.tag), ("x", g.x), ("v", g.v), ("omega", g.omega), ("radius", g.radius)):
            cols[k].append(a)
        nloc.append(n)
    return {k: np.concatenate(v) for k, v in cols.items()}, nloc


def run_ensemble(args):
    """Aggregate MLUPS of the batched-ensemble workload: one ensemble per
    edge class, all replayed concurrently (one stream each) as CUDA graphs;
    then FP32 against FP64 drag on a subset of boxes."""
    import torch

    import lbmpsm

    spec = ensemble_spec(args.boxes)
    classes = {}
    for b, sb in enumerate(spec):
        classes.setdefault(sb["edge"], []).append(b)
    K, W = args.steps, args.warmup

    def build(boxes, storage):
        ens = lbmpsm.Ensemble([ensemble_box_params(sb["edge"], sb["tau"], sb["fx"]) for sb in boxes],
                              storage=storage)
        img, nloc = ensemble_images(boxes)
        ens.step(img["box"], img["tag"], img["x"], img["v"], img["omega"], img["radius"])
        return ens, img, nloc

    ens = {}
    nodes = 0
    for e, ids in sorted(classes.items()):
        ens[e] = build([spec[b] for b in ids], args.storage)
        nodes += len(ids) * e ** 3
    # every edge class is one ensemble; the group steps all of them as one
    # CUDA graph (one launch per step for all boxes)
    grp = lbmpsm.Group([ens[e][0] for e in sorted(ens)])
    grp.run_fixed(max(W, 12))  # the group's tuner takes 8 of these steps
    st = torch.cuda.ExternalStream(grp.stream)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        t_a = time.monotonic()
        e0.record(st)
        grp.run_fixed(K)
        e1.record(st)
        e1.synchronize()
        clk.mark(t_a, time.monotonic())
    t = e0.elapsed_time(e1) / 1e3
    launches = grp.collide_launches
    tune = grp.tune_ms
    # the collide alone: lattice-only steps (no images: the group's graph is
    # the collide launch and nothing else), for the roofline
    for e in sorted(ens):
        en = ens[e][0]
        z3 = np.zeros((0, 3))
        en.step(np.zeros(0, np.int32), np.zeros(0, np.int32), z3, z3, z3, np.zeros(0))
    grp.run_fixed(2)
    torch.cuda.synchronize()
    e0.record(st)
    grp.run_fixed(K)
    e1.record(st)
    e1.synchronize()
    t_col = e0.elapsed_time(e1) / 1e3 / K
    grp.close()
    peak, peak_kind = measured_peak_gbs()
    bpn = BYTES_PER_NODE[args.storage]
    achieved = bpn * nodes / t_col / 1e9
    per_class = {str(e): {"boxes": len(classes[e]), "nodes": len(classes[e]) * e ** 3}
                 for e in sorted(classes)}
    for e in list(ens):
        ens[e][0].close()
    del ens

    # accuracy: FP32 (or FP16) against FP64 drag per box on a subset, acc_steps steps
    acc = None
    if args.acc_boxes > 0:
        errs = []
        for e, ids in sorted(classes.items()):
            sub = [spec[b] for b in ids[:args.acc_boxes]]
            drag = {}
            for storage in (args.storage, "fp64"):
                en, img, nloc = build(sub, storage)
                en.run_fixed(args.acc_steps - 2)
                fh = en.step(img["box"], img["tag"], img["x"], img["v"], img["omega"], img["radius"])[0]
                en.close()
                # per box: total x-drag of its local spheres (images are box-major, locals first)
                out, k = [], 0
                for bi, n in enumerate(nloc):
                    m = int(np.sum(img["box"] == bi))
                    out.append(fh[k:k + n, 0].sum())
                    k += m
                drag[storage] = np.array(out)
            errs.extend(np.abs(drag[args.storage] - drag["fp64"]) / np.abs(drag["fp64"]))
        errs = np.array(errs)
        acc = {"boxes": int(len(errs)), "steps": args.acc_steps, "vs": "FP64 GPU path",
               "drag_rel_err_max": float(errs.max()), "drag_rel_err_median": float(np.median(errs))}
    return {
        "metric": "batched ensemble aggregate MLUPS (D3Q19 PSM, 1 GB300)",
        "value": round(nodes * K / t / 1e6, 1), "unit": "MLUPS", "n_gpus": 1, "steps": K,
        "warmup": W, "ms_per_step": round(t / K * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{args.boxes} periodic D3Q19 boxes, edges in {list(ENS_EDGES)}, "
                               "tau U[0.6,1], Fx U[1e-7,1e-5], 1-40 fixed spheres D U[8,14] "
                               "(seeded RSA)", "nodes": nodes, "storage": args.storage,
                   "classes": per_class,
                   "launch": "one ensemble per edge class; the classes stepped as one group: "
                             "one CUDA graph launch per step for all boxes; the classes' maps and "
                             "reductions as concurrent branches around the collide, which the "
                             "group's tuner runs as ONE launch for every box or as one launch "
                             "per class, whichever it timed faster (collide_launches_per_step, "
                             "group_tuner_ms_per_step)"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None,
                     "kernel": "collide_multi_kernel (one launch for the boxes of every size)"
                               if launches == 1 else "collide_pipe_kernel (one launch per edge class)",
                     "algorithmic_bytes_per_node": bpn, "collide_ms": round(t_col * 1e3, 4),
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "collide_launches_per_step": launches,
        "group_tuner_ms_per_step": {"per_class_launches": round(tune[0], 4),
                                    "one_launch": round(tune[1], 4)},
        "accuracy": acc, "clocks": clk.summary(),
    }


ADJ_EDGE, ADJ_N, ADJ_D, ADJ_TAU, ADJ_FX, ADJ_SEED = 96, 8, 12.0, 0.7, 1e-6, 2024
ADJ_T, ADJ_K = 2000, 100


def adjoint_params(tau=ADJ_TAU, fx=ADJ_FX, edge=ADJ_EDGE):
    nu = (tau - 0.5) / 3.0
    return dict(dimension=3, boxlo=(0.0, 0.0, 0.0), prd=(float(edge),) * 3, periodic=(1, 1, 1),
                nevery=1, Nlc=int(ADJ_D) + 1, lc=ADJ_D, rho=1.0, nu=nu, Re=0.01 * ADJ_D / nu,
                tau=tau, Fext=(fx, 0.0, 0.0))


def adjoint_images(x=None, edge=ADJ_EDGE):
    """8 fixed spheres of diameter 12 by seeded random sequential addition
    (minimum image, gap >= 2 lattice units) and their periodic ghost images."""
    from lbmpsm.host import Domain, ghost_images
    r = ADJ_D / 2
    if x is None:
        rng = np.random.default_rng(ADJ_SEED)
        x = np.zeros((ADJ_N, 3))
        k = 0
        while k < ADJ_N:
            c = rng.uniform(0.0, edge, 3)
            dlt = x[:k] - c
            dlt -= edge * np.round(dlt / edge)
            if k and np.min(np.einsum("ij,ij->i", dlt, dlt)) < (2 * r + 2.0) ** 2:
                continue
            x[k] = c
            k += 1
    dom = Domain(3, (0.0, 0.0, 0.0), (float(edge),) * 3, (1, 1, 1))
    n = len(x)
    return ghost_images(dom, r + 3.0, np.arange(1, n + 1), x, np.zeros((n, 3)), np.zeros((n, 3)),
                        np.full(n, r)), x


def adjoint_J(img, T, t0, **kw):
    """J through the plain step API: steps before the window as one graph
    replay, the window step by step with the forces read back."""
    import lbmpsm
    lat = lbmpsm.Lattice(**adjoint_params(**kw), storage="fp64")
    a = (img.tag, img.x, img.v, img.omega, img.radius)
    lat.step(*a)
    lat.run_fixed(t0 - 2)
    J = 0.0
    for _ in range(t0, T + 1):
        J += float(lat.step(*a)[0][:, 0].sum())
    lat.close()
    return J / (T - t0 + 1)


def run_adjoint(args):
    """Cost of the adjoint sweep against the forward steps it differentiates,
    and its gradient against central finite differences."""
    import torch

    import lbmpsm
    from lbmpsm.host import reverse_comm

    E, T, K = args.adj_edge, args.adj_steps, args.adj_checkpoint
    t0 = T // 2
    img, x = adjoint_images(edge=E)
    a = (img.tag, img.x, img.v, img.omega, img.radius)
    prm = adjoint_params(edge=E)
    # forward: the same FP64 steps replayed as a CUDA graph
    fwd = lbmpsm.Lattice(**prm, storage="fp64")
    fwd.step(*a)
    fwd.synchronize()
    st = torch.cuda.ExternalStream(fwd.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    fwd.run_fixed(T - 1)
    e1.record(st)
    e1.synchronize()
    t_fwd = e0.elapsed_time(e1) / 1e3 * T / (T - 1)
    fwd.close()
    lat = lbmpsm.Lattice(**prm, storage="fp64")
    with ClockSampler(0) as clk:
        t_a = time.monotonic()
        t = time.perf_counter()
        R = lat.adjoint_drag(*a, T, t0, T, checkpoint_every=K)
        t_adj = time.perf_counter() - t
        clk.mark(t_a, time.monotonic())
    lat.close()
    grad = reverse_comm(R["dx"], img.owner, img.swap, img.nlocal)[:img.nlocal]
    adj = {"dtau": R["dtau"], "dFx": float(R["dFext"][0]), "dx0": float(grad[0, 0])}
    fd, rel = None, None
    h, hF = 1e-4, 1e-10
    if not args.no_fd:
        fd = {}
        fd["dtau"] = (adjoint_J(img, T, t0, tau=ADJ_TAU + h, edge=E) -
                      adjoint_J(img, T, t0, tau=ADJ_TAU - h, edge=E)) / (2 * h)
        fd["dFx"] = (adjoint_J(img, T, t0, fx=ADJ_FX + hF, edge=E) -
                     adjoint_J(img, T, t0, fx=ADJ_FX - hF, edge=E)) / (2 * hF)
        xp, xm = x.copy(), x.copy()
        xp[0, 0] += h
        xm[0, 0] -= h
        fd["dx0"] = (adjoint_J(adjoint_images(xp, E)[0], T, t0, edge=E) -
                     adjoint_J(adjoint_images(xm, E)[0], T, t0, edge=E)) / (2 * h)
        rel = {k: abs(adj[k] - fd[k]) / abs(fd[k]) for k in fd}
    nodes = E ** 3
    return {
        "metric": "adjoint cost: d(time-averaged drag)/d(tau, Fext, 24 centres) vs forward, 1 GB300",
        "value": round(t_adj / t_fwd, 3), "unit": "x forward time", "n_gpus": 1, "steps": T,
        "warmup": 1, "ms_per_step": round(t_adj / T * 1e3, 4), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"D3Q19 {E}^3 periodic, tau 0.7, Fext (1e-6,0,0), 8 fixed spheres "
                               f"D=12 (seeded RSA), J = x-drag averaged over steps {t0}-{T}, "
                               f"checkpoints every {K} steps", "nodes": nodes,
                   "images": int(len(img.tag)), "storage": "fp64"},
        "forward_s": round(t_fwd, 4), "adjoint_s": round(t_adj, 4),
        "adjoint_mlups": round(nodes * T / t_adj / 1e6, 1),
        "J": R["J"], "gradient": adj, "finite_difference": fd, "rel_err_vs_fd": rel,
        "fd_steps": {"tau": h, "Fext": hF, "centre": h},
        "clocks": clk.summary(),
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the developed-flow accuracy runs against FP64")
    ap.add_argument("--acc-c2-steps", type=int, default=10000,
                    help="steps of the single-sphere accuracy run")
    ap.add_argument("--edge", type=int, default=EDGE, help="lattice edge (profiling cases)")
    ap.add_argument("--nspheres", type=int, default=NSPHERES)
    ap.add_argument("--storage", choices=["fp32", "fp16", "bf16"], default="fp32")
    ap.add_argument("--workload", choices=["suspension", "ensemble", "adjoint"], default="suspension",
                    help="suspension: the headline line; ensemble: the batched-box workload; "
                         "adjoint: the drag-sensitivity sweep")
    ap.add_argument("--boxes", type=int, default=ENS_BOXES)
    ap.add_argument("--acc-boxes", type=int, default=8, help="ensemble: boxes per class compared with FP64")
    ap.add_argument("--acc-steps", type=int, default=2000,
                    help="steps of the accuracy runs (suspension; ensemble boxes)")
    ap.add_argument("--adj-edge", type=int, default=ADJ_EDGE, help="adjoint: lattice edge")
    ap.add_argument("--adj-steps", type=int, default=ADJ_T, help="adjoint: steps (window: 2nd half)")
    ap.add_argument("--adj-checkpoint", type=int, default=ADJ_K)
    ap.add_argument("--no-fd", action="store_true", help="adjoint: skip the finite differences")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.workload == "ensemble":
        out = run_ensemble(args) if rank == 0 else None
    elif args.workload == "adjoint":
        out = run_adjoint(args) if rank == 0 else None
    elif args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        out = run_ours(args, rank, world)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
