"""ctypes binding of the CPU oracles (TEST INFRASTRUCTURE ONLY).

Loads either the plain-C restatement (``liblbmpsm_oracle.so``) or the
reference's own sources built with stub headers (``_ref/libref_oracle.so``);
both export the interface of ``lbmpsm_oracle.h``.  Only the tests, the smoke
check and bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RESTATEMENT_SO = os.path.join(HERE, "liblbmpsm_oracle.so")
REFERENCE_SO = os.path.join(HERE, "_ref", "libref_oracle.so")
# the reference checkout beside this repository, unless LBMPSM_REFERENCE_SRC names it
REFERENCE_SRC = os.environ.get("LBMPSM_REFERENCE_SRC",
                               os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference", "src"))


class OrcParams(C.Structure):
    _fields_ = [
        ("dimension", C.c_int),
        ("boxlo", C.c_double * 3),
        ("prd", C.c_double * 3),
        ("periodic", C.c_int * 3),
        ("nevery", C.c_int),
        ("Nlc", C.c_int),
        ("lc", C.c_double),
        ("rho", C.c_double),
        ("nu", C.c_double),
        ("Re", C.c_double),
        ("tau", C.c_double),
        ("Fext", C.c_double * 3),
        ("bc_type", C.c_int),
    ]


class OrcInfo(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("q", C.c_int),
        ("dx", C.c_double), ("Uc", C.c_double), ("u_lb", C.c_double), ("tc", C.c_double),
        ("dt_d", C.c_double), ("forceFactor", C.c_double), ("torqueFactor", C.c_double),
        ("volumeForceFactor", C.c_double), ("dt_dem", C.c_double), ("Ma", C.c_double),
        ("F_lbm", C.c_double * 3),
    ]


_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


def build(reference: bool = False) -> None:
    """Compile the restatement (and, when the reference sources exist, the reference build)."""
    subprocess.run(["make", "-s", "-C", HERE, "liblbmpsm_oracle.so"], check=True)
    if reference and os.path.isdir(REFERENCE_SRC):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFERENCE_SRC={REFERENCE_SRC}"], check=True)


def _load(path: str) -> C.CDLL:
    lib = C.CDLL(path)
    lib.orc_create.argtypes = [C.POINTER(OrcParams), C.POINTER(C.c_void_p)]
    lib.orc_create.restype = C.c_int
    lib.orc_destroy.argtypes = [C.c_void_p]
    lib.orc_get_info.argtypes = [C.c_void_p, C.POINTER(OrcInfo)]
    lib.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
    for name in ("orc_step",):
        getattr(lib, name).argtypes = [C.c_void_p, C.c_int, _I, _D, _D, _D, _D, _D, _D, _D]
    lib.orc_map.argtypes = [C.c_void_p, C.c_int, _I, _D, _D, _D, _D]
    lib.orc_collide_stream.argtypes = [C.c_void_p]
    lib.orc_reduce.argtypes = [C.c_void_p, C.c_int, _I, _D, _D, _D, _D, _D]
    lib.orc_apply_bc.argtypes = [C.c_void_p]
    lib.orc_get_f.argtypes = [C.c_void_p, _D]
    lib.orc_set_f.argtypes = [C.c_void_p, _D]
    lib.orc_get_macro.argtypes = [C.c_void_p, _D, _D]
    lib.orc_get_pdata.argtypes = [C.c_void_p, _I, _D, _D, _D]
    lib.orc_export_fields.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, _D, _D, _D]
    lib.orc_make_ghosts.argtypes = [C.c_int, _D, _D, _I, C.c_double, C.c_int, C.c_int,
                                    _I, _D, _D, _D, _D, _I, _I]
    lib.orc_reverse_comm.argtypes = [C.c_int, C.c_int, _I, _I, C.c_int, _D]
    return lib


_LIBS: dict[str, C.CDLL] = {}


def library(kind: str = "restatement") -> C.CDLL:
    path = RESTATEMENT_SO if kind == "restatement" else REFERENCE_SO
    if path not in _LIBS:
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library missing: {path} (run oracle/Makefile)")
        _LIBS[path] = _load(path)
    return _LIBS[path]


def _p(a: np.ndarray, t=_D):
    return a.ctypes.data_as(t)


class Sim:
    """One oracle lattice (a `fix lbm-psm` instance on one rank)."""

    def __init__(self, kind: str = "restatement", **params):
        self.lib = library(kind)
        p = OrcParams()
        p.dimension = params.get("dimension", 3)
        p.boxlo = (C.c_double * 3)(*params.get("boxlo", (0.0, 0.0, 0.0)))
        p.prd = (C.c_double * 3)(*params["prd"])
        p.periodic = (C.c_int * 3)(*params.get("periodic", (1, 1, 1)))
        p.nevery = params.get("nevery", 1)
        p.Nlc = params["Nlc"]
        p.lc = params["lc"]
        p.rho = params.get("rho", 1.0)
        p.nu = params["nu"]
        p.Re = params["Re"]
        p.tau = params.get("tau", 0.7)
        p.Fext = (C.c_double * 3)(*params.get("Fext", (0.0, 0.0, 0.0)))
        p.bc_type = params.get("bc_type", 0)
        self.params = params
        h = C.c_void_p()
        rc = self.lib.orc_create(C.byref(p), C.byref(h))
        if rc != 0:
            raise ValueError(f"orc_create failed with code {rc}")
        self.h = h
        info = OrcInfo()
        self.lib.orc_get_info(self.h, C.byref(info))
        self.info = info
        self.shape = (info.nx, info.ny, info.nz)
        self.q = info.q

    def close(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    __del__ = close

    def set_threads(self, n: int):
        self.lib.orc_set_threads(self.h, int(n))

    @staticmethod
    def _parts(tag, x, v, omega, radius):
        tag = np.ascontiguousarray(tag, dtype=np.int32)
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        omega = np.ascontiguousarray(omega, dtype=np.float64).reshape(-1, 3)
        radius = np.ascontiguousarray(radius, dtype=np.float64)
        return tag, x, v, omega, radius

    def step(self, tag, x, v, omega, radius, bc: bool = False):
        tag, x, v, omega, radius = self._parts(tag, x, v, omega, radius)
        n = len(tag)
        fh = np.zeros((n, 3)); th = np.zeros((n, 3)); S = np.zeros((n, 6))
        rc = self.lib.orc_step(self.h, n, _p(tag, _I), _p(x), _p(v), _p(omega), _p(radius),
                               _p(fh), _p(th), _p(S))
        if rc:
            raise RuntimeError(f"orc_step failed {rc}")
        if bc:
            self.lib.orc_apply_bc(self.h)
        return fh, th, S

    def map(self, tag, x, v, omega, radius):
        tag, x, v, omega, radius = self._parts(tag, x, v, omega, radius)
        self.lib.orc_map(self.h, len(tag), _p(tag, _I), _p(x), _p(v), _p(omega), _p(radius))

    def collide_stream(self):
        self.lib.orc_collide_stream(self.h)

    def apply_bc(self):
        self.lib.orc_apply_bc(self.h)

    def populations(self) -> np.ndarray:
        f = np.empty(self.shape + (self.q,), dtype=np.float64)
        self.lib.orc_get_f(self.h, _p(f))
        return f

    def set_populations(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.float64)
        self.lib.orc_set_f(self.h, _p(f))

    def macro(self):
        rho = np.empty(self.shape); u = np.empty(self.shape + (3,))
        self.lib.orc_get_macro(self.h, _p(rho), _p(u))
        return rho, u

    def pdata(self):
        N = int(np.prod(self.shape))
        ids = np.empty((N, 2), dtype=np.int32); eps = np.empty((N, 2))
        us = np.empty((N, 6)); F = np.empty((N, 6))
        self.lib.orc_get_pdata(self.h, _p(ids, _I), _p(eps), _p(us), _p(F))
        s = self.shape
        return ids.reshape(s + (2,)), eps.reshape(s + (2,)), us.reshape(s + (6,)), F.reshape(s + (6,))

    def export_fields(self, B0=1.0, rho0=1.0, u0=1.0):
        nx, ny, nz = self.shape
        npts = (nx - 2) * (ny - 2) * (nz - 2 if self.params.get("dimension", 3) == 3 else 1)
        solid = np.empty(npts); rho = np.empty(npts); u = np.empty((npts, 3))
        n = self.lib.orc_export_fields(self.h, B0, rho0, u0, _p(solid), _p(rho), _p(u))
        assert n == npts
        return solid, rho, u


def make_ghosts(dimension, boxlo, prd, periodic, cutghost, tag, x, v, omega, radius,
                max_images=None, kind="restatement"):
    """LAMMPS single-rank ghost images (locals first, then ghosts in swap order)."""
    lib = library(kind)
    nloc = len(tag)
    cap = max_images or nloc * 27 + 8
    T = np.zeros(cap, dtype=np.int32); X = np.zeros((cap, 3)); V = np.zeros((cap, 3))
    W = np.zeros((cap, 3)); R = np.zeros(cap)
    owner = np.zeros(cap, dtype=np.int32); swap = np.zeros(cap, dtype=np.int32)
    T[:nloc] = tag; X[:nloc] = np.asarray(x).reshape(-1, 3); V[:nloc] = np.asarray(v).reshape(-1, 3)
    W[:nloc] = np.asarray(omega).reshape(-1, 3); R[:nloc] = radius
    bl = np.ascontiguousarray(boxlo, dtype=np.float64); pr = np.ascontiguousarray(prd, dtype=np.float64)
    pe = np.ascontiguousarray(periodic, dtype=np.int32)
    n = lib.orc_make_ghosts(dimension, _p(bl), _p(pr), _p(pe, _I), float(cutghost), nloc, cap,
                            _p(T, _I), _p(X), _p(V), _p(W), _p(R), _p(owner, _I), _p(swap, _I))
    if n < 0:
        raise ValueError("too many ghost images")
    return dict(tag=T[:n].copy(), x=X[:n].copy(), v=V[:n].copy(), omega=W[:n].copy(),
                radius=R[:n].copy(), owner=owner[:n].copy(), swap=swap[:n].copy(), nlocal=nloc)


def write_vti(folder, name, timestep, binary, use_double, dimension, local, origin, dx, solid,
              rho, u):
    """The reference's VTI piece and PVTI master file for these fields (the C
    restatement in vti_oracle.c; solid, rho one double per interior node, u
    three)."""
    lib = library("restatement")
    fn = lib.orc_write_vti
    fn.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, _I, _D, C.c_double,
                   _D, _D, _D]
    loc = np.ascontiguousarray(local, dtype=np.int32)
    org = np.ascontiguousarray(origin, dtype=np.float64)
    solid = np.ascontiguousarray(solid, dtype=np.float64)
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    rc = fn(str(folder).encode(), name.encode(), int(timestep), int(binary), int(use_double),
            int(dimension), _p(loc, _I), _p(org), float(dx), _p(solid), _p(rho), _p(u))
    if rc != 0:
        raise OSError("orc_write_vti failed")


def reverse_comm(vals: np.ndarray, owner, swap, nlocal, kind="restatement") -> np.ndarray:
    lib = library(kind)
    vals = np.ascontiguousarray(vals, dtype=np.float64).copy()
    n, width = vals.shape
    owner = np.ascontiguousarray(owner, dtype=np.int32); swap = np.ascontiguousarray(swap, dtype=np.int32)
    lib.orc_reverse_comm(n, nlocal, _p(owner, _I), _p(swap, _I), width, _p(vals))
    return vals


class FixOracle:
    """fix_LBM_PSM on one process (TEST INFRASTRUCTURE): the coupling
    bookkeeping of src/fix_LBM_PSM.cpp around an oracle lattice.

    init (src/fix_LBM_PSM.cpp:104-177): the lattice, and the DEM timestep
    update->dt = phys_time(1)/nevery (:120), returned.
    post_force (src/fix_LBM_PSM.cpp:181-266), given the step number and the
    LAMMPS images (locals first, then ghosts, with the owner/swap bookkeeping
    of make_ghosts) and the atoms' f and torque arrays (n x 3, modified in
    place):
      * ntimestep % nevery != 0: the stored hydrodynamic force and torque are
        added to the local atoms (:183-196);
      * else: one coupling step (map, halo, collide, per-image F/T/S); locals
        f += fh, ghosts f = fh (the same for torque); the per-image F/T are
        stored for the steps in between (:252-257); the stresslets are summed
        as v_tally would (:259); then reverse_comm adds the ghost rows into
        their owners (:263).
    apply_bc is fix_LBM_PSM_BC::post_force, which runs on the same steps
    (src/fix_LBM_PSM_BC.cpp:151-156).
    """

    def __init__(self, kind: str = "restatement", **params):
        self.params = params
        self.nevery = int(params.get("nevery", 1))
        self.kind = kind
        self.sim = None
        self.hydrodynamicInteractions = np.zeros((0, 6))
        self.virial = np.zeros(6)

    def init(self) -> float:
        if self.sim is not None:
            self.sim.close()
        self.sim = Sim(self.kind, **self.params)
        self.hydrodynamicInteractions = np.zeros((0, 6))
        return self.sim.info.dt_dem

    def post_force(self, ntimestep: int, img: dict, f: np.ndarray, torque: np.ndarray):
        nl = img["nlocal"]
        if ntimestep % self.nevery:
            hi = self.hydrodynamicInteractions
            for i in range(nl):
                f[i] += hi[i, :3]
                torque[i] += hi[i, 3:]
            return None
        fh, th, S = self.sim.step(img["tag"], img["x"], img["v"], img["omega"], img["radius"])
        n = len(img["tag"])
        for i in range(n):
            if i < nl:
                f[i] += fh[i]
                torque[i] += th[i]
            else:
                f[i] = fh[i]
                torque[i] = th[i]
        self.hydrodynamicInteractions = np.concatenate([fh, th], axis=1)
        self.virial = S.sum(axis=0)
        f[:] = reverse_comm(f, img["owner"], img["swap"], nl, self.kind)
        torque[:] = reverse_comm(torque, img["owner"], img["swap"], nl, self.kind)
        return fh, th, S

    def apply_bc(self, ntimestep: int):
        if ntimestep % self.nevery:
            return
        self.sim.apply_bc()

    def close(self):
        if self.sim is not None:
            self.sim.close()
            self.sim = None
