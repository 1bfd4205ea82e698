"""Python binding of liblbmpsm_gb300.so (the C ABI in include/lbmpsm.h).

``Lattice`` is one ``fix lbm-psm`` lattice resident on a GPU.  Its methods map
one-to-one onto the library's entry points, which replace the reference's
call sites (timnajuch/LAMMPS-LBM-PSM):

    Lattice(...)          fix_LBM_PSM::init              src/fix_LBM_PSM.cpp:104-177
    Lattice.set_bc(kw)    fix lbm-psm-bc keyword + init  src/fix_LBM_PSM_BC.cpp:16-39,145-148
    Lattice.step(...)     LBM branch of post_force        src/fix_LBM_PSM.cpp:197-229
    Lattice.apply_bc()    fix_LBM_PSM_BC::post_force     src/fix_LBM_PSM_BC.cpp:151-402
    Lattice.export_fields execute_write_vti field read   src/fix_LBM_PSM_writeVTI.h:146-169

There is no CPU fallback: constructing a ``Lattice`` without the built library
or without a CUDA device raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .host import FixLbmPsm, FixLbmPsmBC, FixLbmPsmVTI, LammpsError, ghost_images, reverse_comm  # noqa: F401

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "liblbmpsm_gb300.so")

OK = 0
ERR_ARG, ERR_MACH, ERR_GRID, ERR_NOMEM, ERR_CUDA, ERR_STATE, ERR_CAPACITY, ERR_NUMERIC, ERR_TIMEOUT = (
    -1, -2, -3, -4, -5, -6, -7, -8, -9)
STORAGE = {"fp64": 0, "fp32": 1, "fp16": 2, "bf16": 3}
BC = {"none": 0, "shear": 1, "xFlow": 2, "channel": 3, "channel-velIn-pressOut": 4, "closedBox": 5}
WEIGHTING = {"reference": 0, "noble-torczynski": 1}
TUNING = {"auto": 0, "default": 1}  # LBMPSM_TUNE_*

SYMBOLS = (
    "lbmpsm_create", "lbmpsm_destroy", "lbmpsm_last_error", "lbmpsm_get_info", "lbmpsm_set_bc",
    "lbmpsm_step", "lbmpsm_step_device", "lbmpsm_apply_bc", "lbmpsm_request_macro",
    "lbmpsm_export_fields", "lbmpsm_get_populations", "lbmpsm_set_populations",
    "lbmpsm_get_particle_table", "lbmpsm_check", "lbmpsm_synchronize", "lbmpsm_stream",
    "lbmpsm_host_direct",
    "lbmpsm_run_fixed", "lbmpsm_read_forces", "lbmpsm_export_fields_static",
    "lbmpsm_create_batch", "lbmpsm_step_batch", "lbmpsm_select_box",
    "lbmpsm_adjoint_drag", "lbmpsm_tangent_drag",
    "lbmpsm_group_create", "lbmpsm_group_run_fixed", "lbmpsm_group_stream",
    "lbmpsm_group_last_error", "lbmpsm_group_destroy", "lbmpsm_group_collide_launches",
    "lbmpsm_group_tune_ms",
)


class LbmPsmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class FixParams(C.Structure):
    _fields_ = [
        ("dimension", C.c_int), ("boxlo", C.c_double * 3), ("prd", C.c_double * 3),
        ("periodic", C.c_int * 3), ("nevery", C.c_int), ("Nlc", C.c_int), ("lc", C.c_double),
        ("rho", C.c_double), ("nu", C.c_double), ("Re", C.c_double), ("tau", C.c_double),
        ("Fext", C.c_double * 3),
    ]


class Options(C.Structure):
    _fields_ = [
        ("storage", C.c_int), ("device", C.c_int), ("max_images", C.c_int),
        ("max_radius", C.c_double), ("psm_weighting", C.c_int), ("collide_tuning", C.c_int),
    ]


class Info(C.Structure):
    _fields_ = [
        ("dimension", C.c_int), ("q", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("local", C.c_int * 3), ("storage_dims", C.c_int * 3),
        ("dx", C.c_double), ("Uc", C.c_double), ("u_lb", C.c_double), ("tc", C.c_double),
        ("dt_d", C.c_double), ("forceFactor", C.c_double), ("torqueFactor", C.c_double),
        ("volumeForceFactor", C.c_double), ("dt_dem", C.c_double), ("Ma", C.c_double),
        ("F_lbm", C.c_double * 3), ("steps", C.c_int64), ("device_bytes", C.c_size_t),
        ("collide_stages", C.c_int), ("collide_blocks", C.c_int), ("collide_tune_ms", C.c_float * 4),
    ]


_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_lib: C.CDLL | None = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"liblbmpsm_gb300.so not found at {path}: run lammps-lbm-psm_gb300/build.py")
    lib = C.CDLL(path)
    H = C.c_void_p
    lib.lbmpsm_create.argtypes = [C.POINTER(FixParams), C.POINTER(Options), C.POINTER(H)]
    lib.lbmpsm_destroy.argtypes = [H]
    lib.lbmpsm_destroy.restype = None
    lib.lbmpsm_last_error.argtypes = [H]
    lib.lbmpsm_last_error.restype = C.c_char_p
    lib.lbmpsm_get_info.argtypes = [H, C.POINTER(Info)]
    lib.lbmpsm_set_bc.argtypes = [H, C.c_int]
    lib.lbmpsm_step.argtypes = [H, C.c_int, _I, _D, _D, _D, _D, _D, _D, _D]
    lib.lbmpsm_step_device.argtypes = [H, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.lbmpsm_apply_bc.argtypes = [H]
    lib.lbmpsm_request_macro.argtypes = [H]
    lib.lbmpsm_export_fields.argtypes = [H, C.c_int, C.c_double, C.c_double, C.c_double,
                                         C.c_void_p, C.c_void_p, C.c_void_p]
    lib.lbmpsm_get_populations.argtypes = [H, _D]
    lib.lbmpsm_set_populations.argtypes = [H, _D]
    lib.lbmpsm_get_particle_table.argtypes = [H, _I, _D, _D]
    lib.lbmpsm_check.argtypes = [H, _D, _D]
    lib.lbmpsm_synchronize.argtypes = [H]
    lib.lbmpsm_stream.argtypes = [H]
    lib.lbmpsm_stream.restype = C.c_void_p
    lib.lbmpsm_host_direct.argtypes = [H]
    lib.lbmpsm_run_fixed.argtypes = [H, C.c_int]
    lib.lbmpsm_read_forces.argtypes = [H, C.c_int, _D, _D, _D]
    lib.lbmpsm_export_fields_static.argtypes = [H, C.c_int, C.c_double, C.c_double, C.c_double,
                                                C.c_void_p, C.c_void_p, C.c_void_p]
    lib.lbmpsm_create_batch.argtypes = [C.c_int, C.POINTER(FixParams), C.POINTER(Options),
                                        C.POINTER(H)]
    lib.lbmpsm_step_batch.argtypes = [H, C.c_int, _I, _I, _D, _D, _D, _D, _D, _D, _D]
    lib.lbmpsm_select_box.argtypes = [H, C.c_int]
    # the per-step call by raw addresses (its own function object, so that the
    # typed binding above stays as it is): the cheapest conversion per call
    _lib_step_addr = lib["lbmpsm_step"]
    _lib_step_addr.argtypes = [H, C.c_int] + [C.c_void_p] * 8
    lib.step_by_address = _lib_step_addr
    lib.lbmpsm_adjoint_drag.argtypes = [H, C.c_int, _I, _D, _D, _D, _D, C.c_int, C.c_int, C.c_int,
                                        _D, C.c_int, C.c_double, _D, _D, _D, _D, _D]
    lib.lbmpsm_tangent_drag.argtypes = [H, C.c_int, _I, _D, _D, _D, _D, C.c_int, C.c_int, C.c_int,
                                        _D, C.c_double, C.c_double, _D, _D, _D, _D]
    lib.lbmpsm_group_create.argtypes = [C.POINTER(H), C.c_int, C.POINTER(H)]
    lib.lbmpsm_group_run_fixed.argtypes = [H, C.c_int]
    lib.lbmpsm_group_stream.argtypes = [H]
    lib.lbmpsm_group_stream.restype = C.c_void_p
    lib.lbmpsm_group_last_error.argtypes = [H]
    lib.lbmpsm_group_last_error.restype = C.c_char_p
    lib.lbmpsm_group_destroy.argtypes = [H]
    lib.lbmpsm_group_destroy.restype = None
    lib.lbmpsm_group_collide_launches.argtypes = [H]
    lib.lbmpsm_group_tune_ms.argtypes = [H, C.POINTER(C.c_float)]
    _lib = lib
    return lib


def _p(a, t=_D):
    return a.ctypes.data_as(t)


class Lattice:
    """One LBM-PSM lattice on a GPU (a `fix lbm-psm` instance)."""

    def __init__(self, *, dimension: int = 3, boxlo=(0.0, 0.0, 0.0), prd, periodic=(1, 1, 1),
                 nevery: int = 1, Nlc: int, lc: float, rho: float = 1.0, nu: float, Re: float,
                 tau: float = 0.7, Fext=(0.0, 0.0, 0.0), storage: str = "fp64", device: int = 0,
                 max_images: int = 0, max_radius: float = 0.0, weighting: str = "reference",
                 bc: str | int = "none", collide_tuning: str = "auto"):
        self.lib = load()
        p = FixParams()
        p.dimension = dimension
        p.boxlo = (C.c_double * 3)(*boxlo)
        p.prd = (C.c_double * 3)(*prd)
        p.periodic = (C.c_int * 3)(*[int(v) for v in periodic])
        p.nevery, p.Nlc, p.lc, p.rho, p.nu, p.Re, p.tau = nevery, Nlc, lc, rho, nu, Re, tau
        p.Fext = (C.c_double * 3)(*Fext)
        o = Options()
        o.storage = STORAGE[storage]
        o.device = device
        o.max_images = max_images
        o.max_radius = max_radius
        o.psm_weighting = WEIGHTING[weighting]
        o.collide_tuning = TUNING[collide_tuning]
        h = C.c_void_p()
        rc = self.lib.lbmpsm_create(C.byref(p), C.byref(o), C.byref(h))
        if rc != OK:
            raise LbmPsmError(rc, self.lib.lbmpsm_last_error(None).decode())
        self.h = h
        self.dimension = dimension
        self.storage = storage
        self.origin = (float(boxlo[0]), float(boxlo[1]), float(boxlo[2]) if dimension == 3 else 0.0)
        self.info = self.get_info()
        self.local = tuple(self.info.local)
        self.q = self.info.q
        if bc not in ("none", 0):
            self.set_bc(bc)

    # -- lifetime
    def close(self):
        if getattr(self, "h", None):
            self.lib.lbmpsm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int):
        if rc != OK:
            raise LbmPsmError(rc, self.lib.lbmpsm_last_error(self.h).decode())

    def get_info(self) -> Info:
        info = Info()
        self._check(self.lib.lbmpsm_get_info(self.h, C.byref(info)))
        return info

    @property
    def steps(self) -> int:
        return int(self.get_info().steps)

    # -- the coupling step
    def set_bc(self, kind):
        self._check(self.lib.lbmpsm_set_bc(self.h, BC[kind] if isinstance(kind, str) else int(kind)))

    def step(self, tag, x, v, omega, radius, out=None):
        """One coupling step (lbmpsm_step); returns (fh[n,3], th[n,3], S[n,6]).
        ``out``: an optional C-contiguous float64 array of at least 12n
        elements that receives fh | th | S (the returned arrays are views
        of it), as a host program passes the same arrays every step."""
        tag = np.ascontiguousarray(tag, dtype=np.int32)
        n = len(tag)
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(n, 3)
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(n, 3)
        omega = np.ascontiguousarray(omega, dtype=np.float64).reshape(n, 3)
        radius = np.ascontiguousarray(radius, dtype=np.float64).reshape(n)
        if out is None:
            out = np.empty(12 * n)  # fh | th | S, every element written by the call
        elif (out.dtype != np.float64 or not out.flags.c_contiguous or out.size < 12 * n):
            raise ValueError("out must be a C-contiguous float64 array of at least 12n elements")
        out = out.reshape(-1)
        a = out.ctypes.data
        self._check(self.lib.step_by_address(
            self.h, n, tag.ctypes.data, x.ctypes.data, v.ctypes.data, omega.ctypes.data,
            radius.ctypes.data, a, a + 24 * n, a + 48 * n))
        return (out[:3 * n].reshape(n, 3), out[3 * n:6 * n].reshape(n, 3),
                out[6 * n:12 * n].reshape(n, 6))

    @staticmethod
    def _images(tag, x, v, omega, radius):
        tag = np.ascontiguousarray(tag, dtype=np.int32)
        n = len(tag)
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(n, 3)
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(n, 3)
        omega = np.ascontiguousarray(omega, dtype=np.float64).reshape(n, 3)
        radius = np.ascontiguousarray(radius, dtype=np.float64).reshape(n)
        return n, tag, x, v, omega, radius

    def adjoint_drag(self, tag, x, v, omega, radius, nsteps, t0, t1, direction=(1.0, 0.0, 0.0),
                     checkpoint_every=100, centre_step=None):
        """Run nsteps coupling steps with these images held in place and
        return J (the drag along ``direction`` averaged over steps t0..t1) with
        its gradient: dict(J, dtau, dFext[3], dx[n,3] per image row, drag[nsteps])."""
        n, tag, x, v, omega, radius = self._images(tag, x, v, omega, radius)
        d = np.ascontiguousarray(direction, dtype=np.float64)
        h = 1e-4 * self.info.dx if centre_step is None else float(centre_step)
        J = C.c_double(); dtau = C.c_double(); dF = np.zeros(3); dx = np.zeros((max(n, 1), 3))
        drag = np.zeros(int(nsteps))
        self._check(self.lib.lbmpsm_adjoint_drag(
            self.h, n, _p(tag, _I), _p(x), _p(v), _p(omega), _p(radius), int(nsteps), int(t0),
            int(t1), _p(d), int(checkpoint_every), h, C.byref(J), C.byref(dtau), _p(dF), _p(dx),
            _p(drag)))
        return dict(J=J.value, dtau=dtau.value, dFext=dF, dx=dx[:n], drag=drag)

    def tangent_drag(self, tag, x, v, omega, radius, nsteps, t0, t1, direction=(1.0, 0.0, 0.0),
                     dtau=0.0, dFext=None, dx=None, centre_step=None):
        """Forward-mode run along (dtau, dFext, dx): returns (J, dJ)."""
        n, tag, x, v, omega, radius = self._images(tag, x, v, omega, radius)
        d = np.ascontiguousarray(direction, dtype=np.float64)
        h = 1e-4 * self.info.dx if centre_step is None else float(centre_step)
        dF = None if dFext is None else np.ascontiguousarray(dFext, dtype=np.float64).reshape(3)
        dxa = None if dx is None else np.ascontiguousarray(dx, dtype=np.float64).reshape(n, 3)
        J = C.c_double(); dJ = C.c_double()
        self._check(self.lib.lbmpsm_tangent_drag(
            self.h, n, _p(tag, _I), _p(x), _p(v), _p(omega), _p(radius), int(nsteps), int(t0),
            int(t1), _p(d), h, float(dtau), None if dF is None else _p(dF),
            None if dxa is None else _p(dxa), C.byref(J), C.byref(dJ)))
        return J.value, dJ.value

    def step_device(self, n, tag_ptr, x_ptr, v_ptr, omega_ptr, radius_ptr, fh_ptr=None,
                    th_ptr=None, s_ptr=None):
        self._check(self.lib.lbmpsm_step_device(self.h, int(n), tag_ptr, x_ptr, v_ptr, omega_ptr,
                                                radius_ptr, fh_ptr, th_ptr, s_ptr))

    def apply_bc(self):
        self._check(self.lib.lbmpsm_apply_bc(self.h))

    def run_fixed(self, nsteps: int):
        self._check(self.lib.lbmpsm_run_fixed(self.h, int(nsteps)))

    def read_forces(self, n: int):
        fh = np.zeros((n, 3)); th = np.zeros((n, 3)); S = np.zeros((n, 6))
        self._check(self.lib.lbmpsm_read_forces(self.h, n, _p(fh), _p(th), _p(S)))
        return fh, th, S

    def synchronize(self):
        self._check(self.lib.lbmpsm_synchronize(self.h))

    @property
    def stream(self) -> int:
        return int(self.lib.lbmpsm_stream(self.h) or 0)

    @property
    def host_direct(self) -> bool:
        """Host-pointer steps read and write the caller's arrays in place
        (no staging copies); see lbmpsm_host_direct."""
        return self.lib.lbmpsm_host_direct(self.h) == 1

    # -- fields and state
    def request_macro(self):
        self._check(self.lib.lbmpsm_request_macro(self.h))

    def export_fields(self, B0=1.0, rho0=1.0, u0=1.0, as_double=True):
        nx, ny, nz = self.local
        npts = (nx - 2) * (ny - 2) * ((nz - 2) if self.dimension == 3 else 1)
        dt = np.float64 if as_double else np.float32
        solid = np.empty(npts, dt); rho = np.empty(npts, dt); u = np.empty((npts, 3), dt)
        self._check(self.lib.lbmpsm_export_fields(self.h, int(as_double), B0, rho0, u0,
                                                  solid.ctypes.data, rho.ctypes.data, u.ctypes.data))
        return solid, rho, u

    def populations(self) -> np.ndarray:
        f = np.empty(self.local + (self.q,), dtype=np.float64)
        self._check(self.lib.lbmpsm_get_populations(self.h, _p(f)))
        return f

    def set_populations(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(self.local + (self.q,))
        self._check(self.lib.lbmpsm_set_populations(self.h, _p(f)))

    def particle_table(self):
        N = int(np.prod(self.local))
        ids = np.empty((N, 2), np.int32); eps = np.empty((N, 2)); us = np.empty((N, 6))
        self._check(self.lib.lbmpsm_get_particle_table(self.h, _p(ids, _I), _p(eps), _p(us)))
        s = self.local
        return ids.reshape(s + (2,)), eps.reshape(s + (2,)), us.reshape(s + (6,))

    def check(self):
        mass = C.c_double(); mom = (C.c_double * 3)()
        rc = self.lib.lbmpsm_check(self.h, C.byref(mass), mom)
        if rc == ERR_NUMERIC:
            raise LbmPsmError(rc, self.lib.lbmpsm_last_error(self.h).decode())
        self._check(rc)
        return mass.value, np.array(mom[:])

    def stored_mask(self) -> np.ndarray:
        """Nodes of the reference local array that the device stores (periodic halos excluded)."""
        m = np.ones(self.local, dtype=bool)
        dims = self.dimension
        for d in range(dims):
            if self.info.storage_dims[d] != self.local[d]:
                idx = [slice(None)] * 3
                idx[d] = 0
                m[tuple(idx)] = False
                idx[d] = self.local[d] - 1
                m[tuple(idx)] = False
        return m


def _fix_params(dimension=3, boxlo=(0.0, 0.0, 0.0), prd=None, periodic=(1, 1, 1), nevery=1,
                Nlc=None, lc=None, rho=1.0, nu=None, Re=None, tau=0.7, Fext=(0.0, 0.0, 0.0)):
    p = FixParams()
    p.dimension = dimension
    p.boxlo = (C.c_double * 3)(*boxlo)
    p.prd = (C.c_double * 3)(*prd)
    p.periodic = (C.c_int * 3)(*[int(v) for v in periodic])
    p.nevery, p.Nlc, p.lc, p.rho, p.nu, p.Re, p.tau = nevery, Nlc, lc, rho, nu, Re, tau
    p.Fext = (C.c_double * 3)(*Fext)
    return p


class Ensemble(Lattice):
    """Many independent boxes of equal lattice geometry in one device
    allocation, advanced by one set of kernels per step
    (lbmpsm_create_batch).  ``boxes`` is a list of keyword dicts with the
    arguments of :class:`Lattice` that describe one box (tau, Fext, boxlo,
    rho, nu, Re, ...).  Reference-layout calls (populations, export_fields,
    particle_table) address the box chosen with :meth:`select_box`."""

    def __init__(self, boxes, *, storage: str = "fp64", device: int = 0, max_images: int = 0,
                 max_radius: float = 0.0, weighting: str = "reference",
                 collide_tuning: str = "auto"):
        self.lib = load()
        n = len(boxes)
        arr = (FixParams * n)(*[_fix_params(**b) for b in boxes])
        o = Options()
        o.storage = STORAGE[storage]
        o.device = device
        o.max_images = max_images
        o.max_radius = max_radius
        o.psm_weighting = WEIGHTING[weighting]
        o.collide_tuning = TUNING[collide_tuning]
        h = C.c_void_p()
        rc = self.lib.lbmpsm_create_batch(n, arr, C.byref(o), C.byref(h))
        if rc != OK:
            raise LbmPsmError(rc, self.lib.lbmpsm_last_error(None).decode())
        self.h = h
        self.nbox = n
        self.dimension = boxes[0].get("dimension", 3)
        self.storage = storage
        lo = boxes[0].get("boxlo", (0.0, 0.0, 0.0))
        self.origin = (float(lo[0]), float(lo[1]), float(lo[2]) if self.dimension == 3 else 0.0)
        self.info = self.get_info()
        self.local = tuple(self.info.local)
        self.q = self.info.q

    def select_box(self, b: int):
        self._check(self.lib.lbmpsm_select_box(self.h, int(b)))

    def step(self, box, tag, x, v, omega, radius):
        box = np.ascontiguousarray(box, dtype=np.int32)
        tag = np.ascontiguousarray(tag, dtype=np.int32)
        n = len(tag)
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(n, 3)
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(n, 3)
        omega = np.ascontiguousarray(omega, dtype=np.float64).reshape(n, 3)
        radius = np.ascontiguousarray(radius, dtype=np.float64).reshape(n)
        fh = np.zeros((n, 3)); th = np.zeros((n, 3)); S = np.zeros((n, 6))
        self._check(self.lib.lbmpsm_step_batch(self.h, n, _p(box, _I), _p(tag, _I), _p(x), _p(v),
                                               _p(omega), _p(radius), _p(fh), _p(th), _p(S)))
        return fh, th, S



class Group:
    """Several lattices / ensembles (e.g. one per box size) advanced together:
    one CUDA graph launch per step for all members (lbmpsm_group_*).  Destroy
    (close) the group before its members."""

    def __init__(self, members):
        self.lib = load()
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.h.value for m in self.members])
        g = C.c_void_p()
        rc = self.lib.lbmpsm_group_create(arr, len(self.members), C.byref(g))
        if rc != OK:
            raise LbmPsmError(rc, self.lib.lbmpsm_last_error(None).decode())
        self.g = g

    def run_fixed(self, nsteps: int):
        rc = self.lib.lbmpsm_group_run_fixed(self.g, int(nsteps))
        if rc != OK:
            raise LbmPsmError(rc, self.lib.lbmpsm_group_last_error(self.g).decode())

    @property
    def stream(self) -> int:
        return self.lib.lbmpsm_group_stream(self.g)

    @property
    def collide_launches(self) -> int:
        """Collide launches per step: 1 when the members' collides are fused."""
        return int(self.lib.lbmpsm_group_collide_launches(self.g))

    @property
    def tune_ms(self):
        """The tuner's ms per step: (per-member launches, one launch); -1 untimed."""
        ms = (C.c_float * 2)()
        rc = self.lib.lbmpsm_group_tune_ms(self.g, ms)
        if rc != OK:
            raise LbmPsmError(rc, self.lib.lbmpsm_group_last_error(self.g).decode())
        return float(ms[0]), float(ms[1])

    def close(self):
        if getattr(self, "g", None):
            self.lib.lbmpsm_group_destroy(self.g)
            self.g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
