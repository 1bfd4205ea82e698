"""Host side of the LAMMPS drop-in, mirroring the reference's fix classes.

The reference fixes (timnajuch/LAMMPS-LBM-PSM src/fix_LBM_PSM*.cpp) are
LAMMPS ``Fix`` subclasses; LAMMPS keeps DEM integration, ghost atoms and
reverse communication.  These classes keep the fixes' argument syntax,
error messages and per-step bookkeeping and call the GPU library for the
lattice work, over a minimal stand-in for the LAMMPS atom/domain state
(``Atoms``, ``Domain``) so that standalone drivers and tests can run the same
call sequence a LAMMPS build would.

``ghost_images`` / ``reverse_comm`` restate what LAMMPS' CommBrick does on one
process with periodic axes (borders() and reverse_comm()).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np


class LammpsError(RuntimeError):
    """Raised where the reference calls error->all()."""


@dataclass
class Domain:
    dimension: int
    boxlo: tuple
    boxhi: tuple
    periodic: tuple

    @property
    def prd(self):
        return tuple(h - l for l, h in zip(self.boxlo, self.boxhi))


@dataclass
class Atoms:
    """Owned atoms (nlocal) followed by ghost images, LAMMPS order."""
    tag: np.ndarray
    x: np.ndarray
    v: np.ndarray
    omega: np.ndarray
    radius: np.ndarray
    nlocal: int
    f: np.ndarray = None
    torque: np.ndarray = None
    owner: np.ndarray = None  # image -> the image it was copied from
    swap: np.ndarray = None   # swap that created a ghost (-1 for owned atoms)

    def __post_init__(self):
        n = len(self.tag)
        if self.f is None:
            self.f = np.zeros((n, 3))
        if self.torque is None:
            self.torque = np.zeros((n, 3))
        if self.owner is None:
            self.owner = np.arange(n, dtype=np.int32)
        if self.swap is None:
            self.swap = np.full(n, -1, dtype=np.int32)


def ghost_images(domain: Domain, cutghost: float, tag, x, v, omega, radius) -> Atoms:
    """Ghost images as LAMMPS CommBrick::borders() makes them on one process.

    Per periodic dimension (x, y, z; z only in 3-D): first every atom present
    so far with coord <= lo + cutghost is imaged at +prd, then every atom with
    coord >= hi - cutghost at -prd (both swaps scan the same atoms).
    """
    tag = np.asarray(tag, dtype=np.int32)
    nloc = len(tag)
    T = [tag]; X = [np.asarray(x, float).reshape(-1, 3)]; V = [np.asarray(v, float).reshape(-1, 3)]
    W = [np.asarray(omega, float).reshape(-1, 3)]; R = [np.asarray(radius, float).reshape(-1)]
    owner = [np.arange(nloc, dtype=np.int32)]; swap = [np.full(nloc, -1, np.int32)]
    iswap = 0
    prd = domain.prd
    for dim in range(domain.dimension):
        if not domain.periodic[dim]:
            continue
        Tc = np.concatenate(T); Xc = np.concatenate(X); Vc = np.concatenate(V)
        Wc = np.concatenate(W); Rc = np.concatenate(R)
        lo, hi = domain.boxlo[dim], domain.boxhi[dim]
        for ineed in range(2):
            if ineed == 0:
                sel = np.nonzero(Xc[:, dim] <= lo + cutghost)[0]
                shift = prd[dim]
            else:
                sel = np.nonzero(Xc[:, dim] >= hi - cutghost)[0]
                shift = -prd[dim]
            xs = Xc[sel].copy()
            xs[:, dim] = Xc[sel, dim] + shift
            T.append(Tc[sel]); X.append(xs); V.append(Vc[sel]); W.append(Wc[sel]); R.append(Rc[sel])
            owner.append(sel.astype(np.int32)); swap.append(np.full(len(sel), iswap, np.int32))
            iswap += 1
    return Atoms(tag=np.concatenate(T), x=np.concatenate(X), v=np.concatenate(V),
                 omega=np.concatenate(W), radius=np.concatenate(R), nlocal=nloc,
                 owner=np.concatenate(owner), swap=np.concatenate(swap))


def reverse_comm(vals: np.ndarray, owner, swap, nlocal: int) -> np.ndarray:
    """CommBrick::reverse_comm on one process: swaps in reverse order, each
    ghost's row added into the image it was copied from."""
    vals = np.array(vals, dtype=np.float64, copy=True)
    owner = np.asarray(owner); swap = np.asarray(swap)
    if len(vals) == nlocal:
        return vals
    for sw in range(int(swap[nlocal:].max()), -1, -1):
        for g in np.nonzero(swap == sw)[0]:
            vals[owner[g]] += vals[g]
    return vals


def _num(s: str, what: str) -> float:
    try:
        return float(s)
    except ValueError:
        raise LammpsError(f"Expected floating point parameter instead of '{s}' in input script")


def parse_fix_lbm_psm(args: list[str]) -> dict:
    """Argument parsing of fix_LBM_PSM::fix_LBM_PSM (src/fix_LBM_PSM.cpp:15-83).

    ``args`` is the full LAMMPS argument vector: ID group-ID lbm-psm keywords...
    """
    narg = len(args)
    if narg < 15:
        raise LammpsError("Illegal fix lbm-psm command")
    p = dict(tau=0.7, Fext=(0.0, 0.0, 0.0))
    iarg = 3
    while iarg < narg:
        kw = args[iarg]
        if kw == "every":
            if iarg + 2 > narg: raise LammpsError("Illegal fix lbm-psm command")
            p["nevery"] = int(args[iarg + 1])
            if p["nevery"] <= 0: raise LammpsError("Illegal fix lbm-psm command")
            iarg += 2
        elif kw == "Nlc":
            if iarg + 2 > narg: raise LammpsError("Illegal fix lbm-psm command")
            p["Nlc"] = int(args[iarg + 1])
            if p["Nlc"] <= 0: raise LammpsError("Illegal fix lbm-psm command")
            iarg += 2
        elif kw in ("lc", "rho", "nu", "Re"):
            if iarg + 2 > narg: raise LammpsError("Illegal fix lbm-psm command")
            p[kw] = _num(args[iarg + 1], kw)
            if p[kw] <= 0.0: raise LammpsError("Illegal fix lbm-psm command")
            iarg += 2
        elif kw == "tau":
            if iarg + 2 > narg: raise LammpsError("Illegal fix lbm-psm command")
            p["tau"] = _num(args[iarg + 1], kw)
            if p["tau"] <= 0.5: raise LammpsError("Illegal fix lbm-psm command")
            iarg += 2
        elif kw == "Fext":
            if iarg + 4 > narg: raise LammpsError("Illegal fix lbm-psm command")
            p["Fext"] = tuple(_num(a, kw) for a in args[iarg + 1:iarg + 4])
            iarg += 4
        else:
            raise LammpsError("Illegal fix lbm-psm command")
    return p


class FixLbmPsm:
    """`fix ID group lbm-psm every N Nlc N lc L rho R nu NU Re RE [tau T] [Fext fx fy fz]`.

    Mirrors fix_LBM_PSM (src/fix_LBM_PSM.h:48-85): ``init`` builds the GPU
    lattice and sets the DEM timestep, ``post_force`` runs an LBM coupling step
    every ``nevery`` timesteps and re-applies the stored hydrodynamic
    force/torque on the other steps.  Extra keyword-free options (storage
    precision, device) are constructor arguments; defaults keep the
    reference's FP64 arithmetic.
    """

    def __init__(self, args: list[str], storage: str = "fp64", device: int = 0,
                 max_radius: float = 0.0):
        self.params = parse_fix_lbm_psm(args)
        self.nevery = self.params.get("nevery", 1)
        self.storage = storage
        self.device = device
        self.max_radius = max_radius
        self.lattice = None
        self.hydrodynamicInteractions = np.zeros((0, 6))
        self.virial = np.zeros(6)
        self.dt = None

    def init(self, domain: Domain):
        from . import Lattice, LbmPsmError  # local import: the package imports this module

        if self.lattice is not None:  # init() runs again on every `run`: no leak
            self.lattice.close()
        p = self.params
        for k in ("Nlc", "lc", "rho", "nu", "Re"):
            if k not in p:
                raise LammpsError("Illegal fix lbm-psm command")
        try:
            self.lattice = Lattice(dimension=domain.dimension, boxlo=domain.boxlo, prd=domain.prd,
                                   periodic=domain.periodic, nevery=self.nevery, Nlc=p["Nlc"],
                                   lc=p["lc"], rho=p["rho"], nu=p["nu"], Re=p["Re"], tau=p["tau"],
                                   Fext=p["Fext"], storage=self.storage, device=self.device,
                                   max_radius=self.max_radius)
        except LbmPsmError as e:
            raise LammpsError(str(e)) from e
        self.dt = self.lattice.info.dt_dem
        self.hydrodynamicInteractions = np.zeros((0, 6))
        return self.dt

    def get_rho(self) -> float:
        return self.params["rho"]

    def post_force(self, ntimestep: int, atoms: Atoms):
        """src/fix_LBM_PSM.cpp:181-266, with reverse_comm done on the host."""
        n = len(atoms.tag)
        if ntimestep % self.nevery:
            nl = atoms.nlocal
            hi = self.hydrodynamicInteractions
            atoms.f[:nl] += hi[:nl, :3]
            atoms.torque[:nl] += hi[:nl, 3:]
            return
        fh, th, S = self.lattice.step(atoms.tag, atoms.x, atoms.v, atoms.omega, atoms.radius)
        nl = atoms.nlocal
        atoms.f[:nl] += fh[:nl]
        atoms.f[nl:] = fh[nl:]
        atoms.torque[:nl] += th[:nl]
        atoms.torque[nl:] = th[nl:]
        self.hydrodynamicInteractions = np.concatenate([fh, th], axis=1)
        self.virial = S.sum(axis=0)  # v_tally(i, stresslet) summed over all images
        atoms.f[:] = reverse_comm(atoms.f, atoms.owner, atoms.swap, nl)
        atoms.torque[:] = reverse_comm(atoms.torque, atoms.owner, atoms.swap, nl)
        return fh, th, S


class FixLbmPsmBC:
    """`fix ID group lbm-psm-bc KEYWORD` (src/fix_LBM_PSM_BC.cpp:16-39,145-402)."""

    KEYWORDS = ("shear", "xFlow", "channel", "channel-velIn-pressOut", "closedBox")

    def __init__(self, args: list[str], fix: FixLbmPsm):
        if len(args) < 4:
            raise LammpsError("Illegal fix lbm-psm-bc command")
        if args[3] not in self.KEYWORDS:
            raise LammpsError("Illegal fix lbm-psm-bc command")
        self.keyword = args[3]
        self.fix = fix

    def init(self):
        self.fix.lattice.set_bc(self.keyword)

    def post_force(self, ntimestep: int):
        if ntimestep % self.fix.nevery:
            return
        self.fix.lattice.apply_bc()


class FixLbmPsmVTI:
    """`fix ID group lbm-psm-vti every N [binary 0|1] [useDouble 0|1]`.

    Mirrors WriteVTI (src/fix_LBM_PSM_writeVTI.cpp:15-114,
    src/fix_LBM_PSM_writeVTI.h:82-253) on one process: per output step one
    ``.vti`` piece and the ``.pvti`` master file.  The reference reads the
    rho/u arrays of the previous LBM step in pre_force; the device stores
    them only on request, so ``end_of_step`` requests them one LBM step ahead.
    """

    def __init__(self, args: list[str], fix: FixLbmPsm, folder: str = "flow_field_output_data"):
        narg = len(args)
        if narg < 5:
            raise LammpsError("Illegal fix lbm-psm-vti command")
        self.fix = fix
        self.fileName = "flow_field"
        self.binary = True
        self.useDouble = False
        self.nevery = None
        self.folder = folder
        iarg = 3
        while iarg < narg:
            kw = args[iarg]
            if kw == "every":
                if iarg + 2 > narg: raise LammpsError("Illegal fix lbm-psm-vti command")
                self.nevery = int(args[iarg + 1])
                if self.nevery <= 0: raise LammpsError("Illegal fix lbm-psm-vti command")
                iarg += 2
            elif kw in ("binary", "useDouble"):
                if iarg + 2 > narg: raise LammpsError("Illegal fix lbm-psm-vti command")
                val = int(args[iarg + 1])
                if val < 0 or val > 1: raise LammpsError("Illegal fix lbm-psm-vti command")
                setattr(self, kw, bool(val))
                iarg += 2
            else:
                raise LammpsError("Illegal fix lbm-psm-vti command")
        if self.nevery is None:
            raise LammpsError("Illegal fix lbm-psm-vti command")

    def init(self):
        if os.path.exists(self.folder):
            import shutil
            shutil.rmtree(self.folder)
        os.makedirs(self.folder)
        self.write(0, u0=0.0)

    def pre_force(self, ntimestep: int):
        if ntimestep % self.nevery:
            return
        lat = self.fix.lattice
        self.write(ntimestep, u0=lat.info.Uc / lat.info.u_lb)

    def before_lbm_step(self, ntimestep: int):
        """Call before the LBM step of ``ntimestep`` (e.g. from post_force order)."""
        nxt = ntimestep + 1
        # the next pre_force that writes reads the macro fields of the LBM step run before it
        for t in range(nxt, nxt + self.fix.nevery):
            if t % self.nevery == 0:
                self.fix.lattice.request_macro()
                break

    def write(self, timestep: int, u0: float):
        lat = self.fix.lattice
        T = np.float64 if self.useDouble else np.float32
        solid, rho, u = lat.export_fields(B0=1.0, rho0=self.fix.get_rho(), u0=u0,
                                          as_double=self.useDouble)
        return write_vti(self.folder, self.fileName, timestep, lat, solid.astype(T),
                         rho.astype(T), u.astype(T), self.binary)


def restart_file_name(rank: int = 0) -> str:
    """File name of one rank's restart file (src/fix_LBM_PSM_writeReadRestart.cpp:64-67)."""
    return f"LBM-PSM-restartFile-processor-{rank}.bin"


def write_restart(path: str, f: np.ndarray):
    """LBMPSMWriteReadRestart::write_restart (src/fix_LBM_PSM_writeReadRestart.cpp:80-89):
    the number of doubles as a native 32-bit unsigned integer, then the
    populations of the local array (halo included) in the reference layout."""
    f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
    if f.size >= 2 ** 32:
        raise LammpsError("lbm-psm-restart: local array too large for the 32-bit size field")
    with open(path, "wb") as fh:
        fh.write(np.array([f.size], dtype=np.uint32).tobytes())
        fh.write(f.tobytes())


def read_restart(path: str) -> np.ndarray:
    """LBMPSMWriteReadRestart::read_restart (src/fix_LBM_PSM_writeReadRestart.cpp:92-103)."""
    with open(path, "rb") as fh:
        head = fh.read(4)
        if len(head) != 4:
            raise LammpsError(f"lbm-psm-restart: cannot read {path}")
        n = int(np.frombuffer(head, dtype=np.uint32)[0])
        data = fh.read(8 * n)
    if len(data) != 8 * n:
        raise LammpsError(f"lbm-psm-restart: {path} holds fewer than {n} values")
    return np.frombuffer(data, dtype=np.float64).copy()


class FixLbmPsmRestart:
    """`fix ID group lbm-psm-restart every N write 0|1 read 0|1`.

    Mirrors LBMPSMWriteReadRestart (src/fix_LBM_PSM_writeReadRestart.cpp:15-78):
    ``init`` reads this rank's restart file into the lattice when ``read 1``,
    ``pre_force`` writes it every ``N`` timesteps when ``write 1``.  The file
    holds the post-stream populations in the reference layout, so files of
    the CPU code and of the GPU library are interchangeable (the halo entries
    of periodic axes are refreshed before they are used, by either code).
    """

    def __init__(self, args: list[str], fix: FixLbmPsm, rank: int = 0, folder: str = "."):
        narg = len(args)
        if narg < 9:
            raise LammpsError("Illegal fix lbm-psm-restart command")
        self.fix = fix
        self.nevery, self.iWrite, self.iRead = 1, 0, 0
        self.path = os.path.join(folder, restart_file_name(rank))
        iarg = 3
        while iarg < narg:
            kw = args[iarg]
            if kw in ("every", "write", "read"):
                if iarg + 2 > narg:
                    raise LammpsError("Illegal fix lbm-psm-restart command")
                try:
                    val = int(args[iarg + 1])
                except ValueError:
                    raise LammpsError("Illegal fix lbm-psm-restart command")
                if kw == "every":
                    if val <= 0:
                        raise LammpsError("Illegal fix lbm-psm-restart command")
                    self.nevery = val
                else:
                    if val < 0 or val > 1:
                        raise LammpsError("Illegal fix lbm-psm-restart command")
                    setattr(self, "iWrite" if kw == "write" else "iRead", val)
                iarg += 2
            else:
                raise LammpsError("Illegal fix lbm-psm-restart command")

    def init(self):
        if self.iRead == 1:
            lat = self.fix.lattice
            f = read_restart(self.path)
            want = int(np.prod(lat.local)) * lat.q
            if f.size != want:
                raise LammpsError(f"lbm-psm-restart: {self.path} holds {f.size} values, "
                                  f"the lattice needs {want}")
            lat.set_populations(f)

    def pre_force(self, ntimestep: int):
        if ntimestep % self.nevery:
            return
        if self.iWrite == 1:
            write_restart(self.path, self.fix.lattice.populations())


def _fmt(v: float) -> str:
    """std::ostream default formatting of a double (6 significant digits, %g)."""
    return "%g" % v


def write_vti(folder, name, timestep, lat, solid, rho, u, binary=True):
    """One-process form of WriteVTI::execute_write_vti's file output
    (src/fix_LBM_PSM_writeVTI.h:171-253)."""
    nxL, nyL, nzL = lat.local
    dim = lat.dimension
    nx_i, ny_i = nxL - 2, nyL - 2
    nz_i = nzL - 2 if dim == 3 else 1
    dx = lat.info.dx
    # coordinate of local node (1,1,1): origin + i*dx - dx (src/LBM_PSM_lattice.cpp:162-164)
    o = lat.origin
    originX = o[0] + 1 * dx - dx * 1
    originY = o[1] + 1 * dx - dx * 1
    originZ = (o[2] + 1 * dx - dx * 1) if dim == 3 else 0.0
    typeStr = "Float64" if solid.dtype == np.float64 else "Float32"
    base = f"{name}.{timestep:08d}"
    vfname = os.path.join(folder, base + "_rank0.vti")
    ext = f"0 {nx_i - 1} 0 {ny_i - 1} 0 {nz_i - 1}"
    origin = f"{_fmt(originX)} {_fmt(originY)} {_fmt(originZ)}"
    spacing = f"{_fmt(dx)} {_fmt(dx)} {_fmt(dx)}"
    nP = nx_i * ny_i * nz_i
    if binary:
        b_sz = nP * solid.itemsize
        u_sz = 3 * nP * solid.itemsize
        head = ('<?xml version="1.0"?>\n<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" header_type="UInt32">\n'
                f' <ImageData WholeExtent="{ext}" Origin="{origin}" Spacing="{spacing}">\n'
                f'  <Piece Extent="{ext}">\n'
                '   <PointData>\n'
                f'    <DataArray type="{typeStr}" Name="SolidFraction" format="appended" offset="0"/>\n'
                f'    <DataArray type="{typeStr}" Name="Density" format="appended" offset="{4 + b_sz}"/>\n'
                f'    <DataArray type="{typeStr}" Name="Velocity" NumberOfComponents="3" format="appended" offset="{2 * (4 + b_sz)}"/>\n'
                '   </PointData>\n  </Piece>\n </ImageData>\n <AppendedData encoding="raw">_')
        with open(vfname, "wb") as fh:
            fh.write(head.encode())
            fh.write(np.uint32(b_sz).tobytes()); fh.write(solid.tobytes())
            fh.write(np.uint32(b_sz).tobytes()); fh.write(rho.tobytes())
            fh.write(np.uint32(u_sz).tobytes()); fh.write(u.tobytes())
            fh.write(b"\n </AppendedData>\n</VTKFile>")
    else:
        with open(vfname, "w") as fh:
            fh.write('<?xml version="1.0"?>\n<VTKFile type="ImageData" version="0.1">\n')
            fh.write(f' <ImageData WholeExtent="{ext}" Origin="{origin}" Spacing="{spacing}">\n')
            fh.write(f'  <Piece Extent="{ext}">\n   <PointData>\n')
            for nm, comp, data in (("SolidFraction", 1, solid), ("Density", 1, rho), ("Velocity", 3, u.reshape(-1))):
                fh.write(f'    <DataArray type="{typeStr}" Name="{nm}" NumberOfComponents="{comp}" format="ascii">\n')
                vals = data.reshape(-1)
                for i, val in enumerate(vals):
                    fh.write(_fmt(float(val)) + ("\n" if i % 10 == 9 else " "))
                fh.write("\n    </DataArray>\n")
            fh.write("   </PointData>\n  </Piece>\n </ImageData>\n</VTKFile>")
    with open(os.path.join(folder, base + ".pvti"), "w") as fh:
        fh.write('<?xml version="1.0"?>\n<VTKFile type="PImageData" version="0.1">\n')
        fh.write(f' <PImageData WholeExtent="{ext}" Origin="{origin}" Spacing="{spacing}">\n')
        fh.write('  <PPointData>\n')
        fh.write(f'   <PDataArray type="{typeStr}" Name="SolidFraction"/>\n')
        fh.write(f'   <PDataArray type="{typeStr}" Name="Density"/>\n')
        fh.write(f'   <PDataArray type="{typeStr}" Name="Velocity" NumberOfComponents="3"/>\n')
        fh.write('  </PPointData>\n')
        fh.write(f'  <Piece Extent="{ext}" Source="{base}_rank0.vti"/>\n')
        fh.write(' </PImageData>\n</VTKFile>')
    return vfname
