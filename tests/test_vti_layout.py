"""The bytes of the `fix lbm-psm-vti` files, pinned to the reference writer.

oracle/vti_oracle.c restates the file output of WriteVTI::execute_write_vti<T>
(src/fix_LBM_PSM_writeVTI.h:82-253) on one process: the XML headers, the
extents, origin and spacing in std::ostream's default formatting, the raw
appended arrays with their UInt32 byte counts (or ten ascii values per line),
and the .pvti master file.  The repository's two writers -- lbmpsm/host.py
write_vti and the C++ host's write_vti_files (host/lbmpsm_fix.cpp, compiled
here into a small harness) -- must write the same bytes for the same fields:
binary and ascii, Float32 and Float64, 2-D and 3-D.  No GPU is needed: the
fields are synthetic (the GPU export of the fields is pinned to the oracle's
field read by the -m gpu tests).
"""
import os
import subprocess
from types import SimpleNamespace

import numpy as np
import pytest

import cases
import pyoracle
from lbmpsm.host import write_vti

PKG = os.path.join(cases.ROOT, "lammps-lbm-psm_gb300")

HARNESS = r'''
#include <cstdio>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>
#include "lbmpsm_fix.h"
static std::vector<char> slurp(const char* p) {
  std::ifstream f(p, std::ios::binary);
  return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}
int main(int argc, char** argv) {
  if (argc != 16) return 2;
  const int local[3] = {std::stoi(argv[4]), std::stoi(argv[5]), std::stoi(argv[6])};
  const double origin[3] = {std::stod(argv[7]), std::stod(argv[8]), std::stod(argv[9])};
  const auto s = slurp(argv[13]), r = slurp(argv[14]), u = slurp(argv[15]);
  lbmpsm_host::write_vti_files(argv[1], "flow_field", std::stol(argv[2]), std::stoi(argv[3]), local,
                               origin, std::stod(argv[10]), argv[11][0] == '1', argv[12][0] == '1',
                               s.data(), r.data(), u.data());
  return 0;
}
'''


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    d = tmp_path_factory.mktemp("vti_harness")
    src = d / "harness.cpp"
    src.write_text(HARNESS)
    exe = d / "harness"
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(cases.ROOT, "include"), "-I",
           os.path.join(PKG, "host"), str(src), os.path.join(PKG, "host", "lbmpsm_fix.cpp"), "-o",
           str(exe), "-L", PKG, "-llbmpsm_gb300", f"-Wl,-rpath,{PKG}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail("harness build failed:\n" + r.stderr[-2000:])
    return exe


def _fields(rng, dim, local):
    n = (local[0] - 2) * (local[1] - 2) * ((local[2] - 2) if dim == 3 else 1)
    solid = np.clip(rng.uniform(-0.2, 1.3, n), 0.0, 1.0)
    solid[::7] = 1.0
    solid[3::11] = 0.0
    rho = 1000.0 * (1.0 + 1e-5 * rng.standard_normal(n))
    u = rng.standard_normal((n, 3)) * 10.0 ** rng.integers(-9, 3, (n, 3))
    u[::5, 1] = 0.0
    u[1::13, 0] = 1.0e-300  # below the Float32 range
    u[2::17, 2] = -123456.789
    if dim == 2:
        u[:, 2] = 0.0
    return solid, rho, u


@pytest.mark.parametrize("dim", [3, 2])
@pytest.mark.parametrize("binary", [1, 0])
@pytest.mark.parametrize("use_double", [0, 1])
def test_vti_files_equal_the_reference_writer(tmp_path, harness, dim, binary, use_double):
    rng = np.random.default_rng(100 * dim + 10 * binary + use_double)
    local = (8, 7, 6) if dim == 3 else (9, 7, 1)
    origin = (-3.7e-4, 1.3e-4, 2.05e-3)
    dx = 0.0005 / 10
    step = 1234
    solid, rho, u = _fields(rng, dim, local)
    T = np.float64 if use_double else np.float32
    out = {k: tmp_path / k for k in ("oracle", "python", "cpp")}
    for d in out.values():
        d.mkdir()
    pyoracle.write_vti(out["oracle"], "flow_field", step, binary, use_double, dim, local, origin, dx,
                       solid, rho, u)
    lat = SimpleNamespace(local=local, dimension=dim, info=SimpleNamespace(dx=dx),
                          origin=(origin[0], origin[1], origin[2] if dim == 3 else 0.0))
    write_vti(str(out["python"]), "flow_field", step, lat, solid.astype(T), rho.astype(T),
              u.astype(T), bool(binary))
    files = []
    for nm, a in (("s", solid), ("r", rho), ("u", u)):
        p = tmp_path / f"{nm}.bin"
        p.write_bytes(np.ascontiguousarray(a.astype(T)).tobytes())
        files.append(str(p))
    r = subprocess.run([str(harness), str(out["cpp"]), str(step), str(dim), *map(str, local),
                        *map(repr, origin), repr(dx), str(binary), str(use_double), *files],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    names = sorted(os.listdir(out["oracle"]))
    assert names == ["flow_field.00001234.pvti", "flow_field.00001234_rank0.vti"]
    for nm in names:
        ref = (out["oracle"] / nm).read_bytes()
        assert (out["python"] / nm).read_bytes() == ref, ("python", nm)
        assert (out["cpp"] / nm).read_bytes() == ref, ("cpp", nm)
    head = (out["oracle"] / names[1]).read_bytes()[:400]
    assert (b"Float64" if use_double else b"Float32") in head
    assert (b'format="appended"' if binary else b'format="ascii"') in head
