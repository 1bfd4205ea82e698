"""Test configuration: the `gpu` marker, import paths, and on-demand builds
of the CPU oracle and of the native library (both are quick)."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "tests"), os.path.join(ROOT, "oracle"),
          os.path.join(ROOT, "lammps-lbm-psm_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _build_once():
    import pyoracle
    pyoracle.build(reference=True)
    lib = os.path.join(ROOT, "lammps-lbm-psm_gb300", "liblbmpsm_gb300.so")
    if not os.path.exists(lib):
        subprocess.run([sys.executable, os.path.join(ROOT, "lammps-lbm-psm_gb300", "build.py")],
                       check=True)


_build_once()


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def has_gpu():
    return gpu_available()
