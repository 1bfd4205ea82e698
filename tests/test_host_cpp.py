"""The C++ host side (lammps-lbm-psm_gb300/host): deck parsing and the fixes'
argument checks, without a GPU (``lbmpsm_driver --check`` builds the fix
objects only).  Each bad argument list must be rejected with the reference's
error message, the same one the Python mirror (lbmpsm.host) raises."""
import os
import subprocess

import pytest

import cases  # noqa: F401  (puts the package on sys.path)
from lbmpsm.host import FixLbmPsm, FixLbmPsmBC, FixLbmPsmRestart, FixLbmPsmVTI, LammpsError

DRIVER = os.path.join(cases.ROOT, "lammps-lbm-psm_gb300", "lbmpsm_driver")

LBM = "fix 1 all lbm-psm every 1 Nlc 9 lc 8.0 rho 1.0 nu 0.0667 Re 1.2 tau 0.7"


def _check(tmp_path, lines):
    if not os.path.exists(DRIVER):
        pytest.skip("lbmpsm_driver not built")
    deck = tmp_path / "deck.in"
    deck.write_text("\n".join(["dimension 3", "boundary p f p", "box 0 16 0 15 0 16"] + lines) + "\n")
    r = subprocess.run([DRIVER, "--check", str(deck)], capture_output=True, text=True)
    return r.returncode, (r.stdout + r.stderr).strip()


def test_a_valid_deck_is_accepted(tmp_path):
    rc, out = _check(tmp_path, [LBM + " Fext 1e-6 0 0", "fix 2 all lbm-psm-bc shear",
                                "fix 3 all lbm-psm-vti every 10 binary 1 useDouble 0",
                                "fix 4 all lbm-psm-restart every 100 write 1 read 0", "run 10"])
    assert rc == 0 and "deck ok: 4 fixes" in out, out


BAD = [
    # (fix line, Python class, message)
    ("fix 1 all lbm-psm every 1 Nlc 9 lc 8.0 rho 1.0", "lbm", "Illegal fix lbm-psm command"),
    (LBM.replace("tau 0.7", "tau 0.5"), "lbm", "Illegal fix lbm-psm command"),
    (LBM.replace("Nlc 9", "Nlc 0"), "lbm", "Illegal fix lbm-psm command"),
    (LBM.replace("lc 8.0", "lc eight"), "lbm",
     "Expected floating point parameter instead of 'eight' in input script"),
    (LBM + " Fext 1e-6 0", "lbm", "Illegal fix lbm-psm command"),
    (LBM + " bogus 1", "lbm", "Illegal fix lbm-psm command"),
    ("fix 2 all lbm-psm-bc sideways", "bc", "Illegal fix lbm-psm-bc command"),
    ("fix 3 all lbm-psm-vti every 0", "vti", "Illegal fix lbm-psm-vti command"),
    ("fix 3 all lbm-psm-vti every 10 binary 2", "vti", "Illegal fix lbm-psm-vti command"),
    ("fix 4 all lbm-psm-restart every 10 write 1", "restart", "Illegal fix lbm-psm-restart command"),
    ("fix 4 all lbm-psm-restart every 10 write 2 read 0", "restart",
     "Illegal fix lbm-psm-restart command"),
]


@pytest.mark.parametrize("line,kind,msg", BAD)
def test_bad_arguments_give_the_reference_errors(tmp_path, line, kind, msg):
    lines = [line] if kind == "lbm" else [LBM, line]
    rc, out = _check(tmp_path, lines)
    assert rc == 1 and out == "ERROR: " + msg, out
    # the Python mirror rejects the same arguments with the same text
    args = line.split()[1:]
    with pytest.raises(LammpsError) as e:
        if kind == "lbm":
            FixLbmPsm(args)
        else:
            fix = FixLbmPsm(LBM.split()[1:])
            {"bc": FixLbmPsmBC, "vti": FixLbmPsmVTI, "restart": FixLbmPsmRestart}[kind](args, fix)
    assert str(e.value) == msg
