"""Host-side mirror of the reference fixes: argument syntax and errors of
`fix lbm-psm`, `fix lbm-psm-bc`, `fix lbm-psm-vti` and `fix lbm-psm-restart`,
and the restart file layout (no GPU needed)."""
import numpy as np
import pytest

from lbmpsm import host
from lbmpsm.host import FixLbmPsm, FixLbmPsmBC, FixLbmPsmVTI, LammpsError, parse_fix_lbm_psm

GOOD = "1 all lbm-psm every 1 Nlc 31 lc 0.0005 rho 1000.0 nu 0.0001 Re 0.1 tau 0.7".split()


def test_parse_benchmark_deck_line():
    p = parse_fix_lbm_psm(GOOD)
    assert p == dict(nevery=1, Nlc=31, lc=0.0005, rho=1000.0, nu=0.0001, Re=0.1, tau=0.7,
                     Fext=(0.0, 0.0, 0.0))


def test_parse_defaults_and_fext():
    args = "1 all lbm-psm every 5 Nlc 11 lc 0.0005 rho 1000 nu 1e-4 Re 1.0 Fext 1 2 3".split()
    p = parse_fix_lbm_psm(args)
    assert p["tau"] == 0.7 and p["Fext"] == (1.0, 2.0, 3.0) and p["nevery"] == 5


@pytest.mark.parametrize("bad", [
    GOOD[:-4],                                   # fewer than 15 arguments
    GOOD[:-2] + ["tau", "0.5"],                  # tau <= 0.5
    GOOD[:4] + ["0"] + GOOD[5:],                 # every 0
    GOOD + ["bogus", "1"],                       # unknown keyword
    GOOD + ["Fext", "1", "2"],                   # missing component
    [a if a != "1000.0" else "-1" for a in GOOD],  # rho <= 0
])
def test_parse_errors(bad):
    with pytest.raises(LammpsError, match="Illegal fix lbm-psm command"):
        parse_fix_lbm_psm(bad)


def test_bc_keywords():
    fix = FixLbmPsm(GOOD)
    for kw in FixLbmPsmBC.KEYWORDS:
        assert FixLbmPsmBC(["b", "all", "lbm-psm-bc", kw], fix).keyword == kw
    with pytest.raises(LammpsError, match="Illegal fix lbm-psm-bc command"):
        FixLbmPsmBC(["b", "all", "lbm-psm-bc", "periodic"], fix)
    with pytest.raises(LammpsError):
        FixLbmPsmBC(["b", "all", "lbm-psm-bc"], fix)


def test_vti_arguments():
    fix = FixLbmPsm(GOOD)
    v = FixLbmPsmVTI("v all lbm-psm-vti every 100 binary 0 useDouble 1".split(), fix)
    assert v.nevery == 100 and v.binary is False and v.useDouble is True
    for bad in ("v all lbm-psm-vti every".split(), "v all lbm-psm-vti every 0".split(),
                "v all lbm-psm-vti every 10 binary 2".split()):
        with pytest.raises(LammpsError, match="Illegal fix lbm-psm-vti command"):
            FixLbmPsmVTI(bad, fix)


def test_restart_file_layout_and_arguments(tmp_path):
    """The restart file is a native uint32 count followed by the doubles
    (src/fix_LBM_PSM_writeReadRestart.cpp:80-103); the fix's argument rules."""
    import struct

    f = np.random.default_rng(0).normal(size=(4, 5, 3, 19))
    path = str(tmp_path / host.restart_file_name(0))
    host.write_restart(path, f)
    raw = open(path, "rb").read()
    assert raw[:4] == struct.pack("=I", f.size) and len(raw) == 4 + 8 * f.size
    assert np.array_equal(host.read_restart(path), f.reshape(-1))
    # a file written the reference's way reads back identically
    ref = tmp_path / "ref.bin"
    ref.write_bytes(struct.pack("=I", 6) + struct.pack("=6d", *range(6)))
    assert np.array_equal(host.read_restart(str(ref)), np.arange(6.0))
    ref.write_bytes(struct.pack("=I", 7) + struct.pack("=6d", *range(6)))
    with pytest.raises(host.LammpsError):
        host.read_restart(str(ref))
    good = ["rs", "all", "lbm-psm-restart", "every", "10", "write", "1", "read", "0"]
    fx = host.FixLbmPsmRestart(good, fix=None)
    assert (fx.nevery, fx.iWrite, fx.iRead) == (10, 1, 0)
    for bad in (good[:-2], good[:4] + ["0"] + good[5:], good[:6] + ["2"] + good[7:],
                good[:7] + ["reed", "0"]):
        with pytest.raises(host.LammpsError, match="Illegal fix lbm-psm-restart command"):
            host.FixLbmPsmRestart(bad, fix=None)
