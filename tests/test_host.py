"""Host logic of the product library that needs no GPU: bou.in reader,
grid and coefficient construction, configuration checks, exported symbols."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, make_bou, tc

import tc_gb300.initial as ini

HEADER = os.path.join(ROOT, "include", "tc_capi.h")

BOU_TEXT = """ NTM  NZM  NRM  NSST  IDTV    NREAD
 64   64   64   3      1        1
 NTST      TOUT      TMAX     IRESET    WALLTIMEMAX(s)
 199      1.0      10.0      0         3600
 ALX3D    RINT    REXT  ISTR   STR3    LAMB
 6.283185307179586     1.0     1.40    0     4.0    1
 VIROTINT VIROTEXT   AMPL_PERT   FREQ_PERT
  1.0       0.0       0.0         0.5
 1/NU       ROTP    RESID    CFLMAX
 1.0e3      0.0     1.e-2    1.0d3
 TSTA  STAREAD
 0.0    0
  DTMIN    DTMAX  VMAX     CFLLIM(dt fixed)
  1e-3     1e-3    1e3         1.0
 NOUT_RCUT  OUT_THCUT  OUT_STWAVE   TFRAME2D
   0            0           0          0.05
 OUT_3DFIELD TFRAME3D
   0          0.1
MINSTRT (Nx)      MINSTRZ (Nz)     MULTMIN (Nf)
  0                   0               0
"""


def test_library_exports_every_declared_symbol(gpu_lib):
    names = set(re.findall(r"\b(tc_[a-z0-9_]+)\s*\(", open(HEADER).read()))
    assert len(names) > 25
    L = ctypes.CDLL(tc.LIB_PATH)
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    assert set(tc.SIGNATURES) == names


def test_host_alloc_rejects_bad_arguments(gpu_lib):
    """tc_host_alloc / tc_host_free argument checks (no GPU needed)."""
    L = gpu_lib
    p = ctypes.c_void_p()
    assert L.tc_host_alloc(0, ctypes.byref(p)) == 2000
    assert L.tc_host_alloc(16, None) == 2000
    assert L.tc_host_free(ctypes.c_void_p(4096)) == 2000


def test_read_bou(gpu_lib, tmp_path):
    p = tmp_path / "bou.in"
    p.write_text(BOU_TEXT)
    b = tc.read_bou(str(p))
    assert (b["nthm"], b["nzm"], b["nrm"], b["nsst"], b["idtv"], b["nread"]) == (64, 64, 64, 3, 1, 1)
    assert b["ntst"] == 199 and b["tmax"] == 10.0 and b["walltimemax"] == 3600.0
    assert b["alx3"] == 6.283185307179586 and b["rext"] == 1.4 and b["istr"] == 0
    assert b["omegapert"] == 0.5 and b["limitCFL"] == 1.0e3 and b["resid"] == 1e-2
    assert b["dtmin"] == 1e-3 and b["cfllim"] == 1.0 and b["tframe3d"] == 0.1
    assert (b["minstrt"], b["minstrz"], b["multmin"]) == (0, 0, 0)


def test_read_bou_list_directed_forms(gpu_lib, tmp_path):
    """Commas, repeat counts, a record continued on the next line, '/'."""
    lines = BOU_TEXT.splitlines()
    lines[1] = " 32, 2*48, 3"          # too few values: continues on the next record
    lines.insert(2, " 1 0")
    lines[10] = " 5.0e3  0.1  / ignored"  # '/' leaves RESID and CFLMAX unchanged (zero)
    p = tmp_path / "bou.in"
    p.write_text("\n".join(lines) + "\n")
    b = tc.read_bou(str(p))
    assert (b["nthm"], b["nzm"], b["nrm"], b["nsst"], b["idtv"], b["nread"]) == (32, 48, 48, 3, 1, 0)
    assert b["ren"] == 5.0e3 and b["romeg"] == 0.1 and b["resid"] == 0.0 and b["limitCFL"] == 0.0


def test_read_bou_errors(gpu_lib, tmp_path):
    with pytest.raises(tc.TCError) as e:
        tc.read_bou(str(tmp_path / "missing.in"))
    assert e.value.code == 2001
    p = tmp_path / "bad.in"
    p.write_text(BOU_TEXT.replace(" 64   64   64   3", " 64   6.4   64   3"))
    with pytest.raises(tc.TCError) as e:
        tc.read_bou(str(p))
    assert e.value.code == 2002
    p.write_text("\n".join(BOU_TEXT.splitlines()[:9]))
    with pytest.raises(tc.TCError):
        tc.read_bou(str(p))


@pytest.mark.parametrize("case", [dict(), dict(istr=4, str=4.0, nrm=48), dict(istr=6, str=3.0, nrm=40),
                                  dict(nthm=48, nzm=96, lamb=2.0, alx3=3.0)])
def test_host_grid_matches_oracle(gpu_lib, oracle, case):
    bou = make_bou(**case)
    o = oracle.CppOracle(bou)
    for name in tc.GRID_ARRAYS:
        a = tc.grid_array(bou, name)
        b = o.grid(name)
        n = min(len(a), len(b))
        np.testing.assert_allclose(a[:n], b[:n], rtol=1e-14, atol=1e-300, err_msg=name)


@pytest.mark.parametrize("bad,code", [(dict(nthm=15), 2003), (dict(nzm=34), 2003), (dict(nthm=34), 2003),
                                      (dict(istr=1), 2003), (dict(rext=0.5), 2003),
                                      (dict(minstrt=1, multmin=1), 2003), (dict(nrm=2), 2003)])
def test_invalid_configurations(gpu_lib, bad, code):
    bou = make_bou(**bad)
    with pytest.raises(tc.TCError) as e:
        tc.grid_array(bou, "rc")
    assert e.value.code == code


def test_initial_field_is_seeded_and_periodic():
    bou = make_bou(nthm=8, nzm=6, nrm=5)
    a = ini.couette_noise(bou, seed=3)
    b = ini.couette_noise(bou, seed=3)
    c = ini.couette_noise(bou, seed=4)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    assert not np.array_equal(a[0], c[0])
    qt, qr, qz, pr = a
    assert np.all(qr[..., 0] == 0) and np.all(qr[..., -1] == 0) and np.all(pr == 0)
    np.testing.assert_array_equal(qt[0], qt[-2])
    np.testing.assert_array_equal(qt[:, 0], qt[:, -2])
    noise = qz[1:-1, 1:-1, :5]
    assert 0.004 < noise.std() < 0.007 and np.abs(noise).max() <= 0.01


def test_noalloc_wrapper_checks_coefficient_lengths():
    """The Python mirror refuses coefficient arrays shorter than nrm before
    anything reaches the library (the C side would read nrm entries)."""
    with pytest.raises(ValueError):
        tc.check_divergence_noalloc(0, 0, 0, 8, 8, 16, np.ones(15), np.ones(16), 1.0, 1.0)
    with pytest.raises(ValueError):
        tc.check_divergence_noalloc(0, 0, 0, 8, 8, 16, np.ones(16), np.ones(3), 1.0, 1.0)
