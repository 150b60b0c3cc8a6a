"""Shared fixtures: package loader, oracle import, configuration builder."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import __graft_entry__ as entry  # noqa: E402

tc = entry.load()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and libtcgb300.so")


def make_bou(**kw):
    """A bou.in-equivalent dict; defaults are the 64^3 uniform-grid RK3 case
    with fixed dt = DTMAX (IDTV=1, DTMIN = DTMAX, CFLMAX large)."""
    d = dict(nthm=64, nzm=64, nrm=64, nsst=3, idtv=1, nread=1, ntst=100000, tout=1.0e6, tmax=1.0e6,
             ireset=0, walltimemax=1e9, alx3=2 * np.pi, rint=1.0, rext=1.4, istr=0, str=4.0, lamb=1.0,
             virotint=1.0, virotext=0.0, sizepert=0.0, omegapert=0.0, ren=1000.0, romeg=0.0, resid=1e-2,
             limitCFL=1e3, tsta=0.0, starea=0, dtmin=1e-3, dtmax=1e-3, limitVel=1e3, cfllim=1.0,
             nslabr=0, dpthcut=0, dpstave=0, tframe2d=1.0, dpfullf=0, tframe3d=1.0,
             minstrt=0, minstrz=0, multmin=0)
    d.update(kw)
    return d


def rel_err(a, b, interior=True, nk=None, scale=None):
    """max |a-b| / max |b| over the interior (no halo) cells; with `scale`,
    max |a-b| / scale instead."""
    if interior:
        a, b = a[1:-1, 1:-1], b[1:-1, 1:-1]
    if nk is not None:
        a, b = a[..., :nk], b[..., :nk]
    den = float(np.abs(b).max()) if scale is None else float(scale)
    return float(np.abs(a - b).max()) / (den if den > 0 else 1.0)


@pytest.fixture(scope="session")
def oracle():
    import tc_ref
    tc_ref.build()
    return tc_ref


@pytest.fixture(scope="session")
def gpu_lib():
    import tc_gb300.build as b
    b.build()
    return tc.lib()
