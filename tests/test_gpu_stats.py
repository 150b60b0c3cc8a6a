"""Statistics of the output steps on the device against the oracle:
CalcStats (with CalcVorticity) and CalcDissipation, two samples apart by a
step, and WriteStats through the HDF5 writer."""
import numpy as np
import pytest

from conftest import make_bou, tc

import tc_gb300.initial as ini

from test_h5 import walk

pytestmark = pytest.mark.gpu


def _sync_halos(oracle, o):
    for a in (oracle.QT, oracle.QR, oracle.QZ, oracle.PR):
        o.call("update_halo", a)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-4)])
@pytest.mark.parametrize("case", [dict(nthm=48, nzm=40, nrm=32, istr=6, str=3.0, romeg=0.2),
                                  dict(nthm=32, nzm=24, nrm=16, istr=0)], ids=["cheb", "uniform"])
def test_stats_match_oracle(gpu_lib, oracle, precision, tol, case):
    bou = make_bou(**case)
    st = ini.couette_noise(bou, seed=8, amp=0.05)
    g = tc.TaylorCouette(bou, precision=precision)
    g.set_state(*st)
    o = oracle.CppOracle(bou)
    o.set_state(*st)
    nutes = []
    t = 0.0
    for step in range(2):
        g.time_marcher(1e-3, t)
        o.time_marcher(1e-3, t)
        t += 1e-3
        _sync_halos(oracle, o)
        g.calc_stats()
        o.calc_stats()
        nutes.append((g.calc_dissipation(), o.calc_dissipation()))
    assert g.stat_samples == o.stat_samples() == 2
    for a, b in nutes:
        assert abs(a - b) <= tol * abs(b)
    for w, name in enumerate(tc.STATS):
        got, want = g.stat(name), o.stat(w)
        scale = float(np.abs(want).max())
        assert scale > 0, name
        assert float(np.abs(got - want).max()) <= tol * scale, name
    g.reset_stats()
    assert g.stat_samples == 0 and not g.stat("vt_mean").any()
    g.close()


def test_write_stats_files(gpu_lib, tmp_path):
    bou = make_bou(nthm=24, nzm=20, nrm=16)
    g = tc.TaylorCouette(bou)
    g.set_state(*ini.couette_noise(bou, seed=2))
    g.time_marcher(1e-3, 0.0)
    g.calc_stats()
    g.calc_dissipation()
    g.write_stats(str(tmp_path))
    vt = walk(str(tmp_path / "vt_mean.h5"))["vt_mean"]
    assert vt[0] == [20, 16] and np.array_equal(vt[2], g.stat("vt_mean"))
    m = walk(str(tmp_path / "stafield_master.h5"))
    assert m["averaging_time"][2][0] == 1 and m["Reynolds Number"][2][0] == bou["ren"]
    assert np.array_equal(m["R_cordin"][2], tc.grid_array(bou, "rm")[:16])
    # readstats: the files' values are added
    g.write_stats(str(tmp_path), readstats=True)
    assert np.array_equal(tc.h5_read(str(tmp_path / "vt_mean.h5"), "vt_mean"), 2 * g.stat("vt_mean"))
    assert tc.h5_read(str(tmp_path / "stafield_master.h5"), "averaging_time")[0] == 2
    g.close()
