"""Restart files through a handle: WriteFlowField then ReadFlowField give back
the same velocities, the master file carries the reference's scalars, and a
run restarted from the files equals a run loaded from the same arrays."""
import numpy as np
import pytest

from conftest import make_bou, tc

import tc_gb300.initial as ini

from test_h5 import walk

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_continua_round_trip(gpu_lib, tmp_path, precision):
    bou = make_bou(nthm=48, nzm=40, nrm=32, istr=6, str=3.0)
    g = tc.TaylorCouette(bou, precision=precision)
    g.set_state(*ini.couette_noise(bou, seed=4))
    code, n, t, dt = g.run(3, 0, 0.0)
    g.write_continua(str(tmp_path), t)
    want = g.get_state()
    master = walk(str(tmp_path / "continua_master.h5"))
    assert sorted(master) == sorted(["nr", "nth", "nz", "time", "rint", "rext", "istr", "str", "alx3", "lamb"])
    assert master["nr"][2][0] == 33 and master["nth"][2][0] == 49 and master["nz"][2][0] == 41
    assert master["time"][2][0] == t and master["istr"][2][0] == 6 and master["str"][2][0] == 3.0
    var = walk(str(tmp_path / "continua_qt.h5"))["var"]
    assert var[0] == [48, 40, 33]
    assert np.array_equal(var[2][:, :, :32], want[0][1:-1, 1:-1, :32])
    h = tc.TaylorCouette(bou, precision=precision)
    t2 = h.read_continua(str(tmp_path))
    assert t2 == t
    got = h.get_state()
    for a, b, nk in zip(got[:3], want[:3], (32, 33, 32)):
        assert np.array_equal(a[..., :nk], b[..., :nk])
    # a restart from the files equals a start from the same arrays
    ref = tc.TaylorCouette(bou, precision=precision)
    ref.set_state(*want[:3])
    h.run(2, 3, t2)
    ref.run(2, 3, t)
    for a, b in zip(h.get_state()[:3], ref.get_state()[:3]):
        assert np.array_equal(a, b)
    for x in (g, h, ref):
        x.close()


def test_continua_of_another_grid(gpu_lib, tmp_path):
    """A finer grid is interpolated (interp.F90, as the host loader does);
    one more than twice as fine is refused."""
    bou = make_bou(nthm=24, nzm=20, nrm=16)
    g = tc.TaylorCouette(bou)
    g.set_state(*ini.couette_noise(bou, seed=1))
    g.write_continua(str(tmp_path), 0.5)
    finer = make_bou(nthm=32, nzm=24, nrm=20)
    other = tc.TaylorCouette(finer)
    assert other.read_continua(str(tmp_path)) == 0.5
    want = tc.h5_load_continua(finer, str(tmp_path))
    got = other.get_state()
    assert np.array_equal(got[0][1:-1, 1:-1, :20], want[0][1:-1, 1:-1, :20])
    too_fine = tc.TaylorCouette(make_bou(nthm=24, nzm=20, nrm=40))
    with pytest.raises(tc.TCError) as e:
        too_fine.read_continua(str(tmp_path))
    assert e.value.code == 2024 and "twice" in str(e.value)
    for x in (g, other, too_fine):
        x.close()


def test_output_dumps(gpu_lib, tmp_path):
    """DumpFlowField, DumpRCuts, DumpThCuts and DumpStreamwiseAvg against
    the same quantities computed here from the state."""
    bou = make_bou(nthm=24, nzm=20, nrm=16, istr=6, str=3.0)
    g = tc.TaylorCouette(bou)
    g.set_state(*ini.couette_noise(bou, seed=6, amp=0.1))
    code, n, t, dt = g.run(2, 0, 0.0)
    qt, qr, qz, _ = g.get_state()
    usrc, rm = tc.grid_array(bou, "usrc"), tc.grid_array(bou, "rm")
    tag = "%08d" % int(np.floor(1000.0 * t + 0.005 + 0.5))
    d = str(tmp_path)
    g.dump_flow_field(d, t)
    assert np.array_equal(walk(f"{d}/qz_{tag}.h5")["var"][2], qz[1:-1, 1:-1, :])
    assert walk(f"{d}/ms_{tag}.h5")["time"][2][0] == t
    radii = [0.5 * (rm[3] + rm[4]), rm[10] - 1e-9]
    g.dump_rcuts(d, t, radii)
    for m, ks in ((1, 5), (2, 11)):                      # reference k (1-based) of each slab
        vr = walk(f"{d}/slab{m}vr_{tag}.h5")["vr"][2]
        want = (qr[1:-1, 1:-1, ks - 1] * usrc[ks - 1] + qr[1:-1, 1:-1, ks] * usrc[ks]) * 0.5
        # (the host compiler may contract the products into fused multiply-adds)
        assert vr.shape == (24, 20) and np.allclose(vr, want, rtol=1e-13, atol=1e-18)
        assert np.array_equal(walk(f"{d}/slab{m}vt_{tag}.h5")["vt"][2], qt[1:-1, 1:-1, ks - 1])
    g.dump_thcuts(d, t)
    th = walk(f"{d}/slabvt_{tag}.h5")
    assert list(th) == ["vr"]                            # the reference's file name collision, kept
    assert np.array_equal(th["vr"][2], (qr[1, 1:-1, :16] * usrc[:16]))
    assert np.array_equal(walk(f"{d}/slabvz_{tag}.h5")["vz"][2], qz[1, 1:-1, :16])
    g.dump_streamwise_avg(d, t)
    ax = walk(f"{d}/slabvt_ax_{tag}.h5")["vt"][2]
    assert ax.shape == (20, 16) and np.allclose(ax, qt[1:-1, 1:-1, :16].mean(axis=0), rtol=1e-13)
    g.close()
