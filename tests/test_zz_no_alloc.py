"""tc_check_divergence_noalloc: the divergence check on caller-owned device
arrays, with its scratch in a static device array, against the handle's
tc_check_divergence on the same state, two calls in a row.  This file is
collected last so that it also runs after every other GPU test."""
import math

import numpy as np
import pytest

from conftest import make_bou, tc

import tc_gb300.initial as ini

pytestmark = pytest.mark.gpu


def _device_copy(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0")


@pytest.mark.parametrize("case", [
    dict(nthm=48, nzm=40, nrm=32, istr=6, str=3.0),
    dict(nthm=64, nzm=48, nrm=96, istr=6, str=20.0),
], ids=["48x40x32", "64x48x96"])
def test_noalloc_divergence_matches_handle(gpu_lib, case):
    import torch
    bou = make_bou(**case)
    g = tc.TaylorCouette(bou)
    g.set_state(*ini.couette_noise(bou, seed=11))
    g.run(3, 0, 0.0)                       # a projected, nearly solenoidal field
    qt, qr, qz, _ = g.get_state()          # reference layout, halos filled
    want = g.check_divergence()
    nthm, nzm, nrm = bou["nthm"], bou["nzm"], bou["nrm"]
    udx2m, usrm = tc.grid_array(bou, "udx2m"), tc.grid_array(bou, "usrm")
    dxt = nthm * bou["lamb"] / (2.0 * math.pi)
    dxz = nzm / bou["alx3"]
    dq = [_device_copy(a) for a in (qt, qr, qz)]
    torch.cuda.synchronize()
    got = [tc.check_divergence_noalloc(dq[0].data_ptr(), dq[1].data_ptr(), dq[2].data_ptr(), nthm, nzm, nrm,
                                       udx2m, usrm, dxt, dxz) for _ in range(2)]
    assert want > 0.0
    for v in got:
        assert abs(v - want) <= 1e-12 * want
    # a raw, unprojected field: large divergence, same agreement
    st = ini.couette_noise(bou, seed=12, amp=0.5)
    g.set_state(*st)
    want = g.check_divergence()
    qt, qr, qz, _ = g.get_state()
    dq = [_device_copy(a) for a in (qt, qr, qz)]
    torch.cuda.synchronize()
    got = [tc.check_divergence_noalloc(dq[0].data_ptr(), dq[1].data_ptr(), dq[2].data_ptr(), nthm, nzm, nrm,
                                       udx2m, usrm, dxt, dxz) for _ in range(2)]
    for v in got:
        assert abs(v - want) <= 1e-12 * want
    g.close()


def test_noalloc_on_a_side_stream_and_with_a_nan(gpu_lib):
    """The same result on a non-default stream; a NaN in the field gives
    status 169 on both paths instead of a finite maximum."""
    import torch
    bou = make_bou(nthm=32, nzm=24, nrm=20, istr=6, str=3.0)
    g = tc.TaylorCouette(bou)
    g.set_state(*ini.couette_noise(bou, seed=5, amp=0.3))
    want = g.check_divergence()
    qt, qr, qz, pr = g.get_state()
    nthm, nzm, nrm = bou["nthm"], bou["nzm"], bou["nrm"]
    udx2m, usrm = tc.grid_array(bou, "udx2m"), tc.grid_array(bou, "usrm")
    dxt = nthm * bou["lamb"] / (2.0 * math.pi)
    dxz = nzm / bou["alx3"]
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        dq = [_device_copy(a) for a in (qt, qr, qz)]
    side.synchronize()
    got = [tc.check_divergence_noalloc(dq[0].data_ptr(), dq[1].data_ptr(), dq[2].data_ptr(), nthm, nzm, nrm,
                                       udx2m, usrm, dxt, dxz, stream=side.cuda_stream) for _ in range(2)]
    for v in got:
        assert abs(v - want) <= 1e-12 * want
    qt_nan = qt.copy()
    qt_nan[5, 7, 3] = np.nan                  # an interior cell (theta 5, z 7, r 3)
    g.set_state(qt_nan, qr, qz, pr)
    with pytest.raises(tc.TCError) as e:
        g.check_divergence()
    assert e.value.code == 169
    dn = _device_copy(qt_nan)
    torch.cuda.synchronize()
    with pytest.raises(tc.TCError) as e:
        tc.check_divergence_noalloc(dn.data_ptr(), dq[1].data_ptr(), dq[2].data_ptr(), nthm, nzm, nrm,
                                    udx2m, usrm, dxt, dxz)
    assert e.value.code == 169
    g.close()


def test_noalloc_rejects_too_many_radial_cells(gpu_lib):
    import torch
    buf = torch.zeros(16, dtype=torch.float64, device="cuda:0")
    coef = np.ones(8193)
    with pytest.raises(tc.TCError) as e:
        tc.check_divergence_noalloc(buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), 4, 4, 8193, coef, coef,
                                    1.0, 1.0)
    assert e.value.code == 2016 and "8192" in str(e.value)


def test_noalloc_divergence_matches_reference_runs(gpu_lib):
    """On the start and on the final fields of every reference run that
    keeps its whole fields: the reference's CheckDivergence before the loop
    (main.F90:125; O(1) for these starts) within 1e-13 relative, and after
    the run (roundoff) within 1e-13 absolute."""
    import torch
    import refruns as R
    for name in R.CASE_NAMES:
        c = R.case(name)
        if c.get("planes") is not None:
            continue
        bou = c["bou"]
        nthm, nzm, nrm = int(bou["nthm"]), int(bou["nzm"]), int(bou["nrm"])
        udx2m, usrm = tc.grid_array(bou, "udx2m"), tc.grid_array(bou, "usrm")
        dxt = nthm * bou["lamb"] / (2.0 * math.pi)
        dxz = nzm / bou["alx3"]
        for fields, want, rel in ((R.start(c)[:3], float(R.ref(name, "out_dmax")[0]), True),
                                  ([R.ref(name, k) for k in ("qt", "qr", "qz")], float(R.ref(name, "final_dmax")),
                                   False)):
            dq = [_device_copy(a) for a in fields]
            torch.cuda.synchronize()
            got = tc.check_divergence_noalloc(dq[0].data_ptr(), dq[1].data_ptr(), dq[2].data_ptr(), nthm, nzm, nrm,
                                              udx2m, usrm, dxt, dxz)
            err = abs(got - want) / (want if rel else 1.0)
            assert err <= 1e-13, (name, rel, got, want)
