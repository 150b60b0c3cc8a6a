"""The CPU oracle against runs of the reference's own Fortran source.

Every case of tests/golden/reference_runs.npz (see tests/refruns.py) is run
through the C++ restatement (oracle/tc_ref.cpp) one step at a time as
main.F90:152-226 runs it, from the same seeded start and bou.in values, and
compared with what the reference computed:

* velocities: 1e-12 of each field's maximum (measured: below 3e-14);
* pressure with the radial profile of the singular mode removed: 1e-11 of
  max |pr| (measured: below 2e-13);
* the dt sequence, the step times, the CFL numbers behind dt and the
  CalcTorque records of the output steps: 1e-12 relative;
* the stop code and the index of the last step: equal;
* the final CheckDivergence below RESID in both.

This pins the oracle that the GPU parity tests use to the reference itself.
"""
import math
import os

import numpy as np
import pytest

import refruns as R

TOL_Q = 1e-12
TOL_P = 1e-11
TOL_S = 1e-12


def oracle_march(oracle, c):
    o = oracle.CppOracle(c["bou"])
    o.set_state(*R.start(c))

    def step(ntime, t, dt):
        return o.run(ntime, 1, t, dt)

    rec = R.march(step, o.calc_max_cfl, o.calc_torque, c)
    return o, rec


@pytest.mark.parametrize("name", R.CASE_NAMES)
def test_oracle_matches_reference_run(oracle, name):
    c = R.case(name)
    o, rec = oracle_march(oracle, c)
    assert rec["code"] == int(R.ref(name, "errorcode"))
    assert rec["ntime"] == int(R.ref(name, "ntime"))
    se = R.scalar_errors(c, rec)
    fe = R.field_errors(c, o.state())
    print(name, {k: f"{v:.1e}" for k, v in {**fe, **se}.items()})
    for k in ("qt", "qr", "qz"):
        assert fe[k] <= TOL_Q, (k, fe[k])
    assert fe["pr"] <= TOL_P, fe["pr"]
    for k, v in se.items():
        assert v <= TOL_S, (k, v)
    ti, to = o.calc_torque()
    rt = R.ref(name, "final_torque")
    assert abs(ti - rt[1]) <= TOL_S * abs(rt[1]) and abs(to - rt[2]) <= TOL_S * abs(rt[2])
    resid = c["bou"]["resid"]
    assert o.check_divergence() < resid and float(R.ref(name, "final_dmax")) < resid
    assert abs(o.calc_max_cfl() - float(R.ref(name, "final_cfl"))) <= TOL_S * float(R.ref(name, "final_cfl"))


def test_cases_cover_the_stop_codes_and_forms():
    """The fixtures hold runs that end with 555 (NTST reached), 333 (TMAX)
    and 166 (dt below DTMIN), RK3 and AB2, the three radial grids, fixed and
    variable dt, rotation, the oscillating cylinder and patterned slip."""
    codes = {int(R.ref(n, "errorcode")) for n in R.CASE_NAMES}
    assert {555, 333, 166} <= codes
    bous = [c["bou"] for c in R.CASES]
    assert {0, 4, 6} <= {int(b["istr"]) for b in bous}
    assert {1, 3} <= {int(b["nsst"]) for b in bous}
    assert any(b["romeg"] != 0 for b in bous) and any(b["sizepert"] != 0 for b in bous)
    assert any(b["minstrt"] * b["multmin"] != 0 for b in bous)
    assert any(b["dtmin"] < b["dtmax"] for b in bous) and any(b["dtmin"] == b["dtmax"] for b in bous)
    assert any((b["nthm"], b["nzm"], b["nrm"]) == (64, 64, 64) for b in bous)


REF_DIR = os.environ.get("TC_REFERENCE_DIR", "/root/reference")


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF_DIR, "TimeMarcher.F90")),
                    reason="the reference tree is not on this machine")
def test_fixture_reproduces_from_the_reference_source():
    """Re-run the smallest case through the Fortran translator and get the
    committed fixture back bit for bit."""
    pytest.importorskip("scipy")
    import sys
    sys.path.insert(0, R.GOLDEN)
    import make_reference_runs as M
    c = next(x for x in M.CASES if x["name"] == "stops_at_tmax")
    out = M.run_case(REF_DIR, c)
    for k, v in out.items():
        np.testing.assert_array_equal(v, R.ref(c["name"], k), err_msg=k)
