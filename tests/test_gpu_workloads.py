"""Parity of the benchmarked workloads against the CPU oracle.

* The headline production case, 512 x 512 x 384 on the wall-clustered grid
  (ISTR=6, STR3=20), 1/NU = 5000, oscillating inner cylinder, variable dt
  (CFLMAX 1.2, DTMIN 1e-5, DTMAX 3e-4), seed 1234: 20 steps through tc_run,
  the oracle on every host core beside it (main.F90:152-226,
  TimeMarcher.F90:22-54).  Velocities, pressure and torques within 1e-10
  relative, the same dt sequence, divergence below RESID.
* The rotating-frame case with C3's parameters (ROTP = 0.1, 1/NU = 2e4,
  ISTR=6 STR3=20, variable dt, DTMAX 1.8e-4) on a 128 x 96 x 64 grid: the
  FP64 path within 1e-10 after 20 steps, and the mixed forms (FP64 and
  float-float pressure tridiagonals) within 1e-3 on velocities and 1e-4 on
  the torques, their errors printed.  The Coriolis terms are
  ExplicitTermsQT.F90:119-121 and ExplicitTermsQR.F90:142-143.

The workload parameters are imported from bench.py so that the test runs
exactly what is timed there.
"""
import numpy as np
import pytest

from conftest import rel_err, tc

import bench
import tc_gb300.initial as ini

pytestmark = pytest.mark.gpu

TOL_20 = 1e-10


def _pair(oracle, bou, precision="fp64", seed=1234):
    st = ini.couette_noise(bou, seed=seed)
    g = tc.TaylorCouette(bou, precision=precision)
    g.set_state(*st)
    o = oracle.CppOracle(bou)
    o.set_state(*st)
    return g, o


def _errors(g, o, nrm):
    gs, os_ = g.get_state(), o.state()
    return {name: rel_err(a, b, nk=nk) for name, a, b, nk in
            zip(("qt", "qr", "qz", "pr"), gs, os_, (nrm, nrm + 1, nrm, nrm))}


def _torque_err(g, o):
    ti_g, to_g = g.calc_torque()
    ti_o, to_o = o.calc_torque()
    return max(abs(ti_g - ti_o) / abs(ti_o), abs(to_g - to_o) / abs(to_o)), (ti_g, to_g)


def test_headline_workload_twenty_steps(gpu_lib, oracle):
    bou = bench.base_bou(**bench.WORKLOADS["C2"])
    assert (bou["nthm"], bou["nzm"], bou["nrm"]) == (512, 512, 384)
    oracle.set_threads(0)                       # every host core
    g, o = _pair(oracle, bou)
    code_g, n_g, t_g, dt_g = g.run(20, 0, 0.0)
    code_o, t_o, dt_o = o.run(0, 20, 0.0)
    assert code_g == code_o == 0 and n_g == 20
    assert abs(t_g - t_o) <= 1e-12 * t_o and abs(dt_g - dt_o) <= 1e-12 * dt_o
    errs = _errors(g, o, bou["nrm"])
    terr, torques = _torque_err(g, o)
    div = g.check_divergence()
    print("512x512x384 x 20 steps:", errs, "torque", terr, torques, "div", div, "time", t_g)
    assert max(errs.values()) < TOL_20, errs
    assert terr < TOL_20
    assert div < bou["resid"]
    g.close()


C3_REDUCED = dict(bench.WORKLOADS["C3"], nthm=128, nzm=96, nrm=64)


def test_rotating_case_fp64_twenty_steps(gpu_lib, oracle):
    bou = bench.base_bou(**C3_REDUCED)
    assert bou["romeg"] == 0.1 and bou["ren"] == 2e4
    oracle.set_threads(0)
    g, o = _pair(oracle, bou)
    code_g, n_g, t_g, _ = g.run(20, 0, 0.0)
    code_o, t_o, _ = o.run(0, 20, 0.0)
    assert code_g == code_o == 0
    assert abs(t_g - t_o) <= 1e-12 * t_o
    errs = _errors(g, o, bou["nrm"])
    terr, torques = _torque_err(g, o)
    print("rotating 128x96x64 FP64:", errs, "torque", terr, torques)
    assert max(errs.values()) < TOL_20, errs
    assert terr < TOL_20
    assert g.check_divergence() < bou["resid"]
    g.close()


@pytest.mark.parametrize("precision", ["mixed", "mixed-ff"])
def test_rotating_case_mixed_twenty_steps(gpu_lib, oracle, precision):
    bou = bench.base_bou(**C3_REDUCED)
    oracle.set_threads(0)
    g, o = _pair(oracle, bou, precision=precision)
    code_g, n_g, t_g, _ = g.run(20, 0, 0.0)
    code_o, t_o, _ = o.run(0, 20, 0.0)
    assert code_g == code_o == 0
    errs = _errors(g, o, bou["nrm"])
    terr, torques = _torque_err(g, o)
    div = g.check_divergence()
    print(f"rotating 128x96x64 {precision}: velocity", {k: errs[k] for k in ("qt", "qr", "qz")},
          "torque", terr, "div", div, "time", t_g, t_o)
    assert max(errs["qt"], errs["qr"], errs["qz"]) < 1e-3, errs
    assert terr < 1e-4
    assert div < 1e-3 * bou["resid"]
    g.close()
