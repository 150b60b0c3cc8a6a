"""Mixed FP32/FP64 path: velocities, explicit terms, momentum sweeps and FFTs
in FP32; pressure tridiagonals, pressure accumulation and reductions in FP64.
Checked against the FP64 oracle with FP32-level tolerances, and the torque
against the 1e-4 relative bound the mixed form must meet."""
import numpy as np
import pytest

from conftest import make_bou, rel_err, tc

import tc_gb300.initial as ini

pytestmark = pytest.mark.gpu


def pair(oracle, bou, seed=5, precision="mixed"):
    st = ini.couette_noise(bou, seed=seed)
    g = tc.TaylorCouette(bou, precision=precision)
    g.set_state(*st)
    o = oracle.CppOracle(bou)
    o.set_state(*st)
    return g, o


def test_mixed_routines(gpu_lib, oracle):
    """One substep routine by routine: FP32 rounding only (~1e-6)."""
    bou = make_bou(nthm=48, nzm=40, nrm=32, istr=6, str=3.0)
    g, o = pair(oracle, bou)
    assert g.L.tc_precision(g.h) == 1
    g.begin_step(1e-3, 0.0)
    o.call("begin_step", 1e-3, 0.0)
    g.set_substep(1)
    o.call("set_substep", 1)
    g.explicit_terms()
    for f in ("explicit_terms_qt", "explicit_terms_qr", "explicit_terms_qz"):
        o.call(f)
    assert rel_err(g.get_field("dq"), o.get(oracle.DQ), interior=False, nk=32) < 1e-5
    g.implicit_and_update()
    for f in ("implicit_rhs_qt", "solve_imp_eqn_update_qt", "implicit_rhs_qr", "solve_imp_eqn_update_qr",
              "implicit_rhs_qz", "solve_imp_eqn_update_qz"):
        o.call(f)
    gs, os_ = g.get_state(), o.state()
    for a, b, nk in zip(gs[:3], os_[:3], (32, 33, 32)):
        assert rel_err(a, b, nk=nk) < 1e-5
    g.calc_local_divergence()
    o.call("calc_local_divergence")
    g.solve_pressure_correction()
    o.call("solve_pressure_correction")
    # phi itself carries the radially integrated k = 0 mode, whose FP32
    # right-hand side is a small difference of large divergences: loose check
    assert rel_err(g.get_field("dph"), o.get(oracle.DPH), nk=32) < 2e-2
    o.call("update_halo", oracle.DPH)
    g.correct_velocity()
    o.call("correct_velocity")
    g.correct_pressure()
    o.call("correct_pressure")
    # The correction is the gradient of phi; its FP32 error is set by the
    # azimuthal velocity (O(1)) that dominates the divergence, not by the
    # small radial and axial noise, so every component is measured against
    # the largest velocity.
    gs, os_ = g.get_state(), o.state()
    u = float(np.abs(os_[0][1:-1, 1:-1, :32]).max())
    for a, b, nk in zip(gs[:3], os_[:3], (32, 33, 32)):
        assert rel_err(a, b, nk=nk, scale=u) < 1e-4
    g.close()


@pytest.mark.parametrize("case", [
    dict(),
    dict(nthm=64, nzm=48, nrm=96, istr=6, str=20.0, sizepert=0.1, omegapert=0.5, romeg=0.1, ren=5000.0,
         dtmin=1e-5, dtmax=1e-3, limitCFL=1.2),
    # radial sweeps whose levels above the first fill whole checkpoint batches
    # (17 cells: theta and z components; 18: the radial faces)
    dict(nthm=32, nzm=32, nrm=17),
    dict(nthm=32, nzm=32, nrm=18),
], ids=["C1-64cubed", "cheb-variable-dt", "nr17", "nr18"])
@pytest.mark.parametrize("precision", ["mixed", "mixed-ff"])
def test_mixed_twenty_steps_vs_fp64(gpu_lib, oracle, case, precision):
    """Both pressure-solve options: FP64 (the default) and float-float."""
    bou = make_bou(**case)
    g, o = pair(oracle, bou, precision=precision)
    assert g.L.tc_precision(g.h) == {"mixed": 1, "mixed-ff": 2}[precision]
    code_g, n_g, t_g, _ = g.run(20, 0, 0.0)
    code_o, t_o, _ = o.run(0, 20, 0.0)
    assert code_g == code_o == 0
    gs, os_ = g.get_state(), o.state()
    nrm = bou["nrm"]
    errs = [rel_err(a, b, nk=nk) for a, b, nk in zip(gs[:3], os_[:3], (nrm, nrm + 1, nrm))]
    ti_g, to_g = g.calc_torque()
    ti_o, to_o = o.calc_torque()
    terr = max(abs(ti_g - ti_o) / abs(ti_o), abs(to_g - to_o) / abs(to_o))
    div = g.check_divergence()
    print(precision, case, "velocity", errs, "torque", terr, "div", div)
    assert max(errs) < 1e-3
    assert terr < 1e-4
    assert div < 1e-3 * bou["resid"]
    g.close()


@pytest.mark.parametrize("case", [
    dict(nthm=64, nzm=64, nrm=40, istr=6, str=3.0),                    # one theta tile: both periodic edges
    dict(nthm=192, nzm=30, nrm=37, istr=4, str=2.0, romeg=0.1,          # 3 tiles, z and r not multiples of
         sizepert=0.1, omegapert=0.5, dtmin=2e-4, dtmax=2e-4),           # the tile, rotating, oscillating wall
    dict(nthm=96, nzm=20, nrm=17, minstrt=2, minstrz=1, multmin=2),      # partial theta tile, patterned slip
], ids=["64x64x40", "192x30x37-rot", "96x20x17-slip"])
def test_tma_march_equals_cached_march(gpu_lib, case):
    """The TMA-staged march and the march that loads through the read-only
    cache run the same arithmetic on the same values: identical bits after
    several steps (all three RK substeps, the wall rows and the edges)."""
    bou = make_bou(**case)
    st = ini.couette_noise(bou, seed=21, amp=0.05)
    out = []
    for tma in (True, False):
        g = tc.TaylorCouette(bou, precision="mixed")
        g.use_tma(tma)
        g.set_state(*st)
        code, n, t, _ = g.run(4, 0, 0.0)
        assert code == 0
        out.append(g.get_state())
        g.close()
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


def test_tma_unavailable_is_reported(gpu_lib):
    g = tc.TaylorCouette(make_bou(nthm=30, nzm=16, nrm=8), precision="mixed")
    with pytest.raises(tc.TCError) as e:
        g.use_tma(True)
    assert e.value.code == 2019
    g.use_tma(False)
    g.close()


def test_mixed_state_round_trip_is_fp32(gpu_lib):
    bou = make_bou(nthm=24, nzm=18, nrm=10)
    st = ini.couette_noise(bou, seed=3)
    g = tc.TaylorCouette(bou, precision="mixed")
    g.set_state(*st)
    back = g.get_state()
    np.testing.assert_array_equal(back[0][..., :10], st[0][..., :10].astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(back[3], st[3])   # pressure stays FP64
    g.close()


def test_integer_pipe_conversions_match_hardware(gpu_lib):
    """The mixed path converts float <-> double on the integer pipes; every
    result must equal the hardware conversion bit for bit."""
    assert tc.selftest_conversions(1 << 24) == 0
