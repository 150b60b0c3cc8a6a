"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

The oracle (oracle/tc_ref.cpp) restates the reference Fortran routines; both
solve the singular k_theta = k_z = 0 pressure mode with phi(nrm) = 0, so every
field, pressure included, is compared directly.

Tolerances (relative to the max-norm of the oracle field):
  * one routine on the same input: 2e-11 (velocities and explicit terms: the
    flux differences of a stretched grid cancel a few digits, so FMA
    contraction shows), 1e-10 (pressure and phi, which carry the conditioning
    of the near-singular k = 0 mode);
  * one full time step: 1e-12 (velocities), 1e-10 (pressure);
  * 20 RK3 steps: 1e-10 (velocities and pressure), torques 1e-10;
  * one step at the full 512 x 512 x 384 size: 1e-12 (velocities), 1e-10.
"""
import numpy as np
import pytest

from conftest import make_bou, rel_err, tc

import tc_gb300.initial as ini

pytestmark = pytest.mark.gpu

TOL_ROUTINE = 2e-11     # one routine: flux differences on stretched grids cancel digits
TOL_PR = 1e-10          # pressure: carries the near-singular k = 0 mode
TOL_STEP = 1e-12
TOL_20 = 1e-10


def pair(oracle, bou, seed=5, amp=0.01):
    st = ini.couette_noise(bou, seed=seed, amp=amp)
    g = tc.TaylorCouette(bou)
    g.set_state(*st)
    o = oracle.CppOracle(bou)
    o.set_state(*st)
    return g, o, st


def compare_state(g, o, tol, nrm, tol_pr=TOL_PR):
    gs, os_ = g.get_state(), o.state()
    errs = {}
    for name, a, b, nk in zip(("qt", "qr", "qz", "pr"), gs, os_, (nrm, nrm + 1, nrm, nrm)):
        errs[name] = rel_err(a, b, nk=nk)
    assert max(errs["qt"], errs["qr"], errs["qz"]) < tol, errs
    assert errs["pr"] < max(tol, tol_pr), errs
    return errs


@pytest.mark.parametrize("case", [
    dict(),
    dict(nthm=48, nzm=40, nrm=24, istr=4, str=3.0, sizepert=0.1, omegapert=0.5, romeg=0.1, dtmin=1e-4, dtmax=1e-4),
    dict(nthm=32, nzm=96, nrm=20, istr=6, str=3.0),
    dict(nthm=20, nzm=30, nrm=12, nsst=1),
], ids=["uniform64", "tanh-osc-rot", "cheb-radix3", "ab2-radix5"])
def test_routines_one_substep(gpu_lib, oracle, case):
    """Each routine of substep 1 (then 2) on identical input."""
    bou = make_bou(**case)
    g, o, _ = pair(oracle, bou)
    dt = bou["dtmax"]
    nrm = bou["nrm"]
    g.begin_step(dt, 0.37)
    o.call("begin_step", dt, 0.37)
    for ns in range(1, bou["nsst"] + 1):
        g.set_substep(ns)
        o.call("set_substep", ns)
        g.explicit_terms()
        for f in ("explicit_terms_qt", "explicit_terms_qr", "explicit_terms_qz"):
            o.call(f)
        assert rel_err(g.get_field("dq"), o.get(oracle.DQ), interior=False, nk=nrm) < TOL_ROUTINE
        assert rel_err(g.get_field("qcap"), o.get(oracle.QCAP), interior=False, nk=nrm) < TOL_ROUTINE
        hr_o = o.get(oracle.DPH)[1:-1, 1:-1, 1:nrm]
        assert rel_err(g.get_field("hr")[..., 1:nrm], hr_o, interior=False) < TOL_ROUTINE
        g.implicit_and_update()
        for f in ("implicit_rhs_qt", "solve_imp_eqn_update_qt", "implicit_rhs_qr", "solve_imp_eqn_update_qr",
                  "implicit_rhs_qz", "solve_imp_eqn_update_qz"):
            o.call(f)
        for w in (oracle.QT, oracle.QR, oracle.QZ):
            o.call("update_halo", w)
        for name, w in (("ru1", oracle.RU1), ("ru2", oracle.RU2), ("ru3", oracle.RU3)):
            lo = 1 if name == "ru2" else 0
            hi = nrm
            assert rel_err(g.get_field(name)[..., lo:hi], o.get(w)[..., lo:hi], interior=False) < TOL_ROUTINE, name
        compare_state(g, o, TOL_ROUTINE, nrm)
        g.calc_local_divergence()
        o.call("calc_local_divergence")
        assert rel_err(g.get_field("dph"), o.get(oracle.DPH), nk=nrm) < TOL_ROUTINE
        g.solve_pressure_correction()
        o.call("solve_pressure_correction")
        o.call("update_halo", oracle.DPH)
        assert rel_err(g.get_field("dph"), o.get(oracle.DPH), nk=nrm) < TOL_PR
        g.correct_velocity()
        o.call("correct_velocity")
        g.correct_pressure()
        o.call("correct_pressure")
        for w in (oracle.QT, oracle.QR, oracle.QZ, oracle.PR):
            o.call("update_halo", w)
        compare_state(g, o, TOL_ROUTINE, nrm)
    g.close()


@pytest.mark.parametrize("case", [
    dict(nthm=32, nzm=40, nrm=28),
    dict(nthm=48, nzm=40, nrm=24, istr=4, str=3.0, sizepert=0.1, omegapert=0.5, romeg=0.1, dtmin=1e-4, dtmax=1e-4),
    dict(nthm=40, nzm=24, nrm=20, istr=6, str=3.0, minstrt=2, minstrz=1, multmin=2),
], ids=["uniform", "tanh-osc-rot", "cheb-patterned-slip"])
def test_routines_one_component_at_a_time(gpu_lib, oracle, case):
    """The per-component entry points in TimeMarcher.F90:31-37 order, each
    checked against the oracle's routine of the same name right after it
    runs, for two substeps; then the three-component entry points on the
    same input give the same fields."""
    bou = make_bou(**case)
    g, o, st = pair(oracle, bou)
    dt, nrm = bou["dtmax"], bou["nrm"]
    g.begin_step(dt, 0.21)
    o.call("begin_step", dt, 0.21)
    for ns in (1, 2):
        g.set_substep(ns)
        o.call("set_substep", ns)
        g.explicit_terms_qt()
        o.call("explicit_terms_qt")
        assert rel_err(g.get_field("dq"), o.get(oracle.DQ), interior=False, nk=nrm) < TOL_ROUTINE
        g.explicit_terms_qr()
        o.call("explicit_terms_qr")
        hr_o = o.get(oracle.DPH)[1:-1, 1:-1, 1:nrm]
        assert rel_err(g.get_field("hr")[..., 1:nrm], hr_o, interior=False) < TOL_ROUTINE
        g.explicit_terms_qz()
        o.call("explicit_terms_qz")
        assert rel_err(g.get_field("qcap"), o.get(oracle.QCAP), interior=False, nk=nrm) < TOL_ROUTINE
        for comp, ru, w, nk in (("qt", "ru1", oracle.QT, nrm), ("qr", "ru2", oracle.QR, nrm + 1),
                                ("qz", "ru3", oracle.QZ, nrm)):
            getattr(g, "implicit_and_update_" + comp)()
            o.call("implicit_rhs_" + comp)
            o.call("solve_imp_eqn_update_" + comp)
            o.call("update_halo", w)
            lo = 1 if comp == "qr" else 0
            wr = {"ru1": oracle.RU1, "ru2": oracle.RU2, "ru3": oracle.RU3}[ru]
            assert rel_err(g.get_field(ru)[..., lo:nrm], o.get(wr)[..., lo:nrm], interior=False) < TOL_ROUTINE, ru
            got = g.get_state()[("qt", "qr", "qz").index(comp)]
            assert rel_err(got, o.get(w), nk=nk) < TOL_ROUTINE, comp
        g.calc_local_divergence()
        o.call("calc_local_divergence")
        g.solve_pressure_correction()
        o.call("solve_pressure_correction")
        o.call("update_halo", oracle.DPH)
        g.correct_velocity()
        o.call("correct_velocity")
        g.correct_pressure()
        o.call("correct_pressure")
        for w in (oracle.QT, oracle.QR, oracle.QZ, oracle.PR):
            o.call("update_halo", w)
        compare_state(g, o, TOL_ROUTINE, nrm)
    # the grouped entry points run the same arithmetic per component
    h = tc.TaylorCouette(bou)
    for x in (g, h):
        x.set_state(*st)
        x.begin_step(dt, 0.21)
        x.set_substep(1)
    for comp in ("qt", "qr", "qz"):
        getattr(g, "explicit_terms_" + comp)()
    for comp in ("qt", "qr", "qz"):
        getattr(g, "implicit_and_update_" + comp)()
    h.explicit_terms()
    h.implicit_and_update()
    for a, b in zip(g.get_state()[:3], h.get_state()[:3]):
        np.testing.assert_array_equal(a, b)
    g.close()
    h.close()


def test_fused_step_matches_routines(gpu_lib, oracle):
    """tc_time_marcher (fused kernels) equals the oracle's TimeMarcher."""
    bou = make_bou(nthm=32, nzm=48, nrm=32)
    g, o, _ = pair(oracle, bou)
    g.time_marcher(1e-3, 0.0)
    o.time_marcher(1e-3, 0.0)
    compare_state(g, o, TOL_STEP, bou["nrm"])
    g.close()


@pytest.mark.parametrize("case", [
    dict(),
    dict(nthm=64, nzm=48, nrm=96, istr=6, str=20.0, sizepert=0.1, omegapert=0.5, romeg=0.1, ren=5000.0,
         dtmin=1e-5, dtmax=1e-3, limitCFL=1.2),
    dict(nthm=48, nzm=32, nrm=32, istr=4, str=2.0, sizepert=0.1, omegapert=0.5, ren=2000.0,
         dtmin=1e-5, dtmax=2e-4, limitCFL=1.2),
], ids=["C1-64cubed-fixed-dt", "cheb-variable-dt", "tanh-variable-dt"])
def test_twenty_steps(gpu_lib, oracle, case):
    """20 steps (NTST = 19 in the reference's 0..NTST loop) through tc_run."""
    bou = make_bou(**case)
    g, o, _ = pair(oracle, bou)
    code_g, n_g, t_g, dt_g = g.run(20, 0, 0.0)
    code_o, t_o, dt_o = o.run(0, 20, 0.0)
    assert code_g == code_o == 0
    assert n_g == 20
    assert abs(t_g - t_o) <= 1e-12 * abs(t_o)
    errs = compare_state(g, o, TOL_20, bou["nrm"])
    ti_g, to_g = g.calc_torque()
    ti_o, to_o = o.calc_torque()
    assert abs(ti_g - ti_o) <= TOL_20 * abs(ti_o)
    assert abs(to_g - to_o) <= TOL_20 * abs(to_o)
    assert g.check_divergence() < bou["resid"]
    print(case, errs, (ti_g, to_g))
    g.close()


def test_reductions(gpu_lib, oracle):
    bou = make_bou(nthm=48, nzm=64, nrm=40, istr=4)
    g, o, _ = pair(oracle, bou, amp=0.05)
    assert abs(g.calc_max_cfl() - o.calc_max_cfl()) <= 1e-13 * o.calc_max_cfl()
    assert abs(g.check_divergence() - o.check_divergence()) <= 1e-12 * o.check_divergence()
    ti, to = g.calc_torque()
    ri, ro = o.calc_torque()
    assert abs(ti - ri) <= 1e-12 * abs(ri) and abs(to - ro) <= 1e-12 * abs(ro)
    vg, rg = g.velocity_stats()
    vo, ro_ = o.velocity_stats()
    np.testing.assert_allclose(vg, vo, rtol=1e-14)
    np.testing.assert_allclose(rg, ro_, rtol=1e-12)
    g.close()


def test_patterned_slip(gpu_lib, oracle):
    """SlipBCs with MINSTRT, MINSTRZ, MULTMIN non-zero (rotating free-slip bands)."""
    bou = make_bou(nthm=32, nzm=32, nrm=24, minstrt=2, minstrz=1, multmin=2)
    g, o, _ = pair(oracle, bou)
    t = 0.0
    for n in range(3):
        g.time_marcher(1e-3, t)
        o.time_marcher(1e-3, t)
        t += 0.25   # rotate the pattern between steps
    compare_state(g, o, 1e-11, bou["nrm"])
    ti, to = g.calc_torque()
    ri, ro = o.calc_torque()
    assert abs(ti - ri) <= 1e-11 * abs(ri)
    g.close()


def test_dt_changes_between_steps(gpu_lib, oracle):
    """The momentum factors are kept while dt repeats and rebuilt when it
    changes; the inner-wall oscillation (SIZEPERT, OMEGAPERT) changes the
    wall term of every step, cached factors or not."""
    bou = make_bou(nthm=32, nzm=24, nrm=20, istr=4, str=3.0, sizepert=0.1, omegapert=0.5)
    g, o, _ = pair(oracle, bou)
    t = 0.0
    for dt in (1e-3, 1e-3, 5e-4, 5e-4, 1e-3, 7e-4):
        g.time_marcher(dt, t)
        o.time_marcher(dt, t)
        t += dt
    compare_state(g, o, 1e-11, bou["nrm"])
    g.close()


def test_state_round_trip(gpu_lib):
    bou = make_bou(nthm=24, nzm=18, nrm=10)
    st = ini.couette_noise(bou, seed=3)
    g = tc.TaylorCouette(bou)
    g.set_state(*st)
    back = g.get_state()
    for a, b in zip(back[:3], st[:3]):
        np.testing.assert_array_equal(a[..., :bou["nrm"]], b[..., :bou["nrm"]])
    np.testing.assert_array_equal(back[1], st[1])
    g.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_state_transfer_from_pinned_memory(gpu_lib, precision):
    """State transfer from and into pinned host arrays (copy-engine copies at
    the link rate) gives the same fields as from pageable arrays."""
    import torch
    bou = make_bou(nthm=40, nzm=36, nrm=22, istr=6, str=3.0)
    st = ini.couette_noise(bou, seed=9)
    pinned = []
    for a in st:
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
        t.numpy()[...] = a
        pinned.append(t)
    g = tc.TaylorCouette(bou, precision=precision)
    g.set_state(*[t.numpy() for t in pinned])
    g.time_marcher(1e-3, 0.0)
    staged = g.get_state()
    outs = [torch.empty(a.shape, dtype=torch.float64, pin_memory=True) for a in st]
    direct = g.get_state(out=[t.numpy() for t in outs])
    for a, b in zip(staged, direct):
        np.testing.assert_array_equal(a, b)
    h = tc.TaylorCouette(bou, precision=precision)
    h.set_state(*st)                          # pageable: staged upload
    h.time_marcher(1e-3, 0.0)
    for a, b in zip(h.get_state(), staged):
        np.testing.assert_array_equal(a, b)
    g.close()
    h.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_state_transfer_through_host_arrays(gpu_lib, precision):
    """tc_host_alloc buffers (page-locked, on huge pages) in and out give the
    same fields as pageable arrays; the memory goes back when the arrays
    do."""
    import gc
    bou = make_bou(nthm=40, nzm=36, nrm=22, istr=6, str=3.0)
    st = ini.couette_noise(bou, seed=10)
    ins = [tc.host_array(a.shape) for a in st]
    outs = [tc.host_array(a.shape) for a in st]
    for a, b in zip(ins, st):
        assert not a.any() and a.ctypes.data % 4096 == 0
        a[...] = b
    g = tc.TaylorCouette(bou, precision=precision)
    g.set_state(*ins)
    g.time_marcher(1e-3, 0.0)
    g.get_state(out=outs)
    h = tc.TaylorCouette(bou, precision=precision)
    h.set_state(*st)
    h.time_marcher(1e-3, 0.0)
    for a, b in zip(h.get_state(), outs):
        np.testing.assert_array_equal(a, b)
    g.close()
    h.close()
    del ins, outs, a, b
    gc.collect()
    for _ in range(3):                        # allocate and release again
        x = tc.host_array((1 << 20,))
        x[-1] = 1.0
        del x
        gc.collect()


def test_error_codes(gpu_lib, oracle):
    """main.F90 exits: 166 (dt < DTMIN), 333 (time > TMAX), 555 (NTST)."""
    cases = [dict(dtmin=1e-2, dtmax=1e-3, nthm=16, nzm=16, nrm=12),
             dict(tmax=2.5e-3, nthm=16, nzm=16, nrm=12),
             dict(ntst=3, nthm=16, nzm=16, nrm=12)]
    for c in cases:
        bou = make_bou(**c)
        g, o, _ = pair(oracle, bou)
        code_g, n_g, t_g, _ = g.run(10, 0, 0.0)
        code_o, t_o, _ = o.run(0, 10, 0.0)
        assert code_g == code_o != 0, (c, code_g, code_o)
        assert abs(t_g - t_o) < 1e-15
        compare_state(g, o, 1e-11, bou["nrm"])
        g.close()


def test_full_size_one_step(gpu_lib, oracle):
    """The production-size grid (512 x 512 x 384, wall-clustered ISTR=6):
    one variable-dt step through tc_run against the oracle, then
    size-independent properties of a few more steps (divergence at roundoff,
    torques finite, no error code)."""
    bou = make_bou(nthm=512, nzm=512, nrm=384, istr=6, str=20.0, ren=5000.0, sizepert=0.1,
                   omegapert=0.5, dtmin=1e-5, dtmax=1e-3, limitCFL=1.2)
    oracle.set_threads(0)
    g, o, st = pair(oracle, bou, seed=1234)
    del st
    code_g, n_g, t_g, _ = g.run(1, 0, 0.0)
    code_o, t_o, _ = o.run(0, 1, 0.0)
    assert code_g == code_o == 0 and t_g == t_o
    compare_state(g, o, 1e-12, bou["nrm"])
    del o
    d0 = g.check_divergence()
    code, n, t, dt = g.run(3, n_g, t_g)
    assert code == 0 and n == 4
    assert g.check_divergence() < 1e-9 and d0 < 1e-9
    ti, to = g.calc_torque()
    assert 0.1 < ti < 10 and 0.1 < to < 10
    g.close()
