"""The CPU oracle (test infrastructure) checked against an independent
restatement that calls the real LAPACK ?gttrf/?gttrs (scipy) and numpy.fft, and
against physics known-answer tests.  The reference ships no golden vectors, so
this is how the oracle is pinned."""
import numpy as np
import pytest

from conftest import make_bou, rel_err

import tc_gb300.initial as ini
import tc_np


def run_both(oracle, bou, nsteps, dt, pin=True, seed=7):
    st = ini.couette_noise(bou, seed=seed)
    c = oracle.CppOracle(bou, oracle.MODE00_PIN if pin else oracle.MODE00_LAPACK)
    n = tc_np.NpOracle(bou, pin_mode00=pin)
    c.set_state(*st)
    n.set_state(*st)
    t = 0.0
    for _ in range(nsteps):
        c.time_marcher(dt, t)
        n.time_marcher(dt, t)
        t += dt
    return c, n


@pytest.mark.parametrize("case,dt", [
    (dict(nthm=16, nzm=24, nrm=16), 1e-3),
    (dict(nthm=16, nzm=24, nrm=20, istr=4, sizepert=0.1, omegapert=0.5, romeg=0.1), 2e-5),
    (dict(nthm=12, nzm=18, nrm=16, istr=6, str=3.0), 1e-3),
    (dict(nthm=12, nzm=10, nrm=8, nsst=1), 1e-3),
], ids=["uniform", "tanh-osc-rot", "cheb", "ab2"])
def test_cpp_matches_lapack_numpy(oracle, case, dt):
    bou = make_bou(**case)
    c, n = run_both(oracle, bou, 5, dt)
    nrm = bou["nrm"]
    for w, a, nk in ((oracle.QT, n.qt, nrm), (oracle.QR, n.qr, nrm + 1), (oracle.QZ, n.qz, nrm), (oracle.PR, n.pr, nrm)):
        assert rel_err(c.get(w), a, nk=nk) < 1e-11, w
    ti, to = c.calc_torque()
    ni, no = n.calc_torque()
    assert abs(ti - ni) < 1e-12 * abs(ni) and abs(to - no) < 1e-12 * abs(no)
    assert abs(c.calc_max_cfl() - n.calc_max_cfl()) < 1e-12 * n.calc_max_cfl()


def test_mode00_only_moves_pressure(oracle):
    """The singular k=0 pressure mode: LAPACK's roundoff pivot (real LAPACK in
    numpy) versus the pinned solve changes velocities only at roundoff."""
    bou = make_bou(nthm=16, nzm=16, nrm=16)
    st = ini.couette_noise(bou, seed=2)
    c = oracle.CppOracle(bou, oracle.MODE00_PIN)
    n = tc_np.NpOracle(bou, pin_mode00=False)
    c.set_state(*st)
    n.set_state(*st)
    for s in range(10):
        c.time_marcher(1e-3, s * 1e-3)
        n.time_marcher(1e-3, s * 1e-3)
    for w, a, nk in ((oracle.QT, n.qt, 16), (oracle.QR, n.qr, 17), (oracle.QZ, n.qz, 16)):
        assert rel_err(c.get(w), a, nk=nk) < 1e-12


def test_laminar_couette_torque(oracle):
    """CalcTorque normalises by the laminar torque: circular Couette flow gives
    torque -> 1 at both walls as the radial grid is refined (the wall gradient
    of CalcTorque.F90:38-42 is first-order accurate)."""
    errs = []
    for nrm in (32, 64, 128):
        bou = make_bou(nthm=8, nzm=8, nrm=nrm)
        st = ini.couette_noise(bou, seed=1, amp=0.0)
        c = oracle.CppOracle(bou)
        c.set_state(*st)
        for s in range(3):
            c.time_marcher(1e-3, s * 1e-3)
        ti, to = c.calc_torque()
        errs.append(max(abs(ti - 1.0), abs(to - 1.0)))
        assert c.check_divergence() < 1e-12
    assert errs[1] < 0.02
    assert errs[1] < errs[0] / 1.8 and errs[2] < errs[1] / 1.8, errs


def test_projection_is_divergence_free(oracle):
    bou = make_bou(nthm=16, nzm=16, nrm=16, istr=4)
    st = ini.couette_noise(bou, seed=4, amp=0.05)
    c = oracle.CppOracle(bou)
    c.set_state(*st)
    d0 = c.check_divergence()
    c.time_marcher(1e-4, 0.0)
    assert d0 > 1.0
    assert c.check_divergence() < 1e-11 * d0


def test_run_error_codes(oracle):
    bou = make_bou(nthm=8, nzm=8, nrm=8, tmax=2.5e-3)
    st = ini.couette_noise(bou, seed=1)
    c = oracle.CppOracle(bou)
    c.set_state(*st)
    code, t, dt = c.run(0, 10, 0.0)
    assert code == 333 and abs(t - 3e-3) < 1e-15
    bou = make_bou(nthm=8, nzm=8, nrm=8, ntst=2)
    c = oracle.CppOracle(bou)
    c.set_state(*st)
    code, t, dt = c.run(0, 10, 0.0)
    assert code == 555 and abs(t - 3e-3) < 1e-15


def test_thread_count_does_not_change_results(oracle):
    bou = make_bou(nthm=16, nzm=16, nrm=16)
    st = ini.couette_noise(bou, seed=9)
    res = []
    for th in (1, 4):
        oracle.set_threads(th)
        c = oracle.CppOracle(bou)
        c.set_state(*st)
        c.time_marcher(1e-3, 0.0)
        res.append(c.state())
    oracle.set_threads(0)
    for a, b in zip(*res):
        np.testing.assert_array_equal(a, b)


def test_tanh_grid_with_str4_is_unstable_in_the_reference_algorithm(oracle):
    """Why the production workload uses the ISTR=6, STR3=20 radial grid of the
    reference's bou.in: with the tanh grid ISTR=4, STR3=4 at 384 radial cells
    (wall cell 5.7e-6 wide, 700 times smaller than the widest) the reference
    algorithm blows up within a few steps even at dt = 1e-4 (velocity limited
    by CFL, not by this), while ISTR=6 with STR3=20 stays bounded."""
    def vmax_after(istr, st, nsteps=4, dt=1e-4):
        bou = make_bou(nthm=16, nzm=16, nrm=384, istr=istr, str=st, ren=5000.0, sizepert=0.1, omegapert=0.5)
        c = oracle.CppOracle(bou)
        c.set_state(*ini.couette_noise(bou, seed=1234))
        for s in range(nsteps):
            c.time_marcher(dt, s * dt)
        return float(c.velocity_stats()[0].max())
    assert vmax_after(4, 4.0) > 1e3
    assert vmax_after(6, 20.0) < 2.0


# ---- statistics (StatRoutines.F90, CalcVorticity.F90, CalcDissipation.F90) ----

def _couette(oracle_mod, bou):
    import tc_gb300.initial as ini
    st = ini.couette_noise(bou, seed=1, amp=0.0)
    o = oracle_mod.CppOracle(bou)
    o.set_state(*st)
    o.call("update_halo", oracle_mod.QT)
    return o


def test_stats_of_laminar_couette(oracle):
    """Circular Couette flow: the theta mean of qt is the profile itself, its
    rms equals the mean squared, the axial vorticity is 2A in the interior
    (A r + B/r has curl 2A), and the normalised dissipation nute -> 1 as the
    radial grid is refined."""
    from conftest import make_bou
    errs = []
    for nrm in (16, 32, 64):
        bou = make_bou(nthm=16, nzm=8, nrm=nrm, istr=0, virotint=1.0, virotext=0.0)
        o = _couette(oracle, bou)
        o.calc_stats()
        nute = o.calc_dissipation()
        assert o.stat_samples() == 1
        qt = o.state()[0]
        vt = o.stat(oracle.STAT_NAMES.index("vt_mean"))
        assert np.allclose(vt, qt[1, 1:-1, :nrm], rtol=1e-14, atol=1e-15)
        vt2 = o.stat(oracle.STAT_NAMES.index("vt_rms"))
        assert np.allclose(vt2, vt ** 2, rtol=1e-13)
        eta = bou["rint"] / bou["rext"]
        A = (bou["virotext"] - eta * eta * bou["virotint"]) / (1 - eta * eta)
        wz = o.vorticity(2)
        assert np.allclose(wz[:, :, 1:-1], 2 * A, rtol=1e-9)
        errs.append(abs(nute - 1.0))
    # first order in the radial spacing (the outer-wall cell's gradients are one-sided)
    assert 1.8 < errs[0] / errs[1] < 2.4 and 1.8 < errs[1] / errs[2] < 2.4 and errs[2] < 0.011


def test_stats_accumulate_and_quirks(oracle):
    """Two samples of one field are twice one sample; vtvz_mean uses qr(k,j+1)
    as StatRoutines.F90:58 does (not qz), checked against a direct sum."""
    from conftest import make_bou
    import tc_gb300.initial as ini
    bou = make_bou(nthm=12, nzm=10, nrm=8, istr=6, str=3.0)
    st = ini.couette_noise(bou, seed=3, amp=0.3)
    o = oracle.CppOracle(bou)
    o.set_state(*st)
    for a in (oracle.QT, oracle.QR, oracle.QZ, oracle.PR):
        o.call("update_halo", a)
    o.calc_stats()
    one = [o.stat(w).copy() for w in range(len(oracle.STAT_NAMES))]
    o.calc_stats()
    for w in range(len(oracle.STAT_NAMES) - 1):
        assert np.allclose(o.stat(w), 2 * one[w], rtol=1e-13, atol=1e-300)
    qt, qr, qz, _ = o.state()
    usrc = o.grid("usrc")
    nthm, nzm, nrm = 12, 10, 8
    want = np.zeros((nzm, nrm))
    for i in range(1, nthm + 1):
        for j in range(1, nzm + 1):
            for k in range(1, nrm + 1):
                want[j - 1, k - 1] += (qt[i, j, k - 1] + qt[i + 1, j, k - 1]) * (qz[i, j, k - 1] + qr[i, j + 1, k - 1]) \
                    / nthm * 0.25
    assert np.allclose(one[oracle.STAT_NAMES.index("vtvz_mean")], want, rtol=1e-12, atol=1e-15)


def test_clustered_grid_needs_small_dt_in_the_reference_algorithm(oracle):
    """On the C2 radial grid (nrm = 384, ISTR = 6, STR3 = 20, smallest cell
    2.3e-4) an unperturbed Couette flow grows an axial mode from roundoff at
    dt = 1e-3 (U dt / dr_min = 4.3) although its CFL number allows it, and
    stays at roundoff at dt = 3e-4: the reason the clustered bench workloads
    cap DTMAX."""
    from conftest import make_bou
    import tc_gb300.initial as ini
    out = {}
    for dt in (1e-3, 3e-4):
        bou = make_bou(nthm=16, nzm=16, nrm=384, istr=6, str=20.0, ren=5000.0, idtv=1, limitCFL=1.2,
                       dtmin=1e-5, dtmax=dt)
        o = oracle.CppOracle(bou)
        o.set_state(*ini.couette_noise(bou, seed=1, amp=0.0))
        code, t, d = o.run(0, 40, 0.0)
        out[dt] = o.velocity_stats()[0][2]
    assert out[1e-3] > 1e-10 and out[3e-4] < 1e-15
