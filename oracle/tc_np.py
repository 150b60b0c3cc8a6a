"""Second, independent CPU restatement of the reference time step (NumPy/SciPy).

TEST INFRASTRUCTURE ONLY: used by tests/ to cross-check the C++ oracle
(oracle/tc_ref.cpp); never part of the product path.

Unlike the C++ oracle this one is vectorised with NumPy, calls the real LAPACK
``dgttrf/dgttrs/zgttrf/zgttrs`` through ``scipy.linalg.lapack`` (the routines the
reference links, SolveImpEqnUpdate_QT.F90:63,74, SolvePressureCorrection.F90:139,141)
and ``numpy.fft`` (pocketfft) in place of FFTW.  Arrays use the reference memory
layout: a NumPy array of shape (nthm+2, nzm+2, nr) in C order is the Fortran
array q(1:nr, 0:nzm+1, 0:nthm+1); index [i, j, k-1].

Parity status: the C++ oracle it cross-checks is pinned to runs of the
reference's own source (tests/golden/reference_runs.npz, made by
tests/golden/make_reference_runs.py).
"""
from __future__ import annotations

import math

import numpy as np
from scipy.linalg import lapack

BOU_FIELDS = [
    ("nthm", int), ("nzm", int), ("nrm", int), ("nsst", int), ("idtv", int), ("nread", int),
    ("ntst", int), ("tout", float), ("tmax", float), ("ireset", int), ("walltimemax", float),
    ("alx3", float), ("rint", float), ("rext", float), ("istr", int), ("str", float), ("lamb", float),
    ("virotint", float), ("virotext", float), ("sizepert", float), ("omegapert", float),
    ("ren", float), ("romeg", float), ("resid", float), ("limitCFL", float),
    ("tsta", float), ("starea", int),
    ("dtmin", float), ("dtmax", float), ("limitVel", float), ("cfllim", float),
    ("nslabr", int), ("dpthcut", int), ("dpstave", int), ("tframe2d", float),
    ("dpfullf", int), ("tframe3d", float),
    ("minstrt", int), ("minstrz", int), ("multmin", int),
]


class NpOracle:
    """Reference routines restated on whole arrays (serial semantics)."""

    def __init__(self, bou: dict, pin_mode00: bool = True):
        self.b = dict(bou)
        b = self.b
        self.pin = pin_mode00
        self.nthm, self.nzm, self.nrm = int(b["nthm"]), int(b["nzm"]), int(b["nrm"])
        self.nr = self.nrm + 1
        self._init_scheme()
        self._grid()
        self._pressure_init()
        shp = (self.nthm + 2, self.nzm + 2, self.nr)
        self.qt, self.qr, self.qz, self.pr, self.dph = (np.zeros(shp) for _ in range(5))
        shn = (self.nthm, self.nzm, self.nr)
        self.ru1, self.ru2, self.ru3 = (np.zeros(shn) for _ in range(3))
        self.time = 0.0
        self.icylsl = np.ones((self.nthm, self.nzm), dtype=np.int64)  # [i, j]
        self.ocylsl = np.ones((self.nthm, self.nzm), dtype=np.int64)

    # InitTimeMarchScheme.F90:16-49
    def _init_scheme(self):
        if self.b["nsst"] > 1:
            self.gam = [8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0]
            self.rom = [0.0, -17.0 / 60.0, -5.0 / 12.0]
        else:
            self.gam = [1.5, 0.0, 0.0]
            self.rom = [-0.5, 0.0, 0.0]
        self.alm = [g + r for g, r in zip(self.gam, self.rom)]

    # CreateGrid.F90:24-322 (1-based arrays of length nr+1, entry 0 unused)
    def _grid(self):
        b = self.b
        nrm, nr, nthm, nzm = self.nrm, self.nr, self.nthm, self.nzm
        pi = 2.0 * math.asin(1.0)
        self.pi = pi
        self.dxt = (float(nthm) * b["lamb"]) / (2.0 * pi)
        self.dxz = float(nzm) / b["alx3"]
        self.dxr = float(nrm)
        dxr, dxt = self.dxr, self.dxt
        self.dxtq, self.dxzq, self.dxrq = dxt * dxt, self.dxz * self.dxz, dxr * dxr
        dxrq = self.dxrq
        z = lambda: np.zeros(nr + 1)
        rc = z()
        k = np.arange(1, nr + 1)
        if b["istr"] == 0:
            rc[1:] = (b["rext"] - b["rint"]) * ((k - 1) / nrm) + b["rint"]
        elif b["istr"] == 4:
            tstr = math.tanh(b["str"])
            z2dp = (2 * k - nr - 1) / nrm
            rc[1:] = (1 + np.tanh(b["str"] * z2dp) / tstr) * 0.5 * (b["rext"] - b["rint"]) + b["rint"]
            rc[1] = b["rint"]
        elif b["istr"] == 6:
            nclip = int(b["str"])
            nrmo = nr + 2 * nclip
            kk = np.arange(1, nrmo + 1)
            etazm = np.cos(pi * (kk - 0.5) / nrmo)
            etaz = np.zeros(nr + 1)
            etaz[1:] = etazm[nclip:nclip + nr]
            delet = etaz[1] - etaz[nr]
            etaz[1:] = etaz[1:] / (0.5 * delet)
            rc[1] = b["rint"]
            rc[2:nrm + 1] = (b["rext"] - b["rint"]) * (1.0 - etaz[2:nrm + 1]) * 0.5 + b["rint"]
            rc[nr] = b["rext"]
        rm, g2rm, g2rc = z(), z(), z()
        rm[1:nr] = (rc[1:nr] + rc[2:nr + 1]) * 0.5
        g2rm[1:nr] = (rc[2:nr + 1] - rc[1:nr]) * dxr
        g2rc[1] = (rc[2] - rc[1]) * dxr
        g2rc[2:nr] = (rc[3:nr + 1] - rc[1:nr - 1]) * dxr * 0.5
        g2rc[nr] = (rc[nr] - rc[nrm]) * dxr
        usrm, usrc, udx2rm, udx2m, udx2c, rudx2c, udx1vis1, udx1vis2, udx1qm, pvol = (z() for _ in range(10))
        s = slice(1, nr)
        udx1vis1[s] = 2.0 * dxt / (rm[s] ** 2 * b["ren"])
        udx2rm[s] = dxr / (g2rm[s] * rm[s])
        udx2m[s] = dxr / g2rm[s]
        udx2c[s] = dxr / g2rc[s]
        rudx2c[s] = udx2c[s] * rc[s]
        usrm[s] = 1.0 / rm[s]
        udx1qm[s] = self.dxtq / rm[s] ** 2
        pvol[s] = rc[2:nr + 1] ** 2 - rc[1:nr] ** 2
        udx2c[nr] = dxr / g2rc[nr]
        udx1vis2[1:] = dxt / (rc[1:] * b["ren"])
        usrc[1:] = 1.0 / rc[1:]
        self.rc, self.rm, self.g2rm, self.g2rc = rc, rm, g2rm, g2rc
        self.usrm, self.usrc, self.udx2rm, self.udx2m, self.udx2c = usrm, usrc, udx2rm, udx2m, udx2c
        self.rudx2c, self.udx1vis1, self.udx1vis2, self.udx1qm, self.pvol = rudx2c, udx1vis1, udx1vis2, udx1qm, pvol
        self.kmv = np.array([0] + [max(kc - 1, 1) for kc in range(1, nr + 1)])
        self.kpv = np.array([0] + [min(kc + 1, nrm) for kc in range(1, nr + 1)])
        self.kmv[nr] = 0
        self.kpv[nr] = 0
        # q1 coefficients (CreateGrid.F90:191-238)
        ap1j, am1j, ac1j = z(), z(), z()
        for kc in range(2, nrm):
            a22 = dxrq / g2rm[kc] / rm[kc]
            a22p, a22m = a22 * rc[kc + 1] / g2rc[kc + 1], a22 * rc[kc] / g2rc[kc]
            ap1j[kc], am1j[kc], ac1j[kc] = a22p, a22m, -(a22p + a22m) - 1.0 / rm[kc] ** 2
        kc = nrm
        a22 = dxrq / (g2rm[kc] * rm[kc])
        apjjc, amjjc = a22 * rc[kc + 1] / g2rc[kc + 1], a22 * rc[kc] / g2rc[kc]
        ap1j[kc], ac1j[kc], am1j[kc] = 2.0 * apjjc, -2.0 * apjjc - amjjc - 1.0 / rm[kc] ** 2, amjjc
        kc = 1
        urpp = 1.0 / (g2rm[kc] * g2rc[kc + 1])
        a22 = dxrq / g2rm[kc] / rm[kc]
        a22p, a22m = a22 * rc[2] / g2rc[2], a22 * rc[1] / g2rc[1]
        ap1j[1], am1j[1], ac1j[1] = a22p, 2.0 * a22m, -(a22p + 2.0 * a22m) - 1.0 / rm[1] ** 2
        self.ap1j_fs = [0.0, rc[2] ** 3 / (rm[1] ** 2 * rm[2]) * dxrq * urpp, 0.0]
        self.ac1j_fs = [0.0, -rc[2] ** 3 / rm[1] ** 3 * dxrq * urpp, 0.0]
        self.am1j_fs = [0.0, 0.0, 0.0]
        # q2 (CreateGrid.F90:241-276)
        ap2j, am2j, ac2j, ap2je, am2je, ac2je = (z() for _ in range(6))
        ac2j[1] = 1.0
        ac2j[nr] = 1.0
        for kc in range(2, nrm + 1):
            a22 = rc[kc] * dxrq / g2rc[kc]
            a22p, a22m = 1.0 / (rm[kc] * g2rm[kc]), 1.0 / (rm[kc - 1] * g2rm[kc - 1])
            ap2j[kc], am2j[kc], ac2j[kc] = a22 * a22p, a22 * a22m, -(a22 * a22p + a22 * a22m)
            ugmm = dxrq / g2rc[kc]
            b22p = rm[kc] / (rc[kc + 1] * g2rm[kc])
            b22m = rm[kc - 1] / (rc[kc - 1] * g2rm[kc - 1])
            b22 = (rm[kc] / g2rm[kc] + rm[kc - 1] / g2rm[kc - 1]) / rc[kc]
            ap2je[kc], am2je[kc], ac2je[kc] = b22p * ugmm, b22m * ugmm, -b22 * ugmm - 1.0 / rc[kc] ** 2
        # q3 (CreateGrid.F90:279-322)
        ap3j, am3j, ac3j = z(), z(), z()
        for kc in range(2, nrm):
            a22 = dxrq / g2rm[kc] / rm[kc]
            a22p, a22m = a22 * rc[kc + 1] / g2rc[kc + 1], a22 * rc[kc] / g2rc[kc]
            ap3j[kc], am3j[kc], ac3j[kc] = a22p, a22m, -(a22p + a22m)
        a22 = dxrq / g2rm[1] / rm[1]
        a22p, a22m = a22 * rc[2] / g2rc[2], a22 * rc[1] / g2rc[1]
        am3j[1], ap3j[1], ac3j[1] = 0.0, a22p, -(a22p + 2.0 * a22m)
        self.am3j_fs, self.ap3j_fs, self.ac3j_fs = [0.0, 0.0, 0.0], [0.0, a22p, 0.0], [0.0, -a22p, 0.0]
        kc = nrm
        a22 = dxrq / g2rm[kc] / rm[kc]
        a22m, a22p = a22 * rc[kc] / g2rc[kc], a22 * rc[kc + 1] / g2rc[kc + 1]
        am3j[kc], ap3j[kc], ac3j[kc] = a22m, 0.0, -(a22m + 2.0 * a22p)
        self.am3j_fs[2], self.ap3j_fs[2], self.ac3j_fs[2] = a22m, 0.0, -a22m
        self.ap1j, self.am1j, self.ac1j = ap1j, am1j, ac1j
        self.ap2j, self.am2j, self.ac2j = ap2j, am2j, ac2j
        self.ap2je, self.am2je, self.ac2je = ap2je, am2je, ac2je
        self.ap3j, self.am3j, self.ac3j = ap3j, am3j, ac3j

    # InitPressureSolver.F90:22-66
    def _pressure_init(self):
        nrm, nzm, nthm = self.nrm, self.nzm, self.nthm
        rc, rm, g2rc, g2rm, dxrq = self.rc, self.rm, self.g2rc, self.g2rm, self.dxrq
        self.amph, self.apph, self.acph = (np.zeros(self.nr + 1) for _ in range(3))
        for kc in range(1, nrm + 1):
            kmc = 0 if kc == 1 else 1
            kpc = 0 if kc == nrm else 1
            kp = kc + kpc
            a22icc = rc[kc] * kmc * dxrq / g2rc[kc]
            a22icp = rc[kp] * kpc * dxrq / g2rc[kp]
            ugmmm = 1.0 / (rm[kc] * g2rm[kc])
            self.amph[kc], self.apph[kc], self.acph[kc] = a22icc * ugmmm, a22icp * ugmmm, -(a22icc + a22icp) * ugmmm
        pi = self.pi
        j = np.arange(1, nzm + 1)
        ao = np.where(j <= nzm // 2 + 1, (j - 1) * 2.0 * pi, -(nzm - j + 1) * 2.0 * pi)
        self.ak3 = 2.0 * (1.0 - np.cos(ao / nzm)) * (float(nzm) / self.b["alx3"]) ** 2
        i = np.arange(1, nthm + 1)
        ap = np.where(i <= nthm // 2 + 1, (i - 1) * 2.0 * pi, -(nthm - i + 1) * 2.0 * pi)
        self.ak1 = 2.0 * (1.0 - np.cos(ap / nthm)) * self.dxtq

    # ------------------------------------------------------------------
    def halo(self, a):
        """halo_common.f90:64-71,104-108 (z ghosts, then theta ghosts incl. z ghosts)."""
        a[:, -1, :] = a[:, 1, :]
        a[:, 0, :] = a[:, -2, :]
        a[-1, :, :] = a[1, :, :]
        a[0, :, :] = a[-2, :, :]

    def set_state(self, qt, qr, qz, pr):
        for dst, src in ((self.qt, qt), (self.qr, qr), (self.qz, qz), (self.pr, pr)):
            dst[...] = src
            self.halo(dst)

    def _begin_step(self, dt, time):
        b = self.b
        self.dt, self.time = dt, time
        self.beta = dt / b["ren"] * 0.5
        pi = self.pi
        self.vinner_t = b["sizepert"] * math.sin(2.0 * pi * b["omegapert"] * time)
        self.dvinner_t = 2.0 * pi * b["omegapert"] * b["sizepert"] * math.cos(2.0 * pi * b["omegapert"] * time) * dt
        if b["minstrt"] * b["multmin"] + b["minstrz"] * b["multmin"] != 0:
            raise NotImplementedError("patterned slip is checked through the C++ oracle only")

    # ExplicitTermsQT/QR/QZ on the interior, vectorised
    def explicit_terms(self):
        b = self.b
        nrm, nthm, nzm = self.nrm, self.nthm, self.nzm
        qt, qr, qz = self.qt, self.qr, self.qz
        I, Ip, Im = slice(1, nthm + 1), slice(2, nthm + 2), slice(0, nthm)
        J, Jp, Jm = slice(1, nzm + 1), slice(2, nzm + 2), slice(0, nzm)
        kc = np.arange(1, nrm + 1)
        K, Kp = kc - 1, kc
        Kmm = self.kmv[kc] - 1
        Kpp = self.kpv[kc] - 1
        usrm, usrc, rm = self.usrm[kc], self.usrc[kc], self.rm[kc]
        usrcp = self.usrc[kc + 1]
        udxzq, udxz = self.dxzq / b["ren"], self.dxz * 0.25
        udxt = self.dxt * 0.25 * usrm
        udxtq = self.dxtq / (b["ren"] * rm ** 2)
        c = lambda a, i, j, k: a[i, j][..., k]
        h11 = ((c(qt, Ip, J, K) + c(qt, I, J, K)) ** 2 - (c(qt, I, J, K) + c(qt, Im, J, K)) ** 2) * udxt
        h12d = ((c(qr, I, J, Kp) + c(qr, Im, J, Kp)) * (c(qt, I, J, Kpp) + c(qt, I, J, K))
                - (c(qr, I, J, K) + c(qr, Im, J, K)) * (c(qt, I, J, K) + c(qt, I, J, Kmm))) * 0.25 * self.udx2rm[kc]
        h12n = c(qt, I, J, K) * usrm * ((c(qr, I, J, Kp) + c(qr, Im, J, Kp)) * usrcp
                                        + (c(qr, I, J, K) + c(qr, Im, J, K)) * usrc) * 0.25
        h13 = ((c(qz, I, Jp, K) + c(qz, Im, Jp, K)) * (c(qt, I, Jp, K) + c(qt, I, J, K))
               - (c(qz, I, J, K) + c(qz, Im, J, K)) * (c(qt, I, J, K) + c(qt, I, Jm, K))) * udxz
        d11qt = (c(qt, Ip, J, K) - 2.0 * c(qt, I, J, K) + c(qt, Im, J, K)) * udxtq
        d22qt = (c(qt, I, Jp, K) - 2.0 * c(qt, I, J, K) + c(qt, I, Jm, K)) * udxzq
        qre = c(qr, I, J, Kp) * usrcp + c(qr, I, J, K) * usrc
        qrw = c(qr, Im, J, Kp) * usrcp + c(qr, Im, J, K) * usrc
        d11qre = (qre - qrw) * self.udx1vis1[kc] * 0.5
        coriol = -((c(qr, I, J, K) + c(qr, Im, J, K)) * usrc + (c(qr, I, J, Kp) + c(qr, Im, J, Kp)) * usrcp) * 0.25 * b["romeg"]
        self.dq = -(h11 + h12d + h12n + h13) + d11qre + d22qt + d11qt + coriol
        # QR, kc = 2..nrm
        kr = np.arange(2, nrm + 1)
        K, Kp, Kmm = kr - 1, kr, kr - 2
        usrc_c, usrc_p, usrc_m = self.usrc[kr], self.usrc[kr + 1], self.usrc[kr - 1]
        udxt = self.dxt * 0.25 * usrc_c
        udxtq = self.dxtq / (b["ren"] * self.rc[kr] ** 2)
        h11n = ((c(qt, Ip, J, K) + c(qt, Ip, J, Kmm) + c(qt, I, J, K) + c(qt, I, J, Kmm)) * 0.25) ** 2
        h21 = ((c(qt, Ip, J, K) + c(qt, Ip, J, Kmm)) * (c(qr, Ip, J, K) + c(qr, I, J, K))
               - (c(qt, I, J, K) + c(qt, I, J, Kmm)) * (c(qr, I, J, K) + c(qr, Im, J, K))) * udxt
        h22 = ((c(qr, I, J, Kp) * usrc_p + c(qr, I, J, K) * usrc_c) * (c(qr, I, J, Kp) + c(qr, I, J, K))
               - (c(qr, I, J, K) * usrc_c + c(qr, I, J, Kmm) * usrc_m) * (c(qr, I, J, K) + c(qr, I, J, Kmm))) * self.udx2c[kr] * 0.25
        h23 = ((c(qz, I, Jp, K) + c(qz, I, Jp, Kmm)) * (c(qr, I, Jp, K) + c(qr, I, J, K))
               - (c(qz, I, J, K) + c(qz, I, J, Kmm)) * (c(qr, I, J, K) + c(qr, I, Jm, K))) * udxz
        d11qre = -((c(qt, Ip, J, K) + c(qt, Ip, J, Kmm)) - (c(qt, I, J, K) + c(qt, I, J, Kmm))) * self.udx1vis2[kr]
        d11qr = (c(qr, Ip, J, K) - 2.0 * c(qr, I, J, K) + c(qr, Im, J, K)) * udxtq
        d22qr = (c(qr, I, Jp, K) - 2.0 * c(qr, I, J, K) + c(qr, I, Jm, K)) * udxzq
        coriol = (c(qt, I, J, K) + c(qt, Ip, J, K) + c(qt, I, J, Kmm) + c(qt, Ip, J, Kmm)) * 0.25 * self.rc[kr] * b["romeg"]
        self.hr = np.zeros((nthm, nzm, self.nr))
        self.hr[..., 1:nrm] = -(h21 + h22 + h23) + h11n + d11qr + d22qr + d11qre + coriol
        # QZ
        K, Kp = kc - 1, kc
        Kmm = self.kmv[kc] - 1
        Kpp = self.kpv[kc] - 1
        udxt = self.dxt * 0.25 * usrm
        udxtq = self.dxtq / (b["ren"] * rm ** 2)
        h31 = ((c(qt, Ip, J, K) + c(qt, Ip, Jm, K)) * (c(qz, Ip, J, K) + c(qz, I, J, K))
               - (c(qt, I, J, K) + c(qt, I, Jm, K)) * (c(qz, I, J, K) + c(qz, Im, J, K))) * udxt
        h32 = ((c(qr, I, J, Kp) + c(qr, I, Jm, Kp)) * (c(qz, I, J, Kpp) + c(qz, I, J, K))
               - (c(qr, I, J, K) + c(qr, I, Jm, K)) * (c(qz, I, J, K) + c(qz, I, J, Kmm))) * self.udx2rm[kc] * 0.25
        h33 = ((c(qz, I, Jp, K) + c(qz, I, J, K)) ** 2 - (c(qz, I, J, K) + c(qz, I, Jm, K)) ** 2) * udxz
        dqz1 = (c(qz, Im, J, K) - 2.0 * c(qz, I, J, K) + c(qz, Ip, J, K)) * udxtq
        dqz2 = (c(qz, I, Jm, K) - 2.0 * c(qz, I, J, K) + c(qz, I, Jp, K)) * udxzq
        self.qcap = -(h31 + h32 + h33) + dqz1 + dqz2

    def _solve_cols(self, dl, d, du, rhs_cols):
        """Factor once and solve all columns with one dgttrs call."""
        dl2, d2, du2_, dd2, ipiv, info = lapack.dgttrf(dl.copy(), d.copy(), du.copy())
        assert info == 0
        x, info = lapack.dgttrs(dl2, d2, du2_, dd2, ipiv, np.asfortranarray(rhs_cols))
        assert info == 0
        return x

    def implicit_and_update(self):
        b = self.b
        nrm, nr, nthm, nzm = self.nrm, self.nr, self.nthm, self.nzm
        al, ga, ro, dt, beta = self.al, self.ga, self.ro, self.dt, self.beta
        alre = al / b["ren"]
        I, Im = slice(1, nthm + 1), slice(0, nthm)
        J, Jm = slice(1, nzm + 1), slice(0, nzm)
        betadx = beta * al
        # ---- QT: ImplicitAndUpdateQT.F90:40-117 + SolveImpEqnUpdate_QT.F90:34-80
        qt, pr = self.qt, self.pr
        kc = np.arange(1, nrm + 1)
        ap, ac, am = self.ap1j[kc].copy(), self.ac1j[kc].copy(), self.am1j[kc].copy()
        d33 = np.empty((nthm, nzm, nrm))
        d33[..., 1:nrm - 1] = (qt[I, J, 2:nrm] * ap[1:nrm - 1] + qt[I, J, 1:nrm - 1] * ac[1:nrm - 1]
                               + qt[I, J, 0:nrm - 2] * am[1:nrm - 1])
        d33[..., 0] = qt[I, J, 1] * ap[0] + qt[I, J, 0] * ac[0] + (b["virotint"] + self.vinner_t) * am[0]
        d33[..., nrm - 1] = b["virotext"] * ap[nrm - 1] + qt[I, J, nrm - 1] * ac[nrm - 1] + qt[I, J, nrm - 2] * am[nrm - 1]
        dpx = (pr[I, J, :nrm] - pr[Im, J, :nrm]) * self.dxt * al * self.usrm[kc]
        rhs = (ga * self.dq + ro * self.ru1[..., :nrm] + alre * d33 - dpx) * dt
        self.ru1[..., :nrm] = self.dq
        self.rhs_t = rhs
        ackl_b = 1.0 / (1.0 - ac * betadx)
        amk = -am * betadx * ackl_b
        apk = -ap * betadx * ackl_b
        f = rhs * ackl_b
        f[..., 0] = (rhs[..., 0] + 0.5 * al * dt * self.dvinner_t * self.am1j[1] / b["ren"]) * ackl_b[0]
        x = self._solve_cols(amk[1:], np.ones(nrm), apk[:-1], f.reshape(-1, nrm).T)
        qt[I, J, :nrm] += x.T.reshape(nthm, nzm, nrm)
        # ---- QR: ImplicitAndUpdateQR.F90:39-71 + SolveImpEqnUpdate_QR.F90:25-67
        qr = self.qr
        kr = np.arange(2, nrm + 1)
        d33 = qr[I, J, 2:nr] * self.ap2je[kr] + qr[I, J, 1:nrm] * self.ac2je[kr] + qr[I, J, 0:nrm - 1] * self.am2je[kr]
        dpx = (pr[I, J, 1:nrm] - pr[I, J, 0:nrm - 1]) * (self.rc[kr] * al * self.udx2c[kr])
        rhs = (ga * self.hr[..., 1:nrm] + ro * self.ru2[..., 1:nrm] + alre * d33 - dpx) * dt
        self.ru2[..., 1:nrm] = self.hr[..., 1:nrm]
        self.rhs_r = rhs
        ackl_b = 1.0 / (1.0 - self.ac2j[kr] * betadx)
        dl = np.zeros(nr - 1); d = np.ones(nr); du = np.zeros(nr - 1)
        dl[0:nrm - 1] = -self.am2j[kr] * betadx * ackl_b     # amkl(2..nrm) -> dl(1..nrm-1)
        du[1:nrm] = -self.ap2j[kr] * betadx * ackl_b         # apkl(2..nrm) -> du(2..nrm)
        f = np.zeros((nthm * nzm, nr))
        f[:, 1:nrm] = (rhs * ackl_b).reshape(-1, nrm - 1)
        x = self._solve_cols(dl, d, du, f.T)
        qr[I, J, 1:nrm] += x.T.reshape(nthm, nzm, nr)[..., 1:nrm]
        qr[..., 0] = 0.0
        qr[..., nr - 1] = 0.0
        # ---- QZ: ImplicitAndUpdateQZ.F90:36-117 + SolveImpEqnUpdate_QZ.F90:32-70
        qz = self.qz
        ap, ac, am = self.ap3j[kc].copy(), self.ac3j[kc].copy(), self.am3j[kc].copy()
        d33 = np.empty((nthm, nzm, nrm))
        d33[..., 1:nrm - 1] = (qz[I, J, 2:nrm] * ap[1:nrm - 1] + qz[I, J, 1:nrm - 1] * ac[1:nrm - 1]
                               + qz[I, J, 0:nrm - 2] * am[1:nrm - 1])
        d33[..., 0] = qz[I, J, 1] * ap[0] + qz[I, J, 0] * ac[0] + qz[I, J, 0] * am[0]
        # kc = nrm: kp = kpv(nrm) = nrm, app = ap3j(nrm) = 0
        d33[..., nrm - 1] = qz[I, J, nrm - 1] * ap[nrm - 1] + qz[I, J, nrm - 1] * ac[nrm - 1] + qz[I, J, nrm - 2] * am[nrm - 1]
        dpx = (pr[I, J, :nrm] - pr[I, Jm, :nrm]) * (self.dxz * al)
        rhs = (ga * self.qcap + ro * self.ru3[..., :nrm] + alre * d33 - dpx) * dt
        # outer-wall row recomputed with ru3(nrm) already replaced by qcap(nrm)
        rhs[..., nrm - 1] = ((ga * self.qcap[..., nrm - 1] + ro * self.qcap[..., nrm - 1])
                             + alre * d33[..., nrm - 1] - dpx[..., nrm - 1]) * dt
        self.ru3[..., :nrm] = self.qcap
        self.rhs_z = rhs
        ackl_b = 1.0 / (1.0 - ac * betadx)
        amk = -am * betadx * ackl_b
        apk = -ap * betadx * ackl_b
        x = self._solve_cols(amk[1:], np.ones(nrm), apk[:-1], (rhs * ackl_b).reshape(-1, nrm).T)
        qz[I, J, :nrm] += x.T.reshape(nthm, nzm, nrm)
        for a in (qt, qr, qz):
            self.halo(a)

    # CalcLocalDivergence.F90:19-40
    def local_divergence(self):
        nrm, nthm, nzm = self.nrm, self.nthm, self.nzm
        I, Ip, J, Jp = slice(1, nthm + 1), slice(2, nthm + 2), slice(1, nzm + 1), slice(2, nzm + 2)
        kc = np.arange(1, nrm + 1)
        qt, qr, qz = self.qt, self.qr, self.qz
        d = (((qt[Ip, J, :nrm] - qt[I, J, :nrm]) * self.dxt + (qr[I, J, 1:nrm + 1] - qr[I, J, :nrm]) * self.udx2m[kc])
             * self.usrm[kc] + (qz[I, Jp, :nrm] - qz[I, J, :nrm]) * self.dxz)
        return d

    # SolvePressureCorrection.F90:100-163
    def solve_pressure(self, div):
        nrm, nthm, nzm = self.nrm, self.nthm, self.nzm
        rhs = div / (self.al * self.dt)                      # [i, j, k]
        s = np.fft.rfft(rhs, axis=1)                         # along z
        s = np.fft.fft(s, axis=0) / (nthm * nzm)             # along theta
        kc = np.arange(1, nrm + 1)
        dl0, du0 = self.amph[2:nrm + 1].astype(complex), self.apph[1:nrm].astype(complex)
        out = np.empty_like(s)
        for i in range(nthm):
            for j in range(nzm // 2 + 1):
                d = (self.acph[kc] - self.ak3[j] - self.ak1[i] * self.usrm[kc] ** 2).astype(complex)
                if self.pin and i == 0 and j == 0:
                    n1 = nrm - 1
                    dl, d_, du, du2, ipiv, info = lapack.zgttrf(dl0[:n1 - 1].copy(), d[:n1].copy(), du0[:n1 - 1].copy())
                    x, info = lapack.zgttrs(dl, d_, du, du2, ipiv, s[i, j, :n1].copy())
                    out[i, j, :n1] = x
                    out[i, j, n1] = 0.0
                    continue
                dl, d_, du, du2, ipiv, info = lapack.zgttrf(dl0.copy(), d, du0.copy())
                x, info = lapack.zgttrs(dl, d_, du, du2, ipiv, s[i, j, :].copy())
                out[i, j, :] = x
        p = np.fft.ifft(out, axis=0) * nthm
        phi = np.fft.irfft(p, n=nzm, axis=1) * nzm
        return phi

    # CorrectVelocity.F90:28-47 and CorrectPressure.F90:31-49
    def correct(self, phi):
        nrm, nthm, nzm, nr = self.nrm, self.nthm, self.nzm, self.nr
        d = self.dph
        d[1:nthm + 1, 1:nzm + 1, :nrm] = phi
        self.halo(d)
        I, Im, Ip = slice(1, nthm + 1), slice(0, nthm), slice(2, nthm + 2)
        J, Jm, Jp = slice(1, nzm + 1), slice(0, nzm), slice(2, nzm + 2)
        kc = np.arange(1, nrm + 1)
        km = self.kmv[kc] - 1
        kp = self.kpv[kc] - 1
        K = kc - 1
        al, dt = self.al, self.dt
        loc = d[I, J, :nrm]
        self.qt[I, J, :nrm] -= (loc - d[Im, J, :nrm]) * dt * al * self.dxt * self.usrm[kc]
        self.qr[I, J, :nrm] -= (loc - d[I, J][..., km]) * dt * al * self.rudx2c[kc]
        self.qz[I, J, :nrm] -= (loc - d[I, Jm, :nrm]) * al * dt * self.dxz
        self.qr[..., 0] = 0.0
        self.qr[..., nr - 1] = 0.0
        apph, acph = self.apph[kc], self.acph[kc]
        self.pr[I, J, :nrm] += loc - self.beta * (
            (d[Ip, J, :nrm] - 2.0 * loc + d[Im, J, :nrm]) * self.udx1qm[kc]
            + (d[I, Jp, :nrm] - 2.0 * loc + d[I, Jm, :nrm]) * self.dxzq
            + (d[I, J][..., kp] * apph + loc * acph + d[I, J][..., km] * apph))
        for a in (self.qt, self.qr, self.qz, self.pr):
            self.halo(a)

    def time_marcher(self, dt, time):
        self._begin_step(dt, time)
        for ns in range(int(self.b["nsst"])):
            self.al, self.ga, self.ro = self.alm[ns], self.gam[ns], self.rom[ns]
            self.explicit_terms()
            self.implicit_and_update()
            phi = self.solve_pressure(self.local_divergence())
            self.correct(phi)

    def calc_max_cfl(self):
        nrm, nthm, nzm = self.nrm, self.nthm, self.nzm
        I, Ip, J, Jp = slice(1, nthm + 1), slice(2, nthm + 2), slice(1, nzm + 1), slice(2, nzm + 2)
        kc = np.arange(1, nrm + 1)
        q = (np.abs((self.qt[Ip, J, :nrm] + self.qt[I, J, :nrm]) * 0.5 * self.dxt * self.usrm[kc])
             + np.abs((self.qr[I, J, 1:nrm + 1] + self.qr[I, J, :nrm]) * 0.5 * self.udx2rm[kc])
             + np.abs((self.qz[I, Jp, :nrm] + self.qz[I, J, :nrm]) * 0.5 * self.dxz))
        return max(1e-8, float(q.max()))

    def check_divergence(self):
        return float(np.abs(self.local_divergence()).max())

    def calc_torque(self):
        b, nr, nrm = self.b, self.nr, self.nrm
        rc, usrm, usrc = self.rc, self.usrm, self.usrc
        reninv = 1.0 / b["ren"]
        rint, rext = b["rint"], b["rext"]
        jlam = 2.0 * rint * rint * rext * rext * (b["virotint"] / rint - b["virotext"] / rext) / (rext * rext - rint * rint) * reninv
        q = self.qt[1:-1, 1:-1, :]
        low = ((q[..., 1] * usrm[2] + q[..., 0] * usrm[1]) * 0.5 - b["virotint"] * usrc[1]) * (-1.0 / (rc[2] - rc[1]))
        up = (b["virotext"] * usrc[nr] - (q[..., nrm - 2] * usrm[nrm - 1] + q[..., nrm - 1] * usrm[nrm]) * 0.5) * (-1.0 / (rc[nr] - rc[nrm]))
        inner = low.sum() * rc[2] ** 3 * reninv / jlam / (self.nthm * self.nzm)
        outer = up.sum() * rc[nrm] ** 3 * reninv / jlam / (self.nthm * self.nzm)
        return float(inner), float(outer)
