"""ctypes front end of the C++ oracle (oracle/tc_ref.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the checker or as the timed CPU
baseline; the product path never imports it.

``build()`` compiles the oracle with g++ into oracle/_build/ (OpenMP, no FMA
contraction so the arithmetic follows the reference statement order).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libtcref.so")

QT, QR, QZ, PR, DPH, RHS, RU1, RU2, RU3, DQ, QCAP = range(11)
GRID_NAMES = ["rc", "rm", "g2rc", "g2rm", "usrc", "usrm", "udx1vis1", "udx1vis2", "udx1qm",
              "udx2c", "udx2m", "rudx2c", "udx2rm", "ap1j", "am1j", "ac1j", "ap2j", "am2j", "ac2j",
              "ap2je", "am2je", "ac2je", "ap3j", "am3j", "ac3j", "apph", "amph", "acph", "pvol", "udx2mm", "udx2cc",
              "ak1", "ak3"]
# statistics of StatRoutines.F90 / CalcDissipation.F90, in the order of the
# tcref_stat enum and of the file names WriteStats uses
STAT_NAMES = ["vt_mean", "vr_mean", "vz_mean", "wt_mean", "wr_mean", "wz_mean", "vt_rms", "vr_rms", "vz_rms",
              "wt_rms", "wr_rms", "wz_rms", "vtvr_mean", "vtvz_mean", "vrvz_mean", "pr_mean", "pr_rms", "disste"]
MODE00_LAPACK, MODE00_PIN = 0, 1


class Bou(ctypes.Structure):
    """bou.in values in file order (ReadInputFile.F90:17-39)."""
    _fields_ = [
        ("nthm", ctypes.c_int), ("nzm", ctypes.c_int), ("nrm", ctypes.c_int), ("nsst", ctypes.c_int),
        ("idtv", ctypes.c_int), ("nread", ctypes.c_int),
        ("ntst", ctypes.c_int), ("tout", ctypes.c_double), ("tmax", ctypes.c_double),
        ("ireset", ctypes.c_int), ("walltimemax", ctypes.c_double),
        ("alx3", ctypes.c_double), ("rint", ctypes.c_double), ("rext", ctypes.c_double),
        ("istr", ctypes.c_int), ("str", ctypes.c_double), ("lamb", ctypes.c_double),
        ("virotint", ctypes.c_double), ("virotext", ctypes.c_double), ("sizepert", ctypes.c_double),
        ("omegapert", ctypes.c_double),
        ("ren", ctypes.c_double), ("romeg", ctypes.c_double), ("resid", ctypes.c_double),
        ("limitCFL", ctypes.c_double),
        ("tsta", ctypes.c_double), ("starea", ctypes.c_int),
        ("dtmin", ctypes.c_double), ("dtmax", ctypes.c_double), ("limitVel", ctypes.c_double),
        ("cfllim", ctypes.c_double),
        ("nslabr", ctypes.c_int), ("dpthcut", ctypes.c_int), ("dpstave", ctypes.c_int),
        ("tframe2d", ctypes.c_double),
        ("dpfullf", ctypes.c_int), ("tframe3d", ctypes.c_double),
        ("minstrt", ctypes.c_int), ("minstrz", ctypes.c_int), ("multmin", ctypes.c_int),
    ]

    @classmethod
    def from_dict(cls, d: dict) -> "Bou":
        b = cls()
        for name, typ in cls._fields_:
            if name in d:
                setattr(b, name, int(d[name]) if typ is ctypes.c_int else float(d[name]))
        return b

    def to_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "tc_ref.cpp")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["g++", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17",
           "-o", LIB, src]
    subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        L.tcref_create.restype = vp
        L.tcref_create.argtypes = [ctypes.POINTER(Bou), ctypes.c_int]
        L.tcref_destroy.argtypes = [vp]
        L.tcref_set_threads.argtypes = [ctypes.c_int]
        L.tcref_get_threads.restype = ctypes.c_int
        for n in ("tcref_set_array", "tcref_get_array"):
            getattr(L, n).argtypes = [vp, ctypes.c_int, dp]
        L.tcref_get_grid.argtypes = [vp, ctypes.c_int, dp]
        L.tcref_get_grid.restype = ctypes.c_int
        L.tcref_get_scalars.argtypes = [vp, dp]
        L.tcref_get_dvinner.argtypes = [vp, dp]
        L.tcref_get_slip.argtypes = [vp, ip, ip]
        L.tcref_begin_step.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        L.tcref_set_substep.argtypes = [vp, ctypes.c_int]
        L.tcref_update_halo.argtypes = [vp, ctypes.c_int]
        for n in ("explicit_terms_qt", "explicit_terms_qr", "explicit_terms_qz", "implicit_rhs_qt",
                  "implicit_rhs_qr", "implicit_rhs_qz", "solve_imp_eqn_update_qt",
                  "solve_imp_eqn_update_qr", "solve_imp_eqn_update_qz", "calc_local_divergence",
                  "solve_pressure_correction", "correct_velocity", "correct_pressure"):
            getattr(L, "tcref_" + n).argtypes = [vp]
        L.tcref_time_marcher.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        L.tcref_calc_max_cfl.argtypes = [vp]
        L.tcref_calc_max_cfl.restype = ctypes.c_double
        L.tcref_check_divergence.argtypes = [vp]
        L.tcref_check_divergence.restype = ctypes.c_double
        L.tcref_calc_stats.argtypes = [vp]
        L.tcref_calc_dissipation.argtypes = [vp]
        L.tcref_calc_dissipation.restype = ctypes.c_double
        L.tcref_get_stat.argtypes = [vp, ctypes.c_int, dp]
        L.tcref_stat_samples.argtypes = [vp]
        L.tcref_stat_samples.restype = ctypes.c_int
        L.tcref_get_vorticity.argtypes = [vp, ctypes.c_int, dp]
        L.tcref_calc_torque.argtypes = [vp, dp, dp]
        L.tcref_calc_velocity_stats.argtypes = [vp, dp, dp]
        L.tcref_run.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp, dp]
        L.tcref_run.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class CppOracle:
    """One oracle instance; arrays use the reference layout (see tc_ref.h)."""

    def __init__(self, bou: dict, mode00: int = MODE00_PIN):
        self.L = lib()
        self.bou = Bou.from_dict(bou)
        self.h = self.L.tcref_create(ctypes.byref(self.bou), int(mode00))
        if not self.h:
            raise ValueError("oracle rejected the configuration")
        self.nthm, self.nzm, self.nrm = self.bou.nthm, self.bou.nzm, self.bou.nrm
        self.nr = self.nrm + 1
        self.halo_shape = (self.nthm + 2, self.nzm + 2, self.nr)
        self.plain_shape = (self.nthm, self.nzm, self.nr)

    def __del__(self):
        try:
            if self.h:
                self.L.tcref_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def get(self, which: int) -> np.ndarray:
        shp = self.halo_shape if which <= DPH else self.plain_shape
        a = np.empty(shp)
        self.L.tcref_get_array(self.h, which, _dp(a))
        return a

    def set(self, which: int, a: np.ndarray):
        shp = self.halo_shape if which <= DPH else self.plain_shape
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(shp)
        self.L.tcref_set_array(self.h, which, _dp(a))

    def set_state(self, qt, qr, qz, pr):
        for w, a in ((QT, qt), (QR, qr), (QZ, qz), (PR, pr)):
            self.set(w, a)
            self.L.tcref_update_halo(self.h, w)

    def state(self):
        return tuple(self.get(w) for w in (QT, QR, QZ, PR))

    def grid(self, name: str) -> np.ndarray:
        out = np.zeros(max(self.nr, self.nthm, self.nzm) + 1)
        n = self.L.tcref_get_grid(self.h, GRID_NAMES.index(name), _dp(out))
        return out[:n].copy()

    def scalars(self) -> dict:
        o = np.zeros(8)
        self.L.tcref_get_scalars(self.h, _dp(o))
        d = np.zeros(1)
        self.L.tcref_get_dvinner(self.h, _dp(d))
        return dict(zip(["dxt", "dxz", "dxr", "beta", "al", "ga", "ro", "vinner_t"], o.tolist()),
                    dvinner_t=float(d[0]))

    def slip(self):
        ic = np.zeros(self.nthm * self.nzm, dtype=np.int32)
        oc = np.zeros(self.nthm * self.nzm, dtype=np.int32)
        self.L.tcref_get_slip(self.h, ic.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                              oc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        return ic.reshape(self.nthm, self.nzm), oc.reshape(self.nthm, self.nzm)

    def call(self, name: str, *args):
        return getattr(self.L, "tcref_" + name)(self.h, *args)

    def time_marcher(self, dt: float, time: float):
        self.L.tcref_time_marcher(self.h, dt, time)

    def calc_max_cfl(self) -> float:
        return self.L.tcref_calc_max_cfl(self.h)

    def check_divergence(self) -> float:
        return self.L.tcref_check_divergence(self.h)

    def calc_torque(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self.L.tcref_calc_torque(self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def calc_stats(self):
        """CalcStats: accumulate the theta averages."""
        self.L.tcref_calc_stats(self.h)

    def calc_dissipation(self) -> float:
        """CalcDissipation: accumulate disste, return nute."""
        return self.L.tcref_calc_dissipation(self.h)

    def stat(self, which: int) -> np.ndarray:
        """Statistic `which` as an (nzm, nrm) array (Fortran (nrm, nzm))."""
        out = np.zeros((self.nzm, self.nrm))
        self.L.tcref_get_stat(self.h, which, _dp(out))
        return out

    def stat_samples(self) -> int:
        return self.L.tcref_stat_samples(self.h)

    def vorticity(self, comp: int) -> np.ndarray:
        """CalcVorticity component (0 theta, 1 r, 2 z) as (nthm, nzm, nrm)."""
        out = np.zeros((self.nthm, self.nzm, self.nrm))
        self.L.tcref_get_vorticity(self.h, comp, _dp(out))
        return out

    def velocity_stats(self):
        v, r = np.zeros(3), np.zeros(3)
        self.L.tcref_calc_velocity_stats(self.h, _dp(v), _dp(r))
        return v, r

    def run(self, ntime0: int, nsteps: int, time: float, dt: float = 0.0):
        t, d = ctypes.c_double(time), ctypes.c_double(dt)
        code = self.L.tcref_run(self.h, ntime0, nsteps, ctypes.byref(t), ctypes.byref(d))
        return code, t.value, d.value


def set_threads(n: int):
    lib().tcref_set_threads(int(n))


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(LIB)
