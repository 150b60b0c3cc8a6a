"""tc_gb300 -- GB300 (sm_103a) Taylor-Couette time step behind a C ABI.

Host-side mirror of the reference routine interface (rodosti/Taylor-Couette-AFiD):
the methods of :class:`TaylorCouette` carry the names of the Fortran routines
they replace (TimeMarcher, CalcMaxCFL, CheckDivergence, CalcTorque, ...) and
call ``libtcgb300.so`` through ctypes.  There is no CPU fallback: if the
library or a CUDA device is missing, construction raises.

Arrays exchanged with the host use the reference layout.  A NumPy array of
shape ``(nthm+2, nzm+2, nr)`` in C order is the Fortran array
``q(1:nr, 0:nzm+1, 0:nthm+1)`` (r fastest, periodic halo in z and theta).

The package directory is ``taylor-couette-afid_gb300``; load it with
``load()`` from ``__graft_entry__`` or ``tests/conftest.py``, which register it
as ``tc_gb300``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtcgb300.so")

# error codes of main.F90:148-259
ERRORS = {165: "CFL above CFLLIM with fixed dt", 166: "dt below DTMIN", 169: "divergence above RESID",
          266: "velocity above VMAX", 333: "time above TMAX", 555: "NTST steps done"}

GRID_ARRAYS = ["rc", "rm", "g2rc", "g2rm", "usrc", "usrm", "udx1vis1", "udx1vis2", "udx1qm", "udx2c",
               "udx2m", "rudx2c", "udx2rm", "ap1j", "am1j", "ac1j", "ap2j", "am2j", "ac2j", "ap2je",
               "am2je", "ac2je", "ap3j", "am3j", "ac3j", "apph", "amph", "acph", "pvol", "udx2mm", "udx2cc", "ak1",
               "ak3"]
STATS = ["vt_mean", "vr_mean", "vz_mean", "wt_mean", "wr_mean", "wz_mean", "vt_rms", "vr_rms", "vz_rms",
         "wt_rms", "wr_rms", "wz_rms", "vtvr_mean", "vtvz_mean", "vrvz_mean", "pr_mean", "pr_rms", "disste"]
FIELDS = ["qt", "qr", "qz", "pr", "dph", "rhs_t", "rhs_r", "rhs_z", "ru1", "ru2", "ru3", "dq", "hr", "qcap"]
_HALO_FIELDS = 5


class Bou(ctypes.Structure):
    """tc_bou: bou.in values in file order (ReadInputFile.F90:17-39)."""
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


class TCError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None

# C ABI signatures: name -> (restype, argtypes)
_vp, _dp, _ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
SIGNATURES = {
    "tc_read_bou": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Bou), ctypes.c_char_p, ctypes.c_int]),
    "tc_grid_array": (ctypes.c_int, [ctypes.POINTER(Bou), ctypes.c_int, _dp, ctypes.c_int]),
    "tc_version": (ctypes.c_char_p, []),
    "tc_create": (ctypes.c_int, [ctypes.POINTER(Bou), ctypes.POINTER(_vp)]),
    "tc_create_ex": (ctypes.c_int, [ctypes.POINTER(Bou), ctypes.c_int, ctypes.POINTER(_vp)]),
    "tc_precision": (ctypes.c_int, [_vp]),
    "tc_use_tma": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tc_destroy": (None, [_vp]),
    "tc_last_error": (ctypes.c_char_p, [_vp]),
    "tc_set_stream": (ctypes.c_int, [_vp, _vp]),
    "tc_set_tmax": (ctypes.c_int, [_vp, ctypes.c_double]),
    "tc_host_alloc": (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]),
    "tc_host_free": (ctypes.c_int, [_vp]),
    "tc_set_state": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "tc_get_state": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "tc_get_field": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "tc_set_field": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "tc_time_marcher": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double]),
    "tc_run": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp, _dp]),
    "tc_begin_step": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double]),
    "tc_set_substep": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tc_explicit_terms": (ctypes.c_int, [_vp]),
    "tc_implicit_and_update": (ctypes.c_int, [_vp]),
    "tc_explicit_and_rhs": (ctypes.c_int, [_vp]),
    "tc_solve_imp_eqn_update": (ctypes.c_int, [_vp]),
    **{f"tc_{r}_{c}": (ctypes.c_int, [_vp]) for r in ("explicit_terms", "implicit_and_update", "solve_imp_eqn_update")
       for c in ("qt", "qr", "qz")},
    "tc_calc_local_divergence": (ctypes.c_int, [_vp]),
    "tc_solve_pressure_correction": (ctypes.c_int, [_vp]),
    "tc_correct_velocity": (ctypes.c_int, [_vp]),
    "tc_correct_pressure": (ctypes.c_int, [_vp]),
    "tc_calc_max_cfl": (ctypes.c_int, [_vp, _dp]),
    "tc_check_divergence": (ctypes.c_int, [_vp, _dp]),
    "tc_check_divergence_noalloc": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                    _dp, _dp, ctypes.c_double, ctypes.c_double, _vp, _dp]),
    "tc_calc_torque": (ctypes.c_int, [_vp, _dp, _dp]),
    "tc_calc_velocity_stats": (ctypes.c_int, [_vp, _dp, _dp]),
    "tc_kernels_per_step": (ctypes.c_int, [_vp]),
    "tc_device_bytes": (ctypes.c_longlong, [_vp]),
    "tc_launch_count": (ctypes.c_longlong, [_vp]),
    "tc_kernels_per_run_step": (ctypes.c_int, [_vp]),
    "tc_profile": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tc_profile_read": (ctypes.c_int, [_vp, _dp, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]),
    "tc_profile_name": (ctypes.c_char_p, [ctypes.c_int]),
    "tc_measure_fp64_peak": (ctypes.c_int, [_vp, _dp]),
    "tc_selftest_conversions": (ctypes.c_int, [ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]),
    "tc_get_bou": (ctypes.c_int, [_vp, ctypes.POINTER(Bou)]),
    "tc_calc_stats": (ctypes.c_int, [_vp]),
    "tc_calc_dissipation": (ctypes.c_int, [_vp, _dp]),
    "tc_get_stat": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "tc_stat_samples": (ctypes.c_int, [_vp]),
    "tc_reset_stats": (ctypes.c_int, [_vp]),
    "tc_h5_write_stats": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int]),
    "tc_h5_load_continua": (ctypes.c_int, [ctypes.POINTER(Bou), ctypes.c_char_p, _dp, _dp, _dp, _dp]),
    "tc_h5_write_scalars": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), _dp,
                                           _ip]),
    "tc_h5_dump_flow_field": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double]),
    "tc_h5_dump_rcuts": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double, _dp, ctypes.c_int]),
    "tc_h5_dump_thcuts": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double]),
    "tc_h5_dump_streamwise_avg": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double]),
    "tc_h5_write_continua": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double]),
    "tc_h5_read_continua": (ctypes.c_int, [_vp, ctypes.c_char_p, _dp]),
    "tc_h5_write_grid_info": (ctypes.c_int, [ctypes.POINTER(Bou), ctypes.c_char_p]),
    "tc_h5_write_dataset": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_longlong), _dp]),
    "tc_h5_read_dataset": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, _dp, ctypes.c_longlong, _ip,
                                          ctypes.POINTER(ctypes.c_longlong)]),
    "tc_ensemble_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_vp)]),
    "tc_ensemble_destroy": (None, [_vp]),
    "tc_ensemble_last_error": (ctypes.c_char_p, [_vp]),
    "tc_ensemble_set_stream": (ctypes.c_int, [_vp, _vp]),
    "tc_ensemble_add": (ctypes.c_int, [_vp, ctypes.POINTER(Bou), ctypes.c_double, _dp, _dp, _dp, _dp, ctypes.c_int,
                                       _ip]),
    "tc_ensemble_remove": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tc_ensemble_member": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(_vp)]),
    "tc_ensemble_count": (ctypes.c_int, [_vp]),
    "tc_ensemble_tune": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "tc_ensemble_schedule": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "tc_ensemble_get_schedule": (ctypes.c_int, [_vp]),
    "tc_ensemble_persistent_blocks": (ctypes.c_int, [_vp]),
    "tc_ensemble_set_barrier_timeout": (ctypes.c_int, [_vp, ctypes.c_double]),
    "tc_ensemble_stall_next_barrier": (ctypes.c_int, [_vp]),
    "tc_ensemble_step": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tc_ensemble_sync": (ctypes.c_int, [_vp]),
    "tc_ensemble_status": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp, _dp, _ip]),
    "tc_ensemble_target": (ctypes.c_int, [_vp, ctypes.c_int]),
    "tc_ensemble_launch_count": (ctypes.c_longlong, [_vp]),
    "tc_ensemble_launches_per_step": (ctypes.c_int, [_vp]),
    "tc_ensemble_device_bytes": (ctypes.c_longlong, [_vp]),
    "tc_ensemble_cells": (ctypes.c_longlong, [_vp]),
}


def lib() -> ctypes.CDLL:
    """Load libtcgb300.so (build it first with ``tc_gb300.build.build()``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it (python {HERE}/build.py)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def read_bou(path: str) -> dict:
    """ReadInputFile.F90: parse a bou.in file into a dict of its values."""
    b = Bou()
    err = ctypes.create_string_buffer(512)
    rc = lib().tc_read_bou(path.encode(), ctypes.byref(b), err, 512)
    if rc != 0:
        raise TCError(rc, err.value.decode())
    return b.to_dict()


def grid_array(bou: dict, name: str) -> np.ndarray:
    """CreateGrid / InitPressureSolver arrays computed on the host (no GPU)."""
    b = Bou.from_dict(bou)
    n = max(int(bou["nrm"]) + 1, int(bou["nthm"]), int(bou["nzm"]))
    out = np.zeros(n)
    rc = lib().tc_grid_array(ctypes.byref(b), GRID_ARRAYS.index(name), _dptr(out), n)
    if rc < 0:
        raise TCError(-rc, lib().tc_last_error(None).decode())
    return out[:rc].copy()


def check_divergence_noalloc(qt: int, qr: int, qz: int, nthm: int, nzm: int, nrm: int, udx2m: np.ndarray,
                             usrm: np.ndarray, dxt: float, dxz: float, stream: int = 0) -> float:
    """CheckDivergence on caller-owned device arrays (addresses of FP64
    arrays in the reference layout, periodic halos current) with no handle
    and no device allocation; udx2m and usrm are host arrays of nrm
    entries.  Calls on one device must not overlap.  A NaN in the fields
    raises TCError 169 (the reference's divergence error code)."""
    if len(udx2m) < nrm or len(usrm) < nrm:
        raise ValueError(f"udx2m and usrm need nrm = {nrm} entries, got {len(udx2m)} and {len(usrm)}")
    u = np.ascontiguousarray(udx2m[:nrm], dtype=np.float64)
    m = np.ascontiguousarray(usrm[:nrm], dtype=np.float64)
    v = ctypes.c_double()
    L = lib()
    rc = L.tc_check_divergence_noalloc(qt, qr, qz, nthm, nzm, nrm, _dptr(u), _dptr(m), dxt, dxz, stream,
                                       ctypes.byref(v))
    if rc != 0:
        raise TCError(rc, L.tc_last_error(None).decode())
    return v.value


def selftest_conversions(n: int = 1 << 24) -> int:
    """Mismatches of the integer-pipe float <-> double conversions against the
    hardware conversions over n operands (0 expected)."""
    v = ctypes.c_longlong()
    rc = lib().tc_selftest_conversions(int(n), ctypes.byref(v))
    if rc != 0:
        raise TCError(rc, "tc_selftest_conversions")
    return v.value


def host_array(shape, dtype=np.float64) -> np.ndarray:
    """A zeroed host array in page-locked memory on transparent huge pages
    (tc_host_alloc), for state transfers (set_state / get_state(out=...)):
    they keep the CPU-GPU link rate however long the GPU has been busy.  The
    memory is released when the array and every view of it are gone."""
    import weakref
    dt = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dt.itemsize
    L = lib()
    p = ctypes.c_void_p()
    rc = L.tc_host_alloc(max(nbytes, 1), ctypes.byref(p))
    if rc != 0:
        raise TCError(rc, L.tc_last_error(None).decode())
    buf = (ctypes.c_char * max(nbytes, 1)).from_address(p.value)
    weakref.finalize(buf, L.tc_host_free, ctypes.c_void_p(p.value))
    return np.frombuffer(buf, dtype=dt, count=int(np.prod(shape))).reshape(shape)


def h5_write(path: str, name: str, data: np.ndarray):
    """One float64 dataset in a new HDF5 file (C order shape of `data`)."""
    a = np.ascontiguousarray(data, dtype=np.float64)
    dims = (ctypes.c_longlong * a.ndim)(*a.shape)
    rc = lib().tc_h5_write_dataset(path.encode(), name.encode(), a.ndim, dims, _dptr(a))
    if rc != 0:
        raise TCError(rc, lib().tc_last_error(None).decode())


def h5_read(path: str, name: str) -> np.ndarray:
    """Dataset `name` of an HDF5 file as a float64 array of its shape."""
    L = lib()
    rank = ctypes.c_int()
    dims = (ctypes.c_longlong * 8)()
    rc = L.tc_h5_read_dataset(path.encode(), name.encode(), None, 0, ctypes.byref(rank), dims)
    if rc != 0:
        raise TCError(rc, L.tc_last_error(None).decode())
    shape = tuple(dims[i] for i in range(rank.value))
    out = np.empty(shape)
    rc = L.tc_h5_read_dataset(path.encode(), name.encode(), _dptr(out), out.size, ctypes.byref(rank), dims)
    if rc != 0:
        raise TCError(rc, L.tc_last_error(None).decode())
    return out


def h5_write_scalars(path: str, values: dict, ints=()):
    """Scalar datasets in a new HDF5 file; names in `ints` are int32."""
    names = list(values)
    arr = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
    v = np.array([float(values[n]) for n in names])
    flags = np.array([1 if n in ints else 0 for n in names], dtype=np.int32)
    rc = lib().tc_h5_write_scalars(path.encode(), len(names), arr, _dptr(v),
                                   flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    if rc != 0:
        raise TCError(rc, lib().tc_last_error(None).decode())


def h5_load_continua(bou: dict, directory: str = "."):
    """ReadFlowField on the host: (qt, qr, qz, time) on bou's grid, reference
    layout, interpolated when the files hold another grid (interp.F90)."""
    b = Bou.from_dict(bou)
    shape = (b.nthm + 2, b.nzm + 2, b.nrm + 1)
    q = [np.zeros(shape) for _ in range(3)]
    t = ctypes.c_double()
    rc = lib().tc_h5_load_continua(ctypes.byref(b), directory.encode(), *[_dptr(a) for a in q], ctypes.byref(t))
    if rc != 0:
        raise TCError(rc, lib().tc_last_error(None).decode())
    return q[0], q[1], q[2], t.value


def h5_write_grid_info(bou: dict, directory: str = "."):
    """WriteGridInfo: cordin_info.h5 with rm, rc, tm, zm."""
    b = Bou.from_dict(bou)
    rc = lib().tc_h5_write_grid_info(ctypes.byref(b), directory.encode())
    if rc != 0:
        raise TCError(rc, lib().tc_last_error(None).decode())


PREC_FP64, PREC_MIXED, PREC_MIXED_FF = 0, 1, 2
# precision names of the Python mirror -> enum tc_precision_mode
PRECISIONS = {"fp64": PREC_FP64, "mixed": PREC_MIXED, "mixed-ff": PREC_MIXED_FF}


class TaylorCouette:
    """One simulation instance resident on the current CUDA device.

    precision: "fp64" (plain path, the drop-in), "mixed" (FP32 velocities,
    explicit terms, momentum sweeps and FFTs; FP64 pressure tridiagonals,
    pressure accumulation and reductions) or "mixed-ff" ("mixed" with the
    pressure tridiagonals in float-float arithmetic)."""

    def __init__(self, bou: dict, precision: str = "fp64", _handle=None):
        self.L = lib()
        self.bou = dict(bou)
        self._b = Bou.from_dict(bou)
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        self.precision = precision
        self._owned = _handle is None
        if _handle is None:
            h = ctypes.c_void_p()
            rc = self.L.tc_create_ex(ctypes.byref(self._b), PRECISIONS[precision], ctypes.byref(h))
            if rc != 0:
                raise TCError(rc, self.L.tc_last_error(None).decode())
        else:
            h = _handle
        self.h = h
        self.nthm, self.nzm, self.nrm = self._b.nthm, self._b.nzm, self._b.nrm
        self.nr = self.nrm + 1
        self.halo_shape = (self.nthm + 2, self.nzm + 2, self.nr)
        self.plain_shape = (self.nthm, self.nzm, self.nr)

    def close(self):
        if getattr(self, "h", None):
            if self._owned:
                self.L.tc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc: int):
        if rc != 0:
            raise TCError(rc, self.L.tc_last_error(self.h).decode())

    # ---- state -----------------------------------------------------------
    def set_stream(self, stream_ptr: int):
        self._ck(self.L.tc_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def set_tmax(self, tmax: float):
        """TMAX of the stop test 333; a restart adds its time to it
        (ReadFlowField.F90:149), which read_continua does."""
        self._ck(self.L.tc_set_tmax(self.h, float(tmax)))
        self.bou["tmax"] = float(tmax)

    def set_state(self, qt, qr, qz, pr=None):
        """ReadFlowField: load a start (reference layout, halos ignored)."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (qt, qr, qz)]
        for a in arrs:
            if a.shape != self.halo_shape:
                raise ValueError(f"expected shape {self.halo_shape}, got {a.shape}")
        p = None
        if pr is not None:
            p = np.ascontiguousarray(pr, dtype=np.float64)
            if p.shape != self.halo_shape:
                raise ValueError(f"expected shape {self.halo_shape}, got {p.shape}")
        self._ck(self.L.tc_set_state(self.h, *[_dptr(a) for a in arrs], _dptr(p) if p is not None else None))

    def get_state(self, out=None):
        """WriteFlowField's fields (reference layout with halos).  `out`: four
        C-contiguous float64 arrays of the halo shape to fill (for example in
        pinned memory), else new arrays."""
        if out is None:
            out = [np.empty(self.halo_shape) for _ in range(4)]
        else:
            out = list(out)
            for a in out:
                if a.shape != self.halo_shape or a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"expected C-contiguous float64 arrays of shape {self.halo_shape}")
        self._ck(self.L.tc_get_state(self.h, *[_dptr(a) for a in out]))
        return tuple(out)

    # ---- statistics (StatRoutines.F90, CalcDissipation.F90) -----------------
    def calc_stats(self):
        """CalcStats: accumulate one sample of the theta averages."""
        self._ck(self.L.tc_calc_stats(self.h))

    def calc_dissipation(self) -> float:
        """CalcDissipation: accumulate disste, return nute."""
        v = ctypes.c_double()
        self._ck(self.L.tc_calc_dissipation(self.h, ctypes.byref(v)))
        return v.value

    def stat(self, name: str) -> np.ndarray:
        """Statistic `name` as an (nzm, nrm) array (Fortran (nrm, nzm))."""
        out = np.empty((self.nzm, self.nrm))
        self._ck(self.L.tc_get_stat(self.h, STATS.index(name), _dptr(out)))
        return out

    @property
    def stat_samples(self) -> int:
        return self.L.tc_stat_samples(self.h)

    def reset_stats(self):
        self._ck(self.L.tc_reset_stats(self.h))

    def write_stats(self, directory: str = ".", readstats: bool = False):
        """WriteStats: one HDF5 file per statistic plus stafield_master.h5."""
        self._ck(self.L.tc_h5_write_stats(self.h, directory.encode(), 1 if readstats else 0))

    # ---- dumps (DumpFlowField, DumpRCuts, DumpThCuts, DumpStreamwiseAvg) ----
    def dump_flow_field(self, directory: str, time: float):
        self._ck(self.L.tc_h5_dump_flow_field(self.h, directory.encode(), float(time)))

    def dump_rcuts(self, directory: str, time: float, radii):
        r = np.ascontiguousarray(radii, dtype=np.float64)
        self._ck(self.L.tc_h5_dump_rcuts(self.h, directory.encode(), float(time), _dptr(r), len(r)))

    def dump_thcuts(self, directory: str, time: float):
        self._ck(self.L.tc_h5_dump_thcuts(self.h, directory.encode(), float(time)))

    def dump_streamwise_avg(self, directory: str, time: float):
        self._ck(self.L.tc_h5_dump_streamwise_avg(self.h, directory.encode(), float(time)))

    def write_continua(self, directory: str = ".", time: float = 0.0):
        """WriteFlowField: continua_q{t,r,z}.h5 and continua_master.h5."""
        self._ck(self.L.tc_h5_write_continua(self.h, directory.encode(), float(time)))

    def read_continua(self, directory: str = ".") -> float:
        """ReadFlowField: load the continuation files (interpolated when they
        hold another grid) and return their time (0 with IRESET = 1); TMAX
        grows by that time, as ReadFlowField.F90:149 does."""
        t = ctypes.c_double()
        self._ck(self.L.tc_h5_read_continua(self.h, directory.encode(), ctypes.byref(t)))
        self.bou["tmax"] = float(self.bou["tmax"]) + t.value
        return t.value

    def get_field(self, name: str) -> np.ndarray:
        w = FIELDS.index(name)
        a = np.empty(self.halo_shape if w < _HALO_FIELDS else self.plain_shape)
        self._ck(self.L.tc_get_field(self.h, w, _dptr(a)))
        return a

    def set_field(self, name: str, a: np.ndarray):
        w = FIELDS.index(name)
        shp = self.halo_shape if w < _HALO_FIELDS else self.plain_shape
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(shp)
        self._ck(self.L.tc_set_field(self.h, w, _dptr(a)))

    # ---- the step (TimeMarcher.F90, main.F90) -------------------------------
    def time_marcher(self, dt: float, time: float):
        self._ck(self.L.tc_time_marcher(self.h, float(dt), float(time)))

    def run(self, nsteps: int, ntime: int, time: float, dt: float = 0.0):
        """main.F90 loop: returns (errorcode, ntime, time, dt)."""
        n, t, d = ctypes.c_int(ntime), ctypes.c_double(time), ctypes.c_double(dt)
        rc = self.L.tc_run(self.h, int(nsteps), ctypes.byref(n), ctypes.byref(t), ctypes.byref(d))
        if rc != 0 and rc not in ERRORS:
            raise TCError(rc, self.L.tc_last_error(self.h).decode())
        return rc, n.value, t.value, d.value

    def use_tma(self, enable: bool = True):
        """Mixed path: the TMA-staged momentum march (True) or the march that
        loads through the read-only cache (False, the default)."""
        self._ck(self.L.tc_use_tma(self.h, 1 if enable else 0))

    # per-routine entry points (parity bisection)
    def begin_step(self, dt: float, time: float):
        self._ck(self.L.tc_begin_step(self.h, float(dt), float(time)))

    def set_substep(self, ns: int):
        self._ck(self.L.tc_set_substep(self.h, int(ns)))

    def explicit_terms(self):
        self._ck(self.L.tc_explicit_terms(self.h))

    def implicit_and_update(self):
        self._ck(self.L.tc_implicit_and_update(self.h))

    def explicit_and_rhs(self):
        self._ck(self.L.tc_explicit_and_rhs(self.h))

    def solve_imp_eqn_update(self):
        self._ck(self.L.tc_solve_imp_eqn_update(self.h))

    # one component each, as TimeMarcher.F90:31-37 calls them
    def explicit_terms_qt(self):
        self._ck(self.L.tc_explicit_terms_qt(self.h))

    def explicit_terms_qr(self):
        self._ck(self.L.tc_explicit_terms_qr(self.h))

    def explicit_terms_qz(self):
        self._ck(self.L.tc_explicit_terms_qz(self.h))

    def implicit_and_update_qt(self):
        self._ck(self.L.tc_implicit_and_update_qt(self.h))

    def implicit_and_update_qr(self):
        self._ck(self.L.tc_implicit_and_update_qr(self.h))

    def implicit_and_update_qz(self):
        self._ck(self.L.tc_implicit_and_update_qz(self.h))

    def solve_imp_eqn_update_qt(self):
        self._ck(self.L.tc_solve_imp_eqn_update_qt(self.h))

    def solve_imp_eqn_update_qr(self):
        self._ck(self.L.tc_solve_imp_eqn_update_qr(self.h))

    def solve_imp_eqn_update_qz(self):
        self._ck(self.L.tc_solve_imp_eqn_update_qz(self.h))

    def calc_local_divergence(self):
        self._ck(self.L.tc_calc_local_divergence(self.h))

    def solve_pressure_correction(self):
        self._ck(self.L.tc_solve_pressure_correction(self.h))

    def correct_velocity(self):
        self._ck(self.L.tc_correct_velocity(self.h))

    def correct_pressure(self):
        self._ck(self.L.tc_correct_pressure(self.h))

    # ---- reductions ----------------------------------------------------------
    def calc_max_cfl(self) -> float:
        v = ctypes.c_double()
        self._ck(self.L.tc_calc_max_cfl(self.h, ctypes.byref(v)))
        return v.value

    def check_divergence(self) -> float:
        v = ctypes.c_double()
        self._ck(self.L.tc_check_divergence(self.h, ctypes.byref(v)))
        return v.value

    def calc_torque(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._ck(self.L.tc_calc_torque(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def velocity_stats(self):
        v, r = np.zeros(3), np.zeros(3)
        self._ck(self.L.tc_calc_velocity_stats(self.h, _dptr(v), _dptr(r)))
        return v, r

    @property
    def kernels_per_step(self) -> int:
        return self.L.tc_kernels_per_step(self.h)

    @property
    def device_bytes(self) -> int:
        return self.L.tc_device_bytes(self.h)

    @property
    def launch_count(self) -> int:
        return self.L.tc_launch_count(self.h)

    @property
    def kernels_per_run_step(self) -> int:
        return self.L.tc_kernels_per_run_step(self.h)

    def profile(self, enable: bool):
        self._ck(self.L.tc_profile(self.h, 1 if enable else 0))

    def profile_read(self) -> dict:
        ms = np.zeros(16)
        n = np.zeros(16, dtype=np.int64)
        cnt = self.L.tc_profile_read(self.h, _dptr(ms), n.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), 16)
        if cnt < 0:
            raise TCError(cnt, "profile read")
        return {self.L.tc_profile_name(c).decode(): (float(ms[c]), int(n[c])) for c in range(cnt)}

    def measure_fp64_peak(self) -> float:
        v = ctypes.c_double()
        self._ck(self.L.tc_measure_fp64_peak(self.h, ctypes.byref(v)))
        return v.value


SCHEDULES = {"grouped": 0, "persistent": 1}


class Ensemble:
    """Many independent runs resident on one device, stepped together (one
    CUDA graph per step: grouped launches per phase, or one persistent
    cooperative launch per RK substep).  Members are admitted and retired
    between steps; each keeps the single-run arithmetic.

    precision: "fp64", "mixed" or "mixed-ff" for every member."""

    def __init__(self, precision: str = "mixed"):
        self.L = lib()
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        self.precision = precision
        e = ctypes.c_void_p()
        rc = self.L.tc_ensemble_create(PRECISIONS[precision], ctypes.byref(e))
        if rc != 0:
            raise TCError(rc, "tc_ensemble_create")
        self.e = e
        self.bous = {}

    def close(self):
        if getattr(self, "e", None):
            self.L.tc_ensemble_destroy(self.e)
            self.e = None
            self.bous = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc: int):
        if rc != 0:
            raise TCError(rc, (self.L.tc_ensemble_last_error(self.e) or b"").decode())

    def set_stream(self, stream_ptr: int):
        self._ck(self.L.tc_ensemble_set_stream(self.e, ctypes.c_void_p(stream_ptr)))

    def add(self, bou: dict, state, nsteps: int = 0, dt: float = 0.0) -> int:
        """Admit a run with start `state` = (qt, qr, qz[, pr]) in the reference
        layout.  dt > 0: fixed dt; dt <= 0 with IDTV = 1: the reference's
        variable dt every step; dt <= 0 with IDTV = 0: fixed dt from the
        start's CFL number (LIMITCFL / CFL, capped at DTMAX)."""
        b = Bou.from_dict(bou)
        shp = (b.nthm + 2, b.nzm + 2, b.nrm + 1)
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in state[:3]]
        for a in arrs:
            if a.shape != shp:
                raise ValueError(f"expected shape {shp}, got {a.shape}")
        pr = None
        if len(state) > 3 and state[3] is not None:
            pr = np.ascontiguousarray(state[3], dtype=np.float64)
        slot = ctypes.c_int()
        self._ck(self.L.tc_ensemble_add(self.e, ctypes.byref(b), float(dt), *[_dptr(a) for a in arrs],
                                        _dptr(pr) if pr is not None else None, int(nsteps), ctypes.byref(slot)))
        self.bous[slot.value] = dict(bou)
        return slot.value

    def remove(self, slot: int):
        self._ck(self.L.tc_ensemble_remove(self.e, slot))
        self.bous.pop(slot, None)

    def member(self, slot: int) -> TaylorCouette:
        """A non-owning view of the member (get_state, calc_torque, ...)."""
        h = ctypes.c_void_p()
        self._ck(self.L.tc_ensemble_member(self.e, slot, ctypes.byref(h)))
        return TaylorCouette(self.bous[slot], self.precision, _handle=h)

    def tune(self, threads: int = 128, rows: int = 0, schedule: str | None = None, blocks_per_sm: int = 0):
        """Tile shape (threads per tile, rows per theta-FFT item) and, if
        given, the schedule ("grouped" or "persistent", with its cap on
        blocks per SM, 0 = occupancy limit)."""
        self._ck(self.L.tc_ensemble_tune(self.e, threads, rows))
        if schedule is not None:
            self.set_schedule(schedule, blocks_per_sm)

    def set_schedule(self, schedule: str, blocks_per_sm: int = 0):
        if schedule not in SCHEDULES:
            raise ValueError(f"schedule must be one of {sorted(SCHEDULES)}")
        self._ck(self.L.tc_ensemble_schedule(self.e, SCHEDULES[schedule], int(blocks_per_sm)))

    @property
    def schedule(self) -> str:
        v = self.L.tc_ensemble_get_schedule(self.e)
        return {i: k for k, i in SCHEDULES.items()}[v]

    @property
    def persistent_blocks(self) -> int:
        return self.L.tc_ensemble_persistent_blocks(self.e)

    def set_barrier_timeout(self, seconds: float):
        """Bound on one grid-barrier wait of the persistent kernel."""
        self._ck(self.L.tc_ensemble_set_barrier_timeout(self.e, float(seconds)))

    def stall_next_barrier(self):
        """Failure-path test: the next persistent barrier cannot complete, its
        waits run out and the next sync raises TCError(3001)."""
        self._ck(self.L.tc_ensemble_stall_next_barrier(self.e))

    def step(self, nsteps: int = 1):
        self._ck(self.L.tc_ensemble_step(self.e, int(nsteps)))

    def sync(self):
        self._ck(self.L.tc_ensemble_sync(self.e))

    def status(self, slot: int):
        """(steps done, simulated time) of a member."""
        return self.status_full(slot)[:2]

    def status_full(self, slot: int):
        """(steps done, simulated time, last dt, error code) of a member."""
        n, t, d, c = ctypes.c_int(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        self._ck(self.L.tc_ensemble_status(self.e, slot, ctypes.byref(n), ctypes.byref(t), ctypes.byref(d),
                                           ctypes.byref(c)))
        return n.value, t.value, d.value, c.value

    def target(self, slot: int) -> int:
        return self.L.tc_ensemble_target(self.e, slot)

    @property
    def count(self) -> int:
        return self.L.tc_ensemble_count(self.e)

    @property
    def cells(self) -> int:
        return self.L.tc_ensemble_cells(self.e)

    @property
    def launch_count(self) -> int:
        return self.L.tc_ensemble_launch_count(self.e)

    @property
    def launches_per_step(self) -> int:
        return self.L.tc_ensemble_launches_per_step(self.e)

    @property
    def device_bytes(self) -> int:
        return self.L.tc_ensemble_device_bytes(self.e)
