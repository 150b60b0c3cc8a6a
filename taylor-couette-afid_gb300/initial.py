"""Seeded Couette-plus-noise initial fields in the reference layout.

The reference has no random initial condition (CreateInitialConditions.F90:26-43
builds deterministic sinusoids with qt = 0, restated here by
create_initial_conditions); it reads other starts through the NREAD=1
continuation path (ReadFlowField.F90:135-140) with the pressure left at zero.
couette_noise builds such a start:

* qt = A*rm_k + B/rm_k + amp*U, with A, B the laminar circular-Couette
  coefficients the reference computes at CreateInitialConditions.F90:21-23;
* qr = rc_k * amp*U with qr(1) = qr(nr) = 0 (wall values);
* qz = amp*U;  pr = 0.

U is uniform in [-1, 1) from a counter-based SplitMix64 hash of
(seed, field, i, j, k), so the same field comes out in any layout, on any host.
Arrays have the reference shape (nthm+2, nzm+2, nr) in C order, i.e. Fortran
q(1:nr, 0:nzm+1, 0:nthm+1), with the periodic halo filled.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        z = x
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, field: int, nthm: int, nzm: int, nr: int) -> np.ndarray:
    """U[-1,1) on the interior index box, shape (nthm, nzm, nr), [i-1, j-1, k-1]."""
    i = np.arange(1, nthm + 1, dtype=np.uint64)[:, None, None]
    j = np.arange(1, nzm + 1, dtype=np.uint64)[None, :, None]
    k = np.arange(1, nr + 1, dtype=np.uint64)[None, None, :]
    with np.errstate(over="ignore"):
        ctr = (np.uint64(field) << np.uint64(60)) | (i << np.uint64(40)) | (j << np.uint64(20)) | k
        key = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) * np.uint64(0xD1B54A32D192ED03)
        x = _splitmix64(ctr ^ key)
    u = (x >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return 2.0 * u - 1.0


def radial_grid(bou: dict) -> tuple[np.ndarray, np.ndarray]:
    """rc (length nr) and rm (length nrm) as CreateGrid.F90:85-139 builds them."""
    import math
    nrm = int(bou["nrm"])
    nr = nrm + 1
    rint, rext, istr, st = bou["rint"], bou["rext"], int(bou["istr"]), bou["str"]
    k = np.arange(1, nr + 1, dtype=np.float64)
    if istr == 0:
        rc = (rext - rint) * ((k - 1) / nrm) + rint
    elif istr == 4:
        rc = (1 + np.tanh(st * (2 * k - nr - 1) / nrm) / math.tanh(st)) * 0.5 * (rext - rint) + rint
        rc[0] = rint
    elif istr == 6:
        pi = 2.0 * math.asin(1.0)
        nclip = int(st)
        nrmo = nr + 2 * nclip
        etazm = np.cos(pi * (np.arange(1, nrmo + 1) - 0.5) / nrmo)
        etaz = etazm[nclip:nclip + nr]
        etaz = etaz / (0.5 * (etaz[0] - etaz[-1]))
        rc = (rext - rint) * (1.0 - etaz) * 0.5 + rint
        rc[0], rc[-1] = rint, rext
    else:
        raise ValueError(f"ISTR={istr} is not defined by the reference grid generator")
    rm = 0.5 * (rc[:-1] + rc[1:])
    return rc, rm


def fill_halo(a: np.ndarray) -> None:
    """Periodic ghost cells in z then theta (halo_common.f90:64-71,104-108)."""
    a[:, -1, :] = a[:, 1, :]
    a[:, 0, :] = a[:, -2, :]
    a[-1, :, :] = a[1, :, :]
    a[0, :, :] = a[-2, :, :]


def create_initial_conditions(bou: dict):
    """The reference's own start for NREAD = 0 (CreateInitialConditions.F90:18-43
    with the halo update of main.F90:120-123), (qt, qr, qz, pr) with halos:

    * qt = 0 (the laminar profile is computed there but not used);
    * qr = eps*(sin 2πy + sin 4πy + sin 8πy + sin 6πy), y = zm/ALX3D, at the
      radial faces k = 1..nrm, the inner wall's included; the outer wall
      face k = nr stays 0;
    * qz = Σ over m = 2, 4, 6, 8 of sin(2πx)(1 - |sin mπy|) sin(mπy) eps,
      x = (rm - rint)/(rext - rint), for k = 1..nrm;
    * pr = 0; eps = 0.1.

    The arithmetic follows the reference's order of operations."""
    import math
    nthm, nzm, nrm = int(bou["nthm"]), int(bou["nzm"]), int(bou["nrm"])
    nr = nrm + 1
    alx3, rint, rext = float(bou["alx3"]), float(bou["rint"]), float(bou["rext"])
    pi = 2.0 * math.asin(1.0)
    dxz = float(nzm) / alx3
    zm = (np.arange(nzm, dtype=np.float64) + 0.5) / dxz
    _, rm = radial_grid(bou)
    eps = 0.1
    y = (zm / alx3)[:, None]
    x = ((rm - rint) / (rext - rint))[None, :]
    s2, s4, s6, s8 = (np.sin(y * m * pi) for m in (2, 4, 6, 8))
    sx = np.sin(x * 2 * pi)
    qr_jk = np.broadcast_to(eps * (s2 + s4 + s8 + s6), (nzm, nrm))
    qz_jk = (sx * (1 - np.abs(s2)) * s2 * eps + sx * (1 - np.abs(s4)) * s4 * eps
             + sx * (1 - np.abs(s6)) * s6 * eps + sx * (1 - np.abs(s8)) * s8 * eps)
    shp = (nthm + 2, nzm + 2, nr)
    qt, qr, qz, pr = (np.zeros(shp) for _ in range(4))
    qr[1:-1, 1:-1, :nrm] = qr_jk
    qz[1:-1, 1:-1, :nrm] = qz_jk
    for a in (qr, qz):
        fill_halo(a)
    return qt, qr, qz, pr


def couette_noise(bou: dict, seed: int = 1234, amp: float = 0.01):
    """(qt, qr, qz, pr) with halos, shape (nthm+2, nzm+2, nr) each."""
    nthm, nzm, nrm = int(bou["nthm"]), int(bou["nzm"]), int(bou["nrm"])
    nr = nrm + 1
    rc, rm = radial_grid(bou)
    eta = bou["rint"] / bou["rext"]
    A = (bou["virotext"] - eta * eta * bou["virotint"]) / (1 - eta * eta)
    B = (bou["virotint"] - bou["virotext"]) * bou["rint"] * bou["rint"] / (1 - eta * eta)
    shp = (nthm + 2, nzm + 2, nr)
    qt, qr, qz, pr = (np.zeros(shp) for _ in range(4))
    ut = uniform(seed, 1, nthm, nzm, nr)
    ur = uniform(seed, 2, nthm, nzm, nr)
    uz = uniform(seed, 3, nthm, nzm, nr)
    qt[1:-1, 1:-1, :nrm] = A * rm + B / rm + amp * ut[..., :nrm]
    qr[1:-1, 1:-1, :] = rc * (amp * ur)
    qr[..., 0] = 0.0
    qr[..., nr - 1] = 0.0
    qz[1:-1, 1:-1, :nrm] = amp * uz[..., :nrm]
    for a in (qt, qr, qz, pr):
        fill_halo(a)
    return qt, qr, qz, pr
