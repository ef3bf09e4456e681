"""Grid and initial-field setup on the host (product side).

``grd7`` restates initial.f:147-301 for the uniform grid (stretch factors 0,
initial.f:173,209) and ``grd6_setup`` restates initial.f:10-142, both in
normalized units.  Arrays are 0-based copies of the reference's 1-based
arrays (``qx[0]`` is ``qx(1)``).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Coords:
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    delz: float
    qx: np.ndarray
    qy: np.ndarray
    qz: np.ndarray
    dx_grid: np.ndarray
    dy_grid: np.ndarray
    dz_grid: np.ndarray
    dx_cell: np.ndarray
    dy_cell: np.ndarray
    dz_cell: np.ndarray
    xrat: np.ndarray
    yrat: np.ndarray
    zrat: np.ndarray

    ARRAYS = ("qx", "qy", "qz", "dx_grid", "dy_grid", "dz_grid", "dx_cell", "dy_cell", "dz_cell", "xrat", "yrat", "zrat")


def _axis(n: int, d: float):
    # q(1) = d, q(i) = q(i-1) + d (initial.f:193-196); cumulative like the
    # reference so the node values round the same way.
    q = np.empty(n)
    q[0] = d
    for i in range(1, n):
        q[i] = q[i - 1] + d
    dgrid = np.empty(n)
    dgrid[: n - 1] = q[1:] - q[:-1]  # initial.f:198-201
    dgrid[n - 1] = dgrid[n - 2]
    dcell = np.empty(n)
    rat = np.empty(n)
    dcell[0], dcell[n - 1] = dgrid[0], dgrid[n - 1]  # initial.f:246-257
    rat[0] = rat[n - 1] = 0.5
    for i in range(1, n - 1):
        plus = (q[i + 1] + q[i]) / 2.0
        minus = (q[i] + q[i - 1]) / 2.0
        dcell[i] = plus - minus
        rat[i] = (q[i] - minus) / (plus - minus)
    return q, dgrid, dcell, rat


def grd7(nx: int, ny: int, nz: int, dx: float = 1.0, dy: float = 1.0, delz: float = 1.0) -> Coords:
    qx, dxg, dxc, xr = _axis(nx, dx)
    qz, dzg, dzc, zr = _axis(nz, delz)
    # y: q(j) = j*dy (initial.f:159-162), dy_grid = dy
    qy = np.arange(1, ny + 1, dtype=np.float64) * dy
    dyg = np.full(ny, dy)
    dyc = np.empty(ny)
    yr = np.empty(ny)
    dyc[0], dyc[ny - 1] = dyg[0], dyg[ny - 1]
    yr[0] = yr[ny - 1] = 0.5
    for j in range(1, ny - 1):
        plus = (qy[j + 1] + qy[j]) / 2.0
        minus = (qy[j] + qy[j - 1]) / 2.0
        dyc[j] = plus - minus
        yr[j] = (qy[j] - minus) / (plus - minus)
    return Coords(nx, ny, nz, dx, dy, delz, qx, qy, qz, dxg, dyg, dzg, dxc, dyc, dzc, xr, yr, zr)


def grid_zeros(c: Coords, ncomp: int = 3) -> np.ndarray:
    shape = (c.nx, c.ny, c.nz) + ((ncomp,) if ncomp > 1 else ())
    return np.zeros(shape, dtype=np.float64, order="F")


def grd6_setup(c: Coords, b0z: float, nu_init: float):
    """b0 = (0,0,b0z); bt = b12 = b1 = b1p2 = b0; nu = nu_init (initial.f:54-85)."""
    b0 = grid_zeros(c)
    b0[..., 2] = b0z
    fields = {"b0": b0}
    for name in ("b1", "b12", "b1p2", "bt"):
        fields[name] = b0.copy(order="F")
    nu = grid_zeros(c, 1)
    nu[...] = nu_init
    fields["nu"] = nu
    for name in ("btc", "up", "aj", "E"):
        fields[name] = grid_zeros(c)
    fields["np"] = grid_zeros(c, 1)
    return fields
