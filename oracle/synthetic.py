"""Synthetic inputs for the oracle's users without the product's CUDA library.

TEST INFRASTRUCTURE ONLY: the CPU baseline and the reference leg of bench.py
make their tracks here, so that their processes never load
libmuto_gb300.so.  ``phantom`` rasterises blocks at voxel centres (later
blocks win) like the library's muto_phantom; ``generate`` runs the project's
synthetic-muon model compiled into the oracle's library (oracle/synthetic.cpp).
Both equal the library's host functions bit for bit.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import oracle as O


class GenParams(C.Structure):  # == muto_gen_params
    _fields_ = [("seed", C.c_uint64), ("theta_max", C.c_double), ("p_min", C.c_double), ("p_max", C.c_double),
                ("p0", C.c_double), ("plane_gap", C.c_double), ("n_planes", C.c_int32), ("pad", C.c_int32),
                ("hit_sigma", C.c_double)]


def lambda_from_x0(x0_mm: float, p0: float = 3.0) -> float:
    a = 0.0136 / p0  # (13.6 MeV / p0)^2 / X0
    return a * a / x0_mm


def phantom(grid, blocks, background_x0: float, p0: float = 3.0) -> np.ndarray:
    """Flat (V,) lambda image, x fastest: each voxel centre takes the last block containing it."""
    cx = grid.x_min + (np.arange(grid.nx) + 0.5) * grid.dx
    cy = grid.y_min + (np.arange(grid.ny) + 0.5) * grid.dy
    cz = grid.z_min + (np.arange(grid.nz) + 0.5) * grid.dz
    img = np.full((grid.nz, grid.ny, grid.nx), lambda_from_x0(background_x0, p0))
    for b in blocks:
        ix = (b.lo[0] <= cx) & (cx < b.hi[0])
        iy = (b.lo[1] <= cy) & (cy < b.hi[1])
        iz = (b.lo[2] <= cz) & (cz < b.hi[2])
        img[np.ix_(iz, iy, ix)] = lambda_from_x0(b.x0_mm, p0)
    return img.reshape(-1)


def generate(grid, lam: np.ndarray, n: int, seed: int, first: int = 0, theta_max: float = np.pi / 3,
             p_min: float = 1.0, p_max: float = 10.0, p0: float = 3.0, plane_gap: float = 500.0, n_planes: int = 3,
             hit_sigma: float = 1.0) -> np.ndarray:
    """Tracks (n, 14) of muons first .. first+n-1 of the seeded stream (host, OpenMP)."""
    lam = np.ascontiguousarray(lam, np.float64).reshape(-1)
    if lam.size != grid.nx * grid.ny * grid.nz:
        raise ValueError("lambda image does not match the grid")
    prm = GenParams(seed, theta_max, p_min, p_max, p0, plane_gap, n_planes, 0, hit_sigma)
    out = np.empty((n, 14), np.float64)
    g = O.make_grid(grid)
    rc = O.lib().oracle_generate(C.byref(g), O._d(lam), C.byref(prm), first, n, out.ctypes.data_as(C.c_void_p))
    if rc:
        raise ValueError("oracle_generate: invalid parameters")
    return out
