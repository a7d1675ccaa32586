"""GB300 muon-tomography reconstruction (Siddon -> PoCA -> MLSD EM -> MAP).

Python view of the C ABI in ``include/muto_gb300.h``.  The reconstruction
classes mirror the reference's (``MutoPoCA(json)``, ``MutoMLSD(json)``,
``MutoMAP(json)`` with ``reconstruct(rays) -> image``); the compute runs in
the sm_103a kernels of ``lib/libmuto_gb300.so``.  There is no CPU fallback:
without the library or a GPU the calls raise.

Tracks are ``float64`` arrays of shape (N, 14), the reference's RayData
layout: ``ein, eout, pin[3], pout[3], din[3], dout[3]``.  Images are returned
as (nx, ny, nz) Fortran-ordered arrays (x fastest, like the reference's
column-major Eigen tensor).
"""
from __future__ import annotations

import ctypes as C
import json as _json
from dataclasses import dataclass
from typing import Iterable, Sequence

import numpy as np

from . import _lib
from ._lib import MutoError, check

__all__ = [
    "Grid", "Block", "X0_MM", "RAY_FIELDS", "MutoError", "Reconstruction", "MutoPoCA", "MutoPoCut", "MutoSLR", "MutoSLRIter", "MutoMLSD", "MutoMAP",
    "phantom", "generate", "lambda_from_x0", "save_image", "load_image", "siddon_batch", "fit_tracks", "library", "Batch",
]

RAY_FIELDS = ("ein", "eout", "pin", "pout", "din", "dout")

# radiation lengths in mm
X0_MM = {"air": 303900.0, "aluminium": 88.97, "iron": 17.57, "lead": 5.612, "concrete": 115.0, "water": 360.8}


def library():
    return _lib.load()


@dataclass(frozen=True)
class Grid:
    nx: int
    ny: int
    nz: int
    x_min: float = 0.0
    y_min: float = 0.0
    z_min: float = 0.0
    dx: float = 10.0
    dy: float = 10.0
    dz: float = 10.0

    @property
    def nvox(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def shape(self) -> tuple[int, int, int]:
        return (self.nx, self.ny, self.nz)

    def c(self) -> _lib.muto_grid:
        return _lib.muto_grid(self.nx, self.ny, self.nz, 0, self.x_min, self.y_min, self.z_min, self.dx, self.dy,
                              self.dz)

    @staticmethod
    def from_c(g: _lib.muto_grid) -> "Grid":
        return Grid(g.nx, g.ny, g.nz, g.x_min, g.y_min, g.z_min, g.dx, g.dy, g.dz)

    def json(self) -> dict:
        return {"nx": self.nx, "ny": self.ny, "nz": self.nz, "x_min": self.x_min, "y_min": self.y_min,
                "z_min": self.z_min, "dx": self.dx, "dy": self.dy, "dz": self.dz}


@dataclass(frozen=True)
class Block:
    lo: tuple[float, float, float]
    hi: tuple[float, float, float]
    x0_mm: float


def lambda_from_x0(x0_mm: float, p0: float = 3.0) -> float:
    return float(library().muto_lambda_from_x0(x0_mm, p0))


def phantom(grid: Grid, blocks: Sequence[Block], background_x0: float = X0_MM["air"], p0: float = 3.0) -> np.ndarray:
    """Flat (V,) lambda image, x fastest."""
    lib = library()
    arr = (_lib.muto_block * max(len(blocks), 1))()
    for k, b in enumerate(blocks):
        arr[k].lo[:] = b.lo
        arr[k].hi[:] = b.hi
        arr[k].x0_mm = b.x0_mm
    out = np.empty(grid.nvox, dtype=np.float64)
    g = grid.c()
    check(lib.muto_phantom(C.byref(g), arr, len(blocks), background_x0, p0, _lib.dptr(out)), "muto_phantom")
    return out


def generate(grid: Grid, lam: np.ndarray, n: int, seed: int, first: int = 0, theta_max: float = np.pi / 3,
             p_min: float = 1.0, p_max: float = 10.0, p0: float = 3.0, plane_gap: float = 500.0, n_planes: int = 3,
             hit_sigma: float = 1.0) -> np.ndarray:
    """Synthetic tracks (n, 14) of muons first .. first+n-1 of the seeded stream."""
    lib = library()
    lam = np.ascontiguousarray(lam, dtype=np.float64).reshape(-1, order="F") if lam.ndim == 3 else \
        np.ascontiguousarray(lam, dtype=np.float64)
    if lam.size != grid.nvox:
        raise ValueError("lambda image does not match the grid")
    p = _lib.muto_gen_params(seed, theta_max, p_min, p_max, p0, plane_gap, n_planes, 0, hit_sigma)
    out = np.empty((n, 14), dtype=np.float64)
    g = grid.c()
    check(lib.muto_generate(C.byref(g), _lib.dptr(lam), C.byref(p), first, n, out.ctypes.data_as(C.c_void_p)),
          "muto_generate")
    return out


def _as_image(flat: np.ndarray, grid: Grid) -> np.ndarray:
    return flat.reshape(grid.shape, order="F")


def _flat(img: np.ndarray) -> np.ndarray:
    if img.ndim == 3:
        return np.ascontiguousarray(img.reshape(-1, order="F"), dtype=np.float64)
    return np.ascontiguousarray(img, dtype=np.float64)


# methods whose image comes out of prepare (no EM iterations)
ONE_SHOT = ("poca", "pocut", "slr", "slr_iter")


class Reconstruction:
    """One reconstruction handle (``muto_create``).  method: poca | pocut | slr | slr_iter | mlsd | map."""

    def __init__(self, method: str, config: dict | str | None = None):
        self._lib = library()
        self.method = method
        text = config if isinstance(config, str) else _json.dumps(config or {})
        h = C.c_void_p()
        rc = self._lib.muto_create(method.encode(), text.encode(), C.byref(h))
        check(rc, f"muto_create({method})")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.muto_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int, what: str) -> None:
        if rc != _lib.MUTO_OK:
            raise MutoError(rc, f"{what}: {self.status()['message']}")

    # --- reference API ---------------------------------------------------
    def get_current_grid(self) -> Grid:
        g = _lib.muto_grid()
        check(self._lib.muto_get_grid(self._h, C.byref(g)), "muto_get_grid")
        return Grid.from_c(g)

    def set_initial_image(self, img: np.ndarray | None, grid: Grid | None = None) -> None:
        if img is None:
            self._check(self._lib.muto_set_initial_image(self._h, None, None), "muto_set_initial_image")
            return
        flat = _flat(img)
        g = (grid or self.get_current_grid()).c()
        self._check(self._lib.muto_set_initial_image(self._h, _lib.dptr(flat), C.byref(g)), "muto_set_initial_image")
        self._keep = flat

    def reconstruct(self, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        if rays.ndim != 2 or rays.shape[1] != 14:
            raise ValueError("rays must have shape (N, 14)")
        # the output size follows the grid after the initial image is resolved: stage it
        self.load_tracks(rays)
        self.prepare()
        if self.method not in ONE_SHOT:
            self.iterate(self.config_iterations())
        return self.image()

    # --- staged API ------------------------------------------------------
    def load_tracks(self, rays: np.ndarray, on_device_ptr: int | None = None, n: int | None = None) -> None:
        if on_device_ptr is not None:
            self._check(self._lib.muto_load_tracks(self._h, C.c_void_p(on_device_ptr), int(n), 1), "muto_load_tracks")
            return
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        self._check(self._lib.muto_load_tracks(self._h, rays.ctypes.data_as(C.c_void_p), rays.shape[0], 0),
                    "muto_load_tracks")

    def prepare(self) -> None:
        self._check(self._lib.muto_prepare(self._h), "muto_prepare")

    def iterate(self, n: int) -> None:
        self._check(self._lib.muto_iterate(self._h, int(n)), "muto_iterate")

    def image(self) -> np.ndarray:
        g = self.get_current_grid()
        out = np.empty(g.nvox, dtype=np.float64)
        self._check(self._lib.muto_get_image(self._h, _lib.dptr(out), out.size), "muto_get_image")
        return _as_image(out, g)

    def set_image(self, img: np.ndarray) -> None:
        flat = _flat(img)
        self._check(self._lib.muto_set_image(self._h, _lib.dptr(flat), flat.size), "muto_set_image")

    def config_iterations(self) -> int:
        return int(getattr(self, "_n_iter", 10))

    def status(self) -> dict:
        s = _lib.muto_status()
        self._lib.muto_get_status(self._h, C.byref(s))
        d = {name: getattr(s, name) for name, _ in _lib.muto_status._fields_ if name != "message"}
        d["message"] = s.message.decode(errors="replace")
        return d

    # --- probes ----------------------------------------------------------
    def export_paths(self) -> dict:
        st = self.status()
        n, p = st["n_scat_in_grid"], st["n_pairs"]
        kept = np.empty(n, np.uint32)
        info = np.empty((n, 6), np.float64)
        off = np.empty(n + 1, np.uint64)
        idx = np.empty(p, np.uint32)
        ln = np.empty(p, np.float64)
        tl = np.empty(p, np.float64)
        self._check(self._lib.muto_export_paths(self._h, _lib.u32ptr(kept), _lib.dptr(info), _lib.u64ptr(off),
                                                _lib.u32ptr(idx), _lib.dptr(ln), _lib.dptr(tl)), "muto_export_paths")
        return {"kept": kept, "info": info, "off": off, "idx": idx, "len": ln, "tail": tl}

    def poca_assignment(self, n: int) -> np.ndarray:
        out = np.empty((n, 3), np.int64)
        self._check(self._lib.muto_poca_assignment(self._h, _lib.i64ptr(out), n), "muto_poca_assignment")
        return out

    def multiplicity(self) -> np.ndarray:
        g = self.get_current_grid()
        out = np.empty(g.nvox, np.uint32)
        self._check(self._lib.muto_get_multiplicity(self._h, _lib.u32ptr(out), out.size), "muto_get_multiplicity")
        return out

    # --- adjoint ---------------------------------------------------------
    def nll(self, log_lambda: np.ndarray) -> float:
        x = _flat(log_lambda)
        v = C.c_double()
        self._check(self._lib.muto_nll_forward(self._h, _lib.dptr(x), C.byref(v)), "muto_nll_forward")
        return v.value

    def nll_grad(self, log_lambda: np.ndarray) -> tuple[float, np.ndarray]:
        x = _flat(log_lambda)
        g = np.empty_like(x)
        v = C.c_double()
        self._check(self._lib.muto_nll_backward(self._h, _lib.dptr(x), C.byref(v), _lib.dptr(g)), "muto_nll_backward")
        return v.value, g

    def gradient_solve(self, n_iter: int) -> float:
        v = C.c_double()
        self._check(self._lib.muto_gradient_solve(self._h, int(n_iter), C.byref(v)), "muto_gradient_solve")
        return v.value

    def gradient_solve_until(self, target: float, max_iter: int) -> tuple[float, int]:
        """The gradient solver run until F <= target: (F reached, iterations taken)."""
        v, it = C.c_double(), C.c_int()
        self._check(self._lib.muto_gradient_solve_until(self._h, int(max_iter), float(target), C.byref(v),
                                                         C.byref(it)), "muto_gradient_solve_until")
        return v.value, it.value

    # --- profiling -------------------------------------------------------
    def set_profiling(self, on: bool) -> None:
        self._check(self._lib.muto_set_profiling(self._h, 1 if on else 0), "muto_set_profiling")

    def kernel_stats(self, name: str) -> tuple[int, float]:
        n = C.c_uint64()
        t = C.c_double()
        self._lib.muto_kernel_stats(self._h, name.encode(), C.byref(n), C.byref(t))
        return int(n.value), float(t.value)

    def reset_kernel_stats(self) -> None:
        self._lib.muto_reset_kernel_stats(self._h)

    def launch_count(self) -> int:
        n = C.c_uint64()
        self._lib.muto_launch_count(self._h, C.byref(n))
        return int(n.value)


class MutoPoCA(Reconstruction):
    """MutoPoCA(json) / reconstruct (src/MutoPoCA.cpp:24, :51-134)."""

    def __init__(self, config: dict | None = None):
        super().__init__("poca", config)


class MutoPoCut(Reconstruction):
    """MutoPoCut(json) / reconstruct (src/MutoPoCut.cpp:12-121): PoCA keeping, per
    voxel, the lowest ``cut_percentile`` of the scattering values (default 1.0)."""

    def __init__(self, config: dict | None = None):
        super().__init__("pocut", config)


class MutoSLR(Reconstruction):
    """MutoSLR(json) / reconstruct (src/MutoSLR.cpp:21-103): straight-line back-projection
    of the squared scattering angles over the voxels between the grid's top and bottom."""

    def __init__(self, config: dict | None = None):
        super().__init__("slr", config)


class MutoSLRIter(Reconstruction):
    """MutoSLRIter(json) / reconstruct (src/MutoSLRIter.cpp:9-83): SLR repeated
    ``num_iteration`` times (default 1), later passes in place and in muon order."""

    def __init__(self, config: dict | None = None):
        super().__init__("slr_iter", config)


class MutoMLSD(Reconstruction):
    """MutoMLSD(json) / reconstruct (src/MutoMLSD.cpp:47-220)."""

    def __init__(self, config: dict | None = None):
        super().__init__("mlsd", config)
        self._n_iter = int((config or {}).get("num_iteration", 10))


class MutoMAP(Reconstruction):
    """MutoMAP(json) / reconstruct (src/MutoMAP.cpp:12-205)."""

    def __init__(self, config: dict | None = None):
        super().__init__("map", config)
        self._n_iter = int((config or {}).get("num_iteration", 10))


class Batch(Reconstruction):
    """Many independent MLSD scans (own grids and tracks) reconstructed together:
    every pass of an EM iteration is one launch over all scans (muto_batch_*)."""

    def __init__(self, config: dict, grids: Sequence[Grid]):
        self._lib = library()
        self.method = "mlsd"
        arr = (_lib.muto_grid * len(grids))(*[g.c() for g in grids])
        h = C.c_void_p()
        check(self._lib.muto_batch_create(b"mlsd", _json.dumps(config).encode(), len(grids), arr, C.byref(h)),
              "muto_batch_create")
        self._h = h
        self.grids = list(grids)
        self._n_iter = int(config.get("num_iteration", 10))

    def load_scan(self, scan: int, rays: np.ndarray | None = None, on_device_ptr: int | None = None,
                  n: int | None = None) -> None:
        if on_device_ptr is not None:
            self._check(self._lib.muto_batch_load_tracks(self._h, scan, C.c_void_p(on_device_ptr), int(n), 1),
                        "muto_batch_load_tracks")
            return
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        self._keep_rays = getattr(self, "_keep_rays", {})
        self._keep_rays[scan] = rays
        self._check(self._lib.muto_batch_load_tracks(self._h, scan, rays.ctypes.data_as(C.c_void_p), rays.shape[0], 0),
                    "muto_batch_load_tracks")

    def scan_image(self, scan: int) -> np.ndarray:
        g = self.grids[scan]
        out = np.empty(g.nvox, dtype=np.float64)
        self._check(self._lib.muto_batch_get_image(self._h, scan, _lib.dptr(out), out.size), "muto_batch_get_image")
        return _as_image(out, g)

    def scan_info(self, scan: int) -> tuple[int, int]:
        k, p = C.c_uint64(), C.c_uint64()
        self._check(self._lib.muto_batch_scan_info(self._h, scan, C.byref(k), C.byref(p)), "muto_batch_scan_info")
        return int(k.value), int(p.value)

    def reconstruct_all(self, scans: Sequence[np.ndarray]) -> list[np.ndarray]:
        for k, r in enumerate(scans):
            self.load_scan(k, r)
        self.prepare()
        self.iterate(self._n_iter)
        return [self.scan_image(k) for k in range(len(scans))]


def siddon_batch(grid: Grid, p1: np.ndarray, p2: np.ndarray, cap: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """MutoSiddon::getVoxelPath for many segments on the GPU: (xyz (n,cap,3), len (n,cap), counts (n,))."""
    lib = library()
    p1 = np.ascontiguousarray(p1, np.float64)
    p2 = np.ascontiguousarray(p2, np.float64)
    n = p1.shape[0]
    xyz = np.zeros((n, cap, 3), np.uint32)
    ln = np.zeros((n, cap), np.float64)
    cnt = np.zeros(n, np.uint32)
    g = grid.c()
    check(lib.muto_siddon_batch(C.byref(g), _lib.dptr(p1), _lib.dptr(p2), n, cap, _lib.u32ptr(xyz), _lib.dptr(ln),
                                _lib.u32ptr(cnt)), "muto_siddon_batch")
    return xyz, ln, cnt


def fit_tracks(records: np.ndarray, z_layers, n_middle: int) -> np.ndarray:
    """MutoFile::getMuonData's per-record line fit on the GPU (src/MutoFile.cpp:248-304).

    records: (n, 2*nz+2) float32 or float64 rows {ein, x0, y0, ..., eout}; rows
    holding a NaN are dropped.  Returns (kept, 14) tracks in the muto_ray layout."""
    lib = library()
    rec = np.ascontiguousarray(records)
    if rec.dtype not in (np.float32, np.float64):
        rec = rec.astype(np.float64)
    z = np.ascontiguousarray(z_layers, np.float64)
    if rec.ndim != 2 or rec.shape[1] != 2 * z.size + 2:
        raise ValueError(f"records need 2*nz+2 = {2 * z.size + 2} columns, got shape {rec.shape}")
    n = rec.shape[0]
    out = np.zeros((n, 14), np.float64)
    kept = C.c_uint64()
    check(lib.muto_fit_tracks(rec.ctypes.data_as(C.c_void_p), rec.itemsize, n, _lib.dptr(z), z.size, n_middle,
                              out.ctypes.data_as(C.c_void_p), C.byref(kept)), "muto_fit_tracks")
    return out[: kept.value]


def save_image(path: str, img: np.ndarray, grid: Grid, method: str, n_ray: int, n_iter: int, precision: int = 4) -> None:
    lib = library()
    flat = _flat(img)
    g = grid.c()
    check(lib.muto_save_image(str(path).encode(), _lib.dptr(flat), C.byref(g), method.encode(), n_ray, n_iter,
                              precision), f"muto_save_image({path})")


def load_image(path: str) -> tuple[np.ndarray, dict]:
    lib = library()
    g = _lib.muto_grid()
    m = C.create_string_buffer(17)
    nr, ni, pr = C.c_uint32(), C.c_uint32(), C.c_uint32()
    check(lib.muto_load_image(str(path).encode(), None, 0, C.byref(g), m, C.byref(nr), C.byref(ni), C.byref(pr)),
          f"muto_load_image({path})")
    grid = Grid.from_c(g)
    out = np.empty(grid.nvox, np.float64)
    check(lib.muto_load_image(str(path).encode(), _lib.dptr(out), out.size, C.byref(g), m, C.byref(nr), C.byref(ni),
                              C.byref(pr)), f"muto_load_image({path})")
    header = {"grid": grid, "method": m.raw[:16].split(b"\0")[0].decode(errors="replace"), "n_ray": nr.value,
              "n_iter": ni.value, "precision": pr.value}
    return _as_image(out, grid), header
