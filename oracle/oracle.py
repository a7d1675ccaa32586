"""ctypes view of the FP64 CPU oracle (oracle/muto_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline / reference leg of ``bench.py`` -- to check results, never as
the product path.  ``build()`` compiles the oracle into ``oracle/_build`` with
``g++ -O3 -fopenmp -ffp-contract=off`` (with ``synthetic.cpp``, the tracks of
the CPU-baseline legs).  ``fit_records`` (the raw-hit line
fit, with numpy's SVD) is restated here in Python.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "muto_oracle.cpp"
SRCS = [SRC, HERE / "synthetic.cpp"]  # synthetic.cpp: the tracks of the CPU-baseline legs
BUILD = HERE / "_build"
LIB = BUILD / "libmuto_oracle.so"
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]


class Grid(C.Structure):  # == muto_grid
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32), ("pad", C.c_uint32),
                ("x_min", C.c_double), ("y_min", C.c_double), ("z_min", C.c_double),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double)]


class Cfg(C.Structure):  # == oracle_cfg
    _fields_ = [("update_with_mean", C.c_int32), ("mean_percentile", C.c_int32), ("straight_line", C.c_int32),
                ("has_energy", C.c_int32), ("early_stop", C.c_int32), ("num_iteration", C.c_int32),
                ("total_num_rays", C.c_int64), ("error_xy", C.c_double), ("error_dz_outer", C.c_double),
                ("error_dz_inner", C.c_double), ("angle_unit_mag", C.c_double), ("eps", C.c_double),
                ("is_map", C.c_int32), ("add_object_prior", C.c_int32), ("all_neighbours", C.c_int32),
                ("length_weighted", C.c_int32), ("beta", C.c_double), ("p", C.c_double), ("delta", C.c_double)]


def build(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    gen_h = HERE.parent / "muontomography_gb300" / "csrc" / "gen.h"
    if force or not LIB.exists() or any(p.stat().st_mtime > LIB.stat().st_mtime for p in [*SRCS, gen_h]):
        subprocess.run(["g++", *FLAGS, *map(str, SRCS), "-o", str(LIB)], check=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P, D, U32, U64, I64 = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), \
            C.POINTER(C.c_int64)
        L.oracle_siddon_batch.argtypes = [C.POINTER(Grid), D, D, C.c_uint64, C.c_uint32, U32, D, U32]
        L.oracle_poca.argtypes = [C.POINTER(Grid), C.POINTER(Cfg), P, C.c_uint64, D, I64, U64]
        L.oracle_pocut.argtypes = [C.POINTER(Grid), C.POINTER(Cfg), C.c_double, P, C.c_uint64, D, I64, U64]
        L.oracle_slr.argtypes = [C.POINTER(Grid), C.POINTER(Cfg), C.c_int, P, C.c_uint64, D]
        L.oracle_slr_by_level.argtypes = [C.POINTER(Grid), C.POINTER(Cfg), C.c_int, P, C.c_uint64, D]
        L.oracle_mlsd_create.restype = P
        L.oracle_mlsd_create.argtypes = [C.POINTER(Grid), C.POINTER(Cfg), P, C.c_uint64, D, C.c_int]
        L.oracle_mlsd_destroy.argtypes = [P]
        L.oracle_mlsd_counts.argtypes = [P, U64]
        L.oracle_mlsd_export.argtypes = [P, U32, D, D, U64, U32, D, D]
        L.oracle_mlsd_iterate.argtypes = [P, C.c_int]
        L.oracle_mlsd_image.argtypes = [P, D]
        L.oracle_mlsd_set_image.argtypes = [P, D]
        L.oracle_mlsd_costs.argtypes = [P, D, C.c_int]
        L.oracle_mlsd_ml_step.restype = C.c_double
        L.oracle_mlsd_ml_step.argtypes = [P, D, U32]
        L.oracle_mlsd_nll.restype = C.c_double
        L.oracle_mlsd_nll.argtypes = [P, D, D]
        L.oracle_generate.restype = C.c_int
        L.oracle_generate.argtypes = [C.POINTER(Grid), D, P, C.c_uint64, C.c_uint64, P]
        L.oracle_cubic.restype = C.c_int
        L.oracle_cubic.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, D]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_grid(g) -> Grid:
    return Grid(g.nx, g.ny, g.nz, 0, g.x_min, g.y_min, g.z_min, g.dx, g.dy, g.dz)


def make_cfg(d: dict, method: str = "mlsd") -> Cfg:
    return Cfg(int(d.get("update_with_mean", False)), int(d.get("mean_percentile", 100)),
               int(d.get("straight_line", False)), int(d.get("has_energy", False)), int(d.get("early_stop", False)),
               int(d.get("num_iteration", 10)), int(d.get("total_num_rays", 0)), float(d.get("error_xy", 1.0)),
               float(d.get("error_dz_outer", 1000.0)), float(d.get("error_dz_inner", 1000.0)),
               float(d.get("angle_unit_mag", 1.0)), float(d.get("eps", 1e-8)), 1 if method == "map" else 0,
               int(d.get("add_object_prior", False)), int(d.get("all_neighbours", False)),
               int(d.get("length_weighted", False)), float(d.get("beta", 1.0)), float(d.get("p", 1.0)),
               float(d.get("delta", 0.1)))


def siddon_batch(grid, p1: np.ndarray, p2: np.ndarray, cap: int):
    p1 = np.ascontiguousarray(p1, np.float64)
    p2 = np.ascontiguousarray(p2, np.float64)
    n = p1.shape[0]
    xyz = np.zeros((n, cap, 3), np.uint32)
    ln = np.zeros((n, cap), np.float64)
    cnt = np.zeros(n, np.uint32)
    g = make_grid(grid)
    lib().oracle_siddon_batch(C.byref(g), _d(p1), _d(p2), n, cap, xyz.ctypes.data_as(C.POINTER(C.c_uint32)), _d(ln),
                              cnt.ctypes.data_as(C.POINTER(C.c_uint32)))
    return xyz, ln, cnt


def poca(grid, cfg: dict, rays: np.ndarray):
    rays = np.ascontiguousarray(rays, np.float64)
    n = rays.shape[0]
    img = np.zeros(grid.nx * grid.ny * grid.nz, np.float64)
    assign = np.zeros((n, 3), np.int64)
    counters = np.zeros(3, np.uint64)
    g = make_grid(grid)
    c = make_cfg(cfg, "poca")
    lib().oracle_poca(C.byref(g), C.byref(c), rays.ctypes.data_as(C.c_void_p), n, _d(img),
                      assign.ctypes.data_as(C.POINTER(C.c_int64)), counters.ctypes.data_as(C.POINTER(C.c_uint64)))
    return img, assign, counters


def pocut(grid, cfg: dict, rays: np.ndarray):
    """PoCut (src/MutoPoCut.cpp:19-121); cfg["cut_percentile"] defaults to 1.0 (:14)."""
    rays = np.ascontiguousarray(rays, np.float64)
    n = rays.shape[0]
    img = np.zeros(grid.nx * grid.ny * grid.nz, np.float64)
    assign = np.zeros((n, 3), np.int64)
    counters = np.zeros(3, np.uint64)
    g = make_grid(grid)
    c = make_cfg(cfg, "poca")
    lib().oracle_pocut(C.byref(g), C.byref(c), float(cfg.get("cut_percentile", 1.0)), rays.ctypes.data_as(C.c_void_p),
                       n, _d(img), assign.ctypes.data_as(C.POINTER(C.c_int64)),
                       counters.ctypes.data_as(C.POINTER(C.c_uint64)))
    return img, assign, counters


def slr(grid, cfg: dict, rays: np.ndarray, iterative: bool = False):
    """SLR (src/MutoSLR.cpp:47-103) or, iterative, SLRIter (src/MutoSLRIter.cpp:15-83;
    cfg["num_iteration"] defaults to 1, :10)."""
    rays = np.ascontiguousarray(rays, np.float64)
    img = np.zeros(grid.nx * grid.ny * grid.nz, np.float64)
    g = make_grid(grid)
    c = make_cfg(cfg, "poca")
    n_iter = max(int(cfg.get("num_iteration", 1)), 0) if iterative else 0
    if iterative and n_iter == 0:  # no pass at all: nothing added, every voxel 0
        return img
    lib().oracle_slr(C.byref(g), C.byref(c), n_iter, rays.ctypes.data_as(C.c_void_p), rays.shape[0], _d(img))
    return img


def slr_by_level(grid, cfg: dict, rays: np.ndarray, iterative: bool = False):
    """slr() with the muons run level by level (muons sharing no voxel share a
    level; each voxel sees its muons in index order): the schedule a parallel
    SLRIter would use.  Equal to slr() bit for bit when that schedule is exact."""
    rays = np.ascontiguousarray(rays, np.float64)
    img = np.zeros(grid.nx * grid.ny * grid.nz, np.float64)
    g = make_grid(grid)
    c = make_cfg(cfg, "poca")
    n_iter = max(int(cfg.get("num_iteration", 1)), 0) if iterative else 0
    if iterative and n_iter == 0:
        return img
    lib().oracle_slr_by_level(C.byref(g), C.byref(c), n_iter, rays.ctypes.data_as(C.c_void_p), rays.shape[0],
                              _d(img))
    return img


def cubic(p3: float, p2: float, p1: float, p0: float, tol: float = 1e-8):
    roots = np.zeros(3, np.float64)
    n = lib().oracle_cubic(p3, p2, p1, p0, tol, _d(roots))
    return n, roots[: max(n, 0)]


class Mlsd:
    """MutoMLSD / MutoMAP restated on the CPU (serial muon loop, OpenMP over voxels)."""

    def __init__(self, grid, cfg: dict, rays: np.ndarray, init_img: np.ndarray, method: str = "mlsd",
                 keep_paths: bool = True):
        self.grid = grid
        self.V = grid.nx * grid.ny * grid.nz
        self._rays = np.ascontiguousarray(rays, np.float64)
        init = np.ascontiguousarray(np.asarray(init_img, np.float64).reshape(-1, order="F"))
        g = make_grid(grid)
        c = make_cfg(cfg, method)
        self._h = lib().oracle_mlsd_create(C.byref(g), C.byref(c), self._rays.ctypes.data_as(C.c_void_p),
                                           self._rays.shape[0], _d(init), 1 if keep_paths else 0)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_mlsd_destroy(self._h)
            self._h = None

    def counts(self) -> dict:
        o = np.zeros(8, np.uint64)
        lib().oracle_mlsd_counts(self._h, o.ctypes.data_as(C.POINTER(C.c_uint64)))
        keys = ["n_total", "n_scat_in_grid", "n_pairs", "n_singular", "n_nonconverged", "n_bad_index",
                "iterations_done", "stopped"]
        return {k: int(v) for k, v in zip(keys, o)}

    def export(self) -> dict:
        c = self.counts()
        n, p = c["n_scat_in_grid"], c["n_pairs"]
        kept = np.zeros(n, np.uint32)
        info = np.zeros((n, 6), np.float64)
        scat = np.zeros((n, 3), np.float64)
        off = np.zeros(n + 1, np.uint64)
        idx = np.zeros(p, np.uint32)
        ln = np.zeros(p, np.float64)
        tl = np.zeros(p, np.float64)
        u32 = C.POINTER(C.c_uint32)
        lib().oracle_mlsd_export(self._h, kept.ctypes.data_as(u32), _d(info), _d(scat),
                                 off.ctypes.data_as(C.POINTER(C.c_uint64)), idx.ctypes.data_as(u32), _d(ln), _d(tl))
        return {"kept": kept, "info": info, "scat": scat, "off": off, "idx": idx, "len": ln, "tail": tl}

    def iterate(self, n: int) -> int:
        return lib().oracle_mlsd_iterate(self._h, n)

    def image(self) -> np.ndarray:
        out = np.zeros(self.V, np.float64)
        lib().oracle_mlsd_image(self._h, _d(out))
        return out

    def set_image(self, img: np.ndarray) -> None:
        x = np.ascontiguousarray(np.asarray(img, np.float64).reshape(-1, order="F"))
        lib().oracle_mlsd_set_image(self._h, _d(x))

    def costs(self) -> np.ndarray:
        out = np.zeros(4096, np.float64)
        n = lib().oracle_mlsd_costs(self._h, _d(out), 4096)
        return out[:n]

    def ml_step(self) -> tuple[float, np.ndarray, np.ndarray]:
        out = np.zeros(self.V, np.float64)
        mult = np.zeros(self.V, np.uint32)
        c = lib().oracle_mlsd_ml_step(self._h, _d(out), mult.ctypes.data_as(C.POINTER(C.c_uint32)))
        return c, out, mult

    def nll(self, lam: np.ndarray, grad: bool = False):
        lam = np.ascontiguousarray(np.asarray(lam, np.float64).reshape(-1, order="F"))
        if not grad:
            return lib().oracle_mlsd_nll(self._h, _d(lam), None)
        g = np.zeros(self.V, np.float64)
        v = lib().oracle_mlsd_nll(self._h, _d(lam), _d(g))
        return v, g


def fit_records(records: np.ndarray, z_layers, n_middle: int) -> np.ndarray:
    """MutoFile::getMuonData's record loop (src/MutoFile.cpp:58-78) and its
    per-record fit getRayDataFromTemp (:248-304), restated with numpy's SVD
    in place of Eigen's JacobiSVD: each half's hits are centred, the first
    right singular vector is the direction (oriented here with d_z > 0, which
    the SVD leaves open), and the line is evaluated at layer n_middle-1 (in)
    and n_middle (out).  Records holding a NaN are dropped.  Returns
    (kept, 14) rows {ein, eout, pin, pout, din, dout}."""
    rec = np.asarray(records, np.float64)
    z = np.asarray(z_layers, np.float64)
    nz = z.size
    out = []
    for row in rec:
        if np.isnan(row).any():
            continue
        hits = np.stack([row[1:2 * nz + 1:2], row[2:2 * nz + 2:2], z], axis=1)
        ray = [row[0], row[2 * nz + 1]]
        lines = []
        for part, zt in ((hits[:n_middle], z[n_middle - 1]), (hits[n_middle:], z[n_middle])):
            c = part.mean(axis=0)
            d = np.linalg.svd(part - c, full_matrices=False)[2][0]
            d = d if d[2] >= 0 else -d
            t = (zt - c[2]) / d[2]
            lines.append((np.array([c[0] + t * d[0], c[1] + t * d[1], zt]), d))
        ray += list(lines[0][0]) + list(lines[1][0]) + list(lines[0][1]) + list(lines[1][1])
        out.append(ray)
    return np.asarray(out, np.float64).reshape(-1, 14)
