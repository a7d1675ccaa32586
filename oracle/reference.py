"""ctypes view of the reference's own reconstruction code built by
oracle/build_ref.sh (oracle/_ref/libmuto_ref.so, and its MutoFile in
oracle/_ref/libmuto_ref_file.so).

TEST INFRASTRUCTURE ONLY.  Available only where the reference sources are
mounted; used by tests/golden/make_golden.py to produce the committed golden
vectors and by the oracle pin test to compare the restatement with the
reference itself.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_ref" / "libmuto_ref.so"
FILE_LIB = HERE / "_ref" / "libmuto_ref_file.so"
CLI = HERE / "_ref" / "muto_ref_cli"
# the reference's source tree: $MUTO_REFERENCE, else a directory named
# "reference" beside this repository's root
REF = Path(os.environ.get("MUTO_REFERENCE", str(HERE.parent.parent / "reference")))


def available() -> bool:
    return (REF / "src" / "MutoMLSD.cpp").exists()


def build() -> Path:
    srcs = [REF / "src" / f for f in ("MutoSiddon.cpp", "MutoPoCA.cpp", "MutoMLSD.cpp", "MutoMAP.cpp",
                                      "MutoPoCut.cpp", "MutoSLR.cpp", "MutoSLRIter.cpp", "MutoFile.cpp")]
    deps = srcs + [HERE / "ref_harness.cpp", HERE / "ref_file_harness.cpp", HERE / "build_ref.sh"] \
        + list((HERE / "ref_shim").rglob("*"))
    deps.append(REF / "MuToTest.cpp")
    stale = [lib for lib in (LIB, FILE_LIB, CLI) if not lib.exists()
             or any(p.is_file() and p.stat().st_mtime > lib.stat().st_mtime for p in deps)]
    if stale:
        subprocess.run(["sh", str(HERE / "build_ref.sh")], check=True, capture_output=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        D, U32, U64 = C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)
        L.ref_set_initial_image.argtypes = [D, U32, D]
        L.ref_siddon.argtypes = [U32, D, D, D, C.c_uint64, C.c_uint32, U32, D, U32]
        L.ref_reconstruct.argtypes = [C.c_char_p, C.c_char_p, D, C.c_uint64, D, C.c_uint64, U32]
        L.ref_mlsd_paths.argtypes = [C.c_char_p, D, C.c_uint64, U64, U32, D, U64, U32, D, D]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _u32(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def _grid(g):
    return np.array([g.nx, g.ny, g.nz], np.uint32), np.array([g.x_min, g.y_min, g.z_min, g.dx, g.dy, g.dz], np.float64)


def set_initial_image(img: np.ndarray | None, grid=None) -> None:
    if img is None:
        lib().ref_set_initial_image(None, None, None)
        return
    n, f = _grid(grid)
    x = np.ascontiguousarray(np.asarray(img, np.float64).reshape(-1, order="F"))
    lib().ref_set_initial_image(_d(x), _u32(n), _d(f))


def siddon(grid, p1: np.ndarray, p2: np.ndarray, cap: int):
    n, f = _grid(grid)
    p1 = np.ascontiguousarray(p1, np.float64)
    p2 = np.ascontiguousarray(p2, np.float64)
    m = p1.shape[0]
    xyz = np.zeros((m, cap, 3), np.uint32)
    ln = np.zeros((m, cap), np.float64)
    cnt = np.zeros(m, np.uint32)
    lib().ref_siddon(_u32(n), _d(f), _d(p1), _d(p2), m, cap, _u32(xyz), _d(ln), _u32(cnt))
    return xyz, ln, cnt


def reconstruct(method: str, cfg: dict, rays: np.ndarray, nvox_cap: int) -> tuple[np.ndarray, tuple]:
    rays = np.ascontiguousarray(rays, np.float64)
    out = np.zeros(nvox_cap, np.float64)
    dims = np.zeros(3, np.uint32)
    rc = lib().ref_reconstruct(method.encode(), json.dumps(cfg).encode(), _d(rays), rays.shape[0], _d(out), nvox_cap,
                               _u32(dims))
    if rc != 0:
        raise RuntimeError(f"ref_reconstruct rc={rc}")
    v = int(np.prod(dims.astype(np.int64)))
    return out[:v], tuple(int(x) for x in dims)


def mlsd_paths(cfg: dict, rays: np.ndarray) -> dict:
    rays = np.ascontiguousarray(rays, np.float64)
    text = json.dumps(cfg).encode()
    sizes = np.zeros(2, np.uint64)
    L = lib()
    L.ref_mlsd_paths(text, _d(rays), rays.shape[0], sizes.ctypes.data_as(C.POINTER(C.c_uint64)), None, None, None,
                     None, None, None)
    n, p = int(sizes[0]), int(sizes[1])
    kept = np.zeros(n, np.uint32)
    info = np.zeros((n, 6), np.float64)
    off = np.zeros(n + 1, np.uint64)
    idx = np.zeros(p, np.uint32)
    ln = np.zeros(p, np.float64)
    tl = np.zeros(p, np.float64)
    L.ref_mlsd_paths(text, _d(rays), rays.shape[0], sizes.ctypes.data_as(C.POINTER(C.c_uint64)), _u32(kept), _d(info),
                     off.ctypes.data_as(C.POINTER(C.c_uint64)), _u32(idx), _d(ln), _d(tl))
    return {"kept": kept, "info": info, "off": off, "idx": idx, "len": ln, "tail": tl}


_file_lib = None


def file_lib() -> C.CDLL:
    global _file_lib
    if _file_lib is None:
        build()
        L = C.CDLL(str(FILE_LIB))
        D, U32 = C.POINTER(C.c_double), C.POINTER(C.c_uint32)
        L.ref_read_muon_data.restype = C.c_uint64
        L.ref_read_muon_data.argtypes = [C.c_char_p, D, C.c_int, C.c_int, C.c_int, D, C.c_uint64]
        L.ref_save_image.argtypes = [C.c_char_p, D, U32, D, C.c_char_p, C.c_uint32, C.c_uint32, C.c_uint32]
        L.ref_load_image.argtypes = [C.c_char_p, D, C.c_uint64, U32, D, C.c_char_p, U32, U32, U32]
        _file_lib = L
    return _file_lib


def read_muon_data(path, z_layers, n_middle: int, precision: int) -> np.ndarray:
    """MutoFile::getMuonData on one file: (n, 14) tracks as the reference fits them."""
    z = np.ascontiguousarray(z_layers, np.float64)
    L = file_lib()
    n = L.ref_read_muon_data(str(path).encode(), _d(z), z.size, n_middle, precision, None, 0)
    out = np.zeros((n, 14), np.float64)
    L.ref_read_muon_data(str(path).encode(), _d(z), z.size, n_middle, precision, _d(out), n)
    return out


def save_image(path, img: np.ndarray, grid, method: str, n_ray: int, n_iter: int, precision: int) -> None:
    """MutoFile::saveImage; img is (nx, ny, nz) or flat in column-major order."""
    n, f = _grid(grid)
    x = np.ascontiguousarray(np.asarray(img, np.float64).reshape(-1, order="F"))
    rc = file_lib().ref_save_image(str(path).encode(), _d(x), _u32(n), _d(f), method.encode(), n_ray, n_iter,
                                   precision)
    if rc != 0:
        raise RuntimeError(f"reference saveImage failed for {path}")


def load_image(path, cap: int) -> tuple[np.ndarray, dict]:
    """MutoFile::loadImage: (flat column-major image, header fields)."""
    img = np.zeros(cap, np.float64)
    n = np.zeros(3, np.uint32)
    f = np.zeros(6, np.float64)
    m = C.create_string_buffer(16)
    nr, ni, pr = (np.zeros(1, np.uint32) for _ in range(3))
    rc = file_lib().ref_load_image(str(path).encode(), _d(img), cap, _u32(n), _d(f), m, _u32(nr), _u32(ni), _u32(pr))
    if rc != 0:
        raise RuntimeError(f"reference loadImage failed for {path}")
    v = int(n[0]) * int(n[1]) * int(n[2])
    hdr = {"n": [int(k) for k in n], "f": [float(k) for k in f], "method": m.raw.split(b"\0", 1)[0].decode(),
           "n_ray": int(nr[0]), "n_iter": int(ni[0]), "precision": int(pr[0])}
    return img[:v], hdr


def run_cli(config_path) -> str:
    """The reference's command-line program (MuToTest.cpp) on a JSON config; returns its stdout."""
    build()
    r = subprocess.run([str(CLI), str(config_path)], capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        raise RuntimeError(f"reference CLI failed: {r.stdout[-500:]} {r.stderr[-500:]}")
    return r.stdout
