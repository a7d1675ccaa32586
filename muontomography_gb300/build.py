"""Build the native parts in-tree.

* ``muontomography_gb300/lib/libmuto_gb300.so`` -- the CUDA library behind
  ``include/muto_gb300.h`` (sm_103a kernels + host code).
* ``muontomography_gb300/lib/libmuto_facade.so`` and ``lib/muto`` -- the C++
  reconstruction classes (MutoPoCA / MutoMLSD / MutoMAP / MutoFile /
  MutoConfig) over the C ABI, and the command-line program.

Translation units compile in parallel; a unit is rebuilt only when it or a
header it may include is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
CPP = PKG / "cpp"
BUILD = PKG / "_build"
LIB = PKG / "lib"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-O3"] + ARCH
CXX_FLAGS = ["-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function"]

CUDA_UNITS = ["scan.cu", "setup.cu", "em_muon.cu", "em_fused.cu", "em_voxel.cu", "poca.cu", "slr.cu", "adjoint.cu", "gen.cu",
              "fit.cu", "handle.cu", "noalloc.cu"]
HOST_UNITS = ["host.cpp"]
FACADE_UNITS = ["MutoFile.cpp", "MutoReconstruction.cpp", "MutoSiddon.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _newer(src: Path, obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps] if p.exists())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def lib_path() -> Path:
    return LIB / "libmuto_gb300.so"


def facade_lib_path() -> Path:
    return LIB / "libmuto_facade.so"


def cli_path() -> Path:
    return LIB / "muto"


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    cpp_headers = list(CPP.glob("*.h")) + headers
    nv = nvcc()
    steps = []
    objs = []
    for u in CUDA_UNITS:
        src, obj = CSRC / u, BUILD / (u + ".o")
        objs.append(obj)
        if _newer(src, obj, headers):
            steps.append([nv, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)])
    for u in HOST_UNITS:
        src, obj = CSRC / u, BUILD / (u + ".o")
        objs.append(obj)
        if _newer(src, obj, headers):
            steps.append(["g++", *CXX_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)])
    fobjs = []
    for u in FACADE_UNITS:
        src, obj = CPP / u, BUILD / ("facade_" + u + ".o")
        fobjs.append(obj)
        if src.exists() and _newer(src, obj, cpp_headers):
            steps.append(["g++", *CXX_FLAGS, "-I", str(INCLUDE), "-I", str(CPP), "-I", str(CSRC), "-c", str(src),
                          "-o", str(obj)])
    jobs = jobs or min(len(steps) or 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for fut in [ex.submit(_run, s) for s in steps]:
            fut.result()
    lib = lib_path()
    if not lib.exists() or any(o.stat().st_mtime > lib.stat().st_mtime for o in objs):
        _run([nv, "-shared", *ARCH, "-o", str(lib), *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp"])
    fobjs = [o for o in fobjs if o.exists()]
    if fobjs:
        flib = facade_lib_path()
        if not flib.exists() or any(o.stat().st_mtime > flib.stat().st_mtime for o in fobjs) \
                or lib.stat().st_mtime > flib.stat().st_mtime:
            _run(["g++", "-shared", "-o", str(flib), *map(str, fobjs), "-L", str(LIB), "-lmuto_gb300",
                  "-Wl,-rpath,$ORIGIN", "-fopenmp"])
        main = CPP / "muto_main.cpp"
        cli = cli_path()
        if main.exists() and (not cli.exists() or main.stat().st_mtime > cli.stat().st_mtime
                              or flib.stat().st_mtime > cli.stat().st_mtime):
            _run(["g++", *CXX_FLAGS, "-I", str(INCLUDE), "-I", str(CPP), "-I", str(CSRC), str(main), "-o", str(cli),
                  "-L", str(LIB), "-lmuto_facade", "-lmuto_gb300", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
