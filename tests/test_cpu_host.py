"""CPU tests: the C ABI library loads and exports every declared symbol, and
the host-side logic (config parsing, image files, synthetic data) behaves.
No kernel is launched here."""
import ctypes as C
import re

import numpy as np
import pytest

import muontomography_gb300 as M
from muontomography_gb300 import _lib


def header_functions():
    text = _lib.header_path().read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(muto_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_api():
    names = header_functions()
    for must in ("muto_create", "muto_reconstruct", "muto_siddon_batch", "muto_nll_backward", "muto_save_image"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_the_header():
    assert set(header_functions()) <= set(_lib.SIGNATURES), set(header_functions()) - set(_lib.SIGNATURES)


@pytest.mark.parametrize("method,cfg,code", [
    ("mlsd", "{not json", 2),
    ("mlsd", '{"grid": {"nx": "ten"}}', 2),
    ("mlsd", '{"precision": "half"}', 2),
    ("mlsd", '{"grid": {"nx": 0}}', 2),
    ("map", '{"num_iteration": -1}', 2),
    ("mlsd", '{"update_with_mean": 3}', 2),
    ("mlsd", '[1, 2]', 2),
    ("slr_v2", "{}", 1),
    ("slr_iter", '{"num_iteration": -1}', 2),
    ("slr_iter", '{"slr_iter_schedule": "shuffled"}', 2),
    ("mlsd", '{"update_with_mean": true, "fused_variant": "split9"}', 2),
    ("mlsd", '{"path_lists": "sideways"}', 2),
    ("pocut", '{"cut_percentile": "most"}', 2),
    ("mlsd", '{"muon_layout": "spiral"}', 2),
    ("mlsd", '{"muon_pass": "fast"}', 2),
])
def test_config_errors_are_reported_before_any_device_call(lib, method, cfg, code):
    h = C.c_void_p()
    rc = lib.muto_create(method.encode(), cfg.encode(), C.byref(h))
    assert rc == code
    assert not h.value


def test_lambda_from_x0(lib):
    assert M.lambda_from_x0(17.57) == pytest.approx((0.0136 / 3.0) ** 2 / 17.57, rel=1e-15)


@pytest.mark.parametrize("precision", [4, 8])
def test_image_file_roundtrip_and_header_layout(tmp_path, precision):
    g = M.Grid(5, 4, 3, -1.5, -2.0, -2.5, 0.5, 1.0, 1.5)
    img = np.random.default_rng(0).uniform(0, 1e-6, g.nvox).reshape(g.shape, order="F")
    p = tmp_path / "img.bin"
    M.save_image(str(p), img, g, "mlsd", 123456, 50, precision)
    raw = p.read_bytes()
    assert len(raw) == 64 + g.nvox * precision
    assert raw[0] == 64 and raw[1] == 1
    assert raw[2:6] == b"mlsd" and raw[6:18] == b"\0" * 12
    assert int.from_bytes(raw[18:22], "little") == 123456
    assert int.from_bytes(raw[22:24], "little") == 50
    assert int.from_bytes(raw[24:26], "little") == precision
    assert [int.from_bytes(raw[26 + 2 * k:28 + 2 * k], "little") for k in range(3)] == [5, 4, 3]
    assert np.frombuffer(raw[32:56], "<f4").tolist() == [-1.5, -2.0, -2.5, 0.5, 1.0, 1.5]
    assert raw[56:64] == b"\0" * 8
    back, hdr = M.load_image(str(p))
    assert hdr["grid"] == g and hdr["method"] == "mlsd" and hdr["n_iter"] == 50 and hdr["precision"] == precision
    want = img.astype(np.float32).astype(np.float64) if precision == 4 else img
    assert np.array_equal(back, want)
    data = np.frombuffer(raw[64:], "<f4" if precision == 4 else "<f8")
    assert np.array_equal(data, want.reshape(-1, order="F"))  # column-major, x fastest


def test_load_image_missing_file_is_an_io_error(tmp_path):
    with pytest.raises(M.MutoError) as e:
        M.load_image(str(tmp_path / "nope.bin"))
    assert e.value.code == 6


def test_generator_is_deterministic_per_muon():
    g = M.Grid(8, 8, 8, -200.0, -200.0, -200.0, 50.0, 50.0, 50.0)
    lam = M.phantom(g, [M.Block((-50, -50, -50), (50, 50, 50), M.X0_MM["iron"])])
    a = M.generate(g, lam, 400, seed=7)
    b = np.concatenate([M.generate(g, lam, 150, seed=7), M.generate(g, lam, 250, seed=7, first=150)])
    assert np.array_equal(a, b)
    c = M.generate(g, lam, 400, seed=8)
    assert not np.array_equal(a, c)
    # geometry: pin / pout on the grid's top / bottom faces, directions unit with d_z > 0
    assert np.all(a[:, 4] == 200.0) and np.all(a[:, 7] == -200.0)
    for k in (8, 11):
        d = a[:, k:k + 3]
        assert np.allclose(np.linalg.norm(d, axis=1), 1.0) and np.all(d[:, 2] > 0)
    assert np.all((a[:, 0] >= 1.0) & (a[:, 0] <= 10.0))


def test_phantom_voxel_centres():
    g = M.Grid(4, 4, 4, 0.0, 0.0, 0.0, 10.0, 10.0, 10.0)
    lam = M.phantom(g, [M.Block((0, 0, 0), (20, 20, 20), M.X0_MM["lead"])], M.X0_MM["air"])
    img = lam.reshape(g.shape, order="F")
    assert np.all(img[:2, :2, :2] == M.lambda_from_x0(M.X0_MM["lead"]))
    assert img[2, 0, 0] == M.lambda_from_x0(M.X0_MM["air"])


def _bench(*argv, env=None):
    import json
    import os
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    e = dict(os.environ, **(env or {}))
    out = subprocess.run([sys.executable, str(root / "bench.py"), *argv], cwd=root, env=e, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    return [json.loads(ln) for ln in lines]


def test_reference_arm_prints_one_contract_line():
    # the CPU reference arm on a small sample: one JSON line with the bench's keys
    (line,) = _bench("--impl", "reference", "--steps", "1", "--warmup", "0", "--cpu-sample", "3000")
    assert line["impl"] == "reference"
    assert line["metric"] == "EM-iter muon\u00b7voxel updates/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1 and line["n_gpus"] == 1
    assert line["config"]["workload"] == "grid256x256x128_10mm_100M" and line["config"]["mode"] == "mean"
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert "the first 3000 of the 100000000 muons" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_without_work():
    env = {"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2", "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": "29533"}
    assert _bench("--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-sample", "3000",
                  env=env) == []


@pytest.mark.parametrize("argv,method,mode", [
    (("--workload", "map128x128x64_15mm"), "map", "median"),
    (("--workload", "cube100_20mm"), "mlsd", "median"),
    (("--workload", "cube100_20mm", "--mode", "mean"), "mlsd", "mean"),
])
def test_reference_arm_other_workloads(argv, method, mode):
    (line,) = _bench("--impl", "reference", "--steps", "1", "--warmup", "0", "--cpu-sample", "2000", *argv)
    assert line["config"]["method"] == method and line["config"]["mode"] == mode and line["value"] > 0


def test_reference_arm_loads_no_product_library():
    # the reference leg times the CPU port on tracks it makes itself: the
    # product's CUDA library must not be in its process
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    code = ("import atexit, runpy, sys\n"
            "def libs():\n"
            "    print('LIBS', sorted({l.split()[-1] for l in open('/proc/self/maps') if '.so' in l}))\n"
            "atexit.register(libs)\n"
            "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', '--cpu-sample', '2000']\n"
            "runpy.run_path('bench.py', run_name='__main__')\n")
    out = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    libs = [ln for ln in out.stdout.splitlines() if ln.startswith("LIBS")][0]
    assert "libmuto_oracle.so" in libs and "libmuto_gb300" not in libs and "libmuto_facade" not in libs


@pytest.mark.parametrize("name", ["muto_grid", "muto_status", "muto_block", "muto_gen_params"])
def test_ctypes_structs_match_the_c_header(tmp_path, name):
    # the Python bindings' structures have the C header's size and field offsets
    import shutil
    import subprocess

    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    st = getattr(_lib, name)
    fields = [f for f, _ in st._fields_]
    body = "\n".join(f'    printf("%zu\\n", offsetof({name}, {f}));' for f in fields)
    src = tmp_path / "layout.c"
    src.write_text(f"#include <stddef.h>\n#include <stdio.h>\n#include \"muto_gb300.h\"\n"
                   f"int main(void) {{\n    printf(\"%zu\\n\", sizeof({name}));\n{body}\n    return 0;\n}}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(_lib.header_path().parent), str(src), "-o", str(exe)], check=True,
                   capture_output=True, timeout=120)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == C.sizeof(st)
    assert out[1:] == [getattr(st, f).offset for f in fields]


def test_batch64_workload_matches_its_description():
    # 64 scans, cubic grids of 32..128 voxels of 20 mm, 50 k..5 M muons each,
    # seeded: the same scans every time
    from muontomography_gb300 import workloads as W

    wls = W.batch64()
    assert len(wls) == 64
    assert {w.grid.nx for w in wls} <= {32, 64, 96, 128}
    assert all(w.grid.nx == w.grid.ny == w.grid.nz and w.grid.dx == 20.0 for w in wls)
    counts = np.array([w.n_muons for w in wls])
    assert counts.min() >= 50_000 and counts.max() <= 5_000_000
    assert 40e6 < counts.sum() < 100e6
    again = W.batch64()
    assert [w.n_muons for w in again] == list(counts) and [w.grid for w in again] == [w.grid for w in wls]
    assert len({w.seed for w in wls}) == 64
    small = W.batch64(scale=0.01)  # the GPU test's 1/100 of the muons, at least 1 000 a scan
    assert all(1000 <= s.n_muons <= max(1000, 0.01 * w.n_muons + 1) for s, w in zip(small, wls))
