"""Golden vectors produced by the reference's own code (tests/golden/make_golden.py).

CPU: the oracle reproduces every golden vector bit for bit.
GPU: the CUDA path reproduces the voxel lists and paths bit for bit and the
images within the stated tolerances.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import muontomography_gb300 as M

GOLD = Path(__file__).resolve().parent / "golden"


def load():
    s = dict(np.load(GOLD / "siddon.npz"))
    t = dict(np.load(GOLD / "tracks.npz"))
    cfgs = json.loads((GOLD / "configs.json").read_text())
    return s, t, cfgs


def grid_of(a):
    return M.Grid(int(a[0]), int(a[1]), int(a[2]), *map(float, a[3:]))


def bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


S, T, CFG = load()
EM_CASES = [k for k in CFG if k.startswith(("mlsd_", "map_"))]


# ----------------------------------------------------------------- oracle pin
def test_oracle_siddon_matches_golden(oracle):
    g = grid_of(S["grid"])
    cap = S["xyz"].shape[1]
    xyz, ln, cnt = oracle.siddon_batch(g, S["p1"], S["p2"], cap)
    assert np.array_equal(cnt, S["count"])
    assert np.array_equal(xyz, S["xyz"])
    assert np.array_equal(bits(ln), bits(S["len"]))


@pytest.mark.parametrize("name", ["poca_lw", "poca_dz", "poca_straight"])
def test_oracle_poca_matches_golden(oracle, name):
    img, _, _ = oracle.poca(grid_of(T["grid"]), CFG[name], T["rays"])
    assert np.array_equal(bits(img), bits(T[name]))


POCUT_CASES = [k for k in CFG if k.startswith("pocut_")]


@pytest.mark.parametrize("name", POCUT_CASES)
def test_oracle_pocut_matches_golden(oracle, name):
    img, _, _ = oracle.pocut(grid_of(T["grid"]), CFG[name], T["rays"])
    assert np.array_equal(bits(img), bits(T[name]))


SLR_CASES = [k for k in CFG if k.startswith("slr_")]


@pytest.mark.parametrize("name", SLR_CASES)
def test_oracle_slr_matches_golden(oracle, name):
    cfg = CFG[name]
    img = oracle.slr(grid_of(T["grid"]), cfg, T["rays"], iterative=cfg["method"] == "slr_iter")
    assert np.array_equal(bits(img), bits(T[name]))


def test_oracle_paths_match_golden(oracle):
    g = grid_of(T["grid"])
    e = oracle.Mlsd(g, CFG["paths"], T["rays"], np.full(g.nvox, 1e-7)).export()
    for k in ("kept", "off", "idx"):
        assert np.array_equal(e[k], T["paths_" + k]), k
    for k in ("len", "tail", "info"):
        assert np.array_equal(bits(e[k]), bits(T["paths_" + k])), k


@pytest.mark.parametrize("name", EM_CASES)
def test_oracle_em_matches_golden(oracle, name):
    cfg = dict(CFG[name])
    method = cfg.pop("method")
    g = grid_of(T["grid"])
    init = T["poca_seed_image"] if cfg.get("initialize_method") == 0 else np.full(g.nvox, cfg["initialize_value"])
    m = oracle.Mlsd(g, cfg, T["rays"], init, method=method)
    m.iterate(cfg["num_iteration"])
    assert np.array_equal(bits(m.image()), bits(T[name]))


def test_reference_build_still_matches_oracle_when_mounted(oracle):
    from oracle import reference as R

    if not R.available():
        pytest.skip("reference sources not mounted")
    g = grid_of(S["grid"])
    a = R.siddon(g, S["p1"], S["p2"], S["xyz"].shape[1])
    assert np.array_equal(a[2], S["count"]) and np.array_equal(bits(a[1]), bits(S["len"]))


F = dict(np.load(GOLD / "files.npz"))


@pytest.mark.parametrize("prec", [8, 4])
def test_oracle_line_fit_matches_golden(oracle, prec):
    rec = F["records64"] if prec == 8 else F["records32"]
    got = oracle.fit_records(rec, F["z_layers"], int(F["n_middle"]))
    want = F[f"tracks{prec}"]  # the stand-in's SVD orients each direction with d_z >= 0
    assert got.shape == want.shape == (398, 14)
    np.testing.assert_array_equal(got[:, :2], want[:, :2])
    np.testing.assert_allclose(got[:, 2:8], want[:, 2:8], rtol=0, atol=1e-9)
    np.testing.assert_allclose(got[:, 8:], want[:, 8:], rtol=0, atol=1e-12)


def test_reference_file_code_still_matches_golden_when_mounted(tmp_path):
    from oracle import reference as R

    if not R.available():
        pytest.skip("reference sources not mounted")
    f = tmp_path / "hits.bin"
    F["records64"].tofile(f)
    got = R.read_muon_data(f, F["z_layers"], int(F["n_middle"]), 8)
    assert np.array_equal(bits(got), bits(F["tracks8"]))
    a = F["image_grid"]
    R.save_image(tmp_path / "img.bin", F["image"], grid_of(a), "mlsd", 123456, 50, 8)
    ref = F["image_file8"].tobytes()
    ours = (tmp_path / "img.bin").read_bytes()
    assert ours[:7] == ref[:7] and ours[18:] == ref[18:]


CLI = dict(np.load(GOLD / "cli.npz"))
CLI_CFG = json.loads(CLI["configs"].tobytes())
CLI_N_ITER = {"poca": 1, "pocut": 1, "slr": 1, "slr_iter": 1, "mlsd": 5, "map": 3}


def image_file(b: bytes):
    """Header fields and body of a MutoFile image (src/MutoFile.cpp:85-133)."""
    u16 = lambda o: int.from_bytes(b[o:o + 2], "little")  # noqa: E731
    hdr = {"length": b[0], "version": b[1], "method": b[2:18].split(b"\0", 1)[0].decode(),
           "n_ray": int.from_bytes(b[18:22], "little"), "n_iter": u16(22), "precision": u16(24),
           "n": (u16(26), u16(28), u16(30)), "f": tuple(np.frombuffer(b[32:56], np.float32)), "pad": b[56:64]}
    return hdr, np.frombuffer(b[64:], np.float32 if hdr["precision"] == 4 else np.float64)


@pytest.mark.parametrize("method", list(CLI_N_ITER))
def test_oracle_reproduces_reference_cli(oracle, method):
    # MuToTest.cpp end to end (reader, reconstruction, image file; MLSD and MAP
    # start from the PoCA file): the oracle on the reference's fitted tracks
    sec = CLI_CFG[method][method]
    g = M.Grid(**sec["grid"])
    rays = CLI["tracks"]
    hdr, body = image_file(CLI[f"out_{method}"].tobytes())
    assert (hdr["length"], hdr["version"], hdr["method"], hdr["n_ray"], hdr["precision"]) == (64, 1, method, 10000, 4)
    assert hdr["n_iter"] == CLI_N_ITER[method] and hdr["n"] == (g.nx, g.ny, g.nz) and hdr["pad"] == bytes(8)
    assert hdr["f"] == tuple(np.float32([g.x_min, g.y_min, g.z_min, g.dx, g.dy, g.dz]))
    if method in ("poca", "pocut"):
        img = getattr(oracle, method)(g, sec, rays)[0]
    elif method in ("slr", "slr_iter"):
        img = oracle.slr(g, sec, rays, iterative=method == "slr_iter")
    else:
        init = image_file(CLI["out_poca"].tobytes())[1].astype(np.float64)
        o = oracle.Mlsd(g, sec, rays, init, method=method)
        o.iterate(sec["num_iteration"])
        img = o.image()
    assert (body > 0).sum() > 400
    assert np.array_equal(img.astype(np.float32), body)


def test_oracle_line_fit_matches_reference_cli_tracks(oracle):
    got = oracle.fit_records(CLI["records"], CLI["z_layers"], int(CLI["n_middle"]))
    np.testing.assert_allclose(got[:, 2:8], CLI["tracks"][:, 2:8], rtol=0, atol=1e-9)
    np.testing.assert_allclose(got[:, 8:], CLI["tracks"][:, 8:], rtol=0, atol=1e-12)


# ------------------------------------------------------------------ GPU path
@pytest.mark.gpu
def test_gpu_siddon_matches_golden(gpu):
    g = grid_of(S["grid"])
    cap = S["xyz"].shape[1]
    xyz, ln, cnt = M.siddon_batch(g, S["p1"], S["p2"], cap)
    assert np.array_equal(cnt, S["count"])
    assert np.array_equal(xyz, S["xyz"])
    assert np.array_equal(bits(ln), bits(S["len"]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["poca_lw", "poca_dz", "poca_straight"])
def test_gpu_poca_matches_golden(gpu, name):
    with M.MutoPoCA(CFG[name]) as rec:
        img = rec.reconstruct(T["rays"]).reshape(-1, order="F")
    assert rel_l2(img, T[name]) < 1e-12
    assert np.array_equal(img > 0, T[name] > 0)


@pytest.mark.gpu
@pytest.mark.parametrize("name", POCUT_CASES)
def test_gpu_pocut_matches_golden(gpu, name):
    # the kept values are summed in the reference's order (ascending, from 0);
    # the weights are FP64 atomics, as for PoCA
    with M.MutoPoCut(CFG[name]) as rec:
        img = rec.reconstruct(T["rays"]).reshape(-1, order="F")
    assert rel_l2(img, T[name]) < 1e-12 if np.any(T[name]) else not np.any(img)
    assert np.array_equal(img > 0, T[name] > 0)


@pytest.mark.gpu
@pytest.mark.parametrize("name", SLR_CASES)
def test_gpu_slr_matches_golden(gpu, name):
    # voxel walks bit-exact; atan2 (CUDA's, within 2 ulp of the correctly rounded
    # one) and the FP64 atomics of the first pass leave rounding differences
    cfg = dict(CFG[name])
    method = cfg.pop("method")
    rec = M.MutoSLRIter(cfg) if method == "slr_iter" else M.MutoSLR(cfg)
    with rec:
        img = rec.reconstruct(T["rays"]).reshape(-1, order="F")
    assert rel_l2(img, T[name]) < 1e-12
    assert np.array_equal(img > 0, T[name] > 0)


@pytest.mark.gpu
def test_gpu_paths_match_golden(gpu):
    cfg = dict(CFG["paths"], precision="fp64")
    with M.MutoMLSD(cfg) as rec:
        rec.load_tracks(T["rays"])
        rec.prepare()
        e = rec.export_paths()
    for k in ("kept", "off", "idx"):
        assert np.array_equal(e[k], T["paths_" + k]), k
    for k in ("len", "tail"):
        assert np.array_equal(bits(e[k]), bits(T["paths_" + k])), k


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-4)])
@pytest.mark.parametrize("name", EM_CASES)
def test_gpu_em_matches_golden(gpu, name, precision, tol):
    cfg = dict(CFG[name])
    method = cfg.pop("method")
    cfg["precision"] = precision
    g = grid_of(T["grid"])
    with M.Reconstruction(method, cfg) as rec:
        if cfg.get("initialize_method") == 0:
            rec.set_initial_image(T["poca_seed_image"], g)
        rec._n_iter = cfg["num_iteration"]
        img = rec.reconstruct(T["rays"]).reshape(-1, order="F")
    assert rel_l2(img, T[name]) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("method", list(CLI_N_ITER))
def test_library_cli_reproduces_reference_program_files(gpu, tmp_path, method):
    # The library's command-line program (lib/muto, the reference's
    # MuToTest.cpp on this library's classes) on the configurations the
    # reference's own program was run with: the same raw-hit file in, the
    # image file out, against the reference program's file.  MLSD and MAP
    # start from the reference program's PoCA file, as their configurations
    # say, and run in the fp64 form; the files hold float32 images.
    import subprocess

    from muontomography_gb300 import build as B

    (tmp_path / "hits.bin").write_bytes(CLI["records"].tobytes())
    (tmp_path / "poca.bin").write_bytes(CLI["out_poca"].tobytes())
    cfg = json.loads(json.dumps(CLI_CFG[method]).replace("{dir}", str(tmp_path)))
    if method in ("mlsd", "map"):
        cfg[method]["precision"] = "fp64"
    cfg["output_file"] = str(tmp_path / "out.bin")
    (tmp_path / "cfg.json").write_text(json.dumps(cfg))
    r = subprocess.run([str(B.cli_path()), str(tmp_path / "cfg.json")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    want_hdr, want = image_file(CLI[f"out_{method}"].tobytes())
    got_hdr, got = image_file((tmp_path / "out.bin").read_bytes())
    for k in ("length", "version", "method", "n_ray", "n_iter", "precision", "n", "f", "pad"):
        assert got_hdr[k] == want_hdr[k], k
    assert np.array_equal(got > 0, want > 0)
    a, b = got.astype(np.float64), want.astype(np.float64)
    assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(b)
