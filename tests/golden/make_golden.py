"""Generate the golden vectors in tests/golden/ from the reference itself.

The reference's reconstruction sources (src/MutoSiddon.cpp, src/MutoPoCA.cpp,
src/MutoMLSD.cpp, src/MutoMAP.cpp, src/MutoPoCut.cpp, src/MutoSLR.cpp,
src/MutoSLRIter.cpp), its file code (src/MutoFile.cpp) and its command-line
program (MuToTest.cpp) are compiled in place by oracle/build_ref.sh and
called through oracle/reference.py; the inputs
(segments, synthetic tracks) are stored next to the outputs so the tests need
neither the reference nor the generator.  Run where the reference tree is
mounted:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import muontomography_gb300 as M  # noqa: E402
from muontomography_gb300 import workloads as W  # noqa: E402
from oracle import reference as R  # noqa: E402


def siddon_case():
    # the reference's Siddon probe geometry (test/SiddonTest.cpp:8-17): 100^3 voxels
    # of 2 mm at -100, segments uniform in [-500, 500]^3; keep the ones that hit
    g = M.Grid(100, 100, 100, -100.0, -100.0, -100.0, 2.0, 2.0, 2.0)
    rng = np.random.default_rng(2024)
    p1, p2 = rng.uniform(-500, 500, (6000, 3)), rng.uniform(-500, 500, (6000, 3))
    _, _, cnt = R.siddon(g, p1, p2, 512)
    sel = np.nonzero(cnt)[0][:400]
    # plus hand-made edge cases on a 10^3 grid of 10 mm scaled into this grid
    edge = np.array([[[0.0, 0.0, 90.0], [0.0, 0.0, -110.0]],        # along a voxel edge line
                     [[-100.0, -100.0, -100.0], [100.0, 100.0, 100.0]],  # main diagonal
                     [[100.0, 100.0, 100.0], [-100.0, -100.0, -100.0]],
                     [[-100.0, 0.0, 0.0], [100.0, 0.0, 0.0]],          # grazing the x axis plane
                     [[-50.0, 150.0, 7.0], [-50.0, -150.0, 7.0]],
                     [[13.0, 13.0, 13.0], [13.0, 13.0, 13.0]]])        # degenerate
    p1 = np.concatenate([p1[sel], edge[:, 0]])
    p2 = np.concatenate([p2[sel], edge[:, 1]])
    xyz, ln, cnt = R.siddon(g, p1, p2, 512)
    k = int(cnt.max())
    return {"grid": np.array([g.nx, g.ny, g.nz, g.x_min, g.y_min, g.z_min, g.dx, g.dy, g.dz]), "p1": p1, "p2": p2,
            "xyz": xyz[:, :k], "len": ln[:, :k], "count": cnt}


def track_case():
    wl = W.small(n_muons=2500, seed=4242, n=10)
    rays = wl.tracks()
    g = wl.grid
    out = {"grid": np.array([g.nx, g.ny, g.nz, g.x_min, g.y_min, g.z_min, g.dx, g.dy, g.dz]), "rays": rays}
    cases = {}
    for name, cfg in {"poca_lw": wl.poca_config(length_weighted=True),
                      "poca_dz": wl.poca_config(length_weighted=False),
                      "poca_straight": wl.poca_config(straight_line=True)}.items():
        img, _ = R.reconstruct("poca", cfg, rays, g.nvox)
        out[name] = img
        cases[name] = cfg
    # PoCut: cut percentiles 1, 0.9, 0.5 and 0, both weightings, with and without momentum
    for name, cfg in {"pocut_lw_100": wl.poca_config(length_weighted=True, cut_percentile=1.0),
                      "pocut_dz_90": wl.poca_config(length_weighted=False, cut_percentile=0.9),
                      "pocut_lw_50_energy": wl.poca_config(length_weighted=True, has_energy=True,
                                                           cut_percentile=0.5),
                      "pocut_dz_0": wl.poca_config(length_weighted=False, cut_percentile=0.0)}.items():
        img, _ = R.reconstruct("pocut", cfg, rays, g.nvox)
        out[name] = img
        cases[name] = cfg
    # SLR and SLRIter: both weightings, with momentum, 1 and 3 in-place passes
    for name, (method, cfg) in {"slr_lw": ("slr", wl.poca_config(length_weighted=True)),
                                "slr_eq": ("slr", wl.poca_config(length_weighted=False)),
                                "slr_lw_energy": ("slr", wl.poca_config(length_weighted=True, has_energy=True)),
                                "slr_iter_1": ("slr_iter", wl.poca_config(length_weighted=True, num_iteration=1)),
                                "slr_iter_3": ("slr_iter", wl.poca_config(length_weighted=False, has_energy=True,
                                                                          num_iteration=3))}.items():
        img, _ = R.reconstruct(method, cfg, rays, g.nvox)
        out[name] = img
        cases[name] = {"method": method, **cfg}
    cfg = wl.em_config()
    p = R.mlsd_paths(cfg, rays)
    for k, v in p.items():
        out["paths_" + k] = v
    cases["paths"] = cfg
    em = {"mlsd_median": ("mlsd", wl.em_config(num_iteration=6)),
          "mlsd_mean": ("mlsd", wl.em_config(num_iteration=6, update_with_mean=True)),
          "mlsd_pct90": ("mlsd", wl.em_config(num_iteration=6, update_with_mean=True, mean_percentile=90)),
          "mlsd_straight": ("mlsd", wl.em_config(num_iteration=4, straight_line=True)),
          "mlsd_noenergy": ("mlsd", wl.em_config(num_iteration=4, has_energy=False)),
          "map_p1_6": ("map", wl.em_config(num_iteration=4, beta=0.01, p=1.0, delta=0.1)),
          "map_p2_26": ("map", wl.em_config(num_iteration=4, beta=0.01, p=2.0, delta=0.1, all_neighbours=True)),
          "map_p1_26_obj": ("map", wl.em_config(num_iteration=3, beta=0.005, p=1.0, delta=0.2, all_neighbours=True,
                                                add_object_prior=True))}
    for name, (method, cfg) in em.items():
        img, _ = R.reconstruct(method, cfg, rays, g.nvox)
        out[name] = img
        cases[name] = {"method": method, **cfg}
    # PoCA-seeded EM through an initial image (initialize_method 0), as the example JSON files chain them
    seed_img = out["poca_lw"].astype(np.float32).astype(np.float64)
    R.set_initial_image(seed_img, g)
    cfg = wl.em_config(num_iteration=5, initialize_method=0, initial_image_file="poca.bin")
    img, _ = R.reconstruct("mlsd", cfg, rays, g.nvox)
    R.set_initial_image(None)
    out["mlsd_poca_seeded"] = img
    out["poca_seed_image"] = seed_img
    cases["mlsd_poca_seeded"] = {"method": "mlsd", **cfg}
    return out, cases


Z_LAYERS = [1500.0, 1000.0, 500.0, -500.0, -1000.0, -1500.0]  # input/example_mlsd.json:3-4


def image_bytes(path: Path) -> np.ndarray:
    """An image file the reference wrote, with the method field's bytes past
    its NUL zeroed: the reference copies 16 bytes out of a short std::string
    (src/MutoFile.cpp:99), so those bytes are whatever its buffer held."""
    b = bytearray(path.read_bytes())
    end = b.index(0, 2, 18) if 0 in b[2:18] else 18
    b[end:18] = bytes(18 - end)
    return np.frombuffer(bytes(b), np.uint8)


def file_case(tmp: Path):
    """MutoFile: the raw-hit reader on smeared records (float64 and float32
    files, one NaN record) and the image files it writes (both precisions)."""
    g = M.Grid(10, 10, 10, -500.0, -500.0, -500.0, 100.0, 100.0, 100.0)
    n = 400
    rays = M.generate(g, np.full(g.nvox, 1e-7), n, seed=21)
    rng = np.random.default_rng(21)
    rec = np.empty((n, 2 * len(Z_LAYERS) + 2))
    rec[:, 0], rec[:, -1] = rays[:, 0], rays[:, 1]
    for k, zk in enumerate(Z_LAYERS):
        p, d = (rays[:, 2:5], rays[:, 8:11]) if k < 3 else (rays[:, 5:8], rays[:, 11:14])
        t = (zk - p[:, 2]) / d[:, 2]
        rec[:, 1 + 2 * k] = p[:, 0] + t * d[:, 0] + rng.standard_normal(n)
        rec[:, 2 + 2 * k] = p[:, 1] + t * d[:, 1] + rng.standard_normal(n)
    rec[[7, 301], [4, 13]] = np.nan
    out = {"z_layers": np.asarray(Z_LAYERS), "n_middle": np.int64(3), "records64": rec,
           "records32": rec.astype(np.float32)}
    for prec, key in ((8, "records64"), (4, "records32")):
        f = tmp / f"hits{prec}.bin"
        out[key].tofile(f)
        out[f"tracks{prec}"] = R.read_muon_data(f, Z_LAYERS, 3, prec)
    ig = M.Grid(7, 5, 3, -350.5, -250.25, -150.125, 100.0, 80.0, 60.0)
    img = rng.random((7, 5, 3)) * 1e-6
    out["image"] = img
    out["image_grid"] = np.array([7, 5, 3, -350.5, -250.25, -150.125, 100.0, 80.0, 60.0])
    for prec in (8, 4):
        f = tmp / f"image{prec}.bin"
        R.save_image(f, img, ig, "mlsd", 123456, 50, prec)
        out[f"image_file{prec}"] = image_bytes(f)
    return out


CLI_METHODS = ("poca", "pocut", "slr", "slr_iter", "mlsd", "map")


def cli_case(tmp: Path):
    """The reference's command-line program (MuToTest.cpp) end to end on the
    1 m cube of 50 mm voxels: a float32 hit file, one config per method, PoCA
    written first and read back as the initial image of MLSD and MAP (as the
    example JSON files chain them).  Configs hold "{dir}" for the folder."""
    wl = W.cube20_50mm(n_muons=10_000, seed=31)
    rays = wl.tracks()
    rng = np.random.default_rng(31)
    rec = np.empty((rays.shape[0], 2 * len(Z_LAYERS) + 2))
    rec[:, 0], rec[:, -1] = rays[:, 0], rays[:, 1]
    for k, zk in enumerate(Z_LAYERS):
        p, d = (rays[:, 2:5], rays[:, 8:11]) if k < 3 else (rays[:, 5:8], rays[:, 11:14])
        t = (zk - p[:, 2]) / d[:, 2]
        rec[:, 1 + 2 * k] = p[:, 0] + t * d[:, 0] + 0.5 * rng.standard_normal(rays.shape[0])
        rec[:, 2 + 2 * k] = p[:, 1] + t * d[:, 1] + 0.5 * rng.standard_normal(rays.shape[0])
    rec = rec.astype(np.float32)
    (tmp / "hits.bin").write_bytes(rec.tobytes())
    g = wl.grid
    grid = {"nx": g.nx, "ny": g.ny, "nz": g.nz, "x_min": g.x_min, "y_min": g.y_min, "z_min": g.z_min,
            "dx": g.dx, "dy": g.dy, "dz": g.dz}
    common = {"grid": grid, "has_energy": False, "total_num_rays": 0, "eps": 1.0e-8, "log_results": False}
    em = dict(common, straight_line=False, update_with_mean=False, mean_percentile=98, early_stop=False,
              initial_image_file="{dir}/poca.bin", initialize_method=0, initialize_value=1.0e-7,
              error_xy=1.0, error_dz_outer=1000.0, error_dz_inner=1000.0)
    sections = {
        "poca": dict(common, straight_line=False, length_weighted=False),
        "pocut": dict(common, length_weighted=False, cut_percentile=0.9),
        "slr": dict(common, length_weighted=True),
        "slr_iter": dict(common, length_weighted=False, num_iteration=2),
        "mlsd": dict(em, num_iteration=5),
        "map": dict(em, num_iteration=3, beta=0.01, p=1.0, delta=0.1, all_neighbours=True, add_object_prior=False),
    }
    out = {"records": rec, "z_layers": np.asarray(Z_LAYERS), "n_middle": np.int64(3),
           "tracks": R.read_muon_data(tmp / "hits.bin", Z_LAYERS, 3, 4)}
    configs = {}
    for m in CLI_METHODS:
        cfg = {"data_files": ["{dir}/hits.bin"], "detector_height": Z_LAYERS, "detector_middle": 3,
               "output_file": "{dir}/" + m + ".bin", m: sections[m]}
        configs[m] = cfg
        text = json.dumps(cfg).replace("{dir}", str(tmp))
        (tmp / f"{m}.json").write_text(text)
        R.run_cli(tmp / f"{m}.json")
        out[f"out_{m}"] = image_bytes(tmp / f"{m}.bin")
    out["configs"] = np.frombuffer(json.dumps(configs, sort_keys=True).encode(), np.uint8)
    return out


def main() -> None:
    if not R.available():
        raise SystemExit("reference sources are not mounted here")
    R.build()
    np.savez_compressed(HERE / "siddon.npz", **siddon_case())
    tracks, cases = track_case()
    np.savez_compressed(HERE / "tracks.npz", **tracks)
    (HERE / "configs.json").write_text(json.dumps(cases, indent=1, sort_keys=True))
    with tempfile.TemporaryDirectory() as tmp:
        np.savez_compressed(HERE / "files.npz", **file_case(Path(tmp)))
    with tempfile.TemporaryDirectory() as tmp:
        np.savez_compressed(HERE / "cli.npz", **cli_case(Path(tmp)))
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")))


if __name__ == "__main__":
    main()
