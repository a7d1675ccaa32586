"""The mean update over muon-major lists only, and over paths walked again
every iteration, against the FP64 CPU oracle through the C ABI.

update_with_mean with mean_percentile 100 (src/MutoMLSD.cpp:497-499) needs no
voxel-major copy of the lists: lambda_j + lambda_j^2 G_j / (2 M_j) with
G_j = sum_i g_ij.  "muon_major" adds the g_ij to G_j by reductions to global
memory from one pass over the stored lists; "recompute" walks every path in
FP64 twice per iteration instead of storing it.  The summation order of the
reductions differs from the reference's per-voxel sums: lambda agrees within
1e-10 relative L2 in the fp64 form and 1e-4 in the mixed form.
"""
import numpy as np
import pytest

import muontomography_gb300 as M
from muontomography_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-4
LISTS = ["voxel_major", "muon_major", "recompute"]
TOL = {"fp64": FP64_TOL, "mixed": MIXED_TOL}


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _mean_cfg(wl, **over):
    return wl.em_config(update_with_mean=True, mean_percentile=100, **over)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("lists", LISTS)
@pytest.mark.parametrize("straight", [False, True])
def test_mean_update_matches_oracle(gpu, oracle, precision, lists, straight):
    wl = W.small(n_muons=8000, seed=41)
    rays = wl.tracks()
    n_iter = 6
    cfg = _mean_cfg(wl, precision=precision, num_iteration=n_iter, path_lists=lists, straight_line=straight,
                    compute_cost=True)
    init = np.full(wl.grid.nvox, 1e-7)
    ref = oracle.Mlsd(wl.grid, cfg, rays, init)
    ref.iterate(n_iter)
    with M.MutoMLSD(cfg) as rec:
        img = rec.reconstruct(rays)
        st = rec.status()
        mult = rec.multiplicity()
    assert st["path_lists"] == {"voxel_major": 1, "muon_major": 2, "recompute": 3}[lists]
    assert st["muon_pass"] in {"voxel_major": (2,), "muon_major": (3, 5, 6), "recompute": (4,)}[lists]
    assert st["iterations_done"] == n_iter
    assert st["n_pairs"] == ref.counts()["n_pairs"]
    assert st["n_bounds"] == 0 and st["n_path_overflow"] == 0
    assert rel_l2(img.reshape(-1, order="F"), ref.image()) < TOL[precision]
    # the mean cost of the last iteration (src/MutoMLSD.cpp:202)
    assert abs(st["cost"] - ref.costs()[-1]) <= (1e-10 if precision == "fp64" else 1e-5) * abs(ref.costs()[-1])
    assert np.array_equal(mult > 0, np.bincount(ref.export()["idx"], minlength=wl.grid.nvox) > 0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("variant", ["4x8", "8x4", "8x8", "8x16", "16x8", "16x16", "staged", "split", "split8",
                                     "split8_overlap"])
@pytest.mark.parametrize("n,n_muons", [(12, 6000), (200, 1500)])
def test_every_muon_major_variant_matches_oracle(gpu, oracle, precision, variant, n, n_muons):
    # every form of the stored-list pass, forced.  The 200^3 grid gives paths
    # of about 300 pairs: the register variants read their pairs past the held
    # ones again, and a staged batch of 32 such muons overflows the 8 192
    # (mixed) or 4 096 (fp64) pairs staged in shared memory
    wl = W.small(n_muons=n_muons, seed=47, n=n)
    rays = wl.tracks()
    n_iter = 3
    cfg = _mean_cfg(wl, precision=precision, num_iteration=n_iter, path_lists="muon_major", fused_variant=variant,
                    compute_cost=True)
    init = np.full(wl.grid.nvox, 1e-7)
    ref = oracle.Mlsd(wl.grid, cfg, rays, init)
    ref.iterate(n_iter)
    with M.MutoMLSD(cfg) as rec:
        img = rec.reconstruct(rays)
        st = rec.status()
    assert st["muon_pass"] == {"staged": 6, "split": 5, "split8": 5, "split8_overlap": 5}.get(variant, 3)
    if variant.startswith("split"):
        assert st["tile_pairs"] == (4 if variant == "split" else 8)
        assert st["tile_muons"] == (4 if variant == "split8_overlap" else 0)
    if n == 200:
        assert st["n_pairs"] / st["n_scat_in_grid"] > (8192 if precision == "mixed" else 4096) / 32
    assert rel_l2(img.reshape(-1, order="F"), ref.image()) < TOL[precision]
    assert abs(st["cost"] - ref.costs()[-1]) <= (1e-10 if precision == "fp64" else 1e-5) * abs(ref.costs()[-1])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_auto_lists_follow_the_update(gpu, precision):
    wl = W.small(n_muons=2000, seed=42)
    rays = wl.tracks()
    for mean, pct, want in [(True, 100, 2), (True, 90, 1), (False, 100, 1)]:
        cfg = wl.em_config(precision=precision, num_iteration=1, update_with_mean=mean, mean_percentile=pct)
        with M.MutoMLSD(cfg) as rec:
            rec.reconstruct(rays)
            assert rec.status()["path_lists"] == want


def test_lists_reject_the_median(gpu):
    wl = W.small(n_muons=100, seed=43)
    for lists in ("muon_major", "recompute"):
        with pytest.raises(M.MutoError):
            M.MutoMLSD(wl.em_config(path_lists=lists))
        with pytest.raises(M.MutoError):
            M.MutoMLSD(wl.em_config(path_lists=lists, update_with_mean=True, mean_percentile=50))
    with pytest.raises(M.MutoError):
        M.MutoMLSD(wl.em_config(path_lists="elsewhere"))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_muon_major_paths_bit_exact_in_chunks(gpu, oracle, precision):
    # the set-up walks the paths in chunks of muons; tiny chunks (about a
    # dozen muons each) give the same lists, offsets and lengths bit for bit
    wl = W.small(n_muons=6000, seed=31)
    rays = wl.tracks()
    cfg = _mean_cfg(wl, precision=precision)
    init = np.full(wl.grid.nvox, 1e-7)
    r = oracle.Mlsd(wl.grid, dict(cfg, precision="fp64"), rays, init).export()
    for chunk in (0, 400, 9999):
        with M.MutoMLSD(dict(cfg, setup_chunk_pairs=chunk)) as rec:
            rec.load_tracks(rays)
            rec.prepare()
            g = rec.export_paths()
            assert rec.status()["path_lists"] == 2
        assert np.array_equal(g["kept"], r["kept"])
        assert np.array_equal(g["off"], r["off"])
        assert np.array_equal(g["idx"], r["idx"])
        if precision == "fp64":
            assert np.array_equal(g["len"].view(np.uint64), r["len"].view(np.uint64))
            assert np.array_equal(g["tail"].view(np.uint64), r["tail"].view(np.uint64))
        else:
            assert np.array_equal(g["len"], r["len"].astype(np.float32).astype(np.float64))
            assert np.array_equal(g["tail"], r["tail"].astype(np.float32).astype(np.float64))


def test_chunked_voxel_major_set_up_is_unchanged(gpu, oracle):
    # the median path's set-up through the same chunked fill
    wl = W.small(n_muons=6000, seed=32)
    rays = wl.tracks()
    cfg = wl.em_config(precision="fp64", num_iteration=4)
    ref = oracle.Mlsd(wl.grid, cfg, rays, np.full(wl.grid.nvox, 1e-7))
    ref.iterate(4)
    with M.MutoMLSD(dict(cfg, setup_chunk_pairs=500)) as rec:
        img = rec.reconstruct(rays).reshape(-1, order="F")
        g = rec.export_paths()
    assert np.array_equal(g["idx"], ref.export()["idx"])
    assert rel_l2(img, ref.image()) < FP64_TOL


def test_recompute_stores_no_paths(gpu):
    wl = W.small(n_muons=500, seed=44)
    with M.MutoMLSD(_mean_cfg(wl, path_lists="recompute")) as rec:
        rec.load_tracks(wl.tracks())
        rec.prepare()
        st = rec.status()
        with pytest.raises(M.MutoError):
            rec.export_paths()
    assert st["n_pairs"] > 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("lists", ["muon_major", "recompute"])
def test_map_with_mean_ml_step_matches_oracle(gpu, oracle, precision, lists):
    # MAP (src/MutoMAP.cpp:129-198) whose ML step is the mean update
    wl = W.small(n_muons=8000, seed=61)
    rays = wl.tracks()
    n_iter = 4
    cfg = _mean_cfg(wl, precision=precision, num_iteration=n_iter, path_lists=lists)
    cfg.update(beta=0.01, p=1.0, all_neighbours=True, delta=0.1 * float(np.median(wl.lam())) * 1e7)
    init = np.full(wl.grid.nvox, 1e-7)
    ref = oracle.Mlsd(wl.grid, cfg, rays, init, method="map")
    ref.iterate(n_iter)
    with M.MutoMAP(cfg) as rec:
        img = rec.reconstruct(rays).reshape(-1, order="F")
        st = rec.status()
    assert st["n_nonconverged"] == 0
    assert rel_l2(img, ref.image()) < (1e-9 if precision == "fp64" else MIXED_TOL)


@pytest.mark.parametrize("lists", ["muon_major", "recompute"])
def test_gradient_from_lists_and_walks_matches_oracle(gpu, oracle, lists):
    # the backward pass from the stored lists, or from paths walked again
    # (the form for scans whose lists do not fit in memory)
    wl = W.small(n_muons=6000, seed=101)
    rays = wl.tracks()
    cfg = _mean_cfg(wl, precision="fp64", num_iteration=0, path_lists=lists)
    ref = oracle.Mlsd(wl.grid, cfg, rays, np.full(wl.grid.nvox, 1e-7))
    rng = np.random.default_rng(0)
    lam = wl.lam() * rng.uniform(0.5, 1.5, wl.grid.nvox) + 1e-9
    with M.MutoMLSD(cfg) as rec:
        rec.load_tracks(rays)
        rec.prepare()
        mult = rec.multiplicity()
        lam = np.where(mult > 0, lam, 0.0)
        x = np.log(np.where(mult > 0, lam, 1.0))
        v, g = rec.nll_grad(x)
        v2 = rec.nll(x)
        v3, g3 = rec.nll_grad(x)  # the per-voxel sums start from zero every call
    rv, rg = ref.nll(lam, grad=True)
    assert abs(v - rv) <= 1e-10 * abs(rv)
    assert abs(v2 - rv) <= 1e-10 * abs(rv)
    assert rel_l2(g, rg) < 1e-9
    assert rel_l2(g3, g) < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_recompute_equals_stored_lists(gpu, precision):
    wl = W.small(n_muons=20000, seed=45, n=16)
    rays = wl.tracks()
    out = {}
    for lists in ("muon_major", "recompute"):
        with M.MutoMLSD(_mean_cfg(wl, precision=precision, num_iteration=5, path_lists=lists)) as rec:
            out[lists] = rec.reconstruct(rays).reshape(-1, order="F")
    assert rel_l2(out["recompute"], out["muon_major"]) < (1e-12 if precision == "fp64" else 1e-5)


def test_batch_of_scans_with_muon_major_lists(gpu):
    wls = [W.small(n_muons=3000 + 1000 * k, seed=120 + k, n=8 + 2 * k) for k in range(3)]
    tracks = [w.tracks() for w in wls]
    cfg = dict(_mean_cfg(wls[0], precision="fp64", num_iteration=4), initialize_method=2)
    with M.Batch(cfg, [w.grid for w in wls]) as b:
        imgs = b.reconstruct_all(tracks)
        assert b.status()["path_lists"] == 2
    for k, w in enumerate(wls):
        with M.MutoMLSD(dict(cfg, grid=w.grid.json())) as rec:
            one = rec.reconstruct(tracks[k])
        assert rel_l2(imgs[k], one) < 1e-12, k


def test_graph_and_eager_agree_on_muon_major(gpu):
    wl = W.small(n_muons=5000, seed=46)
    rays = wl.tracks()
    out = []
    for graph in (True, False):
        with M.MutoMLSD(_mean_cfg(wl, precision="fp64", num_iteration=5, use_graph=graph)) as rec:
            out.append(rec.reconstruct(rays).reshape(-1, order="F"))
    assert rel_l2(out[0], out[1]) < 1e-12


@pytest.mark.parametrize("lists", ["muon_major", "recompute"])
def test_grid256_mean_mixed_against_fp64(gpu, lists):
    # the 256x256x128 grid of 10 mm voxels with 1 M of its muons
    wl = W.grid256x256x128_10mm(n_muons=1_000_000)
    rays = wl.tracks()
    out = {}
    for prec in ("fp64", "mixed"):
        with M.MutoMLSD(_mean_cfg(wl, precision=prec, num_iteration=5, path_lists=lists)) as rec:
            out[prec] = rec.reconstruct(rays).reshape(-1, order="F")
    assert rel_l2(out["mixed"], out["fp64"]) < MIXED_TOL
