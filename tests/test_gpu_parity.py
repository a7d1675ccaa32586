"""GPU parity against the FP64 CPU oracle, through the C ABI.

Bit-exact: Siddon voxel lists (indices and FP64 lengths), PoCA voxel of every
ray, MLSD kept muons, merged path voxel indices and lengths.
Tolerances: lambda after the same iteration count within 1e-10 relative L2
(fp64 form; summation order of atomics / per-muon sums differs) and 1e-4
(mixed form: FP32 lists and accumulation).
"""
import numpy as np
import pytest

import muontomography_gb300 as M
from muontomography_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-4


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def random_segments(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, size=(n, 3)), rng.uniform(lo, hi, size=(n, 3))


# ---------------------------------------------------------------------------
# Siddon
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("seed", [0, 1])
def test_siddon_random_segments_bit_exact(gpu, oracle, seed):
    # the reference's own Siddon probe geometry: 100^3 voxels of 2 mm at -100,
    # segments uniform in [-500, 500]^3 (test/SiddonTest.cpp:8-17)
    grid = M.Grid(100, 100, 100, -100.0, -100.0, -100.0, 2.0, 2.0, 2.0)
    p1, p2 = random_segments(20000, -500.0, 500.0, seed)
    cap = 512
    gx, gl, gc = M.siddon_batch(grid, p1, p2, cap)
    ox, ol, oc = oracle.siddon_batch(grid, p1, p2, cap)
    assert np.array_equal(gc, oc)
    assert (oc > 0).sum() > 1000
    for r in np.nonzero(oc)[0]:
        k = oc[r]
        assert np.array_equal(gx[r, :k], ox[r, :k]), r
        assert np.array_equal(gl[r, :k].view(np.uint64), ol[r, :k].view(np.uint64)), r


def test_siddon_edge_cases_bit_exact(gpu, oracle):
    grid = M.Grid(10, 10, 10, 0.0, 0.0, 0.0, 10.0, 10.0, 10.0)
    segs = [
        ((5.0, 5.0, 120.0), (5.0, 5.0, -20.0)),      # axis aligned, through centres
        ((0.0, 0.0, 100.0), (100.0, 100.0, 0.0)),    # exact diagonal through corners
        ((10.0, 10.0, 100.0), (10.0, 10.0, 0.0)),    # along a voxel edge
        ((0.0, 50.0, 50.0), (100.0, 50.0, 50.0)),    # grazing a face
        ((-5.0, 5.0, 5.0), (-5.0, 95.0, 95.0)),      # parallel to x outside: empty
        ((50.0, 50.0, 50.0), (50.0, 50.0, 50.0)),    # degenerate point
        ((100.0, 100.0, 100.0), (0.0, 0.0, 0.0)),    # reversed diagonal
        ((33.3, 66.6, 99.9), (33.3000001, 66.6, 0.1)),
        ((50.0, 50.0, 150.0), (51.0, 49.0, 40.0)),   # ends inside
        ((-50.0, -50.0, -50.0), (150.0, 150.0, 150.0)),
    ]
    p1 = np.array([s[0] for s in segs])
    p2 = np.array([s[1] for s in segs])
    gx, gl, gc = M.siddon_batch(grid, p1, p2, 64)
    ox, ol, oc = oracle.siddon_batch(grid, p1, p2, 64)
    assert np.array_equal(gc, oc)
    assert np.array_equal(gx, ox)
    assert np.array_equal(gl.view(np.uint64), ol.view(np.uint64))


# ---------------------------------------------------------------------------
# PoCA
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("length_weighted,straight", [(True, False), (False, False), (True, True)])
def test_poca_assignment_bit_exact(gpu, oracle, length_weighted, straight):
    wl = W.small(n_muons=20000, seed=21)
    rays = wl.tracks()
    cfg = wl.poca_config(length_weighted=length_weighted, straight_line=straight)
    ref_img, ref_assign, ref_cnt = oracle.poca(wl.grid, cfg, rays)
    with M.MutoPoCA(cfg) as rec:
        img = rec.reconstruct(rays)
        assign = rec.poca_assignment(rays.shape[0])
        st = rec.status()
    assert np.array_equal(assign, ref_assign)
    assert st["n_scat_in_grid"] == ref_cnt[2]
    assert st["n_not_parallel"] == ref_cnt[1]
    flat = img.reshape(-1, order="F")
    assert rel_l2(flat, ref_img) < 1e-12


# ---------------------------------------------------------------------------
# MLSD
# ---------------------------------------------------------------------------
def _mlsd_pair(oracle, wl, rays, cfg, init, n_iter, method="mlsd"):
    ref = oracle.Mlsd(wl.grid, cfg, rays, init, method=method)
    ref.iterate(n_iter)
    return ref


@pytest.mark.parametrize("n,n_muons,seed", [(12, 6000, 71), (4, 30000, 72), (2, 120000, 73)])
@pytest.mark.parametrize("cut,lw,energy", [(1.0, True, False), (0.9, False, False), (0.37, True, True),
                                           (0.0, False, False)])
def test_pocut_matches_oracle(gpu, oracle, n, n_muons, seed, cut, lw, energy):
    # src/MutoPoCut.cpp:19-121: 12^3 voxels hold a few values each (warp sorts); 4^3 voxels
    # hundreds to thousands (block sorts in shared memory); 2^3 voxels more than 4096
    # (block sorts in scratch).  The values are summed in the reference's order, so only
    # the FP64 weight atomics differ: 1e-12 relative.
    wl = W.small(n_muons=n_muons, seed=seed, n=n)
    rays = wl.tracks()
    cfg = wl.poca_config(length_weighted=lw, has_energy=energy, cut_percentile=cut, straight_line=True)
    ref, ref_assign, ref_ctr = oracle.pocut(wl.grid, cfg, rays)  # straight_line is ignored by PoCut
    with M.MutoPoCut(cfg) as rec:
        img = rec.reconstruct(rays).reshape(-1, order="F")
        st = rec.status()
        assign = rec.poca_assignment(rays.shape[0])
    assert np.array_equal(assign, ref_assign)
    assert st["n_scat_in_grid"] == int(ref_ctr[2])
    if n == 2 and cut == 1.0:
        assert np.bincount(np.ravel_multi_index(assign[assign[:, 0] >= 0].T, (2, 2, 2), order="F")).max() > 4096
    if np.any(ref):
        assert rel_l2(img, ref) < 1e-12
    assert np.array_equal(img > 0, ref > 0)
    assert np.all(img[ref == 0] == 0)


@pytest.mark.parametrize("n,n_muons,seed", [(12, 5000, 81), (30, 20000, 82)])
@pytest.mark.parametrize("lw,energy,iters", [(True, False, 0), (False, False, 0), (True, True, 0), (True, False, 1),
                                             (False, True, 3), (True, False, 0.5)])
def test_slr_matches_oracle(gpu, oracle, n, n_muons, seed, lw, energy, iters):
    # src/MutoSLR.cpp:47-103 (iters 0) and src/MutoSLRIter.cpp:15-83 (iters passes; 0.5
    # stands for SLRIter with num_iteration 0: an empty image).  Voxel walks are bit-exact;
    # atan2 and the first pass's FP64 atomics leave rounding differences.
    wl = W.small(n_muons=n_muons, seed=seed, n=n)
    rays = wl.tracks()
    cfg = wl.poca_config(length_weighted=lw, has_energy=energy)
    if iters:
        cfg["num_iteration"] = int(iters)
        ref = oracle.slr(wl.grid, cfg, rays, iterative=True)
        rec = M.MutoSLRIter(cfg)
    else:
        ref = oracle.slr(wl.grid, cfg, rays)
        rec = M.MutoSLR(cfg)
    with rec:
        img = rec.reconstruct(rays).reshape(-1, order="F")
    if not np.any(ref):
        assert not np.any(img)
        return
    assert rel_l2(img, ref) < 1e-12
    assert np.array_equal(img > 0, ref > 0)


@pytest.mark.parametrize("n,n_muons,seed", [(12, 5000, 83), (30, 20000, 84), (2, 3000, 85)])
@pytest.mark.parametrize("lw,energy,iters", [(True, False, 2), (False, True, 3)])
def test_slr_iter_levels_equal_sequential_passes(gpu, oracle, n, n_muons, seed, lw, energy, iters):
    # src/MutoSLRIter.cpp:40-71: the later passes in place, each muon on the
    # image the earlier muons left.  Run level by level (muons of one level
    # share no voxel) they give the sequential loop's image; the 2-voxel grid
    # puts most muons on a voxel they share (a level each).  The first pass's
    # FP64 atomics sum in a different order from run to run, so the two
    # schedules (and the oracle) agree to rounding, not bit for bit; the
    # schedule itself is exact on the CPU (test_oracle_kat).
    wl = W.small(n_muons=n_muons, seed=seed, n=n)
    rays = wl.tracks()
    cfg = wl.poca_config(length_weighted=lw, has_energy=energy)
    cfg["num_iteration"] = iters
    ref = oracle.slr(wl.grid, cfg, rays, iterative=True)
    out = {}
    for sch in ("levels", "sequential"):
        with M.MutoSLRIter(dict(cfg, slr_iter_schedule=sch)) as rec:
            out[sch] = rec.reconstruct(rays)
            out[sch + "_levels"] = rec.status()["slr_levels"]
    assert np.any(out["levels"])
    assert rel_l2(out["levels"], out["sequential"]) < 1e-12
    assert rel_l2(out["levels"].reshape(-1, order="F"), ref) < 1e-12
    assert np.array_equal(out["levels"] > 0, out["sequential"] > 0)
    assert out["sequential_levels"] == 0
    assert 1 <= out["levels_levels"] <= n_muons
    if n == 2:
        assert out["levels_levels"] > 10


@pytest.mark.parametrize("straight", [False, True])
def test_mlsd_paths_bit_exact(gpu, oracle, straight):
    wl = W.small(n_muons=6000, seed=31)
    rays = wl.tracks()
    cfg = wl.em_config(precision="fp64", straight_line=straight)
    init = np.full(wl.grid.nvox, 1e-7)
    ref = oracle.Mlsd(wl.grid, cfg, rays, init)
    r = ref.export()
    with M.MutoMLSD(cfg) as rec:
        rec.load_tracks(rays)
        rec.prepare()
        g = rec.export_paths()
    assert np.array_equal(g["kept"], r["kept"])
    assert np.array_equal(g["off"], r["off"])
    assert np.array_equal(g["idx"], r["idx"])
    assert np.array_equal(g["len"].view(np.uint64), r["len"].view(np.uint64))
    assert np.array_equal(g["tail"].view(np.uint64), r["tail"].view(np.uint64))
    np.testing.assert_allclose(g["info"][:, :5], r["info"][:, :5], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
@pytest.mark.parametrize("mode", ["median", "mean", "percentile"])
def test_mlsd_lambda_matches_oracle(gpu, oracle, precision, tol, mode):
    wl = W.small(n_muons=8000, seed=41)
    rays = wl.tracks()
    over = {"median": {}, "mean": {"update_with_mean": True},
            "percentile": {"update_with_mean": True, "mean_percentile": 90}}[mode]
    n_iter = 6
    cfg = wl.em_config(precision=precision, num_iteration=n_iter, **over)
    init = np.full(wl.grid.nvox, 1e-7)
    ref = _mlsd_pair(oracle, wl, rays, cfg, init, n_iter)
    with M.MutoMLSD(cfg) as rec:
        img = rec.reconstruct(rays)
        st = rec.status()
    assert st["iterations_done"] == n_iter
    assert rel_l2(img.reshape(-1, order="F"), ref.image()) < tol


def test_mlsd_cost_and_early_stop(gpu, oracle):
    wl = W.small(n_muons=5000, seed=51)
    rays = wl.tracks()
    cfg = wl.em_config(precision="fp64", num_iteration=8, early_stop=True)
    init = np.full(wl.grid.nvox, 1e-7)
    ref = _mlsd_pair(oracle, wl, rays, cfg, init, 8)
    with M.MutoMLSD(cfg) as rec:
        img = rec.reconstruct(rays)
        st = rec.status()
    rc = ref.counts()
    assert st["iterations_done"] == rc["iterations_done"]
    assert abs(st["cost"] - ref.costs()[-1]) <= 1e-9 * abs(ref.costs()[-1])
    assert rel_l2(img.reshape(-1, order="F"), ref.image()) < FP64_TOL


def test_mlsd_initial_image_grid_adoption(gpu, oracle):
    # an initial image whose nx/ny/nz differ from the config replaces the grid
    wl = W.small(n_muons=3000, seed=61, n=10)
    rays = wl.tracks()
    cfg = wl.em_config(precision="fp64", num_iteration=3, initialize_method=0)
    cfg["grid"] = dict(cfg["grid"], nx=7, ny=7, nz=7)
    init = np.full(wl.grid.nvox, 2e-7)
    ref = _mlsd_pair(oracle, wl, rays, wl.em_config(precision="fp64"), init, 3)
    with M.MutoMLSD(cfg) as rec:
        rec.set_initial_image(init, wl.grid)
        img = rec.reconstruct(rays)
        assert rec.get_current_grid() == wl.grid
    assert rel_l2(img.reshape(-1, order="F"), ref.image()) < FP64_TOL


def test_mlsd_total_num_rays_and_no_energy(gpu, oracle):
    wl = W.small(n_muons=5000, seed=71)
    rays = wl.tracks()
    cfg = wl.em_config(precision="fp64", num_iteration=4, total_num_rays=2500, has_energy=False)
    init = np.full(wl.grid.nvox, 1e-7)
    ref = _mlsd_pair(oracle, wl, rays, cfg, init, 4)
    with M.MutoMLSD(cfg) as rec:
        img = rec.reconstruct(rays)
        st = rec.status()
    assert st["n_scat_in_grid"] == ref.counts()["n_scat_in_grid"]
    assert rel_l2(img.reshape(-1, order="F"), ref.image()) < FP64_TOL


def test_graph_and_eager_agree(gpu):
    wl = W.small(n_muons=5000, seed=81)
    rays = wl.tracks()
    out = []
    for g in (True, False):
        cfg = wl.em_config(precision="fp64", num_iteration=5, use_graph=g, update_with_mean=True)
        with M.MutoMLSD(cfg) as rec:
            out.append(rec.reconstruct(rays))
    assert rel_l2(out[0], out[1]) < 1e-12


# ---------------------------------------------------------------------------
# MAP
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("p,all_nb,obj", [(1.0, False, False), (2.0, True, False), (1.0, True, True)])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", MIXED_TOL)])
def test_map_matches_oracle(gpu, oracle, p, all_nb, obj, precision, tol):
    wl = W.small(n_muons=6000, seed=91)
    rays = wl.tracks()
    cfg = wl.em_config(precision=precision, num_iteration=4, beta=0.01, p=p, delta=0.1, all_neighbours=all_nb,
                       add_object_prior=obj)
    init = np.full(wl.grid.nvox, 1e-7)
    ref = _mlsd_pair(oracle, wl, rays, cfg, init, 4, method="map")
    with M.MutoMAP(cfg) as rec:
        img = rec.reconstruct(rays)
        st = rec.status()
    assert st["n_nonconverged"] == 0
    assert rel_l2(img.reshape(-1, order="F"), ref.image()) < tol


# ---------------------------------------------------------------------------
# Adjoint
# ---------------------------------------------------------------------------
def test_nll_and_gradient_match_oracle(gpu, oracle):
    wl = W.small(n_muons=6000, seed=101)
    rays = wl.tracks()
    cfg = wl.em_config(precision="fp64", num_iteration=0)
    init = np.full(wl.grid.nvox, 1e-7)
    ref = oracle.Mlsd(wl.grid, cfg, rays, init)
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
    rv, rg = ref.nll(lam, grad=True)
    assert abs(v - rv) <= 1e-10 * abs(rv)
    assert abs(v2 - rv) <= 1e-10 * abs(rv)
    assert rel_l2(g, rg) < 1e-9


# ---------------------------------------------------------------------------
# Long voxel segments and the muon-pass variants
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
@pytest.mark.parametrize("mode", ["median", "percentile", "mean"])
def test_long_segments_match_oracle(gpu, oracle, precision, tol, mode):
    # 4^3 voxels and 30k muons: thousands of pairs per voxel, beyond the register budget
    wl = W.small(n_muons=30000, seed=111, n=4)
    rays = wl.tracks()
    over = {"median": {}, "mean": {"update_with_mean": True},
            "percentile": {"update_with_mean": True, "mean_percentile": 80}}[mode]
    cfg = wl.em_config(precision=precision, num_iteration=3, **over)
    ref = oracle.Mlsd(wl.grid, cfg, rays, np.full(wl.grid.nvox, 1e-7))
    ref.iterate(3)
    with M.MutoMLSD(cfg) as rec:
        rec.load_tracks(rays)
        rec.prepare()
        assert rec.multiplicity().max() > 1600
        rec.iterate(3)
        img = rec.image()
    assert rel_l2(img.reshape(-1, order="F"), ref.image()) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("method", ["mlsd", "map"])
def test_muon_layouts_agree(gpu, oracle, precision, method):
    # the per-muon coefficient table in muon order or in column order of the PoCA
    # points (chosen automatically for large tables, forced here): the keys are the
    # same, so the medians are identical; both match the oracle
    wl = W.small(n_muons=8000, seed=171, n=12)
    rays = wl.tracks()
    extra = {"beta": 0.01, "p": 1.0, "delta": 0.1, "all_neighbours": True} if method == "map" else {}
    out = []
    for layout in ("index", "columns"):
        cfg = wl.em_config(precision=precision, num_iteration=4, muon_layout=layout, **extra)
        rec = M.MutoMAP(cfg) if method == "map" else M.MutoMLSD(cfg)
        with rec:
            out.append(rec.reconstruct(rays))
    assert np.array_equal(out[0].view(np.uint64), out[1].view(np.uint64))
    ref = _mlsd_pair(oracle, wl, rays, wl.em_config(precision=precision, num_iteration=4, **extra),
                     np.full(wl.grid.nvox, 1e-7), 4, method=method)
    tol = FP64_TOL if precision == "fp64" else MIXED_TOL
    assert rel_l2(out[1].reshape(-1, order="F"), ref.image()) < (1e-9 if method == "map" and precision == "fp64" else tol)


@pytest.mark.parametrize("variant", ["tile", "warp"])
def test_muon_pass_variants_agree(gpu, oracle, variant):
    wl = W.small(n_muons=8000, seed=121)
    rays = wl.tracks()
    cfg = wl.em_config(precision="fp64", num_iteration=4, muon_pass=variant)
    ref = _mlsd_pair(oracle, wl, rays, cfg, np.full(wl.grid.nvox, 1e-7), 4)
    with M.MutoMLSD(cfg) as rec:
        img = rec.reconstruct(rays)
        st = rec.status()
    assert st["muon_pass"] == {"tile": 1, "warp": 2}[variant]
    assert rel_l2(img.reshape(-1, order="F"), ref.image()) < FP64_TOL


def test_autotuner_reports_its_choice(gpu):
    wl = W.small(n_muons=8000, seed=131)
    with M.MutoMLSD(wl.em_config()) as rec:
        rec.load_tracks(wl.tracks())
        rec.prepare()
        st = rec.status()
    assert st["muon_pass"] in (1, 2) and st["muon_group"] in (8, 16, 32)


# ---------------------------------------------------------------------------
# Batches of independent scans
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("precision,mode", [("fp64", "median"), ("mixed", "mean"), ("mixed", "median")])
def test_batch_equals_separate_scans(gpu, precision, mode):
    wls = [W.small(n_muons=4000, seed=200 + k, n=n) for k, n in enumerate((6, 9, 12))]
    over = {"median": {}, "mean": {"update_with_mean": True}}[mode]
    cfg = wls[0].em_config(precision=precision, num_iteration=4, **over)
    cfg.pop("grid")
    tracks = [wl.tracks() for wl in wls]
    with M.Batch(cfg, [wl.grid for wl in wls]) as b:
        imgs = b.reconstruct_all(tracks)
        st = b.status()
        info = [b.scan_info(k) for k in range(3)]
    assert st["iterations_done"] == 4
    for wl, trk, img, (kept, pairs) in zip(wls, tracks, imgs, info):
        with M.MutoMLSD(dict(cfg, grid=wl.grid.json())) as rec:
            one = rec.reconstruct(trk)
            s1 = rec.status()
        assert kept == s1["n_scat_in_grid"] and pairs == s1["n_pairs"]
        tol = 1e-12 if precision == "fp64" else 1e-6
        assert rel_l2(img, one) < tol


def test_batch_rejects_what_it_cannot_do(gpu):
    g = [W.small(n=6).grid]
    with pytest.raises(M.MutoError):
        M.Batch({"initialize_method": 0}, g)
    with pytest.raises(M.MutoError):
        M.Batch({"initialize_method": 2, "early_stop": True}, g)
