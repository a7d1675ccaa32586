"""Known-answer tests of the FP64 CPU oracle (the reference's tests pin no
values, so these fix the geometry and algebra the oracle restates)."""
import numpy as np
import pytest

import muontomography_gb300 as M


def seg(oracle, grid, p1, p2, cap=256):
    xyz, ln, cnt = oracle.siddon_batch(grid, np.array([p1], float), np.array([p2], float), cap)
    k = int(cnt[0])
    return xyz[0, :k], ln[0, :k]


G10 = M.Grid(10, 10, 10, 0.0, 0.0, 0.0, 10.0, 10.0, 10.0)


def test_siddon_axis_aligned(oracle):
    xyz, ln = seg(oracle, G10, (5.0, 5.0, 120.0), (5.0, 5.0, -20.0))
    assert [tuple(v) for v in xyz] == [(0, 0, z) for z in range(9, -1, -1)]
    assert np.allclose(ln, 10.0, rtol=0, atol=1e-12)


def test_siddon_lengths_sum_to_clipped_segment(oracle):
    rng = np.random.default_rng(3)
    for _ in range(200):
        p1, p2 = rng.uniform(-30, 130, 3), rng.uniform(-30, 130, 3)
        xyz, ln = seg(oracle, G10, p1, p2)
        # clipped length by dense sampling of the segment inside the box
        t = np.linspace(0, 1, 200001)
        pts = p1[None] + t[:, None] * (p2 - p1)[None]
        inside = np.all((pts >= 0) & (pts <= 100), axis=1)
        clip = inside.mean() * np.linalg.norm(p2 - p1)
        assert abs(ln.sum() - clip) < 2e-3 * max(np.linalg.norm(p2 - p1), 1)
        assert np.all((xyz < 10).all(axis=1))


def test_siddon_diagonal_through_corners(oracle):
    xyz, ln = seg(oracle, G10, (0.0, 0.0, 0.0), (100.0, 100.0, 100.0))
    assert len(xyz) == 10
    assert [tuple(v) for v in xyz] == [(i, i, i) for i in range(10)]
    assert np.allclose(ln, 10.0 * np.sqrt(3.0))


def test_siddon_parallel_outside_and_degenerate(oracle):
    assert len(seg(oracle, G10, (-5.0, 5.0, 5.0), (-5.0, 95.0, 95.0))[0]) == 0
    assert len(seg(oracle, G10, (50.0, 50.0, 150.0), (50.0, 50.0, 120.0))[0]) == 0
    # a point inside: all axes parallel, one voxel of zero length is not recorded
    assert len(seg(oracle, G10, (55.0, 55.0, 55.0), (55.0, 55.0, 55.0))[0]) == 1


def ray_through(q, din, dout, z_top, z_bot, e=3.0):
    """A track whose in and out lines meet at q."""
    din = np.asarray(din, float) / np.linalg.norm(din)
    dout = np.asarray(dout, float) / np.linalg.norm(dout)
    pin = q + (z_top - q[2]) / din[2] * din
    pout = q + (z_bot - q[2]) / dout[2] * dout
    return np.concatenate([[e, e], pin, pout, din, dout])


def test_poca_intersecting_lines_bins_the_crossing(oracle):
    g = M.Grid(10, 10, 10, -50.0, -50.0, -50.0, 10.0, 10.0, 10.0)
    q = np.array([12.5, -7.5, 3.0])
    r = ray_through(q, (0.1, 0.05, 1.0), (-0.05, 0.12, 1.0), 50.0, -50.0)
    rays = np.stack([r, r])
    img, assign, cnt = oracle.poca(g, {"length_weighted": True}, rays)
    assert assign[0].tolist() == [6, 4, 5]
    theta2 = ((np.arctan2(r[8], r[10]) - np.arctan2(r[11], r[13])) ** 2 +
              (np.arctan2(r[9], r[10]) - np.arctan2(r[12], r[13])) ** 2) / 2
    j = 6 + 10 * (4 + 10 * 5)
    assert cnt.tolist() == [2, 2, 2]
    # two identical tracks: the voxel holds 2 theta^2 over the summed path length through it
    assert img[j] > 0 and np.count_nonzero(img) == 1
    assert theta2 > 0


def test_poca_parallel_lines_use_the_midpoint(oracle):
    g = M.Grid(10, 10, 10, -50.0, -50.0, -50.0, 10.0, 10.0, 10.0)
    d = np.array([0.0, 0.0, 1.0])
    r = np.concatenate([[3.0, 3.0], [11.0, 21.0, 50.0], [13.0, 23.0, -50.0], d, d])
    img, assign, cnt = oracle.poca(g, {}, r[None])
    assert cnt[1] == 0                      # not counted as non-parallel
    assert assign[0].tolist() == [6, 7, 5]  # midpoint (12, 22, 0)


def test_poca_negative_cast_uses_x86_semantics(oracle):
    # a PoCA point in (-1, 0) voxel units casts to 0 (kept), below -1 wraps (rejected)
    g = M.Grid(10, 10, 10, 0.0, 0.0, -50.0, 10.0, 10.0, 10.0)
    d = np.array([0.0, 0.0, 1.0])
    near = np.concatenate([[3.0, 3.0], [-5.0, 5.0, 50.0], [-5.0, 5.0, -50.0], d, d])
    far = np.concatenate([[3.0, 3.0], [-15.0, 5.0, 50.0], [-15.0, 5.0, -50.0], d, d])
    _, assign, _ = oracle.poca(g, {}, np.stack([near, far]))
    assert assign[0].tolist() == [0, 0, 5]
    assert assign[1].tolist() == [-1, -1, -1]


@pytest.mark.parametrize("coef,roots", [
    ((1, -6, 11, -6), [1, 2, 3]),
    ((2, -3, -11, 6), [-2, 0.5, 3]),
    ((1, -2, 1, 0), [0, 1, 1]),
])
def test_cubic_known_roots(oracle, coef, roots):
    n, r = oracle.cubic(*coef)
    assert n == 3
    assert np.allclose(sorted(r), roots, atol=1e-6)


def test_cubic_single_real_root(oracle):
    n, r = oracle.cubic(1.0, 0.0, 1.0, -2.0)  # x^3 + x - 2 = (x - 1)(x^2 + x + 2)
    assert n == 1 and abs(r[0] - 1.0) < 1e-9


def _small(oracle, cfg_over=None, n=1500, seed=3):
    from muontomography_gb300 import workloads as W

    wl = W.small(n_muons=n, seed=seed, n=8)
    rays = wl.tracks()
    cfg = wl.em_config(**(cfg_over or {}))
    return wl, rays, cfg


def test_em_mean_step_is_a_scaled_gradient_step(oracle):
    """Mean-mode EM: l_new - l = l^2 G / (2 M) with G = -dNLL/dl (the adjoint's gradient)."""
    wl, rays, cfg = _small(oracle, {"update_with_mean": True})
    rng = np.random.default_rng(1)
    lam = wl.lam() * rng.uniform(0.7, 1.3, wl.grid.nvox)
    ref = oracle.Mlsd(wl.grid, cfg, rays, lam)
    _, new, mult = ref.ml_step()
    _, grad_log = ref.nll(lam, grad=True)  # d NLL / d log l = l * dNLL/dl
    m = mult > 0
    lhs = (new[m] - lam[m]) * 2 * mult[m] / lam[m] ** 2
    rhs = -grad_log[m] / lam[m]
    assert np.allclose(lhs, rhs, rtol=1e-7, atol=1e-9 * np.abs(rhs).max())


def test_nll_gradient_central_differences(oracle):
    wl, rays, cfg = _small(oracle)
    rng = np.random.default_rng(2)
    lam = wl.lam() * rng.uniform(0.7, 1.3, wl.grid.nvox) + 1e-9
    ref = oracle.Mlsd(wl.grid, cfg, rays, lam)
    _, g = ref.nll(lam, grad=True)
    eps = 1e-4
    for j in rng.choice(np.nonzero(g)[0], 12, replace=False):
        lp, lm = lam.copy(), lam.copy()
        lp[j] *= np.exp(eps)
        lm[j] *= np.exp(-eps)
        fd = (ref.nll(lp) - ref.nll(lm)) / (2 * eps)
        assert abs(fd - g[j]) <= 1e-5 * abs(g[j]) + 1e-7


def test_median_update_even_and_odd(oracle):
    """At a fixed point of constant lambda the EM output stays positive and finite."""
    wl, rays, cfg = _small(oracle)
    ref = oracle.Mlsd(wl.grid, cfg, rays, np.full(wl.grid.nvox, 1e-7))
    ref.iterate(3)
    img = ref.image()
    c = ref.counts()
    assert np.all(np.isfinite(img)) and img.max() > 0
    assert c["iterations_done"] == 3 and c["n_singular"] == 0


@pytest.mark.parametrize("lw", [False, True])
@pytest.mark.parametrize("iters", [1, 3])
def test_slr_iter_level_schedule_is_exact(oracle, lw, iters):
    # SLRIter's passes are order-dependent (src/MutoSLRIter.cpp:45-67); run
    # level by level (muons of a level share no voxel, every voxel sees its
    # muons in index order, the latest index first inside a level) they give
    # the same image bit for bit: the schedule a parallel form can use
    g = M.Grid(12, 12, 12, -300.0, -300.0, -300.0, 50.0, 50.0, 50.0)
    rays = M.generate(g, np.full(g.nvox, 2e-6), 3000, seed=12)
    cfg = {"length_weighted": lw, "has_energy": True, "num_iteration": iters}
    want = oracle.slr(g, cfg, rays, iterative=True)
    got = oracle.slr_by_level(g, cfg, rays, iterative=True)
    assert np.count_nonzero(want) > 1000
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    # a schedule that breaks a voxel's order does change the result
    perm = np.random.default_rng(0).permutation(rays.shape[0])
    assert not np.array_equal(oracle.slr(g, cfg, rays[perm], iterative=True).view(np.uint64), want.view(np.uint64))


def test_oracle_synthetic_tracks_equal_the_library_generator(oracle):
    # the CPU-baseline legs make their tracks without the product library;
    # they must be the workload's own tracks, bit for bit
    import muontomography_gb300 as M
    from muontomography_gb300 import workloads as W
    from oracle import synthetic as S

    for wl in (W.small(n_muons=2000, seed=5), W.grid256x256x128_10mm(n_muons=1500)):
        lam = S.phantom(wl.grid, wl.blocks, M.X0_MM["air"], 3.0)
        assert np.array_equal(lam, wl.lam())
        a = S.generate(wl.grid, lam, wl.n_muons, wl.seed, first=11)
        b = M.generate(wl.grid, wl.lam(), wl.n_muons, wl.seed, first=11)
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
