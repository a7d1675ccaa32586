"""The adjoint of the reconstruction objective on the GPU, through the C ABI.

F(log lambda) is the MLSD negative log-likelihood (the reference's per-muon
cost, src/MutoMLSD.cpp:465-468) plus, for MAP, the prior whose separable
surrogate the reference's MAP step minimises (src/MutoMAP.cpp:207-350).

* central differences: dF/dlog(lambda_j) from muto_nll_backward against
  (F(x + eps e_j) - F(x - eps e_j)) / (2 eps), eps = 1e-4, on 64 voxels of a
  MAP problem with the 26-neighbour prior and the object prior (fp64 form);
* the EM fixed point: one mean-mode EM step equals a scaled gradient step,
  lambda' - lambda = -lambda * grad / (2 M_j), so its fixed points are the
  stationary points of the likelihood;
* the gradient solver lowers F and leaves the image it reports F of.
"""
import numpy as np
import pytest

import muontomography_gb300 as M
from muontomography_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _start(wl, mult, seed):
    rng = np.random.default_rng(seed)
    lam = wl.lam() * rng.uniform(0.6, 1.4, wl.grid.nvox) + 2e-7
    return np.where(mult > 0, np.log(lam), 0.0)


@pytest.mark.parametrize("p,all_nb,obj", [(1.5, True, True), (2.0, False, False)])
def test_gradient_central_differences(gpu, p, all_nb, obj):
    wl = W.small(n_muons=6000, seed=141, n=8)
    cfg = wl.em_config(precision="fp64", num_iteration=0, beta=0.01, p=p, delta=0.1, all_neighbours=all_nb,
                       add_object_prior=obj)
    eps = 1e-4
    with M.MutoMAP(cfg) as rec:
        rec.load_tracks(wl.tracks())
        rec.prepare()
        mult = rec.multiplicity()
        x = _start(wl, mult, 3)
        f0, g = rec.nll_grad(x)
        assert np.isfinite(f0) and np.all(np.isfinite(g))
        rng = np.random.default_rng(5)
        pick = rng.choice(np.nonzero(mult > 0)[0], size=64, replace=False)
        fd = np.empty(pick.size)
        for k, j in enumerate(pick):
            xp, xm = x.copy(), x.copy()
            xp[j] += eps
            xm[j] -= eps
            fd[k] = (rec.nll(xp) - rec.nll(xm)) / (2 * eps)
    assert rel_l2(fd, g[pick]) < 1e-5
    scale = np.abs(g[pick]).max()
    assert np.all(np.abs(fd - g[pick]) <= 1e-5 * np.abs(g[pick]) + 1e-7 * scale)


def test_mean_em_step_is_a_scaled_gradient_step(gpu):
    wl = W.small(n_muons=6000, seed=151, n=8)
    cfg = wl.em_config(precision="fp64", num_iteration=1, update_with_mean=True, mean_percentile=100)
    with M.MutoMLSD(cfg) as rec:
        rec.load_tracks(wl.tracks())
        rec.prepare()
        mult = rec.multiplicity().astype(np.float64)
        x = _start(wl, mult, 7)
        lam0 = np.where(mult > 0, np.exp(x), 0.0)
        _, g = rec.nll_grad(x)
        rec.set_image(lam0)
        rec.iterate(1)
        lam1 = rec.image().reshape(-1, order="F")
    m = mult > 0
    step = -lam0[m] * g[m] / (2.0 * mult[m])
    assert rel_l2(lam1[m] - lam0[m], step) < 1e-9
    assert np.all(lam1[~m] == 0.0)


def test_gradient_solve_lowers_the_objective(gpu):
    wl = W.small(n_muons=6000, seed=161, n=8)
    cfg = wl.em_config(precision="fp64", num_iteration=0, beta=0.01, p=1.2, delta=0.1, all_neighbours=True)
    with M.MutoMAP(cfg) as rec:
        rec.load_tracks(wl.tracks())
        rec.prepare()
        mult = rec.multiplicity()
        x = _start(wl, mult, 11)
        f0 = rec.nll(x)
        rec.set_image(np.where(mult > 0, np.exp(x), 0.0))
        f1 = rec.gradient_solve(5)
        f2 = rec.gradient_solve(10)
        img = rec.image().reshape(-1, order="F")
        f_img = rec.nll(np.where(mult > 0, np.log(np.where(img > 0, img, 1.0)), 0.0))
    assert f1 < f0 and f2 <= f1
    assert abs(f_img - f2) <= 1e-9 * abs(f2)
    assert np.all(img[mult > 0] > 0)


@pytest.mark.parametrize("beta", [1e-3, 1e-2])
@pytest.mark.parametrize("p", [2.0, 1.0])
def test_gradient_solver_reaches_the_em_objective(gpu, beta, p):
    # the 128x128x64 grid of 15 mm voxels (300 k muons): 20 MAP EM iterations
    # (mean ML step), then the gradient solver from the same start to the
    # objective value EM reached (src/MutoMAP.cpp:129-198 is the EM side)
    wl = W.map128x128x64_15mm(n_muons=300_000)
    rays = wl.tracks()
    cfg = wl.em_config(precision="fp64", num_iteration=20, update_with_mean=True, beta=beta, p=p,
                       all_neighbours=True, delta=0.1 * float(np.median(wl.lam())) * 1e7)
    with M.MutoMAP(cfg) as a:
        img = a.reconstruct(rays).reshape(-1, order="F")
        mult = a.multiplicity()
        f_em = a.nll(np.log(np.where(mult > 0, np.maximum(img, 1e-300), 1.0)))
    with M.MutoMAP(dict(cfg, num_iteration=0)) as b:
        b.load_tracks(rays)
        b.prepare()
        f0 = b.nll(np.log(np.where(mult > 0, 1e-7, 1.0)))
        f_g, it = b.gradient_solve_until(f_em, 50)
    assert f_em < f0  # EM lowered the objective
    assert f_g <= f_em and 1 <= it <= 50
