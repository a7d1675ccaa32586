"""The failure counters of muto_status driven above zero on the GPU.

Singular covariance (src/MutoMLSD.cpp:457-464): with lambda = 0 everywhere
and no measurement error (error_xy 0) every Sigma_i is the zero matrix; the
reference then leaves the inverse at zero (s_ij = 2 lambda_j) and takes the
muon's cost as 0.  Non-converging cubic (src/MutoMAP.cpp:374-381, which has
no iteration cap): with newton_max_iter 1 the capped Newton iteration stops
before its tolerance, and the solves that did are counted.
"""
import numpy as np
import pytest

import muontomography_gb300 as M
from muontomography_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("mode", ["median", "mean"])
def test_singular_covariance_is_counted_and_keeps_lambda(gpu, oracle, precision, mode):
    wl = W.small(n_muons=3000, seed=201)
    rays = wl.tracks()
    over = {"update_with_mean": True} if mode == "mean" else {}
    cfg = wl.em_config(precision=precision, num_iteration=2, initialize_method=2, initialize_value=0.0, error_xy=0.0,
                       compute_cost=True, **over)
    ref = oracle.Mlsd(wl.grid, cfg, rays, np.zeros(wl.grid.nvox))
    ref.iterate(2)
    with M.MutoMLSD(cfg) as rec:
        img = rec.reconstruct(rays)
        st = rec.status()
    kept = st["n_scat_in_grid"]
    assert kept > 0
    assert st["n_singular"] == 2 * kept == ref.counts()["n_singular"]
    assert not np.any(img) and not np.any(ref.image())  # s_ij = 2 lambda_j = 0
    assert st["cost"] == 0.0 and st["iterations_done"] == 2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_newton_cap_is_counted(gpu, precision):
    wl = W.small(n_muons=4000, seed=202)
    rays = wl.tracks()
    cfg = wl.em_config(precision=precision, num_iteration=2, newton_max_iter=1)
    cfg.update(beta=0.01, p=1.0, all_neighbours=True, delta=0.1 * float(np.median(wl.lam())) * 1e7)
    with M.MutoMAP(cfg) as rec:
        img = rec.reconstruct(rays)
        st = rec.status()
    assert st["n_nonconverged"] > 0
    assert np.all(np.isfinite(img))
    with M.MutoMAP(dict(cfg, newton_max_iter=200)) as rec:
        rec.reconstruct(rays)
        assert rec.status()["n_nonconverged"] == 0
