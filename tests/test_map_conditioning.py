"""The MAP update with p = 1 amplifies rounding-sized changes; with p = 2 it
does not.  Shown on the FP64 oracle (the reference's MAP restated,
src/MutoMAP.cpp:129-406): the surrogate's choice among the roots of its
cubic (chooseBestEstimation, :239-259) switches on differences at the level
of one rounding when |l_j - l_m| is near delta, and the iteration carries
the switch on.  This is why the mixed form's MAP image is judged against the
FP64 form's own spread under a 1e-7 change of its input, not against 1e-4."""
import numpy as np
import pytest

from muontomography_gb300 import workloads as W


def spread(oracle, p):
    wl = W.small(n_muons=60000, seed=7, n=24)
    rays = wl.tracks()
    lam = wl.lam()
    cfg = wl.em_config(precision="fp64", num_iteration=20, beta=0.01, p=p, all_neighbours=True,
                       delta=0.1 * float(np.median(lam)) * 1e7)
    init = np.full(wl.grid.nvox, 1e-7)
    pert = init * (1.0 + 1e-7 * np.random.default_rng(3).uniform(-1.0, 1.0, init.size))
    out = []
    runs = [oracle.Mlsd(wl.grid, cfg, rays, x0, method="map") for x0 in (init, pert)]
    done = 0
    for it in (5, 20):
        for r in runs:
            r.iterate(it - done)
        done = it
        a, b = (r.image() for r in runs)
        out.append(float(np.linalg.norm(b - a) / np.linalg.norm(a)))
    return out


def test_p1_amplifies_a_rounding_sized_change(oracle):
    at5, at20 = spread(oracle, 1.0)
    assert at20 > 1e-4 and at20 > 100 * at5


def test_p2_does_not(oracle):
    at5, at20 = spread(oracle, 2.0)
    assert at5 < 1e-6 and at20 < 1e-6
