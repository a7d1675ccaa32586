"""CPU tests of the bench's host-side arithmetic: the algorithmic bytes each
kernel's roofline is computed from, the reference leg's sample size, the
core count and the peak it divides by.  No kernel is launched here."""
import importlib.util
import os
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_algorithmic_bytes_of_the_mean_update(bench):
    P, N, V = 1000, 10, 100
    # mixed form (4-byte reals): the lists once, 12 B per pair
    assert bench.algorithmic_bytes("em_muon", 4, P, N, V) == 12 * P + (8 + 36) * N + 4 * V
    assert bench.algorithmic_bytes("em_scatter", 4, P, N, V) == 12 * P + (8 + 16) * N + 4 * V
    assert bench.algorithmic_bytes("em_fused", 4, P, N, V) == 12 * P + (8 + 20) * N + 8 * V
    assert bench.algorithmic_bytes("em_update", 4, P, N, V) == 20 * V
    # FP64 form: 20 B per pair
    assert bench.algorithmic_bytes("em_muon", 8, P, N, V) == 20 * P + (8 + 72) * N + 8 * V
    assert bench.algorithmic_bytes("no_such_kernel", 4, P, N, V) == 0


def test_algorithmic_bytes_of_the_median_voxel_pass(bench):
    P, N, V = 1000, 10, 100
    assert bench.algorithmic_bytes("em_voxel", 4, P, N, V) == 12 * P + (16 + 24) * V


@pytest.mark.parametrize("steps,warmup,cap,want", [
    (30, 3, 10**9, int(150.0 / 33 * 1.5e7 / 100.0)),  # about 150 s of iterations in all
    (1, 0, 3000, 3000),                               # the cap wins
    (10**6, 0, 10**9, 20_000),                        # never fewer than 20 000 muons
])
def test_reference_sample(bench, steps, warmup, cap, want):
    assert bench.reference_sample(steps, warmup, cap) == want


def test_host_cores_follow_the_affinity_mask(bench):
    assert bench.host_cores() == len(os.sched_getaffinity(0))


def test_peak_is_the_measured_copy_rate(bench):
    p = bench.peaks()
    if (ROOT / "MEASURED_PEAKS.json").exists():
        assert p["source"] == "measured" and p["hbm_gbs"] > 1000.0
    else:
        assert p == {"hbm_gbs": 6800.0, "source": "fallback"}


def test_traffic_per_pair_cites_captures_near_the_algorithmic_bytes(bench):
    # ncu's DRAM bytes per pair of each captured kernel: within a few percent
    # of the 12 algorithmic bytes per pair of the mixed lists
    for (family, kernel), b in bench.TRAFFIC_PER_PAIR.items():
        if family == "grid256":
            assert 12.0 <= b <= 13.5, (kernel, b)
