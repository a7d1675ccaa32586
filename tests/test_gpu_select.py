"""Exact order statistics of the voxel update, through muto_select_probe.

The probe runs the voxel-pass kernels of an EM iteration on chosen segments
(s_i = 2 + x_i, lambda = 1), so every path of the selection is reached on
purpose: staged sorts of short segments, the sampling rounds, the window
misses that fall back to the radix search (sorted inputs put the samples at
one end), duplicates that stop the windows shrinking, every segment-length
class and the scratch-array path of the longest segments, with long
segments held in registers or streamed ("voxel_stream_above"), and passes
that start from the selection windows an earlier pass left, whether those
still hold the target or not.

The median update is compared bit for bit with numpy on the same float32 (or
float64) s_i: halved middle value, or a quarter of the sum of the two middle
values for even counts (src/MutoMLSD.cpp:506-516).  The percentile and mean
updates add values in a different order than numpy: 8e-5 (float) and
8e-12 (double), relative to max(1, |update|).
"""
import ctypes as C

import numpy as np
import pytest

from muontomography_gb300 import _lib

pytestmark = pytest.mark.gpu

LENGTHS = [1, 2, 3, 5, 31, 32, 33, 63, 64, 65, 100, 127, 128, 129, 191, 192, 193, 255, 256, 257, 300, 383, 384,
           385, 511, 512, 513, 600, 767, 768, 769, 1000, 1023, 1024, 1025, 1535, 1536, 1537, 2000, 4096, 10000]


def _segment(rng, m, kind):
    if kind == "uniform":
        return rng.uniform(-1.0, 5.0, m)
    if kind == "dups":
        return rng.integers(0, 7, m).astype(np.float64) * 0.25
    if kind == "equal":
        return np.full(m, 0.75)
    if kind == "ascending":
        return np.sort(rng.uniform(0.0, 3.0, m))
    if kind == "descending":
        return -np.sort(-rng.uniform(-3.0, 3.0, m))
    if kind == "heavy":
        return rng.lognormal(0.0, 2.0, m)
    if kind == "clusters":
        return np.where(rng.random(m) < 0.5, rng.normal(-5.0, 1e-3, m), rng.normal(7.0, 1e-3, m))
    if kind == "negative":
        return rng.uniform(-9.0, -2.5, m)  # s_i below zero
    raise ValueError(kind)


KINDS = ["uniform", "dups", "equal", "ascending", "descending", "heavy", "clusters", "negative"]


def _segments(seed, dtype):
    rng = np.random.default_rng(seed)
    segs = [_segment(rng, m, k).astype(dtype) for m in LENGTHS for k in KINDS]
    segs.append(np.zeros(0, dtype))  # an empty segment: the update is 0
    return segs


def _probe(segs, precision, update_with_mean=0, pct=100, stream_above=-1, earlier=()):
    """The probe's last pass on segs; `earlier` passes (same lengths) run first
    and leave the selection windows the last pass starts from."""
    lib = _lib.load()
    passes = list(earlier) + [segs]
    vals = np.ascontiguousarray(np.concatenate([np.concatenate(p) for p in passes]).astype(np.float64))
    n = vals.size // len(passes)
    off = np.zeros(len(segs) + 1, np.uint64)
    off[1:] = np.cumsum([len(s) for s in segs])
    out = np.full(len(segs), np.nan)
    rc = lib.muto_select_probe(precision, _lib.dptr(vals), n, off.ctypes.data_as(C.POINTER(C.c_uint64)),
                               len(segs), update_with_mean, pct, stream_above, len(passes), _lib.dptr(out))
    assert rc == _lib.MUTO_OK
    return out


def _median_update(x, dtype):
    if x.size == 0:
        return 0.0
    s = np.sort(dtype(2) + x.astype(dtype))
    m = s.size
    if m % 2:
        return float(s[m // 2] * dtype(0.5))
    return float((s[m // 2] + s[m // 2 - 1]) * dtype(0.25))


@pytest.mark.parametrize("precision,dtype", [(0, np.float32), (1, np.float64)])
@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("stream_above", [-1, 256, 512])
def test_median_update_bit_exact(gpu, precision, dtype, seed, stream_above):
    segs = _segments(seed, dtype)
    got = _probe(segs, precision, stream_above=stream_above)
    want = np.array([_median_update(s, dtype) for s in segs])
    bad = np.nonzero(got.view(np.uint64) != want.view(np.uint64))[0]
    assert bad.size == 0, [(len(segs[i]), KINDS[i % len(KINDS)] if i < len(LENGTHS) * len(KINDS) else "empty",
                            got[i], want[i]) for i in bad[:10]]


@pytest.mark.parametrize("precision,dtype,tol", [(0, np.float32, 1e-5), (1, np.float64, 1e-12)])
@pytest.mark.parametrize("pct", [1, 37, 50, 90, 100])
@pytest.mark.parametrize("stream_above", [-1, 256])
def test_percentile_and_mean_update(gpu, precision, dtype, tol, pct, stream_above):
    segs = _segments(7, dtype)
    got = _probe(segs, precision, update_with_mean=1, pct=pct, stream_above=stream_above)
    for i, x in enumerate(segs):
        if x.size == 0:
            assert got[i] == 0.0
            continue
        s = np.sort((dtype(2) + x.astype(dtype)).astype(np.float64))
        if pct == 100:
            want = 1.0 + x.astype(np.float64).sum() / (2.0 * x.size)
        else:
            jm = min(max(int(pct / 100.0 * s.size), 1), s.size)
            want = s[:jm].mean() * 0.5
        assert abs(got[i] - want) <= tol * max(1.0, abs(want)) * 8, (i, s.size, got[i], want)


@pytest.mark.parametrize("precision,dtype", [(0, np.float32), (1, np.float64)])
@pytest.mark.parametrize("before", ["same", "drift", "other"])
def test_median_from_carried_windows_bit_exact(gpu, precision, dtype, before):
    # iterations start from the window the previous one left: exact whether
    # it still holds the median (same values, a small drift) or not (other values)
    segs = _segments(3, dtype)
    if before == "same":
        earlier = [segs, segs]
    elif before == "drift":
        earlier = [[(s * dtype(1.02) - dtype(0.01)).astype(dtype) for s in segs],
                   [(s * dtype(1.01) + dtype(0.003)).astype(dtype) for s in segs]]
    else:
        earlier = [_segments(4, dtype), _segments(5, dtype)]
    got = _probe(segs, precision, earlier=earlier)
    want = np.array([_median_update(s, dtype) for s in segs])
    bad = np.nonzero(got.view(np.uint64) != want.view(np.uint64))[0]
    assert bad.size == 0, [(len(segs[i]), got[i], want[i]) for i in bad[:10]]


@pytest.mark.parametrize("precision,dtype,tol", [(0, np.float32, 1e-5), (1, np.float64, 1e-12)])
def test_percentile_from_carried_windows(gpu, precision, dtype, tol):
    segs = _segments(8, dtype)
    got = _probe(segs, precision, update_with_mean=1, pct=37, earlier=[_segments(9, dtype), segs])
    for i, x in enumerate(segs):
        if x.size == 0:
            continue
        s = np.sort((dtype(2) + x.astype(dtype)).astype(np.float64))
        jm = min(max(int(0.37 * s.size), 1), s.size)
        want = s[:jm].mean() * 0.5
        assert abs(got[i] - want) <= tol * max(1.0, abs(want)) * 8, (i, s.size, got[i], want)
