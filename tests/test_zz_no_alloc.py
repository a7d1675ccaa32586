"""muto_siddon_batch_noalloc against muto_siddon_batch, both through the C ABI.

The allocation-free walk stages its work through one fixed device array that
every call shares, so it is checked on two calls in a row (different inputs
and caps), each against the allocating entry point on the same inputs.  The
Siddon walk is FP64 index and length work: the tolerance is bit-exact.  The
first batch needs several chunks of the shared array (20000 rays at cap 512
is about 200 MB of voxel slots against a 16 MiB array).

This file is collected last on purpose: it must pass both in a fresh process
and after every other test has used the library.
"""
import ctypes as C

import numpy as np
import pytest

import muontomography_gb300 as M
from muontomography_gb300 import _lib

MAX_CAP = 65536  # MUTO_NOALLOC_MAX_CAP


def _segments(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, size=(n, 3)), rng.uniform(lo, hi, size=(n, 3))


def _call(fn_name, grid, p1, p2, cap, with_stream):
    lib = _lib.load()
    p1 = np.ascontiguousarray(p1, np.float64)
    p2 = np.ascontiguousarray(p2, np.float64)
    n = p1.shape[0]
    # filled with a pattern so that slots the call does not write stay visible
    xyz = np.full((n, cap, 3), 0xDEADBEEF, np.uint32)
    ln = np.full((n, cap), -7.0, np.float64)
    cnt = np.full(n, 0xDEADBEEF, np.uint32)
    g = grid.c()
    args = [C.byref(g), _lib.dptr(p1), _lib.dptr(p2), n, cap, _lib.u32ptr(xyz), _lib.dptr(ln), _lib.u32ptr(cnt)]
    if with_stream:
        args.append(None)  # legacy default stream
    rc = getattr(lib, fn_name)(*args)
    return rc, xyz, ln, cnt


def _assert_same_walk(new, old):
    _, nx, nl, nc = new
    _, ox, ol, oc = old
    cap = nx.shape[1]
    assert np.array_equal(nc, oc)
    for r in range(nc.shape[0]):
        k = min(int(oc[r]), cap) if oc[r] != 0xFFFFFFFF else 0
        assert np.array_equal(nx[r, :k], ox[r, :k]), r
        assert np.array_equal(nl[r, :k].view(np.uint64), ol[r, :k].view(np.uint64)), r
        # slots past the count are zeroed, never left over from an earlier call
        assert not nx[r, k:].any() and not nl[r, k:].any(), r


def test_cap_beyond_limit_is_rejected_before_the_device():
    grid = M.Grid(4, 4, 4, 0.0, 0.0, 0.0, 10.0, 10.0, 10.0)
    lib = _lib.load()
    p = np.zeros((1, 3), np.float64)
    xyz = np.zeros(3, np.uint32)
    ln = np.zeros(1, np.float64)
    cnt = np.zeros(1, np.uint32)
    g = grid.c()
    rc = lib.muto_siddon_batch_noalloc(C.byref(g), _lib.dptr(p), _lib.dptr(p), 1, MAX_CAP + 1, _lib.u32ptr(xyz),
                                       _lib.dptr(ln), _lib.u32ptr(cnt), None)
    assert rc == 5  # MUTO_ERR_CAPACITY


@pytest.mark.gpu
def test_noalloc_matches_allocating_walk_two_calls_in_a_row(gpu):
    # 100^3 voxels of 2 mm at -100 with segment ends uniform in [-500, 500]^3
    grid = M.Grid(100, 100, 100, -100.0, -100.0, -100.0, 2.0, 2.0, 2.0)
    first = _segments(20000, -500.0, 500.0, seed=11)
    # second call: other rays, a smaller cap (some counts exceed it), one chunk
    second = _segments(3000, -150.0, 150.0, seed=12)
    seen = []
    for (p1, p2), cap in ((first, 512), (second, 96)):
        old = _call("muto_siddon_batch", grid, p1, p2, cap, with_stream=False)
        new = _call("muto_siddon_batch_noalloc", grid, p1, p2, cap, with_stream=True)
        assert old[0] == _lib.MUTO_OK and new[0] == _lib.MUTO_OK
        assert (old[3] > 0).sum() > 500
        _assert_same_walk(new, old)
        seen.append(old[3])
    assert (seen[1] > 96).sum() > 0  # the second call truncated some paths at cap


@pytest.mark.gpu
def test_noalloc_at_the_cap_limit(gpu):
    # the largest cap leaves room for a dozen rays per chunk: 40 rays take 4 chunks
    grid = M.Grid(100, 100, 100, -100.0, -100.0, -100.0, 2.0, 2.0, 2.0)
    p1, p2 = _segments(40, -300.0, 300.0, seed=13)
    old = _call("muto_siddon_batch", grid, p1, p2, MAX_CAP, with_stream=False)
    new = _call("muto_siddon_batch_noalloc", grid, p1, p2, MAX_CAP, with_stream=True)
    assert old[0] == _lib.MUTO_OK and new[0] == _lib.MUTO_OK
    _assert_same_walk(new, old)
