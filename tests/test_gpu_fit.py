"""Batched GPU line fit of raw detector records (MutoFile::getMuonData's
per-record step, src/MutoFile.cpp:58-78 and :248-304) against the oracle's
SVD restatement (within 1e-9 mm and 1e-12 in the unit directions) and
against the host reader, which runs the same fit on the CPU (bit for bit)."""
import ctypes as C

import numpy as np
import pytest

import muontomography_gb300 as M
from muontomography_gb300 import _lib, build as B

pytestmark = pytest.mark.gpu

Z = [1500.0, 1000.0, 500.0, -500.0, -1000.0, -1500.0]  # input/example_mlsd.json:3-4
N_MIDDLE = 3


def records(n, seed, sigma=1.0):
    """Records of generated tracks with smeared hits and a few NaN rows."""
    g = M.Grid(10, 10, 10, -500.0, -500.0, -500.0, 100.0, 100.0, 100.0)
    rays = M.generate(g, np.full(g.nvox, 1e-7), n, seed=seed)
    rng = np.random.default_rng(seed)
    rec = np.empty((n, 2 * len(Z) + 2))
    rec[:, 0], rec[:, -1] = rays[:, 0], rays[:, 1]
    for k, zk in enumerate(Z):
        p, d = (rays[:, 2:5], rays[:, 8:11]) if k < N_MIDDLE else (rays[:, 5:8], rays[:, 11:14])
        t = (zk - p[:, 2]) / d[:, 2]
        rec[:, 1 + 2 * k] = p[:, 0] + t * d[:, 0] + sigma * rng.standard_normal(n)
        rec[:, 2 + 2 * k] = p[:, 1] + t * d[:, 1] + sigma * rng.standard_normal(n)
    rec[rng.choice(n, 5, replace=False), rng.integers(0, rec.shape[1], 5)] = np.nan
    return rec


def host_reader(path, precision):
    B.build()
    lib = C.CDLL(str(B.facade_lib_path()))
    lib.muto_read_muon_data.argtypes = [C.POINTER(C.c_char_p), C.c_int, C.POINTER(C.c_double), C.c_int, C.c_int,
                                        C.c_int, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]
    arr = (C.c_char_p * 1)(str(path).encode())
    zz = np.asarray(Z, np.float64)
    n = C.c_uint64()
    assert lib.muto_read_muon_data(arr, 1, _lib.dptr(zz), len(Z), N_MIDDLE, precision, None, 0, C.byref(n)) == 0
    out = np.zeros((n.value, 14))
    assert lib.muto_read_muon_data(arr, 1, _lib.dptr(zz), len(Z), N_MIDDLE, precision,
                                   out.ctypes.data_as(C.c_void_p), n.value, C.byref(n)) == 0
    return out[: n.value]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_fit_matches_oracle_and_host_reader(gpu, oracle, tmp_path, dtype):
    rec = records(4000, seed=11).astype(dtype)
    got = M.fit_tracks(rec, Z, N_MIDDLE)
    want = oracle.fit_records(rec, Z, N_MIDDLE)
    assert got.shape == want.shape == (4000 - 5, 14)
    np.testing.assert_array_equal(got[:, :2], want[:, :2])
    np.testing.assert_allclose(got[:, 2:8], want[:, 2:8], rtol=0, atol=1e-9)
    np.testing.assert_allclose(got[:, 8:], want[:, 8:], rtol=0, atol=1e-12)
    f = tmp_path / "hits.bin"
    rec.tofile(f)
    host = host_reader(f, np.dtype(dtype).itemsize)
    assert np.array_equal(got.view(np.uint64), host.view(np.uint64))


def test_fit_chunks_and_edges(gpu, oracle):
    # more records than one device round trip (2^20), exact hits, all-NaN and empty inputs
    rec = records(1_100_000, seed=5, sigma=0.0)
    got = M.fit_tracks(rec, Z, N_MIDDLE)
    assert got.shape == (1_100_000 - 5, 14)
    keep = ~np.isnan(rec).any(axis=1)
    sample = np.nonzero(keep)[0][::997]
    want = oracle.fit_records(rec[sample], Z, N_MIDDLE)
    idx = np.cumsum(keep)[sample] - 1
    np.testing.assert_allclose(got[idx, 2:8], want[:, 2:8], rtol=0, atol=1e-9)
    np.testing.assert_allclose(got[idx, 8:], want[:, 8:], rtol=0, atol=1e-12)
    assert M.fit_tracks(np.full((3, 14), np.nan), Z, N_MIDDLE).shape == (0, 14)
    assert M.fit_tracks(np.zeros((0, 14)), Z, N_MIDDLE).shape == (0, 14)
