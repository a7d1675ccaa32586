"""The C++ host layer: raw-hit reader (MutoFile::getMuonData), the image file
format through MutoFile, and the command-line program (MuToTest.cpp's
replacement) running the reconstruction classes on the GPU."""
import ctypes as C
import json
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import muontomography_gb300 as M
from muontomography_gb300 import _lib, build as B

Z = [1500.0, 1000.0, 500.0, -500.0, -1000.0, -1500.0]  # input/example_mlsd.json:3-4
N_MIDDLE = 3


@pytest.fixture(scope="module")
def facade():
    B.build()
    lib = C.CDLL(str(B.facade_lib_path()))
    lib.muto_read_muon_data.argtypes = [C.POINTER(C.c_char_p), C.c_int, C.POINTER(C.c_double), C.c_int, C.c_int,
                                        C.c_int, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]
    return lib


def read(facade, files, z=Z, n_middle=N_MIDDLE, precision=4):
    arr = (C.c_char_p * len(files))(*[str(f).encode() for f in files])
    zz = np.asarray(z, np.float64)
    n = C.c_uint64()
    rc = facade.muto_read_muon_data(arr, len(files), _lib.dptr(zz), len(z), n_middle, precision, None, 0, C.byref(n))
    assert rc == 0
    out = np.zeros((n.value, 14), np.float64)
    rc = facade.muto_read_muon_data(arr, len(files), _lib.dptr(zz), len(z), n_middle, precision,
                                    out.ctypes.data_as(C.c_void_p), n.value, C.byref(n))
    assert rc == 0
    return out[: n.value]


def hits_from_tracks(rays, z=Z, n_middle=N_MIDDLE):
    """Detector records {ein, x0, y0, ..., eout} of the tracks' in/out lines."""
    recs = []
    for r in rays:
        pin, pout, din, dout = r[2:5], r[5:8], r[8:11], r[11:14]
        row = [r[0]]
        for k, zk in enumerate(z):
            p, d = (pin, din) if k < n_middle else (pout, dout)
            t = (zk - p[2]) / d[2]
            row += [p[0] + t * d[0], p[1] + t * d[1]]
        row.append(r[1])
        recs.append(row)
    return np.asarray(recs)


def test_reader_recovers_exact_lines(facade, tmp_path):
    g = M.Grid(10, 10, 10, -500.0, -500.0, -500.0, 100.0, 100.0, 100.0)
    rays = M.generate(g, np.full(g.nvox, 1e-7), 200, seed=3)
    # the reader puts pin / pout on layers n_middle-1 / n_middle: move the tracks there
    for r in rays:
        for (p, d, zt) in ((slice(2, 5), slice(8, 11), Z[N_MIDDLE - 1]), (slice(5, 8), slice(11, 14), Z[N_MIDDLE])):
            t = (zt - r[p][2]) / r[d][2]
            r[p] = r[p] + t * r[d]
    rec = hits_from_tracks(rays)
    rec[17, 4] = np.nan  # a record with a NaN is skipped (src/MutoFile.cpp:71-76)
    f = tmp_path / "hits.bin"
    rec.astype(np.float64).tofile(f)
    got = read(facade, [f, tmp_path / "missing.bin"], precision=8)
    want = np.delete(rays, 17, axis=0)
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-9)
    rec.astype(np.float32).tofile(f)
    got32 = read(facade, [f], precision=4)
    np.testing.assert_allclose(got32[:, 8:], want[:, 8:], atol=1e-4)


def test_reader_rejects_bad_layouts(facade, tmp_path):
    zz = np.asarray(Z, np.float64)
    n = C.c_uint64()
    arr = (C.c_char_p * 1)(b"x")
    assert facade.muto_read_muon_data(arr, 1, _lib.dptr(zz), 6, 1, 4, None, 0, C.byref(n)) == 1
    assert facade.muto_read_muon_data(arr, 1, _lib.dptr(zz), 6, 3, 2, None, 0, C.byref(n)) == 1


def test_facade_library_exports_io_header(facade):
    text = (B.INCLUDE / "muto_io.h").read_text()
    for name in re.findall(r"\b(muto_[a-z_]+)\s*\(", re.sub(r"/\*.*?\*/", "", text, flags=re.S)):
        assert hasattr(facade, name), name


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["poca", "mlsd", "map"])
def test_cli_end_to_end(gpu, facade, tmp_path, method):
    from muontomography_gb300 import workloads as W

    wl = W.small(n_muons=3000, seed=17, n=10)
    rays = wl.tracks()
    hits = hits_from_tracks(rays, z=[300.0 + 500 * k for k in (2, 1, 0)] + [-300.0 - 500 * k for k in (0, 1, 2)])
    f = tmp_path / "hits.bin"
    hits.astype(np.float32).tofile(f)
    zl = [1300.0, 800.0, 300.0, -300.0, -800.0, -1300.0]
    section = wl.poca_config() if method == "poca" else wl.em_config(num_iteration=4, precision="fp64")
    if method == "map":
        section.update(beta=0.01, p=1.0, delta=0.1)
    cfg = {"data_files": [str(f)], "detector_height": zl, "detector_middle": 3,
           "output_file": str(tmp_path / "out.bin"), method: section}
    (tmp_path / "cfg.json").write_text(json.dumps(cfg))
    r = subprocess.run([str(B.cli_path()), str(tmp_path / "cfg.json")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"Reconstruction with <{method}> took" in r.stdout
    img, hdr = M.load_image(str(tmp_path / "out.bin"))
    assert hdr["method"] == method and hdr["n_ray"] == len(rays) and hdr["precision"] == 4
    # the same tracks through the Python view of the C ABI
    tracks = read(facade, [f], z=zl)
    with M.Reconstruction(method, section) as rec:
        rec._n_iter = section.get("num_iteration", 1)
        want = rec.reconstruct(tracks)
    assert np.array_equal(img, want.astype(np.float32).astype(np.float64))


@pytest.mark.parametrize("precision", [8, 4])
def test_reader_matches_oracle_svd_fit(facade, oracle, tmp_path, precision):
    # smeared hits: the principal-axis fit against the oracle's SVD restatement
    g = M.Grid(10, 10, 10, -500.0, -500.0, -500.0, 100.0, 100.0, 100.0)
    rays = M.generate(g, np.full(g.nvox, 1e-7), 300, seed=8)
    rec = hits_from_tracks(rays)
    rng = np.random.default_rng(8)
    rec[:, 1:-1] += rng.standard_normal((rec.shape[0], rec.shape[1] - 2))
    rec[[4, 250], [0, 9]] = np.nan
    rec = rec.astype(np.float64 if precision == 8 else np.float32)
    f = tmp_path / "hits.bin"
    rec.tofile(f)
    got = read(facade, [f], precision=precision)
    want = oracle.fit_records(rec, Z, N_MIDDLE)
    assert got.shape == want.shape == (298, 14)
    np.testing.assert_array_equal(got[:, :2], want[:, :2])
    np.testing.assert_allclose(got[:, 2:8], want[:, 2:8], rtol=0, atol=1e-9)
    np.testing.assert_allclose(got[:, 8:], want[:, 8:], rtol=0, atol=1e-12)


def test_fit_tracks_rejects_bad_layouts(facade):
    lib = M.library()
    zz = np.asarray(Z, np.float64)
    n = C.c_uint64()
    rec = np.zeros((2, 14))
    p = rec.ctypes.data_as(C.c_void_p)
    out = np.zeros((2, 14)).ctypes.data_as(C.c_void_p)
    assert lib.muto_fit_tracks(p, 2, 2, _lib.dptr(zz), 6, 3, out, C.byref(n)) == 1      # precision
    assert lib.muto_fit_tracks(p, 8, 2, _lib.dptr(zz), 6, 1, out, C.byref(n)) == 1      # one upper layer
    assert lib.muto_fit_tracks(p, 8, 2, _lib.dptr(zz), 6, 5, out, C.byref(n)) == 1      # one lower layer
    assert lib.muto_fit_tracks(p, 8, 2, _lib.dptr(zz), 65, 3, out, C.byref(n)) == 1     # > 64 layers
    assert lib.muto_fit_tracks(p, 8, 2, _lib.dptr(zz), 6, 3, None, C.byref(n)) == 1     # no output
    assert lib.muto_fit_tracks(p, 8, 2, _lib.dptr(zz), 6, 3, out, None) == 1            # no count


GOLD = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("precision", [8, 4])
def test_reader_matches_reference_reader(facade, tmp_path, precision):
    # the reference's own MutoFile::getMuonData on the same records (tests/golden/files.npz)
    F = np.load(GOLD / "files.npz")
    rec = F["records64"] if precision == 8 else F["records32"]
    f = tmp_path / "hits.bin"
    rec.tofile(f)
    got = read(facade, [f], z=list(F["z_layers"]), n_middle=int(F["n_middle"]), precision=precision)
    want = F[f"tracks{precision}"]
    assert got.shape == want.shape == (398, 14)
    np.testing.assert_array_equal(got[:, :2], want[:, :2])
    np.testing.assert_allclose(got[:, 2:8], want[:, 2:8], rtol=0, atol=1e-9)
    np.testing.assert_allclose(got[:, 8:], want[:, 8:], rtol=0, atol=1e-12)


@pytest.mark.parametrize("precision", [8, 4])
def test_image_files_match_reference_files(tmp_path, precision):
    # MutoFile::saveImage / loadImage (src/MutoFile.cpp:85-211) against files the reference wrote
    F = np.load(GOLD / "files.npz")
    a = F["image_grid"]
    g = M.Grid(int(a[0]), int(a[1]), int(a[2]), *map(float, a[3:]))
    ref = F[f"image_file{precision}"].tobytes()
    p = tmp_path / "ours.bin"
    M.save_image(str(p), F["image"], g, "mlsd", 123456, 50, precision)
    ours = p.read_bytes()
    assert len(ours) == len(ref) == 64 + precision * g.nvox
    # bytes 2-17 hold the method copied from a std::string: past its NUL the
    # reference writes whatever the string's buffer holds, the library zeros
    assert ours[:7] == ref[:7] and ours[18:] == ref[18:]
    assert ours[7:18] == bytes(11)
    q = tmp_path / "ref.bin"
    q.write_bytes(ref)
    img, hdr = M.load_image(str(q))
    want = F["image"] if precision == 8 else F["image"].astype(np.float32).astype(np.float64)
    assert np.array_equal(img, want)
    assert (hdr["method"], hdr["n_ray"], hdr["n_iter"], hdr["precision"]) == ("mlsd", 123456, 50, precision)
    assert hdr["grid"] == g


@pytest.mark.parametrize("precision", [8, 4])
def test_reader_drops_a_truncated_last_record(facade, tmp_path, precision):
    # a file cut inside its last record: the whole records are read, the rest
    # ignored (nRay = filesize / nEach / precision, src/MutoFile.cpp:52-55)
    F = np.load(GOLD / "files.npz")
    rec = F["records64"] if precision == 8 else F["records32"]
    f = tmp_path / "hits.bin"
    f.write_bytes(rec.tobytes() + rec[:1].tobytes()[: 5 * precision + 3])
    got = read(facade, [f], z=list(F["z_layers"]), n_middle=int(F["n_middle"]), precision=precision)
    want = F[f"tracks{precision}"]
    assert got.shape == want.shape
    np.testing.assert_allclose(got[:, 2:], want[:, 2:], rtol=0, atol=1e-9)
    # two files: the tracks of both, in file order; an empty file adds nothing
    (tmp_path / "empty.bin").write_bytes(b"")
    both = read(facade, [f, tmp_path / "empty.bin", f], z=list(F["z_layers"]), n_middle=int(F["n_middle"]),
                precision=precision)
    assert np.array_equal(both, np.concatenate([got, got]))


@pytest.mark.parametrize("cfg,message", [
    (None, "Configuration file load error"),
    ({"data_files": [], "detector_height": [1.0, 0.0, -1.0, -2.0], "detector_middle": 2, "output_file": "o.bin"},
     "No supported reconstruction key"),
    ({"detector_height": [1.0, 0.0, -1.0, -2.0]}, "Configuration error"),
    ("{not json", "Configuration file load error"),
])
def test_cli_reports_configuration_errors(facade, tmp_path, cfg, message):
    # the command-line program stops with status 1 before any device work
    path = tmp_path / "cfg.json"
    if cfg is not None:
        path.write_text(cfg if isinstance(cfg, str) else json.dumps(cfg))
    r = subprocess.run([str(B.cli_path()), str(path)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 1
    assert message in r.stdout + r.stderr
    assert not (tmp_path / "o.bin").exists()


USER_PROGRAM = r"""
// a program written against the reference's headers (MuToTest.cpp style)
#include <iostream>
#include "MutoFile.h"
#include "MutoReconstruction.h"
#include "MutoSiddon.h"

int main() {
    VoxelGrid g{10, 10, 10, -50.0, -50.0, -50.0, 10.0, 10.0, 10.0};
    MutoSiddon siddon(g);                      // include/MutoSiddon.h:14
    std::vector<Vector3> none;
    std::cout << siddon.getVoxelPaths(none, none).size() << "\n";  // no segments: no device work
    std::cout << MutoFile::getCurrentPath() << "\n";                // include/MutoFile.h:65
    MutoMuonData data = MutoFile::getMuonData({}, {1.0, 0.0, -1.0, -2.0}, 2);
    std::cout << data.size() << "\n";
    return 0;
}
"""


def test_user_program_compiles_against_the_headers(facade, tmp_path):
    src = tmp_path / "user.cpp"
    src.write_text(USER_PROGRAM)
    exe = tmp_path / "user"
    lib = B.facade_lib_path().parent
    root = lib.parent
    subprocess.run(["g++", "-std=c++17", "-I", str(root.parent / "include"), "-I", str(root / "cpp"), "-I",
                    str(root / "csrc"), str(src), "-o", str(exe), "-L", str(lib), "-lmuto_facade", "-lmuto_gb300",
                    f"-Wl,-rpath,{lib}"], check=True, capture_output=True, timeout=120)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split("\n")[:3] == ["0", str(tmp_path), "0"]


NLOHMANN_STYLE = r"""
#include <cstdio>
#include <string>
#include <vector>
#include "MutoConfig.h"
int main() {
    MutoConfig cfg;
    if (!cfg.loadString("{\"detector_middle\": 3, \"detector_height\": [1500.5, -1500],"
                        " \"output_file\": \"out.bin\", \"mlsd\": {\"early_stop\": true, \"eps\": 1e-8}}"))
        return 2;
    // the reference's driver reads its configuration this way (nlohmann's implicit conversions)
    int middle = cfg.get("detector_middle");
    std::vector<double> zs = cfg.get("detector_height");
    std::string out = cfg.get("output_file");
    bool stop = cfg.get("mlsd")["early_stop"];
    double eps = cfg.get("mlsd")["eps"];
    std::printf("%d %zu %.1f %.1f %s %d %.0e\n", middle, zs.size(), zs[0], zs[1], out.c_str(), stop ? 1 : 0, eps);
    return 0;
}
"""


def test_configuration_reads_like_nlohmann_json(tmp_path):
    # the implicit conversions a driver written for nlohmann::json relies on
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    root = B.facade_lib_path().parent.parent
    src = tmp_path / "cfg.cpp"
    src.write_text(NLOHMANN_STYLE)
    exe = tmp_path / "cfg"
    subprocess.run(["g++", "-std=c++17", "-I", str(root / "cpp"), "-I", str(root / "csrc"), str(src), "-o", str(exe)],
                   check=True, capture_output=True, timeout=120)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == ["3", "2", "1500.5", "-1500.0", "out.bin", "1", "1e-08"]


def test_fit_tracks_host_checks():
    # no records: nothing to fit, no device touched; a record of the wrong width is refused
    assert M.fit_tracks(np.zeros((0, 14)), Z, N_MIDDLE).shape == (0, 14)
    with pytest.raises(ValueError):
        M.fit_tracks(np.zeros((3, 13)), Z, N_MIDDLE)


UNPACK_PROGRAM = r"""
#include <cstdio>
#include "MutoSiddon.h"
int main() {
    const uint32_t xyz[9] = {1, 2, 3, 4, 5, 6, 7, 8, 9};
    const double len[3] = {0.5, 1.5, 2.5};
    bool failed = false;
    std::vector<VoxelData> a = MutoSiddon::unpackPath(2, 3, xyz, len, &failed);
    std::printf("%zu %d %u %u %u %.1f\n", a.size(), failed ? 1 : 0, a[1].x, a[1].y, a[1].z, a[1].length);
    std::vector<VoxelData> b = MutoSiddon::unpackPath(0xffffffffu, 3, xyz, len, &failed);
    std::printf("%zu %d\n", b.size(), failed ? 1 : 0);
    return 0;
}
"""


def test_siddon_facade_reports_a_walk_stopped_by_its_bound(facade, tmp_path):
    # a count of 0xffffffff from the device is a failed walk: an empty path
    # and a failure flag, not cap zero-filled voxels
    src = tmp_path / "unpack.cpp"
    src.write_text(UNPACK_PROGRAM)
    exe = tmp_path / "unpack"
    lib = B.facade_lib_path().parent
    root = lib.parent
    subprocess.run(["g++", "-std=c++17", "-I", str(root.parent / "include"), "-I", str(root / "cpp"), "-I",
                    str(root / "csrc"), str(src), "-o", str(exe), "-L", str(lib), "-lmuto_facade", "-lmuto_gb300",
                    f"-Wl,-rpath,{lib}"], check=True, capture_output=True, timeout=120)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split("\n")[:2] == ["2 0 4 5 6 1.5", "0 1"]


def test_reference_driver_compiles_unchanged(facade, tmp_path):
    # the reference's own command-line program, its source as it is, built
    # against this library's C++ headers and linked to its libraries: the
    # drop-in for the reconstruction classes, MutoConfig and MutoFile
    from oracle import reference as R

    if not R.available():
        pytest.skip("the reference's sources are not mounted here")
    lib = B.facade_lib_path().parent
    root = lib.parent
    exe = tmp_path / "muto_test"
    r = subprocess.run(["g++", "-std=c++17", "-I", str(root / "cpp"), "-I", str(root.parent / "include"), "-I",
                        str(root / "csrc"), str(R.REF / "MuToTest.cpp"), "-o", str(exe), "-L", str(lib),
                        "-lmuto_facade", "-lmuto_gb300", f"-Wl,-rpath,{lib}"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    assert exe.exists()
