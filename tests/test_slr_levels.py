"""CPU test of SLRIter's level schedule (muontomography_gb300/csrc/slr_levels.h),
the host recurrence behind the level-by-level passes of
src/MutoSLRIter.cpp:40-71: compiled with g++ into a small program and run on
random paths.  The schedule must (1) give a voxel's muons strictly
increasing levels in index order and (2) put no two muons that share a voxel
in one level -- together, running a level's muons at once gives every muon
the image the muon-after-muon loop would give it -- and (3) be the lowest
such levels (each muon one above the highest level already on its voxels)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "muontomography_gb300" / "csrc" / "slr_levels.h"

HARNESS = r"""
#include <cstdio>
#include <vector>
#include "slr_levels.h"
int main() {
    unsigned long long nt = 0, np = 0, V = 0;
    if (std::scanf("%llu %llu %llu", &nt, &np, &V) != 3) return 2;
    std::vector<uint64_t> off(nt + 1);
    std::vector<uint32_t> vox(np), level(nt);
    for (auto& o : off) { unsigned long long x; if (std::scanf("%llu", &x) != 1) return 2; o = x; }
    for (auto& v : vox) { unsigned x; if (std::scanf("%u", &x) != 1) return 2; v = x; }
    const uint32_t L = muto::slr_levels(off.data(), vox.data(), nt, V, level.data());
    std::printf("%u\n", L);
    for (auto l : level) std::printf("%u\n", l);
    return 0;
}
"""


@pytest.fixture(scope="module")
def levels_exe(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    d = tmp_path_factory.mktemp("slr_levels")
    (d / "main.cpp").write_text(HARNESS)
    exe = d / "levels"
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{HEADER.parent}", str(d / "main.cpp"), "-o", str(exe)], check=True)
    return exe


def run_levels(exe, off, vox, V):
    text = f"{len(off) - 1} {len(vox)} {V}\n" + " ".join(map(str, off)) + "\n" + " ".join(map(str, vox)) + "\n"
    out = subprocess.run([str(exe)], input=text, capture_output=True, text=True, check=True).stdout.split()
    return int(out[0]), np.array([int(x) for x in out[1:]], np.int64)


def random_paths(rng, nt, V, max_len):
    lens = rng.integers(0, max_len + 1, nt)
    off = np.concatenate([[0], np.cumsum(lens)])
    # each path distinct voxels (a straight line visits a voxel once); a few out-of-grid entries
    vox = np.concatenate([rng.choice(V + 2, size=n, replace=False) for n in lens]) if off[-1] else np.zeros(0, int)
    return off, vox


@pytest.mark.parametrize("nt,V,max_len,seed", [(200, 50, 6, 1), (2000, 400, 12, 2), (500, 8, 3, 3), (1, 5, 4, 4),
                                               (300, 1000, 0, 5)])
def test_level_schedule(levels_exe, nt, V, max_len, seed):
    rng = np.random.default_rng(seed)
    off, vox = random_paths(rng, nt, V, max_len)
    L, level = run_levels(levels_exe, off, vox, V)
    assert level.shape == (nt,) and L == (level.max() if nt else 0)
    last = np.zeros(V, np.int64)
    seen_in_level = {}
    for i in range(nt):
        path = [v for v in vox[off[i]:off[i + 1]] if v < V]
        want = 1 + max((last[v] for v in path), default=0)
        assert level[i] == want  # the lowest level after every earlier muon on its voxels
        for v in path:
            assert last[v] < level[i]  # strictly increasing along each voxel's muons
            key = (level[i], v)
            assert key not in seen_in_level  # no voxel shared inside a level
            seen_in_level[key] = i
            last[v] = level[i]
    if max_len == 0:
        assert L == 1 and np.all(level == 1)  # empty paths: one level
