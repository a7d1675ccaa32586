// The level schedule of SLRIter's in-place passes (src/MutoSLRIter.cpp:40-71).
//
// Muon i's level is one more than the highest level that an earlier muon
// left on any voxel of i's path.  A voxel's muons then have strictly
// increasing levels in index order, and two muons of one level share no
// voxel: running the muons of a level at once, level after level, gives
// every muon the image state of the muon-after-muon loop.  One ordered sweep
// over the pairs; the recurrence is sequential in the muon index.  Plain C++
// (host code, no CUDA types).
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

namespace muto {

// off[0..nt]: each muon's pairs vox[off[i] .. off[i+1]); voxels >= V are
// ignored.  Fills level[0..nt) (1-based) and returns the number of levels.
inline uint32_t slr_levels(const uint64_t* off, const uint32_t* vox, uint64_t nt, uint64_t V, uint32_t* level) {
    std::vector<uint32_t> last(V, 0);
    uint32_t levels = 0;
    for (uint64_t i = 0; i < nt; ++i) {
        uint32_t lv = 0;
        for (uint64_t k = off[i]; k < off[i + 1]; ++k)
            if (vox[k] < V) lv = std::max(lv, last[vox[k]]);
        ++lv;
        for (uint64_t k = off[i]; k < off[i + 1]; ++k)
            if (vox[k] < V) last[vox[k]] = lv;
        level[i] = lv;
        levels = std::max(levels, lv);
    }
    return levels;
}

}  // namespace muto
