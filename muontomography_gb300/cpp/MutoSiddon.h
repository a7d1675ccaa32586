// Siddon voxel walk of the reference's API (include/MutoSiddon.h:12-25), on
// the GPU through muto_siddon_batch (include/muto_gb300.h): the voxels a
// segment crosses, in walk order, with their lengths (src/MutoSiddon.cpp:
// 9-141, bit for bit).  getVoxelPaths walks many segments in one call; a
// single getVoxelPath is one device round trip, so loops over segments
// belong in getVoxelPaths.
#pragma once

#include <cstdint>
#include <vector>

#include "MutoTypes.h"

class MutoSiddon {
public:
    explicit MutoSiddon(const VoxelGrid& grid) : fGrid(grid) {}
    ~MutoSiddon() {}

    // The voxels crossed from p1 to p2 (empty when the segment misses the grid
    // or a device call fails; failures are printed).
    std::vector<VoxelData> getVoxelPath(const Vector3& p1, const Vector3& p2);

    // Segment i runs from p1[i] to p2[i]; out[i] is its path.
    std::vector<std::vector<VoxelData>> getVoxelPaths(const std::vector<Vector3>& p1, const std::vector<Vector3>& p2);

    // One segment's path from muto_siddon_batch's slots: count voxels (at
    // most cap kept) from xyz (3 per voxel) and len.  A count of 0xffffffff
    // marks a walk stopped by its step bound: the path is then empty and
    // *failed is set (it is never set otherwise).
    static std::vector<VoxelData> unpackPath(uint32_t count, uint32_t cap, const uint32_t* xyz, const double* len,
                                             bool* failed);

private:
    VoxelGrid fGrid;
};
