// MutoSiddon over muto_siddon_batch.  See MutoSiddon.h.
#include "MutoSiddon.h"

#include <algorithm>
#include <cstdint>
#include <iostream>

#include "muto_gb300.h"

std::vector<VoxelData> MutoSiddon::getVoxelPath(const Vector3& p1, const Vector3& p2) {
    std::vector<std::vector<VoxelData>> r = getVoxelPaths(std::vector<Vector3>(1, p1), std::vector<Vector3>(1, p2));
    return r.empty() ? std::vector<VoxelData>() : r[0];
}

std::vector<std::vector<VoxelData>> MutoSiddon::getVoxelPaths(const std::vector<Vector3>& p1,
                                                              const std::vector<Vector3>& p2) {
    std::vector<std::vector<VoxelData>> out;
    if (p1.size() != p2.size()) {
        std::cout << "MutoSiddon: " << p1.size() << " start points for " << p2.size() << " end points. " << std::endl;
        return out;
    }
    out.resize(p1.size());
    muto_grid g{};
    g.nx = fGrid.nx;
    g.ny = fGrid.ny;
    g.nz = fGrid.nz;
    g.x_min = fGrid.x_min;
    g.y_min = fGrid.y_min;
    g.z_min = fGrid.z_min;
    g.dx = fGrid.dx;
    g.dy = fGrid.dy;
    g.dz = fGrid.dz;
    // a walk crosses at most nx + ny + nz voxels; segments go in chunks that
    // keep the staged lists near 64 MB
    const uint64_t cap64 = static_cast<uint64_t>(g.nx) + g.ny + g.nz + 8;
    const uint32_t cap = static_cast<uint32_t>(std::min<uint64_t>(cap64, 0xffffffffull));
    const uint64_t per = std::max<uint64_t>(1, (uint64_t(64) << 20) / (cap * 20));
    std::vector<double> a, b, len;
    std::vector<uint32_t> xyz, cnt;
    for (size_t s0 = 0; s0 < p1.size(); s0 += per) {
        const size_t n = static_cast<size_t>(std::min<uint64_t>(per, p1.size() - s0));
        a.resize(3 * n);
        b.resize(3 * n);
        for (size_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) {
                a[3 * i + k] = p1[s0 + i](k);
                b[3 * i + k] = p2[s0 + i](k);
            }
        xyz.assign(3 * n * cap, 0);
        len.assign(n * cap, 0.0);
        cnt.assign(n, 0);
        const int rc = muto_siddon_batch(&g, a.data(), b.data(), n, cap, xyz.data(), len.data(), cnt.data());
        if (rc != MUTO_OK) {
            std::cout << "MutoSiddon: the voxel walk failed (error " << rc << "). " << std::endl;
            out.clear();
            return out;
        }
        for (size_t i = 0; i < n; ++i) {
            bool failed = false;
            out[s0 + i] = unpackPath(cnt[i], cap, xyz.data() + 3 * i * cap, len.data() + i * cap, &failed);
            if (failed)
                std::cout << "MutoSiddon: the walk of segment " << s0 + i
                          << " stopped at its step bound; its path is left empty. " << std::endl;
        }
    }
    return out;
}

std::vector<VoxelData> MutoSiddon::unpackPath(uint32_t count, uint32_t cap, const uint32_t* xyz, const double* len,
                                              bool* failed) {
    std::vector<VoxelData> v;
    if (count == 0xffffffffu) {  // the device marks a walk that hit its step bound
        if (failed) *failed = true;
        return v;
    }
    const uint32_t k = std::min(count, cap);
    v.resize(k);
    for (uint32_t j = 0; j < k; ++j) {
        v[j].x = xyz[3 * j];
        v[j].y = xyz[3 * j + 1];
        v[j].z = xyz[3 * j + 2];
        v[j].length = len[j];
    }
    return v;
}
