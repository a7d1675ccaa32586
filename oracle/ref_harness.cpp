// C entry points over the reference's own reconstruction classes, compiled
// from its sources in place (src/MutoSiddon.cpp, src/MutoPoCA.cpp,
// src/MutoMLSD.cpp, src/MutoMAP.cpp, src/MutoPoCut.cpp, src/MutoSLR.cpp,
// src/MutoSLRIter.cpp) against the stand-in headers in
// oracle/ref_shim.  TEST INFRASTRUCTURE ONLY: used to generate the golden
// vectors under tests/golden/ and to cross-check oracle/muto_oracle.cpp.
//
// MutoFile.cpp (raw-hit reader + SVD) is not compiled; the one MutoFile
// function the path calls, loadImage (src/MutoMLSD.cpp:229), is provided here
// and returns the image handed to ref_set_initial_image.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "MutoFile.h"
#include "MutoMAP.h"
#include "MutoMLSD.h"
#include "MutoPoCA.h"
#include "MutoPoCut.h"
#include "MutoSLR.h"
#include "MutoSLRIter.h"
#include "MutoSiddon.h"

static_assert(sizeof(RayData) == 14 * sizeof(double), "RayData must be 14 doubles");

namespace {
Image g_init;
ImageHeader g_init_header;
bool g_init_set = false;

VoxelGrid to_grid(const uint32_t* n, const double* f) {
    VoxelGrid g;
    g.nx = n[0]; g.ny = n[1]; g.nz = n[2];
    g.x_min = f[0]; g.y_min = f[1]; g.z_min = f[2];
    g.dx = f[3]; g.dy = f[4]; g.dz = f[5];
    return g;
}

MutoMuonData to_rays(const double* r, uint64_t n) {
    MutoMuonData d(n);
    if (n) std::memcpy(&d[0], r, n * sizeof(RayData));
    return d;
}

// exposes the protected setup steps of MutoMLSD
struct Probe : public MutoMLSD {
    explicit Probe(json c) : MutoMLSD(c) {}
    void run(const MutoMuonData& rays, std::vector<uint32_t>& kept, std::vector<double>& info,
             std::vector<uint64_t>& off, std::vector<uint32_t>& idx, std::vector<double>& len,
             std::vector<double>& tail) {
        fNTotal = 0 < fNTotal ? fNTotal : rays.size();
        std::vector<MTindex> index;
        std::vector<MTfloat> sx, sy, dx, dy, p;
        std::vector<Vector3> scat;
        gatherInformation(rays, index, sx, dx, sy, dy, p, scat);
        MutoSiddon siddon(fGrid);
        std::vector<VoxelData> path;
        std::vector<MTfloat> tl;
        off.assign(1, 0);
        for (size_t i = 0; i < index.size(); ++i) {
            kept.push_back(index[i]);
            info.push_back(sx[i]);
            info.push_back(sy[i]);
            info.push_back(dx[i]);
            info.push_back(dy[i]);
            info.push_back(fHasEnergy ? p[i] : p[0]);
            info.push_back(0.0);
            getMuonPathAndTail(rays[index[i]], scat[i], path, tl, siddon);
            for (size_t k = 0; k < path.size(); ++k) {
                idx.push_back(xyz2index(path[k].x, path[k].y, path[k].z));
                len.push_back(path[k].length);
                tail.push_back(tl[k]);
            }
            off.push_back(idx.size());
        }
    }
};

template <typename T>
void copy_out(const std::vector<T>& v, T* dst) {
    if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(T));
}
}  // namespace

std::pair<Image, ImageHeader> MutoFile::loadImage(std::string) {
    if (!g_init_set) return std::pair<Image, ImageHeader>{};
    return std::pair<Image, ImageHeader>{g_init, g_init_header};
}

extern "C" {

void ref_set_initial_image(const double* img, const uint32_t* n, const double* f) {
    if (!img) {
        g_init_set = false;
        return;
    }
    g_init_header.grid = to_grid(n, f);
    g_init = Image(n[0], n[1], n[2]);
    std::memcpy(g_init.data(), img, sizeof(double) * n[0] * n[1] * n[2]);
    g_init_set = true;
}

int ref_siddon(const uint32_t* n, const double* f, const double* p1, const double* p2, uint64_t cnt, uint32_t cap,
               uint32_t* xyz, double* len, uint32_t* counts) {
    MutoSiddon s(to_grid(n, f));
    for (uint64_t r = 0; r < cnt; ++r) {
        Vector3 a, b;
        for (int k = 0; k < 3; ++k) {
            a(k) = p1[3 * r + k];
            b(k) = p2[3 * r + k];
        }
        std::vector<VoxelData> v = s.getVoxelPath(a, b);
        counts[r] = static_cast<uint32_t>(v.size());
        for (size_t k = 0; k < v.size() && k < cap; ++k) {
            xyz[3 * (r * cap + k) + 0] = v[k].x;
            xyz[3 * (r * cap + k) + 1] = v[k].y;
            xyz[3 * (r * cap + k) + 2] = v[k].z;
            len[r * cap + k] = v[k].length;
        }
    }
    return 0;
}

// method: "poca", "pocut", "slr", "slr_iter", "mlsd" or "map"; config: that
// method's JSON object.  out
// gets nx*ny*nz doubles of the grid the object ends with (out_n: its dims).
int ref_reconstruct(const char* method, const char* config, const double* rays, uint64_t n, double* out,
                    uint64_t cap, uint32_t* out_n) {
    const json cfg = json::parse(config);
    const MutoMuonData data = to_rays(rays, n);
    const std::string m(method);
    Image img;
    VoxelGrid g;
    if (m == "poca") {
        MutoPoCA r(cfg);
        img = r.reconstruct(data);
        g = r.getCurrentGrid();
    } else if (m == "pocut") {
        MutoPoCut r(cfg);
        img = r.reconstruct(data);
        g = r.getCurrentGrid();
    } else if (m == "slr") {
        MutoSLR r(cfg);
        img = r.reconstruct(data);
        g = r.getCurrentGrid();
    } else if (m == "slr_iter") {
        MutoSLRIter r(cfg);
        img = r.reconstruct(data);
        g = r.getCurrentGrid();
    } else if (m == "mlsd") {
        MutoMLSD r(cfg);
        img = r.reconstruct(data);
        g = r.getCurrentGrid();
    } else if (m == "map") {
        MutoMAP r(cfg);
        img = r.reconstruct(data);
        g = r.getCurrentGrid();
    } else {
        return -1;
    }
    out_n[0] = g.nx;
    out_n[1] = g.ny;
    out_n[2] = g.nz;
    if (static_cast<uint64_t>(img.size()) > cap) return -2;
    std::memcpy(out, img.data(), sizeof(double) * img.size());
    return 0;
}

// MLSD setup: kept muons, per-muon info and merged paths; call once with null
// outputs to get the sizes (sizes[0] = kept, sizes[1] = pairs).
int ref_mlsd_paths(const char* config, const double* rays, uint64_t n, uint64_t* sizes, uint32_t* kept, double* info,
                   uint64_t* off, uint32_t* idx, double* len, double* tail) {
    Probe p(json::parse(config));
    std::vector<uint32_t> k, ix;
    std::vector<double> in, ln, tl;
    std::vector<uint64_t> of;
    p.run(to_rays(rays, n), k, in, of, ix, ln, tl);
    sizes[0] = k.size();
    sizes[1] = ix.size();
    copy_out(k, kept);
    copy_out(in, info);
    copy_out(of, off);
    copy_out(ix, idx);
    copy_out(ln, len);
    copy_out(tl, tail);
    return 0;
}

}  // extern "C"
