// C entry points over the reference's own MutoFile (src/MutoFile.cpp: the
// raw-hit reader with its per-record SVD line fit, and the image files),
// compiled from its source in place against the stand-in headers in
// oracle/ref_shim.  TEST INFRASTRUCTURE ONLY: used to generate the golden
// vectors of tests/golden/files.npz and to cross-check the library's reader
// and image format with the reference itself.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "MutoFile.h"

static_assert(sizeof(RayData) == 14 * sizeof(double), "RayData must be 14 doubles");

extern "C" {

// MutoFile::getMuonData over one file; returns the number of tracks and
// writes at most cap of them (14 doubles each) to out.
uint64_t ref_read_muon_data(const char* path, const double* z, int nz, int n_middle, int precision, double* out,
                            uint64_t cap) {
    std::vector<std::string> files(1, std::string(path));
    std::vector<MTfloat> zl(z, z + nz);
    MutoMuonData d = MutoFile::getMuonData(files, zl, n_middle, precision);
    for (uint64_t i = 0; i < d.size() && i < cap; ++i) std::memcpy(out + 14 * i, &d[i], sizeof(RayData));
    return d.size();
}

// MutoFile::saveImage; n = {nx, ny, nz}, f = {x_min, y_min, z_min, dx, dy, dz}.
int ref_save_image(const char* path, const double* img, const uint32_t* n, const double* f, const char* method,
                   uint32_t n_ray, uint32_t n_iter, uint32_t precision) {
    ImageHeader h;
    h.method = method;
    h.grid.nx = n[0];
    h.grid.ny = n[1];
    h.grid.nz = n[2];
    h.grid.x_min = f[0];
    h.grid.y_min = f[1];
    h.grid.z_min = f[2];
    h.grid.dx = f[3];
    h.grid.dy = f[4];
    h.grid.dz = f[5];
    h.nRay = n_ray;
    h.nIter = n_iter;
    h.fPrecision = precision;
    Image im(n[0], n[1], n[2]);
    std::memcpy(im.data(), img, sizeof(double) * n[0] * n[1] * n[2]);
    return MutoFile::saveImage(im, h, path) ? 0 : 1;
}

// MutoFile::loadImage; the header's fields as ref_save_image takes them.
int ref_load_image(const char* path, double* img, uint64_t cap, uint32_t* n, double* f, char* method16,
                   uint32_t* n_ray, uint32_t* n_iter, uint32_t* precision) {
    std::pair<Image, ImageHeader> r = MutoFile::loadImage(path);
    const ImageHeader& h = r.second;
    n[0] = h.grid.nx;
    n[1] = h.grid.ny;
    n[2] = h.grid.nz;
    f[0] = h.grid.x_min;
    f[1] = h.grid.y_min;
    f[2] = h.grid.z_min;
    f[3] = h.grid.dx;
    f[4] = h.grid.dy;
    f[5] = h.grid.dz;
    std::memset(method16, 0, 16);
    std::memcpy(method16, h.method.data(), h.method.size() < 16 ? h.method.size() : 16);
    *n_ray = h.nRay;
    *n_iter = h.nIter;
    *precision = h.fPrecision;
    const uint64_t V = static_cast<uint64_t>(r.first.size());
    for (uint64_t i = 0; i < V && i < cap; ++i) img[i] = r.first(static_cast<Index>(i));
    return V > 0 ? 0 : 1;
}

}  // extern "C"
