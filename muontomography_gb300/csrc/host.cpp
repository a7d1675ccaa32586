// Host side of the library: synthetic muon data and the MutoFile image format.
//
// Synthetic data.  Every muon is generated from its own counter-based random
// stream (SplitMix64 keyed by seed and muon index), so a muon is the same
// whatever the thread count or the chunk it is generated in.
//   zenith   cos^2(theta) sin(theta) on [0, theta_max): cos^3(theta) is uniform
//   azimuth  uniform;  momentum log-uniform on [p_min, p_max]
//   entry    uniform over the grid's x-y footprint on its top face
//   transport one step per traversed voxel; per step of length L through
//            lambda, Gaussian (angle, displacement) kicks in the x and y planes
//            with covariance lambda (p0/p)^2 L [[1, L/2], [L/2, L^2/3]]
//   detectors n_planes planes above and below the grid at plane_gap spacing,
//            the inner planes on the grid's top and bottom faces; hits smeared
//            by hit_sigma; in/out lines by least squares, stored with d_z > 0,
//            pin / pout on the inner planes (as the reference's reader places them,
//            src/MutoFile.cpp:248-304).
//
// Image files.  saveImage / loadImage of src/MutoFile.cpp:85-211: a 64-byte
// header {u8 length=64, u8 version=1, char method[16], u32 nRay, u16 nIter,
// u16 precision, u16 nx, ny, nz, f32 x_min, y_min, z_min, dx, dy, dz, 8 zero
// bytes} followed by the column-major image as f32 (precision 4) or f64 (8),
// little-endian.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/muto_gb300.h"
#include "gen.h"

namespace {

void put_u16(unsigned char* p, uint32_t v) {
    p[0] = static_cast<unsigned char>(v & 0xff);
    p[1] = static_cast<unsigned char>((v >> 8) & 0xff);
}
void put_u32(unsigned char* p, uint32_t v) {
    for (int k = 0; k < 4; ++k) p[k] = static_cast<unsigned char>((v >> (8 * k)) & 0xff);
}
uint32_t get_u16(const unsigned char* p) { return static_cast<uint32_t>(p[0]) | (static_cast<uint32_t>(p[1]) << 8); }
uint32_t get_u32(const unsigned char* p) {
    return static_cast<uint32_t>(p[0]) | (static_cast<uint32_t>(p[1]) << 8) | (static_cast<uint32_t>(p[2]) << 16) |
           (static_cast<uint32_t>(p[3]) << 24);
}
void put_f32(unsigned char* p, float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    put_u32(p, u);
}
float get_f32(const unsigned char* p) {
    const uint32_t u = get_u32(p);
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

}  // namespace

extern "C" {

double muto_lambda_from_x0(double x0_mm, double p0_gev) {
    const double a = 0.0136 / p0_gev;  // 13.6 MeV / p0
    return a * a / x0_mm;
}

int muto_phantom(const muto_grid* g, const muto_block* blocks, uint32_t n_blocks, double background_x0_mm,
                 double p0_gev, double* out) {
    if (!g || !out || (n_blocks && !blocks) || !(p0_gev > 0) || !(background_x0_mm > 0)) return MUTO_ERR_ARG;
    const double bg = muto_lambda_from_x0(background_x0_mm, p0_gev);
    for (uint32_t z = 0; z < g->nz; ++z)
        for (uint32_t y = 0; y < g->ny; ++y)
            for (uint32_t x = 0; x < g->nx; ++x) {
                const double c[3] = {g->x_min + (x + 0.5) * g->dx, g->y_min + (y + 0.5) * g->dy,
                                     g->z_min + (z + 0.5) * g->dz};
                double v = bg;
                for (uint32_t b = 0; b < n_blocks; ++b) {
                    bool in = true;
                    for (int k = 0; k < 3; ++k) in = in && blocks[b].lo[k] <= c[k] && c[k] < blocks[b].hi[k];
                    if (in) v = muto_lambda_from_x0(blocks[b].x0_mm, p0_gev);
                }
                out[x + static_cast<uint64_t>(g->nx) * (y + static_cast<uint64_t>(g->ny) * z)] = v;
            }
    return MUTO_OK;
}

int muto_generate(const muto_grid* g, const double* lambda, const muto_gen_params* prm, uint64_t first, uint64_t n,
                  muto_ray* out) {
    if (!g || !lambda || !prm || (n && !out)) return MUTO_ERR_ARG;
    if (!muto::gen::params_ok(*prm)) return MUTO_ERR_ARG;
#pragma omp parallel for schedule(dynamic, 1024)
    for (long long ii = 0; ii < static_cast<long long>(n); ++ii)
        muto::gen::generate_one(*g, lambda, *prm, first + static_cast<uint64_t>(ii), out[ii]);
    return MUTO_OK;
}

int muto_save_image(const char* path, const double* img, const muto_grid* g, const char* method, uint32_t n_ray,
                    uint32_t n_iter, uint32_t precision) {
    if (!path || !img || !g) return MUTO_ERR_ARG;
    if (precision != 4 && precision != 8) return MUTO_ERR_ARG;  // src/MutoFile.cpp:190-198
    unsigned char h[64];
    std::memset(h, 0, sizeof h);
    h[0] = 64;
    h[1] = 1;
    if (method) {
        const size_t n = std::min<size_t>(std::strlen(method), 16);
        std::memcpy(h + 2, method, n);
    }
    put_u32(h + 18, n_ray);
    put_u16(h + 22, n_iter);
    put_u16(h + 24, precision);
    put_u16(h + 26, g->nx);
    put_u16(h + 28, g->ny);
    put_u16(h + 30, g->nz);
    put_f32(h + 32, static_cast<float>(g->x_min));
    put_f32(h + 36, static_cast<float>(g->y_min));
    put_f32(h + 40, static_cast<float>(g->z_min));
    put_f32(h + 44, static_cast<float>(g->dx));
    put_f32(h + 48, static_cast<float>(g->dy));
    put_f32(h + 52, static_cast<float>(g->dz));
    FILE* f = std::fopen(path, "wb");
    if (!f) return MUTO_ERR_IO;
    bool ok = std::fwrite(h, 1, 64, f) == 64;
    const uint64_t V = static_cast<uint64_t>(g->nx) * g->ny * g->nz;
    std::vector<unsigned char> buf(V * precision);
    for (uint64_t j = 0; j < V; ++j) {
        if (precision == 4) {
            put_f32(&buf[4 * j], static_cast<float>(img[j]));
        } else {
            uint64_t u;
            std::memcpy(&u, &img[j], 8);
            for (int k = 0; k < 8; ++k) buf[8 * j + k] = static_cast<unsigned char>((u >> (8 * k)) & 0xff);
        }
    }
    ok = ok && std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? MUTO_OK : MUTO_ERR_IO;
}

int muto_load_image(const char* path, double* img, uint64_t cap, muto_grid* g, char* method16, uint32_t* n_ray,
                    uint32_t* n_iter, uint32_t* precision) {
    if (!path) return MUTO_ERR_ARG;
    FILE* f = std::fopen(path, "rb");
    if (!f) return MUTO_ERR_IO;
    unsigned char h[64];
    if (std::fread(h, 1, 56, f) != 56) {
        std::fclose(f);
        return MUTO_ERR_IO;
    }
    muto_grid gg{};
    gg.nx = get_u16(h + 26);
    gg.ny = get_u16(h + 28);
    gg.nz = get_u16(h + 30);
    gg.x_min = get_f32(h + 32);
    gg.y_min = get_f32(h + 36);
    gg.z_min = get_f32(h + 40);
    gg.dx = get_f32(h + 44);
    gg.dy = get_f32(h + 48);
    gg.dz = get_f32(h + 52);
    const uint32_t prec = get_u16(h + 24);
    if (g) *g = gg;
    if (method16) std::memcpy(method16, h + 2, 16);
    if (n_ray) *n_ray = get_u32(h + 18);
    if (n_iter) *n_iter = get_u16(h + 22);
    if (precision) *precision = prec;
    const uint64_t V = static_cast<uint64_t>(gg.nx) * gg.ny * gg.nz;
    int rc = MUTO_OK;
    if (img) {
        if (cap < V || (prec != 4 && prec != 8)) {
            rc = cap < V ? MUTO_ERR_CAPACITY : MUTO_ERR_IO;
        } else if (std::fseek(f, h[0], SEEK_SET) != 0) {  // data starts at `length` (src/MutoFile.cpp:258)
            rc = MUTO_ERR_IO;
        } else {
            std::vector<unsigned char> buf(V * prec);
            if (std::fread(buf.data(), 1, buf.size(), f) != buf.size()) {
                rc = MUTO_ERR_IO;
            } else {
                for (uint64_t j = 0; j < V; ++j) {
                    if (prec == 4) {
                        img[j] = static_cast<double>(get_f32(&buf[4 * j]));
                    } else {
                        uint64_t u = 0;
                        for (int k = 0; k < 8; ++k) u |= static_cast<uint64_t>(buf[8 * j + k]) << (8 * k);
                        std::memcpy(&img[j], &u, 8);
                    }
                }
            }
        }
    }
    std::fclose(f);
    return rc;
}

}  // extern "C"
