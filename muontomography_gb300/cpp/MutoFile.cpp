// MutoFile: raw-hit reader and image files.  See MutoFile.h.
#include "MutoFile.h"

#include <unistd.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>

#include "muto_gb300.h"
#include "trackfit.h"

namespace {

std::string start_dir() {
    char buf[PATH_MAX];
    return getcwd(buf, sizeof(buf)) ? std::string(buf) : std::string();
}
const std::string g_start_dir = start_dir();

muto_grid to_c(const VoxelGrid& g) {
    muto_grid c{};
    c.nx = g.nx;
    c.ny = g.ny;
    c.nz = g.nz;
    c.x_min = g.x_min;
    c.y_min = g.y_min;
    c.z_min = g.z_min;
    c.dx = g.dx;
    c.dy = g.dy;
    c.dz = g.dz;
    return c;
}

// Reads each file's whole records, a chunk of at most 2^20 at a time, and
// hands them to f(raw bytes, number of records); a file that cannot be
// opened is reported and skipped (src/MutoFile.cpp:42-48).  Sizes are 64-bit.
template <class F>
void read_records(const std::vector<std::string>& flist, size_t rec_bytes, F&& f) {
    const uint64_t chunk = uint64_t(1) << 20;
    std::vector<char> raw;
    for (const std::string& name : flist) {
        std::ifstream file(name.c_str(), std::ios::in | std::ios::binary);
        if (file.fail()) {
            std::cout << "Reading muon data error for : " << name << std::endl;
            continue;
        }
        file.seekg(0, std::ios::end);
        const uint64_t filesize = static_cast<uint64_t>(file.tellg());
        file.seekg(0, std::ios::beg);
        const uint64_t nRay = filesize / rec_bytes;
        for (uint64_t r0 = 0; r0 < nRay; r0 += chunk) {
            const uint64_t m = std::min(chunk, nRay - r0);
            raw.resize(static_cast<size_t>(m * rec_bytes));
            file.read(raw.data(), static_cast<std::streamsize>(raw.size()));
            const uint64_t got = static_cast<uint64_t>(file.gcount()) / rec_bytes;  // whole records read
            if (got) f(raw.data(), got);
            if (got < m) break;
        }
    }
}

void to_doubles(const char* raw, size_t n, int precision, double* out) {
    for (size_t k = 0; k < n; ++k) {
        if (precision == 4) {
            float v;
            std::memcpy(&v, raw + 4 * k, 4);
            out[k] = v;
        } else {
            std::memcpy(&out[k], raw + 8 * k, 8);
        }
    }
}

}  // namespace

std::string MutoFile::getCurrentPath() { return g_start_dir; }

void MutoFile::fitLine(const double* x, const double* y, const double* z, int n, double* c, double* d) {
    muto::fit::fit_line(x, y, z, n, c, d);
}

MutoMuonData MutoFile::getMuonData(std::vector<std::string> flist, std::vector<MTfloat> zlayers, int nMiddle,
                                   int fPrecision) {
    MutoMuonData data;
    if (fPrecision != 4 && fPrecision != 8) {
        std::cerr << "Floating point precision not supported. " << std::endl;
        return data;
    }
    const int nz = static_cast<int>(zlayers.size());
    if (nMiddle < 2 || nz - nMiddle < 2) {
        std::cerr << "Error: at least two layers of detectors for both up and down area. " << std::endl;
        return data;
    }
    if (nz > muto::fit::kMaxLayers) {
        std::cerr << "Error: at most " << muto::fit::kMaxLayers << " layers of detectors. " << std::endl;
        return data;
    }
    const size_t nEach = 2 * static_cast<size_t>(nz) + 2;  // two extra values for in and out energy
    std::vector<muto_ray> fitted;
    std::vector<unsigned char> keep;
    read_records(flist, nEach * static_cast<size_t>(fPrecision), [&](const char* raw, uint64_t n) {
        // records are independent: each thread fits its own share, the kept
        // tracks are then appended in record order
        fitted.resize(n);
        keep.resize(n);
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < static_cast<long long>(n); ++i) {
            double rec[2 * muto::fit::kMaxLayers + 2];
            to_doubles(raw + static_cast<size_t>(i) * nEach * static_cast<size_t>(fPrecision), nEach, fPrecision,
                       rec);
            keep[i] = muto::fit::fit_record(rec, zlayers.data(), nz, nMiddle, &fitted[i]) ? 1 : 0;  // 0: a NaN
        }
        static_assert(sizeof(RayData) == sizeof(muto_ray), "RayData mirrors muto_ray");
        if (data.capacity() < data.size() + n) data.reserve(std::max<size_t>(2 * data.capacity(), data.size() + n));
        for (uint64_t i = 0; i < n; ++i) {
            if (!keep[i]) continue;
            RayData ray;
            std::memcpy(&ray, &fitted[i], sizeof(muto_ray));
            data.push_back(ray);
        }
    });
    return data;
}

bool MutoFile::saveImage(const Image& img, const ImageHeader& header, std::string filename) {
    const muto_grid g = to_c(header.grid);
    if (static_cast<uint64_t>(img.size()) != static_cast<uint64_t>(g.nx) * g.ny * g.nz) {
        std::cout << "Writing image to file: " << filename << " failed (size does not match the grid). " << std::endl;
        return false;
    }
    const int rc = muto_save_image(filename.c_str(), img.data(), &g, header.method.c_str(), header.nRay, header.nIter,
                                   header.fPrecision);
    if (rc == MUTO_ERR_ARG) std::cout << "Floating point precision not supported. " << std::endl;
    else if (rc != MUTO_OK) std::cout << "Writing image to file: " << filename << " failed. " << std::endl;
    return rc == MUTO_OK;
}

bool MutoFile::saveImagePure(const Image& img, std::string filename, MTindex fPrecision) {
    if (fPrecision != 4 && fPrecision != 8) {
        std::cout << "Floating point precision not supported. " << std::endl;
        return false;
    }
    FILE* f = std::fopen(filename.c_str(), "wb");
    if (!f) {
        std::cout << "Writing image to file: " << filename << " failed. " << std::endl;
        return false;
    }
    bool ok = true;
    for (std::ptrdiff_t i = 0; i < img.size() && ok; ++i) {
        if (fPrecision == 8) {
            const double v = img(i);
            ok = std::fwrite(&v, 8, 1, f) == 1;
        } else {
            const float v = static_cast<float>(img(i));
            ok = std::fwrite(&v, 4, 1, f) == 1;
        }
    }
    return (std::fclose(f) == 0) && ok;
}

std::pair<Image, ImageHeader> MutoFile::loadImage(std::string filename) {
    muto_grid g{};
    char method[17] = {0};
    uint32_t nRay = 0, nIter = 0, prec = 0;
    if (muto_load_image(filename.c_str(), nullptr, 0, &g, method, &nRay, &nIter, &prec) != MUTO_OK) {
        std::cout << "Reading image file: " << filename << " failed. " << std::endl;
        return std::pair<Image, ImageHeader>{};
    }
    Image img(g.nx, g.ny, g.nz);
    if (muto_load_image(filename.c_str(), img.data(), static_cast<uint64_t>(img.size()), &g, method, &nRay, &nIter,
                        &prec) != MUTO_OK) {
        std::cout << "Reading image file: " << filename << " failed. " << std::endl;
        return std::pair<Image, ImageHeader>{};
    }
    ImageHeader h;
    h.method = std::string(method, strnlen(method, 16));
    h.grid = VoxelGrid{g.nx, g.ny, g.nz, g.x_min, g.y_min, g.z_min, g.dx, g.dy, g.dz};
    h.nRay = nRay;
    h.nIter = nIter;
    h.fPrecision = prec;
    return std::pair<Image, ImageHeader>{img, h};
}

Image MutoFile::loadImagePure(std::string filename, VoxelGrid grid, MTindex fPrecision) {
    std::ifstream file(filename.c_str(), std::ios::in | std::ios::binary);
    if (file.fail()) {
        std::cout << "Reading image file: " << filename << " failed. " << std::endl;
        return Image{};
    }
    if (fPrecision != 4 && fPrecision != 8) {
        std::cout << "Floating point precision not supported. " << std::endl;
        return Image{};
    }
    file.seekg(0, std::ios::end);
    const uint64_t size = static_cast<uint64_t>(file.tellg());
    file.seekg(0, std::ios::beg);
    const uint64_t V = static_cast<uint64_t>(grid.nx) * grid.ny * grid.nz;
    if (V * fPrecision != size) {
        std::cout << "Wrong size of the image file and grid: " << filename << std::endl;
        return Image{};
    }
    Image img(grid.nx, grid.ny, grid.nz);
    for (uint64_t i = 0; i < V; ++i) {
        if (fPrecision == 8) {
            file.read(reinterpret_cast<char*>(&img(static_cast<std::ptrdiff_t>(i))), 8);
        } else {
            float f;
            file.read(reinterpret_cast<char*>(&f), 4);
            img(static_cast<std::ptrdiff_t>(i)) = f;
        }
    }
    return img;
}

// ---------------------------------------------------------------------------
// C entry (include/muto_io.h)
// ---------------------------------------------------------------------------
#include "muto_io.h"

extern "C" int muto_read_muon_data(const char* const* files, int n_files, const double* z_layers, int nz,
                                   int n_middle, int precision, muto_ray* out, uint64_t cap, uint64_t* n_out) {
    if (!n_out || (n_files > 0 && !files) || nz <= 0 || !z_layers) return MUTO_ERR_ARG;
    if (precision != 4 && precision != 8) return MUTO_ERR_ARG;
    if (n_middle < 2 || nz - n_middle < 2 || nz > muto::fit::kMaxLayers) return MUTO_ERR_ARG;
    std::vector<std::string> fl;
    for (int i = 0; i < n_files; ++i) fl.push_back(files[i] ? files[i] : "");
    if (!out) {  // count the records without a NaN, fitting nothing
        const size_t each = 2 * static_cast<size_t>(nz) + 2;
        uint64_t kept = 0;
        read_records(fl, each * static_cast<size_t>(precision), [&](const char* raw, uint64_t n) {
            uint64_t k = 0;
#pragma omp parallel for schedule(static) reduction(+ : k)
            for (long long i = 0; i < static_cast<long long>(n); ++i) {
                double rec[2 * muto::fit::kMaxLayers + 2];
                to_doubles(raw + static_cast<size_t>(i) * each * static_cast<size_t>(precision), each, precision, rec);
                bool nan = false;
                for (size_t j = 0; j < each; ++j) nan = nan || rec[j] != rec[j];
                k += nan ? 0 : 1;
            }
            kept += k;
        });
        *n_out = kept;
        return MUTO_OK;
    }
    const std::vector<MTfloat> z(z_layers, z_layers + nz);
    const MutoMuonData d = MutoFile::getMuonData(fl, z, n_middle, precision);
    const uint64_t n = d.size() < cap ? d.size() : cap;
    if (n) std::memcpy(out, d.data(), n * sizeof(muto_ray));
    *n_out = n;
    return MUTO_OK;
}
