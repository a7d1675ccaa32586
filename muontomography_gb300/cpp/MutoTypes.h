// Types of the reconstruction API (the reference's include/MutoTypes.h:1-64),
// without Eigen: a 3-vector, a column-major 3-D image, and the plain structs.
// RayData keeps the reference's memory layout (14 doubles) so a
// MutoMuonData buffer is passed to the GPU library as is.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

typedef double MTfloat;
typedef unsigned int MTindex;

// Row 3-vector (Eigen Matrix<double,1,3> in the reference)
struct Vector3 {
    MTfloat v[3];
    Vector3() : v{0.0, 0.0, 0.0} {}
    Vector3(MTfloat x, MTfloat y, MTfloat z) : v{x, y, z} {}
    MTfloat& operator()(int i) { return v[i]; }
    MTfloat operator()(int i) const { return v[i]; }
    MTfloat dot(const Vector3& o) const { return (v[0] * o.v[0] + v[1] * o.v[1]) + v[2] * o.v[2]; }
};

// 3-D image, column-major (x fastest) like Eigen::Tensor<double, 3>
class Image {
public:
    Image() : n_{0, 0, 0} {}
    Image(std::ptrdiff_t nx, std::ptrdiff_t ny, std::ptrdiff_t nz)
        : n_{nx, ny, nz}, d_(static_cast<size_t>(nx * ny * nz), 0.0) {}
    MTfloat& operator()(std::ptrdiff_t i) { return d_[static_cast<size_t>(i)]; }
    MTfloat operator()(std::ptrdiff_t i) const { return d_[static_cast<size_t>(i)]; }
    MTfloat& operator()(std::ptrdiff_t x, std::ptrdiff_t y, std::ptrdiff_t z) { return d_[idx(x, y, z)]; }
    MTfloat operator()(std::ptrdiff_t x, std::ptrdiff_t y, std::ptrdiff_t z) const { return d_[idx(x, y, z)]; }
    std::ptrdiff_t size() const { return static_cast<std::ptrdiff_t>(d_.size()); }
    std::ptrdiff_t dimension(int k) const { return n_[k]; }
    MTfloat* data() { return d_.data(); }
    const MTfloat* data() const { return d_.data(); }
    void setZero() { setConstant(0.0); }
    void setConstant(MTfloat v) {
        for (auto& x : d_) x = v;
    }

private:
    size_t idx(std::ptrdiff_t x, std::ptrdiff_t y, std::ptrdiff_t z) const {
        return static_cast<size_t>(x + n_[0] * (y + n_[1] * z));
    }
    std::ptrdiff_t n_[3];
    std::vector<MTfloat> d_;
};

struct VoxelGrid {
    MTindex nx;
    MTindex ny;
    MTindex nz;
    MTfloat x_min;
    MTfloat y_min;
    MTfloat z_min;
    MTfloat dx;
    MTfloat dy;
    MTfloat dz;
};

struct VoxelData {
    MTindex x;
    MTindex y;
    MTindex z;
    MTfloat length;
};

struct RayData {
    MTfloat ein;
    MTfloat eout;
    Vector3 pin;
    Vector3 pout;
    Vector3 din;
    Vector3 dout;
};
static_assert(sizeof(RayData) == 14 * sizeof(double), "RayData must be 14 doubles (muto_ray)");

typedef std::vector<RayData> MutoMuonData;

struct ImageHeader {
    std::string method;  // only the first 16 chars are written to the file header
    VoxelGrid grid;
    MTindex nRay;
    MTindex nIter;
    MTindex fPrecision;
};
