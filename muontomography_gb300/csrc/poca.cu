// PoCA reconstruction (MutoPoCA::reconstruct, src/MutoPoCA.cpp:51-134), one
// thread per ray: PoCA point, mean squared angle, unsigned-cast binning with
// the reference's reject test, then the Siddon weights of the in and out
// halves (or the straight line).  Sums are FP64 atomics; the voxel each ray
// is binned to is bit-exact with the reference.
#include "common.cuh"

namespace muto {
namespace {

struct WeightSink {
    double* weight;
    uint32_t nx, ny, nz;
    double dz;
    int length_weighted;
    int skip_scat;  // out-half, not length weighted: skip the scattering voxel (:166-168)
    uint32_t sx, sy, sz;
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) {
        if (x >= nx || y >= ny || z >= nz) return;  // never for an in-grid walk
        if (skip_scat && x == sx && y == sy && z == sz) return;
        const uint64_t j = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * (y + static_cast<uint64_t>(ny) * z);
        atomicAdd(weight + j, length_weighted ? l : dz);
    }
};

__global__ void k_poca(PocaArgs a) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    bool parallel_ok = false, kept = false;
    if (i < a.n) {
        const DevGrid g = make_dev_grid(a.g);
        const muto_ray r = a.rays[i];
        const double zmin = a.rays[0].pout[2], zmax = a.rays[0].pin[2];  // :111-112
        double ps[3];
        parallel_ok = poca_point(r, a.eps, ps);
        const double a2 = scat_angle_square(r.din, r.dout, a.mag);
        const uint32_t xs = u32_cast_x86(ddiv(dsub(ps[0], g.lo[0]), g.w[0]));  // :121-123
        const uint32_t ys = u32_cast_x86(ddiv(dsub(ps[1], g.lo[1]), g.w[1]));
        const uint32_t zs = u32_cast_x86(ddiv(dsub(ps[2], g.lo[2]), g.w[2]));
        kept = !(g.n[0] <= xs || g.n[1] <= ys || g.n[2] <= zs || ps[2] < zmin || zmax < ps[2]);  // :125-129
        if (a.assign) {
            a.assign[3 * i + 0] = kept ? static_cast<long long>(xs) : -1;
            a.assign[3 * i + 1] = kept ? static_cast<long long>(ys) : -1;
            a.assign[3 * i + 2] = kept ? static_cast<long long>(zs) : -1;
        }
        if (kept) {
            const uint64_t js = static_cast<uint64_t>(xs) + static_cast<uint64_t>(g.n[0]) * (ys + static_cast<uint64_t>(g.n[1]) * zs);
            atomicAdd(a.img + js, a.has_energy ? dmul(dmul(a2, r.ein), r.ein) : a2);  // :134-138
            WeightSink sink{a.weight, g.n[0], g.n[1], g.n[2], g.w[2], a.length_weighted, 0, xs, ys, zs};
            if (a.straight) {
                siddon_walk(g, r.pin, r.pout, sink);
            } else {
                siddon_walk(g, r.pin, ps, sink);
                sink.skip_scat = !a.length_weighted;
                siddon_walk(g, ps, r.pout, sink);
            }
        }
    }
    warp_count(&a.ctr->not_parallel, parallel_ok);
    warp_count(&a.ctr->in_grid, kept);
}

__global__ void k_poca_normalize(double* __restrict__ img, const double* __restrict__ weight, uint64_t V, double eps) {
    const uint64_t j = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j < V) img[j] = weight[j] < eps ? 0 : ddiv(img[j], weight[j]);  // :180-182
}

}  // namespace

void launch_poca(const PocaArgs& a, cudaStream_t s) {
    if (a.n == 0) return;
    const unsigned nb = static_cast<unsigned>((a.n + 127) / 128);
    k_poca<<<nb, 128, 0, s>>>(a); count_launches(1);
}

void launch_poca_normalize(double* img, const double* weight, uint64_t V, double eps, cudaStream_t s) {
    if (V == 0) return;
    k_poca_normalize<<<static_cast<unsigned>((V + 255) / 256), 256, 0, s>>>(img, weight, V, eps); count_launches(1);
}

}  // namespace muto
