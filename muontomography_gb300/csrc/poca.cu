// PoCA reconstruction (MutoPoCA::reconstruct, src/MutoPoCA.cpp:51-134), one
// thread per ray: PoCA point, mean squared angle, unsigned-cast binning with
// the reference's reject test, then the Siddon weights of the in and out
// halves (or the straight line).  Sums are FP64 atomics; the voxel each ray
// is binned to is bit-exact with the reference.
//
// PoCut (MutoPoCut::reconstruct, src/MutoPoCut.cpp:19-121) runs the same ray
// kernel, keeping each ray's value and voxel instead of summing it, then a
// per-voxel step: the values grouped by voxel, sorted, and the lowest
// floor(M * cut) summed in ascending order from 0.0, as std::accumulate over
// the sorted vector does (:113-117) — so the numerator is bit-exact and only
// the weights carry the atomics' rounding.
#include <cmath>

#include "common.cuh"

namespace muto {
namespace {

// The weights are summed in 64-bit fixed point (value * wscale rounded to an
// integer, wscale a power of two chosen by the host so that no voxel's sum
// can overflow): integer reductions are native to L2 where FP64 ones are
// slow, and the integer sums are exact and independent of the order in which
// the rays add them.  They are turned into doubles once all rays are done.
struct WeightSink {
    unsigned long long* wfix;
    double wscale;
    uint32_t nx, ny, nz;
    double dz;
    int length_weighted;
    int skip_scat;  // out-half, not length weighted: skip the scattering voxel (:166-168)
    uint32_t sx, sy, sz;
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) {
        if (x >= nx || y >= ny || z >= nz) return;  // never for an in-grid walk
        if (skip_scat && x == sx && y == sy && z == sz) return;
        const uint64_t j = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * (y + static_cast<uint64_t>(ny) * z);
        atomicAdd(wfix + j, __double2ull_rn((length_weighted ? l : dz) * wscale));
    }
};

// the fixed-point weight sums to doubles, in place
__global__ void k_weight_from_fixed(double* __restrict__ weight, uint64_t V, double inv_scale) {
    const uint64_t j = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j < V) {
        const unsigned long long w = reinterpret_cast<const unsigned long long*>(weight)[j];
        weight[j] = static_cast<double>(w) * inv_scale;
    }
}

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
        if (a.vox) a.vox[i] = 0xffffffffu;
        if (kept) {
            const uint64_t js = static_cast<uint64_t>(xs) + static_cast<uint64_t>(g.n[0]) * (ys + static_cast<uint64_t>(g.n[1]) * zs);
            const double v = a.has_energy ? dmul(dmul(a2, r.ein), r.ein) : a2;  // :134-138 (PoCut :60-64)
            if (a.vox) {
                a.vox[i] = static_cast<uint32_t>(js);
                a.value[i] = v;
            } else {
                atomicAdd(a.img + js, v);
            }
            WeightSink sink{reinterpret_cast<unsigned long long*>(a.weight), a.wscale, g.n[0], g.n[1], g.n[2],
                            g.w[2], a.length_weighted, 0, xs, ys, zs};
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

__global__ void k_pocut_hist(const uint32_t* __restrict__ vox, uint64_t n, uint32_t* __restrict__ counts) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n && vox[i] != 0xffffffffu) atomicAdd(counts + vox[i], 1u);
}

__global__ void k_pocut_scatter(const uint32_t* __restrict__ vox, const double* __restrict__ value, uint64_t n,
                                const uint64_t* __restrict__ off, uint32_t* __restrict__ cursor,
                                unsigned long long* __restrict__ keys) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t j = vox[i];
    if (j == 0xffffffffu) return;
    keys[off[j] + atomicAdd(cursor + j, 1u)] = to_key(value[i]);  // values >= 0: keys order as the values
}

// the threshold of a voxel of m values, static_cast<MTindex>(size * fPercentile)
// (:114), taking at most all of them
__device__ __forceinline__ uint32_t pocut_threshold(uint32_t m, double cut) {
    const uint32_t t = u32_cast_x86(dmul(static_cast<double>(m), cut));
    return t < m ? t : m;
}

__device__ __forceinline__ double pocut_pixel(double sum, double w, double eps) {
    return w < eps ? 0.0 : ddiv(sum, w);  // :117
}

__global__ void k_pocut_empty(const uint32_t* __restrict__ counts, const double* __restrict__ weight,
                              double* __restrict__ img, uint64_t V, double eps) {
    const uint64_t j = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j < V && counts[j] == 0) img[j] = pocut_pixel(0.0, weight[j], eps);
}

// one warp per voxel of at most 32 values: a warp bitonic sort, then the
// lowest values added one after the other in ascending order
__global__ void k_pocut_small(const uint32_t* __restrict__ list, uint32_t n, const uint64_t* __restrict__ off,
                              const uint32_t* __restrict__ counts, const unsigned long long* __restrict__ keys,
                              const double* __restrict__ weight, double* __restrict__ img, double eps, double cut) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n) return;  // whole warps leave together
    const uint32_t j = list[w], m = counts[j];
    unsigned long long k = static_cast<uint32_t>(lane) < m ? keys[off[j] + lane] : ~0ull;
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const unsigned long long o = __shfl_xor_sync(kFull, k, stride);
            const bool up = (lane & size) == 0 || size == 32;
            const bool lower = (lane & stride) == 0;
            k = (lower == up) ? (o < k ? o : k) : (o > k ? o : k);
        }
    }
    const uint32_t t = pocut_threshold(m, cut);
    double sum = 0.0;
    for (uint32_t q = 0; q < t; ++q) {
        const unsigned long long v = __shfl_sync(kFull, k, static_cast<int>(q));
        sum = dadd(sum, from_key(v));
    }
    if (lane == 0) img[j] = pocut_pixel(sum, weight[j], eps);
}

// ascending bitonic sort of n2 (a power of two) keys at a, by one block
__device__ void block_bitonic(unsigned long long* a, uint32_t n2) {
    for (uint32_t size = 2; size <= n2; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t i = threadIdx.x; i < n2 / 2; i += blockDim.x) {
                const uint32_t lo = (i / stride) * stride * 2 + (i % stride), hi = lo + stride;
                const bool up = (lo & size) == 0;
                const unsigned long long x = a[lo], y = a[hi];
                if ((x > y) == up) {
                    a[lo] = y;
                    a[hi] = x;
                }
            }
            __syncthreads();
        }
    }
}

constexpr int kPocutBigThreads = 256;

// one block per voxel of more than 32 values
__global__ void __launch_bounds__(kPocutBigThreads)
    k_pocut_big(const uint32_t* __restrict__ list, uint32_t n, const uint64_t* __restrict__ off,
                const uint32_t* __restrict__ counts, const unsigned long long* __restrict__ keys,
                const uint64_t* __restrict__ scratch_off, unsigned long long* __restrict__ scratch,
                const double* __restrict__ weight, double* __restrict__ img, double eps, double cut) {
    __shared__ unsigned long long sk[kPocutSmemKeys];
    const uint32_t j = list[blockIdx.x], m = counts[j];
    uint32_t n2 = 1;
    while (n2 < m) n2 <<= 1;
    unsigned long long* a = n2 <= kPocutSmemKeys ? sk : scratch + scratch_off[blockIdx.x];
    for (uint32_t i = threadIdx.x; i < n2; i += blockDim.x) a[i] = i < m ? keys[off[j] + i] : ~0ull;
    __syncthreads();
    block_bitonic(a, n2);
    if (threadIdx.x == 0) {
        const uint32_t t = pocut_threshold(m, cut);
        double sum = 0.0;
        for (uint32_t q = 0; q < t; ++q) sum = dadd(sum, from_key(a[q]));
        img[j] = pocut_pixel(sum, weight[j], eps);
    }
}

__global__ void k_poca_normalize(double* __restrict__ img, const double* __restrict__ weight, uint64_t V, double eps) {
    const uint64_t j = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j < V) img[j] = weight[j] < eps ? 0 : ddiv(img[j], weight[j]);  // :180-182
}

}  // namespace

void launch_poca(const PocaArgs& a, cudaStream_t s) {
    if (a.n == 0) return;  // the weights stay all-zero bits, which is 0.0
    const unsigned nb = static_cast<unsigned>((a.n + 127) / 128);
    k_poca<<<nb, 128, 0, s>>>(a);
    const uint64_t V = static_cast<uint64_t>(a.g.nx) * a.g.ny * a.g.nz;
    k_weight_from_fixed<<<static_cast<unsigned>((V + 255) / 256), 256, 0, s>>>(a.weight, V, 1.0 / a.wscale);
    count_launches(2);
}

double poca_weight_scale(uint64_t n_rays, const muto_grid& g, int length_weighted) {
    // a ray adds at most twice (in and out half) the longest in-voxel length
    // (or dz) to a voxel; the sum over all rays must stay below 2^62
    const double wmax = length_weighted ? std::sqrt(g.dx * g.dx + g.dy * g.dy + g.dz * g.dz) : g.dz;
    const double worst = 2.0 * static_cast<double>(n_rays > 0 ? n_rays : 1) * (wmax > 0 ? wmax : 1.0);
    int e = 0;
    std::frexp(4.611686018427387904e18 / worst, &e);  // 2^62 / worst = f * 2^e, f in [0.5, 1)
    e -= 1;                                           // 2^e <= 2^62 / worst
    e = e < -60 ? -60 : (e > 60 ? 60 : e);
    return std::ldexp(1.0, e);
}

void launch_pocut_hist(const uint32_t* vox, uint64_t n, uint32_t* counts, cudaStream_t s) {
    if (n == 0) return;
    k_pocut_hist<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(vox, n, counts);
    count_launches(1);
}

void launch_pocut_scatter(const uint32_t* vox, const double* value, uint64_t n, const uint64_t* off,
                          uint32_t* cursor, unsigned long long* keys, cudaStream_t s) {
    if (n == 0) return;
    k_pocut_scatter<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(vox, value, n, off, cursor, keys);
    count_launches(1);
}

void launch_pocut_empty(const uint32_t* counts, const double* weight, double* img, uint64_t V, double eps,
                        cudaStream_t s) {
    if (V == 0) return;
    k_pocut_empty<<<static_cast<unsigned>((V + 255) / 256), 256, 0, s>>>(counts, weight, img, V, eps);
    count_launches(1);
}

void launch_pocut_small(const uint32_t* list, uint32_t n, const uint64_t* off, const uint32_t* counts,
                        const unsigned long long* keys, const double* weight, double* img, double eps, double cut,
                        cudaStream_t s) {
    if (n == 0) return;
    k_pocut_small<<<static_cast<unsigned>((uint64_t(n) * 32 + 255) / 256), 256, 0, s>>>(list, n, off, counts, keys,
                                                                                      weight, img, eps, cut);
    count_launches(1);
}

void launch_pocut_big(const uint32_t* list, uint32_t n, const uint64_t* off, const uint32_t* counts,
                      const unsigned long long* keys, const uint64_t* scratch_off, unsigned long long* scratch,
                      const double* weight, double* img, double eps, double cut, cudaStream_t s) {
    if (n == 0) return;
    k_pocut_big<<<n, kPocutBigThreads, 0, s>>>(list, n, off, counts, keys, scratch_off, scratch, weight, img, eps,
                                               cut);
    count_launches(1);
}

void launch_poca_normalize(double* img, const double* weight, uint64_t V, double eps, cudaStream_t s) {
    if (V == 0) return;
    k_poca_normalize<<<static_cast<unsigned>((V + 255) / 256), 256, 0, s>>>(img, weight, V, eps); count_launches(1);
}

}  // namespace muto
