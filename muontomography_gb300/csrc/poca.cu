// PoCA reconstruction (MutoPoCA::reconstruct, src/MutoPoCA.cpp:51-134): a
// thread per ray for the PoCA point, mean squared angle, unsigned-cast binning
// with the reference's reject test and the image sum; then a thread per kept
// ray for the Siddon weights of the in and out halves (or the straight line).
// Sums are FP64 atomics; the voxel each ray is binned to is bit-exact with
// the reference.
//
// PoCut (MutoPoCut::reconstruct, src/MutoPoCut.cpp:19-121) runs the same ray
// kernel, keeping each ray's value and voxel instead of summing it, then a
// per-voxel step: the values grouped by voxel, sorted, and the lowest
// floor(M * cut) summed in ascending order from 0.0, as std::accumulate over
// the sorted vector does (:113-117) — so the numerator is bit-exact and only
// the weights carry the atomics' rounding.
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

// Per ray: PoCA point, value and binning; the image sum (or PoCut's value
// and voxel); kept rays are appended to a.walk (warp-aggregated) for the
// walk kernel, so that the FP64 walks run on full warps (a warp of rays
// usually keeps fewer than half of them, and an FP64 instruction takes the
// same pipe time however few of its lanes are active), with a bound on each
// walk by which the list is then ordered (a warp's walks of similar length).
__device__ __forceinline__ bool poca_bin(const DevGrid& g, const muto_ray& r, double eps, double zmin, double zmax,
                                         double* ps, uint32_t* xyz, bool* parallel_ok) {
    *parallel_ok = poca_point(r, eps, ps);
    xyz[0] = u32_cast_x86(ddiv(dsub(ps[0], g.lo[0]), g.w[0]));  // :121-123
    xyz[1] = u32_cast_x86(ddiv(dsub(ps[1], g.lo[1]), g.w[1]));
    xyz[2] = u32_cast_x86(ddiv(dsub(ps[2], g.lo[2]), g.w[2]));
    return !(g.n[0] <= xyz[0] || g.n[1] <= xyz[1] || g.n[2] <= xyz[2] || ps[2] < zmin || zmax < ps[2]);  // :125-129
}

__global__ void k_poca(PocaArgs a) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    bool parallel_ok = false, kept = false;
    uint32_t wlen = 0;  // a bound on the kept ray's walk, for the walk list's order
    if (i < a.n) {
        const DevGrid g = make_dev_grid(a.g);
        const muto_ray r = a.rays[i];
        const double zmin = a.rays[0].pout[2], zmax = a.rays[0].pin[2];  // :111-112
        double ps[3];
        uint32_t xyz[3];
        kept = poca_bin(g, r, a.eps, zmin, zmax, ps, xyz, &parallel_ok);
        if (kept && a.walk_len)
            wlen = a.straight ? walk_bound(g, r.pin, r.pout) : walk_bound(g, r.pin, ps) + walk_bound(g, ps, r.pout);
        if (a.assign) {
            a.assign[3 * i + 0] = kept ? static_cast<long long>(xyz[0]) : -1;
            a.assign[3 * i + 1] = kept ? static_cast<long long>(xyz[1]) : -1;
            a.assign[3 * i + 2] = kept ? static_cast<long long>(xyz[2]) : -1;
        }
        if (a.vox) a.vox[i] = 0xffffffffu;
        if (kept) {
            const uint64_t js = static_cast<uint64_t>(xyz[0]) +
                                static_cast<uint64_t>(g.n[0]) * (xyz[1] + static_cast<uint64_t>(g.n[1]) * xyz[2]);
            const double a2 = scat_angle_square(r.din, r.dout, a.mag);
            const double v = a.has_energy ? dmul(dmul(a2, r.ein), r.ein) : a2;  // :134-138 (PoCut :60-64)
            if (a.vox) {
                a.vox[i] = static_cast<uint32_t>(js);
                a.value[i] = v;
            } else {
                atomicAdd(a.img + js, v);
            }
        }
    }
    // kept rays to the walk list, one atomic per warp
    const unsigned act = __activemask(), b = __ballot_sync(act, kept);
    const int lane = threadIdx.x & 31, lead = __ffs(act) - 1;
    unsigned long long base = 0;
    if (lane == lead && b) base = atomicAdd(a.walk_count, static_cast<unsigned long long>(__popc(b)));
    base = __shfl_sync(act, base, lead);
    if (kept) {
        const uint64_t pos = base + __popc(b & ((1u << lane) - 1u));
        a.walk[pos] = static_cast<uint32_t>(i);
        if (a.walk_len) a.walk_len[pos] = wlen;
    }
    warp_count(&a.ctr->not_parallel, parallel_ok);
    warp_count(&a.ctr->in_grid, kept);
}

// Entries by decreasing walk bound (buckets of 4 voxels), so that the lanes
// of a warp walk paths of about the same length: block-local counts, one
// global reservation per block and bucket, then each entry's place.  The
// number of entries is read on the device (count) or given (n_fixed).
constexpr int kOrderBuckets = 256;
constexpr int kOrderPerThread = 4;
__device__ __forceinline__ uint32_t order_bucket(uint32_t len) {
    const uint32_t b = len >> 2;
    return kOrderBuckets - 1 - (b < kOrderBuckets - 1 ? b : kOrderBuckets - 1);
}

__global__ void k_order_hist(const uint32_t* __restrict__ len, const unsigned long long* __restrict__ count,
                             uint64_t n_fixed, uint32_t* __restrict__ hist) {
    __shared__ uint32_t cnt[kOrderBuckets];
    const uint64_t n = count ? *count : n_fixed;
    for (int t = threadIdx.x; t < kOrderBuckets; t += blockDim.x) cnt[t] = 0;
    __syncthreads();
    for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        atomicAdd(&cnt[order_bucket(len[i])], 1u);
    __syncthreads();
    for (int t = threadIdx.x; t < kOrderBuckets; t += blockDim.x)
        if (cnt[t]) atomicAdd(&hist[t], cnt[t]);
}

// exclusive scan of the bucket counts into cursors (one block of kOrderBuckets threads)
__global__ void k_order_starts(const uint32_t* __restrict__ hist, uint32_t* __restrict__ cursor) {
    __shared__ uint32_t v[kOrderBuckets];
    const int t = threadIdx.x;
    v[t] = hist[t];
    __syncthreads();
    for (int o = 1; o < kOrderBuckets; o <<= 1) {
        const uint32_t x = t >= o ? v[t - o] : 0u;
        __syncthreads();
        v[t] += x;
        __syncthreads();
    }
    cursor[t] = v[t] - hist[t];
}

__global__ void k_order_place(const uint32_t* __restrict__ len, const unsigned long long* __restrict__ count,
                              uint64_t n_fixed, uint32_t* __restrict__ cursor, uint32_t* __restrict__ order) {
    __shared__ uint32_t cnt[kOrderBuckets], base[kOrderBuckets];
    const uint64_t n = count ? *count : n_fixed;
    for (int t = threadIdx.x; t < kOrderBuckets; t += blockDim.x) cnt[t] = 0;
    __syncthreads();
    const uint64_t first = static_cast<uint64_t>(blockIdx.x) * blockDim.x * kOrderPerThread;
    uint32_t bk[kOrderPerThread], rank[kOrderPerThread];
#pragma unroll
    for (int e = 0; e < kOrderPerThread; ++e) {
        const uint64_t i = first + static_cast<uint64_t>(e) * blockDim.x + threadIdx.x;
        bk[e] = i < n ? order_bucket(len[i]) : 0u;
        rank[e] = i < n ? atomicAdd(&cnt[bk[e]], 1u) : 0u;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < kOrderBuckets; t += blockDim.x) base[t] = cnt[t] ? atomicAdd(&cursor[t], cnt[t]) : 0u;
    __syncthreads();
#pragma unroll
    for (int e = 0; e < kOrderPerThread; ++e) {
        const uint64_t i = first + static_cast<uint64_t>(e) * blockDim.x + threadIdx.x;
        if (i < n) order[base[bk[e]] + rank[e]] = static_cast<uint32_t>(i);
    }
}

// The Siddon weights of the kept rays (:100-121), a thread per listed ray
// (not a grid-stride loop: lanes that finished a ray would start their next
// one while the others still walk, and the warp would not step together
// again).
__global__ void k_poca_walk(PocaArgs a) {
    const uint64_t n = *a.walk_count;
    const DevGrid g = make_dev_grid(a.g);
    const double zmin = a.rays[0].pout[2], zmax = a.rays[0].pin[2];
    const uint64_t t = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const unsigned lanes = walk_lanes(t < n);
    if (t < n) {
        const muto_ray r = a.rays[a.walk[a.walk_order ? a.walk_order[t] : t]];
        double ps[3];
        uint32_t xyz[3];
        bool parallel_ok;
        poca_bin(g, r, a.eps, zmin, zmax, ps, xyz, &parallel_ok);  // the kernel above kept it
        WeightSink sink{a.weight, g.n[0], g.n[1], g.n[2], g.w[2], a.length_weighted, 0, xyz[0], xyz[1], xyz[2]};
        if (a.straight) {
            siddon_walk(g, r.pin, r.pout, sink);
        } else {
            siddon_walk(g, r.pin, ps, sink);
            sink.skip_scat = !a.length_weighted;
            __syncwarp(lanes);
            siddon_walk(g, ps, r.pout, sink);
        }
    }
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

void launch_length_order(const uint32_t* len, const unsigned long long* count, uint64_t n, uint32_t* order,
                         uint32_t* work, cudaStream_t s) {
    if (n == 0) return;
    (void)cudaMemsetAsync(work, 0, kOrderBuckets * sizeof(uint32_t), s);  // an error surfaces at the caller's check
    const uint64_t hb = (n + 255) / 256;
    k_order_hist<<<static_cast<unsigned>(hb < 1024 ? hb : 1024), 256, 0, s>>>(len, count, n, work);
    k_order_starts<<<1, kOrderBuckets, 0, s>>>(work, work + kOrderBuckets);
    k_order_place<<<static_cast<unsigned>((n + 256 * kOrderPerThread - 1) / (256 * kOrderPerThread)), 256, 0, s>>>(
        len, count, n, work + kOrderBuckets, order);
    count_launches(3);
}

void launch_poca(const PocaArgs& a, cudaStream_t s) {
    if (a.n == 0) return;
    cudaMemsetAsync(a.walk_count, 0, sizeof(unsigned long long), s);
    const unsigned nb = static_cast<unsigned>((a.n + 127) / 128);
    k_poca<<<nb, 128, 0, s>>>(a);
    if (a.walk_len && a.walk_order && a.order_work)  // the list by decreasing walk bound
        launch_length_order(a.walk_len, a.walk_count, a.n, a.walk_order, a.order_work, s);
    k_poca_walk<<<nb, 128, 0, s>>>(a);  // one thread per ray that can have been kept
    count_launches(2);
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
