// muto_siddon_batch_noalloc: the batched Siddon walk without any allocation.
//
// muto_siddon_batch allocates device buffers for the segment ends and the
// voxel lists on every call and frees them afterwards.  Some callers cannot
// allow that: a process whose device memory is all reserved up front by its
// own pool allocator has nothing left for a library to allocate from, and a
// loop that keeps other streams of the device busy (a data-acquisition or
// online-monitoring loop) cannot take the device-wide synchronisation that
// cudaFree performs.  This entry point instead stages its work, chunk by
// chunk of rays, through one fixed array compiled into the library.  It calls
// no cudaMalloc/cudaFree and no allocating library routine, and it makes no
// host allocation either.
//
// The array is shared by every call on a device.  Nothing in it has to start
// at zero for the counts and the voxels below each count to be right; the
// voxel slots of a chunk are zeroed before its walk only so that the slots
// past a ray's count come back as zeros rather than another call's data.
// Calls that overlap in time on one device (several host threads, or several
// streams) race on the array: the caller serialises them.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <mutex>

#include "../../include/muto_gb300.h"
#include "common.cuh"
#include "geometry.cuh"

// The scratch array: MUTO_NOALLOC_SCRATCH_BYTES (16 MiB) per device, the same
// for every call.  Device code could name it directly; host code must ask the
// runtime for its address, which happens once per device below.
static __device__ __align__(256) unsigned char g_siddon_scratch[MUTO_NOALLOC_SCRATCH_BYTES];

namespace muto {
namespace {

constexpr size_t kScratchBytes = MUTO_NOALLOC_SCRATCH_BYTES;
constexpr size_t kAlign = 256;
constexpr int kMaxDevices = 64;

// Bytes one ray takes in the scratch: both segment ends, its count, and cap
// voxel slots of three uint32 indices and one double length.
constexpr size_t row_bytes(uint32_t cap) { return 6 * sizeof(double) + sizeof(uint32_t) + size_t(cap) * 20; }
constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// The largest cap still leaves room for at least a dozen rays per chunk.
static_assert(MUTO_NOALLOC_MAX_CAP >= 1, "cap limit");
static_assert(12 * row_bytes(MUTO_NOALLOC_MAX_CAP) + 5 * kAlign <= kScratchBytes, "scratch too small for the cap limit");

// Byte offsets of the five regions of one chunk, each 256-byte aligned.
struct Layout {
    size_t p1, p2, counts, xyz, len;
    uint32_t rays;  // rays per chunk
};

Layout layout_for(uint32_t cap) {
    Layout l{};
    const size_t m = (kScratchBytes - 5 * kAlign) / row_bytes(cap);
    l.rays = static_cast<uint32_t>(std::min<size_t>(m, 1u << 30));
    l.p1 = 0;
    l.p2 = align_up(l.p1 + size_t(l.rays) * 3 * sizeof(double));
    l.counts = align_up(l.p2 + size_t(l.rays) * 3 * sizeof(double));
    l.xyz = align_up(l.counts + size_t(l.rays) * sizeof(uint32_t));
    l.len = align_up(l.xyz + size_t(l.rays) * cap * 3 * sizeof(uint32_t));
    return l;
}

// Set-up, once per device, with that device current: the device address of
// the scratch array.  A failed look-up is remembered and returned again.
struct DeviceScratch {
    std::once_flag once;
    void* ptr = nullptr;
    cudaError_t err = cudaSuccess;
};
DeviceScratch g_devices[kMaxDevices];

int scratch_of_current_device(unsigned char** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return MUTO_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return MUTO_ERR_CUDA;
    DeviceScratch& d = g_devices[dev];
    std::call_once(d.once, [&d] { d.err = cudaGetSymbolAddress(&d.ptr, g_siddon_scratch); });
    if (d.err != cudaSuccess || d.ptr == nullptr) return MUTO_ERR_CUDA;
    *out = static_cast<unsigned char*>(d.ptr);
    return MUTO_OK;
}

struct ScratchSink {
    uint32_t* xyz;
    double* len;
    uint32_t cap, k = 0;
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) {
        if (k < cap) {
            xyz[3 * k + 0] = x;
            xyz[3 * k + 1] = y;
            xyz[3 * k + 2] = z;
            len[k] = l;
        }
        ++k;
    }
};

// One thread per ray of the chunk; everything it reads and writes lies in
// the scratch array at the offsets of `l`.
__global__ void k_siddon_batch_scratch(DevGrid g, unsigned char* __restrict__ scratch, Layout l, uint32_t c,
                                       uint32_t cap) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= c) return;
    const double* p1 = reinterpret_cast<const double*>(scratch + l.p1) + size_t(r) * 3;
    const double* p2 = reinterpret_cast<const double*>(scratch + l.p2) + size_t(r) * 3;
    const double a[3] = {p1[0], p1[1], p1[2]};
    const double b[3] = {p2[0], p2[1], p2[2]};
    ScratchSink s{reinterpret_cast<uint32_t*>(scratch + l.xyz) + size_t(r) * cap * 3,
                  reinterpret_cast<double*>(scratch + l.len) + size_t(r) * cap, cap};
    const int n = siddon_walk(g, a, b, s);
    reinterpret_cast<uint32_t*>(scratch + l.counts)[r] = n < 0 ? 0xffffffffu : static_cast<uint32_t>(n);
}

}  // namespace
}  // namespace muto

extern "C" int muto_siddon_batch_noalloc(const muto_grid* g, const double* p1, const double* p2, uint64_t n,
                                         uint32_t cap, uint32_t* xyz, double* len, uint32_t* counts, void* stream) {
    using namespace muto;
    if (!g || (n > 0 && (!p1 || !p2 || !counts)) || (cap > 0 && n > 0 && (!xyz || !len))) return MUTO_ERR_ARG;
    if (cap > MUTO_NOALLOC_MAX_CAP) return MUTO_ERR_CAPACITY;
    if (n == 0) return MUTO_OK;
    unsigned char* base = nullptr;
    if (const int rc = scratch_of_current_device(&base); rc != MUTO_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const Layout l = layout_for(cap);
    const DevGrid dg = make_dev_grid(*g);
    // A failure after work was queued drains the stream before returning:
    // copies still queued would otherwise land in the caller's buffers (and
    // the next call could reuse the scratch array) after this call returned.
#define NOALLOC_CK(call)                              \
    do {                                              \
        if ((call) != cudaSuccess) {                  \
            (void)cudaStreamSynchronize(s);           \
            return MUTO_ERR_CUDA;                     \
        }                                             \
    } while (0)
    for (uint64_t r0 = 0; r0 < n; r0 += l.rays) {
        const uint32_t c = static_cast<uint32_t>(std::min<uint64_t>(l.rays, n - r0));
        NOALLOC_CK(cudaMemcpyAsync(base + l.p1, p1 + 3 * r0, size_t(c) * 3 * sizeof(double), cudaMemcpyHostToDevice, s));
        NOALLOC_CK(cudaMemcpyAsync(base + l.p2, p2 + 3 * r0, size_t(c) * 3 * sizeof(double), cudaMemcpyHostToDevice, s));
        if (cap > 0) {
            NOALLOC_CK(cudaMemsetAsync(base + l.xyz, 0, size_t(c) * cap * 3 * sizeof(uint32_t), s));
            NOALLOC_CK(cudaMemsetAsync(base + l.len, 0, size_t(c) * cap * sizeof(double), s));
        }
        k_siddon_batch_scratch<<<(c + 127) / 128, 128, 0, s>>>(dg, base, l, c, cap);
        count_launches(1);
        NOALLOC_CK(cudaGetLastError());
        if (cap > 0) {
            NOALLOC_CK(cudaMemcpyAsync(xyz + 3 * r0 * cap, base + l.xyz, size_t(c) * cap * 3 * sizeof(uint32_t),
                                       cudaMemcpyDeviceToHost, s));
            NOALLOC_CK(cudaMemcpyAsync(len + r0 * cap, base + l.len, size_t(c) * cap * sizeof(double),
                                       cudaMemcpyDeviceToHost, s));
        }
        NOALLOC_CK(cudaMemcpyAsync(counts + r0, base + l.counts, size_t(c) * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                   s));
    }
    NOALLOC_CK(cudaStreamSynchronize(s));
#undef NOALLOC_CK
    return MUTO_OK;
}
