// Exclusive prefix sum (uint32 in, uint64 out) used for the kept-muon
// compaction, the per-muon pair offsets and the per-voxel segment starts.
// Three phases per level: per-block totals, a scan of the totals (recursive),
// and a block-local scan plus the block's base.
#include "common.cuh"

namespace muto {
namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr uint64_t kScanTile = static_cast<uint64_t>(kScanThreads) * kScanItems;

template <typename In>
__device__ __forceinline__ uint64_t load_or_zero(const In* in, uint64_t i, uint64_t n) {
    return i < n ? static_cast<uint64_t>(in[i]) : 0ull;
}

__device__ __forceinline__ uint64_t block_exclusive(uint64_t v, uint64_t* warp_tot, uint64_t* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint64_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        uint64_t w = lane < nw ? warp_tot[lane] : 0ull;
        uint64_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t t = __shfl_up_sync(kFull, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < nw) warp_tot[lane] = wi - w;
        if (lane == nw - 1) *total = wi;
    }
    __syncthreads();
    return incl - v + warp_tot[wid];
}

template <typename In>
__global__ void __launch_bounds__(kScanThreads) k_block_totals(const In* in, uint64_t n, uint64_t* totals) {
    __shared__ uint64_t red[kScanThreads / 32];
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kScanTile;
    uint64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) s += load_or_zero(in, base + threadIdx.x + static_cast<uint64_t>(k) * kScanThreads, n);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint64_t v = threadIdx.x < kScanThreads / 32 ? red[threadIdx.x] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
        if (threadIdx.x == 0) totals[blockIdx.x] = v;
    }
}

// out[i] = exclusive prefix; base[b] is the block's starting value; out[n] = total when last block
template <typename In>
__global__ void __launch_bounds__(kScanThreads) k_block_scan(const In* in, uint64_t n, const uint64_t* base,
                                                            uint64_t* out) {
    __shared__ uint64_t warp_tot[kScanThreads / 32];
    __shared__ uint64_t total;
    const uint64_t b0 = static_cast<uint64_t>(blockIdx.x) * kScanTile;
    const uint64_t mine = b0 + static_cast<uint64_t>(threadIdx.x) * kScanItems;  // blocked arrangement
    uint64_t v[kScanItems];
    uint64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = load_or_zero(in, mine + k, n);
        s += v[k];
    }
    uint64_t ex = block_exclusive(s, warp_tot, &total) + (base ? base[blockIdx.x] : 0ull);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (mine + k < n) out[mine + k] = ex;
        ex += v[k];
        if (mine + k == n - 1) out[n] = ex;
    }
}

uint64_t n_tiles(uint64_t n) { return (n + kScanTile - 1) / kScanTile; }

}  // namespace

size_t scan_scratch_bytes(uint64_t n) {
    size_t bytes = 0;
    uint64_t m = n_tiles(n);
    while (m > 1) {
        bytes += (2 * (m + 1)) * sizeof(uint64_t);
        m = n_tiles(m);
    }
    return bytes + 64;
}

namespace {
template <typename In>
void scan_rec(const In* in, uint64_t* out, uint64_t n, uint64_t* scratch, cudaStream_t s) {
    const uint64_t nb = n_tiles(n);
    if (nb <= 1) {
        k_block_scan<In><<<1, kScanThreads, 0, s>>>(in, n, nullptr, out); count_launches(1);
        return;
    }
    uint64_t* totals = scratch;
    uint64_t* bases = scratch + (nb + 1);
    k_block_totals<In><<<static_cast<unsigned>(nb), kScanThreads, 0, s>>>(in, n, totals); count_launches(1);
    scan_rec<uint64_t>(totals, bases, nb, scratch + 2 * (nb + 1), s);
    k_block_scan<In><<<static_cast<unsigned>(nb), kScanThreads, 0, s>>>(in, n, bases, out); count_launches(1);
}
}  // namespace

void scan_u32_to_u64(const uint32_t* in, uint64_t* out, uint64_t n, void* scratch, cudaStream_t s) {
    if (n == 0) {
        cudaMemsetAsync(out, 0, sizeof(uint64_t), s);
        return;
    }
    scan_rec<uint32_t>(in, out, n, static_cast<uint64_t*>(scratch), s);
}

}  // namespace muto

namespace muto {
namespace {
__global__ void k_add_u64(uint64_t* __restrict__ a, uint64_t n, uint64_t add) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) a[i] += add;
}
}  // namespace

void launch_add_u64(uint64_t* a, uint64_t n, uint64_t add, cudaStream_t s) {
    if (n == 0 || add == 0) return;
    k_add_u64<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(a, n, add);
    count_launches(1);
}
}  // namespace muto
