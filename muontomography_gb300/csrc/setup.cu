// Setup kernels of the MLSD/MAP path (run once per reconstruction):
//   keep flags + compaction   gatherInformation, src/MutoMLSD.cpp:268-326
//   muon info                 getScatteringAngle / getDisplacement / pr, :350-376, :320-322
//   path count + fill         getMuonPathAndTail + generateWeightMatrix, :382-430
//   voxel multiplicity/slots  allocateSValueMatrix + S_index, :432-437, :173-181
// and the batched Siddon probe (MutoSiddon::getVoxelPath, src/MutoSiddon.cpp:9).
#include "common.cuh"

namespace muto {
namespace {

constexpr int kThreads = 256;

inline unsigned blocks_for(uint64_t n, int threads = kThreads) {
    const uint64_t b = (n + threads - 1) / threads;
    return static_cast<unsigned>(b > 0 ? b : 1);
}

// in-grid and detector-zone test of gatherInformation (src/MutoMLSD.cpp:273-274, :298-304)
__device__ __forceinline__ bool keep_muon(const muto_ray& r, const DevGrid& g, double eps, double zdet_min,
                                          double zdet_max, double* ps) {
    poca_point(r, eps, ps);
    const double xhi = dsub(dadd(g.lo[0], dmul(g.w[0], static_cast<double>(g.n[0]))), eps);
    const double yhi = dsub(dadd(g.lo[1], dmul(g.w[1], static_cast<double>(g.n[1]))), eps);
    const double zhi = dsub(dadd(g.lo[2], dmul(g.w[2], static_cast<double>(g.n[2]))), eps);
    return !(ps[0] < dadd(g.lo[0], eps) || xhi < ps[0] || ps[1] < dadd(g.lo[1], eps) || yhi < ps[1] ||
             ps[2] < dadd(g.lo[2], eps) || zhi < ps[2] || ps[2] < dadd(zdet_min, eps) || dsub(zdet_max, eps) <= ps[2]);
}

__global__ void k_keep_flags(const muto_ray* __restrict__ rays, uint64_t n, DevGrid g, double eps,
                             uint32_t* __restrict__ flags) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double zmin = rays[0].pout[2], zmax = rays[0].pin[2];  // detector zone from ray 0, :273-274
    double ps[3];
    flags[i] = keep_muon(rays[i], g, eps, zmin, zmax, ps) ? 1u : 0u;
}

__global__ void k_compact(const uint32_t* __restrict__ flags, const uint64_t* __restrict__ pos, uint64_t n,
                          uint32_t* __restrict__ kept) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n && flags[i]) kept[pos[i]] = static_cast<uint32_t>(i);
}

template <typename Real>
__global__ void k_muon_info(const muto_ray* __restrict__ rays, const uint32_t* __restrict__ kept, uint64_t n,
                            DevGrid g, double eps, int has_energy, typename Vec4<Real>::type* __restrict__ sd,
                            Real* __restrict__ pr2, double* __restrict__ scat, double* __restrict__ pr_out) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const muto_ray r = rays[kept[i]];
    double ps[3];
    poca_point(r, eps, ps);
    scat[3 * i + 0] = ps[0];
    scat[3 * i + 1] = ps[1];
    scat[3 * i + 2] = ps[2];
    double sx, sy, dx, dy;
    scat_angles(r.din, r.dout, &sx, &sy);
    displacement(r, g.lo[2], &dx, &dy);
    typename Vec4<Real>::type v;
    v.x = static_cast<Real>(sx);
    v.y = static_cast<Real>(dx);
    v.z = static_cast<Real>(sy);
    v.w = static_cast<Real>(dy);
    sd[i] = v;
    const double pr = has_energy ? ddiv(3.0, r.ein) : 1.0;  // pr = p0 / p, :288, :321
    pr2[i] = static_cast<Real>(pr * pr);
    if (pr_out) pr_out[i] = pr;
}

struct CountSink {
    int n = 0;
    __device__ void operator()(uint32_t, uint32_t, uint32_t, double) { ++n; }
};

__global__ void k_path_count(const muto_ray* __restrict__ rays, const uint32_t* __restrict__ kept,
                             const double* __restrict__ scat, uint64_t n, DevGrid g, int straight,
                             uint32_t* __restrict__ counts, Counters* ctr) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const muto_ray& r = rays[kept[i]];
    const double ps[3] = {scat[3 * i], scat[3 * i + 1], scat[3 * i + 2]};
    int total = 0;
    bool overflow = false;
    CountSink a, b;
    if (straight) {
        const int c = siddon_walk(g, r.pin, r.pout, a);
        overflow = c < 0;
        total = overflow ? 0 : c;
    } else {
        const int ci = siddon_walk(g, r.pin, ps, a);
        const int co = siddon_walk(g, ps, r.pout, b);
        overflow = ci < 0 || co < 0;
        // in-half, then the out-half without its first voxel (merged into the
        // last in-voxel, or dropped when the in-half is empty), :396-402
        total = overflow ? 0 : ci + (co > 0 ? co - 1 : 0);
    }
    if (overflow) atomicAdd(&ctr->overflow, 1ull);
    counts[i] = static_cast<uint32_t>(total);
}

// Writes the merged path of one muon: voxel index (xyz2index, include/MutoMLSD.h:76,
// in 32-bit unsigned arithmetic) and FP64 length.
struct FillSink {
    uint32_t* vidx;
    double* l64;
    uint64_t pos, end;  // the muon's segment [pos, end) from the count pass
    uint32_t nx, nxy;
    bool pending = false;      // buffered last voxel of the in-half
    uint32_t pj = 0;
    double pl = 0.0;
    int phase = 0;             // 0: in-half, 1: first out voxel, 2: rest of out-half
    __device__ void emit(uint32_t j, double l) {
        if (pos < end) {  // the fill walk repeats the count walk exactly; never past the segment
            vidx[pos] = j;
            l64[pos] = l;
        }
        ++pos;
    }
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) {
        const uint32_t j = x + y * nx + z * nxy;
        if (phase == 0) {
            if (pending) emit(pj, pl);
            pending = true;
            pj = j;
            pl = l;
        } else if (phase == 1) {
            if (pending) {
                emit(pj, dadd(pl, l));  // voxelsIn.back().length += voxelsOut[0].length
                pending = false;
            }
            phase = 2;
        } else {
            emit(j, l);
        }
    }
};

struct StraightSink {
    uint32_t* vidx;
    double* l64;
    uint64_t pos, end;
    uint32_t nx, nxy;
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) {
        if (pos < end) {
            vidx[pos] = x + y * nx + z * nxy;
            l64[pos] = l;
        }
        ++pos;
    }
};

template <typename Real>
__global__ void k_path_fill(const muto_ray* __restrict__ rays, const uint32_t* __restrict__ kept,
                            const double* __restrict__ scat, const uint64_t* __restrict__ off, uint64_t n, DevGrid g,
                            int straight, uint32_t* __restrict__ vidx, double* __restrict__ l64, Real* __restrict__ L,
                            Real* __restrict__ T) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t b = off[i], e = off[i + 1];
    if (e == b) return;  // empty (or overflowed) path
    const muto_ray& r = rays[kept[i]];
    const double ps[3] = {scat[3 * i], scat[3 * i + 1], scat[3 * i + 2]};
    const uint32_t nx = g.n[0], nxy = g.n[0] * g.n[1];
    if (straight) {
        StraightSink s{vidx, l64, b, e, nx, nxy};
        siddon_walk(g, r.pin, r.pout, s);
    } else {
        FillSink s{vidx, l64, b, e, nx, nxy};
        siddon_walk(g, r.pin, ps, s);
        s.phase = 1;
        siddon_walk(g, ps, r.pout, s);
        if (s.pending) s.emit(s.pj, dadd(s.pl, 0.0));  // out-half empty: length += 0.0
    }
    // tail lengths, summed backwards in FP64 like src/MutoMLSD.cpp:407-413
    double t = 0.0;
    for (uint64_t k = e; k-- > b;) {
        const double lk = l64[k];
        if (L != reinterpret_cast<Real*>(l64)) L[k] = static_cast<Real>(lk);
        T[k] = static_cast<Real>(t);
        t = dadd(t, lk);
    }
}


__global__ void k_path_bound(const muto_ray* __restrict__ rays, const uint32_t* __restrict__ kept,
                             const double* __restrict__ scat, uint64_t n, DevGrid g, int straight,
                             uint32_t* __restrict__ bounds) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const muto_ray& r = rays[kept[i]];
    if (straight) {
        bounds[i] = walk_bound(g, r.pin, r.pout);
    } else {
        const double ps[3] = {scat[3 * i], scat[3 * i + 1], scat[3 * i + 2]};
        bounds[i] = walk_bound(g, r.pin, ps) + walk_bound(g, ps, r.pout);
    }
}

// the fill walk into bounded slots [boff[i], boff[i+1]) - slot_base; counts[i]
// = the path's length (0 for a walk that hit its step guard, as in the count walk)
template <typename Real>
__global__ void k_path_fill_bounded(const muto_ray* __restrict__ rays, const uint32_t* __restrict__ kept,
                                    const double* __restrict__ scat, const uint64_t* __restrict__ boff, uint64_t n,
                                    DevGrid g, int straight, uint32_t* __restrict__ vidx, double* __restrict__ l64,
                                    Real* __restrict__ L, Real* __restrict__ T, uint32_t* __restrict__ counts,
                                    Counters* ctr, uint64_t slot_base) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const unsigned lanes = walk_lanes(i < n);
    if (i >= n) return;
    const uint64_t b = boff[i] - slot_base, e = boff[i + 1] - slot_base;
    const muto_ray& r = rays[kept[i]];
    const double ps[3] = {scat[3 * i], scat[3 * i + 1], scat[3 * i + 2]};
    const uint32_t nx = g.n[0], nxy = g.n[0] * g.n[1];
    uint64_t end;
    bool overflow = false;
    if (straight) {
        StraightSink s{vidx, l64, b, e, nx, nxy};
        overflow = siddon_walk(g, r.pin, r.pout, s) < 0;
        end = s.pos;
    } else {
        FillSink s{vidx, l64, b, e, nx, nxy};
        const int ci = siddon_walk(g, r.pin, ps, s);
        s.phase = 1;
        __syncwarp(lanes);
        const int co = siddon_walk(g, ps, r.pout, s);
        if (s.pending) s.emit(s.pj, dadd(s.pl, 0.0));  // out-half empty: length += 0.0
        overflow = ci < 0 || co < 0;
        end = s.pos;
    }
    if (overflow) {  // dropped, like the count walk does
        atomicAdd(&ctr->overflow, 1ull);
        end = b;
    }
    if (end > e) {
        atomicAdd(&ctr->over_bound, 1ull);
        end = e;
    }
    counts[i] = static_cast<uint32_t>(end - b);
    // tail lengths, summed backwards in FP64 like src/MutoMLSD.cpp:407-413
    double t = 0.0;
    for (uint64_t k = end; k-- > b;) {
        const double lk = l64[k];
        if (L != reinterpret_cast<Real*>(l64)) L[k] = static_cast<Real>(lk);
        T[k] = static_cast<Real>(t);
        t = dadd(t, lk);
    }
}

// warp per muon: its path from the bounded slots (boff[i] - slot_base) to the exact ones
template <typename Real>
__global__ void k_path_compact(const uint64_t* __restrict__ boff, uint64_t slot_base, const uint64_t* __restrict__ off,
                               uint64_t n, const uint32_t* __restrict__ vidx_b, const Real* __restrict__ L_b,
                               const Real* __restrict__ T_b, uint32_t* __restrict__ vidx, Real* __restrict__ L,
                               Real* __restrict__ T) {
    const uint64_t i = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const uint64_t src = boff[i] - slot_base, dst = off[i], m = off[i + 1] - dst;
    for (uint64_t k = lane; k < m; k += 32) {
        vidx[dst + k] = vidx_b[src + k];
        L[dst + k] = L_b[src + k];
        T[dst + k] = T_b[src + k];
    }
}

__global__ void k_offset_voxels(uint32_t* __restrict__ vidx, uint64_t n, uint32_t v_scan, uint32_t voff) {
    const uint64_t k = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < n) {
        const uint32_t j = vidx[k];
        vidx[k] = j < v_scan ? voff + j : 0xffffffffu;
    }
}

__global__ void k_voxel_hist(const uint32_t* __restrict__ vidx, uint64_t P, uint32_t V, uint32_t* __restrict__ mult,
                             Counters* ctr) {
    const uint64_t k = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    bool bad = false;
    if (k < P) {
        const uint32_t j = vidx[k];
        if (j < V) atomicAdd(&mult[j], 1u);
        else bad = true;
    }
    warp_count(&ctr->bounds, bad);
}

template <typename Real> __device__ __forceinline__ Real index_bits(uint32_t i);
template <> __device__ __forceinline__ float index_bits<float>(uint32_t i) { return __uint_as_float(i); }
template <> __device__ __forceinline__ double index_bits<double>(uint32_t i) {
    return __longlong_as_double(static_cast<long long>(i));
}
__device__ __forceinline__ uint32_t bits_index(float x) { return __float_as_uint(x); }
__device__ __forceinline__ uint32_t bits_index(double x) { return static_cast<uint32_t>(__double_as_longlong(x)); }

// Voxel-major lists in two steps.  First a warp per muon reads its pairs
// coalesced and scatters each as one record (muon, L, T) to its slot in its
// voxel's segment (one aligned store per pair: scattered partial stores of
// the separate arrays cost twice as much).  Then a coalesced pass splits the
// records into the muon and (L, T) arrays the voxel pass streams.
template <typename Real>
__global__ void k_build_voxel_major(const uint64_t* __restrict__ off, uint64_t n, const uint32_t* __restrict__ vidx,
                                    const Real* __restrict__ L, const Real* __restrict__ T, uint32_t V,
                                    const uint64_t* __restrict__ start, uint32_t* __restrict__ cursor,
                                    typename Vec4<Real>::type* __restrict__ rec) {
    const uint64_t i = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const uint64_t pe = off[i + 1];
    for (uint64_t p = off[i] + lane; p < pe; p += 32) {
        const uint32_t j = vidx[p];
        if (j >= V) continue;  // counted by k_voxel_hist
        const uint64_t at = start[j] + atomicAdd(&cursor[j], 1u);
        typename Vec4<Real>::type r;
        r.x = index_bits<Real>(static_cast<uint32_t>(i));  // the index's bits, moved, never computed on
        r.y = L[p];
        r.z = T[p];
        r.w = Real(0);
        rec[at] = r;
    }
}

template <typename Real>
__global__ void k_split_records(const typename Vec4<Real>::type* __restrict__ rec, uint64_t P,
                                uint32_t* __restrict__ vm_mu, typename Vec2<Real>::type* __restrict__ vm_LT,
                                const uint32_t* __restrict__ kslot) {
    const uint64_t p = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const typename Vec4<Real>::type r = rec[p];
    const uint32_t m = bits_index(r.x);
    vm_mu[p] = kslot ? kslot[m] : m;
    typename Vec2<Real>::type lt;
    lt.x = r.y;
    lt.y = r.z;
    vm_LT[p] = lt;
}

struct BatchSink {
    uint32_t* xyz;
    double* len;
    uint64_t base;
    uint32_t cap, k = 0;
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) {
        if (k < cap) {
            xyz[(base + k) * 3 + 0] = x;
            xyz[(base + k) * 3 + 1] = y;
            xyz[(base + k) * 3 + 2] = z;
            len[base + k] = l;
        }
        ++k;
    }
};

__global__ void k_siddon_batch(DevGrid g, const double* __restrict__ p1, const double* __restrict__ p2, uint64_t n,
                               uint32_t cap, uint32_t* __restrict__ xyz, double* __restrict__ len,
                               uint32_t* __restrict__ counts) {
    const uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const double a[3] = {p1[3 * r], p1[3 * r + 1], p1[3 * r + 2]};
    const double b[3] = {p2[3 * r], p2[3 * r + 1], p2[3 * r + 2]};
    BatchSink s{xyz, len, r * cap, cap};
    const int c = siddon_walk(g, a, b, s);
    counts[r] = c < 0 ? 0xffffffffu : static_cast<uint32_t>(c);
}

// Voxel classes on the device: a stable partition of the voxels by segment
// length class (one counting pass of a radix sort with kVoxClasses buckets).
// Per block of 256 voxels: the class counts (class-major, so one exclusive
// scan gives every block's first slot in every class), then the scatter of
// each voxel's descriptor to its slot.  Within a class the voxels are in
// column order (z fastest, then x, then y) when a grid is given, else in
// index order: vertically adjacent voxels, which share many of their (mostly
// steep) muons, are then processed side by side and their coefficient
// gathers hit the same cache lines.
__device__ __forceinline__ uint32_t class_order_voxel(uint32_t t, uint32_t nx, uint32_t ny, uint32_t nz) {
    if (nz == 0) return t;
    const uint32_t z = t % nz, r = t / nz;
    return r % nx + nx * (r / nx + ny * z);
}

// Segment starts in column order: the voxel-major segments of vertically
// adjacent voxels sit next to each other, so a stream through the lists
// meets a steep muon in several consecutive segments (its coefficients are
// still in L1 the second time).  mcol[t] = M of the t-th voxel in column
// order; after the scan, start[j] = scol[t] for that voxel.
__global__ void k_column_mult(const uint32_t* __restrict__ mult, uint32_t V, uint32_t nx, uint32_t ny, uint32_t nz,
                              uint32_t* __restrict__ mcol) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < V) mcol[t] = mult[class_order_voxel(t, nx, ny, nz)];
}
__global__ void k_column_starts(const uint64_t* __restrict__ scol, uint32_t V, uint32_t nx, uint32_t ny, uint32_t nz,
                                uint64_t* __restrict__ start) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < V) start[class_order_voxel(t, nx, ny, nz)] = scol[t];
    if (t == 0) start[V] = scol[V];
}

template <typename Real>
__global__ void k_class_count(const uint32_t* __restrict__ mult, uint32_t V, uint32_t nblocks, uint32_t nx,
                              uint32_t ny, uint32_t nz, uint32_t* __restrict__ counts) {
    __shared__ uint32_t c_s[kVoxClasses];
    if (threadIdx.x < kVoxClasses) c_s[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t j = t < V ? class_order_voxel(t, nx, ny, nz) : 0u;
    const int cls = t < V ? vox_class_of<Real>(mult[j]) : -1;
    const int lane = threadIdx.x & 31;
    for (int c = 0; c < kVoxClasses; ++c) {
        const uint32_t n = __popc(__ballot_sync(kFull, cls == c));
        if (lane == 0 && n) atomicAdd(&c_s[c], n);
    }
    __syncthreads();
    if (threadIdx.x < kVoxClasses) counts[threadIdx.x * nblocks + blockIdx.x] = c_s[threadIdx.x];
}

template <typename Real>
__global__ void k_class_scatter(const uint32_t* __restrict__ mult, const uint64_t* __restrict__ start, uint32_t V,
                                uint32_t nblocks, uint32_t nx, uint32_t ny, uint32_t nz,
                                const uint64_t* __restrict__ first, VoxDesc* __restrict__ out) {
    constexpr int W = kThreads / 32;
    __shared__ uint32_t wc[W][kVoxClasses];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t j = t < V ? class_order_voxel(t, nx, ny, nz) : 0u;
    const int cls = t < V ? vox_class_of<Real>(mult[j]) : -1;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t my_rank = 0;
    for (int c = 0; c < kVoxClasses; ++c) {
        const unsigned m = __ballot_sync(kFull, cls == c);
        if (cls == c) my_rank = __popc(m & ((1u << lane) - 1u));
        if (lane == 0) wc[w][c] = __popc(m);
    }
    __syncthreads();
    if (cls >= 0) {
        uint32_t before = 0;
        for (int q = 0; q < w; ++q) before += wc[q][cls];
        const uint64_t at = first[static_cast<uint64_t>(cls) * nblocks + blockIdx.x] + before + my_rank;
        out[at] = VoxDesc{j, mult[j], start[j]};
    }
}

__global__ void k_brick_indices(uint32_t* __restrict__ vidx, uint64_t n, BrickDims b, uint32_t V) {
    const uint64_t k = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < n) {
        const uint32_t j = vidx[k];
        if (j < V) vidx[k] = brick_of(j, b);
    }
}

__global__ void k_unbrick_indices(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint64_t n,
                                  BrickDims b) {
    const uint64_t k = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < n) {
        const uint32_t jb = in[k];
        out[k] = jb == 0xffffffffu ? jb : unbrick(jb, b);
    }
}

template <typename Real>
__global__ void k_brick_lambda(const Real* __restrict__ lam, uint32_t V, BrickDims b, Real* __restrict__ lam_b) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < V) lam_b[brick_of(j, b)] = lam[j];
}

}  // namespace

void launch_keep_flags(const muto_ray* rays, uint64_t n_total, muto_grid g, double eps, uint32_t* flags,
                       cudaStream_t s) {
    if (n_total == 0) return;
    k_keep_flags<<<blocks_for(n_total), kThreads, 0, s>>>(rays, n_total, make_dev_grid(g), eps, flags); count_launches(1);
}

void launch_compact(const uint32_t* flags, const uint64_t* pos, uint64_t n, uint32_t* kept, cudaStream_t s) {
    if (n == 0) return;
    k_compact<<<blocks_for(n), kThreads, 0, s>>>(flags, pos, n, kept); count_launches(1);
}

template <typename Real>
void launch_muon_info(const muto_ray* rays, const uint32_t* kept, uint64_t n, muto_grid g, double eps, int has_energy,
                      typename Vec4<Real>::type* sd, Real* pr2, double* scat, double* pr_out, cudaStream_t s) {
    if (n == 0) return;
    k_muon_info<Real><<<blocks_for(n), kThreads, 0, s>>>(rays, kept, n, make_dev_grid(g), eps, has_energy, sd, pr2,
                                                           scat, pr_out); count_launches(1);
}
template void launch_muon_info<float>(const muto_ray*, const uint32_t*, uint64_t, muto_grid, double, int, float4*,
                                      float*, double*, double*, cudaStream_t);
template void launch_muon_info<double>(const muto_ray*, const uint32_t*, uint64_t, muto_grid, double, int, double4*,
                                       double*, double*, double*, cudaStream_t);

void launch_path_count(const muto_ray* rays, const uint32_t* kept, const double* scat, uint64_t n, muto_grid g,
                       int straight, uint32_t* counts, Counters* ctr, cudaStream_t s) {
    if (n == 0) return;
    k_path_count<<<blocks_for(n, 128), 128, 0, s>>>(rays, kept, scat, n, make_dev_grid(g), straight, counts, ctr); count_launches(1);
}

template <typename Real>
void launch_path_fill(const muto_ray* rays, const uint32_t* kept, const double* scat, const uint64_t* off, uint64_t n,
                      muto_grid g, int straight, uint32_t* vidx, double* l64, Real* L, Real* T, cudaStream_t s) {
    if (n == 0) return;
    k_path_fill<Real><<<blocks_for(n, 128), 128, 0, s>>>(rays, kept, scat, off, n, make_dev_grid(g), straight, vidx,
                                                          l64, L, T); count_launches(1);
}
template void launch_path_fill<float>(const muto_ray*, const uint32_t*, const double*, const uint64_t*, uint64_t,
                                      muto_grid, int, uint32_t*, double*, float*, float*, cudaStream_t);
template void launch_path_fill<double>(const muto_ray*, const uint32_t*, const double*, const uint64_t*, uint64_t,
                                       muto_grid, int, uint32_t*, double*, double*, double*, cudaStream_t);

void launch_path_bound(const muto_ray* rays, const uint32_t* kept, const double* scat, uint64_t n, muto_grid g,
                       int straight, uint32_t* bounds, cudaStream_t s) {
    if (n == 0) return;
    k_path_bound<<<blocks_for(n), kThreads, 0, s>>>(rays, kept, scat, n, make_dev_grid(g), straight, bounds);
    count_launches(1);
}

template <typename Real>
void launch_path_fill_bounded(const muto_ray* rays, const uint32_t* kept, const double* scat, const uint64_t* boff,
                              uint64_t slot_base, uint64_t n, muto_grid g, int straight, uint32_t* vidx, double* l64,
                              Real* L, Real* T, uint32_t* counts, Counters* ctr, cudaStream_t s) {
    if (n == 0) return;
    k_path_fill_bounded<Real><<<blocks_for(n, 128), 128, 0, s>>>(rays, kept, scat, boff, n, make_dev_grid(g), straight,
                                                                  vidx, l64, L, T, counts, ctr, slot_base);
    count_launches(1);
}
template void launch_path_fill_bounded<float>(const muto_ray*, const uint32_t*, const double*, const uint64_t*,
                                              uint64_t, uint64_t, muto_grid, int, uint32_t*, double*, float*, float*,
                                              uint32_t*, Counters*, cudaStream_t);
template void launch_path_fill_bounded<double>(const muto_ray*, const uint32_t*, const double*, const uint64_t*,
                                               uint64_t, uint64_t, muto_grid, int, uint32_t*, double*, double*,
                                               double*, uint32_t*, Counters*, cudaStream_t);

template <typename Real>
void launch_path_compact(const uint64_t* boff, uint64_t slot_base, const uint64_t* off, uint64_t n,
                         const uint32_t* vidx_b, const Real* L_b, const Real* T_b, uint32_t* vidx, Real* L, Real* T,
                         cudaStream_t s) {
    if (n == 0) return;
    k_path_compact<Real><<<blocks_for(n * 32), kThreads, 0, s>>>(boff, slot_base, off, n, vidx_b, L_b, T_b, vidx, L,
                                                                 T);
    count_launches(1);
}
template void launch_path_compact<float>(const uint64_t*, uint64_t, const uint64_t*, uint64_t, const uint32_t*,
                                         const float*, const float*, uint32_t*, float*, float*, cudaStream_t);
template void launch_path_compact<double>(const uint64_t*, uint64_t, const uint64_t*, uint64_t, const uint32_t*,
                                          const double*, const double*, uint32_t*, double*, double*, cudaStream_t);

void launch_offset_voxels(uint32_t* vidx, uint64_t n, uint32_t v_scan, uint32_t voff, cudaStream_t s) {
    if (n == 0) return;
    k_offset_voxels<<<blocks_for(n), kThreads, 0, s>>>(vidx, n, v_scan, voff);
    count_launches(1);
}

void launch_voxel_hist(const uint32_t* vidx, uint64_t P, uint32_t V, uint32_t* mult, Counters* ctr, cudaStream_t s) {
    if (P == 0) return;
    k_voxel_hist<<<blocks_for(P), kThreads, 0, s>>>(vidx, P, V, mult, ctr); count_launches(1);
}

template <typename Real>
void launch_build_voxel_major(const uint64_t* off, uint64_t n, const uint32_t* vidx, const Real* L, const Real* T,
                              uint32_t V, const uint64_t* start, uint32_t* cursor, uint64_t P,
                              typename Vec4<Real>::type* rec, uint32_t* vm_mu, typename Vec2<Real>::type* vm_LT,
                              const uint32_t* kslot, cudaStream_t s) {
    if (n == 0) return;
    k_build_voxel_major<Real><<<blocks_for(n * 32), kThreads, 0, s>>>(off, n, vidx, L, T, V, start, cursor, rec);
    count_launches(1);
    if (P == 0) return;
    k_split_records<Real><<<blocks_for(P), kThreads, 0, s>>>(rec, P, vm_mu, vm_LT, kslot);
    count_launches(1);
}
template void launch_build_voxel_major<float>(const uint64_t*, uint64_t, const uint32_t*, const float*, const float*,
                                              uint32_t, const uint64_t*, uint32_t*, uint64_t, float4*, uint32_t*,
                                              float2*, const uint32_t*, cudaStream_t);
template void launch_build_voxel_major<double>(const uint64_t*, uint64_t, const uint32_t*, const double*,
                                               const double*, uint32_t, const uint64_t*, uint32_t*, uint64_t,
                                               double4*, uint32_t*, double2*, const uint32_t*, cudaStream_t);

// the (x, y) cell of each kept muon's PoCA point, clamped to the grid, and
// the muons per cell
__global__ void k_muon_cells(const double* __restrict__ scat, uint64_t n, DevGrid g, uint32_t* __restrict__ cell,
                             uint32_t* __restrict__ hist) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t c[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const double u = (scat[3 * i + k] - g.lo[k]) / g.w[k];
        c[k] = u >= 0.0 ? (u < static_cast<double>(g.n[k]) ? static_cast<uint32_t>(u) : g.n[k] - 1) : 0u;
    }
    const uint32_t x = c[0] + g.n[0] * c[1];
    cell[i] = x;
    atomicAdd(hist + x, 1u);
}

__global__ void k_muon_slots(const uint32_t* __restrict__ cell, uint64_t n, const uint64_t* __restrict__ cstart,
                             uint32_t* __restrict__ cursor, uint32_t* __restrict__ kslot) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t x = cell[i];
    kslot[i] = static_cast<uint32_t>(cstart[x] + atomicAdd(cursor + x, 1u));
}

void launch_muon_slots(const double* scat, uint64_t n, muto_grid g, uint32_t* cell, uint32_t* hist,
                       uint64_t* cstart, uint32_t* cursor, void* scan_scratch, uint32_t* kslot, cudaStream_t s) {
    if (n == 0) return;
    const uint64_t nc = static_cast<uint64_t>(g.nx) * g.ny;
    (void)cudaMemsetAsync(hist, 0, (nc + 1) * sizeof(uint32_t), s);
    (void)cudaMemsetAsync(cursor, 0, (nc + 1) * sizeof(uint32_t), s);
    k_muon_cells<<<blocks_for(n), kThreads, 0, s>>>(scat, n, make_dev_grid(g), cell, hist);
    count_launches(1);
    scan_u32_to_u64(hist, cstart, nc, scan_scratch, s);
    k_muon_slots<<<blocks_for(n), kThreads, 0, s>>>(cell, n, cstart, cursor, kslot);
    count_launches(1);
}

void launch_siddon_batch(muto_grid g, const double* p1, const double* p2, uint64_t n, uint32_t cap, uint32_t* xyz,
                         double* len, uint32_t* counts, cudaStream_t s) {
    if (n == 0) return;
    k_siddon_batch<<<blocks_for(n, 128), 128, 0, s>>>(make_dev_grid(g), p1, p2, n, cap, xyz, len, counts); count_launches(1);
}

}  // namespace muto

namespace muto {

uint32_t voxel_class_blocks(uint64_t V) { return blocks_for(V); }

void launch_segment_starts(const uint32_t* mult, uint32_t V, const muto_grid* column_order, uint32_t* mcol,
                           uint64_t* scol, void* scan_scratch, uint64_t* start, cudaStream_t s) {
    if (!column_order || static_cast<uint64_t>(column_order->nx) * column_order->ny * column_order->nz != V ||
        V == 0) {
        scan_u32_to_u64(mult, start, V, scan_scratch, s);
        return;
    }
    const uint32_t nx = column_order->nx, ny = column_order->ny, nz = column_order->nz;
    k_column_mult<<<blocks_for(V), kThreads, 0, s>>>(mult, V, nx, ny, nz, mcol);
    count_launches(1);
    scan_u32_to_u64(mcol, scol, V, scan_scratch, s);
    k_column_starts<<<blocks_for(V), kThreads, 0, s>>>(scol, V, nx, ny, nz, start);
    count_launches(1);
}

template <typename Real>
void launch_voxel_classes(const uint32_t* mult, const uint64_t* start, uint32_t V, const muto_grid* column_order,
                          uint32_t* counts, uint64_t* first, void* scan_scratch, VoxDesc* out, cudaStream_t s) {
    if (V == 0) return;
    const uint32_t nb = blocks_for(V);
    uint32_t nx = 0, ny = 0, nz = 0;
    if (column_order && static_cast<uint64_t>(column_order->nx) * column_order->ny * column_order->nz == V) {
        nx = column_order->nx;
        ny = column_order->ny;
        nz = column_order->nz;
    }
    k_class_count<Real><<<nb, kThreads, 0, s>>>(mult, V, nb, nx, ny, nz, counts);
    count_launches(1);
    scan_u32_to_u64(counts, first, static_cast<uint64_t>(nb) * kVoxClasses, scan_scratch, s);
    k_class_scatter<Real><<<nb, kThreads, 0, s>>>(mult, start, V, nb, nx, ny, nz, first, out);
    count_launches(1);
}
template void launch_voxel_classes<float>(const uint32_t*, const uint64_t*, uint32_t, const muto_grid*, uint32_t*,
                                          uint64_t*, void*, VoxDesc*, cudaStream_t);
template void launch_voxel_classes<double>(const uint32_t*, const uint64_t*, uint32_t, const muto_grid*, uint32_t*,
                                           uint64_t*, void*, VoxDesc*, cudaStream_t);

}  // namespace muto

namespace muto {

void launch_brick_indices(uint32_t* vidx, uint64_t n, BrickDims b, uint32_t V, cudaStream_t s) {
    if (n == 0) return;
    k_brick_indices<<<blocks_for(n), kThreads, 0, s>>>(vidx, n, b, V);
    count_launches(1);
}

void launch_unbrick_indices(const uint32_t* in, uint32_t* out, uint64_t n, BrickDims b, cudaStream_t s) {
    if (n == 0) return;
    k_unbrick_indices<<<blocks_for(n), kThreads, 0, s>>>(in, out, n, b);
    count_launches(1);
}

template <typename Real>
void launch_brick_lambda(const Real* lam, uint32_t V, BrickDims b, Real* lam_b, cudaStream_t s) {
    if (V == 0) return;
    k_brick_lambda<Real><<<blocks_for(V), kThreads, 0, s>>>(lam, V, b, lam_b);
    count_launches(1);
}
template void launch_brick_lambda<float>(const float*, uint32_t, BrickDims, float*, cudaStream_t);
template void launch_brick_lambda<double>(const double*, uint32_t, BrickDims, double*, cudaStream_t);

}  // namespace muto
