// Straight-line reconstruction (MutoSLR::reconstruct, src/MutoSLR.cpp:47-103)
// and the first pass of its iterative form (MutoSLRIter, src/MutoSLRIter.cpp:
// 15-83), one thread per ray: the incoming and outgoing lines cut at the
// grid's top and bottom planes, the Siddon walk of the straight line between
// the two points (bit-exact, as for the other methods), and per voxel the
// mean squared projected angle shared by length^2 or equally.  Sums are FP64
// atomics.  The later passes of the iterative form are order-dependent (each
// muon sees the image the muons before it left): they run over the walked
// paths level by level (k_slr_iter_levels: muons of one level share no
// voxel), or muon after muon on one warp (k_slr_iter_pass).
#include "common.cuh"
#include "geometry.cuh"

namespace muto {
namespace {

// per-ray quantities of :63-77
struct SlrRay {
    double a2;        // axz^2 + ayz^2
    double p_in[3], p_out[3];
    double l_total;   // |p_in - p_out|
};

__device__ __forceinline__ SlrRay slr_ray(const muto_ray& r, const DevGrid& g, double z_lo, double z_hi, double mag) {
    SlrRay o;
    const double axz = dmul(dsub(atan2(r.din[0], r.din[2]), atan2(r.dout[0], r.dout[2])), mag);
    const double ayz = dmul(dsub(atan2(r.din[1], r.din[2]), atan2(r.dout[1], r.dout[2])), mag);
    o.a2 = dadd(dmul(axz, axz), dmul(ayz, ayz));
    const double t_in = ddiv(dsub(z_hi, r.pin[2]), r.din[2]);
    const double t_out = ddiv(dsub(z_lo, r.pout[2]), r.dout[2]);
    double d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        o.p_in[k] = dadd(r.pin[k], dmul(t_in, r.din[k]));
        o.p_out[k] = dadd(r.pout[k], dmul(t_out, r.dout[k]));
        d[k] = dsub(o.p_in[k], o.p_out[k]);
    }
    o.l_total = __dsqrt_rn(dot3(d, d));
    (void)g;
    return o;
}

struct CountSink {
    uint32_t n = 0;
    __device__ void operator()(uint32_t, uint32_t, uint32_t, double) { ++n; }
};

struct SlrSink {
    double* img;
    double* weight;
    uint32_t nx, ny, nz;
    double dz, a2, l_total, share, e2;  // share: a2 / 2 / n^2 (equal shares)
    int length_weighted, has_energy;
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) {
        if (x >= nx || y >= ny || z >= nz) return;  // never for a walk inside the grid
        const uint64_t j = static_cast<uint64_t>(x) + static_cast<uint64_t>(nx) * (y + static_cast<uint64_t>(ny) * z);
        double iv;
        if (length_weighted) {  // :80-83
            atomicAdd(weight + j, ddiv(l, dz));
            const double f = ddiv(l, l_total);
            iv = dmul(dmul(dmul(a2, 0.5), f), f);
        } else {  // :84-86
            atomicAdd(weight + j, 1.0);
            iv = share;
        }
        if (has_energy) iv = dmul(iv, e2);  // :87-89
        atomicAdd(img + j, iv);
    }
};

__global__ void k_slr(SlrArgs a) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const DevGrid g = make_dev_grid(a.g);
    const muto_ray r = a.rays[i];
    const double z_lo = a.g.z_min;                                               // :57
    const double z_hi = dadd(a.g.z_min, dmul(a.g.dz, static_cast<double>(a.g.nz)));  // :58
    const SlrRay s = slr_ray(r, g, z_lo, z_hi, a.mag);
    double share = 0.0;
    if (!a.length_weighted) {  // the equal share needs the path's voxel count first
        CountSink c;
        siddon_walk(g, s.p_in, s.p_out, c);
        const uint64_t n = c.n;
        share = ddiv(dmul(s.a2, 0.5), static_cast<double>(n * n));
    }
    SlrSink sink{a.img, a.weight, g.n[0], g.n[1], g.n[2], a.g.dz, s.a2, s.l_total, share, dmul(r.ein, r.ein),
                 a.length_weighted, a.has_energy};
    siddon_walk(g, s.p_in, s.p_out, sink);
}

// The walked straight lines, for the in-place passes: per ray its voxel
// count (first call) or its voxels and lengths at off[i] (second call).
struct PathSink {
    uint32_t* vox;
    double* len;
    uint32_t nx, ny;
    uint32_t k = 0;
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) {
        if (vox) {
            vox[k] = x + nx * (y + ny * z);
            len[k] = l;
        }
        ++k;
    }
};

__global__ void k_slr_paths(SlrArgs a, const uint64_t* __restrict__ off, uint32_t* __restrict__ counts,
                            uint32_t* __restrict__ vox, double* __restrict__ len) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const DevGrid g = make_dev_grid(a.g);
    const double z_lo = a.g.z_min;
    const double z_hi = dadd(a.g.z_min, dmul(a.g.dz, static_cast<double>(a.g.nz)));
    const SlrRay s = slr_ray(a.rays[i], g, z_lo, z_hi, a.mag);
    PathSink p{off ? vox + off[i] : nullptr, off ? len + off[i] : nullptr, g.n[0], g.n[1]};
    siddon_walk(g, s.p_in, s.p_out, p);
    if (!off) counts[i] = p.k;
}

// The pass-independent terms of every pair, once at set-up: the weight
// increment (length / dz, or 1) and the image increment before it is scaled
// by the voxel's part of the path's sum (a^2 / 2 (length / l_total)^2, or the
// equal share a^2 / 2 / n^2), with the arithmetic of :80-89; and ein^2 per
// muon.  A thread per muon.
__global__ void k_slr_pair_terms(SlrArgs a, SlrPass p) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const DevGrid g = make_dev_grid(a.g);
    const double z_lo = a.g.z_min;
    const double z_hi = dadd(a.g.z_min, dmul(a.g.dz, static_cast<double>(a.g.nz)));
    const muto_ray r = a.rays[i];
    const SlrRay s = slr_ray(r, g, z_lo, z_hi, a.mag);
    const uint64_t p0 = p.off[i];
    const uint32_t n = static_cast<uint32_t>(p.off[i + 1] - p0);
    const double share = ddiv(dmul(s.a2, 0.5), static_cast<double>(static_cast<uint64_t>(n) * n));
    for (uint32_t k = 0; k < n; ++k) {
        const double l = p.len[p0 + k];
        if (a.length_weighted) {
            p.winc[p0 + k] = ddiv(l, a.g.dz);
            const double f = ddiv(l, s.l_total);
            p.iv0[p0 + k] = dmul(dmul(dmul(s.a2, 0.5), f), f);
        } else {
            p.winc[p0 + k] = 1.0;
            p.iv0[p0 + k] = share;
        }
    }
    p.e2[i] = dmul(r.ein, r.ein);
}

// One muon of a later pass of the iterative form (src/MutoSLRIter.cpp:40-71
// with iter != 0), on one warp: the warp reads the image on the muon's path,
// sums it (lane partials, then the warp's sum), and adds to each voxel its
// increment times the voxel's part of that sum (:64-66).
// img / weight: the image and weight sums (global memory, or a copy in
// shared memory).
__device__ __forceinline__ void slr_iter_muon(const SlrArgs& a, const SlrPass& p, uint64_t i, int lane, double* img,
                                              double* weight) {
    const uint64_t p0 = p.off[i];
    const uint32_t n = static_cast<uint32_t>(p.off[i + 1] - p0);
    double part = 0.0;  // :49-52
    for (uint32_t k = lane; k < n; k += 32) part = dadd(part, img[p.vox[p0 + k]]);
    const double total = warp_sum(part);
    const double e2 = a.has_energy ? p.e2[i] : 0.0;
    for (uint32_t k = lane; k < n; k += 32) {
        const uint32_t j = p.vox[p0 + k];
        weight[j] = dadd(weight[j], p.winc[p0 + k]);
        double iv = dmul(p.iv0[p0 + k], ddiv(img[j], total));
        if (a.has_energy) iv = dmul(iv, e2);  // :87-89
        img[j] = dadd(img[j], iv);
    }
}

// A later pass muon after muon on a single warp: a muon's stores are ordered
// before the next muon's loads by __syncwarp; no other warp touches the image.
__global__ void k_slr_iter_pass(SlrArgs a, SlrPass p) {
    const int lane = threadIdx.x & 31;
    if (threadIdx.x >= 32) return;
    for (uint64_t i = 0; i < a.n; ++i) {
        slr_iter_muon(a, p, i, lane, a.img, a.weight);
        __syncwarp();
    }
}

// The pairs of every muon copied into level order: muon q of the level
// order (order[q]) gets its pairs at fo[q] .. fo[q+1], so a level's data is
// contiguous and found from the level's start alone.  A warp per muon.
__global__ void k_slr_flatten(SlrPass p, const uint32_t* __restrict__ order, uint64_t nt, SlrFlat f) {
    const uint64_t q = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= nt) return;
    const uint32_t i = order[q];
    const uint64_t s0 = p.off[i], n = p.off[i + 1] - s0, d0 = f.fo[q];
    for (uint64_t k = lane; k < n; k += 32) {
        f.vox[d0 + k] = p.vox[s0 + k];
        f.iv0[d0 + k] = p.iv0[s0 + k];
        f.winc[d0 + k] = p.winc[s0 + k];
    }
    if (lane == 0) f.e2[q] = p.e2[i];
}

// One muon of the level order on one warp, the arithmetic of slr_iter_muon;
// the first pair of each lane (k = lane) comes in already loaded (v0, i0,
// w0; valid when lane < n), the rest is loaded here.
__device__ __forceinline__ void slr_flat_muon(const SlrArgs& a, const SlrFlat& f, uint64_t p0, uint32_t n, double e2,
                                              uint32_t v0, double i0, double w0, int lane, double* img,
                                              double* weight) {
    double part = 0.0;  // :49-52, the same order of additions as slr_iter_muon
    if (static_cast<uint32_t>(lane) < n) part = dadd(part, img[v0]);
    for (uint32_t k = lane + 32; k < n; k += 32) part = dadd(part, img[f.vox[p0 + k]]);
    const double total = warp_sum(part);
    if (static_cast<uint32_t>(lane) < n) {
        weight[v0] = dadd(weight[v0], w0);
        double iv = dmul(i0, ddiv(img[v0], total));
        if (a.has_energy) iv = dmul(iv, e2);  // :87-89
        img[v0] = dadd(img[v0], iv);
    }
    for (uint32_t k = lane + 32; k < n; k += 32) {
        const uint32_t j = f.vox[p0 + k];
        weight[j] = dadd(weight[j], f.winc[p0 + k]);
        double iv = dmul(f.iv0[p0 + k], ddiv(img[j], total));
        if (a.has_energy) iv = dmul(iv, e2);
        img[j] = dadd(img[j], iv);
    }
}

// A later pass level by level.  A muon's level is one more than the highest
// level among the earlier muons that share a voxel with it, so two muons of
// one level share no voxel, and every voxel meets its muons in index order:
// each muon reads and writes the image state it would see in the sequential
// loop, whatever the order inside a level.  One block: its warps take the
// muons of a level, and the block barrier orders the levels (global stores
// before it are visible to the whole block after it).  With SMEM the image
// and weight sums (2 V doubles) are copied into shared memory for the pass
// and back after it.  The next level's muon offsets are loaded while the
// current level runs, and its first pair per lane just before the barrier
// (neither depends on the image).
template <bool SMEM>
__global__ void __launch_bounds__(1024) k_slr_iter_levels(SlrArgs a, SlrFlat f, const uint32_t* __restrict__ lstart,
                                                          uint32_t levels) {
    extern __shared__ double slr_smem[];
    const int lane = threadIdx.x & 31;
    const uint32_t warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t V = a.g.nx * a.g.ny * a.g.nz;
    double* img = a.img;
    double* weight = a.weight;
    if (SMEM) {
        img = slr_smem;
        weight = slr_smem + V;
        for (uint32_t j = threadIdx.x; j < V; j += blockDim.x) {
            img[j] = a.img[j];
            weight[j] = a.weight[j];
        }
        __syncthreads();
    }
    // this warp's first muon of level 0 and its first pair per lane
    uint32_t e = lstart[1];
    uint32_t q = lstart[0] + warp;
    uint64_t p0 = 0;
    uint32_t n = 0, v0 = 0;
    double i0 = 0.0, w0 = 0.0, e2 = 0.0;
    if (q < e) {
        p0 = f.fo[q];
        n = static_cast<uint32_t>(f.fo[q + 1] - p0);
        e2 = f.e2[q];
        if (static_cast<uint32_t>(lane) < n) {
            v0 = f.vox[p0 + lane];
            i0 = f.iv0[p0 + lane];
            w0 = f.winc[p0 + lane];
        }
    }
    for (uint32_t l = 0; l < levels; ++l) {
        // the next level's first muon for this warp: its offsets now
        const uint32_t en = l + 1 < levels ? lstart[l + 2] : e;
        const uint32_t qn = e + warp;
        const bool has_next = l + 1 < levels && qn < en;
        uint64_t p0n = 0, p1n = 0;
        if (has_next) {
            p0n = f.fo[qn];
            p1n = f.fo[qn + 1];
        }
        if (q < e) slr_flat_muon(a, f, p0, n, e2, v0, i0, w0, lane, img, weight);
        for (uint32_t q2 = q + nw; q2 < e; q2 += nw) {  // more muons than warps in this level
            const uint64_t s0 = f.fo[q2];
            const uint32_t m = static_cast<uint32_t>(f.fo[q2 + 1] - s0);
            const bool in = static_cast<uint32_t>(lane) < m;
            slr_flat_muon(a, f, s0, m, f.e2[q2], in ? f.vox[s0 + lane] : 0u, in ? f.iv0[s0 + lane] : 0.0,
                          in ? f.winc[s0 + lane] : 0.0, lane, img, weight);
        }
        // the next level's first pair per lane, before the barrier
        q = qn;
        e = en;
        n = 0;
        if (has_next) {
            p0 = p0n;
            n = static_cast<uint32_t>(p1n - p0n);
            e2 = f.e2[qn];
            if (static_cast<uint32_t>(lane) < n) {
                v0 = f.vox[p0 + lane];
                i0 = f.iv0[p0 + lane];
                w0 = f.winc[p0 + lane];
            }
        }
        __syncthreads();
    }
    if (SMEM) {
        for (uint32_t j = threadIdx.x; j < V; j += blockDim.x) {
            a.img[j] = img[j];
            a.weight[j] = weight[j];
        }
    }
}

}  // namespace

void launch_slr(const SlrArgs& a, cudaStream_t s) {
    if (a.n == 0) return;
    k_slr<<<static_cast<unsigned>((a.n + 127) / 128), 128, 0, s>>>(a);
    count_launches(1);
}

void launch_slr_paths(const SlrArgs& a, const uint64_t* off, uint32_t* counts, uint32_t* vox, double* len,
                      cudaStream_t s) {
    if (a.n == 0) return;
    k_slr_paths<<<static_cast<unsigned>((a.n + 127) / 128), 128, 0, s>>>(a, off, counts, vox, len);
    count_launches(1);
}

void launch_slr_pair_terms(const SlrArgs& a, const SlrPass& p, cudaStream_t s) {
    if (a.n == 0) return;
    k_slr_pair_terms<<<static_cast<unsigned>((a.n + 127) / 128), 128, 0, s>>>(a, p);
    count_launches(1);
}

void launch_slr_iter_pass(const SlrArgs& a, const SlrPass& p, cudaStream_t s) {
    if (a.n == 0) return;
    k_slr_iter_pass<<<1, 32, 0, s>>>(a, p);
    count_launches(1);
}

void launch_slr_flatten(const SlrPass& p, const uint32_t* order, uint64_t nt, const SlrFlat& f, cudaStream_t s) {
    if (nt == 0) return;
    k_slr_flatten<<<static_cast<unsigned>((nt * 32 + 255) / 256), 256, 0, s>>>(p, order, nt, f);
    count_launches(1);
}

void launch_slr_iter_levels(const SlrArgs& a, const SlrFlat& f, const uint32_t* lstart, uint32_t levels,
                            size_t smem_optin, cudaStream_t s) {
    if (a.n == 0 || levels == 0) return;
    const size_t bytes = 2 * sizeof(double) * static_cast<size_t>(a.g.nx) * a.g.ny * a.g.nz;
    if (bytes <= smem_optin &&
        cudaFuncSetAttribute(k_slr_iter_levels<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(bytes)) == cudaSuccess) {
        k_slr_iter_levels<true><<<1, 1024, bytes, s>>>(a, f, lstart, levels);
    } else {
        (void)cudaGetLastError();  // a refused attribute: the pass stays in global memory
        k_slr_iter_levels<false><<<1, 1024, 0, s>>>(a, f, lstart, levels);
    }
    count_launches(1);
}

}  // namespace muto
