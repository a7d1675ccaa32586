// Muon pass of an EM iteration (src/MutoMLSD.cpp:188-195): for every kept muon
// the covariance gather Sigma_i = pr^2 sum_j lambda_j W_ij + E
// (getCovarianceMatrix, :442-449), its determinant, inverse and cost
// (updateSValueMatrix, :451-469), folded into three coefficients
//     pr^2 (1/2 xyS_ij - tr(Sigma_i^-1 W_ij)) = k0 W00 + k1 W01 + k2 W11
// (xyS = sum over the x and y planes of u^T W u with u = Sigma_i^-1 (S, D)),
// which the voxel pass (em_voxel.cu) turns into s_ij = 2 l + g l^2.
//
// Work layout.  Kept muons are cut into tiles of consecutive muons whose pairs
// (voxel index, L, T) fit in shared memory.  A persistent CTA walks its tiles
// with two stage buffers: while it works on one tile, the TMA engine copies the
// next one (cp.async.bulk global -> shared, completion on an mbarrier), so
// every pair byte is read from HBM once per iteration with the copy latency
// hidden.  Per tile:
//   gather  every thread fetches lambda_j (L2-resident) for 8 pairs at once;
//   sum     GROUP lanes per muon add lambda_j W_ij in the storage precision;
//   2x2     one thread per muon: Sigma in FP64, determinant and inverse in
//           FP64, cost in FP64, the k coefficients written to global memory.
#include "common.cuh"

namespace muto {
namespace {

constexpr int kThreads = 256;
constexpr int kGatherUnroll = 8;

// Shared memory: two stage buffers (per-pair buffers hold TP + 8 entries, the
// tile's range widened to 16-byte boundaries) and the working arrays.
template <typename Real>
struct MuonLayout {
    size_t off[2], sd[2], pr2[2], idx[2], L[2], T[2], lam, sig, bar, total;
    __host__ __device__ MuonLayout(int TP, int TM) {
        auto up = [](size_t x) { return (x + 15) & ~static_cast<size_t>(15); };
        size_t p = 0;
        for (int b = 0; b < 2; ++b) {
            off[b] = p; p = up(p + sizeof(uint64_t) * (TM + 4));
            sd[b] = p;  p = up(p + sizeof(typename Vec4<Real>::type) * TM);
            pr2[b] = p; p = up(p + sizeof(Real) * (TM + 8));
            idx[b] = p; p = up(p + sizeof(uint32_t) * (TP + 8));
            L[b] = p;   p = up(p + sizeof(Real) * (TP + 8));
            T[b] = p;   p = up(p + sizeof(Real) * (TP + 8));
        }
        lam = p; p = up(p + sizeof(Real) * TP);
        sig = p; p = up(p + sizeof(Real) * 3 * TM);
        bar = p; p = up(p + 2 * sizeof(uint64_t));
        total = p;
    }
};

// --- TMA bulk copy + mbarrier (PTX) -----------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// [b, e) of an array of `size`-byte elements widened to 16-byte boundaries
__device__ __forceinline__ void widen(uint64_t b, uint64_t e, uint32_t size, uint64_t* first, uint32_t* bytes) {
    const uint64_t per = 16 / size;
    const uint64_t f = b - b % per;
    const uint64_t l = ((e + per - 1) / per) * per;
    *first = f;
    *bytes = static_cast<uint32_t>((l - f) * size);
}

// Bounded wait; false (and a recorded timeout) if the copies did not land.
__device__ __forceinline__ bool wait_stage(uint64_t* bar, uint32_t parity, Counters* ctr) {
    for (uint32_t spin = 0; spin < (1u << 22); ++spin)
        if (mbar_try_wait(bar, parity)) return true;
    if (threadIdx.x == 0) atomicAdd(&ctr->timeouts, 1ull);
    return false;
}

template <typename Real>
struct Stage {
    uint64_t* off;
    typename Vec4<Real>::type* sd;
    Real* pr2;
    uint32_t* idx;
    Real* L;
    Real* T;
};

// thread 0: copy tile t into a stage buffer
template <typename Real>
__device__ __forceinline__ void issue_tile(const MuonPassArgs<Real>& a, uint32_t t, const Stage<Real>& st,
                                           uint64_t* bar) {
    using R4 = typename Vec4<Real>::type;
    const uint32_t mb = a.tile_mb[t], me = a.tile_mb[t + 1];
    const uint64_t pb = a.off[mb], pe = a.off[me];
    uint64_t f4, fr, fo, fp;
    uint32_t b4, br, bo, bp;
    widen(pb, pe, 4, &f4, &b4);
    widen(pb, pe, sizeof(Real), &fr, &br);
    widen(mb, me + 1, 8, &fo, &bo);
    widen(mb, me, sizeof(Real), &fp, &bp);
    const uint32_t bsd = static_cast<uint32_t>((me - mb) * sizeof(R4));
    fence_proxy_async();  // earlier generic-proxy reads of this buffer are ordered before the copies
    mbar_arrive_expect_tx(bar, b4 + 2u * br + bo + bsd + bp);
    if (b4) {  // a tile of muons with empty paths has no pair bytes
        bulk_load(st.idx, a.vidx + f4, b4, bar);
        bulk_load(st.L, a.L + fr, br, bar);
        bulk_load(st.T, a.T + fr, br, bar);
    }
    bulk_load(st.off, a.off + fo, bo, bar);
    bulk_load(st.sd, a.sd + mb, bsd, bar);
    bulk_load(st.pr2, a.pr2 + fp, bp, bar);
}

template <typename Real, int GROUP>
__global__ void __launch_bounds__(kThreads, 2) k_em_muon(MuonPassArgs<Real> a, int TP, int TM) {
    using R4 = typename Vec4<Real>::type;
    extern __shared__ __align__(128) unsigned char smem[];
    const MuonLayout<Real> lay(TP, TM);
    Stage<Real> st[2];
    for (int b = 0; b < 2; ++b) {
        st[b].off = reinterpret_cast<uint64_t*>(smem + lay.off[b]);
        st[b].sd = reinterpret_cast<R4*>(smem + lay.sd[b]);
        st[b].pr2 = reinterpret_cast<Real*>(smem + lay.pr2[b]);
        st[b].idx = reinterpret_cast<uint32_t*>(smem + lay.idx[b]);
        st[b].L = reinterpret_cast<Real*>(smem + lay.L[b]);
        st[b].T = reinterpret_cast<Real*>(smem + lay.T[b]);
    }
    Real* s_lam = reinterpret_cast<Real*>(smem + lay.lam);
    Real* s_sig = reinterpret_cast<Real*>(smem + lay.sig);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + lay.bar);

    const int tid = threadIdx.x, lane = tid & 31;
    const int group = tid / GROUP, glane = tid % GROUP;
    constexpr int kGroups = kThreads / GROUP;
    const unsigned gmask = GROUP == 32 ? kFull : (((1u << GROUP) - 1u) << (lane & ~(GROUP - 1)));
    const uint32_t V = a.V;
    double cost_local = 0.0;
    unsigned long long singular_local = 0;

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
    }
    __syncthreads();
    if (tid == 0 && blockIdx.x < a.ntiles) issue_tile(a, blockIdx.x, st[0], &bar[0]);

    uint32_t it = 0;
    for (uint32_t t = blockIdx.x; t < a.ntiles; t += gridDim.x, ++it) {
        const int b = static_cast<int>(it & 1u);
        const uint32_t tn = t + gridDim.x;
        // the other buffer was released by the barrier that closed the previous tile
        if (tid == 0 && tn < a.ntiles) issue_tile(a, tn, st[b ^ 1], &bar[b ^ 1]);
        const bool landed = wait_stage(&bar[b], (it >> 1) & 1u, a.ctr);
        if (!__syncthreads_and(landed)) break;  // uniform exit; never expected

        const Stage<Real>& S = st[b];
        const uint32_t mb = a.tile_mb[t], me = a.tile_mb[t + 1];
        const int nm = static_cast<int>(me - mb);
        const uint64_t pb = a.off[mb];
        const int np = static_cast<int>(a.off[me] - pb);
        const int sh4 = static_cast<int>(pb % 4u);                       // 4-byte arrays
        const int shr = static_cast<int>(pb % (16u / sizeof(Real)));    // Real arrays
        const int sho = static_cast<int>(mb % 2u);                       // offsets
        const int shp = static_cast<int>(mb % (16u / sizeof(Real)));    // pr^2

        // ---- gather lambda for every pair of the tile ------------------------
        for (int k0 = tid; k0 < np; k0 += kGatherUnroll * kThreads) {
            Real lv[kGatherUnroll];
#pragma unroll
            for (int u = 0; u < kGatherUnroll; ++u) {
                const int k = k0 + u * kThreads;
                const uint32_t j = k < np ? S.idx[sh4 + k] : 0xffffffffu;
                lv[u] = j < V ? __ldg(a.lam + j) : Real(0);
            }
#pragma unroll
            for (int u = 0; u < kGatherUnroll; ++u) {
                const int k = k0 + u * kThreads;
                if (k < np) s_lam[k] = lv[u];
            }
        }
        __syncthreads();

        // ---- covariance sums, GROUP lanes per muon ---------------------------
        for (int m = group; m < nm; m += kGroups) {
            const int kb = static_cast<int>(S.off[sho + m] - pb), ke = static_cast<int>(S.off[sho + m + 1] - pb);
            Real c0 = 0, c1 = 0, c2 = 0;
            for (int k = kb + glane; k < ke; k += GROUP) {
                const Real L = S.L[shr + k], T = S.T[shr + k], l = s_lam[k];
                const Real LT = L * T;
                c0 += l * L;
                c1 += l * (LT + L * L * Real(0.5));
                c2 += l * (L * L * L * Real(1.0 / 3.0) + (L + T) * LT);
            }
#pragma unroll
            for (int o = GROUP / 2; o > 0; o >>= 1) {
                c0 += __shfl_xor_sync(gmask, c0, o, GROUP);
                c1 += __shfl_xor_sync(gmask, c1, o, GROUP);
                c2 += __shfl_xor_sync(gmask, c2, o, GROUP);
            }
            if (glane == 0) {
                s_sig[3 * m + 0] = c0;
                s_sig[3 * m + 1] = c1;
                s_sig[3 * m + 2] = c2;
            }
        }
        __syncthreads();

        // ---- per-muon 2x2 algebra, one thread per muon -----------------------
        for (int m = tid; m < nm; m += kThreads) {
            const Real pr2 = S.pr2[shp + m];
            const double p2 = static_cast<double>(pr2);
            const double S00 = p2 * static_cast<double>(s_sig[3 * m + 0]) + a.E00;
            const double S01 = p2 * static_cast<double>(s_sig[3 * m + 1]) + a.E01;
            const double S11 = p2 * static_cast<double>(s_sig[3 * m + 2]) + a.E11;
            const double det = S00 * S11 - S01 * S01;
            R4 kv;
            kv.x = kv.y = kv.z = kv.w = Real(0);
            if (fabs(det) > 1e-12) {  // Eigen computeInverseAndDetWithCheck threshold
                const double r = 1.0 / det;
                const double i00 = S11 * r, i01 = -S01 * r, i11 = S00 * r;
                const R4 v = S.sd[m];
                // u = Sigma^-1 (S, D) per plane, in the storage precision
                const Real f00 = static_cast<Real>(i00), f01 = static_cast<Real>(i01), f11 = static_cast<Real>(i11);
                const Real ux0 = f00 * v.x + f01 * v.y, ux1 = f01 * v.x + f11 * v.y;
                const Real uy0 = f00 * v.z + f01 * v.w, uy1 = f01 * v.z + f11 * v.w;
                kv.x = pr2 * (Real(0.5) * (ux0 * ux0 + uy0 * uy0) - f00);
                kv.y = pr2 * ((ux0 * ux1 + uy0 * uy1) - Real(2) * f01);
                kv.z = pr2 * (Real(0.5) * (ux1 * ux1 + uy1 * uy1) - f11);
                if (det <= 0) {
                    ++singular_local;
                } else if (a.compute_cost) {
                    const double sx = v.x, dx = v.y, sy = v.z, dy = v.w;
                    cost_local += log(det) + ((sx * sx + sy * sy) * i00 + (dx * dx + dy * dy) * i11 +
                                              (sx * dx + sy * dy) * 2.0 * i01) * 0.5;
                }
            } else {
                ++singular_local;  // inverse left at zero: s_ij = 2 l_j
            }
            a.kout[a.kslot ? a.kslot[mb + m] : mb + m] = kv;
        }
        __syncthreads();  // closes the tile: its stage buffer may be refilled
    }

    // block reduction of the cost and singular counts
    __shared__ double red[kThreads / 32];
    __shared__ unsigned long long redn[kThreads / 32];
    double c = warp_sum(cost_local);
    unsigned long long ns = singular_local;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ns += __shfl_xor_sync(kFull, ns, o);
    if (lane == 0) {
        red[tid >> 5] = c;
        redn[tid >> 5] = ns;
    }
    __syncthreads();
    if (tid == 0) {
        double tc = 0.0;
        unsigned long long tn = 0;
        for (int w = 0; w < kThreads / 32; ++w) {
            tc += red[w];
            tn += redn[w];
        }
        if (a.compute_cost && tc != 0.0) atomicAdd(&a.ctr->cost_sum, tc);
        if (tn) atomicAdd(&a.ctr->singular, tn);
    }
}

// ---------------------------------------------------------------------------
// Warp-batched variant: no shared memory and no block barriers.  A warp takes
// 32 consecutive muons; GROUP lanes sum one muon's lambda_j W_ij with
// coalesced streaming loads of its pairs and L2 gathers of lambda, the sum
// lands in the lane of that muon, and the 32 lanes then do the FP64 2x2
// algebra of their 32 muons together (the FP64 pipe is busy for one warp
// instruction per 32 muons, not per muon).
// ---------------------------------------------------------------------------
template <typename Real, int GROUP>
__global__ void __launch_bounds__(kThreads) k_em_muon_warp(MuonPassArgs<Real> a, uint32_t n_muons) {
    using R4 = typename Vec4<Real>::type;
    constexpr int U = 5;                    // pair loads in flight per lane per round
    constexpr int kPer = 32 / GROUP;        // muons summed at once per warp
    const int lane = threadIdx.x & 31;
    const int sub = lane / GROUP, glane = lane % GROUP;
    const unsigned gmask = GROUP == 32 ? kFull : (((1u << GROUP) - 1u) << (lane & ~(GROUP - 1)));
    const uint32_t V = a.V;
    const uint64_t warp = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
    const uint64_t nbatch = (static_cast<uint64_t>(n_muons) + 31) / 32;
    double cost_local = 0.0;
    unsigned long long singular_local = 0;

    for (uint64_t bt = warp; bt < nbatch; bt += nwarps) {
        const uint64_t m0 = bt * 32;
        Real my0 = 0, my1 = 0, my2 = 0;  // the sums of muon m0 + lane
        for (int q = 0; q < 32; q += kPer) {
            const uint64_t m = m0 + q + sub;
            Real c0 = 0, c1 = 0, c2 = 0;
            if (m < n_muons) {
                const uint64_t pb = a.off[m], pe = a.off[m + 1];
                for (uint64_t k0 = pb + glane; k0 < pe; k0 += GROUP * U) {
                    uint32_t jj[U];
                    Real ll[U], tt[U], lam[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const uint64_t k = k0 + static_cast<uint64_t>(u) * GROUP;
                        jj[u] = 0xffffffffu;
                        if (k < pe) {
                            jj[u] = __ldcs(a.vidx + k);
                            ll[u] = __ldcs(a.L + k);
                            tt[u] = __ldcs(a.T + k);
                        }
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) lam[u] = jj[u] < V ? __ldg(a.lam + jj[u]) : Real(0);
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        if (jj[u] != 0xffffffffu) {
                            const Real L = ll[u], T = tt[u], l = lam[u];
                            const Real LT = L * T;
                            c0 += l * L;
                            c1 += l * (LT + L * L * Real(0.5));
                            c2 += l * (L * L * L * Real(1.0 / 3.0) + (L + T) * LT);
                        }
                    }
                }
            }
#pragma unroll
            for (int o = GROUP / 2; o > 0; o >>= 1) {
                c0 += __shfl_xor_sync(gmask, c0, o, GROUP);
                c1 += __shfl_xor_sync(gmask, c1, o, GROUP);
                c2 += __shfl_xor_sync(gmask, c2, o, GROUP);
            }
            // lane q+s takes the sums of group s (its leader is lane s*GROUP)
            const int src = (lane - q >= 0 && lane - q < kPer) ? (lane - q) * GROUP : 0;
            const Real v0 = __shfl_sync(kFull, c0, src), v1 = __shfl_sync(kFull, c1, src),
                       v2 = __shfl_sync(kFull, c2, src);
            if (lane - q >= 0 && lane - q < kPer) {
                my0 = v0;
                my1 = v1;
                my2 = v2;
            }
        }
        // ---- FP64 2x2 algebra of the warp's 32 muons, one per lane ----------
        const uint64_t m = m0 + lane;
        if (m < n_muons) {
            const Real pr2 = a.pr2[m];
            const double p2 = static_cast<double>(pr2);
            const double S00 = p2 * static_cast<double>(my0) + a.E00;
            const double S01 = p2 * static_cast<double>(my1) + a.E01;
            const double S11 = p2 * static_cast<double>(my2) + a.E11;
            const double det = S00 * S11 - S01 * S01;
            R4 kv;
            kv.x = kv.y = kv.z = kv.w = Real(0);
            if (fabs(det) > 1e-12) {  // Eigen computeInverseAndDetWithCheck threshold
                const double r = 1.0 / det;
                const double i00 = S11 * r, i01 = -S01 * r, i11 = S00 * r;
                const R4 v = a.sd[m];
                const Real f00 = static_cast<Real>(i00), f01 = static_cast<Real>(i01), f11 = static_cast<Real>(i11);
                const Real ux0 = f00 * v.x + f01 * v.y, ux1 = f01 * v.x + f11 * v.y;
                const Real uy0 = f00 * v.z + f01 * v.w, uy1 = f01 * v.z + f11 * v.w;
                kv.x = pr2 * (Real(0.5) * (ux0 * ux0 + uy0 * uy0) - f00);
                kv.y = pr2 * ((ux0 * ux1 + uy0 * uy1) - Real(2) * f01);
                kv.z = pr2 * (Real(0.5) * (ux1 * ux1 + uy1 * uy1) - f11);
                if (det <= 0) {
                    ++singular_local;
                } else if (a.compute_cost) {
                    const double sx = v.x, dx = v.y, sy = v.z, dy = v.w;
                    cost_local += log(det) + ((sx * sx + sy * sy) * i00 + (dx * dx + dy * dy) * i11 +
                                              (sx * dx + sy * dy) * 2.0 * i01) * 0.5;
                }
            } else {
                ++singular_local;
            }
            a.kout[a.kslot ? a.kslot[m] : m] = kv;
        }
    }
    const double c = warp_sum(cost_local);
    unsigned long long ns = singular_local;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ns += __shfl_xor_sync(kFull, ns, o);
    if (lane == 0) {
        if (a.compute_cost && c != 0.0) atomicAdd(&a.ctr->cost_sum, c);
        if (ns) atomicAdd(&a.ctr->singular, ns);
    }
}

template <typename Real, int G>
cudaError_t set_smem(size_t smem) {
    return cudaFuncSetAttribute(k_em_muon<Real, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
}

}  // namespace

template <typename Real>
size_t em_muon_smem_bytes(int tile_pairs, int tile_muons) {
    return MuonLayout<Real>(tile_pairs, tile_muons).total;
}
template size_t em_muon_smem_bytes<float>(int, int);
template size_t em_muon_smem_bytes<double>(int, int);

template <typename Real>
cudaError_t em_muon_configure(int tile_pairs, int tile_muons) {
    const size_t smem = em_muon_smem_bytes<Real>(tile_pairs, tile_muons);
    cudaError_t e = set_smem<Real, 8>(smem);
    if (e == cudaSuccess) e = set_smem<Real, 16>(smem);
    if (e == cudaSuccess) e = set_smem<Real, 32>(smem);
    return e;
}
template cudaError_t em_muon_configure<float>(int, int);
template cudaError_t em_muon_configure<double>(int, int);

template <typename Real>
int em_muon_blocks(int tile_pairs, int tile_muons, int group) {
    const size_t smem = em_muon_smem_bytes<Real>(tile_pairs, tile_muons);
    int n = 0;
    cudaError_t e;
    if (group <= 8) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_em_muon<Real, 8>, kThreads, smem);
    else if (group <= 16) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_em_muon<Real, 16>, kThreads, smem);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_em_muon<Real, 32>, kThreads, smem);
    return (e == cudaSuccess && n > 0) ? n : 1;
}
template int em_muon_blocks<float>(int, int, int);
template int em_muon_blocks<double>(int, int, int);

template <typename Real>
void launch_em_muon(const MuonPassArgs<Real>& a, int tile_pairs, int tile_muons, int blocks, int group,
                    cudaStream_t s) {
    if (a.ntiles == 0) return;
    const size_t smem = em_muon_smem_bytes<Real>(tile_pairs, tile_muons);
    const unsigned nb = static_cast<unsigned>(blocks < static_cast<int>(a.ntiles) ? blocks : a.ntiles);
    if (group <= 8) k_em_muon<Real, 8><<<nb, kThreads, smem, s>>>(a, tile_pairs, tile_muons);
    else if (group <= 16) k_em_muon<Real, 16><<<nb, kThreads, smem, s>>>(a, tile_pairs, tile_muons);
    else k_em_muon<Real, 32><<<nb, kThreads, smem, s>>>(a, tile_pairs, tile_muons);
    count_launches(1);
}
template void launch_em_muon<float>(const MuonPassArgs<float>&, int, int, int, int, cudaStream_t);
template void launch_em_muon<double>(const MuonPassArgs<double>&, int, int, int, int, cudaStream_t);

template <typename Real>
int em_muon_warp_blocks(int group) {
    int n = 0;
    cudaError_t e;
    if (group <= 8) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_em_muon_warp<Real, 8>, kThreads, 0);
    else if (group <= 16) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_em_muon_warp<Real, 16>, kThreads, 0);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_em_muon_warp<Real, 32>, kThreads, 0);
    return (e == cudaSuccess && n > 0) ? n : 1;
}
template int em_muon_warp_blocks<float>(int);
template int em_muon_warp_blocks<double>(int);

template <typename Real>
void launch_em_muon_warp(const MuonPassArgs<Real>& a, uint32_t n_muons, int blocks, int group, cudaStream_t s) {
    if (n_muons == 0) return;
    const uint64_t batches = (static_cast<uint64_t>(n_muons) + 31) / 32;
    const uint64_t need = (batches + kThreads / 32 - 1) / (kThreads / 32);
    const unsigned nb = static_cast<unsigned>(need < static_cast<uint64_t>(blocks) ? need : blocks);
    if (group <= 8) k_em_muon_warp<Real, 8><<<nb, kThreads, 0, s>>>(a, n_muons);
    else if (group <= 16) k_em_muon_warp<Real, 16><<<nb, kThreads, 0, s>>>(a, n_muons);
    else k_em_muon_warp<Real, 32><<<nb, kThreads, 0, s>>>(a, n_muons);
    count_launches(1);
}
template void launch_em_muon_warp<float>(const MuonPassArgs<float>&, uint32_t, int, int, cudaStream_t);
template void launch_em_muon_warp<double>(const MuonPassArgs<double>&, uint32_t, int, int, cudaStream_t);

}  // namespace muto
