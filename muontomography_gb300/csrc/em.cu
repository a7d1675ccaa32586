// EM iteration kernels of the MLSD/MAP path.
//
//  k_em_tile    one pass over all kept muons (src/MutoMLSD.cpp:188-195):
//               covariance gather (getCovarianceMatrix, :442-449), the 2x2
//               inverse/determinant/cost (updateSValueMatrix, :451-469) and the
//               per-pair EM term s_ij (:471-488).
//  k_select     per-voxel median / percentile mean of s_ij (updateImageVoxel,
//               :493-517) by an exact radix selection.
//  k_voxel_mean per-voxel mean of s_ij (:498-499) from accumulated sums.
//  k_map_voxel  MAP surrogate step (src/MutoMAP.cpp:228-247 with :207-406).
//
// Work layout of k_em_tile.  Kept muons are cut into tiles of consecutive
// muons whose pairs fit in shared memory.  A CTA loops over tiles:
//   stage    one thread issues bulk asynchronous copies (cp.async.bulk, the
//            TMA engine) of the tile's contiguous per-pair arrays (voxel index,
//            L, T, slot) and per-muon arrays (offsets, S/D, pr^2) into shared
//            memory, completing on an mbarrier; every pair byte is read from
//            HBM exactly once per iteration.  Ranges are widened to 16-byte
//            boundaries (the arrays carry padding for that).
//   gather   every thread fetches lambda_j for 8 pairs at once (L2-resident).
//   sum      GROUP lanes per muon sum lambda_j * W_ij from shared memory.
//   2x2      one thread per muon: Sigma = pr^2 sum + E, determinant and
//            inverse in FP64, cost, and three coefficients k with
//              pr^2 (1/2 xyS_ij - tr(Sigma^-1 W_ij)) = k0 W00 + k1 W01 + k2 W11
//            (xyS = sum over the x and y planes of u^T W u, u = Sigma^-1 (S, D)).
//   scatter  one thread per pair: g_ij and s_ij = 2 l + g l^2 written to the
//            pair's voxel-major slot (median / percentile) or g_ij added to the
//            voxel's sum (mean / gradient).
// Several CTAs per SM overlap one CTA's copies with another's arithmetic.
#include "common.cuh"

namespace muto {
namespace {

constexpr int kTileThreads = 256;
constexpr int kGatherUnroll = 8;

// per-tile shared-memory layout; per-pair buffers hold TP + 8 entries (the
// tile's range widened to 16-byte boundaries at both ends)
template <typename Real>
struct TileLayout {
    size_t off, sd, pr2, idx, L, T, slot, lam, mu, sig, k, bar, total;
    __host__ __device__ TileLayout(int TP, int TM) {
        auto up = [](size_t x) { return (x + 15) & ~static_cast<size_t>(15); };
        size_t p = 0;
        off = p;  p = up(p + sizeof(uint64_t) * (TM + 4));
        sd = p;   p = up(p + sizeof(typename Vec4<Real>::type) * TM);
        pr2 = p;  p = up(p + sizeof(Real) * (TM + 8));
        idx = p;  p = up(p + sizeof(uint32_t) * (TP + 8));
        L = p;    p = up(p + sizeof(Real) * (TP + 8));
        T = p;    p = up(p + sizeof(Real) * (TP + 8));
        slot = p; p = up(p + sizeof(uint32_t) * (TP + 8));
        lam = p;  p = up(p + sizeof(Real) * TP);
        mu = p;   p = up(p + sizeof(uint16_t) * TP);
        sig = p;  p = up(p + sizeof(Real) * 3 * TM);
        k = p;    p = up(p + sizeof(Real) * 3 * TM);
        bar = p;  p = up(p + sizeof(uint64_t));
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

// The element range [b, e) of an array of `size`-byte elements widened to
// 16-byte boundaries: returns the first element and the byte count.
__device__ __forceinline__ void widen(uint64_t b, uint64_t e, uint32_t size, uint64_t* first, uint32_t* bytes) {
    const uint64_t per = 16 / size;
    const uint64_t f = b - b % per;
    const uint64_t l = ((e + per - 1) / per) * per;
    *first = f;
    *bytes = static_cast<uint32_t>((l - f) * size);
}

// Bounded wait on the tile barrier; false (and a recorded timeout) if the
// copies did not land within the limit.
__device__ __forceinline__ bool wait_tile(uint64_t* bar, uint32_t parity, Counters* ctr) {
    for (uint32_t spin = 0; spin < (1u << 22); ++spin)
        if (mbar_try_wait(bar, parity)) return true;
    if (threadIdx.x == 0) atomicAdd(&ctr->timeouts, 1ull);
    return false;
}

template <typename Real, int GROUP>
__global__ void __launch_bounds__(kTileThreads, 3) k_em_tile(EmArgs<Real> a, int TP, int TM) {
    using R4 = typename Vec4<Real>::type;
    extern __shared__ __align__(128) unsigned char smem[];
    const TileLayout<Real> lay(TP, TM);
    uint64_t* s_off = reinterpret_cast<uint64_t*>(smem + lay.off);
    R4* s_sd = reinterpret_cast<R4*>(smem + lay.sd);
    Real* s_pr2 = reinterpret_cast<Real*>(smem + lay.pr2);
    uint32_t* s_idx = reinterpret_cast<uint32_t*>(smem + lay.idx);
    Real* s_L = reinterpret_cast<Real*>(smem + lay.L);
    Real* s_T = reinterpret_cast<Real*>(smem + lay.T);
    uint32_t* s_slot = reinterpret_cast<uint32_t*>(smem + lay.slot);
    Real* s_lam = reinterpret_cast<Real*>(smem + lay.lam);
    uint16_t* s_mu = reinterpret_cast<uint16_t*>(smem + lay.mu);
    Real* s_sig = reinterpret_cast<Real*>(smem + lay.sig);
    Real* s_k = reinterpret_cast<Real*>(smem + lay.k);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + lay.bar);

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int group = tid / GROUP, glane = tid % GROUP;
    constexpr int kGroups = kTileThreads / GROUP;
    const unsigned gmask = GROUP == 32 ? kFull : (((1u << GROUP) - 1u) << (lane & ~(GROUP - 1)));
    const uint32_t V = a.V;
    const bool median = a.mode == kEmMedian;
    double cost_local = 0.0;
    unsigned long long singular_local = 0;

    if (tid == 0) mbar_init(bar, 1);
    __syncthreads();

    uint32_t parity = 0;
    for (uint32_t t = blockIdx.x; t < a.ntiles; t += gridDim.x, parity ^= 1u) {
        const uint32_t mb = a.tile_mb[t], me = a.tile_mb[t + 1];
        const int nm = static_cast<int>(me - mb);
        const uint64_t pb = a.off[mb], pe = a.off[me];
        const int np = static_cast<int>(pe - pb);
        uint64_t f_pair, f_off, f_pr2;
        uint32_t b_idx, b_real, b_off, b_pr2;
        widen(pb, pe, 4, &f_pair, &b_idx);
        {
            uint64_t fr;
            widen(pb, pe, sizeof(Real), &fr, &b_real);
            // 4-byte arrays start at f_pair; Real arrays at fr (== f_pair for float)
            if (tid == 0) {
                widen(mb, me + 1, 8, &f_off, &b_off);
                widen(mb, me, sizeof(Real), &f_pr2, &b_pr2);
                const uint32_t b_sd = static_cast<uint32_t>(nm * sizeof(R4));
                const uint32_t total = b_idx * (median ? 2u : 1u) + 2u * b_real + b_off + b_sd + b_pr2;
                fence_proxy_async();
                mbar_arrive_expect_tx(bar, total);
                if (b_idx) {  // a tile of muons with empty paths has no pair bytes
                    bulk_load(s_idx, a.vidx + f_pair, b_idx, bar);
                    if (median) bulk_load(s_slot, a.slot + f_pair, b_idx, bar);
                    bulk_load(s_L, a.L + fr, b_real, bar);
                    bulk_load(s_T, a.T + fr, b_real, bar);
                }
                bulk_load(s_off, a.off + f_off, b_off, bar);
                if (b_sd) bulk_load(s_sd, a.sd + mb, b_sd, bar);
                bulk_load(s_pr2, a.pr2 + f_pr2, b_pr2, bar);
            }
            // shifts from the widened range starts to the tile's first element
            const int sh_pair = static_cast<int>(pb - f_pair);
            const int sh_real = static_cast<int>(pb - fr);
            const int sh_off = static_cast<int>(mb - (mb - mb % 2));
            const int sh_pr2 = static_cast<int>(mb % (16 / sizeof(Real)));
            const bool landed = wait_tile(bar, parity, a.ctr);
            if (!__syncthreads_and(landed)) break;  // uniform: every thread leaves together

            // ---- gather lambda for every pair of the tile (loads in flight together)
            for (int k0 = tid; k0 < np; k0 += kGatherUnroll * kTileThreads) {
                Real lv[kGatherUnroll];
#pragma unroll
                for (int u = 0; u < kGatherUnroll; ++u) {
                    const int k = k0 + u * kTileThreads;
                    const uint32_t j = k < np ? s_idx[sh_pair + k] : 0xffffffffu;
                    lv[u] = j < V ? __ldg(a.lam + j) : Real(0);
                }
#pragma unroll
                for (int u = 0; u < kGatherUnroll; ++u) {
                    const int k = k0 + u * kTileThreads;
                    if (k < np) s_lam[k] = lv[u];
                }
            }
            __syncthreads();

            // ---- covariance sums, GROUP lanes per muon ------------------------
            for (int m = group; m < nm; m += kGroups) {
                const int b = static_cast<int>(s_off[sh_off + m] - pb), e = static_cast<int>(s_off[sh_off + m + 1] - pb);
                Real c0 = 0, c1 = 0, c2 = 0;
                for (int k = b + glane; k < e; k += GROUP) {
                    s_mu[k] = static_cast<uint16_t>(m);
                    const Real L = s_L[sh_real + k], T = s_T[sh_real + k], l = s_lam[k];
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

            // ---- per-muon 2x2 algebra, one thread per muon --------------------
            for (int m = tid; m < nm; m += kTileThreads) {
                const double p2 = static_cast<double>(s_pr2[sh_pr2 + m]);
                const double S00 = p2 * static_cast<double>(s_sig[3 * m + 0]) + a.E00;
                const double S01 = p2 * static_cast<double>(s_sig[3 * m + 1]) + a.E01;
                const double S11 = p2 * static_cast<double>(s_sig[3 * m + 2]) + a.E11;
                const double det = S00 * S11 - S01 * S01;
                Real k0 = 0, k1 = 0, k2 = 0;
                if (fabs(det) > 1e-12) {  // Eigen computeInverseAndDetWithCheck threshold
                    const double r = 1.0 / det;
                    const double i00 = S11 * r, i01 = -S01 * r, i11 = S00 * r;
                    const R4 v = s_sd[m];
                    // u = Sigma^-1 (S, D) per plane; in the storage precision
                    const Real f00 = static_cast<Real>(i00), f01 = static_cast<Real>(i01), f11 = static_cast<Real>(i11);
                    const Real ux0 = f00 * v.x + f01 * v.y, ux1 = f01 * v.x + f11 * v.y;
                    const Real uy0 = f00 * v.z + f01 * v.w, uy1 = f01 * v.z + f11 * v.w;
                    const Real pr2 = s_pr2[sh_pr2 + m];
                    k0 = pr2 * (Real(0.5) * (ux0 * ux0 + uy0 * uy0) - f00);
                    k1 = pr2 * ((ux0 * ux1 + uy0 * uy1) - Real(2) * f01);
                    k2 = pr2 * (Real(0.5) * (ux1 * ux1 + uy1 * uy1) - f11);
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
                s_k[3 * m + 0] = k0;
                s_k[3 * m + 1] = k1;
                s_k[3 * m + 2] = k2;
            }
            __syncthreads();

            // ---- per-pair EM term ---------------------------------------------
            if (a.mode != kEmCostOnly) {
                for (int k = tid; k < np; k += kTileThreads) {
                    const uint32_t j = s_idx[sh_pair + k];
                    if (j >= V) continue;
                    const int m = s_mu[k];
                    const Real L = s_L[sh_real + k], T = s_T[sh_real + k], l = s_lam[k];
                    const Real LT = L * T;
                    const Real w01 = LT + L * L * Real(0.5);
                    const Real w11 = L * L * L * Real(1.0 / 3.0) + (L + T) * LT;
                    const Real g = s_k[3 * m + 0] * L + s_k[3 * m + 1] * w01 + s_k[3 * m + 2] * w11;
                    if (median) a.S[s_slot[sh_pair + k]] = Real(2) * l + g * l * l;
                    else atomicAdd(a.G + j, g);
                }
            }
        }
        __syncthreads();  // the buffers are overwritten by the next tile's copies
    }

    // block reduction of the cost and singular counts
    __shared__ double red[kTileThreads / 32];
    __shared__ unsigned long long redn[kTileThreads / 32];
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
        for (int w = 0; w < kTileThreads / 32; ++w) {
            tc += red[w];
            tn += redn[w];
        }
        if (a.compute_cost && tc != 0.0) atomicAdd(&a.ctr->cost_sum, tc);
        if (tn) atomicAdd(&a.ctr->singular, tn);
    }
}

// ---------------------------------------------------------------------------
// Exact k-th smallest of a voxel's s_ij, one warp per voxel.
// ---------------------------------------------------------------------------
template <typename K>
__device__ __forceinline__ K warp_min_k(K v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const K t = __shfl_xor_sync(kFull, v, o);
        v = t < v ? t : v;
    }
    return v;
}
template <typename K>
__device__ __forceinline__ K warp_max_k(K v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const K t = __shfl_xor_sync(kFull, v, o);
        v = t > v ? t : v;
    }
    return v;
}
__device__ __forceinline__ int clz_k(uint32_t x) { return __clz(x); }
__device__ __forceinline__ int clz_k(unsigned long long x) { return __clzll(x); }

// Keys held in registers: element r*32+lane of the segment.
template <typename Real, int R>
struct RegKeys {
    using K = typename KeyOf<Real>::type;
    K key[R];
    uint32_t M;
    int lane;
    __device__ void load(const Real* seg, uint32_t m, int ln) {
        M = m;
        lane = ln;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t i = static_cast<uint32_t>(r * 32 + lane);
            key[r] = i < M ? to_key(seg[i]) : K(0);
        }
    }
    template <class F>
    __device__ __forceinline__ void each(F f) const {
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (static_cast<uint32_t>(r * 32 + lane) < M) f(key[r]);
    }
};

// Keys streamed from global memory (segments too long for registers).
template <typename Real>
struct MemKeys {
    using K = typename KeyOf<Real>::type;
    const Real* seg;
    uint32_t M;
    int lane;
    template <class F>
    __device__ __forceinline__ void each(F f) const {
        for (uint32_t i = lane; i < M; i += 32) f(to_key(seg[i]));
    }
};

template <typename K, class Src>
__device__ K kth_key(const Src& src, uint32_t k) {
    constexpr int B = sizeof(K) * 8;
    K mn = ~K(0), mx = K(0);
    src.each([&](K x) {
        mn = x < mn ? x : mn;
        mx = x > mx ? x : mx;
    });
    mn = warp_min_k(mn);
    mx = warp_max_k(mx);
    if (mn == mx) return mn;
    const int hb = B - 1 - clz_k(mn ^ mx);
    const K low = (hb + 1 >= B) ? ~K(0) : ((K(1) << (hb + 1)) - 1);
    K prefix = mn & ~low;
    K hmask = ~low;
    for (int b = hb; b >= 0; --b) {
        const K bit = K(1) << b;
        uint32_t cnt = 0;
        src.each([&](K x) { cnt += ((x & hmask) == prefix && !(x & bit)) ? 1u : 0u; });
        cnt = __reduce_add_sync(kFull, cnt);
        if (k >= cnt) {
            k -= cnt;
            prefix |= bit;
        }
        hmask |= bit;
    }
    return prefix;
}

// count and max of the keys strictly below v
template <typename K, class Src>
__device__ void below(const Src& src, K v, uint32_t* cnt, K* mxb) {
    uint32_t c = 0;
    K m = K(0);
    src.each([&](K x) {
        if (x < v) {
            ++c;
            m = x > m ? x : m;
        }
    });
    *cnt = __reduce_add_sync(kFull, c);
    *mxb = warp_max_k(m);
}

template <typename Real, typename K, class Src>
__device__ double voxel_value(const Src& src, uint32_t M, int use_mean, int pct) {
    if (!use_mean) {  // median, src/MutoMLSD.cpp:506-516
        const K k1 = kth_key<K>(src, M / 2);
        const double v1 = static_cast<double>(from_key(k1));
        if (M % 2 == 0) {
            uint32_t c;
            K mb;
            below<K>(src, k1, &c, &mb);
            const double v0 = c < M / 2 ? v1 : static_cast<double>(from_key(mb));
            return (v1 + v0) * 0.25;
        }
        return v1 * 0.5;
    }
    // mean of the lowest floor(pct/100*M) values (at least 1), :500-504
    uint32_t jm = u32_cast_x86(pct / 100.0 * M);
    if (jm < 1) jm = 1;
    if (jm > M) jm = M;
    const K kt = kth_key<K>(src, jm - 1);
    const double t = static_cast<double>(from_key(kt));
    double s = 0.0;
    uint32_t c = 0;
    src.each([&](K x) {
        if (x < kt) {
            s += static_cast<double>(from_key(x));
            ++c;
        }
    });
    s = warp_sum(s);
    c = __reduce_add_sync(kFull, c);
    s += static_cast<double>(jm - c) * t;
    return s / static_cast<double>(jm) * 0.5;
}

template <typename Real, int R>
__device__ __forceinline__ double select_regs(const Real* seg, uint32_t M, int lane, int use_mean, int pct) {
    using K = typename KeyOf<Real>::type;
    RegKeys<Real, R> src;
    src.load(seg, M, lane);
    return voxel_value<Real, K>(src, M, use_mean, pct);
}

template <typename Real, typename OutT>
__global__ void __launch_bounds__(256) k_select(const Real* __restrict__ S, const uint64_t* __restrict__ start,
                                                const uint32_t* __restrict__ mult, uint32_t V, int use_mean, int pct,
                                                OutT* __restrict__ out) {
    using K = typename KeyOf<Real>::type;
    const int lane = threadIdx.x & 31;
    const uint32_t w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t j = w0; j < V; j += nw) {
        const uint32_t M = mult[j];
        double v = 0.0;
        if (M > 0) {
            const Real* seg = S + start[j];
            // registers per lane sized to the segment (the passes touch only those)
            if (M <= 32u) v = select_regs<Real, 1>(seg, M, lane, use_mean, pct);
            else if (M <= 64u) v = select_regs<Real, 2>(seg, M, lane, use_mean, pct);
            else if (M <= 128u) v = select_regs<Real, 4>(seg, M, lane, use_mean, pct);
            else if (M <= 192u) v = select_regs<Real, 6>(seg, M, lane, use_mean, pct);
            else if (M <= 256u) v = select_regs<Real, 8>(seg, M, lane, use_mean, pct);
            else if (M <= 384u) v = select_regs<Real, 12>(seg, M, lane, use_mean, pct);
            else if (M <= 512u) v = select_regs<Real, 16>(seg, M, lane, use_mean, pct);
            else if (M <= 768u) v = select_regs<Real, 24>(seg, M, lane, use_mean, pct);
            else if (M <= 1024u) v = select_regs<Real, 32>(seg, M, lane, use_mean, pct);
            else {
                MemKeys<Real> src{seg, M, lane};
                v = voxel_value<Real, K>(src, M, use_mean, pct);
            }
        }
        if (lane == 0) out[j] = static_cast<OutT>(v);
    }
}

// mean update: (sum_i s_ij) / M / 2 = l + l^2 (sum_i pr^2 g_ij) / (2 M)
template <typename Real, typename OutT>
__global__ void k_voxel_mean(const Real* __restrict__ lam, Real* __restrict__ G, const uint32_t* __restrict__ mult,
                             uint32_t V, OutT* __restrict__ out) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= V) return;
    const uint32_t M = mult[j];
    const double l = static_cast<double>(lam[j]);
    const double g = static_cast<double>(G[j]);
    G[j] = Real(0);
    out[j] = static_cast<OutT>(M == 0 ? 0.0 : l + l * l * g / (2.0 * static_cast<double>(M)));
}

__global__ void k_finalize_cost(Counters* ctr, double n_muons, double* hist, uint32_t cap) {
    const double c = n_muons > 0 ? ctr->cost_sum / n_muons : 0.0;
    ctr->cost_prev = ctr->cost_last;
    ctr->cost_last = c;
    if (hist && ctr->iteration < cap) hist[ctr->iteration] = c;
    ctr->iteration += 1;
    ctr->cost_sum = 0.0;
}

// ---------------------------------------------------------------------------
// MAP step, one thread per voxel, FP64 (src/MutoMAP.cpp:228-247)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double pow_e(double x, double e) {
    if (e == 0.0) return 1.0;        // p = 2
    if (e == -0.5) return rsqrt(x);  // p = 1
    return pow(x, e);
}

template <typename LamT>
__global__ void k_map_voxel(const LamT* __restrict__ last, double* __restrict__ ml_inout,
                            const uint32_t* __restrict__ mult, DevGrid g, MapParams mp, Counters* ctr) {
    const uint32_t V = g.n[0] * g.n[1] * g.n[2];
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    bool nonconv = false;
    if (j < V) {
        const uint32_t Mj = mult[j];
        if (Mj == 0) {
            ml_inout[j] = 0.0;
        } else {
            const double unit = 1.0e7;
            const uint32_t nx = g.n[0], ny = g.n[1], nz = g.n[2], nxy = nx * ny;
            const uint32_t x = j % nxy % nx, y = j % nxy / nx, z = j / nxy;  // index2xyz, :283-290
            const uint32_t xp = x < nx - 1 ? x + 1 : nx - 1, yp = y < ny - 1 ? y + 1 : ny - 1,
                           zp = z < nz - 1 ? z + 1 : nz - 1;
            const uint32_t xm = 0 < x ? x - 1 : 0, ym = 0 < y ? y - 1 : 0, zm = 0 < z ? z - 1 : 0;
            auto at = [&](uint32_t a, uint32_t b, uint32_t c) {
                return static_cast<double>(last[a + b * nx + c * nxy]) * unit;
            };
            double lm[26];
            int nn = 0;
            lm[nn++] = at(xp, y, z); lm[nn++] = at(xm, y, z);
            lm[nn++] = at(x, yp, z); lm[nn++] = at(x, ym, z);
            lm[nn++] = at(x, y, zp); lm[nn++] = at(x, y, zm);
            if (mp.all_neighbours) {
                lm[nn++] = at(xp, yp, z); lm[nn++] = at(xm, yp, z); lm[nn++] = at(xp, ym, z); lm[nn++] = at(xm, ym, z);
                lm[nn++] = at(x, yp, zp); lm[nn++] = at(x, ym, zp); lm[nn++] = at(x, yp, zm); lm[nn++] = at(x, ym, zm);
                lm[nn++] = at(xp, y, zp); lm[nn++] = at(xm, y, zp); lm[nn++] = at(xp, y, zm); lm[nn++] = at(xm, y, zm);
                lm[nn++] = at(xp, yp, zp); lm[nn++] = at(xm, yp, zp); lm[nn++] = at(xp, ym, zp); lm[nn++] = at(xm, ym, zp);
                lm[nn++] = at(xp, yp, zm); lm[nn++] = at(xm, yp, zm); lm[nn++] = at(xp, ym, zm); lm[nn++] = at(xm, ym, zm);
            }
            const double w2 = 1.0 / sqrt(2.0), w3 = 1.0 / sqrt(3.0);
            const double e = (mp.p - 2.0) / 2.0;
            const double dd2 = mp.delta * mp.delta;
            const double lj = static_cast<double>(last[j]) * unit;
            double q[26];  // ((l_j - l_m)^2 + delta^2)^((p-2)/2), shared by p2/p3 and the surrogate
            double p2 = 0.0, p3 = 0.0;
            for (int k = 0; k < nn; ++k) {
                const double wk = k < 6 ? 1.0 : (k < 18 ? w2 : w3);
                const double d = lj - lm[k];
                q[k] = pow_e(d * d + dd2, e);
                const double t1 = wk * mp.p * q[k];
                p2 += t1 * 2.0 * (lj + lm[k]);
                p3 += t1 * 4.0;
            }
            const double qobj = mp.add_object_prior ? pow_e(lj * lj + dd2, e) : 0.0;
            if (mp.add_object_prior) p3 += mp.p * qobj;
            p2 *= -mp.beta / static_cast<double>(Mj);
            p3 *= mp.beta / static_cast<double>(Mj);
            const double ljml = ml_inout[j] * unit;
            const double p0 = -ljml, p1 = 1.0;
            // cubicEqnSolver, :353-406, Newton capped at newton_max_iter
            double roots[3];
            int nr;
            {
                const double ca = p2 / p3, cb = p1 / p3, cc = p0 / p3;
                const double r = 1 + smax(smax(fabs(ca), fabs(cb)), fabs(cc));
                const double xi = -ca / 3;
                const double gxi = xi * xi * xi + ca * xi * xi + cb * xi + cc;
                double xk = 0 < gxi ? -r : r;
                double rel = mp.eps * 2;
                int it = 0;
                while (rel > mp.eps) {
                    if (++it > mp.newton_max_iter) {
                        nonconv = true;
                        break;
                    }
                    const double xk2 = xk * xk;
                    const double gx = xk2 * xk + ca * xk2 + cb * xk + cc;
                    const double gp = 3 * xk2 + 2 * ca * xk + cb;
                    const double xn = xk - gx / gp;
                    rel = fabs((xn - xk) / xk);
                    xk = xn;
                }
                const double D = xk + ca;
                const double Ec = D * xk + cb;
                const double sgn = 0 <= D ? 1.0 : -1.0;
                const double disc = D * D - 4 * Ec;
                roots[0] = xk;
                if (disc < 0) {
                    nr = 1;
                } else {
                    const double qq = -0.5 * (D + sgn * sqrt(disc));
                    roots[1] = qq;
                    roots[2] = mp.eps < fabs(qq) ? Ec / qq : qq;
                    nr = 3;
                }
            }
            // chooseBestEstimation / surrogateFunctionValue, :239-281
            double best = 0.0;
            int bi = 0;
            for (int c = 0; c <= nr; ++c) {
                const double xv = c < nr ? roots[c] : ljml;
                double v;
                if (xv < 0) {
                    v = 1.7976931348623157e308;
                } else {
                    v = 0 < xv ? static_cast<double>(Mj) * (log(xv) + ljml / xv) : 0.0;
                    for (int k = 0; k < nn; ++k) {
                        const double wk = k < 6 ? 1.0 : (k < 18 ? w2 : w3);
                        const double tt = 2.0 * xv - lj - lm[k];
                        v += 0.5 * mp.beta * mp.p * wk * q[k] * (tt * tt);
                    }
                    if (mp.add_object_prior) v += 0.5 * mp.beta * mp.p * xv * xv * qobj;
                }
                if (c == 0 || v < best) {
                    best = v;
                    bi = c;
                }
            }
            ml_inout[j] = bi < nr ? roots[bi] / unit : ml_inout[j];
        }
    }
    warp_count(&ctr->nonconverged, nonconv);
}

template <typename LamT>
__global__ void k_copy_to(const double* __restrict__ in, LamT* __restrict__ out, uint64_t n) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = static_cast<LamT>(in[i]);
}

inline unsigned blocks_for(uint64_t n, int threads) {
    const uint64_t b = (n + threads - 1) / threads;
    return static_cast<unsigned>(b > 0 ? b : 1);
}

}  // namespace

template <typename Real>
size_t em_tile_smem_bytes(int tile_pairs, int tile_muons) {
    return TileLayout<Real>(tile_pairs, tile_muons).total;
}
template size_t em_tile_smem_bytes<float>(int, int);
template size_t em_tile_smem_bytes<double>(int, int);

template <typename Real>
cudaError_t em_tile_configure(int tile_pairs, int tile_muons) {
    const int smem = static_cast<int>(em_tile_smem_bytes<Real>(tile_pairs, tile_muons));
    cudaError_t e = cudaFuncSetAttribute(k_em_tile<Real, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_em_tile<Real, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_em_tile<Real, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    return e;
}
template cudaError_t em_tile_configure<float>(int, int);

// resident CTAs per SM of the k_em_tile variant used for a gather group width
template <typename Real>
int em_tile_blocks(int tile_pairs, int tile_muons, int group) {
    const size_t smem = em_tile_smem_bytes<Real>(tile_pairs, tile_muons);
    int n = 0;
    cudaError_t e;
    if (group <= 8) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_em_tile<Real, 8>, kTileThreads, smem);
    else if (group <= 16) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_em_tile<Real, 16>, kTileThreads, smem);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_em_tile<Real, 32>, kTileThreads, smem);
    return (e == cudaSuccess && n > 0) ? n : 1;
}
template int em_tile_blocks<float>(int, int, int);
template int em_tile_blocks<double>(int, int, int);
template cudaError_t em_tile_configure<double>(int, int);

template <typename Real>
void launch_em_tile(const EmArgs<Real>& a, int tile_pairs, int tile_muons, int blocks, int group, cudaStream_t s) {
    if (a.ntiles == 0) return;
    const size_t smem = em_tile_smem_bytes<Real>(tile_pairs, tile_muons);
    const unsigned nb = static_cast<unsigned>(blocks < static_cast<int>(a.ntiles) ? blocks : a.ntiles);
    // lanes sharing one muon in the gather phase (chosen from the mean path length)
    if (group <= 8) {
        k_em_tile<Real, 8><<<nb, kTileThreads, smem, s>>>(a, tile_pairs, tile_muons); count_launches(1);
    } else if (group <= 16) {
        k_em_tile<Real, 16><<<nb, kTileThreads, smem, s>>>(a, tile_pairs, tile_muons); count_launches(1);
    } else {
        k_em_tile<Real, 32><<<nb, kTileThreads, smem, s>>>(a, tile_pairs, tile_muons); count_launches(1);
    }
}
template void launch_em_tile<float>(const EmArgs<float>&, int, int, int, int, cudaStream_t);
template void launch_em_tile<double>(const EmArgs<double>&, int, int, int, int, cudaStream_t);

template <typename Real, typename OutT>
void launch_select(const Real* S, const uint64_t* start, const uint32_t* mult, uint32_t V, int use_mean, int pct,
                   OutT* out, cudaStream_t s) {
    if (V == 0) return;
    const uint64_t warps = V;
    const unsigned nb = blocks_for(warps * 32, 256);
    k_select<Real, OutT><<<nb, 256, 0, s>>>(S, start, mult, V, use_mean, pct, out); count_launches(1);
}
template void launch_select<float, float>(const float*, const uint64_t*, const uint32_t*, uint32_t, int, int, float*,
                                          cudaStream_t);
template void launch_select<float, double>(const float*, const uint64_t*, const uint32_t*, uint32_t, int, int,
                                           double*, cudaStream_t);
template void launch_select<double, double>(const double*, const uint64_t*, const uint32_t*, uint32_t, int, int,
                                            double*, cudaStream_t);

template <typename Real, typename OutT>
void launch_voxel_mean(const Real* lam, Real* G, const uint32_t* mult, uint32_t V, OutT* out, cudaStream_t s) {
    if (V == 0) return;
    k_voxel_mean<Real, OutT><<<blocks_for(V, 256), 256, 0, s>>>(lam, G, mult, V, out); count_launches(1);
}
template void launch_voxel_mean<float, float>(const float*, float*, const uint32_t*, uint32_t, float*, cudaStream_t);
template void launch_voxel_mean<float, double>(const float*, float*, const uint32_t*, uint32_t, double*,
                                               cudaStream_t);
template void launch_voxel_mean<double, double>(const double*, double*, const uint32_t*, uint32_t, double*,
                                                cudaStream_t);

void launch_finalize_cost(Counters* ctr, double n_muons, double* hist, uint32_t cap, cudaStream_t s) {
    k_finalize_cost<<<1, 1, 0, s>>>(ctr, n_muons, hist, cap); count_launches(1);
}

template <typename LamT>
void launch_map_voxel(const LamT* last, double* ml_inout, const uint32_t* mult, DevGrid g, MapParams mp,
                      Counters* ctr, cudaStream_t s) {
    const uint64_t V = static_cast<uint64_t>(g.n[0]) * g.n[1] * g.n[2];
    if (V == 0) return;
    k_map_voxel<LamT><<<blocks_for(V, 128), 128, 0, s>>>(last, ml_inout, mult, g, mp, ctr); count_launches(1);
}
template void launch_map_voxel<float>(const float*, double*, const uint32_t*, DevGrid, MapParams, Counters*,
                                      cudaStream_t);
template void launch_map_voxel<double>(const double*, double*, const uint32_t*, DevGrid, MapParams, Counters*,
                                       cudaStream_t);

template <typename LamT>
void launch_copy_to(const double* in, LamT* out, uint64_t n, cudaStream_t s) {
    if (n == 0) return;
    k_copy_to<LamT><<<blocks_for(n, 256), 256, 0, s>>>(in, out, n); count_launches(1);
}
template void launch_copy_to<float>(const double*, float*, uint64_t, cudaStream_t);
template void launch_copy_to<double>(const double*, double*, uint64_t, cudaStream_t);

}  // namespace muto
