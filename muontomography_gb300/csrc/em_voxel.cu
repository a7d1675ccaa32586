// Voxel pass of an EM iteration: the per-voxel update of src/MutoMLSD.cpp:493-517
// (updateImageVoxel, run for every voxel at :197-200), and the MAP step of
// src/MutoMAP.cpp:228-247.
//
// The pairs are also stored voxel-major (muon, L, T), built once at setup, so
// one warp per voxel reads its M_j pairs with coalesced streaming loads,
// gathers each muon's coefficients k_i (written by the muon pass, small enough
// to stay in L2) and forms in registers
//     s_ij = 2 l_j + (k0 W00 + k1 W01 + k2 W11) l_j^2,
// the reference's 2 l + (1/2 xyS - tr(Sigma^-1 W)) pr^2 l^2.  No s_ij array is
// written; nothing is accumulated with atomics.
//   median       exact order statistics of the s_ij (nth_element semantics):
//                a 32-element sample of the segment is sorted in the warp, the
//                window around the target rank is counted and its members
//                compacted in shared memory, and the k-th key is found there by
//                a bitwise radix search; a window that misses falls back to
//                the radix search over all keys.
//   percentile   mean of the lowest floor(pct/100 M) values: the order
//                statistic t plus the sum of the values below it.
//   mean         l + l^2 (sum_i g_ij) / (2 M)  ==  (sum_i s_ij) / M / 2.
//   gradient     d NLL / d log l_j = -l_j sum_i g_ij (the adjoint).
#include "common.cuh"

namespace muto {
namespace {

constexpr int kVoxThreads = 256;
constexpr int kWarps = kVoxThreads / 32;
constexpr int kCap = 640;  // window candidates kept per warp

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }
__device__ __forceinline__ double4 ldg4(const double4* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
    const double2 a = __ldg(q), b = __ldg(q + 1);
    double4 r;
    r.x = a.x;
    r.y = a.y;
    r.z = b.x;
    r.w = b.y;
    return r;
}

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

// k-th smallest key (0-based) of a key source, by bitwise radix search over
// the bits below the common prefix of the minimum and maximum.
template <typename K, class Src>
__device__ K kth_radix(const Src& src, uint32_t k) {
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

// keys in memory (the window candidates in shared memory, or a long
// segment's keys in the global scratch array)
template <typename K>
struct PtrKeys {
    const K* p;
    uint32_t n;
    int lane;
    template <class F>
    __device__ __forceinline__ void each(F f) const {
        for (uint32_t i = lane; i < n; i += 32) f(p[i]);
    }
    template <class F>
    __device__ __forceinline__ void each_all(F f) const {
        for (uint32_t i0 = 0; i0 < n; i0 += 32) {
            const uint32_t i = i0 + lane;
            f(i < n ? p[i] : K(0), i < n);
        }
    }
    __device__ __forceinline__ K sample() const { return p[(static_cast<uint64_t>(lane) * n) / 32u]; }
    __device__ __forceinline__ uint32_t size() const { return n; }
};

// The voxel's s_ij as order-preserving keys, element r*32+lane in key[r].
template <typename Real, int R>
struct VoxKeys {
    using K = typename KeyOf<Real>::type;
    K key[R];
    uint32_t M;
    int lane;
    template <class F>
    __device__ __forceinline__ void each(F f) const {
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (static_cast<uint32_t>(r * 32 + lane) < M) f(key[r]);
    }
    template <class F>
    __device__ __forceinline__ void each_all(F f) const {
#pragma unroll
        for (int r = 0; r < R; ++r) f(key[r], static_cast<uint32_t>(r * 32 + lane) < M);
    }
    __device__ __forceinline__ K sample() const { return key[0]; }  // element `lane`: positions follow slot order
    __device__ __forceinline__ uint32_t size() const { return M; }
};

// k-th smallest with a sampled window, exact: sort 32 samples, take the
// samples 6 ranks either side of the target as the window, count the keys
// below it and compact the keys inside it into shared memory, then search the
// window; a window that misses the target falls back to the full search.
template <typename K, class Src>
__device__ K kth_window(const Src& v, uint32_t k, K* cand, int lane) {
    const uint32_t M = v.size();
    K s = v.sample();
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const K o = __shfl_xor_sync(kFull, s, stride);
            const bool up = (lane & size) == 0 || size == 32;
            const bool lower = (lane & stride) == 0;
            s = (lower == up) ? (o < s ? o : s) : (o > s ? o : s);
        }
    }
    const int pos = static_cast<int>((static_cast<uint64_t>(k) * 32u) / M);
    const int ql = pos - 6, qh = pos + 6;
    const K slo = __shfl_sync(kFull, s, ql < 0 ? 0 : ql);
    const K shi = __shfl_sync(kFull, s, qh > 31 ? 31 : qh);
    const K lo = ql < 0 ? K(0) : slo;
    const K hi = qh > 31 ? ~K(0) : shi;
    uint32_t c_lo = 0, c_in = 0;
    const unsigned below_me = (1u << lane) - 1u;
    // lanes walk the keys in lock step (each() visits r*32+lane / i = lane + 32 t)
    auto visit = [&](K x, bool valid) {
        const bool lt = valid && x < lo;
        const bool in = valid && !lt && x <= hi;
        c_lo += __popc(__ballot_sync(kFull, lt));
        const unsigned m = __ballot_sync(kFull, in);
        if (in) {
            const uint32_t at = c_in + __popc(m & below_me);
            if (at < kCap) cand[at] = x;
        }
        c_in += __popc(m);
    };
    v.each_all(visit);
    __syncwarp();
    K res;
    if (c_lo <= k && k < c_lo + c_in && c_in <= kCap) {
        PtrKeys<K> src{cand, c_in, lane};
        res = kth_radix<K>(src, k - c_lo);
    } else {
        res = kth_radix<K>(v, k);
    }
    __syncwarp();  // cand is reused by the next selection
    return res;
}

template <typename Real, int R>
__device__ __forceinline__ typename KeyOf<Real>::type kth_any(const VoxKeys<Real, R>& v, uint32_t k,
                                                              typename KeyOf<Real>::type* cand) {
    using K = typename KeyOf<Real>::type;
    if (R >= 4) return kth_window<K>(v, k, cand, v.lane);
    return kth_radix<K>(v, k);
}
template <typename K>
__device__ __forceinline__ K kth_any(const PtrKeys<K>& v, uint32_t k, K* cand) {
    return kth_window<K>(v, k, cand, v.lane);
}

// the voxel's new value from its keys (median or percentile mean)
template <typename Real, class Src>
__device__ double order_update(const Src& src, uint32_t M, int mode, int pct, typename KeyOf<Real>::type* cand) {
    using K = typename KeyOf<Real>::type;
    if (mode == kVoxMedian) {  // src/MutoMLSD.cpp:506-516
        const K k1 = kth_any(src, M / 2, cand);
        const double v1 = static_cast<double>(from_key(k1));
        if (M % 2 == 0) {  // s_(M/2-1) is v1 itself or the largest key below it
            uint32_t c = 0;
            K mb = K(0);
            src.each([&](K x) {
                if (x < k1) {
                    ++c;
                    mb = x > mb ? x : mb;
                }
            });
            c = __reduce_add_sync(kFull, c);
            mb = warp_max_k(mb);
            const double v0 = c < M / 2 ? v1 : static_cast<double>(from_key(mb));
            return (v1 + v0) * 0.25;
        }
        return v1 * 0.5;
    }
    // mean of the lowest floor(pct/100 M) values, at least 1 (src/MutoMLSD.cpp:500-504)
    uint32_t jm = u32_cast_x86(pct / 100.0 * M);
    if (jm < 1) jm = 1;
    if (jm > M) jm = M;
    const K kt = kth_any(src, jm - 1, cand);
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

template <typename Real, int R, typename OutT>
__device__ __forceinline__ void voxel_regs(const VoxelPassArgs<Real, OutT>& a, uint32_t j, uint64_t base, uint32_t M,
                                           int lane, typename KeyOf<Real>::type* cand) {
    using R4 = typename Vec4<Real>::type;
    const Real lam = a.lam[j];
    const bool keys = a.mode == kVoxMedian || a.mode == kVoxPercentile;
    VoxKeys<Real, R> v;
    v.M = M;
    v.lane = lane;
    double gs = 0.0;
    constexpr int C = R < 8 ? R : 8;  // loads in flight per lane per chunk
#pragma unroll
    for (int r0 = 0; r0 < R; r0 += C) {
        uint32_t mu[C];
        Real L[C], T[C];
#pragma unroll
        for (int u = 0; u < C; ++u) {
            const uint32_t e = static_cast<uint32_t>((r0 + u) * 32 + lane);
            if (r0 + u < R && e < M) {
                mu[u] = __ldcs(a.vm_mu + base + e);
                L[u] = __ldcs(a.vm_L + base + e);
                T[u] = __ldcs(a.vm_T + base + e);
            }
        }
#pragma unroll
        for (int u = 0; u < C; ++u) {
            if (r0 + u >= R) break;
            const uint32_t e = static_cast<uint32_t>((r0 + u) * 32 + lane);
            v.key[r0 + u] = 0;
            if (e < M) {
                const R4 k = ldg4(a.kvec + mu[u]);
                const Real l = L[u], t = T[u];
                const Real lt = l * t;
                const Real g =
                    k.x * l + k.y * (lt + l * l * Real(0.5)) + k.z * (l * l * l * Real(1.0 / 3.0) + (l + t) * lt);
                if (keys) v.key[r0 + u] = to_key(Real(2) * lam + g * lam * lam);
                else gs += static_cast<double>(g);
            }
        }
    }
    double out;
    if (keys) {
        out = order_update<Real>(v, M, a.mode, a.pct, cand);
    } else {
        gs = warp_sum(gs);
        if (a.mode == kVoxGradient) {
            if (lane == 0) a.grad[j] = -a.lam64[j] * gs;
            return;
        }
        const double l = static_cast<double>(lam);
        out = l + l * l * gs / (2.0 * static_cast<double>(M));
    }
    if (lane == 0) a.out[j] = static_cast<OutT>(out);
}

// segments longer than the register budget: the keys go once to the scratch
// array (same offsets as the voxel-major lists) and the selection reads them there
template <typename Real, typename OutT>
__device__ void voxel_stream(const VoxelPassArgs<Real, OutT>& a, uint32_t j, uint64_t base, uint32_t M, int lane,
                             typename KeyOf<Real>::type* cand) {
    using K = typename KeyOf<Real>::type;
    const Real lam = a.lam[j];
    const bool keys = a.mode == kVoxMedian || a.mode == kVoxPercentile;
    K* kp = a.scratch + base;
    double gs = 0.0;
    for (uint32_t i = lane; i < M; i += 32) {
        const auto k = ldg4(a.kvec + __ldcs(a.vm_mu + base + i));
        const Real l = __ldcs(a.vm_L + base + i), t = __ldcs(a.vm_T + base + i);
        const Real lt = l * t;
        const Real g = k.x * l + k.y * (lt + l * l * Real(0.5)) + k.z * (l * l * l * Real(1.0 / 3.0) + (l + t) * lt);
        if (keys) kp[i] = to_key(Real(2) * lam + g * lam * lam);
        else gs += static_cast<double>(g);
    }
    double out;
    if (keys) {
        __syncwarp();  // the lanes' key stores are visible to the whole warp
        PtrKeys<K> src{kp, M, lane};
        out = order_update<Real>(src, M, a.mode, a.pct, cand);
    } else {
        gs = warp_sum(gs);
        if (a.mode == kVoxGradient) {
            if (lane == 0) a.grad[j] = -a.lam64[j] * gs;
            return;
        }
        const double l = static_cast<double>(lam);
        out = l + l * l * gs / (2.0 * static_cast<double>(M));
    }
    if (lane == 0) a.out[j] = static_cast<OutT>(out);
}

template <typename Real, typename OutT>
__global__ void __launch_bounds__(kVoxThreads) k_em_voxel(VoxelPassArgs<Real, OutT> a) {
    using K = typename KeyOf<Real>::type;
    __shared__ K cand_all[kWarps][kCap];
    const int lane = threadIdx.x & 31;
    K* cand = cand_all[threadIdx.x >> 5];
    const uint64_t j64 = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (j64 >= a.V) return;  // whole warps leave together
    const uint32_t j = static_cast<uint32_t>(j64);
    const uint32_t M = a.mult[j];
    if (M == 0) {  // no muon crossed the voxel, src/MutoMLSD.cpp:494-496
        if (lane == 0) {
            if (a.mode == kVoxGradient) a.grad[j] = 0.0;
            else a.out[j] = OutT(0);
        }
        return;
    }
    const uint64_t base = a.start[j];
    // registers per lane sized to the segment; the loops touch only those
    if (M <= 32u) voxel_regs<Real, 1>(a, j, base, M, lane, cand);
    else if (M <= 64u) voxel_regs<Real, 2>(a, j, base, M, lane, cand);
    else if (M <= 128u) voxel_regs<Real, 4>(a, j, base, M, lane, cand);
    else if (M <= 192u) voxel_regs<Real, 6>(a, j, base, M, lane, cand);
    else if (M <= 256u) voxel_regs<Real, 8>(a, j, base, M, lane, cand);
    else if (M <= 384u) voxel_regs<Real, 12>(a, j, base, M, lane, cand);
    else if (M <= 512u) voxel_regs<Real, 16>(a, j, base, M, lane, cand);
    else if (M <= 768u) voxel_regs<Real, 24>(a, j, base, M, lane, cand);
    else {
        if constexpr (voxel_register_cap<Real>() > 768u) {  // 64-bit keys stay at 24 registers per lane
            if (M <= 1024u) {
                voxel_regs<Real, 32>(a, j, base, M, lane, cand);
                return;
            }
            if (M <= 1536u) {
                voxel_regs<Real, 48>(a, j, base, M, lane, cand);
                return;
            }
        }
        voxel_stream<Real, OutT>(a, j, base, M, lane, cand);
    }
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

template <typename Real, typename OutT>
void launch_em_voxel(const VoxelPassArgs<Real, OutT>& a, cudaStream_t s) {
    if (a.V == 0) return;
    const uint64_t threads = static_cast<uint64_t>(a.V) * 32u;
    k_em_voxel<Real, OutT><<<blocks_for(threads, kVoxThreads), kVoxThreads, 0, s>>>(a);
    count_launches(1);
}
template void launch_em_voxel<float, float>(const VoxelPassArgs<float, float>&, cudaStream_t);
template void launch_em_voxel<float, double>(const VoxelPassArgs<float, double>&, cudaStream_t);
template void launch_em_voxel<double, double>(const VoxelPassArgs<double, double>&, cudaStream_t);

void launch_finalize_cost(Counters* ctr, double n_muons, double* hist, uint32_t cap, cudaStream_t s) {
    k_finalize_cost<<<1, 1, 0, s>>>(ctr, n_muons, hist, cap);
    count_launches(1);
}

template <typename LamT>
void launch_map_voxel(const LamT* last, double* ml_inout, const uint32_t* mult, DevGrid g, MapParams mp,
                      Counters* ctr, cudaStream_t s) {
    const uint64_t V = static_cast<uint64_t>(g.n[0]) * g.n[1] * g.n[2];
    if (V == 0) return;
    k_map_voxel<LamT><<<blocks_for(V, 128), 128, 0, s>>>(last, ml_inout, mult, g, mp, ctr);
    count_launches(1);
}
template void launch_map_voxel<float>(const float*, double*, const uint32_t*, DevGrid, MapParams, Counters*,
                                      cudaStream_t);
template void launch_map_voxel<double>(const double*, double*, const uint32_t*, DevGrid, MapParams, Counters*,
                                       cudaStream_t);

template <typename LamT>
void launch_copy_to(const double* in, LamT* out, uint64_t n, cudaStream_t s) {
    if (n == 0) return;
    k_copy_to<LamT><<<blocks_for(n, 256), 256, 0, s>>>(in, out, n);
    count_launches(1);
}
template void launch_copy_to<float>(const double*, float*, uint64_t, cudaStream_t);
template void launch_copy_to<double>(const double*, double*, uint64_t, cudaStream_t);

}  // namespace muto
