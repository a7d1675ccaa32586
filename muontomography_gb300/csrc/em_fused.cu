// Mean-update EM iteration over the muon-major lists (update_with_mean with
// mean_percentile 100, src/MutoMLSD.cpp:497-499).
//
// The mean of s_ij = 2 l_j + g_ij l_j^2 over the M_j pairs of voxel j is
//     mean_j / 2 = l_j + l_j^2 G_j / (2 M_j),      G_j = sum_i g_ij,
// so the voxel side of a mean-update iteration is a per-voxel sum of the
// per-pair terms g_ij = k0 W00 + k1 W01 + k2 W11, where (k0, k1, k2) are the
// per-muon coefficients of the covariance Sigma_i (getCovarianceMatrix and
// updateSValueMatrix, :442-491) and W_ij the weight matrix of the pair
// (generateWeightMatrix, :417-430).  No voxel-major copy of the lists is
// needed: every muon adds its g_ij to G_j with a reduction to global memory
// (G is L2-resident), and a small voxel kernel finishes the update.
//
// Stored-list pass (k_em_fused_lists).  A CTA takes 32 consecutive muons at a
// time, GROUP lanes per muon.  Each lane loads its share of the muon's pairs
// (voxel index, L, T) once, keeps the first RC of them in registers, and
// gathers lambda_j; the GROUP lanes sum Sigma's three entries; one warp then
// runs the FP64 2x2 determinant, inverse and cost for all 32 muons of the
// batch, a muon per lane (the FP64 pipe of this part issues one warp
// instruction per 32 muons); finally every lane forms g_ij for the pairs it
// holds and adds them to G_j.  Pairs beyond the RC held per lane are read a
// second time, from L1 or L2: RC is kept small so that several CTAs (several
// batches) are resident on an SM and the batches' latencies overlap.  The
// staged variant (k_em_staged, run when asked for) copies a batch's whole
// pair range into shared memory instead.
//
// Split form (launch_em_scatter).  The muon pass of the median path
// (em_muon.cu: warp-batched, no block barriers, its FP64 2x2 algebra a muon
// per lane) writes every muon's coefficients; a second pass streams the lists
// again and only adds g_ij to G_j, 4 or 8 pairs in flight per lane.  Twice
// the list traffic from HBM, but neither pass waits at a block barrier; the
// autotuner times it beside the one-pass variants, and on the largest scans
// it is the one picked.
//
// Recompute pass (k_em_fused_walk).  The same sums without stored lists: a
// thread per muon (one muon each, so that a warp's lanes walk in step; the
// muons in order of decreasing path bound) walks its merged path in FP64 (the
// bit-exact Siddon walk of the set-up) once to sum Sigma, does the 2x2
// algebra (a muon per lane), and walks it again to add g_ij to G_j.  T_ij
// comes from the muon's total in-grid length (kept per muon at set-up) minus
// the running length.
#include "common.cuh"

namespace muto {
namespace {

constexpr int kBatch = 32;  // muons per CTA batch: one per lane of the 2x2 warp

// W_ij entries from (L, T) (src/MutoMLSD.cpp:417-430) folded into the three
// per-muon sums and the per-pair term g_ij
template <typename Real>
__device__ __forceinline__ void add_sigma(Real l, Real L, Real T, Real& c0, Real& c1, Real& c2) {
    const Real LT = L * T;
    c0 += l * L;
    c1 += l * (LT + L * L * Real(0.5));
    c2 += l * (L * L * L * Real(1.0 / 3.0) + (L + T) * LT);
}
template <typename Real>
__device__ __forceinline__ Real g_term(Real k0, Real k1, Real k2, Real L, Real T) {
    const Real LT = L * T;
    return k0 * L + k1 * (LT + L * L * Real(0.5)) + k2 * (L * L * L * Real(1.0 / 3.0) + (L + T) * LT);
}

// FP64 2x2 algebra of one muon: Sigma = pr^2 c + E, its determinant and
// inverse (Eigen's computeInverseAndDetWithCheck threshold 1e-12,
// src/MutoMLSD.cpp:460), the cost (:465-468) and k such that
// g_ij = k0 W00 + k1 W01 + k2 W11 = pr^2 (1/2 xyS_ij - tr(Sigma^-1 W_ij)).
template <typename Real>
__device__ __forceinline__ void muon_coefficients(Real c0, Real c1, Real c2, Real pr2,
                                                  const typename Vec4<Real>::type& v, double E00, double E01,
                                                  double E11, bool want_cost, Real& k0, Real& k1, Real& k2,
                                                  double& cost, unsigned long long& singular) {
    const double p2 = static_cast<double>(pr2);
    const double S00 = p2 * static_cast<double>(c0) + E00;
    const double S01 = p2 * static_cast<double>(c1) + E01;
    const double S11 = p2 * static_cast<double>(c2) + E11;
    const double det = S00 * S11 - S01 * S01;
    k0 = k1 = k2 = Real(0);
    if (fabs(det) > 1e-12) {
        const double r = 1.0 / det;
        const double i00 = S11 * r, i01 = -S01 * r, i11 = S00 * r;
        const Real f00 = static_cast<Real>(i00), f01 = static_cast<Real>(i01), f11 = static_cast<Real>(i11);
        const Real ux0 = f00 * v.x + f01 * v.y, ux1 = f01 * v.x + f11 * v.y;
        const Real uy0 = f00 * v.z + f01 * v.w, uy1 = f01 * v.z + f11 * v.w;
        k0 = pr2 * (Real(0.5) * (ux0 * ux0 + uy0 * uy0) - f00);
        k1 = pr2 * ((ux0 * ux1 + uy0 * uy1) - Real(2) * f01);
        k2 = pr2 * (Real(0.5) * (ux1 * ux1 + uy1 * uy1) - f11);
        if (det <= 0) {
            ++singular;  // inverse used, cost 0 (:461-464)
        } else if (want_cost) {
            const double sx = v.x, dx = v.y, sy = v.z, dy = v.w;
            cost += log(det) + ((sx * sx + sy * sy) * i00 + (dx * dx + dy * dy) * i11 + (sx * dx + sy * dy) * 2.0 * i01) * 0.5;
        }
    } else {
        ++singular;  // inverse left at zero: s_ij = 2 l_j
    }
}

// asynchronous global -> shared copies (cp.async), completed by the issuing thread's wait
__device__ __forceinline__ void cp_async_4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// a muon's (Sx, Dx, Sy, Dy) and pr^2 into shared memory
__device__ __forceinline__ void stage_muon(float4* sd_s, float* pr2_s, const float4* sd, const float* pr2) {
    cp_async_16(sd_s, sd);
    cp_async_4(pr2_s, pr2);
}
__device__ __forceinline__ void stage_muon(double4* sd_s, double* pr2_s, const double4* sd, const double* pr2) {
    cp_async_16(sd_s, sd);
    cp_async_16(reinterpret_cast<char*>(sd_s) + 16, reinterpret_cast<const char*>(sd) + 16);
    cp_async_8(pr2_s, pr2);
}

// L2 residency of lambda and G.  Every pass streams the pair lists (far more
// than L2) once; lambda and the per-voxel sums G (4 bytes per voxel each) are
// touched by every pair.  Their gathers and reductions carry an L2
// evict_last policy so that the streamed lists do not push them out.
__device__ __forceinline__ uint64_t l2_keep_policy() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ float ld_keep(const float* p, uint64_t pol) {
    float v;
    asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ double ld_keep(const double* p, uint64_t pol) {
    double v;
    asm volatile("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
    return v;
}
// reduction to global memory (red: no value returned), relaxed, GPU scope
__device__ __forceinline__ void red_add(float* p, float v, uint64_t pol) {
    asm volatile("red.global.add.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void red_add(double* p, double v, uint64_t pol) {
    asm volatile("red.global.add.L2::cache_hint.f64 [%0], %1, %2;" ::"l"(p), "d"(v), "l"(pol) : "memory");
}

// block-wide sum of the cost and singular counts into the counters
template <int kThreads>
__device__ __forceinline__ void flush_counters(double cost, unsigned long long singular, int want_cost, Counters* ctr) {
    __shared__ double red[kThreads / 32];
    __shared__ unsigned long long redn[kThreads / 32];
    const int tid = threadIdx.x, lane = tid & 31;
    const double c = warp_sum(cost);
    unsigned long long ns = singular;
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
        if (want_cost && tc != 0.0) atomicAdd(&ctr->cost_sum, tc);
        if (tn) atomicAdd(&ctr->singular, tn);
    }
}

// resident CTAs per SM each variant is compiled for (registers per thread
// are capped so that many batches are in flight on an SM at once)
__host__ __device__ constexpr int fused_min_blocks(int group, int rc) {
    return group >= 16 ? (rc >= 16 ? 1 : 2) : group == 8 ? (rc >= 16 ? 2 : 3) : 6;
}

template <typename Real, int GROUP, int RC>
__global__ void __launch_bounds__(32 * GROUP, fused_min_blocks(GROUP, RC)) k_em_fused_lists(FusedArgs<Real> a) {
    using R4 = typename Vec4<Real>::type;
    constexpr int kThreads = 32 * GROUP;
    constexpr int U = 4;  // loads in flight per lane for the pairs beyond the held ones
    __shared__ Real s_sum[3][kBatch];
    __shared__ Real s_k[3][kBatch];
    __shared__ __align__(16) R4 s_sd[kBatch];
    __shared__ Real s_pr2[kBatch];
    const int tid = threadIdx.x, lane = tid & 31;
    const int ms = tid / GROUP, glane = tid % GROUP;
    const unsigned gmask = GROUP == 32 ? kFull : (((1u << GROUP) - 1u) << (lane & ~(GROUP - 1)));
    const uint32_t V = a.V;
    const uint64_t nbatch = (static_cast<uint64_t>(a.N) + kBatch - 1) / kBatch;
    const uint64_t keep = l2_keep_policy();
    double cost_local = 0.0;
    unsigned long long singular_local = 0;

    for (uint64_t b = blockIdx.x; b < nbatch; b += gridDim.x) {
        const uint64_t mfirst = b * kBatch;
        // the 2x2 warp's per-muon inputs, copied to shared memory while the sums are formed
        if (tid < kBatch && mfirst + tid < a.N) stage_muon(&s_sd[tid], &s_pr2[tid], a.sd + mfirst + tid, a.pr2 + mfirst + tid);
        if (tid == 0 && a.prefetch) {  // the CTA's next batch into L2 while this one is worked on
            const uint64_t nb = b + gridDim.x;
            if (nb < nbatch) {
                const uint64_t m0 = nb * kBatch, m1 = min(m0 + kBatch, static_cast<uint64_t>(a.N));
                const uint64_t p0 = a.off[m0], p1 = a.off[m1];
                if (p1 > p0) {
                    prefetch_l2(a.vidx + p0, (p1 - p0) * sizeof(uint32_t));
                    prefetch_l2(a.L + p0, (p1 - p0) * sizeof(Real));
                    prefetch_l2(a.T + p0, (p1 - p0) * sizeof(Real));
                }
            }
        }
        const uint64_t m = mfirst + ms;
        uint64_t pb = 0, pe = 0;
        if (m < a.N) {
            pb = a.off[m];
            pe = a.off[m + 1];
        }
        // ---- the muon's pairs: the first GROUP*RC held in registers ----------
        uint32_t cj[RC];
        Real cL[RC], cT[RC];
#pragma unroll
        for (int r = 0; r < RC; ++r) {
            const uint64_t k = pb + glane + static_cast<uint64_t>(r) * GROUP;
            cj[r] = 0xffffffffu;
            cL[r] = Real(0);
            cT[r] = Real(0);
            if (k < pe) {
                cj[r] = __ldcs(a.vidx + k);
                cL[r] = __ldcs(a.L + k);
                cT[r] = __ldcs(a.T + k);
            }
        }
        Real c0 = 0, c1 = 0, c2 = 0;
#pragma unroll
        for (int r = 0; r < RC; ++r) {
            const Real l = cj[r] < V ? ld_keep(a.lam + cj[r], keep) : Real(0);
            if (cj[r] != 0xffffffffu) add_sigma(l, cL[r], cT[r], c0, c1, c2);
        }
        // pairs beyond the held ones (long paths): streamed, read again below
        const uint64_t ob = pb + static_cast<uint64_t>(GROUP) * RC;  // first pair beyond the held ones
        for (uint64_t k0 = ob + glane; k0 < pe; k0 += static_cast<uint64_t>(GROUP) * U) {
            uint32_t jj[U];
            Real ll[U], tt[U], lv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint64_t k = k0 + static_cast<uint64_t>(u) * GROUP;
                jj[u] = 0xffffffffu;
                if (k < pe) {
                    jj[u] = __ldg(a.vidx + k);
                    ll[u] = __ldg(a.L + k);
                    tt[u] = __ldg(a.T + k);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) lv[u] = jj[u] < V ? ld_keep(a.lam + jj[u], keep) : Real(0);
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (jj[u] != 0xffffffffu) add_sigma(lv[u], ll[u], tt[u], c0, c1, c2);
        }
#pragma unroll
        for (int o = GROUP / 2; o > 0; o >>= 1) {
            c0 += __shfl_xor_sync(gmask, c0, o, GROUP);
            c1 += __shfl_xor_sync(gmask, c1, o, GROUP);
            c2 += __shfl_xor_sync(gmask, c2, o, GROUP);
        }
        if (glane == 0) {
            s_sum[0][ms] = c0;
            s_sum[1][ms] = c1;
            s_sum[2][ms] = c2;
        }
        __syncthreads();
        // ---- FP64 2x2 algebra of the batch, a muon per lane of warp 0 --------
        if (tid < kBatch) {
            Real k0 = 0, k1 = 0, k2 = 0;
            cp_async_wait_all();  // this lane's own staged entries
            if (mfirst + tid < a.N)
                muon_coefficients<Real>(s_sum[0][tid], s_sum[1][tid], s_sum[2][tid], s_pr2[tid], s_sd[tid], a.E00,
                                        a.E01, a.E11, a.compute_cost != 0, k0, k1, k2, cost_local, singular_local);
            s_k[0][tid] = k0;
            s_k[1][tid] = k1;
            s_k[2][tid] = k2;
        }
        __syncthreads();
        // ---- g_ij of every pair added to G_j ------------------------------------
        const Real k0 = s_k[0][ms], k1 = s_k[1][ms], k2 = s_k[2][ms];
#pragma unroll
        for (int r = 0; r < RC; ++r)
            if (cj[r] < V) red_add(a.G + cj[r], g_term(k0, k1, k2, cL[r], cT[r]), keep);
        for (uint64_t k0p = ob + glane; k0p < pe; k0p += static_cast<uint64_t>(GROUP) * U) {
            uint32_t jj[U];
            Real ll[U], tt[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint64_t k = k0p + static_cast<uint64_t>(u) * GROUP;
                jj[u] = 0xffffffffu;
                if (k < pe) {  // read a second time (the first read left them in L1 or L2), and last
                    jj[u] = __ldcs(a.vidx + k);
                    ll[u] = __ldcs(a.L + k);
                    tt[u] = __ldcs(a.T + k);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (jj[u] < V) red_add(a.G + jj[u], g_term(k0, k1, k2, ll[u], tt[u]), keep);
        }
    }
    flush_counters<kThreads>(cost_local, singular_local, a.compute_cost, a.ctr);
}

// ---------------------------------------------------------------------------
// Staged one-pass variant: a CTA batch's pairs copied to shared memory.
// ---------------------------------------------------------------------------
// The 32 muons of a batch own one contiguous range of the muon-major lists.
// The CTA copies that range (up to kStagedPairs pairs) into shared memory
// with 16-byte cp.async copies, so the lists leave HBM once and the scatter
// reads them back from shared memory instead of from L2/HBM; pairs of a batch
// beyond the staged ones are read from global memory in both steps.  Two
// CTAs are resident per SM, so one copies its batch while the other works.
template <typename Real>
struct Staged {
    static constexpr int kPairs = sizeof(Real) == sizeof(float) ? 8192 : 4096;
    static constexpr int kSlots = kPairs + 8;  // room for the 16-byte widening at both ends
    static constexpr size_t kSmem = static_cast<size_t>(kSlots) * (sizeof(uint32_t) + 2 * sizeof(Real));
};
constexpr int kStagedGroup = 16;

template <typename Real>
__global__ void __launch_bounds__(32 * kStagedGroup, 2) k_em_staged(FusedArgs<Real> a) {
    using R4 = typename Vec4<Real>::type;
    using S = Staged<Real>;
    constexpr int GROUP = kStagedGroup;
    constexpr int kThreads = 32 * GROUP;
    constexpr int U = 4;                       // gathers in flight per lane
    constexpr int EJ = 16 / sizeof(uint32_t);  // elements per 16-byte copy
    constexpr int ER = 16 / sizeof(Real);
    extern __shared__ __align__(16) unsigned char staged_smem[];
    uint32_t* s_j = reinterpret_cast<uint32_t*>(staged_smem);
    Real* s_L = reinterpret_cast<Real*>(staged_smem + static_cast<size_t>(S::kSlots) * sizeof(uint32_t));
    Real* s_T = s_L + S::kSlots;
    __shared__ Real s_sum[3][kBatch];
    __shared__ Real s_k[3][kBatch];
    __shared__ __align__(16) R4 s_sd[kBatch];
    __shared__ Real s_pr2[kBatch];
    __shared__ uint32_t s_off[kBatch + 1];
    const int tid = threadIdx.x, lane = tid & 31;
    const int ms = tid / GROUP, glane = tid % GROUP;
    const unsigned gmask = ((1u << GROUP) - 1u) << (lane & ~(GROUP - 1));
    const uint32_t V = a.V;
    const uint64_t nbatch = (static_cast<uint64_t>(a.N) + kBatch - 1) / kBatch;
    const uint64_t keep = l2_keep_policy();
    double cost_local = 0.0;
    unsigned long long singular_local = 0;

    for (uint64_t b = blockIdx.x; b < nbatch; b += gridDim.x) {
        const uint64_t mfirst = b * kBatch;
        const uint64_t mend = min(mfirst + kBatch, static_cast<uint64_t>(a.N));
        const uint64_t p0 = a.off[mfirst], p1 = a.off[mend];
        const uint32_t nst = static_cast<uint32_t>(min(p1 - p0, static_cast<uint64_t>(S::kPairs)));  // staged
        // ---- the batch's pairs into shared memory ------------------------------
        // each array's copy starts at the 16-byte boundary at or below p0; the
        // arrays are padded past their last pair, so the widened end stays inside
        const uint64_t aj = p0 & ~static_cast<uint64_t>(EJ - 1), ar = p0 & ~static_cast<uint64_t>(ER - 1);
        const uint32_t sj = static_cast<uint32_t>(p0 - aj), sr = static_cast<uint32_t>(p0 - ar);
        const uint32_t cj = (sj + nst + EJ - 1) / EJ, cr = (sr + nst + ER - 1) / ER;
        for (uint32_t c = tid; c < cj; c += kThreads) cp_async_16(s_j + c * EJ, a.vidx + aj + c * EJ);
        for (uint32_t c = tid; c < cr; c += kThreads) {
            cp_async_16(s_L + c * ER, a.L + ar + c * ER);
            cp_async_16(s_T + c * ER, a.T + ar + c * ER);
        }
        if (tid < kBatch && mfirst + tid < mend) stage_muon(&s_sd[tid], &s_pr2[tid], a.sd + mfirst + tid, a.pr2 + mfirst + tid);
        if (tid <= kBatch) s_off[tid] = static_cast<uint32_t>(a.off[min(mfirst + tid, mend)] - p0);
        cp_async_wait_all();
        __syncthreads();
        // pair k of the batch (0-based): from shared memory, or global beyond the staged ones
        auto pair = [&](uint32_t k, uint32_t& j, Real& L, Real& T) {
            if (k < nst) {
                j = s_j[sj + k];
                L = s_L[sr + k];
                T = s_T[sr + k];
            } else {
                j = __ldg(a.vidx + p0 + k);
                L = __ldg(a.L + p0 + k);
                T = __ldg(a.T + p0 + k);
            }
        };
        uint32_t kb = 0, ke = 0;
        if (mfirst + ms < mend) {
            kb = s_off[ms];
            ke = s_off[ms + 1];
        }
        // ---- the covariance sums: GROUP lanes per muon, U gathers in flight ----
        Real c0 = 0, c1 = 0, c2 = 0;
        for (uint32_t k0 = kb + glane; k0 < ke; k0 += GROUP * U) {
            uint32_t jj[U];
            Real ll[U], tt[U], lv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t k = k0 + u * GROUP;
                jj[u] = 0xffffffffu;
                ll[u] = tt[u] = Real(0);
                if (k < ke) pair(k, jj[u], ll[u], tt[u]);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) lv[u] = jj[u] < V ? ld_keep(a.lam + jj[u], keep) : Real(0);
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (jj[u] != 0xffffffffu) add_sigma(lv[u], ll[u], tt[u], c0, c1, c2);
        }
#pragma unroll
        for (int o = GROUP / 2; o > 0; o >>= 1) {
            c0 += __shfl_xor_sync(gmask, c0, o, GROUP);
            c1 += __shfl_xor_sync(gmask, c1, o, GROUP);
            c2 += __shfl_xor_sync(gmask, c2, o, GROUP);
        }
        if (glane == 0) {
            s_sum[0][ms] = c0;
            s_sum[1][ms] = c1;
            s_sum[2][ms] = c2;
        }
        __syncthreads();
        // ---- FP64 2x2 algebra of the batch, a muon per lane of warp 0 --------
        if (tid < kBatch) {
            Real k0 = 0, k1 = 0, k2 = 0;
            if (mfirst + tid < mend)
                muon_coefficients<Real>(s_sum[0][tid], s_sum[1][tid], s_sum[2][tid], s_pr2[tid], s_sd[tid], a.E00,
                                        a.E01, a.E11, a.compute_cost != 0, k0, k1, k2, cost_local, singular_local);
            s_k[0][tid] = k0;
            s_k[1][tid] = k1;
            s_k[2][tid] = k2;
        }
        __syncthreads();
        // ---- g_ij of every pair added to G_j, the pairs read back -------------
        const Real k0 = s_k[0][ms], k1 = s_k[1][ms], k2 = s_k[2][ms];
        for (uint32_t q0 = kb + glane; q0 < ke; q0 += GROUP * U) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t k = q0 + u * GROUP;
                if (k < ke) {
                    uint32_t j;
                    Real L, T;
                    pair(k, j, L, T);
                    if (j < V) red_add(a.G + j, g_term(k0, k1, k2, L, T), keep);
                }
            }
        }
        __syncthreads();  // the staging buffers are refilled by the next batch
    }
    flush_counters<kThreads>(cost_local, singular_local, a.compute_cost, a.ctr);
}

// ---------------------------------------------------------------------------
// Recompute pass: the merged path walked in FP64 twice per iteration.
// ---------------------------------------------------------------------------
// The merged split path of getMuonPathAndTail (src/MutoMLSD.cpp:382-415): the
// in-half, then the out-half without its first voxel, whose length is added to
// the last in-voxel (dropped when the in-half is empty) -- the same rule as
// the set-up's fill walk, handing every pair to `emit(x, y, z, length)`.
template <class Emit>
struct MergedSink {
    Emit* e;
    int phase = 0;  // 0: in-half, 1: first out voxel, 2: rest of the out-half
    bool pending = false;
    uint32_t px = 0, py = 0, pz = 0;
    double pl = 0.0;
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) {
        if (phase == 0) {
            if (pending) (*e)(px, py, pz, pl);
            pending = true;
            px = x;
            py = y;
            pz = z;
            pl = l;
        } else if (phase == 1) {
            if (pending) {
                (*e)(px, py, pz, dadd(pl, l));
                pending = false;
            }
            phase = 2;
        } else {
            (*e)(x, y, z, l);
        }
    }
    __device__ void finish() {
        if (pending) (*e)(px, py, pz, dadd(pl, 0.0));  // out-half empty: length += 0.0
        pending = false;
    }
};
template <class Emit>
struct PlainSink {  // straight_line: the segment pin -> pout as it is
    Emit* e;
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) { (*e)(x, y, z, l); }
};

// Walks the muon's path as the set-up does and hands every pair to emit;
// false when a walk hit its step bound (the set-up drops such a muon).
// `lanes`: the warp's lanes making this walk (walk_lanes), synced between the halves.
template <class Emit>
__device__ __forceinline__ bool walk_path(const DevGrid& g, const muto_ray& r, const double* ps, int straight,
                                          Emit& emit, unsigned lanes) {
    if (straight) {
        PlainSink<Emit> s{&emit};
        return siddon_walk(g, r.pin, r.pout, s) >= 0;
    }
    MergedSink<Emit> s{&emit};
    const int ci = siddon_walk(g, r.pin, ps, s);
    s.phase = 1;
    __syncwarp(lanes);
    const int co = siddon_walk(g, ps, r.pout, s);
    s.finish();
    return ci >= 0 && co >= 0;
}

struct VoxelIndexer {
    uint32_t nx, nxy;
    BrickDims b;
    int brick;
    __device__ __forceinline__ uint32_t operator()(uint32_t x, uint32_t y, uint32_t z) const {
        if (!brick) return x + y * nx + z * nxy;  // xyz2index, include/MutoMLSD.h:76
        return brick_xyz(x, y, z, b);
    }
};

// The covariance sums along a walk.  The lambda gathers are pipelined three
// pairs deep (a shift register of fixed slots, so it stays in registers):
// pair k's gather is issued when the walk reaches it and consumed three
// pairs later, so the walk's FP64 steps overlap the gathers' L2 latency.
template <typename Real>
struct SumEmit {
    const Real* lam;
    VoxelIndexer ix;
    uint64_t keep;
    double ltot, run = 0.0;
    Real c0 = 0, c1 = 0, c2 = 0;
    int n = 0;  // pairs in flight (0..3)
    Real l0 = 0, l1 = 0, l2 = 0, L0 = 0, L1 = 0, L2 = 0, T0 = 0, T1 = 0, T2 = 0;
    __device__ __forceinline__ void shift_in(Real l, Real L, Real T) {
        if (n == 3) add_sigma(l0, L0, T0, c0, c1, c2);
        l0 = l1; L0 = L1; T0 = T1;
        l1 = l2; L1 = L2; T1 = T2;
        l2 = l; L2 = L; T2 = T;
        n = n < 3 ? n + 1 : 3;
    }
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) {
        run += l;
        const double t = ltot - run;  // T_ij: the in-grid length after the pair
        shift_in(ld_keep(lam + ix(x, y, z), keep), static_cast<Real>(l), static_cast<Real>(t > 0.0 ? t : 0.0));
    }
    __device__ void drain() {  // the pairs still in flight, oldest first
        for (int k = 0; k < 3; ++k) shift_in(Real(0), Real(0), Real(0));
    }
};
template <typename Real>
struct ScatterEmit {
    Real* G;
    VoxelIndexer ix;
    uint64_t keep;
    double ltot, run = 0.0;
    Real k0, k1, k2;
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) {
        run += l;
        const double t = ltot - run;
        red_add(G + ix(x, y, z), g_term(k0, k1, k2, static_cast<Real>(l), static_cast<Real>(t > 0.0 ? t : 0.0)), keep);
    }
};

template <typename Real>
__global__ void __launch_bounds__(128) k_em_fused_walk(FusedArgs<Real> a) {
    using R4 = typename Vec4<Real>::type;
    double cost_local = 0.0;
    unsigned long long singular_local = 0;
    const VoxelIndexer ix{a.g.n[0], a.g.n[0] * a.g.n[1], a.bdims, a.brick};
    const uint64_t keep = l2_keep_policy();
    // a thread per muon (not a grid-stride loop, whose lanes would drift out
    // of step), the muons in a.order (by decreasing path bound) when given
    const uint64_t t = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const uint64_t i = (a.order && t < a.N) ? a.order[t] : t;
    // (ltot < 0: a walk the set-up dropped at its step bound: no pairs)
    const double ltot = i < a.N ? a.ltot[i] : -1.0;
    const unsigned lanes = walk_lanes(ltot >= 0.0);
    if (ltot >= 0.0) {
        const muto_ray r = a.rays[a.kept[i]];
        const double ps[3] = {a.scat[3 * i], a.scat[3 * i + 1], a.scat[3 * i + 2]};
        SumEmit<Real> se{a.lam, ix, keep, ltot};
        walk_path(a.g, r, ps, a.straight, se, lanes);
        se.drain();
        Real k0, k1, k2;
        muon_coefficients<Real>(se.c0, se.c1, se.c2, a.pr2[i], a.sd[i], a.E00, a.E01, a.E11, a.compute_cost != 0,
                                k0, k1, k2, cost_local, singular_local);
        ScatterEmit<Real> ce{a.G, ix, keep, ltot, 0.0, k0, k1, k2};
        __syncwarp(lanes);
        walk_path(a.g, r, ps, a.straight, ce, lanes);
    }
    flush_counters<128>(cost_local, singular_local, a.compute_cost, a.ctr);
}

// Set-up of the recompute form: every kept muon's in-grid length (its merged
// path walked once, -1 for a walk that hit its step bound, which the set-up
// drops) and the pairs per voxel M_j.
struct StatEmit {
    uint32_t* mult;
    uint32_t nx, nxy;
    double run = 0.0;
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double l) {
        run += l;
        atomicAdd(mult + (x + y * nx + z * nxy), 1u);
    }
};
__global__ void k_path_stats(const muto_ray* __restrict__ rays, const uint32_t* __restrict__ kept,
                             const double* __restrict__ scat, uint64_t n, DevGrid g, int straight,
                             double* __restrict__ ltot, uint32_t* __restrict__ mult, Counters* ctr) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const unsigned lanes = walk_lanes(i < n);
    if (i >= n) return;
    const muto_ray r = rays[kept[i]];
    const double ps[3] = {scat[3 * i], scat[3 * i + 1], scat[3 * i + 2]};
    StatEmit e{mult, g.n[0], g.n[0] * g.n[1]};
    if (!walk_path(g, r, ps, straight, e, lanes)) {
        // dropped like the set-up's fill walk drops it; its voxels were counted
        // as they were walked, so count the same walk again with -1
        atomicAdd(&ctr->overflow, 1ull);
        ltot[i] = -1.0;
        return;
    }
    ltot[i] = e.run;
}

struct UncountEmit {
    uint32_t* mult;
    uint32_t nx, nxy;
    __device__ void operator()(uint32_t x, uint32_t y, uint32_t z, double) { atomicSub(mult + (x + y * nx + z * nxy), 1u); }
};
__global__ void k_path_uncount(const muto_ray* __restrict__ rays, const uint32_t* __restrict__ kept,
                               const double* __restrict__ scat, uint64_t n, DevGrid g, int straight,
                               const double* __restrict__ ltot, uint32_t* __restrict__ mult) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool again = i < n && ltot[i] < 0.0;
    const unsigned lanes = walk_lanes(again);
    if (!again) return;
    const muto_ray r = rays[kept[i]];
    const double ps[3] = {scat[3 * i], scat[3 * i + 1], scat[3 * i + 2]};
    UncountEmit e{mult, g.n[0], g.n[0] * g.n[1]};
    walk_path(g, r, ps, straight, e, lanes);
}

// The voxel side: lambda_j + lambda_j^2 G_j / (2 M_j) (0 when M_j = 0), or the
// gradient -lambda_j G_j of the NLL with respect to log(lambda_j); G_j is
// cleared for the next pass.  Each thread takes kUpdateVox voxels a block's
// width apart and issues all their loads before using any: the pass is bound
// by load latency, not bandwidth, with one voxel per thread.
constexpr int kUpdateVox = 4;
constexpr int kUpdateThreads = 256;

template <typename Real, typename OutT>
__global__ void __launch_bounds__(kUpdateThreads) k_mean_update(const Real* __restrict__ lam, Real* __restrict__ G,
                                                                const uint32_t* __restrict__ mult, uint32_t V,
                                                                BrickDims bd, int brick, OutT* __restrict__ out,
                                                                double* __restrict__ grad,
                                                                const double* __restrict__ lam64) {
    const uint32_t base = blockIdx.x * (kUpdateThreads * kUpdateVox) + threadIdx.x;
    uint32_t jb[kUpdateVox];
    Real gj[kUpdateVox], lj[kUpdateVox];
    uint32_t Mj[kUpdateVox];
    double l64[kUpdateVox];
#pragma unroll
    for (int u = 0; u < kUpdateVox; ++u) {
        const uint32_t j = base + u * kUpdateThreads;
        jb[u] = j < V ? (brick ? brick_of(j, bd) : j) : 0xffffffffu;
        gj[u] = jb[u] != 0xffffffffu ? G[jb[u]] : Real(0);
        Mj[u] = j < V ? mult[j] : 0u;
        if (grad) l64[u] = j < V ? lam64[j] : 0.0;
        else lj[u] = j < V ? lam[j] : Real(0);
    }
#pragma unroll
    for (int u = 0; u < kUpdateVox; ++u) {
        const uint32_t j = base + u * kUpdateThreads;
        if (j >= V) break;
        G[jb[u]] = Real(0);
        const uint32_t M = Mj[u];
        if (grad) {
            grad[j] = M ? -l64[u] * static_cast<double>(gj[u]) : 0.0;
            continue;
        }
        if constexpr (sizeof(Real) == sizeof(float)) {
            // the mixed form: lambda is stored in FP32, so its increment is
            // formed in FP32 too (GB300 issues FP64 at a sixty-fourth of the
            // FP32 rate; an FP64 division per voxel cost more than the loads)
            const float l = lj[u];
            const float inc = l * l * gj[u] / (2.0f * static_cast<float>(M));
            if constexpr (sizeof(OutT) == sizeof(float)) out[j] = M ? l + inc : 0.0f;
            else out[j] = M ? static_cast<double>(l) + static_cast<double>(inc) : 0.0;
        } else {
            const double l = static_cast<double>(lj[u]);
            out[j] = M ? static_cast<OutT>(l + l * l * static_cast<double>(gj[u]) / (2.0 * static_cast<double>(M)))
                       : OutT(0);
        }
    }
}

template <typename Real, int GROUP, int RC>
int fused_blocks_per_sm() {
    int n = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_em_fused_lists<Real, GROUP, RC>, 32 * GROUP, 0);
    return (e == cudaSuccess && n > 0) ? n : 1;
}

// The scatter of the split form: the per-muon coefficients come from the
// muon pass (em_muon.cu) in kvec; GROUP lanes per muon stream its pairs a
// second time and add g_ij to G_j.  No block barrier and no FP64.  U pairs
// are in flight per lane; with AHEAD the next muon's offsets and
// coefficients are loaded while the current muon's pairs are, so a muon's
// pair loads do not wait on its offsets.
template <typename Real, int GROUP, int U, bool AHEAD>
__global__ void __launch_bounds__(256) k_em_scatter(FusedArgs<Real> a, const typename Vec4<Real>::type* __restrict__ kvec) {
    using R4 = typename Vec4<Real>::type;
    const uint64_t gid = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / GROUP;
    const uint64_t ngroups = (static_cast<uint64_t>(gridDim.x) * blockDim.x) / GROUP;
    const int glane = threadIdx.x % GROUP;
    const uint32_t V = a.V;
    const uint64_t keep = l2_keep_policy();
    uint64_t m = gid;
    R4 kv{};
    uint64_t pb = 0, pe = 0;
    if (AHEAD && m < a.N) {
        kv = kvec[m];
        pb = a.off[m];
        pe = a.off[m + 1];
    }
    for (; m < a.N; m += ngroups) {
        R4 kn{};
        uint64_t pbn = 0, pen = 0;
        if (AHEAD) {
            const uint64_t mn = m + ngroups;
            if (mn < a.N) {
                kn = kvec[mn];
                pbn = a.off[mn];
                pen = a.off[mn + 1];
            }
        } else {
            kv = kvec[m];
            pb = a.off[m];
            pe = a.off[m + 1];
        }
        for (uint64_t k0 = pb + glane; k0 < pe; k0 += static_cast<uint64_t>(GROUP) * U) {
            uint32_t jj[U];
            Real ll[U], tt[U];
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
            for (int u = 0; u < U; ++u)
                if (jj[u] < V) red_add(a.G + jj[u], g_term(kv.x, kv.y, kv.z, ll[u], tt[u]), keep);
        }
        if (AHEAD) {
            kv = kn;
            pb = pbn;
            pe = pen;
        }
    }
}

}  // namespace

// (GROUP, RC) of each stored-list variant; the last is the staged one (GROUP
// lanes per muon, its batch's pairs in shared memory)
static constexpr int kFusedGroup[kFusedVariants] = {4, 8, 8, 16, 16, 8, kStagedGroup};
static constexpr int kFusedHeld[kFusedVariants] = {8, 8, 16, 8, 16, 4, 0};
int fused_variant_group(int v) { return kFusedGroup[v]; }
int fused_variant_held(int v) {
    return v == kFusedStaged ? Staged<float>::kPairs / kBatch : kFusedGroup[v] * kFusedHeld[v];
}

template <typename Real>
int staged_blocks_per_sm() {
    int n = 0;
    if (cudaFuncSetAttribute(k_em_staged<Real>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(Staged<Real>::kSmem)) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_em_staged<Real>, 32 * kStagedGroup, Staged<Real>::kSmem) !=
            cudaSuccess)
        n = 0;
    return n > 0 ? n : 1;
}

template <typename Real>
int em_fused_blocks(int variant) {
    switch (variant) {
        case kFusedStaged: return staged_blocks_per_sm<Real>();
        case 0: return fused_blocks_per_sm<Real, 4, 8>();
        case 1: return fused_blocks_per_sm<Real, 8, 8>();
        case 2: return fused_blocks_per_sm<Real, 8, 16>();
        case 3: return fused_blocks_per_sm<Real, 16, 8>();
        case 4: return fused_blocks_per_sm<Real, 16, 16>();
        default: return fused_blocks_per_sm<Real, 8, 4>();
    }
}
template int em_fused_blocks<float>(int);
template int em_fused_blocks<double>(int);

template <typename Real>
void launch_em_fused(const FusedArgs<Real>& a, int variant, int blocks, cudaStream_t s) {
    if (a.N == 0) return;
    const uint64_t batches = (static_cast<uint64_t>(a.N) + kBatch - 1) / kBatch;
    const unsigned nb = static_cast<unsigned>(batches < static_cast<uint64_t>(blocks) ? batches : blocks);
#define MUTO_FUSED_LAUNCH(G, RC) k_em_fused_lists<Real, G, RC><<<nb, 32 * G, 0, s>>>(a)
    switch (variant) {
        case kFusedStaged:
            k_em_staged<Real><<<nb, 32 * kStagedGroup, Staged<Real>::kSmem, s>>>(a);
            break;
        case 0: MUTO_FUSED_LAUNCH(4, 8); break;
        case 1: MUTO_FUSED_LAUNCH(8, 8); break;
        case 2: MUTO_FUSED_LAUNCH(8, 16); break;
        case 3: MUTO_FUSED_LAUNCH(16, 8); break;
        case 4: MUTO_FUSED_LAUNCH(16, 16); break;
        default: MUTO_FUSED_LAUNCH(8, 4); break;
    }
#undef MUTO_FUSED_LAUNCH
    count_launches(1);
}
template void launch_em_fused<float>(const FusedArgs<float>&, int, int, cudaStream_t);

template <typename Real, int GROUP, int U, bool AHEAD>
int scatter_blocks_per_sm() {
    int n = 0;
    const cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_em_scatter<Real, GROUP, U, AHEAD>, 256, 0);
    return (e == cudaSuccess && n > 0) ? n : 1;
}

template <typename Real>
int em_scatter_blocks(int group, int depth) {
    if (depth > 4) {
        if (group <= 8) return scatter_blocks_per_sm<Real, 8, 8, true>();
        if (group <= 16) return scatter_blocks_per_sm<Real, 16, 8, true>();
        return scatter_blocks_per_sm<Real, 32, 8, true>();
    }
    if (group <= 8) return scatter_blocks_per_sm<Real, 8, 4, false>();
    if (group <= 16) return scatter_blocks_per_sm<Real, 16, 4, false>();
    return scatter_blocks_per_sm<Real, 32, 4, false>();
}
template int em_scatter_blocks<float>(int, int);
template int em_scatter_blocks<double>(int, int);

template <typename Real>
void launch_em_scatter(const FusedArgs<Real>& a, const typename Vec4<Real>::type* kvec, int group, int depth,
                       int blocks, cudaStream_t s) {
    if (a.N == 0) return;
    const uint64_t need = (static_cast<uint64_t>(a.N) * group + 255) / 256;
    const unsigned nb = static_cast<unsigned>(need < static_cast<uint64_t>(blocks) ? need : blocks);
    if (depth > 4) {
        if (group <= 8) k_em_scatter<Real, 8, 8, true><<<nb, 256, 0, s>>>(a, kvec);
        else if (group <= 16) k_em_scatter<Real, 16, 8, true><<<nb, 256, 0, s>>>(a, kvec);
        else k_em_scatter<Real, 32, 8, true><<<nb, 256, 0, s>>>(a, kvec);
    } else {
        if (group <= 8) k_em_scatter<Real, 8, 4, false><<<nb, 256, 0, s>>>(a, kvec);
        else if (group <= 16) k_em_scatter<Real, 16, 4, false><<<nb, 256, 0, s>>>(a, kvec);
        else k_em_scatter<Real, 32, 4, false><<<nb, 256, 0, s>>>(a, kvec);
    }
    count_launches(1);
}
template void launch_em_scatter<float>(const FusedArgs<float>&, const float4*, int, int, int, cudaStream_t);
template void launch_em_scatter<double>(const FusedArgs<double>&, const double4*, int, int, int, cudaStream_t);
template void launch_em_fused<double>(const FusedArgs<double>&, int, int, cudaStream_t);

template <typename Real>
void launch_em_fused_walk(const FusedArgs<Real>& a, int num_sms, cudaStream_t s) {
    if (a.N == 0) return;
    (void)num_sms;
    k_em_fused_walk<Real><<<static_cast<unsigned>((static_cast<uint64_t>(a.N) + 127) / 128), 128, 0, s>>>(a);
    count_launches(1);
}
template void launch_em_fused_walk<float>(const FusedArgs<float>&, int, cudaStream_t);
template void launch_em_fused_walk<double>(const FusedArgs<double>&, int, cudaStream_t);

void launch_path_stats(const muto_ray* rays, const uint32_t* kept, const double* scat, uint64_t n, muto_grid g,
                       int straight, double* ltot, uint32_t* mult, Counters* ctr, cudaStream_t s) {
    if (n == 0) return;
    const unsigned nb = static_cast<unsigned>((n + 127) / 128);
    k_path_stats<<<nb, 128, 0, s>>>(rays, kept, scat, n, make_dev_grid(g), straight, ltot, mult, ctr);
    k_path_uncount<<<nb, 128, 0, s>>>(rays, kept, scat, n, make_dev_grid(g), straight, ltot, mult);
    count_launches(2);
}

template <typename Real, typename OutT>
void launch_mean_update(const Real* lam, Real* G, const uint32_t* mult, uint32_t V, const BrickDims* brick, OutT* out,
                        double* grad, const double* lam64, cudaStream_t s) {
    if (V == 0) return;
    const uint32_t per_block = kUpdateThreads * kUpdateVox;
    k_mean_update<Real, OutT><<<(V + per_block - 1) / per_block, kUpdateThreads, 0, s>>>(
        lam, G, mult, V, brick ? *brick : BrickDims{}, brick ? 1 : 0, out, grad, lam64);
    count_launches(1);
}
template void launch_mean_update<float, float>(const float*, float*, const uint32_t*, uint32_t, const BrickDims*,
                                               float*, double*, const double*, cudaStream_t);
template void launch_mean_update<float, double>(const float*, float*, const uint32_t*, uint32_t, const BrickDims*,
                                                double*, double*, const double*, cudaStream_t);
template void launch_mean_update<double, double>(const double*, double*, const uint32_t*, uint32_t,
                                                 const BrickDims*, double*, double*, const double*, cudaStream_t);

}  // namespace muto
