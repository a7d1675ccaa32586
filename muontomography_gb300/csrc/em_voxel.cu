// Voxel pass of an EM iteration: the per-voxel update of src/MutoMLSD.cpp:493-517
// (updateImageVoxel, run for every voxel at :197-200), and the MAP step of
// src/MutoMAP.cpp:228-247.
//
// The pairs are also stored voxel-major (muon, L, T), built once at setup.
// Two steps:
//   key pass     one thread per pair streams the lists, gathers its muon's
//                coefficients k_i (written by the muon pass; rows in column
//                order of the PoCA points when the table outgrows L2) and
//                writes g_ij = k0 W00 + k1 W01 + k2 W11 as an order-preserving
//                integer key, voxel-major.  The gather runs at full
//                occupancy, apart from the selection.
//   class pass   one warp per voxel reads its M_j keys (coalesced, 4 or 8 B
//                each) and selects on them; s_ij = 2 l_j + g_ij l_j^2, the
//                reference's 2 l + (1/2 xyS - tr(Sigma^-1 W)) pr^2 l^2, is
//                non-decreasing in g_ij, so an order statistic of the keys is
//                one of the s_ij, formed only for the values the update uses.
// Nothing is accumulated with atomics.
//   median       exact order statistics of the s_ij (nth_element semantics).
//                Each voxel starts from the window its previous selection
//                left (one pass: keys below it counted, keys inside kept in
//                shared memory, sorted by a warp bitonic sort when <= 64).
//                Without one, or when it misses, rounds of sampling narrow
//                the search: 32 samples spread over the segment are sorted in
//                the warp, the keys within 6 sample ranks of the target are
//                counted and kept, the same is done on the kept keys, and the
//                survivors (<= 64) are sorted.  A window that misses the
//                target twice falls back to a bitwise radix search.
//   percentile   mean of the lowest floor(pct/100 M) values: the order
//                statistic t plus the sum of the values below it.
//   mean         l + l^2 (sum_i g_ij) / (2 M)  ==  (sum_i s_ij) / M / 2.
//   gradient     d NLL / d log l_j = -l_j sum_i g_ij (the adjoint).
// Voxels are grouped by segment length into classes, each its own kernel
// instantiation, so short segments run with few registers and many warps.
#include <algorithm>
#include <utility>

#include "common.cuh"

namespace muto {
namespace {

constexpr int kVoxThreads = 256;
constexpr int kWarps = kVoxThreads / 32;

// Rows of 32 keys in each of a warp's two candidate buffers.  Segments held
// in registers get enough for any first window (at most R rows per lane).
// Streamed segments get about 0.6 R + 4, at most 28 (a first window keeps
// about 3/8 of the keys); the class beyond the register budget keeps 48
// (32-bit keys) or 24 rows.  A window that does not fit its buffer ends in
// the radix search over the key array.
template <typename K, int C, bool STREAMED>
__host__ __device__ constexpr int cand_rows() {
    return STREAMED ? (vox_class_rows(C) == 0 || (vox_class_rows(C) * 5) / 8 + 4 > 28 ? 28
                                                                               : (vox_class_rows(C) * 5) / 8 + 4)
         : vox_class_rows(C) == 0 ? (sizeof(K) == 4 ? 48 : 24)
         : (vox_class_rows(C) < 8 ? 8 : vox_class_rows(C));
}
// resident blocks per SM each class kernel is compiled for (its register cap)
__host__ __device__ constexpr int vox_min_blocks(int C, bool streamed) {
    return streamed ? 4 : C <= 4 ? 5 : C <= 6 ? 4 : C == 7 ? 4 : C == 8 ? 3 : C == 9 ? 2 : 5;
}
// classes whose segments are long enough (M > 256) to be selected by the
// streamed path
__host__ __device__ constexpr bool streamable(int C) { return C >= 5; }
template <typename K, int C, bool STREAMED>
__host__ __device__ constexpr size_t voxel_smem_bytes() {
    return size_t(2) * kWarps * cand_rows<K, C, STREAMED>() * 32 * sizeof(K);
}

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

// Keys are order-preserving images of finite values, so the all-ones key
// (a NaN pattern) never occurs: it marks empty slots.
template <typename K>
__device__ __forceinline__ constexpr K empty_key() { return ~K(0); }

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

// Key sources.  Each gives rows() rows of one key per lane (get(r), the
// empty key where a lane has none), one sample per lane, and each() over
// its own keys only.

// The voxel's s_ij in registers: element r*32+lane in key[r], empty past M.
template <typename Real, int R>
struct VoxKeys {
    using K = typename KeyOf<Real>::type;
    K key[R];
    uint32_t M;
    int lane;
    static constexpr bool kBounded = true;  // a lane never has more than R keys
    __device__ __forceinline__ uint32_t rows() const { return R; }
    __device__ __forceinline__ K get(int r) const { return key[r]; }
    // one key per lane from rows spread over the segment (row lane*R/32, or
    // the last row holding an element of this lane), so that the samples do
    // not all come from the segment's first 32 elements
    __device__ __forceinline__ K sample() const {
        uint32_t t = (static_cast<uint32_t>(lane) * R) >> 5;
        const uint32_t last = M > static_cast<uint32_t>(lane) ? (M - 1 - lane) >> 5 : 0;
        if (t > last) t = last;
        K s = key[0];
#pragma unroll
        for (int r = 1; r < R; ++r)
            if (static_cast<uint32_t>(r) == t) s = key[r];
        return s;
    }
    template <class F>
    __device__ __forceinline__ void each(F f) const {
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (static_cast<uint32_t>(r * 32 + lane) < M) f(key[r]);
    }
};

// A segment's keys in the global key array, contiguous.
template <typename K>
struct PtrKeys {
    const K* p;
    uint32_t n;
    int lane;
    static constexpr bool kBounded = false;
    __device__ __forceinline__ uint32_t rows() const { return (n + 31) >> 5; }
    __device__ __forceinline__ K get(uint32_t r) const {
        const uint32_t i = r * 32 + lane;
        return i < n ? p[i] : empty_key<K>();
    }
    __device__ __forceinline__ K sample() const { return p[(lane * n) >> 5]; }
    template <class F>
    __device__ __forceinline__ void each(F f) const {
        constexpr uint32_t B = 8;  // eight loads in flight
        uint32_t i = lane;
        for (; i + 32 * (B - 1) < n; i += 32 * B) {
            K x[B];
#pragma unroll
            for (uint32_t b = 0; b < B; ++b) x[b] = p[i + 32 * b];
#pragma unroll
            for (uint32_t b = 0; b < B; ++b) f(x[b]);
        }
        for (; i < n; i += 32) f(p[i]);
    }
};

// Window candidates in shared memory, ragged: lane l holds t keys, at rows
// 0 .. t-1 of column l; rows is the largest t of the warp.
template <typename K>
struct Ragged {
    K* buf;
    uint32_t t, nrows;
    int lane;
    static constexpr bool kBounded = false;
    __device__ __forceinline__ uint32_t rows() const { return nrows; }
    __device__ __forceinline__ K get(uint32_t r) const { return r < t ? buf[r * 32 + lane] : empty_key<K>(); }
    __device__ __forceinline__ K sample() const { return t > 0 ? buf[lane] : empty_key<K>(); }
    template <class F>
    __device__ __forceinline__ void each(F f) const {
        for (uint32_t r = 0; r < t; ++r) f(buf[r * 32 + lane]);
    }
};

// order statistic k of a segment and, when the final candidates hold it,
// order statistic k-1 (the lower median of an even segment)
template <typename K>
struct Sel {
    K kth, prev;
    bool have_prev;
    K wlo, whi;     // smallest and largest key of the final sorted candidates
    uint32_t nfin;  // their number (0: the selection ended in a radix search)
};

// ascending warp bitonic sort of one key per lane
template <typename K>
__device__ __forceinline__ K sort32(K s, int lane) {
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
    return s;
}

// order statistics k and k-1 of n <= 32 contiguous keys in shared memory
template <typename K>
__device__ Sel<K> sel32(const K* c, uint32_t n, uint32_t k, int lane) {
    const K s = sort32(static_cast<uint32_t>(lane) < n ? c[lane] : empty_key<K>(), lane);
    Sel<K> r;
    r.kth = __shfl_sync(kFull, s, static_cast<int>(k));
    r.prev = __shfl_sync(kFull, s, static_cast<int>(k ? k - 1 : 0));
    r.have_prev = k >= 1;
    r.wlo = __shfl_sync(kFull, s, 0);
    r.whi = __shfl_sync(kFull, s, static_cast<int>(n - 1));
    r.nfin = n;
    return r;
}

// order statistics k and k-1 of n <= 64 contiguous keys in shared memory:
// warp bitonic sort of 64 (element e = 2 lane + t in register t of its lane)
template <typename K>
__device__ Sel<K> sel64(const K* c, uint32_t n, uint32_t k, int lane) {
    K a = static_cast<uint32_t>(2 * lane) < n ? c[2 * lane] : empty_key<K>();
    K b = static_cast<uint32_t>(2 * lane + 1) < n ? c[2 * lane + 1] : empty_key<K>();
#pragma unroll
    for (int size = 2; size <= 64; size <<= 1) {
        const bool up = ((2 * lane) & size) == 0 || size == 64;
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride == 1) {
                const K lo = a < b ? a : b, hi = a < b ? b : a;
                a = up ? lo : hi;
                b = up ? hi : lo;
            } else {
                const int ls = stride >> 1;
                const K pa = __shfl_xor_sync(kFull, a, ls), pb = __shfl_xor_sync(kFull, b, ls);
                const bool keep_min = ((lane & ls) == 0) == up;
                a = keep_min ? (pa < a ? pa : a) : (pa > a ? pa : a);
                b = keep_min ? (pb < b ? pb : b) : (pb > b ? pb : b);
            }
        }
    }
    const uint32_t kp = k ? k - 1 : 0;
    const K va = __shfl_sync(kFull, a, static_cast<int>(k >> 1)), vb = __shfl_sync(kFull, b, static_cast<int>(k >> 1));
    const K pa = __shfl_sync(kFull, a, static_cast<int>(kp >> 1)), pb = __shfl_sync(kFull, b, static_cast<int>(kp >> 1));
    const uint32_t kl = n - 1;
    const K la = __shfl_sync(kFull, a, static_cast<int>(kl >> 1)), lb = __shfl_sync(kFull, b, static_cast<int>(kl >> 1));
    Sel<K> r;
    r.kth = (k & 1u) ? vb : va;
    r.prev = (kp & 1u) ? pb : pa;
    r.have_prev = k >= 1;
    r.wlo = __shfl_sync(kFull, a, 0);
    r.whi = (kl & 1u) ? lb : la;
    r.nfin = n;
    return r;
}

// Outcome of a window pass.
enum WinStatus { kWinCand = 0, kWinEqual = 1, kWinFail = 2 };

// One pass over n keys with the window [lo, hi]: counts the keys below it
// and appends those inside to the lane's own column of `out` (no cross-lane
// compaction).  kWinCand: `res` holds the candidates and rank k is among
// them.  kWinEqual: the window is one key value and holds rank k, so that
// value is the answer, written to *direct (runs of equal keys need no more
// rounds).  kWinFail: the window misses rank k, overflows `out_rows` or
// keeps everything.
template <typename K, class Src>
__device__ __forceinline__ int window_pass(const Src& v, uint32_t n, uint32_t k, K lo, K hi, K* out,
                                           uint32_t out_rows, int lane, Ragged<K>& res, uint32_t& below,
                                           Sel<K>* direct) {
    uint32_t c_lo = 0, t = 0;
    const uint32_t nr = v.rows();
    auto one = [&](K x) {
        const bool lt = x < lo;
        c_lo += lt ? 1u : 0u;
        if (!lt && x <= hi) {
            if (Src::kBounded || t < out_rows) out[t * 32 + lane] = x;
            ++t;
        }
    };
    if constexpr (Src::kBounded) {  // keys in registers
#pragma unroll
        for (uint32_t r = 0; r < nr; ++r) one(v.get(r));
    } else {  // keys in memory: eight rows' loads in flight before their stores
        constexpr uint32_t B = 8;
        uint32_t r = 0;
        for (; r + B <= nr; r += B) {
            K x[B];
#pragma unroll
            for (uint32_t b = 0; b < B; ++b) x[b] = v.get(r + b);
#pragma unroll
            for (uint32_t b = 0; b < B; ++b) one(x[b]);
        }
        for (; r < nr; ++r) one(v.get(r));
    }
    below = __reduce_add_sync(kFull, c_lo);
    const uint32_t n_in = __reduce_add_sync(kFull, t);
    const uint32_t rows = __reduce_max_sync(kFull, t);
    res.buf = out;
    res.t = t;
    res.nrows = rows;
    res.lane = lane;
    const bool hit = below <= k && k < below + n_in;
    if (hit && lo == hi) {
        direct->kth = lo;
        direct->prev = lo;
        direct->have_prev = k > below;
        direct->wlo = lo;
        direct->whi = lo;
        direct->nfin = n_in;
        return kWinEqual;
    }
    return hit && rows <= out_rows && n_in < n ? kWinCand : kWinFail;
}

// One sampling round: the (up to 32) samples are sorted in the warp and the
// window is the keys within `reach` (6) sample ranks of rank k (window_pass).
template <typename K, class Src>
__device__ __forceinline__ int sample_round(const Src& v, uint32_t n, uint32_t k, K* out, uint32_t out_rows,
                                            int lane, Ragged<K>& res, uint32_t& below, Sel<K>* direct,
                                            int reach = 6) {
    const K smp = v.sample();
    const uint32_t ns = __popc(__ballot_sync(kFull, smp != empty_key<K>()));
    const K s = sort32(smp, lane);  // empty samples sort last
    const int pos = static_cast<int>((static_cast<float>(k) * static_cast<float>(ns)) / static_cast<float>(n));
    const int ql = pos - reach, qh = pos + reach;
    const K slo = __shfl_sync(kFull, s, ql < 0 ? 0 : (ql > 31 ? 31 : ql));
    const K shi = __shfl_sync(kFull, s, qh > 31 ? 31 : (qh < 0 ? 0 : qh));
    const K lo = ql <= 0 ? K(0) : slo;
    const K hi = qh >= static_cast<int>(ns) - 1 ? empty_key<K>() - 1 : shi;
    return window_pass<K>(v, n, k, lo, hi, out, out_rows, lane, res, below, direct);
}

// Order statistics kk and kk-1 of the candidates in `cur`, exact: more
// sampling rounds between the two buffers until at most 64 remain, which
// are gathered and sorted.  A round that fails falls back to a bitwise radix
// search of the candidates.  Shared by every segment length, so out of line.
template <typename K>
__device__ __noinline__ Sel<K> select_candidates(K* cur_buf, K* oth_buf, uint32_t cap_rows, uint32_t t,
                                                 uint32_t nrows, uint32_t n, uint32_t kk, int lane) {
    Ragged<K> cur{cur_buf, t, nrows, lane};
    K* oth = oth_buf;
    Sel<K> r;
    r.have_prev = false;
    r.nfin = 0;
#pragma unroll 1
    for (int round = 0; n > 64 && round < 8; ++round) {
        Ragged<K> nxt;
        uint32_t b2;
        const int st = sample_round<K>(cur, n, kk, oth, cap_rows, lane, nxt, b2, &r);
        if (st == kWinEqual) {
            __syncwarp();
            return r;
        }
        if (st == kWinFail) {
            r.kth = kth_radix<K>(cur, kk);
            __syncwarp();
            return r;
        }
        kk -= b2;
        n = __reduce_add_sync(kFull, nxt.t);
        oth = cur.buf;
        cur = nxt;
    }
    if (n > 64) {
        r.kth = kth_radix<K>(cur, kk);
        __syncwarp();
        return r;
    }
    // gather the ragged candidates into oth[0 .. n)
    uint32_t incl = cur.t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += y;
    }
    const uint32_t first = incl - cur.t;
    for (uint32_t q = 0; q < cur.t; ++q) oth[first + q] = cur.buf[q * 32 + lane];
    __syncwarp();
    r = n <= 32 ? sel32<K>(oth, n, kk, lane) : sel64<K>(oth, n, kk, lane);
    __syncwarp();  // the candidate buffers are reused by the next selection
    return r;
}

// Order statistic k (and usually k-1) of a key source of M keys, exact.
// Short segments are staged and sorted; longer ones go through a first
// sampling round into buffer a (once more, twice as wide, if it misses),
// then select_candidates.
template <typename K, class Src>
__device__ Sel<K> kth_select(const Src& v, uint32_t M, uint32_t k, K* a, K* b, uint32_t cap_rows, int lane) {
    if (M <= 64) {
        const uint32_t nr = v.rows();
#pragma unroll
        for (uint32_t r = 0; r < nr; ++r) {
            const uint32_t i = r * 32 + lane;
            if (i < M) a[i] = v.get(r);
        }
        __syncwarp();
        const Sel<K> r = M <= 32 ? sel32<K>(a, M, k, lane) : sel64<K>(a, M, k, lane);
        __syncwarp();
        return r;
    }
    Ragged<K> cur;
    uint32_t b1;
    Sel<K> r;
    int st = sample_round<K>(v, M, k, a, cap_rows, lane, cur, b1, &r);
    if (st == kWinFail) {  // the samples sit off-centre (a few % of segments): twice as wide a window
        __syncwarp();
        st = sample_round<K>(v, M, k, a, cap_rows, lane, cur, b1, &r, 12);
    }
    if (st == kWinEqual) {
        __syncwarp();
        return r;
    }
    if (st == kWinFail) {
        r.have_prev = false;
        r.nfin = 0;
        r.kth = kth_radix<K>(v, k);
        __syncwarp();
        return r;
    }
    return select_candidates<K>(a, b, cap_rows, cur.t, cur.nrows, __reduce_add_sync(kFull, cur.t), k - b1, lane);
}

// kth_select starting from a predicted window [lo, hi] (the previous
// iteration's): one pass keeps the keys inside it and, if it holds rank k,
// the candidate rounds follow; otherwise the sampled path.  *hit tells which.
template <typename K, class Src>
__device__ Sel<K> kth_select_from(const Src& v, uint32_t M, uint32_t k, K lo, K hi, K* a, K* b, uint32_t cap_rows,
                                  int lane, bool* hit) {
    *hit = false;
    if (M > 64) {
        Ragged<K> cur;
        uint32_t b1;
        Sel<K> r;
        const int st = window_pass<K>(v, M, k, lo, hi, a, cap_rows, lane, cur, b1, &r);
        if (st == kWinEqual) {
            *hit = true;
            __syncwarp();
            return r;
        }
        if (st == kWinCand) {
            *hit = true;
            return select_candidates<K>(a, b, cap_rows, cur.t, cur.nrows, __reduce_add_sync(kFull, cur.t), k - b1,
                                        lane);
        }
        __syncwarp();
    }
    return kth_select<K>(v, M, k, a, b, cap_rows, lane);
}

struct CandBufs {
    void* a;
    void* b;
    uint32_t rows;
};

// A voxel's selection window from the previous iteration, in the units of
// its keys: the order statistic found then (center) and a half-width.
template <typename Real>
struct Pred {
    Real center, half;
};

// Next window: centred on the order statistic just found, wide enough for
// about 24 keys at the density of the final sorted candidates (so that most
// windows end in the 32-key warp sort), and for
// twice the drift since the last prediction (twice the old width after a
// miss).  0: no prediction (sampling next time).
template <typename Real, typename K>
__device__ __forceinline__ Pred<Real> next_window(const Sel<K>& sel, bool used, bool hit, const Pred<Real>& old) {
    const Real c = from_key(sel.kth);
    Real h = 0;
    if (sel.nfin >= 2) h = (from_key(sel.whi) - from_key(sel.wlo)) * Real(12) / static_cast<Real>(sel.nfin);
    if (used) {
        const Real drift = c > old.center ? c - old.center : old.center - c;
        h = h > Real(2) * drift ? h : Real(2) * drift;
        if (!hit) h = h > Real(2) * old.half ? h : Real(2) * old.half;
    }
    if (!(h > Real(0)) || !isfinite(h) || !isfinite(c)) h = 0;
    return Pred<Real>{c, h};
}

// The voxel's new value from its keys (median or percentile mean); val(key)
// is the s_ij a key stands for.  With `win`, the selection starts from the
// voxel's predicted window and the window for the next iteration is stored.
template <typename Real, class Src, class Val>
__device__ Real order_update(const Src& src, uint32_t M, int mode, int pct, const CandBufs& cb, int lane, Val val,
                             Pred<Real>* win) {
    using K = typename KeyOf<Real>::type;
    K* ba = static_cast<K*>(cb.a);
    K* bb = static_cast<K*>(cb.b);
    uint32_t k, jm = 0;
    if (mode == kVoxMedian) {  // src/MutoMLSD.cpp:506-516
        k = M / 2;
    } else {  // mean of the lowest floor(pct/100 M) values, at least 1 (src/MutoMLSD.cpp:500-504)
        jm = u32_cast_x86(pct / 100.0 * M);
        if (jm < 1) jm = 1;
        if (jm > M) jm = M;
        k = jm - 1;
    }
    Sel<K> sel;
    bool used = false, hit = false;
    Pred<Real> old{0, 0};
    if (win && M > 64) {
        old = *win;
        used = old.half > Real(0);
    }
    if (used) {
        sel = kth_select_from<K>(src, M, k, to_key(old.center - old.half), to_key(old.center + old.half), ba, bb,
                                 cb.rows, lane, &hit);
    } else {
        sel = kth_select<K>(src, M, k, ba, bb, cb.rows, lane);
    }
    if (win && M > 64 && lane == 0) *win = next_window<Real, K>(sel, used, hit, old);
    if (mode == kVoxMedian) {
        const Real v1 = val(sel.kth);
        if (M % 2 == 0) {  // s_(M/2-1): from the sorted candidates, else v1 itself or the largest key below it
            Real v0;
            if (sel.have_prev) {
                v0 = val(sel.prev);
            } else {
                uint32_t c = 0;
                K mb = K(0);
                src.each([&](K x) {
                    if (x < sel.kth) {
                        ++c;
                        mb = x > mb ? x : mb;
                    }
                });
                c = __reduce_add_sync(kFull, c);
                mb = warp_max_k(mb);
                v0 = c < M / 2 ? v1 : val(mb);
            }
            return (v1 + v0) * Real(0.25);
        }
        return v1 * Real(0.5);
    }
    const Real t = val(sel.kth);
    Real s = 0;
    uint32_t c = 0;
    src.each([&](K x) {
        if (x < sel.kth) {
            s += val(x);
            ++c;
        }
    });
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
    c = __reduce_add_sync(kFull, c);
    s += static_cast<Real>(jm - c) * t;
    return s / static_cast<Real>(jm) * Real(0.5);
}

template <typename Real>
__device__ __forceinline__ Real pair_g(const typename Vec4<Real>::type& k, Real l, Real t) {
    const Real lt = l * t;
    return k.x * l + k.y * (lt + l * l * Real(0.5)) + k.z * (l * l * l * Real(1.0 / 3.0) + (l + t) * lt);
}

// the voxel's keys held in registers, R per lane
template <typename Real, int R, typename OutT>
__device__ __forceinline__ void voxel_regs(const VoxelPassArgs<Real, OutT>& a, uint32_t j, uint64_t base, uint32_t M,
                                           int lane, const CandBufs& cb) {
    using K = typename KeyOf<Real>::type;
    const Real lam = a.lam[j];
    VoxKeys<Real, R> v;
    v.M = M;
    v.lane = lane;
    const K* kp = a.keys + base;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t e = static_cast<uint32_t>(r * 32 + lane);
        v.key[r] = e < M ? __ldcs(kp + e) : empty_key<K>();
    }
    Real out;
    if (a.mode == kVoxMedian || a.mode == kVoxPercentile) {
        auto val = [lam](K x) {  // s_ij = 2 l + g l^2 is non-decreasing in g
            const Real g = from_key(x);
            return Real(2) * lam + g * lam * lam;
        };
        out = order_update<Real>(v, M, a.mode, a.pct, cb, lane, val,
                                 a.win ? reinterpret_cast<Pred<Real>*>(a.win) + j : nullptr);
    } else {
        Real gs = 0;
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (static_cast<uint32_t>(r * 32 + lane) < M) gs += from_key(v.key[r]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) gs += __shfl_xor_sync(kFull, gs, o);
        if (a.mode == kVoxGradient) {
            if (lane == 0) a.grad[j] = -a.lam64[j] * static_cast<double>(gs);
            return;
        }
        out = lam + lam * lam * gs / (Real(2) * static_cast<Real>(M));
    }
    if (lane == 0) a.out[j] = static_cast<OutT>(out);
}

// segments longer than the register budget, and those of the streamed
// classes: the selection reads the keys where the key pass left them
// (contiguous, through L1) instead of holding them
template <typename Real, typename OutT>
__device__ void voxel_stream(const VoxelPassArgs<Real, OutT>& a, uint32_t j, uint64_t base, uint32_t M, int lane,
                             const CandBufs& cb) {
    using K = typename KeyOf<Real>::type;
    const Real lam = a.lam[j];
    const PtrKeys<K> src{a.keys + base, M, lane};
    Real out;
    if (a.mode == kVoxMedian || a.mode == kVoxPercentile) {
        auto val = [lam](K x) {
            const Real g = from_key(x);
            return Real(2) * lam + g * lam * lam;
        };
        out = order_update<Real>(src, M, a.mode, a.pct, cb, lane, val,
                                 a.win ? reinterpret_cast<Pred<Real>*>(a.win) + j : nullptr);
    } else {
        Real gs = 0;
        src.each([&](K x) { gs += from_key(x); });
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) gs += __shfl_xor_sync(kFull, gs, o);
        if (a.mode == kVoxGradient) {
            if (lane == 0) a.grad[j] = -a.lam64[j] * static_cast<double>(gs);
            return;
        }
        out = lam + lam * lam * gs / (Real(2) * static_cast<Real>(M));
    }
    if (lane == 0) a.out[j] = static_cast<OutT>(out);
}

// The key pass: every pair's order key to_key(g_ij), g_ij = k_i . W(L, T),
// written in voxel-major order for the class kernels.  One thread per pair,
// U pairs of a thread in flight at once.  Persistent blocks, one per SM,
// take the tiles of the column-ordered lists round robin, so the whole GPU
// advances through a window of a few dozen adjacent columns: the muons
// those columns share are gathered while their coefficients are in L2 (and
// within a tile, the vertically adjacent segments of one column go through
// the same SM's L1), whatever the size of the coefficient table.  The lists
// and the keys pass through marked evict-first.
constexpr int kKeyThreads = 1024;
constexpr int kKeyUnroll = 8;
constexpr uint64_t kKeyTile = uint64_t(kKeyThreads) * kKeyUnroll;
template <typename Real>
__global__ void __launch_bounds__(kKeyThreads)
    k_pair_keys(const uint32_t* __restrict__ vm_mu, const typename Vec2<Real>::type* __restrict__ vm_LT,
                const typename Vec4<Real>::type* __restrict__ kvec, typename KeyOf<Real>::type* __restrict__ keys,
                uint64_t P) {
    using R2 = typename Vec2<Real>::type;
    constexpr int U = kKeyUnroll;
    const uint64_t r1 = P;
    for (uint64_t t0 = uint64_t(blockIdx.x) * kKeyTile; t0 < P; t0 += uint64_t(gridDim.x) * kKeyTile) {
        uint32_t mu[U];
        R2 lt[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t i = t0 + uint64_t(u) * kKeyThreads + threadIdx.x;
            if (i < r1) {
                mu[u] = __ldcs(vm_mu + i);
                lt[u] = __ldcs(vm_LT + i);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t i = t0 + uint64_t(u) * kKeyThreads + threadIdx.x;
            if (i < r1) __stcs(keys + i, to_key(pair_g<Real>(ldg4(kvec + mu[u]), lt[u].x, lt[u].y)));
        }
    }
}

// Voxels of class C, one warp per voxel: registers hold vox_class_rows(C)
// keys per lane (the last class, and streamed classes, select from the key
// array).  Each warp also prefetches into L2 the keys of the voxel `ahead`
// places further down the class list, which a warp of the next wave of
// resident blocks will read.  Dynamic shared memory: two candidate buffers
// per warp.
template <typename Real, typename OutT, int C, bool STREAMED>
__global__ void __launch_bounds__(kVoxThreads, vox_min_blocks(C, STREAMED))
    k_em_voxel(VoxelPassArgs<Real, OutT> a, const VoxDesc* __restrict__ desc, uint32_t n, uint32_t ahead) {
    using K = typename KeyOf<Real>::type;
    constexpr int R = vox_class_rows(C);
    constexpr int RB = cand_rows<K, C, STREAMED>();
    if constexpr (R * 32 > static_cast<int>(voxel_register_cap<Real>()) || (STREAMED && !streamable(C))) {
        return;  // no voxel of this precision is put in the class
    } else {
        extern __shared__ __align__(16) unsigned char vox_smem[];
        const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
        K* bufs = reinterpret_cast<K*>(vox_smem);
        const CandBufs cb{bufs + (2 * wib) * RB * 32, bufs + (2 * wib + 1) * RB * 32, static_cast<uint32_t>(RB)};
        const uint64_t w = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
        if (w >= n) return;  // whole warps leave together
        const VoxDesc d = desc[w];
        if (lane == 0 && w + ahead < n) {
            const VoxDesc f = desc[w + ahead];
            if (f.M > 0) prefetch_l2(a.keys + f.start, size_t(f.M) * sizeof(K));
        }
        if (d.M == 0) {  // no muon crossed the voxel, src/MutoMLSD.cpp:494-496
            if (lane == 0) {
                if (a.mode == kVoxGradient) a.grad[d.j] = 0.0;
                else a.out[d.j] = OutT(0);
            }
            return;
        }
        if constexpr (STREAMED || R == 0) voxel_stream<Real, OutT>(a, d.j, d.start, d.M, lane, cb);
        else voxel_regs<Real, R>(a, d.j, d.start, d.M, lane, cb);
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
                // the reference goes on while |(x_n - x_k) / x_k| > eps; the same
                // test without the FP64 division: |x_n - x_k| > eps |x_k| (also
                // for x_k = 0, where the ratio is inf or, at x_n = 0, NaN, and
                // for a NaN step: both stop)
                bool more = true;
                int it = 0;
                while (more) {
                    if (++it > mp.newton_max_iter) {
                        nonconv = true;
                        break;
                    }
                    const double xk2 = xk * xk;
                    const double gx = xk2 * xk + ca * xk2 + cb * xk + cc;
                    const double gp = 3 * xk2 + 2 * ca * xk + cb;
                    const double xn = xk - gx / gp;
                    more = fabs(xn - xk) > mp.eps * fabs(xk);
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
            // chooseBestEstimation / surrogateFunctionValue, :239-281.  The
            // neighbour sum  sum_k w_k q_k (2x - a_k)^2,  a_k = l_j + l_k, is
            // expanded once into  4x^2 S0 - 4x S1 + S2,  so each candidate
            // costs a few operations instead of a pass over the neighbours
            // (the same value up to rounding: only the order of the sums
            // differs from the reference's loop)
            double S0 = 0.0, S1 = 0.0, S2 = 0.0;
            for (int k = 0; k < nn; ++k) {
                const double wq = (k < 6 ? 1.0 : (k < 18 ? w2 : w3)) * q[k];
                const double ak = lj + lm[k];
                S0 += wq;
                S1 += wq * ak;
                S2 += wq * ak * ak;
            }
            const double hb = 0.5 * mp.beta * mp.p;
            double best = 0.0;
            int bi = 0;
            for (int c = 0; c <= nr; ++c) {
                const double xv = c < nr ? roots[c] : ljml;
                double v;
                if (xv < 0) {
                    v = 1.7976931348623157e308;
                } else {
                    v = 0 < xv ? static_cast<double>(Mj) * (log(xv) + ljml / xv) : 0.0;
                    v += hb * ((4.0 * xv * xv) * S0 - (4.0 * xv) * S1 + S2);
                    if (mp.add_object_prior) v += hb * xv * xv * qobj;
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

template <typename Real, typename OutT, int C, bool STREAMED>
int voxel_blocks_per_sm() {
    using K = typename KeyOf<Real>::type;
    constexpr size_t smem = voxel_smem_bytes<K, C, STREAMED>();
    int nb = 0;
    if (cudaFuncSetAttribute(k_em_voxel<Real, OutT, C, STREAMED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem)) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_em_voxel<Real, OutT, C, STREAMED>, kVoxThreads, smem) !=
            cudaSuccess)
        nb = 0;
    return nb > 0 ? nb : 1;
}

template <typename Real, typename OutT, int... C>
void occupancy_all(int* regs, int* streamed, std::integer_sequence<int, C...>) {
    ((regs[C] = voxel_blocks_per_sm<Real, OutT, C, false>()), ...);
    ((streamed[C] = streamable(C) ? voxel_blocks_per_sm<Real, OutT, C, true>() : 0), ...);
}

template <typename Real, typename OutT, int... C>
void launch_all(const VoxelPassArgs<Real, OutT>& a, const VoxDesc* const* lists, const uint32_t* counts,
                const int* resident_blocks, uint32_t streamed, int num_sms, const ClassFan* fan, cudaStream_t s,
                std::integer_sequence<int, C...>) {
    using K = typename KeyOf<Real>::type;
    if (a.P > 0) {  // one persistent block per SM, tiles round robin
        const uint64_t tiles = (a.P + kKeyTile - 1) / kKeyTile;
        const uint64_t want = static_cast<uint64_t>(num_sms > 0 ? num_sms : 1);
        const unsigned nb = static_cast<unsigned>(tiles < want ? tiles : want);
        k_pair_keys<Real><<<nb, kKeyThreads, 0, s>>>(a.vm_mu, a.vm_LT, a.kvec, a.keys, a.P);
        count_launches(1);
    }
    // classes to streams: the heaviest first, each to the least loaded stream
    // (work ~ voxels x a typical segment length of the class)
    cudaStream_t on[kVoxClasses];
    for (int c = 0; c < kVoxClasses; ++c) on[c] = s;
    const int ns = fan ? 1 + std::min(fan->n, ClassFan::kSide) : 1;
    if (ns > 1) {
        double work[kVoxClasses], load[1 + ClassFan::kSide] = {};
        int order[kVoxClasses];
        for (int c = 0; c < kVoxClasses; ++c) {
            const double lo = c == 0 ? 0.0 : vox_class_hi(c - 1);
            const double m = c == kVoxClasses - 1 ? 4.0 * lo : 0.5 * (lo + vox_class_hi(c));
            work[c] = static_cast<double>(counts[c]) * (m + 32.0);
            order[c] = c;
        }
        std::sort(order, order + kVoxClasses, [&](int x, int y) { return work[x] > work[y]; });
        // failures here surface through cudaGetLastError after the pass
        (void)cudaEventRecord(fan->fork, s);
        for (int k = 1; k < ns; ++k) (void)cudaStreamWaitEvent(fan->side[k - 1], fan->fork, 0);
        for (int q = 0; q < kVoxClasses; ++q) {
            const int c = order[q];
            if (counts[c] == 0) continue;
            int best = 0;
            for (int k = 1; k < ns; ++k)
                if (load[k] < load[best]) best = k;
            load[best] += work[c];
            on[c] = best == 0 ? s : fan->side[best - 1];
        }
    }
    auto one = [&](auto cc) {
        constexpr int c = decltype(cc)::value;
        if (counts[c] == 0) return;
        cudaStream_t s = on[c];
        const bool st = streamable(c) && ((streamed >> c) & 1u);
        const unsigned nb = blocks_for(static_cast<uint64_t>(counts[c]) * 32u, kVoxThreads);
        const uint32_t ahead = static_cast<uint32_t>(resident_blocks[st ? kVoxClasses + c : c]) * kWarps;
        if (st)
            k_em_voxel<Real, OutT, c, true>
                <<<nb, kVoxThreads, voxel_smem_bytes<K, c, true>(), s>>>(a, lists[c], counts[c], ahead);
        else
            k_em_voxel<Real, OutT, c, false>
                <<<nb, kVoxThreads, voxel_smem_bytes<K, c, false>(), s>>>(a, lists[c], counts[c], ahead);
        count_launches(1);
    };
    (one(std::integral_constant<int, C>{}), ...);
    if (ns > 1) {
        for (int k = 1; k < ns; ++k) {
            (void)cudaEventRecord(fan->join[k - 1], fan->side[k - 1]);
            (void)cudaStreamWaitEvent(s, fan->join[k - 1], 0);
        }
    }
}

template <typename Real, typename OutT>
void em_voxel_occupancy(int blocks_per_sm[2 * kVoxClasses]) {
    occupancy_all<Real, OutT>(blocks_per_sm, blocks_per_sm + kVoxClasses,
                              std::make_integer_sequence<int, kVoxClasses>{});
}
template void em_voxel_occupancy<float, float>(int*);
template void em_voxel_occupancy<float, double>(int*);
template void em_voxel_occupancy<double, double>(int*);

template <typename Real, typename OutT>
void launch_em_voxel(const VoxelPassArgs<Real, OutT>& a, const VoxDesc* const* lists, const uint32_t* counts,
                     const int* resident_blocks, uint32_t streamed, int num_sms, const ClassFan* fan,
                     cudaStream_t s) {
    launch_all<Real, OutT>(a, lists, counts, resident_blocks, streamed, num_sms, fan, s,
                           std::make_integer_sequence<int, kVoxClasses>{});
}
template void launch_em_voxel<float, float>(const VoxelPassArgs<float, float>&, const VoxDesc* const*,
                                            const uint32_t*, const int*, uint32_t, int, const ClassFan*,
                                            cudaStream_t);
template void launch_em_voxel<float, double>(const VoxelPassArgs<float, double>&, const VoxDesc* const*,
                                             const uint32_t*, const int*, uint32_t, int, const ClassFan*,
                                             cudaStream_t);
template void launch_em_voxel<double, double>(const VoxelPassArgs<double, double>&, const VoxDesc* const*,
                                              const uint32_t*, const int*, uint32_t, int, const ClassFan*,
                                              cudaStream_t);

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
