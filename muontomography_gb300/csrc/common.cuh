// Shared device helpers and the kernel-launch interface between the handle
// (handle.cu) and the kernel files (setup.cu, em_muon.cu, em_voxel.cu, poca.cu,
// adjoint.cu, scan.cu, gen.cu).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include "geometry.cuh"

namespace muto {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------
// Precision traits: Real is the storage/accumulation type of the per-pair
// data (float in the mixed form, double in the plain FP64 form).
// ---------------------------------------------------------------------------
template <typename Real> struct Vec4;
template <> struct Vec4<float> { using type = float4; };
template <> struct Vec4<double> { using type = double4; };
template <typename Real> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };

// Order-preserving integer keys for the per-voxel selection.
__device__ __forceinline__ uint32_t to_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float from_key(uint32_t k) {
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}
__device__ __forceinline__ unsigned long long to_key(double f) {
    const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(f));
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_key(unsigned long long k) {
    const unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double(static_cast<long long>(u));
}
// one bulk prefetch of [p, p + bytes) into L2, widened to 16-byte bounds
// (callers keep the widened range inside their arrays' padding)
__device__ __forceinline__ void prefetch_l2(const void* p, size_t bytes) {
    const uintptr_t a0 = reinterpret_cast<uintptr_t>(p) & ~uintptr_t(15);
    const uintptr_t a1 = (reinterpret_cast<uintptr_t>(p) + bytes + 15) & ~uintptr_t(15);
    if (a1 > a0)
        asm volatile(
            "{\n\t.reg .u64 ga;\n\tcvta.to.global.u64 ga, %0;\n\tcp.async.bulk.prefetch.L2.global [ga], %1;\n\t}"
            ::"l"(static_cast<unsigned long long>(a0)), "r"(static_cast<uint32_t>(a1 - a0))
            : "memory");
}

template <typename Real> struct KeyOf;
template <> struct KeyOf<float> { using type = uint32_t; static constexpr int bits = 32; };
template <> struct KeyOf<double> { using type = unsigned long long; static constexpr int bits = 64; };

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// Warp-aggregated increment of a global counter by the number of lanes with pred.
__device__ __forceinline__ void warp_count(unsigned long long* ctr, bool pred) {
    const unsigned b = __ballot_sync(__activemask(), pred);
    const unsigned lead = __ffs(__activemask()) - 1;
    if ((threadIdx.x & 31) == lead && b) atomicAdd(ctr, static_cast<unsigned long long>(__popc(b)));
}

// Device-side counters shared by all kernels of a handle.
struct Counters {
    unsigned long long singular;
    unsigned long long nonconverged;
    unsigned long long bounds;
    unsigned long long overflow;
    unsigned long long not_parallel;
    unsigned long long in_grid;
    unsigned long long iteration;   // device iteration index (graph replays)
    unsigned long long timeouts;    // bounded waits that gave up (never expected)
    double cost_sum;                // cost of the current iteration
    double cost_last;               // mean cost of the last finished iteration
    double cost_prev;               // mean cost of the one before
    unsigned long long over_bound;  // paths longer than their set-up bound (then counted exactly)
};

// ---------------------------------------------------------------------------
// Kernel launch wrappers (all asynchronous on `s`)
// ---------------------------------------------------------------------------
// scan.cu: out[i] = sum_{k<i} in[k] (exclusive), out has n+1 entries
// (out[n] = total).  scratch must hold scan_scratch_bytes(n) bytes.
size_t scan_scratch_bytes(uint64_t n);
void scan_u32_to_u64(const uint32_t* in, uint64_t* out, uint64_t n, void* scratch, cudaStream_t s);
// a[i] += add for i < n
void launch_add_u64(uint64_t* a, uint64_t n, uint64_t add, cudaStream_t s);

// setup.cu
void launch_keep_flags(const muto_ray* rays, uint64_t n_total, muto_grid g, double eps, uint32_t* flags,
                       cudaStream_t s);
void launch_compact(const uint32_t* flags, const uint64_t* pos, uint64_t n, uint32_t* kept, cudaStream_t s);
template <typename Real>
void launch_muon_info(const muto_ray* rays, const uint32_t* kept, uint64_t n, muto_grid g, double eps, int has_energy,
                      typename Vec4<Real>::type* sd, Real* pr2, double* scat, double* pr_out, cudaStream_t s);
void launch_path_count(const muto_ray* rays, const uint32_t* kept, const double* scat, uint64_t n, muto_grid g,
                       int straight, uint32_t* counts, Counters* ctr, cudaStream_t s);
template <typename Real>
void launch_path_fill(const muto_ray* rays, const uint32_t* kept, const double* scat, const uint64_t* off, uint64_t n,
                      muto_grid g, int straight, uint32_t* vidx, double* l64, Real* L, Real* T, cudaStream_t s);
// Single-walk set-up: an upper bound on every kept muon's merged path
// (index spans of the pieces on the grid, FP32, with a margin of 2 per axis
// and end), the walk into slots sized by those bounds with the actual
// counts, and the compaction to slots sized by the counts.  A path longer
// than its bound (never expected) is counted in ctr->over_bound and the
// caller falls back to the exact count walk.  The bounded slots of muon i
// are [boff[i], boff[i+1]) - slot_base, so a chunk of muons can be walked
// into scratch sized for the chunk alone.
void launch_path_bound(const muto_ray* rays, const uint32_t* kept, const double* scat, uint64_t n, muto_grid g,
                       int straight, uint32_t* bounds, cudaStream_t s);
template <typename Real>
void launch_path_fill_bounded(const muto_ray* rays, const uint32_t* kept, const double* scat, const uint64_t* boff,
                              uint64_t slot_base, uint64_t n, muto_grid g, int straight, uint32_t* vidx, double* l64,
                              Real* L, Real* T, uint32_t* counts, Counters* ctr, cudaStream_t s);
template <typename Real>
void launch_path_compact(const uint64_t* boff, uint64_t slot_base, const uint64_t* off, uint64_t n,
                         const uint32_t* vidx_b, const Real* L_b, const Real* T_b, uint32_t* vidx, Real* L, Real* T,
                         cudaStream_t s);
// scan-local voxel indices j < V_scan become voff + j; others become 0xffffffff
void launch_offset_voxels(uint32_t* vidx, uint64_t n, uint32_t v_scan, uint32_t voff, cudaStream_t s);
void launch_voxel_hist(const uint32_t* vidx, uint64_t P, uint32_t V, uint32_t* mult, Counters* ctr, cudaStream_t s);
// voxel-major copy of the pair lists: (muon, L, T) at start[j] + rank within voxel j
// (rec: P staging records, free after the call's work is done)
// kslot (optional): vm_mu holds kslot[muon] instead of the muon's index
template <typename Real>
void launch_build_voxel_major(const uint64_t* off, uint64_t n, const uint32_t* vidx, const Real* L, const Real* T,
                              uint32_t V, const uint64_t* start, uint32_t* cursor, uint64_t P,
                              typename Vec4<Real>::type* rec, uint32_t* vm_mu, typename Vec2<Real>::type* vm_LT,
                              const uint32_t* kslot, cudaStream_t s);
// Rows of the per-muon coefficient table in column order of the muons' PoCA
// points (x, y cell of the grid, clamped): the muons crossing a column of
// voxels then sit in a compact block of rows, so the key pass's gathers for
// a run of columns touch a slice of the table that stays in L2 even when the
// whole table does not.  cell: n scratch; hist, cursor: nx*ny + 1 scratch
// (zeroed here); cstart: nx*ny + 1; scan_scratch as for scan_u32_to_u64 of
// nx*ny
void launch_muon_slots(const double* scat, uint64_t n, muto_grid g, uint32_t* cell, uint32_t* hist,
                       uint64_t* cstart, uint32_t* cursor, void* scan_scratch, uint32_t* kslot, cudaStream_t s);
void launch_siddon_batch(muto_grid g, const double* p1, const double* p2, uint64_t n, uint32_t cap, uint32_t* xyz,
                         double* len, uint32_t* counts, cudaStream_t s);

// poca.cu
struct PocaArgs {
    const muto_ray* rays;
    uint64_t n;
    muto_grid g;
    double eps, mag;
    int has_energy, straight, length_weighted;
    double* img;        // PoCA: the summed values (null for PoCut)
    double* weight;
    uint32_t* walk;                  // n slots: the kept rays, listed by the first kernel for the walks
    unsigned long long* walk_count;  // their number (device)
    uint32_t* walk_len;              // n slots (or null): a bound on each listed ray's walk
    uint32_t* walk_order;            // n slots (or null): the list by decreasing bound, walked in that order
    uint32_t* order_work;            // 512 words of scratch for the ordering
    long long* assign;  // 3 per ray, optional
    Counters* ctr;
    uint32_t* vox;      // PoCut: per ray its voxel, 0xffffffff when rejected (null for PoCA)
    double* value;      // PoCut: per ray its value (angle^2, times p^2 with momentum)
};
void launch_poca(const PocaArgs& a, cudaStream_t s);
// order[0..n) = the entries 0..n-1 by decreasing len[] (buckets of 4; any
// order inside a bucket); n is *count when count is given (at most n
// entries), else n; work: 512 uint32 of scratch
void launch_length_order(const uint32_t* len, const unsigned long long* count, uint64_t n, uint32_t* order,
                         uint32_t* work, cudaStream_t s);
void launch_poca_normalize(double* img, const double* weight, uint64_t V, double eps, cudaStream_t s);
// slr.cu: straight-line reconstruction (src/MutoSLR.cpp:47-103) and the
// iterative form's passes (src/MutoSLRIter.cpp:15-83)
struct SlrArgs {
    const muto_ray* rays;
    uint64_t n;
    muto_grid g;
    double mag;
    int has_energy, length_weighted;
    double* img;     // summed values
    double* weight;  // summed weights
};
// the first pass: every ray at once (atomics)
void launch_slr(const SlrArgs& a, cudaStream_t s);
// the walked straight lines: off == null: counts[i] = voxels of ray i; else
// ray i's voxels (x + nx (y + ny z)) and lengths at vox/len + off[i]
void launch_slr_paths(const SlrArgs& a, const uint64_t* off, uint32_t* counts, uint32_t* vox, double* len,
                      cudaStream_t s);
// the later, in-place passes over the walked lines: per pair its voxel, its
// weight increment and its image increment before the path's scaling; per
// muon ein^2
struct SlrPass {
    const uint64_t* off;
    const uint32_t* vox;
    const double* len;
    double* iv0;
    double* winc;
    double* e2;
};
void launch_slr_pair_terms(const SlrArgs& a, const SlrPass& p, cudaStream_t s);
// one later pass, muon after muon
void launch_slr_iter_pass(const SlrArgs& a, const SlrPass& p, cudaStream_t s);
// the same pairs in level order: muon q of the level order (order[q]) has
// its pairs at fo[q] .. fo[q+1]
struct SlrFlat {
    const uint64_t* fo;
    uint32_t* vox;
    double* iv0;
    double* winc;
    double* e2;
};
void launch_slr_flatten(const SlrPass& p, const uint32_t* order, uint64_t nt, const SlrFlat& f, cudaStream_t s);
// the same pass level by level: level l's muons are q = lstart[l] ..
// lstart[l+1] of the level order; the image and weight sums are kept in
// shared memory when 2 V doubles fit in smem_optin bytes
void launch_slr_iter_levels(const SlrArgs& a, const SlrFlat& f, const uint32_t* lstart, uint32_t levels,
                            size_t smem_optin, cudaStream_t s);

// PoCut's per-voxel step (src/MutoPoCut.cpp:113-118), after launch_poca:
// the kept values grouped by voxel (counts, then offsets, then a scatter of
// order keys into the voxels' segments), sorted per voxel and the lowest
// floor(M cut) summed in ascending order.
void launch_pocut_hist(const uint32_t* vox, uint64_t n, uint32_t* counts, cudaStream_t s);
void launch_pocut_scatter(const uint32_t* vox, const double* value, uint64_t n, const uint64_t* off,
                          uint32_t* cursor, unsigned long long* keys, cudaStream_t s);
// voxels of no value: img = weight < eps ? 0 : 0 / weight
void launch_pocut_empty(const uint32_t* counts, const double* weight, double* img, uint64_t V, double eps,
                        cudaStream_t s);
// voxels of at most 32 values, one warp each (list: voxel indices)
void launch_pocut_small(const uint32_t* list, uint32_t n, const uint64_t* off, const uint32_t* counts,
                        const unsigned long long* keys, const double* weight, double* img, double eps, double cut,
                        cudaStream_t s);
// voxels of more, one block each: sorted in shared memory up to kPocutSmemKeys
// values, else in scratch (scratch_off[i]: first of next_pow2(M) slots)
constexpr uint32_t kPocutSmemKeys = 4096;
void launch_pocut_big(const uint32_t* list, uint32_t n, const uint64_t* off, const uint32_t* counts,
                      const unsigned long long* keys, const uint64_t* scratch_off, unsigned long long* scratch,
                      const double* weight, double* img, double eps, double cut, cudaStream_t s);

// em_muon.cu: the muon pass (per-muon coefficients k)
template <typename Real>
struct MuonPassArgs {
    const uint64_t* off;                      // N+1 pair offsets (+ padding)
    const uint32_t* tile_mb;                  // ntiles+1 first muon of each tile
    uint32_t ntiles;
    const uint32_t* vidx;                     // P (+ padding) voxel of each pair
    const Real* L;                            // P (+ padding)
    const Real* T;                            // P (+ padding)
    const typename Vec4<Real>::type* sd;      // N: Sx, Dx, Sy, Dy
    const Real* pr2;                          // N (+ padding)
    const Real* lam;                          // V: lambda gathered by the muons
    typename Vec4<Real>::type* kout;          // N: (k0, k1, k2, 0)
    const uint32_t* kslot;                    // N: the row of kout each muon writes (null: its own index)
    uint32_t V;
    double E00, E01, E11;
    int compute_cost;
    Counters* ctr;
};
template <typename Real>
void launch_em_muon(const MuonPassArgs<Real>& a, int tile_pairs, int tile_muons, int blocks, int group,
                    cudaStream_t s);
template <typename Real>
size_t em_muon_smem_bytes(int tile_pairs, int tile_muons);
// sets the dynamic shared-memory limit of every k_em_muon variant (call outside graph capture)
template <typename Real>
cudaError_t em_muon_configure(int tile_pairs, int tile_muons);
// resident CTAs per SM (persistent grid = this x SM count)
template <typename Real>
int em_muon_blocks(int tile_pairs, int tile_muons, int group);
// warp-batched variant of the muon pass (no shared memory)
template <typename Real>
void launch_em_muon_warp(const MuonPassArgs<Real>& a, uint32_t n_muons, int blocks, int group, cudaStream_t s);
template <typename Real>
int em_muon_warp_blocks(int group);

// em_voxel.cu: the voxel pass
enum VoxelMode { kVoxMedian = 0, kVoxPercentile = 1, kVoxMean = 2, kVoxGradient = 3 };
template <typename Real, typename OutT>
struct VoxelPassArgs {
    const uint64_t* start;                    // V+1 segment starts of the voxel-major lists
    const uint32_t* mult;                     // V pairs per voxel
    const uint32_t* vm_mu;                    // P muon of each voxel-major pair
    const typename Vec2<Real>::type* vm_LT;   // P (L, T) of each voxel-major pair
    const typename Vec4<Real>::type* kvec;    // N per-muon coefficients
    const Real* lam;                          // V lambda of the iteration
    uint32_t V;
    int mode;                                 // VoxelMode
    int pct;                                  // mean_percentile
    OutT* out;                                // V new value (median / percentile / mean)
    double* grad;                             // V gradient (kVoxGradient)
    const double* lam64;                      // V lambda in FP64 (kVoxGradient)
    typename KeyOf<Real>::type* keys;         // P order keys of g_ij, voxel-major (the key pass writes them)
    uint64_t P;                               // pairs in the voxel-major lists
    Real* win;                                // 2V selection window per voxel (center, half), or NULL
};
// segments up to this many pairs are selected from registers
template <typename Real>
__host__ __device__ constexpr uint32_t voxel_register_cap() { return sizeof(Real) == 4 ? 1536u : 768u; }
// Voxel classes by segment length, one voxel-pass kernel each: class c holds
// the voxels with vox_class_lo(c) < M <= vox_class_hi(c) and keeps
// vox_class_rows(c) keys per lane in registers; the last class (rows 0)
// selects from the scratch array.  Voxels without pairs go with class 0.
constexpr int kVoxClasses = 11;
__host__ __device__ constexpr uint32_t vox_class_hi(int c) {
    return c == 0 ? 32u : c == 1 ? 64u : c == 2 ? 128u : c == 3 ? 192u : c == 4 ? 256u : c == 5 ? 384u
         : c == 6 ? 512u : c == 7 ? 768u : c == 8 ? 1024u : c == 9 ? 1536u : 0xffffffffu;
}
__host__ __device__ constexpr int vox_class_rows(int c) { return c < kVoxClasses - 1 ? int(vox_class_hi(c) / 32u) : 0; }
template <typename Real>
__host__ __device__ constexpr int vox_class_of(uint32_t M) {
    int c = 0;
    while (c < kVoxClasses - 1 && M > vox_class_hi(c)) ++c;
    if (M > voxel_register_cap<Real>()) c = kVoxClasses - 1;
    return c;
}
// one voxel of a class list: its index, pair count and first voxel-major pair
struct alignas(16) VoxDesc {
    uint32_t j, M;
    unsigned long long start;
};
// Side streams the class kernels of a voxel pass are spread over (they touch
// disjoint voxels), with the events that fork them from the launching stream
// and join them back; inside stream capture they become parallel branches.
struct ClassFan {
    static constexpr int kSide = 3;
    cudaStream_t side[kSide];
    cudaEvent_t fork, join[kSide];
    int n = 0;  // side streams in use (0: every class on the launching stream)
};
// The key pass over a.P pairs, then the class kernels.  lists[c], counts[c]:
// the descriptors of class c; resident_blocks[c] and [kVoxClasses + c]:
// blocks of class c's register and streamed kernels resident on the whole
// GPU at once; bit c of `streamed`: class c (M > 256 only) selects from the
// key array instead of holding its keys in registers; num_sms sizes the key
// pass's grid.
template <typename Real, typename OutT>
void launch_em_voxel(const VoxelPassArgs<Real, OutT>& a, const VoxDesc* const* lists, const uint32_t* counts,
                     const int* resident_blocks, uint32_t streamed, int num_sms, const ClassFan* fan,
                     cudaStream_t s);
// Bricked voxel order for the muon passes' lambda gathers and the per-voxel
// sums: 4x4x4 bricks of 64 consecutive entries, each brick made of eight
// 2x2x2 micro-blocks of 8 entries (one 32-byte sector in FP32), so the
// consecutive voxels of a muon's path, which differ by one step on one
// axis, fall into the same sector about half the time instead of lying a
// grid row or plane apart.
struct BrickDims {
    uint32_t nx, ny, nz, nbx, nby, nbz;
};
__host__ __device__ inline BrickDims brick_dims(const muto_grid& g) {
    return BrickDims{g.nx, g.ny, g.nz, (g.nx + 3) / 4, (g.ny + 3) / 4, (g.nz + 3) / 4};
}
__host__ __device__ inline uint64_t brick_volume(const BrickDims& b) {
    return static_cast<uint64_t>(b.nbx) * b.nby * b.nbz * 64;
}
__host__ __device__ inline uint32_t brick_xyz(uint32_t x, uint32_t y, uint32_t z, const BrickDims& b) {
    const uint32_t in = (((z >> 1) & 1u) << 5) | (((y >> 1) & 1u) << 4) | (((x >> 1) & 1u) << 3) | ((z & 1u) << 2) |
                        ((y & 1u) << 1) | (x & 1u);
    return (((z >> 2) * b.nby + (y >> 2)) * b.nbx + (x >> 2)) * 64u + in;
}
__host__ __device__ inline uint32_t brick_of(uint32_t j, const BrickDims& b) {
    const uint32_t x = j % b.nx, t = j / b.nx, y = t % b.ny, z = t / b.ny;
    return brick_xyz(x, y, z, b);
}
__host__ __device__ inline uint32_t unbrick(uint32_t jb, const BrickDims& b) {
    const uint32_t in = jb & 63u, blk = jb >> 6;
    const uint32_t bx = blk % b.nbx, t = blk / b.nbx, by = t % b.nby, bz = t / b.nby;
    const uint32_t x = bx * 4 + (((in >> 3) & 1u) << 1) + (in & 1u);
    const uint32_t y = by * 4 + (((in >> 4) & 1u) << 1) + ((in >> 1) & 1u);
    const uint32_t z = bz * 4 + (((in >> 5) & 1u) << 1) + ((in >> 2) & 1u);
    return x + b.nx * (y + b.ny * z);
}
// voxel indices to bricked ones in place (indices >= V are left alone)
void launch_brick_indices(uint32_t* vidx, uint64_t n, BrickDims b, uint32_t V, cudaStream_t s);
// bricked indices back to voxel indices
void launch_unbrick_indices(const uint32_t* in, uint32_t* out, uint64_t n, BrickDims b, cudaStream_t s);
// lambda (voxel order, V) to its bricked copy
template <typename Real>
void launch_brick_lambda(const Real* lam, uint32_t V, BrickDims b, Real* lam_b, cudaStream_t s);

// em_fused.cu: the mean-update iteration over the muon-major lists (or over
// paths walked again every iteration) with per-voxel sums G_j = sum_i g_ij
// accumulated by reductions to global memory
template <typename Real>
struct FusedArgs {
    const uint64_t* off;                      // N+1 pair offsets (stored lists)
    const uint32_t* vidx;                     // voxel of each pair (bricked when lam/G are)
    const Real* L;
    const Real* T;
    const typename Vec4<Real>::type* sd;      // N: Sx, Dx, Sy, Dy
    const Real* pr2;                          // N
    const Real* lam;                          // lambda gathered by the muons (bricked copy when brick)
    Real* G;                                  // per-voxel sums of g_ij, zero on entry
    uint32_t V;                               // entries of lam and G
    uint32_t N;                               // kept muons
    double E00, E01, E11;
    int compute_cost;
    int prefetch;                             // stored lists: prefetch every CTA's next batch into L2
    Counters* ctr;
    // recompute form: the walk's inputs
    const muto_ray* rays;
    const uint32_t* kept;
    const double* scat;                       // 3N PoCA points
    const double* ltot;                       // N in-grid path lengths (-1: dropped walk)
    const uint32_t* order;                    // N (or null): the muons in the order their walks run
    DevGrid g;
    int straight;
    BrickDims bdims;
    int brick;
};
// stored-list variants: lanes per muon and pairs held in registers per muon
constexpr int kFusedVariants = 7;
constexpr int kFusedStaged = 6;  // the variant whose batches are staged in shared memory
int fused_variant_group(int v);
int fused_variant_held(int v);
template <typename Real>
int em_fused_blocks(int variant);  // resident CTAs per SM
template <typename Real>
void launch_em_fused(const FusedArgs<Real>& a, int variant, int blocks, cudaStream_t s);
template <typename Real>
void launch_em_fused_walk(const FusedArgs<Real>& a, int num_sms, cudaStream_t s);
// split form: g_ij of every pair from the muon pass's coefficients kvec, added to G
template <typename Real>
int em_scatter_blocks(int group, int depth);  // resident 256-thread CTAs per SM (depth: pairs in flight per lane)
template <typename Real>
void launch_em_scatter(const FusedArgs<Real>& a, const typename Vec4<Real>::type* kvec, int group, int depth,
                       int blocks, cudaStream_t s);
// recompute set-up: in-grid length per kept muon and pairs per voxel (mult zeroed by the caller)
void launch_path_stats(const muto_ray* rays, const uint32_t* kept, const double* scat, uint64_t n, muto_grid g,
                       int straight, double* ltot, uint32_t* mult, Counters* ctr, cudaStream_t s);
// out_j = M_j ? l_j + l_j^2 G_j / (2 M_j) : 0, or grad_j = M_j ? -lam64_j G_j : 0 when grad is
// given; G (bricked by `brick` when given) is cleared
template <typename Real, typename OutT>
void launch_mean_update(const Real* lam, Real* G, const uint32_t* mult, uint32_t V, const BrickDims* brick, OutT* out,
                        double* grad, const double* lam64, cudaStream_t s);

// descriptors of all voxels partitioned by class (within a class in column
// order of column_order's grid when it covers the V voxels, else in index
// order): counts needs kVoxClasses * voxel_class_blocks(V) entries, first one
// more (exclusive scan; class c starts at first[c * blocks]); scan_scratch
// as for scan_u32_to_u64 of that length
uint32_t voxel_class_blocks(uint64_t V);
// start (V+1) of each voxel's voxel-major segment from the pair counts:
// segments laid out in the column order of column_order's grid when it
// covers the V voxels (mcol: V, scol: V+1 entries of scratch), else in index
// order; scan_scratch as for scan_u32_to_u64 of V
void launch_segment_starts(const uint32_t* mult, uint32_t V, const muto_grid* column_order, uint32_t* mcol,
                           uint64_t* scol, void* scan_scratch, uint64_t* start, cudaStream_t s);
template <typename Real>
void launch_voxel_classes(const uint32_t* mult, const uint64_t* start, uint32_t V, const muto_grid* column_order,
                          uint32_t* counts, uint64_t* first, void* scan_scratch, VoxDesc* out, cudaStream_t s);
// classes that hold segments of more than `pairs` pairs: the streamed mask
__host__ __device__ constexpr uint32_t vox_streamed_mask(uint32_t pairs) {
    uint32_t m = 0;
    for (int c = 5; c < kVoxClasses; ++c)
        if (vox_class_hi(c - 1) >= pairs) m |= 1u << c;
    return m;
}
// resident blocks per SM of the class kernels (also sets their shared-memory
// limit: call before any launch, outside stream capture)
template <typename Real, typename OutT>
void em_voxel_occupancy(int blocks_per_sm[2 * kVoxClasses]);
void launch_finalize_cost(Counters* ctr, double n_muons, double* hist, uint32_t hist_cap, cudaStream_t s);

struct MapParams {
    double beta, p, delta, eps;
    int all_neighbours, add_object_prior, newton_max_iter;
};
template <typename LamT>
void launch_map_voxel(const LamT* last, double* ml_inout, const uint32_t* mult, DevGrid g, MapParams mp,
                      Counters* ctr, cudaStream_t s);
template <typename LamT>
void launch_copy_to(const double* in, LamT* out, uint64_t n, cudaStream_t s);

// adjoint.cu
template <typename Real>
void launch_exp_lambda(const double* loglam, const uint32_t* mult, uint32_t V, Real* lam, cudaStream_t s);
// adds d prior / d log(lambda) to grad and the prior's value to *value;
// dl_scratch: V doubles, zero on entry and on return
void launch_prior(const double* lam64, const uint32_t* mult, DevGrid g, MapParams mp, double* dl_scratch, double* grad,
                  double* value, cudaStream_t s);

// gen.cu
void launch_generate(const muto_grid& g, const double* lambda, const muto_gen_params& p, uint64_t first, uint64_t n,
                     muto_ray* out, cudaStream_t s);

// fit.cu: the detector layers of a batched line fit (nz <= 64)
struct FitLayers {
    double z[64];
    int nz, n_middle;
};
// rec: n records of 2*nz+2 values (float when precision is 4, else double);
// all, keep: n tracks and flags; pos: n+1 slots; scan_scratch as for
// scan_u32_to_u64 of n.  out receives the kept tracks in record order and
// pos[n] their number.
void launch_fit_records(const void* rec, int precision, uint64_t n, const FitLayers& zl, muto_ray* all,
                        uint32_t* keep, uint64_t* pos, void* scan_scratch, muto_ray* out, cudaStream_t s);

// Kernel launches issued by the library (all handles), for the launch count.
void count_launches(unsigned long long n);
unsigned long long launches_so_far();

}  // namespace muto
