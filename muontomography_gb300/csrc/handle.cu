// C ABI of the reconstruction library (include/muto_gb300.h): handle state,
// configuration, device memory, the setup pipeline and the EM / MAP
// iteration, captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/muto_gb300.h"
#include "slr_levels.h"
#include "common.cuh"
#include "gen.h"
#include "json.hpp"

namespace muto {

static std::atomic<unsigned long long> g_launches{0};
void count_launches(unsigned long long n) { g_launches += n; }
unsigned long long launches_so_far() { return g_launches.load(); }

namespace {

constexpr uint64_t kPad = 8;

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(call)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            throw Error(e_ == cudaErrorMemoryAllocation ? MUTO_ERR_NOMEM : MUTO_ERR_CUDA,              \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                           \
    } while (0)

// Device memory comes from one pool per device that keeps freed blocks
// mapped, so the next handle (the next scan) reuses them instead of paying
// for new mappings; the pool grows to the largest working set seen.  Frees
// keep cudaFree's ordering: they wait for the device to be idle first.
cudaMemPool_t device_pool(int dev) {
    constexpr int kMaxDevices = 64;
    static std::once_flag once[kMaxDevices];
    static cudaMemPool_t pools[kMaxDevices];
    static cudaError_t errs[kMaxDevices];
    if (dev < 0 || dev >= kMaxDevices) throw Error(MUTO_ERR_CUDA, "device ordinal out of range");
    std::call_once(once[dev], [dev] {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        errs[dev] = cudaMemPoolCreate(&pools[dev], &props);
        if (errs[dev] == cudaSuccess) {
            unsigned long long keep = ~0ull;
            errs[dev] = cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
        }
    });
    CK(errs[dev]);
    return pools[dev];
}

// Owned device allocation.
class DevMem {
public:
    DevMem() = default;
    DevMem(const DevMem&) = delete;
    DevMem& operator=(const DevMem&) = delete;
    ~DevMem() { release(); }
    void alloc(size_t bytes, std::atomic<uint64_t>* tally) {
        release();
        if (bytes == 0) bytes = 16;
        int dev = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaMallocFromPoolAsync(&p_, bytes, device_pool(dev), 0));
        CK(cudaStreamSynchronize(0));  // usable from any stream once this returns
        bytes_ = bytes;
        tally_ = tally;
        if (tally_) *tally_ += bytes_;
    }
    void release() {
        if (p_) {
            cudaDeviceSynchronize();
            cudaFreeAsync(p_, 0);
            if (tally_) *tally_ -= bytes_;
        }
        p_ = nullptr;
        bytes_ = 0;
    }
    template <typename T> T* as() const { return static_cast<T*>(p_); }
    size_t bytes() const { return bytes_; }
    bool empty() const { return p_ == nullptr; }

private:
    void* p_ = nullptr;
    size_t bytes_ = 0;
    std::atomic<uint64_t>* tally_ = nullptr;
};

// A non-blocking stream owned by one call, destroyed on every way out.
struct OwnedStream {
    cudaStream_t s = nullptr;
    OwnedStream() { CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
    ~OwnedStream() {
        if (s) cudaStreamDestroy(s);
    }
    OwnedStream(const OwnedStream&) = delete;
    OwnedStream& operator=(const OwnedStream&) = delete;
};

enum Method { kPoca, kMlsd, kMap };

struct Params {
    muto_grid grid{};
    // MLSD / MAP keys, src/MutoMLSD.cpp:47-84 and src/MutoMAP.cpp:12-19
    bool update_with_mean = false;
    int mean_percentile = 100;
    bool straight_line = false, has_energy = false, early_stop = false, log_results = false;
    int64_t total_num_rays = 0;
    int num_iteration = 10;
    int initialize_method = 0;
    double initialize_value = 1.0e-7;
    std::string initial_image_file;
    double error_xy = 1.0, error_dz_outer = 1000.0, error_dz_inner = 1000.0;
    double angle_unit_mag = 1.0, eps = 1.0e-8;
    double beta = 1.0, p = 1.0, delta = 0.1;
    bool add_object_prior = false, all_neighbours = false;
    // PoCA, src/MutoPoCA.cpp:24-47; PoCut, src/MutoPoCut.cpp:12-15
    bool length_weighted = false;
    bool pocut = false;          // PoCut: the PoCA handle keeps a percentile of the values per voxel
    double cut_percentile = 1.0;
    // SLR, src/MutoSLR.cpp:21-45; SLRIter, src/MutoSLRIter.cpp:9-11
    int slr = 0;                 // 1 straight-line reconstruction, 2 its iterative form
    int slr_iterations = 1;
    bool slr_sequential = false;  // later passes muon after muon instead of level by level
    // this library
    int precision = 0;  // 0 mixed, 1 fp64
    bool use_graph = true;
    bool seed_set = false;
    uint64_t random_seed = 0;
    int compute_cost = -1;
    int newton_max_iter = 200;
    int tile_pairs = 0;
    int muon_pass = 0;  // 0 autotune, 1 tile (TMA), 2 warp-batched
    long long voxel_stream_above = -1;  // segments longer than this are selected without registers (-1: none, -2: tuned)
    int muon_layout = 0;  // coefficient rows: 0 auto (column order when the table outgrows L2), 1 columns, 2 index
    int path_lists = 0;   // 0 auto, 1 voxel-major copy, 2 muon-major lists only, 3 recomputed every iteration
    long long setup_chunk_pairs = 0;  // bounded pairs per set-up chunk (0: sized from free device memory)
    int fused_variant = -1;           // stored-list fused pass: -1 autotune, else the variant index
    bool fused_prefetch = false;      // stored-list fused pass: L2 prefetch of each CTA's next batch
};

// how an EM / MAP handle keeps its pair lists
enum Lists { kListsVoxelMajor = 1, kListsMuonMajor = 2, kListsRecompute = 3 };

// variant of the one-shot (PoCA) handle: 0 PoCA, 1 PoCut, 2 SLR, 3 SLRIter
Params parse_params(Method m, const std::string& text, int variant = 0) {
    Params P;
    P.grid = muto_grid{100, 100, 100, 0, 0.0, 0.0, 0.0, 10.0, 10.0, 10.0};
    json cfg;
    try {
        cfg = text.empty() ? json::parse("{}") : json::parse(text);
    } catch (const std::exception& e) {
        throw Error(MUTO_ERR_CONFIG, std::string("config JSON: ") + e.what());
    }
    if (!cfg.is_object()) throw Error(MUTO_ERR_CONFIG, "config must be a JSON object");
    try {
        if (cfg.contains("grid")) {  // a missing "grid" keeps the defaults (src/MutoMLSD.cpp:60)
            const json& g = cfg.at("grid");
            const int64_t nx = g.value("nx", int64_t(100)), ny = g.value("ny", int64_t(100)),
                          nz = g.value("nz", int64_t(100));
            if (nx <= 0 || ny <= 0 || nz <= 0 || nx * ny * nz > 0xffffffffLL)
                throw Error(MUTO_ERR_CONFIG, "grid nx, ny, nz must be positive and nx*ny*nz < 2^32");
            P.grid.nx = static_cast<uint32_t>(nx);
            P.grid.ny = static_cast<uint32_t>(ny);
            P.grid.nz = static_cast<uint32_t>(nz);
            P.grid.x_min = g.value("x_min", 0.0);
            P.grid.y_min = g.value("y_min", 0.0);
            P.grid.z_min = g.value("z_min", 0.0);
            P.grid.dx = g.value("dx", 10.0);
            P.grid.dy = g.value("dy", 10.0);
            P.grid.dz = g.value("dz", 10.0);
            if (!(P.grid.dx > 0 && P.grid.dy > 0 && P.grid.dz > 0))
                throw Error(MUTO_ERR_CONFIG, "grid dx, dy, dz must be positive");
        }
        P.straight_line = cfg.value("straight_line", false);
        P.has_energy = cfg.value("has_energy", false);
        P.log_results = cfg.value("log_results", false);
        P.total_num_rays = cfg.value("total_num_rays", int64_t(0));
        P.angle_unit_mag = cfg.value("angle_unit_mag", 1.0);
        P.eps = cfg.value("eps", 1.0e-8);
        if (m == kPoca) {
            P.length_weighted = cfg.value("length_weighted", false);
            if (variant == 1) {  // MutoPoCut(json): MutoPoCA's keys, then straight_line off and cut_percentile
                P.pocut = true;
                P.straight_line = false;
                P.cut_percentile = cfg.value("cut_percentile", 1.0);
            } else if (variant >= 2) {  // MutoSLR(json): the grid and the common keys; SLRIter: num_iteration
                P.slr = variant - 1;
                if (P.slr == 2) P.slr_iterations = cfg.value("num_iteration", 1);
                if (P.slr_iterations < 0) throw Error(MUTO_ERR_CONFIG, "num_iteration must be >= 0");
                const std::string sch = cfg.value("slr_iter_schedule", std::string("levels"));
                if (sch != "levels" && sch != "sequential")
                    throw Error(MUTO_ERR_CONFIG, "slr_iter_schedule must be \"levels\" or \"sequential\"");
                P.slr_sequential = sch == "sequential";
            }
        } else {
            P.update_with_mean = cfg.value("update_with_mean", false);
            P.early_stop = cfg.value("early_stop", false);
            P.mean_percentile = cfg.value("mean_percentile", 100);
            P.num_iteration = cfg.value("num_iteration", 10);
            P.initialize_method = cfg.value("initialize_method", 0);
            P.initialize_value = cfg.value("initialize_value", 1.0e-7);
            P.initial_image_file = cfg.value("initial_image_file", "");
            P.error_xy = cfg.value("error_xy", 1.0);
            P.error_dz_outer = cfg.value("error_dz_outer", 1000.0);
            P.error_dz_inner = cfg.value("error_dz_inner", 1000.0);
            if (m == kMap) {
                P.beta = cfg.value("beta", 1.0);
                P.p = cfg.value("p", 1.0);
                P.delta = cfg.value("delta", 0.1);
                P.add_object_prior = cfg.value("add_object_prior", false);
                P.all_neighbours = cfg.value("all_neighbours", false);
            }
            if (P.mean_percentile <= 0) throw Error(MUTO_ERR_CONFIG, "mean_percentile must be positive");
            if (P.num_iteration < 0) throw Error(MUTO_ERR_CONFIG, "num_iteration must be >= 0");
        }
        const std::string prec = cfg.value("precision", "mixed");
        if (prec == "mixed") P.precision = 0;
        else if (prec == "fp64") P.precision = 1;
        else throw Error(MUTO_ERR_CONFIG, "precision must be \"mixed\" or \"fp64\"");
        P.use_graph = cfg.value("use_graph", true);
        if (cfg.contains("random_seed")) {
            P.seed_set = true;
            P.random_seed = static_cast<uint64_t>(cfg.value("random_seed", int64_t(0)));
        }
        if (cfg.contains("compute_cost")) P.compute_cost = cfg.value("compute_cost", false) ? 1 : 0;
        P.newton_max_iter = cfg.value("newton_max_iter", 200);
        P.tile_pairs = cfg.value("tile_pairs", 0);
        const std::string mp = cfg.value("muon_pass", "auto");
        if (mp == "auto") P.muon_pass = 0;
        else if (mp == "tile") P.muon_pass = 1;
        else if (mp == "warp") P.muon_pass = 2;
        else throw Error(MUTO_ERR_CONFIG, "muon_pass must be \"auto\", \"tile\" or \"warp\"");
        if (cfg.contains("voxel_stream_above") && cfg.at("voxel_stream_above").is_string()) {
            if (cfg.value("voxel_stream_above", "") != "auto")
                throw Error(MUTO_ERR_CONFIG, "voxel_stream_above must be an integer or \"auto\"");
            P.voxel_stream_above = -2;  // chosen by timing at prepare
        } else {
            P.voxel_stream_above = cfg.value("voxel_stream_above", static_cast<int64_t>(-1));
            if (P.voxel_stream_above < -1) throw Error(MUTO_ERR_CONFIG, "voxel_stream_above must be >= -1");
        }
        const std::string ml = cfg.value("muon_layout", "auto");
        if (ml == "auto") P.muon_layout = 0;
        else if (ml == "columns") P.muon_layout = 1;
        else if (ml == "index") P.muon_layout = 2;
        else throw Error(MUTO_ERR_CONFIG, "muon_layout must be \"auto\", \"columns\" or \"index\"");
        if (P.newton_max_iter < 1) throw Error(MUTO_ERR_CONFIG, "newton_max_iter must be >= 1");
        const std::string fv = cfg.value("fused_variant", "auto");
        if (fv == "auto") P.fused_variant = -1;
        else if (fv == "4x8") P.fused_variant = 0;
        else if (fv == "8x8") P.fused_variant = 1;
        else if (fv == "8x16") P.fused_variant = 2;
        else if (fv == "16x8") P.fused_variant = 3;
        else if (fv == "16x16") P.fused_variant = 4;
        else if (fv == "8x4") P.fused_variant = 5;
        else if (fv == "staged") P.fused_variant = kFusedStaged;
        else if (fv == "split") P.fused_variant = kFusedVariants;
        else if (fv == "split8") P.fused_variant = kFusedVariants + 2;  // its scatter 8 pairs deep per lane
        else if (fv == "split8_overlap") P.fused_variant = kFusedVariants + 4;  // and overlapped with the muon pass
        else throw Error(MUTO_ERR_CONFIG, "fused_variant must be \"auto\", \"4x8\", \"8x4\", \"8x8\", \"8x16\", "
                                          "\"16x8\", \"16x16\", \"staged\", \"split\", \"split8\" or \"split8_overlap\"");
        P.fused_prefetch = cfg.value("fused_prefetch", false);
        P.setup_chunk_pairs = cfg.value("setup_chunk_pairs", static_cast<int64_t>(0));
        if (P.setup_chunk_pairs < 0) throw Error(MUTO_ERR_CONFIG, "setup_chunk_pairs must be >= 0");
        const std::string pl = cfg.value("path_lists", "auto");
        if (pl == "auto") P.path_lists = 0;
        else if (pl == "voxel_major") P.path_lists = kListsVoxelMajor;
        else if (pl == "muon_major") P.path_lists = kListsMuonMajor;
        else if (pl == "recompute") P.path_lists = kListsRecompute;
        else throw Error(MUTO_ERR_CONFIG, "path_lists must be \"auto\", \"voxel_major\", \"muon_major\" or \"recompute\"");
        const bool mean_update = P.update_with_mean && P.mean_percentile == 100;
        if (m != kPoca && P.path_lists >= kListsMuonMajor && !mean_update)
            throw Error(MUTO_ERR_CONFIG, "path_lists \"muon_major\" and \"recompute\" take the mean update "
                                         "(update_with_mean true, mean_percentile 100)");
    } catch (const json::type_error& e) {
        throw Error(MUTO_ERR_CONFIG, std::string("config value of the wrong type: ") + e.what());
    } catch (const json::out_of_range& e) {
        throw Error(MUTO_ERR_CONFIG, e.what());
    }
    return P;
}

// CUDA-event timing of launches, also inside captured graphs (external event nodes)
class Profiler {
public:
    bool on = false;
    struct Rec {
        std::string name;
        cudaEvent_t a, b;
    };
    std::vector<Rec> pool;   // events reused across flushes
    size_t used = 0;
    std::map<std::string, std::pair<uint64_t, double>> stats;

    ~Profiler() {
        for (auto& r : pool) {
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
    }
    Rec* begin(const char* name, cudaStream_t s, bool capturing) {
        if (!on) return nullptr;
        if (used == pool.size()) {
            Rec r;
            CK(cudaEventCreate(&r.a));
            CK(cudaEventCreate(&r.b));
            pool.push_back(r);
        }
        Rec* r = &pool[used++];
        r->name = name;
        CK(cudaEventRecordWithFlags(r->a, s, capturing ? cudaEventRecordExternal : cudaEventRecordDefault));
        return r;
    }
    void end(Rec* r, cudaStream_t s, bool capturing) {
        if (!r) return;
        CK(cudaEventRecordWithFlags(r->b, s, capturing ? cudaEventRecordExternal : cudaEventRecordDefault));
    }
    // Accumulate records [first, used) after the stream has synchronised.
    void harvest(size_t first, size_t last) {
        for (size_t i = first; i < last; ++i) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, pool[i].a, pool[i].b) == cudaSuccess) {
                auto& st = stats[pool[i].name];
                st.first += 1;
                st.second += ms;
            }
        }
    }
};

}  // namespace
}  // namespace muto

using namespace muto;

struct muto_handle {
    Method method = kMlsd;
    Params P;
    muto_grid grid{};          // current grid (may be adopted from the initial image)
    cudaStream_t stream = nullptr;
    ClassFan fan;                 // side streams of the voxel pass's class kernels
    int device = 0, num_sms = 148;
    uint64_t l2_bytes = 0;         // the device's L2 size
    size_t smem_optin = 0;
    std::atomic<uint64_t> dev_bytes{0};
    Profiler prof;
    bool capturing = false;
    unsigned long long launches = 0;   // launches of this handle (graph replays included)

    // tracks (scan 0; a batch handle keeps scans 1.. in batch_rays)
    DevMem rays;
    uint64_t n_rays = 0;
    bool batch = false;
    struct ScanMeta {
        muto_grid grid{};
        uint64_t n_rays = 0, n_total = 0, N = 0, noff = 0, V = 0, voff = 0;
    };
    std::vector<ScanMeta> scans;                       // per scan (one entry when not a batch)
    std::vector<std::unique_ptr<DevMem>> batch_rays;   // tracks of scans 1..
    uint64_t vtot = 0;                                 // voxels of all scans
    // initial image (host)
    bool init_set = false;
    bool init_missing = false;
    std::vector<double> init_img;
    muto_grid init_grid{};

    // counters
    DevMem ctr_mem;
    Counters* ctr() { return ctr_mem.as<Counters>(); }
    uint64_t n_total = 0;

    // kept muons
    uint64_t N = 0, npairs = 0;
    DevMem kept, sd, pr2, scat, pr64, off;
    DevMem vidx, L, T;            // muon-major pair lists
    DevMem vm_mu, vm_LT;          // voxel-major copy (muon, (L, T))
    DevMem vclass;                // VoxDesc of every voxel, by segment-length class
    uint32_t vclass_n[kVoxClasses] = {};
    int vox_blocks_real[2 * kVoxClasses] = {}, vox_blocks_f64[2 * kVoxClasses] = {};  // resident blocks per class kernel
    uint32_t vox_streamed = 0;  // classes selected by the streamed path
    long long vox_stream_above = -1;  // the threshold vox_streamed stands for (-1: none)
    uint32_t slr_levels = 0;          // levels of the SLRIter schedule (0: none or sequential)
    uint64_t vclass_off[kVoxClasses] = {};
    DevMem kslot;                     // per kept muon: its row of kvec (empty: its own index)
    DevMem walk_order;                // recompute form: the kept muons by decreasing path bound
    DevMem mult, start, kvec, keys;   // keys: the voxel pass's order key of every pair
    DevMem win;                       // per voxel: the last selection window (center, half-width)
    int lists = kListsVoxelMajor;     // how the pair lists are kept (Lists)
    DevMem gsum;                      // muon-major / recompute: per-voxel sums of g_ij (bricked like lam_b)
    DevMem ltot;                      // recompute: in-grid path length per kept muon
    int fused_variant = 1, fused_blocks = 0;  // stored-list fused pass: variant and persistent grid
    int scatter_group = 32, scatter_blocks = 0;  // split form's scatter pass (fused_variant == kFusedVariants)
    int scatter_depth = 4;                       // its pairs in flight per lane
    // the split form overlapped: muon pass and scatter on chunks of the muons,
    // the scatter of chunk c on the side stream while the muon pass of c+1 runs
    static constexpr int kOverlapChunks = 4;
    bool overlap = false;
    int warp_blocks_ov = 0, scatter_blocks_ov = 0;  // each kernel's grid when they share the GPU
    cudaEvent_t ov_ev[kOverlapChunks + 1] = {};
    bool brick = false;               // path voxel indices are bricked (single scans), see lam_b
    BrickDims bdims{};
    uint64_t vb = 0;                  // bricked index space (>= V)
    DevMem lam_b;                     // lambda in bricked order, refreshed before every muon pass
    DevMem lam, lam_ml, cost_hist;
    DevMem tiles;
    uint32_t ntiles = 0;
    int tile_pairs = 0, tile_muons = 0, group = 32, tile_blocks = 0;
    int muon_kind = 1, muon_group = 32, warp_blocks = 0;  // chosen muon-pass variant
    float tune_ms[4] = {0, 0, 0, 0};
    bool prepared = false;
    int iters = 0;
    bool stopped = false;
    // PoCA outputs
    DevMem img64, weight, assign;
    // adjoint scratch
    DevMem lam64, grad, dl, fval, loglam;
    // graph
    cudaGraphExec_t graph = nullptr;
    size_t graph_prof_first = 0, graph_prof_last = 0;
    unsigned long long graph_launches = 0;

    std::string last_msg;
    int last_err = 0;

    bool fp64() const { return P.precision == 1; }
    uint64_t V() const { return batch ? vtot : static_cast<uint64_t>(grid.nx) * grid.ny * grid.nz; }
    const muto_ray* scan_rays(size_t s) const {
        return s == 0 ? rays.as<muto_ray>() : batch_rays[s - 1]->as<muto_ray>();
    }
    bool want_cost() const { return P.compute_cost >= 0 ? P.compute_cost != 0 : (P.early_stop || P.log_results); }

    void drop_graph() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
    }
    ~muto_handle() {
        drop_graph();
        for (int k = 0; k < fan.n; ++k) {
            cudaStreamDestroy(fan.side[k]);
            cudaEventDestroy(fan.join[k]);
        }
        if (fan.n) cudaEventDestroy(fan.fork);
        for (cudaEvent_t e : ov_ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

void set_err(muto_handle* h, int code, const std::string& msg) {
    if (!h) return;
    h->last_err = code;
    h->last_msg = msg;
}

template <class F>
int guarded(muto_handle* h, F&& f) {
    try {
        f();
        return MUTO_OK;
    } catch (const Error& e) {
        set_err(h, e.code, e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_err(h, MUTO_ERR_NOMEM, "host allocation failed");
        return MUTO_ERR_NOMEM;
    } catch (const std::exception& e) {
        set_err(h, MUTO_ERR_ARG, e.what());
        return MUTO_ERR_ARG;
    }
}

// launch helper: profiling + launch accounting
template <class F>
void run(muto_handle* h, const char* name, F&& f) {
    const unsigned long long before = launches_so_far();
    Profiler::Rec* r = h->prof.begin(name, h->stream, h->capturing);
    f();
    h->prof.end(r, h->stream, h->capturing);
    if (!h->capturing) h->launches += launches_so_far() - before;
    CK(cudaGetLastError());
}

// An NVTX range over one entry point's call.
struct NvtxRange {
    nvtxRangeId_t id;
    explicit NvtxRange(const char* n) : id(nvtxRangeStartA(n)) {}
    ~NvtxRange() { nvtxRangeEnd(id); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Wall time of a host-side set-up phase (including the device waits inside
// it), kept with the kernel statistics under "host:<phase>" when profiling,
// and an NVTX range over it (start/end, not push/pop: a phase is replaced
// while the next one starts) for a profiler attached to the process.
struct HostPhase {
    muto_handle* h;
    const char* name;
    std::chrono::steady_clock::time_point t0;
    nvtxRangeId_t range;
    HostPhase(muto_handle* hh, const char* n)
        : h(hh), name(n), t0(std::chrono::steady_clock::now()), range(nvtxRangeStartA(n)) {}
    ~HostPhase() {
        nvtxRangeEnd(range);
        if (!h->prof.on) return;
        const double ms =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        auto& st = h->prof.stats[std::string("host:") + name];
        st.first += 1;
        st.second += ms;
    }
};

void sync_and_harvest(muto_handle* h, size_t first) {
    CK(cudaStreamSynchronize(h->stream));
    h->prof.harvest(first, h->prof.used);
    h->prof.used = first;
}

// ---------------------------------------------------------------------------
// Setup
// ---------------------------------------------------------------------------
void resolve_initial_image(muto_handle* h, std::vector<double>& img, uint64_t seed_offset = 0) {
    int method = h->P.initialize_method;
    if (method == 0) {  // src/MutoMLSD.cpp:228-245
        if (!h->init_set || h->init_missing || h->init_img.empty()) {
            method = 1;  // file missing -> random
        } else {
            if (h->init_grid.nx != h->grid.nx || h->init_grid.ny != h->grid.ny || h->init_grid.nz != h->grid.nz)
                h->grid = h->init_grid;  // adopt the image's grid
            img = h->init_img;
            return;
        }
    }
    img.assign(static_cast<uint64_t>(h->grid.nx) * h->grid.ny * h->grid.nz, 0.0);
    if (method == 1) {  // N(2, 0.5) * 1e-7, at least 1e-10 (src/MutoMLSD.cpp:251-261)
        uint64_t seed = (h->P.seed_set ? h->P.random_seed : std::random_device{}()) + seed_offset;
        std::mt19937_64 gen(seed);
        const double two_pi = 6.283185307179586;
        for (uint64_t i = 0; i < img.size(); ++i) {
            const double u1 = (static_cast<double>(gen() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
            const double u2 = static_cast<double>(gen() >> 11) * (1.0 / 9007199254740992.0);
            const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(two_pi * u2);
            const double v = (2.0 + 0.5 * z) * 1.0e-7;
            img[i] = 1.0e-10 <= v ? v : 1.0e-10;
        }
    } else {
        std::fill(img.begin(), img.end(), h->P.initialize_value);
    }
}

void alloc_counters(muto_handle* h) {
    if (h->ctr_mem.empty()) h->ctr_mem.alloc(sizeof(Counters), &h->dev_bytes);
    CK(cudaMemsetAsync(h->ctr_mem.as<void>(), 0, sizeof(Counters), h->stream));
}

// SLR (src/MutoSLR.cpp:47-103) and SLRIter (src/MutoSLRIter.cpp:15-83): the
// first pass over every ray at once; the iterative form's later passes, in
// place and in muon order, over the walked straight lines kept on the device
// The level schedule of SLRIter's later passes (slr_levels.h), made once
// from the walked paths, which do not change between passes; the muons are
// then grouped by level (index order inside a level) for the device.
void slr_level_schedule(muto_handle* h, const DevMem& off, const DevMem& vox, uint64_t nt, uint64_t np, DevMem& order,
                        DevMem& lstart, DevMem& fo) {
    const uint64_t V = h->V();
    cudaStream_t s = h->stream;
    if (nt >= 0xffffffffull) throw Error(MUTO_ERR_CAPACITY, "slr_iter: more than 2^32-1 rays");
    std::vector<uint64_t> off_h(nt + 1);
    std::vector<uint32_t> vox_h(np);
    CK(cudaMemcpyAsync(off_h.data(), off.as<uint64_t>(), (nt + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    if (np > 0) CK(cudaMemcpyAsync(vox_h.data(), vox.as<uint32_t>(), np * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::vector<uint32_t> level(nt);
    const uint32_t levels = slr_levels(off_h.data(), vox_h.data(), nt, V, level.data());
    std::vector<uint32_t> start(static_cast<size_t>(levels) + 1, 0), order_h(nt);
    for (uint64_t i = 0; i < nt; ++i) ++start[level[i]];  // level l (1-based) counted at start[l]
    uint32_t acc = 0;
    for (uint32_t l = 0; l <= levels; ++l) {
        const uint32_t c = start[l];
        start[l] = acc;
        acc += c;
    }
    // start[l] is now where level l begins (level 0 is empty); the device
    // reads level l (0-based) at start[l + 1] .. start[l + 2]
    std::vector<uint32_t> cur(start.begin(), start.end());
    for (uint64_t i = 0; i < nt; ++i) order_h[cur[level[i]]++] = static_cast<uint32_t>(i);
    start.push_back(static_cast<uint32_t>(nt));
    // where each muon's pairs go in level order
    std::vector<uint64_t> fo_h(nt + 1, 0);
    for (uint64_t q = 0; q < nt; ++q) fo_h[q + 1] = fo_h[q] + (off_h[order_h[q] + 1] - off_h[order_h[q]]);
    order.alloc(std::max<uint64_t>(nt, 1) * sizeof(uint32_t), &h->dev_bytes);
    lstart.alloc(start.size() * sizeof(uint32_t), &h->dev_bytes);
    fo.alloc((nt + 1) * sizeof(uint64_t), &h->dev_bytes);
    CK(cudaMemcpyAsync(order.as<uint32_t>(), order_h.data(), nt * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(lstart.as<uint32_t>(), start.data() + 1, (start.size() - 1) * sizeof(uint32_t),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(fo.as<uint64_t>(), fo_h.data(), (nt + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // the host vectors go out of scope
    h->slr_levels = levels;
}

void prepare_slr(muto_handle* h, uint64_t nt) {
    const uint64_t V = h->V();
    cudaStream_t s = h->stream;
    SlrArgs a;
    a.rays = h->rays.as<muto_ray>();
    a.n = nt;
    a.g = h->grid;
    a.mag = h->P.angle_unit_mag;
    a.has_energy = h->P.has_energy;
    a.length_weighted = h->P.length_weighted;
    a.img = h->img64.as<double>();
    a.weight = h->weight.as<double>();
    const int passes = h->P.slr == 2 ? h->P.slr_iterations : 1;
    if (passes >= 1) run(h, "slr", [&] { launch_slr(a, s); });
    if (passes >= 2 && nt > 0) {
        DevMem counts, off, vox, len, scan_scr;
        counts.alloc(nt * sizeof(uint32_t), &h->dev_bytes);
        off.alloc((nt + 1) * sizeof(uint64_t), &h->dev_bytes);
        scan_scr.alloc(scan_scratch_bytes(nt + 1), &h->dev_bytes);
        run(h, "slr_paths", [&] {
            launch_slr_paths(a, nullptr, counts.as<uint32_t>(), nullptr, nullptr, s);
            scan_u32_to_u64(counts.as<uint32_t>(), off.as<uint64_t>(), nt, scan_scr.as<void>(), s);
        });
        uint64_t np = 0;
        CK(cudaMemcpyAsync(&np, off.as<uint64_t>() + nt, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        vox.alloc(std::max<uint64_t>(np, 1) * sizeof(uint32_t), &h->dev_bytes);
        len.alloc(std::max<uint64_t>(np, 1) * sizeof(double), &h->dev_bytes);
        run(h, "slr_paths", [&] {
            launch_slr_paths(a, off.as<uint64_t>(), nullptr, vox.as<uint32_t>(), len.as<double>(), s);
        });
        // the pass-independent terms of every pair, once
        DevMem iv0, winc, e2;
        iv0.alloc(std::max<uint64_t>(np, 1) * sizeof(double), &h->dev_bytes);
        winc.alloc(std::max<uint64_t>(np, 1) * sizeof(double), &h->dev_bytes);
        e2.alloc(nt * sizeof(double), &h->dev_bytes);
        const SlrPass sp{off.as<uint64_t>(), vox.as<uint32_t>(), len.as<double>(), iv0.as<double>(), winc.as<double>(),
                         e2.as<double>()};
        run(h, "slr_paths", [&] { launch_slr_pair_terms(a, sp, s); });
        DevMem order, lstart, fo, fvox, fiv0, fwinc, fe2;
        SlrFlat fl{};
        if (!h->P.slr_sequential) {
            {
                HostPhase ph(h, "slr_levels");
                slr_level_schedule(h, off, vox, nt, np, order, lstart, fo);
            }
            // the pairs copied into level order
            fvox.alloc(std::max<uint64_t>(np, 1) * sizeof(uint32_t), &h->dev_bytes);
            fiv0.alloc(std::max<uint64_t>(np, 1) * sizeof(double), &h->dev_bytes);
            fwinc.alloc(std::max<uint64_t>(np, 1) * sizeof(double), &h->dev_bytes);
            fe2.alloc(nt * sizeof(double), &h->dev_bytes);
            fl = SlrFlat{fo.as<uint64_t>(), fvox.as<uint32_t>(), fiv0.as<double>(), fwinc.as<double>(), fe2.as<double>()};
            run(h, "slr_paths", [&] { launch_slr_flatten(sp, order.as<uint32_t>(), nt, fl, s); });
        }
        for (int p = 1; p < passes; ++p)
            run(h, "slr_iter_pass", [&] {
                if (h->P.slr_sequential)
                    launch_slr_iter_pass(a, sp, s);
                else
                    launch_slr_iter_levels(a, fl, lstart.as<uint32_t>(), h->slr_levels, h->smem_optin, s);
            });
        CK(cudaStreamSynchronize(s));  // the path arrays go out of scope
    }
    run(h, "poca_normalize", [&] { launch_poca_normalize(h->img64.as<double>(), h->weight.as<double>(), V, h->P.eps, s); });
}

void prepare_poca(muto_handle* h) {
    const uint64_t V = h->V();
    h->img64.alloc(V * sizeof(double), &h->dev_bytes);
    h->weight.alloc(V * sizeof(double), &h->dev_bytes);
    h->assign.alloc(std::max<uint64_t>(h->n_rays, 1) * 3 * sizeof(long long), &h->dev_bytes);
    CK(cudaMemsetAsync(h->img64.as<void>(), 0, V * sizeof(double), h->stream));
    CK(cudaMemsetAsync(h->weight.as<void>(), 0, V * sizeof(double), h->stream));
    CK(cudaMemsetAsync(h->assign.as<void>(), 0xff, std::max<uint64_t>(h->n_rays, 1) * 3 * sizeof(long long), h->stream));
    uint64_t nt = h->P.total_num_rays > 0 ? static_cast<uint64_t>(h->P.total_num_rays) : h->n_rays;
    if (nt > h->n_rays) nt = h->n_rays;  // the reference would read past the end
    h->n_total = nt;
    PocaArgs a;
    a.rays = h->rays.as<muto_ray>();
    a.n = nt;
    a.g = h->grid;
    a.eps = h->P.eps;
    a.mag = h->P.angle_unit_mag;
    a.has_energy = h->P.has_energy;
    a.straight = h->P.straight_line;
    a.length_weighted = h->P.length_weighted;
    a.img = h->img64.as<double>();
    a.weight = h->weight.as<double>();
    a.assign = h->assign.as<long long>();
    a.ctr = h->ctr();
    a.vox = nullptr;
    a.value = nullptr;
    if (h->P.slr) {
        prepare_slr(h, nt);
        return;
    }
    DevMem walk, wlen, worder, owork;  // the kept rays' list for the walk kernel, its length, its order
    walk.alloc((std::max<uint64_t>(nt, 1) + 2) * sizeof(uint32_t) + sizeof(unsigned long long), &h->dev_bytes);
    a.walk_count = walk.as<unsigned long long>();
    a.walk = reinterpret_cast<uint32_t*>(walk.as<unsigned long long>() + 1);
    wlen.alloc(std::max<uint64_t>(nt, 1) * sizeof(uint32_t), &h->dev_bytes);
    worder.alloc(std::max<uint64_t>(nt, 1) * sizeof(uint32_t), &h->dev_bytes);
    owork.alloc(512 * sizeof(uint32_t), &h->dev_bytes);
    a.walk_len = wlen.as<uint32_t>();
    a.walk_order = worder.as<uint32_t>();
    a.order_work = owork.as<uint32_t>();
    if (!h->P.pocut) {
        run(h, "poca", [&] { launch_poca(a, h->stream); });
        run(h, "poca_normalize", [&] { launch_poca_normalize(h->img64.as<double>(), h->weight.as<double>(), V, h->P.eps, h->stream); });
        return;
    }
    // PoCut (src/MutoPoCut.cpp:19-121): the same ray kernel keeping each value
    // and voxel, then the values grouped by voxel, sorted, cut and summed
    cudaStream_t s = h->stream;
    DevMem vox, value, counts, off, cursor, keys, scan_scr, small, big, big_off, scratch;
    vox.alloc(std::max<uint64_t>(nt, 1) * sizeof(uint32_t), &h->dev_bytes);
    value.alloc(std::max<uint64_t>(nt, 1) * sizeof(double), &h->dev_bytes);
    counts.alloc(std::max<uint64_t>(V, 1) * sizeof(uint32_t), &h->dev_bytes);
    cursor.alloc(std::max<uint64_t>(V, 1) * sizeof(uint32_t), &h->dev_bytes);
    off.alloc((V + 1) * sizeof(uint64_t), &h->dev_bytes);
    scan_scr.alloc(scan_scratch_bytes(V + 1), &h->dev_bytes);
    CK(cudaMemsetAsync(counts.as<void>(), 0, std::max<uint64_t>(V, 1) * sizeof(uint32_t), s));
    CK(cudaMemsetAsync(cursor.as<void>(), 0, std::max<uint64_t>(V, 1) * sizeof(uint32_t), s));
    a.img = nullptr;
    a.vox = vox.as<uint32_t>();
    a.value = value.as<double>();
    run(h, "poca", [&] { launch_poca(a, s); });
    run(h, "pocut_group", [&] {
        launch_pocut_hist(vox.as<uint32_t>(), nt, counts.as<uint32_t>(), s);
        scan_u32_to_u64(counts.as<uint32_t>(), off.as<uint64_t>(), V, scan_scr.as<void>(), s);
    });
    uint64_t nkeys = 0;
    CK(cudaMemcpyAsync(&nkeys, off.as<uint64_t>() + V, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    std::vector<uint32_t> cnt(V);
    if (V) CK(cudaMemcpyAsync(cnt.data(), counts.as<void>(), V * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    keys.alloc(std::max<uint64_t>(nkeys, 1) * sizeof(unsigned long long), &h->dev_bytes);
    run(h, "pocut_group", [&] {
        launch_pocut_scatter(vox.as<uint32_t>(), value.as<double>(), nt, off.as<uint64_t>(), cursor.as<uint32_t>(),
                             keys.as<unsigned long long>(), s);
    });
    // voxels of up to 32 values: a warp each; more: a block each, sorting in
    // shared memory, or in scratch of next_pow2(M) keys beyond kPocutSmemKeys
    std::vector<uint32_t> small_h, big_h;
    std::vector<uint64_t> big_off_h;
    uint64_t nscratch = 0;
    for (uint64_t j = 0; j < V; ++j) {
        const uint32_t m = cnt[j];
        if (m == 0) continue;
        if (m <= 32) {
            small_h.push_back(static_cast<uint32_t>(j));
            continue;
        }
        big_h.push_back(static_cast<uint32_t>(j));
        uint64_t n2 = 1;
        while (n2 < m) n2 <<= 1;
        big_off_h.push_back(nscratch);
        if (n2 > kPocutSmemKeys) nscratch += n2;
    }
    small.alloc(std::max<size_t>(small_h.size(), 1) * sizeof(uint32_t), &h->dev_bytes);
    big.alloc(std::max<size_t>(big_h.size(), 1) * sizeof(uint32_t), &h->dev_bytes);
    big_off.alloc(std::max<size_t>(big_off_h.size(), 1) * sizeof(uint64_t), &h->dev_bytes);
    scratch.alloc(std::max<uint64_t>(nscratch, 1) * sizeof(unsigned long long), &h->dev_bytes);
    if (!small_h.empty())
        CK(cudaMemcpyAsync(small.as<void>(), small_h.data(), small_h.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    if (!big_h.empty()) {
        CK(cudaMemcpyAsync(big.as<void>(), big_h.data(), big_h.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(big_off.as<void>(), big_off_h.data(), big_off_h.size() * sizeof(uint64_t),
                           cudaMemcpyHostToDevice, s));
    }
    const double eps = h->P.eps, cut = h->P.cut_percentile;
    run(h, "pocut_select", [&] {
        launch_pocut_empty(counts.as<uint32_t>(), h->weight.as<double>(), h->img64.as<double>(), V, eps, s);
        launch_pocut_small(small.as<uint32_t>(), static_cast<uint32_t>(small_h.size()), off.as<uint64_t>(),
                           counts.as<uint32_t>(), keys.as<unsigned long long>(), h->weight.as<double>(),
                           h->img64.as<double>(), eps, cut, s);
        launch_pocut_big(big.as<uint32_t>(), static_cast<uint32_t>(big_h.size()), off.as<uint64_t>(),
                         counts.as<uint32_t>(), keys.as<unsigned long long>(), big_off.as<uint64_t>(),
                         scratch.as<unsigned long long>(), h->weight.as<double>(), h->img64.as<double>(), eps, cut, s);
    });
    CK(cudaStreamSynchronize(s));  // the scratch arrays go out of scope
}

// The merged paths of all kept muons into the muon-major lists (vidx, L, T)
// with their offsets.  Per chunk of muons: one FP64 walk into slots sized by
// the FP32 path bounds (scratch for the chunk alone), then compaction to the
// exact slots after the chunks before it.  The lists are allocated for the
// bounds' total (a few percent above the pairs), so the set-up's peak is the
// lists plus one chunk's scratch.  counts holds every muon's bound on entry
// and its path length on return.  scan_off: each scan's first pair and the
// total; off_h: every muon's offset when the TMA tile pass needs them.
template <typename Real>
void fill_lists(muto_handle* h, DevMem& counts, DevMem& scratch, std::vector<uint64_t>& scan_off,
                std::vector<uint64_t>& off_h) {
    const Params& P = h->P;
    cudaStream_t s = h->stream;
    const uint64_t N = h->N;
    const size_t S = h->scans.size();
    const bool real64 = std::is_same<Real, double>::value;
    HostPhase ph(h, "fill");
    DevMem boff;
    boff.alloc((N + 1) * sizeof(uint64_t), &h->dev_bytes);
    run(h, "scan", [&] { scan_u32_to_u64(counts.as<uint32_t>(), boff.as<uint64_t>(), N, scratch.as<void>(), s); });
    uint64_t Pb = 0;
    CK(cudaMemcpyAsync(&Pb, boff.as<uint64_t>() + N, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    h->off.alloc((N + 1 + kPad) * sizeof(uint64_t), &h->dev_bytes);
    CK(cudaMemsetAsync(h->off.as<void>(), 0, (N + 1 + kPad) * sizeof(uint64_t), s));
    h->vidx.alloc((Pb + kPad) * sizeof(uint32_t), &h->dev_bytes);
    h->L.alloc((Pb + kPad) * sizeof(Real), &h->dev_bytes);
    h->T.alloc((Pb + kPad) * sizeof(Real), &h->dev_bytes);
    // one chunk's bounded slots: voxel, FP64 length (tails are summed in FP64), L, T
    const uint64_t per_pair = sizeof(uint32_t) + sizeof(double) + (real64 ? 0 : sizeof(Real)) + sizeof(Real);
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const uint64_t budget = std::min<uint64_t>(free_b / 4, uint64_t(12) << 30);
    uint64_t cap = std::min<uint64_t>(std::max<uint64_t>(Pb, 1), std::max<uint64_t>(budget / per_pair, uint64_t(1) << 20));
    if (P.setup_chunk_pairs > 0) cap = static_cast<uint64_t>(P.setup_chunk_pairs);
    DevMem vidx_b, l64_b, L_b, T_b;
    vidx_b.alloc((cap + kPad) * sizeof(uint32_t), &h->dev_bytes);
    l64_b.alloc((cap + kPad) * sizeof(double), &h->dev_bytes);
    if (!real64) L_b.alloc((cap + kPad) * sizeof(Real), &h->dev_bytes);
    T_b.alloc((cap + kPad) * sizeof(Real), &h->dev_bytes);
    Real* Lb = real64 ? reinterpret_cast<Real*>(l64_b.as<double>()) : L_b.as<Real>();
    const double avg = N ? static_cast<double>(Pb) / static_cast<double>(N) : 1.0;
    const uint64_t chunk0 = std::max<uint64_t>(P.setup_chunk_pairs > 0 ? 1 : 1024,
                                               static_cast<uint64_t>(static_cast<double>(cap) / (1.25 * avg + 1.0)));
    uint64_t base = 0;
    for (size_t k = 0; k < S; ++k) {
        const auto& sc = h->scans[k];
        const uint64_t end = sc.noff + sc.N;
        for (uint64_t m = sc.noff; m < end;) {
            uint64_t nc = std::min<uint64_t>(end - m, chunk0);
            uint64_t b[2] = {0, 0};
            for (;;) {  // the chunk's bounded slots must fit the scratch
                CK(cudaMemcpyAsync(&b[0], boff.as<uint64_t>() + m, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
                CK(cudaMemcpyAsync(&b[1], boff.as<uint64_t>() + m + nc, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
                CK(cudaStreamSynchronize(s));
                if (b[1] - b[0] <= cap || nc == 1) break;
                nc = (nc + 1) / 2;
            }
            if (b[1] - b[0] > cap) throw Error(MUTO_ERR_CAPACITY, "a muon's path bound exceeds the set-up scratch");
            run(h, "siddon_fill", [&] {
                launch_path_fill_bounded<Real>(h->scan_rays(k), h->kept.as<uint32_t>() + m, h->scat.as<double>() + 3 * m,
                                               boff.as<uint64_t>() + m, b[0], nc, sc.grid, P.straight_line,
                                               vidx_b.as<uint32_t>(), l64_b.as<double>(), Lb, T_b.as<Real>(),
                                               counts.as<uint32_t>() + m, h->ctr(), s);
            });
            run(h, "scan", [&] {
                scan_u32_to_u64(counts.as<uint32_t>() + m, h->off.as<uint64_t>() + m, nc, scratch.as<void>(), s);
                launch_add_u64(h->off.as<uint64_t>() + m, nc + 1, base, s);
            });
            run(h, "path_compact", [&] {
                launch_path_compact<Real>(boff.as<uint64_t>() + m, b[0], h->off.as<uint64_t>() + m, nc,
                                          vidx_b.as<uint32_t>(), Lb, T_b.as<Real>(), h->vidx.as<uint32_t>(),
                                          h->L.as<Real>(), h->T.as<Real>(), s);
            });
            CK(cudaMemcpyAsync(&base, h->off.as<uint64_t>() + m + nc, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            m += nc;
        }
    }
    vidx_b.release();
    l64_b.release();
    L_b.release();
    T_b.release();
    boff.release();
    unsigned long long over_bound = 0;
    CK(cudaMemcpyAsync(&over_bound, &h->ctr()->over_bound, sizeof(over_bound), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (over_bound > 0) {  // a bound was short (never expected): count exactly, then walk into exact slots
        CK(cudaMemsetAsync(&h->ctr()->overflow, 0, sizeof(unsigned long long), s));
        for (size_t k = 0; k < S; ++k) {
            const auto& sc = h->scans[k];
            run(h, "siddon_count", [&] {
                launch_path_count(h->scan_rays(k), h->kept.as<uint32_t>() + sc.noff, h->scat.as<double>() + 3 * sc.noff,
                                  sc.N, sc.grid, P.straight_line, counts.as<uint32_t>() + sc.noff, h->ctr(), s);
            });
        }
        run(h, "scan", [&] { scan_u32_to_u64(counts.as<uint32_t>(), h->off.as<uint64_t>(), N, scratch.as<void>(), s); });
        uint64_t Pe = 0;
        CK(cudaMemcpyAsync(&Pe, h->off.as<uint64_t>() + N, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        h->vidx.alloc((Pe + kPad) * sizeof(uint32_t), &h->dev_bytes);
        h->L.alloc((Pe + kPad) * sizeof(Real), &h->dev_bytes);
        h->T.alloc((Pe + kPad) * sizeof(Real), &h->dev_bytes);
        DevMem l64tmp;
        double* l64 = reinterpret_cast<double*>(h->L.as<Real>());
        if (!real64) {
            l64tmp.alloc(std::max<uint64_t>(Pe, 1) * sizeof(double), &h->dev_bytes);
            l64 = l64tmp.as<double>();
        }
        for (size_t k = 0; k < S; ++k) {
            const auto& sc = h->scans[k];
            run(h, "siddon_fill", [&] {
                launch_path_fill<Real>(h->scan_rays(k), h->kept.as<uint32_t>() + sc.noff,
                                       h->scat.as<double>() + 3 * sc.noff, h->off.as<uint64_t>() + sc.noff, sc.N,
                                       sc.grid, P.straight_line, h->vidx.as<uint32_t>(), l64, h->L.as<Real>(),
                                       h->T.as<Real>(), s);
            });
        }
        CK(cudaStreamSynchronize(s));
    }
    counts.release();
    // pair offsets on the host: each scan's first pair and the total, and
    // every muon's for the tile schedule
    for (size_t k = 0; k < S; ++k)
        CK(cudaMemcpyAsync(&scan_off[k], h->off.as<uint64_t>() + h->scans[k].noff, sizeof(uint64_t),
                           cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&scan_off[S], h->off.as<uint64_t>() + N, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    if (P.muon_pass == 1 && h->lists == kListsVoxelMajor) {
        off_h.resize(N + 1);
        CK(cudaMemcpyAsync(off_h.data(), h->off.as<uint64_t>(), (N + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
    h->npairs = scan_off[S];
}

template <typename Real>
void prepare_em(muto_handle* h) {
    using R4 = typename Vec4<Real>::type;
    const Params& P = h->P;
    cudaStream_t s = h->stream;
    std::vector<double> init;
    if (!h->batch) {
        resolve_initial_image(h, init);  // may adopt a new grid
        h->scans.resize(1);
        h->scans[0].grid = h->grid;
        h->scans[0].n_rays = h->n_rays;
    }
    const size_t S = h->scans.size();
    uint64_t V = 0;  // voxels of all scans: scan s owns [voff, voff + V_s)
    for (auto& sc : h->scans) {
        sc.V = static_cast<uint64_t>(sc.grid.nx) * sc.grid.ny * sc.grid.nz;
        sc.voff = V;
        V += sc.V;
    }
    if (V >= 0xffffffffull) throw Error(MUTO_ERR_CAPACITY, "more than 2^32-1 voxels in the batch");
    h->vtot = V;
    if (h->batch) {  // one initial image per scan (initialize_method 1 or 2)
        init.clear();
        for (size_t k = 0; k < S; ++k) {
            std::vector<double> one;
            h->grid = h->scans[k].grid;
            resolve_initial_image(h, one, k);
            init.insert(init.end(), one.begin(), one.end());
        }
        h->grid = h->scans[0].grid;
    }
    uint64_t nt_max = 0;
    for (auto& sc : h->scans) {
        uint64_t nt = P.total_num_rays > 0 ? static_cast<uint64_t>(P.total_num_rays) : sc.n_rays;
        sc.n_total = nt > sc.n_rays ? sc.n_rays : nt;  // the reference would read past the end
        nt_max = std::max(nt_max, sc.n_total);
    }
    h->n_total = 0;
    for (auto& sc : h->scans) h->n_total += sc.n_total;

    // --- gatherInformation per scan: keep flags, order-preserving compaction ---
    // (the flags are computed again in the second loop; the flag buffer is shared)
    DevMem flags, scratch;
    std::vector<std::unique_ptr<DevMem>> pos(S);
    std::unique_ptr<HostPhase> ph(new HostPhase(h, "gather"));
    flags.alloc(std::max<uint64_t>(nt_max, 1) * sizeof(uint32_t), &h->dev_bytes);
    uint64_t N = 0;
    for (size_t k = 0; k < S; ++k) {
        auto& sc = h->scans[k];
        pos[k].reset(new DevMem());
        pos[k]->alloc((sc.n_total + 1) * sizeof(uint64_t), &h->dev_bytes);
        if (scratch.bytes() < scan_scratch_bytes(sc.n_total + 1))
            scratch.alloc(scan_scratch_bytes(std::max<uint64_t>(sc.n_total, V) + 1), &h->dev_bytes);
        run(h, "keep_flags", [&] { launch_keep_flags(h->scan_rays(k), sc.n_total, sc.grid, P.eps, flags.as<uint32_t>(), s); });
        run(h, "scan", [&] { scan_u32_to_u64(flags.as<uint32_t>(), pos[k]->as<uint64_t>(), sc.n_total, scratch.as<void>(), s); });
        uint64_t n = 0;
        CK(cudaMemcpyAsync(&n, pos[k]->as<uint64_t>() + sc.n_total, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        sc.N = n;
        sc.noff = N;
        N += n;
    }
    if (N >= 0xffffffffull) throw Error(MUTO_ERR_CAPACITY, "more than 2^32-1 kept muons");
    h->N = N;
    h->kept.alloc(std::max<uint64_t>(N, 1) * sizeof(uint32_t), &h->dev_bytes);
    h->sd.alloc(std::max<uint64_t>(N, 1) * sizeof(R4), &h->dev_bytes);
    // per-pair and per-muon arrays carry kPad extra entries: the tile stage copies
    // ranges widened to 16-byte boundaries
    h->pr2.alloc((N + kPad) * sizeof(Real), &h->dev_bytes);
    h->scat.alloc(std::max<uint64_t>(N, 1) * 3 * sizeof(double), &h->dev_bytes);
    h->pr64.alloc(std::max<uint64_t>(N, 1) * sizeof(double), &h->dev_bytes);
    // --- how the lists are kept: the voxel-major copy for the median and
    // percentile updates; for the mean update the muon-major lists alone, or
    // none (the paths walked again every iteration) ---
    h->lists = P.path_lists ? P.path_lists
                            : (P.update_with_mean && P.mean_percentile == 100 ? kListsMuonMajor : kListsVoxelMajor);
    if (h->lists == kListsRecompute && h->batch)
        throw Error(MUTO_ERR_CONFIG, "path_lists \"recompute\" takes one scan per handle");
    // --- merged paths: one walk per muon into slots sized by an upper bound
    // on its path, then compaction to the exact slots (the walk is FP64 and
    // the set-up's costliest step, so it is not run twice to count first) ---
    DevMem counts;
    counts.alloc(std::max<uint64_t>(N, 1) * sizeof(uint32_t), &h->dev_bytes);
    ph.reset(new HostPhase(h, "info_count"));
    for (size_t k = 0; k < S; ++k) {
        const auto& sc = h->scans[k];
        const muto_ray* r = h->scan_rays(k);
        uint32_t* kept = h->kept.as<uint32_t>() + sc.noff;
        double* scat = h->scat.as<double>() + 3 * sc.noff;
        run(h, "keep_flags", [&] { launch_keep_flags(r, sc.n_total, sc.grid, P.eps, flags.as<uint32_t>(), s); });
        run(h, "compact", [&] { launch_compact(flags.as<uint32_t>(), pos[k]->as<uint64_t>(), sc.n_total, kept, s); });
        run(h, "muon_info", [&] {
            launch_muon_info<Real>(r, kept, sc.N, sc.grid, P.eps, P.has_energy, h->sd.as<R4>() + sc.noff,
                                   h->pr2.as<Real>() + sc.noff, scat, h->pr64.as<double>() + sc.noff, s);
        });
        if (h->lists != kListsRecompute)
            run(h, "path_bound", [&] {
                launch_path_bound(r, kept, scat, sc.N, sc.grid, P.straight_line, counts.as<uint32_t>() + sc.noff, s);
            });
    }
    flags.release();
    pos.clear();
    if (scratch.bytes() < scan_scratch_bytes(std::max<uint64_t>(N, V) + 1))
        scratch.alloc(scan_scratch_bytes(std::max<uint64_t>(N, V) + 1), &h->dev_bytes);
    h->mult.alloc(V * sizeof(uint32_t), &h->dev_bytes);
    CK(cudaMemsetAsync(h->mult.as<void>(), 0, V * sizeof(uint32_t), s));
    std::vector<uint64_t> scan_off(S + 1), off_h;
    if (h->lists == kListsRecompute) {
        // no lists: every kept muon's in-grid length and the pairs per voxel,
        // from one walk of every path
        counts.release();
        ph.reset(new HostPhase(h, "path_stats"));
        h->ltot.alloc(std::max<uint64_t>(N, 1) * sizeof(double), &h->dev_bytes);
        const auto& sc = h->scans[0];
        run(h, "path_stats", [&] {
            launch_path_stats(h->scan_rays(0), h->kept.as<uint32_t>(), h->scat.as<double>(), sc.N, sc.grid,
                              P.straight_line, h->ltot.as<double>(), h->mult.as<uint32_t>(), h->ctr(), s);
        });
        // the walks of every iteration run in order of decreasing path bound,
        // so that a warp's lanes walk paths of about the same length
        {
            DevMem bounds, work;
            bounds.alloc(std::max<uint64_t>(N, 1) * sizeof(uint32_t), &h->dev_bytes);
            work.alloc(512 * sizeof(uint32_t), &h->dev_bytes);
            h->walk_order.alloc(std::max<uint64_t>(N, 1) * sizeof(uint32_t), &h->dev_bytes);
            run(h, "path_order", [&] {
                launch_path_bound(h->scan_rays(0), h->kept.as<uint32_t>(), h->scat.as<double>(), sc.N, sc.grid,
                                  P.straight_line, bounds.as<uint32_t>(), s);
                launch_length_order(bounds.as<uint32_t>(), nullptr, N, h->walk_order.as<uint32_t>(),
                                    work.as<uint32_t>(), s);
            });
            CK(cudaStreamSynchronize(s));  // the bounds go out of scope
        }
        DevMem moff;
        moff.alloc((V + 1) * sizeof(uint64_t), &h->dev_bytes);
        run(h, "scan", [&] { scan_u32_to_u64(h->mult.as<uint32_t>(), moff.as<uint64_t>(), V, scratch.as<void>(), s); });
        CK(cudaMemcpyAsync(&h->npairs, moff.as<uint64_t>() + V, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    } else {
        fill_lists<Real>(h, counts, scratch, scan_off, off_h);
        // scan-local voxel indices into the batch's voxel space
        if (h->batch) {
            for (size_t k = 0; k < S; ++k) {
                const auto& sc = h->scans[k];
                const uint64_t pb = scan_off[k], pe = scan_off[k + 1];
                run(h, "voxel_offset", [&] {
                    launch_offset_voxels(h->vidx.as<uint32_t>() + pb, pe - pb, static_cast<uint32_t>(sc.V),
                                         static_cast<uint32_t>(sc.voff), s);
                });
            }
        }
        run(h, "voxel_hist", [&] {
            launch_voxel_hist(h->vidx.as<uint32_t>(), h->npairs, static_cast<uint32_t>(V), h->mult.as<uint32_t>(),
                              h->ctr(), s);
        });
        CK(cudaStreamSynchronize(s));
    }
    const uint64_t Pn = h->npairs;

    // --- the voxel-major copy of the lists (median / percentile updates) -----
    if (h->lists == kListsVoxelMajor) {
        ph.reset(new HostPhase(h, "voxel_major"));
        h->start.alloc((V + 1) * sizeof(uint64_t), &h->dev_bytes);
        {
            DevMem mcol, scol;
            if (!h->batch) {
                mcol.alloc(std::max<uint64_t>(V, 1) * sizeof(uint32_t), &h->dev_bytes);
                scol.alloc((V + 1) * sizeof(uint64_t), &h->dev_bytes);
            }
            run(h, "scan", [&] {
                launch_segment_starts(h->mult.as<uint32_t>(), static_cast<uint32_t>(V), h->batch ? nullptr : &h->grid,
                                      mcol.as<uint32_t>(), scol.as<uint64_t>(), scratch.as<void>(), h->start.as<uint64_t>(), s);
            });
            CK(cudaStreamSynchronize(s));
        }
        {
            DevMem cursor;
            cursor.alloc(V * sizeof(uint32_t), &h->dev_bytes);
            CK(cudaMemsetAsync(cursor.as<void>(), 0, V * sizeof(uint32_t), s));
            h->vm_mu.alloc((Pn + kPad) * sizeof(uint32_t), &h->dev_bytes);
            h->vm_LT.alloc((Pn + kPad) * sizeof(typename Vec2<Real>::type), &h->dev_bytes);
            DevMem staging;
            staging.alloc(std::max<uint64_t>(Pn, 1) * sizeof(R4), &h->dev_bytes);
            // coefficient rows in column order of the PoCA points, when asked or
            // when the table would take more than a third of L2
            h->kslot.release();
            const bool columns = P.muon_layout == 1 || (P.muon_layout == 0 && N * sizeof(R4) > h->l2_bytes / 3);
            if (columns && !h->batch && N > 0) {
                const uint64_t nc = static_cast<uint64_t>(h->grid.nx) * h->grid.ny;
                DevMem cell, hist, cstart, ccur, cscr;
                h->kslot.alloc(N * sizeof(uint32_t), &h->dev_bytes);
                cell.alloc(N * sizeof(uint32_t), &h->dev_bytes);
                hist.alloc((nc + 1) * sizeof(uint32_t), &h->dev_bytes);
                ccur.alloc((nc + 1) * sizeof(uint32_t), &h->dev_bytes);
                cstart.alloc((nc + 1) * sizeof(uint64_t), &h->dev_bytes);
                cscr.alloc(scan_scratch_bytes(nc + 1), &h->dev_bytes);
                run(h, "muon_slots", [&] {
                    launch_muon_slots(h->scat.as<double>(), N, h->grid, cell.as<uint32_t>(), hist.as<uint32_t>(),
                                      cstart.as<uint64_t>(), ccur.as<uint32_t>(), cscr.as<void>(), h->kslot.as<uint32_t>(),
                                      s);
                });
                CK(cudaStreamSynchronize(s));
            }
            run(h, "voxel_major", [&] {
                launch_build_voxel_major<Real>(h->off.as<uint64_t>(), N, h->vidx.as<uint32_t>(), h->L.as<Real>(),
                                               h->T.as<Real>(), static_cast<uint32_t>(V), h->start.as<uint64_t>(),
                                               cursor.as<uint32_t>(), Pn, staging.as<R4>(), h->vm_mu.as<uint32_t>(),
                                               h->vm_LT.as<typename Vec2<Real>::type>(),
                                               h->kslot.empty() ? nullptr : h->kslot.as<uint32_t>(), s);
            });
            CK(cudaStreamSynchronize(s));
        }
        h->kvec.alloc((N + kPad) * sizeof(R4), &h->dev_bytes);
        ph.reset(new HostPhase(h, "classes"));
        {
            // voxel classes by segment length, one voxel-pass kernel each, built on
            // the device; a descriptor carries the voxel, its pair count and its
            // first voxel-major pair
            const uint32_t nb = voxel_class_blocks(V);
            const uint64_t nc = static_cast<uint64_t>(nb) * kVoxClasses;
            DevMem ccount, cfirst, cscr;
            ccount.alloc(nc * sizeof(uint32_t), &h->dev_bytes);
            cfirst.alloc((nc + 1) * sizeof(uint64_t), &h->dev_bytes);
            cscr.alloc(scan_scratch_bytes(nc + 1), &h->dev_bytes);
            h->vclass.alloc(std::max<uint64_t>(V, 1) * sizeof(VoxDesc), &h->dev_bytes);
            run(h, "voxel_classes", [&] {
                launch_voxel_classes<Real>(h->mult.as<uint32_t>(), h->start.as<uint64_t>(), static_cast<uint32_t>(V),
                                           h->batch ? nullptr : &h->grid, ccount.as<uint32_t>(), cfirst.as<uint64_t>(),
                                           cscr.as<void>(), h->vclass.as<VoxDesc>(), s);
            });
            uint64_t bnd[kVoxClasses + 1];
            for (int c = 0; c <= kVoxClasses; ++c)
                CK(cudaMemcpyAsync(&bnd[c], cfirst.as<uint64_t>() + static_cast<uint64_t>(c) * nb, sizeof(uint64_t),
                                   cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (bnd[kVoxClasses] != V) throw Error(MUTO_ERR_STATE, "voxel classes do not cover the voxels");
            for (int c = 0; c < kVoxClasses; ++c) {
                h->vclass_off[c] = bnd[c];
                h->vclass_n[c] = static_cast<uint32_t>(bnd[c + 1] - bnd[c]);
            }
            // the voxel pass's key array (kPad past the end: the class kernels'
            // L2 prefetches round out to 16 bytes)
            h->vox_stream_above = P.voxel_stream_above == -2 ? -1 : P.voxel_stream_above;
            h->vox_streamed = P.voxel_stream_above < 0 ? 0u
                              : vox_streamed_mask(static_cast<uint32_t>(std::min<long long>(P.voxel_stream_above, 0xffffffffLL)));
            h->keys.alloc((Pn + kPad) * sizeof(typename KeyOf<Real>::type), &h->dev_bytes);
            em_voxel_occupancy<Real, Real>(h->vox_blocks_real);
            em_voxel_occupancy<Real, double>(h->vox_blocks_f64);
            for (int c = 0; c < 2 * kVoxClasses; ++c) {
                h->vox_blocks_real[c] *= h->num_sms;
                h->vox_blocks_f64[c] *= h->num_sms;
            }
        }
    }
    scratch.release();

    // --- tiles of consecutive muons fitting the shared-memory stage ----------
    // (only for the TMA tile pass)
    ph.reset(new HostPhase(h, "tiles"));
    const double avg = N > 0 ? static_cast<double>(Pn) / static_cast<double>(N) : 0.0;
    h->group = avg <= 32 ? 8 : (avg <= 64 ? 16 : 32);
    h->ntiles = 0;
    h->tile_pairs = 0;
    h->tile_muons = 0;
    if (P.muon_pass == 1 && h->lists == kListsVoxelMajor) {
        uint64_t maxpath = 0;
        for (uint64_t i = 0; i < N; ++i) maxpath = std::max<uint64_t>(maxpath, off_h[i + 1] - off_h[i]);
        int TP = P.tile_pairs > 0 ? P.tile_pairs : (std::is_same<Real, double>::value ? 1024 : 2048);
        while (static_cast<uint64_t>(TP) < maxpath) TP *= 2;
        const int TM = std::is_same<Real, double>::value ? 128 : 256;
        if (em_muon_smem_bytes<Real>(TP, TM) > h->smem_optin)
            throw Error(MUTO_ERR_CAPACITY, "longest muon path (" + std::to_string(maxpath) + " voxels) does not fit the shared-memory tile");
        std::vector<uint32_t> tb;
        tb.push_back(0);
        uint64_t cs = 0;
        for (uint64_t i = 0; i < N; ++i) {
            if (off_h[i + 1] - off_h[cs] > static_cast<uint64_t>(TP) || i - cs >= static_cast<uint64_t>(TM)) {
                tb.push_back(static_cast<uint32_t>(i));
                cs = i;
            }
        }
        if (N > 0) tb.push_back(static_cast<uint32_t>(N));
        h->ntiles = static_cast<uint32_t>(tb.size() - 1);
        h->tiles.alloc(tb.size() * sizeof(uint32_t), &h->dev_bytes);
        CK(cudaMemcpyAsync(h->tiles.as<void>(), tb.data(), tb.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        h->tile_pairs = TP;
        h->tile_muons = TM;
        CK(em_muon_configure<Real>(TP, TM));
        h->tile_blocks = em_muon_blocks<Real>(TP, TM, h->group) * h->num_sms;
    }

    // --- image ---------------------------------------------------------------
    ph.reset(new HostPhase(h, "image"));
    // the muon pass gathers lambda through bricked indices (single scans)
    h->brick = false;
    h->lam_b.release();
    if (!h->batch) {
        h->bdims = brick_dims(h->grid);
        h->vb = brick_volume(h->bdims);
        if (h->vb < 0xffffffffull) {
            h->brick = true;
            h->lam_b.alloc(h->vb * sizeof(Real), &h->dev_bytes);
            CK(cudaMemsetAsync(h->lam_b.as<void>(), 0, h->vb * sizeof(Real), s));
            if (h->lists != kListsRecompute)
                run(h, "brick_indices", [&] {
                    launch_brick_indices(h->vidx.as<uint32_t>(), Pn, h->bdims, static_cast<uint32_t>(V), s);
                });
        }
    }
    h->lam.alloc(V * sizeof(Real), &h->dev_bytes);
    h->gsum.release();
    h->win.release();
    if (h->lists == kListsVoxelMajor) {
        h->win.alloc(2 * V * sizeof(Real), &h->dev_bytes);
        CK(cudaMemsetAsync(h->win.as<void>(), 0, 2 * V * sizeof(Real), s));  // half-width 0: no prediction yet
    } else {  // the per-voxel sums of g_ij, in the index space of the gathered lambda
        const uint64_t ng = h->brick ? h->vb : V;
        h->gsum.alloc((ng + kPad) * sizeof(Real), &h->dev_bytes);
        CK(cudaMemsetAsync(h->gsum.as<void>(), 0, (ng + kPad) * sizeof(Real), s));
        // the split form's per-muon coefficients
        if (h->lists == kListsMuonMajor) h->kvec.alloc((N + kPad) * sizeof(R4), &h->dev_bytes);
        h->kslot.release();
    }
    {
        std::vector<Real> init_r(init.begin(), init.end());
        CK(cudaMemcpyAsync(h->lam.as<void>(), init_r.data(), V * sizeof(Real), cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
    }
    if (h->method == kMap) h->lam_ml.alloc(V * sizeof(double), &h->dev_bytes);
    h->cost_hist.alloc(std::max(P.num_iteration, 1) * 4 * sizeof(double) + 4096 * sizeof(double), &h->dev_bytes);
    CK(cudaStreamSynchronize(s));
}

template <typename Real>
void launch_muon_pass(muto_handle* h, const MuonPassArgs<Real>& a_in, cudaStream_t s) {
    MuonPassArgs<Real> a = a_in;
    if (h->brick) {  // a.lam is in voxel order; the pass gathers from the bricked copy
        launch_brick_lambda<Real>(a_in.lam, static_cast<uint32_t>(h->V()), h->bdims, h->lam_b.as<Real>(), s);
        a.lam = h->lam_b.as<Real>();
        a.V = static_cast<uint32_t>(h->vb);
    }
    if (h->muon_kind == 2)
        launch_em_muon_warp<Real>(a, static_cast<uint32_t>(h->N), h->warp_blocks, h->muon_group, s);
    else
        launch_em_muon<Real>(a, h->tile_pairs, h->tile_muons, h->tile_blocks, h->group, s);
}

template <typename Real>
MuonPassArgs<Real> muon_args(muto_handle* h, const Real* lam, bool cost) {
    using R4 = typename Vec4<Real>::type;
    const Params& P = h->P;
    const double exy = P.error_xy, ezo = P.error_dz_outer, ezi = P.error_dz_inner;  // src/MutoMLSD.cpp:168-170
    MuonPassArgs<Real> a;
    a.off = h->off.as<uint64_t>();
    a.tile_mb = h->tiles.as<uint32_t>();
    a.ntiles = h->ntiles;
    a.vidx = h->vidx.as<uint32_t>();
    a.L = h->L.as<Real>();
    a.T = h->T.as<Real>();
    a.sd = h->sd.as<R4>();
    a.pr2 = h->pr2.as<Real>();
    a.lam = lam;
    a.kout = h->kvec.as<R4>();
    a.kslot = h->kslot.empty() ? nullptr : h->kslot.as<uint32_t>();
    a.V = static_cast<uint32_t>(h->V());
    a.E00 = 4.0 * exy * exy / (ezo * ezo);
    a.E11 = 2.0 * exy * exy * (1.0 + (ezi / ezo + 1.0) * ezi / ezo);
    a.E01 = 2.0 * exy * exy * ezi / (ezo * ezo);
    a.compute_cost = cost ? 1 : 0;
    a.ctr = h->ctr();
    return a;
}

// Choices of the muon-pass tuner, kept for the process: scans of the same
// shape (precision, device, muons to within a factor of 2, mean path to
// within 8 voxels) reuse the choice instead of timing again.
struct TuneShape {
    int fp64, device, log2n, path8;
    bool operator<(const TuneShape& o) const {
        return std::tie(fp64, device, log2n, path8) < std::tie(o.fp64, o.device, o.log2n, o.path8);
    }
};
std::mutex g_tune_mu;
std::map<TuneShape, std::pair<int, int>> g_tune_choice;

// The mean-update pass over muon-major lists or recomputed paths: lambda
// (voxel order) is copied to its bricked order first when the path indices
// are bricked; the pass adds every g_ij to h->gsum.  With `profiled` each
// launch goes through run() under its own name (em_fused, em_walk, or the
// split form's em_muon and em_scatter).
template <typename Real>
void launch_fused_pass(muto_handle* h, const Real* lam, bool cost, cudaStream_t s, bool profiled = false) {
    auto launch = [&](const char* name, auto&& f) {
        if (profiled) run(h, name, f);
        else f();
    };
    using R4 = typename Vec4<Real>::type;
    const Params& P = h->P;
    const double exy = P.error_xy, ezo = P.error_dz_outer, ezi = P.error_dz_inner;  // src/MutoMLSD.cpp:168-170
    FusedArgs<Real> a{};
    a.off = h->off.as<uint64_t>();
    a.vidx = h->vidx.as<uint32_t>();
    a.L = h->L.as<Real>();
    a.T = h->T.as<Real>();
    a.sd = h->sd.as<R4>();
    a.pr2 = h->pr2.as<Real>();
    a.lam = lam;
    a.V = static_cast<uint32_t>(h->V());
    const bool split = h->lists == kListsMuonMajor && h->fused_variant == kFusedVariants;
    if (h->brick) {  // (the split form's muon pass refreshes the bricked copy itself)
        if (!split)
            launch("brick_lambda", [&] {
                launch_brick_lambda<Real>(lam, static_cast<uint32_t>(h->V()), h->bdims, h->lam_b.as<Real>(), s);
            });
        a.lam = h->lam_b.as<Real>();
        a.V = static_cast<uint32_t>(h->vb);
    }
    a.G = h->gsum.as<Real>();
    a.N = static_cast<uint32_t>(h->N);
    a.E00 = 4.0 * exy * exy / (ezo * ezo);
    a.E11 = 2.0 * exy * exy * (1.0 + (ezi / ezo + 1.0) * ezi / ezo);
    a.E01 = 2.0 * exy * exy * ezi / (ezo * ezo);
    a.compute_cost = cost ? 1 : 0;
    a.prefetch = P.fused_prefetch ? 1 : 0;
    a.ctr = h->ctr();
    if (h->lists == kListsMuonMajor && h->fused_variant == kFusedVariants) {
        // split form: the muon pass writes every muon's coefficients, the scatter adds g_ij
        const MuonPassArgs<Real> m = muon_args<Real>(h, lam, cost);
        if (!h->overlap || profiled || h->N < static_cast<uint64_t>(muto_handle::kOverlapChunks)) {
            // (profiled passes time each kernel alone)
            launch("em_muon", [&] { launch_muon_pass<Real>(h, m, s); });
            launch("em_scatter", [&] {
                launch_em_scatter<Real>(a, h->kvec.as<R4>(), h->scatter_group, h->scatter_depth, h->scatter_blocks, s);
            });
            return;
        }
        // overlapped: chunk c's scatter on the side stream once chunk c's
        // muon pass is done, while the muon pass of chunk c+1 runs; each
        // kernel on a grid of about half the GPU
        MuonPassArgs<Real> mb = m;
        if (h->brick) {
            launch_brick_lambda<Real>(lam, static_cast<uint32_t>(h->V()), h->bdims, h->lam_b.as<Real>(), s);
            mb.lam = h->lam_b.as<Real>();
            mb.V = static_cast<uint32_t>(h->vb);
        }
        cudaStream_t side = h->fan.side[0];
        constexpr int C = muto_handle::kOverlapChunks;
        for (int c = 0; c < C; ++c) {
            const uint64_t m0 = h->N * c / C, m1 = h->N * (c + 1) / C;
            MuonPassArgs<Real> mc = mb;
            mc.off += m0;
            mc.sd += m0;
            mc.pr2 += m0;
            mc.kout += m0;
            launch_em_muon_warp<Real>(mc, static_cast<uint32_t>(m1 - m0), h->warp_blocks_ov, h->muon_group, s);
            CK(cudaEventRecord(h->ov_ev[c], s));
            CK(cudaStreamWaitEvent(side, h->ov_ev[c], 0));
            FusedArgs<Real> ac = a;
            ac.off += m0;
            ac.N = static_cast<uint32_t>(m1 - m0);
            launch_em_scatter<Real>(ac, h->kvec.as<R4>() + m0, h->scatter_group, h->scatter_depth,
                                    h->scatter_blocks_ov, side);
        }
        CK(cudaEventRecord(h->ov_ev[C], side));
        CK(cudaStreamWaitEvent(s, h->ov_ev[C], 0));
        return;
    }
    if (h->lists == kListsRecompute) {
        a.rays = h->rays.as<muto_ray>();
        a.kept = h->kept.as<uint32_t>();
        a.scat = h->scat.as<double>();
        a.ltot = h->ltot.as<double>();
        a.g = make_dev_grid(h->grid);
        a.straight = P.straight_line ? 1 : 0;
        a.bdims = h->bdims;
        a.brick = h->brick ? 1 : 0;
        a.order = h->walk_order.empty() ? nullptr : h->walk_order.as<uint32_t>();
        launch("em_walk", [&] { launch_em_fused_walk<Real>(a, h->num_sms, s); });
    } else {
        launch("em_fused", [&] { launch_em_fused<Real>(a, h->fused_variant, h->fused_blocks, s); });
    }
}

// the voxel side of a mean-update pass: out = l + l^2 G / (2M) (or the
// gradient into grad); clears h->gsum
template <typename Real, typename OutT>
void launch_fused_update(muto_handle* h, const Real* lam, OutT* out, double* grad, const double* lam64,
                         cudaStream_t s) {
    launch_mean_update<Real, OutT>(lam, h->gsum.as<Real>(), h->mult.as<uint32_t>(), static_cast<uint32_t>(h->V()),
                                   h->brick ? &h->bdims : nullptr, out, grad, lam64, s);
}

// In-project autotuner of the stored-list pass: the variants whose held
// pairs suit the scan's mean path, timed on the scan's own lists (one
// warm-up and two timed launches each); the per-voxel sums are cleared after.
std::map<TuneShape, int> g_fused_choice;  // the tuner's pick per scan shape (guarded by g_tune_mu)

template <typename Real>
void autotune_fused(muto_handle* h) {
    if (h->lists != kListsMuonMajor || h->N == 0) return;
    HostPhase ph(h, "autotune");
    const double avg = static_cast<double>(h->npairs) / static_cast<double>(h->N);
    int log2n = 0;
    while ((h->N >> log2n) > 1) ++log2n;
    const TuneShape shape{h->fp64() ? 1 : 0, h->device, log2n, static_cast<int>(avg / 8.0)};
    std::vector<int> cands;
    const bool forced = h->P.fused_variant >= 0;
    if (forced) cands.push_back(h->P.fused_variant);
    for (int v = 0; v < kFusedVariants && !forced; ++v) {
        const int held = fused_variant_held(v);
        // a one-pass variant is a candidate when its lanes per muon suit the
        // mean path: 4 or 8 lanes below 48 pairs, 8 or 16 up to 160, 16 beyond
        const int g = fused_variant_group(v);
        const bool fit = avg < 48.0 ? g <= 8 && held <= 64 : avg < 160.0 ? g >= 8 && held <= 128 : g == 16;
        // the staged variant runs only when asked for: slower than the split
        // form on every workload measured (its fixed batches of 32 muons wait
        // on their longest path)
        if (fit && v != kFusedStaged) cands.push_back(v);
    }
    // the split form: its scatter with g and g/2 lanes per muon, 4 or 8 pairs in
    // flight per lane.  (The overlapped form, kFusedVariants + 4, runs only
    // when asked for: it measured no faster, the two kernels being bound by
    // the same memory system.)
    if (!forced)
        for (int c = 0; c < 4; ++c) cands.push_back(kFusedVariants + c);
    auto apply = [&](int v) {
        h->fused_variant = v >= kFusedVariants ? kFusedVariants : v;
        if (v >= kFusedVariants) {  // split: the warp-batched muon pass and the scatter pass
            const int g = avg <= 32 ? 8 : (avg <= 64 ? 16 : 32);
            const int c = v - kFusedVariants;
            h->muon_kind = 2;
            h->muon_group = g;
            h->warp_blocks = em_muon_warp_blocks<Real>(g) * h->num_sms;
            h->scatter_group = c % 2 == 0 ? g : std::max(8, g / 2);
            h->scatter_depth = c >= 2 ? 8 : 4;
            h->scatter_blocks = em_scatter_blocks<Real>(h->scatter_group, h->scatter_depth) * h->num_sms;
            h->overlap = c == 4;
            h->warp_blocks_ov = std::max(1, em_muon_warp_blocks<Real>(g) / 2) * h->num_sms;
            h->scatter_blocks_ov = std::max(1, em_scatter_blocks<Real>(h->scatter_group, h->scatter_depth) / 2) * h->num_sms;
        } else {
            h->fused_blocks = em_fused_blocks<Real>(v) * h->num_sms;
            h->overlap = false;
        }
    };
    if (cands.size() == 1) {
        apply(cands[0]);
        return;
    }
    {  // scans of the same shape reuse the choice instead of timing again
        std::lock_guard<std::mutex> lock(g_tune_mu);
        const auto it = g_fused_choice.find(shape);
        if (it != g_fused_choice.end()) {
            apply(it->second);
            return;
        }
    }
    cudaStream_t s = h->stream;
    Counters saved;
    CK(cudaMemcpyAsync(&saved, h->ctr(), sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    int pick = cands[0];
    // a scan of more than 2^30 pairs takes tens of milliseconds per pass:
    // one timed pass per candidate, no warm-up, is then well above the noise
    const bool big = h->npairs > (uint64_t(1) << 30);
    const int reps = big ? 1 : 2;
    for (size_t i = 0; i < cands.size(); ++i) {
        apply(cands[i]);
        if (!big) launch_fused_pass<Real>(h, h->lam.as<Real>(), false, s);
        CK(cudaEventRecord(e0, s));
        for (int r = 0; r < reps; ++r) launch_fused_pass<Real>(h, h->lam.as<Real>(), false, s);
        CK(cudaEventRecord(e1, s));
        CK(cudaEventSynchronize(e1));
        CK(cudaGetLastError());
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        ms /= static_cast<float>(reps);
        if (i < 4) h->tune_ms[i] = ms;
        // a one-pass variant must beat the split form by 5 %: where the two
        // are that close, run to run noise would otherwise flip the pick
        const float score = cands[i] >= kFusedVariants ? ms : 1.05f * ms;
        if (score < best) {
            best = score;
            pick = cands[i];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h->launches += (big ? 1 : 3) * cands.size() * (h->brick ? 2 : 1);
    apply(pick);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_fused_choice[shape] = pick;
    }
    const uint64_t ng = h->brick ? h->vb : h->V();
    CK(cudaMemsetAsync(h->gsum.as<void>(), 0, (ng + kPad) * sizeof(Real), s));
    CK(cudaMemcpyAsync(h->ctr(), &saved, sizeof(Counters), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
}


// In-project autotuner: time the candidate muon-pass variants on this scan's
// own lists (one warm-up and two timed launches each) and keep the fastest.
template <typename Real>
void autotune_muon_pass(muto_handle* h) {
    if (h->N == 0) return;
    HostPhase ph(h, "autotune");
    int log2n = 0;
    while ((h->N >> log2n) > 1) ++log2n;
    const TuneShape shape{h->fp64() ? 1 : 0, h->device, log2n,
                          static_cast<int>(static_cast<double>(h->npairs) / static_cast<double>(h->N) / 8.0)};
    if (h->P.muon_pass == 0) {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        const auto it = g_tune_choice.find(shape);
        if (it != g_tune_choice.end()) {
            h->muon_kind = it->second.first;
            h->muon_group = it->second.second;
            if (h->muon_kind == 2) h->warp_blocks = em_muon_warp_blocks<Real>(h->muon_group) * h->num_sms;
            return;
        }
    }
    struct Cand {
        int kind, group;
    };
    std::vector<Cand> cands;
    // "auto": the warp-batched pass at the group size the mean path length
    // suggests and its neighbour (the TMA tile pass, slower on every workload
    // measured, runs only when asked for)
    if (h->P.muon_pass == 1) cands.push_back({1, h->group});
    if (h->P.muon_pass != 1) {
        cands.push_back({2, h->group});
        cands.push_back({2, h->group == 32 ? 16 : h->group * 2});
    }
    auto apply = [&](const Cand& c) {
        h->muon_kind = c.kind;
        h->muon_group = c.group;
        if (c.kind == 2) h->warp_blocks = em_muon_warp_blocks<Real>(c.group) * h->num_sms;
    };
    if (cands.size() == 1) {
        apply(cands[0]);
        return;
    }
    cudaStream_t s = h->stream;
    Counters saved;
    CK(cudaMemcpyAsync(&saved, h->ctr(), sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const MuonPassArgs<Real> a = muon_args<Real>(h, h->lam.as<Real>(), false);
    float best = 1e30f;
    Cand pick = cands[0];
    for (size_t i = 0; i < cands.size(); ++i) {
        apply(cands[i]);
        launch_muon_pass<Real>(h, a, s);
        CK(cudaEventRecord(e0, s));
        for (int r = 0; r < 2; ++r) launch_muon_pass<Real>(h, a, s);
        CK(cudaEventRecord(e1, s));
        CK(cudaEventSynchronize(e1));
        CK(cudaGetLastError());
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        ms /= 2.f;
        if (i < 4) h->tune_ms[i] = ms;
        if (ms < best) {
            best = ms;
            pick = cands[i];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h->launches += 3 * cands.size();
    apply(pick);
    if (h->P.muon_pass == 0) {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_choice[shape] = {pick.kind, pick.group};
    }
    CK(cudaMemcpyAsync(h->ctr(), &saved, sizeof(Counters), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
}

std::map<std::pair<TuneShape, int>, long long> g_voxel_choice;  // per shape and log2(V) (guarded by g_tune_mu)

template <typename Real, typename OutT>
VoxelPassArgs<Real, OutT> voxel_args(muto_handle* h, const Real* lam, int mode, OutT* out);
template <typename Real, typename OutT>
void launch_voxel_pass(muto_handle* h, const VoxelPassArgs<Real, OutT>& v, cudaStream_t s);
int voxel_mode(const Params& P);

// In-project autotuner of the voxel pass's launch shape ("voxel_stream_above"
// "auto"): the class kernels holding a voxel's keys in registers for every
// segment up to the register budget, or streaming the classes beyond 512
// pairs from the key array, timed on the scan's own lists after one muon
// pass (one warm-up and two timed voxel passes each, into scratch, without
// selection windows so that the iterations start as untuned ones do).
template <typename Real>
void autotune_voxel_pass(muto_handle* h) {
    if (h->lists != kListsVoxelMajor || h->N == 0 || h->P.voxel_stream_above != -2) return;
    HostPhase ph(h, "autotune");
    int log2n = 0, log2v = 0;
    while ((h->N >> log2n) > 1) ++log2n;
    while ((h->V() >> log2v) > 1) ++log2v;
    const std::pair<TuneShape, int> shape{TuneShape{h->fp64() ? 1 : 0, h->device, log2n,
                                                    static_cast<int>(static_cast<double>(h->npairs) / h->N / 8.0)},
                                          log2v};
    auto apply = [&](long long above) {
        h->vox_stream_above = above;
        h->vox_streamed = above < 0 ? 0u : vox_streamed_mask(static_cast<uint32_t>(above));
    };
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        const auto it = g_voxel_choice.find(shape);
        if (it != g_voxel_choice.end()) {
            apply(it->second);
            return;
        }
    }
    cudaStream_t s = h->stream;
    Counters saved;
    CK(cudaMemcpyAsync(&saved, h->ctr(), sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    launch_muon_pass<Real>(h, muon_args<Real>(h, h->lam.as<Real>(), false), s);  // the coefficients the pass reads
    DevMem out;
    out.alloc(h->V() * sizeof(Real), nullptr);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const long long cands[2] = {-1, 512};
    float best = 1e30f;
    long long pick = -1;
    for (long long above : cands) {
        apply(above);
        auto v = voxel_args<Real, Real>(h, h->lam.as<Real>(), voxel_mode(h->P), out.as<Real>());
        v.win = nullptr;
        launch_voxel_pass<Real, Real>(h, v, s);
        CK(cudaEventRecord(e0, s));
        for (int r = 0; r < 2; ++r) launch_voxel_pass<Real, Real>(h, v, s);
        CK(cudaEventRecord(e1, s));
        CK(cudaEventSynchronize(e1));
        CK(cudaGetLastError());
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            pick = above;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    apply(pick);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_voxel_choice[shape] = pick;
    }
    CK(cudaMemcpyAsync(h->ctr(), &saved, sizeof(Counters), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
}

template <typename Real, typename OutT>
VoxelPassArgs<Real, OutT> voxel_args(muto_handle* h, const Real* lam, int mode, OutT* out) {
    using R4 = typename Vec4<Real>::type;
    VoxelPassArgs<Real, OutT> v{};
    v.start = h->start.as<uint64_t>();
    v.mult = h->mult.as<uint32_t>();
    v.vm_mu = h->vm_mu.as<uint32_t>();
    v.vm_LT = h->vm_LT.as<typename Vec2<Real>::type>();
    v.kvec = h->kvec.as<R4>();
    v.lam = lam;
    v.V = static_cast<uint32_t>(h->V());
    v.mode = mode;
    v.pct = h->P.mean_percentile;
    v.out = out;
    v.grad = nullptr;
    v.lam64 = nullptr;
    v.keys = h->keys.as<typename KeyOf<Real>::type>();
    v.P = h->npairs;
    v.win = (mode == kVoxMedian || mode == kVoxPercentile) && !h->win.empty() ? h->win.as<Real>() : nullptr;
    return v;
}

template <typename Real, typename OutT>
void launch_voxel_pass(muto_handle* h, const VoxelPassArgs<Real, OutT>& v, cudaStream_t s) {
    const VoxDesc* lists[kVoxClasses];
    for (int c = 0; c < kVoxClasses; ++c) lists[c] = h->vclass.as<VoxDesc>() + h->vclass_off[c];
    launch_em_voxel<Real, OutT>(v, lists, h->vclass_n,
                                std::is_same<OutT, Real>::value ? h->vox_blocks_real : h->vox_blocks_f64,
                                h->vox_streamed, h->num_sms, &h->fan, s);
}

int voxel_mode(const Params& P) {
    if (!P.update_with_mean) return kVoxMedian;
    return P.mean_percentile == 100 ? kVoxMean : kVoxPercentile;
}

// ---------------------------------------------------------------------------
// One EM / MAP iteration (device work only; graph-capturable)
// ---------------------------------------------------------------------------
template <typename Real>
void enqueue_iteration(muto_handle* h) {
    const Params& P = h->P;
    cudaStream_t s = h->stream;
    const uint32_t cap = static_cast<uint32_t>(h->cost_hist.bytes() / sizeof(double));
    if (h->lists != kListsVoxelMajor) {  // the mean update over muon-major lists or recomputed paths
        launch_fused_pass<Real>(h, h->lam.as<Real>(), h->want_cost(), s, true);
        if (h->method == kMap) {  // ML step into lambda_ML, then the MAP step (src/MutoMAP.cpp:138-184)
            run(h, "em_update", [&] {
                launch_fused_update<Real, double>(h, h->lam.as<Real>(), h->lam_ml.as<double>(), nullptr, nullptr, s);
            });
            MapParams mp{P.beta, P.p, P.delta, P.eps, P.all_neighbours, P.add_object_prior, P.newton_max_iter};
            run(h, "map_voxel", [&] {
                launch_map_voxel<Real>(h->lam.as<Real>(), h->lam_ml.as<double>(), h->mult.as<uint32_t>(),
                                       make_dev_grid(h->grid), mp, h->ctr(), s);
            });
            run(h, "map_copy", [&] { launch_copy_to<Real>(h->lam_ml.as<double>(), h->lam.as<Real>(), h->V(), s); });
        } else {  // each thread reads only its own voxel's lambda before writing it: in place
            run(h, "em_update", [&] {
                launch_fused_update<Real, Real>(h, h->lam.as<Real>(), h->lam.as<Real>(), nullptr, nullptr, s);
            });
        }
        run(h, "cost", [&] { launch_finalize_cost(h->ctr(), static_cast<double>(h->N), h->cost_hist.as<double>(), cap, s); });
        return;
    }
    const MuonPassArgs<Real> a = muon_args<Real>(h, h->lam.as<Real>(), h->want_cost());
    run(h, "em_muon", [&] { launch_muon_pass<Real>(h, a, s); });
    const int mode = voxel_mode(P);
    if (h->method == kMap) {  // ML step into lambda_ML, then the MAP step from the snapshot (src/MutoMAP.cpp:138-184)
        const auto v = voxel_args<Real, double>(h, h->lam.as<Real>(), mode, h->lam_ml.as<double>());
        run(h, "em_voxel", [&] { launch_voxel_pass<Real, double>(h, v, s); });
        MapParams mp{P.beta, P.p, P.delta, P.eps, P.all_neighbours, P.add_object_prior, P.newton_max_iter};
        run(h, "map_voxel", [&] {
            launch_map_voxel<Real>(h->lam.as<Real>(), h->lam_ml.as<double>(), h->mult.as<uint32_t>(),
                                   make_dev_grid(h->grid), mp, h->ctr(), s);
        });
        run(h, "map_copy", [&] { launch_copy_to<Real>(h->lam_ml.as<double>(), h->lam.as<Real>(), h->V(), s); });
    } else {  // each warp reads only its own voxel's lambda before writing it: in place
        const auto v = voxel_args<Real, Real>(h, h->lam.as<Real>(), mode, h->lam.as<Real>());
        run(h, "em_voxel", [&] { launch_voxel_pass<Real, Real>(h, v, s); });
    }
    run(h, "cost", [&] { launch_finalize_cost(h->ctr(), static_cast<double>(h->N), h->cost_hist.as<double>(), cap, s); });
}

template <typename Real>
void iterate_impl(muto_handle* h, int n) {
    const bool sync_each = h->P.early_stop || h->prof.on;
    for (int it = 0; it < n && !h->stopped; ++it) {
        const size_t pf = h->prof.used;
        if (h->P.use_graph) {
            if (!h->graph) {
                // capture one iteration once; replays reuse the same buffers
                HostPhase ph(h, "graph_capture");
                const unsigned long long before = launches_so_far();
                CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
                h->capturing = true;
                h->graph_prof_first = h->prof.used;
                try {
                    enqueue_iteration<Real>(h);
                } catch (...) {
                    cudaGraph_t gtmp;
                    cudaStreamEndCapture(h->stream, &gtmp);
                    if (gtmp) cudaGraphDestroy(gtmp);
                    h->capturing = false;
                    throw;
                }
                h->capturing = false;
                h->graph_prof_last = h->prof.used;
                cudaGraph_t graph;
                CK(cudaStreamEndCapture(h->stream, &graph));
                const cudaError_t e = cudaGraphInstantiate(&h->graph, graph, 0);
                cudaGraphDestroy(graph);
                CK(e);
                h->graph_launches = launches_so_far() - before;
            }
            CK(cudaGraphLaunch(h->graph, h->stream));
            h->launches += h->graph_launches;
        } else {
            enqueue_iteration<Real>(h);
        }
        h->iters += 1;
        if (sync_each) {
            CK(cudaStreamSynchronize(h->stream));
            if (h->prof.on) {
                if (h->P.use_graph) h->prof.harvest(h->graph_prof_first, h->graph_prof_last);
                else sync_and_harvest(h, pf);
            }
            if (h->P.early_stop) {
                Counters c;
                CK(cudaMemcpy(&c, h->ctr(), sizeof(Counters), cudaMemcpyDeviceToHost));
                // the reference compares with an uninitialised value on iteration 0 (src/MutoMLSD.cpp:184,209);
                // here the first possible stop is after the second iteration
                if (h->iters > 1 && c.cost_prev < c.cost_last) h->stopped = true;
            }
        }
    }
}

void check_handle(muto_handle* h) {
    if (!h) throw Error(MUTO_ERR_ARG, "null handle");
}

template <typename Real>
void download_image(muto_handle* h, double* out) {
    const uint64_t V = h->V();
    std::vector<Real> tmp(V);
    CK(cudaMemcpyAsync(tmp.data(), h->lam.as<Real>(), V * sizeof(Real), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (uint64_t j = 0; j < V; ++j) out[j] = static_cast<double>(tmp[j]);
}

template <typename Real>
void upload_image(muto_handle* h, const double* in) {
    const uint64_t V = h->V();
    std::vector<Real> tmp(in, in + V);
    CK(cudaMemcpyAsync(h->lam.as<Real>(), tmp.data(), V * sizeof(Real), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
}

// ---------------------------------------------------------------------------
// Adjoint
// ---------------------------------------------------------------------------
template <typename Real>
double nll_eval(muto_handle* h, const double* loglam_host, double* grad_host) {
    const uint64_t V = h->V();
    cudaStream_t s = h->stream;
    const size_t pf = h->prof.used;
    if (h->loglam.empty()) h->loglam.alloc(V * sizeof(double), &h->dev_bytes);
    if (h->lam64.empty()) h->lam64.alloc(V * sizeof(double), &h->dev_bytes);
    if (h->grad.empty()) h->grad.alloc(V * sizeof(double), &h->dev_bytes);
    if (h->dl.empty()) {
        h->dl.alloc(V * sizeof(double), &h->dev_bytes);
        CK(cudaMemsetAsync(h->dl.as<void>(), 0, V * sizeof(double), s));
    }
    if (h->fval.empty()) h->fval.alloc(sizeof(double), &h->dev_bytes);
    CK(cudaMemcpyAsync(h->loglam.as<double>(), loglam_host, V * sizeof(double), cudaMemcpyHostToDevice, s));
    // lambda in FP64 (prior, chain rule) and in the storage precision (muon pass)
    run(h, "exp_lambda", [&] { launch_exp_lambda<double>(h->loglam.as<double>(), h->mult.as<uint32_t>(), static_cast<uint32_t>(V), h->lam64.as<double>(), s); });
    DevMem lamR;
    const Real* lam_r = reinterpret_cast<const Real*>(h->lam64.as<double>());
    if (!std::is_same<Real, double>::value) {
        lamR.alloc(V * sizeof(Real), &h->dev_bytes);
        run(h, "exp_lambda", [&] { launch_exp_lambda<Real>(h->loglam.as<double>(), h->mult.as<uint32_t>(), static_cast<uint32_t>(V), lamR.as<Real>(), s); });
        lam_r = lamR.as<Real>();
    }
    Counters c0;
    CK(cudaMemcpyAsync(&c0, h->ctr(), sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaMemsetAsync(&h->ctr()->cost_sum, 0, sizeof(double), s));
    CK(cudaMemsetAsync(h->fval.as<void>(), 0, sizeof(double), s));
    if (h->lists != kListsVoxelMajor) {
        // one pass over the muon-major lists (or the paths walked again): the
        // cost and the per-voxel sums of g_ij; d NLL / d log l_j = -l_j sum_i g_ij
        launch_fused_pass<Real>(h, lam_r, true, s, true);
        run(h, "em_update_grad", [&] {
            launch_fused_update<Real, Real>(h, lam_r, nullptr, h->grad.as<double>(), h->lam64.as<double>(), s);
        });
    } else {
    const MuonPassArgs<Real> a = muon_args<Real>(h, lam_r, true);
    run(h, grad_host ? "nll_backward" : "nll_forward",
        [&] { launch_muon_pass<Real>(h, a, s); });
    if (grad_host) {  // d NLL / d log l_j = -l_j sum_i g_ij, per voxel
        auto v = voxel_args<Real, Real>(h, lam_r, kVoxGradient, nullptr);
        v.grad = h->grad.as<double>();
        v.lam64 = h->lam64.as<double>();
        run(h, "em_voxel_grad", [&] { launch_voxel_pass<Real, Real>(h, v, s); });
    }
    }
    const Params& P = h->P;
    if (h->method == kMap) {
        MapParams mp{P.beta, P.p, P.delta, P.eps, P.all_neighbours, P.add_object_prior, P.newton_max_iter};
        DevMem gdummy;
        double* gp = h->grad.as<double>();
        if (!grad_host) {
            gdummy.alloc(V * sizeof(double), &h->dev_bytes);
            gp = gdummy.as<double>();
        }
        run(h, "prior", [&] { launch_prior(h->lam64.as<double>(), h->mult.as<uint32_t>(), make_dev_grid(h->grid), mp, h->dl.as<double>(), gp, h->fval.as<double>(), s); });
        CK(cudaStreamSynchronize(s));
    }
    Counters c1;
    double prior = 0.0;
    CK(cudaMemcpyAsync(&c1, h->ctr(), sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&prior, h->fval.as<double>(), sizeof(double), cudaMemcpyDeviceToHost, s));
    if (grad_host) CK(cudaMemcpyAsync(grad_host, h->grad.as<double>(), V * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    // the singular counter counts covariance failures of iterations only
    CK(cudaMemcpy(&h->ctr()->singular, &c0.singular, sizeof(unsigned long long), cudaMemcpyHostToDevice));
    sync_and_harvest(h, pf);
    return c1.cost_sum + prior;
}

int n_prepared_check(muto_handle* h) {
    if (!h->prepared) throw Error(MUTO_ERR_STATE, "call muto_prepare (or muto_reconstruct) first");
    return 0;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
namespace {

// the voxel pass on synthetic segments: pair i has L = 1, T = 0 and its own
// muon with k = (x_i, 0, 0), every voxel lambda = 1, so s_i = 2 + x_i
template <typename Real>
void select_probe_run(const double* values, uint64_t n, const uint64_t* seg_off, uint32_t n_segs, int mode, int pct,
                      uint32_t streamed, uint32_t repeat, double* out) {
    using R2 = typename Vec2<Real>::type;
    using R4 = typename Vec4<Real>::type;
    OwnedStream owned;
    cudaStream_t s = owned.s;
    std::vector<uint32_t> mu(n);
    std::vector<R2> lt(n);
    std::vector<R4> kv(n);
    for (uint64_t i = 0; i < n; ++i) {
        mu[i] = static_cast<uint32_t>(i);
        lt[i].x = Real(1);
        lt[i].y = Real(0);
        kv[i].y = kv[i].z = kv[i].w = Real(0);
    }
    std::vector<VoxDesc> cls[kVoxClasses];
    for (uint32_t j = 0; j < n_segs; ++j) {
        const uint64_t m64 = seg_off[j + 1] - seg_off[j];
        if (seg_off[j + 1] < seg_off[j] || seg_off[j + 1] > n || m64 > 0xffffffffull)
            throw Error(MUTO_ERR_ARG, "segment offsets must be non-decreasing and within the values");
        const uint32_t m = static_cast<uint32_t>(m64);
        cls[vox_class_of<Real>(m)].push_back(VoxDesc{j, m, seg_off[j]});
    }
    std::vector<Real> lam(n_segs, Real(1));
    DevMem d_mu, d_lt, d_kv, d_lam, d_out, d_desc, d_keys, d_win;
    const uint64_t np = n + kPad;
    d_mu.alloc(np * sizeof(uint32_t), nullptr);
    d_lt.alloc(np * sizeof(R2), nullptr);
    d_kv.alloc(np * sizeof(R4), nullptr);
    d_lam.alloc(std::max<uint64_t>(n_segs, 1) * sizeof(Real), nullptr);
    d_out.alloc(std::max<uint64_t>(n_segs, 1) * sizeof(Real), nullptr);
    d_desc.alloc(std::max<uint64_t>(n_segs, 1) * sizeof(VoxDesc), nullptr);
    d_keys.alloc(np * sizeof(typename KeyOf<Real>::type), nullptr);
    d_win.alloc(std::max<uint64_t>(n_segs, 1) * 2 * sizeof(Real), nullptr);
    CK(cudaMemsetAsync(d_win.as<void>(), 0, std::max<uint64_t>(n_segs, 1) * 2 * sizeof(Real), s));
    if (n) {
        CK(cudaMemcpyAsync(d_mu.as<void>(), mu.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d_lt.as<void>(), lt.data(), n * sizeof(R2), cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemcpyAsync(d_lam.as<void>(), lam.data(), n_segs * sizeof(Real), cudaMemcpyHostToDevice, s));
    const VoxDesc* lists[kVoxClasses];
    uint32_t counts[kVoxClasses];
    uint64_t at = 0;
    for (int c = 0; c < kVoxClasses; ++c) {
        lists[c] = d_desc.as<VoxDesc>() + at;
        counts[c] = static_cast<uint32_t>(cls[c].size());
        if (counts[c])
            CK(cudaMemcpyAsync(d_desc.as<VoxDesc>() + at, cls[c].data(), counts[c] * sizeof(VoxDesc),
                               cudaMemcpyHostToDevice, s));
        at += counts[c];
    }
    int dev = 0, sms = 1;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int resident[2 * kVoxClasses];
    em_voxel_occupancy<Real, Real>(resident);
    for (int c = 0; c < 2 * kVoxClasses; ++c) resident[c] *= sms;
    VoxelPassArgs<Real, Real> v{};
    v.vm_mu = d_mu.as<uint32_t>();
    v.vm_LT = d_lt.as<R2>();
    v.kvec = d_kv.as<R4>();
    v.lam = d_lam.as<Real>();
    v.V = n_segs;
    v.mode = mode;
    v.pct = pct;
    v.out = d_out.as<Real>();
    v.keys = d_keys.as<typename KeyOf<Real>::type>();
    v.P = n;
    v.win = mode == kVoxMedian || mode == kVoxPercentile ? d_win.as<Real>() : nullptr;
    for (uint32_t rep = 0; rep < repeat; ++rep) {  // each pass its own values; windows carry over
        for (uint64_t i = 0; i < n; ++i) kv[i].x = static_cast<Real>(values[rep * n + i]);
        if (n) CK(cudaMemcpyAsync(d_kv.as<void>(), kv.data(), n * sizeof(R4), cudaMemcpyHostToDevice, s));
        launch_em_voxel<Real, Real>(v, lists, counts, resident, streamed, sms, nullptr, s);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(s));  // kv is rewritten by the next pass
    }
    std::vector<Real> o(n_segs);
    CK(cudaMemcpyAsync(o.data(), d_out.as<void>(), n_segs * sizeof(Real), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (uint32_t j = 0; j < n_segs; ++j) out[j] = static_cast<double>(o[j]);
}

}  // namespace

extern "C" {

const char* muto_version(void) { return "muto-gb300 0.1 (sm_103a)"; }

int muto_create(const char* method, const char* config_json, muto_handle** out) {
    if (!method || !out) return MUTO_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<muto_handle> h(new muto_handle());
    const std::string m(method);
    const int variant = m == "pocut" ? 1 : m == "slr" ? 2 : m == "slr_iter" ? 3 : 0;
    if (m == "poca" || variant > 0) h->method = kPoca;
    else if (m == "mlsd") h->method = kMlsd;
    else if (m == "map") h->method = kMap;
    else return MUTO_ERR_ARG;
    const int rc = guarded(h.get(), [&] {
        h->P = parse_params(h->method, config_json ? config_json : "", variant);
        h->grid = h->P.grid;
        CK(cudaGetDevice(&h->device));
        CK(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device));
        int l2 = 0;
        CK(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, h->device));
        h->l2_bytes = static_cast<uint64_t>(l2);
        int optin = 0;
        CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
        h->smem_optin = static_cast<size_t>(optin);
        CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&h->fan.fork, cudaEventDisableTiming));
        for (int k = 0; k < ClassFan::kSide; ++k) {
            CK(cudaStreamCreateWithFlags(&h->fan.side[k], cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&h->fan.join[k], cudaEventDisableTiming));
            h->fan.n = k + 1;
        }
        for (cudaEvent_t& e : h->ov_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        alloc_counters(h.get());
        CK(cudaStreamSynchronize(h->stream));
    });
    if (rc != MUTO_OK) return rc;
    *out = h.release();
    return MUTO_OK;
}

int muto_destroy(muto_handle* h) {
    if (!h) return MUTO_ERR_ARG;
    if (h->stream) cudaStreamSynchronize(h->stream);
    delete h;
    return MUTO_OK;
}

int muto_get_grid(const muto_handle* h, muto_grid* out) {
    if (!h || !out) return MUTO_ERR_ARG;
    *out = h->grid;
    return MUTO_OK;
}

int muto_get_status(const muto_handle* hc, muto_status* out) {
    if (!hc || !out) return MUTO_ERR_ARG;
    muto_handle* h = const_cast<muto_handle*>(hc);
    std::memset(out, 0, sizeof(*out));
    Counters c{};
    if (!h->ctr_mem.empty()) {
        if (cudaStreamSynchronize(h->stream) == cudaSuccess)
            cudaMemcpy(&c, h->ctr(), sizeof(Counters), cudaMemcpyDeviceToHost);
    }
    out->last_error = h->last_err;
    out->iterations_done = h->iters;
    out->early_stopped = h->stopped ? 1 : 0;
    out->precision = h->P.precision;
    out->n_total = h->n_total;
    out->n_scat_in_grid = h->method == kPoca ? c.in_grid : h->N;
    out->n_not_parallel = c.not_parallel;
    out->n_pairs = h->npairs;
    out->n_singular = c.singular;
    out->n_nonconverged = c.nonconverged;
    out->n_bounds = c.bounds;
    out->n_path_overflow = c.overflow + c.timeouts;
    out->cost = c.cost_last;
    out->cost_prev = c.cost_prev;
    out->device_bytes = h->dev_bytes.load();
    out->muon_pass = h->method == kPoca ? 0 : h->muon_kind;
    out->muon_group = h->muon_kind == 2 ? h->muon_group : h->group;
    out->tile_pairs = h->tile_pairs;
    out->tile_muons = h->tile_muons;
    out->path_lists = h->method == kPoca ? 0 : h->lists;
    out->slr_levels = static_cast<int32_t>(std::min<uint32_t>(h->slr_levels, 0x7fffffffu));
    out->reserved = 0;
    out->voxel_stream_above = h->method == kPoca || h->lists != kListsVoxelMajor
                                  ? -1 : static_cast<int32_t>(std::min<long long>(h->vox_stream_above, 0x7fffffffLL));
    if (h->method != kPoca && h->lists == kListsMuonMajor && h->fused_variant == kFusedVariants) {
        out->muon_pass = 5;
        out->muon_group = h->scatter_group;
        out->tile_pairs = h->scatter_depth;
        out->tile_muons = h->overlap ? muto_handle::kOverlapChunks : 0;
    } else if (h->method != kPoca && h->lists == kListsMuonMajor) {
        const bool staged = h->fused_variant == kFusedStaged;
        out->muon_pass = staged ? 6 : 3;
        out->muon_group = fused_variant_group(h->fused_variant);
        out->tile_pairs = staged ? 32 * fused_variant_held(h->fused_variant) : fused_variant_held(h->fused_variant);
        out->tile_muons = 32;
    } else if (h->method != kPoca && h->lists == kListsRecompute) {
        out->muon_pass = 4;
        out->muon_group = 1;
        out->tile_pairs = 0;
        out->tile_muons = 0;
    }
    std::snprintf(out->message, sizeof(out->message), "%s", h->last_msg.c_str());
    return MUTO_OK;
}

int muto_set_initial_image(muto_handle* h, const double* img, const muto_grid* grid) {
    if (!h) return MUTO_ERR_ARG;
    return guarded(h, [&] {
        if (h->prepared) throw Error(MUTO_ERR_STATE, "initial image must be set before prepare");
        h->init_set = true;
        if (!img || !grid) {
            h->init_missing = true;
            h->init_img.clear();
            return;
        }
        const uint64_t V = static_cast<uint64_t>(grid->nx) * grid->ny * grid->nz;
        if (V == 0) throw Error(MUTO_ERR_ARG, "empty initial image grid");
        h->init_missing = false;
        h->init_grid = *grid;
        h->init_img.assign(img, img + V);
    });
}

int muto_load_tracks(muto_handle* h, const muto_ray* rays, uint64_t n, int on_device) {
    if (!h) return MUTO_ERR_ARG;
    return guarded(h, [&] {
        if (n > 0 && !rays) throw Error(MUTO_ERR_ARG, "null rays");
        if (n >= 0xffffffffull) throw Error(MUTO_ERR_CAPACITY, "at most 2^32-1 tracks per handle");
        h->drop_graph();
        h->prepared = false;
        h->n_rays = n;
        {
            HostPhase ph(h, "load_alloc");
            h->rays.alloc(std::max<uint64_t>(n, 1) * sizeof(muto_ray), &h->dev_bytes);
        }
        HostPhase ph(h, "load_copy");
        if (n > 0)
            CK(cudaMemcpyAsync(h->rays.as<void>(), rays, n * sizeof(muto_ray),
                               on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    });
}

int muto_prepare(muto_handle* h) {
    if (!h) return MUTO_ERR_ARG;
    NvtxRange nv("muto_prepare");
    return guarded(h, [&] {
        if (h->rays.empty()) throw Error(MUTO_ERR_STATE, "load tracks first");
        for (const auto& r : h->batch_rays)
            if (!r || r->empty()) throw Error(MUTO_ERR_STATE, "load the tracks of every scan first");
        h->drop_graph();
        h->iters = 0;
        h->stopped = false;
        if (!h->batch) h->grid = h->P.grid;
        alloc_counters(h);
        const size_t pf = h->prof.used;
        if (h->method == kPoca) {
            prepare_poca(h);
        } else if (h->fp64()) {
            prepare_em<double>(h);
            if (h->lists == kListsVoxelMajor) {
                autotune_muon_pass<double>(h);
                autotune_voxel_pass<double>(h);
            } else {
                autotune_fused<double>(h);
            }
        } else {
            prepare_em<float>(h);
            if (h->lists == kListsVoxelMajor) {
                autotune_muon_pass<float>(h);
                autotune_voxel_pass<float>(h);
            } else {
                autotune_fused<float>(h);
            }
        }
        sync_and_harvest(h, pf);
        h->prepared = true;
    });
}

int muto_iterate(muto_handle* h, int n_iter) {
    if (!h) return MUTO_ERR_ARG;
    NvtxRange nv("muto_iterate");
    return guarded(h, [&] {
        n_prepared_check(h);
        if (h->method == kPoca) return;  // PoCA has no iterations
        if (n_iter < 0) throw Error(MUTO_ERR_ARG, "n_iter must be >= 0");
        if (h->fp64()) iterate_impl<double>(h, n_iter);
        else iterate_impl<float>(h, n_iter);
    });
}

int muto_get_image(muto_handle* h, double* out, uint64_t len) {
    if (!h || !out) return MUTO_ERR_ARG;
    return guarded(h, [&] {
        n_prepared_check(h);
        if (h->batch) throw Error(MUTO_ERR_STATE, "a batch handle returns images per scan (muto_batch_get_image)");
        if (len != h->V()) throw Error(MUTO_ERR_ARG, "image length does not match nx*ny*nz of the current grid");
        if (h->method == kPoca) {
            CK(cudaMemcpyAsync(out, h->img64.as<double>(), len * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
        } else if (h->fp64()) {
            download_image<double>(h, out);
        } else {
            download_image<float>(h, out);
        }
    });
}

int muto_set_image(muto_handle* h, const double* img, uint64_t len) {
    if (!h || !img) return MUTO_ERR_ARG;
    return guarded(h, [&] {
        n_prepared_check(h);
        if (h->method == kPoca) throw Error(MUTO_ERR_STATE, "PoCA has no iterate image");
        if (len != h->V()) throw Error(MUTO_ERR_ARG, "image length does not match nx*ny*nz of the current grid");
        if (h->fp64()) upload_image<double>(h, img);
        else upload_image<float>(h, img);
    });
}

int muto_reconstruct(muto_handle* h, const muto_ray* rays, uint64_t n, double* out_img, uint64_t out_len) {
    if (!h) return MUTO_ERR_ARG;
    int rc = muto_load_tracks(h, rays, n, 0);
    if (rc) return rc;
    rc = muto_prepare(h);
    if (rc) return rc;
    if (h->method != kPoca) {
        rc = muto_iterate(h, h->P.num_iteration);
        if (rc) return rc;
    }
    return muto_get_image(h, out_img, out_len);
}

int muto_select_probe(int precision, const double* values, uint64_t n, const uint64_t* seg_off, uint32_t n_segs,
                      int update_with_mean, int mean_percentile, long long stream_above, uint32_t repeat,
                      double* out) {
    if ((n > 0 && !values) || !seg_off || (n_segs > 0 && !out) || (precision != 0 && precision != 1) ||
        mean_percentile < 0 || mean_percentile > 100 || n > 0xffffffffull || repeat < 1)
        return MUTO_ERR_ARG;
    const int mode = !update_with_mean ? kVoxMedian : (mean_percentile == 100 ? kVoxMean : kVoxPercentile);
    return guarded(nullptr, [&] {
        if (n_segs == 0) return;
        const uint32_t streamed =
            stream_above < 0 ? 0u : vox_streamed_mask(static_cast<uint32_t>(std::min<long long>(stream_above, 0xffffffffLL)));
        if (precision == 1)
            select_probe_run<double>(values, n, seg_off, n_segs, mode, mean_percentile, streamed, repeat, out);
        else
            select_probe_run<float>(values, n, seg_off, n_segs, mode, mean_percentile, streamed, repeat, out);
    });
}

int muto_siddon_batch(const muto_grid* g, const double* p1, const double* p2, uint64_t n, uint32_t cap, uint32_t* xyz,
                      double* len, uint32_t* counts) {
    if (!g || (n > 0 && (!p1 || !p2 || !counts)) || (cap > 0 && n > 0 && (!xyz || !len))) return MUTO_ERR_ARG;
    return guarded(nullptr, [&] {
        if (n == 0) return;
        OwnedStream owned;
        cudaStream_t s = owned.s;
        DevMem d1, d2, dx, dl, dc;
        d1.alloc(n * 3 * sizeof(double), nullptr);
        d2.alloc(n * 3 * sizeof(double), nullptr);
        dx.alloc(std::max<uint64_t>(n * cap, 1) * 3 * sizeof(uint32_t), nullptr);
        dl.alloc(std::max<uint64_t>(n * cap, 1) * sizeof(double), nullptr);
        dc.alloc(n * sizeof(uint32_t), nullptr);
        if (cap > 0) {  // slots past a ray's count read as 0
            CK(cudaMemsetAsync(dx.as<void>(), 0, n * cap * 3 * sizeof(uint32_t), s));
            CK(cudaMemsetAsync(dl.as<void>(), 0, n * cap * sizeof(double), s));
        }
        CK(cudaMemcpyAsync(d1.as<void>(), p1, n * 3 * sizeof(double), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d2.as<void>(), p2, n * 3 * sizeof(double), cudaMemcpyHostToDevice, s));
        launch_siddon_batch(*g, d1.as<double>(), d2.as<double>(), n, cap, dx.as<uint32_t>(), dl.as<double>(),
                            dc.as<uint32_t>(), s);
        CK(cudaGetLastError());
        if (cap > 0) {
            CK(cudaMemcpyAsync(xyz, dx.as<void>(), n * cap * 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpyAsync(len, dl.as<void>(), n * cap * sizeof(double), cudaMemcpyDeviceToHost, s));
        }
        CK(cudaMemcpyAsync(counts, dc.as<void>(), n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    });
}

int muto_export_paths(muto_handle* h, uint32_t* kept, double* info, uint64_t* off, uint32_t* idx, double* len,
                      double* tail) {
    if (!h) return MUTO_ERR_ARG;
    return guarded(h, [&] {
        n_prepared_check(h);
        if (h->method == kPoca) throw Error(MUTO_ERR_STATE, "PoCA stores no paths");
        if (h->lists == kListsRecompute && (idx || len || tail || off))
            throw Error(MUTO_ERR_STATE, "path_lists \"recompute\" stores no paths");
        cudaStream_t s = h->stream;
        const uint64_t N = h->N, Pn = h->npairs;
        if (kept && N) CK(cudaMemcpyAsync(kept, h->kept.as<void>(), N * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        if (off) CK(cudaMemcpyAsync(off, h->off.as<void>(), (N + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        if (idx && Pn) {
            if (h->brick) {  // the stored indices are bricked
                DevMem tmp;
                tmp.alloc(Pn * sizeof(uint32_t), nullptr);
                launch_unbrick_indices(h->vidx.as<uint32_t>(), tmp.as<uint32_t>(), Pn, h->bdims, s);
                CK(cudaMemcpyAsync(idx, tmp.as<void>(), Pn * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
                CK(cudaStreamSynchronize(s));
            } else {
                CK(cudaMemcpyAsync(idx, h->vidx.as<void>(), Pn * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
            }
        }
        auto fetch = [&](const DevMem& m, double* dst, uint64_t count) {
            if (!dst || count == 0) return;
            if (h->fp64()) {
                CK(cudaMemcpyAsync(dst, m.as<void>(), count * sizeof(double), cudaMemcpyDeviceToHost, s));
            } else {
                std::vector<float> tmp(count);
                CK(cudaMemcpyAsync(tmp.data(), m.as<void>(), count * sizeof(float), cudaMemcpyDeviceToHost, s));
                CK(cudaStreamSynchronize(s));
                for (uint64_t k = 0; k < count; ++k) dst[k] = tmp[k];
            }
        };
        fetch(h->L, len, Pn);
        fetch(h->T, tail, Pn);
        if (info && N) {
            std::vector<double> pr(N);
            CK(cudaMemcpyAsync(pr.data(), h->pr64.as<void>(), N * sizeof(double), cudaMemcpyDeviceToHost, s));
            std::vector<double> sd(4 * N);
            if (h->fp64()) {
                CK(cudaMemcpyAsync(sd.data(), h->sd.as<void>(), 4 * N * sizeof(double), cudaMemcpyDeviceToHost, s));
                CK(cudaStreamSynchronize(s));
            } else {
                std::vector<float> t(4 * N);
                CK(cudaMemcpyAsync(t.data(), h->sd.as<void>(), 4 * N * sizeof(float), cudaMemcpyDeviceToHost, s));
                CK(cudaStreamSynchronize(s));
                for (uint64_t k = 0; k < 4 * N; ++k) sd[k] = t[k];
            }
            for (uint64_t i = 0; i < N; ++i) {  // stored as (Sx, Dx, Sy, Dy)
                info[6 * i + 0] = sd[4 * i + 0];
                info[6 * i + 1] = sd[4 * i + 2];
                info[6 * i + 2] = sd[4 * i + 1];
                info[6 * i + 3] = sd[4 * i + 3];
                info[6 * i + 4] = pr[i];
                info[6 * i + 5] = 0.0;
            }
        }
        CK(cudaStreamSynchronize(s));
    });
}

int muto_poca_assignment(muto_handle* h, int64_t* assign, uint64_t n) {
    if (!h || !assign) return MUTO_ERR_ARG;
    return guarded(h, [&] {
        n_prepared_check(h);
        if (h->method != kPoca) throw Error(MUTO_ERR_STATE, "only PoCA bins PoCA points");
        if (n != h->n_rays) throw Error(MUTO_ERR_ARG, "n must equal the number of loaded tracks");
        if (n) CK(cudaMemcpy(assign, h->assign.as<void>(), n * 3 * sizeof(long long), cudaMemcpyDeviceToHost));
    });
}

int muto_get_multiplicity(muto_handle* h, uint32_t* out, uint64_t len) {
    if (!h || !out) return MUTO_ERR_ARG;
    return guarded(h, [&] {
        n_prepared_check(h);
        if (h->method == kPoca) throw Error(MUTO_ERR_STATE, "PoCA has no multiplicity");
        if (len != h->V()) throw Error(MUTO_ERR_ARG, "length does not match nx*ny*nz");
        CK(cudaMemcpy(out, h->mult.as<void>(), len * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    });
}

int muto_nll_forward(muto_handle* h, const double* log_lambda, double* out_value) {
    if (!h || !log_lambda || !out_value) return MUTO_ERR_ARG;
    return guarded(h, [&] {
        n_prepared_check(h);
        if (h->method == kPoca) throw Error(MUTO_ERR_STATE, "PoCA has no likelihood");
        *out_value = h->fp64() ? nll_eval<double>(h, log_lambda, nullptr) : nll_eval<float>(h, log_lambda, nullptr);
    });
}

int muto_nll_backward(muto_handle* h, const double* log_lambda, double* out_value, double* out_grad) {
    if (!h || !log_lambda || !out_grad) return MUTO_ERR_ARG;
    return guarded(h, [&] {
        n_prepared_check(h);
        if (h->method == kPoca) throw Error(MUTO_ERR_STATE, "PoCA has no likelihood");
        const double v = h->fp64() ? nll_eval<double>(h, log_lambda, out_grad) : nll_eval<float>(h, log_lambda, out_grad);
        if (out_value) *out_value = v;
    });
}

int muto_gradient_solve(muto_handle* h, int n_iter, double* out_value) {
    return muto_gradient_solve_until(h, n_iter, -HUGE_VAL, out_value, nullptr);
}

int muto_gradient_solve_until(muto_handle* h, int max_iter, double target, double* out_value, int* out_iters) {
    if (!h) return MUTO_ERR_ARG;
    const int n_iter = max_iter;
    if (out_iters) *out_iters = 0;
    return guarded(h, [&] {
        n_prepared_check(h);
        if (h->method == kPoca) throw Error(MUTO_ERR_STATE, "PoCA has no likelihood");
        const uint64_t V = h->V();
        std::vector<double> lam(V), x(V), g(V), xt(V);
        std::vector<uint32_t> M(V);
        if (h->fp64()) download_image<double>(h, lam.data());
        else download_image<float>(h, lam.data());
        CK(cudaMemcpy(M.data(), h->mult.as<void>(), V * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        const double floor_l = 1e-12;
        for (uint64_t j = 0; j < V; ++j) x[j] = std::log(std::max(lam[j], floor_l));
        auto F = [&](const std::vector<double>& xx, std::vector<double>* gg) {
            if (gg) return h->fp64() ? nll_eval<double>(h, xx.data(), gg->data()) : nll_eval<float>(h, xx.data(), gg->data());
            return h->fp64() ? nll_eval<double>(h, xx.data(), nullptr) : nll_eval<float>(h, xx.data(), nullptr);
        };
        double f = F(x, &g);
        double step = 1.0;
        int done = 0;
        for (int it = 0; it < n_iter && !(f <= target); ++it) {
            // step preconditioned by 1/(2 M_j): at step 1 it is the mean-mode EM move in log space
            double slope = 0.0;
            for (uint64_t j = 0; j < V; ++j) {
                if (!M[j]) continue;
                const double d = -g[j] / (2.0 * M[j]);
                slope += g[j] * d;
            }
            if (slope >= 0) break;
            double ft = f;
            bool accepted = false;
            for (int ls = 0; ls < 30; ++ls) {
                for (uint64_t j = 0; j < V; ++j) xt[j] = M[j] ? x[j] - step * g[j] / (2.0 * M[j]) : x[j];
                ft = F(xt, nullptr);
                if (ft <= f + 1e-4 * step * slope) {
                    accepted = true;
                    break;
                }
                step *= 0.5;
            }
            if (!accepted) break;
            x.swap(xt);
            f = F(x, &g);
            step = std::min(step * 2.0, 4.0);
            done = it + 1;
        }
        if (out_iters) *out_iters = done;
        for (uint64_t j = 0; j < V; ++j) lam[j] = M[j] ? std::exp(x[j]) : 0.0;
        if (h->fp64()) upload_image<double>(h, lam.data());
        else upload_image<float>(h, lam.data());
        if (out_value) *out_value = f;
    });
}

int muto_set_profiling(muto_handle* h, int enable) {
    if (!h) return MUTO_ERR_ARG;
    return guarded(h, [&] {
        if (h->prof.on != (enable != 0)) h->drop_graph();  // recapture with / without event nodes
        h->prof.on = enable != 0;
    });
}

int muto_kernel_stats(muto_handle* h, const char* name, uint64_t* launches, double* total_ms) {
    if (!h || !name) return MUTO_ERR_ARG;
    auto it = h->prof.stats.find(name);
    if (launches) *launches = it == h->prof.stats.end() ? 0 : it->second.first;
    if (total_ms) *total_ms = it == h->prof.stats.end() ? 0.0 : it->second.second;
    return MUTO_OK;
}

int muto_reset_kernel_stats(muto_handle* h) {
    if (!h) return MUTO_ERR_ARG;
    h->prof.stats.clear();
    return MUTO_OK;
}

int muto_launch_count(muto_handle* h, uint64_t* out) {
    if (!h || !out) return MUTO_ERR_ARG;
    *out = h->launches;
    return MUTO_OK;
}

int muto_batch_create(const char* method, const char* config_json, uint32_t n_scans, const muto_grid* grids,
                      muto_handle** out) {
    if (!method || !out || !grids || n_scans == 0) return MUTO_ERR_ARG;
    *out = nullptr;
    if (std::string(method) != "mlsd") return MUTO_ERR_ARG;  // MAP stencils need one grid
    muto_handle* h = nullptr;
    int rc = muto_create(method, config_json, &h);
    if (rc != MUTO_OK) return rc;
    rc = guarded(h, [&] {
        if (h->P.initialize_method == 0)
            throw Error(MUTO_ERR_CONFIG, "a batch starts from initialize_method 1 or 2 (no per-scan image files)");
        if (h->P.early_stop) throw Error(MUTO_ERR_CONFIG, "early_stop applies to one scan, not to a batch");
        h->batch = true;
        h->scans.resize(n_scans);
        for (uint32_t k = 0; k < n_scans; ++k) {
            const muto_grid& g = grids[k];
            if (g.nx == 0 || g.ny == 0 || g.nz == 0 || !(g.dx > 0 && g.dy > 0 && g.dz > 0))
                throw Error(MUTO_ERR_ARG, "scan " + std::to_string(k) + ": invalid grid");
            h->scans[k].grid = g;
        }
        h->grid = grids[0];
        h->batch_rays.resize(n_scans - 1);
    });
    if (rc != MUTO_OK) {
        muto_destroy(h);
        return rc;
    }
    *out = h;
    return MUTO_OK;
}

int muto_batch_load_tracks(muto_handle* h, uint32_t scan, const muto_ray* rays, uint64_t n, int on_device) {
    if (!h) return MUTO_ERR_ARG;
    if (!h->batch) return scan == 0 ? muto_load_tracks(h, rays, n, on_device) : MUTO_ERR_ARG;
    if (scan >= h->scans.size()) return MUTO_ERR_ARG;
    if (scan == 0) {
        const int rc = muto_load_tracks(h, rays, n, on_device);
        if (rc == MUTO_OK) h->scans[0].n_rays = n;
        return rc;
    }
    return guarded(h, [&] {
        if (n > 0 && !rays) throw Error(MUTO_ERR_ARG, "null rays");
        if (n >= 0xffffffffull) throw Error(MUTO_ERR_CAPACITY, "at most 2^32-1 tracks per scan");
        h->drop_graph();
        h->prepared = false;
        auto& slot = h->batch_rays[scan - 1];
        slot.reset(new DevMem());
        slot->alloc(std::max<uint64_t>(n, 1) * sizeof(muto_ray), &h->dev_bytes);
        if (n > 0)
            CK(cudaMemcpyAsync(slot->as<void>(), rays, n * sizeof(muto_ray),
                               on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        h->scans[scan].n_rays = n;
    });
}

int muto_batch_get_image(muto_handle* h, uint32_t scan, double* out, uint64_t len) {
    if (!h || !out) return MUTO_ERR_ARG;
    if (!h->batch) return scan == 0 ? muto_get_image(h, out, len) : MUTO_ERR_ARG;
    return guarded(h, [&] {
        n_prepared_check(h);
        if (scan >= h->scans.size()) throw Error(MUTO_ERR_ARG, "no such scan");
        const auto& sc = h->scans[scan];
        if (len != sc.V) throw Error(MUTO_ERR_ARG, "image length does not match the scan's grid");
        const size_t es = h->fp64() ? sizeof(double) : sizeof(float);
        std::vector<unsigned char> tmp(len * es);
        CK(cudaMemcpyAsync(tmp.data(), static_cast<const unsigned char*>(h->lam.as<void>()) + sc.voff * es, len * es,
                           cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        for (uint64_t j = 0; j < len; ++j)
            out[j] = h->fp64() ? reinterpret_cast<const double*>(tmp.data())[j]
                               : static_cast<double>(reinterpret_cast<const float*>(tmp.data())[j]);
    });
}

int muto_batch_scan_info(muto_handle* h, uint32_t scan, uint64_t* kept, uint64_t* pairs) {
    if (!h) return MUTO_ERR_ARG;
    return guarded(h, [&] {
        n_prepared_check(h);
        if (scan >= h->scans.size()) throw Error(MUTO_ERR_ARG, "no such scan");
        const auto& sc = h->scans[scan];
        std::vector<uint64_t> o(2);
        CK(cudaMemcpy(&o[0], h->off.as<uint64_t>() + sc.noff, sizeof(uint64_t), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&o[1], h->off.as<uint64_t>() + sc.noff + sc.N, sizeof(uint64_t), cudaMemcpyDeviceToHost));
        if (kept) *kept = sc.N;
        if (pairs) *pairs = o[1] - o[0];
    });
}

int muto_get_stream(muto_handle* h, void** out) {
    if (!h || !out) return MUTO_ERR_ARG;
    *out = static_cast<void*>(h->stream);
    return MUTO_OK;
}

int muto_generate_device(const muto_grid* g, const double* lambda_dev, const muto_gen_params* p, uint64_t first,
                         uint64_t n, muto_ray* out_dev, void* stream) {
    if (!g || !lambda_dev || !p || (n && !out_dev)) return MUTO_ERR_ARG;
    if (!gen::params_ok(*p)) return MUTO_ERR_ARG;
    return guarded(nullptr, [&] {
        launch_generate(*g, lambda_dev, *p, first, n, out_dev, static_cast<cudaStream_t>(stream));
        CK(cudaGetLastError());
    });
}

int muto_fit_tracks(const void* records, int precision, uint64_t n, const double* z_layers, int nz, int n_middle,
                    muto_ray* out, uint64_t* n_out) {
    if (!n_out || !z_layers || (n > 0 && (!records || !out))) return MUTO_ERR_ARG;
    if (precision != 4 && precision != 8) return MUTO_ERR_ARG;
    if (nz > static_cast<int>(sizeof(FitLayers::z) / sizeof(double)) || n_middle < 2 || nz - n_middle < 2)
        return MUTO_ERR_ARG;
    return guarded(nullptr, [&] {
        *n_out = 0;
        if (n == 0) return;
        FitLayers zl{};
        for (int i = 0; i < nz; ++i) zl.z[i] = z_layers[i];
        zl.nz = nz;
        zl.n_middle = n_middle;
        const uint64_t rec_bytes = (2 * static_cast<uint64_t>(nz) + 2) * static_cast<uint64_t>(precision);
        const uint64_t chunk = std::min<uint64_t>(n, uint64_t(1) << 20);  // records per round trip
        OwnedStream owned;
        cudaStream_t s = owned.s;
        DevMem rec, all, keep, pos, scr, kept;
        rec.alloc(chunk * rec_bytes, nullptr);
        all.alloc(chunk * sizeof(muto_ray), nullptr);
        keep.alloc(chunk * sizeof(uint32_t), nullptr);
        pos.alloc((chunk + 1) * sizeof(uint64_t), nullptr);
        scr.alloc(scan_scratch_bytes(chunk), nullptr);
        kept.alloc(chunk * sizeof(muto_ray), nullptr);
        uint64_t written = 0;
        for (uint64_t r0 = 0; r0 < n; r0 += chunk) {
            const uint64_t m = std::min(chunk, n - r0);
            CK(cudaMemcpyAsync(rec.as<void>(), static_cast<const char*>(records) + r0 * rec_bytes, m * rec_bytes,
                               cudaMemcpyHostToDevice, s));
            launch_fit_records(rec.as<void>(), precision, m, zl, all.as<muto_ray>(), keep.as<uint32_t>(),
                               pos.as<uint64_t>(), scr.as<void>(), kept.as<muto_ray>(), s);
            CK(cudaGetLastError());
            uint64_t k = 0;
            CK(cudaMemcpyAsync(&k, pos.as<uint64_t>() + m, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (k) CK(cudaMemcpyAsync(out + written, kept.as<void>(), k * sizeof(muto_ray), cudaMemcpyDeviceToHost, s));
            written += k;
        }
        CK(cudaStreamSynchronize(s));
        *n_out = written;
    });
}

}  // extern "C"
