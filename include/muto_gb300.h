/*
 * muto_gb300.h -- C ABI of the GB300 muon-tomography reconstruction library.
 *
 * The library replaces the reconstruction path of LasDes/MuonTomography:
 *   MutoVReconstruction::reconstruct   include/MutoVReconstruction.h:16
 *   MutoPoCA(json)  / reconstruct      include/MutoPoCA.h:23,28   src/MutoPoCA.cpp:24, :51-134
 *   MutoMLSD(json)  / reconstruct      include/MutoMLSD.h:33,38   src/MutoMLSD.cpp:47-220
 *   MutoMAP(json)   / reconstruct      include/MutoMAP.h:22,27    src/MutoMAP.cpp:12, :39-205
 *   MutoSiddon::getVoxelPath           include/MutoSiddon.h:24    src/MutoSiddon.cpp:9-141
 *   MutoFile::saveImage / loadImage    include/MutoFile.h:49,59   src/MutoFile.cpp:85-211
 *
 * Conventions
 *  - Every function returns MUTO_OK (0) or a MUTO_ERR_* code; no exception
 *    or C++ type crosses this boundary.  The handle's last error text is in
 *    muto_status.message.
 *  - Images are column-major doubles, x fastest: voxel (x,y,z) is element
 *    x + nx*(y + ny*z)  (include/MutoMLSD.h:76).
 *  - Tracks are the reference's RayData layout: 14 doubles per muon
 *    {ein, eout, pin[3], pout[3], din[3], dout[3]} (include/MutoTypes.h:47-54).
 *  - A handle owns one CUDA stream and its device buffers.  A handle is not
 *    thread-safe; different handles are independent.
 */
#ifndef MUTO_GB300_H
#define MUTO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MUTO_OK = 0,
    MUTO_ERR_ARG = 1,      /* null pointer, size mismatch, unknown name */
    MUTO_ERR_CONFIG = 2,   /* malformed JSON or a key of the wrong type / range */
    MUTO_ERR_CUDA = 3,     /* a CUDA runtime call failed (message has the CUDA error) */
    MUTO_ERR_STATE = 4,    /* call made in the wrong order (e.g. iterate before prepare) */
    MUTO_ERR_CAPACITY = 5, /* a documented size limit was exceeded */
    MUTO_ERR_IO = 6,       /* file could not be opened / read / written */
    MUTO_ERR_NOMEM = 7     /* device or host allocation failed */
};

/* VoxelGrid, include/MutoTypes.h:25-37 (pad keeps the doubles 8-byte aligned) */
typedef struct muto_grid {
    uint32_t nx, ny, nz, pad;
    double x_min, y_min, z_min;
    double dx, dy, dz;
} muto_grid;

/* RayData, include/MutoTypes.h:47-54 */
typedef struct muto_ray {
    double ein, eout;
    double pin[3], pout[3], din[3], dout[3];
} muto_ray;

typedef struct muto_status {
    int32_t last_error;         /* MUTO_* code of the last failing call, 0 if none */
    int32_t iterations_done;    /* EM / MAP iterations run since prepare */
    int32_t early_stopped;      /* 1 when early_stop ended the iterations */
    int32_t precision;          /* 0 = mixed (FP32 lists/accumulation), 1 = fp64 */
    uint64_t n_total;           /* rays considered (fNTotal) */
    uint64_t n_scat_in_grid;    /* muons kept (fNScatInGrid) */
    uint64_t n_not_parallel;    /* PoCA: rays whose in/out lines are not parallel */
    uint64_t n_pairs;           /* muon-voxel pairs on the stored paths */
    uint64_t n_singular;        /* covariance matrices found singular (all iterations) */
    uint64_t n_nonconverged;    /* MAP cubic solves stopped by the Newton iteration cap */
    uint64_t n_bounds;          /* path voxels outside the grid (skipped) */
    uint64_t n_path_overflow;   /* Siddon walks stopped by the step bound */
    double cost;                /* mean cost of the last iteration (when computed) */
    double cost_prev;           /* mean cost of the iteration before */
    uint64_t device_bytes;      /* device memory held by the handle */
    int32_t muon_pass;          /* muon-pass variant in use: 1 TMA tiles, 2 warp-batched, 3 the mean
                                   update's one-pass form over stored lists, 4 its pass over recomputed
                                   paths, 5 its split form (warp-batched muon pass, then a scatter pass),
                                   6 its one-pass form with each batch's pairs staged in shared memory */
    int32_t muon_group;         /* lanes per muon in its covariance sums */
    int32_t tile_pairs;         /* pairs per tile (TMA variant), pairs per muon held in registers
                                   (fused stored-list pass), pairs staged per batch (staged pass),
                                   pairs in flight per lane (split form's scatter); 0 otherwise */
    int32_t tile_muons;         /* muons per tile (TMA variant), muons per CTA batch (fused pass),
                                   chunks of muons whose muon pass and scatter overlap (split form;
                                   0: not overlapped) */
    int32_t path_lists;         /* how the pairs are kept: 1 muon-major lists and their voxel-major copy,
                                   2 muon-major lists only, 3 none (paths walked every iteration);
                                   0 for the one-shot methods */
    int32_t voxel_stream_above; /* voxel pass in use: segments longer than this are selected from the
                                   key array instead of registers (-1: none); "auto" picks it */
    int32_t slr_levels;         /* slr_iter: levels of the later passes' schedule (muons of one level
                                   share no voxel); 0 when they run muon after muon or not at all */
    int32_t reserved;
    char message[256];          /* text of the last error */
} muto_status;

typedef struct muto_handle muto_handle;

/* ---------------------------------------------------------------------------
 * Reconstruction handles
 * ------------------------------------------------------------------------- */

/* Create a reconstruction: method is "poca", "pocut", "slr", "slr_iter",
 * "mlsd" or "map"; config_json is the JSON object of that method (the value
 * of the key of the same name, as passed to the constructors MutoPoCA(json)
 * src/MutoPoCA.cpp:24, MutoPoCut(json) src/MutoPoCut.cpp:12 (PoCA's keys
 * plus "cut_percentile", 1.0; straight_line is always off), MutoSLR(json)
 * src/MutoSLR.cpp:21, MutoSLRIter(json) src/MutoSLRIter.cpp:9 (plus
 * "num_iteration", 1), MutoMLSD(json) src/MutoMLSD.cpp:47, MutoMAP(json)
 * src/MutoMAP.cpp:12).  poca, pocut, slr and slr_iter compute their image in
 * muto_prepare.
 * The reference's keys and defaults apply; extra keys: "precision"
 * ("mixed" default, or "fp64"), "use_graph" (true), "random_seed",
 * "compute_cost" (computed when early_stop/log_results is set, or when true),
 * "newton_max_iter" (MAP cubic cap, 200), "tile_pairs" (pairs per TMA tile),
 * "muon_pass" ("auto": the warp-batched variant, its group size chosen by
 * timing on the scan's data at prepare and reused for later scans of the
 * same shape in the process; "tile" or "warp" force one),
 * "muon_layout" ("auto": the per-muon coefficient table in column order of
 * the muons' PoCA points when it would take more than a third of L2, else
 * in muon order; "columns" or "index" force one),
 * "voxel_stream_above" (-1: every segment up to 1536 pairs (768 in fp64)
 * is selected from registers; n >= 256: segments longer than n are
 * selected without holding their keys; "auto": -1 or 512, whichever is
 * faster on the scan's own lists, timed at prepare and reused for later
 * scans of the same shape in the process),
 * "path_lists" (how the muon-voxel pairs are kept: "voxel_major" -- the
 * muon-major lists plus a voxel-major copy, which the median and
 * percentile updates need; "muon_major" -- the muon-major lists alone
 * (12 bytes per pair mixed, 20 fp64), with the mean update's per-voxel
 * sums formed by reductions to global memory; "recompute" -- no lists,
 * every path walked again (FP64, bit-exact walk) twice per iteration, one
 * scan per handle; "auto" (default): "muon_major" for the mean update
 * (update_with_mean true, mean_percentile 100), else "voxel_major";
 * "muon_major" and "recompute" require the mean update),
 * "fused_variant" ("auto": the mean update's pass over muon-major lists
 * takes the lanes per muon and pairs held per lane by timing the variants
 * that suit the scan's mean path and the split form (the muon pass, then a
 * second pass over the lists adding the terms) at prepare; "4x8", "8x4",
 * "8x8", "8x16", "16x8", "16x16", "split", "split8" (its scatter with 8
 * pairs in flight per lane), "split8_overlap" (the same, the scatter of one
 * chunk of muons running beside the muon pass of the next) or "staged"
 * (each batch's pairs
 * copied to shared memory once and read back there for the second step)
 * force one), "fused_prefetch"
 * (false; true: the one-pass form
 * prefetches every CTA's next batch of pairs into L2),
 * "setup_chunk_pairs" (0: the set-up walks the paths in chunks of muons
 * whose bounded slots take at most a quarter of the free device memory,
 * 12 GiB at most; n > 0: chunks of at most n bounded pairs),
 * "slr_iter_schedule" (slr_iter only: "levels", the default, runs the later
 * passes level by level, muons that share no voxel at once, each voxel
 * meeting its muons in index order; "sequential" runs them muon after
 * muon). */
int muto_create(const char* method, const char* config_json, muto_handle** out);
int muto_destroy(muto_handle* h);

/* getCurrentGrid(), include/MutoMLSD.h:41 / include/MutoPoCA.h:31 */
int muto_get_grid(const muto_handle* h, muto_grid* out);
int muto_get_status(const muto_handle* h, muto_status* out);

/* Initial image for initialize_method 0 (src/MutoMLSD.cpp:228-245): the
 * image read from initial_image_file.  When grid differs from the
 * configured nx/ny/nz the handle adopts it, as the reference does.
 * img may be NULL to say "file missing" (the reference then falls back to
 * random initialisation). */
int muto_set_initial_image(muto_handle* h, const double* img, const muto_grid* grid);

/* MutoVReconstruction::reconstruct (include/MutoVReconstruction.h:16): host
 * tracks in, host image out (out_len must equal nx*ny*nz of the current
 * grid).  Equivalent to load_tracks + prepare + iterate(num_iteration) +
 * get_image. */
int muto_reconstruct(muto_handle* h, const muto_ray* rays, uint64_t n, double* out_img, uint64_t out_len);

/* Staged form of the same work.  on_device != 0: rays is a device pointer
 * (it is copied; the caller keeps ownership). */
int muto_load_tracks(muto_handle* h, const muto_ray* rays, uint64_t n, int on_device);
/* PoCA: runs the whole method.  MLSD/MAP: gatherInformation + paths + W
 * setup (src/MutoMLSD.cpp:99-152) and the initial image. */
int muto_prepare(muto_handle* h);
/* MLSD/MAP: n_iter more iterations (src/MutoMLSD.cpp:179-213,
 * src/MutoMAP.cpp:192-261); stops early when early_stop triggers. */
int muto_iterate(muto_handle* h, int n_iter);
int muto_get_image(muto_handle* h, double* out_img, uint64_t out_len);
/* Replace the current image lambda (host, nx*ny*nz doubles). */
int muto_set_image(muto_handle* h, const double* img, uint64_t len);

/* ---------------------------------------------------------------------------
 * Parity probes
 * ------------------------------------------------------------------------- */

/* Batched MutoSiddon::getVoxelPath (src/MutoSiddon.cpp:9-141) on the GPU.
 * Host buffers.  Ray r's voxels go to xyz[(r*cap+k)*3 + {0,1,2}] and
 * len[r*cap+k] for k < min(counts[r], cap); counts[r] is the full count;
 * the slots past it are 0. */
int muto_siddon_batch(const muto_grid* g, const double* p1, const double* p2, uint64_t n, uint32_t cap,
                      uint32_t* xyz, double* len, uint32_t* counts);

/* The same batched Siddon walk without any allocation.  No counterpart in
 * the reference.
 *
 * For callers that cannot let a library allocate device memory: a process
 * whose device memory is all reserved up front by its own pool allocator
 * has none left to give, and a loop that keeps other streams of the device
 * busy (data acquisition, online monitoring) cannot take the device-wide
 * synchronisation that cudaFree performs.  Inputs, outputs and errors are
 * those of muto_siddon_batch, plus MUTO_ERR_CAPACITY for cap; this call
 * keeps no handle, so a failure is reported by its return code alone.
 * The work runs on `stream` (a cudaStream_t; NULL is the legacy default
 * stream) and the call returns when it is done, also when it fails after
 * queuing work (it then waits for the queued work before returning).
 *
 * Instead of allocating, the call stages rays and voxel lists, a chunk of
 * rays at a time, through one fixed device array of
 * MUTO_NOALLOC_SCRATCH_BYTES compiled into the library.  n is unbounded;
 * cap above MUTO_NOALLOC_MAX_CAP returns MUTO_ERR_CAPACITY before the
 * device is touched.  The first call on a device looks up the array's
 * address on that device (the current one) and keeps it for the rest of
 * the process; make that first call before any stream capture begins.  The
 * kept address is not valid after cudaDeviceReset, so do not use this call
 * in a process that resets a device it has called it on.  All calls on one device share the array:
 * calls that overlap in time (several host threads, or several streams)
 * race on it, so the caller must serialise them. */
#define MUTO_NOALLOC_SCRATCH_BYTES (16u << 20)
#define MUTO_NOALLOC_MAX_CAP 65536u
int muto_siddon_batch_noalloc(const muto_grid* g, const double* p1, const double* p2, uint64_t n, uint32_t cap,
                              uint32_t* xyz, double* len, uint32_t* counts, void* stream);

/* The voxel update of the EM step (src/MutoMLSD.cpp:493-517) on synthetic
 * segments, through the same kernels as an iteration: segment j holds
 * values[seg_off[j] .. seg_off[j+1]) and its pairs get s_i = 2 + x_i
 * (lambda = 1, L = 1, T = 0, per-muon coefficients (x_i, 0, 0)), computed
 * in float (precision 0) or double (1).  out[j] is the updated lambda of
 * segment j: the halved median of the s_i (even counts: the mean of the two
 * middle values), or with update_with_mean the halved mean of the lowest
 * mean_percentile % (100: all).  stream_above is the "voxel_stream_above"
 * key of the configuration (-1: never).  With repeat > 1, values holds
 * repeat * n values and the pass runs repeat times, pass r on values
 * [r*n, (r+1)*n), each starting from the selection windows the previous
 * pass left (as iterations do); out is the last pass's.  Not in the
 * reference: a probe that lets tests check the exact order statistics on
 * chosen inputs. */
int muto_select_probe(int precision, const double* values, uint64_t n, const uint64_t* seg_off, uint32_t n_segs,
                      int update_with_mean, int mean_percentile, long long stream_above, uint32_t repeat,
                      double* out);

/* MLSD/MAP after prepare: the kept muons and their merged paths
 * (src/MutoMLSD.cpp:268-326, :382-430).  Any pointer may be NULL.
 * kept: n_scat_in_grid ray indices; info: 6 doubles per kept muon
 * {Sx, Sy, Dx, Dy, pr, 0}; off: n_scat_in_grid+1 pair offsets;
 * idx/len/tail: n_pairs flat voxel index, L and T (in the stored precision). */
int muto_export_paths(muto_handle* h, uint32_t* kept, double* info, uint64_t* off, uint32_t* idx, double* len,
                      double* tail);

/* PoCA after prepare: the voxel each ray's PoCA point was binned to
 * (src/MutoPoCA.cpp:121-132), 3 int64 per ray, -1 when rejected. */
int muto_poca_assignment(muto_handle* h, int64_t* assign, uint64_t n);

/* ---------------------------------------------------------------------------
 * Adjoint: MLSD negative log-likelihood plus MAP prior (not in the reference)
 *
 * F(lambda) = sum_i [log det S_i + 1/2 sum_planes v^T S_i^-1 v]      (cost of
 *             src/MutoMLSD.cpp:465-468 summed over kept muons)
 *           + 2 * beta * sum_j sum_{m in N(j)} w_jm psi(l_j - l_m)
 *             [+ 2 * beta * sum_j psi(l_j) with add_object_prior]
 * with l = 1e7 * lambda, psi(t) = (t^2 + delta^2)^(p/2) and the neighbour
 * stencil, weights and edge clamping of src/MutoMAP.cpp:207-350.  The
 * prior is the one whose separable surrogate the MAP update minimises;
 * for method "mlsd" beta is 0.  Voxels with no pairs are held at 0.
 * log_lambda: nx*ny*nz doubles (host); entries of voxels without pairs are
 * ignored.  grad: d F / d log(lambda_j), nx*ny*nz doubles (host). */
int muto_nll_forward(muto_handle* h, const double* log_lambda, double* out_value);
int muto_nll_backward(muto_handle* h, const double* log_lambda, double* out_value, double* out_grad);

/* Gradient-based MAP solver beside the EM: n_iter iterations of
 * preconditioned gradient descent with backtracking on F over log(lambda),
 * starting from the current image.  Leaves the result as the image and the
 * final F in *out_value. */
int muto_gradient_solve(muto_handle* h, int n_iter, double* out_value);
/* The same solver stopped as soon as F <= target (or after max_iter
 * iterations, or when no step lowers F): *out_value is the F reached and
 * *out_iters (may be NULL) the iterations taken.  Used to run the solver
 * to the objective value an EM run reached. */
int muto_gradient_solve_until(muto_handle* h, int max_iter, double target, double* out_value, int* out_iters);

/* ---------------------------------------------------------------------------
 * Batches: many independent scans (each its own grid and tracks) in one
 * handle.  Their muons and voxels are concatenated, so every pass of an EM
 * iteration is one launch over all scans.  Not in the reference, which runs
 * one scan per process.  Method "mlsd" only; initialize_method 1 or 2; no
 * early_stop.  muto_prepare / muto_iterate / muto_get_status apply to the
 * whole batch; images are read per scan.
 * ------------------------------------------------------------------------- */
int muto_batch_create(const char* method, const char* config_json, uint32_t n_scans, const muto_grid* grids,
                      muto_handle** out);
int muto_batch_load_tracks(muto_handle* h, uint32_t scan, const muto_ray* rays, uint64_t n, int on_device);
int muto_batch_get_image(muto_handle* h, uint32_t scan, double* out_img, uint64_t out_len);
/* kept muons and muon-voxel pairs of one scan, after prepare */
int muto_batch_scan_info(muto_handle* h, uint32_t scan, uint64_t* kept, uint64_t* pairs);

/* ---------------------------------------------------------------------------
 * Multiplicity per voxel (number of pairs M_j), after prepare.
 * ------------------------------------------------------------------------- */
int muto_get_multiplicity(muto_handle* h, uint32_t* out, uint64_t len);

/* ---------------------------------------------------------------------------
 * Profiling: CUDA-event timing of every kernel launch on the handle's stream
 * ------------------------------------------------------------------------- */
int muto_set_profiling(muto_handle* h, int enable);
/* name: kernel family ("em_tile", "em_select", "em_voxel", "map_voxel",
 * "siddon_fill", ...).  Sums since the last reset. */
int muto_kernel_stats(muto_handle* h, const char* name, uint64_t* launches, double* total_ms);
int muto_reset_kernel_stats(muto_handle* h);
/* Kernel launches issued by the handle since creation. */
int muto_launch_count(muto_handle* h, uint64_t* out);

/* ---------------------------------------------------------------------------
 * Synthetic muon data (host, deterministic per (seed, muon index))
 * ------------------------------------------------------------------------- */
typedef struct muto_block {
    double lo[3], hi[3];   /* axis-aligned box, mm */
    double x0_mm;          /* radiation length of the material, mm */
} muto_block;

typedef struct muto_gen_params {
    uint64_t seed;
    double theta_max;      /* zenith cut, rad (cos^2 spectrum below it) */
    double p_min, p_max;   /* log-uniform momentum range, GeV/c */
    double p0;             /* nominal momentum of lambda, GeV/c (3) */
    double plane_gap;      /* detector plane spacing, mm (500) */
    int32_t n_planes;      /* planes above and below the grid (3) */
    int32_t pad;
    double hit_sigma;      /* hit smearing, mm (1) */
} muto_gen_params;

/* lambda of a material: (13.6 MeV / p0)^2 / X0  [rad^2/mm] */
double muto_lambda_from_x0(double x0_mm, double p0_gev);
/* Voxel-centre rasterisation of blocks over a background (later blocks win). */
int muto_phantom(const muto_grid* g, const muto_block* blocks, uint32_t n_blocks, double background_x0_mm,
                 double p0_gev, double* out_lambda);
/* Muons first..first+n-1 of the stream: transport through lambda with one
 * Gaussian (angle, displacement) kick per traversed voxel, detector hits
 * with smearing, least-squares in/out lines.  Host, OpenMP. */
int muto_generate(const muto_grid* g, const double* lambda, const muto_gen_params* p, uint64_t first, uint64_t n,
                  muto_ray* out);
/* The same generator on the GPU, one thread per muon: lambda_dev and
 * out_dev are device pointers; stream is a cudaStream_t (NULL: default).
 * Returns after the launch; synchronise on the stream before reading. */
int muto_generate_device(const muto_grid* g, const double* lambda_dev, const muto_gen_params* p, uint64_t first,
                         uint64_t n, muto_ray* out_dev, void* stream);

/* Batched line fit of raw detector records on the GPU, one thread per
 * record: the per-record step of MutoFile::getMuonData (src/MutoFile.cpp:
 * 58-78 and getRayDataFromTemp, :248-304).  records holds n records of
 * 2*nz+2 values {ein, x0, y0, ..., x_{nz-1}, y_{nz-1}, eout}, float32 when
 * precision is 4, float64 when 8, at z = z_layers[0..nz-1] (nz <= 64).
 * Layers 0..n_middle-1 give the incoming line and n_middle..nz-1 the
 * outgoing one (n_middle >= 2 and nz - n_middle >= 2): each line is the
 * principal axis of its hits (the first right singular vector the
 * reference takes from JacobiSVD), oriented with d_z > 0, with pin on
 * layer n_middle-1 and pout on layer n_middle.  Records holding a NaN are
 * dropped (:71-76).  Host buffers: out must hold n tracks; it receives the
 * kept records' tracks in record order and *n_out their number.  The
 * result is bit for bit that of muto_read_muon_data (include/muto_io.h),
 * which reads the same records from files on the host. */
int muto_fit_tracks(const void* records, int precision, uint64_t n, const double* z_layers, int nz, int n_middle,
                    muto_ray* out, uint64_t* n_out);

/* The handle's CUDA stream (a cudaStream_t), for callers that order their
 * own work (events, copies) with the handle's. */
int muto_get_stream(muto_handle* h, void** out);

/* ---------------------------------------------------------------------------
 * Image files: MutoFile format (64-byte header + column-major f32/f64),
 * src/MutoFile.cpp:85-211
 * ------------------------------------------------------------------------- */
int muto_save_image(const char* path, const double* img, const muto_grid* g, const char* method, uint32_t n_ray,
                    uint32_t n_iter, uint32_t precision);
/* Reads the header; then, when img != NULL and cap >= nx*ny*nz, the data. */
int muto_load_image(const char* path, double* img, uint64_t cap, muto_grid* g, char* method16, uint32_t* n_ray,
                    uint32_t* n_iter, uint32_t* precision);

/* Library version string. */
const char* muto_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MUTO_GB300_H */
