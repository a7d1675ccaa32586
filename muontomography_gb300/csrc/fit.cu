// Batched line fit of raw detector records: the per-record step of
// MutoFile::getMuonData (src/MutoFile.cpp:58-78 and :248-304), one thread
// per record, with the fit of trackfit.h (the host reader's, bit for bit).
// A chunk of records goes through three launches: the fit writes every
// record's track and a keep flag (0 for a record holding a NaN), a scan of
// the flags gives each kept record its slot, and a gather writes the kept
// tracks in record order.
#include "common.cuh"
#include "trackfit.h"

namespace muto {
namespace {

template <typename T>
__global__ void k_fit_records(const T* __restrict__ rec, uint64_t n, FitLayers zl, muto_ray* __restrict__ all,
                              uint32_t* __restrict__ keep) {
    const uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const uint64_t each = 2 * static_cast<uint64_t>(zl.nz) + 2;
    muto_ray t;
    const bool ok = fit::fit_record(rec + r * each, zl.z, zl.nz, zl.n_middle, &t);
    keep[r] = ok ? 1u : 0u;
    if (ok) all[r] = t;
}

__global__ void k_gather_kept(const muto_ray* __restrict__ all, const uint32_t* __restrict__ keep,
                              const uint64_t* __restrict__ pos, uint64_t n, muto_ray* __restrict__ out) {
    const uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r < n && keep[r]) out[pos[r]] = all[r];
}

}  // namespace

void launch_fit_records(const void* rec, int precision, uint64_t n, const FitLayers& zl, muto_ray* all,
                        uint32_t* keep, uint64_t* pos, void* scan_scratch, muto_ray* out, cudaStream_t s) {
    if (n == 0) return;
    const unsigned blocks = static_cast<unsigned>((n + 127) / 128);
    if (precision == 4)
        k_fit_records<float><<<blocks, 128, 0, s>>>(static_cast<const float*>(rec), n, zl, all, keep);
    else
        k_fit_records<double><<<blocks, 128, 0, s>>>(static_cast<const double*>(rec), n, zl, all, keep);
    count_launches(1);
    scan_u32_to_u64(keep, pos, n, scan_scratch, s);
    k_gather_kept<<<blocks, 128, 0, s>>>(all, keep, pos, n, out);
    count_launches(1);
}

}  // namespace muto
