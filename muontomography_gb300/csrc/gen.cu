// Device entry point of the synthetic muon generator (gen.h): one thread per
// muon, for workloads too large to generate on the host in reasonable time.
#include "common.cuh"
#include "gen.h"

namespace muto {
namespace {
__global__ void k_generate(muto_grid g, const double* __restrict__ lambda, muto_gen_params p, uint64_t first,
                           uint64_t n, muto_ray* __restrict__ out) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    muto_ray r;
    gen::generate_one(g, lambda, p, first + i, r);
    out[i] = r;
}
}  // namespace

void launch_generate(const muto_grid& g, const double* lambda, const muto_gen_params& p, uint64_t first, uint64_t n,
                     muto_ray* out, cudaStream_t s) {
    if (n == 0) return;
    k_generate<<<static_cast<unsigned>((n + 127) / 128), 128, 0, s>>>(g, lambda, p, first, n, out);
    count_launches(1);
}
}  // namespace muto
