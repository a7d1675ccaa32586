// Synthetic tracks for the oracle's users -- the CPU baseline and the
// reference leg of bench.py -- without the product's CUDA library.
//
// TEST INFRASTRUCTURE ONLY, like muto_oracle.cpp.  The tracks come from the
// project's own synthetic-muon model (muontomography_gb300/csrc/gen.h, which
// the library's host generator muto_generate also compiles), built here into
// the oracle's library with the same flags, so both give the same tracks bit
// for bit (tests/test_oracle_kat.py checks it).  The reference itself has no
// generator: it reads detector data, which does not exist here.
#include <cstdint>

#include "../muontomography_gb300/csrc/gen.h"

extern "C" int oracle_generate(const muto_grid* g, const double* lambda, const muto_gen_params* prm, uint64_t first,
                               uint64_t n, muto_ray* out) {
    if (!g || !lambda || !prm || (n && !out) || !muto::gen::params_ok(*prm)) return 1;
#pragma omp parallel for schedule(dynamic, 1024)
    for (long long i = 0; i < static_cast<long long>(n); ++i)
        muto::gen::generate_one(*g, lambda, *prm, first + static_cast<uint64_t>(i), out[i]);
    return 0;
}
