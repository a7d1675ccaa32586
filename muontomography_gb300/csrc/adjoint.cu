// Adjoint of the MLSD negative log-likelihood plus the MAP prior with respect
// to log(lambda).  Not in the reference; it differentiates the model whose EM
// and MAP updates the reference implements:
//   NLL(l)   = sum_i log det Sigma_i + 1/2 sum_planes v^T Sigma_i^-1 v
//              (the per-muon cost of src/MutoMLSD.cpp:465-468)
//   dNLL/dl_j = sum_i pr^2 (tr(Sigma_i^-1 W_ij) - 1/2 xyS_ij) = -sum_i g_ij,
//              summed per voxel by the voxel pass in gradient mode (em_voxel.cu).
//   prior    = 2 beta sum_j sum_{m in N(j)} w_jm psi(l_j - l_m) [+ 2 beta sum_j psi(l_j)],
//              psi(t) = (t^2 + delta^2)^(p/2), l = 1e7 lambda, stencil and edge
//              clamping of src/MutoMAP.cpp:283-350: the penalty whose separable
//              surrogate is minimised by the MAP step (src/MutoMAP.cpp:207-281).
// The gradient of the prior is formed by scattering each stencil term's
// derivative to both of its voxels, which is exact also at clamped edges.
#include "common.cuh"

namespace muto {
namespace {

inline unsigned blocks_for(uint64_t n, int threads) {
    const uint64_t b = (n + threads - 1) / threads;
    return static_cast<unsigned>(b > 0 ? b : 1);
}

template <typename Real>
__global__ void k_exp_lambda(const double* __restrict__ loglam, const uint32_t* __restrict__ mult, uint32_t V,
                             Real* __restrict__ lam) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < V) lam[j] = mult[j] > 0 ? static_cast<Real>(exp(loglam[j])) : Real(0);
}

__device__ __forceinline__ void psi_and_slope(double t, double p, double d2, double* psi, double* slope) {
    // psi = (t^2 + d^2)^(p/2), slope = d psi / dt = p t (t^2 + d^2)^((p-2)/2)
    const double u = t * t + d2;
    double q;  // u^((p-2)/2)
    if (p == 2.0) q = 1.0;
    else if (p == 1.0) q = rsqrt(u);
    else q = pow(u, (p - 2.0) / 2.0);
    *psi = u * q;
    *slope = p * t * q;
}

// dF/dl for every voxel (l = 1e7 lambda) into dl, and the prior value
__global__ void k_prior_terms(const double* __restrict__ lam64, DevGrid g, MapParams mp, double* __restrict__ dl,
                              double* __restrict__ value) {
    const uint32_t nx = g.n[0], ny = g.n[1], nz = g.n[2], nxy = nx * ny;
    const uint32_t V = nxy * nz;
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (j < V) {
        const double unit = 1.0e7;
        const uint32_t x = j % nxy % nx, y = j % nxy / nx, z = j / nxy;
        const uint32_t xs[3] = {0 < x ? x - 1 : 0, x, x < nx - 1 ? x + 1 : nx - 1};
        const uint32_t ys[3] = {0 < y ? y - 1 : 0, y, y < ny - 1 ? y + 1 : ny - 1};
        const uint32_t zs[3] = {0 < z ? z - 1 : 0, z, z < nz - 1 ? z + 1 : nz - 1};
        const double lj = lam64[j] * unit;
        const double d2 = mp.delta * mp.delta;
        const double w2 = 1.0 / sqrt(2.0), w3 = 1.0 / sqrt(3.0);
        double own = 0.0;
        for (int c = 0; c < 27; ++c) {
            const int ox = c % 3 - 1, oy = (c / 3) % 3 - 1, oz = c / 9 - 1;
            const int nzero = (ox != 0) + (oy != 0) + (oz != 0);
            if (nzero == 0) continue;
            if (!mp.all_neighbours && nzero > 1) continue;
            const double w = nzero == 1 ? 1.0 : (nzero == 2 ? w2 : w3);
            const uint32_t m = xs[ox + 1] + ys[oy + 1] * nx + zs[oz + 1] * nxy;
            const double lm = lam64[m] * unit;
            double psi, slope;
            psi_and_slope(lj - lm, mp.p, d2, &psi, &slope);
            v += 2.0 * mp.beta * w * psi;
            const double dd = 2.0 * mp.beta * w * slope;
            own += dd;
            if (m != j) atomicAdd(dl + m, -dd);
        }
        if (mp.add_object_prior) {
            double psi, slope;
            psi_and_slope(lj, mp.p, d2, &psi, &slope);
            v += 2.0 * mp.beta * psi;
            own += 2.0 * mp.beta * slope;
        }
        atomicAdd(dl + j, own);
    }
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(value, v);
}

// grad_j += l_j * dF/dl_j for voxels with pairs (chain rule through l = 1e7 exp(x))
__global__ void k_prior_finish(const double* __restrict__ lam64, const uint32_t* __restrict__ mult, uint32_t V,
                               double* __restrict__ dl, double* __restrict__ grad) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= V) return;
    if (mult[j] > 0) grad[j] += lam64[j] * 1.0e7 * dl[j];
    dl[j] = 0.0;
}

}  // namespace

template <typename Real>
void launch_exp_lambda(const double* loglam, const uint32_t* mult, uint32_t V, Real* lam, cudaStream_t s) {
    k_exp_lambda<Real><<<blocks_for(V, 256), 256, 0, s>>>(loglam, mult, V, lam); count_launches(1);
}
template void launch_exp_lambda<float>(const double*, const uint32_t*, uint32_t, float*, cudaStream_t);
template void launch_exp_lambda<double>(const double*, const uint32_t*, uint32_t, double*, cudaStream_t);

void launch_prior(const double* lam64, const uint32_t* mult, DevGrid g, MapParams mp, double* dl_scratch, double* grad,
                  double* value, cudaStream_t s) {
    const uint32_t V = g.n[0] * g.n[1] * g.n[2];
    k_prior_terms<<<blocks_for(V, 128), 128, 0, s>>>(lam64, g, mp, dl_scratch, value); count_launches(1);
    k_prior_finish<<<blocks_for(V, 256), 256, 0, s>>>(lam64, mult, V, dl_scratch, grad); count_launches(1);
}

}  // namespace muto
