// Synthetic muon generator shared by the host (OpenMP) and device (one thread
// per muon) entry points.  See host.cpp for the model.  The two builds use
// their platform's libm, so host- and device-generated tracks agree to
// rounding, not bit for bit; each is deterministic on its own.
#pragma once

#include <cmath>
#include <cstdint>

#include "../../include/muto_gb300.h"

#ifdef __CUDACC__
#define MUTO_HD __host__ __device__
#else
#define MUTO_HD
#endif

namespace muto {
namespace gen {

struct Rng {
    uint64_t s;
    bool have = false;
    double spare = 0.0;
    MUTO_HD uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    MUTO_HD double uniform() { return (static_cast<double>(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    MUTO_HD double normal() {  // Box-Muller
        if (have) {
            have = false;
            return spare;
        }
        const double u1 = uniform(), u2 = uniform();
        const double rad = sqrt(-2.0 * log(u1));
        const double a = 6.283185307179586 * u2;
        spare = rad * sin(a);
        have = true;
        return rad * cos(a);
    }
};

MUTO_HD inline void line_fit(const double* z, const double* x, const double* y, int n, double* ax, double* bx,
                             double* ay, double* by) {
    double zm = 0, xm = 0, ym = 0;
    for (int k = 0; k < n; ++k) {
        zm += z[k];
        xm += x[k];
        ym += y[k];
    }
    zm /= n;
    xm /= n;
    ym /= n;
    double szz = 0, szx = 0, szy = 0;
    for (int k = 0; k < n; ++k) {
        szz += (z[k] - zm) * (z[k] - zm);
        szx += (z[k] - zm) * (x[k] - xm);
        szy += (z[k] - zm) * (y[k] - ym);
    }
    *bx = szz > 0 ? szx / szz : 0.0;
    *by = szz > 0 ? szy / szz : 0.0;
    *ax = xm - *bx * zm;
    *ay = ym - *by * zm;
}

// Muon `id` of the stream: writes one track.
MUTO_HD inline void generate_one(const muto_grid& g, const double* lambda, const muto_gen_params& prm, uint64_t id,
                                 muto_ray& r) {
    const double lo[3] = {g.x_min, g.y_min, g.z_min};
    const double w[3] = {g.dx, g.dy, g.dz};
    const uint32_t nn[3] = {g.nx, g.ny, g.nz};
    const double hi[3] = {lo[0] + nn[0] * w[0], lo[1] + nn[1] * w[1], lo[2] + nn[2] * w[2]};
    const double ctm = cos(prm.theta_max);
    const double c3 = ctm * ctm * ctm;
    const int np = prm.n_planes;
    const long long max_steps = 4LL * (nn[0] + nn[1] + nn[2]) + 16;
    Rng G;
    G.s = prm.seed * 0xD1B54A32D192ED03ull ^ (id + 1) * 0x9E3779B97F4A7C15ull;
    G.next();
    // zenith from cos^2(theta) sin(theta): cos^3(theta) uniform on [cos^3(theta_max), 1]
    const double ct = cbrt(c3 + G.uniform() * (1.0 - c3));
    const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    const double phi = 6.283185307179586 * G.uniform();
    const double p = prm.p_min * pow(prm.p_max / prm.p_min, G.uniform());
    double pos[3] = {lo[0] + G.uniform() * (hi[0] - lo[0]), lo[1] + G.uniform() * (hi[1] - lo[1]), hi[2]};
    double sx = st * cos(phi) / ct, sy = st * sin(phi) / ct;  // projected slopes of d = (sx, sy, -1)/|.|
    const double zin0 = hi[2];
    double hz[16], hx[16], hy[16];
    for (int k = 0; k < np; ++k) {  // upper planes, straight incoming line
        const double z = zin0 + k * prm.plane_gap;
        hz[k] = z;
        hx[k] = pos[0] - sx * (z - zin0) + prm.hit_sigma * G.normal();
        hy[k] = pos[1] - sy * (z - zin0) + prm.hit_sigma * G.normal();
    }
    double in_ax, in_bx, in_ay, in_by;
    line_fit(hz, hx, hy, np, &in_ax, &in_bx, &in_ay, &in_by);
    const double k2 = (prm.p0 / p) * (prm.p0 / p);
    for (long long step = 0; step < max_steps; ++step) {  // one kick per traversed voxel
        if (pos[0] < lo[0] || pos[0] >= hi[0] || pos[1] < lo[1] || pos[1] >= hi[1] || pos[2] <= lo[2] || pos[2] > hi[2])
            break;
        const double nrm = sqrt(sx * sx + sy * sy + 1.0);
        const double d[3] = {sx / nrm, sy / nrm, -1.0 / nrm};
        uint32_t iv[3];
        double L = 1e300;
        for (int a = 0; a < 3; ++a) {
            const double f = (pos[a] - lo[a]) / w[a] + (d[a] >= 0 ? 1e-9 : -1e-9);
            long long ia = static_cast<long long>(floor(f));
            ia = ia < 0 ? 0 : (ia > static_cast<long long>(nn[a]) - 1 ? static_cast<long long>(nn[a]) - 1 : ia);
            iv[a] = static_cast<uint32_t>(ia);
            if (fabs(d[a]) > 1e-15) {
                const double b = lo[a] + (ia + (d[a] > 0 ? 1 : 0)) * w[a];
                const double s = (b - pos[a]) / d[a];
                L = s < L ? s : L;
            }
        }
        L = L > 1e-6 ? L : 1e-6;
        const double lam = lambda[iv[0] + static_cast<uint64_t>(nn[0]) * (iv[1] + static_cast<uint64_t>(nn[1]) * iv[2])];
        for (int a = 0; a < 3; ++a) pos[a] += L * d[a];
        if (lam > 0) {
            const double s = sqrt(lam * k2 * L);
            const double z1 = G.normal(), z2 = G.normal(), z3 = G.normal(), z4 = G.normal();
            // (angle, displacement) with covariance s^2 [[1, L/2], [L/2, L^2/3]] per plane
            pos[0] += s * L * (0.5 * z1 + 0.28867513459481287 * z2);
            pos[1] += s * L * (0.5 * z3 + 0.28867513459481287 * z4);
            sx = tan(atan(sx) + s * z1);
            sy = tan(atan(sy) + s * z3);
        }
    }
    const double zout0 = lo[2];
    for (int k = 0; k < np; ++k) {  // lower planes, straight outgoing line
        const double z = zout0 - k * prm.plane_gap;
        hz[k] = z;
        hx[k] = pos[0] - sx * (z - pos[2]) + prm.hit_sigma * G.normal();
        hy[k] = pos[1] - sy * (z - pos[2]) + prm.hit_sigma * G.normal();
    }
    double out_ax, out_bx, out_ay, out_by;
    line_fit(hz, hx, hy, np, &out_ax, &out_bx, &out_ay, &out_by);
    r.ein = p;
    r.eout = p;
    const double ni = sqrt(in_bx * in_bx + in_by * in_by + 1.0);
    const double no = sqrt(out_bx * out_bx + out_by * out_by + 1.0);
    r.din[0] = in_bx / ni;
    r.din[1] = in_by / ni;
    r.din[2] = 1.0 / ni;
    r.dout[0] = out_bx / no;
    r.dout[1] = out_by / no;
    r.dout[2] = 1.0 / no;
    r.pin[0] = in_ax + in_bx * zin0;
    r.pin[1] = in_ay + in_by * zin0;
    r.pin[2] = zin0;
    r.pout[0] = out_ax + out_bx * zout0;
    r.pout[1] = out_ay + out_by * zout0;
    r.pout[2] = zout0;
}

MUTO_HD inline bool params_ok(const muto_gen_params& p) {
    return p.n_planes >= 2 && p.n_planes <= 16 && p.p_min > 0 && p.p_max >= p.p_min && p.theta_max > 0 &&
           p.theta_max < 1.5 && p.p0 > 0;
}

}  // namespace gen
}  // namespace muto
