// Device geometry for the reconstruction path: Siddon/Jacobs voxel walk,
// point of closest approach, projected scattering angles and displacement.
//
// Bit-exactness.  The voxel lists and PoCA voxels must equal the reference's
// (src/MutoSiddon.cpp, src/MutoPoCA.cpp, src/MutoMLSD.cpp) bit for bit, so
// every FP64 operation on those paths goes through the _rn intrinsics, which
// nvcc never contracts into FMA, in the reference's evaluation order.  The
// reference's `static_cast<unsigned>(double)` is given its x86-64 GCC meaning
// (truncate to int64, keep the low 32 bits), which differs from the device's
// saturating conversion for values <= -1.
#pragma once

#include <cstdint>
#include "../../include/muto_gb300.h"

namespace muto {

struct DevGrid {
    uint32_t n[3];
    double lo[3];
    double w[3];
};

__host__ __device__ inline DevGrid make_dev_grid(const muto_grid& g) {
    DevGrid d;
    d.n[0] = g.nx; d.n[1] = g.ny; d.n[2] = g.nz;
    d.lo[0] = g.x_min; d.lo[1] = g.y_min; d.lo[2] = g.z_min;
    d.w[0] = g.dx; d.w[1] = g.dy; d.w[2] = g.dz;
    return d;
}

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
// std::max / std::min argument semantics
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }

// x86-64 GCC `static_cast<unsigned int>(double)`
__device__ __forceinline__ uint32_t u32_cast_x86(double v) {
    if (!(v > -9223372036854775808.0 && v < 9223372036854775808.0)) return 0u;
    return static_cast<uint32_t>(static_cast<unsigned long long>(__double2ll_rz(v)));
}

// Eigen Vector3::dot order: (a0*b0 + a1*b1) + a2*b2
__device__ __forceinline__ double dot3(const double* a, const double* b) {
    return dadd(dadd(dmul(a[0], b[0]), dmul(a[1], b[1])), dmul(a[2], b[2]));
}

// Order of doubles through their bit patterns: for two values whose sign
// bits are clear (non-negative, and not -0.0) the signed 64-bit integers
// order exactly as the doubles do, so the walk's comparisons can run on the
// integer pipe; it falls back to FP64 compares when a sign bit is set.
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

// Upper bound on the steps of one walk: every step crosses one plane of the
// grid, and a segment crosses each of the n+1 planes of an axis at most once.
__device__ __forceinline__ int siddon_step_bound(const DevGrid& g) {
    return static_cast<int>(g.n[0] + g.n[1] + g.n[2]) + 8;
}

// The lanes of a warp that walk paths, for __syncwarp between consecutive
// walks: a thread-per-path kernel calls this once at its start, with every
// lane of the warp present (no lane has returned yet) and `walks` true on the
// lanes that will make every one of the walks.  Without the sync, lanes that
// finish a walk early start the next one on their own and the warp's lanes
// no longer step together.
__device__ __forceinline__ unsigned walk_lanes(bool walks) { return __ballot_sync(0xffffffffu, walks); }

// Voxel walk of the segment p1 -> p2 (src/MutoSiddon.cpp:9-141).  For every
// voxel with a recorded length the sink is called as sink(ix, iy, iz, len).
// Returns the number of voxels, or -1 if the step bound was hit (never for a
// walk that ends, kept as a guard against a non-terminating loop).
// voxels a walk of a -> b can record: 1 + the index span on each axis of
// the endpoints clamped to the grid (the pieces on the grid lie between
// them), +2 per axis for rounding at either end
__device__ __forceinline__ uint32_t walk_bound(const DevGrid& g, const double* a, const double* b) {
    uint32_t n = 1;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float lo = static_cast<float>(g.lo[k]), w = static_cast<float>(g.w[k]);
        const float top = static_cast<float>(g.n[k] - 1);
        const float ia = fminf(fmaxf(floorf((static_cast<float>(a[k]) - lo) / w), 0.f), top);
        const float ib = fminf(fmaxf(floorf((static_cast<float>(b[k]) - lo) / w), 0.f), top);
        n += static_cast<uint32_t>(fabsf(ia - ib)) + 2u;
    }
    return n;
}

template <class Sink>
__device__ __forceinline__ int siddon_walk(const DevGrid& g, const double* p1, const double* p2, Sink& sink) {
    const double eps = 1.0e-6;  // :19
    double d[3], first[3], last[3];
    for (int k = 0; k < 3; ++k) d[k] = dsub(p2[k], p1[k]);
    const double seg = __dsqrt_rn(dot3(d, d));  // :14
#pragma unroll
    for (int k = 0; k < 3; ++k) {  // :25-48
        double a0 = -0.1, an = 1.1;
        const double hi = dadd(g.lo[k], dmul(g.w[k], static_cast<double>(g.n[k])));
        if (eps < fabs(d[k])) {
            a0 = ddiv(dsub(g.lo[k], p1[k]), d[k]);
            an = ddiv(dsub(hi, p1[k]), d[k]);
        } else if (p1[k] < g.lo[k] || hi <= p1[k]) {
            return 0;
        }
        first[k] = (an < a0) ? an : a0;
        last[k] = (an < a0) ? a0 : an;
    }
    const double amin = smax(smax(smax(first[0], first[1]), first[2]), 0.0);  // :50
    const double amax = smin(smin(smin(last[0], last[1]), last[2]), 1.0);     // :51
    if (amax <= amin) return 0;

    double alpha = amin;
    uint32_t idx[3];
    int dir[3];
    double da[3], an[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {  // :62-81
        const double nudge = (d[k] <= 0) ? -eps : eps;
        idx[k] = u32_cast_x86(dadd(ddiv(dsub(dadd(dmul(alpha, d[k]), p1[k]), g.lo[k]), g.w[k]), nudge));
        dir[k] = 0;
        da[k] = 0.0;
        if (eps < fabs(d[k])) {
            da[k] = ddiv(g.w[k], fabs(d[k]));
            dir[k] = d[k] < 0 ? -1 : 1;
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {  // :85-103
        an[k] = 1.1;
        if (fabs(dsub(amin, first[k])) < eps) {
            an[k] = dadd(amin, da[k]);
        } else if (dir[k] != 0) {
            const double plane = dsub(dadd(dmul(static_cast<double>(idx[k]), g.w[k]), g.lo[k]), p1[k]);
            an[k] = dadd(ddiv(plane, d[k]), dir[k] == 1 ? da[k] : 0.0);
        }
    }
    double alpha_last = alpha;
    int count = 0;
    const int bound = siddon_step_bound(g);
    int steps = 0;
    // integer compares need finite values (then every later crossing is finite too)
    const bool fast = isfinite(alpha) && isfinite(amax) && isfinite(an[0]) && isfinite(an[1]) && isfinite(an[2]);
    const long long amax_b = fast ? dbits(amax) : -1, eps_b = dbits(eps);
    // The lanes of a warp that walk together step together: every iteration
    // starts with a ballot over the lanes still walking, which makes it a
    // reconvergence point (the three-way step below would otherwise let the
    // lanes drift apart for the rest of the walk, each then issuing its own
    // FP64 instructions).
    unsigned live = __activemask();
    for (;;) {  // :108-138
        const long long alpha_b = fast ? dbits(alpha) : -1;
        const bool more = (alpha_b | amax_b) >= 0 ? alpha_b < amax_b : alpha < amax;
        const bool over = more && steps >= bound;  // the step bound: never for a walk that ends
        live = __ballot_sync(live, more && !over);
        if (!more) break;
        if (over) return -1;
        ++steps;
        const uint32_t vx = idx[0], vy = idx[1], vz = idx[2];
        // min of the three next crossings, reference tie-break order
        const long long b0 = fast ? dbits(an[0]) : -1, b1 = dbits(an[1]), b2 = dbits(an[2]);
        bool t0, t1;
        if ((b0 | b1 | b2) >= 0) {
            t0 = b0 < b1 && b0 < b2;
            t1 = b1 < b2;
        } else {
            t0 = an[0] < an[1] && an[0] < an[2];
            t1 = an[1] < an[2];
        }
        // the axis stepped, then one FP64 add for it: the lanes of a warp step
        // along different axes, and a branch per axis would issue the add
        // once per axis taken in the warp (selects are integer instructions)
        const int k = t0 ? 0 : (t1 ? 1 : 2);
        const double ak = k == 0 ? an[0] : (k == 1 ? an[1] : an[2]);
        const double dk = k == 0 ? da[0] : (k == 1 ? da[1] : da[2]);
        const double next = dadd(ak, dk);
        alpha = ak;
        an[0] = k == 0 ? next : an[0];
        an[1] = k == 1 ? next : an[1];
        an[2] = k == 2 ? next : an[2];
        idx[0] += k == 0 ? static_cast<uint32_t>(dir[0]) : 0u;
        idx[1] += k == 1 ? static_cast<uint32_t>(dir[1]) : 0u;
        idx[2] += k == 2 ? static_cast<uint32_t>(dir[2]) : 0u;
        const long long ab = dbits(alpha);
        const double upto = (ab | amax_b) >= 0 ? (amax_b < ab ? amax : alpha) : smin(alpha, amax);
        const double dalpha = dsub(upto, alpha_last);
        if (fast ? eps_b < dbits(dalpha) : eps < dalpha) {  // eps is positive
            sink(vx, vy, vz, dmul(dalpha, seg));
            ++count;
            alpha_last = alpha;
        }
    }
    return count;
}

// Point of closest approach of the in and out lines (src/MutoMLSD.cpp:328-348,
// src/MutoPoCA.cpp:192-213).  Returns true when the lines are not parallel.
__device__ __forceinline__ bool poca_point(const muto_ray& r, double eps, double* out) {
    double w0[3];
    for (int k = 0; k < 3; ++k) w0[k] = dsub(r.pin[k], r.pout[k]);
    const double a = dot3(r.din, r.din);
    const double b = dot3(r.din, r.dout);
    const double c = dot3(r.dout, r.dout);
    const double d = dot3(r.din, w0);
    const double e = dot3(r.dout, w0);
    const double den = dsub(dmul(a, c), dmul(b, b));
    if (fabs(den) < eps) {
        for (int k = 0; k < 3; ++k) out[k] = dmul(0.5, dadd(r.pin[k], r.pout[k]));
        return false;
    }
    const double cin = ddiv(dsub(dmul(b, e), dmul(c, d)), den);
    const double cout = ddiv(dsub(dmul(a, e), dmul(b, d)), den);
    for (int k = 0; k < 3; ++k)
        out[k] = dmul(0.5, dadd(dadd(dadd(r.pin[k], dmul(cin, r.din[k])), r.pout[k]), dmul(cout, r.dout[k])));
    return true;
}

// Projected scattering angles (src/MutoMLSD.cpp:350-354)
__device__ __forceinline__ void scat_angles(const double* d1, const double* d2, double* ax, double* ay) {
    *ax = dsub(atan2(d1[0], d1[2]), atan2(d2[0], d2[2]));
    *ay = dsub(atan2(d1[1], d1[2]), atan2(d2[1], d2[2]));
}

// PoCA mean squared angle (src/MutoPoCA.cpp:215-224)
__device__ __forceinline__ double scat_angle_square(const double* d1, const double* d2, double mag) {
    const double axz = dmul(dsub(atan2(d1[0], d1[2]), atan2(d2[0], d2[2])), mag);
    const double ayz = dmul(dsub(atan2(d1[1], d1[2]), atan2(d2[1], d2[2])), mag);
    return ddiv(dadd(dmul(axz, axz), dmul(ayz, ayz)), 2.0);
}

// Displacement in the xz and yz planes (src/MutoMLSD.cpp:356-376)
__device__ __forceinline__ void displacement(const muto_ray& r, double z_min, double* dxz, double* dyz) {
    const double axin = atan2(r.din[0], r.din[2]);
    const double axout = atan2(r.dout[0], r.dout[2]);
    const double ayin = atan2(r.din[1], r.din[2]);
    const double ayout = atan2(r.dout[1], r.dout[2]);
    const double sin_ = ddiv(dsub(z_min, r.pin[2]), r.din[2]);
    const double sout = ddiv(dsub(z_min, r.pout[2]), r.dout[2]);
    const double xp = dadd(r.pin[0], dmul(sin_, r.din[0]));
    const double yp = dadd(r.pin[1], dmul(sin_, r.din[1]));
    const double xt = dadd(r.pout[0], dmul(sout, r.dout[0]));
    const double yt = dadd(r.pout[1], dmul(sout, r.dout[1]));
    const double tx = tan(axin), ty = tan(ayin);
    const double lxy = __dsqrt_rn(dadd(dadd(1.0, dmul(tx, tx)), dmul(ty, ty)));
    *dxz = ddiv(dmul(dmul(dmul(dsub(xt, xp), cos(axin)), lxy), cos(axout)), cos(dsub(axout, axin)));
    *dyz = ddiv(dmul(dmul(dmul(dsub(yt, yp), cos(ayin)), lxy), cos(ayout)), cos(dsub(ayout, ayin)));
}

}  // namespace muto
