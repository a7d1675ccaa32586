// FP64 CPU oracle for the muon-tomography reconstruction path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this file;
// only the tests, `__graft_entry__.smoke()` and the CPU-baseline leg of
// `bench.py` load it (through oracle/oracle.py), and only to check results.
//
// It restates, function by function, the reference's reconstruction code
// (LasDes/MuonTomography) with every quirk kept:
//   siddon_path          src/MutoSiddon.cpp:9-141
//   poca_point           src/MutoMLSD.cpp:328-348 (== src/MutoPoCA.cpp:142-163)
//   scat_angles          src/MutoMLSD.cpp:350-354
//   scat_angle_square    src/MutoPoCA.cpp:165-174
//   displacement         src/MutoMLSD.cpp:356-376
//   Poca::run            src/MutoPoCA.cpp:51-134
//   PoCut::run           src/MutoPoCut.cpp:19-121
//   slr_run              src/MutoSLR.cpp:47-103, src/MutoSLRIter.cpp:15-83
//                        (by_level: the same passes in a level order, a
//                        check of that schedule, not the reference's order)
//   Mlsd::gather         src/MutoMLSD.cpp:268-326
//   Mlsd::path_and_tail  src/MutoMLSD.cpp:382-415
//   Mlsd::weights        src/MutoMLSD.cpp:417-430
//   Mlsd::covariance     src/MutoMLSD.cpp:442-449
//   Mlsd::s_update       src/MutoMLSD.cpp:451-491
//   Mlsd::voxel_update   src/MutoMLSD.cpp:493-517
//   Mlsd::iterate        src/MutoMLSD.cpp:179-213 and src/MutoMAP.cpp:192-261
//   map_* helpers        src/MutoMAP.cpp:207-406
// The reference's own build needs Eigen 3 and nlohmann/json; the three
// pieces of Eigen arithmetic it relies on are restated here from Eigen's
// documented semantics: Vector3::dot sums (x0*y0 + x1*y1) + x2*y2 (the SSE2 /
// NEON packet order of Eigen's unrolled redux), the 2x2 determinant is
// m00*m11 - m10*m01, and computeInverseAndDetWithCheck returns the adjugate
// times 1/det when |det| > 1e-12 (NumTraits<double>::dummy_precision()).
//
// Casting a double to `unsigned int` is done with x86-64 semantics (truncate
// to int64, keep the low 32 bits), the behaviour of the reference when built
// with GCC on x86-64.  Build with -ffp-contract=off so no FMA is formed.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#include <cfloat>

namespace {

struct Grid {  // layout == muto_grid in include/muto_gb300.h
    uint32_t nx, ny, nz, pad_;
    double x_min, y_min, z_min, dx, dy, dz;
};

struct Ray {  // layout == reference RayData (include/MutoTypes.h:47-54): 14 doubles
    double ein, eout;
    double pin[3], pout[3], din[3], dout[3];
};

struct Voxel {  // reference VoxelData (include/MutoTypes.h:40-45)
    uint32_t x, y, z;
    double length;
};

struct M2 {  // 2x2 matrix, a(r,c) = m[r][c]
    double m[2][2];
};

inline uint32_t u32_cast_x86(double v) {
    // static_cast<unsigned>(double) as compiled by GCC on x86-64: cvttsd2si
    // into a 64-bit register (NaN / out of range -> 0x8000000000000000) and
    // the low 32 bits kept.
    if (!(v > -9223372036854775808.0 && v < 9223372036854775808.0)) return 0u;
    return static_cast<uint32_t>(static_cast<uint64_t>(static_cast<int64_t>(v)));
}

inline double dot3(const double* a, const double* b) {
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

inline double smax(double a, double b) { return (a < b) ? b : a; }  // std::max
inline double smin(double a, double b) { return (b < a) ? b : a; }  // std::min

// ---------------------------------------------------------------------------
// Siddon / Jacobs traversal, src/MutoSiddon.cpp:9-141
// ---------------------------------------------------------------------------
void siddon_path(const Grid& g, const double* p1, const double* p2, std::vector<Voxel>& out) {
    out.clear();
    const double eps = 1.0e-6;  // :19
    const double d[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    const double seg = std::sqrt(dot3(d, d));  // :14
    const double lo[3] = {g.x_min, g.y_min, g.z_min};
    const double w[3] = {g.dx, g.dy, g.dz};
    const uint32_t n[3] = {g.nx, g.ny, g.nz};

    double first[3], last[3];
    for (int k = 0; k < 3; ++k) {  // :25-43
        double a0 = -0.1, an = 1.1;
        const double hi = lo[k] + w[k] * static_cast<double>(n[k]);
        if (eps < std::fabs(d[k])) {
            a0 = (lo[k] - p1[k]) / d[k];
            an = (hi - p1[k]) / d[k];
        } else if (p1[k] < lo[k] || hi <= p1[k]) {
            return;  // parallel ray outside the slab
        }
        // std::minmax(a0, an), :46-48
        first[k] = (an < a0) ? an : a0;
        last[k] = (an < a0) ? a0 : an;
    }
    const double amin = smax(smax(smax(first[0], first[1]), first[2]), 0.0);  // :50
    const double amax = smin(smin(smin(last[0], last[1]), last[2]), 1.0);     // :51
    if (amax <= amin) return;                                                 // :54

    double alpha = amin;
    uint32_t idx[3];
    int dir[3];
    double da[3], anext[3];
    for (int k = 0; k < 3; ++k) {  // :62-64 start voxel with the +-eps nudge
        const double nudge = (d[k] <= 0) ? -eps : eps;
        idx[k] = u32_cast_x86((alpha * d[k] + p1[k] - lo[k]) / w[k] + nudge);
    }
    for (int k = 0; k < 3; ++k) {  // :67-81
        dir[k] = 0;
        da[k] = 0.0;
        if (eps < std::fabs(d[k])) {
            da[k] = w[k] / std::fabs(d[k]);
            dir[k] = d[k] < 0 ? -1 : 1;
        }
    }
    for (int k = 0; k < 3; ++k) {  // :85-103 first crossing after the start voxel
        anext[k] = 1.1;
        if (std::fabs(amin - first[k]) < eps) {
            anext[k] = amin + da[k];
        } else if (dir[k] != 0) {
            anext[k] = (static_cast<double>(idx[k]) * w[k] + lo[k] - p1[k]) / d[k] + (dir[k] == 1 ? da[k] : 0.0);
        }
    }
    double alpha_last = alpha;  // :106
    while (alpha < amax) {      // :108-138
        Voxel v{idx[0], idx[1], idx[2], 0.0};
        int k;
        if (anext[0] < anext[1] && anext[0] < anext[2]) k = 0;
        else if (anext[1] < anext[2]) k = 1;
        else k = 2;
        idx[k] += static_cast<uint32_t>(dir[k]);  // unsigned wrap like MTindex += int
        alpha = anext[k];
        anext[k] += da[k];
        const double dalpha = smin(alpha, amax) - alpha_last;
        if (eps < dalpha) {
            v.length = dalpha * seg;
            out.push_back(v);
            alpha_last = alpha;
        }
    }
}

// ---------------------------------------------------------------------------
// Per-muon geometry
// ---------------------------------------------------------------------------
// src/MutoMLSD.cpp:328-348; returns true when the lines are not parallel
bool poca_point(const Ray& r, double eps, double* out) {
    const double w0[3] = {r.pin[0] - r.pout[0], r.pin[1] - r.pout[1], r.pin[2] - r.pout[2]};
    const double a = dot3(r.din, r.din);
    const double b = dot3(r.din, r.dout);
    const double c = dot3(r.dout, r.dout);
    const double d = dot3(r.din, w0);
    const double e = dot3(r.dout, w0);
    const double den = a * c - b * b;
    if (std::fabs(den) < eps) {
        for (int k = 0; k < 3; ++k) out[k] = 0.5 * (r.pin[k] + r.pout[k]);
        return false;
    }
    const double cin = (b * e - c * d) / den;
    const double cout = (a * e - b * d) / den;
    for (int k = 0; k < 3; ++k) out[k] = 0.5 * (((r.pin[k] + cin * r.din[k]) + r.pout[k]) + cout * r.dout[k]);
    return true;
}

// src/MutoMLSD.cpp:350-354
void scat_angles(const double* d1, const double* d2, double* ax, double* ay) {
    *ax = std::atan2(d1[0], d1[2]) - std::atan2(d2[0], d2[2]);
    *ay = std::atan2(d1[1], d1[2]) - std::atan2(d2[1], d2[2]);
}

// src/MutoPoCA.cpp:165-174
double scat_angle_square(const double* d1, const double* d2, double mag) {
    const double axz = (std::atan2(d1[0], d1[2]) - std::atan2(d2[0], d2[2])) * mag;
    const double ayz = (std::atan2(d1[1], d1[2]) - std::atan2(d2[1], d2[2])) * mag;
    return (axz * axz + ayz * ayz) / 2.0;
}

// src/MutoMLSD.cpp:356-376 (pow(x, 2) is x*x)
void displacement(const Ray& r, double z_min, double* dxz, double* dyz) {
    const double axin = std::atan2(r.din[0], r.din[2]);
    const double axout = std::atan2(r.dout[0], r.dout[2]);
    const double ayin = std::atan2(r.din[1], r.din[2]);
    const double ayout = std::atan2(r.dout[1], r.dout[2]);
    const double sin_ = (z_min - r.pin[2]) / r.din[2];
    const double sout = (z_min - r.pout[2]) / r.dout[2];
    const double xp = r.pin[0] + sin_ * r.din[0];
    const double yp = r.pin[1] + sin_ * r.din[1];
    const double xt = r.pout[0] + sout * r.dout[0];
    const double yt = r.pout[1] + sout * r.dout[1];
    const double tx = std::tan(axin), ty = std::tan(ayin);
    const double lxy = std::sqrt(1 + tx * tx + ty * ty);
    *dxz = (xt - xp) * std::cos(axin) * lxy * std::cos(axout) / std::cos(axout - axin);
    *dyz = (yt - yp) * std::cos(ayin) * lxy * std::cos(ayout) / std::cos(ayout - ayin);
}

}  // namespace

// ===========================================================================
// C interface used by oracle/oracle.py
// ===========================================================================
extern "C" {

typedef struct {
    int32_t update_with_mean;   // src/MutoMLSD.cpp:63
    int32_t mean_percentile;    // :69
    int32_t straight_line;      // :64
    int32_t has_energy;         // :65
    int32_t early_stop;         // :66
    int32_t num_iteration;      // :70
    int64_t total_num_rays;     // :68
    double error_xy;            // :78
    double error_dz_outer;      // :79
    double error_dz_inner;      // :80
    double angle_unit_mag;      // :82
    double eps;                 // :83
    int32_t is_map;             // MutoMAP instead of MutoMLSD
    int32_t add_object_prior;   // src/MutoMAP.cpp:80
    int32_t all_neighbours;     // src/MutoMAP.cpp:81
    int32_t length_weighted;    // src/MutoPoCA.cpp:90 (PoCA only)
    double beta;                // src/MutoMAP.cpp:77
    double p;                   // :78
    double delta;               // :79
} oracle_cfg;

// Batched getVoxelPath: for ray r the voxels go to xyz[(r*cap + k)*3 + 0..2]
// and len[r*cap + k] for k < min(count, cap); counts[r] = full count.
int oracle_siddon_batch(const Grid* g, const double* p1, const double* p2, uint64_t n, uint32_t cap,
                        uint32_t* xyz, double* len, uint32_t* counts) {
    std::vector<Voxel> path;
    path.reserve(2 * g->nz);
    for (uint64_t r = 0; r < n; ++r) {
        siddon_path(*g, p1 + 3 * r, p2 + 3 * r, path);
        counts[r] = static_cast<uint32_t>(path.size());
        const size_t m = std::min<size_t>(path.size(), cap);
        for (size_t k = 0; k < m; ++k) {
            xyz[(r * cap + k) * 3 + 0] = path[k].x;
            xyz[(r * cap + k) * 3 + 1] = path[k].y;
            xyz[(r * cap + k) * 3 + 2] = path[k].z;
            len[r * cap + k] = path[k].length;
        }
    }
    return 0;
}

// PoCA reconstruction, src/MutoPoCA.cpp:51-134, and PoCut, src/MutoPoCut.cpp:19-121
// (cut != nullptr: the percentile *cut).  PoCut differs in two places: the
// path is always the two halves around the PoCA point (its constructor sets
// fStraightLine = false, :11-15), and instead of summing the scattering
// values per voxel it keeps them, sorts each voxel's values ascending and
// sums the lowest floor(count * cut) of them in that order from 0.0
// (:113-117).  A cut that would take more values than the voxel holds (the
// reference would read past the end) takes all of them.
static int poca_run(const Grid* gp, const oracle_cfg* cfg, const double* cut, const Ray* rays, uint64_t n_rays,
                    double* img, int64_t* assign, uint64_t* counters) {
    const Grid& g = *gp;
    const uint64_t V = static_cast<uint64_t>(g.nx) * g.ny * g.nz;
    std::vector<double> weight(V, 0.0);
    std::vector<std::vector<double>> values(cut ? V : 0);  // PoCut: the values of each voxel
    std::fill(img, img + V, 0.0);
    if (n_rays == 0) return 0;
    const bool straight = cut ? false : cfg->straight_line != 0;
    uint64_t n_total = cfg->total_num_rays > 0 ? static_cast<uint64_t>(cfg->total_num_rays) : n_rays;
    if (n_total > n_rays) n_total = n_rays;  // the reference would read past the end
    uint64_t not_parallel = 0, in_grid = 0;
    const double z_det_min = rays[0].pout[2];  // :111
    const double z_det_max = rays[0].pin[2];   // :112
    std::vector<Voxel> vin, vout;
    auto at = [&](uint32_t x, uint32_t y, uint32_t z) -> uint64_t {
        return static_cast<uint64_t>(x) + static_cast<uint64_t>(g.nx) * (static_cast<uint64_t>(y) + static_cast<uint64_t>(g.ny) * z);
    };
    for (uint64_t i = 0; i < n_total; ++i) {
        const Ray& r = rays[i];
        double ps[3];
        if (poca_point(r, cfg->eps, ps)) ++not_parallel;
        const double a2 = scat_angle_square(r.din, r.dout, cfg->angle_unit_mag);
        const uint32_t xs = u32_cast_x86((ps[0] - g.x_min) / g.dx);  // :121-123
        const uint32_t ys = u32_cast_x86((ps[1] - g.y_min) / g.dy);
        const uint32_t zs = u32_cast_x86((ps[2] - g.z_min) / g.dz);
        // :125-128 (the "< 0" tests on unsigned values are always false)
        if (g.nx <= xs || g.ny <= ys || g.nz <= zs || ps[2] < z_det_min || z_det_max < ps[2]) {
            if (assign) assign[3 * i] = assign[3 * i + 1] = assign[3 * i + 2] = -1;
            continue;
        }
        ++in_grid;
        if (assign) { assign[3 * i] = xs; assign[3 * i + 1] = ys; assign[3 * i + 2] = zs; }
        const double v = cfg->has_energy ? a2 * r.ein * r.ein : a2;  // :134-138 (PoCut :60-64)
        if (cut) values[at(xs, ys, zs)].push_back(v);
        else img[at(xs, ys, zs)] += v;
        // a walk inside the grid never yields an out-of-range voxel; the check
        // only keeps a malformed input from writing outside the image
        auto addw = [&](const Voxel& w, double l) {
            if (w.x < g.nx && w.y < g.ny && w.z < g.nz) weight[at(w.x, w.y, w.z)] += l;
        };
        if (straight) {  // :141-149
            siddon_path(g, r.pin, r.pout, vin);
            for (const Voxel& w : vin) addw(w, cfg->length_weighted ? w.length : g.dz);
        } else {  // :150-171
            siddon_path(g, r.pin, ps, vin);
            siddon_path(g, ps, r.pout, vout);
            for (const Voxel& w : vin) addw(w, cfg->length_weighted ? w.length : g.dz);
            for (const Voxel& w : vout) {
                if (cfg->length_weighted) addw(w, w.length);
                else if (w.x != xs || w.y != ys || w.z != zs) addw(w, g.dz);
            }
        }
    }
    if (cut) {  // src/MutoPoCut.cpp:113-118
        for (uint64_t j = 0; j < V; ++j) {
            std::vector<double>& s = values[j];
            std::sort(s.begin(), s.end());
            uint64_t t = u32_cast_x86(static_cast<double>(s.size()) * *cut);
            if (t > s.size()) t = s.size();
            const double sum = std::accumulate(s.begin(), s.begin() + static_cast<std::ptrdiff_t>(t), 0.0);
            img[j] = weight[j] < cfg->eps ? 0 : sum / weight[j];
        }
    } else {
        for (uint64_t j = 0; j < V; ++j) img[j] = weight[j] < cfg->eps ? 0 : img[j] / weight[j];  // :180-182
    }
    if (counters) { counters[0] = n_total; counters[1] = not_parallel; counters[2] = in_grid; }
    return 0;
}

// img: V doubles (column-major, x fastest).  assign (optional): 3 int64 per
// ray, the PoCA voxel of each ray or -1 when the ray was rejected.
// counters (optional): [n_total, n_not_parallel, n_scat_in_grid].
int oracle_poca(const Grid* gp, const oracle_cfg* cfg, const Ray* rays, uint64_t n_rays, double* img,
                int64_t* assign, uint64_t* counters) {
    return poca_run(gp, cfg, nullptr, rays, n_rays, img, assign, counters);
}

// Straight-line reconstruction, src/MutoSLR.cpp:47-103 (n_iter = 0), and its
// iterative form, src/MutoSLRIter.cpp:15-83 (n_iter >= 1 passes, in place:
// every muon sees the image as the muons before it left it, and each pass
// adds its weights again).  Each muon's incoming and outgoing lines are cut
// at the grid's top and bottom planes and the straight line between the two
// points is walked; its voxels get the mean squared projected angle, shared
// by length^2 (length_weighted) or equally.
// by_level: run the muons level by level instead of in index order (a
// muon's level is one more than the highest level among the earlier muons
// sharing a voxel with it), the latest index first within a level.  Not the
// reference's order: a check that this schedule, which a parallel form would
// use, leaves every result bit for bit as the index order does.
static int slr_run(const Grid* gp, const oracle_cfg* cfg, int n_iter, const Ray* rays, uint64_t n_rays, double* img,
                   bool by_level = false) {
    const Grid& g = *gp;
    const uint64_t V = static_cast<uint64_t>(g.nx) * g.ny * g.nz;
    std::vector<double> weight(V, 0.0);
    std::fill(img, img + V, 0.0);
    uint64_t n_total = cfg->total_num_rays > 0 ? static_cast<uint64_t>(cfg->total_num_rays) : n_rays;
    if (n_total > n_rays) n_total = n_rays;  // the reference would read past the end
    const double z_lo = g.z_min;                                   // :57
    const double z_hi = g.z_min + g.dz * static_cast<double>(g.nz);  // :58
    const double mag = cfg->angle_unit_mag;
    auto at = [&](const Voxel& v) -> uint64_t {
        return static_cast<uint64_t>(v.x) + static_cast<uint64_t>(g.nx) * (static_cast<uint64_t>(v.y) + static_cast<uint64_t>(g.ny) * v.z);
    };
    std::vector<Voxel> path;
    std::vector<uint64_t> order(n_total);
    std::iota(order.begin(), order.end(), uint64_t(0));
    if (by_level) {
        std::vector<uint32_t> last(V, 0), level(n_total, 0);
        for (uint64_t i = 0; i < n_total; ++i) {
            const Ray& r = rays[i];
            const double t_in = (z_hi - r.pin[2]) / r.din[2];
            const double t_out = (z_lo - r.pout[2]) / r.dout[2];
            double p_in[3], p_out[3];
            for (int k = 0; k < 3; ++k) {
                p_in[k] = r.pin[k] + t_in * r.din[k];
                p_out[k] = r.pout[k] + t_out * r.dout[k];
            }
            siddon_path(g, p_in, p_out, path);
            uint32_t lv = 0;
            for (const Voxel& v : path) lv = std::max(lv, last[at(v)]);
            level[i] = lv + 1;
            for (const Voxel& v : path) last[at(v)] = lv + 1;
        }
        std::sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) {
            return level[a] != level[b] ? level[a] < level[b] : a > b;
        });
    }
    const int passes = n_iter > 0 ? n_iter : 1;
    for (int iter = 0; iter < passes; ++iter) {
        for (uint64_t q = 0; q < n_total; ++q) {
            const uint64_t i = order[q];
            const Ray& r = rays[i];
            const double axz = (std::atan2(r.din[0], r.din[2]) - std::atan2(r.dout[0], r.dout[2])) * mag;  // :63-64
            const double ayz = (std::atan2(r.din[1], r.din[2]) - std::atan2(r.dout[1], r.dout[2])) * mag;
            const double t_in = (z_hi - r.pin[2]) / r.din[2];  // :67-70
            const double t_out = (z_lo - r.pout[2]) / r.dout[2];
            double p_in[3], p_out[3], d[3];
            for (int k = 0; k < 3; ++k) {
                p_in[k] = r.pin[k] + t_in * r.din[k];
                p_out[k] = r.pout[k] + t_out * r.dout[k];
                d[k] = p_in[k] - p_out[k];
            }
            siddon_path(g, p_in, p_out, path);
            const double l_total = std::sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);  // :77
            double val_total = 0.0;  // src/MutoSLRIter.cpp:49-52
            if (n_iter > 0)
                for (const Voxel& v : path) val_total += img[at(v)];
            const double a2 = axz * axz + ayz * ayz;
            for (const Voxel& v : path) {
                const uint64_t j = at(v);
                double iv;
                if (cfg->length_weighted) {  // :80-86
                    weight[j] += v.length / g.dz;
                    iv = a2 * 0.5 * (v.length / l_total) * (v.length / l_total);
                } else {
                    weight[j] += 1.0;
                    iv = a2 * 0.5 / static_cast<double>(path.size() * path.size());
                }
                if (n_iter > 0 && iter != 0) iv *= img[j] / val_total;  // src/MutoSLRIter.cpp:64-66
                if (cfg->has_energy) iv *= r.ein * r.ein;                 // :87-89
                img[j] += iv;
            }
        }
    }
    for (uint64_t j = 0; j < V; ++j) img[j] = weight[j] < cfg->eps ? 0 : img[j] / weight[j];  // :98-100
    return 0;
}

// SLR (n_iter = 0) or SLRIter (n_iter = its "num_iteration", >= 1).
int oracle_slr(const Grid* gp, const oracle_cfg* cfg, int n_iter, const Ray* rays, uint64_t n_rays, double* img) {
    return slr_run(gp, cfg, n_iter, rays, n_rays, img);
}

// oracle_slr with the muons run level by level (see slr_run): equal to
// oracle_slr bit for bit exactly when that schedule keeps the results.
int oracle_slr_by_level(const Grid* gp, const oracle_cfg* cfg, int n_iter, const Ray* rays, uint64_t n_rays,
                        double* img) {
    return slr_run(gp, cfg, n_iter, rays, n_rays, img, true);
}

// PoCut with percentile cut (the "cut_percentile" key); outputs as oracle_poca.
int oracle_pocut(const Grid* gp, const oracle_cfg* cfg, double cut, const Ray* rays, uint64_t n_rays, double* img,
                 int64_t* assign, uint64_t* counters) {
    return poca_run(gp, cfg, &cut, rays, n_rays, img, assign, counters);
}

}  // extern "C"

// ===========================================================================
// MLSD / MAP
// ===========================================================================
namespace {

struct Mlsd {
    Grid g;
    oracle_cfg cfg;
    // gatherInformation outputs (src/MutoMLSD.cpp:110-116)
    std::vector<uint32_t> kept;
    std::vector<double> sx, sy, dx, dy, pr;
    std::vector<double> scat;  // 3 per kept muon
    // weight matrices and S lists (src/MutoMLSD.cpp:132-139)
    std::vector<std::vector<std::pair<uint32_t, M2>>> W;
    std::vector<std::vector<double>> S;
    std::vector<uint32_t> S_index;
    // per-kept-muon merged path (for parity export)
    std::vector<uint64_t> path_off;
    std::vector<uint32_t> path_idx;
    std::vector<double> path_len, path_tail;
    bool keep_paths = true;
    std::vector<double> img;
    M2 E;
    double cost = 0.0, cost_prev = 0.0;
    int iters_done = 0;
    bool stopped = false;
    uint64_t n_total = 0, n_scat = 0;
    uint64_t n_singular = 0, n_nonconv = 0, n_bad_index = 0, n_pairs = 0;
    std::vector<double> cost_hist;

    uint64_t V() const { return static_cast<uint64_t>(g.nx) * g.ny * g.nz; }
    // xyz2index, include/MutoMLSD.h:76 (MTindex arithmetic)
    uint32_t flat(uint32_t x, uint32_t y, uint32_t z) const { return x + y * g.nx + z * g.nx * g.ny; }

    // src/MutoMLSD.cpp:268-326
    void gather(const Ray* data, uint64_t n) {
        const double z_det_min = data[0].pout[2];
        const double z_det_max = data[0].pin[2];
        const double p_nominal = 3.0;
        if (!cfg.has_energy) pr.push_back(p_nominal / p_nominal);
        const double eps = cfg.eps;
        const double xhi = g.x_min + g.dx * g.nx - eps;
        const double yhi = g.y_min + g.dy * g.ny - eps;
        const double zhi = g.z_min + g.dz * g.nz - eps;
        for (uint64_t i = 0; i < n; ++i) {
            if (i == n_total) break;
            const Ray& r = data[i];
            double ps[3];
            poca_point(r, eps, ps);
            if (ps[0] < g.x_min + eps || xhi < ps[0] || ps[1] < g.y_min + eps || yhi < ps[1] ||
                ps[2] < g.z_min + eps || zhi < ps[2] || ps[2] < z_det_min + eps || z_det_max - eps <= ps[2])
                continue;
            kept.push_back(static_cast<uint32_t>(i));
            scat.insert(scat.end(), ps, ps + 3);
            ++n_scat;
            double ax, ay, ddx, ddy;
            scat_angles(r.din, r.dout, &ax, &ay);
            displacement(r, g.z_min, &ddx, &ddy);
            sx.push_back(ax);
            sy.push_back(ay);
            dx.push_back(ddx);
            dy.push_back(ddy);
            if (cfg.has_energy) pr.push_back(p_nominal / r.ein);
        }
    }

    // src/MutoMLSD.cpp:382-415: merged two-segment path and tail lengths
    void path_and_tail(const Ray& r, const double* ps, std::vector<Voxel>& path, std::vector<double>& tail,
                       std::vector<Voxel>& vin, std::vector<Voxel>& vout) {
        path.clear();
        if (cfg.straight_line) {
            siddon_path(g, r.pin, r.pout, path);
        } else {
            siddon_path(g, r.pin, ps, vin);
            siddon_path(g, ps, r.pout, vout);
            if (!vin.empty()) {
                vin.back().length += !vout.empty() ? vout[0].length : 0.0;
                path.insert(path.end(), vin.begin(), vin.end());
            }
            if (!vout.empty()) path.insert(path.end(), vout.begin() + 1, vout.end());
        }
        tail.assign(path.size(), 0.0);  // tail.back() on an empty path is undefined in the reference
        for (long k = static_cast<long>(tail.size()) - 2; k >= 0; --k) tail[k] = tail[k + 1] + path[k + 1].length;
    }

    void setup(const Ray* data, uint64_t n, const double* init) {
        n_total = cfg.total_num_rays > 0 ? static_cast<uint64_t>(cfg.total_num_rays) : n;
        img.assign(init, init + V());
        if (n > 0) gather(data, n);
        W.assign(kept.size(), {});
        S.assign(V(), {});
        S_index.assign(V(), 0);
        std::vector<Voxel> path, vin, vout;
        std::vector<double> tail;
        path_off.assign(1, 0);
        for (size_t i = 0; i < kept.size(); ++i) {  // src/MutoMLSD.cpp:145-152
            path_and_tail(data[kept[i]], &scat[3 * i], path, tail, vin, vout);
            for (size_t k = 0; k < path.size(); ++k) {  // generateWeightMatrix, :417-430
                const double L = path[k].length, T = tail[k];
                const double LT = L * T;
                M2 w;
                w.m[0][0] = L;
                w.m[0][1] = w.m[1][0] = LT + L * L * 0.5;
                w.m[1][1] = L * L * L / 3.0 + (L + T) * LT;
                const uint32_t j = flat(path[k].x, path[k].y, path[k].z);
                W[i].push_back({j, w});
                if (j < V()) S[j].push_back(0.0);  // allocateSValueMatrix, :432-437
                else ++n_bad_index;
                ++n_pairs;
                if (keep_paths) {
                    path_idx.push_back(j);
                    path_len.push_back(L);
                    path_tail.push_back(T);
                }
            }
            path_off.push_back(n_pairs);
        }
        const double exy = cfg.error_xy, ezo = cfg.error_dz_outer, ezi = cfg.error_dz_inner;  // :168-170
        E.m[0][0] = 4.0 * exy * exy / (ezo * ezo);
        E.m[1][1] = 2.0 * exy * exy * (1.0 + (ezi / ezo + 1.0) * ezi / ezo);
        E.m[0][1] = E.m[1][0] = 2.0 * exy * exy * ezi / (ezo * ezo);
    }

    // src/MutoMLSD.cpp:442-449 plus Sigma += ErrorM (:191)
    M2 covariance(const std::vector<double>& lam, const std::vector<std::pair<uint32_t, M2>>& Wi, double p) const {
        M2 c{{{0.0, 0.0}, {0.0, 0.0}}};
        for (const auto& wj : Wi) {
            const double l = wj.first < lam.size() ? lam[wj.first] : 0.0;
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b) c.m[a][b] += l * wj.second.m[a][b];
        }
        const double p2 = p * p;
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b) c.m[a][b] = p2 * c.m[a][b] + E.m[a][b];
        return c;
    }

    static M2 mul(const M2& A, const M2& B) {
        M2 C;
        for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 2; ++c) C.m[r][c] = A.m[r][0] * B.m[0][c] + A.m[r][1] * B.m[1][c];
        return C;
    }

    // src/MutoMLSD.cpp:451-491; returns the muon's cost
    double s_update(const std::vector<double>& lam, const M2& cov, size_t i, double p) {
        const double det = cov.m[0][0] * cov.m[1][1] - cov.m[1][0] * cov.m[0][1];
        const bool invertible = std::fabs(det) > 1e-12;
        M2 inv{{{0.0, 0.0}, {0.0, 0.0}}};
        if (invertible) {
            const double r = 1.0 / det;
            inv.m[0][0] = cov.m[1][1] * r;
            inv.m[1][0] = -cov.m[1][0] * r;
            inv.m[0][1] = -cov.m[0][1] * r;
            inv.m[1][1] = cov.m[0][0] * r;
        }
        const double Sx = sx[i], Sy = sy[i], Dx = dx[i], Dy = dy[i];
        double cost = 0.0;
        if (!invertible || det <= 0) {
            ++n_singular;
        } else {
            cost = std::log(det) + ((Sx * Sx + Sy * Sy) * inv.m[0][0] + (Dx * Dx + Dy * Dy) * inv.m[1][1] +
                                    (Sx * Dx + Sy * Dy) * 2.0 * inv.m[0][1]) * 0.5;
        }
        for (const auto& wj : W[i]) {
            const uint32_t j = wj.first;
            if (j >= V()) continue;
            const double lj = lam[j];
            const double pr2lj2 = p * p * lj * lj;
            const M2 IW = mul(inv, wj.second);
            const double tr = IW.m[0][0] + IW.m[1][1];
            const M2 C = mul(IW, inv);
            const double xyS = (Sx * Sx + Sy * Sy) * C.m[0][0] + (Dx * Dx + Dy * Dy) * C.m[1][1] +
                               (Sx * Dx + Sy * Dy) * (C.m[0][1] + C.m[1][0]);
            const double s = 2.0 * lj + (0.5 * xyS - tr) * pr2lj2;
            S[j][S_index[j]] = s;
            S_index[j]++;
        }
        return cost;
    }

    // src/MutoMLSD.cpp:493-517
    double voxel_update(std::vector<double>& Sj, uint32_t Mj) const {
        if (Mj == 0) return 0.0;
        if (cfg.update_with_mean) {
            if (cfg.mean_percentile == 100) {
                return std::accumulate(Sj.begin(), Sj.begin() + Mj, 0.0) / static_cast<double>(Mj) * 0.5;
            }
            uint32_t jm = u32_cast_x86(cfg.mean_percentile / 100.0 * Mj);
            if (jm < 1) jm = 1;
            std::sort(Sj.begin(), Sj.end());
            return std::accumulate(Sj.begin(), Sj.begin() + jm, 0.0) / static_cast<double>(jm) * 0.5;
        }
        std::nth_element(Sj.begin(), Sj.begin() + Mj / 2, Sj.begin() + Mj);
        const double med = Sj[Mj / 2];
        if (Mj % 2 == 0) {
            std::nth_element(Sj.begin(), Sj.begin() + Mj / 2 - 1, Sj.begin() + Mj);
            return (med + Sj[Mj / 2 - 1]) * 0.25;
        }
        return med * 0.5;
    }

    // ML (EM) step on `lam`; fills `out` with the updated image; returns mean cost
    double ml_step(const std::vector<double>& lam, std::vector<double>& out) {
        std::fill(S_index.begin(), S_index.end(), 0u);
        double c = 0.0;
        for (size_t i = 0; i < kept.size(); ++i) {
            const double p = cfg.has_energy ? pr[i] : pr[0];
            const M2 cov = covariance(lam, W[i], p);
            c += s_update(lam, cov, i, p);
        }
        const long long nv = static_cast<long long>(V());
#pragma omp parallel for schedule(dynamic, 256)
        for (long long j = 0; j < nv; ++j) out[j] = voxel_update(S[j], S_index[j]);
        return c / static_cast<double>(kept.size());
    }

    // ---------------- MAP helpers, src/MutoMAP.cpp:207-406 ----------------
    static constexpr double kUnit = 1.0e7;  // src/MutoMAP.cpp:96

    // neighbour values (x1e7) in the reference's order; returns the count
    int neighbours(uint32_t j, const std::vector<double>& lam, double* lm, double* wm) const {
        const uint32_t nxy = g.nx * g.ny;
        const uint32_t x = j % nxy % g.nx, y = j % nxy / g.nx, z = j / nxy;  // index2xyz :283-290
        const uint32_t xp = x < g.nx - 1 ? x + 1 : g.nx - 1, yp = y < g.ny - 1 ? y + 1 : g.ny - 1,
                       zp = z < g.nz - 1 ? z + 1 : g.nz - 1;
        const uint32_t xm = 0 < x ? x - 1 : 0, ym = 0 < y ? y - 1 : 0, zm = 0 < z ? z - 1 : 0;
        auto at = [&](uint32_t a, uint32_t b, uint32_t c) { return lam[flat(a, b, c)] * kUnit; };
        int k = 0;
        // faces :301-306 / :320-325
        lm[k++] = at(xp, y, z); lm[k++] = at(xm, y, z);
        lm[k++] = at(x, yp, z); lm[k++] = at(x, ym, z);
        lm[k++] = at(x, y, zp); lm[k++] = at(x, y, zm);
        for (int q = 0; q < 6; ++q) wm[q] = 1.0;
        if (!cfg.all_neighbours) return 6;
        // edges :327-338
        lm[k++] = at(xp, yp, z); lm[k++] = at(xm, yp, z); lm[k++] = at(xp, ym, z); lm[k++] = at(xm, ym, z);
        lm[k++] = at(x, yp, zp); lm[k++] = at(x, ym, zp); lm[k++] = at(x, yp, zm); lm[k++] = at(x, ym, zm);
        lm[k++] = at(xp, y, zp); lm[k++] = at(xm, y, zp); lm[k++] = at(xp, y, zm); lm[k++] = at(xm, y, zm);
        // corners :340-347
        lm[k++] = at(xp, yp, zp); lm[k++] = at(xm, yp, zp); lm[k++] = at(xp, ym, zp); lm[k++] = at(xm, ym, zp);
        lm[k++] = at(xp, yp, zm); lm[k++] = at(xm, yp, zm); lm[k++] = at(xp, ym, zm); lm[k++] = at(xm, ym, zm);
        const double w2 = 1.0 / std::sqrt(2.0), w3 = 1.0 / std::sqrt(3.0);  // :214-215
        for (int q = 6; q < 18; ++q) wm[q] = w2;
        for (int q = 18; q < 26; ++q) wm[q] = w3;
        return 26;
    }

    // src/MutoMAP.cpp:353-406; Newton capped at `cap` iterations (the reference has no cap)
    int cubic(double* roots, double p3, double p2, double p1, double p0, double tol, long cap) {
        const double a = p2 / p3, b = p1 / p3, c = p0 / p3;
        const double r = 1 + smax(smax(std::fabs(a), std::fabs(b)), std::fabs(c));
        const double xi = -a / 3;
        const double gxi = xi * xi * xi + a * xi * xi + b * xi + c;
        double xk = 0 < gxi ? -r : r;
        double rel = tol * 2;
        long it = 0;
        while (rel > tol) {
            if (++it > cap) {
#pragma omp atomic
                ++n_nonconv;
                break;
            }
            const double xk2 = xk * xk;
            const double gx = xk2 * xk + a * xk2 + b * xk + c;
            const double gp = 3 * xk2 + 2 * a * xk + b;
            const double xn = xk - gx / gp;
            rel = std::fabs((xn - xk) / xk);
            xk = xn;
        }
        const double x1 = xk;
        const double D = x1 + a;
        const double Ec = D * x1 + b;
        const double sgn = 0 <= D ? 1 : -1;
        const double disc = D * D - 4 * Ec;
        if (disc < 0) { roots[0] = x1; return 1; }
        const double q = -0.5 * (D + sgn * std::sqrt(disc));
        roots[0] = x1;
        roots[1] = q;
        roots[2] = tol < std::fabs(q) ? Ec / q : q;
        return 3;
    }

    // src/MutoMAP.cpp:261-281
    double surrogate(uint32_t Mj, double ljn, double ljml, double x, const double* w, const double* lm, int nn) const {
        if (x < 0) return DBL_MAX;
        double v = 0.0;
        v += 0 < x ? static_cast<double>(Mj) * (std::log(x) + ljml / x) : 0.0;
        const double e = (cfg.p - 2.0) / 2.0;
        for (int k = 0; k < nn; ++k) {
            const double dd = ljn - lm[k];
            const double t = 2.0 * x - ljn - lm[k];
            v += 0.5 * cfg.beta * cfg.p * w[k] * std::pow(dd * dd + cfg.delta * cfg.delta, e) * (t * t);
        }
        if (cfg.add_object_prior)
            v += 0.5 * cfg.beta * cfg.p * x * x * std::pow(ljn * ljn + cfg.delta * cfg.delta, e);
        return v;
    }

    // MAP step for voxel j, src/MutoMAP.cpp:228-246 with :207-259
    double map_voxel(uint32_t j, const std::vector<double>& last, const std::vector<double>& ml, uint32_t Mj) {
        double lm[26], wm[26];
        const int nn = neighbours(j, last, lm, wm);
        const double e = (cfg.p - 2.0) / 2.0;
        const double lj = last[j] * kUnit;
        double p2 = 0.0, p3 = 0.0;
        for (int k = 0; k < nn; ++k) {
            const double dd = lj - lm[k];
            const double t1 = wm[k] * cfg.p * std::pow(dd * dd + cfg.delta * cfg.delta, e);
            p2 += t1 * 2.0 * (lj + lm[k]);
            p3 += t1 * 4.0;
        }
        if (cfg.add_object_prior) p3 += cfg.p * std::pow(lj * lj + cfg.delta * cfg.delta, e);
        p2 *= -cfg.beta / static_cast<double>(Mj);
        p3 *= cfg.beta / static_cast<double>(Mj);
        const double p0 = -ml[j] * kUnit, p1 = 1.0;
        double roots[3];
        const int nr = cubic(roots, p3, p2, p1, p0, cfg.eps, 1000000);
        // chooseBestEstimation :239-259 (first minimum wins)
        const double ljn = last[j] * kUnit, ljml = ml[j] * kUnit;
        double best = 0.0;
        int bi = 0;
        for (int k = 0; k <= nr; ++k) {
            const double v = surrogate(Mj, ljn, ljml, k < nr ? roots[k] : ljml, wm, lm, nn);
            if (k == 0 || v < best) { best = v; bi = k; }
        }
        return bi < nr ? roots[bi] / kUnit : ml[j];
    }

    // one iteration; src/MutoMLSD.cpp:179-213 (MLSD) or src/MutoMAP.cpp:192-261 (MAP)
    void iterate_once() {
        if (stopped) return;
        cost_prev = cost;
        double c;
        if (!cfg.is_map) {
            std::vector<double> out(V());
            c = ml_step(img, out);
            img.swap(out);
        } else {
            const std::vector<double> last = img;
            std::vector<double> ml(V());
            c = ml_step(last, ml);
            const long long nv = static_cast<long long>(V());
            std::vector<uint64_t> nonconv(1, 0);
#pragma omp parallel for schedule(dynamic, 256)
            for (long long j = 0; j < nv; ++j) {
                if (S_index[j] == 0) { img[j] = 0.0; continue; }
                img[j] = map_voxel(static_cast<uint32_t>(j), last, ml, S_index[j]);
            }
        }
        cost = c;
        cost_hist.push_back(c);
        ++iters_done;
        // the reference compares with an uninitialised value on iteration 0; here no stop is possible there
        if (cfg.early_stop && iters_done > 1 && cost_prev < cost) stopped = true;
    }
};

}  // namespace

extern "C" {

// keep_paths != 0 keeps a copy of every merged path (index, L, T) for
// oracle_mlsd_export; 0 saves that memory for timing runs.
void* oracle_mlsd_create(const Grid* g, const oracle_cfg* cfg, const Ray* rays, uint64_t n, const double* init_img,
                         int keep_paths) {
    Mlsd* m = new Mlsd();
    m->g = *g;
    m->cfg = *cfg;
    m->keep_paths = keep_paths != 0;
    m->setup(rays, n, init_img);
    return m;
}

void oracle_mlsd_destroy(void* h) { delete static_cast<Mlsd*>(h); }

// counts: [n_total, n_scat_in_grid, n_pairs, n_singular, n_nonconverged, n_bad_index, iterations_done, stopped]
void oracle_mlsd_counts(void* h, uint64_t* out) {
    Mlsd* m = static_cast<Mlsd*>(h);
    out[0] = m->n_total;
    out[1] = m->n_scat;
    out[2] = m->n_pairs;
    out[3] = m->n_singular;
    out[4] = m->n_nonconv;
    out[5] = m->n_bad_index;
    out[6] = m->iters_done;
    out[7] = m->stopped ? 1 : 0;
}

// kept: n_scat ints; info: 6 doubles per kept muon (Sx, Sy, Dx, Dy, pr, unused);
// scat: 3 per kept; off: n_scat+1; idx/len/tail: n_pairs
void oracle_mlsd_export(void* h, uint32_t* kept, double* info, double* scat, uint64_t* off, uint32_t* idx, double* len,
                        double* tail) {
    Mlsd* m = static_cast<Mlsd*>(h);
    const size_t n = m->kept.size();
    for (size_t i = 0; i < n; ++i) {
        if (kept) kept[i] = m->kept[i];
        if (info) {
            info[6 * i + 0] = m->sx[i];
            info[6 * i + 1] = m->sy[i];
            info[6 * i + 2] = m->dx[i];
            info[6 * i + 3] = m->dy[i];
            info[6 * i + 4] = m->cfg.has_energy ? m->pr[i] : m->pr[0];
            info[6 * i + 5] = 0.0;
        }
        if (scat) for (int k = 0; k < 3; ++k) scat[3 * i + k] = m->scat[3 * i + k];
    }
    if (off) std::copy(m->path_off.begin(), m->path_off.end(), off);
    if (idx) std::copy(m->path_idx.begin(), m->path_idx.end(), idx);
    if (len) std::copy(m->path_len.begin(), m->path_len.end(), len);
    if (tail) std::copy(m->path_tail.begin(), m->path_tail.end(), tail);
}

// runs n more iterations (stops early when early_stop triggers); returns iterations done in total
int oracle_mlsd_iterate(void* h, int n) {
    Mlsd* m = static_cast<Mlsd*>(h);
    for (int k = 0; k < n && !m->stopped; ++k) m->iterate_once();
    return m->iters_done;
}

void oracle_mlsd_image(void* h, double* out) {
    Mlsd* m = static_cast<Mlsd*>(h);
    std::copy(m->img.begin(), m->img.end(), out);
}

void oracle_mlsd_set_image(void* h, const double* in) {
    Mlsd* m = static_cast<Mlsd*>(h);
    std::copy(in, in + m->V(), m->img.begin());
}

// per-iteration mean cost history (n entries)
int oracle_mlsd_costs(void* h, double* out, int cap) {
    Mlsd* m = static_cast<Mlsd*>(h);
    const int n = static_cast<int>(m->cost_hist.size());
    for (int k = 0; k < n && k < cap; ++k) out[k] = m->cost_hist[k];
    return n;
}

// One ML step on the current image without changing it: writes the updated
// image to out and the per-voxel multiplicity M_j to mult (optional).
double oracle_mlsd_ml_step(void* h, double* out, uint32_t* mult) {
    Mlsd* m = static_cast<Mlsd*>(h);
    std::vector<double> o(m->V());
    const double c = m->ml_step(m->img, o);
    std::copy(o.begin(), o.end(), out);
    if (mult) std::copy(m->S_index.begin(), m->S_index.end(), mult);
    return c;
}

// Negative log-likelihood of the MLSD model (sum over kept muons of
// log det(Sigma) + 1/2 (a inv00 + b inv11 + 2 c inv01), the per-muon cost of
// src/MutoMLSD.cpp:465-468) and its gradient with respect to log(lambda):
// d/dlog(l_j) = l_j * sum_i pr^2 (tr(Sigma^-1 W_ij) - 1/2 xyS_ij).
// grad may be null.  Not part of the reference (it has no adjoint); it uses
// the same algebra as updateSValueMatrix.
double oracle_mlsd_nll(void* h, const double* lam, double* grad) {
    Mlsd* m = static_cast<Mlsd*>(h);
    const std::vector<double> l(lam, lam + m->V());
    if (grad) std::fill(grad, grad + m->V(), 0.0);
    double total = 0.0;
    for (size_t i = 0; i < m->kept.size(); ++i) {
        const double p = m->cfg.has_energy ? m->pr[i] : m->pr[0];
        const M2 cov = m->covariance(l, m->W[i], p);
        const double det = cov.m[0][0] * cov.m[1][1] - cov.m[1][0] * cov.m[0][1];
        if (!(std::fabs(det) > 1e-12) || det <= 0) continue;
        const double r = 1.0 / det;
        M2 inv;
        inv.m[0][0] = cov.m[1][1] * r;
        inv.m[1][0] = -cov.m[1][0] * r;
        inv.m[0][1] = -cov.m[0][1] * r;
        inv.m[1][1] = cov.m[0][0] * r;
        const double Sx = m->sx[i], Sy = m->sy[i], Dx = m->dx[i], Dy = m->dy[i];
        total += std::log(det) + ((Sx * Sx + Sy * Sy) * inv.m[0][0] + (Dx * Dx + Dy * Dy) * inv.m[1][1] +
                                  (Sx * Dx + Sy * Dy) * 2.0 * inv.m[0][1]) * 0.5;
        if (!grad) continue;
        for (const auto& wj : m->W[i]) {
            const uint32_t j = wj.first;
            if (j >= m->V()) continue;
            const M2 IW = Mlsd::mul(inv, wj.second);
            const M2 C = Mlsd::mul(IW, inv);
            const double xyS = (Sx * Sx + Sy * Sy) * C.m[0][0] + (Dx * Dx + Dy * Dy) * C.m[1][1] +
                               (Sx * Dx + Sy * Dy) * (C.m[0][1] + C.m[1][0]);
            grad[j] += p * p * ((IW.m[0][0] + IW.m[1][1]) - 0.5 * xyS);
        }
    }
    if (grad)
        for (uint64_t j = 0; j < m->V(); ++j) grad[j] *= lam[j];
    return total;
}

}  // extern "C"

extern "C" {
// cubicEqnSolver (src/MutoMAP.cpp:353-406) on its own, for known-answer tests;
// returns the number of roots (1 or 3), -1 when the Newton cap was hit.
int oracle_cubic(double p3, double p2, double p1, double p0, double tol, double* roots) {
    Mlsd m;
    const int n = m.cubic(roots, p3, p2, p1, p0, tol, 1000000);
    return m.n_nonconv ? -1 : n;
}
}
