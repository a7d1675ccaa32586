// Least-squares 3-D line fit of one detector record, shared by the host
// reader (MutoFile::getMuonData) and the batched GPU fit (fit.cu).
//
// The reference fits each half of a record (src/MutoFile.cpp:248-304) with
// Eigen's JacobiSVD of the centred hits and takes the first right singular
// vector as the direction.  That vector is the principal axis of the hits'
// 3x3 scatter matrix, found here by cyclic Jacobi rotations on the
// symmetric matrix (Golub & Van Loan, "Matrix Computations", sec. 8.5),
// then oriented with d_z > 0 (the SVD leaves the sign open).  The point is
// the line at the layer next to the grid: pin on layer n_middle-1, pout on
// layer n_middle.
//
// Every product and sum goes through fm/fa/fs, which round each operation
// on its own on the device and on the host (built without contraction), so
// the two builds give the same bits.
#pragma once

#include <cmath>
#include <cstdint>

#include "../../include/muto_gb300.h"

#ifdef __CUDACC__
#define MUTO_FIT_HD __host__ __device__
#else
#define MUTO_FIT_HD
#endif

namespace muto {
namespace fit {

constexpr int kMaxLayers = 64;  // detector layers a record may hold

MUTO_FIT_HD inline double fm(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
MUTO_FIT_HD inline double fa(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
MUTO_FIT_HD inline double fs(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}

// Unit eigenvector of the largest eigenvalue of the symmetric a (which the
// rotations overwrite).
MUTO_FIT_HD inline void principal_axis(double a[3][3], double* out) {
    double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int sweep = 0; sweep < 50; ++sweep) {
        const double off = fa(fa(fm(a[0][1], a[0][1]), fm(a[0][2], a[0][2])), fm(a[1][2], a[1][2]));
        const double diag = fa(fa(fm(a[0][0], a[0][0]), fm(a[1][1], a[1][1])), fm(a[2][2], a[2][2]));
        if (off == 0.0 || off < fm(1e-30, diag)) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (a[p][q] == 0.0) continue;
                const double theta = fs(a[q][q], a[p][p]) / fm(2.0, a[p][q]);
                const double t = (theta >= 0 ? 1.0 : -1.0) / fa(fabs(theta), sqrt(fa(fm(theta, theta), 1.0)));
                const double c = 1.0 / sqrt(fa(fm(t, t), 1.0)), s = fm(t, c);
                for (int k = 0; k < 3; ++k) {  // A <- A J
                    const double akp = a[k][p], akq = a[k][q];
                    a[k][p] = fs(fm(c, akp), fm(s, akq));
                    a[k][q] = fa(fm(s, akp), fm(c, akq));
                }
                for (int k = 0; k < 3; ++k) {  // A <- J^T A
                    const double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = fs(fm(c, apk), fm(s, aqk));
                    a[q][k] = fa(fm(s, apk), fm(c, aqk));
                }
                for (int k = 0; k < 3; ++k) {  // V <- V J
                    const double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = fs(fm(c, vkp), fm(s, vkq));
                    v[k][q] = fa(fm(s, vkp), fm(c, vkq));
                }
            }
    }
    int best = 0;
    for (int k = 1; k < 3; ++k)
        if (a[k][k] > a[best][best]) best = k;
    for (int k = 0; k < 3; ++k) out[k] = v[k][best];
}

// Centroid c and unit direction d (d_z >= 0) of the n hits (x, y, z);
// src/MutoFile.cpp:262-276 and :287-299.
MUTO_FIT_HD inline void fit_line(const double* x, const double* y, const double* z, int n, double* c, double* d) {
    c[0] = c[1] = c[2] = 0.0;
    for (int i = 0; i < n; ++i) {
        c[0] = fa(c[0], x[i]);
        c[1] = fa(c[1], y[i]);
        c[2] = fa(c[2], z[i]);
    }
    const double nn = static_cast<double>(n > 0 ? n : 1);
    for (int k = 0; k < 3; ++k) c[k] = c[k] / nn;
    double a[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int i = 0; i < n; ++i) {
        const double r[3] = {fs(x[i], c[0]), fs(y[i], c[1]), fs(z[i], c[2])};
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q) a[p][q] = fa(a[p][q], fm(r[p], r[q]));
    }
    principal_axis(a, d);
    const double nrm = sqrt(fa(fa(fm(d[0], d[0]), fm(d[1], d[1])), fm(d[2], d[2])));
    if (!(nrm > 0)) {
        d[0] = d[1] = 0.0;
        d[2] = 1.0;
        return;
    }
    const double sgn = d[2] < 0 ? -1.0 : 1.0;
    for (int k = 0; k < 3; ++k) d[k] = fm(sgn, d[k]) / nrm;
}

// One record {ein, x0, y0, ..., x_{nz-1}, y_{nz-1}, eout} (nz <= kMaxLayers)
// to its track (src/MutoFile.cpp:248-304).  Returns false, writing nothing,
// for a record holding a NaN (src/MutoFile.cpp:71-76 drops those).
template <typename T>
MUTO_FIT_HD inline bool fit_record(const T* rec, const double* zl, int nz, int n_middle, muto_ray* out) {
    double hx[kMaxLayers], hy[kMaxLayers];
    const double ein = static_cast<double>(rec[0]);
    const double eout = static_cast<double>(rec[2 * nz + 1]);
    bool nan = ein != ein || eout != eout;
    for (int i = 0; i < nz; ++i) {
        hx[i] = static_cast<double>(rec[1 + 2 * i]);
        hy[i] = static_cast<double>(rec[2 + 2 * i]);
        nan = nan || hx[i] != hx[i] || hy[i] != hy[i];
    }
    if (nan) return false;
    muto_ray r;
    r.ein = ein;
    r.eout = eout;
    double c[3], d[3];
    fit_line(hx, hy, zl, n_middle, c, d);  // upper layers
    double t = fs(zl[n_middle - 1], c[2]) / d[2];
    for (int k = 0; k < 3; ++k) r.din[k] = d[k];
    r.pin[0] = fa(fm(t, d[0]), c[0]);
    r.pin[1] = fa(fm(t, d[1]), c[1]);
    r.pin[2] = zl[n_middle - 1];
    fit_line(hx + n_middle, hy + n_middle, zl + n_middle, nz - n_middle, c, d);  // lower layers
    t = fs(zl[n_middle], c[2]) / d[2];
    for (int k = 0; k < 3; ++k) r.dout[k] = d[k];
    r.pout[0] = fa(fm(t, d[0]), c[0]);
    r.pout[1] = fa(fm(t, d[1]), c[1]);
    r.pout[2] = zl[n_middle];
    *out = r;
    return true;
}

}  // namespace fit
}  // namespace muto
