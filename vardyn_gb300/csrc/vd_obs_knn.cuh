// Neighbour search of one observation for the observation-operator
// construction (mapping/src/obsop.py:417-460 and, with an exclusion table,
// 197-219), as a host+device function with no CUDA header: the kernel of
// vd_obs.cu runs it per observation and a host build of the same code can be
// checked on the CPU.
//
// On a uniform planar grid (point (i, j) at (i dx, j dy) km) every neighbour
// that survives the dmax test lies within dmax of the observation, so
// scanning the grid points of that disc and keeping the npix nearest gives
// exactly the valid neighbours of a k-nearest search. Ties in distance go to
// the smaller flat index. An excluded point keeps its place among the npix
// nearest but gets no weight.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define VD_KNN_HD __host__ __device__ __forceinline__
#else
#define VD_KNN_HD inline
#endif

namespace vd {

// idx[4], w[4]: grid index (-1 when unused) and normalised weight of each slot.
VD_KNN_HD void obs_knn_point(double xo, double yo, int ny, int nx, double dx, double dy, int npix, double dmax,
                             const unsigned char* excl, long long* idx, double* w)
{
    double bd[4];
    long long bi[4];
    for (int k = 0; k < 4; ++k) {
        bd[k] = INFINITY;
        bi[k] = -1;
    }
    const double d2max = dmax * dmax;
    const int rx = (int)ceil(dmax / dx) + 1, ry = (int)ceil(dmax / dy) + 1;
    const double fx = floor(xo / dx), fy = floor(yo / dy);
    // the disc may lie outside the grid: clamp the scan box in double first
    const double i0d = fmax(fx - rx, 0.0), i1d = fmin(fx + rx + 1, (double)(nx - 1));
    const double j0d = fmax(fy - ry, 0.0), j1d = fmin(fy + ry + 1, (double)(ny - 1));
    if (i0d <= i1d && j0d <= j1d) {
        const int i0 = (int)i0d, i1 = (int)i1d, j0 = (int)j0d, j1 = (int)j1d;
        for (int j = j0; j <= j1; ++j) {
            const double ey = (double)j * dy - yo;
            for (int i = i0; i <= i1; ++i) {
                const double ex = (double)i * dx - xo;
                const double d2 = ex * ex + ey * ey;
                if (d2 > d2max) continue;
                const long long fi = (long long)j * nx + i;
                // insertion into the sorted npix-best list (distance, then index)
                int p = npix;
                while (p > 0 && (d2 < bd[p - 1] || (d2 == bd[p - 1] && fi < bi[p - 1]))) --p;
                if (p >= npix) continue;
                for (int k = npix - 1; k > p; --k) {
                    bd[k] = bd[k - 1];
                    bi[k] = bi[k - 1];
                }
                bd[p] = d2;
                bi[p] = fi;
            }
        }
    }
    double D[4], ww[4], s = 0.0;
    const double c = 2.0 * (0.5 * dmax) * (0.5 * dmax);
    for (int k = 0; k < npix; ++k) {
        D[k] = sqrt(bd[k]);
        // an excluded point keeps its place among the npix nearest but gets no weight
        const bool valid = bi[k] >= 0 && D[k] <= dmax && !(excl && excl[bi[k]]);
        ww[k] = npix > 1 ? (valid ? exp(-D[k] * D[k] / c) : 0.0) : (valid ? 1.0 : 0.0);
        if (!valid) bi[k] = -1;
    }
    for (int k = 0; k < npix; ++k) s += ww[k];
    for (int k = 0; k < 4; ++k) {
        idx[k] = k < npix ? bi[k] : -1;
        w[k] = k < npix ? (npix > 1 ? (s > 0 ? ww[k] / s : 0.0) : ww[k]) : 0.0;
    }
}

}  // namespace vd
