// Point rules of the QG 1.5-layer model with passive tracers
// (mapping/models/model_qg1l/jqgm.py, class Qgm_trac, 1551-2151): the tracer
// tendency, the tracer boundary update and the Runge-Kutta combination.
//
// Written as host+device functions of one grid point with no CUDA header, so
// the kernels of vd_qgtrac.cu and a host build of the same code run the same
// arithmetic.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define VD_TRAC_HD __host__ __device__ __forceinline__
#else
#define VD_TRAC_HD inline
#endif

namespace vd {

struct TracGeom {
    int ny, nx;
    double cx, cy;      // 1/(6 dx), 1/(6 dy)            (upwind coefficients, jqgm.py:1827-1866)
    double Kx, Ky;      // Kdiffus_trac/dx^2, /dy^2     (used when hasK)
    int hasK;
    double rx, ry;      // (0.5 dt)/dx, (0.5 dt)/dy     (open-boundary ratios, jqgm.py:1965-1972)
    int obc;            // 1: open boundaries on the edge; 0: boundary values on the ring classes
    const int8_t* mask; // [ny][nx]: 0 land, 1/2 rings, 3 interior
};

template <typename T> VD_TRAC_HD T trac_abs(T x) { return x < T(0) ? -x : x; }

// Tracer tendency at (j, i) (jqgm.py:1827-1866): third-order upwind
// advection by the velocities on T points, 0.5 (u(j,i) + u(j,i+1)) and
// 0.5 (v(j,i) + v(j+1,i)), on rows and columns 2..n-3, plus diffusion there;
// NaN -> 0; land -> 0. u, v, c point at the window's / tracer's plane.
template <typename T>
VD_TRAC_HD T trac_rhs_point(const TracGeom& G, const T* u, const T* v, const T* c, int j, int i)
{
    if (j < 2 || j > G.ny - 3 || i < 2 || i > G.nx - 3) return T(0);
    const int nx = G.nx;
    const long long o = (long long)j * nx + i;
    if (G.mask[o] == 0) return T(0);
    const T uT = T(0.5) * (u[o] + u[o + 1]);
    const T vT = T(0.5) * (v[o] + v[o + nx]);
    const T up = uT < T(0) ? T(0) : uT, um = uT > T(0) ? T(0) : uT;
    const T vp = vT < T(0) ? T(0) : vT, vm = vT > T(0) ? T(0) : vT;
    const T cc = c[o];
    const T e1 = c[o + 1], e2 = c[o + 2], w1 = c[o - 1], w2 = c[o - 2];
    const T n1 = c[o + nx], n2 = c[o + 2 * nx], s1 = c[o - nx], s2 = c[o - 2 * nx];
    const T cx = T(G.cx), cy = T(G.cy);
    T r = -up * cx * (T(2) * e1 + T(3) * cc - T(6) * w1 + w2) + um * cx * (e2 - T(6) * e1 + T(3) * cc + T(2) * w1) -
          vp * cy * (T(2) * n1 + T(3) * cc - T(6) * s1 + s2) + vm * cy * (n2 - T(6) * n1 + T(3) * cc + T(2) * s1);
    if (G.hasK) r += T(G.Kx) * (e1 + w1 - T(2) * cc) + T(G.Ky) * (n1 + s1 - T(2) * cc);
    return r != r ? T(0) : r;
}

// Boundary update of one tracer value x = var1(j, i) after a step
// (jqgm.py:1957-2006). a = var0 (start of step), b = boundary field, u, v the
// start-of-step velocities, W the relaxation weights.
// - obc: on the edge (corners excluded) the upstream/downstream blend of
//   Mellor (1996) with ratios r1 = r (w + |w|), r2 = r (w - |w|), w the
//   velocity one point inside (v on rows 1 and ny-1, u on columns 1 and
//   nx-1);
// - otherwise x = b on the ring classes 1 and 2;
// - then on rows and columns 1..n-2: x = W b + (1 - W) x.
template <typename T>
VD_TRAC_HD T trac_bc_point(const TracGeom& G, const T* u, const T* v, const T* a, const T* b, const T* W, T x, int j,
                           int i)
{
    const int ny = G.ny, nx = G.nx;
    const long long o = (long long)j * nx + i;
    const bool in_i = i >= 1 && i <= nx - 2, in_j = j >= 1 && j <= ny - 2;
    if (G.obc) {
        const T ry = T(G.ry), rx = T(G.rx);
        if (j == 0 && in_i) {
            const T w = v[(long long)nx + i];
            const T r1 = ry * (w + trac_abs(w)), r2 = ry * (w - trac_abs(w));
            x = a[o] - (r1 * (a[o] - b[o]) + r2 * (a[o + nx] - a[o]));
        } else if (j == ny - 1 && in_i) {
            const T w = v[o];
            const T r1 = ry * (w + trac_abs(w)), r2 = ry * (w - trac_abs(w));
            x = a[o] - (r1 * (a[o] - a[o - nx]) + r2 * (b[o] - a[o]));
        } else if (i == 0 && in_j) {
            const T w = u[o + 1];
            const T r1 = rx * (w + trac_abs(w)), r2 = rx * (w - trac_abs(w));
            x = a[o] - (r1 * (a[o] - b[o]) + r2 * (a[o + 1] - a[o]));
        } else if (i == nx - 1 && in_j) {
            const T w = u[o];
            const T r1 = rx * (w + trac_abs(w)), r2 = rx * (w - trac_abs(w));
            x = a[o] - (r1 * (a[o] - a[o - 1]) + r2 * (b[o] - a[o]));
        }
    } else if (G.mask[o] == 1 || G.mask[o] == 2) {
        x = b[o];
    }
    if (in_i && in_j) x = W[o] * b[o] + (T(1) - W[o]) * x;
    return x;
}

// Runge-Kutta combination of one value (jqgm.py:1897-1922 and the classical
// fourth-order scheme): k = r dt, then by mode
//   0: out = base + a k                          (Euler a = 1; rk2 a = 1/2, 1)
//   1: acc = k;          out = base + k / 2      (RK4 stage 1)
//   2: acc = acc + 2 k;  out = base + a k        (RK4 stages 2, 3: a = 1/2, 1)
//   3: out = base + (acc + k) / 6                (RK4 stage 4)
template <typename T>
VD_TRAC_HD T rk_combine(int mode, T a, T dt, T r, T base, T* acc)
{
    const T k = r * dt;
    switch (mode) {
    case 1: *acc = k; return base + T(0.5) * k;
    case 2: *acc = *acc + T(2) * k; return base + a * k;
    case 3: return base + (*acc + k) / T(6);
    default: return base + a * k;
    }
}

}  // namespace vd
