// Multilayer rotating shallow-water model (mapping/models/model_qgsw/sw.py
// SW, with masks.py, flux.py, reconstruction.py, finite_diff.py): forward
// RK3-SSP steps, their tangent-linear and adjoint, on one GPU.
//
// Layout is the reference's: [batch][layer][x][y] with y contiguous; u on
// (nx+1, ny), v on (nx, ny+1), h on (nx, ny), vorticity on (nx+1, ny+1).
// Inside the model the prognostic fields carry the metric terms
// (u*dx, v*dy, h*area; sw.py:84-100).
//
// One right-hand side is three kernels:
//   k_sw_diag    vorticity (sw.py:678-696), KE + pressure (698-718) and the
//                clamped total thickness (468-481);
//   k_sw_tend    u and v tendencies (483-568: vortex force by WENO-Z fluxes,
//                Coriolis, KE + pressure gradient, wind, drag, viscosity) and
//                the thickness fluxes through the u and v faces;
//   k_sw_update  thickness divergence and diffusion, sponge and the RK3-SSP
//                stage combination (831-877).
// The kernels are templates over the arithmetic type: T for the forward,
// a one-direction dual number for the tangent-linear (jax.jvp of step,
// sw.py:906-922). The adjoint (jax.vjp, 924-938) recomputes each step from
// its stored start and runs hand-written transposes: per face the local
// gradient of the WENO flux (a 6-direction dual number through the same
// reconstruction code) is scattered with atomics, then a gather kernel
// transposes the diagnostics. max(u, 0) takes derivative 1/2 at u = 0, the
// rule of jax's lax.max.
#include "vd_internal.cuh"

#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

namespace vd {
namespace sw {

constexpr int MAXL = 8;
constexpr double WENO_EPS = 1e-4;   // reconstruction.py:13

// ------------------------------------------------------------------ duals
template <typename T, int N>
struct DN {
    T v;
    T d[N];
};

template <typename T> __device__ __forceinline__ T val(T x) { return x; }
template <typename T, int N> __device__ __forceinline__ T val(const DN<T, N>& x) { return x.v; }

#define DN_BIN(OP, DV)                                                                               \
    template <typename T, int N>                                                                     \
    __device__ __forceinline__ DN<T, N> operator OP(const DN<T, N>& a, const DN<T, N>& b)            \
    {                                                                                                \
        DN<T, N> r;                                                                                  \
        r.v = a.v OP b.v;                                                                            \
        _Pragma("unroll") for (int k = 0; k < N; ++k) r.d[k] = DV;                                   \
        return r;                                                                                    \
    }
DN_BIN(+, a.d[k] + b.d[k])
DN_BIN(-, a.d[k] - b.d[k])
DN_BIN(*, a.d[k] * b.v + a.v * b.d[k])
#undef DN_BIN

template <typename T, int N>
__device__ __forceinline__ DN<T, N> operator/(const DN<T, N>& a, const DN<T, N>& b)
{
    DN<T, N> r;
    r.v = a.v / b.v;
    const T ib = T(1) / b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
template <typename T, int N>
__device__ __forceinline__ DN<T, N> operator*(T s, const DN<T, N>& a)
{
    DN<T, N> r;
    r.v = s * a.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = s * a.d[k];
    return r;
}
template <typename T, int N>
__device__ __forceinline__ DN<T, N> operator*(const DN<T, N>& a, T s) { return s * a; }
template <typename T, int N>
__device__ __forceinline__ DN<T, N> operator+(const DN<T, N>& a, T s)
{
    DN<T, N> r = a;
    r.v = a.v + s;
    return r;
}
template <typename T, int N>
__device__ __forceinline__ DN<T, N> operator+(T s, const DN<T, N>& a) { return a + s; }
template <typename T, int N>
__device__ __forceinline__ DN<T, N> operator-(const DN<T, N>& a, T s)
{
    DN<T, N> r = a;
    r.v = a.v - s;
    return r;
}
template <typename T, int N>
__device__ __forceinline__ DN<T, N> operator-(T s, const DN<T, N>& a)
{
    DN<T, N> r;
    r.v = s - a.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
    return r;
}
template <typename T, int N>
__device__ __forceinline__ DN<T, N> operator-(const DN<T, N>& a)
{
    DN<T, N> r;
    r.v = -a.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
    return r;
}
template <typename T, int N>
__device__ __forceinline__ DN<T, N> operator/(const DN<T, N>& a, T s)
{
    DN<T, N> r;
    r.v = a.v / s;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] / s;
    return r;
}
template <typename T, int N>
__device__ __forceinline__ DN<T, N> operator/(T s, const DN<T, N>& b)
{
    DN<T, N> r;
    r.v = s / b.v;
    const T f = -r.v / b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = f * b.d[k];
    return r;
}
template <typename T, int N>
__device__ __forceinline__ DN<T, N> dsqrt(const DN<T, N>& a)
{
    DN<T, N> r;
    r.v = sqrt(a.v);
    const T f = T(0.5) / r.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = f * a.d[k];
    return r;
}
template <typename T> __device__ __forceinline__ T dsqrt(T a) { return sqrt(a); }

// max(x, 0) with jax's tie rule (derivative 1/2 at x = 0)
template <typename T> __device__ __forceinline__ T relu(T x) { return x > T(0) ? x : T(0); }
template <typename T, int N>
__device__ __forceinline__ DN<T, N> relu(const DN<T, N>& x)
{
    DN<T, N> r;
    const T s = x.v > T(0) ? T(1) : (x.v < T(0) ? T(0) : T(0.5));
    r.v = x.v > T(0) ? x.v : T(0);
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = s * x.d[k];
    return r;
}

// softplus(x) = log(1 + e^x) (jax.nn.softplus = logaddexp(x, 0)) and its slope
template <typename T> __device__ __forceinline__ T softplus_v(T x) { return fmax(x, T(0)) + log1p(exp(-fabs(x))); }
template <typename T> __device__ __forceinline__ T sigmoid_v(T x)
{
    if (x >= T(0)) return T(1) / (T(1) + exp(-x));
    const T e = exp(x);
    return e / (T(1) + e);
}
// smooth_clamp (sw.py:27-33): xmin + softplus((x - xmin) s) / s
template <typename T> __device__ __forceinline__ T sclamp(T x, T xmin, T s) { return xmin + softplus_v((x - xmin) * s) / s; }
template <typename T, int N>
__device__ __forceinline__ DN<T, N> sclamp(const DN<T, N>& x, T xmin, T s)
{
    DN<T, N> r;
    const T z = (x.v - xmin) * s;
    r.v = xmin + softplus_v(z) / s;
    const T g = sigmoid_v(z);
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = g * x.d[k];
    return r;
}

template <typename S> __device__ __forceinline__ S sq(const S& x) { return x * x; }

// Division of the WENO-Z weights: IEEE in float64; the fast intrinsic (at
// most 2 ulp) in float32, whose results are compared within float32
// tolerances. The tangent and the local gradient use the same quotient.
__device__ __forceinline__ float qdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double qdiv(double a, double b) { return a / b; }
template <typename T, int N>
__device__ __forceinline__ DN<T, N> qdiv(const DN<T, N>& a, const DN<T, N>& b)
{
    DN<T, N> r;
    r.v = qdiv(a.v, b.v);
    const T ib = qdiv(T(1), b.v);
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}

// ------------------------------------------------------------------ reconstructions
// wenoz4_left / wenoz6_left (reconstruction.py:98-169)
template <typename T, typename S>
__device__ __forceinline__ S wenoz4(const S& qmm, const S& qm, const S& qp, const S& qpp)
{
    (void)qpp;
    const S q1 = T(-0.5) * qmm + T(1.5) * qm;
    const S q2 = T(0.5) * (qm + qp);
    const S b1 = sq(qm - qmm), b2 = sq(qp - qm);
    const S tau = dsqrt(sq(b2 - b1) + T(WENO_EPS * WENO_EPS));
    const S w1 = T(1.0 / 3.0) * (T(1) + qdiv(tau, b1 + T(WENO_EPS)));
    const S w2 = T(2.0 / 3.0) * (T(1) + qdiv(tau, b2 + T(WENO_EPS)));
    return qdiv(w1 * q1 + w2 * q2, w1 + w2);
}

template <typename T, typename S>
__device__ __forceinline__ S wenoz6(const S& q0, const S& q1, const S& q2, const S& q3, const S& q4, const S& q5)
{
    (void)q5;
    const S r1 = T(1.0 / 3.0) * q0 - T(7.0 / 6.0) * q1 + T(11.0 / 6.0) * q2;
    const S r2 = T(-1.0 / 6.0) * q1 + T(5.0 / 6.0) * q2 + T(1.0 / 3.0) * q3;
    const S r3 = T(1.0 / 3.0) * q2 + T(5.0 / 6.0) * q3 - T(1.0 / 6.0) * q4;
    const T k1 = T(13.0 / 12.0), k2 = T(0.25);
    const S b1 = k1 * sq(q0 - T(2) * q1 + q2) + k2 * sq(q0 - T(4) * q1 + T(3) * q2);
    const S b2 = k1 * sq(q1 - T(2) * q2 + q3) + k2 * sq(q1 - q3);
    const S b3 = k1 * sq(q2 - T(2) * q3 + q4) + k2 * sq(T(3) * q2 - T(4) * q3 + q4);
    const S tau = dsqrt(sq(b1 - b3) + T(WENO_EPS * WENO_EPS));
    const S w1 = T(0.1) * (T(1) + qdiv(tau, b1 + T(WENO_EPS)));
    const S w2 = T(0.6) * (T(1) + qdiv(tau, b2 + T(WENO_EPS)));
    const S w3 = T(0.3) * (T(1) + qdiv(tau, b3 + T(WENO_EPS)));
    return qdiv(w1 * r1 + w2 * r2 + w3 * r3, w1 + w2 + w3);
}

// Mask bits of one face: 1 = 2-point, 2 = 4-point, 4 = 6-point term.
// ok4 / ok6: the face is at least 1 / 2 faces from the ends (else that
// reconstruction is the reference's zero padding).
template <typename T, typename S>
__device__ __forceinline__ S recon(const S* q, int bits, bool ok4, bool ok6, bool reverse)
{
    S r = T(0) * q[2];
    if (bits & 1) r = T(0.5) * (q[2] + q[3]);
    if ((bits & 2) && ok4)
        r = r + (reverse ? wenoz4<T>(q[4], q[3], q[2], q[1]) : wenoz4<T>(q[1], q[2], q[3], q[4]));
    if ((bits & 4) && ok6)
        r = r + (reverse ? wenoz6<T>(q[5], q[4], q[3], q[2], q[1], q[0]) : wenoz6<T>(q[0], q[1], q[2], q[3], q[4], q[5]));
    return r;
}

// flux.py:39-90 at one face: q[0..5] = cells k-2..k+3 around face k.
// The velocity's sign selects the upwind stencil: the 6 values are reversed
// lane by lane (selects, no divergent branch) and one reconstruction is
// formed, F = vel * R, which equals up * P + un * N (the other product is an
// exact zero). At vel = 0 the tangent takes both reconstructions with weight
// 1/2 (jax's tie rule for max), a rare branch.
template <typename T, typename S>
__device__ __forceinline__ S weno_flux(const S* q, const S& vel, int bits, bool ok4, bool ok6)
{
    const bool rev = val(vel) < T(0);
    S qq[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) qq[k] = rev ? q[5 - k] : q[k];
    S F = vel * recon<T>(qq, bits, ok4, ok6, false);
    if (val(vel) == T(0)) {
        const S up = relu(vel);
        const S un = vel - up;
        F = up * recon<T>(q, bits, ok4, ok6, false) + un * recon<T>(q, bits, ok4, ok6, true);
    }
    return F;
}

// Reverse-mode gradients of the reconstructions (the same quotients as the
// forward): wenoz4 of (q[1..4]) and wenoz6 of (q[0..5]) accumulate dR/dq
// into g and return R.
template <typename T>
__device__ __forceinline__ T wenoz4_grad(const T* q, T* g)
{
    const T qmm = q[1], qm = q[2], qp = q[3];
    const T q1 = T(-0.5) * qmm + T(1.5) * qm;
    const T q2 = T(0.5) * (qm + qp);
    const T e1 = qm - qmm, e2 = qp - qm;
    const T b1 = e1 * e1, b2 = e2 * e2;
    const T dd = b2 - b1;
    const T tau = sqrt(dd * dd + T(WENO_EPS * WENO_EPS));
    const T s1 = qdiv(T(1), b1 + T(WENO_EPS)), s2 = qdiv(T(1), b2 + T(WENO_EPS));
    const T w1 = T(1.0 / 3.0) * (T(1) + qdiv(tau, b1 + T(WENO_EPS)));
    const T w2 = T(2.0 / 3.0) * (T(1) + qdiv(tau, b2 + T(WENO_EPS)));
    const T W = w1 + w2;
    const T R = qdiv(w1 * q1 + w2 * q2, W);
    const T iW = qdiv(T(1), W);
    const T aw1 = (q1 - R) * iW, aw2 = (q2 - R) * iW;       // dR/dw
    const T ar1 = w1 * iW, ar2 = w2 * iW;                    // dR/dq1, dR/dq2
    const T atau = aw1 * T(1.0 / 3.0) * s1 + aw2 * T(2.0 / 3.0) * s2;
    const T dtau = qdiv(dd, tau);
    const T ab1 = -aw1 * T(1.0 / 3.0) * tau * s1 * s1 - atau * dtau;
    const T ab2 = -aw2 * T(2.0 / 3.0) * tau * s2 * s2 + atau * dtau;
    // b1 = (qm - qmm)^2, b2 = (qp - qm)^2
    g[1] += ar1 * T(-0.5) - ab1 * T(2) * e1;
    g[2] += ar1 * T(1.5) + ar2 * T(0.5) + ab1 * T(2) * e1 - ab2 * T(2) * e2;
    g[3] += ar2 * T(0.5) + ab2 * T(2) * e2;
    return R;
}

template <typename T>
__device__ __forceinline__ T wenoz6_grad(const T* q, T* g)
{
    const T k1 = T(13.0 / 12.0), k2 = T(0.25);
    const T r1 = T(1.0 / 3.0) * q[0] - T(7.0 / 6.0) * q[1] + T(11.0 / 6.0) * q[2];
    const T r2 = T(-1.0 / 6.0) * q[1] + T(5.0 / 6.0) * q[2] + T(1.0 / 3.0) * q[3];
    const T r3 = T(1.0 / 3.0) * q[2] + T(5.0 / 6.0) * q[3] - T(1.0 / 6.0) * q[4];
    const T d1 = q[0] - T(2) * q[1] + q[2], f1 = q[0] - T(4) * q[1] + T(3) * q[2];
    const T d2 = q[1] - T(2) * q[2] + q[3], f2 = q[1] - q[3];
    const T d3 = q[2] - T(2) * q[3] + q[4], f3 = T(3) * q[2] - T(4) * q[3] + q[4];
    const T b1 = k1 * (d1 * d1) + k2 * (f1 * f1);
    const T b2 = k1 * (d2 * d2) + k2 * (f2 * f2);
    const T b3 = k1 * (d3 * d3) + k2 * (f3 * f3);
    const T dd = b1 - b3;
    const T tau = sqrt(dd * dd + T(WENO_EPS * WENO_EPS));
    const T s1 = qdiv(T(1), b1 + T(WENO_EPS)), s2 = qdiv(T(1), b2 + T(WENO_EPS)), s3 = qdiv(T(1), b3 + T(WENO_EPS));
    const T w1 = T(0.1) * (T(1) + qdiv(tau, b1 + T(WENO_EPS)));
    const T w2 = T(0.6) * (T(1) + qdiv(tau, b2 + T(WENO_EPS)));
    const T w3 = T(0.3) * (T(1) + qdiv(tau, b3 + T(WENO_EPS)));
    const T W = w1 + w2 + w3;
    const T R = qdiv(w1 * r1 + w2 * r2 + w3 * r3, W);
    const T iW = qdiv(T(1), W);
    const T aw1 = (r1 - R) * iW, aw2 = (r2 - R) * iW, aw3 = (r3 - R) * iW;
    const T ar1 = w1 * iW, ar2 = w2 * iW, ar3 = w3 * iW;
    const T atau = aw1 * T(0.1) * s1 + aw2 * T(0.6) * s2 + aw3 * T(0.3) * s3;
    const T dtau = qdiv(dd, tau);
    const T ab1 = -aw1 * T(0.1) * tau * s1 * s1 + atau * dtau;
    const T ab2 = -aw2 * T(0.6) * tau * s2 * s2;
    const T ab3 = -aw3 * T(0.3) * tau * s3 * s3 - atau * dtau;
    const T c1 = T(2) * k1 * d1 * ab1, h1 = T(2) * k2 * f1 * ab1;
    const T c2 = T(2) * k1 * d2 * ab2, h2 = T(2) * k2 * f2 * ab2;
    const T c3 = T(2) * k1 * d3 * ab3, h3 = T(2) * k2 * f3 * ab3;
    g[0] += ar1 * T(1.0 / 3.0) + c1 + h1;
    g[1] += ar1 * T(-7.0 / 6.0) + ar2 * T(-1.0 / 6.0) - T(2) * c1 - T(4) * h1 + c2 + h2;
    g[2] += ar1 * T(11.0 / 6.0) + ar2 * T(5.0 / 6.0) + ar3 * T(1.0 / 3.0) + c1 + T(3) * h1 - T(2) * c2 + c3 +
            T(3) * h3;
    g[3] += ar2 * T(1.0 / 3.0) + ar3 * T(5.0 / 6.0) + c2 - h2 - T(2) * c3 - T(4) * h3;
    g[4] += ar3 * T(-1.0 / 6.0) + c3 + h3;
    return R;
}

// Local gradient of the face flux: dF/dq[0..5], dF/dvel.
template <typename T>
__device__ __forceinline__ void weno_flux_grad(const T* q, T vel, int bits, bool ok4, bool ok6, T* g, T& gv)
{
#pragma unroll
    for (int k = 0; k < 6; ++k) g[k] = T(0);
    if (vel == T(0)) {
        const T P = recon<T>(q, bits, ok4, ok6, false), M = recon<T>(q, bits, ok4, ok6, true);
        gv = T(0.5) * (P + M);
        return;
    }
    const bool rev = vel < T(0);
    T qq[6], gg[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        qq[k] = rev ? q[5 - k] : q[k];
        gg[k] = T(0);
    }
    T R = T(0);
    if (bits & 1) {
        R = T(0.5) * (qq[2] + qq[3]);
        gg[2] += T(0.5);
        gg[3] += T(0.5);
    }
    if ((bits & 2) && ok4) R = R + wenoz4_grad(qq, gg);
    if ((bits & 4) && ok6) R = R + wenoz6_grad(qq, gg);
#pragma unroll
    for (int k = 0; k < 6; ++k) g[k] = vel * (rev ? gg[5 - k] : gg[k]);
    gv = R;
}

// ------------------------------------------------------------------ tables
template <typename T>
struct Tab {
    int nx, ny, nl;
    long long su, sv, sh, sw;     // per-layer slab sizes
    const T *dxu, *dyu, *dxv, *dyv, *dxh, *dyh, *area, *areau, *areav;
    const T *fsu, *fsv;           // f* on the u / v grids
    const T *wa, *wb;             // omega = wa*dx(v) - wb*dy(u) (sw.py:687-696)
    const T *wfu, *wfv;           // wind factors dx/(rho H_ref) on interior faces, masked
    const T *href, *hrefu, *hrefv;   // [nl][...] reference thickness (H times area)
    const T *dxp, *dyp;           // [nl][nx-1][ny], [nl][nx][ny-1] or null
    const T *taux, *tauy;         // default wind stress [nx-1][ny], [nx][ny-1]
    const T *gu, *gv, *gh;        // sponge rates (sponge_coef/dt) * sponge
    const T *idxu2, *idxu, *idyu2;   // reciprocals on the u grid: 1/dx^2, 1/dx, 1/dy^2
    const T *idyv2, *idyv, *idxv2;   // on the v grid: 1/dy^2, 1/dy, 1/dx^2
    const T *iarea, *idx2h, *idy2h;  // on the h grid: 1/area, 1/dx^2, 1/dy^2
    const uint8_t *fh, *fu, *fv;  // flag bytes
    const T *dwu, *dwv;           // d(wind factor)/d(face H_ref) on interior faces, masked
    // cotangent accumulators of the H / h_wind dependent tables, summed over
    // batch, stages and steps by the adjoint kernels (null: not accumulated)
    T *ad_href, *ad_hrefu, *ad_hrefv, *ad_dxp, *ad_dyp, *ad_wfu, *ad_wfv;
    // tangents of the same tables (jvp with respect to H / h_wind), read by
    // the dual-number kernels when registered (null: not perturbed)
    const T *d_href, *d_hrefu, *d_hrefv, *d_dxp, *d_dyp, *d_wfu, *d_wfv;
    int wind_mode;                // h_wind: 0 from H (layer 0), 1 scalar, 2 field
    T G[MAXL];                    // G[l] = sum_{k<=l} g'_k
    T gp[MAXL];
    T drag, visc, diff, hmin, sharp, dt;
    T bf_c, bf_gt;                // barotropic filter: 1 / (g dt tau), g tau
    int linear, has_sponge, hxy_dxp, hxy_dyp;
};

// u flags: 1 mask_u, 2/4/8 h-stencil x eq2/eq4/gt6, 16/32/64 w-stencil y eq2/eq4/gt4
// v flags: 1 mask_v, 2/4/8 h-stencil y eq2/eq4/gt6, 16/32/64 w-stencil x eq2/eq4/gt6
// h flags: 1 mask_h

// ------------------------------------------------------------------ accessors
template <typename T>
struct R1 {
    const T* p;
    __device__ __forceinline__ T operator()(long long i) const { return p[i]; }
};
template <typename T>
struct RD {
    const T* p;
    const T* d;
    __device__ __forceinline__ DN<T, 1> operator()(long long i) const
    {
        DN<T, 1> r;
        r.v = p[i];
        r.d[0] = d[i];
        return r;
    }
};
template <typename T>
struct W1 {
    T* p;
    __device__ __forceinline__ void operator()(long long i, T x) const { p[i] = x; }
};
template <typename T>
struct WD {
    T* p;
    T* d;
    __device__ __forceinline__ void operator()(long long i, const DN<T, 1>& x) const
    {
        p[i] = x.v;
        d[i] = x.d[0];
    }
};

template <typename R> struct Tri { R u, v, h; };

// A table value as the kernel's arithmetic type: the plain value, or for the
// dual-number (tangent) kernels the value with its registered tangent
// (0 when none); p null reads as 0.
template <typename T>
__device__ __forceinline__ T tab_val(const T* p, const T*, long long i, T*)
{
    return p ? p[i] : T(0);
}
template <typename T>
__device__ __forceinline__ DN<T, 1> tab_val(const T* p, const T* d, long long i, DN<T, 1>*)
{
    DN<T, 1> r;
    r.v = p ? p[i] : T(0);
    r.d[0] = d ? d[i] : T(0);
    return r;
}
#define VD_TAB(S, p, d, i) tab_val((p), (d), (i), (S*)nullptr)

// ------------------------------------------------------------------ k_sw_diag
// One thread per (x, y) of the vorticity grid and batch member; loops over
// layers (pressure is a cumulative sum over layers).
template <typename T, typename S, typename R, typename W>
__global__ void k_sw_diag(Tab<T> t, Tri<R> x, W om, W kp, W ht)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const int nx = t.nx, ny = t.ny, nl = t.nl;
    if (i > nx || j > ny) return;
    const long long wi = (long long)i * (ny + 1) + j;
    const T wa = t.wa[wi], wb = t.wb[wi];
    const bool hp = (i < nx && j < ny);
    const long long hi = (long long)i * ny + j;
    S pacc = T(0) * x.h((long long)b * nl * t.sh);
    S hl[MAXL];
    for (int l = 0; l < nl; ++l) {
        const long long ob = (long long)(b * nl + l);
        const R& U = x.u;
        const R& V = x.v;
        // omega: dx(v) with v = 0 outside x in [0, nx); dy(u) with u = 0 outside y in [0, ny)
        const S z = T(0) * U(ob * t.su);
        const S vr = (i < nx) ? V(ob * t.sv + (long long)i * (ny + 1) + j) : z;
        const S vl = (i > 0) ? V(ob * t.sv + (long long)(i - 1) * (ny + 1) + j) : z;
        const S uu = (j < ny) ? U(ob * t.su + (long long)i * ny + j) : z;
        const S ud = (j > 0) ? U(ob * t.su + (long long)i * ny + j - 1) : z;
        om(ob * t.sw + wi, wa * (vr - vl) - wb * (uu - ud));
        if (hp) hl[l] = x.h(ob * t.sh + hi);
    }
    if (!hp) return;
    const T mh = (t.fh[hi] & 1) ? T(1) : T(0);
    const T ar = t.area[hi], iar = t.iarea[hi];
    // eta_l = sum_{m>=l} h_m / area; p_l = sum_{k<=l} g'_k eta_k (sw.py:705-706)
    S eta[MAXL];
    {
        S acc = hl[nl - 1] * iar;
        eta[nl - 1] = acc;
        for (int l = nl - 2; l >= 0; --l) {
            acc = hl[l] * iar + acc;
            eta[l] = acc;
        }
    }
    for (int l = 0; l < nl; ++l) {
        const long long ob = (long long)(b * nl + l);
        pacc = pacc + t.gp[l] * eta[l];
        // kinetic energy (finite_diff.py:20-24): 0.25 (u U + ... ) * mask_h
        const long long u0 = ob * t.su + (long long)i * ny + j, u1 = u0 + ny;
        const long long v0 = ob * t.sv + (long long)i * (ny + 1) + j, v1 = v0 + 1;
        const S a = x.u(u1), c = x.u(u0), d = x.v(v1), e = x.v(v0);
        const T iu1 = t.idxu2[(long long)(i + 1) * ny + j], iu0 = t.idxu2[(long long)i * ny + j];
        const T iv1 = t.idyv2[(long long)i * (ny + 1) + j + 1], iv0 = t.idyv2[(long long)i * (ny + 1) + j];
        const S ke = T(0.25) * (a * (a * iu1) + c * (c * iu0) + d * (d * iv1) + e * (e * iv0)) * mh;
        kp(ob * t.sh + hi, ke + pacc);
        const S hr = VD_TAB(S, t.href, t.d_href, (long long)l * t.sh + hi);
        if (t.linear) ht(ob * t.sh + hi, hr + T(0) * hl[l]);
        else ht(ob * t.sh + hi, sclamp(hr + hl[l], t.hmin * ar, t.sharp));
    }
}

// ------------------------------------------------------------------ k_sw_tend
// u / v tendencies (masked) and the thickness fluxes through interior faces.
template <typename T, typename S, typename R, typename W>
__global__ void k_sw_tend(Tab<T> t, Tri<R> x, R om, R kp, R ht, const T* taux, const T* tauy, W tu, W tv, W fx,
                          W fy)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int bl = blockIdx.z;
    const int nx = t.nx, ny = t.ny, nl = t.nl, l = bl % nl;
    if (i > nx || j > ny) return;
    const long long ob = bl;
    const S z = T(0) * x.h(ob * t.sh);
    // ---------------- u point (i, j)
    if (j < ny) {
        const long long ui = (long long)i * ny + j;
        const int fl = t.fu[ui];
        S du = z, F = z;
        if (i >= 1 && i <= nx - 1) {
            // V at u points: interp_TP(V) (finite_diff.py:6-7)
            const long long vb = ob * t.sv;
            auto Vv = [&](int a, int c) {
                const long long k = (long long)a * (ny + 1) + c;
                return x.v(vb + k) * t.idyv2[k];
            };
            const S Vm = T(0.25) * (Vv(i, j + 1) + Vv(i, j) + Vv(i - 1, j + 1) + Vv(i - 1, j));
            // vortex force: WENO flux of omega[i][.] along y through face j
            S q[6];
            const long long wb = ob * t.sw + (long long)i * (ny + 1);
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const int jj = j - 2 + k;
                q[k] = (jj >= 0 && jj <= ny) ? om(wb + jj) : z;
            }
            const int bits = (fl >> 4) & 7;
            const S oVm = weno_flux<T>(q, Vm, bits, j >= 1 && j <= ny - 2, j >= 2 && j <= ny - 3);
            du = oVm + t.fsu[ui] * Vm;
            const S kpd = kp(ob * t.sh + ui) - kp(ob * t.sh + ui - ny);
            const long long pi = (long long)l * (nx - 1) * ny + (long long)(i - 1) * ny + j;
            if constexpr (std::is_same<S, T>::value) {
                du = du - (t.hxy_dxp ? kpd + t.dxp[pi] : kpd);
                if (l == 0) du = du + (taux ? taux : t.taux)[(long long)(i - 1) * ny + j] * t.wfu[ui];
            } else {
                du = du - ((t.hxy_dxp || t.d_dxp) ? kpd + VD_TAB(S, t.hxy_dxp ? t.dxp : nullptr, t.d_dxp, pi) : kpd);
                if (l == 0) du = du + (taux ? taux : t.taux)[(long long)(i - 1) * ny + j] * VD_TAB(S, t.wfu, t.d_wfu, ui);
            }
            if (l == nl - 1) du = du - t.drag * x.u(ob * t.su + ui);
            if (t.visc > T(0)) {
                const long long ub = ob * t.su;
                auto up = [&](int a, int c) {
                    c = c < 0 ? 0 : (c > ny - 1 ? ny - 1 : c);
                    const long long k = (long long)a * ny + c;
                    return x.u(ub + k) * t.idxu[k];
                };
                const S c0 = up(i, j);
                const S lap = (up(i + 1, j) - T(2) * c0 + up(i - 1, j)) * t.idxu2[ui] +
                              (up(i, j + 1) - T(2) * c0 + up(i, j - 1)) * t.idyu2[ui];
                du = du + t.visc * lap * t.dxu[ui];
            }
            du = du * ((fl & 1) ? T(1) : T(0));
            // thickness flux along x through u face i
            const S Uf = x.u(ob * t.su + ui) * t.idxu2[ui];
            S hq[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const int ii = i - 3 + k;   // cells i-3 .. i+2 around face i (between cells i-1, i)
                hq[k] = (ii >= 0 && ii < nx) ? ht(ob * t.sh + (long long)ii * ny + j) : z;
            }
            F = weno_flux<T>(hq, Uf, (fl >> 1) & 7, i >= 2 && i <= nx - 2, i >= 3 && i <= nx - 3);
        }
        tu(ob * t.su + ui, du);
        fx(ob * t.su + ui, F);
    }
    // ---------------- v point (i, j)
    if (i < nx) {
        const long long vi = (long long)i * (ny + 1) + j;
        const int fl = t.fv[vi];
        S dv = z, F = z;
        if (j >= 1 && j <= ny - 1) {
            const long long ub = ob * t.su;
            auto Uu = [&](int a, int c) {
                const long long k = (long long)a * ny + c;
                return x.u(ub + k) * t.idxu2[k];
            };
            const S Um = T(0.25) * (Uu(i + 1, j) + Uu(i + 1, j - 1) + Uu(i, j) + Uu(i, j - 1));
            S q[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const int ii = i - 2 + k;
                q[k] = (ii >= 0 && ii <= nx) ? om(ob * t.sw + (long long)ii * (ny + 1) + j) : z;
            }
            const int bits = (fl >> 4) & 7;
            const S oUm = weno_flux<T>(q, Um, bits, i >= 1 && i <= nx - 2, i >= 2 && i <= nx - 3);
            dv = -(oUm + t.fsv[vi] * Um);
            const long long hi = (long long)i * ny + j;
            const S kpd = kp(ob * t.sh + hi) - kp(ob * t.sh + hi - 1);
            const long long pj = (long long)l * nx * (ny - 1) + (long long)i * (ny - 1) + j - 1;
            if constexpr (std::is_same<S, T>::value) {
                dv = dv - (t.hxy_dyp ? kpd + t.dyp[pj] : kpd);
                if (l == 0) dv = dv + (tauy ? tauy : t.tauy)[(long long)i * (ny - 1) + j - 1] * t.wfv[vi];
            } else {
                dv = dv - ((t.hxy_dyp || t.d_dyp) ? kpd + VD_TAB(S, t.hxy_dyp ? t.dyp : nullptr, t.d_dyp, pj) : kpd);
                if (l == 0) dv = dv + (tauy ? tauy : t.tauy)[(long long)i * (ny - 1) + j - 1] * VD_TAB(S, t.wfv, t.d_wfv, vi);
            }
            if (l == nl - 1) dv = dv - t.drag * x.v(ob * t.sv + vi);
            if (t.visc > T(0)) {
                const long long vb = ob * t.sv;
                auto vp = [&](int a, int c) {
                    a = a < 0 ? 0 : (a > nx - 1 ? nx - 1 : a);
                    const long long k = (long long)a * (ny + 1) + c;
                    return x.v(vb + k) * t.idyv[k];
                };
                const S c0 = vp(i, j);
                const S lap = (vp(i + 1, j) - T(2) * c0 + vp(i - 1, j)) * t.idxv2[vi] +
                              (vp(i, j + 1) - T(2) * c0 + vp(i, j - 1)) * t.idyv2[vi];
                dv = dv + t.visc * lap * t.dyv[vi];
            }
            dv = dv * ((fl & 1) ? T(1) : T(0));
            const S Vf = x.v(ob * t.sv + vi) * t.idyv2[vi];
            S hq[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const int jj = j - 3 + k;
                hq[k] = (jj >= 0 && jj < ny) ? ht(ob * t.sh + (long long)i * ny + jj) : z;
            }
            F = weno_flux<T>(hq, Vf, (fl >> 1) & 7, j >= 2 && j <= ny - 2, j >= 3 && j <= ny - 3);
        }
        tv(ob * t.sv + vi, dv);
        fy(ob * t.sv + vi, F);
    }
}

// ------------------------------------------------------------------ k_sw_update
// k_s = tendency + sponge; next = RK3-SSP stage combination (+ forcing).
struct StageArgs {
    int stage;        // 0, 1, 2
    int forcing;      // stage 2: add dt*F
};

template <typename T, typename S, typename R, typename W>
__global__ void k_sw_update(Tab<T> t, StageArgs sa, Tri<R> x, R tu, R tv, R fx, R fy, Tri<R> k0, Tri<R> k1,
                            Tri<R> xb, Tri<R> F, Tri<W> ks, Tri<W> nx_)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int bl = blockIdx.z;
    const int nx = t.nx, ny = t.ny;
    if (i > nx || j > ny) return;
    const long long ob = bl;
    const T dt = t.dt;
    auto combine = [&](const S& xv, const S& k, const R& K0, const R& K1, const R& FF, long long idx, const W& wk,
                       const W& wn) {
        if (sa.stage == 0) {
            wk(idx, k);
            wn(idx, xv + dt * k);
        } else if (sa.stage == 1) {
            wk(idx, k);
            wn(idx, xv + (dt / T(4)) * (k - T(3) * K0(idx)));
        } else {
            S n = xv + (dt / T(12)) * (T(8) * k - K1(idx) - K0(idx));
            if (sa.forcing) n = n + dt * FF(idx);
            wn(idx, n);
        }
    };
    if (j < ny) {   // u point
        const long long ui = (long long)i * ny + j, idx = ob * t.su + ui;
        const S xv = x.u(idx);
        S k = tu(idx);
        if (t.has_sponge) k = k + t.gu[ui] * (xb.u(idx) - xv);
        combine(xv, k, k0.u, k1.u, F.u, idx, ks.u, nx_.u);
    }
    if (i < nx) {   // v point
        const long long vi = (long long)i * (ny + 1) + j, idx = ob * t.sv + vi;
        const S xv = x.v(idx);
        S k = tv(idx);
        if (t.has_sponge) k = k + t.gv[vi] * (xb.v(idx) - xv);
        combine(xv, k, k0.v, k1.v, F.v, idx, ks.v, nx_.v);
    }
    if (i < nx && j < ny) {   // h point
        const long long hi = (long long)i * ny + j, idx = ob * t.sh + hi;
        const S xv = x.h(idx);
        const T mh = (t.fh[hi] & 1) ? T(1) : T(0);
        // div_nofluxbc (finite_diff.py:44-52): no x (y) contribution in the
        // first and last cells along x (y)
        const S z = T(0) * xv;
        S dvx = z, dvy = z;
        if (i >= 1 && i <= nx - 2)
            dvx = fx(ob * t.su + (long long)(i + 1) * ny + j) - fx(ob * t.su + (long long)i * ny + j);
        if (j >= 1 && j <= ny - 2)
            dvy = fy(ob * t.sv + (long long)i * (ny + 1) + j + 1) - fy(ob * t.sv + (long long)i * (ny + 1) + j);
        S k = -(dvy + dvx) * mh;
        if (t.diff > T(0)) {
            auto hp = [&](int a, int c) {
                a = a < 0 ? 0 : (a > nx - 1 ? nx - 1 : a);
                c = c < 0 ? 0 : (c > ny - 1 ? ny - 1 : c);
                const long long q = (long long)a * ny + c;
                return x.h(ob * t.sh + q) * t.iarea[q];
            };
            const S c0 = hp(i, j);
            const S lap = (hp(i + 1, j) - T(2) * c0 + hp(i - 1, j)) * t.idx2h[hi] +
                          (hp(i, j + 1) - T(2) * c0 + hp(i, j - 1)) * t.idy2h[hi];
            k = k + t.diff * lap * t.area[hi] * mh;
        }
        if (t.has_sponge) k = k + t.gh[hi] * (xb.h(idx) - xv);
        combine(xv, k, k0.h, k1.h, F.h, idx, ks.h, nx_.h);
    }
}

// ------------------------------------------------------------------ mass-consistent forcing
// replicate_pad (sw.py:36-48) value at padded cell (pi, pj) of field f.
template <typename T, typename S, typename R>
__device__ __forceinline__ S rep_pad(const Tab<T>& t, const R& f, long long base, int pi, int pj)
{
    const int nx = t.nx, ny = t.ny;
    auto cl = [](int a, int n) { return a < 0 ? 0 : (a > n - 1 ? n - 1 : a); };
    const int ci = cl(pi - 1, nx), cj = cl(pj - 1, ny);
    if (t.fh[(long long)ci * ny + cj] & 1) return f(base + (long long)ci * ny + cj);
    S s = T(0) * f(base);
    int ms = 0;
    for (int a = pi - 1; a <= pi + 1; ++a)
        for (int c = pj - 1; c <= pj + 1; ++c) {
            if (a < 0 || a > nx + 1 || c < 0 || c > ny + 1) continue;
            const int ai = cl(a - 1, nx), aj = cl(c - 1, ny);
            s = s + f(base + (long long)ai * ny + aj);
            ms += (t.fh[(long long)ai * ny + aj] & 1);
        }
    return s / T(ms > 1 ? ms : 1);
}

template <typename T, typename S, typename R, typename W>
__global__ void k_sw_force_mc(Tab<T> t, Tri<R> x, Tri<R> F, Tri<W> out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int bl = blockIdx.z, l = bl % t.nl;
    const int nx = t.nx, ny = t.ny;
    if (i > nx || j > ny) return;
    const long long ob = bl, hb = ob * t.sh;
    const T dt = t.dt;
    if (j < ny) {
        const long long ui = (long long)i * ny + j, idx = ob * t.su + ui;
        const S hu = T(0.5) * (rep_pad<T, S>(t, x.h, hb, i + 1, j + 1) + rep_pad<T, S>(t, x.h, hb, i, j + 1));
        const S fu = T(0.5) * (rep_pad<T, S>(t, F.h, hb, i + 1, j + 1) + rep_pad<T, S>(t, F.h, hb, i, j + 1));
        const S htu = sclamp(VD_TAB(S, t.hrefu, t.d_hrefu, (long long)l * t.su + ui) + hu, t.hmin * t.areau[ui], t.sharp);
        const S u = x.u(idx);
        S n = u + dt * ((-u) / htu * fu);
        out.u(idx, n + dt * F.u(idx));
    }
    if (i < nx) {
        const long long vi = (long long)i * (ny + 1) + j, idx = ob * t.sv + vi;
        const S hv = T(0.5) * (rep_pad<T, S>(t, x.h, hb, i + 1, j + 1) + rep_pad<T, S>(t, x.h, hb, i + 1, j));
        const S fv = T(0.5) * (rep_pad<T, S>(t, F.h, hb, i + 1, j + 1) + rep_pad<T, S>(t, F.h, hb, i + 1, j));
        const S htv = sclamp(VD_TAB(S, t.hrefv, t.d_hrefv, (long long)l * t.sv + vi) + hv, t.hmin * t.areav[vi], t.sharp);
        const S v = x.v(idx);
        S n = v + dt * ((-v) / htv * fv);
        out.v(idx, n + dt * F.v(idx));
    }
    if (i < nx && j < ny) {
        const long long idx = hb + (long long)i * ny + j;
        out.h(idx, x.h(idx) + dt * F.h(idx));
    }
}

// ------------------------------------------------------------------ H / h_wind cotangents
// Pull the accumulated table cotangents back to H (every layer's thickness,
// [nl][nx][ny]) and to a field h_wind ([nx][ny]), transposing the plan's
// table construction (sw.py:386-406 reference values, 567-640 wind depth):
//   h_ref = H area; h_ref on u / v faces = edge-padded averages;
//   eta_l = -sum_{m<l} H_m, p_l = sum_{k<=l} g'_k eta_k, dxp / dyp = diffs of p;
//   wind factor = dx / (rho max(H_face, h_min)), H_face from h_wind (average
//   of the two cells); without h_wind it comes from the model's own H, which
//   the H argument does not reach (sw.py:622-630), so it adds nothing to adH.
template <typename T>
__global__ void k_sw_ref_pullback(Tab<T> t, const T* a_href, const T* a_hrefu, const T* a_hrefv, const T* a_dxp,
                                  const T* a_dyp, const T* a_wfu, const T* a_wfv, T* adH, T* adhw)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int nx = t.nx, ny = t.ny, nl = t.nl;
    if (i >= nx || j >= ny) return;
    const long long hi = (long long)i * ny + j;
    auto Au = [&](int l, int f) { return a_hrefu[(long long)l * t.su + (long long)f * ny + j]; };
    auto Av = [&](int l, int c) { return a_hrefv[(long long)l * t.sv + (long long)i * (ny + 1) + c]; };
    T aH[MAXL];
    for (int l = 0; l < nl; ++l) {
        T a = a_href[(long long)l * t.sh + hi];
        a += T(0.5) * (Au(l, i) + Au(l, i + 1));
        if (i == 0) a += T(0.5) * Au(l, 0);
        if (i == nx - 1) a += T(0.5) * Au(l, nx);
        a += T(0.5) * (Av(l, j) + Av(l, j + 1));
        if (j == 0) a += T(0.5) * Av(l, 0);
        if (j == ny - 1) a += T(0.5) * Av(l, ny);
        aH[l] = a * t.area[hi];
    }
    if (t.hxy_dxp) {
        T ap[MAXL], aeta[MAXL];
        for (int l = 0; l < nl; ++l) {
            const long long bx = (long long)l * (nx - 1) * ny, by = (long long)l * nx * (ny - 1);
            T a = T(0);
            if (i >= 1) a += a_dxp[bx + (long long)(i - 1) * ny + j];
            if (i <= nx - 2) a -= a_dxp[bx + (long long)i * ny + j];
            if (j >= 1) a += a_dyp[by + (long long)i * (ny - 1) + j - 1];
            if (j <= ny - 2) a -= a_dyp[by + (long long)i * (ny - 1) + j];
            ap[l] = a;
        }
        T suf = T(0);
        for (int l = nl - 1; l >= 0; --l) {
            suf += ap[l];
            aeta[l] = t.gp[l] * suf;
        }
        T above = T(0);
        for (int m = nl - 1; m >= 0; --m) {
            aH[m] -= above;
            above += aeta[m];
        }
    }
    for (int l = 0; l < nl; ++l) adH[(long long)l * t.sh + hi] = aH[l];
    if (adhw) {
        T a = T(0);
        if (t.wind_mode == 2) {
            auto Gu = [&](int f) -> T {
                if (f < 1 || f > nx - 1) return T(0);
                const long long k = (long long)f * ny + j;
                return a_wfu[k] * t.dwu[k];
            };
            auto Gv = [&](int c) -> T {
                if (c < 1 || c > ny - 1) return T(0);
                const long long k = (long long)i * (ny + 1) + c;
                return a_wfv[k] * t.dwv[k];
            };
            a = T(0.5) * (Gu(i) + Gu(i + 1) + Gv(j) + Gv(j + 1));
        }
        adhw[hi] = a;
    }
}

// ------------------------------------------------------------------ conversions
// set_input_uvh (sw.py:432-450) and get_physical_uvh (421-427); the adjoint
// of either is the same diagonal scaling.
template <typename T>
__global__ void k_sw_scale(Tab<T> t, int nf, int mode, const T* u, const T* v, const T* h, T* uo, T* vo, T* ho)
{
    // mode 0: to model (mask, times metric); 1: to physical (divide)
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int f = blockIdx.z;
    const int nx = t.nx, ny = t.ny;
    if (i > nx || j > ny || f >= nf) return;
    if (j < ny && u) {
        const long long k = (long long)i * ny + j, o = f * t.su + k;
        uo[o] = mode == 0 ? u[o] * ((t.fu[k] & 1) ? T(1) : T(0)) * t.dxu[k] : u[o] / t.dxu[k];
    }
    if (i < nx && v) {
        const long long k = (long long)i * (ny + 1) + j, o = f * t.sv + k;
        vo[o] = mode == 0 ? v[o] * ((t.fv[k] & 1) ? T(1) : T(0)) * t.dyv[k] : v[o] / t.dyv[k];
    }
    if (i < nx && j < ny && h) {
        const long long k = (long long)i * ny + j, o = f * t.sh + k;
        ho[o] = mode == 0 ? h[o] * ((t.fh[k] & 1) ? T(1) : T(0)) * t.area[k] : h[o] / t.area[k];
    }
}

// ------------------------------------------------------------------ adjoint kernels
// Reverse of k_sw_update for one stage (elementwise): from the adjoint of the
// stage output (adn, updated in place to the adjoint of the stage input's
// direct path) build adk (adjoint of this stage's k) and accumulate the
// adjoints of the earlier k's and of the sponge target.
template <typename T>
__global__ void k_sw_update_adj(Tab<T> t, int stage, int nf, T* adn_u, T* adn_v, T* adn_h, T* adk_u, T* adk_v,
                                T* adk_h, T* a0_u, T* a0_v, T* a0_h, T* a1_u, T* a1_v, T* a1_h, T* ab_u, T* ab_v,
                                T* ab_h)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int f = blockIdx.z;
    const int nx = t.nx, ny = t.ny;
    if (i > nx || j > ny || f >= nf) return;
    const T dt = t.dt;
    auto one = [&](long long o, T g, T* an, T* ak, T* a0, T* a1, T* ab) {
        const T a = an[o];
        T k;
        if (stage == 2) {
            k = (dt / T(12)) * T(8) * a;
            a1[o] += -(dt / T(12)) * a;
            a0[o] += -(dt / T(12)) * a;
        } else if (stage == 1) {
            k = a1[o] + (dt / T(4)) * a;
            a0[o] += -(dt / T(4)) * T(3) * a;
        } else {
            k = a0[o] + dt * a;
        }
        ak[o] = k;
        if (t.has_sponge) {
            an[o] = a - g * k;
            if (ab) ab[o] += g * k;
        }
    };
    if (j < ny) {
        const long long k = (long long)i * ny + j;
        one(f * t.su + k, t.has_sponge ? t.gu[k] : T(0), adn_u, adk_u, a0_u, a1_u, ab_u);
    }
    if (i < nx) {
        const long long k = (long long)i * (ny + 1) + j;
        one(f * t.sv + k, t.has_sponge ? t.gv[k] : T(0), adn_v, adk_v, a0_v, a1_v, ab_v);
    }
    if (i < nx && j < ny) {
        const long long k = (long long)i * ny + j;
        one(f * t.sh + k, t.has_sponge ? t.gh[k] : T(0), adn_h, adk_h, a0_h, a1_h, ab_h);
    }
}

// Atomic accumulation, used only where sums run over the batch into the H /
// h_wind table cotangents and by the mass-consistent forcing adjoint.
template <typename T> __device__ __forceinline__ void aadd(T* p, T v) { atomicAdd(p, v); }

// Adjoint of k_sw_tend and of the divergence / diffusion part of
// k_sw_update, in two passes with no atomics.
//
// Pass 1 (k_sw_tend_adj_src, one thread per point): every source point of
// the forward tendency stores the cotangents it contributes, one value per
// (source, term): at u faces the tendency cotangent a (KE + pressure, drag),
// a * dF/dq_k of its vorticity WENO flux (k = 0..5), the V-average term, the
// viscosity coefficient, aF * dF/dq_k of the thickness flux through the face
// and the face's own flux-velocity term; the same at v faces; and the
// thickness-diffusion coefficient at h points. Every index in range is
// written (zeros where a point contributes nothing).
// Pass 2 (k_sw_tend_adj_gather, one thread per target point): each target
// sums, in a fixed order, the stored terms of the sources whose stencils
// reach it (the inverse of each forward stencil, including the clamped
// viscosity and diffusion neighbours at the edges). The sums are therefore
// the same on every run. The H / h_wind table cotangents (only when
// registered) still accumulate with atomics over the batch.

template <typename T>
struct SwSrc {
    T *ua, *uvm, *uc, *uf;   // [bl][su] u faces: a, V-average term, viscosity coefficient, own flux term
    T *uw, *uh;              // [6][bl][su]: vorticity and thickness WENO terms
    T *va, *vum, *vc, *vf;   // [bl][sv] v faces
    T *vw, *vh;              // [6][bl][sv]
    T *hd;                   // [bl][sh] thickness-diffusion coefficient
    long long nu, nv;        // bl * su, bl * sv: stride of the six-term arrays
};

template <typename T>
__global__ void k_sw_tend_adj_src(Tab<T> t, const T* u, const T* v, const T* h, const T* om, const T* ht,
                                  const T* adk_u, const T* adk_v, const T* adk_h, SwSrc<T> S, const T* taux,
                                  const T* tauy)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int bl = blockIdx.z;
    const int nx = t.nx, ny = t.ny, nl = t.nl, l = bl % nl;
    if (i > nx || j > ny) return;
    const long long ob = bl;
    const T* hb = adk_h + ob * t.sh;
    auto mh = [&](long long k) { return (t.fh[k] & 1) ? T(1) : T(0); };
    // ---------------- u face (i, j)
    if (j < ny) {
        const long long ui = (long long)i * ny + j, so = ob * t.su + ui;
        T a_s = T(0), vm_s = T(0), c_s = T(0), f_s = T(0), w_s[6], h_s[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) w_s[k] = h_s[k] = T(0);
        if (i >= 1 && i <= nx - 1) {
            const int fl = t.fu[ui];
            const T a = adk_u[so] * ((fl & 1) ? T(1) : T(0));
            if (a != T(0)) {
                const long long vb = ob * t.sv;
                auto Vv = [&](int p, int c) {
                    const long long k = (long long)p * (ny + 1) + c;
                    return v[vb + k] * t.idyv2[k];
                };
                const T Vm = T(0.25) * (Vv(i, j + 1) + Vv(i, j) + Vv(i - 1, j + 1) + Vv(i - 1, j));
                T q[6];
                const long long wb = ob * t.sw + (long long)i * (ny + 1);
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    const int jj = j - 2 + k;
                    q[k] = (jj >= 0 && jj <= ny) ? om[wb + jj] : T(0);
                }
                T g[6], gv;
                weno_flux_grad<T>(q, Vm, (fl >> 4) & 7, j >= 1 && j <= ny - 2, j >= 2 && j <= ny - 3, g, gv);
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    const int jj = j - 2 + k;
                    if (jj >= 0 && jj <= ny && g[k] != T(0)) w_s[k] = a * g[k];
                }
                vm_s = T(0.25) * a * (gv + t.fsu[ui]);
                a_s = a;
                // reference pressure gradient and wind factor (H / h_wind cotangents)
                if (t.ad_dxp && t.hxy_dxp)
                    aadd(&t.ad_dxp[(long long)l * (nx - 1) * ny + (long long)(i - 1) * ny + j], -a);
                if (t.ad_wfu && l == 0) aadd(&t.ad_wfu[ui], a * (taux ? taux : t.taux)[(long long)(i - 1) * ny + j]);
                if (t.visc > T(0)) c_s = t.visc * t.dxu[ui] * a;
            }
            // thickness flux through u face i: dt_h[c] = -div_x[c] * mask_h[c]
            T aF = T(0);
            if (i - 1 >= 1 && i - 1 <= nx - 2) aF -= mh((long long)(i - 1) * ny + j) * hb[(long long)(i - 1) * ny + j];
            if (i >= 1 && i <= nx - 2) aF += mh(ui) * hb[ui];
            if (aF != T(0)) {
                const T iu2 = t.idxu2[ui];
                const T Uf = u[so] * iu2;
                T q[6];
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    const int ii = i - 3 + k;
                    q[k] = (ii >= 0 && ii < nx) ? ht[ob * t.sh + (long long)ii * ny + j] : T(0);
                }
                T g[6], gv;
                weno_flux_grad<T>(q, Uf, (fl >> 1) & 7, i >= 2 && i <= nx - 2, i >= 3 && i <= nx - 3, g, gv);
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    const int ii = i - 3 + k;
                    if (ii >= 0 && ii < nx && g[k] != T(0)) h_s[k] = aF * g[k];
                }
                f_s = aF * gv * iu2;
            }
        }
        S.ua[so] = a_s;
        S.uvm[so] = vm_s;
        S.uc[so] = c_s;
        S.uf[so] = f_s;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            S.uw[k * S.nu + so] = w_s[k];
            S.uh[k * S.nu + so] = h_s[k];
        }
    }
    // ---------------- v face (i, j)
    if (i < nx) {
        const long long vi = (long long)i * (ny + 1) + j, so = ob * t.sv + vi;
        T a_s = T(0), um_s = T(0), c_s = T(0), f_s = T(0), w_s[6], h_s[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) w_s[k] = h_s[k] = T(0);
        if (j >= 1 && j <= ny - 1) {
            const int fl = t.fv[vi];
            const T a = adk_v[so] * ((fl & 1) ? T(1) : T(0));
            if (a != T(0)) {
                const long long ub = ob * t.su;
                auto Uu = [&](int p, int c) {
                    const long long k = (long long)p * ny + c;
                    return u[ub + k] * t.idxu2[k];
                };
                const T Um = T(0.25) * (Uu(i + 1, j) + Uu(i + 1, j - 1) + Uu(i, j) + Uu(i, j - 1));
                T q[6];
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    const int ii = i - 2 + k;
                    q[k] = (ii >= 0 && ii <= nx) ? om[ob * t.sw + (long long)ii * (ny + 1) + j] : T(0);
                }
                T g[6], gv;
                weno_flux_grad<T>(q, Um, (fl >> 4) & 7, i >= 1 && i <= nx - 2, i >= 2 && i <= nx - 3, g, gv);
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    const int ii = i - 2 + k;
                    if (ii >= 0 && ii <= nx && g[k] != T(0)) w_s[k] = -a * g[k];
                }
                um_s = -T(0.25) * a * (gv + t.fsv[vi]);
                a_s = a;
                if (t.ad_dyp && t.hxy_dyp)
                    aadd(&t.ad_dyp[(long long)l * nx * (ny - 1) + (long long)i * (ny - 1) + j - 1], -a);
                if (t.ad_wfv && l == 0) aadd(&t.ad_wfv[vi], a * (tauy ? tauy : t.tauy)[(long long)i * (ny - 1) + j - 1]);
                if (t.visc > T(0)) c_s = t.visc * t.dyv[vi] * a;
            }
            T aF = T(0);
            const long long hj0 = (long long)i * ny + j - 1, hj1 = (long long)i * ny + j;
            if (j - 1 >= 1 && j - 1 <= ny - 2) aF -= mh(hj0) * hb[hj0];
            if (j >= 1 && j <= ny - 2) aF += mh(hj1) * hb[hj1];
            if (aF != T(0)) {
                const T iv2 = t.idyv2[vi];
                const T Vf = v[so] * iv2;
                T q[6];
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    const int jj = j - 3 + k;
                    q[k] = (jj >= 0 && jj < ny) ? ht[ob * t.sh + (long long)i * ny + jj] : T(0);
                }
                T g[6], gv;
                weno_flux_grad<T>(q, Vf, (fl >> 1) & 7, j >= 2 && j <= ny - 2, j >= 3 && j <= ny - 3, g, gv);
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    const int jj = j - 3 + k;
                    if (jj >= 0 && jj < ny && g[k] != T(0)) h_s[k] = aF * g[k];
                }
                f_s = aF * gv * iv2;
            }
        }
        S.va[so] = a_s;
        S.vum[so] = um_s;
        S.vc[so] = c_s;
        S.vf[so] = f_s;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            S.vw[k * S.nv + so] = w_s[k];
            S.vh[k * S.nv + so] = h_s[k];
        }
    }
    // ---------------- thickness diffusion coefficient at h (i, j)
    if (i < nx && j < ny) {
        const long long hi = (long long)i * ny + j;
        S.hd[ob * t.sh + hi] = t.diff > T(0) ? hb[hi] * mh(hi) * t.diff * t.area[hi] : T(0);
    }
}

// Pass 2: every target of the tendency adjoint sums the stored terms of its
// sources. adom, adkp, adht are written (every index once); adu, adv, adh
// are added to.
template <typename T>
__global__ void k_sw_tend_adj_gather(Tab<T> t, SwSrc<T> S, T* adom, T* adkp, T* adht, T* adu, T* adv, T* adh)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int bl = blockIdx.z;
    const int nx = t.nx, ny = t.ny, nl = t.nl, l = bl % nl;
    if (i > nx || j > ny) return;
    const long long ob = bl;
    // stored terms of u face (p, c) / v face (p, c); 0 outside the grid
    auto U = [&](const T* A, int p, int c) {
        return (p >= 0 && p <= nx && c >= 0 && c < ny) ? A[ob * t.su + (long long)p * ny + c] : T(0);
    };
    auto V = [&](const T* A, int p, int c) {
        return (p >= 0 && p < nx && c >= 0 && c <= ny) ? A[ob * t.sv + (long long)p * (ny + 1) + c] : T(0);
    };
    // ---- vorticity point (i, j): u face (i, j+2-k) and v face (i+2-k, j) reach it with term k
    {
        T s = T(0);
#pragma unroll
        for (int k = 0; k < 6; ++k) s += U(S.uw + k * S.nu, i, j + 2 - k);
#pragma unroll
        for (int k = 0; k < 6; ++k) s += V(S.vw + k * S.nv, i + 2 - k, j);
        adom[ob * t.sw + (long long)i * (ny + 1) + j] = s;
    }
    // ---- h point (i, j)
    if (i < nx && j < ny) {
        const long long hi = (long long)i * ny + j;
        // KE + pressure: u faces i (-a) and i+1 (+a), v faces j (-a) and j+1 (+a)
        adkp[ob * t.sh + hi] = (-U(S.ua, i, j) + U(S.ua, i + 1, j)) + (-V(S.va, i, j) + V(S.va, i, j + 1));
        // thickness fluxes: u face (i+3-k, j) and v face (i, j+3-k) reach it with term k
        T sh_ = T(0);
#pragma unroll
        for (int k = 0; k < 6; ++k) sh_ += U(S.uh + k * S.nu, i + 3 - k, j);
#pragma unroll
        for (int k = 0; k < 6; ++k) sh_ += V(S.vh + k * S.nv, i, j + 3 - k);
        adht[ob * t.sh + hi] = sh_;
        if (t.diff > T(0)) {
            // the diffusion stencil of cell (p, c): (p+-1, c), (p, c+-1) clamped to the grid, and (p, c)
            const T* D = S.hd + ob * t.sh;
            const T ia = t.iarea[hi];
            T s = T(0);
            if (i >= 1) s += D[hi - ny] * t.idx2h[hi - ny] * ia;
            if (i + 1 <= nx - 1) s += D[hi + ny] * t.idx2h[hi + ny] * ia;
            if (j >= 1) s += D[hi - 1] * t.idy2h[hi - 1] * ia;
            if (j + 1 <= ny - 1) s += D[hi + 1] * t.idy2h[hi + 1] * ia;
            const T a0 = D[hi], ix2 = t.idx2h[hi], iy2 = t.idy2h[hi];
            s += a0 * (-T(2) * ix2 - T(2) * iy2) * ia;
            if (i == nx - 1) s += a0 * ix2 * ia;
            if (i == 0) s += a0 * ix2 * ia;
            if (j == ny - 1) s += a0 * iy2 * ia;
            if (j == 0) s += a0 * iy2 * ia;
            adh[ob * t.sh + hi] += s;
        }
    }
    // ---- u face (i, j)
    if (j < ny) {
        const long long ui = (long long)i * ny + j;
        const T iu2 = t.idxu2[ui];
        // U-average of the v faces (i-1, j), (i-1, j+1), (i, j), (i, j+1)
        T s = V(S.vum, i - 1, j) * iu2 + V(S.vum, i - 1, j + 1) * iu2 + V(S.vum, i, j) * iu2 +
              V(S.vum, i, j + 1) * iu2;
        const T a0 = U(S.ua, i, j);
        if (l == nl - 1) s += -t.drag * a0;
        if (t.visc > T(0)) {
            // viscosity stencil of u face (p, c): (p+-1, c), (p, c+-1) with c clamped, and (p, c)
            const T id = t.idxu[ui];
            if (i >= 1) s += U(S.uc, i - 1, j) * t.idxu2[ui - ny] * id;
            if (i + 1 <= nx) s += U(S.uc, i + 1, j) * t.idxu2[ui + ny] * id;
            if (j >= 1) s += U(S.uc, i, j - 1) * t.idyu2[ui - 1] * id;
            if (j + 1 <= ny - 1) s += U(S.uc, i, j + 1) * t.idyu2[ui + 1] * id;
            const T c0 = U(S.uc, i, j), ix2 = t.idxu2[ui], iy2 = t.idyu2[ui];
            s += c0 * (-T(2) * ix2 - T(2) * iy2) * id;
            if (j == ny - 1) s += c0 * iy2 * id;
            if (j == 0) s += c0 * iy2 * id;
        }
        s += U(S.uf, i, j);
        adu[ob * t.su + ui] += s;
    }
    // ---- v face (i, j)
    if (i < nx) {
        const long long vi = (long long)i * (ny + 1) + j;
        const T iv2 = t.idyv2[vi];
        // V-average of the u faces (i, j-1), (i, j), (i+1, j-1), (i+1, j)
        T s = U(S.uvm, i, j - 1) * iv2 + U(S.uvm, i, j) * iv2 + U(S.uvm, i + 1, j - 1) * iv2 +
              U(S.uvm, i + 1, j) * iv2;
        const T a0 = V(S.va, i, j);
        if (l == nl - 1) s += -t.drag * a0;
        if (t.visc > T(0)) {
            // viscosity stencil of v face (p, c): (p+-1, c) with p clamped, (p, c+-1), and (p, c)
            const T id = t.idyv[vi];
            if (i >= 1) s += V(S.vc, i - 1, j) * t.idxv2[vi - (ny + 1)] * id;
            if (i + 1 <= nx - 1) s += V(S.vc, i + 1, j) * t.idxv2[vi + (ny + 1)] * id;
            if (j >= 1) s += V(S.vc, i, j - 1) * t.idyv2[vi - 1] * id;
            if (j + 1 <= ny) s += V(S.vc, i, j + 1) * t.idyv2[vi + 1] * id;
            const T c0 = V(S.vc, i, j), ix2 = t.idxv2[vi], iy2 = t.idyv2[vi];
            s += c0 * (-T(2) * ix2 - T(2) * iy2) * id;
            if (i == nx - 1) s += c0 * ix2 * id;
            if (i == 0) s += c0 * ix2 * id;
        }
        s += V(S.vf, i, j);
        adv[ob * t.sv + vi] += s;
    }
}

// Adjoint of k_sw_diag (gather): adds into adu, adv, adh.
template <typename T>
__global__ void k_sw_diag_adj(Tab<T> t, const T* u, const T* v, const T* h, const T* adom, const T* adkp,
                              const T* adht, T* adu, T* adv, T* adh)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const int nx = t.nx, ny = t.ny, nl = t.nl;
    if (i > nx || j > ny) return;
    auto mh = [&](int p, int c) { return (t.fh[(long long)p * ny + c] & 1) ? T(1) : T(0); };
    for (int l = 0; l < nl; ++l) {
        const long long ob = (long long)(b * nl + l);
        const T* AO = adom + ob * t.sw;
        const T* AK = adkp + ob * t.sh;
        if (j < ny) {   // u point: dy(u) at w (i, j) (+) and (i, j+1) (-); KE of cells i-1, i
            const long long ui = (long long)i * ny + j, o = ob * t.su + ui;
            T a = -t.wb[(long long)i * (ny + 1) + j] * AO[(long long)i * (ny + 1) + j] +
                  t.wb[(long long)i * (ny + 1) + j + 1] * AO[(long long)i * (ny + 1) + j + 1];
            T kk = T(0);
            if (i >= 1) kk += mh(i - 1, j) * AK[(long long)(i - 1) * ny + j];
            if (i < nx) kk += mh(i, j) * AK[(long long)i * ny + j];
            a += T(0.5) * kk * u[o] * t.idxu2[ui];
            adu[o] += a;
        }
        if (i < nx) {   // v point: dx(v) at w (i, j) (+) and (i+1, j) (-); KE of cells j-1, j
            const long long vi = (long long)i * (ny + 1) + j, o = ob * t.sv + vi;
            T a = t.wa[(long long)i * (ny + 1) + j] * AO[(long long)i * (ny + 1) + j] -
                  t.wa[(long long)(i + 1) * (ny + 1) + j] * AO[(long long)(i + 1) * (ny + 1) + j];
            T kk = T(0);
            if (j >= 1) kk += mh(i, j - 1) * AK[(long long)i * ny + j - 1];
            if (j < ny) kk += mh(i, j) * AK[(long long)i * ny + j];
            a += T(0.5) * kk * v[o] * t.idyv2[vi];
            adv[o] += a;
        }
    }
    if (i < nx && j < ny) {
        const long long hi = (long long)i * ny + j;
        const T ar = t.area[hi];
        // pressure: p_l = sum_m h_m/area * G[min(l, m)]
        T ap[MAXL];
        for (int l = 0; l < nl; ++l) ap[l] = adkp[(long long)(b * nl + l) * t.sh + hi];
        for (int m = 0; m < nl; ++m) {
            const long long o = (long long)(b * nl + m) * t.sh + hi;
            T a = T(0);
            for (int l = 0; l < nl; ++l) a += ap[l] * t.G[l < m ? l : m];
            a = a * t.iarea[hi];
            T aref = adht[o];   // d h_tot / d h_ref (linear: h_tot = h_ref)
            if (!t.linear) {
                const T z = (t.href[(long long)m * t.sh + hi] + h[o] - t.hmin * ar) * t.sharp;
                aref = adht[o] * sigmoid_v(z);
                a += aref;
            }
            adh[o] += a;
            if (t.ad_href) aadd(&t.ad_href[(long long)m * t.sh + hi], aref);
        }
    }
}

// Adjoint of k_sw_force_mc (scatter to the thickness and Fh of the replicate
// padding stencil, atomics). adn: adjoint of the output (in place: becomes the
// adjoint of the input u, v, h direct paths).
// Adjoint of the mass-consistent forcing (sw.py:880-898), without atomics:
// the face terms (the cotangents the face's thickness and forcing averages
// hand to each of their two padded cells) are recomputed where they are
// gathered. mc_face_u / mc_face_v give them for one face from the face's
// incoming velocity cotangent.
template <typename T>
__device__ __forceinline__ void mc_face_u(const Tab<T>& t, const T* u, const T* h, const T* Fh, const T* adu,
                                          long long bl, int i, int j, T& gh, T& gf, T& fu, T& htu, T& sz)
{
    const int ny = t.ny, l = (int)(bl % t.nl);
    const long long ui = (long long)i * ny + j, idx = bl * t.su + ui, hb = bl * t.sh;
    R1<T> H{h}, FH{Fh};
    const T hu = T(0.5) * (rep_pad<T, T>(t, H, hb, i + 1, j + 1) + rep_pad<T, T>(t, H, hb, i, j + 1));
    fu = T(0.5) * (rep_pad<T, T>(t, FH, hb, i + 1, j + 1) + rep_pad<T, T>(t, FH, hb, i, j + 1));
    const T xmin = t.hmin * t.areau[ui];
    const T zz = (t.hrefu[(long long)l * t.su + ui] + hu - xmin) * t.sharp;
    htu = xmin + softplus_v(zz) / t.sharp;
    sz = sigmoid_v(zz);
    const T a = adu[idx], uu = u[idx];
    gh = T(0.5) * (a * t.dt * uu * fu / (htu * htu) * sz);
    gf = T(0.5) * (-a * t.dt * uu / htu);
}

template <typename T>
__device__ __forceinline__ void mc_face_v(const Tab<T>& t, const T* v, const T* h, const T* Fh, const T* adv,
                                          long long bl, int i, int j, T& gh, T& gf, T& fv, T& htv, T& sz)
{
    const int ny = t.ny, l = (int)(bl % t.nl);
    const long long vi = (long long)i * (ny + 1) + j, idx = bl * t.sv + vi, hb = bl * t.sh;
    R1<T> H{h}, FH{Fh};
    const T hv = T(0.5) * (rep_pad<T, T>(t, H, hb, i + 1, j + 1) + rep_pad<T, T>(t, H, hb, i + 1, j));
    fv = T(0.5) * (rep_pad<T, T>(t, FH, hb, i + 1, j + 1) + rep_pad<T, T>(t, FH, hb, i + 1, j));
    const T xmin = t.hmin * t.areav[vi];
    const T zz = (t.hrefv[(long long)l * t.sv + vi] + hv - xmin) * t.sharp;
    htv = xmin + softplus_v(zz) / t.sharp;
    sz = sigmoid_v(zz);
    const T a = adv[idx], vv = v[idx];
    gh = T(0.5) * (a * t.dt * vv * fv / (htv * htv) * sz);
    gf = T(0.5) * (-a * t.dt * vv / htv);
}

// Step 1, one thread per cell (i, j) and field: the cotangents of h and Fh.
// A padded cell (pi, pj) of replicate_pad (sw.py:36-48) takes its clamped
// cell when that is ocean, else the mean over the ocean count of its 3 x 3
// clamped neighbourhood; it is read by up to two u faces and two v faces.
// The cell gathers, over the padded cells within reach, its multiplicity in
// each padded cell's value times that padded cell's face terms, in a fixed
// order. Must run before step 2, which overwrites adu / adv.
template <typename T>
__global__ void k_sw_force_mc_adj_h(Tab<T> t, const T* u, const T* v, const T* h, const T* Fh, const T* adu,
                                    const T* adv, T* adh_acc, T* adFh)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const long long bl = blockIdx.z;
    const int nx = t.nx, ny = t.ny;
    if (i >= nx || j >= ny) return;
    auto cl = [](int q, int n) { return q < 0 ? 0 : (q > n - 1 ? n - 1 : q); };
    T sh = T(0), sf = T(0);
    for (int pi = (i > 0 ? i - 1 : 0); pi <= (i + 3 < nx + 1 ? i + 3 : nx + 1); ++pi)
        for (int pj = (j > 0 ? j - 1 : 0); pj <= (j + 3 < ny + 1 ? j + 3 : ny + 1); ++pj) {
            const int ci = cl(pi - 1, nx), cj = cl(pj - 1, ny);
            T wgt;
            if (t.fh[(long long)ci * ny + cj] & 1) {
                if (ci != i || cj != j) continue;
                wgt = T(1);
            } else {
                int cnt = 0, ms = 0;
                for (int a = pi - 1; a <= pi + 1; ++a)
                    for (int c = pj - 1; c <= pj + 1; ++c) {
                        if (a < 0 || a > nx + 1 || c < 0 || c > ny + 1) continue;
                        const int ai = cl(a - 1, nx), aj = cl(c - 1, ny);
                        ms += (t.fh[(long long)ai * ny + aj] & 1);
                        cnt += (ai == i && aj == j);
                    }
                if (!cnt) continue;
                wgt = T(cnt) / T(ms > 1 ? ms : 1);
            }
            T gh = T(0), gf = T(0), a, b, f, ht, sz;
            if (pj >= 1 && pj <= ny) {   // u faces (pi - 1, pj - 1) and (pi, pj - 1)
                if (pi >= 1) {
                    mc_face_u(t, u, h, Fh, adu, bl, pi - 1, pj - 1, a, b, f, ht, sz);
                    gh += a;
                    gf += b;
                }
                if (pi <= nx) {
                    mc_face_u(t, u, h, Fh, adu, bl, pi, pj - 1, a, b, f, ht, sz);
                    gh += a;
                    gf += b;
                }
            }
            if (pi >= 1 && pi <= nx) {   // v faces (pi - 1, pj - 1) and (pi - 1, pj)
                if (pj >= 1) {
                    mc_face_v(t, v, h, Fh, adv, bl, pi - 1, pj - 1, a, b, f, ht, sz);
                    gh += a;
                    gf += b;
                }
                if (pj <= ny) {
                    mc_face_v(t, v, h, Fh, adv, bl, pi - 1, pj, a, b, f, ht, sz);
                    gh += a;
                    gf += b;
                }
            }
            sh += wgt * gh;
            sf += wgt * gf;
        }
    const long long o = bl * t.sh + (long long)i * ny + j;
    adh_acc[o] += sh;
    if (adFh) adFh[o] += sf;
}

// Step 2, one thread per face point: u_new = u - dt u Fh_u / htot_u, so
// adu <- adu (1 - dt Fh_u / htot_u) in place; the face thickness cotangent
// also goes to the H table's cotangent when one is registered.
template <typename T>
__global__ void k_sw_force_mc_adj(Tab<T> t, const T* u, const T* v, const T* h, const T* Fh, T* adu, T* adv)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const long long bl = blockIdx.z;
    const int l = (int)(bl % t.nl);
    const int nx = t.nx, ny = t.ny;
    if (i > nx || j > ny) return;
    T gh, gf, f, ht, sz;
    if (j < ny) {
        const long long ui = (long long)i * ny + j, idx = bl * t.su + ui;
        mc_face_u(t, u, h, Fh, adu, bl, i, j, gh, gf, f, ht, sz);
        if (t.ad_hrefu) aadd(&t.ad_hrefu[(long long)l * t.su + ui], T(2) * gh);
        adu[idx] = adu[idx] * (T(1) - t.dt * f / ht);
    }
    if (i < nx) {
        const long long vi = (long long)i * (ny + 1) + j, idx = bl * t.sv + vi;
        mc_face_v(t, v, h, Fh, adv, bl, i, j, gh, gf, f, ht, sz);
        if (t.ad_hrefv) aadd(&t.ad_hrefv[(long long)l * t.sv + vi], T(2) * gh);
        adv[idx] = adv[idx] * (T(1) - t.dt * f / ht);
    }
}

// ------------------------------------------------------------------ barotropic filter
// Spectral barotropic filter (sw.py:720-750, filter_barotropic_waves, with
// the face thicknesses of compute_diagnostic_variables, 688-692): on faces
//   u* = (u + dt du) / dx_u,  ubar = sum_l u*_l htu_l / sum_l htu_l,
//   htu_l = smooth_clamp(h_ref_u,l + (h_l[i] + h_l[i-1]) / 2, h_min area_u, s)
// (replicate_pad of an all-ocean mask is an edge pad: the wall faces take
// their one cell twice), at cells
//   rhs = (diff_x ubar / dx + diff_y vbar / dy) / (g dt tau),
// w = the Neumann solve of rhs, and every layer's tendency gains
// -g tau diff_x w on the interior u faces and -g tau diff_y w on the interior
// v faces, masked. The forward and tangent kernels are templates over the
// arithmetic type like the right-hand side's; the adjoint is hand-written
// (the solve is symmetric, so its transpose is the same solve).
template <typename T, typename S, typename R>
__device__ __forceinline__ S bf_ubar(const Tab<T>& t, const Tri<R>& x, const R& tu, int b, int i, int j)
{
    const int nx = t.nx, ny = t.ny, nl = t.nl;
    const int c0 = i < nx ? i : nx - 1, c1 = i > 0 ? i - 1 : 0;
    const long long fi = (long long)i * ny + j;
    const T xmin = t.hmin * t.areau[fi], dxu = t.dxu[fi];
    S num = T(0) * x.u(fi), den = num;
    for (int l = 0; l < nl; ++l) {
        const long long ob = (long long)b * nl + l;
        const S hu = T(0.5) * (x.h(ob * t.sh + (long long)c0 * ny + j) + x.h(ob * t.sh + (long long)c1 * ny + j));
        const S ht = sclamp(VD_TAB(S, t.hrefu, t.d_hrefu, (long long)l * t.su + fi) + hu, xmin, t.sharp);
        const S us = (x.u(ob * t.su + fi) + t.dt * tu(ob * t.su + fi)) / dxu;
        num = num + us * ht;
        den = den + ht;
    }
    return num / den;
}

template <typename T, typename S, typename R>
__device__ __forceinline__ S bf_vbar(const Tab<T>& t, const Tri<R>& x, const R& tv, int b, int i, int j)
{
    const int ny = t.ny, nl = t.nl;
    const int c0 = j < ny ? j : ny - 1, c1 = j > 0 ? j - 1 : 0;
    const long long fi = (long long)i * (ny + 1) + j;
    const T xmin = t.hmin * t.areav[fi], dyv = t.dyv[fi];
    S num = T(0) * x.v(fi), den = num;
    for (int l = 0; l < nl; ++l) {
        const long long ob = (long long)b * nl + l;
        const long long hb = ob * t.sh + (long long)i * ny;
        const S hv = T(0.5) * (x.h(hb + c0) + x.h(hb + c1));
        const S ht = sclamp(VD_TAB(S, t.hrefv, t.d_hrefv, (long long)l * t.sv + fi) + hv, xmin, t.sharp);
        const S vs = (x.v(ob * t.sv + fi) + t.dt * tv(ob * t.sv + fi)) / dyv;
        num = num + vs * ht;
        den = den + ht;
    }
    return num / den;
}

// ubar on every u face and vbar on every v face of one batch member (one
// thread per point of the (nx+1) x (ny+1) index space), into [B][nx+1][ny]
// and [B][nx][ny+1]
template <typename T, typename S, typename R, typename W>
__global__ void k_bf_bar(Tab<T> t, Tri<R> x, R tu, R tv, W ub, W vb)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const int nx = t.nx, ny = t.ny;
    if (i > nx || j > ny) return;
    if (j < ny) ub((long long)b * (nx + 1) * ny + (long long)i * ny + j, bf_ubar<T, S>(t, x, tu, b, i, j));
    if (i < nx) vb((long long)b * nx * (ny + 1) + (long long)i * (ny + 1) + j, bf_vbar<T, S>(t, x, tv, b, i, j));
}

// right-hand side of the filter's solve from the face transports, one
// thread per cell and batch member
template <typename T, typename S, typename R, typename W>
__global__ void k_bf_rhs(Tab<T> t, R ub, R vb, W rhs)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const int nx = t.nx, ny = t.ny;
    if (i >= nx || j >= ny) return;
    const long long hi = (long long)i * ny + j;
    const long long u0 = (long long)b * (nx + 1) * ny + hi, v0 = (long long)b * nx * (ny + 1) + (long long)i * (ny + 1) + j;
    const S du = ub(u0 + ny) - ub(u0);
    const S dv = vb(v0 + 1) - vb(v0);
    rhs((long long)b * nx * ny + hi, t.bf_c * (du / t.dxh[hi] + dv / t.dyh[hi]));
}

// tendencies += the filter's velocity correction from the solved w
template <typename T, typename S, typename R, typename W>
__global__ void k_bf_apply(Tab<T> t, R w, R tu_r, R tv_r, W tu_w, W tv_w)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const int nx = t.nx, ny = t.ny, nl = t.nl;
    if (i > nx || j > ny) return;
    const long long wb = (long long)b * nx * ny;
    if (j < ny && i >= 1 && i <= nx - 1 && (t.fu[(long long)i * ny + j] & 1)) {
        const S f = (-t.bf_gt) * (w(wb + (long long)i * ny + j) - w(wb + (long long)(i - 1) * ny + j));
        for (int l = 0; l < nl; ++l) {
            const long long idx = ((long long)b * nl + l) * t.su + (long long)i * ny + j;
            tu_w(idx, tu_r(idx) + f);
        }
    }
    if (i < nx && j >= 1 && j <= ny - 1 && (t.fv[(long long)i * (ny + 1) + j] & 1)) {
        const S f = (-t.bf_gt) * (w(wb + (long long)i * ny + j) - w(wb + (long long)i * ny + j - 1));
        for (int l = 0; l < nl; ++l) {
            const long long idx = ((long long)b * nl + l) * t.sv + (long long)i * (ny + 1) + j;
            tv_w(idx, tv_r(idx) + f);
        }
    }
}

// Adjoint, step 1: cotangent of w from the tendency cotangents,
// ad_w[i][j] = -g tau (A_u[i] - A_u[i+1] + A_v[j] - A_v[j+1]) with A the layer
// sums of the cotangents on the interior masked faces (0 elsewhere).
template <typename T>
__global__ void k_bf_adw(Tab<T> t, const T* __restrict__ atu, const T* __restrict__ atv, T* __restrict__ adw)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const int nx = t.nx, ny = t.ny, nl = t.nl;
    if (i >= nx || j >= ny) return;
    auto Au = [&](int a) -> T {
        if (a < 1 || a > nx - 1 || !(t.fu[(long long)a * ny + j] & 1)) return T(0);
        T s = T(0);
        for (int l = 0; l < nl; ++l) s += atu[((long long)b * nl + l) * t.su + (long long)a * ny + j];
        return s;
    };
    auto Av = [&](int c) -> T {
        if (c < 1 || c > ny - 1 || !(t.fv[(long long)i * (ny + 1) + c] & 1)) return T(0);
        T s = T(0);
        for (int l = 0; l < nl; ++l) s += atv[((long long)b * nl + l) * t.sv + (long long)i * (ny + 1) + c];
        return s;
    };
    adw[(long long)b * nx * ny + (long long)i * ny + j] = -t.bf_gt * (Au(i) - Au(i + 1) + Av(j) - Av(j + 1));
}

// Adjoint, step 3 (after the solve of ad_w into ar), one thread per face
// point and batch member: the cotangents of ubar / vbar from ar, then per
// layer those of u / v (adu, adv +=), of the tendencies (atu2 = atu + dt ...,
// written for every face), and of the face thicknesses through the clamp
// (ghu / ghv, written for every face; also summed into the H table's
// cotangent when one is registered).
template <typename T>
__global__ void k_bf_face_adj(Tab<T> t, const T* __restrict__ u, const T* __restrict__ v, const T* __restrict__ h,
                              const T* __restrict__ tu, const T* __restrict__ tv, const T* __restrict__ ar,
                              const T* __restrict__ atu, const T* __restrict__ atv, T* adu, T* adv,
                              T* __restrict__ atu2, T* __restrict__ atv2, T* __restrict__ ghu, T* __restrict__ ghv)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const int nx = t.nx, ny = t.ny, nl = t.nl;
    if (i > nx || j > ny) return;
    const long long rb = (long long)b * nx * ny;
    T ht[MAXL], tr[MAXL], z[MAXL];
    if (j < ny) {   // u face (i, j)
        const long long fi = (long long)i * ny + j;
        T a = T(0);
        if (i >= 1) a += ar[rb + (long long)(i - 1) * ny + j] / t.dxh[(long long)(i - 1) * ny + j];
        if (i <= nx - 1) a -= ar[rb + fi] / t.dxh[fi];
        a *= t.bf_c;
        const int c0 = i < nx ? i : nx - 1, c1 = i > 0 ? i - 1 : 0;
        const T xmin = t.hmin * t.areau[fi], dxu = t.dxu[fi];
        T num = T(0), den = T(0);
        for (int l = 0; l < nl; ++l) {
            const long long ob = (long long)b * nl + l;
            const T hu = T(0.5) * (h[ob * t.sh + (long long)c0 * ny + j] + h[ob * t.sh + (long long)c1 * ny + j]);
            const T xx = t.hrefu[(long long)l * t.su + fi] + hu;
            z[l] = (xx - xmin) * t.sharp;
            ht[l] = sclamp(xx, xmin, t.sharp);
            tr[l] = (u[ob * t.su + fi] + t.dt * tu[ob * t.su + fi]) / dxu;
            num += tr[l] * ht[l];
            den += ht[l];
        }
        const T bar = num / den;
        for (int l = 0; l < nl; ++l) {
            const long long idx = ((long long)b * nl + l) * t.su + fi;
            const T g = a * ht[l] / den / dxu;
            adu[idx] += g;
            atu2[idx] = atu[idx] + t.dt * g;
            const T gh = a * (tr[l] - bar) / den * sigmoid_v(z[l]);
            ghu[idx] = gh;
            if (t.ad_hrefu) aadd(t.ad_hrefu + (long long)l * t.su + fi, gh);
        }
    }
    if (i < nx) {   // v face (i, j)
        const long long fi = (long long)i * (ny + 1) + j;
        const long long hrow = (long long)i * ny;
        T a = T(0);
        if (j >= 1) a += ar[rb + hrow + j - 1] / t.dyh[hrow + j - 1];
        if (j <= ny - 1) a -= ar[rb + hrow + j] / t.dyh[hrow + j];
        a *= t.bf_c;
        const int c0 = j < ny ? j : ny - 1, c1 = j > 0 ? j - 1 : 0;
        const T xmin = t.hmin * t.areav[fi], dyv = t.dyv[fi];
        T num = T(0), den = T(0);
        for (int l = 0; l < nl; ++l) {
            const long long ob = (long long)b * nl + l;
            const T hv = T(0.5) * (h[ob * t.sh + hrow + c0] + h[ob * t.sh + hrow + c1]);
            const T xx = t.hrefv[(long long)l * t.sv + fi] + hv;
            z[l] = (xx - xmin) * t.sharp;
            ht[l] = sclamp(xx, xmin, t.sharp);
            tr[l] = (v[ob * t.sv + fi] + t.dt * tv[ob * t.sv + fi]) / dyv;
            num += tr[l] * ht[l];
            den += ht[l];
        }
        const T bar = num / den;
        for (int l = 0; l < nl; ++l) {
            const long long idx = ((long long)b * nl + l) * t.sv + fi;
            const T g = a * ht[l] / den / dyv;
            adv[idx] += g;
            atv2[idx] = atv[idx] + t.dt * g;
            const T gh = a * (tr[l] - bar) / den * sigmoid_v(z[l]);
            ghv[idx] = gh;
            if (t.ad_hrefv) aadd(t.ad_hrefv + (long long)l * t.sv + fi, gh);
        }
    }
}

// Adjoint, step 4: the face-thickness cotangents gathered on the cells
// (face i averages cells i - 1 and i, the wall faces their one cell twice).
template <typename T>
__global__ void k_bf_h_adj(Tab<T> t, const T* __restrict__ ghu, const T* __restrict__ ghv, T* adh)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const long long bl = blockIdx.z;   // batch member * nl + layer
    const int nx = t.nx, ny = t.ny;
    if (i >= nx || j >= ny) return;
    const T* gu = ghu + bl * t.su;
    const T* gv = ghv + bl * t.sv;
    const long long u0 = (long long)i * ny + j, v0 = (long long)i * (ny + 1) + j;
    T g = T(0.5) * (gu[u0] + gu[u0 + ny]) + T(0.5) * (gv[v0] + gv[v0 + 1]);
    if (i == 0) g += T(0.5) * gu[u0];
    if (i == nx - 1) g += T(0.5) * gu[u0 + ny];
    if (j == 0) g += T(0.5) * gv[v0];
    if (j == ny - 1) g += T(0.5) * gv[v0 + 1];
    adh[bl * t.sh + u0] += g;
}

template <typename T>
__global__ void k_axpy(long long n, T a, const T* x, T* y)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) y[k] += a * x[k];
}
template <typename T>
__global__ void k_copy(long long n, const T* x, T* y)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) y[k] = x[k];
}

}  // namespace sw
}  // namespace vd

// ====================================================================== host
using namespace vd::sw;
using vd::Arena;

struct vd_sw_plan {
    vd_sw_desc d;
    int nx, ny, nl;
    size_t esz;
    void* dev;           // one allocation for every table
    size_t dev_bytes;
    Tab<float> tf;
    Tab<double> td;
    int has_taux, has_tauy;
    // host copies for the tangent tables of vd_sw_set_ref_tangent
    std::vector<double> h_area, h_dwu, h_dwv, h_gp;
    std::vector<uint8_t> h_fu, h_fv;
    int h_wind_mode = 0;
    vd_neumann_plan* bf = nullptr;   // the barotropic filter's solve (null: no filter)
};

namespace {

// window sums of a 0/1 field with zero padding (tools.py avg_pool2d)
struct Grid2 {
    int n0, n1;
    std::vector<int> a;
    int at(int i, int j) const { return (i < 0 || j < 0 || i >= n0 || j >= n1) ? 0 : a[(size_t)i * n1 + j]; }
};
static Grid2 pool(const Grid2& g, int k0, int k1, int p0, int p1)
{
    Grid2 r;
    r.n0 = g.n0 + 2 * p0 - k0 + 1;
    r.n1 = g.n1 + 2 * p1 - k1 + 1;
    r.a.assign((size_t)r.n0 * r.n1, 0);
    for (int i = 0; i < r.n0; ++i)
        for (int j = 0; j < r.n1; ++j) {
            int s = 0;
            for (int a = 0; a < k0; ++a)
                for (int b = 0; b < k1; ++b) s += g.at(i - p0 + a, j - p1 + b);
            r.a[(size_t)i * r.n1 + j] = s;
        }
    return r;
}

struct SWMasksHost {
    int nx, ny;
    std::vector<uint8_t> fh, fu, fv, fw;   // fw bits: 1 valid, 2 cornerout, 4 vertical, 8 horizontal, 16 w, 32 psi
};

// masks.py:57-158 with averages compared through integer window sums
static void build_masks(int nx, int ny, const double* mask, SWMasksHost& M)
{
    M.nx = nx;
    M.ny = ny;
    Grid2 h{nx, ny, std::vector<int>((size_t)nx * ny, 1)};
    if (mask)
        for (size_t k = 0; k < h.a.size(); ++k) h.a[k] = mask[k] > 0.5 ? 1 : 0;
    Grid2 u2 = pool(h, 2, 1, 1, 0), v2 = pool(h, 1, 2, 0, 1), w4 = pool(h, 2, 2, 1, 1);
    Grid2 U{nx + 1, ny, {}}, V{nx, ny + 1, {}}, W{nx + 1, ny + 1, {}};
    U.a.resize((size_t)(nx + 1) * ny);
    V.a.resize((size_t)nx * (ny + 1));
    W.a.resize((size_t)(nx + 1) * (ny + 1));
    for (size_t k = 0; k < U.a.size(); ++k) U.a[k] = u2.a[k] == 2;
    for (size_t k = 0; k < V.a.size(); ++k) V.a[k] = v2.a[k] == 2;
    for (size_t k = 0; k < W.a.size(); ++k) W.a[k] = w4.a[k] >= 1;
    Grid2 nv = pool(V, 2, 1, 1, 0), nu = pool(U, 1, 2, 0, 1);
    M.fw.assign(W.a.size(), 0);
    for (size_t k = 0; k < W.a.size(); ++k) {
        const bool w = W.a[k], a = nv.a[k] == 1, b = nu.a[k] == 1;
        const bool vb = w && a && !b, hb = w && b && !a, co = w && a && b;
        const bool valid = w && !vb && !hb && !co;
        M.fw[k] = (valid ? 1 : 0) | (co ? 2 : 0) | (vb ? 4 : 0) | (hb ? 8 : 0) | (w ? 16 : 0) | (w4.a[k] == 4 ? 32 : 0);
    }
    M.fh.assign(h.a.size(), 0);
    for (size_t k = 0; k < h.a.size(); ++k) M.fh[k] = h.a[k] ? 1 : 0;
    // u grid: h stencils along x, w stencils along y
    Grid2 hx4 = pool(h, 4, 1, 2, 0), hx6 = pool(h, 6, 1, 3, 0);
    Grid2 wy2 = pool(W, 1, 2, 0, 0), wy4 = pool(W, 1, 4, 0, 1), wy6 = pool(W, 1, 6, 0, 2);
    M.fu.assign(U.a.size(), 0);
    for (size_t k = 0; k < U.a.size(); ++k) {
        const bool u = U.a[k];
        const bool heq2 = (u2.a[k] == 2) && hx4.a[k] < 4 && u;
        const bool hgt4 = !heq2 && u;
        const bool heq4 = hx6.a[k] < 6 && hgt4;
        const bool hgt6 = !heq4 && hgt4;
        const bool weq2 = (wy2.a[k] == 2) && wy4.a[k] < 4 && u;
        const bool wgt4 = !weq2 && u;
        const bool weq4 = wy6.a[k] < 6 && wgt4;
        M.fu[k] = (u ? 1 : 0) | (heq2 ? 2 : 0) | (heq4 ? 4 : 0) | (hgt6 ? 8 : 0) | (weq2 ? 16 : 0) | (weq4 ? 32 : 0) |
                  (wgt4 ? 64 : 0);
    }
    // v grid: h stencils along y, w stencils along x
    Grid2 hy4 = pool(h, 1, 4, 0, 2), hy6 = pool(h, 1, 6, 0, 3);
    Grid2 wx2 = pool(W, 2, 1, 0, 0), wx4 = pool(W, 4, 1, 1, 0), wx6 = pool(W, 6, 1, 2, 0);
    M.fv.assign(V.a.size(), 0);
    for (size_t k = 0; k < V.a.size(); ++k) {
        const bool v = V.a[k];
        const bool heq2 = (v2.a[k] == 2) && hy4.a[k] < 4 && v;
        const bool hgt4 = !heq2 && v;
        const bool heq4 = hy6.a[k] < 6 && hgt4;
        const bool hgt6 = !heq4 && hgt4;
        const bool weq2 = (wx2.a[k] == 2) && wx4.a[k] < 4 && v;
        const bool wgt4 = !weq2 && v;
        const bool weq4 = wx6.a[k] < 6 && wgt4;
        const bool wgt6 = !weq4 && wgt4;
        M.fv[k] = (v ? 1 : 0) | (heq2 ? 2 : 0) | (heq4 ? 4 : 0) | (hgt6 ? 8 : 0) | (weq2 ? 16 : 0) | (weq4 ? 32 : 0) |
                  (wgt6 ? 64 : 0);
    }
}

static void edge_avg0(const std::vector<double>& a, int n0, int n1, std::vector<double>& out)
{   // n0 x n1 -> (n0+1) x n1, 0.5*(edge-padded neighbours) along axis 0
    out.resize((size_t)(n0 + 1) * n1);
    for (int i = 0; i <= n0; ++i)
        for (int j = 0; j < n1; ++j) {
            const int a0 = i - 1 < 0 ? 0 : i - 1, a1 = i > n0 - 1 ? n0 - 1 : i;
            out[(size_t)i * n1 + j] = 0.5 * (a[(size_t)a1 * n1 + j] + a[(size_t)a0 * n1 + j]);
        }
}
static void edge_avg1(const std::vector<double>& a, int n0, int n1, std::vector<double>& out)
{   // n0 x n1 -> n0 x (n1+1) along axis 1
    out.resize((size_t)n0 * (n1 + 1));
    for (int i = 0; i < n0; ++i)
        for (int j = 0; j <= n1; ++j) {
            const int a0 = j - 1 < 0 ? 0 : j - 1, a1 = j > n1 - 1 ? n1 - 1 : j;
            out[(size_t)i * (n1 + 1) + j] = 0.5 * (a[(size_t)i * n1 + a1] + a[(size_t)i * n1 + a0]);
        }
}

template <typename T>
static void fill_tab(Tab<T>& t, vd_sw_plan* p, const std::vector<size_t>& off)
{
    char* base = (char*)p->dev;
    int k = 0;
    auto P = [&](void) -> T* { return (T*)(base + off[k++]); };
    t.dxu = P(); t.dyu = P(); t.dxv = P(); t.dyv = P(); t.dxh = P(); t.dyh = P(); t.area = P();
    t.areau = P(); t.areav = P(); t.fsu = P(); t.fsv = P(); t.wa = P(); t.wb = P(); t.wfu = P(); t.wfv = P();
    t.href = P(); t.hrefu = P(); t.hrefv = P(); t.dxp = P(); t.dyp = P(); t.taux = P(); t.tauy = P();
    t.gu = P(); t.gv = P(); t.gh = P();
    t.idxu2 = P(); t.idxu = P(); t.idyu2 = P(); t.idyv2 = P(); t.idyv = P(); t.idxv2 = P();
    t.iarea = P(); t.idx2h = P(); t.idy2h = P();
    t.dwu = P(); t.dwv = P();
    t.ad_href = t.ad_hrefu = t.ad_hrefv = t.ad_dxp = t.ad_dyp = t.ad_wfu = t.ad_wfv = nullptr;
    t.d_href = t.d_hrefu = t.d_hrefv = t.d_dxp = t.d_dyp = t.d_wfu = t.d_wfv = nullptr;
    t.fh = (const uint8_t*)(base + off[k++]);
    t.fu = (const uint8_t*)(base + off[k++]);
    t.fv = (const uint8_t*)(base + off[k++]);
}

}  // namespace

extern "C" vd_status vd_sw_masks(int nx, int ny, const double* mask, uint8_t* fh, uint8_t* fu, uint8_t* fv,
                                 uint8_t* fw)
{
    if (nx < 2 || ny < 2) return VD_ERR_ARG;
    SWMasksHost M;
    build_masks(nx, ny, mask, M);
    if (fh) std::memcpy(fh, M.fh.data(), M.fh.size());
    if (fu) std::memcpy(fu, M.fu.data(), M.fu.size());
    if (fv) std::memcpy(fv, M.fv.data(), M.fv.size());
    if (fw) std::memcpy(fw, M.fw.data(), M.fw.size());
    return VD_OK;
}

extern "C" vd_status vd_sw_plan_create(vd_sw_plan** out, const vd_sw_desc* d)
{
    if (!out || !d) return VD_ERR_ARG;
    *out = nullptr;
    const int nx = d->nx, ny = d->ny, nl = d->nl;
    if (nx < 4 || ny < 4 || nl < 1 || nl > MAXL) return VD_ERR_ARG;
    if (d->dtype != VD_F32 && d->dtype != VD_F64) return VD_ERR_ARG;
    if (!d->dx_host || !d->dy_host || !d->f_host || !d->H_host || !d->g_prime_host) return VD_ERR_ARG;
    if (!(d->dt > 0) || d->slip_coef < 0 || d->slip_coef > 1) return VD_ERR_ARG;
    if (d->forcing_momentum != 0 && d->forcing_momentum != 1) return VD_ERR_ARG;
    if (d->h_wind_mode < 0 || d->h_wind_mode > 2 || (d->h_wind_mode == 2 && !d->h_wind_host)) return VD_ERR_ARG;
    if (d->barotropic_filter != 0 && d->barotropic_filter != 1) return VD_ERR_ARG;
    const size_t su = (size_t)(nx + 1) * ny, sv = (size_t)nx * (ny + 1), sh = (size_t)nx * ny,
                 sw = (size_t)(nx + 1) * (ny + 1);
    SWMasksHost M;
    build_masks(nx, ny, d->mask_host, M);
    if (d->flag_obc) {
        // open boundaries: only the face masks themselves change, after the
        // stencil selectors are built from the closed ones (sw.py:365-369)
        for (int j = 0; j < ny; ++j) {
            M.fu[(size_t)j] |= 1;
            M.fu[(size_t)nx * ny + j] |= 1;
        }
        for (int i = 0; i < nx; ++i) {
            M.fv[(size_t)i * (ny + 1)] |= 1;
            M.fv[(size_t)i * (ny + 1) + ny] |= 1;
        }
    }
    // metrics (sw.py:147-167)
    std::vector<double> dx(d->dx_host, d->dx_host + sh), dy(d->dy_host, d->dy_host + sh), dxu, dyu, dxv, dyv;
    for (size_t k = 0; k < sh; ++k)
        if (!(dx[k] > 0) || !(dy[k] > 0)) return VD_ERR_ARG;
    edge_avg0(dx, nx, ny, dxu);
    edge_avg0(dy, nx, ny, dyu);
    edge_avg1(dx, nx, ny, dxv);
    edge_avg1(dy, nx, ny, dyv);
    std::vector<double> area(sh), areau(su), areav(sv);
    for (size_t k = 0; k < sh; ++k) area[k] = dx[k] * dy[k];
    for (size_t k = 0; k < su; ++k) areau[k] = dxu[k] * dyu[k];
    for (size_t k = 0; k < sv; ++k) areav[k] = dxv[k] * dyv[k];
    // Coriolis on u / v grids times area (sw.py:193-201); f is [nx+1][ny+1]
    const double* f = d->f_host;
    std::vector<double> fsu(su), fsv(sv);
    for (int i = 0; i <= nx; ++i)
        for (int j = 0; j < ny; ++j)
            fsu[(size_t)i * ny + j] = 0.5 * (f[(size_t)i * (ny + 1) + j + 1] + f[(size_t)i * (ny + 1) + j]) *
                                      areau[(size_t)i * ny + j];
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j <= ny; ++j)
            fsv[(size_t)i * (ny + 1) + j] = 0.5 * (f[(size_t)(i + 1) * (ny + 1) + j] + f[(size_t)i * (ny + 1) + j]) *
                                           areav[(size_t)i * (ny + 1) + j];
    // vorticity coefficients (sw.py:687-696)
    const double slip = d->slip_coef, alpha = 2 * (1 - slip);
    std::vector<double> wa(sw), wb(sw);
    for (size_t k = 0; k < sw; ++k) {
        const int fw = M.fw[k];
        const double c = ((fw & 1) ? 1.0 : 0.0) + ((fw & 2) ? (1 - slip) : 0.0);
        wa[k] = c + ((fw & 4) ? alpha : 0.0);
        wb[k] = c + ((fw & 8) ? alpha : 0.0);
    }
    // reference values (sw.py:385-410)
    const int Hs = d->H_spatial ? 1 : 0;
    std::vector<double> Hf((size_t)nl * sh);
    for (int l = 0; l < nl; ++l)
        for (size_t k = 0; k < sh; ++k) Hf[(size_t)l * sh + k] = Hs ? d->H_host[(size_t)l * sh + k] : d->H_host[l];
    std::vector<double> href((size_t)nl * sh), hrefu((size_t)nl * su), hrefv((size_t)nl * sv);
    for (int l = 0; l < nl; ++l) {
        std::vector<double> hr(sh), a, b;
        for (size_t k = 0; k < sh; ++k) hr[k] = Hf[(size_t)l * sh + k] * area[k];
        std::copy(hr.begin(), hr.end(), href.begin() + (size_t)l * sh);
        edge_avg0(hr, nx, ny, a);
        edge_avg1(hr, nx, ny, b);
        std::copy(a.begin(), a.end(), hrefu.begin() + (size_t)l * su);
        std::copy(b.begin(), b.end(), hrefv.begin() + (size_t)l * sv);
    }
    // p_ref = cumsum_l(g'_l * eta_ref_l), eta_ref_l = -sum H + reverse_cumsum(H)_l
    std::vector<double> pref((size_t)nl * sh);
    for (size_t k = 0; k < sh; ++k) {
        double tot = 0;
        for (int l = 0; l < nl; ++l) tot += Hf[(size_t)l * sh + k];
        double cs = 0, p = 0;
        for (int l = 0; l < nl; ++l) {
            // reverse_cumsum(x)_l = x_l + sum(x) - cumsum(x)_l
            cs += Hf[(size_t)l * sh + k];
            const double rc = Hf[(size_t)l * sh + k] + tot - cs;
            p += d->g_prime_host[l] * (-tot + rc);
            pref[(size_t)l * sh + k] = p;
        }
    }
    std::vector<double> dxp, dyp;
    if (Hs) {
        dxp.assign((size_t)nl * (nx - 1) * ny, 0.0);
        dyp.assign((size_t)nl * nx * (ny - 1), 0.0);
        for (int l = 0; l < nl; ++l) {
            for (int i = 0; i < nx - 1; ++i)
                for (int j = 0; j < ny; ++j)
                    dxp[((size_t)l * (nx - 1) + i) * ny + j] =
                        pref[(size_t)l * sh + (size_t)(i + 1) * ny + j] - pref[(size_t)l * sh + (size_t)i * ny + j];
            for (int i = 0; i < nx; ++i)
                for (int j = 0; j < ny - 1; ++j)
                    dyp[((size_t)l * nx + i) * (ny - 1) + j] =
                        pref[(size_t)l * sh + (size_t)i * ny + j + 1] - pref[(size_t)l * sh + (size_t)i * ny + j];
        }
    }
    // wind factors (sw.py:570-669): dx_u / (rho H_ref_u) on interior u faces, masked;
    // without h_wind the depth is the layer-0 reference thickness of the
    // model's own H (Hwind_host when given)
    const double rho = d->rho_water > 0 ? d->rho_water : 1025.0, hmin = d->h_min;
    std::vector<double> hwu(hrefu.begin(), hrefu.begin() + su), hwv(hrefv.begin(), hrefv.begin() + sv);
    if (d->h_wind_mode == 0 && d->Hwind_host) {
        std::vector<double> hr(sh);
        for (size_t k = 0; k < sh; ++k) hr[k] = d->Hwind_host[k] * area[k];
        edge_avg0(hr, nx, ny, hwu);
        edge_avg1(hr, nx, ny, hwv);
    }
    std::vector<double> wfu(su, 0.0), wfv(sv, 0.0);
    for (int i = 1; i < nx; ++i)
        for (int j = 0; j < ny; ++j) {
            const size_t k = (size_t)i * ny + j;
            if (!(M.fu[k] & 1)) continue;
            double Hu;
            if (d->h_wind_mode == 1) Hu = d->h_wind_scalar;
            else if (d->h_wind_mode == 2) Hu = 0.5 * (d->h_wind_host[(size_t)(i - 1) * ny + j] + d->h_wind_host[(size_t)i * ny + j]);
            else Hu = hwu[k] / areau[k];
            Hu = Hu > hmin ? Hu : hmin;
            wfu[k] = dxu[k] / (rho * Hu);
        }
    for (int i = 0; i < nx; ++i)
        for (int j = 1; j < ny; ++j) {
            const size_t k = (size_t)i * (ny + 1) + j;
            if (!(M.fv[k] & 1)) continue;
            double Hv;
            if (d->h_wind_mode == 1) Hv = d->h_wind_scalar;
            else if (d->h_wind_mode == 2) Hv = 0.5 * (d->h_wind_host[(size_t)i * ny + j - 1] + d->h_wind_host[(size_t)i * ny + j]);
            else Hv = hwv[k] / areav[k];
            Hv = Hv > hmin ? Hv : hmin;
            wfv[k] = dyv[k] / (rho * Hv);
        }
    // d(wind factor)/d(face H_ref) with jnp.maximum's rule (1 above h_min,
    // 1/2 at a tie, 0 below), for the cotangents of H and h_wind
    std::vector<double> dwu(su, 0.0), dwv(sv, 0.0);
    auto dclamp = [&](double x) { return x > hmin ? 1.0 : (x == hmin ? 0.5 : 0.0); };
    for (int i = 1; i < nx; ++i)
        for (int j = 0; j < ny; ++j) {
            const size_t k = (size_t)i * ny + j;
            if (!(M.fu[k] & 1)) continue;
            double Hu;
            if (d->h_wind_mode == 1) Hu = d->h_wind_scalar;
            else if (d->h_wind_mode == 2) Hu = 0.5 * (d->h_wind_host[(size_t)(i - 1) * ny + j] + d->h_wind_host[(size_t)i * ny + j]);
            else Hu = hwu[k] / areau[k];
            const double Hc = Hu > hmin ? Hu : hmin;
            dwu[k] = -dxu[k] / (rho * Hc * Hc) * dclamp(Hu);
        }
    for (int i = 0; i < nx; ++i)
        for (int j = 1; j < ny; ++j) {
            const size_t k = (size_t)i * (ny + 1) + j;
            if (!(M.fv[k] & 1)) continue;
            double Hv;
            if (d->h_wind_mode == 1) Hv = d->h_wind_scalar;
            else if (d->h_wind_mode == 2) Hv = 0.5 * (d->h_wind_host[(size_t)i * ny + j - 1] + d->h_wind_host[(size_t)i * ny + j]);
            else Hv = hwv[k] / areav[k];
            const double Hc = Hv > hmin ? Hv : hmin;
            dwv[k] = -dyv[k] / (rho * Hc * Hc) * dclamp(Hv);
        }
    // default wind stress
    std::vector<double> taux((size_t)(nx - 1) * ny), tauy((size_t)nx * (ny - 1));
    for (size_t k = 0; k < taux.size(); ++k) taux[k] = d->taux_host ? d->taux_host[k] : d->taux_scalar;
    for (size_t k = 0; k < tauy.size(); ++k) tauy[k] = d->tauy_host ? d->tauy_host[k] : d->tauy_scalar;
    // sponge rates
    const double gs = d->sponge_coef / d->dt;
    std::vector<double> gu(su, 0.0), gv(sv, 0.0), gh(sh, 0.0);
    int has_sponge = 0;
    if (d->sponge_u_host) for (size_t k = 0; k < su; ++k) { gu[k] = gs * d->sponge_u_host[k]; has_sponge |= gu[k] != 0; }
    if (d->sponge_v_host) for (size_t k = 0; k < sv; ++k) { gv[k] = gs * d->sponge_v_host[k]; has_sponge |= gv[k] != 0; }
    if (d->sponge_h_host) for (size_t k = 0; k < sh; ++k) { gh[k] = gs * d->sponge_h_host[k]; has_sponge |= gh[k] != 0; }

    // reciprocal metric tables (products instead of divisions in the kernels)
    auto recip = [](const std::vector<double>& a, int pw) {
        std::vector<double> r(a.size());
        for (size_t k = 0; k < a.size(); ++k) r[k] = pw == 2 ? 1.0 / (a[k] * a[k]) : 1.0 / a[k];
        return r;
    };
    std::vector<double> idxu2 = recip(dxu, 2), idxu = recip(dxu, 1), idyu2 = recip(dyu, 2);
    std::vector<double> idyv2 = recip(dyv, 2), idyv = recip(dyv, 1), idxv2 = recip(dxv, 2);
    std::vector<double> iarea = recip(area, 1), idx2h = recip(dx, 2), idy2h = recip(dy, 2);

    // ---------------- upload: one allocation
    const size_t esz = d->dtype == VD_F64 ? 8 : 4;
    std::vector<const std::vector<double>*> arrs = {&dxu, &dyu, &dxv, &dyv, &dx, &dy, &area, &areau, &areav,
                                                   &fsu, &fsv, &wa, &wb, &wfu, &wfv, &href, &hrefu, &hrefv,
                                                   &dxp, &dyp, &taux, &tauy, &gu, &gv, &gh,
                                                   &idxu2, &idxu, &idyu2, &idyv2, &idyv, &idxv2,
                                                   &iarea, &idx2h, &idy2h, &dwu, &dwv};
    std::vector<size_t> off;
    size_t tot = 0;
    for (auto* a : arrs) {
        off.push_back(tot);
        tot += (a->size() * esz + 255) & ~size_t(255);
    }
    for (auto* a : {&M.fh, &M.fu, &M.fv}) {
        off.push_back(tot);
        tot += (a->size() + 255) & ~size_t(255);
    }
    std::vector<char> host(tot, 0);
    for (size_t a = 0; a < arrs.size(); ++a) {
        const auto& v = *arrs[a];
        for (size_t k = 0; k < v.size(); ++k) {
            if (esz == 8) ((double*)(host.data() + off[a]))[k] = v[k];
            else ((float*)(host.data() + off[a]))[k] = (float)v[k];
        }
    }
    std::memcpy(host.data() + off[arrs.size()], M.fh.data(), M.fh.size());
    std::memcpy(host.data() + off[arrs.size() + 1], M.fu.data(), M.fu.size());
    std::memcpy(host.data() + off[arrs.size() + 2], M.fv.data(), M.fv.size());
    // barotropic filter (sw.py:305-320): tau = 2 dt, g = g'_0,
    // lambd = 1 / (g dt tau H_tot) with H_tot the layer sum of the model's H
    std::vector<double> bf_lam;
    int bf_lam_spatial = 0;
    const double bf_g = d->g_prime_host[0], bf_tau = 2.0 * d->dt;
    if (d->barotropic_filter) {
        for (size_t k = 0; k < sh; ++k)
            if (!(M.fh[k] & 1)) return VD_ERR_UNSUPPORTED;
        if (!(bf_g != 0.0)) return VD_ERR_ARG;
        if (d->bf_lambd_host) {
            bf_lam_spatial = d->bf_lambd_spatial ? 1 : 0;
            bf_lam.assign(d->bf_lambd_host, d->bf_lambd_host + (bf_lam_spatial ? sh : 1));
        } else {
            bf_lam_spatial = Hs;
            bf_lam.assign(Hs ? sh : 1, 0.0);
            for (size_t k = 0; k < bf_lam.size(); ++k) {
                double Ht = 0;
                for (int l = 0; l < nl; ++l) Ht += Hf[(size_t)l * sh + k];
                bf_lam[k] = 1.0 / (bf_g * d->dt * bf_tau * Ht);
            }
        }
    }
    vd_sw_plan* p = new (std::nothrow) vd_sw_plan();
    if (!p) return VD_ERR_CUDA;
    p->d = *d;
    p->d.mask_host = nullptr; p->d.dx_host = p->d.dy_host = p->d.f_host = p->d.H_host = p->d.g_prime_host = nullptr;
    p->d.h_wind_host = p->d.taux_host = p->d.tauy_host = nullptr;
    p->d.sponge_u_host = p->d.sponge_v_host = p->d.sponge_h_host = nullptr;
    p->d.Hwind_host = nullptr;
    p->d.bf_lambd_host = nullptr;
    p->nx = nx; p->ny = ny; p->nl = nl; p->esz = esz;
    p->h_area = area;
    p->h_dwu = dwu;
    p->h_dwv = dwv;
    p->h_gp.assign(d->g_prime_host, d->g_prime_host + nl);
    p->h_fu.assign(M.fu.begin(), M.fu.end());
    p->h_fv.assign(M.fv.begin(), M.fv.end());
    p->h_wind_mode = d->h_wind_mode;
    if (cudaMalloc(&p->dev, tot) != cudaSuccess) {
        delete p;
        return VD_ERR_CUDA;
    }
    p->dev_bytes = tot;
    if (cudaMemcpy(p->dev, host.data(), tot, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(p->dev);
        delete p;
        return VD_ERR_CUDA;
    }
    if (d->barotropic_filter) {
        const vd_status rc = vd_neumann_plan_create(&p->bf, nx, ny, d->dtype, dx.data(), dy.data(), 1, bf_lam.data(),
                                                    bf_lam_spatial);
        if (rc != VD_OK) {
            cudaFree(p->dev);
            delete p;
            return rc;
        }
    }
    auto common = [&](auto& t) {
        using TT = std::remove_reference_t<decltype(t.drag)>;
        t.nx = nx; t.ny = ny; t.nl = nl;
        t.su = su; t.sv = sv; t.sh = sh; t.sw = sw;
        double G = 0;
        for (int l = 0; l < MAXL; ++l) {
            const double g = l < nl ? d->g_prime_host[l] : 0.0;
            G += g;
            t.gp[l] = (TT)g;
            t.G[l] = (TT)G;
        }
        t.drag = (TT)d->bottom_drag_coef; t.visc = (TT)(d->visc_coef > 0 ? d->visc_coef : 0);
        t.diff = (TT)(d->diff_coef > 0 ? d->diff_coef : 0); t.hmin = (TT)hmin;
        t.sharp = (TT)(d->h_min_sharpness > 0 ? d->h_min_sharpness : 10.0); t.dt = (TT)d->dt;
        t.linear = d->flag_linear ? 1 : 0; t.has_sponge = has_sponge; t.hxy_dxp = Hs; t.hxy_dyp = Hs;
        t.wind_mode = d->h_wind_mode;
        t.bf_c = (TT)(1.0 / (bf_g * d->dt * bf_tau));
        t.bf_gt = (TT)(bf_g * bf_tau);
        fill_tab(t, p, off);
        if (!Hs) { t.dxp = nullptr; t.dyp = nullptr; }
    };
    if (esz == 8) common(p->td);
    else common(p->tf);
    *out = p;
    return VD_OK;
}

// Cotangent accumulators of the H / h_wind dependent tables: one buffer of
// nl*(sh + su + sv) + nl*((nx-1)*ny + nx*(ny-1)) + su + sv elements.
static size_t ref_adj_elems(const vd_sw_plan* p)
{
    const size_t nx = p->nx, ny = p->ny, nl = p->nl;
    const size_t sh = nx * ny, su = (nx + 1) * ny, sv = nx * (ny + 1);
    return nl * (sh + su + sv) + nl * ((nx - 1) * ny + nx * (ny - 1)) + su + sv;
}

template <typename T>
static void set_ref_adj(vd_sw_plan* p, Tab<T>& t, void* buf)
{
    if (!buf) {
        t.ad_href = t.ad_hrefu = t.ad_hrefv = t.ad_dxp = t.ad_dyp = t.ad_wfu = t.ad_wfv = nullptr;
        return;
    }
    const long long nx = p->nx, ny = p->ny, nl = p->nl;
    T* b = (T*)buf;
    t.ad_href = b; b += nl * t.sh;
    t.ad_hrefu = b; b += nl * t.su;
    t.ad_hrefv = b; b += nl * t.sv;
    t.ad_dxp = b; b += nl * (nx - 1) * ny;
    t.ad_dyp = b; b += nl * nx * (ny - 1);
    t.ad_wfu = b; b += t.su;
    t.ad_wfv = b;
}

extern "C" size_t vd_sw_ref_adj_bytes(const vd_sw_plan* p) { return p ? ref_adj_elems(p) * p->esz : 0; }

extern "C" vd_status vd_sw_set_ref_adj(vd_sw_plan* p, void* buf)
{
    if (!p) return VD_ERR_ARG;
    if (p->esz == 8) set_ref_adj(p, p->td, buf);
    else set_ref_adj(p, p->tf, buf);
    return VD_OK;
}

extern "C" vd_status vd_sw_ref_pullback(const vd_sw_plan* p, const void* buf, void* adH, void* adhw, void* stream)
{
    if (!p || !buf || !adH) return VD_ERR_ARG;
    const dim3 block(32, 8), grid((unsigned)((p->ny + 31) / 32), (unsigned)((p->nx + 7) / 8));
    cudaStream_t st = (cudaStream_t)stream;
    auto go = [&](auto tab) {
        using T = std::remove_reference_t<decltype(*tab.area)>;
        using TT = std::remove_const_t<T>;
        Tab<TT> t = tab;
        set_ref_adj(const_cast<vd_sw_plan*>(p), t, const_cast<void*>(buf));
        k_sw_ref_pullback<TT><<<grid, block, 0, st>>>(t, t.ad_href, t.ad_hrefu, t.ad_hrefv, t.ad_dxp, t.ad_dyp,
                                                      t.ad_wfu, t.ad_wfv, (TT*)adH, (TT*)adhw);
    };
    if (p->esz == 8) go(p->td);
    else go(p->tf);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

// Tangent of the H / h_wind dependent tables (the same layout as the
// cotangent buffer): the reference thickness H area and its face averages,
// the reference pressure gradients (linear in H: eta_l = -sum_{m<l} H_m,
// p_l = sum_{k<=l} g'_k eta_k, then differences), and the wind factors, which
// a perturbed H leaves alone (the wind depth is the model's own, sw.py:
// 622-630) and a perturbed h_wind moves by d(wind factor)/d(face depth) times
// the face average of dh_wind.
template <typename T>
static int set_ref_tangent(vd_sw_plan* p, Tab<T>& t, const double* dH, const double* dhw, void* buf)
{
    if (!buf) {
        t.d_href = t.d_hrefu = t.d_hrefv = t.d_dxp = t.d_dyp = t.d_wfu = t.d_wfv = nullptr;
        return VD_OK;
    }
    const int nx = p->nx, ny = p->ny, nl = p->nl;
    const size_t sh = (size_t)nx * ny, su = (size_t)(nx + 1) * ny, sv = (size_t)nx * (ny + 1);
    std::vector<double> out;
    out.reserve(ref_adj_elems(p));
    std::vector<double> dref((size_t)nl * sh, 0.0);
    for (int l = 0; l < nl; ++l)
        for (size_t k = 0; k < sh; ++k) dref[(size_t)l * sh + k] = dH ? dH[(size_t)l * sh + k] * p->h_area[k] : 0.0;
    out.insert(out.end(), dref.begin(), dref.end());
    std::vector<double> au((size_t)nl * su), av((size_t)nl * sv);
    for (int l = 0; l < nl; ++l) {
        std::vector<double> hr(dref.begin() + (size_t)l * sh, dref.begin() + (size_t)(l + 1) * sh), a, b;
        edge_avg0(hr, nx, ny, a);
        edge_avg1(hr, nx, ny, b);
        std::copy(a.begin(), a.end(), au.begin() + (size_t)l * su);
        std::copy(b.begin(), b.end(), av.begin() + (size_t)l * sv);
    }
    out.insert(out.end(), au.begin(), au.end());
    out.insert(out.end(), av.begin(), av.end());
    std::vector<double> pref((size_t)nl * sh, 0.0);
    if (dH) {
        for (size_t k = 0; k < sh; ++k) {
            double tot = 0;
            for (int l = 0; l < nl; ++l) tot += dH[(size_t)l * sh + k];
            double cs = 0, pp = 0;
            for (int l = 0; l < nl; ++l) {
                cs += dH[(size_t)l * sh + k];
                const double rc = dH[(size_t)l * sh + k] + tot - cs;
                pp += p->h_gp[l] * (-tot + rc);
                pref[(size_t)l * sh + k] = pp;
            }
        }
    }
    for (int l = 0; l < nl; ++l)
        for (int i = 0; i < nx - 1; ++i)
            for (int j = 0; j < ny; ++j)
                out.push_back(pref[(size_t)l * sh + (size_t)(i + 1) * ny + j] - pref[(size_t)l * sh + (size_t)i * ny + j]);
    for (int l = 0; l < nl; ++l)
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny - 1; ++j)
                out.push_back(pref[(size_t)l * sh + (size_t)i * ny + j + 1] - pref[(size_t)l * sh + (size_t)i * ny + j]);
    std::vector<double> wu(su, 0.0), wv(sv, 0.0);
    if (dhw && p->h_wind_mode != 0) {
        for (int i = 1; i < nx; ++i)
            for (int j = 0; j < ny; ++j) {
                const size_t k = (size_t)i * ny + j;
                if (!(p->h_fu[k] & 1)) continue;
                const double dd = p->h_wind_mode == 1 ? dhw[0]
                                                      : 0.5 * (dhw[(size_t)(i - 1) * ny + j] + dhw[(size_t)i * ny + j]);
                wu[k] = p->h_dwu[k] * dd;
            }
        for (int i = 0; i < nx; ++i)
            for (int j = 1; j < ny; ++j) {
                const size_t k = (size_t)i * (ny + 1) + j;
                if (!(p->h_fv[k] & 1)) continue;
                const double dd = p->h_wind_mode == 1 ? dhw[0]
                                                      : 0.5 * (dhw[(size_t)i * ny + j - 1] + dhw[(size_t)i * ny + j]);
                wv[k] = p->h_dwv[k] * dd;
            }
    }
    out.insert(out.end(), wu.begin(), wu.end());
    out.insert(out.end(), wv.begin(), wv.end());
    if (out.size() != ref_adj_elems(p)) return VD_ERR_ARG;
    std::vector<T> cast(out.begin(), out.end());
    VD_CUDA_TRY(cudaMemcpy(buf, cast.data(), cast.size() * sizeof(T), cudaMemcpyHostToDevice));
    const long long nxl = nx, nyl = ny;
    const T* b = (const T*)buf;
    t.d_href = b; b += (long long)nl * t.sh;
    t.d_hrefu = b; b += (long long)nl * t.su;
    t.d_hrefv = b; b += (long long)nl * t.sv;
    t.d_dxp = b; b += (long long)nl * (nxl - 1) * nyl;
    t.d_dyp = b; b += (long long)nl * nxl * (nyl - 1);
    t.d_wfu = b; b += t.su;
    t.d_wfv = b;
    return VD_OK;
}

extern "C" vd_status vd_sw_set_ref_tangent(vd_sw_plan* p, const double* dH_host, const double* dhwind_host, void* buf)
{
    if (!p) return VD_ERR_ARG;
    return p->esz == 8 ? set_ref_tangent(p, p->td, dH_host, dhwind_host, buf)
                       : set_ref_tangent(p, p->tf, dH_host, dhwind_host, buf);
}

extern "C" void vd_sw_plan_destroy(vd_sw_plan* p)
{
    if (!p) return;
    vd_neumann_plan_destroy(p->bf);
    if (p->dev) cudaFree(p->dev);
    delete p;
}

// ---------------------------------------------------------------- drivers
namespace {

template <typename T> Tab<T>& tab(vd_sw_plan* p);
template <> Tab<float>& tab<float>(vd_sw_plan* p) { return p->tf; }
template <> Tab<double>& tab<double>(vd_sw_plan* p) { return p->td; }

struct Sizes {
    long long su, sv, sh, sw;   // per batch member (all layers)
};
static Sizes sizes(const vd_sw_plan* p)
{
    const long long nl = p->nl, nx = p->nx, ny = p->ny;
    return {nl * (nx + 1) * ny, nl * nx * (ny + 1), nl * nx * ny, nl * (nx + 1) * (ny + 1)};
}

template <typename T>
struct Fields {
    T *u, *v, *h;
};

template <typename T>
static bool take_uvh(Arena& ws, const Sizes& s, int B, Fields<T>& f)
{
    f.u = (T*)ws.take(sizeof(T) * s.su * B);
    f.v = (T*)ws.take(sizeof(T) * s.sv * B);
    f.h = (T*)ws.take(sizeof(T) * s.sh * B);
    return f.u && f.v && f.h;
}

// Per-source buffers of the two-pass tendency adjoint (16 values per u and v
// face, one per h point, every field of the batch).
template <typename T>
static bool take_src(Arena& ws, const Sizes& s, int B, SwSrc<T>& S)
{
    const long long nu = s.su * B, nv = s.sv * B, nh = s.sh * B;
    T* b = (T*)ws.take(sizeof(T) * (size_t)(16 * nu + 16 * nv + nh));
    if (!b) return false;
    S.nu = nu;
    S.nv = nv;
    S.ua = b; b += nu;
    S.uvm = b; b += nu;
    S.uc = b; b += nu;
    S.uf = b; b += nu;
    S.uw = b; b += 6 * nu;
    S.uh = b; b += 6 * nu;
    S.va = b; b += nv;
    S.vum = b; b += nv;
    S.vc = b; b += nv;
    S.vf = b; b += nv;
    S.vw = b; b += 6 * nv;
    S.vh = b; b += 6 * nv;
    S.hd = b;
    return true;
}

struct Launch {
    dim3 grid, block;
};
static Launch lgrid(const vd_sw_plan* p, int z)
{
    Launch L;
    L.block = dim3(32, 8, 1);
    L.grid = dim3((unsigned)((p->ny + 1 + 31) / 32), (unsigned)((p->nx + 1 + 7) / 8), (unsigned)z);
    return L;
}

// One RK3-SSP run of nstep steps in model space, forward (S = T) or
// tangent-linear (S = DN<T,1>). State x is advanced in place; traj (forward
// only) receives the state at the start of every step.
template <typename T>
struct Work {
    Fields<T> x1, x2, k0, k1, tuvh;   // tuvh.u/.v = tendencies, tuvh.h unused
    T *fx, *fy, *om, *kp, *ht;
    // barotropic filter (null without one): the solve's field [B][nx][ny],
    // the pre-filter tendency cotangents and the face-thickness cotangents
    T *bf = nullptr, *bau = nullptr, *bav = nullptr, *ghu = nullptr, *ghv = nullptr;
};

// elements of one batch member's filter field (0: the plan has no filter)
static long long bf_elems(const vd_sw_plan* p) { return p->bf ? (long long)p->nx * p->ny : 0; }

template <typename T>
static int take_work(Arena& ws, const Sizes& s, int B, Work<T>& w, long long bfn)
{
    if (!take_uvh(ws, s, B, w.x1) || !take_uvh(ws, s, B, w.x2) || !take_uvh(ws, s, B, w.k0) ||
        !take_uvh(ws, s, B, w.k1))
        return VD_ERR_WORKSPACE;
    w.tuvh.u = (T*)ws.take(sizeof(T) * s.su * B);
    w.tuvh.v = (T*)ws.take(sizeof(T) * s.sv * B);
    w.tuvh.h = nullptr;
    w.fx = (T*)ws.take(sizeof(T) * s.su * B);
    w.fy = (T*)ws.take(sizeof(T) * s.sv * B);
    w.om = (T*)ws.take(sizeof(T) * s.sw * B);
    w.kp = (T*)ws.take(sizeof(T) * s.sh * B);
    w.ht = (T*)ws.take(sizeof(T) * s.sh * B);
    if (!w.tuvh.u || !w.tuvh.v || !w.fx || !w.fy || !w.om || !w.kp || !w.ht) return VD_ERR_WORKSPACE;
    if (bfn > 0) {
        w.bf = (T*)ws.take(sizeof(T) * bfn * B);
        w.bau = (T*)ws.take(sizeof(T) * s.su * B);
        w.bav = (T*)ws.take(sizeof(T) * s.sv * B);
        w.ghu = (T*)ws.take(sizeof(T) * s.su * B);
        w.ghv = (T*)ws.take(sizeof(T) * s.sv * B);
        if (!w.bf || !w.bau || !w.bav || !w.ghu || !w.ghv) return VD_ERR_WORKSPACE;
    }
    return VD_OK;
}

template <typename T>
static size_t work_bytes(const Sizes& s, int B, long long bfn)
{
    const size_t F3 = sizeof(T) * (s.su + s.sv + s.sh) * B + 3 * 256;
    size_t n = 4 * F3 + sizeof(T) * (3 * s.su + 3 * s.sv + s.sw + 2 * s.sh) * B + 8 * 256;
    if (bfn > 0) n += sizeof(T) * (bfn + 2 * s.su + 2 * s.sv) * B + 5 * 256;
    return n;
}

template <typename T>
static R1<T> r(const T* p) { return R1<T>{p}; }
template <typename T>
static W1<T> w(T* p) { return W1<T>{p}; }
template <typename T>
static Tri<R1<T>> rt(const Fields<T>& f) { return {R1<T>{f.u}, R1<T>{f.v}, R1<T>{f.h}}; }
template <typename T>
static Tri<W1<T>> wt(const Fields<T>& f) { return {W1<T>{f.u}, W1<T>{f.v}, W1<T>{f.h}}; }
template <typename T>
static Tri<RD<T>> rtd(const Fields<T>& f, const Fields<T>& d) { return {RD<T>{f.u, d.u}, RD<T>{f.v, d.v}, RD<T>{f.h, d.h}}; }
template <typename T>
static Tri<WD<T>> wtd(const Fields<T>& f, const Fields<T>& d) { return {WD<T>{f.u, d.u}, WD<T>{f.v, d.v}, WD<T>{f.h, d.h}}; }

// One right-hand side's diagnostics and tendencies of state cur (wk.om,
// wk.kp, wk.ht; u / v tendencies in wk.tuvh, thickness fluxes in wk.fx /
// wk.fy), with the barotropic filter when the plan has one.
template <typename T>
static int tend_fwd(vd_sw_plan* p, int B, Fields<T> cur, Work<T>& wk, const T* taux, const T* tauy, cudaStream_t st)
{
    Tab<T>& t = tab<T>(p);
    const Launch Ld = lgrid(p, B), Ll = lgrid(p, B * p->nl);
    k_sw_diag<T, T><<<Ld.grid, Ld.block, 0, st>>>(t, rt(cur), w(wk.om), w(wk.kp), w(wk.ht));
    VD_LAUNCH_CHECK();
    k_sw_tend<T, T><<<Ll.grid, Ll.block, 0, st>>>(t, rt(cur), r<T>(wk.om), r<T>(wk.kp), r<T>(wk.ht), taux, tauy,
                                                   w(wk.tuvh.u), w(wk.tuvh.v), w(wk.fx), w(wk.fy));
    VD_LAUNCH_CHECK();
    if (p->bf) {
        // face transports into the adjoint's scratch (free in a forward pass)
        k_bf_bar<T, T><<<Ld.grid, Ld.block, 0, st>>>(t, rt(cur), r<T>(wk.tuvh.u), r<T>(wk.tuvh.v), w(wk.bau),
                                                      w(wk.bav));
        VD_LAUNCH_CHECK();
        k_bf_rhs<T, T><<<Ld.grid, Ld.block, 0, st>>>(t, r<T>(wk.bau), r<T>(wk.bav), w(wk.bf));
        VD_LAUNCH_CHECK();
        const int rc = vd::neumann_solve<T>(p->bf, B, wk.bf, wk.bf, st);
        if (rc) return rc;
        k_bf_apply<T, T><<<Ld.grid, Ld.block, 0, st>>>(t, r<T>(wk.bf), r<T>(wk.tuvh.u), r<T>(wk.tuvh.v),
                                                        w(wk.tuvh.u), w(wk.tuvh.v));
        VD_LAUNCH_CHECK();
    }
    return VD_OK;
}

// The same with tangents (dual numbers; tangents in dk).
template <typename T>
static int tend_tgl(vd_sw_plan* p, int B, Fields<T> cur, Fields<T> dcur, Work<T>& wk, Work<T>& dk, const T* taux,
                    const T* tauy, cudaStream_t st)
{
    Tab<T>& t = tab<T>(p);
    const Launch Ld = lgrid(p, B), Ll = lgrid(p, B * p->nl);
    using S = DN<T, 1>;
    k_sw_diag<T, S><<<Ld.grid, Ld.block, 0, st>>>(t, rtd(cur, dcur), WD<T>{wk.om, dk.om}, WD<T>{wk.kp, dk.kp},
                                                   WD<T>{wk.ht, dk.ht});
    VD_LAUNCH_CHECK();
    k_sw_tend<T, S><<<Ll.grid, Ll.block, 0, st>>>(
        t, rtd(cur, dcur), RD<T>{wk.om, dk.om}, RD<T>{wk.kp, dk.kp}, RD<T>{wk.ht, dk.ht}, taux, tauy,
        WD<T>{wk.tuvh.u, dk.tuvh.u}, WD<T>{wk.tuvh.v, dk.tuvh.v}, WD<T>{wk.fx, dk.fx}, WD<T>{wk.fy, dk.fy});
    VD_LAUNCH_CHECK();
    if (p->bf) {
        k_bf_bar<T, S><<<Ld.grid, Ld.block, 0, st>>>(t, rtd(cur, dcur), RD<T>{wk.tuvh.u, dk.tuvh.u},
                                                      RD<T>{wk.tuvh.v, dk.tuvh.v}, WD<T>{wk.bau, dk.bau},
                                                      WD<T>{wk.bav, dk.bav});
        VD_LAUNCH_CHECK();
        k_bf_rhs<T, S><<<Ld.grid, Ld.block, 0, st>>>(t, RD<T>{wk.bau, dk.bau}, RD<T>{wk.bav, dk.bav},
                                                      WD<T>{wk.bf, dk.bf});
        VD_LAUNCH_CHECK();
        int rc = vd::neumann_solve<T>(p->bf, B, wk.bf, wk.bf, st);
        if (rc || (rc = vd::neumann_solve<T>(p->bf, B, dk.bf, dk.bf, st))) return rc;
        k_bf_apply<T, S><<<Ld.grid, Ld.block, 0, st>>>(t, RD<T>{wk.bf, dk.bf}, RD<T>{wk.tuvh.u, dk.tuvh.u},
                                                        RD<T>{wk.tuvh.v, dk.tuvh.v}, WD<T>{wk.tuvh.u, dk.tuvh.u},
                                                        WD<T>{wk.tuvh.v, dk.tuvh.v});
        VD_LAUNCH_CHECK();
    }
    return VD_OK;
}

// forward step loop
template <typename T>
static int run_fwd(vd_sw_plan* p, int B, Fields<T> x, int nstep, Fields<T> xb, Fields<T> F, int hasF, const T* taux,
                   const T* tauy, Work<T>& wk, Fields<T>* traj, cudaStream_t st)
{
    Tab<T>& t = tab<T>(p);
    const Sizes s = sizes(p);
    const Launch Ld = lgrid(p, B), Ll = lgrid(p, B * p->nl);
    const int mc = p->d.forcing_momentum == 1;
    for (int n = 0; n < nstep; ++n) {
        if (traj) {
            k_copy<T><<<(unsigned)((s.su * B + 255) / 256), 256, 0, st>>>(s.su * B, x.u, traj[n].u);
            VD_LAUNCH_CHECK();
            k_copy<T><<<(unsigned)((s.sv * B + 255) / 256), 256, 0, st>>>(s.sv * B, x.v, traj[n].v);
            VD_LAUNCH_CHECK();
            k_copy<T><<<(unsigned)((s.sh * B + 255) / 256), 256, 0, st>>>(s.sh * B, x.h, traj[n].h);
            VD_LAUNCH_CHECK();
        }
        Fields<T> cur = x;
        for (int stg = 0; stg < 3; ++stg) {
            const int rc = tend_fwd<T>(p, B, cur, wk, taux, tauy, st);
            if (rc) return rc;
            Fields<T> nxt = stg == 0 ? wk.x1 : (stg == 1 ? wk.x2 : (mc ? wk.x1 : x));
            StageArgs sa{stg, (stg == 2 && hasF && !mc) ? 1 : 0};
            Fields<T> ks = stg == 0 ? wk.k0 : wk.k1;
            k_sw_update<T, T><<<Ll.grid, Ll.block, 0, st>>>(t, sa, rt(cur), r<T>(wk.tuvh.u), r<T>(wk.tuvh.v),
                                                             r<T>(wk.fx), r<T>(wk.fy), rt(wk.k0), rt(wk.k1), rt(xb),
                                                             rt(F), wt(ks), wt(nxt));
            VD_LAUNCH_CHECK();
            cur = nxt;
        }
        if (mc) {
            k_sw_force_mc<T, T><<<Ll.grid, Ll.block, 0, st>>>(t, rt(wk.x1), rt(F), wt(x));
            VD_LAUNCH_CHECK();
        }
    }
    return VD_OK;
}

// tangent-linear step loop (x, dx advanced in place)
template <typename T>
static int run_tgl(vd_sw_plan* p, int B, Fields<T> x, Fields<T> dx, int nstep, Fields<T> xb, Fields<T> dxb,
                   Fields<T> F, Fields<T> dF, int hasF, const T* taux, const T* tauy, Work<T>& wk, Work<T>& dk,
                   cudaStream_t st)
{
    Tab<T>& t = tab<T>(p);
    const Launch Ld = lgrid(p, B), Ll = lgrid(p, B * p->nl);
    const int mc = p->d.forcing_momentum == 1;
    using S = DN<T, 1>;
    for (int n = 0; n < nstep; ++n) {
        Fields<T> cur = x, dcur = dx;
        for (int stg = 0; stg < 3; ++stg) {
            const int rc = tend_tgl<T>(p, B, cur, dcur, wk, dk, taux, tauy, st);
            if (rc) return rc;
            Fields<T> nxt = stg == 0 ? wk.x1 : (stg == 1 ? wk.x2 : (mc ? wk.x1 : x));
            Fields<T> dnxt = stg == 0 ? dk.x1 : (stg == 1 ? dk.x2 : (mc ? dk.x1 : dx));
            StageArgs sa{stg, (stg == 2 && hasF && !mc) ? 1 : 0};
            Fields<T> ks = stg == 0 ? wk.k0 : wk.k1, dks = stg == 0 ? dk.k0 : dk.k1;
            k_sw_update<T, S><<<Ll.grid, Ll.block, 0, st>>>(
                t, sa, rtd(cur, dcur), RD<T>{wk.tuvh.u, dk.tuvh.u}, RD<T>{wk.tuvh.v, dk.tuvh.v}, RD<T>{wk.fx, dk.fx},
                RD<T>{wk.fy, dk.fy}, rtd(wk.k0, dk.k0), rtd(wk.k1, dk.k1), rtd(xb, dxb), rtd(F, dF), wtd(ks, dks),
                wtd(nxt, dnxt));
            VD_LAUNCH_CHECK();
            cur = nxt;
            dcur = dnxt;
        }
        if (mc) {
            k_sw_force_mc<T, S><<<Ll.grid, Ll.block, 0, st>>>(t, rtd(wk.x1, dk.x1), rtd(F, dF), wtd(x, dx));
            VD_LAUNCH_CHECK();
        }
    }
    return VD_OK;
}

template <typename T>
static int scale(vd_sw_plan* p, int B, int mode, const T* u, const T* v, const T* h, T* uo, T* vo, T* ho,
                 cudaStream_t st)
{
    const Launch L = lgrid(p, B * p->nl);
    k_sw_scale<T><<<L.grid, L.block, 0, st>>>(tab<T>(p), B * p->nl, mode, u, v, h, uo, vo, ho);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename T>
static int zero(Fields<T> f, const Sizes& s, int B, cudaStream_t st)
{
    VD_CUDA_TRY(cudaMemsetAsync(f.u, 0, sizeof(T) * s.su * B, st));
    VD_CUDA_TRY(cudaMemsetAsync(f.v, 0, sizeof(T) * s.sv * B, st));
    VD_CUDA_TRY(cudaMemsetAsync(f.h, 0, sizeof(T) * s.sh * B, st));
    return VD_OK;
}

template <typename T>
static int addto(Fields<T> y, T a, Fields<T> x, const Sizes& s, int B, cudaStream_t st)
{
    const long long n[3] = {s.su * B, s.sv * B, s.sh * B};
    T* ys[3] = {y.u, y.v, y.h};
    const T* xs[3] = {x.u, x.v, x.h};
    for (int k = 0; k < 3; ++k) {
        k_axpy<T><<<(unsigned)((n[k] + 255) / 256), 256, 0, st>>>(n[k], a, xs[k], ys[k]);
        VD_LAUNCH_CHECK();
    }
    return VD_OK;
}

// Inputs shared by the drivers: physical fields (device pointers, nullable
// where optional) converted to model space in the workspace.
template <typename T>
struct Inputs {
    Fields<T> x, xb, F;
    int hasb, hasF;
};

template <typename T>
static int prep_inputs(vd_sw_plan* p, int B, const void* u0, const void* v0, const void* h0, const void* ub,
                       const void* vb, const void* hb, const void* Fu, const void* Fv, const void* Fh, Arena& ws,
                       Inputs<T>& in, cudaStream_t st)
{
    const Sizes s = sizes(p);
    if (!take_uvh(ws, s, B, in.x) || !take_uvh(ws, s, B, in.xb) || !take_uvh(ws, s, B, in.F)) return VD_ERR_WORKSPACE;
    int rc = scale<T>(p, B, 0, (const T*)u0, (const T*)v0, (const T*)h0, in.x.u, in.x.v, in.x.h, st);
    if (rc) return rc;
    in.hasb = (ub || vb || hb) ? 1 : 0;
    rc = scale<T>(p, B, 0, (const T*)(ub ? ub : u0), (const T*)(vb ? vb : v0), (const T*)(hb ? hb : h0), in.xb.u,
                  in.xb.v, in.xb.h, st);
    if (rc) return rc;
    in.hasF = (Fu || Fv || Fh) ? 1 : 0;
    if ((rc = zero(in.F, s, B, st))) return rc;
    if (in.hasF) rc = scale<T>(p, B, 0, (const T*)Fu, (const T*)Fv, (const T*)Fh, in.F.u, in.F.v, in.F.h, st);
    return rc;
}

}  // namespace

extern "C" size_t vd_sw_workspace_bytes(const vd_sw_plan* p, int batch, int nstep)
{
    if (!p || batch <= 0 || nstep < 0) return 0;
    const Sizes s = sizes(p);
    const size_t esz = p->esz;
    const size_t F3 = esz * (s.su + s.sv + s.sh) * batch + 3 * 256;
    const long long bfn = bf_elems(p);
    const size_t wk = (esz == 8 ? work_bytes<double>(s, batch, bfn) : work_bytes<float>(s, batch, bfn));
    // inputs (x, xb, F), their tangents / adjoints, two work sets, adjoint
    // accumulators, the per-source buffers of the tendency adjoint, and the
    // per-step trajectory
    return 14 * F3 + 2 * wk + (size_t)nstep * F3 + esz * (s.sw + 2 * s.sh) * batch +
           esz * (16 * s.su + 16 * s.sv + s.sh) * batch + 64 * 256;
}

namespace {

template <typename T>
static int sw_step_t(vd_sw_plan* p, int B, const void* u0, const void* v0, const void* h0, int nstep, const void* ub,
                     const void* vb, const void* hb, const void* Fu, const void* Fv, const void* Fh, const void* taux,
                     const void* tauy, void* u1, void* v1, void* h1, Arena& ws, cudaStream_t st)
{
    Inputs<T> in;
    int rc = prep_inputs<T>(p, B, u0, v0, h0, ub, vb, hb, Fu, Fv, Fh, ws, in, st);
    if (rc) return rc;
    Work<T> wk;
    if ((rc = take_work<T>(ws, sizes(p), B, wk, bf_elems(p)))) return rc;
    rc = run_fwd<T>(p, B, in.x, nstep, in.xb, in.F, in.hasF, (const T*)taux, (const T*)tauy, wk, nullptr, st);
    if (rc) return rc;
    return scale<T>(p, B, 1, in.x.u, in.x.v, in.x.h, (T*)u1, (T*)v1, (T*)h1, st);
}

template <typename T>
static int sw_tgl_t(vd_sw_plan* p, int B, const void* u0, const void* v0, const void* h0, const void* du0,
                    const void* dv0, const void* dh0, int nstep, const void* ub, const void* vb, const void* hb,
                    const void* dub, const void* dvb, const void* dhb, const void* Fu, const void* Fv, const void* Fh,
                    const void* dFu, const void* dFv, const void* dFh, const void* taux, const void* tauy, void* du1,
                    void* dv1, void* dh1, Arena& ws, cudaStream_t st)
{
    Inputs<T> in, din;
    int rc = prep_inputs<T>(p, B, u0, v0, h0, ub, vb, hb, Fu, Fv, Fh, ws, in, st);
    if (rc) return rc;
    // tangents: boundary fields default to the initial state's tangent when
    // the boundary fields themselves default to the initial state
    const void* tub = ub ? dub : du0;
    const void* tvb = vb ? dvb : dv0;
    const void* thb = hb ? dhb : dh0;
    const Sizes s = sizes(p);
    if (!take_uvh(ws, s, B, din.x) || !take_uvh(ws, s, B, din.xb) || !take_uvh(ws, s, B, din.F))
        return VD_ERR_WORKSPACE;
    if ((rc = scale<T>(p, B, 0, (const T*)du0, (const T*)dv0, (const T*)dh0, din.x.u, din.x.v, din.x.h, st))) return rc;
    if ((rc = zero(din.xb, s, B, st))) return rc;
    if ((rc = scale<T>(p, B, 0, (const T*)tub, (const T*)tvb, (const T*)thb, din.xb.u, din.xb.v, din.xb.h, st))) return rc;
    if ((rc = zero(din.F, s, B, st))) return rc;
    if ((rc = scale<T>(p, B, 0, (const T*)dFu, (const T*)dFv, (const T*)dFh, din.F.u, din.F.v, din.F.h, st))) return rc;
    Work<T> wk, dk;
    if ((rc = take_work<T>(ws, s, B, wk, bf_elems(p))) || (rc = take_work<T>(ws, s, B, dk, bf_elems(p)))) return rc;
    rc = run_tgl<T>(p, B, in.x, din.x, nstep, in.xb, din.xb, in.F, din.F, in.hasF || dFu || dFv || dFh,
                    (const T*)taux, (const T*)tauy, wk, dk, st);
    if (rc) return rc;
    return scale<T>(p, B, 1, din.x.u, din.x.v, din.x.h, (T*)du1, (T*)dv1, (T*)dh1, st);
}

// adjoint of one right-hand side at state x (model space): adk -> adx (+=)
template <typename T>
static int rhs_adj(vd_sw_plan* p, int B, Fields<T> x, Fields<T> adk, Fields<T> adx, Work<T>& wk, T* adom, T* adkp,
                   T* adht, const SwSrc<T>& src, const T* taux, const T* tauy, cudaStream_t st)
{
    Tab<T>& t = tab<T>(p);
    const Launch Ld = lgrid(p, B), Ll = lgrid(p, B * p->nl);
    k_sw_diag<T, T><<<Ld.grid, Ld.block, 0, st>>>(t, rt(x), w(wk.om), w(wk.kp), w(wk.ht));
    VD_LAUNCH_CHECK();
    Fields<T> ak = adk;
    if (p->bf) {
        // the filter's transpose first: it needs the pre-filter tendencies of
        // x, and leaves the cotangents of those tendencies in wk.bau / wk.bav
        k_sw_tend<T, T><<<Ll.grid, Ll.block, 0, st>>>(t, rt(x), r<T>(wk.om), r<T>(wk.kp), r<T>(wk.ht), taux, tauy,
                                                       w(wk.tuvh.u), w(wk.tuvh.v), w(wk.fx), w(wk.fy));
        VD_LAUNCH_CHECK();
        k_bf_adw<T><<<Ld.grid, Ld.block, 0, st>>>(t, adk.u, adk.v, wk.bf);
        VD_LAUNCH_CHECK();
        const int rc = vd::neumann_solve<T>(p->bf, B, wk.bf, wk.bf, st);
        if (rc) return rc;
        k_bf_face_adj<T><<<Ld.grid, Ld.block, 0, st>>>(t, x.u, x.v, x.h, wk.tuvh.u, wk.tuvh.v, wk.bf, adk.u, adk.v,
                                                        adx.u, adx.v, wk.bau, wk.bav, wk.ghu, wk.ghv);
        VD_LAUNCH_CHECK();
        k_bf_h_adj<T><<<Ll.grid, Ll.block, 0, st>>>(t, wk.ghu, wk.ghv, adx.h);
        VD_LAUNCH_CHECK();
        ak.u = wk.bau;
        ak.v = wk.bav;
    }
    k_sw_tend_adj_src<T><<<Ll.grid, Ll.block, 0, st>>>(t, x.u, x.v, x.h, wk.om, wk.ht, ak.u, ak.v, ak.h, src,
                                                        taux, tauy);
    VD_LAUNCH_CHECK();
    k_sw_tend_adj_gather<T><<<Ll.grid, Ll.block, 0, st>>>(t, src, adom, adkp, adht, adx.u, adx.v, adx.h);
    VD_LAUNCH_CHECK();
    k_sw_diag_adj<T><<<Ld.grid, Ld.block, 0, st>>>(t, x.u, x.v, x.h, adom, adkp, adht, adx.u, adx.v, adx.h);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename T>
static int sw_adj_t(vd_sw_plan* p, int B, const void* u0, const void* v0, const void* h0, const void* adu1,
                    const void* adv1, const void* adh1, int nstep, const void* ub, const void* vb, const void* hb,
                    const void* Fu, const void* Fv, const void* Fh, const void* taux, const void* tauy, void* adu0,
                    void* adv0, void* adh0, void* adub, void* advb, void* adhb, void* adFu, void* adFv, void* adFh,
                    Arena& ws, cudaStream_t st)
{
    Inputs<T> in;
    int rc = prep_inputs<T>(p, B, u0, v0, h0, ub, vb, hb, Fu, Fv, Fh, ws, in, st);
    if (rc) return rc;
    const Sizes s = sizes(p);
    Work<T> wk;
    if ((rc = take_work<T>(ws, s, B, wk, bf_elems(p)))) return rc;
    std::vector<Fields<T>> traj((size_t)(nstep > 0 ? nstep : 1));
    for (int n = 0; n < nstep; ++n)
        if (!take_uvh(ws, s, B, traj[n])) return VD_ERR_WORKSPACE;
    Fields<T> ad, adk, a0, a1, adb, adF, x1, x2;
    if (!take_uvh(ws, s, B, ad) || !take_uvh(ws, s, B, adk) || !take_uvh(ws, s, B, a0) || !take_uvh(ws, s, B, a1) ||
        !take_uvh(ws, s, B, adb) || !take_uvh(ws, s, B, adF) || !take_uvh(ws, s, B, x1) || !take_uvh(ws, s, B, x2))
        return VD_ERR_WORKSPACE;
    T* adom = (T*)ws.take(sizeof(T) * s.sw * B);
    T* adkp = (T*)ws.take(sizeof(T) * s.sh * B);
    T* adht = (T*)ws.take(sizeof(T) * s.sh * B);
    SwSrc<T> src;
    if (!adom || !adkp || !adht || !take_src(ws, s, B, src)) return VD_ERR_WORKSPACE;
    // forward sweep storing the state at the start of every step
    Fields<T> xr;
    if (!take_uvh(ws, s, B, xr)) return VD_ERR_WORKSPACE;
    VD_CUDA_TRY(cudaMemcpyAsync(xr.u, in.x.u, sizeof(T) * s.su * B, cudaMemcpyDeviceToDevice, st));
    VD_CUDA_TRY(cudaMemcpyAsync(xr.v, in.x.v, sizeof(T) * s.sv * B, cudaMemcpyDeviceToDevice, st));
    VD_CUDA_TRY(cudaMemcpyAsync(xr.h, in.x.h, sizeof(T) * s.sh * B, cudaMemcpyDeviceToDevice, st));
    rc = run_fwd<T>(p, B, xr, nstep, in.xb, in.F, in.hasF, (const T*)taux, (const T*)tauy, wk, traj.data(), st);
    if (rc) return rc;
    // adjoint of the physical output -> model space
    if ((rc = scale<T>(p, B, 1, (const T*)adu1, (const T*)adv1, (const T*)adh1, ad.u, ad.v, ad.h, st))) return rc;
    if ((rc = zero(adb, s, B, st)) || (rc = zero(adF, s, B, st))) return rc;
    Tab<T>& t = tab<T>(p);
    const Launch Ll = lgrid(p, B * p->nl);
    const int mc = p->d.forcing_momentum == 1;
    for (int n = nstep - 1; n >= 0; --n) {
        // recompute the stage states of step n
        Fields<T> stages[3] = {traj[n], x1, x2};
        {
            Fields<T> cur = traj[n];
            const Launch Ld = lgrid(p, B);
            for (int stg = 0; stg < 2; ++stg) {
                if ((rc = tend_fwd<T>(p, B, cur, wk, (const T*)taux, (const T*)tauy, st))) return rc;
                Fields<T> nxt = stg == 0 ? x1 : x2;
                StageArgs sa{stg, 0};
                Fields<T> ks = stg == 0 ? wk.k0 : wk.k1;
                k_sw_update<T, T><<<Ll.grid, Ll.block, 0, st>>>(t, sa, rt(cur), r<T>(wk.tuvh.u), r<T>(wk.tuvh.v),
                                                                 r<T>(wk.fx), r<T>(wk.fy), rt(wk.k0), rt(wk.k1),
                                                                 rt(in.xb), rt(in.F), wt(ks), wt(nxt));
                VD_LAUNCH_CHECK();
                cur = nxt;
            }
            if (mc) {
                // x3 (before the forcing) is needed by the forcing adjoint: rebuild it in wk.x1
                if ((rc = tend_fwd<T>(p, B, x2, wk, (const T*)taux, (const T*)tauy, st))) return rc;
                StageArgs sa{2, 0};
                k_sw_update<T, T><<<Ll.grid, Ll.block, 0, st>>>(t, sa, rt(x2), r<T>(wk.tuvh.u), r<T>(wk.tuvh.v),
                                                                 r<T>(wk.fx), r<T>(wk.fy), rt(wk.k0), rt(wk.k1),
                                                                 rt(in.xb), rt(in.F), wt(wk.k1), wt(wk.x1));
                VD_LAUNCH_CHECK();
            }
        }
        // forcing adjoints
        if (in.hasF || adFu || adFv || adFh) {
            if ((rc = addto(adF, t.dt, ad, s, B, st))) return rc;
        }
        if (mc) {
            // u_new = u3 - dt u3 Fh_u / htot_u(h3): ad -> ad(u3), ad(h3) (+= into ad.h), ad(Fh)
            k_sw_force_mc_adj_h<T><<<Ll.grid, Ll.block, 0, st>>>(t, wk.x1.u, wk.x1.v, wk.x1.h, in.F.h, ad.u, ad.v,
                                                                 ad.h, adF.h);
            VD_LAUNCH_CHECK();
            k_sw_force_mc_adj<T><<<Ll.grid, Ll.block, 0, st>>>(t, wk.x1.u, wk.x1.v, wk.x1.h, in.F.h, ad.u, ad.v);
            VD_LAUNCH_CHECK();
        }
        if ((rc = zero(a0, s, B, st)) || (rc = zero(a1, s, B, st))) return rc;
        for (int stg = 2; stg >= 0; --stg) {
            k_sw_update_adj<T><<<Ll.grid, Ll.block, 0, st>>>(t, stg, B * p->nl, ad.u, ad.v, ad.h, adk.u, adk.v, adk.h,
                                                             a0.u, a0.v, a0.h, a1.u, a1.v, a1.h, adb.u, adb.v, adb.h);
            VD_LAUNCH_CHECK();
            if ((rc = rhs_adj<T>(p, B, stages[stg], adk, ad, wk, adom, adkp, adht, src, (const T*)taux,
                                 (const T*)tauy, st)))
                return rc;
        }
    }
    // boundary fields that default to the initial state feed its adjoint
    if (!in.hasb) {
        if ((rc = addto(ad, T(1), adb, s, B, st))) return rc;
    }
    if ((rc = scale<T>(p, B, 0, ad.u, ad.v, ad.h, (T*)adu0, (T*)adv0, (T*)adh0, st))) return rc;
    if (in.hasb && (adub || advb || adhb)) {
        if ((rc = scale<T>(p, B, 0, adb.u, adb.v, adb.h, (T*)adub, (T*)advb, (T*)adhb, st))) return rc;
    }
    if (adFu || adFv || adFh) {
        if ((rc = scale<T>(p, B, 0, adF.u, adF.v, adF.h, (T*)adFu, (T*)adFv, (T*)adFh, st))) return rc;
    }
    return VD_OK;
}

template <typename T>
static int sw_rhs_t(vd_sw_plan* p, int B, const void* u, const void* v, const void* h, const void* taux,
                    const void* tauy, void* du, void* dv, void* dh, Arena& ws, cudaStream_t st)
{
    Tab<T>& t = tab<T>(p);
    const Sizes s = sizes(p);
    Work<T> wk;
    int rc = take_work<T>(ws, s, B, wk, bf_elems(p));
    if (rc) return rc;
    const Launch Ld = lgrid(p, B), Ll = lgrid(p, B * p->nl);
    Fields<T> x{(T*)u, (T*)v, (T*)h};
    if ((rc = tend_fwd<T>(p, B, x, wk, (const T*)taux, (const T*)tauy, st))) return rc;
    // stage-0 update with dt*k into a scratch state, k0 = tendency (no sponge: zero rates are
    // not guaranteed, so the sponge is removed by passing x as its own target)
    Fields<T> k{(T*)du, (T*)dv, (T*)dh};
    StageArgs sa{0, 0};
    k_sw_update<T, T><<<Ll.grid, Ll.block, 0, st>>>(t, sa, rt(x), r<T>(wk.tuvh.u), r<T>(wk.tuvh.v), r<T>(wk.fx),
                                                     r<T>(wk.fy), rt(wk.k0), rt(wk.k1), rt(x), rt(x), wt(k), wt(wk.x1));
    VD_LAUNCH_CHECK();
    return VD_OK;
}

}  // namespace

#define SW_DISPATCH(fn, ...) \
    (p->esz == 8 ? fn<double>(__VA_ARGS__) : fn<float>(__VA_ARGS__))

extern "C" vd_status vd_sw_step(vd_sw_plan* p, int batch, const void* u0, const void* v0, const void* h0, int nstep,
                                const void* ub, const void* vb, const void* hb, const void* Fu, const void* Fv,
                                const void* Fh, const void* taux, const void* tauy, void* u1, void* v1, void* h1,
                                void* work, size_t work_bytes_, void* stream)
{
    if (!p || batch <= 0 || nstep < 0 || !u0 || !v0 || !h0 || !u1 || !v1 || !h1 || !work) return VD_ERR_ARG;
    if ((Fu || Fv || Fh) && !(Fu && Fv && Fh)) return VD_ERR_ARG;
    if ((ub || vb || hb) && !(ub && vb && hb)) return VD_ERR_ARG;
    if ((long long)batch * p->nl > 65535) return VD_ERR_ARG;
    Arena ws{(char*)work, work_bytes_, 0};
    return SW_DISPATCH(sw_step_t, p, batch, u0, v0, h0, nstep, ub, vb, hb, Fu, Fv, Fh, taux, tauy, u1, v1, h1, ws,
                       (cudaStream_t)stream);
}

extern "C" vd_status vd_sw_step_tgl(vd_sw_plan* p, int batch, const void* u0, const void* v0, const void* h0,
                                    const void* du0, const void* dv0, const void* dh0, int nstep, const void* ub,
                                    const void* vb, const void* hb, const void* dub, const void* dvb, const void* dhb,
                                    const void* Fu, const void* Fv, const void* Fh, const void* dFu, const void* dFv,
                                    const void* dFh, const void* taux, const void* tauy, void* du1, void* dv1,
                                    void* dh1, void* work, size_t work_bytes_, void* stream)
{
    if (!p || batch <= 0 || nstep < 0 || !u0 || !v0 || !h0 || !du0 || !dv0 || !dh0 || !du1 || !dv1 || !dh1 || !work)
        return VD_ERR_ARG;
    if ((Fu || Fv || Fh) && !(Fu && Fv && Fh)) return VD_ERR_ARG;
    if ((dFu || dFv || dFh) && !(dFu && dFv && dFh)) return VD_ERR_ARG;
    if ((ub || vb || hb) && !(ub && vb && hb)) return VD_ERR_ARG;
    if ((dub || dvb || dhb) && !(ub && dub && dvb && dhb)) return VD_ERR_ARG;
    if ((long long)batch * p->nl > 65535) return VD_ERR_ARG;
    Arena ws{(char*)work, work_bytes_, 0};
    return SW_DISPATCH(sw_tgl_t, p, batch, u0, v0, h0, du0, dv0, dh0, nstep, ub, vb, hb, dub, dvb, dhb, Fu, Fv, Fh,
                       dFu, dFv, dFh, taux, tauy, du1, dv1, dh1, ws, (cudaStream_t)stream);
}

extern "C" vd_status vd_sw_step_adj(vd_sw_plan* p, int batch, const void* u0, const void* v0, const void* h0,
                                    const void* adu1, const void* adv1, const void* adh1, int nstep, const void* ub,
                                    const void* vb, const void* hb, const void* Fu, const void* Fv, const void* Fh,
                                    const void* taux, const void* tauy, void* adu0, void* adv0, void* adh0,
                                    void* adub, void* advb, void* adhb, void* adFu, void* adFv, void* adFh,
                                    void* work, size_t work_bytes_, void* stream)
{
    if (!p || batch <= 0 || nstep < 0 || !u0 || !v0 || !h0 || !adu1 || !adv1 || !adh1 || !adu0 || !adv0 || !adh0 ||
        !work)
        return VD_ERR_ARG;
    if ((Fu || Fv || Fh) && !(Fu && Fv && Fh)) return VD_ERR_ARG;
    if ((ub || vb || hb) && !(ub && vb && hb)) return VD_ERR_ARG;
    if ((adub || advb || adhb) && !(adub && advb && adhb)) return VD_ERR_ARG;
    if ((adFu || adFv || adFh) && !(adFu && adFv && adFh)) return VD_ERR_ARG;
    if ((long long)batch * p->nl > 65535) return VD_ERR_ARG;
    Arena ws{(char*)work, work_bytes_, 0};
    return SW_DISPATCH(sw_adj_t, p, batch, u0, v0, h0, adu1, adv1, adh1, nstep, ub, vb, hb, Fu, Fv, Fh, taux, tauy,
                       adu0, adv0, adh0, adub, advb, adhb, adFu, adFv, adFh, ws, (cudaStream_t)stream);
}

extern "C" vd_status vd_sw_rhs(vd_sw_plan* p, int batch, const void* u, const void* v, const void* h,
                               const void* taux, const void* tauy, void* du, void* dv, void* dh, void* work,
                               size_t work_bytes_, void* stream)
{
    if (!p || batch <= 0 || !u || !v || !h || !du || !dv || !dh || !work) return VD_ERR_ARG;
    if ((long long)batch * p->nl > 65535) return VD_ERR_ARG;
    Arena ws{(char*)work, work_bytes_, 0};
    return SW_DISPATCH(sw_rhs_t, p, batch, u, v, h, taux, tauy, du, dv, dh, ws, (cudaStream_t)stream);
}

// ---------------------------------------------------------------- building blocks
// Model-space pieces for drivers that insert an operator between the
// right-hand side and the RK3-SSP combination (the QG model projects every
// SW tendency, qg.py:335-345).
namespace {

template <typename T>
static int sw_rhs_tgl_t(vd_sw_plan* p, int B, const void* u, const void* v, const void* h, const void* du,
                        const void* dv, const void* dh, const void* taux, const void* tauy, void* ku, void* kv,
                        void* kh, void* dku, void* dkv, void* dkh, Arena& ws, cudaStream_t st)
{
    Tab<T>& t = tab<T>(p);
    const Sizes s = sizes(p);
    Work<T> wk, dk;
    int rc = take_work<T>(ws, s, B, wk, bf_elems(p));
    if (rc || (rc = take_work<T>(ws, s, B, dk, bf_elems(p)))) return rc;
    const Launch Ld = lgrid(p, B), Ll = lgrid(p, B * p->nl);
    Fields<T> x{(T*)u, (T*)v, (T*)h}, dx{(T*)du, (T*)dv, (T*)dh};
    using S = DN<T, 1>;
    if ((rc = tend_tgl<T>(p, B, x, dx, wk, dk, (const T*)taux, (const T*)tauy, st))) return rc;
    Fields<T> k{(T*)ku, (T*)kv, (T*)kh}, dkk{(T*)dku, (T*)dkv, (T*)dkh};
    StageArgs sa{0, 0};
    k_sw_update<T, S><<<Ll.grid, Ll.block, 0, st>>>(t, sa, rtd(x, dx), RD<T>{wk.tuvh.u, dk.tuvh.u},
                                                     RD<T>{wk.tuvh.v, dk.tuvh.v}, RD<T>{wk.fx, dk.fx},
                                                     RD<T>{wk.fy, dk.fy}, rtd(wk.k0, dk.k0), rtd(wk.k1, dk.k1),
                                                     rtd(x, dx), rtd(x, dx), wtd(k, dkk), wtd(wk.x1, dk.x1));
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename T>
static int sw_rhs_adj_t(vd_sw_plan* p, int B, const void* u, const void* v, const void* h, const void* aku,
                        const void* akv, const void* akh, void* adu, void* adv, void* adh, Arena& ws, cudaStream_t st)
{
    const Sizes s = sizes(p);
    Work<T> wk;
    int rc = take_work<T>(ws, s, B, wk, bf_elems(p));
    if (rc) return rc;
    T* adom = (T*)ws.take(sizeof(T) * s.sw * B);
    T* adkp = (T*)ws.take(sizeof(T) * s.sh * B);
    T* adht = (T*)ws.take(sizeof(T) * s.sh * B);
    SwSrc<T> src;
    if (!adom || !adkp || !adht || !take_src(ws, s, B, src)) return VD_ERR_WORKSPACE;
    Fields<T> x{(T*)u, (T*)v, (T*)h}, ak{(T*)aku, (T*)akv, (T*)akh}, ad{(T*)adu, (T*)adv, (T*)adh};
    return rhs_adj<T>(p, B, x, ak, ad, wk, adom, adkp, adht, src, nullptr, nullptr, st);
}

// elementwise stage combination: k = rhs + sponge; stage 0/1 store k
template <typename T>
__global__ void k_sw_stage(Tab<T> t, int stage, int nf, int forcing, Fields<T> x, Fields<T> r, Fields<T> k0,
                           Fields<T> k1, Fields<T> xb, Fields<T> F, Fields<T> ks, Fields<T> nx_)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int f = blockIdx.z;
    const int nx = t.nx, ny = t.ny;
    if (i > nx || j > ny || f >= nf) return;
    const T dt = t.dt;
    auto one = [&](long long o, T g, const T* X, const T* R, const T* K0, const T* K1, const T* XB, const T* FF, T* KS,
                   T* NX) {
        const T xv = X[o];
        T k = R[o];
        if (t.has_sponge) k = k + g * (XB[o] - xv);
        if (stage == 0) {
            KS[o] = k;
            NX[o] = xv + dt * k;
        } else if (stage == 1) {
            KS[o] = k;
            NX[o] = xv + (dt / T(4)) * (k - T(3) * K0[o]);
        } else {
            T n = xv + (dt / T(12)) * (T(8) * k - K1[o] - K0[o]);
            if (forcing) n = n + dt * FF[o];
            NX[o] = n;
        }
    };
    if (j < ny) {
        const long long q = (long long)i * ny + j;
        one(f * t.su + q, t.has_sponge ? t.gu[q] : T(0), x.u, r.u, k0.u, k1.u, xb.u, F.u, ks.u, nx_.u);
    }
    if (i < nx) {
        const long long q = (long long)i * (ny + 1) + j;
        one(f * t.sv + q, t.has_sponge ? t.gv[q] : T(0), x.v, r.v, k0.v, k1.v, xb.v, F.v, ks.v, nx_.v);
    }
    if (i < nx && j < ny) {
        const long long q = (long long)i * ny + j;
        one(f * t.sh + q, t.has_sponge ? t.gh[q] : T(0), x.h, r.h, k0.h, k1.h, xb.h, F.h, ks.h, nx_.h);
    }
}

template <typename T>
static Fields<T> F3(const void* a, const void* b, const void* c) { return Fields<T>{(T*)a, (T*)b, (T*)c}; }

}  // namespace

extern "C" vd_status vd_sw_rhs_tgl(vd_sw_plan* p, int batch, const void* u, const void* v, const void* h,
                                   const void* du, const void* dv, const void* dh, const void* taux,
                                   const void* tauy, void* ku, void* kv, void* kh, void* dku, void* dkv, void* dkh,
                                   void* work, size_t work_bytes_, void* stream)
{
    if (!p || batch <= 0 || !u || !v || !h || !du || !dv || !dh || !ku || !kv || !kh || !dku || !dkv || !dkh || !work)
        return VD_ERR_ARG;
    if ((long long)batch * p->nl > 65535) return VD_ERR_ARG;
    Arena ws{(char*)work, work_bytes_, 0};
    return SW_DISPATCH(sw_rhs_tgl_t, p, batch, u, v, h, du, dv, dh, taux, tauy, ku, kv, kh, dku, dkv, dkh, ws,
                       (cudaStream_t)stream);
}

extern "C" vd_status vd_sw_rhs_adj(vd_sw_plan* p, int batch, const void* u, const void* v, const void* h,
                                   const void* aku, const void* akv, const void* akh, void* adu, void* adv,
                                   void* adh, void* work, size_t work_bytes_, void* stream)
{
    if (!p || batch <= 0 || !u || !v || !h || !aku || !akv || !akh || !adu || !adv || !adh || !work)
        return VD_ERR_ARG;
    if ((long long)batch * p->nl > 65535) return VD_ERR_ARG;
    Arena ws{(char*)work, work_bytes_, 0};
    return SW_DISPATCH(sw_rhs_adj_t, p, batch, u, v, h, aku, akv, akh, adu, adv, adh, ws, (cudaStream_t)stream);
}

namespace {
template <typename T>
static int sw_stage_t(vd_sw_plan* p, int B, int stage, const void* const* f, cudaStream_t st)
{
    const Launch L = lgrid(p, B * p->nl);
    const int forcing = f[15] != nullptr;
    k_sw_stage<T><<<L.grid, L.block, 0, st>>>(tab<T>(p), stage, B * p->nl, forcing, F3<T>(f[0], f[1], f[2]),
                                              F3<T>(f[3], f[4], f[5]), F3<T>(f[6], f[7], f[8]),
                                              F3<T>(f[9], f[10], f[11]), F3<T>(f[12], f[13], f[14]),
                                              F3<T>(f[15], f[16], f[17]), F3<T>(f[18], f[19], f[20]),
                                              F3<T>(f[21], f[22], f[23]));
    VD_LAUNCH_CHECK();
    return VD_OK;
}
template <typename T>
static int sw_stage_adj_t(vd_sw_plan* p, int B, int stage, void* const* f, cudaStream_t st)
{
    const Launch L = lgrid(p, B * p->nl);
    k_sw_update_adj<T><<<L.grid, L.block, 0, st>>>(tab<T>(p), stage, B * p->nl, (T*)f[0], (T*)f[1], (T*)f[2],
                                                   (T*)f[3], (T*)f[4], (T*)f[5], (T*)f[6], (T*)f[7], (T*)f[8],
                                                   (T*)f[9], (T*)f[10], (T*)f[11], (T*)f[12], (T*)f[13], (T*)f[14]);
    VD_LAUNCH_CHECK();
    return VD_OK;
}
template <typename T>
static int sw_force_mc_t(vd_sw_plan* p, int B, const void* const* f, cudaStream_t st)
{
    const Launch L = lgrid(p, B * p->nl);
    k_sw_force_mc<T, T><<<L.grid, L.block, 0, st>>>(tab<T>(p), rt(F3<T>(f[0], f[1], f[2])),
                                                     rt(F3<T>(f[3], f[4], f[5])), wt(F3<T>(f[6], f[7], f[8])));
    VD_LAUNCH_CHECK();
    return VD_OK;
}
template <typename T>
static int sw_force_mc_adj_t(vd_sw_plan* p, int B, const void* const* f, cudaStream_t st)
{
    const Launch L = lgrid(p, B * p->nl);
    k_sw_force_mc_adj_h<T><<<L.grid, L.block, 0, st>>>(tab<T>(p), (const T*)f[0], (const T*)f[1], (const T*)f[2],
                                                       (const T*)f[3], (const T*)f[4], (const T*)f[5], (T*)f[6],
                                                       (T*)f[7]);
    VD_LAUNCH_CHECK();
    k_sw_force_mc_adj<T><<<L.grid, L.block, 0, st>>>(tab<T>(p), (const T*)f[0], (const T*)f[1], (const T*)f[2],
                                                     (const T*)f[3], (T*)f[4], (T*)f[5]);
    VD_LAUNCH_CHECK();
    return VD_OK;
}
}  // namespace

extern "C" vd_status vd_sw_stage(vd_sw_plan* p, int batch, int stage, const void* const* fields, void* stream)
{
    if (!p || batch <= 0 || stage < 0 || stage > 2 || !fields) return VD_ERR_ARG;
    for (int k = 0; k < 24; ++k) {
        const bool optional = (k >= 15 && k < 18) || (k >= 6 && k < 12 && stage == 0) || (k >= 9 && k < 12 && stage == 1) ||
                              (k >= 18 && k < 21 && stage == 2);
        if (!fields[k] && !optional) return VD_ERR_ARG;
    }
    if ((long long)batch * p->nl > 65535) return VD_ERR_ARG;
    return SW_DISPATCH(sw_stage_t, p, batch, stage, fields, (cudaStream_t)stream);
}

extern "C" vd_status vd_sw_stage_adj(vd_sw_plan* p, int batch, int stage, void* const* fields, void* stream)
{
    if (!p || batch <= 0 || stage < 0 || stage > 2 || !fields) return VD_ERR_ARG;
    for (int k = 0; k < 15; ++k)
        if (!fields[k]) return VD_ERR_ARG;
    if ((long long)batch * p->nl > 65535) return VD_ERR_ARG;
    return SW_DISPATCH(sw_stage_adj_t, p, batch, stage, fields, (cudaStream_t)stream);
}

extern "C" vd_status vd_sw_scale(vd_sw_plan* p, int batch, int to_physical, const void* u, const void* v,
                                 const void* h, void* uo, void* vo, void* ho, void* stream)
{
    if (!p || batch <= 0 || (u && !uo) || (v && !vo) || (h && !ho)) return VD_ERR_ARG;
    if ((long long)batch * p->nl > 65535) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->esz == 8 ? scale<double>(p, batch, to_physical ? 1 : 0, (const double*)u, (const double*)v,
                                       (const double*)h, (double*)uo, (double*)vo, (double*)ho, st)
                       : scale<float>(p, batch, to_physical ? 1 : 0, (const float*)u, (const float*)v,
                                      (const float*)h, (float*)uo, (float*)vo, (float*)ho, st);
}

extern "C" vd_status vd_sw_force_mc(vd_sw_plan* p, int batch, const void* const* fields, void* stream)
{
    if (!p || batch <= 0 || !fields) return VD_ERR_ARG;
    for (int k = 0; k < 9; ++k)
        if (!fields[k]) return VD_ERR_ARG;
    if ((long long)batch * p->nl > 65535) return VD_ERR_ARG;
    return SW_DISPATCH(sw_force_mc_t, p, batch, fields, (cudaStream_t)stream);
}

extern "C" vd_status vd_sw_force_mc_adj(vd_sw_plan* p, int batch, const void* const* fields, void* stream)
{
    if (!p || batch <= 0 || !fields) return VD_ERR_ARG;
    for (int k = 0; k < 7; ++k)
        if (!fields[k]) return VD_ERR_ARG;
    if ((long long)batch * p->nl > 65535) return VD_ERR_ARG;
    return SW_DISPATCH(sw_force_mc_adj_t, p, batch, fields, (cudaStream_t)stream);
}
