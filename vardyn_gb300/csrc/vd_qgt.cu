// Overlapping-tile QG 1.5-layer model: forward, tangent linear and adjoint
// (mapping/models/model_qg1l/jqgm.py, QgmWithTiles 1033-1376).
//
// Every tile is an independent QG1.5L model: tile-mean f and c, no beta and
// no bathymetry term, the domain's masks sliced to the tile, PV computed on
// the tile interior, Dirichlet values hb on the tile edge. One CTA steps one
// tile for all nstep steps with every field of the tile in shared memory;
// the Helmholtz inversion of the tile interior is the orthonormal DST-I as a
// dense n x n matrix in both directions (S X S, division by the tile's
// eigenvalues, S X S; n = tile - 2). A second kernel blends the weighted
// tiles per domain point, summing the tiles in index order, and divides by
// the summed weights.
#include "vd_internal.cuh"

#include <cmath>
#include <mutex>

namespace vd {

template <typename R>
struct QgtGeom {
    int ny, nx, T, n, ntiles, scheme, hasK;
    R dx, dy, dt, g, K;
};

template <typename R>
__device__ __forceinline__ R qgt_nan()
{
    return sizeof(R) == 8 ? (R)nan("") : (R)nanf("");
}

// class bits of a tile point: 1 = ring class (1 or 2) of the domain, 2 = land
__device__ __forceinline__ bool is12(int8_t c) { return (c & 1) != 0; }
__device__ __forceinline__ bool is0(int8_t c) { return (c & 2) != 0; }

// SSH -> PV of one tile (jqgm.py:1124-1147)
template <typename R>
__device__ void qgt_h2pv(const QgtGeom<R>& G, const R* h, const R* hb, const int8_t* cls, R gf, R gfc2, R* q)
{
    const int T = G.T;
    for (int e = threadIdx.x; e < T * T; e += blockDim.x) {
        const int a = e / T, b = e - a * T;
        R val = R(0);
        if (a >= 1 && a <= T - 2 && b >= 1 && b <= T - 2) {
            const R c = h[e];
            val = gf * ((h[e + T] + h[e - T] - R(2) * c) / (G.dy * G.dy) +
                        (h[e + 1] + h[e - 1] - R(2) * c) / (G.dx * G.dx)) - gfc2 * c;
            if (isnan(val)) val = R(0);
        }
        if (is12(cls[e])) val = -gfc2 * hb[e];
        if (is0(cls[e])) val = R(0);
        q[e] = val;
    }
}

// geostrophic velocities (jqgm.py:1105-1122)
template <typename R>
__device__ void qgt_h2uv(const QgtGeom<R>& G, const R* h, R gf, R* u, R* v)
{
    const int T = G.T;
    for (int e = threadIdx.x; e < T * T; e += blockDim.x) {
        const int a = e / T, b = e - a * T;
        R uu = R(0), vv = R(0);
        if (a >= 1 && a <= T - 2 && b >= 1)
            uu = -gf * (h[e + T - 1] + h[e + T] - h[e - T] - h[e - T - 1]) / (R(4) * G.dy);
        if (a >= 1 && b >= 1 && b <= T - 2)
            vv = gf * (h[e + 1] + h[e - T + 1] - h[e - T - 1] - h[e - 1]) / (R(4) * G.dx);
        u[e] = isnan(uu) ? R(0) : uu;
        v[e] = isnan(vv) ? R(0) : vv;
    }
}

// PV tendency of one tile (jqgm.py:1184-1231): 3rd-order upwind advection and
// diffusion on [2:-2, 2:-2], zero on the domain's ring classes and land
template <typename R>
__device__ void qgt_rhs(const QgtGeom<R>& G, const R* u, const R* v, const R* q, const int8_t* cls, R* k)
{
    const int T = G.T;
    const R cx = R(1) / (R(6) * G.dx), cy = R(1) / (R(6) * G.dy);
    for (int e = threadIdx.x; e < T * T; e += blockDim.x) {
        const int a = e / T, b = e - a * T;
        R r = R(0);
        if (a >= 2 && a <= T - 3 && b >= 2 && b <= T - 3) {
            const R uT = R(0.5) * (u[e] + u[e + 1]);
            const R vT = R(0.5) * (v[e] + v[e + T]);
            const R up = uT < R(0) ? R(0) : uT, um = uT > R(0) ? R(0) : uT;
            const R vp = vT < R(0) ? R(0) : vT, vm = vT > R(0) ? R(0) : vT;
            const R c = q[e];
            r = -up * cx * (R(2) * q[e + 1] + R(3) * c - R(6) * q[e - 1] + q[e - 2]) +
                um * cx * (q[e + 2] - R(6) * q[e + 1] + R(3) * c + R(2) * q[e - 1]) -
                vp * cy * (R(2) * q[e + T] + R(3) * c - R(6) * q[e - T] + q[e - 2 * T]) +
                vm * cy * (q[e + 2 * T] - R(6) * q[e + T] + R(3) * c + R(2) * q[e - T]);
            if (G.hasK)
                r += G.K / (G.dx * G.dx) * (q[e + 1] + q[e - 1] - R(2) * c) +
                     G.K / (G.dy * G.dy) * (q[e + T] + q[e - T] - R(2) * c);
        }
        if (isnan(r) || cls[e] != 0) r = R(0);
        k[e] = r;
    }
}

// out = X S (transform along the last axis) or S X (along the first), n x n
template <typename R>
__device__ void qgt_mul(int n, const R* X, const R* S, R* out, bool right)
{
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int p = e / n, s = e - p * n;
        R acc = R(0);
        if (right)
            for (int t = 0; t < n; ++t) acc += X[p * n + t] * S[t * n + s];
        else
            for (int t = 0; t < n; ++t) acc += S[p * n + t] * X[t * n + s];
        out[e] = acc;
    }
}

// A <- S (S (S A S) / (gf lap - gfc2)) S: the interior Helmholtz inversion,
// symmetric because S is (B is scratch)
template <typename R>
__device__ void qgt_invert(int n, const R* S, const R* lap, R gf, R gfc2, R* A, R* B)
{
    qgt_mul(n, A, S, B, true);
    __syncthreads();
    qgt_mul(n, B, S, A, false);
    __syncthreads();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) A[e] = A[e] / (gf * lap[e] - gfc2);
    __syncthreads();
    qgt_mul(n, A, S, B, true);
    __syncthreads();
    qgt_mul(n, B, S, A, false);
    __syncthreads();
}

// PV -> SSH of one tile (jqgm.py:1149-1170): h = hb + the inversion of
// q - qb on the interior, the edge keeps hb. With qb and hb NULL this is the
// linear map dq -> dh of the tangent (zero on the edge).
template <typename R>
__device__ void qgt_pv2h(const QgtGeom<R>& G, const R* q, const R* qb, const R* hb, const R* S, const R* lap,
                         R gf, R gfc2, R* A, R* B, R* h)
{
    const int T = G.T, n = G.n;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int p = e / n, s = e - p * n;
        const int o = (p + 1) * T + (s + 1);
        A[e] = qb ? q[o] - qb[o] : q[o];
    }
    __syncthreads();
    qgt_invert(n, S, lap, gf, gfc2, A, B);
    for (int e = threadIdx.x; e < T * T; e += blockDim.x) {
        const int a = e / T, b = e - a * T;
        const bool in = a >= 1 && a <= T - 2 && b >= 1 && b <= T - 2;
        const R x = in ? A[(a - 1) * n + (b - 1)] : R(0);
        h[e] = hb ? hb[e] + x : x;
    }
    __syncthreads();
}

template <typename R>
__global__ void __launch_bounds__(256)
k_qgt_tile(QgtGeom<R> G, const int32_t* __restrict__ org, const double* __restrict__ ftile,
           const double* __restrict__ ctile, const int8_t* __restrict__ mask, const R* __restrict__ Sg,
           const R* __restrict__ lapg, const R* __restrict__ wg, const R* __restrict__ mdt,
           const R* __restrict__ h0, const R* __restrict__ hbg, int nstep, R* __restrict__ tout)
{
    extern __shared__ __align__(16) unsigned char qgt_smem[];
    const int T = G.T, n = G.n, TT = T * T, nn = n * n;
    R* h = reinterpret_cast<R*>(qgt_smem);
    R* q = h + TT;
    R* qb = q + TT;
    R* hb = qb + TT;
    R* q12 = hb + TT;
    R* u = q12 + TT;
    R* v = u + TT;
    R* k = v + TT;
    R* A = k + TT;
    R* B = A + nn;
    R* S = B + nn;
    R* lap = S + nn;
    int8_t* cls = reinterpret_cast<int8_t*>(lap + nn);
    const int t = blockIdx.x;
    const int ys = org[2 * t], xs = org[2 * t + 1];
    const R f = (R)ftile[t], c = (R)ctile[t];
    const R gf = G.g / f, gfc2 = G.g * f / (c * c);
    for (int e = threadIdx.x; e < TT; e += blockDim.x) {
        const int a = e / T, b = e - a * T;
        const long long o = (long long)(ys + a) * G.nx + (xs + b);
        const R m = mdt ? mdt[o] : R(0);
        h[e] = h0[o] + m;
        hb[e] = hbg[o] + m;
        const int8_t cl = mask[o];
        cls[e] = (int8_t)((cl == 1 || cl == 2 ? 1 : 0) | (cl == 0 ? 2 : 0));
    }
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        S[e] = Sg[e];
        lap[e] = lapg[e];
    }
    __syncthreads();
    qgt_h2pv(G, h, hb, cls, gf, gfc2, q);
    qgt_h2pv(G, hb, hb, cls, gf, gfc2, qb);
    __syncthreads();
    for (int step = 0; step < nstep; ++step) {
        qgt_h2uv(G, h, gf, u, v);
        __syncthreads();
        qgt_rhs(G, u, v, q, cls, k);
        __syncthreads();
        if (G.scheme == VD_RK2) {
            // q12 = q + dt/2 k, h12 = pv2h(q12), k = rhs(h2uv(h12), q12)
            for (int e = threadIdx.x; e < TT; e += blockDim.x) q12[e] = q[e] + R(0.5) * k[e] * G.dt;
            __syncthreads();
            qgt_pv2h(G, q12, qb, hb, S, lap, gf, gfc2, A, B, h);
            qgt_h2uv(G, h, gf, u, v);
            __syncthreads();
            qgt_rhs(G, u, v, q12, cls, k);
            __syncthreads();
        }
        for (int e = threadIdx.x; e < TT; e += blockDim.x) q[e] = q[e] + G.dt * k[e];
        __syncthreads();
        qgt_pv2h(G, q, qb, hb, S, lap, gf, gfc2, A, B, h);
    }
    R* out = tout + (long long)t * TT;
    for (int e = threadIdx.x; e < TT; e += blockDim.x) out[e] = wg[e] * (is0(cls[e]) ? qgt_nan<R>() : h[e]);
}

// h1 = sum over the tiles covering a point of their weighted SSH / summed
// weights, minus the MDT (jqgm.py:1340-1356)
template <typename R>
__global__ void k_qgt_blend(QgtGeom<R> G, const int32_t* __restrict__ org, const R* __restrict__ tout,
                            const R* __restrict__ wsum, const R* __restrict__ mdt, R* __restrict__ h1)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= G.nx || y >= G.ny) return;
    const int T = G.T;
    R acc = R(0);
    for (int t = 0; t < G.ntiles; ++t) {
        const int a = y - org[2 * t], b = x - org[2 * t + 1];
        if (a >= 0 && a < T && b >= 0 && b < T) acc += tout[(long long)t * T * T + a * T + b];
    }
    const long long o = (long long)y * G.nx + x;
    R r = wsum ? acc / wsum[o] : acc;
    if (mdt) r -= mdt[o];
    h1[o] = r;
}

// ---------------------------------------------------------------------------
// Tangent linear and adjoint of the blended step with respect to h0
// (jax.jvp / jax.vjp, jqgm.py:1358-1376). Every tile's Jacobian is that of
// its own QG1.5L model: the upwind branches and the NaN guards of the
// trajectory select the linear map (a guarded value passes no derivative;
// where(u < 0, 0, u) passes it for u >= 0, where(u > 0, 0, u) for u <= 0).
// One CTA per tile; the dense DST matrix, the eigenvalues and the two n x n
// work blocks sit in shared memory, the tile's fields in a per-tile global
// slab (L2-resident), the adjoint's forward trajectory (the stage inputs
// (h_s, q_s) of every step) behind it. Every adjoint operator is written as
// a gather, so no atomics are needed and the result is deterministic.
// ---------------------------------------------------------------------------

// fields of the tangent's per-tile slab
enum { QGT_TL_FIELDS = 14 };
// fields of the adjoint's per-tile slab
enum { QGT_AD_FIELDS = 20 };

template <typename R>
__device__ __forceinline__ R qgt_at(const R* x, int T, int a, int b)
{
    return (a >= 0 && a < T && b >= 0 && b < T) ? x[a * T + b] : R(0);
}

// raw (unguarded) PV of an interior point
template <typename R>
__device__ __forceinline__ R qgt_pv_raw(const QgtGeom<R>& G, const R* h, int e, R gf, R gfc2)
{
    const int T = G.T;
    const R c = h[e];
    return gf * ((h[e + T] + h[e - T] - R(2) * c) / (G.dy * G.dy) + (h[e + 1] + h[e - 1] - R(2) * c) / (G.dx * G.dx)) -
           gfc2 * c;
}

// raw geostrophic velocities at a point; valid flags carry the index ranges
template <typename R>
__device__ __forceinline__ void qgt_uv_raw(const QgtGeom<R>& G, const R* h, int a, int b, R gf, R& uu, R& vv,
                                           bool& ue, bool& ve)
{
    const int T = G.T, e = a * T + b;
    ue = a >= 1 && a <= T - 2 && b >= 1;
    ve = a >= 1 && b >= 1 && b <= T - 2;
    uu = ue ? -gf * (h[e + T - 1] + h[e + T] - h[e - T] - h[e - T - 1]) / (R(4) * G.dy) : R(0);
    vv = ve ? gf * (h[e + 1] + h[e - T + 1] - h[e - T - 1] - h[e - 1]) / (R(4) * G.dx) : R(0);
}

// upwind stencils of q at a core point: Dp = 2q[+1] + 3q - 6q[-1] + q[-2],
// Dm = q[+2] - 6q[+1] + 3q + 2q[-1], along x (stride 1) and y (stride T)
template <typename R>
struct QgtStencil {
    R px, mx, py, my, lx, ly;
};

template <typename R>
__device__ __forceinline__ QgtStencil<R> qgt_stencil(const R* q, int e, int T)
{
    QgtStencil<R> d;
    const R c = q[e];
    d.px = R(2) * q[e + 1] + R(3) * c - R(6) * q[e - 1] + q[e - 2];
    d.mx = q[e + 2] - R(6) * q[e + 1] + R(3) * c + R(2) * q[e - 1];
    d.py = R(2) * q[e + T] + R(3) * c - R(6) * q[e - T] + q[e - 2 * T];
    d.my = q[e + 2 * T] - R(6) * q[e + T] + R(3) * c + R(2) * q[e - T];
    d.lx = q[e + 1] + q[e - 1] - R(2) * c;
    d.ly = q[e + T] + q[e - T] - R(2) * c;
    return d;
}

__device__ __forceinline__ bool qgt_core(int T, int a, int b) { return a >= 2 && a <= T - 3 && b >= 2 && b <= T - 3; }

// raw tendency at a core point (the forward formula, unguarded)
template <typename R>
__device__ __forceinline__ R qgt_rhs_raw(const QgtGeom<R>& G, const R* u, const R* v, const R* q, int e)
{
    const int T = G.T;
    const R cx = R(1) / (R(6) * G.dx), cy = R(1) / (R(6) * G.dy);
    const R uT = R(0.5) * (u[e] + u[e + 1]);
    const R vT = R(0.5) * (v[e] + v[e + T]);
    const R up = uT < R(0) ? R(0) : uT, um = uT > R(0) ? R(0) : uT;
    const R vp = vT < R(0) ? R(0) : vT, vm = vT > R(0) ? R(0) : vT;
    const QgtStencil<R> d = qgt_stencil(q, e, T);
    R r = -up * cx * d.px + um * cx * d.mx - vp * cy * d.py + vm * cy * d.my;
    if (G.hasK) r += G.K / (G.dx * G.dx) * d.lx + G.K / (G.dy * G.dy) * d.ly;
    return r;
}

// dq = tangent of the tile PV: the interior stencil of dh on the free points
// whose raw PV is a number
template <typename R>
__device__ void qgt_h2pv_tl(const QgtGeom<R>& G, const R* dh, const R* h, const int8_t* cls, R gf, R gfc2, R* dq)
{
    const int T = G.T;
    for (int e = threadIdx.x; e < T * T; e += blockDim.x) {
        const int a = e / T, b = e - a * T;
        R val = R(0);
        if (a >= 1 && a <= T - 2 && b >= 1 && b <= T - 2 && cls[e] == 0 && !isnan(qgt_pv_raw(G, h, e, gf, gfc2)))
            val = qgt_pv_raw(G, dh, e, gf, gfc2);
        dq[e] = val;
    }
}

template <typename R>
__device__ void qgt_h2uv_tl(const QgtGeom<R>& G, const R* dh, const R* h, R gf, R* du, R* dv)
{
    const int T = G.T;
    for (int e = threadIdx.x; e < T * T; e += blockDim.x) {
        const int a = e / T, b = e - a * T;
        R uu, vv, du_, dv_;
        bool ue, ve;
        qgt_uv_raw(G, h, a, b, gf, uu, vv, ue, ve);
        qgt_uv_raw(G, dh, a, b, gf, du_, dv_, ue, ve);
        du[e] = isnan(uu) ? R(0) : du_;
        dv[e] = isnan(vv) ? R(0) : dv_;
    }
}

template <typename R>
__device__ void qgt_rhs_tl(const QgtGeom<R>& G, const R* u, const R* v, const R* du, const R* dv, const R* q,
                           const R* dq, const int8_t* cls, R* dk)
{
    const int T = G.T;
    const R cx = R(1) / (R(6) * G.dx), cy = R(1) / (R(6) * G.dy);
    for (int e = threadIdx.x; e < T * T; e += blockDim.x) {
        const int a = e / T, b = e - a * T;
        R r = R(0);
        if (qgt_core(T, a, b) && cls[e] == 0 && !isnan(qgt_rhs_raw(G, u, v, q, e))) {
            const R uT = R(0.5) * (u[e] + u[e + 1]), vT = R(0.5) * (v[e] + v[e + T]);
            const R duT = R(0.5) * (du[e] + du[e + 1]), dvT = R(0.5) * (dv[e] + dv[e + T]);
            const R up = uT < R(0) ? R(0) : uT, um = uT > R(0) ? R(0) : uT;
            const R vp = vT < R(0) ? R(0) : vT, vm = vT > R(0) ? R(0) : vT;
            const R dup = uT < R(0) ? R(0) : duT, dum = uT > R(0) ? R(0) : duT;
            const R dvp = vT < R(0) ? R(0) : dvT, dvm = vT > R(0) ? R(0) : dvT;
            const QgtStencil<R> s = qgt_stencil(q, e, T);
            const QgtStencil<R> d = qgt_stencil(dq, e, T);
            r = -dup * cx * s.px + dum * cx * s.mx - dvp * cy * s.py + dvm * cy * s.my -
                up * cx * d.px + um * cx * d.mx - vp * cy * d.py + vm * cy * d.my;
            if (G.hasK) r += G.K / (G.dx * G.dx) * d.lx + G.K / (G.dy * G.dy) * d.ly;
        }
        dk[e] = r;
    }
}

// loads one tile: h = h0 + mdt, hb = hb + mdt, point classes, S and lap
template <typename R>
__device__ void qgt_load(const QgtGeom<R>& G, int ys, int xs, const int8_t* mask, const R* mdt, const R* h0,
                         const R* hbg, const R* Sg, const R* lapg, R* h, R* hb, int8_t* cls, R* S, R* lap)
{
    const int T = G.T, nn = G.n * G.n;
    for (int e = threadIdx.x; e < T * T; e += blockDim.x) {
        const int a = e / T, b = e - a * T;
        const long long o = (long long)(ys + a) * G.nx + (xs + b);
        const R m = mdt ? mdt[o] : R(0);
        h[e] = h0[o] + m;
        hb[e] = hbg[o] + m;
        const int8_t cl = mask[o];
        cls[e] = (int8_t)((cl == 1 || cl == 2 ? 1 : 0) | (cl == 0 ? 2 : 0));
    }
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        S[e] = Sg[e];
        lap[e] = lapg[e];
    }
}

template <typename R>
__global__ void __launch_bounds__(256)
k_qgt_tile_tl(QgtGeom<R> G, const int32_t* __restrict__ org, const double* __restrict__ ftile,
              const double* __restrict__ ctile, const int8_t* __restrict__ mask, const R* __restrict__ Sg,
              const R* __restrict__ lapg, const R* __restrict__ wg, const R* __restrict__ mdt,
              const R* __restrict__ h0, const R* __restrict__ hbg, const R* __restrict__ dh0, int nstep,
              R* __restrict__ scratch, R* __restrict__ tout)
{
    extern __shared__ __align__(16) unsigned char qgt_smem[];
    const int T = G.T, n = G.n, TT = T * T, nn = n * n;
    R* S = reinterpret_cast<R*>(qgt_smem);
    R* lap = S + nn;
    R* A = lap + nn;
    R* B = A + nn;
    int8_t* cls = reinterpret_cast<int8_t*>(B + nn);
    const int t = blockIdx.x;
    R* h = scratch + (size_t)t * QGT_TL_FIELDS * TT;
    R *q = h + TT, *qb = q + TT, *hb = qb + TT, *q12 = hb + TT, *u = q12 + TT, *v = u + TT, *k = v + TT;
    R *dh = k + TT, *dq = dh + TT, *dq12 = dq + TT, *du = dq12 + TT, *dv = du + TT, *dk = dv + TT;
    const int ys = org[2 * t], xs = org[2 * t + 1];
    const R f = (R)ftile[t], c = (R)ctile[t];
    const R gf = G.g / f, gfc2 = G.g * f / (c * c);
    qgt_load(G, ys, xs, mask, mdt, h0, hbg, Sg, lapg, h, hb, cls, S, lap);
    for (int e = threadIdx.x; e < TT; e += blockDim.x) {
        const int a = e / T, b = e - a * T;
        dh[e] = dh0[(long long)(ys + a) * G.nx + (xs + b)];
    }
    __syncthreads();
    qgt_h2pv(G, h, hb, cls, gf, gfc2, q);
    qgt_h2pv(G, hb, hb, cls, gf, gfc2, qb);
    qgt_h2pv_tl(G, dh, h, cls, gf, gfc2, dq);
    __syncthreads();
    for (int step = 0; step < nstep; ++step) {
        qgt_h2uv(G, h, gf, u, v);
        qgt_h2uv_tl(G, dh, h, gf, du, dv);
        __syncthreads();
        qgt_rhs(G, u, v, q, cls, k);
        qgt_rhs_tl(G, u, v, du, dv, q, dq, cls, dk);
        __syncthreads();
        if (G.scheme == VD_RK2) {
            for (int e = threadIdx.x; e < TT; e += blockDim.x) {
                q12[e] = q[e] + R(0.5) * k[e] * G.dt;
                dq12[e] = dq[e] + R(0.5) * dk[e] * G.dt;
            }
            __syncthreads();
            qgt_pv2h(G, q12, qb, hb, S, lap, gf, gfc2, A, B, h);
            qgt_pv2h<R>(G, dq12, nullptr, nullptr, S, lap, gf, gfc2, A, B, dh);
            qgt_h2uv(G, h, gf, u, v);
            qgt_h2uv_tl(G, dh, h, gf, du, dv);
            __syncthreads();
            qgt_rhs(G, u, v, q12, cls, k);
            qgt_rhs_tl(G, u, v, du, dv, q12, dq12, cls, dk);
            __syncthreads();
        }
        for (int e = threadIdx.x; e < TT; e += blockDim.x) {
            q[e] = q[e] + G.dt * k[e];
            dq[e] = dq[e] + G.dt * dk[e];
        }
        __syncthreads();
        qgt_pv2h(G, q, qb, hb, S, lap, gf, gfc2, A, B, h);
        qgt_pv2h<R>(G, dq, nullptr, nullptr, S, lap, gf, gfc2, A, B, dh);
    }
    R* out = tout + (size_t)t * TT;
    for (int e = threadIdx.x; e < TT; e += blockDim.x) out[e] = wg[e] * (is0(cls[e]) ? R(0) : dh[e]);
}

// adjoint of one stage tendency k = rhs(h2uv(h), q) at the stage input
// (h, q): adh = the h-adjoint (overwritten), adq = the q-adjoint
// (overwritten); u, v, a, aduT, advT, adu, adv are scratch
template <typename R>
__device__ void qgt_tend_adj(const QgtGeom<R>& G, const R* h, const R* q, const R* adk, const int8_t* cls, R gf,
                             R* u, R* v, R* a, R* aduT, R* advT, R* adu, R* adv, R* adh, R* adq)
{
    const int T = G.T, TT = T * T;
    const R cx = R(1) / (R(6) * G.dx), cy = R(1) / (R(6) * G.dy);
    const R kx = G.hasK ? G.K / (G.dx * G.dx) : R(0), ky = G.hasK ? G.K / (G.dy * G.dy) : R(0);
    qgt_h2uv(G, h, gf, u, v);
    __syncthreads();
    // the tendency's adjoint input where the tendency is live, and the
    // adjoints of the T-point velocities uT, vT
    for (int e = threadIdx.x; e < TT; e += blockDim.x) {
        const int ea = e / T, eb = e - ea * T;
        R ae = R(0), au = R(0), av = R(0);
        if (qgt_core(T, ea, eb) && cls[e] == 0 && !isnan(qgt_rhs_raw(G, u, v, q, e))) {
            ae = adk[e];
            const R uT = R(0.5) * (u[e] + u[e + 1]), vT = R(0.5) * (v[e] + v[e + T]);
            const QgtStencil<R> d = qgt_stencil(q, e, T);
            au = (uT < R(0) ? R(0) : -cx * d.px * ae) + (uT > R(0) ? R(0) : cx * d.mx * ae);
            av = (vT < R(0) ? R(0) : -cy * d.py * ae) + (vT > R(0) ? R(0) : cy * d.my * ae);
        }
        a[e] = ae;
        aduT[e] = au;
        advT[e] = av;
    }
    __syncthreads();
    // q-adjoint (gather of the upwind and diffusion stencils' transposes)
    // and the adjoints of u, v (uT = (u[e] + u[e+1]) / 2, vT = (v[e] + v[e+T]) / 2)
    for (int p = threadIdx.x; p < TT; p += blockDim.x) {
        const int pa = p / T, pb = p - pa * T;
        R acc = R(0);
        // x neighbours e = p - d contribute the coefficient of q[e + d]
        for (int d = -2; d <= 2; ++d) {
            const int eb = pb - d;
            if (!qgt_core(T, pa, eb)) continue;
            const int e = pa * T + eb;
            const R ae = a[e];
            if (ae == R(0)) continue;
            const R uT = R(0.5) * (u[e] + u[e + 1]);
            const R up = uT < R(0) ? R(0) : uT, um = uT > R(0) ? R(0) : uT;
            R cf;
            switch (d) {
            case 2: cf = cx * um; break;
            case 1: cf = -R(2) * cx * up - R(6) * cx * um + kx; break;
            case 0: {
                const R vT = R(0.5) * (v[e] + v[e + T]);
                const R vp = vT < R(0) ? R(0) : vT, vm = vT > R(0) ? R(0) : vT;
                cf = -R(3) * cx * up + R(3) * cx * um - R(3) * cy * vp + R(3) * cy * vm - R(2) * kx - R(2) * ky;
                break;
            }
            case -1: cf = R(6) * cx * up + R(2) * cx * um + kx; break;
            default: cf = -cx * up; break;
            }
            acc += cf * ae;
        }
        for (int d = -2; d <= 2; ++d) {
            if (d == 0) continue;
            const int ea = pa - d;
            if (!qgt_core(T, ea, pb)) continue;
            const int e = ea * T + pb;
            const R ae = a[e];
            if (ae == R(0)) continue;
            const R vT = R(0.5) * (v[e] + v[e + T]);
            const R vp = vT < R(0) ? R(0) : vT, vm = vT > R(0) ? R(0) : vT;
            R cf;
            switch (d) {
            case 2: cf = cy * vm; break;
            case 1: cf = -R(2) * cy * vp - R(6) * cy * vm + ky; break;
            case -1: cf = R(6) * cy * vp + R(2) * cy * vm + ky; break;
            default: cf = -cy * vp; break;
            }
            acc += cf * ae;
        }
        adq[p] = acc;
        R uu, vv;
        bool ue, ve;
        qgt_uv_raw(G, h, pa, pb, gf, uu, vv, ue, ve);
        R au = R(0.5) * (aduT[p] + (pb >= 1 ? aduT[p - 1] : R(0)));
        R av = R(0.5) * (advT[p] + (pa >= 1 ? advT[p - T] : R(0)));
        adu[p] = (ue && !isnan(uu)) ? au : R(0);
        adv[p] = (ve && !isnan(vv)) ? av : R(0);
    }
    __syncthreads();
    // h-adjoint of the geostrophic velocities
    const R cu = -gf / (R(4) * G.dy), cv = gf / (R(4) * G.dx);
    for (int p = threadIdx.x; p < TT; p += blockDim.x) {
        const int pa = p / T, pb = p - pa * T;
        adh[p] = cu * (qgt_at(adu, T, pa - 1, pb + 1) + qgt_at(adu, T, pa - 1, pb) - qgt_at(adu, T, pa + 1, pb) -
                       qgt_at(adu, T, pa + 1, pb + 1)) +
                 cv * (qgt_at(adv, T, pa, pb - 1) + qgt_at(adv, T, pa + 1, pb - 1) - qgt_at(adv, T, pa + 1, pb + 1) -
                       qgt_at(adv, T, pa, pb + 1));
    }
    __syncthreads();
}

// adq[interior] += pv2h adjoint of adh (the symmetric interior inversion)
template <typename R>
__device__ void qgt_pv2h_adj_add(const QgtGeom<R>& G, const R* adh, const R* S, const R* lap, R gf, R gfc2, R* A,
                                 R* B, R* adq)
{
    const int T = G.T, n = G.n;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int p = e / n, s = e - p * n;
        A[e] = adh[(p + 1) * T + (s + 1)];
    }
    __syncthreads();
    qgt_invert(n, S, lap, gf, gfc2, A, B);
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int p = e / n, s = e - p * n;
        adq[(p + 1) * T + (s + 1)] += A[e];
    }
    __syncthreads();
}

template <typename R>
__global__ void __launch_bounds__(256)
k_qgt_tile_adj(QgtGeom<R> G, const int32_t* __restrict__ org, const double* __restrict__ ftile,
               const double* __restrict__ ctile, const int8_t* __restrict__ mask, const R* __restrict__ Sg,
               const R* __restrict__ lapg, const R* __restrict__ wg, const R* __restrict__ wsum,
               const R* __restrict__ mdt, const R* __restrict__ h0, const R* __restrict__ hbg,
               const R* __restrict__ adh1, int nstep, R* __restrict__ scratch, R* __restrict__ traj,
               R* __restrict__ tout)
{
    extern __shared__ __align__(16) unsigned char qgt_smem[];
    const int T = G.T, n = G.n, TT = T * T, nn = n * n;
    const int ns = G.scheme == VD_RK2 ? 2 : 1;
    R* S = reinterpret_cast<R*>(qgt_smem);
    R* lap = S + nn;
    R* A = lap + nn;
    R* B = A + nn;
    int8_t* cls = reinterpret_cast<int8_t*>(B + nn);
    const int t = blockIdx.x;
    R* hi = scratch + (size_t)t * QGT_AD_FIELDS * TT;
    R *hb = hi + TT, *qb = hb + TT, *h = qb + TT, *q = h + TT, *q12 = q + TT, *u = q12 + TT, *v = u + TT;
    R *k = v + TT, *adh = k + TT, *adq = adh + TT, *acc = adq + TT, *adk0 = acc + TT, *a = adk0 + TT;
    R *aduT = a + TT, *advT = aduT + TT, *adu = advT + TT, *adv = adu + TT, *xh = adv + TT, *xq = xh + TT;
    R* tr = traj + (size_t)t * nstep * ns * 2 * TT;
    const int ys = org[2 * t], xs = org[2 * t + 1];
    const R f = (R)ftile[t], c = (R)ctile[t];
    const R gf = G.g / f, gfc2 = G.g * f / (c * c);
    qgt_load(G, ys, xs, mask, mdt, h0, hbg, Sg, lapg, hi, hb, cls, S, lap);
    __syncthreads();
    qgt_h2pv(G, hi, hb, cls, gf, gfc2, q);
    qgt_h2pv(G, hb, hb, cls, gf, gfc2, qb);
    for (int e = threadIdx.x; e < TT; e += blockDim.x) h[e] = hi[e];
    __syncthreads();
    // forward, keeping the stage inputs of every step
    for (int step = 0; step < nstep; ++step) {
        R* s0 = tr + (size_t)step * ns * 2 * TT;
        for (int e = threadIdx.x; e < TT; e += blockDim.x) {
            s0[e] = h[e];
            s0[TT + e] = q[e];
        }
        qgt_h2uv(G, h, gf, u, v);
        __syncthreads();
        qgt_rhs(G, u, v, q, cls, k);
        __syncthreads();
        if (G.scheme == VD_RK2) {
            for (int e = threadIdx.x; e < TT; e += blockDim.x) q12[e] = q[e] + R(0.5) * k[e] * G.dt;
            __syncthreads();
            qgt_pv2h(G, q12, qb, hb, S, lap, gf, gfc2, A, B, h);
            R* s1 = s0 + 2 * TT;
            for (int e = threadIdx.x; e < TT; e += blockDim.x) {
                s1[e] = h[e];
                s1[TT + e] = q12[e];
            }
            qgt_h2uv(G, h, gf, u, v);
            __syncthreads();
            qgt_rhs(G, u, v, q12, cls, k);
            __syncthreads();
        }
        for (int e = threadIdx.x; e < TT; e += blockDim.x) q[e] = q[e] + G.dt * k[e];
        __syncthreads();
        qgt_pv2h(G, q, qb, hb, S, lap, gf, gfc2, A, B, h);
    }
    // adjoint of the tile's output w * where(land, NaN, h) and of the blend's
    // division by the summed weights; NaN in the incoming adjoint reads as 0
    for (int e = threadIdx.x; e < TT; e += blockDim.x) {
        const int ea = e / T, eb = e - ea * T;
        const long long o = (long long)(ys + ea) * G.nx + (xs + eb);
        R x = wg[e] * (adh1[o] / wsum[o]);
        if (is0(cls[e]) || isnan(x)) x = R(0);
        adh[e] = x;
        adq[e] = R(0);
    }
    __syncthreads();
    for (int step = nstep - 1; step >= 0; --step) {
        const R* s0 = tr + (size_t)step * ns * 2 * TT;
        qgt_pv2h_adj_add(G, adh, S, lap, gf, gfc2, A, B, adq);
        for (int e = threadIdx.x; e < TT; e += blockDim.x) {
            acc[e] = adq[e];
            if (G.scheme == VD_RK2) {
                k[e] = G.dt * adq[e];           // adjoint of the second stage's tendency
                adk0[e] = R(0) * adq[e];
            } else {
                adk0[e] = G.dt * adq[e];
            }
        }
        __syncthreads();
        if (G.scheme == VD_RK2) {
            const R* s1 = s0 + 2 * TT;
            qgt_tend_adj(G, s1, s1 + TT, k, cls, gf, u, v, a, aduT, advT, adu, adv, xh, xq);
            qgt_pv2h_adj_add(G, xh, S, lap, gf, gfc2, A, B, xq);
            for (int e = threadIdx.x; e < TT; e += blockDim.x) {
                acc[e] += xq[e];
                adk0[e] += R(0.5) * G.dt * xq[e];
            }
            __syncthreads();
        }
        qgt_tend_adj(G, s0, s0 + TT, adk0, cls, gf, u, v, a, aduT, advT, adu, adv, xh, xq);
        for (int e = threadIdx.x; e < TT; e += blockDim.x) {
            adh[e] = xh[e];
            adq[e] = acc[e] + xq[e];
        }
        __syncthreads();
    }
    // h-adjoint of the initial PV (interior free points whose raw PV is a number)
    for (int e = threadIdx.x; e < TT; e += blockDim.x) {
        const int ea = e / T, eb = e - ea * T;
        const bool live = ea >= 1 && ea <= T - 2 && eb >= 1 && eb <= T - 2 && cls[e] == 0 &&
                          !isnan(qgt_pv_raw(G, hi, e, gf, gfc2));
        a[e] = live ? adq[e] : R(0);
    }
    __syncthreads();
    const R cyy = gf / (G.dy * G.dy), cxx = gf / (G.dx * G.dx);
    R* out = tout + (size_t)t * TT;
    for (int p = threadIdx.x; p < TT; p += blockDim.x) {
        const int pa = p / T, pb = p - pa * T;
        out[p] = adh[p] + cyy * (qgt_at(a, T, pa - 1, pb) + qgt_at(a, T, pa + 1, pb)) +
                 cxx * (qgt_at(a, T, pa, pb - 1) + qgt_at(a, T, pa, pb + 1)) +
                 (-R(2) * cyy - R(2) * cxx - gfc2) * a[p];
    }
}

template <typename R>
static size_t qgt_smem(int T)
{
    const size_t n = (size_t)T - 2;
    return (8 * (size_t)T * T + 4 * n * n) * sizeof(R) + (size_t)T * T;
}

template <typename R>
static int qgt_run(const vd_qgt_desc* d, const void* h0, const void* hb, int nstep, void* h1, void* work,
                   cudaStream_t st)
{
    static PerDeviceOnce once;
    const cudaError_t attr = once.run([]() -> cudaError_t {
        return cudaFuncSetAttribute(k_qgt_tile<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    });
    if (attr != cudaSuccess) return VD_ERR_CUDA;
    QgtGeom<R> G;
    G.ny = d->ny; G.nx = d->nx; G.T = d->tile; G.n = d->tile - 2; G.ntiles = d->ntiles;
    G.scheme = d->time_scheme; G.hasK = d->has_Kdiffus;
    G.dx = (R)d->dx; G.dy = (R)d->dy; G.dt = (R)d->dt; G.g = (R)d->g; G.K = (R)d->Kdiffus;
    k_qgt_tile<R><<<(unsigned)d->ntiles, 256, qgt_smem<R>(d->tile), st>>>(
        G, d->origins, d->f_tile, d->c_tile, d->mask, (const R*)d->S, (const R*)d->lap, (const R*)d->weights,
        (const R*)d->mdt, (const R*)h0, (const R*)hb, nstep, (R*)work);
    VD_LAUNCH_CHECK();
    k_qgt_blend<R><<<dim3((unsigned)((d->nx + 127) / 128), (unsigned)d->ny), 128, 0, st>>>(
        G, d->origins, (const R*)work, (const R*)d->wsum, (const R*)d->mdt, (R*)h1);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename R>
static size_t qgt_ad_smem(int T)
{
    const size_t n = (size_t)T - 2;
    return 4 * n * n * sizeof(R) + (size_t)T * T;
}

static size_t qgt_ad_elems(const vd_qgt_desc* d, int nstep, int adjoint)
{
    const size_t TT = (size_t)d->tile * d->tile, nt = (size_t)d->ntiles;
    const size_t ns = d->time_scheme == VD_RK2 ? 2 : 1;
    if (!adjoint) return nt * TT * (1 + QGT_TL_FIELDS);
    return nt * TT * (1 + QGT_AD_FIELDS + (size_t)nstep * ns * 2);
}

template <typename R>
static int qgt_run_ad(const vd_qgt_desc* d, int adjoint, const void* x, const void* h0, const void* hb, int nstep,
                      void* out, void* work, cudaStream_t st)
{
    static PerDeviceOnce once;
    const cudaError_t attr = once.run([]() -> cudaError_t {
        cudaError_t e = cudaFuncSetAttribute(k_qgt_tile_tl<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             227 * 1024);
        if (e != cudaSuccess) return e;
        return cudaFuncSetAttribute(k_qgt_tile_adj<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    });
    if (attr != cudaSuccess) return VD_ERR_CUDA;
    QgtGeom<R> G;
    G.ny = d->ny; G.nx = d->nx; G.T = d->tile; G.n = d->tile - 2; G.ntiles = d->ntiles;
    G.scheme = d->time_scheme; G.hasK = d->has_Kdiffus;
    G.dx = (R)d->dx; G.dy = (R)d->dy; G.dt = (R)d->dt; G.g = (R)d->g; G.K = (R)d->Kdiffus;
    const size_t TT = (size_t)d->tile * d->tile;
    R* tout = (R*)work;
    R* scratch = tout + (size_t)d->ntiles * TT;
    const size_t smem = qgt_ad_smem<R>(d->tile);
    if (!adjoint) {
        k_qgt_tile_tl<R><<<(unsigned)d->ntiles, 256, smem, st>>>(
            G, d->origins, d->f_tile, d->c_tile, d->mask, (const R*)d->S, (const R*)d->lap, (const R*)d->weights,
            (const R*)d->mdt, (const R*)h0, (const R*)hb, (const R*)x, nstep, scratch, tout);
        VD_LAUNCH_CHECK();
        k_qgt_blend<R><<<dim3((unsigned)((d->nx + 127) / 128), (unsigned)d->ny), 128, 0, st>>>(
            G, d->origins, tout, (const R*)d->wsum, nullptr, (R*)out);
    } else {
        R* traj = scratch + (size_t)d->ntiles * QGT_AD_FIELDS * TT;
        k_qgt_tile_adj<R><<<(unsigned)d->ntiles, 256, smem, st>>>(
            G, d->origins, d->f_tile, d->c_tile, d->mask, (const R*)d->S, (const R*)d->lap, (const R*)d->weights,
            (const R*)d->wsum, (const R*)d->mdt, (const R*)h0, (const R*)hb, (const R*)x, nstep, scratch, traj,
            tout);
        VD_LAUNCH_CHECK();
        k_qgt_blend<R><<<dim3((unsigned)((d->nx + 127) / 128), (unsigned)d->ny), 128, 0, st>>>(
            G, d->origins, tout, nullptr, nullptr, (R*)out);
    }
    VD_LAUNCH_CHECK();
    return VD_OK;
}

}  // namespace vd

extern "C" size_t vd_qgt_shared_bytes(int tile, int dtype)
{
    return dtype == VD_F64 ? vd::qgt_smem<double>(tile) : vd::qgt_smem<float>(tile);
}

extern "C" size_t vd_qgt_workspace_bytes(const vd_qgt_desc* d)
{
    if (!d) return 0;
    return (size_t)d->ntiles * d->tile * d->tile * (d->dtype == VD_F64 ? 8 : 4);
}

extern "C" vd_status vd_qgt_step(const vd_qgt_desc* d, const void* h0, const void* hb, int nstep, void* h1,
                                 void* work, size_t work_bytes, void* stream)
{
    if (!d || !h0 || !hb || !h1 || !work || nstep < 0) return VD_ERR_ARG;
    if (d->tile < 8 || d->tile > d->ny || d->tile > d->nx || d->ntiles < 1 || !d->origins || !d->f_tile ||
        !d->c_tile || !d->mask || !d->S || !d->lap || !d->weights || !d->wsum)
        return VD_ERR_ARG;
    if (d->time_scheme != VD_EULER && d->time_scheme != VD_RK2) return VD_ERR_ARG;
    if (d->dtype != VD_F32 && d->dtype != VD_F64) return VD_ERR_ARG;
    if (work_bytes < vd_qgt_workspace_bytes(d)) return VD_ERR_WORKSPACE;
    if (vd_qgt_shared_bytes(d->tile, d->dtype) > 227 * 1024) return VD_ERR_UNSUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;
    return d->dtype == VD_F64 ? vd::qgt_run<double>(d, h0, hb, nstep, h1, work, st)
                              : vd::qgt_run<float>(d, h0, hb, nstep, h1, work, st);
}

extern "C" size_t vd_qgt_ad_workspace_bytes(const vd_qgt_desc* d, int nstep, int adjoint)
{
    if (!d || nstep < 0) return 0;
    return vd::qgt_ad_elems(d, nstep, adjoint) * (d->dtype == VD_F64 ? 8 : 4);
}

static vd_status qgt_ad_entry(const vd_qgt_desc* d, int adjoint, const void* x, const void* h0, const void* hb,
                              int nstep, void* out, void* work, size_t work_bytes, void* stream)
{
    if (!d || !x || !h0 || !hb || !out || !work || nstep < 0) return VD_ERR_ARG;
    if (d->tile < 8 || d->tile > d->ny || d->tile > d->nx || d->ntiles < 1 || !d->origins || !d->f_tile ||
        !d->c_tile || !d->mask || !d->S || !d->lap || !d->weights || !d->wsum)
        return VD_ERR_ARG;
    if (d->time_scheme != VD_EULER && d->time_scheme != VD_RK2) return VD_ERR_ARG;
    if (d->dtype != VD_F32 && d->dtype != VD_F64) return VD_ERR_ARG;
    if (work_bytes < vd_qgt_ad_workspace_bytes(d, nstep, adjoint)) return VD_ERR_WORKSPACE;
    const size_t smem = d->dtype == VD_F64 ? vd::qgt_ad_smem<double>(d->tile) : vd::qgt_ad_smem<float>(d->tile);
    if (smem > 227 * 1024) return VD_ERR_UNSUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;
    return d->dtype == VD_F64 ? vd::qgt_run_ad<double>(d, adjoint, x, h0, hb, nstep, out, work, st)
                              : vd::qgt_run_ad<float>(d, adjoint, x, h0, hb, nstep, out, work, st);
}

extern "C" vd_status vd_qgt_step_tgl(const vd_qgt_desc* d, const void* dh0, const void* h0, const void* hb,
                                     int nstep, void* dh1, void* work, size_t work_bytes, void* stream)
{
    return qgt_ad_entry(d, 0, dh0, h0, hb, nstep, dh1, work, work_bytes, stream);
}

extern "C" vd_status vd_qgt_step_adj(const vd_qgt_desc* d, const void* adh1, const void* h0, const void* hb,
                                     int nstep, void* adh0, void* work, size_t work_bytes, void* stream)
{
    return qgt_ad_entry(d, 1, adh1, h0, hb, nstep, adh0, work, work_bytes, stream);
}
