// Tangent linear and adjoint of the QG 1.5-layer model with passive tracers
// (Qgm_trac.step_tgl / step_adj, mapping/models/model_qg1l/jqgm.py:2141-2151:
// jax.jvp / jax.vjp of step with respect to X0 = [SSH, tracers...]; the
// boundary fields Xb are not differentiated).
//
// The state is stacked plane-major, var = [P][B][ny][nx] with P = 1 + ntrac
// planes (plane 0 the PV q of every window, planes 1.. the tracers), so the
// PV planes of all windows are one contiguous batch for the QG plan's h2pv,
// h2uv and Helmholtz inversion. The time scheme is the plan's Butcher table
// (Euler, rk2; rk4 the classical extension): a stage tendency of every plane
// is one kernel, the stage inputs and the update are linear combinations.
// Derivative rules are jax's for the forward's jnp.where / abs: where(u < 0,
// 0, u) passes the derivative for u >= 0, where(u > 0, 0, u) for u <= 0, a
// NaN-guarded value passes none, |w| has derivative sign(w), values
// overwritten with constants pass none.
//
// The adjoint runs the forward once keeping every stage input (h_s, var_s)
// of every step in the workspace, then sweeps back recomputing the stage
// velocities; every transposed stencil (upwind advection, diffusion, the
// velocity stencils, the PV stencil, the open boundaries) is a gather, so
// there are no atomics and the result is deterministic.
#include "vd_internal.cuh"
#include "vd_qgtrac.cuh"

#include <initializer_list>
#include <utility>

namespace vd {

struct TtGeom {
    int ny, nx, B, P;
    long long fs;
    double cu, cv, cx, cy, gf, gfc2, idx2, idy2;
    double Kx, Ky;      // PV diffusion (hasK)
    int hasK;
    double Ktx, Kty;    // tracer diffusion (hasKt)
    int hasKt;
    double rx, ry;      // open-boundary ratios 0.5 dt / dx, 0.5 dt / dy
    int obc, advect_pv;
    const int8_t* mask;
    const void* beta;   // T[ny][nx] (full-grid aligned) or nullptr
    const void* W;      // T[ny][nx] relaxation weights
};

static const dim3 kTT(32, 8);
static inline dim3 ttgrid(int ny, int nx, int nz) { return dim3((nx + 31) / 32, (ny + 7) / 8, nz); }

template <typename T>
struct TtCross {
    T c, e1, e2, w1, w2, n1, n2, s1, s2;
    __device__ __forceinline__ void load(const T* a, long long o, int nx)
    {
        c = a[o];
        e1 = a[o + 1]; e2 = a[o + 2]; w1 = a[o - 1]; w2 = a[o - 2];
        n1 = a[o + nx]; n2 = a[o + 2 * nx]; s1 = a[o - nx]; s2 = a[o - 2 * nx];
    }
    __device__ __forceinline__ T px() const { return T(2) * e1 + T(3) * c - T(6) * w1 + w2; }
    __device__ __forceinline__ T mx() const { return e2 - T(6) * e1 + T(3) * c + T(2) * w1; }
    __device__ __forceinline__ T py() const { return T(2) * n1 + T(3) * c - T(6) * s1 + s2; }
    __device__ __forceinline__ T my() const { return n2 - T(6) * n1 + T(3) * c + T(2) * s1; }
    __device__ __forceinline__ T lx() const { return e1 + w1 - T(2) * c; }
    __device__ __forceinline__ T ly() const { return n1 + s1 - T(2) * c; }
};

__device__ __forceinline__ bool tt_core(int ny, int nx, int j, int i)
{
    return j >= 2 && j <= ny - 3 && i >= 2 && i <= nx - 3;
}

// raw geostrophic velocities at (j, i) of one window's h; ue / ve: inside
// the range the forward assigns (u on rows 1..ny-2, columns >= 1; v on rows
// >= 1, columns 1..nx-2)
template <typename T>
__device__ __forceinline__ void tt_uv_raw(const TtGeom& G, const T* h, int j, int i, T& u, T& v, bool& ue,
                                          bool& ve)
{
    const int nx = G.nx;
    const long long o = (long long)j * nx + i;
    ue = j >= 1 && j <= G.ny - 2 && i >= 1;
    ve = j >= 1 && i >= 1 && i <= nx - 2;
    u = ue ? T(G.cu) * (h[o + nx - 1] + h[o + nx] - h[o - nx] - h[o - nx - 1]) : T(0);
    v = ve ? T(G.cv) * (h[o + 1] + h[o - nx + 1] - h[o - nx - 1] - h[o - 1]) : T(0);
}

// raw PV of an interior point (no guard)
template <typename T>
__device__ __forceinline__ T tt_pv_raw(const TtGeom& G, const T* h, long long o)
{
    const int nx = G.nx;
    const T c = h[o];
    return T(G.gf) * ((h[o + nx] + h[o - nx] - T(2) * c) * T(G.idy2) + (h[o + 1] + h[o - 1] - T(2) * c) * T(G.idx2)) -
           T(G.gfc2) * c;
}

// whether the plane's tendency at (j, i) is live (before the NaN guard):
// PV on class-3 points, tracers on the core rows / columns off land
__device__ __forceinline__ bool tt_live(const TtGeom& G, int plane, int j, int i)
{
    const int8_t m = G.mask[(long long)j * G.nx + i];
    return plane == 0 ? m == 3 : (tt_core(G.ny, G.nx, j, i) && m != 0);
}

// raw tendency of one plane at a live point (u, v: the window's guarded
// velocities; a: the plane)
template <typename T>
__device__ __forceinline__ T tt_rhs_raw(const TtGeom& G, int plane, const T* u, const T* v, const T* a, int j, int i)
{
    const int nx = G.nx;
    const long long o = (long long)j * nx + i;
    TtCross<T> s;
    s.load(a, o, nx);
    T r = T(0);
    if (plane > 0 || G.advect_pv) {
        const T uT = T(0.5) * (u[o] + u[o + 1]), vT = T(0.5) * (v[o] + v[o + nx]);
        const T up = uT < T(0) ? T(0) : uT, um = uT > T(0) ? T(0) : uT;
        const T vp = vT < T(0) ? T(0) : vT, vm = vT > T(0) ? T(0) : vT;
        const T cx = T(G.cx), cy = T(G.cy);
        r = -up * cx * s.px() + um * cx * s.mx() - vp * cy * s.py() + vm * cy * s.my();
        if (plane == 0 && G.beta) r -= ((const T*)G.beta)[o] * (v[o] + v[o + nx]) / T(2);
    }
    if (plane == 0 && G.hasK) r += T(G.Kx) * s.lx() + T(G.Ky) * s.ly();
    if (plane > 0 && G.hasKt) r += T(G.Ktx) * s.lx() + T(G.Kty) * s.ly();
    return r;
}

// ---------------------------------------------------------------------------
// forward and tangent kernels
// ---------------------------------------------------------------------------

// h = h0 + mdt, hb = hb + mdt; tracer planes of var / varb from c0 / cb
// ([B][ntrac]) with land zeroed; optional tangent tracer planes likewise
template <typename T>
__global__ void k_tt_prep(TtGeom G, const T* __restrict__ h0, const T* __restrict__ hb, const T* __restrict__ mdt,
                          const T* __restrict__ c0, const T* __restrict__ cb, const T* __restrict__ dc0,
                          T* __restrict__ h, T* __restrict__ hbm, T* __restrict__ var, T* __restrict__ varb,
                          T* __restrict__ dvar)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const long long p = (long long)j * G.nx + i, o = b * G.fs + p;
    const T m = mdt ? mdt[p] : T(0);
    h[o] = h0[o] + m;
    hbm[o] = hb[o] + m;
    const bool land = G.mask[p] == 0;
    const int nt = G.P - 1;
    for (int t = 0; t < nt; ++t) {
        const long long oi = ((long long)b * nt + t) * G.fs + p;
        const long long ov = ((long long)(1 + t) * G.B + b) * G.fs + p;
        var[ov] = land ? T(0) : c0[oi];
        varb[ov] = land ? T(0) : cb[oi];
        if (dvar) dvar[ov] = land ? T(0) : dc0[oi];
    }
}

// tangent of the initial PV: the interior stencil of dh on class-3 points
// whose raw PV is a number (plane 0 of dvar)
template <typename T>
__global__ void k_tt_h2pv_tl(TtGeom G, const T* __restrict__ h, const T* __restrict__ dh, T* __restrict__ dq)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const long long p = (long long)j * G.nx + i, o = b * G.fs + p;
    T r = T(0);
    if (G.mask[p] == 3 && !isnan(tt_pv_raw(G, h + b * G.fs, p))) r = tt_pv_raw(G, dh + b * G.fs, p);
    dq[o] = r;
}

// du, dv = h2uv(dh) where the raw velocities of h are numbers
template <typename T>
__global__ void k_tt_uv_tl(TtGeom G, const T* __restrict__ h, const T* __restrict__ dh, T* __restrict__ du,
                           T* __restrict__ dv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const long long o = b * G.fs + (long long)j * G.nx + i;
    T u, v, du_, dv_;
    bool ue, ve;
    tt_uv_raw(G, h + b * G.fs, j, i, u, v, ue, ve);
    tt_uv_raw(G, dh + b * G.fs, j, i, du_, dv_, ue, ve);
    du[o] = isnan(u) ? T(0) : du_;
    dv[o] = isnan(v) ? T(0) : dv_;
}

// stage tendency of every plane (z = plane * B + window) and, when dk is
// given, its tangent
template <typename T>
__global__ void k_tt_stage(TtGeom G, const T* __restrict__ u, const T* __restrict__ v, const T* __restrict__ du,
                           const T* __restrict__ dv, const T* __restrict__ var, const T* __restrict__ dvar,
                           T* __restrict__ k, T* __restrict__ dk)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const int b = z % G.B, plane = z / G.B;
    const long long p = (long long)j * G.nx + i, o = z * G.fs + p, ob = b * G.fs;
    T r = T(0), dr = T(0);
    if (tt_live(G, plane, j, i)) {
        const T* a = var + z * G.fs;
        const T raw = tt_rhs_raw(G, plane, u + ob, v + ob, a, j, i);
        if (!isnan(raw)) {
            r = raw;
            if (dk) {
                const int nx = G.nx;
                const T *uu = u + ob, *vv = v + ob, *duu = du + ob, *dvv = dv + ob;
                TtCross<T> s, d;
                s.load(a, p, nx);
                d.load(dvar + z * G.fs, p, nx);
                if (plane > 0 || G.advect_pv) {
                    const T uT = T(0.5) * (uu[p] + uu[p + 1]), vT = T(0.5) * (vv[p] + vv[p + nx]);
                    const T duT = T(0.5) * (duu[p] + duu[p + 1]), dvT = T(0.5) * (dvv[p] + dvv[p + nx]);
                    const T up = uT < T(0) ? T(0) : uT, um = uT > T(0) ? T(0) : uT;
                    const T vp = vT < T(0) ? T(0) : vT, vm = vT > T(0) ? T(0) : vT;
                    const T dup = uT < T(0) ? T(0) : duT, dum = uT > T(0) ? T(0) : duT;
                    const T dvp = vT < T(0) ? T(0) : dvT, dvm = vT > T(0) ? T(0) : dvT;
                    const T cx = T(G.cx), cy = T(G.cy);
                    dr = -dup * cx * s.px() + dum * cx * s.mx() - dvp * cy * s.py() + dvm * cy * s.my() -
                         up * cx * d.px() + um * cx * d.mx() - vp * cy * d.py() + vm * cy * d.my();
                    if (plane == 0 && G.beta) dr -= ((const T*)G.beta)[p] * (dvv[p] + dvv[p + nx]) / T(2);
                }
                if (plane == 0 && G.hasK) dr += T(G.Kx) * d.lx() + T(G.Ky) * d.ly();
                if (plane > 0 && G.hasKt) dr += T(G.Ktx) * d.lx() + T(G.Kty) * d.ly();
            }
        }
    }
    k[o] = r;
    if (dk) dk[o] = dr;
}

// out = base + sum_t c[t] x[t] (base nullable: 0), elementwise; out may be base
template <typename T>
struct TtLin {
    const T* x[4];
    T c[4];
    int n;
};

template <typename T>
__global__ void k_tt_lin(long long n, const T* base, TtLin<T> L, T* out)
{
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    T acc = base ? base[o] : T(0);
#pragma unroll
    for (int t = 0; t < 4; ++t)
        if (t < L.n) acc += L.c[t] * L.x[t][o];
    out[o] = acc;
}

template <typename T>
__device__ __forceinline__ T tt_sign(T w) { return w > T(0) ? T(1) : (w < T(0) ? T(-1) : T(0)); }

// boundary update of the tracer planes (jqgm.py:1957-2006) and its tangent,
// in place on var1 / dvar1 (each point reads var1 only at itself); u, v the
// start-of-step velocities, var0 the start-of-step state
template <typename T>
__global__ void k_tt_bc(TtGeom G, const T* __restrict__ u, const T* __restrict__ v, const T* __restrict__ du,
                        const T* __restrict__ dv, const T* __restrict__ var0, const T* __restrict__ dvar0,
                        const T* __restrict__ varb, T* __restrict__ var1, T* __restrict__ dvar1)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = G.B + blockIdx.z;        // tracer planes only
    if (i >= G.nx || j >= G.ny) return;
    const int ny = G.ny, nx = G.nx, b = z % G.B;
    const long long p = (long long)j * nx + i, o = z * G.fs + p, ob = b * G.fs;
    const T *a = var0 + z * G.fs, *bb = varb + z * G.fs;
    const T* da = dvar0 ? dvar0 + z * G.fs : nullptr;
    const T *uu = u + ob, *vv = v + ob;
    const T* duu = du ? du + ob : nullptr;
    const T* dvv = dv ? dv + ob : nullptr;
    T x = var1[o], dx = dvar1 ? dvar1[o] : T(0);
    const bool in_i = i >= 1 && i <= nx - 2, in_j = j >= 1 && j <= ny - 2;
    if (G.obc) {
        // rows 0 / ny-1 with w = v one point inside, columns 0 / nx-1 with u;
        // s0 = the neighbour inward, "up" = whether the value upstream is b
        int kind = -1;
        T w = T(0), dw = T(0), r = T(0);
        long long inner = 0;
        if (j == 0 && in_i) { kind = 0; w = vv[nx + i]; dw = dvv ? dvv[nx + i] : T(0); r = T(G.ry); inner = p + nx; }
        else if (j == ny - 1 && in_i) { kind = 1; w = vv[p]; dw = dvv ? dvv[p] : T(0); r = T(G.ry); inner = p - nx; }
        else if (i == 0 && in_j) { kind = 0; w = uu[p + 1]; dw = duu ? duu[p + 1] : T(0); r = T(G.rx); inner = p + 1; }
        else if (i == nx - 1 && in_j) { kind = 1; w = uu[p]; dw = duu ? duu[p] : T(0); r = T(G.rx); inner = p - 1; }
        if (kind >= 0) {
            const T aw = w < T(0) ? -w : w, sg = tt_sign(w);
            const T r1 = r * (w + aw), r2 = r * (w - aw);
            const T d1 = r * (dw + sg * dw), d2 = r * (dw - sg * dw);
            const T dap = da ? da[p] : T(0), dai = da ? da[inner] : T(0);
            if (kind == 0) {
                // x = a - (r1 (a - b) + r2 (a_in - a))
                x = a[p] - (r1 * (a[p] - bb[p]) + r2 * (a[inner] - a[p]));
                dx = dap - (d1 * (a[p] - bb[p]) + r1 * dap + d2 * (a[inner] - a[p]) + r2 * (dai - dap));
            } else {
                // x = a - (r1 (a - a_in) + r2 (b - a))
                x = a[p] - (r1 * (a[p] - a[inner]) + r2 * (bb[p] - a[p]));
                dx = dap - (d1 * (a[p] - a[inner]) + r1 * (dap - dai) + d2 * (bb[p] - a[p]) - r2 * dap);
            }
        }
    } else if (G.mask[p] == 1 || G.mask[p] == 2) {
        x = bb[p];
        dx = T(0);
    }
    if (in_i && in_j) {
        const T W = ((const T*)G.W)[p];
        x = W * bb[p] + (T(1) - W) * x;
        dx = (T(1) - W) * dx;
    }
    var1[o] = x;
    if (dvar1) dvar1[o] = dx;
}

// tangent outputs: dh1 (land 0), tracer planes back to [B][ntrac] (land 0)
template <typename T>
__global__ void k_tt_final(TtGeom G, const T* __restrict__ dh, const T* __restrict__ dvar, T* __restrict__ dh1,
                           T* __restrict__ dc1)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const long long p = (long long)j * G.nx + i, o = b * G.fs + p;
    const bool land = G.mask[p] == 0;
    dh1[o] = land ? T(0) : dh[o];
    const int nt = G.P - 1;
    for (int t = 0; t < nt; ++t)
        dc1[((long long)b * nt + t) * G.fs + p] = land ? T(0) : dvar[((long long)(1 + t) * G.B + b) * G.fs + p];
}

// ---------------------------------------------------------------------------
// adjoint kernels
// ---------------------------------------------------------------------------

// incoming adjoints: NaN -> 0, land -> 0; PV plane 0
template <typename T>
__global__ void k_ta_prep(TtGeom G, const T* __restrict__ adh1, const T* __restrict__ adc1, T* __restrict__ adh,
                          T* __restrict__ advar)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const long long p = (long long)j * G.nx + i, o = b * G.fs + p;
    const bool land = G.mask[p] == 0;
    const T x = adh1[o];
    adh[o] = (land || isnan(x)) ? T(0) : x;
    advar[o] = T(0);
    const int nt = G.P - 1;
    for (int t = 0; t < nt; ++t) {
        const T y = adc1[((long long)b * nt + t) * G.fs + p];
        advar[((long long)(1 + t) * G.B + b) * G.fs + p] = (land || isnan(y)) ? T(0) : y;
    }
}

// coefficients of the open-boundary formula at an edge point (kind 0: the
// upstream value is b at the edge; kind 1: at the inner neighbour)
template <typename T>
struct TtEdge {
    int kind;            // -1: not an edge point of the update
    long long inner;     // the inward neighbour
    T w, r;              // velocity one point inside, ratio
};

template <typename T>
__device__ __forceinline__ TtEdge<T> tt_edge(const TtGeom& G, const T* uu, const T* vv, int j, int i)
{
    const int ny = G.ny, nx = G.nx;
    const long long p = (long long)j * nx + i;
    const bool in_i = i >= 1 && i <= nx - 2, in_j = j >= 1 && j <= ny - 2;
    TtEdge<T> e;
    e.kind = -1; e.inner = 0; e.w = T(0); e.r = T(0);
    if (!G.obc) return e;
    if (j == 0 && in_i) { e.kind = 0; e.w = vv[nx + i]; e.r = T(G.ry); e.inner = p + nx; }
    else if (j == ny - 1 && in_i) { e.kind = 1; e.w = vv[p]; e.r = T(G.ry); e.inner = p - nx; }
    else if (i == 0 && in_j) { e.kind = 0; e.w = uu[p + 1]; e.r = T(G.rx); e.inner = p + 1; }
    else if (i == nx - 1 && in_j) { e.kind = 1; e.w = uu[p]; e.r = T(G.rx); e.inner = p - 1; }
    return e;
}

// adjoint of the boundary update for every plane (z = plane * B + window):
// adpre = adjoint of var1 before the update, ad0 = adjoint of var0 (gathered
// from the edge formulas that read it); the PV plane passes through
template <typename T>
__global__ void k_ta_bc(TtGeom G, const T* __restrict__ u, const T* __restrict__ v, const T* __restrict__ var0,
                        const T* __restrict__ adx, T* __restrict__ adpre, T* __restrict__ ad0)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const int ny = G.ny, nx = G.nx, b = z % G.B, plane = z / G.B;
    const long long p = (long long)j * nx + i, o = z * G.fs + p, ob = b * G.fs;
    const T* g = adx + z * G.fs;
    if (plane == 0) {
        adpre[o] = g[p];
        ad0[o] = T(0);
        return;
    }
    const T *uu = u + ob, *vv = v + ob;
    const bool in_i = i >= 1 && i <= nx - 2, in_j = j >= 1 && j <= ny - 2;
    T x = g[p];
    if (in_i && in_j) x = (T(1) - ((const T*)G.W)[p]) * x;
    T a0 = T(0);
    if (G.obc) {
        const TtEdge<T> e = tt_edge(G, uu, vv, j, i);
        if (e.kind >= 0) {
            const T aw = e.w < T(0) ? -e.w : e.w;
            const T r1 = e.r * (e.w + aw), r2 = e.r * (e.w - aw);
            a0 += g[p] * (T(1) - r1 + r2);
            x = T(0);
        }
        // this point as the inward neighbour of an edge point
        const int nb[4][2] = {{0, i}, {ny - 1, i}, {j, 0}, {j, nx - 1}};
        const bool near[4] = {j == 1 && in_i, j == ny - 2 && in_i, i == 1 && in_j, i == nx - 2 && in_j};
        for (int s = 0; s < 4; ++s) {
            if (!near[s]) continue;
            const TtEdge<T> f = tt_edge(G, uu, vv, nb[s][0], nb[s][1]);
            if (f.kind < 0) continue;
            const long long q = (long long)nb[s][0] * nx + nb[s][1];
            const T aw = f.w < T(0) ? -f.w : f.w;
            const T r1 = f.r * (f.w + aw), r2 = f.r * (f.w - aw);
            a0 += g[q] * (f.kind == 0 ? -r2 : r1);
        }
    } else if (G.mask[p] == 1 || G.mask[p] == 2) {
        x = T(0);
    }
    adpre[o] = x;
    ad0[o] = a0;
}

// velocity adjoint of the open boundaries (summed over the tracers), per
// window: v on rows 1 and ny-1, u on columns 1 and nx-1
template <typename T>
__global__ void k_ta_bc_uv(TtGeom G, const T* __restrict__ u, const T* __restrict__ v, const T* __restrict__ var0,
                           const T* __restrict__ varb, const T* __restrict__ adx, T* __restrict__ adub,
                           T* __restrict__ advb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const int ny = G.ny, nx = G.nx;
    const long long p = (long long)j * nx + i, o = b * G.fs + p, ob = b * G.fs;
    const T *uu = u + ob, *vv = v + ob;
    T au = T(0), av = T(0);
    if (G.obc && G.P > 1) {
        const bool in_i = i >= 1 && i <= nx - 2, in_j = j >= 1 && j <= ny - 2;
        // (edge point, this velocity is its w): row 0 <- v(1, i), row ny-1 <-
        // v(ny-1, i), column 0 <- u(j, 1), column nx-1 <- u(j, nx-1)
        const int ne = 4;
        const int ej[ne] = {0, ny - 1, j, j}, ei[ne] = {i, i, 0, nx - 1};
        const bool on[ne] = {j == 1 && in_i, j == ny - 1 && in_i, i == 1 && in_j, i == nx - 1 && in_j};
        for (int s = 0; s < ne; ++s) {
            if (!on[s]) continue;
            const TtEdge<T> e = tt_edge(G, uu, vv, ej[s], ei[s]);
            if (e.kind < 0) continue;
            const long long q = (long long)ej[s] * nx + ei[s];
            const T sg = tt_sign(e.w);
            T acc = T(0);
            for (int t = 1; t < G.P; ++t) {
                const long long zo = ((long long)t * G.B + b) * G.fs;
                const T *a = var0 + zo, *bb = varb + zo;
                const T gq = adx[zo + q];
                T gr1, gr2;
                if (e.kind == 0) {
                    gr1 = -gq * (a[q] - bb[q]);
                    gr2 = -gq * (a[e.inner] - a[q]);
                } else {
                    gr1 = -gq * (a[q] - a[e.inner]);
                    gr2 = -gq * (bb[q] - a[q]);
                }
                acc += e.r * (gr1 * (T(1) + sg) + gr2 * (T(1) - sg));
            }
            if (s < 2) av += acc; else au += acc;
        }
    }
    adub[o] = au;
    advb[o] = av;
}

// stage adjoint, part 1: the live adjoint input of every plane (a) and the
// adjoints of the T-point velocities uT, vT summed over the planes
template <typename T>
__global__ void k_ta_stage_a(TtGeom G, const T* __restrict__ u, const T* __restrict__ v, const T* __restrict__ var,
                             const T* __restrict__ adk, T* __restrict__ a, T* __restrict__ aduT,
                             T* __restrict__ advT)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const int nx = G.nx;
    const long long p = (long long)j * nx + i, ob = b * G.fs;
    const T *uu = u + ob, *vv = v + ob;
    T su = T(0), sv = T(0);
    for (int plane = 0; plane < G.P; ++plane) {
        const long long zo = ((long long)plane * G.B + b) * G.fs;
        T ae = T(0);
        if (tt_live(G, plane, j, i) && !isnan(tt_rhs_raw(G, plane, uu, vv, var + zo, j, i))) {
            ae = adk[zo + p];
            if (plane > 0 || G.advect_pv) {
                TtCross<T> s;
                s.load(var + zo, p, nx);
                const T uT = T(0.5) * (uu[p] + uu[p + 1]), vT = T(0.5) * (vv[p] + vv[p + nx]);
                const T cx = T(G.cx), cy = T(G.cy);
                su += (uT < T(0) ? T(0) : -cx * s.px() * ae) + (uT > T(0) ? T(0) : cx * s.mx() * ae);
                sv += (vT < T(0) ? T(0) : -cy * s.py() * ae) + (vT > T(0) ? T(0) : cy * s.my() * ae);
            }
        }
        a[zo + p] = ae;
    }
    aduT[ob + p] = su;
    advT[ob + p] = sv;
}

// stage adjoint, part 2: the state adjoint of every plane (gather of the
// transposed upwind and diffusion stencils) and, per window, the adjoints of
// the guarded velocities u, v (T-point averages, the beta term, the
// boundary update's velocities at the first stage)
template <typename T>
__global__ void k_ta_stage_b(TtGeom G, const T* __restrict__ u, const T* __restrict__ v, const T* __restrict__ h,
                             const T* __restrict__ a, const T* __restrict__ aduT, const T* __restrict__ advT,
                             const T* __restrict__ adub, const T* __restrict__ advb, T* __restrict__ advs,
                             T* __restrict__ adu, T* __restrict__ adv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const int ny = G.ny, nx = G.nx;
    const long long p = (long long)j * nx + i, ob = b * G.fs;
    const T *uu = u + ob, *vv = v + ob;
    const T cx = T(G.cx), cy = T(G.cy);
    for (int plane = 0; plane < G.P; ++plane) {
        const long long zo = ((long long)plane * G.B + b) * G.fs;
        const T* ap = a + zo;
        const bool advect = plane > 0 || G.advect_pv;
        const T kx = plane == 0 ? (G.hasK ? T(G.Kx) : T(0)) : (G.hasKt ? T(G.Ktx) : T(0));
        const T ky = plane == 0 ? (G.hasK ? T(G.Ky) : T(0)) : (G.hasKt ? T(G.Kty) : T(0));
        T acc = T(0);
        // x neighbours e = (j, i - d) contribute the coefficient of a[e + d]
        for (int d = -2; d <= 2; ++d) {
            const int ei = i - d;
            if (!tt_core(ny, nx, j, ei)) continue;
            const long long e = (long long)j * nx + ei;
            const T ae = ap[e];
            if (ae == T(0)) continue;
            T up = T(0), um = T(0), vp = T(0), vm = T(0);
            if (advect) {
                const T uT = T(0.5) * (uu[e] + uu[e + 1]);
                up = uT < T(0) ? T(0) : uT;
                um = uT > T(0) ? T(0) : uT;
                if (d == 0) {
                    const T vT = T(0.5) * (vv[e] + vv[e + nx]);
                    vp = vT < T(0) ? T(0) : vT;
                    vm = vT > T(0) ? T(0) : vT;
                }
            }
            T cf;
            switch (d) {
            case 2: cf = cx * um; break;
            case 1: cf = -T(2) * cx * up - T(6) * cx * um + kx; break;
            case 0: cf = -T(3) * cx * up + T(3) * cx * um - T(3) * cy * vp + T(3) * cy * vm - T(2) * kx - T(2) * ky; break;
            case -1: cf = T(6) * cx * up + T(2) * cx * um + kx; break;
            default: cf = -cx * up; break;
            }
            acc += cf * ae;
        }
        for (int d = -2; d <= 2; ++d) {
            if (d == 0) continue;
            const int ej = j - d;
            if (!tt_core(ny, nx, ej, i)) continue;
            const long long e = (long long)ej * nx + i;
            const T ae = ap[e];
            if (ae == T(0)) continue;
            T vp = T(0), vm = T(0);
            if (advect) {
                const T vT = T(0.5) * (vv[e] + vv[e + nx]);
                vp = vT < T(0) ? T(0) : vT;
                vm = vT > T(0) ? T(0) : vT;
            }
            T cf;
            switch (d) {
            case 2: cf = cy * vm; break;
            case 1: cf = -T(2) * cy * vp - T(6) * cy * vm + ky; break;
            case -1: cf = T(6) * cy * vp + T(2) * cy * vm + ky; break;
            default: cf = -cy * vp; break;
            }
            acc += cf * ae;
        }
        advs[zo + p] = acc;
    }
    T ru, rv;
    bool ue, ve;
    tt_uv_raw(G, h + ob, j, i, ru, rv, ue, ve);
    T au = T(0.5) * (aduT[ob + p] + (i >= 1 ? aduT[ob + p - 1] : T(0)));
    T av = T(0.5) * (advT[ob + p] + (j >= 1 ? advT[ob + p - nx] : T(0)));
    if (G.beta && G.advect_pv) {
        const T* be = (const T*)G.beta;
        const T* a0 = a + ob;            // plane 0 of this window
        av -= be[p] * a0[p] / T(2);
        if (j >= 1) av -= be[p - nx] * a0[p - nx] / T(2);
    }
    if (adub) au += adub[ob + p];
    if (advb) av += advb[ob + p];
    adu[ob + p] = (ue && !isnan(ru)) ? au : T(0);
    adv[ob + p] = (ve && !isnan(rv)) ? av : T(0);
}

template <typename T>
__device__ __forceinline__ T tt_at(const T* x, int ny, int nx, int j, int i)
{
    return (j >= 0 && j < ny && i >= 0 && i < nx) ? x[(long long)j * nx + i] : T(0);
}

// adh = h2uv^T (adu, adv)
template <typename T>
__global__ void k_ta_h2uv(TtGeom G, const T* __restrict__ adu, const T* __restrict__ adv, T* __restrict__ adh)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const int ny = G.ny, nx = G.nx;
    const long long ob = b * G.fs;
    const T *au = adu + ob, *av = adv + ob;
    adh[ob + (long long)j * nx + i] =
        T(G.cu) * (tt_at(au, ny, nx, j - 1, i + 1) + tt_at(au, ny, nx, j - 1, i) - tt_at(au, ny, nx, j + 1, i) -
                   tt_at(au, ny, nx, j + 1, i + 1)) +
        T(G.cv) * (tt_at(av, ny, nx, j, i - 1) + tt_at(av, ny, nx, j + 1, i - 1) - tt_at(av, ny, nx, j + 1, i + 1) -
                   tt_at(av, ny, nx, j, i + 1));
}

// adh += h2pv^T (adq) at the initial state h (class-3 interior points whose
// raw PV is a number)
template <typename T>
__global__ void k_ta_h2pv(TtGeom G, const T* __restrict__ h, const T* __restrict__ adq, T* __restrict__ adh)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const int ny = G.ny, nx = G.nx;
    const long long ob = b * G.fs;
    auto live = [&](int jj, int ii) -> T {
        if (jj < 1 || jj > ny - 2 || ii < 1 || ii > nx - 2) return T(0);
        const long long q = (long long)jj * nx + ii;
        if (G.mask[q] != 3 || isnan(tt_pv_raw(G, h + ob, q))) return T(0);
        return adq[ob + q];
    };
    const T gy = T(G.gf) * T(G.idy2), gx = T(G.gf) * T(G.idx2);
    const T s = gy * (live(j - 1, i) + live(j + 1, i)) + gx * (live(j, i - 1) + live(j, i + 1)) +
                (-T(2) * gy - T(2) * gx - T(G.gfc2)) * live(j, i);
    adh[ob + (long long)j * nx + i] += s;
}

// adjoint outputs: tracer planes back to [B][ntrac], land 0
template <typename T>
__global__ void k_ta_final(TtGeom G, const T* __restrict__ advar, T* __restrict__ adc0)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const long long p = (long long)j * G.nx + i;
    const bool land = G.mask[p] == 0;
    const int nt = G.P - 1;
    for (int t = 0; t < nt; ++t)
        adc0[((long long)b * nt + t) * G.fs + p] = land ? T(0) : advar[((long long)(1 + t) * G.B + b) * G.fs + p];
}

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------

static TtGeom tt_geom(const vd_qg1l_plan* p, const vd_qgtrac_desc* d, int B)
{
    TtGeom G;
    const QGGeom& Q = p->geom;
    G.ny = Q.ny; G.nx = Q.nx; G.B = B; G.P = 1 + d->ntrac; G.fs = Q.fs;
    G.cu = Q.cu; G.cv = Q.cv; G.cx = Q.cx; G.cy = Q.cy; G.gf = Q.gf; G.gfc2 = Q.gfc2;
    G.idx2 = Q.idx2; G.idy2 = Q.idy2;
    G.Kx = Q.Kx; G.Ky = Q.Ky; G.hasK = Q.hasK;
    G.hasKt = d->has_Kdiffus_trac;
    G.Ktx = d->has_Kdiffus_trac ? d->Kdiffus_trac / (p->d.dx * p->d.dx) : 0.0;
    G.Kty = d->has_Kdiffus_trac ? d->Kdiffus_trac / (p->d.dy * p->d.dy) : 0.0;
    G.rx = 0.5 * p->d.dt / p->d.dx;
    G.ry = 0.5 * p->d.dt / p->d.dy;
    G.obc = d->bc_obc;
    G.advect_pv = d->advect_pv;
    G.mask = p->d_mask;
    G.beta = p->d_beta;
    G.W = d->wbc;
    return G;
}

struct TtBufs {
    // state
    void *h, *hbm, *var, *varb, *vs, *hs, *u0, *v0, *u, *v, *k, *var1, *hinit;
    // tangent
    void *dh, *dvar, *dvs, *dhs, *du0, *dv0, *du, *dv, *dk, *dvar1;
    // adjoint
    void *traj, *adh, *advar, *adpre, *ad0, *adk, *acc, *advs, *a, *aduT, *advT, *adu, *adv, *adub, *advb, *adhs,
        *tmp;
    void* pv2h_ws;
    size_t pv2h_bytes;
};

// mode 0: tangent, 1: adjoint
static size_t tt_layout(const vd_qg1l_plan* p, const vd_qgtrac_desc* d, int B, int nstep, int mode, TtBufs* tb,
                        char* base, size_t cap)
{
    *tb = TtBufs{};
    const size_t F = size_t(p->geom.fs) * elem_size(p->d.dtype);
    const size_t BF = size_t(B) * F, PF = size_t(1 + d->ntrac) * BF;
    const size_t S = (size_t)p->nstage;
    const size_t pv2h = spec_bytes(p, B) + 2 * 256;
    Arena ar{base, cap, 0};
    size_t need = 0;
    auto take = [&](void** s, size_t bytes) {
        *s = base ? ar.take(bytes) : nullptr;
        need += (bytes + 255) & ~size_t(255);
    };
    for (void** s : {&tb->h, &tb->hbm, &tb->hs, &tb->u0, &tb->v0, &tb->u, &tb->v, &tb->hinit}) take(s, BF);
    for (void** s : {&tb->var, &tb->varb, &tb->vs, &tb->var1}) take(s, PF);
    take(&tb->k, S * PF);
    if (mode == 0) {
        for (void** s : {&tb->dh, &tb->dhs, &tb->du0, &tb->dv0, &tb->du, &tb->dv}) take(s, BF);
        for (void** s : {&tb->dvar, &tb->dvs, &tb->dvar1}) take(s, PF);
        take(&tb->dk, S * PF);
    } else {
        take(&tb->traj, (size_t)nstep * S * (BF + PF));
        for (void** s : {&tb->adh, &tb->aduT, &tb->advT, &tb->adu, &tb->adv, &tb->adub, &tb->advb, &tb->adhs,
                         &tb->tmp})
            take(s, BF);
        for (void** s : {&tb->advar, &tb->adpre, &tb->ad0, &tb->acc, &tb->advs, &tb->a}) take(s, PF);
        take(&tb->adk, S * PF);
    }
    take(&tb->pv2h_ws, pv2h);
    tb->pv2h_bytes = pv2h;
    return need + 256;
}

template <typename T>
static void tt_lin(long long n, const T* base, std::initializer_list<std::pair<const T*, double>> terms, T* out,
                   cudaStream_t st)
{
    TtLin<T> L{};
    L.n = 0;
    for (auto& t : terms) {
        if (t.second == 0.0) continue;
        L.x[L.n] = t.first;
        L.c[L.n] = (T)t.second;
        ++L.n;
    }
    k_tt_lin<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, base, L, out);
}

template <typename T>
static int tt_run(const vd_qg1l_plan* p, const vd_qgtrac_desc* d, int B, int mode, const T* h0, const T* c0,
                  const T* hb, const T* cb, const T* xh, const T* xc, int nstep, T* outh, T* outc, char* work,
                  size_t work_bytes, cudaStream_t st)
{
    TtBufs tb;
    const size_t need = tt_layout(p, d, B, nstep, mode, &tb, work, work_bytes);
    if (need > work_bytes) return VD_ERR_WORKSPACE;
    const TtGeom G = tt_geom(p, d, B);
    const int ny = G.ny, nx = G.nx, P = G.P, S = p->nstage;
    const long long BF = (long long)B * G.fs, PF = (long long)P * BF;
    T *h = (T*)tb.h, *hbm = (T*)tb.hbm, *var = (T*)tb.var, *varb = (T*)tb.varb, *vs = (T*)tb.vs, *hs = (T*)tb.hs;
    T *u0 = (T*)tb.u0, *v0 = (T*)tb.v0, *u = (T*)tb.u, *v = (T*)tb.v, *k = (T*)tb.k, *var1 = (T*)tb.var1;
    T* hinit = (T*)tb.hinit;
    const T* mdt = (const T*)d->mdt;
    const T* qb = varb;        // plane 0 of varb: the boundary PV
    int rc;
    auto ck = [&]() { return cudaGetLastError() == cudaSuccess ? VD_OK : VD_ERR_CUDA; };
    auto pv2h = [&](const T* q, const T* hbv, const T* qbv, T* out) {
        return vd_qg1l_pv2h(p, B, q, hbv, qbv, out, tb.pv2h_ws, tb.pv2h_bytes, st);
    };

    T *dh = nullptr, *dvar = nullptr, *dvs = nullptr, *dhs = nullptr, *du0 = nullptr, *dv0 = nullptr;
    T *du = nullptr, *dv = nullptr, *dk = nullptr, *dvar1 = nullptr;
    if (mode == 0) {
        dh = (T*)tb.dh; dvar = (T*)tb.dvar; dvs = (T*)tb.dvs; dhs = (T*)tb.dhs; du0 = (T*)tb.du0;
        dv0 = (T*)tb.dv0; du = (T*)tb.du; dv = (T*)tb.dv; dk = (T*)tb.dk; dvar1 = (T*)tb.dvar1;
    }
    k_tt_prep<T><<<ttgrid(ny, nx, B), kTT, 0, st>>>(G, h0, hb, mdt, c0, cb, mode == 0 ? xc : nullptr, h, hbm, var,
                                                     varb, dvar);
    if ((rc = ck())) return rc;
    if ((rc = vd_qg1l_h2pv(p, B, h, hbm, var, st))) return rc;
    if ((rc = vd_qg1l_h2pv(p, B, hbm, hbm, varb, st))) return rc;
    VD_CUDA_TRY(cudaMemcpyAsync(hinit, h, BF * sizeof(T), cudaMemcpyDeviceToDevice, st));
    if (mode == 0) {
        VD_CUDA_TRY(cudaMemcpyAsync(dh, xh, BF * sizeof(T), cudaMemcpyDeviceToDevice, st));
        k_tt_h2pv_tl<T><<<ttgrid(ny, nx, B), kTT, 0, st>>>(G, h, dh, dvar);
        if ((rc = ck())) return rc;
    }
    T* traj = mode == 1 ? (T*)tb.traj : nullptr;

    // ---- forward (and tangent) sweep
    for (int n = 0; n < nstep; ++n) {
        for (int s = 0; s < S; ++s) {
            const T *hsv = h, *vsv = var, *dhsv = dh, *dvsv = dvar;
            if (s > 0) {
                TtLin<T> L{};
                L.n = 0;
                for (int t = 0; t < s; ++t)
                    if (p->A[s][t] != 0.0) { L.x[L.n] = k + t * PF; L.c[L.n] = (T)p->A[s][t]; ++L.n; }
                k_tt_lin<T><<<(unsigned)((PF + 255) / 256), 256, 0, st>>>(PF, var, L, vs);
                if ((rc = ck())) return rc;
                if ((rc = pv2h(vs, hbm, qb, hs))) return rc;
                hsv = hs;
                vsv = vs;
                if (mode == 0) {
                    TtLin<T> D{};
                    D.n = 0;
                    for (int t = 0; t < s; ++t)
                        if (p->A[s][t] != 0.0) { D.x[D.n] = dk + t * PF; D.c[D.n] = (T)p->A[s][t]; ++D.n; }
                    k_tt_lin<T><<<(unsigned)((PF + 255) / 256), 256, 0, st>>>(PF, dvar, D, dvs);
                    if ((rc = ck())) return rc;
                    if ((rc = pv2h(dvs, nullptr, nullptr, dhs))) return rc;
                    dhsv = dhs;
                    dvsv = dvs;
                }
            }
            if (traj) {
                T* slot = traj + ((size_t)n * S + s) * (BF + PF);
                VD_CUDA_TRY(cudaMemcpyAsync(slot, hsv, BF * sizeof(T), cudaMemcpyDeviceToDevice, st));
                VD_CUDA_TRY(cudaMemcpyAsync(slot + BF, vsv, PF * sizeof(T), cudaMemcpyDeviceToDevice, st));
            }
            T* uu = s == 0 ? u0 : u;
            T* vv = s == 0 ? v0 : v;
            if ((rc = vd_qg1l_h2uv(p, B, hsv, uu, vv, st))) return rc;
            T* duu = nullptr;
            T* dvv = nullptr;
            if (mode == 0) {
                duu = s == 0 ? du0 : du;
                dvv = s == 0 ? dv0 : dv;
                k_tt_uv_tl<T><<<ttgrid(ny, nx, B), kTT, 0, st>>>(G, hsv, dhsv, duu, dvv);
                if ((rc = ck())) return rc;
            }
            k_tt_stage<T><<<ttgrid(ny, nx, P * B), kTT, 0, st>>>(G, uu, vv, duu, dvv, vsv, dvsv, k + s * PF,
                                                                  mode == 0 ? dk + s * PF : nullptr);
            if ((rc = ck())) return rc;
        }
        TtLin<T> L{};
        L.n = 0;
        for (int s = 0; s < S; ++s)
            if (p->b[s] != 0.0) { L.x[L.n] = k + s * PF; L.c[L.n] = (T)p->b[s]; ++L.n; }
        k_tt_lin<T><<<(unsigned)((PF + 255) / 256), 256, 0, st>>>(PF, var, L, var1);
        if ((rc = ck())) return rc;
        if ((rc = pv2h(var1, hbm, qb, h))) return rc;
        if (mode == 0) {
            TtLin<T> D{};
            D.n = 0;
            for (int s = 0; s < S; ++s)
                if (p->b[s] != 0.0) { D.x[D.n] = dk + s * PF; D.c[D.n] = (T)p->b[s]; ++D.n; }
            k_tt_lin<T><<<(unsigned)((PF + 255) / 256), 256, 0, st>>>(PF, dvar, D, dvar1);
            if ((rc = ck())) return rc;
            if ((rc = pv2h(dvar1, nullptr, nullptr, dh))) return rc;
        }
        if (P > 1) {
            k_tt_bc<T><<<ttgrid(ny, nx, (P - 1) * B), kTT, 0, st>>>(G, u0, v0, du0, dv0, var, dvar, varb, var1,
                                                                     mode == 0 ? dvar1 : nullptr);
            if ((rc = ck())) return rc;
        }
        T* t = var; var = var1; var1 = t;
        if (mode == 0) { t = dvar; dvar = dvar1; dvar1 = t; }
    }
    if (mode == 0) {
        k_tt_final<T><<<ttgrid(ny, nx, B), kTT, 0, st>>>(G, dh, dvar, outh, outc);
        return ck();
    }

    // ---- adjoint sweep
    T *adh = (T*)tb.adh, *advar = (T*)tb.advar, *adpre = (T*)tb.adpre, *ad0 = (T*)tb.ad0, *adk = (T*)tb.adk;
    T *acc = (T*)tb.acc, *advs = (T*)tb.advs, *a = (T*)tb.a, *aduT = (T*)tb.aduT, *advT = (T*)tb.advT;
    T *adu = (T*)tb.adu, *adv = (T*)tb.adv, *adub = (T*)tb.adub, *advb = (T*)tb.advb, *adhs = (T*)tb.adhs;
    T* tmp = (T*)tb.tmp;
    k_ta_prep<T><<<ttgrid(ny, nx, B), kTT, 0, st>>>(G, xh, xc, adh, advar);
    if ((rc = ck())) return rc;
    for (int n = nstep - 1; n >= 0; --n) {
        const T* h0s = traj + (size_t)n * S * (BF + PF);
        const T* var0s = h0s + BF;
        if ((rc = vd_qg1l_h2uv(p, B, h0s, u0, v0, st))) return rc;
        k_ta_bc<T><<<ttgrid(ny, nx, P * B), kTT, 0, st>>>(G, u0, v0, var0s, advar, adpre, ad0);
        if ((rc = ck())) return rc;
        k_ta_bc_uv<T><<<ttgrid(ny, nx, B), kTT, 0, st>>>(G, u0, v0, var0s, varb, advar, adub, advb);
        if ((rc = ck())) return rc;
        // h1 = pv2h(var1[0]): the inversion is symmetric
        if ((rc = pv2h(adh, nullptr, nullptr, tmp))) return rc;
        tt_lin<T>(BF, adpre, {{tmp, 1.0}}, adpre, st);
        for (int s = 0; s < S; ++s) tt_lin<T>(PF, nullptr, {{adpre, p->b[s]}}, adk + s * PF, st);
        tt_lin<T>(PF, adpre, {{ad0, 1.0}}, acc, st);
        if ((rc = ck())) return rc;
        for (int s = S - 1; s >= 0; --s) {
            const T* hsv = traj + ((size_t)n * S + s) * (BF + PF);
            const T* vsv = hsv + BF;
            T* uu = s == 0 ? u0 : u;
            T* vv = s == 0 ? v0 : v;
            if (s > 0 && (rc = vd_qg1l_h2uv(p, B, hsv, uu, vv, st))) return rc;
            k_ta_stage_a<T><<<ttgrid(ny, nx, B), kTT, 0, st>>>(G, uu, vv, vsv, adk + s * PF, a, aduT, advT);
            if ((rc = ck())) return rc;
            k_ta_stage_b<T><<<ttgrid(ny, nx, B), kTT, 0, st>>>(G, uu, vv, hsv, a, aduT, advT,
                                                                s == 0 ? adub : nullptr, s == 0 ? advb : nullptr,
                                                                advs, adu, adv);
            if ((rc = ck())) return rc;
            k_ta_h2uv<T><<<ttgrid(ny, nx, B), kTT, 0, st>>>(G, adu, adv, s == 0 ? adh : adhs);
            if ((rc = ck())) return rc;
            if (s > 0) {
                if ((rc = pv2h(adhs, nullptr, nullptr, tmp))) return rc;
                tt_lin<T>(BF, advs, {{tmp, 1.0}}, advs, st);
                for (int t = 0; t < s; ++t)
                    if (p->A[s][t] != 0.0) tt_lin<T>(PF, adk + t * PF, {{advs, p->A[s][t]}}, adk + t * PF, st);
            }
            tt_lin<T>(PF, acc, {{advs, 1.0}}, acc, st);
            if ((rc = ck())) return rc;
        }
        T* t = advar; advar = acc; acc = t;
    }
    k_ta_h2pv<T><<<ttgrid(ny, nx, B), kTT, 0, st>>>(G, hinit, advar, adh);
    if ((rc = ck())) return rc;
    VD_CUDA_TRY(cudaMemcpyAsync(outh, adh, BF * sizeof(T), cudaMemcpyDeviceToDevice, st));
    if (P > 1) {
        k_ta_final<T><<<ttgrid(ny, nx, B), kTT, 0, st>>>(G, advar, outc);
        if ((rc = ck())) return rc;
    }
    return VD_OK;
}

static bool tt_desc_ok(const vd_qg1l_plan* p, const vd_qgtrac_desc* d)
{
    if (!p || !d || d->ntrac < 0) return false;
    if (d->time_scheme != VD_EULER && d->time_scheme != VD_RK2 && d->time_scheme != VD_RK4) return false;
    if (p->d.time_scheme != d->time_scheme) return false;
    if (p->d_fB) return false;
    if (d->ntrac > 0 && !d->wbc) return false;
    return true;
}

}  // namespace vd

using namespace vd;

extern "C" size_t vd_qgtrac_ad_workspace_bytes(const vd_qg1l_plan* p, const vd_qgtrac_desc* d, int batch, int nstep,
                                               int adjoint)
{
    if (!tt_desc_ok(p, d) || batch <= 0 || nstep < 0) return 0;
    TtBufs tb;
    return tt_layout(p, d, batch, nstep, adjoint ? 1 : 0, &tb, nullptr, 0);
}

static vd_status tt_entry(const vd_qg1l_plan* p, const vd_qgtrac_desc* d, int batch, int mode, const void* h0,
                          const void* c0, const void* hb, const void* cb, const void* xh, const void* xc, int nstep,
                          void* outh, void* outc, void* work, size_t work_bytes, void* stream)
{
    if (!tt_desc_ok(p, d) || batch <= 0 || nstep < 0 || !h0 || !hb || !xh || !outh || !work) return VD_ERR_ARG;
    if ((long long)batch * (1 + d->ntrac) > 65535) return VD_ERR_UNSUPPORTED;   // grid z
    if (d->ntrac > 0 && (!c0 || !cb || !xc || !outc)) return VD_ERR_ARG;
    if (work_bytes < vd_qgtrac_ad_workspace_bytes(p, d, batch, nstep, mode)) return VD_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    if (p->d.dtype == VD_F32)
        return tt_run<float>(p, d, batch, mode, (const float*)h0, (const float*)c0, (const float*)hb,
                             (const float*)cb, (const float*)xh, (const float*)xc, nstep, (float*)outh,
                             (float*)outc, (char*)work, work_bytes, st);
    return tt_run<double>(p, d, batch, mode, (const double*)h0, (const double*)c0, (const double*)hb,
                          (const double*)cb, (const double*)xh, (const double*)xc, nstep, (double*)outh,
                          (double*)outc, (char*)work, work_bytes, st);
}

extern "C" vd_status vd_qgtrac_step_tgl(const vd_qg1l_plan* p, const vd_qgtrac_desc* d, int batch, const void* h0,
                                        const void* c0, const void* hb, const void* cb, const void* dh0,
                                        const void* dc0, int nstep, void* dh1, void* dc1, void* work,
                                        size_t work_bytes, void* stream)
{
    return tt_entry(p, d, batch, 0, h0, c0, hb, cb, dh0, dc0, nstep, dh1, dc1, work, work_bytes, stream);
}

extern "C" vd_status vd_qgtrac_step_adj(const vd_qg1l_plan* p, const vd_qgtrac_desc* d, int batch, const void* h0,
                                        const void* c0, const void* hb, const void* cb, const void* adh1,
                                        const void* adc1, int nstep, void* adh0, void* adc0, void* work,
                                        size_t work_bytes, void* stream)
{
    return tt_entry(p, d, batch, 1, h0, c0, hb, cb, adh1, adc1, nstep, adh0, adc0, work, work_bytes, stream);
}
