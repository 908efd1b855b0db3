// QG 1.5-layer model kernels: SSH->PV, the fused Runge-Kutta stage (geostrophic
// velocities, 3rd-order upwind PV advection, beta, bathymetry and diffusion
// terms, masks, stage combination), its tangent-linear and adjoint, and the
// host-side drivers that chain them with the Helmholtz solve.
//
// Reference: mapping/models/model_qg1l/jqgm.py, class Qgm — h2uv 238-262,
// h2pv 264-293, rhs 321-375, adv 377-396, euler/rk2/rk3 398-477,
// one_step 480-503, step 517-557, step_tgl/step_adj 559-569.
//
// Masks. mask==3 ("M3") marks the points where the PV tendency is computed
// (jqgm.py:372-373 zero it on mask 1/2 and on land); they lie in rows/cols
// 2..n-4 and have no land within two cells (jqgm.py:196-211). Consequently the
// NaN guards on u, v (jqgm.py:259-260) never act on a value that reaches an M3
// tendency unless the caller's SSH holds NaN away from the land of the mask;
// the adjoint kernels rely on this and omit the u, v guard.
#include "vd_internal.cuh"
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cstring>
#include <mutex>

namespace vd {

template <typename T> __device__ __forceinline__ T guard0(T x) { return isnan(x) ? T(0) : x; }

// Plans without diffusion, bathymetry and beta run the stage kernels
// compiled without those terms.
static inline bool plain_geom(const QGGeom& G) { return !G.hasK && !G.fB && !G.beta; }

// Round-to-nearest add / subtract that the compiler neither contracts nor
// reassociates (the error-free transformations below rely on it).
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// Compensated state update of float32 plans. The prognostic PV of a step is
// held as an unevaluated pair q + q_lo (q_lo a few ulps of q at most). The
// last stage of a step adds its increment with TwoSum (Knuth), folds the
// rounding error into q_lo and renormalises with Fast2Sum, so the 2880
// roundings of a 30-day window do not accumulate in the trajectory. Earlier
// stages evaluate q_n + (increment + q_lo) in plain arithmetic: their values
// only feed the tendency of the next stage.
template <typename T>
__device__ __forceinline__ void comp_update(T base, T inc, T& q_out, T& lo)
{
    const T s = add_rn(base, inc);
    const T bb = sub_rn(s, base);
    const T e = add_rn(sub_rn(base, sub_rn(s, bb)), sub_rn(inc, bb));
    const T l2 = add_rn(lo, e);
    const T hi = add_rn(s, l2);
    lo = sub_rn(l2, sub_rn(hi, s));
    q_out = hi;
}

template <typename T>
struct Cross {
    T c, e1, e2, w1, w2, n1, n2, s1, s2;   // (j,i), (j,i+1), (j,i+2), (j,i-1), ... (j-1,i), (j-2,i)
    __device__ __forceinline__ void load(const T* __restrict__ p, int nx) {
        c = p[0]; e1 = p[1]; e2 = p[2]; w1 = p[-1]; w2 = p[-2];
        n1 = p[nx]; n2 = p[2 * nx]; s1 = p[-nx]; s2 = p[-2 * nx];
    }
    __device__ __forceinline__ void add(const Cross& o) {
        c += o.c; e1 += o.e1; e2 += o.e2; w1 += o.w1; w2 += o.w2;
        n1 += o.n1; n2 += o.n2; s1 += o.s1; s2 += o.s2;
    }
    __device__ __forceinline__ T Dpx() const { return T(2) * e1 + T(3) * c - T(6) * w1 + w2; }
    __device__ __forceinline__ T Dmx() const { return e2 - T(6) * e1 + T(3) * c + T(2) * w1; }
    __device__ __forceinline__ T Dpy() const { return T(2) * n1 + T(3) * c - T(6) * s1 + s2; }
    __device__ __forceinline__ T Dmy() const { return n2 - T(6) * n1 + T(3) * c + T(2) * s1; }
};

// Staggered velocities around T point (j,i): u(j,i), u(j,i+1), v(j,i), v(j+1,i)
template <typename T>
struct Vel {
    T u0, u1, v0, v1;
    // from the SSH at rows j-1 (s), j, j+1 (n) and columns i-1 (w), i, i+1 (e)
    __device__ __forceinline__ void set(const QGGeom& G, T hs_w, T hs_c, T hs_e, T h_w, T h_e, T hn_w, T hn_c,
                                        T hn_e) {
        const T cu = T(G.cu), cv = T(G.cv);
        u0 = cu * (hn_w + hn_c - hs_c - hs_w);
        u1 = cu * (hn_c + hn_e - hs_e - hs_c);
        v0 = cv * (h_e + hs_e - hs_w - h_w);
        v1 = cv * (hn_e + h_e - h_w - hn_w);
    }
    __device__ __forceinline__ void load(const QGGeom& G, const T* __restrict__ hc) {
        const int nx = G.nx;
        set(G, hc[-nx - 1], hc[-nx], hc[-nx + 1], hc[-1], hc[1], hc[nx - 1], hc[nx], hc[nx + 1]);
    }
};

// Raw PV tendency at an M3 point from velocities and PV crosses. MAYK false:
// the caller knows the plan has no diffusion.
template <typename T, bool MAYK = true>
__device__ __forceinline__ T tendency(const QGGeom& G, const Vel<T>& V, const Cross<T>& qa,
                                      const Cross<T>& q, T beta)
{
    const T uT = T(0.5) * (V.u0 + V.u1);
    const T vT = T(0.5) * (V.v0 + V.v1);
    const T up = uT < T(0) ? T(0) : uT;
    const T um = uT > T(0) ? T(0) : uT;
    const T vp = vT < T(0) ? T(0) : vT;
    const T vm = vT > T(0) ? T(0) : vT;
    const T cx = T(G.cx), cy = T(G.cy);
    T r = -up * cx * qa.Dpx() + um * cx * qa.Dmx() - vp * cy * qa.Dpy() + vm * cy * qa.Dmy();
    r -= beta * ((V.v0 + V.v1) / T(2));
    if (MAYK && G.hasK)
        r += T(G.Kx) * (q.e1 + q.w1 - T(2) * q.c) + T(G.Ky) * (q.n1 + q.s1 - T(2) * q.c);
    return r;
}

// ---------------------------------------------------------------------------
// h2pv (jqgm.py:264-293). Fields f >= ntan0 are tangents: their ring value is
// 0 (hb fixed) and their NaN guard follows the primal field f - ntan0.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T lap_helm(const QGGeom& G, const T* __restrict__ hc)
{
    const int nx = G.nx;
    const T c = hc[0];
    return T(G.gf) * ((hc[nx] + hc[-nx] - T(2) * c) * T(G.idy2) +
                      (hc[1] + hc[-1] - T(2) * c) * T(G.idx2)) - T(G.gfc2) * c;
}

template <typename T>
__device__ __forceinline__ double lap_helm_f64(const QGGeom& G, const T* __restrict__ hc)
{
    const int nx = G.nx;
    const double c = hc[0];
    return G.gf * (((double)hc[nx] + (double)hc[-nx] - 2.0 * c) * G.idy2 +
                   ((double)hc[1] + (double)hc[-1] - 2.0 * c) * G.idx2) - G.gfc2 * c;
}

// With qlo != nullptr (float32 plans) the PV is evaluated in float64 from
// the float32 SSH and returned as the pair q + qlo of the compensated state.
template <typename T>
__global__ void k_h2pv(QGGeom G, int nf, int ntan0, const T* __restrict__ h,
                       const T* __restrict__ hb, T* __restrict__ q, T* __restrict__ qlo)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int f = blockIdx.z;
    if (i >= G.nx || j >= G.ny || f >= nf) return;
    const long long o = f * G.fs + (long long)j * G.nx + i;
    const int m = G.mask[j * G.nx + i];
    if (qlo) {
        double val = 0.0;
        if (m == 3) {
            val = lap_helm_f64<T>(G, h + o);
            const double prim = f >= ntan0 ? lap_helm_f64<T>(G, h + o - ntan0 * G.fs) : val;
            if (isnan(prim)) val = 0.0;
        } else if (m != 0 && f < ntan0) {
            val = -G.gfc2 * (double)hb[o];
        }
        const T hi = (T)val;
        q[o] = hi;
        qlo[o] = (T)(val - (double)hi);
        return;
    }
    T val = T(0);
    if (m == 3) {
        val = lap_helm<T>(G, h + o);
        if (f >= ntan0) {
            const T prim = lap_helm<T>(G, h + o - ntan0 * G.fs);
            if (isnan(prim)) val = T(0);
        } else {
            val = guard0(val);
        }
    } else if (m != 0 && f < ntan0) {
        val = -T(G.gfc2) * hb[o];
    }
    q[o] = val;
}

// adh += (d h2pv / d h)^T adq, masked to M3 points whose primal PV was finite.
template <typename T>
__global__ void k_h2pv_adj(QGGeom G, int nf, const T* __restrict__ h, const T* __restrict__ adq,
                           T* __restrict__ adh)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int f = blockIdx.z;
    if (i >= G.nx || j >= G.ny || f >= nf) return;
    const long long o = f * G.fs + (long long)j * G.nx + i;
    const T gfy = T(G.gf) * T(G.idy2), gfx = T(G.gf) * T(G.idx2);
    const int di[5] = {0, 1, -1, 0, 0};
    const int dj[5] = {0, 0, 0, 1, -1};
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const int jj = j + dj[k], ii = i + di[k];
        if (jj < 0 || jj >= G.ny || ii < 0 || ii >= G.nx) continue;
        if (G.mask[jj * G.nx + ii] != 3) continue;
        const long long po = f * G.fs + (long long)jj * G.nx + ii;
        if (isnan(lap_helm<T>(G, h + po))) continue;
        const T coef = (k == 0) ? (-T(2) * gfy - T(2) * gfx - T(G.gfc2)) : (k < 3 ? gfx : gfy);
        acc += coef * adq[po];
    }
    adh[o] += acc;
}

// ---------------------------------------------------------------------------
// Forward stage: k = rhs(h2uv(hs), qs); qout = qbase + sum_i cin[i] k_i + cself k
// ---------------------------------------------------------------------------
template <typename T>
struct StageIn {
    const T* k[4];
    T c[4];
    int nk;
};

// One point's PV tendency, loading its own stencil (M3 points only). PLAIN:
// the plan has no diffusion, bathymetry or beta term.
template <typename T, bool PLAIN = false>
__device__ __forceinline__ T stage_point(const QGGeom& G, const T* __restrict__ hs, const T* __restrict__ qs,
                                         long long o, long long go)
{
    Vel<T> V;
    V.load(G, hs + o);
    V.u0 = guard0(V.u0); V.u1 = guard0(V.u1); V.v0 = guard0(V.v0); V.v1 = guard0(V.v1);
    Cross<T> q;
    q.load(qs + o, G.nx);
    Cross<T> qa = q;
    if (!PLAIN && G.fB) { Cross<T> b; b.load((const T*)G.fB + go, G.nx); qa.add(b); }
    const T beta = (!PLAIN && G.beta) ? ((const T*)G.beta)[go] : T(0);
    return guard0(tendency<T, !PLAIN>(G, V, qa, q, beta));
}

// The PV crosses of the points (j, i) and (j+1, i) from one column of six
// rows (j-2 .. j+3) and the four x-neighbours of rows j and j+1.
template <typename T>
__device__ __forceinline__ void cross_pair(const T* __restrict__ p, int nx, Cross<T>& a, Cross<T>& b)
{
    const T c_2 = p[-2 * nx], c_1 = p[-nx], c0 = p[0], c1 = p[nx], c2 = p[2 * nx], c3 = p[3 * nx];
    a.c = c0; a.e1 = p[1]; a.e2 = p[2]; a.w1 = p[-1]; a.w2 = p[-2];
    a.n1 = c1; a.n2 = c2; a.s1 = c_1; a.s2 = c_2;
    const T* r = p + nx;
    b.c = c1; b.e1 = r[1]; b.e2 = r[2]; b.w1 = r[-1]; b.w2 = r[-2];
    b.n1 = c2; b.n2 = c3; b.s1 = c0; b.s2 = c_1;
}

// Forward stage: k = rhs(h2uv(hs), qs); qout = qbase + sum_i cin[i] k_i + cself k.
// Each thread takes the points (j, i) and (j+1, i) (blocks of 32 x 4 threads
// cover 32 x 8 points): when both are M3 points their SSH and PV stencils
// overlap, so the pair is loaded once (12 + 14 values instead of 16 + 18) and
// each point then runs the same arithmetic as a single point.
template <typename T, bool PLAIN>
__global__ void k_stage_fwd(QGGeom G, int nf, const T* __restrict__ hs, const T* __restrict__ qs,
                            const T* __restrict__ qbase, StageIn<T> kin, T cself,
                            T* __restrict__ kout, T* __restrict__ qout, T* __restrict__ qlo, int last)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * (2 * blockDim.y) + 2 * threadIdx.y;
    const int f = blockIdx.z;
    if (i >= G.nx || j >= G.ny || f >= nf) return;
    const bool two = j + 1 < G.ny;
    const int nx = G.nx;
    const long long go = (long long)j * nx + i, o = f * G.fs + go;
    const int m0 = G.mask[go], m1 = two ? G.mask[go + nx] : 0;
    T r[2] = {T(0), T(0)};
    if (m0 == 3 && m1 == 3) {
        const T* h = hs + o;
        const T s_w = h[-nx - 1], s_c = h[-nx], s_e = h[-nx + 1];
        const T m_w = h[-1], m_c = h[0], m_e = h[1];
        const T n_w = h[nx - 1], n_c = h[nx], n_e = h[nx + 1];
        const T t_w = h[2 * nx - 1], t_c = h[2 * nx], t_e = h[2 * nx + 1];
        Vel<T> V[2];
        V[0].set(G, s_w, s_c, s_e, m_w, m_e, n_w, n_c, n_e);
        V[1].set(G, m_w, m_c, m_e, n_w, n_e, t_w, t_c, t_e);
        Cross<T> q[2], qa[2];
        cross_pair(qs + o, nx, q[0], q[1]);
        qa[0] = q[0];
        qa[1] = q[1];
        if (!PLAIN && G.fB) {
            Cross<T> b[2];
            cross_pair((const T*)G.fB + go, nx, b[0], b[1]);
            qa[0].add(b[0]);
            qa[1].add(b[1]);
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            V[u].u0 = guard0(V[u].u0); V[u].u1 = guard0(V[u].u1);
            V[u].v0 = guard0(V[u].v0); V[u].v1 = guard0(V[u].v1);
            const T beta = (!PLAIN && G.beta) ? ((const T*)G.beta)[go + u * nx] : T(0);
            r[u] = guard0(tendency<T, !PLAIN>(G, V[u], qa[u], q[u], beta));
        }
    } else {
        if (m0 == 3) r[0] = stage_point<T, PLAIN>(G, hs, qs, o, go);
        if (m1 == 3) r[1] = stage_point<T, PLAIN>(G, hs, qs, o + nx, go + nx);
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        if (u == 1 && !two) break;
        const long long ou = o + u * nx;
        if (qlo) {
            T inc = cself * r[u];
#pragma unroll
            for (int t = 0; t < 4; ++t)
                if (t < kin.nk) inc += kin.c[t] * kin.k[t][ou];
            T lo = qlo[ou];
            if (last) {
                T qo;
                comp_update(qbase[ou], inc, qo, lo);
                qout[ou] = qo;
                qlo[ou] = lo;
            } else {
                qout[ou] = qbase[ou] + (inc + lo);
            }
        } else {
            T acc = qbase[ou];
#pragma unroll
            for (int t = 0; t < 4; ++t)
                if (t < kin.nk) acc += kin.c[t] * kin.k[t][ou];
            acc += cself * r[u];
            qout[ou] = acc;
        }
        if (kout) kout[ou] = r[u];
    }
}

// Tangent stage on dual arrays: fields [0, B) primal, [B, 2B) tangent.
template <typename T>
__global__ void k_stage_tl(QGGeom G, int B, const T* __restrict__ hs, const T* __restrict__ qs,
                           const T* __restrict__ qbase, StageIn<T> kin, T cself,
                           T* __restrict__ kout, T* __restrict__ qout, T* __restrict__ qlo, int last)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int f = blockIdx.z;
    if (i >= G.nx || j >= G.ny || f >= B) return;
    const long long o = f * G.fs + (long long)j * G.nx + i;
    const long long od = o + B * G.fs;
    const long long go = (long long)j * G.nx + i;
    T r = T(0), dr = T(0);
    if (G.mask[go] == 3) {
        Vel<T> V, dV;
        V.load(G, hs + o);
        dV.load(G, hs + od);
        if (isnan(V.u0)) { V.u0 = T(0); dV.u0 = T(0); }
        if (isnan(V.u1)) { V.u1 = T(0); dV.u1 = T(0); }
        if (isnan(V.v0)) { V.v0 = T(0); dV.v0 = T(0); }
        if (isnan(V.v1)) { V.v1 = T(0); dV.v1 = T(0); }
        Cross<T> q, dq;
        q.load(qs + o, G.nx);
        dq.load(qs + od, G.nx);
        Cross<T> qa = q;
        if (G.fB) { Cross<T> b; b.load((const T*)G.fB + go, G.nx); qa.add(b); }
        const T beta = G.beta ? ((const T*)G.beta)[go] : T(0);
        const T raw = tendency<T>(G, V, qa, q, beta);
        if (!isnan(raw)) {
            r = raw;
            const T uT = T(0.5) * (V.u0 + V.u1), vT = T(0.5) * (V.v0 + V.v1);
            const T duT = T(0.5) * (dV.u0 + dV.u1), dvT = T(0.5) * (dV.v0 + dV.v1);
            const T up = uT < T(0) ? T(0) : uT, um = uT > T(0) ? T(0) : uT;
            const T vp = vT < T(0) ? T(0) : vT, vm = vT > T(0) ? T(0) : vT;
            const T dup = uT < T(0) ? T(0) : duT, dum = uT > T(0) ? T(0) : duT;
            const T dvp = vT < T(0) ? T(0) : dvT, dvm = vT > T(0) ? T(0) : dvT;
            const T cx = T(G.cx), cy = T(G.cy);
            dr = -dup * cx * qa.Dpx() + dum * cx * qa.Dmx() - dvp * cy * qa.Dpy() + dvm * cy * qa.Dmy()
                 - up * cx * dq.Dpx() + um * cx * dq.Dmx() - vp * cy * dq.Dpy() + vm * cy * dq.Dmy();
            dr -= beta * ((dV.v0 + dV.v1) / T(2));
            if (G.hasK)
                dr += T(G.Kx) * (dq.e1 + dq.w1 - T(2) * dq.c) + T(G.Ky) * (dq.n1 + dq.s1 - T(2) * dq.c);
        }
    }
    if (qlo) {
        T inc = cself * r, dinc = cself * dr;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            if (t >= kin.nk) break;
            inc += kin.c[t] * kin.k[t][o];
            dinc += kin.c[t] * kin.k[t][od];
        }
        T lo = qlo[o], dlo = qlo[od];
        if (last) {
            T qo, dqo;
            comp_update(qbase[o], inc, qo, lo);
            comp_update(qbase[od], dinc, dqo, dlo);
            qout[o] = qo; qout[od] = dqo;
            qlo[o] = lo; qlo[od] = dlo;
        } else {
            qout[o] = qbase[o] + (inc + lo);
            qout[od] = qbase[od] + (dinc + dlo);
        }
    } else {
        T acc = qbase[o], dacc = qbase[od];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            if (t >= kin.nk) break;
            acc += kin.c[t] * kin.k[t][o];
            dacc += kin.c[t] * kin.k[t][od];
        }
        qout[o] = acc + cself * r;
        qout[od] = dacc + cself * dr;
    }
    if (kout) { kout[o] = r; kout[od] = dr; }
}

// ---------------------------------------------------------------------------
// Adjoint of one Runge-Kutta stage, in gather form, one 32x32 tile per CTA.
//   phase A (tile + 2-cell halo, per tendency point P): lk = sum_t c_t G_t(P)
//     (the stage-increment adjoint), the T-point velocities uT, vT and their
//     adjoints aut = lk * d(adv)/d(uT), avt = lk * d(adv)/d(vT) - beta*lk,
//     with jax's where-derivative convention (uT >= 0 feeds up, uT <= 0 um);
//   phase B (tile, every point X): the PV adjoint from the upwind and
//     diffusion stencils of the tendency points around X, and the SSH adjoint
//     through the T-point averages and h2uv (a Sobel-like 3x3 stencil of
//     aut / avt). With gacc.nk > 0 the PV adjoint is returned as
//     M3 * (sum of gacc + local), the final combination of a step.
// h (halo 3) and q (halo 4) are staged in shared memory once; the phase-A
// quantities never leave shared memory, and phase A stores lk times the split
// T-point velocities (lk u+, lk u-, lk v+, lk v-) so phase B's upwind
// transpose reads them without re-splitting.
//
// Two forms of staging. With grids whose rows are a multiple of 16 elements
// (and 16-byte aligned fields), one thread issues bulk tensor copies
// (cp.async.bulk.tensor, TMA) of the h and q tiles, q + bathymetry, the stage
// adjoints G_t, beta and the mask over the tile and its halos; the copies
// fill out-of-grid cells with zeros, so the threads run no index arithmetic,
// bounds checks or global loads for them. Otherwise the threads load the same
// tiles with bounds-checked loads. Tile x origins are i0 - 4 (fields) and
// i0 - 16 (the int8 mask), multiples of 16 bytes as a tiled copy requires.
// ---------------------------------------------------------------------------
constexpr int AT_Y = 32, AT_X = 32;                 // output tile
constexpr int AH_Y = AT_Y + 6, AH_X = AT_X + 8;     // h tile: rows j0-3.., columns i0-4..
constexpr int AQ_Y = AT_Y + 8, AQ_X = AT_X + 8;     // q tile: rows j0-4.., columns i0-4..
constexpr int AA_Y = AT_Y + 4, AA_X = AT_X + 4;     // phase-A region: rows j0-2.., columns i0-2..
constexpr int AG_Y = AA_Y, AG_X = AT_X + 8;         // G_t / beta tiles: rows j0-2.., columns i0-4..
constexpr int AM_Y = AA_Y, AM_X = AT_X + 32;        // mask tile (bytes): rows j0-2.., columns i0-16..

// Tensor maps of the staged tiles (fields [nf][ny][nx]; beta, bathymetry and
// mask [ny][nx]).
struct AdjMaps {
    CUtensorMap h, q, g[4], beta, fB, mask;
};

// Byte offsets of one CTA's shared regions (each 128-byte aligned, as tensor
// copies into shared memory require): h tile, q tile, q + bathymetry (only
// with a bathymetry term), the phase-A outputs (lk u+, lk u-, lk v+, lk v-,
// aut, avt, and lk with diffusion) which the staged G_t and beta tiles alias
// (they are read into registers before phase A writes), and the mask tile.
struct AdjLayout {
    uint32_t h, q, qa, out, beta, mask, total;
};

__host__ __device__ inline uint32_t adj_al(uint32_t x) { return (x + 127u) & ~127u; }

__host__ __device__ inline AdjLayout adj_layout(int esz, bool hasK, bool hasB, bool tma, int ng, bool hasBeta)
{
    AdjLayout L;
    uint32_t o = 0;
    L.h = o; o = adj_al(o + (uint32_t)(AH_Y * AH_X * esz));
    L.q = o; o = adj_al(o + (uint32_t)(AQ_Y * AQ_X * esz));
    L.qa = o; if (hasB) o = adj_al(o + (uint32_t)(AQ_Y * AQ_X * esz));
    L.out = o;
    const uint32_t nout = (uint32_t)((6 + (hasK ? 1 : 0)) * AA_Y * AA_X * esz);
    const uint32_t gtile = adj_al((uint32_t)(AG_Y * AG_X * esz));
    L.beta = o + (uint32_t)ng * gtile;
    const uint32_t nin = tma ? (uint32_t)ng * gtile + (hasBeta ? gtile : 0u) : 0u;
    o = adj_al(o + (nout > nin ? nout : nin));
    L.mask = o; if (tma) o = adj_al(o + (uint32_t)(AM_Y * AM_X));
    L.total = o;
    return L;
}

template <typename T>
struct AdjSmem {
    T (*h)[AH_X];
    T (*q)[AQ_X];
    T (*lup)[AA_X];
    T (*lum)[AA_X];
    T (*lvp)[AA_X];
    T (*lvm)[AA_X];
    T (*aut)[AA_X];
    T (*avt)[AA_X];
    T (*lk)[AA_X];           // only when the plan has diffusion
    T (*qa)[AQ_X];           // only with a bathymetry term
};

template <typename T>
__device__ __forceinline__ AdjSmem<T> adj_smem(unsigned char* raw, const AdjLayout& L, bool hasK, bool hasB)
{
    AdjSmem<T> S;
    S.h = reinterpret_cast<T(*)[AH_X]>(raw + L.h);
    S.q = reinterpret_cast<T(*)[AQ_X]>(raw + L.q);
    S.qa = hasB ? reinterpret_cast<T(*)[AQ_X]>(raw + L.qa) : nullptr;
    T* b = reinterpret_cast<T*>(raw + L.out);
    S.lup = reinterpret_cast<T(*)[AA_X]>(b); b += AA_Y * AA_X;
    S.lum = reinterpret_cast<T(*)[AA_X]>(b); b += AA_Y * AA_X;
    S.lvp = reinterpret_cast<T(*)[AA_X]>(b); b += AA_Y * AA_X;
    S.lvm = reinterpret_cast<T(*)[AA_X]>(b); b += AA_Y * AA_X;
    S.aut = reinterpret_cast<T(*)[AA_X]>(b); b += AA_Y * AA_X;
    S.avt = reinterpret_cast<T(*)[AA_X]>(b); b += AA_Y * AA_X;
    S.lk = hasK ? reinterpret_cast<T(*)[AA_X]>(b) : nullptr;
    return S;
}

__device__ int g_qg_tile_error = 0;

__device__ __forceinline__ uint64_t qg_gtimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool qg_mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for phase 0 of `bar`, at most `ns` nanoseconds of %globaltimer.
__device__ __forceinline__ bool qg_mbar_wait(uint32_t bar, uint64_t ns)
{
    if (qg_mbar_try(bar, 0)) return true;
    const uint64_t t0 = qg_gtimer();
    while (!qg_mbar_try(bar, 0))
        if (qg_gtimer() - t0 > ns) return false;
    return true;
}

__device__ __forceinline__ void tma_tile_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_tile_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// Four CTAs per SM in float32 (shared memory allows four), two in float64.
// PLAIN: the plan has no diffusion, bathymetry or beta term (compiled out).
// NG / NA >= 0: the numbers of stage adjoints and accumulated adjoints, known
// at compile time (the RK2 stages' forms); -1: read from gin / gacc.
template <typename T, bool TMA, bool PLAIN, int NG = -1, int NA = -1>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2)
k_adj_stage_fused(QGGeom G, int nf, const T* __restrict__ hs, const T* __restrict__ qs, StageIn<T> gin,
                  StageIn<T> gacc, T* __restrict__ adq_out, T* __restrict__ adh_out, const __grid_constant__ AdjMaps M)
{
    if constexpr (NG >= 0) gin.nk = NG;
    if constexpr (NA >= 0) gacc.nk = NA;
    extern __shared__ unsigned char smem_dyn[];
    __shared__ __align__(8) uint64_t tbar;
    unsigned char* smem_raw = (unsigned char*)(((uintptr_t)smem_dyn + 127) & ~(uintptr_t)127);
    const bool hasB = !PLAIN && G.fB != nullptr;
    const bool hasK = !PLAIN && G.hasK != 0;
    const bool hasBeta = !PLAIN && G.beta != nullptr;
    const AdjLayout L = adj_layout((int)sizeof(T), hasK, hasB, TMA, gin.nk, hasBeta);
    const AdjSmem<T> S = adj_smem<T>(smem_raw, L, hasK, hasB);
    const int f = blockIdx.z;
    const int j0 = blockIdx.y * AT_Y, i0 = blockIdx.x * AT_X;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const long long fo = f * G.fs;
    // phase A runs on vertical pairs of points (rows a, a+1 of the region)
    constexpr int NPA = (AA_Y / 2) * AA_X;
    constexpr int NAL = (NPA + 255) / 256;
    T lkv[NAL][2], bev[NAL][2];
    bool m3a[NAL][2];
    if constexpr (TMA) {
        // ---- bulk tensor copies of every staged tile, one mbarrier ----
        const uint32_t sb = (uint32_t)__cvta_generic_to_shared(smem_raw);
        const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&tbar);
        const uint32_t gtile = adj_al((uint32_t)(AG_Y * AG_X * sizeof(T)));
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            const uint32_t bytes = (uint32_t)sizeof(T) * (AH_Y * AH_X + AQ_Y * AQ_X + (hasB ? AQ_Y * AQ_X : 0) +
                                                          (gin.nk + (hasBeta ? 1 : 0)) * AG_Y * AG_X) +
                                   AM_Y * AM_X;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
            tma_tile_3d(sb + L.h, &M.h, i0 - 4, j0 - 3, f, bar);
            tma_tile_3d(sb + L.q, &M.q, i0 - 4, j0 - 4, f, bar);
            if (hasB) tma_tile_2d(sb + L.qa, &M.fB, i0 - 4, j0 - 4, bar);
            for (int t = 0; t < gin.nk; ++t) tma_tile_3d(sb + L.out + t * gtile, &M.g[t], i0 - 4, j0 - 2, f, bar);
            if (hasBeta) tma_tile_2d(sb + L.beta, &M.beta, i0 - 4, j0 - 2, bar);
            tma_tile_2d(sb + L.mask, &M.mask, i0 - 16, j0 - 2, bar);
        }
        __syncthreads();   // the barrier is initialised before anyone polls it
        const bool ok = qg_mbar_wait(bar, 2000000000ull);
        if (!__syncthreads_and(ok)) {
            // copies that did not arrive in 2 s: flag it, give them another
            // bounded interval to land in this CTA's shared memory, and leave
            if (tid == 0) {
                atomicOr(&g_qg_tile_error, 8);
                qg_mbar_wait(bar, 2000000000ull);
            }
            return;
        }
        if (hasB)
            for (int e = tid; e < AQ_Y * AQ_X; e += 256) (&S.qa[0][0])[e] += (&S.q[0][0])[e];
        const int8_t* mk = reinterpret_cast<const int8_t*>(smem_raw + L.mask);
        const T* bt = reinterpret_cast<const T*>(smem_raw + L.beta);
#pragma unroll
        for (int k = 0; k < NAL; ++k) {
            const int e = tid + 256 * k;
            const int ap = e / AA_X, b = e - ap * AA_X;
            const bool in = e < NPA;
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int a = 2 * ap + u;
                T lk = T(0);
#pragma unroll
                for (int t = 0; t < 4; ++t)
                    if (t < gin.nk && in)
                        lk += gin.c[t] * reinterpret_cast<const T*>(smem_raw + L.out + t * gtile)[a * AG_X + b + 2];
                lkv[k][u] = lk;
                m3a[k][u] = in && mk[a * AM_X + b + 14] == 3;
                bev[k][u] = (in && hasBeta) ? bt[a * AG_X + b + 2] : T(0);
            }
        }
    } else {
        // ---- bounds-checked loads: every load of the thread before any store ----
        constexpr int NHL = (AH_Y * AH_X + 255) / 256, NQL = (AQ_Y * AQ_X + 255) / 256;
        T hv[NHL], qv[NQL];
#pragma unroll
        for (int k = 0; k < NHL; ++k) {
            const int e = tid + 256 * k;
            const int a = e / AH_X, b = e - a * AH_X;
            const int j = j0 - 3 + a, i = i0 - 4 + b;
            hv[k] = (e < AH_Y * AH_X && j >= 0 && j < G.ny && i >= 0 && i < G.nx) ? hs[fo + (long long)j * G.nx + i]
                                                                                  : T(0);
        }
#pragma unroll
        for (int k = 0; k < NQL; ++k) {
            const int e = tid + 256 * k;
            const int a = e / AQ_X, b = e - a * AQ_X;
            const int j = j0 - 4 + a, i = i0 - 4 + b;
            qv[k] = (e < AQ_Y * AQ_X && j >= 0 && j < G.ny && i >= 0 && i < G.nx) ? qs[fo + (long long)j * G.nx + i]
                                                                                  : T(0);
        }
#pragma unroll
        for (int k = 0; k < NHL; ++k) {
            const int e = tid + 256 * k;
            if (e < AH_Y * AH_X) (&S.h[0][0])[e] = hv[k];
        }
#pragma unroll
        for (int k = 0; k < NQL; ++k) {
            const int e = tid + 256 * k;
            if (e < AQ_Y * AQ_X) (&S.q[0][0])[e] = qv[k];
        }
        if (hasB) {
            for (int e = tid; e < AQ_Y * AQ_X; e += 256) {
                const int a = e / AQ_X, b = e - a * AQ_X;
                const int j = j0 - 4 + a, i = i0 - 4 + b;
                const bool in = (j >= 0 && j < G.ny && i >= 0 && i < G.nx);
                S.qa[a][b] = S.q[a][b] + (in ? ((const T*)G.fB)[(long long)j * G.nx + i] : T(0));
            }
        }
        // per-point inputs of phase A (tendency adjoint, interior flag, beta)
#pragma unroll
        for (int k = 0; k < NAL; ++k) {
            const int e = tid + 256 * k;
            const int ap = e / AA_X, b = e - ap * AA_X;
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int a = 2 * ap + u;
                const int j = j0 - 2 + a, i = i0 - 2 + b;
                const bool in = e < NPA && j >= 0 && j < G.ny && i >= 0 && i < G.nx;
                const long long g2 = (long long)j * G.nx + i;
                const long long o = fo + g2;
                T lk = T(0);
#pragma unroll
                for (int t = 0; t < 4; ++t)
                    if (t < gin.nk && in) lk += gin.c[t] * gin.k[t][o];
                lkv[k][u] = lk;
                m3a[k][u] = in && G.mask[g2] == 3;
                bev[k][u] = (in && hasBeta) ? ((const T*)G.beta)[g2] : T(0);
            }
        }
    }
    __syncthreads();
    // ---- phase A on the tile + halo 2, two vertically adjacent points per
    // thread: their SSH and PV stencils overlap, so the pair reads 12 h and
    // 14 q values (each point alone 8 and 9) and then runs the single-point
    // arithmetic on each ----
    const T cx = T(G.cx), cy = T(G.cy), cu = T(G.cu), cv = T(G.cv);
#pragma unroll
    for (int k = 0; k < NAL; ++k) {
        const int e = tid + 256 * k;
        if (e >= NPA) break;
        const int ap = e / AA_X, b = e - ap * AA_X;
        const int a0 = 2 * ap;
        T lk[2] = {T(0), T(0)}, uT[2] = {T(0), T(0)}, vT[2] = {T(0), T(0)}, aut[2] = {T(0), T(0)},
          avt[2] = {T(0), T(0)};
        if (m3a[k][0] || m3a[k][1]) {
            const int ha = a0 + 1, hb = b + 2;     // h-tile index of the first point
            T hv[4][3];                            // rows ha-1 .. ha+2, columns hb-1 .. hb+1
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) hv[r][c] = S.h[ha - 1 + r][hb - 1 + c];
            const int qa_ = a0 + 2, qb_ = b + 2;   // q-tile index of the first point
            T vq[6], hq[2][4];                     // column qb_ rows qa_-2 .. qa_+3; rows qa_, qa_+1 at qb_-2, -1, +1, +2
            T vqa[6], hqa[2][4];
#pragma unroll
            for (int r = 0; r < 6; ++r) vq[r] = S.q[qa_ - 2 + r][qb_];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                hq[u][0] = S.q[qa_ + u][qb_ - 2]; hq[u][1] = S.q[qa_ + u][qb_ - 1];
                hq[u][2] = S.q[qa_ + u][qb_ + 1]; hq[u][3] = S.q[qa_ + u][qb_ + 2];
            }
            if (hasB) {
#pragma unroll
                for (int r = 0; r < 6; ++r) vqa[r] = S.qa[qa_ - 2 + r][qb_];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    hqa[u][0] = S.qa[qa_ + u][qb_ - 2]; hqa[u][1] = S.qa[qa_ + u][qb_ - 1];
                    hqa[u][2] = S.qa[qa_ + u][qb_ + 1]; hqa[u][3] = S.qa[qa_ + u][qb_ + 2];
                }
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (!m3a[k][u]) continue;
                lk[u] = lkv[k][u];
                // rows of this point: s = u, m = u + 1, n = u + 2 in hv
                const T(&hs_)[3] = hv[u];
                const T(&hm_)[3] = hv[u + 1];
                const T(&hn_)[3] = hv[u + 2];
                Vel<T> V;
                V.u0 = guard0(cu * (hn_[0] + hn_[1] - hs_[1] - hs_[0]));
                V.u1 = guard0(cu * (hn_[1] + hn_[2] - hs_[2] - hs_[1]));
                V.v0 = guard0(cv * (hm_[2] + hs_[2] - hs_[0] - hm_[0]));
                V.v1 = guard0(cv * (hn_[2] + hm_[2] - hm_[0] - hn_[0]));
                Cross<T> q;
                q.c = vq[2 + u]; q.e1 = hq[u][2]; q.e2 = hq[u][3]; q.w1 = hq[u][1]; q.w2 = hq[u][0];
                q.n1 = vq[3 + u]; q.n2 = vq[4 + u]; q.s1 = vq[1 + u]; q.s2 = vq[u];
                Cross<T> qa = q;
                if (hasB) {
                    qa.c = vqa[2 + u]; qa.e1 = hqa[u][2]; qa.e2 = hqa[u][3]; qa.w1 = hqa[u][1]; qa.w2 = hqa[u][0];
                    qa.n1 = vqa[3 + u]; qa.n2 = vqa[4 + u]; qa.s1 = vqa[1 + u]; qa.s2 = vqa[u];
                }
                const T beta = bev[k][u];
                if (isnan(tendency<T, !PLAIN>(G, V, qa, q, beta))) lk[u] = T(0);
                uT[u] = T(0.5) * (V.u0 + V.u1);
                vT[u] = T(0.5) * (V.v0 + V.v1);
                const T gu = (uT[u] >= T(0) ? -cx * qa.Dpx() : T(0)) + (uT[u] <= T(0) ? cx * qa.Dmx() : T(0));
                const T gv = (vT[u] >= T(0) ? -cy * qa.Dpy() : T(0)) + (vT[u] <= T(0) ? cy * qa.Dmy() : T(0));
                aut[u] = lk[u] * gu;
                avt[u] = lk[u] * gv - beta * lk[u];
            }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int a = a0 + u;
            S.lup[a][b] = lk[u] * (uT[u] < T(0) ? T(0) : uT[u]);
            S.lum[a][b] = lk[u] * (uT[u] > T(0) ? T(0) : uT[u]);
            S.lvp[a][b] = lk[u] * (vT[u] < T(0) ? T(0) : vT[u]);
            S.lvm[a][b] = lk[u] * (vT[u] > T(0) ? T(0) : vT[u]);
            S.aut[a][b] = aut[u];
            S.avt[a][b] = avt[u];
            if (hasK) S.lk[a][b] = lk[u];
        }
    }
    __syncthreads();
    // ---- phase B on the tile, vertical pairs of points (accumulated adjoints
    // and flags loaded first); the pair shares its y-stencil, diffusion and
    // h2uv-transpose reads ----
    constexpr int NPB = (AT_Y / 2) * AT_X;
    constexpr int NBL = (NPB + 255) / 256;
    T accv[NBL][2];
    bool m3b[NBL][2];
#pragma unroll
    for (int k = 0; k < NBL; ++k) {
        const int e = tid + 256 * k;
        const int ap = e / AT_X, b = e - ap * AT_X;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int a = 2 * ap + u;
            const int j = j0 + a, i = i0 + b;
            const bool in = e < NPB && j < G.ny && i < G.nx;
            const long long o = fo + (long long)j * G.nx + i;
            T sacc = T(0);
#pragma unroll
            for (int t = 0; t < 4; ++t)
                if (t < gacc.nk && in) sacc += gacc.k[t][o];
            accv[k][u] = sacc;
            if constexpr (TMA)
                m3b[k][u] = in && reinterpret_cast<const int8_t*>(smem_raw + L.mask)[(a + 2) * AM_X + b + 16] == 3;
            else
                m3b[k][u] = in && G.mask[(long long)j * G.nx + i] == 3;
        }
    }
    const T hu = T(0.5) * cu, hv2 = T(0.5) * cv;
#pragma unroll
    for (int k = 0; k < NBL; ++k) {
        const int e = tid + 256 * k;
        if (e >= NPB) break;
        const int ap = e / AT_X, b = e - ap * AT_X;
        const int a0 = 2 * ap;
        const int i = i0 + b;
        if (j0 + a0 >= G.ny || i >= G.nx) continue;
        const int A = a0 + 2, Bc = b + 2;    // phase-A index of the first point
        T vp[5], vm[5];                      // VP rows A-1 .. A+3, VM rows A-2 .. A+2 (column Bc)
#pragma unroll
        for (int r = 0; r < 5; ++r) {
            vp[r] = S.lvp[A - 1 + r][Bc];
            vm[r] = S.lvm[A - 2 + r][Bc];
        }
        T at[4][3], av[4][2];                // aut rows A-1 .. A+2 x columns Bc-1 .. Bc+1; avt at Bc-1, Bc+1
#pragma unroll
        for (int r = 0; r < 4; ++r) {
#pragma unroll
            for (int c = 0; c < 3; ++c) at[r][c] = S.aut[A - 1 + r][Bc - 1 + c];
            av[r][0] = S.avt[A - 1 + r][Bc - 1];
            av[r][1] = S.avt[A - 1 + r][Bc + 1];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int Au = A + u;
            const int j = j0 + a0 + u;
            if (j >= G.ny) break;
            auto UP = [&](int db) { return S.lup[Au][Bc + db]; };
            auto UM = [&](int db) { return S.lum[Au][Bc + db]; };
            // VP(d) = vp[u + 1 + d], VM(d) = vm[u + 2 + d]
            T aq = cx * (-T(2) * UP(-1) - T(6) * UM(-1)
                         - T(3) * UP(0) + T(3) * UM(0)
                         + T(6) * UP(1) + T(2) * UM(1)
                         - UP(2) + UM(-2))
                 + cy * (-T(2) * vp[u] - T(6) * vm[u + 1]
                         - T(3) * vp[u + 1] + T(3) * vm[u + 2]
                         + T(6) * vp[u + 2] + T(2) * vm[u + 3]
                         - vp[u + 3] + vm[u]);
            if (hasK) {
                const T lc = S.lk[Au][Bc];
                aq += T(G.Kx) * (S.lk[Au][Bc - 1] + S.lk[Au][Bc + 1] - T(2) * lc)
                    + T(G.Ky) * (S.lk[Au - 1][Bc] + S.lk[Au + 1][Bc] - T(2) * lc);
            }
            const long long o = fo + (long long)j * G.nx + i;
            adq_out[o] = m3b[k][u] ? aq + accv[k][u] : T(0);
            // aut rows Au-1, Au+1 = at[u], at[u + 2]; avt rows Au-1 .. Au+1 = av[u .. u + 2]
            adh_out[o] = hu * (at[u][0] + T(2) * at[u][1] + at[u][2]
                               - at[u + 2][0] - T(2) * at[u + 2][1] - at[u + 2][2])
                       + hv2 * (av[u][0] + T(2) * av[u + 1][0] + av[u + 2][0]
                                - av[u][1] - T(2) * av[u + 1][1] - av[u + 2][1]);
        }
    }
}

// ---- host side of the adjoint stage ----------------------------------------

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, []() {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            (void)cudaGetLastError();
    });
    return fn;
}

// A tiled map over [nz][ny][nx] elements of `esz` bytes (rank 3, fields z
// apart) or [ny][nx] (rank 2), box bx x by (x 1). False when the driver
// refuses it.
static bool tile_map(CUtensorMap* m, const void* base, int esz, int nx, int ny, int nz, long long zstride, int bx,
                     int by, int rank)
{
    auto enc = tensor_map_encoder();
    if (!enc || !base || ((uintptr_t)base & 15)) return false;
    const CUtensorMapDataType dt = esz == 8   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                                   : esz == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                              : CU_TENSOR_MAP_DATA_TYPE_UINT8;
    const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t strides[2] = {(cuuint64_t)nx * esz, (cuuint64_t)zstride * esz};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return enc(m, dt, (cuuint32_t)rank, const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The staged form needs rows of a multiple of 16 elements (16-byte row
// strides of the int8 mask and of every field, 16-byte aligned field bases).
template <typename T>
static bool adj_tma_maps(const vd_qg1l_plan* p, int nf, const T* hs, const T* qs, const StageIn<T>& gin,
                         AdjMaps& M)
{
    const QGGeom& G = p->geom;
    if (p->sched.stencil_loads == 1 || G.nx % 16 != 0 || G.fs % 16 != 0) return false;
    // the field maps span the nf fields of this launch (z = field)
    auto fmap = [&](CUtensorMap* m, const T* base, int by) {
        return tile_map(m, base, sizeof(T), G.nx, G.ny, nf, G.fs, AG_X, by, 3);
    };
    if (!fmap(&M.h, hs, AH_Y) || !fmap(&M.q, qs, AQ_Y)) return false;
    for (int t = 0; t < gin.nk; ++t)
        if (!fmap(&M.g[t], gin.k[t], AG_Y)) return false;
    if (G.beta && !tile_map(&M.beta, G.beta, sizeof(T), G.nx, G.ny, 1, G.fs, AG_X, AG_Y, 2)) return false;
    if (G.fB && !tile_map(&M.fB, G.fB, sizeof(T), G.nx, G.ny, 1, G.fs, AQ_X, AQ_Y, 2)) return false;
    return tile_map(&M.mask, G.mask, 1, G.nx, G.ny, 1, G.fs, AM_X, AM_Y, 2);
}

template <typename T>
static cudaError_t adj_stage_attrs()
{
    static PerDeviceOnce once;
    return once.run([]() -> cudaError_t {
        const int big = (int)adj_layout(sizeof(T), true, true, true, 4, true).total + 128;
        cudaError_t e = cudaFuncSetAttribute(k_adj_stage_fused<T, true, false>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        if (!e)
            e = cudaFuncSetAttribute(k_adj_stage_fused<T, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     big);
        if (!e)
            e = cudaFuncSetAttribute(k_adj_stage_fused<T, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     big);
        if (!e)
            e = cudaFuncSetAttribute(k_adj_stage_fused<T, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     big);
        if (!e)
            e = cudaFuncSetAttribute(k_adj_stage_fused<T, true, true, 1, 0>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        if (!e)
            e = cudaFuncSetAttribute(k_adj_stage_fused<T, true, true, 1, 2>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, big);
        return e;
    });
}

// One adjoint stage over nf fields: the staged (TMA) form when the grid
// allows it, the bounds-checked form otherwise.
template <typename T>
static int launch_adj_stage(const vd_qg1l_plan* p, int nf, const T* hs, const T* qs, const StageIn<T>& gin,
                            const StageIn<T>& gacc, T* adq_out, T* adh_out, cudaStream_t st)
{
    if (adj_stage_attrs<T>() != cudaSuccess) return VD_ERR_CUDA;
    const QGGeom& G = p->geom;
    const dim3 agrid((p->d.nx + AT_X - 1) / AT_X, (p->d.ny + AT_Y - 1) / AT_Y, nf);
    const dim3 block(32, 8);
    AdjMaps M;
    std::memset(&M, 0, sizeof(M));
    const bool tma = adj_tma_maps<T>(p, nf, hs, qs, gin, M);
    const size_t smem = adj_layout(sizeof(T), G.hasK != 0, G.fB != nullptr, tma, gin.nk, G.beta != nullptr).total + 128;
    const bool plain = plain_geom(G);
    // the two stage forms of RK2 (midpoint: b = (0, dt); s = 1: one stage
    // adjoint; s = 0: one, plus the two accumulated adjoints) with their
    // counts compiled in
    if (tma && plain && gin.nk == 1 && gacc.nk == 0)
        k_adj_stage_fused<T, true, true, 1, 0><<<agrid, block, smem, st>>>(G, nf, hs, qs, gin, gacc, adq_out, adh_out,
                                                                           M);
    else if (tma && plain && gin.nk == 1 && gacc.nk == 2)
        k_adj_stage_fused<T, true, true, 1, 2><<<agrid, block, smem, st>>>(G, nf, hs, qs, gin, gacc, adq_out, adh_out,
                                                                           M);
    else if (tma && plain)
        k_adj_stage_fused<T, true, true><<<agrid, block, smem, st>>>(G, nf, hs, qs, gin, gacc, adq_out, adh_out, M);
    else if (tma)
        k_adj_stage_fused<T, true, false><<<agrid, block, smem, st>>>(G, nf, hs, qs, gin, gacc, adq_out, adh_out, M);
    else if (plain)
        k_adj_stage_fused<T, false, true><<<agrid, block, smem, st>>>(G, nf, hs, qs, gin, gacc, adq_out, adh_out, M);
    else
        k_adj_stage_fused<T, false, false><<<agrid, block, smem, st>>>(G, nf, hs, qs, gin, gacc, adq_out, adh_out, M);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

int qg_tile_error(int* flags, int reset)
{
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_qg_tile_error, sizeof(int)) != cudaSuccess) return VD_ERR_CUDA;
    *flags |= v;
    if (reset) {
        const int zero = 0;
        if (cudaMemcpyToSymbol(g_qg_tile_error, &zero, sizeof(int)) != cudaSuccess) return VD_ERR_CUDA;
    }
    return VD_OK;
}

// ---------------------------------------------------------------------------
// Small kernels: copies, finalize, h2uv / rhs on given fields (API pieces)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_copy_masked(QGGeom G, int nf, const T* __restrict__ src, T* __restrict__ dst, int zero_land)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int f = blockIdx.z;
    if (i >= G.nx || j >= G.ny || f >= nf) return;
    const long long o = f * G.fs + (long long)j * G.nx + i;
    T v = src[o];
    if (zero_land && G.mask[(long long)j * G.nx + i] == 0) v = T(0);
    dst[o] = v;
}

template <typename T>
__global__ void k_fill(long long n, T v, T* __restrict__ x)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) x[k] = v;
}

// out = (land ? {h, NaN, 0}[land_mode] : (wall ? (hb or 0) : h)) + coef*forcing
template <typename T>
__global__ void k_finalize(QGGeom G, int nf, const T* __restrict__ h, const T* __restrict__ hb,
                           const T* __restrict__ forcing, T coef, const double* __restrict__ coefv,
                           int land_mode, T* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int f = blockIdx.z;
    if (i >= G.nx || j >= G.ny || f >= nf) return;
    const long long o = f * G.fs + (long long)j * G.nx + i;
    const bool wall = (i == 0 || j == 0 || i == G.nx - 1 || j == G.ny - 1);
    T v;
    if (wall)
        v = hb ? hb[o] : T(0);
    else
        v = h[o];
    if (G.mask[(long long)j * G.nx + i] == 0 && land_mode != 0)
        v = land_mode == 1 ? T(NAN) : T(0);
    if (forcing) v += (coefv ? T(coefv[f]) : coef) * forcing[o];
    out[o] = v;
}

// Adjoint of k_finalize: the forcing adjoint takes coef[f] * adh_out
// everywhere (mod.py:1058-1068); the state adjoint is adh_out except on the
// walls (set to hb) and on land (set to a constant), where it is 0.
template <typename T>
__global__ void k_finalize_adj(QGGeom G, int nf, const T* __restrict__ adout, T* __restrict__ adforcing,
                               const double* __restrict__ coefv, T* __restrict__ adh)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int f = blockIdx.z;
    if (i >= G.nx || j >= G.ny || f >= nf) return;
    const long long o = f * G.fs + (long long)j * G.nx + i;
    const T a = adout[o];
    if (adforcing) adforcing[o] += T(coefv[f]) * a;
    const bool wall = (i == 0 || j == 0 || i == G.nx - 1 || j == G.ny - 1);
    adh[o] = (wall || G.mask[(long long)j * G.nx + i] == 0) ? T(0) : a;
}

template <typename T>
__global__ void k_h2uv(QGGeom G, int nf, const T* __restrict__ h, T* __restrict__ u, T* __restrict__ v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int f = blockIdx.z;
    if (i >= G.nx || j >= G.ny || f >= nf) return;
    const long long o = f * G.fs + (long long)j * G.nx + i;
    const int nx = G.nx;
    T uu = T(0), vv = T(0);
    if (j >= 1 && j <= G.ny - 2 && i >= 1)
        uu = T(G.cu) * (h[o + nx - 1] + h[o + nx] - h[o - nx] - h[o - nx - 1]);
    if (j >= 1 && i >= 1 && i <= G.nx - 2)
        vv = T(G.cv) * (h[o + 1] + h[o - nx + 1] - h[o - nx - 1] - h[o - 1]);
    u[o] = guard0(uu);
    v[o] = guard0(vv);
}

template <typename T>
__global__ void k_rhs_uv(QGGeom G, int nf, const T* __restrict__ u, const T* __restrict__ v,
                         const T* __restrict__ q, T* __restrict__ rhs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int f = blockIdx.z;
    if (i >= G.nx || j >= G.ny || f >= nf) return;
    const long long o = f * G.fs + (long long)j * G.nx + i;
    const long long go = (long long)j * G.nx + i;
    T r = T(0);
    if (G.mask[go] == 3) {
        Vel<T> V;
        V.u0 = u[o]; V.u1 = u[o + 1]; V.v0 = v[o]; V.v1 = v[o + G.nx];
        Cross<T> qq;
        qq.load(q + o, G.nx);
        Cross<T> qa = qq;
        if (G.fB) { Cross<T> b; b.load((const T*)G.fB + go, G.nx); qa.add(b); }
        const T beta = G.beta ? ((const T*)G.beta)[go] : T(0);
        r = guard0(tendency<T>(G, V, qa, qq, beta));
    }
    rhs[o] = r;
}

// ---------------------------------------------------------------------------
// Host drivers
// ---------------------------------------------------------------------------
static inline dim3 pgrid(const vd_qg1l_plan* p, int nf) { return dim3((p->d.nx + 31) / 32, (p->d.ny + 7) / 8, nf); }
static const dim3 kBlock(32, 8);

template <typename T> static QGGeom geomT(const vd_qg1l_plan* p) { return p->geom; }

// Does a later combination use k_s?  (stage s writes q_{s+1}; k_s is needed by
// stages t >= s+2 or by the final combination when s is not the last stage)
static bool need_k(const vd_qg1l_plan* p, int s)
{
    const int S = p->nstage;
    if (s == S - 1) return false;
    if (p->b[s] != 0.0) return true;
    for (int t = s + 2; t < S; ++t)
        if (p->A[t][s] != 0.0) return true;
    return false;
}

template <typename T>
struct TrajView {
    T* base;
    int S;
    long long fb;   // elements per batch-field (nf * fs)
    T* h(int n, int s) const { return base + ((long long)(n * S + s) * 2 + 0) * fb; }
    T* q(int n, int s) const { return base + ((long long)(n * S + s) * 2 + 1) * fb; }
};

// One forward step (stage loop) between explicit buffers.
template <typename T>
static int step_once(const vd_qg1l_plan* p, int nf, T* const* hsv, T* const* qsv, T* hnew, T* qnew,
                     T* const* kbuf, const T* hb, const T* qb, T* spec, cudaStream_t st, bool tangent, T* qlo)
{
    const int S = p->nstage;
    const int B = tangent ? nf / 2 : nf;
    for (int s = 0; s < S; ++s) {
        const bool last = (s == S - 1);
        StageIn<T> kin{};
        kin.nk = 0;
        for (int i = 0; i < s; ++i) {
            const double c = last ? p->b[i] : p->A[s + 1][i];
            if (c != 0.0) { kin.k[kin.nk] = kbuf[i]; kin.c[kin.nk] = (T)c; ++kin.nk; }
        }
        const T cself = (T)(last ? p->b[s] : p->A[s + 1][s]);
        T* kout = need_k(p, s) ? kbuf[s] : nullptr;
        T* qo = last ? qnew : qsv[s + 1];
        T* ho = last ? hnew : hsv[s + 1];
        if (tangent)
            k_stage_tl<T><<<pgrid(p, B), kBlock, 0, st>>>(p->geom, B, hsv[s], qsv[s], qsv[0], kin, cself, kout, qo,
                                                          qlo, last ? 1 : 0);
        else if (plain_geom(p->geom))
            k_stage_fwd<T, true><<<pgrid(p, nf), dim3(32, 4), 0, st>>>(p->geom, nf, hsv[s], qsv[s], qsv[0], kin, cself,
                                                                       kout, qo, qlo, last ? 1 : 0);
        else
            k_stage_fwd<T, false><<<pgrid(p, nf), dim3(32, 4), 0, st>>>(p->geom, nf, hsv[s], qsv[s], qsv[0], kin,
                                                                        cself, kout, qo, qlo, last ? 1 : 0);
        VD_LAUNCH_CHECK();
        SolveArgs a;
        a.src = qo; a.sub = qb; a.sub_batches = B;
        a.out = ho; a.add = hb; a.add_batches = B; a.epi = EPI_H;
        int rc = helmholtz_solve<T>(p, nf, a, spec, st);
        if (rc) return rc;
    }
    return VD_OK;
}

template <typename T>
int advance_impl(const vd_qg1l_plan* p, int nf, T* traj, int traj_steps, int first, int nstep,
                 const T* hb, const T* qb, T* qlo, Arena& ws, cudaStream_t st)
{
    if (first < 0 || nstep < 0 || first + nstep > traj_steps) return VD_ERR_ARG;
    const int S = p->nstage;
    const long long fb = (long long)nf * p->geom.fs;
    TrajView<T> tv{traj, S, fb};
    T* kbuf[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int s = 0; s < S; ++s)
        if (need_k(p, s) && !(kbuf[s] = (T*)ws.take(fb * sizeof(T)))) return VD_ERR_WORKSPACE;
    T* spec = (T*)ws.take(spec_bytes(p, nf));
    if (!spec) return VD_ERR_WORKSPACE;
    for (int n = first; n < first + nstep; ++n) {
        T* hs[4]; T* qs[4];
        for (int s = 0; s < S; ++s) { hs[s] = tv.h(n, s); qs[s] = tv.q(n, s); }
        int rc = step_once<T>(p, nf, hs, qs, tv.h(n + 1, 0), tv.q(n + 1, 0), kbuf, hb, qb, spec, st, false, qlo);
        if (rc) return rc;
    }
    return VD_OK;
}

// Forward without trajectory: ping-pong states in the workspace.
template <typename T>
int forward_nostore(const vd_qg1l_plan* p, int nf, T* h, T* q, int nstep, const T* hb, const T* qb,
                    T* qlo, Arena& ws, cudaStream_t st, bool tangent)
{
    const int S = p->nstage;
    const long long fb = (long long)nf * p->geom.fs;
    T* kbuf[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int s = 0; s < S; ++s)
        if (need_k(p, s) && !(kbuf[s] = (T*)ws.take(fb * sizeof(T)))) return VD_ERR_WORKSPACE;
    T* hs[4]; T* qs[4];
    hs[0] = h; qs[0] = q;
    for (int s = 1; s < S; ++s) {
        hs[s] = (T*)ws.take(fb * sizeof(T));
        qs[s] = (T*)ws.take(fb * sizeof(T));
        if (!hs[s] || !qs[s]) return VD_ERR_WORKSPACE;
    }
    T* h2 = (T*)ws.take(fb * sizeof(T));
    T* q2 = (T*)ws.take(fb * sizeof(T));
    T* spec = (T*)ws.take(spec_bytes(p, nf));
    if (!h2 || !q2 || !spec) return VD_ERR_WORKSPACE;
    T* cur_h = h; T* cur_q = q; T* nxt_h = h2; T* nxt_q = q2;
    for (int n = 0; n < nstep; ++n) {
        hs[0] = cur_h; qs[0] = cur_q;
        int rc = step_once<T>(p, nf, hs, qs, nxt_h, nxt_q, kbuf, hb, qb, spec, st, tangent, qlo);
        if (rc) return rc;
        T* t1 = cur_h; cur_h = nxt_h; nxt_h = t1;
        T* t2 = cur_q; cur_q = nxt_q; nxt_q = t2;
    }
    if (cur_h != h) {
        VD_CUDA_TRY(cudaMemcpyAsync(h, cur_h, fb * sizeof(T), cudaMemcpyDeviceToDevice, st));
        VD_CUDA_TRY(cudaMemcpyAsync(q, cur_q, fb * sizeof(T), cudaMemcpyDeviceToDevice, st));
    }
    return VD_OK;
}

template <typename T>
int advance_adj_impl(const vd_qg1l_plan* p, int nf, const T* traj, int traj_steps, int first, int nstep,
                     T* adh, T* adq, Arena& ws, cudaStream_t st)
{
    if (first < 0 || nstep < 0 || first + nstep > traj_steps) return VD_ERR_ARG;
    const int S = p->nstage;
    const long long fb = (long long)nf * p->geom.fs;
    TrajView<T> tv{const_cast<T*>(traj), S, fb};
    T* Gb[4];
    for (int s = 0; s < S; ++s)
        if (!(Gb[s] = (T*)ws.take(fb * sizeof(T)))) return VD_ERR_WORKSPACE;
    T* adql = (T*)ws.take(fb * sizeof(T));
    T* adhs = (T*)ws.take(fb * sizeof(T));
    T* spec = (T*)ws.take(spec_bytes(p, nf));
    if (!adql || !adhs || !spec) return VD_ERR_WORKSPACE;

    for (int n = first + nstep - 1; n >= first; --n) {
        // adjoint of h_{n+1} = I(q_{n+1}): G0 = M3*(solve(adh) + adq)
        SolveArgs a0;
        a0.src = adh; a0.sub = nullptr; a0.sub_batches = 0;
        a0.out = Gb[0]; a0.add = adq; a0.add_batches = nf; a0.epi = EPI_ADJQ;
        int rc = helmholtz_solve<T>(p, nf, a0, spec, st);
        if (rc) return rc;
        for (int s = S - 1; s >= 0; --s) {
            StageIn<T> gin{};
            gin.nk = 0;
            if (p->b[s] != 0.0) { gin.k[gin.nk] = Gb[0]; gin.c[gin.nk] = (T)p->b[s]; ++gin.nk; }
            for (int t = s + 1; t < S; ++t)
                if (p->A[t][s] != 0.0) { gin.k[gin.nk] = Gb[t]; gin.c[gin.nk] = (T)p->A[t][s]; ++gin.nk; }
            if (s >= 1) {
                StageIn<T> none{};
                none.nk = 0;
                rc = launch_adj_stage<T>(p, nf, tv.h(n, s), tv.q(n, s), gin, none, adql, adhs, st);
                if (rc) return rc;
                SolveArgs a;
                a.src = adhs; a.sub = nullptr; a.sub_batches = 0;
                a.out = Gb[s]; a.add = adql; a.add_batches = nf; a.epi = EPI_ADJQ;
                rc = helmholtz_solve<T>(p, nf, a, spec, st);
                if (rc) return rc;
            } else {
                StageIn<T> acc{};
                acc.nk = 0;
                for (int t = 0; t < S; ++t) { acc.k[acc.nk] = Gb[t]; acc.c[acc.nk] = T(1); ++acc.nk; }
                rc = launch_adj_stage<T>(p, nf, tv.h(n, s), tv.q(n, s), gin, acc, adq, adh, st);
                if (rc) return rc;
            }
        }
    }
    return VD_OK;
}

// One forward stage and one adjoint stage on caller buffers: the kernels of
// step_once / advance_adj_impl, launched alone (building blocks and kernel
// timing).
template <typename T>
int rk_stage_impl(const vd_qg1l_plan* p, int nf, const T* hs, const T* qs, const T* qbase, int nk,
                  const T* const* k, const double* c, double cself, T* kout, T* qout, cudaStream_t st)
{
    StageIn<T> kin{};
    kin.nk = nk;
    for (int t = 0; t < nk; ++t) { kin.k[t] = k[t]; kin.c[t] = (T)c[t]; }
    if (plain_geom(p->geom))
        k_stage_fwd<T, true><<<pgrid(p, nf), dim3(32, 4), 0, st>>>(p->geom, nf, hs, qs, qbase, kin, (T)cself, kout,
                                                                   qout, (T*)nullptr, 0);
    else
        k_stage_fwd<T, false><<<pgrid(p, nf), dim3(32, 4), 0, st>>>(p->geom, nf, hs, qs, qbase, kin, (T)cself, kout,
                                                                    qout, (T*)nullptr, 0);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename T>
int rk_stage_adj_impl(const vd_qg1l_plan* p, int nf, const T* hs, const T* qs, int ng, const T* const* g,
                      const double* c, int nacc, const T* const* acc, T* adq_out, T* adh_out, cudaStream_t st)
{
    StageIn<T> gin{}, gac{};
    gin.nk = ng;
    for (int t = 0; t < ng; ++t) { gin.k[t] = g[t]; gin.c[t] = (T)c[t]; }
    gac.nk = nacc;
    for (int t = 0; t < nacc; ++t) { gac.k[t] = acc[t]; gac.c[t] = T(1); }
    return launch_adj_stage<T>(p, nf, hs, qs, gin, gac, adq_out, adh_out, st);
}

template <typename T>
int init_state_impl(const vd_qg1l_plan* p, int nf, int ntan0, const T* h, const T* hb, T* q, T* qb,
                    T* qlo, cudaStream_t st)
{
    k_h2pv<T><<<pgrid(p, nf), kBlock, 0, st>>>(p->geom, nf, ntan0, h, hb, q, qlo);
    VD_LAUNCH_CHECK();
    if (qb) {
        k_h2pv<T><<<pgrid(p, ntan0), kBlock, 0, st>>>(p->geom, ntan0, ntan0, hb, hb, qb, (T*)nullptr);
        VD_LAUNCH_CHECK();
    }
    return VD_OK;
}

template <typename T>
int init_state_adj_impl(const vd_qg1l_plan* p, int nf, const T* h, const T* adq, T* adh, cudaStream_t st)
{
    k_h2pv_adj<T><<<pgrid(p, nf), kBlock, 0, st>>>(p->geom, nf, h, adq, adh);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename T>
int finalize_impl(const vd_qg1l_plan* p, int nf, const T* h, const T* hb, const T* forcing, double coef,
                  const double* coefv, int land_mode, T* out, cudaStream_t st)
{
    k_finalize<T><<<pgrid(p, nf), kBlock, 0, st>>>(p->geom, nf, h, hb, forcing, (T)coef, coefv, land_mode, out);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename T>
int finalize_adj_impl(const vd_qg1l_plan* p, int nf, const T* adout, T* adforcing, const double* coefv, T* adh,
                      cudaStream_t st)
{
    k_finalize_adj<T><<<pgrid(p, nf), kBlock, 0, st>>>(p->geom, nf, adout, adforcing, coefv, adh);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename T>
int copy_impl(const vd_qg1l_plan* p, int nf, const T* src, T* dst, int zero_land, cudaStream_t st)
{
    k_copy_masked<T><<<pgrid(p, nf), kBlock, 0, st>>>(p->geom, nf, src, dst, zero_land);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename T>
int zero_impl(long long n, T* x, cudaStream_t st)
{
    if (n <= 0) return VD_OK;
    k_fill<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, T(0), x);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename T>
int h2uv_impl(const vd_qg1l_plan* p, int nf, const T* h, T* u, T* v, cudaStream_t st)
{
    k_h2uv<T><<<pgrid(p, nf), kBlock, 0, st>>>(p->geom, nf, h, u, v);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template <typename T>
int rhs_impl(const vd_qg1l_plan* p, int nf, const T* u, const T* v, const T* q, T* r, cudaStream_t st)
{
    k_rhs_uv<T><<<pgrid(p, nf), kBlock, 0, st>>>(p->geom, nf, u, v, q, r);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

#define VD_INST(T)                                                                                        \
    template int rk_stage_impl<T>(const vd_qg1l_plan*, int, const T*, const T*, const T*, int, const T* const*, \
                                  const double*, double, T*, T*, cudaStream_t);                           \
    template int rk_stage_adj_impl<T>(const vd_qg1l_plan*, int, const T*, const T*, int, const T* const*,  \
                                      const double*, int, const T* const*, T*, T*, cudaStream_t);         \
    template int advance_impl<T>(const vd_qg1l_plan*, int, T*, int, int, int, const T*, const T*, T*,     \
                                 Arena&, cudaStream_t);                                                   \
    template int forward_nostore<T>(const vd_qg1l_plan*, int, T*, T*, int, const T*, const T*, T*,        \
                                    Arena&, cudaStream_t, bool);                                          \
    template int advance_adj_impl<T>(const vd_qg1l_plan*, int, const T*, int, int, int, T*, T*, Arena&,   \
                                     cudaStream_t);                                                       \
    template int init_state_impl<T>(const vd_qg1l_plan*, int, int, const T*, const T*, T*, T*, T*,        \
                                    cudaStream_t);                                                        \
    template int init_state_adj_impl<T>(const vd_qg1l_plan*, int, const T*, const T*, T*, cudaStream_t);  \
    template int finalize_impl<T>(const vd_qg1l_plan*, int, const T*, const T*, const T*, double,         \
                                  const double*, int, T*, cudaStream_t);                                  \
    template int finalize_adj_impl<T>(const vd_qg1l_plan*, int, const T*, T*, const double*, T*,          \
                                      cudaStream_t);                                                      \
    template int copy_impl<T>(const vd_qg1l_plan*, int, const T*, T*, int, cudaStream_t);                 \
    template int zero_impl<T>(long long, T*, cudaStream_t);                                               \
    template int h2uv_impl<T>(const vd_qg1l_plan*, int, const T*, T*, T*, cudaStream_t);                  \
    template int rhs_impl<T>(const vd_qg1l_plan*, int, const T*, const T*, const T*, T*, cudaStream_t);

VD_INST(float)
VD_INST(double)

}  // namespace vd
