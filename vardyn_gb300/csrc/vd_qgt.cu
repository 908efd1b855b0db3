// Overlapping-tile QG 1.5-layer model, forward (mapping/models/model_qg1l/
// jqgm.py, QgmWithTiles 1033-1376).
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

// PV -> SSH of one tile (jqgm.py:1149-1170): h = hb + the inversion of
// q - qb on the interior, the edge keeps hb
template <typename R>
__device__ void qgt_pv2h(const QgtGeom<R>& G, const R* q, const R* qb, const R* hb, const R* S, const R* lap,
                         R gf, R gfc2, R* A, R* B, R* h)
{
    const int T = G.T, n = G.n;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int p = e / n, s = e - p * n;
        const int o = (p + 1) * T + (s + 1);
        A[e] = q[o] - qb[o];
    }
    __syncthreads();
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
    for (int e = threadIdx.x; e < T * T; e += blockDim.x) {
        const int a = e / T, b = e - a * T;
        const bool in = a >= 1 && a <= T - 2 && b >= 1 && b <= T - 2;
        h[e] = hb[e] + (in ? A[(a - 1) * n + (b - 1)] : R(0));
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
    R r = acc / wsum[o];
    if (mdt) r -= mdt[o];
    h1[o] = r;
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
