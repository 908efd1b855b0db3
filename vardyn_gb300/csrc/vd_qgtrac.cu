// QG 1.5-layer model with passive tracers, forward
// (mapping/models/model_qg1l/jqgm.py, class Qgm_trac, 1551-2151).
//
// The SSH/PV part is the QG1.5L model of vd_qg1l.cu, used through its
// primitives (h2pv, h2uv, rhs, pv2h) on a plan without bathymetry. The tracers
// add three kernels:
// - k_trac_stage: tendency of every tracer plane (third-order upwind, own
//   diffusion, zero on land only) fused with the Runge-Kutta combination;
// - k_trac_bc: open boundaries or ring values, then relaxation to the
//   boundary field;
// - k_trac_prep / k_trac_final: land zeroing and MDT in, NaN on land and MDT
//   out (jqgm.py:2057-2139).
// The PV combination is k_rk_combine over the PV planes.
//
// Tracer planes are [batch][ntrac][ny][nx]; SSH/PV planes [batch][ny][nx].
// Every kernel is one thread per grid point with the window or tracer plane
// on blockIdx.z: the tracer model is a handful of HBM passes per stage, each
// bound by DRAM bandwidth, and its elliptic solve is the QG plan's.
#include "vd_internal.cuh"
#include "vd_qgtrac.cuh"
#include <initializer_list>

namespace vd {

static const dim3 kTB(32, 8);
static inline dim3 tgrid(int ny, int nx, int nz) { return dim3((nx + 31) / 32, (ny + 7) / 8, nz); }

template <typename T>
__global__ void k_trac_prep(int ny, int nx, int ntrac, const int8_t* __restrict__ mask, const T* __restrict__ h0,
                            const T* __restrict__ hb, const T* __restrict__ mdt, const T* __restrict__ c0,
                            const T* __restrict__ cb, T* __restrict__ h, T* __restrict__ hbm, T* __restrict__ c,
                            T* __restrict__ cbz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= nx || j >= ny) return;
    const long long fs = (long long)ny * nx, p = (long long)j * nx + i, o = b * fs + p;
    const T m = mdt ? mdt[p] : T(0);
    h[o] = mdt ? h0[o] + m : h0[o];
    hbm[o] = mdt ? hb[o] + m : hb[o];
    const bool land = mask[p] == 0;
    for (int t = 0; t < ntrac; ++t) {
        const long long ot = ((long long)b * ntrac + t) * fs + p;
        c[ot] = land ? T(0) : c0[ot];
        cbz[ot] = land ? T(0) : cb[ot];
    }
}

template <typename T>
__global__ void k_trac_stage(TracGeom G, int ntrac, const T* __restrict__ u, const T* __restrict__ v,
                             const T* __restrict__ cin, const T* __restrict__ cbase, T* __restrict__ cout,
                             T* __restrict__ acc, int mode, T a, T dt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;   // window * ntrac + tracer
    if (i >= G.nx || j >= G.ny) return;
    const long long fs = (long long)G.ny * G.nx, p = (long long)j * G.nx + i, o = z * fs + p;
    const long long ob = (long long)(z / ntrac) * fs;
    const T r = trac_rhs_point<T>(G, u + ob, v + ob, cin + z * fs, j, i);
    T ac = (mode == 2 || mode == 3) ? acc[o] : T(0);
    cout[o] = rk_combine<T>(mode, a, dt, r, cbase[o], &ac);
    if (mode == 1 || mode == 2) acc[o] = ac;
}

template <typename T>
__global__ void k_rk_combine(long long n, const T* __restrict__ r, const T* __restrict__ base, T* __restrict__ out,
                             T* __restrict__ acc, int mode, T a, T dt)
{
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    T ac = (mode == 2 || mode == 3) ? acc[o] : T(0);
    out[o] = rk_combine<T>(mode, a, dt, r[o], base[o], &ac);
    if (mode == 1 || mode == 2) acc[o] = ac;
}

template <typename T>
__global__ void k_trac_bc(TracGeom G, int ntrac, const T* __restrict__ u, const T* __restrict__ v,
                          const T* __restrict__ c0, const T* __restrict__ cb, const T* __restrict__ W,
                          T* __restrict__ c1)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (i >= G.nx || j >= G.ny) return;
    const long long fs = (long long)G.ny * G.nx, o = z * fs + (long long)j * G.nx + i;
    const long long ob = (long long)(z / ntrac) * fs;
    c1[o] = trac_bc_point<T>(G, u + ob, v + ob, c0 + z * fs, cb + z * fs, W, c1[o], j, i);
}

template <typename T>
__global__ void k_trac_final(int ny, int nx, int ntrac, const int8_t* __restrict__ mask, const T* __restrict__ h,
                             const T* __restrict__ mdt, const T* __restrict__ c, T* __restrict__ h1,
                             T* __restrict__ c1)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    if (i >= nx || j >= ny) return;
    const long long fs = (long long)ny * nx, p = (long long)j * nx + i, o = b * fs + p;
    const bool land = mask[p] == 0;
    const T nan = T(NAN);
    const T hv = land ? nan : h[o];
    h1[o] = mdt ? hv - mdt[p] : hv;
    for (int t = 0; t < ntrac; ++t) {
        const long long ot = ((long long)b * ntrac + t) * fs + p;
        c1[ot] = land ? nan : c[ot];
    }
}

static TracGeom trac_geom(const vd_qg1l_plan* p, const vd_qgtrac_desc* d)
{
    TracGeom G;
    G.ny = p->d.ny;
    G.nx = p->d.nx;
    G.cx = 1.0 / (6.0 * p->d.dx);
    G.cy = 1.0 / (6.0 * p->d.dy);
    G.hasK = d->has_Kdiffus_trac;
    G.Kx = d->has_Kdiffus_trac ? d->Kdiffus_trac / (p->d.dx * p->d.dx) : 0.0;
    G.Ky = d->has_Kdiffus_trac ? d->Kdiffus_trac / (p->d.dy * p->d.dy) : 0.0;
    G.rx = 0.5 * p->d.dt / p->d.dx;
    G.ry = 0.5 * p->d.dt / p->d.dy;
    G.obc = d->bc_obc;
    G.mask = p->d_mask;
    return G;
}

struct TracBufs {
    void *h, *hbm, *q, *qb, *u, *v, *us, *vs, *rq, *qs, *qacc, *qn, *hs, *zero;
    void *c, *cbz, *cs, *cs2, *cacc, *cn;
    void* pv2h_ws;
    size_t pv2h_bytes;
};

static size_t trac_layout(const vd_qg1l_plan* p, const vd_qgtrac_desc* d, int B, TracBufs* tb, char* base,
                          size_t cap)
{
    const size_t F = size_t(p->geom.fs) * elem_size(p->d.dtype);
    const size_t BF = size_t(B) * F, CF = size_t(B) * size_t(d->ntrac) * F;
    const size_t pv2h = spec_bytes(p, B) + 2 * 256;
    Arena ar{base, cap, 0};
    void** one[] = {&tb->h, &tb->hbm, &tb->q, &tb->qb, &tb->u, &tb->v, &tb->us, &tb->vs,
                    &tb->rq, &tb->qs, &tb->qacc, &tb->qn, &tb->hs, &tb->zero};
    void** many[] = {&tb->c, &tb->cbz, &tb->cs, &tb->cs2, &tb->cacc, &tb->cn};
    size_t need = 0;
    for (void** s : one) { *s = base ? ar.take(BF) : nullptr; need += (BF + 255) & ~size_t(255); }
    for (void** s : many) { *s = (base && CF) ? ar.take(CF) : nullptr; need += (CF + 255) & ~size_t(255); }
    tb->pv2h_ws = base ? ar.take(pv2h) : nullptr;
    tb->pv2h_bytes = pv2h;
    need += (pv2h + 255) & ~size_t(255);
    return need + 256;
}

template <typename T>
static int trac_stage(const vd_qg1l_plan* p, const TracGeom& G, int B, int nt, const T* u, const T* v,
                      const T* uq, const T* vq, const T* qin, const T* qbase, T* qout, T* qacc, T* rq,
                      const T* cin, const T* cbase, T* cout, T* cacc, int mode, double a, cudaStream_t st)
{
    int rc = vd_qg1l_rhs(p, B, uq, vq, qin, rq, st);
    if (rc) return rc;
    const long long n = (long long)B * p->geom.fs;
    k_rk_combine<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, rq, qbase, qout, qacc, mode, T(a),
                                                                  T(p->d.dt));
    VD_LAUNCH_CHECK();
    if (nt > 0) {
        k_trac_stage<T><<<tgrid(G.ny, G.nx, B * nt), kTB, 0, st>>>(G, nt, u, v, cin, cbase, cout, cacc, mode,
                                                                    T(a), T(p->d.dt));
        VD_LAUNCH_CHECK();
    }
    return VD_OK;
}

template <typename T>
static int trac_step(const vd_qg1l_plan* p, const vd_qgtrac_desc* d, int B, const T* h0, const T* c0, const T* hb,
                     const T* cb, int nstep, T* h1, T* c1, char* work, size_t work_bytes, cudaStream_t st)
{
    TracBufs tb;
    trac_layout(p, d, B, &tb, work, work_bytes);
    const int nt = d->ntrac;
    for (void* b : {tb.h, tb.hbm, tb.q, tb.qb, tb.u, tb.v, tb.us, tb.vs, tb.rq, tb.qs, tb.qacc, tb.qn, tb.hs, tb.zero,
                    tb.pv2h_ws})
        if (!b) return VD_ERR_WORKSPACE;
    if (nt > 0)
        for (void* b : {tb.c, tb.cbz, tb.cs, tb.cs2, tb.cacc, tb.cn})
            if (!b) return VD_ERR_WORKSPACE;
    const TracGeom G = trac_geom(p, d);
    const int ny = G.ny, nx = G.nx;
    const long long BF = (long long)B * p->geom.fs;
    T *h = (T*)tb.h, *hbm = (T*)tb.hbm, *q = (T*)tb.q, *qb = (T*)tb.qb, *u = (T*)tb.u, *v = (T*)tb.v;
    T *us = (T*)tb.us, *vs = (T*)tb.vs, *rq = (T*)tb.rq, *qs = (T*)tb.qs, *qacc = (T*)tb.qacc, *qn = (T*)tb.qn;
    T *hs = (T*)tb.hs, *zero = (T*)tb.zero;
    T *c = (T*)tb.c, *cbz = (T*)tb.cbz, *cs = (T*)tb.cs, *cs2 = (T*)tb.cs2, *cacc = (T*)tb.cacc, *cn = (T*)tb.cn;
    const T* mdt = (const T*)d->mdt;
    const T* W = (const T*)d->wbc;
    int rc;

    k_trac_prep<T><<<tgrid(ny, nx, B), kTB, 0, st>>>(ny, nx, nt, p->d_mask, h0, hb, mdt, c0, cb, h, hbm, c, cbz);
    VD_LAUNCH_CHECK();
    if (!d->advect_pv) VD_CUDA_TRY(cudaMemsetAsync(zero, 0, BF * sizeof(T), st));
    if ((rc = vd_qg1l_h2pv(p, B, h, hbm, q, st))) return rc;
    if ((rc = vd_qg1l_h2pv(p, B, hbm, hbm, qb, st))) return rc;

    // PV tendency velocities: the geostrophic ones, or zero when the PV is
    // not advected (jqgm.py:1806-1815: only its diffusion remains)
    auto uq = [&](const T* uu) { return d->advect_pv ? uu : (const T*)zero; };
    auto solve_vel = [&](const T* qq, T* hh, T* uu, T* vv) {
        int r = vd_qg1l_pv2h(p, B, qq, hbm, qb, hh, tb.pv2h_ws, tb.pv2h_bytes, st);
        if (r) return r;
        return vd_qg1l_h2uv(p, B, hh, uu, vv, st);
    };

    for (int n = 0; n < nstep; ++n) {
        if ((rc = vd_qg1l_h2uv(p, B, h, u, v, st))) return rc;
        switch (d->time_scheme) {
        case VD_EULER:
            rc = trac_stage<T>(p, G, B, nt, u, v, uq(u), uq(v), q, q, qn, nullptr, rq, c, c, cn, nullptr, 0, 1.0,
                               st);
            if (rc) return rc;
            break;
        case VD_RK2:
            rc = trac_stage<T>(p, G, B, nt, u, v, uq(u), uq(v), q, q, qs, nullptr, rq, c, c, cs, nullptr, 0, 0.5,
                               st);
            if (rc || (rc = solve_vel(qs, hs, us, vs))) return rc;
            rc = trac_stage<T>(p, G, B, nt, us, vs, uq(us), uq(vs), qs, q, qn, nullptr, rq, cs, c, cn, nullptr, 0,
                               1.0, st);
            if (rc) return rc;
            break;
        default: {   // VD_RK4, classical
            rc = trac_stage<T>(p, G, B, nt, u, v, uq(u), uq(v), q, q, qs, qacc, rq, c, c, cs, cacc, 1, 0.5, st);
            if (rc) return rc;
            // stages 2 and 3 read the tracer state of the previous stage with a
            // stencil, so they alternate between cs and cs2; the PV combination
            // is pointwise and rewrites qs in place after rhs has read it
            T* cprev = cs;
            T* cnext = cs2;
            for (int s = 2; s <= 3; ++s) {
                if ((rc = solve_vel(qs, hs, us, vs))) return rc;
                rc = trac_stage<T>(p, G, B, nt, us, vs, uq(us), uq(vs), qs, q, qs, qacc, rq, cprev, c, cnext, cacc,
                                   2, s == 2 ? 0.5 : 1.0, st);
                if (rc) return rc;
                T* t = cprev;
                cprev = cnext;
                cnext = t;
            }
            if ((rc = solve_vel(qs, hs, us, vs))) return rc;
            rc = trac_stage<T>(p, G, B, nt, us, vs, uq(us), uq(vs), qs, q, qn, qacc, rq, cprev, c, cn, cacc, 3, 1.0,
                               st);
            if (rc) return rc;
        }
        }
        if ((rc = vd_qg1l_pv2h(p, B, qn, hbm, qb, h, tb.pv2h_ws, tb.pv2h_bytes, st))) return rc;
        if (nt > 0) {
            k_trac_bc<T><<<tgrid(ny, nx, B * nt), kTB, 0, st>>>(G, nt, u, v, c, cbz, W, cn);
            VD_LAUNCH_CHECK();
        }
        T* t = q;
        q = qn;
        qn = t;
        t = c;
        c = cn;
        cn = t;
    }
    k_trac_final<T><<<tgrid(ny, nx, B), kTB, 0, st>>>(ny, nx, nt, p->d_mask, h, mdt, c, h1, c1);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

}  // namespace vd

using namespace vd;

static bool trac_desc_ok(const vd_qg1l_plan* p, const vd_qgtrac_desc* d)
{
    if (!p || !d || d->ntrac < 0) return false;
    if (d->time_scheme != VD_EULER && d->time_scheme != VD_RK2 && d->time_scheme != VD_RK4) return false;
    if (p->d_fB) return false;   // the tracer model has no bathymetry term
    if (d->ntrac > 0 && !d->wbc) return false;
    return true;
}

extern "C" size_t vd_qgtrac_workspace_bytes(const vd_qg1l_plan* p, const vd_qgtrac_desc* d, int batch)
{
    if (!trac_desc_ok(p, d) || batch <= 0) return 0;
    TracBufs tb;
    return trac_layout(p, d, batch, &tb, nullptr, 0);
}

extern "C" vd_status vd_qgtrac_step(const vd_qg1l_plan* p, const vd_qgtrac_desc* d, int batch, const void* h0,
                                    const void* c0, const void* hb, const void* cb, int nstep, void* h1, void* c1,
                                    void* work, size_t work_bytes, void* stream)
{
    if (!trac_desc_ok(p, d) || batch <= 0 || nstep < 0 || !h0 || !hb || !h1 || !work) return VD_ERR_ARG;
    if ((long long)batch * (d->ntrac > 0 ? d->ntrac : 1) > 65535) return VD_ERR_UNSUPPORTED;   // grid z
    if (d->ntrac > 0 && (!c0 || !cb || !c1)) return VD_ERR_ARG;
    if (work_bytes < vd_qgtrac_workspace_bytes(p, d, batch)) return VD_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    if (p->d.dtype == VD_F32)
        return trac_step<float>(p, d, batch, (const float*)h0, (const float*)c0, (const float*)hb, (const float*)cb,
                                nstep, (float*)h1, (float*)c1, (char*)work, work_bytes, st);
    return trac_step<double>(p, d, batch, (const double*)h0, (const double*)c0, (const double*)hb,
                             (const double*)cb, nstep, (double*)h1, (double*)c1, (char*)work, work_bytes, st);
}
