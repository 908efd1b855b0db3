// C ABI entry points of libvardyn_gb300 (declared in include/vardyn_gb300.h).
#include "vd_internal.cuh"
#include <algorithm>
#include <vector>
#include <new>
#include <cstring>

#include <atomic>

namespace vd {

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

size_t elem_size(int dtype) { return dtype == VD_F64 ? 8 : 4; }

template <typename T>
int advance_impl(const vd_qg1l_plan*, int, T*, int, int, int, const T*, const T*, T*, Arena&, cudaStream_t);
template <typename T>
int forward_nostore(const vd_qg1l_plan*, int, T*, T*, int, const T*, const T*, T*, Arena&, cudaStream_t, bool);
template <typename T>
int advance_adj_impl(const vd_qg1l_plan*, int, const T*, int, int, int, T*, T*, Arena&, cudaStream_t);
template <typename T>
int init_state_impl(const vd_qg1l_plan*, int, int, const T*, const T*, T*, T*, T*, cudaStream_t);
template <typename T>
int init_state_adj_impl(const vd_qg1l_plan*, int, const T*, const T*, T*, cudaStream_t);
template <typename T>
int finalize_impl(const vd_qg1l_plan*, int, const T*, const T*, const T*, double, const double*, int, T*,
                  cudaStream_t);
template <typename T>
int finalize_adj_impl(const vd_qg1l_plan*, int, const T*, T*, const double*, T*, cudaStream_t);
template <typename T>
int copy_impl(const vd_qg1l_plan*, int, const T*, T*, int, cudaStream_t);
template <typename T>
int zero_impl(long long, T*, cudaStream_t);
template <typename T>
int h2uv_impl(const vd_qg1l_plan*, int, const T*, T*, T*, cudaStream_t);
template <typename T>
int rhs_impl(const vd_qg1l_plan*, int, const T*, const T*, const T*, T*, cudaStream_t);

static void butcher(int scheme, double dt, int* S, double A[4][4], double b[4])
{
    for (int i = 0; i < 4; ++i) {
        b[i] = 0.0;
        for (int j = 0; j < 4; ++j) A[i][j] = 0.0;
    }
    switch (scheme) {
    case VD_EULER:
        *S = 1; b[0] = dt; break;
    case VD_RK2:
        *S = 2; A[1][0] = 0.5 * dt; b[1] = dt; break;
    case VD_RK3:
        *S = 3; A[1][0] = 0.5 * dt; A[2][0] = -dt; A[2][1] = 2 * dt;
        b[0] = dt / 6; b[1] = 4 * dt / 6; b[2] = dt / 6; break;
    default:   // VD_RK4
        *S = 4; A[1][0] = 0.5 * dt; A[2][1] = 0.5 * dt; A[3][2] = dt;
        b[0] = dt / 6; b[1] = dt / 3; b[2] = dt / 3; b[3] = dt / 6; break;
    }
}

// Mask of jqgm.py:178-194 for a domain without land.
static void default_mask(int ny, int nx, std::vector<int8_t>& m)
{
    m.assign(size_t(ny) * nx, 3);
    auto at = [&](int j, int i) -> int8_t& { return m[size_t(j) * nx + i]; };
    for (int i = 0; i < nx; ++i) { at(0, i) = 1; at(ny - 1, i) = 1; }
    for (int j = 0; j < ny; ++j) { at(j, 0) = 1; at(j, nx - 1) = 1; }
    for (int i = 1; i < nx - 1; ++i) { at(1, i) = 2; at(ny - 2, i) = 2; at(ny - 3, i) = 2; }
    for (int j = 1; j < ny - 1; ++j) { at(j, 1) = 2; at(j, nx - 2) = 2; at(j, nx - 3) = 2; }
}

template <typename T>
static int upload_field(const double* h, size_t n, void** d)
{
    std::vector<T> tmp(h, h + n);
    VD_CUDA_TRY(cudaMalloc(d, n * sizeof(T)));
    VD_CUDA_TRY(cudaMemcpy(*d, tmp.data(), n * sizeof(T), cudaMemcpyHostToDevice));
    return VD_OK;
}

static int nk_count(const vd_qg1l_plan* p)
{
    int c = 0;
    for (int s = 0; s < p->nstage - 1; ++s) {
        bool need = p->b[s] != 0.0;
        for (int t = s + 2; t < p->nstage; ++t) need = need || p->A[t][s] != 0.0;
        c += need;
    }
    return c;
}

}  // namespace vd

using namespace vd;

#define VD_DISPATCH(p, FN, ...)                                              \
    ((p)->d.dtype == VD_F32 ? FN<float>(__VA_ARGS__) : FN<double>(__VA_ARGS__))

extern "C" long long vd_launch_count(void) { return g_launches.load(); }

namespace vd {
template <typename T>
int dst_x_only(const vd_qg1l_plan*, int, const T*, T*, int, T*, cudaStream_t);
}

namespace vd {
template <typename T>
int tridiag_only(const vd_qg1l_plan*, int, T*, cudaStream_t);
}

extern "C" vd_status vd_qg1l_tridiag_y(const vd_qg1l_plan* p, int B, void* spec, void* stream)
{
    if (!p || B <= 0 || !spec) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32 ? tridiag_only<float>(p, B, (float*)spec, st)
                                : tridiag_only<double>(p, B, (double*)spec, st);
}

extern "C" size_t vd_qg1l_spec_bytes(const vd_qg1l_plan* p, int batch)
{
    return (p && batch > 0) ? spec_bytes(p, batch) : 0;
}

extern "C" vd_status vd_qg1l_dst_x(const vd_qg1l_plan* p, int B, const void* field, void* spec, int inverse,
                                   void* out, void* stream)
{
    if (!p || B <= 0 || !spec || inverse < 0 || inverse > 2 || (inverse != 1 && !field) || (inverse && !out))
        return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? dst_x_only<float>(p, B, (const float*)field, (float*)spec, inverse, (float*)out, st)
               : dst_x_only<double>(p, B, (const double*)field, (double*)spec, inverse, (double*)out, st);
}

extern "C" const char* vd_version(void)
{
    return "vardyn_gb300 0.1 (sm_103a; QG1.5L step/TL/adjoint, DST-x + tridiagonal-y Helmholtz, obs misfit)";
}

extern "C" vd_status vd_qg1l_plan_create(vd_qg1l_plan** out, const vd_qg1l_desc* d)
{
    if (!out || !d) return VD_ERR_ARG;
    *out = nullptr;
    if (d->ny < 8 || d->nx < 8) return VD_ERR_UNSUPPORTED;
    if (d->nx - 2 > 4096 || d->ny - 2 > 4096) return VD_ERR_UNSUPPORTED;
    if (d->dtype != VD_F32 && d->dtype != VD_F64) return VD_ERR_ARG;
    if (d->time_scheme < VD_EULER || d->time_scheme > VD_RK4) return VD_ERR_ARG;
    if (d->dst_engine != VD_DST_AUTO && d->dst_engine != VD_DST_FMA) return VD_ERR_ARG;
    if (!(d->dx > 0) || !(d->dy > 0) || !(d->f != 0) || !(d->c > 0) || !(d->g != 0)) return VD_ERR_ARG;
    vd_qg1l_plan* p = new (std::nothrow) vd_qg1l_plan();   // value-initialised: every member zero
    if (!p) return VD_ERR_ARG;
    p->d = *d;
    p->d.mask_host = nullptr;
    p->d.beta_host = nullptr;
    p->d.fbathy_host = nullptr;
    cudaGetDevice(&p->device);
    butcher(d->time_scheme, d->dt, &p->nstage, p->A, p->b);

    const int ny = d->ny, nx = d->nx;
    const size_t N = size_t(ny) * nx;
    std::vector<int8_t> mask;
    if (d->mask_host) mask.assign(d->mask_host, d->mask_host + N);
    else default_mask(ny, nx, mask);
    // The stencils of a tendency point (mask 3) reach two cells out: such
    // points must lie in rows/columns 2 .. n-3 (the reference's mask keeps
    // them in 2 .. n-4).
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int8_t m = mask[size_t(j) * nx + i];
            if (m < 0 || m > 3) { delete p; return VD_ERR_ARG; }
            if (m == 3 && (j < 2 || j > ny - 3 || i < 2 || i > nx - 3)) { delete p; return VD_ERR_ARG; }
        }
    int rc = VD_OK;
    auto fail = [&](int code) { vd_qg1l_plan_destroy(p); return code; };
    if (cudaMalloc(&p->d_mask, N) != cudaSuccess) return fail(VD_ERR_CUDA);
    if (cudaMemcpy(p->d_mask, mask.data(), N, cudaMemcpyHostToDevice) != cudaSuccess) return fail(VD_ERR_CUDA);
    if (d->beta_host) {
        rc = d->dtype == VD_F32 ? upload_field<float>(d->beta_host, N, &p->d_beta)
                                : upload_field<double>(d->beta_host, N, &p->d_beta);
        if (rc) return fail(rc);
    }
    if (d->fbathy_host) {
        rc = d->dtype == VD_F32 ? upload_field<float>(d->fbathy_host, N, &p->d_fB)
                                : upload_field<double>(d->fbathy_host, N, &p->d_fB);
        if (rc) return fail(rc);
    }
    QGGeom& G = p->geom;
    G.ny = ny; G.nx = nx; G.fs = (long long)N;
    G.gf = d->g / d->f;
    G.gfc2 = d->g * d->f / (d->c * d->c);
    G.cu = -d->g / d->f / (4 * d->dy);
    G.cv = d->g / d->f / (4 * d->dx);
    G.cx = 1.0 / (6 * d->dx);
    G.cy = 1.0 / (6 * d->dy);
    G.idx2 = 1.0 / (d->dx * d->dx);
    G.idy2 = 1.0 / (d->dy * d->dy);
    G.hasK = d->has_Kdiffus ? 1 : 0;
    G.Kx = d->has_Kdiffus ? d->Kdiffus / (d->dx * d->dx) : 0.0;
    G.Ky = d->has_Kdiffus ? d->Kdiffus / (d->dy * d->dy) : 0.0;
    G.mask = p->d_mask;
    G.beta = p->d_beta;
    G.fB = p->d_fB;
    if ((rc = build_dst_tables(p))) return fail(rc);
    if (d->dtype == VD_F32 && d->dst_engine == VD_DST_AUTO) {
        if ((rc = build_tc_images(p))) return fail(rc);
    }
    *out = p;
    return VD_OK;
}

extern "C" vd_status vd_qg1l_plan_destroy(vd_qg1l_plan* p)
{
    if (!p) return VD_OK;
    free_tc_images(p);
    free_dst_tables(p);
    cudaFree(p->d_mask);
    cudaFree(p->d_beta);
    cudaFree(p->d_fB);
    delete p;
    return VD_OK;
}

extern "C" vd_status vd_qg1l_set_schedule(vd_qg1l_plan* p, const vd_qg1l_schedule* s)
{
    if (!p || !s) return VD_ERR_ARG;
    if (s->engine < 0 || s->engine > 2) return VD_ERR_ARG;
    for (int g : {s->tc_group_fwd, s->tc_group_inv})
        if (g != 0 && g != 1 && g != 2 && g != 4 && g != 8) return VD_ERR_ARG;
    if (s->fma_rows != 0 && s->fma_rows != 16 && s->fma_rows != 32 && s->fma_rows != 64) return VD_ERR_ARG;
    if (s->tridiag_rows != 0 && s->tridiag_rows != 8 && s->tridiag_rows != 16 && s->tridiag_rows != 32)
        return VD_ERR_ARG;
    if (s->tridiag_lean != 0 && s->tridiag_lean != 1) return VD_ERR_ARG;
    if (s->tridiag_lean == 1 && p->d.dtype != VD_F32) return VD_ERR_UNSUPPORTED;
    if (s->stencil_loads != 0 && s->stencil_loads != 1) return VD_ERR_ARG;
    if (s->engine == 2 && !p->dst.tc) return VD_ERR_UNSUPPORTED;
    if (s->fma_rows) {
        const size_t es = elem_size(p->d.dtype);
        if (s->fma_rows == 64 && es == 8) return VD_ERR_UNSUPPORTED;
        const size_t c = (size_t)s->fma_rows;
        const size_t smem = (2 * (size_t)p->dst.kpad * c + std::max<size_t>(2 * DST_KC * DST_NC, c * DST_NC)) * es;
        if (smem > 200 * 1024) return VD_ERR_UNSUPPORTED;
    }
    p->sched = *s;
    return VD_OK;
}

extern "C" vd_status vd_qg1l_get_schedule(const vd_qg1l_plan* p, vd_qg1l_schedule* s)
{
    if (!p || !s) return VD_ERR_ARG;
    *s = p->sched;
    return VD_OK;
}

extern "C" int vd_qg1l_nstage(const vd_qg1l_plan* p) { return p ? p->nstage : 0; }

extern "C" size_t vd_qg1l_traj_bytes(const vd_qg1l_plan* p, int batch, int nstep)
{
    if (!p || batch <= 0 || nstep < 0) return 0;
    return (size_t(nstep) * p->nstage + 1) * 2 * size_t(batch) * p->geom.fs * elem_size(p->d.dtype);
}

extern "C" size_t vd_qg1l_workspace_bytes(const vd_qg1l_plan* p, int B)
{
    if (!p || B <= 0) return 0;
    const size_t F = size_t(p->geom.fs) * elem_size(p->d.dtype);
    const int S = p->nstage, nk = nk_count(p);
    // the low part of the compensated PV state (float32 plans): one field
    // per forward field
    auto fwd = [&](int nf) { return (nk + 2 * (S - 1) + 3) * nf * F + spec_bytes(p, nf); };
    const size_t step = 3 * B * F + fwd(B);
    const size_t tgl = 5 * B * F + fwd(2 * B);
    const size_t adv_part = nk * B * F + spec_bytes(p, B);
    const size_t adj_part = (2 + S + 7) * B * F + spec_bytes(p, B);
    const size_t adj = 2 * B * F + (adv_part > adj_part ? adv_part : adj_part) + 2 * B * F;
    size_t m = step > tgl ? step : tgl;
    m = m > adj ? m : adj;
    return m + 64 * 256;
}

static inline long long fb_elems(const vd_qg1l_plan* p, int B) { return (long long)B * p->geom.fs; }

extern "C" vd_status vd_qg1l_h2pv(const vd_qg1l_plan* p, int B, const void* h, const void* hb, void* q, void* stream)
{
    if (!p || B <= 0 || !h || !hb || !q) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? init_state_impl<float>(p, B, B, (const float*)h, (const float*)hb, (float*)q, nullptr, nullptr, st)
               : init_state_impl<double>(p, B, B, (const double*)h, (const double*)hb, (double*)q, nullptr, nullptr,
                                         st);
}

extern "C" vd_status vd_qg1l_h2uv(const vd_qg1l_plan* p, int B, const void* h, void* u, void* v, void* stream)
{
    if (!p || B <= 0 || !h || !u || !v) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32 ? h2uv_impl<float>(p, B, (const float*)h, (float*)u, (float*)v, st)
                                : h2uv_impl<double>(p, B, (const double*)h, (double*)u, (double*)v, st);
}

extern "C" vd_status vd_qg1l_rhs(const vd_qg1l_plan* p, int B, const void* u, const void* v, const void* q,
                                 void* r, void* stream)
{
    if (!p || B <= 0 || !u || !v || !q || !r) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? rhs_impl<float>(p, B, (const float*)u, (const float*)v, (const float*)q, (float*)r, st)
               : rhs_impl<double>(p, B, (const double*)u, (const double*)v, (const double*)q, (double*)r, st);
}

template <typename T>
static int pv2h_t(const vd_qg1l_plan* p, int B, const T* q, const T* hb, const T* qb, T* h, Arena& ws,
                  cudaStream_t st)
{
    T* spec = (T*)ws.take(spec_bytes(p, B));
    if (!spec) return VD_ERR_WORKSPACE;
    SolveArgs a;
    a.src = q; a.sub = qb; a.sub_batches = qb ? B : 0;
    a.out = h; a.add = hb; a.add_batches = hb ? B : 0; a.epi = EPI_H;
    int rc = helmholtz_solve<T>(p, B, a, spec, st);
    if (rc) return rc;
    return finalize_impl<T>(p, B, h, hb, nullptr, 0.0, nullptr, 0, h, st);
}

extern "C" vd_status vd_qg1l_pv2h(const vd_qg1l_plan* p, int B, const void* q, const void* hb, const void* qb,
                                  void* h, void* work, size_t work_bytes, void* stream)
{
    if (!p || B <= 0 || !q || !h || !work) return VD_ERR_ARG;
    Arena ws{(char*)work, work_bytes, 0};
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? pv2h_t<float>(p, B, (const float*)q, (const float*)hb, (const float*)qb, (float*)h, ws, st)
               : pv2h_t<double>(p, B, (const double*)q, (const double*)hb, (const double*)qb, (double*)h, ws, st);
}

// Low part of the compensated PV state: float32 plans carry one, float64
// plans step with the reference's plain arithmetic.
template <typename T>
static int take_qlo(const vd_qg1l_plan* p, long long n, Arena& ws, T** qlo)
{
    *qlo = nullptr;
    if (p->d.dtype != VD_F32) return VD_OK;
    *qlo = (T*)ws.take(n * sizeof(T));
    return *qlo ? VD_OK : VD_ERR_WORKSPACE;
}

template <typename T>
static int step_t(const vd_qg1l_plan* p, int B, const T* h0, const T* hb, int nstep, T* hout, T* traj, Arena& ws,
                  cudaStream_t st)
{
    const long long fb = fb_elems(p, B);
    T* qb = (T*)ws.take(fb * sizeof(T));
    if (!qb) return VD_ERR_WORKSPACE;
    T* qlo;
    int rc;
    if ((rc = take_qlo<T>(p, fb, ws, &qlo))) return rc;
    if (traj) {
        T* h = traj;
        T* q = traj + fb;
        VD_CUDA_TRY(cudaMemcpyAsync(h, h0, fb * sizeof(T), cudaMemcpyDeviceToDevice, st));
        if ((rc = init_state_impl<T>(p, B, B, h, hb, q, qb, qlo, st))) return rc;
        if ((rc = advance_impl<T>(p, B, traj, nstep, 0, nstep, hb, qb, qlo, ws, st))) return rc;
        const T* hN = traj + (long long)nstep * p->nstage * 2 * fb;
        return finalize_impl<T>(p, B, hN, hb, nullptr, 0.0, nullptr, 1, hout, st);
    }
    T* h = (T*)ws.take(fb * sizeof(T));
    T* q = (T*)ws.take(fb * sizeof(T));
    if (!h || !q) return VD_ERR_WORKSPACE;
    VD_CUDA_TRY(cudaMemcpyAsync(h, h0, fb * sizeof(T), cudaMemcpyDeviceToDevice, st));
    if ((rc = init_state_impl<T>(p, B, B, h, hb, q, qb, qlo, st))) return rc;
    if ((rc = forward_nostore<T>(p, B, h, q, nstep, hb, qb, qlo, ws, st, false))) return rc;
    return finalize_impl<T>(p, B, h, hb, nullptr, 0.0, nullptr, 1, hout, st);
}

extern "C" vd_status vd_qg1l_step(const vd_qg1l_plan* p, int B, const void* h0, const void* hb, int nstep,
                                  void* h_out, void* traj, void* work, size_t work_bytes, void* stream)
{
    if (!p || B <= 0 || nstep < 0 || !h0 || !hb || !h_out || !work) return VD_ERR_ARG;
    if (work_bytes < vd_qg1l_workspace_bytes(p, B)) return VD_ERR_WORKSPACE;
    Arena ws{(char*)work, work_bytes, 0};
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? step_t<float>(p, B, (const float*)h0, (const float*)hb, nstep, (float*)h_out, (float*)traj, ws, st)
               : step_t<double>(p, B, (const double*)h0, (const double*)hb, nstep, (double*)h_out, (double*)traj,
                                ws, st);
}

template <typename T>
static int step_tgl_t(const vd_qg1l_plan* p, int B, const T* dh0, const T* h0, const T* hb, int nstep, T* dhout,
                      Arena& ws, cudaStream_t st)
{
    const long long fb = fb_elems(p, B);
    T* h = (T*)ws.take(2 * fb * sizeof(T));
    T* q = (T*)ws.take(2 * fb * sizeof(T));
    T* qb = (T*)ws.take(fb * sizeof(T));
    if (!h || !q || !qb) return VD_ERR_WORKSPACE;
    T* qlo;
    int rc;
    if ((rc = take_qlo<T>(p, 2 * fb, ws, &qlo))) return rc;
    VD_CUDA_TRY(cudaMemcpyAsync(h, h0, fb * sizeof(T), cudaMemcpyDeviceToDevice, st));
    VD_CUDA_TRY(cudaMemcpyAsync(h + fb, dh0, fb * sizeof(T), cudaMemcpyDeviceToDevice, st));
    if ((rc = init_state_impl<T>(p, 2 * B, B, h, hb, q, qb, qlo, st))) return rc;
    if ((rc = forward_nostore<T>(p, 2 * B, h, q, nstep, hb, qb, qlo, ws, st, true))) return rc;
    return finalize_impl<T>(p, B, h + fb, nullptr, nullptr, 0.0, nullptr, 2, dhout, st);
}

extern "C" vd_status vd_qg1l_step_tgl(const vd_qg1l_plan* p, int B, const void* dh0, const void* h0,
                                      const void* hb, int nstep, void* dh_out, void* work, size_t work_bytes,
                                      void* stream)
{
    if (!p || B <= 0 || nstep < 0 || !dh0 || !h0 || !hb || !dh_out || !work) return VD_ERR_ARG;
    if (work_bytes < vd_qg1l_workspace_bytes(p, B)) return VD_ERR_WORKSPACE;
    Arena ws{(char*)work, work_bytes, 0};
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? step_tgl_t<float>(p, B, (const float*)dh0, (const float*)h0, (const float*)hb, nstep,
                                   (float*)dh_out, ws, st)
               : step_tgl_t<double>(p, B, (const double*)dh0, (const double*)h0, (const double*)hb, nstep,
                                    (double*)dh_out, ws, st);
}

template <typename T>
static int step_adj_t(const vd_qg1l_plan* p, int B, const T* adh1, const T* h0, const T* hb, int nstep, T* adhout,
                      T* traj, int traj_ready, Arena& ws, cudaStream_t st)
{
    const long long fb = fb_elems(p, B);
    int rc;
    T* adh = (T*)ws.take(fb * sizeof(T));
    T* adq = (T*)ws.take(fb * sizeof(T));
    if (!adh || !adq) return VD_ERR_WORKSPACE;
    if (!traj_ready) {
        T* qb = (T*)ws.take(fb * sizeof(T));
        if (!qb) return VD_ERR_WORKSPACE;
        T* qlo;
        if ((rc = take_qlo<T>(p, fb, ws, &qlo))) return rc;
        VD_CUDA_TRY(cudaMemcpyAsync(traj, h0, fb * sizeof(T), cudaMemcpyDeviceToDevice, st));
        if ((rc = init_state_impl<T>(p, B, B, traj, hb, traj + fb, qb, qlo, st))) return rc;
        Arena sub = ws;
        if ((rc = advance_impl<T>(p, B, traj, nstep, 0, nstep, hb, qb, qlo, sub, st))) return rc;
    }
    if ((rc = copy_impl<T>(p, B, adh1, adh, 1, st))) return rc;
    if ((rc = zero_impl<T>(fb, adq, st))) return rc;
    if ((rc = advance_adj_impl<T>(p, B, traj, nstep, 0, nstep, adh, adq, ws, st))) return rc;
    if ((rc = init_state_adj_impl<T>(p, B, traj, adq, adh, st))) return rc;
    VD_CUDA_TRY(cudaMemcpyAsync(adhout, adh, fb * sizeof(T), cudaMemcpyDeviceToDevice, st));
    return VD_OK;
}

extern "C" vd_status vd_qg1l_step_adj(const vd_qg1l_plan* p, int B, const void* adh1, const void* h0,
                                      const void* hb, int nstep, void* adh_out, void* traj, int traj_ready,
                                      void* work, size_t work_bytes, void* stream)
{
    if (!p || B <= 0 || nstep < 0 || !adh1 || !h0 || !hb || !adh_out || !traj || !work) return VD_ERR_ARG;
    if (work_bytes < vd_qg1l_workspace_bytes(p, B)) return VD_ERR_WORKSPACE;
    Arena ws{(char*)work, work_bytes, 0};
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? step_adj_t<float>(p, B, (const float*)adh1, (const float*)h0, (const float*)hb, nstep,
                                   (float*)adh_out, (float*)traj, traj_ready, ws, st)
               : step_adj_t<double>(p, B, (const double*)adh1, (const double*)h0, (const double*)hb, nstep,
                                    (double*)adh_out, (double*)traj, traj_ready, ws, st);
}

namespace vd {
template <typename T>
int rk_stage_impl(const vd_qg1l_plan*, int, const T*, const T*, const T*, int, const T* const*, const double*,
                  double, T*, T*, cudaStream_t);
template <typename T>
int rk_stage_adj_impl(const vd_qg1l_plan*, int, const T*, const T*, int, const T* const*, const double*, int,
                      const T* const*, T*, T*, cudaStream_t);
}

extern "C" vd_status vd_qg1l_rk_stage(const vd_qg1l_plan* p, int B, const void* hs, const void* qs, const void* qbase,
                                      int nk, const void* const* k, const double* c, double cself, void* k_out,
                                      void* q_out, void* stream)
{
    if (!p || B <= 0 || !hs || !qs || !qbase || !q_out || nk < 0 || nk > 4 || (nk && (!k || !c))) return VD_ERR_ARG;
    for (int t = 0; t < nk; ++t)
        if (!k[t]) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? rk_stage_impl<float>(p, B, (const float*)hs, (const float*)qs, (const float*)qbase, nk,
                                      (const float* const*)k, c, cself, (float*)k_out, (float*)q_out, st)
               : rk_stage_impl<double>(p, B, (const double*)hs, (const double*)qs, (const double*)qbase, nk,
                                       (const double* const*)k, c, cself, (double*)k_out, (double*)q_out, st);
}

extern "C" vd_status vd_qg1l_rk_stage_adj(const vd_qg1l_plan* p, int B, const void* hs, const void* qs, int ng,
                                          const void* const* g, const double* c, int nacc, const void* const* acc,
                                          void* adq_out, void* adh_out, void* stream)
{
    if (!p || B <= 0 || !hs || !qs || !adq_out || !adh_out || ng < 0 || ng > 4 || nacc < 0 || nacc > 4 ||
        (ng && (!g || !c)) || (nacc && !acc))
        return VD_ERR_ARG;
    for (int t = 0; t < ng; ++t)
        if (!g[t]) return VD_ERR_ARG;
    for (int t = 0; t < nacc; ++t)
        if (!acc[t]) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? rk_stage_adj_impl<float>(p, B, (const float*)hs, (const float*)qs, ng, (const float* const*)g, c,
                                          nacc, (const float* const*)acc, (float*)adq_out, (float*)adh_out, st)
               : rk_stage_adj_impl<double>(p, B, (const double*)hs, (const double*)qs, ng, (const double* const*)g,
                                           c, nacc, (const double* const*)acc, (double*)adq_out, (double*)adh_out,
                                           st);
}

extern "C" vd_status vd_qg1l_init_state(const vd_qg1l_plan* p, int B, const void* h, const void* hb, void* q,
                                        void* qb, void* qlo, void* stream)
{
    if (!p || B <= 0 || !h || !hb || !q) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? init_state_impl<float>(p, B, B, (const float*)h, (const float*)hb, (float*)q, (float*)qb,
                                        (float*)qlo, st)
               : init_state_impl<double>(p, B, B, (const double*)h, (const double*)hb, (double*)q, (double*)qb,
                                         (double*)qlo, st);
}

extern "C" vd_status vd_qg1l_advance(const vd_qg1l_plan* p, int B, void* traj, int traj_steps, int first_step,
                                     int nstep, const void* hb, const void* qb, void* qlo, void* work,
                                     size_t work_bytes, void* stream)
{
    // hb == NULL / qb == NULL mean a zero background SSH / PV: the solves then
    // skip the addition / subtraction. qlo == NULL steps with plain arithmetic.
    if (!p || B <= 0 || !traj || !work) return VD_ERR_ARG;
    Arena ws{(char*)work, work_bytes, 0};
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? advance_impl<float>(p, B, (float*)traj, traj_steps, first_step, nstep, (const float*)hb,
                                     (const float*)qb, (float*)qlo, ws, st)
               : advance_impl<double>(p, B, (double*)traj, traj_steps, first_step, nstep, (const double*)hb,
                                      (const double*)qb, (double*)qlo, ws, st);
}

extern "C" vd_status vd_qg1l_advance_adj(const vd_qg1l_plan* p, int B, const void* traj, int traj_steps,
                                         int first_step, int nstep, void* adh, void* adq, void* work,
                                         size_t work_bytes, void* stream)
{
    if (!p || B <= 0 || !traj || !adh || !adq || !work) return VD_ERR_ARG;
    Arena ws{(char*)work, work_bytes, 0};
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? advance_adj_impl<float>(p, B, (const float*)traj, traj_steps, first_step, nstep, (float*)adh,
                                         (float*)adq, ws, st)
               : advance_adj_impl<double>(p, B, (const double*)traj, traj_steps, first_step, nstep, (double*)adh,
                                          (double*)adq, ws, st);
}

extern "C" vd_status vd_qg1l_init_state_adj(const vd_qg1l_plan* p, int B, const void* h, const void* adq,
                                            void* adh, void* stream)
{
    if (!p || B <= 0 || !h || !adq || !adh) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? init_state_adj_impl<float>(p, B, (const float*)h, (const float*)adq, (float*)adh, st)
               : init_state_adj_impl<double>(p, B, (const double*)h, (const double*)adq, (double*)adh, st);
}

extern "C" vd_status vd_qg1l_finalize(const vd_qg1l_plan* p, int B, const void* h, const void* hb,
                                      const void* forcing, double coef, void* h_out, void* stream)
{
    if (!p || B <= 0 || !h || !h_out) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? finalize_impl<float>(p, B, (const float*)h, (const float*)hb, (const float*)forcing, coef, nullptr,
                                      1, (float*)h_out, st)
               : finalize_impl<double>(p, B, (const double*)h, (const double*)hb, (const double*)forcing, coef,
                                       nullptr, 1, (double*)h_out, st);
}

extern "C" vd_status vd_qg1l_force(const vd_qg1l_plan* p, int B, const void* h, const void* hb, const void* forcing,
                                   const double* coef, void* h_out, void* stream)
{
    if (!p || B <= 0 || !h || !h_out || !forcing || !coef) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? finalize_impl<float>(p, B, (const float*)h, (const float*)hb, (const float*)forcing, 0.0, coef, 1,
                                      (float*)h_out, st)
               : finalize_impl<double>(p, B, (const double*)h, (const double*)hb, (const double*)forcing, 0.0, coef,
                                       1, (double*)h_out, st);
}

extern "C" vd_status vd_qg1l_force_adj(const vd_qg1l_plan* p, int B, const void* adh_out, void* adforcing,
                                       const double* coef, void* adh, void* stream)
{
    if (!p || B <= 0 || !adh_out || !adh || !adforcing || !coef) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? finalize_adj_impl<float>(p, B, (const float*)adh_out, (float*)adforcing, coef, (float*)adh, st)
               : finalize_adj_impl<double>(p, B, (const double*)adh_out, (double*)adforcing, coef, (double*)adh, st);
}
