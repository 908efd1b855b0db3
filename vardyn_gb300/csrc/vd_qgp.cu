// QG projector of the multilayer QG model (mapping/models/model_qgsw/qg.py:
// Q 300-308, QoG_inv 222-298 without background field, G 198-219) around the
// spectral Helmholtz solves, and the transposes of every piece. Fields are
// [batch][layer][x][y] like the shallow-water model; the modal right-hand
// sides and solutions use the solvers' [mode][batch][nx+1][ny+1] layout.
#include "vd_internal.cuh"

#include <cstring>
#include <new>
#include <vector>

namespace vd {
namespace qgp {

constexpr int MAXL = 8;

template <typename T>
struct Tab {
    int nx, ny, nl, B;
    long long su, sv, sh, sw;   // per-layer slab sizes
    T dx, dy, f0, area;
    T H[MAXL];
    T A[MAXL * MAXL], Cl2m[MAXL * MAXL], Cm2l[MAXL * MAXL];
    const uint8_t *fu, *fv, *fh, *fpsi;
    int cmm;
};

// Q: elliptic right-hand side per layer on interior w points, mixed to modes
template <typename T>
__global__ void k_qgp_Q(Tab<T> t, const T* u, const T* v, const T* h, T* out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const int nx = t.nx, ny = t.ny, nl = t.nl;
    if (i > nx || j > ny) return;
    const long long wi = (long long)i * (ny + 1) + j;
    const bool in = i >= 1 && i <= nx - 1 && j >= 1 && j <= ny - 1;
    T e[MAXL];
    if (in) {
        for (int l = 0; l < nl; ++l) {
            const long long ob = (long long)(b * nl + l);
            const T* U = u + ob * t.su;
            const T* V = v + ob * t.sv;
            const T* Hh = h + ob * t.sh;
            const T om = (V[(long long)i * (ny + 1) + j] - V[(long long)(i - 1) * (ny + 1) + j]) -
                         (U[(long long)i * ny + j] - U[(long long)i * ny + j - 1]);
            const T itp = T(0.25) * (Hh[(long long)i * ny + j] + Hh[(long long)i * ny + j - 1] +
                                     Hh[(long long)(i - 1) * ny + j] + Hh[(long long)(i - 1) * ny + j - 1]);
            e[l] = (om - t.f0 * itp / t.H[l]) * (t.f0 / t.area);
        }
    }
    const T ps = (t.cmm && !(t.fpsi[wi] & 1)) ? T(0) : T(1);
    for (int m = 0; m < nl; ++m) {
        T a = T(0);
        if (in) {
            for (int l = 0; l < nl; ++l) a += t.Cl2m[m * MAXL + l] * e[l];
            if (t.cmm) a = a * ps;
        }
        out[((long long)m * t.B + b) * t.sw + wi] = a;
    }
}

// Transpose of k_qgp_Q: ad (interior of [mode][batch][w]) -> adu, adv, adh (written)
template <typename T>
__global__ void k_qgp_Q_adj(Tab<T> t, const T* ad, T* adu, T* adv, T* adh)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const int nx = t.nx, ny = t.ny, nl = t.nl;
    if (i > nx || j > ny) return;
    auto ae = [&](int l, int p, int q) -> T {   // adjoint of e_l at w (p, q), zero off the interior
        if (p < 1 || p > nx - 1 || q < 1 || q > ny - 1) return T(0);
        const long long wi = (long long)p * (ny + 1) + q;
        const T ps = (t.cmm && !(t.fpsi[wi] & 1)) ? T(0) : T(1);
        T a = T(0);
        for (int m = 0; m < nl; ++m) a += t.Cl2m[m * MAXL + l] * ad[((long long)m * t.B + b) * t.sw + wi];
        return a * ps * (t.f0 / t.area);
    };
    for (int l = 0; l < nl; ++l) {
        const long long ob = (long long)(b * nl + l);
        if (j < ny) adu[ob * t.su + (long long)i * ny + j] = -ae(l, i, j) + ae(l, i, j + 1);
        if (i < nx) adv[ob * t.sv + (long long)i * (ny + 1) + j] = ae(l, i, j) - ae(l, i + 1, j);
        if (i < nx && j < ny)
            adh[ob * t.sh + (long long)i * ny + j] =
                -(t.f0 / t.H[l]) * T(0.25) * (ae(l, i, j) + ae(l, i, j + 1) + ae(l, i + 1, j) + ae(l, i + 1, j + 1));
    }
}

// per-field sums (optionally weighted by a per-mode field) in float64: block
// partial sums, then a fixed-order sum per field (deterministic)
constexpr int SUM_BLOCKS = 64;

template <typename T>
__global__ void k_qgp_sum_part(Tab<T> t, const T* x, const T* wgt, double* part)
{
    const int f = blockIdx.y;   // mode * B + batch
    const int m = f / t.B;
    const T* X = x + (long long)f * t.sw;
    const T* W = wgt ? wgt + (long long)m * t.sw : nullptr;
    double a = 0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < t.sw; k += (long long)gridDim.x * blockDim.x)
        a += W ? (double)W[k] * (double)X[k] : (double)X[k];
    __shared__ double red[256];
    red[threadIdx.x] = a;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(long long)f * gridDim.x + blockIdx.x] = red[0];
}

__global__ void k_qgp_sum_final(int nf, int nb, const double* part, double* out)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    double s = 0;
    for (int k = 0; k < nb; ++k) s += part[(long long)f * nb + k];
    out[f] = s;
}

// p_qg[b][l] = sum_m Cm2l[l][m] (p_m + alpha_m homsol_m), alpha = -mean(p_m)/hmean_m
template <typename T>
__global__ void k_qgp_P(Tab<T> t, const T* pm, const double* sums, const double* hmean, const T* homsol, T* pqg)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    const int nl = t.nl;
    if (k >= t.sw) return;
    T pp[MAXL];
    for (int m = 0; m < nl; ++m) {
        const T alpha = (T)(-(sums[m * t.B + b] / (double)t.sw) / hmean[m]);
        pp[m] = pm[((long long)m * t.B + b) * t.sw + k] + alpha * homsol[(long long)m * t.sw + k];
    }
    for (int l = 0; l < nl; ++l) {
        T a = T(0);
        for (int m = 0; m < nl; ++m) a += t.Cm2l[l * MAXL + m] * pp[m];
        pqg[(long long)(b * nl + l) * t.sw + k] = a;
    }
}

// Transpose: ad_pm'[m][b] = sum_l Cm2l[l][m] ad_pqg[b][l]
template <typename T>
__global__ void k_qgp_P_adj(Tab<T> t, const T* adpqg, T* adpm)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    const int nl = t.nl;
    if (k >= t.sw) return;
    for (int m = 0; m < nl; ++m) {
        T a = T(0);
        for (int l = 0; l < nl; ++l) a += t.Cm2l[l * MAXL + m] * adpqg[(long long)(b * nl + l) * t.sw + k];
        adpm[((long long)m * t.B + b) * t.sw + k] = a;
    }
}

// Transpose of the homogeneous correction: ad_p -= sum(homsol ad_p') / (N hmean)
template <typename T>
__global__ void k_qgp_hcorr_adj(Tab<T> t, const double* sums, const double* hmean, T* adpm)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (k >= t.sw) return;
    const int m = f / t.B;
    adpm[(long long)f * t.sw + k] -= (T)(sums[f] / ((double)t.sw * hmean[m]));
}

template <typename T> __device__ __forceinline__ T nan0(T x) { return x != x ? T(0) : x; }

// G: geostrophic u, v and thickness from p_qg (qg.py:198-219)
template <typename T>
__global__ void k_qgp_G(Tab<T> t, const T* pqg, T* u, T* v, T* h)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const int nx = t.nx, ny = t.ny, nl = t.nl;
    if (i > nx || j > ny) return;
    T pi[MAXL];
    const bool hp = i < nx && j < ny;
    for (int l = 0; l < nl; ++l) {
        const long long ob = (long long)(b * nl + l);
        const T* P = pqg + ob * t.sw;
        if (j < ny) {
            const long long q = (long long)i * ny + j;
            T a = -(P[(long long)i * (ny + 1) + j + 1] - P[(long long)i * (ny + 1) + j]) / t.dy / t.f0 * t.dx *
                  ((t.fu[q] & 1) ? T(1) : T(0));
            a = nan0(a);
            u[ob * t.su + q] = j == 0 ? T(0) : a;
        }
        if (i < nx) {
            const long long q = (long long)i * (ny + 1) + j;
            T a = (P[(long long)(i + 1) * (ny + 1) + j] - P[(long long)i * (ny + 1) + j]) / t.dx / t.f0 * t.dy *
                  ((t.fv[q] & 1) ? T(1) : T(0));
            a = nan0(a);
            v[ob * t.sv + q] = i == 0 ? T(0) : a;
        }
        if (hp)
            pi[l] = T(0.25) * (P[(long long)(i + 1) * (ny + 1) + j + 1] + P[(long long)(i + 1) * (ny + 1) + j] +
                               P[(long long)i * (ny + 1) + j + 1] + P[(long long)i * (ny + 1) + j]);
    }
    if (!hp) return;
    const long long q = (long long)i * ny + j;
    const T mh = (t.fh[q] & 1) ? T(1) : T(0);
    for (int l = 0; l < nl; ++l) {
        T a = T(0);
        for (int k = 0; k < nl; ++k) a += t.A[l * MAXL + k] * pi[k];
        h[(long long)(b * nl + l) * t.sh + q] = nan0(t.H[l] * a * t.area * mh);
    }
}

// Transpose of k_qgp_G (gather at w points)
template <typename T>
__global__ void k_qgp_G_adj(Tab<T> t, const T* adu, const T* adv, const T* adh, T* adpqg)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const int b = blockIdx.z;
    const int nx = t.nx, ny = t.ny, nl = t.nl;
    if (i > nx || j > ny) return;
    const T cu = T(1) / t.dy / t.f0 * t.dx, cv = T(1) / t.dx / t.f0 * t.dy;
    for (int k = 0; k < nl; ++k) {
        const long long ob = (long long)(b * nl + k);
        T a = T(0);
        // u(i, q) = -(p[i][q+1] - p[i][q]) cu mu, q >= 1
        if (j - 1 >= 1 && j - 1 <= ny - 1) {
            const long long q = (long long)i * ny + j - 1;
            a -= cu * ((t.fu[q] & 1) ? T(1) : T(0)) * adu[ob * t.su + q];
        }
        if (j >= 1 && j <= ny - 1) {
            const long long q = (long long)i * ny + j;
            a += cu * ((t.fu[q] & 1) ? T(1) : T(0)) * adu[ob * t.su + q];
        }
        // v(p, j) = (p[p+1][j] - p[p][j]) cv mv, p >= 1
        if (i - 1 >= 1 && i - 1 <= nx - 1) {
            const long long q = (long long)(i - 1) * (ny + 1) + j;
            a += cv * ((t.fv[q] & 1) ? T(1) : T(0)) * adv[ob * t.sv + q];
        }
        if (i >= 1 && i <= nx - 1) {
            const long long q = (long long)i * (ny + 1) + j;
            a -= cv * ((t.fv[q] & 1) ? T(1) : T(0)) * adv[ob * t.sv + q];
        }
        // h cells around w (i, j)
        T hs = T(0);
        for (int di = -1; di <= 0; ++di)
            for (int dj = -1; dj <= 0; ++dj) {
                const int ci = i + di, cj = j + dj;
                if (ci < 0 || ci >= nx || cj < 0 || cj >= ny) continue;
                const long long q = (long long)ci * ny + cj;
                if (!(t.fh[q] & 1)) continue;
                T s = T(0);
                for (int l = 0; l < nl; ++l)
                    s += adh[(long long)(b * nl + l) * t.sh + q] * t.H[l] * t.A[l * MAXL + k];
                hs += s;
            }
        a += T(0.25) * t.area * hs;
        adpqg[ob * t.sw + (long long)i * (ny + 1) + j] = a;
    }
}

}  // namespace qgp
}  // namespace vd

using namespace vd::qgp;

struct vd_qgp_plan {
    int nx, ny, nl, dtype;
    void* dev;
    Tab<float> tf;
    Tab<double> td;
};

extern "C" vd_status vd_qgp_plan_create(vd_qgp_plan** out, const vd_qgp_desc* d)
{
    if (!out || !d) return VD_ERR_ARG;
    *out = nullptr;
    const int nx = d->nx, ny = d->ny, nl = d->nl;
    if (nx < 4 || ny < 4 || nl < 1 || nl > MAXL || (d->dtype != VD_F32 && d->dtype != VD_F64)) return VD_ERR_ARG;
    if (!d->H_host || !d->A_host || !d->Cl2m_host || !d->Cm2l_host) return VD_ERR_ARG;
    if (!(d->dx > 0) || !(d->dy > 0) || d->f0 == 0) return VD_ERR_ARG;
    // masks: reuse the shallow-water mask builder
    std::vector<uint8_t> fh((size_t)nx * ny), fu((size_t)(nx + 1) * ny), fv((size_t)nx * (ny + 1)),
        fw((size_t)(nx + 1) * (ny + 1));
    vd_status rc = vd_sw_masks(nx, ny, d->mask_host, fh.data(), fu.data(), fv.data(), fw.data());
    if (rc) return rc;
    std::vector<uint8_t> fpsi(fw.size());
    for (size_t k = 0; k < fw.size(); ++k) fpsi[k] = (fw[k] >> 5) & 1;
    const size_t o1 = 0, o2 = (fh.size() + 255) & ~size_t(255), o3 = o2 + ((fu.size() + 255) & ~size_t(255)),
                 o4 = o3 + ((fv.size() + 255) & ~size_t(255)), tot = o4 + fpsi.size();
    std::vector<uint8_t> host(tot, 0);
    std::memcpy(host.data() + o1, fh.data(), fh.size());
    std::memcpy(host.data() + o2, fu.data(), fu.size());
    std::memcpy(host.data() + o3, fv.data(), fv.size());
    std::memcpy(host.data() + o4, fpsi.data(), fpsi.size());
    vd_qgp_plan* p = new (std::nothrow) vd_qgp_plan();
    if (!p) return VD_ERR_CUDA;
    p->nx = nx; p->ny = ny; p->nl = nl; p->dtype = d->dtype;
    if (cudaMalloc(&p->dev, tot) != cudaSuccess) {
        delete p;
        return VD_ERR_CUDA;
    }
    if (cudaMemcpy(p->dev, host.data(), tot, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(p->dev);
        delete p;
        return VD_ERR_CUDA;
    }
    auto fill = [&](auto& t) {
        using TT = decltype(t.dx);
        t.nx = nx; t.ny = ny; t.nl = nl; t.B = 0;
        t.su = (long long)(nx + 1) * ny; t.sv = (long long)nx * (ny + 1); t.sh = (long long)nx * ny;
        t.sw = (long long)(nx + 1) * (ny + 1);
        t.dx = (TT)d->dx; t.dy = (TT)d->dy; t.f0 = (TT)d->f0; t.area = (TT)(d->dx * d->dy);
        for (int a = 0; a < MAXL; ++a) {
            t.H[a] = a < nl ? (TT)d->H_host[a] : TT(1);
            for (int c = 0; c < MAXL; ++c) {
                const bool ok = a < nl && c < nl;
                t.A[a * MAXL + c] = ok ? (TT)d->A_host[a * nl + c] : TT(0);
                t.Cl2m[a * MAXL + c] = ok ? (TT)d->Cl2m_host[a * nl + c] : TT(0);
                t.Cm2l[a * MAXL + c] = ok ? (TT)d->Cm2l_host[a * nl + c] : TT(0);
            }
        }
        const uint8_t* base = (const uint8_t*)p->dev;
        t.fh = base + o1; t.fu = base + o2; t.fv = base + o3; t.fpsi = base + o4;
        t.cmm = d->cmm ? 1 : 0;
    };
    if (d->dtype == VD_F64) fill(p->td);
    else fill(p->tf);
    *out = p;
    return VD_OK;
}

extern "C" void vd_qgp_plan_destroy(vd_qgp_plan* p)
{
    if (!p) return;
    if (p->dev) cudaFree(p->dev);
    delete p;
}

namespace {
template <typename T> Tab<T> qtab(const vd_qgp_plan* p, int B);
template <> Tab<float> qtab<float>(const vd_qgp_plan* p, int B) { Tab<float> t = p->tf; t.B = B; return t; }
template <> Tab<double> qtab<double>(const vd_qgp_plan* p, int B) { Tab<double> t = p->td; t.B = B; return t; }

static dim3 wgrid(const vd_qgp_plan* p, int z) { return dim3((unsigned)((p->ny + 1 + 31) / 32), (unsigned)((p->nx + 1 + 7) / 8), (unsigned)z); }

template <typename T>
static int op_t(const vd_qgp_plan* p, int op, int B, const void* const* a, cudaStream_t st)
{
    const Tab<T> t = qtab<T>(p, B);
    const dim3 blk(32, 8, 1);
    const unsigned nb = (unsigned)((t.sw + 255) / 256);
    switch (op) {
    case 0:   // Q: u, v, h -> modes
        k_qgp_Q<T><<<wgrid(p, B), blk, 0, st>>>(t, (const T*)a[0], (const T*)a[1], (const T*)a[2], (T*)a[3]);
        break;
    case 1:   // Q^T: modes -> adu, adv, adh
        k_qgp_Q_adj<T><<<wgrid(p, B), blk, 0, st>>>(t, (const T*)a[0], (T*)a[1], (T*)a[2], (T*)a[3]);
        break;
    case 2: {   // sums: x, weight (nullable) -> double[nl*B]; partials in out[nl*B ..]
        const int nf = p->nl * B;
        double* part = (double*)a[2] + nf;
        k_qgp_sum_part<T><<<dim3(SUM_BLOCKS, (unsigned)nf), 256, 0, st>>>(t, (const T*)a[0], (const T*)a[1], part);
        VD_LAUNCH_CHECK();
        k_qgp_sum_final<<<(unsigned)((nf + 127) / 128), 128, 0, st>>>(nf, SUM_BLOCKS, part, (double*)a[2]);
        break;
    }
    case 3:   // P: pm, sums, hmean, homsol -> pqg
        k_qgp_P<T><<<dim3(nb, (unsigned)B), 256, 0, st>>>(t, (const T*)a[0], (const double*)a[1],
                                                          (const double*)a[2], (const T*)a[3], (T*)a[4]);
        break;
    case 4:   // P^T (mixing only): adpqg -> adpm
        k_qgp_P_adj<T><<<dim3(nb, (unsigned)B), 256, 0, st>>>(t, (const T*)a[0], (T*)a[1]);
        break;
    case 5:   // homogeneous-correction transpose: sums, hmean, adpm (in place)
        k_qgp_hcorr_adj<T><<<dim3(nb, (unsigned)(p->nl * B)), 256, 0, st>>>(t, (const double*)a[0],
                                                                           (const double*)a[1], (T*)a[2]);
        break;
    case 6:   // G: pqg -> u, v, h
        k_qgp_G<T><<<wgrid(p, B), blk, 0, st>>>(t, (const T*)a[0], (T*)a[1], (T*)a[2], (T*)a[3]);
        break;
    case 7:   // G^T: adu, adv, adh -> adpqg
        k_qgp_G_adj<T><<<wgrid(p, B), blk, 0, st>>>(t, (const T*)a[0], (const T*)a[1], (const T*)a[2], (T*)a[3]);
        break;
    default:
        return VD_ERR_ARG;
    }
    VD_LAUNCH_CHECK();
    return VD_OK;
}
}  // namespace

extern "C" vd_status vd_qgp_op(const vd_qgp_plan* p, int op, int batch, const void* const* args, void* stream)
{
    static const int nargs[8] = {4, 4, 2, 5, 2, 3, 4, 4};
    static const int optional[8] = {-1, -1, 1, -1, -1, -1, -1, -1};
    if (!p || batch <= 0 || op < 0 || op > 7 || !args) return VD_ERR_ARG;
    if ((long long)batch * p->nl > 65535) return VD_ERR_ARG;
    for (int k = 0; k < nargs[op] + (op == 2 ? 1 : 0); ++k)
        if (!args[k] && k != optional[op]) return VD_ERR_ARG;
    return p->dtype == VD_F64 ? op_t<double>(p, op, batch, args, (cudaStream_t)stream)
                              : op_t<float>(p, op, batch, args, (cudaStream_t)stream);
}
