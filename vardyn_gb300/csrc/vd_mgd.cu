// Node-centred Dirichlet multigrid for the masked Helmholtz problems of the
// multilayer QG PV inversion (mapping/models/model_qgsw/qg.py:222-298): per
// vertical mode m, on the interior nodes of the psi grid,
//     (u_E + u_W - 2u)/d0^2 + (u_N + u_S - 2u)/d1^2 - lambda_m u = b
// at ocean nodes, u = 0 at land nodes and beyond the outer boundary. The
// reference solves the same discrete problem with a DST solve and a
// capacitance-matrix correction at the irregular boundary points
// (helmholtz.py:146-184), which needs one DST solve per irregular point and an
// M x M inverse; at 20 % land that is tens of thousands of solves. Here a
// geometric V-cycle solves it directly:
//   - node-centred coarsening (coarse node I at fine node 2I+1; n -> (n+1)/2-1),
//     a coarse node an unknown where its 3 x 3 fine neighbourhood is, the
//     operator rediscretised on every level;
//   - red-black Gauss-Seidel smoothing (2 + 2 sweeps), full-weighting
//     restriction and bilinear prolongation of the correction, both masked;
//   - the coarsest level solved exactly with a float64 inverse built on the host;
//   - the symmetric V-cycle (red-black pre-smoothing, black-red post-smoothing)
//     preconditions conjugate gradients: the conservative coarse masks keep
//     the coarse levels from bridging land, and the Krylov iteration removes
//     the few coastal modes they resolve poorly;
//   - the scalars of every system live in device memory, the float64 dot
//     products are reduced in a fixed order (per-block partial sums, then one
//     thread per system); when ||r|| <= tol ||b|| a system's flag makes every
//     later kernel of that system return at once, so a solve is a fixed
//     launch sequence (it can be captured in a CUDA graph) that stops
//     computing at the tolerance.
// Systems are [nsys = nmode * batch] slices of the caller's arrays with a row
// pitch `ld` and a system stride `fs` (the interior of a (nx+1) x (ny+1) psi
// field in place).
#include "vd_internal.cuh"
#include <algorithm>
#include <cmath>
#include <functional>
#include <new>
#include <vector>

namespace vd {

struct MgdLevel {
    int n0, n1;
    double d0, d1;
    int8_t* mask;       // [n0][n1] device
};

template <typename T>
struct MgdArgs {
    int n0, n1;
    T c0, c1;            // 1/d0^2, 1/d1^2
    const int8_t* mask;
    const T* lam;        // [nmode]
    int batch;           // systems per mode
    const int* done;     // [nsys] converged flags
};

template <typename T>
__device__ __forceinline__ T mgd_get(const T* u, int n0, int n1, long long ld, int i, int j)
{
    return (i >= 0 && i < n0 && j >= 0 && j < n1) ? u[(long long)i * ld + j] : T(0);
}

// one red-black Gauss-Seidel half sweep on nodes with (i + j) % 2 == color
template <typename T>
__global__ void k_mgd_smooth(MgdArgs<T> A, int color, T* __restrict__ u, long long ldu, long long fsu,
                             const T* __restrict__ b, long long ldb, long long fsb)
{
    const int s = blockIdx.z;
    if (A.done[s]) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= A.n0 || j >= A.n1 || ((i + j) & 1) != color) return;
    if (!A.mask[i * A.n1 + j]) return;
    T* us = u + s * fsu;
    const T lam = A.lam[s / A.batch];
    const T nb = A.c0 * (mgd_get(us, A.n0, A.n1, ldu, i - 1, j) + mgd_get(us, A.n0, A.n1, ldu, i + 1, j)) +
                 A.c1 * (mgd_get(us, A.n0, A.n1, ldu, i, j - 1) + mgd_get(us, A.n0, A.n1, ldu, i, j + 1));
    us[(long long)i * ldu + j] = (nb - b[s * fsb + (long long)i * ldb + j]) / (T(2) * A.c0 + T(2) * A.c1 + lam);
}

// r = b - A u (0 on land; b == nullptr: r = -A u)
template <typename T>
__global__ void k_mgd_resid(MgdArgs<T> A, const T* __restrict__ u, long long ldu, long long fsu,
                            const T* __restrict__ b, long long ldb, long long fsb, T* __restrict__ r)
{
    const int s = blockIdx.z;
    if (A.done[s]) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= A.n0 || j >= A.n1) return;
    const long long o = (long long)s * A.n0 * A.n1 + (long long)i * A.n1 + j;
    if (!A.mask[i * A.n1 + j]) { r[o] = T(0); return; }
    const T* us = u + s * fsu;
    const T lam = A.lam[s / A.batch];
    const T uc = us[(long long)i * ldu + j];
    const T Au = A.c0 * (mgd_get(us, A.n0, A.n1, ldu, i - 1, j) + mgd_get(us, A.n0, A.n1, ldu, i + 1, j) - T(2) * uc) +
                 A.c1 * (mgd_get(us, A.n0, A.n1, ldu, i, j - 1) + mgd_get(us, A.n0, A.n1, ldu, i, j + 1) - T(2) * uc) -
                 lam * uc;
    r[o] = (b ? b[s * fsb + (long long)i * ldb + j] : T(0)) - Au;
}

// coarse b = full weighting of the fine residual (1/16 [1 2 1; 2 4 2; 1 2 1])
template <typename T>
__global__ void k_mgd_restrict(int n0f, int n1f, int n0c, int n1c, const int8_t* __restrict__ maskc,
                               const int* __restrict__ done, const T* __restrict__ rf, T* __restrict__ bc)
{
    const int s = blockIdx.z;
    if (done[s]) return;
    const int J = blockIdx.x * blockDim.x + threadIdx.x;
    const int I = blockIdx.y * blockDim.y + threadIdx.y;
    if (I >= n0c || J >= n1c) return;
    const long long oc = (long long)s * n0c * n1c + (long long)I * n1c + J;
    if (!maskc[I * n1c + J]) { bc[oc] = T(0); return; }
    const T* r = rf + (long long)s * n0f * n1f;
    const int i = 2 * I + 1, j = 2 * J + 1;
    const long long ld = n1f;
    const T v = T(4) * r[(long long)i * ld + j] +
                T(2) * (r[(long long)(i - 1) * ld + j] + r[(long long)(i + 1) * ld + j] + r[(long long)i * ld + j - 1] +
                        r[(long long)i * ld + j + 1]) +
                r[(long long)(i - 1) * ld + j - 1] + r[(long long)(i - 1) * ld + j + 1] +
                r[(long long)(i + 1) * ld + j - 1] + r[(long long)(i + 1) * ld + j + 1];
    bc[oc] = v / T(16);
}

// fine u += bilinear interpolation of the coarse correction (0 on land)
template <typename T>
__global__ void k_mgd_prolong(int n0f, int n1f, int n0c, int n1c, const int8_t* __restrict__ maskf,
                              const int* __restrict__ done, const T* __restrict__ ec, T* __restrict__ u, long long ldu,
                              long long fsu)
{
    const int s = blockIdx.z;
    if (done[s]) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n0f || j >= n1f || !maskf[i * n1f + j]) return;
    const T* e = ec + (long long)s * n0c * n1c;
    // fine index 2I+1 is coarse I; an even fine index lies between I-1 and I
    const int i0 = (i - 1) >> 1, j0 = (j - 1) >> 1;       // floor for odd, lower neighbour for even
    const bool io = i & 1, jo = j & 1;
    auto E = [&](int I, int J) { return mgd_get(e, n0c, n1c, (long long)n1c, I, J); };
    T v;
    if (io && jo) v = E(i0, j0);
    else if (io) v = T(0.5) * (E(i0, j0) + E(i0, j0 + 1));
    else if (jo) v = T(0.5) * (E(i0, j0) + E(i0 + 1, j0));
    else v = T(0.25) * (E(i0, j0) + E(i0 + 1, j0) + E(i0, j0 + 1) + E(i0 + 1, j0 + 1));
    u[s * fsu + (long long)i * ldu + j] += v;
}

template <typename T>
__global__ void k_mgd_zero_strided(int n0, int n1, T* __restrict__ u, long long ldu, long long fsu)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < n0 && j < n1) u[blockIdx.z * fsu + (long long)i * ldu + j] = T(0);
}

template <typename T>
__global__ void k_mgd_zero(int n, const int* __restrict__ done, T* __restrict__ x)
{
    const int s = blockIdx.y;
    if (done[s]) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) x[(long long)s * n + k] = T(0);
}

// coarsest level: u[idx[m]] = sum_k inv[mode][m][k] b[idx[k]] in float64
template <typename T>
__global__ void k_mgd_coarse(int nb, int ncell, int batch, const int* __restrict__ done, const int32_t* __restrict__ idx,
                             const double* __restrict__ inv, const T* __restrict__ b, T* __restrict__ u)
{
    const int s = blockIdx.y;
    if (done[s]) return;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nb) return;
    const double* row = inv + ((long long)(s / batch) * nb + m) * nb;
    const T* bs = b + (long long)s * ncell;
    double acc = 0.0;
    for (int k = 0; k < nb; ++k) acc += row[k] * (double)bs[idx[k]];
    u[(long long)s * ncell + idx[m]] = (T)acc;
}

// ---- preconditioned conjugate gradients around the V-cycle (per system,
//      scalars in device memory, float64 dot products reduced in a fixed
//      order: per-block partial sums, then one thread per system) ----
constexpr int MGD_PARTS = 64;
constexpr int MGD_SCAL = 4;            // per system: ||b||^2, rho, alpha, relative residual

template <typename T>
__global__ void k_mgd_dot_part(int n, const int* __restrict__ done, const T* __restrict__ x, const T* __restrict__ y,
                               double* __restrict__ part)
{
    const int s = blockIdx.y;
    __shared__ double sh[256];
    double a = 0.0;
    if (!done[s]) {
        const T* xs = x + (long long)s * n;
        const T* ys = y + (long long)s * n;
        for (int k = blockIdx.x * 256 + threadIdx.x; k < n; k += gridDim.x * 256) a += (double)xs[k] * (double)ys[k];
    }
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(long long)s * gridDim.x + blockIdx.x] = sh[0];
}

__device__ __forceinline__ double mgd_sum(const double* part, int s, int np)
{
    double v = 0.0;
    for (int k = 0; k < np; ++k) v += part[(long long)s * np + k];
    return v;
}

// what: 0 = ||b||^2 (init), 1 = rho = r.z, 2 = alpha = rho / (p.Ap),
// 3 = convergence test on r.r, 4 = beta = r.z / rho (stored in beta[]), rho updated
__global__ void k_mgd_scal(int nsys, int np, int what, double tol, const double* __restrict__ part,
                           int* __restrict__ done, double* __restrict__ sc, double* __restrict__ beta,
                           double* __restrict__ rel)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys || done[s]) return;
    double* c = sc + (long long)s * MGD_SCAL;
    const double v = mgd_sum(part, s, np);
    if (what == 0) {
        c[0] = v;
        if (v == 0.0) { done[s] = 1; c[3] = 0.0; if (rel) rel[s] = 0.0; }
    } else if (what == 1) {
        c[1] = v;
    } else if (what == 2) {
        c[2] = v != 0.0 ? c[1] / v : 0.0;
    } else if (what == 3) {
        const double q = c[0] > 0.0 ? sqrt(v / c[0]) : 0.0;
        c[3] = q;
        if (rel) rel[s] = q;
        if (q <= tol) done[s] = 1;
    } else {
        beta[s] = c[1] != 0.0 ? v / c[1] : 0.0;
        c[1] = v;
    }
}

// With q = -A p and sc[2] = rho / (p.q) = -alpha: x (strided) += alpha p,
// r -= alpha A p
template <typename T>
__global__ void k_mgd_xr(int n0, int n1, const int* __restrict__ done, const double* __restrict__ sc,
                         const T* __restrict__ pv, const T* __restrict__ qv, T* __restrict__ x, long long ldx,
                         long long fsx, T* __restrict__ r)
{
    const int s = blockIdx.z;
    if (done[s]) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n0 || j >= n1) return;
    const T al = (T)sc[(long long)s * MGD_SCAL + 2];
    const long long o = (long long)s * n0 * n1 + (long long)i * n1 + j;
    x[s * fsx + (long long)i * ldx + j] -= al * pv[o];
    r[o] -= al * qv[o];
}

// p = z + beta p (beta = 0 on the first iteration: p = z)
template <typename T>
__global__ void k_mgd_p(int n, const int* __restrict__ done, const double* __restrict__ beta, int first,
                        const T* __restrict__ z, T* __restrict__ pv)
{
    const int s = blockIdx.y;
    if (done[s]) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long o = (long long)s * n + k;
    pv[o] = first ? z[o] : z[o] + (T)beta[s] * pv[o];
}

__global__ void k_mgd_fill_int(int n, int v, int* __restrict__ x)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) x[k] = v;
}

// Gauss-Jordan inverse with partial pivoting of a dense float64 matrix
static bool invert(std::vector<double>& A, int n, std::vector<double>& inv)
{
    inv.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) inv[(size_t)i * n + i] = 1.0;
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(A[(size_t)r * n + c]) > std::fabs(A[(size_t)p * n + c])) p = r;
        if (A[(size_t)p * n + c] == 0.0) return false;
        if (p != c)
            for (int k = 0; k < n; ++k) {
                std::swap(A[(size_t)p * n + k], A[(size_t)c * n + k]);
                std::swap(inv[(size_t)p * n + k], inv[(size_t)c * n + k]);
            }
        const double d = 1.0 / A[(size_t)c * n + c];
        for (int k = 0; k < n; ++k) { A[(size_t)c * n + k] *= d; inv[(size_t)c * n + k] *= d; }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = A[(size_t)r * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) {
                A[(size_t)r * n + k] -= f * A[(size_t)c * n + k];
                inv[(size_t)r * n + k] -= f * inv[(size_t)c * n + k];
            }
        }
    }
    return true;
}

}  // namespace vd

using namespace vd;

struct vd_mgd_plan {
    vd_mgd_desc d;
    std::vector<MgdLevel> lv;
    void* lam = nullptr;            // [nmode] plan dtype
    int nb = 0;                     // coarsest unknowns
    int32_t* cidx = nullptr;        // [nb]
    double* cinv = nullptr;         // [nmode][nb][nb]
};

static int mgd_coarsenable(int n) { return (n + 1) % 2 == 0 && (n + 1) / 2 - 1 >= 3; }

extern "C" vd_status vd_mgd_plan_create(vd_mgd_plan** out, const vd_mgd_desc* d)
{
    if (!out || !d) return VD_ERR_ARG;
    *out = nullptr;
    if (d->n0 < 1 || d->n1 < 1 || d->nmode < 1 || !d->lambda_host || !(d->d0 > 0) || !(d->d1 > 0) ||
        d->max_cycles < 1 || !(d->tol > 0) || (d->dtype != VD_F32 && d->dtype != VD_F64))
        return VD_ERR_ARG;
    vd_mgd_plan* p = new (std::nothrow) vd_mgd_plan();
    if (!p) return VD_ERR_ARG;
    p->d = *d;
    p->d.mask_host = nullptr;
    p->d.lambda_host = nullptr;
    auto fail = [&](int code) { vd_mgd_plan_destroy(p); return code; };
    // level hierarchy on the host
    std::vector<std::vector<int8_t>> masks;
    std::vector<int8_t> m0((size_t)d->n0 * d->n1, 1);
    if (d->mask_host)
        for (size_t k = 0; k < m0.size(); ++k) m0[k] = d->mask_host[k] != 0.0;
    masks.push_back(m0);
    std::vector<int> n0s{d->n0}, n1s{d->n1};
    std::vector<double> d0s{d->d0}, d1s{d->d1};
    while (mgd_coarsenable(n0s.back()) && mgd_coarsenable(n1s.back()) && n0s.back() * n1s.back() > 64) {
        const int n0 = n0s.back(), n1 = n1s.back();
        const int c0 = (n0 + 1) / 2 - 1, c1 = (n1 + 1) / 2 - 1;
        // a coarse node is an unknown only if the 3 x 3 fine nodes around it
        // are: a coarse level never bridges a fine land barrier (which would
        // join basins that the fine problem keeps apart)
        std::vector<int8_t> mc((size_t)c0 * c1);
        const std::vector<int8_t>& mf = masks.back();
        for (int I = 0; I < c0; ++I)
            for (int J = 0; J < c1; ++J) {
                int8_t v = 1;
                for (int a = -1; a <= 1; ++a)
                    for (int c = -1; c <= 1; ++c) v &= mf[(size_t)(2 * I + 1 + a) * n1 + 2 * J + 1 + c];
                mc[(size_t)I * c1 + J] = v;
            }
        masks.push_back(mc);
        n0s.push_back(c0); n1s.push_back(c1);
        d0s.push_back(2 * d0s.back()); d1s.push_back(2 * d1s.back());
    }
    const int nlev = (int)masks.size();
    // coarsest level: float64 inverse per mode over its unknowns
    const int cn0 = n0s.back(), cn1 = n1s.back();
    std::vector<int32_t> idx;
    for (int k = 0; k < cn0 * cn1; ++k)
        if (masks.back()[k]) idx.push_back(k);
    p->nb = (int)idx.size();
    if (p->nb > 4096) return fail(VD_ERR_UNSUPPORTED);
    std::vector<double> invs((size_t)d->nmode * p->nb * p->nb);
    {
        const double a0 = 1.0 / (d0s.back() * d0s.back()), a1 = 1.0 / (d1s.back() * d1s.back());
        std::vector<int> pos((size_t)cn0 * cn1, -1);
        for (int k = 0; k < p->nb; ++k) pos[idx[k]] = k;
        for (int m = 0; m < d->nmode; ++m) {
            std::vector<double> A((size_t)p->nb * p->nb, 0.0), inv;
            for (int k = 0; k < p->nb; ++k) {
                const int i = idx[k] / cn1, j = idx[k] % cn1;
                A[(size_t)k * p->nb + k] = -2 * a0 - 2 * a1 - d->lambda_host[m];
                const int nbs[4][2] = {{i - 1, j}, {i + 1, j}, {i, j - 1}, {i, j + 1}};
                for (int t = 0; t < 4; ++t) {
                    const int ii = nbs[t][0], jj = nbs[t][1];
                    if (ii < 0 || ii >= cn0 || jj < 0 || jj >= cn1) continue;
                    const int q = pos[(size_t)ii * cn1 + jj];
                    if (q >= 0) A[(size_t)k * p->nb + q] += t < 2 ? a0 : a1;
                }
            }
            if (p->nb && !invert(A, p->nb, inv)) return fail(VD_ERR_ARG);
            std::copy(inv.begin(), inv.end(), invs.begin() + (size_t)m * p->nb * p->nb);
        }
    }
    // device tables
    p->lv.resize(nlev);
    for (int l = 0; l < nlev; ++l) {
        MgdLevel& L = p->lv[l];
        L.n0 = n0s[l]; L.n1 = n1s[l]; L.d0 = d0s[l]; L.d1 = d1s[l];
        if (cudaMalloc(&L.mask, masks[l].size()) != cudaSuccess) return fail(VD_ERR_CUDA);
        if (cudaMemcpy(L.mask, masks[l].data(), masks[l].size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(VD_ERR_CUDA);
    }
    const size_t es = d->dtype == VD_F64 ? 8 : 4;
    std::vector<char> lamb(es * d->nmode);
    for (int m = 0; m < d->nmode; ++m) {
        if (es == 8) reinterpret_cast<double*>(lamb.data())[m] = d->lambda_host[m];
        else reinterpret_cast<float*>(lamb.data())[m] = (float)d->lambda_host[m];
    }
    if (cudaMalloc(&p->lam, lamb.size()) != cudaSuccess ||
        cudaMemcpy(p->lam, lamb.data(), lamb.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(VD_ERR_CUDA);
    if (p->nb) {
        if (cudaMalloc(&p->cidx, idx.size() * 4) != cudaSuccess ||
            cudaMemcpy(p->cidx, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMalloc(&p->cinv, invs.size() * 8) != cudaSuccess ||
            cudaMemcpy(p->cinv, invs.data(), invs.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(VD_ERR_CUDA);
    }
    *out = p;
    return VD_OK;
}

extern "C" vd_status vd_mgd_plan_destroy(vd_mgd_plan* p)
{
    if (!p) return VD_OK;
    for (auto& L : p->lv) cudaFree(L.mask);
    cudaFree(p->lam);
    cudaFree(p->cidx);
    cudaFree(p->cinv);
    delete p;
    return VD_OK;
}

extern "C" int vd_mgd_levels(const vd_mgd_plan* p) { return p ? (int)p->lv.size() : 0; }
extern "C" int vd_mgd_coarse_unknowns(const vd_mgd_plan* p) { return p ? p->nb : 0; }

// per level: u, b, r buffers of nsys systems; then the conjugate-gradient
// vectors r, z, p, q of level 0; flags; dot partial sums; scalars; beta
static size_t mgd_layout(const vd_mgd_plan* p, int nsys, std::vector<size_t>* off)
{
    const size_t es = p->d.dtype == VD_F64 ? 8 : 4;
    size_t o = 0;
    auto take = [&](size_t bytes) { const size_t a = o; o = (o + bytes + 255) & ~size_t(255); return a; };
    if (off) off->clear();
    for (size_t l = 0; l < p->lv.size(); ++l)
        for (int w = 0; w < 3; ++w) {
            const size_t a = take(es * (size_t)nsys * p->lv[l].n0 * p->lv[l].n1);
            if (off) off->push_back(a);
        }
    const size_t n0 = es * (size_t)nsys * p->lv[0].n0 * p->lv[0].n1;
    const size_t cr = take(n0), cz = take(n0), cp = take(n0), cq = take(n0);
    const size_t fl = take(4 * (size_t)nsys);
    const size_t pa = take(8 * (size_t)nsys * MGD_PARTS);
    const size_t sc = take(8 * (size_t)nsys * MGD_SCAL);
    const size_t be = take(8 * (size_t)nsys);
    if (off) for (size_t a : {cr, cz, cp, cq, fl, pa, sc, be}) off->push_back(a);
    return o;
}

extern "C" size_t vd_mgd_workspace_bytes(const vd_mgd_plan* p, int batch)
{
    if (!p || batch < 1) return 0;
    return mgd_layout(p, batch * p->d.nmode, nullptr);
}

template <typename T>
static int mgd_solve_t(const vd_mgd_plan* p, int batch, const T* b, long long ldb, long long fsb, T* u, long long ldu,
                       long long fsu, double* rel, char* ws, cudaStream_t st)
{
    const int nsys = batch * p->d.nmode;
    std::vector<size_t> off;
    mgd_layout(p, nsys, &off);
    const int nlev = (int)p->lv.size();
    auto buf = [&](int l, int w) { return (T*)(ws + off[3 * l + w]); };
    T* cr = (T*)(ws + off[3 * nlev]);
    T* cz = (T*)(ws + off[3 * nlev + 1]);
    T* cp = (T*)(ws + off[3 * nlev + 2]);
    T* cq = (T*)(ws + off[3 * nlev + 3]);
    int* done = (int*)(ws + off[3 * nlev + 4]);
    double* part = (double*)(ws + off[3 * nlev + 5]);
    double* sc = (double*)(ws + off[3 * nlev + 6]);
    double* beta = (double*)(ws + off[3 * nlev + 7]);
    auto args = [&](int l) {
        MgdArgs<T> A;
        A.n0 = p->lv[l].n0; A.n1 = p->lv[l].n1;
        A.c0 = T(1.0 / (p->lv[l].d0 * p->lv[l].d0)); A.c1 = T(1.0 / (p->lv[l].d1 * p->lv[l].d1));
        A.mask = p->lv[l].mask; A.lam = (const T*)p->lam; A.batch = batch; A.done = done;
        return A;
    };
    const dim3 blk(32, 8);
    auto grid = [&](int l) { return dim3((p->lv[l].n1 + 31) / 32, (p->lv[l].n0 + 7) / 8, nsys); };
    const int n0 = p->lv[0].n0, n1 = p->lv[0].n1, ncell = n0 * n1;
    const int nparts = std::max(1, std::min(MGD_PARTS, (ncell + 8191) / 8192));
    auto zero_level = [&](int l, T* x) {
        const int n = p->lv[l].n0 * p->lv[l].n1;
        k_mgd_zero<T><<<dim3((n + 255) / 256, nsys), 256, 0, st>>>(n, done, x);
        VD_LAUNCH_CHECK();
        return VD_OK;
    };
    auto dot = [&](const T* x, const T* y, int what) {
        k_mgd_dot_part<T><<<dim3(nparts, nsys), 256, 0, st>>>(ncell, done, x, y, part);
        VD_LAUNCH_CHECK();
        k_mgd_scal<<<(nsys + 127) / 128, 128, 0, st>>>(nsys, nparts, what, p->d.tol, part, done, sc, beta, rel);
        VD_LAUNCH_CHECK();
        return VD_OK;
    };
    const int nu = 2;
    // V-cycle on contiguous level buffers (level 0: u = z, b = r); the
    // pre-smoothing sweeps red then black, the post-smoothing black then red,
    // so that the cycle is a symmetric preconditioner
    std::function<int(int, T*, const T*)> vcycle;
    vcycle = [&](int l, T* ul, const T* bl) -> int {
        const long long ld = p->lv[l].n1, fs = (long long)p->lv[l].n0 * p->lv[l].n1;
        if (l == nlev - 1) {
            if (p->nb) {
                k_mgd_coarse<T><<<dim3((p->nb + 127) / 128, nsys), 128, 0, st>>>(p->nb, (int)fs, batch, done,
                                                                                  p->cidx, p->cinv, bl, ul);
                VD_LAUNCH_CHECK();
            }
            return VD_OK;
        }
        const MgdArgs<T> A = args(l);
        for (int k = 0; k < nu; ++k)
            for (int c = 0; c < 2; ++c) {
                k_mgd_smooth<T><<<grid(l), blk, 0, st>>>(A, c, ul, ld, fs, bl, ld, fs);
                VD_LAUNCH_CHECK();
            }
        T* r = buf(l, 2);
        k_mgd_resid<T><<<grid(l), blk, 0, st>>>(A, ul, ld, fs, bl, ld, fs, r);
        VD_LAUNCH_CHECK();
        const MgdLevel& F = p->lv[l];
        const MgdLevel& C = p->lv[l + 1];
        k_mgd_restrict<T><<<grid(l + 1), blk, 0, st>>>(F.n0, F.n1, C.n0, C.n1, C.mask, done, r, buf(l + 1, 1));
        VD_LAUNCH_CHECK();
        int e;
        if ((e = zero_level(l + 1, buf(l + 1, 0)))) return e;
        if ((e = vcycle(l + 1, buf(l + 1, 0), buf(l + 1, 1)))) return e;
        k_mgd_prolong<T><<<grid(l), blk, 0, st>>>(F.n0, F.n1, C.n0, C.n1, F.mask, done, buf(l + 1, 0), ul, ld, fs);
        VD_LAUNCH_CHECK();
        for (int k = 0; k < nu; ++k)
            for (int c = 1; c >= 0; --c) {
                k_mgd_smooth<T><<<grid(l), blk, 0, st>>>(A, c, ul, ld, fs, bl, ld, fs);
                VD_LAUNCH_CHECK();
            }
        return VD_OK;
    };
    auto precond = [&]() {           // z = V(r)
        int e;
        if ((e = zero_level(0, cz))) return e;
        return vcycle(0, cz, cr);
    };
    int rc;
    k_mgd_fill_int<<<(nsys + 255) / 256, 256, 0, st>>>(nsys, 0, done);
    VD_LAUNCH_CHECK();
    // x = 0 on the caller's array (land included), r = b
    k_mgd_zero_strided<T><<<grid(0), blk, 0, st>>>(n0, n1, u, ldu, fsu);
    VD_LAUNCH_CHECK();
    // r = b on the ocean nodes (land nodes carry no equation)
    {
        const MgdArgs<T> A = args(0);
        k_mgd_resid<T><<<grid(0), blk, 0, st>>>(A, u, ldu, fsu, b, ldb, fsb, cr);
        VD_LAUNCH_CHECK();
    }
    if ((rc = dot(cr, cr, 0))) return rc;
    if ((rc = precond())) return rc;
    if ((rc = dot(cr, cz, 1))) return rc;
    for (int it = 0; it < p->d.max_cycles; ++it) {
        k_mgd_p<T><<<dim3((ncell + 255) / 256, nsys), 256, 0, st>>>(ncell, done, beta, it == 0 ? 1 : 0, cz, cp);
        VD_LAUNCH_CHECK();
        {
            // q = -A p (the residual kernel with b = 0)
            const MgdArgs<T> A = args(0);
            k_mgd_resid<T><<<grid(0), blk, 0, st>>>(A, cp, n1, ncell, (const T*)nullptr, n1, ncell, cq);
            VD_LAUNCH_CHECK();
        }
        // sc[2] = rho / (p . q) = -alpha
        if ((rc = dot(cp, cq, 2))) return rc;
        k_mgd_xr<T><<<grid(0), blk, 0, st>>>(n0, n1, done, sc, cp, cq, u, ldu, fsu, cr);
        VD_LAUNCH_CHECK();
        if ((rc = dot(cr, cr, 3))) return rc;
        if ((rc = precond())) return rc;
        if ((rc = dot(cr, cz, 4))) return rc;
    }
    return VD_OK;
}

extern "C" vd_status vd_mgd_solve(const vd_mgd_plan* p, int batch, const void* b, long long ldb, long long fsb,
                                  void* u, long long ldu, long long fsu, double* rel, void* work, size_t work_bytes,
                                  void* stream)
{
    if (!p || batch < 1 || !b || !u || !work || ldb < p->d.n1 || ldu < p->d.n1 || fsb < ldb * p->d.n0 ||
        fsu < ldu * p->d.n0)
        return VD_ERR_ARG;
    if (work_bytes < vd_mgd_workspace_bytes(p, batch)) return VD_ERR_WORKSPACE;
    if (p->lv.size() < 2) return VD_ERR_UNSUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F64
               ? mgd_solve_t<double>(p, batch, (const double*)b, ldb, fsb, (double*)u, ldu, fsu, rel, (char*)work, st)
               : mgd_solve_t<float>(p, batch, (const float*)b, ldb, fsb, (float*)u, ldu, fsu, rel, (char*)work, st);
}

