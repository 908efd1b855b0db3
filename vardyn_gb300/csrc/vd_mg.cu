// Masked multigrid Helmholtz solver: div(c grad u) - lambda u = rhs on cell
// centres of a masked domain in an n0 x n1 rectangle, homogeneous Neumann
// walls on cell edges (mapping/models/model_qgsw/helmholtz_multigrid.py,
// MG_Helmholtz 156-419): damped Jacobi (omega = 0.95, 6 sweeps per smooth,
// 73-99), residual (102-114), cell-centred restriction / 9-3-3-1
// prolongation with mask-count divisors (117-151, 265-278), mask and
// coefficient hierarchies (248-293), full-multigrid start then max_ite
// V-cycles (322-419), bottom solve by pseudo-inverse (226-237) or Jacobi.
//
// A batch of nsys systems shares the grid and coefficient; system b uses
// lambda[b]. Arrays are row-major [nsys][n0][n1]. Every level keeps its
// mask, edge coefficients, divisors and Jacobi factor on the device; the
// recursion runs on the host and only launches kernels on the caller's
// stream, so a whole solve can be captured in a CUDA graph.
#include "vd_internal.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

namespace {

struct HLevel {
    int n0 = 0, n1 = 0;
    double d0 = 0, d1 = 0;
    std::vector<double> mask, cu, cv, divr, divp, factor;   // factor [nsys][n0][n1]
};

int mg_nlevels(int n)
{
    if (n <= 8) return 1;
    int h = 0;
    while (((n >> h) & 1) == 0) ++h;
    while ((n >> h) < 8) --h;
    return 1 + h;
}

double at(const std::vector<double>& a, int n0, int n1, int i, int j)
{
    return (i < 0 || j < 0 || i >= n0 || j >= n1) ? 0.0 : a[(size_t)i * n1 + j];
}

// pseudo-inverse of a symmetric matrix (cyclic Jacobi eigenvalues; the cut
// |lambda| <= 1e-15 max|lambda| of numpy.linalg.pinv's default rcond)
std::vector<double> pinv_sym(std::vector<double> A, int N)
{
    std::vector<double> V((size_t)N * N, 0.0);
    for (int i = 0; i < N; ++i) V[(size_t)i * N + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                const double v = A[(size_t)i * N + j] * A[(size_t)i * N + j];
                tot += v;
                if (i != j) off += v;
            }
        if (off <= 1e-30 * tot) break;
        for (int p = 0; p < N - 1; ++p)
            for (int q = p + 1; q < N; ++q) {
                const double apq = A[(size_t)p * N + q];
                if (apq == 0.0) continue;
                const double app = A[(size_t)p * N + p], aqq = A[(size_t)q * N + q];
                const double theta = (aqq - app) / (2 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
                const double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < N; ++k) {
                    const double akp = A[(size_t)k * N + p], akq = A[(size_t)k * N + q];
                    A[(size_t)k * N + p] = c * akp - s * akq;
                    A[(size_t)k * N + q] = s * akp + c * akq;
                }
                for (int k = 0; k < N; ++k) {
                    const double apk = A[(size_t)p * N + k], aqk = A[(size_t)q * N + k];
                    A[(size_t)p * N + k] = c * apk - s * aqk;
                    A[(size_t)q * N + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < N; ++k) {
                    const double vkp = V[(size_t)k * N + p], vkq = V[(size_t)k * N + q];
                    V[(size_t)k * N + p] = c * vkp - s * vkq;
                    V[(size_t)k * N + q] = s * vkp + c * vkq;
                }
            }
    }
    double emax = 0.0;
    for (int i = 0; i < N; ++i) emax = std::max(emax, std::fabs(A[(size_t)i * N + i]));
    std::vector<double> P((size_t)N * N, 0.0);
    for (int e = 0; e < N; ++e) {
        const double lam = A[(size_t)e * N + e];
        if (std::fabs(lam) <= 1e-15 * emax) continue;
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) P[(size_t)i * N + j] += V[(size_t)i * N + e] * V[(size_t)j * N + e] / lam;
    }
    return P;
}

}  // namespace

struct vd_mg_plan {
    int n0 = 0, n1 = 0, nsys = 0, dtype = VD_F64, nlev = 0, max_ite = 20, niter_bottom = -1;
    double omega = 0.95;
    std::vector<double> lambda;
    std::vector<HLevel> lv;
    int nb = 0;                          // bottom cells
    int lc = 0;                          // first level run by the one-block coarse kernel (nlev: none)
    void* dev = nullptr;
    struct DLev {
        const void *mask = nullptr, *cu = nullptr, *cv = nullptr, *factor = nullptr, *divr = nullptr,
                   *divp = nullptr;
    };
    std::vector<DLev> dl;
    const void* lam = nullptr;           // [nsys]
    const int32_t* bot_idx = nullptr;    // [nb] flat bottom cell index
    const void* bot_inv = nullptr;       // [nsys][nb][nb]
    // the bottom level's 6 niter_bottom damped sweeps as one linear map,
    // f = N rhs (+ M f on a one-level grid): [nsys][N, M][input k][output m]
    const void* bot_sm = nullptr;
    // the whole solve as one CUDA graph on plan-owned rhs / solution buffers
    // (captured at the first solve with a given workspace, replayed after)
    void* gbuf = nullptr;                // [2][nsys][n0][n1]: rhs, solution
    cudaStream_t gstream = nullptr;      // capture stream
    cudaGraphExec_t gexec = nullptr;
    const void* gws = nullptr;           // workspace the graph was captured with
    std::vector<size_t> ws_off;          // per level: f, rhs, tmp offsets (elements)
    size_t ws_elems = 0;
};

namespace vd {

// One level on the device. The edge coefficients are stored pre-scaled by
// 1/d0^2 and 1/d1^2 and the Jacobi factor pre-multiplied by omega: the sweep
// is then 7 FP64 instructions a cell (10 in the reference's grouping), the
// rate that bounds it on this part (same operator, rounding order differs).
template <typename T>
struct MgLev {
    int n0, n1;
    const T *mask, *cu, *cv, *factor, *lam;   // cu = c_u/d0^2, cv = c_v/d1^2, factor = omega mask/den
};

template <typename T>
__device__ __forceinline__ T fat(const T* f, int n0, int n1, int i, int j)
{
    return (i < 0 || j < 0 || i >= n0 || j >= n1) ? T(0) : f[(long long)i * n1 + j];
}

// Per-point arithmetic, shared by the level-wide kernels and the one-block
// coarse-level kernel so that both give the same bits.

// one damped Jacobi update at (i, j) (helmholtz_multigrid.py:86-98)
template <typename T>
__device__ __forceinline__ T mg_sweep_pt(const MgLev<T>& L, const T* F, T rhs, T factor, int i, int j, T omega)
{
    const long long o = (long long)i * L.n1 + j;
    const T cup = L.cu[(long long)(i + 1) * L.n1 + j], cui = L.cu[o];
    const T cvp = L.cv[(long long)i * (L.n1 + 1) + j + 1], cvi = L.cv[(long long)i * (L.n1 + 1) + j];
    const T s = cup * fat(F, L.n0, L.n1, i + 1, j) + cui * fat(F, L.n0, L.n1, i - 1, j) +
                cvp * fat(F, L.n0, L.n1, i, j + 1) + cvi * fat(F, L.n0, L.n1, i, j - 1);
    return factor * (s - rhs) + (T(1) - omega) * F[o];
}

// rhs - mask (div(c grad f) - lambda f) at (i, j)  (helmholtz_multigrid.py:102-114)
template <typename T>
__device__ __forceinline__ T mg_residual_pt(const MgLev<T>& L, const T* F, T rhs, T lam, int i, int j)
{
    const long long o = (long long)i * L.n1 + j;
    const T fc = F[o];
    const T cup = L.cu[(long long)(i + 1) * L.n1 + j], cui = L.cu[o];
    const T cvp = L.cv[(long long)i * (L.n1 + 1) + j + 1], cvi = L.cv[(long long)i * (L.n1 + 1) + j];
    const T hx = cup * (fat(F, L.n0, L.n1, i + 1, j) - fc) - cui * (fc - fat(F, L.n0, L.n1, i - 1, j));
    const T hy = cvp * (fat(F, L.n0, L.n1, i, j + 1) - fc) - cvi * (fc - fat(F, L.n0, L.n1, i, j - 1));
    const T Hf = (hx + hy - lam * fc) * L.mask[o];
    return rhs - Hf;
}

// (sum of the 2x2 fine cells) / div * mask_coarse at coarse (I, J)  (147-151)
template <typename T>
__device__ __forceinline__ T mg_restrict_pt(const T* fine, int n1c, int I, int J, const T* divr, const T* maskc)
{
    const int n1f = 2 * n1c;
    const T* F = fine + (long long)(2 * I) * n1f + 2 * J;
    const long long o = (long long)I * n1c + J;
    const T s = F[0] + F[n1f] + F[1] + F[n1f + 1];
    return s / divr[o] * maskc[o];
}

// prolong(coarse) / div * mask_fine at fine (i, j)  (117-144)
template <typename T>
__device__ __forceinline__ T mg_prolong_pt(const T* V, int n0c, int n1c, int i_f, int jf, const T* divp,
                                           const T* maskf)
{
    const int I = i_f >> 1, J = jf >> 1;
    const int di = (i_f & 1) ? 1 : -1, dj = (jf & 1) ? 1 : -1;
    const T q = T(9) * fat(V, n0c, n1c, I, J) + T(3) * (fat(V, n0c, n1c, I, J + dj) + fat(V, n0c, n1c, I + di, J)) +
                fat(V, n0c, n1c, I + di, J + dj);
    const long long o = (long long)i_f * (2 * n1c) + jf;
    return q / divp[o] * maskf[o];
}

template <typename T>
__global__ void k_mg_sweep(MgLev<T> L, const T* __restrict__ f, const T* __restrict__ rhs, T* __restrict__ out,
                           T omega)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y, b = blockIdx.z;
    if (j >= L.n1) return;
    const long long fs = (long long)L.n0 * L.n1, o = (long long)i * L.n1 + j;
    out[b * fs + o] = mg_sweep_pt(L, f + b * fs, rhs[b * fs + o], L.factor[b * fs + o], i, j, omega);
}

template <typename T>
__global__ void k_mg_residual(MgLev<T> L, const T* __restrict__ f, const T* __restrict__ rhs, T* __restrict__ res)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y, b = blockIdx.z;
    if (j >= L.n1) return;
    const long long fs = (long long)L.n0 * L.n1, o = (long long)i * L.n1 + j;
    res[b * fs + o] = mg_residual_pt(L, f + b * fs, rhs[b * fs + o], L.lam[b], i, j);
}

template <typename T>
__global__ void k_mg_restrict(int n0c, int n1c, const T* __restrict__ fine, const T* __restrict__ divr,
                              const T* __restrict__ maskc, T* __restrict__ coarse)
{
    const int J = blockIdx.x * blockDim.x + threadIdx.x;
    const int I = blockIdx.y, b = blockIdx.z;
    if (J >= n1c) return;
    const long long fsc = (long long)n0c * n1c;
    coarse[b * fsc + (long long)I * n1c + J] = mg_restrict_pt(fine + b * 4 * fsc, n1c, I, J, divr, maskc);
}

template <typename T>
__global__ void k_mg_prolong(int n0c, int n1c, const T* __restrict__ coarse, const T* __restrict__ divp,
                             const T* __restrict__ maskf, T* __restrict__ fine, int add)
{
    const int jf = blockIdx.x * blockDim.x + threadIdx.x;
    const int i_f = blockIdx.y, b = blockIdx.z;
    const int n1f = 2 * n1c;
    if (jf >= n1f) return;
    const long long fsc = (long long)n0c * n1c, fsf = 4 * fsc;
    const T v = mg_prolong_pt(coarse + b * fsc, n0c, n1c, i_f, jf, divp, maskf);
    const long long o = (long long)i_f * n1f + jf;
    fine[b * fsf + o] = add ? fine[b * fsf + o] + v : v;
}

// bottom: f[b][idx[m]] = sum_l rhs[b][idx[l]] inv[b][l][m]  (341-346)
template <typename T>
__global__ void k_mg_bottom(int nb, long long fs, const int32_t* __restrict__ idx, const T* __restrict__ inv,
                            const T* __restrict__ rhs, T* __restrict__ f)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (m >= nb) return;
    const T* R = rhs + b * fs;
    const T* P = inv + (long long)b * nb * nb;
    T s = T(0);
    for (int l = 0; l < nb; ++l) s += R[idx[l]] * P[(long long)l * nb + m];
    f[b * fs + idx[m]] = s;
}

// ---------------------------------------------------------------------------
// Coarse levels in one block per system. Below a few thousand cells a level's
// sweep is shorter than a kernel launch, and the bottom smoothing alone is
// 6 x niter_bottom sweeps per V-cycle; this kernel runs everything from level
// l0 down (the V-cycle, or the full-multigrid start) with the block's threads
// striding over the level and __syncthreads() between phases. The solution,
// right-hand side and scratch of every level from l0 down live in shared
// memory (level l0's come in from, and its solution goes back to, global
// memory); the coefficients are read-only global tables; the arithmetic is
// the per-point functions above.
// ---------------------------------------------------------------------------
constexpr int MG_MAXLEV = 16;

template <typename T>
struct MgCoarseArgs {
    int l0, nlev, niter_bottom, nb, fmg;
    T omega;
    MgLev<T> L[MG_MAXLEV];
    const T* divr[MG_MAXLEV];   // restriction divisor of coarse level l
    const T* divp[MG_MAXLEV];   // prolongation divisor of fine level l
    int soff[MG_MAXLEV];        // shared-memory offset of level l: f, rhs, scratch (n0 n1 each)
    T* f0;                      // level l0 solution (system-0 base): in (V-cycle) and out
    const T* rhs0;              // level l0 right-hand side (system-0 base)
    const int32_t* bot_idx;
    const T* bot_inv;
    const T* bot_sm;            // bottom smoothing as matrices, or nullptr
};

template <typename T>
struct MgcLevel {
    T *f, *rhs, *tmp;
    int n;
};

template <typename T>
__device__ __forceinline__ MgcLevel<T> mgc_level(const MgCoarseArgs<T>& A, T* sm, int l)
{
    MgcLevel<T> v;
    v.n = A.L[l].n0 * A.L[l].n1;
    v.f = sm + A.soff[l];
    v.rhs = v.f + v.n;
    v.tmp = v.rhs + v.n;
    return v;
}

template <typename T>
__device__ void mgc_smooth(const MgCoarseArgs<T>& A, T* sm, int l, int b, int times)
{
    const MgLev<T>& L = A.L[l];
    const MgcLevel<T> v = mgc_level(A, sm, l);
    const T* fac = L.factor + (long long)b * v.n;
    for (int t = 0; t < times; ++t)
        for (int s = 0; s < 6; ++s) {
            const T* src = (s % 2 == 0) ? v.f : v.tmp;
            T* dst = (s % 2 == 0) ? v.tmp : v.f;
            for (int o = threadIdx.x; o < v.n; o += blockDim.x) {
                const int i = o / L.n1, j = o - i * L.n1;
                dst[o] = mg_sweep_pt(L, src, v.rhs[o], __ldg(fac + o), i, j, A.omega);
            }
            __syncthreads();
        }
}

template <typename T>
__device__ void mgc_bottom(const MgCoarseArgs<T>& A, T* sm, int b)
{
    const int l = A.nlev - 1;
    if (A.niter_bottom > 0 && A.bot_sm != nullptr) {
        // f = N rhs (+ M f when the grid has one level; below it f is zero here)
        const MgcLevel<T> v = mgc_level(A, sm, l);
        const long long n2 = (long long)v.n * v.n;
        const T* Nm = A.bot_sm + (long long)b * 2 * n2;
        const T* Mm = Nm + n2;
        for (int m = threadIdx.x; m < v.n; m += blockDim.x) {
            T s = T(0);
            for (int k = 0; k < v.n; ++k) s += __ldg(Nm + (long long)k * v.n + m) * v.rhs[k];
            if (A.nlev == 1)
                for (int k = 0; k < v.n; ++k) s += __ldg(Mm + (long long)k * v.n + m) * v.f[k];
            v.tmp[m] = s;
        }
        __syncthreads();
        for (int m = threadIdx.x; m < v.n; m += blockDim.x) v.f[m] = v.tmp[m];
        __syncthreads();
        return;
    }
    if (A.niter_bottom > 0) {
        mgc_smooth(A, sm, l, b, A.niter_bottom);
        return;
    }
    const MgcLevel<T> v = mgc_level(A, sm, l);
    for (int o = threadIdx.x; o < v.n; o += blockDim.x) v.f[o] = T(0);
    __syncthreads();
    const T* P = A.bot_inv + (long long)b * A.nb * A.nb;
    for (int m = threadIdx.x; m < A.nb; m += blockDim.x) {
        T s = T(0);
        for (int k = 0; k < A.nb; ++k) s += v.rhs[__ldg(A.bot_idx + k)] * __ldg(P + (long long)k * A.nb + m);
        v.f[__ldg(A.bot_idx + m)] = s;
    }
    __syncthreads();
}

// rhs of level lc from a fine-level field (shared memory)
template <typename T>
__device__ void mgc_restrict(const MgCoarseArgs<T>& A, T* sm, const T* fine, int lc)
{
    const MgLev<T>& C = A.L[lc];
    const MgcLevel<T> v = mgc_level(A, sm, lc);
    for (int o = threadIdx.x; o < v.n; o += blockDim.x) {
        const int I = o / C.n1, J = o - I * C.n1;
        v.rhs[o] = mg_restrict_pt(fine, C.n1, I, J, A.divr[lc], C.mask);
    }
}

template <typename T>
__device__ void mgc_prolong(const MgCoarseArgs<T>& A, T* sm, int l, bool add)
{
    const MgLev<T>& Fl = A.L[l];
    const MgLev<T>& C = A.L[l + 1];
    const MgcLevel<T> vf = mgc_level(A, sm, l), vc = mgc_level(A, sm, l + 1);
    for (int o = threadIdx.x; o < vf.n; o += blockDim.x) {
        const int i = o / Fl.n1, j = o - i * Fl.n1;
        const T x = mg_prolong_pt(vc.f, C.n0, C.n1, i, j, A.divp[l], Fl.mask);
        vf.f[o] = add ? vf.f[o] + x : x;
    }
    __syncthreads();
}

template <typename T>
__device__ void mgc_vcycle(const MgCoarseArgs<T>& A, T* sm, int l0, int b)
{
    const int last = A.nlev - 1;
    for (int l = l0; l < last; ++l) {
        mgc_smooth(A, sm, l, b, 1);
        const MgLev<T>& L = A.L[l];
        const MgcLevel<T> v = mgc_level(A, sm, l);
        for (int o = threadIdx.x; o < v.n; o += blockDim.x) {
            const int i = o / L.n1, j = o - i * L.n1;
            v.tmp[o] = mg_residual_pt(L, v.f, v.rhs[o], L.lam[b], i, j);
        }
        __syncthreads();
        mgc_restrict(A, sm, v.tmp, l + 1);
        const MgcLevel<T> c = mgc_level(A, sm, l + 1);
        for (int o = threadIdx.x; o < c.n; o += blockDim.x) c.f[o] = T(0);
        __syncthreads();
    }
    mgc_bottom(A, sm, b);
    for (int l = last - 1; l >= l0; --l) {
        mgc_prolong(A, sm, l, true);
        mgc_smooth(A, sm, l, b, 1);
    }
}

template <typename T>
__global__ void __launch_bounds__(1024) k_mg_coarse(MgCoarseArgs<T> A)
{
    extern __shared__ __align__(16) unsigned char mg_smem[];
    T* sm = reinterpret_cast<T*>(mg_smem);
    const int b = blockIdx.x;
    const MgcLevel<T> v0 = mgc_level(A, sm, A.l0);
    const long long g0 = (long long)b * v0.n;
    for (int o = threadIdx.x; o < v0.n; o += blockDim.x) {
        v0.rhs[o] = A.rhs0[g0 + o];
        if (!A.fmg) v0.f[o] = A.f0[g0 + o];
    }
    __syncthreads();
    if (!A.fmg) {
        mgc_vcycle(A, sm, A.l0, b);
    } else {
        const int last = A.nlev - 1;
        for (int l = A.l0 + 1; l <= last; ++l) {
            mgc_restrict(A, sm, mgc_level(A, sm, l - 1).rhs, l);
            __syncthreads();
        }
        const MgcLevel<T> vb = mgc_level(A, sm, last);
        for (int o = threadIdx.x; o < vb.n; o += blockDim.x) vb.f[o] = T(0);
        __syncthreads();
        mgc_bottom(A, sm, b);
        for (int l = last - 1; l >= A.l0; --l) {
            mgc_prolong(A, sm, l, false);
            mgc_vcycle(A, sm, l, b);
        }
    }
    for (int o = threadIdx.x; o < v0.n; o += blockDim.x) A.f0[g0 + o] = v0.f[o];
}

template <typename T>
__global__ void k_mg_zero(long long n, T* __restrict__ x)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) x[k] = T(0);
}

}  // namespace vd

namespace {

template <typename T>
struct MgRun {
    const vd_mg_plan* p;
    T* ws;
    cudaStream_t st;

    vd::MgLev<T> lev(int l) const
    {
        const vd_mg_plan::DLev& D = p->dl[l];
        vd::MgLev<T> L;
        L.n0 = p->lv[l].n0;
        L.n1 = p->lv[l].n1;
        L.mask = (const T*)D.mask;
        L.cu = (const T*)D.cu;
        L.cv = (const T*)D.cv;
        L.factor = (const T*)D.factor;
        L.lam = (const T*)p->lam;
        return L;
    }
    T* buf(int l, int which) const { return ws + p->ws_off[3 * l + which]; }
    long long nel(int l) const { return (long long)p->nsys * p->lv[l].n0 * p->lv[l].n1; }
    dim3 grid(int n0, int n1) const { return dim3((unsigned)((n1 + 127) / 128), (unsigned)n0, (unsigned)p->nsys); }

    int zero(T* x, long long n) const
    {
        vd::k_mg_zero<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, x);
        VD_LAUNCH_CHECK();
        return VD_OK;
    }
    // `times` smooths of 6 damped sweeps, ping-pong through the level's tmp buffer
    int smooth(int l, T* f, const T* rhs, int times) const
    {
        const vd::MgLev<T> L = lev(l);
        T* tmp = buf(l, 2);
        const dim3 g = grid(L.n0, L.n1);
        for (int t = 0; t < times; ++t)
            for (int s = 0; s < 6; ++s) {
                const T* src = (s % 2 == 0) ? f : tmp;
                T* dst = (s % 2 == 0) ? tmp : f;
                vd::k_mg_sweep<T><<<g, 128, 0, st>>>(L, src, rhs, dst, T(p->omega));
                VD_LAUNCH_CHECK();
            }
        return VD_OK;
    }
    int bottom(T* f, const T* rhs) const
    {
        const int l = p->nlev - 1;
        if (p->niter_bottom <= 0) {
            const long long fs = (long long)p->lv[l].n0 * p->lv[l].n1;
            int rc = zero(f, nel(l));
            if (rc) return rc;
            if (p->nb > 0) {
                vd::k_mg_bottom<T><<<dim3((unsigned)((p->nb + 127) / 128), (unsigned)p->nsys), 128, 0, st>>>(
                    p->nb, fs, p->bot_idx, (const T*)p->bot_inv, rhs, f);
                VD_LAUNCH_CHECK();
            }
            return VD_OK;
        }
        return smooth(l, f, rhs, p->niter_bottom);
    }
    // levels >= l0 in one block per system (p->lc <= l0): a V-cycle on (f, rhs)
    // at l0, or (fmg) the full-multigrid start from the restricted rhs at l0
    int coarse(T* f, const T* rhs, int l0, bool fmg) const
    {
        vd::MgCoarseArgs<T> A;
        A.l0 = l0; A.nlev = p->nlev; A.niter_bottom = p->niter_bottom; A.nb = p->nb; A.fmg = fmg ? 1 : 0;
        A.omega = T(p->omega);
        int off = 0;
        for (int l = 0; l < p->nlev; ++l) {
            A.L[l] = lev(l);
            A.divr[l] = (const T*)p->dl[l].divr;
            A.divp[l] = (const T*)p->dl[l].divp;
            A.soff[l] = off;
            if (l >= l0) off += 3 * p->lv[l].n0 * p->lv[l].n1;
        }
        A.f0 = f;
        A.rhs0 = rhs;
        A.bot_idx = p->bot_idx;
        A.bot_inv = (const T*)p->bot_inv;
        A.bot_sm = (const T*)p->bot_sm;
        vd::k_mg_coarse<T><<<(unsigned)p->nsys, 1024, (size_t)off * sizeof(T), st>>>(A);
        VD_LAUNCH_CHECK();
        return VD_OK;
    }
    int vcycle(T* f, const T* rhs, int l) const
    {
        if (l >= p->lc) return coarse(f, rhs, l, false);
        if (l == p->nlev - 1) return bottom(f, rhs);
        int rc;
        if ((rc = smooth(l, f, rhs, 1))) return rc;
        const vd::MgLev<T> L = lev(l);
        T* res = buf(l, 2);
        vd::k_mg_residual<T><<<grid(L.n0, L.n1), 128, 0, st>>>(L, f, rhs, res);
        VD_LAUNCH_CHECK();
        const int n0c = p->lv[l + 1].n0, n1c = p->lv[l + 1].n1;
        T* rcz = buf(l + 1, 1);
        T* ec = buf(l + 1, 0);
        vd::k_mg_restrict<T><<<grid(n0c, n1c), 128, 0, st>>>(n0c, n1c, res, (const T*)p->dl[l + 1].divr,
                                                              (const T*)p->dl[l + 1].mask, rcz);
        VD_LAUNCH_CHECK();
        if ((rc = zero(ec, nel(l + 1)))) return rc;
        if ((rc = vcycle(ec, rcz, l + 1))) return rc;
        vd::k_mg_prolong<T><<<grid(L.n0, L.n1), 128, 0, st>>>(n0c, n1c, ec, (const T*)p->dl[l].divp,
                                                              (const T*)p->dl[l].mask, f, 1);
        VD_LAUNCH_CHECK();
        return smooth(l, f, rhs, 1);
    }
    // FMG_Helmholtz (helmholtz_multigrid.py:380-419)
    int solve(const T* rhs, T* out) const
    {
        const int n = p->nlev;
        int rc;
        if (n == 1) {
            if ((rc = zero(out, nel(0)))) return rc;
            if ((rc = bottom(out, rhs))) return rc;
        } else if (p->lc < n) {
            // host levels down to lc, then the coarse kernel's full-multigrid start
            const int lc = p->lc;
            for (int i = 1; i <= lc; ++i) {
                const T* src = (i == 1) ? rhs : buf(i - 1, 1);
                vd::k_mg_restrict<T><<<grid(p->lv[i].n0, p->lv[i].n1), 128, 0, st>>>(
                    p->lv[i].n0, p->lv[i].n1, src, (const T*)p->dl[i].divr, (const T*)p->dl[i].mask, buf(i, 1));
                VD_LAUNCH_CHECK();
            }
            if ((rc = coarse(lc == 0 ? out : buf(lc, 0), lc == 0 ? rhs : buf(lc, 1), lc, true))) return rc;
            for (int L = lc - 1; L >= 0; --L) {
                T* fL = (L == 0) ? out : buf(L, 0);
                const T* rL = (L == 0) ? rhs : buf(L, 1);
                vd::k_mg_prolong<T><<<grid(p->lv[L].n0, p->lv[L].n1), 128, 0, st>>>(
                    p->lv[L + 1].n0, p->lv[L + 1].n1, buf(L + 1, 0), (const T*)p->dl[L].divp,
                    (const T*)p->dl[L].mask, fL, 0);
                VD_LAUNCH_CHECK();
                if ((rc = vcycle(fL, rL, L))) return rc;
            }
        } else {
            for (int i = 1; i < n; ++i) {
                const T* src = (i == 1) ? rhs : buf(i - 1, 1);
                vd::k_mg_restrict<T><<<grid(p->lv[i].n0, p->lv[i].n1), 128, 0, st>>>(
                    p->lv[i].n0, p->lv[i].n1, src, (const T*)p->dl[i].divr, (const T*)p->dl[i].mask, buf(i, 1));
                VD_LAUNCH_CHECK();
            }
            T* fb = buf(n - 1, 0);
            if ((rc = zero(fb, nel(n - 1)))) return rc;
            if ((rc = bottom(fb, buf(n - 1, 1)))) return rc;
            for (int i = 2; i <= n; ++i) {
                const int L = n - i;
                T* fL = (L == 0) ? out : buf(L, 0);
                const T* rL = (L == 0) ? rhs : buf(L, 1);
                vd::k_mg_prolong<T><<<grid(p->lv[L].n0, p->lv[L].n1), 128, 0, st>>>(
                    p->lv[L + 1].n0, p->lv[L + 1].n1, buf(L + 1, 0), (const T*)p->dl[L].divp,
                    (const T*)p->dl[L].mask, fL, 0);
                VD_LAUNCH_CHECK();
                if ((rc = vcycle(fL, rL, L))) return rc;
            }
        }
        for (int it = 0; it < p->max_ite; ++it)
            if ((rc = vcycle(out, rhs, 0))) return rc;
        return VD_OK;
    }
};

// ---- hierarchy construction (host, float64; helmholtz_multigrid.py:248-293) ----
std::vector<double> restrict_h(const std::vector<double>& v, int n0, int n1, const std::vector<double>* div, double d)
{
    const int n0c = n0 / 2, n1c = n1 / 2;
    std::vector<double> o((size_t)n0c * n1c);
    for (int I = 0; I < n0c; ++I)
        for (int J = 0; J < n1c; ++J) {
            const double s = v[(size_t)(2 * I) * n1 + 2 * J] + v[(size_t)(2 * I + 1) * n1 + 2 * J] +
                             v[(size_t)(2 * I) * n1 + 2 * J + 1] + v[(size_t)(2 * I + 1) * n1 + 2 * J + 1];
            o[(size_t)I * n1c + J] = s / (div ? (*div)[(size_t)I * n1c + J] : d);
        }
    return o;
}

std::vector<double> prolong_h(const std::vector<double>& v, int n0c, int n1c)
{
    const int n0 = 2 * n0c, n1 = 2 * n1c;
    std::vector<double> o((size_t)n0 * n1);
    for (int i = 0; i < n0; ++i)
        for (int j = 0; j < n1; ++j) {
            const int I = i >> 1, J = j >> 1, di = (i & 1) ? 1 : -1, dj = (j & 1) ? 1 : -1;
            o[(size_t)i * n1 + j] = 9 * at(v, n0c, n1c, I, J) + 3 * (at(v, n0c, n1c, I, J + dj) +
                                    at(v, n0c, n1c, I + di, J)) + at(v, n0c, n1c, I + di, J + dj);
        }
    return o;
}

void uv_masks(const std::vector<double>& m, int n0, int n1, std::vector<double>& mu, std::vector<double>& mv)
{
    mu.assign((size_t)(n0 + 1) * n1, 0.0);
    mv.assign((size_t)n0 * (n1 + 1), 0.0);
    for (int i = 0; i <= n0; ++i)
        for (int j = 0; j < n1; ++j) mu[(size_t)i * n1 + j] = (at(m, n0, n1, i - 1, j) + at(m, n0, n1, i, j)) > 1.5;
    for (int i = 0; i < n0; ++i)
        for (int j = 0; j <= n1; ++j)
            mv[(size_t)i * (n1 + 1) + j] = (at(m, n0, n1, i, j - 1) + at(m, n0, n1, i, j)) > 1.5;
}

// H f on one level (helmholtz_multigrid.py:53-62), for the bottom matrix
void helm_apply(const HLevel& L, double lam, const std::vector<double>& f, std::vector<double>& out)
{
    const int n0 = L.n0, n1 = L.n1;
    out.assign((size_t)n0 * n1, 0.0);
    for (int i = 0; i < n0; ++i)
        for (int j = 0; j < n1; ++j) {
            const double fc = f[(size_t)i * n1 + j];
            const double hx = L.cu[(size_t)(i + 1) * n1 + j] * (at(f, n0, n1, i + 1, j) - fc) -
                              L.cu[(size_t)i * n1 + j] * (fc - at(f, n0, n1, i - 1, j));
            const double hy = L.cv[(size_t)i * (n1 + 1) + j + 1] * (at(f, n0, n1, i, j + 1) - fc) -
                              L.cv[(size_t)i * (n1 + 1) + j] * (fc - at(f, n0, n1, i, j - 1));
            out[(size_t)i * n1 + j] = (hx / (L.d0 * L.d0) + hy / (L.d1 * L.d1) - lam * fc) * L.mask[(size_t)i * n1 + j];
        }
}

// The bottom level's K damped Jacobi sweeps (the device formula, in float64)
// as f_K = M f_0 + N rhs, by sweeping unit vectors; appended to `out` as
// N then M (zeros when !with_m), each [input k][output m].
void bottom_sweep_matrices(const HLevel& L, const double* factor, double omega, int K, bool with_m,
                           std::vector<double>& out)
{
    const int n0 = L.n0, n1 = L.n1, n = n0 * n1;
    const double dxm2 = 1.0 / (L.d0 * L.d0), dym2 = 1.0 / (L.d1 * L.d1);
    std::vector<double> f(n), g(n), r(n);
    auto sweep = [&](const std::vector<double>& src, std::vector<double>& dst) {
        for (int i = 0; i < n0; ++i)
            for (int j = 0; j < n1; ++j) {
                const size_t o = (size_t)i * n1 + j;
                const double sx = L.cu[(size_t)(i + 1) * n1 + j] * at(src, n0, n1, i + 1, j) +
                                  L.cu[o] * at(src, n0, n1, i - 1, j);
                const double sy = L.cv[(size_t)i * (n1 + 1) + j + 1] * at(src, n0, n1, i, j + 1) +
                                  L.cv[(size_t)i * (n1 + 1) + j] * at(src, n0, n1, i, j - 1);
                const double s = dxm2 * sx + dym2 * sy;
                dst[o] = omega * factor[o] * (s - r[o]) + (1.0 - omega) * src[o];
            }
    };
    const size_t base = out.size();
    out.resize(base + 2 * (size_t)n * n, 0.0);
    for (int pass = 0; pass < (with_m ? 2 : 1); ++pass)
        for (int k = 0; k < n; ++k) {
            std::fill(f.begin(), f.end(), 0.0);
            std::fill(r.begin(), r.end(), 0.0);
            (pass == 0 ? r : f)[k] = 1.0;
            for (int t = 0; t < K; ++t) {
                sweep(f, g);
                f.swap(g);
            }
            double* dst = out.data() + base + (size_t)pass * n * n + (size_t)k * n;
            std::copy(f.begin(), f.end(), dst);
        }
}

struct Blob {
    std::vector<unsigned char> b;
    size_t add(const void* p, size_t n)
    {
        const size_t off = (b.size() + 255) & ~size_t(255);
        b.resize(off + n + 1);
        if (n) std::memcpy(b.data() + off, p, n);
        return off;
    }
    template <typename T>
    size_t addv(const std::vector<double>& v)
    {
        std::vector<T> t(v.begin(), v.end());
        return add(t.data(), t.size() * sizeof(T));
    }
};

template <typename T>
int mg_upload(vd_mg_plan* p, const std::vector<int32_t>& idx, const std::vector<double>& inv,
              const std::vector<double>& bsm)
{
    Blob bl;
    struct Off { size_t mask, cu, cv, factor, divr, divp; };
    std::vector<Off> off(p->nlev);
    for (int l = 0; l < p->nlev; ++l) {
        const HLevel& L = p->lv[l];
        off[l].mask = bl.addv<T>(L.mask);
        const double dxm2 = 1.0 / (L.d0 * L.d0), dym2 = 1.0 / (L.d1 * L.d1);
        std::vector<double> cus(L.cu), cvs(L.cv), fw(L.factor);
        for (double& v : cus) v *= dxm2;
        for (double& v : cvs) v *= dym2;
        for (double& v : fw) v *= p->omega;
        off[l].cu = bl.addv<T>(cus);
        off[l].cv = bl.addv<T>(cvs);
        off[l].factor = bl.addv<T>(fw);
        off[l].divr = L.divr.empty() ? 0 : bl.addv<T>(L.divr);
        off[l].divp = L.divp.empty() ? 0 : bl.addv<T>(L.divp);
    }
    const size_t o_lam = bl.addv<T>(p->lambda);
    const size_t o_idx = bl.add(idx.data(), idx.size() * sizeof(int32_t));
    const size_t o_inv = bl.addv<T>(inv);
    const size_t o_bsm = bl.addv<T>(bsm);
    VD_CUDA_TRY(cudaMalloc(&p->dev, bl.b.size()));
    VD_CUDA_TRY(cudaMemcpy(p->dev, bl.b.data(), bl.b.size(), cudaMemcpyHostToDevice));
    unsigned char* b = (unsigned char*)p->dev;
    p->dl.resize(p->nlev);
    for (int l = 0; l < p->nlev; ++l) {
        p->dl[l].mask = b + off[l].mask;
        p->dl[l].cu = b + off[l].cu;
        p->dl[l].cv = b + off[l].cv;
        p->dl[l].factor = b + off[l].factor;
        p->dl[l].divr = p->lv[l].divr.empty() ? nullptr : b + off[l].divr;
        p->dl[l].divp = p->lv[l].divp.empty() ? nullptr : b + off[l].divp;
    }
    p->lam = b + o_lam;
    p->bot_idx = (const int32_t*)(b + o_idx);
    p->bot_inv = b + o_inv;
    p->bot_sm = bsm.empty() ? nullptr : b + o_bsm;
    return VD_OK;
}

}  // namespace

extern "C" vd_status vd_mg_plan_create(vd_mg_plan** out, const vd_mg_desc* d)
{
    if (!out || !d) return VD_ERR_ARG;
    *out = nullptr;
    if (d->n0 < 1 || d->n1 < 1 || d->nsys < 1 || !d->lambda_host || !d->coef_u_host || !d->coef_v_host ||
        !(d->d0 > 0) || !(d->d1 > 0) || d->max_ite < 0 || (d->dtype != VD_F32 && d->dtype != VD_F64))
        return VD_ERR_ARG;
    const int nlev = d->n_levels > 0 ? d->n_levels : std::min(mg_nlevels(d->n0), mg_nlevels(d->n1));
    const int N = 1 << (nlev - 1);
    if (d->n0 % N || d->n1 % N) return VD_ERR_ARG;
    vd_mg_plan* p = new (std::nothrow) vd_mg_plan();
    if (!p) return VD_ERR_ARG;
    p->n0 = d->n0; p->n1 = d->n1; p->nsys = d->nsys; p->dtype = d->dtype; p->nlev = nlev;
    p->max_ite = d->max_ite; p->niter_bottom = d->niter_bottom;
    p->lambda.assign(d->lambda_host, d->lambda_host + d->nsys);
    // level 0
    p->lv.resize(nlev);
    HLevel& L0 = p->lv[0];
    L0.n0 = d->n0; L0.n1 = d->n1; L0.d0 = d->d0; L0.d1 = d->d1;
    L0.mask.assign((size_t)d->n0 * d->n1, 1.0);
    if (d->mask_host) std::copy(d->mask_host, d->mask_host + (size_t)d->n0 * d->n1, L0.mask.begin());
    std::vector<double> mu, mv;
    uv_masks(L0.mask, L0.n0, L0.n1, mu, mv);
    std::vector<double> cu0(d->coef_u_host, d->coef_u_host + (size_t)(d->n0 + 1) * d->n1);
    std::vector<double> cv0(d->coef_v_host, d->coef_v_host + (size_t)d->n0 * (d->n1 + 1));
    std::vector<double> coef((size_t)d->n0 * d->n1);
    for (int i = 0; i < d->n0; ++i)
        for (int j = 0; j < d->n1; ++j)
            coef[(size_t)i * d->n1 + j] = 0.25 * (cu0[(size_t)(i + 1) * d->n1 + j] + cu0[(size_t)i * d->n1 + j] +
                                                  cv0[(size_t)i * (d->n1 + 1) + j + 1] +
                                                  cv0[(size_t)i * (d->n1 + 1) + j]);
    L0.cu.resize(cu0.size());
    L0.cv.resize(cv0.size());
    for (size_t k = 0; k < cu0.size(); ++k) L0.cu[k] = cu0[k] * mu[k];
    for (size_t k = 0; k < cv0.size(); ++k) L0.cv[k] = cv0[k] * mv[k];
    for (int l = 1; l < nlev; ++l) {
        const HLevel& F = p->lv[l - 1];
        HLevel& C = p->lv[l];
        C.n0 = F.n0 / 2; C.n1 = F.n1 / 2; C.d0 = F.d0 * 2; C.d1 = F.d1 * 2;
        std::vector<double> m4 = restrict_h(F.mask, F.n0, F.n1, nullptr, 4.0);
        C.mask.resize(m4.size());
        for (size_t k = 0; k < m4.size(); ++k) C.mask[k] = m4[k] > 0.5;
        C.divr = restrict_h(F.mask, F.n0, F.n1, nullptr, 1.0);
        for (double& v : C.divr) v = std::max(v, 1.0);
        coef = restrict_h(coef, F.n0, F.n1, &C.divr, 0.0);
        for (size_t k = 0; k < coef.size(); ++k) coef[k] *= C.mask[k];
        uv_masks(C.mask, C.n0, C.n1, mu, mv);
        C.cu.assign((size_t)(C.n0 + 1) * C.n1, 0.0);
        C.cv.assign((size_t)C.n0 * (C.n1 + 1), 0.0);
        for (int i = 0; i <= C.n0; ++i)
            for (int j = 0; j < C.n1; ++j)
                C.cu[(size_t)i * C.n1 + j] = (at(coef, C.n0, C.n1, i - 1, j) + at(coef, C.n0, C.n1, i, j)) / 2 *
                                             mu[(size_t)i * C.n1 + j];
        for (int i = 0; i < C.n0; ++i)
            for (int j = 0; j <= C.n1; ++j)
                C.cv[(size_t)i * (C.n1 + 1) + j] = (at(coef, C.n0, C.n1, i, j - 1) + at(coef, C.n0, C.n1, i, j)) /
                                                   2 * mv[(size_t)i * (C.n1 + 1) + j];
    }
    for (int l = 0; l + 1 < nlev; ++l) {
        p->lv[l].divp = prolong_h(p->lv[l + 1].mask, p->lv[l + 1].n0, p->lv[l + 1].n1);
        for (double& v : p->lv[l].divp) v = std::max(v, 1.0);
    }
    for (int l = 0; l < nlev; ++l) {
        HLevel& L = p->lv[l];
        const double dxm2 = 1.0 / (L.d0 * L.d0), dym2 = 1.0 / (L.d1 * L.d1);
        L.factor.assign((size_t)p->nsys * L.n0 * L.n1, 0.0);
        for (int b = 0; b < p->nsys; ++b)
            for (int i = 0; i < L.n0; ++i)
                for (int j = 0; j < L.n1; ++j) {
                    const double den = p->lambda[b] +
                                       dxm2 * (L.cu[(size_t)(i + 1) * L.n1 + j] + L.cu[(size_t)i * L.n1 + j]) +
                                       dym2 * (L.cv[(size_t)i * (L.n1 + 1) + j + 1] + L.cv[(size_t)i * (L.n1 + 1) + j]);
                    L.factor[((size_t)b * L.n0 + i) * L.n1 + j] = L.mask[(size_t)i * L.n1 + j] / den;
                }
    }
    // bottom pseudo-inverse
    std::vector<int32_t> idx;
    std::vector<double> inv;
    const HLevel& Bt = p->lv[nlev - 1];
    if (p->niter_bottom <= 0) {
        for (int i = 0; i < Bt.n0; ++i)
            for (int j = 0; j < Bt.n1; ++j)
                if (Bt.mask[(size_t)i * Bt.n1 + j] != 0) idx.push_back(i * Bt.n1 + j);
        p->nb = (int)idx.size();
        if (p->nb > 4096) {
            delete p;
            return VD_ERR_UNSUPPORTED;
        }
        inv.assign((size_t)p->nsys * p->nb * p->nb, 0.0);
        std::vector<double> e((size_t)Bt.n0 * Bt.n1), He;
        for (int b = 0; b < p->nsys; ++b) {
            std::vector<double> H((size_t)p->nb * p->nb);
            for (int k = 0; k < p->nb; ++k) {
                std::fill(e.begin(), e.end(), 0.0);
                e[idx[k]] = 1.0;
                helm_apply(Bt, p->lambda[b], e, He);
                for (int jrow = 0; jrow < p->nb; ++jrow) H[(size_t)jrow * p->nb + k] = He[idx[jrow]];
            }
            const std::vector<double> P = pinv_sym(H, p->nb);
            std::copy(P.begin(), P.end(), inv.begin() + (size_t)b * p->nb * p->nb);
        }
    }
    // workspace: per level f, rhs, tmp
    size_t offw = 0;
    p->ws_off.resize(3 * nlev);
    for (int l = 0; l < nlev; ++l)
        for (int w = 0; w < 3; ++w) {
            p->ws_off[3 * l + w] = offw;
            offw += (size_t)p->nsys * p->lv[l].n0 * p->lv[l].n1;
            offw = (offw + 63) & ~size_t(63);
        }
    p->ws_elems = offw;
    // the one-block coarse kernel takes the levels of at most 4096 cells (1024
    // in float64: one SM's FP64 rate is ~1/64 of its FP32 rate, so a float64
    // level of 3072 cells runs faster spread over the GPU) whose solution, rhs
    // and scratch fit 200 KB of shared memory
    p->lc = nlev;
    const size_t esz = p->dtype == VD_F64 ? 8 : 4;
    const long long max_cells = p->dtype == VD_F64 ? 1024 : 4096;
    for (int l = 0; l < nlev; ++l) {
        size_t sm = 0;
        for (int k = l; k < nlev; ++k) sm += 3 * (size_t)p->lv[k].n0 * p->lv[k].n1 * esz;
        if ((long long)p->lv[l].n0 * p->lv[l].n1 <= max_cells && sm <= 200 * 1024) {
            p->lc = l;
            break;
        }
    }
    if (nlev > vd::MG_MAXLEV) p->lc = nlev;
    if (p->lc < nlev) {
        const cudaError_t e = p->dtype == VD_F64
            ? cudaFuncSetAttribute(vd::k_mg_coarse<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024)
            : cudaFuncSetAttribute(vd::k_mg_coarse<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e != cudaSuccess) {
            if (p->dev) cudaFree(p->dev);
            delete p;
            return VD_ERR_CUDA;
        }
    }
    // bottom smoothing of the coarse kernel as matrices (bottom levels of at
    // most 512 cells: 2 x 512^2 entries a system, built in well under a second)
    std::vector<double> bsm;
    if (p->niter_bottom > 0 && p->lc < nlev && (long long)Bt.n0 * Bt.n1 <= 512) {
        const size_t nbc = (size_t)Bt.n0 * Bt.n1;
        for (int b = 0; b < p->nsys; ++b)
            bottom_sweep_matrices(Bt, Bt.factor.data() + b * nbc, p->omega, 6 * p->niter_bottom, nlev == 1, bsm);
    }
    const int st = p->dtype == VD_F64 ? mg_upload<double>(p, idx, inv, bsm) : mg_upload<float>(p, idx, inv, bsm);
    if (st != VD_OK) {
        if (p->dev) cudaFree(p->dev);
        delete p;
        return st;
    }
    *out = p;
    return VD_OK;
}

extern "C" vd_status vd_mg_plan_destroy(vd_mg_plan* p)
{
    if (!p) return VD_ERR_ARG;
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    if (p->gstream) cudaStreamDestroy(p->gstream);
    if (p->gbuf) cudaFree(p->gbuf);
    if (p->dev) cudaFree(p->dev);
    delete p;
    return VD_OK;
}

extern "C" int vd_mg_levels(const vd_mg_plan* p) { return p ? p->nlev : 0; }

extern "C" size_t vd_mg_workspace_bytes(const vd_mg_plan* p)
{
    return p ? p->ws_elems * (p->dtype == VD_F64 ? 8 : 4) : 0;
}

static int mg_run(const vd_mg_plan* p, const void* rhs, void* f, void* ws, cudaStream_t st)
{
    if (p->dtype == VD_F64) {
        MgRun<double> r{p, (double*)ws, st};
        return r.solve((const double*)rhs, (double*)f);
    }
    MgRun<float> r{p, (float*)ws, st};
    return r.solve((const float*)rhs, (float*)f);
}

// (Re)capture the solve on the plan's buffers with workspace ws.
static int mg_capture(vd_mg_plan* p, void* ws)
{
    const size_t bytes = (size_t)p->nsys * p->n0 * p->n1 * (p->dtype == VD_F64 ? 8 : 4);
    if (!p->gbuf) VD_CUDA_TRY(cudaMalloc(&p->gbuf, 2 * bytes));
    if (!p->gstream) VD_CUDA_TRY(cudaStreamCreateWithFlags(&p->gstream, cudaStreamNonBlocking));
    if (p->gexec) {
        cudaGraphExecDestroy(p->gexec);
        p->gexec = nullptr;
    }
    char* g = (char*)p->gbuf;
    VD_CUDA_TRY(cudaStreamBeginCapture(p->gstream, cudaStreamCaptureModeRelaxed));
    const int rc = mg_run(p, g, g + bytes, ws, p->gstream);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(p->gstream, &graph);
    if (rc != VD_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    VD_CUDA_TRY(ec);
    const cudaError_t ei = cudaGraphInstantiate(&p->gexec, graph, 0);
    cudaGraphDestroy(graph);
    VD_CUDA_TRY(ei);
    p->gws = ws;
    return VD_OK;
}

extern "C" vd_status vd_mg_solve(const vd_mg_plan* p, const void* rhs, void* f, void* ws, size_t wsb, void* stream)
{
    if (!p || !rhs || !f || !ws) return VD_ERR_ARG;
    if (wsb < vd_mg_workspace_bytes(p)) return VD_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    // a caller that is itself capturing records the launches directly
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    VD_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone) return mg_run(p, rhs, f, ws, st);
    // a solve is ~25 kernel launches per level per V-cycle; replaying them as
    // one graph removes their host launch cost
    vd_mg_plan* q = const_cast<vd_mg_plan*>(p);
    if (!q->gexec || q->gws != ws) {
        const int rc = mg_capture(q, ws);
        if (rc != VD_OK) return rc;
    }
    const size_t bytes = (size_t)p->nsys * p->n0 * p->n1 * (p->dtype == VD_F64 ? 8 : 4);
    char* g = (char*)q->gbuf;
    VD_CUDA_TRY(cudaMemcpyAsync(g, rhs, bytes, cudaMemcpyDeviceToDevice, st));
    VD_CUDA_TRY(cudaGraphLaunch(q->gexec, st));
    VD_CUDA_TRY(cudaMemcpyAsync(f, g + bytes, bytes, cudaMemcpyDeviceToDevice, st));
    return VD_OK;
}

extern "C" vd_status vd_mg_residual(const vd_mg_plan* p, const void* f, const void* rhs, void* res, void* stream)
{
    if (!p || !f || !rhs || !res) return VD_ERR_ARG;
    const dim3 g((unsigned)((p->n1 + 127) / 128), (unsigned)p->n0, (unsigned)p->nsys);
    if (p->dtype == VD_F64) {
        MgRun<double> r{p, nullptr, (cudaStream_t)stream};
        vd::k_mg_residual<double><<<g, 128, 0, (cudaStream_t)stream>>>(r.lev(0), (const double*)f,
                                                                       (const double*)rhs, (double*)res);
    } else {
        MgRun<float> r{p, nullptr, (cudaStream_t)stream};
        vd::k_mg_residual<float><<<g, 128, 0, (cudaStream_t)stream>>>(r.lev(0), (const float*)f, (const float*)rhs,
                                                                      (float*)res);
    }
    VD_LAUNCH_CHECK();
    return VD_OK;
}
