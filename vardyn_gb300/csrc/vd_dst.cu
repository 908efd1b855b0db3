// Helmholtz PV->SSH inversion on a rectangle with Dirichlet walls.
//
// The reference inverts g/f*lap5 - g*f/c^2 by a 2-D orthonormal DST-I,
// division by the operator's eigenvalues and a second 2-D DST-I
// (mapping/models/model_qg1l/jqgm.py:75-91, eigenvalues 166-172). DST-I
// vectors are the exact eigenvectors of the 1-D Dirichlet second difference,
// so the same solution is obtained with ONE transform direction:
//
//   1. DST-I along x of every interior row          (dense half-size GEMMs)
//   2. for every x-wavenumber k, the tridiagonal system along y
//        a*X[j-1] + b_k*X[j] + a*X[j+1] = F[j],  a = g/f/dy^2,
//        b_k = g/f*(-2/dy^2 + mu_k) - g*f/c^2,  mu_k = 2(cos(pi(k+1)/(nx-1))-1)/dx^2
//      (Thomas algorithm with precomputed multipliers)
//   3. DST-I along x again (the orthonormal DST-I is its own inverse).
//
// DST-I even/odd split: with n = nx-2, S[p][k] = sqrt(2/(n+1)) sin(pi(p+1)(k+1)/(n+1))
// satisfies S[n-1-p][k] = (-1)^k S[p][k], so
//   forward:  F_even-k = (x[p] + x[n-1-p]) . Wodd,   F_odd-k = (x[p] - x[n-1-p]) . Weven
//   inverse:  A = Xe . Wodd^T, B = Xo . Weven;  y[p] = A+B, y[n-1-p] = A-B
// which halves the multiply-adds of a dense transform. Spectral rows are kept
// in parity-split order: columns [0, ne) hold k = 0,2,4..., [ne, n) hold k = 1,3,...
#include "vd_internal.cuh"
#include <vector>
#include <mutex>
#include <algorithm>
#include <cmath>

namespace vd {

template <typename T> struct Vec8;
template <> struct Vec8<float> {
    static __device__ __forceinline__ void load(const float* p, float (&r)[8]) {
        float4 a = *reinterpret_cast<const float4*>(p);
        float4 b = *reinterpret_cast<const float4*>(p + 4);
        r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w;
        r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
    }
};
template <> struct Vec8<double> {
    static __device__ __forceinline__ void load(const double* p, double (&r)[8]) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            double2 a = reinterpret_cast<const double2*>(p)[i];
            r[2 * i] = a.x; r[2 * i + 1] = a.y;
        }
    }
};

struct GemmGeom {
    int n, ne, no, my, nx;
    long long fs;
    int R;          // rows = nfields * my
    int kpad, ldw, lds;
};

enum { MODE_FWD = 0, MODE_INV = 1 };

template <int TR> struct GemmShape {
    static constexpr int NT = 2 * (TR / 8) * 16;   // threads per CTA
};

template <typename T, int TR>
__host__ __device__ constexpr size_t gemm_smem_elems(int kpad) {
    return size_t(2) * kpad * TR +
           (size_t(2) * DST_KC * DST_NC > size_t(TR) * DST_NC ? size_t(2) * DST_KC * DST_NC
                                                              : size_t(TR) * DST_NC);
}

// One CTA: TR interior rows x DST_NC output columns of BOTH halves.
// Threads [0, NT/2) multiply by W1 (the even-k half), [NT/2, NT) by W2.
template <typename T, int TR, int MODE, int EPI>
__global__ void __launch_bounds__(GemmShape<TR>::NT)
dst_gemm_kernel(GemmGeom g, const T* __restrict__ W1, const T* __restrict__ W2,
                const T* __restrict__ src, const T* __restrict__ sub, int sub_batches,
                T* __restrict__ spec, T* __restrict__ out, const T* __restrict__ add,
                int add_batches, const int8_t* __restrict__ mask)
{
    constexpr int NT = GemmShape<TR>::NT;
    constexpr int NC = DST_NC;
    constexpr int KC = DST_KC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* As = reinterpret_cast<T*>(smem_raw);
    T* Bs = As + size_t(g.kpad) * TR;
    T* Ws = Bs + size_t(g.kpad) * TR;     // W1 chunk | W2 chunk, later the exchange tile
    T* W1s = Ws;
    T* W2s = Ws + KC * NC;

    const int tid = threadIdx.x;
    const int row0 = blockIdx.y * TR;
    const int c0 = blockIdx.x * NC;
    const int n = g.n, ne = g.ne, no = g.no, my = g.my;

    // ---- prologue: operands, transposed to [k][row] -------------------------
    for (int idx = tid; idx < g.kpad * TR; idx += NT) {
        const int r = idx % TR;
        const int p = idx / TR;
        const int row = row0 + r;
        T a = T(0), b = T(0);
        if (row < g.R) {
            if (MODE == MODE_FWD) {
                if (p < ne) {
                    const int f = row / my;
                    const int j = row - f * my + 1;
                    const T* s = src + f * g.fs + (long long)j * g.nx + 1;
                    const T* sb = (sub != nullptr && f < sub_batches)
                                      ? sub + f * g.fs + (long long)j * g.nx + 1 : nullptr;
                    T x1 = s[p];
                    if (sb) x1 -= sb[p];
                    if (p < no) {
                        T x2 = s[n - 1 - p];
                        if (sb) x2 -= sb[n - 1 - p];
                        a = x1 + x2;
                        b = x1 - x2;
                    } else {
                        a = x1;   // middle point of an odd-length transform
                    }
                }
            } else {
                const T* s = spec + (long long)row * g.lds;
                if (p < ne) a = s[p];
                if (p < no) b = s[ne + p];
            }
        }
        As[p * TR + r] = a;
        Bs[p * TR + r] = b;
    }

    const int grp = tid / (NT / 2);
    const int lt = tid % (NT / 2);
    const int ty = lt / 16;
    const int tx = lt % 16;
    const T* Aop = grp == 0 ? As : Bs;
    const T* Wop = grp == 0 ? W1s : W2s;

    T acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = T(0);

    for (int k0 = 0; k0 < g.kpad; k0 += KC) {
        __syncthreads();
        for (int e = tid; e < KC * NC; e += NT) {
            const int kk = e / NC;
            const int cc = e - kk * NC;
            const size_t goff = size_t(k0 + kk) * g.ldw + c0 + cc;
            W1s[e] = W1[goff];
            W2s[e] = W2[goff];
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < KC; ++kk) {
            T a[8], w[8];
            Vec8<T>::load(Aop + (k0 + kk) * TR + ty * 8, a);
            Vec8<T>::load(Wop + kk * NC + tx * 8, w);
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fma(a[i], w[j], acc[i][j]);
        }
    }

    const int rb = row0 + ty * 8;
    const int cb = c0 + tx * 8;
    if (MODE == MODE_FWD) {
        const int lim = grp == 0 ? ne : no;
        const int coff = grp == 0 ? 0 : ne;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int row = rb + i;
            if (row >= g.R) continue;
            T* d = spec + (long long)row * g.lds + coff;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int t = cb + j;
                if (t < lim) d[t] = acc[i][j];
            }
        }
    } else {
        __syncthreads();
        T* X = Ws;   // [TR][NC] exchange tile
        if (grp == 1) {
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) X[(ty * 8 + i) * NC + tx * 8 + j] = acc[i][j];
        }
        __syncthreads();
        if (grp == 0) {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int row = rb + i;
                if (row >= g.R) continue;
                const int f = row / my;
                const int j = row - f * my + 1;
                const long long base = f * g.fs + (long long)j * g.nx + 1;
#pragma unroll
                for (int jj = 0; jj < 8; ++jj) {
                    const int p = cb + jj;
                    if (p >= ne) continue;
                    const T A = acc[i][jj];
                    const T B = (p < no) ? X[(ty * 8 + i) * NC + tx * 8 + jj] : T(0);
                    const int ps[2] = {p, n - 1 - p};
                    const T ys[2] = {A + B, A - B};
                    const int cnt = (p < no) ? 2 : 1;
                    for (int u = 0; u < cnt; ++u) {
                        const long long o = base + ps[u];
                        if (EPI == EPI_H) {
                            T y = ys[u];
                            if (add != nullptr && f < add_batches) y += add[o];
                            out[o] = y;
                        } else {
                            const int mi = j * g.nx + 1 + ps[u];
                            out[o] = (mask[mi] == 3) ? ys[u] + add[o] : T(0);
                        }
                    }
                }
            }
        }
    }
}

// Chunked Thomas algorithm. Both sweeps are first-order linear recurrences
// with the multiplier alpha_j = -a*m_j: forward d_j = m_j F_j + alpha_j
// d_{j-1}, backward x_j = d_j + alpha_j x_{j+1}. A row piece runs from a zero
// carry while accumulating the product of its alphas; the true values follow
// by adding carry * partial product. |alpha| < 1 (diagonal dominance), so
// the products only shrink.
// CW spectral columns per CTA; the warp's lanes are CW columns x (32/CW)
// row pieces, so a CTA holds nw*(32/CW) pieces of CH rows per column. Each
// thread keeps its piece (values and multipliers) in registers and runs both
// Thomas sweeps locally (the recurrences are affine, so a piece is summarised
// by its end value and the product of its multipliers). The pieces of a
// column are then combined by a scan of the affine maps (d, P) o (d', P') =
// (d + P d', P P'): a shuffle scan over the warp's 32/CW pieces, then the
// warp totals through shared memory; every piece applies the carry it
// receives. Eight columns per CTA: 1024 CTAs for 16 fields of 512^2, 128 for
// one 1024^2 field.
// LEAN caps the registers at 80 (16-row pieces in float32 otherwise take
// ~124): three 256-thread CTAs fit an SM instead of two (a schedule choice,
// picked by timing). 8-row pieces are capped at 64 registers, so two CTAs
// of up to 512 threads fit an SM.
template <typename T, int CW, int CH, bool LEAN = false>
__global__ void __maxnreg__(LEAN ? 80 : (CH <= 8 ? 64 : 128))
tridiag_chunked_kernel(T* __restrict__ spec, const T* __restrict__ trim, int my, int n, int lds, T a)
{
    constexpr int SUB = 32 / CW;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nw = blockDim.y;
    T* wD = reinterpret_cast<T*>(smem_raw);         // [nw][CW] warp totals: end value
    T* wP = wD + (size_t)nw * CW;                   // [nw][CW] warp totals: product
    const int f = blockIdx.y;
    const int lane = threadIdx.x, w = threadIdx.y;
    const int c = lane % CW;
    const int sp = lane / CW;                       // piece within the warp
    const int pc = w * SUB + sp;
    const int t = blockIdx.x * CW + c;
    const bool col_ok = t < n;
    T* S = spec + (long long)f * my * lds + t;
    const T* M = trim + t;
    const int j0 = pc * CH;
    const int cnt = col_ok ? max(0, min(CH, my - j0)) : 0;
    T x[CH], al[CH];
#pragma unroll
    for (int i = 0; i < CH; ++i) {
        const bool v = i < cnt;
        x[i] = v ? S[(long long)(j0 + i) * lds] : T(0);
        al[i] = v ? __ldg(M + (long long)(j0 + i) * lds) : T(0);
    }

    // forward sweep, piece-local: d_j = m_j F_j + (-a m_j) d_{j-1}
    T d = T(0), P = T(1);
#pragma unroll
    for (int i = 0; i < CH; ++i) {
        if (i < cnt) {
            const T m = al[i];
            al[i] = -a * m;
            d = m * x[i] + al[i] * d;
            x[i] = d;
            P *= al[i];
        }
    }
    {
        // inclusive scan over the pieces of the warp (lanes CW apart)
        T sd = d, sP = P;
#pragma unroll
        for (int o = 1; o < SUB; o <<= 1) {
            const T od = __shfl_up_sync(0xffffffffu, sd, o * CW);
            const T oP = __shfl_up_sync(0xffffffffu, sP, o * CW);
            if (sp >= o) {
                sd = sd + sP * od;
                sP = sP * oP;
            }
        }
        if (sp == SUB - 1) {
            wD[w * CW + c] = sd;
            wP[w * CW + c] = sP;
        }
        __syncthreads();
        // carry into this warp: the warps before it, in order
        T cw = T(0);
        for (int v = 0; v < w; ++v) cw = wD[v * CW + c] + wP[v * CW + c] * cw;
        // end value of the previous piece
        const T pd = __shfl_up_sync(0xffffffffu, sd, CW);
        const T pP = __shfl_up_sync(0xffffffffu, sP, CW);
        const T cin = sp == 0 ? cw : pd + pP * cw;
        if (pc > 0) {
            T pr = T(1);
#pragma unroll
            for (int i = 0; i < CH; ++i) {
                if (i < cnt) {
                    pr *= al[i];
                    x[i] += pr * cin;
                }
            }
        }
    }
    __syncthreads();   // the warp totals are read before they are rewritten

    // backward sweep, piece-local from the piece end: x_j = d_j + (-a m_j) x_{j+1}
    T xr = T(0);
    P = T(1);
#pragma unroll
    for (int i = CH - 1; i >= 0; --i) {
        if (i < cnt) {
            xr = x[i] + al[i] * xr;
            x[i] = xr;
            P *= al[i];
        }
    }
    {
        // inclusive scan from the last piece of the warp down to the first
        T sd = xr, sP = P;
#pragma unroll
        for (int o = 1; o < SUB; o <<= 1) {
            const T od = __shfl_down_sync(0xffffffffu, sd, o * CW);
            const T oP = __shfl_down_sync(0xffffffffu, sP, o * CW);
            if (sp + o < SUB) {
                sd = sd + sP * od;
                sP = sP * oP;
            }
        }
        if (sp == 0) {
            wD[w * CW + c] = sd;
            wP[w * CW + c] = sP;
        }
        __syncthreads();
        T cw = T(0);
        for (int v = nw - 1; v > w; --v) cw = wD[v * CW + c] + wP[v * CW + c] * cw;
        const T nd = __shfl_down_sync(0xffffffffu, sd, CW);
        const T nP = __shfl_down_sync(0xffffffffu, sP, CW);
        const T cin = sp == SUB - 1 ? cw : nd + nP * cw;
        if (pc < nw * SUB - 1) {
            T pr = T(1);
#pragma unroll
            for (int i = CH - 1; i >= 0; --i) {
                if (i < cnt) {
                    pr *= al[i];
                    x[i] += pr * cin;
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < CH; ++i)
        if (i < cnt) S[(long long)(j0 + i) * lds] = x[i];
}

// Same recurrences directly on the spectral buffer, for column blocks too tall
// for shared memory (float64 at the largest grids).
template <typename T>
__global__ void __launch_bounds__(32)
tridiag_global_kernel(T* __restrict__ spec, const T* __restrict__ trim, int my, int n, int lds, T a)
{
    const int f = blockIdx.y;
    const int t = blockIdx.x * 32 + threadIdx.x;
    if (t >= n) return;
    T* S = spec + (long long)f * my * lds + t;
    const T* M = trim + t;
    T d = S[0] * __ldg(M);
    S[0] = d;
    for (int j = 1; j < my; ++j) {
        d = (S[(long long)j * lds] - a * d) * __ldg(M + (long long)j * lds);
        S[(long long)j * lds] = d;
    }
    T x = d;
    for (int j = my - 2; j >= 0; --j) {
        x = S[(long long)j * lds] - a * __ldg(M + (long long)j * lds) * x;
        S[(long long)j * lds] = x;
    }
}

// ---------------------------------------------------------------------------
// Float64 DST-I by FFT
//
// The FP64 rate of this part is a small fraction of its FP32 / tensor rate, so
// the O(n^2) dense transform above costs ~3 ms a field at n ~ 1000 even at
// the FP64 peak; an FFT does the same transform in O(n log n). Two real rows
// a, b are packed as z = a + i b into their odd extension of length
// L = 2(n+1): z_0 = z_{n+1} = 0, z_{p+1} = a_p + i b_p, z_{L-1-p} = -z_{p+1}.
// The DFT of a real odd sequence is purely imaginary,
//   A_m = -2i sum_p a_p sin(pi (p+1) m / (n+1)),
// so Z = A + i B gives both rows at once: DST_a(m) = -Im Z_m / 2 and
// DST_b(m) = Re Z_m / 2, times sqrt(2/(n+1)) for the orthonormal form. The
// FFT is a Stockham autosort (each stage reads v_r = x[j + r L/R], applies the
// twiddles e^{-2 pi i k r / (Ns R)} with k = j mod Ns, takes the length-R DFT
// and writes y[(j/Ns) Ns R + k + r Ns]; the output is in natural order) with
// radix 4, 2, 3 and 5 stages, ping-ponging between two shared-memory buffers.
// The orthonormal DST-I is its own inverse, so the inverse pass is the same
// transform from the parity-split spectral rows to the field.
// ---------------------------------------------------------------------------
struct FftGeom {
    int L, N, n, ne, my, nx, R, lds, nst, pp;
    long long fs;
    double scale;        // sqrt(2/N) / 2
    int rad[24];
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
// -i * a
__device__ __forceinline__ double2 cmi(double2 a) { return make_double2(a.y, -a.x); }

template <int R> struct Dft;
template <> struct Dft<2> {
    static __device__ __forceinline__ void run(double2 (&v)[2])
    {
        const double2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};
template <> struct Dft<4> {
    static __device__ __forceinline__ void run(double2 (&v)[4])
    {
        const double2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
        const double2 c = cadd(v[1], v[3]), d = cmi(csub(v[1], v[3]));
        v[0] = cadd(a, c);
        v[2] = csub(a, c);
        v[1] = cadd(b, d);
        v[3] = csub(b, d);
    }
};
template <> struct Dft<3> {
    // y1,2 = v0 - (v1+v2)/2 -/+ i (sqrt(3)/2) (v1 - v2)
    static __device__ __forceinline__ void run(double2 (&v)[3])
    {
        constexpr double S3 = 0.86602540378443864676;   // sqrt(3)/2
        const double2 t = cadd(v[1], v[2]);
        const double2 m = make_double2(v[0].x - 0.5 * t.x, v[0].y - 0.5 * t.y);
        const double2 d = cmi(csub(v[1], v[2]));
        const double2 e = make_double2(S3 * d.x, S3 * d.y);
        v[0] = cadd(v[0], t);
        v[1] = cadd(m, e);
        v[2] = csub(m, e);
    }
};
template <> struct Dft<5> {
    // pairs r, 5-r: t1 = v1+v4, t2 = v2+v3, d1 = v1-v4, d2 = v2-v3;
    // y1,4 = v0 + c1 t1 + c2 t2 -/+ i (s1 d1 + s2 d2)
    // y2,3 = v0 + c2 t1 + c1 t2 -/+ i (s2 d1 - s1 d2)
    static __device__ __forceinline__ void run(double2 (&v)[5])
    {
        constexpr double C1 = 0.30901699437494742410;    // cos(2 pi / 5)
        constexpr double C2 = -0.80901699437494742410;   // cos(4 pi / 5)
        constexpr double S1 = 0.95105651629515357212;    // sin(2 pi / 5)
        constexpr double S2 = 0.58778525229247312917;    // sin(4 pi / 5)
        const double2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
        const double2 d1 = cmi(csub(v[1], v[4])), d2 = cmi(csub(v[2], v[3]));
        const double2 a1 = make_double2(v[0].x + C1 * t1.x + C2 * t2.x, v[0].y + C1 * t1.y + C2 * t2.y);
        const double2 a2 = make_double2(v[0].x + C2 * t1.x + C1 * t2.x, v[0].y + C2 * t1.y + C1 * t2.y);
        const double2 b1 = make_double2(S1 * d1.x + S2 * d2.x, S1 * d1.y + S2 * d2.y);
        const double2 b2 = make_double2(S2 * d1.x - S1 * d2.x, S2 * d1.y - S1 * d2.y);
        v[0] = cadd(v[0], cadd(t1, t2));
        v[1] = cadd(a1, b1);
        v[4] = csub(a1, b1);
        v[2] = cadd(a2, b2);
        v[3] = csub(a2, b2);
    }
};

template <int R>
__device__ __forceinline__ void fft_stage(const double2* __restrict__ in, double2* __restrict__ out,
                                          const double2* __restrict__ tw, int L, int Ns, int pp)
{
    const int T = L / R;
    const int tstep = L / (Ns * R);
    for (int idx = threadIdx.x; idx < pp * T; idx += blockDim.x) {
        const int q = idx / T;
        const int j = idx - q * T;
        const int k = j % Ns;
        const double2* I = in + (long long)q * L;
        double2* O = out + (long long)q * L;
        double2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = I[j + r * T];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(tw + (long long)k * r * tstep));
        }
        Dft<R>::run(v);
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) O[base + r * Ns] = v[r];
    }
}

// One CTA: g.pp pairs of rows (2 g.pp consecutive rows of the R row list).
template <int MODE, int EPI>
__global__ void __launch_bounds__(256)
dst_fft_kernel(FftGeom g, const double2* __restrict__ tw, const double* __restrict__ src,
               const double* __restrict__ sub, int sub_batches, double* __restrict__ spec,
               double* __restrict__ out, const double* __restrict__ add, int add_batches,
               const int8_t* __restrict__ mask)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2* b0 = reinterpret_cast<double2*>(smem_raw);
    double2* b1 = b0 + (size_t)g.pp * g.L;
    const int L = g.L, N = g.N, n = g.n;
    const int row_base = 2 * blockIdx.x * g.pp;

    auto load = [&](int row, int p) -> double {
        if (row >= g.R) return 0.0;
        if (MODE == MODE_FWD) {
            const int f = row / g.my;
            const int j = row - f * g.my + 1;
            const long long o = f * g.fs + (long long)j * g.nx + 1 + p;
            double x = src[o];
            if (sub != nullptr && f < sub_batches) x -= sub[o];
            return x;
        } else {
            const int t = (p & 1) ? g.ne + (p >> 1) : (p >> 1);
            return spec[(long long)row * g.lds + t];
        }
    };
    for (int idx = threadIdx.x; idx < g.pp * n; idx += blockDim.x) {
        const int q = idx / n;
        const int p = idx - q * n;
        const int ra = row_base + 2 * q;
        const double xa = load(ra, p), xb = load(ra + 1, p);
        double2* Z = b0 + (size_t)q * L;
        Z[p + 1] = make_double2(xa, xb);
        Z[L - 1 - p] = make_double2(-xa, -xb);
    }
    for (int q = threadIdx.x; q < g.pp; q += blockDim.x) {
        b0[(size_t)q * L] = make_double2(0.0, 0.0);
        b0[(size_t)q * L + N] = make_double2(0.0, 0.0);
    }
    __syncthreads();
    int Ns = 1;
    for (int s = 0; s < g.nst; ++s) {
        const int R = g.rad[s];
        switch (R) {
            case 4: fft_stage<4>(b0, b1, tw, L, Ns, g.pp); break;
            case 2: fft_stage<2>(b0, b1, tw, L, Ns, g.pp); break;
            case 3: fft_stage<3>(b0, b1, tw, L, Ns, g.pp); break;
            default: fft_stage<5>(b0, b1, tw, L, Ns, g.pp); break;
        }
        __syncthreads();
        double2* t = b0; b0 = b1; b1 = t;
        Ns *= R;
    }
    for (int idx = threadIdx.x; idx < g.pp * n; idx += blockDim.x) {
        const int q = idx / n;
        const int k = idx - q * n;
        const double2 Zm = b0[(size_t)q * L + k + 1];
        const double ys[2] = {-Zm.y * g.scale, Zm.x * g.scale};
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int row = row_base + 2 * q + u;
            if (row >= g.R) continue;
            if (MODE == MODE_FWD) {
                const int t = (k & 1) ? g.ne + (k >> 1) : (k >> 1);
                spec[(long long)row * g.lds + t] = ys[u];
            } else {
                const int f = row / g.my;
                const int j = row - f * g.my + 1;
                const long long o = f * g.fs + (long long)j * g.nx + 1 + k;
                if (EPI == EPI_H) {
                    double y = ys[u];
                    if (add != nullptr && f < add_batches) y += add[o];
                    out[o] = y;
                } else {
                    const int mi = j * g.nx + 1 + k;
                    out[o] = (mask[mi] == 3) ? ys[u] + add[o] : 0.0;
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
size_t spec_bytes(const vd_qg1l_plan* p, int nf)
{
    return size_t(nf) * p->dst.my * p->dst.lds * elem_size(p->d.dtype);
}

template <typename T>
static int upload(const std::vector<double>& h, void** d)
{
    std::vector<T> tmp(h.begin(), h.end());
    VD_CUDA_TRY(cudaMalloc(d, tmp.size() * sizeof(T)));
    VD_CUDA_TRY(cudaMemcpy(*d, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice));
    return VD_OK;
}

// FFT radices for L = 2(n+1) (radix 4 first, then 2, 3, 5); false when L has
// another prime factor or its buffers do not fit shared memory.
static bool fft_factor(int L, std::vector<int>& rad)
{
    rad.clear();
    if (L < 4 || size_t(2) * L * sizeof(double2) > 200 * 1024) return false;
    int m = L;
    while (m % 4 == 0) { rad.push_back(4); m /= 4; }
    while (m % 2 == 0) { rad.push_back(2); m /= 2; }
    while (m % 3 == 0) { rad.push_back(3); m /= 3; }
    while (m % 5 == 0) { rad.push_back(5); m /= 5; }
    return m == 1 && rad.size() <= 24;
}

static int build_fft_tables(DSTTables& t)
{
    const int L = 2 * (t.n + 1);
    std::vector<int> rad;
    if (!fft_factor(L, rad)) return VD_OK;
    std::vector<double> tw(size_t(2) * L);
    for (int m = 0; m < L; ++m) {
        // e^{-2 pi i m / L} in float64 on the host
        const double a = 2.0 * M_PI * double(m) / double(L);
        tw[2 * m] = std::cos(a);
        tw[2 * m + 1] = -std::sin(a);
    }
    int rc;
    if ((rc = upload<double>(tw, &t.fft_tw))) return rc;
    t.fft_L = L;
    t.fft_nst = (int)rad.size();
    for (size_t i = 0; i < rad.size(); ++i) t.fft_rad[i] = rad[i];
    return VD_OK;
}

int build_dst_tables(vd_qg1l_plan* p)
{
    DSTTables& t = p->dst;
    const int n = p->d.nx - 2;
    const int my = p->d.ny - 2;
    t.n = n;
    t.my = my;
    t.no = n / 2;
    t.ne = n - t.no;
    t.ncol_tiles = (t.ne + DST_NC - 1) / DST_NC;
    t.kpad = ((t.ne + DST_KC - 1) / DST_KC) * DST_KC;
    t.ldw = t.ncol_tiles * DST_NC;
    t.lds = ((n + 3) / 4) * 4;

    const double scale = std::sqrt(2.0 / (n + 1));
    const long long period = 2LL * (n + 1);   // sin(pi*m/(n+1)) has period 2(n+1) in m
    auto s = [&](long long m) {
        m %= period;
        return scale * std::sin(M_PI * double(m) / double(n + 1));
    };
    std::vector<double> wodd(size_t(t.kpad) * t.ldw, 0.0), woddT(wodd.size(), 0.0),
        weven(wodd.size(), 0.0);
    for (int a = 0; a < t.ne; ++a)
        for (int b = 0; b < t.ne; ++b) {
            const double v = s((long long)(a + 1) * (2 * b + 1));
            wodd[size_t(a) * t.ldw + b] = v;
            woddT[size_t(b) * t.ldw + a] = v;
        }
    for (int a = 0; a < t.no; ++a)
        for (int b = 0; b < t.no; ++b)
            weven[size_t(a) * t.ldw + b] = s((long long)(a + 1) * (2 * b + 2));

    // Thomas multipliers per spectral column (parity-split order)
    const double gf = p->d.g / p->d.f;
    const double gfc2 = p->d.g * p->d.f / (p->d.c * p->d.c);
    const double dx = p->d.dx, dy = p->d.dy;
    const double a = gf / (dy * dy);
    t.tri_a = a;
    std::vector<double> trim(size_t(my) * t.lds, 0.0);
    for (int col = 0; col < n; ++col) {
        const int k = col < t.ne ? 2 * col : 2 * (col - t.ne) + 1;   // 0-based wavenumber
        const double mu = 2.0 * (std::cos(M_PI / (p->d.nx - 1) * (k + 1)) - 1.0) / (dx * dx);
        const double bk = gf * (-2.0 / (dy * dy) + mu) - gfc2;
        double c_prev = 0.0;
        for (int j = 0; j < my; ++j) {
            const double m = 1.0 / (bk - a * c_prev);
            trim[size_t(j) * t.lds + col] = m;
            c_prev = a * m;
        }
    }
    int rc;
    if (p->d.dtype == VD_F64 && (rc = build_fft_tables(t))) return rc;
    if (p->d.dtype == VD_F32) {
        if ((rc = upload<float>(wodd, &t.Wodd))) return rc;
        if ((rc = upload<float>(woddT, &t.WoddT))) return rc;
        if ((rc = upload<float>(weven, &t.Weven))) return rc;
        if ((rc = upload<float>(trim, &t.trim))) return rc;
    } else {
        if ((rc = upload<double>(wodd, &t.Wodd))) return rc;
        if ((rc = upload<double>(woddT, &t.WoddT))) return rc;
        if ((rc = upload<double>(weven, &t.Weven))) return rc;
        if ((rc = upload<double>(trim, &t.trim))) return rc;
    }
    return VD_OK;
}

void free_dst_tables(vd_qg1l_plan* p)
{
    cudaFree(p->dst.Wodd);
    cudaFree(p->dst.WoddT);
    cudaFree(p->dst.Weven);
    cudaFree(p->dst.trim);
    cudaFree(p->dst.fft_tw);
}

template <typename T, int TR>
static cudaError_t set_smem_attrs()
{
    const int maxb = 227 * 1024;
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(dst_gemm_kernel<T, TR, MODE_FWD, EPI_H>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, maxb))) return e;
    if ((e = cudaFuncSetAttribute(dst_gemm_kernel<T, TR, MODE_INV, EPI_H>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, maxb))) return e;
    return cudaFuncSetAttribute(dst_gemm_kernel<T, TR, MODE_INV, EPI_ADJQ>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, maxb);
}

// The y-direction tridiagonal solves of nf fields: 8 columns per CTA,
// pieces of 16 rows (32 for fields of 1025-2048 rows; 8, in up to 32 warps,
// as a schedule choice for fields of up to 1024 rows) in at most 16 warps;
// taller fields fall back to one sequential thread per column. (Measured on
// GB300 against 32- and 16-column groups, shared-memory staging and a
// warp-shuffle chain of the pieces: this form is the fastest or tied at both
// 16 x 510^2 and 1 x 1022^2.)
template <typename T>
static int launch_tridiag(const vd_qg1l_plan* p, int nf, T* spec, cudaStream_t st)
{
    const DSTTables& t = p->dst;
    const T a = (T)t.tri_a;
    constexpr int CW = 8, SUB = 32 / CW;
    const dim3 grid((t.n + CW - 1) / CW, nf);
    const int nw8 = ((t.my + 7) / 8 + SUB - 1) / SUB;
    const int nw16 = ((t.my + 15) / 16 + SUB - 1) / SUB;
    const int nw32 = ((t.my + 31) / 32 + SUB - 1) / SUB;
    const bool want32 = p->sched.tridiag_rows == 32 && nw32 <= 16;
    const bool want8 = p->sched.tridiag_rows == 8 && nw8 <= 32;
    if (want8) {
        tridiag_chunked_kernel<T, CW, 8><<<grid, dim3(32, nw8), 2 * nw8 * CW * sizeof(T), st>>>(
            spec, (const T*)t.trim, t.my, t.n, t.lds, a);
    } else if (nw16 <= 16 && !want32 && p->sched.tridiag_lean == 1 && sizeof(T) == 4) {
        tridiag_chunked_kernel<T, CW, 16, true><<<grid, dim3(32, nw16), 2 * nw16 * CW * sizeof(T), st>>>(
            spec, (const T*)t.trim, t.my, t.n, t.lds, a);
    } else if (nw16 <= 16 && !want32) {
        tridiag_chunked_kernel<T, CW, 16><<<grid, dim3(32, nw16), 2 * nw16 * CW * sizeof(T), st>>>(
            spec, (const T*)t.trim, t.my, t.n, t.lds, a);
    } else if (nw32 <= 16) {
        tridiag_chunked_kernel<T, CW, 32><<<grid, dim3(32, nw32), 2 * nw32 * CW * sizeof(T), st>>>(
            spec, (const T*)t.trim, t.my, t.n, t.lds, a);
    } else {
        tridiag_global_kernel<T><<<dim3((t.n + 31) / 32, nf), 32, 0, st>>>(spec, (const T*)t.trim, t.my, t.n,
                                                                           t.lds, a);
    }
    VD_LAUNCH_CHECK();
    return VD_OK;
}

static PerDeviceOnce g_attr_once;

static cudaError_t configure_kernels()
{
    return g_attr_once.run([]() -> cudaError_t {
        cudaError_t e = cudaSuccess;
        if (!e) e = set_smem_attrs<float, 16>();
        if (!e) e = set_smem_attrs<float, 32>();
        if (!e) e = set_smem_attrs<float, 64>();
        if (!e) e = set_smem_attrs<double, 16>();
        if (!e) e = set_smem_attrs<double, 32>();
        const int maxb = 227 * 1024;
        if (!e) e = cudaFuncSetAttribute(dst_fft_kernel<MODE_FWD, EPI_H>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, maxb);
        if (!e) e = cudaFuncSetAttribute(dst_fft_kernel<MODE_INV, EPI_H>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, maxb);
        if (!e) e = cudaFuncSetAttribute(dst_fft_kernel<MODE_INV, EPI_ADJQ>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, maxb);
        return e;
    });
}

template <typename T, int TR>
static int launch_pair(const vd_qg1l_plan* p, const GemmGeom& g, const SolveArgs& a,
                       T* spec, cudaStream_t st, bool fwd)
{
    const DSTTables& t = p->dst;
    constexpr int NT = GemmShape<TR>::NT;
    const size_t smem = gemm_smem_elems<T, TR>(g.kpad) * sizeof(T);
    dim3 grid(t.ncol_tiles, (g.R + TR - 1) / TR);
    if (fwd) {
        dst_gemm_kernel<T, TR, MODE_FWD, EPI_H><<<grid, NT, smem, st>>>(
            g, (const T*)t.Wodd, (const T*)t.Weven, (const T*)a.src, (const T*)a.sub,
            a.sub_batches, spec, nullptr, nullptr, 0, nullptr);
    } else if (a.epi == EPI_H) {
        dst_gemm_kernel<T, TR, MODE_INV, EPI_H><<<grid, NT, smem, st>>>(
            g, (const T*)t.WoddT, (const T*)t.Weven, nullptr, nullptr, 0, spec, (T*)a.out,
            (const T*)a.add, a.add_batches, p->d_mask);
    } else {
        dst_gemm_kernel<T, TR, MODE_INV, EPI_ADJQ><<<grid, NT, smem, st>>>(
            g, (const T*)t.WoddT, (const T*)t.Weven, nullptr, nullptr, 0, spec, (T*)a.out,
            (const T*)a.add, a.add_batches, p->d_mask);
    }
    VD_LAUNCH_CHECK();
    return VD_OK;
}

// The float64 FFT pass over g.R rows: pairs of rows per CTA chosen for about
// two CTAs per SM-wave slot and at most ~100 KB of shared memory per CTA.
static int launch_fft(const vd_qg1l_plan* p, const GemmGeom& g, const SolveArgs& a, double* spec,
                      cudaStream_t st, bool fwd)
{
    const DSTTables& t = p->dst;
    FftGeom fg;
    fg.L = t.fft_L; fg.N = t.n + 1; fg.n = t.n; fg.ne = t.ne; fg.my = t.my; fg.nx = g.nx;
    fg.R = g.R; fg.lds = t.lds; fg.nst = t.fft_nst; fg.fs = g.fs;
    fg.scale = 0.5 * std::sqrt(2.0 / double(t.n + 1));
    for (int i = 0; i < 24; ++i) fg.rad[i] = t.fft_rad[i];
    const int pairs = (g.R + 1) / 2;
    const size_t per_pair = size_t(2) * t.fft_L * sizeof(double2);
    int pp = std::max(1, std::min<int>(8, int((100 * 1024) / per_pair)));
    pp = std::max(1, std::min(pp, pairs / (2 * 152)));
    fg.pp = pp;
    const size_t smem = per_pair * pp;
    const dim3 grid((pairs + pp - 1) / pp);
    const double2* tw = (const double2*)t.fft_tw;
    if (fwd) {
        dst_fft_kernel<MODE_FWD, EPI_H><<<grid, 256, smem, st>>>(fg, tw, (const double*)a.src,
                                                                 (const double*)a.sub, a.sub_batches, spec,
                                                                 nullptr, nullptr, 0, nullptr);
    } else if (a.epi == EPI_H) {
        dst_fft_kernel<MODE_INV, EPI_H><<<grid, 256, smem, st>>>(fg, tw, nullptr, nullptr, 0, spec, (double*)a.out,
                                                                 (const double*)a.add, a.add_batches, p->d_mask);
    } else {
        dst_fft_kernel<MODE_INV, EPI_ADJQ><<<grid, 256, smem, st>>>(fg, tw, nullptr, nullptr, 0, spec,
                                                                    (double*)a.out, (const double*)a.add,
                                                                    a.add_batches, p->d_mask);
    }
    VD_LAUNCH_CHECK();
    return VD_OK;
}

// Rows per CTA: the largest tile that still gives about two waves of CTAs on
// the 152 SMs and fits shared memory.
template <typename T>
static int pick_tr(const vd_qg1l_plan* p, int R)
{
    const DSTTables& t = p->dst;
    if (p->sched.fma_rows == 16 || p->sched.fma_rows == 32 || (p->sched.fma_rows == 64 && sizeof(T) == 4))
        return p->sched.fma_rows;
    const int cand[3] = {64, 32, 16};
    for (int c : cand) {
        if (sizeof(T) == 8 && c == 64) continue;
        const size_t smem = (size_t(2) * t.kpad * c + size_t(std::max(2 * DST_KC * DST_NC, c * DST_NC))) * sizeof(T);
        if (smem > 200 * 1024) continue;
        const long long ctas = (long long)t.ncol_tiles * ((R + c - 1) / c);
        if (ctas >= 2 * 152) return c;
    }
    return 16;
}

template <typename T>
int helmholtz_solve(const vd_qg1l_plan* p, int nf, const SolveArgs& a, T* spec, cudaStream_t st)
{
    if (configure_kernels() != cudaSuccess) return VD_ERR_CUDA;
    const DSTTables& t = p->dst;
    GemmGeom g;
    g.n = t.n; g.ne = t.ne; g.no = t.no; g.my = t.my; g.nx = p->d.nx;
    g.fs = (long long)p->d.ny * p->d.nx;
    g.R = nf * t.my;
    g.kpad = t.kpad; g.ldw = t.ldw; g.lds = t.lds;
    const int tr = pick_tr<T>(p, g.R);
    int rc;
    auto run = [&](bool fwd) -> int {
        if constexpr (sizeof(T) == 4) {
            if (use_tc(p, nf)) return dst_pass_tc(p, nf, a, (float*)spec, fwd, st);
            if (tr == 64) return launch_pair<T, 64>(p, g, a, spec, st, fwd);
        } else {
            if (p->dst.fft_L) return launch_fft(p, g, a, (double*)spec, st, fwd);
        }
        if (tr == 32) return launch_pair<T, 32>(p, g, a, spec, st, fwd);
        return launch_pair<T, 16>(p, g, a, spec, st, fwd);
    };
    if ((rc = run(true))) return rc;
    if ((rc = launch_tridiag<T>(p, nf, spec, st))) return rc;
    return run(false);
}

template int helmholtz_solve<float>(const vd_qg1l_plan*, int, const SolveArgs&, float*, cudaStream_t);
template int helmholtz_solve<double>(const vd_qg1l_plan*, int, const SolveArgs&, double*, cudaStream_t);

// The x-direction DST-I pass alone (forward: field interior -> spectral rows;
// inverse: spectral rows -> field interior).
template <typename T>
int dst_x_only(const vd_qg1l_plan* p, int nf, const T* field, T* spec, int inverse, T* out, cudaStream_t st)
{
    if (configure_kernels() != cudaSuccess) return VD_ERR_CUDA;
    const DSTTables& t = p->dst;
    GemmGeom g;
    g.n = t.n; g.ne = t.ne; g.no = t.no; g.my = t.my; g.nx = p->d.nx;
    g.fs = (long long)p->d.ny * p->d.nx;
    g.R = nf * t.my;
    g.kpad = t.kpad; g.ldw = t.ldw; g.lds = t.lds;
    SolveArgs a;
    a.src = field; a.sub = nullptr; a.sub_batches = 0;
    a.out = out; a.add = nullptr; a.add_batches = 0; a.epi = EPI_H;
    if (inverse == 2) {            // adjoint epilogue: out = M3 * (x + field)
        a.src = nullptr;
        a.add = field; a.add_batches = nf; a.epi = EPI_ADJQ;
    }
    const int tr = pick_tr<T>(p, g.R);
    if constexpr (sizeof(T) == 4) {
        if (use_tc(p, nf)) return dst_pass_tc(p, nf, a, (float*)spec, !inverse, st);
        if (tr == 64) return launch_pair<T, 64>(p, g, a, spec, st, !inverse);
    } else {
        if (p->dst.fft_L) return launch_fft(p, g, a, (double*)spec, st, !inverse);
    }
    if (tr == 32) return launch_pair<T, 32>(p, g, a, spec, st, !inverse);
    return launch_pair<T, 16>(p, g, a, spec, st, !inverse);
}

// The y-direction tridiagonal solve alone, in place on spectral rows.
template <typename T>
int tridiag_only(const vd_qg1l_plan* p, int nf, T* spec, cudaStream_t st)
{
    if (configure_kernels() != cudaSuccess) return VD_ERR_CUDA;
    return launch_tridiag<T>(p, nf, spec, st);
}

template int tridiag_only<float>(const vd_qg1l_plan*, int, float*, cudaStream_t);
template int tridiag_only<double>(const vd_qg1l_plan*, int, double*, cudaStream_t);
template int dst_x_only<float>(const vd_qg1l_plan*, int, const float*, float*, int, float*, cudaStream_t);
template int dst_x_only<double>(const vd_qg1l_plan*, int, const double*, double*, int, double*, cudaStream_t);

}  // namespace vd
