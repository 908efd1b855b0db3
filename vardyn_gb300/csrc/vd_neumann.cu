// Spectral Helmholtz solve with Neumann boundaries on a rectangular domain
// (mapping/models/model_qgsw/helmholtz.py: compute_laplace_dctII 22-30,
// dctII / idctII 33-58, solve_helmholtz_dctII 81-87 and
// HelmholtzNeumannSolver 187-303 on an all-ocean mask, where the solve is
// G alone): w = idct2(dct2(rhs) / helm), both transforms the unnormalised
// DCT-II pair along each axis of [nf][nx][ny] fields.
//
// A length-N DCT-II goes through one N-point complex FFT (the reordering
// v_m = x_2m, v_{N-1-m} = x_2m+1 of helmholtz.py:33-40): y_k = Re(E_k V_k),
// E_k = 2 e^{-i pi k / (2N)}. Its inverse (helmholtz.py:43-58) builds
// W_k = (y_k - i y_{N-k}) e^{i pi k / (2N)} / 2 (y_N = 0) and takes the real
// inverse FFT back through the same reordering. Two real sequences a, b share
// one complex transform:
//   forward  z = a + i b: A_k = (Z_k + conj Z_{N-k}) / 2,
//                         B_k = -i (Z_k - conj Z_{N-k}) / 2;
//   inverse  W = W_a + i W_b: the inverse FFT is a + i b (both real), taken
//            as conj(FFT(conj W)) / N.
// Three passes, each one CTA per group of sequence pairs, all in shared
// memory:
//   k_dct_rows_fwd  DCT-II along y of row pairs;
//   k_dct_cols      per pair of columns: DCT-II along x, division by helm,
//                   inverse along x (the whole column stays on chip);
//   k_dct_rows_inv  inverse along y of row pairs.
// Each pass may run in place (a CTA reads all its sequences before writing).
// The FFT is a Stockham autosort with radix 4, 2, 3, 5 stages and a direct
// stage for any other prime factor, ping-ponging between two buffers; the
// twiddles e^{-2 pi i m / N} and E_k are host-computed float64 tables rounded
// to the arithmetic type. Any N >= 2 works (the reference's reordering needs
// even N; the oracle, scipy's DCT, any N).
#include "vd_internal.cuh"

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

namespace vd {
namespace nm {

constexpr int MAX_STAGES = 32;

template <typename T>
struct alignas(2 * sizeof(T)) cx {
    T x, y;
};
template <typename T> __device__ __forceinline__ cx<T> mk(T a, T b) { cx<T> r; r.x = a; r.y = b; return r; }
template <typename T> __device__ __forceinline__ cx<T> add(cx<T> a, cx<T> b) { return mk(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ cx<T> sub(cx<T> a, cx<T> b) { return mk(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ cx<T> mul(cx<T> a, cx<T> b)
{
    return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T> __device__ __forceinline__ cx<T> cj(cx<T> a) { return mk(a.x, -a.y); }
// -i * a
template <typename T> __device__ __forceinline__ cx<T> mi(cx<T> a) { return mk(a.y, -a.x); }
template <typename T> __device__ __forceinline__ cx<T> scl(T s, cx<T> a) { return mk(s * a.x, s * a.y); }

// One transform direction: length, twiddle tables, radix plan.
struct Dir {
    int N, nst;
    const void* tw;   // cx<T>[N]: e^{-2 pi i m / N}
    const void* E;    // cx<T>[N]: 2 e^{-i pi k / (2N)}
    int rad[MAX_STAGES];
};

template <typename T, int R> struct Dft;
template <typename T> struct Dft<T, 2> {
    static __device__ __forceinline__ void run(cx<T> (&v)[2])
    {
        const cx<T> a = v[0], b = v[1];
        v[0] = add(a, b);
        v[1] = sub(a, b);
    }
};
template <typename T> struct Dft<T, 4> {
    static __device__ __forceinline__ void run(cx<T> (&v)[4])
    {
        const cx<T> a = add(v[0], v[2]), b = sub(v[0], v[2]);
        const cx<T> c = add(v[1], v[3]), d = mi(sub(v[1], v[3]));
        v[0] = add(a, c);
        v[2] = sub(a, c);
        v[1] = add(b, d);
        v[3] = sub(b, d);
    }
};
template <typename T> struct Dft<T, 3> {
    // y1,2 = v0 - (v1+v2)/2 -/+ i (sqrt(3)/2) (v1 - v2)
    static __device__ __forceinline__ void run(cx<T> (&v)[3])
    {
        const T S3 = T(0.86602540378443864676);
        const cx<T> t = add(v[1], v[2]);
        const cx<T> m = mk(v[0].x - T(0.5) * t.x, v[0].y - T(0.5) * t.y);
        const cx<T> e = scl(S3, mi(sub(v[1], v[2])));
        v[0] = add(v[0], t);
        v[1] = add(m, e);
        v[2] = sub(m, e);
    }
};
template <typename T> struct Dft<T, 5> {
    // y1,4 = v0 + c1 t1 + c2 t2 -/+ i (s1 d1 + s2 d2),
    // y2,3 = v0 + c2 t1 + c1 t2 -/+ i (s2 d1 - s1 d2),
    // t1 = v1+v4, t2 = v2+v3, d1 = v1-v4, d2 = v2-v3
    static __device__ __forceinline__ void run(cx<T> (&v)[5])
    {
        const T C1 = T(0.30901699437494742410), C2 = T(-0.80901699437494742410);
        const T S1 = T(0.95105651629515357212), S2 = T(0.58778525229247312917);
        const cx<T> t1 = add(v[1], v[4]), t2 = add(v[2], v[3]);
        const cx<T> d1 = mi(sub(v[1], v[4])), d2 = mi(sub(v[2], v[3]));
        const cx<T> a1 = mk(v[0].x + C1 * t1.x + C2 * t2.x, v[0].y + C1 * t1.y + C2 * t2.y);
        const cx<T> a2 = mk(v[0].x + C2 * t1.x + C1 * t2.x, v[0].y + C2 * t1.y + C1 * t2.y);
        const cx<T> b1 = mk(S1 * d1.x + S2 * d2.x, S1 * d1.y + S2 * d2.y);
        const cx<T> b2 = mk(S2 * d1.x - S1 * d2.x, S2 * d1.y - S1 * d2.y);
        v[0] = add(v[0], add(t1, t2));
        v[1] = add(a1, b1);
        v[4] = sub(a1, b1);
        v[2] = add(a2, b2);
        v[3] = sub(a2, b2);
    }
};

// Stockham stage over pp transforms of length N: butterfly j in [0, N/R)
// reads v_r = in[j + r N/R], applies e^{-2 pi i k r / (Ns R)} (k = j mod Ns),
// takes the length-R DFT and writes out[(j/Ns) Ns R + k + r Ns].
template <typename T, int R>
__device__ __forceinline__ void stage(const cx<T>* __restrict__ in, cx<T>* __restrict__ out,
                                      const cx<T>* __restrict__ tw, int N, int Ns, int pp)
{
    const int Tn = N / R;
    const int tstep = N / (Ns * R);
    for (int idx = threadIdx.x; idx < pp * Tn; idx += blockDim.x) {
        const int q = idx / Tn;
        const int j = idx - q * Tn;
        const int k = j % Ns;
        const cx<T>* I = in + (size_t)q * N;
        cx<T>* O = out + (size_t)q * N;
        cx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = I[j + r * Tn];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) v[r] = mul(v[r], tw[k * r * tstep]);
        }
        Dft<T, R>::run(v);
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) O[base + r * Ns] = v[r];
    }
}

// The same stage for any radix R, one output per thread: output m of
// butterfly j is sum_r in[j + r N/R] e^{-2 pi i r (k + m Ns) / (Ns R)}, the
// exponent r (k + m Ns) N / (Ns R) taken modulo N in the twiddle table.
template <typename T>
__device__ __forceinline__ void stage_any(const cx<T>* __restrict__ in, cx<T>* __restrict__ out,
                                          const cx<T>* __restrict__ tw, int N, int R, int Ns, int pp)
{
    const int Tn = N / R;
    const int tstep = N / (Ns * R);
    for (int idx = threadIdx.x; idx < pp * N; idx += blockDim.x) {
        const int q = idx / N;
        const int rem = idx - q * N;
        const int j = rem / R;
        const int m = rem - j * R;
        const int k = j % Ns;
        const cx<T>* I = in + (size_t)q * N;
        const int step = (k + m * Ns) * tstep;   // < N
        cx<T> y = mk(T(0), T(0));
        int e = 0;
        for (int r = 0; r < R; ++r) {
            y = add(y, mul(I[j + r * Tn], tw[e]));
            e += step;
            if (e >= N) e -= N;
        }
        out[(size_t)q * N + (j / Ns) * Ns * R + k + m * Ns] = y;
    }
}

// Forward FFT of pp transforms held in a, twiddles tw (shared or global
// memory); returns the buffer holding the result (a or b). a must be
// complete (synchronised) on entry; the result is synchronised on return.
template <typename T>
__device__ cx<T>* fft(cx<T>* a, cx<T>* b, const cx<T>* tw, const Dir& D, int pp)
{
    int Ns = 1;
    for (int s = 0; s < D.nst; ++s) {
        const int R = D.rad[s];
        switch (R) {
            case 4: stage<T, 4>(a, b, tw, D.N, Ns, pp); break;
            case 2: stage<T, 2>(a, b, tw, D.N, Ns, pp); break;
            case 3: stage<T, 3>(a, b, tw, D.N, Ns, pp); break;
            case 5: stage<T, 5>(a, b, tw, D.N, Ns, pp); break;
            default: stage_any<T>(a, b, tw, D.N, R, Ns, pp); break;
        }
        __syncthreads();
        cx<T>* t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

// Shared memory of a pass: the twiddle and E tables when they fit (stw),
// then the two buffers of g transforms. Returns the buffers' start; tw / E
// point at the tables the pass reads (shared copies once synchronised).
template <typename T>
__device__ __forceinline__ cx<T>* stage_tables(unsigned char* raw, const Dir& D, int stw, const cx<T>*& tw,
                                               const cx<T>*& E)
{
    const int N = D.N;
    tw = static_cast<const cx<T>*>(D.tw);
    E = static_cast<const cx<T>*>(D.E);
    cx<T>* base = reinterpret_cast<cx<T>*>(raw);
    if (!stw) return base;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        base[k] = tw[k];
        base[N + k] = E[k];
    }
    tw = base;
    E = base + N;
    return base + 2 * N;
}

// position of sequence element p in the reordered sequence
__device__ __forceinline__ int perm(int p, int N) { return (p & 1) ? N - 1 - (p >> 1) : (p >> 1); }

// Re(E * V)
template <typename T> __device__ __forceinline__ T re_mul(cx<T> e, cx<T> v) { return e.x * v.x - e.y * v.y; }

// Spectra of the two real sequences packed in Z at mode k (A: real part's,
// B: imaginary part's).
template <typename T>
__device__ __forceinline__ void split(const cx<T>* Z, int k, int N, cx<T>& A, cx<T>& B)
{
    const cx<T> z = Z[k], w = cj(Z[k ? N - k : 0]);
    A = scl(T(0.5), add(z, w));
    B = scl(T(0.5), mi(sub(z, w)));
}

// conj of the packed inverse input W = W_a + i W_b at mode k, from the DCT
// coefficients ya = (a_k, a_{N-k}), yb = (b_k, b_{N-k}) (a_N = b_N = 0):
// W_a = (a_k - i a_{N-k}) e^{i pi k/(2N)} / 2 = conj(E_k)/4 (a_k - i a_{N-k}).
template <typename T>
__device__ __forceinline__ cx<T> pack_inv(cx<T> E, T ak, T akr, T bk, T bkr)
{
    const cx<T> P = mk(T(0.25) * E.x, T(-0.25) * E.y);
    return cj(mul(P, mk(ak + bkr, bk - akr)));
}

// ---------------------------------------------------------------------------
// DCT-II along the rows (length D.N) of nrows rows; rows 2q, 2q+1 of the
// CTA's group share one transform.
template <typename T>
__global__ void __launch_bounds__(256) k_dct_rows_fwd(Dir D, long long nrows, int pp, int stw, const T* src, T* dst)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = D.N;
    const cx<T>*tw, *E;
    cx<T>* a = stage_tables<T>(smem_raw, D, stw, tw, E);
    cx<T>* b = a + (size_t)pp * N;
    const long long r0 = 2LL * blockIdx.x * pp;
    for (int idx = threadIdx.x; idx < pp * N; idx += blockDim.x) {
        const int q = idx / N;
        const int p = idx - q * N;
        const long long ra = r0 + 2 * q;
        const T xa = ra < nrows ? src[ra * N + p] : T(0);
        const T xb = ra + 1 < nrows ? src[(ra + 1) * N + p] : T(0);
        a[(size_t)q * N + perm(p, N)] = mk(xa, xb);
    }
    __syncthreads();
    const cx<T>* Z = fft<T>(a, b, tw, D, pp);
    for (int idx = threadIdx.x; idx < pp * N; idx += blockDim.x) {
        const int q = idx / N;
        const int k = idx - q * N;
        const long long ra = r0 + 2 * q;
        cx<T> A, B;
        split(Z + (size_t)q * N, k, N, A, B);
        const cx<T> e = E[k];
        if (ra < nrows) dst[ra * N + k] = re_mul(e, A);
        if (ra + 1 < nrows) dst[(ra + 1) * N + k] = re_mul(e, B);
    }
}

// Inverse DCT-II along the rows.
template <typename T>
__global__ void __launch_bounds__(256) k_dct_rows_inv(Dir D, long long nrows, int pp, int stw, const T* src, T* dst)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = D.N;
    const cx<T>*tw, *Es;
    cx<T>* a = stage_tables<T>(smem_raw, D, stw, tw, Es);
    cx<T>* b = a + (size_t)pp * N;
    const long long r0 = 2LL * blockIdx.x * pp;
    const cx<T>* E = static_cast<const cx<T>*>(D.E);   // read before the tables are synchronised
    for (int idx = threadIdx.x; idx < pp * N; idx += blockDim.x) {
        const int q = idx / N;
        const int k = idx - q * N;
        const long long ra = r0 + 2 * q;
        const int kr = N - k;   // mode N - k (absent for k = 0)
        T ak = T(0), akr = T(0), bk = T(0), bkr = T(0);
        if (ra < nrows) {
            ak = src[ra * N + k];
            if (k) akr = src[ra * N + kr];
        }
        if (ra + 1 < nrows) {
            bk = src[(ra + 1) * N + k];
            if (k) bkr = src[(ra + 1) * N + kr];
        }
        a[(size_t)q * N + k] = pack_inv(E[k], ak, akr, bk, bkr);
    }
    __syncthreads();
    const cx<T>* O = fft<T>(a, b, tw, D, pp);
    const T iN = T(1) / T(N);
    for (int idx = threadIdx.x; idx < pp * N; idx += blockDim.x) {
        const int q = idx / N;
        const int p = idx - q * N;
        const long long ra = r0 + 2 * q;
        const cx<T> o = O[(size_t)q * N + perm(p, N)];
        if (ra < nrows) dst[ra * N + p] = o.x * iN;
        if (ra + 1 < nrows) dst[(ra + 1) * N + p] = -o.y * iN;
    }
}

// Columns of one field: 2 cp consecutive columns per CTA (cp transforms),
// DCT-II along x (length D.N = nx), division by helm (stored transposed,
// helmT[j][k]), inverse along x; in place on s[f] = [nx][ny].
template <typename T>
__global__ void __launch_bounds__(256) k_dct_cols(Dir D, int ny, int cp, int stw, const T* __restrict__ helmT, T* s)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = D.N;
    const cx<T>*tw, *E;
    cx<T>* a = stage_tables<T>(smem_raw, D, stw, tw, E);
    cx<T>* b = a + (size_t)cp * N;
    const int j0 = blockIdx.x * 2 * cp;
    T* S = s + (size_t)blockIdx.y * N * ny;
    const int w2 = 2 * cp;
    for (int idx = threadIdx.x; idx < N * w2; idx += blockDim.x) {
        const int i = idx / w2;
        const int c = idx - i * w2;
        const int j = j0 + c;
        const T v = j < ny ? S[(size_t)i * ny + j] : T(0);
        T* slot = reinterpret_cast<T*>(a + (size_t)(c >> 1) * N + perm(i, N));
        slot[c & 1] = v;
    }
    __syncthreads();
    cx<T>* Z = fft<T>(a, b, tw, D, cp);
    cx<T>* Wb = (Z == a) ? b : a;
    for (int idx = threadIdx.x; idx < cp * N; idx += blockDim.x) {
        const int q = idx / N;
        const int k = idx - q * N;
        const int ja = j0 + 2 * q, jb = ja + 1;
        const T* ha = helmT + (size_t)(ja < ny ? ja : 0) * N;
        const T* hb = helmT + (size_t)(jb < ny ? jb : 0) * N;
        cx<T> A, B;
        split(Z + (size_t)q * N, k, N, A, B);
        // DCT coefficients at k and N - k (conj spectra there), divided by helm
        const T ak = re_mul(E[k], A) / ha[k];
        const T bk = re_mul(E[k], B) / hb[k];
        T akr = T(0), bkr = T(0);
        if (k) {
            akr = re_mul(E[N - k], cj(A)) / ha[N - k];
            bkr = re_mul(E[N - k], cj(B)) / hb[N - k];
        }
        Wb[(size_t)q * N + k] = pack_inv(E[k], ak, akr, bk, bkr);
    }
    __syncthreads();
    const cx<T>* O = fft<T>(Wb, Z, tw, D, cp);
    const T iN = T(1) / T(N);
    for (int idx = threadIdx.x; idx < N * w2; idx += blockDim.x) {
        const int i = idx / w2;
        const int c = idx - i * w2;
        const int j = j0 + c;
        if (j >= ny) continue;
        const cx<T> o = O[(size_t)(c >> 1) * N + perm(i, N)];
        S[(size_t)i * ny + j] = (c & 1) ? -o.y * iN : o.x * iN;
    }
}

static bool factor(int N, Dir& D)
{
    int m = N, n = 0;
    auto push = [&](int r) {
        if (n >= MAX_STAGES) return false;
        D.rad[n++] = r;
        return true;
    };
    for (int r : {4, 2, 3, 5})
        while (m % r == 0) {
            if (!push(r)) return false;
            m /= r;
        }
    for (int p = 7; m > 1; p += 2)
        while (m % p == 0) {
            if (!push(p)) return false;
            m /= p;
        }
    D.nst = n;
    return true;
}

constexpr size_t SMEM_MAX = 200 * 1024;

}  // namespace nm
}  // namespace vd

struct vd_neumann_plan {
    int nx = 0, ny = 0, dtype = 0;
    size_t esz = 0;
    void* dev = nullptr;   // twiddles of both directions, helmT
    vd::nm::Dir dx{}, dy{};
    const void* helmT = nullptr;
    int pp = 1, cp = 1;    // row pairs / column pairs per CTA
};

namespace {
using namespace vd;
using namespace vd::nm;

PerDeviceOnce g_nm_once;

static cudaError_t nm_configure()
{
    return g_nm_once.run([]() -> cudaError_t {
        cudaError_t e = cudaSuccess;
        const int mx = 227 * 1024;
        if (!e) e = cudaFuncSetAttribute(k_dct_rows_fwd<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        if (!e) e = cudaFuncSetAttribute(k_dct_rows_fwd<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        if (!e) e = cudaFuncSetAttribute(k_dct_rows_inv<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        if (!e) e = cudaFuncSetAttribute(k_dct_rows_inv<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        if (!e) e = cudaFuncSetAttribute(k_dct_cols<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        if (!e) e = cudaFuncSetAttribute(k_dct_cols<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        return e;
    });
}

template <typename T>
static void put(std::vector<unsigned char>& img, size_t off, double v)
{
    const T t = (T)v;
    std::memcpy(img.data() + off, &t, sizeof(T));
}

template <typename T>
static void fill_dir(std::vector<unsigned char>& img, size_t tw_off, size_t e_off, int N)
{
    for (int m = 0; m < N; ++m) {
        const double a = 2.0 * M_PI * double(m) / double(N);   // e^{-2 pi i m / N}
        put<T>(img, tw_off + (2 * m) * sizeof(T), std::cos(a));
        put<T>(img, tw_off + (2 * m + 1) * sizeof(T), -std::sin(a));
        const double b = M_PI * double(m) / (2.0 * double(N));   // 2 e^{-i pi m / (2N)}
        put<T>(img, e_off + (2 * m) * sizeof(T), 2.0 * std::cos(b));
        put<T>(img, e_off + (2 * m + 1) * sizeof(T), -2.0 * std::sin(b));
    }
}

}  // namespace

extern "C" vd_status vd_neumann_plan_create(vd_neumann_plan** out, int nx, int ny, int dtype, const double* dx_host,
                                            const double* dy_host, int dxy_spatial, const double* lambd_host,
                                            int lambd_spatial)
{
    if (!out) return VD_ERR_ARG;
    *out = nullptr;
    if (nx < 2 || ny < 2 || (dtype != VD_F32 && dtype != VD_F64) || !dx_host || !dy_host || !lambd_host)
        return VD_ERR_ARG;
    const size_t esz = dtype == VD_F64 ? 8 : 4, csz = 2 * esz;
    vd_neumann_plan* p = new (std::nothrow) vd_neumann_plan();
    if (!p) return VD_ERR_ARG;
    p->nx = nx;
    p->ny = ny;
    p->dtype = dtype;
    p->esz = esz;
    if (!factor(nx, p->dx) || !factor(ny, p->dy)) {
        delete p;
        return VD_ERR_UNSUPPORTED;
    }
    p->dx.N = nx;
    p->dy.N = ny;
    // row pairs per CTA (2 when two CTAs of them fit an SM), column pairs
    // per CTA (4, 2 or 1: 8, 4 or 2 consecutive values of a row per load);
    // the solve lowers both for small batches (more CTAs)
    const size_t row1 = 2 * (size_t)ny * csz, col1 = 2 * (size_t)nx * csz;
    if (row1 > SMEM_MAX || col1 > SMEM_MAX) {
        delete p;
        return VD_ERR_UNSUPPORTED;
    }
    p->pp = 2 * row1 <= 96 * 1024 ? 2 : 1;
    p->cp = 4 * col1 <= SMEM_MAX ? 4 : (2 * col1 <= SMEM_MAX ? 2 : 1);
    // compute_laplace_dctII(nx, ny, dx, dy) - lambd, per point of [nx][ny]
    const size_t n = (size_t)nx * ny;
    std::vector<double> helm(n);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j) {
            const size_t k = (size_t)i * ny + j;
            const double dx = dxy_spatial ? dx_host[k] : dx_host[0];
            const double dy = dxy_spatial ? dy_host[k] : dy_host[0];
            const double lam = lambd_spatial ? lambd_host[k] : lambd_host[0];
            const double h = 2.0 * (std::cos(M_PI / nx * i) - 1.0) / (dx * dx) +
                             2.0 * (std::cos(M_PI / ny * j) - 1.0) / (dy * dy) - lam;
            if (!(h != 0.0) || !std::isfinite(h)) {
                delete p;
                return VD_ERR_ARG;
            }
            helm[k] = h;
        }
    // device image: twx, Ex, twy, Ey, helmT, each 256-byte aligned
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t o_twx = 0, o_ex = al(o_twx + nx * csz), o_twy = al(o_ex + nx * csz), o_ey = al(o_twy + ny * csz),
                 o_h = al(o_ey + ny * csz), total = al(o_h + n * esz);
    std::vector<unsigned char> img(total, 0);
    if (esz == 8) {
        fill_dir<double>(img, o_twx, o_ex, nx);
        fill_dir<double>(img, o_twy, o_ey, ny);
    } else {
        fill_dir<float>(img, o_twx, o_ex, nx);
        fill_dir<float>(img, o_twy, o_ey, ny);
    }
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j) {
            const size_t off = o_h + ((size_t)j * nx + i) * esz;
            if (esz == 8) put<double>(img, off, helm[(size_t)i * ny + j]);
            else put<float>(img, off, helm[(size_t)i * ny + j]);
        }
    if (cudaMalloc(&p->dev, total) != cudaSuccess) {
        (void)cudaGetLastError();
        delete p;
        return VD_ERR_CUDA;
    }
    if (cudaMemcpy(p->dev, img.data(), total, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(p->dev);
        delete p;
        return VD_ERR_CUDA;
    }
    char* base = (char*)p->dev;
    p->dx.tw = base + o_twx;
    p->dx.E = base + o_ex;
    p->dy.tw = base + o_twy;
    p->dy.E = base + o_ey;
    p->helmT = base + o_h;
    *out = p;
    return VD_OK;
}

extern "C" void vd_neumann_plan_destroy(vd_neumann_plan* p)
{
    if (!p) return;
    if (p->dev) cudaFree(p->dev);
    delete p;
}

namespace vd {

template <typename T>
int neumann_solve(const vd_neumann_plan* p, int nf, const T* src, T* dst, cudaStream_t st)
{
    if (nf == 0) return VD_OK;
    if (nm_configure() != cudaSuccess) return VD_ERR_CUDA;
    const int nx = p->nx, ny = p->ny;
    const long long nrows = (long long)nf * nx;
    const size_t csz = 2 * sizeof(T);
    // fewer sequences per CTA while a pass would have under two CTAs an SM
    constexpr long long kFill = 2 * 152;
    int pp = p->pp, cp = p->cp;
    while (pp > 1 && (nrows + 2LL * pp - 1) / (2LL * pp) < kFill) pp /= 2;
    while (cp > 1 && (long long)((ny + 2 * cp - 1) / (2 * cp)) * nf < kFill) cp /= 2;
    const long long rb = (nrows + 2LL * pp - 1) / (2LL * pp);
    if (rb > 0x7fffffffLL) return VD_ERR_UNSUPPORTED;
    // twiddle and E tables in shared memory when they fit beside the buffers
    size_t rsm = 2 * (size_t)pp * ny * csz, csm = 2 * (size_t)cp * nx * csz;
    const int rstw = rsm + 2 * (size_t)ny * csz <= nm::SMEM_MAX ? 1 : 0;
    const int cstw = csm + 2 * (size_t)nx * csz <= nm::SMEM_MAX ? 1 : 0;
    rsm += rstw ? 2 * (size_t)ny * csz : 0;
    csm += cstw ? 2 * (size_t)nx * csz : 0;
    nm::k_dct_rows_fwd<T><<<(unsigned)rb, 256, rsm, st>>>(p->dy, nrows, pp, rstw, src, dst);
    VD_LAUNCH_CHECK();
    const dim3 cg((unsigned)((ny + 2 * cp - 1) / (2 * cp)), (unsigned)nf);
    nm::k_dct_cols<T><<<cg, 256, csm, st>>>(p->dx, ny, cp, cstw, static_cast<const T*>(p->helmT), dst);
    VD_LAUNCH_CHECK();
    nm::k_dct_rows_inv<T><<<(unsigned)rb, 256, rsm, st>>>(p->dy, nrows, pp, rstw, dst, dst);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

template int neumann_solve<float>(const vd_neumann_plan*, int, const float*, float*, cudaStream_t);
template int neumann_solve<double>(const vd_neumann_plan*, int, const double*, double*, cudaStream_t);

}  // namespace vd

extern "C" vd_status vd_neumann_solve(const vd_neumann_plan* p, int nfield, const void* rhs, void* out, void* stream)
{
    if (!p || nfield < 0 || nfield > 65535) return VD_ERR_ARG;
    if (nfield == 0) return VD_OK;
    if (!rhs || !out) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    return p->dtype == VD_F64 ? vd::neumann_solve<double>(p, nfield, (const double*)rhs, (double*)out, st)
                              : vd::neumann_solve<float>(p, nfield, (const float*)rhs, (float*)out, st);
}
