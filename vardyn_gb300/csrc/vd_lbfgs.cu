// Batched vector kernels of the outer minimisation (L-BFGS without bounds
// for B independent windows, the quasi-Newton loop of mapping/src/inv.py:
// 309-414): deterministic float64 dot products and axpys whose coefficients
// live on the device, so the two-loop recursion runs without host round trips.
#include "vd_internal.cuh"

namespace vd {

constexpr int LB_THREADS = 256;

// partial sums of x[b] . y[b] over blocks of the window: part[b][blk]
__global__ void k_bdot_part(long long n, const double* __restrict__ x, const double* __restrict__ y,
                            double* __restrict__ part)
{
    const int b = blockIdx.y, nb = gridDim.x;
    const double* X = x + (long long)b * n;
    const double* Y = y + (long long)b * n;
    double a = 0;
    for (long long k = (long long)blockIdx.x * LB_THREADS + threadIdx.x; k < n; k += (long long)nb * LB_THREADS)
        a += X[k] * Y[k];
    __shared__ double red[LB_THREADS];
    red[threadIdx.x] = a;
    __syncthreads();
    for (int s = LB_THREADS / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(long long)b * nb + blockIdx.x] = red[0];
}

// out[b] = c0[b] + c1[b] * sum(part[b][:]) (fixed order)
__global__ void k_bdot_final(int B, int nb, const double* __restrict__ part, const double* __restrict__ c0,
                             const double* __restrict__ c1, double* __restrict__ out)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    double s = 0;
    for (int k = 0; k < nb; ++k) s += part[(long long)b * nb + k];
    out[b] = (c0 ? c0[b] : 0.0) + (c1 ? c1[b] : 1.0) * s;
}

// y[b] = beta * y[b] + scale * coef[b] * x[b]  (coef nullable -> 1)
__global__ void k_baxpy(long long n, double scale, const double* __restrict__ coef, const double* __restrict__ x,
                        double beta, double* __restrict__ y)
{
    const int b = blockIdx.y;
    const double c = scale * (coef ? coef[b] : 1.0);
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long o = (long long)b * n + k;
        y[o] = beta * y[o] + c * x[o];
    }
}

// z[b] = x[b] + coef[b] * y[b]
__global__ void k_bxpay(long long n, const double* __restrict__ x, const double* __restrict__ coef,
                        const double* __restrict__ y, double* __restrict__ z)
{
    const int b = blockIdx.y;
    const double c = coef[b];
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long o = (long long)b * n + k;
        z[o] = x[o] + c * y[o];
    }
}

static int nblocks(long long n)
{
    long long nb = (n + LB_THREADS * 8 - 1) / (LB_THREADS * 8);
    if (nb < 1) nb = 1;
    if (nb > 1024) nb = 1024;
    return (int)nb;
}

}  // namespace vd

extern "C" size_t vd_bdot_workspace_bytes(int batch, long long n)
{
    if (batch <= 0 || n <= 0) return 0;
    return sizeof(double) * (size_t)batch * vd::nblocks(n);
}

extern "C" vd_status vd_bdot_f64(int batch, long long n, const double* x, const double* y, const double* c0,
                                 const double* c1, double* out, void* work, size_t work_bytes, void* stream)
{
    if (batch <= 0 || batch > 65535 || n <= 0 || !x || !y || !out || !work) return VD_ERR_ARG;
    const int nb = vd::nblocks(n);
    if (work_bytes < sizeof(double) * (size_t)batch * nb) return VD_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    vd::k_bdot_part<<<dim3((unsigned)nb, (unsigned)batch), vd::LB_THREADS, 0, st>>>(n, x, y, (double*)work);
    VD_LAUNCH_CHECK();
    vd::k_bdot_final<<<(unsigned)((batch + 127) / 128), 128, 0, st>>>(batch, nb, (const double*)work, c0, c1, out);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

extern "C" vd_status vd_baxpy_f64(int batch, long long n, double scale, const double* coef, const double* x,
                                  double beta, double* y, void* stream)
{
    if (batch <= 0 || batch > 65535 || n <= 0 || !x || !y) return VD_ERR_ARG;
    const unsigned g = (unsigned)((n + 255) / 256 < 2048 ? (n + 255) / 256 : 2048);
    vd::k_baxpy<<<dim3(g, (unsigned)batch), 256, 0, (cudaStream_t)stream>>>(n, scale, coef, x, beta, y);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

extern "C" vd_status vd_bxpay_f64(int batch, long long n, const double* x, const double* coef, const double* y,
                                  double* z, void* stream)
{
    if (batch <= 0 || batch > 65535 || n <= 0 || !x || !coef || !y || !z) return VD_ERR_ARG;
    const unsigned g = (unsigned)((n + 255) / 256 < 2048 ? (n + 255) / 256 : 2048);
    vd::k_bxpay<<<dim3(g, (unsigned)batch), 256, 0, (cudaStream_t)stream>>>(n, x, coef, y, z);
    VD_LAUNCH_CHECK();
    return VD_OK;
}
