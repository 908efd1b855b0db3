// Along-track observation operator and FP64 reductions.
//
// Reference: mapping/src/obsop.py, Obsop_interp_l3_jax — operator rows from
// _sparse_op (417-460: up to Npix nearest grid points, Gaussian weights,
// normalised, invalid neighbours dropped), the misfit (610-628) and its
// adjoint through jax.vjp (630-678); cost terms of
// mapping/src/tools_4Dvar.py:252-400 (Jo = misfit.R^-1.misfit, Jb = X0.X0).
#include "vd_internal.cuh"
#include "vd_obs_knn.cuh"

namespace vd {

template <typename T>
__global__ void k_obs_misfit(int nobs, const T* __restrict__ fields, long long stride,
                             const int32_t* __restrict__ obs_field, const int32_t* __restrict__ idx4,
                             const T* __restrict__ w4, const T* __restrict__ yobs,
                             const T* __restrict__ inverr, T* __restrict__ misfit)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nobs) return;
    const T* x = fields + (obs_field ? (long long)obs_field[o] * stride : 0LL);
    T hx = T(0);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const int g = idx4[4 * o + m];
        if (g >= 0) hx += w4[4 * o + m] * x[g];
    }
    T d = hx - yobs[o];
    if (isnan(d)) d = T(0);
    misfit[o] = inverr[o] * d;
}

template <typename T>
__global__ void k_obs_adjoint(int npts, T* __restrict__ ad, long long stride,
                              const int32_t* __restrict__ pt_field, const int32_t* __restrict__ pt_index,
                              const int32_t* __restrict__ rowptr, const int32_t* __restrict__ ent_obs,
                              const T* __restrict__ ent_w, const T* __restrict__ inverr,
                              const T* __restrict__ cot)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npts) return;
    T acc = T(0);
    for (int e = rowptr[k]; e < rowptr[k + 1]; ++e) {
        const int o = ent_obs[e];
        acc += ent_w[e] * (inverr[o] * cot[o]);
    }
    T* a = ad + (pt_field ? (long long)pt_field[k] * stride : 0LL);
    a[pt_index[k]] += acc;
}

// One CTA per segment, fixed-order tree reduction in double.
template <typename T>
__global__ void __launch_bounds__(256)
k_sumsq_seg(const int32_t* __restrict__ off, const T* __restrict__ x, double* __restrict__ out)
{
    __shared__ double sh[256];
    const int s = blockIdx.x;
    double acc = 0.0;
    for (int k = off[s] + threadIdx.x; k < off[s + 1]; k += 256) {
        const double v = (double)x[k];
        acc = fma(v, v, acc);
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[s] = sh[0];
}

constexpr int kDotBlocks = 1024;

template <typename T>
__global__ void __launch_bounds__(256)
k_dot_partial(long long n, const T* __restrict__ x, const T* __restrict__ y, double* __restrict__ part)
{
    __shared__ double sh[256];
    double acc = 0.0;
    for (long long k = (long long)blockIdx.x * 256 + threadIdx.x; k < n; k += (long long)gridDim.x * 256)
        acc = fma((double)x[k], (double)y[k], acc);
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(256) k_dot_final(int np, const double* __restrict__ part, double* __restrict__ out)
{
    __shared__ double sh[256];
    double acc = 0.0;
    for (int k = threadIdx.x; k < np; k += 256) acc += part[k];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

template <typename T>
__global__ void k_axpby(long long n, T a, const T* __restrict__ x, T b, T* __restrict__ y)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) y[k] = a * x[k] + b * y[k];
}

}  // namespace vd

using namespace vd;

extern "C" vd_status vd_obs_misfit(int dtype, int nobs, const void* fields, long long field_stride,
                                   const int32_t* obs_field, const int32_t* idx4, const void* w4,
                                   const void* yobs, const void* inverr, void* misfit, void* stream)
{
    if (nobs < 0 || (dtype != VD_F32 && dtype != VD_F64)) return VD_ERR_ARG;
    if (nobs == 0) return VD_OK;
    if (!fields || !idx4 || !w4 || !yobs || !inverr || !misfit) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = (nobs + 255) / 256;
    if (dtype == VD_F32)
        k_obs_misfit<float><<<grid, 256, 0, st>>>(nobs, (const float*)fields, field_stride, obs_field, idx4,
                                                  (const float*)w4, (const float*)yobs, (const float*)inverr,
                                                  (float*)misfit);
    else
        k_obs_misfit<double><<<grid, 256, 0, st>>>(nobs, (const double*)fields, field_stride, obs_field, idx4,
                                                   (const double*)w4, (const double*)yobs,
                                                   (const double*)inverr, (double*)misfit);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

extern "C" vd_status vd_obs_adjoint(int dtype, int npoints, void* ad_fields, long long field_stride,
                                    const int32_t* pt_field, const int32_t* pt_index, const int32_t* rowptr,
                                    const int32_t* ent_obs, const void* ent_w, const void* inverr,
                                    const void* cot, void* stream)
{
    if (npoints < 0 || (dtype != VD_F32 && dtype != VD_F64)) return VD_ERR_ARG;
    if (npoints == 0) return VD_OK;
    if (!ad_fields || !pt_index || !rowptr || !ent_obs || !ent_w || !inverr || !cot) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = (npoints + 255) / 256;
    if (dtype == VD_F32)
        k_obs_adjoint<float><<<grid, 256, 0, st>>>(npoints, (float*)ad_fields, field_stride, pt_field, pt_index,
                                                   rowptr, ent_obs, (const float*)ent_w, (const float*)inverr,
                                                   (const float*)cot);
    else
        k_obs_adjoint<double><<<grid, 256, 0, st>>>(npoints, (double*)ad_fields, field_stride, pt_field,
                                                    pt_index, rowptr, ent_obs, (const double*)ent_w,
                                                    (const double*)inverr, (const double*)cot);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

extern "C" vd_status vd_sumsq_f64(int dtype, int nseg, const int32_t* seg_off, const void* x, double* out,
                                  void* stream)
{
    if (nseg < 0 || (dtype != VD_F32 && dtype != VD_F64)) return VD_ERR_ARG;
    if (nseg == 0) return VD_OK;
    if (!seg_off || !x || !out) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == VD_F32)
        k_sumsq_seg<float><<<nseg, 256, 0, st>>>(seg_off, (const float*)x, out);
    else
        k_sumsq_seg<double><<<nseg, 256, 0, st>>>(seg_off, (const double*)x, out);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

// `out` must have room for kDotBlocks + 1 doubles: the partial sums follow the
// result (out[1..]) so that the call allocates nothing.
extern "C" vd_status vd_dot_f64(int dtype, long long n, const void* x, const void* y, double* out, void* stream)
{
    if (n < 0 || (dtype != VD_F32 && dtype != VD_F64) || !out) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    double* part = out + 1;
    if (n == 0) {
        k_dot_final<<<1, 256, 0, st>>>(0, part, out);
        VD_LAUNCH_CHECK();
        return VD_OK;
    }
    if (!x || !y) return VD_ERR_ARG;
    if (dtype == VD_F32)
        k_dot_partial<float><<<kDotBlocks, 256, 0, st>>>(n, (const float*)x, (const float*)y, part);
    else
        k_dot_partial<double><<<kDotBlocks, 256, 0, st>>>(n, (const double*)x, (const double*)y, part);
    VD_LAUNCH_CHECK();
    k_dot_final<<<1, 256, 0, st>>>(kDotBlocks, part, out);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

extern "C" vd_status vd_axpby(int dtype, long long n, double a, const void* x, double b, void* y, void* stream)
{
    if (n < 0 || (dtype != VD_F32 && dtype != VD_F64)) return VD_ERR_ARG;
    if (n == 0) return VD_OK;
    if (!x || !y) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (dtype == VD_F32)
        k_axpby<float><<<grid, 256, 0, st>>>(n, (float)a, (const float*)x, (float)b, (float*)y);
    else
        k_axpby<double><<<grid, 256, 0, st>>>(n, a, (const double*)x, b, (double*)y);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

namespace vd {

template <typename T>
__global__ void __launch_bounds__(256)
k_sumsq_gather(const int32_t* __restrict__ off, const int32_t* __restrict__ perm, const T* __restrict__ x,
               double scale, double* __restrict__ out)
{
    __shared__ double sh[256];
    const int s = blockIdx.x;
    double acc = 0.0;
    for (int k = off[s] + threadIdx.x; k < off[s + 1]; k += 256) {
        const double v = (double)x[perm[k]];
        acc = fma(v, v, acc);
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[s] = scale * sh[0];
}

template <typename T>
__global__ void k_diag_axpy(long long n, long long period, const T* __restrict__ d, const T* x, const T* y,
                            T* out)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const T v = d[k % period] * x[k] + (y ? y[k] : T(0));
    out[k] = v;
}

template <typename T>
__global__ void k_fill_value(long long n, T v, T* __restrict__ y)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) y[k] = v;
}

}  // namespace vd

extern "C" vd_status vd_sumsq_gather_f64(int dtype, int nseg, const int32_t* seg_off, const int32_t* perm,
                                         const void* x, double scale, double* out, void* stream)
{
    if (nseg < 0 || (dtype != VD_F32 && dtype != VD_F64)) return VD_ERR_ARG;
    if (nseg == 0) return VD_OK;
    if (!seg_off || !perm || !x || !out) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == VD_F32)
        k_sumsq_gather<float><<<nseg, 256, 0, st>>>(seg_off, perm, (const float*)x, scale, out);
    else
        k_sumsq_gather<double><<<nseg, 256, 0, st>>>(seg_off, perm, (const double*)x, scale, out);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

extern "C" vd_status vd_copy(int dtype, long long n, const void* x, void* y, void* stream)
{
    if (n < 0 || (dtype != VD_F32 && dtype != VD_F64)) return VD_ERR_ARG;
    if (n == 0) return VD_OK;
    if (!x || !y) return VD_ERR_ARG;
    VD_CUDA_TRY(cudaMemcpyAsync(y, x, size_t(n) * elem_size(dtype), cudaMemcpyDeviceToDevice,
                                (cudaStream_t)stream));
    return VD_OK;
}

extern "C" vd_status vd_fill(int dtype, long long n, double value, void* y, void* stream)
{
    if (n < 0 || (dtype != VD_F32 && dtype != VD_F64)) return VD_ERR_ARG;
    if (n == 0) return VD_OK;
    if (!y) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (dtype == VD_F32)
        k_fill_value<float><<<grid, 256, 0, st>>>(n, (float)value, (float*)y);
    else
        k_fill_value<double><<<grid, 256, 0, st>>>(n, value, (double*)y);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

extern "C" vd_status vd_diag_axpy(int dtype, long long n, long long period, const void* d, const void* x,
                                  const void* y, void* out, void* stream)
{
    if (n < 0 || period <= 0 || (dtype != VD_F32 && dtype != VD_F64)) return VD_ERR_ARG;
    if (n == 0) return VD_OK;
    if (!d || !x || !out) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (dtype == VD_F32)
        k_diag_axpy<float><<<grid, 256, 0, st>>>(n, period, (const float*)d, (const float*)x, (const float*)y,
                                                 (float*)out);
    else
        k_diag_axpy<double><<<grid, 256, 0, st>>>(n, period, (const double*)d, (const double*)x,
                                                  (const double*)y, (double*)out);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

// ---------------------------------------------------------------------------
// Observation-operator construction: one thread per observation runs the
// neighbour search of vd_obs_knn.cuh.
// ---------------------------------------------------------------------------
namespace vd {
__global__ void k_obs_knn(long long nobs, const double* __restrict__ x, const double* __restrict__ y, int ny, int nx,
                          double dx, double dy, int npix, double dmax, const unsigned char* __restrict__ excl,
                          long long* __restrict__ idx, double* __restrict__ w)
{
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nobs) return;
    obs_knn_point(x[o], y[o], ny, nx, dx, dy, npix, dmax, excl, idx + o * 4, w + o * 4);
}
}  // namespace vd

extern "C" vd_status vd_obs_knn_excl(long long nobs, const double* x_km, const double* y_km, int ny, int nx,
                                     double dx_km, double dy_km, int npix, double dmax_km, const unsigned char* exclude,
                                     long long* idx, double* w, void* stream)
{
    if (nobs < 0 || ny < 1 || nx < 1 || npix < 1 || npix > 4 || !(dx_km > 0) || !(dy_km > 0) || !(dmax_km > 0))
        return VD_ERR_ARG;
    if (nobs == 0) return VD_OK;
    if (!x_km || !y_km || !idx || !w) return VD_ERR_ARG;
    vd::k_obs_knn<<<(unsigned)((nobs + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
        nobs, x_km, y_km, ny, nx, dx_km, dy_km, npix, dmax_km, exclude, idx, w);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

extern "C" vd_status vd_obs_knn(long long nobs, const double* x_km, const double* y_km, int ny, int nx, double dx_km,
                                double dy_km, int npix, double dmax_km, long long* idx, double* w, void* stream)
{
    return vd_obs_knn_excl(nobs, x_km, y_km, ny, nx, dx_km, dy_km, npix, dmax_km, nullptr, idx, w, stream);
}
