// Spectral Helmholtz helpers of mapping/models/model_qgsw/helmholtz.py: the
// edge padding of solve_helmholtz_dstI (138-143, jnp.pad mode='edge') and the
// capacitance-matrix correction of solve_helmholtz_dstI_cmm (172-184). The
// DST-I solves themselves are the QG plan's pv2h (x-DST, y-tridiagonal,
// x-DST) on a plan whose operator is laplace_dstI - shift.
#include "vd_internal.cuh"

namespace vd {

// dst[i][j] = src[clamp(i, 1, n0-2)][clamp(j, 1, n1-2)] * mask[i][j]; in
// place (src == dst, no mask) only the walls are written.
template <typename T>
__global__ void k_edge_pad(int n0, int n1, const T* __restrict__ src, const T* __restrict__ mask, T* dst,
                           bool walls_only)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y, b = blockIdx.z;
    if (j >= n1) return;
    const bool wall = (i == 0 || i == n0 - 1 || j == 0 || j == n1 - 1);
    if (walls_only && !wall) return;
    const int si = min(max(i, 1), n0 - 2), sj = min(max(j, 1), n1 - 2);
    const long long base = (long long)b * n0 * n1;
    T v = src[base + (long long)si * n1 + sj];
    if (mask) v *= mask[(long long)i * n1 + j];
    dst[base + (long long)i * n1 + j] = v;
}

template <typename T>
__global__ void k_copy_fields(long long n, const T* __restrict__ a, T* __restrict__ b)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) b[k] = a[k];
}

// Field f = s * nper + r belongs to system s:
// out[f][bidx[i]] += sum_j cap[s][i][j] * (-sol[f][bidx[j]]).
template <typename T>
__global__ void k_cmm_add(int nper, int M, long long fs, const T* __restrict__ cap,
                          const int32_t* __restrict__ bidx, const T* __restrict__ sol, T* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= M) return;
    const T* C = cap + (long long)(f / nper) * M * M + (long long)i * M;
    const T* S = sol + f * fs;
    T a = T(0);
    for (int j = 0; j < M; ++j) a -= C[j] * S[bidx[j]];
    out[f * fs + bidx[i]] += a;
}

}  // namespace vd

extern "C" vd_status vd_edge_pad(int dtype, int nfield, int n0, int n1, const void* src, const void* mask,
                                 void* dst, void* stream)
{
    if (nfield < 0 || n0 < 3 || n1 < 3 || (dtype != VD_F32 && dtype != VD_F64)) return VD_ERR_ARG;
    if (nfield == 0) return VD_OK;
    if (!src || !dst || nfield > 65535 || n0 > 65535) return VD_ERR_ARG;
    const bool in_place = (src == dst);
    if (in_place && mask) return VD_ERR_ARG;
    const dim3 g((unsigned)((n1 + 127) / 128), (unsigned)n0, (unsigned)nfield);
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == VD_F32)
        vd::k_edge_pad<float><<<g, 128, 0, st>>>(n0, n1, (const float*)src, (const float*)mask, (float*)dst,
                                                 in_place);
    else
        vd::k_edge_pad<double><<<g, 128, 0, st>>>(n0, n1, (const double*)src, (const double*)mask, (double*)dst,
                                                  in_place);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

extern "C" vd_status vd_cmm_correct(int dtype, int nsys, int nper, int M, long long field_elems, const void* cap,
                                    const int32_t* bidx, const void* sol, const void* rhs, void* out,
                                    void* stream)
{
    if (nsys < 1 || nper < 0 || M < 0 || field_elems < 1 || (dtype != VD_F32 && dtype != VD_F64))
        return VD_ERR_ARG;
    if (nper == 0) return VD_OK;
    const long long nfield = (long long)nsys * nper;
    if (!sol || !rhs || !out || out == sol || (M > 0 && (!cap || !bidx)) || nfield > 65535) return VD_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const long long n = nfield * field_elems;
    const unsigned nb = (unsigned)((n + 255) / 256);
    if (out != rhs) {
        if (dtype == VD_F32) vd::k_copy_fields<float><<<nb, 256, 0, st>>>(n, (const float*)rhs, (float*)out);
        else vd::k_copy_fields<double><<<nb, 256, 0, st>>>(n, (const double*)rhs, (double*)out);
        VD_LAUNCH_CHECK();
    }
    if (M == 0) return VD_OK;
    const dim3 g((unsigned)((M + 127) / 128), (unsigned)nfield);
    if (dtype == VD_F32)
        vd::k_cmm_add<float><<<g, 128, 0, st>>>(nper, M, field_elems, (const float*)cap, bidx, (const float*)sol,
                                                (float*)out);
    else
        vd::k_cmm_add<double><<<g, 128, 0, st>>>(nper, M, field_elems, (const double*)cap, bidx,
                                                 (const double*)sol, (double*)out);
    VD_LAUNCH_CHECK();
    return VD_OK;
}

namespace vd {
// Transpose of k_edge_pad: interior cell (i, j) gathers mask * ad from every
// padded position that copies it (itself and, on the interior's edge, the
// adjacent wall and corner cells); walls of the result are zero.
template <typename T>
__global__ void k_edge_pad_adj(int n0, int n1, const T* __restrict__ ad, const T* __restrict__ mask, T* __restrict__ out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y, b = blockIdx.z;
    if (j >= n1) return;
    const long long base = (long long)b * n0 * n1;
    if (i == 0 || i == n0 - 1 || j == 0 || j == n1 - 1) {
        out[base + (long long)i * n1 + j] = T(0);
        return;
    }
    int is[3], js[3], ni = 0, nj = 0;
    is[ni++] = i;
    if (i == 1) is[ni++] = 0;
    if (i == n0 - 2) is[ni++] = n0 - 1;
    js[nj++] = j;
    if (j == 1) js[nj++] = 0;
    if (j == n1 - 2) js[nj++] = n1 - 1;
    T a = T(0);
    for (int p = 0; p < ni; ++p)
        for (int q = 0; q < nj; ++q) {
            const long long k = (long long)is[p] * n1 + js[q];
            a += mask ? mask[k] * ad[base + k] : ad[base + k];
        }
    out[base + (long long)i * n1 + j] = a;
}
}  // namespace vd

extern "C" vd_status vd_edge_pad_adj(int dtype, int nfield, int n0, int n1, const void* ad, const void* mask,
                                     void* out, void* stream)
{
    if (nfield < 0 || n0 < 3 || n1 < 3 || (dtype != VD_F32 && dtype != VD_F64)) return VD_ERR_ARG;
    if (nfield == 0) return VD_OK;
    if (!ad || !out || ad == out || nfield > 65535 || n0 > 65535) return VD_ERR_ARG;
    const dim3 g((unsigned)((n1 + 127) / 128), (unsigned)n0, (unsigned)nfield);
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == VD_F32)
        vd::k_edge_pad_adj<float><<<g, 128, 0, st>>>(n0, n1, (const float*)ad, (const float*)mask, (float*)out);
    else
        vd::k_edge_pad_adj<double><<<g, 128, 0, st>>>(n0, n1, (const double*)ad, (const double*)mask, (double*)out);
    VD_LAUNCH_CHECK();
    return VD_OK;
}
