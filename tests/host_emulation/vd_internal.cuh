// Host emulation of the CUDA runtime and kernel launches, for CPU tests of
// the library's kernel sources (test infrastructure; never part of the
// product library). A translation unit of the library copied next to this
// file and compiled with g++ sees this header instead of the library's own
// vd_internal.cuh. Memory is host memory; a launch runs the kernel body once
// per thread of the grid in sequence (kernels without barriers), or once per
// block with a one-thread block for kernels whose block-stride loops are
// separated by barriers (each phase then completes before the next starts).
#pragma once
#include <stdint.h>
#include <stddef.h>
#include <math.h>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include "vardyn_gb300.h"

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __shared__
#define __align__(n)
#define __grid_constant__
#define __syncthreads() ((void)0)

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2, cudaErrorInvalidDevice = 101 };
typedef void* cudaStream_t;
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice,
                      cudaMemcpyDefault };
enum { cudaFuncAttributeMaxDynamicSharedMemorySize = 8 };

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct emu_idx {
    unsigned x, y, z;
};
extern emu_idx threadIdx, blockIdx, blockDim, gridDim;

inline cudaError_t cudaMalloc(void** p, size_t n)
{
    *p = std::aligned_alloc(256, (n + 255) & ~size_t(255));
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaFree(void* p) { std::free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) { std::memmove(d, s, n); return cudaSuccess; }
inline cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind, cudaStream_t = 0)
{
    std::memmove(d, s, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemsetAsync(void* d, int v, size_t n, cudaStream_t = 0) { std::memset(d, v, n); return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaGetDevice(int* d) { *d = 0; return cudaSuccess; }
template <class K> inline cudaError_t cudaFuncSetAttribute(K, int, int) { return cudaSuccess; }

inline float atomicAdd(float* p, float v) { const float o = *p; *p = o + v; return o; }
inline double atomicAdd(double* p, double v) { const double o = *p; *p = o + v; return o; }
inline float __fdividef(float a, float b) { return a / b; }
template <class T> inline T __ldg(const T* p) { return *p; }

namespace vd_emu {
extern long long launches;
template <class F, class G, class B>
void launch(bool coop, F f, G grid, B block, size_t = 0, cudaStream_t = 0)
{
    const dim3 g(grid), b(block);
    ++launches;
    gridDim = {g.x, g.y, g.z};
    blockDim = coop ? emu_idx{1, 1, 1} : emu_idx{b.x, b.y, b.z};
    for (unsigned bz = 0; bz < g.z; ++bz)
        for (unsigned by = 0; by < g.y; ++by)
            for (unsigned bx = 0; bx < g.x; ++bx) {
                blockIdx = {bx, by, bz};
                for (unsigned tz = 0; tz < blockDim.z; ++tz)
                    for (unsigned ty = 0; ty < blockDim.y; ++ty)
                        for (unsigned tx = 0; tx < blockDim.x; ++tx) {
                            threadIdx = {tx, ty, tz};
                            f();
                        }
            }
}
}  // namespace vd_emu

#define VD_CUDA_TRY(expr)                                  \
    do {                                                   \
        cudaError_t _e = (expr);                           \
        if (_e != cudaSuccess) return VD_ERR_CUDA;         \
    } while (0)
#define VD_LAUNCH_CHECK() ((void)0)

namespace vd {
struct PerDeviceOnce {
    template <typename F>
    cudaError_t run(F&& fn) { return fn(); }
};
struct Arena {
    char* base;
    size_t cap;
    size_t off;
    void* take(size_t bytes)
    {
        size_t a = (off + 255) & ~size_t(255);
        if (a + bytes > cap) return nullptr;
        off = a + bytes;
        return base + a;
    }
};
template <typename T>
int neumann_solve(const vd_neumann_plan* p, int nf, const T* src, T* dst, cudaStream_t st);
}  // namespace vd
