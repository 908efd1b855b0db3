// PV -> SSH inversion for callers that cannot allocate GPU memory.
//
// Some hosts of this library cannot call cudaMalloc: code running inside a
// captured or replayed CUDA graph whose memory plan is frozen, plugins loaded
// into a process whose GPU memory is owned by another allocator (a framework
// caching allocator or a pool the host application manages), and FFI callers
// (Go, Java, JavaScript bindings) that only hand over buffers they already
// own. vd_qg1l_pv2h needs a caller-provided workspace for its spectral
// intermediate; vd_qg1l_pv2h_noalloc instead keeps that intermediate in a
// fixed array compiled into the library, so the caller passes only the
// inputs and the output.
//
// The array below is allocated once per device when the library's module is
// loaded on it and is held until the process exits. Its name is only a
// host-side handle: kernels must be given the device address that
// cudaGetSymbolAddress returns for the current device.
#include "vd_internal.cuh"
#include <mutex>

#define VD_NOALLOC_SCRATCH_BYTES (16u << 20)

static __device__ __align__(256) unsigned char g_pv2h_scratch[VD_NOALLOC_SCRATCH_BYTES];

namespace vd {
template <typename T>
int finalize_impl(const vd_qg1l_plan*, int, const T*, const T*, const T*, double, const double*, int, T*,
                  cudaStream_t);
}

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device, looked up on
// the first call for that device and cached until the process exits (a
// cudaDeviceReset while the library is loaded is not supported).
int scratch_for_current_device(void** out)
{
    int dev = -1;
    VD_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return VD_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        VD_CUDA_TRY(cudaGetSymbolAddress(&ptr, g_pv2h_scratch));
        if (!ptr) return VD_ERR_CUDA;
        g_scratch_ptr[dev] = ptr;
    }
    *out = g_scratch_ptr[dev];
    return VD_OK;
}

template <typename T>
int pv2h_noalloc_t(const vd_qg1l_plan* p, int B, const T* q, const T* hb, const T* qb, T* h, T* spec,
                   cudaStream_t st)
{
    vd::SolveArgs a;
    a.src = q; a.sub = qb; a.sub_batches = qb ? B : 0;
    a.out = h; a.add = hb; a.add_batches = hb ? B : 0; a.epi = vd::EPI_H;
    int rc = vd::helmholtz_solve<T>(p, B, a, spec, st);
    if (rc) return rc;
    return vd::finalize_impl<T>(p, B, h, hb, nullptr, 0.0, nullptr, 0, h, st);
}

}  // namespace

extern "C" size_t vd_qg1l_pv2h_noalloc_max_bytes(void) { return VD_NOALLOC_SCRATCH_BYTES; }

extern "C" vd_status vd_qg1l_pv2h_noalloc(const vd_qg1l_plan* p, int B, const void* q, const void* hb,
                                          const void* qb, void* h, void* stream)
{
    if (!p || B <= 0 || !q || !h) return VD_ERR_ARG;
    // every spectral element the solve reads is written earlier in the same
    // call, so the array needs no clearing between calls
    if (vd::spec_bytes(p, B) > VD_NOALLOC_SCRATCH_BYTES) return VD_ERR_SIZE;
    void* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    return p->d.dtype == VD_F32
               ? pv2h_noalloc_t<float>(p, B, (const float*)q, (const float*)hb, (const float*)qb, (float*)h,
                                       (float*)scratch, st)
               : pv2h_noalloc_t<double>(p, B, (const double*)q, (const double*)hb, (const double*)qb,
                                        (double*)h, (double*)scratch, st);
}
