// Definitions behind the host emulation header (test infrastructure).
#include "vd_internal.cuh"

emu_idx threadIdx, blockIdx, blockDim, gridDim;
namespace vd_emu {
long long launches = 0;
}
namespace vd {
namespace nm {
alignas(16) unsigned char smem_raw[256 * 1024];
}
}  // namespace vd
extern "C" long long vd_emu_launches() { return vd_emu::launches; }
