// Fixed scratch of eithot_transpose_noalloc, in a translation unit of its
// own.  Each .cu file is a separate device module, and under CUDA's default
// lazy module loading a module is loaded on a device (its device variables
// allocated) the first time its code or variables are used there.  Kept
// apart from the kernels, the 32 MiB array is therefore only placed on a
// device once eithot_transpose_noalloc looks it up there, not on every GPU
// that runs a transpose.  With CUDA_MODULE_LOADING=EAGER every module, this
// one included, is loaded when the runtime starts on a device.
#include <cuda_runtime.h>

#include <string>

#include "exec.h"

namespace eithot {

// A file-scope device array, so the entry point never allocates.  Once
// loaded on a GPU it stays there until the process exits; all calls share it.
static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

int noalloc_scratch(uint8_t** ptr, std::string* err) {
    // In host code g_noalloc_scratch names a host-side stand-in; its device
    // address is looked up on every call (a host-side table lookup, no
    // allocation), with the caller's device current, so it follows the
    // current device and context, also after a device reset.
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
        *err = std::string("cudaGetSymbolAddress(fixed scratch): ") + cudaGetErrorString(e);
        return EITHOT_STATUS_CUDA;
    }
    *ptr = static_cast<uint8_t*>(p);
    return 0;
}

}  // namespace eithot
