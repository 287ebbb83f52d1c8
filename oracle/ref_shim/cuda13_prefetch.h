// Build shim for compiling the reference's own sources against CUDA 13
// (baseline use only): CUDA 13's cudaMemPrefetchAsync takes a
// cudaMemLocation and flags, while the reference passes a device ordinal and
// a stream (ITNT/src/util.h:25).  Force-included ahead of the reference's
// translation units, this overload keeps the reference's call meaning the
// same: prefetch to device `device` on stream `stream`.
#pragma once
#include <cuda_runtime.h>

static inline cudaError_t cudaMemPrefetchAsync(const void* ptr, size_t count, int device, cudaStream_t stream) {
    cudaMemLocation loc = {};
    loc.type = cudaMemLocationTypeDevice;
    loc.id = device;
    return cudaMemPrefetchAsync(ptr, count, loc, 0u, stream);
}
