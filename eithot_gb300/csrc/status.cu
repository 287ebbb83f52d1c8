// Per-call device status words, in a translation unit of their own.
//
// Call id k owns word k mod kStatusRing of a file-scope device array; a call
// zeroes its word on its stream before its first pass and its kernels OR
// kCallIndexFault / kCallSyncTimeout into it through the pointer they are
// given.  The host looks the array up on every call (cudaGetSymbolAddress),
// which needs the module holding it loaded on the device; kept in a small
// module of its own, that lookup and the status reads never depend on the
// module of the kernels.
#include <cuda_runtime.h>

#include <atomic>
#include <string>

#include "exec.h"

namespace eithot {

namespace {
__device__ unsigned int g_call_status[kStatusRing];
std::atomic<uint64_t> g_next_call{1};
}  // namespace

uint64_t next_call_id() { return g_next_call.load(); }

int begin_call(cudaStream_t stream, uint64_t* id, unsigned** status, std::string* err) {
    // The device address is looked up on every call (a host-side table
    // lookup), so it follows the current device and survives a device reset.
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_call_status);
    if (e != cudaSuccess || p == nullptr) {
        *err = std::string("cudaGetSymbolAddress(call status): ") + cudaGetErrorString(e);
        return EITHOT_STATUS_CUDA;
    }
    const uint64_t k = g_next_call.fetch_add(1);
    unsigned* word = static_cast<unsigned*>(p) + (k % kStatusRing);
    e = cudaMemsetAsync(word, 0, sizeof(unsigned), stream);
    if (e != cudaSuccess) {
        *err = std::string("cudaMemsetAsync(call status): ") + cudaGetErrorString(e);
        return EITHOT_STATUS_CUDA;
    }
    *id = k;
    *status = word;
    return 0;
}

int read_call_status(uint64_t id, cudaStream_t stream, unsigned* bits, std::string* err) {
    const uint64_t next = g_next_call.load();
    if (id == 0 || id >= next) {
        *err = "unknown call id";
        return EITHOT_STATUS_INVALID;
    }
    if (next - id > kStatusRing) {
        *err = "the call's status word has been reused by a later call";
        return EITHOT_STATUS_INVALID;
    }
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_call_status);
    unsigned v = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&v, static_cast<unsigned*>(p) + (id % kStatusRing), sizeof(v), cudaMemcpyDeviceToHost,
                            stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        *err = std::string("reading the call status: ") + cudaGetErrorString(e);
        return EITHOT_STATUS_CUDA;
    }
    if (g_next_call.load() - id > kStatusRing) {  // reused while we read it
        *err = "the call's status word has been reused by a later call";
        return EITHOT_STATUS_INVALID;
    }
    *bits = v;
    return 0;
}


}  // namespace eithot
