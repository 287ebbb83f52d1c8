// Device-side content generator and permutation check for tensors too large
// to verify against a host copy (a 100 GB tensor leaves no room for a second
// one).  Element i of a generated tensor holds the low bytes of
// mix64(seed ^ i * 0xD1B54A32D192ED03) (splitmix64's finaliser; byte k of a
// wider element is byte k mod 8 of that value).  After an in-place
// permutation, output element o must hold the value of the source element
// it came from; the check recomputes that source index from o's output
// coordinates alone, so it shares no code with the transpose kernels.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "exec.h"
#include "index_math.cuh"

namespace eithot {
namespace {

constexpr int kCheckThreads = 256;
constexpr int kMaxCheckRank = 16;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t hash_value(uint64_t seed, uint64_t index) {
    return mix64(seed ^ (index * 0xD1B54A32D192ED03ull));
}

template <typename U>
__global__ void k_fill_hash(U* data, uint64_t n, uint64_t seed, uint64_t first) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        data[i] = static_cast<U>(hash_value(seed, first + i));
}

__global__ void k_fill_hash_bytes(uint8_t* data, uint64_t n, uint32_t elem, uint64_t seed, uint64_t first) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t v = hash_value(seed, first + i);
        for (uint32_t k = 0; k < elem; ++k) data[i * elem + k] = static_cast<uint8_t>(v >> (8 * (k % 8)));
    }
}

struct CheckArgs {
    int rank;
    uint64_t n;
    FastDiv od[kMaxCheckRank];           // output dims, axis 0 fastest
    uint64_t src_stride[kMaxCheckRank];  // input stride of the input axis behind output axis j
};

__device__ unsigned long long g_check_bad;
__device__ unsigned long long g_check_first;

__device__ __forceinline__ uint64_t source_of(const CheckArgs& a, uint64_t o) {
    uint64_t s = 0;
    for (int j = 0; j < a.rank; ++j) {
        uint64_t q, c;
        a.od[j].divmod(o, q, c);
        s += c * a.src_stride[j];
        o = q;
    }
    return s;
}

template <typename U>
__global__ void k_check_hash(const U* data, CheckArgs a, uint64_t seed) {
    unsigned long long bad = 0, first = ~0ull;
    for (uint64_t o = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; o < a.n;
         o += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const U want = static_cast<U>(hash_value(seed, source_of(a, o)));
        if (data[o] != want) {
            ++bad;
            if (o < first) first = o;
        }
    }
    if (bad) {
        atomicAdd(&g_check_bad, bad);
        atomicMin(&g_check_first, first);
    }
}

__global__ void k_check_hash_bytes(const uint8_t* data, CheckArgs a, uint32_t elem, uint64_t seed) {
    unsigned long long bad = 0, first = ~0ull;
    for (uint64_t o = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; o < a.n;
         o += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t v = hash_value(seed, source_of(a, o));
        bool ok = true;
        for (uint32_t k = 0; k < elem; ++k) ok &= data[o * elem + k] == static_cast<uint8_t>(v >> (8 * (k % 8)));
        if (!ok) {
            ++bad;
            if (o < first) first = o;
        }
    }
    if (bad) {
        atomicAdd(&g_check_bad, bad);
        atomicMin(&g_check_first, first);
    }
}

int grid_of(uint64_t n) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t blocks = (n + kCheckThreads - 1) / kCheckThreads;
    const uint64_t cap = static_cast<uint64_t>(sms) * 8;
    return static_cast<int>(blocks < cap ? (blocks ? blocks : 1) : cap);
}

}  // namespace

int fill_hash(void* d, int64_t n, size_t elem, uint64_t seed, int64_t first, cudaStream_t s, std::string* err) {
    if (n <= 0) return 0;
    const uint64_t un = static_cast<uint64_t>(n), uf = static_cast<uint64_t>(first);
    const int grid = grid_of(un);
    const uintptr_t addr = reinterpret_cast<uintptr_t>(d);
    if (elem == 8 && addr % 8 == 0) k_fill_hash<uint64_t><<<grid, kCheckThreads, 0, s>>>(static_cast<uint64_t*>(d), un, seed, uf);
    else if (elem == 4 && addr % 4 == 0) k_fill_hash<uint32_t><<<grid, kCheckThreads, 0, s>>>(static_cast<uint32_t*>(d), un, seed, uf);
    else if (elem == 2 && addr % 2 == 0) k_fill_hash<uint16_t><<<grid, kCheckThreads, 0, s>>>(static_cast<uint16_t*>(d), un, seed, uf);
    else if (elem == 1) k_fill_hash<uint8_t><<<grid, kCheckThreads, 0, s>>>(static_cast<uint8_t*>(d), un, seed, uf);
    else k_fill_hash_bytes<<<grid, kCheckThreads, 0, s>>>(static_cast<uint8_t*>(d), un, static_cast<uint32_t>(elem), seed, uf);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { *err = std::string("fill kernel: ") + cudaGetErrorString(e); return EITHOT_STATUS_CUDA; }
    return 0;
}

int check_hash(const void* d, int rank, const int64_t* dims, const int* perm1, size_t elem, uint64_t seed,
               cudaStream_t s, uint64_t* mismatches, int64_t* first_bad, std::string* err) {
    if (rank < 1 || rank > kMaxCheckRank) { *err = "check: rank must be 1..16"; return EITHOT_STATUS_INVALID; }
    CheckArgs a;
    a.rank = rank;
    uint64_t istride[kMaxCheckRank];
    uint64_t n = 1;
    for (int i = 0; i < rank; ++i) {
        if (dims[i] < 1) { *err = "check: dims must be positive"; return EITHOT_STATUS_INVALID; }
        istride[i] = n;
        n *= static_cast<uint64_t>(dims[i]);
    }
    unsigned seen = 0;
    for (int j = 0; j < rank; ++j) {
        const int p = perm1[j] - 1;
        if (p < 0 || p >= rank || ((seen >> p) & 1u)) { *err = "check: invalid permutation"; return EITHOT_STATUS_INVALID; }
        seen |= 1u << p;
        a.od[j] = FastDiv::make(static_cast<uint64_t>(dims[p]), n);
        a.src_stride[j] = istride[p];
    }
    a.n = n;
    const unsigned long long init[2] = {0ull, ~0ull};
    cudaError_t e = cudaMemcpyToSymbolAsync(g_check_bad, &init[0], sizeof(init[0]), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(g_check_first, &init[1], sizeof(init[1]), 0, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) { *err = std::string("check: ") + cudaGetErrorString(e); return EITHOT_STATUS_CUDA; }
    const int grid = grid_of(n);
    const uintptr_t addr = reinterpret_cast<uintptr_t>(d);
    if (elem == 8 && addr % 8 == 0) k_check_hash<uint64_t><<<grid, kCheckThreads, 0, s>>>(static_cast<const uint64_t*>(d), a, seed);
    else if (elem == 4 && addr % 4 == 0) k_check_hash<uint32_t><<<grid, kCheckThreads, 0, s>>>(static_cast<const uint32_t*>(d), a, seed);
    else if (elem == 2 && addr % 2 == 0) k_check_hash<uint16_t><<<grid, kCheckThreads, 0, s>>>(static_cast<const uint16_t*>(d), a, seed);
    else if (elem == 1) k_check_hash<uint8_t><<<grid, kCheckThreads, 0, s>>>(static_cast<const uint8_t*>(d), a, seed);
    else k_check_hash_bytes<<<grid, kCheckThreads, 0, s>>>(static_cast<const uint8_t*>(d), a, static_cast<uint32_t>(elem), seed);
    e = cudaGetLastError();
    unsigned long long out[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyFromSymbolAsync(&out[0], g_check_bad, sizeof(out[0]), 0, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyFromSymbolAsync(&out[1], g_check_first, sizeof(out[1]), 0, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { *err = std::string("check: ") + cudaGetErrorString(e); return EITHOT_STATUS_CUDA; }
    *mismatches = out[0];
    *first_bad = out[0] ? static_cast<int64_t>(out[1]) : -1;
    return 0;
}

}  // namespace eithot
