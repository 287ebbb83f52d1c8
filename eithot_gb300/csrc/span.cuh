// Staging of byte ranges at any alignment into word-aligned shared memory,
// shared by the narrow-element kernels (1- and 2-byte units).
#pragma once

#include <cstdint>

namespace eithot {

// One staging unit: destination words 4t .. 4t+3 of a copy of the L bytes at
// `src` (any alignment) to `dst` (4-byte aligned).  Each destination word is
// the funnel shift of the two aligned source words it spans, by the source's
// misalignment.  Only source words holding a byte of the range are read (a
// word never crosses a page); destination words start below L, and the bytes
// of the last one past L (up to L rounded up to 4) take don't-care values, so
// the destination must own them (padding of a staged row or piece).
struct SpanUnit {
    uint8_t* dst;
    const uint8_t* src;
    uint32_t L, t;
    bool ok;  // false: no unit (past the end of the loop)
};

__device__ __forceinline__ void span_load(const SpanUnit& u, uint32_t (&v)[5]) {
    const uintptr_t s = reinterpret_cast<uintptr_t>(u.src);
    const uint32_t h = static_cast<uint32_t>(s & 3u);
    const uint32_t* w = reinterpret_cast<const uint32_t*>(s - h);
    const uint32_t nw = u.ok ? (h + u.L + 3) / 4 : 0;  // source words holding range bytes
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const uint32_t i = 4 * u.t + k;
        v[k] = i < nw ? w[i] : 0u;
    }
}

__device__ __forceinline__ void span_store(const SpanUnit& u, const uint32_t (&v)[5]) {
    if (!u.ok) return;
    const uint32_t h = static_cast<uint32_t>(reinterpret_cast<uintptr_t>(u.src) & 3u);
    const uint32_t nd = (u.L + 3) / 4;  // destination words
    uint32_t* d = reinterpret_cast<uint32_t*>(u.dst);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t m = 4 * u.t + k;
        if (m < nd) d[m] = __funnelshift_r(v[k], v[k + 1], 8 * h);
    }
}

// Runs `total` staging units, unit x described by unit_of(x), two per thread
// at a time with all their loads issued before either unit's stores (ten
// words in flight per thread).
template <typename UnitOf>
__device__ __forceinline__ void span_stage(uint32_t total, UnitOf unit_of) {
    for (uint32_t x0 = threadIdx.x; x0 < total; x0 += 2 * blockDim.x) {
        const uint32_t x1 = x0 + blockDim.x;
        SpanUnit u0 = unit_of(x0);
        SpanUnit u1 = x1 < total ? unit_of(x1) : SpanUnit{nullptr, nullptr, 0, 0, false};
        uint32_t v0[5], v1[5];
        span_load(u0, v0);
        span_load(u1, v1);
        span_store(u0, v0);
        span_store(u1, v1);
    }
}

}  // namespace eithot
