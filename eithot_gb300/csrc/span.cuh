// Staging of byte ranges at any alignment into word-aligned shared memory,
// shared by the narrow-element kernels (1- and 2-byte units).
#pragma once

#include <cstdint>

namespace eithot {

// Destination words 4t .. 4t+3 of a copy of the L bytes at `src` (any
// alignment) to `dst` (4-byte aligned): each destination word is the funnel
// shift of the two aligned source words it spans, by the source's
// misalignment.  Only source words holding a byte of the range are read (a
// word never crosses a page); destination words start below L, and the bytes
// of the last one past L (up to L rounded up to 4) take don't-care values, so
// the destination must own them (padding of a staged row or piece).
__device__ __forceinline__ void span_chunk(uint8_t* dst, const uint8_t* src, uint32_t L, uint32_t t) {
    const uintptr_t s = reinterpret_cast<uintptr_t>(src);
    const uint32_t h = static_cast<uint32_t>(s & 3u);
    const uint32_t* w = reinterpret_cast<const uint32_t*>(s - h);
    const uint32_t nw = (h + L + 3) / 4;  // source words holding range bytes
    const uint32_t nd = (L + 3) / 4;      // destination words
    uint32_t v[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const uint32_t i = 4 * t + k;
        v[k] = i < nw ? w[i] : 0u;
    }
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t m = 4 * t + k;
        if (m < nd) d[m] = __funnelshift_r(v[k], v[k + 1], 8 * h);
    }
}

}  // namespace eithot
