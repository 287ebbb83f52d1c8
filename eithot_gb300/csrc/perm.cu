// sm_103a kernels of the pass-minimising planner's single-pass moves
// (search.cpp): the slab permutation (leading axes of every slab permuted on
// chip) and the block permutation (blocks of leading axes moved along the
// permutation's cycles).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "exec.h"
#include "index_math.cuh"
#include "passes.h"
#include "search.h"
#include "span.cuh"

namespace eithot {

namespace {

constexpr int kMaxAxes = 8;

template <int S> struct UnitT;
template <> struct UnitT<1> { using T = uint8_t; };
template <> struct UnitT<2> { using T = uint16_t; };
template <> struct UnitT<4> { using T = uint32_t; };
template <> struct UnitT<8> { using T = uint2; };
template <> struct UnitT<16> { using T = uint4; };

template <int US>
__device__ __forceinline__ void stage_unit(uint8_t* sdst, const uint8_t* gsrc) {
    using U = typename UnitT<US>::T;
    if constexpr (US >= 4) {
        const uint32_t sa = static_cast<uint32_t>(__cvta_generic_to_shared(sdst));
        if constexpr (US == 16)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gsrc) : "memory");
        else
            asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(gsrc), "n"(US) : "memory");
    } else {
        *reinterpret_cast<U*>(sdst) = *reinterpret_cast<const U*>(gsrc);
    }
}

// ---------------------------------------------------------------------------
// Slab permutation: B slabs of `count` elements (E bytes each; an element is
// moved in strips of w bytes when it is wider than 128 B), each staged whole
// in one CTA's shared memory and written back in the output order of its q
// axes.  Output element o (row-major in the output's axis order, fastest
// first) holds input element sum_j c_j(o) * istr[j], c_j(o) the coordinate of
// output axis j.  kPack > 1: whole 1- or 2-byte elements, kPack consecutive
// outputs packed into one 4-byte store.
// ---------------------------------------------------------------------------
struct SlabPermArgs {
    uint8_t* base;
    uint64_t items, slab_bytes;
    uint32_t count, E, w, upw, last_upw, nstrips, q;
    FastDiv div_strips;
    FastDiv32 div_upw;
    // 1- and 2-byte units: every element's piece (its strip, up to w bytes)
    // read in the aligned 16-byte chunks around it (`slots` per piece) and
    // written as the aligned 4-byte words inside it (`wslots` per piece)
    uint32_t words, slots, wslots;
    FastDiv32 div_slots, div_wslots;
    FastDiv32 od[kMaxAxes];   // output dims, output order
    uint32_t istr[kMaxAxes];  // input stride (elements) of output axis j
};

__device__ __forceinline__ uint32_t slab_src(const SlabPermArgs& a, uint32_t o) {
    uint32_t idx = 0;
#pragma unroll
    for (int j = 0; j < kMaxAxes; ++j) {
        if (j >= static_cast<int>(a.q)) break;
        uint32_t qt, c;
        a.od[j].divmod(o, qt, c);
        idx += c * a.istr[j];
        o = qt;
    }
    return idx;
}

// Places the bytes of an aligned 16-byte chunk whose first byte is byte b of
// a range of L bytes (b wraps below 0 for chunk bytes before the range) at
// dst[b + j], keeping only those inside the range.
__device__ __forceinline__ void place_chunk16(uint8_t* dst, const uint4& v, uint32_t b, uint32_t L) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const uint32_t bj = b + j;
        if (bj < L) dst[bj] = static_cast<uint8_t>(w[j >> 2] >> (8 * (j & 3)));
    }
}

// The word path of k_slab_perm (pieces of L bytes at any alignment; chunks
// and words never cross a page; bytes outside a piece are read and dropped,
// never written).
__device__ __forceinline__ void slab_perm_words(const SlabPermArgs& a, uint8_t* smem, uint8_t* slab, uint32_t L) {
    constexpr int kDepth = 4;  // chunk loads in flight per thread
    const uint32_t total = a.count * a.slots;
    for (uint32_t x0 = threadIdx.x; x0 < total; x0 += kDepth * blockDim.x) {
        uint4 v[kDepth];
        uint32_t e[kDepth], b[kDepth];
        bool ok[kDepth];
#pragma unroll
        for (int d = 0; d < kDepth; ++d) {
            const uint32_t x = x0 + d * blockDim.x;
            ok[d] = false;
            if (x >= total) continue;
            uint32_t k;
            a.div_slots.divmod(x, e[d], k);
            const uintptr_t lo = reinterpret_cast<uintptr_t>(slab + static_cast<uint64_t>(e[d]) * a.E);
            const uint32_t h = static_cast<uint32_t>(lo & 15u);
            if (16 * k >= h + L) continue;
            v[d] = *reinterpret_cast<const uint4*>(lo - h + 16 * k);
            b[d] = 16 * k - h;
            ok[d] = true;
        }
#pragma unroll
        for (int d = 0; d < kDepth; ++d)
            if (ok[d]) place_chunk16(smem + e[d] * a.w, v[d], b[d], L);
    }
    __syncthreads();
    const uint32_t wtotal = a.count * a.wslots;
    for (uint32_t x = threadIdx.x; x < wtotal; x += blockDim.x) {
        uint32_t o, k;
        a.div_wslots.divmod(x, o, k);
        const uintptr_t lo = reinterpret_cast<uintptr_t>(slab + static_cast<uint64_t>(o) * a.E);
        const uint32_t h = static_cast<uint32_t>(lo & 3u);
        if (4 * k >= h + L) continue;
        const uint8_t* src = smem + slab_src(a, o) * a.w;
        const uint32_t b0 = 4 * k - h;
        if (4 * k >= h && b0 + 4 <= L) {
            const uint32_t v = static_cast<uint32_t>(src[b0]) | static_cast<uint32_t>(src[b0 + 1]) << 8 |
                               static_cast<uint32_t>(src[b0 + 2]) << 16 | static_cast<uint32_t>(src[b0 + 3]) << 24;
            *reinterpret_cast<uint32_t*>(lo - h + 4 * k) = v;
        } else {
            uint8_t* dst = reinterpret_cast<uint8_t*>(lo - h + 4 * k);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t bj = b0 + j;
                if (bj < L) dst[j] = src[bj];
            }
        }
    }
}

template <int US, int kPack>
__global__ void __launch_bounds__(512) k_slab_perm(SlabPermArgs a) {
    using U = typename UnitT<US>::T;
    extern __shared__ __align__(16) uint8_t smem[];
    for (uint64_t it = blockIdx.x; it < a.items; it += gridDim.x) {
        uint64_t b, s;
        a.div_strips.divmod(it, b, s);
        const uint32_t lim = (s + 1 == a.nstrips) ? a.last_upw : a.upw;
        uint8_t* slab = a.base + b * a.slab_bytes + s * a.w;
        if constexpr (US < 4 && kPack == 1) {
            if (a.words) {
                slab_perm_words(a, smem, slab, lim * US);
                __syncthreads();
                continue;
            }
        }
        const uint32_t units = a.count * a.upw;
        if (a.w == a.E) {  // whole elements: the slab is contiguous
            for (uint32_t x = threadIdx.x; x < units; x += blockDim.x)
                stage_unit<US>(smem + x * US, slab + static_cast<uint64_t>(x) * US);
        } else {
            for (uint32_t x = threadIdx.x; x < units; x += blockDim.x) {
                uint32_t e, u;
                a.div_upw.divmod(x, e, u);
                if (u >= lim) continue;
                stage_unit<US>(smem + e * a.w + u * US, slab + static_cast<uint64_t>(e) * a.E + u * US);
            }
        }
        if constexpr (US >= 4) asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();
        if constexpr (kPack > 1) {
            const uint32_t groups = a.count / kPack;
            for (uint32_t g = threadIdx.x; g < groups; g += blockDim.x) {
                const uint32_t o0 = g * kPack;
                uint32_t word = 0;
#pragma unroll
                for (int k = 0; k < kPack; ++k)
                    word |= static_cast<uint32_t>(*reinterpret_cast<const U*>(smem + slab_src(a, o0 + k) * US))
                            << (8 * US * k);
                *reinterpret_cast<uint32_t*>(slab + static_cast<uint64_t>(o0) * US) = word;
            }
            for (uint32_t o = groups * kPack + threadIdx.x; o < a.count; o += blockDim.x)
                *reinterpret_cast<U*>(slab + static_cast<uint64_t>(o) * US) =
                    *reinterpret_cast<const U*>(smem + slab_src(a, o) * US);
        } else {
            for (uint32_t x = threadIdx.x; x < units; x += blockDim.x) {
                uint32_t o, u;
                a.div_upw.divmod(x, o, u);
                if (u >= lim) continue;
                const uint32_t src = slab_src(a, o);
                *reinterpret_cast<U*>(slab + static_cast<uint64_t>(o) * a.E + u * US) =
                    *reinterpret_cast<const U*>(smem + src * a.w + u * US);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Slab permutation of narrow whole elements (E <= 16 bytes): every thread
// writes runs of K = V / E consecutive outputs as one V-byte store.  The slab
// is staged row by row (a row = the input's fastest axis) at a padded pitch
// (an odd number of max(4, E)-byte granules) so that the strided gathers of
// a warp spread over the banks; a thread finds the first element of its run
// with one divide per axis and steps to the next ones by adding the axes'
// strides in shared memory, carrying from axis to axis.
// ---------------------------------------------------------------------------
struct SlabRunArgs {
    uint8_t* base;
    uint64_t batches, slab_bytes;
    uint32_t count, q, nrows, row_bytes, pitch, su;
    bool chunks16;            // slab base, slab size and row size are 16-byte multiples
    FastDiv32 div_upr;        // staging: unit index -> (row, unit of the row)
    FastDiv32 od[kMaxAxes];   // output dims, output order
    uint32_t odim[kMaxAxes];
    uint32_t step[kMaxAxes];  // shared-memory bytes per step of output axis j
    // Aligned runs: when the output dims below axis m multiply to a divisor
    // P of the run length K and K divides P * odim[m], every run starts at
    // coordinate 0 of the axes below m and never carries past axis m, so
    // the t-th output of every run lies delta[t] bytes after the run's
    // first element, whose address only axes m.. determine (through the
    // run index times K / P).
    uint32_t aligned, m_axis, nhi, rmul;
    // Otherwise, when the fastest output dim is at least K, a run wraps that
    // axis at most once (`wrap`): its elements are found by stepping axis 0
    // with one jump.
    uint32_t wrap;
    // Rows of 1- or 2-byte units (odd row lengths): the slab is read in
    // 4-byte words (every slab 4-byte aligned, its size a multiple of 4) and
    // their bytes placed into the padded rows.
    uint32_t stage_words;
    FastDiv32 div_rowb;       // slab byte -> (row, byte of the row)
    uint32_t kind;            // 100 * E + V (the queue kernel's dispatch)
    // 2D transposes of 1-byte elements (slab dims (C, R) written as (R, C)),
    // R a multiple of 4, slabs word-aligned: written as 4 x 4 byte tiles
    uint32_t tiles, tile_R, tile_w;
    FastDiv32 div_rt, div_tR;
    FastDiv32 hod[kMaxAxes];  // output dims m.., output order
    uint32_t hstep[kMaxAxes];
    uint32_t delta[16];
};

template <int E> struct ElemT;
template <> struct ElemT<1> { using T = uint8_t; };
template <> struct ElemT<2> { using T = uint16_t; };
template <> struct ElemT<4> { using T = uint32_t; };
template <> struct ElemT<8> { using T = uint2; };
template <> struct ElemT<16> { using T = uint4; };

__device__ __forceinline__ void stage_words(const SlabRunArgs& a, uint8_t* smem, const uint8_t* slab) {
    constexpr int kDepth = 4;  // word loads in flight per thread
    const uint32_t words = static_cast<uint32_t>(a.slab_bytes / 4);
    for (uint32_t x0 = threadIdx.x; x0 < words; x0 += kDepth * blockDim.x) {
        uint32_t w[kDepth];
#pragma unroll
        for (int j = 0; j < kDepth; ++j) {
            const uint32_t x = x0 + j * blockDim.x;
            w[j] = x < words ? reinterpret_cast<const uint32_t*>(slab)[x] : 0u;
        }
#pragma unroll
        for (int j = 0; j < kDepth; ++j) {
            const uint32_t x = x0 + j * blockDim.x;
            if (x >= words) break;
            const uint32_t v = w[j];
            uint32_t r, c;
            a.div_rowb.divmod(x * 4, r, c);
            if ((c & 3) == 0 && c + 4 <= a.row_bytes) {
                *reinterpret_cast<uint32_t*>(smem + r * a.pitch + c) = v;
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    smem[r * a.pitch + c] = static_cast<uint8_t>(v >> (8 * k));
                    if (++c == a.row_bytes) {
                        c = 0;
                        ++r;
                    }
                }
            }
        }
    }
}

template <int SU>
__device__ __forceinline__ void stage_rows(const SlabRunArgs& a, uint8_t* smem, const uint8_t* slab) {
    if constexpr (SU < 4) {
        if (a.stage_words) {
            stage_words(a, smem, slab);
            return;
        }
    }
    const uint32_t upr = a.row_bytes / SU;
    const uint32_t total = a.nrows * upr;
    for (uint32_t x = threadIdx.x; x < total; x += blockDim.x) {
        uint32_t r, u;
        a.div_upr.divmod(x, r, u);
        stage_unit<SU>(smem + r * a.pitch + u * SU, slab + static_cast<uint64_t>(r) * a.row_bytes + u * SU);
    }
    if constexpr (SU >= 4) asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

__device__ __forceinline__ uint32_t run_start(const SlabRunArgs& a, uint32_t o, uint32_t* c) {
    uint32_t addr = 0;
#pragma unroll
    for (int j = 0; j < kMaxAxes; ++j) {
        c[j] = 0;
        if (j < static_cast<int>(a.q)) {
            uint32_t qt;
            a.od[j].divmod(o, qt, c[j]);
            addr += c[j] * a.step[j];
            o = qt;
        }
    }
    return addr;
}

// Stores the K = V / E elements of one run as one V-byte store.
template <int E, int V>
__device__ __forceinline__ void store_run(uint8_t* dst, const typename ElemT<E>::T* v) {
    using T = typename ElemT<E>::T;
    constexpr int K = V / E;
    if constexpr (E >= 4) {
#pragma unroll
        for (int t = 0; t < K; ++t) reinterpret_cast<T*>(dst)[t] = v[t];
    } else {
        constexpr int W = V / 4;
        uint32_t w[W];
#pragma unroll
        for (int i = 0; i < W; ++i) w[i] = 0;
#pragma unroll
        for (int t = 0; t < K; ++t) w[t * E / 4] |= static_cast<uint32_t>(v[t]) << (8 * ((t * E) % 4));
        if constexpr (V == 16) *reinterpret_cast<uint4*>(dst) = make_uint4(w[0], w[1], w[2], w[3]);
        else if constexpr (V == 8) *reinterpret_cast<uint2*>(dst) = make_uint2(w[0], w[1]);
        else *reinterpret_cast<uint32_t*>(dst) = w[0];
    }
}

// Writes the staged slab back in output order: runs of K outputs per thread.
// Writes the transpose of a staged w x R block of 1-byte elements (row i of
// R rows at smem + i * pitch, column j at byte j; R a multiple of 4) as w
// output rows of R bytes at `out` (word-aligned): a thread loads the 4 x 4
// byte tile of rows i0..i0+3, columns j0..j0+3 as four words, transposes it
// with byte permutes and stores one word into each of output rows j0..j0+3
// (row groups fastest across threads); the last w % 4 columns byte by byte.
// div_rt divides by R / 4, div_R by R.
__device__ __forceinline__ void write_byte_tiles(const uint8_t* smem, uint32_t pitch, uint8_t* out, uint32_t w,
                                                 uint32_t R, const FastDiv32& div_rt, const FastDiv32& div_R) {
    const uint32_t w4 = w & ~3u, tiles = (w4 / 4) * (R / 4);
    for (uint32_t x = threadIdx.x; x < tiles; x += blockDim.x) {
        uint32_t jt, it;
        div_rt.divmod(x, jt, it);
        const uint32_t j0 = jt * 4, i0 = it * 4;
        const uint8_t* s0 = smem + i0 * pitch + j0;
        const uint32_t w0 = *reinterpret_cast<const uint32_t*>(s0);
        const uint32_t w1 = *reinterpret_cast<const uint32_t*>(s0 + pitch);
        const uint32_t w2 = *reinterpret_cast<const uint32_t*>(s0 + 2 * pitch);
        const uint32_t w3 = *reinterpret_cast<const uint32_t*>(s0 + 3 * pitch);
        const uint32_t t0 = __byte_perm(w0, w1, 0x5140), t1 = __byte_perm(w2, w3, 0x5140);
        const uint32_t t2 = __byte_perm(w0, w1, 0x7362), t3 = __byte_perm(w2, w3, 0x7362);
        uint8_t* o = out + j0 * R + i0;
        *reinterpret_cast<uint32_t*>(o) = __byte_perm(t0, t1, 0x5410);
        *reinterpret_cast<uint32_t*>(o + R) = __byte_perm(t0, t1, 0x7632);
        *reinterpret_cast<uint32_t*>(o + 2 * R) = __byte_perm(t2, t3, 0x5410);
        *reinterpret_cast<uint32_t*>(o + 3 * R) = __byte_perm(t2, t3, 0x7632);
    }
    const uint32_t rest = (w - w4) * R;
    for (uint32_t x = threadIdx.x; x < rest; x += blockDim.x) {
        uint32_t jj, i;
        div_R.divmod(x, jj, i);
        out[(w4 + jj) * R + i] = smem[i * pitch + w4 + jj];
    }
}

template <int E, int V>
__device__ __forceinline__ void write_runs(const SlabRunArgs& a, const uint8_t* sm, uint8_t* slab) {
    using T = typename ElemT<E>::T;
    constexpr int K = V / E;
    if constexpr (E == 1) {
        if (a.tiles) {
            write_byte_tiles(sm, a.pitch, slab, a.tile_w, a.tile_R, a.div_rt, a.div_tR);
            return;
        }
    }
    const uint32_t runs = a.count / K;
    if (a.aligned) {
        for (uint32_t g = threadIdx.x; g < runs; g += blockDim.x) {
            uint32_t x = g * a.rmul, addr = 0;
#pragma unroll
            for (int j = 0; j < kMaxAxes; ++j) {
                if (j < static_cast<int>(a.nhi)) {
                    uint32_t qt, c;
                    a.hod[j].divmod(x, qt, c);
                    addr += c * a.hstep[j];
                    x = qt;
                }
            }
            T v[K];
#pragma unroll
            for (int t = 0; t < K; ++t) v[t] = *reinterpret_cast<const T*>(sm + addr + a.delta[t]);
            store_run<E, V>(slab + static_cast<uint64_t>(g) * V, v);
        }
        return;
    }
    if (a.wrap) {
        // A run crosses at most one end of the fastest output axis: its
        // elements lie step[0] apart, with one jump (the carry into the
        // next axes, found once per run) after the first w of them.
        for (uint32_t g = threadIdx.x; g < runs; g += blockDim.x) {
            uint32_t c[kMaxAxes];
            const uint32_t addr = run_start(a, g * K, c);
            const uint32_t w = a.odim[0] - c[0];
            uint32_t jump = 0;
            if (w < K) {
                jump = 0u - a.odim[0] * a.step[0];
                bool carry = true;
#pragma unroll
                for (int j = 1; j < kMaxAxes; ++j) {
                    if (carry && j < static_cast<int>(a.q)) {
                        if (c[j] + 1 < a.odim[j]) {
                            jump += a.step[j];
                            carry = false;
                        } else {
                            jump -= (a.odim[j] - 1) * a.step[j];
                        }
                    }
                }
            }
            T v[K];
#pragma unroll
            for (int t = 0; t < K; ++t)
                v[t] = *reinterpret_cast<const T*>(sm + addr + t * a.step[0] + (static_cast<uint32_t>(t) >= w ? jump : 0u));
            store_run<E, V>(slab + static_cast<uint64_t>(g) * V, v);
        }
    } else {
    for (uint32_t g = threadIdx.x; g < runs; g += blockDim.x) {
        uint32_t c[kMaxAxes];
        uint32_t addr = run_start(a, g * K, c);
        T v[K];
#pragma unroll
        for (int t = 0; t < K; ++t) {
            v[t] = *reinterpret_cast<const T*>(sm + addr);
            if (t + 1 < K) {  // next output: axis 0 steps, carrying into the next axes
                bool carry = true;
#pragma unroll
                for (int j = 0; j < kMaxAxes; ++j) {
                    if (carry && j < static_cast<int>(a.q)) {
                        addr += a.step[j];
                        if (++c[j] == a.odim[j]) {
                            c[j] = 0;
                            addr -= a.odim[j] * a.step[j];
                        } else {
                            carry = false;
                        }
                    }
                }
            }
        }
        store_run<E, V>(slab + static_cast<uint64_t>(g) * V, v);
    }
    }
    for (uint32_t o = runs * K + threadIdx.x; o < a.count; o += blockDim.x) {
        uint32_t c[kMaxAxes];
        const uint32_t addr = run_start(a, o, c);
        *reinterpret_cast<T*>(slab + static_cast<uint64_t>(o) * E) = *reinterpret_cast<const T*>(sm + addr);
    }
}

template <int E, int V, int SU>
__global__ void __launch_bounds__(512) k_slab_runs(SlabRunArgs a) {
    extern __shared__ __align__(16) uint8_t smem[];
    for (uint64_t b = blockIdx.x; b < a.batches; b += gridDim.x) {
        uint8_t* slab = a.base + b * a.slab_bytes;
        stage_rows<SU>(a, smem, slab);
        __syncthreads();
        write_runs<E, V>(a, smem, slab);
        __syncthreads();
    }
}

// The same for slabs of up to kPfRegs * 16 * 512 bytes that leave room for
// one CTA per SM only: the next slab is loaded into registers (16-byte
// loads, kPfRegs per thread) while the current one is written back, so
// reads and writes overlap without a second shared-memory buffer.  Rows are
// whole 16-byte chunks (a chunk never straddles two rows).
constexpr int kPfRegs = 16;

template <int E, int V>
__global__ void __launch_bounds__(512, 1) k_slab_runs_pf(SlabRunArgs a) {
    extern __shared__ __align__(16) uint8_t smem[];
    const uint32_t chunks = static_cast<uint32_t>(a.slab_bytes / 16);
    uint4 v[kPfRegs];
    auto fetch = [&](uint64_t b) {
        const uint4* src = reinterpret_cast<const uint4*>(a.base + b * a.slab_bytes) + threadIdx.x;
#pragma unroll
        for (int k = 0; k < kPfRegs; ++k)
            if (threadIdx.x + k * 512u < chunks) v[k] = src[k * 512];
    };
    if (blockIdx.x < a.batches) fetch(blockIdx.x);
    for (uint64_t b = blockIdx.x; b < a.batches; b += gridDim.x) {
#pragma unroll
        for (int k = 0; k < kPfRegs; ++k) {
            const uint32_t ch = threadIdx.x + k * 512u;
            if (ch < chunks) {
                uint32_t r, cb;
                a.div_upr.divmod(ch, r, cb);  // div_upr counts 16-byte chunks per row here
                uint32_t* d = reinterpret_cast<uint32_t*>(smem + r * a.pitch + cb * 16);
                d[0] = v[k].x;
                d[1] = v[k].y;
                d[2] = v[k].z;
                d[3] = v[k].w;
            }
        }
        __syncthreads();  // the slab is in shared memory
        const uint64_t nxt = b + gridDim.x;
        if (nxt < a.batches) fetch(nxt);  // in flight during the write-back
        write_runs<E, V>(a, smem, a.base + b * a.slab_bytes);
        __syncthreads();  // shared memory is free for the next slab
    }
}

// ---------------------------------------------------------------------------
// The batched form's queue of whole-tensor slab permutations: one persistent
// launch whose CTAs take entries from a device counter (atomicAdd) until the
// queue is empty.  An entry is one small tensor permuted in a single slab (its
// run-kernel arguments, built on the host); entries are independent, so no
// CTA ever waits for another.  The entry's arguments are copied to shared
// memory first; staging and write-back dispatch on its unit and element.
// ---------------------------------------------------------------------------
template <int E, int V>
__device__ __forceinline__ void queue_write(const SlabRunArgs& a, const uint8_t* sm, uint8_t* slab) {
    write_runs<E, V>(a, sm, slab);
}

__global__ void __launch_bounds__(512) k_slab_queue(const SlabRunArgs* entries, uint32_t n, unsigned* next) {
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ __align__(16) SlabRunArgs s_a;
    __shared__ uint32_t s_k;
    constexpr uint32_t kWords = sizeof(SlabRunArgs) / 4;
    for (;;) {
        if (threadIdx.x == 0) s_k = atomicAdd(next, 1u);
        __syncthreads();
        const uint32_t k = s_k;
        if (k >= n) break;
        const uint32_t* src = reinterpret_cast<const uint32_t*>(entries + k);
        for (uint32_t x = threadIdx.x; x < kWords; x += blockDim.x) reinterpret_cast<uint32_t*>(&s_a)[x] = src[x];
        __syncthreads();
        const SlabRunArgs& a = s_a;
        uint8_t* slab = a.base;
        switch (a.su) {
            case 16: stage_rows<16>(a, smem, slab); break;
            case 8: stage_rows<8>(a, smem, slab); break;
            case 4: stage_rows<4>(a, smem, slab); break;
            case 2: stage_rows<2>(a, smem, slab); break;
            default: stage_rows<1>(a, smem, slab); break;
        }
        __syncthreads();
        switch (a.kind) {
            case 104: queue_write<1, 4>(a, smem, slab); break;
            case 108: queue_write<1, 8>(a, smem, slab); break;
            case 116: queue_write<1, 16>(a, smem, slab); break;
            case 204: queue_write<2, 4>(a, smem, slab); break;
            case 208: queue_write<2, 8>(a, smem, slab); break;
            case 216: queue_write<2, 16>(a, smem, slab); break;
            case 404: queue_write<4, 4>(a, smem, slab); break;
            case 408: queue_write<4, 8>(a, smem, slab); break;
            case 416: queue_write<4, 16>(a, smem, slab); break;
            case 808: queue_write<8, 8>(a, smem, slab); break;
            case 816: queue_write<8, 16>(a, smem, slab); break;
            default: queue_write<16, 16>(a, smem, slab); break;
        }
        __syncthreads();  // shared memory and s_k are free for the next entry
    }
}

static_assert(sizeof(SlabRunArgs) % 4 == 0, "queue entries are copied in words");

// ---------------------------------------------------------------------------
// Column-band cluster slab: B matrices of R x C elements with few rows, each
// transposed in one pass by a cluster of K CTAs.  CTA k stages the band of
// columns [k P, k P + w) of every row (R segments of w E bytes, from the
// aligned 4-byte words around them), the cluster synchronises (every CTA's
// loads of a matrix precede any CTA's writes to it), and CTA k writes output
// rows k P .. k P + w - 1: one contiguous range of w R elements, written in
// runs of V-byte stores from its own shared memory (the run kernel's
// write-back of a w x R slab).  The row-band form (k_slab_cluster) writes a
// band's Q = R / K elements into every output row instead: a few bytes each
// when R is small.
// ---------------------------------------------------------------------------
struct ColBandArgs {
    uint8_t* base;
    uint64_t items, mat_bytes, row_bytes;
    uint32_t R, C, E, P;
    // su = 4, 8 or 16: every row segment (and its padded row in shared
    // memory) starts on an su-byte boundary and is su-byte units long, staged
    // by cp.async; su = 0: segments at any alignment, staged 16 bytes per
    // thread from the aligned words they span.  wpr_* = staging units per row.
    uint32_t su;
    uint32_t wpr_full, wpr_last;
    FastDiv32 div_full, div_last;
    // any_align: some band's output range does not start on a store-width
    // boundary (an odd base or matrix size): written in aligned 4-byte words
    // gathered byte by byte (div_R: output element -> (output row, element))
    uint32_t any_align;
    FastDiv32 div_R;
    // tiles: 1-byte elements, R a multiple of 4, ranges word-aligned: 4 x 4
    // byte tiles transposed in registers (div_rt: tile index -> (column
    // group, row group), R / 4 row groups)
    uint32_t tiles;
    FastDiv32 div_rt;
    SlabRunArgs full, last;       // write-back of a band of P columns / of the last band
};

// Byte b of a band's output range: output element o = b / E of the w x R
// output block (output row j = o / R = column j of the band, element i = o % R
// = row i), read from the staged band.
template <int E>
__device__ __forceinline__ uint32_t colband_byte(const ColBandArgs& a, const uint8_t* smem, uint32_t pitch,
                                                 uint32_t b) {
    uint32_t j, i;
    a.div_R.divmod(b / E, j, i);
    return smem[i * pitch + j * E + b % E];
}

// Writes a band's output range of n bytes at any alignment: the aligned words
// inside it as whole words, the at most 3 bytes before and after one by one.
template <int E>
__device__ __forceinline__ void colband_write_any(const ColBandArgs& a, const uint8_t* smem, uint32_t pitch,
                                                  uint8_t* out, uint32_t n) {
    const uint32_t head = min(n, static_cast<uint32_t>((4 - (reinterpret_cast<uintptr_t>(out) & 3u)) & 3u));
    const uint32_t words = (n - head) / 4;
    for (uint32_t x = threadIdx.x; x < words; x += blockDim.x) {
        const uint32_t b = head + 4 * x;
        uint32_t j, i;  // the word's first byte: output row j, element i (input row i)
        a.div_R.divmod(b / E, j, i);
        uint32_t e = b % E;
        uint32_t v = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v |= static_cast<uint32_t>(smem[i * pitch + j * E + e]) << (8 * k);
            if (++e == E) {
                e = 0;
                if (++i == a.R) {
                    i = 0;
                    ++j;
                }
            }
        }
        *reinterpret_cast<uint32_t*>(out + b) = v;
    }
    const uint32_t rest = head + (n - head - words * 4);  // bytes outside whole words
    for (uint32_t x = threadIdx.x; x < rest; x += blockDim.x) {
        const uint32_t b = x < head ? x : head + words * 4 + (x - head);
        out[b] = static_cast<uint8_t>(colband_byte<E>(a, smem, pitch, b));
    }
}

// Stages the band's R row segments of wb bytes, each starting row_bytes after
// the previous one at `seg`, into rows of `pitch` bytes of shared memory.
__device__ __forceinline__ void colband_stage(const ColBandArgs& a, uint8_t* smem, const uint8_t* seg,
                                              uint32_t pitch, uint32_t wb, uint32_t wpr, const FastDiv32& dv) {
    const uint32_t total = a.R * wpr;
    if (a.su >= 4) {
        for (uint32_t x = threadIdx.x; x < total; x += blockDim.x) {
            uint32_t r, u;
            dv.divmod(x, r, u);
            uint8_t* sd = smem + r * pitch + u * a.su;
            const uint8_t* gs = seg + static_cast<uint64_t>(r) * a.row_bytes + u * a.su;
            if (a.su == 16)
                stage_unit<16>(sd, gs);
            else if (a.su == 8)
                stage_unit<8>(sd, gs);
            else
                stage_unit<4>(sd, gs);
        }
        asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
        return;
    }
    // each row segment 16 bytes per unit from the aligned words it spans
    span_stage(total, [&](uint32_t x) {
        uint32_t r, t;
        dv.divmod(x, r, t);
        return SpanUnit{smem + r * pitch, seg + static_cast<uint64_t>(r) * a.row_bytes, wb, t, true};
    });
}

template <int E, int V>
__global__ void __launch_bounds__(512) k_slab_colband(ColBandArgs a) {
    extern __shared__ __align__(16) uint8_t smem[];
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const unsigned K = cl.num_blocks(), kr = cl.block_rank();
    const uint64_t cid = blockIdx.x / K, ncl = gridDim.x / K;
    const uint32_t c0 = kr * a.P;
    const uint32_t w = c0 < a.C ? min(a.P, a.C - c0) : 0;
    const bool last = w != a.P;
    const SlabRunArgs& s = last ? a.last : a.full;
    const uint32_t wb = w * a.E;
    const uint32_t wpr = last ? a.wpr_last : a.wpr_full;
    const FastDiv32& dv = last ? a.div_last : a.div_full;
    for (uint64_t it = cid; it < a.items; it += ncl) {
        uint8_t* mat = a.base + it * a.mat_bytes;
        if (w > 0) colband_stage(a, smem, mat + static_cast<uint64_t>(c0) * a.E, s.pitch, wb, wpr, dv);
        __syncthreads();
        asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
        asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
        if (w > 0) {
            uint8_t* out = mat + static_cast<uint64_t>(c0) * a.R * a.E;
            if (a.any_align)
                colband_write_any<E>(a, smem, s.pitch, out, w * a.R * a.E);
            else if (E == 1 && a.tiles)
                write_byte_tiles(smem, s.pitch, out, w, a.R, a.div_rt, a.div_R);
            else
                write_runs<E, V>(s, smem, out);
        }
        __syncthreads();  // shared memory is free for the next matrix
    }
}

// ---------------------------------------------------------------------------
// Block permutation along cycles.  Blocks of `blk` bytes are indexed by q
// axes; the block at output index t comes from input index src(t).  The
// cycles are cut into segments (host table): a first launch copies the block
// at every segment's head to scratch; a second walks every segment backwards
// from its tail: position t <- block at src(t), then t = src(t), the last step
// taking the head's saved copy.  Every position is written once and read
// before it is written, by the same thread for the same bytes (each thread
// owns fixed byte lanes of every block), so no barrier is needed.  Segments
// are processed in chunks of whole cycles (a cycle's segments depend only on
// one another).
// ---------------------------------------------------------------------------
struct CycleArgs {
    uint8_t* base;
    uint8_t* saved;
    const uint64_t* head;
    const uint64_t* tail;
    const uint64_t* len;
    uint64_t seg0, nseg, blk, units;
    uint32_t q;
    FastDiv div_units;
    FastDiv od[kMaxAxes];     // output dims, output order
    uint64_t istr[kMaxAxes];  // input stride (blocks) of output axis j
};

__device__ __forceinline__ uint64_t cycle_src(const CycleArgs& a, uint64_t t) {
    uint64_t idx = 0;
#pragma unroll
    for (int j = 0; j < kMaxAxes; ++j) {
        if (j >= static_cast<int>(a.q)) break;
        uint64_t qt, c;
        a.od[j].divmod(t, qt, c);
        idx += c * a.istr[j];
        t = qt;
    }
    return idx;
}

template <int US>
__global__ void __launch_bounds__(512) k_cycle_save(CycleArgs a) {
    using U = typename UnitT<US>::T;
    const uint64_t total = a.nseg * a.units;
    for (uint64_t x = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; x < total;
         x += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        uint64_t i, u;
        a.div_units.divmod(x, i, u);
        *reinterpret_cast<U*>(a.saved + i * a.blk + u * US) =
            *reinterpret_cast<const U*>(a.base + a.head[a.seg0 + i] * a.blk + u * US);
    }
}

constexpr int kFollowThreads = 256;
constexpr int kFollowBatch = 4;  // units in flight per thread

template <int US>
__global__ void __launch_bounds__(kFollowThreads) k_cycle_follow(CycleArgs a) {
    using U = typename UnitT<US>::T;
    for (uint64_t sg = blockIdx.x; sg < a.nseg; sg += gridDim.x) {
        uint64_t t = a.tail[a.seg0 + sg];
        const uint64_t n = a.len[a.seg0 + sg];
        for (uint64_t step = 0; step < n; ++step) {
            const uint64_t p = cycle_src(a, t);
            const uint8_t* from = (step + 1 == n) ? a.saved + sg * a.blk : a.base + p * a.blk;
            uint8_t* to = a.base + t * a.blk;
            for (uint64_t x0 = threadIdx.x; x0 < a.units; x0 += kFollowBatch * kFollowThreads) {
                U v[kFollowBatch];
#pragma unroll
                for (int k = 0; k < kFollowBatch; ++k) {
                    const uint64_t x = x0 + k * kFollowThreads;
                    if (x < a.units) v[k] = *reinterpret_cast<const U*>(from + x * US);
                }
#pragma unroll
                for (int k = 0; k < kFollowBatch; ++k) {
                    const uint64_t x = x0 + k * kFollowThreads;
                    if (x < a.units) *reinterpret_cast<U*>(to + x * US) = v[k];
                }
            }
            t = p;
        }
    }
}

uint64_t pow2_unit(std::initializer_list<uint64_t> vals) {
    uint64_t u = 16;
    for (uint64_t v : vals)
        while (u > 1 && v % u != 0) u /= 2;
    return u;
}

#define PM_CHECK(expr)                                                    \
    do {                                                                  \
        cudaError_t e__ = (expr);                                         \
        if (e__ != cudaSuccess) {                                         \
            ctx.err = std::string(#expr) + ": " + cudaGetErrorString(e__); \
            return EITHOT_STATUS_CUDA;                                    \
        }                                                                 \
    } while (0)

int device_sms(const ExecContext& ctx) { return std::max(1, ctx.caps.sms); }

template <int US, int kPack>
int launch_slab_perm(const SlabPermArgs& a, size_t smem, ExecContext& ctx) {
    auto kern = k_slab_perm<US, kPack>;
    PM_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int per_sm = 0;
    PM_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 512, smem));
    const uint64_t cap = static_cast<uint64_t>(std::max(per_sm, 1)) * device_sms(ctx);
    const unsigned grid = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>(a.items, cap)));
    kern<<<grid, 512, smem, ctx.stream>>>(a);
    PM_CHECK(cudaGetLastError());
    ctx.launches++;
    return 0;
}

template <int US>
int launch_cycles(const CycleArgs& a, ExecContext& ctx) {
    const uint64_t total = a.nseg * a.units;
    const unsigned g1 = static_cast<unsigned>(std::max<uint64_t>(
        1, std::min<uint64_t>((total + 511) / 512, static_cast<uint64_t>(device_sms(ctx)) * 4)));
    k_cycle_save<US><<<g1, 512, 0, ctx.stream>>>(a);
    PM_CHECK(cudaGetLastError());
    const unsigned g2 = static_cast<unsigned>(
        std::max<uint64_t>(1, std::min<uint64_t>(a.nseg, static_cast<uint64_t>(device_sms(ctx)) * 8)));
    k_cycle_follow<US><<<g2, kFollowThreads, 0, ctx.stream>>>(a);
    PM_CHECK(cudaGetLastError());
    ctx.launches += 2;
    return 0;
}

// Output dims in output order and the input stride of each output axis.
void out_geometry(const Pass& p, std::vector<uint64_t>* od, std::vector<uint64_t>* istr) {
    const int q = static_cast<int>(p.nd_dims.size());
    std::vector<uint64_t> in_stride(q);
    uint64_t st = 1;
    for (int i = 0; i < q; ++i) {
        in_stride[i] = st;
        st *= p.nd_dims[i];
    }
    od->resize(q);
    istr->resize(q);
    for (int j = 0; j < q; ++j) {
        (*od)[j] = p.nd_dims[p.nd_perm[j]];
        (*istr)[j] = in_stride[p.nd_perm[j]];
    }
}

constexpr size_t kSlabTwoPerSmBytes = 110 * 1024;  // staged slabs above this leave one CTA per SM

uint64_t table_bytes(uint64_t nseg) { return (3 * nseg * sizeof(uint64_t) + 255) / 256 * 256; }

}  // namespace

namespace {

template <int E, int V, int SU>
int launch_slab_runs(const SlabRunArgs& a, size_t smem, ExecContext& ctx) {
    auto kern = k_slab_runs<E, V, SU>;
    PM_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int per_sm = 0;
    PM_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 512, smem));
    const uint64_t cap = static_cast<uint64_t>(std::max(per_sm, 1)) * device_sms(ctx);
    const unsigned grid = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>(a.batches, cap)));
    kern<<<grid, 512, smem, ctx.stream>>>(a);
    PM_CHECK(cudaGetLastError());
    ctx.launches++;
    return 0;
}

template <int E, int V>
int launch_slab_runs_pf(SlabRunArgs a, size_t smem, ExecContext& ctx) {
    auto kern = k_slab_runs_pf<E, V>;
    a.div_upr = FastDiv32::make(a.row_bytes / 16);
    PM_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    const unsigned grid = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>(a.batches, device_sms(ctx))));
    kern<<<grid, 512, smem, ctx.stream>>>(a);
    PM_CHECK(cudaGetLastError());
    ctx.launches++;
    return 0;
}

template <int E, int V>
int dispatch_su(const SlabRunArgs& a, size_t smem, ExecContext& ctx) {
    // one CTA per SM: prefetch the next slab into registers instead
    if (smem > kSlabTwoPerSmBytes && a.slab_bytes <= static_cast<uint64_t>(kPfRegs) * 16 * 512 && a.chunks16 &&
        tuning().slab_prefetch)
        return launch_slab_runs_pf<E, V>(a, smem, ctx);
    switch (a.su) {
        case 16: return launch_slab_runs<E, V, 16>(a, smem, ctx);
        case 8: return launch_slab_runs<E, V, 8>(a, smem, ctx);
        case 4: return launch_slab_runs<E, V, 4>(a, smem, ctx);
        case 2: return launch_slab_runs<E, V, 2>(a, smem, ctx);
        default: return launch_slab_runs<E, V, 1>(a, smem, ctx);
    }
}

template <int E>
int dispatch_v(const SlabRunArgs& a, size_t smem, uint64_t V, ExecContext& ctx) {
    if constexpr (E <= 4) {
        if (V == 16) return dispatch_su<E, 16>(a, smem, ctx);
        if (V == 8) return dispatch_su<E, 8>(a, smem, ctx);
        return dispatch_su<E, 4>(a, smem, ctx);
    } else if constexpr (E == 8) {
        if (V == 16) return dispatch_su<E, 16>(a, smem, ctx);
        return dispatch_su<E, 8>(a, smem, ctx);
    } else {
        return dispatch_su<E, 16>(a, smem, ctx);
    }
}

// Fills the aligned-run fields when runs of K outputs qualify (see
// SlabRunArgs); leaves `aligned` 0 otherwise.
void set_aligned_runs(SlabRunArgs* a, uint64_t K) {
    a->aligned = 0;
    if (K == 0 || K > 16 || a->count % K != 0) return;
    uint64_t P = 1;
    for (uint32_t m = 0; m < a->q; ++m) {
        const uint64_t P1 = P * a->odim[m];
        if (K % P == 0 && P1 % K == 0) {
            a->aligned = 1;
            a->m_axis = m;
            a->rmul = static_cast<uint32_t>(K / P);
            a->nhi = a->q - m;
            for (uint32_t j = m; j < a->q; ++j) {
                a->hod[j - m] = a->od[j];
                a->hstep[j - m] = a->step[j];
            }
            for (uint64_t t = 0; t < K; ++t) {
                uint64_t off = 0, r = t;
                for (uint32_t j = 0; j < m; ++j) {
                    off += (r % a->odim[j]) * a->step[j];
                    r /= a->odim[j];
                }
                off += r * a->step[m];  // r = t / P < K / P <= odim[m]
                a->delta[t] = static_cast<uint32_t>(off);
            }
            return;
        }
        P = P1;
        if (P > K) return;
    }
}

// The run kernel for whole elements of 1-16 bytes when its padded staging
// fits; returns -1 when it does not apply.
// Fills the run kernel's arguments for pass p (count elements per slab);
// false when the kernel does not apply.  *V: the store width.
bool make_slab_runs(uint8_t* data, const Pass& p, uint64_t count, const DeviceCaps& caps, SlabRunArgs* out,
                    size_t* smem_out, uint64_t* V_out, uint64_t V_force = 0) {
    const uint64_t E = p.elem;
    if (!(E == 1 || E == 2 || E == 4 || E == 8 || E == 16) || (p.strip && p.strip != E)) return false;
    const int q = static_cast<int>(p.nd_dims.size());
    const uint64_t row_bytes = p.nd_dims[0] * E;
    const uint64_t g = std::max<uint64_t>(4, E);
    uint64_t pitch = (row_bytes + g - 1) / g * g;
    if ((pitch / g) % 2 == 0) pitch += g;
    const uint64_t nrows = count / p.nd_dims[0];
    const size_t smem = nrows * pitch;
    if (smem > smem_cap_of(caps)) return false;
    uint8_t* base = data + p.offset;
    const uint64_t addr = reinterpret_cast<uintptr_t>(base);
    const uint64_t slab_bytes = count * E;
    // V_force: the caller has checked that the slab's start is V_force-aligned
    // (runs of whole stores, the remainder written element by element)
    const uint64_t V = V_force ? V_force : pow2_unit({addr, slab_bytes});
    if (V < std::max<uint64_t>(4, E)) return false;  // stores of at least a word (and a whole element)
    SlabRunArgs& a = *out;
    std::memset(&a, 0, sizeof(a));
    a.base = base;
    a.batches = p.batches;
    a.slab_bytes = slab_bytes;
    a.count = static_cast<uint32_t>(count);
    a.q = static_cast<uint32_t>(q);
    a.nrows = static_cast<uint32_t>(nrows);
    a.row_bytes = static_cast<uint32_t>(row_bytes);
    a.pitch = static_cast<uint32_t>(pitch);
    a.su = static_cast<uint32_t>(pow2_unit({addr, row_bytes, pitch, slab_bytes}));
    a.chunks16 = pow2_unit({addr, row_bytes, slab_bytes}) == 16;
    a.div_upr = FastDiv32::make(row_bytes / a.su);
    a.div_rowb = FastDiv32::make(row_bytes);
    a.stage_words = a.su < 4 && addr % 4 == 0 && slab_bytes % 4 == 0 && tuning().narrow_words;
    // input strides: axis 0 moves E bytes inside a row, axis i >= 1 moves
    // rows (prod of dims 1..i-1 of them) of `pitch` bytes
    std::vector<uint64_t> istep(q);
    istep[0] = E;
    uint64_t rows = 1;
    for (int i = 1; i < q; ++i) {
        istep[i] = rows * pitch;
        rows *= p.nd_dims[i];
    }
    for (int j = 0; j < q; ++j) {
        const uint64_t d = p.nd_dims[p.nd_perm[j]];
        a.od[j] = FastDiv32::make(d);
        a.odim[j] = static_cast<uint32_t>(d);
        a.step[j] = static_cast<uint32_t>(istep[p.nd_perm[j]]);
    }
    if (tuning().slab_runs == 1) {
        set_aligned_runs(&a, V / E);
        a.wrap = !a.aligned && a.odim[0] >= V / E;
    }
    // V >= 4: every slab starts on a word and is whole words long
    a.tiles = E == 1 && q == 2 && p.nd_perm[0] == 1 && p.nd_dims[1] % 4 == 0 && V >= 4 && V_force == 0 &&
              tuning().narrow_words;
    a.tile_R = static_cast<uint32_t>(q == 2 ? p.nd_dims[1] : 1);
    a.tile_w = static_cast<uint32_t>(p.nd_dims[0]);
    a.div_rt = FastDiv32::make(std::max<uint32_t>(1, a.tile_R / 4));
    a.div_tR = FastDiv32::make(a.tile_R);
    a.kind = static_cast<uint32_t>(E * 100 + V);
    *smem_out = smem;
    *V_out = V;
    return true;
}

int try_slab_runs(uint8_t* data, const Pass& p, uint64_t count, ExecContext& ctx) {
    SlabRunArgs a;
    size_t smem = 0;
    uint64_t V = 0;
    if (!make_slab_runs(data, p, count, ctx.caps, &a, &smem, &V)) return -1;
    switch (p.elem) {
        case 1: return dispatch_v<1>(a, smem, V, ctx);
        case 2: return dispatch_v<2>(a, smem, V, ctx);
        case 4: return dispatch_v<4>(a, smem, V, ctx);
        case 8: return dispatch_v<8>(a, smem, V, ctx);
        default: return dispatch_v<16>(a, smem, V, ctx);
    }
}

}  // namespace

namespace {

template <int E, int V>
int launch_colband(const ColBandArgs& a, int K, size_t smem, ExecContext& ctx) {
    auto kern = k_slab_colband<E, V>;
    PM_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    if (K > 8) PM_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = K;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(512);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx.stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(static_cast<unsigned>(K * 1024));
    int max_clusters = 0;
    PM_CHECK(cudaOccupancyMaxActiveClusters(&max_clusters, kern, &cfg));
    if (max_clusters < 1) {
        ctx.err = "column-band cluster slab: no cluster fits";
        return EITHOT_STATUS_CUDA;
    }
    cfg.gridDim = dim3(static_cast<unsigned>(std::min<uint64_t>(a.items, static_cast<uint64_t>(max_clusters)) * K));
    PM_CHECK(cudaLaunchKernelEx(&cfg, kern, a));
    ctx.launches++;
    return 0;
}

template <int E>
int colband_v(const ColBandArgs& a, int K, size_t smem, uint64_t V, ExecContext& ctx) {
    if constexpr (E <= 4) {
        if (V == 16) return launch_colband<E, 16>(a, K, smem, ctx);
        if (V == 8) return launch_colband<E, 8>(a, K, smem, ctx);
        return launch_colband<E, 4>(a, K, smem, ctx);
    } else if constexpr (E == 8) {
        if (V == 16) return launch_colband<E, 16>(a, K, smem, ctx);
        return launch_colband<E, 8>(a, K, smem, ctx);
    } else {
        return launch_colband<E, 16>(a, K, smem, ctx);
    }
}

}  // namespace

// The write-back arguments of a band of w columns of a matrix with R rows
// whose output range starts at `out` (false when the run kernel does not
// apply, e.g. stores narrower than a word).
static bool colband_runs(uint8_t* out, uint64_t w, uint64_t R, uint64_t E, uint64_t V, const DeviceCaps& caps,
                         SlabRunArgs* a, size_t* smem) {
    Pass q;
    q.type = kSlabPerm;
    q.batches = 1;
    q.elem = E;
    q.strip = E;
    q.nd_dims = {w, R};
    q.nd_perm = {1, 0};
    uint64_t Vo = 0;
    return make_slab_runs(out, q, w * R, caps, a, smem, &Vo, V);
}

int run_slab_colband(uint8_t* data, const Pass& p, ExecContext& ctx) {
    ColBandArgs a;
    std::memset(&a, 0, sizeof(a));
    a.base = data + p.offset;
    a.items = p.batches;
    a.R = static_cast<uint32_t>(p.rows);
    a.C = static_cast<uint32_t>(p.cols);
    a.E = static_cast<uint32_t>(p.elem);
    a.P = static_cast<uint32_t>(p.band);
    a.row_bytes = p.cols * p.elem;
    a.mat_bytes = p.rows * a.row_bytes;
    const int K = static_cast<int>((p.cols + p.band - 1) / p.band);
    if (K < 2 || K > 16) return -1;
    const uint64_t wl = p.cols - static_cast<uint64_t>(K - 1) * p.band;  // the last band's columns
    size_t smem_f = 0, smem_l = 0;
    // one store width for every band of every matrix: band k's output starts
    // k P R E bytes into its matrix, matrix b b mat_bytes into the tensor
    uint64_t Vf = pow2_unit({reinterpret_cast<uintptr_t>(a.base), static_cast<uint64_t>(a.P) * a.R * a.E,
                             a.items > 1 ? a.mat_bytes : 0});
    const uint64_t Vmin = std::max<uint64_t>(4, a.E);
    auto runs = [&](uint64_t V) {
        return colband_runs(a.base, a.P, a.R, a.E, V, ctx.caps, &a.full, &smem_f) &&
               colband_runs(a.base, wl, a.R, a.E, V, ctx.caps, &a.last, &smem_l);
    };
    // The store width: elements of 4-16 bytes take the widest (runs of at
    // most 4 elements: table offsets, one jump or a short carry chain).  1-
    // and 2-byte elements take the widest whose runs have table offsets, else
    // the widest whose runs wrap the output row once; runs that would walk a
    // carry chain of 8-16 elements (odd or short output rows) and ranges off
    // the store width take the any-alignment write instead.
    if (Vf < Vmin) {
        a.any_align = 1;
        Vf = Vmin;
    } else if (a.E < 4) {
        uint64_t pick = 0;
        for (uint64_t V = Vf; V >= Vmin && !pick; V /= 2)
            if (runs(V) && a.full.aligned && a.last.aligned) pick = V;
        if (!pick && runs(Vf) && a.full.wrap && a.last.wrap) pick = Vf;
        if (pick)
            Vf = pick;
        else
            a.any_align = 1;
    }
    a.div_R = FastDiv32::make(a.R);
    a.tiles = a.E == 1 && a.R % 4 == 0 && !a.any_align && tuning().narrow_words;
    a.div_rt = FastDiv32::make(std::max<uint32_t>(1, a.R / 4));
    if (!runs(Vf)) return -1;
    const uint64_t su = pow2_unit({reinterpret_cast<uintptr_t>(a.base), a.row_bytes, static_cast<uint64_t>(a.P) * a.E,
                                   wl * a.E, a.full.pitch, a.last.pitch, a.items > 1 ? a.mat_bytes : 0});
    a.su = su >= 4 ? static_cast<uint32_t>(su) : 0;
    if (a.su) {
        a.wpr_full = a.P * a.E / a.su;
        a.wpr_last = static_cast<uint32_t>(wl * a.E / a.su);
    } else {  // 16-byte staging units per row segment
        a.wpr_full = (a.P * a.E + 15) / 16;
        a.wpr_last = static_cast<uint32_t>((wl * a.E + 15) / 16);
    }
    a.div_full = FastDiv32::make(a.wpr_full);
    a.div_last = FastDiv32::make(a.wpr_last);
    const size_t smem = std::max(smem_f, smem_l);
    switch (p.elem) {
        case 1: return colband_v<1>(a, K, smem, Vf, ctx);
        case 2: return colband_v<2>(a, K, smem, Vf, ctx);
        case 4: return colband_v<4>(a, K, smem, Vf, ctx);
        case 8: return colband_v<8>(a, K, smem, Vf, ctx);
        default: return colband_v<16>(a, K, smem, Vf, ctx);
    }
}

size_t slab_queue_entry_bytes() { return sizeof(SlabRunArgs); }

bool slab_queue_entry(uint8_t* data, const Pass& p, const DeviceCaps& caps, void* entry, size_t* smem) {
    uint64_t count = 1;
    for (auto d : p.nd_dims) count *= d;
    if (p.batches != 1 || count >= (uint64_t(1) << 31) || tuning().slab_runs == 0) return false;
    SlabRunArgs a;
    uint64_t V = 0;
    if (!make_slab_runs(data, p, count, caps, &a, smem, &V)) return false;
    a.batches = 1;
    std::memcpy(entry, &a, sizeof(a));
    return true;
}

int launch_slab_queue(const void* d_entries, uint32_t n, unsigned* d_next, size_t smem, ExecContext& ctx) {
    if (n == 0) return 0;
    PM_CHECK(cudaMemsetAsync(d_next, 0, sizeof(unsigned), ctx.stream));
    PM_CHECK(cudaFuncSetAttribute(k_slab_queue, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int per_sm = 0;
    PM_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_slab_queue, 512, smem));
    const uint64_t cap = static_cast<uint64_t>(std::max(per_sm, 1)) * device_sms(ctx);
    const unsigned grid = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>(n, cap)));
    k_slab_queue<<<grid, 512, smem, ctx.stream>>>(static_cast<const SlabRunArgs*>(d_entries), n, d_next);
    PM_CHECK(cudaGetLastError());
    ctx.launches++;
    return 0;
}

int try_slab_runs_pass(uint8_t* data, const Pass& p, ExecContext& ctx) {
    uint64_t count = 1;
    for (auto d : p.nd_dims) count *= d;
    if (count >= (uint64_t(1) << 31) || !tuning().slab_runs) return -1;
    return try_slab_runs(data, p, count, ctx);
}

int run_slab_perm(uint8_t* data, const Pass& p, ExecContext& ctx) {
    const int q = static_cast<int>(p.nd_dims.size());
    if (q < 1 || q > kMaxAxes || static_cast<int>(p.nd_perm.size()) != q) {
        ctx.err = "internal: slab permutation of more than 8 axes";
        return EITHOT_STATUS_INVALID;
    }
    uint64_t count = 1;
    for (auto d : p.nd_dims) count *= d;
    if (count < (uint64_t(1) << 31) && tuning().slab_runs) {
        const int rc = try_slab_runs(data, p, count, ctx);
        if (rc >= 0) return rc;
    }
    const uint64_t w = p.strip ? p.strip : p.elem;
    const size_t smem = count * w;
    if (smem > smem_cap_of(ctx.caps) || count >= (uint64_t(1) << 31)) {
        ctx.err = "internal: slab permutation beyond one CTA's shared memory";
        return EITHOT_STATUS_INVALID;
    }
    SlabPermArgs a;
    std::memset(&a, 0, sizeof(a));
    a.base = data + p.offset;
    a.slab_bytes = count * p.elem;
    a.count = static_cast<uint32_t>(count);
    a.E = static_cast<uint32_t>(p.elem);
    a.w = static_cast<uint32_t>(w);
    a.nstrips = static_cast<uint32_t>((p.elem + w - 1) / w);
    a.items = p.batches * a.nstrips;
    a.q = static_cast<uint32_t>(q);
    a.div_strips = FastDiv::make(a.nstrips, a.items);
    std::vector<uint64_t> od, istr;
    out_geometry(p, &od, &istr);
    for (int j = 0; j < q; ++j) {
        a.od[j] = FastDiv32::make(od[j]);
        a.istr[j] = static_cast<uint32_t>(istr[j]);
    }
    const uint64_t addr = reinterpret_cast<uintptr_t>(a.base);
    const uint64_t last = p.elem - (a.nstrips - 1) * w;
    const uint64_t US = pow2_unit({addr, p.elem, w, last, a.slab_bytes});
    a.upw = static_cast<uint32_t>(w / US);
    a.last_upw = static_cast<uint32_t>(last / US);
    a.div_upw = FastDiv32::make(a.upw);
    const bool whole = a.nstrips == 1;
    // pieces of 8 bytes or more in chunks and words (shorter ones gain little)
    a.words = US < 4 && w >= 8 && tuning().narrow_words;
    a.slots = static_cast<uint32_t>((w + 15) / 16 + 1);
    a.div_slots = FastDiv32::make(a.slots);
    a.wslots = static_cast<uint32_t>((w + 3) / 4 + 1);
    a.div_wslots = FastDiv32::make(a.wslots);
    switch (US) {
        case 16: return launch_slab_perm<16, 1>(a, smem, ctx);
        case 8: return launch_slab_perm<8, 1>(a, smem, ctx);
        case 4: return launch_slab_perm<4, 1>(a, smem, ctx);
        case 2:
            if (whole && p.elem == 2 && addr % 4 == 0 && a.slab_bytes % 4 == 0) return launch_slab_perm<2, 2>(a, smem, ctx);
            return launch_slab_perm<2, 1>(a, smem, ctx);
        default:
            if (whole && p.elem == 1 && addr % 4 == 0 && a.slab_bytes % 4 == 0) return launch_slab_perm<1, 4>(a, smem, ctx);
            return launch_slab_perm<1, 1>(a, smem, ctx);
    }
}

size_t block_perm_workspace(const Pass& p, bool ideal) {
    const CycleTable& tab = cycle_table(p.nd_dims, p.nd_perm);
    const uint64_t nseg = tab.head.size();
    if (nseg == 0) return 0;
    return table_bytes(nseg) + (ideal ? nseg : tab.max_cycle_segments) * p.block;
}

int run_block_perm(uint8_t* data, const Pass& p, ExecContext& ctx) {
    const int q = static_cast<int>(p.nd_dims.size());
    if (q < 1 || q > kMaxAxes || static_cast<int>(p.nd_perm.size()) != q) {
        ctx.err = "internal: block permutation of more than 8 axes";
        return EITHOT_STATUS_INVALID;
    }
    const CycleTable& tab = cycle_table(p.nd_dims, p.nd_perm);
    const uint64_t nseg = tab.head.size();
    if (nseg == 0) return 0;  // every block stays
    const uint64_t tb = table_bytes(nseg);
    if (ctx.scratch == nullptr || ctx.scratch_bytes < tb + tab.max_cycle_segments * p.block) {
        ctx.err = "workspace too small for the block permutation's segment table and saved blocks";
        return EITHOT_STATUS_NOMEM;
    }
    uint64_t* dev_tab = reinterpret_cast<uint64_t*>(ctx.scratch);
    PM_CHECK(cudaMemcpyAsync(dev_tab, tab.head.data(), nseg * sizeof(uint64_t), cudaMemcpyHostToDevice, ctx.stream));
    PM_CHECK(cudaMemcpyAsync(dev_tab + nseg, tab.tail.data(), nseg * sizeof(uint64_t), cudaMemcpyHostToDevice,
                             ctx.stream));
    PM_CHECK(cudaMemcpyAsync(dev_tab + 2 * nseg, tab.len.data(), nseg * sizeof(uint64_t), cudaMemcpyHostToDevice,
                             ctx.stream));
    CycleArgs a;
    std::memset(&a, 0, sizeof(a));
    a.base = data + p.offset;
    a.saved = ctx.scratch + tb;
    a.head = dev_tab;
    a.tail = dev_tab + nseg;
    a.len = dev_tab + 2 * nseg;
    a.blk = p.block;
    a.q = static_cast<uint32_t>(q);
    std::vector<uint64_t> od, istr;
    out_geometry(p, &od, &istr);
    uint64_t nblocks = 1;
    for (auto d : p.nd_dims) nblocks *= d;
    for (int j = 0; j < q; ++j) {
        a.od[j] = FastDiv::make(od[j], nblocks);
        a.istr[j] = istr[j];
    }
    const uint64_t US = pow2_unit({reinterpret_cast<uintptr_t>(a.base), reinterpret_cast<uintptr_t>(a.saved), p.block});
    a.units = p.block / US;
    const uint64_t cap_seg = (ctx.scratch_bytes - tb) / p.block;  // saved blocks per chunk
    // chunks of whole cycles
    size_t c = 0;
    const size_t ncyc = tab.cycle_first.size() - 1;
    while (c < ncyc) {
        const uint64_t s0 = tab.cycle_first[c];
        size_t c1 = c + 1;
        while (c1 < ncyc && tab.cycle_first[c1 + 1] - s0 <= cap_seg) ++c1;
        a.seg0 = s0;
        a.nseg = tab.cycle_first[c1] - s0;
        a.div_units = FastDiv::make(a.units, a.nseg * a.units);
        int rc = 0;
        switch (US) {
            case 16: rc = launch_cycles<16>(a, ctx); break;
            case 8: rc = launch_cycles<8>(a, ctx); break;
            case 4: rc = launch_cycles<4>(a, ctx); break;
            case 2: rc = launch_cycles<2>(a, ctx); break;
            default: rc = launch_cycles<1>(a, ctx); break;
        }
        if (rc) return rc;
        c = c1;
    }
    return 0;
}

}  // namespace eithot
