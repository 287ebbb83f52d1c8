// sm_103a data-movement kernels of the in-place passes, and the executor
// that launches them for a list of passes (see passes.h).
//
// Each kernel moves "units" of U bytes (U in {1,2,4,8,16}, chosen from the
// alignment of every address the pass touches); an element of E bytes is
// split into strips of w bytes (whole elements up to 128 B) and a strip into
// w/U units.  Row and column passes stage one item (a row strip, or a
// column-tile strip over all rows) in shared memory, synchronise the block
// and write the permuted item back; when an item does not fit on chip it is
// staged in global scratch by a grid-wide copy-in launch followed by a
// copy-out launch, one group of items at a time (stream order replaces any
// device-wide barrier).
//
// The file is compiled once per unit size U (-DEITHOT_UNIT=U: the kernels
// and launchers of passes that move U-byte units, run_pass_unit_U) and once
// without it (the host-side executor, which picks the unit of each pass and
// calls into the matching object).  Each compilation is a device module of
// its own, so a process only loads the device code of the unit sizes its
// passes use (a module is loaded on its first use; loading all of this file's
// kernels at once took about 8 ms on GB300, one unit's share 1.5-2 ms).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include "exec.h"
#include "fn_build.h"
#include "index_math.cuh"
#include "passes.h"
#include "span.cuh"

namespace eithot {

namespace {

constexpr int kThreads = 512;
// Word loads a thread issues before placing their bytes (loops that stage
// narrow units from aligned words): one load in flight per thread leaves
// 2 KB in flight per CTA, far from what HBM needs.
constexpr int kWordDepth = 4;

// Places the bytes of an aligned 16-byte chunk whose first byte is byte b of
// a range of L bytes (b wraps below 0 for chunk bytes before the range) at
// dst[b + j], keeping only those inside the range.
__device__ __forceinline__ void place_chunk(uint8_t* dst, const uint4& v, uint32_t b, uint32_t L) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const uint32_t bj = b + j;
        if (bj < L) dst[bj] = static_cast<uint8_t>(w[j >> 2] >> (8 * (j & 3)));
    }
}

// Set when an index map returns a position outside its row or column; the
// access is skipped instead of faulting.  Read (and cleared) by
// eithot_index_faults().
__device__ unsigned int g_index_faults = 0;

// Per-call device status words live in status.cu (a small module of their
// own); kernels get their call's word as an argument and OR
// kCallIndexFault / kCallSyncTimeout into it.

__device__ __forceinline__ void raise_status(unsigned* status, unsigned bit) {
    if (status) atomicOr(status, bit);
}

__device__ __forceinline__ bool in_range(uint64_t v, uint64_t n, unsigned* status) {
    if (v < n) return true;
    atomicAdd(&g_index_faults, 1u);
    raise_status(status, kCallIndexFault);
    return false;
}

namespace cg = cooperative_groups;

// Global -> shared copy of one unit.  4/8/16-byte units use cp.async so a
// thread keeps many loads in flight; 1/2-byte units go through registers.
template <int US, typename U>
__device__ __forceinline__ void copy_in(uint8_t* sdst, const uint8_t* gsrc) {
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

template <int US>
__device__ __forceinline__ void copy_in_wait() {
    if constexpr (US >= 4) asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

template <int S> struct UnitOf;
template <> struct UnitOf<1> { using T = uint8_t; };
template <> struct UnitOf<2> { using T = uint16_t; };
template <> struct UnitOf<4> { using T = uint32_t; };
template <> struct UnitOf<8> { using T = uint2; };
template <> struct UnitOf<16> { using T = uint4; };

// Strip geometry shared by the kernels: `upw` units per full strip; the
// last strip of an element holds `last_upw` units.
struct StripGeom {
    uint64_t E, w, nstrips, upw, last_upw;
    FastDiv div_upw, div_strips;
};

// Cluster barriers.  The middle barrier of an item publishes the staged
// shared-memory data (release/acquire); the end-of-item barrier only has to
// keep a CTA from restaging before its peers finished reading it, and every
// such read has returned its value before the reader arrives, so it is
// relaxed and does not wait for the item's global stores to drain.
__device__ __forceinline__ void cluster_sync_publish() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_sync_reuse() {
    asm volatile("barrier.cluster.arrive.relaxed.aligned;\n" ::: "memory");
    asm volatile("barrier.cluster.wait.aligned;\n" ::: "memory");
}

// Generic addresses of every peer CTA's dynamic shared memory (K <= 16).
__device__ __forceinline__ void load_peers(uint8_t** peers, uint8_t* smem, unsigned K) {
    cg::cluster_group cl = cg::this_cluster();
    if (threadIdx.x < K) peers[threadIdx.x] = static_cast<uint8_t*>(cl.map_shared_rank(static_cast<void*>(smem), threadIdx.x));
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Slab transpose: B matrices of R x C elements, one strip of one matrix per
// work item, staged with a padded pitch so the transposed reads are
// conflict-free.  All intra-item indices are 32-bit (an item is at most the
// 227 KB of one CTA's shared memory).
// ---------------------------------------------------------------------------
struct SlabArgs {
    uint8_t* base;
    uint64_t items, E, mat_bytes;
    uint32_t R, C, pitch, w, upw, last_upw, rowunits;  // rowunits = C*upw (flat loads)
    bool flat;                                          // whole elements: rows contiguous
    FastDiv div_strips;
    FastDiv32 div_C, div_R, div_upw, div_rowunits;
    uint32_t nstrips;
    // pieces (an element's strip: up to w bytes at any alignment) staged 16
    // bytes per thread from the aligned words they span (`slots` per piece)
    // and written as the aligned 4-byte words inside them (`wslots` per piece)
    bool words;
    uint32_t slots, wslots;
    FastDiv32 div_slots, div_wslots;
    // whole narrow elements (sizes not a multiple of 4, up to 16 bytes) at
    // any alignment: the contiguous matrix read in aligned 16-byte chunks,
    // the output written as aligned 4-byte words gathered byte by byte
    bool flat_words;
    FastDiv32 div_E, div_rowb;
    uint32_t rowchunks;  // 16-byte staging units per row (C*E bytes)
    FastDiv32 div_rowchunks;
};

// The flat word path of k_slab: matrix bytes [0, n) at `mat` (rows of C*E
// bytes staged at `pitch` from the aligned words they span); output byte b
// holds byte b % E of input element (r, c), (c, r) = divmod(b / E, R).
__device__ __forceinline__ void slab_flat_words(const SlabArgs& a, uint8_t* smem, uint8_t* mat) {
    const uint32_t n = static_cast<uint32_t>(a.mat_bytes);
    const uintptr_t lo = reinterpret_cast<uintptr_t>(mat);
    const uint32_t rowb = a.C * static_cast<uint32_t>(a.E);
    span_stage(a.R * a.rowchunks, [&](uint32_t x) {  // rows staged 16 bytes per unit
        uint32_t r, t;
        a.div_rowchunks.divmod(x, r, t);
        return SpanUnit{smem + r * a.pitch, mat + static_cast<uint64_t>(r) * rowb, rowb, t, true};
    });
    __syncthreads();
    auto byte_of = [&](uint32_t b) -> uint32_t {
        uint32_t o, e, c, r;
        a.div_E.divmod(b, o, e);
        a.div_R.divmod(o, c, r);
        return smem[r * a.pitch + c * a.E + e];
    };
    const uint32_t hw = min(n, static_cast<uint32_t>((4 - (lo & 3u)) & 3u));
    const uint32_t words = (n - hw) / 4;
    for (uint32_t x = threadIdx.x; x < words; x += blockDim.x) {
        const uint32_t b = hw + 4 * x;
        uint32_t o, e, c, r;  // the word's first byte: byte e of output element o = c*R + r
        a.div_E.divmod(b, o, e);
        a.div_R.divmod(o, c, r);
        uint32_t v = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v |= static_cast<uint32_t>(smem[r * a.pitch + c * a.E + e]) << (8 * k);
            if (++e == a.E) {  // next output element: next input row, wrapping to the next column
                e = 0;
                if (++r == a.R) {
                    r = 0;
                    ++c;
                }
            }
        }
        *reinterpret_cast<uint32_t*>(mat + b) = v;
    }
    const uint32_t rest = n - words * 4;  // bytes outside whole words: hw before, the tail after
    for (uint32_t x = threadIdx.x; x < rest; x += blockDim.x) {
        const uint32_t b = x < hw ? x : hw + words * 4 + (x - hw);
        mat[b] = static_cast<uint8_t>(byte_of(b));
    }
}

// Slab of 1- or 2-byte units in pieces of L bytes (piece p of the input
// starts p*E bytes after `mat`, staged at (p / C)*pitch + (p % C)*w): every
// piece staged from the aligned words it spans (funnel shifts), transposed,
// and written as the aligned words
// inside each output piece, the at most 3 bytes at either end one by one
// (the words there hold other pieces' bytes).
__device__ __forceinline__ void slab_pieces_words(const SlabArgs& a, uint8_t* smem, uint8_t* mat, uint32_t L) {
    span_stage(a.R * a.C * a.slots, [&](uint32_t x) {
        uint32_t p, t, r, c;
        a.div_slots.divmod(x, p, t);
        a.div_C.divmod(p, r, c);
        return SpanUnit{smem + r * a.pitch + c * a.w, mat + static_cast<uint64_t>(p) * a.E, L, t, 16 * t < L};
    });
    __syncthreads();
    const uint32_t wtotal = a.R * a.C * a.wslots;
    for (uint32_t x = threadIdx.x; x < wtotal; x += blockDim.x) {
        uint32_t o, k, c, r;
        a.div_wslots.divmod(x, o, k);
        a.div_R.divmod(o, c, r);  // output o = c*R + r holds input (r, c)
        const uint8_t* src = smem + r * a.pitch + c * a.w;
        const uintptr_t lo = reinterpret_cast<uintptr_t>(mat + static_cast<uint64_t>(o) * a.E);
        const uint32_t h = static_cast<uint32_t>(lo & 3u);
        if (4 * k >= h + L) continue;
        const uint32_t b0 = 4 * k - h;
        if (4 * k >= h && b0 + 4 <= L) {
            // the piece's slot is word-aligned: the output word is the funnel
            // shift of the two slot words it spans (the second only when the
            // word is misaligned, so that it starts inside the piece)
            const uint32_t* sw = reinterpret_cast<const uint32_t*>(src);
            const uint32_t q = b0 >> 2, m = b0 & 3u;
            const uint32_t v = m ? __funnelshift_r(sw[q], sw[q + 1], 8 * m) : sw[q];
            *reinterpret_cast<uint32_t*>(lo - h + 4 * k) = v;
        } else {
            uint8_t* dst = reinterpret_cast<uint8_t*>(lo - h + 4 * k);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t b = b0 + j;
                if (b < L) dst[j] = src[b];
            }
        }
    }
}

template <int US, int kPack>
__global__ void __launch_bounds__(kThreads) k_slab(SlabArgs a) {
    using U = typename UnitOf<US>::T;
    extern __shared__ __align__(16) uint8_t smem[];
    const uint32_t units = a.R * a.C * a.upw;
    for (uint64_t it = blockIdx.x; it < a.items; it += gridDim.x) {
        uint64_t b, s;
        a.div_strips.divmod(it, b, s);
        const uint32_t lim = (s + 1 == a.nstrips) ? a.last_upw : a.upw;
        uint8_t* mat = a.base + b * a.mat_bytes + s * a.w;
        if constexpr (US < 4 && kPack == 1) {
            if (a.words) {
                slab_pieces_words(a, smem, mat, lim * US);
                __syncthreads();
                continue;
            }
            if (a.flat_words) {
                slab_flat_words(a, smem, mat);
                __syncthreads();
                continue;
            }
        }
        if (a.flat) {
            // the slab is R*C*E contiguous bytes: row r of the staging holds
            // bytes [r*C*E, (r+1)*C*E)
            for (uint32_t x = threadIdx.x; x < units; x += blockDim.x) {
                uint32_t r, rem;
                a.div_rowunits.divmod(x, r, rem);
                copy_in<US, U>(smem + r * a.pitch + rem * US, mat + static_cast<uint64_t>(x) * US);
            }
        } else {
            for (uint32_t x = threadIdx.x; x < units; x += blockDim.x) {
                uint32_t p, u, r, c;
                a.div_upw.divmod(x, p, u);
                if (u >= lim) continue;
                a.div_C.divmod(p, r, c);
                copy_in<US, U>(smem + r * a.pitch + c * a.w + u * US, mat + p * a.E + u * US);
            }
        }
        copy_in_wait<US>();
        __syncthreads();
        if constexpr (kPack > 1) {
            // whole 1/2-byte elements: kPack consecutive outputs (across
            // output rows) gathered into one 4-byte store, then the tail
            const uint32_t groups = units / kPack;
            for (uint32_t g = threadIdx.x; g < groups; g += blockDim.x) {
                const uint32_t o0 = g * kPack;
                uint32_t c, r;
                a.div_R.divmod(o0, c, r);
                uint32_t word = 0;
#pragma unroll
                for (int k = 0; k < kPack; ++k) {
                    word |= static_cast<uint32_t>(*reinterpret_cast<const U*>(smem + r * a.pitch + c * US)) << (8 * US * k);
                    if (++r == a.R) { r = 0; ++c; }
                }
                *reinterpret_cast<uint32_t*>(mat + static_cast<uint64_t>(o0) * US) = word;
            }
            for (uint32_t o = groups * kPack + threadIdx.x; o < units; o += blockDim.x) {
                uint32_t c, r;
                a.div_R.divmod(o, c, r);
                *reinterpret_cast<U*>(mat + static_cast<uint64_t>(o) * US) = *reinterpret_cast<const U*>(smem + r * a.pitch + c * US);
            }
        } else {
            for (uint32_t x = threadIdx.x; x < units; x += blockDim.x) {
                uint32_t o, u, c, r;
                a.div_upw.divmod(x, o, u);
                if (u >= lim) continue;
                a.div_R.divmod(o, c, r);  // output o = c*R + r holds input (r, c)
                const U v = *reinterpret_cast<const U*>(smem + r * a.pitch + c * a.w + u * US);
                *reinterpret_cast<U*>(mat + o * a.E + u * US) = v;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Slab transpose of a matrix over a K-CTA cluster, owner-computed: CTA k
// stages input rows [k*Q, (k+1)*Q) and, after the cluster barrier, writes
// its band's segment of every output row (output row c, positions k*Q ..
// k*Q+Q-1) from its own shared memory.  One pass for matrices up to K x
// 110 KB; the barrier only orders every CTA's loads of a matrix before any
// CTA's writes to it.  kPack > 1: elements of US bytes packed kPack to a
// 4-byte store.
// ---------------------------------------------------------------------------
struct SlabClusterArgs {
    uint8_t* base;
    uint64_t items, mat_bytes, row_bytes;
    uint32_t R, C, E, Q, pitch, upr, upw, wpr;
    bool load4;  // rows are whole 4-byte words at a 4-byte aligned base: load words
    // otherwise, narrow units: each row of the band is staged from the
    // aligned words it spans (funnel shifts; rowchunks 16-byte units a row)
    bool stage_words;
    uint32_t rowchunks;
    FastDiv32 div_rowchunks;
    FastDiv32 div_upr, div_upw, div_Qupw, div_Qpack, div_wpr, div_rowb;
    // wide elements of 1- or 2-byte units: each output row's segment (the
    // band's nr elements, contiguous) written by one warp as the aligned
    // 4-byte words inside it, gathered byte by byte
    bool write_words;
    FastDiv32 div_E;
};

template <int US, int kPack>
__global__ void __launch_bounds__(kThreads) k_slab_cluster(SlabClusterArgs a) {
    using U = typename UnitOf<US>::T;
    extern __shared__ __align__(16) uint8_t smem[];
    cg::cluster_group cl = cg::this_cluster();
    const unsigned K = cl.num_blocks();
    const unsigned kr = cl.block_rank();
    const uint64_t cid = blockIdx.x / K, ncl = gridDim.x / K;
    const uint32_t r0 = kr * a.Q;
    const uint32_t nr = r0 < a.R ? min(a.Q, a.R - r0) : 0;
    for (uint64_t it = cid; it < a.items; it += ncl) {
        uint8_t* mat = a.base + it * a.mat_bytes;
        const uint8_t* band = mat + static_cast<uint64_t>(r0) * a.row_bytes;
        if (a.load4) {  // rows of whole 4-byte words, 4-byte aligned: word copies
            const uint32_t in_words = nr * a.wpr;
            for (uint32_t x = threadIdx.x; x < in_words; x += blockDim.x) {
                uint32_t rr, cw;
                a.div_wpr.divmod(x, rr, cw);
                copy_in<4, uint32_t>(smem + rr * a.pitch + cw * 4, band + static_cast<uint64_t>(x) * 4);
            }
            copy_in_wait<4>();
        } else if (US < 4 && a.stage_words) {
            // each row staged 16 bytes per thread from the aligned words it
            // spans; a CTA past the last row (K Q > R) has no band (its band
            // pointer lies beyond the matrix, possibly beyond the allocation)
            // and reads nothing
            const uint32_t rowb = static_cast<uint32_t>(a.row_bytes);
            span_stage(nr * a.rowchunks, [&](uint32_t x) {
                uint32_t rr, t;
                a.div_rowchunks.divmod(x, rr, t);
                return SpanUnit{smem + rr * a.pitch, band + static_cast<uint64_t>(rr) * rowb, rowb, t, true};
            });
        } else {
            const uint32_t in_units = nr * a.upr;
            for (uint32_t x = threadIdx.x; x < in_units; x += blockDim.x) {
                uint32_t rr, cu;
                a.div_upr.divmod(x, rr, cu);
                copy_in<US, U>(smem + rr * a.pitch + cu * US, band + static_cast<uint64_t>(x) * US);
            }
            copy_in_wait<US>();
        }
        cluster_sync_reuse();  // every CTA holds its band: writes may start
        if constexpr (kPack > 1) {
            const uint32_t groups = a.C * (a.Q / kPack);
            for (uint32_t x = threadIdx.x; x < groups; x += blockDim.x) {
                uint32_t c, g;
                a.div_Qpack.divmod(x, c, g);
                const uint32_t rr = g * kPack;
                if (rr >= nr) continue;  // nr is a multiple of kPack
                uint32_t word = 0;
#pragma unroll
                for (int k = 0; k < kPack; ++k)
                    word |= static_cast<uint32_t>(*reinterpret_cast<const U*>(smem + (rr + k) * a.pitch + c * US))
                            << (8 * US * k);
                *reinterpret_cast<uint32_t*>(mat + (static_cast<uint64_t>(c) * a.R + r0 + rr) * US) = word;
            }
        } else if (US < 4 && a.write_words) {
            const uint32_t segb = nr * a.E;
            const uint32_t lane = threadIdx.x & 31u, nw = blockDim.x / 32;
            for (uint32_t c = threadIdx.x / 32; c < a.C && segb; c += nw) {
                uint8_t* dst = mat + (static_cast<uint64_t>(c) * a.R + r0) * a.E;
                const uint8_t* col = smem + c * a.E;
                auto byte_of = [&](uint32_t s) -> uint32_t {
                    uint32_t rr, e;
                    a.div_E.divmod(s, rr, e);
                    return col[rr * a.pitch + e];
                };
                const uint32_t hw = min(segb, static_cast<uint32_t>((4 - (reinterpret_cast<uintptr_t>(dst) & 3u)) & 3u));
                const uint32_t words = (segb - hw) / 4;
                for (uint32_t k = lane; k < words; k += 32) {
                    const uint32_t s = hw + 4 * k;
                    uint32_t rr, e;  // byte e of the segment's element rr
                    a.div_E.divmod(s, rr, e);
                    uint32_t v = 0;
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        v |= static_cast<uint32_t>(col[rr * a.pitch + e]) << (8 * j);
                        if (++e == a.E) {
                            e = 0;
                            ++rr;
                        }
                    }
                    *reinterpret_cast<uint32_t*>(dst + s) = v;
                }
                const uint32_t rest = segb - words * 4;  // hw bytes before the words, the tail after
                for (uint32_t x = lane; x < rest; x += 32) {
                    const uint32_t s = x < hw ? x : hw + words * 4 + (x - hw);
                    dst[s] = static_cast<uint8_t>(byte_of(s));
                }
            }
        } else {
            const uint32_t out_units = a.C * a.Q * a.upw;
            for (uint32_t x = threadIdx.x; x < out_units; x += blockDim.x) {
                uint32_t c, rest, rr, u;
                a.div_Qupw.divmod(x, c, rest);
                a.div_upw.divmod(rest, rr, u);
                if (rr >= nr) continue;
                *reinterpret_cast<U*>(mat + (static_cast<uint64_t>(c) * a.R + r0 + rr) * a.E + u * US) =
                    *reinterpret_cast<const U*>(smem + rr * a.pitch + c * a.E + u * US);
            }
        }
        __syncthreads();  // the band's buffer is free for the next matrix
    }
}

// Copies `bytes` contiguous bytes from global memory into shared memory:
// 16-byte cp.async chunks when both ends and the size allow it (vec16),
// else US-byte units.  Completes before returning.
// Copies `bytes` contiguous bytes at any alignment from global memory to
// shared memory through the aligned 16-byte chunks around them (bytes of the
// first and last chunk outside the range are read and dropped; a chunk never
// crosses a page).  For 1- and 2-byte units: one load per 16 bytes instead of
// one per unit.
__device__ __forceinline__ void words_copy_in(uint8_t* sm, const uint8_t* g, uint32_t bytes) {
    const uintptr_t lo = reinterpret_cast<uintptr_t>(g);
    const uint32_t head = static_cast<uint32_t>(lo & 15u);
    const uint4* cp = reinterpret_cast<const uint4*>(lo - head);
    const uint32_t chunks = bytes ? (head + bytes + 15) / 16 : 0;  // nothing read for an empty range
    constexpr int kDepth = 2;  // chunks in flight per thread (register-bound callers)
    for (uint32_t x0 = threadIdx.x; x0 < chunks; x0 += kDepth * blockDim.x) {
        uint4 v[kDepth];
#pragma unroll
        for (int j = 0; j < kDepth; ++j) {
            const uint32_t x = x0 + j * blockDim.x;
            if (x < chunks) v[j] = cp[x];
        }
#pragma unroll
        for (int j = 0; j < kDepth; ++j) {
            const uint32_t x = x0 + j * blockDim.x;
            if (x >= chunks) break;
            place_chunk(sm, v[j], x * 16 - head, bytes);
        }
    }
}

template <int US>
__device__ __forceinline__ void block_copy_in(uint8_t* sm, const uint8_t* g, uint32_t bytes, bool vec16,
                                              bool words) {
    using U = typename UnitOf<US>::T;
    if (vec16) {
        for (uint32_t x = threadIdx.x; x < bytes / 16; x += blockDim.x) copy_in<16, uint4>(sm + x * 16, g + x * 16);
        copy_in_wait<16>();
    } else if (US < 4 && words && bytes >= 64) {
        words_copy_in(sm, g, bytes);
    } else {
        for (uint32_t x = threadIdx.x; x < bytes / US; x += blockDim.x) copy_in<US, U>(sm + x * US, g + x * US);
        copy_in_wait<US>();
    }
}

// Small matrices (a few KB or less): an item is a block of k consecutive
// matrices, loaded contiguously; every output element reads its input in
// shared memory.  Millions of 3x5 matrices would otherwise take one CTA item
// each.  Whole elements only.
struct SlabPackArgs {
    uint8_t* base;
    uint64_t batches, items, mat_bytes, E;
    uint32_t k, R, C, upw, mat_units;
    bool vec16;  // base and matrix size are 16-byte multiples
    bool words;  // narrow units: stage from aligned 4-byte words (knob narrow_words)
    FastDiv32 div_mat_units, div_upw, div_R;
};

template <int US, int kPack>
__global__ void __launch_bounds__(kThreads) k_slab_pack(SlabPackArgs a) {
    using U = typename UnitOf<US>::T;
    extern __shared__ __align__(16) uint8_t smem[];
    for (uint64_t it = blockIdx.x; it < a.items; it += gridDim.x) {
        const uint64_t m0 = it * a.k;
        const uint64_t left = a.batches - m0;
        const uint32_t nm = static_cast<uint32_t>(left < a.k ? left : a.k);
        uint8_t* blk = a.base + m0 * a.mat_bytes;
        const uint32_t units = nm * a.mat_units;
        block_copy_in<US>(smem, blk, units * US, a.vec16 && (units * US) % 16 == 0, a.words);
        __syncthreads();
        if constexpr (kPack > 1) {
            // kPack consecutive output elements (they may cross output rows
            // and matrices) gathered into one 4-byte store
            const uint32_t groups = units / kPack;
            for (uint32_t g = threadIdx.x; g < groups; g += blockDim.x) {
                const uint32_t x = g * kPack;
                uint32_t m, o, c, r;
                a.div_mat_units.divmod(x, m, o);
                a.div_R.divmod(o, c, r);
                uint32_t word = 0;
#pragma unroll
                for (int k = 0; k < kPack; ++k) {
                    word |= static_cast<uint32_t>(*reinterpret_cast<const U*>(smem + (m * a.mat_units + r * a.C + c) * US))
                            << (8 * US * k);
                    if (++r == a.R) {
                        r = 0;
                        if (++c == a.C) { c = 0; ++m; }
                    }
                }
                *reinterpret_cast<uint32_t*>(blk + static_cast<uint64_t>(x) * US) = word;
            }
            for (uint32_t x = groups * kPack + threadIdx.x; x < units; x += blockDim.x) {  // the tail
                uint32_t m, o, c, r;
                a.div_mat_units.divmod(x, m, o);
                a.div_R.divmod(o, c, r);
                *reinterpret_cast<U*>(blk + static_cast<uint64_t>(x) * US) =
                    *reinterpret_cast<const U*>(smem + (m * a.mat_units + r * a.C + c) * US);
            }
        } else {
            for (uint32_t x = threadIdx.x; x < units; x += blockDim.x) {
                uint32_t m, rest, o, u, c, r;
                a.div_mat_units.divmod(x, m, rest);
                a.div_upw.divmod(rest, o, u);
                a.div_R.divmod(o, c, r);  // output o = c*R + r holds input (r, c)
                const uint32_t src = m * a.mat_units + (r * a.C + c) * a.upw + u;
                *reinterpret_cast<U*>(blk + static_cast<uint64_t>(x) * US) = *reinterpret_cast<const U*>(smem + src * US);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Row pass staged in the distributed shared memory of a K-CTA cluster: item
// = one strip of one row; CTA k of the cluster owns pieces [k*P, (k+1)*P).
// Gather: each CTA loads its own pieces, the cluster synchronises, then each
// CTA writes its pieces reading f(i,j) from whichever CTA holds it.
// Scatter: each CTA loads its pieces and stores piece j into the CTA that
// owns f(i,j); after the cluster barrier each CTA writes its own range.
// Items are double-buffered: the loads of the next item are issued before
// the write-back of the current one, so HBM reads overlap the gathers.
// ---------------------------------------------------------------------------
struct RowArgs {
    uint8_t* base;
    unsigned* status;  // the call's status word
    uint64_t items, E, row_bytes;
    uint32_t rows, cols, P, w, upw, last_upw, nstrips, buf_bytes;
    bool flat;  // w == E: a CTA's pieces are contiguous bytes
    bool dbuf;  // two item buffers: the next item's loads overlap this item's write-back
    bool words; // narrow units: stage contiguous pieces from aligned 4-byte words (knob narrow_words)
    FastDiv div_strips, div_rows;
    FastDiv32 div_upw, div_P;
};

constexpr int kBatch = 4;  // remote shared-memory loads in flight per thread

template <int US, typename Fn, bool kScatter>
__device__ __forceinline__ void row_stage_in(const RowArgs& a, const Fn& fn, uint8_t* const* peers, uint8_t* buf,
                                             uint32_t boff, uint64_t it, uint32_t j0, uint32_t my_units) {
    using U = typename UnitOf<US>::T;
    using I = typename Fn::index_type;
    uint64_t bi, s;
    a.div_strips.divmod(it, bi, s);
    const uint32_t lim = (s + 1 == a.nstrips) ? a.last_upw : a.upw;
    const uint8_t* row = a.base + bi * a.row_bytes + s * a.w;
    if constexpr (kScatter) {
        // kLoadBatch global loads in flight per thread before the pushes
        constexpr int kLoadBatch = US >= 8 ? 4 : 8;
        const I i = static_cast<I>(a.div_rows.mod(bi));
        for (uint32_t x0 = threadIdx.x; x0 < my_units; x0 += kLoadBatch * blockDim.x) {
            U v[kLoadBatch];
            uint32_t jq[kLoadBatch], uq[kLoadBatch];
            bool ok[kLoadBatch];
#pragma unroll
            for (int q = 0; q < kLoadBatch; ++q) {
                const uint32_t x = x0 + q * blockDim.x;
                ok[q] = false;
                if (x >= my_units) continue;
                a.div_upw.divmod(x, jq[q], uq[q]);
                if (uq[q] >= lim) continue;
                jq[q] += j0;
                v[q] = *reinterpret_cast<const U*>(row + static_cast<uint64_t>(jq[q]) * a.E + uq[q] * US);
                ok[q] = true;
            }
#pragma unroll
            for (int q = 0; q < kLoadBatch; ++q) {
                if (!ok[q]) continue;
                const I dst = fn(i, static_cast<I>(jq[q]));
                if (!in_range(dst, a.cols, a.status)) continue;
                uint32_t owner, off;
                a.div_P.divmod(static_cast<uint32_t>(dst), owner, off);
                *reinterpret_cast<U*>(peers[owner] + boff + off * a.w + uq[q] * US) = v[q];
            }
        }
    } else if (a.flat) {
        const uint8_t* src = row + static_cast<uint64_t>(j0) * a.E;
        if (US < 4 && a.words && my_units * US >= 64) {
            words_copy_in(buf, src, my_units * US);
        } else {
            for (uint32_t x = threadIdx.x; x < my_units; x += blockDim.x)
                copy_in<US, U>(buf + x * US, src + static_cast<uint64_t>(x) * US);
        }
    } else {
        for (uint32_t x = threadIdx.x; x < my_units; x += blockDim.x) {
            uint32_t jj, u;
            a.div_upw.divmod(x, jj, u);
            if (u >= lim) continue;
            copy_in<US, U>(buf + jj * a.w + u * US, row + static_cast<uint64_t>(j0 + jj) * a.E + u * US);
        }
    }
    if constexpr (US >= 4 && !kScatter) asm volatile("cp.async.commit_group;\n" ::: "memory");
}

template <int US, typename Fn, bool kScatter>
__global__ void __launch_bounds__(kThreads) k_row_cluster(RowArgs a, Fn fn) {
    using U = typename UnitOf<US>::T;
    using I = typename Fn::index_type;
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ uint8_t* peers[16];
    cg::cluster_group cl = cg::this_cluster();
    const unsigned K = cl.num_blocks();
    const unsigned kr = cl.block_rank();
    load_peers(peers, smem, K);
    const uint64_t cid = blockIdx.x / K, ncl = gridDim.x / K;
    const uint32_t j0 = kr * a.P;
    const uint32_t jn = min(a.cols, j0 + a.P);
    const uint32_t my_units = (jn > j0 ? jn - j0 : 0) * a.upw;
    cluster_sync_reuse();  // every CTA of the cluster is running before any DSMEM access
    if (a.dbuf && cid < a.items) row_stage_in<US, Fn, kScatter>(a, fn, peers, smem, 0, cid, j0, my_units);
    uint32_t k = 0;
    for (uint64_t it = cid; it < a.items; it += ncl, ++k) {
        const uint32_t boff = a.dbuf ? (k & 1) * a.buf_bytes : 0;
        if (!a.dbuf) row_stage_in<US, Fn, kScatter>(a, fn, peers, smem, 0, it, j0, my_units);
        if constexpr (US >= 4 && !kScatter) asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        cluster_sync_publish();
        const uint64_t nxt = it + ncl;
        if (a.dbuf && nxt < a.items)
            row_stage_in<US, Fn, kScatter>(a, fn, peers, smem + (boff ^ a.buf_bytes), boff ^ a.buf_bytes, nxt, j0, my_units);
        uint64_t bi, s;
        a.div_strips.divmod(it, bi, s);
        const I i = static_cast<I>(a.div_rows.mod(bi));
        const uint32_t lim = (s + 1 == a.nstrips) ? a.last_upw : a.upw;
        uint8_t* row = a.base + bi * a.row_bytes + s * a.w;
        for (uint32_t x0 = threadIdx.x; x0 < my_units; x0 += kBatch * blockDim.x) {
            U v[kBatch];
            uint8_t* dst[kBatch];
#pragma unroll
            for (int q = 0; q < kBatch; ++q) {
                dst[q] = nullptr;
                const uint32_t x = x0 + q * blockDim.x;
                if (x >= my_units) continue;
                uint32_t jj, u;
                a.div_upw.divmod(x, jj, u);
                if (u >= lim) continue;
                const uint32_t j = j0 + jj;
                if constexpr (kScatter) {
                    v[q] = *reinterpret_cast<const U*>(smem + boff + jj * a.w + u * US);
                } else {
                    const I src = fn(i, static_cast<I>(j));
                    if (!in_range(src, a.cols, a.status)) continue;
                    uint32_t owner, off;
                    a.div_P.divmod(static_cast<uint32_t>(src), owner, off);
                    v[q] = *reinterpret_cast<const U*>(peers[owner] + boff + off * a.w + u * US);
                }
                dst[q] = row + static_cast<uint64_t>(j) * a.E + u * US;
            }
#pragma unroll
            for (int q = 0; q < kBatch; ++q)
                if (dst[q]) *reinterpret_cast<U*>(dst[q]) = v[q];
        }
        cluster_sync_reuse();
    }
}

// ---------------------------------------------------------------------------
// Row pass for short rows (a few KB or less): an item is a block of k
// consecutive rows, loaded contiguously into one CTA's shared memory; each
// output element of the block gathers from its own row there.  Tall, skinny
// matrices (millions of rows of a few elements) would otherwise spend one
// CTA item per row.  Gather form only.
// ---------------------------------------------------------------------------
struct RowBlockArgs {
    uint8_t* base;
    unsigned* status;  // the call's status word
    uint64_t total_rows, items, row_bytes, E;
    uint32_t k, cols, upw, units_per_row;
    bool vec16;
    bool words;                // narrow units: stage from aligned 4-byte words (knob narrow_words)                // base and row size are 16-byte multiples
    FastDiv div_rows;          // global row -> row within its matrix
    FastDiv32 div_units_row;   // unit of the block -> (row of the block, unit of the row)
    FastDiv32 div_upw;
};

template <int US, typename Fn>
__global__ void __launch_bounds__(kThreads) k_row_block(RowBlockArgs a, Fn fn) {
    using U = typename UnitOf<US>::T;
    using I = typename Fn::index_type;
    extern __shared__ __align__(16) uint8_t smem[];
    for (uint64_t it = blockIdx.x; it < a.items; it += gridDim.x) {
        const uint64_t r0 = it * a.k;
        const uint64_t left = a.total_rows - r0;
        const uint32_t nr = static_cast<uint32_t>(left < a.k ? left : a.k);
        uint8_t* blk = a.base + r0 * a.row_bytes;
        const uint32_t units = nr * a.units_per_row;
        block_copy_in<US>(smem, blk, units * US, a.vec16 && (units * US) % 16 == 0, a.words);
        __syncthreads();
        for (uint32_t x0 = threadIdx.x; x0 < units; x0 += kBatch * blockDim.x) {
            U v[kBatch];
            uint32_t dst[kBatch];
#pragma unroll
            for (int q = 0; q < kBatch; ++q) {
                dst[q] = ~0u;
                const uint32_t x = x0 + q * blockDim.x;
                if (x >= units) continue;
                uint32_t rr, jx, j, u;
                a.div_units_row.divmod(x, rr, jx);
                a.div_upw.divmod(jx, j, u);
                const I i = static_cast<I>(a.div_rows.mod(r0 + rr));
                const I src = fn(i, static_cast<I>(j));
                if (!in_range(src, a.cols, a.status)) continue;
                v[q] = *reinterpret_cast<const U*>(smem + rr * a.row_bytes + static_cast<uint32_t>(src) * a.E + u * US);
                dst[q] = x;
            }
#pragma unroll
            for (int q = 0; q < kBatch; ++q)
                if (dst[q] != ~0u) *reinterpret_cast<U*>(blk + static_cast<uint64_t>(dst[q]) * US) = v[q];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Row pass for rows that fill one CTA's shared memory (one CTA per SM, no
// room for a second item buffer): the next item is prefetched into
// registers (kRegs units of US bytes per thread, up to 128 KB per CTA)
// while the current item is gathered out of shared memory, so HBM reads
// overlap the write-back.  Gather form only (out[i][j] = in[i][fn(i,j)]).
// ---------------------------------------------------------------------------
template <int US, typename Fn, int kRegs>
__global__ void __launch_bounds__(kThreads) k_row_solo(RowArgs a, Fn fn) {
    using U = typename UnitOf<US>::T;
    using I = typename Fn::index_type;
    extern __shared__ __align__(16) uint8_t smem[];
    // flat items only (w == E): unit x of a row is bytes [x*US, (x+1)*US)
    const uint32_t units = a.cols * a.upw;
    U v[kRegs];
    auto fetch = [&](uint64_t it) {
        const U* row = reinterpret_cast<const U*>(a.base + it * a.row_bytes) + threadIdx.x;
#pragma unroll
        for (int q = 0; q < kRegs; ++q)
            if (threadIdx.x + q * kThreads < units) v[q] = row[q * kThreads];
    };
    if (blockIdx.x < a.items) fetch(blockIdx.x);
    for (uint64_t it = blockIdx.x; it < a.items; it += gridDim.x) {
        U* st = reinterpret_cast<U*>(smem) + threadIdx.x;
#pragma unroll
        for (int q = 0; q < kRegs; ++q)
            if (threadIdx.x + q * kThreads < units) st[q * kThreads] = v[q];
        __syncthreads();  // the item is in shared memory
        const uint64_t nxt = it + gridDim.x;
        if (nxt < a.items) fetch(nxt);  // in flight during the write-back below
        const I i = static_cast<I>(a.div_rows.mod(it));
        U* row = reinterpret_cast<U*>(a.base + it * a.row_bytes);
        const U* sm = reinterpret_cast<const U*>(smem);
        for (uint32_t x0 = threadIdx.x; x0 < units; x0 += kBatch * kThreads) {
            U w[kBatch];
            uint32_t dst[kBatch];
#pragma unroll
            for (int q = 0; q < kBatch; ++q) {
                dst[q] = ~0u;
                const uint32_t x = x0 + q * kThreads;
                if (x >= units) continue;
                uint32_t j, u;
                a.div_upw.divmod(x, j, u);
                const I src = fn(i, static_cast<I>(j));
                if (!in_range(src, a.cols, a.status)) continue;
                w[q] = sm[static_cast<uint32_t>(src) * a.upw + u];
                dst[q] = x;
            }
#pragma unroll
            for (int q = 0; q < kBatch; ++q)
                if (dst[q] != ~0u) row[dst[q]] = w[q];
        }
        __syncthreads();  // shared memory is free for the next item
    }
}

// ---------------------------------------------------------------------------
// Column pass staged in a K-CTA cluster: item = one strip of a tile of tw
// adjacent columns over all rows; CTA k owns rows [k*Q, (k+1)*Q).  When the
// tw*upw units of a staged row divide the block, every thread keeps one
// fixed unit of the row and walks the rows with a pointer stride.  Items are
// double-buffered like the row pass.
// ---------------------------------------------------------------------------
struct ColArgs {
    uint8_t* base;
    unsigned* status;  // the call's status word
    uint64_t items, E, row_bytes, mat_bytes;
    uint32_t rows, cols, tw, ntiles, pitch, Q, w, upw, last_upw, nstrips, RU, buf_bytes;  // RU = tw*upw
    bool dbuf;
    FastDiv div_strips, div_tiles;
    FastDiv32 div_RU, div_upw, div_Q;
};

struct ColItem {
    uint8_t* mat;
    uint32_t col0, tcols, lim;
};

__device__ __forceinline__ ColItem col_item(const ColArgs& a, uint64_t it) {
    uint64_t bt, s, b, t;
    a.div_strips.divmod(it, bt, s);
    a.div_tiles.divmod(bt, b, t);
    ColItem c;
    c.col0 = static_cast<uint32_t>(t) * a.tw;
    c.tcols = min(a.tw, a.cols - c.col0);
    c.lim = (s + 1 == a.nstrips) ? a.last_upw : a.upw;
    c.mat = a.base + b * a.mat_bytes + static_cast<uint64_t>(c.col0) * a.E + s * a.w;
    return c;
}

template <int US, bool kLanes>
__device__ __forceinline__ void col_stage_in(const ColArgs& a, uint8_t* buf, uint64_t it, uint32_t r0,
                                             uint32_t myrows, uint32_t lc, uint32_t lu, uint32_t ii0,
                                             uint32_t step) {
    using U = typename UnitOf<US>::T;
    const ColItem ci = col_item(a, it);
    if constexpr (kLanes) {
        if (lc < ci.tcols && lu < ci.lim) {
            const uint64_t gstep = static_cast<uint64_t>(step) * a.row_bytes;
            const uint8_t* g = ci.mat + static_cast<uint64_t>(r0 + ii0) * a.row_bytes + static_cast<uint64_t>(lc) * a.E + lu * US;
            uint8_t* sm = buf + ii0 * a.pitch + lc * a.w + lu * US;
            for (uint32_t ii = ii0; ii < myrows; ii += step, g += gstep, sm += step * a.pitch) copy_in<US, U>(sm, g);
        }
    } else {
        const uint32_t my_units = myrows * a.RU;
        for (uint32_t x = threadIdx.x; x < my_units; x += blockDim.x) {
            uint32_t ii, r, c, u;
            a.div_RU.divmod(x, ii, r);
            a.div_upw.divmod(r, c, u);
            if (c >= ci.tcols || u >= ci.lim) continue;
            copy_in<US, U>(buf + ii * a.pitch + c * a.w + u * US,
                           ci.mat + static_cast<uint64_t>(r0 + ii) * a.row_bytes + static_cast<uint64_t>(c) * a.E + u * US);
        }
    }
    if constexpr (US >= 4) asm volatile("cp.async.commit_group;\n" ::: "memory");
}

template <int US, typename Fn, bool kLanes, int kB>
__global__ void __launch_bounds__(kThreads) k_col_cluster(ColArgs a, Fn fn) {
    using U = typename UnitOf<US>::T;
    using I = typename Fn::index_type;
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ uint8_t* peers[16];
    cg::cluster_group cl = cg::this_cluster();
    const unsigned K = cl.num_blocks();
    const unsigned kr = cl.block_rank();
    load_peers(peers, smem, K);
    const uint64_t cid = blockIdx.x / K, ncl = gridDim.x / K;
    const uint32_t r0 = kr * a.Q;
    const uint32_t rn = min(a.rows, r0 + a.Q);
    const uint32_t myrows = rn > r0 ? rn - r0 : 0;
    uint32_t lc = 0, lu = 0, ii0 = 0, step = 1;
    if constexpr (kLanes) {
        uint32_t lr;
        a.div_RU.divmod(threadIdx.x, ii0, lr);
        a.div_upw.divmod(lr, lc, lu);
        step = blockDim.x / a.RU;
    }
    cluster_sync_reuse();  // every CTA of the cluster is running before any DSMEM access
    if (a.dbuf && cid < a.items) col_stage_in<US, kLanes>(a, smem, cid, r0, myrows, lc, lu, ii0, step);
    uint32_t k = 0;
    for (uint64_t it = cid; it < a.items; it += ncl, ++k) {
        const uint32_t boff = a.dbuf ? (k & 1) * a.buf_bytes : 0;
        if (!a.dbuf) col_stage_in<US, kLanes>(a, smem, it, r0, myrows, lc, lu, ii0, step);
        if constexpr (US >= 4) asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        cluster_sync_publish();
        const uint64_t nxt = it + ncl;
        if (a.dbuf && nxt < a.items) col_stage_in<US, kLanes>(a, smem + (boff ^ a.buf_bytes), nxt, r0, myrows, lc, lu, ii0, step);
        const ColItem ci = col_item(a, it);
        if constexpr (kLanes) {
            if (lc < ci.tcols && lu < ci.lim) {
                const uint64_t gstep = static_cast<uint64_t>(step) * a.row_bytes;
                uint8_t* g = ci.mat + static_cast<uint64_t>(r0 + ii0) * a.row_bytes + static_cast<uint64_t>(lc) * a.E + lu * US;
                const uint32_t soff = boff + lc * a.w + lu * US;
                const I col = static_cast<I>(ci.col0 + lc);
                for (uint32_t ii = ii0; ii < myrows; ii += kB * step, g += kB * gstep) {
                    U v[kB];
                    bool ok[kB];
#pragma unroll
                    for (int q = 0; q < kB; ++q) {
                        const uint32_t iq = ii + q * step;
                        ok[q] = false;
                        if (iq >= myrows) continue;
                        const I src = fn(static_cast<I>(r0 + iq), col);
                        if (!in_range(src, a.rows, a.status)) continue;
                        uint32_t owner, off;
                        a.div_Q.divmod(static_cast<uint32_t>(src), owner, off);
                        v[q] = *reinterpret_cast<const U*>(peers[owner] + off * a.pitch + soff);
                        ok[q] = true;
                    }
#pragma unroll
                    for (int q = 0; q < kB; ++q)
                        if (ok[q]) *reinterpret_cast<U*>(g + q * gstep) = v[q];
                }
            }
        } else {
            const uint32_t my_units = myrows * a.RU;
            for (uint32_t x = threadIdx.x; x < my_units; x += blockDim.x) {
                uint32_t ii, r, c, u;
                a.div_RU.divmod(x, ii, r);
                a.div_upw.divmod(r, c, u);
                if (c >= ci.tcols || u >= ci.lim) continue;
                const I src = fn(static_cast<I>(r0 + ii), static_cast<I>(ci.col0 + c));
                if (!in_range(src, a.rows, a.status)) continue;
                uint32_t owner, off;
                a.div_Q.divmod(static_cast<uint32_t>(src), owner, off);
                *reinterpret_cast<U*>(ci.mat + static_cast<uint64_t>(r0 + ii) * a.row_bytes + static_cast<uint64_t>(c) * a.E + u * US) =
                    *reinterpret_cast<const U*>(peers[owner] + boff + off * a.pitch + c * a.w + u * US);
            }
        }
        cluster_sync_reuse();
    }
}

// ---------------------------------------------------------------------------
// Owner-computed column pass (c2r column shuffle, c2r pre-rotation, r2c
// post-rotation; see the owner maps in index_math.cuh).  CTA k of the
// cluster stages source rows [k*Q - Hlo, (k+1)*Q + Hhi) (mod m) of the tile;
// after the cluster barrier it writes, for every owned source row x, the
// whole row piece of output row row_of(x, j0), reading only its own shared
// memory.  The barrier only orders every CTA's loads of the tile before any
// CTA's writes to it, so it is relaxed: a load that has returned its value
// cannot be affected by a later write.
// ---------------------------------------------------------------------------
struct ColOwnArgs {
    uint8_t* base;
    unsigned* status;  // the call's status word
    uint64_t items, E, row_bytes, mat_bytes;
    uint32_t rows, cols, tw, ntiles, pitch, Q, Hlo, Hhi, w, upw, last_upw, nstrips, RU, buf_bytes;
    uint32_t hbase;  // (-Hlo) mod m: slot x0 - Hlo is slot (x0 + hbase) mod m, also when Hlo > m
    bool dbuf;
    bool whole;      // one CTA holds all m slots of a tile: no halo, slots indexed modulo m
    uint32_t dofs;   // whole: a multiple of m above every |delta difference| of a tile
    // narrow whole elements: each slot's row piece is staged from the aligned
    // 16-byte chunks around it (wpp chunks per piece at most; bytes outside
    // the piece read and dropped, a chunk never crosses a page)
    bool stage_words;
    uint32_t wpp;
    FastDiv div_strips, div_tiles;
    FastDiv32 div_RU, div_upw, div_m, div_wpp;
};

// Staged slot holding the source of output slot ii's element at column
// offset d = delta(j0 + c) - delta(j0).
__device__ __forceinline__ int64_t own_local(const ColOwnArgs& a, uint32_t ii, int64_t d) {
    if (a.whole) return a.div_m.mod(static_cast<uint32_t>(static_cast<int64_t>(ii) + d + a.dofs));
    return static_cast<int64_t>(ii + a.Hlo) + d;
}

struct OwnItem {
    uint8_t* mat;
    uint32_t col0, tcols, lim;
};

__device__ __forceinline__ OwnItem own_item(const ColOwnArgs& a, uint64_t it) {
    uint64_t bt, s, b, t;
    a.div_strips.divmod(it, bt, s);
    a.div_tiles.divmod(bt, b, t);
    OwnItem c;
    c.col0 = static_cast<uint32_t>(t) * a.tw;
    c.tcols = min(a.tw, a.cols - c.col0);
    c.lim = (s + 1 == a.nstrips) ? a.last_upw : a.upw;
    c.mat = a.base + b * a.mat_bytes + static_cast<uint64_t>(c.col0) * a.E + s * a.w;
    return c;
}

// Row tables of the owner-computed forms.  A CTA's staged slots hold the same source
// rows for every item (stage_of depends on the slot alone), so they are
// computed once per CTA; the output rows of its owned slots depend on the
// item's first column and are computed once per item, by one thread per row
// instead of by every lane of the row.
template <typename Own>
__device__ __forceinline__ void own_fill_stage_rows(const ColOwnArgs& a, const Own& own,
                                                    typename Own::index_type* srow, uint32_t x0, uint32_t nstage) {
    using I = typename Own::index_type;
    const uint32_t tbase = x0 + a.hbase;
    for (uint32_t ii = threadIdx.x; ii < nstage; ii += blockDim.x)
        srow[ii] = own.stage_of(static_cast<I>(a.div_m.mod(tbase + ii)));
}

template <typename Own>
__device__ __forceinline__ void own_fill_write_rows(const Own& own, typename Own::index_type* wrow, uint32_t x0,
                                                    uint32_t myrows, uint32_t col0) {
    using I = typename Own::index_type;
    for (uint32_t ii = threadIdx.x; ii < myrows; ii += blockDim.x)
        wrow[ii] = own.row_of(static_cast<I>(x0 + ii), static_cast<I>(col0));
}

// own_stage_in with the source rows read from the CTA's table.
template <int US, typename I, bool kLanes>
__device__ __forceinline__ void own_stage_in_tab(const ColOwnArgs& a, const I* srow, uint8_t* buf, uint64_t it,
                                                 uint32_t nstage, uint32_t lc, uint32_t lu, uint32_t ii0,
                                                 uint32_t step) {
    using U = typename UnitOf<US>::T;
    const OwnItem ci = own_item(a, it);
    if constexpr (US < 4) {
        if (a.stage_words) {
            const uint32_t pb = ci.tcols * static_cast<uint32_t>(a.E);  // bytes of a row piece
            const uint32_t total = nstage * a.wpp;
            for (uint32_t x0 = threadIdx.x; x0 < total; x0 += kWordDepth * blockDim.x) {
                uint4 v[kWordDepth];
                uint32_t ii[kWordDepth], b[kWordDepth];
                bool ok[kWordDepth];
#pragma unroll
                for (int j = 0; j < kWordDepth; ++j) {
                    const uint32_t x = x0 + j * blockDim.x;
                    ok[j] = false;
                    if (x >= total) continue;
                    uint32_t q;
                    a.div_wpp.divmod(x, ii[j], q);
                    const I gr = srow[ii[j]];
                    if (!in_range(gr, a.rows, a.status)) continue;
                    const uintptr_t lo = reinterpret_cast<uintptr_t>(ci.mat + static_cast<uint64_t>(gr) * a.row_bytes);
                    const uint32_t head = static_cast<uint32_t>(lo & 15u);
                    if (q * 16 >= head + pb) continue;  // offset in the aligned span; the piece starts at `head`
                    v[j] = *reinterpret_cast<const uint4*>(lo - head + q * 16);
                    b[j] = q * 16 - head;  // piece byte of the chunk's first byte (wraps below 0)
                    ok[j] = true;
                }
#pragma unroll
                for (int j = 0; j < kWordDepth; ++j)
                    if (ok[j]) place_chunk(buf + ii[j] * a.pitch, v[j], b[j], pb);
            }
            return;
        }
    }
    if constexpr (kLanes) {
        if (lc < ci.tcols && lu < ci.lim) {
            const uint8_t* src = ci.mat + static_cast<uint64_t>(lc) * a.E + lu * US;
            uint8_t* dst = buf + lc * a.w + lu * US;
            for (uint32_t ii = ii0; ii < nstage; ii += step) {
                const I gr = srow[ii];
                if (!in_range(gr, a.rows, a.status)) continue;
                copy_in<US, U>(dst + ii * a.pitch, src + static_cast<uint64_t>(gr) * a.row_bytes);
            }
        }
    } else {
        const uint32_t units = nstage * a.RU;
        for (uint32_t x = threadIdx.x; x < units; x += blockDim.x) {
            uint32_t ii, r, c, u;
            a.div_RU.divmod(x, ii, r);
            a.div_upw.divmod(r, c, u);
            if (c >= ci.tcols || u >= ci.lim) continue;
            const I gr = srow[ii];
            if (!in_range(gr, a.rows, a.status)) continue;
            copy_in<US, U>(buf + ii * a.pitch + c * a.w + u * US,
                           ci.mat + static_cast<uint64_t>(gr) * a.row_bytes + static_cast<uint64_t>(c) * a.E + u * US);
        }
    }
    if constexpr (US >= 4) asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// Writes the CTA's output rows of item ci from its staged slots, the output
// rows read from the CTA's table: output row ii is wrow[ii], its element at
// column offset c comes from local ii + Hlo + delta(col0 + c) - delta(col0).
template <int US, typename Own, bool kLanes>
__device__ __forceinline__ void own_write_rows_tab(const ColOwnArgs& a, const Own& own, const uint8_t* buf,
                                                   const OwnItem& ci, const typename Own::index_type* wrow,
                                                   uint32_t myrows, uint32_t nstage, uint32_t lc, uint32_t lu,
                                                   uint32_t ii0, uint32_t step) {
    using U = typename UnitOf<US>::T;
    using I = typename Own::index_type;
    if constexpr (kLanes) {
        if (lc < ci.tcols && lu < ci.lim) {
            const int64_t d = own.delta(static_cast<I>(ci.col0 + lc)) - own.delta(static_cast<I>(ci.col0));
            const uint8_t* src = buf + lc * a.w + lu * US;
            uint8_t* dst = ci.mat + static_cast<uint64_t>(lc) * a.E + lu * US;
            for (uint32_t ii = ii0; ii < myrows; ii += step) {
                const I i = wrow[ii];
                const int64_t local = own_local(a, ii, d);
                if (!in_range(i, a.rows, a.status) || !in_range(static_cast<uint64_t>(local), nstage, a.status)) continue;
                *reinterpret_cast<U*>(dst + static_cast<uint64_t>(i) * a.row_bytes) =
                    *reinterpret_cast<const U*>(src + static_cast<uint32_t>(local) * a.pitch);
            }
        }
    } else {
        const uint32_t units = myrows * a.RU;
        for (uint32_t x = threadIdx.x; x < units; x += blockDim.x) {
            uint32_t ii, rr, c, u;
            a.div_RU.divmod(x, ii, rr);
            a.div_upw.divmod(rr, c, u);
            if (c >= ci.tcols || u >= ci.lim) continue;
            const int64_t d = own.delta(static_cast<I>(ci.col0 + c)) - own.delta(static_cast<I>(ci.col0));
            const I i = wrow[ii];
            const int64_t local = own_local(a, ii, d);
            if (!in_range(i, a.rows, a.status) || !in_range(static_cast<uint64_t>(local), nstage, a.status)) continue;
            *reinterpret_cast<U*>(ci.mat + static_cast<uint64_t>(i) * a.row_bytes + static_cast<uint64_t>(c) * a.E + u * US) =
                *reinterpret_cast<const U*>(buf + static_cast<uint32_t>(local) * a.pitch + c * a.w + u * US);
        }
    }
}

template <int US, typename Own, bool kLanes>
__global__ void __launch_bounds__(kThreads) k_col_owner(ColOwnArgs a, Own own) {
    using I = typename Own::index_type;
    extern __shared__ __align__(16) uint8_t smem[];
    cg::cluster_group cl = cg::this_cluster();
    const unsigned K = cl.num_blocks();
    const unsigned kr = cl.block_rank();
    const uint64_t cid = blockIdx.x / K, ncl = gridDim.x / K;
    const uint32_t x0 = kr * a.Q;
    const uint32_t myrows = x0 < a.rows ? min(a.Q, a.rows - x0) : 0;
    const uint32_t nstage = myrows ? myrows + a.Hlo + a.Hhi : 0;
    // row tables behind the slot buffer(s): Q + Hlo + Hhi source rows, Q output rows
    I* srow = reinterpret_cast<I*>(smem + (a.dbuf ? 2 : 1) * a.buf_bytes);
    I* wrow = srow + (a.Q + a.Hlo + a.Hhi);
    uint32_t lc = 0, lu = 0, ii0 = 0, step = 1;
    if constexpr (kLanes) {
        uint32_t lr;
        a.div_RU.divmod(threadIdx.x, ii0, lr);
        a.div_upw.divmod(lr, lc, lu);
        step = blockDim.x / a.RU;
    }
    own_fill_stage_rows(a, own, srow, x0, nstage);
    __syncthreads();
    if (a.dbuf && cid < a.items) own_stage_in_tab<US, I, kLanes>(a, srow, smem, cid, nstage, lc, lu, ii0, step);
    uint32_t k = 0;
    for (uint64_t it = cid; it < a.items; it += ncl, ++k) {
        const uint32_t boff = a.dbuf ? (k & 1) * a.buf_bytes : 0;
        if (!a.dbuf) own_stage_in_tab<US, I, kLanes>(a, srow, smem, it, nstage, lc, lu, ii0, step);
        const OwnItem ci = own_item(a, it);
        own_fill_write_rows(own, wrow, x0, myrows, ci.col0);
        if constexpr (US >= 4) asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();       // the CTA's slots and output rows are visible to all its threads
        cluster_sync_reuse();  // every CTA holds its rows of this tile: writes may start
        const uint64_t nxt = it + ncl;
        if (a.dbuf && nxt < a.items)
            own_stage_in_tab<US, I, kLanes>(a, srow, smem + (boff ^ a.buf_bytes), nxt, nstage, lc, lu, ii0, step);
        own_write_rows_tab<US, Own, kLanes>(a, own, smem + boff, ci, wrow, myrows, nstage, lc, lu, ii0, step);
        __syncthreads();  // this CTA's threads are done with the buffer and the output rows
    }
    if constexpr (US >= 4) asm volatile("cp.async.wait_group 0;\n" ::: "memory");  // no copy outlives the CTA
}

// ---------------------------------------------------------------------------
// Owner-computed column pass over groups of G co-resident CTAs (a
// cooperative launch guarantees co-residency), for tiles larger than a
// cluster's shared memory.  Group g takes items g, g + nG, ...; its CTA r
// owns slots [r*Q, (r+1)*Q).  The barrier between the group's loads and its
// writes is a monotonic arrival counter per group in global memory (zeroed
// before the launch): after its loads of the group's k-th item have landed
// in shared memory a CTA adds 1, and it writes once the counter has reached
// (k+1)*G (acquire).  The only hazard is write-after-read, and a read whose
// value has landed in shared memory cannot see a later write, so the add
// needs no release semantics (a knob restores them).  Every wait is bounded: a CTA
// that gives up (or sees another give up) counts a sync timeout, raises the
// launch's abort flag and returns after its own copies have landed.
// ---------------------------------------------------------------------------
struct GroupSync {
    unsigned* counters;  // nG arrival counters, then the abort flag
    unsigned* status;    // the call's status word (kCallSyncTimeout on a give-up)
    unsigned G, nG;
    unsigned spin_limit; // polls before a wait gives up
    unsigned sleep_ns;   // back-off between polls
    bool relaxed;        // arrive without release semantics (the arriving CTA's loads have completed)
    bool l2_prefetch;    // single-buffered: prefetch the next item into L2 while waiting
};

__device__ unsigned g_sync_timeouts;


__device__ __forceinline__ void group_arrive(unsigned* ctr, bool relaxed) {
    if (relaxed)
        asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;\n" ::"l"(ctr) : "memory");
    else
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;\n" ::"l"(ctr) : "memory");
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Thread 0 waits until *ctr >= target, polling at most spin_limit times;
// false when it gave up or the launch was aborted.  A give-up is counted
// (g_sync_timeouts) and recorded in the call's status word.  (A fence after
// relaxed polls would also wait for the CTA's own prefetches in flight;
// acquire loads do not.)
__device__ bool group_wait(const unsigned* ctr, unsigned target, unsigned* abort_flag, unsigned sleep_ns,
                           unsigned spin_limit, unsigned* status) {
    for (uint32_t it = 0; it < spin_limit; ++it) {
        if (ld_acquire(ctr) >= target) return true;
        if ((it & 31) == 31 && ld_acquire(abort_flag) != 0) return false;
        if (sleep_ns) __nanosleep(sleep_ns);
    }
    atomicAdd(&g_sync_timeouts, 1u);
    raise_status(status, kCallSyncTimeout);
    atomicExch(abort_flag, 1u);
    return false;
}

// Asks L2 for the row pieces of item `it` that this CTA will stage (one
// prefetch per 128-byte line), so that its loads after the barrier hit L2.
template <typename Own>
__device__ __forceinline__ void own_prefetch_l2(const ColOwnArgs& a, const Own& own, uint64_t it, uint32_t x0,
                                                uint32_t nstage) {
    using I = typename Own::index_type;
    const OwnItem ci = own_item(a, it);
    const uint32_t piece = ci.tcols * a.w;  // bytes of a staged row piece (whole elements: w == E)
    const uint32_t lines = (piece + 127) / 128 + 1;  // +1: a piece need not start on a line
    const uint32_t tbase = x0 + a.hbase;
    for (uint32_t x = threadIdx.x; x < nstage * lines; x += blockDim.x) {
        const uint32_t ii = x / lines, l = x - ii * lines;
        const I gr = own.stage_of(static_cast<I>(a.div_m.mod(tbase + ii)));
        if (!in_range(gr, a.rows, a.status)) continue;
        // an address inside the piece on every line it touches (the last one
        // is the piece's last byte)
        const uint8_t* p = ci.mat + static_cast<uint64_t>(gr) * a.row_bytes + min(l * 128, piece - 1);
        asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p));
    }
}

template <int US, typename Own, bool kLanes>
__global__ void __launch_bounds__(kThreads) k_col_group(ColOwnArgs a, Own own, GroupSync gs) {
    using U = typename UnitOf<US>::T;
    using I = typename Own::index_type;
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ int s_ok;
    const unsigned grp = blockIdx.x / gs.G, r = blockIdx.x - grp * gs.G;
    if (grp >= gs.nG) return;  // never launched: the grid is nG * G CTAs
    unsigned* ctr = gs.counters + grp;
    unsigned* abort_flag = gs.counters + gs.nG;
    const uint32_t x0 = r * a.Q;
    const uint32_t myrows = x0 < a.rows ? min(a.Q, a.rows - x0) : 0;
    const uint32_t nstage = myrows ? myrows + a.Hlo + a.Hhi : 0;
    // row tables behind the slot buffer(s): Q + Hlo + Hhi source rows, Q output rows
    I* srow = reinterpret_cast<I*>(smem + (a.dbuf ? 2 : 1) * a.buf_bytes);
    I* wrow = srow + (a.Q + a.Hlo + a.Hhi);
    uint32_t lc = 0, lu = 0, ii0 = 0, step = 1;
    if constexpr (kLanes) {
        uint32_t lr;
        a.div_RU.divmod(threadIdx.x, ii0, lr);
        a.div_upw.divmod(lr, lc, lu);
        step = blockDim.x / a.RU;
    }
    own_fill_stage_rows(a, own, srow, x0, nstage);
    __syncthreads();
    if (a.dbuf && grp < a.items) own_stage_in_tab<US, I, kLanes>(a, srow, smem, grp, nstage, lc, lu, ii0, step);
    uint32_t k = 0;
    for (uint64_t it = grp; it < a.items; it += gs.nG, ++k) {
        const uint32_t boff = a.dbuf ? (k & 1) * a.buf_bytes : 0;
        if (!a.dbuf) own_stage_in_tab<US, I, kLanes>(a, srow, smem, it, nstage, lc, lu, ii0, step);
        if constexpr (US >= 4) asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();  // this CTA's slots of the item are in shared memory
        if (threadIdx.x == 0 && gs.G > 1) group_arrive(ctr, gs.relaxed);
        const uint64_t nxt = it + gs.nG;
        if (a.dbuf && nxt < a.items)
            own_stage_in_tab<US, I, kLanes>(a, srow, smem + (boff ^ a.buf_bytes), nxt, nstage, lc, lu, ii0, step);
        if (!a.dbuf && gs.l2_prefetch && nxt < a.items)  // the next item's rows head for L2 during the wait
            own_prefetch_l2(a, own, nxt, x0, nstage);
        const OwnItem ci = own_item(a, it);
        own_fill_write_rows(own, wrow, x0, myrows, ci.col0);  // while thread 0 waits
        if (threadIdx.x == 0)
            s_ok = gs.G <= 1 || group_wait(ctr, (k + 1) * gs.G, abort_flag, gs.sleep_ns, gs.spin_limit, gs.status);
        __syncthreads();  // every CTA of the group holds its slots: writes may start
        if (!s_ok) break;
        own_write_rows_tab<US, Own, kLanes>(a, own, smem + boff, ci, wrow, myrows, nstage, lc, lu, ii0, step);
        __syncthreads();  // this CTA's threads are done with the buffer and the output rows
    }
    if constexpr (US >= 4) asm volatile("cp.async.wait_group 0;\n" ::: "memory");  // no copy outlives the CTA
}

// ---------------------------------------------------------------------------
// The group column pass with its slots staged by the bulk-copy engine: one
// cp.async.bulk per staged row piece (a row piece of a tile is contiguous
// when elements are whole, w == E), issued by the lanes of warp 0 and
// completed on an mbarrier per slot buffer.  Two slot buffers: the copies of
// the group's next item are issued as soon as this CTA has arrived at the
// group barrier, so they land while the CTA waits for the group and writes
// the current item; no thread spends registers or issue slots on staging.
// Preconditions (checked by the launcher): the tile's row pieces are whole
// elements, 16-byte aligned and multiples of 16 bytes, and so is the pitch.
// Every mbarrier wait is bounded; a CTA that gives up marks the call's
// status, raises the abort flag and returns once its copies have landed.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile(
        "{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_addr(bar))
        : "memory");
}

// Waits for phase `parity` of the barrier to complete, at most `limit`
// probes; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, uint32_t limit) {
    const uint32_t a = smem_addr(bar);
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done = 0;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void bulk_load(void* sdst, const void* gsrc, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_addr(sdst)),
        "l"(gsrc), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

constexpr uint32_t kMbarWaitLimit = 1u << 22;  // try_wait probes before a slot-buffer wait gives up

// Warp 0 issues the bulk copies of item `it`'s slots into `buf`: slot ii
// holds the row piece of source row srow[ii].  Each lane announces the bytes
// of its own copies before issuing them; lane 0 arrives once every lane has.
template <typename I>
__device__ __forceinline__ void own_stage_bulk(const ColOwnArgs& a, const I* srow, uint8_t* buf, uint64_t it,
                                               uint32_t nstage, uint64_t* bar) {
    const unsigned lane = threadIdx.x & 31;
    const OwnItem ci = own_item(a, it);
    const unsigned piece = ci.tcols * a.w;
    unsigned mine = 0;
    for (uint32_t ii = lane; ii < nstage; ii += 32)
        if (srow[ii] < static_cast<I>(a.rows)) mine += piece;
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // earlier generic reads of buf come first
    if (mine) mbar_expect_tx(bar, mine);
    for (uint32_t ii = lane; ii < nstage; ii += 32) {
        const I gr = srow[ii];
        if (!in_range(gr, a.rows, a.status)) continue;
        bulk_load(buf + ii * a.pitch, ci.mat + static_cast<uint64_t>(gr) * a.row_bytes, piece, bar);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(bar);
}

template <int US, typename Own, bool kLanes>
__global__ void __launch_bounds__(kThreads) k_col_group_bulk(ColOwnArgs a, Own own, GroupSync gs) {
    using I = typename Own::index_type;
    extern __shared__ __align__(128) uint8_t smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int s_ok;
    const unsigned grp = blockIdx.x / gs.G, r = blockIdx.x - grp * gs.G;
    if (grp >= gs.nG) return;  // never launched: the grid is nG * G CTAs
    unsigned* ctr = gs.counters + grp;
    unsigned* abort_flag = gs.counters + gs.nG;
    const uint32_t x0 = r * a.Q;
    const uint32_t myrows = x0 < a.rows ? min(a.Q, a.rows - x0) : 0;
    const uint32_t nstage = myrows ? myrows + a.Hlo + a.Hhi : 0;
    I* srow = reinterpret_cast<I*>(smem + 2 * a.buf_bytes);
    I* wrow = srow + (a.Q + a.Hlo + a.Hhi);
    uint32_t lc = 0, lu = 0, ii0 = 0, step = 1;
    if constexpr (kLanes) {
        uint32_t lr;
        a.div_RU.divmod(threadIdx.x, ii0, lr);
        a.div_upw.divmod(lr, lc, lu);
        step = blockDim.x / a.RU;
    }
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    own_fill_stage_rows(a, own, srow, x0, nstage);
    __syncthreads();  // barriers initialised, source-row table filled
    const bool warp0 = threadIdx.x < 32;
    if (warp0 && grp < a.items) own_stage_bulk(a, srow, smem, grp, nstage, &bars[0]);
    uint32_t k = 0;
    int inflight = -1;  // buffer whose copies may still be in flight when the loop ends early
    for (uint64_t it = grp; it < a.items; it += gs.nG, ++k) {
        const uint32_t b = k & 1;
        const bool landed = __syncthreads_and(mbar_wait(&bars[b], (k >> 1) & 1, kMbarWaitLimit));
        if (!landed) {
            if (threadIdx.x == 0) {
                raise_status(gs.status, kCallSyncTimeout);
                atomicExch(abort_flag, 1u);
            }
            inflight = static_cast<int>(b);
            break;
        }
        if (threadIdx.x == 0 && gs.G > 1) group_arrive(ctr, gs.relaxed);
        const uint64_t nxt = it + gs.nG;
        // the other buffer was last read by the previous item's writes, which
        // every thread finished before the loop's closing barrier
        if (nxt < a.items && warp0) own_stage_bulk(a, srow, smem + (b ^ 1) * a.buf_bytes, nxt, nstage, &bars[b ^ 1]);
        const OwnItem ci = own_item(a, it);
        own_fill_write_rows(own, wrow, x0, myrows, ci.col0);  // while thread 0 waits
        if (threadIdx.x == 0)
            s_ok = gs.G <= 1 || group_wait(ctr, (k + 1) * gs.G, abort_flag, gs.sleep_ns, gs.spin_limit, gs.status);
        __syncthreads();  // every CTA of the group holds its slots: writes may start
        if (!s_ok) {
            if (nxt < a.items) inflight = static_cast<int>(b ^ 1);
            ++k;  // the in-flight buffer's use is item k + 1
            break;
        }
        own_write_rows_tab<US, Own, kLanes>(a, own, smem + b * a.buf_bytes, ci, wrow, myrows, nstage, lc, lu, ii0,
                                            step);
        __syncthreads();  // this CTA's threads are done with the buffer and the output rows
    }
    // no copy outlives the CTA: copies issued before an early exit land
    // before it returns (bounded); item k used buffer k & 1 at phase (k >> 1) & 1
    if (inflight >= 0) mbar_wait(&bars[inflight], (k >> 1) & 1, kMbarWaitLimit);
}

// Launch-time self-test of the bounded wait: one CTA waits on a counter
// that nothing increments and must give up, counting one sync timeout.
#ifndef EITHOT_UNIT
__global__ void k_wait_selftest(unsigned* counters) {
    if (threadIdx.x == 0) group_wait(counters, 1u, counters + 1, 256, kDefaultSpinLimit, nullptr);
}
#endif

// ---------------------------------------------------------------------------
// Grid-staged row / column passes for items larger than shared memory.
// Items [it0, it0 + n) are copied to scratch (item-major, natural layout
// for gathers, permuted layout for scatters) by k_*_stage_in, then written
// back by k_*_stage_out; each launch spreads all units over the grid.
// ---------------------------------------------------------------------------
struct StageRowArgs {
    uint8_t* base;
    unsigned* status;  // the call's status word
    uint8_t* scratch;
    uint64_t rows, cols, it0, n;
    StripGeom g;
    FastDiv div_rows, div_itemunits;  // itemunits = cols * upw
};

template <int US, typename Fn, bool kScatter, bool kIn>
__global__ void __launch_bounds__(kThreads) k_row_stage(StageRowArgs a, Fn fn) {
    using U = typename UnitOf<US>::T;
    const uint64_t item_units = a.cols * a.g.upw;
    const uint64_t total = a.n * item_units;
    const uint64_t row_bytes = a.cols * a.g.E;
    const uint64_t item_bytes = a.cols * a.g.w;
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < total;
         x += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t gi, rem, j, u;
        a.div_itemunits.divmod(x, gi, rem);
        a.g.div_upw.divmod(rem, j, u);
        uint64_t bi, s;
        a.g.div_strips.divmod(a.it0 + gi, bi, s);
        const uint64_t lim = (s + 1 == a.g.nstrips) ? a.g.last_upw : a.g.upw;
        if (u >= lim) continue;
        const uint64_t i = a.div_rows.mod(bi);
        uint8_t* row = a.base + bi * row_bytes + s * a.g.w;
        uint8_t* st = a.scratch + gi * item_bytes;
        if (kIn) {
            const uint64_t slot = kScatter ? fn(i, j) : j;
            if (!in_range(slot, a.cols, a.status)) continue;
            *reinterpret_cast<U*>(st + slot * a.g.w + u * US) =
                *reinterpret_cast<const U*>(row + j * a.g.E + u * US);
        } else {
            const uint64_t slot = kScatter ? j : fn(i, j);
            if (!in_range(slot, a.cols, a.status)) continue;
            *reinterpret_cast<U*>(row + j * a.g.E + u * US) =
                *reinterpret_cast<const U*>(st + slot * a.g.w + u * US);
        }
    }
}

struct StageColArgs {
    uint8_t* base;
    unsigned* status;  // the call's status word
    uint8_t* scratch;
    uint64_t rows, cols, tw, ntiles, it0, n;
    StripGeom g;
    FastDiv div_tiles, div_itemunits, div_rowunits;  // itemunits = rows*tw*upw
};

template <int US, typename Fn, bool kIn>
__global__ void __launch_bounds__(kThreads) k_col_stage(StageColArgs a, Fn fn) {
    using U = typename UnitOf<US>::T;
    const uint64_t rowunits = a.tw * a.g.upw;
    const uint64_t item_units = a.rows * rowunits;
    const uint64_t total = a.n * item_units;
    const uint64_t row_bytes = a.cols * a.g.E;
    const uint64_t mat_bytes = a.rows * row_bytes;
    const uint64_t spitch = a.tw * a.g.w;
    const uint64_t item_bytes = a.rows * spitch;
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < total;
         x += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t gi, rem, i, r2, c, u;
        a.div_itemunits.divmod(x, gi, rem);
        a.div_rowunits.divmod(rem, i, r2);
        a.g.div_upw.divmod(r2, c, u);
        uint64_t bt, s, b, t;
        a.g.div_strips.divmod(a.it0 + gi, bt, s);
        a.div_tiles.divmod(bt, b, t);
        const uint64_t col0 = t * a.tw;
        const uint64_t lim = (s + 1 == a.g.nstrips) ? a.g.last_upw : a.g.upw;
        if (col0 + c >= a.cols || u >= lim) continue;
        uint8_t* mat = a.base + b * mat_bytes + col0 * a.g.E + s * a.g.w;
        uint8_t* st = a.scratch + gi * item_bytes;
        if (kIn) {
            *reinterpret_cast<U*>(st + i * spitch + c * a.g.w + u * US) =
                *reinterpret_cast<const U*>(mat + i * row_bytes + c * a.g.E + u * US);
        } else {
            const uint64_t src = fn(i, col0 + c);
            if (!in_range(src, a.rows, a.status)) continue;
            *reinterpret_cast<U*>(mat + i * row_bytes + c * a.g.E + u * US) =
                *reinterpret_cast<const U*>(st + src * spitch + c * a.g.w + u * US);
        }
    }
}

// ---------------------------------------------------------------------------
// Block copy: blocks s in [s0, s0+count) of `blk` bytes move from
// src + s*sp to dst + s*dp.  The host guarantees that no destination of the
// launch overlaps a source of the launch.
// ---------------------------------------------------------------------------
struct BlockArgs {
    const uint8_t* src;
    uint8_t* dst;
    uint64_t blk, sp, dp, s0, count;
    FastDiv div_blkunits;
};

template <int US>
__global__ void __launch_bounds__(kThreads) k_block_copy(BlockArgs a) {
    using U = typename UnitOf<US>::T;
    const uint64_t bu = a.blk / US;
    const uint64_t total = a.count * bu;
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < total;
         x += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t k, u;
        a.div_blkunits.divmod(x, k, u);
        const uint64_t s = a.s0 + k;
        *reinterpret_cast<U*>(a.dst + s * a.dp + u * US) =
            *reinterpret_cast<const U*>(a.src + s * a.sp + u * US);
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

uint64_t pow2_div(uint64_t v) {
    uint64_t u = 1;
    while (u < 16 && v % (u * 2) == 0) u *= 2;
    return u;
}

uint64_t unit_for(std::initializer_list<uint64_t> vals) {
    uint64_t u = 16;
    for (uint64_t v : vals) u = std::min(u, pow2_div(v));
    return u;
}

StripGeom make_strips(uint64_t E, uint64_t w, uint64_t U, uint64_t outer, uint64_t extra_units_bound) {
    StripGeom g;
    g.E = E;
    g.w = w;
    g.nstrips = (E + w - 1) / w;
    g.upw = w / U;
    const uint64_t last = E - (g.nstrips - 1) * w;
    g.last_upw = last / U;
    g.div_upw = FastDiv::make(g.upw, extra_units_bound);
    g.div_strips = FastDiv::make(g.nstrips, outer * g.nstrips);
    return g;
}

// Launch-configuration queries are costly host calls (several us each) and
// their answers depend only on (device, kernel, shared memory, cluster
// size): they are made once and remembered.
struct LaunchKey {
    int dev;
    const void* kernel;
    size_t smem;
    int K;
    int kind;
    bool operator<(const LaunchKey& o) const {
        return std::tie(dev, kernel, smem, K, kind) < std::tie(o.dev, o.kernel, o.smem, o.K, o.kind);
    }
};
enum { kQuerySmemSet = 0, kQueryNonPortable = 1, kQueryBlocks = 2, kQueryClusters = 3 };

std::mutex g_launch_mu;
std::map<LaunchKey, int> g_launch_cache;

int current_device() {
    int dev = 0;
    cudaGetDevice(&dev);
    return dev;
}

bool cached(const LaunchKey& k, int* v) {
    std::lock_guard<std::mutex> lock(g_launch_mu);
    auto it = g_launch_cache.find(k);
    if (it == g_launch_cache.end()) return false;
    *v = it->second;
    return true;
}

void remember(const LaunchKey& k, int v) {
    std::lock_guard<std::mutex> lock(g_launch_mu);
    g_launch_cache[k] = v;
}

int grid_for(const void* kernel, size_t smem, uint64_t items, const ExecContext& ctx) {
    const LaunchKey key{current_device(), kernel, smem, 1, kQueryBlocks};
    int per_sm = 0;
    if (!cached(key, &per_sm)) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem);
        remember(key, per_sm);
    }
    if (per_sm < 1) per_sm = 1;
    const uint64_t cap = static_cast<uint64_t>(per_sm) * ctx.caps.sms;
    return static_cast<int>(std::max<uint64_t>(1, std::min<uint64_t>(items, cap)));
}

int grid_for_elems(uint64_t total, const ExecContext& ctx) {
    const uint64_t blocks = (total + kThreads - 1) / kThreads;
    const uint64_t cap = static_cast<uint64_t>(ctx.caps.sms) * 4;
    return static_cast<int>(std::max<uint64_t>(1, std::min<uint64_t>(blocks, cap)));
}

// Raises the kernel's dynamic shared-memory limit to at least `smem` (the
// largest value set so far on this device is remembered).
cudaError_t prep_smem(const void* kernel, size_t smem) {
    const LaunchKey key{current_device(), kernel, 0, 0, kQuerySmemSet};
    int have = -1;
    if (cached(key, &have) && static_cast<size_t>(have) >= smem) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(smem));
    if (e == cudaSuccess) remember(key, static_cast<int>(smem));
    return e;
}

// Launches `kernel` as clusters of K CTAs, as many clusters as can be
// resident at once (at most `items`).
template <typename... KArgs, typename... Args>
cudaError_t launch_clusters(void (*kernel)(KArgs...), int K, size_t smem, uint64_t items,
                            ExecContext& ctx, Args&&... args) {
    const void* kp = reinterpret_cast<const void*>(kernel);
    const int dev = current_device();
    cudaError_t e = prep_smem(kp, smem);
    if (e != cudaSuccess) return e;
    int flag = 0;
    if (K > 8 && !cached(LaunchKey{dev, kp, 0, 0, kQueryNonPortable}, &flag)) {
        e = cudaFuncSetAttribute(kp, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
        remember(LaunchKey{dev, kp, 0, 0, kQueryNonPortable}, 1);
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = K;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx.stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(K * 1024);
    const LaunchKey key{dev, kp, smem, K, kQueryClusters};
    int max_clusters = 0;
    if (!cached(key, &max_clusters)) {
        e = cudaOccupancyMaxActiveClusters(&max_clusters, kp, &cfg);
        if (e != cudaSuccess) return e;
        remember(key, max_clusters);
    }
    if (max_clusters < 1) return cudaErrorLaunchOutOfResources;
    const uint64_t nclusters = std::min<uint64_t>(items, static_cast<uint64_t>(max_clusters));
    cfg.gridDim = dim3(static_cast<unsigned>(nclusters * K));
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

#define EI_CHECK(expr)                                                    \
    do {                                                                  \
        cudaError_t e__ = (expr);                                         \
        if (e__ != cudaSuccess) {                                         \
            ctx.err = std::string(#expr) + ": " + cudaGetErrorString(e__); \
            return EITHOT_STATUS_CUDA;                                    \
        }                                                                 \
    } while (0)

// Rows larger than this leave no room for a second CTA or item buffer on
// the SM; they prefetch the next row into registers instead.
// Rows this short are staged k at a time (k = kRowBlockBytes / row bytes,
// at least kRowBlockMinRows) by k_row_block.
constexpr uint64_t kRowBlockBytes = 48 * 1024;
constexpr uint64_t kRowBlockMinRows = 8;
// Matrices this small are transposed k at a time by k_slab_pack.
constexpr uint64_t kSlabPackBytes = 64 * 1024;
constexpr uint64_t kSlabPackMinMats = 4;

// ---- slab ----------------------------------------------------------------
template <int US>
int launch_slab(uint8_t* data, const Pass& p, ExecContext& ctx) {
    const uint64_t mat_bytes = p.rows * p.cols * p.elem;
    if (mat_bytes * kSlabPackMinMats <= kSlabPackBytes && tuning().slab_pack) {  // whole matrices: any strip
        SlabPackArgs b;
        b.words = tuning().narrow_words != 0;
        b.base = data + p.offset;
        b.batches = p.batches;
        b.mat_bytes = mat_bytes;
        b.E = p.elem;
        b.k = static_cast<uint32_t>(kSlabPackBytes / mat_bytes);
        b.items = (p.batches + b.k - 1) / b.k;
        b.R = static_cast<uint32_t>(p.rows);
        b.C = static_cast<uint32_t>(p.cols);
        b.upw = static_cast<uint32_t>(p.elem / US);
        b.mat_units = b.R * b.C * b.upw;
        b.div_mat_units = FastDiv32::make(b.mat_units);
        b.div_upw = FastDiv32::make(b.upw);
        b.div_R = FastDiv32::make(b.R);
        b.vec16 = reinterpret_cast<uintptr_t>(b.base) % 16 == 0 && mat_bytes % 16 == 0;
        const size_t smem = (static_cast<size_t>(b.k) * mat_bytes + 127) / 128 * 128;
        constexpr int kPack = US < 4 ? 4 / US : 1;
        const uint64_t addr = reinterpret_cast<uintptr_t>(b.base);
        if (kPack > 1 && p.elem == US && addr % 4 == 0) {
            // items start on 4-byte boundaries: k * mat_bytes a multiple of 4
            const uint32_t q = mat_bytes % 4 == 0 ? 1 : mat_bytes % 2 == 0 ? 2 : 4;
            b.k = std::max<uint32_t>(q, b.k / q * q);
            b.items = (p.batches + b.k - 1) / b.k;
            const size_t smem4 = (static_cast<size_t>(b.k) * mat_bytes + 127) / 128 * 128;
            const void* k = reinterpret_cast<const void*>(&k_slab_pack<US, kPack>);
            EI_CHECK(prep_smem(k, smem4));
            const int grid = grid_for(k, smem4, b.items, ctx);
            k_slab_pack<US, kPack><<<grid, kThreads, smem4, ctx.stream>>>(b);
        } else {
            const void* k = reinterpret_cast<const void*>(&k_slab_pack<US, 1>);
            EI_CHECK(prep_smem(k, smem));
            const int grid = grid_for(k, smem, b.items, ctx);
            k_slab_pack<US, 1><<<grid, kThreads, smem, ctx.stream>>>(b);
        }
        EI_CHECK(cudaGetLastError());
        ctx.launches++;
        return 0;
    }
    if (tuning().slab2d_runs && p.strip == p.elem && (p.elem == 1 || p.elem == 2 || p.elem == 4 || p.elem == 8 ||
                                                      p.elem == 16) && (tuning().slab2d_runs == 2 || p.elem <= 2)) {
        // The matrices as slabs of dims (C, R) written back in the order
        // (R, C): the slab-permutation run kernel (whole 16-byte stores).
        Pass q = p;
        q.type = kSlabPerm;
        q.nd_dims = {p.cols, p.rows};
        q.nd_perm = {1, 0};
        const int rc = try_slab_runs_pass(data, q, ctx);
        if (rc >= 0) return rc;
    }
    SlabArgs a;
    a.base = data + p.offset;
    a.E = p.elem;
    a.mat_bytes = p.rows * p.cols * p.elem;
    a.R = static_cast<uint32_t>(p.rows);
    a.C = static_cast<uint32_t>(p.cols);
    a.w = static_cast<uint32_t>(p.strip);
    a.pitch = static_cast<uint32_t>(slab_pitch(p.cols, p.strip));
    a.upw = a.w / US;
    a.nstrips = static_cast<uint32_t>((p.elem + p.strip - 1) / p.strip);
    a.last_upw = static_cast<uint32_t>((p.elem - (a.nstrips - 1) * p.strip) / US);
    a.flat = (p.strip == p.elem);
    a.rowunits = a.C * a.upw;
    a.items = p.batches * a.nstrips;
    a.div_strips = FastDiv::make(a.nstrips, a.items);
    a.div_C = FastDiv32::make(a.C);
    a.div_R = FastDiv32::make(a.R);
    a.div_upw = FastDiv32::make(a.upw);
    a.div_rowunits = FastDiv32::make(a.rowunits);
    const size_t smem = slab_smem_bytes(p.rows, p.cols, p.strip);
    constexpr int kPack = US < 4 ? 4 / US : 1;
    const bool pack = kPack > 1 && a.flat && p.elem == US && a.nstrips == 1 &&
                      reinterpret_cast<uintptr_t>(a.base) % 4 == 0 && a.mat_bytes % 4 == 0;
    // strips of 16 bytes or more (word-aligned slots of w bytes in shared
    // memory) as pieces; whole elements through the flat word path
    a.words = US < 4 && !pack && std::min<uint64_t>(p.strip, p.elem) >= 16 && a.w % 4 == 0 && tuning().narrow_words;
    a.flat_words = US < 4 && !pack && !a.words && a.flat && tuning().narrow_words;
    a.div_E = FastDiv32::make(p.elem);
    a.div_rowb = FastDiv32::make(p.cols * p.elem);
    a.rowchunks = static_cast<uint32_t>((p.cols * p.elem + 15) / 16);
    a.div_rowchunks = FastDiv32::make(a.rowchunks);
    a.slots = (a.w + 15) / 16;
    a.div_slots = FastDiv32::make(a.slots);
    a.wslots = (a.w + 3) / 4 + 1;
    a.div_wslots = FastDiv32::make(a.wslots);
    const void* k = pack ? reinterpret_cast<const void*>(&k_slab<US, kPack>)
                         : reinterpret_cast<const void*>(&k_slab<US, 1>);
    EI_CHECK(prep_smem(k, smem));
    const int grid = grid_for(k, smem, a.items, ctx);
    if (pack)
        k_slab<US, kPack><<<grid, kThreads, smem, ctx.stream>>>(a);
    else
        k_slab<US, 1><<<grid, kThreads, smem, ctx.stream>>>(a);
    EI_CHECK(cudaGetLastError());
    ctx.launches++;
    return 0;
}

template <int US>
int launch_slab_cluster(uint8_t* data, const Pass& p, ExecContext& ctx) {
    if constexpr (US > 4) {  // staged rows sit at a pitch of odd 4-byte words
        ctx.err = "internal: cluster slab with a unit above 4 bytes";
        return EITHOT_STATUS_INVALID;
    } else {
    SlabClusterArgs a;
    a.base = data + p.offset;
    a.items = p.batches;
    a.row_bytes = p.cols * p.elem;
    a.mat_bytes = p.rows * a.row_bytes;
    a.R = static_cast<uint32_t>(p.rows);
    a.C = static_cast<uint32_t>(p.cols);
    a.E = static_cast<uint32_t>(p.elem);
    a.pitch = static_cast<uint32_t>(slab_cluster_pitch(a.row_bytes));
    const int K = p.cluster;
    a.upr = static_cast<uint32_t>(a.row_bytes / US);
    a.upw = static_cast<uint32_t>(p.elem / US);
    // pack 4/US elements to a 4-byte store when every store stays aligned
    constexpr int kPack = US < 4 ? 4 / US : 1;
    const uint64_t addr = reinterpret_cast<uintptr_t>(a.base);
    uint32_t Q = static_cast<uint32_t>((p.rows + K - 1) / K);
    const uint32_t Qp = (Q + kPack - 1) / kPack * kPack;  // bands start on a packed word
    const bool pack = kPack > 1 && p.elem == US && p.rows % kPack == 0 && addr % 4 == 0 && a.mat_bytes % 4 == 0 &&
                      static_cast<uint64_t>(Qp) * a.pitch + 127 <= smem_cap_of(ctx.caps);
    if (pack) Q = Qp;
    a.Q = Q;
    a.div_upr = FastDiv32::make(a.upr);
    a.div_upw = FastDiv32::make(a.upw);
    a.load4 = US < 4 && a.row_bytes % 4 == 0 && addr % 4 == 0;
    a.stage_words = US < 4 && !a.load4 && tuning().narrow_words;
    a.rowchunks = static_cast<uint32_t>((p.cols * p.elem + 15) / 16);
    a.div_rowchunks = FastDiv32::make(a.rowchunks);
    a.write_words = US < 4 && p.elem >= 16 && tuning().narrow_words;
    a.div_E = FastDiv32::make(p.elem);
    a.div_rowb = FastDiv32::make(a.row_bytes);
    a.wpr = static_cast<uint32_t>(a.row_bytes / 4);
    a.div_wpr = FastDiv32::make(a.wpr ? a.wpr : 1);
    a.div_Qupw = FastDiv32::make(static_cast<uint64_t>(Q) * a.upw);
    a.div_Qpack = FastDiv32::make(kPack > 1 ? Q / kPack : 1);
    const size_t smem = (static_cast<size_t>(Q) * a.pitch + 127) / 128 * 128;
    if (pack)
        EI_CHECK(launch_clusters(k_slab_cluster<US, kPack>, K, smem, a.items, ctx, a));
    else
        EI_CHECK(launch_clusters(k_slab_cluster<US, 1>, K, smem, a.items, ctx, a));
    EI_CHECK(cudaGetLastError());
    ctx.launches++;
    return 0;
    }
}

// ---- rows ------------------------------------------------------------------

template <int US, typename Fn, bool kScatter>
int launch_row_staged(uint8_t* data, const Pass& p, const Staging& st, ExecContext& ctx, const Fn& fn);

template <int US, typename FnOnChip, typename Fn64, bool kScatter>
int launch_row(uint8_t* data, const Pass& p, const FnOnChip& fn, const Fn64& fn64, ExecContext& ctx) {
    const size_t cap = smem_cap_of(ctx.caps);
    const Staging st = plan_row_staging(p.cols, p.elem, cap, kScatter);
    if (!st.on_chip) return launch_row_staged<US, Fn64, kScatter>(data, p, st, ctx, fn64);
    if constexpr (!kScatter) {
        const uint64_t row_bytes = p.cols * p.elem;
        if (row_bytes * kRowBlockMinRows <= kRowBlockBytes && tuning().row_block) {  // whole rows: any strip
            RowBlockArgs b;
            b.words = tuning().narrow_words != 0;
            b.status = ctx.status;
            b.base = data + p.offset;
            b.total_rows = p.batches * p.rows;
            b.row_bytes = row_bytes;
            b.E = p.elem;
            b.k = static_cast<uint32_t>(kRowBlockBytes / row_bytes);
            b.items = (b.total_rows + b.k - 1) / b.k;
            b.cols = static_cast<uint32_t>(p.cols);
            b.upw = static_cast<uint32_t>(p.elem / US);
            b.units_per_row = b.cols * b.upw;
            b.div_rows = FastDiv::make(p.rows, b.total_rows);
            b.div_units_row = FastDiv32::make(b.units_per_row);
            b.div_upw = FastDiv32::make(b.upw);
            b.vec16 = reinterpret_cast<uintptr_t>(b.base) % 16 == 0 && row_bytes % 16 == 0;
            const size_t smem = (static_cast<size_t>(b.k) * row_bytes + 127) / 128 * 128;
            const void* k = reinterpret_cast<const void*>(&k_row_block<US, FnOnChip>);
            EI_CHECK(prep_smem(k, smem));
            const int grid = grid_for(k, smem, b.items, ctx);
            k_row_block<US, FnOnChip><<<grid, kThreads, smem, ctx.stream>>>(b, fn);
            EI_CHECK(cudaGetLastError());
            ctx.launches++;
            return 0;
        }
    }
    RowArgs a;
    a.words = tuning().narrow_words != 0;
    a.status = ctx.status;
    a.base = data + p.offset;
    a.E = p.elem;
    a.row_bytes = p.cols * p.elem;
    a.rows = static_cast<uint32_t>(p.rows);
    a.cols = static_cast<uint32_t>(p.cols);
    a.w = static_cast<uint32_t>(st.w);
    a.upw = a.w / US;
    a.nstrips = static_cast<uint32_t>((p.elem + st.w - 1) / st.w);
    a.last_upw = static_cast<uint32_t>((p.elem - (a.nstrips - 1) * st.w) / US);
    a.flat = (st.w == p.elem);
    a.P = static_cast<uint32_t>((p.cols + st.K - 1) / st.K);
    a.items = p.batches * p.rows * a.nstrips;
    a.div_strips = FastDiv::make(a.nstrips, a.items);
    a.div_rows = FastDiv::make(p.rows, p.batches * p.rows);
    a.div_upw = FastDiv32::make(a.upw);
    a.div_P = FastDiv32::make(a.P);
    a.buf_bytes = static_cast<uint32_t>((static_cast<uint64_t>(a.P) * st.w + 127) / 128 * 128);
    a.dbuf = st.dbuf;
    const size_t smem = (st.dbuf ? 2 : 1) * static_cast<size_t>(a.buf_bytes);
    constexpr int kRegs = 256 / US;  // 64 registers of prefetched data per thread
    if constexpr (US >= 4 && !kScatter) {
        const uint64_t units = static_cast<uint64_t>(a.cols) * a.upw;
        if (st.K == 1 && !st.dbuf && a.flat && a.nstrips == 1 &&
            smem > static_cast<size_t>(tuning().row_solo_kb) * 1024 &&
            units <= static_cast<uint64_t>(kRegs) * kThreads && tuning().row_prefetch) {
            const void* k = reinterpret_cast<const void*>(&k_row_solo<US, FnOnChip, kRegs>);
            EI_CHECK(prep_smem(k, smem));
            const int grid = grid_for(k, smem, a.items, ctx);
            k_row_solo<US, FnOnChip, kRegs><<<grid, kThreads, smem, ctx.stream>>>(a, fn);
            EI_CHECK(cudaGetLastError());
            ctx.launches++;
            return 0;
        }
    }
    EI_CHECK(launch_clusters(k_row_cluster<US, FnOnChip, kScatter>, st.K, smem, a.items, ctx, a, fn));
    EI_CHECK(cudaGetLastError());
    ctx.launches++;
    return 0;
}

template <int US, typename Fn, bool kScatter>
int launch_row_staged(uint8_t* data, const Pass& p, const Staging& st, ExecContext& ctx, const Fn& fn) {
    const uint64_t upw = st.w / US;
    const StripGeom g = make_strips(p.elem, st.w, US, p.batches * p.rows, p.cols * upw);
    const uint64_t items = p.batches * p.rows * g.nstrips;
    const uint64_t item_bytes = p.cols * st.w;
    if (ctx.scratch_bytes < item_bytes || ctx.scratch == nullptr) {
        ctx.err = "workspace too small for a staged row pass";
        return EITHOT_STATUS_NOMEM;
    }
    const uint64_t per_group = std::max<uint64_t>(1, ctx.scratch_bytes / item_bytes);
    StageRowArgs a;
    a.status = ctx.status;
    a.base = data + p.offset;
    a.scratch = ctx.scratch;
    a.rows = p.rows; a.cols = p.cols;
    a.g = g;
    a.div_rows = FastDiv::make(p.rows, p.batches * p.rows);
    a.div_itemunits = FastDiv::make(p.cols * upw, per_group * p.cols * upw);
    for (uint64_t it0 = 0; it0 < items; it0 += per_group) {
        a.it0 = it0;
        a.n = std::min<uint64_t>(per_group, items - it0);
        const int grid = grid_for_elems(a.n * p.cols * upw, ctx);
        k_row_stage<US, Fn, kScatter, true><<<grid, kThreads, 0, ctx.stream>>>(a, fn);
        k_row_stage<US, Fn, kScatter, false><<<grid, kThreads, 0, ctx.stream>>>(a, fn);
        EI_CHECK(cudaGetLastError());
        ctx.launches += 2;
    }
    return 0;
}

// ---- columns ---------------------------------------------------------------
template <int US, typename Fn>
int launch_col_staged(uint8_t* data, const Pass& p, const Staging& st, ExecContext& ctx, const Fn& fn) {
    const uint64_t upw = st.w / US;
    const uint64_t ntiles = (p.cols + st.tw - 1) / st.tw;
    const StripGeom g = make_strips(p.elem, st.w, US, p.batches * ntiles, p.rows * st.tw * upw);
    const uint64_t items = p.batches * ntiles * g.nstrips;
    const uint64_t item_bytes = p.rows * st.tw * st.w;
    if (ctx.scratch_bytes < item_bytes || ctx.scratch == nullptr) {
        ctx.err = "workspace too small for a staged column pass";
        return EITHOT_STATUS_NOMEM;
    }
    const uint64_t per_group = std::max<uint64_t>(1, ctx.scratch_bytes / item_bytes);
    StageColArgs a;
    a.status = ctx.status;
    a.base = data + p.offset;
    a.scratch = ctx.scratch;
    a.rows = p.rows; a.cols = p.cols; a.tw = st.tw; a.ntiles = ntiles;
    a.g = g;
    a.div_tiles = FastDiv::make(ntiles, p.batches * ntiles);
    const uint64_t item_units = p.rows * st.tw * upw;
    a.div_itemunits = FastDiv::make(item_units, per_group * item_units);
    a.div_rowunits = FastDiv::make(st.tw * upw, item_units);
    for (uint64_t it0 = 0; it0 < items; it0 += per_group) {
        a.it0 = it0;
        a.n = std::min<uint64_t>(per_group, items - it0);
        const int grid = grid_for_elems(a.n * item_units, ctx);
        k_col_stage<US, Fn, true><<<grid, kThreads, 0, ctx.stream>>>(a, fn);
        k_col_stage<US, Fn, false><<<grid, kThreads, 0, ctx.stream>>>(a, fn);
        EI_CHECK(cudaGetLastError());
        ctx.launches += 2;
    }
    return 0;
}

template <int US, typename FnOnChip, typename Fn64>
int launch_col(uint8_t* data, const Pass& p, const FnOnChip& fn, const Fn64& fn64, ExecContext& ctx) {
    const size_t cap = smem_cap_of(ctx.caps);
    const Staging st = plan_col_staging(p.rows, p.elem, cap, p.cols);
    if (!st.on_chip) return launch_col_staged<US, Fn64>(data, p, st, ctx, fn64);
    ColArgs a;
    a.status = ctx.status;
    a.base = data + p.offset;
    a.E = p.elem;
    a.row_bytes = p.cols * p.elem;
    a.mat_bytes = p.rows * a.row_bytes;
    a.rows = static_cast<uint32_t>(p.rows);
    a.cols = static_cast<uint32_t>(p.cols);
    a.tw = static_cast<uint32_t>(st.tw);
    a.ntiles = static_cast<uint32_t>((p.cols + st.tw - 1) / st.tw);
    a.pitch = static_cast<uint32_t>(st.pitch);
    a.w = static_cast<uint32_t>(st.w);
    a.upw = a.w / US;
    a.nstrips = static_cast<uint32_t>((p.elem + st.w - 1) / st.w);
    a.last_upw = static_cast<uint32_t>((p.elem - (a.nstrips - 1) * st.w) / US);
    a.RU = a.tw * a.upw;
    a.Q = static_cast<uint32_t>((p.rows + st.K - 1) / st.K);
    a.items = p.batches * a.ntiles * a.nstrips;
    a.div_strips = FastDiv::make(a.nstrips, a.items);
    a.div_tiles = FastDiv::make(a.ntiles, p.batches * a.ntiles);
    a.div_RU = FastDiv32::make(a.RU);
    a.div_upw = FastDiv32::make(a.upw);
    a.div_Q = FastDiv32::make(a.Q);
    a.buf_bytes = static_cast<uint32_t>((static_cast<uint64_t>(a.Q) * st.pitch + 127) / 128 * 128);
    a.dbuf = st.dbuf;
    const size_t smem = (st.dbuf ? 2 : 1) * static_cast<size_t>(a.buf_bytes);
    if (kThreads % a.RU != 0)
        EI_CHECK(launch_clusters(k_col_cluster<US, FnOnChip, false, 4>, st.K, smem, a.items, ctx, a, fn));
    else if (tuning().col_batch >= 8)
        EI_CHECK(launch_clusters(k_col_cluster<US, FnOnChip, true, 8>, st.K, smem, a.items, ctx, a, fn));
    else
        EI_CHECK(launch_clusters(k_col_cluster<US, FnOnChip, true, 4>, st.K, smem, a.items, ctx, a, fn));
    EI_CHECK(cudaGetLastError());
    ctx.launches++;
    return 0;
}

// launch_col_group's answer when the device holds fewer co-resident CTAs
// than the group form was planned for (the caller plans again without it).
constexpr int kRetryWithoutGroups = -2;

ColOwnArgs col_owner_args(uint8_t* data, const Pass& p, const Staging& st, int US, unsigned* status) {
    ColOwnArgs a;
    a.status = status;
    a.base = data + p.offset;
    a.E = p.elem;
    a.row_bytes = p.cols * p.elem;
    a.mat_bytes = p.rows * a.row_bytes;
    a.rows = static_cast<uint32_t>(p.rows);
    a.cols = static_cast<uint32_t>(p.cols);
    a.tw = static_cast<uint32_t>(st.tw);
    a.ntiles = static_cast<uint32_t>((p.cols + st.tw - 1) / st.tw);
    a.pitch = static_cast<uint32_t>(st.pitch);
    a.w = static_cast<uint32_t>(st.w);
    a.upw = a.w / US;
    a.nstrips = static_cast<uint32_t>((p.elem + st.w - 1) / st.w);
    a.last_upw = static_cast<uint32_t>((p.elem - (a.nstrips - 1) * st.w) / US);
    a.RU = a.tw * a.upw;
    const uint64_t parts = st.group ? static_cast<uint64_t>(st.G) : static_cast<uint64_t>(st.K);
    a.Q = static_cast<uint32_t>((p.rows + parts - 1) / parts);
    a.Hlo = static_cast<uint32_t>(st.hlo);
    a.Hhi = static_cast<uint32_t>(st.hhi);
    a.hbase = static_cast<uint32_t>((p.rows - st.hlo % p.rows) % p.rows);
    a.whole = st.whole;
    a.dofs = st.whole ? static_cast<uint32_t>((st.tw / p.rows + 1) * p.rows) : 0;
    a.items = p.batches * a.ntiles * a.nstrips;
    a.div_strips = FastDiv::make(a.nstrips, a.items);
    a.div_tiles = FastDiv::make(a.ntiles, p.batches * a.ntiles);
    a.div_RU = FastDiv32::make(a.RU);
    a.div_upw = FastDiv32::make(a.upw);
    a.div_m = FastDiv32::make(p.rows);
    const uint64_t slots = static_cast<uint64_t>(a.Q) + a.Hlo + a.Hhi;
    a.buf_bytes = static_cast<uint32_t>((slots * st.pitch + 127) / 128 * 128);
    a.dbuf = st.dbuf;
    a.stage_words = US < 4 && a.nstrips == 1 && a.w == a.E && tuning().narrow_words;
    a.wpp = static_cast<uint32_t>((a.tw * a.E + 15) / 16 + 1);
    a.div_wpp = FastDiv32::make(a.wpp);
    return a;
}

// Shared memory of the row tables behind an owner-computed pass's slot
// buffer(s): Q + Hlo + Hhi source rows and Q output rows.
template <typename Own>
size_t owner_table_bytes(const ColOwnArgs& a) {
    const size_t bytes = (2 * static_cast<size_t>(a.Q) + a.Hlo + a.Hhi) * sizeof(typename Own::index_type);
    return (bytes + 15) / 16 * 16;
}

template <int US, typename Own>
int launch_col_owner(uint8_t* data, const Pass& p, const Staging& st, const Own& own, ExecContext& ctx) {
    const ColOwnArgs a = col_owner_args(data, p, st, US, ctx.status);
    const size_t smem = (st.dbuf ? 2 : 1) * static_cast<size_t>(a.buf_bytes) + owner_table_bytes<Own>(a);
    if (kThreads % a.RU != 0)
        EI_CHECK(launch_clusters(k_col_owner<US, Own, false>, st.K, smem, a.items, ctx, a, own));
    else
        EI_CHECK(launch_clusters(k_col_owner<US, Own, true>, st.K, smem, a.items, ctx, a, own));
    EI_CHECK(cudaGetLastError());
    ctx.launches++;
    return 0;
}

// Cooperative launch of nG groups of G CTAs, nG as large as residency
// allows (at most one group per item, at most max_groups).
template <typename Own>
cudaError_t launch_groups(void (*kernel)(ColOwnArgs, Own, GroupSync), size_t smem, const ColOwnArgs& a,
                          const Own& own, GroupSync gs, unsigned max_groups, ExecContext& ctx) {
    const void* kp = reinterpret_cast<const void*>(kernel);
    // the cooperative launch checks co-residency against the kernel's
    // shared-memory limit, so the limit is this launch's size exactly
    cudaError_t e = cudaFuncSetAttribute(kp, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    remember(LaunchKey{current_device(), kp, 0, 0, kQuerySmemSet}, static_cast<int>(smem));
    const LaunchKey key{current_device(), kp, smem, 1, kQueryBlocks};
    int per_sm = 0;
    if (!cached(key, &per_sm)) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kp, kThreads, smem);
        if (e != cudaSuccess) return e;
        remember(key, per_sm);
    }
    const uint64_t resident = static_cast<uint64_t>(per_sm) * ctx.caps.sms;
    ctx.group_per_sm_seen = per_sm;
    if (resident < gs.G) return cudaErrorCooperativeLaunchTooLarge;
    gs.nG = static_cast<unsigned>(std::min<uint64_t>({a.items, resident / gs.G, static_cast<uint64_t>(max_groups)}));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx.stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(gs.nG * gs.G);
    return cudaLaunchKernelEx(&cfg, kernel, a, own, gs);
}

// Group-synchronised passes never overlap on the device, whichever streams
// or threads issue them: each one waits for an event recorded after the
// previous one on that device.  Two of them in flight at once could each hold
// part of the SMs while waiting for CTAs of their own that cannot be placed;
// ordered, each waits only for kernels that finish on their own.  (A stream
// being captured into a graph is not ordered this way: the batched form,
// which captures, never uses group passes.)
}  // namespace
// One chain per process, shared by every unit's object (defined in the
// host-side object).
extern std::mutex g_chain_mu;
extern std::map<int, cudaEvent_t> g_chain;  // device -> event after its last group pass
namespace {

class GroupChain {
public:
    explicit GroupChain(cudaStream_t stream) : lock_(g_chain_mu), stream_(stream) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess) {
            cudaGetLastError();
            cs = cudaStreamCaptureStatusNone;
        }
        capturing_ = cs != cudaStreamCaptureStatusNone;
    }
    // Makes the stream wait for the previous group pass on this device.
    cudaError_t before() {
        if (capturing_) return cudaSuccess;
        dev_ = current_device();
        auto it = g_chain.find(dev_);
        if (it == g_chain.end()) return cudaSuccess;
        cudaError_t e = cudaStreamWaitEvent(stream_, it->second, 0);
        if (e == cudaErrorInvalidResourceHandle) {  // the device was reset since: start a new chain
            cudaGetLastError();
            g_chain.erase(it);
            return cudaSuccess;
        }
        return e;
    }
    // Records the end of this group pass as the next one's predecessor.
    cudaError_t after() {
        if (capturing_) return cudaSuccess;
        auto it = g_chain.find(dev_);
        if (it == g_chain.end()) {
            cudaEvent_t ev = nullptr;
            const cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
            if (e != cudaSuccess) return e;
            it = g_chain.emplace(dev_, ev).first;
        }
        return cudaEventRecord(it->second, stream_);
    }

private:
    std::lock_guard<std::mutex> lock_;
    cudaStream_t stream_;
    bool capturing_ = false;
    int dev_ = 0;
};

// A double-buffered group pass stages its slots with bulk copies when every
// row piece is whole elements, 16-byte aligned and a multiple of 16 bytes
// (so is the slot pitch) and the knob allows it.
template <int US>
bool bulk_ok(const ColOwnArgs& a, const Staging& st) {
    if constexpr (US < 16) {  // instantiated for 16-byte units only (fewer kernels to load)
        return false;
    } else {
        return st.dbuf && st.bulk && tuning().col_bulk && a.nstrips == 1 && a.w == a.E && a.pitch % 16 == 0 &&
               a.row_bytes % 16 == 0 && reinterpret_cast<uintptr_t>(a.base) % 16 == 0;
    }
}

template <int US, typename Own>
int launch_col_group(uint8_t* data, const Pass& p, const Staging& st, const Own& own, ExecContext& ctx) {
    const ColOwnArgs a = col_owner_args(data, p, st, US, ctx.status);
    const size_t smem = (st.dbuf ? 2 : 1) * static_cast<size_t>(a.buf_bytes) + owner_table_bytes<Own>(a);
    if (ctx.scratch == nullptr || ctx.scratch_bytes < kGroupSyncBytes) {
        ctx.err = "workspace too small for a group-synchronised column pass";
        return EITHOT_STATUS_NOMEM;
    }
    GroupSync gs;
    gs.counters = reinterpret_cast<unsigned*>(ctx.scratch);
    gs.G = static_cast<unsigned>(st.G);
    gs.nG = 0;
    gs.status = ctx.status;
    gs.spin_limit = static_cast<unsigned>(tuning().sync_spin_limit);
    gs.sleep_ns = static_cast<unsigned>(tuning().sync_sleep_ns);
    gs.relaxed = tuning().sync_relaxed != 0;
    gs.l2_prefetch = tuning().l2_prefetch != 0;
    const unsigned max_groups = static_cast<unsigned>(kGroupSyncBytes / sizeof(unsigned)) - 1;
    EI_CHECK(cudaMemsetAsync(ctx.scratch, 0, kGroupSyncBytes, ctx.stream));  // counters and abort flag
    GroupChain chain(ctx.stream);
    EI_CHECK(chain.before());
    cudaError_t e;
    bool bulk = false;
    if constexpr (US == 16) {
        if (bulk_ok<US>(a, st)) {
            bulk = true;
            e = kThreads % a.RU != 0 ? launch_groups(k_col_group_bulk<US, Own, false>, smem, a, own, gs, max_groups, ctx)
                                     : launch_groups(k_col_group_bulk<US, Own, true>, smem, a, own, gs, max_groups, ctx);
        }
    }
    if (!bulk)
        e = kThreads % a.RU != 0 ? launch_groups(k_col_group<US, Own, false>, smem, a, own, gs, max_groups, ctx)
                                 : launch_groups(k_col_group<US, Own, true>, smem, a, own, gs, max_groups, ctx);
    if (e == cudaErrorCooperativeLaunchTooLarge) {  // fewer CTAs resident than planned: no group form
        cudaGetLastError();
        return kRetryWithoutGroups;
    }
    EI_CHECK(e);
    EI_CHECK(cudaGetLastError());
    EI_CHECK(chain.after());
    ctx.launches++;
    return 0;
}

// ---- block moves -------------------------------------------------------------
constexpr uint64_t kBlockPieceMin = 4ull << 20;  // smallest scratch for a block move, bytes
template <int US>
int copy_blocks(const uint8_t* src, uint8_t* dst, uint64_t blk, uint64_t sp, uint64_t dp,
                uint64_t s0, uint64_t count, ExecContext& ctx) {
    if (count == 0 || blk == 0) return 0;
    BlockArgs a;
    a.src = src; a.dst = dst; a.blk = blk; a.sp = sp; a.dp = dp; a.s0 = s0; a.count = count;
    a.div_blkunits = FastDiv::make(blk / US, count * (blk / US));
    const int grid = grid_for_elems(count * (blk / US), ctx);
    k_block_copy<US><<<grid, kThreads, 0, ctx.stream>>>(a);
    EI_CHECK(cudaGetLastError());
    ctx.launches++;
    return 0;
}

// Moves blocks s = 1..n-1 (block 0 never moves) from s*sp to s*dp in place.
// Spreading (dp > sp) proceeds from the last block down, compacting from
// the first block up, so a launch never overwrites a block that has not
// been moved yet; a launch whose blocks would overlap themselves goes
// through scratch.
template <int US>
int block_move(uint8_t* data, const Pass& p, ExecContext& ctx) {
    const uint64_t n = p.n_blocks, blk = p.block, sp = p.src_pitch, dp = p.dst_pitch;
    if (n <= 1 || sp == dp) return 0;
    const uint64_t scratch_blocks = ctx.scratch ? ctx.scratch_bytes / blk : 0;
    int rc;
    // One block through scratch smaller than the block: in pieces, from the
    // end moved towards first (front to back when moving down, back to front
    // when moving up), so a piece's destination covers only pieces already
    // moved and the piece itself, which is in scratch by then.
    auto piecewise = [&](uint64_t b) -> int {
        const uint64_t S = ctx.scratch ? ctx.scratch_bytes / US * US : 0;
        if (S == 0) { ctx.err = "workspace too small for padding"; return EITHOT_STATUS_NOMEM; }
        const uint64_t pieces = (blk + S - 1) / S;
        for (uint64_t k = 0; k < pieces; ++k) {
            const uint64_t idx = dp < sp ? k : pieces - 1 - k;
            const uint64_t off = idx * S, len = std::min<uint64_t>(S, blk - off);
            int r;
            if ((r = copy_blocks<US>(data + b * sp + off, ctx.scratch, len, 0, 0, 0, 1, ctx))) return r;
            if ((r = copy_blocks<US>(ctx.scratch, data + b * dp + off, len, 0, 0, 0, 1, ctx))) return r;
        }
        return 0;
    };
    if (dp > sp) {
        uint64_t s = n - 1;  // highest block not yet moved
        while (s >= 1) {
            if (s * (dp - sp) >= blk) {
                // blocks [lo, s] whose destinations lie above every source among them
                uint64_t lo = (s * sp + blk + dp - 1) / dp;
                lo = std::max<uint64_t>(1, std::min(lo, s));
                if ((rc = copy_blocks<US>(data, data, blk, sp, dp, lo, s - lo + 1, ctx))) return rc;
                s = lo - 1;
            } else {
                if (scratch_blocks == 0) {
                    if ((rc = piecewise(s))) return rc;
                    --s;
                    continue;
                }
                const uint64_t lo = s + 1 > scratch_blocks ? std::max<uint64_t>(1, s + 1 - scratch_blocks) : 1;
                const uint64_t cnt = s - lo + 1;
                if ((rc = copy_blocks<US>(data + lo * sp, ctx.scratch, blk, sp, blk, 0, cnt, ctx))) return rc;
                if ((rc = copy_blocks<US>(ctx.scratch, data + lo * dp, blk, blk, dp, 0, cnt, ctx))) return rc;
                s = lo - 1;
            }
        }
    } else {
        uint64_t s = 1;  // lowest block not yet moved
        while (s < n) {
            if (s * (sp - dp) >= blk) {
                // blocks [s, hi) whose destinations all lie below the lowest
                // source among them: (hi-1)*dp + blk <= s*sp
                uint64_t hi = (s * sp - blk) / dp + 1;
                hi = std::min<uint64_t>(std::max<uint64_t>(hi, s + 1), n);
                if ((rc = copy_blocks<US>(data, data, blk, sp, dp, s, hi - s, ctx))) return rc;
                s = hi;
            } else {
                if (scratch_blocks == 0) {
                    if ((rc = piecewise(s))) return rc;
                    ++s;
                    continue;
                }
                const uint64_t cnt = std::min<uint64_t>(scratch_blocks, n - s);
                if ((rc = copy_blocks<US>(data + s * sp, ctx.scratch, blk, sp, blk, 0, cnt, ctx))) return rc;
                if ((rc = copy_blocks<US>(ctx.scratch, data + s * dp, blk, blk, dp, 0, cnt, ctx))) return rc;
                s += cnt;
            }
        }
    }
    return 0;
}

// ---- dispatch ------------------------------------------------------------------
template <int US, template <typename> class FnT, typename Make32, typename Make64, typename Own32, typename Own64>
int run_col(uint8_t* data, const Pass& p, ExecContext& ctx, Make32 m32, Make64 m64, Own32 o32, Own64 o64) {
    const Staging st = plan_col_pass(p, ctx.caps);
    if (st.owner && st.group) {
        const int rc = fits32(p) ? launch_col_group<US>(data, p, st, o32(p), ctx)
                                 : launch_col_group<US>(data, p, st, o64(p), ctx);
        if (rc != kRetryWithoutGroups) return rc;
        const int seen = ctx.group_per_sm_seen;
        if (seen >= 1 && seen < 4 && tuning().group_per_sm != seen) {
            // plan the groups again for the residency this kernel really has
            Tuning t = tuning();
            t.group_per_sm = seen;
            t.col_form = 2;
            ScopedTuning scope(t);
            const Staging again = plan_col_pass(p, ctx.caps);
            if (again.on_chip && again.group) return run_col<US, FnT>(data, p, ctx, m32, m64, o32, o64);
        }
        Tuning t = tuning();  // plan the pass again without groups, if its scratch fits
        t.col_form = 1;
        ScopedTuning scope(t);
        const Staging alt = plan_col_pass(p, ctx.caps);
        if (!alt.on_chip && ctx.scratch_bytes < p.rows * alt.tw * alt.w) {
            ctx.err = "fewer CTAs co-resident than the group column pass needs, and too little workspace "
                      "for the staged form";
            return EITHOT_STATUS_CUDA;
        }
        return run_col<US, FnT>(data, p, ctx, m32, m64, o32, o64);
    }
    if (st.owner) {
        if (fits32(p)) return launch_col_owner<US>(data, p, st, o32(p), ctx);
        return launch_col_owner<US>(data, p, st, o64(p), ctx);
    }
    const FnT<uint64_t> f64 = m64(p);
    if (fits32(p)) return launch_col<US>(data, p, m32(p), f64, ctx);
    return launch_col<US>(data, p, f64, f64, ctx);
}

template <int US>
int run_pass_u(uint8_t* data, const Pass& p, ExecContext& ctx) {
    switch (p.type) {
        case kSlabTranspose: return launch_slab<US>(data, p, ctx);
        case kSlabCluster:
            if (p.band) {
                const int rc = run_slab_colband(data, p, ctx);
                if (rc >= 0) return rc;
            }
            return launch_slab_cluster<US>(data, p, ctx);
        case kRowGather:
        case kRowScatter: {
            // A row pass is run as a gather when one CTA holds the whole row
            // (cp.async loads, local gathers) or when it moves wide granules;
            // otherwise as a scatter (remote pushes beat remote pulls for
            // 16-32 byte granules).  The inverse map turns one into the other.
            const Staging st = plan_row_staging(p.cols, p.elem, smem_cap_of(ctx.caps), p.type == kRowScatter);
            const bool gather = !st.on_chip || st.K == 1 || st.w >= 64;
            const bool use_inverse = gather == (p.type == kRowScatter);
            if (!st.on_chip) {  // staged: keep the pass's own direction
                const FnRowShuffleT<uint64_t> f64 = make_rowshuffle<uint64_t>(p);
                return p.type == kRowScatter
                           ? launch_row<US, FnRowShuffleT<uint64_t>, FnRowShuffleT<uint64_t>, true>(data, p, f64, f64, ctx)
                           : launch_row<US, FnRowShuffleT<uint64_t>, FnRowShuffleT<uint64_t>, false>(data, p, f64, f64, ctx);
            }
            if (use_inverse) {
                const FnRowShuffleInvT<uint64_t> h64 = make_rowshuffle_inv<uint64_t>(p);
                if (fits32(p)) {
                    const FnRowShuffleInvT<uint32_t> h32 = make_rowshuffle_inv<uint32_t>(p);
                    return gather ? launch_row<US, FnRowShuffleInvT<uint32_t>, FnRowShuffleInvT<uint64_t>, false>(data, p, h32, h64, ctx)
                                  : launch_row<US, FnRowShuffleInvT<uint32_t>, FnRowShuffleInvT<uint64_t>, true>(data, p, h32, h64, ctx);
                }
                return gather ? launch_row<US, FnRowShuffleInvT<uint64_t>, FnRowShuffleInvT<uint64_t>, false>(data, p, h64, h64, ctx)
                              : launch_row<US, FnRowShuffleInvT<uint64_t>, FnRowShuffleInvT<uint64_t>, true>(data, p, h64, h64, ctx);
            }
            const FnRowShuffleT<uint64_t> f64 = make_rowshuffle<uint64_t>(p);
            if (fits32(p)) {
                const FnRowShuffleT<uint32_t> f32 = make_rowshuffle<uint32_t>(p);
                return gather ? launch_row<US, FnRowShuffleT<uint32_t>, FnRowShuffleT<uint64_t>, false>(data, p, f32, f64, ctx)
                              : launch_row<US, FnRowShuffleT<uint32_t>, FnRowShuffleT<uint64_t>, true>(data, p, f32, f64, ctx);
            }
            return gather ? launch_row<US, FnRowShuffleT<uint64_t>, FnRowShuffleT<uint64_t>, false>(data, p, f64, f64, ctx)
                          : launch_row<US, FnRowShuffleT<uint64_t>, FnRowShuffleT<uint64_t>, true>(data, p, f64, f64, ctx);
        }
        case kColGather:
            switch (p.fn) {
                case kFnC2RPreRot:
                    return run_col<US, FnC2RPreRotT>(data, p, ctx, make_prerot<uint32_t>, make_prerot<uint64_t>,
                                                     make_owner_prerot<uint32_t>, make_owner_prerot<uint64_t>);
                case kFnC2RColShuffle:
                    return run_col<US, FnC2RColShuffleT>(data, p, ctx, make_c2r_colshuf<uint32_t>, make_c2r_colshuf<uint64_t>,
                                                         make_owner_colshuf<uint32_t>, make_owner_colshuf<uint64_t>);
                case kFnR2CColShuffle:
                    return run_col<US, FnR2CColShuffleT>(data, p, ctx, make_r2c_colshuf<uint32_t>, make_r2c_colshuf<uint64_t>,
                                                         make_owner_r2c_colshuf<uint32_t>, make_owner_r2c_colshuf<uint64_t>);
                case kFnR2CPostRot:
                    return run_col<US, FnR2CPostRotT>(data, p, ctx, make_postrot<uint32_t>, make_postrot<uint64_t>,
                                                      make_owner_postrot<uint32_t>, make_owner_postrot<uint64_t>);
                default: break;
            }
            break;
        case kBlockMove: return block_move<US>(data, p, ctx);
        default: break;
    }
    ctx.err = "internal: unknown pass";
    return EITHOT_STATUS_INVALID;
}

uint64_t pass_unit(const uint8_t* data, const Pass& p, const DeviceCaps& caps) {
    const size_t smem_cap = smem_cap_of(caps);
    const uint64_t addr = reinterpret_cast<uintptr_t>(data) + p.offset;
    switch (p.type) {
        case kSlabTranspose:
            return unit_for({addr, p.elem, p.strip, p.elem % p.strip == 0 ? p.strip : p.elem % p.strip});
        case kSlabCluster:  // staged rows sit at a pitch of odd 4-byte words
            return unit_for({addr, p.elem, 4});
        case kRowGather:
        case kRowScatter: {
            const Staging st = plan_row_staging(p.cols, p.elem, smem_cap, p.type == kRowScatter);
            return unit_for({addr, p.elem, st.w, p.elem % st.w == 0 ? st.w : p.elem % st.w});
        }
        case kColGather: {
            const Staging st = plan_col_pass(p, caps);
            return unit_for({addr, p.elem, st.w, st.pitch, p.elem % st.w == 0 ? st.w : p.elem % st.w});
        }
        case kBlockMove:
            return unit_for({addr, p.block, p.src_pitch, p.dst_pitch});
        default:
            return 1;
    }
}

}  // namespace

// Reads and clears this object's counter `which` (0: index faults, 1: sync
// timeouts).
static int read_counter(int which, unsigned int* out) {
    unsigned int v = 0, zero = 0;
    cudaError_t e = which == 0 ? cudaMemcpyFromSymbol(&v, g_index_faults, sizeof(v))
                               : cudaMemcpyFromSymbol(&v, g_sync_timeouts, sizeof(v));
    if (e == cudaSuccess)
        e = which == 0 ? cudaMemcpyToSymbol(g_index_faults, &zero, sizeof(zero))
                       : cudaMemcpyToSymbol(g_sync_timeouts, &zero, sizeof(zero));
    *out = v;
    return e == cudaSuccess ? 0 : EITHOT_STATUS_CUDA;
}

#define EITHOT_CAT2(a, b) a##b
#define EITHOT_CAT(a, b) EITHOT_CAT2(a, b)

#ifdef EITHOT_UNIT

int EITHOT_CAT(run_pass_unit_, EITHOT_UNIT)(uint8_t* data, const Pass& p, ExecContext& ctx) {
    return run_pass_u<EITHOT_UNIT>(data, p, ctx);
}

int EITHOT_CAT(read_unit_counter_, EITHOT_UNIT)(int which, unsigned int* out) { return read_counter(which, out); }

#else  // the host-side executor

std::mutex g_chain_mu;
std::map<int, cudaEvent_t> g_chain;

#define EITHOT_UNIT_DECL(U)                                                          \
    int run_pass_unit_##U(uint8_t* data, const Pass& p, ExecContext& ctx); \
    int read_unit_counter_##U(int which, unsigned int* out);
EITHOT_UNIT_DECL(1)
EITHOT_UNIT_DECL(2)
EITHOT_UNIT_DECL(4)
EITHOT_UNIT_DECL(8)
EITHOT_UNIT_DECL(16)

// Sums and clears counter `which` over this object and every unit's (reading
// a unit's counter loads that unit's device module).
static int read_all_counters(int which, unsigned int* out) {
    unsigned int total = 0, v = 0;
    int rc = read_counter(which, &v);
    total += v;
    int (*const readers[])(int, unsigned int*) = {read_unit_counter_1, read_unit_counter_2, read_unit_counter_4,
                                                   read_unit_counter_8, read_unit_counter_16};
    for (auto* rd : readers) {
        v = 0;
        if (const int r = rd(which, &v)) rc = r;
        total += v;
    }
    *out = total;
    return rc;
}


size_t pass_workspace_bytes(const Pass& p, const DeviceCaps& caps) {
    const size_t cap = smem_cap_of(caps);
    switch (p.type) {
        case kBlockPerm:
            return block_perm_workspace(p, false);
        case kRowGather:
        case kRowScatter: {
            const Staging st = plan_row_staging(p.cols, p.elem, cap, p.type == kRowScatter);
            return st.on_chip ? 0 : p.cols * st.w;
        }
        case kColGather: {
            const Staging st = plan_col_pass(p, caps);
            if (st.on_chip) return st.group ? kGroupSyncBytes : 0;
            return p.rows * st.tw * st.w;
        }
        case kBlockMove: {
            // scratch is needed only where a block's shift is smaller than
            // the block itself
            const uint64_t sh = p.dst_pitch > p.src_pitch ? p.dst_pitch - p.src_pitch : p.src_pitch - p.dst_pitch;
            if (p.n_blocks <= 1 || sh == 0) return 0;
            // blocks larger than this move through scratch in pieces
            return sh >= p.block ? 0 : std::min<uint64_t>(p.block, kBlockPieceMin);
        }
        default:
            return 0;
    }
}

size_t pass_workspace_ideal(const Pass& p, const DeviceCaps& caps) {
    const size_t cap = smem_cap_of(caps);
    switch (p.type) {
        case kBlockPerm:
            return block_perm_workspace(p, true);
        case kRowGather:
        case kRowScatter: {
            const Staging st = plan_row_staging(p.cols, p.elem, cap, p.type == kRowScatter);
            if (st.on_chip) return 0;
            const uint64_t ns = (p.elem + st.w - 1) / st.w;
            return p.batches * p.rows * ns * p.cols * st.w;
        }
        case kColGather: {
            const Staging st = plan_col_pass(p, caps);
            if (st.on_chip) return st.group ? kGroupSyncBytes : 0;
            const uint64_t ns = (p.elem + st.w - 1) / st.w;
            const uint64_t nt = (p.cols + st.tw - 1) / st.tw;
            return p.batches * nt * ns * p.rows * st.tw * st.w;
        }
        case kBlockMove:
            return pass_workspace_bytes(p, caps) ? p.block * std::max<uint64_t>(1, p.n_blocks - 1) : 0;
        default:
            return 0;
    }
}

int run_passes(uint8_t* data, const std::vector<Pass>& passes, ExecContext& ctx) {
    // Profiling appends one event before the first pass and one after each
    // pass to the caller's pool; pass k spans events (first + k, first + k + 1).
    size_t ev = ctx.profile ? ctx.events_used : 0;
    auto record = [&]() -> int {
        if (!ctx.profile) return 0;
        if (ev == ctx.events->size()) {
            cudaEvent_t e;
            EI_CHECK(cudaEventCreate(&e));
            ctx.events->push_back(e);
        }
        EI_CHECK(cudaEventRecord((*ctx.events)[ev++], ctx.stream));
        return 0;
    };
    if (ctx.profile) {
        if (int rc = record()) return rc;
    }
    for (const Pass& p : passes) {
        int rc;
        if (p.type == kSlabPerm) {
            rc = run_slab_perm(data, p, ctx);
        } else if (p.type == kBlockPerm) {
            rc = run_block_perm(data, p, ctx);
        } else {
            const uint64_t U = pass_unit(data, p, ctx.caps);
            switch (U) {
                case 16: rc = run_pass_unit_16(data, p, ctx); break;
                case 8: rc = run_pass_unit_8(data, p, ctx); break;
                case 4: rc = run_pass_unit_4(data, p, ctx); break;
                case 2: rc = run_pass_unit_2(data, p, ctx); break;
                default: rc = run_pass_unit_1(data, p, ctx); break;
            }
        }
        if (rc) return rc;
        ctx.passes++;
        if (ctx.profile) {
            if ((rc = record())) return rc;
            ctx.spans->push_back({ev - 2, ev - 1});
            ctx.names->push_back(p.what);
            const double moved = p.type == kBlockMove
                ? 2.0 * static_cast<double>(p.block) * static_cast<double>(p.n_blocks > 0 ? p.n_blocks - 1 : 0)
                : 2.0 * static_cast<double>(p.batches) * p.rows * p.cols * p.elem;
            ctx.bytes->push_back(moved);
        }
    }
    if (ctx.profile) ctx.events_used = ev;
    return 0;
}

int read_index_faults(unsigned int* out) { return read_all_counters(0, out); }

int read_sync_timeouts(unsigned int* out) { return read_all_counters(1, out); }

int run_wait_selftest(unsigned int* timeouts, std::string* err) {
    unsigned int pending = 0;  // timeouts of earlier launches are cleared, not reported here
    if (read_sync_timeouts(&pending)) { *err = "reading the sync-timeout counter failed"; return EITHOT_STATUS_CUDA; }
    unsigned* flags = nullptr;
    cudaError_t e = cudaMalloc(&flags, 2 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(flags, 0, 2 * sizeof(unsigned));
    if (e == cudaSuccess) {
        k_wait_selftest<<<1, 32>>>(flags);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (flags) cudaFree(flags);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return EITHOT_STATUS_CUDA; }
    if (read_sync_timeouts(timeouts)) { *err = "reading the sync-timeout counter failed"; return EITHOT_STATUS_CUDA; }
    return 0;
}

bool query_caps(int device, DeviceCaps* caps, std::string* err) {
    static std::mutex mu;
    static std::vector<std::pair<int, DeviceCaps>> cache;
    std::lock_guard<std::mutex> lock(mu);
    for (auto& e : cache) if (e.first == device) { *caps = e.second; return true; }
    DeviceCaps c;
    int v = 0;
    cudaError_t e = cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return false; }
    c.sms = v;
    e = cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return false; }
    c.smem_optin = static_cast<size_t>(v);
    e = cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return false; }
    c.smem_per_sm = static_cast<size_t>(v);
    cache.emplace_back(device, c);
    *caps = c;
    return true;
}

#endif  // EITHOT_UNIT

}  // namespace eithot
