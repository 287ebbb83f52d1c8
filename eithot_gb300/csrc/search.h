// Pass-minimising plans: a search over sequences of single-pass and
// Catanzaro moves, scored by the lowering's cost model, as an alternative to
// the reference's pre/post/mixed series.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "passes.h"

namespace eithot {

// Modelled time of a pass list in units of one streaming pass over the
// passes' data (the lowering's cost model; new pass kinds included).
double passes_model_cost(const std::vector<Pass>& passes, const DeviceCaps& caps);

// Searches the cheapest sequence of moves that permutes the tensor (dims,
// 1-based perm, elem bytes, one tensor, no sub-tensors) and lowers it to
// passes.  Moves: any batched 2D transpose of adjacent axis groups (lowered
// as today: slab, cluster slab, Catanzaro or factor split); an on-chip
// permutation of a slab of leading axes into the target's order (the
// reference's row linearisations _3214 and 5D _43215, generalised); a
// permutation of blocks of leading axes by following its cycles (the
// reference's column linearisations _1432, _14325, _15432, generalised).
// Returns false when the tensor needs no device pass or the search gave up;
// *cost and *desc describe the plan found.
bool search_plan(const std::vector<int64_t>& dims, const std::vector<int>& perm1, uint64_t elem,
                 const DeviceCaps& caps, std::vector<Pass>* passes, double* cost, std::string* desc);

// Smallest block (bytes) a cycle-following block permutation moves.
constexpr uint64_t kMinCycleBlock = 4096;

// Shortest chain one segment of a cycle-following pass walks, and the most
// segments one cycle is cut into (longer cycles get longer segments).
constexpr uint64_t kCycleSegment = 128;
constexpr uint64_t kMaxCycleSegments = 4096;

// Shared memory (bytes) one CTA may use to stage a slab permutation.
uint64_t slab_perm_capacity(const DeviceCaps& caps);

// Strip width of a slab permutation of `count` elements of E bytes.
uint64_t slab_perm_strip(uint64_t E, uint64_t count, const DeviceCaps& caps);

// Cycle segments of a block permutation (blocks indexed by `dims`, block
// at input index s moves to output index dst(s), output axis j = input axis
// perm[j]): segment k walks from head[k] (whose block is saved first) for
// len[k] steps and ends at tail[k], the next segment's head.  Computed once
// per shape and kept.
struct CycleTable {
    std::vector<uint64_t> head, tail, len;
    std::vector<uint64_t> cycle_first;  // first segment of every cycle, then the segment count
    uint64_t moved = 0;                 // blocks that move (not fixed points)
    uint64_t max_cycle_segments = 0;    // segments of the longest cycle
};
const CycleTable& cycle_table(const std::vector<uint64_t>& dims, const std::vector<int>& perm);

}  // namespace eithot
