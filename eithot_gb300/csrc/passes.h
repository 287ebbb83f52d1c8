// Device passes: the lowering of an N-d plan into in-place data movements.
//
// Every low-order transpose of the series, and the partition / join steps,
// is a batched in-place transpose X(B, R, C, E): B contiguous R x C
// row-major matrices of E-byte elements each become C x R.  X is executed
// either as one "slab" pass (each matrix staged whole on chip) or as the
// two/three Catanzaro passes (c2r on the R x C view or r2c on the C x R
// view).  Padding steps are block moves.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "plan.h"

namespace eithot {

enum PassType {
    kSlabTranspose = 0,  // each of B matrices (R x C) transposed on chip
    kRowGather = 1,      // out[i][j] = in[i][f(i,j)]
    kRowScatter = 2,     // out[i][f(i,j)] = in[i][j]
    kColGather = 3,      // out[i][j] = in[g(i,j)][j]
    kBlockMove = 4,      // n_blocks blocks of `block` bytes: s*src_pitch -> s*dst_pitch
    kSlabCluster = 5,    // each of B matrices (R x C) transposed by a K-CTA cluster, owner-computed
    kSlabPerm = 6,       // each of B slabs (axes nd_dims, elements of `elem` bytes) permuted on chip by nd_perm
    kBlockPerm = 7,      // blocks of `block` bytes, indexed by axes nd_dims, permuted by nd_perm along its cycles
};

enum FnType {
    kFnNone = 0,
    kFnRowShuffle = 1,
    kFnC2RPreRot = 2,
    kFnC2RColShuffle = 3,
    kFnR2CColShuffle = 4,
    kFnR2CPostRot = 5,
};

struct Pass {
    int type = kSlabTranspose;
    int fn = kFnNone;
    uint64_t offset = 0;                 // byte offset of the first batch
    uint64_t batches = 1, rows = 1, cols = 1, elem = 1;
    // Catanzaro parameters of the view (m rows x n cols)
    uint64_t m = 0, n = 0, c = 1, k = 0, a = 0, b = 0, q = 0;
    uint64_t strip = 0;                  // slab passes: strip width in bytes
    int cluster = 1;                     // kSlabCluster: CTAs per matrix
    uint64_t band = 0;                   // kSlabCluster: 0 row bands; else columns per CTA (column bands)
    // block moves
    uint64_t block = 0, n_blocks = 0, src_pitch = 0, dst_pitch = 0;
    // slab and block permutations: the permuted axes (fastest first) and the
    // output order (output axis j is input axis nd_perm[j])
    std::vector<uint64_t> nd_dims;
    std::vector<int> nd_perm;
    std::string what;
};

// One batched in-place transpose.
struct Xpose {
    uint64_t offset = 0, B = 1, R = 1, C = 1, E = 1;
};

// Device resources the lowering and the executor size against.
struct DeviceCaps {
    int sms = 152;
    size_t smem_optin = 232448;      // max dynamic shared memory per block (227 KiB)
    size_t smem_per_sm = 233472;
    int max_cluster = 8;             // portable cluster size
};

// Shared memory the single-CTA kernels may use per block.
size_t smem_cap_of(const DeviceCaps& caps);

// Process-wide tuning of the lowering (set through eithot_tune_set; the
// autotuner fills these per shape).
struct Tuning {
    int max_cluster = 16;  // largest thread-block cluster used
    int variant = 0;       // 0: cost model, 1: force c2r, 2: force r2c
    int dbuf = 1;          // allow double-buffered cluster items
    int col_batch = 4;     // remote loads in flight per thread in column passes (4 or 8)
    int col_chunk = 0;     // 0: cost model; 32/64/128: bytes per staged row piece of column passes
    int col_owner = 1;     // column passes: 1 owner-computed writes, 0 gathers through distributed smem
    int col_form = 0;      // owner-computed column passes: 0 cost model, 1 clusters, 2 CTA groups
    int row_prefetch = 1;  // rows filling a CTA: prefetch the next row into registers
    int row_block = 1;     // short rows: stage blocks of consecutive rows per CTA item
    int slab_pack = 1;     // small matrices: transpose blocks of consecutive matrices per CTA item
    int slab_cluster = 1;  // matrices beyond one CTA's share: one owner-computed pass over a cluster
    int factor = 1;        // split a transpose along a factor of R or C when a pass would stage globally
    int sync_sleep_ns = 64;  // group barriers: back-off between polls
    int sync_spin_limit = 1 << 20;  // group barriers: polls before a wait gives up (>= ~0.5 s)
    int sync_relaxed = 1;    // group barriers: arrive without release semantics (every load of the
                             // arriving CTA has landed in shared memory before it arrives)
    int group_per_sm = 0;    // group form: 0 cost model, 1 or 2 CTAs per SM
    int l2_prefetch = 0;     // group form, single-buffered: prefetch the next item into L2 (slower on GB300)
    int cycle_moves = 1;     // fewest-pass plans may move blocks along cycles (host-built segment tables):
                             // 0 no, 1 cost model, 2 preferred
    int slab_perm = 1;       // fewest-pass plans: 0 no slab permutations, 1 cost model, 2 preferred
    int slab_runs = 1;       // slab permutations of 1-16 byte elements: runs of outputs per thread, padded rows
                             // (1: runs whose outputs share offsets read them from a host table, runs that
                             // wrap the fastest output axis once step it with one jump; 2: every run steps
                             // through the axes element by element)
    int slab_prefetch = 1;   // slab permutations at one CTA per SM: the next slab prefetched into registers
    int slab_colband = 256;  // cluster slabs whose row bands give output rows fewer bytes per CTA than this
                             // write column bands (contiguous output ranges); 0 never
    int narrow_words = 1;    // contiguous ranges of 1- and 2-byte units are staged from aligned 4-byte words
    int row_solo_kb = 48;    // rows held by one CTA above this many KB run one CTA per SM with the next
                             // row prefetched into registers (up to 128 KB), smaller ones two or more per SM
                             // (96 KB rows of 32-byte elements: 6.18 TB/s against 4.81 at two per SM)
    int slab2d_runs = 1;     // slab transposes of whole elements beyond the packed sizes through the slab-
                             // permutation run kernel: 0 never, 1 elements of 1-2 bytes, 2 of 1-16 bytes
    int col_bulk = 0;        // group form: double-buffered CTAs staging their slots with bulk copies (slower on GB300)
    int batch_graph = 1;     // batched form: a run repeating the previous run's buffers replays a CUDA graph
    int batch_queue = 1;     // batched form: small tensors permuted by one persistent launch over a device queue
    int batch_lanes = 16;    // batched form: internal streams the other tensors are spread over (1..64)
};
Tuning& tuning();

// Knobs recorded for one exact request shape (dims, 1-based perm, element
// size), e.g. by an autotuner; looked up by the single-tensor entry points.
bool shape_tuning(const std::vector<int64_t>& dims, const std::vector<int>& perm, uint64_t elem, Tuning* out);
void set_shape_tuning(const std::vector<int64_t>& dims, const std::vector<int>& perm, uint64_t elem, const Tuning& t);
void clear_shape_tuning();
int shape_tuning_count();

// Makes tuning() return `t` on the calling thread for the scope's lifetime
// (the batched form lowers and runs its passes under its own knobs).
class ScopedTuning {
public:
    explicit ScopedTuning(const Tuning& t);
    ~ScopedTuning();
    ScopedTuning(const ScopedTuning&) = delete;
    ScopedTuning& operator=(const ScopedTuning&) = delete;

private:
    Tuning t_;
    Tuning* prev_;
};

// How one item of a row or column pass is staged.  A row item is one strip
// (w bytes of every element) of one row; a column item is one strip of a
// tile of `tw` adjacent columns over all rows.  An item is split over the K
// CTAs of a thread-block cluster (K <= 16) and staged in their distributed
// shared memory; items too large even for that are staged in global scratch.
struct Staging {
    uint64_t w = 0;        // strip width in bytes
    uint64_t tw = 1;       // columns per item (column passes)
    uint64_t pitch = 0;    // bytes per staged row (column passes)
    uint64_t item_bytes = 0;
    int K = 1;             // CTAs of the thread-block cluster sharing one item
    uint64_t per_cta = 0;  // shared-memory bytes each CTA stages per item
    bool dbuf = false;     // two item buffers per CTA (next item's loads overlap)
    bool on_chip = false;  // the item fits the cluster's distributed shared memory
    bool owner = false;    // column pass run owner-computed (each CTA writes from its own rows)
    uint64_t hlo = 0, hhi = 0;  // owner-computed: halo rows staged below / above the owned ones
    bool bulk = false;     // group form staged by bulk copies (whole-element 16-byte pieces, double-buffered)
    bool group = false;    // owner-computed over a group of G co-resident CTAs (global-memory
    int G = 0;             //   barrier, any size) instead of a thread-block cluster
    int per_sm = 1;        // CTAs per SM the footprint was sized for
    bool whole = false;    // owner-computed, one CTA holds every row of a tile (short columns)
    double cost = 0;       // modelled time in units of one streaming pass
};

// scatter: the row pass pushes elements to their destinations (r2c);
// otherwise it pulls them (c2r).
Staging plan_row_staging(uint64_t cols, uint64_t E, size_t smem_cap, bool scatter = false);
// cols: the matrix's column count (0: unknown); a tile never spans more.
Staging plan_col_staging(uint64_t rows, uint64_t E, size_t smem_cap, uint64_t cols = 0);

// Rows of halo an owner-computed column tile of tw columns needs below (lo)
// and above (hi) its owned rows for column map `fn` (b = n / gcd(m, n)).
void owner_halo(int fn, uint64_t b, uint64_t tw, uint64_t* lo, uint64_t* hi);

// Staging of column pass `p` (fn, rows, elem, b): owner-computed when the
// tuning allows and the tile fits on chip, else plan_col_staging's.
Staging plan_col_pass(const Pass& p, const DeviceCaps& caps);

// Bytes at the start of the workspace that group-synchronised passes use
// for their barrier counters.
constexpr size_t kGroupSyncBytes = 4096;

// Default number of polls before a group-barrier wait gives up.
constexpr unsigned kDefaultSpinLimit = 1u << 20;

// Lowers every step of `plan` for element size `elem` into passes.
bool lower_plan(const NdPlan& plan, uint64_t elem, const DeviceCaps& caps,
                std::vector<Pass>* passes, std::string* err);

// Lowers one batched transpose (exposed for tests).
void lower_xpose(const Xpose& x, const DeviceCaps& caps, std::vector<Pass>* passes);

// Modelled time of the passes lower_xpose emits for x, in streaming passes.
double xpose_cost(const Xpose& x, const DeviceCaps& caps);

// Modelled time of a list of slab, row and column passes (the lowering's
// own cost model), in streaming passes.
double passes_cost_of(const std::vector<Pass>& passes, const DeviceCaps& caps);

// Maps one low-order op acting on `n_sub` back-to-back sub-tensors onto a
// batched transpose.
Xpose xpose_of(const LowOp& op, uint64_t elem, uint64_t n_sub, uint64_t base_offset);

// Extended Euclid: gcd and the inverse of a mod b (0 when b == 1).
void gcd_inverse(uint64_t a, uint64_t b, uint64_t* g, uint64_t* inv);

// Slab transposes stage an R x C matrix of w-byte pieces with a padded row
// pitch so that the transposed reads hit distinct banks.
uint64_t slab_pitch(uint64_t C, uint64_t w);
size_t slab_smem_bytes(uint64_t R, uint64_t C, uint64_t w);
// Row pitch (bytes) of a cluster slab's staged rows of row_bytes each.
uint64_t slab_cluster_pitch(uint64_t row_bytes);

// Strip width (bytes) for elements of E bytes when `count` elements are
// staged together: whole elements up to 128 B; wider elements in strips of
// a multiple of 128 B, as wide as keeps count * strip within `budget`
// (few, very wide elements move in long contiguous strips).
constexpr uint64_t kWideStripBytes = 32 * 1024;
uint64_t strip_width(uint64_t E, uint64_t count, uint64_t budget);

}  // namespace eithot
