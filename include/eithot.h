/*
 * eithot.h — C ABI of the GB300 (sm_103a) in-place high-order tensor transposer.
 *
 * Layout convention (identical to EITHOT): a tensor of rank r with dims
 * (d0, d1, ..., d{r-1}) is stored with d0 the fastest-varying axis
 * (stride 1), d1 next, and so on (ITNT/src/Nd_transpose.cpp:53-59,
 * ITNT/src/tensor_util.cpp:27-29).  A permutation p (1-based at this ABI,
 * as on the reference's command line, ITNT/src/test_inplace.cpp:142-158)
 * produces the tensor whose output axis j is input axis p[j]-1; output
 * dims are (d{p0-1}, d{p1-1}, ...).
 *
 * Every entry point returns an int status (EITHOT_OK on success) and never
 * exits the process; eithot_last_error() returns a message for the calling
 * thread's most recent failure.  Device work is issued on the caller's
 * stream (a cudaStream_t passed as void*; NULL = legacy default stream) and
 * is stream-ordered: no entry point synchronises the device except where
 * stated.
 */
#ifndef EITHOT_H_
#define EITHOT_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define EITHOT_OK            0
#define EITHOT_EINVAL        1  /* bad dims / perm / element size / capacity */
#define EITHOT_ENOMEM        2  /* workspace could not be allocated or is too small */
#define EITHOT_ETIMEOUT      3  /* a bounded device wait gave up */
#define EITHOT_ECUDA         4  /* a CUDA runtime call failed */
#define EITHOT_EUNSUPPORTED  5  /* valid request outside what this build handles */
#define EITHOT_EBUSY         6  /* admission refused (served form) */
#define EITHOT_EFAULT        7  /* a kernel found an index-map result outside its row or column */

/* ---- REORDER_TYPE (ITNT/src/Nd_transpose.cpp:22-28) ------------------- */
#define EITHOT_ORDER_MIXED   0  /* reference default: fewer non-linearized rounds wins, tie -> post */
#define EITHOT_ORDER_PRE     1
#define EITHOT_ORDER_POST    2
/* No reference counterpart: the plan with the fewest modelled device passes,
 * searched over batched 2D transposes, on-chip slab permutations and
 * cycle-following block permutations (the reference's unwired 4D/5D
 * single-pass linearisations, generalised); the reference's mixed series
 * when the search finds nothing clearly cheaper, and always for tensors
 * split into sub-tensors. */
#define EITHOT_ORDER_FEWEST  3

/* ---- step roles in a plan --------------------------------------------- */
#define EITHOT_STEP_ROUND     0  /* one low-order transpose of the series */
#define EITHOT_STEP_PARTITION 1  /* NdPartition: 132 linearisation (ITNT/src/Nd_decompose.cpp:49-56) */
#define EITHOT_STEP_JOIN      2  /* NdJoin (ITNT/src/Nd_decompose.cpp:66-82) */
#define EITHOT_STEP_PAD_PRE   3  /* Nd_padding_pre_process (ITNT/src/Nd_padding.cu:103-161) */
#define EITHOT_STEP_PAD_POST  4  /* Nd_padding_post_process (ITNT/src/Nd_padding.cu:169-223) */

/* One low-order step of a plan.  For ROUND/PARTITION/JOIN, `code` is the
 * decimal-encoded 1-based low-order permutation (21, 132, 213, 231, 312,
 * 1324) exactly as the reference's Low_order_transpose switch reads it
 * (ITNT/src/Nd_transpose.cpp:62-99) and dims/perm describe that low-order
 * tensor.  A ROUND step applies to every sub-tensor (`num_sub_tensors` of
 * them, contiguous, `sub_tensor_elems` elements each).  For PAD steps,
 * dims[0] = decomposed-dim position, dims[1] = original size, dims[2] =
 * padded size. */
typedef struct eithot_step {
    int     role;
    int     code;
    int     rank;
    int     perm[4];
    int64_t dims[4];
} eithot_step;

typedef struct eithot_plan_info {
    int     order_used;        /* EITHOT_ORDER_PRE or EITHOT_ORDER_POST */
    int     num_sub_tensors;   /* applied (forced to 1 below the 32/alpha gate) */
    int     decompose_dim;     /* -1 when the tensor is not partitioned */
    int     padded;            /* 1 when the decomposed dim is padded */
    int64_t padded_dim_size;
    int64_t volume;            /* elements of the tensor */
    int64_t padded_volume;     /* elements while padded (== volume if not) */
    int64_t sub_tensor_elems;
    int     n_steps;           /* total steps (may exceed max_steps passed in) */
} eithot_plan_info;

/* Execution statistics of the last eithot_transpose* call on this thread. */
typedef struct eithot_stats {
    size_t  workspace_bytes;   /* device scratch the call used */
    size_t  free_before;       /* cudaMemGetInfo free bytes at entry (0 unless profiling is on) */
    size_t  free_after_alloc;  /* cudaMemGetInfo free bytes once scratch was allocated (idem) */
    int     n_passes;          /* device passes launched (excl. no-ops) */
    int     n_launches;        /* kernel launches issued */
    double  algorithmic_bytes; /* 2 * volume * elem_size */
} eithot_stats;

/* ---- planning (host only, no GPU needed) ------------------------------ */

/* Replaces the planning half of _Nd::transpose / Series_Low_order_transpose
 * (ITNT/src/Nd_transpose.cpp:160-304, permutation_util.cpp:300-374): the
 * same pre/post/mixed decomposition, sub-tensor gate (max dim > 32/alpha and
 * nb > 1) and padding decision, in 64-bit arithmetic.  Writes up to
 * max_steps steps; info->n_steps reports the full count. */
int eithot_plan(int rank, const int64_t* dims, const int* perm_1based,
                int num_sub_tensors, double alpha, int reorder_type,
                eithot_plan_info* info, eithot_step* steps, int max_steps);

/* ---- the transpose ---------------------------------------------------- */

/* Replaces inplace::transpose (ITNT/include/transpose.h:8,
 * ITNT/src/transpose.cpp:21-30).  In-place permutation of the tensor at
 * d_data.  elem_size in {1,2,4,8} (the reference accepts 4 and 8 only).
 * capacity_bytes is the size of the caller's buffer: when the plan pads the
 * decomposed dim (nb > 1, dim % nb != 0) the padded tensor must fit, exactly
 * as the reference requires caller slack (ITNT/src/test_inplace.cpp:11,22).
 * Scratch is taken from the stream-ordered allocator (cudaMallocAsync) and
 * bounded by alpha * bytes where the tensor is large enough for that bound
 * to hold; the call returns before the device work completes. */
int eithot_transpose(void* d_data, size_t capacity_bytes, int rank,
                     const int64_t* dims, const int* perm_1based,
                     size_t elem_size, int num_sub_tensors, double alpha,
                     void* stream);

/* As eithot_transpose with an explicit REORDER_TYPE and an optional
 * caller-owned workspace (d_workspace may be NULL: the library allocates).
 * When a workspace is given it must hold eithot_workspace_size() bytes. */
int eithot_transpose_ex(void* d_data, size_t capacity_bytes, int rank,
                        const int64_t* dims, const int* perm_1based,
                        size_t elem_size, int num_sub_tensors, double alpha,
                        int reorder_type, void* d_workspace,
                        size_t workspace_bytes, void* stream);

/* No counterpart in the reference (whose kernels allocate managed temporaries
 * per pass).  As eithot_transpose, but it allocates nothing: the scratch the
 * staged passes and the padding moves need comes from a fixed 32 MiB device
 * array inside the library.  The array sits in a device module of its own:
 * under CUDA's default lazy module loading a GPU holds it from the first
 * eithot_transpose_noalloc call there until the process exits (with
 * CUDA_MODULE_LOADING=EAGER, from when the library's device code is loaded,
 * as for every module).  For callers that may not allocate device memory
 * during the call, e.g. because another allocator owns the device's memory.
 * Requests needing more than 32 MiB of scratch fail with EITHOT_EINVAL.  Each
 * call looks up the array's address on the current device (no allocation;
 * the first lookup on a device may load the library's device code, so make
 * the first call before any stream capture).  Calls share the array: calls
 * whose device work overlaps race on it. */
int eithot_transpose_noalloc(void* d_data, size_t capacity_bytes, int rank,
                             const int64_t* dims, const int* perm_1based,
                             size_t elem_size, int num_sub_tensors, double alpha,
                             void* stream);

/* ---- per-call device status --------------------------------------------
 * No reference counterpart (the reference exits the process on any CUDA
 * error, ITNT/src/cudacheck.cpp:4-10).  Every eithot_transpose,
 * eithot_transpose_ex and eithot_transpose_noalloc call that reaches the
 * device gets a call id and a device status word of its own, zeroed on the
 * call's stream before its first pass.  A kernel of the call sets it when a
 * bounded group-barrier wait gives up (the launch then skips its remaining
 * writes, so the tensor is left partly permuted) or when an index-map
 * result falls outside its row or column (skipped, never dereferenced).
 * eithot_last_call returns the id of the calling thread's most recent such
 * call.  eithot_call_status synchronises `stream` (the call's stream), reads
 * the word and sets *status to EITHOT_OK, EITHOT_ETIMEOUT or EITHOT_EFAULT;
 * the output of a call whose status is not EITHOT_OK is invalid.  The words
 * form a ring of 65536: a call's status can be read until 65536 later calls
 * have started (then EITHOT_EINVAL). */
int eithot_last_call(uint64_t* call_id);
int eithot_call_status(uint64_t call_id, void* stream, int* status);

/* Device scratch bytes eithot_transpose_ex needs for this request. */
int eithot_workspace_size(int rank, const int64_t* dims, const int* perm_1based,
                          size_t elem_size, int num_sub_tensors, double alpha,
                          int reorder_type, size_t* bytes_out);

/* ---- the batched form -------------------------------------------------------
 * No reference counterpart (the reference transposes one tensor per call).
 * eithot_batch_create plans `count` independent transposes once, host only:
 * every tensor is planned for the fewest modelled passes (as
 * EITHOT_ORDER_FEWEST, without cycle-following moves, so that every pass can
 * be captured in a graph); tensor t has rank ranks[t]; its dims and 1-based
 * permutation are the next
 * ranks[t] entries of `dims` and `perms_1based` (tensors back to back);
 * elem_sizes[t] as for eithot_transpose; num_sub_tensors and alpha apply to
 * every tensor.  eithot_batch_run transposes all of them in place
 * (d_data[t] with capacities[t] bytes, as for eithot_transpose), issuing
 * the work on up to 16 internal streams (knob "batch_lanes") forked from and joined back into
 * `stream`: the call is stream-ordered with respect to `stream` and returns
 * before the device work completes.  d_workspace (NULL: the library takes
 * it from cudaMallocAsync on `stream`) must hold
 * eithot_batch_workspace_size() bytes.  A batch may be run any number of
 * times, on any buffers of the planned shapes, on the device it was planned
 * on; runs of one batch must not overlap.  A run whose buffers, capacities
 * and (caller-provided) workspace repeat the previous run's is replayed from
 * a CUDA graph of that work, captured on the first repeat: one graph launch
 * instead of thousands of kernel launches from the host.  Small tensors whose
 * whole permutation fits one CTA's shared memory are permuted by one
 * persistent launch that takes them from a device queue (knob "batch_queue");
 * the queue's table is device memory the batch allocates at its first run
 * and frees in eithot_batch_destroy.  eithot_batch_launches
 * reports the kernel launches of the last run (the graph's kernel nodes when
 * it was replayed). */
typedef struct eithot_batch eithot_batch;

int eithot_batch_create(int count, const int* ranks, const int64_t* dims, const int* perms_1based,
                        const size_t* elem_sizes, int num_sub_tensors, double alpha,
                        eithot_batch** out);
int eithot_batch_workspace_size(const eithot_batch* batch, size_t* bytes);
int eithot_batch_run(eithot_batch* batch, void* const* d_data, const size_t* capacities,
                     void* d_workspace, size_t workspace_bytes, void* stream);
int eithot_batch_launches(const eithot_batch* batch, int* launches);
int eithot_batch_destroy(eithot_batch* batch);

/* ---- the served form ---------------------------------------------------------
 * No reference counterpart.  A server takes requests for in-place
 * transposes of tensors already resident on the device and runs them on
 * `streams` executor streams (1..16) with scratch from a pool of
 * `workspace_bytes` device bytes that eithot_server_create allocates once.
 * Admission: a request's scratch (at most alpha times its bytes, the same
 * workspace eithot_transpose would take) is charged to the pool; one that
 * does not fit now waits.  A request whose scratch exceeds the whole pool is
 * admitted against the device's free HBM instead (cudaMemGetInfo, keeping
 * 256 MB free): it runs alone with scratch allocated when it starts, and
 * such requests wait for one another while free HBM cannot hold them all;
 * it is refused with EITHOT_EBUSY only when free HBM cannot hold it at
 * submission.  Every request is planned for the fewest modelled passes
 * (EITHOT_ORDER_FEWEST).  Requests run in arrival order; consecutive requests under
 * 64 MB at the head of the queue are run together as one batch (continuous
 * batching; a batch whose lane workspaces exceed the pool is halved until
 * it fits), larger ones alone.
 * The server has no thread of its own: work is retired and dispatched
 * inside eithot_server_submit and eithot_server_poll, which never block.
 * eithot_server_poll hands back up to max_done tickets of finished
 * requests; a request's buffer must stay untouched until its ticket comes
 * back.  eithot_server_destroy waits for the work in flight. */
typedef struct eithot_server eithot_server;

int eithot_server_create(size_t workspace_bytes, int streams, eithot_server** out);
int eithot_server_submit(eithot_server* server, void* d_data, size_t capacity_bytes, int rank,
                         const int64_t* dims, const int* perm_1based, size_t elem_size,
                         int num_sub_tensors, double alpha, uint64_t* ticket);
int eithot_server_poll(eithot_server* server, uint64_t* done, int max_done, int* n_done);
/* As eithot_server_poll, also giving each finished ticket's device status
 * (statuses[i] for done[i]; EITHOT_OK, or EITHOT_ETIMEOUT / EITHOT_EFAULT as
 * eithot_call_status reports them, whose result is invalid). */
int eithot_server_poll_status(eithot_server* server, uint64_t* done, int* statuses, int max_done, int* n_done);
/* Bytes of the tensors of queued and running requests, the pool's size, and
 * the scratch that running requests admitted beyond the pool hold in HBM. */
int eithot_server_memory(const eithot_server* server, size_t* resident_bytes, size_t* pool_bytes,
                         size_t* hbm_scratch_bytes);
int eithot_server_pending(const eithot_server* server, int* queued, int* running);
int eithot_server_launches(const eithot_server* server, int* launches);
int eithot_server_destroy(eithot_server* server);

/* ---- the extra-memory estimator --------------------------------------- */

/* Replaces Nd_estimation (Nd_memory_estimation/src/test_inplace.cpp:19-147):
 * the reference's own procedure (max temp over rounds, nb = 2^ceil(log2(
 * tmp/size/alpha)), alpha raised to 1/sqrt(vol/32), padding/partition/join
 * costs, nb halving) evaluated with the reference kernels' cost model for a
 * device with `smem_per_block` bytes of default shared memory per block and
 * `padding_blocks` resident 1024-thread blocks (pass 0 for either to query
 * the current device).  Outputs the nb and alpha the reference would write
 * to proper_input.txt and its modelled extra bytes.  elem_size is treated as
 * the reference does (4 -> 4-byte, otherwise 8-byte). */
int eithot_estimate(int rank, const int64_t* dims, const int* perm_1based,
                    size_t elem_size, int num_sub_tensors, double alpha,
                    size_t smem_per_block, int padding_blocks,
                    int* nb_out, double* alpha_out, size_t* extra_bytes_out);

/* Everything the reference estimator program prints for one request
 * (Nd_memory_estimation/src/test_inplace.cpp:36-44, :61-77, :116-132), for
 * drop-in replacements of that program.  Arguments as eithot_estimate. */
typedef struct eithot_estimate_info {
    int     nb;                  /* sub-tensor count written to proper_input.txt */
    double  alpha;               /* alpha written to proper_input.txt */
    size_t  init_extra_bytes;    /* "init Extra Memory size" */
    double  alpha_raised;        /* "new ratio" (printed when init_extra_bytes > 0) */
    int     decomposed;          /* 1: the sub-tensor branch ran ("Final Extra Memory Size" line) */
    size_t  final_extra_bytes;   /* "Final Extra Memory Size" */
    double  final_ratio;         /* "take ... percent input data size" */
} eithot_estimate_info;

int eithot_estimate_report(int rank, const int64_t* dims, const int* perm_1based,
                           size_t elem_size, double alpha, size_t smem_per_block,
                           int padding_blocks, eithot_estimate_info* info);

/* ---- tuning ----------------------------------------------------------------
 * No reference counterpart (the reference fixes its kernel choices at
 * compile time).  Process-wide knobs of the lowering, used by the autotuner:
 *   "dbuf"        1 allow double-buffered cluster items, 0 single buffer
 *   "max_cluster" largest thread-block cluster (1, 2, 4, 8, 16)
 *   "variant"     0 cost model, 1 force c2r, 2 force r2c for 2D transposes
 *   "col_batch"   remote loads in flight per thread in column passes (4, 8)
 *   "col_chunk"   0 cost model, or 32/64/128/256/512 bytes per staged column-row piece
 *   "col_owner"   1 column passes write from the rows each CTA staged itself,
 *                 0 gather through distributed shared memory
 *   "col_form"    owner-computed column passes: 0 cost model, 1 thread-block
 *                 clusters only, 2 groups of co-resident CTAs only
 *   "row_prefetch" 1 rows that fill a CTA prefetch the next row into
 *                 registers during the write-back, 0 no prefetch
 *   "row_block"   1 rows of 6 KB or less are staged in blocks of consecutive
 *                 rows per CTA, 0 one row per CTA item
 *   "slab_pack"   1 matrices of 16 KB or less are transposed in blocks of
 *                 consecutive matrices per CTA, 0 one matrix per CTA item
 *   "slab_cluster" 1 matrices of up to 16 x 110 KB are transposed in one
 *                 owner-computed pass over a thread-block cluster, 0 not
 *   "factor"      1 a transpose whose passes would stage through global
 *                 scratch is split along a factor of its rows or columns
 *                 into two on-chip transposes when that is cheaper, 0 not
 *   "sync_sleep_ns" back-off between polls of a group barrier (0..100000)
 *   "sync_spin_limit" polls of a group barrier before a wait gives up
 *                 (0..2^26; default 2^20, at least about half a second);
 *                 a give-up is reported by eithot_call_status
 *   "sync_relaxed" 1 group-barrier arrivals without release semantics
 *                 (default: the arriving CTA's loads have all landed in
 *                 shared memory), 0 release arrivals
 *   "group_per_sm" group form: 0 cost model, 1..4 resident CTAs per SM
 *   "slab_perm"   plans for the fewest passes: 0 no on-chip slab
 *                 permutations, 1 cost model (default), 2 preferred
 *   "slab_runs"   1 slab permutations of 1-16 byte elements write runs of
 *                 consecutive outputs per thread from rows staged at a padded
 *                 pitch, with the offsets of a run's outputs from a host-built
 *                 table where every run shares them, else stepping the fastest
 *                 output axis with one jump where a run wraps it at most once
 *                 (default); 2 the runs step through every axis per element;
 *                 0 one divide chain per element
 *   "slab_colband" 256 cluster slabs whose row bands would give each output
 *                 row fewer bytes per CTA than this (0..4096) take column
 *                 bands instead (each CTA writes one contiguous range of the
 *                 output); 0 always row bands
 *   "narrow_words" 1 ranges of 1- and 2-byte units (slabs, strips of wide
 *                 odd-sized elements, row pieces, bands, column row pieces)
 *                 are staged from the aligned words or 16-byte chunks around
 *                 them and written as aligned words; 1-byte 2D transposes and
 *                 column bands of 4k rows as 4 x 4 byte tiles (default); 0
 *                 unit by unit
 *   "row_solo_kb" rows held whole by one CTA that are larger than this many
 *                 KB (16..128, default 48) run one CTA per SM with the next
 *                 row prefetched into registers; smaller ones two or more CTAs
 *                 per SM
 *   "slab2d_runs" slab transposes of whole elements beyond the sizes packed
 *                 several matrices to a CTA run through the slab-permutation
 *                 run kernel: 0 never, 1 for 1- and 2-byte elements
 *                 (default), 2 for 1- to 16-byte elements
 *   "slab_prefetch" 1 slab permutations whose padded slab leaves one CTA per
 *                 SM prefetch the next slab into registers (up to 128 KB),
 *                 0 not
 *   "cycle_moves" plans for the fewest passes (EITHOT_ORDER_FEWEST): 1 may
 *                 permute blocks along the permutation's cycles where the
 *                 cost model expects it to pay (the segment table is copied
 *                 from the host each call; default), 2 prefer such moves,
 *                 0 never
 *   "col_bulk"    1 group passes may run double-buffered with their row pieces
 *                 staged by bulk copies (cp.async.bulk, mbarrier completion)
 *                 when the pass moves 16-byte units and every piece is whole
 *                 16-byte-aligned elements, 0 not
 *                 (default; measured slower than three single-buffered CTAs
 *                 per SM on GB300)
 *   "l2_prefetch" 1 single-buffered group passes prefetch the next item into
 *                 L2 while they wait at the barrier, 0 not (default; slower)
 *   "batch_graph" 1 a batch run on the same buffers and workspace as the
 *                 batch's previous run replays the work as a CUDA graph
 *                 (captured on the first repeat), 0 always issue directly
 *   "batch_lanes" internal streams a batch spreads its other tensors over
 *                 (1..64, default 16; 8 to 64 measured within 1 % of one
 *                 another on the 4096-tensor mix)
 *   "batch_queue" 1 a batch's small tensors (whole permutation in one CTA's
 *                 shared memory, up to 192 KB) are permuted by one
 *                 persistent launch over a device queue whose table the
 *                 batch allocates at its first run (default), 0 every tensor
 *                 runs its planned passes on the lanes */
int eithot_tune_set(const char* key, double value);
int eithot_tune_get(const char* key, double* value);

/* Knobs for one exact request (dims, 1-based perm, element size), for an
 * autotuner: the first call for a shape copies the process-wide knobs, then
 * sets `key`; eithot_transpose, eithot_transpose_ex, eithot_workspace_size
 * and eithot_batch_create use the shape's knobs for that shape (the batched
 * form without group-synchronised column passes; the allocation-free entry
 * point not at all).  Clear drops
 * every shape's entry. */
int eithot_tune_shape_set(int rank, const int64_t* dims, const int* perm_1based, size_t elem_size,
                          const char* key, double value);
int eithot_tune_shape_clear(void);
int eithot_tune_shape_count(int* count);

/* ---- per-pass profiling -------------------------------------------------
 * No reference counterpart (the reference times only whole calls,
 * ITNT/src/test_inplace.cpp:43-69).  When enabled for the calling thread,
 * every eithot_transpose* call records a CUDA event on the caller's stream
 * before its first pass and after each pass, appending to a list that
 * eithot_profile_reset clears; once the stream is synchronised,
 * eithot_profile_get returns listed pass i's name, its event-timed duration
 * in ms and the bytes it reads plus writes. */
int eithot_set_profiling(int enable);
int eithot_profile_reset(void);
int eithot_profile_count(void);
int eithot_profile_get(int i, char* name, size_t name_len, double* ms, double* bytes_moved);

/* ---- self-check --------------------------------------------------------
 * No reference counterpart.  Every kernel checks that each index-map result
 * lies inside its row or column; a result outside is skipped (never
 * dereferenced) and counted.  Returns and clears the count; synchronises
 * the device. */
int eithot_index_faults(unsigned int* count);

/* Column passes whose tiles exceed a thread-block cluster synchronise a
 * group of co-resident CTAs through a barrier in global memory (a
 * cooperative launch).  Such launches never overlap one another on a device,
 * whichever streams or threads issue them: each waits for an event recorded
 * after the previous one (except on a stream that is being captured into a
 * graph).  Every wait on the barrier is bounded (about half a second by
 * default, knob "sync_spin_limit"); a CTA that gives up aborts the launch's
 * remaining writes, marks its call's status EITHOT_ETIMEOUT (see
 * eithot_call_status) and is counted here.  A nonzero count means that some
 * call's output is invalid.  Returns and clears the process-wide count;
 * synchronises the device. */
int eithot_sync_timeouts(unsigned int* count);

/* Runs one bounded wait that nothing releases (a single 32-thread block
 * waiting on a zeroed counter) and reports the timeouts it counted: 1 when
 * the wait gave up as designed.  Allocates 8 bytes; synchronises the device;
 * the context stays usable. */
int eithot_selftest_wait(unsigned int* timeouts);

/* ---- content generator and permutation check ---------------------------
 * No reference counterpart (the reference fills host iota data and compares
 * host copies, ITNT/src/tensor_util.cpp:54-56, :113-142, which a 100 GB
 * tensor cannot afford).  Element i of a generated tensor holds the low
 * elem_size bytes of splitmix64's finaliser applied to
 * seed ^ (i * 0xD1B54A32D192ED03) (byte k of a wider element is byte k mod 8
 * of that value).  eithot_fill_hash writes elements first_index ..
 * first_index + n_elems - 1 of that sequence to d_data, stream-ordered.
 * eithot_check_hash checks that d_data holds the permutation (dims, perm)
 * of such a tensor (generated with first_index 0): output element o must
 * hold the value of the source element its output coordinates name.  It
 * synchronises `stream` and returns the number of mismatching elements and
 * the first mismatching output index (-1 if none).  Calls of
 * eithot_check_hash that overlap on the GPU share one result slot. */
int eithot_fill_hash(void* d_data, int64_t n_elems, size_t elem_size, uint64_t seed, int64_t first_index,
                     void* stream);
int eithot_check_hash(const void* d_data, int rank, const int64_t* dims, const int* perm_1based,
                      size_t elem_size, uint64_t seed, void* stream, uint64_t* mismatches, int64_t* first_bad);

/* ---- misc ------------------------------------------------------------- */
const char* eithot_last_error(void);
int eithot_last_stats(eithot_stats* out);
int eithot_version(void);

#ifdef __cplusplus
}  /* extern "C" */

/* Source-compatible drop-in for the reference's C++ entry point
 * (ITNT/include/transpose.h:6-8): 0-based int permutation, int dims, device
 * pointer `data` advanced by `source` elements, legacy default stream,
 * synchronous like the reference.  sizeofType 4 or 8 as in the reference
 * (other sizes are accepted too).  Errors are printed to stderr and leave
 * the data untouched where possible; the reference exits instead. */
namespace inplace {
void transpose(void* data, int source, int rank, void* dim, void* permutation,
               size_t sizeofType, int num_block, double LARGE_RATIO);
}
#endif

#endif  /* EITHOT_H_ */
