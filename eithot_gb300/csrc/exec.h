// Executor interface: runs lowered passes on a stream.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "passes.h"

namespace eithot {

enum Status {
    EITHOT_STATUS_OK = 0,
    EITHOT_STATUS_INVALID = 1,
    EITHOT_STATUS_NOMEM = 2,
    EITHOT_STATUS_TIMEOUT = 3,
    EITHOT_STATUS_CUDA = 4,
    EITHOT_STATUS_UNSUPPORTED = 5,
    EITHOT_STATUS_BUSY = 6,
};

// Per-call device status: a ring of status words in device memory, one per
// call id (id mod kStatusRing); kernels OR these bits into their call's word.
constexpr unsigned kStatusRing = 1u << 16;
constexpr unsigned kCallIndexFault = 1u;   // an index-map result fell outside its row or column
constexpr unsigned kCallSyncTimeout = 2u;  // a bounded group-barrier wait gave up

struct ExecContext {
    DeviceCaps caps;
    cudaStream_t stream = nullptr;
    unsigned* status = nullptr;  // this call's device status word (may be null)
    uint8_t* scratch = nullptr;
    size_t scratch_bytes = 0;
    int launches = 0;
    int group_per_sm_seen = 0;  // CTAs per SM the last group launch could have resident
    int passes = 0;
    std::string err;
    // When profiling, one event is recorded on `stream` before the first pass
    // and after every pass (events[i], events[i+1] bracket pass i).
    bool profile = false;
    size_t events_used = 0;
    std::vector<cudaEvent_t>* events = nullptr;
    std::vector<std::pair<size_t, size_t>>* spans = nullptr;
    std::vector<std::string>* names = nullptr;
    std::vector<double>* bytes = nullptr;
};

// Minimum scratch one pass needs (one staged item), and the scratch that
// lets it run in a single group.
size_t pass_workspace_bytes(const Pass& p, const DeviceCaps& caps);
size_t pass_workspace_ideal(const Pass& p, const DeviceCaps& caps);

// The planner's slab and block permutations (perm.cu); scratch of a block
// permutation: its segment table and the saved blocks of its longest cycle
// (ideal: of every cycle at once).
int run_slab_perm(uint8_t* data, const Pass& p, ExecContext& ctx);
// The run kernel of a slab permutation (whole elements of 1-16 bytes whose
// padded slab fits one CTA); -1 when it does not apply.
int try_slab_runs_pass(uint8_t* data, const Pass& p, ExecContext& ctx);

// The batched form's queue of whole-tensor slab permutations: the size of one
// entry, an entry for pass p on data (false when the run kernel does not
// apply; *smem the shared memory it needs), and one persistent launch over n
// entries in device memory (*d_next: a counter the launch zeroes first).
// A column-band cluster slab (kSlabCluster with band > 0), at any alignment;
// -1 when the band count is outside 2..16 (the caller runs the row bands).
int run_slab_colband(uint8_t* data, const Pass& p, ExecContext& ctx);

size_t slab_queue_entry_bytes();
bool slab_queue_entry(uint8_t* data, const Pass& p, const DeviceCaps& caps, void* entry, size_t* smem);
int launch_slab_queue(const void* d_entries, uint32_t n, unsigned* d_next, size_t smem, ExecContext& ctx);
int run_block_perm(uint8_t* data, const Pass& p, ExecContext& ctx);
size_t block_perm_workspace(const Pass& p, bool ideal);

// Launches every pass in order on ctx.stream.  Returns a Status.
int run_passes(uint8_t* data, const std::vector<Pass>& passes, ExecContext& ctx);

bool query_caps(int device, DeviceCaps* caps, std::string* err);

// Size of the fixed device scratch behind eithot_transpose_noalloc.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;

// Device address of that scratch on the current device (looked up on every
// call: no allocation, and valid after a device reset).
int noalloc_scratch(uint8_t** ptr, std::string* err);

// Count of index-map results that fell outside their row/column since the
// last read (the kernels skip such accesses).  Synchronises the device.
int read_index_faults(unsigned int* out);

// Counter-hash content and its permutation check (checks.cu).
int fill_hash(void* d, int64_t n, size_t elem, uint64_t seed, int64_t first, cudaStream_t s, std::string* err);
int check_hash(const void* d, int rank, const int64_t* dims, const int* perm1, size_t elem, uint64_t seed,
               cudaStream_t s, uint64_t* mismatches, int64_t* first_bad, std::string* err);

// Starts a call: takes the next call id, points *status at its device status
// word on the current device and zeroes that word on `stream`.
int begin_call(cudaStream_t stream, uint64_t* id, unsigned** status, std::string* err);

// The call ids handed out so far (the next id to be issued).
uint64_t next_call_id();

// Reads call `id`'s status word on `stream` (stream-ordered, then
// synchronises the stream).  False when the id is unknown or its word has
// been reused by a later call.
int read_call_status(uint64_t id, cudaStream_t stream, unsigned* bits, std::string* err);

// Returns and clears the number of bounded group-barrier waits that gave up
// (their launch aborted its writes); synchronises the device.
int read_sync_timeouts(unsigned int* out);

// Launches one CTA that waits on a counter nothing increments; it must give
// up after its spin limit.  *timeouts = timeouts counted (1 when the bound
// holds).  Synchronises the device.
int run_wait_selftest(unsigned int* timeouts, std::string* err);

}  // namespace eithot
