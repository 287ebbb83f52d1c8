// The batched form: many independent in-place transposes planned once and
// run together.  Each tensor's passes stay in order on one of up to 16
// internal streams ("lanes", knob batch_lanes); every tensor is planned for the fewest
// modelled passes (without cycle-following moves, whose segment tables are
// copied from the host); tensors are spread over the lanes
// largest-first onto the least-loaded lane, so the small passes of
// different tensors overlap on the GPU instead of queueing behind one
// another.  Column passes use thread-block clusters only (no
// group-synchronised passes, which rely on all their CTAs being resident
// while other lanes' kernels occupy SMs).  Every lane has its own scratch
// slice of the batch workspace.  A tensor whose shape has recorded knobs
// (eithot_tune_shape_set, e.g. from the autotuner) is planned and run with
// them.  Work is issued round-robin over the lanes so that every lane has
// work queued from the start; a run that repeats the previous run's buffers
// is captured once into a CUDA graph and replayed from then on.  Small
// tensors whose whole permutation fits one CTA's shared memory skip the lanes:
// one persistent launch takes them from a device queue (an atomic counter over
// a table of their slab-permutation arguments, in device memory the batch
// owns), so a thousand 4-200 KB tensors cost one launch instead of one or more
// each.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "api_util.h"
#include "eithot.h"
#include "exec.h"
#include "passes.h"
#include "plan.h"

using namespace eithot;
using namespace eithot::api;

struct eithot_batch {
    int device = -1;
    int order = EITHOT_ORDER_FEWEST;  // plans with the fewest modelled passes
    DeviceCaps caps;
    Tuning tuning;
    struct Item {
        Tuning tuning;         // the batch's knobs, or the shape's (eithot_tune_shape_set)
        std::vector<Pass> passes;
        size_t need = 0;       // bytes the (padded) tensor occupies
        size_t scratch = 0;    // workspace its passes use
        double bytes = 0;      // tensor bytes
        int lane = 0;
        bool queued = false;   // permuted by the queue launch (one whole-tensor slab permutation)
        Pass whole;            // that slab permutation
    };
    std::vector<Item> items;
    // the queue of whole-tensor slab permutations
    std::vector<int> queue;            // tensors permuted by the queue launch
    uint8_t* d_queue = nullptr;        // entries, then the counter (device memory the batch owns)
    size_t queue_entry = 0, queue_smem = 0;
    uint32_t queue_n = 0;              // entries uploaded by the last direct run
    std::vector<int> queue_fallback;   // queued tensors whose entry did not apply on those buffers
    cudaStream_t qstream = nullptr;
    cudaEvent_t qdone = nullptr;
    std::vector<std::vector<int>> lane_items;
    std::vector<size_t> lane_offset, lane_bytes;
    size_t workspace = 0;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> done;
    cudaEvent_t fork = nullptr;
    int last_launches = 0;
    // the graph form: the previous run's buffers, and the capture of a run on them
    std::vector<void*> prev_data;
    std::vector<size_t> prev_caps;
    void* prev_ws = nullptr;
    bool have_prev = false;
    cudaStream_t origin = nullptr;  // capture stream
    cudaGraphExec_t exec = nullptr;
    bool graph_failed = false;      // the capture on these buffers did not succeed: issue directly
    int graph_launches = 0;
};

namespace {

constexpr size_t kQueueBytes = 192 * 1024;   // tensors up to this size may go to the queue
constexpr size_t kQueueSmem = 200 * 1024;    // shared memory of one queue entry at most

int make_streams(eithot_batch* b) {
    if (!b->streams.empty()) return EITHOT_OK;
    const int lanes = static_cast<int>(b->lane_items.size());
    cudaError_t e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (int l = 0; l < lanes && e == cudaSuccess; ++l) {
        cudaStream_t s = nullptr;
        cudaEvent_t ev = nullptr;
        e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        b->streams.push_back(s);
        b->done.push_back(ev);
    }
    if (e == cudaSuccess && !b->queue.empty()) {
        // the queue's table lives in device memory the batch owns, allocated
        // at its first run (planning touches no device memory)
        void* p = nullptr;
        e = cudaMalloc(&p, b->queue.size() * b->queue_entry + 256);
        b->d_queue = static_cast<uint8_t*>(p);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->qstream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->qdone, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) return fail(EITHOT_ECUDA, std::string("batch streams: ") + cudaGetErrorString(e));
    return EITHOT_OK;
}

// Builds the queue's entries for these buffers and uploads them (stream
// ordered on the queue stream, after the previous run's queue launch); a
// queued tensor whose entry does not apply on its buffer is run through its
// planned passes instead (queue_fallback).
int upload_queue(eithot_batch* b, void* const* d_data) {
    b->queue_fallback.clear();
    std::vector<uint8_t> host(b->queue.size() * b->queue_entry);
    uint32_t n = 0;
    for (int t : b->queue) {
        size_t smem = 0;
        ScopedTuning scope(b->items[t].tuning);
        if (slab_queue_entry(static_cast<uint8_t*>(d_data[t]), b->items[t].whole, b->caps,
                             host.data() + n * b->queue_entry, &smem) && smem <= b->queue_smem) {
            ++n;
        } else {
            b->queue_fallback.push_back(t);
        }
    }
    b->queue_n = n;
    if (n == 0) return EITHOT_OK;
    // pageable source: the call returns once the bytes are staged
    const cudaError_t e = cudaMemcpyAsync(b->d_queue, host.data(), n * b->queue_entry, cudaMemcpyHostToDevice, b->qstream);
    if (e != cudaSuccess) return fail(EITHOT_ECUDA, std::string("batch queue upload: ") + cudaGetErrorString(e));
    return cudaStreamSynchronize(b->qstream) == cudaSuccess ? EITHOT_OK
                                                             : fail(EITHOT_ECUDA, "batch queue upload: synchronise");
}

// Forks the lanes from `from`, issues every tensor's passes on its lane
// (round-robin over the lanes) and joins every forked lane back into `from`,
// whatever happened.
int enqueue(eithot_batch* b, void* const* d_data, uint8_t* ws, cudaStream_t from) {
    cudaError_t e = cudaEventRecord(b->fork, from);
    const size_t lanes = b->streams.size();
    std::vector<bool> forked(lanes, false);
    for (size_t l = 0; l < lanes && e == cudaSuccess; ++l) {
        e = cudaStreamWaitEvent(b->streams[l], b->fork, 0);
        forked[l] = e == cudaSuccess;
    }
    int rc = EITHOT_OK;
    std::string err;
    b->last_launches = 0;
    bool qforked = false;
    if (e == cudaSuccess && b->queue_n > 0) {
        e = cudaStreamWaitEvent(b->qstream, b->fork, 0);
        qforked = e == cudaSuccess;
        if (qforked) {
            ExecContext ctx;
            ctx.caps = b->caps;
            ctx.stream = b->qstream;
            rc = launch_slab_queue(b->d_queue, b->queue_n, reinterpret_cast<unsigned*>(b->d_queue + b->queue.size() * b->queue_entry),
                                   b->queue_smem, ctx);
            if (rc) err = "queue: " + ctx.err;
            b->last_launches += ctx.launches;
        }
    }
    // queued tensors whose entry did not apply on these buffers: their own passes, on lane 0
    for (size_t f = 0; f < b->queue_fallback.size() && e == cudaSuccess && rc == EITHOT_OK && lanes > 0; ++f) {
        const int t = b->queue_fallback[f];
        ScopedTuning scope(b->items[t].tuning);
        ExecContext ctx;
        ctx.caps = b->caps;
        ctx.stream = b->streams[0];
        ctx.scratch = ws ? ws + b->lane_offset[0] : nullptr;
        ctx.scratch_bytes = ws ? b->lane_bytes[0] : 0;
        rc = run_passes(static_cast<uint8_t*>(d_data[t]), b->items[t].passes, ctx);
        if (rc) err = "tensor " + std::to_string(t) + ": " + ctx.err;
        b->last_launches += ctx.launches;
    }
    size_t rounds = 0;
    for (const auto& li : b->lane_items) rounds = std::max(rounds, li.size());
    for (size_t r = 0; r < rounds && e == cudaSuccess && rc == EITHOT_OK; ++r) {
        for (size_t l = 0; l < lanes && rc == EITHOT_OK; ++l) {
            if (r >= b->lane_items[l].size()) continue;
            const int t = b->lane_items[l][r];
            ScopedTuning scope(b->items[t].tuning);
            ExecContext ctx;
            ctx.caps = b->caps;
            ctx.stream = b->streams[l];
            ctx.scratch = ws ? ws + b->lane_offset[l] : nullptr;
            ctx.scratch_bytes = ws ? b->lane_bytes[l] : 0;
            rc = run_passes(static_cast<uint8_t*>(d_data[t]), b->items[t].passes, ctx);
            if (rc) err = "tensor " + std::to_string(t) + ": " + ctx.err;
            b->last_launches += ctx.launches;
        }
    }
    for (size_t l = 0; l < lanes; ++l) {
        if (!forked[l]) continue;
        const cudaError_t j = cudaEventRecord(b->done[l], b->streams[l]);
        if (j == cudaSuccess) cudaStreamWaitEvent(from, b->done[l], 0);
        if (e == cudaSuccess) e = j;
    }
    if (qforked) {
        const cudaError_t j = cudaEventRecord(b->qdone, b->qstream);
        if (j == cudaSuccess) cudaStreamWaitEvent(from, b->qdone, 0);
        if (e == cudaSuccess) e = j;
    }
    if (rc) return fail(rc, err);
    if (e != cudaSuccess) return fail(EITHOT_ECUDA, std::string("batch: ") + cudaGetErrorString(e));
    return EITHOT_OK;
}

void drop_graph(eithot_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
}

// Captures one run on the remembered buffers into b->exec; false (and no
// graph) when the capture or instantiation did not succeed.
bool capture(eithot_batch* b, void* const* d_data, uint8_t* ws) {
    if (!b->origin && cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        b->origin = nullptr;
        return false;
    }
    if (cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const int rc = enqueue(b, d_data, ws, b->origin);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->origin, &g);
    if (rc == EITHOT_OK && e == cudaSuccess && g) e = cudaGraphInstantiate(&b->exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (rc != EITHOT_OK || e != cudaSuccess || !b->exec) {
        cudaGetLastError();
        b->exec = nullptr;
        return false;
    }
    b->graph_launches = b->last_launches;
    return true;
}

}  // namespace

extern "C" {

int eithot_batch_create(int count, const int* ranks, const int64_t* dims, const int* perms_1based,
                        const size_t* elem_sizes, int num_sub_tensors, double alpha, eithot_batch** out) {
    if (!out) return fail(EITHOT_EINVAL, "null out");
    *out = nullptr;
    if (count < 0 || (count > 0 && (!ranks || !dims || !perms_1based || !elem_sizes)))
        return fail(EITHOT_EINVAL, "null or negative batch description");
    auto* b = new eithot_batch();
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) {
        std::string err;
        if (!query_caps(dev, &b->caps, &err)) b->caps = DeviceCaps();
        b->device = dev;
    } else {
        cudaGetLastError();
    }
    b->tuning = tuning();
    b->tuning.col_form = 1;     // clusters only: no pass relies on grid-wide residency
    b->tuning.cycle_moves = 0;  // every pass can be captured in a graph (no host-to-device table copies)
    b->items.resize(count);
    size_t off = 0;
    for (int t = 0; t < count; ++t) {
        NdPlan plan;
        auto& it = b->items[t];
        it.tuning = b->tuning;
        if (ranks[t] >= 1 &&
            shape_tuning(std::vector<int64_t>(dims + off, dims + off + ranks[t]),
                         std::vector<int>(perms_1based + off, perms_1based + off + ranks[t]), elem_sizes[t],
                         &it.tuning)) {
            it.tuning.col_form = 1;  // a shape's knobs, still without group passes
            it.tuning.cycle_moves = 0;
        }
        ScopedTuning scope(it.tuning);
        const int rc = build(ranks[t], dims + off, perms_1based + off, elem_sizes[t], num_sub_tensors, alpha,
                             b->order, b->caps, &plan, &it.passes);
        if (rc) {
            delete b;
            return fail(rc, "tensor " + std::to_string(t) + ": " + eithot_last_error());
        }
        off += static_cast<size_t>(ranks[t]);
        it.need = static_cast<size_t>(plan.padded_volume) * elem_sizes[t];
        it.bytes = static_cast<double>(plan.volume) * static_cast<double>(elem_sizes[t]);
        it.scratch = choose_workspace(it.passes, b->caps, alpha, it.bytes);
        // a small tensor whose whole permutation fits one CTA goes to the queue
        if (b->tuning.batch_queue && num_sub_tensors <= 1 && !it.passes.empty() && ranks[t] <= 8 &&
            it.bytes <= static_cast<double>(kQueueBytes)) {
            Pass w;
            w.type = kSlabPerm;
            w.batches = 1;
            w.elem = elem_sizes[t];
            w.strip = elem_sizes[t];
            for (int a = 0; a < ranks[t]; ++a) {
                w.nd_dims.push_back(static_cast<uint64_t>(dims[off - ranks[t] + a]));
                w.nd_perm.push_back(perms_1based[off - ranks[t] + a] - 1);
            }
            w.rows = static_cast<uint64_t>(it.bytes / static_cast<double>(elem_sizes[t]));
            w.what = "queue slab-perm";
            std::vector<uint8_t> entry(slab_queue_entry_bytes());
            size_t smem = 0;
            // a 256-byte aligned stand-in address: the entry is only sized here
            if (slab_queue_entry(reinterpret_cast<uint8_t*>(uintptr_t(256)), w, b->caps, entry.data(), &smem) &&
                smem <= kQueueSmem) {
                it.queued = true;
                it.whole = w;
                b->queue.push_back(t);
                b->queue_smem = std::max(b->queue_smem, smem);
            }
        }
    }
    b->queue_entry = (slab_queue_entry_bytes() + 15) / 16 * 16;
    // largest first: the counter hands entries out in table order
    std::stable_sort(b->queue.begin(), b->queue.end(), [&](int x, int y) { return b->items[x].bytes > b->items[y].bytes; });
    // largest first onto the least-loaded lane
    const int lanes = std::max(1, std::min(count, b->tuning.batch_lanes));
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->items[x].bytes > b->items[y].bytes; });
    std::vector<double> load(lanes, 0.0);
    b->lane_items.assign(lanes, {});
    b->lane_bytes.assign(lanes, 0);
    for (int t : order) {
        if (b->items[t].queued) continue;
        const int l = static_cast<int>(std::min_element(load.begin(), load.end()) - load.begin());
        load[l] += b->items[t].bytes + 64.0 * 1024;  // a launch's fixed cost, in bytes
        b->items[t].lane = l;
        b->lane_items[l].push_back(t);
        b->lane_bytes[l] = std::max(b->lane_bytes[l], b->items[t].scratch);
    }
    // a queued tensor whose entry does not apply on its buffers runs its own
    // passes on lane 0, with lane 0's scratch
    for (int t : b->queue) b->lane_bytes[0] = std::max(b->lane_bytes[0], b->items[t].scratch);
    b->lane_offset.assign(lanes, 0);
    for (int l = 0; l < lanes; ++l) {
        b->lane_offset[l] = b->workspace;
        b->workspace += (b->lane_bytes[l] + 255) / 256 * 256;
    }
    *out = b;
    return EITHOT_OK;
}

int eithot_batch_workspace_size(const eithot_batch* b, size_t* bytes) {
    if (!b || !bytes) return fail(EITHOT_EINVAL, "null argument");
    *bytes = b->workspace;
    return EITHOT_OK;
}

int eithot_batch_run(eithot_batch* b, void* const* d_data, const size_t* capacities, void* d_workspace,
                     size_t workspace_bytes, void* stream) {
    if (!b || (!b->items.empty() && (!d_data || !capacities))) return fail(EITHOT_EINVAL, "null argument");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || (b->device >= 0 && dev != b->device))
        return fail(EITHOT_EINVAL, "the batch was planned for another device");
    for (size_t t = 0; t < b->items.size(); ++t) {
        if (!d_data[t]) return fail(EITHOT_EINVAL, "tensor " + std::to_string(t) + ": null data pointer");
        if (capacities[t] < b->items[t].need)
            return fail(EITHOT_EINVAL, "tensor " + std::to_string(t) + ": capacity below the (padded) tensor");
    }
    if (b->items.empty()) return EITHOT_OK;
    if (int rc = make_streams(b)) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint8_t* ws = static_cast<uint8_t*>(d_workspace);
    bool owned = false;
    if (b->workspace > 0) {
        if (ws) {
            if (workspace_bytes < b->workspace) return fail(EITHOT_ENOMEM, "workspace smaller than eithot_batch_workspace_size()");
        } else {
            void* p = nullptr;
            const cudaError_t e = cudaMallocAsync(&p, b->workspace, st);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return fail(EITHOT_ENOMEM, std::string("batch workspace: ") + cudaGetErrorString(e));
            }
            ws = static_cast<uint8_t*>(p);
            owned = true;
        }
    }
    const bool same = b->have_prev && b->prev_ws == ws &&
                      std::equal(b->prev_data.begin(), b->prev_data.end(), d_data) &&
                      std::equal(b->prev_caps.begin(), b->prev_caps.end(), capacities);
    // a graph replays only caller-provided workspace (or none)
    if (same && !owned && b->tuning.batch_graph && !b->graph_failed) {
        if (!b->exec) b->graph_failed = !capture(b, d_data, ws);
        if (b->exec) {
            const cudaError_t e = cudaGraphLaunch(b->exec, st);
            if (e != cudaSuccess) return fail(EITHOT_ECUDA, std::string("batch graph: ") + cudaGetErrorString(e));
            b->last_launches = b->graph_launches;
            return EITHOT_OK;
        }
    }
    if (!same) {
        drop_graph(b);
        b->graph_failed = false;
        b->prev_data.assign(d_data, d_data + b->items.size());
        b->prev_caps.assign(capacities, capacities + b->items.size());
        b->prev_ws = ws;
        b->have_prev = true;
    }
    if (!b->queue.empty()) {
        if (int rc = upload_queue(b, d_data)) {
            if (owned) cudaFreeAsync(ws, st);
            return rc;
        }
    }
    const int rc = enqueue(b, d_data, ws, st);
    if (owned) cudaFreeAsync(ws, st);
    return rc;
}

int eithot_batch_launches(const eithot_batch* b, int* launches) {
    if (!b || !launches) return fail(EITHOT_EINVAL, "null argument");
    *launches = b->last_launches;
    return EITHOT_OK;
}

int eithot_batch_destroy(eithot_batch* b) {
    if (!b) return EITHOT_OK;
    drop_graph(b);
    if (b->origin) cudaStreamDestroy(b->origin);
    for (auto s : b->streams) cudaStreamDestroy(s);
    for (auto ev : b->done) cudaEventDestroy(ev);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->qstream) cudaStreamDestroy(b->qstream);
    if (b->qdone) cudaEventDestroy(b->qdone);
    if (b->d_queue) cudaFree(b->d_queue);
    delete b;
    return EITHOT_OK;
}

}  // extern "C"
