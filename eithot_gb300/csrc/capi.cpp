// The C ABI (include/eithot.h) and the reference-signature shim.
#include "eithot.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <optional>
#include <string>
#include <vector>

#include "api_util.h"
#include "estimator.h"
#include "exec.h"
#include "passes.h"
#include "plan.h"
#include "search.h"

namespace {

thread_local std::string g_err;
thread_local eithot_stats g_stats;
thread_local bool g_profile = false;
thread_local std::vector<cudaEvent_t> g_events;
thread_local size_t g_events_used = 0;
thread_local std::vector<std::pair<size_t, size_t>> g_spans;
thread_local std::vector<std::string> g_pass_names;
thread_local std::vector<double> g_pass_bytes;
thread_local uint64_t g_last_call = 0;

}  // namespace

namespace eithot {
namespace api {

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

bool elem_ok(size_t e) { return e >= 1 && e <= 64; }

// Scratch for a pass list: at least one staged item of every pass, at most
// what lets each pass run as a single group, capped at alpha * bytes when
// that cap still covers the minimum.
size_t choose_workspace(const std::vector<eithot::Pass>& passes, const eithot::DeviceCaps& caps,
                        double alpha, double bytes) {
    size_t lo = 0, ideal = 0;
    for (const auto& p : passes) {
        lo = std::max(lo, eithot::pass_workspace_bytes(p, caps));
        ideal = std::max(ideal, eithot::pass_workspace_ideal(p, caps));
    }
    if (lo == 0) return 0;
    const double cap = alpha * bytes;
    size_t ws = (ideal + 255) / 256 * 256;
    // under the cap: round down to 256 bytes, never below the minimum
    if (static_cast<double>(ws) > cap) ws = static_cast<size_t>(cap) / 256 * 256;
    return std::max(ws, (lo + 255) / 256 * 256);
}

int device_caps(eithot::DeviceCaps* caps) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(EITHOT_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    std::string err;
    if (!eithot::query_caps(dev, caps, &err)) return fail(EITHOT_ECUDA, "device query: " + err);
    return EITHOT_OK;
}

int build(int rank, const int64_t* dims, const int* perm, size_t elem, int nb, double alpha,
          int order, const eithot::DeviceCaps& caps, eithot::NdPlan* plan,
          std::vector<eithot::Pass>* passes) {
    if (!elem_ok(elem)) return fail(EITHOT_EINVAL, "elem_size must be in [1, 64] bytes");
    std::string err;
    if (!eithot::make_nd_plan(rank, dims, perm, nb, alpha, order, plan, &err)) return fail(EITHOT_EINVAL, err);
    if (static_cast<double>(plan->padded_volume) * static_cast<double>(elem) > 1.15e18)
        return fail(EITHOT_EINVAL, "tensor too large");
    if (!eithot::lower_plan(*plan, elem, caps, passes, &err)) return fail(EITHOT_EINVAL, err);
    if (order == EITHOT_ORDER_FEWEST && plan->nb == 1 && !plan->padded) {
        // the pass-minimising search, kept only for a clear modelled gain
        std::vector<eithot::Pass> alt;
        double cost = 0;
        if (eithot::search_plan(plan->dims, plan->perm, elem, caps, &alt, &cost, nullptr) &&
            cost < eithot::passes_model_cost(*passes, caps) - 0.2)
            passes->swap(alt);
    }
    return EITHOT_OK;
}

}  // namespace api
}  // namespace eithot

using namespace eithot::api;

namespace {
std::vector<int64_t> dims_of(int rank, const int64_t* dims) { return std::vector<int64_t>(dims, dims + rank); }
std::vector<int> perm_of(int rank, const int* perm) { return std::vector<int>(perm, perm + rank); }
}  // namespace

extern "C" {

const char* eithot_last_error(void) { return g_err.c_str(); }

int eithot_version(void) { return 100; }

}  // extern "C"

namespace {

// Sets knob `key` of `t` (the keys of eithot_tune_set).
int apply_knob(eithot::Tuning& t, const char* key, double value) {
    if (!key) return fail(EITHOT_EINVAL, "null key");
    const std::string k(key);
    if (k == "dbuf") {
        t.dbuf = value != 0.0 ? 1 : 0;
    } else if (k == "col_batch") {
        t.col_batch = value >= 8 ? 8 : 4;
    } else if (k == "col_owner") {
        t.col_owner = value != 0.0 ? 1 : 0;
    } else if (k == "sync_sleep_ns") {
        if (value < 0 || value > 100000) return fail(EITHOT_EINVAL, "sync_sleep_ns must be 0..100000");
        t.sync_sleep_ns = static_cast<int>(value);
    } else if (k == "cycle_moves") {
        const int v = static_cast<int>(value);
        if (v < 0 || v > 2) return fail(EITHOT_EINVAL, "cycle_moves must be 0, 1 or 2");
        t.cycle_moves = v;
    } else if (k == "slab_perm") {
        const int v = static_cast<int>(value);
        if (v < 0 || v > 2) return fail(EITHOT_EINVAL, "slab_perm must be 0, 1 or 2");
        t.slab_perm = v;
    } else if (k == "slab_runs") {
        const int v = static_cast<int>(value);
        if (v < 0 || v > 2) return fail(EITHOT_EINVAL, "slab_runs must be 0, 1 or 2");
        t.slab_runs = v;
    } else if (k == "slab_colband") {
        const int v = static_cast<int>(value);
        if (v < 0 || v > 4096) return fail(EITHOT_EINVAL, "slab_colband must be 0..4096");
        t.slab_colband = v;
    } else if (k == "narrow_words") {
        t.narrow_words = value != 0.0 ? 1 : 0;
    } else if (k == "row_solo_kb") {
        const int v = static_cast<int>(value);
        if (v < 16 || v > 128) return fail(EITHOT_EINVAL, "row_solo_kb must be 16..128");
        t.row_solo_kb = v;
    } else if (k == "slab2d_runs") {
        const int v = static_cast<int>(value);
        if (v < 0 || v > 2) return fail(EITHOT_EINVAL, "slab2d_runs must be 0, 1 or 2");
        t.slab2d_runs = v;
    } else if (k == "slab_prefetch") {
        t.slab_prefetch = value != 0.0 ? 1 : 0;
    } else if (k == "col_bulk") {
        t.col_bulk = value != 0.0 ? 1 : 0;
    } else if (k == "l2_prefetch") {
        t.l2_prefetch = value != 0.0 ? 1 : 0;
    } else if (k == "group_per_sm") {
        const int v = static_cast<int>(value);
        if (v < 0 || v > 4) return fail(EITHOT_EINVAL, "group_per_sm must be 0..4");
        t.group_per_sm = v;
    } else if (k == "sync_spin_limit") {
        if (value < 0 || value > static_cast<double>(1 << 26)) return fail(EITHOT_EINVAL, "sync_spin_limit must be 0..2^26");
        t.sync_spin_limit = static_cast<int>(value);
    } else if (k == "sync_relaxed") {
        t.sync_relaxed = value != 0.0 ? 1 : 0;
    } else if (k == "factor") {
        t.factor = value != 0.0 ? 1 : 0;
    } else if (k == "slab_cluster") {
        t.slab_cluster = value != 0.0 ? 1 : 0;
    } else if (k == "slab_pack") {
        t.slab_pack = value != 0.0 ? 1 : 0;
    } else if (k == "row_block") {
        t.row_block = value != 0.0 ? 1 : 0;
    } else if (k == "row_prefetch") {
        t.row_prefetch = value != 0.0 ? 1 : 0;
    } else if (k == "col_form") {
        const int v = static_cast<int>(value);
        if (v < 0 || v > 2) return fail(EITHOT_EINVAL, "col_form must be 0, 1 or 2");
        t.col_form = v;
    } else if (k == "col_chunk") {
        const int v = static_cast<int>(value);
        if (v != 0 && v != 32 && v != 64 && v != 128 && v != 256 && v != 512)
            return fail(EITHOT_EINVAL, "col_chunk must be 0, 32, 64, 128, 256 or 512");
        t.col_chunk = v;
    } else if (k == "batch_lanes") {
        const int v = static_cast<int>(value);
        if (v < 1 || v > 64) return fail(EITHOT_EINVAL, "batch_lanes must be 1..64");
        t.batch_lanes = v;
    } else if (k == "batch_queue") {
        t.batch_queue = value != 0 ? 1 : 0;
    } else if (k == "batch_graph") {
        t.batch_graph = value != 0 ? 1 : 0;
    } else if (k == "max_cluster") {
        const int v = static_cast<int>(value);
        if (v != 1 && v != 2 && v != 4 && v != 8 && v != 16) return fail(EITHOT_EINVAL, "max_cluster must be 1, 2, 4, 8 or 16");
        t.max_cluster = v;
    } else if (k == "variant") {
        const int v = static_cast<int>(value);
        if (v < 0 || v > 2) return fail(EITHOT_EINVAL, "variant must be 0, 1 or 2");
        t.variant = v;
    } else {
        return fail(EITHOT_EINVAL, "unknown tuning key " + k);
    }
    return EITHOT_OK;
}

}  // namespace

extern "C" {

int eithot_tune_set(const char* key, double value) { return apply_knob(eithot::tuning(), key, value); }

int eithot_tune_shape_set(int rank, const int64_t* dims, const int* perm_1based, size_t elem_size,
                          const char* key, double value) {
    if (rank < 1 || !dims || !perm_1based) return fail(EITHOT_EINVAL, "null or empty shape");
    eithot::Tuning t;
    if (!eithot::shape_tuning(dims_of(rank, dims), perm_of(rank, perm_1based), elem_size, &t)) t = eithot::tuning();
    if (int rc = apply_knob(t, key, value)) return rc;
    eithot::set_shape_tuning(dims_of(rank, dims), perm_of(rank, perm_1based), elem_size, t);
    return EITHOT_OK;
}

int eithot_tune_shape_clear(void) {
    eithot::clear_shape_tuning();
    return EITHOT_OK;
}

int eithot_tune_shape_count(int* count) {
    if (!count) return fail(EITHOT_EINVAL, "null count");
    *count = eithot::shape_tuning_count();
    return EITHOT_OK;
}

int eithot_tune_get(const char* key, double* value) {
    if (!key || !value) return fail(EITHOT_EINVAL, "null argument");
    const eithot::Tuning& t = eithot::tuning();
    const std::string k(key);
    if (k == "dbuf") *value = t.dbuf;
    else if (k == "col_batch") *value = t.col_batch;
    else if (k == "col_owner") *value = t.col_owner;
    else if (k == "col_form") *value = t.col_form;
    else if (k == "row_prefetch") *value = t.row_prefetch;
    else if (k == "row_block") *value = t.row_block;
    else if (k == "slab_pack") *value = t.slab_pack;
    else if (k == "slab_cluster") *value = t.slab_cluster;
    else if (k == "factor") *value = t.factor;
    else if (k == "sync_sleep_ns") *value = t.sync_sleep_ns;
    else if (k == "sync_relaxed") *value = t.sync_relaxed;
    else if (k == "sync_spin_limit") *value = t.sync_spin_limit;
    else if (k == "group_per_sm") *value = t.group_per_sm;
    else if (k == "l2_prefetch") *value = t.l2_prefetch;
    else if (k == "col_bulk") *value = t.col_bulk;
    else if (k == "cycle_moves") *value = t.cycle_moves;
    else if (k == "slab_perm") *value = t.slab_perm;
    else if (k == "slab_runs") *value = t.slab_runs;
    else if (k == "slab_prefetch") *value = t.slab_prefetch;
    else if (k == "slab2d_runs") *value = t.slab2d_runs;
    else if (k == "row_solo_kb") *value = t.row_solo_kb;
    else if (k == "narrow_words") *value = t.narrow_words;
    else if (k == "slab_colband") *value = t.slab_colband;
    else if (k == "batch_graph") *value = t.batch_graph;
    else if (k == "batch_queue") *value = t.batch_queue;
    else if (k == "batch_lanes") *value = t.batch_lanes;
    else if (k == "col_chunk") *value = t.col_chunk;
    else if (k == "max_cluster") *value = t.max_cluster;
    else if (k == "variant") *value = t.variant;
    else return fail(EITHOT_EINVAL, "unknown tuning key " + k);
    return EITHOT_OK;
}

int eithot_set_profiling(int enable) {
    g_profile = enable != 0;
    return EITHOT_OK;
}

int eithot_profile_reset(void) {
    g_events_used = 0;
    g_spans.clear();
    g_pass_names.clear();
    g_pass_bytes.clear();
    return EITHOT_OK;
}

int eithot_profile_count(void) { return static_cast<int>(g_pass_names.size()); }

int eithot_profile_get(int i, char* name, size_t name_len, double* ms, double* bytes_moved) {
    if (i < 0 || i >= static_cast<int>(g_pass_names.size()))
        return fail(EITHOT_EINVAL, "profile index out of range");
    if (name && name_len) {
        std::strncpy(name, g_pass_names[i].c_str(), name_len);
        name[name_len - 1] = 0;
    }
    if (bytes_moved) *bytes_moved = g_pass_bytes[i];
    if (ms) {
        float t = 0.f;
        cudaError_t e = cudaEventElapsedTime(&t, g_events[g_spans[i].first], g_events[g_spans[i].second]);
        if (e != cudaSuccess) return fail(EITHOT_ECUDA, std::string("profile: ") + cudaGetErrorString(e));
        *ms = t;
    }
    return EITHOT_OK;
}

int eithot_index_faults(unsigned int* count) {
    if (!count) return fail(EITHOT_EINVAL, "null count");
    if (eithot::read_index_faults(count)) return fail(EITHOT_ECUDA, "reading the index-fault counter failed");
    return EITHOT_OK;
}

int eithot_fill_hash(void* d_data, int64_t n_elems, size_t elem_size, uint64_t seed, int64_t first_index,
                     void* stream) {
    if (!d_data && n_elems > 0) return fail(EITHOT_EINVAL, "null data");
    if (elem_size < 1 || elem_size > 64) return fail(EITHOT_EINVAL, "element size must be 1..64 bytes");
    if (n_elems < 0 || first_index < 0) return fail(EITHOT_EINVAL, "negative count or index");
    std::string err;
    if (int rc = eithot::fill_hash(d_data, n_elems, elem_size, seed, first_index, static_cast<cudaStream_t>(stream), &err))
        return fail(rc, err);
    return EITHOT_OK;
}

int eithot_check_hash(const void* d_data, int rank, const int64_t* dims, const int* perm_1based, size_t elem_size,
                      uint64_t seed, void* stream, uint64_t* mismatches, int64_t* first_bad) {
    if (!d_data || !dims || !perm_1based || !mismatches || !first_bad) return fail(EITHOT_EINVAL, "null argument");
    if (elem_size < 1 || elem_size > 64) return fail(EITHOT_EINVAL, "element size must be 1..64 bytes");
    std::string err;
    if (int rc = eithot::check_hash(d_data, rank, dims, perm_1based, elem_size, seed, static_cast<cudaStream_t>(stream),
                                    mismatches, first_bad, &err))
        return fail(rc, err);
    return EITHOT_OK;
}

int eithot_sync_timeouts(unsigned int* count) {
    if (!count) return fail(EITHOT_EINVAL, "null count");
    if (eithot::read_sync_timeouts(count)) return fail(EITHOT_ECUDA, "reading the sync-timeout counter failed");
    return EITHOT_OK;
}

int eithot_selftest_wait(unsigned int* timeouts) {
    if (!timeouts) return fail(EITHOT_EINVAL, "null count");
    std::string err;
    if (eithot::run_wait_selftest(timeouts, &err)) return fail(EITHOT_ECUDA, err);
    return EITHOT_OK;
}

int eithot_last_call(uint64_t* call_id) {
    if (!call_id) return fail(EITHOT_EINVAL, "null call_id");
    if (g_last_call == 0) return fail(EITHOT_EINVAL, "no transpose has been issued on this thread");
    *call_id = g_last_call;
    return EITHOT_OK;
}

int eithot_call_status(uint64_t call_id, void* stream, int* status) {
    if (!status) return fail(EITHOT_EINVAL, "null status");
    unsigned bits = 0;
    std::string err;
    if (int rc = eithot::read_call_status(call_id, static_cast<cudaStream_t>(stream), &bits, &err))
        return fail(rc, err);
    if (bits & eithot::kCallSyncTimeout) *status = EITHOT_ETIMEOUT;
    else if (bits & eithot::kCallIndexFault) *status = EITHOT_EFAULT;
    else *status = EITHOT_OK;
    return EITHOT_OK;
}

int eithot_last_stats(eithot_stats* out) {
    if (!out) return fail(EITHOT_EINVAL, "null stats");
    *out = g_stats;
    return EITHOT_OK;
}

int eithot_plan(int rank, const int64_t* dims, const int* perm_1based, int num_sub_tensors,
                double alpha, int reorder_type, eithot_plan_info* info, eithot_step* steps,
                int max_steps) {
    eithot::NdPlan plan;
    std::string err;
    if (!eithot::make_nd_plan(rank, dims, perm_1based, num_sub_tensors, alpha, reorder_type, &plan, &err))
        return fail(EITHOT_EINVAL, err);
    if (info) {
        info->order_used = plan.order_used;
        info->num_sub_tensors = plan.nb;
        info->decompose_dim = plan.decompose_pos;
        info->padded = plan.padded ? 1 : 0;
        info->padded_dim_size = plan.padded ? plan.padded_dim : 0;
        info->volume = plan.volume;
        info->padded_volume = plan.padded_volume;
        info->sub_tensor_elems = plan.sub_volume;
        info->n_steps = static_cast<int>(plan.steps.size());
    }
    for (int i = 0; steps && i < max_steps && i < static_cast<int>(plan.steps.size()); ++i) {
        const auto& s = plan.steps[i];
        eithot_step& o = steps[i];
        std::memset(&o, 0, sizeof(o));
        o.role = s.role;
        if (s.role == eithot::kPadPre || s.role == eithot::kPadPost) {
            o.code = 0;
            o.rank = 0;
            o.dims[0] = s.pad_pos;
            o.dims[1] = s.pad_orig;
            o.dims[2] = s.pad_size;
        } else {
            o.code = s.op.code();
            o.rank = s.op.rank;
            for (int k = 0; k < s.op.rank; ++k) {
                o.dims[k] = s.op.dims[k];
                o.perm[k] = s.op.perm[k];
            }
        }
    }
    return EITHOT_OK;
}

int eithot_workspace_size(int rank, const int64_t* dims, const int* perm_1based, size_t elem_size,
                          int num_sub_tensors, double alpha, int reorder_type, size_t* bytes_out) {
    if (!bytes_out) return fail(EITHOT_EINVAL, "null bytes_out");
    eithot::DeviceCaps caps;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) {
        std::string err;
        if (!eithot::query_caps(dev, &caps, &err)) caps = eithot::DeviceCaps();
    } else {
        cudaGetLastError();
    }
    eithot::Tuning shape_t;
    std::optional<eithot::ScopedTuning> shape_scope;
    if (rank >= 1 && dims && perm_1based &&
        eithot::shape_tuning(dims_of(rank, dims), perm_of(rank, perm_1based), elem_size, &shape_t))
        shape_scope.emplace(shape_t);
    eithot::NdPlan plan;
    std::vector<eithot::Pass> passes;
    int rc = build(rank, dims, perm_1based, elem_size, num_sub_tensors, alpha, reorder_type, caps, &plan, &passes);
    if (rc) return rc;
    *bytes_out = choose_workspace(passes, caps, alpha, static_cast<double>(plan.volume) * elem_size);
    return EITHOT_OK;
}

int eithot_transpose_ex(void* d_data, size_t capacity_bytes, int rank, const int64_t* dims,
                        const int* perm_1based, size_t elem_size, int num_sub_tensors, double alpha,
                        int reorder_type, void* d_workspace, size_t workspace_bytes, void* stream) {
    std::memset(&g_stats, 0, sizeof(g_stats));
    if (!d_data) return fail(EITHOT_EINVAL, "null data pointer");
    eithot::DeviceCaps caps;
    int rc = device_caps(&caps);
    if (rc) return rc;
    {
        cudaPointerAttributes attr;
        cudaError_t e = cudaPointerGetAttributes(&attr, d_data);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(EITHOT_EINVAL, std::string("data pointer: ") + cudaGetErrorString(e));
        }
        if (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)
            return fail(EITHOT_EINVAL, "data must be device or managed memory");
    }
    // knobs recorded for this exact shape (an autotuner's choice) hold for
    // the planning and the run of this call
    eithot::Tuning shape_t;
    std::optional<eithot::ScopedTuning> shape_scope;
    if (rank >= 1 && dims && perm_1based &&
        eithot::shape_tuning(dims_of(rank, dims), perm_of(rank, perm_1based), elem_size, &shape_t))
        shape_scope.emplace(shape_t);
    eithot::NdPlan plan;
    std::vector<eithot::Pass> passes;
    rc = build(rank, dims, perm_1based, elem_size, num_sub_tensors, alpha, reorder_type, caps, &plan, &passes);
    if (rc) return rc;
    const double need = static_cast<double>(plan.padded_volume) * static_cast<double>(elem_size);
    if (need > static_cast<double>(capacity_bytes))
        return fail(EITHOT_EINVAL, "buffer capacity is smaller than the (padded) tensor");
    const double bytes = static_cast<double>(plan.volume) * static_cast<double>(elem_size);
    g_stats.algorithmic_bytes = 2.0 * bytes;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    size_t min_ws = 0;
    for (const auto& p : passes) min_ws = std::max(min_ws, eithot::pass_workspace_bytes(p, caps));
    eithot::ExecContext ctx;
    ctx.caps = caps;
    ctx.stream = st;
    ctx.profile = g_profile;
    ctx.events_used = g_events_used;
    ctx.events = &g_events;
    ctx.spans = &g_spans;
    ctx.names = &g_pass_names;
    ctx.bytes = &g_pass_bytes;
    size_t fb = 0, tb = 0;
    if (g_profile) {  // a device-wide query: only while profiling
        cudaMemGetInfo(&fb, &tb);
        g_stats.free_before = fb;
    }
    bool owned = false;
    if (d_workspace) {
        if (workspace_bytes < min_ws) return fail(EITHOT_ENOMEM, "caller workspace is smaller than eithot_workspace_size()");
        ctx.scratch = static_cast<uint8_t*>(d_workspace);
        ctx.scratch_bytes = workspace_bytes;
    } else {
        const size_t ws = choose_workspace(passes, caps, alpha, bytes);
        if (ws > 0) {
            void* p = nullptr;
            cudaError_t e = cudaMallocAsync(&p, ws, st);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return fail(EITHOT_ENOMEM, std::string("workspace allocation: ") + cudaGetErrorString(e));
            }
            ctx.scratch = static_cast<uint8_t*>(p);
            ctx.scratch_bytes = ws;
            owned = true;
        }
    }
    if (g_profile) {
        cudaMemGetInfo(&fb, &tb);
        g_stats.free_after_alloc = fb;
    }
    g_stats.workspace_bytes = ctx.scratch_bytes;
    {
        std::string err;
        if ((rc = eithot::begin_call(st, &g_last_call, &ctx.status, &err))) {
            if (owned) cudaFreeAsync(ctx.scratch, st);
            return fail(rc, err);
        }
    }
    rc = eithot::run_passes(static_cast<uint8_t*>(d_data), passes, ctx);
    g_events_used = ctx.events_used;
    if (owned) cudaFreeAsync(ctx.scratch, st);
    g_stats.n_passes = ctx.passes;
    g_stats.n_launches = ctx.launches;
    if (rc) return fail(rc, ctx.err);
    return EITHOT_OK;
}

// The no-allocation variant: scratch comes from the library's fixed device
// array instead of cudaMallocAsync.  For callers that may not allocate
// device memory during the call: their device memory is owned by another
// allocator (a framework's caching pool that has reserved the free HBM, so an
// extra allocation would fail or fragment it), or the call sits on a path
// that must not pay for an allocation.  Every call looks up the array's
// device address on the current device (cudaGetSymbolAddress, no
// allocation); make the first call on a device before any stream capture.
// All calls share the array and it keeps the
// last call's contents; nothing in it needs to start at zero.  Calls whose
// device work overlaps (other streams, other host threads) race on it.
int eithot_transpose_noalloc(void* d_data, size_t capacity_bytes, int rank, const int64_t* dims,
                             const int* perm_1based, size_t elem_size, int num_sub_tensors,
                             double alpha, void* stream) {
    std::memset(&g_stats, 0, sizeof(g_stats));
    if (!d_data) return fail(EITHOT_EINVAL, "null data pointer");
    eithot::DeviceCaps caps;
    int rc = device_caps(&caps);
    if (rc) return rc;
    {
        cudaPointerAttributes attr;
        cudaError_t e = cudaPointerGetAttributes(&attr, d_data);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(EITHOT_EINVAL, std::string("data pointer: ") + cudaGetErrorString(e));
        }
        if (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)
            return fail(EITHOT_EINVAL, "data must be device or managed memory");
    }
    eithot::NdPlan plan;
    std::vector<eithot::Pass> passes;
    rc = build(rank, dims, perm_1based, elem_size, num_sub_tensors, alpha, EITHOT_ORDER_MIXED, caps, &plan,
               &passes);
    if (rc) return rc;
    if (static_cast<double>(plan.padded_volume) * static_cast<double>(elem_size) > static_cast<double>(capacity_bytes))
        return fail(EITHOT_EINVAL, "buffer capacity is smaller than the (padded) tensor");
    size_t need = 0;
    for (const auto& p : passes) need = std::max(need, eithot::pass_workspace_bytes(p, caps));
    if (need > eithot::kNoAllocScratchBytes)
        return fail(EITHOT_EINVAL, "this transpose needs " + std::to_string(need) +
                                       " bytes of scratch, more than the fixed " +
                                       std::to_string(eithot::kNoAllocScratchBytes) +
                                       " bytes of eithot_transpose_noalloc; use eithot_transpose_ex");
    eithot::ExecContext ctx;
    ctx.caps = caps;
    ctx.stream = static_cast<cudaStream_t>(stream);
    if (need > 0) {
        std::string err;
        if ((rc = eithot::noalloc_scratch(&ctx.scratch, &err))) return fail(rc, err);
        ctx.scratch_bytes = eithot::kNoAllocScratchBytes;
    }
    g_stats.algorithmic_bytes = 2.0 * static_cast<double>(plan.volume) * static_cast<double>(elem_size);
    g_stats.workspace_bytes = ctx.scratch_bytes;
    {
        std::string err;
        if ((rc = eithot::begin_call(ctx.stream, &g_last_call, &ctx.status, &err))) return fail(rc, err);
    }
    rc = eithot::run_passes(static_cast<uint8_t*>(d_data), passes, ctx);
    g_stats.n_passes = ctx.passes;
    g_stats.n_launches = ctx.launches;
    if (rc) return fail(rc, ctx.err);
    return EITHOT_OK;
}

int eithot_transpose(void* d_data, size_t capacity_bytes, int rank, const int64_t* dims,
                     const int* perm_1based, size_t elem_size, int num_sub_tensors, double alpha,
                     void* stream) {
    return eithot_transpose_ex(d_data, capacity_bytes, rank, dims, perm_1based, elem_size,
                               num_sub_tensors, alpha, EITHOT_ORDER_MIXED, nullptr, 0, stream);
}

namespace {
int run_estimate(int rank, const int64_t* dims, const int* perm_1based, size_t elem_size, double alpha,
                 size_t smem_per_block, int padding_blocks, eithot::Estimate* est) {
    eithot::NdPlan plan;
    std::string err;
    if (!eithot::make_nd_plan(rank, dims, perm_1based, 1, alpha, EITHOT_ORDER_MIXED, &plan, &err))
        return fail(EITHOT_EINVAL, err);
    if (!elem_ok(elem_size)) return fail(EITHOT_EINVAL, "elem_size must be in [1, 64] bytes");
    if (!(alpha > 0.0)) return fail(EITHOT_EINVAL, "alpha must be positive");
    if (smem_per_block == 0 || padding_blocks <= 0) {
        int dev = 0, v = 0, sms = 152;
        size_t smem = 49152;
        if (cudaGetDevice(&dev) == cudaSuccess) {
            if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlock, dev) == cudaSuccess) smem = v;
            if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess) sms = v;
        } else {
            cudaGetLastError();
        }
        if (smem_per_block == 0) smem_per_block = smem;
        if (padding_blocks <= 0) padding_blocks = 2 * sms;
    }
    std::vector<int64_t> d(dims, dims + rank);
    std::vector<int> p(perm_1based, perm_1based + rank);
    eithot::estimate(d, p, elem_size, alpha, smem_per_block, static_cast<uint64_t>(padding_blocks), est);
    return EITHOT_OK;
}
}  // namespace

int eithot_estimate(int rank, const int64_t* dims, const int* perm_1based, size_t elem_size,
                    int num_sub_tensors, double alpha, size_t smem_per_block, int padding_blocks,
                    int* nb_out, double* alpha_out, size_t* extra_bytes_out) {
    (void)num_sub_tensors;  // the reference estimator ignores the requested nb
    eithot::Estimate est;
    if (int rc = run_estimate(rank, dims, perm_1based, elem_size, alpha, smem_per_block, padding_blocks, &est))
        return rc;
    if (nb_out) *nb_out = est.nb;
    if (alpha_out) *alpha_out = est.alpha;
    if (extra_bytes_out) *extra_bytes_out = est.final_tmp;
    return EITHOT_OK;
}

int eithot_estimate_report(int rank, const int64_t* dims, const int* perm_1based, size_t elem_size, double alpha,
                           size_t smem_per_block, int padding_blocks, eithot_estimate_info* info) {
    if (!info) return fail(EITHOT_EINVAL, "null info");
    eithot::Estimate est;
    if (int rc = run_estimate(rank, dims, perm_1based, elem_size, alpha, smem_per_block, padding_blocks, &est))
        return rc;
    info->nb = est.nb;
    info->alpha = est.alpha;
    info->init_extra_bytes = est.init_tmp;
    info->alpha_raised = est.alpha_raised;
    info->decomposed = est.decomposed ? 1 : 0;
    info->final_extra_bytes = est.final_tmp;
    info->final_ratio = est.ratio;
    return EITHOT_OK;
}

}  // extern "C"

namespace inplace {

void transpose(void* data, int source, int rank, void* dim, void* permutation, size_t sizeofType,
               int num_block, double LARGE_RATIO) {
    if (rank < 1 || !data || !dim || !permutation) {
        std::fprintf(stderr, "inplace::transpose: invalid arguments\n");
        return;
    }
    const int* d = static_cast<const int*>(dim);
    const int* p = static_cast<const int*>(permutation);
    std::vector<int64_t> dims(d, d + rank);
    std::vector<int> perm(rank);
    for (int i = 0; i < rank; ++i) perm[i] = p[i] + 1;
    uint8_t* base = static_cast<uint8_t*>(data) + static_cast<size_t>(source) * sizeofType;
    int rc = eithot_transpose(base, SIZE_MAX, rank, dims.data(), perm.data(), sizeofType, num_block,
                              LARGE_RATIO, nullptr);
    if (rc == EITHOT_OK) {
        cudaError_t e = cudaStreamSynchronize(nullptr);
        if (e != cudaSuccess) {
            std::fprintf(stderr, "inplace::transpose: %s\n", cudaGetErrorString(e));
            return;
        }
        uint64_t id = 0;
        int status = EITHOT_OK;
        if (eithot_last_call(&id) == EITHOT_OK && eithot_call_status(id, nullptr, &status) == EITHOT_OK &&
            status != EITHOT_OK)
            std::fprintf(stderr, "inplace::transpose: %s; the output is invalid\n",
                         status == EITHOT_ETIMEOUT ? "a bounded device wait gave up"
                                                   : "an index map left its row or column");
    } else {
        std::fprintf(stderr, "inplace::transpose: %s\n", eithot_last_error());
    }
}

}  // namespace inplace
