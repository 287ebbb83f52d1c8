// The served form: requests (tensors already resident on the device) are
// queued, admitted against a fixed workspace pool (or, for a request whose
// scratch exceeds the pool, against the device's free HBM) and run on a few
// executor streams.  Consecutive small requests at the head of the queue
// are run together as one batch (continuous batching); a large request runs
// alone.  Progress is made inside submit and poll calls (no thread of its
// own): a finished unit returns its workspace to the pool and its tickets to
// the caller, and the next units are dispatched.
#include <cuda_runtime.h>

#include <algorithm>
#include <deque>
#include <string>
#include <vector>

#include "api_util.h"
#include "eithot.h"
#include "exec.h"
#include "passes.h"
#include "plan.h"

using namespace eithot;
using namespace eithot::api;

namespace {

constexpr size_t kSmallBytes = 64ull << 20;     // requests below this are batched
constexpr size_t kBatchBytes = 1ull << 30;      // at most this much tensor data per batch
constexpr int kBatchCount = 1024;               // and at most this many requests
constexpr size_t kMaxQueue = 1 << 16;

struct Request {
    uint64_t ticket = 0;
    void* data = nullptr;
    size_t capacity = 0;
    int rank = 0;
    std::vector<int64_t> dims;
    std::vector<int> perm;
    size_t elem = 0;
    int nb = 1;
    double alpha = 0.01;
    size_t bytes = 0;
    size_t scratch = 0;  // workspace when run alone
    bool from_hbm = false;  // scratch beyond the pool: allocated from free HBM when it runs
};

// First-fit allocator over the pool (offsets, 256-byte granules).
struct Pool {
    size_t size = 0;
    std::vector<std::pair<size_t, size_t>> free_list;  // (offset, length), sorted
    void reset(size_t n) {
        size = n;
        free_list.assign(1, {0, n});
    }
    bool take(size_t n, size_t* off) {
        n = (n + 255) / 256 * 256;
        if (n == 0) { *off = 0; return true; }
        for (size_t i = 0; i < free_list.size(); ++i) {
            if (free_list[i].second >= n) {
                *off = free_list[i].first;
                free_list[i].first += n;
                free_list[i].second -= n;
                if (free_list[i].second == 0) free_list.erase(free_list.begin() + i);
                return true;
            }
        }
        return false;
    }
    void give(size_t off, size_t n) {
        n = (n + 255) / 256 * 256;
        if (n == 0) return;
        free_list.push_back({off, n});
        std::sort(free_list.begin(), free_list.end());
        std::vector<std::pair<size_t, size_t>> merged;
        for (auto& r : free_list) {
            if (!merged.empty() && merged.back().first + merged.back().second == r.first) merged.back().second += r.second;
            else merged.push_back(r);
        }
        free_list.swap(merged);
    }
};

struct Unit {
    std::vector<uint64_t> tickets;
    eithot_batch* batch = nullptr;
    size_t ws_off = 0, ws_bytes = 0;
    uint64_t call = 0;       // call id of a request run alone (its device status word)
    size_t resident = 0;     // tensor bytes the unit's requests occupy
    size_t own_scratch = 0;  // scratch taken from free HBM instead of the pool
    bool busy = false;
};

}  // namespace

struct eithot_server {
    int device = 0;
    DeviceCaps caps;
    uint8_t* pool_base = nullptr;
    Pool pool;
    std::deque<Request> queue;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    std::vector<Unit> units;   // one per stream
    std::vector<std::pair<uint64_t, int>> done;  // finished tickets and their status
    size_t resident = 0;       // tensor bytes of queued and running requests
    size_t hbm_scratch = 0;    // scratch of running requests allocated from free HBM
    uint64_t next_ticket = 1;
    int launches = 0;
    std::string last_err;
};

namespace {

// Headroom left free on the device when scratch beyond the pool is admitted.
constexpr size_t kHbmReserve = 256ull << 20;

// True when `bytes` more device memory is free now (cudaMemGetInfo), above
// the reserve.
bool hbm_fits(size_t bytes) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return free_b > kHbmReserve && bytes <= free_b - kHbmReserve;
}

// Dispatches the head of the queue onto stream `slot`; *started is false
// when the head waits for workspace.  A head that fails to start is dropped
// from the queue and its error returned.
int dispatch_one(eithot_server* s, int slot, bool* started) {
    *started = false;
    Unit& u = s->units[slot];
    const cudaStream_t st = s->streams[slot];
    Request& head = s->queue.front();
    // Runs the head alone, its scratch from the pool or (a request admitted
    // beyond the pool) from free HBM; false when it has to wait.
    auto run_alone = [&](int* rc) -> bool {
        size_t off = 0;
        if (head.from_hbm) {
            // admitted against free HBM: wait while other such requests hold it
            if (s->hbm_scratch > 0 && !hbm_fits(head.scratch + s->hbm_scratch)) return false;
        } else if (!s->pool.take(head.scratch, &off)) {
            return false;  // wait for workspace
        }
        *rc = eithot_transpose_ex(head.data, head.capacity, head.rank, head.dims.data(), head.perm.data(), head.elem,
                                  head.nb, head.alpha, EITHOT_ORDER_FEWEST,
                                  head.scratch && !head.from_hbm ? s->pool_base + off : nullptr,
                                  head.from_hbm ? 0 : head.scratch, st);
        if (*rc != EITHOT_OK) {
            if (!head.from_hbm) s->pool.give(off, head.scratch);
            s->resident -= head.capacity;
            s->queue.pop_front();
            return true;
        }
        eithot_stats stats;
        eithot_last_stats(&stats);
        s->launches += stats.n_launches;
        eithot_last_call(&u.call);
        u.tickets.assign(1, head.ticket);
        u.ws_off = head.from_hbm ? 0 : off;
        u.ws_bytes = head.from_hbm ? 0 : head.scratch;
        u.own_scratch = head.from_hbm ? head.scratch : 0;
        s->hbm_scratch += u.own_scratch;
        u.resident = head.capacity;
        s->queue.pop_front();
        return true;
    };
    if (head.bytes >= kSmallBytes || head.from_hbm) {
        // a large request runs alone with its own workspace
        int rc = EITHOT_OK;
        if (!run_alone(&rc)) return EITHOT_OK;
        if (rc != EITHOT_OK) return rc;
    } else {
        // consecutive small requests at the head of the queue, one batch
        std::vector<int> ranks;
        std::vector<int64_t> dims;
        std::vector<int> perms;
        std::vector<size_t> elems;
        std::vector<void*> ptrs;
        std::vector<size_t> caps;
        size_t total = 0;
        size_t n = 0;
        int nb = s->queue.front().nb;
        double alpha = s->queue.front().alpha;
        while (n < s->queue.size() && static_cast<int>(n) < kBatchCount) {
            const Request& r = s->queue[n];
            if (r.bytes >= kSmallBytes || r.from_hbm || r.nb != nb || r.alpha != alpha) break;
            if (n > 0 && total + r.bytes > kBatchBytes) break;
            ranks.push_back(r.rank);
            dims.insert(dims.end(), r.dims.begin(), r.dims.end());
            perms.insert(perms.end(), r.perm.begin(), r.perm.end());
            elems.push_back(r.elem);
            ptrs.push_back(r.data);
            caps.push_back(r.capacity);
            total += r.bytes;
            ++n;
        }
        eithot_batch* b = nullptr;
        auto drop = [&]() {
            for (size_t i = 0; i < n; ++i) {
                s->resident -= s->queue.front().capacity;
                s->queue.pop_front();
            }
        };
        int rc = eithot_batch_create(static_cast<int>(n), ranks.data(), dims.data(), perms.data(), elems.data(), nb,
                                     alpha, &b);
        if (rc != EITHOT_OK) {
            drop();
            return rc;
        }
        size_t need = 0, off = 0;
        eithot_batch_workspace_size(b, &need);
        // The batch plans its tensors for concurrent lanes, so its workspace
        // (the sum over lanes) can exceed what any one request needs alone:
        // halve the batch until it fits the pool; a single request that still
        // does not fit runs alone, as a large request does.
        while (need > s->pool.size && n > 1) {
            eithot_batch_destroy(b);
            b = nullptr;
            n = (n + 1) / 2;
            ranks.resize(n);
            elems.resize(n);
            ptrs.resize(n);
            caps.resize(n);
            size_t nd = 0;
            for (size_t i = 0; i < n; ++i) nd += static_cast<size_t>(ranks[i]);
            dims.resize(nd);
            perms.resize(nd);
            rc = eithot_batch_create(static_cast<int>(n), ranks.data(), dims.data(), perms.data(), elems.data(), nb,
                                     alpha, &b);
            if (rc != EITHOT_OK) {
                drop();
                return rc;
            }
            eithot_batch_workspace_size(b, &need);
        }
        if (need > s->pool.size) {
            eithot_batch_destroy(b);
            int rc1 = EITHOT_OK;
            if (!run_alone(&rc1)) return EITHOT_OK;
            if (rc1 != EITHOT_OK) return rc1;
            u.busy = true;
            *started = true;
            const cudaError_t e = cudaEventRecord(s->events[slot], st);
            if (e != cudaSuccess) return fail(EITHOT_ECUDA, std::string("server: ") + cudaGetErrorString(e));
            return EITHOT_OK;
        }
        if (!s->pool.take(need, &off)) {
            eithot_batch_destroy(b);
            return EITHOT_OK;  // wait for workspace
        }
        rc = eithot_batch_run(b, ptrs.data(), caps.data(), need ? s->pool_base + off : nullptr, need, st);
        if (rc != EITHOT_OK) {
            s->pool.give(off, need);
            eithot_batch_destroy(b);
            drop();
            return rc;
        }
        int l = 0;
        eithot_batch_launches(b, &l);
        s->launches += l;
        u.tickets.clear();
        u.resident = 0;
        for (size_t i = 0; i < n; ++i) {
            u.tickets.push_back(s->queue.front().ticket);
            u.resident += s->queue.front().capacity;
            s->queue.pop_front();
        }
        u.batch = b;
        u.ws_off = off;
        u.ws_bytes = need;
    }
    u.busy = true;
    *started = true;
    const cudaError_t e = cudaEventRecord(s->events[slot], st);
    if (e != cudaSuccess) return fail(EITHOT_ECUDA, std::string("server: ") + cudaGetErrorString(e));
    return EITHOT_OK;
}

// Retires finished units, then dispatches queued requests onto free streams.
int pump(eithot_server* s) {
    for (size_t i = 0; i < s->units.size(); ++i) {
        Unit& u = s->units[i];
        if (!u.busy) continue;
        const cudaError_t q = cudaEventQuery(s->events[i]);
        if (q == cudaErrorNotReady) continue;
        if (q != cudaSuccess) return fail(EITHOT_ECUDA, std::string("server: ") + cudaGetErrorString(q));
        int status = EITHOT_OK;
        if (u.call) {
            // the unit's stream has finished: reading its status word does not wait
            if (eithot_call_status(u.call, s->streams[i], &status) != EITHOT_OK) status = EITHOT_ECUDA;
        }
        for (uint64_t t : u.tickets) s->done.push_back({t, status});
        s->pool.give(u.ws_off, u.ws_bytes);
        s->resident -= u.resident;
        s->hbm_scratch -= u.own_scratch;
        if (u.batch) eithot_batch_destroy(u.batch);
        u = Unit();
    }
    for (size_t i = 0; i < s->units.size() && !s->queue.empty(); ++i) {
        if (s->units[i].busy) continue;
        bool started = false;
        if (int rc = dispatch_one(s, static_cast<int>(i), &started)) return rc;
        if (!started) break;  // the head waits for workspace
    }
    return EITHOT_OK;
}

}  // namespace

extern "C" {

int eithot_server_create(size_t workspace_bytes, int streams, eithot_server** out) {
    if (!out) return fail(EITHOT_EINVAL, "null out");
    *out = nullptr;
    if (streams < 1 || streams > 16) return fail(EITHOT_EINVAL, "streams must be 1..16");
    auto* s = new eithot_server();
    if (int rc = device_caps(&s->caps)) {
        delete s;
        return rc;
    }
    cudaGetDevice(&s->device);
    if (workspace_bytes) {
        void* p = nullptr;
        const cudaError_t e = cudaMalloc(&p, workspace_bytes);
        if (e != cudaSuccess) {
            delete s;
            cudaGetLastError();
            return fail(EITHOT_ENOMEM, std::string("server workspace: ") + cudaGetErrorString(e));
        }
        s->pool_base = static_cast<uint8_t*>(p);
    }
    s->pool.reset(workspace_bytes);
    for (int i = 0; i < streams; ++i) {
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        s->streams.push_back(st);
        s->events.push_back(ev);
    }
    s->units.resize(streams);
    *out = s;
    return EITHOT_OK;
}

int eithot_server_submit(eithot_server* s, void* d_data, size_t capacity_bytes, int rank, const int64_t* dims,
                         const int* perm_1based, size_t elem_size, int num_sub_tensors, double alpha,
                         uint64_t* ticket) {
    if (!s || !d_data || !dims || !perm_1based || !ticket) return fail(EITHOT_EINVAL, "null argument");
    if (s->queue.size() >= kMaxQueue) return fail(EITHOT_EBUSY, "server queue is full");
    Request r;
    NdPlan plan;
    std::vector<Pass> passes;
    if (int rc = build(rank, dims, perm_1based, elem_size, num_sub_tensors, alpha, EITHOT_ORDER_FEWEST, s->caps,
                       &plan, &passes))
        return rc;
    r.bytes = static_cast<size_t>(plan.volume) * elem_size;
    if (static_cast<double>(plan.padded_volume) * elem_size > static_cast<double>(capacity_bytes))
        return fail(EITHOT_EINVAL, "buffer capacity is smaller than the (padded) tensor");
    r.scratch = choose_workspace(passes, s->caps, alpha, static_cast<double>(r.bytes));
    if (r.scratch > s->pool.size) {
        // beyond the pool: admitted against the device's free HBM (its
        // scratch allocated when it runs), refused when that cannot hold it
        if (!hbm_fits(r.scratch)) return fail(EITHOT_EBUSY, "request needs more workspace than the server's pool "
                                                            "holds and than the device has free");
        r.from_hbm = true;
    }
    r.ticket = s->next_ticket++;
    r.data = d_data;
    r.capacity = capacity_bytes;
    r.rank = rank;
    r.dims.assign(dims, dims + rank);
    r.perm.assign(perm_1based, perm_1based + rank);
    r.elem = elem_size;
    r.nb = num_sub_tensors;
    r.alpha = alpha;
    *ticket = r.ticket;
    s->resident += capacity_bytes;
    s->queue.push_back(std::move(r));
    return pump(s);
}

int eithot_server_poll_status(eithot_server* s, uint64_t* done, int* statuses, int max_done, int* n_done) {
    if (!s || !n_done || (max_done > 0 && !done)) return fail(EITHOT_EINVAL, "null argument");
    if (int rc = pump(s)) return rc;
    const int n = std::min<int>(max_done, static_cast<int>(s->done.size()));
    for (int i = 0; i < n; ++i) {
        done[i] = s->done[i].first;
        if (statuses) statuses[i] = s->done[i].second;
    }
    s->done.erase(s->done.begin(), s->done.begin() + n);
    *n_done = n;
    return EITHOT_OK;
}

int eithot_server_poll(eithot_server* s, uint64_t* done, int max_done, int* n_done) {
    return eithot_server_poll_status(s, done, nullptr, max_done, n_done);
}

int eithot_server_memory(const eithot_server* s, size_t* resident_bytes, size_t* pool_bytes, size_t* hbm_scratch_bytes) {
    if (!s) return fail(EITHOT_EINVAL, "null server");
    if (resident_bytes) *resident_bytes = s->resident;
    if (pool_bytes) *pool_bytes = s->pool.size;
    if (hbm_scratch_bytes) *hbm_scratch_bytes = s->hbm_scratch;
    return EITHOT_OK;
}

int eithot_server_pending(const eithot_server* s, int* queued, int* running) {
    if (!s || !queued || !running) return fail(EITHOT_EINVAL, "null argument");
    *queued = static_cast<int>(s->queue.size());
    *running = 0;
    for (const auto& u : s->units) *running += u.busy ? static_cast<int>(u.tickets.size()) : 0;
    return EITHOT_OK;
}

int eithot_server_launches(const eithot_server* s, int* launches) {
    if (!s || !launches) return fail(EITHOT_EINVAL, "null argument");
    *launches = s->launches;
    return EITHOT_OK;
}

int eithot_server_destroy(eithot_server* s) {
    if (!s) return EITHOT_OK;
    for (auto st : s->streams) cudaStreamSynchronize(st);
    for (auto& u : s->units)
        if (u.batch) eithot_batch_destroy(u.batch);
    for (auto st : s->streams) cudaStreamDestroy(st);
    for (auto ev : s->events) cudaEventDestroy(ev);
    if (s->pool_base) cudaFree(s->pool_base);
    delete s;
    return EITHOT_OK;
}

}  // extern "C"
