// Test infrastructure: applies the library's lowered pass list on host
// memory with the same index maps the kernels use (eithot_gb300/csrc/
// fn_build.h, index_math.cuh).  It checks the planner -> lowering ->
// index-map chain on the CPU; the device kernels are checked separately by
// the GPU tests.  Never loaded by the product.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fn_build.h"
#include "passes.h"
#include "plan.h"
#include "search.h"

using namespace eithot;

namespace {

thread_local std::string g_err;

template <typename Fn>
void col_gather(uint8_t* base, const Pass& p, const Fn& fn) {
    const uint64_t E = p.elem, R = p.rows, C = p.cols;
    std::vector<uint8_t> tmp(R * E);
    for (uint64_t b = 0; b < p.batches; ++b) {
        uint8_t* m = base + b * R * C * E;
        for (uint64_t j = 0; j < C; ++j) {
            for (uint64_t i = 0; i < R; ++i) std::memcpy(&tmp[i * E], m + (i * C + j) * E, E);
            for (uint64_t i = 0; i < R; ++i) std::memcpy(m + (i * C + j) * E, &tmp[fn(i, j) * E], E);
        }
    }
}

// Input index (in the pass's axes) of output index o: output axis j is
// input axis perm[j].
uint64_t nd_src(const std::vector<uint64_t>& dims, const std::vector<int>& perm, uint64_t o) {
    const size_t q = dims.size();
    std::vector<uint64_t> in_stride(q);
    uint64_t st = 1;
    for (size_t i = 0; i < q; ++i) {
        in_stride[i] = st;
        st *= dims[i];
    }
    uint64_t idx = 0;
    for (size_t j = 0; j < q; ++j) {
        const uint64_t d = dims[perm[j]];
        idx += (o % d) * in_stride[perm[j]];
        o /= d;
    }
    return idx;
}

void apply(uint8_t* data, const Pass& p) {
    uint8_t* base = data + p.offset;
    const uint64_t E = p.elem;
    switch (p.type) {
        case kSlabPerm: {
            uint64_t count = 1;
            for (auto d : p.nd_dims) count *= d;
            std::vector<uint8_t> tmp(count * E);
            for (uint64_t b = 0; b < p.batches; ++b) {
                uint8_t* m = base + b * count * E;
                std::memcpy(tmp.data(), m, count * E);
                for (uint64_t o = 0; o < count; ++o)
                    std::memcpy(m + o * E, &tmp[nd_src(p.nd_dims, p.nd_perm, o) * E], E);
            }
            break;
        }
        case kBlockPerm: {
            // the device algorithm, in place: save every segment's head,
            // then walk every segment backwards from its tail
            const CycleTable& tab = cycle_table(p.nd_dims, p.nd_perm);
            const uint64_t blk = p.block, nseg = tab.head.size();
            std::vector<uint8_t> saved(nseg * blk);
            for (uint64_t k = 0; k < nseg; ++k) std::memcpy(&saved[k * blk], base + tab.head[k] * blk, blk);
            for (uint64_t k = 0; k < nseg; ++k) {
                uint64_t t = tab.tail[k];
                for (uint64_t step = 0; step < tab.len[k]; ++step) {
                    const uint64_t src = nd_src(p.nd_dims, p.nd_perm, t);
                    const uint8_t* from = step + 1 == tab.len[k] ? &saved[k * blk] : base + src * blk;
                    std::memmove(base + t * blk, from, blk);
                    t = src;
                }
            }
            break;
        }
        case kSlabCluster:
        case kSlabTranspose: {
            const uint64_t R = p.rows, C = p.cols;
            std::vector<uint8_t> tmp(R * C * E);
            for (uint64_t b = 0; b < p.batches; ++b) {
                uint8_t* m = base + b * R * C * E;
                std::memcpy(tmp.data(), m, R * C * E);
                for (uint64_t o = 0; o < R * C; ++o) {
                    const uint64_t c = o / R, r = o % R;
                    std::memcpy(m + o * E, &tmp[(r * C + c) * E], E);
                }
            }
            break;
        }
        case kRowGather:
        case kRowScatter: {
            const FnRowShuffle fn = make_rowshuffle<uint64_t>(p);
            std::vector<uint8_t> tmp(p.cols * E);
            for (uint64_t bi = 0; bi < p.batches * p.rows; ++bi) {
                const uint64_t i = bi % p.rows;
                uint8_t* row = base + bi * p.cols * E;
                std::memcpy(tmp.data(), row, p.cols * E);
                for (uint64_t j = 0; j < p.cols; ++j) {
                    if (p.type == kRowGather) std::memcpy(row + j * E, &tmp[fn(i, j) * E], E);
                    else std::memcpy(row + fn(i, j) * E, &tmp[j * E], E);
                }
            }
            break;
        }
        case kColGather:
            switch (p.fn) {
                case kFnC2RPreRot: col_gather(base, p, make_prerot<uint64_t>(p)); break;
                case kFnC2RColShuffle: col_gather(base, p, make_c2r_colshuf<uint64_t>(p)); break;
                case kFnR2CColShuffle: col_gather(base, p, make_r2c_colshuf<uint64_t>(p)); break;
                case kFnR2CPostRot: col_gather(base, p, make_postrot<uint64_t>(p)); break;
            }
            break;
        case kBlockMove:
            if (p.dst_pitch > p.src_pitch) {
                for (uint64_t s = p.n_blocks; s-- > 1;)
                    std::memmove(data + s * p.dst_pitch, data + s * p.src_pitch, p.block);
            } else {
                for (uint64_t s = 1; s < p.n_blocks; ++s)
                    std::memmove(data + s * p.dst_pitch, data + s * p.src_pitch, p.block);
            }
            break;
    }
}

// The pass list the C ABI executes for this plan: the lowered reference
// series, replaced by the pass-minimising search's when the request asks for
// the fewest passes and the search finds a clearly cheaper plan (as
// eithot_transpose_ex decides it).
bool lower_plan_as_executed(const NdPlan& plan, size_t elem, int order, const DeviceCaps& caps,
                            std::vector<Pass>* passes) {
    if (!lower_plan(plan, elem, caps, passes, &g_err)) return false;
    if (order == kOrderFewest && plan.nb == 1 && !plan.padded) {
        std::vector<Pass> alt;
        double cost = 0;
        if (search_plan(plan.dims, plan.perm, elem, caps, &alt, &cost, nullptr) &&
            cost < passes_model_cost(*passes, caps) - 0.2)
            passes->swap(alt);
    }
    return true;
}

}  // namespace

extern "C" {

const char* hs_last_error() { return g_err.c_str(); }

// Returns the number of passes applied, or -1 on error.
int hs_transpose(void* data, size_t capacity, int rank, const int64_t* dims, const int* perm,
                 size_t elem, int nb, double alpha, int order) {
    NdPlan plan;
    if (!make_nd_plan(rank, dims, perm, nb, alpha, order, &plan, &g_err)) return -1;
    if (static_cast<double>(plan.padded_volume) * elem > static_cast<double>(capacity)) {
        g_err = "capacity";
        return -1;
    }
    std::vector<Pass> passes;
    DeviceCaps caps;
    if (!lower_plan_as_executed(plan, elem, order, caps, &passes)) return -1;
    for (const Pass& p : passes) apply(static_cast<uint8_t*>(data), p);
    return static_cast<int>(passes.size());
}

// Writes a one-line description per pass into buf (newline separated).
int hs_describe(char* buf, size_t len, int rank, const int64_t* dims, const int* perm, size_t elem,
                int nb, double alpha, int order) {
    NdPlan plan;
    if (!make_nd_plan(rank, dims, perm, nb, alpha, order, &plan, &g_err)) return -1;
    std::vector<Pass> passes;
    DeviceCaps caps;
    if (!lower_plan_as_executed(plan, elem, order, caps, &passes)) return -1;
    std::string s;
    for (const Pass& p : passes) s += p.what + "\n";
    std::strncpy(buf, s.c_str(), len);
    if (len) buf[len - 1] = 0;
    return static_cast<int>(passes.size());
}

// One line per pass: its description and, for column passes, the staging
// the executor will use (form, CTAs per tile, row-piece bytes, buffering).
int hs_describe_staging(char* buf, size_t len, int rank, const int64_t* dims, const int* perm, size_t elem,
                        int nb, double alpha, int order) {
    NdPlan plan;
    if (!make_nd_plan(rank, dims, perm, nb, alpha, order, &plan, &g_err)) return -1;
    std::vector<Pass> passes;
    DeviceCaps caps;
    if (!lower_plan_as_executed(plan, elem, order, caps, &passes)) return -1;
    std::string s;
    for (const Pass& p : passes) {
        s += p.what;
        if (p.type == kColGather) {
            const Staging st = plan_col_pass(p, caps);
            char tmp[256];
            std::snprintf(tmp, sizeof(tmp), " | %s K=%d G=%d piece=%llu dbuf=%d per_cta=%llu halo=%llu+%llu cost=%.3f",
                          !st.on_chip ? "staged" : st.group ? "group" : st.whole ? "whole-tile" : st.owner ? "cluster-owner" : "cluster-gather",
                          st.K, st.G, static_cast<unsigned long long>(st.pitch), st.dbuf ? 1 : 0,
                          static_cast<unsigned long long>(st.per_cta), static_cast<unsigned long long>(st.hlo),
                          static_cast<unsigned long long>(st.hhi), st.cost);
            s += tmp;
        }
        s += "\n";
    }
    std::strncpy(buf, s.c_str(), len);
    if (len) buf[len - 1] = 0;
    return static_cast<int>(passes.size());
}

// Shared memory every owner-computed column pass of the plan launches with,
// computed as the executor computes it (the slot buffer(s), 128-byte
// rounded, then the row tables: Q + Hlo + Hhi source rows and Q output rows
// of the pass's index type, 16-byte rounded), against what the planner may
// use: at most the per-block opt-in limit, and for group passes at most the
// SM's share for the planned CTAs per SM less the 1 KB the hardware
// reserves per block.  Returns the number of passes over budget (or -1).
long hs_check_owner_smem(int rank, const int64_t* dims, const int* perm, size_t elem, int nb, double alpha,
                         int order, int* owner_passes) {
    NdPlan plan;
    if (!make_nd_plan(rank, dims, perm, nb, alpha, order, &plan, &g_err)) return -1;
    std::vector<Pass> passes;
    DeviceCaps caps;
    if (!lower_plan(plan, elem, caps, &passes, &g_err)) return -1;
    long bad = 0;
    int owners = 0;
    for (const Pass& p : passes) {
        if (p.type != kColGather) continue;
        const Staging st = plan_col_pass(p, caps);
        if (!st.on_chip || !st.owner) continue;
        ++owners;
        const uint64_t parts = st.group ? static_cast<uint64_t>(st.G) : static_cast<uint64_t>(st.K);
        const uint64_t Q = (p.rows + parts - 1) / parts;
        const uint64_t slots = Q + st.hlo + st.hhi;
        const uint64_t buf = (slots * st.pitch + 127) / 128 * 128;
        const uint64_t idx = fits32(p) ? 4 : 8;
        const uint64_t tables = ((2 * Q + st.hlo + st.hhi) * idx + 15) / 16 * 16;
        const uint64_t smem = (st.dbuf ? 2 : 1) * buf + tables;
        bool over = smem > caps.smem_optin;
        if (st.group) over = over || smem + 1024 > caps.smem_per_sm / static_cast<uint64_t>(st.per_sm);
        if (over) {
            ++bad;
            g_err = p.what + ": " + std::to_string(smem) + " bytes of shared memory";
        }
    }
    if (owner_passes) *owner_passes = owners;
    return bad;
}

// Compares the 32-bit flavour of every Catanzaro map the plan uses with the
// 64-bit flavour over all (i, j) when m*n <= max_full, else a strided
// sample.  Returns the number of disagreements (or -1 on error).
long hs_check_fn32(int rank, const int64_t* dims, const int* perm, size_t elem, int nb, double alpha,
                   int order, long max_full) {
    NdPlan plan;
    if (!make_nd_plan(rank, dims, perm, nb, alpha, order, &plan, &g_err)) return -1;
    std::vector<Pass> passes;
    DeviceCaps caps;
    if (!lower_plan(plan, elem, caps, &passes, &g_err)) return -1;
    long bad = 0;
    for (const Pass& p : passes) {
        if (p.type != kRowGather && p.type != kRowScatter && p.type != kColGather) continue;
        if (!fits32(p)) continue;
        const uint64_t total = p.m * p.n;
        const uint64_t stride = total <= static_cast<uint64_t>(max_full) ? 1 : total / max_full + 1;
        for (uint64_t x = 0; x < total; x += stride) {
            const uint64_t i = x / p.n, j = x % p.n;
            uint64_t a = 0, b = 0;
            switch (p.type == kColGather ? p.fn : -1) {
                case -1: a = make_rowshuffle<uint64_t>(p)(i, j); b = make_rowshuffle<uint32_t>(p)(i, j); break;
                case kFnC2RPreRot: a = make_prerot<uint64_t>(p)(i, j); b = make_prerot<uint32_t>(p)(i, j); break;
                case kFnC2RColShuffle: a = make_c2r_colshuf<uint64_t>(p)(i, j); b = make_c2r_colshuf<uint32_t>(p)(i, j); break;
                case kFnR2CColShuffle: a = make_r2c_colshuf<uint64_t>(p)(i, j); b = make_r2c_colshuf<uint32_t>(p)(i, j); break;
                case kFnR2CPostRot: a = make_postrot<uint64_t>(p)(i, j); b = make_postrot<uint32_t>(p)(i, j); break;
            }
            if (a != b) ++bad;
        }
    }
    return bad;
}

// For every row pass of the plan, checks that the inverse map undoes the
// row shuffle (both flavours) on all (i, j) when m*n <= max_full, else a
// strided sample.  Returns the number of failures (or -1 on error).
long hs_check_inverse(int rank, const int64_t* dims, const int* perm, size_t elem, int nb, double alpha,
                      int order, long max_full) {
    NdPlan plan;
    if (!make_nd_plan(rank, dims, perm, nb, alpha, order, &plan, &g_err)) return -1;
    std::vector<Pass> passes;
    DeviceCaps caps;
    if (!lower_plan(plan, elem, caps, &passes, &g_err)) return -1;
    long bad = 0;
    for (const Pass& p : passes) {
        if (p.type != kRowGather && p.type != kRowScatter) continue;
        const auto f = make_rowshuffle<uint64_t>(p);
        const auto h = make_rowshuffle_inv<uint64_t>(p);
        const bool f32ok = fits32(p);
        const uint64_t total = p.m * p.n;
        const uint64_t stride = total <= static_cast<uint64_t>(max_full) ? 1 : total / max_full + 1;
        for (uint64_t x = 0; x < total; x += stride) {
            const uint64_t i = x / p.n, j = x % p.n;
            if (f(i, h(i, j)) != j || h(i, f(i, j)) != j) ++bad;
            if (f32ok) {
                const auto h32 = make_rowshuffle_inv<uint32_t>(p);
                if (h32(static_cast<uint32_t>(i), static_cast<uint32_t>(j)) != h(i, j)) ++bad;
            }
        }
    }
    return bad;
}

}  // extern "C"

namespace {
// Checks one owner map against the column gather it replaces: for tiles of
// tw columns starting at j0, slot t's output row i = row_of(t, j0) must take,
// at column j0 + c, the source row the gather names, held by slot
// t + delta(j0 + c) - delta(j0), within the planned halo.
template <typename Own, typename Fn>
long check_owner(const Pass& p, const Own& own, const Fn& g, uint64_t tw, long max_full) {
    uint64_t lo, hi;
    owner_halo(p.fn, p.b, tw, &lo, &hi);
    long bad = 0;
    const uint64_t m = p.m, n = p.n;
    const uint64_t ntiles = (n + tw - 1) / tw;
    const uint64_t total = m * ntiles;
    const uint64_t stride = total <= static_cast<uint64_t>(max_full) ? 1 : total / max_full + 1;
    std::vector<uint8_t> seen;
    for (uint64_t x = 0; x < total; x += stride) {
        const uint64_t t = x % m, j0 = (x / m) * tw;
        using I = typename Own::index_type;
        const uint64_t i = own.row_of(static_cast<I>(t), static_cast<I>(j0));
        if (i >= m) { ++bad; continue; }
        if (stride == 1) {  // row_of(., j0) is a bijection of the m slots
            if (t == 0) seen.assign(m, 0);
            if (seen[i]++) ++bad;
        }
        for (uint64_t c = 0; c < tw && j0 + c < n; ++c) {
            const int64_t d = own.delta(static_cast<I>(j0 + c)) - own.delta(static_cast<I>(j0));
            if (d < -static_cast<int64_t>(lo) || d > static_cast<int64_t>(hi)) { ++bad; continue; }
            const int64_t sm = static_cast<int64_t>(m);
            const uint64_t slot = static_cast<uint64_t>(((static_cast<int64_t>(t) + d) % sm + sm) % sm);
            if (static_cast<uint64_t>(own.stage_of(static_cast<I>(slot))) != static_cast<uint64_t>(g(i, j0 + c))) ++bad;
        }
    }
    return bad;
}

template <typename I>
long check_owner_pass(const Pass& p, uint64_t tw, long max_full) {
    switch (p.fn) {
        case kFnC2RPreRot: return check_owner(p, make_owner_prerot<I>(p), make_prerot<uint64_t>(p), tw, max_full);
        case kFnC2RColShuffle: return check_owner(p, make_owner_colshuf<I>(p), make_c2r_colshuf<uint64_t>(p), tw, max_full);
        case kFnR2CColShuffle: return check_owner(p, make_owner_r2c_colshuf<I>(p), make_r2c_colshuf<uint64_t>(p), tw, max_full);
        case kFnR2CPostRot: return check_owner(p, make_owner_postrot<I>(p), make_postrot<uint64_t>(p), tw, max_full);
        default: return 0;
    }
}
}  // namespace

extern "C" {

// Owner-computed column passes of both 2D variants of the plan agree with
// the column gathers they stand for (tiles of 1..128 columns); returns the
// number of disagreements, -1 on a planning error.  Counts every column pass
// visited in *n_checked.
long hs_check_owner(int rank, const int64_t* dims, const int* perm, size_t elem, int nb, double alpha,
                    int order, long max_full, long* n_checked) {
    NdPlan plan;
    if (!make_nd_plan(rank, dims, perm, nb, alpha, order, &plan, &g_err)) return -1;
    long bad = 0, visited = 0;
    const int saved = tuning().variant;
    for (int variant : {1, 2}) {
        tuning().variant = variant;
        std::vector<Pass> passes;
        DeviceCaps caps;
        if (!lower_plan(plan, elem, caps, &passes, &g_err)) { tuning().variant = saved; return -1; }
        for (const Pass& p : passes) {
            if (p.type != kColGather) continue;
            ++visited;
            for (uint64_t tw : {1, 2, 4, 8, 16, 32, 128}) {
                bad += check_owner_pass<uint64_t>(p, tw, max_full);
                if (fits32(p)) bad += check_owner_pass<uint32_t>(p, tw, max_full);
            }
        }
    }
    tuning().variant = saved;
    if (n_checked) *n_checked = visited;
    return bad;
}

}  // extern "C"

extern "C" {

// Sets one lowering knob of this process (max_cluster, col_form, factor,
// slab_cluster); returns 0, or -1 for an unknown key.
int hs_tune(const char* key, int value) {
    const std::string k(key);
    Tuning& t = tuning();
    if (k == "max_cluster") t.max_cluster = value;
    else if (k == "col_form") t.col_form = value;
    else if (k == "group_per_sm") t.group_per_sm = value;
    else if (k == "dbuf") t.dbuf = value;
    else if (k == "factor") t.factor = value;
    else if (k == "slab_cluster") t.slab_cluster = value;
    else if (k == "slab_colband") t.slab_colband = value;
    else return -1;
    return 0;
}

}  // extern "C"
