// Pass-minimising plans (see search.h).
//
// The reference decomposes a permutation into a series of low-order
// transposes chosen by a fixed rule (pre/post/mixed order,
// ITNT/src/Nd_transpose.cpp:146-250) and lowers each separately.  Its
// 4D/5D single-pass "linearisations" (_4d::_1432, _4d::_3214,
// _5d::_14325/_15432/_43215, ITNT/src/4dtranspose.cpp:194-315,
// ITNT/src/5dtranspose.cpp:59-273) are written but never reached.  Here the
// series is searched instead: states are arrangements of the tensor's axes
// (after merging axes that stay adjacent), moves are
//   X     a batched 2D transpose of two adjacent axis groups, lowered and
//         costed exactly as a reference round is (slab, cluster slab,
//         Catanzaro, factor split);
//   slab  the leading axes of a slab (that fits one CTA's shared memory,
//         elements of any width) permuted into the target's order of those
//         axes, every slab independently: one pass (_3214 and _43215 keep
//         their last axes; here any number of trailing axes stays);
//   cycle blocks of the leading axes (at least 4 KB) permuted as units into
//         the target's order of the other axes, by following the
//         permutation's cycles: one pass plus a copy of one block per
//         segment (_1432, _14325, _15432 keep their first axis; here any
//         leading block stays);
// and Dijkstra's algorithm finds the cheapest sequence under the cost model.
#include "search.h"

#include <algorithm>
#include <map>
#include <mutex>
#include <queue>
#include <sstream>
#include <tuple>

#include "index_math.cuh"

namespace eithot {

uint64_t slab_perm_capacity(const DeviceCaps& caps) { return smem_cap_of(caps); }

uint64_t slab_perm_strip(uint64_t E, uint64_t count, const DeviceCaps& caps) {
    return strip_width(E, count, slab_perm_capacity(caps));
}

namespace {

// True when a slab permutation's write-back runs qualify for offsets read
// from a table (the run kernel's aligned form): with runs of K = V / E
// outputs per V-byte store (V the largest power of two up to 16 dividing the
// slab's bytes), the output dims below some axis m multiply to a divisor of
// K that K times ... divides the product up to and including axis m.
bool slab_runs_aligned(uint64_t E, const std::vector<uint64_t>& odims) {
    if (E > 16 || (E & (E - 1)) != 0) return false;
    uint64_t count = 1;
    for (auto d : odims) count *= d;
    uint64_t V = 16;
    while (V > E && (count * E) % V != 0) V /= 2;
    if (V < 4 || V < E) return false;
    const uint64_t K = V / E;
    uint64_t P = 1;
    for (uint64_t d : odims) {
        if (K % P == 0 && (P * d) % K == 0) return true;
        P *= d;
        if (P > K) return false;
    }
    return false;
}

// Modelled cost of a slab permutation of `count` elements of E bytes per
// slab (`odims`: the slab's dims in output order), the copy rate over the
// rate measured on GB300.  Runs with table offsets (3- and 4-axis slabs of
// 64-128 KB): E = 16, 32: 6.0-6.1 TB/s; 8: 4.8; 4: 4.6-5.7; 2: 4.8-6.2;
// slabs of 110 KB or less run two CTAs per SM without register prefetch and
// sit at the low end.  Runs stepping through the axes per element: E = 8:
// 3.6-3.8; 4: 2.4-3.0; 2: 1.4-1.9; 1: 0.7-1.0.
double slab_perm_cost(uint64_t E, uint64_t count, const std::vector<uint64_t>& odims, const DeviceCaps& caps) {
    const uint64_t w = slab_perm_strip(E, count, caps);
    const uint64_t bytes = count * w;
    if (bytes > slab_perm_capacity(caps)) return -1.0;
    if (E >= 16) return 1.08;
    if (slab_runs_aligned(E, odims)) {
        const double c = E >= 8 ? 1.3 : E >= 4 ? 1.15 : E >= 2 ? 1.1 : 1.6;
        return bytes <= 110 * 1024 ? c + 0.25 : c;
    }
    return E >= 8 ? 1.8 : E >= 4 ? 2.4 : E >= 2 ? 4.0 : 7.5;
}

// Extra cost of a lowered 2D transpose the lowering's model underrates:
// one-CTA slab transposes of 1- and 2-byte elements whose rows are short
// (64 bytes or less) ran at 0.9-2.1 TB/s on GB300 against the 1.0-1.25
// passes the model gives any slab.
double narrow_slab_penalty(const std::vector<Pass>& ps) {
    double c = 0;
    for (const Pass& p : ps)
        if (p.type == kSlabTranspose && p.elem <= 2 && p.cols * p.elem <= 64) c += p.elem == 1 ? 5.0 : 2.0;
    return c;
}

// Modelled cost of moving `n` blocks of `blk` bytes along their cycles.  A
// segment is walked by one CTA, step after step, at about 2.6 GB/s (measured
// on GB300 both when 1216 CTAs saturate HBM, 32 KB blocks of the 100.7 GB
// tensor at 6.4 TB/s, and for 120 blocks of 108 KB at 14 GB/s); at most
// 8 CTAs per SM walk at once.  So the pass lasts about max(the longest
// segment, the blocks per walking CTA) steps, each of blk / 2.6 GB/s,
// against a streaming pass of 2 n blk bytes at 6.5 TB/s.
double block_perm_cost(uint64_t blk, uint64_t n, const DeviceCaps& caps) {
    if (blk < kMinCycleBlock) return -1.0;
    double c = 1.05 + 2.0 / static_cast<double>(kCycleSegment);
    if (blk < 16384) c += 0.15;
    if (blk < 8192) c += 0.15;
    const double walkers = 8.0 * std::max(1, caps.sms);
    const double steps = std::max(std::min(static_cast<double>(n), static_cast<double>(kCycleSegment)),
                                  static_cast<double>(n) / walkers);
    const double t_walk = steps * static_cast<double>(blk) / 2.6e9;
    const double t_pass = 2.0 * static_cast<double>(n) * static_cast<double>(blk) / 6.5e12;
    return std::max(c, t_walk / t_pass);
}

std::string join(const std::vector<uint64_t>& v) {
    std::ostringstream os;
    for (size_t i = 0; i < v.size(); ++i) os << (i ? "," : "") << v[i];
    return os.str();
}
std::string join(const std::vector<int>& v) {
    std::ostringstream os;
    for (size_t i = 0; i < v.size(); ++i) os << (i ? "," : "") << v[i];
    return os.str();
}

struct Move {
    int kind = 0;  // 0 X, 1 slab, 2 cycle
    int i = 0, j = 0, k = 0;
};

struct Node {
    std::vector<int> state;
    double cost = 0;
    int parent = -1;
    Move move;
};

}  // namespace

double passes_model_cost_new(const Pass& p, const DeviceCaps& caps) {
    if (p.type == kSlabPerm) {
        uint64_t count = 1;
        for (auto d : p.nd_dims) count *= d;
        std::vector<uint64_t> od;
        for (int j : p.nd_perm) od.push_back(p.nd_dims[j]);
        const double c = slab_perm_cost(p.elem, count, od, caps);
        return c < 0 ? 3.0 : c;
    }
    if (p.type == kBlockPerm) {
        const double c = block_perm_cost(p.block, p.n_blocks, caps);
        return c < 0 ? 3.0 : c;
    }
    return 0.0;
}

namespace {
bool search_plan_uncached(const std::vector<int64_t>& dims, const std::vector<int>& perm1, uint64_t elem,
                          const DeviceCaps& caps, std::vector<Pass>* passes, double* cost, std::string* desc);

struct SearchMemo {
    bool ok = false;
    std::vector<Pass> passes;
    double cost = 0;
    std::string desc;
};
}  // namespace

// Plans are remembered per request shape, device and knobs (a search costs
// up to tens of milliseconds; the cost model depends on both).
bool search_plan(const std::vector<int64_t>& dims, const std::vector<int>& perm1, uint64_t elem,
                 const DeviceCaps& caps, std::vector<Pass>* passes, double* cost, std::string* desc) {
    static std::mutex mu;
    static std::map<std::string, SearchMemo> memo;
    std::string key;
    for (auto d : dims) key += std::to_string(d) + ",";
    key += "|";
    for (auto q : perm1) key += std::to_string(q) + ",";
    key += "|" + std::to_string(elem) + "|" + std::to_string(caps.sms) + "," + std::to_string(caps.smem_optin) + "," +
           std::to_string(caps.smem_per_sm) + "|";
    const Tuning& t = tuning();
    key.append(reinterpret_cast<const char*>(&t), sizeof(Tuning));
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = memo.find(key);
        if (it != memo.end()) {
            if (!it->second.ok) return false;
            *passes = it->second.passes;
            *cost = it->second.cost;
            if (desc) *desc = it->second.desc;
            return true;
        }
    }
    SearchMemo m;
    m.ok = search_plan_uncached(dims, perm1, elem, caps, &m.passes, &m.cost, &m.desc);
    {
        std::lock_guard<std::mutex> lock(mu);
        if (memo.size() > 4096) memo.clear();
        memo[key] = m;
    }
    if (!m.ok) return false;
    *passes = m.passes;
    *cost = m.cost;
    if (desc) *desc = m.desc;
    return true;
}

namespace {
bool search_plan_uncached(const std::vector<int64_t>& dims, const std::vector<int>& perm1, uint64_t elem,
                          const DeviceCaps& caps, std::vector<Pass>* passes, double* cost, std::string* desc) {
    const int r0 = static_cast<int>(dims.size());
    // position of every input axis in the output
    std::vector<int> out_pos(r0);
    for (int j = 0; j < r0; ++j) out_pos[perm1[j] - 1] = j;
    // merge input axes that stay adjacent and in order; size-1 axes drop out
    std::vector<int> live;
    for (int i = 0; i < r0; ++i)
        if (dims[i] > 1) live.push_back(i);
    std::vector<uint64_t> size;       // merged axis sizes, indexed by merged id (input order)
    std::vector<int> first_out;       // output position of each merged axis's first input axis
    for (size_t t = 0; t < live.size(); ++t) {
        const int a = live[t];
        if (t > 0) {
            const int prev = live[t - 1];
            // adjacent among the live axes in the output too?
            bool adjacent = out_pos[a] > out_pos[prev];
            for (int q = out_pos[prev] + 1; adjacent && q < out_pos[a]; ++q)
                if (dims[perm1[q] - 1] > 1) adjacent = false;
            if (adjacent) {
                size.back() *= static_cast<uint64_t>(dims[a]);
                continue;
            }
        }
        size.push_back(static_cast<uint64_t>(dims[a]));
        first_out.push_back(out_pos[a]);
    }
    const int r = static_cast<int>(size.size());
    if (r <= 1) return false;  // nothing moves
    if (r > 8) return false;   // beyond the search's reach: the reference's series
    std::vector<int> target(r);
    {
        std::vector<int> ids(r);
        for (int m = 0; m < r; ++m) ids[m] = m;
        std::sort(ids.begin(), ids.end(), [&](int x, int y) { return first_out[x] < first_out[y]; });
        target = ids;
    }
    std::vector<int> tpos(r);
    for (int q = 0; q < r; ++q) tpos[target[q]] = q;
    auto prod = [&](const std::vector<int>& L, int a, int b) {
        uint64_t v = 1;
        for (int q = a; q < b; ++q) v *= size[L[q]];
        return v;
    };
    auto by_target = [&](std::vector<int> v) {
        std::sort(v.begin(), v.end(), [&](int x, int y) { return tpos[x] < tpos[y]; });
        return v;
    };

    std::map<std::tuple<uint64_t, uint64_t, uint64_t, uint64_t>, double> xcache;
    auto xcost = [&](uint64_t B, uint64_t R, uint64_t C, uint64_t E) {
        auto key = std::make_tuple(B, R, C, E);
        auto it = xcache.find(key);
        if (it != xcache.end()) return it->second;
        std::vector<Pass> ps;
        lower_xpose(Xpose{0, B, R, C, E}, caps, &ps);
        const double c = passes_cost_of(ps, caps) + narrow_slab_penalty(ps);
        xcache.emplace(key, c);
        return c;
    };

    std::vector<Node> nodes;
    std::map<std::vector<int>, int> index;
    using QE = std::pair<double, int>;
    std::priority_queue<QE, std::vector<QE>, std::greater<QE>> pq;
    std::vector<int> start(r);
    for (int m = 0; m < r; ++m) start[m] = m;
    nodes.push_back(Node{start, 0.0, -1, Move{}});
    index[start] = 0;
    pq.push({0.0, 0});
    int found = -1;
    const size_t kMaxNodes = 6000;
    auto relax = [&](int from, std::vector<int> next, double c, const Move& mv) {
        const double nc = nodes[from].cost + c;
        auto it = index.find(next);
        if (it == index.end()) {
            if (nodes.size() >= kMaxNodes) return;
            index[next] = static_cast<int>(nodes.size());
            nodes.push_back(Node{std::move(next), nc, from, mv});
            pq.push({nc, static_cast<int>(nodes.size()) - 1});
        } else if (nc < nodes[it->second].cost - 1e-9) {
            nodes[it->second].cost = nc;
            nodes[it->second].parent = from;
            nodes[it->second].move = mv;
            pq.push({nc, it->second});
        }
    };
    std::vector<char> closed;
    while (!pq.empty()) {
        const auto [c, u] = pq.top();
        pq.pop();
        if (static_cast<int>(closed.size()) <= u) closed.resize(nodes.size(), 0);
        if (closed[u] || c > nodes[u].cost + 1e-9) continue;
        closed[u] = 1;
        const std::vector<int> L = nodes[u].state;
        if (L == target) {
            found = u;
            break;
        }
        // X moves: swap groups L[i:j] and L[j:k]
        for (int i = 0; i < r; ++i)
            for (int j = i + 1; j < r; ++j)
                for (int k = j + 1; k <= r; ++k) {
                    std::vector<int> next(L.begin(), L.begin() + i);
                    next.insert(next.end(), L.begin() + j, L.begin() + k);
                    next.insert(next.end(), L.begin() + i, L.begin() + j);
                    next.insert(next.end(), L.begin() + k, L.end());
                    const double xc = xcost(prod(L, k, r), prod(L, j, k), prod(L, i, j), elem * prod(L, 0, i));
                    relax(u, std::move(next), xc, Move{0, i, j, k});
                }
        // slab moves: L[i:k] into the target's order, elements of L[0:i]
        for (int i = 0; tuning().slab_perm && i < r; ++i)
            for (int k = i + 2; k <= r; ++k) {
                std::vector<int> mid(L.begin() + i, L.begin() + k);
                std::vector<int> sorted = by_target(mid);
                if (sorted == mid) continue;
                std::vector<uint64_t> od;
                for (int a : sorted) od.push_back(size[a]);
                double sc = slab_perm_cost(elem * prod(L, 0, i), prod(L, i, k), od, caps);
                if (sc < 0) continue;
                if (tuning().slab_perm == 2) sc *= 0.25;
                std::vector<int> next(L.begin(), L.begin() + i);
                next.insert(next.end(), sorted.begin(), sorted.end());
                next.insert(next.end(), L.begin() + k, L.end());
                relax(u, std::move(next), sc, Move{1, i, 0, k});
            }
        // cycle moves: blocks of L[0:i], the rest into the target's order
        for (int i = 1; tuning().cycle_moves && i + 1 < r; ++i) {
            std::vector<int> rest(L.begin() + i, L.end());
            std::vector<int> sorted = by_target(rest);
            if (sorted == rest) continue;
            double bc = block_perm_cost(elem * prod(L, 0, i), prod(L, i, r), caps);
            if (bc < 0) continue;
            if (tuning().cycle_moves == 2) bc = std::min(bc, 1.0) * 0.25;
            std::vector<int> next(L.begin(), L.begin() + i);
            next.insert(next.end(), sorted.begin(), sorted.end());
            relax(u, std::move(next), bc, Move{2, i, 0, r});
        }
    }
    if (found < 0) return false;
    // the moves, first to last
    std::vector<int> path;
    for (int u = found; u > 0; u = nodes[u].parent) path.push_back(u);
    std::reverse(path.begin(), path.end());
    std::ostringstream ds;
    passes->clear();
    for (int u : path) {
        const std::vector<int>& L = nodes[nodes[u].parent].state;
        const Move& mv = nodes[u].move;
        if (mv.kind == 0) {
            const Xpose x{0, prod(L, mv.k, r), prod(L, mv.j, mv.k), prod(L, mv.i, mv.j), elem * prod(L, 0, mv.i)};
            lower_xpose(x, caps, passes);
            ds << "X(B=" << x.B << ",R=" << x.R << ",C=" << x.C << ",E=" << x.E << ") ";
        } else {
            const int i = mv.i, k = mv.k;
            std::vector<int> mid(L.begin() + i, L.begin() + k);
            std::vector<int> sorted = by_target(mid);
            Pass p;
            p.type = mv.kind == 1 ? kSlabPerm : kBlockPerm;
            for (int q = i; q < k; ++q) p.nd_dims.push_back(size[L[q]]);
            for (int q = 0; q < k - i; ++q)
                p.nd_perm.push_back(static_cast<int>(std::find(mid.begin(), mid.end(), sorted[q]) - mid.begin()));
            const uint64_t inner = elem * prod(L, 0, i);
            uint64_t count = 1;
            for (auto d : p.nd_dims) count *= d;
            p.rows = count;  // the profile's byte count: 2 * batches * rows * cols * elem
            p.cols = 1;
            if (mv.kind == 1) {
                p.batches = prod(L, k, r);
                p.elem = inner;
                p.strip = slab_perm_strip(inner, count, caps);
                p.what = "slab-perm B=" + std::to_string(p.batches) + " dims=(" + join(p.nd_dims) + ") order=(" +
                         join(p.nd_perm) + ") E=" + std::to_string(inner);
            } else {
                p.batches = 1;
                p.block = inner;
                p.elem = inner;
                p.n_blocks = count;
                p.what = "cycle-perm block=" + std::to_string(inner) + " dims=(" + join(p.nd_dims) + ") order=(" +
                         join(p.nd_perm) + ")";
            }
            passes->push_back(p);
            ds << p.what << " ";
        }
    }
    *cost = nodes[found].cost;
    if (desc) *desc = ds.str();
    return true;
}
}  // namespace

double passes_model_cost(const std::vector<Pass>& passes, const DeviceCaps& caps) {
    double c = 0;
    for (const Pass& p : passes) {
        if (p.type == kSlabPerm || p.type == kBlockPerm) {
            c += passes_model_cost_new(p, caps);
        } else if (p.type == kBlockMove) {
            c += 1.0;
        } else {
            std::vector<Pass> one(1, p);
            c += passes_cost_of(one, caps) + narrow_slab_penalty(one);
        }
    }
    return c;
}

const CycleTable& cycle_table(const std::vector<uint64_t>& dims, const std::vector<int>& perm) {
    static std::mutex mu;
    static std::map<std::pair<std::vector<uint64_t>, std::vector<int>>, CycleTable> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto key = std::make_pair(dims, perm);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    if (cache.size() > 64) cache.clear();  // bounded: tables of recent shapes only
    const int q = static_cast<int>(dims.size());
    uint64_t n = 1;
    for (auto d : dims) n *= d;
    // dst(s): input coordinates of s, recombined with the output strides
    std::vector<uint64_t> ostride(q);
    {
        uint64_t st = 1;
        for (int j = 0; j < q; ++j) {
            ostride[perm[j]] = st;
            st *= dims[perm[j]];
        }
    }
    auto dst = [&](uint64_t s) {
        uint64_t t = 0;
        for (int a = 0; a < q; ++a) {
            t += (s % dims[a]) * ostride[a];
            s /= dims[a];
        }
        return t;
    };
    CycleTable tab;
    std::vector<uint64_t> seen((n + 63) / 64, 0);
    std::vector<uint64_t> cyc;
    for (uint64_t s0 = 0; s0 < n; ++s0) {
        if (seen[s0 >> 6] >> (s0 & 63) & 1) continue;
        cyc.clear();
        uint64_t s = s0;
        do {
            seen[s >> 6] |= uint64_t(1) << (s & 63);
            cyc.push_back(s);
            s = dst(s);
        } while (s != s0);
        const uint64_t L = cyc.size();
        if (L == 1) continue;
        tab.moved += L;
        // segments of kCycleSegment steps or more (a cycle has at most
        // kMaxCycleSegments of them); the last one ends where the first began
        const uint64_t seg = std::max<uint64_t>(kCycleSegment, (L + kMaxCycleSegments - 1) / kMaxCycleSegments);
        tab.cycle_first.push_back(tab.head.size());
        for (uint64_t a = 0; a < L; a += seg) {
            const uint64_t len = std::min<uint64_t>(seg, L - a);
            tab.head.push_back(cyc[a]);
            tab.tail.push_back(cyc[(a + len) % L]);
            tab.len.push_back(len);
        }
    }
    tab.cycle_first.push_back(tab.head.size());
    for (size_t c = 0; c + 1 < tab.cycle_first.size(); ++c)
        tab.max_cycle_segments = std::max<uint64_t>(tab.max_cycle_segments, tab.cycle_first[c + 1] - tab.cycle_first[c]);
    return cache.emplace(key, std::move(tab)).first->second;
}

}  // namespace eithot
