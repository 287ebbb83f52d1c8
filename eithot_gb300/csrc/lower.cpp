// Lowering of an N-d plan to device passes (see passes.h).
#include "passes.h"

#include <algorithm>
#include <map>
#include <mutex>
#include <sstream>
#include <tuple>

namespace eithot {

void gcd_inverse(uint64_t a, uint64_t b, uint64_t* g, uint64_t* inv) {
    // Extended Euclid on (a, b); inv = a^-1 mod b when gcd == 1, 0 if b == 1.
    __int128 r0 = static_cast<__int128>(a), r1 = static_cast<__int128>(b);
    __int128 s0 = 1, s1 = 0;
    while (r1 != 0) {
        const __int128 qt = r0 / r1;
        const __int128 r2 = r0 - qt * r1;
        r0 = r1; r1 = r2;
        const __int128 s2 = s0 - qt * s1;
        s0 = s1; s1 = s2;
    }
    *g = static_cast<uint64_t>(r0);
    if (r0 != 1 || b <= 1) { *inv = 0; return; }
    __int128 x = s0 % static_cast<__int128>(b);
    if (x < 0) x += b;
    *inv = static_cast<uint64_t>(x);
}

size_t smem_cap_of(const DeviceCaps& caps) {
    // Leave room for the block's static shared memory and the CUDA
    // runtime's per-block reservation.
    return caps.smem_optin > 2048 ? caps.smem_optin - 2048 : caps.smem_optin;
}

uint64_t strip_width(uint64_t E, uint64_t count, uint64_t budget) {
    if (E <= 128) return E;
    const uint64_t w = budget / std::max<uint64_t>(count, 1) / 128 * 128;
    if (w >= E) return E;
    return std::max<uint64_t>(128, w);
}

namespace {
uint64_t pow2_divisor(uint64_t v, uint64_t cap) {
    uint64_t u = 1;
    while (u < cap && v % (u * 2) == 0) u *= 2;
    return u;
}
}  // namespace

uint64_t slab_pitch(uint64_t C, uint64_t w) {
    const uint64_t g = std::max<uint64_t>(4, pow2_divisor(w, 16));
    uint64_t pitch = (C * w + g - 1) / g * g;
    if ((pitch / g) % 2 == 0) pitch += g;
    return pitch;
}

size_t slab_smem_bytes(uint64_t R, uint64_t C, uint64_t w) { return R * slab_pitch(C, w); }

uint64_t slab_cluster_pitch(uint64_t row_bytes) {
    uint64_t pitch = (row_bytes + 3) / 4 * 4;
    if ((pitch / 4) % 2 == 0) pitch += 4;  // odd words: a column read walks distinct banks
    return pitch;
}

namespace {
constexpr int kClusterSizes[] = {1, 2, 4, 8, 16};

int log2i(int K) {
    int l = 0;
    while ((1 << l) < K) ++l;
    return l;
}

// Modelled slowdown of staging an item over K CTAs, per doubling of K, for
// items moved in granules of g bytes through distributed shared memory
// (measured on GB300: 128-byte pulls lose ~10-15% per doubling, 16-byte
// pulls 40-70%, 16-byte pushes ~30%).
// Modelled cost, per doubling of the cluster, of a row pass that moves 1- or
// 2-byte granules through distributed shared memory.
constexpr double kNarrowRemote = 3.0;
// Extra modelled cost of a Catanzaro pass whose elements move in 1-byte
// units (odd sizes; an index map per byte: 40-600 GB/s measured on such
// passes), half of it for 2-byte units.
constexpr double kNarrowPass = 4.0;

double narrow_pass_cost(uint64_t E) {
    if (E % 2) return kNarrowPass;
    if (E % 4) return kNarrowPass / 2;
    return 0.0;
}

double dsmem_penalty(uint64_t g, bool push) {
    if (g >= 128) return 0.12;
    if (g >= 64) return 0.2;
    if (g >= 32) return 0.3;
    return push ? 0.35 : 0.7;
}
}  // namespace

namespace {
thread_local Tuning* t_scoped = nullptr;
}  // namespace

Tuning& tuning() {
    static Tuning t;
    return t_scoped ? *t_scoped : t;
}

ScopedTuning::ScopedTuning(const Tuning& t) : t_(t), prev_(t_scoped) { t_scoped = &t_; }
ScopedTuning::~ScopedTuning() { t_scoped = prev_; }

namespace {
using ShapeKey = std::tuple<std::vector<int64_t>, std::vector<int>, uint64_t>;
std::mutex g_shape_mu;
std::map<ShapeKey, Tuning>& shape_table() {
    static std::map<ShapeKey, Tuning> table;
    return table;
}
}  // namespace

bool shape_tuning(const std::vector<int64_t>& dims, const std::vector<int>& perm, uint64_t elem, Tuning* out) {
    std::lock_guard<std::mutex> lock(g_shape_mu);
    auto& tab = shape_table();
    if (tab.empty()) return false;
    auto it = tab.find(ShapeKey{dims, perm, elem});
    if (it == tab.end()) return false;
    *out = it->second;
    return true;
}

void set_shape_tuning(const std::vector<int64_t>& dims, const std::vector<int>& perm, uint64_t elem, const Tuning& t) {
    std::lock_guard<std::mutex> lock(g_shape_mu);
    shape_table()[ShapeKey{dims, perm, elem}] = t;
}

void clear_shape_tuning() {
    std::lock_guard<std::mutex> lock(g_shape_mu);
    shape_table().clear();
}

int shape_tuning_count() {
    std::lock_guard<std::mutex> lock(g_shape_mu);
    return static_cast<int>(shape_table().size());
}

namespace {
// A CTA footprint at most this large lets two CTAs share an SM (GB300:
// 228 KB of shared memory per SM); clusters of CTAs that each fill an SM
// leave SMs unused when whole clusters no longer fit a GPC.
constexpr uint64_t kTwoPerSm = 110 * 1024;
constexpr double kOnePerSmPenalty = 0.25;
}  // namespace

Staging plan_row_staging(uint64_t cols, uint64_t E, size_t cap, bool scatter) {
    (void)scatter;
    Staging s;
    const uint64_t w0 = strip_width(E, cols, kWideStripBytes);
    for (uint64_t w : {w0, uint64_t(128), uint64_t(64), uint64_t(32)}) {
        if (w > w0 || w < std::min<uint64_t>(E, 32)) continue;
        // a whole row strip in one CTA
        if (cols * w <= cap) {
            s.w = w; s.K = 1; s.per_cta = cols * w; s.item_bytes = cols * w;
            s.on_chip = true; s.dbuf = false;
            s.cost = 1.0 + (w < E ? 0.05 : 0.0);
            return s;
        }
    }
    for (uint64_t occ_limit : {kTwoPerSm, static_cast<uint64_t>(cap)}) {
        for (uint64_t w : {w0, uint64_t(128), uint64_t(64), uint64_t(32)}) {
            if (w > w0 || w < std::min<uint64_t>(E, 32)) continue;
            for (int K : kClusterSizes) {
                if (K > tuning().max_cluster) break;
                const uint64_t per = (cols + K - 1) / K * w;
                for (bool db : {true, false}) {
                    if (db && !tuning().dbuf) continue;
                    const uint64_t foot = per * (db ? 2 : 1);
                    if (foot > cap || foot > occ_limit) continue;
                    s.w = w; s.K = K; s.per_cta = per; s.item_bytes = cols * w;
                    s.on_chip = true; s.dbuf = db;
                    // 16-32 byte granules are pushed whatever the pass's own
                    // direction (the inverse map turns a gather into a scatter);
                    // 1- and 2-byte granules cost one remote access each
                    // (rows of 0.3-2 MB over 16 CTAs: 75-370 GB/s)
                    s.cost = 1.0 + (w < 4 ? kNarrowRemote : dsmem_penalty(w, true)) * log2i(K) + (db ? 0.0 : 0.1) +
                             (foot > kTwoPerSm ? kOnePerSmPenalty : 0.0);
                    return s;
                }
            }
        }
    }
    s.w = w0;
    s.K = 1;
    s.item_bytes = cols * w0;
    s.per_cta = s.item_bytes;
    s.on_chip = false;
    s.cost = 2.5;
    return s;
}

Staging plan_col_staging(uint64_t rows, uint64_t E, size_t cap, uint64_t cols) {
    Staging s;
    for (uint64_t occ_limit : {kTwoPerSm, static_cast<uint64_t>(cap)}) {
        for (uint64_t tb : {uint64_t(128), uint64_t(64), uint64_t(32)}) {
            if (tuning().col_chunk && tb != static_cast<uint64_t>(tuning().col_chunk)) continue;
            uint64_t w, tw;
            if (E <= tb) { w = E; tw = std::max<uint64_t>(1, std::min(tb / E, cols ? cols : tb / E)); }
            else { w = tb; tw = 1; }
            // tw*w contiguous bytes per staged row: a quarter-warp of 16-byte
            // reads (or a warp of 4-byte reads) covers one row piece, so the
            // row pitch needs no bank padding
            const uint64_t pitch = tw * w;
            for (int K : kClusterSizes) {
                if (K > tuning().max_cluster) break;
                const uint64_t per = (rows + K - 1) / K * pitch;
                for (bool db : {true, false}) {
                    if (db && (!tuning().dbuf || K == 1)) continue;
                    const uint64_t foot = per * (db ? 2 : 1);
                    if (foot > cap || foot > occ_limit) continue;
                    s.w = w; s.tw = tw; s.pitch = pitch; s.K = K; s.per_cta = per;
                    s.item_bytes = rows * pitch; s.on_chip = true; s.dbuf = db;
                    s.cost = 1.0 + dsmem_penalty(pitch, false) * log2i(K) + (tb < 128 ? 0.1 : 0.0) +
                             (foot > kTwoPerSm ? kOnePerSmPenalty : 0.0);
                    return s;
                }
            }
        }
    }
    // Global staging: 128-byte row pieces.
    s.w = E <= 128 ? E : 128;
    s.tw = E <= 128 ? std::max<uint64_t>(1, std::min<uint64_t>(128 / E, cols ? cols : 128 / E)) : 1;
    s.pitch = s.tw * s.w;
    s.K = 1;
    s.item_bytes = rows * s.pitch;
    s.per_cta = s.item_bytes;
    s.on_chip = false;
    s.cost = 2.5;
    return s;
}

void owner_halo(int fn, uint64_t b, uint64_t tw, uint64_t* lo, uint64_t* hi) {
    *lo = 0;
    *hi = 0;
    if (tw <= 1) return;
    // delta(j0 + c) - delta(j0) over c < tw: c for the shuffles, at most
    // (tw - 1) / b + 1 steps of j / b for the rotations
    const bool shuffle = fn == kFnC2RColShuffle || fn == kFnR2CColShuffle;
    const uint64_t spread = shuffle ? tw - 1 : (tw - 1) / std::max<uint64_t>(b, 1) + 1;
    if (fn == kFnR2CPostRot || fn == kFnR2CColShuffle) *lo = spread; else *hi = spread;
}

namespace {
// Relative DRAM efficiency of moving row pieces of `piece` contiguous bytes
// scattered over rows (measured on GB300, read + write of 2.6 GB: 32 B 1.8
// TB/s, 64 B 2.9-3.4, 128 B 5.1, 256 B and up 6.6 = a streaming copy).
double piece_efficiency(uint64_t piece) {
    if (piece >= 256) return 1.0;
    if (piece >= 128) return 0.77;
    if (piece >= 64) return 0.47;
    return 0.28;
}

// Fraction of the SMs that clusters of K CTAs keep busy (clusters must fit
// a GPC; GB300 runs 14 clusters of 16 two-per-SM CTAs, 112 of 152 SMs).
double cluster_utilisation(int K) {
    if (K >= 16) return 0.74;
    if (K >= 8) return 0.95;
    return 1.0;
}

// Owner-computed column staging.  Each CTA stages Q consecutive slots of
// the tile plus the halo and writes whole output row pieces from its own
// shared memory; the tile's CTAs need only a barrier between their loads
// and their writes, a thread-block cluster's (K <= 16) or, for tiles too
// large for a cluster, a global-memory barrier over a group of G
// co-resident CTAs.  Candidates are costed by row-piece efficiency, SM
// utilisation, halo re-reads and buffering.
Staging plan_col_owner(uint64_t rows, uint64_t cols, uint64_t batches, uint64_t E, int fn, uint64_t b,
                       const DeviceCaps& caps) {
    const size_t cap = smem_cap_of(caps);
    const int form = tuning().col_form;
    // bytes of one row-table entry: the pass's index type (32-bit when
    // m*n + m + n < 2^31, as the kernels choose it)
    const uint64_t idx = rows * cols + rows + cols < (uint64_t(1) << 31) ? 4 : 8;
    Staging best;
    best.on_chip = false;
    best.cost = 1e30;
    auto consider = [&](const Staging& s) {
        if (s.cost < best.cost) best = s;
    };
    // short columns: one CTA stages every row of a tile of as many columns
    // as its share of shared memory holds (slots indexed modulo the row
    // count, no halo); enough tiles are left for every SM
    if (form != 2 && E <= 128 && !tuning().col_chunk) {
        for (bool db : {true, false}) {
            if (db && !tuning().dbuf) continue;
            const uint64_t tables = 2 * rows * idx + 16;  // source and output row tables
            if (kTwoPerSm <= tables + 256) continue;
            const uint64_t budget = (kTwoPerSm - tables) / (db ? 2 : 1) - 127;
            const uint64_t tw_cap = std::min<uint64_t>(cols, budget / (rows * E));
            if (tw_cap < 1 || tw_cap * E < 128) continue;
            const uint64_t want_tiles = 4 * static_cast<uint64_t>(caps.sms);
            const uint64_t tiles_per_batch = (want_tiles + std::max<uint64_t>(batches, 1) - 1) / std::max<uint64_t>(batches, 1);
            uint64_t tw = std::min<uint64_t>(tw_cap, std::max<uint64_t>((cols + tiles_per_batch - 1) / tiles_per_batch,
                                                                        (256 + E - 1) / E));
            tw = std::max<uint64_t>(1, std::min(tw, tw_cap));
            Staging s;
            s.w = E; s.tw = tw; s.pitch = tw * E; s.K = 1; s.per_cta = rows * s.pitch;
            s.item_bytes = rows * s.pitch; s.on_chip = true; s.dbuf = db;
            s.owner = true; s.whole = true; s.per_sm = 2;
            s.cost = 1.0 / piece_efficiency(s.pitch) + (db ? 0.0 : 0.1);
            consider(s);
            break;
        }
    }
    for (uint64_t tb : {uint64_t(512), uint64_t(256), uint64_t(128), uint64_t(64), uint64_t(32)}) {
        if (tuning().col_chunk && tb != static_cast<uint64_t>(tuning().col_chunk)) continue;
        uint64_t w, tw;
        if (E <= tb) { w = E; tw = std::max<uint64_t>(1, std::min(tb / E, cols ? cols : tb / E)); }
        else { w = tb; tw = 1; }
        const uint64_t pitch = tw * w;
        uint64_t lo, hi;
        owner_halo(fn, b, tw, &lo, &hi);
        const double eff = piece_efficiency(pitch);
        // thread-block clusters
        if (form != 2) {
            for (int K : kClusterSizes) {
                if (K > tuning().max_cluster) break;
                const uint64_t Q = (rows + K - 1) / K;
                const uint64_t per = (Q + lo + hi) * pitch;
                for (bool db : {true, false}) {
                    if (db && !tuning().dbuf) continue;
                    // slot buffer(s), 128-byte rounded, and the row tables
                    const uint64_t foot = (per + 127) / 128 * 128 * (db ? 2 : 1) + (2 * Q + lo + hi) * idx + 16;
                    if (foot > cap) continue;
                    Staging s;
                    s.w = w; s.tw = tw; s.pitch = pitch; s.K = K; s.per_cta = per;
                    s.item_bytes = rows * pitch; s.on_chip = true; s.dbuf = db;
                    s.owner = true; s.hlo = lo; s.hhi = hi;
                    s.per_sm = foot <= kTwoPerSm ? 2 : 1;
                    s.cost = 1.0 / (eff * cluster_utilisation(K)) +
                             0.5 * static_cast<double>((lo + hi) * K) / static_cast<double>(rows) +
                             0.03 * log2i(K) + (db ? 0.0 : 0.1) + (s.per_sm == 1 && !db ? kOnePerSmPenalty : 0.0);
                    consider(s);
                    break;  // double buffering preferred when it fits
                }
            }
        }
        // groups of co-resident CTAs: several single-buffered CTAs per SM
        // overlap one another's barrier waits better than one
        // double-buffered CTA
        if (form != 1) {
            for (int per_sm : {2, 3, 4, 1}) {
                if (tuning().group_per_sm && per_sm != tuning().group_per_sm) continue;
                const uint64_t sm_share = caps.smem_per_sm / per_sm;
                if (sm_share < 4096) continue;
                const uint64_t per_cta_cap = std::min<uint64_t>(cap, sm_share - 3072);
                // bulk-copy staging: whole elements in 16-byte pieces at a
                // 16-byte pitch, double-buffered
                const bool bulk_able = tuning().col_bulk && E <= tb && pitch % 16 == 0 && (cols * E) % 16 == 0;
                for (bool db : {false, true}) {
                    if (db && !tuning().dbuf) continue;
                    // the slot buffer(s) (128-byte rounded) and the CTA's row
                    // tables: Q + lo + hi source rows and Q output rows of the
                    // pass's index type (32-bit when m*n + m + n < 2^31)
                    const uint64_t nbuf = db ? 2 : 1;
                    const uint64_t fixed = 16 + nbuf * 127 + (lo + hi) * (nbuf * pitch + idx);
                    if (per_cta_cap <= fixed) continue;
                    const uint64_t qmax = (per_cta_cap - fixed) / (nbuf * pitch + 2 * idx);
                    if (qmax == 0) continue;
                    const uint64_t slots = static_cast<uint64_t>(per_sm) * caps.sms;
                    const uint64_t gmin = (rows + qmax - 1) / qmax;
                    if (gmin > slots) continue;
                    const uint64_t ngroups = slots / gmin;
                    uint64_t G = std::min<uint64_t>(slots / ngroups, rows);
                    const uint64_t Q = (rows + G - 1) / G;
                    G = (rows + Q - 1) / Q;  // CTAs that own at least one slot
                    Staging s;
                    s.w = w; s.tw = tw; s.pitch = pitch; s.K = 1; s.G = static_cast<int>(G);
                    s.per_cta = (Q + lo + hi) * pitch;
                    s.item_bytes = rows * pitch; s.on_chip = true; s.dbuf = db;
                    s.owner = true; s.group = true; s.hlo = lo; s.hhi = hi; s.per_sm = per_sm;
                    const double util = static_cast<double>(ngroups * G) / static_cast<double>(slots);
                    // measured on GB300 (20011-row pass, 256-byte pieces): 3 single-buffered
                    // CTAs per SM 2.13 ms, 2 per SM 2.22, 2 double-buffered 2.32, 1 double 2.64
                    const double residency = per_sm == 1 ? (db ? 0.17 : 0.4)
                                           : per_sm == 2 ? (db ? 0.05 : 0.02)
                                           : per_sm == 3 ? (db ? 0.04 : 0.0) : 0.03;
                    s.bulk = db && bulk_able;
                    // bulk-staged CTAs overlap their next item's loads with the
                    // barrier wait and the writes without spending registers on them
                    const double bulk_gain = s.bulk ? (per_sm <= 2 ? 0.06 : 0.0) : 0.0;
                    s.cost = 1.0 / (eff * util) + 0.5 * static_cast<double>((lo + hi) * G) / static_cast<double>(rows) +
                             (G > 1 ? 0.08 : 0.0) + (s.bulk ? residency - 0.05 - bulk_gain : residency);
                    consider(s);
                }
            }
        }
    }
    return best;
}
}  // namespace

Staging plan_col_pass(const Pass& p, const DeviceCaps& caps) {
    if (tuning().col_owner) {
        const Staging s = plan_col_owner(p.rows, p.cols, p.batches, p.elem, p.fn, p.b, caps);
        if (s.on_chip) return s;
    }
    return plan_col_staging(p.rows, p.elem, smem_cap_of(caps), p.cols);
}

Xpose xpose_of(const LowOp& op, uint64_t elem, uint64_t n_sub, uint64_t base_offset) {
    Xpose x;
    x.offset = base_offset;
    const uint64_t* d = reinterpret_cast<const uint64_t*>(op.dims);
    switch (op.code()) {
        case 21:   x.B = n_sub;        x.R = d[1];        x.C = d[0];        x.E = elem; break;
        case 213:  x.B = n_sub * d[2]; x.R = d[1];        x.C = d[0];        x.E = elem; break;
        case 132:  x.B = n_sub;        x.R = d[2];        x.C = d[1];        x.E = d[0] * elem; break;
        case 1324: x.B = n_sub * d[3]; x.R = d[2];        x.C = d[1];        x.E = d[0] * elem; break;
        case 231:  x.B = n_sub;        x.R = d[1] * d[2]; x.C = d[0];        x.E = elem; break;
        case 312:  x.B = n_sub;        x.R = d[2];        x.C = d[0] * d[1]; x.E = elem; break;
        default:   x.B = 0; break;  // never produced by the planner
    }
    return x;
}

namespace {

double row_cost(uint64_t cols, uint64_t E, size_t cap, bool scatter) {
    return plan_row_staging(cols, E, cap, scatter).cost;
}
double col_cost(uint64_t rows, uint64_t cols, uint64_t batches, uint64_t E, int fn, uint64_t b, const DeviceCaps& caps) {
    Pass p;
    p.rows = rows; p.cols = cols; p.batches = batches; p.elem = E; p.fn = fn; p.b = b;
    return plan_col_pass(p, caps).cost;
}

std::string geom(const char* name, uint64_t B, uint64_t r, uint64_t c, uint64_t E) {
    std::ostringstream os;
    os << name << " B=" << B << " rows=" << r << " cols=" << c << " E=" << E;
    return os.str();
}

}  // namespace

namespace {
void lower_xpose_direct(const Xpose& x, const DeviceCaps& caps, std::vector<Pass>* passes);

// Columns per CTA of a column-band cluster slab of R x C elements of E
// bytes (0 when none applies): the fewest CTAs (2-16) whose band of every row
// fits a CTA's shared memory in the run kernel's padded layout (rows of the
// band at an odd number of max(4, E)-byte granules), two CTAs per SM when
// that is possible, each band's row segments and output range starting on a
// 16-byte boundary of its matrix (P E a multiple of 16).
uint64_t colband_width(uint64_t R, uint64_t C, uint64_t E, const DeviceCaps& caps) {
    if (!(E == 1 || E == 2 || E == 4 || E == 8 || E == 16)) return 0;
    const uint64_t m = 16 / E;
    const uint64_t cap = smem_cap_of(caps);
    for (uint64_t budget : {static_cast<uint64_t>(kTwoPerSm), cap - 1024}) {
        for (int K = 2; K <= std::min(16, tuning().max_cluster); ++K) {
            uint64_t P = (C + K - 1) / K;
            P = (P + m - 1) / m * m;
            const uint64_t k = (C + P - 1) / P;
            if (k < 2 || k > 16) continue;
            const uint64_t g = std::max<uint64_t>(4, E);
            uint64_t pitch = (P * E + g - 1) / g * g;
            if ((pitch / g) % 2 == 0) pitch += g;
            if (R * pitch <= budget) return P;
        }
    }
    return 0;
}

// Modelled time of a pass list, in units of one streaming pass; *staged is
// set when a pass goes through global scratch.
double passes_cost(const std::vector<Pass>& ps, const DeviceCaps& caps, bool* staged) {
    const size_t cap = smem_cap_of(caps);
    double c = 0;
    for (const Pass& p : ps) {
        switch (p.type) {
            case kSlabTranspose: c += slab_smem_bytes(p.rows, p.cols, p.strip) > kTwoPerSm ? 1.25 : 1.0; break;
            case kSlabCluster: c += 1.05; break;
            case kRowGather:
            case kRowScatter: {
                const Staging st = plan_row_staging(p.cols, p.elem, cap, p.type == kRowScatter);
                if (!st.on_chip) *staged = true;
                c += (st.on_chip ? st.cost : 3.0) + narrow_pass_cost(p.elem);
                break;
            }
            case kColGather: {
                const Staging st = plan_col_pass(p, caps);
                if (!st.on_chip) *staged = true;
                c += (st.on_chip ? st.cost : 3.0) + narrow_pass_cost(p.elem);
                break;
            }
            default: break;
        }
    }
    return c;
}

// Divisors d of v with 2 <= d <= v / 2, at most `limit` of them spread over
// the range.
std::vector<uint64_t> divisors(uint64_t v, size_t limit) {
    std::vector<uint64_t> lo, hi;
    for (uint64_t d = 2; d * d <= v; ++d) {
        if (v % d) continue;
        lo.push_back(d);
        if (d * d != v) hi.push_back(v / d);
    }
    lo.insert(lo.end(), hi.rbegin(), hi.rend());
    if (lo.size() <= limit) return lo;
    std::vector<uint64_t> out;
    for (size_t i = 0; i < limit; ++i) out.push_back(lo[i * lo.size() / limit]);
    return out;
}
}  // namespace

// A batched transpose whose Catanzaro passes would stage through global
// scratch (a row or a column too long for on-chip staging), or of elements
// that move in 1- or 2-byte units, may instead be split along a
// factorisation of its rows R = Ra*Rb (or columns C = Ca*Cb) into two
// transposes of wider granules:
//   R: Rb x C matrices (B*Ra of them), then Ra x C with elements of Rb*E bytes;
//   C: R x Ca with elements of Cb*E bytes, then R x Cb matrices (B*Ca of them).
void lower_xpose(const Xpose& x, const DeviceCaps& caps, std::vector<Pass>* passes) {
    if (x.B == 0 || x.R <= 1 || x.C <= 1) return;  // identity
    std::vector<Pass> direct;
    lower_xpose_direct(x, caps, &direct);
    bool staged = false;
    const double direct_cost = passes_cost(direct, caps, &staged);
    bool narrow = false;  // a Catanzaro pass of 1- or 2-byte units
    for (const Pass& p : direct)
        narrow = narrow || ((p.type == kRowGather || p.type == kRowScatter || p.type == kColGather) && p.elem % 4);
    if ((!staged && !narrow) || !tuning().factor) {
        passes->insert(passes->end(), direct.begin(), direct.end());
        return;
    }
    double best = direct_cost - 0.25;  // factor only for a clear gain
    std::vector<Pass> chosen;
    auto consider = [&](const Xpose& a, const Xpose& b) {
        std::vector<Pass> ps;
        lower_xpose_direct(a, caps, &ps);
        lower_xpose_direct(b, caps, &ps);
        bool st = false;
        const double c = passes_cost(ps, caps, &st);
        if (c < best) {
            best = c;
            chosen.swap(ps);
        }
    };
    for (uint64_t rb : divisors(x.R, 48)) {
        const uint64_t ra = x.R / rb;
        consider(Xpose{x.offset, x.B * ra, rb, x.C, x.E}, Xpose{x.offset, x.B, ra, x.C, rb * x.E});
    }
    for (uint64_t cb : divisors(x.C, 48)) {
        const uint64_t ca = x.C / cb;
        consider(Xpose{x.offset, x.B, x.R, ca, cb * x.E}, Xpose{x.offset, x.B * ca, x.R, cb, x.E});
    }
    if (chosen.empty()) chosen.swap(direct);
    passes->insert(passes->end(), chosen.begin(), chosen.end());
}

double passes_cost_of(const std::vector<Pass>& ps, const DeviceCaps& caps) {
    bool staged = false;
    return passes_cost(ps, caps, &staged);
}

double xpose_cost(const Xpose& x, const DeviceCaps& caps) {
    std::vector<Pass> ps;
    lower_xpose(x, caps, &ps);
    bool staged = false;
    return passes_cost(ps, caps, &staged);
}

namespace {
void lower_xpose_direct(const Xpose& x, const DeviceCaps& caps, std::vector<Pass>* passes) {
    if (x.B == 0 || x.R <= 1 || x.C <= 1) return;  // identity
    const size_t cap = smem_cap_of(caps);
    const uint64_t w0 = strip_width(x.E, x.R * x.C, kWideStripBytes);
    // A matrix beyond two-per-SM shared memory: one owner-computed pass over
    // a cluster of K CTAs (each stages a band of rows and writes that band's
    // segment of every output row) instead of a one-CTA-per-SM slab or the
    // two or three Catanzaro passes.
    if (tuning().slab_cluster && slab_smem_bytes(x.R, x.C, w0) > kTwoPerSm && x.C * x.E <= cap - 4) {
        const uint64_t pitch = slab_cluster_pitch(x.C * x.E);
        // two CTAs per SM if a cluster of 16 allows it, else one (still one pass)
        const uint64_t need = (x.R + std::min(16, tuning().max_cluster) - 1) / std::min(16, tuning().max_cluster) * pitch;
        const uint64_t budget = need <= kTwoPerSm ? kTwoPerSm : static_cast<uint64_t>(cap) - 4;
        for (int K : kClusterSizes) {
            if (K > tuning().max_cluster) break;
            if (K == 1) continue;
            const uint64_t Q = (x.R + K - 1) / K;
            if (Q * pitch > budget) continue;
            Pass p;
            p.type = kSlabCluster;
            p.offset = x.offset;
            p.batches = x.B; p.rows = x.R; p.cols = x.C; p.elem = x.E;
            p.strip = x.E;
            p.cluster = K;
            p.what = geom("slab-cluster", x.B, x.R, x.C, x.E);
            // few rows: each CTA's row band would give every output row a few
            // bytes; column bands write contiguous output ranges instead
            if (Q * x.E < static_cast<uint64_t>(tuning().slab_colband)) {
                p.band = colband_width(x.R, x.C, x.E, caps);
                if (p.band) p.what = geom("slab-colband", x.B, x.R, x.C, x.E);
            }
            passes->push_back(p);
            return;
        }
    }
    // rows longer than one CTA's shared memory, few of them: column bands
    // still make it one pass
    if (tuning().slab_cluster && tuning().slab_colband && slab_smem_bytes(x.R, x.C, w0) > kTwoPerSm &&
        x.C * x.E > cap - 4) {
        const uint64_t P = colband_width(x.R, x.C, x.E, caps);
        if (P) {
            Pass p;
            p.type = kSlabCluster;
            p.offset = x.offset;
            p.batches = x.B; p.rows = x.R; p.cols = x.C; p.elem = x.E;
            p.strip = x.E;
            p.cluster = static_cast<int>((x.C + P - 1) / P);
            p.band = P;
            p.what = geom("slab-colband", x.B, x.R, x.C, x.E);
            passes->push_back(p);
            return;
        }
    }
    for (uint64_t w : {w0, uint64_t(128), uint64_t(64), uint64_t(32)}) {
        if (w > w0 || w < std::min<uint64_t>(x.E, 32)) continue;
        if (slab_smem_bytes(x.R, x.C, w) <= cap) {
            Pass p;
            p.type = kSlabTranspose;
            p.offset = x.offset;
            p.batches = x.B; p.rows = x.R; p.cols = x.C; p.elem = x.E;
            p.strip = w;
            p.what = geom("slab", x.B, x.R, x.C, x.E);
            passes->push_back(p);
            return;
        }
    }
    // Catanzaro: c2r on the R x C view, or r2c on the C x R view.
    uint64_t g, inv;
    gcd_inverse(x.R, x.C, &g, &inv);
    const double c2r = (g > 1 ? col_cost(x.R, x.C, x.B, x.E, kFnC2RPreRot, x.C / g, caps) : 0.0) + row_cost(x.C, x.E, cap, false) +
                       col_cost(x.R, x.C, x.B, x.E, kFnC2RColShuffle, x.C / g, caps);
    const double r2c = col_cost(x.C, x.R, x.B, x.E, kFnR2CColShuffle, x.R / g, caps) + row_cost(x.R, x.E, cap, true) +
                       (g > 1 ? col_cost(x.C, x.R, x.B, x.E, kFnR2CPostRot, x.R / g, caps) : 0.0);
    bool use_c2r = (c2r < r2c) || (c2r == r2c && x.C >= x.R);
    if (tuning().variant == 1) use_c2r = true;
    if (tuning().variant == 2) use_c2r = false;
    Pass base;
    base.offset = x.offset;
    base.batches = x.B;
    base.elem = x.E;
    if (use_c2r) {
        const uint64_t m = x.R, n = x.C;
        uint64_t unused, k, q;
        gcd_inverse(m / g, n / g, &unused, &k);  // k = (m/g)^-1 mod (n/g)
        gcd_inverse(n / g, m / g, &unused, &q);  // q = (n/g)^-1 mod (m/g), for the inverse column map
        base.rows = m; base.cols = n;
        base.m = m; base.n = n; base.c = g; base.k = k; base.q = q; base.a = m / g; base.b = n / g;
        if (g > 1) {
            Pass p = base; p.type = kColGather; p.fn = kFnC2RPreRot;
            p.what = geom("c2r-prerotate", x.B, m, n, x.E);
            passes->push_back(p);
        }
        Pass p1 = base; p1.type = kRowGather; p1.fn = kFnRowShuffle;
        p1.what = geom("c2r-rowshuffle", x.B, m, n, x.E);
        passes->push_back(p1);
        Pass p2 = base; p2.type = kColGather; p2.fn = kFnC2RColShuffle;
        p2.what = geom("c2r-colshuffle", x.B, m, n, x.E);
        passes->push_back(p2);
    } else {
        const uint64_t m = x.C, n = x.R;  // the output's view: C rows x R cols
        uint64_t unused, q, k;
        gcd_inverse(n / g, m / g, &unused, &q);  // q = (n/g)^-1 mod (m/g)
        gcd_inverse(m / g, n / g, &unused, &k);  // k = (m/g)^-1 mod (n/g)
        base.rows = m; base.cols = n;
        base.m = m; base.n = n; base.c = g; base.k = k; base.q = q; base.a = m / g; base.b = n / g;
        Pass p0 = base; p0.type = kColGather; p0.fn = kFnR2CColShuffle;
        p0.what = geom("r2c-colshuffle", x.B, m, n, x.E);
        passes->push_back(p0);
        Pass p1 = base; p1.type = kRowScatter; p1.fn = kFnRowShuffle;
        p1.what = geom("r2c-rowscatter", x.B, m, n, x.E);
        passes->push_back(p1);
        if (g > 1) {
            Pass p2 = base; p2.type = kColGather; p2.fn = kFnR2CPostRot;
            p2.what = geom("r2c-postrotate", x.B, m, n, x.E);
            passes->push_back(p2);
        }
    }
}

}  // namespace

bool lower_plan(const NdPlan& plan, uint64_t elem, const DeviceCaps& caps,
                std::vector<Pass>* passes, std::string* err) {
    for (const NdStep& st : plan.steps) {
        switch (st.role) {
            case kPadPre: {
                const auto& d = st.pad_layout;
                const int p = st.pad_pos;
                uint64_t lo = 1, hi = 1;
                for (int i = 0; i < p; ++i) lo *= d[i];
                for (size_t i = p + 1; i < d.size(); ++i) hi *= d[i];
                Pass ps;
                ps.type = kBlockMove;
                ps.block = lo * d[p] * elem;
                ps.n_blocks = hi;
                ps.src_pitch = lo * d[p] * elem;
                ps.dst_pitch = lo * st.pad_size * elem;
                ps.what = "pad-spread";
                passes->push_back(ps);
                break;
            }
            case kPadPost: {
                const auto& d = st.pad_layout;
                const int q = st.pad_pos;
                uint64_t lo = 1, hi = 1;
                for (int i = 0; i < q; ++i) lo *= d[i];
                for (size_t i = q + 1; i < d.size(); ++i) hi *= d[i];
                Pass ps;
                ps.type = kBlockMove;
                ps.block = lo * st.pad_orig * elem;
                ps.n_blocks = hi;
                ps.src_pitch = lo * st.pad_size * elem;
                ps.dst_pitch = lo * st.pad_orig * elem;
                ps.what = "pad-compact";
                passes->push_back(ps);
                break;
            }
            case kPartition:
            case kJoin:
                lower_xpose(xpose_of(st.op, elem, 1, 0), caps, passes);
                break;
            case kRound: {
                const Xpose x = xpose_of(st.op, elem, static_cast<uint64_t>(plan.nb), 0);
                if (x.B == 0) { *err = "internal: unsupported low-order permutation"; return false; }
                lower_xpose(x, caps, passes);
                break;
            }
            default:
                *err = "internal: unknown step";
                return false;
        }
    }
    return true;
}

}  // namespace eithot
