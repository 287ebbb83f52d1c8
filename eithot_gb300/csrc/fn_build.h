// Construction of the pass index maps from a Pass, shared by the device
// executor and host-side tools.  Each divisor is sized for the largest
// dividend its map can see.
#pragma once

#include <algorithm>

#include "index_math.cuh"
#include "passes.h"

namespace eithot {

// The 32-bit flavour of a Catanzaro map is exact when every intermediate
// value stays below 2^31; the largest is below m*n + m + n.
inline bool fits32(const Pass& p) {
    const unsigned __int128 v = static_cast<unsigned __int128>(p.m) * p.n + p.m + p.n;
    return v < (static_cast<unsigned __int128>(1) << 31);
}

template <typename I> struct MakeDiv;
template <> struct MakeDiv<uint32_t> {
    static FastDiv32 make(uint64_t d, uint64_t) { return FastDiv32::make(d); }
};
template <> struct MakeDiv<uint64_t> {
    static FastDiv make(uint64_t d, uint64_t max_dividend) { return FastDiv::make(d, max_dividend); }
};

template <typename I>
inline FnRowShuffleT<I> make_rowshuffle(const Pass& p) {
    FnRowShuffleT<I> f;
    f.m = static_cast<I>(p.m);
    f.n = static_cast<I>(p.n);
    f.c = static_cast<I>(p.c);
    f.k = static_cast<I>(p.k);
    f.b = static_cast<I>(p.b);
    const uint64_t fmax = p.n + p.m * p.n + p.m;
    f.divc = MakeDiv<I>::make(p.c, fmax);
    f.divb = MakeDiv<I>::make(p.b, fmax / std::max<uint64_t>(p.c, 1) + 1);
    f.divb_mul = FastDiv::make(p.b, p.b * p.b);
    return f;
}
template <typename I>
inline FnRowShuffleInvT<I> make_rowshuffle_inv(const Pass& p) {
    FnRowShuffleInvT<I> f;
    f.m = static_cast<I>(p.m);
    f.n = static_cast<I>(p.n);
    f.divb = MakeDiv<I>::make(p.b, p.n);
    f.divm = MakeDiv<I>::make(p.m, p.n / std::max<uint64_t>(p.b, 1) + p.m);
    f.divn = MakeDiv<I>::make(p.n, p.m + p.n * p.m);
    return f;
}

template <typename I>
inline FnC2RPreRotT<I> make_prerot(const Pass& p) {
    FnC2RPreRotT<I> f;
    f.m = static_cast<I>(p.m);
    f.divb = MakeDiv<I>::make(p.b, p.n);
    return f;
}
template <typename I>
inline FnR2CPostRotT<I> make_postrot(const Pass& p) {
    FnR2CPostRotT<I> f;
    f.m = static_cast<I>(p.m);
    f.divb = MakeDiv<I>::make(p.b, p.n);
    return f;
}
template <typename I>
inline FnC2RColShuffleT<I> make_c2r_colshuf(const Pass& p) {
    FnC2RColShuffleT<I> f;
    f.n = static_cast<I>(p.n);
    f.c = static_cast<I>(p.c);
    f.divm = MakeDiv<I>::make(p.m, p.m * p.n + p.n + p.m * p.c);
    return f;
}
template <typename I>
inline FnR2CColShuffleT<I> make_r2c_colshuf(const Pass& p) {
    FnR2CColShuffleT<I> f;
    f.m = static_cast<I>(p.m);
    f.a = static_cast<I>(p.a);
    f.c = static_cast<I>(p.c);
    f.q = static_cast<I>(p.q);
    f.divm = MakeDiv<I>::make(p.m, p.n + p.m);
    f.divc = MakeDiv<I>::make(p.c, p.c * p.m + p.c + p.m);
    f.diva = MakeDiv<I>::make(p.a, p.m + p.c);
    f.diva_mul = FastDiv::make(p.a, p.a * p.a);
    return f;
}

// Owner maps of the column passes that have one (see index_math.cuh).
template <typename I>
inline OwnerColShuffleT<I> make_owner_colshuf(const Pass& p) {
    OwnerColShuffleT<I> o;
    o.inv = make_r2c_colshuf<I>(p);
    return o;
}
template <typename I>
inline OwnerPreRotT<I> make_owner_prerot(const Pass& p) {
    OwnerPreRotT<I> o;
    o.inv = make_postrot<I>(p);
    return o;
}
template <typename I>
inline OwnerPostRotT<I> make_owner_postrot(const Pass& p) {
    OwnerPostRotT<I> o;
    o.inv = make_prerot<I>(p);
    return o;
}
template <typename I>
inline OwnerR2CColShuffleT<I> make_owner_r2c_colshuf(const Pass& p) {
    OwnerR2CColShuffleT<I> o;
    o.fn = make_r2c_colshuf<I>(p);
    return o;
}

}  // namespace eithot
