// Construction of the pass index maps from a Pass, shared by the device
// executor and host-side tools.  Each FastDiv is sized for the largest
// dividend its map can see.
#pragma once

#include <algorithm>

#include "index_math.cuh"
#include "passes.h"

namespace eithot {

inline FnRowShuffle make_rowshuffle(const Pass& p) {
    FnRowShuffle f;
    f.m = static_cast<int64_t>(p.m);
    f.n = static_cast<int64_t>(p.n);
    f.c = static_cast<int64_t>(p.c);
    f.k = p.k;
    f.b = p.b;
    const uint64_t fmax = p.n + p.m * p.n + p.m;
    f.divc = FastDiv::make(p.c, fmax);
    const uint64_t bmax = std::max<uint64_t>(fmax / std::max<uint64_t>(p.c, 1) + 1, p.b * p.b);
    f.divb = FastDiv::make(p.b, bmax);
    return f;
}
inline FnC2RPreRot make_prerot(const Pass& p) {
    FnC2RPreRot f;
    f.m = p.m;
    f.divb = FastDiv::make(p.b, p.n);
    return f;
}
inline FnR2CPostRot make_postrot(const Pass& p) {
    FnR2CPostRot f;
    f.m = p.m;
    f.divb = FastDiv::make(p.b, p.n);
    return f;
}
inline FnC2RColShuffle make_c2r_colshuf(const Pass& p) {
    FnC2RColShuffle f;
    f.n = p.n;
    f.c = p.c;
    f.divm = FastDiv::make(p.m, p.m * p.n + p.n + p.m * p.c);
    return f;
}
inline FnR2CColShuffle make_r2c_colshuf(const Pass& p) {
    FnR2CColShuffle f;
    f.m = p.m; f.a = p.a; f.c = p.c; f.q = p.q;
    f.divm = FastDiv::make(p.m, p.n + p.m);
    f.divc = FastDiv::make(p.c, p.c * p.m + p.c + p.m);
    f.diva = FastDiv::make(p.a, std::max<uint64_t>(p.m + p.c, p.a * p.a));
    return f;
}

}  // namespace eithot
