// Index arithmetic shared by the host planner and the sm_103a kernels:
// division by run-time-invariant divisors and the permutation index maps of
// the in-place passes.  Every map exists in a 32-bit flavour (used when the
// host has checked that all its intermediate values stay below 2^31) and a
// 64-bit flavour.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define EI_HD __host__ __device__ __forceinline__
#else
#define EI_HD inline
#endif

namespace eithot {

EI_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return static_cast<uint64_t>((static_cast<unsigned __int128>(a) * b) >> 64);
#endif
}

EI_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return static_cast<uint32_t>((static_cast<uint64_t>(a) * b) >> 32);
#endif
}

// Division by an invariant divisor d >= 1 using the round-up multiplier
// method (Granlund & Montgomery, PLDI 1994, Thm 4.2): with l = ceil(log2 d)
// and N the dividend width, m = ceil(2^(N+l) / d) gives
// floor(x/d) = floor(x*m / 2^(N+l)) for every x < 2^N.  N = 31 when the host
// knows all dividends stay below 2^31 (one 32-bit multiply-high), else
// N = 62 (one 64-bit multiply-high).
struct FastDiv {
    uint64_t d = 1;
    uint64_t m = 0;
    uint32_t s = 0;
    uint32_t mode = 0;  // 0: d==1, 1: power of two, 2: 32-bit magic, 3: 64-bit magic

    // max_dividend: an upper bound (inclusive) on every x passed to div().
    static FastDiv make(uint64_t divisor, uint64_t max_dividend) {
        FastDiv f;
        f.d = divisor;
        if (divisor <= 1) { f.mode = 0; return f; }
        uint32_t l = 0;
        while ((uint64_t(1) << l) < divisor) ++l;  // l = ceil(log2 d)
        if ((divisor & (divisor - 1)) == 0) { f.mode = 1; f.s = l; return f; }
        if (max_dividend < (uint64_t(1) << 31)) {
            f.mode = 2;
            f.m = ((uint64_t(1) << (31 + l)) + divisor - 1) / divisor;   // < 2^32
            f.s = l - 1;
        } else {
            f.mode = 3;
            unsigned __int128 num = (static_cast<unsigned __int128>(1) << (62 + l));
            f.m = static_cast<uint64_t>((num + divisor - 1) / divisor);  // <= 2^63
            f.s = l - 2;
        }
        return f;
    }

    EI_HD uint64_t div(uint64_t x) const {
        switch (mode) {
            case 0: return x;
            case 1: return x >> s;
            case 2: return mulhi32(static_cast<uint32_t>(x), static_cast<uint32_t>(m)) >> s;
            default: return mulhi64(x, m) >> s;
        }
    }
    EI_HD uint64_t mod(uint64_t x) const { return x - div(x) * d; }
    EI_HD void divmod(uint64_t x, uint64_t& q, uint64_t& r) const { q = div(x); r = x - q * d; }
};

// 32-bit-only variant: divisor and every dividend below 2^31.
struct FastDiv32 {
    uint32_t d = 1;
    uint32_t m = 0;
    uint32_t s = 0;
    uint32_t mode = 0;  // 0: d==1, 1: power of two, 2: magic

    static FastDiv32 make(uint64_t divisor) {
        const FastDiv f = FastDiv::make(divisor, 0);
        FastDiv32 g;
        g.d = static_cast<uint32_t>(f.d);
        g.m = static_cast<uint32_t>(f.m);
        g.s = f.s;
        g.mode = f.mode;
        return g;
    }
    EI_HD uint32_t div(uint32_t x) const {
        return mode == 2 ? (mulhi32(x, m) >> s) : (mode == 1 ? (x >> s) : x);
    }
    EI_HD uint32_t mod(uint32_t x) const { return x - div(x) * d; }
    EI_HD void divmod(uint32_t x, uint32_t& q, uint32_t& r) const { q = div(x); r = x - q * d; }
};

template <typename I> struct DivOf;
template <> struct DivOf<uint32_t> { using T = FastDiv32; };
template <> struct DivOf<uint64_t> { using T = FastDiv; };

// (a * b) mod n for a, b < n; n built with max_dividend >= (n-1)^2 when
// n <= 2^31.
EI_HD uint64_t mulmod(uint64_t a, uint64_t b, const FastDiv& n) {
    if (n.d <= (uint64_t(1) << 31)) return n.mod(a * b);  // a*b < 2^62
    unsigned __int128 p = static_cast<unsigned __int128>(a) * b;
    return static_cast<uint64_t>(p % n.d);
}

// ---------------------------------------------------------------------------
// Index maps.  A "row op" permutes the elements of each row of a row-major
// rows x cols matrix; a "col op" permutes the elements of each column.
//   row gather : out[i][j] = in[i][f(i,j)]
//   row scatter: out[i][f(i,j)] = in[i][j]
//   col gather : out[i][j] = in[g(i,j)][j]
// Catanzaro, Keller & Garland, "A decomposition for in-place matrix
// transposition" (PPoPP 2014), parameterised as in EITHOT
// (ITNT/src/equations.h:319-534, ITNT/src/2dtranspose.cpp:130-181).
// View: m rows x n cols; c = gcd(m, n); b = n / c; k = (m/c)^-1 mod (n/c).
// ---------------------------------------------------------------------------

// c2r pre-rotation (col gather): row i of column j takes row (i + j/b) mod m.
template <typename I>
struct FnC2RPreRotT {
    using index_type = I;
    I m;
    typename DivOf<I>::T divb;
    EI_HD I operator()(I i, I j) const {
        const I x = i + divb.div(j);
        return x >= m ? x - m : x;
    }
};

// Row shuffle used as a gather by c2r and as a scatter by r2c: with
// f = j + i(n-1) (+ m when i - (j mod c) > m - c),
// index = (k * (f / c) mod b) + (f mod c) * b.
template <typename I>
struct FnRowShuffleT {
    using index_type = I;
    I m, n, c, k, b;
    typename DivOf<I>::T divc, divb;
    FastDiv divb_mul;  // b, for the product k * x < b^2
    EI_HD I operator()(I i, I j) const {
        I f = j + i * (n - 1);
        const I jc = divc.mod(j);
        if (static_cast<int64_t>(i) - static_cast<int64_t>(jc) > static_cast<int64_t>(m) - static_cast<int64_t>(c))
            f += m;
        I fq, fr;
        divc.divmod(f, fq, fr);
        return static_cast<I>(mulmod(k, divb.mod(fq), divb_mul)) + fr * b;
    }
};

// Inverse of the row shuffle (EITHOT's otherwise unused r2c::row_shuffle,
// ITNT/src/equations.h:440-464): j -> ((j/b + i) mod m + j*m) mod n.  A
// gather with this map equals a scatter with FnRowShuffleT and vice versa,
// so either row pass can be run in whichever direction stages better.
template <typename I>
struct FnRowShuffleInvT {
    using index_type = I;
    I m, n;
    typename DivOf<I>::T divb, divm, divn;
    EI_HD I operator()(I i, I j) const {
        I r = divb.div(j) + i;
        if (r >= m) r = divm.mod(r);
        return divn.mod(r + j * m);
    }
};

// c2r column shuffle (col gather): row i of column j takes
// (i*n - floor(i*c/m) + j) mod m.
template <typename I>
struct FnC2RColShuffleT {
    using index_type = I;
    I n, c;
    typename DivOf<I>::T divm;
    EI_HD I operator()(I i, I j) const { return divm.mod(i * n - divm.div(i * c) + j); }
};

// r2c column shuffle (col gather): row i of column j takes
// p((i + m - (j mod m)) mod m) with
// p(x) = a*((c-1)x mod c) + (floor((c-1+x)/c) * q mod a).
template <typename I>
struct FnR2CColShuffleT {
    using index_type = I;
    I m, a, c, q;
    typename DivOf<I>::T divm, divc, diva;
    FastDiv diva_mul;  // a, for the product (.) * q < a^2
    EI_HD I operator()(I i, I j) const {
        I x = i + m - divm.mod(j);
        if (x >= m) x -= m;
        const I t1 = a * divc.mod((c - 1) * x);
        const I t2 = static_cast<I>(mulmod(diva.mod(divc.div(c - 1 + x)), q, diva_mul));
        return t1 + t2;
    }
};

// r2c post-rotation (col gather): row i of column j takes (i + m - j/b) mod m.
template <typename I>
struct FnR2CPostRotT {
    using index_type = I;
    I m;
    typename DivOf<I>::T divb;
    EI_HD I operator()(I i, I j) const {
        const I x = i + m - divb.div(j);
        return x >= m ? x - m : x;
    }
};

// ---------------------------------------------------------------------------
// Owner maps.  Every column gather above reads, for output row i of column
// j, source row sigma((T(i) + delta(j)) mod m) with T and sigma bijections.
// A CTA that stages "slots" t (slot t holds source row sigma(t)) can then
// write the whole row piece of output row T^-1((t - delta(j0)) mod m) of a
// tile starting at column j0, element j0+c coming from slot
// t + delta(j0+c) - delta(j0):
//   c2r column shuffle: sigma = id, delta = j;    output row = r2c column shuffle at (t, j0)
//   c2r pre-rotation:   sigma = id, delta = j/b;  output row = r2c post-rotation at (t, j0)
//   r2c post-rotation:  sigma = id, delta = -j/b; output row = c2r pre-rotation at (t, j0)
//   r2c column shuffle: sigma = p(., 0), T = id, delta = -j; output row = (t + j0) mod m
// (the r2c column shuffle is p((i - j) mod m), p(x) its value at column 0).
// ---------------------------------------------------------------------------
template <typename I>
struct OwnerColShuffleT {
    using index_type = I;
    FnR2CColShuffleT<I> inv;
    EI_HD I stage_of(I t) const { return t; }
    EI_HD I row_of(I t, I j0) const { return inv(t, j0); }
    EI_HD int64_t delta(I j) const { return static_cast<int64_t>(j); }
};
template <typename I>
struct OwnerPreRotT {
    using index_type = I;
    FnR2CPostRotT<I> inv;
    EI_HD I stage_of(I t) const { return t; }
    EI_HD I row_of(I t, I j0) const { return inv(t, j0); }
    EI_HD int64_t delta(I j) const { return static_cast<int64_t>(inv.divb.div(j)); }
};
template <typename I>
struct OwnerPostRotT {
    using index_type = I;
    FnC2RPreRotT<I> inv;
    EI_HD I stage_of(I t) const { return t; }
    EI_HD I row_of(I t, I j0) const { return inv(t, j0); }
    EI_HD int64_t delta(I j) const { return -static_cast<int64_t>(inv.divb.div(j)); }
};
template <typename I>
struct OwnerR2CColShuffleT {
    using index_type = I;
    FnR2CColShuffleT<I> fn;
    EI_HD I stage_of(I t) const { return fn(t, 0); }
    EI_HD I row_of(I t, I j0) const { return fn.divm.mod(t + j0); }
    EI_HD int64_t delta(I j) const { return -static_cast<int64_t>(j); }
};

using FnC2RPreRot = FnC2RPreRotT<uint64_t>;
using FnRowShuffle = FnRowShuffleT<uint64_t>;
using FnC2RColShuffle = FnC2RColShuffleT<uint64_t>;
using FnR2CColShuffle = FnR2CColShuffleT<uint64_t>;
using FnR2CPostRot = FnR2CPostRotT<uint64_t>;

}  // namespace eithot
