// Index arithmetic shared by the host planner and the sm_103a kernels:
// division by run-time-invariant divisors and the permutation index maps of
// the in-place passes.  All maps are pure functions of 64-bit indices.
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

    FastDiv() = default;

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

// (a * b) mod n for a, b < n.
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
// ---------------------------------------------------------------------------

// Transpose of an R x C matrix flattened into one row of R*C elements
// (the single-pass "linearisation" of EITHOT's 213 row_shuffle,
// ITNT/src/equations.h:285-311, generalised to any element width):
// output o = c*R + r takes input r*C + c.
struct FnTranspose {
    uint64_t R, C;
    FastDiv divR;
    EI_HD uint64_t operator()(uint64_t, uint64_t o) const {
        uint64_t c, r;
        divR.divmod(o, c, r);
        return r * C + c;
    }
};

// Catanzaro, Keller & Garland, "A decomposition for in-place matrix
// transposition" (PPoPP 2014), as parameterised by EITHOT
// (ITNT/src/equations.h:319-534, ITNT/src/2dtranspose.cpp:130-181).
// View: m rows x n cols; c = gcd(m, n); b = n / c; k = (m/c)^-1 mod (n/c).

// c2r pre-rotation (col gather): row i of column j takes row (i + j/b) mod m.
struct FnC2RPreRot {
    uint64_t m;
    FastDiv divb;
    EI_HD uint64_t operator()(uint64_t i, uint64_t j) const {
        uint64_t x = i + divb.div(j);
        return x >= m ? x - m : x;
    }
};

// Row shuffle used as a gather by c2r and as a scatter by r2c: with
// f = j + i(n-1) (+ m when i - (j mod c) > m - c),
// index = (k * (f / c) mod b) + (f mod c) * b.
struct FnRowShuffle {
    int64_t m, n, c;
    uint64_t k, b;
    FastDiv divc, divb;
    EI_HD uint64_t operator()(uint64_t i, uint64_t j) const {
        uint64_t f = j + i * static_cast<uint64_t>(n - 1);
        const uint64_t jc = divc.mod(j);
        if (static_cast<int64_t>(i) - static_cast<int64_t>(jc) > m - c) f += static_cast<uint64_t>(m);
        uint64_t fq, fr;
        divc.divmod(f, fq, fr);
        return mulmod(k, divb.mod(fq), divb) + fr * b;
    }
};

// c2r column shuffle (col gather): row i of column j takes
// (i*n - floor(i*c/m) + j) mod m.
struct FnC2RColShuffle {
    uint64_t n, c;
    FastDiv divm;
    EI_HD uint64_t operator()(uint64_t i, uint64_t j) const {
        return divm.mod(i * n - divm.div(i * c) + j);
    }
};

// r2c column shuffle (col gather): row i of column j takes
// p((i + m - (j mod m)) mod m), p(x) = a*((c-1)x mod c) + ((ceil-ish(x/c))*q mod a).
struct FnR2CColShuffle {
    uint64_t m, a, c, q;
    FastDiv divm, divc, diva;
    EI_HD uint64_t operator()(uint64_t i, uint64_t j) const {
        uint64_t x = i + m - divm.mod(j);
        if (x >= m) x -= m;
        const uint64_t t1 = a * divc.mod((c - 1) * x);
        const uint64_t t2 = mulmod(diva.mod(divc.div(c - 1 + x)), q, diva);
        return t1 + t2;
    }
};

// r2c post-rotation (col gather): row i of column j takes (i + m - j/b) mod m.
struct FnR2CPostRot {
    uint64_t m;
    FastDiv divb;
    EI_HD uint64_t operator()(uint64_t i, uint64_t j) const {
        uint64_t x = i + m - divb.div(j);
        return x >= m ? x - m : x;
    }
};

}  // namespace eithot
