/*
 * ORACLE — test infrastructure only.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load this; the product never does.
 *
 * CPU restatement of the reference's host out-of-place permutation
 * TensorUtil<T>::seq_tt (ITNT/src/tensor_util.cpp:92-104): for every source
 * linear index, the destination index is sum_i coord_i * stride_d(i), where
 * stride_d(i) is the product of the output dims that precede input axis i
 * in the output order.  Restated in 64-bit (the reference's verify_inplace
 * uses int, tensor_util.cpp:117-122) for any element size, with an OpenMP
 * variant used as the timed CPU baseline.
 *
 * Pinned against the reference's own seq_tt compiled from its source
 * (oracle/_ref/ref_seqtt) by tests/golden/make_golden.py.
 */
#include <stdint.h>
#include <stddef.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_MAX_RANK 32

/* perm1[j] (1-based) = input axis placed at output position j. */
static int out_strides(int rank, const int64_t *dims, const int *perm1, int64_t *ostride) {
    int64_t acc = 1;
    int seen[ORACLE_MAX_RANK] = {0};
    if (rank < 1 || rank > ORACLE_MAX_RANK) return -1;
    for (int j = 0; j < rank; ++j) {
        int a = perm1[j] - 1;
        if (a < 0 || a >= rank || seen[a]) return -1;
        seen[a] = 1;
        ostride[a] = acc;
        acc *= dims[a];
    }
    return 0;
}

static inline void copy_elem(unsigned char *dst, const unsigned char *src, size_t elem) {
    switch (elem) {
        case 1: *dst = *src; break;
        case 2: memcpy(dst, src, 2); break;
        case 4: memcpy(dst, src, 4); break;
        case 8: memcpy(dst, src, 8); break;
        default: memcpy(dst, src, elem); break;
    }
}

/* Walks source indices [lo, hi) with an odometer over the input coordinates. */
static void permute_range(const unsigned char *in, unsigned char *out, int rank,
                          const int64_t *dims, const int64_t *ostride, size_t elem,
                          int64_t lo, int64_t hi) {
    int64_t coord[ORACLE_MAX_RANK];
    int64_t rem = lo, dst = 0;
    for (int i = 0; i < rank; ++i) {
        coord[i] = rem % dims[i];
        rem /= dims[i];
        dst += coord[i] * ostride[i];
    }
    for (int64_t src = lo; src < hi; ++src) {
        copy_elem(out + (size_t)dst * elem, in + (size_t)src * elem, elem);
        for (int i = 0; i < rank; ++i) {
            if (++coord[i] < dims[i]) { dst += ostride[i]; break; }
            dst -= (dims[i] - 1) * ostride[i];
            coord[i] = 0;
        }
    }
}

/* Single-threaded, like the reference. Returns 0 on success. */
int oracle_permute(const void *in, void *out, int rank, const int64_t *dims,
                   const int *perm1, size_t elem) {
    int64_t ostride[ORACLE_MAX_RANK];
    int64_t vol = 1;
    if (out_strides(rank, dims, perm1, ostride)) return -1;
    for (int i = 0; i < rank; ++i) vol *= dims[i];
    permute_range((const unsigned char *)in, (unsigned char *)out, rank, dims, ostride, elem, 0, vol);
    return 0;
}

/* Same result on `threads` OpenMP threads (<= 0: all available). */
int oracle_permute_mt(const void *in, void *out, int rank, const int64_t *dims,
                      const int *perm1, size_t elem, int threads) {
    int64_t ostride[ORACLE_MAX_RANK];
    int64_t vol = 1;
    if (out_strides(rank, dims, perm1, ostride)) return -1;
    for (int i = 0; i < rank; ++i) vol *= dims[i];
#ifdef _OPENMP
    int nt = threads > 0 ? threads : omp_get_max_threads();
    int64_t chunk = (vol + 4 * nt - 1) / (4 * nt);
    if (chunk < 4096) chunk = 4096;
    int64_t nchunks = (vol + chunk - 1) / chunk;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1)
    for (int64_t c = 0; c < nchunks; ++c) {
        int64_t lo = c * chunk, hi = lo + chunk < vol ? lo + chunk : vol;
        permute_range((const unsigned char *)in, (unsigned char *)out, rank, dims, ostride, elem, lo, hi);
    }
#else
    (void)threads;
    permute_range((const unsigned char *)in, (unsigned char *)out, rank, dims, ostride, elem, 0, vol);
#endif
    return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Destination index of one source index (used for sampled checks). */
int64_t oracle_dest_index(int rank, const int64_t *dims, const int *perm1, int64_t src) {
    int64_t ostride[ORACLE_MAX_RANK];
    int64_t dst = 0;
    if (out_strides(rank, dims, perm1, ostride)) return -1;
    for (int i = 0; i < rank; ++i) {
        dst += (src % dims[i]) * ostride[i];
        src /= dims[i];
    }
    return dst;
}

/* splitmix64 finaliser: the counter-based content generator shared by the
 * tests, the bench and the device fill kernel (value of element i for seed s
 * is the low elem-size bytes of mix(s ^ (i * golden))). */
static inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

uint64_t oracle_hash_value(uint64_t seed, uint64_t index) {
    return mix64(seed ^ (index * 0xD1B54A32D192ED03ULL));
}

void oracle_fill_hash(void *buf, int64_t n, size_t elem, uint64_t seed, int64_t first_index) {
    unsigned char *b = (unsigned char *)buf;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint64_t v = oracle_hash_value(seed, (uint64_t)(first_index + i));
        unsigned char tmp[8];
        memcpy(tmp, &v, 8); /* little-endian on both build machines */
        for (size_t k = 0; k < elem; ++k) b[(size_t)i * elem + k] = tmp[k % 8];
    }
}
