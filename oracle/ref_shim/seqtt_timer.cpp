// Test infrastructure (baseline side): times the reference's own host
// out-of-place permutation TensorUtil<T>::seq_tt (ITNT/src/tensor_util.cpp:
// 92-104), compiled from the reference's sources, on iota data
// (TensorUtil::init_data, :54-56), single-threaded as the reference runs it.
// usage: ref_seqtt_timer elem(4|8) runs warmup d0..d{r-1} p0..p{r-1}(1-based)
// prints: "<seconds per run> <runs> <an output element>" (median of the timed
// runs, after `warmup` untimed ones)
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "tensor_util.h"

template <typename T>
static int run(int runs, int warmup, int rank, int* dim, int* perm0) {
    TensorUtil<T> tu(nullptr, rank, dim, 0, perm0);
    std::vector<T> in(tu.vol), out(tu.vol);
    tu.init_data(in.data());
    for (int r = 0; r < warmup; ++r) tu.seq_tt(out.data(), in.data());
    std::vector<double> t;
    for (int r = 0; r < runs; ++r) {
        const auto t0 = std::chrono::steady_clock::now();
        tu.seq_tt(out.data(), in.data());
        t.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    }
    std::sort(t.begin(), t.end());
    // the output depends on every input element: print one so the work stays
    std::printf("%.6f %d %lld\n", t[t.size() / 2], runs, static_cast<long long>(out[tu.vol / 2]));
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 6 || (argc - 4) % 2 != 0) return 2;
    const int elem = std::atoi(argv[1]);
    const int runs = std::max(1, std::atoi(argv[2]));
    const int warmup = std::max(0, std::atoi(argv[3]));
    const int rank = (argc - 4) / 2;
    std::vector<int> dim(rank), perm(rank);
    for (int i = 0; i < rank; ++i) dim[i] = std::atoi(argv[4 + i]);
    for (int i = 0; i < rank; ++i) perm[i] = std::atoi(argv[4 + rank + i]) - 1;
    if (elem == 4) return run<int>(runs, warmup, rank, dim.data(), perm.data());
    if (elem == 8) return run<long long>(runs, warmup, rank, dim.data(), perm.data());
    return 2;
}
