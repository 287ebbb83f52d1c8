// Test infrastructure (oracle side): runs the reference's own host
// out-of-place permutation TensorUtil<T>::seq_tt (ITNT/src/tensor_util.cpp:
// 92-104), compiled from where it lies, on raw bytes.
// usage: ref_seqtt elem(4|8) d0..d{r-1} p0..p{r-1}(1-based) < in.bin > out.bin
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "tensor_util.h"

template <typename T>
static int run(int rank, int* dim, int* perm0) {
    TensorUtil<T> tu(nullptr, rank, dim, 0, perm0);
    std::vector<T> in(tu.vol), out(tu.vol);
    if (std::fread(in.data(), sizeof(T), tu.vol, stdin) != tu.vol) return 3;
    tu.seq_tt(out.data(), in.data());
    std::fwrite(out.data(), sizeof(T), tu.vol, stdout);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 4 || (argc - 2) % 2 != 0) return 2;
    const int elem = std::atoi(argv[1]);
    const int rank = (argc - 2) / 2;
    std::vector<int> dim(rank), perm(rank);
    for (int i = 0; i < rank; ++i) dim[i] = std::atoi(argv[2 + i]);
    for (int i = 0; i < rank; ++i) perm[i] = std::atoi(argv[2 + rank + i]) - 1;
    if (elem == 4) return run<int>(rank, dim.data(), perm.data());
    if (elem == 8) return run<long long>(rank, dim.data(), perm.data());
    return 2;
}
