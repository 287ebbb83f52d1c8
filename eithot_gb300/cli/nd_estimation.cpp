// Drop-in replacement for the reference's Nd_estimation program
// (Nd_memory_estimation/src/test_inplace.cpp:19-147, main at :148-181):
//
//   Nd_estimation dims... perm(1-based)... type_size nb alpha [filename]
//
// prints the same lines to stdout and appends the same
// "dims perm type_size nb alpha" line to proper_input.txt in the working
// directory, with the estimate computed by eithot_estimate_report (64-bit:
// no 22 GB limit, no int overflow).  The requested nb and the optional
// filename are accepted and ignored, as by the reference.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "eithot.h"

int main(int argc, char** argv) {
    const int rank = (argc - 1) / 2 - 1;
    if (rank < 1 || (argc != 2 * (rank + 1) + 2 && argc != 2 * (rank + 1) + 3)) {
        std::fprintf(stderr, "usage: %s dims... perm(1-based)... type_size nb alpha [filename]\n", argv[0]);
        return 2;
    }
    std::vector<int64_t> dims(rank);
    std::vector<int> perm(rank);
    int k = 1;
    for (int i = 0; i < rank; ++i) dims[i] = std::atoll(argv[k++]);
    for (int i = 0; i < rank; ++i) perm[i] = std::atoi(argv[k++]);
    const int type_size = std::atoi(argv[k++]);
    (void)std::atoi(argv[k++]);  // requested nb: the estimator chooses its own
    const double alpha = std::atof(argv[k++]);

    eithot_estimate_info info;
    if (eithot_estimate_report(rank, dims.data(), perm.data(), static_cast<size_t>(type_size > 0 ? type_size : 8),
                               alpha, 0, 0, &info) != EITHOT_OK) {
        std::fprintf(stderr, "Nd_estimation: %s\n", eithot_last_error());
        return 1;
    }
    std::printf("init Extra Memory size = %.5f MB\n", static_cast<double>(info.init_extra_bytes) / 1e6);
    if (info.init_extra_bytes > 0) std::printf("new ratio = %f\n", info.alpha_raised);
    if (info.decomposed)
        std::printf("Final Extra Memory Size = %.5f MB, take %.5f percent input data size\n",
                    static_cast<double>(info.final_extra_bytes) / 1e6, info.final_ratio);
    std::printf("\t");
    for (int i = 0; i < rank; ++i) std::printf("%lld ", static_cast<long long>(dims[i]));
    for (int i = 0; i < rank; ++i) std::printf("%d ", perm[i]);
    std::printf("%d %d %.2f\n", type_size, info.nb, info.alpha);
    if (FILE* f = std::fopen("proper_input.txt", "a+")) {
        for (int i = 0; i < rank; ++i) std::fprintf(f, "%lld ", static_cast<long long>(dims[i]));
        for (int i = 0; i < rank; ++i) std::fprintf(f, "%d ", perm[i]);
        std::fprintf(f, "%d %d %.2f\n", type_size, info.nb, info.alpha);
        std::fclose(f);
    }
    return 0;
}
