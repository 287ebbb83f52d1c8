// Test infrastructure (oracle side): records the low-order calls that the
// reference's own N-d orchestration makes.  Linked with the reference's
// ITNT/src/Nd_transpose.cpp, permutation_util.cpp, Nd_decompose.cpp and
// util.cpp, compiled from where they lie; this file supplies the layer below
// them (the 2D/3D/4D transposes and the padding kernels) as recorders, so the
// printed sequence is exactly what ITNT/src/Nd_transpose.cpp:256-304 issues.
//
// usage: ref_plan d0 .. d{r-1} p0 .. p{r-1} (1-based) nb alpha
// prints one line per call:  <tag> <source> <dims...>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace inplace {
namespace _Nd {
template <typename T>
void transpose(T* data, int source, void* dim, void* permutation, int rank, int num_block, double LARGE_RATIO);
}

namespace _2d {
template <typename T>
void transpose(T*, int source, void* dim, int, double) {
    int* d = reinterpret_cast<int*>(dim);
    std::printf("21 %d %d %d\n", source, d[0], d[1]);
}
template void transpose(float*, int, void*, int, double);
template void transpose(double*, int, void*, int, double);
}  // namespace _2d

namespace _3d {
#define EITHOT_REC3(NS, TAG)                                                   \
    namespace NS {                                                            \
    template <typename T>                                                     \
    void transpose(T*, int source, int d1, int d2, int d3, int, double) {     \
        std::printf(TAG " %d %d %d %d\n", source, d1, d2, d3);                \
    }                                                                         \
    template void transpose(float*, int, int, int, int, int, double);         \
    template void transpose(double*, int, int, int, int, int, double);        \
    }
EITHOT_REC3(_231, "231")
EITHOT_REC3(_312, "312")
EITHOT_REC3(_213, "213")
EITHOT_REC3(_132, "132")
}  // namespace _3d

namespace _4d {
namespace _1324 {
template <typename T>
void transpose(T*, int source, int d1, int d2, int d3, int d4, int, double) {
    std::printf("1324 %d %d %d %d %d\n", source, d1, d2, d3, d4);
}
template void transpose(float*, int, int, int, int, int, int, double);
template void transpose(double*, int, int, int, int, int, int, double);
}  // namespace _1324
}  // namespace _4d

template <typename T>
void Nd_padding_pre_process(T*, int* dim, size_t*, int rank, int pos, int nb) {
    std::printf("PADPRE 0 %d %d %d", pos, dim[pos], nb);
    for (int i = 0; i < rank; ++i) std::printf(" %d", dim[i]);
    std::printf("\n");
}
template <typename T>
void Nd_padding_post_process(T*, int* dim, int* perm, int rank, int pos, int nb) {
    std::printf("PADPOST 0 %d %d %d", pos, dim[pos], nb);
    for (int i = 0; i < rank; ++i) std::printf(" %d", perm[i]);
    std::printf("\n");
}
template void Nd_padding_pre_process(float*, int*, size_t*, int, int, int);
template void Nd_padding_pre_process(double*, int*, size_t*, int, int, int);
template void Nd_padding_post_process(float*, int*, int*, int, int, int);
template void Nd_padding_post_process(double*, int*, int*, int, int, int);
}  // namespace inplace

int main(int argc, char** argv) {
    if (argc < 6 || (argc - 3) % 2 != 0) {
        std::fprintf(stderr, "usage: ref_plan dims.. perm(1-based).. nb alpha\n");
        return 2;
    }
    const int rank = (argc - 3) / 2;
    std::vector<int> dim(rank), perm(rank);
    int k = 1;
    for (int i = 0; i < rank; ++i) dim[i] = std::atoi(argv[k++]);
    for (int i = 0; i < rank; ++i) perm[i] = std::atoi(argv[k++]) - 1;  // the library takes 0-based
    const int nb = std::atoi(argv[k++]);
    const double alpha = std::atof(argv[k++]);
    inplace::_Nd::transpose(static_cast<float*>(nullptr), 0, dim.data(), perm.data(), rank, nb, alpha);
    return 0;
}
