// Test infrastructure (oracle side): stands in for the reference estimator's
// Nd_padding.cu, whose two functions only return the temp size of the
// padding kernels, sizeof(T) * n_blocks * 1024 with n_blocks the resident
// 1024-thread blocks of the whole GPU (Nd_memory_estimation/src/
// Nd_padding.cu:96-118).  n_blocks comes from EITHOT_REF_PAD_BLOCKS
// (default 152 SMs x 2 blocks) because the occupancy query needs a GPU.
#include <cstdlib>
#include <cstddef>

static size_t pad_blocks() {
    const char* v = std::getenv("EITHOT_REF_PAD_BLOCKS");
    return v ? static_cast<size_t>(std::atol(v)) : 304;
}
namespace inplace {
template <typename T>
size_t Dimension_Pre_Padding(T*, int*, size_t*, int, int, int) { return sizeof(T) * pad_blocks() * 1024; }
template <typename T>
size_t Dimension_Post_Padding(T*, int*, int*, int, int, int) { return sizeof(T) * pad_blocks() * 1024; }
template size_t Dimension_Pre_Padding(int*, int*, size_t*, int, int, int);
template size_t Dimension_Pre_Padding(long long*, int*, size_t*, int, int, int);
template size_t Dimension_Pre_Padding(float*, int*, size_t*, int, int, int);
template size_t Dimension_Pre_Padding(double*, int*, size_t*, int, int, int);
template size_t Dimension_Post_Padding(int*, int*, int*, int, int, int);
template size_t Dimension_Post_Padding(long long*, int*, int*, int, int, int);
template size_t Dimension_Post_Padding(float*, int*, int*, int, int, int);
template size_t Dimension_Post_Padding(double*, int*, int*, int, int, int);
}  // namespace inplace
