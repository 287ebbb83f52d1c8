// Drop-in replacement for the reference's test_inplace benchmark driver
// (ITNT/src/test_inplace.cpp, memcpy path :15-88, main :142-175):
//
//   test_inplace dims... perm(1-based)... type_size nb alpha [filename]
//
// fills a pinned host tensor with iota (element i = i, TensorUtil::init_data,
// ITNT/src/tensor_util.cpp:54-56), copies it to a device buffer with 3 %
// padding slack, transposes it in place through eithot_transpose, copies it
// back, checks it as TensorUtil::verify_inplace does (tensor_util.cpp:
// 113-142) and prints the same lines; the total time and the throughput
// 2 * bytes / time are appended to inplace_bench.txt and
// inplace_bench_throughput.txt in the working directory.  type_size 4 moves
// 32-bit and type_size > 4 64-bit elements as in the reference; 1 and 2
// (8- and 16-bit elements, whose iota wraps) are accepted too.  Dims are
// 64-bit: there is no 22 GB limit.  Errors print a message and exit 1
// instead of the reference's exit(-1).
//
// EITHOT_REORDER_TYPE=0|1|2|3 in the environment selects the decomposition
// order the reference selects at compile time (REORDER_TYPE in
// ITNT/src/Nd_transpose.cpp:22-28: 0 mixed, 1 pre-order, 2 post-order; its
// README's experiment 6 rebuilds the program for each), or 3 for this
// library's fewest-pass plans; unset, the reference's default (mixed).
//
// EITHOT_MEMORY_TYPE=2 in the environment selects the reference's managed
// path, which it selects at compile time (MEMORY_TYPE 2,
// padding_managed_transpose, ITNT/src/test_inplace.cpp:91-136): the tensor
// lives in cudaMallocManaged memory with 3 % slack (host-filled, transposed
// where it lies, checked in place by the host), its own output lines, and
// the throughput 2 * slack-padded bytes / time.  The reference never
// records its start event there, so its elapsed-time call fails; this
// program records it before the transpose.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "eithot.h"

namespace {

constexpr double kPaddingSlack = 0.03;

// EITHOT_REORDER_TYPE from the environment (0 mixed when unset).
int reorder_type() {
    const char* v = std::getenv("EITHOT_REORDER_TYPE");
    const int t = v ? std::atoi(v) : EITHOT_ORDER_MIXED;
    return (t >= EITHOT_ORDER_MIXED && t <= EITHOT_ORDER_FEWEST) ? t : EITHOT_ORDER_MIXED;
}

#define CLI_CHECK(expr)                                                                   \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            std::fprintf(stderr, "test_inplace: %s: %s\n", #expr, cudaGetErrorString(e_)); \
            std::exit(1);                                                                 \
        }                                                                                 \
    } while (0)

template <typename T>
void init_iota(T* h, int64_t n) {
    const unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([=] {
            const int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
            for (int64_t i = lo; i < hi; ++i) h[i] = static_cast<T>(i);
        });
    for (auto& x : th) x.join();
}

// Every source element s must sit at its destination: output axis j is
// input axis perm[j]-1, axis 0 fastest.
template <typename T>
bool verify_inplace(const T* h, const std::vector<int64_t>& dims, const std::vector<int>& perm) {
    const int rank = static_cast<int>(dims.size());
    std::vector<int64_t> ostride(rank);
    int64_t acc = 1;
    for (int j = 0; j < rank; ++j) {
        ostride[perm[j] - 1] = acc;
        acc *= dims[perm[j] - 1];
    }
    const int64_t n = acc;
    const unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::atomic<bool> ok(true);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            const int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
            if (lo >= hi) return;
            std::vector<int64_t> c(rank);
            int64_t r = lo, d = 0;
            for (int i = 0; i < rank; ++i) {
                c[i] = r % dims[i];
                r /= dims[i];
                d += c[i] * ostride[i];
            }
            for (int64_t s = lo; s < hi; ++s) {
                if (h[d] != static_cast<T>(s)) { ok = false; return; }
                for (int i = 0; i < rank; ++i) {  // odometer step of the source coordinates
                    d += ostride[i];
                    if (++c[i] < dims[i]) break;
                    d -= c[i] * ostride[i];
                    c[i] = 0;
                }
            }
        });
    for (auto& x : th) x.join();
    return ok;
}

template <typename T>
int run(const std::vector<int64_t>& dims, const std::vector<int>& perm, int nb, double alpha) {
    const int rank = static_cast<int>(dims.size());
    int64_t vol = 1;
    for (auto d : dims) vol *= d;
    const size_t data_size = static_cast<size_t>(vol) * sizeof(T);
    const size_t gpu_size = static_cast<size_t>((1.0 + kPaddingSlack) * static_cast<double>(data_size));
    T* h = nullptr;
    void* d = nullptr;
    CLI_CHECK(cudaMallocHost(&h, data_size));
    CLI_CHECK(cudaMalloc(&d, gpu_size));
    init_iota(h, vol);

    long long perm_int = 0, pow10 = 1;
    for (int i = 0; i < rank; ++i, pow10 *= 10) perm_int += pow10 * perm[rank - i - 1];
    std::printf("%dD Inplace %lld transpose\n", rank, perm_int);
    std::printf("number of sub_tensors = %d\n", nb);
    std::printf("Dims =");
    for (auto x : dims) std::printf(" %lld", static_cast<long long>(x));
    std::printf(", Data size = %.5f GB\n", static_cast<double>(data_size) / 1e9);

    cudaEvent_t start, stop, h2d, trans, d2h;
    CLI_CHECK(cudaEventCreate(&start));
    CLI_CHECK(cudaEventCreate(&stop));
    CLI_CHECK(cudaEventCreate(&h2d));
    CLI_CHECK(cudaEventCreate(&trans));
    CLI_CHECK(cudaEventCreate(&d2h));
    CLI_CHECK(cudaEventRecord(start, 0));
    CLI_CHECK(cudaMemcpy(d, h, data_size, cudaMemcpyHostToDevice));
    CLI_CHECK(cudaEventRecord(h2d, 0));
    if (eithot_transpose_ex(d, gpu_size, rank, dims.data(), perm.data(), sizeof(T), nb, alpha, reorder_type(), nullptr, 0,
                            nullptr) != EITHOT_OK) {
        std::fprintf(stderr, "test_inplace: %s\n", eithot_last_error());
        return 1;
    }
    CLI_CHECK(cudaEventRecord(trans, 0));
    CLI_CHECK(cudaMemcpy(h, d, data_size, cudaMemcpyDeviceToHost));
    CLI_CHECK(cudaEventRecord(d2h, 0));
    CLI_CHECK(cudaDeviceSynchronize());
    CLI_CHECK(cudaEventRecord(stop, 0));
    CLI_CHECK(cudaEventSynchronize(stop));
    float t = 0, h2d_ms = 0, d2h_ms = 0;
    CLI_CHECK(cudaEventElapsedTime(&h2d_ms, start, h2d));
    CLI_CHECK(cudaEventElapsedTime(&d2h_ms, trans, d2h));
    CLI_CHECK(cudaEventElapsedTime(&t, start, stop));

    std::printf("Inplace transpose verify_inplace\n");
    unsigned faults = 0, timeouts = 0;
    eithot_index_faults(&faults);
    eithot_sync_timeouts(&timeouts);
    const bool ok = verify_inplace(h, dims, perm) && faults == 0 && timeouts == 0;
    std::printf(ok ? "Correct transpose\n" : "Incorrect transpose\n");

    const double throughput = static_cast<double>(data_size) * 2 / 1e6 / t;
    std::printf("Execution Time without h2d2h: %.5fms\n", t - h2d_ms - d2h_ms);
    std::printf("Execution Time: %.5fms\n", t);
    if (FILE* f = std::fopen("inplace_bench.txt", "a+")) {
        std::fprintf(f, "%.5f\n", t);
        std::fclose(f);
    }
    if (FILE* f = std::fopen("inplace_bench_throughput.txt", "a+")) {
        std::fprintf(f, "%.5f\n", throughput);
        std::fclose(f);
    }
    CLI_CHECK(cudaFreeHost(h));
    CLI_CHECK(cudaFree(d));
    return ok ? 0 : 3;
}

template <typename T>
int run_managed(const std::vector<int64_t>& dims, const std::vector<int>& perm, int nb, double alpha) {
    const int rank = static_cast<int>(dims.size());
    int64_t vol = 1;
    for (auto d : dims) vol *= d;
    const size_t gpu_size =
        static_cast<size_t>((1.0 + kPaddingSlack) * static_cast<double>(vol) * static_cast<double>(sizeof(T)));
    T* m = nullptr;
    CLI_CHECK(cudaMallocManaged(&m, std::max(gpu_size, sizeof(T))));
    init_iota(m, vol);

    long long perm_int = 0, pow10 = 1;
    for (int i = 0; i < rank; ++i, pow10 *= 10) perm_int += pow10 * perm[rank - i - 1];
    std::printf("%dD Inplace %lld transpose", rank, perm_int);
    std::printf(", Data size = %.5f GB\n", static_cast<double>(gpu_size) / 1e9);
    std::printf("number of sub_tensors = %d\n", nb);

    cudaEvent_t start, stop;
    CLI_CHECK(cudaEventCreate(&start));
    CLI_CHECK(cudaEventCreate(&stop));
    CLI_CHECK(cudaEventRecord(start, 0));
    if (eithot_transpose_ex(m, gpu_size, rank, dims.data(), perm.data(), sizeof(T), nb, alpha, reorder_type(), nullptr, 0,
                            nullptr) != EITHOT_OK) {
        std::fprintf(stderr, "test_inplace: %s\n", eithot_last_error());
        return 1;
    }
    CLI_CHECK(cudaDeviceSynchronize());
    CLI_CHECK(cudaEventRecord(stop, 0));
    CLI_CHECK(cudaEventSynchronize(stop));
    float t = 0;
    CLI_CHECK(cudaEventElapsedTime(&t, start, stop));

    std::printf("Inplace transpose verify_inplace\n");
    unsigned faults = 0, timeouts = 0;
    eithot_index_faults(&faults);
    eithot_sync_timeouts(&timeouts);
    const bool ok = verify_inplace(m, dims, perm) && faults == 0 && timeouts == 0;
    std::printf(ok ? "Correct transpose\n" : "Incorrect transpose\n");

    const double throughput = static_cast<double>(gpu_size) * 2 / 1e6 / t;
    std::printf("Execution Time: %.5fms\n", t);
    if (FILE* f = std::fopen("inplace_bench.txt", "a+")) {
        std::fprintf(f, "%.5f\n", t);
        std::fclose(f);
    }
    if (FILE* f = std::fopen("inplace_bench_throughput.txt", "a+")) {
        std::fprintf(f, "%.5f\n", throughput);
        std::fclose(f);
    }
    CLI_CHECK(cudaFree(m));
    return ok ? 0 : 3;
}

template <typename T>
int run_mode(bool managed, const std::vector<int64_t>& dims, const std::vector<int>& perm, int nb, double alpha) {
    return managed ? run_managed<T>(dims, perm, nb, alpha) : run<T>(dims, perm, nb, alpha);
}

}  // namespace

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
    const int nb = std::atoi(argv[k++]);
    const double alpha = std::atof(argv[k++]);
    if (argc == k + 1) {  // the reference opens (and truncates) the output file without writing it
        if (FILE* f = std::fopen(argv[k], "wb")) std::fclose(f);
    }
    for (int i = 0; i < rank; ++i)
        if (dims[i] < 1) { std::printf("Invalid rank or type size\n"); return 0; }
    const char* mt = std::getenv("EITHOT_MEMORY_TYPE");
    const bool managed = mt && std::atoi(mt) == 2;
    if (type_size == 4) return run_mode<int32_t>(managed, dims, perm, nb, alpha);
    if (type_size > 4) return run_mode<int64_t>(managed, dims, perm, nb, alpha);
    if (type_size == 2) return run_mode<uint16_t>(managed, dims, perm, nb, alpha);
    if (type_size == 1) return run_mode<uint8_t>(managed, dims, perm, nb, alpha);
    std::printf("Invalid rank or type size\n");
    return 0;
}
