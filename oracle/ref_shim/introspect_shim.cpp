// Test infrastructure (oracle side): stands in for the reference's
// introspect.cpp so its estimator can run on a machine without a GPU.  The
// device properties the reference reads (Nd_memory_estimation/src/
// introspect.cpp:7-26) are taken from the environment, defaulting to a
// GB300's values: 48 KiB default shared memory per block, 152 SMs, 2048
// threads per SM.
#include <cstdlib>
#include <cstddef>

static long env_or(const char* name, long dflt) {
    const char* v = std::getenv(name);
    return v ? std::atol(v) : dflt;
}
int n_sms() { return static_cast<int>(env_or("EITHOT_REF_SMS", 152)); }
size_t gpu_memory_size() { return static_cast<size_t>(env_or("EITHOT_REF_GMEM", 298023223296L)); }
size_t shared_mem_per_block() { return static_cast<size_t>(env_or("EITHOT_REF_SMEM", 49152)); }
int max_n_threads_per_sm() { return static_cast<int>(env_or("EITHOT_REF_THREADS_PER_SM", 2048)); }
int current_sm() { return static_cast<int>(env_or("EITHOT_REF_CC", 1003)); }
