#pragma once

#include <cstdint>
#include <vector>

namespace eithot {

struct Estimate {
    int nb = 1;
    double alpha = 0.0;
    uint64_t init_tmp = 0;   // max temp over the rounds of the undivided tensor
    uint64_t final_tmp = 0;  // modelled extra bytes for the chosen nb
    bool decomposed = false;
    double alpha_raised = 0.0;  // alpha after the 1/sqrt(vol/32) floor (printed as "new ratio")
    double ratio = 0.0;         // final_tmp / bytes as printed (rounded up to 0.01 when nb was searched)
};

// perm is 1-based.  smem_per_block: the reference's default shared memory per
// block (48 KiB on every CUDA GPU since Kepler); pad_blocks: resident
// 1024-thread blocks of the whole GPU (the padding kernels' grid).
bool estimate(const std::vector<int64_t>& dims, const std::vector<int>& perm, uint64_t elem_size,
              double alpha, uint64_t smem_per_block, uint64_t pad_blocks, Estimate* out);

}  // namespace eithot
