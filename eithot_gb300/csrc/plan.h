// Host-side planning: permutation decomposition (pre/post/mixed ordering),
// the N-d orchestration (padding, partition, per-sub-tensor series, join,
// unpadding) and its lowering to device passes.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace eithot {

// kOrderFewest: the reference's mixed series for the plan's steps, and the
// executor may replace its passes with a pass-minimising search's.
enum Order { kOrderMixed = 0, kOrderPre = 1, kOrderPost = 2, kOrderFewest = 3 };

// A low-order transpose: rank 2..4 tensor, 1-based permutation.
struct LowOp {
    int rank = 0;
    int64_t dims[4] = {0, 0, 0, 0};
    int perm[4] = {0, 0, 0, 0};
    int code() const;  // decimal encoding, e.g. {1,3,2,4} -> 1324
};

// One round of the series: the low-order op it performs and the arrangement
// of original axes after it.
struct Round {
    LowOp op;
    std::vector<int> next;  // next[p] = original axis (1-based) at position p
};

// Computes one pre-order (pre=true) or post-order round.  Returns false when
// the arrangement `cur` already equals `target` (the reference signals this
// by returning rank+1).
bool plan_round(const std::vector<int>& cur, const std::vector<int64_t>& dims,
                const std::vector<int>& target, bool pre, Round* out);

// 1 if the low-order op is NOT one of the reference's single-pass
// "linearisations" (ITNT/src/Nd_transpose.cpp:104-113).
int non_linearized(const LowOp& op);

// Full series for one tensor.  order_in: kOrderMixed/Pre/Post.  Returns the
// order actually used (kOrderPre or kOrderPost).
int plan_series(const std::vector<int64_t>& dims, const std::vector<int>& target,
                int order_in, std::vector<LowOp>* ops);

enum StepRole { kRound = 0, kPartition = 1, kJoin = 2, kPadPre = 3, kPadPost = 4 };

struct NdStep {
    int role = kRound;
    LowOp op;              // ROUND / PARTITION / JOIN
    // PAD steps: position of the padded dim (in the layout the step sees),
    // original and padded extents, and the layout dims it sees.
    int pad_pos = -1;
    int64_t pad_orig = 0, pad_size = 0;
    std::vector<int64_t> pad_layout;  // dims of the (unpadded) layout
};

struct NdPlan {
    int rank = 0;
    std::vector<int64_t> dims;
    std::vector<int> perm;   // 1-based target
    int order_used = kOrderPost;
    int nb = 1;
    int decompose_pos = -1;
    bool padded = false;
    int64_t padded_dim = 0;
    int64_t volume = 0, padded_volume = 0, sub_volume = 0;
    std::vector<NdStep> steps;
};

// Validates inputs and builds the N-d plan.  On failure returns false and
// sets *err.
bool make_nd_plan(int rank, const int64_t* dims, const int* perm_1based,
                  int nb, double alpha, int order, NdPlan* plan, std::string* err);

}  // namespace eithot
