// Permutation decomposition and N-d orchestration.
//
// The series follows EITHOT's method (ITNT/src/permutation_util.cpp:99-374,
// ITNT/src/Nd_transpose.cpp:104-304): each round fixes the first (pre-order)
// or last (post-order) position whose axis differs from the target by moving
// one contiguous block of axes there, and the round is executed as a single
// low-order transpose in which every group of axes that stays together is
// fused into one dimension.  Restated here in 64-bit arithmetic (the
// reference uses int and overflows past 2^31 elements).
#include "plan.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace eithot {

int LowOp::code() const {
    int c = 0;
    for (int i = 0; i < rank; ++i) c = c * 10 + perm[i];
    return c;
}

namespace {

int64_t prod(const std::vector<int64_t>& v, int lo, int hi) {  // [lo, hi)
    int64_t p = 1;
    for (int i = lo; i < hi; ++i) p *= v[i];
    return p;
}

// Builds the low-order op from groups listed in memory (source) order and the
// order in which those groups appear in the output.
LowOp make_op(const std::vector<int64_t>& group_dims, const std::vector<int>& out_order) {
    LowOp op;
    op.rank = static_cast<int>(group_dims.size());
    for (int g = 0; g < op.rank; ++g) {
        op.dims[g] = group_dims[g];
        op.perm[g] = out_order[g] + 1;
    }
    return op;
}

}  // namespace

// Pre-order round (permutation_util.cpp:300-337 with :99-110, :125-132,
// :146-180, :232-243, :16-97).  With u the first mismatched position and the
// wanted axis found at s > u, the run of L axes starting at s that already
// appears in target order at u is moved to u.  Groups in memory order:
// P = [0,u) (fused, omitted if u == 0), X = [u,s), Y = [s,s+L), Z = [s+L,r)
// (omitted if empty); output order P, Y, X, Z.
// Post-order round (:339-374 with :112-123, :134-143, :183-230, :245-255):
// with u the last mismatched position and the wanted axis at s < u, the run
// of L axes ending at s that matches the target ending at u moves to end at
// u.  Groups: W = [0,s-L+1), Y = [s-L+1,s+1), X = [s+1,u+1), T = [u+1,r)
// (T fused); output order W, X, Y, T.
bool plan_round(const std::vector<int>& cur, const std::vector<int64_t>& dims,
                const std::vector<int>& target, bool pre, Round* out) {
    const int r = static_cast<int>(cur.size());
    // dims in the current arrangement
    std::vector<int64_t> d(r);
    for (int p = 0; p < r; ++p) d[p] = dims[cur[p] - 1];

    int u = -1;
    if (pre) {
        for (int p = 0; p < r; ++p) if (cur[p] != target[p]) { u = p; break; }
    } else {
        for (int p = r - 1; p >= 0; --p) if (cur[p] != target[p]) { u = p; break; }
    }
    if (u < 0) return false;
    const int s = static_cast<int>(std::find(cur.begin(), cur.end(), target[u]) - cur.begin());

    std::vector<int64_t> gdims;
    std::vector<int> order;  // output order as indices into gdims
    std::vector<int> next;
    next.reserve(r);
    if (pre) {
        int L = 1;
        while (u + L < r && s + L < r && target[u + L] == cur[s + L]) ++L;
        // next = cur[0,u) ++ cur[s,s+L) ++ cur[u,s) ++ cur[s+L,r)
        next.insert(next.end(), cur.begin(), cur.begin() + u);
        next.insert(next.end(), cur.begin() + s, cur.begin() + s + L);
        next.insert(next.end(), cur.begin() + u, cur.begin() + s);
        next.insert(next.end(), cur.begin() + s + L, cur.end());
        const bool hasP = u > 0, hasZ = s + L < r;
        int iP = -1, iX, iY, iZ = -1;
        if (hasP) { iP = 0; gdims.push_back(prod(d, 0, u)); }
        iX = static_cast<int>(gdims.size()); gdims.push_back(prod(d, u, s));
        iY = static_cast<int>(gdims.size()); gdims.push_back(prod(d, s, s + L));
        if (hasZ) { iZ = static_cast<int>(gdims.size()); gdims.push_back(prod(d, s + L, r)); }
        if (hasP) order.push_back(iP);
        order.push_back(iY);
        order.push_back(iX);
        if (hasZ) order.push_back(iZ);
    } else {
        int L = 1;
        while (u - L >= 0 && s - L >= 0 && target[u - L] == cur[s - L]) ++L;
        const int y0 = s - L + 1;
        // next = cur[0,y0) ++ cur[s+1,u+1) ++ cur[y0,s+1) ++ cur[u+1,r)
        next.insert(next.end(), cur.begin(), cur.begin() + y0);
        next.insert(next.end(), cur.begin() + s + 1, cur.begin() + u + 1);
        next.insert(next.end(), cur.begin() + y0, cur.begin() + s + 1);
        next.insert(next.end(), cur.begin() + u + 1, cur.end());
        const bool hasW = y0 > 0, hasT = u + 1 < r;
        int iW = -1, iX, iY, iT = -1;
        if (hasW) { iW = 0; gdims.push_back(prod(d, 0, y0)); }
        iY = static_cast<int>(gdims.size()); gdims.push_back(prod(d, y0, s + 1));
        iX = static_cast<int>(gdims.size()); gdims.push_back(prod(d, s + 1, u + 1));
        if (hasT) { iT = static_cast<int>(gdims.size()); gdims.push_back(prod(d, u + 1, r)); }
        if (hasW) order.push_back(iW);
        order.push_back(iX);
        order.push_back(iY);
        if (hasT) order.push_back(iT);
    }
    // perm[g] (1-based) = which memory-order group lands at output position g
    out->op = make_op(gdims, order);
    out->next = std::move(next);
    return true;
}

// Linearization_condition (ITNT/src/Nd_transpose.cpp:104-113): 213 with
// d3 >= 8, 132 with d1 >= 48, 1324 with d4 >= 4 or d1 >= 96 are single-pass.
int non_linearized(const LowOp& op) {
    if (op.rank == 3) {
        if (op.perm[2] == 3 && op.dims[2] >= 8) return 0;
        if (op.perm[0] == 1 && op.dims[0] >= 48) return 0;
    } else if (op.rank == 4) {
        if (op.perm[3] == 4 && op.dims[3] >= 4) return 0;
        if (op.perm[0] == 1 && op.dims[0] >= 96) return 0;
    }
    return 1;
}

namespace {

void run_series(const std::vector<int64_t>& dims, const std::vector<int>& target,
                bool pre, std::vector<LowOp>* ops) {
    const int r = static_cast<int>(dims.size());
    std::vector<int> cur(r);
    std::iota(cur.begin(), cur.end(), 1);
    // At most r rounds, as the reference's loop bound (Nd_transpose.cpp:192).
    for (int round = 0; round < r; ++round) {
        Round rd;
        if (!plan_round(cur, dims, target, pre, &rd)) break;
        ops->push_back(rd.op);
        cur = rd.next;
        if (cur == target) break;
    }
}

}  // namespace

// method_selection (ITNT/src/Nd_transpose.cpp:115-157): count rounds that
// are not linearisations under each order; pre-order only if strictly fewer.
int plan_series(const std::vector<int64_t>& dims, const std::vector<int>& target,
                int order_in, std::vector<LowOp>* ops) {
    int order = order_in;
    if (order == kOrderMixed) {
        std::vector<LowOp> a, b;
        run_series(dims, target, true, &a);
        run_series(dims, target, false, &b);
        int na = 0, nb = 0;
        for (auto& o : a) na += non_linearized(o);
        for (auto& o : b) nb += non_linearized(o);
        order = (na < nb) ? kOrderPre : kOrderPost;
    }
    run_series(dims, target, order == kOrderPre, ops);
    return order;
}

bool make_nd_plan(int rank, const int64_t* dims_in, const int* perm_1based,
                  int nb, double alpha, int order, NdPlan* plan, std::string* err) {
    if (rank < 1 || rank > 32) { *err = "rank must be in [1, 32]"; return false; }
    if (!dims_in || !perm_1based) { *err = "null dims or permutation"; return false; }
    if (order < kOrderMixed || order > kOrderFewest) { *err = "reorder_type must be 0, 1, 2 or 3"; return false; }
    if (order == kOrderFewest) order = kOrderMixed;  // the plan's own steps follow the reference's series
    if (!(alpha > 0.0) || !std::isfinite(alpha)) { *err = "alpha must be a positive finite ratio"; return false; }
    if (nb < 1) { *err = "num_sub_tensors must be >= 1"; return false; }
    std::vector<int64_t> dims(dims_in, dims_in + rank);
    std::vector<int> perm(perm_1based, perm_1based + rank);
    {
        std::vector<int> seen(rank + 1, 0);
        for (int i = 0; i < rank; ++i) {
            if (dims[i] < 1) { *err = "every dim must be >= 1"; return false; }
            if (perm[i] < 1 || perm[i] > rank || seen[perm[i]]++) {
                *err = "permutation must be a 1-based permutation of 1..rank";
                return false;
            }
        }
    }
    long double vol_ld = 1.0L;
    for (auto v : dims) vol_ld *= static_cast<long double>(v);
    if (vol_ld > 9.0e18L) { *err = "tensor volume exceeds 2^63 elements"; return false; }

    *plan = NdPlan();
    plan->rank = rank;
    plan->dims = dims;
    plan->perm = perm;
    int64_t vol = 1;
    for (auto v : dims) vol *= v;
    plan->volume = vol;
    plan->padded_volume = vol;

    // Sub-tensor gate (Nd_transpose.cpp:265-275): the first largest dim is
    // decomposed when it exceeds int(32 * (1/alpha)) and nb > 1.
    const int64_t large = static_cast<int64_t>(32.0 * (1.0 / alpha));
    const int maxpos = static_cast<int>(std::max_element(dims.begin(), dims.end()) - dims.begin());
    std::vector<int64_t> work = dims;  // dims of the (possibly padded) tensor
    if (dims[maxpos] > large && nb > 1) {
        plan->decompose_pos = maxpos;
        if (dims[maxpos] % nb != 0) {
            plan->padded = true;
            plan->padded_dim = (dims[maxpos] / nb + 1) * nb;
        }
    } else {
        nb = 1;
    }
    plan->nb = nb;

    if (plan->padded) {
        NdStep st;
        st.role = kPadPre;
        st.pad_pos = maxpos;
        st.pad_orig = dims[maxpos];
        st.pad_size = plan->padded_dim;
        st.pad_layout = dims;
        plan->steps.push_back(st);
        work[maxpos] = plan->padded_dim;
        plan->padded_volume = vol / dims[maxpos] * plan->padded_dim;
    }
    const int64_t pvol = plan->padded_volume;

    if (plan->decompose_pos >= 0) {
        // NdPartition (Nd_decompose.cpp:17-25, :49-56): 132 on (ds/nb, nb, nds)
        const int p = plan->decompose_pos;
        int64_t ds = 1, nds = 1;
        for (int i = 0; i <= p; ++i) ds *= work[i];
        for (int i = p + 1; i < rank; ++i) nds *= work[i];
        NdStep st;
        st.role = kPartition;
        st.op.rank = 3;
        st.op.dims[0] = ds / nb; st.op.dims[1] = nb; st.op.dims[2] = nds;
        st.op.perm[0] = 1; st.op.perm[1] = 3; st.op.perm[2] = 2;
        plan->steps.push_back(st);
    }

    std::vector<int64_t> sub = work;
    if (plan->decompose_pos >= 0) sub[plan->decompose_pos] /= nb;
    plan->sub_volume = pvol / nb;

    std::vector<LowOp> ops;
    plan->order_used = plan_series(sub, perm, order, &ops);
    for (auto& o : ops) {
        NdStep st;
        st.role = kRound;
        st.op = o;
        plan->steps.push_back(st);
    }

    if (plan->decompose_pos >= 0) {
        // NdJoin (Nd_decompose.cpp:33-41, :66-82): 132 on (ds/nb, nds, nb)
        // over the permuted (padded) dims.
        const int p = plan->decompose_pos;
        int q = -1;
        std::vector<int64_t> pd(rank);
        for (int i = 0; i < rank; ++i) {
            pd[i] = work[perm[i] - 1];
            if (perm[i] - 1 == p) q = i;
        }
        int64_t ds = 1, nds = 1;
        for (int i = 0; i <= q; ++i) ds *= pd[i];
        for (int i = q + 1; i < rank; ++i) nds *= pd[i];
        NdStep st;
        st.role = kJoin;
        st.op.rank = 3;
        st.op.dims[0] = ds / nb; st.op.dims[1] = nds; st.op.dims[2] = nb;
        st.op.perm[0] = 1; st.op.perm[1] = 3; st.op.perm[2] = 2;
        plan->steps.push_back(st);
    }

    if (plan->padded) {
        // Nd_padding_post_process (Nd_padding.cu:169-223): compact the
        // padded dim in the permuted layout.
        NdStep st;
        st.role = kPadPost;
        std::vector<int64_t> pd(rank);
        int q = -1;
        for (int i = 0; i < rank; ++i) {
            pd[i] = dims[perm[i] - 1];
            if (perm[i] - 1 == maxpos) q = i;
        }
        st.pad_pos = q;
        st.pad_orig = dims[maxpos];
        st.pad_size = plan->padded_dim;
        st.pad_layout = pd;
        plan->steps.push_back(st);
    }
    return true;
}

}  // namespace eithot
