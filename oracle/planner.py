"""ORACLE — test infrastructure only (never imported by the product).

CPU restatement of EITHOT's permutation planner and N-d orchestration:

* one round: ITNT/src/permutation_util.cpp:300-337 (pre-order) and
  :339-374 (post-order), built from find_unmatched_index_* (:99-123),
  merge_matched_dim_* (:125-143), *_round_trans_perm_generation (:146-230),
  merge_matched_perm_* (:232-255), merge_seq_perm_in_dim (:40-79),
  merge_seq_perm (:81-97) and rerank_permutation (:16-38);
* the series and mixed-order selection: ITNT/src/Nd_transpose.cpp:104-250;
* the N-d orchestration (sub-tensor gate, padding, partition, join):
  ITNT/src/Nd_transpose.cpp:256-304 and ITNT/src/Nd_decompose.cpp:17-82.

This follows the reference procedure step by step (round permutation as an
explicit array, then run merging), unlike the product's planner which
derives the same result from the moved block directly.  Python ints do not
overflow, so results differ from the reference only where its 32-bit `int`
arithmetic wraps.  Pinned against the reference's own code compiled here
(oracle/_ref/ref_plan) by tests/golden/make_golden.py.
"""
from __future__ import annotations

PRE, POST = 1, 2


def _rerank(vals):
    order = sorted(set(vals))
    rank = {v: i + 1 for i, v in enumerate(order)}
    return [rank[v] for v in vals]


def _runs(perm):
    """Split a 1-based permutation into maximal runs of consecutive values."""
    runs, start = [], 0
    for x in range(1, len(perm) + 1):
        if x == len(perm) or perm[x] != perm[x - 1] + 1:
            runs.append(perm[start:x])
            start = x
    return runs


def _merge_runs(mdims, mperm):
    """merge_seq_perm_in_dim + merge_seq_perm: fuse dims of each run
    (runs are ranges of source positions) and rerank the run heads."""
    runs = _runs(mperm)
    acc = [0] * len(mperm)
    for run in runs:
        acc[run[0] - 1] = len(run) - 1
    low_dims, i = [], 0
    while i < len(mdims):
        d = 1
        for k in range(acc[i] + 1):
            d *= mdims[i + k]
        low_dims.append(d)
        i += acc[i] + 1
    low_perm = _rerank([run[0] for run in runs])
    return low_dims, low_perm


def round_pre(cur, dims, target):
    r = len(cur)
    u = next((p for p in range(r) if cur[p] != target[p]), r)
    if u == r:
        return None
    reordered = [dims[a - 1] for a in cur]
    if u != 0:
        pre = 1
        for i in range(u):
            pre *= reordered[i]
        mdims = [pre] + reordered[u:]
    else:
        mdims = list(reordered)
    # round permutation: new position -> 1-based source position
    s = cur.index(target[u])
    L = 1
    while u + L < r and s + L < r and target[u + L] == cur[s + L]:
        L += 1
    rp = [0] * r
    for x in range(L):
        rp[u + x] = s + x + 1
    block = set(range(s + 1, s + L + 1))
    for val in range(1, r + 1):
        if val in block:
            continue
        rp[rp.index(0)] = val
    if u != 0:
        mperm = [1] + [v - (u - 1) for v in rp[u:]]
    else:
        mperm = list(rp)
    low_dims, low_perm = _merge_runs(mdims, mperm)
    nxt = [cur[rp[i] - 1] for i in range(r)]
    return low_dims, low_perm, nxt


def round_post(cur, dims, target):
    r = len(cur)
    u = next((p for p in range(r - 1, -1, -1) if cur[p] != target[p]), 0)
    if u == 0:
        return None
    reordered = [dims[a - 1] for a in cur]
    if u < r - 2:
        tail = 1
        for i in range(u + 1, r):
            tail *= reordered[i]
        mdims = reordered[:u + 1] + [tail]
    else:
        mdims = list(reordered)
    s = cur.index(target[u])
    L = 1
    while u - L >= 0 and s - L >= 0 and target[u - L] == cur[s - L]:
        L += 1
    rp = [0] * r
    for x in range(L):
        rp[u - L + 1 + x] = s - L + 2 + x
    block = set(range(s - L + 2, s + 2))
    for val in range(r, 0, -1):
        if val in block:
            continue
        pos = max(i for i in range(r) if rp[i] == 0)
        rp[pos] = val
    if u < r - 2:
        mperm = rp[:u + 1] + [u + 2]
    else:
        mperm = list(rp)
    low_dims, low_perm = _merge_runs(mdims, mperm)
    nxt = [cur[rp[i] - 1] for i in range(r)]
    return low_dims, low_perm, nxt


def non_linearized(low_dims, low_perm):
    k = len(low_perm)
    if k == 3:
        if low_perm[2] == 3 and low_dims[2] >= 8:
            return 0
        if low_perm[0] == 1 and low_dims[0] >= 48:
            return 0
    elif k == 4:
        if low_perm[3] == 4 and low_dims[3] >= 4:
            return 0
        if low_perm[0] == 1 and low_dims[0] >= 96:
            return 0
    return 1


def series(dims, target, order):
    r = len(dims)
    fn = round_pre if order == PRE else round_post
    cur = list(range(1, r + 1))
    ops = []
    for _ in range(r):
        res = fn(cur, dims, target)
        if res is None:
            break
        low_dims, low_perm, cur = res
        ops.append((low_dims, low_perm))
        if cur == list(target):
            break
    return ops


def choose_order(dims, target, reorder_type=0):
    if reorder_type in (PRE, POST):
        return reorder_type
    pre = sum(non_linearized(d, p) for d, p in series(dims, target, PRE))
    post = sum(non_linearized(d, p) for d, p in series(dims, target, POST))
    return PRE if pre < post else POST


def code(perm):
    c = 0
    for v in perm:
        c = c * 10 + v
    return c


def nd_plan(dims, perm1, nb, alpha, reorder_type=0):
    """Steps in the order the reference issues them, one series per
    sub-tensor: list of (tag, source_offset_elems, dims-or-args)."""
    dims = list(dims)
    perm1 = list(perm1)
    r = len(dims)
    vol = 1
    for d in dims:
        vol *= d
    large = int(32 * (1.0 / alpha))
    maxpos = dims.index(max(dims))
    steps = []
    work = list(dims)
    padded = False
    if dims[maxpos] > large and nb > 1:
        decomp = maxpos
        if dims[maxpos] % nb != 0:
            padded = True
            padsize = (dims[maxpos] // nb + 1) * nb
    else:
        nb = 1
        decomp = -1
    if padded:
        steps.append(("PADPRE", 0, [maxpos, dims[maxpos], nb] + list(dims)))
        work[maxpos] = padsize
        vol = vol // dims[maxpos] * padsize
    if decomp >= 0:
        ds = 1
        for i in range(decomp + 1):
            ds *= work[i]
        nds = vol // ds
        steps.append(("132", 0, [ds // nb, nb, nds]))
        sub = list(work)
        sub[decomp] //= nb
    else:
        sub = list(work)
    order = choose_order(sub, perm1, reorder_type)
    ops = series(sub, perm1, order)
    sub_vol = vol // nb
    for i in range(nb):
        for low_dims, low_perm in ops:
            steps.append((str(code(low_perm)), i * sub_vol, list(low_dims)))
    if decomp >= 0:
        pd = [work[p - 1] for p in perm1]
        q = [p - 1 for p in perm1].index(decomp)
        ds = 1
        for i in range(q + 1):
            ds *= pd[i]
        nds = vol // ds
        steps.append(("132", 0, [ds // nb, nds, nb]))
    if padded:
        steps.append(("PADPOST", 0, [maxpos, dims[maxpos], nb] + [p - 1 for p in perm1]))
    return steps, order
