"""ORACLE — test infrastructure only (never imported by the product).

CPU restatement of EITHOT's extra-memory estimator (Nd_estimation):

* driver: Nd_memory_estimation/src/test_inplace.cpp:19-147;
* per-round temp sizes: the size-only mirrors of the kernels' launchers,
  Nd_memory_estimation/src/col_op.cu:16-176 and row_op.cu:14-173, and the
  low-order drivers 2dtranspose.cpp:21-102, 3dtranspose.cpp (213 / 132 /
  231 / 312), 4dtranspose.cpp (1324);
* partition / join temps: Nd_decompose.cpp (132 on (ds/nb, nb, nds) and
  (ds/nb, nds, nb) of the unpadded dims);
* padding temp: Nd_padding.cu:96-104, sizeof(T) * resident_blocks * 1024.

The cost model is the reference's (48 KiB default shared memory per block
on every GPU it ran on, including GB300); `smem` and `pad_blocks` are
parameters.  Pinned against the README screenshot values (tests/golden/
estimator_readme.json) and the reference estimator compiled here
(oracle/_ref/Nd_estimation) by tests/golden/make_golden.py.
"""
from __future__ import annotations

import math

from . import planner

WARP = 32


def _msb(x):
    return int(math.log2(x))


def _gcd(a, b):
    return math.gcd(a, b)


class _Cost:
    def __init__(self, st, smem):
        self.st = st
        self.smem = smem

    # --- launch-level sizes -------------------------------------------
    def col2d(self, d1, d2, rotate):  # _2d::col_op, also _3d::_213::col_op
        if self.smem // (self.st * d2) >= 16:
            return 0
        nt = 256 if rotate or _msb(d1) > 18 else 32
        return self.st * nt * d2

    def row2d(self, d1):  # _2d / _3d::_213 row_gather_op / row_scatter_op
        if 2 * d1 * self.st <= self.smem // 32:
            return 0
        if self.st * d1 <= self.smem:
            return 0
        return self.st * d1

    def col132(self, d1, d2, rotate):  # _3d::_132::col_op
        st, smem = self.st, self.smem
        if 2 * st * d1 * d2 <= smem // 32:
            return 0
        if st * d1 * d2 <= smem:
            return 0
        if smem // (st * d2) >= 16:
            return 0
        nt = 256 if rotate or _msb(d1) > 18 else 32
        return st * nt * d2

    def row132(self, d1, d3):  # _3d::_132 row ops
        return 0 if self.st * d1 * d3 <= self.smem else self.st * d1 * d3

    # --- Catanzaro ------------------------------------------------------
    def c2r_2d(self, d1, d2):
        c = _gcd(d2, d1)
        t = self.col2d(d1, d2, True) if c > 1 else 0
        return max(t, self.row2d(d1), self.col2d(d1, d2, False))

    def r2c_2d(self, d1, d2):
        c = _gcd(d1, d2)
        t = max(self.col2d(d1, d2, False), self.row2d(d1))
        if c > 1:
            t = max(t, self.col2d(d1, d2, True))
        return t

    def t2d(self, d1, d2):
        return self.c2r_2d(d1, d2) if d1 >= d2 else self.r2c_2d(d2, d1)

    def c2r_213(self, d1, d2, d3):
        c = _gcd(d2, d1)
        t = self.col2d(d1, d2, True) if c > 1 else 0
        return max(t, self.row2d(d1), self.col2d(d1, d2, False))

    def r2c_213(self, d1, d2, d3):
        c = _gcd(d1, d2)
        t = max(self.col2d(d1, d2, False), self.row2d(d1))
        if c > 1:
            t = max(t, self.col2d(d1, d2, True))
        return t

    def c2r_132(self, d1, d2, d3):
        c = _gcd(d2, d3)
        t = self.col132(d1, d2, True) if c > 1 else 0
        return max(t, self.row132(d1, d3), self.col132(d1, d2, False))

    def r2c_132(self, d1, d2, d3):
        c = _gcd(d3, d2)
        t = max(self.col132(d1, d2, False), self.row132(d1, d3))
        if c > 1:
            t = max(t, self.col132(d1, d2, True))
        return t

    # --- low-order ops -------------------------------------------------
    def t213(self, d1, d2, d3):
        if d3 >= 8:
            return self.row2d(d1 * d2)
        return self.c2r_213(d1, d2, d3) if d1 > d2 else self.r2c_213(d2, d1, d3)

    def t132(self, d1, d2, d3):
        if d1 >= 48:
            return self.col2d(d1, d2 * d3, False)
        if d1 > 12:
            return self.c2r_132(d1, d3, d2) if d2 > d3 else self.r2c_132(d1, d2, d3)
        if d2 >= d3:
            return max(self.t2d(d1 * d2, d3), self.row2d(d3 * d1))
        return max(self.row2d(d1 * d2), self.t2d(d2, d1 * d3))

    def t1324(self, d1, d2, d3, d4):
        if d1 >= 96:
            return self.col2d(d1, d2 * d3 * d4, False)
        if d4 >= 4:
            return self.row2d(d1 * d2 * d3)
        if d2 >= d3:
            return max(self.t213(d1 * d2, d3, d4), self.t213(d3, d1, d2 * d4))
        return max(self.row2d(d1 * d2), self.t2d(d2, d1 * d3 * d4),
                   self.col2d(d1 * d3, d4 * d2, False))

    def low(self, dims, perm):
        c = planner.code(perm)
        if c == 21:
            return self.t2d(dims[0], dims[1])
        if c == 231:
            return self.t2d(dims[0], dims[1] * dims[2])
        if c == 312:
            return self.t2d(dims[0] * dims[1], dims[2])
        if c == 213:
            return self.t213(*dims)
        if c == 132:
            return self.t132(*dims)
        if c == 1324:
            return self.t1324(*dims)
        raise ValueError("unsupported low-order permutation %d" % c)

    def series(self, dims, perm1):
        order = planner.choose_order(dims, perm1)
        return max([0] + [self.low(d, p) for d, p in planner.series(dims, perm1, order)])


def estimate(dims, perm1, type_size, nb_in, alpha, smem=49152, pad_blocks=304):
    """Returns dict(nb, alpha, alpha_str, init_tmp, final_tmp) as the
    reference estimator would print/write them."""
    dims = list(dims)
    perm1 = list(perm1)
    st = 4 if type_size == 4 else 8
    cost = _Cost(st, smem)
    vol = math.prod(dims)
    data_size = vol * st
    rank = len(dims)
    maxpos = dims.index(max(dims))
    transpose_tmp = cost.series(dims, perm1)
    init_tmp = transpose_tmp
    percent = int(transpose_tmp / data_size / alpha)
    nb = 1 if percent == 0 else int(2 ** math.ceil(math.log2(percent)))
    if nb == 0:
        nb = 1
    if transpose_tmp > 0:
        alpha = max(alpha, 1 / math.sqrt(vol / WARP))
    large = int(WARP / alpha)
    if not (dims[maxpos] > large and nb > 1):
        alpha = math.ceil(alpha * 100.0) / 100.0
        return dict(nb=nb, alpha=alpha, alpha_str="%.2f" % alpha, init_tmp=init_tmp,
                    final_tmp=None)
    padding = dims[maxpos] % nb != 0
    padding_tmp = 0
    if padding:
        padding_dim = (dims[maxpos] // nb + 1) * nb
        padding_tmp = vol // dims[maxpos] * (padding_dim - dims[maxpos]) * st
    transpose_tmp //= nb
    if padding:
        padding_tmp = max(padding_tmp, st * pad_blocks * 1024)
    ds = math.prod(dims[:maxpos + 1])
    nds = vol // ds
    decompose_tmp = cost.t132(ds // nb, nb, nds)
    pd = [dims[p - 1] for p in perm1]
    q = [p - 1 for p in perm1].index(maxpos)
    ds2 = math.prod(pd[:q + 1])
    nds2 = vol // ds2
    decompose_tmp = max(decompose_tmp, cost.t132(ds2 // nb, nds2, nb))
    final_tmp = padding_tmp + max(decompose_tmp, transpose_tmp)
    mem_ratio = final_tmp / data_size
    if mem_ratio > alpha:
        new_final = final_tmp
        new_nb = nb
        while final_tmp >= new_final and nb > 1:
            nb = new_nb
            final_tmp = new_final
            new_nb //= 2
            if new_nb == 0:
                # the reference divides by zero here (SIGFPE) on its way out
                # of the loop; nb and final_tmp are already final
                break
            padding_dim = (dims[maxpos] // new_nb + 1) * new_nb
            padding_tmp = vol // dims[maxpos] * (padding_dim - dims[maxpos]) * st
            transpose_tmp *= 2
            decompose_tmp //= 2
            new_final = padding_tmp + max(decompose_tmp, transpose_tmp)
        mem_ratio = final_tmp / data_size
        mem_ratio = math.ceil(mem_ratio * 100.0) / 100.0
        alpha = max(mem_ratio, alpha)
    return dict(nb=nb, alpha=alpha, alpha_str="%.2f" % alpha, init_tmp=init_tmp,
                final_tmp=final_tmp)
