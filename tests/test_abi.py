"""The C ABI library loads and exports every entry point include/eithot.h
declares; host-only entry points work without a GPU."""
import ctypes
import os
import re
import subprocess

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "eithot.h")).read()
    c_part = text.split('#ifdef __cplusplus\n}')[0]
    return sorted(set(re.findall(r"\b(eithot_[a-z_]+)\s*\(", c_part)))


def test_exports(E):
    syms = declared_symbols()
    assert len(syms) >= 8
    lib = ctypes.CDLL(E.LIB_PATH)
    for s in syms:
        assert hasattr(lib, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", E.LIB_PATH], capture_output=True, text=True).stdout
    # the reference-signature C++ shim inplace::transpose(void*, int, int, void*, void*, size_t, int, double)
    assert "_ZN7inplace9transposeEPviiS0_S0_mid" in out


def test_errors_do_not_exit(E):
    import pytest
    with pytest.raises(E.EithotError) as ei:
        E.workspace_size([4, 4], [1, 1], 4)
    assert ei.value.code == E.EINVAL
    assert "permutation" in E.lib.eithot_last_error().decode()
    with pytest.raises(E.EithotError):
        E.workspace_size([4, 4], [2, 1], 0)


def test_workspace_sizes_host_only(E):
    # on-chip passes need at most the group barrier's counters
    assert E.workspace_size([3001, 4096], [2, 1], 4) <= 4096
    ws = E.workspace_size([4, 20011, 8192, 2], [1, 3, 2, 4], 4)
    assert 0 <= ws <= 0.0101 * 4 * 20011 * 8192 * 8


def test_invalid_requests_are_refused(E):
    import pytest
    cases = [([0, 5], [2, 1], 4), ([4, 5], [1, 1], 4), ([4, 5], [2, 3], 4), ([4, 5], [2, 1], 0),
             ([4, 5], [2, 1], 65), ([4, 5, 6], [2, 1], 4)]
    for dims, perm, elem in cases:
        with pytest.raises(E.EithotError) as ei:
            E.workspace_size(dims, perm, elem)
        assert ei.value.code == E.EINVAL, (dims, perm, elem)
        assert E.lib.eithot_last_error()
