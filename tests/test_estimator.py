"""The product estimator (C ABI eithot_estimate) against the reference's
known answers and the reference estimator binary."""
import json
import os

from conftest import GOLDEN


def test_readme_known_answers(E):
    doc = json.load(open(os.path.join(GOLDEN, "estimator_readme.json")))
    for c in doc["cases"]:
        nb, alpha, extra = E.estimate(c["dims"], c["perm"], c["elem"], c["nb"], c["alpha"], 49152, 82)
        assert nb == c["nb_out"] and "%.2f" % alpha == c["alpha_out"], (c, nb, alpha)
    nb, alpha, extra = E.estimate([7248, 7248], [2, 1], 4, 1, 0.01, 49152, 82)
    assert "%.5f" % (extra / 1e6) == doc["final_extra_mb"]["1"]


def test_reference_binary_cases(E):
    doc = json.load(open(os.path.join(GOLDEN, "estimates_ref.json")))
    n = 0
    for c in doc["cases"]:
        if "crash" in c:
            continue
        nb, alpha, _ = E.estimate(c["dims"], c["perm"], c["elem"], c["nb"], c["alpha"], 49152, 304)
        assert (nb, "%.2f" % alpha) == (c["nb_out"], c["alpha_out"]), c
        n += 1
    assert n > 100


def test_reference_crash_case_is_handled(E):
    """The reference estimator divides by zero in its nb-halving loop for
    this tuple; the product returns the values the loop had settled on."""
    doc = json.load(open(os.path.join(GOLDEN, "estimates_ref.json")))
    crashes = [c for c in doc["cases"] if "crash" in c]
    for c in crashes:
        nb, alpha, _ = E.estimate(c["dims"], c["perm"], c["elem"], c["nb"], c["alpha"], 49152, 304)
        assert nb >= 1 and alpha > 0


def test_benchmark_shapes(E):
    """3001x4096 int32 and (4,20011,8192,2) int32 perm (1 3 2 4) at alpha 0.01."""
    assert E.estimate([3001, 4096], [2, 1], 4, 1, 0.01, 49152, 304)[:2] == (1, 0.01)
    nb, alpha, extra = E.estimate([4, 20011, 8192, 2], [1, 3, 2, 4], 4, 1, 0.01, 49152, 304)
    assert (nb, alpha) == (1, 0.01) and extra == 4 * 256 * 8192
