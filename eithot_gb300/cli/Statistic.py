"""Summary of the per-case files that test_inplace appends to, for the
reference's Benchmark/Bench.sh (which runs `python3 Statistic.py` in the
directory of the programs after each case file and then moves
Statistic.txt; the reference repository does not ship the script).

Reads inplace_bench.txt (total time per case, ms) and
inplace_bench_throughput.txt (throughput per case) from the working
directory and prints, and writes to Statistic.txt, the mean and the
population standard deviation of each:

    Bench time:
    \tAvg:  <mean>
    \tStd:  <std>
    Throughput:
    \tAvg:  <mean>
    \tStd:  <std>
"""
import math
import statistics


def read_values(path):
    try:
        with open(path) as f:
            return [float(x) for x in f.read().split()]
    except FileNotFoundError:
        return []


def summary(times, throughputs):
    lines = []
    for title, values in (("Bench time:", times), ("Throughput:", throughputs)):
        mean = statistics.fmean(values) if values else math.nan
        std = statistics.pstdev(values) if values else math.nan
        lines += [title, "\tAvg:  " + str(mean), "\tStd:  " + str(std)]
    return "\n".join(lines) + "\n"


def main():
    text = summary(read_values("inplace_bench.txt"), read_values("inplace_bench_throughput.txt"))
    print(text, end="")
    with open("Statistic.txt", "w") as f:
        f.write(text)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
