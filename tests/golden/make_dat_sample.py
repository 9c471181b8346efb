"""Extracts tests/golden/initwo_sample.dat: records of the reference's own text snapshot
initwo.dat, written by its output_file (benchmark_2d_dg.f90:14 with the format of
2d/benchmark_2d_dg.f90:468-495, '(7(1PE12.5,1X))'; 150 x 150 cells, x index outer, six
values per record).  Run here, where the reference is mounted; the tests read only the
committed sample.  The records are copied verbatim: every 150th record (one per x column),
and the first ten that hold a negative value and the first ten with an exponent E-03.

    python tests/golden/make_dat_sample.py [path/to/initwo.dat]
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/initwo.dat"


def main():
    lines = open(SRC).read().split("\n")
    if lines and lines[-1] == "":
        lines = lines[:-1]
    pick = set(range(0, len(lines), 150))
    neg = [i for i, ln in enumerate(lines) if any(t.startswith("-") for t in ln.split())]
    e03 = [i for i, ln in enumerate(lines) if "E-03" in ln]
    pick.update(neg[:10])
    pick.update(e03[:10])
    with open(os.path.join(HERE, "initwo_sample.dat"), "w") as f:
        for i in sorted(pick):
            f.write(lines[i] + "\n")
    print("wrote %d records" % len(pick))


if __name__ == "__main__":
    main()
