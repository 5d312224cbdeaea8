"""Writes tests/golden/ratran_vanZadelhoff_1{a,b}.npz: the cell radii (ra, rb) and the
fractional level populations (lp0, lp1) of the RATRAN results the reference ships with
its van Zadelhoff problem-1 benchmark (tests/benchmarks/numeric/Ratran_results/
vanZadelhoff_1{a,b}.out, columns id, ra, rb, nh, tk, nm, vr, db, td, lp0, lp1 after 14
header lines, read as vanZadelhoff_1_1D.py:117 reads them).

Run from the repository root with the environment variable REFERENCE naming the root of
a Magritte checkout:  REFERENCE=<checkout> python tests/golden/make_ratran_fixtures.py"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    reference = os.environ.get("REFERENCE")
    if not reference:
        sys.exit("set REFERENCE to the root of a Magritte checkout")
    for kind in ("a", "b"):
        src = os.path.join(reference, "tests", "benchmarks", "numeric", "Ratran_results", f"vanZadelhoff_1{kind}.out")
        cols = np.loadtxt(src, skiprows=14, unpack=True)
        out = os.path.join(HERE, f"ratran_vanZadelhoff_1{kind}.npz")
        np.savez(out, ra=cols[1], rb=cols[2], lp0=cols[9], lp1=cols[10])
        print(out, cols.shape[1], "cells")


if __name__ == "__main__":
    sys.exit(main())
