"""Writes tests/golden/fortran_visco_lmax32.npz from the reference's fixtures.

Reads, from the reference's tests/data directory (the first argument, by
default the checkout this was made from):
  - prem.simp.vm1: the Fortran sl3d's 1D model (title; nknot ntau; rows
    r [m], rho [kg m^-3], kappa [GPa], mu [GPa], log10 viscosity [Pa s],
    0 meaning none);
  - fortran_visco_test.txt: the Fortran visco_test's surface coefficients at
    lmax 32 (rows: output index (t = 1000 yr each), l, m, Re/Im U [m],
    Re/Im phi [m^2 s^-2]; the m < 0 rows are the Hermitian images).
Keeps the model's knots and the rows of outputs 1..5 with m >= 0, as the
reference's benchmarks/fortran_gate.cpp compares them (degree 1 excluded by
the comparison, kept here).

  python tests/golden/make_fortran_gate.py [reference tests/data directory]
"""

import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent


def main():
    data = pathlib.Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/tests/data")
    lines = (data / "prem.simp.vm1").read_text().splitlines()
    nknot = int(lines[1].split()[0])
    knots = np.array([[float(v) for v in line.split()[:5]] for line in lines[2:2 + nknot]])
    rows = np.loadtxt(data / "fortran_visco_test.txt")
    keep = (rows[:, 0] >= 1) & (rows[:, 2] >= 0)
    rows = rows[keep]
    np.savez_compressed(HERE / "fortran_visco_lmax32.npz", knots=knots, output=rows[:, 0].astype(np.int32),
                        l=rows[:, 1].astype(np.int32), m=rows[:, 2].astype(np.int32),
                        U=rows[:, 3] + 1j * rows[:, 4], phi=rows[:, 5] + 1j * rows[:, 6])
    print(f"{len(knots)} knots, {len(rows)} rows")


if __name__ == "__main__":
    main()
