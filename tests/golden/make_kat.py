"""Writes kat_test_library.npz: the known answers of the reference's
test_library.cpp (A(i,j) = j*m + i, x_j = j, y_j = j + 1; dgemv and ddot),
computed exactly with Python integers at the sizes the tests use."""
from pathlib import Path

import numpy as np

SIZES = [(1, 1), (7, 3), (128, 128), (257, 129), (1000, 1000)]


def main():
    out = {}
    for m, n in SIZES:
        s1 = sum(j * j for j in range(n))
        s0 = sum(range(n))
        out[f"Ax_{m}x{n}"] = np.array([float(m * s1 + i * s0) for i in range(m)])
        out[f"xy_{m}x{n}"] = np.array(float(sum(j * (j + 1) for j in range(n))))
    np.savez(Path(__file__).resolve().parent / "kat_test_library.npz", **out)


if __name__ == "__main__":
    main()
