"""Regenerates the golden fixtures that come from the reference's own code.

Run in a checkout where the reference project is available (its root given
as the first argument); the outputs are committed, so the tests never need
the reference at run time:
  * fib_spiral_100.npy — src/py/points.py fibonacci_spiral(100), the Python
    twin of fib_spiral (src/cpp/illum.cpp:468-483);
  * arma_dense.bin — a 3 x 4 float64 matrix written by src/py/arma.py tofile,
    the ARMA_MAT_BIN_FN008 format of the reference's outputs.
"""
import os
import sys

import numpy as np


def main(ref_root: str) -> None:
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(ref_root, "src", "py"))
    import points  # noqa: E402
    import arma    # noqa: E402
    X, Y = points.fibonacci_spiral(100)
    np.save(os.path.join(here, "fib_spiral_100.npy"), np.stack([X, Y], 1))
    M = np.arange(12, dtype=np.float64).reshape(3, 4) * 0.25 - 1.0
    arma.tofile(M, os.path.join(here, "arma_dense.bin"))
    np.save(os.path.join(here, "arma_dense_values.npy"), M)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <root of the reference checkout>")
    main(sys.argv[1])
