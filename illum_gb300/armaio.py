"""Armadillo binary matrix files (ARMA_MAT_BIN_*), the format of the
reference's outputs (horizons.bin, rad*.bin, therm*.bin: arma_util::save_mat,
src/cpp/arma_util.hpp:8-13) and inputs (horizon_file, form_factors_file,
init_temp).

Layout: a text header ``ARMA_MAT_BIN_<type>\\n<n_rows> <n_cols>\\n`` and the
raw elements. Armadillo stores column-major (order="F", the default here);
the reference's Python helper reads and writes C order (src/py/arma.py:4-35),
available as order="C".
"""
from __future__ import annotations

import numpy as np

_TYPES = {"FN008": np.float64, "FN004": np.float32, "IU004": np.uint32, "IU008": np.uint64, "IS008": np.int64,
          "IS004": np.int32, "FC016": np.complex128}
_NAMES = {np.dtype(v): k for k, v in _TYPES.items()}


def save(path: str, X, order: str = "F") -> None:
    X = np.asarray(X)
    if X.ndim == 1:
        X = X.reshape(-1, 1) if order == "F" else X
    if X.dtype not in _NAMES:
        raise ValueError(f"unsupported dtype {X.dtype}")
    with open(path, "wb") as f:
        f.write(b"ARMA_MAT_BIN_%s\n" % _NAMES[X.dtype].encode())
        if X.ndim == 1:
            f.write(b"%d\n" % X.size)
        else:
            f.write(b"%d %d\n" % X.shape)
        f.write(np.asarray(X).tobytes(order=order))


def load(path: str, order: str = "F") -> np.ndarray:
    with open(path, "rb") as f:
        head = f.readline().strip()
        if not head.startswith(b"ARMA_MAT_BIN_"):
            raise ValueError("not an ARMA_MAT_BIN file")
        dt = _TYPES[head[len(b"ARMA_MAT_BIN_"):].decode()]
        dims = tuple(int(x) for x in f.readline().split())
        data = np.frombuffer(f.read(), dtype=dt)
    if len(dims) == 1:
        return data.copy()
    return data.reshape(dims, order=order).copy()
