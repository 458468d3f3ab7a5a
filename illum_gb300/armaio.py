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


def save_sparse(path: str, rowptr, col, val, n_cols: int | None = None) -> None:
    """Write a CSR matrix (rows = receivers, as the library's F) as an
    Armadillo sparse binary file, ARMA_SPM_BIN_FN008: header
    ``ARMA_SPM_BIN_FN008\\n<n_rows> <n_cols> <n_nonzero>\\n``, then the values,
    the row indices and the column pointers (u64) of the compressed-column
    form, which is how Armadillo stores sp_mat (the reference's
    form_factors.bin, src/cpp/illum_cli.cpp:282 through arma_util::save_mat,
    src/cpp/arma_util.hpp:8-13)."""
    rowptr = np.asarray(rowptr, np.int64)
    col = np.asarray(col, np.int64)
    val = np.asarray(val, np.float64)
    n_rows = rowptr.size - 1
    n_cols = n_rows if n_cols is None else int(n_cols)
    rows = np.repeat(np.arange(n_rows, dtype=np.int64), np.diff(rowptr))
    order = np.lexsort((rows, col))          # column-major: by column, then row
    r, c, v = rows[order], col[order], val[order]
    colptr = np.zeros(n_cols + 1, np.uint64)
    np.add.at(colptr, c + 1, 1)
    colptr = np.cumsum(colptr).astype(np.uint64)
    with open(path, "wb") as f:
        f.write(b"ARMA_SPM_BIN_FN008\n%d %d %d\n" % (n_rows, n_cols, v.size))
        f.write(v.tobytes())
        f.write(r.astype(np.uint64).tobytes())
        f.write(colptr.tobytes())


def load_sparse(path: str):
    """Read an ARMA_SPM_BIN_FN008 file (64-bit indices) and return the matrix
    as CSR (rowptr int64, col int32, val float64, n_cols), the layout
    IllumContext.set_F takes."""
    with open(path, "rb") as f:
        head = f.readline().strip()
        if head != b"ARMA_SPM_BIN_FN008":
            raise ValueError("not an ARMA_SPM_BIN_FN008 file")
        n_rows, n_cols, nnz = (int(x) for x in f.readline().split())
        v = np.frombuffer(f.read(8 * nnz), np.float64)
        r = np.frombuffer(f.read(8 * nnz), np.uint64).astype(np.int64)
        colptr = np.frombuffer(f.read(8 * (n_cols + 1)), np.uint64).astype(np.int64)
    if colptr[-1] != nnz:
        raise ValueError("inconsistent column pointers")
    c = np.repeat(np.arange(n_cols, dtype=np.int64), np.diff(colptr))
    order = np.lexsort((c, r))
    rowptr = np.zeros(n_rows + 1, np.int64)
    np.add.at(rowptr, r + 1, 1)
    return np.cumsum(rowptr), c[order].astype(np.int32), v[order].copy(), n_cols


def load_sun_positions(path: str, unit: str = "km") -> np.ndarray:
    """Sun positions from a whitespace-separated text file, one position per
    line, columns beyond the third ignored, as the reference loads
    sun_pos_file (src/cpp/illum_cli.cpp:325-345: raw ASCII, rows shed past 3,
    metres rescaled to km when sun_unit is "m"). Returns n x 3 in km."""
    if unit not in ("km", "m"):
        raise ValueError("unit must be 'km' or 'm'")
    S = np.loadtxt(path, dtype=np.float64, ndmin=2)
    if S.shape[1] < 3:
        raise ValueError("sun position file needs three columns")
    S = S[:, :3].copy()
    if unit == "m":
        S /= 1000.0
    return S
