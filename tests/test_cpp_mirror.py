"""The C++ front-end (include/illum_gb300.hpp) compiles against the C ABI
and, on a GPU, reproduces the oracle for one reference-style step."""
import os
import subprocess

import numpy as np
import pytest

from illum_gb300 import meshgen

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _compile(ilg, tmp_path):
    exe = str(tmp_path / "mirror_example")
    libdir = os.path.dirname(ilg.library_path())
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "cpp", "mirror_example.cpp"),
           "-L", libdir, "-lillum_gb300", "-Wl,-rpath," + libdir, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def test_cpp_front_end_compiles_and_links(ilg, tmp_path):
    assert os.path.exists(_compile(ilg, tmp_path))


@pytest.mark.gpu
def test_cpp_front_end_matches_oracle(ilg, oracle_mod, tmp_path):
    v, f = meshgen.icosphere_craters(3, seed=2, n_craters=8, dmin_m=150.0, dmax_m=400.0)
    mesh = tmp_path / "mesh.txt"
    with open(mesh, "w") as fh:
        fh.write(f"{v.shape[0]} {f.shape[0]}\n")
        fh.write(" ".join(repr(float(x)) for x in v.ravel()) + "\n")
        fh.write(" ".join(str(int(x)) for x in f.ravel()) + "\n")
    exe = _compile(ilg, tmp_path)
    out = subprocess.run([exe, str(mesh)], check=True, capture_output=True, text=True).stdout.split()
    nnz = int(out[0])
    ts = np.array([float(x) for x in out[1:]])
    H = oracle_mod.horizons(v, f, 16)
    rows, cols, vals, _ = oracle_mod.form_factors(v, f, albedo_scalar=0.1)
    assert nnz == len(vals)
    rp, c, x = oracle_mod.coo_to_csr(f.shape[0], rows, cols, vals)
    E, _ = oracle_mod.direct(v, f, H, np.array([2.2e8, 1.0e7, 3.0e7]), oracle_mod.fib_spiral(100))
    rad, _, _ = oracle_mod.gauss_seidel(rp, c, x, E, tol=1e-12)
    z = 0.001 * np.arange(1, 21) ** 2
    Ts = np.zeros(f.shape[0])
    for k in range(f.shape[0]):
        _, Ts[k], _ = oracle_mod.conductionq(z, 600.0, 0.0, rad[k], np.full(20, 233.0), np.full(20, 300.0),
                                             np.full(20, 1.05e6), 0.999, 233.0)
    assert np.abs(ts - Ts).max() <= 1e-9
