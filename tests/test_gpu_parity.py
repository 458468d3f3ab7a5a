"""GPU parity: every CUDA path through the C ABI against the CPU oracle.

Exactness bars: ray hits, horizons, visibility sets, form-factor values and
direct insolation are compared bit for bit; radiosity to the solve
tolerance; temperatures of the FP64 path to 1e-9 K; the mixed-precision path
to 0.05 K.
"""
import math

import numpy as np
import pytest

from illum_gb300 import meshgen

pytestmark = pytest.mark.gpu

TOL_T_FP64 = 1e-9      # K
TOL_T_MIXED = 0.05     # K


@pytest.fixture(scope="module")
def mesh_l4():
    return meshgen.icosphere_craters(4, seed=0)          # 5,120 facets (the CPU-runnable configuration)


@pytest.fixture(scope="module")
def mesh_l3():
    return meshgen.icosphere_craters(3, seed=3, n_craters=12, dmin_m=150.0, dmax_m=450.0)


def _rays(oracle_mod, v, f, n, seed):
    c, nn, r, a = oracle_mod.facet_geometry(v, f)
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, len(f), n)
    o = (c[idx] + 1e-5 * nn[idx]).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    return o, d


def test_trace_bit_exact(ilg, oracle_mod, mesh_l3):
    v, f = mesh_l3
    ctx = ilg.IllumContext(v, f)
    o, d = _rays(oracle_mod, v, f, 20000, 1)
    hg, tg = ctx.trace(o, d)
    ho, to = oracle_mod.trace(v, f, o, d)
    assert np.array_equal(hg, ho)
    assert np.array_equal(tg[hg >= 0], to[ho >= 0])
    ag, _ = ctx.trace(o, d, any_hit=True)
    ao, _ = oracle_mod.trace(v, f, o, d, any_hit=True)
    assert np.array_equal(ag >= 0, ao >= 0)


def test_trace_grazing_rays_bit_exact(ilg, oracle_mod, mesh_l3):
    """Rays aimed at triangle vertices and edge midpoints (where the float
    filter must defer to the double-precision predicate)."""
    v, f = mesh_l3
    ctx = ilg.IllumContext(v, f)
    rng = np.random.default_rng(7)
    tgt_f = rng.integers(0, len(f), 4000)
    w = rng.integers(0, 3, 4000)
    tv = v[f[tgt_f, w]].astype(np.float64)
    tv2 = v[f[tgt_f, (w + 1) % 3]].astype(np.float64)
    tgt = np.where((np.arange(4000) % 2 == 0)[:, None], tv, 0.5 * (tv + tv2))
    src = rng.normal(size=(4000, 3))
    src = 2.0 * src / np.linalg.norm(src, axis=1, keepdims=True)
    d = tgt - src
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    o = src.astype(np.float32)
    hg, tg = ctx.trace(o, d)
    ho, to = oracle_mod.trace(v, f, o, d, brute=True)
    assert np.array_equal(hg, ho)
    assert np.array_equal(tg[hg >= 0], to[ho >= 0])


def test_horizons_bit_exact(ilg, oracle_mod, mesh_l4):
    v, f = mesh_l4
    ctx = ilg.IllumContext(v, f)
    ctx.make_horizons(nphi=32, theta_eps=1e-3, offset=1e-5)
    Hg = ctx.horizons
    Ho = oracle_mod.horizons(v, f, 32, 1e-3, 1e-5).T
    assert Hg.shape == (32, f.shape[0])
    assert np.array_equal(Hg, Ho)


def test_horizons_other_eps_bit_exact(ilg, oracle_mod, mesh_l3):
    v, f = mesh_l3
    ctx = ilg.IllumContext(v, f)
    for nphi, eps in ((9, 1e-2), (17, 3e-4)):
        ctx.make_horizons(nphi=nphi, theta_eps=eps)
        assert np.array_equal(ctx.horizons, oracle_mod.horizons(v, f, nphi, eps).T)


def test_form_factors_bit_exact(ilg, oracle_mod, mesh_l4):
    v, f = mesh_l4
    ctx = ilg.IllumContext(v, f)
    rowptr, col, val = ctx.compute_F(albedo=0.1)
    ro, co, vo, rays = oracle_mod.form_factors(v, f, albedo_scalar=0.1)
    rp, c, x = oracle_mod.coo_to_csr(f.shape[0], ro, co, vo)
    assert ctx.visibility_rays == rays
    assert np.array_equal(rowptr, rp) and np.array_equal(col, c) and np.array_equal(val, x)


@pytest.mark.parametrize("chunk", [997, 20000])
def test_form_factors_several_chunks_bit_exact(ilg, oracle_mod, mesh_l4, chunk):
    """The build in source chunks of `chunk` candidate pairs (many chunks,
    each deduplicated on its own, then merged by a global sort) gives the
    one-chunk build's matrix and the oracle's, bit for bit, and the radiosity
    tiles built from it solve the same system."""
    v, f = mesh_l4
    ctx = ilg.IllumContext(v, f)
    try:
        ilg.debug_ff_chunk(chunk)
        rowptr, col, val = ctx.compute_F(albedo=0.1)
    finally:
        ilg.debug_ff_chunk(0)
    ro, co, vo, rays = oracle_mod.form_factors(v, f, albedo_scalar=0.1)
    rp, c, x = oracle_mod.coo_to_csr(f.shape[0], ro, co, vo)
    assert ctx.visibility_rays == rays
    assert np.array_equal(rowptr, rp) and np.array_equal(col, c) and np.array_equal(val, x)
    ref = ilg.IllumContext(v, f)
    ref.compute_F(albedo=0.1)
    E = np.random.default_rng(5).uniform(0.0, 800.0, f.shape[0])
    assert np.array_equal(ctx.radiosity_solve(E, tol=1e-10)[0], ref.radiosity_solve(E, tol=1e-10)[0])


def test_form_factors_per_facet_albedo(ilg, oracle_mod, mesh_l3):
    v, f = mesh_l3
    alb = np.random.default_rng(2).uniform(0.05, 0.3, f.shape[0])
    ctx = ilg.IllumContext(v, f)
    rowptr, col, val = ctx.compute_F(albedo=alb)
    ro, co, vo, _ = oracle_mod.form_factors(v, f, albedo=alb)
    rp, c, x = oracle_mod.coo_to_csr(f.shape[0], ro, co, vo)
    assert np.array_equal(rowptr, rp) and np.array_equal(col, c) and np.array_equal(val, x)


@pytest.mark.parametrize("cutoff_m", [15.0, 40.0])
def test_form_factors_cutoff_bit_exact(ilg, oracle_mod, cutoff_m):
    """Terrain patch with the distance cutoff: same pairs, rays and values as
    the oracle's brute-force loop with the same cutoff test."""
    v, f = meshgen.heightmap_terrain(n=40, n_bowls=6, seed=3)
    ctx = ilg.IllumContext(v, f)
    rowptr, col, val = ctx.compute_F(albedo=0.1, cutoff=cutoff_m / 1000.0)
    ro, co, vo, rays = oracle_mod.form_factors(v, f, albedo_scalar=0.1, cutoff=cutoff_m / 1000.0)
    rp, c, x = oracle_mod.coo_to_csr(f.shape[0], ro, co, vo)
    assert ctx.visibility_rays == rays
    assert np.array_equal(rowptr, rp) and np.array_equal(col, c) and np.array_equal(val, x)
    assert len(val) > 0


@pytest.mark.parametrize("norm_mode,interp", [(0, 0), (1, 0), (1, 1)])
def test_direct_bit_exact(ilg, oracle_mod, mesh_l4, norm_mode, interp):
    v, f = mesh_l4
    ctx = ilg.IllumContext(v, f)
    ctx.make_horizons(nphi=32)
    H = ctx.horizons
    ctx.set_insolation(norm_mode, interp, 1361.0)
    disk = ilg.fib_spiral(100)
    suns = meshgen.spin_sun_positions(24, 6 * 3600.0, 900.0)
    for s in suns:
        dg = ctx.get_direct_radiosity(s, disk)
        do, _ = oracle_mod.direct(v, f, H.T, s, disk, norm_mode, interp, 1361.0)
        assert np.array_equal(dg, do)


def test_radiosity_converges_to_oracle(ilg, oracle_mod, mesh_l4):
    v, f = mesh_l4
    n = f.shape[0]
    ctx = ilg.IllumContext(v, f)
    rowptr, col, val = ctx.compute_F(albedo=0.1)
    E = np.random.default_rng(3).uniform(0, 600, n)
    x, res, sweeps = ctx.radiosity_solve(E, tol=1e-10, max_sweeps=200)
    xo, reso, _ = oracle_mod.gauss_seidel(rowptr, col, val, E, mode=1, tol=1e-12)
    assert res <= 1e-10 and sweeps >= 1
    assert np.abs(x - xo).max() <= 1e-10
    # residual computed independently
    A_x = x.copy()
    for i in range(n):
        A_x[i] -= val[rowptr[i]:rowptr[i + 1]] @ x[col[rowptr[i]:rowptr[i + 1]]]
    assert np.linalg.norm(A_x - E) <= 1e-10


def test_set_F_round_trip(ilg, oracle_mod, mesh_l3):
    v, f = mesh_l3
    ctx = ilg.IllumContext(v, f)
    rp, c, x = ctx.compute_F(albedo=0.1)
    ctx2 = ilg.IllumContext(v, f)
    ctx2.set_F(rp, c, x)
    E = np.linspace(0, 500, f.shape[0])
    a, _, _ = ctx.radiosity_solve(E)
    b, _, _ = ctx2.radiosity_solve(E)
    assert np.array_equal(a, b)


# ------------------------------------------------------------ conduction
def _profile(nz):
    return meshgen.geometric_depths(nz), np.full(nz, 300.0), np.full(nz, 1.05e6)


@pytest.mark.parametrize("bc_mode", [0, 1])
def test_conduction_batch_vs_oracle(ilg, oracle_mod, bc_mode):
    nz, ncol = 40, 777
    z, ti, rhoc = _profile(nz)
    rng = np.random.default_rng(4)
    T = rng.uniform(180, 320, (nz, ncol))
    Ts = rng.uniform(180, 320, ncol)
    Qn = rng.uniform(0, 800, ncol)
    Qp = rng.uniform(0, 800, ncol)
    Tg, Tsg, Fsg = ilg.conductionQ_batch(z, 30.0, Qn, Qp, T, ti, rhoc, 0.95, Ts, bc_mode=bc_mode)
    for k in range(ncol):
        if bc_mode == 0:
            To, tso, fso = oracle_mod.conductionq(z, 30.0, Qn[k], Qp[k], T[:, k], ti, rhoc, 0.95, Ts[k])
        else:
            To, tso, fso, _ = oracle_mod.conductionq_newton(z, 30.0, Qp[k], T[:, k], ti, rhoc, 0.95, Ts[k])
        assert np.abs(Tg[:, k] - To).max() <= 1e-9
        assert abs(Tsg[k] - tso) <= 1e-9
        assert abs(Fsg[k] - fso) <= 1e-9 * max(1.0, abs(fso))


def test_fortran_abi_symbols(ilg, oracle_mod):
    """conductionq_ / conductiont_ with the reference's exact signatures."""
    z, ti, rhoc = _profile(25)
    T = np.linspace(260, 210, 25)
    Tg, tsg, fsg = ilg.conductionQ(z, 60.0, 100.0, 450.0, T, ti, rhoc, 0.999, 255.0)
    To, tso, fso = oracle_mod.conductionq(z, 60.0, 100.0, 450.0, T, ti, rhoc, 0.999, 255.0)
    assert np.abs(Tg - To).max() <= 1e-9 and abs(tsg - tso) <= 1e-9
    Tg2, fg2 = ilg.conductionT(z, 60.0, T, 255.0, 270.0, ti, rhoc)
    To2, fo2 = oracle_mod.conductiont(z, 60.0, T, 255.0, 270.0, ti, rhoc)
    assert np.abs(Tg2 - To2).max() <= 1e-9 and abs(fg2 - fo2) <= 1e-9 * max(1, abs(fo2))


def test_thermal_model_step_vs_oracle(ilg, oracle_mod, mesh_l3):
    v, f = mesh_l3
    n = f.shape[0]
    ctx = ilg.IllumContext(v, f)
    z, ti, rhoc = _profile(30)
    tm = ilg.ThermalModel(ctx, z, 300.0, 1.05e6, 233.0)
    T = np.full((n, 31), 233.0)
    Qprev = np.zeros(n)
    Fs = np.zeros(n)
    rng = np.random.default_rng(5)
    for step in range(5):
        Q = rng.uniform(0, 700, n)
        tm.step(600.0, Q)
        for k in range(n):
            T[k, 1:], T[k, 0], Fs[k] = oracle_mod.conductionq(z, 600.0, Qprev[k], Q[k], T[k, 1:], ti, rhoc, 0.999,
                                                              T[k, 0])
        Qprev = Q
    assert np.abs(tm.T - T.T).max() <= TOL_T_FP64
    assert np.abs(tm.get_radiosity() + Fs).max() <= 1e-9 * max(1, np.abs(Fs).max())


# ------------------------------------------------------------ fused loop
def _setup_run(ilg, oracle_mod, v, f, nphi, nz, nsteps, period=6 * 3600.0, steps_per_rot=360, use_graph=1,
               precision=0, bc_mode=1, coupling=1):
    ctx = ilg.IllumContext(v, f)
    ctx.make_horizons(nphi=nphi)
    ctx.set_insolation(1, 0, 1361.0)
    rp, c, x = ctx.compute_F(albedo=0.1)
    dt = period / steps_per_rot
    suns = meshgen.spin_sun_positions(nsteps, period, dt)
    disk = ilg.fib_spiral(100)
    ctx.set_suns(suns, disk)
    z, ti, rhoc = _profile(nz)
    tm = ilg.ThermalModel(ctx, z, 300.0, 1.05e6, 200.0, emissivity=0.95, bc_mode=bc_mode, precision=precision)
    opts = ilg.RunOpts(dt=dt, tol=1e-10, max_sweeps=200, use_radiosity=1, use_graph=use_graph, precision=precision,
                       coupling=coupling)
    return ctx, tm, opts, (rp, c, x), suns, disk, (z, ti, rhoc), dt


@pytest.mark.parametrize("coupling,nsteps", [(0, 120), (1, 360)])
def test_run_steps_vs_oracle_fp64(ilg, oracle_mod, mesh_l4, coupling, nsteps):
    """Run on the 5,120-facet icosphere (L4, 32 azimuths, 40 layers, Newton boundary, radiosity
    to 1e-10): surface and subsurface temperatures within 1e-9 K, with the
    reference's E = -Fsurf + direct coupling and with E = direct."""
    v, f = mesh_l4
    ctx, tm, opts, csr, suns, disk, (z, ti, rhoc), dt = _setup_run(ilg, oracle_mod, v, f, 32, 40, nsteps,
                                                                   coupling=coupling)
    hist = ctx.run_steps(opts, 0, nsteps, record_tsurf=True)
    st = oracle_mod.thermal_run(v, f, ctx.horizons.T, suns, disk, csr, z, ti, rhoc, dt=dt, T0=200.0, emiss=0.95,
                                solar_const=1361.0, norm_mode=1, bc_mode=1, rad_mode=1, tol=1e-10,
                                record_tsurf=True, coupling=coupling)
    assert np.abs(hist - st["tsurf_hist"]).max() <= TOL_T_FP64
    assert np.abs(tm.T - st["T"].T).max() <= TOL_T_FP64
    out = ctx.outputs()
    assert np.abs(out["therm_avg"] - st["therm_avg"]).max() <= TOL_T_FP64
    assert np.abs(out["rad_avg"] - st["rad_avg"]).max() <= 1e-8


def test_run_steps_reference_boundary(ilg, oracle_mod, mesh_l3):
    v, f = mesh_l3
    nsteps = 60
    ctx, tm, opts, csr, suns, disk, (z, ti, rhoc), dt = _setup_run(ilg, oracle_mod, v, f, 16, 30, nsteps, bc_mode=0,
                                                                   coupling=0)
    ctx.run_steps(opts, 0, nsteps)
    st = oracle_mod.thermal_run(v, f, ctx.horizons.T, suns, disk, csr, z, ti, rhoc, dt=dt, T0=200.0, emiss=0.95,
                                solar_const=1361.0, norm_mode=1, bc_mode=0, rad_mode=1, tol=1e-10, coupling=0)
    assert np.abs(tm.T - st["T"].T).max() <= TOL_T_FP64


@pytest.mark.parametrize("coupling", [0, 1])
def test_run_steps_without_form_factors_vs_oracle(ilg, oracle_mod, mesh_l3, coupling):
    """Steps without the radiosity solve: the conduction takes the frame's
    direct flux itself (with the reference's -Fsurf coupling or without) and
    records it as the radiosity; temperatures and averages as the oracle's
    loop without form factors."""
    v, f = mesh_l3
    nsteps = 60
    ctx, tm, opts, csr, suns, disk, (z, ti, rhoc), dt = _setup_run(ilg, oracle_mod, v, f, 16, 30, nsteps,
                                                                   coupling=coupling)
    opts.use_radiosity = 0
    hist = ctx.run_steps(opts, 0, nsteps, record_tsurf=True)
    st = oracle_mod.thermal_run(v, f, ctx.horizons.T, suns, disk, None, z, ti, rhoc, dt=dt, T0=200.0, emiss=0.95,
                                solar_const=1361.0, norm_mode=1, bc_mode=1, record_tsurf=True, coupling=coupling)
    assert np.abs(hist - st["tsurf_hist"]).max() <= TOL_T_FP64
    assert np.abs(tm.T - st["T"].T).max() <= TOL_T_FP64
    out = ctx.outputs()
    assert np.abs(out["rad"] - st["rad"]).max() <= 1e-8
    assert np.abs(out["rad_avg"] - st["rad_avg"]).max() <= 1e-8


def test_graph_equals_eager_and_host_driven(ilg, oracle_mod, mesh_l3):
    v, f = mesh_l3
    runs = []
    for mode in ("graph", "eager", "host"):
        ctx, tm, opts, csr, suns, disk, _, _ = _setup_run(ilg, oracle_mod, v, f, 16, 30, 40,
                                                          use_graph=0 if mode == "eager" else 1)
        if mode == "host":
            h = ctx.run_steps_host(opts, suns)
        else:
            h = ctx.run_steps(opts, 0, 40, record_tsurf=True)
        runs.append((h, tm.T))
    for h, T in runs[1:]:
        assert np.array_equal(h, runs[0][0]) and np.array_equal(T, runs[0][1])


@pytest.mark.parametrize("precision,coupling,use_radiosity", [(0, 0, 1), (1, 1, 1), (0, 0, 0), (1, 1, 0)])
def test_pipelined_steps_equal_serial_order(ilg, oracle_mod, mesh_l3, precision, coupling, use_radiosity):
    """Graph and eager steps run the next frame's direct insolation beside
    the current conduction; phase-timed steps run direct -> radiosity ->
    conduction in order. Both give the same temperatures and outputs bit for
    bit, with either coupling and for a mesh stepped without form factors
    (its conduction reads the direct flux itself)."""
    v, f = mesh_l3
    runs = []
    for mode in ("serial", "graph", "eager"):
        ctx, tm, opts, _, _, _, _, _ = _setup_run(ilg, oracle_mod, v, f, 16, 30, 24, precision=precision,
                                                  coupling=coupling, use_graph=0 if mode == "eager" else 1)
        opts.use_radiosity = use_radiosity
        if precision == ilg.PREC_MIXED:
            opts.tol, opts.max_sweeps = 1e-3, 2
        ctx.set_timing(mode == "serial")
        h = ctx.run_steps(opts, 0, 24, record_tsurf=True)
        ctx.set_timing(False)
        out = ctx.outputs()
        runs.append((h, tm.T.copy(), out["rad"], out["rad_avg"], out["therm_avg"]))
    for r in runs[1:]:
        for a, b in zip(r, runs[0]):
            assert np.array_equal(a, b)


def test_refine_every_graph_equals_eager(ilg, oracle_mod, mesh_l3):
    """The one-pass mixed solve (refine_every = 3): graph, eager and
    phase-timed steps give the same results bit for bit, with one sweep
    per step."""
    v, f = mesh_l3
    runs = []
    for mode in ("serial", "graph", "eager"):
        ctx, tm, opts, _, _, _, _, _ = _setup_run(ilg, oracle_mod, v, f, 16, 30, 24, precision=1,
                                                  use_graph=0 if mode == "eager" else 1)
        opts.tol, opts.max_sweeps, opts.refine_every = 1e-3, 1, 3
        ctx.set_timing(mode == "serial")
        h = ctx.run_steps(opts, 0, 24, record_tsurf=True)
        if mode == "serial":   # phase-timed steps record their sweep counts
            assert ctx.stats()["radiosity_sweeps"] == 24
        ctx.set_timing(False)
        runs.append((h, tm.T.copy(), ctx.outputs()["rad"]))
    for r in runs[1:]:
        for a, b in zip(r, runs[0]):
            assert np.array_equal(a, b)


def test_refine_every_is_checked(ilg, oracle_mod, mesh_l3):
    """refine_every belongs to the mixed precision, and is >= 0."""
    v, f = mesh_l3
    ctx, tm, opts, _, _, _, _, _ = _setup_run(ilg, oracle_mod, v, f, 16, 30, 4, precision=0)
    opts.refine_every = 2
    with pytest.raises(ilg.IlgError):
        ctx.run_steps(opts, 0, 2)
    ctx, tm, opts, _, _, _, _, _ = _setup_run(ilg, oracle_mod, v, f, 16, 30, 4, precision=1)
    opts.refine_every = -1
    with pytest.raises(ilg.IlgError):
        ctx.run_steps(opts, 0, 2)


@pytest.mark.parametrize("precision,refine_every", [(0, 0), (1, 4)])
def test_split_runs_equal_one_run(ilg, oracle_mod, mesh_l3, precision, refine_every):
    """Runs continue where the last one stopped (warm start, and the
    one-pass mixed solve's reference step schedule and reference)."""
    v, f = mesh_l3
    runs = []
    for split in ((30,), (10, 11, 9)):
        ctx, tm, opts, *_ = _setup_run(ilg, oracle_mod, v, f, 16, 30, 30, precision=precision)
        if precision:
            opts.tol, opts.max_sweeps, opts.refine_every = 1e-3, 1, refine_every
        s0 = 0
        for n in split:
            ctx.run_steps(opts, s0, n)
            s0 += n
        runs.append((tm.T.copy(), ctx.outputs()["rad"]))
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1], runs[1][1])


@pytest.mark.parametrize("tol,max_sweeps,refine_every", [(1e-10, 200, 0), (1e-3, 2, 0), (1e-3, 1, 0),
                                                         (1e-3, 1, 1), (1e-3, 1, 4), (1e-3, 1, 16)])
def test_mixed_precision_within_tolerance(ilg, oracle_mod, mesh_l4, tol, max_sweeps, refine_every):
    """Mixed path (bf16 form factors, fp32 conduction) against the FP64 path:
    solved to tolerance, with one refinement round per step (a budget of
    two sweeps, or of one, stops the solve after its first update; the
    round runs that many bf16 sweeps), and with one pass per step whose
    f32 reference pass comes every refine_every steps."""
    v, f = mesh_l4
    nsteps = 360
    ref = _setup_run(ilg, oracle_mod, v, f, 32, 40, nsteps, precision=0)
    mix = _setup_run(ilg, oracle_mod, v, f, 32, 40, nsteps, precision=1)
    mix[2].tol = tol
    mix[2].max_sweeps = max_sweeps
    mix[2].refine_every = refine_every
    ha = ref[0].run_steps(ref[2], 0, nsteps, record_tsurf=True)
    hb = mix[0].run_steps(mix[2], 0, nsteps, record_tsurf=True)
    err_s = np.abs(ha - hb).max()
    err_t = np.abs(ref[1].T - mix[1].T).max()
    assert err_s <= TOL_T_MIXED and err_t <= TOL_T_MIXED, (err_s, err_t)


def test_mixed_precision_conductive_material(ilg, oracle_mod, mesh_l4):
    """High thermal inertia (conductive top layer, k1 ~ 1e4 W/m^2 K): the
    Newton boundary's root is 2 k1 / |g'| times more sensitive to the
    boundary's P than to the layers, which the fp32 state must not feel."""
    v, f = mesh_l4
    nsteps = 300
    ref = _setup_run(ilg, oracle_mod, v, f, 32, 79, nsteps, precision=0)
    mix = _setup_run(ilg, oracle_mod, v, f, 32, 79, nsteps, precision=1)
    out = []
    for ctx, _, opts, *_ in (ref, mix):
        tm = ilg.ThermalModel(ctx, meshgen.geometric_depths(79), 1515.0, 1.05e6, 200.0, emissivity=0.95,
                              bc_mode=1, precision=opts.precision)
        if opts.precision == 1:
            opts.tol, opts.max_sweeps = 1e-3, 2
        ctx.run_steps(opts, 0, nsteps)
        out.append(tm.T.copy())
    err = np.abs(out[0] - out[1]).max()
    assert err <= TOL_T_MIXED, err


# ------------------------------------------------------------ edge cases
def test_single_triangle_and_no_form_factors(ilg, oracle_mod):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    f = np.array([[0, 1, 2]], np.int32)
    ctx = ilg.IllumContext(v, f)
    rp, c, x = ctx.compute_F(albedo=0.1)
    assert rp.tolist() == [0, 0] and len(x) == 0
    ctx.make_horizons(nphi=8)
    assert np.array_equal(ctx.horizons, oracle_mod.horizons(v, f, 8).T)
    E = np.array([5.0])
    xs, res, sw = ctx.radiosity_solve(E)
    assert xs.tolist() == [5.0]


def test_convex_sphere_has_empty_F(ilg, oracle_mod):
    v, f = meshgen.icosphere_craters(3, 0, n_craters=0, sigma_m=0.0)
    ctx = ilg.IllumContext(v, f)
    rp, c, x = ctx.compute_F()
    ro, co, vo, rays = oracle_mod.form_factors(v, f)
    assert len(x) == len(vo) == 0 and ctx.visibility_rays == rays


def test_errors_are_reported(ilg):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    with pytest.raises(ilg.IlgError):
        ilg.IllumContext(v, np.array([[0, 1, 5]], np.int32))
    ctx = ilg.IllumContext(v, np.array([[0, 1, 2]], np.int32))
    with pytest.raises(ilg.IlgError):
        ctx.make_horizons(nphi=1)
    with pytest.raises(ilg.IlgError):
        ctx.radiosity_solve(np.zeros(1))        # no form factors yet
    with pytest.raises(ilg.IlgError):
        ilg.conductionQ_batch(np.array([0.1]), 1.0, None, np.zeros(1), np.zeros((1, 1)), np.ones(1), np.ones(1),
                              1.0, np.zeros(1))   # nz < 2


def _grid_faces(n):
    idx = np.arange(n * n).reshape(n, n)
    a = idx[:-1, :-1].ravel(); b = idx[1:, :-1].ravel(); c = idx[1:, 1:].ravel(); d = idx[:-1, 1:].ravel()
    return np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)]).astype(np.int32)


def test_horizons_with_separate_mesh_bit_exact(ilg, oracle_mod):
    """A separate horizon mesh (src/cpp/illum.cpp:333-349): the facets of a
    33 x 33 patch cut from the middle of a 97 x 97 terrain take their
    horizons from the whole terrain. Bit for bit against the oracle, and
    different from the patch's own horizons (the surroundings rise above
    them)."""
    n, m0, m = 97, 32, 33
    hv, hf = meshgen.heightmap_terrain(n=n, spacing_m=2.0, seed=4, rms_m=8.0, n_bowls=12, dmin_m=10.0, dmax_m=60.0)
    sub = (np.arange(m0, m0 + m)[:, None] * n + np.arange(m0, m0 + m)[None, :]).ravel()
    v = np.ascontiguousarray(hv[sub])
    f = _grid_faces(m)
    ctx = ilg.IllumContext(v, f)
    ctx.set_horizon_mesh(hv, hf)
    ctx.make_horizons(nphi=24)
    Ho = oracle_mod.horizons(v, f, 24, horizon_mesh=(hv, hf))
    assert np.array_equal(ctx.horizons.T, Ho)
    own = ilg.IllumContext(v, f)
    own.make_horizons(nphi=24)
    assert np.array_equal(own.horizons.T, oracle_mod.horizons(v, f, 24))
    assert (own.horizons > ctx.horizons + 1e-3).mean() > 0.2


def test_visibility_sample_counts_match_F(ilg):
    """Sampled visibility (no F built): every source listed gives exactly the
    column counts of the form factors computed with the same cutoff, and the
    within-radius counts follow the entries' centroid distances."""
    v, f = meshgen.heightmap_terrain(n=65, spacing_m=2.0, seed=5, rms_m=6.0, n_bowls=8, dmin_m=10.0, dmax_m=50.0)
    ctx = ilg.IllumContext(v, f)
    cut = 0.04
    rp, col, val = ctx.compute_F(albedo=0.1, cutoff=cut)
    n = f.shape[0]
    colcount = np.bincount(col, minlength=n)
    allsrc = ctx.visibility_sample(np.arange(n), cutoff=cut, radii=[0.01, 0.02, cut])
    assert np.array_equal(allsrc["per_source"], colcount)
    # the cutoff compares float squared distances, the radii double distances:
    # pairs within rounding of the cutoff may fall on either side
    assert abs(int(allsrc["within_radius"][-1]) - len(val)) <= 2
    assert allsrc["rays"] == ctx.visibility_rays
    rows = np.repeat(np.arange(n), np.diff(rp))
    cen = v[f].astype(np.float64).mean(axis=1)
    d = np.linalg.norm(cen[rows] - cen[col], axis=1)
    for r, w in zip([0.01, 0.02], allsrc["within_radius"][:2]):
        exp = int(np.count_nonzero(d <= r))
        assert abs(int(w) - exp) <= 2 + 1e-4 * exp     # float centroids vs the float64 recomputation
    sub = np.random.default_rng(3).choice(n, 300, replace=False).astype(np.int32)
    part = ctx.visibility_sample(sub, cutoff=cut)
    assert np.array_equal(part["per_source"], colcount[sub])


def test_unbiased_layer_rounding_long_run(ilg, oracle_mod):
    """layer_rounding = 1: the mixed path's FP32 layer updates rounded
    without bias. Over a long run (10 rotations of 1,440 steps, thermal
    inertia 50, 80 layers) round-to-nearest loses the increments below half
    an ulp at depth and the layers drift from the FP64 run's; unbiased
    rounding keeps them at least twice closer, and the surface within the
    mixed path's 0.05 K."""
    v, f = meshgen.icosphere_craters(3, seed=5, n_craters=12, dmin_m=120.0, dmax_m=400.0)
    spr, nrot = 1440, 10
    period = 2 * 3600.0
    dt = period / spr
    n = spr * nrot
    z = meshgen.geometric_depths(80)
    res = {}
    for name, prec, lr in (("fp64", 0, 0), ("nearest", 1, 0), ("unbiased", 1, 1)):
        ctx = ilg.IllumContext(v, f)
        ctx.make_horizons(nphi=16)
        ctx.set_insolation(1, 0, 1361.0)
        ctx.compute_F(albedo=0.1)
        ctx.set_suns(meshgen.spin_sun_positions(n, period, dt), ilg.fib_spiral(100))
        tm = ilg.ThermalModel(ctx, z, 50.0, 1.05e6, 200.0, emissivity=0.95, bc_mode=ilg.BC_NEWTON, precision=prec)
        o = ilg.RunOpts(dt=dt, tol=1e-10 if prec == 0 else 1e-3, max_sweeps=200 if prec == 0 else 1, use_radiosity=1,
                        use_graph=1, precision=prec, coupling=1, refine_every=4 if prec else 0, layer_rounding=lr)
        ctx.run_steps(o, 0, n - 1)
        last = ctx.run_steps(o, n - 1, 1, record_tsurf=True)[-1]
        res[name] = (tm.T.copy(), last.copy())
    e_near = np.abs(res["nearest"][0] - res["fp64"][0]).max()
    e_unb = np.abs(res["unbiased"][0] - res["fp64"][0]).max()
    s_unb = np.abs(res["unbiased"][1] - res["fp64"][1]).max()
    assert e_unb < 0.5 * e_near, (e_unb, e_near)
    assert s_unb <= TOL_T_MIXED, s_unb
