"""The reference's fixed-sweep radiosity solve on the GPU (forward solve +
gs_steps natural-order Gauss-Seidel sweeps, src/cpp/illum_cli.cpp:425-433,
src/cpp/arma_util.cpp:4-17) against the CPU oracle's restatement of the same
order: bit for bit for the solve, within 1e-9 K for a thermal run."""
import numpy as np
import pytest

from illum_gb300 import meshgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c0_mesh():
    return meshgen.icosphere_craters(4, seed=0)          # 5,120 facets, 20 craters


def _ctx_with_F(ilg, v, f, nphi=32):
    ctx = ilg.IllumContext(v, f)
    ctx.make_horizons(nphi=nphi)
    ctx.set_insolation(1, 0, 1361.0)
    csr = ctx.compute_F(albedo=0.1)
    return ctx, csr


@pytest.mark.parametrize("gs_steps", [0, 1, 3])
def test_fixed_sweeps_bit_exact(ilg, oracle_mod, c0_mesh, gs_steps):
    v, f = c0_mesh
    ctx, (rp, col, val) = _ctx_with_F(ilg, v, f)
    disk = ilg.fib_spiral(100)
    sun = meshgen.spin_sun_positions(3, 6 * 3600.0, 2000.0)[2]
    E = ctx.get_direct_radiosity(sun, disk)
    x, res = ctx.radiosity_solve_gs(E, gs_steps)
    xo, reso, sweeps = oracle_mod.gauss_seidel(rp, col, val, E, mode=0, gs_steps=gs_steps)
    assert sweeps == 1 + gs_steps
    assert np.array_equal(x, xo)
    assert res == reso
    assert 1 < ctx.radiosity_levels() < f.shape[0]
    # more sweeps reduce the residual (albedo-scaled F: a contraction)
    if gs_steps:
        _, res0 = ctx.radiosity_solve_gs(E, 0)
        assert res < res0


def test_fixed_sweeps_with_diagonal_entries(ilg, oracle_mod):
    """A user matrix with diagonal entries (set_F): L's diagonal 1 - F_ii
    divides, U includes F_ii, as Armadillo's trimatl / trimatu do."""
    v, f = meshgen.icosphere_craters(3, seed=3, n_craters=12, dmin_m=150.0, dmax_m=450.0)
    ctx, (rp, col, val) = _ctx_with_F(ilg, v, f, nphi=16)
    n = f.shape[0]
    rows = np.repeat(np.arange(n), np.diff(rp))
    r2 = np.concatenate([rows, np.arange(0, n, 7)])
    c2 = np.concatenate([col, np.arange(0, n, 7)]).astype(np.int32)
    x2 = np.concatenate([val, np.full(len(range(0, n, 7)), 0.05)])
    rp3, c3, x3 = oracle_mod.coo_to_csr(n, r2, c2, x2)
    ctx.set_F(rp3, c3, x3)
    E = np.random.default_rng(2).uniform(0.0, 600.0, n)
    x, res = ctx.radiosity_solve_gs(E, 2)
    xo, reso, _ = oracle_mod.gauss_seidel(rp3, c3, x3, E, mode=0, gs_steps=2)
    assert np.array_equal(x, xo) and res == reso


def test_fixed_sweep_run_vs_oracle(ilg, oracle_mod, c0_mesh):
    """The fused FP64 steps in the fixed-sweep mode (gs_steps = 1, the
    reference's default) against the oracle's loop with the same solve:
    temperatures within 1e-9 K, radiosity averages within 1e-8."""
    v, f = c0_mesh
    ctx, csr = _ctx_with_F(ilg, v, f)
    nsteps, period, spr = 40, 6 * 3600.0, 360
    dt = period / spr
    suns = meshgen.spin_sun_positions(nsteps, period, dt)
    disk = ilg.fib_spiral(100)
    ctx.set_suns(suns, disk)
    z = meshgen.geometric_depths(40)
    ti, rhoc = np.full(40, 300.0), np.full(40, 1.05e6)
    tm = ilg.ThermalModel(ctx, z, 300.0, 1.05e6, 200.0, emissivity=0.95, bc_mode=ilg.BC_NEWTON)
    ctx.set_radiosity_mode(ilg.RAD_GS, 1)
    for coupling in (ilg.COUPLE_DIRECT,):
        opts = ilg.RunOpts(dt=dt, tol=0.0, max_sweeps=1, use_radiosity=1, use_graph=1, precision=ilg.PREC_FP64,
                           coupling=coupling)
        hist = ctx.run_steps(opts, 0, nsteps, record_tsurf=True)
        st = oracle_mod.thermal_run(v, f, ctx.horizons.T, suns, disk, csr, z, ti, rhoc, dt=dt, T0=200.0, emiss=0.95,
                                    solar_const=1361.0, norm_mode=1, bc_mode=1, rad_mode=0, gs_steps=1,
                                    record_tsurf=True, coupling=coupling)
        assert np.abs(hist - st["tsurf_hist"]).max() <= 1e-9
        assert np.abs(tm.T - st["T"].T).max() <= 1e-9
        out = ctx.outputs()
        assert np.abs(out["rad"] - st["rad"]).max() <= 1e-8 * max(1.0, np.abs(st["rad"]).max())


def test_fixed_sweep_mode_limits(ilg, c0_mesh):
    """FP64 single contexts only: mixed precision and batches refuse it."""
    v, f = c0_mesh
    ctx, _ = _ctx_with_F(ilg, v, f, nphi=16)
    suns = meshgen.spin_sun_positions(4, 6 * 3600.0, 60.0)
    ctx.set_suns(suns, ilg.fib_spiral(100))
    ilg.ThermalModel(ctx, meshgen.geometric_depths(20), 300.0, 1.05e6, 200.0, bc_mode=ilg.BC_NEWTON,
                     precision=ilg.PREC_MIXED)
    ctx.set_radiosity_mode(ilg.RAD_GS, 1)
    mixed = ilg.RunOpts(dt=60.0, tol=1e-3, max_sweeps=1, use_radiosity=1, use_graph=1, precision=ilg.PREC_MIXED,
                        coupling=ilg.COUPLE_DIRECT)
    with pytest.raises(ilg.IlgError, match="FP64"):
        ctx.run_steps(mixed, 0, 1)
    with pytest.raises(ilg.IlgError, match="single contexts"):
        ilg.Batch([ctx], [mixed])
    with pytest.raises(ilg.IlgError):
        ctx.set_radiosity_mode(7, 1)
