"""Thermal records: the reference's per-step temperature statistics
(thermal.hpp:86-126) and the FP64 energy sums, reduced on the device,
against the same quantities computed on the host from the step's state;
deterministic, and a batch member records what it records alone."""
import numpy as np
import pytest

from illum_gb300 import meshgen

pytestmark = pytest.mark.gpu

SIGMA = 5.6704e-8     # the reference's value (conductionQ.f:39)


def _setup(ilg, precision, seed=4, nsteps=12):
    v, f = meshgen.icosphere_craters(3, seed=seed, n_craters=8, dmin_m=120.0, dmax_m=400.0)
    ctx = ilg.IllumContext(v, f)
    ctx.make_horizons(nphi=16)
    ctx.set_insolation(1, 0, 1361.0)
    ctx.compute_F(albedo=0.1)
    dt = 6 * 3600.0 / 360
    ctx.set_suns(meshgen.spin_sun_positions(nsteps, 6 * 3600.0, dt), ilg.fib_spiral(100))
    tm = ilg.ThermalModel(ctx, meshgen.geometric_depths(30), 300.0, 1.05e6, 220.0, emissivity=0.95,
                          bc_mode=ilg.BC_NEWTON, precision=precision)
    opts = ilg.RunOpts(dt=dt, tol=1e-10, max_sweeps=200, use_radiosity=1, use_graph=1, precision=precision,
                       coupling=1)
    return v, f, ctx, tm, opts


def _host_record(T, rad, Fs, area, emiss):
    Ts = T[0]
    row = []
    for X in (T.ravel(), Ts, T[-1]):
        row += [X.max(), X.min(), X.mean(), X.std(ddof=1)]
    row += [np.sum(area * rad), np.sum(area * emiss * SIGMA * Ts ** 4), np.sum(area * Fs)]
    return np.array(row)


@pytest.mark.parametrize("precision", [0, 1])
def test_records_match_host_statistics(ilg, oracle_mod, precision):
    v, f, ctx, tm, opts = _setup(ilg, precision)
    area = oracle_mod.facet_geometry(v, f)[3]
    ctx.record_thermal(12)
    expect = []
    for s in range(12):
        ctx.run_steps(opts, s, 1)
        T = tm.T                                # (nz + 1) x N, row 0 = surface
        expect.append(_host_record(T, ctx.outputs()["rad"], -tm.get_radiosity(), area, 0.95))
    rec = ctx.thermal_records()
    assert rec.shape == (12, 15)
    expect = np.array(expect)
    assert np.array_equal(rec[:, [0, 1, 4, 5, 8, 9]], expect[:, [0, 1, 4, 5, 8, 9]])      # extrema exactly
    assert np.allclose(rec[:, [2, 6, 10]], expect[:, [2, 6, 10]], rtol=1e-13, atol=0)     # means
    assert np.allclose(rec[:, [3, 7, 11]], expect[:, [3, 7, 11]], rtol=1e-9, atol=1e-12)  # sample std
    assert np.allclose(rec[:, 12:], expect[:, 12:], rtol=1e-12, atol=1e-18)               # energy sums


def test_records_deterministic_and_equal_in_batch(ilg):
    runs = []
    for _ in range(2):
        v, f, ctx, tm, opts = _setup(ilg, 0)
        ctx.record_thermal(10)
        ctx.run_steps(opts, 0, 10)
        runs.append(ctx.thermal_records())
    assert np.array_equal(runs[0], runs[1])
    a = _setup(ilg, 0)
    b = _setup(ilg, 0, seed=9)
    for m in (a, b):
        m[2].record_thermal(10)
    bt = ilg.Batch([a[2], b[2]], [a[4], b[4]])
    bt.run(10)
    bt.sync()
    assert np.array_equal(a[2].thermal_records(), runs[0])
    alone_b = _setup(ilg, 0, seed=9)
    alone_b[2].record_thermal(10)
    alone_b[2].run_steps(alone_b[4], 0, 10)
    assert np.array_equal(b[2].thermal_records(), alone_b[2].thermal_records())
