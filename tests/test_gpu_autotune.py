"""Launch-shape autotuner (ilg_autotune): it picks supported shapes, leaves
the context's state untouched, and no result depends on the shapes."""
import numpy as np
import pytest

from illum_gb300 import meshgen

pytestmark = pytest.mark.gpu

SHAPES = [(256, 8, 64), (128, 4, 32), (512, 32, 128), (256, 16, 128)]


def _model(ilg, precision, seed=3, nsteps=24):
    v, f = meshgen.icosphere_craters(4, seed=seed, n_craters=12, dmin_m=120.0, dmax_m=400.0)
    ctx = ilg.IllumContext(v, f)
    ctx.make_horizons(nphi=32)
    ctx.set_insolation(1, 0, 1361.0)
    ctx.compute_F(albedo=0.1)
    dt = 6 * 3600.0 / 360
    ctx.set_suns(meshgen.spin_sun_positions(nsteps, 6 * 3600.0, dt), ilg.fib_spiral(100))
    tm = ilg.ThermalModel(ctx, meshgen.geometric_depths(40), 300.0, 1.05e6, 220.0, emissivity=0.95,
                          bc_mode=ilg.BC_NEWTON, precision=precision)
    opts = ilg.RunOpts(dt=dt, tol=1e-10 if precision == 0 else 1e-3, max_sweeps=200 if precision == 0 else 2,
                       use_radiosity=1, use_graph=1, precision=precision, coupling=1)
    return ctx, tm, opts


@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_choice_and_state(ilg, precision):
    ctx, tm, opts = _model(ilg, precision)
    ctx.run_steps(opts, 0, 5)
    T0 = tm.T.copy()
    out0 = ctx.outputs()
    t = ctx.autotune(opts, first_sun=5)
    assert t["classify_threads"] in (128, 256, 512)
    assert t["exact_facets"] in (4, 8, 16, 32)
    assert t["conduct_threads"] in (32, 64, 128)
    assert t["direct_us"] > 0 and t["conduct_us"] > 0
    assert ctx.get_tune() == {k: t[k] for k in ("classify_threads", "exact_facets", "conduct_threads")}
    # the timing runs worked on copies: state and outputs are as before
    assert np.array_equal(tm.T, T0)
    out1 = ctx.outputs()
    for k in out0:
        assert np.array_equal(out0[k], out1[k]), k
    ctx.run_steps(opts, 5, 10)


@pytest.mark.parametrize("precision", [0, 1])
def test_results_do_not_depend_on_shapes(ilg, precision):
    runs = []
    for cb, nf, bs in SHAPES:
        ctx, tm, opts = _model(ilg, precision)
        ctx.set_tune(cb, nf, bs)
        h = ctx.run_steps(opts, 0, 24, record_tsurf=True)
        runs.append((h, tm.T.copy(), ctx.outputs()["rad"].copy()))
    for h, T, rad in runs[1:]:
        assert np.array_equal(h, runs[0][0])
        assert np.array_equal(T, runs[0][1])
        assert np.array_equal(rad, runs[0][2])


def test_unsupported_shape_is_rejected(ilg):
    ctx, tm, opts = _model(ilg, 0, nsteps=2)
    with pytest.raises(RuntimeError):
        ctx.set_tune(96, 8, 64)
