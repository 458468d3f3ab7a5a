"""Batched stepping (many meshes, one launch per phase): every member's
result is bitwise the same as when it runs alone."""
import numpy as np
import pytest

from illum_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _member(ilg, level, seed, nz, period_h, nsteps, precision, coupling=1, ti=300.0):
    v, f = meshgen.icosphere_craters(level, seed=seed, n_craters=10, dmin_m=120.0, dmax_m=400.0)
    ctx = ilg.IllumContext(v, f)
    ctx.make_horizons(nphi=16)
    ctx.set_insolation(1, 0, 1361.0)
    ctx.compute_F(albedo=0.1)
    dt = period_h * 3600.0 / 360
    ctx.set_suns(meshgen.spin_sun_positions(nsteps, period_h * 3600.0, dt), ilg.fib_spiral(100))
    tm = ilg.ThermalModel(ctx, meshgen.geometric_depths(nz), ti, 1.05e6, 210.0, emissivity=0.95,
                          bc_mode=ilg.BC_NEWTON, precision=precision)
    opts = ilg.RunOpts(dt=dt, tol=1e-10, max_sweeps=200, use_radiosity=1, use_graph=1, precision=precision,
                       coupling=coupling)
    return ctx, tm, opts, nsteps


@pytest.mark.parametrize("precision,refine_every", [(0, 0), (1, 0), (1, 3)])
def test_batch_members_equal_alone(ilg, precision, refine_every):
    """refine_every = 3: one pass per step, the f32 form factors on every
    third step of each member (its own count, from its first step)."""
    specs = [(3, 11, 20, 4.0, 30), (2, 12, 35, 7.0, 18), (3, 13, 50, 2.5, 24)]
    alone = []
    for sp in specs:
        ctx, tm, opts, n = _member(ilg, *sp, precision)
        opts.refine_every = refine_every
        h = ctx.run_steps(opts, 0, n, record_tsurf=True)
        alone.append((h[-1], tm.T, ctx.outputs()))
    mem = [_member(ilg, *sp, precision) for sp in specs]
    for m in mem:
        m[2].refine_every = refine_every
    b = ilg.Batch([m[0] for m in mem], [m[2] for m in mem])
    b.run(max(sp[4] for sp in specs))
    act, done, _ = b.status()
    assert list(done) == [sp[4] for sp in specs] and not act.any()
    b.sync()
    for (ctx, tm, opts, n), (ts, T, outs) in zip(mem, alone):
        assert np.array_equal(tm.T, T)
        o = ctx.outputs()
        for k in ("rad", "rad_avg", "therm_avg", "therm_max"):
            assert np.array_equal(o[k], outs[k]), k


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_members_equal_alone_coarse_tiles(ilg, precision):
    """Members whose row tiles are cut for few blocks (the batch workloads'
    setting): the same bitwise alone and in the batch, and the solve agrees
    with the default tiling to the tolerance."""
    specs = [(3, 31, 20, 4.0, 16), (3, 32, 40, 6.0, 12)]
    alone = []
    for sp in specs:
        ctx, tm, opts, n = _member(ilg, *sp, precision)
        ctx.set_radiosity_blocks(2)
        h = ctx.run_steps(opts, 0, n, record_tsurf=True)
        alone.append((tm.T, ctx.outputs()))
    mem = [_member(ilg, *sp, precision) for sp in specs]
    for m in mem:
        m[0].set_radiosity_blocks(2)
        assert m[0].F_info()["row_tiles"] <= 2 * 2 + 2
    b = ilg.Batch([m[0] for m in mem], [m[2] for m in mem])
    b.run(max(sp[4] for sp in specs))
    b.sync()
    for (ctx, tm, opts, n), (T, outs) in zip(mem, alone):
        assert np.array_equal(tm.T, T)
        assert np.array_equal(ctx.outputs()["rad"], outs["rad"])
    ctx, _, _, _ = _member(ilg, *specs[0], 0)
    E = np.random.default_rng(3).uniform(0.0, 900.0, ctx.num_faces)
    x0 = ctx.radiosity_solve(E, tol=1e-10)[0]
    ctx.set_radiosity_blocks(1)
    x1 = ctx.radiosity_solve(E, tol=1e-10)[0]
    assert np.abs(x1 - x0).max() <= 1e-9 * max(1.0, np.abs(x0).max())


def test_batch_member_switched_off(ilg):
    specs = [(2, 21, 20, 4.0, 20), (2, 22, 20, 4.0, 20)]
    mem = [_member(ilg, *sp, 0) for sp in specs]
    b = ilg.Batch([m[0] for m in mem], [m[2] for m in mem])
    b.run(5)
    b.set_active(1, False)
    b.run(5)
    act, done, _ = b.status()
    assert list(done) == [10, 5]
    ctx, tm, opts, n = _member(ilg, *specs[1], 0)
    h = ctx.run_steps(opts, 0, 5, record_tsurf=True)
    assert np.array_equal(b.tsurf(1), h[-1])


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_autotune_keeps_results(ilg, precision):
    """The batch's own direct-insolation shapes: supported ones, timed, and
    the members' results the same bit for bit with and without them."""
    specs = [(3, 41, 20, 4.0, 20), (2, 42, 35, 7.0, 14)]
    out = []
    for tune in (False, True):
        mem = [_member(ilg, *sp, precision) for sp in specs]
        b = ilg.Batch([m[0] for m in mem], [m[2] for m in mem])
        if tune:
            t = b.autotune()
            assert t["classify_threads"] in (128, 256, 512) and t["exact_facets"] in (4, 8, 16, 32)
            assert t["direct_us"] > 0
        b.run(max(sp[4] for sp in specs))
        b.sync()
        out.append([(m[1].T.copy(), m[0].outputs()["rad"].copy()) for m in mem])
        b.close()
    for (ta, ra), (tb, rb) in zip(*out):
        assert np.array_equal(ta, tb) and np.array_equal(ra, rb)
