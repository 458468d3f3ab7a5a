"""Bounded device waits: the radiosity solver's grid barrier gives up after
its poll limit, records the failure, and the call reports ILG_ERR_DEVICE
while the context stays usable. The wait is made to run out by a barrier
that expects one more block than the launch has (nothing else faults or
hangs), with the limit shrunk to a few thousand polls."""
import time

import numpy as np
import pytest

from illum_gb300 import meshgen

pytestmark = pytest.mark.gpu


def test_grid_barrier_wait_runs_out(ilg, oracle_mod):
    v, f = meshgen.icosphere_craters(3, seed=3, n_craters=12, dmin_m=150.0, dmax_m=450.0)
    ctx = ilg.IllumContext(v, f)
    rp, col, val = ctx.compute_F(albedo=0.1)
    t0 = time.perf_counter()
    rc = ctx.debug_barrier_timeout(blocks=4, polls=4096, unreachable=True)
    elapsed = time.perf_counter() - t0
    assert rc == -6, rc                                  # ILG_ERR_DEVICE
    assert "grid barrier" in ilg.lib().ilg_last_error().decode()
    assert elapsed < 5.0
    # a barrier that can open passes with the same small limit
    assert ctx.debug_barrier_timeout(blocks=4, polls=4096, unreachable=False) == 0
    # the context still answers: a full solve afterwards, at the standard limit
    E = np.random.default_rng(1).uniform(0.0, 500.0, f.shape[0])
    x, res, sweeps = ctx.radiosity_solve(E, tol=1e-10, max_sweeps=200)
    xo, _, _ = oracle_mod.gauss_seidel(rp, col, val, E, mode=1, tol=1e-12, max_sweeps=500)
    assert res <= 1e-10 and np.abs(x - xo).max() <= 1e-9
