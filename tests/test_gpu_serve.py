"""Serving loop: jobs admitted over time, co-batched, each result the same
as the job run alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("workers,min_rebuild_s,refine_every", [(1, 0.0, 4), (4, 0.25, 4), (4, 0.0, 0)])
def test_serving_results_equal_alone(ilg, workers, min_rebuild_s, refine_every):
    """Jobs built concurrently, finished members switched off in place and
    batches re-formed: every job's final surface temperature equals the
    job run alone, bitwise (the one-pass solve's reference travels with the
    job from batch to batch)."""
    from illum_gb300 import serve
    reqs = serve.request_stream(8, rate_hz=200.0, levels=(2, 3), rotations=(1, 2), steps_per_rot=(40, 60))
    srv = serve.Server(budget_bytes=int(2e9), chunk_steps=7, setup_workers=workers, min_rebuild_s=min_rebuild_s,
                       refine_every=refine_every)
    done = srv.run(reqs)
    assert len(done) == len(reqs) and srv.rebuilds >= 2
    assert sorted(j.req.rid for j in done) == list(range(len(reqs)))
    for j in done:
        alone = srv.build_job(j.req)
        h = alone.ctx.run_steps(alone.opts, 0, j.req.nsteps, record_tsurf=True)
        assert np.array_equal(h[-1], j.tsurf), j.req.rid


def test_admission_respects_budget(ilg):
    """Jobs reserve device memory before their set-up: a level's first job
    4x the a priori estimate (built alone), the later ones 1.5x the largest
    footprint measured at that level; each reservation is replaced by the
    measured footprint (context + batch copy) once the job is built. The
    reserved total never exceeds the budget."""
    from illum_gb300 import serve
    reqs = serve.request_stream(6, rate_hz=1000.0, levels=(3,), rotations=(1, 1), steps_per_rot=(30, 31))
    first = 4 * serve.footprint_bytes(3, 80, 32, ilg.PREC_MIXED)
    srv = serve.Server(budget_bytes=int(1.5 * first), chunk_steps=10, setup_workers=4)
    done = srv.run(reqs)
    st = srv.stats()
    assert len(done) == 6
    assert 3 in srv.per_facet                      # calibrated from a measured footprint
    assert st["max_reserved_bytes"] <= srv.budget
    assert st["measured_over_reserved"]["max"] <= 1.0
