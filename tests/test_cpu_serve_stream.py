"""The serving loop's host logic that needs no GPU: the seeded request
stream (the C4 configuration's ranges, Poisson arrivals, the step-count
scale of a bounded sample) and the a priori footprint estimate."""
import numpy as np

import illum_gb300 as ig
from illum_gb300 import serve


def test_request_stream_ranges_and_determinism():
    a = serve.request_stream(400)
    b = serve.request_stream(400)
    assert [(r.level, r.nsteps, r.nz, r.ti, r.arrival) for r in a] == \
           [(r.level, r.nsteps, r.nz, r.ti, r.arrival) for r in b]
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0)
    # Poisson arrivals at 20/s: mean gap 50 ms (within a few percent on 400 draws)
    assert abs(np.diff(arr).mean() - 0.05) < 0.01
    assert {r.level for r in a} == {3, 4, 5, 6, 7}
    assert all(1 <= r.rotations <= 20 and 360 <= r.steps_per_rot <= 1440 for r in a)
    assert all(30 <= r.nz <= 80 and 50.0 <= r.ti <= 2000.0 and 2.0 <= r.period_h <= 12.0 for r in a)
    assert all(r.nsteps == r.rotations * r.steps_per_rot for r in a)


def test_request_stream_step_scale():
    full = serve.request_stream(50)
    small = serve.request_stream(50, step_scale=0.02)
    for f, s in zip(full, small):
        assert (f.level, f.nz, f.ti, f.arrival) == (s.level, s.nz, s.ti, s.arrival)
        assert s.nsteps == max(1, int(round(f.rotations * f.steps_per_rot * 0.02)))


def test_footprint_estimate_grows_with_size_and_precision():
    e = [serve.footprint_bytes(L, 60, 32, ig.PREC_MIXED) for L in (3, 4, 5, 6, 7)]
    assert all(b > 3.9 * a for a, b in zip(e, e[1:]))          # ~4x facets per level
    assert serve.footprint_bytes(5, 60, 32, ig.PREC_FP64) > serve.footprint_bytes(5, 60, 32, ig.PREC_MIXED)
    assert serve.footprint_bytes(5, 80, 32, ig.PREC_MIXED) > serve.footprint_bytes(5, 30, 32, ig.PREC_MIXED)
