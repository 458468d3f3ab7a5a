"""The one-pass mixed solve's warm start (k_radiosity_lagged), restated in
numpy on a synthetic scattering matrix: one Jacobi sweep per step from
S(n) + F (E(n+1) - E(n)) tracks the exact solution about as well as a
refinement round (a residual and a correction sweep: two applications of F
per step), and far better than one sweep from the extrapolated start
2 S(n) - S(n-1) when facets cross the terminator (E jumps)."""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl


def _problem(n=600, nsteps=120, seed=4):
    rng = np.random.default_rng(seed)
    # a sparse non-negative matrix with row sums ~0.04 (albedo x visible fraction)
    F = sp.random(n, n, density=0.03, random_state=seed, data_rvs=rng.random).tocsr()
    F.setdiag(0.0)
    F.eliminate_zeros()
    F = sp.diags(0.04 / np.maximum(np.asarray(F.sum(1)).ravel(), 1e-30)) @ F
    # direct flux: a terminator sweeping over the facets (values jump 0 <-> ~1000)
    phase = rng.uniform(0, 2 * np.pi, n)
    t = np.linspace(0, 2 * np.pi, nsteps + 1)
    E = np.maximum(0.0, 1000.0 * np.cos(phase[None, :] - t[:, None]))
    E[E < 150.0] = 0.0
    return F.tocsr(), E


def _track(F, E, scheme):
    n = F.shape[0]
    lu = spl.splu((sp.identity(n) - F).tocsc())
    s_prev = np.zeros(n)
    s_pp = np.zeros(n)
    P = np.zeros(n)
    errs = []
    for k in range(E.shape[0] - 1):
        if k == 0:
            s0 = np.zeros(n)
        elif scheme == "predicted":
            s0 = s_prev + P
        elif k == 1:
            s0 = s_prev
        else:
            s0 = 2 * s_prev - s_pp
        x = E[k] + s0
        if scheme == "round":
            r = F @ x - s0
            s = s0 + r + F @ r
        else:
            s = F @ x
        if scheme == "predicted":
            P = F @ (E[k + 1] - E[k])
        exact = lu.solve(E[k]) - E[k]
        errs.append(np.abs(s - exact).max())
        s_pp, s_prev = s_prev, s
    return max(errs[3:])


def test_predicted_one_pass_tracks_like_a_refinement_round():
    F, E = _problem()
    e_round = _track(F, E, "round")
    e_pred = _track(F, E, "predicted")
    e_extra = _track(F, E, "extrapolated")
    assert e_pred <= 2.0 * e_round
    assert e_extra >= 10.0 * e_pred
