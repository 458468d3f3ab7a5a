"""Known-answer checks of the oracle's geometry that do not go through its
shared geometry header: horizons, sun-disk sample tests and form factors
recomputed here in numpy (float64, libm trigonometry) from the raw vertices,
following the reference's formulas (src/cpp/illum.cpp:100-119, 244-262,
274-324, 382-466). The oracle and the GPU share one header for these
formulas, so a restatement error there would be invisible to the GPU-vs-
oracle parity tests; these tests catch it."""
import math

import numpy as np
import pytest

from illum_gb300 import meshgen

SUN_RADIUS_KM = 695508.0     # src/cpp/constants.hpp:7-8
ONE_AU_KM = 149.5978707e6


# ---------------------------------------------------------------- helpers
def frames(verts, faces):
    """Centroid, unit normal, Frenet frame (b, t, n) of every facet in float64
    from the float32 vertices (src/cpp/illum.cpp:244-262)."""
    v = verts.astype(np.float64)
    v0, v1, v2 = v[faces[:, 0]], v[faces[:, 1]], v[faces[:, 2]]
    c = (v0 + v1 + v2) / 3.0
    n = np.cross(v1 - v0, v2 - v0)
    area = 0.5 * np.linalg.norm(n, axis=1)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    t = (v1 - v0) / np.linalg.norm(v1 - v0, axis=1, keepdims=True)
    b = np.cross(t, n)
    return c, n, t, b, area


def bowl_plane(n=161, spacing_m=1.0, D_m=120.0, depth_m=24.0):
    """Flat square patch with one spherical-cap bowl at its centre (km).
    Returns (verts, faces, height function of (x, y) in km)."""
    xs = np.arange(n) * spacing_m
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    c0 = xs[-1] / 2.0
    Rc = ((D_m / 2) ** 2 + depth_m ** 2) / (2 * depth_m)

    def height_m(x, y):
        s = np.hypot(x - c0, y - c0)
        z = np.zeros_like(s)
        m = s < D_m / 2
        z[m] = -(np.sqrt(Rc * Rc - s[m] ** 2) - (Rc - depth_m))
        return z

    Z = height_m(X, Y)
    verts = (np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1) / 1000.0).astype(np.float32)
    idx = np.arange(n * n).reshape(n, n)
    a = idx[:-1, :-1].ravel(); b = idx[1:, :-1].ravel(); c = idx[1:, 1:].ravel(); d = idx[:-1, 1:].ravel()
    faces = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)]).astype(np.int32)
    return verts, faces, (lambda xk, yk: height_m(xk * 1000.0, yk * 1000.0) / 1000.0), c0 / 1000.0, xs[-1] / 1000.0


def analytic_horizon(p, b, t, n, phi, height, extent, offset=1e-5):
    """Zenith angle (from the facet normal) of the horizon of the analytic
    surface seen from p + offset n in azimuth phi of the frame (b, t, n):
    the smallest zenith angle whose ray passes below the surface somewhere
    inside the patch, by bisection on a dense sampling of each ray."""
    o = p + offset * n
    ts = np.concatenate([np.linspace(1e-6, 0.01, 4000), np.linspace(0.01, 0.4, 8000)])

    def hits(th):
        d = math.sin(th) * (math.cos(phi) * b + math.sin(phi) * t) + math.cos(th) * n
        pts = o[None, :] + ts[:, None] * d[None, :]
        inside = (pts[:, 0] >= 0) & (pts[:, 0] <= extent) & (pts[:, 1] >= 0) & (pts[:, 1] <= extent)
        return bool(np.any(pts[inside, 2] < height(pts[inside, 0], pts[inside, 1])))

    lo, hi = 0.0, math.pi
    for _ in range(40):
        mid = 0.5 * (lo + hi)
        if hits(mid):
            hi = mid
        else:
            lo = mid
    return 0.5 * (lo + hi)


# ---------------------------------------------------------------- horizons
@pytest.mark.parametrize("where_m", [(0.3, 0.3), (25.3, 0.7), (-31.6, 18.2)])
def test_horizon_in_spherical_bowl(oracle_mod, where_m):
    """Horizons of facets on the floor and wall of a spherical-cap bowl
    (src/cpp/illum.cpp:274-324) against the analytic surface, azimuth by
    azimuth. The mesh's linear rim cuts the analytic corner by less than a
    few mrad at 1 m spacing; the bisection stops at 1e-4."""
    verts, faces, height, c0, extent = bowl_plane()
    c, n, t, b, _ = frames(verts, faces)
    target = np.array([c0 + where_m[0] / 1000.0, c0 + where_m[1] / 1000.0])
    f = int(np.argmin(np.hypot(c[:, 0] - target[0], c[:, 1] - target[1])))
    nphi = 12
    H = oracle_mod.horizons(verts, faces, nphi, theta_eps=1e-4)[f]
    phis = np.linspace(0.0, 2.0 * math.pi, nphi)
    exp = np.array([analytic_horizon(c[f], b[f], t[f], n[f], ph, height, extent) for ph in phis])
    assert np.abs(H - exp).max() < 0.012, (H, exp)
    # the horizon is not trivial: every azimuth sees the rim above the plane of the facet
    assert np.all(exp < math.pi / 2 - 0.1)


# ---------------------------------------------------------------- direct insolation
def sun_frame(Nv):
    """Deterministic disk tangent: the coordinate axis least aligned with N,
    projected onto N's orthogonal plane (the reference draws it at random,
    src/cpp/illum.cpp:405-407; any unit vector orthogonal to N gives the
    same disk up to a rotation)."""
    ax = np.abs(Nv)
    e = np.zeros(3)
    e[0 if (ax[0] <= ax[1] and ax[0] <= ax[2]) else (1 if ax[1] <= ax[2] else 2)] = 1.0
    T = e - Nv * np.dot(Nv, e)
    T /= np.linalg.norm(T)
    return T, np.cross(T, Nv)


def direct_numpy(verts, faces, H, sun, disk_xy, solar=1372.0):
    """src/cpp/illum.cpp:382-466 in numpy: per facet the lit count of the
    ndisk - 1 disk samples against its horizon and the flux. Returns
    (flux, count, margin): margin = smallest |theta - threshold| of the
    facet's samples (where libm and the oracle's own trigonometry could
    legitimately disagree)."""
    c, n, t, b, _ = frames(verts, faces)
    # the sun cosine uses the triangle's float normal (Vector3), normalised
    v32 = verts.astype(np.float32)
    e1 = v32[faces[:, 1]] - v32[faces[:, 0]]
    e2 = v32[faces[:, 2]] - v32[faces[:, 0]]
    n32 = np.cross(e1, e2).astype(np.float32)
    n32 = (n32 / np.linalg.norm(n32, axis=1, keepdims=True).astype(np.float32)).astype(np.float64)
    n32 /= np.linalg.norm(n32, axis=1, keepdims=True)
    nt, nphi = H.shape
    dphi = 2.0 * math.pi / (nphi - 1)
    S = np.asarray(sun, np.float64)
    flux = np.zeros(nt); cnt = np.zeros(nt, np.int64); margin = np.full(nt, np.inf)
    for f in range(nt):
        p = c[f]
        Nv = (S - p) / np.linalg.norm(S - p)
        T, B = sun_frame(Nv)
        for s in range(disk_xy.shape[0] - 1):
            q = S + SUN_RADIUS_KM * (disk_xy[s, 0] * T + disk_xy[s, 1] * B)
            w = q - p
            w /= np.linalg.norm(w)
            x, y, z = np.dot(b[f], w), np.dot(t[f], w), np.dot(n[f], w)
            th = math.acos(max(-1.0, min(1.0, z)))
            ph = math.atan2(y, x)
            if ph < 0:
                ph += 2.0 * math.pi
            k = min(int(math.floor(ph / dphi)), nphi - 1)
            tt = (ph - k * dphi) / dphi
            thr = H[f, k] + tt * dphi
            margin[f] = min(margin[f], abs(th - thr))
            cnt[f] += th < thr
        flux[f] = cnt[f] / (nphi - 1) * max(0.0, float(np.dot(Nv, n32[f]))) * solar * (ONE_AU_KM / np.linalg.norm(S)) ** 2
    return flux, cnt, margin


def test_lit_counts_against_numpy(oracle_mod):
    """Lit-sample counts and fluxes for synthetic horizons and several sun
    positions: the oracle's geometry header against numpy/libm. Samples
    within 1e-9 rad of a threshold may differ (own trigonometry vs libm);
    a facet with such a sample is skipped."""
    v, f = meshgen.icosphere_craters(2, seed=3, n_craters=4, dmin_m=200.0, dmax_m=400.0)
    nt = f.shape[0]
    rng = np.random.default_rng(11)
    nphi = 17
    H = rng.uniform(0.6, 1.6, size=(nt, nphi))
    disk = oracle_mod.fib_spiral(100)
    checked = 0
    for sun in meshgen.spin_sun_positions(5, 6 * 3600.0, 3000.0, 10.0, 1.5):
        flux_o, cnt_o = oracle_mod.direct(v, f, H, sun, disk, norm_mode=0, interp=0, solar_const=1372.0)
        flux_n, cnt_n, margin = direct_numpy(v, f, H, sun, disk)
        ok = margin > 1e-9
        assert np.array_equal(cnt_o[ok], cnt_n[ok])
        assert np.allclose(flux_o[ok], flux_n[ok], rtol=1e-12, atol=1e-9)
        checked += int(ok.sum())
        assert cnt_n.max() > 0 and cnt_n.min() < 99   # lit, partly lit and shadowed facets occur
    assert checked > 0.95 * 5 * nt


# ---------------------------------------------------------------- form factors
def test_form_factors_against_numpy(oracle_mod):
    """F_ij = max(0, n_i . n_ij) max(0, -n_j . n_ij) A_j / (pi r^2) x albedo_i
    with n_ij = (p_j - p_i)/r (src/cpp/illum.cpp:100-119, 225-234),
    recomputed in float64 from the raw vertices for every entry the oracle
    keeps on the 5,120-facet crater mesh. The reference forms p_ij and the
    dot products in float (Vector3), so agreement is to ~1e-6 relative."""
    v, f = meshgen.icosphere_craters(4, seed=0, n_craters=20, dmin_m=80.0, dmax_m=300.0)
    rows, cols, vals, _ = oracle_mod.form_factors(v, f, albedo_scalar=0.1)
    assert len(vals) > 10000
    c, n, t, b, area = frames(v, f)
    pij = c[cols] - c[rows]
    r = np.linalg.norm(pij, axis=1)
    nij = pij / r[:, None]
    mu_ij = np.maximum(0.0, np.sum(n[rows] * nij, 1))
    mu_ji = np.maximum(0.0, -np.sum(n[cols] * nij, 1))
    scale = area[cols] / (math.pi * r * r) * 0.1          # F with both cosines 1
    F = mu_ij * mu_ji * scale
    assert np.all(F > 0)
    # the float dot products are good to ~1e-7 absolute in each cosine, so
    # the error is bounded relative to the cosine-free scale, and relative to
    # F itself wherever the pair is not grazing
    assert (np.abs(vals - F) / scale).max() < 2e-6
    ok = mu_ij * mu_ji > 1e-3
    rel = np.abs(vals[ok] - F[ok]) / F[ok]
    assert ok.mean() > 0.75 and rel.max() < 1e-3 and np.median(rel) < 5e-6, (rel.max(), np.median(rel))


# ---------------------------------------------------------------- coupling
def test_reference_coupling_oscillates(oracle_mod):
    """The reference feeds the conducted surface flux of the previous step
    back as rad = -Fsurf + direct (src/cpp/illum_cli.cpp:411-421). With the
    thin top layer of the benchmark profiles that feedback makes the surface
    temperature zig-zag from step to step; E = direct (the coupling the
    benchmarks use) does not. Both stay bounded here."""
    v, f = meshgen.icosphere_craters(3, 0, n_craters=6, dmin_m=150.0, dmax_m=400.0)
    nt = f.shape[0]
    H = oracle_mod.horizons(v, f, 16)
    r, c, val, _ = oracle_mod.form_factors(v, f, albedo_scalar=0.1)
    csr = oracle_mod.coo_to_csr(nt, r, c, val)
    z = meshgen.geometric_depths(40)
    suns = meshgen.spin_sun_positions(180, 6 * 3600.0, 60.0)
    disk = oracle_mod.fib_spiral(100)
    flips = {}
    for coupling in (0, 1):
        st = oracle_mod.thermal_run(v, f, H, suns, disk, csr, z, np.full(40, 300.0), np.full(40, 1.05e6), dt=60.0,
                                    T0=200.0, emiss=0.95, bc_mode=1, rad_mode=1, tol=1e-10, coupling=coupling,
                                    record_tsurf=True, norm_mode=1, solar_const=1361.0)
        h = st["tsurf_hist"]
        assert np.all(np.isfinite(h)) and h.min() > 100.0 and h.max() < 400.0
        d = np.sign(np.diff(h, axis=0))
        flips[coupling] = int(np.count_nonzero(d[1:] * d[:-1] < 0))
    assert flips[0] > 10 * max(1, flips[1]), flips
