"""Seeded synthetic shape models and sun/thermal set-ups.

The reference reads Vesta/Ceres OBJ files and sun-position files from a
``data/`` directory that it does not ship (src/cpp/CMakeLists.txt:65-69,
src/sh/runjob.sh:4-9). These generators stand in for them with the shapes,
sizes and value distributions of the benchmark configurations:

* ``icosphere_craters``: icosphere of a given subdivision level, radial
  Gaussian field smoothed over 2-ring neighbours, spherical-cap craters.
* ``heightmap_terrain``: square fBm heightmap patch with power-law bowls.
* ``spin_sun_positions``: sun positions (km, body frame) for a body spinning
  about +z with a given period and sub-solar latitude.
* ``geometric_depths``: the conduction grid z_k = dz1 (q^k - 1)/(q - 1).

All randomness comes from a counter-based generator (SplitMix64 applied to
``seed * 2^32 + stream * 2^24 + counter``), so every draw is reproducible
from its seed alone. Lengths of meshes are in km (the reference's mesh unit,
src/cpp/illum_cli.cpp mesh_unit default), vertices float32, faces int32,
wound counter-clockwise seen from outside (normals point out / up).
"""
from __future__ import annotations

import numpy as np

AU_KM = 149.5978707e6

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """n uniform doubles in [0, 1) for (seed, stream)."""
    base = np.uint64((seed & 0xFFFFFFFF) << 32) + np.uint64((stream & 0xFF) << 24)
    ctr = np.arange(n, dtype=np.uint64) + base
    z = _splitmix64(ctr)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    """n standard normal draws (Box-Muller on two uniform streams)."""
    u1 = uniform(seed, stream, n)
    u2 = uniform(seed, stream + 128, n)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)


# ----------------------------------------------------------------- icosphere
def icosphere(level: int):
    """Unit icosphere: (verts float64 [V,3], faces int64 [F,3]), F = 20*4^level."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(level):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (nv + 1) + e[:, 1]
        uk, inv = np.unique(key, return_inverse=True)
        a = uk // (nv + 1)
        b = uk % (nv + 1)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid])
        m = inv.reshape(3, -1).T + nv          # midpoints of edges (01, 12, 20)
        m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], 1),
            np.stack([f[:, 1], m12, m01], 1),
            np.stack([f[:, 2], m20, m12], 1),
            np.stack([m01, m12, m20], 1)])
    # wind every face counter-clockwise seen from outside
    c = v[f].mean(axis=1)
    nrm = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    flip = (nrm * c).sum(1) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v, f


_ICO_CACHE: dict = {}


def _icosphere_cached(level: int):
    """icosphere(level) and the 2-ring smoothing operator of its vertices,
    built once per level (the generators copy what they modify)."""
    if level not in _ICO_CACHE:
        v, f = icosphere(level)
        _ICO_CACHE[level] = (v, f, None)
    return _ICO_CACHE[level]


def _two_ring(level: int):
    v, f, A2 = _icosphere_cached(level)
    if A2 is None:
        A = _vertex_adjacency(v.shape[0], f)
        A2 = (A @ A)
        A2.data[:] = 1.0
        _ICO_CACHE[level] = (v, f, A2)
    return A2


def _vertex_adjacency(nv: int, f: np.ndarray):
    import scipy.sparse as sp
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    rows = np.concatenate([e[:, 0], e[:, 1], np.arange(nv)])
    cols = np.concatenate([e[:, 1], e[:, 0], np.arange(nv)])
    A = sp.csr_matrix((np.ones(rows.size), (rows, cols)), shape=(nv, nv))
    A.data[:] = 1.0
    return A


def icosphere_craters(level: int, seed: int, radius_m: float = 1000.0, sigma_m: float = 15.0,
                      n_craters: int = 20, dmin_m: float = 80.0, dmax_m: float = 300.0,
                      depth_ratio: float = 0.2):
    """Icosphere + smoothed Gaussian radial field + spherical-cap craters.

    Returns (verts float32 [V,3] in km, faces int32 [F,3])."""
    v, f, _ = _icosphere_cached(level)
    nv = v.shape[0]
    if sigma_m != 0.0:
        g = normal(seed, 1, nv)
        A2 = _two_ring(level)
        deg = np.asarray(A2.sum(axis=1)).ravel()
        h = (A2 @ g) / deg
        h = h - h.mean()
        sd = h.std()
        if sd > 0:
            h *= sigma_m / sd
        r = radius_m + h
    else:
        r = np.full(nv, radius_m)
    if n_craters > 0:
        cu = uniform(seed, 2, n_craters)
        cv = uniform(seed, 3, n_craters)
        cd = uniform(seed, 4, n_craters)
        cz = 2.0 * cu - 1.0
        cphi = 2.0 * np.pi * cv
        cs = np.sqrt(np.maximum(0.0, 1.0 - cz * cz))
        centres = np.stack([cs * np.cos(cphi), cs * np.sin(cphi), cz], 1)
        diam = dmin_m + (dmax_m - dmin_m) * cd
        for k in range(n_craters):
            D = diam[k]
            d = depth_ratio * D
            Rc = ((D / 2.0) ** 2 + d * d) / (2.0 * d)
            ang = np.arccos(np.clip(v @ centres[k], -1.0, 1.0))
            s = radius_m * ang
            inside = s < D / 2.0
            x = s[inside]
            r[inside] -= np.sqrt(Rc * Rc - x * x) - (Rc - d)
    verts = (v * r[:, None]) / 1000.0
    return verts.astype(np.float32), f.astype(np.int32)


# ----------------------------------------------------------------- terrain
def heightmap_terrain(n: int = 1024, spacing_m: float = 2.0, seed: int = 7, hurst: float = 0.8,
                      rms_m: float = 25.0, n_bowls: int = 2000, dmin_m: float = 10.0,
                      dmax_m: float = 400.0, bowl_index: float = -3.0, depth_ratio: float = 0.2):
    """n x n fBm heightmap (spectral synthesis, Hurst exponent H, given RMS)
    with power-law bowls; 2 (n-1)^2 triangles. Returns (verts km, faces)."""
    kx = np.fft.fftfreq(n)
    k = np.sqrt(kx[:, None] ** 2 + kx[None, :] ** 2)
    k[0, 0] = 1.0
    amp = k ** (-(hurst + 1.0))
    amp[0, 0] = 0.0
    ph = 2.0 * np.pi * uniform(seed, 1, n * n).reshape(n, n)
    gn = normal(seed, 2, n * n).reshape(n, n)
    z = np.real(np.fft.ifft2(amp * gn * np.exp(1j * ph)))
    z -= z.mean()
    z *= rms_m / z.std()
    xs = np.arange(n) * spacing_m
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    if n_bowls > 0:
        u = uniform(seed, 3, n_bowls)
        a = bowl_index + 1.0
        D = (dmin_m ** a + u * (dmax_m ** a - dmin_m ** a)) ** (1.0 / a)
        cx = uniform(seed, 4, n_bowls) * xs[-1]
        cy = uniform(seed, 5, n_bowls) * xs[-1]
        for b in range(n_bowls):
            d = depth_ratio * D[b]
            Rc = ((D[b] / 2.0) ** 2 + d * d) / (2.0 * d)
            i0 = max(0, int((cx[b] - D[b]) / spacing_m)); i1 = min(n, int((cx[b] + D[b]) / spacing_m) + 2)
            j0 = max(0, int((cy[b] - D[b]) / spacing_m)); j1 = min(n, int((cy[b] + D[b]) / spacing_m) + 2)
            s = np.hypot(X[i0:i1, j0:j1] - cx[b], Y[i0:i1, j0:j1] - cy[b])
            m = s < D[b] / 2.0
            zz = z[i0:i1, j0:j1]
            zz[m] -= np.sqrt(Rc * Rc - s[m] ** 2) - (Rc - d)
    verts = np.stack([X.ravel(), Y.ravel(), z.ravel()], 1) / 1000.0
    idx = np.arange(n * n).reshape(n, n)
    a = idx[:-1, :-1].ravel(); b = idx[1:, :-1].ravel(); c = idx[1:, 1:].ravel(); d = idx[:-1, 1:].ravel()
    faces = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)])
    return verts.astype(np.float32), faces.astype(np.int32)


# ----------------------------------------------------------------- sun / thermal
def spin_sun_positions(nsteps: int, period_s: float, dt_s: float, subsolar_lat_deg: float = 10.0,
                       distance_au: float = 1.5, t0_s: float = 0.0) -> np.ndarray:
    """Sun positions in km in the body frame of a body spinning about +z.
    Returns [nsteps, 3] float64; step s is at time t0 + s*dt."""
    t = t0_s + dt_s * np.arange(nsteps)
    w = -2.0 * np.pi * t / period_s
    lat = np.deg2rad(subsolar_lat_deg)
    d = distance_au * AU_KM
    return np.stack([d * np.cos(lat) * np.cos(w), d * np.cos(lat) * np.sin(w),
                     np.full(nsteps, d * np.sin(lat))], 1)


def site_sun_positions(nsteps: int, period_s: float, dt_s: float, site_lat_deg: float = 0.0,
                       subsolar_lat_deg: float = 10.0, distance_au: float = 1.5, t0_s: float = 0.0) -> np.ndarray:
    """Sun positions in km in the local frame of a surface patch (x east,
    y north, z up) at latitude site_lat_deg on a body spinning with the given
    period; the sun crosses the meridian at t = 0. Returns [nsteps, 3]."""
    t = t0_s + dt_s * np.arange(nsteps)
    h = 2.0 * np.pi * t / period_s
    dec = np.deg2rad(subsolar_lat_deg)
    phi = np.deg2rad(site_lat_deg)
    d = distance_au * AU_KM
    east = -np.cos(dec) * np.sin(h)
    north = np.cos(phi) * np.sin(dec) - np.sin(phi) * np.cos(dec) * np.cos(h)
    up = np.sin(phi) * np.sin(dec) + np.cos(phi) * np.cos(dec) * np.cos(h)
    return d * np.stack([east, north, up], 1)


def geometric_depths(nz: int, zmax_m: float = 0.5, ratio: float = 1.1) -> np.ndarray:
    """Layer depths z_1..z_nz (m) with z_k = dz1 (ratio^k - 1)/(ratio - 1), z_nz = zmax."""
    kk = np.arange(1, nz + 1, dtype=np.float64)
    dz1 = zmax_m * (ratio - 1.0) / (ratio ** nz - 1.0)
    return dz1 * (ratio ** kk - 1.0) / (ratio - 1.0)


def load_obj(path: str, shape_index: int = 0, scale: float = 0.01):
    """Triangles of one OBJ shape as the reference ingests them
    (src/cpp/obj_util.cpp:9-96): faces in file order (polygons fan-split),
    vertices multiplied by `scale` (the reference divides by 100), and each
    face normal normalise((v1-v0) x (v2-v0)) flipped when it disagrees with
    the sum of the three vertex normals. Like the reference, vertex normals
    are looked up by vertex index. Returns (verts float32 n x 3, faces int32
    m x 3, normals float32 m x 3) for IllumContext(verts, faces, normals)."""
    V, N, shapes = [], [], [[]]
    with open(path) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "v":
                V.append([float(x) for x in t[1:4]])
            elif t[0] == "vn":
                N.append([float(x) for x in t[1:4]])
            elif t[0] in ("o", "g") and shapes[-1]:
                shapes.append([])
            elif t[0] == "f":
                idx = []
                for tok in t[1:]:
                    k = int(tok.split("/")[0])
                    idx.append(k - 1 if k > 0 else len(V) + k)
                for j in range(1, len(idx) - 1):
                    shapes[-1].append((idx[0], idx[j], idx[j + 1]))
    shapes = [s for s in shapes if s]
    if shape_index >= len(shapes):
        raise ValueError(f"{path} has {len(shapes)} shapes")
    F = np.asarray(shapes[shape_index], np.int64)
    V = np.asarray(V, np.float32)
    v0, v1, v2 = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    n = np.cross(v1 - v0, v2 - v0).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True).astype(np.float32)
    if N:
        Nv = np.asarray(N, np.float32)
        if Nv.shape[0] < V.shape[0]:
            raise ValueError("vertex normals are looked up by vertex index and there are fewer of them")
        s = Nv[F[:, 0]] + Nv[F[:, 1]] + Nv[F[:, 2]]
        flip = np.sum(n * s, axis=1) < 0
        n[flip] = -n[flip]
    Vs = (V * np.float32(scale)).astype(np.float32)
    return Vs, F.astype(np.int32), n
