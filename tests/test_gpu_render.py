"""Ray-cast map renderer (src/cpp/illum_renderer_cli.cpp:160-316): pixel
rays built as the reference builds them, one closest hit each."""
import math

import numpy as np
import pytest

from illum_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _ortho_rays(cen, az_deg, el_deg, w, h):
    """The orthographic camera of illum_renderer_cli.cpp:228-256, in the
    library's arithmetic (double set-up, float Vector3 per pixel)."""
    mx = my = mz = 0.0
    for q in cen:
        mx += float(q[0]); my += float(q[1]); mz += float(q[2])
    n = len(cen)
    mx /= n; my /= n; mz /= n
    r_model = 0.0
    for q in cen:
        r_model = max(r_model, math.sqrt((float(q[0]) - mx) ** 2 + (float(q[1]) - my) ** 2 + (float(q[2]) - mz) ** 2))
    rad = 1.1 * r_model
    az, el = az_deg * math.pi / 180.0, el_deg * math.pi / 180.0
    f = np.float32

    def sph(phi, theta, r):
        return [f(r * math.cos(phi) * math.sin(theta)), f(r * math.sin(phi) * math.sin(theta)), f(r * math.cos(theta))]

    p = sph(az, el, rad)
    up = sph(az, el - math.pi / 2, 1.0)
    pl = np.sqrt(f(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]), dtype=np.float32)
    e = [f(-p[0] / pl), f(-p[1] / pl), f(-p[2] / pl)]
    r = [f(e[1] * up[2] - e[2] * up[1]), f(e[2] * up[0] - e[0] * up[2]), f(e[0] * up[1] - e[1] * up[0])]
    c = [f(mx), f(my), f(mz)]
    pc = [f(p[k] + c[k]) for k in range(3)]
    orig = np.zeros((h, w, 3), np.float32)
    for i in range(h):
        ye = f((2.0 * (1.0 - i / (h - 1)) - 1.0) * rad)
        for j in range(w):
            xe = f((2.0 * j / (w - 1) - 1.0) * (w / h) * rad)
            orig[i, j] = [f(f(pc[k] + f(ye * up[k])) + f(xe * r[k])) for k in range(3)]
    dirs = np.broadcast_to(np.array(e, np.float32), orig.shape)
    return orig.reshape(-1, 3), np.ascontiguousarray(dirs.reshape(-1, 3))


def test_orthographic_pixels_equal_traced_rays(ilg, oracle_mod):
    v, f = meshgen.icosphere_craters(3, seed=2, n_craters=6, dmin_m=150.0, dmax_m=400.0)
    ctx = ilg.IllumContext(v, f)
    from illum_gb300 import render
    w, h = 48, 40
    idx = render.facet_image(ctx, "ortho", 30.0, 60.0, w, h)
    cen = oracle_mod.facet_geometry(v, f)[0]
    o, d = _ortho_rays(cen, 30.0, 60.0, w, h)
    hit, _ = ctx.trace(o, d)
    assert np.array_equal(idx.ravel(), hit)
    frac = (idx >= 0).mean()
    assert 0.3 < frac < 0.9          # the body's disk inside the frame


def test_equal_area_map_and_png(ilg, oracle_mod, tmp_path):
    """Every pixel sees the body. As in the reference, the map's polar angle
    is asin(2 (i+1)/(h+1) - 1) (illum_renderer_cli.cpp:263-266), so the
    cameras sit at z > 0 and the map shows the upper hemisphere."""
    v, f = meshgen.icosphere_craters(3, seed=2, n_craters=6, dmin_m=150.0, dmax_m=400.0)
    ctx = ilg.IllumContext(v, f)
    from illum_gb300 import render
    idx = render.facet_image(ctx, "eac", 0.0, 0.0, 64, 32)
    assert (idx >= 0).all()
    cen = oracle_mod.facet_geometry(v, f)[0]
    assert (cen[np.unique(idx), 2] > -0.05).all()
    assert len(np.unique(idx)) > 0.25 * f.shape[0]
    data = np.arange(f.shape[0], dtype=np.float64)
    img = render.render(ctx, data, "eac", 0.0, 0.0, 64, 32, cmap="grayscale")
    assert img.shape == (32, 64, 3)
    p = tmp_path / "m.png"
    render.write_png(str(p), img)
    assert np.array_equal(render.read_png(str(p)), img)
