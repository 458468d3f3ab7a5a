"""ctypes front-end of the CPU oracle (oracle.cpp). TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check and the CPU-baseline leg of the benchmark use
this module. Parity status: UNPINNED against the reference's own outputs
except for the Fibonacci spiral and the ARMA file format (see oracle.cpp).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < max(
            os.path.getmtime(os.path.join(_HERE, "oracle.cpp")),
            os.path.getmtime(os.path.join(_HERE, "..", "illum_gb300", "csrc", "geom.h"))):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB)
        _lib.orc_form_factors.restype = C.c_int64
        _lib.orc_last_visibility_rays.restype = C.c_int64
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def set_threads(n: int) -> None:
    lib().orc_set_threads(C.c_int(n))


def facet_geometry(verts, faces):
    verts = np.ascontiguousarray(verts, np.float32)
    faces = np.ascontiguousarray(faces, np.int32)
    nt = faces.shape[0]
    c = np.zeros((nt, 3), np.float32); n = np.zeros((nt, 3), np.float32)
    r = np.zeros(nt, np.float32); a = np.zeros(nt, np.float64)
    lib().orc_facet_geometry(_p(verts), _p(faces), C.c_int(nt), _p(c), _p(n), _p(r), _p(a))
    return c, n, r, a


def trace(verts, faces, orig, dirs, any_hit=False, brute=False):
    verts = np.ascontiguousarray(verts, np.float32)
    faces = np.ascontiguousarray(faces, np.int32)
    orig = np.ascontiguousarray(orig, np.float32)
    dirs = np.ascontiguousarray(dirs, np.float32)
    nr = orig.shape[0]
    hit = np.zeros(nr, np.int32); t = np.zeros(nr, np.float64)
    lib().orc_trace(_p(verts), _p(faces), C.c_int(faces.shape[0]), C.c_int(nr), _p(orig), _p(dirs),
                    C.c_int(int(any_hit)), C.c_int(int(brute)), _p(hit), _p(t))
    return hit, t


def form_factors(verts, faces, offset=1e-5, albedo=None, albedo_scalar=1.0, cutoff=0.0):
    """Returns (rows, cols, vals) in the reference's column-major order and the
    number of visibility rays cast. cutoff > 0 keeps only pairs whose
    centroids are at most that far apart (not in the reference)."""
    verts = np.ascontiguousarray(verts, np.float32)
    faces = np.ascontiguousarray(faces, np.int32)
    alb = None if albedo is None else np.ascontiguousarray(albedo, np.float64)
    L = lib()
    nnz = L.orc_form_factors(_p(verts), _p(faces), C.c_int(faces.shape[0]), C.c_double(offset), _p(alb),
                             C.c_double(albedo_scalar), C.c_double(cutoff), None, None, None)
    if nnz < 0:
        raise RuntimeError("computed a NaN form factor")
    rows = np.zeros(nnz, np.int32); cols = np.zeros(nnz, np.int32); vals = np.zeros(nnz, np.float64)
    L.orc_form_factors(None, None, C.c_int(0), C.c_double(0), None, C.c_double(0), C.c_double(0), _p(rows),
                       _p(cols), _p(vals))
    return rows, cols, vals, int(L.orc_last_visibility_rays())


def coo_to_csr(n, rows, cols, vals):
    order = np.lexsort((cols, rows))
    r = rows[order]; c = cols[order].astype(np.int32); v = vals[order]
    rowptr = np.zeros(n + 1, np.int64)
    np.add.at(rowptr, r + 1, 1)
    rowptr = np.cumsum(rowptr)
    return rowptr, c, v


def horizons(verts, faces, nphi, theta_eps=1e-3, offset=1e-5, horizon_mesh=None):
    """nt x nphi zenith angles; horizon_mesh = (verts, faces) of a separate
    mesh the rays are traced against (src/cpp/illum.cpp:333-349)."""
    verts = np.ascontiguousarray(verts, np.float32)
    faces = np.ascontiguousarray(faces, np.int32)
    nt = faces.shape[0]
    out = np.zeros((nt, nphi), np.float64)   # row f = column f of the nphi x N matrix
    if horizon_mesh is None:
        lib().orc_horizons(_p(verts), _p(faces), C.c_int(nt), C.c_int(nphi), C.c_double(theta_eps),
                           C.c_double(offset), _p(out))
    else:
        hv = np.ascontiguousarray(horizon_mesh[0], np.float32)
        hf = np.ascontiguousarray(horizon_mesh[1], np.int32)
        lib().orc_horizons_mesh(_p(verts), _p(faces), C.c_int(nt), _p(hv), _p(hf), C.c_int(hf.shape[0]),
                                C.c_int(nphi), C.c_double(theta_eps), C.c_double(offset), _p(out))
    return out


def fib_spiral(n=100):
    xy = np.zeros((2, n), np.float64)
    lib().orc_fib_spiral(_p(xy), C.c_int(n))
    return xy.T.copy()          # n x 2


class _normals:
    """Face normals for the oracle's direct insolation during a call (the
    OBJ reader's normals), or the computed ones when None."""

    def __init__(self, normals):
        self.n = None if normals is None else np.ascontiguousarray(normals, np.float32)

    def __enter__(self):
        lib().orc_set_normals(_p(self.n))

    def __exit__(self, *exc):
        lib().orc_set_normals(None)


def direct(verts, faces, hor, sun, disk_xy, norm_mode=0, interp=0, solar_const=1372.0, normals=None):
    verts = np.ascontiguousarray(verts, np.float32)
    faces = np.ascontiguousarray(faces, np.int32)
    hor = np.ascontiguousarray(hor, np.float64)
    nt, nphi = hor.shape
    sun = np.ascontiguousarray(sun, np.float64)
    dxy = np.ascontiguousarray(np.asarray(disk_xy, np.float64).T)   # column-major n x 2
    out = np.zeros(nt, np.float64); cnt = np.zeros(nt, np.int32)
    with _normals(normals):
        lib().orc_direct(_p(verts), _p(faces), C.c_int(nt), _p(hor), C.c_int(nphi), _p(sun), _p(dxy),
                         C.c_int(disk_xy.shape[0]), C.c_int(norm_mode), C.c_int(interp),
                         C.c_double(solar_const), _p(out), _p(cnt))
    return out, cnt


def gauss_seidel(rowptr, col, val, E, mode=1, gs_steps=1, tol=1e-10, max_sweeps=200):
    n = E.shape[0]
    x = np.zeros(n, np.float64); res = C.c_double(0)
    rowptr = np.ascontiguousarray(rowptr, np.int64); col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64); E = np.ascontiguousarray(E, np.float64)
    sw = lib().orc_gauss_seidel(C.c_int(n), _p(rowptr), _p(col), _p(val), _p(E), C.c_int(mode),
                                C.c_int(gs_steps), C.c_double(tol), C.c_int(max_sweeps), _p(x), C.byref(res))
    return x, res.value, sw


def conductionq(z, dt, Qn, Qnp1, T, ti, rhoc, emiss, Tsurf, Fgeo=0.0):
    T = np.array(T, np.float64)
    ts = C.c_double(Tsurf); fs = C.c_double(0)
    rc = lib().orc_conductionq(C.c_int(len(z)), _p(np.ascontiguousarray(z, np.float64)), C.c_double(dt),
                               C.c_double(Qn), C.c_double(Qnp1), _p(T), _p(np.ascontiguousarray(ti, np.float64)),
                               _p(np.ascontiguousarray(rhoc, np.float64)), C.c_double(emiss), C.byref(ts),
                               C.c_double(Fgeo), C.byref(fs))
    if rc:
        raise ZeroDivisionError("zero pivot")
    return T, ts.value, fs.value


def conductionq_newton(z, dt, Qnp1, T, ti, rhoc, emiss, Tsurf, Fgeo=0.0):
    T = np.array(T, np.float64)
    ts = C.c_double(Tsurf); fs = C.c_double(0); it = C.c_int(0)
    rc = lib().orc_conductionq_newton(C.c_int(len(z)), _p(np.ascontiguousarray(z, np.float64)), C.c_double(dt),
                                      C.c_double(Qnp1), _p(T), _p(np.ascontiguousarray(ti, np.float64)),
                                      _p(np.ascontiguousarray(rhoc, np.float64)), C.c_double(emiss),
                                      C.byref(ts), C.c_double(Fgeo), C.byref(fs), C.byref(it))
    if rc:
        raise ZeroDivisionError("zero pivot")
    return T, ts.value, fs.value, it.value


def conductiont(z, dt, T, Tsurf, Tsurfp1, ti, rhoc, Fgeo=0.0):
    T = np.array(T, np.float64)
    fs = C.c_double(0)
    rc = lib().orc_conductiont(C.c_int(len(z)), _p(np.ascontiguousarray(z, np.float64)), C.c_double(dt), _p(T),
                               C.c_double(Tsurf), C.c_double(Tsurfp1), _p(np.ascontiguousarray(ti, np.float64)),
                               _p(np.ascontiguousarray(rhoc, np.float64)), C.c_double(Fgeo), C.byref(fs))
    if rc:
        raise ZeroDivisionError("zero pivot")
    return T, fs.value


class RunParams(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nt", "nz", "nsteps", "nphi", "ndisk", "norm_mode", "interp", "bc_mode",
                                       "rad_mode", "gs_steps", "max_sweeps", "use_radiosity", "coupling")] + \
               [(n, C.c_double) for n in ("dt", "emiss", "solar_const", "tol", "Fgeo")]


def thermal_run(verts, faces, hor, suns, disk_xy, csr, z, ti, rhoc, *, dt, T0, emiss=0.999,
                solar_const=1372.0, norm_mode=0, interp=0, bc_mode=0, rad_mode=1, gs_steps=1,
                tol=1e-10, max_sweeps=200, state=None, frame0=0, record_tsurf=False, direct_all=None,
                coupling=0, normals=None):
    """Time-step loop of src/cpp/illum_cli.cpp:403-468. Returns a dict of the
    final state (T is (nz+1) x N column-major as a [N, nz+1] array).
    normals: face normals for the direct insolation (an OBJ's, as read by
    the reference), or None for the ones computed from the vertices."""
    verts = np.ascontiguousarray(verts, np.float32)
    faces = np.ascontiguousarray(faces, np.int32)
    nt = faces.shape[0]
    nz = len(z)
    hor = np.ascontiguousarray(hor, np.float64)
    suns = np.ascontiguousarray(suns, np.float64)
    nsteps = suns.shape[0] if direct_all is None else direct_all.shape[0]
    dxy = np.ascontiguousarray(np.asarray(disk_xy, np.float64).T)
    P = RunParams(nt=nt, nz=nz, nsteps=nsteps, nphi=hor.shape[1], ndisk=disk_xy.shape[0], norm_mode=norm_mode,
                  interp=interp, bc_mode=bc_mode, rad_mode=rad_mode, gs_steps=gs_steps, max_sweeps=max_sweeps,
                  use_radiosity=int(csr is not None), coupling=coupling, dt=dt, emiss=emiss, solar_const=solar_const, tol=tol, Fgeo=0.0)
    if state is None:
        state = dict(T=np.full((nt, nz + 1), T0, np.float64), Qprev=np.zeros(nt), Fsurf=np.zeros(nt),
                     rad=np.zeros(nt), rad_avg=np.zeros(nt), therm_avg=np.zeros(nt), therm_max=np.zeros(nt))
    else:
        state = {k: np.array(v) for k, v in state.items()}
    if csr is not None:
        rowptr, col, val = (np.ascontiguousarray(csr[0], np.int64), np.ascontiguousarray(csr[1], np.int32),
                            np.ascontiguousarray(csr[2], np.float64))
    else:
        rowptr = col = val = None
    hist = np.zeros((nsteps, nt), np.float64) if record_tsurf else None
    da = None if direct_all is None else np.ascontiguousarray(direct_all, np.float64)
    with _normals(normals):
        rc = lib().orc_thermal_run(C.byref(P), _p(verts), _p(faces), _p(hor), _p(suns), _p(dxy), _p(da),
                                   _p(rowptr), _p(col), _p(val), _p(np.ascontiguousarray(z, np.float64)),
                                   _p(np.ascontiguousarray(ti, np.float64)),
                                   _p(np.ascontiguousarray(rhoc, np.float64)), _p(state["T"]), _p(state["Qprev"]),
                                   _p(state["Fsurf"]), _p(state["rad"]), _p(state["rad_avg"]),
                                   _p(state["therm_avg"]), _p(state["therm_max"]), C.c_int(frame0), _p(hist))
    if rc:
        raise ZeroDivisionError("zero pivot in conduction")
    if record_tsurf:
        state["tsurf_hist"] = hist
    return state
