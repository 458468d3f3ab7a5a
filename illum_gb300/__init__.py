"""illum_gb300 — GB300-native illumination + thermal path (sm_103a CUDA).

Python front-end over the C ABI of include/illum_gb300.h (libillum_gb300.so,
built in-tree by ``illum_gb300._build``). The class and method names mirror
the reference's C++ API (sampotter/illum):

* ``IllumContext``  ~ ``illum_context`` (src/cpp/illum.hpp:6-48):
  ``compute_F``, ``make_horizons``, ``horizons``, ``get_direct_radiosity``;
* ``ThermalModel``  ~ ``thermal_model`` (src/cpp/thermal.hpp:7-127):
  ``step``, ``T``, ``get_radiosity``;
* ``fib_spiral``    ~ ``fib_spiral`` (src/cpp/illum.cpp:468-483);
* ``conductionQ``   ~ ``conductionQ`` (src/cpp/conduction.hpp:16-28).

There is no CPU fallback: importing works without a GPU, but every compute
call goes through the CUDA library and raises if it is missing or fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

__all__ = ["IllumContext", "ThermalModel", "Batch", "IlgError", "fib_spiral", "conductionQ", "conductionQ_batch", "lib",
           "library_path", "RunOpts", "Tune", "PREC_FP64", "PREC_MIXED", "BC_LINEARISED", "BC_NEWTON",
           "COUPLE_REFERENCE", "COUPLE_DIRECT", "RAD_TOL", "RAD_GS"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "libillum_gb300.so")

PREC_FP64, PREC_MIXED = 0, 1
BC_LINEARISED, BC_NEWTON = 0, 1
COUPLE_REFERENCE, COUPLE_DIRECT = 0, 1
RAD_TOL, RAD_GS = 0, 1

ERRORS = {-1: "ILG_ERR_ARG", -2: "ILG_ERR_CUDA", -3: "ILG_ERR_NAN", -4: "ILG_ERR_PIVOT", -5: "ILG_ERR_NOMEM",
          -6: "ILG_ERR_DEVICE", -7: "ILG_ERR_NOTCONV"}


class IlgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class RunOpts(C.Structure):
    _fields_ = [("dt", C.c_double), ("tol", C.c_double), ("max_sweeps", C.c_int), ("use_radiosity", C.c_int),
                ("use_graph", C.c_int), ("precision", C.c_int), ("coupling", C.c_int), ("refine_every", C.c_int),
                ("layer_rounding", C.c_int)]


class Tune(C.Structure):
    """Launch shapes of the step kernels (include/illum_gb300.h ilg_tune)."""
    _fields_ = [("classify_threads", C.c_int), ("exact_facets", C.c_int), ("conduct_threads", C.c_int),
                ("direct_us", C.c_double), ("conduct_us", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None

# (name, restype, argtypes) of every exported entry point
_SIGS = {
    "ilg_last_error": (C.c_char_p, []),
    "ilg_version": (C.c_int, []),
    "ilg_ctx_create": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_void_p)]),
    "ilg_ctx_destroy": (C.c_int, [C.c_void_p]),
    "ilg_ctx_num_faces": (C.c_int, [C.c_void_p]),
    "ilg_ctx_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int)]),
    "ilg_ctx_device_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "ilg_trace": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "ilg_compute_F": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.POINTER(C.c_int64),
                                C.POINTER(C.c_int64)]),
    "ilg_compute_F_cutoff": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "ilg_visibility_sample": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                        C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]),
    "ilg_get_F": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ilg_record_thermal": (C.c_int, [C.c_void_p, C.c_int]),
    "ilg_render": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.c_void_p]),
    "ilg_get_thermal_records": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]),
    "ilg_set_F": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ilg_F_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int),
                             C.POINTER(C.c_int)]),
    "ilg_device_pool_high": (C.c_int, [C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int]),
    "ilg_F_tiles": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]),
    "ilg_make_horizons": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double]),
    "ilg_make_horizons_mesh": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_double,
                                         C.c_double]),
    "ilg_get_horizons": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ilg_set_horizons": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "ilg_set_insolation": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double]),
    "ilg_fib_spiral": (None, [C.c_void_p, C.c_int]),
    "ilg_direct_radiosity": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "ilg_radiosity_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_void_p,
                                      C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "ilg_set_radiosity_blocks": (C.c_int, [C.c_void_p, C.c_int]),
    "ilg_radiosity_solve_gs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_double)]),
    "ilg_radiosity_levels": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "ilg_debug_barrier_timeout": (C.c_int, [C.c_void_p, C.c_int, C.c_longlong, C.c_int]),
    "ilg_debug_ff_chunk": (C.c_int, [C.c_longlong]),
    "ilg_set_radiosity_mode": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "ilg_thermal_init": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                                   C.c_double, C.c_double, C.c_int, C.c_int]),
    "ilg_thermal_step": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p]),
    "ilg_thermal_get": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ilg_set_suns": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int]),
    "ilg_run_steps": (C.c_int, [C.c_void_p, C.POINTER(RunOpts), C.c_int, C.c_int, C.c_void_p]),
    "ilg_run_steps_host": (C.c_int, [C.c_void_p, C.POINTER(RunOpts), C.c_int, C.c_void_p, C.c_void_p]),
    "ilg_bench_steps": (C.c_int, [C.c_void_p, C.POINTER(RunOpts), C.c_int, C.c_int, C.c_double, C.c_void_p,
                                  C.c_void_p]),
    "ilg_get_outputs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ilg_set_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "ilg_autotune": (C.c_int, [C.c_void_p, C.POINTER(RunOpts), C.c_int, C.POINTER(Tune)]),
    "ilg_set_tune": (C.c_int, [C.c_void_p, C.POINTER(Tune)]),
    "ilg_get_tune": (C.c_int, [C.c_void_p, C.POINTER(Tune)]),
    "ilg_get_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "ilg_batch_create": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_void_p)]),
    "ilg_batch_destroy": (C.c_int, [C.c_void_p]),
    "ilg_batch_run": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "ilg_batch_bench": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_void_p]),
    "ilg_batch_bench_phases": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_void_p]),
    "ilg_batch_autotune": (C.c_int, [C.c_void_p, C.POINTER(Tune)]),
    "ilg_batch_status": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ilg_batch_set_active": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "ilg_batch_get_tsurf": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "ilg_batch_sync": (C.c_int, [C.c_void_p]),
    "conductionq_": (None, [C.POINTER(C.c_int), C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                            C.POINTER(C.c_double), C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                            C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "conductiont_": (None, [C.POINTER(C.c_int), C.c_void_p, C.POINTER(C.c_double), C.c_void_p,
                            C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p, C.c_void_p,
                            C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ilg_conductionq_batch": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_double, C.c_void_p,
                                        C.c_int]),
    "ilg_conductionq_batch_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                                                C.c_double, C.c_void_p, C.c_int, C.c_void_p]),
}


def library_path() -> str:
    return _SO


def lib():
    """Load libillum_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_SO):
            raise ImportError(f"{_SO} is missing: build it with `python -m illum_gb300._build` "
                              "(or __graft_entry__.build())")
        L = C.CDLL(_SO)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int):
    if rc != 0:
        raise IlgError(rc, lib().ilg_last_error().decode())


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def fib_spiral(n: int = 100) -> np.ndarray:
    """n x 2 Fibonacci-spiral disk samples (src/cpp/illum.cpp:468-483)."""
    xy = np.zeros((2, n), np.float64)   # column-major n x 2
    lib().ilg_fib_spiral(_p(xy), n)
    return xy.T.copy()


class IllumContext:
    """Mesh + device-resident LBVH; mirrors illum_context."""

    def __init__(self, verts, faces, normals=None):
        self._verts = np.ascontiguousarray(verts, np.float32)
        self._faces = np.ascontiguousarray(faces, np.int32)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
        h = C.c_void_p()
        _check(lib().ilg_ctx_create(_p(self._verts), self._verts.shape[0], _p(self._faces), self._faces.shape[0],
                                    _p(nrm), C.byref(h)))
        self._h = h
        self.num_faces = self._faces.shape[0]
        self.nphi = 0
        self.nnz = 0
        self.visibility_rays = 0

    def close(self):
        if getattr(self, "_h", None):
            lib().ilg_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_num_faces(self) -> int:
        return self.num_faces

    def info(self):
        n = C.c_int64(); d = C.c_int()
        _check(lib().ilg_ctx_info(self._h, C.byref(n), C.byref(d)))
        return {"bvh_nodes": n.value, "bvh_depth": d.value}

    def device_bytes(self) -> int:
        """Device memory the context holds now (bytes)."""
        n = C.c_int64()
        _check(lib().ilg_ctx_device_bytes(self._h, C.byref(n)))
        return n.value

    # -- ray queries
    def trace(self, orig, dirs, any_hit=False):
        o = np.ascontiguousarray(orig, np.float32); d = np.ascontiguousarray(dirs, np.float32)
        n = o.shape[0]
        hit = np.zeros(n, np.int32); t = np.zeros(n, np.float64)
        _check(lib().ilg_trace(self._h, n, _p(o), _p(d), int(any_hit), _p(hit), _p(t)))
        return hit, t

    # -- form factors
    def compute_F(self, albedo=1.0, offset=1e-5, cutoff=None, fetch=True):
        """Returns the form-factor matrix as (rowptr, col, val) CSR by receiver
        row (None with fetch=False: it stays on the device). cutoff: keep
        only pairs whose centroids are at most this far apart."""
        alb = None
        scalar = 1.0
        if np.isscalar(albedo):
            scalar = float(albedo)
        else:
            alb = _f64(albedo)
        nnz = C.c_int64(); rays = C.c_int64()
        if cutoff is None:
            _check(lib().ilg_compute_F(self._h, _p(alb), scalar, offset, C.byref(nnz), C.byref(rays)))
        else:
            _check(lib().ilg_compute_F_cutoff(self._h, _p(alb), scalar, offset, float(cutoff), C.byref(nnz),
                                              C.byref(rays)))
        self.nnz = nnz.value
        self.visibility_rays = rays.value
        if not fetch:
            return None
        return self.get_F()

    def visibility_sample(self, sources, cutoff=None, radii=(), offset=1e-5):
        """Nonzero form-factor entries of the listed source columns (and of
        the sample within each radius) without building F; cutoff None: none."""
        src = np.ascontiguousarray(sources, np.int32)
        rad = np.ascontiguousarray(radii, np.float64)
        per = np.zeros(src.shape[0], np.int64)
        within = np.zeros(max(1, rad.shape[0]), np.int64)
        rays = C.c_int64()
        _check(lib().ilg_visibility_sample(self._h, 0.0 if cutoff is None else float(cutoff), offset, _p(src),
                                           src.shape[0], _p(rad) if rad.shape[0] else None, rad.shape[0], _p(per),
                                           _p(within), C.byref(rays)))
        return {"per_source": per, "within_radius": within[:rad.shape[0]], "rays": rays.value}

    def get_F(self):
        rowptr = np.zeros(self.num_faces + 1, np.int64)
        col = np.zeros(max(self.nnz, 1), np.int32); val = np.zeros(max(self.nnz, 1), np.float64)
        _check(lib().ilg_get_F(self._h, _p(rowptr), _p(col), _p(val)))
        return rowptr, col[:self.nnz], val[:self.nnz]

    def F_info(self):
        a, b = C.c_int64(), C.c_int64()
        c, d = C.c_int(), C.c_int()
        _check(lib().ilg_F_info(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return {"nnz": a.value, "stored_entries": b.value, "row_tiles": c.value, "active_rows": d.value}

    def F_tiles(self):
        """Per radiosity row tile: entries per thread, rows, halo facets."""
        n = C.c_int()
        _check(lib().ilg_F_tiles(self._h, 0, None, None, None, C.byref(n)))
        lam, rows, halo = (np.zeros(n.value, np.int32) for _ in range(3))
        _check(lib().ilg_F_tiles(self._h, n.value, _p(lam), _p(rows), _p(halo), C.byref(n)))
        return {"entries_per_thread": lam, "rows": rows, "halo": halo}

    def set_F(self, rowptr, col, val):
        rowptr = np.ascontiguousarray(rowptr, np.int64); col = np.ascontiguousarray(col, np.int32); val = _f64(val)
        _check(lib().ilg_set_F(self._h, val.shape[0], _p(rowptr), _p(col), _p(val)))
        self.nnz = val.shape[0]

    # -- horizons
    def set_horizon_mesh(self, verts, faces):
        """A separate mesh the horizon rays are cast against
        (illum_context::set_horizon_obj_file, src/cpp/illum.hpp:36-37);
        None clears it."""
        if verts is None:
            self._hmesh = None
        else:
            self._hmesh = (np.ascontiguousarray(verts, np.float32), np.ascontiguousarray(faces, np.int32))

    def make_horizons(self, nphi=361, theta_eps=1e-3, offset=1e-5):
        hm = getattr(self, "_hmesh", None)
        if hm is None:
            _check(lib().ilg_make_horizons(self._h, nphi, theta_eps, offset))
        else:
            v, f = hm
            _check(lib().ilg_make_horizons_mesh(self._h, _p(v), v.shape[0], _p(f), f.shape[0], nphi, theta_eps,
                                                offset))
        self.nphi = nphi

    @property
    def horizons(self) -> np.ndarray:
        """nphi x N (one column of zenith angles per facet)."""
        out = np.zeros((self.num_faces, self.nphi), np.float64)
        _check(lib().ilg_get_horizons(self._h, _p(out)))
        return out.T

    def set_horizons(self, H):
        """H: nphi x N."""
        H = np.asarray(H, np.float64)
        buf = np.ascontiguousarray(H.T)
        _check(lib().ilg_set_horizons(self._h, H.shape[0], _p(buf)))
        self.nphi = H.shape[0]

    # -- direct insolation
    def set_insolation(self, norm_mode=0, interp=0, solar_const=1372.0):
        _check(lib().ilg_set_insolation(self._h, norm_mode, interp, solar_const))

    def get_direct_radiosity(self, sun_position, disk_xy):
        s = _f64(sun_position).reshape(3)
        d = np.asarray(disk_xy, np.float64)
        dcm = np.ascontiguousarray(d.T)     # column-major n x 2
        out = np.zeros(self.num_faces, np.float64)
        _check(lib().ilg_direct_radiosity(self._h, _p(s), _p(dcm), d.shape[0], _p(out)))
        return out

    # -- radiosity
    def radiosity_solve(self, E, tol=1e-10, max_sweeps=200):
        E = _f64(E)
        x = np.zeros(self.num_faces, np.float64)
        res = C.c_double(); sw = C.c_int()
        _check(lib().ilg_radiosity_solve(self._h, _p(E), tol, max_sweeps, _p(x), C.byref(res), C.byref(sw)))
        return x, res.value, sw.value

    def set_radiosity_blocks(self, blocks: int):
        """Cut the radiosity row tiles for `blocks` blocks (0: all the device holds)."""
        _check(lib().ilg_set_radiosity_blocks(self._h, int(blocks)))

    def radiosity_solve_gs(self, E, gs_steps=1):
        """The reference's solve: forward solve + gs_steps natural-order
        Gauss-Seidel sweeps (src/cpp/illum_cli.cpp:425-433). Returns (x, res)."""
        E = _f64(E)
        x = np.zeros(self.num_faces, np.float64)
        res = C.c_double()
        _check(lib().ilg_radiosity_solve_gs(self._h, _p(E), int(gs_steps), _p(x), C.byref(res)))
        return x, res.value

    def debug_barrier_timeout(self, blocks=4, polls=4096, unreachable=True):
        """Status of one grid-barrier wait with a `polls` limit (test entry):
        0 when the barrier opened, ILG_ERR_DEVICE when the wait ran out."""
        return lib().ilg_debug_barrier_timeout(self._h, int(blocks), int(polls), int(bool(unreachable)))

    def radiosity_levels(self) -> int:
        n = C.c_int()
        _check(lib().ilg_radiosity_levels(self._h, C.byref(n)))
        return n.value

    def set_radiosity_mode(self, mode, gs_steps=1):
        """RAD_TOL: fused FP64 steps solve to the run's tolerance; RAD_GS:
        the reference's fixed sweeps (forward solve + gs_steps sweeps)."""
        _check(lib().ilg_set_radiosity_mode(self._h, int(mode), int(gs_steps)))

    # -- fused loop
    def set_suns(self, suns, disk_xy):
        s = _f64(suns).reshape(-1, 3)
        d = np.asarray(disk_xy, np.float64)
        dcm = np.ascontiguousarray(d.T)
        _check(lib().ilg_set_suns(self._h, s.shape[0], _p(s), _p(dcm), d.shape[0]))

    def run_steps(self, opts: RunOpts, first_sun: int, nsteps: int, record_tsurf=False):
        out = np.zeros((nsteps, self.num_faces), np.float64) if record_tsurf else None
        _check(lib().ilg_run_steps(self._h, C.byref(opts), first_sun, nsteps, _p(out)))
        return out

    def run_steps_host(self, opts: RunOpts, suns, record_tsurf=True):
        s = _f64(suns).reshape(-1, 3)
        out = np.zeros((s.shape[0], self.num_faces), np.float64) if record_tsurf else None
        _check(lib().ilg_run_steps_host(self._h, C.byref(opts), s.shape[0], _p(s), _p(out)))
        return out

    def bench_steps(self, opts: RunOpts, first_sun: int, nsteps: int, flush_mb=256.0):
        """Per-step device times (ms) with an L2 flush before each step; with
        opts.use_graph == 0 also the summed per-phase times."""
        ms = np.zeros(nsteps, np.float64)
        ph = np.zeros(3, np.float64)
        _check(lib().ilg_bench_steps(self._h, C.byref(opts), first_sun, nsteps, flush_mb, _p(ms), _p(ph)))
        return ms, {"direct": ph[0], "radiosity": ph[1], "conduction": ph[2]}

    def outputs(self):
        n = self.num_faces
        r, ra, ta, tm = (np.zeros(n) for _ in range(4))
        _check(lib().ilg_get_outputs(self._h, _p(r), _p(ra), _p(ta), _p(tm)))
        return {"rad": r, "rad_avg": ra, "therm_avg": ta, "therm_max": tm}

    RECORD_COLUMNS = ("Tmax", "Tmin", "Tavg", "Tstd", "Tmax_top", "Tmin_top", "Tavg_top", "Tstd_top",
                      "Tmax_bot", "Tmin_bot", "Tavg_bot", "Tstd_bot", "E_absorbed", "E_emitted", "E_conducted")

    def record_thermal(self, capacity: int):
        """Record per-step temperature statistics and FP64 energy sums for the
        next `capacity` steps (columns RECORD_COLUMNS); 0 stops."""
        _check(lib().ilg_record_thermal(self._h, int(capacity)))

    def thermal_records(self):
        n = C.c_int()
        _check(lib().ilg_get_thermal_records(self._h, None, C.byref(n)))
        out = np.zeros((n.value, 15), np.float64)
        if n.value:
            _check(lib().ilg_get_thermal_records(self._h, _p(out), C.byref(n)))
        return out

    def set_timing(self, enable=True):
        _check(lib().ilg_set_timing(self._h, int(enable)))

    def autotune(self, opts, first_sun=0):
        """Times every launch shape of the step kernels on this context's
        workload (its state is left as it was) and keeps the fastest;
        returns the chosen shapes and their measured times."""
        t = Tune()
        _check(lib().ilg_autotune(self._h, C.byref(opts), int(first_sun), C.byref(t)))
        return t.as_dict()

    def set_tune(self, classify_threads=256, exact_facets=8, conduct_threads=64):
        t = Tune(classify_threads, exact_facets, conduct_threads, 0.0, 0.0)
        _check(lib().ilg_set_tune(self._h, C.byref(t)))

    def get_tune(self):
        t = Tune()
        _check(lib().ilg_get_tune(self._h, C.byref(t)))
        return {k: v for k, v in t.as_dict().items() if not k.endswith("_us")}

    def stats(self):
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        amb, sw = C.c_int64(), C.c_int64()
        _check(lib().ilg_get_stats(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(amb), C.byref(sw)))
        return {"ms_direct": a.value, "ms_radiosity": b.value, "ms_conduction": c.value,
                "ambiguous_facets": amb.value, "radiosity_sweeps": sw.value}


class ThermalModel:
    """thermal_model on the device: T is (nz+1) x N (row 0 = surface)."""

    def __init__(self, ctx: IllumContext, depths, thermal_inertia, rhoc, init_temp, emissivity=0.999,
                 Fgeotherm=0.0, bc_mode=BC_LINEARISED, precision=PREC_FP64):
        z = _f64(depths)
        nz = z.shape[0]
        ti = _f64(np.broadcast_to(np.asarray(thermal_inertia, np.float64), (nz,)))
        rc = _f64(np.broadcast_to(np.asarray(rhoc, np.float64), (nz,)))
        full = None
        T0 = 0.0
        if np.isscalar(init_temp):
            T0 = float(init_temp)
        else:
            full = np.asarray(init_temp, np.float64)
            if full.shape != (nz + 1, ctx.num_faces):
                raise ValueError("initial temperature profile is an incompatible size")
            full = np.ascontiguousarray(full.T)
        self.ctx = ctx
        self.nz = nz
        self.t = 0.0
        _check(lib().ilg_thermal_init(ctx._h, nz, _p(z), _p(ti), _p(rc), T0, _p(full), emissivity, Fgeotherm,
                                      bc_mode, precision))

    def step(self, dt, Q):
        _check(lib().ilg_thermal_step(self.ctx._h, dt, _p(_f64(Q))))
        self.t += dt

    @property
    def T(self) -> np.ndarray:
        out = np.zeros((self.ctx.num_faces, self.nz + 1), np.float64)
        _check(lib().ilg_thermal_get(self.ctx._h, _p(out), None, None))
        return out.T

    def visibility_sample(self, sources, cutoff=None, radii=(), offset=1e-5):
        """Nonzero form-factor entries of the listed source columns (and of
        the sample within each radius) without building F; cutoff None: none."""
        src = np.ascontiguousarray(sources, np.int32)
        rad = np.ascontiguousarray(radii, np.float64)
        per = np.zeros(src.shape[0], np.int64)
        within = np.zeros(max(1, rad.shape[0]), np.int64)
        rays = C.c_int64()
        _check(lib().ilg_visibility_sample(self._h, 0.0 if cutoff is None else float(cutoff), offset, _p(src),
                                           src.shape[0], _p(rad) if rad.shape[0] else None, rad.shape[0], _p(per),
                                           _p(within), C.byref(rays)))
        return {"per_source": per, "within_radius": within[:rad.shape[0]], "rays": rays.value}

    def get_F(self):
        F = np.zeros(self.ctx.num_faces)
        _check(lib().ilg_thermal_get(self.ctx._h, None, _p(F), None))
        return F

    def get_radiosity(self):
        return -self.get_F()


class Batch:
    """Several contexts stepped together (ilg_batch_*): one launch per phase
    for all members; each member keeps its own RunOpts (same precision)."""

    def __init__(self, contexts, opts):
        self.contexts = list(contexts)
        n = len(self.contexts)
        arr = (RunOpts * n)(*opts)
        hs = (C.c_void_p * n)(*[c._h for c in self.contexts])
        h = C.c_void_p()
        _check(lib().ilg_batch_create(hs, n, arr, C.byref(h)))
        self._h = h
        self.n = n

    def close(self):
        if getattr(self, "_h", None):
            lib().ilg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, nsteps, use_graph=True):
        _check(lib().ilg_batch_run(self._h, nsteps, int(use_graph)))

    def bench(self, nsteps, flush_mb=256.0):
        ms = np.zeros(nsteps)
        _check(lib().ilg_batch_bench(self._h, nsteps, flush_mb, _p(ms)))
        return ms

    def bench_phases(self, nsteps, flush_mb=256.0):
        """Eager serial steps; returns (step_ms, [direct, radiosity, conduction] ms summed)."""
        ms = np.zeros(nsteps)
        ph = np.zeros(3)
        _check(lib().ilg_batch_bench_phases(self._h, nsteps, flush_mb, _p(ms), _p(ph)))
        return ms, ph

    def autotune(self):
        """Times every direct-insolation launch shape on the batch's own
        workload and keeps the fastest; returns the shapes and their time."""
        t = Tune()
        _check(lib().ilg_batch_autotune(self._h, C.byref(t)))
        return {k: v for k, v in t.as_dict().items() if k != "conduct_us"}

    def status(self):
        a = np.zeros(self.n, np.int32); d = np.zeros(self.n, np.int32); w = np.zeros(self.n, np.int32)
        _check(lib().ilg_batch_status(self._h, _p(a), _p(d), _p(w)))
        return a, d, w

    def set_active(self, member, active):
        _check(lib().ilg_batch_set_active(self._h, member, int(active)))

    def tsurf(self, member):
        out = np.zeros(self.contexts[member].num_faces)
        _check(lib().ilg_batch_get_tsurf(self._h, member, _p(out)))
        return out

    def sync(self):
        _check(lib().ilg_batch_sync(self._h))


def radiosity_blocks_for(nnz: int, entries_per_tile: int = 200_000) -> int:
    """A block count that gives tiles of about `entries_per_tile` entries
    (at least one block): for meshes solved beside others."""
    return max(1, -(-int(nnz) // entries_per_tile))


def debug_ff_chunk(pairs):
    """Candidate pairs per form-factor build chunk (test entry; 0: default)."""
    _check(lib().ilg_debug_ff_chunk(int(pairs)))


def device_pool_high(reset=False):
    """(used, reserved) high-water bytes of the device's allocation pool."""
    u, r = C.c_int64(), C.c_int64()
    _check(lib().ilg_device_pool_high(C.byref(u), C.byref(r), int(reset)))
    return u.value, r.value


def conductionQ(z, dt, Qn, Qnp1, T, ti, rhoc, emiss, Tsurf, Fgeotherm=0.0):
    """One column through the Fortran-ABI symbol conductionq_. Returns
    (T, Tsurf, Fsurf)."""
    z = _f64(z); T = np.array(T, np.float64); ti = _f64(ti); rhoc = _f64(rhoc)
    nz = C.c_int(z.shape[0]); dt_ = C.c_double(dt); qn = C.c_double(Qn); qp = C.c_double(Qnp1)
    em = C.c_double(emiss); ts = C.c_double(Tsurf); fg = C.c_double(Fgeotherm); fs = C.c_double(0)
    lib().conductionq_(C.byref(nz), _p(z), C.byref(dt_), C.byref(qn), C.byref(qp), _p(T), _p(ti), _p(rhoc),
                       C.byref(em), C.byref(ts), C.byref(fg), C.byref(fs))
    return T, ts.value, fs.value


def conductionT(z, dt, T, Tsurf, Tsurfp1, ti, rhoc, Fgeotherm=0.0):
    z = _f64(z); T = np.array(T, np.float64); ti = _f64(ti); rhoc = _f64(rhoc)
    nz = C.c_int(z.shape[0]); dt_ = C.c_double(dt); a = C.c_double(Tsurf); b = C.c_double(Tsurfp1)
    fg = C.c_double(Fgeotherm); fs = C.c_double(0)
    lib().conductiont_(C.byref(nz), _p(z), C.byref(dt_), _p(T), C.byref(a), C.byref(b), _p(ti), _p(rhoc),
                       C.byref(fg), C.byref(fs))
    return T, fs.value


def conductionQ_batch(z, dt, Qn, Qnp1, T, ti, rhoc, emiss, Tsurf, Fgeotherm=0.0, bc_mode=BC_LINEARISED):
    """ncol columns: T is nz x ncol (column per facet). Returns (T, Tsurf, Fsurf)."""
    z = _f64(z); T = np.asfortranarray(np.array(T, np.float64)); ti = _f64(ti); rhoc = _f64(rhoc)
    ncol = T.shape[1]
    Ts = np.array(Tsurf, np.float64).reshape(ncol); Fs = np.zeros(ncol)
    qn = None if Qn is None else _f64(Qn)
    _check(lib().ilg_conductionq_batch(ncol, z.shape[0], _p(z), dt, _p(qn), _p(_f64(Qnp1)), T.ctypes.data_as(C.c_void_p),
                                       _p(ti), _p(rhoc), emiss, _p(Ts), Fgeotherm, _p(Fs), bc_mode))
    return T, Ts, Fs
