"""ilg_conductionq_batch_noalloc (device arrays, fixed library scratch, no
allocation) against the allocating ilg_conductionq_batch on the same columns,
two steps in a row. Collected last so that it also runs after every other
test in the same process; it passes alone as well."""
import ctypes as C

import numpy as np
import pytest

from illum_gb300 import meshgen

TOL_K = 1e-9       # temperatures (K): same kernel and coefficients on both paths


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _profile(nz):
    return meshgen.geometric_depths(nz), np.full(nz, 300.0), np.full(nz, 1.05e6)


def test_noalloc_rejects_oversize_without_device(ilg):
    """A request beyond the fixed scratch fails with a clear message before
    any device pointer is touched (the pointers here are NULL)."""
    z, ti, rhoc = _profile(400)
    L = ilg.lib()
    rc = L.ilg_conductionq_batch_noalloc(1_000_000, 400, _p(z), 30.0, None, None, None, _p(ti), _p(rhoc), 0.95,
                                         None, 0.0, None, ilg.BC_NEWTON, None)
    assert rc == -1
    msg = L.ilg_last_error().decode()
    assert "scratch" in msg and "1000000 columns of 400 layers" in msg


def _fits(ilg, ncol, nz):
    """True when ncol columns of nz layers pass the scratch-size check. With
    NULL device pointers the call then stops at the argument check, still
    before touching the device; a request that is too large stops earlier
    with the scratch message."""
    z, ti, rhoc = _profile(nz)
    L = ilg.lib()
    rc = L.ilg_conductionq_batch_noalloc(ncol, nz, _p(z), 30.0, None, None, None, _p(ti), _p(rhoc), 0.95,
                                         None, 0.0, None, ilg.BC_NEWTON, None)
    assert rc == -1
    msg = L.ilg_last_error().decode()
    assert ("scratch" in msg) != ("invalid arguments" in msg), msg
    return "invalid arguments" in msg


def max_columns(ilg, nz):
    """The largest column count accepted for nz layers (bisection on the
    size check; no device involved)."""
    lo, hi = 1, 1 << 26
    assert _fits(ilg, lo, nz) and not _fits(ilg, hi, nz)
    while hi - lo > 1:
        mid = (lo + hi) // 2
        lo, hi = (mid, hi) if _fits(ilg, mid, nz) else (lo, mid)
    return lo


@pytest.mark.parametrize("nz", [2, 60, 160, 161, 400])
def test_noalloc_size_limit_edges(ilg, nz):
    """At the limit: the largest accepted request and one column more, which
    is rejected; the limit follows the documented sizes (about 8 ncol +
    40 nz bytes up to 160 layers, plus 8 nz ncol above; a few hundred bytes
    of flags and the mesh record, each region on a 256-byte boundary)."""
    n = max_columns(ilg, nz)
    assert _fits(ilg, n, nz) and not _fits(ilg, n + 1, nz)
    scratch = 16 << 20
    per_col = 8 if nz <= 160 else 8 * nz + 8
    lo, hi = (scratch - 40 * nz - 2048) // per_col, (scratch - 40 * nz) // per_col
    assert lo <= n <= hi, (n, lo, hi)


@pytest.mark.gpu
@pytest.mark.parametrize("nz,ncol,bc_mode,with_qn", [(60, 5000, 0, True), (60, 5000, 1, True),
                                                      (40, 777, 0, False), (200, 3000, 1, True),
                                                      (160, 1500, 1, True), (161, 1500, 1, True),
                                                      (2, "max", 1, True)])
def test_noalloc_matches_allocating_path_two_steps(ilg, nz, ncol, bc_mode, with_qn):
    if ncol == "max":
        ncol = max_columns(ilg, nz)   # a request exactly at the scratch limit
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    z, ti, rhoc = _profile(nz)
    rng = np.random.default_rng(nz * 1000 + ncol + bc_mode)
    T0 = rng.uniform(180, 320, (nz, ncol))            # [layer, column]
    Ts0 = rng.uniform(180, 320, ncol)
    Q = [rng.uniform(0, 800, ncol) for _ in range(3)]  # Q at time levels n, n+1, n+2
    dt, emiss, fgeo = 30.0, 0.95, 0.02

    # allocating entry point on host arrays (column-major nz x ncol)
    Th, Tsh = T0, Ts0
    host = []
    for k in range(2):
        qn = (Q[k] if with_qn else None) if k == 0 else Q[k]
        Th, Tsh, Fsh = ilg.conductionQ_batch(z, dt, qn, Q[k + 1], Th, ti, rhoc, emiss, Tsh, Fgeotherm=fgeo,
                                             bc_mode=bc_mode)
        host.append((np.array(Th), np.array(Tsh), np.array(Fsh)))

    # no-allocation entry point on device arrays (layer-major nz x ncol)
    dev = torch.device("cuda:0")
    Td = torch.tensor(np.ascontiguousarray(T0), dtype=torch.float64, device=dev)
    Tsd = torch.tensor(Ts0, dtype=torch.float64, device=dev)
    Fsd = torch.zeros(ncol, dtype=torch.float64, device=dev)
    Qd = [torch.tensor(q, dtype=torch.float64, device=dev) for q in Q]
    stream = torch.cuda.current_stream(dev).cuda_stream
    L = ilg.lib()
    for k in range(2):
        qn = (Qd[k].data_ptr() if with_qn else None) if k == 0 else Qd[k].data_ptr()
        rc = L.ilg_conductionq_batch_noalloc(ncol, nz, _p(z), dt, qn, Qd[k + 1].data_ptr(), Td.data_ptr(), _p(ti),
                                             _p(rhoc), emiss, Tsd.data_ptr(), fgeo, Fsd.data_ptr(), bc_mode,
                                             C.c_void_p(stream))
        assert rc == 0, L.ilg_last_error().decode()
        Th, Tsh, Fsh = host[k]
        Tg = Td.cpu().numpy()
        assert np.abs(Tg - Th).max() <= TOL_K, f"step {k}"
        assert np.abs(Tsd.cpu().numpy() - Tsh).max() <= TOL_K, f"step {k}"
        Fg = Fsd.cpu().numpy()
        assert np.all(np.abs(Fg - Fsh) <= TOL_K * np.maximum(1.0, np.abs(Fsh))), f"step {k}"


@pytest.mark.gpu
def test_noalloc_refuses_a_capturing_stream(ilg):
    """The call copies pageable host memory and synchronises its stream, so on
    a stream that is being captured it returns ILG_ERR_ARG before queuing
    anything (the capture stays valid)."""
    torch = pytest.importorskip("torch")
    nz, ncol = 20, 64
    z, ti, rhoc = _profile(nz)
    dev = torch.device("cuda:0")
    Td = torch.full((nz, ncol), 250.0, dtype=torch.float64, device=dev)
    Tsd = torch.full((ncol,), 250.0, dtype=torch.float64, device=dev)
    Fsd = torch.zeros(ncol, dtype=torch.float64, device=dev)
    Qd = torch.full((ncol,), 300.0, dtype=torch.float64, device=dev)
    side = torch.cuda.Stream(dev)
    L = ilg.lib()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            Td.add_(0.0)   # something to capture
            rc = L.ilg_conductionq_batch_noalloc(ncol, nz, _p(z), 30.0, None, Qd.data_ptr(), Td.data_ptr(), _p(ti),
                                                 _p(rhoc), 0.95, Tsd.data_ptr(), 0.0, Fsd.data_ptr(), ilg.BC_NEWTON,
                                                 C.c_void_p(side.cuda_stream))
    assert rc == -1 and "captured" in L.ilg_last_error().decode()
    g.replay()
    torch.cuda.synchronize()
    assert float(Td[0, 0]) == 250.0
