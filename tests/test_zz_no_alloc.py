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


@pytest.mark.gpu
@pytest.mark.parametrize("nz,ncol,bc_mode,with_qn", [(60, 5000, 0, True), (60, 5000, 1, True),
                                                      (40, 777, 0, False), (200, 3000, 1, True)])
def test_noalloc_matches_allocating_path_two_steps(ilg, nz, ncol, bc_mode, with_qn):
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
