"""The task front-end end to end on a small OBJ: horizons, form factors and
a radiosity + thermal run write the reference's output files; the values
match the library's API and, for the thermal run (the reference's
forward solve + gs_steps sweeps, its coupling and linearised boundary), the
CPU oracle."""
import numpy as np
import pytest

from illum_gb300 import armaio, meshgen

pytestmark = pytest.mark.gpu


def _write_obj(path, v, f):
    n = v / np.linalg.norm(v, axis=1, keepdims=True)
    with open(path, "w") as fh:
        for p in v * 100.0:                     # the reader divides by 100
            fh.write("v %.9g %.9g %.9g\n" % tuple(p))
        for q in n:
            fh.write("vn %.9g %.9g %.9g\n" % tuple(q))
        for t in f + 1:
            fh.write("f %d//%d %d//%d %d//%d\n" % (t[0], t[0], t[1], t[1], t[2], t[2]))


def test_cli_tasks(ilg, oracle_mod, tmp_path):
    from illum_gb300 import cli
    v, f = meshgen.icosphere_craters(2, seed=3, n_craters=4, dmin_m=150.0, dmax_m=400.0)
    obj = tmp_path / "shape.obj"
    _write_obj(str(obj), v.astype(np.float64), f)
    out = tmp_path / "out"
    cli.main(["--task", "horizons", "--path", str(obj), "--nphi", "16", "--output_dir", str(out)])
    H = armaio.load(str(out / "horizons.bin"))
    V, Fc, N = meshgen.load_obj(str(obj))
    ctx = ilg.IllumContext(V, Fc, N)
    ctx.make_horizons(nphi=16)
    assert np.array_equal(H, ctx.horizons)
    cli.main(["--task", "form_factors", "--path", str(obj), "--albedo", "0.1", "--output_dir", str(out)])
    rp, c, x, _ = armaio.load_sparse(str(out / "form_factors.bin"))
    rp2, c2, x2 = ctx.compute_F(albedo=0.1)
    assert np.array_equal(rp, rp2) and np.array_equal(c, c2) and np.array_equal(x, x2)
    suns = meshgen.spin_sun_positions(8, 6 * 3600.0, 600.0) * 1000.0     # metres, as sun_unit m
    np.savetxt(str(tmp_path / "sun.txt"), suns)
    cfg = tmp_path / "job.yaml"
    cfg.write_text("radiosity: true\nthermal: true\nnphi: 16\ndt: 600\nti: 300\nrhoc: 1.05e6\nT0: 220\n"
                   "depths: [0.002, 0.005, 0.01, 0.02, 0.05, 0.1]\nrecord_therm_stats: true\n"
                   f"sun_pos_file: {tmp_path / 'sun.txt'}\nform_factors_file: {out / 'form_factors.bin'}\n"
                   f"horizon_file: {out / 'horizons.bin'}\noutput_dir: {out}\n")
    res = cli.main(["--task", "radiosity", "--path", str(obj), "--config", str(cfg)])
    for name in ("rad", "rad_avg", "therm", "therm_avg", "therm_max", "therm_stats", "therm_energy"):
        assert (out / (name + ".bin")).exists(), name
    therm = armaio.load(str(out / "therm.bin")).ravel()
    assert therm.shape == (Fc.shape[0],) and np.all(np.isfinite(therm))
    assert armaio.load(str(out / "therm_stats.bin")).shape == (8, 12)
    assert np.array_equal(res["therm"], therm)
    # the same job on the CPU oracle: reference solve (gs_steps 1 by
    # default), rad = -Fsurf + direct, linearised boundary, emissivity 0.999,
    # lit counts over nphi - 1, 1372 W/m^2 at 1 AU
    depths = np.array([0.002, 0.005, 0.01, 0.02, 0.05, 0.1])
    nz = len(depths)
    st = oracle_mod.thermal_run(V, Fc, H.T, suns / 1000.0, ilg.fib_spiral(100), (rp, c, x), depths,
                                np.full(nz, 300.0), np.full(nz, 1.05e6), dt=600.0, T0=220.0, emiss=0.999,
                                solar_const=1372.0, norm_mode=0, bc_mode=0, rad_mode=0, gs_steps=1, coupling=0,
                                normals=N)
    assert np.abs(therm - st["T"][:, 0]).max() <= 1e-9
    assert np.abs(armaio.load(str(out / "rad.bin")).ravel() - st["rad"]).max() <= 1e-9 * np.abs(st["rad"]).max()
    assert np.abs(armaio.load(str(out / "therm_avg.bin")).ravel() - st["therm_avg"]).max() <= 1e-9


def test_cli_horizon_obj_file(ilg, oracle_mod, tmp_path):
    """horizon_obj_file: the horizons of the shape's facets traced against a
    second OBJ (src/cpp/illum_cli.cpp:899-901), as the oracle traces them."""
    from illum_gb300 import cli
    v, f = meshgen.icosphere_craters(2, seed=3, n_craters=4, dmin_m=150.0, dmax_m=400.0)
    hv, hf = meshgen.icosphere_craters(3, seed=9, n_craters=30, dmin_m=150.0, dmax_m=500.0)
    obj, hobj = tmp_path / "shape.obj", tmp_path / "horizon.obj"
    _write_obj(str(obj), v.astype(np.float64), f)
    _write_obj(str(hobj), hv.astype(np.float64), hf)
    out = tmp_path / "out"
    cli.main(["--task", "horizons", "--path", str(obj), "--horizon_obj_file", str(hobj), "--nphi", "16",
              "--output_dir", str(out)])
    H = armaio.load(str(out / "horizons.bin"))
    V, Fc, _ = meshgen.load_obj(str(obj))
    HV, HF, _ = meshgen.load_obj(str(hobj))
    assert np.array_equal(H, oracle_mod.horizons(V, Fc, 16, horizon_mesh=(HV, HF)).T)



def test_cli_mixed_one_pass(ilg, tmp_path):
    """--precision mixed --refine_every 4 (one radiosity pass per step): the
    thermal job's surface temperatures within the mixed path's 0.05 K of the
    same job in FP64 solved to --tol 1e-10; the option needs the mixed
    precision and a thermal run."""
    from illum_gb300 import cli
    v, f = meshgen.icosphere_craters(2, seed=3, n_craters=4, dmin_m=150.0, dmax_m=400.0)
    obj = tmp_path / "shape.obj"
    _write_obj(str(obj), v.astype(np.float64), f)
    suns = meshgen.spin_sun_positions(24, 6 * 3600.0, 600.0) * 1000.0
    np.savetxt(str(tmp_path / "sun.txt"), suns)
    cfg = tmp_path / "job.yaml"
    cfg.write_text("radiosity: true\nthermal: true\nnphi: 16\ndt: 600\nti: 300\nrhoc: 1.05e6\nT0: 220\n"
                   "albedo: 0.1\ndepths: [0.002, 0.005, 0.01, 0.02, 0.05, 0.1]\n"
                   f"sun_pos_file: {tmp_path / 'sun.txt'}\n")
    base = ["--task", "radiosity", "--path", str(obj), "--config", str(cfg)]
    r64 = cli.main(base + ["--tol", "1e-10", "--output_dir", str(tmp_path / "o64")])
    rmx = cli.main(base + ["--precision", "mixed", "--refine_every", "4", "--output_dir", str(tmp_path / "omx")])
    assert np.abs(rmx["therm"] - r64["therm"]).max() <= 0.05
    with pytest.raises(SystemExit):
        cli.main(base + ["--refine_every", "4", "--output_dir", str(tmp_path / "bad")])
