"""Task front-end with the reference CLI's tasks, options, YAML keys and
output files (src/cpp/illum_cli.cpp:29-156 config, 268-540 tasks,
543-711 options), driving the GPU library:

    python -m illum_gb300.cli --task horizons --path shape.obj --nphi 361
    python -m illum_gb300.cli --task form_factors --path shape.obj --albedo 0.12
    python -m illum_gb300.cli --task radiosity --config job.yaml

The radiosity solve is the reference's: a forward solve plus --gs_steps
natural-order Gauss-Seidel sweeps (default 1, src/cpp/illum_cli.cpp:425-433),
computed on the GPU in the reference's summation order. Given --tol (2-norm
of the residual), it instead solves to that tolerance. The thermal run is
the library's fused step (direct -> radiosity -> conduction on the GPU),
with the reference's coupling rad = -Fsurf + direct. --precision mixed
selects the BF16/FP32 path, which solves to --tol, or with --refine_every K
makes one pass over the form factors per step (the f32 values every K-th
step; RunOpts.refine_every). A YAML config holds flat
`key: value` pairs and lists (inline [a, b] or `- item` lines); command-line
options given explicitly override it.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

TASKS = ("form_factors", "horizons", "radiosity", "residuals")
D_SUN_M = 227390024000.0      # default sun distance (illum_cli.cpp:337)


def parse_yaml(text: str) -> dict:
    """The flat subset of YAML the reference's job files use."""
    out, key = {}, None
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].rstrip()
        if not line.strip():
            continue
        s = line.strip()
        if s.startswith("- ") and key is not None:
            if not isinstance(out.get(key), list):
                out[key] = []
            out[key].append(_scalar(s[2:].strip()))
            continue
        if ":" not in s:
            raise ValueError(f"cannot parse config line: {raw!r}")
        key, val = (t.strip() for t in s.split(":", 1))
        if val == "":
            out[key] = []
        elif val.startswith("[") and val.endswith("]"):
            out[key] = [_scalar(t.strip()) for t in val[1:-1].split(",") if t.strip()]
        else:
            out[key] = _scalar(val)
    return out


def _scalar(t: str):
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        return t[1:-1]
    low = t.lower()
    if low in ("true", "yes", "on"):
        return True
    if low in ("false", "no", "off"):
        return False
    try:
        return int(t)
    except ValueError:
        pass
    try:
        return float(t)
    except ValueError:
        return t


def build_parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(prog="illum_gb300.cli", description="Available tasks: " + ", ".join(TASKS))
    add = ap.add_argument
    add("--task", default="radiosity", choices=TASKS)
    add("--config", help="path to YAML configuration file")
    add("--path", help="path to input OBJ file")
    add("--shape", type=int, default=0, help="shape index in the OBJ file")
    add("--offset", type=float, default=1e-5)
    add("--theta_eps", type=float, default=1e-3)
    add("--nphi", type=int, default=361)
    add("--radiosity", type=_bool, default=False)
    add("--gs_steps", type=int, default=1,
        help="Gauss-Seidel sweeps after the forward solve (the reference's solve, used unless --tol is given)")
    add("--tol", type=float, default=None,
        help="radiosity residual 2-norm tolerance: solve to it instead of the fixed sweeps")
    add("--print_residual", type=_bool, default=False)
    add("--thermal", type=_bool, default=False)
    add("--quiet", type=_bool, default=False)
    add("--dt", type=float, default=600.0)
    add("--albedo", default="0.12", help="number, or path of an ARMA vector of per-facet albedo")
    add("--depths", type=float, nargs="+")
    add("--ti", type=float, default=70.0)
    add("--rhoc", type=float, nargs="+")
    add("--T0", default="233.0", help="number, or path of an ARMA (nz+1) x N matrix")
    add("--output_dir", default=".")
    add("--form_factors_file")
    add("--horizon_file")
    add("--horizon_obj_file")
    add("--sun_pos_file")
    add("--sun_unit", default="m", choices=["m", "km"])
    add("--mesh_unit", default="km", choices=["m", "km"])
    add("--save_full_thermal", type=_bool, default=False)
    add("--record_therm_stats", type=_bool, default=False)
    add("--repeat", type=int)
    add("--print_config", type=_bool, default=False)
    add("--precision", default="fp64", choices=["fp64", "mixed"])
    add("--refine_every", type=int, default=0,
        help="mixed precision: one radiosity pass per step, the f32 form factors every K-th step (0: solve to --tol)")
    add("--seed", type=int, default=0, help="seed of the random sun direction when no sun file is given")
    return ap


def _bool(s) -> bool:
    if isinstance(s, bool):
        return s
    return str(s).lower() in ("1", "true", "yes", "on")


def resolve(argv=None) -> argparse.Namespace:
    ap = build_parser()
    args = ap.parse_args(argv)
    if args.config:
        with open(args.config) as f:
            cfg = parse_yaml(f.read())
        given = {a.split("=")[0].lstrip("-") for a in (argv if argv is not None else sys.argv[1:])
                 if a.startswith("--")}
        for k, val in cfg.items():
            if not hasattr(args, k):
                raise ValueError(f"unknown config key {k!r}")
            if k in given:
                continue
            if k in ("depths", "rhoc"):
                val = val if isinstance(val, list) else [val]
                val = [float(x) for x in val]
            setattr(args, k, val)
    if args.mesh_unit == "m":
        print("mesh_unit m: vertices are taken as given (the reference has not implemented it)")
    return args


def _timed(msg, fn):
    t = time.perf_counter()
    print(msg, end="", flush=True)
    r = fn()
    print(f" [{time.perf_counter() - t:.3f} s]")
    return r


def _context(args):
    import illum_gb300 as ig
    from illum_gb300 import meshgen
    if not args.path:
        raise SystemExit("--path is required")
    v, f, n = _timed(f"- loading {args.path}", lambda: meshgen.load_obj(args.path, args.shape))
    ctx = _timed("- building LBVH", lambda: ig.IllumContext(v, f, n))
    if args.horizon_obj_file:
        # a separate mesh for the horizon rays (src/cpp/illum_cli.cpp:899-901)
        hv, hf, _ = _timed(f"- loading horizon mesh {args.horizon_obj_file}",
                           lambda: meshgen.load_obj(args.horizon_obj_file, 0))
        ctx.set_horizon_mesh(hv, hf)
    return ig, ctx


def _albedo(args, n):
    try:
        return float(args.albedo)
    except (TypeError, ValueError):
        from illum_gb300 import armaio
        a = armaio.load(str(args.albedo)).ravel()
        if a.size != n:
            raise SystemExit("albedo vector has the wrong size")
        return a


def task_form_factors(args):
    from illum_gb300 import armaio
    ig, ctx = _context(args)
    rp, col, val = _timed("- computing form factors",
                          lambda: ctx.compute_F(albedo=_albedo(args, ctx.num_faces), offset=args.offset))
    print(f"  [nnz = {len(val)}]")
    os.makedirs(args.output_dir, exist_ok=True)
    _timed("- saving form factor matrix",
           lambda: armaio.save_sparse(os.path.join(args.output_dir, "form_factors.bin"), rp, col, val))


def task_horizons(args):
    from illum_gb300 import armaio
    ig, ctx = _context(args)
    _timed("- building horizon map", lambda: ctx.make_horizons(args.nphi, args.theta_eps, args.offset))
    if not args.quiet:
        os.makedirs(args.output_dir, exist_ok=True)
        path = os.path.join(args.output_dir, "horizons.bin")
        _timed(f"- saving horizon map to {path}", lambda: armaio.save(path, ctx.horizons))


def task_radiosity(args):
    from illum_gb300 import armaio, meshgen
    ig, ctx = _context(args)
    N = ctx.num_faces
    if args.horizon_file:
        H = _timed(f"- loading horizon map from {args.horizon_file}", lambda: armaio.load(args.horizon_file))
        ctx.set_horizons(H)
    else:
        _timed("- building horizon map", lambda: ctx.make_horizons(args.nphi, args.theta_eps, args.offset))
    if args.sun_pos_file:
        suns = armaio.load_sun_positions(args.sun_pos_file, unit=args.sun_unit)
    else:
        d = meshgen.normal(args.seed, 0, 3)
        suns = (D_SUN_M * d / np.linalg.norm(d))[None, :]
        if args.sun_unit == "m":
            suns = suns / 1000.0
    reps = args.repeat or 1
    suns = np.tile(suns, (reps, 1))
    disk = ig.fib_spiral(100)
    if args.radiosity:
        if args.form_factors_file:
            rp, col, val, _ = armaio.load_sparse(args.form_factors_file)
            _timed("- loading form factor matrix", lambda: ctx.set_F(rp, col, val))
        else:
            _timed("- assembling form factor matrix",
                   lambda: ctx.compute_F(albedo=_albedo(args, N), offset=args.offset, fetch=False))
    prec = ig.PREC_MIXED if args.precision == "mixed" else ig.PREC_FP64
    fixed = args.tol is None          # the reference's forward solve + gs_steps sweeps
    if args.refine_every < 0 or (args.refine_every > 0 and (prec != ig.PREC_MIXED or not args.thermal)):
        raise SystemExit("--refine_every K >= 1 goes with --precision mixed and --thermal")
    if fixed and prec == ig.PREC_MIXED and args.refine_every == 0:
        raise SystemExit("--precision mixed solves to a tolerance: give --tol (or --refine_every K)")
    if args.refine_every > 0:
        fixed = False
    if args.gs_steps < 0:
        raise SystemExit("--gs_steps must be >= 0")
    out = {}
    if args.thermal:
        if not args.depths:
            raise SystemExit("--depths is required with --thermal")
        nz = len(args.depths)
        rhoc = args.rhoc if args.rhoc else [1.0]
        rhoc = np.full(nz, rhoc[0]) if len(rhoc) == 1 else np.asarray(rhoc, np.float64)
        try:
            T0, T0_full = float(args.T0), None
        except (TypeError, ValueError):
            T0, T0_full = 0.0, armaio.load(str(args.T0))
        ctx.set_suns(suns, disk)
        tm = ig.ThermalModel(ctx, np.asarray(args.depths, np.float64), args.ti, rhoc, T0 if T0_full is None else T0_full,
                             emissivity=0.999, bc_mode=ig.BC_LINEARISED, precision=prec)
        if args.record_therm_stats:
            ctx.record_thermal(len(suns))
        if fixed:
            ctx.set_radiosity_mode(ig.RAD_GS, args.gs_steps)
        opts = ig.RunOpts(dt=args.dt, tol=0.0 if fixed or args.tol is None else args.tol, max_sweeps=1000,
                          use_radiosity=int(bool(args.radiosity)), use_graph=1, precision=prec,
                          coupling=ig.COUPLE_REFERENCE, refine_every=args.refine_every)
        _timed(f"- {len(suns)} steps (direct, radiosity, conduction)", lambda: ctx.run_steps(opts, 0, len(suns)))
        o = ctx.outputs()
        out = {"rad": o["rad"], "rad_avg": o["rad_avg"], "therm_avg": o["therm_avg"], "therm_max": o["therm_max"],
               "therm": tm.T if args.save_full_thermal else tm.T[0]}
        if args.record_therm_stats:
            rec = ctx.thermal_records()
            out["therm_stats"] = rec[:, :12]
            out["therm_energy"] = rec[:, 12:]
    else:
        rad_avg = np.zeros(N)
        rad = np.zeros(N)
        for j, s in enumerate(suns):
            rad = ctx.get_direct_radiosity(s, disk)
            if args.radiosity:
                if fixed:
                    rad, res = ctx.radiosity_solve_gs(rad, args.gs_steps)
                    sweeps = 1 + args.gs_steps
                else:
                    rad, res, sweeps = ctx.radiosity_solve(rad, tol=args.tol, max_sweeps=1000)
                if args.print_residual:
                    print(f"  [{j + 1}/{len(suns)}: res = {res:.3e} after {sweeps} sweeps]")
            rad_avg += (rad - rad_avg) / (j + 1)
        out = {"rad": rad, "rad_avg": rad_avg}
    if not args.quiet:
        os.makedirs(args.output_dir, exist_ok=True)
        for k, v in out.items():
            armaio.save(os.path.join(args.output_dir, k + ".bin"), v)
    return out


def main(argv=None):
    args = resolve(argv)
    if args.print_config:
        for k, v in sorted(vars(args).items()):
            print(f"{k}: {v}")
    if args.task == "residuals":
        raise SystemExit("residuals: the reference implements this task as a stub")
    return {"form_factors": task_form_factors, "horizons": task_horizons, "radiosity": task_radiosity}[args.task](args)


if __name__ == "__main__":
    main()
