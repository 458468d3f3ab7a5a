"""Benchmark of the illumination + thermal time-step loop on one GB300.

Headline workload (the plain FP64 GPU drop-in): icosphere level 6 (81,920
facets), seed 1, 200 craters of 30-300 m on a 1 km body, 64 horizon
azimuths, form factors with albedo 0.1, radiosity to 1e-10, 60-layer
conduction column (geometric 1.1 to 0.5 m, thermal inertia 300, rho*c
1.05e6, emissivity 0.95, Newton surface boundary), sun 1361 W/m^2 at 1.5 AU,
spin period 6 h, sub-solar latitude 10 deg, 720 steps per rotation (dt =
30 s). Synthetic seeded mesh (the reference's shape models are not
distributed).

A step = direct insolation + radiosity solve + conduction for all facets
(src/cpp/illum_cli.cpp:403-456). value = facet-steps/s of the plain FP64
path with device-resident inputs, device time of each step measured with
CUDA events on the library's stream, L2 (129 MB) flushed by a 256 MB write
before every step. e2e = the same metric through ilg_run_steps_host (72
steps per call): every step's sun position copied host->device and its
surface temperatures copied device->host into the caller's host array, host
wall clock.

The same line carries:
  parity_vs_oracle  the GPU's horizons and form factors of this workload
                    against the CPU oracle's, bit for bit, and its
                    temperatures after the first PARITY_STEPS steps against
                    the oracle's (whose timing is cpu_baseline);
  mixed             the same workload in mixed precision vs FP64;
  batch / terrain / serve
                    the 64-mesh batch, the 1024 x 1024 terrain patch and the
                    serving loop, each mixed precision against FP64 on the
                    same work, with its own clocks.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU oracle (the reference cannot be built here;
the oracle restates its path) on the host cores: horizons and form factors
built by the oracle, then W warm-up steps and K timed steps of the same
workload. It loads no CUDA code.

N > 1 runs independent replicas (one process per GPU; the path has no
cross-GPU exchange): value is the sum over ranks of facets*steps divided by
the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "facet-steps/s at <=0.05 K max err vs FP64; visibility rays/s; serve p50/p99 ms"
UNIT = "facet-steps/s"

# Radiosity tolerance of the mixed-precision path (2-norm, W/m^2): about
# 1e-8 of ||E|| for these workloads. The FP64 path keeps the configured 1e-10;
# the mixed path's bar is its temperature error against the FP64 path.
MIXED_TOL = 1e-3
# Sweep budget of the mixed path: one refinement round per step (an
# FP64-accumulated residual, one bf16 sweep, the update); the next step's
# first residual includes what the round left.
MIXED_SWEEPS = 1
# Refinement spacing of the mixed path's per-step solve (RunOpts.refine_every):
# 0 = a refinement round every step (residual pass + bf16 sweep); K >= 1 =
# one pass over the matrix per step from a predicted warm start, with the
# f32 form factors every K-th step and the bf16 copy applied to the change
# since then in between.
MIXED_REFINE = 4

CFG = dict(level=6, seed=1, n_craters=200, dmin_m=30.0, dmax_m=300.0, nphi=64, theta_eps=1e-3, offset=1e-5,
           albedo=0.1, nz=60, ti=300.0, rhoc=1500.0 * 700.0, emiss=0.95, T0=200.0, solar=1361.0, dist_au=1.5,
           period_s=6 * 3600.0, steps_per_rot=720, rotations=10, tol=1e-10, lat_deg=10.0)
# The workload label, the same string in both arms.
WORKLOAD_C1 = ("icosphere L6, 81,920 facets, seed 1, 200 craters 30-300 m, nphi 64, theta_eps 1e-3, albedo 0.1, "
               "nz 60 (geometric 1.1 to 0.5 m), ti 300, rho c 1.05e6, emissivity 0.95, Newton surface boundary, "
               "dt 30 s (720 steps per rotation), radiosity tol 1e-10, E = direct coupling, FP64")
# Steps of the GPU-vs-oracle temperature comparison (and of the CPU baseline).
PARITY_STEPS = 60
# Most time steps one run of the reference arm times (and warms up with).
REF_MAX_STEPS = 200


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(name: str, key: str = "dram_bytes_per_launch"):
    """A figure recorded in profiles/<name>.md (the line `<key>: <value>` of
    an ncu capture summary), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", name + ".md")) as f:
            m = re.search(r"^" + key + r":\s*([0-9.eE+]+)", f.read(), re.M)
        return float(m.group(1)) if m else None
    except OSError:
        return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=2)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1])); mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- C1 workload
def c1_mesh(meshgen):
    c = CFG
    return meshgen.icosphere_craters(c["level"], c["seed"], n_craters=c["n_craters"], dmin_m=c["dmin_m"],
                                     dmax_m=c["dmax_m"])


def c1_suns(meshgen, nsun):
    c = CFG
    dt = c["period_s"] / c["steps_per_rot"]
    return meshgen.spin_sun_positions(nsun, c["period_s"], dt, c["lat_deg"], c["dist_au"]), dt


def build_workload(ig, meshgen, precision=0):
    """The C1 mesh on the GPU: LBVH, horizons, form factors, suns, thermal model."""
    c = CFG
    v, f = c1_mesh(meshgen)
    t0 = time.perf_counter()
    ctx = ig.IllumContext(v, f)
    t_bvh = time.perf_counter() - t0
    t0 = time.perf_counter()
    ctx.make_horizons(nphi=c["nphi"], theta_eps=c["theta_eps"], offset=c["offset"])
    t_hor = time.perf_counter() - t0
    t0 = time.perf_counter()
    csr = ctx.compute_F(albedo=c["albedo"], offset=c["offset"])
    t_ff = time.perf_counter() - t0
    ctx.set_insolation(1, 0, c["solar"])
    nsun = c["steps_per_rot"] * c["rotations"]
    suns, dt = c1_suns(meshgen, nsun)
    disk = ig.fib_spiral(100)
    ctx.set_suns(suns, disk)
    z = meshgen.geometric_depths(c["nz"])
    tm = new_thermal(ig, ctx, z, precision)
    setup = {"bvh_s": t_bvh, "horizons_s": t_hor, "form_factors_s": t_ff,
             "horizon_rays": int(f.shape[0] * c["nphi"] * 11), "visibility_rays": int(ctx.visibility_rays),
             "nnz": int(ctx.nnz)}
    return dict(v=v, f=f, ctx=ctx, tm=tm, csr=csr, suns=suns, disk=disk, z=z, dt=dt, nsun=nsun, setup=setup)


def new_thermal(ig, ctx, z, precision):
    """A fresh thermal state on ctx (T = T0, frame 0, no warm start)."""
    c = CFG
    return ig.ThermalModel(ctx, z, c["ti"], c["rhoc"], c["T0"], emissivity=c["emiss"], bc_mode=ig.BC_NEWTON,
                           precision=precision)


def mixed_dtype():
    if MIXED_REFINE > 0:
        return "bf16 F + f32 reference passes + fp32 conduction"
    return "bf16 F + fp32 conduction (fp64 residual)"


def mixed_solve_label():
    if MIXED_REFINE > 0:
        return (f"one matrix pass per step from a predicted warm start, f32 form factors every {MIXED_REFINE}th "
                "step, bf16 between")
    return "one refinement round per step (f32 residual pass, one bf16 sweep)"


def c1_opts(ig, dt, precision, use_graph=1):
    if precision == ig.PREC_MIXED:
        return ig.RunOpts(dt=dt, tol=MIXED_TOL, max_sweeps=MIXED_SWEEPS, use_radiosity=1, use_graph=use_graph,
                          precision=precision, coupling=ig.COUPLE_DIRECT, refine_every=MIXED_REFINE)
    return ig.RunOpts(dt=dt, tol=CFG["tol"], max_sweeps=200, use_radiosity=1, use_graph=use_graph,
                      precision=precision, coupling=ig.COUPLE_DIRECT)


# ----------------------------------------------------------------- oracle legs
def oracle_module():
    """The CPU oracle (test infrastructure: the checker and the CPU baseline)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    return oracle


def oracle_setup(O, v, f):
    """Horizons and form factors of the C1 mesh by the oracle
    (src/cpp/illum.cpp:42-363 restated), timed."""
    c = CFG
    t0 = time.perf_counter()
    H = O.horizons(v, f, c["nphi"], theta_eps=c["theta_eps"], offset=c["offset"])   # N x nphi
    t_hor = time.perf_counter() - t0
    t0 = time.perf_counter()
    r, cl, val, rays = O.form_factors(v, f, offset=c["offset"], albedo_scalar=c["albedo"])
    csr = O.coo_to_csr(f.shape[0], r, cl, val)
    t_ff = time.perf_counter() - t0
    return dict(H=H, csr=csr, rays=rays, horizons_s=t_hor, form_factors_s=t_ff,
                horizon_rays=int(f.shape[0] * c["nphi"] * 11))


def oracle_steps(O, v, f, osu, suns, disk, z, state=None, frame0=0):
    """Time steps of the oracle (src/cpp/illum_cli.cpp:403-456): direct
    insolation threaded over facets, Gauss-Seidel and conduction serial as
    in the reference. Returns (state, seconds)."""
    c = CFG
    nz = len(z)
    dt = c["period_s"] / c["steps_per_rot"]
    t0 = time.perf_counter()
    st = O.thermal_run(v, f, osu["H"], suns, disk, osu["csr"], z, np.full(nz, c["ti"]), np.full(nz, c["rhoc"]),
                       dt=dt, T0=c["T0"], emiss=c["emiss"], solar_const=c["solar"], norm_mode=1, bc_mode=1,
                       rad_mode=1, tol=c["tol"], coupling=1, state=state, frame0=frame0)
    return st, time.perf_counter() - t0


def reference_arm(args, rank):
    """The reference's CPU path (the oracle) on the host cores. Loads no
    CUDA code: the mesh generator is numpy, horizons, form factors and the
    time steps are the oracle's."""
    if rank != 0:
        return
    from illum_gb300 import meshgen   # numpy only; the package loads its CUDA library on first use
    O = oracle_module()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    v, f = c1_mesh(meshgen)
    N = f.shape[0]
    osu = oracle_setup(O, v, f)
    # a bounded sample: at most REF_MAX_STEPS timed steps (~0.3 s each on 16 cores)
    W = max(0, min(args.warmup, REF_MAX_STEPS))
    K = max(1, min(args.steps, REF_MAX_STEPS))
    suns, _ = c1_suns(meshgen, W + K)
    disk = O.fib_spiral(100)
    z = meshgen.geometric_depths(CFG["nz"])
    state = None
    if W:
        state, _ = oracle_steps(O, v, f, osu, suns[:W], disk, z)
    state, el = oracle_steps(O, v, f, osu, suns[W:], disk, z, state=state, frame0=W)
    value = N * K / el
    sample = (f"{K} time steps after {W} warm-up steps of the workload on {threads} host threads (direct insolation "
              f"threaded, Gauss-Seidel and conduction serial as in the reference); horizons and form factors "
              f"built by the oracle beforehand (untimed)")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": K, "warmup": W,
            "ms_per_step": 1000.0 * el / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD_C1, "facets": N, "nnz": int(len(osu["csr"][2]))},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "setup_s": {"horizons_s": osu["horizons_s"], "form_factors_s": osu["form_factors_s"]},
            "visibility_rays": osu["rays"], "visibility_rays_per_s": osu["rays"] / osu["form_factors_s"],
            "horizon_rays_per_s": osu["horizon_rays"] / osu["horizons_s"]}
    print(json.dumps(line), flush=True)


def parity_c1(ig, O, W, steps):
    """C1-size parity: the GPU's horizons and CSR against the oracle's, bit
    for bit (src/cpp/illum.cpp:42-363), and the FP64 GPU temperatures after
    `steps` steps against the oracle's (src/cpp/illum_cli.cpp:403-456,
    src/cpp/conductionQ.f:1-99) on the oracle's own horizons and form
    factors. Returns (parity dict, cpu_baseline dict)."""
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    v, f, ctx = W["v"], W["f"], W["ctx"]
    osu = oracle_setup(O, v, f)
    Hg = ctx.horizons.T                      # N x nphi
    hor_ok = bool(np.array_equal(Hg, osu["H"]))
    rp, cl, val = W["csr"]
    orp, ocl, oval = osu["csr"]
    vis_ok = bool(np.array_equal(rp, orp) and np.array_equal(cl, ocl))
    ff_ok = bool(vis_ok and np.array_equal(val, oval))
    # temperatures: a fresh FP64 state on the GPU context, the same steps
    tm = new_thermal(ig, ctx, W["z"], ig.PREC_FP64)
    ctx.run_steps(c1_opts(ig, W["dt"], ig.PREC_FP64), 0, steps)
    Tg = tm.T
    st, el = oracle_steps(O, v, f, osu, W["suns"][:steps], O.fib_spiral(100), W["z"])
    To = st["T"].T
    err = float(np.abs(Tg - To).max())
    err_s = float(np.abs(Tg[0] - To[0]).max())
    N = f.shape[0]
    parity = {"horizons_bit_exact": hor_ok, "visibility_bit_exact": vis_ok, "form_factors_bit_exact": ff_ok,
              "horizon_bins_differing": int(np.count_nonzero(Hg != osu["H"])),
              "nnz_gpu": int(len(val)), "nnz_oracle": int(len(oval)),
              "visibility_rays_gpu": int(W["setup"]["visibility_rays"]), "visibility_rays_oracle": int(osu["rays"]),
              "steps": steps, "max_err_K_vs_oracle": err, "max_err_surface_K_vs_oracle": err_s,
              "bar_K": 1e-9, "within_bar": bool(err <= 1e-9),
              "oracle_setup_s": {"horizons_s": osu["horizons_s"], "form_factors_s": osu["form_factors_s"]}}
    cpu = {"value": N * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"the first {steps} time steps of the workload ({el:.1f} s, the parity run); direct insolation "
                     f"threaded, Gauss-Seidel and conduction serial as in the reference"}
    return parity, cpu


# ----------------------------------------------------------------- C2 batch
BATCH = dict(nmesh=64, seed0=2, levels=(3, 4, 5, 6), crater_rate=0.0025, dmin_m=30.0, dmax_m=300.0, nz=(30, 80),
             ti=(50.0, 2000.0), period_h=(2.0, 12.0), steps_per_rot=(360, 720), nphi=32, albedo=0.1, tol=1e-10)


def c2_member_params(seed):
    """Per-mesh draws of the batched workload (seeded, counter-based)."""
    from illum_gb300 import meshgen
    u = meshgen.uniform(seed, 9, 8)
    level = BATCH["levels"][min(3, int(u[0] * 4))]
    nfaces = 20 * 4 ** level
    lam = BATCH["crater_rate"] * nfaces
    # Poisson(lam) by inversion of the CDF with one uniform
    k, p, cdf = 0, np.exp(-lam), np.exp(-lam)
    while u[1] > cdf and k < 10 * lam + 20:
        k += 1
        p *= lam / k
        cdf += p
    nz = BATCH["nz"][0] + min(BATCH["nz"][1] - BATCH["nz"][0], int(u[2] * (BATCH["nz"][1] - BATCH["nz"][0] + 1)))
    ti = float(np.exp(np.log(BATCH["ti"][0]) + u[3] * (np.log(BATCH["ti"][1]) - np.log(BATCH["ti"][0]))))
    period_h = BATCH["period_h"][0] + u[4] * (BATCH["period_h"][1] - BATCH["period_h"][0])
    spr = BATCH["steps_per_rot"][int(u[5] * 2) % 2]
    return dict(level=level, craters=int(k), nz=nz, ti=ti, period_h=period_h, steps_per_rot=spr)


def c2_thermal(ig, m, precision):
    """A fresh thermal state and run options of batch member m."""
    q = m["q"]
    tm = ig.ThermalModel(m["ctx"], m["z"], q["ti"], CFG["rhoc"], CFG["T0"], emissivity=CFG["emiss"],
                         bc_mode=ig.BC_NEWTON, precision=precision)
    mixed = precision == ig.PREC_MIXED
    opts = ig.RunOpts(dt=m["dt"], tol=MIXED_TOL if mixed else BATCH["tol"], max_sweeps=MIXED_SWEEPS if mixed else 200,
                      use_radiosity=1, use_graph=1, precision=precision, coupling=ig.COUPLE_DIRECT,
                      refine_every=MIXED_REFINE if mixed else 0)
    return tm, opts


def build_c2(ig, meshgen, precision, nmesh=None, nsteps=None):
    members = []
    nm = nmesh or BATCH["nmesh"]
    for seed in range(BATCH["seed0"], BATCH["seed0"] + nm):
        q = c2_member_params(seed)
        v, f = meshgen.icosphere_craters(q["level"], seed, n_craters=q["craters"], dmin_m=BATCH["dmin_m"],
                                         dmax_m=BATCH["dmax_m"])
        ctx = ig.IllumContext(v, f)
        ctx.make_horizons(nphi=BATCH["nphi"])
        ctx.set_insolation(1, 0, CFG["solar"])
        ctx.compute_F(albedo=BATCH["albedo"], fetch=False)
        # tiles of ~200k entries: the batch, not one member, fills the GPU
        ctx.set_radiosity_blocks(ig.radiosity_blocks_for(ctx.F_info()["nnz"]))
        period = q["period_h"] * 3600.0
        dt = period / q["steps_per_rot"]
        n = nsteps or q["steps_per_rot"]
        ctx.set_suns(meshgen.spin_sun_positions(n, period, dt, CFG["lat_deg"], CFG["dist_au"]), ig.fib_spiral(100))
        m = dict(ctx=ctx, q=q, z=meshgen.geometric_depths(q["nz"]), dt=dt, nfaces=f.shape[0], nsteps=n)
        m["tm"], m["opts"] = c2_thermal(ig, m, precision)
        members.append(m)
    return members


# Vector bytes per facet of one one-pass mixed solve (k_radiosity_lagged):
# start pass 16 (warm-start record) + 16 (direct flux of two frames) + 9
# (permutation, row flag, mesh) + 8 (reference iterate) + 32 written (E,
# s0, x, halo vector); the halo vector gathered once, 8; row finishing 16
# read + 12 written; result pass 16 + 4 + 8 read, 8 + 16 written.
LAGGED_VEC_BYTES = 176


def batch_roofline(stored, nf, ms_rad):
    """HBM roofline of the batch's mixed radiosity launch: algorithmic bytes
    per step (entry stream + vectors) over its CUDA-event time; traffic from
    the ncu capture of a bf16 step and a reference step, weighted as the
    steps come."""
    peak, peak_kind = _peaks()
    if MIXED_REFINE > 0:
        k = MIXED_REFINE
        b = stored * (4.0 * (k - 1) + 6.0) / k + nf * LAGGED_VEC_BYTES
        t_bf = profile_traffic("k_radiosity_lagged_batch64")
        t_rf = profile_traffic("k_radiosity_lagged_batch64", "dram_bytes_per_ref_launch")
        traffic = (t_bf * (k - 1) + t_rf) / k if t_bf and t_rf else None
        kernel = "k_radiosity_lagged"
    else:
        b = stored * 10.0 + nf * LAGGED_VEC_BYTES
        traffic = None
        kernel = "k_radiosity_mixed"
    ach = b / (ms_rad * 1e-3) / 1e9
    out = {"kernel": kernel, "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
           "peak_kind": peak_kind, "algorithmic_bytes": b, "avg_ms": ms_rad, "traffic": traffic,
           "traffic_unit": "bytes per launch"}
    if traffic:
        out["traffic_source"] = "profiles/k_radiosity_lagged_batch64.md (ncu, one bf16 and one reference step)"
    return out


def nested_batch(ig, meshgen, K, W):
    """64 meshes stepped as one batch (one launch per phase, CUDA graph per
    step): mixed precision, then FP64 on the same meshes from the same
    initial state. value = facet-steps/s over K timed steps after W warm-up
    steps (every member active); max_err_K = largest temperature difference
    (all layers) of the mixed batch against the FP64 batch after W + K steps."""
    t0 = time.perf_counter()
    mem = build_c2(ig, meshgen, ig.PREC_MIXED)
    t_setup = time.perf_counter() - t0
    P = 8   # eager phase-timed steps after the timed ones
    K = max(1, min(K, min(m["nsteps"] for m in mem) - W - P))
    nf = sum(m["nfaces"] for m in mem)
    out = {}
    Tm = None
    for prec in (ig.PREC_MIXED, ig.PREC_FP64):
        if prec == ig.PREC_FP64:
            for m in mem:
                m["tm"], m["opts"] = c2_thermal(ig, m, prec)
        b = ig.Batch([m["ctx"] for m in mem], [m["opts"] for m in mem])
        tune = b.autotune()   # the batch's own direct-insolation shapes (untimed)
        b.run(W)
        clk = ClockSampler(0).start()
        ms = b.bench(K, 256.0)
        cl = clk.stop()
        _, ph = b.bench_phases(P, 256.0)
        b.sync()
        b.close()
        out[prec] = dict(value=nf * K / (ms.sum() / 1000.0), ms=float(ms.mean()), clocks=cl, autotune=tune,
                         phases={k: float(v) / P for k, v in zip(("direct", "radiosity", "conduction"), ph)})
        if prec == ig.PREC_MIXED:
            Tm = [m["tm"].T for m in mem]
    err = max(float(np.abs(m["tm"].T - t).max()) for m, t in zip(mem, Tm))
    stored = sum(m["ctx"].F_info()["stored_entries"] for m in mem)
    for m in mem:
        m["ctx"].close()
    mx, d = out[ig.PREC_MIXED], out[ig.PREC_FP64]
    roof = batch_roofline(stored, nf, mx["phases"]["radiosity"])
    return {"value": mx["value"], "unit": UNIT, "steps": K, "warmup": W, "ms_per_step": mx["ms"],
            "dtype": mixed_dtype(),
            "config": {"workload": "64 meshes seeds 2-65, icosphere L3-L6, Poisson craters 0.0025/facet, nz 30-80, "
                                   "ti log-U[50,2000], P U[2,12] h, 360/720 steps per rotation, nphi 32, albedo 0.1, "
                                   "one batch, one launch per phase, CUDA graph per step, radiosity row tiles of ~200k "
                                   "entries per member; FP64 arm radiosity tol 1e-10; mixed arm "
                                   + mixed_solve_label(),
                       "facets": nf, "l2": "256 MB flush before every timed step"},
            "fp64_value": d["value"], "fp64_ms_per_step": d["ms"], "mixed_vs_fp64": mx["value"] / d["value"],
            "phases_ms_per_step": mx["phases"], "fp64_phases_ms_per_step": d["phases"],
            "max_err_K_vs_fp64": err, "err_after_steps": W + K + P, "setup_s": t_setup, "roofline_radiosity": roof,
            "autotune": mx["autotune"], "fp64_autotune": d["autotune"],
            "clocks": mx["clocks"], "fp64_clocks": d["clocks"], "gpu_launches": 5 * K}


# ----------------------------------------------------------------- C3 terrain
TERRAIN = dict(seed=7, spacing_m=2.0, hurst=0.8, rms_m=25.0, n_bowls=2000, dmin_m=10.0, dmax_m=400.0, nphi=128,
               albedo=0.1, rel_tol=1e-8, nz=40, ti=300.0, rhoc=1500.0 * 700.0, emiss=0.95, T0=200.0,
               period_s=6 * 3600.0, steps_per_rot=360, site_lat_deg=0.0)


def mixed_radiosity_bytes(F, rounds, sweeps, N):
    """Bytes one mixed radiosity launch must move at least: per residual
    pass every stored entry's f32 value and u16 column (6 B), per bf16 sweep
    its bf16 value and column (4 B) plus the rows' f32 scales, and per pass
    the iterate vectors (x gathered as a double-float: 8 B read, s and the
    result written: 8 + 8 B) and E (8 B)."""
    se = F["stored_entries"]
    return rounds * (se * 6 + N * 32) + sweeps * (se * 4 + F["active_rows"] * 4 + N * 16)


# Device bytes per stored form-factor entry once built: CSR 4 + 8, row
# tiles 2 + 4 + 4 + 2. The build's peak per entry is measured (allocation
# pool high-water mark) on the base cutoff.
F_BYTES_RESIDENT = 24
TERRAIN_RADII_M = (30.0, 45.0, 60.0, 90.0, 120.0, 200.0, 400.0, 1000.0, 2000.0)
TERRAIN_BASE_CUTOFF_M = 30.0   # first build: measures the peak bytes per entry
F_BYTES_PEAK_FLOOR = 48.0      # per entry: kept keys and values, sort buffers, CSR, row tiles
TERRAIN_BUILD_CAP_S = 90.0     # longest form-factor build the bench attempts


def device_memory_bytes():
    """(total, used) bytes of GPU 0 as nvidia-smi reports them, or None."""
    try:
        out = subprocess.run(["nvidia-smi", "--query-gpu=memory.total,memory.used", "--format=csv,noheader,nounits",
                              "-i", "0"], capture_output=True, text=True, timeout=20).stdout.strip().split(",")
        return float(out[0]) * 1048576.0, float(out[1]) * 1048576.0
    except Exception:
        return None


def terrain_cutoff_sizing(ctx, N, frac, peak_per_entry, budget_bytes, max_radius_m):
    """The configured 2 km cutoff, sized without building F: visibility of a
    seeded sample of source facets with the 2 km cutoff, giving per source
    the entries its column would hold (nnz estimate N x mean, standard error
    N x std / sqrt(n)) and the sample's entries within each listed radius.
    A radius fits when its estimated entries times the build's peak bytes
    per entry stay within the budget (device memory free for it) and it
    does not exceed max_radius_m (the build-time cap)."""
    import numpy as np
    from illum_gb300 import meshgen
    n = max(16, int(round(frac * N)))
    order = np.argsort(meshgen.uniform(77, 1, N))
    src = np.sort(order[:n]).astype(np.int32)
    t0 = time.perf_counter()
    r = ctx.visibility_sample(src, cutoff=2.0, radii=[x / 1000.0 for x in TERRAIN_RADII_M])
    el = time.perf_counter() - t0
    per = r["per_source"].astype(np.float64)
    est = {f"{int(x)} m": float(w) * N / n for x, w in zip(TERRAIN_RADII_M, r["within_radius"])}
    fit = [x for x, w in zip(TERRAIN_RADII_M, r["within_radius"])
           if float(w) * N / n * peak_per_entry <= budget_bytes and x <= max_radius_m]
    nnz2k = float(per.mean() * N)
    return {"sample_sources": n, "sample_seed": 77, "rays": r["rays"], "seconds": el,
            "nnz_2km_estimate": nnz2k, "nnz_2km_stderr": float(per.std(ddof=1) * N / np.sqrt(n)),
            "bytes_2km_bf16_u16": nnz2k * 4.0, "nnz_estimate_by_cutoff": est,
            "build_peak_bytes_per_entry": peak_per_entry, "bytes_per_entry_resident": F_BYTES_RESIDENT,
            "budget_bytes": budget_bytes, "build_time_cap_radius_m": max_radius_m,
            "largest_listed_cutoff_fitting_m": max(fit) if fit else None}


def nested_terrain(ig, meshgen, n, cutoff_m, K, W, sample_frac=0.0025):
    """Heightmap terrain patch (fBm + power-law bowls) with form factors
    within a distance cutoff, 128 horizon azimuths, radiosity refined to
    rel_tol of ||E|| at noon: mixed precision, then FP64 on the same context
    from the same initial state. The radiosity roofline is taken here: the
    bf16 matrix is larger than L2."""
    c = TERRAIN
    t0 = time.perf_counter()
    v, f = meshgen.heightmap_terrain(n=n, spacing_m=c["spacing_m"], seed=c["seed"], hurst=c["hurst"],
                                     rms_m=c["rms_m"], n_bowls=c["n_bowls"] * (n * n) // (1024 * 1024),
                                     dmin_m=c["dmin_m"], dmax_m=c["dmax_m"])
    t_mesh = time.perf_counter() - t0
    N = f.shape[0]
    dt = c["period_s"] / c["steps_per_rot"]
    nsun = c["steps_per_rot"]
    suns = meshgen.site_sun_positions(nsun, c["period_s"], dt, c["site_lat_deg"])
    disk = ig.fib_spiral(100)
    z = meshgen.geometric_depths(c["nz"])
    t0 = time.perf_counter()
    ctx = ig.IllumContext(v, f)
    t_bvh = time.perf_counter() - t0
    t0 = time.perf_counter()
    ctx.make_horizons(nphi=c["nphi"])
    t_hor = time.perf_counter() - t0
    # F at the base cutoff, with the allocation pool's high-water mark: the
    # build's peak device bytes per stored entry
    ig.device_pool_high(reset=True)
    used0, _ = ig.device_pool_high()
    t0 = time.perf_counter()
    ctx.compute_F(albedo=c["albedo"], cutoff=TERRAIN_BASE_CUTOFF_M / 1000.0, fetch=False)
    t_ff = time.perf_counter() - t0
    used1, _ = ig.device_pool_high()
    F = ctx.F_info()
    measured = (used1 - used0) / max(1, F["nnz"])
    peak_per_entry = max(measured, F_BYTES_PEAK_FLOOR)
    base = {"cutoff_m": TERRAIN_BASE_CUTOFF_M, "nnz": F["nnz"], "form_factors_s": t_ff,
            "visibility_rays": int(ctx.visibility_rays), "build_peak_bytes": used1 - used0,
            "build_peak_bytes_per_entry_measured": measured}
    # candidate pairs grow as the radius squared: the radius whose build
    # would take TERRAIN_BUILD_CAP_S at the base build's rate
    max_radius = TERRAIN_BASE_CUTOFF_M * float(np.sqrt(TERRAIN_BUILD_CAP_S / max(t_ff, 1e-3)))
    sizing = None
    run_cut = TERRAIN_BASE_CUTOFF_M if cutoff_m is None else cutoff_m
    if sample_frac > 0:
        mem = device_memory_bytes()
        budget = 0.85 * (mem[0] - mem[1]) if mem else 150e9
        sizing = terrain_cutoff_sizing(ctx, N, sample_frac, peak_per_entry, budget, max_radius)
        if cutoff_m is None and sizing["largest_listed_cutoff_fitting_m"]:
            run_cut = sizing["largest_listed_cutoff_fitting_m"]
    # the chosen radius, else the next smaller listed ones (a build can still
    # fail: device memory, or a facet seeing more facets than a row tile's
    # halo holds), down to the base cutoff, whose F is rebuilt last
    fallback = []
    tries = [run_cut] + [x for x in sorted(TERRAIN_RADII_M, reverse=True) if TERRAIN_BASE_CUTOFF_M < x < run_cut]
    if cutoff_m is not None:
        tries = [run_cut]
    for cut in tries + [TERRAIN_BASE_CUTOFF_M]:
        if cut == TERRAIN_BASE_CUTOFF_M and not fallback and run_cut == TERRAIN_BASE_CUTOFF_M:
            break   # the base F is in place
        try:
            t0 = time.perf_counter()
            ctx.compute_F(albedo=c["albedo"], cutoff=cut / 1000.0, fetch=False)
            t_ff = time.perf_counter() - t0
            run_cut = cut
            break
        except ig.IlgError as e:
            fallback.append(f"{cut:g} m failed ({e})")
    fallback = "; ".join(fallback) if fallback else None
    cutoff_m = run_cut
    rays = int(ctx.visibility_rays)
    F = ctx.F_info()
    ctx.set_insolation(1, 0, CFG["solar"])
    ctx.set_suns(suns, disk)
    E = ctx.get_direct_radiosity(suns[0], disk)
    tol = c["rel_tol"] * float(np.linalg.norm(E))
    K = max(1, min(K, nsun - W))
    res = {}
    for prec in (ig.PREC_MIXED, ig.PREC_FP64):
        tm = ig.ThermalModel(ctx, z, c["ti"], c["rhoc"], c["T0"], emissivity=c["emiss"], bc_mode=ig.BC_NEWTON,
                             precision=prec)
        opts = ig.RunOpts(dt=dt, tol=tol, max_sweeps=400, use_radiosity=1, use_graph=1, precision=prec,
                          coupling=ig.COUPLE_DIRECT)
        ctx.run_steps(opts, 0, W)
        clk = ClockSampler(0).start()
        ms, _ = ctx.bench_steps(opts, W, K, flush_mb=256.0)
        cl = clk.stop()
        res[prec] = dict(ms=float(np.sum(ms)), T=tm.T, rad=ctx.outputs()["rad"].copy(), clocks=cl)
        if prec == ig.PREC_MIXED:
            # per-phase device times of a few eager steps in the serial order
            # (continuing the same run) for the radiosity roofline
            nph = min(8, nsun - W - K)
            eager = ig.RunOpts(dt=dt, tol=tol, max_sweeps=400, use_radiosity=1, use_graph=0, precision=prec,
                               coupling=ig.COUPLE_DIRECT)
            ctx.set_timing(True)
            _, ph = ctx.bench_steps(eager, W + K, nph, flush_mb=256.0)
            st = ctx.stats()
            ctx.set_timing(False)
            res["phases"] = {k: v / nph for k, v in ph.items()}
            res["sweeps_per_step"] = st["radiosity_sweeps"] / nph
        del tm
    m, d = res[ig.PREC_MIXED], res[ig.PREC_FP64]
    err_K = float(np.abs(m["T"] - d["T"]).max())
    rad_rel = float(np.abs(m["rad"] - d["rad"]).max() / max(1e-300, np.abs(d["rad"]).max()))
    ctx.close()
    # roofline of the mixed radiosity launch (bf16 matrix > L2: HBM-bound)
    peak, peak_kind = _peaks()
    sw = res["sweeps_per_step"]
    inner = min(2, 400)
    rounds = sw / inner + 1.0
    b = mixed_radiosity_bytes(F, rounds, sw, N)
    ms_rad = res["phases"]["radiosity"]
    ach = b / (ms_rad * 1e-3) / 1e9
    roof = {"kernel": "k_radiosity_mixed", "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "peak_kind": peak_kind, "algorithmic_bytes": b, "avg_ms": ms_rad,
            "sweeps_per_step": sw, "residual_passes_per_step": rounds,
            "traffic": None, "traffic_unit": "bytes per launch"}
    # ncu's DRAM bytes of the captured 512 x 512 launch per algorithmic byte,
    # scaled to this launch's algorithmic bytes (traffic grows with them)
    cap_t = profile_traffic("k_radiosity_mixed_terrain512")
    cap_a = profile_traffic("k_radiosity_mixed_terrain512", "algorithmic_bytes_per_launch")
    if cap_t and cap_a:
        roof["traffic"] = b * cap_t / cap_a
        roof["traffic_source"] = ("profiles/k_radiosity_mixed_terrain512.md (ncu, 512 x 512 terrain), "
                                  "scaled by algorithmic bytes")
    why = "the configuration states 2 km"
    if sizing:
        why += (f": estimated {sizing['nnz_2km_estimate']:.3g} entries, {sizing['bytes_2km_bf16_u16'] / 1e9:.0f} GB "
                f"as bf16 + u16 alone, beyond the device")
        if fallback:
            why += f"; {fallback}; ran {cutoff_m:g} m"
        elif cutoff_m == sizing["largest_listed_cutoff_fitting_m"]:
            why += f"; {cutoff_m:g} m is the largest listed radius whose build fits"
    label = (f"heightmap {n}x{n} at {c['spacing_m']} m ({N} facets), fBm H {c['hurst']} RMS {c['rms_m']} m, "
             f"power-law bowls, form factors within {cutoff_m:g} m ({why}), nphi {c['nphi']}, "
             f"radiosity to {c['rel_tol']} of ||E||, nz {c['nz']}, equatorial site, 360 steps per rotation")
    return {"value": N * K / (m["ms"] * 1e-3), "unit": UNIT, "steps": K, "warmup": W, "ms_per_step": m["ms"] / K,
            "dtype": "bf16 F + fp32 conduction (fp64 residual)",
            "config": {"workload": label, "facets": N, "cutoff_m": cutoff_m, "l2": "256 MB flush before every timed step"},
            "fp64_value": N * K / (d["ms"] * 1e-3), "mixed_vs_fp64": d["ms"] / m["ms"],
            "max_err_K_vs_fp64": err_K, "max_rel_radiance_err_vs_fp64": rad_rel, "radiosity_tol": tol, "F": F,
            "visibility_rays": rays, "phases_ms_per_step": res["phases"], "roofline_radiosity": roof,
            "setup_s": {"mesh_s": t_mesh, "bvh_s": t_bvh, "horizons_s": t_hor, "form_factors_s": t_ff},
            "horizon_rays_per_s": N * c["nphi"] * 11 / t_hor, "visibility_rays_per_s": rays / t_ff,
            "cutoff_sizing": sizing, "base_build": base, "cutoff_fallback": fallback,
            "clocks": m["clocks"], "fp64_clocks": d["clocks"], "gpu_launches": 5 * K}


# ----------------------------------------------------------------- C4 serving
def nested_serve(ig, nreq, scale, rate):
    """The serving loop on the seeded request stream, mixed precision, then
    FP64 on the same stream. A job's result in the mix is bitwise the job
    run alone (tested), so the FP64 arm's per-job surface temperatures are
    the FP64 results of each job alone: max_err_K_vs_fp64 is the largest
    difference over all jobs."""
    from illum_gb300 import serve
    reqs = serve.request_stream(nreq, rate_hz=rate, step_scale=scale)
    out = {}
    for prec in (ig.PREC_MIXED, ig.PREC_FP64):
        srv = serve.Server(budget_bytes=int(48e9), precision=prec,
                           tol=MIXED_TOL if prec == ig.PREC_MIXED else 1e-10,
                           refine_every=MIXED_REFINE if prec == ig.PREC_MIXED else 0)
        clk = ClockSampler(0).start()
        t0 = time.perf_counter()
        done = srv.run(reqs)
        wall = time.perf_counter() - t0
        cl = clk.stop()
        lat = np.array([j.t_done - j.req.arrival for j in done])
        fs = sum(j.nfaces * j.req.nsteps for j in done)
        out[prec] = dict(value=fs / wall, wall=wall, p50=float(np.percentile(lat, 50) * 1000),
                         p99=float(np.percentile(lat, 99) * 1000), tsurf={j.req.rid: j.tsurf for j in done},
                         rebuilds=srv.rebuilds, clocks=cl, n=len(done), steps=int(sum(j.req.nsteps for j in done)),
                         stats=srv.stats())
    m, d = out[ig.PREC_MIXED], out[ig.PREC_FP64]
    err = max(float(np.abs(m["tsurf"][k] - d["tsurf"][k]).max()) for k in m["tsurf"])
    return {"value": m["value"], "unit": UNIT, "steps": m["steps"], "p50_ms": m["p50"], "p99_ms": m["p99"],
            "dtype": mixed_dtype(),
            "config": {"workload": f"serving: the first {nreq} requests of the seeded stream (Poisson {rate:g}/s, "
                                   f"icosphere L3-L7, 20 craters 80-300 m, 1-20 rotations x 360-1440 steps per "
                                   f"rotation scaled by {scale:g}, materials as the batch workload), 48 GB admission "
                                   f"budget; FP64 arm radiosity tol 1e-10; mixed arm " + mixed_solve_label(),
                       "requests": nreq, "step_scale": scale},
            "requests_done": m["n"], "wall_s": m["wall"], "batch_rebuilds": m["rebuilds"],
            "fp64_value": d["value"], "fp64_p50_ms": d["p50"], "fp64_p99_ms": d["p99"], "fp64_wall_s": d["wall"],
            "mixed_vs_fp64": m["value"] / d["value"], "max_err_K_vs_fp64": err,
            "err_quantity": "surface temperature of every job at its last step",
            "server": m["stats"], "fp64_server": d["stats"], "clocks": m["clocks"], "fp64_clocks": d["clocks"]}


# ----------------------------------------------------------------- helpers
def slowest_rank_ms(ms, dist=None):
    """The timed region's length as the slowest replica saw it: max over
    ranks (NCCL tensor on the GPU, gloo on the CPU), ms itself for one
    process."""
    if dist is None:
        return float(ms)
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, facets, steps, slowest_ms):
    """Whole-job facet-steps/s of `world` independent replicas, each stepping
    `facets` facets `steps` times, timed by the slowest one."""
    return world * facets * steps / (slowest_ms / 1000.0)


def run_chunks(fn, first, n, nsun):
    """Call fn(first_sun, count) over [first, first+n) wrapping the sun table."""
    out = []
    s = first % nsun
    left = n
    while left > 0:
        k = min(left, nsun - s)
        out.append(fn(s, k))
        left -= k
        s = (s + k) % nsun
    return out


def mixed_vs_fp64_c1(ig, W, nchk, autotune):
    """The C1 workload in mixed precision against FP64 from the same initial
    state over nchk steps (same context, fresh thermal state each)."""
    ctx, N = W["ctx"], W["f"].shape[0]
    opts = c1_opts(ig, W["dt"], ig.PREC_FP64)
    tm = new_thermal(ig, ctx, W["z"], ig.PREC_FP64)
    ctx.run_steps(opts, 0, nchk)
    T64 = tm.T
    mopts = c1_opts(ig, W["dt"], ig.PREC_MIXED)
    tm = new_thermal(ig, ctx, W["z"], ig.PREC_MIXED)
    mtune = ctx.autotune(mopts, first_sun=0) if autotune else None
    clk = ClockSampler(0).start()
    ms, _ = ctx.bench_steps(mopts, 0, nchk, 256.0)
    cl = clk.stop()
    err = float(np.abs(T64 - tm.T).max())
    return {"value": N * nchk / (ms.sum() / 1000.0), "unit": UNIT, "steps": nchk, "max_err_K": err,
            "ms_per_step": float(ms.mean()), "radiosity_tol": MIXED_TOL, "radiosity_max_sweeps": MIXED_SWEEPS,
            "radiosity_refine_every": MIXED_REFINE,
            "autotune": mtune, "clocks": cl}


def standalone(args, ig, meshgen):
    """--workload batch|terrain|serve: that object alone as the line."""
    if args.workload == "batch":
        d = nested_batch(ig, meshgen, args.nested_steps, max(3, args.warmup))
    elif args.workload == "terrain":
        d = nested_terrain(ig, meshgen, args.terrain_n, args.terrain_cutoff_m, args.nested_steps, max(3, args.warmup),
                           args.terrain_sample)
    else:
        d = nested_serve(ig, args.serve_requests, args.serve_scale, args.serve_rate)
    line = {"metric": METRIC, "n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "data": "synthetic"}
    line.update(d)
    print(json.dumps(line), flush=True)


def main():
    global MIXED_REFINE
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1440)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-parity", action="store_true", help="skip the C1-size oracle comparison (and cpu_baseline)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="default launch shapes (profiling runs)")
    ap.add_argument("--mixed-steps", type=int, default=720, help="steps of the mixed-precision comparison run")
    ap.add_argument("--nested", default="batch,terrain,serve",
                    help="nested workloads of the default line (comma list, or 'none')")
    ap.add_argument("--nested-steps", type=int, default=60, help="timed steps of the batch and terrain objects")
    ap.add_argument("--workload", default="c1", choices=["c1", "batch", "serve", "terrain"],
                    help="c1: the default line; batch / terrain / serve: that nested object alone as the line")
    ap.add_argument("--terrain-n", type=int, default=1024, help="terrain grid points per side (1024: 2,093,058 facets)")
    ap.add_argument("--terrain-cutoff-m", type=float, default=None,
                    help="form-factor cutoff in m (default: the largest listed radius whose build fits the device; "
                         "the terrain configuration states 2000 m)")
    ap.add_argument("--terrain-sample", type=float, default=0.0025,
                    help="fraction of source facets whose visibility at the configured 2 km cutoff sizes F (0: skip)")
    ap.add_argument("--serve-requests", type=int, default=500)
    ap.add_argument("--serve-scale", type=float, default=0.02, help="step-count scale of the serving sample")
    ap.add_argument("--serve-rate", type=float, default=20.0, help="Poisson arrival rate of the serving stream (1/s)")
    ap.add_argument("--refine-every", type=int, default=MIXED_REFINE,
                    help="mixed path: RunOpts.refine_every (0: a refinement round per step; K: one pass per step)")
    args = ap.parse_args()
    MIXED_REFINE = args.refine_every

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        reference_arm(args, rank)
        return

    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))

    import __graft_entry__
    __graft_entry__.build()
    import illum_gb300 as ig
    from illum_gb300 import meshgen

    if args.workload != "c1":
        if rank == 0:
            standalone(args, ig, meshgen)
        return

    t_start = time.perf_counter()
    W = build_workload(ig, meshgen)
    ctx = W["ctx"]
    N = W["f"].shape[0]
    nsun = W["nsun"]
    opts = c1_opts(ig, W["dt"], ig.PREC_FP64)
    # launch shapes of the step kernels, timed on this workload (state untouched)
    tune = None if args.no_autotune else ctx.autotune(opts, first_sun=0)
    # warm-up (graph capture included)
    run_chunks(lambda s, k: ctx.bench_steps(opts, s, k, 256.0), 0, args.warmup, nsun)
    sun_pos = args.warmup
    if dist is not None:
        dist.barrier()
    clocks = ClockSampler(local).start()
    res = run_chunks(lambda s, k: ctx.bench_steps(opts, s, k, 256.0), sun_pos, args.steps, nsun)
    step_ms = np.concatenate([r[0] for r in res])
    sun_pos += args.steps
    clk = clocks.stop()
    total_ms = float(step_ms.sum())
    total_ms = slowest_rank_ms(total_ms, dist)
    value = replica_value(world, N, args.steps, total_ms)

    # per-phase breakdown (eager launches with events between phases)
    eager = c1_opts(ig, W["dt"], ig.PREC_FP64, use_graph=0)
    ctx.set_timing(True)    # resets the counters read by ctx.stats()
    nph = min(args.steps, 720)
    res = run_chunks(lambda s, k: ctx.bench_steps(eager, s, k, 256.0), sun_pos, nph, nsun)
    sun_pos += nph
    ph = {k: sum(r[1][k] for r in res) / nph for k in ("direct", "radiosity", "conduction")}
    st = ctx.stats()
    ctx.set_timing(False)
    sweeps_per_step = st["radiosity_sweeps"] / nph
    amb_per_step = st["ambiguous_facets"] / nph
    nz = CFG["nz"]
    peak, peak_kind = _peaks()
    bytes_cond = N * (2 * nz * 8 + 6 * 8)
    nnz = W["setup"]["nnz"]
    bytes_rad = sweeps_per_step * (nnz * (8 + 4) + N * (4 + 8 + 8 + 8))
    kern = {"conduction": (bytes_cond, ph["conduction"], "k_conduct_dfloat_c1"),
            "radiosity": (bytes_rad, ph["radiosity"], "k_radiosity64_c1")}
    dom = max(kern, key=lambda k: kern[k][1])
    b, ms, prof = kern[dom]
    achieved = b / (ms / 1000.0) / 1e9
    roofline = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind, "traffic": profile_traffic(prof),
                "traffic_unit": "bytes per launch", "traffic_source": f"profiles/{prof}.md (ncu, one launch)",
                "algorithmic_bytes": b, "avg_ms": ms}
    if dom == "radiosity":
        roofline["note"] = ("the FP64 matrix (10 B per stored entry) stays in the 129 MB L2 across the step's sweeps, "
                            "so this is an L2-streaming rate against the HBM denominator; the HBM-bound radiosity "
                            "roofline is the terrain object's")

    e2e = None
    if not args.no_e2e:
        nE = min(args.steps, 720)
        chunk = 72
        nE = max(chunk, nE - nE % chunk)
        suns = np.array([W["suns"][(sun_pos + i) % nsun] for i in range(nE)])
        t_tot = 0.0
        for i in range(0, nE, chunk):
            t0 = time.perf_counter()
            ctx.run_steps_host(opts, suns[i:i + chunk], record_tsurf=True)
            t_tot += time.perf_counter() - t0
        e2e = {"value": world * N * nE / t_tot, "unit": UNIT, "h2d_bytes_per_step": 56,
               "d2h_bytes_per_step": 8 * N, "steps": nE,
               "note": f"ilg_run_steps_host, {chunk} steps per call: every step's sun position host->device and "
                       "surface temperatures device->host inside the timed region, host wall clock"}
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank != 0:
        return

    walls = {"c1_s": time.perf_counter() - t_start}
    t0 = time.perf_counter()
    mixed = mixed_vs_fp64_c1(ig, W, args.mixed_steps, not args.no_autotune)
    walls["mixed_s"] = time.perf_counter() - t0
    parity, cpu = (None, None)
    if not args.no_parity:
        t0 = time.perf_counter()
        parity, cpu = parity_c1(ig, oracle_module(), W, PARITY_STEPS)
        walls["parity_s"] = time.perf_counter() - t0
    su = W["setup"]
    F_c1 = ctx.F_info()
    ctx.close()
    nested = {}
    which = [] if args.nested == "none" else [s for s in args.nested.split(",") if s]
    for name in which:
        t0 = time.perf_counter()
        try:
            if name == "batch":
                nested[name] = nested_batch(ig, meshgen, args.nested_steps, max(3, min(args.warmup, 10)))
            elif name == "terrain":
                nested[name] = nested_terrain(ig, meshgen, args.terrain_n, args.terrain_cutoff_m, args.nested_steps,
                                              max(3, min(args.warmup, 10)), args.terrain_sample)
            elif name == "serve":
                nested[name] = nested_serve(ig, args.serve_requests, args.serve_scale, args.serve_rate)
        except Exception as e:  # reported, not hidden
            nested[name] = {"error": f"{type(e).__name__}: {e}"}
        walls[name + "_s"] = time.perf_counter() - t0
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "arithmetic": "FP64 state, iterates, residuals and surface boundary; radiosity dot products and "
                          "conduction layer recurrences in double-float (FP32 pairs, ~2^-46 relative)",
            "config": {"workload": WORKLOAD_C1, "facets": N, "nnz": nnz, "l2": "256 MB flush before every timed step",
                       "parallelism": f"replicas x{world}"},
            "e2e": e2e, "gpu_launches": 5 * args.steps, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clk, "parity_vs_oracle": parity,
            "phases_ms_per_step": ph, "radiosity_sweeps_per_step": sweeps_per_step, "autotune": tune,
            "ambiguous_facets_per_step": amb_per_step,
            "direct_samples_per_s": (N * (len(W["disk"]) - 1) / (ph["direct"] * 1e-3) if ph.get("direct") else None),
            "visibility_rays_per_s": su["visibility_rays"] / su["form_factors_s"],
            "horizon_rays_per_s": su["horizon_rays"] / su["horizons_s"],
            "setup_s": {k: su[k] for k in ("bvh_s", "horizons_s", "form_factors_s")},
            "mixed": mixed, "F": F_c1, "bench_wall_s": walls}
    line.update(nested)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
