"""Continuous-batching request loop for thermal-model jobs.

A job is a shape model with a spin state and a material: its mesh is
generated, its LBVH, horizons and form factors are built, and its time
steps run until its last sun position. Requests arrive over time; an
admission thread admits them in arrival order while the estimated device
footprint of the admitted jobs stays under a budget and hands each to a pool
of set-up workers, which build jobs concurrently, each context on its own
CUDA stream (overlapping one another and the steps already running). The
stepping loop keeps the admitted jobs in one batch (ilg_batch_*): one launch
per phase steps every job, each at its own dt, depth grid and sun table. A
job that finishes is read out and switched off in place; the batch is
rebuilt (state written back to the contexts, a new batch formed, finished
jobs' memory released) when new jobs are waiting, at most every
min_rebuild_s, or when nothing in it is running. A job's results do not
depend on which other jobs shared its batch (bitwise, for a fixed
precision).
"""
from __future__ import annotations

import queue
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np

import illum_gb300 as ig
from illum_gb300 import meshgen

AU_KM = meshgen.AU_KM


@dataclass
class Request:
    rid: int
    arrival: float             # seconds after the start of the run
    level: int
    seed: int
    rotations: float
    steps_per_rot: int
    nz: int
    ti: float
    period_h: float
    n_craters: int = 20
    nsteps: int = 0


@dataclass
class Job:
    req: Request
    ctx: object = None
    tm: object = None
    opts: object = None
    nfaces: int = 0
    footprint: int = 0
    t_ready: float = 0.0
    t_done: float = 0.0
    tsurf: np.ndarray = None
    finished: bool = False


def request_stream(n: int, rate_hz: float = 20.0, seed: int = 4242, levels=(3, 4, 5, 6, 7),
                   rotations=(1, 20), steps_per_rot=(360, 1440), step_scale: float = 1.0):
    """Seeded request stream: Poisson arrivals at rate_hz; level uniform over
    `levels` (log-uniform facet count); integer rotations and steps per
    rotation uniform in their ranges; nz, thermal inertia and period drawn as
    in the batched workload. step_scale < 1 shortens every job (a bounded
    sample of the same stream)."""
    u = meshgen.uniform(seed, 20, n)
    arrivals = np.cumsum(-np.log1p(-u) / rate_hz)
    out = []
    for k in range(n):
        w = meshgen.uniform(seed + 7919 * (k + 1), 21, 8)
        level = levels[min(len(levels) - 1, int(w[0] * len(levels)))]
        rot = rotations[0] + min(rotations[1] - rotations[0], int(w[1] * (rotations[1] - rotations[0] + 1)))
        spr = steps_per_rot[0] + int(w[2] * (steps_per_rot[1] - steps_per_rot[0]))
        nz = 30 + min(50, int(w[3] * 51))
        ti = float(np.exp(np.log(50.0) + w[4] * (np.log(2000.0) - np.log(50.0))))
        period = 2.0 + 10.0 * w[5]
        r = Request(rid=k, arrival=float(arrivals[k]), level=level, seed=seed * 10 + k, rotations=rot,
                    steps_per_rot=spr, nz=nz, ti=ti, period_h=period)
        r.nsteps = max(1, int(round(rot * spr * step_scale)))
        out.append(r)
    return out


def footprint_bytes(level: int, nz: int, nphi: int, precision: int) -> int:
    """A priori estimate of the device bytes a job holds while it runs (its
    context plus its copy in a batch): geometry + LBVH + horizons ~ (400 +
    8 nphi) B per facet, layer state nz * (4|8) B twice, ~12 facet arrays of
    8 B twice, and form factors estimated at 150 entries per facet * 30 B
    (CSR, row-tile and bf16 copies). The server replaces it by the measured
    footprint once the job is built (Server._build_one)."""
    n = 20 * 4 ** level
    s_t = 4 if precision == ig.PREC_MIXED else 8
    return int(n * (400 + 8 * nphi + 2 * nz * s_t + 2 * 12 * 8 + 150 * 30))


class Server:
    def __init__(self, budget_bytes: int, precision: int = ig.PREC_MIXED, chunk_steps: int = 30, nphi: int = 32,
                 tol: float = 1e-3, solar: float = 1361.0, setup_workers: int = 4, min_rebuild_s: float = 0.25,
                 refine_every: int = 4):
        self.budget = budget_bytes
        self.workers = max(1, setup_workers)
        self.min_rebuild_s = min_rebuild_s
        self.precision = precision
        self.chunk = chunk_steps
        self.nphi = nphi
        self.tol = tol
        self.refine_every = refine_every if precision == ig.PREC_MIXED else 0
        self.solar = solar
        self.used = 0
        self.lock = threading.Condition()
        self.ready: "queue.Queue[Job]" = queue.Queue()
        self.done: list = []
        self.t0 = 0.0
        self.error = None
        self.max_used = 0              # largest reserved total (estimates, then measured footprints)
        self.per_facet = {}            # level -> largest measured bytes per facet of a built job
        self.est_ratio = []            # measured / reserved per job
        self.setup_s = []
        self.phase_s = []              # per job: mesh, LBVH, horizons, form factors, suns + thermal (s)
        self.first_building = set()    # levels whose first job is being built

    # -------------------------------------------------------------- setup
    def build_job(self, r: Request) -> Job:
        # craters as in the CPU-runnable configuration (20 caps, 80-300 m), no
        # extra radial roughness
        t = [time.perf_counter()]
        v, f = meshgen.icosphere_craters(r.level, r.seed, sigma_m=0.0, n_craters=r.n_craters, dmin_m=80.0,
                                         dmax_m=300.0)
        t.append(time.perf_counter())
        ctx = ig.IllumContext(v, f)
        t.append(time.perf_counter())
        ctx.make_horizons(nphi=self.nphi)
        t.append(time.perf_counter())
        ctx.set_insolation(1, 0, self.solar)
        ctx.compute_F(albedo=0.1, fetch=False)
        # row tiles of ~200k entries: the batch, not one job, fills the GPU
        ctx.set_radiosity_blocks(ig.radiosity_blocks_for(ctx.F_info()["nnz"]))
        t.append(time.perf_counter())
        period = r.period_h * 3600.0
        dt = period / r.steps_per_rot
        ctx.set_suns(meshgen.spin_sun_positions(r.nsteps, period, dt), ig.fib_spiral(100))
        tm = ig.ThermalModel(ctx, meshgen.geometric_depths(r.nz), r.ti, 1.05e6, 200.0, emissivity=0.95,
                             bc_mode=ig.BC_NEWTON, precision=self.precision)
        t.append(time.perf_counter())
        self.phase_s.append(np.diff(t))
        # mixed: one refinement round per step (one bf16 sweep), or with
        # refine_every = K one pass per step (f32 form factors every K-th)
        opts = ig.RunOpts(dt=dt, tol=self.tol, max_sweeps=1 if self.precision == ig.PREC_MIXED else 200,
                          use_radiosity=1, use_graph=1,
                          precision=self.precision, coupling=ig.COUPLE_DIRECT, refine_every=self.refine_every)
        return Job(req=r, ctx=ctx, tm=tm, opts=opts, nfaces=f.shape[0])

    def _estimate(self, r: Request) -> int:
        """Bytes to reserve for r (called with the lock held): once a job of
        the same level has been built, 1.5 x the largest measured bytes per
        facet at that level (form factors per facet vary with the craters:
        up to 1.43 x a level's earlier maximum in the 500-request sample);
        before that, 4 x the a priori estimate (a level-7 job measured up
        to 3.45 x it at full step counts)."""
        pf = self.per_facet.get(r.level)
        if pf is not None:
            return int(1.5 * pf * 20 * 4 ** r.level)
        return 4 * footprint_bytes(r.level, r.nz, self.nphi, self.precision)

    def _build_one(self, r: Request, need: int):
        try:
            t0 = time.perf_counter()
            job = self.build_job(r)
            self.setup_s.append(time.perf_counter() - t0)
            # the measured footprint: the context, and its copy in a batch
            actual = 2 * job.ctx.device_bytes()
            with self.lock:
                self.used += actual - need
                self.max_used = max(self.max_used, self.used)
                self.per_facet[r.level] = max(self.per_facet.get(r.level, 0.0), actual / job.nfaces)
                self.first_building.discard(r.level)
                self.lock.notify_all()
            self.est_ratio.append(actual / need)
            job.footprint = actual
            job.t_ready = time.perf_counter() - self.t0
            self.ready.put(job)
        except Exception as e:   # surfaced by run()
            self.error = e
            with self.lock:
                self.first_building.discard(r.level)
                self.lock.notify_all()
            self.ready.put(None)

    def stats(self) -> dict:
        """Admission and set-up figures of the last run."""
        er = np.array(self.est_ratio) if self.est_ratio else np.zeros(1)
        st = np.array(self.setup_s) if self.setup_s else np.zeros(1)
        ph = np.array(self.phase_s) if self.phase_s else np.zeros((1, 5))
        names = ("mesh", "lbvh", "horizons", "form_factors", "suns_thermal")
        return {"setup_phase_sum_s": {n: float(x) for n, x in zip(names, ph.sum(0))},
                "budget_bytes": self.budget, "max_reserved_bytes": self.max_used,
                "max_reserved_over_budget": self.max_used / self.budget,
                "measured_over_reserved": {"max": float(er.max()), "median": float(np.median(er))},
                "setup_s": {"median": float(np.median(st)), "max": float(st.max()), "sum": float(st.sum())},
                "setup_workers": self.workers, "batch_rebuilds": getattr(self, "rebuilds", 0)}

    def _setup_loop(self, reqs):
        pool = ThreadPoolExecutor(max_workers=self.workers)
        try:
            for r in reqs:
                wait = r.arrival - (time.perf_counter() - self.t0)
                if wait > 0:
                    time.sleep(wait)
                with self.lock:
                    # a level's first job is built alone: the jobs after it
                    # reserve what it measured
                    while r.level in self.first_building and not self.error:
                        self.lock.wait()
                    need = self._estimate(r)
                    while self.used + need > self.budget and self.used > 0 and not self.error:
                        self.lock.wait()
                    self.used += need
                    self.max_used = max(self.max_used, self.used)
                    if r.level not in self.per_facet:
                        self.first_building.add(r.level)
                if self.error:
                    break
                pool.submit(self._build_one, r, need)
        except Exception as e:   # surfaced by run()
            self.error = e
        finally:
            pool.shutdown(wait=True)
            self.ready.put(None)

    # -------------------------------------------------------------- stepping
    def _release(self, j: Job) -> None:
        j.ctx.close()
        j.ctx = j.tm = None
        with self.lock:
            self.used -= j.footprint
            self.lock.notify_all()

    def run(self, reqs):
        """Serve the request stream; returns the finished jobs."""
        self.t0 = time.perf_counter()
        th = threading.Thread(target=self._setup_loop, args=(reqs,), daemon=True)
        th.start()
        active: list = []          # jobs in the current batch (finished ones switched off)
        pending: list = []         # built, waiting for the next batch
        batch = None
        last_rebuild = -1e30
        setup_open = True
        self.rebuilds = 0
        while True:
            running = [j for j in active if not j.finished]
            # take whatever is ready (block only when there is nothing to step)
            while True:
                try:
                    job = self.ready.get(block=not running and not pending and setup_open, timeout=0.05)
                except queue.Empty:
                    break
                if job is None:
                    setup_open = False
                    break
                pending.append(job)
            if self.error:
                break
            now = time.perf_counter() - self.t0
            if (pending and (not running or now - last_rebuild >= self.min_rebuild_s)) or \
                    (batch is not None and not running):
                if batch is not None:
                    batch.sync()
                    batch.close()
                    batch = None
                for j in active:
                    if j.finished:
                        self._release(j)
                active = running + pending
                pending = []
                running = list(active)
                if active:
                    batch = ig.Batch([j.ctx for j in active], [j.opts for j in active])
                    self.rebuilds += 1
                    last_rebuild = now
            if not running:
                if not setup_open and not pending:
                    break
                continue
            steps = min(self.chunk, max(1, min(j.req.nsteps - self._steps_done(j) for j in running)))
            batch.run(steps)
            act, done_steps, _ = batch.status()
            now = time.perf_counter() - self.t0
            for k, (j, d) in enumerate(zip(active, done_steps)):
                j._done = int(d)
                if not j.finished and d >= j.req.nsteps:
                    j.tsurf = batch.tsurf(k)
                    j.t_done = now
                    j.finished = True
                    batch.set_active(k, False)
                    self.done.append(j)
        if batch is not None:
            batch.sync()
            batch.close()
        for j in active:
            if j.ctx is not None:
                self._release(j)
        th.join()
        if self.error:
            raise self.error
        return self.done

    @staticmethod
    def _steps_done(j) -> int:
        return getattr(j, "_done", 0)
