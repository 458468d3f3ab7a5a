/*
 * illum_gb300.h — C ABI of the GB300-native illumination + thermal library.
 *
 * Each entry point replaces one piece of sampotter/illum's path (paths are
 * relative to the reference project's root):
 *
 *   ilg_ctx_create          illum_context::illum_context(obj_path)
 *                           (src/cpp/illum.cpp:22-27, src/cpp/illum.hpp:9-10):
 *                           triangles in, acceleration structure (here an LBVH
 *                           on the GPU) built.
 *   ilg_compute_F/_get_F    illum_context::compute_F (src/cpp/illum.cpp:31-237,
 *                           src/cpp/illum.hpp:18-20)
 *   ilg_set_F               loading form_factors_file (src/cpp/illum_cli.cpp:385-389)
 *   ilg_make_horizons       illum_context::make_horizons (src/cpp/illum.cpp:326-363)
 *   ilg_get/set_horizons    save_horizons / load_horizons (src/cpp/illum.cpp:365-375)
 *   ilg_direct_radiosity    illum_context::get_direct_radiosity
 *                           (src/cpp/illum.cpp:382-466)
 *   ilg_fib_spiral          fib_spiral (src/cpp/illum.cpp:468-483)
 *   ilg_radiosity_solve     arma_util::forward_solve + the Gauss-Seidel loop
 *                           (src/cpp/arma_util.cpp:4-17, src/cpp/illum_cli.cpp:425-440)
 *   ilg_thermal_init/_step/_get
 *                           thermal_model ctor / step / T, F members
 *                           (src/cpp/thermal.hpp:17-105)
 *   ilg_run_steps           the time-step loop of do_radiosity_task
 *                           (src/cpp/illum_cli.cpp:403-468)
 *   ilg_trace               BVH::getIntersection (call sites src/cpp/illum.cpp:73,301)
 *   conductionq_/conductiont_
 *                           the Fortran subroutines' exact C symbols
 *                           (src/cpp/conduction.cpp:3-6,17-20)
 *   ilg_conductionq_batch   many conductionQ columns in one call
 *
 * Conventions: every ilg_* function returns ILG_OK (0) or a negative status;
 * ilg_last_error() gives the message of the calling thread's last failure.
 * All array arguments are HOST pointers owned by the caller (device state is
 * owned by the context). Dense matrices use the reference's column-major
 * (Armadillo) layout. A context is not thread-safe; separate contexts are
 * independent. Lengths are in the mesh's unit (km by default, as the
 * reference), temperatures in K, fluxes in W/m^2.
 */
#ifndef ILLUM_GB300_H
#define ILLUM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ILG_OK 0
#define ILG_ERR_ARG (-1)      /* invalid argument or call order */
#define ILG_ERR_CUDA (-2)     /* CUDA runtime error */
#define ILG_ERR_NAN (-3)      /* NaN form factor (reference throws, illum.cpp:121-123) */
#define ILG_ERR_PIVOT (-4)    /* zero pivot in a tridiagonal solve (tridag.for stops) */
#define ILG_ERR_NOMEM (-5)    /* device allocation failed */
#define ILG_ERR_DEVICE (-6)   /* a kernel reported an error (stack overflow, wait limit) */
#define ILG_ERR_NOTCONV (-7)  /* radiosity did not reach the tolerance in max_sweeps */

typedef struct ilg_ctx ilg_ctx;

/* Precision of the time-step loop. */
#define ILG_PREC_FP64 0       /* plain method: FP64 radiosity and conduction */
#define ILG_PREC_MIXED 1      /* BF16 form factors + FP32 conduction, FP64 residual refinement */

/* Surface boundary of the conduction step. */
#define ILG_BC_LINEARISED 0   /* conductionQ.f:76-82 (one-shot linearisation) */
#define ILG_BC_NEWTON 1       /* Newton solve of emiss*sigma*Ts^4 at the new time level */

const char* ilg_last_error(void);
int ilg_version(void);

/* ---- context (illum_context) ------------------------------------------- */
/* verts: nv x 3 float (row-major xyz); tris: nt x 3 int32 vertex indices;
 * normals: nt x 3 float face normals, or NULL to use the normalised
 * (v1-v0)x(v2-v0) of each face. */
int ilg_ctx_create(const float* verts, int nv, const int32_t* tris, int nt,
                   const float* normals, ilg_ctx** out);
int ilg_ctx_destroy(ilg_ctx* ctx);
int ilg_ctx_num_faces(const ilg_ctx* ctx);
int ilg_ctx_info(const ilg_ctx* ctx, int64_t* bvh_nodes, int* bvh_depth);
/* Device bytes the context holds now (every buffer it allocated: geometry,
 * LBVH, horizons, form factors and their row tiles, thermal state, step
 * scratch). No reference counterpart: the serving loop admits jobs by this
 * footprint. */
int ilg_ctx_device_bytes(const ilg_ctx* ctx, int64_t* bytes);
/* High-water marks of the current device's stream-ordered allocation pool,
 * which every context allocates from: bytes in use and bytes reserved, since
 * the last reset (reset != 0 clears both after reading). No reference
 * counterpart: sizing aid for builds that approach the device's memory. */
int ilg_device_pool_high(int64_t* used_high, int64_t* reserved_high, int reset);

/* ---- closest / any hit (BVH::getIntersection) ----------------------------- */
/* hit[r] = index of the closest triangle hit by ray r (or the first found
 * with any_hit != 0), -1 for none; t[r] its ray parameter (may be NULL). */
int ilg_trace(ilg_ctx* ctx, int nrays, const float* orig, const float* dir, int any_hit,
              int32_t* hit, double* t);

/* ---- map renderer (illum_renderer_cli) ------------------------------------ */
/* One closest-hit ray per pixel (src/cpp/illum_renderer_cli.cpp:228-276):
 * mode 0 orthographic view from azimuth/elevation (degrees) at 1.1 x the
 * model radius, mode 1 equal-area cylindrical map. facet_out: height x width
 * row-major facet indices, -1 where no facet is hit. Colouring and the
 * image file are the caller's (illum_gb300.render). */
int ilg_render(ilg_ctx* ctx, int mode, double az_deg, double el_deg, int width, int height,
               int32_t* facet_out);

/* ---- form factors (compute_F) -------------------------------------------- */
/* Visibility + form factors, rows scaled by albedo (albedo: nt values, or
 * NULL to use albedo_scalar). Result stays on the device as CSR by receiver
 * row; *nnz receives its size and *rays the number of visibility rays. */
int ilg_compute_F(ilg_ctx* ctx, const double* albedo, double albedo_scalar, double offset,
                  int64_t* nnz, int64_t* rays);
/* As ilg_compute_F, keeping only pairs whose centroids are at most `cutoff`
 * apart (mesh units). The reference has no cutoff; it makes large terrain
 * patches tractable (a facet then sees O(cutoff^2) facets, not O(N)). */
int ilg_compute_F_cutoff(ilg_ctx* ctx, const double* albedo, double albedo_scalar, double offset,
                         double cutoff, int64_t* nnz, int64_t* rays);
/* Size of F from a sample of source facets, without building it (no
 * reference counterpart; it sizes a cutoff before committing memory):
 * visibility and form factors of the listed sources only (distinct, in
 * [0, nt)) with the given cutoff (0: none). per_source[q] receives the
 * nonzero entries of column sources[q] (what compute_F would store for that
 * source); within_radius[k] (may be NULL) the sample's nonzero entries whose
 * centroid distance is at most radii[k] (mesh units); *rays (may be NULL)
 * the visibility rays cast. */
int ilg_visibility_sample(ilg_ctx* ctx, double cutoff, double offset, const int32_t* sources, int nsrc,
                          const double* radii, int nradii, int64_t* per_source, int64_t* within_radius,
                          int64_t* rays);
/* rowptr: nt+1, col: nnz, val: nnz */
int ilg_get_F(ilg_ctx* ctx, int64_t* rowptr, int32_t* col, double* val);
int ilg_set_F(ilg_ctx* ctx, int64_t nnz, const int64_t* rowptr, const int32_t* col,
              const double* val);
/* Sizes of the device copy: entries, entries stored for the radiosity
 * sweeps (row tiles padded to whole thread runs), row tiles, rows with
 * entries (any may be NULL). */
int ilg_F_info(const ilg_ctx* ctx, int64_t* nnz, int64_t* stored_entries, int* row_tiles,
               int* active_rows);
/* The radiosity row tiles of the context's form factors (a diagnostic of
 * the GPU layout, no counterpart in the reference): per tile, the entries
 * each of its threads streams per sweep, its rows and its halo facets. The
 * first min(cap, *ntiles) tiles are written; *ntiles receives the count. */
int ilg_F_tiles(const ilg_ctx* ctx, int cap, int* entries_per_thread, int* rows, int* halo, int* ntiles);

/* ---- horizons ----------------------------------------------------------- */
int ilg_make_horizons(ilg_ctx* ctx, int nphi, double theta_eps, double offset);
/* make_horizons with a separate horizon mesh (illum_context::
 * set_horizon_obj_file, src/cpp/illum.hpp:36-37, used at
 * src/cpp/illum.cpp:333-349): every facet of the context keeps its own
 * centroid, normal and frame, and its horizon rays are cast against the
 * triangles verts / tris (nv x 3 float, nt x 3 int32), e.g. a larger patch
 * of terrain around the mesh. The horizon mesh's LBVH lives for the call. */
int ilg_make_horizons_mesh(ilg_ctx* ctx, const float* verts, int nv, const int32_t* tris, int nt, int nphi,
                           double theta_eps, double offset);
/* out: nphi x nt column-major (nphi zenith angles per facet) */
int ilg_get_horizons(ilg_ctx* ctx, double* out);
int ilg_set_horizons(ilg_ctx* ctx, int nphi, const double* h);

/* ---- direct insolation -------------------------------------------------- */
/* Insolation options: norm_mode 0 divides the lit count by nphi - 1 as the
 * reference does (illum.cpp:441), 1 by the number of samples used;
 * interp 0 keeps the reference's threshold h[k] + t*dphi (illum.cpp:434),
 * 1 interpolates h[k]..h[k+1]; solar_const is the flux at 1 AU
 * (1372 in illum.cpp:451). */
int ilg_set_insolation(ilg_ctx* ctx, int norm_mode, int interp, double solar_const);
void ilg_fib_spiral(double* xy /* n x 2 column-major */, int n);
/* sun: 3 doubles (km); disk_xy: ndisk x 2 column-major (ndisk-1 samples
 * used); out: nt doubles. */
int ilg_direct_radiosity(ilg_ctx* ctx, const double* sun, const double* disk_xy, int ndisk,
                         double* out);

/* ---- radiosity ---------------------------------------------------------- */
/* Solves (I - F) x = E for the context's F to ||(I-F)x - E||_2 <= tol
 * (at most max_sweeps sweeps). x: nt doubles out; *res the residual bound
 * and *sweeps the sweeps used (either may be NULL). */
int ilg_radiosity_solve(ilg_ctx* ctx, const double* E, double tol, int max_sweeps, double* x,
                        double* res, int* sweeps);

/* Cut the context's radiosity row tiles for `blocks` blocks (0: every block
 * the device holds at once, the default), rebuilding them if form factors
 * exist. Fewer, larger tiles suit a mesh that is solved beside others (a
 * batch or the serving loop): each tile costs a fixed set-up besides its
 * entries. A context's results depend on its tiling in the last bits only,
 * and are the same alone and in a batch for a given setting. No reference
 * counterpart. */
int ilg_set_radiosity_blocks(ilg_ctx* ctx, int blocks);
/* The reference's own solve: a forward solve of L x = E with
 * L = I - tril(F), then gs_steps Gauss-Seidel sweeps x = L^{-1}(E - U x),
 * U = -triu(F), in natural row order (src/cpp/arma_util.cpp:4-17,
 * src/cpp/illum_cli.cpp:425-433; its default gs_steps is 1,
 * illum_cli.cpp:607-610). Each row sums in the reference's order, so x
 * equals the CPU restatement's bit for bit. *res (may be NULL) receives
 * ||(I - F) x - E||_2. Rows run level by level (rows whose lower columns
 * are all final); the levels are found on the first call after F changes. */
int ilg_radiosity_solve_gs(ilg_ctx* ctx, const double* E, int gs_steps, double* x, double* res);
/* Number of dependency levels of the fixed-sweep solve (0 before its first
 * use on the current form factors). */
int ilg_radiosity_levels(const ilg_ctx* ctx, int* levels);
/* Which solve the fused FP64 steps run: ILG_RAD_TOL (default) solves to the
 * run's tolerance; ILG_RAD_GS runs the reference's fixed sweeps as
 * ilg_radiosity_solve_gs with gs_steps (single contexts, FP64 only). */
#define ILG_RAD_TOL 0
#define ILG_RAD_GS 1
int ilg_set_radiosity_mode(ilg_ctx* ctx, int mode, int gs_steps);

/* ---- thermal model -------------------------------------------------------- */
/* z, ti, rhoc: nz per-layer values (the reference shares one profile across
 * facets, thermal.hpp:23-42); T0: uniform start temperature, or T0_full
 * ((nz+1) x nt column-major, row 0 = surface) when non-NULL. */
int ilg_thermal_init(ilg_ctx* ctx, int nz, const double* z, const double* ti, const double* rhoc,
                     double T0, const double* T0_full, double emissivity, double Fgeotherm,
                     int bc_mode, int precision);
/* thermal_model::step(dt, Q): Q is nt doubles (host). */
int ilg_thermal_step(ilg_ctx* ctx, double dt, const double* Q);
/* T: (nz+1) x nt column-major (row 0 = surface temperature); Fsurf, Qprev: nt.
 * Any pointer may be NULL. */
int ilg_thermal_get(ilg_ctx* ctx, double* T, double* Fsurf, double* Qprev);

/* ---- fused time-step loop (do_radiosity_task's step lambda) ---------------- */
/* Run-level options for ilg_run_steps. */
typedef struct ilg_run_opts {
  double dt;               /* s */
  double tol;              /* radiosity tolerance (2-norm of the residual) */
  int max_sweeps;          /* radiosity sweep limit */
  int use_radiosity;       /* 0: rad = E (no F) */
  int use_graph;           /* capture the step in a CUDA graph */
  int precision;           /* ILG_PREC_FP64 / ILG_PREC_MIXED */
  int coupling;            /* ILG_COUPLE_REFERENCE / ILG_COUPLE_DIRECT */
  int refine_every;        /* mixed precision only. 0: each step's solve runs refinement rounds
                              (residual with the f32 form factors, bf16 sweeps) until tol or
                              max_sweeps. K >= 1: one pass over the matrix per step from the
                              warm start s0 = s(n) + F (E(n+1) - E(n)) (the next frame's direct
                              flux is computed ahead; needs device-resident suns, not
                              ilg_run_steps_host); every K-th step of a mesh (and its first)
                              applies the f32 form factors and keeps (s, x) as the reference,
                              the steps between apply the bf16 copy to the change since then,
                              s = s_ref + F~ (x - x_ref). The reference carries over to the
                              context's next run and through batches (tol and max_sweeps
                              unused) */
  int layer_rounding;      /* mixed precision only. 0: the FP32 layers' updates T + dT round to
                              nearest; 1: without bias (up one ulp with probability remainder /
                              ulp, from a hash of facet, layer and frame), so that increments
                              below half an ulp at depth are not lost over long runs */
} ilg_run_opts;

/* What the radiosity solve of a step starts from. ILG_COUPLE_REFERENCE is
 * the reference's E = -Fsurf + direct (src/cpp/illum_cli.cpp:411-421): the
 * conductive surface flux of the previous step is fed back through the
 * radiosity solve, and with a thin top layer (the millimetre first layer of
 * the benchmark profiles) the surface temperature then zig-zags from step
 * to step (the CPU restatement does the same; bounded on the 1,280- and
 * 5,120-facet crater meshes, with ~26x more sign changes of the step-to-step
 * change than E = direct). ILG_COUPLE_DIRECT starts from the direct
 * insolation alone (E = direct), so the radiosity solve redistributes
 * scattered sunlight and the conduction step receives it. Both are tested
 * against the CPU oracle. */
#define ILG_COUPLE_REFERENCE 0
#define ILG_COUPLE_DIRECT 1

/* Upload sun positions (nsun x 3, row-major, km) kept on the device for
 * ilg_run_steps; disk_xy as in ilg_direct_radiosity. */
int ilg_set_suns(ilg_ctx* ctx, int nsun, const double* suns, const double* disk_xy, int ndisk);
/* Advance nsteps steps using device-resident sun positions starting at
 * index first_sun. tsurf_out: nsteps x nt host array (NULL: none) receiving
 * the surface temperature after every step. */
int ilg_run_steps(ilg_ctx* ctx, const ilg_run_opts* opts, int first_sun, int nsteps,
                  double* tsurf_out);
/* Same, with the sun position of each step passed from the host: suns is
 * nsteps x 3. */
int ilg_run_steps_host(ilg_ctx* ctx, const ilg_run_opts* opts, int nsteps, const double* suns,
                       double* tsurf_out);
/* Measurement loop over device-resident suns: before every step a kernel
 * overwrites flush_mb MB of device memory (evicting L2), then the step runs
 * between two CUDA events on the context's stream. step_ms: nsteps device
 * times; with opts->use_graph == 0 phase_ms (3 values, may be NULL) receives
 * the summed direct / radiosity / conduction phase times. */
int ilg_bench_steps(ilg_ctx* ctx, const ilg_run_opts* opts, int first_sun, int nsteps, double flush_mb,
                    double* step_ms, double* phase_ms);
/* rad, rad_avg, therm_avg, therm_max: nt doubles each (any may be NULL). */
int ilg_get_outputs(ilg_ctx* ctx, double* rad, double* rad_avg, double* therm_avg,
                    double* therm_max);
/* Per-phase device times (ms) of the last ilg_run_steps call with timing
 * enabled, and per-call counters. */
int ilg_set_timing(ilg_ctx* ctx, int enable);

/* ---- bounded device waits (no reference counterpart) ------------------------- */
/* Test entry for the radiosity solver's grid barrier, whose waits are
 * bounded: one cooperative launch of `blocks` (1..8) blocks waits at a
 * barrier with the poll limit set to `polls` for that launch. With
 * unreachable != 0 the barrier expects one more arrival than there are
 * blocks, so every wait runs out: the call returns ILG_ERR_DEVICE ("grid
 * barrier wait exceeded its limit") and the context stays usable. With
 * unreachable == 0 the barrier opens and the call returns ILG_OK. The poll
 * limit is a per-device setting for the duration of the launch: do not run
 * radiosity solves on the same device meanwhile. */
int ilg_debug_barrier_timeout(ilg_ctx* ctx, int blocks, long long polls, int unreachable);
/* Test entry for the form-factor build: candidate pairs per source chunk
 * (process-wide; <= 0 restores the default of 2^29). A small value runs a
 * small mesh through the several-chunk path, whose matrix must equal the
 * one-chunk build's. Not for concurrent use with other builds. */
int ilg_debug_ff_chunk(long long pairs);

/* ---- launch-shape autotuner (no reference counterpart) ------------------------ */
/* Launch shapes of the step kernels. No result depends on them (every
 * facet's work is independent of the block it runs in, and the sums are
 * per facet), only the step's speed. */
typedef struct ilg_tune {
  int classify_threads;   /* direct-insolation pass 1, threads per block: 128, 256, 512 */
  int exact_facets;       /* direct-insolation pass 2, undecided facets per block: 4, 8, 16, 32 */
  int conduct_threads;    /* conduction, columns per block (single-mesh steps): 32, 64, 128 */
  double direct_us;       /* ilg_autotune: measured time of the chosen direct shapes (us per step) */
  double conduct_us;      /* ilg_autotune: measured time of the chosen conduction shape */
} ilg_tune;
/* Times every shape on the context's own workload for opts (sun position
 * first_sun) on scratch copies of the buffers the kernels write (the
 * context's state is not changed), keeps the fastest and returns it in
 * *chosen (may be NULL). Requires what ilg_run_steps requires. */
int ilg_autotune(ilg_ctx* ctx, const ilg_run_opts* opts, int first_sun, ilg_tune* chosen);
int ilg_set_tune(ilg_ctx* ctx, const ilg_tune* tune);
int ilg_get_tune(const ilg_ctx* ctx, ilg_tune* tune);

/* ---- thermal records (thermal_model record_stats) ---------------------------- */
/* Records, for each of the next `capacity` steps (ilg_run_steps,
 * ilg_run_steps_host, or a batch holding the context), 15 FP64 values: the
 * reference's 12 temperature statistics (thermal.hpp:86-126: Tmax, Tmin,
 * Tavg, Tstd over all layers and the surface; the same over the surface
 * row; the same over the bottom layer; std with N - 1) and three energy
 * sums: sum of area x absorbed flux Q, of area x emitted emiss sigma Ts^4,
 * of area x conducted Fsurf (area in the mesh's unit squared, fluxes in
 * W/m^2). Adds a reduction per step. capacity 0 stops recording. */
int ilg_record_thermal(ilg_ctx* ctx, int capacity);
/* out: count x 15 row-major (may be NULL); count = steps recorded. */
int ilg_get_thermal_records(ilg_ctx* ctx, double* out, int* count);
int ilg_get_stats(ilg_ctx* ctx, double* ms_direct, double* ms_radiosity, double* ms_conduction,
                  int64_t* ambiguous_facets, int64_t* radiosity_sweeps);

/* ---- batches: many meshes stepped together ---------------------------------- */
/* A batch steps its member contexts (each with horizons, suns set by
 * ilg_set_suns and an initialised thermal model) together: one launch per
 * phase for all members, each with its own opts (dt, tolerance, coupling,
 * radiosity on/off; the precision must be the same for all). Members start
 * at their first sun position and switch off after their last one. The
 * batch owns a copy of the members' state; ilg_batch_sync writes it back to
 * the contexts. A member's results are bitwise the same as when it runs
 * alone (per-mesh radiosity convergence, no cross-mesh reductions). A
 * member resumes at its context's frame count (sun index = frames done), so
 * after ilg_batch_sync the contexts can be regrouped into a new batch. */
typedef struct ilg_batch ilg_batch;
int ilg_batch_create(ilg_ctx** members, int n, const ilg_run_opts* opts, ilg_batch** out);
int ilg_batch_destroy(ilg_batch* batch);
int ilg_batch_run(ilg_batch* batch, int nsteps, int use_graph);
/* nsteps timed steps (L2 flushed by a flush_mb write before each);
 * step_ms: nsteps device times. */
int ilg_batch_bench(ilg_batch* batch, int nsteps, double flush_mb, double* step_ms);
/* Eager steps in the serial order with per-phase device times summed into
 * phase_ms[0..2] (direct, radiosity, conduction); step_ms[s] = their sum. */
int ilg_batch_bench_phases(ilg_batch* batch, int nsteps, double flush_mb, double* step_ms, double* phase_ms);
/* The direct-insolation launch shapes of the batch's steps (a batch starts
 * with its first member's; its conduction runs on the batch's own block
 * table): every supported shape timed on the batch's own workload (no state
 * changes), the fastest kept for the batch's later steps; *chosen (may be
 * NULL) receives the shapes and their time per step (direct_us). No result
 * depends on the shapes. */
int ilg_batch_autotune(ilg_batch* batch, ilg_tune* chosen);
/* per member (arrays of n, any may be NULL): still active, steps done in
 * total (including before this batch), radiosity sweeps of the last step */
int ilg_batch_status(ilg_batch* batch, int* active, int* steps_done, int* sweeps);
int ilg_batch_set_active(ilg_batch* batch, int member, int active);
int ilg_batch_get_tsurf(ilg_batch* batch, int member, double* out);
int ilg_batch_sync(ilg_batch* batch);

/* ---- conduction (Fortran ABI) -------------------------------------------- */
/* Exact symbols of conductionQ.f / conductionT.f as the reference's C++
 * wrapper declares them (conduction.cpp:3-6,17-20). Each runs one column on
 * the GPU; errors are reported on stderr (the Fortran has no status). */
void conductionq_(int* nz, const double z[], double* dt, double* Qn, double* Qnp1, double T[],
                  const double ti[], const double rhoc[], double* emiss, double* Tsurf,
                  double* Fgeotherm, double* Fsurf);
void conductiont_(int* nz, const double z[], double* dt, double T[], double* Tsurf,
                  double* Tsurfp1, const double ti[], const double rhoc[], double* Fgeotherm,
                  double* Fsurf);
/* ncol columns sharing z/ti/rhoc: T is nz x ncol column-major (each column's
 * nz layer temperatures contiguous); Qn, Qnp1, Tsurf, Fsurf are ncol values.
 * bc_mode as in ilg_thermal_init (Qn unused for ILG_BC_NEWTON). */
int ilg_conductionq_batch(int ncol, int nz, const double* z, double dt, const double* Qn,
                          const double* Qnp1, double* T, const double* ti, const double* rhoc,
                          double emiss, double* Tsurf, double Fgeotherm, double* Fsurf,
                          int bc_mode);

/* ---- conduction columns without allocation -------------------------------- */
/* No counterpart in the reference (which has no device code): a variant of
 * ilg_conductionq_batch for callers that cannot call cudaMalloc when they
 * step their columns, e.g. code whose device memory belongs to another
 * framework's caching allocator, or that runs under an exhausted memory
 * budget. It allocates no device memory: its scratch is one fixed
 * ILG_NOALLOC_SCRATCH_MB MiB array in the library, shared by all calls.
 *
 * T, Qn, Qnp1, Tsurf and Fsurf are DEVICE arrays of the current device; T is
 * layer-major (T[i * ncol + f], layer i of column f), the transpose of
 * ilg_conductionq_batch's host layout. z, ti, rhoc are nz host values. Qn
 * may be NULL (zero; unused for ILG_BC_NEWTON). Work is queued on `stream`
 * (a cudaStream_t; NULL = the legacy default stream) and the call returns
 * once it has finished.
 *
 * Scratch needed: about 8*ncol + 40*nz bytes, plus 8*nz*ncol for columns
 * deeper than 160 layers; a call needing more than the fixed array returns
 * ILG_ERR_ARG without touching the device (split the columns into smaller
 * calls). Every call looks up the scratch's address on the current device
 * (cudaGetSymbolAddress) before it queues anything. The call copies from
 * pageable host memory and synchronises its stream, so it must not be made
 * on a stream that is being captured into a graph: it checks, and returns
 * ILG_ERR_ARG before queuing anything. Calls on one device share that
 * device's scratch, so overlapping calls would race on it: calls on the same
 * device serialise on a lock of that device (calls on different devices do
 * not wait for one another). */
#define ILG_NOALLOC_SCRATCH_MB 16
int ilg_conductionq_batch_noalloc(int ncol, int nz, const double* z, double dt,
                                  const double* Qn, const double* Qnp1, double* T,
                                  const double* ti, const double* rhoc, double emiss,
                                  double* Tsurf, double Fgeotherm, double* Fsurf, int bc_mode,
                                  void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ILLUM_GB300_H */
