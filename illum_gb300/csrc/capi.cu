// capi.cu — the C ABI of include/illum_gb300.h: context lifecycle, the
// drop-in entry points for the reference's illum_context / thermal_model /
// conduction calls, and the fused time-step loop of do_radiosity_task
// (src/cpp/illum_cli.cpp:403-468), optionally captured as a CUDA graph.
#include <stdarg.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "geom.h"
#include "internal.cuh"

namespace ilg {

static thread_local std::string g_err;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}

Context::~Context() {
  if (graph) cudaGraphExecDestroy(graph);
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  if (pinned_aux) cudaFreeHost(pinned_aux);
  if (pinned_tsurf) cudaFreeHost(pinned_tsurf);
  for (cudaEvent_t e : slot_ev)
    if (e) cudaEventDestroy(e);
  // the stream itself goes last (owned_stream), after the buffers' frees
}

thread_local cudaStream_t t_alloc_stream = nullptr;

int alloc_pool_setup() {
  static std::mutex mu;
  static std::vector<int> done;
  int dev = 0;
  ILG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if (std::find(done.begin(), done.end(), dev) != done.end()) return ILG_OK;
  cudaMemPool_t pool;
  ILG_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
  uint64_t keep = UINT64_MAX;   // keep freed memory in the process's pool
  ILG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  done.push_back(dev);
  return ILG_OK;
}

// Return the pool's unused reserved memory to the device (after a build
// whose scratch was large, so that a later allocation outside the pool
// finds the memory free).
int pool_trim(cudaStream_t s) {
  int dev = 0;
  ILG_CUDA(cudaGetDevice(&dev));
  cudaMemPool_t pool;
  ILG_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
  ILG_CUDA(cudaStreamSynchronize(s));
  ILG_CUDA(cudaMemPoolTrimTo(pool, 0));
  return ILG_OK;
}

int read_device_errors(Context& c) {
  int h[DERR_COUNT];
  ILG_CUDA(cudaMemcpyAsync(h, c.derr.p, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  bool any = false;
  for (int i = 0; i < DERR_COUNT; ++i) any |= h[i] != 0;
  if (!any) return ILG_OK;
  ILG_CUDA(cudaMemsetAsync(c.derr.p, 0, sizeof(h), c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  if (h[DERR_NAN]) { set_error("computed a NaN form factor"); return ILG_ERR_NAN; }
  if (h[DERR_PIVOT]) { set_error("zero pivot in a conduction column"); return ILG_ERR_PIVOT; }
  if (h[DERR_STACK]) { set_error("BVH traversal stack overflow"); return ILG_ERR_DEVICE; }
  if (h[DERR_BARRIER]) { set_error("radiosity grid barrier wait exceeded its limit"); return ILG_ERR_DEVICE; }
  if (h[DERR_HORIZON]) { set_error("horizon bisection deeper than its table"); return ILG_ERR_DEVICE; }
  if (h[DERR_STREAM]) { set_error("radiosity entry-stream copy wait exceeded its limit"); return ILG_ERR_DEVICE; }
  set_error("device error flags set");
  return ILG_ERR_DEVICE;
}

static int set_disk(Context& c, const double* disk_xy, int ndisk) {
  if (!disk_xy || ndisk < 2) { set_error("disk_xy needs at least 2 rows"); return ILG_ERR_ARG; }
  std::vector<double> h(disk_xy, disk_xy + 2 * (size_t)ndisk);
  double rmax = 0.0;
  for (int s = 0; s < ndisk - 1; ++s) rmax = std::max(rmax, std::sqrt(h[s] * h[s] + h[ndisk + s] * h[ndisk + s]));
  std::vector<float> h32(h.begin(), h.end());
  ILG_TRY(c.disk.alloc(2 * (size_t)ndisk));
  ILG_TRY(c.disk32.alloc(2 * (size_t)ndisk));
  ILG_CUDA(cudaMemcpyAsync(c.disk.p, h.data(), h.size() * 8, cudaMemcpyHostToDevice, c.stream));
  ILG_CUDA(cudaMemcpyAsync(c.disk32.p, h32.data(), h32.size() * 4, cudaMemcpyHostToDevice, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  c.ndisk = ndisk;
  c.disk_rmax = rmax;
  return ILG_OK;
}

static void invalidate_graph(Context& c) {
  if (c.graph) cudaGraphExecDestroy(c.graph);
  if (c.graph_b) cudaGraphExecDestroy(c.graph_b);
  c.graph = nullptr;
  c.graph_b = nullptr;
  for (int& k : c.graph_key) k = -1;
}

// L2 eviction between benchmark steps: writes n float4 with the evict-last
// policy the radiosity sweeps use for the form-factor matrix, so lines kept
// at that priority are displaced too (the buffer is twice the L2).
__global__ void k_flush(float4* buf, size_t n, unsigned salt) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x, st = (size_t)gridDim.x * blockDim.x;
  float v = (float)salt;
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  for (; i < n; i += st)
    asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %1, %1, %1}, %2;" ::"l"(buf + i), "f"(v), "l"(pol)
                 : "memory");
}

// Advance every active mesh by one step; a mesh driven from its sun table
// switches itself off after its last sun position.
__global__ void k_advance(MeshDesc* md, int nmesh) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmesh) return;
  MeshDesc& M = md[m];
  if (!M.active) return;
  M.sun_idx += 1;
  M.frame += 1;
  M.done_steps += 1;
  if (!M.host_sun && M.sun_idx >= M.nsun) M.active = 0;
}

int advance_launch(const StepView& v, cudaStream_t s) {
  k_advance<<<div_up(v.nmesh, 128), 128, 0, s>>>(v.md, v.nmesh);
  ILG_CUDA(cudaGetLastError());
  return ILG_OK;
}

int flush_launch(float4* buf, size_t n, unsigned salt, cudaStream_t s) {
  k_flush<<<4 * 152, 256, 0, s>>>(buf, n, salt);
  ILG_CUDA(cudaGetLastError());
  return ILG_OK;
}

// A step's radiosity solve into v.rad: to the run's tolerance, or the
// reference's fixed-sweep Gauss-Seidel when the context is in that mode.
static int radiosity_phase(const StepView& v, const StepPlan& p, cudaStream_t s) {
  if (p.gs_ctx) return gs_step_launch(*p.gs_ctx, v, p.gs_steps, s);
  return radiosity_launch(v, v.rad, 1, p.precision, p.rad_grid, p.rad_inner, p.rad_lagged, s);
}

// One step of a view: direct -> radiosity -> conduction -> advance. With
// ev (4 events), the phase boundaries are recorded. The one-pass mixed
// solve also reads the next frame's direct flux: its steps compute that one
// (the current frame's came from the previous step or the serial prologue).
int enqueue_step(const StepView& v, const StepPlan& p, cudaStream_t s, cudaEvent_t* ev) {
  if (ev) ILG_CUDA(cudaEventRecord(ev[0], s));
  ILG_TRY(direct_launch(v, 0, p.precision == ILG_PREC_MIXED ? 1 : 0, p.rad_lagged ? 1 : 0, s));
  if (ev) ILG_CUDA(cudaEventRecord(ev[1], s));
  if (p.rad_on) ILG_TRY(radiosity_phase(v, p, s));
  if (ev) ILG_CUDA(cudaEventRecord(ev[2], s));
  ILG_TRY(conduction_launch(v, v.rad, p.precision, 1, p.nz_max, s, p.layer_sr));
  if (p.rec_on) ILG_TRY(record_launch(v, p.precision, v.cblocks ? v.ncblocks : div_up(v.nt, conduction_step_threads()), s));
  if (ev) ILG_CUDA(cudaEventRecord(ev[3], s));
  return advance_launch(v, s);
}

int StepPipe::init() {
  if (!s2) ILG_CUDA(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
  if (!fork) ILG_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  if (!join) ILG_CUDA(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
  return ILG_OK;
}

StepPipe::~StepPipe() {
  if (fork) cudaEventDestroy(fork);
  if (join) cudaEventDestroy(join);
  if (s2) cudaStreamDestroy(s2);
}

// The current frame's direct flux (and the next frame's for the one-pass
// mixed solve), before the first pipelined step of a run.
int enqueue_prologue(const StepView& v, const StepPlan& p, cudaStream_t s) {
  ILG_TRY(direct_launch(v, 0, p.precision == ILG_PREC_MIXED ? 1 : 0, 0, s));
  if (p.rad_lagged) ILG_TRY(direct_launch(v, 0, 1, 1, s));
  return ILG_OK;
}

int enqueue_serial_prologue(const StepView& v, const StepPlan& p, cudaStream_t s) {
  return p.rad_lagged ? direct_launch(v, 0, 1, 0, s) : ILG_OK;
}

// The step's radiosity reads its frame's E slot (the one-pass mixed solve
// also the next frame's); the direct insolation of the frame after those
// then writes its own slot on s2 while the conduction runs on s (the two
// share no array: the conduction reads the radiosity solution, or the
// current slot for meshes without form factors). Both finish before the
// advance. Results equal the serial order's bit for bit.
int enqueue_step_pipe(const StepView& v, const StepPlan& p, cudaStream_t s, const StepPipe& pipe) {
  if (p.rad_on) ILG_TRY(radiosity_phase(v, p, s));
  ILG_CUDA(cudaEventRecord(pipe.fork, s));
  ILG_CUDA(cudaStreamWaitEvent(pipe.s2, pipe.fork, 0));
  ILG_TRY(direct_launch(v, 0, p.precision == ILG_PREC_MIXED ? 1 : 0, p.rad_lagged ? 2 : 1, pipe.s2));
  ILG_CUDA(cudaEventRecord(pipe.join, pipe.s2));
  ILG_TRY(conduction_launch(v, v.rad, p.precision, 1, p.nz_max, s, p.layer_sr));
  if (p.rec_on) ILG_TRY(record_launch(v, p.precision, v.cblocks ? v.ncblocks : div_up(v.nt, conduction_step_threads()), s));
  ILG_CUDA(cudaStreamWaitEvent(s, pipe.join, 0));
  return advance_launch(v, s);
}

static int ensure_pinned(Context& c) {
  if (!c.pinned_aux) ILG_CUDA(cudaMallocHost((void**)&c.pinned_aux, 2 * sizeof(SunAux)));
  if (!c.pinned_tsurf) ILG_CUDA(cudaMallocHost((void**)&c.pinned_tsurf, 2 * (size_t)c.nt * 8));
  for (cudaEvent_t& e : c.slot_ev)
    if (!e) ILG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return ILG_OK;
}

// The context as a one-mesh view (device pointers of its own buffers).
static StepView solo_view(Context& c, int precision) {
  StepView v{};
  v.nt = c.nt;
  v.nmesh = 1;
  v.md = c.md.p;
  v.mesh_of = nullptr;
  v.cen = c.cen.p; v.nrm = c.nrm.p; v.frame32 = c.frame32.p;
  v.frame = c.frame.p; v.H = c.H.p; v.H32 = c.H32.p; v.hmm32 = c.hmm32.p; v.disk = c.disk.p; v.area = c.area.p;
  v.rec = c.rec_cap > 0 ? c.rec.p : nullptr;
  v.rec_part = c.rec_part.p;
  v.disk32 = c.disk32.p;
  v.ndisk = c.ndisk;
  v.suns = c.sun_aux.p;
  v.Tsurf = c.Tsurf.p; v.Fsurf = c.Fsurf.p; v.Qprev = c.Qprev.p; v.rad = c.rad.p; v.rad_avg = c.rad_avg.p;
  v.therm_avg = c.therm_avg.p; v.therm_max = c.therm_max.p; v.E = c.E.p; v.sprev = c.sprev.p;
  v.x32 = c.x32.p;
  v.T64 = nullptr; v.Tdf = c.Tdf.p; v.T32 = c.T32.p;
  v.coef64 = nullptr; v.coefdf = c.coefdf.p; v.coef32 = c.coef32.p;
  v.tiles = c.tiles.p; v.ntiles = c.have_F ? c.ntiles : 0;
  v.blk_start = c.sched_start.p; v.blk_tile = c.sched_tile.p; v.sched_grid = c.sched_grid;
  v.l2_stream = radiosity_l2_stream(c.tile_elems);
  v.t_cf = c.t_cf.p; v.t_vhi = c.t_vhi.p; v.t_vlo = c.t_vlo.p; v.t_vbf = c.t_vbf.p;
  v.t_row = c.t_row.p; v.t_halo = c.t_halo.p; v.t_start = c.t_start.p; v.t_scale = c.t_scale.p;
  v.tile_d2 = c.tile_d2.p;
  v.row_act = c.row_act.p; v.rperm = c.rperm.p;
  v.rbuf = c.xtmp.p;
  v.cblocks = nullptr; v.ncblocks = 0;
  v.work = c.work.p; v.counters = c.counters.p; v.derr = c.derr.p; v.mesh_flag = c.mesh_flag.p;
  v.barrier = c.barrier.p;
  v.rho64 = nullptr; v.rho32 = nullptr;
  v.tune = c.tune;
  (void)precision;
  return v;
}

// Host mirror of the context's mesh descriptor for a run (or a drop-in call).
MeshDesc solo_desc(const Context& c, const ilg_run_opts* o, int first_sun) {
  MeshDesc M{};
  M.facet0 = 0;
  M.nfacet = c.nt;
  M.nphi = c.nphi;
  M.interp = c.interp;
  M.H0 = 0;
  M.dphi = c.dphi;
  M.dphi32 = (float)c.dphi;
  M.denom = c.norm_mode == 0 ? (double)(c.nphi - 1) : (double)(c.ndisk - 1);
  M.nsamp = c.ndisk - 1;
  M.lit_all = (double)M.nsamp / M.denom;
  M.coupling = o ? o->coupling : ILG_COUPLE_DIRECT;
  M.sun0 = 0;
  M.nsun = c.nsun;
  M.sun_idx = first_sun;
  M.frame = c.frame_no;
  M.host_sun = 0;
  M.host_slot = c.nsun;
  M.nz = c.nz;
  M.coef0 = 0;
  M.T0 = 0;
  M.cs = c.cond_cs;
  M.tile0 = 0;
  M.ntiles = (o && o->use_radiosity && c.have_F) ? c.ntiles : 0;
  M.cb0 = 0;
  M.ncb = div_up(c.nt, conduction_step_threads());
  M.rec0 = 0;
  M.rec_cap = c.rec_cap;
  M.rec_frame0 = c.rec_frame0;
  M.tol2 = o ? o->tol * o->tol : 0.0;
  M.max_sweeps = o ? o->max_sweeps : 1;
  M.refine_every = o ? o->refine_every : 0;
  M.ref_age = c.ref_age;
  M.active = 1;
  return M;
}

// After a run's steps: the one-pass mixed solve's reference carries over to
// the context's next run (its age from the mesh table, s_ref and x_ref stay
// in xtmp); any other radiosity solve reuses those buffers, so it ends the
// reference.
static int keep_reference(Context& c, const StepPlan& p) {
  if (!p.rad_on) return ILG_OK;
  if (!p.rad_lagged) {
    c.ref_age = -1;
    return ILG_OK;
  }
  MeshDesc M;
  ILG_CUDA(cudaMemcpyAsync(&M, c.md.p, sizeof(MeshDesc), cudaMemcpyDeviceToHost, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  c.ref_age = M.ref_age;
  return ILG_OK;
}

static int upload_desc(Context& c, const MeshDesc& M) {
  c.mh = M;
  ILG_CUDA(cudaMemcpyAsync(c.md.p, &c.mh, sizeof(MeshDesc), cudaMemcpyHostToDevice, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  return ILG_OK;
}

// Per-context scratch of the step kernels, sized before any capture.
static int ensure_step_buffers(Context& c, int precision) {
  ILG_TRY(c.pipe.init());
  ILG_TRY(c.E.reserve(E_SLOTS * (size_t)c.nt));   // the direct flux of consecutive frames
  ILG_TRY(c.Q.reserve(c.nt));
  ILG_TRY(c.xtmp.reserve((size_t)6 * c.nt));   // radiosity E, two iterates, double-float copies of both and of E
  if (c.sprev.n < 2 * (size_t)c.nt) {
    ILG_TRY(c.sprev.alloc(2 * (size_t)c.nt));
    ILG_CUDA(cudaMemset(c.sprev.p, 0, 2 * (size_t)c.nt * sizeof(float2)));
  }
  if (precision == ILG_PREC_MIXED) ILG_TRY(c.x32.reserve((size_t)3 * c.nt));
  ILG_TRY(c.md.reserve(1));
  ILG_TRY(c.mesh_flag.reserve(1));
  return ILG_OK;
}

// host_driven: the sun of each step comes from the host slot, so no sun
// table is needed.
int check_run(Context& c, const ilg_run_opts* o, bool host_driven) {
  if (!o) { set_error("opts is NULL"); return ILG_ERR_ARG; }
  if (!c.have_thermal) { set_error("ilg_thermal_init has not been called"); return ILG_ERR_ARG; }
  if (!c.H.p || c.nphi < 2) { set_error("horizons are not set"); return ILG_ERR_ARG; }
  if (c.ndisk < 2) { set_error("sun disk samples are not set (ilg_set_suns)"); return ILG_ERR_ARG; }
  if (!host_driven && c.nsun < 1) { set_error("sun positions are not set (ilg_set_suns)"); return ILG_ERR_ARG; }
  if (!(o->dt > 0.0)) { set_error("dt must be > 0"); return ILG_ERR_ARG; }
  if (o->precision != ILG_PREC_FP64 && o->precision != ILG_PREC_MIXED) { set_error("bad precision"); return ILG_ERR_ARG; }
  if (o->coupling != ILG_COUPLE_REFERENCE && o->coupling != ILG_COUPLE_DIRECT) { set_error("bad coupling"); return ILG_ERR_ARG; }
  if (o->use_radiosity && !c.have_F) { set_error("use_radiosity set but no form factors"); return ILG_ERR_ARG; }
  if (o->max_sweeps < 1) { set_error("max_sweeps must be >= 1"); return ILG_ERR_ARG; }
  if (o->refine_every < 0) { set_error("refine_every must be >= 0"); return ILG_ERR_ARG; }
  if (o->refine_every > 0 && o->precision != ILG_PREC_MIXED) {
    set_error("refine_every applies to the mixed precision only");
    return ILG_ERR_ARG;
  }
  if (o->layer_rounding != 0 && o->layer_rounding != 1) { set_error("layer_rounding must be 0 or 1"); return ILG_ERR_ARG; }
  if (o->layer_rounding && o->precision != ILG_PREC_MIXED) {
    set_error("layer_rounding applies to the mixed precision's FP32 layers only");
    return ILG_ERR_ARG;
  }
  if (o->refine_every > 0 && host_driven) {
    set_error("refine_every needs the sun positions on the device (ilg_run_steps): its solve reads the next frame's flux");
    return ILG_ERR_ARG;
  }
  if (c.rad_mode == ILG_RAD_GS && o->use_radiosity && c.have_F) {
    if (o->precision != ILG_PREC_FP64) {
      set_error("the fixed-sweep Gauss-Seidel mode runs in FP64 precision only");
      return ILG_ERR_ARG;
    }
    ILG_TRY(gs_prepare(c));
  }
  ILG_TRY(conduction_prepare(c, o->dt, o->precision));
  ILG_TRY(conduction_state_convert(c, o->precision));
  ILG_TRY(ensure_step_buffers(c, o->precision));
  return ILG_OK;
}

static StepPlan solo_plan(Context& c, const ilg_run_opts& o) {
  StepPlan p;
  p.precision = o.precision;
  p.rad_on = o.use_radiosity && c.have_F && c.ntiles > 0;
  p.rad_grid = p.rad_on ? radiosity_grid(c.ntiles, o.precision) : 1;
  p.rad_inner = radiosity_inner(o.max_sweeps);
  p.rad_lagged = o.precision == ILG_PREC_MIXED && o.refine_every > 0;
  p.layer_sr = o.precision == ILG_PREC_MIXED && o.layer_rounding == 1;
  p.nz_max = c.nz;
  p.rec_on = c.rec_cap > 0;
  if (p.rad_on && c.rad_mode == ILG_RAD_GS) {
    p.gs_ctx = &c;
    p.gs_steps = c.gs_steps;
  }
  return p;
}

// Captures one pipelined step; slot >= 0 adds the upload of the next
// frame's sun from pinned slot `slot` into host slot `slot` before, and the
// surface-temperature download into pinned slot `slot` after the step
// (host-driven steps: the graph of slot q runs the steps whose next frame
// has parity q).
static int capture_step(Context& c, const ilg_run_opts& o, int slot, cudaGraphExec_t* out) {
  StepView v = solo_view(c, o.precision);
  StepPlan p = solo_plan(c, o);
  cudaGraph_t g;
  ILG_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
  int rc = ILG_OK;
  if (slot >= 0)
    if (cudaMemcpyAsync(c.sun_aux.p + c.nsun + slot, c.pinned_aux + slot * sizeof(SunAux), sizeof(SunAux),
                        cudaMemcpyHostToDevice, c.stream) != cudaSuccess)
      rc = ILG_ERR_CUDA;
  if (rc == ILG_OK) rc = enqueue_step_pipe(v, p, c.stream, c.pipe);
  if (rc == ILG_OK && slot >= 0)
    if (cudaMemcpyAsync(c.pinned_tsurf + (size_t)slot * c.nt, c.Tsurf.p, (size_t)c.nt * 8, cudaMemcpyDeviceToHost,
                        c.stream) != cudaSuccess)
      rc = ILG_ERR_CUDA;
  cudaError_t e = cudaStreamEndCapture(c.stream, &g);
  if (rc != ILG_OK || e != cudaSuccess) {
    cudaGetLastError();
    if (e == cudaSuccess) cudaGraphDestroy(g);
    set_error("step capture failed: %s", cudaGetErrorString(e));
    return rc != ILG_OK ? rc : ILG_ERR_CUDA;
  }
  cudaError_t ei = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) {
    *out = nullptr;
    set_error("graph instantiation failed: %s", cudaGetErrorString(ei));
    return ILG_ERR_CUDA;
  }
  return ILG_OK;
}

// Graph of one step (with_copies: the two host-driven slot graphs, out[0]
// and out[1]; otherwise out[0] only).
static int get_graph(Context& c, const ilg_run_opts& o, bool with_copies, cudaGraphExec_t* out) {
  int key[6] = {(o.precision * 4 + o.coupling * 2 + (o.use_radiosity ? 1 : 0)) * 4 + radiosity_inner(o.max_sweeps),
                (with_copies ? 1 : 0) + 2 * c.rec_cap,
                c.nz, c.ntiles, c.rad_mode == ILG_RAD_GS ? 1 + c.gs_steps : 0, (o.refine_every > 0 ? 1 : 0) + 2 * (o.layer_rounding ? 1 : 0)};
  if (c.graph && std::equal(key, key + 6, c.graph_key)) {
    out[0] = c.graph;
    if (with_copies) out[1] = c.graph_b;
    return ILG_OK;
  }
  invalidate_graph(c);
  ILG_TRY(capture_step(c, o, with_copies ? 0 : -1, &c.graph));
  if (with_copies) {
    int rc = capture_step(c, o, 1, &c.graph_b);
    if (rc != ILG_OK) { invalidate_graph(c); return rc; }
    out[1] = c.graph_b;
  }
  std::copy(key, key + 6, c.graph_key);
  out[0] = c.graph;
  return ILG_OK;
}

static int collect_stats(Context& c, bool phases) {
  int h0 = 0;
  MeshDesc md;
  ILG_CUDA(cudaMemcpyAsync(&h0, c.counters.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  ILG_CUDA(cudaMemcpyAsync(&md, c.md.p, sizeof(md), cudaMemcpyDeviceToHost, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  c.stats_ambiguous += h0;
  c.stats_sweeps += md.sweeps;
  if (phases) {
    float a, b, d;
    ILG_CUDA(cudaEventElapsedTime(&a, c.ev[0], c.ev[1]));
    ILG_CUDA(cudaEventElapsedTime(&b, c.ev[1], c.ev[2]));
    ILG_CUDA(cudaEventElapsedTime(&d, c.ev[2], c.ev[3]));
    c.ms_direct += a;
    c.ms_rad += b;
    c.ms_cond += d;
  }
  return ILG_OK;
}

// Sun positions of the context: a SunAux table of nsun entries plus one
// host slot (index nsun) for host-driven steps and drop-in calls.
static int upload_suns(Context& c, const double* suns, int nsun) {
  std::vector<SunAux> aux((size_t)nsun + 2);   // the table, then the two host slots
  for (int i = 0; i < nsun; ++i) aux[i] = make_sun_aux(suns + 3 * (size_t)i, c.solar_const, c.scene_mag, c.disk_rmax);
  aux[nsun] = aux[nsun + 1] = aux[nsun > 0 ? nsun - 1 : 0];
  ILG_TRY(c.sun_aux.alloc(aux.size()));
  ILG_CUDA(cudaMemcpyAsync(c.sun_aux.p, aux.data(), aux.size() * sizeof(SunAux), cudaMemcpyHostToDevice, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  c.nsun = nsun;
  return ILG_OK;
}

// Put one sun position into the host slot of frame c.frame_no (allocating
// the two host slots when no sun table exists yet).
static int set_host_sun(Context& c, const double* sun) {
  ILG_TRY(ensure_pinned(c));
  if (!c.sun_aux.p) {
    ILG_TRY(c.sun_aux.alloc(2));
    c.nsun = 0;
  }
  *(SunAux*)c.pinned_aux = make_sun_aux(sun, c.solar_const, c.scene_mag, c.disk_rmax);
  ILG_CUDA(cudaMemcpyAsync(c.sun_aux.p + c.nsun + (c.frame_no & 1), c.pinned_aux, sizeof(SunAux),
                           cudaMemcpyHostToDevice, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));   // the pinned slot is reused at once
  return ILG_OK;
}

}  // namespace ilg

using namespace ilg;

// Autotuner helpers (ilg_autotune).
namespace {
// Mean device time (us) of `reps` launches after two warm-up launches.
template <class F>
int time_launches(Context& c, F&& launch, int reps, double* us) {
  cudaEvent_t a = nullptr, b = nullptr;
  ILG_CUDA(cudaEventCreate(&a));
  ILG_CUDA(cudaEventCreate(&b));
  int rc = ILG_OK;
  for (int i = 0; i < 2 && rc == ILG_OK; ++i) rc = launch();
  if (rc == ILG_OK) rc = cudaEventRecord(a, c.stream) == cudaSuccess ? ILG_OK : ILG_ERR_CUDA;
  for (int i = 0; i < reps && rc == ILG_OK; ++i) rc = launch();
  float ms = 0.f;
  if (rc == ILG_OK && (cudaEventRecord(b, c.stream) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
                       cudaEventElapsedTime(&ms, a, b) != cudaSuccess)) {
    set_error("autotune timing failed");
    rc = ILG_ERR_CUDA;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *us = 1000.0 * ms / reps;
  return rc;
}

int scratch_copy(dbuf<double>& d, const double* src, size_t n, cudaStream_t s) {
  ILG_TRY(d.alloc(n));
  ILG_CUDA(cudaMemcpyAsync(d.p, src, n * 8, cudaMemcpyDeviceToDevice, s));
  return ILG_OK;
}
}  // namespace

extern "C" {

const char* ilg_last_error(void) { return g_err.c_str(); }
int ilg_version(void) { return 10000; }

int ilg_ctx_create(const float* verts, int nv, const int32_t* tris, int nt, const float* normals, ilg_ctx** out) {
  if (!out || !verts || !tris || nv < 3 || nt < 1) { set_error("invalid mesh arguments"); return ILG_ERR_ARG; }
  *out = nullptr;
  ILG_TRY(alloc_pool_setup());
  ilg_ctx* h = new ilg_ctx();
  Context& c = h->c;
  c.nt = nt;
  int rc = ILG_OK;
  if (cudaStreamCreateWithFlags(&c.owned_stream.s, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("cudaStreamCreate failed");
    delete h;
    return ILG_ERR_CUDA;
  }
  c.stream = c.owned_stream.s;
  AllocOn on(c.stream);
  for (auto& e : c.ev)
    if (cudaEventCreate(&e) != cudaSuccess) { set_error("cudaEventCreate failed"); delete h; return ILG_ERR_CUDA; }
  if ((rc = c.derr.alloc(DERR_COUNT)) || (rc = c.counters.alloc(8)) || (rc = c.work.alloc(nt)) ||
      (rc = c.barrier.alloc(radiosity_barrier_words(1))) || (rc = c.md.alloc(1)) || (rc = c.mesh_flag.alloc(1))) {
    delete h;
    return rc;
  }
  cudaMemsetAsync(c.derr.p, 0, DERR_COUNT * sizeof(int), c.stream);
  cudaMemsetAsync(c.counters.p, 0, 8 * sizeof(int), c.stream);
  rc = bvh_build(c, verts, nv, tris, normals);
  if (rc == ILG_OK) rc = read_device_errors(c);
  if (rc != ILG_OK) { delete h; return rc; }
  *out = h;
  return ILG_OK;
}

int ilg_ctx_destroy(ilg_ctx* ctx) {
  delete ctx;
  return ILG_OK;
}

int ilg_ctx_num_faces(const ilg_ctx* ctx) { return ctx ? ctx->c.nt : 0; }

int ilg_ctx_info(const ilg_ctx* ctx, int64_t* bvh_nodes, int* bvh_depth) {
  if (!ctx) { set_error("ctx is NULL"); return ILG_ERR_ARG; }
  if (bvh_nodes) *bvh_nodes = ctx->c.bvh_nodes;
  if (bvh_depth) *bvh_depth = ctx->c.bvh_depth;
  return ILG_OK;
}

extern "C++" {
namespace {
template <class T>
int64_t nbytes(const dbuf<T>& b) { return (int64_t)(b.n * sizeof(T)); }
template <class T, class... R>
int64_t nbytes(const dbuf<T>& b, const R&... rest) { return nbytes(b) + nbytes(rest...); }
}  // namespace
}

int ilg_ctx_device_bytes(const ilg_ctx* ctx, int64_t* bytes) {
  if (!ctx || !bytes) { set_error("ctx or bytes is NULL"); return ILG_ERR_ARG; }
  const Context& c = ctx->c;
  *bytes = nbytes(c.tri_o, c.cen, c.nrm, c.frame32, c.nodes, c.tri_s, c.flush) +
           nbytes(c.area, c.frame, c.H, c.val, c.tile_d2, c.rho64, c.Tsurf, c.Fsurf, c.Qprev, c.rad, c.rad_avg,
                  c.therm_avg, c.therm_max, c.E, c.xtmp, c.Q, c.sprev, c.rec, c.rec_part, c.disk) +
           nbytes(c.H32, c.row_scale, c.t_vhi, c.t_vlo, c.t_scale, c.coef32, c.rho32, c.T32, c.disk32, c.x32) +
           nbytes(c.hmm32, c.coefdf, c.Tdf) + nbytes(c.rowptr) + nbytes(c.col) + nbytes(c.tiles) +
           nbytes(c.t_cf) + nbytes(c.t_vbf) + nbytes(c.row_act) +
           nbytes(c.morton_order, c.t_row, c.t_halo, c.t_start, c.rperm) +
           nbytes(c.work, c.counters, c.derr, c.mesh_flag) + nbytes(c.barrier) + nbytes(c.sun_aux) + nbytes(c.md) +
           nbytes(c.scan.a, c.scan.b, c.scan.c, c.sort.keys_alt, c.sort.hist, c.sort.scan.a, c.sort.scan.b,
                  c.sort.scan.c) +
           nbytes(c.sort.vals_alt);
  return ILG_OK;
}

int ilg_F_info(const ilg_ctx* ctx, int64_t* nnz, int64_t* stored_entries, int* row_tiles, int* active_rows) {
  if (!ctx || !ctx->c.have_F) { set_error("no form factors"); return ILG_ERR_ARG; }
  const Context& c = ctx->c;
  if (nnz) *nnz = c.nnz;
  if (stored_entries) *stored_entries = c.tile_elems;
  if (row_tiles) *row_tiles = c.ntiles;
  if (active_rows) *active_rows = c.n_active;
  return ILG_OK;
}

int ilg_device_pool_high(int64_t* used_high, int64_t* reserved_high, int reset) {
  ILG_TRY(alloc_pool_setup());
  int dev = 0;
  ILG_CUDA(cudaGetDevice(&dev));
  cudaMemPool_t pool;
  ILG_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
  uint64_t u = 0, r = 0;
  ILG_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &u));
  ILG_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemHigh, &r));
  if (used_high) *used_high = (int64_t)u;
  if (reserved_high) *reserved_high = (int64_t)r;
  if (reset) {
    uint64_t z = 0;
    ILG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &z));
    ILG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReservedMemHigh, &z));
  }
  return ILG_OK;
}

int ilg_F_tiles(const ilg_ctx* ctx, int cap, int* entries_per_thread, int* rows, int* halo, int* ntiles) {
  if (!ctx || !ctx->c.have_F || !ntiles || cap < 0) { set_error("invalid arguments"); return ILG_ERR_ARG; }
  const Context& c = ctx->c;
  *ntiles = c.ntiles;
  for (int t = 0; t < c.ntiles && t < cap; ++t) {
    const RowTile& T = c.tiles_h[t];
    if (entries_per_thread) entries_per_thread[t] = T.lam;
    if (rows) rows[t] = T.nrows;
    if (halo) halo[t] = T.nhalo;
  }
  return ILG_OK;
}

int ilg_trace(ilg_ctx* ctx, int nrays, const float* orig, const float* dir, int any_hit, int32_t* hit, double* t) {
  if (!ctx || nrays < 0 || (nrays > 0 && (!orig || !dir || !hit))) { set_error("invalid trace arguments"); return ILG_ERR_ARG; }
  AllocOn on_(ctx->c.stream);
  return bvh_trace(ctx->c, nrays, orig, dir, any_hit, hit, t);
}

int ilg_render(ilg_ctx* ctx, int mode, double az_deg, double el_deg, int width, int height, int32_t* facet_out) {
  if (!ctx || !facet_out || (mode != 0 && mode != 1) || width < 2 || height < 2) {
    set_error("invalid render arguments");
    return ILG_ERR_ARG;
  }
  AllocOn on_(ctx->c.stream);
  return bvh_render(ctx->c, mode, az_deg, el_deg, width, height, facet_out);
}

int ilg_compute_F(ilg_ctx* ctx, const double* albedo, double albedo_scalar, double offset, int64_t* nnz, int64_t* rays) {
  if (!ctx) { set_error("ctx is NULL"); return ILG_ERR_ARG; }
  AllocOn on_(ctx->c.stream);
  invalidate_graph(ctx->c);
  ILG_TRY(form_factors_build(ctx->c, albedo, albedo_scalar, offset, 0.0, rays));
  if (nnz) *nnz = ctx->c.nnz;
  return ILG_OK;
}

int ilg_compute_F_cutoff(ilg_ctx* ctx, const double* albedo, double albedo_scalar, double offset, double cutoff,
                         int64_t* nnz, int64_t* rays) {
  if (!ctx) { set_error("ctx is NULL"); return ILG_ERR_ARG; }
  if (!(cutoff > 0.0)) { set_error("cutoff must be > 0"); return ILG_ERR_ARG; }
  AllocOn on_(ctx->c.stream);
  invalidate_graph(ctx->c);
  ILG_TRY(form_factors_build(ctx->c, albedo, albedo_scalar, offset, cutoff, rays));
  if (nnz) *nnz = ctx->c.nnz;
  return ILG_OK;
}

int ilg_visibility_sample(ilg_ctx* ctx, double cutoff, double offset, const int32_t* sources, int nsrc,
                          const double* radii, int nradii, int64_t* per_source, int64_t* within_radius,
                          int64_t* rays) {
  if (!ctx || !per_source) { set_error("ctx or per_source is NULL"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  return visibility_sample(c, cutoff, offset, sources, nsrc, radii, nradii, per_source, within_radius, rays);
}

int ilg_get_F(ilg_ctx* ctx, int64_t* rowptr, int32_t* col, double* val) {
  if (!ctx || !ctx->c.have_F) { set_error("no form factors"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  if (rowptr) ILG_CUDA(cudaMemcpyAsync(rowptr, c.rowptr.p, ((size_t)c.nt + 1) * 8, cudaMemcpyDeviceToHost, c.stream));
  if (c.nnz > 0) {
    if (col) ILG_CUDA(cudaMemcpyAsync(col, c.col.p, (size_t)c.nnz * 4, cudaMemcpyDeviceToHost, c.stream));
    if (val) ILG_CUDA(cudaMemcpyAsync(val, c.val.p, (size_t)c.nnz * 8, cudaMemcpyDeviceToHost, c.stream));
  }
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  return ILG_OK;
}

int ilg_set_F(ilg_ctx* ctx, int64_t nnz, const int64_t* rowptr, const int32_t* col, const double* val) {
  if (!ctx || nnz < 0 || !rowptr || (nnz > 0 && (!col || !val))) { set_error("invalid F arguments"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  if (rowptr[0] != 0 || rowptr[c.nt] != nnz) { set_error("rowptr does not span nnz"); return ILG_ERR_ARG; }
  for (int i = 0; i < c.nt; ++i)
    if (rowptr[i + 1] < rowptr[i]) { set_error("rowptr decreases at row %d", i); return ILG_ERR_ARG; }
  for (int64_t k = 0; k < nnz; ++k)
    if (col[k] < 0 || col[k] >= c.nt) { set_error("column index out of range at %lld", (long long)k); return ILG_ERR_ARG; }
  invalidate_graph(c);
  ILG_TRY(c.rowptr.alloc((size_t)c.nt + 1));
  ILG_TRY(c.col.alloc(nnz > 0 ? nnz : 1));
  ILG_TRY(c.val.alloc(nnz > 0 ? nnz : 1));
  ILG_CUDA(cudaMemcpyAsync(c.rowptr.p, rowptr, ((size_t)c.nt + 1) * 8, cudaMemcpyHostToDevice, c.stream));
  if (nnz > 0) {
    ILG_CUDA(cudaMemcpyAsync(c.col.p, col, (size_t)nnz * 4, cudaMemcpyHostToDevice, c.stream));
    ILG_CUDA(cudaMemcpyAsync(c.val.p, val, (size_t)nnz * 8, cudaMemcpyHostToDevice, c.stream));
  }
  c.nnz = nnz;
  c.have_F = true;
  c.gs_ready = false;
  ILG_TRY(radiosity_prepare(c));
  c.sort.release();
  c.scan.release();
  return ILG_OK;
}

int ilg_make_horizons(ilg_ctx* ctx, int nphi, double theta_eps, double offset) {
  if (!ctx) { set_error("ctx is NULL"); return ILG_ERR_ARG; }
  AllocOn on_(ctx->c.stream);
  invalidate_graph(ctx->c);
  return horizons_build(ctx->c, nphi, theta_eps, offset);
}

int ilg_make_horizons_mesh(ilg_ctx* ctx, const float* verts, int nv, const int32_t* tris, int nt, int nphi,
                           double theta_eps, double offset) {
  if (!ctx) { set_error("ctx is NULL"); return ILG_ERR_ARG; }
  ilg_ctx* hm = nullptr;
  ILG_TRY(ilg_ctx_create(verts, nv, tris, nt, nullptr, &hm));   // the horizon mesh's LBVH (synchronised)
  AllocOn on_(ctx->c.stream);
  invalidate_graph(ctx->c);
  const int rc = horizons_build(ctx->c, nphi, theta_eps, offset, &hm->c);
  ilg_ctx_destroy(hm);
  return rc;
}

int ilg_get_horizons(ilg_ctx* ctx, double* out) {
  if (!ctx || !ctx->c.H.p || !out) { set_error("no horizons"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  ILG_CUDA(cudaMemcpyAsync(out, c.H.p, (size_t)c.nt * c.nphi * 8, cudaMemcpyDeviceToHost, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  return ILG_OK;
}

int ilg_set_horizons(ilg_ctx* ctx, int nphi, const double* h) {
  if (!ctx || nphi < 2 || !h) { set_error("invalid horizon arguments"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  invalidate_graph(c);
  size_t n = (size_t)c.nt * nphi;
  for (size_t k = 0; k < n; ++k)
    if (!(h[k] == h[k])) { set_error("horizon column %d holds NaN", (int)(k / nphi)); return ILG_ERR_ARG; }
  ILG_TRY(c.H.alloc(n));
  ILG_CUDA(cudaMemcpyAsync(c.H.p, h, n * 8, cudaMemcpyHostToDevice, c.stream));
  c.nphi = nphi;
  c.dphi = TWO_PI / (double)(nphi - 1);
  return horizons_f32(c);
}

int ilg_set_insolation(ilg_ctx* ctx, int norm_mode, int interp, double solar_const) {
  if (!ctx || (norm_mode != 0 && norm_mode != 1) || (interp != 0 && interp != 1) || !(solar_const >= 0.0)) {
    set_error("invalid insolation options");
    return ILG_ERR_ARG;
  }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  invalidate_graph(c);
  c.norm_mode = norm_mode;
  c.interp = interp;
  c.solar_const = solar_const;
  if (c.nsun > 0) ILG_TRY(upload_suns(c, c.suns_h.data(), c.nsun));   // flux is baked into the table
  return ILG_OK;
}

void ilg_fib_spiral(double* xy, int n) {
  if (xy && n > 0) fib_spiral(xy, n);
}

int ilg_direct_radiosity(ilg_ctx* ctx, const double* sun, const double* disk_xy, int ndisk, double* out) {
  if (!ctx || !sun || !out) { set_error("invalid direct arguments"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  if (!c.H.p || c.nphi < 2) { set_error("horizons are not set"); return ILG_ERR_ARG; }
  ILG_TRY(set_disk(c, disk_xy, ndisk));
  ILG_TRY(ensure_step_buffers(c, ILG_PREC_FP64));
  ILG_TRY(set_host_sun(c, sun));
  MeshDesc M = solo_desc(c, nullptr, 0);
  M.host_sun = 1;
  ILG_TRY(upload_desc(c, M));
  ILG_TRY(direct_launch(solo_view(c, ILG_PREC_FP64), 1, 0, 0, c.stream));
  ILG_CUDA(cudaMemcpyAsync(out, c.E.p, (size_t)c.nt * 8, cudaMemcpyDeviceToHost, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  return read_device_errors(c);
}

int ilg_radiosity_solve(ilg_ctx* ctx, const double* E, double tol, int max_sweeps, double* x, double* res, int* sweeps) {
  if (!ctx || !E || !x || max_sweeps < 1 || !(tol >= 0.0)) { set_error("invalid radiosity arguments"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  if (!c.have_F) { set_error("no form factors"); return ILG_ERR_ARG; }
  c.ref_age = -1;   // the solve below reuses the buffers of a one-pass reference
  if (c.ntiles == 0) {
    std::memcpy(x, E, (size_t)c.nt * 8);
    if (res) *res = 0.0;
    if (sweeps) *sweeps = 0;
    return ILG_OK;
  }
  ILG_TRY(ensure_step_buffers(c, ILG_PREC_FP64));
  ilg_run_opts o{};
  o.tol = tol;
  o.max_sweeps = max_sweeps;
  o.use_radiosity = 1;
  o.coupling = ILG_COUPLE_DIRECT;   // E as given
  MeshDesc M = solo_desc(c, &o, 0);
  ILG_TRY(upload_desc(c, M));
  ILG_CUDA(cudaMemcpyAsync(c.E.p + e_slot(M.frame) * c.nt, E, (size_t)c.nt * 8, cudaMemcpyHostToDevice,
                           c.stream));
  StepView v = solo_view(c, ILG_PREC_FP64);
  ILG_TRY(radiosity_launch(v, c.Q.p, 0, ILG_PREC_FP64, radiosity_grid(c.ntiles, ILG_PREC_FP64), 1, false, c.stream));
  MeshDesc out;
  ILG_CUDA(cudaMemcpyAsync(x, c.Q.p, (size_t)c.nt * 8, cudaMemcpyDeviceToHost, c.stream));
  ILG_CUDA(cudaMemcpyAsync(&out, c.md.p, sizeof(out), cudaMemcpyDeviceToHost, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  ILG_TRY(read_device_errors(c));
  if (res) *res = std::sqrt(out.res2);
  if (sweeps) *sweeps = out.sweeps;
  if (out.res2 > tol * tol) {
    set_error("radiosity residual %g above tol after %d sweeps", std::sqrt(out.res2), out.sweeps);
    return ILG_ERR_NOTCONV;
  }
  return ILG_OK;
}

int ilg_set_radiosity_mode(ilg_ctx* ctx, int mode, int gs_steps) {
  if (!ctx || (mode != ILG_RAD_TOL && mode != ILG_RAD_GS) || gs_steps < 0) {
    set_error("invalid radiosity mode (%d, gs_steps %d)", mode, gs_steps);
    return ILG_ERR_ARG;
  }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  c.rad_mode = mode;
  c.gs_steps = gs_steps;
  invalidate_graph(c);
  return ILG_OK;
}

int ilg_set_radiosity_blocks(ilg_ctx* ctx, int blocks) {
  if (!ctx || blocks < 0) { set_error("invalid radiosity block count %d", blocks); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  if (c.tile_blocks == blocks) return ILG_OK;
  c.tile_blocks = blocks;
  if (!c.have_F) return ILG_OK;
  invalidate_graph(c);
  ILG_TRY(radiosity_prepare(c));
  c.sort.release();
  c.scan.release();
  return ILG_OK;
}

int ilg_radiosity_solve_gs(ilg_ctx* ctx, const double* E, int gs_steps, double* x, double* res) {
  if (!ctx || !E || !x || gs_steps < 0) { set_error("invalid radiosity arguments"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  if (!c.have_F) { set_error("no form factors"); return ILG_ERR_ARG; }
  ILG_TRY(gs_prepare(c));
  ILG_TRY(ensure_step_buffers(c, ILG_PREC_FP64));
  double* Ed = c.gs_x.p + 2 * (size_t)c.nt;
  ILG_CUDA(cudaMemcpyAsync(Ed, E, (size_t)c.nt * 8, cudaMemcpyHostToDevice, c.stream));
  ILG_TRY(gs_solve_launch(c, Ed, c.Q.p, gs_steps, c.stream));
  std::vector<double> r2;
  if (res) {
    ILG_TRY(gs_residual_launch(c, Ed, c.Q.p, c.gs_x.p, c.stream));
    r2.resize(c.nt);
    ILG_CUDA(cudaMemcpyAsync(r2.data(), c.gs_x.p, (size_t)c.nt * 8, cudaMemcpyDeviceToHost, c.stream));
  }
  ILG_CUDA(cudaMemcpyAsync(x, c.Q.p, (size_t)c.nt * 8, cudaMemcpyDeviceToHost, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  if (res) {
    double acc = 0.0;   // row order, as the CPU oracle sums
    for (double q : r2) acc += q;
    *res = std::sqrt(acc);
  }
  return ILG_OK;
}

int ilg_debug_ff_chunk(long long pairs) { return ff_set_chunk((int64_t)pairs); }

int ilg_debug_barrier_timeout(ilg_ctx* ctx, int blocks, long long polls, int unreachable) {
  if (!ctx) { set_error("ctx is NULL"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  ILG_TRY(c.barrier.reserve(radiosity_barrier_words(1)));
  ILG_TRY(c.derr.reserve(DERR_COUNT));
  ILG_CUDA(cudaMemsetAsync(c.derr.p, 0, DERR_COUNT * sizeof(int), c.stream));
  ILG_TRY(radiosity_barrier_probe(c.barrier.p, c.derr.p, blocks, polls, unreachable, c.stream));
  return read_device_errors(c);   // ILG_ERR_DEVICE once the wait ran out (the flags are cleared)
}

int ilg_radiosity_levels(const ilg_ctx* ctx, int* levels) {
  if (!ctx || !levels) { set_error("ctx or levels is NULL"); return ILG_ERR_ARG; }
  *levels = gs_levels(ctx->c);
  return ILG_OK;
}

int ilg_thermal_init(ilg_ctx* ctx, int nz, const double* z, const double* ti, const double* rhoc, double T0,
                     const double* T0_full, double emissivity, double Fgeotherm, int bc_mode, int precision) {
  if (!ctx || nz < 2 || !z || !ti || !rhoc) { set_error("invalid thermal arguments"); return ILG_ERR_ARG; }
  if (bc_mode != ILG_BC_LINEARISED && bc_mode != ILG_BC_NEWTON) { set_error("bad bc_mode"); return ILG_ERR_ARG; }
  if (precision != ILG_PREC_FP64 && precision != ILG_PREC_MIXED) { set_error("bad precision"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  invalidate_graph(c);
  int nt = c.nt;
  c.nz = nz;
  c.z_h.assign(z, z + nz);
  c.ti_h.assign(ti, ti + nz);
  c.rhoc_h.assign(rhoc, rhoc + nz);
  c.emiss = emissivity;
  c.Fgeo = Fgeotherm;
  c.bc_mode = bc_mode;
  c.coef_dt = -1.0;
  c.coef_prec = -1;
  size_t n = (size_t)nz * nt;
  std::vector<float2> Tl(n);
  std::vector<double> ts(nt);
  for (int f = 0; f < nt; ++f) {
    ts[f] = T0_full ? T0_full[(size_t)f * (nz + 1)] : T0;
    for (int i = 0; i < nz; ++i)
      Tl[(size_t)i * nt + f] = split_df_host(T0_full ? T0_full[(size_t)f * (nz + 1) + 1 + i] : T0);
  }
  ILG_TRY(c.Tdf.alloc(n));
  ILG_TRY(c.Tsurf.alloc(nt));
  ILG_TRY(c.Fsurf.alloc(nt));
  ILG_TRY(c.Qprev.alloc(nt));
  ILG_TRY(c.rad.alloc(nt));
  ILG_TRY(c.rad_avg.alloc(nt));
  ILG_TRY(c.therm_avg.alloc(nt));
  ILG_TRY(c.therm_max.alloc(nt));
  ILG_TRY(c.E.reserve(E_SLOTS * (size_t)nt));
  ILG_TRY(c.Q.reserve(nt));
  ILG_CUDA(cudaMemcpyAsync(c.Tdf.p, Tl.data(), n * 8, cudaMemcpyHostToDevice, c.stream));
  ILG_CUDA(cudaMemcpyAsync(c.Tsurf.p, ts.data(), (size_t)nt * 8, cudaMemcpyHostToDevice, c.stream));
  for (double* p : {c.Fsurf.p, c.Qprev.p, c.rad.p, c.rad_avg.p, c.therm_avg.p, c.therm_max.p})
    ILG_CUDA(cudaMemsetAsync(p, 0, (size_t)nt * 8, c.stream));
  ILG_CUDA(cudaMemsetAsync(c.counters.p, 0, 8 * sizeof(int), c.stream));
  if (c.sprev.p) ILG_CUDA(cudaMemsetAsync(c.sprev.p, 0, c.sprev.n * sizeof(float2), c.stream));
  invalidate_graph(c);
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  c.state_prec = ILG_PREC_FP64;
  c.frame_no = 0;
  c.have_thermal = true;
  return conduction_state_convert(c, precision);
}

int ilg_thermal_step(ilg_ctx* ctx, double dt, const double* Q) {
  if (!ctx || !Q || !(dt > 0.0)) { set_error("invalid thermal step arguments"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  if (!c.have_thermal) { set_error("ilg_thermal_init has not been called"); return ILG_ERR_ARG; }
  ILG_TRY(conduction_prepare(c, dt, c.state_prec));
  ILG_TRY(ensure_step_buffers(c, c.state_prec));
  MeshDesc M = solo_desc(c, nullptr, 0);
  ILG_TRY(upload_desc(c, M));
  ILG_CUDA(cudaMemcpyAsync(c.Q.p, Q, (size_t)c.nt * 8, cudaMemcpyHostToDevice, c.stream));
  ILG_TRY(conduction_launch(solo_view(c, c.state_prec), c.Q.p, c.state_prec, 0, c.nz, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  return read_device_errors(c);
}

int ilg_thermal_get(ilg_ctx* ctx, double* T, double* Fsurf, double* Qprev) {
  if (!ctx) { set_error("ctx is NULL"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  if (!c.have_thermal) { set_error("ilg_thermal_init has not been called"); return ILG_ERR_ARG; }
  int nt = c.nt, nz = c.nz;
  if (T) {
    size_t n = (size_t)nz * nt;
    std::vector<double> Tl(n), ts(nt);
    if (c.state_prec == ILG_PREC_MIXED) {
      std::vector<float> t32(n);
      ILG_CUDA(cudaMemcpyAsync(t32.data(), c.T32.p, n * 4, cudaMemcpyDeviceToHost, c.stream));
      ILG_CUDA(cudaStreamSynchronize(c.stream));
      for (size_t i = 0; i < n; ++i) Tl[i] = t32[i];
    } else {
      std::vector<float2> tdf(n);
      ILG_CUDA(cudaMemcpyAsync(tdf.data(), c.Tdf.p, n * 8, cudaMemcpyDeviceToHost, c.stream));
      ILG_CUDA(cudaStreamSynchronize(c.stream));
      for (size_t i = 0; i < n; ++i) Tl[i] = (double)tdf[i].x + (double)tdf[i].y;
    }
    ILG_CUDA(cudaMemcpyAsync(ts.data(), c.Tsurf.p, (size_t)nt * 8, cudaMemcpyDeviceToHost, c.stream));
    ILG_CUDA(cudaStreamSynchronize(c.stream));
    for (int f = 0; f < nt; ++f) {
      T[(size_t)f * (nz + 1)] = ts[f];
      for (int i = 0; i < nz; ++i) T[(size_t)f * (nz + 1) + 1 + i] = Tl[(size_t)i * nt + f];
    }
  }
  if (Fsurf) ILG_CUDA(cudaMemcpyAsync(Fsurf, c.Fsurf.p, (size_t)nt * 8, cudaMemcpyDeviceToHost, c.stream));
  if (Qprev) ILG_CUDA(cudaMemcpyAsync(Qprev, c.Qprev.p, (size_t)nt * 8, cudaMemcpyDeviceToHost, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  return ILG_OK;
}

int ilg_set_suns(ilg_ctx* ctx, int nsun, const double* suns, const double* disk_xy, int ndisk) {
  if (!ctx || nsun < 1 || !suns) { set_error("invalid sun arguments"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  invalidate_graph(c);
  ILG_TRY(set_disk(c, disk_xy, ndisk));
  c.suns_h.assign(suns, suns + 3 * (size_t)nsun);
  return upload_suns(c, suns, nsun);
}

int ilg_run_steps(ilg_ctx* ctx, const ilg_run_opts* opts, int first_sun, int nsteps, double* tsurf_out) {
  if (!ctx) { set_error("ctx is NULL"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  ILG_TRY(check_run(c, opts, false));
  if (nsteps < 0 || first_sun < 0 || first_sun + nsteps > c.nsun) { set_error("sun range out of bounds"); return ILG_ERR_ARG; }
  if (tsurf_out) ILG_TRY(ensure_pinned(c));   // page-locked staging, only where host copies are made
  const ilg_run_opts& o = *opts;
  ILG_TRY(upload_desc(c, solo_desc(c, &o, first_sun)));
  bool timing = c.timing;
  cudaGraphExec_t g = nullptr;
  if (o.use_graph && !timing && !c.graph_broken)
    if (get_graph(c, o, false, &g) != ILG_OK) { c.graph_broken = true; g = nullptr; cudaGetLastError(); }
  StepView v = solo_view(c, o.precision);
  StepPlan p = solo_plan(c, o);
  // pipelined steps (graph or eager) after a prologue; the phase-timed steps
  // run in the serial order (same results)
  if (!timing && nsteps > 0) ILG_TRY(enqueue_prologue(v, p, c.stream));
  if (timing && nsteps > 0) ILG_TRY(enqueue_serial_prologue(v, p, c.stream));
  for (int s = 0; s < nsteps; ++s) {
    if (g) ILG_CUDA(cudaGraphLaunch(g, c.stream));
    else if (timing) ILG_TRY(enqueue_step(v, p, c.stream, c.ev));
    else ILG_TRY(enqueue_step_pipe(v, p, c.stream, c.pipe));
    if (timing) ILG_TRY(collect_stats(c, true));
    if (tsurf_out) {
      ILG_CUDA(cudaMemcpyAsync(c.pinned_tsurf, c.Tsurf.p, (size_t)c.nt * 8, cudaMemcpyDeviceToHost, c.stream));
      ILG_CUDA(cudaStreamSynchronize(c.stream));
      std::memcpy(tsurf_out + (size_t)s * c.nt, c.pinned_tsurf, (size_t)c.nt * 8);
    }
  }
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  ILG_TRY(keep_reference(c, solo_plan(c, o)));
  c.frame_no += nsteps;
  return read_device_errors(c);
}

int ilg_run_steps_host(ilg_ctx* ctx, const ilg_run_opts* opts, int nsteps, const double* suns, double* tsurf_out) {
  if (!ctx || (nsteps > 0 && !suns)) { set_error("invalid arguments"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  if (!opts) { set_error("opts is NULL"); return ILG_ERR_ARG; }
  if (c.ndisk < 2) { set_error("sun disk samples are not set (ilg_set_suns)"); return ILG_ERR_ARG; }
  if (!c.sun_aux.p) { ILG_TRY(c.sun_aux.alloc(2)); c.nsun = 0; }
  ILG_TRY(check_run(c, opts, true));
  ILG_TRY(ensure_pinned(c));
  const ilg_run_opts& o = *opts;
  MeshDesc M = solo_desc(c, &o, 0);
  M.host_sun = 1;
  ILG_TRY(upload_desc(c, M));
  bool timing = c.timing;
  cudaGraphExec_t g[2] = {nullptr, nullptr};
  if (o.use_graph && !timing && !c.graph_broken)
    if (get_graph(c, o, true, g) != ILG_OK) { c.graph_broken = true; g[0] = g[1] = nullptr; cudaGetLastError(); }
  SunAux* aux = reinterpret_cast<SunAux*>(c.pinned_aux);
  SunAux* dslot = c.sun_aux.p + c.nsun;   // host slots: frame f uses dslot[f & 1]
  const int f0 = c.frame_no;
  auto sun_of = [&](int s) {   // step s's sun (the last one for steps past the call)
    return make_sun_aux(suns + 3 * (size_t)std::min(s, nsteps - 1), c.solar_const, c.scene_mag, c.disk_rmax);
  };
  if (g[0] && nsteps > 0) {
    // Pipelined: step s runs graph q = (f0 + s + 1) & 1, which uploads step
    // s+1's sun into host slot q for the next frame's direct insolation and
    // copies step s's surface temperatures into pinned slot q. Step s+1 is
    // queued before step s's temperatures are read, so the GPU runs the steps
    // back to back; a pinned slot is rewritten only after the step that
    // last used it has completed.
    StepView v = solo_view(c, o.precision);
    StepPlan p = solo_plan(c, o);
    aux[f0 & 1] = sun_of(0);
    ILG_CUDA(cudaMemcpyAsync(dslot + (f0 & 1), aux + (f0 & 1), sizeof(SunAux), cudaMemcpyHostToDevice, c.stream));
    ILG_TRY(enqueue_prologue(v, p, c.stream));
    ILG_CUDA(cudaStreamSynchronize(c.stream));
    int q = (f0 + 1) & 1;
    aux[q] = sun_of(1);
    ILG_CUDA(cudaGraphLaunch(g[q], c.stream));
    ILG_CUDA(cudaEventRecord(c.slot_ev[q], c.stream));
    for (int s = 0; s < nsteps; ++s) {
      q = (f0 + s + 1) & 1;
      const int nq = q ^ 1;
      if (s + 1 < nsteps) {
        aux[nq] = sun_of(s + 2);
        ILG_CUDA(cudaGraphLaunch(g[nq], c.stream));
        ILG_CUDA(cudaEventRecord(c.slot_ev[nq], c.stream));
      }
      ILG_CUDA(cudaEventSynchronize(c.slot_ev[q]));
      if (tsurf_out) std::memcpy(tsurf_out + (size_t)s * c.nt, c.pinned_tsurf + (size_t)q * c.nt, (size_t)c.nt * 8);
    }
  } else {
    StepView v = solo_view(c, o.precision);
    StepPlan p = solo_plan(c, o);
    for (int s = 0; s < nsteps; ++s) {
      const int q = (f0 + s) & 1;
      aux[q] = sun_of(s);
      ILG_CUDA(cudaMemcpyAsync(dslot + q, aux + q, sizeof(SunAux), cudaMemcpyHostToDevice, c.stream));
      ILG_TRY(enqueue_step(v, p, c.stream, timing ? c.ev : nullptr));
      ILG_CUDA(cudaMemcpyAsync(c.pinned_tsurf, c.Tsurf.p, (size_t)c.nt * 8, cudaMemcpyDeviceToHost, c.stream));
      ILG_CUDA(cudaStreamSynchronize(c.stream));
      if (timing) ILG_TRY(collect_stats(c, true));
      if (tsurf_out) std::memcpy(tsurf_out + (size_t)s * c.nt, c.pinned_tsurf, (size_t)c.nt * 8);
    }
  }
  ILG_TRY(keep_reference(c, solo_plan(c, o)));
  c.frame_no += nsteps;
  return read_device_errors(c);
}

// Benchmark loop: before every step a kernel overwrites flush_mb MB (evicting
// the 129 MB L2), then the step runs between two events on the context's
// stream. step_ms[s] receives each step's device time; with use_graph == 0
// the steps run eagerly and phase_ms[0..2] accumulates the direct,
// radiosity and conduction phases.
int ilg_bench_steps(ilg_ctx* ctx, const ilg_run_opts* opts, int first_sun, int nsteps, double flush_mb,
                    double* step_ms, double* phase_ms) {
  if (!ctx || !step_ms) { set_error("invalid arguments"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  ILG_TRY(check_run(c, opts, false));
  if (nsteps < 0 || first_sun < 0 || first_sun + nsteps > c.nsun) { set_error("sun range out of bounds"); return ILG_ERR_ARG; }
  const ilg_run_opts& o = *opts;
  size_t nflush = flush_mb > 0 ? (size_t)(flush_mb * 1048576.0 / 16.0) : 0;
  if (nflush) ILG_TRY(c.flush.reserve(nflush));
  ILG_TRY(upload_desc(c, solo_desc(c, &o, first_sun)));
  cudaGraphExec_t g = nullptr;
  if (o.use_graph && !c.graph_broken)
    if (get_graph(c, o, false, &g) != ILG_OK) { c.graph_broken = true; g = nullptr; cudaGetLastError(); }
  StepView v = solo_view(c, o.precision);
  StepPlan p = solo_plan(c, o);
  cudaEvent_t a = c.ev[0], b = c.ev[3];
  if (phase_ms) phase_ms[0] = phase_ms[1] = phase_ms[2] = 0.0;
  // graph steps are pipelined (prologue untimed); eager steps run in the
  // serial order with their phase boundaries recorded
  if (g && nsteps > 0) ILG_TRY(enqueue_prologue(v, p, c.stream));
  if (!g && nsteps > 0) ILG_TRY(enqueue_serial_prologue(v, p, c.stream));
  for (int s = 0; s < nsteps; ++s) {
    if (nflush) ILG_TRY(flush_launch(c.flush.p, nflush, (unsigned)s, c.stream));
    if (g) {
      ILG_CUDA(cudaEventRecord(a, c.stream));
      ILG_CUDA(cudaGraphLaunch(g, c.stream));
      ILG_CUDA(cudaEventRecord(b, c.stream));
    } else {
      ILG_TRY(enqueue_step(v, p, c.stream, c.ev));
    }
    ILG_CUDA(cudaEventSynchronize(b));
    float ms = 0.f;
    ILG_CUDA(cudaEventElapsedTime(&ms, a, b));
    step_ms[s] = ms;
    if (!g) {
      float p0, p1, p2;
      ILG_CUDA(cudaEventElapsedTime(&p0, c.ev[0], c.ev[1]));
      ILG_CUDA(cudaEventElapsedTime(&p1, c.ev[1], c.ev[2]));
      ILG_CUDA(cudaEventElapsedTime(&p2, c.ev[2], c.ev[3]));
      if (phase_ms) { phase_ms[0] += p0; phase_ms[1] += p1; phase_ms[2] += p2; }
    }
    ILG_TRY(collect_stats(c, false));
  }
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  ILG_TRY(keep_reference(c, solo_plan(c, o)));
  c.frame_no += nsteps;
  return read_device_errors(c);
}

int ilg_get_outputs(ilg_ctx* ctx, double* rad, double* rad_avg, double* therm_avg, double* therm_max) {
  if (!ctx) { set_error("ctx is NULL"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  if (!c.have_thermal) { set_error("ilg_thermal_init has not been called"); return ILG_ERR_ARG; }
  size_t b = (size_t)c.nt * 8;
  if (rad) ILG_CUDA(cudaMemcpyAsync(rad, c.rad.p, b, cudaMemcpyDeviceToHost, c.stream));
  if (rad_avg) ILG_CUDA(cudaMemcpyAsync(rad_avg, c.rad_avg.p, b, cudaMemcpyDeviceToHost, c.stream));
  if (therm_avg) ILG_CUDA(cudaMemcpyAsync(therm_avg, c.therm_avg.p, b, cudaMemcpyDeviceToHost, c.stream));
  if (therm_max) ILG_CUDA(cudaMemcpyAsync(therm_max, c.therm_max.p, b, cudaMemcpyDeviceToHost, c.stream));
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  return ILG_OK;
}

int ilg_record_thermal(ilg_ctx* ctx, int capacity) {
  if (!ctx || capacity < 0) { set_error("invalid arguments"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  invalidate_graph(c);
  if (capacity == 0) { c.rec_cap = 0; return ILG_OK; }
  ILG_TRY(c.rec.alloc((size_t)capacity * REC_W));
  ILG_TRY(c.rec_part.alloc((size_t)div_up(c.nt, conduction_step_threads()) * REC_PART));
  ILG_CUDA(cudaMemset(c.rec.p, 0, (size_t)capacity * REC_W * 8));
  c.rec_cap = capacity;
  c.rec_frame0 = c.frame_no;
  return ILG_OK;
}

int ilg_get_thermal_records(ilg_ctx* ctx, double* out, int* count) {
  if (!ctx || !count) { set_error("invalid arguments"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  int n = std::max(0, std::min(c.rec_cap, c.frame_no - c.rec_frame0));
  *count = n;
  if (out && n > 0) {
    ILG_CUDA(cudaMemcpyAsync(out, c.rec.p, (size_t)n * REC_W * 8, cudaMemcpyDeviceToHost, c.stream));
    ILG_CUDA(cudaStreamSynchronize(c.stream));
  }
  return ILG_OK;
}

// ---- launch-shape autotuner ----------------------------------------------------
int ilg_autotune(ilg_ctx* ctx, const ilg_run_opts* opts, int first_sun, ilg_tune* chosen) {
  if (!ctx) { set_error("ctx is NULL"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  ILG_TRY(check_run(c, opts, false));
  if (first_sun < 0 || first_sun >= c.nsun) { set_error("first_sun out of range"); return ILG_ERR_ARG; }
  const ilg_run_opts& o = *opts;
  cudaStream_t s = c.stream;
  ILG_TRY(upload_desc(c, solo_desc(c, &o, first_sun)));
  // the step kernels run on copies of everything they write
  StepView v = solo_view(c, o.precision);
  const size_t nt = (size_t)c.nt, nl = (size_t)c.nz * nt;
  dbuf<double> sE, srad, sTs, sFs, sQp, sra, sta, stm;
  ILG_TRY(scratch_copy(sE, c.E.p, E_SLOTS * nt, s));
  ILG_TRY(scratch_copy(srad, c.rad.p, nt, s));
  ILG_TRY(scratch_copy(sTs, c.Tsurf.p, nt, s));
  ILG_TRY(scratch_copy(sFs, c.Fsurf.p, nt, s));
  ILG_TRY(scratch_copy(sQp, c.Qprev.p, nt, s));
  ILG_TRY(scratch_copy(sra, c.rad_avg.p, nt, s));
  ILG_TRY(scratch_copy(sta, c.therm_avg.p, nt, s));
  ILG_TRY(scratch_copy(stm, c.therm_max.p, nt, s));
  v.E = sE.p; v.rad = srad.p; v.Tsurf = sTs.p; v.Fsurf = sFs.p; v.Qprev = sQp.p;
  v.rad_avg = sra.p; v.therm_avg = sta.p; v.therm_max = stm.p;
  dbuf<float> sT32;
  dbuf<float2> sTdf;
  if (o.precision == ILG_PREC_MIXED) {
    ILG_TRY(sT32.alloc(nl));
    ILG_CUDA(cudaMemcpyAsync(sT32.p, c.T32.p, nl * 4, cudaMemcpyDeviceToDevice, s));
    v.T32 = sT32.p;
  } else {
    ILG_TRY(sTdf.alloc(nl));
    ILG_CUDA(cudaMemcpyAsync(sTdf.p, c.Tdf.p, nl * 8, cudaMemcpyDeviceToDevice, s));
    v.Tdf = sTdf.p;
  }
  const int mu32 = o.precision == ILG_PREC_MIXED ? 1 : 0;
  const int reps = 10;
  TuneCfg best = c.tune;
  double best_d = 1e300, best_c = 1e300, us = 0.0;
  for (int cb : {128, 256, 512})
    for (int nf : {4, 8, 16, 32}) {
      v.tune.classify_threads = cb;
      v.tune.exact_facets = nf;
      ILG_TRY(time_launches(c, [&] { return direct_launch(v, 0, mu32, 0, s); }, reps, &us));
      if (us < best_d) { best_d = us; best.classify_threads = cb; best.exact_facets = nf; }
    }
  v.tune.classify_threads = best.classify_threads;
  v.tune.exact_facets = best.exact_facets;
  for (int bs : {32, 64, 128}) {
    v.tune.conduct_threads = bs;
    ILG_TRY(time_launches(c, [&] { return conduction_launch(v, v.rad, o.precision, 1, c.nz, s); }, reps, &us));
    if (us < best_c) { best_c = us; best.conduct_threads = bs; }
  }
  ILG_CUDA(cudaStreamSynchronize(s));
  ILG_TRY(read_device_errors(c));
  c.tune = best;
  invalidate_graph(c);   // captured with the previous shapes
  if (chosen) {
    chosen->classify_threads = best.classify_threads;
    chosen->exact_facets = best.exact_facets;
    chosen->conduct_threads = best.conduct_threads;
    chosen->direct_us = best_d;
    chosen->conduct_us = best_c;
  }
  return ILG_OK;
}

int ilg_set_tune(ilg_ctx* ctx, const ilg_tune* t) {
  if (!ctx || !t) { set_error("invalid arguments"); return ILG_ERR_ARG; }
  if ((t->classify_threads != 128 && t->classify_threads != 256 && t->classify_threads != 512) ||
      (t->exact_facets != 4 && t->exact_facets != 8 && t->exact_facets != 16 && t->exact_facets != 32) ||
      (t->conduct_threads != 32 && t->conduct_threads != 64 && t->conduct_threads != 128)) {
    set_error("unsupported launch shape");
    return ILG_ERR_ARG;
  }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  c.tune.classify_threads = t->classify_threads;
  c.tune.exact_facets = t->exact_facets;
  c.tune.conduct_threads = t->conduct_threads;
  invalidate_graph(c);
  return ILG_OK;
}

int ilg_get_tune(const ilg_ctx* ctx, ilg_tune* t) {
  if (!ctx || !t) { set_error("invalid arguments"); return ILG_ERR_ARG; }
  t->classify_threads = ctx->c.tune.classify_threads;
  t->exact_facets = ctx->c.tune.exact_facets;
  t->conduct_threads = ctx->c.tune.conduct_threads;
  t->direct_us = 0.0;
  t->conduct_us = 0.0;
  return ILG_OK;
}

int ilg_set_timing(ilg_ctx* ctx, int enable) {
  if (!ctx) { set_error("ctx is NULL"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  c.timing = enable != 0;
  c.ms_direct = c.ms_rad = c.ms_cond = 0.f;
  c.stats_ambiguous = c.stats_sweeps = 0;
  return ILG_OK;
}

int ilg_get_stats(ilg_ctx* ctx, double* ms_direct, double* ms_radiosity, double* ms_conduction, int64_t* ambiguous,
                  int64_t* sweeps) {
  if (!ctx) { set_error("ctx is NULL"); return ILG_ERR_ARG; }
  Context& c = ctx->c;
  AllocOn on_(c.stream);
  if (ms_direct) *ms_direct = c.ms_direct;
  if (ms_radiosity) *ms_radiosity = c.ms_rad;
  if (ms_conduction) *ms_conduction = c.ms_cond;
  if (ambiguous) *ambiguous = c.stats_ambiguous;
  if (sweeps) *sweeps = c.stats_sweeps;
  return ILG_OK;
}

void conductionq_(int* nz, const double z[], double* dt, double* Qn, double* Qnp1, double T[], const double ti[],
                  const double rhoc[], double* emiss, double* Tsurf, double* Fgeotherm, double* Fsurf) {
  int rc = conduction_batch_host(1, *nz, z, *dt, Qn, Qnp1, T, ti, rhoc, *emiss, Tsurf, *Fgeotherm, Fsurf,
                                 ILG_BC_LINEARISED);
  if (rc != ILG_OK) fprintf(stderr, "conductionq_: %s\n", g_err.c_str());
}

void conductiont_(int* nz, const double z[], double* dt, double T[], double* Tsurf, double* Tsurfp1, const double ti[],
                  const double rhoc[], double* Fgeotherm, double* Fsurf) {
  int rc = conductiont_host(*nz, z, *dt, T, *Tsurf, *Tsurfp1, ti, rhoc, *Fgeotherm, Fsurf);
  if (rc != ILG_OK) fprintf(stderr, "conductiont_: %s\n", g_err.c_str());
}

int ilg_conductionq_batch(int ncol, int nz, const double* z, double dt, const double* Qn, const double* Qnp1, double* T,
                          const double* ti, const double* rhoc, double emiss, double* Tsurf, double Fgeotherm,
                          double* Fsurf, int bc_mode) {
  if (ncol < 0 || !z || !Qnp1 || !T || !ti || !rhoc || !Tsurf || !Fsurf) { set_error("invalid arguments"); return ILG_ERR_ARG; }
  return conduction_batch_host(ncol, nz, z, dt, Qn, Qnp1, T, ti, rhoc, emiss, Tsurf, Fgeotherm, Fsurf, bc_mode);
}

}  // extern "C"
