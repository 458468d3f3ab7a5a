// batch.cu — many meshes stepped together: ilg_batch_* of include/illum_gb300.h.
//
// A batch concatenates its member contexts into one scene: facet arrays,
// horizons, layer blocks ([nz][N] per mesh), conduction tables, sun tables
// and the radiosity SELL slices (columns and rows shifted by the mesh's
// first facet), plus a mesh table (MeshDesc) that every step kernel reads.
// One step is then one launch per phase for all active meshes. Each mesh
// keeps its own dt, layer count, thermal profile, sun table, coupling and
// radiosity tolerance; meshes switch off after their last sun position.
// Radiosity convergence is decided per mesh with fixed-order reductions,
// so a mesh's results are bitwise the same alone and in any mix.
#include <algorithm>
#include <cstring>
#include <vector>

#include "internal.cuh"

namespace ilg {

namespace {

__global__ void k_fill_int(int* a, int64_t n, int v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

// shift non-negative entries by off (a member's facet positions)
__global__ void k_shift(int32_t* a, int64_t n, int off) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && a[i] >= 0) a[i] += off;
}

__global__ void k_iota(uint32_t* a, int64_t n, int off) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = (uint32_t)(off + i);
}

}  // namespace

struct Batch {
  OwnedStream owned_stream;   // destroyed after every buffer (they are freed on it)
  std::vector<ilg_ctx*> members;
  std::vector<ilg_run_opts> opts;
  std::vector<MeshDesc> mh;
  int nt = 0, precision = 0, nz_max = 0, ntiles = 0;
  int64_t nel = 0;
  cudaStream_t stream = nullptr;
  StepPipe pipe;
  cudaGraphExec_t graph = nullptr;
  bool graph_broken = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  StepView v{};
  StepPlan plan{};
  // owned scene arrays
  dbuf<MeshDesc> md;
  dbuf<int> mesh_of;
  dbuf<int2> cblocks;
  dbuf<float4> cen, nrm, frame32;
  dbuf<double> frame, H, disk, area, rec, rec_part;
  dbuf<float> H32, disk32;
  dbuf<float2> hmm32;
  dbuf<SunAux> suns;
  dbuf<double> Tsurf, Fsurf, Qprev, rad, rad_avg, therm_avg, therm_max, E, xtmp;
  dbuf<float2> sprev;
  dbuf<float> x32;
  dbuf<float2> Tdf, coefdf;
  dbuf<float> T32, coef32;
  dbuf<RowTile> tiles;
  dbuf<uint16_t> t_cf;
  dbuf<float> t_vhi, t_vlo;
  dbuf<double> tile_d2;
  dbuf<int> sched_start, sched_tile;   // per-block tile schedule of the batch's radiosity grid
  int sched_grid = 0;
  dbuf<__nv_bfloat16> t_vbf;
  dbuf<uint32_t> t_row, t_halo, t_start;
  dbuf<float> t_scale;
  dbuf<uint8_t> row_act;
  dbuf<uint32_t> rperm;
  dbuf<int> work, counters, derr, mesh_flag;
  dbuf<unsigned> barrier;
  dbuf<float4> flush;
  ~Batch() {
    if (graph) cudaGraphExecDestroy(graph);
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
  }
};

template <class T>
static int cat(dbuf<T>& dst, size_t off, const T* src, size_t n, cudaStream_t s) {
  if (n == 0 || !src) return ILG_OK;
  ILG_CUDA(cudaMemcpyAsync(dst.p + off, src, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
  return ILG_OK;
}

static int build(Batch& b) {
  int n = (int)b.members.size();
  cudaStream_t s = b.stream;
  // sizes and offsets
  int64_t nt = 0, nH = 0, nT = 0, ncoef = 0, nsun = 0, ntl = 0, nel = 0, ncb = 0, nrow = 0, nhal = 0, nrec = 0;
  b.mh.assign(n, MeshDesc{});
  b.nz_max = 0;
  int ndisk = -1;
  for (int i = 0; i < n; ++i) {
    Context& c = b.members[i]->c;
    const ilg_run_opts& o = b.opts[i];
    if (c.rad_mode == ILG_RAD_GS && o.use_radiosity) {
      set_error("batch member %d is in the fixed-sweep Gauss-Seidel mode, which runs on single contexts", i);
      return ILG_ERR_ARG;
    }
    {
      AllocOn onm(c.stream);   // the member's own buffers live (and are freed) on its stream
      ILG_TRY(check_run(c, &o, false));
    }
    ILG_CUDA(cudaStreamSynchronize(c.stream));
    if (ndisk < 0) ndisk = c.ndisk;
    if (c.ndisk != ndisk) { set_error("batch members must share the sun-disk samples"); return ILG_ERR_ARG; }
    // a member resumes at its own frame: the sun table covers its whole run
    MeshDesc M = solo_desc(c, &o, c.frame_no);
    M.done_steps = c.frame_no;
    M.active = c.frame_no < c.nsun ? 1 : 0;
    M.facet0 = (int)nt;
    M.H0 = nH;
    M.T0 = nT;
    M.coef0 = (int)ncoef;
    M.sun0 = (int)nsun;
    M.host_slot = (int)(nsun + c.nsun);
    M.tile0 = (int)ntl;
    M.cb0 = (int)ncb;
    M.rec0 = (int)nrec;
    nrec += M.rec_cap;
    b.mh[i] = M;
    nt += c.nt;
    nH += (int64_t)c.nt * c.nphi;
    nT += (int64_t)c.nt * c.nz;
    ncoef += (int64_t)c.nz * 5;
    nsun += c.nsun + 2;   // the table and its two host slots
    ntl += M.ntiles;
    if (M.ntiles) {
      nel += c.tile_elems;
      nrow += c.n_active;
      for (const RowTile& T : c.tiles_h) nhal += T.nhalo;
    }
    ncb += div_up(c.nt, conduction_step_threads());
    b.nz_max = std::max(b.nz_max, c.nz);
  }
  b.nt = (int)nt;
  b.ntiles = (int)ntl;
  b.nel = nel;
  bool mixed = b.precision == ILG_PREC_MIXED;
  // allocations
  ILG_TRY(b.md.alloc(n));
  ILG_TRY(b.mesh_of.alloc(nt));
  ILG_TRY(b.cblocks.alloc(ncb));
  ILG_TRY(b.cen.alloc(nt)); ILG_TRY(b.nrm.alloc(nt)); ILG_TRY(b.frame32.alloc(3 * nt));
  ILG_TRY(b.area.alloc(nt));
  ILG_TRY(b.rec.alloc(nrec > 0 ? nrec * REC_W : 1));
  ILG_TRY(b.rec_part.alloc((ncb > 0 ? ncb : 1) * REC_PART));
  ILG_TRY(b.frame.alloc(9 * nt)); ILG_TRY(b.H.alloc(nH)); ILG_TRY(b.H32.alloc(nH)); ILG_TRY(b.hmm32.alloc(nt));
  ILG_TRY(b.disk.alloc(2 * (size_t)ndisk));
  ILG_TRY(b.disk32.alloc(2 * (size_t)ndisk));
  ILG_TRY(b.suns.alloc(nsun));
  for (dbuf<double>* d : {&b.Tsurf, &b.Fsurf, &b.Qprev, &b.rad, &b.rad_avg, &b.therm_avg, &b.therm_max})
    ILG_TRY(d->alloc(nt));
  ILG_TRY(b.E.alloc(E_SLOTS * (size_t)nt));   // the direct flux of consecutive frames
  ILG_TRY(b.sprev.alloc(2 * nt));
  ILG_TRY(b.xtmp.alloc(6 * nt));
  ILG_TRY(b.rperm.alloc(nt));
  if (mixed) {
    ILG_TRY(b.x32.alloc(3 * nt));
    ILG_TRY(b.T32.alloc(nT));
    ILG_TRY(b.coef32.alloc(ncoef));
  } else {
    ILG_TRY(b.Tdf.alloc(nT));
    ILG_TRY(b.coefdf.alloc(ncoef));
  }
  const int RT = radiosity_threads();
  int64_t ntl1 = ntl > 0 ? ntl : 1, nel1 = nel > 0 ? nel : 1;
  ILG_TRY(b.tiles.alloc(ntl1)); ILG_TRY(b.tile_d2.alloc(2 * ntl1)); ILG_TRY(b.t_start.alloc(ntl1 * RT));
  ILG_TRY(b.t_cf.alloc(nel1)); ILG_TRY(b.t_vhi.alloc(nel1)); ILG_TRY(b.t_vlo.alloc(nel1)); ILG_TRY(b.t_vbf.alloc(nel1));
  ILG_TRY(b.t_row.alloc(nrow > 0 ? nrow : 1)); ILG_TRY(b.t_scale.alloc(nrow > 0 ? nrow : 1));
  ILG_TRY(b.t_halo.alloc(nhal > 0 ? nhal : 1));
  ILG_TRY(b.row_act.alloc(nt));
  ILG_TRY(b.work.alloc(nt)); ILG_TRY(b.counters.alloc(8)); ILG_TRY(b.derr.alloc(DERR_COUNT));
  ILG_TRY(b.mesh_flag.alloc(n)); ILG_TRY(b.barrier.alloc(radiosity_barrier_words(n)));
  // the members' tiles, shifted to the scene's arrays
  std::vector<RowTile> th;
  {
    int64_t e_off = 0, r_off = 0, h_off = 0;
    for (int i = 0; i < n; ++i) {
      Context& c = b.members[i]->c;
      if (!b.mh[i].ntiles) continue;
      for (RowTile T : c.tiles_h) {
        T.e0 += e_off;
        T.r0 += (int)r_off;
        T.h0 += (int)h_off;
        T.mesh = i;
        th.push_back(T);
      }
      e_off += c.tile_elems;
      r_off += c.n_active;
      for (const RowTile& T : c.tiles_h) h_off += T.nhalo;
    }
    if (r_off > INT32_MAX || h_off > INT32_MAX) { set_error("batch too large for the radiosity tiles"); return ILG_ERR_ARG; }
  }
  if (!th.empty())
    ILG_CUDA(cudaMemcpyAsync(b.tiles.p, th.data(), th.size() * sizeof(RowTile), cudaMemcpyHostToDevice, s));
  b.sched_grid = radiosity_grid((int)th.size(), b.precision);
  ILG_TRY(radiosity_schedule(th, b.sched_grid, b.sched_start, b.sched_tile, s));
  ILG_CUDA(cudaMemsetAsync(b.row_act.p, 0, nt, s));
  ILG_CUDA(cudaMemsetAsync(b.counters.p, 0, 8 * sizeof(int), s));
  ILG_CUDA(cudaMemsetAsync(b.derr.p, 0, DERR_COUNT * sizeof(int), s));
  // copies
  std::vector<int2> cbh;
  int64_t el = 0, ro = 0, ho = 0, to = 0;
  for (int i = 0; i < n; ++i) {
    Context& c = b.members[i]->c;
    MeshDesc& M = b.mh[i];
    size_t f0 = M.facet0, N = c.nt;
    ILG_TRY(cat(b.cen, f0, c.cen.p, N, s));
    ILG_TRY(cat(b.nrm, f0, c.nrm.p, N, s));
    ILG_TRY(cat(b.frame32, 3 * f0, c.frame32.p, 3 * N, s));
    ILG_TRY(cat(b.frame, 9 * f0, c.frame.p, 9 * N, s));
    ILG_TRY(cat(b.area, f0, c.area.p, N, s));
    if (M.rec_cap > 0) ILG_TRY(cat(b.rec, (size_t)M.rec0 * REC_W, c.rec.p, (size_t)M.rec_cap * REC_W, s));
    ILG_TRY(cat(b.H, (size_t)M.H0, c.H.p, N * c.nphi, s));
    ILG_TRY(cat(b.H32, (size_t)M.H0, c.H32.p, N * c.nphi, s));
    ILG_TRY(cat(b.hmm32, f0, c.hmm32.p, N, s));
    ILG_TRY(cat(b.suns, (size_t)M.sun0, c.sun_aux.p, (size_t)c.nsun + 2, s));
    ILG_TRY(cat(b.Tsurf, f0, c.Tsurf.p, N, s));
    ILG_TRY(cat(b.Fsurf, f0, c.Fsurf.p, N, s));
    ILG_TRY(cat(b.Qprev, f0, c.Qprev.p, N, s));
    ILG_TRY(cat(b.rad, f0, c.rad.p, N, s));
    ILG_TRY(cat(b.rad_avg, f0, c.rad_avg.p, N, s));
    ILG_TRY(cat(b.therm_avg, f0, c.therm_avg.p, N, s));
    ILG_TRY(cat(b.therm_max, f0, c.therm_max.p, N, s));
    ILG_TRY(cat(b.sprev, f0, c.sprev.p, N, s));
    ILG_TRY(cat(b.sprev, (size_t)nt + f0, c.sprev.p + N, N, s));
    if (M.refine_every > 0 && M.ref_age >= 0) {
      // the one-pass solve's reference (s_ref, x_ref by position: xtmp's S1, H1)
      ILG_TRY(cat(b.xtmp, 2 * (size_t)nt + f0, c.xtmp.p + 2 * N, N, s));
      ILG_TRY(cat(b.xtmp, 4 * (size_t)nt + f0, c.xtmp.p + 4 * N, N, s));
    }
    if (mixed) {
      ILG_TRY(cat(b.T32, (size_t)M.T0, c.T32.p, N * c.nz, s));
      ILG_TRY(cat(b.coef32, (size_t)M.coef0, c.coef32.p, (size_t)c.nz * 5, s));
    } else {
      ILG_TRY(cat(b.Tdf, (size_t)M.T0, c.Tdf.p, N * c.nz, s));
      ILG_TRY(cat(b.coefdf, (size_t)M.coef0, c.coefdf.p, (size_t)c.nz * 5, s));
    }
    if (c.have_F) {
      ILG_TRY(cat(b.row_act, f0, c.row_act.p, N, s));
      ILG_TRY(cat(b.rperm, f0, c.rperm.p, N, s));
      k_shift<<<div_up(N, 256), 256, 0, s>>>((int32_t*)(b.rperm.p + f0), N, (int)f0);
    } else {
      k_iota<<<div_up(N, 256), 256, 0, s>>>(b.rperm.p + f0, N, (int)f0);
    }
    if (M.ntiles > 0) {
      int64_t nh = 0;
      for (const RowTile& T : c.tiles_h) nh += T.nhalo;
      ILG_TRY(cat(b.t_cf, (size_t)el, c.t_cf.p, (size_t)c.tile_elems, s));
      ILG_TRY(cat(b.t_vhi, (size_t)el, c.t_vhi.p, (size_t)c.tile_elems, s));
      ILG_TRY(cat(b.t_vlo, (size_t)el, c.t_vlo.p, (size_t)c.tile_elems, s));
      ILG_TRY(cat(b.t_vbf, (size_t)el, c.t_vbf.p, (size_t)c.tile_elems, s));
      ILG_TRY(cat(b.t_start, (size_t)to * RT, c.t_start.p, (size_t)M.ntiles * RT, s));
      ILG_TRY(cat(b.t_row, (size_t)ro, c.t_row.p, (size_t)c.n_active, s));
      ILG_TRY(cat(b.t_scale, (size_t)ro, c.t_scale.p, (size_t)c.n_active, s));
      ILG_TRY(cat(b.t_halo, (size_t)ho, c.t_halo.p, (size_t)nh, s));
      k_shift<<<div_up(c.n_active, 256), 256, 0, s>>>((int32_t*)(b.t_row.p + ro), c.n_active, (int)f0);
      k_shift<<<div_up(nh, 256), 256, 0, s>>>((int32_t*)(b.t_halo.p + ho), nh, (int)f0);
      ILG_CUDA(cudaGetLastError());
      el += c.tile_elems;
      ro += c.n_active;
      ho += nh;
      to += M.ntiles;
    }
    k_fill_int<<<div_up(N, 256), 256, 0, s>>>(b.mesh_of.p + f0, N, i);
    ILG_CUDA(cudaGetLastError());
    const int cbs = conduction_step_threads();
    for (int k = 0; k < div_up(c.nt, cbs); ++k) cbh.push_back(make_int2(i, k * cbs));
  }
  ILG_TRY(cat(b.disk, 0, b.members[0]->c.disk.p, 2 * (size_t)ndisk, s));
  ILG_TRY(cat(b.disk32, 0, b.members[0]->c.disk32.p, 2 * (size_t)ndisk, s));
  ILG_CUDA(cudaMemcpyAsync(b.cblocks.p, cbh.data(), cbh.size() * sizeof(int2), cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemcpyAsync(b.md.p, b.mh.data(), n * sizeof(MeshDesc), cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  // view
  StepView& v = b.v;
  v = StepView{};
  v.nt = b.nt; v.nmesh = n; v.md = b.md.p; v.mesh_of = b.mesh_of.p;
  v.cen = b.cen.p; v.nrm = b.nrm.p; v.frame32 = b.frame32.p; v.frame = b.frame.p; v.H = b.H.p;
  v.H32 = b.H32.p; v.hmm32 = b.hmm32.p; v.disk = b.disk.p; v.disk32 = b.disk32.p; v.ndisk = ndisk;
  v.area = b.area.p;
  v.rec = nrec > 0 ? b.rec.p : nullptr;
  v.rec_part = b.rec_part.p;
  v.suns = b.suns.p;
  v.Tsurf = b.Tsurf.p; v.Fsurf = b.Fsurf.p; v.Qprev = b.Qprev.p; v.rad = b.rad.p; v.rad_avg = b.rad_avg.p;
  v.therm_avg = b.therm_avg.p; v.therm_max = b.therm_max.p; v.E = b.E.p; v.sprev = b.sprev.p;
  v.x32 = b.x32.p; v.Tdf = b.Tdf.p; v.T32 = b.T32.p; v.coefdf = b.coefdf.p; v.coef32 = b.coef32.p;
  v.tiles = b.tiles.p; v.ntiles = b.ntiles;
  v.blk_start = b.sched_start.p; v.blk_tile = b.sched_tile.p; v.sched_grid = b.sched_grid;
  v.l2_stream = radiosity_l2_stream(b.nel);
  v.t_cf = b.t_cf.p; v.t_vhi = b.t_vhi.p; v.t_vlo = b.t_vlo.p; v.t_vbf = b.t_vbf.p;
  v.t_row = b.t_row.p; v.t_halo = b.t_halo.p; v.t_start = b.t_start.p; v.t_scale = b.t_scale.p;
  v.tile_d2 = b.tile_d2.p;
  v.row_act = b.row_act.p;
  v.rperm = b.rperm.p; v.rbuf = b.xtmp.p;
  v.cblocks = b.cblocks.p; v.ncblocks = (int)ncb;
  v.work = b.work.p; v.counters = b.counters.p; v.derr = b.derr.p; v.mesh_flag = b.mesh_flag.p;
  v.barrier = b.barrier.p;
  v.tune = b.members[0]->c.tune;   // direct-insolation shapes; conduction uses the block table
  b.plan.precision = b.precision;
  b.plan.rad_on = b.ntiles > 0;
  b.plan.rec_on = nrec > 0;
  b.plan.rad_grid = b.plan.rad_on ? radiosity_grid(b.ntiles, b.precision) : 1;
  int min_sweeps = b.opts[0].max_sweeps;
  for (const ilg_run_opts& o : b.opts) min_sweeps = std::min(min_sweeps, o.max_sweeps);
  b.plan.rad_inner = radiosity_inner(min_sweeps);
  b.plan.rad_lagged = b.precision == ILG_PREC_MIXED && b.opts[0].refine_every > 0;
  b.plan.layer_sr = b.precision == ILG_PREC_MIXED && b.opts[0].layer_rounding == 1;
  b.plan.nz_max = b.nz_max;
  return ILG_OK;
}

static int batch_errors(Batch& b) {
  int h[DERR_COUNT];
  ILG_CUDA(cudaMemcpyAsync(h, b.derr.p, sizeof(h), cudaMemcpyDeviceToHost, b.stream));
  ILG_CUDA(cudaStreamSynchronize(b.stream));
  for (int i = 0; i < DERR_COUNT; ++i)
    if (h[i]) {
      ILG_CUDA(cudaMemsetAsync(b.derr.p, 0, sizeof(h), b.stream));
      set_error("device error flag %d set during a batch step", i);
      return i == DERR_PIVOT ? ILG_ERR_PIVOT : ILG_ERR_DEVICE;
    }
  return ILG_OK;
}

static int batch_graph(Batch& b, cudaGraphExec_t* out) {
  if (b.graph) { *out = b.graph; return ILG_OK; }
  cudaGraph_t g;
  ILG_CUDA(cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_step_pipe(b.v, b.plan, b.stream, b.pipe);
  cudaError_t e = cudaStreamEndCapture(b.stream, &g);
  if (rc != ILG_OK || e != cudaSuccess) {
    cudaGetLastError();
    if (e == cudaSuccess) cudaGraphDestroy(g);
    set_error("batch step capture failed: %s", cudaGetErrorString(e));
    return rc != ILG_OK ? rc : ILG_ERR_CUDA;
  }
  cudaError_t ei = cudaGraphInstantiate(&b.graph, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) { b.graph = nullptr; set_error("graph instantiation failed"); return ILG_ERR_CUDA; }
  *out = b.graph;
  return ILG_OK;
}

}  // namespace ilg

using namespace ilg;

struct ilg_batch {
  Batch b;
};

extern "C" {

int ilg_batch_create(ilg_ctx** members, int n, const ilg_run_opts* opts, ilg_batch** out) {
  if (!members || n < 1 || !opts || !out) { set_error("invalid batch arguments"); return ILG_ERR_ARG; }
  if (n > radiosity_max_meshes()) { set_error("a batch holds at most %d meshes", radiosity_max_meshes()); return ILG_ERR_ARG; }
  for (int i = 1; i < n; ++i)
    if (opts[i].precision != opts[0].precision) { set_error("batch members must share one precision"); return ILG_ERR_ARG; }
  for (int i = 1; i < n; ++i)
    if (opts[i].layer_rounding != opts[0].layer_rounding) {
      set_error("batch members must share one layer_rounding");
      return ILG_ERR_ARG;
    }
  for (int i = 1; i < n; ++i)
    if ((opts[i].refine_every > 0) != (opts[0].refine_every > 0)) {
      set_error("batch members must all use refine_every > 0 or all 0");
      return ILG_ERR_ARG;
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j)
      if (members[i] == members[j]) { set_error("a context appears twice in the batch"); return ILG_ERR_ARG; }
  *out = nullptr;
  ilg_batch* h = new ilg_batch();
  Batch& b = h->b;
  b.members.assign(members, members + n);
  b.opts.assign(opts, opts + n);
  b.precision = opts[0].precision;
  if (cudaStreamCreateWithFlags(&b.owned_stream.s, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    set_error("cudaStreamCreate failed");
    return ILG_ERR_CUDA;
  }
  b.stream = b.owned_stream.s;
  AllocOn on(b.stream);
  for (auto& e : b.ev)
    if (cudaEventCreate(&e) != cudaSuccess) { delete h; set_error("cudaEventCreate failed"); return ILG_ERR_CUDA; }
  if (b.pipe.init() != ILG_OK) { delete h; return ILG_ERR_CUDA; }
  int rc = build(b);
  if (rc != ILG_OK) { delete h; return rc; }
  *out = h;
  return ILG_OK;
}

int ilg_batch_destroy(ilg_batch* batch) {
  delete batch;
  return ILG_OK;
}

int ilg_batch_run(ilg_batch* batch, int nsteps, int use_graph) {
  if (!batch || nsteps < 0) { set_error("invalid arguments"); return ILG_ERR_ARG; }
  Batch& b = batch->b;
  cudaGraphExec_t g = nullptr;
  if (use_graph && !b.graph_broken)
    if (batch_graph(b, &g) != ILG_OK) { b.graph_broken = true; g = nullptr; cudaGetLastError(); }
  if (nsteps > 0) ILG_TRY(enqueue_prologue(b.v, b.plan, b.stream));
  for (int s = 0; s < nsteps; ++s) {
    if (g) ILG_CUDA(cudaGraphLaunch(g, b.stream));
    else ILG_TRY(enqueue_step_pipe(b.v, b.plan, b.stream, b.pipe));
  }
  ILG_CUDA(cudaStreamSynchronize(b.stream));
  return batch_errors(b);
}

int ilg_batch_bench(ilg_batch* batch, int nsteps, double flush_mb, double* step_ms) {
  if (!batch || nsteps < 0 || !step_ms) { set_error("invalid arguments"); return ILG_ERR_ARG; }
  Batch& b = batch->b;
  AllocOn on_(b.stream);
  size_t nflush = flush_mb > 0 ? (size_t)(flush_mb * 1048576.0 / 16.0) : 0;
  if (nflush) ILG_TRY(b.flush.reserve(nflush));
  cudaGraphExec_t g = nullptr;
  if (!b.graph_broken)
    if (batch_graph(b, &g) != ILG_OK) { b.graph_broken = true; g = nullptr; cudaGetLastError(); }
  if (nsteps > 0) ILG_TRY(enqueue_prologue(b.v, b.plan, b.stream));   // untimed
  for (int s = 0; s < nsteps; ++s) {
    if (nflush) ILG_TRY(flush_launch(b.flush.p, nflush, (unsigned)s, b.stream));
    ILG_CUDA(cudaEventRecord(b.ev[0], b.stream));
    if (g) ILG_CUDA(cudaGraphLaunch(g, b.stream));
    else ILG_TRY(enqueue_step_pipe(b.v, b.plan, b.stream, b.pipe));
    ILG_CUDA(cudaEventRecord(b.ev[3], b.stream));
    ILG_CUDA(cudaEventSynchronize(b.ev[3]));
    float ms = 0.f;
    ILG_CUDA(cudaEventElapsedTime(&ms, b.ev[0], b.ev[3]));
    step_ms[s] = ms;
  }
  return batch_errors(b);
}

// Eager steps in the serial order (no graph, no pipelining) with their
// phase boundaries recorded: phase_ms[0..2] accumulates the direct,
// radiosity and conduction phases of all members.
int ilg_batch_bench_phases(ilg_batch* batch, int nsteps, double flush_mb, double* step_ms, double* phase_ms) {
  if (!batch || nsteps < 0 || !step_ms || !phase_ms) { set_error("invalid arguments"); return ILG_ERR_ARG; }
  Batch& b = batch->b;
  AllocOn on_(b.stream);
  size_t nflush = flush_mb > 0 ? (size_t)(flush_mb * 1048576.0 / 16.0) : 0;
  if (nflush) ILG_TRY(b.flush.reserve(nflush));
  phase_ms[0] = phase_ms[1] = phase_ms[2] = 0.0;
  if (nsteps > 0) ILG_TRY(enqueue_serial_prologue(b.v, b.plan, b.stream));
  for (int s = 0; s < nsteps; ++s) {
    if (nflush) ILG_TRY(flush_launch(b.flush.p, nflush, (unsigned)s, b.stream));
    ILG_TRY(enqueue_step(b.v, b.plan, b.stream, b.ev));
    ILG_CUDA(cudaEventSynchronize(b.ev[3]));
    float p0, p1, p2;
    ILG_CUDA(cudaEventElapsedTime(&p0, b.ev[0], b.ev[1]));
    ILG_CUDA(cudaEventElapsedTime(&p1, b.ev[1], b.ev[2]));
    ILG_CUDA(cudaEventElapsedTime(&p2, b.ev[2], b.ev[3]));
    step_ms[s] = (double)p0 + p1 + p2;
    phase_ms[0] += p0;
    phase_ms[1] += p1;
    phase_ms[2] += p2;
  }
  ILG_CUDA(cudaStreamSynchronize(b.stream));
  return batch_errors(b);
}

int ilg_batch_autotune(ilg_batch* batch, ilg_tune* chosen) {
  if (!batch) { set_error("batch is NULL"); return ILG_ERR_ARG; }
  Batch& b = batch->b;
  AllocOn on_(b.stream);
  cudaStream_t s = b.stream;
  // the direct passes write the flux slots (timed on a copy) and the
  // undecided-facet list and count (scratch of the pass itself)
  dbuf<double> sE;
  ILG_TRY(sE.alloc(b.E.n));
  ILG_CUDA(cudaMemcpyAsync(sE.p, b.E.p, b.E.n * 8, cudaMemcpyDeviceToDevice, s));
  StepView v = b.v;
  v.E = sE.p;
  const int mu32 = b.precision == ILG_PREC_MIXED ? 1 : 0;
  cudaEvent_t e0 = b.ev[0], e1 = b.ev[3];
  const int reps = 10;
  double best = 1e300;
  int best_cb = v.tune.classify_threads, best_nf = v.tune.exact_facets;
  for (int cb : {128, 256, 512})
    for (int nf : {4, 8, 16, 32}) {
      v.tune.classify_threads = cb;
      v.tune.exact_facets = nf;
      for (int i = 0; i < 2; ++i) ILG_TRY(direct_launch(v, 0, mu32, 0, s));
      ILG_CUDA(cudaEventRecord(e0, s));
      for (int i = 0; i < reps; ++i) ILG_TRY(direct_launch(v, 0, mu32, 0, s));
      ILG_CUDA(cudaEventRecord(e1, s));
      ILG_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      ILG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      const double us = 1000.0 * ms / reps;
      if (us < best) { best = us; best_cb = cb; best_nf = nf; }
    }
  ILG_TRY(batch_errors(b));
  b.v.tune.classify_threads = best_cb;
  b.v.tune.exact_facets = best_nf;
  if (b.graph) {   // captured with the previous shapes
    cudaGraphExecDestroy(b.graph);
    b.graph = nullptr;
  }
  if (chosen) {
    chosen->classify_threads = best_cb;
    chosen->exact_facets = best_nf;
    chosen->conduct_threads = conduction_step_threads();
    chosen->direct_us = best;
    chosen->conduct_us = 0.0;
  }
  return ILG_OK;
}

int ilg_batch_status(ilg_batch* batch, int* active, int* steps_done, int* sweeps) {
  if (!batch) { set_error("batch is NULL"); return ILG_ERR_ARG; }
  Batch& b = batch->b;
  int n = (int)b.members.size();
  std::vector<MeshDesc> m(n);
  ILG_CUDA(cudaMemcpyAsync(m.data(), b.md.p, n * sizeof(MeshDesc), cudaMemcpyDeviceToHost, b.stream));
  ILG_CUDA(cudaStreamSynchronize(b.stream));
  for (int i = 0; i < n; ++i) {
    if (active) active[i] = m[i].active;
    if (steps_done) steps_done[i] = m[i].done_steps;
    if (sweeps) sweeps[i] = m[i].sweeps;
  }
  return ILG_OK;
}

int ilg_batch_set_active(ilg_batch* batch, int member, int active) {
  if (!batch || member < 0 || member >= (int)batch->b.members.size()) { set_error("invalid member"); return ILG_ERR_ARG; }
  Batch& b = batch->b;
  MeshDesc* d = b.md.p + member;
  int a = active ? 1 : 0;
  ILG_CUDA(cudaMemcpyAsync(&d->active, &a, sizeof(int), cudaMemcpyHostToDevice, b.stream));
  ILG_CUDA(cudaStreamSynchronize(b.stream));
  return ILG_OK;
}

int ilg_batch_get_tsurf(ilg_batch* batch, int member, double* out) {
  if (!batch || !out || member < 0 || member >= (int)batch->b.members.size()) { set_error("invalid member"); return ILG_ERR_ARG; }
  Batch& b = batch->b;
  const MeshDesc& M = b.mh[member];
  ILG_CUDA(cudaMemcpyAsync(out, b.Tsurf.p + M.facet0, (size_t)M.nfacet * 8, cudaMemcpyDeviceToHost, b.stream));
  ILG_CUDA(cudaStreamSynchronize(b.stream));
  return ILG_OK;
}

// Copy every member's state back into its context (temperatures, fluxes,
// averages, radiosity history, frame counter).
int ilg_batch_sync(ilg_batch* batch) {
  if (!batch) { set_error("batch is NULL"); return ILG_ERR_ARG; }
  Batch& b = batch->b;
  int n = (int)b.members.size();
  std::vector<MeshDesc> m(n);
  ILG_CUDA(cudaMemcpyAsync(m.data(), b.md.p, n * sizeof(MeshDesc), cudaMemcpyDeviceToHost, b.stream));
  ILG_CUDA(cudaStreamSynchronize(b.stream));
  bool mixed = b.precision == ILG_PREC_MIXED;
  for (int i = 0; i < n; ++i) {
    Context& c = b.members[i]->c;
    const MeshDesc& M = b.mh[i];
    size_t f0 = M.facet0, N = c.nt, bytes = N * 8;
    cudaStream_t s = b.stream;
    ILG_CUDA(cudaMemcpyAsync(c.Tsurf.p, b.Tsurf.p + f0, bytes, cudaMemcpyDeviceToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.Fsurf.p, b.Fsurf.p + f0, bytes, cudaMemcpyDeviceToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.Qprev.p, b.Qprev.p + f0, bytes, cudaMemcpyDeviceToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.rad.p, b.rad.p + f0, bytes, cudaMemcpyDeviceToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.rad_avg.p, b.rad_avg.p + f0, bytes, cudaMemcpyDeviceToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.therm_avg.p, b.therm_avg.p + f0, bytes, cudaMemcpyDeviceToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.therm_max.p, b.therm_max.p + f0, bytes, cudaMemcpyDeviceToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.sprev.p, b.sprev.p + f0, bytes, cudaMemcpyDeviceToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.sprev.p + N, b.sprev.p + (size_t)b.nt + f0, bytes, cudaMemcpyDeviceToDevice, s));
    if (b.plan.rad_lagged && M.ntiles > 0) {
      c.ref_age = m[i].ref_age;
      if (c.ref_age >= 0) {
        ILG_CUDA(cudaMemcpyAsync(c.xtmp.p + 2 * N, b.xtmp.p + 2 * (size_t)b.nt + f0, bytes, cudaMemcpyDeviceToDevice, s));
        ILG_CUDA(cudaMemcpyAsync(c.xtmp.p + 4 * N, b.xtmp.p + 4 * (size_t)b.nt + f0, bytes, cudaMemcpyDeviceToDevice, s));
      }
    } else if (M.ntiles > 0) {
      c.ref_age = -1;
    }
    if (mixed)
      ILG_CUDA(cudaMemcpyAsync(c.T32.p, b.T32.p + M.T0, N * c.nz * 4, cudaMemcpyDeviceToDevice, s));
    else
      ILG_CUDA(cudaMemcpyAsync(c.Tdf.p, b.Tdf.p + M.T0, N * c.nz * 8, cudaMemcpyDeviceToDevice, s));
    if (M.rec_cap > 0)
      ILG_CUDA(cudaMemcpyAsync(c.rec.p, b.rec.p + (size_t)M.rec0 * REC_W, (size_t)M.rec_cap * REC_W * 8,
                               cudaMemcpyDeviceToDevice, s));
    c.frame_no = m[i].frame;
  }
  ILG_CUDA(cudaStreamSynchronize(b.stream));
  return ILG_OK;
}

}  // extern "C"
