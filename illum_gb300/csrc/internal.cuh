// internal.cuh — the context object behind ilg_ctx and the launchers each
// translation unit provides. Device layout (all resident in HBM):
//
//   facets (original order):  tri_o  3 x float4 per facet (v0, v1, v2)
//                             cen    float4 (centroid xyz, bounding radius)
//                             nrm    float4 (normal xyz, 0)
//                             area   double
//                             frame  9 doubles per facet (b, t, n columns)
//   LBVH (Karras, BVH2):      nodes  4 x float4 per internal node: both
//                                    children's boxes + child codes
//                                    (>= 0 internal, ~k leaf k)
//                             tri_s  3 x float4 per leaf in Morton order,
//                                    v0.w = original facet index (int bits)
//   horizons:                 H      nphi doubles per facet (= the reference's
//                                    nphi x N column-major matrix)
//   form factors:             CSR by receiver row (rowptr int64, col int32,
//                                    val double | bf16 + row scale)
//   thermal state:            T      layer-major [nz][N] (one coalesced row
//                                    per layer), Tsurf, Fsurf, Qprev, rad,
//                                    rad_avg, therm_avg, therm_max [N]
#pragma once

#include <cuda_bf16.h>

#include <vector>

#include "common.cuh"

namespace ilg {

constexpr int TRACE_STACK = 64;

struct HorizonNode {   // one node of the zenith-angle bisection tree
  double mid, s, c;    // mid angle and its sin / cos (geom.h sincos_x)
  int terminal;        // 1: the bisection returns mid here without a ray
  int pad;
};

// Scalars of a conduction table set (conduction.cu build_tables).
struct CondScalars {
  double alpha0, gamma0, k1, f0, gamma1, Ap, k0, z0, cgeo, es;
  double inv_Ap, S_top, B_top, kz;   // 1/Ap, 2 gamma0/Ap, 2 k1 (S_top - 1), k0/z0
  int nz, bc;                        // bc: 0 linearised, 1 Newton, 2 prescribed Ts (conductionT)
  float esf, B_topf;                 // es, B_top rounded to fp32 (the fp32 Newton root)
  // double-float copies (hi, lo) of the Newton boundary's scalars, for the
  // segmented step kernels: alpha0, gamma0, f0, inv_Ap, S_top, 2 k1,
  // B_top, es, kz
  float2 d_al0, d_g0, d_f0, d_inv_Ap, d_S_top, d_2k1, d_B_top, d_es, d_kz;
};

// Per sun position, precomputed on the host (direct.cu make_sun_aux).
struct SunAux {
  double sx, sy, sz;     // position (km)
  double flux;           // solar_const * (AU / |S|)^2
  float ux, uy, uz;      // unit direction S / |S|
  float alpha;           // bound on the disk samples' angular offset
  float mu_eps;          // bound on |mu32 - mu64|
  float ang_eps;         // bound on the angle between S/|S| and S - p
};

// A run of Morton-consecutive rows of the form-factor matrix solved by one
// block (radiosity.cu): its entries, split evenly over the block's threads,
// and the compact set of facets its rows see (the halo).
struct RowTile {
  int64_t e0;                  // first stored entry (lam x 1024 entries)
  int lam;                     // entries per thread (multiple of 4)
  int nrows;                   // rows (all with entries)
  int r0;                      // first row in t_row / t_scale
  int h0, nhalo;               // halo entries in t_halo
  int mesh;
};

// One mesh of a scene: where its facets, horizons, layers, suns and
// radiosity tiles live in the scene's arrays, and its run state. The step
// kernels read it from device memory, so a captured step graph stays valid
// while meshes advance, finish or are switched off.
// Slots of the direct-flux buffer: frames f, f + 1 and f + 2 (the one-pass
// mixed solve of frame f reads the next frame's flux, computed two frames
// ahead beside the conduction).
constexpr int E_SLOTS = 3;
__host__ __device__ __forceinline__ size_t e_slot(int frame) { return (size_t)(frame % E_SLOTS); }

struct MeshDesc {
  int facet0, nfacet;          // facet range in the scene
  int nphi, interp;
  int64_t H0;                  // offset of the mesh's horizons (nphi per facet)
  double dphi, denom;          // azimuth step; lit-count divisor
  double lit_all;              // nsamp / denom (every sample lit), as the device would divide
  int nsamp, coupling;         // sun-disk samples used; ILG_COUPLE_*
  float dphi32;                // fp32 copy of dphi
  int sun0, nsun;              // the mesh's sun table in the scene's table
  int sun_idx, frame;          // current sun index and frame (advanced per step)
  int host_sun, host_slot;     // 1: take the sun from host_slot (host-driven steps)
  int nz, coef0;               // layers; offset of the conduction table
  int64_t T0;                  // offset of the mesh's [nz][nfacet] layer block
  CondScalars cs;
  int tile0, ntiles;           // radiosity row tiles (0: no radiosity)
  double tol2;                 // squared residual tolerance
  int max_sweeps;
  int refine_every;            // mixed solve: 0 = refinement rounds to tol each step; K >= 1 = one
                               // pass per step, with fl(F) every K-th step (k_radiosity_lagged)
  int ref_age;                 // that solve: steps since its reference pass (-1: none yet)
  int sweeps;                  // out: sweeps of the last solve
  double res2;                 // out: squared residual bound of the last solve
  int active;                  // 0: skipped by the step kernels
  int done_steps;              // steps taken since the run started
  int cb0, ncb;                // the mesh's conduction blocks (thermal records)
  int rec0, rec_cap;           // thermal records: offset (records) and capacity, 0 = not recording
  int rec_frame0;              // frame of record 0
};

// Everything a step kernel touches, as plain device pointers.
// Launch shapes of the step kernels (ilg_autotune picks them by timing; no
// result depends on them).
struct TuneCfg {
  int classify_threads = 256;   // k_direct_classify threads per block
  int exact_facets = 8;         // undecided facets per k_direct_exact block
  int conduct_threads = 64;     // conduction threads per block (single-mesh views)
};

struct StepView {
  TuneCfg tune;
  int nt, nmesh;
  MeshDesc* md;
  const int* mesh_of;          // per facet, or nullptr for a single mesh
  const float4 *cen, *nrm, *frame32;
  const double *frame, *H, *disk, *area;
  const float* H32;            // fp32 copy of H
  const float2* hmm32;         // per facet: fp32 min and max of its horizon
  const float* disk32;         // fp32 copy of the disk samples
  int ndisk;
  const SunAux* suns;
  double *Tsurf, *Fsurf, *Qprev, *rad, *rad_avg, *therm_avg, *therm_max;
  double* E;                   // E_SLOTS x nt: the direct flux of frame f in slot e_slot(f) (before
                               // the coupling, which its readers apply); a drop-in direct call writes slot 0
  float2* sprev;               // 2 x nt by radiosity position, double-floats: scattered radiosity x - E of the last
                               // solve, and its change (the one-pass mixed solve: its predicted change for the
                               // next step)
  float* x32;                  // 3 x nt (mixed radiosity)
  double* T64;                 // [nz][nt] fp64 layers (standalone column entry points)
  float2* Tdf;                 // [nz][nt] double-float layers (the FP64 step)
  float* T32;                  // [nz][nt] fp32 layers (the mixed step)
  const double* coef64;
  const float2* coefdf;
  const float* coef32;
  // radiosity row tiles
  const RowTile* tiles;
  int ntiles;
  const int* blk_start;        // per radiosity block b: its tiles are blk_tile[blk_start[b] .. blk_start[b + 1])
  const int* blk_tile;
  int sched_grid;              // the radiosity grid the schedule was made for
  int l2_stream;               // 1: the stored matrix is much larger than L2 (stream it evict-first)
  const uint16_t* t_cf;        // per stored entry: halo index | row end << 15
  const float* t_vhi;          // double-float values: hi = fl(F)
  const float* t_vlo;          //   and lo = fl(F - hi)
  const __nv_bfloat16* t_vbf;  // value / row scale
  const uint32_t *t_row, *t_halo, *t_start;   // tile rows and halos (positions); per-thread first row
  const float* t_scale;        // per tile row: bf16 scale
  double* tile_d2;             // 2 x ntiles residual partials
  const uint8_t* row_act;      // per radiosity position: its row has entries
  const uint32_t* rperm;       // radiosity position -> facet (Morton order within each mesh)
  double* rbuf;                // 6 x nt: E, two iterates, double-float copies of both and of E (radiosity positions)
  // conduction blocks: (mesh, first local facet), or nullptr for a single mesh
  const int2* cblocks;
  int ncblocks;
  // scratch
  int *work, *counters, *derr, *mesh_flag;
  unsigned* barrier;
  double* rec;                 // thermal records, REC_W doubles each (or nullptr)
  double* rec_part;            // per conduction block: REC_PART doubles
  double* rho64;               // deep-column conduction scratch [nz][nt] (or nullptr)
  float* rho32;
};

// Second stream and fork/join events of the pipelined step (created on
// first use; capi.cu).
struct StepPipe {
  cudaStream_t s2 = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  int init();
  ~StepPipe();
};

struct Context {
  OwnedStream owned_stream;   // destroyed after every buffer (they are freed on it)
  TuneCfg tune;
  int nt = 0;
  cudaStream_t stream = nullptr;   // = owned_stream.s
  StepPipe pipe;
  float scene_mag = 1.0f;   // max |coordinate|
  float r_max = 0.0f;       // max facet bounding radius

  dbuf<float4> tri_o, cen, nrm;
  dbuf<double> area, frame;
  dbuf<float4> frame32;           // float copy of the frame (3 x float4)
  dbuf<float4> nodes, tri_s;
  int root = 0;             // child code of the root (0, or ~0 for one facet)
  dbuf<uint32_t> morton_order;   // facet at each position of the LBVH's Morton order
  int64_t bvh_nodes = 0;
  int bvh_depth = 0;

  // horizons
  int nphi = 0;
  double dphi = 0.0;
  dbuf<double> H;
  dbuf<float> H32;          // fp32 copy (the insolation filters run in fp32)
  dbuf<float2> hmm32;       // per facet: (min_k H, max_k H) in fp32

  // insolation options
  int norm_mode = 0, interp = 0;
  double solar_const = 1372.0;

  // form factors
  bool have_F = false;
  int64_t nnz = 0;
  dbuf<int64_t> rowptr;
  dbuf<int32_t> col;
  dbuf<double> val;
  int n_active = 0;               // rows with at least one entry
  dbuf<float> row_scale;          // per facet: max |F_ij| of its row
  // row tiles of the active rows for the sweeps (radiosity.cu)
  int ntiles = 0;
  int64_t tile_elems = 0;
  std::vector<RowTile> tiles_h;
  dbuf<RowTile> tiles;
  dbuf<uint16_t> t_cf;
  dbuf<float> t_vhi, t_vlo;
  dbuf<__nv_bfloat16> t_vbf;
  dbuf<uint32_t> t_row, t_halo, t_start;
  dbuf<float> t_scale;
  dbuf<double> tile_d2;
  dbuf<int> sched_start, sched_tile;   // per-block tile schedule (radiosity_schedule)
  int sched_grid = 0;
  int tile_blocks = 0;                 // row tiles cut for this many blocks (0: every co-resident block)
  dbuf<uint8_t> row_act;
  dbuf<uint32_t> rperm;           // Morton position -> facet (radiosity's internal order)
  // the reference's fixed-sweep Gauss-Seidel (gauss_seidel.cu)
  int rad_mode = 0;               // ILG_RAD_TOL / ILG_RAD_GS
  int gs_steps = 1;
  bool gs_ready = false;          // gs_rows / gs_lptr describe the current form factors
  dbuf<uint32_t> gs_rows;         // rows in dependency-level order
  std::vector<int> gs_lptr;       // level boundaries in gs_rows
  dbuf<double> gs_x;              // 3 x N: two iterates and the right-hand side

  // thermal
  bool have_thermal = false;
  int nz = 0;
  int bc_mode = 0;
  double emiss = 0.999, Fgeo = 0.0;
  std::vector<double> z_h, ti_h, rhoc_h;
  double coef_dt = -1.0;          // dt the coefficient tables were built for
  int coef_prec = -1;
  dbuf<float2> coefdf;            // per-layer tables (see conduction.cu)
  dbuf<float> coef32;
  CondScalars cond_cs{};
  dbuf<double> rho64;             // deep-column fallback scratch
  dbuf<float> rho32;
  dbuf<float2> Tdf;               // [nz][N] double-float layers (FP64 precision)
  dbuf<float> T32;                // [nz][N] fp32 layers (mixed precision)
  int state_prec = 0;             // which of Tdf / T32 holds the state
  dbuf<double> Tsurf, Fsurf, Qprev;
  dbuf<double> rad, rad_avg, therm_avg, therm_max, E, xtmp, Q;
  dbuf<float2> sprev;             // 2 x N by radiosity position (double-floats): x - E of the last radiosity solve,
                                  // and its change
  int frame_no = 0;
  int ref_age = -1;               // the one-pass mixed solve: steps since its reference step, whose
                                  // s_ref and x_ref (by position) stay in xtmp's S1 and H1; -1: none
  int rec_cap = 0, rec_frame0 = 0;  // thermal records (ilg_record_thermal)
  dbuf<double> rec, rec_part;

  // suns and step machinery
  int nsun = 0;
  std::vector<double> suns_h;     // nsun x 3 positions (to rebuild the table)
  dbuf<double> disk;              // ndisk x 2 column-major
  dbuf<float> disk32;
  int ndisk = 0;
  double disk_rmax = 0.0;
  dbuf<int> work;                 // ambiguous facets
  dbuf<int> counters;             // [0] work count, [1] step (sun index), [2] frame, [3] sweeps
  dbuf<int> derr;                 // DERR_COUNT error flags
  dbuf<unsigned> barrier;         // grid barrier state of the radiosity kernel
  dbuf<float> x32;                // mixed-precision radiosity iterates (3 x N)
  dbuf<SunAux> sun_aux;           // nsun entries + the host slot
  unsigned char* pinned_aux = nullptr;   // 2 SunAux slots (host-driven steps alternate)
  MeshDesc mh{};                  // host mirror of the one-mesh descriptor
  dbuf<MeshDesc> md;
  dbuf<int> mesh_flag;
  double* pinned_tsurf = nullptr;        // 2 x N surface temperatures (alternating slots)
  cudaEvent_t slot_ev[2] = {nullptr, nullptr};
  int64_t stats_ambiguous = 0, stats_sweeps = 0;
  bool timing = false;
  float ms_direct = 0, ms_rad = 0, ms_cond = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};

  // CUDA graph of one step
  cudaGraphExec_t graph = nullptr;       // without copies, or with the copies of slot 0
  cudaGraphExec_t graph_b = nullptr;     // with the copies of slot 1
  int graph_key[6] = {-1, -1, -1, -1, -1, -1};
  bool graph_broken = false;      // capture failed once: launch eagerly

  dbuf<float4> flush;              // L2-eviction buffer of the benchmark loop

  // scratch
  ScanScratch scan;
  SortScratch sort;

  ~Context();
};

// What one step launches (capi.cu enqueue_step).
struct StepPlan {
  int precision;
  bool rad_on;
  bool rec_on;                 // thermal records after conduction
  int rad_grid;
  int rad_inner;               // mixed solve: bf16 sweeps per refinement round (1..radiosity_max_inner())
  bool rad_lagged = false;     // mixed solve: one pass per step, refinement every refine_every steps
  bool layer_sr = false;       // mixed conduction: FP32 layer updates rounded without bias
  int nz_max;
  const Context* gs_ctx = nullptr;   // fixed-sweep Gauss-Seidel of this context instead of the tolerance solve
  int gs_steps = 0;
};

// ---- bvh.cu ----
int bvh_build(Context& c, const float* verts_h, int nv, const int32_t* tris_h, const float* normals_h);
int bvh_trace(Context& c, int nrays, const float* orig_h, const float* dir_h, int any_hit, int32_t* hit_h,
              double* t_h);
// hmesh: the context of a separate horizon mesh whose LBVH the horizon
// rays are traced against (nullptr: c's own)
int horizons_build(Context& c, int nphi, double theta_eps, double offset, const Context* hmesh = nullptr);
int horizons_f32(Context& c);   // H32 and hmm32 from H
int bvh_render(Context& c, int mode, double az_deg, double el_deg, int width, int height, int32_t* out_h);
int form_factors_build(Context& c, const double* albedo_h, double albedo_scalar, double offset,
                       double cutoff, int64_t* rays_out);
int visibility_sample(Context& c, double cutoff, double offset, const int* src_h, int nsrc, const double* radii_h,
                      int nradii, int64_t* per_src_h, int64_t* within_h, int64_t* rays_out);

// ---- direct.cu ----
SunAux make_sun_aux(const double* s, double solar_const, double scene_mag, double disk_rmax);
// ahead = 1: the flux of the frame after each mesh's current one (the
// pipelined step computes it beside the current frame's conduction).
int direct_launch(const StepView& v, int dropin, int mu32_flux, int ahead, cudaStream_t s);

// ---- radiosity.cu ----
int radiosity_prepare(Context& c);
int radiosity_grid(int ntiles, int precision);
int ff_set_chunk(int64_t pairs);   // candidate pairs per form-factor chunk (<= 0: the default)
// Balanced assignment of row tiles to the grid's blocks (longest tiles
// first, each to the least loaded block); uploads it to start/order.
int radiosity_schedule(const std::vector<RowTile>& tiles, int grid, dbuf<int>& start, dbuf<int>& order,
                       cudaStream_t s);
int radiosity_max_meshes();
// whether a matrix of `stored` entries is streamed (larger than ~3/4 of L2)
int radiosity_l2_stream(int64_t stored);
int radiosity_threads();
// unsigned words of a view's barrier buffer: the grid barrier's counter and
// the per-mesh residual accumulators of the radiosity kernels
size_t radiosity_barrier_words(int nmesh);
int radiosity_launch(const StepView& v, double* x, int warm, int precision, int grid, int inner, bool lagged,
                     cudaStream_t s);
int radiosity_barrier_probe(unsigned* bar, int* derr, int blocks, long long polls, int unreachable, cudaStream_t s);
// inner sweeps of a mixed refinement round for a sweep budget (the smallest
// budget of a view's meshes): the budget, at most radiosity_max_inner()
int radiosity_inner(int max_sweeps);

// ---- gauss_seidel.cu ----
int gs_prepare(Context& c);       // dependency levels of the current form factors (once per F)
int gs_levels(const Context& c);
// 1 + gs_steps natural-order sweeps from zero for right-hand side E (device,
// facet order) into x (device, facet order)
int gs_solve_launch(const Context& c, const double* E, double* x, int gs_steps, cudaStream_t s);
// a fused step's solve: the frame's coupled direct flux into v.rad
int gs_step_launch(const Context& c, const StepView& v, int gs_steps, cudaStream_t s);
int gs_residual_launch(const Context& c, const double* E, const double* x, double* r2, cudaStream_t s);

// ---- capi.cu ----
int read_device_errors(Context& c);
int check_run(Context& c, const ilg_run_opts* o, bool host_driven);
MeshDesc solo_desc(const Context& c, const ilg_run_opts* o, int first_sun);
int enqueue_step(const StepView& v, const StepPlan& p, cudaStream_t s, cudaEvent_t* ev);
// Pipelined step: radiosity of the current frame, then its conduction on s
// beside the next frame's direct insolation on pipe.s2, then the advance.
// The current frame's direct flux must be in its E slot already: from the
// previous pipelined step or from enqueue_prologue at the start of a run.
int enqueue_step_pipe(const StepView& v, const StepPlan& p, cudaStream_t s, const StepPipe& pipe);
int enqueue_prologue(const StepView& v, const StepPlan& p, cudaStream_t s);
// Before the first of a run's serial (phase-timed) steps.
int enqueue_serial_prologue(const StepView& v, const StepPlan& p, cudaStream_t s);
int advance_launch(const StepView& v, cudaStream_t s);
int flush_launch(float4* buf, size_t n, unsigned salt, cudaStream_t s);

// ---- conduction.cu ----
int conduction_prepare(Context& c, double dt, int precision);
int conduction_setup();
// Thermal records: per step and mesh, the reference's 12 temperature
// statistics (thermal.hpp:86-126: max, min, mean, sample std over all
// layers incl. the surface, over the surface row, over the bottom layer)
// and three FP64 energy sums (area x absorbed flux, area x emitted flux
// emiss sigma Ts^4, area x conducted flux Fsurf).
constexpr int REC_W = 15;
constexpr int REC_PART = 18;
int record_launch(const StepView& v, int precision, int ncblocks, cudaStream_t s);
int conduction_step_threads();   // facets per conduction block of a scene step
// Q: heat flux at the new time level per facet (global index); upd: also
// update rad_avg / therm_avg / therm_max; nz_max: deepest mesh of the view.
int conduction_launch(const StepView& v, const double* Q, int precision, int upd, int nz_max, cudaStream_t s,
                      bool sr = false);
int conduction_state_convert(Context& c, int precision);
int conduction_batch_host(int ncol, int nz, const double* z, double dt, const double* Qn, const double* Qnp1,
                          double* T, const double* ti, const double* rhoc, double emiss, double* Tsurf,
                          double Fgeo, double* Fsurf, int bc_mode);
int conductiont_host(int nz, const double* z, double dt, double* T, double Tsurf, double Tsurfp1,
                     const double* ti, const double* rhoc, double Fgeo, double* Fsurf);

}  // namespace ilg

struct ilg_ctx {
  ilg::Context c;
};
