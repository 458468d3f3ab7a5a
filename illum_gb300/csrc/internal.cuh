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
  int nz, bc;                        // bc: 0 linearised, 1 Newton, 2 prescribed Ts (conductionT)
};

struct Context {
  int nt = 0;
  cudaStream_t stream = nullptr;
  float scene_mag = 1.0f;   // max |coordinate|
  float r_max = 0.0f;       // max facet bounding radius

  dbuf<float4> tri_o, cen, nrm;
  dbuf<double> area, frame;
  dbuf<float4> frame32;           // float copy of the frame (3 x float4)
  dbuf<float4> nodes, tri_s;
  int root = 0;             // child code of the root (0, or ~0 for one facet)
  int64_t bvh_nodes = 0;
  int bvh_depth = 0;

  // horizons
  int nphi = 0;
  double dphi = 0.0;
  dbuf<double> H;
  dbuf<double> hmin, hmax;  // per facet: min_k H, max_k H

  // insolation options
  int norm_mode = 0, interp = 0;
  double solar_const = 1372.0;

  // form factors
  bool have_F = false;
  int64_t nnz = 0;
  dbuf<int64_t> rowptr;
  dbuf<int32_t> col;
  dbuf<double> val;
  dbuf<int32_t> active;           // rows with at least one entry
  int n_active = 0;
  dbuf<__nv_bfloat16> val_bf16;   // mixed precision copy
  dbuf<float> row_scale;
  bool have_bf16 = false;
  // SELL-32 copy of the active rows for the sweeps (radiosity.cu)
  int sell_nslices = 0;
  int64_t sell_elems = 0;
  dbuf<int64_t> sell_ptr;
  dbuf<int32_t> sell_len, sell_split, sell_row, sell_m, sell_col;
  dbuf<double> sell_val;
  dbuf<__nv_bfloat16> sell_vbf;

  // thermal
  bool have_thermal = false;
  int nz = 0;
  int bc_mode = 0;
  double emiss = 0.999, Fgeo = 0.0;
  std::vector<double> z_h, ti_h, rhoc_h;
  double coef_dt = -1.0;          // dt the coefficient tables were built for
  int coef_prec = -1;
  dbuf<double> coef64;            // per-layer tables (see conduction.cu)
  dbuf<float> coef32;
  CondScalars cond_cs{};
  dbuf<double> rho64;             // deep-column fallback scratch
  dbuf<float> rho32;
  dbuf<double> T64;               // [nz][N]
  dbuf<float> T32;
  int state_prec = 0;             // which of T64 / T32 holds the state
  dbuf<double> Tsurf, Fsurf, Qprev;
  dbuf<double> rad, rad_avg, therm_avg, therm_max, E, xtmp, Q;
  dbuf<double> xprev;             // radiosity solution of the step before
  int frame_no = 0;

  // suns and step machinery
  int nsun = 0;
  dbuf<double> suns;              // nsun x 3
  dbuf<double> disk;              // ndisk x 2 column-major
  int ndisk = 0;
  double disk_rmax = 0.0;
  dbuf<int> work;                 // ambiguous facets
  dbuf<int> counters;             // [0] work count, [1] step (sun index), [2] frame, [3] sweeps
  dbuf<int> derr;                 // DERR_COUNT error flags
  dbuf<double> partials;          // radiosity residual partials (2 x grid + 1)
  dbuf<unsigned> barrier;         // grid barrier state of the radiosity kernel
  dbuf<float> x32;                // mixed-precision radiosity iterates (3 x N)
  int rad_grid = 0;
  int rad_grid_prec = -1;
  dbuf<unsigned char> sun_aux;    // per-sun precomputed data (direct.cu SunAux)
  dbuf<unsigned char> host_sun_aux;  // one entry for host-driven steps
  unsigned char* pinned_aux = nullptr;
  double* pinned_tsurf = nullptr;
  int64_t stats_ambiguous = 0, stats_sweeps = 0;
  bool timing = false;
  float ms_direct = 0, ms_rad = 0, ms_cond = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};

  // CUDA graph of one step
  cudaGraphExec_t graph = nullptr;
  int graph_key[4] = {-1, -1, -1, -1};
  bool graph_broken = false;      // capture failed once: launch eagerly

  dbuf<float4> flush;              // L2-eviction buffer of the benchmark loop

  // scratch
  ScanScratch scan;
  SortScratch sort;

  ~Context();
};

// ---- bvh.cu ----
int bvh_build(Context& c, const float* verts_h, int nv, const int32_t* tris_h, const float* normals_h);
int bvh_trace(Context& c, int nrays, const float* orig_h, const float* dir_h, int any_hit, int32_t* hit_h,
              double* t_h);
int horizons_build(Context& c, int nphi, double theta_eps, double offset);
int form_factors_build(Context& c, const double* albedo_h, double albedo_scalar, double offset,
                       int64_t* rays_out);

// ---- direct.cu ----
int sun_aux_bytes();
int sun_aux_fill(const Context& c, const double* suns_h, int nsun, void* out_h);
int direct_launch_aux(Context& c, const void* suns_dev, int from_counter, const double* base_neg,
                      double* out_dev);

// ---- radiosity.cu ----
int radiosity_prepare(Context& c);
int radiosity_setup(Context& c, int precision);
int radiosity_launch(Context& c, const double* E_dev, double* x_dev, double tol, int max_sweeps,
                     int precision, bool warm_start);

// ---- capi.cu ----
int read_device_errors(Context& c);

// ---- conduction.cu ----
int conduction_prepare(Context& c, double dt, int precision);
int conduction_setup();
int conduction_launch(Context& c, const double* Q_dev, int precision, bool update_outputs);
int conduction_state_convert(Context& c, int precision);
int conduction_batch_host(int ncol, int nz, const double* z, double dt, const double* Qn, const double* Qnp1,
                          double* T, const double* ti, const double* rhoc, double emiss, double* Tsurf,
                          double Fgeo, double* Fsurf, int bc_mode);
int conductiont_host(int nz, const double* z, double dt, double* T, double Tsurf, double Tsurfp1,
                     const double* ti, const double* rhoc, double Fgeo, double* Fsurf);

}  // namespace ilg
