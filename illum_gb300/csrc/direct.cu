// direct.cu — direct insolation, src/cpp/illum.cpp:382-466.
//
// The reference counts, for every facet and step, how many of 99 sun-disk
// samples lie above the facet's horizon (two transcendentals per sample).
// On the GPU that count is kept exact, but most facets never evaluate a
// sample:
//   pass 1 (one thread per facet, FP32): the sun disk subtends at most alpha
//     around its centre direction; if the whole disk is certainly above the
//     facet's lowest horizon value the count is 99, if it is certainly below
//     the highest threshold the count is 0, and a facet facing away from
//     the sun contributes 0 whatever the count. The tests carry margins that
//     dominate every rounding error, so they never decide differently from
//     the per-sample evaluation.
//   pass 2 (one warp per remaining facet, FP64): the per-sample evaluation of
//     geom.h sample_lit, bit-identical to the CPU oracle.
// Compiled with -fmad=false (geom.h requirement).
#include "geom.h"
#include "internal.cuh"

namespace ilg {

namespace {

struct SunAux {          // per sun position, precomputed on the host
  double sx, sy, sz;     // position (km)
  double flux;           // solar_const * (AU / |S|)^2
  float ux, uy, uz;      // unit direction S / |S|
  float alpha;           // bound on the disk samples' angular offset
  float mu_eps;          // bound on |mu32 - mu64|
  float pad;
};

struct DirectArgs {
  const float4* cen;
  const float4* nrm;
  const double* frame;
  const double* H;
  const double* hmin;
  const double* hmax;
  const double* disk;     // ndisk x 2 column-major
  int nt, nphi, ndisk, nsamp;
  double dphi, denom;
  int interp;
};

__device__ __forceinline__ frame3 load_frame(const double* fr) {
  frame3 F;
  F.b = mkd(fr[0], fr[1], fr[2]);
  F.t = mkd(fr[3], fr[4], fr[5]);
  F.n = mkd(fr[6], fr[7], fr[8]);
  return F;
}

__device__ __forceinline__ const SunAux* pick_sun(const SunAux* suns, const int* counters, int from_counter) {
  return from_counter ? suns + counters[1] : suns;
}

__global__ void k_direct_classify(DirectArgs a, const SunAux* __restrict__ suns, const int* __restrict__ counters,
                                  int from_counter, const double* __restrict__ base_neg, double* __restrict__ out,
                                  int* __restrict__ work, int* __restrict__ work_count) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  bool amb = false;
  if (f < a.nt) {
    const SunAux* S = pick_sun(suns, counters, from_counter);
    float4 n4 = a.nrm[f];
    float mu32 = (n4.x * S->ux + n4.y * S->uy) + n4.z * S->uz;
    float eps = S->mu_eps;
    double dv = 0.0;
    bool done = true;
    if (mu32 < -eps) {
      dv = 0.0;                      // facing away: max(0, mu) = 0
    } else {
      const float MARG = 1e-6f, CEPS = 1e-6f;
      float alo = (float)a.hmin[f] - S->alpha - MARG;
      float ahi = (float)a.hmax[f] + (float)a.dphi + S->alpha + MARG;
      bool all_lit = alo > 0.f && (mu32 - eps) > cosf(alo) + CEPS;
      bool all_dark = ahi < 3.14159f && (mu32 + eps) < cosf(ahi) - CEPS;
      if (all_lit || all_dark) {
        float4 c4 = a.cen[f];
        d3 p = mkd((double)c4.x, (double)c4.y, (double)c4.z);
        d3 N = normalise(sub(mkd(S->sx, S->sy, S->sz), p));
        const double* fr = a.frame + 9 * (int64_t)f;
        double mu = dot(N, mkd(fr[6], fr[7], fr[8]));
        int count = all_lit ? a.nsamp : 0;
        dv = (double)count / a.denom;
        dv *= (mu > 0.0 ? mu : 0.0);
        dv *= S->flux;
      } else {
        done = false;
      }
    }
    if (done) out[f] = base_neg ? (-base_neg[f] + dv) : dv;
    amb = !done;
  }
  // warp-aggregated append of undecided facets
  unsigned m = __ballot_sync(0xffffffffu, amb);
  if (m) {
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(work_count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (amb) work[base + __popc(m & ((1u << lane) - 1u))] = f;
  }
}

__global__ void k_direct_exact(DirectArgs a, const SunAux* __restrict__ suns, const int* __restrict__ counters,
                               int from_counter, const double* __restrict__ base_neg, double* __restrict__ out,
                               const int* __restrict__ work, const int* __restrict__ work_count) {
  const SunAux* S = pick_sun(suns, counters, from_counter);
  int nw = *work_count;
  int lane = threadIdx.x & 31;
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int nwarps = (gridDim.x * blockDim.x) >> 5;
  d3 Sv = mkd(S->sx, S->sy, S->sz);
  for (int w = warp; w < nw; w += nwarps) {
    int f = work[w];
    float4 c4 = a.cen[f];
    d3 p = mkd((double)c4.x, (double)c4.y, (double)c4.z);
    d3 N = normalise(sub(Sv, p));
    d3 T, B;
    sun_frame(N, &T, &B);
    frame3 BTN = load_frame(a.frame + 9 * (int64_t)f);
    const double* h = a.H + (int64_t)f * a.nphi;
    auto hl = [&](int k) { return h[k]; };
    int count = 0;
    for (int s = lane; s < a.nsamp; s += 32) {
      double x = a.disk[s], y = a.disk[a.ndisk + s];
      d3 disk = add(Sv, scl(add(scl(T, x), scl(B, y)), SUN_RADIUS_KM));
      count += sample_lit(p, disk, BTN, hl, a.nphi, a.dphi, a.interp);
    }
    for (int o = 16; o; o >>= 1) count += __shfl_xor_sync(0xffffffffu, count, o);
    if (lane == 0) {
      double dv = (double)count / a.denom;
      double mu = dot(N, BTN.n);
      dv *= (mu > 0.0 ? mu : 0.0);
      dv *= S->flux;
      out[f] = base_neg ? (-base_neg[f] + dv) : dv;
    }
  }
}

}  // namespace

// Host-side SunAux for one sun position.
static SunAux make_sun_aux(const Context& c, const double* s) {
  SunAux a;
  a.sx = s[0]; a.sy = s[1]; a.sz = s[2];
  double d = norm(mkd(s[0], s[1], s[2]));
  double scale_au = ONE_AU_KM / d;
  a.flux = c.solar_const * (scale_au * scale_au);
  a.ux = (float)(s[0] / d); a.uy = (float)(s[1] / d); a.uz = (float)(s[2] / d);
  double pmax = 1.7320508 * (double)c.scene_mag;
  double dmin = d - pmax;
  if (dmin <= 0.0) {              // sun inside the scene bounds: nothing is decided in pass 1
    a.alpha = 10.0f;
    a.mu_eps = 10.0f;
  } else {
    a.alpha = (float)(SUN_RADIUS_KM * c.disk_rmax / dmin * (1.0 + 1e-6) + 1e-9);
    a.mu_eps = (float)(4e-6 + 2.0 * pmax / dmin);
  }
  a.pad = 0.f;
  return a;
}

int sun_aux_bytes() { return (int)sizeof(SunAux); }

int sun_aux_fill(const Context& c, const double* suns_h, int nsun, void* out_h) {
  SunAux* o = (SunAux*)out_h;
  for (int i = 0; i < nsun; ++i) o[i] = make_sun_aux(c, suns_h + 3 * i);
  return ILG_OK;
}

static DirectArgs make_args(const Context& c) {
  DirectArgs a;
  a.cen = c.cen.p; a.nrm = c.nrm.p; a.frame = c.frame.p; a.H = c.H.p; a.hmin = c.hmin.p; a.hmax = c.hmax.p;
  a.disk = c.disk.p;
  a.nt = c.nt; a.nphi = c.nphi; a.ndisk = c.ndisk; a.nsamp = c.ndisk - 1;
  a.dphi = c.dphi;
  a.denom = c.norm_mode == 0 ? (double)(c.nphi - 1) : (double)(c.ndisk - 1);
  a.interp = c.interp;
  return a;
}

// suns_dev: SunAux array (device); from_counter: index it by counters[1].
// base_neg: when non-null, out = -base_neg + direct (the step's E).
int direct_launch_aux(Context& c, const void* suns_dev, int from_counter, const double* base_neg, double* out_dev) {
  if (c.nphi < 2 || !c.H.p) { set_error("horizons are not set"); return ILG_ERR_ARG; }
  if (c.ndisk < 2) { set_error("sun disk samples are not set"); return ILG_ERR_ARG; }
  DirectArgs a = make_args(c);
  cudaStream_t s = c.stream;
  ILG_CUDA(cudaMemsetAsync(c.counters.p, 0, sizeof(int), s));
  k_direct_classify<<<div_up(c.nt, 256), 256, 0, s>>>(a, (const SunAux*)suns_dev, c.counters.p, from_counter,
                                                      base_neg, out_dev, c.work.p, c.counters.p);
  ILG_CUDA(cudaGetLastError());
  int nsm = 152;
  k_direct_exact<<<nsm * 4, 256, 0, s>>>(a, (const SunAux*)suns_dev, c.counters.p, from_counter, base_neg, out_dev,
                                         c.work.p, c.counters.p);
  ILG_CUDA(cudaGetLastError());
  return ILG_OK;
}

}  // namespace ilg
