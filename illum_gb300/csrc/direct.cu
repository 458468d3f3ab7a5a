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
//   pass 2 (one warp per remaining facet): each sample is classified in FP32
//     with margins, and only samples close to the threshold take the exact
//     per-sample evaluation of geom.h sample_lit in FP64, bit-identical to
//     the CPU oracle.
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
  float ang_eps;         // bound on the angle between S/|S| and S - p
};

struct DirectArgs {
  const float4* cen;
  const float4* nrm;
  const double* frame;
  const float4* frame32;  // float copy: b, t, n (xyz) per facet
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

// Range of the horizon threshold of src/cpp/illum.cpp:431-434 over the
// azimuth interval [a, b] (0 <= a <= b <= 2 pi), bins of width dphi.
__device__ __forceinline__ bool thr_range(const double* __restrict__ h, int nphi, float dphi, int interp, float a,
                                          float b, float& tmin, float& tmax) {
  int k0 = (int)floorf(a / dphi), k1 = (int)floorf(b / dphi);
  k0 = max(0, min(k0, nphi - 1));
  k1 = max(0, min(k1, nphi - 1));
  if (k1 - k0 > 6) return false;
  for (int k = k0; k <= k1; ++k) {
    float lo = fmaxf(a, (float)k * dphi), hi = fminf(b, (float)(k + 1) * dphi);
    if (hi < lo) hi = lo;
    float hk = (float)h[k];
    float v0, v1;
    if (interp == 0) {
      v0 = hk + (lo - (float)k * dphi);
      v1 = hk + (hi - (float)k * dphi);
    } else {
      float hk1 = (float)h[k + 1 < nphi ? k + 1 : nphi - 1];
      v0 = hk + (lo - (float)k * dphi) / dphi * (hk1 - hk);
      v1 = hk + (hi - (float)k * dphi) / dphi * (hk1 - hk);
    }
    tmin = fminf(tmin, fminf(v0, v1));
    tmax = fmaxf(tmax, fmaxf(v0, v1));
  }
  return true;
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
    int decided = 0;                 // 1 dark, 2 lit
    if (mu32 < -eps) {
      decided = 1;                   // facing away: max(0, mu) = 0
    } else {
      const float MARG = 1e-6f, CEPS = 1e-6f;
      float alo = (float)a.hmin[f] - S->alpha - MARG;
      float ahi = (float)a.hmax[f] + (float)a.dphi + S->alpha + MARG;
      if (alo > 0.f && (mu32 - eps) > cosf(alo) + CEPS) decided = 2;
      else if (ahi < 3.14159f && (mu32 + eps) < cosf(ahi) - CEPS) decided = 1;
      else {
        // Bin-aware test: the disk's samples lie within sa of the centre
        // direction, so their azimuths lie within dp of the centre's; the
        // threshold is evaluated only over the bins that interval touches.
        const float4* F4 = a.frame32 + 3 * (size_t)f;
        float4 fb = F4[0], ft = F4[1], fn = F4[2];
        float dx = (fb.x * S->ux + fb.y * S->uy) + fb.z * S->uz;
        float dy = (ft.x * S->ux + ft.y * S->uy) + ft.z * S->uz;
        float dz = (fn.x * S->ux + fn.y * S->uy) + fn.z * S->uz;
        float th = atan2f(sqrtf(dx * dx + dy * dy), dz);
        float sa = S->alpha + S->ang_eps + 2e-6f;
        float sth = sinf(th) - sa - 4e-6f;
        if (th > 0.05f && sth > 0.f) {
          float dp = asinf(fminf(1.f, (sinf(sa) + 1e-6f) / sth)) + 2e-5f;
          if (dp < 0.5f) {
            float ph = atan2f(dy, dx);
            const float TWO_PI_F = 6.2831853f;
            if (ph < 0.f) ph += TWO_PI_F;
            float dphi = (float)a.dphi;
            const double* h = a.H + (size_t)f * a.nphi;
            float tmin = 3e38f, tmax = -3e38f;
            float lo = ph - dp, hi = ph + dp;
            bool ok = true;
            if (lo < 0.f) {
              ok = thr_range(h, a.nphi, dphi, a.interp, lo + TWO_PI_F, TWO_PI_F, tmin, tmax) &&
                   thr_range(h, a.nphi, dphi, a.interp, 0.f, hi, tmin, tmax);
            } else if (hi > TWO_PI_F) {
              ok = thr_range(h, a.nphi, dphi, a.interp, lo, TWO_PI_F, tmin, tmax) &&
                   thr_range(h, a.nphi, dphi, a.interp, 0.f, hi - TWO_PI_F, tmin, tmax);
            } else {
              ok = thr_range(h, a.nphi, dphi, a.interp, lo, hi, tmin, tmax);
            }
            float mt = 3e-5f + S->ang_eps;
            if (ok) {
              if (th + sa + mt < tmin) decided = 2;
              else if (th - sa - mt > tmax) decided = 1;
            }
          }
        }
      }
    }
    if (decided) {
      double dv = 0.0;
      if (decided == 2) {
        float4 c4 = a.cen[f];
        d3 p = mkd((double)c4.x, (double)c4.y, (double)c4.z);
        const double* fr = a.frame + 9 * (int64_t)f;
        double mu = sun_mu(mkd(S->sx, S->sy, S->sz), p, mkd(fr[6], fr[7], fr[8]));
        dv = (double)a.nsamp / a.denom;
        dv *= (mu > 0.0 ? mu : 0.0);
        dv *= S->flux;
      }
      out[f] = base_neg ? (-base_neg[f] + dv) : dv;
    }
    amb = !decided;
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

// Pass 2: one warp per undecided facet. Each sample is first classified
// in FP32 (direction N + kappa (x T + y B) in the facet frame, atan2f);
// only samples within MT of the threshold or MP of a bin edge, or facets
// with the sun near the zenith, are evaluated with the exact FP64
// sample_lit. MT and MP dominate the FP32 errors (~1e-6 rad).
__global__ void k_direct_exact(DirectArgs a, const SunAux* __restrict__ suns, const int* __restrict__ counters,
                               int from_counter, const double* __restrict__ base_neg, double* __restrict__ out,
                               const int* __restrict__ work, const int* __restrict__ work_count) {
  const SunAux* S = pick_sun(suns, counters, from_counter);
  int nw = *work_count;
  int lane = threadIdx.x & 31;
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int nwarps = (gridDim.x * blockDim.x) >> 5;
  d3 Sv = mkd(S->sx, S->sy, S->sz);
  const float MT = 2e-5f, MP = 2e-5f;
  const float dphi = (float)a.dphi;
  for (int w = warp; w < nw; w += nwarps) {
    int f = work[w];
    float4 c4 = a.cen[f];
    d3 p = mkd((double)c4.x, (double)c4.y, (double)c4.z);
    d3 SP = sub(Sv, p);
    double dist = norm(SP);
    d3 N = mkd(SP.x / dist, SP.y / dist, SP.z / dist);   // = geom.h normalise(S - p)
    d3 T, B;
    sun_frame(N, &T, &B);
    frame3 BTN = load_frame(a.frame + 9 * (int64_t)f);
    const double* h = a.H + (int64_t)f * a.nphi;
    auto hl = [&](int k) { return h[k]; };
    const float4* F4 = a.frame32 + 3 * (size_t)f;
    float4 fb = F4[0], ft = F4[1], fn = F4[2];
    float kap = (float)(SUN_RADIUS_KM / dist);
    float Nx = (float)N.x, Ny = (float)N.y, Nz = (float)N.z;
    float Tx = (float)T.x, Ty = (float)T.y, Tz = (float)T.z;
    float Bx = (float)B.x, By = (float)B.y, Bz = (float)B.z;
    int count = 0;
    for (int s = lane; s < a.nsamp; s += 32) {
      double x = a.disk[s], y = a.disk[a.ndisk + s];
      float xf = kap * (float)x, yf = kap * (float)y;
      float vx = Nx + (xf * Tx + yf * Bx), vy = Ny + (xf * Ty + yf * By), vz = Nz + (xf * Tz + yf * Bz);
      float lx = (fb.x * vx + fb.y * vy) + fb.z * vz;
      float ly = (ft.x * vx + ft.y * vy) + ft.z * vz;
      float lz = (fn.x * vx + fn.y * vy) + fn.z * vz;
      float th = atan2f(sqrtf(lx * lx + ly * ly), lz);
      int lit = -1;
      if (th > 0.05f) {
        float ph = atan2f(ly, lx);
        if (ph < 0.f) ph += 6.2831853f;
        int k = (int)floorf(ph / dphi);
        float edge = fminf(ph - (float)k * dphi, (float)(k + 1) * dphi - ph);
        if (k >= 0 && k < a.nphi - 1 && edge > MP) {
          float hk = (float)h[k];
          float thr = a.interp == 0 ? hk + (ph - (float)k * dphi)
                                    : hk + (ph - (float)k * dphi) / dphi * ((float)h[k + 1] - hk);
          float dlt = th - thr;
          if (dlt < -MT) lit = 1;
          else if (dlt > MT) lit = 0;
        }
      }
      if (lit < 0) {
        d3 disk = add(Sv, scl(add(scl(T, x), scl(B, y)), SUN_RADIUS_KM));
        lit = sample_lit(p, disk, BTN, hl, a.nphi, a.dphi, a.interp);
      }
      count += lit;
    }
    for (int o = 16; o; o >>= 1) count += __shfl_xor_sync(0xffffffffu, count, o);
    if (lane == 0) {
      double dv = (double)count / a.denom;
      double mu = sun_mu(Sv, p, BTN.n);
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
    a.ang_eps = 10.0f;
  } else {
    a.alpha = (float)(SUN_RADIUS_KM * c.disk_rmax / dmin * (1.0 + 1e-6) + 1e-9);
    a.mu_eps = (float)(4e-6 + 2.0 * pmax / dmin);
    a.ang_eps = (float)(1e-6 + 2.0 * pmax / dmin);
  }
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
  a.cen = c.cen.p; a.nrm = c.nrm.p; a.frame = c.frame.p; a.frame32 = c.frame32.p; a.H = c.H.p; a.hmin = c.hmin.p; a.hmax = c.hmax.p;
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
