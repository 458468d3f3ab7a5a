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

__device__ __forceinline__ frame3 load_frame(const double* fr) {
  frame3 F;
  F.b = mkd(fr[0], fr[1], fr[2]);
  F.t = mkd(fr[3], fr[4], fr[5]);
  F.n = mkd(fr[6], fr[7], fr[8]);
  return F;
}

__device__ __forceinline__ const SunAux* mesh_sun(const StepView& v, const MeshDesc& M) {
  return v.suns + (M.host_sun ? M.host_slot : M.sun0 + M.sun_idx);
}

// Where a facet's direct flux goes: the step's E (radiosity follows), rad
// directly (no radiosity for this mesh), or E alone (drop-in call).
__device__ __forceinline__ void store_direct(const StepView& v, const MeshDesc& M, int g, double dv, int dropin) {
  if (dropin) { v.E[g] = dv; return; }
  double e = M.coupling == ILG_COUPLE_REFERENCE ? (-v.Fsurf[g] + dv) : dv;
  if (M.ntiles > 0) v.E[g] = e; else v.rad[g] = e;
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

__global__ void k_direct_classify(StepView v, int dropin) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  bool amb = false;
  const MeshDesc* Mp = nullptr;
  if (f < v.nt) {
    Mp = &v.md[v.mesh_of ? v.mesh_of[f] : 0];
    if (!Mp->active) Mp = nullptr;
  }
  if (Mp) {
    const MeshDesc& M = *Mp;
    const SunAux* S = mesh_sun(v, M);
    float4 n4 = v.nrm[f];
    float mu32 = (n4.x * S->ux + n4.y * S->uy) + n4.z * S->uz;
    float eps = S->mu_eps;
    int decided = 0;                 // 1 dark, 2 lit
    if (mu32 < -eps) {
      decided = 1;                   // facing away: max(0, mu) = 0
    } else {
      const float MARG = 1e-6f, CEPS = 1e-6f;
      float alo = (float)v.hmin[f] - S->alpha - MARG;
      float ahi = (float)v.hmax[f] + (float)M.dphi + S->alpha + MARG;
      if (alo > 0.f && (mu32 - eps) > cosf(alo) + CEPS) decided = 2;
      else if (ahi < 3.14159f && (mu32 + eps) < cosf(ahi) - CEPS) decided = 1;
      else {
        // Bin-aware test: the disk's samples lie within sa of the centre
        // direction, so their azimuths lie within dp of the centre's; the
        // threshold is evaluated only over the bins that interval touches.
        const float4* F4 = v.frame32 + 3 * (size_t)f;
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
            float dphi = (float)M.dphi;
            const double* h = v.H + M.H0 + (size_t)(f - M.facet0) * M.nphi;
            float tmin = 3e38f, tmax = -3e38f;
            float lo = ph - dp, hi = ph + dp;
            bool ok = true;
            if (lo < 0.f) {
              ok = thr_range(h, M.nphi, dphi, M.interp, lo + TWO_PI_F, TWO_PI_F, tmin, tmax) &&
                   thr_range(h, M.nphi, dphi, M.interp, 0.f, hi, tmin, tmax);
            } else if (hi > TWO_PI_F) {
              ok = thr_range(h, M.nphi, dphi, M.interp, lo, TWO_PI_F, tmin, tmax) &&
                   thr_range(h, M.nphi, dphi, M.interp, 0.f, hi - TWO_PI_F, tmin, tmax);
            } else {
              ok = thr_range(h, M.nphi, dphi, M.interp, lo, hi, tmin, tmax);
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
        float4 c4 = v.cen[f];
        d3 p = mkd((double)c4.x, (double)c4.y, (double)c4.z);
        const double* fr = v.frame + 9 * (int64_t)f;
        double mu = sun_mu(mkd(S->sx, S->sy, S->sz), p, mkd(fr[6], fr[7], fr[8]));
        dv = (double)M.nsamp / M.denom;
        dv *= (mu > 0.0 ? mu : 0.0);
        dv *= S->flux;
      }
      store_direct(v, M, f, dv, dropin);
    }
    amb = !decided;
  }
  // warp-aggregated append of undecided facets
  unsigned m = __ballot_sync(0xffffffffu, amb);
  if (m) {
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&v.counters[0], __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (amb) v.work[base + __popc(m & ((1u << lane) - 1u))] = f;
  }
}

// Pass 2: one warp per undecided facet. Each sample is first classified
// in FP32 (direction N + kappa (x T + y B) in the facet frame, atan2f);
// only samples within MT of the threshold or MP of a bin edge, or facets
// with the sun near the zenith, are evaluated with the exact FP64
// sample_lit. MT and MP dominate the FP32 errors (~1e-6 rad).
__global__ void k_direct_exact(StepView v, int dropin) {
  int nw = v.counters[0];
  int lane = threadIdx.x & 31;
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int nwarps = (gridDim.x * blockDim.x) >> 5;
  const float MT = 2e-5f, MP = 2e-5f;
  for (int w = warp; w < nw; w += nwarps) {
    int f = v.work[w];
    const MeshDesc& M = v.md[v.mesh_of ? v.mesh_of[f] : 0];
    const SunAux* S = mesh_sun(v, M);
    d3 Sv = mkd(S->sx, S->sy, S->sz);
    const float dphi = (float)M.dphi;
    float4 c4 = v.cen[f];
    d3 p = mkd((double)c4.x, (double)c4.y, (double)c4.z);
    d3 SP = sub(Sv, p);
    double dist = norm(SP);
    d3 N = mkd(SP.x / dist, SP.y / dist, SP.z / dist);   // = geom.h normalise(S - p)
    d3 T, B;
    sun_frame(N, &T, &B);
    frame3 BTN = load_frame(v.frame + 9 * (int64_t)f);
    const double* h = v.H + M.H0 + (int64_t)(f - M.facet0) * M.nphi;
    auto hl = [&](int k) { return h[k]; };
    const float4* F4 = v.frame32 + 3 * (size_t)f;
    float4 fb = F4[0], ft = F4[1], fn = F4[2];
    float kap = (float)(SUN_RADIUS_KM / dist);
    float Nx = (float)N.x, Ny = (float)N.y, Nz = (float)N.z;
    float Tx = (float)T.x, Ty = (float)T.y, Tz = (float)T.z;
    float Bx = (float)B.x, By = (float)B.y, Bz = (float)B.z;
    int count = 0;
    for (int s = lane; s < M.nsamp; s += 32) {
      double x = v.disk[s], y = v.disk[v.ndisk + s];
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
        if (k >= 0 && k < M.nphi - 1 && edge > MP) {
          float hk = (float)h[k];
          float thr = M.interp == 0 ? hk + (ph - (float)k * dphi)
                                    : hk + (ph - (float)k * dphi) / dphi * ((float)h[k + 1] - hk);
          float dlt = th - thr;
          if (dlt < -MT) lit = 1;
          else if (dlt > MT) lit = 0;
        }
      }
      if (lit < 0) {
        d3 disk = add(Sv, scl(add(scl(T, x), scl(B, y)), SUN_RADIUS_KM));
        lit = sample_lit(p, disk, BTN, hl, M.nphi, M.dphi, M.interp);
      }
      count += lit;
    }
    for (int o = 16; o; o >>= 1) count += __shfl_xor_sync(0xffffffffu, count, o);
    if (lane == 0) {
      double dv = (double)count / M.denom;
      double mu = sun_mu(Sv, p, BTN.n);
      dv *= (mu > 0.0 ? mu : 0.0);
      dv *= S->flux;
      store_direct(v, M, f, dv, dropin);
    }
  }
}

}  // namespace

// Host-side SunAux for one sun position. scene_mag bounds |p| over the
// facets (max coordinate magnitude), disk_rmax the samples' radius.
SunAux make_sun_aux(const double* s, double solar_const, double scene_mag, double disk_rmax) {
  SunAux a;
  a.sx = s[0]; a.sy = s[1]; a.sz = s[2];
  double d = norm(mkd(s[0], s[1], s[2]));
  double scale_au = ONE_AU_KM / d;
  a.flux = solar_const * (scale_au * scale_au);
  a.ux = (float)(s[0] / d); a.uy = (float)(s[1] / d); a.uz = (float)(s[2] / d);
  double pmax = 1.7320508 * scene_mag;
  double dmin = d - pmax;
  if (dmin <= 0.0) {              // sun inside the scene bounds: nothing is decided in pass 1
    a.alpha = 10.0f;
    a.mu_eps = 10.0f;
    a.ang_eps = 10.0f;
  } else {
    a.alpha = (float)(SUN_RADIUS_KM * disk_rmax / dmin * (1.0 + 1e-6) + 1e-9);
    a.mu_eps = (float)(4e-6 + 2.0 * pmax / dmin);
    a.ang_eps = (float)(1e-6 + 2.0 * pmax / dmin);
  }
  return a;
}

// Direct insolation for every active mesh of the view (dropin: E = direct
// only). counters[0] is cleared first.
int direct_launch(const StepView& v, int dropin, cudaStream_t s) {
  ILG_CUDA(cudaMemsetAsync(v.counters, 0, sizeof(int), s));
  k_direct_classify<<<div_up(v.nt, 256), 256, 0, s>>>(v, dropin);
  ILG_CUDA(cudaGetLastError());
  k_direct_exact<<<152 * 4, 256, 0, s>>>(v, dropin);
  ILG_CUDA(cudaGetLastError());
  return ILG_OK;
}

}  // namespace ilg
