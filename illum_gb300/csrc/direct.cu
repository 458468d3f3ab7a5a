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

// The sun of frame M.frame + ahead: from the mesh's table, or from the
// host slot of that frame's parity (host-driven steps keep two).
__device__ __forceinline__ const SunAux* mesh_sun(const StepView& v, const MeshDesc& M, int ahead) {
  return v.suns + (M.host_sun ? M.host_slot + ((M.frame + ahead) & 1) : M.sun0 + M.sun_idx + ahead);
}

// Meshes whose flux this pass computes: active, with a sun for the frame.
__device__ __forceinline__ bool direct_on(const MeshDesc& M, int ahead) {
  return M.active && (M.host_sun || M.sun_idx + ahead < M.nsun);
}

// A facet's direct flux goes into the E slot of its frame (the radiosity
// solve, or the conduction of a mesh without form factors, reads it and
// adds the coupling), or into E alone for a drop-in call.
__device__ __forceinline__ void store_direct(const StepView& v, const MeshDesc& M, int g, double dv, int dropin,
                                             int ahead) {
  if (dropin) { v.E[g] = dv; return; }
  v.E[e_slot(M.frame + ahead) * v.nt + g] = dv;
}

// Range of the horizon threshold of src/cpp/illum.cpp:431-434 over the
// azimuth interval [a, b] (0 <= a <= b <= 2 pi), bins of width dphi.
__device__ __forceinline__ bool thr_range(const float* __restrict__ h, int nphi, float dphi, int interp, float a,
                                          float b, float& tmin, float& tmax) {
  int k0 = (int)floorf(a / dphi), k1 = (int)floorf(b / dphi);
  k0 = max(0, min(k0, nphi - 1));
  k1 = max(0, min(k1, nphi - 1));
  if (k1 - k0 > 6) return false;
  for (int k = k0; k <= k1; ++k) {
    float lo = fmaxf(a, (float)k * dphi), hi = fminf(b, (float)(k + 1) * dphi);
    if (hi < lo) hi = lo;
    float hk = h[k];
    float v0, v1;
    if (interp == 0) {
      v0 = hk + (lo - (float)k * dphi);
      v1 = hk + (hi - (float)k * dphi);
    } else {
      float hk1 = h[k + 1 < nphi ? k + 1 : nphi - 1];
      v0 = hk + (lo - (float)k * dphi) / dphi * (hk1 - hk);
      v1 = hk + (hi - (float)k * dphi) / dphi * (hk1 - hk);
    }
    tmin = fminf(tmin, fminf(v0, v1));
    tmax = fmaxf(tmax, fmaxf(v0, v1));
  }
  return true;
}

// mu32: the cosine of the sun centre in FP32 (n . u, u the unit sun vector;
// relative error ~2e-7) instead of the reference's FP64 value; the lit
// sample count stays exact either way.
__global__ void k_direct_classify(StepView v, int dropin, int mu32_flux, int ahead) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  bool amb = false;
  const MeshDesc* Mp = nullptr;
  if (f < v.nt) {
    Mp = &v.md[v.mesh_of ? v.mesh_of[f] : 0];
    if (!direct_on(*Mp, ahead)) Mp = nullptr;
  }
  if (Mp) {
    const MeshDesc& M = *Mp;
    const SunAux* S = mesh_sun(v, M, ahead);
    float4 n4 = v.nrm[f];
    float mu32 = (n4.x * S->ux + n4.y * S->uy) + n4.z * S->uz;
    float eps = S->mu_eps;
    int decided = 0;                 // 1 dark, 2 lit
    if (mu32 < -eps) {
      decided = 1;                   // facing away: max(0, mu) = 0
    } else {
      const float MARG = 1e-6f, CEPS = 1e-6f;
      const float2 hmm = v.hmm32[f];
      float alo = hmm.x - S->alpha - MARG;
      float ahi = hmm.y + M.dphi32 + S->alpha + MARG;
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
            float dphi = M.dphi32;
            const float* h = v.H32 + M.H0 + (size_t)(f - M.facet0) * M.nphi;
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
      if (decided == 2 && mu32_flux) {
        dv = M.lit_all * S->flux * (double)fmaxf(mu32, 0.f);
      } else if (decided == 2) {
        float4 c4 = v.cen[f];
        d3 p = mkd((double)c4.x, (double)c4.y, (double)c4.z);
        const double* fr = v.frame + 9 * (int64_t)f;
        double mu = sun_mu(mkd(S->sx, S->sy, S->sz), p, mkd(fr[6], fr[7], fr[8]));
        dv = M.lit_all;   // (double)nsamp / denom
        dv *= (mu > 0.0 ? mu : 0.0);
        dv *= S->flux;
      }
      store_direct(v, M, f, dv, dropin, ahead);
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

// Pass 2: blocks of NF undecided facets (4..32, chosen by ilg_autotune; few
// per block spread the FP64 work over many SMs). The GPU's FP64 pipe is slow
// per instruction, so FP64 runs one lane per facet or per ambiguous
// sample, and the FP64 set-up overlaps the FP32 filter:
//   warp 0, one lane per facet: the sun frame (T, B) of geom.h sun_frame and
//     the cosine mu in FP64 (the values the exact test and the flux need);
//   warps 1.., concurrently: an FP32 set-up per facet (direction N, frame,
//     kappa), then one thread per (facet, sample): the sample is classified
//     in FP32 (direction N + kappa (x T + y B) in the facet frame, atan2f);
//     lit samples count, samples within MT of the threshold or MP of a bin
//     edge (or with the sun near the zenith) are listed;
//   all threads: the listed samples with the exact FP64 sample_lit,
//     bit-identical to the CPU oracle;
//   warp 0: count / denom * mu * flux as the reference.
// The FP32 set-up differs from the rounded FP64 one by ~1e-7 rad (p is
// negligible next to |S|), far below MT and MP, which dominate the FP32
// errors; a facet whose sun-frame axis choice is within rounding of a tie
// lists all its samples. Counts are integer sums, so the result does not
// depend on the order.
constexpr int DX_THREADS = 512;
constexpr int DX_LIST = 4096;   // (facet, sample) pairs per round of the filter

struct DxFacet {
  double Tx, Ty, Tz, Bx, By, Bz;   // sun frame (FP64, for sample_lit)
  double mu;                       // cosine of the sun centre (FP64, or FP32 with mu32_flux)
  float4 fb, ft, fn;               // facet frame (FP32)
  float Nx, Ny, Nz, Tfx, Tfy, Tfz, Bfx, Bfy, Bfz, kap;
  int f, mesh, all_amb, count;
};

__device__ __forceinline__ int dx_classify(const StepView& v, const MeshDesc& M, const DxFacet& F, int s) {
  const float MT = 2e-5f, MP = 2e-5f;
  if (F.all_amb) return -1;
  const float dphi = M.dphi32;
  float xf = F.kap * v.disk32[s], yf = F.kap * v.disk32[v.ndisk + s];
  float vx = F.Nx + (xf * F.Tfx + yf * F.Bfx), vy = F.Ny + (xf * F.Tfy + yf * F.Bfy),
        vz = F.Nz + (xf * F.Tfz + yf * F.Bfz);
  float lx = (F.fb.x * vx + F.fb.y * vy) + F.fb.z * vz;
  float ly = (F.ft.x * vx + F.ft.y * vy) + F.ft.z * vz;
  float lz = (F.fn.x * vx + F.fn.y * vy) + F.fn.z * vz;
  float th = atan2f(sqrtf(lx * lx + ly * ly), lz);
  if (th > 0.05f) {
    float ph = atan2f(ly, lx);
    if (ph < 0.f) ph += 6.2831853f;
    int k = (int)floorf(ph / dphi);
    float edge = fminf(ph - (float)k * dphi, (float)(k + 1) * dphi - ph);
    if (k >= 0 && k < M.nphi - 1 && edge > MP) {
      const float* h = v.H32 + M.H0 + (int64_t)(F.f - M.facet0) * M.nphi;
      float hk = h[k];
      float thr = M.interp == 0 ? hk + (ph - (float)k * dphi)
                                : hk + (ph - (float)k * dphi) / dphi * (h[k + 1] - hk);
      float dlt = th - thr;
      if (dlt < -MT) return 1;
      if (dlt > MT) return 0;
    }
  }
  return -1;
}

// FP32 sun direction, frame and kappa of one facet; all_amb when the axis
// choice of sun_frame is within rounding of a tie.
__device__ __forceinline__ void dx_setup32(const StepView& v, DxFacet& F, int f, int ahead) {
  const MeshDesc& M = v.md[v.mesh_of ? v.mesh_of[f] : 0];
  const SunAux* S = mesh_sun(v, M, ahead);
  float4 c4 = v.cen[f];
  float sx = (float)S->sx - c4.x, sy = (float)S->sy - c4.y, sz = (float)S->sz - c4.z;
  float dist = sqrtf(sx * sx + sy * sy + sz * sz);
  float nx = sx / dist, ny = sy / dist, nz = sz / dist;
  float ax = fabsf(nx), ay = fabsf(ny), az = fabsf(nz);
  const float TIE = 1e-5f;
  F.all_amb = (fabsf(ax - ay) < TIE || fabsf(ax - az) < TIE || fabsf(ay - az) < TIE) ? 1 : 0;
  float ex = 0.f, ey = 0.f, ez = 0.f;
  if (ax <= ay && ax <= az) ex = 1.f;
  else if (ay <= az) ey = 1.f;
  else ez = 1.f;
  float ne = nx * ex + ny * ey + nz * ez;
  float tx = ex - nx * ne, ty = ey - ny * ne, tz = ez - nz * ne;
  float tl = sqrtf(tx * tx + ty * ty + tz * tz);
  tx /= tl; ty /= tl; tz /= tl;
  F.Nx = nx; F.Ny = ny; F.Nz = nz;
  F.Tfx = tx; F.Tfy = ty; F.Tfz = tz;
  F.Bfx = ty * nz - tz * ny; F.Bfy = tz * nx - tx * nz; F.Bfz = tx * ny - ty * nx;   // T x N
  F.kap = (float)SUN_RADIUS_KM / dist;
  const float4* F4 = v.frame32 + 3 * (size_t)f;
  F.fb = F4[0]; F.ft = F4[1]; F.fn = F4[2];
  F.f = f;
  F.mesh = v.mesh_of ? v.mesh_of[f] : 0;
  F.count = 0;
}

__device__ __forceinline__ void dx_exact_sample(const StepView& v, DxFacet& F, int s, int ahead) {
  const MeshDesc& M = v.md[F.mesh];
  const SunAux* S = mesh_sun(v, M, ahead);
  d3 Sv = mkd(S->sx, S->sy, S->sz);
  float4 c4 = v.cen[F.f];
  d3 p = mkd((double)c4.x, (double)c4.y, (double)c4.z);
  d3 T = mkd(F.Tx, F.Ty, F.Tz), B = mkd(F.Bx, F.By, F.Bz);
  double x = v.disk[s], y = v.disk[v.ndisk + s];
  d3 disk = add(Sv, scl(add(scl(T, x), scl(B, y)), SUN_RADIUS_KM));
  frame3 BTN = load_frame(v.frame + 9 * (int64_t)F.f);
  const double* h = v.H + M.H0 + (int64_t)(F.f - M.facet0) * M.nphi;
  auto hl = [&](int k) { return h[k]; };
  if (sample_lit(p, disk, BTN, hl, M.nphi, M.dphi, M.interp)) atomicAdd(&F.count, 1);
}

template <int NF>
__global__ void __launch_bounds__(DX_THREADS) k_direct_exact(StepView v, int dropin, int mu32_flux, int ahead) {
  __shared__ DxFacet fs[NF];
  __shared__ int list[DX_LIST];
  __shared__ int nlist;
  const int nw = v.counters[0];
  const int nsamp = v.ndisk - 1;   // samples per facet (the meshes of a view share the disk)
  const int FT = DX_THREADS - 32;  // filter threads (warps 1..)
  for (int base = blockIdx.x * NF; base < nw; base += gridDim.x * NF) {
    const int nf = min(NF, nw - base);
    const int total = nf * nsamp;
    if (threadIdx.x < 32) {
      // FP64 set-up, one lane per facet (overlaps the filter below)
      if (threadIdx.x < nf) {
        DxFacet& F = fs[threadIdx.x];
        int f = v.work[base + threadIdx.x];
        const MeshDesc& M = v.md[v.mesh_of ? v.mesh_of[f] : 0];
        const SunAux* S = mesh_sun(v, M, ahead);
        float4 c4 = v.cen[f];
        d3 p = mkd((double)c4.x, (double)c4.y, (double)c4.z);
        d3 Sv = mkd(S->sx, S->sy, S->sz);
        d3 SP = sub(Sv, p);
        double dist = norm(SP);
        d3 N = mkd(SP.x / dist, SP.y / dist, SP.z / dist);   // = geom.h normalise(S - p)
        d3 T, B;
        sun_frame(N, &T, &B);
        F.Tx = T.x; F.Ty = T.y; F.Tz = T.z;
        F.Bx = B.x; F.By = B.y; F.Bz = B.z;
        if (mu32_flux) {
          float4 n4 = v.nrm[f];
          F.mu = (double)((n4.x * S->ux + n4.y * S->uy) + n4.z * S->uz);
        } else {
          const double* fr = v.frame + 9 * (int64_t)f;
          F.mu = sun_mu(Sv, p, mkd(fr[6], fr[7], fr[8]));
        }
      }
    } else {
      if (threadIdx.x - 32 < nf) dx_setup32(v, fs[threadIdx.x - 32], v.work[base + threadIdx.x - 32], ahead);
      if (threadIdx.x == 32) nlist = 0;
      asm volatile("bar.sync 1, %0;" ::"r"(FT));   // the filter warps only
      const int q1 = min(total, DX_LIST);
      for (int q = threadIdx.x - 32; q < q1; q += FT) {
        const int j = q / nsamp, s = q - j * nsamp;
        int lit = dx_classify(v, v.md[fs[j].mesh], fs[j], s);
        if (lit == 1) atomicAdd(&fs[j].count, 1);
        if (lit < 0) list[atomicAdd(&nlist, 1)] = q;
      }
    }
    __syncthreads();
    for (int q0 = 0;;) {
      const int nl = nlist;
      for (int a = threadIdx.x; a < nl; a += DX_THREADS) {
        const int q = list[a];
        const int j = q / nsamp;
        dx_exact_sample(v, fs[j], q - j * nsamp, ahead);
      }
      q0 += DX_LIST;
      if (q0 >= total) break;
      // more pairs than one round holds (more than DX_LIST / DX_FACETS samples per facet)
      __syncthreads();
      if (threadIdx.x == 0) nlist = 0;
      __syncthreads();
      const int q1 = min(total, q0 + DX_LIST);
      for (int q = q0 + threadIdx.x; q < q1; q += DX_THREADS) {
        const int j = q / nsamp, s = q - j * nsamp;
        int lit = dx_classify(v, v.md[fs[j].mesh], fs[j], s);
        if (lit == 1) atomicAdd(&fs[j].count, 1);
        if (lit < 0) list[atomicAdd(&nlist, 1) ] = q;
      }
      __syncthreads();
    }
    __syncthreads();
    // the facet's flux, one thread per facet
    if (threadIdx.x < nf) {
      const DxFacet& F = fs[threadIdx.x];
      const MeshDesc& M = v.md[F.mesh];
      const SunAux* S = mesh_sun(v, M, ahead);
      double dv = (double)F.count / M.denom;
      double mu = F.mu;
      dv *= (mu > 0.0 ? mu : 0.0);
      dv *= S->flux;
      store_direct(v, M, F.f, dv, dropin, ahead);
    }
    __syncthreads();
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

// Direct insolation for every active mesh of the view that has a sun for
// frame M.frame + ahead (dropin: E = direct only; mu32_flux: FP32 sun
// cosine in the flux). counters[0] is cleared first.
int direct_launch(const StepView& v, int dropin, int mu32_flux, int ahead, cudaStream_t s) {
  ILG_CUDA(cudaMemsetAsync(v.counters, 0, sizeof(int), s));
  const int cb = v.tune.classify_threads;
  if (cb != 128 && cb != 256 && cb != 512) { set_error("classify_threads must be 128, 256 or 512"); return ILG_ERR_ARG; }
  k_direct_classify<<<div_up(v.nt, cb), cb, 0, s>>>(v, dropin, mu32_flux, ahead);
  ILG_CUDA(cudaGetLastError());
  switch (v.tune.exact_facets) {
    case 4: k_direct_exact<4><<<152 * 4, DX_THREADS, 0, s>>>(v, dropin, mu32_flux, ahead); break;
    case 8: k_direct_exact<8><<<152 * 4, DX_THREADS, 0, s>>>(v, dropin, mu32_flux, ahead); break;
    case 16: k_direct_exact<16><<<152 * 4, DX_THREADS, 0, s>>>(v, dropin, mu32_flux, ahead); break;
    case 32: k_direct_exact<32><<<152 * 4, DX_THREADS, 0, s>>>(v, dropin, mu32_flux, ahead); break;
    default: set_error("exact_facets must be 4, 8, 16 or 32"); return ILG_ERR_ARG;
  }
  ILG_CUDA(cudaGetLastError());
  return ILG_OK;
}

}  // namespace ilg
