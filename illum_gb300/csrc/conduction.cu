// conduction.cu — batched Crank-Nicolson conduction, one thread per facet
// column: conductionQ.f (src/cpp/conductionQ.f:1-99) as driven by
// thermal_model::step (src/cpp/thermal.hpp:65-83), plus conductionT.f
// (src/cpp/conductionT.f:1-71) for the ABI.
//
// The reference rebuilds every coefficient and runs a full Thomas solve per
// facet per step. Here the depth profile (z, ti, rho*c) is shared by all
// facets of a mesh, so rows 2..nz of the tridiagonal matrix are the same for
// every column: their bottom-up elimination factors (1/beta_i and
// c_i/beta_{i+1}) are computed once per (mesh, dt) on the host. Per column
// and step only the right-hand side changes:
//   upward pass:   rho_i = r_i - (c_i/beta_{i+1}) rho_{i+1}   (i = nz..2)
//   top row:       the surface boundary, linearised as in conductionQ.f:76-82
//                  or solved by Newton's method for emiss*sigma*Ts^4
//                  (T1 is affine in Ts once rows 2..nz are eliminated, so the
//                  Newton iteration is scalar)
//   downward pass: T_i = (rho_i + gamma_i T_{i-1}) / beta_i
// rho is staged in shared memory ([layer][thread], conflict-free). The
// temperature state is layer-major [nz][N], so every layer access of a warp
// is one coalesced 256-byte (8-byte values) or 128-byte (fp32) transaction.
//
// Arithmetic: GB300 executes FP64 at about one fused multiply-add per clock
// per SM, so the FP64 step of a scene keeps its layers as double-float
// pairs (hi + lo floats, 48 significant bits) and runs the layer recurrences
// in double-float arithmetic on the FP32 pipes (error-free products by FMA,
// TwoSum additions; Dekker 1971). It solves for the increment
// dT = T(n+1) - T(n), whose right-hand side 2 gamma (T(i-1) - T(i)) +
// 2 alpha (T(i+1) - T(i)) carries no large cancellation when the diffusion
// numbers are large, so rounding stays relative to the increment and the
// stored state is within ~1e-12 K of FP64 per step. The surface boundary
// (linearised or Newton) is solved in FP64. The mixed step uses the same
// increment form in plain FP32; the standalone column entry points
// (conductionq_, ilg_conductionq_batch) run the reference's rows in FP64.
#include <atomic>
#include <cmath>
#include <mutex>
#include <type_traits>
#include <vector>

#include "geom.h"
#include "internal.cuh"

namespace ilg {

namespace {

constexpr int COND_THREADS = 128;       // standalone column entry points
constexpr int COND_STEP_THREADS = 64;   // scene steps: 7 blocks of 60-layer columns per SM
constexpr int TAB_W = 5;            // g, m, al, f, inv_beta per layer
constexpr size_t SMEM_LIMIT = 160 * 1024;

// Double-float number: value = h + l with |l| <= ulp(h) / 2. The
// intrinsics keep the compiler from contracting or reassociating the
// error-free steps.
struct dfloat {
  float h, l;
  __host__ __device__ __forceinline__ dfloat() {}
  __device__ __forceinline__ dfloat(float a, float b) : h(a), l(b) {}
  __device__ __forceinline__ explicit dfloat(double x) {
    h = __double2float_rn(x);
    l = __double2float_rn(x - (double)h);
  }
  __device__ __forceinline__ explicit dfloat(int x) : h((float)x), l(0.f) {}
  __device__ __forceinline__ explicit operator double() const { return (double)h + (double)l; }
};
// s + e renormalised, |s| >= |e| (Fast2Sum)
__device__ __forceinline__ dfloat df_norm(float s, float e) {
  float t = __fadd_rn(s, e);
  return dfloat(t, __fsub_rn(e, __fsub_rn(t, s)));
}
__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
  float s = __fadd_rn(a.h, b.h);
  float bb = __fsub_rn(s, a.h);
  float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));   // TwoSum error
  return df_norm(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat(-a.h, -a.l); }
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }
__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
  float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);   // exact error of the product
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return df_norm(p, e);
}

// 2x, exact
__device__ __forceinline__ double twice(double a) { return 2.0 * a; }
__device__ __forceinline__ float twice(float a) { return 2.f * a; }
__device__ __forceinline__ dfloat twice(dfloat a) { return dfloat(2.f * a.h, 2.f * a.l); }

// Layer loads bypass L1 (each value is read once per pass), so the small
// per-layer coefficient table, read by every thread at every layer, stays
// L1-resident next to the shared-memory rho arrays.
__device__ __forceinline__ double ld_layer(const double* p) { return __ldcg(p); }
__device__ __forceinline__ float ld_layer(const float* p) { return __ldcg(p); }
__device__ __forceinline__ dfloat ld_layer(const dfloat* p) {
  float2 t = __ldcg(reinterpret_cast<const float2*>(p));
  return dfloat(t.x, t.y);
}

template <class R> R* rho_scratch_host(const StepView& v);
template <> double* rho_scratch_host<double>(const StepView& v) { return v.rho64; }
template <> float* rho_scratch_host<float>(const StepView& v) { return v.rho32; }
template <> dfloat* rho_scratch_host<dfloat>(const StepView&) { return nullptr; }

template <class R> __device__ __forceinline__ R* state_T(const StepView& v);
template <> __device__ __forceinline__ double* state_T<double>(const StepView& v) { return v.T64; }
template <> __device__ __forceinline__ float* state_T<float>(const StepView& v) { return v.T32; }
template <> __device__ __forceinline__ dfloat* state_T<dfloat>(const StepView& v) {
  return reinterpret_cast<dfloat*>(v.Tdf);
}
template <class R> __device__ __forceinline__ const R* coef_tab(const StepView& v);
template <> __device__ __forceinline__ const double* coef_tab<double>(const StepView& v) { return v.coef64; }
template <> __device__ __forceinline__ const float* coef_tab<float>(const StepView& v) { return v.coef32; }
template <> __device__ __forceinline__ const dfloat* coef_tab<dfloat>(const StepView& v) {
  return reinterpret_cast<const dfloat*>(v.coefdf);
}
template <class R> __device__ __forceinline__ R* rho_scratch(const StepView& v);
template <> __device__ __forceinline__ double* rho_scratch<double>(const StepView& v) { return v.rho64; }
template <> __device__ __forceinline__ float* rho_scratch<float>(const StepView& v) { return v.rho32; }
template <> __device__ __forceinline__ dfloat* rho_scratch<dfloat>(const StepView&) { return nullptr; }

// Surface boundary of the FP32 and double-float steps: Newton's method for
// emiss sigma Ts^4 in double-float arithmetic (FP32 iterations, then, for
// the FP64 step, two double-float polishing steps), so no FP64 arithmetic
// is on the Newton path.
__device__ __forceinline__ dfloat to_df(float x) { return dfloat(x, 0.f); }
__device__ __forceinline__ dfloat to_df(dfloat x) { return x; }
__device__ __forceinline__ dfloat to_df(float2 x) { return dfloat(x.x, x.y); }
template <class R> __device__ __forceinline__ R from_df(dfloat x);
template <> __device__ __forceinline__ float from_df<float>(dfloat x) { return __fadd_rn(x.h, x.l); }
template <> __device__ __forceinline__ dfloat from_df<dfloat>(dfloat x) { return x; }
__device__ __forceinline__ double df_to_double(dfloat x) { return (double)x.h + (double)x.l; }

// Newton surface boundary in double-float. T0, T1: the top two layers at
// time n; rho1: the eliminated right-hand side of layer 1; Ts: the surface
// temperature at n; Q: the absorbed flux at n+1. Solves
// g(x) = A + B x - es x^4 = 0 with A = Q + 2 k1 (T0 + P), the top layer's
// increment being P + S_top x. polish: double-float Newton steps after the
// FP32 ones (the FP64 step's accuracy).
struct TopResult { dfloat dtop, top, tsn; };
__device__ __forceinline__ TopResult newton_top(const CondScalars& cs, dfloat T0, dfloat T1, dfloat rho1, dfloat Tsd,
                                                dfloat Qd, bool polish) {
  const dfloat al0 = to_df(cs.d_al0), g0 = to_df(cs.d_g0), f0 = to_df(cs.d_f0), iAp = to_df(cs.d_inv_Ap);
  const dfloat two(2.f, 0.f), four(4.f, 0.f);
  // R0 = 2 al0 (T1 - T0) + 4 g0 (Ts - T0) - 2 g0 Ts; P = (R0 - f0 rho1) / Ap
  const dfloat R0 = two * al0 * (T1 - T0) + four * g0 * (Tsd - T0) - two * g0 * Tsd;
  const dfloat P = (R0 - f0 * rho1) * iAp;
  const dfloat A = Qd + to_df(cs.d_2k1) * (T0 + P);
  const float Af = __fadd_rn(A.h, A.l), Bf = cs.B_topf, esf = cs.esf;
  const float tol = polish ? 1e-6f : 2.4e-7f;
  float xf = __fadd_rn(Tsd.h, Tsd.l);
  // from the previous surface temperature Newton converges in a few steps;
  // it stops at the tolerance or once a step no longer shrinks (the FP32
  // rounding floor of g)
  float prev = INFINITY;
  for (int it = 0; it < 20; ++it) {
    const float x3 = xf * xf * xf;
    const float dT = __fmul_rn(Af + Bf * xf - esf * x3 * xf, __frcp_rn(Bf - 4.f * esf * x3));
    xf -= dT;
    const float adt = fabsf(dT);
    if (adt <= tol * fabsf(xf) || adt >= prev) break;
    prev = adt;
  }
  dfloat x(xf, 0.f);
  if (polish) {
    const dfloat B = to_df(cs.d_B_top), es = to_df(cs.d_es);
    for (int it = 0; it < 2; ++it) {
      const dfloat x2 = x * x;
      const dfloat gx = A + B * x - es * (x2 * x2);
      const float x3 = x.h * x.h * x.h;
      const float step = __fmul_rn(__fadd_rn(gx.h, gx.l), __frcp_rn(Bf - 4.f * esf * x3));
      x = x - dfloat(step, 0.f);
    }
  }
  TopResult r;
  r.dtop = P + to_df(cs.d_S_top) * x;
  r.top = T0 + r.dtop;
  r.tsn = x;
  return r;
}

// Unbiased rounding of an FP32 layer update a + b: the exact sum is
// s + e (TwoSum, s = fl(a + b)); s moves one ulp toward e with probability
// |e| / ulp, so the expected stored value is a + b and increments smaller
// than half an ulp are not lost on average. The uniform draw is a hash of
// (facet within its mesh, layer, frame): reproducible, and the same alone
// and in a batch. The hash is the lowbias32 integer finaliser (C. Wellons,
// "Prospecting for hash functions", 2018).
__device__ __forceinline__ uint32_t sr_hash(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
__device__ __forceinline__ float sr_add(float a, float b, uint32_t key) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  if (e == 0.f || s == 0.f) return s;
  const float n = __int_as_float(__float_as_int(s) + (((e > 0.f) == (s > 0.f)) ? 1 : -1));
  const float u = (float)(sr_hash(key) >> 8) * 5.9604644775390625e-8f;   // [0, 1) in steps of 2^-24
  return fabsf(e) > u * fabsf(__fsub_rn(n, s)) ? n : s;
}

// One thread per facet column. Block b covers facets [cb.y, cb.y + BS) of
// mesh cb.x. Q: the new time level's flux per facet. SR: the FP32 layers'
// updates rounded without bias (sr_add).
template <class R, bool SMEM, int BS, bool SR = false>
__global__ void __launch_bounds__(BS)
k_conduct(StepView v, const double* __restrict__ Qnp1, int upd) {
  extern __shared__ unsigned char smem_raw[];
  R* rho_s = reinterpret_cast<R*>(smem_raw);
  int2 cb = v.cblocks ? v.cblocks[blockIdx.x] : make_int2(0, blockIdx.x * BS);
  const MeshDesc& M = v.md[cb.x];
  if (!M.active) return;
  int fl = cb.y + threadIdx.x;
  if (fl >= M.nfacet) return;
  const int g = M.facet0 + fl;
  const CondScalars cs = M.cs;
  const int nz = cs.nz;
  const size_t N = (size_t)M.nfacet;
  R* __restrict__ T = state_T<R>(v) + M.T0 + fl;
  const R* __restrict__ tab = coef_tab<R>(v) + M.coef0;
  R* __restrict__ rho_g = SMEM ? nullptr : rho_scratch<R>(v) + g;
#define RHO(i) (SMEM ? rho_s[(size_t)(i) * BS + threadIdx.x] : rho_g[(size_t)(i) * v.nt])
  // FP64 solves for T(n+1) directly (the reference's rows); FP32 and
  // double-float solve for the increment dT = T(n+1) - T(n), whose
  // right-hand side 2 gamma (T(i-1) - T(i)) + 2 alpha (T(i+1) - T(i))
  // carries no large cancellation when the diffusion numbers alpha, gamma
  // are large.
  constexpr bool INC = !std::is_same<R, double>::value;
  // The facet's scalars, loaded before the column work so that their
  // latency overlaps it. A scene step's flux: the radiosity solution, or for
  // a mesh without form factors the frame's direct flux, coupled as
  // src/cpp/illum_cli.cpp:415-421 (rad = -Fsurf_prev + direct) when the mesh
  // follows the reference, and recorded as the mesh's radiosity. Fsurf is
  // read before this thread overwrites it below.
  const bool direct_only = upd && M.ntiles == 0;
  const double Qsrc = direct_only ? v.E[e_slot(M.frame) * v.nt + g] : Qnp1[g];
  const double Fs_prev = (direct_only && M.coupling == ILG_COUPLE_REFERENCE) ? v.Fsurf[g] : 0.0;
  const double Ts_prev = v.Tsurf[g];
  // Stage the column in the rho slots (slot i <- T_i): the upward pass then
  // reads T from shared memory and overwrites slot i with rho_i once T_i is
  // in registers. In shared memory the copies are asynchronous (cp.async,
  // every layer in flight at once; each thread waits for its own copies).
  if (SMEM) {
    for (int i = 0; i < nz; ++i) {
      unsigned sa = (unsigned)__cvta_generic_to_shared(&rho_s[(size_t)i * BS + threadIdx.x]);
      const R* ga = T + (size_t)i * N;
      if (sizeof(R) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(ga) : "memory");
      else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(ga) : "memory");
    }
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
  } else {
    for (int i0 = 0; i0 < nz; i0 += 8) {
      R t[8];
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (i0 + j < nz) t[j] = ld_layer(T + (size_t)(i0 + j) * N);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (i0 + j < nz) RHO(i0 + j) = t[j];
    }
  }
  // upward pass
  R Tip1 = RHO(nz - 1);
  R Ti = RHO(nz - 2);
  const R* cb_t = tab + (size_t)(nz - 1) * TAB_W;
  R dn = Ti - Tip1;   // increment form: layer differences d_i = T(i-1) - T(i), each formed once
  R rho_next = INC ? twice(cb_t[0] * dn) + (R)cs.cgeo : cb_t[0] * Ti + cb_t[1] * Tip1 + (R)cs.cgeo;
  RHO(nz - 1) = rho_next;
#pragma unroll 4
  for (int i = nz - 2; i >= 1; --i) {
    R Tim1 = RHO(i - 1);
    const R* c = tab + (size_t)i * TAB_W;
    R r;
    if (INC) {
      R dm = Tim1 - Ti;
      r = twice(c[0] * dm - c[2] * dn);
      dn = dm;
    } else {
      r = c[0] * Tim1 + c[1] * Ti + c[2] * Tip1;
    }
    R rh = r - c[3] * rho_next;
    RHO(i) = rh;
    rho_next = rh;
    Tip1 = Ti;
    Ti = Tim1;
  }
  // top row (Ti = T_1, Tip1 = T_2 in the Fortran's numbering). In increment
  // form rho1 is the increment's; T1(n+1) = T0 + (increment) below.
  double Q = Qsrc;
  if (direct_only) {
    if (M.coupling == ILG_COUPLE_REFERENCE) Q = -Fs_prev + Qsrc;
    v.rad[g] = Q;
  }
  double T0n, Tsn, Fs;
  R top, dtop;   // T1(n+1) and its increment, in the state's type
  bool done_top = false;
  if constexpr (!std::is_same<R, double>::value) {
    if (cs.bc == 1) {
      // FP32 and double-float states: P, A and the top layer in double-float
      // (P = T1(n+1) - S_top Ts(n+1) is a small difference of
      // temperature-sized terms), the root by FP32 Newton steps, polished in
      // double-float for the FP64 step (no FP64 arithmetic)
      // the double-float step takes Ts and Q to 48 bits; the FP32 step in
      // FP32 (its layers are FP32), converting each once
      constexpr bool DF = std::is_same<R, dfloat>::value;
      const dfloat Tsd = DF ? dfloat(Ts_prev) : dfloat(__double2float_rn(Ts_prev), 0.f);
      const dfloat Qd = DF ? dfloat(Q) : dfloat(__double2float_rn(Q), 0.f);
      const TopResult tr = newton_top(cs, to_df(Ti), to_df(Tip1), to_df(rho_next), Tsd, Qd, DF);
      const dfloat fsd = (tr.top - tr.tsn) * to_df(cs.d_kz);
      Tsn = DF ? df_to_double(tr.tsn) : (double)__fadd_rn(tr.tsn.h, tr.tsn.l);
      top = from_df<R>(tr.top);
      dtop = from_df<R>(tr.dtop);
      Fs = DF ? -df_to_double(fsd) : -(double)__fadd_rn(fsd.h, fsd.l);
      T0n = 0.0;
      done_top = true;
    }
  }
  if (!done_top) {
  double T0 = (double)Ti, T1 = (double)Tip1, rho1 = (double)rho_next;
  double Ts = Ts_prev;
  if (cs.bc == 0) {
    double Qn = v.Qprev[g];
    double Tr3 = Ts * Ts * Ts;
    double arad = -3.0 * cs.es * Tr3 * Ts;
    double brad = 2.0 * cs.es * Tr3;
    double den = cs.k1 + brad;
    double ann = (Qn - arad) / den, annp1 = (Q - arad) / den, bn = (cs.k1 - brad) / den;
    double b0 = 1.0 + cs.alpha0 + cs.gamma0 - cs.gamma0 * bn;
    double r0 = cs.gamma0 * (annp1 + ann) + (1.0 - cs.alpha0 - cs.gamma0 + cs.gamma0 * bn) * T0 + cs.alpha0 * T1;
    double piv = b0 + cs.f0 * cs.gamma1;
    if (piv == 0.0) { atomicExch(&v.derr[DERR_PIVOT], 1); return; }
    if (INC) r0 -= b0 * T0 - cs.alpha0 * T1;   // the row applied to T(n)
    T0n = (r0 - cs.f0 * rho1) / piv;
    if (INC) T0n += T0;
    Tsn = 0.5 * (annp1 + bn * T0n + T0n);
  } else if (cs.bc == 1) {
    double R0 = (1.0 - cs.alpha0 - cs.gamma0) * T0 + cs.alpha0 * T1 + cs.gamma0 * (2.0 * Ts - T0);
    if (INC) R0 = 2.0 * cs.alpha0 * (T1 - T0) + 4.0 * cs.gamma0 * (Ts - T0) - 2.0 * cs.gamma0 * Ts;
    double P = (R0 - cs.f0 * rho1) * cs.inv_Ap;
    if (INC) P += T0;
    // Root of g(x) = Q + 2 k1 (P + (S - 1) x) - es x^4 = A + B x - es x^4
    // (g' = B - 4 es x^3 < 0): Newton in FP32 to ~1e-6, then FP64 steps
    // whose g is exact to FP64 and whose step uses an FP32 reciprocal of
    // g' (relative error ~6e-8, so each step gains ~7 digits). The FP32
    // stage leaves x within ~1e-7 of the root (its rounding floor), so one
    // FP64 step that moves x by at most 1e-7 |x| leaves ~6e-8 |dT| +
    // 2 |dT|^2 / |x| < 1e-11 K and ends the polish; a larger first step
    // (an FP32 stage that did not converge) continues to the FP64 tolerance.
    const double A = Q + 2.0 * cs.k1 * P;
    float xf = (float)Ts;
    {
      const float Af = (float)A, Bf = (float)cs.B_top, esf = (float)cs.es;
      for (int it = 0; it < 30; ++it) {
        float x3 = xf * xf * xf;
        float dT = (Af + Bf * xf - esf * x3 * xf) / (Bf - 4.f * esf * x3);
        xf -= dT;
        if (fabsf(dT) <= 1e-6f * fabsf(xf)) break;
      }
    }
    double x = (double)xf;
    double tolr = std::is_same<R, float>::value ? 1e-12 : 1e-13;
    for (int it = 0; it < 8; ++it) {
      double x3 = x * x * x;
      double gx = A + cs.B_top * x - cs.es * x3 * x;
      double dT = gx * (double)__frcp_rn((float)(cs.B_top - 4.0 * cs.es * x3));
      x -= dT;
      if (fabs(dT) <= (it == 0 ? 1e-7 : tolr) * fabs(x)) break;
    }
    Tsn = x;
    T0n = P + cs.S_top * Tsn;
  } else {
    // prescribed surface temperature: Ts at n, Q holds Ts at n+1
    double b0 = 1.0 + cs.alpha0 + cs.gamma0;
    double r0 = cs.alpha0 * T1 + (1.0 - cs.alpha0 - cs.gamma0) * T0 + cs.gamma0 * (Ts + Q);
    if (INC) r0 -= b0 * T0 - cs.alpha0 * T1;
    T0n = (r0 - cs.f0 * rho1) / (b0 + cs.f0 * cs.gamma1);
    if (INC) T0n += T0;
    Tsn = Q;
  }
  Fs = -(T0n - Tsn) * cs.kz;
  top = (R)T0n;
  dtop = (R)(T0n - T0);
  }
  // downward pass
  if (INC) {
    R dprev = dtop;
    T[0] = top;
#pragma unroll 4
    for (int i = 1; i < nz; ++i) {   // the increments, into the rho slots
      const R* c = tab + (size_t)i * TAB_W;
      R d = (RHO(i) + c[0] * dprev) * c[4];
      RHO(i) = d;
      dprev = d;
    }
    for (int i0 = 1; i0 < nz; i0 += 16) {   // T(n+1) = T(n) + dT, sixteen layers in flight
      R t[16];
#pragma unroll
      for (int j = 0; j < 16; ++j)
        if (i0 + j < nz) t[j] = ld_layer(T + (size_t)(i0 + j) * N);
#pragma unroll
      for (int j = 0; j < 16; ++j)
        if (i0 + j < nz) {
          if constexpr (SR && std::is_same<R, float>::value)
            T[(size_t)(i0 + j) * N] = sr_add(t[j], RHO(i0 + j),
                                             (uint32_t)fl * 0x9E3779B9u + (uint32_t)(i0 + j) * 0x85EBCA6Bu +
                                                 (uint32_t)M.frame * 0xC2B2AE35u);
          else
            T[(size_t)(i0 + j) * N] = t[j] + RHO(i0 + j);
        }
    }
  } else {
    R prev = top;
    T[0] = prev;
    for (int i = 1; i < nz; ++i) {
      const R* c = tab + (size_t)i * TAB_W;
      R t = (RHO(i) + c[0] * prev) * c[4];
      T[(size_t)i * N] = t;
      prev = t;
    }
  }
#undef RHO
  v.Fsurf[g] = Fs;
  if (cs.bc != 2) {
    v.Tsurf[g] = Tsn;
    v.Qprev[g] = Q;
  }
  if (upd) {
    // running means: 1/(frame + 1) by an FP32 reciprocal and two FP64
    // Newton steps (no FP64 division; computing it here is cheaper than
    // loading a per-mesh value at the end of the column)
    const double n = (double)(M.frame + 1);
    double rn = (double)__frcp_rn((float)n);
    rn = rn * (2.0 - n * rn);
    rn = rn * (2.0 - n * rn);
    v.rad_avg[g] += (Q - v.rad_avg[g]) * rn;
    v.therm_avg[g] += (Tsn - v.therm_avg[g]) * rn;
    if (M.frame > 50) v.therm_max[g] = fmax(v.therm_max[g], Tsn);
  }
}

__global__ void k_df_to_f(const float2* __restrict__ in, float* __restrict__ out, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)((double)in[i].x + (double)in[i].y);
}
__global__ void k_f_to_df(const float* __restrict__ in, float2* __restrict__ out, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_float2(in[i], 0.f);
}

// Coefficients of conductionQ.f:50-73 / conductionT.f:28-45 and the shared
// elimination factors. tab: nz x TAB_W.
int build_tables(int nz, const double* z, const double* ti, const double* rhoc, double dt, double emiss, double Fgeo,
                 int bc, std::vector<double>& tab, CondScalars& cs) {
  if (nz < 2) { set_error("conduction needs nz >= 2 (got %d)", nz); return ILG_ERR_ARG; }
  std::vector<double> k(nz), alpha(nz, 0.0), gamma(nz, 0.0), a(nz), b(nz), c(nz), beta(nz, 0.0);
  for (int i = 0; i < nz; ++i) {
    if (!(rhoc[i] > 0.0)) { set_error("rhoc[%d] must be > 0", i); return ILG_ERR_ARG; }
    k[i] = ti[i] * ti[i] / rhoc[i];
  }
  for (int i = 1; i < nz; ++i)
    if (!(z[i] > z[i - 1])) { set_error("depths must increase (z[%d] <= z[%d])", i, i - 1); return ILG_ERR_ARG; }
  if (!(z[0] > 0.0)) { set_error("z[0] must be > 0"); return ILG_ERR_ARG; }
  double dz = 2.0 * z[0];
  if (bc == 2) {
    alpha[0] = k[1] * dt / rhoc[0] / (z[1] - z[0]) / z[1];
    gamma[0] = k[0] * dt / rhoc[0] / z[0] / z[1];
  } else {
    double bt = dt / rhoc[0] / (2.0 * dz * dz);
    alpha[0] = bt * k[1];
    gamma[0] = bt * k[0];
  }
  for (int i = 1; i < nz - 1; ++i) {
    double buf = dt / (z[i + 1] - z[i - 1]);
    alpha[i] = 2.0 * k[i + 1] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i]);
    gamma[i] = 2.0 * k[i] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1]);
  }
  double buf = dt / ((z[nz - 1] - z[nz - 2]) * (z[nz - 1] - z[nz - 2]));
  gamma[nz - 1] = k[nz - 1] * buf / (2.0 * rhoc[nz - 1]);
  for (int i = 0; i < nz; ++i) {
    a[i] = -gamma[i];
    b[i] = 1.0 + alpha[i] + gamma[i];
    c[i] = -alpha[i];
  }
  b[nz - 1] = 1.0 + gamma[nz - 1];
  beta[nz - 1] = b[nz - 1];
  for (int i = nz - 2; i >= 1; --i) {
    if (beta[i + 1] == 0.0) { set_error("zero pivot in the conduction matrix"); return ILG_ERR_PIVOT; }
    beta[i] = b[i] - c[i] * a[i + 1] / beta[i + 1];
  }
  if (beta[1] == 0.0) { set_error("zero pivot in the conduction matrix"); return ILG_ERR_PIVOT; }
  tab.assign((size_t)nz * TAB_W, 0.0);
  for (int i = 0; i < nz; ++i) {
    double* t = &tab[(size_t)i * TAB_W];
    t[0] = gamma[i];
    t[1] = (i == nz - 1) ? 1.0 - gamma[i] : 1.0 - alpha[i] - gamma[i];
    t[2] = alpha[i];
    t[3] = (i <= nz - 2) ? c[i] / beta[i + 1] : 0.0;
    t[4] = (i >= 1) ? 1.0 / beta[i] : 0.0;
  }
  cs.alpha0 = alpha[0];
  cs.gamma0 = gamma[0];
  cs.k1 = k[0] / dz;
  cs.f0 = c[0] / beta[1];
  cs.gamma1 = gamma[1];
  cs.Ap = (1.0 + alpha[0] + 2.0 * gamma[0]) + cs.f0 * gamma[1];
  cs.k0 = k[0];
  cs.z0 = z[0];
  cs.inv_Ap = 1.0 / cs.Ap;
  cs.S_top = 2.0 * gamma[0] / cs.Ap;
  cs.B_top = 2.0 * cs.k1 * (cs.S_top - 1.0);
  cs.kz = k[0] / z[0];
  cs.cgeo = dt / rhoc[nz - 1] * Fgeo / (z[nz - 1] - z[nz - 2]);
  cs.es = emiss * SIGMA_SB;
  cs.esf = (float)cs.es;
  cs.B_topf = (float)cs.B_top;
  cs.d_al0 = split_df_host(cs.alpha0);
  cs.d_g0 = split_df_host(cs.gamma0);
  cs.d_f0 = split_df_host(cs.f0);
  cs.d_inv_Ap = split_df_host(cs.inv_Ap);
  cs.d_S_top = split_df_host(cs.S_top);
  cs.d_2k1 = split_df_host(2.0 * cs.k1);
  cs.d_B_top = split_df_host(cs.B_top);
  cs.d_es = split_df_host(cs.es);
  cs.d_kz = split_df_host(cs.kz);
  cs.nz = nz;
  cs.bc = bc;
  return ILG_OK;
}

template <class R, int BS>
int launch_conduct(const StepView& v, const double* Q, int upd, int nz_max, cudaStream_t s, bool sr = false) {
  size_t smem = (size_t)nz_max * BS * sizeof(R);
  int grid = v.cblocks ? v.ncblocks : div_up(v.nt, BS);
  if (grid <= 0) return ILG_OK;
  if constexpr (std::is_same<R, float>::value) {
    if (sr) {   // unbiased layer rounding (FP32 layers, shared-memory columns)
      if (smem > SMEM_LIMIT) { set_error("unbiased layer rounding: %d layers do not fit a column block", nz_max); return ILG_ERR_ARG; }
      k_conduct<R, true, BS, true><<<grid, BS, smem, s>>>(v, Q, upd);
      ILG_CUDA(cudaGetLastError());
      return ILG_OK;
    }
  }
  if (smem <= SMEM_LIMIT) {
    k_conduct<R, true, BS><<<grid, BS, smem, s>>>(v, Q, upd);
  } else {
    if (!rho_scratch_host<R>(v)) { set_error("conduction: %d layers need the deep-column scratch", nz_max); return ILG_ERR_ARG; }
    k_conduct<R, false, BS><<<grid, BS, 0, s>>>(v, Q, upd);
  }
  ILG_CUDA(cudaGetLastError());
  return ILG_OK;
}

}  // namespace

// Opt the shared-memory kernels into SMEM_LIMIT bytes (once per process,
// before any capture).
int conduction_step_threads() { return COND_STEP_THREADS; }

int conduction_setup() {
  static std::mutex mu;
  static std::atomic<bool> done{false};
  if (done.load(std::memory_order_acquire)) return ILG_OK;
  std::lock_guard<std::mutex> lock(mu);
  if (done.load(std::memory_order_relaxed)) return ILG_OK;
  ILG_CUDA(cudaFuncSetAttribute(k_conduct<double, true, COND_THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SMEM_LIMIT));
  ILG_CUDA(cudaFuncSetAttribute(k_conduct<dfloat, true, COND_STEP_THREADS>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LIMIT));
  ILG_CUDA(cudaFuncSetAttribute(k_conduct<float, true, COND_STEP_THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SMEM_LIMIT));
  // the other block sizes ilg_autotune may choose for single-mesh steps
  ILG_CUDA(cudaFuncSetAttribute(k_conduct<dfloat, true, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LIMIT));
  ILG_CUDA(cudaFuncSetAttribute(k_conduct<dfloat, true, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LIMIT));
  ILG_CUDA(cudaFuncSetAttribute(k_conduct<float, true, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LIMIT));
  ILG_CUDA(cudaFuncSetAttribute(k_conduct<float, true, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LIMIT));
  // the unbiased-rounding variants of the FP32 kernels
  ILG_CUDA(cudaFuncSetAttribute(k_conduct<float, true, 32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SMEM_LIMIT));
  ILG_CUDA(cudaFuncSetAttribute(k_conduct<float, true, COND_STEP_THREADS, true>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_LIMIT));
  ILG_CUDA(cudaFuncSetAttribute(k_conduct<float, true, 128, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SMEM_LIMIT));
  done.store(true, std::memory_order_release);
  return ILG_OK;
}

int conduction_prepare(Context& c, double dt, int precision) {
  if (!c.have_thermal) { set_error("thermal model not initialised"); return ILG_ERR_ARG; }
  ILG_TRY(conduction_setup());
  if (c.coef_dt == dt && c.coef_prec == precision) return ILG_OK;
  std::vector<double> tab;
  CondScalars cs;
  ILG_TRY(build_tables(c.nz, c.z_h.data(), c.ti_h.data(), c.rhoc_h.data(), dt, c.emiss, c.Fgeo, c.bc_mode, tab, cs));
  if (precision == ILG_PREC_MIXED) {
    std::vector<float> t32(tab.size());
    for (size_t i = 0; i < tab.size(); ++i) t32[i] = (float)tab[i];
    ILG_TRY(c.coef32.alloc(t32.size()));
    ILG_CUDA(cudaMemcpy(c.coef32.p, t32.data(), t32.size() * 4, cudaMemcpyHostToDevice));
  } else {
    std::vector<float2> tdf(tab.size());
    for (size_t i = 0; i < tab.size(); ++i) tdf[i] = split_df_host(tab[i]);
    ILG_TRY(c.coefdf.alloc(tdf.size()));
    ILG_CUDA(cudaMemcpy(c.coefdf.p, tdf.data(), tdf.size() * 8, cudaMemcpyHostToDevice));
  }
  c.cond_cs = cs;
  c.coef_dt = dt;
  c.coef_prec = precision;
  return ILG_OK;
}

// Move the layer state between double-float and fp32 storage.
int conduction_state_convert(Context& c, int precision) {
  if (c.state_prec == precision) return ILG_OK;
  size_t n = (size_t)c.nz * c.nt;
  if (precision == ILG_PREC_MIXED) {
    ILG_TRY(c.T32.alloc(n));
    k_df_to_f<<<div_up(n, 256), 256, 0, c.stream>>>(c.Tdf.p, c.T32.p, n);
  } else {
    ILG_TRY(c.Tdf.alloc(n));
    k_f_to_df<<<div_up(n, 256), 256, 0, c.stream>>>(c.T32.p, c.Tdf.p, n);
  }
  ILG_CUDA(cudaGetLastError());
  c.state_prec = precision;
  return ILG_OK;
}

// Threads per block: the view's tuned value for a single mesh (a batch's
// block table is cut at COND_STEP_THREADS), COND_STEP_THREADS where the
// tuned size would not fit the column in shared memory. sr: the FP32
// layers' updates rounded without bias (mixed precision).
int conduction_launch(const StepView& v, const double* Q, int precision, int upd, int nz_max, cudaStream_t s,
                      bool sr) {
  int bs = v.cblocks ? COND_STEP_THREADS : v.tune.conduct_threads;
  if (bs != 32 && bs != 64 && bs != 128) { set_error("conduct_threads must be 32, 64 or 128"); return ILG_ERR_ARG; }
  const size_t elt = precision == ILG_PREC_MIXED ? sizeof(float) : sizeof(dfloat);
  if ((size_t)nz_max * bs * elt > SMEM_LIMIT) bs = COND_STEP_THREADS;
  if (precision == ILG_PREC_MIXED) {
    if (bs == 32) return launch_conduct<float, 32>(v, Q, upd, nz_max, s, sr);
    if (bs == 128) return launch_conduct<float, 128>(v, Q, upd, nz_max, s, sr);
    return launch_conduct<float, COND_STEP_THREADS>(v, Q, upd, nz_max, s, sr);
  }
  if (bs == 32) return launch_conduct<dfloat, 32>(v, Q, upd, nz_max, s);
  if (bs == 128) return launch_conduct<dfloat, 128>(v, Q, upd, nz_max, s);
  return launch_conduct<dfloat, COND_STEP_THREADS>(v, Q, upd, nz_max, s);
}

// ---- thermal records ----------------------------------------------------------
namespace {

// Sums of (T - REC_SHIFT) and of its square (the variance stays well
// conditioned for temperatures of a few hundred K), minima and maxima, per
// conduction block, then per mesh, both in a fixed order (deterministic).
// Group g of a partial: [5g] min, [5g+1] max, [5g+2] count, [5g+3] sum,
// [5g+4] sum of squares, for g = all layers and the surface, the surface
// row, the bottom layer; [15..17] the energy sums.
constexpr double REC_SHIFT = 250.0;

__device__ __forceinline__ double layer_value(const double* T, size_t i) { return T[i]; }
__device__ __forceinline__ double layer_value(const float* T, size_t i) { return (double)T[i]; }
__device__ __forceinline__ double layer_value(const dfloat* T, size_t i) { return (double)T[i]; }

__device__ __forceinline__ void rec_neutral(double* q) {
  for (int g = 0; g < 3; ++g) {
    q[5 * g] = INFINITY;
    q[5 * g + 1] = -INFINITY;
    q[5 * g + 2] = q[5 * g + 3] = q[5 * g + 4] = 0.0;
  }
  q[15] = q[16] = q[17] = 0.0;
}
__device__ __forceinline__ void rec_add(double* q, int g, double x) {
  q[5 * g] = fmin(q[5 * g], x);
  q[5 * g + 1] = fmax(q[5 * g + 1], x);
  double d = x - REC_SHIFT;
  q[5 * g + 2] += 1.0;
  q[5 * g + 3] += d;
  q[5 * g + 4] += d * d;
}
__device__ __forceinline__ void rec_merge(double* a, const double* b) {
  for (int g = 0; g < 3; ++g) {
    a[5 * g] = fmin(a[5 * g], b[5 * g]);
    a[5 * g + 1] = fmax(a[5 * g + 1], b[5 * g + 1]);
    a[5 * g + 2] += b[5 * g + 2];
    a[5 * g + 3] += b[5 * g + 3];
    a[5 * g + 4] += b[5 * g + 4];
  }
  a[15] += b[15];
  a[16] += b[16];
  a[17] += b[17];
}

template <class R>
__global__ void __launch_bounds__(COND_STEP_THREADS) k_rec_partial(StepView v) {
  __shared__ double sh[COND_STEP_THREADS][REC_PART];
  int2 cb = v.cblocks ? v.cblocks[blockIdx.x] : make_int2(0, blockIdx.x * COND_STEP_THREADS);
  const MeshDesc& M = v.md[cb.x];
  double* q = sh[threadIdx.x];
  rec_neutral(q);
  const int fl = cb.y + threadIdx.x;
  if (M.active && M.rec_cap > 0 && fl < M.nfacet) {
    const int g = M.facet0 + fl;
    const R* T = state_T<R>(v) + M.T0 + fl;
    const size_t N = (size_t)M.nfacet;
    const int nz = M.cs.nz;
    double Ts = v.Tsurf[g];
    rec_add(q, 0, Ts);
    rec_add(q, 1, Ts);
    for (int i = 0; i < nz; ++i) {
      double x = layer_value(T, (size_t)i * N);
      rec_add(q, 0, x);
      if (i == nz - 1) rec_add(q, 2, x);
    }
    const double A = v.area[g];
    double t2 = Ts * Ts;
    q[15] = A * v.rad[g];
    q[16] = A * (M.cs.es * (t2 * t2));
    q[17] = A * v.Fsurf[g];
  }
  __syncthreads();
  for (int off = COND_STEP_THREADS / 2; off; off >>= 1) {
    if (threadIdx.x < off) rec_merge(sh[threadIdx.x], sh[threadIdx.x + off]);
    __syncthreads();
  }
  if (threadIdx.x < REC_PART) v.rec_part[(size_t)blockIdx.x * REC_PART + threadIdx.x] = sh[0][threadIdx.x];
}

constexpr int REC_FINAL_THREADS = 128;

__global__ void __launch_bounds__(REC_FINAL_THREADS) k_rec_final(StepView v) {
  __shared__ double sh[REC_FINAL_THREADS][REC_PART];
  const MeshDesc& M = v.md[blockIdx.x];
  if (!M.active || M.rec_cap <= 0) return;
  const int slot = M.frame - M.rec_frame0;
  if (slot < 0 || slot >= M.rec_cap) return;
  double* q = sh[threadIdx.x];
  rec_neutral(q);
  for (int b = M.cb0 + threadIdx.x; b < M.cb0 + M.ncb; b += REC_FINAL_THREADS)
    rec_merge(q, v.rec_part + (size_t)b * REC_PART);
  __syncthreads();
  for (int off = REC_FINAL_THREADS / 2; off; off >>= 1) {
    if (threadIdx.x < off) rec_merge(sh[threadIdx.x], sh[threadIdx.x + off]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double* r = sh[0];
    double* out = v.rec + (size_t)(M.rec0 + slot) * REC_W;
    for (int g = 0; g < 3; ++g) {   // the reference's column order: max, min, mean, std
      double n = r[5 * g + 2], s1 = r[5 * g + 3], s2 = r[5 * g + 4];
      double var = n > 1.0 ? (s2 - s1 * s1 / n) / (n - 1.0) : 0.0;
      out[4 * g] = r[5 * g + 1];
      out[4 * g + 1] = r[5 * g];
      out[4 * g + 2] = REC_SHIFT + s1 / n;
      out[4 * g + 3] = sqrt(fmax(var, 0.0));
    }
    out[12] = r[15];
    out[13] = r[16];
    out[14] = r[17];
  }
}

}  // namespace

int record_launch(const StepView& v, int precision, int ncblocks, cudaStream_t s) {
  if (!v.rec || ncblocks <= 0) return ILG_OK;
  if (precision == ILG_PREC_MIXED) k_rec_partial<float><<<ncblocks, COND_STEP_THREADS, 0, s>>>(v);
  else k_rec_partial<dfloat><<<ncblocks, COND_STEP_THREADS, 0, s>>>(v);
  ILG_CUDA(cudaGetLastError());
  k_rec_final<<<v.nmesh, REC_FINAL_THREADS, 0, s>>>(v);
  ILG_CUDA(cudaGetLastError());
  return ILG_OK;
}

// Standalone batched columns (host arrays, reference layout: column-major
// nz x ncol). Runs on the current device with a private stream.
static int run_columns(int ncol, int nz, const double* z, double dt, const double* Qn, const double* Qnp1, double* T,
                       const double* ti, const double* rhoc, double emiss, double* Tsurf, double Fgeo,
                       double* Fsurf, int bc) {
  if (ncol <= 0) return ILG_OK;
  std::vector<double> tab;
  CondScalars cs;
  ILG_TRY(build_tables(nz, z, ti, rhoc, dt, emiss, Fgeo, bc, tab, cs));
  ILG_TRY(conduction_setup());
  cudaStream_t s;
  ILG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } guard{s};
  dbuf<double> dtab, dT, dTs, dFs, dQn, dQ, rho;
  dbuf<int> derr;
  dbuf<MeshDesc> dmd;
  ILG_TRY(dtab.alloc(tab.size()));
  ILG_TRY(dT.alloc((size_t)nz * ncol));
  ILG_TRY(dTs.alloc(ncol));
  ILG_TRY(dFs.alloc(ncol));
  ILG_TRY(dQn.alloc(ncol));
  ILG_TRY(dQ.alloc(ncol));
  ILG_TRY(derr.alloc(DERR_COUNT));
  ILG_TRY(dmd.alloc(1));
  size_t smem = (size_t)nz * 128 * sizeof(double);
  if (smem > SMEM_LIMIT) ILG_TRY(rho.alloc((size_t)nz * ncol));
  MeshDesc md{};
  md.facet0 = 0; md.nfacet = ncol; md.nz = nz; md.coef0 = 0; md.T0 = 0; md.cs = cs; md.active = 1;
  std::vector<double> Tl((size_t)nz * ncol);
  for (int f = 0; f < ncol; ++f)
    for (int i = 0; i < nz; ++i) Tl[(size_t)i * ncol + f] = T[(size_t)f * nz + i];
  ILG_CUDA(cudaMemcpyAsync(dmd.p, &md, sizeof(md), cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemcpyAsync(dtab.p, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemcpyAsync(dT.p, Tl.data(), Tl.size() * 8, cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemcpyAsync(dTs.p, Tsurf, (size_t)ncol * 8, cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemcpyAsync(dQ.p, Qnp1, (size_t)ncol * 8, cudaMemcpyHostToDevice, s));
  if (Qn) ILG_CUDA(cudaMemcpyAsync(dQn.p, Qn, (size_t)ncol * 8, cudaMemcpyHostToDevice, s));
  else ILG_CUDA(cudaMemsetAsync(dQn.p, 0, (size_t)ncol * 8, s));
  ILG_CUDA(cudaMemsetAsync(derr.p, 0, DERR_COUNT * sizeof(int), s));
  StepView v{};
  v.nt = ncol; v.nmesh = 1; v.md = dmd.p;
  v.Tsurf = dTs.p; v.Fsurf = dFs.p; v.Qprev = dQn.p; v.T64 = dT.p; v.coef64 = dtab.p; v.rho64 = rho.p;
  v.derr = derr.p;
  ILG_TRY((launch_conduct<double, COND_THREADS>(v, dQ.p, 0, nz, s)));
  int herr[DERR_COUNT];
  ILG_CUDA(cudaMemcpyAsync(Tl.data(), dT.p, Tl.size() * 8, cudaMemcpyDeviceToHost, s));
  if (bc != 2) ILG_CUDA(cudaMemcpyAsync(Tsurf, dTs.p, (size_t)ncol * 8, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaMemcpyAsync(Fsurf, dFs.p, (size_t)ncol * 8, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaMemcpyAsync(herr, derr.p, sizeof(herr), cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  if (herr[DERR_PIVOT]) { set_error("zero pivot in a conduction column"); return ILG_ERR_PIVOT; }
  for (int f = 0; f < ncol; ++f)
    for (int i = 0; i < nz; ++i) T[(size_t)f * nz + i] = Tl[(size_t)i * ncol + f];
  return ILG_OK;
}

int conduction_batch_host(int ncol, int nz, const double* z, double dt, const double* Qn, const double* Qnp1,
                          double* T, const double* ti, const double* rhoc, double emiss, double* Tsurf, double Fgeo,
                          double* Fsurf, int bc_mode) {
  if (bc_mode != ILG_BC_LINEARISED && bc_mode != ILG_BC_NEWTON) { set_error("bad bc_mode %d", bc_mode); return ILG_ERR_ARG; }
  return run_columns(ncol, nz, z, dt, Qn, Qnp1, T, ti, rhoc, emiss, Tsurf, Fgeo, Fsurf, bc_mode);
}

int conductiont_host(int nz, const double* z, double dt, double* T, double Tsurf, double Tsurfp1, const double* ti,
                     const double* rhoc, double Fgeo, double* Fsurf) {
  double ts = Tsurf;
  return run_columns(1, nz, z, dt, nullptr, &Tsurfp1, T, ti, rhoc, 1.0, &ts, Fgeo, Fsurf, 2);
}

// ---- conduction columns without allocation ----------------------------------
//
// ilg_conductionq_batch_noalloc runs the same k_conduct kernel as the
// allocating entry point on caller-owned device arrays. Its device scratch is
// one fixed file-scope array, sized once at library load, so the call itself
// never allocates device memory. It serves callers that cannot call
// cudaMalloc at the time they step the columns: code running inside another
// framework's caching allocator (whose memory it must not fragment or
// double-count), host code under a memory budget that is already spent, and
// callers that must not stall on the driver's allocation lock.
//
// Scratch layout (each region starts on a 256-byte boundary):
//   error flags   DERR_COUNT ints; zeroed by every call before its launch
//   mesh record   one MeshDesc, written by every call
//   layer table   nz x 5 doubles, written by every call
//   Qn copy       ncol doubles (Qn, or zeros), written by every call; the
//                 kernel replaces it with Qnp1 as the allocating path does
//   rho           nz x ncol doubles, only for columns deeper than the
//                 shared-memory stage holds (nz > 160); written before read
// Only the error flags must start at zero, and each call clears them itself.
// All calls on one device share that device's copy of the array: two calls
// that overlap on the device would race on it. Calls therefore take a lock
// per device and return only after their work has finished, so calls from
// one process never overlap on a device (calls on different devices do not
// wait for one another).

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)ILG_NOALLOC_SCRATCH_MB << 20;
static __device__ __align__(256) unsigned char g_cond_scratch[NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu[NOALLOC_MAX_DEVICES];   // one lock per device's copy of the scratch

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct NoallocLayout {
  size_t flags, md, tab, qprev, rho, total;
};

NoallocLayout noalloc_layout(int ncol, int nz, bool deep) {
  NoallocLayout L;
  L.flags = 0;
  L.md = L.flags + align256(DERR_COUNT * sizeof(int));
  L.tab = L.md + align256(sizeof(MeshDesc));
  L.qprev = L.tab + align256((size_t)nz * TAB_W * sizeof(double));
  L.rho = L.qprev + align256((size_t)ncol * sizeof(double));
  L.total = L.rho + (deep ? align256((size_t)nz * ncol * sizeof(double)) : 0);
  return L;
}

// On every call, with the caller's device current: the scratch's device
// address on that device and the shared-memory opt-in of the kernel. Both
// are taken afresh each time (they are cheap next to the call's stream
// synchronisation), so a device reset or a new primary context between
// calls cannot leave a stale address behind.
int noalloc_setup(int dev, unsigned char** out) {
  void* ptr = nullptr;
  ILG_CUDA(cudaGetSymbolAddress(&ptr, g_cond_scratch));
  ILG_CUDA(cudaFuncSetAttribute(k_conduct<double, true, COND_THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SMEM_LIMIT));
  (void)dev;
  *out = static_cast<unsigned char*>(ptr);
  return ILG_OK;
}

}  // namespace

}  // namespace ilg

extern "C" int ilg_conductionq_batch_noalloc(int ncol, int nz, const double* z, double dt, const double* Qn,
                                             const double* Qnp1, double* T, const double* ti, const double* rhoc,
                                             double emiss, double* Tsurf, double Fgeotherm, double* Fsurf,
                                             int bc_mode, void* stream) {
  using namespace ilg;
  if (ncol < 0 || nz < 2) { set_error("invalid sizes (ncol %d, nz %d)", ncol, nz); return ILG_ERR_ARG; }
  const bool deep = (size_t)nz * COND_THREADS * sizeof(double) > SMEM_LIMIT;
  const NoallocLayout L = noalloc_layout(ncol, nz, deep);
  if (L.total > NOALLOC_SCRATCH_BYTES) {
    set_error("%d columns of %d layers need %zu bytes of scratch; the fixed scratch holds %zu "
              "(split the columns into smaller calls)", ncol, nz, L.total, NOALLOC_SCRATCH_BYTES);
    return ILG_ERR_ARG;
  }
  if (bc_mode != ILG_BC_LINEARISED && bc_mode != ILG_BC_NEWTON) { set_error("bad bc_mode %d", bc_mode); return ILG_ERR_ARG; }
  if (!z || !ti || !rhoc || (ncol > 0 && (!Qnp1 || !T || !Tsurf || !Fsurf))) {
    set_error("invalid arguments");
    return ILG_ERR_ARG;
  }
  std::vector<double> tab;
  CondScalars cs;
  ILG_TRY(build_tables(nz, z, ti, rhoc, dt, emiss, Fgeotherm, bc_mode, tab, cs));
  if (ncol == 0) return ILG_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the call copies from pageable host memory and synchronises the stream,
  // neither of which a capturing stream allows
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  ILG_CUDA(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone) {
    set_error("ilg_conductionq_batch_noalloc cannot run on a stream that is being captured into a graph");
    return ILG_ERR_ARG;
  }
  int dev = 0;
  ILG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) { set_error("device %d out of range", dev); return ILG_ERR_ARG; }
  std::lock_guard<std::mutex> lock(g_noalloc_mu[dev]);
  unsigned char* base = nullptr;
  ILG_TRY(noalloc_setup(dev, &base));
  MeshDesc md{};
  md.facet0 = 0; md.nfacet = ncol; md.nz = nz; md.coef0 = 0; md.T0 = 0; md.cs = cs; md.active = 1;
  int* flags = reinterpret_cast<int*>(base + L.flags);
  MeshDesc* dmd = reinterpret_cast<MeshDesc*>(base + L.md);
  double* dtab = reinterpret_cast<double*>(base + L.tab);
  double* qprev = reinterpret_cast<double*>(base + L.qprev);
  ILG_CUDA(cudaMemsetAsync(flags, 0, DERR_COUNT * sizeof(int), s));
  ILG_CUDA(cudaMemcpyAsync(dmd, &md, sizeof(md), cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemcpyAsync(dtab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  if (Qn) ILG_CUDA(cudaMemcpyAsync(qprev, Qn, (size_t)ncol * sizeof(double), cudaMemcpyDeviceToDevice, s));
  else ILG_CUDA(cudaMemsetAsync(qprev, 0, (size_t)ncol * sizeof(double), s));
  StepView v{};
  v.nt = ncol; v.nmesh = 1; v.md = dmd;
  v.Tsurf = Tsurf; v.Fsurf = Fsurf; v.Qprev = qprev; v.T64 = T; v.coef64 = dtab;
  v.rho64 = deep ? reinterpret_cast<double*>(base + L.rho) : nullptr;
  v.derr = flags;
  ILG_TRY((launch_conduct<double, COND_THREADS>(v, Qnp1, 0, nz, s)));
  int herr[DERR_COUNT];
  ILG_CUDA(cudaMemcpyAsync(herr, flags, sizeof(herr), cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  if (herr[DERR_PIVOT]) { set_error("zero pivot in a conduction column"); return ILG_ERR_PIVOT; }
  return ILG_OK;
}
