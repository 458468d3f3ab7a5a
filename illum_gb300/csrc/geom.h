// geom.h — exact, portable geometry primitives shared by the CUDA kernels,
// the library's host code and the CPU oracle.
//
// Every function here is written with IEEE-754 +, -, *, / and sqrt only, in a
// fixed evaluation order, so that host (x86-64 / aarch64) and device (sm_103a)
// produce bit-identical results. That is what makes visibility sets, horizon
// bins and sunlit-sample counts reproducible across the CPU oracle and the GPU.
// Requirements on every translation unit that includes this file:
//   * device code: compiled with -fmad=false (no FMA contraction);
//   * host code:   compiled with -ffp-contract=off (aarch64 gcc contracts by
//                  default) and without -ffast-math;
//   * no flush-to-zero (nvcc default without --use_fast_math).
// Transcendentals (sin, cos, atan2, acos) are implemented here from their
// Taylor series (with quadrant reduction for sin / cos and a table of
// atan(k/16) for atan2) instead of calling libm or CUDA's math library,
// whose last-ulp results differ between platforms.
//
// Reference semantics mirrored (sampotter/illum, paths relative to its root):
//   * Vector3 arithmetic is single precision (src/cpp/kdtree.cpp:47 passes a
//     Vector3 as const float*), so centroids, normals, ray origins and ray
//     directions are float (src/cpp/illum.cpp:47-50,72,284-286).
//   * Frenet frame: src/cpp/illum.cpp:244-262.
//   * Form factor formula: src/cpp/illum.cpp:100-127.
//   * Horizon ray direction: src/cpp/illum.cpp:290-297.
//   * Direct-insolation sample test: src/cpp/illum.cpp:421-437.
// The BVH library the reference links (Fast-BVH, absent from the reference
// tree) defines the ray/triangle predicate; this project defines it as the
// double-precision Moller-Trumbore test below (mt64), evaluated on the float
// triangle and ray. The float test (mt32_classify) is only a conservative
// filter in front of it: it never changes an answer.
#pragma once

#if defined(__CUDACC__)
#define ILG_HD __host__ __device__ __forceinline__
#else
#define ILG_HD inline
#endif

#include <math.h>
#include <stdint.h>

namespace ilg {

// ---------------------------------------------------------------- vectors
struct f3 { float x, y, z; };
struct d3 { double x, y, z; };

ILG_HD f3 mk(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
ILG_HD d3 mkd(double x, double y, double z) { d3 r; r.x = x; r.y = y; r.z = z; return r; }
ILG_HD d3 to_d(f3 a) { return mkd((double)a.x, (double)a.y, (double)a.z); }

ILG_HD f3 add(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
ILG_HD f3 sub(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
ILG_HD f3 scl(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
ILG_HD float dot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
ILG_HD f3 cross(f3 a, f3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
ILG_HD float len(f3 a) { return sqrtf(dot(a, a)); }
ILG_HD f3 normalize(f3 a) { float l = len(a); return mk(a.x / l, a.y / l, a.z / l); }
ILG_HD float l1(f3 a) { return (fabsf(a.x) + fabsf(a.y)) + fabsf(a.z); }

ILG_HD d3 add(d3 a, d3 b) { return mkd(a.x + b.x, a.y + b.y, a.z + b.z); }
ILG_HD d3 sub(d3 a, d3 b) { return mkd(a.x - b.x, a.y - b.y, a.z - b.z); }
ILG_HD d3 scl(d3 a, double s) { return mkd(a.x * s, a.y * s, a.z * s); }
ILG_HD double dot(d3 a, d3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
ILG_HD d3 cross(d3 a, d3 b) {
  return mkd(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
ILG_HD double norm(d3 a) { return sqrt(dot(a, a)); }
ILG_HD d3 normalise(d3 a) { double l = norm(a); return mkd(a.x / l, a.y / l, a.z / l); }

// ---------------------------------------------------------------- constants
constexpr double PI = 3.141592653589793;
constexpr double TWO_PI = 6.283185307179586;
constexpr double HALF_PI = 1.5707963267948966;
// pi/2 split for Cody-Waite reduction: head has 24 significant bits, so k*P1
// is exact for |k| < 2^29.
constexpr double PIO2_1 = 1.570796251296997;
constexpr double PIO2_2 = 7.549789954891882e-08;
constexpr double PIO2_3 = -2.6718907338610155e-24;
constexpr double ONE_AU_KM = 149.5978707e6;      // src/cpp/constants.hpp:6
constexpr double SUN_RADIUS_KM = 695508.0;       // src/cpp/constants.hpp:7
constexpr double GOLDEN_RATIO = 1.6180339887498949;
constexpr double SIGMA_SB = 5.6704e-8;           // src/cpp/conductionQ.f:39

// ---------------------------------------------------------------- trig
// sin and cos of r in [-pi/4, pi/4] by Taylor series (terms to r^19 / r^18,
// truncation < 1e-19), Horner form in r^2.
ILG_HD double sin_kernel(double r) {
  double z = r * r;
  double p = -8.22063524662433e-18;           // -1/19!
  p = p * z + 2.8114572543455206e-15;         //  1/17!
  p = p * z - 7.647163731819816e-13;          // -1/15!
  p = p * z + 1.6059043836821613e-10;         //  1/13!
  p = p * z - 2.505210838544172e-08;          // -1/11!
  p = p * z + 2.7557319223985893e-06;         //  1/9!
  p = p * z - 0.0001984126984126984;          // -1/7!
  p = p * z + 0.008333333333333333;           //  1/5!
  p = p * z - 0.16666666666666666;            // -1/3!
  return r + (r * z) * p;
}
ILG_HD double cos_kernel(double r) {
  double z = r * r;
  double p = 1.5619206968586225e-16;          //  1/18!
  p = p * z - 4.779477332387385e-14;          // -1/16!
  p = p * z + 1.1470745597729725e-11;         //  1/14!
  p = p * z - 2.08767569878681e-09;           // -1/12!
  p = p * z + 2.755731922398589e-07;          //  1/10!
  p = p * z - 2.48015873015873e-05;           // -1/8!
  p = p * z + 0.001388888888888889;           //  1/6!
  p = p * z - 0.041666666666666664;           // -1/4!
  p = p * z + 0.5;                            //  1/2!  (subtracted below)
  return 1.0 - z * p;
}

// sin(x), cos(x) for |x| up to ~1e6: quadrant reduction by a three-part pi/2.
ILG_HD void sincos_x(double x, double* s, double* c) {
  double kf = x * (1.0 / HALF_PI);
  kf = (kf >= 0.0) ? (double)(int64_t)(kf + 0.5) : -(double)(int64_t)(0.5 - kf);
  double r = ((x - kf * PIO2_1) - kf * PIO2_2) - kf * PIO2_3;
  double sr = sin_kernel(r), cr = cos_kernel(r);
  int q = (int)(((int64_t)kf) & 3);
  switch (q) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
  }
}

// atan(k/16), k = 0..16, correctly rounded (computed to 60 digits).
ILG_HD double atan_tab16(int k) {
  switch (k) {
    case 0: return 0.0;
    case 1: return 0.06241880999595735;
    case 2: return 0.12435499454676144;
    case 3: return 0.18534794999569476;
    case 4: return 0.24497866312686414;
    case 5: return 0.3028848683749714;
    case 6: return 0.35877067027057225;
    case 7: return 0.4124104415973873;
    case 8: return 0.4636476090008061;
    case 9: return 0.5123894603107377;
    case 10: return 0.5585993153435624;
    case 11: return 0.6022873461349642;
    case 12: return 0.6435011087932844;
    case 13: return 0.6823165548747481;
    case 14: return 0.7188299996216245;
    case 15: return 0.7531512809621944;
    default: return 0.7853981633974483;
  }
}

// atan(n / d) for 0 <= n <= d, d > 0, by a table reduction:
// atan(n/d) = atan(c) + atan(u), c = k/16 near n/d (k from an fp32 estimate,
// correctly rounded on every IEEE platform, so CPU and GPU pick the same k),
// u = (n - c d) / (d + c n), |u| <= ~1/32, and the series
// atan(u) = u + u y (-1/3 + y/5 - y^2/7 + y^3/9 - y^4/11 + y^5/13), y = u^2,
// evaluated in Estrin form (truncation < 1e-19 relative). One division and a
// short dependent chain: the FP64 pipe of the GPU is slow per instruction.
ILG_HD double atan_ratio(double n, double d) {
  if (d < 7.888609052210118e-31) {   // 2^-100: keep the fp32 estimate in range (exact scaling)
    n *= 1.6069380442589903e60;      // 2^200
    d *= 1.6069380442589903e60;
  }
  float rf = (float)n / (float)d;
  int k = (int)(rf * 16.0f + 0.5f);
  if (k < 0) k = 0;
  if (k > 16) k = 16;
  double c = (double)k * 0.0625;
  double u = (n - c * d) / (d + c * n);
  double y = u * u;
  double y2 = y * y;
  double p01 = -0.3333333333333333 + 0.2 * y;
  double p23 = -0.14285714285714285 + 0.1111111111111111 * y;
  double p45 = -0.09090909090909091 + 0.07692307692307693 * y;
  double p = p01 + y2 * (p23 + y2 * p45);
  return atan_tab16(k) + (u + (u * y) * p);
}

// atan2 with the usual quadrant conventions; atan2(0, 0) = 0.
ILG_HD double atan2_x(double y, double x) {
  double ax = fabs(x), ay = fabs(y);
  if (ax == 0.0 && ay == 0.0) return 0.0;
  bool swap = ay > ax;
  double a = swap ? atan_ratio(ax, ay) : atan_ratio(ay, ax);
  if (swap) a = HALF_PI - a;
  if (x < 0.0) a = PI - a;
  return (y < 0.0) ? -a : a;
}

ILG_HD double acos_x(double x) {
  if (x > 1.0) x = 1.0;
  if (x < -1.0) x = -1.0;
  return atan2_x(sqrt((1.0 - x) * (1.0 + x)), x);
}

// ---------------------------------------------------------------- triangles
// Quantities the reference takes from its Tri object (Fast-BVH), in float.
ILG_HD f3 tri_centroid(f3 v0, f3 v1, f3 v2) {
  f3 s = add(add(v0, v1), v2);
  return mk(s.x / 3.0f, s.y / 3.0f, s.z / 3.0f);
}
ILG_HD f3 tri_normal(f3 v0, f3 v1, f3 v2) {
  return normalize(cross(sub(v1, v0), sub(v2, v0)));
}
// Bounding radius: largest centroid-to-vertex distance.
ILG_HD float tri_radius(f3 v0, f3 v1, f3 v2, f3 c) {
  float r0 = len(sub(v0, c)), r1 = len(sub(v1, c)), r2 = len(sub(v2, c));
  float r = r0 > r1 ? r0 : r1;
  return r > r2 ? r : r2;
}
// A_j = |(v1 - v0) x (v2 - v0)| / 2   (src/cpp/illum.cpp:101)
ILG_HD double tri_area(f3 v0, f3 v1, f3 v2) {
  return (double)len(cross(sub(v1, v0), sub(v2, v0))) / 2.0;
}
// Ray origin / horizon origin: centroid displaced along the normal
// (src/cpp/illum.cpp:50, 286).
ILG_HD f3 offset_point(f3 p, f3 n, double offset) {
  float o = (float)offset;
  return add(p, scl(n, o));
}

// Mutual-facing prefilter of src/cpp/illum.cpp:65-68: a pair (j -> i) is
// skipped when (p_i - p_j) . n_j <= -r_i.
ILG_HD bool facing(f3 p_i, float r_i, f3 p_j, f3 n_j) {
  return !(dot(sub(p_i, p_j), n_j) <= -r_i);
}

// Distance cutoff of the visibility pairs (not in the reference, which has
// none; a cutoff makes terrain patches tractable): |p_i - p_j|^2 <= cut2 in
// float, cut2 < 0 meaning no cutoff.
ILG_HD bool within_cutoff(f3 p_i, f3 p_j, float cut2) {
  if (cut2 < 0.0f) return true;
  f3 d = sub(p_i, p_j);
  return dot(d, d) <= cut2;
}

// Form factor F_ij of src/cpp/illum.cpp:108-119. Returns 0 for the
// zero-distance case (the reference skips it).
ILG_HD double form_factor(f3 p_i, f3 n_i, f3 p_j, f3 n_j, double A_j) {
  f3 p_ij = sub(p_j, p_i);
  double r_ij = (double)len(p_ij);
  if (r_ij < 2.220446049250313e-16) return 0.0;
  float rf = (float)r_ij;
  f3 n_ij = mk(p_ij.x / rf, p_ij.y / rf, p_ij.z / rf);
  double a = (double)dot(n_i, n_ij);
  double b = -(double)dot(n_j, n_ij);
  double mu_ij = a > 0.0 ? a : 0.0;
  double mu_ji = b > 0.0 ? b : 0.0;
  return ((mu_ij * mu_ji) * A_j) / ((PI * r_ij) * r_ij);
}

// Frenet frame of src/cpp/illum.cpp:244-262: columns b = t x n,
// t = (v1 - v0)/|v1 - v0| (difference taken in float), n = normal.
struct frame3 { d3 b, t, n; };
ILG_HD frame3 tri_frame(f3 v0, f3 v1, f3 n) {
  frame3 F;
  F.n = normalise(to_d(n));
  F.t = normalise(to_d(sub(v1, v0)));
  F.b = cross(F.t, F.n);
  return F;
}
// F * (c0, c1, c2), rows summed left to right.
ILG_HD d3 frame_apply(const frame3& F, double c0, double c1, double c2) {
  return mkd((F.b.x * c0 + F.t.x * c1) + F.n.x * c2,
             (F.b.y * c0 + F.t.y * c1) + F.n.y * c2,
             (F.b.z * c0 + F.t.z * c1) + F.n.z * c2);
}
// F^T * v
ILG_HD d3 frame_apply_t(const frame3& F, d3 v) {
  return mkd(dot(F.b, v), dot(F.t, v), dot(F.n, v));
}
// Horizon ray direction for azimuth (cos phi, sin phi) and zenith
// (cos th, sin th), rounded to float as the reference's Vector3 does.
ILG_HD f3 horizon_dir(const frame3& F, double cph, double sph, double cth, double sth) {
  d3 v = frame_apply(F, cph * sth, sph * sth, cth);
  return mk((float)v.x, (float)v.y, (float)v.z);
}

// ---------------------------------------------------------------- ray/triangle
// Canonical predicate: double-precision Moller-Trumbore on float inputs, in
// division-free form. Hit iff det != 0, u >= 0, v >= 0, u + v <= 1, t > 0.
ILG_HD bool mt64(f3 of, f3 df, f3 v0f, f3 v1f, f3 v2f, double* t_out) {
  d3 o = to_d(of), d = to_d(df), v0 = to_d(v0f);
  d3 e1 = sub(to_d(v1f), v0), e2 = sub(to_d(v2f), v0);
  d3 p = cross(d, e2);
  double det = dot(e1, p);
  if (det == 0.0) return false;
  d3 s = sub(o, v0);
  double U = dot(s, p);
  d3 q = cross(s, e1);
  double V = dot(d, q);
  double T = dot(e2, q);
  if (det < 0.0) { det = -det; U = -U; V = -V; T = -T; }
  if (U < 0.0 || V < 0.0 || U + V > det || !(T > 0.0)) return false;
  *t_out = T / det;
  return true;
}

// Conservative single-precision filter in front of mt64.
//   returns 0: mt64 certainly misses;
//           1: mt64 certainly hits, with its t inside [*tlo, *thi];
//           2: undecided (evaluate mt64).
// Error bounds: every computed triple product differs from the exact value
// (for the float inputs) by at most ~8 u * (sum of |products|) with
// u = 2^-24; the bounds below use 64 u times an l1-norm product that
// dominates that sum, which also covers mt64's own (2^-53) rounding.
ILG_HD int mt32_classify(f3 o, f3 d, f3 v0, f3 v1, f3 v2, float* tlo, float* thi) {
  const float K = 64.0f * 5.9604645e-08f;
  f3 e1 = sub(v1, v0), e2 = sub(v2, v0), s = sub(o, v0);
  f3 p = cross(d, e2);
  float det = dot(e1, p);
  f3 q = cross(s, e1);
  float U = dot(s, p), V = dot(d, q), T = dot(e2, q);
  float n1 = l1(e1), n2 = l1(e2), ns = l1(s), nd = l1(d);
  float Bd = K * (n1 * nd) * n2;
  float Bu = K * (ns * nd) * n2;
  float Bv = K * (ns * nd) * n1;
  float Bt = K * (n2 * ns) * n1;
  if (det < 0.0f) { det = -det; U = -U; V = -V; T = -T; }
  if (det <= Bd) return 2;
  if (U + Bu < 0.0f || V + Bv < 0.0f || T + Bt <= 0.0f) return 0;
  if ((U - Bu) + (V - Bv) > det + Bd) return 0;
  if (U - Bu > 0.0f && V - Bv > 0.0f && (U + Bu) + (V + Bv) < det - Bd && T - Bt > 0.0f) {
    *tlo = ((T - Bt) / (det + Bd)) * (1.0f - 4.0f * 5.9604645e-08f);
    *thi = ((T + Bt) / (det - Bd)) * (1.0f + 4.0f * 5.9604645e-08f);
    return 1;
  }
  return 2;
}

// ---------------------------------------------------------------- boxes
// Slab test, float. Zero direction components are replaced by +-1e-30 in the
// reciprocal so no 0*inf NaN can arise. Boxes are inflated at build time, so
// this never rejects a box that contains an mt64 hit.
struct ray_inv { f3 o, inv; };
ILG_HD ray_inv make_ray_inv(f3 o, f3 d) {
  ray_inv r;
  r.o = o;
  float dx = fabsf(d.x) < 1e-30f ? (d.x < 0.0f ? -1e-30f : 1e-30f) : d.x;
  float dy = fabsf(d.y) < 1e-30f ? (d.y < 0.0f ? -1e-30f : 1e-30f) : d.y;
  float dz = fabsf(d.z) < 1e-30f ? (d.z < 0.0f ? -1e-30f : 1e-30f) : d.z;
  r.inv = mk(1.0f / dx, 1.0f / dy, 1.0f / dz);
  return r;
}
// Returns the entry parameter (>= 0) or a negative value on a miss.
ILG_HD float slab(const ray_inv& r, f3 lo, f3 hi, float tmax) {
  float tx0 = (lo.x - r.o.x) * r.inv.x, tx1 = (hi.x - r.o.x) * r.inv.x;
  float ty0 = (lo.y - r.o.y) * r.inv.y, ty1 = (hi.y - r.o.y) * r.inv.y;
  float tz0 = (lo.z - r.o.z) * r.inv.z, tz1 = (hi.z - r.o.z) * r.inv.z;
  float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
  float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
  // relative slack covers the rounding of the six products
  return (tn <= tf * 1.0000005f) ? tn : -1.0f;
}

// ---------------------------------------------------------------- insolation
// Fibonacci-spiral sun-disk samples (src/cpp/illum.cpp:468-483).
inline void fib_spiral(double* xy /* n x 2, column-major */, int n) {
  double a = 0.0, da = TWO_PI * (GOLDEN_RATIO - 1.0) / GOLDEN_RATIO;
  double r = 0.0, dr = 1.0 / (double)(n + 1);
  for (int i = 0; i < n; ++i) {
    double s, c;
    sincos_x(a, &s, &c);
    xy[i] = r * c;
    xy[n + i] = r * s;
    double an = a + da;
    a = an - TWO_PI * (double)(int64_t)(an / TWO_PI);   // fmod for an >= 0
    if (a < 0.0) a += TWO_PI;
    r += dr;
  }
}

// Deterministic sun-disk frame (replaces the random tangent of
// src/cpp/illum.cpp:406): T is the component of the coordinate axis least
// aligned with N orthogonal to N; B = T x N.
ILG_HD void sun_frame(d3 N, d3* T, d3* B) {
  double ax = fabs(N.x), ay = fabs(N.y), az = fabs(N.z);
  d3 e;
  if (ax <= ay && ax <= az) e = mkd(1.0, 0.0, 0.0);
  else if (ay <= az) e = mkd(0.0, 1.0, 0.0);
  else e = mkd(0.0, 0.0, 1.0);
  double ne = dot(N, e);
  *T = normalise(sub(e, scl(N, ne)));
  *B = cross(*T, N);
}

// Cosine between the sun-centre direction seen from p and the facet normal n
// (src/cpp/illum.cpp:405,446: dot(normalise(sun - p), n)), written as
// dot(sun - p, n) / |sun - p| (one division instead of three).
ILG_HD double sun_mu(d3 S, d3 p, d3 n) {
  d3 v = sub(S, p);
  return dot(v, n) / norm(v);
}

// One sun-disk sample of src/cpp/illum.cpp:422-436: returns 1 when the sample
// direction lies above the horizon. h points at the facet's nphi horizon
// zenith angles. interp = 0 keeps the reference's threshold
// h[k] + t*dphi; interp = 1 interpolates h[k] .. h[k+1] linearly.
//
// The reference takes acos of the normalised direction's z; with the
// orthonormal frame the same angles come from the unnormalised direction,
// theta = atan2(|(x, y)|, z) and phi = atan2(y, x), which drops the
// normalisation's square root and three divisions from the dependent chain
// (FP64 latency dominates this test on the GPU). The bin and its fraction
// come from one division, q = phi / dphi.
template <class HLoad>
ILG_HD int sample_lit(d3 p, d3 disk, const frame3& BTN, HLoad h, int nphi, double dphi, int interp) {
  d3 dir = frame_apply_t(BTN, sub(disk, p));
  double theta = atan2_x(sqrt(dir.x * dir.x + dir.y * dir.y), dir.z);
  double phi = atan2_x(dir.y, dir.x);
  if (phi < 0.0) phi += TWO_PI;
  double q = phi / dphi;
  int k = (int)floor(q);
  if (k < 0) k = 0;
  if (k > nphi - 1) k = nphi - 1;
  double t = q - (double)k;
  double thr;
  if (interp == 0) {
    thr = h(k) + t * dphi;
  } else {
    int k1 = k + 1 < nphi ? k + 1 : nphi - 1;
    thr = h(k) + t * (h(k1) - h(k));
  }
  return theta < thr ? 1 : 0;
}

}  // namespace ilg
