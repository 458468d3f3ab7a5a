// bvh.cu — LBVH build (Morton codes, radix sort, Karras hierarchy, bottom-up
// boxes), closest-hit / any-hit traversal, the horizon bisection kernel
// (src/cpp/illum.cpp:274-363) and the visibility + form-factor assembly
// (src/cpp/illum.cpp:31-237). Compiled with -fmad=false: the ray origins,
// directions and the mt64 predicate must round exactly as geom.h specifies.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <vector>

#include "geom.h"
#include "internal.cuh"

namespace ilg {

namespace {

typedef unsigned long long u64;

__device__ __forceinline__ f3 f3of(float4 a) { return mk(a.x, a.y, a.z); }

// ------------------------------------------------------------------ build
__global__ void k_prepare(const float* __restrict__ verts, const int32_t* __restrict__ tris,
                          const float* __restrict__ normals, int nt, float4* tri_o, float4* cen, float4* nrm,
                          double* area, double* frame, float4* frame32) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const float* a = verts + 3 * (int64_t)tris[3 * t];
  const float* b = verts + 3 * (int64_t)tris[3 * t + 1];
  const float* d = verts + 3 * (int64_t)tris[3 * t + 2];
  f3 v0 = mk(a[0], a[1], a[2]), v1 = mk(b[0], b[1], b[2]), v2 = mk(d[0], d[1], d[2]);
  f3 c = tri_centroid(v0, v1, v2);
  f3 n = normals ? mk(normals[3 * t], normals[3 * t + 1], normals[3 * t + 2]) : tri_normal(v0, v1, v2);
  float r = tri_radius(v0, v1, v2, c);
  tri_o[3 * t] = make_float4(v0.x, v0.y, v0.z, 0.f);
  tri_o[3 * t + 1] = make_float4(v1.x, v1.y, v1.z, 0.f);
  tri_o[3 * t + 2] = make_float4(v2.x, v2.y, v2.z, 0.f);
  cen[t] = make_float4(c.x, c.y, c.z, r);
  nrm[t] = make_float4(n.x, n.y, n.z, 0.f);
  area[t] = tri_area(v0, v1, v2);
  frame3 F = tri_frame(v0, v1, n);
  double* fr = frame + 9 * (int64_t)t;
  fr[0] = F.b.x; fr[1] = F.b.y; fr[2] = F.b.z;
  fr[3] = F.t.x; fr[4] = F.t.y; fr[5] = F.t.z;
  fr[6] = F.n.x; fr[7] = F.n.y; fr[8] = F.n.z;
  frame32[3 * t] = make_float4((float)F.b.x, (float)F.b.y, (float)F.b.z, 0.f);
  frame32[3 * t + 1] = make_float4((float)F.t.x, (float)F.t.y, (float)F.t.z, 0.f);
  frame32[3 * t + 2] = make_float4((float)F.n.x, (float)F.n.y, (float)F.n.z, 0.f);
}

__device__ __forceinline__ u64 spread3(u64 x) {   // 21 bits -> every third bit
  x &= 0x1fffffull;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

__global__ void k_morton(const float4* __restrict__ cen, int nt, float3 lo, float3 inv_ext, u64* keys,
                         uint32_t* vals) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  float4 c = cen[t];
  float q = 2097151.0f;
  float x = fminf(fmaxf((c.x - lo.x) * inv_ext.x, 0.f), 1.f) * q;
  float y = fminf(fmaxf((c.y - lo.y) * inv_ext.y, 0.f), 1.f) * q;
  float z = fminf(fmaxf((c.z - lo.z) * inv_ext.z, 0.f), 1.f) * q;
  keys[t] = (spread3((u64)x) << 2) | (spread3((u64)y) << 1) | spread3((u64)z);
  vals[t] = (uint32_t)t;
}

__device__ __forceinline__ int delta(const u64* keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  u64 a = keys[i], b = keys[j];
  if (a == b) return 64 + __clz((unsigned)(i ^ j));
  return __clzll((long long)(a ^ b));
}

// Karras (2012) radix-tree construction: internal node i covers a key range
// and splits it at the highest differing bit. Child codes: >= 0 internal,
// ~k leaf k. parent arrays: [0, n-1) internal, [n-1, 2n-1) leaves.
__global__ void k_karras(const u64* __restrict__ keys, int n, int2* child, int* parent) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = delta(keys, n, i, j);
  int s = 0;
  int t = l;
  do {
    t = (t + 1) >> 1;
    if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  int g = i + s * d + (d < 0 ? -1 : 0);
  int lo = i < j ? i : j, hi = i < j ? j : i;
  int left = (lo == g) ? ~g : g;
  int right = (hi == g + 1) ? ~(g + 1) : (g + 1);
  child[i] = make_int2(left, right);
  parent[left >= 0 ? left : (n - 1) + ~left] = i;
  parent[right >= 0 ? right : (n - 1) + ~right] = i;
}

// Leaf boxes (inflated by pad) and bottom-up union: the second child to
// arrive at a node computes its box (atomic arrival counter, no waiting).
__global__ void k_refit(const float4* __restrict__ tri_o, const uint32_t* __restrict__ order, int n,
                        const int2* __restrict__ child, const int* __restrict__ parent, float4* box_lo,
                        float4* box_hi, int* flags, float pad, float4* tri_s, int* depth_out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int t = (int)order[k];
  float4 a = tri_o[3 * t], b = tri_o[3 * t + 1], c = tri_o[3 * t + 2];
  tri_s[3 * k] = make_float4(a.x, a.y, a.z, __int_as_float(t));
  tri_s[3 * k + 1] = b;
  tri_s[3 * k + 2] = c;
  float4 lo = make_float4(fminf(fminf(a.x, b.x), c.x) - pad, fminf(fminf(a.y, b.y), c.y) - pad,
                          fminf(fminf(a.z, b.z), c.z) - pad, 0.f);
  float4 hi = make_float4(fmaxf(fmaxf(a.x, b.x), c.x) + pad, fmaxf(fmaxf(a.y, b.y), c.y) + pad,
                          fmaxf(fmaxf(a.z, b.z), c.z) + pad, 0.f);
  int slot = (n - 1) + k;
  box_lo[slot] = lo;
  box_hi[slot] = hi;
  if (n == 1) return;
  int depth = 0;
  int p = parent[slot];
  while (p >= 0) {
    __threadfence();
    if (atomicAdd(&flags[p], 1) == 0) return;
    int2 ch = child[p];
    int sl = ch.x >= 0 ? ch.x : (n - 1) + ~ch.x;
    int sr = ch.y >= 0 ? ch.y : (n - 1) + ~ch.y;
    float4 l0 = __ldcg(&box_lo[sl]), h0 = __ldcg(&box_hi[sl]);
    float4 l1 = __ldcg(&box_lo[sr]), h1 = __ldcg(&box_hi[sr]);
    box_lo[p] = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.f);
    box_hi[p] = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.f);
    ++depth;
    p = parent[p];
  }
  atomicMax(depth_out, depth);
}

__global__ void k_pack_nodes(const int2* __restrict__ child, const float4* __restrict__ box_lo,
                             const float4* __restrict__ box_hi, int n, float4* nodes) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int2 ch = child[i];
  int sl = ch.x >= 0 ? ch.x : (n - 1) + ~ch.x;
  int sr = ch.y >= 0 ? ch.y : (n - 1) + ~ch.y;
  float4 l0 = box_lo[sl], h0 = box_hi[sl], l1 = box_lo[sr], h1 = box_hi[sr];
  nodes[4 * i] = make_float4(l0.x, l0.y, l0.z, h0.x);
  nodes[4 * i + 1] = make_float4(h0.y, h0.z, l1.x, l1.y);
  nodes[4 * i + 2] = make_float4(l1.z, h1.x, h1.y, h1.z);
  nodes[4 * i + 3] = make_float4(__int_as_float(ch.x), __int_as_float(ch.y), 0.f, 0.f);
}

// ------------------------------------------------------------------ traversal
struct NodeBoxes { f3 llo, lhi, rlo, rhi; int left, right; };

__device__ __forceinline__ NodeBoxes load_node(const float4* __restrict__ nodes, int i) {
  float4 a = __ldg(&nodes[4 * i]), b = __ldg(&nodes[4 * i + 1]), c = __ldg(&nodes[4 * i + 2]),
         d = __ldg(&nodes[4 * i + 3]);
  NodeBoxes nb;
  nb.llo = mk(a.x, a.y, a.z); nb.lhi = mk(a.w, b.x, b.y);
  nb.rlo = mk(b.z, b.w, c.x); nb.rhi = mk(c.y, c.z, c.w);
  nb.left = __float_as_int(d.x); nb.right = __float_as_int(d.y);
  return nb;
}

// Closest hit under geom.h's mt64 (smallest t, ties to the smaller original
// index). Returns the original facet index or -1; sets *err on stack
// overflow; *t_out (if given) receives the hit's mt64 t.
//
// The FP64 test runs only where single precision cannot decide. A leaf that
// mt32_classify calls a certain hit comes with an enclosure [tlo, thi] of its
// mt64 t; the best hit so far is kept as such an enclosure [blo, bhi] and
// compared by intervals: tlo > bhi means certainly farther, thi < blo
// certainly closer (so no tie is possible). Only when the intervals overlap,
// or the leaf is undecided, are the exact t of both hits computed and
// compared with the tie rule. The argmin of (t, index) over all mt64 hits is
// therefore the one an all-FP64 traversal finds; rays aimed at facet
// centroids almost never need the FP64 path.
__device__ int trace_closest(const float4* __restrict__ nodes, const float4* __restrict__ tri_s, int root,
                             f3 o, f3 d, double* t_out, int* err) {
  ray_inv ri = make_ray_inv(o, d);
  int besti = -1, bk = 0;
  float blo = 3.0e38f, bhi = 3.0e38f;   // encloses the best hit's mt64 t
  double bt = 0.0;                      // that t, once computed (bex)
  bool bex = false;
  float tmaxf = 3.0e38f;
  int stack[TRACE_STACK];
  int sp = 0;
  int node = root;
  for (;;) {
    if (node < 0) {
      int k = ~node;
      float4 a = __ldg(&tri_s[3 * k]), b = __ldg(&tri_s[3 * k + 1]), c = __ldg(&tri_s[3 * k + 2]);
      f3 v0 = f3of(a), v1 = f3of(b), v2 = f3of(c);
      int idx = __float_as_int(a.w);
      float tlo, thi;
      int cls = mt32_classify(o, d, v0, v1, v2, &tlo, &thi);
      bool take = false;
      if (cls == 1 && (besti < 0 || thi < blo)) {
        take = true;                    // certainly the closest so far
        bex = false;
        blo = tlo;
        bhi = thi;
      } else if (cls == 2 || (cls == 1 && !(tlo > bhi))) {
        double th;
        if (mt64(o, d, v0, v1, v2, &th)) {
          if (besti >= 0 && !bex) {     // exact t of the current best
            float4 ba = __ldg(&tri_s[3 * bk]), bb = __ldg(&tri_s[3 * bk + 1]), bc = __ldg(&tri_s[3 * bk + 2]);
            bex = mt64(o, d, f3of(ba), f3of(bb), f3of(bc), &bt);
          }
          if (besti < 0 || th < bt || (th == bt && idx < besti)) {
            take = true;
            bex = true;
            bt = th;
            float tf = (float)th;
            blo = tf * (1.0f - 2.4e-7f);
            bhi = tf * (1.0f + 2.4e-7f) + 1e-37f;
          }
        }
      }
      if (take) {
        besti = idx;
        bk = k;
        tmaxf = bhi * 1.000001f + 1e-30f;
      }
      if (sp == 0) break;
      node = stack[--sp];
      continue;
    }
    NodeBoxes nb = load_node(nodes, node);
    float tl = slab(ri, nb.llo, nb.lhi, tmaxf);
    float tr = slab(ri, nb.rlo, nb.rhi, tmaxf);
    bool hl = tl >= 0.f, hr = tr >= 0.f;
    if (hl && hr) {
      if (sp == TRACE_STACK) { atomicExch(err, 1); break; }
      if (tl <= tr) { stack[sp++] = nb.right; node = nb.left; }
      else { stack[sp++] = nb.left; node = nb.right; }
    } else if (hl) {
      node = nb.left;
    } else if (hr) {
      node = nb.right;
    } else {
      if (sp == 0) break;
      node = stack[--sp];
    }
  }
  if (t_out) {
    if (besti >= 0 && !bex) {
      float4 ba = __ldg(&tri_s[3 * bk]), bb = __ldg(&tri_s[3 * bk + 1]), bc = __ldg(&tri_s[3 * bk + 2]);
      mt64(o, d, f3of(ba), f3of(bb), f3of(bc), &bt);
    }
    *t_out = besti >= 0 ? bt : 1e300;
  }
  return besti;
}

// Any hit under mt64.
__device__ bool trace_any(const float4* __restrict__ nodes, const float4* __restrict__ tri_s, int root, f3 o,
                          f3 d, int* err) {
  ray_inv ri = make_ray_inv(o, d);
  int stack[TRACE_STACK];
  int sp = 0;
  int node = root;
  for (;;) {
    if (node < 0) {
      int k = ~node;
      float4 a = __ldg(&tri_s[3 * k]), b = __ldg(&tri_s[3 * k + 1]), c = __ldg(&tri_s[3 * k + 2]);
      f3 v0 = f3of(a), v1 = f3of(b), v2 = f3of(c);
      float tlo, thi;
      int cls = mt32_classify(o, d, v0, v1, v2, &tlo, &thi);
      if (cls == 1) return true;
      if (cls == 2) {
        double th;
        if (mt64(o, d, v0, v1, v2, &th)) return true;
      }
      if (sp == 0) return false;
      node = stack[--sp];
      continue;
    }
    NodeBoxes nb = load_node(nodes, node);
    float tl = slab(ri, nb.llo, nb.lhi, 3.0e38f);
    float tr = slab(ri, nb.rlo, nb.rhi, 3.0e38f);
    bool hl = tl >= 0.f, hr = tr >= 0.f;
    if (hl && hr) {
      if (sp == TRACE_STACK) { atomicExch(err, 1); return false; }
      if (tl <= tr) { stack[sp++] = nb.right; node = nb.left; }
      else { stack[sp++] = nb.left; node = nb.right; }
    } else if (hl) {
      node = nb.left;
    } else if (hr) {
      node = nb.right;
    } else {
      if (sp == 0) return false;
      node = stack[--sp];
    }
  }
}

__global__ void k_trace(const float4* __restrict__ nodes, const float4* __restrict__ tri_s, int root, int nrays,
                        const float* __restrict__ orig, const float* __restrict__ dir, int any_hit, int32_t* hit,
                        double* thit, int* derr) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrays) return;
  f3 o = mk(orig[3 * r], orig[3 * r + 1], orig[3 * r + 2]);
  f3 d = mk(dir[3 * r], dir[3 * r + 1], dir[3 * r + 2]);
  if (any_hit) {
    hit[r] = trace_any(nodes, tri_s, root, o, d, &derr[DERR_STACK]) ? 1 : -1;
    thit[r] = -1.0;
  } else {
    double t;
    int h = trace_closest(nodes, tri_s, root, o, d, &t, &derr[DERR_STACK]);
    hit[r] = h;
    thit[r] = h >= 0 ? t : -1.0;
  }
}

// ------------------------------------------------------------------ renderer
// One closest-hit ray per pixel of src/cpp/illum_renderer_cli.cpp:228-276:
// mode 0 orthographic from direction (az, el) at distance 1.1 r_model,
// mode 1 equal-area cylindrical map (rays from a sphere of radius
// 1.1 r_model towards the model centre). out: facet index or -1.
struct RenderCam {
  int mode, width, height;
  double rad, aspect, az, el;
  float px, py, pz, ex, ey, ez, ux, uy, uz, rx, ry, rz;   // orthographic camera (float, as Vector3)
  float cx, cy, cz;                                     // model centre
};

__global__ void k_render(const float4* __restrict__ nodes, const float4* __restrict__ tri_s, int root, RenderCam cam,
                         int32_t* out, int* derr) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)cam.width * cam.height) return;
  const int i = (int)(k / cam.width), j = (int)(k % cam.width);
  f3 o, d;
  if (cam.mode == 0) {
    double y_eye = (2.0 * (1.0 - (double)i / (cam.height - 1)) - 1.0) * cam.rad;
    double x_eye = (2.0 * (double)j / (cam.width - 1) - 1.0) * cam.aspect * cam.rad;
    float ye = (float)y_eye, xe = (float)x_eye;
    o = mk(cam.px + ye * cam.ux + xe * cam.rx, cam.py + ye * cam.uy + xe * cam.ry, cam.pz + ye * cam.uz + xe * cam.rz);
    d = mk(cam.ex, cam.ey, cam.ez);
  } else {
    const double PI_D = 3.141592653589793;
    double theta = asin(2.0 * (double)(i + 1) / (cam.height + 1) - 1.0) - cam.el;
    double phi = 2.0 * PI_D * (double)j / cam.width - cam.az;
    f3 p = mk((float)(cam.rad * cos(phi) * sin(theta)), (float)(cam.rad * sin(phi) * sin(theta)),
              (float)(cam.rad * cos(theta)));
    d = normalize(mk(-p.x, -p.y, -p.z));
    o = mk(p.x + cam.cx, p.y + cam.cy, p.z + cam.cz);
  }
  out[k] = trace_closest(nodes, tri_s, root, o, d, nullptr, &derr[DERR_STACK]);
}

// ------------------------------------------------------------------ horizons
// One thread per (facet, azimuth): walk the precomputed bisection tree of
// src/cpp/illum.cpp:304-316 (hit -> hi = mid, miss -> lo = mid), one any-hit
// ray per level, until a terminal node.
__global__ void k_horizons(const float4* __restrict__ nodes, const float4* __restrict__ tri_s, int root,
                           const float4* __restrict__ tri_o, const float4* __restrict__ cen,
                           const float4* __restrict__ nrm, int nt, int nphi, const double* __restrict__ cph,
                           const double* __restrict__ sph, const HorizonNode* __restrict__ tree, int tree_size,
                           float offset, double* H, int* derr) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (int64_t)nt * nphi) return;
  int f = (int)(g / nphi), k = (int)(g % nphi);
  float4 c4 = cen[f], n4 = nrm[f];
  f3 c = f3of(c4), n = f3of(n4);
  f3 o = add(c, scl(n, offset));
  frame3 F = tri_frame(f3of(tri_o[3 * f]), f3of(tri_o[3 * f + 1]), n);
  double cp = cph[k], sp = sph[k];
  int node = 1;
  for (;;) {
    if (node >= tree_size) { atomicExch(&derr[DERR_HORIZON], 1); H[g] = 0.0; return; }
    HorizonNode hn = tree[node];
    if (hn.terminal) { H[g] = hn.mid; return; }
    f3 d = horizon_dir(F, cp, sp, hn.c, hn.s);
    bool hit = trace_any(nodes, tri_s, root, o, d, &derr[DERR_STACK]);
    node = 2 * node + (hit ? 0 : 1);
  }
}

// fp32 copies of a facet's horizon and of its min / max (the insolation
// filters compare in fp32 with margins).
__global__ void k_horizon_f32(const double* __restrict__ H, int nt, int nphi, float* H32, float2* hmm) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nt) return;
  const double* h = H + (int64_t)f * nphi;
  float* h32 = H32 + (int64_t)f * nphi;
  double lo = h[0], hi = h[0];
  for (int k = 0; k < nphi; ++k) {
    lo = fmin(lo, h[k]);
    hi = fmax(hi, h[k]);
    h32[k] = (float)h[k];
  }
  hmm[f] = make_float2((float)lo, (float)hi);
}

// ------------------------------------------------------------------ visibility
// Candidate enumeration for source j: every i != j passing the facing test
// of src/cpp/illum.cpp:65-68 (and the optional distance cutoff), found by a
// half-space query over the BVH (boxes whose farthest point along n_j is
// below -r_max are skipped, and with a cutoff boxes farther than it plus
// r_max).
__device__ __forceinline__ float box_dist2(f3 p, f3 lo, f3 hi) {
  float dx = fmaxf(fmaxf(lo.x - p.x, p.x - hi.x), 0.f);
  float dy = fmaxf(fmaxf(lo.y - p.y, p.y - hi.y), 0.f);
  float dz = fmaxf(fmaxf(lo.z - p.z, p.z - hi.z), 0.f);
  return dx * dx + dy * dy + dz * dz;
}

// Up to FF_SPLIT disjoint subtrees covering every leaf (breadth-first from
// the root), so that one source's query splits into FF_SPLIT work items.
constexpr int FF_SPLIT = 32;

__global__ void k_frontier(const float4* __restrict__ nodes, int root, int* front, int* nfront) {
  int f[FF_SPLIT];
  int n = 1;
  f[0] = root;
  bool grew = true;
  while (grew) {
    grew = false;
    for (int k = 0; k < n && n < FF_SPLIT; ++k) {
      if (f[k] < 0) continue;
      float4 d = __ldg(&nodes[4 * f[k] + 3]);
      f[k] = __float_as_int(d.x);
      f[n++] = __float_as_int(d.y);
      grew = true;
    }
  }
  for (int k = 0; k < FF_SPLIT; ++k) front[k] = k < n ? f[k] : 0;
  *nfront = n;
}

// Work item (source number q in [j0, j1), subtree sub), stored at
// t = (q - j0) FF_SPLIT + sub so that a source's candidates are contiguous;
// the source facet is q, or src[q] for a list of sources. Threads run
// subtree-major: a warp holds consecutive sources on the same subtree
// (similar queries). Counting writes count[t]; FILL writes the item's
// candidates from offs[t] - base0 on.
template <bool FILL>
__global__ void k_candidates(const float4* __restrict__ nodes, const float4* __restrict__ tri_s,
                             const int* __restrict__ front, const int* __restrict__ nfront,
                             const float4* __restrict__ cen, const float4* __restrict__ nrm, int j0, int j1,
                             const int* __restrict__ src, float r_max, float slack, float cut2, float box_cut2,
                             uint32_t* count, const unsigned long long* __restrict__ offs, unsigned long long base0,
                             int32_t* cand_i, int32_t* cand_j, int* derr) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nsrc = j1 - j0;
  const int sub = (int)(u / nsrc), q = j0 + (int)(u % nsrc);
  if (sub >= FF_SPLIT) return;
  const int j = src ? src[q] : q;
  const int64_t t = (int64_t)(q - j0) * FF_SPLIT + sub;
  uint32_t cnt = 0;
  if (sub >= *nfront) {
    if (!FILL) count[t] = 0;
    return;
  }
  float4 cj4 = cen[j], nj4 = nrm[j];
  f3 p_j = f3of(cj4), n_j = f3of(nj4);
  float lim = -r_max - slack;
  unsigned long long base = FILL ? offs[t] - base0 : 0ull;
  int stack[TRACE_STACK];
  int sp = 0;
  int node = front[sub];
  for (;;) {
    if (node < 0) {
      int k = ~node;
      int i = __float_as_int(__ldg(&tri_s[3 * k]).w);
      if (i != j) {
        float4 ci4 = __ldg(&cen[i]);
        if (facing(f3of(ci4), ci4.w, p_j, n_j) && within_cutoff(f3of(ci4), p_j, cut2)) {
          if (FILL) { cand_i[base + cnt] = i; cand_j[base + cnt] = j; }
          ++cnt;
        }
      }
      if (sp == 0) break;
      node = stack[--sp];
      continue;
    }
    NodeBoxes nb = load_node(nodes, node);
    float ml = (n_j.x >= 0.f ? (nb.lhi.x - p_j.x) * n_j.x : (nb.llo.x - p_j.x) * n_j.x) +
               (n_j.y >= 0.f ? (nb.lhi.y - p_j.y) * n_j.y : (nb.llo.y - p_j.y) * n_j.y) +
               (n_j.z >= 0.f ? (nb.lhi.z - p_j.z) * n_j.z : (nb.llo.z - p_j.z) * n_j.z);
    float mr = (n_j.x >= 0.f ? (nb.rhi.x - p_j.x) * n_j.x : (nb.rlo.x - p_j.x) * n_j.x) +
               (n_j.y >= 0.f ? (nb.rhi.y - p_j.y) * n_j.y : (nb.rlo.y - p_j.y) * n_j.y) +
               (n_j.z >= 0.f ? (nb.rhi.z - p_j.z) * n_j.z : (nb.rlo.z - p_j.z) * n_j.z);
    bool hl = ml > lim, hr = mr > lim;
    if (cut2 >= 0.f) {   // boxes are around triangles, centroids lie inside them
      hl = hl && box_dist2(p_j, nb.llo, nb.lhi) <= box_cut2;
      hr = hr && box_dist2(p_j, nb.rlo, nb.rhi) <= box_cut2;
    }
    if (hl && hr) {
      if (sp == TRACE_STACK) { atomicExch(&derr[DERR_STACK], 1); break; }
      stack[sp++] = nb.right;
      node = nb.left;
    } else if (hl) {
      node = nb.left;
    } else if (hr) {
      node = nb.right;
    } else {
      if (sp == 0) break;
      node = stack[--sp];
    }
  }
  if (!FILL) count[t] = cnt;
}

// One visibility ray per candidate pair (src/cpp/illum.cpp:72-83): from the
// offset centroid q_j towards p_i. A ray that hits a facet h other than j
// yields the key (h << bits) | j. Consecutive pairs share their source, so a
// warp's keys repeat (rays stopped by the same occluder): each distinct key
// of a warp is appended once to ukeys (one atomic per warp); the order of
// ukeys is irrelevant, it is sorted and made unique afterwards. The launch
// covers whole warps (no early exit before the warp-wide vote).
__global__ void k_vis_rays(const float4* __restrict__ nodes, const float4* __restrict__ tri_s, int root,
                           const float4* __restrict__ cen, const float4* __restrict__ nrm, int64_t npairs,
                           const int32_t* __restrict__ cand_i, const int32_t* __restrict__ cand_j, float offset,
                           int bits, unsigned long long* ukeys, unsigned long long* ucount, int* derr) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned long long NONE = ~0ull;
  unsigned long long key = NONE;
  if (k < npairs) {
    int i = cand_i[k], j = cand_j[k];
    f3 p_j = f3of(cen[j]), n_j = f3of(nrm[j]);
    f3 q_j = add(p_j, scl(n_j, offset));
    f3 d = normalize(sub(f3of(cen[i]), q_j));
    int h = trace_closest(nodes, tri_s, root, q_j, d, nullptr, &derr[DERR_STACK]);
    if (h >= 0 && h != j) key = ((unsigned long long)h << bits) | (unsigned long long)j;
  }
  const int lane = threadIdx.x & 31;
  unsigned same = __match_any_sync(0xffffffffu, key);
  bool lead = key != NONE && (__ffs(same) - 1) == lane;
  unsigned vote = __ballot_sync(0xffffffffu, lead);
  unsigned long long base = 0;
  if (lane == 0 && vote) base = atomicAdd(ucount, (unsigned long long)__popc(vote));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (lead) ukeys[base + __popc(vote & ((1u << lane) - 1u))] = key;
}

// After sorting: first occurrence of each (row, col) -> form factor
// (src/cpp/illum.cpp:100-130), albedo row scale (:225-234); zeros dropped.
__global__ void k_ff_values(const unsigned long long* __restrict__ keys, int64_t n, int bits, int nt,
                            const float4* __restrict__ cen, const float4* __restrict__ nrm,
                            const double* __restrict__ area, const double* __restrict__ albedo, double albedo_scalar,
                            uint32_t* keep, double* fval, int* derr) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  unsigned long long key = keys[k];
  unsigned long long mask = (1ull << bits) - 1ull;
  int i = (int)(key >> bits), j = (int)(key & mask);
  uint32_t kp = 0;
  double F = 0.0;
  if (k == 0 || keys[k - 1] != key) {
    F = form_factor(f3of(cen[i]), f3of(nrm[i]), f3of(cen[j]), f3of(nrm[j]), area[j]);
    if (isnan(F)) {
      atomicExch(&derr[DERR_NAN], 1);
    } else if (F != 0.0) {
      double rho = albedo ? albedo[i] : albedo_scalar;
      F = F * rho;
      kp = 1;
    }
  }
  keep[k] = kp;
  fval[k] = F;
}

// Sampled visibility: every distinct (hit i, source j) key with a nonzero
// form factor counts for its source's sample slot, and for every radius its
// centroid distance does not exceed.
__global__ void k_sample_count(const unsigned long long* __restrict__ keys, int64_t n, int bits,
                               const float4* __restrict__ cen, const float4* __restrict__ nrm,
                               const double* __restrict__ area, const int* __restrict__ slot,
                               const double* __restrict__ radii, int nradii, unsigned long long* per_src,
                               unsigned long long* within) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const unsigned long long key = keys[k];
  if (k > 0 && keys[k - 1] == key) return;
  const unsigned long long mask = (1ull << bits) - 1ull;
  const int i = (int)(key >> bits), j = (int)(key & mask);
  const double F = form_factor(f3of(cen[i]), f3of(nrm[i]), f3of(cen[j]), f3of(nrm[j]), area[j]);
  if (!(F > 0.0)) return;
  atomicAdd(&per_src[slot[j]], 1ull);
  const float4 a = cen[i], b = cen[j];
  const double dx = (double)a.x - b.x, dy = (double)a.y - b.y, dz = (double)a.z - b.z;
  const double d = sqrt(dx * dx + dy * dy + dz * dz);
  for (int q = 0; q < nradii; ++q)
    if (d <= radii[q]) atomicAdd(&within[q], 1ull);
}

__global__ void k_ff_compact(const unsigned long long* __restrict__ keys, int64_t n, int bits,
                             const uint32_t* __restrict__ keep, const unsigned long long* __restrict__ pos,
                             const double* __restrict__ fval, int32_t* rows, int32_t* col, double* val) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n || !keep[k]) return;
  unsigned long long key = keys[k];
  int64_t p = (int64_t)pos[k];
  rows[p] = (int32_t)(key >> bits);
  col[p] = (int32_t)(key & ((1ull << bits) - 1ull));
  val[p] = fval[k];
}

// A chunk's kept entries (first occurrence, nonzero form factor): key and
// value at their scan position.
__global__ void k_ff_pack(const unsigned long long* __restrict__ keys, int64_t n, const uint32_t* __restrict__ keep,
                          const unsigned long long* __restrict__ pos, const double* __restrict__ fval,
                          unsigned long long* okey, double* oval) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n || !keep[k]) return;
  const int64_t p = (int64_t)pos[k];
  okey[p] = keys[k];
  oval[p] = fval[k];
}

// The entries in (row, column) order: row and column from the sorted key,
// the value through the sort's permutation (idx == nullptr: no
// permutation).
__global__ void k_ff_unpack(const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ idx,
                            const double* __restrict__ vals, int64_t n, int bits, int32_t* rows, int32_t* col,
                            double* val) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const unsigned long long key = keys[k];
  rows[k] = (int32_t)(key >> bits);
  col[k] = (int32_t)(key & ((1ull << bits) - 1ull));
  val[k] = vals[idx ? idx[k] : k];
}

__global__ void k_iota_u32(uint32_t* a, int64_t n) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) a[k] = (uint32_t)k;
}

__global__ void k_rowptr(const int32_t* __restrict__ rows, int64_t nnz, int nt, int64_t* rowptr) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > nt) return;
  int64_t lo = 0, hi = nnz;   // first index with rows[idx] >= r
  while (lo < hi) {
    int64_t m = (lo + hi) >> 1;
    if (rows[m] < r) lo = m + 1; else hi = m;
  }
  rowptr[r] = lo;
}

}  // namespace

// ====================================================================== host

int bvh_build(Context& c, const float* verts_h, int nv, const int32_t* tris_h, const float* normals_h) {
  int nt = c.nt;
  cudaStream_t s = c.stream;
  // scene bounds and magnitude (host)
  float lo[3] = {3e38f, 3e38f, 3e38f}, hi[3] = {-3e38f, -3e38f, -3e38f};
  float mag = 0.f;
  for (int v = 0; v < nv; ++v)
    for (int a = 0; a < 3; ++a) {
      float x = verts_h[3 * v + a];
      if (!(x == x) || std::isinf(x)) { set_error("vertex %d has a non-finite coordinate", v); return ILG_ERR_ARG; }
      lo[a] = std::min(lo[a], x); hi[a] = std::max(hi[a], x); mag = std::max(mag, std::fabs(x));
    }
  for (int t = 0; t < 3 * nt; ++t)
    if (tris_h[t] < 0 || tris_h[t] >= nv) { set_error("triangle %d has vertex index %d out of range", t / 3, tris_h[t]); return ILG_ERR_ARG; }
  c.scene_mag = mag > 0.f ? mag : 1.f;

  dbuf<float> dverts, dnormals;
  dbuf<int32_t> dtris;
  ILG_TRY(dverts.alloc((size_t)nv * 3));
  ILG_TRY(dtris.alloc((size_t)nt * 3));
  ILG_CUDA(cudaMemcpyAsync(dverts.p, verts_h, (size_t)nv * 12, cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemcpyAsync(dtris.p, tris_h, (size_t)nt * 12, cudaMemcpyHostToDevice, s));
  if (normals_h) {
    ILG_TRY(dnormals.alloc((size_t)nt * 3));
    ILG_CUDA(cudaMemcpyAsync(dnormals.p, normals_h, (size_t)nt * 12, cudaMemcpyHostToDevice, s));
  }
  ILG_TRY(c.tri_o.alloc((size_t)nt * 3));
  ILG_TRY(c.cen.alloc(nt));
  ILG_TRY(c.nrm.alloc(nt));
  ILG_TRY(c.area.alloc(nt));
  ILG_TRY(c.frame.alloc((size_t)nt * 9));
  ILG_TRY(c.frame32.alloc((size_t)nt * 3));
  k_prepare<<<div_up(nt, 256), 256, 0, s>>>(dverts.p, dtris.p, dnormals.p, nt, c.tri_o.p, c.cen.p, c.nrm.p,
                                            c.area.p, c.frame.p, c.frame32.p);
  ILG_CUDA(cudaGetLastError());

  // r_max on the host copy of the radii
  std::vector<float4> cen_h(nt);
  ILG_CUDA(cudaMemcpyAsync(cen_h.data(), c.cen.p, (size_t)nt * 16, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  float rmax = 0.f;
  for (int t = 0; t < nt; ++t) rmax = std::max(rmax, cen_h[t].w);
  c.r_max = rmax;

  dbuf<unsigned long long> keys;
  dbuf<uint32_t>& order = c.morton_order;   // kept: facets in Morton order
  ILG_TRY(keys.alloc(nt));
  ILG_TRY(order.alloc(nt));
  float3 blo = make_float3(lo[0], lo[1], lo[2]);
  float3 inv = make_float3(hi[0] > lo[0] ? 1.f / (hi[0] - lo[0]) : 0.f, hi[1] > lo[1] ? 1.f / (hi[1] - lo[1]) : 0.f,
                           hi[2] > lo[2] ? 1.f / (hi[2] - lo[2]) : 0.f);
  k_morton<<<div_up(nt, 256), 256, 0, s>>>(c.cen.p, nt, blo, inv, keys.p, order.p);
  ILG_CUDA(cudaGetLastError());
  ILG_TRY(radix_sort_u64(keys.p, order.p, nt, 63, c.sort, s));

  dbuf<int2> child;
  dbuf<int> parent, flags, depth;
  dbuf<float4> box_lo, box_hi;
  int ni = nt > 1 ? nt - 1 : 1;
  ILG_TRY(child.alloc(ni));
  ILG_TRY(parent.alloc((size_t)2 * nt));
  ILG_TRY(flags.alloc(ni));
  ILG_TRY(depth.alloc(1));
  ILG_TRY(box_lo.alloc((size_t)2 * nt));
  ILG_TRY(box_hi.alloc((size_t)2 * nt));
  ILG_TRY(c.tri_s.alloc((size_t)nt * 3));
  ILG_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int) * ni, s));
  ILG_CUDA(cudaMemsetAsync(depth.p, 0, sizeof(int), s));
  ILG_CUDA(cudaMemsetAsync(parent.p, 0xff, sizeof(int) * 2 * nt, s));   // -1: root has no parent
  if (nt > 1) {
    k_karras<<<div_up(nt - 1, 256), 256, 0, s>>>(keys.p, nt, child.p, parent.p);
    ILG_CUDA(cudaGetLastError());
  }
  float pad = 1e-6f * c.scene_mag;
  k_refit<<<div_up(nt, 256), 256, 0, s>>>(c.tri_o.p, order.p, nt, child.p, parent.p, box_lo.p, box_hi.p, flags.p,
                                          pad, c.tri_s.p, depth.p);
  ILG_CUDA(cudaGetLastError());
  if (nt > 1) {
    ILG_TRY(c.nodes.alloc((size_t)(nt - 1) * 4));
    k_pack_nodes<<<div_up(nt - 1, 256), 256, 0, s>>>(child.p, box_lo.p, box_hi.p, nt, c.nodes.p);
    ILG_CUDA(cudaGetLastError());
    c.root = 0;
  } else {
    ILG_TRY(c.nodes.alloc(4));
    c.root = ~0;
  }
  int dh = 0;
  ILG_CUDA(cudaMemcpyAsync(&dh, depth.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  c.bvh_depth = dh;
  c.bvh_nodes = nt > 1 ? 2LL * nt - 1 : 1;
  if (dh + 2 > TRACE_STACK) {
    set_error("LBVH depth %d exceeds the traversal stack (%d)", dh, TRACE_STACK);
    return ILG_ERR_DEVICE;
  }
  return ILG_OK;
}

int bvh_trace(Context& c, int nrays, const float* orig_h, const float* dir_h, int any_hit, int32_t* hit_h,
              double* t_h) {
  if (nrays <= 0) return ILG_OK;
  cudaStream_t s = c.stream;
  dbuf<float> o, d;
  dbuf<int32_t> h;
  dbuf<double> t;
  ILG_TRY(o.alloc((size_t)nrays * 3));
  ILG_TRY(d.alloc((size_t)nrays * 3));
  ILG_TRY(h.alloc(nrays));
  ILG_TRY(t.alloc(nrays));
  ILG_CUDA(cudaMemcpyAsync(o.p, orig_h, (size_t)nrays * 12, cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemcpyAsync(d.p, dir_h, (size_t)nrays * 12, cudaMemcpyHostToDevice, s));
  k_trace<<<div_up(nrays, 128), 128, 0, s>>>(c.nodes.p, c.tri_s.p, c.root, nrays, o.p, d.p, any_hit, h.p, t.p,
                                             c.derr.p);
  ILG_CUDA(cudaGetLastError());
  ILG_CUDA(cudaMemcpyAsync(hit_h, h.p, (size_t)nrays * 4, cudaMemcpyDeviceToHost, s));
  if (t_h) ILG_CUDA(cudaMemcpyAsync(t_h, t.p, (size_t)nrays * 8, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  return read_device_errors(c);
}

int bvh_render(Context& c, int mode, double az_deg, double el_deg, int width, int height, int32_t* out_h) {
  cudaStream_t s = c.stream;
  std::vector<float4> cen((size_t)c.nt);
  ILG_CUDA(cudaMemcpyAsync(cen.data(), c.cen.p, (size_t)c.nt * sizeof(float4), cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  double mx = 0, my = 0, mz = 0;
  for (const float4& q : cen) { mx += q.x; my += q.y; mz += q.z; }
  mx /= c.nt; my /= c.nt; mz /= c.nt;
  double r_model = 0;
  for (const float4& q : cen)
    r_model = std::max(r_model, std::sqrt((q.x - mx) * (q.x - mx) + (q.y - my) * (q.y - my) + (q.z - mz) * (q.z - mz)));
  RenderCam cam{};
  cam.mode = mode; cam.width = width; cam.height = height;
  cam.rad = 1.1 * r_model;
  cam.aspect = (double)width / height;
  const double D2R = 3.141592653589793 / 180.0;
  cam.az = az_deg * D2R;
  cam.el = el_deg * D2R;
  cam.cx = (float)mx; cam.cy = (float)my; cam.cz = (float)mz;
  if (mode == 0) {
    auto sph = [](double phi, double theta, double r, float* v) {
      v[0] = (float)(r * std::cos(phi) * std::sin(theta));
      v[1] = (float)(r * std::sin(phi) * std::sin(theta));
      v[2] = (float)(r * std::cos(theta));
    };
    float p[3], up[3];
    sph(cam.az, cam.el, cam.rad, p);
    sph(cam.az, cam.el - 3.141592653589793 / 2, 1.0, up);
    float pl = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    float e[3] = {-p[0] / pl, -p[1] / pl, -p[2] / pl};
    cam.ex = e[0]; cam.ey = e[1]; cam.ez = e[2];
    cam.ux = up[0]; cam.uy = up[1]; cam.uz = up[2];
    cam.rx = e[1] * up[2] - e[2] * up[1];   // n_eye x n_up
    cam.ry = e[2] * up[0] - e[0] * up[2];
    cam.rz = e[0] * up[1] - e[1] * up[0];
    cam.px = p[0] + cam.cx; cam.py = p[1] + cam.cy; cam.pz = p[2] + cam.cz;
  }
  const int64_t npx = (int64_t)width * height;
  dbuf<int32_t> dout;
  ILG_TRY(dout.alloc(npx));
  k_render<<<div_up(npx, 128), 128, 0, s>>>(c.nodes.p, c.tri_s.p, c.root, cam, dout.p, c.derr.p);
  ILG_CUDA(cudaGetLastError());
  ILG_CUDA(cudaMemcpyAsync(out_h, dout.p, (size_t)npx * 4, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  return read_device_errors(c);
}

// Bisection tree of src/cpp/illum.cpp:304-316 for a given theta_eps, in heap
// order (root 1, hit child 2k, miss child 2k+1). Node values are produced by
// exactly the reference's double arithmetic, so the returned mid values are
// the reference's.
static int build_horizon_tree(double theta_eps, std::vector<HorizonNode>& tree) {
  const int MAXD = 20;
  tree.assign(2, HorizonNode{0, 0, 0, 0, 0});
  struct St { double lo, hi, mid; };
  std::vector<St> st(2);
  st[1] = St{0.0, PI, PI / 2.0};
  tree[1].mid = PI / 2.0;
  tree[1].terminal = 0;
  sincos_x(tree[1].mid, &tree[1].s, &tree[1].c);
  for (int depth = 0; depth < MAXD; ++depth) {
    size_t b = (size_t)1 << depth, e = (size_t)1 << (depth + 1);
    bool any = false;
    tree.resize(2 * e);
    st.resize(2 * e);
    for (size_t k = b; k < e; ++k) {
      if (tree[k].terminal || (k > 1 && tree[k].pad)) {   // pad marks unreachable
        tree[2 * k] = HorizonNode{0, 0, 0, 1, 1};
        tree[2 * k + 1] = HorizonNode{0, 0, 0, 1, 1};
        continue;
      }
      any = true;
      St cur = st[k];
      for (int h = 0; h < 2; ++h) {
        double lo = cur.lo, hi = cur.hi;
        if (h == 0) hi = cur.mid; else lo = cur.mid;
        double mid = (lo + hi) / 2.0;
        HorizonNode nd;
        nd.mid = mid;
        sincos_x(mid, &nd.s, &nd.c);
        nd.terminal = std::fabs(mid - cur.mid) > theta_eps ? 0 : 1;
        nd.pad = 0;
        tree[2 * k + h] = nd;
        st[2 * k + h] = St{lo, hi, mid};
      }
    }
    if (!any) { tree.resize(e); return ILG_OK; }
  }
  for (size_t k = (size_t)1 << MAXD; k < tree.size(); ++k)
    if (!tree[k].terminal) {
      set_error("theta_eps %g needs more than %d bisection levels", theta_eps, MAXD);
      return ILG_ERR_ARG;
    }
  return ILG_OK;
}

int horizons_build(Context& c, int nphi, double theta_eps, double offset, const Context* hmesh) {
  if (nphi < 2) { set_error("nphi must be >= 2"); return ILG_ERR_ARG; }
  if (!(theta_eps > 0.0)) { set_error("theta_eps must be > 0"); return ILG_ERR_ARG; }
  cudaStream_t s = c.stream;
  std::vector<HorizonNode> tree;
  ILG_TRY(build_horizon_tree(theta_eps, tree));
  std::vector<double> cph(nphi), sph(nphi);
  double dphi = TWO_PI / (double)(nphi - 1);
  for (int k = 0; k < nphi; ++k) {
    double ph = (k == nphi - 1) ? TWO_PI : (double)k * dphi;   // arma::linspace
    sincos_x(ph, &sph[k], &cph[k]);
  }
  dbuf<HorizonNode> dtree;
  dbuf<double> dc, ds;
  ILG_TRY(dtree.alloc(tree.size()));
  ILG_TRY(dc.alloc(nphi));
  ILG_TRY(ds.alloc(nphi));
  ILG_CUDA(cudaMemcpyAsync(dtree.p, tree.data(), tree.size() * sizeof(HorizonNode), cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemcpyAsync(dc.p, cph.data(), nphi * 8, cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemcpyAsync(ds.p, sph.data(), nphi * 8, cudaMemcpyHostToDevice, s));
  ILG_TRY(c.H.alloc((size_t)c.nt * nphi));
  int64_t total = (int64_t)c.nt * nphi;
  // the rays of a separate horizon mesh's facets-independent BVH, or the
  // context's own (src/cpp/illum.cpp:333-360)
  const Context& hb = hmesh ? *hmesh : c;
  k_horizons<<<div_up(total, 128), 128, 0, s>>>(hb.nodes.p, hb.tri_s.p, hb.root, c.tri_o.p, c.cen.p, c.nrm.p, c.nt,
                                                nphi, dc.p, ds.p, dtree.p, (int)tree.size(), (float)offset, c.H.p,
                                                c.derr.p);
  ILG_CUDA(cudaGetLastError());
  c.nphi = nphi;
  c.dphi = dphi;
  ILG_TRY(horizons_f32(c));
  return read_device_errors(c);
}

int horizons_f32(Context& c) {
  ILG_TRY(c.H32.alloc((size_t)c.nt * c.nphi));
  ILG_TRY(c.hmm32.alloc(c.nt));
  k_horizon_f32<<<div_up(c.nt, 256), 256, 0, c.stream>>>(c.H.p, c.nt, c.nphi, c.H32.p, c.hmm32.p);
  ILG_CUDA(cudaGetLastError());
  ILG_CUDA(cudaStreamSynchronize(c.stream));
  return ILG_OK;
}

// Candidate pairs held on the device at once (8 bytes each).
constexpr int64_t FF_CHUNK = int64_t(1) << 29;
// The chunk size in force (a test entry may lower it to exercise the
// several-chunk path on a small mesh).
std::atomic<int64_t> g_ff_chunk{FF_CHUNK};

int ff_set_chunk(int64_t pairs) {
  g_ff_chunk.store(pairs > 0 ? pairs : FF_CHUNK);
  return ILG_OK;
}

int form_factors_build(Context& c, const double* albedo_h, double albedo_scalar, double offset, double cutoff,
                       int64_t* rays_out) {
  cudaStream_t s = c.stream;
  int nt = c.nt;
  dbuf<uint32_t> cnt;
  dbuf<unsigned long long> offs;
  ILG_TRY(cnt.alloc((size_t)nt * FF_SPLIT));
  ILG_TRY(offs.alloc((size_t)nt * FF_SPLIT));
  float slack = 1e-5f * c.scene_mag;
  const float cut2 = cutoff > 0.0 ? (float)(cutoff * cutoff) : -1.0f;
  // box test: the squared distance to a box is computed in float with at
  // most a few ulps of error; the margin keeps every centroid within the
  // cutoff reachable
  const float box_cut2 = cutoff > 0.0 ? (float)((cutoff + 1e-5 * c.scene_mag) * (cutoff + 1e-5 * c.scene_mag)) * 1.0001f
                                      : -1.0f;
  const int64_t nitems = (int64_t)nt * FF_SPLIT;
  dbuf<int> front;
  ILG_TRY(front.alloc(FF_SPLIT + 1));
  k_frontier<<<1, 1, 0, s>>>(c.nodes.p, c.root, front.p, front.p + FF_SPLIT);
  ILG_CUDA(cudaGetLastError());
  k_candidates<false><<<div_up(nitems, 128), 128, 0, s>>>(c.nodes.p, c.tri_s.p, front.p, front.p + FF_SPLIT, c.cen.p,
                                                          c.nrm.p, 0, nt, nullptr, c.r_max, slack, cut2, box_cut2,
                                                          cnt.p, nullptr, 0ull, nullptr, nullptr, c.derr.p);
  ILG_CUDA(cudaGetLastError());
  ILG_TRY(scan_exclusive_u32_to_u64(cnt.p, offs.p, nitems, c.scan, s));
  // per-source offsets: every FF_SPLIT-th item offset, and the total
  std::vector<unsigned long long> offs_h((size_t)nt + 1);
  uint32_t last_cnt = 0;
  unsigned long long last_off = 0;
  ILG_CUDA(cudaMemcpy2DAsync(offs_h.data(), 8, offs.p, 8 * FF_SPLIT, 8, nt, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaMemcpyAsync(&last_off, offs.p + (nitems - 1), 8, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaMemcpyAsync(&last_cnt, cnt.p + (nitems - 1), 4, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  offs_h[nt] = last_off + last_cnt;
  const int64_t npairs = (int64_t)offs_h[nt];
  if (rays_out) *rays_out = npairs;
  int bits = 1;
  while ((1LL << bits) < nt) ++bits;   // row and column fields

  // Sources in chunks of at most FF_CHUNK pairs (a source with more pairs is
  // a chunk of its own): candidate pairs exist for one chunk at a time.
  const int64_t chunk = g_ff_chunk.load();
  std::vector<int> cut{0};
  int64_t cap = 1;
  while (cut.back() < nt) {
    int a = cut.back(), b = a + 1;
    while (b < nt && (int64_t)(offs_h[b + 1] - offs_h[a]) <= chunk) ++b;
    cap = std::max<int64_t>(cap, (int64_t)(offs_h[b] - offs_h[a]));
    cut.push_back(b);
  }
  c.have_F = false;
  c.gs_ready = false;
  c.ntiles = 0;
  // Per chunk: its rays' distinct hit keys (sorted), their form factors, and
  // the kept entries (first occurrence, nonzero) packed into the chunk's own
  // arrays. Chunks own disjoint sources, so no key repeats across chunks and
  // only the kept entries outlive their chunk.
  std::vector<dbuf<unsigned long long>> ck;
  std::vector<dbuf<double>> cv;
  std::vector<int64_t> cn;
  {
    dbuf<int32_t> ci, cj;
    dbuf<unsigned long long> ukeys, ucount, pos;
    dbuf<uint32_t> keep;
    dbuf<double> fval, alb;
    ILG_TRY(ci.alloc(cap));
    ILG_TRY(cj.alloc(cap));
    ILG_TRY(ukeys.alloc(cap));
    ILG_TRY(keep.alloc(cap));
    ILG_TRY(fval.alloc(cap));
    ILG_TRY(pos.alloc(cap));
    ILG_TRY(ucount.alloc(1));
    if (albedo_h) {
      ILG_TRY(alb.alloc(nt));
      ILG_CUDA(cudaMemcpyAsync(alb.p, albedo_h, (size_t)nt * 8, cudaMemcpyHostToDevice, s));
    }
    for (size_t q = 0; q + 1 < cut.size(); ++q) {
      const int a = cut[q], b = cut[q + 1];
      const int64_t np = (int64_t)(offs_h[b] - offs_h[a]);
      if (np == 0) continue;
      ILG_CUDA(cudaMemsetAsync(ucount.p, 0, 8, s));
      k_candidates<true><<<div_up((int64_t)(b - a) * FF_SPLIT, 128), 128, 0, s>>>(
          c.nodes.p, c.tri_s.p, front.p, front.p + FF_SPLIT, c.cen.p, c.nrm.p, a, b, nullptr, c.r_max, slack, cut2,
          box_cut2, nullptr, offs.p + (size_t)a * FF_SPLIT, offs_h[a], ci.p, cj.p, c.derr.p);
      ILG_CUDA(cudaGetLastError());
      k_vis_rays<<<div_up(np, 128), 128, 0, s>>>(c.nodes.p, c.tri_s.p, c.root, c.cen.p, c.nrm.p, np, ci.p, cj.p,
                                                 (float)offset, bits, ukeys.p, ucount.p, c.derr.p);
      ILG_CUDA(cudaGetLastError());
      unsigned long long nk = 0;
      ILG_CUDA(cudaMemcpyAsync(&nk, ucount.p, 8, cudaMemcpyDeviceToHost, s));
      ILG_CUDA(cudaStreamSynchronize(s));
      if (nk == 0) continue;
      if (nk > 1) ILG_TRY(radix_sort_u64(ukeys.p, nullptr, (int64_t)nk, 2 * bits, c.sort, s));
      k_ff_values<<<div_up((int64_t)nk, 256), 256, 0, s>>>(ukeys.p, (int64_t)nk, bits, nt, c.cen.p, c.nrm.p,
                                                          c.area.p, alb.p, albedo_scalar, keep.p, fval.p, c.derr.p);
      ILG_CUDA(cudaGetLastError());
      ILG_TRY(scan_exclusive_u32_to_u64(keep.p, pos.p, (int64_t)nk, c.scan, s));
      unsigned long long lp = 0;
      uint32_t lk = 0;
      ILG_CUDA(cudaMemcpyAsync(&lp, pos.p + (nk - 1), 8, cudaMemcpyDeviceToHost, s));
      ILG_CUDA(cudaMemcpyAsync(&lk, keep.p + (nk - 1), 4, cudaMemcpyDeviceToHost, s));
      ILG_CUDA(cudaStreamSynchronize(s));
      const int64_t nkeep = (int64_t)lp + lk;
      if (nkeep == 0) continue;
      ck.emplace_back();
      cv.emplace_back();
      ILG_TRY(ck.back().alloc(nkeep));
      ILG_TRY(cv.back().alloc(nkeep));
      cn.push_back(nkeep);
      k_ff_pack<<<div_up((int64_t)nk, 256), 256, 0, s>>>(ukeys.p, (int64_t)nk, keep.p, pos.p, fval.p,
                                                         ck.back().p, cv.back().p);
      ILG_CUDA(cudaGetLastError());
    }
  }
  int64_t nnz = 0;
  for (int64_t x : cn) nnz += x;
  if (nnz > (int64_t)0xffffffffLL) { set_error("%lld form-factor entries exceed the 32-bit entry index", (long long)nnz); return ILG_ERR_ARG; }
  ILG_TRY(read_device_errors(c));
  // all entries in (row, column) order: one chunk is sorted already; several
  // are concatenated and sorted by key, the values following the permutation
  dbuf<int32_t> rows;
  auto alloc_csr = [&]() -> int {
    ILG_TRY(rows.alloc(nnz > 0 ? nnz : 1));
    ILG_TRY(c.col.alloc(nnz > 0 ? nnz : 1));
    ILG_TRY(c.val.alloc(nnz > 0 ? nnz : 1));
    return ILG_OK;
  };
  ILG_TRY(c.rowptr.alloc((size_t)nt + 1));
  if (ck.size() <= 1) ILG_TRY(alloc_csr());
  if (ck.size() == 1) {
    k_ff_unpack<<<div_up(nnz, 256), 256, 0, s>>>(ck[0].p, nullptr, cv[0].p, nnz, bits, rows.p, c.col.p, c.val.p);
    ILG_CUDA(cudaGetLastError());
    ck.clear();
    cv.clear();
  } else if (ck.size() > 1) {
    dbuf<unsigned long long> ekeys;
    dbuf<double> evals;
    dbuf<uint32_t> eidx;
    ILG_TRY(ekeys.alloc(nnz));
    ILG_TRY(evals.alloc(nnz));
    int64_t off = 0;
    for (size_t q = 0; q < ck.size(); ++q) {
      ILG_CUDA(cudaMemcpyAsync(ekeys.p + off, ck[q].p, (size_t)cn[q] * 8, cudaMemcpyDeviceToDevice, s));
      ILG_CUDA(cudaMemcpyAsync(evals.p + off, cv[q].p, (size_t)cn[q] * 8, cudaMemcpyDeviceToDevice, s));
      off += cn[q];
      ck[q].release();
      cv[q].release();
    }
    ck.clear();
    cv.clear();
    ILG_TRY(eidx.alloc(nnz));
    k_iota_u32<<<div_up(nnz, 256), 256, 0, s>>>(eidx.p, nnz);
    ILG_CUDA(cudaGetLastError());
    ILG_TRY(radix_sort_u64(ekeys.p, eidx.p, nnz, 2 * bits, c.sort, s));
    c.sort.release();
    ILG_TRY(alloc_csr());
    k_ff_unpack<<<div_up(nnz, 256), 256, 0, s>>>(ekeys.p, eidx.p, evals.p, nnz, bits, rows.p, c.col.p, c.val.p);
    ILG_CUDA(cudaGetLastError());
  }
  k_rowptr<<<div_up(nt + 1, 256), 256, 0, s>>>(rows.p, nnz, nt, c.rowptr.p);
  ILG_CUDA(cudaGetLastError());
  ILG_CUDA(cudaStreamSynchronize(s));
  c.nnz = nnz;
  c.have_F = true;
  rows.release();
  ILG_TRY(radiosity_prepare(c));
  // the sort and scan scratch grew to the entry count: not kept resident
  c.sort.release();
  c.scan.release();
  if (nnz > (int64_t(1) << 26)) ILG_TRY(pool_trim(s));
  return read_device_errors(c);
}

int visibility_sample(Context& c, double cutoff, double offset, const int* src_h, int nsrc, const double* radii_h,
                      int nradii, int64_t* per_src_h, int64_t* within_h, int64_t* rays_out) {
  if (nsrc < 1 || !src_h || nradii < 0 || (nradii > 0 && !radii_h)) { set_error("invalid sample"); return ILG_ERR_ARG; }
  cudaStream_t s = c.stream;
  const int nt = c.nt;
  std::vector<int> slot_h((size_t)nt, -1);
  for (int q = 0; q < nsrc; ++q) {
    if (src_h[q] < 0 || src_h[q] >= nt) { set_error("source %d out of range", src_h[q]); return ILG_ERR_ARG; }
    if (slot_h[src_h[q]] >= 0) { set_error("source %d listed twice", src_h[q]); return ILG_ERR_ARG; }
    slot_h[src_h[q]] = q;
  }
  dbuf<int> dsrc, dslot, front;
  dbuf<double> dradii;
  dbuf<unsigned long long> per_src, within, offs, ukeys, ucount;
  dbuf<uint32_t> cnt;
  ILG_TRY(dsrc.alloc(nsrc));
  ILG_TRY(dslot.alloc(nt));
  ILG_TRY(dradii.alloc(std::max(nradii, 1)));
  ILG_TRY(per_src.alloc(nsrc));
  ILG_TRY(within.alloc(std::max(nradii, 1)));
  ILG_TRY(front.alloc(FF_SPLIT + 1));
  const int64_t nitems = (int64_t)nsrc * FF_SPLIT;
  ILG_TRY(cnt.alloc(nitems));
  ILG_TRY(offs.alloc(nitems));
  ILG_TRY(ucount.alloc(1));
  ILG_CUDA(cudaMemcpyAsync(dsrc.p, src_h, (size_t)nsrc * 4, cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemcpyAsync(dslot.p, slot_h.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, s));
  if (nradii > 0) ILG_CUDA(cudaMemcpyAsync(dradii.p, radii_h, (size_t)nradii * 8, cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemsetAsync(per_src.p, 0, (size_t)nsrc * 8, s));
  ILG_CUDA(cudaMemsetAsync(within.p, 0, (size_t)std::max(nradii, 1) * 8, s));
  ILG_CUDA(cudaMemsetAsync(ucount.p, 0, 8, s));
  const float slack = 1e-5f * c.scene_mag;
  const float cut2 = cutoff > 0.0 ? (float)(cutoff * cutoff) : -1.0f;
  const float box_cut2 = cutoff > 0.0 ? (float)((cutoff + 1e-5 * c.scene_mag) * (cutoff + 1e-5 * c.scene_mag)) * 1.0001f
                                      : -1.0f;
  k_frontier<<<1, 1, 0, s>>>(c.nodes.p, c.root, front.p, front.p + FF_SPLIT);
  k_candidates<false><<<div_up(nitems, 128), 128, 0, s>>>(c.nodes.p, c.tri_s.p, front.p, front.p + FF_SPLIT, c.cen.p,
                                                          c.nrm.p, 0, nsrc, dsrc.p, c.r_max, slack, cut2, box_cut2,
                                                          cnt.p, nullptr, 0ull, nullptr, nullptr, c.derr.p);
  ILG_CUDA(cudaGetLastError());
  ILG_TRY(scan_exclusive_u32_to_u64(cnt.p, offs.p, nitems, c.scan, s));
  std::vector<unsigned long long> offs_h((size_t)nsrc + 1);
  uint32_t last_cnt = 0;
  unsigned long long last_off = 0;
  ILG_CUDA(cudaMemcpy2DAsync(offs_h.data(), 8, offs.p, 8 * FF_SPLIT, 8, nsrc, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaMemcpyAsync(&last_off, offs.p + (nitems - 1), 8, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaMemcpyAsync(&last_cnt, cnt.p + (nitems - 1), 4, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  offs_h[nsrc] = last_off + last_cnt;
  if (rays_out) *rays_out = (int64_t)offs_h[nsrc];
  int bits = 1;
  while ((1LL << bits) < nt) ++bits;
  // chunks of at most FF_CHUNK candidate pairs; each chunk's distinct hit
  // keys are sorted, counted and dropped (the sample's keys never coexist)
  std::vector<int> cutq{0};
  int64_t cap = 1;
  while (cutq.back() < nsrc) {
    int a = cutq.back(), b = a + 1;
    while (b < nsrc && (int64_t)(offs_h[b + 1] - offs_h[a]) <= FF_CHUNK) ++b;
    cap = std::max<int64_t>(cap, (int64_t)(offs_h[b] - offs_h[a]));
    cutq.push_back(b);
  }
  dbuf<int32_t> ci, cj;
  ILG_TRY(ci.alloc(cap));
  ILG_TRY(cj.alloc(cap));
  ILG_TRY(ukeys.alloc(cap));
  for (size_t q = 0; q + 1 < cutq.size(); ++q) {
    const int a = cutq[q], b = cutq[q + 1];
    const int64_t np = (int64_t)(offs_h[b] - offs_h[a]);
    if (np == 0) continue;
    ILG_CUDA(cudaMemsetAsync(ucount.p, 0, 8, s));
    k_candidates<true><<<div_up((int64_t)(b - a) * FF_SPLIT, 128), 128, 0, s>>>(
        c.nodes.p, c.tri_s.p, front.p, front.p + FF_SPLIT, c.cen.p, c.nrm.p, a, b, dsrc.p, c.r_max, slack, cut2,
        box_cut2, nullptr, offs.p + (size_t)a * FF_SPLIT, offs_h[a], ci.p, cj.p, c.derr.p);
    ILG_CUDA(cudaGetLastError());
    k_vis_rays<<<div_up(np, 128), 128, 0, s>>>(c.nodes.p, c.tri_s.p, c.root, c.cen.p, c.nrm.p, np, ci.p, cj.p,
                                               (float)offset, bits, ukeys.p, ucount.p, c.derr.p);
    ILG_CUDA(cudaGetLastError());
    unsigned long long nk = 0;
    ILG_CUDA(cudaMemcpyAsync(&nk, ucount.p, 8, cudaMemcpyDeviceToHost, s));
    ILG_CUDA(cudaStreamSynchronize(s));
    if (nk > 1) ILG_TRY(radix_sort_u64(ukeys.p, nullptr, (int64_t)nk, 2 * bits, c.sort, s));
    if (nk > 0) {
      k_sample_count<<<div_up((int64_t)nk, 256), 256, 0, s>>>(ukeys.p, (int64_t)nk, bits, c.cen.p, c.nrm.p, c.area.p,
                                                             dslot.p, dradii.p, nradii, per_src.p, within.p);
      ILG_CUDA(cudaGetLastError());
    }
  }
  ILG_CUDA(cudaMemcpyAsync(per_src_h, per_src.p, (size_t)nsrc * 8, cudaMemcpyDeviceToHost, s));
  if (nradii > 0 && within_h) ILG_CUDA(cudaMemcpyAsync(within_h, within.p, (size_t)nradii * 8, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  return read_device_errors(c);
}

}  // namespace ilg
