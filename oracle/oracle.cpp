// oracle.cpp — CPU restatement of sampotter/illum's illumination + thermal
// path. TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the
// CPU-baseline leg of the benchmark load this; the product library never does.
//
// Parity status: the reference has no tests, golden vectors or fixtures for
// this path, and it cannot be built here (gfortran, Armadillo, Boost, TBB and
// the Fast-BVH submodule are absent). Parity is therefore UNPINNED against the
// reference's own outputs, except for the two pieces the reference's Python
// can regenerate (Fibonacci spiral, src/py/points.py:71-86; ARMA binary
// format, src/py/arma.py:4-35). Everything else is a line-by-line restatement
// of the cited reference code in double precision, using the project's
// canonical ray/triangle predicate (geom.h mt64) in place of Fast-BVH.
//
// Algorithms here are deliberately the plain ones: brute-force O(N^2) facing
// test, a simple median-split BVH (different from the GPU's LBVH) traversed in
// double precision with mt64 on every visited triangle, per-sample direct
// insolation without any fast path, natural-order serial Gauss-Seidel, and a
// top-down Thomas solve per facet column with coefficients rebuilt per call.
//
// Build: oracle/Makefile (g++ -O2 -ffp-contract=off -pthread -shared).
#include "../illum_gb300/csrc/geom.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

using namespace ilg;

namespace {

int g_threads = 0;
int nthreads() {
  if (g_threads > 0) return g_threads;
  unsigned n = std::thread::hardware_concurrency();
  return n ? (int)n : 1;
}

template <class F>
void parallel_for(int64_t n, F&& f) {
  int nt = nthreads();
  if (nt <= 1 || n < 64) {
    for (int64_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<int64_t> next{0};
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&] {
      for (;;) {
        int64_t b = next.fetch_add(16);
        if (b >= n) break;
        int64_t e = std::min<int64_t>(n, b + 16);
        for (int64_t i = b; i < e; ++i) f(i);
      }
    });
  for (auto& t : th) t.join();
}

// ------------------------------------------------------------------ mesh
struct Mesh {
  int nt = 0;
  std::vector<f3> v0, v1, v2, c, n;
  std::vector<float> r;
  std::vector<double> area;
};

Mesh make_mesh(const float* verts, const int32_t* tris, int nt, const float* normals) {
  Mesh m;
  m.nt = nt;
  m.v0.resize(nt); m.v1.resize(nt); m.v2.resize(nt);
  m.c.resize(nt); m.n.resize(nt); m.r.resize(nt); m.area.resize(nt);
  for (int k = 0; k < nt; ++k) {
    const float* a = verts + 3 * tris[3 * k];
    const float* b = verts + 3 * tris[3 * k + 1];
    const float* d = verts + 3 * tris[3 * k + 2];
    m.v0[k] = mk(a[0], a[1], a[2]);
    m.v1[k] = mk(b[0], b[1], b[2]);
    m.v2[k] = mk(d[0], d[1], d[2]);
    m.c[k] = tri_centroid(m.v0[k], m.v1[k], m.v2[k]);
    m.n[k] = normals ? mk(normals[3 * k], normals[3 * k + 1], normals[3 * k + 2])
                     : tri_normal(m.v0[k], m.v1[k], m.v2[k]);
    m.r[k] = tri_radius(m.v0[k], m.v1[k], m.v2[k], m.c[k]);
    m.area[k] = tri_area(m.v0[k], m.v1[k], m.v2[k]);
  }
  return m;
}

// ------------------------------------------------------------------ BVH
// Median split on the longest centroid axis, leaves of <= 4 triangles,
// double-precision boxes inflated by a relative 1e-9 so the slab test never
// rejects a box holding an mt64 hit.
struct Node { double lo[3], hi[3]; int left, right, first, count; };

struct BVH {
  std::vector<Node> nodes;
  std::vector<int> idx;
  const Mesh* m = nullptr;

  void build(const Mesh& mesh) {
    m = &mesh;
    idx.resize(mesh.nt);
    for (int i = 0; i < mesh.nt; ++i) idx[i] = i;
    nodes.clear();
    nodes.reserve(2 * mesh.nt + 1);
    if (mesh.nt) rec(0, mesh.nt);
  }
  int rec(int b, int e) {
    int id = (int)nodes.size();
    nodes.push_back(Node{});
    Node nd;
    for (int a = 0; a < 3; ++a) { nd.lo[a] = 1e300; nd.hi[a] = -1e300; }
    double clo[3] = {1e300, 1e300, 1e300}, chi[3] = {-1e300, -1e300, -1e300};
    for (int k = b; k < e; ++k) {
      int t = idx[k];
      const f3* vs[3] = {&m->v0[t], &m->v1[t], &m->v2[t]};
      for (auto* v : vs) {
        double x[3] = {v->x, v->y, v->z};
        for (int a = 0; a < 3; ++a) { nd.lo[a] = std::min(nd.lo[a], x[a]); nd.hi[a] = std::max(nd.hi[a], x[a]); }
      }
      double cc[3] = {m->c[t].x, m->c[t].y, m->c[t].z};
      for (int a = 0; a < 3; ++a) { clo[a] = std::min(clo[a], cc[a]); chi[a] = std::max(chi[a], cc[a]); }
    }
    double ext = 0, mag = 0;
    for (int a = 0; a < 3; ++a) {
      ext = std::max(ext, nd.hi[a] - nd.lo[a]);
      mag = std::max(mag, std::max(std::fabs(nd.lo[a]), std::fabs(nd.hi[a])));
    }
    double pad = 1e-9 * ext + 1e-9 * mag + 1e-30;
    for (int a = 0; a < 3; ++a) { nd.lo[a] -= pad; nd.hi[a] += pad; }
    if (e - b <= 4) {
      nd.left = nd.right = -1; nd.first = b; nd.count = e - b;
      nodes[id] = nd;
      return id;
    }
    int ax = 0;
    for (int a = 1; a < 3; ++a) if (chi[a] - clo[a] > chi[ax] - clo[ax]) ax = a;
    int mid = (b + e) / 2;
    auto key = [&](int t) { const f3& c = m->c[t]; return ax == 0 ? c.x : (ax == 1 ? c.y : c.z); };
    std::nth_element(idx.begin() + b, idx.begin() + mid, idx.begin() + e,
                     [&](int p, int q) { float kp = key(p), kq = key(q); return kp < kq || (kp == kq && p < q); });
    nd.first = -1; nd.count = 0;
    nd.left = rec(b, mid);
    nd.right = rec(mid, e);
    nodes[id] = nd;
    return id;
  }

  static double slab(const Node& nd, const double o[3], const double inv[3]) {
    double tn = 0.0, tf = 1e300;
    for (int a = 0; a < 3; ++a) {
      double t0 = (nd.lo[a] - o[a]) * inv[a], t1 = (nd.hi[a] - o[a]) * inv[a];
      if (t0 > t1) std::swap(t0, t1);
      tn = std::max(tn, t0);
      tf = std::min(tf, t1);
    }
    return tn <= tf * (1.0 + 1e-12) ? tn : -1.0;
  }

  // Closest hit under mt64: smallest t, ties to the smaller index. Returns the
  // triangle index or -1. any_hit = true stops at the first hit.
  // Children are visited nearer-entry first and a box is skipped once its
  // entry lies beyond the best hit (with a relative margin). The answer is the
  // minimum over every triangle whose box the ray enters before the best hit,
  // so the visiting order changes the running time, never the result.
  int trace(f3 of, f3 df, bool any_hit, double* t_out) const {
    if (nodes.empty()) return -1;
    double o[3] = {of.x, of.y, of.z};
    double d[3] = {df.x, df.y, df.z}, inv[3];
    for (int a = 0; a < 3; ++a) {
      double x = std::fabs(d[a]) < 1e-300 ? (d[a] < 0 ? -1e-300 : 1e-300) : d[a];
      inv[a] = 1.0 / x;
    }
    double best = 1e300;
    int besti = -1;
    int stack[128];
    double tent[128];
    int sp = 0;
    double t_root = slab(nodes[0], o, inv);
    if (t_root >= 0.0) { stack[sp] = 0; tent[sp++] = t_root; }
    while (sp) {
      --sp;
      if (tent[sp] > best * (1.0 + 1e-12)) continue;
      const Node& nd = nodes[stack[sp]];
      if (nd.count) {
        for (int k = nd.first; k < nd.first + nd.count; ++k) {
          int t = idx[k];
          double th;
          if (mt64(of, df, m->v0[t], m->v1[t], m->v2[t], &th)) {
            if (th < best || (th == best && t < besti)) { best = th; besti = t; }
            if (any_hit) { if (t_out) *t_out = best; return besti; }
          }
        }
      } else {
        double tl = slab(nodes[nd.left], o, inv), tr = slab(nodes[nd.right], o, inv);
        bool l_ok = tl >= 0.0 && tl <= best * (1.0 + 1e-12);
        bool r_ok = tr >= 0.0 && tr <= best * (1.0 + 1e-12);
        // push the farther child first so the nearer one is popped next
        if (l_ok && r_ok) {
          if (tl <= tr) { stack[sp] = nd.right; tent[sp++] = tr; stack[sp] = nd.left; tent[sp++] = tl; }
          else { stack[sp] = nd.left; tent[sp++] = tl; stack[sp] = nd.right; tent[sp++] = tr; }
        } else if (l_ok) { stack[sp] = nd.left; tent[sp++] = tl; }
        else if (r_ok) { stack[sp] = nd.right; tent[sp++] = tr; }
      }
    }
    if (t_out) *t_out = best;
    return besti;
  }
};

}  // namespace

// Face normals that replace the computed ones in the direct insolation
// (the thermal loop included): the normals of an OBJ as the reference reads
// them (src/cpp/obj_util.cpp:70-88). nullptr: computed from the vertices.
static const float* g_normals = nullptr;

extern "C" {

void orc_set_threads(int n) { g_threads = n; }
void orc_set_normals(const float* normals) { g_normals = normals; }

// Derived per-facet quantities (centroid, normal, bounding radius, area),
// as the reference's Tri object provides them (src/cpp/obj_util.cpp:70-92).
void orc_facet_geometry(const float* verts, const int32_t* tris, int nt,
                        float* centroid, float* normal, float* radius, double* area) {
  Mesh m = make_mesh(verts, tris, nt, nullptr);
  for (int k = 0; k < nt; ++k) {
    centroid[3 * k] = m.c[k].x; centroid[3 * k + 1] = m.c[k].y; centroid[3 * k + 2] = m.c[k].z;
    normal[3 * k] = m.n[k].x; normal[3 * k + 1] = m.n[k].y; normal[3 * k + 2] = m.n[k].z;
    radius[k] = m.r[k];
    area[k] = m.area[k];
  }
}

// Closest-hit query (stand-in for BVH::getIntersection, call sites
// src/cpp/illum.cpp:73,301). brute = 1 tests every triangle.
void orc_trace(const float* verts, const int32_t* tris, int nt, int nrays,
               const float* orig, const float* dir, int any_hit, int brute,
               int32_t* hit, double* thit) {
  Mesh m = make_mesh(verts, tris, nt, nullptr);
  BVH bvh;
  if (!brute) bvh.build(m);
  parallel_for(nrays, [&](int64_t r) {
    f3 o = mk(orig[3 * r], orig[3 * r + 1], orig[3 * r + 2]);
    f3 d = mk(dir[3 * r], dir[3 * r + 1], dir[3 * r + 2]);
    int best = -1;
    double bt = 1e300;
    if (brute) {
      for (int t = 0; t < nt; ++t) {
        double th;
        if (mt64(o, d, m.v0[t], m.v1[t], m.v2[t], &th)) {
          if (th < bt || (th == bt && t < best)) { bt = th; best = t; }
          if (any_hit) break;
        }
      }
    } else {
      best = bvh.trace(o, d, any_hit != 0, &bt);
    }
    hit[r] = best;
    if (thit) thit[r] = best >= 0 ? bt : -1.0;
  });
}

// Visibility + form factors: src/cpp/illum.cpp:42-133 (per source facet j),
// then the sort into column-major order (:184-191) and the albedo row scaling
// (:225-234). Output triplets (i = receiver row, j = source column, F) in
// column-major order. Two-call protocol: with rows == nullptr only the count
// is returned (and cached); the second call copies the cached triplets.
// albedo: per-facet array or nullptr (then albedo_scalar). Returns nnz, or
// -1 on a NaN form factor (the reference throws, :121-123).
static std::vector<int32_t> s_i, s_j;
static std::vector<double> s_f;
static int64_t s_rays = 0;

int64_t orc_form_factors(const float* verts, const int32_t* tris, int nt, double offset,
                         const double* albedo, double albedo_scalar, double cutoff,
                         int32_t* rows, int32_t* cols, double* vals) {
  if (rows) {
    std::memcpy(rows, s_i.data(), s_i.size() * 4);
    std::memcpy(cols, s_j.data(), s_j.size() * 4);
    std::memcpy(vals, s_f.data(), s_f.size() * 8);
    return (int64_t)s_f.size();
  }
  Mesh m = make_mesh(verts, tris, nt, nullptr);
  BVH bvh;
  bvh.build(m);
  std::vector<std::vector<int32_t>> hits_of(nt);
  std::vector<std::vector<double>> f_of(nt);
  std::atomic<int64_t> rays{0};
  std::atomic<int> bad{0};
  const float cut2 = cutoff > 0.0 ? (float)(cutoff * cutoff) : -1.0f;
  parallel_for(nt, [&](int64_t jj) {
    int j = (int)jj;
    f3 p_j = m.c[j], n_j = m.n[j];
    f3 q_j = offset_point(p_j, n_j, offset);
    std::vector<int32_t> hits;
    int64_t nr = 0;
    for (int i = 0; i < nt; ++i) {
      if (i == j) continue;
      if (!facing(m.c[i], m.r[i], p_j, n_j)) continue;
      if (!within_cutoff(m.c[i], p_j, cut2)) continue;
      f3 d = normalize(sub(m.c[i], q_j));
      ++nr;
      int h = bvh.trace(q_j, d, false, nullptr);
      if (h < 0 || h == j) continue;
      auto lb = std::lower_bound(hits.begin(), hits.end(), h);
      if (lb == hits.end() || *lb != h) hits.insert(lb, h);
    }
    rays += nr;
    std::vector<int32_t> keep;
    std::vector<double> fv;
    for (int i : hits) {
      double F = form_factor(m.c[i], m.n[i], p_j, n_j, m.area[j]);
      if (std::isnan(F)) { bad = 1; continue; }
      if (F == 0.0) continue;
      keep.push_back(i);
      fv.push_back(F);
    }
    hits_of[j] = std::move(keep);
    f_of[j] = std::move(fv);
  });
  s_rays = rays;
  if (bad) return -1;
  s_i.clear(); s_j.clear(); s_f.clear();
  for (int j = 0; j < nt; ++j)
    for (size_t k = 0; k < hits_of[j].size(); ++k) {
      int i = hits_of[j][k];
      double rho = albedo ? albedo[i] : albedo_scalar;
      s_i.push_back(i);
      s_j.push_back(j);
      s_f.push_back(f_of[j][k] * rho);
    }
  return (int64_t)s_f.size();
}

int64_t orc_last_visibility_rays() { return s_rays; }

// Horizon bisection: src/cpp/illum.cpp:274-324 for every facet (:326-363).
// phi = linspace(0, 2 pi, nphi) with the endpoint (:329). Output nphi x nt,
// column-major (one column of nphi zenith angles per facet).
void orc_horizons_mesh(const float* verts, const int32_t* tris, int nt, const float* hverts,
                       const int32_t* htris, int hnt, int nphi, double theta_eps, double offset, double* out);

void orc_horizons(const float* verts, const int32_t* tris, int nt, int nphi,
                  double theta_eps, double offset, double* out) {
  orc_horizons_mesh(verts, tris, nt, nullptr, nullptr, 0, nphi, theta_eps, offset, out);
}

// The same with a separate horizon mesh (src/cpp/illum.cpp:333-349): rays
// from the facets of (verts, tris), traced against (hverts, htris); hverts
// NULL traces against the mesh itself.
void orc_horizons_mesh(const float* verts, const int32_t* tris, int nt, const float* hverts,
                       const int32_t* htris, int hnt, int nphi, double theta_eps, double offset, double* out) {
  Mesh m = make_mesh(verts, tris, nt, nullptr);
  Mesh hmesh = hverts ? make_mesh(hverts, htris, hnt, nullptr) : Mesh{};
  BVH bvh;
  bvh.build(hverts ? hmesh : m);
  std::vector<double> cph(nphi), sph(nphi);
  double dphi = nphi > 1 ? TWO_PI / (double)(nphi - 1) : 0.0;
  for (int k = 0; k < nphi; ++k) {
    double ph = (k == nphi - 1 && nphi > 1) ? TWO_PI : (double)k * dphi;
    sincos_x(ph, &sph[k], &cph[k]);
  }
  parallel_for(nt, [&](int64_t f) {
    f3 p = offset_point(m.c[f], m.n[f], offset);
    frame3 F = tri_frame(m.v0[f], m.v1[f], m.n[f]);
    for (int k = 0; k < nphi; ++k) {
      double lo = 0.0, hi = PI, mid = hi / 2.0, prev;
      do {
        prev = mid;
        double s, c;
        sincos_x(mid, &s, &c);
        f3 d = horizon_dir(F, cph[k], sph[k], c, s);
        if (bvh.trace(p, d, true, nullptr) >= 0) hi = mid; else lo = mid;
        mid = (lo + hi) / 2.0;
      } while (std::fabs(mid - prev) > theta_eps);
      out[(int64_t)f * nphi + k] = mid;
    }
  });
}

// Fibonacci spiral of src/cpp/illum.cpp:468-483, n x 2 column-major.
void orc_fib_spiral(double* xy, int n) { fib_spiral(xy, n); }

// Direct insolation of src/cpp/illum.cpp:382-466 with a deterministic disk
// tangent (geom.h sun_frame). horizons: nphi x nt column-major. disk_xy: ndisk
// x 2 column-major; ndisk - 1 samples are used (:421). norm_mode 0 divides the
// lit count by nphi - 1 (:441); 1 divides by the number of samples used.
// interp: 0 = reference threshold (:434), 1 = linear interpolation.
// solar_const is the flux at 1 AU (1372 in :451).
void orc_direct(const float* verts, const int32_t* tris, int nt, const double* horizons, int nphi,
                const double* sun, const double* disk_xy, int ndisk, int norm_mode, int interp,
                double solar_const, double* out, int32_t* counts) {
  Mesh m = make_mesh(verts, tris, nt, g_normals);
  double dphi = TWO_PI / (double)(nphi - 1);
  d3 S = mkd(sun[0], sun[1], sun[2]);
  double scale_au = ONE_AU_KM / norm(S);
  double flux = solar_const * (scale_au * scale_au);
  int nsamp = ndisk - 1;
  parallel_for(nt, [&](int64_t f) {
    d3 p = to_d(m.c[f]);
    d3 N = normalise(sub(S, p));
    d3 T, B;
    sun_frame(N, &T, &B);
    frame3 BTN = tri_frame(m.v0[f], m.v1[f], m.n[f]);
    const double* h = horizons + f * (int64_t)nphi;
    auto hl = [&](int k) { return h[k]; };
    int count = 0;
    for (int s = 0; s < nsamp; ++s) {
      double x = disk_xy[s], y = disk_xy[ndisk + s];
      d3 disk = add(S, scl(add(scl(T, x), scl(B, y)), SUN_RADIUS_KM));
      count += sample_lit(p, disk, BTN, hl, nphi, dphi, interp);
    }
    double denom = norm_mode == 0 ? (double)(nphi - 1) : (double)nsamp;
    double dv = (double)count / denom;
    double mu = sun_mu(S, p, BTN.n);
    dv *= (mu > 0.0 ? mu : 0.0);
    dv *= flux;
    out[f] = dv;
    if (counts) counts[f] = count;
  });
}

// Radiosity solve, src/cpp/arma_util.cpp:4-17 with the loop of
// src/cpp/illum_cli.cpp:425-440: L = I - tril(F), U = -triu(F);
// x = L^{-1} E, then sweeps x = L^{-1}(E - U x) in natural row order. F given
// as CSR by receiver row. mode 0: exactly 1 + gs_steps sweeps (reference);
// mode 1: sweep until ||(I - F) x - E||_2 <= tol or max_sweeps.
// Returns the number of sweeps done; *res gets the final residual.
int orc_gauss_seidel(int n, const int64_t* rowptr, const int32_t* col, const double* val,
                     const double* E, int mode, int gs_steps, double tol, int max_sweeps,
                     double* x, double* res) {
  for (int i = 0; i < n; ++i) x[i] = 0.0;
  auto residual = [&]() {
    double s = 0.0;
    for (int i = 0; i < n; ++i) {
      double ax = x[i];
      for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) ax -= val[k] * x[col[k]];
      double r = ax - E[i];
      s += r * r;
    }
    return std::sqrt(s);
  };
  int sweeps = 0;
  int limit = mode == 0 ? 1 + gs_steps : max_sweeps;
  double r = 0.0;
  std::vector<double> b(mode == 0 ? n : 0);
  while (sweeps < limit) {
    if (mode == 0) {
      // the reference's order: b = E - U x with U = -triu(F) (diagonal
      // included), the product accumulated from zero over each row's
      // columns in ascending order (Armadillo's sparse product), then the
      // forward solve of L x = b with L = I - tril(F), adding the lower
      // terms in ascending column order and dividing by L's diagonal
      // 1 - F_ii (src/cpp/arma_util.cpp:4-17, src/cpp/illum_cli.cpp:425-433;
      // -(-a) b terms are exact sign flips of a b). The first solve has no
      // upper term.
      for (int i = 0; i < n; ++i) {
        double u = 0.0;
        if (sweeps > 0)
          for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
            if (col[k] >= i) u += val[k] * x[col[k]];
        b[i] = sweeps > 0 ? E[i] + u : E[i];
      }
      for (int i = 0; i < n; ++i) {
        double xi = b[i], fii = 0.0;
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
          if (col[k] < i) xi += val[k] * x[col[k]];
          else if (col[k] == i) fii = val[k];
        }
        x[i] = xi / (1.0 - fii);
      }
    } else {
      for (int i = 0; i < n; ++i) {
        double xi = E[i];
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) xi += val[k] * x[col[k]];
        x[i] = xi;
      }
    }
    ++sweeps;
    if (mode == 1) {
      r = residual();
      if (r <= tol) break;
    }
  }
  if (mode == 0) r = residual();
  if (res) *res = r;
  return sweeps;
}

// ------------------------------------------------------------------ conduction
// Thomas algorithm for a tridiagonal system (textbook LU recurrence):
// a = sub-diagonal (a[0] unused), b = diagonal, c = super-diagonal
// (c[n-1] unused). Returns 0, or -1 on a zero pivot (the reference's solver
// stops the program there).
static int thomas(int n, const double* a, const double* b, const double* c, const double* r,
                  double* x, double* cp, double* dp) {
  if (b[0] == 0.0) return -1;
  cp[0] = c[0] / b[0];
  dp[0] = r[0] / b[0];
  for (int i = 1; i < n; ++i) {
    double m = b[i] - a[i] * cp[i - 1];
    if (m == 0.0) return -1;
    cp[i] = c[i] / m;
    dp[i] = (r[i] - a[i] * dp[i - 1]) / m;
  }
  x[n - 1] = dp[n - 1];
  for (int i = n - 2; i >= 0; --i) x[i] = dp[i] - cp[i] * x[i + 1];
  return 0;
}

// Coefficients of src/cpp/conductionQ.f:50-73 (0-based: index i is the
// Fortran's i+1).
struct CNCoef {
  std::vector<double> k, alpha, gamma, a, b, c;
  double k1 = 0;
};
static void cn_coefficients(int nz, const double* z, double dt, const double* ti, const double* rhoc,
                            CNCoef& C) {
  C.k.assign(nz, 0); C.alpha.assign(nz, 0); C.gamma.assign(nz, 0);
  C.a.assign(nz, 0); C.b.assign(nz, 0); C.c.assign(nz, 0);
  for (int i = 0; i < nz; ++i) C.k[i] = ti[i] * ti[i] / rhoc[i];
  double dz = 2.0 * z[0];
  double beta = dt / rhoc[0] / (2.0 * dz * dz);
  C.alpha[0] = beta * C.k[1];
  C.gamma[0] = beta * C.k[0];
  for (int i = 1; i < nz - 1; ++i) {
    double buf = dt / (z[i + 1] - z[i - 1]);
    C.alpha[i] = 2.0 * C.k[i + 1] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i]);
    C.gamma[i] = 2.0 * C.k[i] * buf / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1]);
  }
  double buf = dt / ((z[nz - 1] - z[nz - 2]) * (z[nz - 1] - z[nz - 2]));
  C.gamma[nz - 1] = C.k[nz - 1] * buf / (2.0 * rhoc[nz - 1]);
  C.k1 = C.k[0] / dz;
  for (int i = 0; i < nz; ++i) {
    C.a[i] = -C.gamma[i];
    C.b[i] = 1.0 + C.alpha[i] + C.gamma[i];
    C.c[i] = -C.alpha[i];
  }
  C.b[nz - 1] = 1.0 + C.gamma[nz - 1];
}

// Interior right-hand side rows 2..nz of src/cpp/conductionQ.f:68-74.
static void cn_rhs_interior(int nz, const CNCoef& C, const double* T, double dt, const double* z,
                            const double* rhoc, double Fgeo, double* r) {
  for (int i = 1; i < nz - 1; ++i)
    r[i] = C.gamma[i] * T[i - 1] + (1.0 - C.alpha[i] - C.gamma[i]) * T[i] + C.alpha[i] * T[i + 1];
  r[nz - 1] = C.gamma[nz - 1] * T[nz - 2] + (1.0 - C.gamma[nz - 1]) * T[nz - 1] +
              dt / rhoc[nz - 1] * Fgeo / (z[nz - 1] - z[nz - 2]);
}

// conductionQ (src/cpp/conductionQ.f:1-99): Crank-Nicolson step with the
// radiative surface boundary linearised once about the previous Tsurf.
int orc_conductionq(int nz, const double* z, double dt, double Qn, double Qnp1, double* T,
                    const double* ti, const double* rhoc, double emiss, double* Tsurf,
                    double Fgeo, double* Fsurf) {
  CNCoef C;
  cn_coefficients(nz, z, dt, ti, rhoc, C);
  double Tr = *Tsurf;
  double Tr3 = Tr * Tr * Tr;
  double arad = -3.0 * emiss * SIGMA_SB * Tr3 * Tr;
  double brad = 2.0 * emiss * SIGMA_SB * Tr3;
  double ann = (Qn - arad) / (C.k1 + brad);
  double annp1 = (Qnp1 - arad) / (C.k1 + brad);
  double bn = (C.k1 - brad) / (C.k1 + brad);
  std::vector<double> b = C.b, r(nz), cp(nz), dp(nz);
  b[0] = 1.0 + C.alpha[0] + C.gamma[0] - C.gamma[0] * bn;
  r[0] = C.gamma[0] * (annp1 + ann) + (1.0 - C.alpha[0] - C.gamma[0] + C.gamma[0] * bn) * T[0] +
         C.alpha[0] * T[1];
  cn_rhs_interior(nz, C, T, dt, z, rhoc, Fgeo, r.data());
  if (thomas(nz, C.a.data(), b.data(), C.c.data(), r.data(), T, cp.data(), dp.data())) return -1;
  *Tsurf = 0.5 * (annp1 + bn * T[0] + T[0]);
  *Fsurf = -C.k[0] * (T[0] - *Tsurf) / z[0];
  return 0;
}

// Newton variant (this project's extension for the nonlinear radiative
// boundary): the same Crank-Nicolson rows, with the ghost node tied to the
// surface temperature, T0 = 2 Ts - T1, at both time levels, and the boundary
// Q + 2 k1 (T1 - Ts) = emiss sigma Ts^4 at n+1 solved by Newton's method on
// Ts. T1(n+1) is affine in Ts(n+1): T1 = P + S Ts, with P from one Thomas
// solve (Ts = 0) and S from a second solve with the unit response 2 gamma1
// in row 1. Iterates until |dTs| <= 1e-13 Ts or 30 iterations.
int orc_conductionq_newton(int nz, const double* z, double dt, double Qnp1, double* T,
                           const double* ti, const double* rhoc, double emiss, double* Tsurf,
                           double Fgeo, double* Fsurf, int* iters) {
  CNCoef C;
  cn_coefficients(nz, z, dt, ti, rhoc, C);
  double Ts = *Tsurf;
  std::vector<double> b = C.b, r(nz), e(nz, 0.0), x0(nz), x1(nz), cp(nz), dp(nz);
  b[0] = 1.0 + C.alpha[0] + 2.0 * C.gamma[0];
  r[0] = (1.0 - C.alpha[0] - C.gamma[0]) * T[0] + C.alpha[0] * T[1] + C.gamma[0] * (2.0 * Ts - T[0]);
  cn_rhs_interior(nz, C, T, dt, z, rhoc, Fgeo, r.data());
  if (thomas(nz, C.a.data(), b.data(), C.c.data(), r.data(), x0.data(), cp.data(), dp.data())) return -1;
  e[0] = 2.0 * C.gamma[0];
  if (thomas(nz, C.a.data(), b.data(), C.c.data(), e.data(), x1.data(), cp.data(), dp.data())) return -1;
  double P = x0[0], S = x1[0];
  double es = emiss * SIGMA_SB;
  int it = 0;
  for (; it < 30; ++it) {
    double Ts3 = Ts * Ts * Ts;
    double g = Qnp1 + 2.0 * C.k1 * (P + (S - 1.0) * Ts) - es * Ts3 * Ts;
    double dg = 2.0 * C.k1 * (S - 1.0) - 4.0 * es * Ts3;
    double dT = g / dg;
    Ts -= dT;
    if (std::fabs(dT) <= 1e-13 * std::fabs(Ts)) { ++it; break; }
  }
  for (int i = 0; i < nz; ++i) T[i] = x0[i] + x1[i] * Ts;
  *Tsurf = Ts;
  *Fsurf = -C.k[0] * (T[0] - Ts) / z[0];
  if (iters) *iters = it;
  return 0;
}

// conductionT (src/cpp/conductionT.f:1-71): prescribed surface temperature.
int orc_conductiont(int nz, const double* z, double dt, double* T, double Tsurf, double Tsurfp1,
                    const double* ti, const double* rhoc, double Fgeo, double* Fsurf) {
  std::vector<double> k(nz), alpha(nz, 0.0), gamma(nz, 0.0), a(nz), b(nz), c(nz), r(nz), cp(nz), dp(nz);
  for (int i = 0; i < nz; ++i) k[i] = ti[i] * ti[i] / rhoc[i];
  alpha[0] = k[1] * dt / rhoc[0] / (z[1] - z[0]) / z[1];
  gamma[0] = k[0] * dt / rhoc[0] / z[0] / z[1];
  for (int i = 1; i < nz - 1; ++i) {
    double buf = dt / (z[i + 1] - z[i - 1]);
    alpha[i] = k[i + 1] * buf * 2.0 / (rhoc[i] + rhoc[i + 1]) / (z[i + 1] - z[i]);
    gamma[i] = k[i] * buf * 2.0 / (rhoc[i] + rhoc[i + 1]) / (z[i] - z[i - 1]);
  }
  double buf = dt / ((z[nz - 1] - z[nz - 2]) * (z[nz - 1] - z[nz - 2]));
  gamma[nz - 1] = k[nz - 1] * buf / (rhoc[nz - 1] + rhoc[nz - 1]);
  for (int i = 0; i < nz; ++i) { a[i] = -gamma[i]; b[i] = 1.0 + alpha[i] + gamma[i]; c[i] = -alpha[i]; }
  b[nz - 1] = 1.0 + gamma[nz - 1];
  r[0] = alpha[0] * T[1] + (1.0 - alpha[0] - gamma[0]) * T[0] + gamma[0] * (Tsurf + Tsurfp1);
  for (int i = 1; i < nz - 1; ++i)
    r[i] = gamma[i] * T[i - 1] + (1.0 - alpha[i] - gamma[i]) * T[i] + alpha[i] * T[i + 1];
  r[nz - 1] = gamma[nz - 1] * T[nz - 2] + (1.0 - gamma[nz - 1]) * T[nz - 1] +
              dt / rhoc[nz - 1] * Fgeo / (z[nz - 1] - z[nz - 2]);
  if (thomas(nz, a.data(), b.data(), c.data(), r.data(), T, cp.data(), dp.data())) return -1;
  *Fsurf = -k[0] * (T[0] - Tsurfp1) / z[0];
  return 0;
}

// ------------------------------------------------------------------ step driver
// One run of the time-step loop of src/cpp/illum_cli.cpp:403-468 with the
// thermal model of src/cpp/thermal.hpp:17-105:
//   rad = -Fsurf_prev + direct(sun_s); rad = radiosity(F, rad);
//   rad_avg += (rad - rad_avg)/(frame+1); thermal step with Q = rad;
//   therm_avg update; therm_max after frame 50.
// direct_all: nsteps x nt precomputed direct fluxes (row-major by step), or
// nullptr to compute them here from sun positions (nsteps x 3).
// T: (nz+1) x nt column-major in/out (row 0 = surface), the reference's
// layout (src/cpp/thermal.hpp:48). bc_mode 0 = conductionQ, 1 = Newton.
// rad_mode: 0 = reference sweeps (1 + gs_steps), 1 = to tolerance.
// coupling: 0 = E = -Fsurf + direct (src/cpp/illum_cli.cpp:411-421),
// 1 = E = direct.
struct orc_run_params {
  int nt, nz, nsteps, nphi, ndisk, norm_mode, interp, bc_mode, rad_mode, gs_steps, max_sweeps, use_radiosity,
      coupling;
  double dt, emiss, solar_const, tol, Fgeo;
};

int orc_thermal_run(const orc_run_params* P, const float* verts, const int32_t* tris,
                    const double* horizons, const double* sun, const double* disk_xy,
                    const double* direct_all, const int64_t* rowptr, const int32_t* col,
                    const double* val, const double* z, const double* ti, const double* rhoc,
                    double* T, double* Qprev, double* Fsurf, double* rad, double* rad_avg,
                    double* therm_avg, double* therm_max, int frame0, double* tsurf_hist) {
  int nt = P->nt, nz = P->nz;
  std::vector<double> direct(nt), E(nt), x(nt);
  std::vector<int32_t> cnt(nt);
  for (int s = 0; s < P->nsteps; ++s) {
    if (direct_all) {
      std::memcpy(direct.data(), direct_all + (int64_t)s * nt, nt * 8);
    } else {
      orc_direct(verts, tris, nt, horizons, P->nphi, sun + 3 * s, disk_xy, P->ndisk, P->norm_mode,
                 P->interp, P->solar_const, direct.data(), cnt.data());
    }
    if (P->coupling == 0)
      for (int i = 0; i < nt; ++i) E[i] = -Fsurf[i] + direct[i];
    else
      for (int i = 0; i < nt; ++i) E[i] = direct[i];
    if (P->use_radiosity) {
      double res;
      orc_gauss_seidel(nt, rowptr, col, val, E.data(), P->rad_mode, P->gs_steps, P->tol,
                       P->max_sweeps, x.data(), &res);
    } else {
      x = E;
    }
    int frame = frame0 + s;
    for (int i = 0; i < nt; ++i) {
      rad[i] = x[i];
      rad_avg[i] += (x[i] - rad_avg[i]) / (double)(frame + 1);
    }
    for (int i = 0; i < nt; ++i) {
      double* col_T = T + (int64_t)i * (nz + 1);
      int rc;
      if (P->bc_mode == 0)
        rc = orc_conductionq(nz, z, P->dt, Qprev[i], x[i], col_T + 1, ti, rhoc, P->emiss, col_T,
                             P->Fgeo, &Fsurf[i]);
      else
        rc = orc_conductionq_newton(nz, z, P->dt, x[i], col_T + 1, ti, rhoc, P->emiss, col_T,
                                    P->Fgeo, &Fsurf[i], nullptr);
      if (rc) return -1;
      Qprev[i] = x[i];
      double th = col_T[0];
      therm_avg[i] += (th - therm_avg[i]) / (double)(frame + 1);
      if (frame > 50) therm_max[i] = std::max(therm_max[i], th);
      if (tsurf_hist) tsurf_hist[(int64_t)s * nt + i] = th;
    }
  }
  return 0;
}

}  // extern "C"
