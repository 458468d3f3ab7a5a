// radiosity.cu — solve (I - F) x = E for the form-factor matrix (CSR by
// receiver row), the linear system the reference solves with a forward
// solve plus Gauss-Seidel sweeps (src/cpp/arma_util.cpp:4-17,
// src/cpp/illum_cli.cpp:425-440).
//
// GPU scheme: Jacobi sweeps x <- E + F x over the rows that have entries
// (rows without entries are x = E exactly) inside ONE persistent cooperative
// kernel. The matrix is stored as SELL-32 (slices of 32 rows, column-major,
// one lane per row or row chunk, fixed summation order) and the solve works
// on facets renumbered in the LBVH's Morton order, so the gathers of x hit
// few cache lines. A grid barrier separates sweeps and every block reduces
// the residual partials in the same fixed order, so all blocks take the same
// stop decision and results are run-to-run deterministic. The residual of
// iterate x_k is E - (I - F) x_k = x_{k+1} - x_k, so it comes for free
// with the next sweep; iteration stops once its 2-norm is <= tol.
// With albedo-scaled form factors the iteration matrix has spectral radius
// well below 1, so Jacobi converges in a handful of sweeps; a multicolour
// Gauss-Seidel would need one grid barrier per colour, and the cliques of
// mutually visible crater facets force hundreds of colours.
//
// Mixed precision: values stored as bf16 with a per-row fp32 scale, fp32
// accumulation for the sweeps, and an outer refinement whose residual is
// evaluated with the fp64 values in fp64 (so the fixed point is the fp64
// system's).
#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace ilg {

namespace {

constexpr int RAD_THREADS = 1024;

// Grid barrier for a cooperative launch (all blocks co-resident). The wait
// is bounded: after ~2^26 polls it records DERR_BARRIER and returns false.
__device__ bool grid_barrier(unsigned* bar, unsigned nblocks, int* derr) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned* gen = bar + 1;
    unsigned g = *gen;
    __threadfence();
    if (atomicAdd(bar, 1u) == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long it = 0;
      while (*gen == g) {
        if (++it > (1LL << 26) || *(volatile int*)&derr[DERR_BARRIER]) {
          atomicExch(&derr[DERR_BARRIER], 1);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

__device__ __forceinline__ int mesh_of_facet(const StepView& v, int g) { return v.mesh_of ? v.mesh_of[g] : 0; }
__device__ __forceinline__ int mesh_of_slice(const StepView& v, int sl) { return v.sl_mesh ? v.sl_mesh[sl] : 0; }

// Loads of the matrix carry an L2 evict-last policy on a fraction of the
// lines: the SELL arrays (~12-16 B per entry) are re-read by every sweep of
// a solve, and when they are about as large as GB300's 126 MB L2 a plain
// cyclic scan would evict every line before its reuse. Keeping 3/4 of the
// lines at evict-last lets sweeps after the first hit L2 for most of the
// matrix while the rest streams from HBM.
__device__ __forceinline__ uint64_t l2_keep_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 0.75;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ int ld_keep(const int32_t* p, uint64_t pol) {
  int v;
  asm volatile("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ double ld_keep(const double* p, uint64_t pol) {
  double v;
  asm volatile("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ __nv_bfloat16 ld_keep(const __nv_bfloat16* p, uint64_t pol) {
  unsigned short v;
  asm volatile("ld.global.nc.L2::cache_hint.b16 %0, [%1], %2;" : "=h"(v) : "l"(p), "l"(pol));
  return __ushort_as_bfloat16(v);
}

// One SELL-32 slice: lane l accumulates its (chunk of a) row sequentially
// (four independent loads in flight), then rows split into several chunks
// are combined into their first lane in a fixed order.
template <class V, class X, class Acc>
__device__ __forceinline__ Acc slice_dot(const StepView& v, const V* __restrict__ sval, const X* __restrict__ x,
                                         int sl, int lane) {
  int64_t base = v.sl_ptr[sl] + lane;
  int len = v.sl_len[sl];
  const uint64_t pol = l2_keep_policy();
  Acc p = 0;
  int k = 0;
  for (; k + 8 <= len; k += 8) {
    int c[8];
    V w[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      c[j] = ld_keep(v.s_col + base + (int64_t)(k + j) * 32, pol);
      w[j] = ld_keep(sval + base + (int64_t)(k + j) * 32, pol);
    }
    X xv[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) xv[j] = x[c[j]];
#pragma unroll
    for (int j = 0; j < 8; ++j) p += (Acc)w[j] * (Acc)xv[j];
  }
  if (k < len) {   // len is a multiple of 4
    int c[4];
    V w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      c[j] = ld_keep(v.s_col + base + (int64_t)(k + j) * 32, pol);
      w[j] = ld_keep(sval + base + (int64_t)(k + j) * 32, pol);
    }
    X xv[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) xv[j] = x[c[j]];
#pragma unroll
    for (int j = 0; j < 4; ++j) p += (Acc)w[j] * (Acc)xv[j];
  }
  int mmax = v.sl_split[sl];
  if (mmax > 1) {
    int m = v.ln_m[(int64_t)sl * 32 + lane];
    Acc tot = p;
    for (int j = 1; j < mmax; ++j) {
      Acc q = __shfl_down_sync(0xffffffffu, p, j);
      if (j < m) tot += q;
    }
    p = tot;
  }
  return p;
}

__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Per-mesh convergence. Residual partials are reduced in a fixed order that
// depends only on the mesh's own slices: each slice's partial (warp sum),
// then chunks of RAD_CHUNK consecutive slices of the mesh (one warp per
// chunk), then the mesh's chunks in order. Every block repeats the last
// stage for every mesh and keeps the stop flags in shared memory, so all
// blocks take the same decisions without another barrier, and a mesh's
// decisions are the same alone and in a batch.
constexpr int RAD_CHUNK = 256;
constexpr int RAD_MAX_MESH = 1024;

struct MeshState {
  int done[RAD_MAX_MESH];
  int sweeps[RAD_MAX_MESH];
};

__device__ __forceinline__ void init_meshes(const StepView& v, MeshState& st) {
  for (int m = threadIdx.x; m < v.nmesh; m += blockDim.x) {
    const MeshDesc& M = v.md[m];
    st.done[m] = (M.active && M.nslices > 0) ? 0 : 1;
    st.sweeps[m] = 0;
  }
}

// chunk sums of all meshes still running (one warp per chunk)
__device__ __forceinline__ void chunk_sums(const StepView& v, const MeshState& st, int gw, int nwarps, int lane) {
  for (int k = gw; k < v.nchunks; k += nwarps) {
    int4 ch = v.chunks[k];   // (first slice, count, mesh, -)
    if (st.done[ch.z]) continue;
    double w[RAD_CHUNK / 32];
#pragma unroll
    for (int j = 0; j < RAD_CHUNK / 32; ++j) {
      int idx = lane + 32 * j;
      w[j] = idx < ch.y ? v.sl_d2[ch.x + idx] : 0.0;
    }
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < RAD_CHUNK / 32; ++j) t += w[j];
    t = warp_sum(t);
    if (lane == 0) v.ch_d2[k] = t;
  }
}

// Every block: totals per running mesh (its chunks in order), stop
// decisions, and the number of meshes still running. Block 0 records the
// sweep counts and residuals in the mesh table.
__device__ __forceinline__ int decide_meshes(const StepView& v, MeshState& st, int inc, int first) {
  __syncthreads();
  for (int m = threadIdx.x; m < v.nmesh; m += blockDim.x) {
    if (st.done[m]) continue;
    const MeshDesc& M = v.md[m];
    double t = 0.0;
    for (int c0 = 0; c0 < M.nchunks; c0 += 8) {   // loads issued together, summed in order
      double w[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) w[j] = c0 + j < M.nchunks ? v.ch_d2[M.chunk0 + c0 + j] : 0.0;
#pragma unroll
      for (int j = 0; j < 8; ++j) t += w[j];
    }
    int sw = st.sweeps[m] + (first ? 0 : inc);
    st.sweeps[m] = sw;
    bool stop = t <= M.tol2 || sw >= M.max_sweeps;
    if (stop) st.done[m] = 1;
    if (blockIdx.x == 0) {
      v.md[m].sweeps = sw;
      v.md[m].res2 = t;
    }
  }
  __syncthreads();
  int running = 0;
  for (int m0 = 0; m0 < v.nmesh; m0 += blockDim.x) {
    int m = m0 + threadIdx.x;
    running += __syncthreads_count(m < v.nmesh && !st.done[m]);
  }
  return running;
}

// The solve works on radiosity positions (Morton order within each mesh):
// EP = E, P0 / P1 = iterates, gathered through rperm at entry. Start values:
// rows without entries are x = E exactly; the others start at E (cold) or
// at the mesh's previous solution, extrapolated linearly once two solutions
// exist (warm).
__device__ __forceinline__ void init_x(const StepView& v, const double* x, int warm, int gt, int nthreads) {
  double* EP = v.rbuf;
  double* P0 = v.rbuf + v.nt;
  double* P1 = v.rbuf + 2 * (size_t)v.nt;
  for (int p = gt; p < v.nt; p += nthreads) {
    int g = (int)v.rperm[p];
    const MeshDesc& M = v.md[mesh_of_facet(v, g)];
    if (!M.active || M.nslices == 0) continue;
    double e = v.E[g];
    EP[p] = e;
    P1[p] = e;
    if (!warm || !v.row_act[g]) {
      P0[p] = e;
    } else {
      double xn = x[g];
      P0[p] = M.frame >= 2 ? 2.0 * xn - v.xprev[g] : xn;
      v.xprev[g] = xn;
    }
    if (v.x32) {
      v.x32[p] = 0.f;
      v.x32[v.nt + p] = 0.f;
    }
  }
}

// Scatter the solved meshes' last iterate back to facet order.
__device__ __forceinline__ void scatter_x(const StepView& v, const MeshState& st, double* x, int gt, int nthreads,
                                          bool mixed) {
  const double* P0 = v.rbuf + v.nt;
  const double* P1 = v.rbuf + 2 * (size_t)v.nt;
  for (int p = gt; p < v.nt; p += nthreads) {
    int g = (int)v.rperm[p];
    int m = mesh_of_facet(v, g);
    const MeshDesc& M = v.md[m];
    if (!M.active || M.nslices == 0) continue;
    x[g] = (!mixed && (st.sweeps[m] & 1)) ? P1[p] : P0[p];
  }
}

// FP64 Jacobi to each mesh's tolerance. x: solution (and warm start).
__global__ void __launch_bounds__(RAD_THREADS, 1) k_radiosity64(StepView v, double* x, int warm) {
  __shared__ MeshState st;
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * RAD_THREADS + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * RAD_THREADS) >> 5;
  const int gt = blockIdx.x * RAD_THREADS + threadIdx.x;
  const int nthreads = gridDim.x * RAD_THREADS;
  init_meshes(v, st);
  init_x(v, x, warm, gt, nthreads);
  if (!grid_barrier(v.barrier, gridDim.x, v.derr)) return;
  const double* EP = v.rbuf;
  double* cur = v.rbuf + v.nt;
  double* nxt = v.rbuf + 2 * (size_t)v.nt;
  for (;;) {
    for (int sl = gw; sl < v.nslices; sl += nwarps) {
      if (st.done[mesh_of_slice(v, sl)]) continue;
      double s = slice_dot<double, double, double>(v, v.s_val, cur, sl, lane);
      int64_t li = (int64_t)sl * 32 + lane;
      double d2 = 0.0;
      if (v.ln_m[li] > 0) {
        int i = v.ln_row[li];
        double xn = EP[i] + s;
        double df = xn - cur[i];
        nxt[i] = xn;
        d2 = df * df;
      }
      d2 = warp_sum(d2);
      if (lane == 0) v.sl_d2[sl] = d2;
    }
    if (!grid_barrier(v.barrier, gridDim.x, v.derr)) return;
    chunk_sums(v, st, gw, nwarps, lane);
    if (!grid_barrier(v.barrier, gridDim.x, v.derr)) return;
    double* t = cur; cur = nxt; nxt = t;
    if (decide_meshes(v, st, 1, 0) == 0) break;
  }
  scatter_x(v, st, x, gt, nthreads, false);
}

// Mixed precision: outer refinement with an fp64 residual r = E - (I - F) x
// (fp64 values), inner fp32 Jacobi on (I - F~) d = r with bf16 F~ (4 sweeps),
// x += d. A mesh stops when ||r||_2 <= tol.
__global__ void __launch_bounds__(RAD_THREADS, 1) k_radiosity_mixed(StepView v, double* x, int warm) {
  __shared__ MeshState st;
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * RAD_THREADS + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * RAD_THREADS) >> 5;
  const int gt = blockIdx.x * RAD_THREADS + threadIdx.x;
  const int nthreads = gridDim.x * RAD_THREADS;
  float* xa = v.x32;
  float* xb = v.x32 + v.nt;
  float* r32 = v.x32 + 2 * (size_t)v.nt;
  init_meshes(v, st);
  init_x(v, x, warm, gt, nthreads);
  if (!grid_barrier(v.barrier, gridDim.x, v.derr)) return;
  const double* EP = v.rbuf;
  double* X = v.rbuf + v.nt;          // the fp64 iterate (radiosity positions)
  int first = 1;
  for (;;) {
    for (int sl = gw; sl < v.nslices; sl += nwarps) {
      if (st.done[mesh_of_slice(v, sl)]) continue;
      double s = slice_dot<double, double, double>(v, v.s_val, X, sl, lane);
      int64_t li = (int64_t)sl * 32 + lane;
      double r2 = 0.0;
      if (v.ln_m[li] > 0) {
        int i = v.ln_row[li];
        double r = EP[i] + s - X[i];
        r32[i] = (float)r;
        xa[i] = (float)r;     // inner start: d0 = r
        r2 = r * r;
      }
      r2 = warp_sum(r2);
      if (lane == 0) v.sl_d2[sl] = r2;
    }
    if (!grid_barrier(v.barrier, gridDim.x, v.derr)) return;
    chunk_sums(v, st, gw, nwarps, lane);
    if (!grid_barrier(v.barrier, gridDim.x, v.derr)) return;
    int running = decide_meshes(v, st, 4, first);
    first = 0;
    if (running == 0) break;   // scatter below
    float* cur = xa;
    float* nxt = xb;
    for (int it = 0; it < 4; ++it) {
      for (int sl = gw; sl < v.nslices; sl += nwarps) {
        if (st.done[mesh_of_slice(v, sl)]) continue;
        float s = slice_dot<__nv_bfloat16, float, float>(v, v.s_vbf, cur, sl, lane);
        int64_t li = (int64_t)sl * 32 + lane;
        if (v.ln_m[li] > 0) {
          int i = v.ln_row[li];
          nxt[i] = r32[i] + v.rscale[v.rperm[i]] * s;
        }
      }
      if (!grid_barrier(v.barrier, gridDim.x, v.derr)) return;
      float* t = cur; cur = nxt; nxt = t;
    }
    for (int sl = gw; sl < v.nslices; sl += nwarps) {
      if (st.done[mesh_of_slice(v, sl)]) continue;
      int64_t li = (int64_t)sl * 32 + lane;
      if (v.ln_m[li] > 0) X[v.ln_row[li]] += (double)cur[v.ln_row[li]];
    }
    if (!grid_barrier(v.barrier, gridDim.x, v.derr)) return;
  }
  scatter_x(v, st, x, gt, nthreads, true);
}

__global__ void k_active_rows(const int64_t* __restrict__ rowptr, int nt, uint32_t* flag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nt) flag[i] = rowptr[i + 1] != rowptr[i] ? 1u : 0u;
}
__global__ void k_active_compact(const uint32_t* __restrict__ flag, const unsigned long long* __restrict__ pos,
                                 int nt, int32_t* active) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nt && flag[i]) active[pos[i]] = i;
}

// SELL fill: element e takes CSR entry src[e] (value, and its bf16 copy
// scaled by its row's scale), or zero for padding (src < 0).
__global__ void k_sell_fill(const int64_t* __restrict__ src, int64_t nel, const int64_t* __restrict__ sl_ptr,
                            int nslices, const int32_t* __restrict__ ln_row, const uint32_t* __restrict__ rperm,
                            const double* __restrict__ val, const float* __restrict__ rscale, double* s_val,
                            __nv_bfloat16* s_vbf) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  int64_t k = src[e];
  if (k < 0) {
    s_val[e] = 0.0;
    s_vbf[e] = __float2bfloat16_rn(0.f);
    return;
  }
  // the element's slice and lane give its row (Morton position -> facet)
  int lo = 0, hi = nslices - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (sl_ptr[mid] <= e) lo = mid; else hi = mid - 1;
  }
  int lane = (int)((e - sl_ptr[lo]) & 31);
  int row = (int)rperm[ln_row[(int64_t)lo * 32 + lane]];
  double v = val[k];
  s_val[e] = v;
  s_vbf[e] = __float2bfloat16_rn((float)(v / (double)rscale[row]));
}

__global__ void k_rank(const uint32_t* __restrict__ order, int nt, uint32_t* rank) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < nt) rank[order[p]] = (uint32_t)p;
}

// key = row << rb | Morton position of the column; value = CSR entry.
__global__ void k_row_keys(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                           const uint32_t* __restrict__ rank, int nt, int rb, unsigned long long* key,
                           uint32_t* src) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  unsigned long long hi = (unsigned long long)i << rb;
  for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    key[k] = hi | rank[col[k]];
    src[k] = (uint32_t)k;
  }
}

// Per-row fp32 scale = max |F_ij| of the row; values stored as bf16(F/scale).
__global__ void k_to_bf16(const int64_t* __restrict__ rowptr, const double* __restrict__ val, int nt,
                          __nv_bfloat16* vbf, float* rscale) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  int64_t b = rowptr[i], e = rowptr[i + 1];
  double m = 0.0;
  for (int64_t k = b; k < e; ++k) m = fmax(m, fabs(val[k]));
  float sc = m > 0.0 ? (float)m : 1.f;
  rscale[i] = sc;
  for (int64_t k = b; k < e; ++k) vbf[k] = __float2bfloat16_rn((float)(val[k] / (double)sc));
}

}  // namespace

int radiosity_prepare(Context& c) {
  cudaStream_t s = c.stream;
  int nt = c.nt;
  dbuf<uint32_t> flag;
  dbuf<unsigned long long> pos;
  ILG_TRY(flag.alloc(nt));
  ILG_TRY(pos.alloc(nt));
  k_active_rows<<<div_up(nt, 256), 256, 0, s>>>(c.rowptr.p, nt, flag.p);
  ILG_CUDA(cudaGetLastError());
  ILG_TRY(scan_exclusive_u32_to_u64(flag.p, pos.p, nt, c.scan, s));
  unsigned long long lp = 0;
  uint32_t lf = 0;
  ILG_CUDA(cudaMemcpyAsync(&lp, pos.p + (nt - 1), 8, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaMemcpyAsync(&lf, flag.p + (nt - 1), 4, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  c.n_active = (int)(lp + lf);
  ILG_TRY(c.active.alloc(c.n_active > 0 ? c.n_active : 1));
  k_active_compact<<<div_up(nt, 256), 256, 0, s>>>(flag.p, pos.p, nt, c.active.p);
  ILG_CUDA(cudaGetLastError());
  // mixed-precision copy
  ILG_TRY(c.val_bf16.alloc(c.nnz > 0 ? c.nnz : 1));
  ILG_TRY(c.row_scale.alloc(nt));
  k_to_bf16<<<div_up(nt, 256), 256, 0, s>>>(c.rowptr.p, c.val.p, nt, c.val_bf16.p, c.row_scale.p);
  ILG_CUDA(cudaGetLastError());
  c.have_bf16 = true;

  // SELL-32 layout of the active rows, in Morton order. Inside the solve a
  // facet is addressed by its position in the LBVH's Morton order, so
  // facets near each other in space are near each other in memory. Rows are
  // grouped by length class (half octaves, longest first) and by Morton
  // position within a class; each row's entries are sorted by their
  // column's Morton position. Neighbouring lanes of a slice are then
  // neighbouring facets whose visible sets overlap, so the k-th columns of a
  // slice's 32 lanes fall in few cache lines. Rows longer than L are split
  // into nearly equal chunks in adjacent lanes of one slice; each slice is
  // column-major and padded to its longest chunk (rounded up to 4).
  // Per-row columns in Morton order, sorted on the device: key = (row,
  // Morton position of the column), value = CSR entry.
  int rb = 1;
  while ((1 << rb) < nt) ++rb;
  int64_t nnz = c.nnz;
  std::vector<int64_t> rp((size_t)nt + 1);
  std::vector<unsigned long long> skey((size_t)(nnz > 0 ? nnz : 1));
  std::vector<uint32_t> ssrc32((size_t)(nnz > 0 ? nnz : 1));
  std::vector<uint32_t> order((size_t)nt);
  ILG_CUDA(cudaMemcpyAsync(rp.data(), c.rowptr.p, rp.size() * 8, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaMemcpyAsync(order.data(), c.morton_order.p, (size_t)nt * 4, cudaMemcpyDeviceToHost, s));
  if (nnz > 0) {
    dbuf<uint32_t> drank, dsv;
    dbuf<unsigned long long> dkey;
    ILG_TRY(drank.alloc(nt));
    ILG_TRY(dkey.alloc(nnz));
    ILG_TRY(dsv.alloc(nnz));
    k_rank<<<div_up(nt, 256), 256, 0, s>>>(c.morton_order.p, nt, drank.p);
    ILG_CUDA(cudaGetLastError());
    k_row_keys<<<div_up(nt, 256), 256, 0, s>>>(c.rowptr.p, c.col.p, drank.p, nt, rb, dkey.p, dsv.p);
    ILG_CUDA(cudaGetLastError());
    ILG_TRY(radix_sort_u64(dkey.p, dsv.p, nnz, 2 * rb, c.sort, s));
    ILG_CUDA(cudaMemcpyAsync(skey.data(), dkey.p, (size_t)nnz * 8, cudaMemcpyDeviceToHost, s));
    ILG_CUDA(cudaMemcpyAsync(ssrc32.data(), dsv.p, (size_t)nnz * 4, cudaMemcpyDeviceToHost, s));
    ILG_CUDA(cudaStreamSynchronize(s));
  }
  ILG_CUDA(cudaStreamSynchronize(s));
  const unsigned long long cmask = (1ull << rb) - 1;
  std::vector<int32_t> rank((size_t)nt);
  for (int p = 0; p < nt; ++p) rank[order[p]] = p;
  std::vector<int> rows;
  int64_t maxlen = 0;
  for (int i = 0; i < nt; ++i)
    if (rp[i + 1] > rp[i]) { rows.push_back(i); maxlen = std::max<int64_t>(maxlen, rp[i + 1] - rp[i]); }
  auto len_class = [&](int i) {
    double l = (double)(rp[i + 1] - rp[i]);
    return (int)std::floor(2.0 * std::log2(l));
  };
  std::sort(rows.begin(), rows.end(), [&](int p, int q) {
    int cp = len_class(p), cq = len_class(q);
    return cp != cq ? cp > cq : rank[p] < rank[q];
  });
  // Inside windows of 256 Morton-consecutive rows of one class, longest
  // first: the slices cut from a window keep their spatial neighbourhood but
  // pad less.
  for (size_t a = 0; a < rows.size();) {
    size_t b = a;
    int ca = len_class(rows[a]);
    while (b < rows.size() && b - a < 256 && len_class(rows[b]) == ca) ++b;
    std::stable_sort(rows.begin() + a, rows.begin() + b,
                     [&](int p, int q) { return rp[p + 1] - rp[p] > rp[q + 1] - rp[q]; });
    a = b;
  }
  int64_t L = 64;                 // chunk length: bounds the per-sweep critical path
  while ((maxlen + L - 1) / L > 32) L *= 2;
  std::vector<int64_t> sl_ptr;
  std::vector<int32_t> sl_len, sl_split, ln_row, ln_m, ln_cnt;
  std::vector<int64_t> ln_first;   // offset of the lane's chunk in the sorted entries
  int lane = 32;   // force a new slice first
  int64_t off = 0;
  auto close_slice = [&]() {
    if (sl_len.empty()) return;
    while (lane < 32) {          // pad lanes
      ln_row.push_back(-1); ln_m.push_back(-1); ln_cnt.push_back(0); ln_first.push_back(0);
      ++lane;
    }
    int len = (sl_len.back() + 3) & ~3;
    sl_len.back() = len;
    off += (int64_t)len * 32;
  };
  for (int i : rows) {
    int64_t len = rp[i + 1] - rp[i];
    int64_t row0 = rp[i];   // the row's sorted entries: skey/ssrc32[rp[i], rp[i+1])
    int m = (int)((len + L - 1) / L);
    int64_t csz = (len + m - 1) / m;   // nearly equal chunks: little padding next to similar rows
    if (lane + m > 32) {
      close_slice();
      sl_ptr.push_back(off);
      sl_len.push_back(0);
      sl_split.push_back(1);
      lane = 0;
    }
    for (int k = 0; k < m; ++k) {
      int64_t first = (int64_t)k * csz;
      int cnt = (int)std::max<int64_t>(0, std::min<int64_t>(csz, len - first));
      ln_row.push_back(rank[i]);
      ln_m.push_back(k == 0 ? m : 0);
      ln_cnt.push_back(cnt);
      ln_first.push_back(row0 + first);
      sl_len.back() = std::max(sl_len.back(), cnt);
      ++lane;
    }
    sl_split.back() = std::max(sl_split.back(), m);
  }
  close_slice();
  c.sell_nslices = (int)sl_len.size();
  int ns = c.sell_nslices > 0 ? c.sell_nslices : 1;
  int64_t nel = off > 0 ? off : 1;
  // element arrays built on the host: column position and CSR source
  std::vector<int32_t> ecol((size_t)nel, 0);
  std::vector<int64_t> esrc((size_t)nel, -1);
  for (int sl = 0; sl < c.sell_nslices; ++sl)
    for (int l = 0; l < 32; ++l) {
      size_t li = (size_t)sl * 32 + l;
      for (int k = 0; k < ln_cnt[li]; ++k) {
        size_t o = (size_t)sl_ptr[sl] + (size_t)k * 32 + l;
        ecol[o] = (int32_t)(skey[ln_first[li] + k] & cmask);
        esrc[o] = (int64_t)ssrc32[ln_first[li] + k];
      }
    }
  ILG_TRY(c.sell_ptr.alloc(ns));
  ILG_TRY(c.sell_len.alloc(ns));
  ILG_TRY(c.sell_split.alloc(ns));
  ILG_TRY(c.sell_row.alloc((size_t)ns * 32));
  ILG_TRY(c.sell_m.alloc((size_t)ns * 32));
  ILG_TRY(c.sell_col.alloc(nel));
  ILG_TRY(c.sell_val.alloc(nel));
  ILG_TRY(c.sell_vbf.alloc(nel));
  ILG_TRY(c.rperm.alloc(nt));
  ILG_CUDA(cudaMemcpyAsync(c.rperm.p, order.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, s));
  if (c.sell_nslices > 0) {
    dbuf<int64_t> dsrc;
    ILG_TRY(dsrc.alloc(nel));
    ILG_CUDA(cudaMemcpyAsync(c.sell_ptr.p, sl_ptr.data(), sl_ptr.size() * 8, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.sell_len.p, sl_len.data(), sl_len.size() * 4, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.sell_split.p, sl_split.data(), sl_split.size() * 4, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.sell_row.p, ln_row.data(), ln_row.size() * 4, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.sell_m.p, ln_m.data(), ln_m.size() * 4, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.sell_col.p, ecol.data(), (size_t)nel * 4, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(dsrc.p, esrc.data(), (size_t)nel * 8, cudaMemcpyHostToDevice, s));
    k_sell_fill<<<div_up(nel, 256), 256, 0, s>>>(dsrc.p, nel, c.sell_ptr.p, c.sell_nslices, c.sell_row.p,
                                                c.rperm.p, c.val.p, c.row_scale.p, c.sell_val.p, c.sell_vbf.p);
    ILG_CUDA(cudaGetLastError());
    ILG_CUDA(cudaStreamSynchronize(s));
  }
  c.sell_elems = off;
  // residual-reduction chunks of the slices
  {
    int ns = c.sell_nslices;
    int nch = (ns + RAD_CHUNK - 1) / RAD_CHUNK;
    std::vector<int4> ch(nch > 0 ? nch : 1);
    for (int k = 0; k < nch; ++k) ch[k] = make_int4(k * RAD_CHUNK, std::min(RAD_CHUNK, ns - k * RAD_CHUNK), 0, 0);
    ILG_TRY(c.chunks.alloc(ch.size()));
    ILG_TRY(c.ch_d2.alloc(ch.size()));
    ILG_CUDA(cudaMemcpyAsync(c.chunks.p, ch.data(), ch.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
    c.nchunks = nch;
  }
  // per-facet flag: the row has entries
  std::vector<uint8_t> act((size_t)nt, 0);
  for (int i : rows) act[i] = 1;
  ILG_TRY(c.row_act.alloc(nt));
  ILG_CUDA(cudaMemcpyAsync(c.row_act.p, act.data(), (size_t)nt, cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  return ILG_OK;
}

// Cooperative grid size for nslices slices (at most the co-resident blocks).
int radiosity_chunk() { return RAD_CHUNK; }
int radiosity_max_meshes() { return RAD_MAX_MESH; }

int radiosity_grid(int nslices, int precision) {
  static int nsm = 0, per_sm64 = 0, per_smm = 0;
  if (!nsm) {
    int dev;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm64, k_radiosity64, RAD_THREADS, 0) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_smm, k_radiosity_mixed, RAD_THREADS, 0) != cudaSuccess) {
      nsm = 0;
      return 1;
    }
  }
  int per_sm = precision == ILG_PREC_MIXED ? per_smm : per_sm64;
  int want = div_up((int64_t)(nslices > 0 ? nslices : 1) * 32, RAD_THREADS);
  int grid = per_sm * nsm;
  if (want < grid) grid = want;
  return grid < 1 ? 1 : grid;
}

// Launches the cooperative solve for every active mesh of the view with
// slices. x: result (also the warm start when warm). Per-mesh sweep counts
// and residuals land in the mesh table.
int radiosity_launch(const StepView& v, double* x, int warm, int precision, int grid, cudaStream_t s) {
  ILG_CUDA(cudaMemsetAsync(v.barrier, 0, 2 * sizeof(unsigned), s));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(RAD_THREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;   // all blocks co-resident: the grid barrier is safe
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (precision == ILG_PREC_MIXED)
    ILG_CUDA(cudaLaunchKernelEx(&cfg, k_radiosity_mixed, v, x, warm));
  else
    ILG_CUDA(cudaLaunchKernelEx(&cfg, k_radiosity64, v, x, warm));
  return ILG_OK;
}

}  // namespace ilg
