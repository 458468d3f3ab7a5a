// radiosity.cu — solve (I - F) x = E for the form-factor matrix (CSR by
// receiver row), the linear system the reference solves with a forward
// solve plus Gauss-Seidel sweeps (src/cpp/arma_util.cpp:4-17,
// src/cpp/illum_cli.cpp:425-440).
//
// GPU scheme: Jacobi sweeps x <- E + F x over the rows that have entries
// (rows without entries are x = E exactly), one warp per row with a fixed
// lane-strided summation order, inside ONE persistent cooperative kernel:
// a grid barrier separates sweeps and every block reduces the per-block
// residual partials in the same order, so all blocks take the same stop
// decision and results are run-to-run deterministic. The residual of
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
#include <vector>

#include "internal.cuh"

namespace ilg {

namespace {

constexpr int RAD_THREADS = 512;
constexpr int RAD_WARPS = RAD_THREADS / 32;

struct RadArgs {
  // SELL-32 copy of the active rows (see radiosity_prepare)
  const int64_t* sl_ptr;    // per slice: offset of its first element
  const int32_t* sl_len;    // per slice: elements per lane (multiple of 4)
  const int32_t* sl_split;  // per slice: largest chunk count of its rows (1: no split rows)
  const int32_t* ln_row;    // per lane: row, or -1 (padding lane)
  const int32_t* ln_m;      // per lane: chunks of its row if it is the row's first lane, else 0
  const int32_t* s_col;
  const double* s_val;
  const __nv_bfloat16* s_vbf;
  int nslices;
  const int64_t* rowptr;
  const int32_t* col;
  const double* val;
  const __nv_bfloat16* vbf;
  const float* rscale;
  const int32_t* active;
  int n_active, nt;
  const double* E;
  double* x;       // result (and warm start)
  double* xt;      // second iterate buffer
  double* xprev;   // solution of the step before (extrapolated warm start)
  float* x32a;     // fp32 iterate buffers (mixed)
  float* x32b;
  float* r32;      // fp32 correction right-hand side (mixed)
  double tol2;
  int max_sweeps;
  int warm;
  int mixed;
  double* partials;   // 2 x gridDim.x
  unsigned* bar;      // [0] arrival count, [1] generation
  int* counters;
  int* derr;
};

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

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < RAD_WARPS; ++i) t += sh[i];
  return t;
}

// Sum of the grid's partials in a fixed order (same value in every block).
__device__ __forceinline__ double grid_total(const double* part, int nb, double* sh) {
  double v = 0.0;
  for (int b = threadIdx.x; b < nb; b += RAD_THREADS) v += part[b];
  // fixed-order tree: warp shuffles then warps in order
  return block_sum(v, sh);
}

// sum_k val[k] * x[col[k]] over one row, lanes strided, four independent
// loads per lane in flight; fixed summation order (deterministic).
template <class V, class X, class Acc>
__device__ __forceinline__ Acc row_dot(const int32_t* __restrict__ col, const V* __restrict__ val,
                                       const X* __restrict__ x, int64_t b, int64_t e, int lane) {
  Acc s = 0;
  for (int64_t k0 = b; k0 < e; k0 += 128) {
    int c[4];
    V v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int64_t k = k0 + lane + 32 * j;
      bool ok = k < e;
      c[j] = ok ? __ldg(col + k) : 0;
      v[j] = ok ? __ldg(val + k) : V(0);
    }
    X xv[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) xv[j] = x[c[j]];
#pragma unroll
    for (int j = 0; j < 4; ++j) s += (Acc)v[j] * (Acc)xv[j];
  }
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// One SELL-32 slice: lane l accumulates its (chunk of a) row sequentially
// (four independent loads in flight), then rows split into several chunks
// are combined into their first lane in a fixed order.
template <class V, class X, class Acc>
__device__ __forceinline__ Acc slice_dot(const RadArgs& a, const V* __restrict__ sval, const X* __restrict__ x,
                                         int sl, int lane) {
  int64_t base = a.sl_ptr[sl] + lane;
  int len = a.sl_len[sl];
  Acc p = 0;
  for (int k = 0; k < len; k += 4) {
    int c[4];
    V v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      c[j] = __ldg(a.s_col + base + (int64_t)(k + j) * 32);
      v[j] = __ldg(sval + base + (int64_t)(k + j) * 32);
    }
    X xv[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) xv[j] = x[c[j]];
#pragma unroll
    for (int j = 0; j < 4; ++j) p += (Acc)v[j] * (Acc)xv[j];
  }
  int mmax = a.sl_split[sl];
  if (mmax > 1) {
    int m = a.ln_m[(int64_t)sl * 32 + lane];
    Acc tot = p;
    for (int j = 1; j < mmax; ++j) {
      Acc q = __shfl_down_sync(0xffffffffu, p, j);
      if (j < m) tot += q;
    }
    p = tot;
  }
  return p;
}

// FP64 Jacobi to tolerance.
__global__ void __launch_bounds__(RAD_THREADS, 2) k_radiosity64(RadArgs a) {
  __shared__ double sh[RAD_WARPS];
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * RAD_THREADS + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * RAD_THREADS) >> 5;
  const int gt = blockIdx.x * RAD_THREADS + threadIdx.x;
  const int nthreads = gridDim.x * RAD_THREADS;
  // all rows: both buffers start at E (inactive rows keep it); active rows
  // of x keep the previous solution when warm-starting
  // warm start: x_{n-1} (or 2 x_{n-1} - x_{n-2} once two solutions exist)
  const bool extrap = a.warm && a.counters[2] >= 2;
  for (int i = gt; i < a.nt; i += nthreads) {
    double e = a.E[i];
    a.xt[i] = e;
    bool act = a.rowptr[i + 1] != a.rowptr[i];
    if (!a.warm || !act) {
      a.x[i] = e;
    } else {
      double xn = a.x[i];
      if (extrap) a.x[i] = 2.0 * xn - a.xprev[i];
      a.xprev[i] = xn;
    }
  }
  if (!grid_barrier(a.bar, gridDim.x, a.derr)) return;
  double* cur = a.x;
  double* nxt = a.xt;
  int sweeps = 0;
  for (;;) {
    double d2 = 0.0;
    for (int sl = gw; sl < a.nslices; sl += nwarps) {
      double s = slice_dot<double, double, double>(a, a.s_val, cur, sl, lane);
      int64_t li = (int64_t)sl * 32 + lane;
      if (a.ln_m[li] > 0) {
        int i = a.ln_row[li];
        double xn = a.E[i] + s;
        double df = xn - cur[i];
        nxt[i] = xn;
        d2 += df * df;
      }
    }
    ++sweeps;
    double bs = block_sum(d2, sh);
    double* part = a.partials + (sweeps & 1) * gridDim.x;
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
    if (!grid_barrier(a.bar, gridDim.x, a.derr)) return;
    double tot = grid_total(part, gridDim.x, sh);
    double* t = cur; cur = nxt; nxt = t;
    if (tot <= a.tol2 || sweeps >= a.max_sweeps) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.counters[3] = sweeps;
        a.partials[2 * gridDim.x] = tot;
      }
      break;
    }
  }
  // make sure the final iterate is in x
  if (cur != a.x) {
    for (int w = gt; w < a.n_active; w += nthreads) {
      int i = a.active[w];
      a.x[i] = cur[i];
    }
  }
}

// Mixed precision: outer refinement with an fp64 residual r = E - (I - F) x
// (fp64 values), inner fp32 Jacobi on (I - F~) d = r with bf16 F~, x += d.
// The outer loop stops when ||r||_2 <= tol.
__global__ void __launch_bounds__(RAD_THREADS, 2) k_radiosity_mixed(RadArgs a) {
  __shared__ double sh[RAD_WARPS];
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * RAD_THREADS + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * RAD_THREADS) >> 5;
  const int gt = blockIdx.x * RAD_THREADS + threadIdx.x;
  const int nthreads = gridDim.x * RAD_THREADS;
  const bool extrap = a.warm && a.counters[2] >= 2;
  for (int i = gt; i < a.nt; i += nthreads) {
    bool act = a.rowptr[i + 1] != a.rowptr[i];
    if (!a.warm || !act) {
      a.x[i] = a.E[i];
    } else {
      double xn = a.x[i];
      if (extrap) a.x[i] = 2.0 * xn - a.xprev[i];
      a.xprev[i] = xn;
    }
    a.x32a[i] = 0.f;
    a.x32b[i] = 0.f;
  }
  if (!grid_barrier(a.bar, gridDim.x, a.derr)) return;
  int sweeps = 0, outer = 0;
  for (;;) {
    // fp64 residual on active rows (inactive rows are exact)
    double r2 = 0.0;
    for (int sl = gw; sl < a.nslices; sl += nwarps) {
      double s = slice_dot<double, double, double>(a, a.s_val, a.x, sl, lane);
      int64_t li = (int64_t)sl * 32 + lane;
      if (a.ln_m[li] > 0) {
        int i = a.ln_row[li];
        double r = a.E[i] + s - a.x[i];
        a.r32[i] = (float)r;
        a.x32a[i] = (float)r;     // inner start: d0 = r
        r2 += r * r;
      }
    }
    double bs = block_sum(r2, sh);
    double* part = a.partials + (outer & 1) * gridDim.x;
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
    if (!grid_barrier(a.bar, gridDim.x, a.derr)) return;
    double tot = grid_total(part, gridDim.x, sh);
    ++outer;
    if (tot <= a.tol2 || sweeps >= a.max_sweeps) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.counters[3] = sweeps;
        a.partials[2 * gridDim.x] = tot;
      }
      return;
    }
    // inner fp32 Jacobi: d <- r + F~ d, a fixed 4 sweeps (each gains ~1.5 digits)
    float* cur = a.x32a;
    float* nxt = a.x32b;
    for (int it = 0; it < 4; ++it) {
      for (int sl = gw; sl < a.nslices; sl += nwarps) {
        float s = slice_dot<__nv_bfloat16, float, float>(a, a.s_vbf, cur, sl, lane);
        int64_t li = (int64_t)sl * 32 + lane;
        if (a.ln_m[li] > 0) {
          int i = a.ln_row[li];
          nxt[i] = a.r32[i] + a.rscale[i] * s;
        }
      }
      ++sweeps;
      if (!grid_barrier(a.bar, gridDim.x, a.derr)) return;
      float* t = cur; cur = nxt; nxt = t;
    }
    for (int w = gt; w < a.n_active; w += nthreads) {
      int i = a.active[w];
      a.x[i] += (double)cur[i];
    }
    if (!grid_barrier(a.bar, gridDim.x, a.derr)) return;
  }
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

// SELL fill: lane (slice, l) copies elements [first, first + cnt) of its row
// into column k of the slice; the rest of the slice column is padding
// (column = 0, value = 0).
__global__ void k_sell_fill(const int64_t* __restrict__ sl_ptr, const int32_t* __restrict__ sl_len,
                            const int64_t* __restrict__ ln_first, const int32_t* __restrict__ ln_cnt,
                            const int32_t* __restrict__ ln_row, const int32_t* __restrict__ col,
                            const double* __restrict__ val, const float* __restrict__ rscale, int nslices,
                            int32_t* s_col, double* s_val, __nv_bfloat16* s_vbf) {
  int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (int64_t)nslices * 32) return;
  int sl = (int)(g >> 5), lane = (int)(g & 31);
  int len = sl_len[sl];
  int64_t base = sl_ptr[sl] + lane;
  int64_t first = ln_first[g];
  int cnt = ln_cnt[g];
  int row = ln_row[g];
  float sc = row >= 0 ? rscale[row] : 1.f;
  for (int k = 0; k < len; ++k) {
    int64_t o = base + (int64_t)k * 32;
    if (k < cnt) {
      s_col[o] = col[first + k];
      s_val[o] = val[first + k];
      s_vbf[o] = __float2bfloat16_rn((float)(val[first + k] / (double)sc));
    } else {
      s_col[o] = 0;
      s_val[o] = 0.0;
      s_vbf[o] = __float2bfloat16_rn(0.f);
    }
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

  // SELL-32 layout of the active rows: rows sorted by length (longest
  // first), rows longer than L split into chunks of at most L placed in
  // adjacent lanes of one slice, each slice column-major and padded to the
  // longest chunk (rounded up to 4).
  std::vector<int64_t> rp((size_t)nt + 1);
  ILG_CUDA(cudaMemcpyAsync(rp.data(), c.rowptr.p, rp.size() * 8, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  std::vector<int> rows;
  int64_t maxlen = 0;
  for (int i = 0; i < nt; ++i)
    if (rp[i + 1] > rp[i]) { rows.push_back(i); maxlen = std::max<int64_t>(maxlen, rp[i + 1] - rp[i]); }
  std::stable_sort(rows.begin(), rows.end(), [&](int p, int q) { return rp[p + 1] - rp[p] > rp[q + 1] - rp[q]; });
  int64_t L = 32;                 // chunk length: bounds the per-sweep critical path
  while ((maxlen + L - 1) / L > 32) L *= 2;
  std::vector<int64_t> sl_ptr;
  std::vector<int32_t> sl_len, sl_split, ln_row, ln_m, ln_cnt;
  std::vector<int64_t> ln_first;
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
    int m = (int)((len + L - 1) / L);
    if (lane + m > 32) {
      close_slice();
      sl_ptr.push_back(off);
      sl_len.push_back(0);
      sl_split.push_back(1);
      lane = 0;
    }
    for (int k = 0; k < m; ++k) {
      int64_t first = rp[i] + (int64_t)k * L;
      int cnt = (int)std::min<int64_t>(L, rp[i + 1] - first);
      ln_row.push_back(i);
      ln_m.push_back(k == 0 ? m : 0);
      ln_cnt.push_back(cnt);
      ln_first.push_back(first);
      sl_len.back() = std::max(sl_len.back(), cnt);
      ++lane;
    }
    sl_split.back() = std::max(sl_split.back(), m);
  }
  close_slice();
  c.sell_nslices = (int)sl_len.size();
  int ns = c.sell_nslices > 0 ? c.sell_nslices : 1;
  int64_t nel = off > 0 ? off : 1;
  ILG_TRY(c.sell_ptr.alloc(ns));
  ILG_TRY(c.sell_len.alloc(ns));
  ILG_TRY(c.sell_split.alloc(ns));
  ILG_TRY(c.sell_row.alloc((size_t)ns * 32));
  ILG_TRY(c.sell_m.alloc((size_t)ns * 32));
  ILG_TRY(c.sell_col.alloc(nel));
  ILG_TRY(c.sell_val.alloc(nel));
  ILG_TRY(c.sell_vbf.alloc(nel));
  if (c.sell_nslices > 0) {
    dbuf<int64_t> dfirst;
    dbuf<int32_t> dcnt;
    ILG_TRY(dfirst.alloc(ln_first.size()));
    ILG_TRY(dcnt.alloc(ln_cnt.size()));
    ILG_CUDA(cudaMemcpyAsync(c.sell_ptr.p, sl_ptr.data(), sl_ptr.size() * 8, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.sell_len.p, sl_len.data(), sl_len.size() * 4, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.sell_split.p, sl_split.data(), sl_split.size() * 4, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.sell_row.p, ln_row.data(), ln_row.size() * 4, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.sell_m.p, ln_m.data(), ln_m.size() * 4, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(dfirst.p, ln_first.data(), ln_first.size() * 8, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(dcnt.p, ln_cnt.data(), ln_cnt.size() * 4, cudaMemcpyHostToDevice, s));
    int64_t nl = (int64_t)c.sell_nslices * 32;
    k_sell_fill<<<div_up(nl, 256), 256, 0, s>>>(c.sell_ptr.p, c.sell_len.p, dfirst.p, dcnt.p, c.sell_row.p, c.col.p,
                                               c.val.p, c.row_scale.p, c.sell_nslices, c.sell_col.p, c.sell_val.p,
                                               c.sell_vbf.p);
    ILG_CUDA(cudaGetLastError());
    ILG_CUDA(cudaStreamSynchronize(s));
  }
  c.sell_elems = off;
  return ILG_OK;
}

// Sizes the cooperative grid and reserves the solve's buffers. Called
// before any stream capture (no allocation may happen while capturing).
int radiosity_setup(Context& c, int precision) {
  static int nsm = 0, per_sm64 = 0, per_smm = 0;
  if (!nsm) {
    int dev;
    ILG_CUDA(cudaGetDevice(&dev));
    ILG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    ILG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm64, k_radiosity64, RAD_THREADS, 0));
    ILG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_smm, k_radiosity_mixed, RAD_THREADS, 0));
  }
  bool mixed = precision == ILG_PREC_MIXED;
  int per_sm = mixed ? per_smm : per_sm64;
  int want = div_up((int64_t)(c.sell_nslices > 0 ? c.sell_nslices : 1) * 32, RAD_THREADS);
  int grid = per_sm * nsm;
  if (want < grid) grid = want;
  if (grid < 1) grid = 1;
  ILG_TRY(c.partials.reserve((size_t)2 * grid + 2));
  ILG_TRY(c.xtmp.reserve(c.nt));
  if (c.xprev.n < (size_t)c.nt) {
    ILG_TRY(c.xprev.alloc(c.nt));
    ILG_CUDA(cudaMemset(c.xprev.p, 0, (size_t)c.nt * 8));
  }
  if (mixed) ILG_TRY(c.x32.reserve((size_t)3 * c.nt));
  c.rad_grid = grid;
  c.rad_grid_prec = precision;
  return ILG_OK;
}

// Launches the cooperative solve on c.stream. x_dev: result (also the warm
// start when warm_start). Sweep count lands in counters[3] and the final
// squared residual in partials[2*grid].
int radiosity_launch(Context& c, const double* E_dev, double* x_dev, double tol, int max_sweeps, int precision,
                     bool warm_start) {
  if (c.rad_grid_prec != precision || c.rad_grid < 1) ILG_TRY(radiosity_setup(c, precision));
  bool mixed = precision == ILG_PREC_MIXED;
  int grid = c.rad_grid;
  RadArgs a;
  a.sl_ptr = c.sell_ptr.p; a.sl_len = c.sell_len.p; a.sl_split = c.sell_split.p; a.ln_row = c.sell_row.p;
  a.ln_m = c.sell_m.p; a.s_col = c.sell_col.p; a.s_val = c.sell_val.p; a.s_vbf = c.sell_vbf.p;
  a.nslices = c.sell_nslices;
  a.rowptr = c.rowptr.p; a.col = c.col.p; a.val = c.val.p; a.vbf = c.val_bf16.p; a.rscale = c.row_scale.p;
  a.active = c.active.p; a.n_active = c.n_active; a.nt = c.nt;
  a.E = E_dev; a.x = x_dev; a.xt = c.xtmp.p; a.xprev = c.xprev.p;
  a.x32a = mixed ? c.x32.p : nullptr;
  a.x32b = mixed ? c.x32.p + c.nt : nullptr;
  a.r32 = mixed ? c.x32.p + 2 * (size_t)c.nt : nullptr;
  a.tol2 = tol * tol; a.max_sweeps = max_sweeps; a.warm = warm_start ? 1 : 0; a.mixed = mixed ? 1 : 0;
  a.partials = c.partials.p; a.bar = (unsigned*)c.barrier.p; a.counters = c.counters.p; a.derr = c.derr.p;
  ILG_CUDA(cudaMemsetAsync(c.barrier.p, 0, 2 * sizeof(unsigned), c.stream));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(RAD_THREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = c.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;   // all blocks co-resident: the grid barrier is safe
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (mixed)
    ILG_CUDA(cudaLaunchKernelEx(&cfg, k_radiosity_mixed, a));
  else
    ILG_CUDA(cudaLaunchKernelEx(&cfg, k_radiosity64, a));
  return ILG_OK;
}

}  // namespace ilg
