// primitives.cu — device prefix scan and stable LSD radix sort used by the
// LBVH build (Morton codes) and the form-factor CSR assembly (row/column
// keys). Reduce-then-scan with 2048-element tiles; the radix sort ranks keys
// inside a tile with warp match masks, which keeps it stable.
#include "common.cuh"

namespace ilg {

namespace {

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

typedef unsigned long long u64;

template <class T>
__global__ void k_tile_sums(const T* __restrict__ in, u64* __restrict__ sums, int64_t n) {
  __shared__ u64 wsum[SCAN_THREADS / 32];
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  u64 s = 0;
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    int64_t idx = base + (int64_t)i * SCAN_THREADS + threadIdx.x;
    if (idx < n) s += (u64)in[idx];
  }
  for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    u64 v = threadIdx.x < SCAN_THREADS / 32 ? wsum[threadIdx.x] : 0;
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) sums[blockIdx.x] = v;
  }
}

// Exclusive scan of one tile (thread t owns SCAN_ITEMS consecutive elements),
// plus the tile's offset.
template <class T>
__global__ void k_tile_scan(const T* __restrict__ in, u64* __restrict__ out, int64_t n,
                            const u64* __restrict__ offsets) {
  __shared__ u64 wsum[SCAN_THREADS / 32];
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
  u64 v[SCAN_ITEMS];
  u64 local = 0;
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    int64_t idx = base + i;
    v[i] = idx < n ? (u64)in[idx] : 0;
    local += v[i];
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  u64 inc = local;
  for (int o = 1; o < 32; o <<= 1) {
    u64 y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    u64 x = lane < SCAN_THREADS / 32 ? wsum[lane] : 0;
    u64 xi = x;
    for (int o = 1; o < 32; o <<= 1) {
      u64 y = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += y;
    }
    if (lane < SCAN_THREADS / 32) wsum[lane] = xi - x;
  }
  __syncthreads();
  u64 run = (offsets ? offsets[blockIdx.x] : 0) + wsum[w] + (inc - local);
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    int64_t idx = base + i;
    if (idx < n) out[idx] = run;
    run += v[i];
  }
}

template <class T>
int scan_impl(const T* in, u64* out, int64_t n, ScanScratch& tmp, cudaStream_t s, int depth) {
  if (n <= 0) return ILG_OK;
  int nb = div_up(n, SCAN_TILE);
  if (nb == 1) {
    k_tile_scan<T><<<1, SCAN_THREADS, 0, s>>>(in, out, n, nullptr);
    ILG_CUDA(cudaGetLastError());
    return ILG_OK;
  }
  // level buffers: a (depth 0), b (depth 1), c (depth 2); three levels cover
  // 2048^3 elements.
  dbuf<u64>& sums = depth == 0 ? tmp.a : (depth == 1 ? tmp.b : tmp.c);
  if (depth > 2) { set_error("scan: input too large"); return ILG_ERR_ARG; }
  ILG_TRY(sums.reserve((size_t)nb));
  u64* sp = sums.p;
  k_tile_sums<T><<<nb, SCAN_THREADS, 0, s>>>(in, sp, n);
  ILG_CUDA(cudaGetLastError());
  ILG_TRY(scan_impl<u64>(sp, sp, nb, tmp, s, depth + 1));
  k_tile_scan<T><<<nb, SCAN_THREADS, 0, s>>>(in, out, n, sp);
  ILG_CUDA(cudaGetLastError());
  return ILG_OK;
}

// ---------------------------------------------------------------- radix sort
constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 8;                       // per thread
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;    // 2048 keys per block
constexpr int RS_WTILE = RS_TILE / RS_WARPS;      // 256 keys per warp

__global__ void k_radix_hist(const u64* __restrict__ keys, int64_t n, int shift, u64* __restrict__ hist,
                             int nblocks) {
  __shared__ unsigned h[256];
  for (int i = threadIdx.x; i < 256; i += RS_THREADS) h[i] = 0;
  __syncthreads();
  int64_t base = (int64_t)blockIdx.x * RS_TILE;
  for (int i = 0; i < RS_ITEMS; ++i) {
    int64_t idx = base + (int64_t)i * RS_THREADS + threadIdx.x;
    if (idx < n) atomicAdd(&h[(unsigned)((keys[idx] >> shift) & 255ull)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += RS_THREADS) hist[(int64_t)d * nblocks + blockIdx.x] = h[d];
}

template <bool HASV>
__global__ void k_radix_scatter(const u64* __restrict__ kin, const uint32_t* __restrict__ vin,
                                u64* __restrict__ kout, uint32_t* __restrict__ vout, int64_t n, int shift,
                                const u64* __restrict__ offs, int nblocks) {
  __shared__ unsigned wcnt[RS_WARPS][256];
  __shared__ u64 boff[256];
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < RS_WARPS * 256; i += RS_THREADS) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  int64_t wbase = (int64_t)blockIdx.x * RS_TILE + (int64_t)warp * RS_WTILE;
  u64 k[RS_ITEMS];
  uint32_t v[RS_ITEMS];
  unsigned rank[RS_ITEMS];
  int dig[RS_ITEMS];
  const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
  for (int it = 0; it < RS_ITEMS; ++it) {
    int64_t idx = wbase + it * 32 + lane;
    bool valid = idx < n;
    k[it] = valid ? kin[idx] : 0ull;
    if (HASV) v[it] = valid ? vin[idx] : 0u;
    int d = valid ? (int)((k[it] >> shift) & 255ull) : 256;
    dig[it] = d;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    unsigned before = peers & lt_mask;
    unsigned base = d < 256 ? wcnt[warp][d] : 0u;
    __syncwarp();
    if (d < 256 && before == 0) wcnt[warp][d] = base + __popc(peers);
    __syncwarp();
    rank[it] = base + __popc(before);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += RS_THREADS) {
    unsigned run = 0;
    for (int w = 0; w < RS_WARPS; ++w) {
      unsigned c = wcnt[w][d];
      wcnt[w][d] = run;
      run += c;
    }
    boff[d] = offs[(int64_t)d * nblocks + blockIdx.x];
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < RS_ITEMS; ++it) {
    int d = dig[it];
    if (d < 256) {
      u64 pos = boff[d] + wcnt[warp][d] + rank[it];
      kout[pos] = k[it];
      if (HASV) vout[pos] = v[it];
    }
  }
}

}  // namespace

int scan_exclusive_u64(const u64* in, u64* out, int64_t n, ScanScratch& tmp, cudaStream_t s) {
  return scan_impl<u64>(in, out, n, tmp, s, 0);
}
int scan_exclusive_u32_to_u64(const uint32_t* in, u64* out, int64_t n, ScanScratch& tmp, cudaStream_t s) {
  return scan_impl<uint32_t>(in, out, n, tmp, s, 0);
}

int radix_sort_u64(u64* keys, uint32_t* vals, int64_t n, int bits, SortScratch& tmp, cudaStream_t s) {
  if (n <= 1) return ILG_OK;
  int nb = div_up(n, RS_TILE);
  ILG_TRY(tmp.keys_alt.reserve((size_t)n));
  if (vals) ILG_TRY(tmp.vals_alt.reserve((size_t)n));
  ILG_TRY(tmp.hist.reserve((size_t)nb * 256));
  u64 *ka = keys, *kb = tmp.keys_alt.p;
  uint32_t *va = vals, *vb = vals ? tmp.vals_alt.p : nullptr;
  int passes = 0;
  for (int shift = 0; shift < bits; shift += 8, ++passes) {
    k_radix_hist<<<nb, RS_THREADS, 0, s>>>(ka, n, shift, tmp.hist.p, nb);
    ILG_CUDA(cudaGetLastError());
    ILG_TRY(scan_exclusive_u64(tmp.hist.p, tmp.hist.p, (int64_t)nb * 256, tmp.scan, s));
    if (vals)
      k_radix_scatter<true><<<nb, RS_THREADS, 0, s>>>(ka, va, kb, vb, n, shift, tmp.hist.p, nb);
    else
      k_radix_scatter<false><<<nb, RS_THREADS, 0, s>>>(ka, nullptr, kb, nullptr, n, shift, tmp.hist.p, nb);
    ILG_CUDA(cudaGetLastError());
    u64* t = ka; ka = kb; kb = t;
    uint32_t* tv = va; va = vb; vb = tv;
  }
  if (passes & 1) {
    ILG_CUDA(cudaMemcpyAsync(keys, ka, (size_t)n * 8, cudaMemcpyDeviceToDevice, s));
    if (vals) ILG_CUDA(cudaMemcpyAsync(vals, va, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
  }
  return ILG_OK;
}

}  // namespace ilg
