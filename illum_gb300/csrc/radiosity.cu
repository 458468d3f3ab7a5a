// radiosity.cu — solve (I - F) x = E for the form-factor matrix (CSR by
// receiver row), the linear system the reference solves with a forward
// solve plus Gauss-Seidel sweeps (src/cpp/arma_util.cpp:4-17,
// src/cpp/illum_cli.cpp:425-440).
//
// GPU scheme: Jacobi sweeps x <- E + F x over the rows that have entries
// (rows without entries are x = E exactly) inside ONE persistent cooperative
// kernel, one grid barrier per sweep. The solve works on facets renumbered in
// the LBVH's Morton order, and the matrix is cut into row tiles: runs of
// Morton-consecutive rows with about nnz / (co-resident blocks) entries each.
// A tile's rows see a compact set of facets (its halo), so a block first
// gathers the halo's x values into shared memory and then streams the tile's
// entries, each a 16-bit halo index (plus a row-end bit) and a value. The
// stream reaches shared memory by bulk copies (cp.async.bulk with mbarrier
// completion) that one producer warp issues ahead of the 31 consumer warps,
// so DRAM keeps working while the consumers gather the next tile's halo or
// finish a tile's rows. The
// tile's entries, row after row, are split into equal runs, one per thread
// (entries of a row that straddles threads are combined in a fixed order),
// so every thread of every block does the same amount of work whatever the
// row lengths. The per-tile residual partials meet in integer accumulators
// (order-independent sums), so all blocks take the same stop decisions and
// results are run-to-run deterministic. The residual of iterate x_k is
// E - (I - F) x_k = x_{k+1} - x_k, so it comes for free with the next sweep;
// iteration stops once its 2-norm is <= tol.
// With albedo-scaled form factors the iteration matrix has spectral radius
// well below 1, so Jacobi converges in a handful of sweeps; a multicolour
// Gauss-Seidel would need one grid barrier per colour, and the cliques of
// mutually visible crater facets force hundreds of colours.
//
// FP64 arithmetic runs at about one fused multiply-add per clock per SM on
// GB300, so the double-precision sweeps evaluate their dot products in
// FP32-pair ("double-float") arithmetic on the FP32 pipes instead: each
// value and each x is split into hi + lo floats (48 significant bits), the
// product hi*hi is taken exactly with an FMA, the cross terms are added,
// and the running sum is kept as an unevaluated float pair by TwoSum
// (Dekker 1971; Knuth TAOCP vol. 2, 4.2.2). The relative error of a row sum
// is ~2^-46 (vs 2^-53 for FP64), orders of magnitude below the solve
// tolerance. The iterate is kept as its scattered part s = x - E, also a
// double-float, with E in FP64: x = E + s is formed in FP64 only when the
// solve ends, so the result carries E exactly and s to ~2^-46 of |s|
// (|s| <= albedo * max x). Per row and sweep the finishing work (s' = F x,
// the change s' - s, the halo copy x' = E + s') is FP32 arithmetic, and the
// squared changes are summed in FP32 (a stop decision needs a few digits).
//
// The double-float values are stored as two arrays, hi = fl(F) and
// lo = fl(F - hi).
//
// Mixed precision: values stored as bf16 with a per-row fp32 scale, fp32
// accumulation for the inner sweeps, and an outer refinement whose residual
// r = fl(F) x - s is accumulated in double-float from the fp32 values hi (x and
// s in double-float, E in FP64, r rounded to fp32 for the inner sweeps): the
// fixed point is that of (I - fl(F)) x = E,
// within ~1e-7 of the scattered flux of the fp64 system's. A mesh whose
// sweep budget runs out in a refinement round stops after the round's update
// without another residual pass. A round runs min(budget, RAD_INNER) inner
// sweeps (the smallest budget of the launch's meshes), so max_sweeps = 1 or
// 2 gives one refinement round per step (the next step's first residual
// includes what is left).
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <limits>
#include <mutex>
#include <thread>
#include <vector>

#include "internal.cuh"

namespace ilg {

namespace {

constexpr int RAD_THREADS = 992;             // consumer threads (31 warps): one entry run each
constexpr int RAD_BLOCK = RAD_THREADS + 32;  // and one producer warp that issues the entry-stream copies
constexpr int RAD_HALO = 8192;           // halo values per tile (double-float: 64 KB of shared memory)
constexpr int RAD_ROWS = 3072;           // rows per tile (their sums: 24 KB of shared memory)
constexpr int RAD_MAX_MESH = 1024;
constexpr int RAD_INNER = 2;             // most fp32 sweeps per refinement of the mixed solve: the bf16 error
                                         // (~4e-3 of the correction) already dominates rho^(k+1), rho ~ 0.013
constexpr int64_t RAD_MIN_TILE = 16384;  // entries: smaller tiles cost more in staging than they balance
constexpr int64_t RAD_SPLIT_MIN = 131072;  // entries: tiles above twice the split target are halved
// Tile balance, in stored entries: a block's sweep time is about
// c + 1.35e-4 us per stored entry + 8.8e-4 us per row + 1.5e-4 us per halo
// facet (per-block timings of the FP64 sweep on GB300, 152 tiles of an
// 81,920-facet mesh), i.e. a row costs ~7 entries and a halo facet ~1.
constexpr int64_t RAD_ROW_COST = 7;
constexpr int64_t RAD_HALO_COST = 1;
constexpr int64_t RAD_GROUP = 4 * RAD_THREADS;  // stored entries per group (4 per thread): a tile's stream is whole groups
// One group in shared memory: its columns (u16), then its values (f32 hi,
// f32 lo for the FP64 sweeps; f32 hi for the mixed residual; bf16 for the
// mixed inner sweeps). Every piece is a multiple of 16 bytes, and a group
// starts at a multiple of RAD_GROUP entries, so each is one bulk copy.
constexpr int RAD_CF_BYTES = (int)RAD_GROUP * 2;
constexpr int RAD_F32_BYTES = (int)RAD_GROUP * 4;
constexpr int RAD_STAGE64 = RAD_CF_BYTES + 2 * RAD_F32_BYTES;   // FP64 sweeps: 3 stages
constexpr int RAD_STAGEM = RAD_CF_BYTES + RAD_F32_BYTES;        // mixed solve: 5 stages
constexpr int RAD_NST64 = 3;
constexpr int RAD_NSTM = 5;
constexpr int RAD_NST_MAX = 8;
constexpr size_t RAD_RING = (size_t)(RAD_NST64 * RAD_STAGE64 > RAD_NSTM * RAD_STAGEM ? RAD_NST64 * RAD_STAGE64
                                                                                        : RAD_NSTM * RAD_STAGEM);
static_assert(RAD_CF_BYTES % 16 == 0 && RAD_F32_BYTES % 16 == 0, "bulk copies move multiples of 16 bytes");
static_assert(RAD_NST64 <= RAD_NST_MAX && RAD_NSTM <= RAD_NST_MAX, "stage barriers");
constexpr size_t RAD_SMEM = RAD_RING + (size_t)RAD_HALO * sizeof(float2) + RAD_THREADS * sizeof(float2) +
                            RAD_ROWS * sizeof(float2) + RAD_THREADS + 2 * RAD_NST_MAX * sizeof(unsigned long long);

// Most polls of one grid-barrier wait (about 2^26 x 32 ns before it gives
// up). A device variable so that a test can shrink it (ilg_debug_barrier_
// timeout) and watch a wait run out without a long stall.
constexpr long long BARRIER_POLLS = 1LL << 26;
__device__ long long g_barrier_polls = BARRIER_POLLS;

// Grid barrier for a cooperative launch (all blocks co-resident) on an
// arrival counter that only grows during the launch (zeroed before it):
// every block counts its barriers in gen, and barrier number gen opens once
// the counter reaches gen * nblocks, so the last block to arrive releases
// the others with its own increment (no reset on the critical path). The
// wait is bounded: after g_barrier_polls polls it records DERR_BARRIER and
// returns false (as does every block that sees the flag while waiting).
// The fences make the iterates written before the barrier visible to the
// loads after it.
__device__ bool grid_barrier(unsigned* bar, unsigned nblocks, unsigned& gen, int* derr) {
  __shared__ int ok;
  ++gen;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    const unsigned target = gen * nblocks;
    const long long limit = g_barrier_polls;
    __threadfence();
    if (atomicAdd(bar, 1u) + 1u < target) {
      long long it = 0;
      while (*(volatile unsigned*)bar < target) {
        if (++it > limit || *(volatile int*)&derr[DERR_BARRIER]) {
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

// Matrix loads: read-only for the whole solve, so the non-coherent path, no
// L1 allocation (each entry is used once per sweep), and an L2 evict-last
// policy on 3/4 of the lines so that repeated sweeps find most of the
// matrix in L2 when it is about as large as L2. A matrix much larger than
// L2 is streamed with evict-first instead (nothing of it survives until the
// next pass, and evict-last lines would only crowd out the iterates).
__device__ __forceinline__ uint64_t l2_keep_policy(int stream) {
  uint64_t pol;
  if (stream)
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  else
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 0.75;" : "=l"(pol));
  return pol;
}
// The entry stream of a block's tiles reaches shared memory by 1-D bulk
// copies (cp.async.bulk) into a ring of stages: the producer warp's lane 0
// waits until a stage is free (its empty barrier), announces the bytes on the
// stage's full barrier and issues the copies; consumers wait on the full
// barrier, read their four entries and arrive on the empty barrier. Both
// sides walk the same sequence of (tile, group) pairs, numbered q from the
// start of the launch: stage q % nst, use number q / nst, so each wait is on
// the parity of that use. Every wait is bounded: after RAD_MBAR_POLLS polls
// it records DERR_STREAM, and from then on the block's waits return at once
// and its consumers treat the stream as empty (all-zero entries, which index
// no halo value beyond slot 0 and end no row).
constexpr long long RAD_MBAR_POLLS = 1LL << 22;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// true once the use with this parity has completed; false after the poll
// limit (flagged) or when the block's stream has already failed
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int* bad, int* derr) {
  if (*(volatile int*)bad) return false;
  const unsigned a = smem_u32(bar);
  for (long long it = 0; it < RAD_MBAR_POLLS; ++it) {
    unsigned done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done) : "r"(a), "r"(parity) : "memory");
    if (done) return true;
    if (*(volatile int*)bad) return false;
  }
  *(volatile int*)bad = 1;
  atomicExch(&derr[DERR_STREAM], 1);
  return false;
}
__device__ __forceinline__ void bulk_copy(unsigned dst, const void* src, unsigned bytes, unsigned long long* bar,
                                          uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;"
      ::"r"(dst), "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol) : "memory");
}

// Value sources of tile_rows: how a group's values are copied into a stage
// (after its columns) and read back, four consecutive entries per thread.
struct ValsDF { const float* hi; const float* lo; };   // double-float (hi, lo)
struct ValsHi { const float* hi; };                    // fl(F) as a double-float with lo = 0
struct ValsBF { const __nv_bfloat16* v; };             // bf16, scaled per row
struct ValsHiF { const float* hi; };                   // fl(F) as a float
__device__ __forceinline__ unsigned vals_bytes(ValsDF) { return 2 * RAD_F32_BYTES; }
__device__ __forceinline__ unsigned vals_bytes(ValsHi) { return RAD_F32_BYTES; }
__device__ __forceinline__ unsigned vals_bytes(ValsHiF) { return RAD_F32_BYTES; }
__device__ __forceinline__ unsigned vals_bytes(ValsBF) { return RAD_CF_BYTES; }
__device__ __forceinline__ void copy_vals(ValsDF s, unsigned dst, size_t e, unsigned long long* bar, uint64_t pol) {
  bulk_copy(dst, s.hi + e, RAD_F32_BYTES, bar, pol);
  bulk_copy(dst + RAD_F32_BYTES, s.lo + e, RAD_F32_BYTES, bar, pol);
}
__device__ __forceinline__ void copy_vals(ValsHi s, unsigned dst, size_t e, unsigned long long* bar, uint64_t pol) {
  bulk_copy(dst, s.hi + e, RAD_F32_BYTES, bar, pol);
}
__device__ __forceinline__ void copy_vals(ValsHiF s, unsigned dst, size_t e, unsigned long long* bar, uint64_t pol) {
  bulk_copy(dst, s.hi + e, RAD_F32_BYTES, bar, pol);
}
__device__ __forceinline__ void copy_vals(ValsBF s, unsigned dst, size_t e, unsigned long long* bar, uint64_t pol) {
  bulk_copy(dst, s.v + e, RAD_CF_BYTES, bar, pol);
}
__device__ __forceinline__ void read_vals(ValsDF, const unsigned char* st, int tid, float2 (&w)[4]) {
  const float4 h = *reinterpret_cast<const float4*>(st + 16 * tid);
  const float4 l = *reinterpret_cast<const float4*>(st + RAD_F32_BYTES + 16 * tid);
  w[0] = make_float2(h.x, l.x);
  w[1] = make_float2(h.y, l.y);
  w[2] = make_float2(h.z, l.z);
  w[3] = make_float2(h.w, l.w);
}
__device__ __forceinline__ void read_vals(ValsHi, const unsigned char* st, int tid, float2 (&w)[4]) {
  const float4 h = *reinterpret_cast<const float4*>(st + 16 * tid);
  w[0] = make_float2(h.x, 0.f);
  w[1] = make_float2(h.y, 0.f);
  w[2] = make_float2(h.z, 0.f);
  w[3] = make_float2(h.w, 0.f);
}
__device__ __forceinline__ void read_vals(ValsHiF, const unsigned char* st, int tid, float (&w)[4]) {
  const float4 h = *reinterpret_cast<const float4*>(st + 16 * tid);
  w[0] = h.x;
  w[1] = h.y;
  w[2] = h.z;
  w[3] = h.w;
}
__device__ __forceinline__ void read_vals(ValsBF, const unsigned char* st, int tid, float (&w)[4]) {
  const uint2 r = *reinterpret_cast<const uint2*>(st + 8 * tid);
  w[0] = __uint_as_float(r.x << 16);
  w[1] = __uint_as_float(r.x & 0xffff0000u);
  w[2] = __uint_as_float(r.y << 16);
  w[3] = __uint_as_float(r.y & 0xffff0000u);
}
template <class W> __device__ __forceinline__ void zero_vals(W (&w)[4]);
template <> __device__ __forceinline__ void zero_vals(float2 (&w)[4]) {
  for (int j = 0; j < 4; ++j) w[j] = make_float2(0.f, 0.f);
}
template <> __device__ __forceinline__ void zero_vals(float (&w)[4]) {
  for (int j = 0; j < 4; ++j) w[j] = 0.f;
}

// The block's stream ring and its sequence position (per thread; every
// consumer and the producer lane advance it identically).
struct Pipe {
  unsigned char* ring;
  unsigned long long* full;
  unsigned long long* empty;
  int* bad;
  int nst;
  int stage_bytes;
  unsigned q;
};

// Producer (lane 0 of the producer warp): the copies of every group of tile T.
template <class V>
__device__ __forceinline__ void produce_tile(Pipe& p, const StepView& v, const RowTile& T, V vals, uint64_t pol) {
  const int ng = T.lam >> 2;
  const unsigned bytes = (unsigned)RAD_CF_BYTES + vals_bytes(vals);
  for (int g = 0; g < ng; ++g, ++p.q) {
    const unsigned s = p.q % (unsigned)p.nst, n = p.q / (unsigned)p.nst;
    if (n > 0 && !mbar_wait(p.empty + s, (n - 1) & 1u, p.bad, v.derr)) continue;
    if (*(volatile int*)p.bad) continue;
    const unsigned dst = smem_u32(p.ring + (size_t)s * p.stage_bytes);
    const size_t e = (size_t)T.e0 + (size_t)g * RAD_GROUP;
    mbar_expect(p.full + s, bytes);
    bulk_copy(dst, v.t_cf + e, RAD_CF_BYTES, p.full + s, pol);
    copy_vals(vals, dst + RAD_CF_BYTES, e, p.full + s, pol);
  }
}

// Consumer: the next group's four entries of this thread (columns and
// values), then the stage is released.
template <class V, class W>
__device__ __forceinline__ void take_group(Pipe& p, const StepView& v, V vals, uint2& c, W (&w)[4]) {
  const unsigned s = p.q % (unsigned)p.nst, n = p.q / (unsigned)p.nst;
  ++p.q;
  const unsigned char* st = p.ring + (size_t)s * p.stage_bytes;
  if (mbar_wait(p.full + s, n & 1u, p.bad, v.derr)) {
    c = *reinterpret_cast<const uint2*>(st + 8 * threadIdx.x);
    read_vals(vals, st + RAD_CF_BYTES, threadIdx.x, w);
  } else {
    c = make_uint2(0u, 0u);
    zero_vals(w);
  }
  mbar_arrive(p.empty + s);
}

// Barrier of the consumer threads only (the producer warp does not take
// part in the tile work).
__device__ __forceinline__ void cbar() { asm volatile("bar.sync 1, %0;" ::"n"(RAD_THREADS) : "memory"); }

__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Double-float: v = hi + lo with hi = fl(v), lo = fl(v - hi).
__device__ __forceinline__ float2 split_df(double x) {
  float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(x - (double)h));
}

// Running sum of double-float products. add(): p + e = w.hi * x.hi exactly
// (FMA), plus the cross terms w.hi * x.lo + w.lo * x.hi in e; (h, l) += p
// by TwoSum, l += e. Intrinsics keep the compiler from contracting or
// reassociating the error-free steps.
struct AccDF {
  typedef float2 W;
  typedef float2 X;
  typedef float2 Part;
  typedef float2 Sum;
  float h, l;
  __device__ __forceinline__ void zero() { h = 0.f; l = 0.f; }
  __device__ __forceinline__ void two_sum(float p) {
    float t = __fadd_rn(h, p);
    float bp = __fsub_rn(t, h);
    float err = __fadd_rn(__fsub_rn(h, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    h = t;
    l = __fadd_rn(l, err);
  }
  __device__ __forceinline__ void add(float2 w, float2 x) {
    float p = __fmul_rn(w.x, x.x);
    float e = __fmaf_rn(w.x, x.x, -p);
    e = __fmaf_rn(w.x, x.y, e);
    e = __fmaf_rn(w.y, x.x, e);
    two_sum(p);
    l = __fadd_rn(l, e);
  }
  __device__ __forceinline__ Part part() const { return make_float2(h, l); }
  __device__ __forceinline__ void merge(Part q) {
    two_sum(q.x);
    l = __fadd_rn(l, q.y);
  }
  __device__ __forceinline__ float2 get() const { return make_float2(h, l); }
};

__device__ __forceinline__ double df_value(float2 s) { return (double)s.x + (double)s.y; }

// Double-float sum a + b (TwoSum of the high parts, then renormalised),
// FP32 operations only.
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  float s = __fadd_rn(a.x, b.x);
  float bb = __fsub_rn(s, a.x);
  float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
  e = __fadd_rn(e, __fadd_rn(a.y, b.y));
  float t = __fadd_rn(s, e);
  return make_float2(t, __fsub_rn(e, __fsub_rn(t, s)));
}

__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }

// Plain fp32 sum (mixed inner sweeps: bf16 values, fp32 iterates).
struct AccF32 {
  typedef float W;
  typedef float X;
  typedef float Part;
  typedef float Sum;
  float s;
  __device__ __forceinline__ void zero() { s = 0.f; }
  __device__ __forceinline__ void add(float w, float x) { s = fmaf(w, x, s); }
  __device__ __forceinline__ Part part() const { return s; }
  __device__ __forceinline__ void merge(Part q) { s += q; }
  __device__ __forceinline__ float get() const { return s; }
};

// Two fp32 sums over the same entries (the one-pass mixed solve: the
// iterate's change and the next frame's change of the direct flux).
struct AccF2 {
  typedef float W;
  typedef float2 X;
  typedef float2 Part;
  typedef float2 Sum;
  float a, b;
  __device__ __forceinline__ void zero() { a = 0.f; b = 0.f; }
  __device__ __forceinline__ void add(float w, float2 x) {
    a = fmaf(w, x.x, a);
    b = fmaf(w, x.y, b);
  }
  __device__ __forceinline__ Part part() const { return make_float2(a, b); }
  __device__ __forceinline__ void merge(Part q) {
    a += q.x;
    b += q.y;
  }
  __device__ __forceinline__ float2 get() const { return make_float2(a, b); }
};

__device__ __forceinline__ float2 to_halo(float2 x, float2*) { return x; }
__device__ __forceinline__ float to_halo(float x, float*) { return x; }

// Iterates written by other blocks during the solve are read at L2 (never
// from a possibly stale L1 line).
__device__ __forceinline__ double ld_it(const double* p) { return __ldcg(p); }
__device__ __forceinline__ float ld_it(const float* p) { return __ldcg(p); }
__device__ __forceinline__ float2 ld_it(const float2* p) { return __ldcg(p); }

// Gather the tile's halo values x[halo[h]] into shared memory.
template <class XS, class XG>
__device__ __forceinline__ void stage_halo(const StepView& v, const RowTile& T, const XG* xg, XS* sx) {
  const uint32_t* hp = v.t_halo + T.h0;
  int h = threadIdx.x;
  for (; h + 3 * RAD_THREADS < T.nhalo; h += 4 * RAD_THREADS) {
    uint32_t a = __ldg(hp + h), b = __ldg(hp + h + RAD_THREADS), c = __ldg(hp + h + 2 * RAD_THREADS),
             d = __ldg(hp + h + 3 * RAD_THREADS);
    XG xa = ld_it(xg + a), xb = ld_it(xg + b), xc = ld_it(xg + c), xd = ld_it(xg + d);
    sx[h] = to_halo(xa, sx);
    sx[h + RAD_THREADS] = to_halo(xb, sx);
    sx[h + 2 * RAD_THREADS] = to_halo(xc, sx);
    sx[h + 3 * RAD_THREADS] = to_halo(xd, sx);
  }
  for (; h < T.nhalo; h += RAD_THREADS) sx[h] = to_halo(ld_it(xg + __ldg(hp + h)), sx);
  cbar();
}

// One tile: thread t owns entries [t*lam, (t+1)*lam) of the tile's entry
// stream (rows in order, each row's entries in column order), stored so that
// a group of 4 RAD_THREADS entries is contiguous: entry k of thread t at
// e0 + (k/4)*RAD_GROUP + 4t + k%4. The groups arrive in shared memory by
// bulk copies (the block's Pipe). Each thread accumulates sequentially and
// stores the sum of every row that starts and ends in its run in rs[row]
// (shared memory). A row that began in an earlier thread is completed by the
// thread where it ends: the partial sums of the threads it spans, in thread
// order, then its own part. Ends with a consumer barrier: rs holds every
// row sum of the tile.
template <class Acc, class V>
__device__ __forceinline__ void tile_rows(const StepView& v, const RowTile& T, int t, Pipe& p, V vals,
                                          const typename Acc::X* sx, typename Acc::Part* tail, unsigned char* tnew,
                                          typename Acc::Sum* rs) {
  typedef typename Acc::W W;
  const int tid = threadIdx.x;
  const uint32_t s0 = __ldg(v.t_start + (size_t)t * RAD_THREADS + tid);
  int r = (int)(s0 & 0x7fffffffu);
  const bool cont = (s0 >> 31) != 0;
  bool any = false, has_head = false;
  int head_row = 0;
  Acc acc, head;
  acc.zero();
  head.zero();
  const int ng = T.lam >> 2;
  auto elem = [&](uint32_t c, W w) {
    acc.add(w, sx[c & 0x7fffu]);
    if (c & 0x8000u) {
      if (cont && !any) {
        head = acc;
        head_row = r;
        has_head = true;
      } else {
        rs[r] = acc.get();
      }
      ++r;
      acc.zero();
      any = true;
    }
  };
  for (int g = 0; g < ng; ++g) {
    uint2 c;
    W w[4];
    take_group(p, v, vals, c, w);
    elem(c.x & 0xffffu, w[0]);
    elem(c.x >> 16, w[1]);
    elem(c.y & 0xffffu, w[2]);
    elem(c.y >> 16, w[3]);
  }
  tail[tid] = acc.part();
  tnew[tid] = (any || !cont) ? 1 : 0;
  cbar();
  if (has_head) {
    int u = tid - 1;
    while (!tnew[u]) --u;   // thread 0 starts a row, so this stops
    Acc s;
    s.zero();
    for (; u < tid; ++u) s.merge(tail[u]);
    s.merge(head.part());
    rs[head_row] = s.get();
  }
  cbar();
}

// Sum over the consumer threads in a fixed order (FP32), valid in thread 0.
// Ends with a consumer barrier (the tile's shared arrays are free again).
__device__ __forceinline__ float warp_sumf(float x) {
  for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ float block_sum(float d, float* red) {
  d = warp_sumf(d);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = d;
  cbar();
  float t = 0.f;
  if (threadIdx.x < 32) t = warp_sumf(threadIdx.x < RAD_THREADS / 32 ? red[threadIdx.x] : 0.f);
  cbar();
  return t;
}

// Per-mesh convergence. Each tile's squared change (FP32 partial) is
// recorded in tile_d2 (double-buffered by sweep parity) and added, as an
// integer, to its mesh's accumulator: the partial in units of tol^2 / 2^20,
// rounded up and capped at 2^40 (a NaN counts as the cap). Integer sums do
// not depend on the order of the atomic adds, so every block reads the same
// total after the grid barrier and takes the same decision with one load,
// and a mesh's decisions are the same alone and in a batch. A mesh stops
// when its total is <= 2^20 units, i.e. sum of partials <= tol^2 (at most
// ntiles units conservative). The accumulators follow the barrier's two
// counter words, three buffers of nmesh by residual number mod 3: buffer
// k + 1 is cleared during residual k (its last reader, decision k - 2,
// finished before the barrier that precedes residual k), and the accumulators
// of residual 0 are cleared before the first barrier.
constexpr unsigned long long RES_UNITS = 1ull << 20;
constexpr unsigned long long RES_CAP = 1ull << 40;

__device__ __forceinline__ unsigned long long* res_acc(const StepView& v, int k) {
  return reinterpret_cast<unsigned long long*>(v.barrier + 2) + (size_t)(k % 3) * v.nmesh;
}

// done[m]: 0 running; 1 + (parity of the mesh's last residual) once
// stopped; 1 for meshes that never ran. unit[m]: residual units per unit of
// squared change, 2^20 / tol^2 enlarged by 2^-16 so that the FP32 products
// below never round a partial's units down (+inf when tol is 0).
struct MeshState {
  int done[RAD_MAX_MESH];
  int sweeps[RAD_MAX_MESH];
  float unit[RAD_MAX_MESH];
  unsigned char now[RAD_MAX_MESH];   // stopped at the latest decision
};

__device__ __forceinline__ unsigned long long res_units(float d2, float unit) {
  if (isnan(d2)) return RES_CAP;
  if (!(d2 > 0.f)) return 0ull;
  const float q = __fmul_ru(d2, unit);
  return q < (float)RES_CAP ? (unsigned long long)ceilf(q) : RES_CAP;
}

// Thread 0, after block_sum: record tile t's partial of residual k.
__device__ __forceinline__ void post_partial(const StepView& v, const MeshState& st, const RowTile& T, int t, int k,
                                             float d2) {
  if (threadIdx.x != 0) return;
  v.tile_d2[(size_t)(k & 1) * v.ntiles + t] = (double)d2;
  atomicAdd(res_acc(v, k) + T.mesh, res_units(d2, st.unit[T.mesh]));
  res_acc(v, k + 1)[T.mesh] = 0ull;
}

__device__ __forceinline__ void init_meshes(const StepView& v, MeshState& st) {
  for (int m = threadIdx.x; m < v.nmesh; m += blockDim.x) {
    const MeshDesc& M = v.md[m];
    st.done[m] = (M.active && M.ntiles > 0) ? 0 : 1;
    st.sweeps[m] = 0;
    st.unit[m] = M.tol2 > 0.0 ? (float)((double)RES_UNITS / M.tol2 * (1.0 + 1.0 / 65536.0)) : INFINITY;
  }
  // accumulators of residual 0 (read only after the first barrier)
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  for (int m = gt; m < v.nmesh; m += gridDim.x * blockDim.x) res_acc(v, 0)[m] = 0ull;
}

// Every block, after the barrier that completes residual k: stop decisions
// and the number of meshes still running. Block 0 records the sweep counts.
__device__ __forceinline__ int decide_meshes(const StepView& v, MeshState& st, int inc, int first, int k) {
  __syncthreads();
  const unsigned long long* acc = res_acc(v, k);
  for (int m = threadIdx.x; m < v.nmesh; m += blockDim.x) {
    st.now[m] = 0;
    if (st.done[m]) continue;
    const unsigned long long q = __ldcg(acc + m);
    const int sw = st.sweeps[m] + (first ? 0 : inc);
    st.sweeps[m] = sw;
    if (q <= RES_UNITS || sw >= v.md[m].max_sweeps) {
      st.done[m] = 1 + (k & 1);
      st.now[m] = 1;
    }
    if (blockIdx.x == 0) v.md[m].sweeps = sw;
  }
  int running = 0;
  for (int m0 = 0; m0 < v.nmesh; m0 += blockDim.x) {
    int m = m0 + threadIdx.x;
    running += __syncthreads_count(m < v.nmesh && !st.done[m]);
  }
  return running;
}

// Block 0, at the end of the launch: each solved mesh's last residual
// (sum of its tiles' partials, lane-strided then a fixed warp tree) into
// the mesh table.
__device__ __forceinline__ void record_residuals(const StepView& v, const MeshState& st) {
  if (blockIdx.x != 0 || threadIdx.x >= RAD_THREADS) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int m = warp; m < v.nmesh; m += RAD_THREADS / 32) {
    const MeshDesc& M = v.md[m];
    if (!M.active || M.ntiles == 0) continue;
    const double* d2 = v.tile_d2 + (size_t)(st.done[m] - 1) * v.ntiles;
    double t = 0.0;
    for (int j = lane; j < M.ntiles; j += 32) t += ld_it(d2 + M.tile0 + j);
    t = warp_sum(t);
    if (lane == 0) v.md[m].res2 = t;
  }
}

// The solve works on radiosity positions (Morton order within each mesh),
// gathered through rperm at entry: EP = E (FP64), S0 / S1 = the iterates'
// scattered parts s = x - E (double-floats), H0 / H1 = the iterates
// x = E + s as double-floats (what the halos gather) and EH = E as a
// double-float. Start values: rows without entries are x = E exactly
// (s = 0); the others start at s = 0 (cold) or at the mesh's previous
// solution, extrapolated linearly once two solutions exist (warm). The warm
// start predicts the scattered part and takes the step's own E:
// s0 = S(n) + (S(n) - S(n-1)). E jumps where a facet enters or leaves
// shadow; S = F x varies smoothly, so the start is off by about F dE there
// instead of dE. sprev holds S(n) and, after it, its last change; for the
// one-pass mixed solve (predicted) the predicted change F (E(n+1) - E(n))
// instead, so that s0 = S(n) + P from the second step on.
struct RadBufs {
  double* EP;
  float2 *S0, *S1, *H0, *H1, *EH;
  __device__ __forceinline__ explicit RadBufs(const StepView& v) {
    EP = v.rbuf;
    S0 = reinterpret_cast<float2*>(v.rbuf + v.nt);
    S1 = reinterpret_cast<float2*>(v.rbuf + 2 * (size_t)v.nt);
    H0 = reinterpret_cast<float2*>(v.rbuf + 3 * (size_t)v.nt);
    H1 = H0 + v.nt;
    EH = H1 + v.nt;
  }
};

// The solve's own per-row state is kept by radiosity position p (Morton
// order): the warm-start record sprev, row_act, and the mesh of a position
// (a mesh's positions and facets occupy the same range, so mesh_of serves
// both). Only E (read) and x (written) are in facet order: one gather and
// one scatter through rperm per row and solve. Each thread takes
// RAD_ILP positions at once so that their loads are in flight together.
constexpr int RAD_ILP = 4;

// free_rows (the mixed solve): also write the result of the rows without
// entries (x = E, s = 0) and their warm-start record, for a kernel that
// scatters its tile rows itself; that solve reads only EP, S0 and H0 (and
// x32), the FP64 sweeps also S1, H1 and EH.
// kind (the one-pass mixed solve, per mesh: 0 bf16 step, 1 reference step, 2
// first reference step): the warm start is S(n) + P, and the pass's halo
// vector EH = (x - x_ref, E(n+1) - E(n)) and the reference iterate H1 are
// written here too; x32 then holds only P (zero for rows without entries).
__device__ __forceinline__ void init_x(const StepView& v, double* x, int warm, int gt, int nthreads,
                                       bool free_rows, const unsigned char* kind = nullptr) {
  const RadBufs B(v);
  const bool predicted = kind != nullptr;
  for (int p0 = gt; p0 < v.nt; p0 += RAD_ILP * nthreads) {
    int g[RAD_ILP], mi[RAD_ILP];   // facet and mesh of each position (mesh -1: none)
    double d[RAD_ILP];
    float2 sp0[RAD_ILP], sp1[RAD_ILP];
    float de[RAD_ILP];
    uint8_t act[RAD_ILP];
#pragma unroll
    for (int k = 0; k < RAD_ILP; ++k) {
      const int p = p0 + k * nthreads;
      g[k] = 0;
      mi[k] = -1;
      if (p >= v.nt) continue;
      const int mk = mesh_of_facet(v, p);
      const MeshDesc* m = v.md + mk;
      if (!m->active || m->ntiles == 0) continue;
      mi[k] = mk;
      g[k] = (int)v.rperm[p];
      act[k] = v.row_act[p];
      sp0[k] = warm ? v.sprev[p] : make_float2(0.f, 0.f);
      sp1[k] = warm ? v.sprev[v.nt + p] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < RAD_ILP; ++k) {
      if (mi[k] < 0) continue;
      const MeshDesc& Mk = v.md[mi[k]];
      const double dk = v.E[e_slot(Mk.frame) * v.nt + g[k]];
      const bool ref = Mk.coupling == ILG_COUPLE_REFERENCE;
      const double fs = ref ? v.Fsurf[g[k]] : 0.0;
      // the change of the direct flux to the next frame (none after the
      // table's last sun)
      if (predicted)
        de[k] = (!Mk.host_sun && Mk.sun_idx + 1 < Mk.nsun)
                    ? (float)(v.E[e_slot(Mk.frame + 1) * v.nt + g[k]] - dk)
                    : 0.f;
      // the frame's direct flux, coupled as src/cpp/illum_cli.cpp:415-421
      // when the mesh follows the reference (rad = -Fsurf_prev + direct)
      d[k] = ref ? (-fs + dk) : dk;
    }
#pragma unroll
    for (int k = 0; k < RAD_ILP; ++k) {
      if (mi[k] < 0) continue;
      const int p = p0 + k * nthreads;
      const MeshDesc& Mk = v.md[mi[k]];
      const double e = d[k];
      float2 s0 = make_float2(0.f, 0.f);
      if (warm && act[k] && Mk.frame >= 1) s0 = Mk.frame >= 2 || predicted ? df_add(sp0[k], sp1[k]) : sp0[k];
      if (free_rows && !act[k]) {
        x[g[k]] = e;
        if (warm) {
          v.sprev[v.nt + p] = df_neg(sp0[k]);
          v.sprev[p] = make_float2(0.f, 0.f);
        }
      }
      const float2 eh = split_df(e);
      const float2 x0 = df_add(eh, s0);
      B.EP[p] = e;
      B.S0[p] = s0;
      B.H0[p] = x0;
      if (predicted) {
        // x - x_ref, high parts first (exact when within a factor of 2)
        const int kd = kind[mi[k]];
        float dx;
        if (kd == 2) {
          dx = __fadd_rn(x0.x, x0.y);
        } else {
          const float2 xr = B.H1[p];
          dx = __fadd_rn(__fsub_rn(x0.x, xr.x), __fsub_rn(x0.y, xr.y));
        }
        if (kd) B.H1[p] = x0;
        B.EH[p] = make_float2(dx, de[k]);
        if (!act[k]) v.x32[v.nt + p] = 0.f;
      } else if (free_rows) {
        v.x32[p] = 0.f;
        v.x32[v.nt + p] = 0.f;
      } else {
        B.S1[p] = make_float2(0.f, 0.f);
        B.H1[p] = x0;
        B.EH[p] = eh;
      }
    }
  }
}

// Scatter the solved meshes' last iterate x = E + s back to facet order
// (FP64; the FP64 solve's result is in S1 after an odd number of sweeps);
// warm solves also record s and its change for the next step's start. Rows
// without entries keep s = 0 in both buffers.
__device__ __forceinline__ void scatter_x(const StepView& v, const MeshState& st, double* x, int warm, int gt,
                                          int nthreads) {
  const RadBufs B(v);
  for (int p0 = gt; p0 < v.nt; p0 += RAD_ILP * nthreads) {
    int g[RAD_ILP];
    bool ok[RAD_ILP];
    double e[RAD_ILP];
    float2 s[RAD_ILP], sp[RAD_ILP];
#pragma unroll
    for (int k = 0; k < RAD_ILP; ++k) {
      const int p = p0 + k * nthreads;
      ok[k] = false;
      if (p >= v.nt) continue;
      const int m = mesh_of_facet(v, p);
      const MeshDesc& M = v.md[m];
      if (!M.active || M.ntiles == 0) continue;
      ok[k] = true;
      g[k] = (int)v.rperm[p];
      s[k] = ld_it(((st.sweeps[m] & 1) ? B.S1 : B.S0) + p);
      e[k] = B.EP[p];
      sp[k] = warm ? v.sprev[p] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < RAD_ILP; ++k) {
      if (!ok[k]) continue;
      const int p = p0 + k * nthreads;
      x[g[k]] = e[k] + df_value(s[k]);
      if (warm) {
        v.sprev[v.nt + p] = df_add(s[k], df_neg(sp[k]));
        v.sprev[p] = s[k];
      }
    }
  }
}

// The rows of this block's tiles whose mesh stopped at the latest decision
// (st.now): x = E + s into facet order, and the warm-start record, as
// scatter_x. The block's rows are dealt to its consumer threads in one run
// over all its tiles (a thread takes every RAD_THREADS-th row of the
// concatenation), so each thread has a few rows in a row instead of a
// fraction of one per tile.
__device__ __forceinline__ void scatter_block(const StepView& v, const MeshState& st, const float2* S, double* x,
                                              int warm, const float* pred = nullptr) {
  const RadBufs B(v);
  int r = threadIdx.x;
  for (int k = v.blk_start[blockIdx.x]; k < v.blk_start[blockIdx.x + 1]; ++k) {
    const int t = v.blk_tile[k];
    const RowTile T = v.tiles[t];
    if (!st.now[T.mesh]) continue;
    const uint32_t* rows = v.t_row + T.r0;
    for (; r < T.nrows; r += RAD_THREADS) {
      const uint32_t i = __ldg(rows + r);
      const int g = (int)v.rperm[i];
      const float2 sv = ld_it(S + i);
      x[g] = B.EP[i] + df_value(sv);
      if (warm) {
        v.sprev[v.nt + i] = pred ? make_float2(ld_it(pred + i), 0.f) : df_add(sv, df_neg(v.sprev[i]));
        v.sprev[i] = sv;
      }
    }
    r -= T.nrows;
  }
}

struct RadSmem {
  unsigned char* ring;       // entry-stream stages (RAD_RING bytes)
  float2* sx;                // halo values (RAD_HALO double-floats, or floats)
  float2* tail;              // per-thread open-row partials
  float2* rs;                // row sums of the tile (RAD_ROWS double-floats, or floats)
  unsigned char* tnew;       // per thread: its last open row began in its run
  unsigned long long* full;  // per stage: its copies have landed
  unsigned long long* empty; // per stage: every consumer has read it
};

__device__ __forceinline__ RadSmem rad_smem() {
  extern __shared__ __align__(128) unsigned char rad_dyn[];
  RadSmem m;
  m.ring = rad_dyn;
  m.sx = reinterpret_cast<float2*>(rad_dyn + RAD_RING);
  m.tail = m.sx + RAD_HALO;
  m.rs = m.tail + RAD_THREADS;
  m.tnew = reinterpret_cast<unsigned char*>(m.rs + RAD_ROWS);
  m.full = reinterpret_cast<unsigned long long*>(m.tnew + RAD_THREADS);
  m.empty = m.full + RAD_NST_MAX;
  return m;
}
static_assert((RAD_RING + (size_t)(RAD_HALO + RAD_THREADS + RAD_ROWS) * 8 + RAD_THREADS) % 8 == 0,
              "stage barriers are 8-byte aligned");

// The ring's barriers, set up by thread 0 before the launch's first block
// barrier (inside init_meshes' caller): full counts the producer's one
// arrival plus the copied bytes, empty one arrival per consumer thread.
__device__ __forceinline__ Pipe make_pipe(const RadSmem& m, int nst, int stage_bytes, int* bad) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < nst; ++s) {
      mbar_init(m.full + s, 1);
      mbar_init(m.empty + s, RAD_THREADS);
    }
    *bad = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  Pipe p;
  p.ring = m.ring;
  p.full = m.full;
  p.empty = m.empty;
  p.bad = bad;
  p.nst = nst;
  p.stage_bytes = stage_bytes;
  p.q = 0;
  return p;
}

// Producer warp: the copies of one pass over the block's tiles (lane 0
// issues; the other lanes only follow the launch's block barriers).
template <class V>
__device__ __forceinline__ void produce_pass(Pipe& p, const StepView& v, const MeshState& st, V vals, uint64_t pol) {
  if ((threadIdx.x & 31) != 0) return;
  for (int k = v.blk_start[blockIdx.x]; k < v.blk_start[blockIdx.x + 1]; ++k) {
    const int t = v.blk_tile[k];
    const RowTile T = v.tiles[t];
    if (st.done[T.mesh]) continue;
    produce_tile(p, v, T, vals, pol);
  }
}

// FP64 Jacobi to each mesh's tolerance. x: solution (and warm start).
__global__ void __launch_bounds__(RAD_BLOCK, 1) k_radiosity64(StepView v, double* x, int warm) {
  __shared__ MeshState st;
  __shared__ float red[32];
  __shared__ int bad;
  const RadSmem sm = rad_smem();
  const bool producer = threadIdx.x >= RAD_THREADS;
  const int gt = blockIdx.x * RAD_THREADS + threadIdx.x;
  const int nthreads = gridDim.x * RAD_THREADS;
  unsigned gen = 0;
  Pipe pipe = make_pipe(sm, RAD_NST64, RAD_STAGE64, &bad);
  init_meshes(v, st);
  if (!producer) init_x(v, x, warm, gt, nthreads, false);
  if (!grid_barrier(v.barrier, gridDim.x, gen, v.derr)) return;
  const uint64_t pol = l2_keep_policy(v.l2_stream);
  const ValsDF vals{v.t_vhi, v.t_vlo};
  for (int it = 0;; ++it) {
    if (producer) {
      produce_pass(pipe, v, st, vals, pol);
      __syncwarp();
    } else {
      for (int k = v.blk_start[blockIdx.x]; k < v.blk_start[blockIdx.x + 1]; ++k) {
    const int t = v.blk_tile[k];
        const RowTile T = v.tiles[t];
        if (st.done[T.mesh]) continue;
        const RadBufs B(v);
        stage_halo(v, T, (it & 1) ? B.H1 : B.H0, sm.sx);
        tile_rows<AccDF>(v, T, t, pipe, vals, sm.sx, sm.tail, sm.tnew, sm.rs);
        const uint32_t* rows = v.t_row + T.r0;
        const float2* cur = (it & 1) ? B.S1 : B.S0;
        float2* nxt = (it & 1) ? B.S0 : B.S1;
        float2* nxth = (it & 1) ? B.H0 : B.H1;
        float d2 = 0.f;
        for (int r = threadIdx.x; r < T.nrows; r += RAD_THREADS) {
          uint32_t i = __ldg(rows + r);
          const float2 sn = sm.rs[r];          // s' = F x
          const float2 sc = ld_it(cur + i);
          // s' - s: exact high-part difference when the two are within a
          // factor of two, else rounded relative to the change itself
          const float df = __fadd_rn(__fsub_rn(sn.x, sc.x), __fsub_rn(sn.y, sc.y));
          nxt[i] = sn;
          nxth[i] = df_add(__ldg(B.EH + i), sn);
          d2 = __fmaf_rn(df, df, d2);
        }
        post_partial(v, st, T, t, it, block_sum(d2, red));
      }
    }
    if (!grid_barrier(v.barrier, gridDim.x, gen, v.derr)) return;
    if (decide_meshes(v, st, 1, 0, it) == 0) break;
  }
  if (!producer) scatter_x(v, st, x, warm, gt, nthreads);
  record_residuals(v, st);
}

// Mixed precision: outer refinement with the residual r = E - (I - fl(F)) x
// = fl(F) x - s (double-float sums), inner fp32 Jacobi on (I - F~) d = r with
// bf16 F~ (inner sweeps, 1..RAD_INNER), s += d. A mesh stops when
// ||r||_2 <= tol, or after the update of the round that reaches max_sweeps;
// each tile's block writes its rows' results.
__global__ void __launch_bounds__(RAD_BLOCK, 1) k_radiosity_mixed(StepView v, double* x, int warm, int inner) {
  __shared__ MeshState st;
  __shared__ float red[32];
  __shared__ int bad;
  const RadSmem sm = rad_smem();
  const bool producer = threadIdx.x >= RAD_THREADS;
  float* sxf = reinterpret_cast<float*>(sm.sx);
  float* tailf = reinterpret_cast<float*>(sm.tail);
  float* rsf = reinterpret_cast<float*>(sm.rs);
  const int gt = blockIdx.x * RAD_THREADS + threadIdx.x;
  const int nthreads = gridDim.x * RAD_THREADS;
  float* xa = v.x32;
  float* xb = v.x32 + v.nt;
  float* r32 = v.x32 + 2 * (size_t)v.nt;
  unsigned gen = 0;
  Pipe pipe = make_pipe(sm, RAD_NSTM, RAD_STAGEM, &bad);
  init_meshes(v, st);
  if (!producer) init_x(v, x, warm, gt, nthreads, true);
  if (!grid_barrier(v.barrier, gridDim.x, gen, v.derr)) return;
  const uint64_t pol = l2_keep_policy(v.l2_stream);
  const RadBufs B(v);
  const ValsHi vhi{v.t_vhi};
  const ValsBF vbf{v.t_vbf};
  float2* S = B.S0;     // the iterate's scattered part s = x - E (radiosity positions)
  float2* XH = B.H0;    // x = E + s, what the halos gather
  int first = 1;
  for (int round = 0;; ++round) {
    if (producer) {
      produce_pass(pipe, v, st, vhi, pol);
      __syncwarp();
    } else {
      for (int k = v.blk_start[blockIdx.x]; k < v.blk_start[blockIdx.x + 1]; ++k) {
    const int t = v.blk_tile[k];
        const RowTile T = v.tiles[t];
        if (st.done[T.mesh]) continue;
        stage_halo(v, T, XH, sm.sx);
        tile_rows<AccDF>(v, T, t, pipe, vhi, sm.sx, sm.tail, sm.tnew, sm.rs);
        const uint32_t* rows = v.t_row + T.r0;
        float d2 = 0.f;
        for (int r = threadIdx.x; r < T.nrows; r += RAD_THREADS) {
          uint32_t i = __ldg(rows + r);
          // r = E + fl(F) x - x = fl(F) x - s
          const float2 fx = sm.rs[r], s = ld_it(S + i);
          const float res = __fadd_rn(__fsub_rn(fx.x, s.x), __fsub_rn(fx.y, s.y));
          r32[i] = res;
          xa[i] = res;     // inner start: d0 = r
          d2 = __fmaf_rn(res, res, d2);
        }
        post_partial(v, st, T, t, round, block_sum(d2, red));
      }
    }
    if (!grid_barrier(v.barrier, gridDim.x, gen, v.derr)) return;
    int running = decide_meshes(v, st, inner, first, round);
    first = 0;
    // meshes that stopped on their residual: each block writes its own
    // tiles' rows (their s was last written by this block)
    if (!producer) scatter_block(v, st, S, x, warm);
    if (running == 0) break;
    float* cur = xa;
    float* nxt = xb;
    for (int it = 0; it < inner; ++it) {
      if (producer) {
        produce_pass(pipe, v, st, vbf, pol);
        __syncwarp();
      } else {
        for (int k = v.blk_start[blockIdx.x]; k < v.blk_start[blockIdx.x + 1]; ++k) {
    const int t = v.blk_tile[k];
          const RowTile T = v.tiles[t];
          if (st.done[T.mesh]) continue;
          stage_halo(v, T, cur, sxf);
          tile_rows<AccF32>(v, T, t, pipe, vbf, sxf, tailf, sm.tnew, rsf);
          const uint32_t* rows = v.t_row + T.r0;
          const float* scale = v.t_scale + T.r0;
          if (it + 1 < inner) {
            for (int r = threadIdx.x; r < T.nrows; r += RAD_THREADS) {
              uint32_t i = __ldg(rows + r);
              nxt[i] = ld_it(r32 + i) + __ldg(scale + r) * rsf[r];
            }
          } else {   // last sweep: nobody reads d again, s += d directly
            // (x for the halos only if the mesh runs another round)
            const bool more = st.sweeps[T.mesh] + inner < v.md[T.mesh].max_sweeps;
            for (int r = threadIdx.x; r < T.nrows; r += RAD_THREADS) {
              uint32_t i = __ldg(rows + r);
              const float2 d = make_float2(ld_it(r32 + i) + __ldg(scale + r) * rsf[r], 0.f);
              S[i] = df_add(ld_it(S + i), d);
              if (more) XH[i] = df_add(ld_it(XH + i), d);
            }
          }
          cbar();
        }
      }
      if (it + 1 < inner) {
        if (!grid_barrier(v.barrier, gridDim.x, gen, v.derr)) return;
        float* tmp = cur; cur = nxt; nxt = tmp;
      }
    }
    // meshes whose budget this round used up stop here (same decision in
    // every block: it depends on the counts only) and take their results
    // (each block its own tiles' rows, whose s it wrote)
    int left = 0;
    for (int m0 = 0; m0 < v.nmesh; m0 += blockDim.x) {
      int m = m0 + threadIdx.x;
      bool run = m < v.nmesh && !st.done[m];
      if (m < v.nmesh) st.now[m] = 0;
      if (run && st.sweeps[m] + inner >= v.md[m].max_sweeps) {
        st.done[m] = 1 + (round & 1);
        st.sweeps[m] += inner;
        st.now[m] = 1;
        if (blockIdx.x == 0) v.md[m].sweeps = st.sweeps[m];
        run = false;
      }
      left += __syncthreads_count(run);
    }
    if (!producer) scatter_block(v, st, S, x, warm);
    if (left == 0) break;   // every result is written (by its tile's block)
    if (!grid_barrier(v.barrier, gridDim.x, gen, v.derr)) return;
  }
  record_residuals(v, st);
}

// Mixed precision, one pass over the matrix per step (refine_every = K >=
// 1). The pass applies F to x - x_ref, where x = E + s0 is the step's
// iterate and x_ref the iterate of the mesh's last reference step:
//   s = s_ref + F (x - x_ref),
// with the f32 values on a reference step (every K-th step of a mesh, and
// a step without an earlier reference, where x_ref = 0 and s_ref = 0: the
// mesh's first, or its first after a new matrix or another solve on its
// buffers), which then keeps (s, x) as the new reference, and the bf16 copy
// F~ on the steps between:
// s = F x - (F - F~)(x - x_ref), the bf16 error confined to the change
// since the reference step. Sums in FP32 (the terms are changes); s and
// s_ref stay double-float. A single sweep from the previous solution would
// leave the multiple scattering of a change of E one order behind (F^2 dE
// for a facet that crosses the terminator), so the warm start predicts it:
// the same pass also forms P = F (E(n+1) - E(n)) with the next frame's
// direct flux (a second right-hand side on the same matrix entries, 8 B
// halos of (x - x_ref, dE)), and the next step starts from s0 = s + P, off by
// F^2 dE instead of F dE. The step's squared change |s - s0|^2 is recorded
// as its residual.
__global__ void __launch_bounds__(RAD_BLOCK, 1) k_radiosity_lagged(StepView v, double* x, int warm) {
  __shared__ MeshState st;
  __shared__ float red[32];
  __shared__ int bad;
  // each mesh's kind of pass (0: bf16 step, 1: reference step, 2: reference
  // step without an earlier reference) lives in st.now until the pass is
  // over (the static shared memory has no room for another array beside the
  // ring)
  unsigned char* kind = st.now;
  const RadSmem sm = rad_smem();
  const bool producer = threadIdx.x >= RAD_THREADS;
  const int gt = blockIdx.x * RAD_THREADS + threadIdx.x;
  const int nthreads = gridDim.x * RAD_THREADS;
  const RadBufs B(v);
  float2* XD = B.EH;            // by position: (x - x_ref, E(n+1) - E(n))
  float* pred = v.x32 + v.nt;   // by position: P, the predicted change of s
  unsigned gen = 0;
  Pipe pipe = make_pipe(sm, RAD_NSTM, RAD_STAGEM, &bad);
  init_meshes(v, st);
  for (int m = threadIdx.x; m < v.nmesh; m += blockDim.x) {
    const MeshDesc& M = v.md[m];
    kind[m] = M.ref_age < 0 ? 2 : (M.ref_age + 1 >= M.refine_every ? 1 : 0);
  }
  __syncthreads();
  if (!producer) init_x(v, x, warm, gt, nthreads, true, kind);
  if (!grid_barrier(v.barrier, gridDim.x, gen, v.derr)) return;
  // every block has read the ages: block 0 advances them
  if (blockIdx.x == 0)
    for (int m = threadIdx.x; m < v.nmesh; m += blockDim.x)
      if (!st.done[m]) v.md[m].ref_age = kind[m] ? 0 : v.md[m].ref_age + 1;
  const uint64_t pol = l2_keep_policy(v.l2_stream);
  const ValsHiF vhi{v.t_vhi};
  const ValsBF vbf{v.t_vbf};
  if (producer) {
    if ((threadIdx.x & 31) == 0)
      for (int k = v.blk_start[blockIdx.x]; k < v.blk_start[blockIdx.x + 1]; ++k) {
        const RowTile T = v.tiles[v.blk_tile[k]];
        if (st.done[T.mesh]) continue;
        if (kind[T.mesh]) produce_tile(pipe, v, T, vhi, pol);
        else produce_tile(pipe, v, T, vbf, pol);
      }
    __syncwarp();
  } else {
    for (int k = v.blk_start[blockIdx.x]; k < v.blk_start[blockIdx.x + 1]; ++k) {
      const int t = v.blk_tile[k];
      const RowTile T = v.tiles[t];
      if (st.done[T.mesh]) continue;
      const int kd = kind[T.mesh];
      stage_halo(v, T, XD, sm.sx);
      if (kd) tile_rows<AccF2>(v, T, t, pipe, vhi, sm.sx, sm.tail, sm.tnew, sm.rs);
      else tile_rows<AccF2>(v, T, t, pipe, vbf, sm.sx, sm.tail, sm.tnew, sm.rs);
      const uint32_t* rows = v.t_row + T.r0;
      const float* scale = v.t_scale + T.r0;
      float d2 = 0.f;
      for (int r = threadIdx.x; r < T.nrows; r += RAD_THREADS) {
        const uint32_t i = __ldg(rows + r);
        const float2 a = sm.rs[r];   // F (x - x_ref), F dE of the row
        const float sc = kd ? 1.f : __ldg(scale + r);
        const float2 sref = kd == 2 ? make_float2(0.f, 0.f) : ld_it(B.S1 + i);
        const float2 sn = df_add(sref, make_float2(sc * a.x, 0.f));
        const float2 s0 = ld_it(B.S0 + i);
        const float df = __fadd_rn(__fsub_rn(sn.x, s0.x), __fsub_rn(sn.y, s0.y));
        if (kd) B.S1[i] = sn;
        B.S0[i] = sn;
        pred[i] = sc * a.y;
        d2 = __fmaf_rn(df, df, d2);
      }
      post_partial(v, st, T, t, 0, block_sum(d2, red));
    }
  }
  // every solved mesh stops after this pass: each block writes its own
  // tiles' rows (whose s and P it wrote); the residual record waits for all
  // tiles
  __syncthreads();
  for (int m = threadIdx.x; m < v.nmesh; m += blockDim.x) {
    st.now[m] = st.done[m] ? 0 : 1;
    if (!st.done[m]) {
      st.done[m] = 1;
      st.sweeps[m] = 1;
      if (blockIdx.x == 0) v.md[m].sweeps = 1;
    }
  }
  __syncthreads();
  if (!producer) scatter_block(v, st, B.S0, x, warm, pred);
  if (!grid_barrier(v.barrier, gridDim.x, gen, v.derr)) return;
  record_residuals(v, st);
}

// Per-row fp32 scale = max |F_ij| of the row (the bf16 copy stores F/scale).
__global__ void k_row_scale(const int64_t* __restrict__ rowptr, const double* __restrict__ val, int nt,
                            float* rscale) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  double m = 0.0;
  for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) m = fmax(m, fabs(val[k]));
  rscale[i] = m > 0.0 ? (float)m : 1.f;
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

// Tile build on the device.
// key = (tile of the entry's row) << rb | Morton rank of its column; value =
// the entry's index in the row-sorted order.
__global__ void k_tile_keys(const unsigned long long* __restrict__ skey, int64_t n, int rb,
                            const int* __restrict__ tile_of, unsigned long long* key, uint32_t* idx) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const unsigned long long cm = (1ull << rb) - 1;
  const int g = (int)(skey[k] >> rb);
  key[k] = ((unsigned long long)tile_of[g] << rb) | (skey[k] & cm);
  idx[k] = (uint32_t)k;
}

// 1 where a (tile, column) run starts in the sorted keys.
__global__ void k_run_flags(const unsigned long long* __restrict__ key, int64_t n, uint32_t* flag) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  flag[i] = (i == 0 || key[i] != key[i - 1]) ? 1u : 0u;
}

// Runs are the tiles' halo facets, in (tile, Morton rank) order: the run
// index is the facet's slot in t_halo, and a tile's first run is its h0.
__global__ void k_halo_runs(const unsigned long long* __restrict__ key, const uint32_t* __restrict__ flag,
                            const unsigned long long* __restrict__ before, int64_t n, int rb, uint32_t* t_halo,
                            int* tile_first) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !flag[i]) return;
  const unsigned long long cm = (1ull << rb) - 1;
  const int64_t r = (int64_t)before[i];
  t_halo[r] = (uint32_t)(key[i] & cm);
  const int t = (int)(key[i] >> rb);
  if (i == 0 || (int)(key[i - 1] >> rb) != t) tile_first[t] = (int)r;
}

// Each entry to its stored slot: entry j of a tile (rows in Morton order,
// each row's entries in column order) belongs to thread t = j / lam as its
// kk = j % lam-th, stored at e0 + (kk / 4) RAD_GROUP + 4 t + kk % 4; the slot
// holds the entry's halo index (run - h0) with the row-end bit, the CSR
// entry it takes its value from, and its row (for the row scale).
__global__ void k_tile_slots(const unsigned long long* __restrict__ key, const uint32_t* __restrict__ idx,
                             const uint32_t* __restrict__ flag, const unsigned long long* __restrict__ before,
                             int64_t n, int rb, const unsigned long long* __restrict__ skey,
                             const uint32_t* __restrict__ ssrc, const int64_t* __restrict__ rowptr,
                             const int* __restrict__ rowoff, const RowTile* __restrict__ tiles, uint16_t* cf,
                             uint32_t* esrc, uint32_t* efac) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int t = (int)(key[i] >> rb);
  const RowTile T = tiles[t];
  const int64_t run = (int64_t)before[i] + flag[i] - 1;
  const uint32_t loc = (uint32_t)(run - T.h0);
  const int64_t k = idx[i];
  const int g = (int)(skey[k] >> rb);
  const int64_t j = rowoff[g] + (k - rowptr[g]);
  const int64_t th = j / T.lam, kk = j - th * T.lam;
  const int64_t off = T.e0 + (kk >> 2) * 4 * RAD_THREADS + 4 * th + (kk & 3);
  cf[off] = (uint16_t)(loc | (k + 1 == rowptr[g + 1] ? 0x8000u : 0u));
  esrc[off] = ssrc[k];
  efac[off] = (uint32_t)g;
}

// Each thread's first row (with a continuation bit when its run starts
// inside the row): rowj0 holds each tile row's first entry index within the
// tile, tile rows in order.
__global__ void k_tile_starts(const RowTile* __restrict__ tiles, int ntiles, const int64_t* __restrict__ ne,
                              const int* __restrict__ rowj0, uint32_t* tstart) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)ntiles * RAD_THREADS) return;
  const int tid = (int)(q / RAD_THREADS), t = (int)(q % RAD_THREADS);
  const RowTile T = tiles[tid];
  const int64_t j0 = (int64_t)t * T.lam;
  if (j0 >= ne[tid]) { tstart[q] = (uint32_t)T.nrows; return; }
  const int* rj = rowj0 + T.r0;
  int lo = 0, hi = T.nrows;   // last row with rj <= j0
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if ((int64_t)rj[mid] <= j0) lo = mid; else hi = mid;
  }
  tstart[q] = (uint32_t)lo | ((int64_t)rj[lo] != j0 ? 0x80000000u : 0u);
}

// Stored entry e takes CSR entry src[e] (value as a double-float, and its
// bf16 copy scaled by its row's scale), or zero for padding (src = ~0).
__global__ void k_tile_fill(const uint32_t* __restrict__ src, const uint32_t* __restrict__ fac, int64_t n,
                            const double* __restrict__ val, const float* __restrict__ rscale, float* t_vhi,
                            float* t_vlo, __nv_bfloat16* t_vbf) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  uint32_t k = src[e];
  double w = k == 0xffffffffu ? 0.0 : val[k];
  float2 hl = split_df(w);
  t_vhi[e] = hl.x;
  t_vlo[e] = hl.y;
  t_vbf[e] = __float2bfloat16_rn(k == 0xffffffffu ? 0.f : (float)(w / (double)rscale[fac[e]]));
}

__global__ void k_tile_scale(const uint32_t* __restrict__ t_row, const uint32_t* __restrict__ rperm, int n,
                             const float* __restrict__ rscale, float* t_scale) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) t_scale[k] = rscale[rperm[t_row[k]]];
}

int g_rad_nsm = 0, g_rad_per_sm64 = 0, g_rad_per_smm = 0;
std::atomic<bool> g_rad_ready{false};
std::mutex g_rad_mu;

// Once per process, before any capture: the kernels' shared-memory opt-in
// and their co-residency. Safe to call from several host threads.
int radiosity_setup() {
  if (g_rad_ready.load(std::memory_order_acquire)) return ILG_OK;
  std::lock_guard<std::mutex> lock(g_rad_mu);
  if (g_rad_ready.load(std::memory_order_relaxed)) return ILG_OK;
  int dev, nsm;
  ILG_CUDA(cudaGetDevice(&dev));
  ILG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  ILG_CUDA(cudaFuncSetAttribute(k_radiosity64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RAD_SMEM));
  ILG_CUDA(cudaFuncSetAttribute(k_radiosity_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RAD_SMEM));
  ILG_CUDA(cudaFuncSetAttribute(k_radiosity_lagged, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RAD_SMEM));
  ILG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_rad_per_sm64, k_radiosity64, RAD_BLOCK, RAD_SMEM));
  ILG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_rad_per_smm, k_radiosity_mixed, RAD_BLOCK, RAD_SMEM));
  int per_lagged = 0;   // the two mixed kernels share the grid
  ILG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_lagged, k_radiosity_lagged, RAD_BLOCK, RAD_SMEM));
  g_rad_per_smm = std::min(g_rad_per_smm, per_lagged);
  if (g_rad_per_sm64 < 1 || g_rad_per_smm < 1) { set_error("radiosity kernel cannot be resident"); return ILG_ERR_CUDA; }
  g_rad_nsm = nsm;
  g_rad_ready.store(true, std::memory_order_release);
  return ILG_OK;
}

}  // namespace

// Row tiles of the form-factor matrix in Morton order (see the top of the
// file). Tile sizes target nnz / (co-resident blocks) entries, at least
// RAD_MIN_TILE, and a tile closes early when its halo would exceed RAD_HALO
// or its rows RAD_ROWS.
int radiosity_prepare(Context& c) {
  ILG_TRY(radiosity_setup());
  c.ref_age = -1;   // a new matrix or layout: no one-pass reference
  cudaStream_t s = c.stream;
  const int nt = c.nt;
  const int64_t nnz = c.nnz;
  ILG_TRY(c.row_scale.alloc(nt));
  k_row_scale<<<div_up(nt, 256), 256, 0, s>>>(c.rowptr.p, c.val.p, nt, c.row_scale.p);
  ILG_CUDA(cudaGetLastError());
  ILG_TRY(c.rperm.alloc(nt));
  ILG_CUDA(cudaMemcpyAsync(c.rperm.p, c.morton_order.p, (size_t)nt * 4, cudaMemcpyDeviceToDevice, s));

  // Each row's entries in Morton order of their columns, sorted on the
  // device: key = (row, Morton position of the column), value = CSR entry.
  // Only N-sized data (row pointers, the Morton order, per-row halo bounds)
  // comes to the host, which cuts the tiles; everything per entry stays on
  // the device.
  int rb = 1;
  while ((1 << rb) < nt) ++rb;
  std::vector<int64_t> rp((size_t)nt + 1);
  std::vector<uint32_t> order((size_t)nt);
  ILG_CUDA(cudaMemcpyAsync(rp.data(), c.rowptr.p, rp.size() * 8, cudaMemcpyDeviceToHost, s));
  ILG_CUDA(cudaMemcpyAsync(order.data(), c.morton_order.p, (size_t)nt * 4, cudaMemcpyDeviceToHost, s));
  dbuf<unsigned long long> dkey;
  dbuf<uint32_t> dsv;
  const unsigned long long cmask = (1ull << rb) - 1;
  if (nnz > 0) {
    dbuf<uint32_t> drank;
    ILG_TRY(drank.alloc(nt));
    ILG_TRY(dkey.alloc(nnz));
    ILG_TRY(dsv.alloc(nnz));
    k_rank<<<div_up(nt, 256), 256, 0, s>>>(c.morton_order.p, nt, drank.p);
    ILG_CUDA(cudaGetLastError());
    k_row_keys<<<div_up(nt, 256), 256, 0, s>>>(c.rowptr.p, c.col.p, drank.p, nt, rb, dkey.p, dsv.p);
    ILG_CUDA(cudaGetLastError());
    ILG_TRY(radix_sort_u64(dkey.p, dsv.p, nnz, 2 * rb, c.sort, s));
  }
  ILG_CUDA(cudaStreamSynchronize(s));

  // active rows (with entries) in Morton order
  std::vector<uint8_t> act((size_t)nt, 0);
  std::vector<int> arow;   // positions
  for (int p = 0; p < nt; ++p) {
    int g = (int)order[p];
    int64_t len = rp[g + 1] - rp[g];
    if (len > 0) {
      if (len > RAD_HALO) {
        set_error("facet %d sees %lld facets; the radiosity solve supports at most %d per facet", g,
                  (long long)len, RAD_HALO);
        return ILG_ERR_ARG;
      }
      act[p] = 1;
      arow.push_back(p);
    }
  }
  c.n_active = (int)arow.size();

  // Tile cuts. A tile's stream time follows its whole groups (every thread
  // runs ceil(entries / RAD_GROUP) groups of four), so tiles get equal group
  // counts: the smallest ng for which a greedy pass with at most ng * RAD_GROUP
  // entries per tile needs no more tiles than co-resident blocks. A second
  // pass also closes a tile early once its weighed cost (entries + rows)
  // exceeds ng * RAD_GROUP plus the first pass's mean row cost, so row-heavy
  // tiles carry fewer entries; it is kept if it still fits the grid. If the
  // row cap forces more tiles than blocks (very large meshes), the cuts are
  // equal shares of the estimated work (entries + rows), several tiles per
  // block. Halos are then counted exactly on the device and a tile whose
  // halo exceeds the shared-memory capacity is split in two, until none
  // does.
  const int Gdev = g_rad_nsm * std::min(g_rad_per_sm64, g_rad_per_smm);
  const int G = c.tile_blocks > 0 ? std::min(Gdev, c.tile_blocks) : Gdev;
  std::vector<RowTile> tiles;
  std::vector<size_t> tile_a;   // first active row of each tile
  std::vector<int64_t> tile_ne;  // entries of each tile
  const int64_t NOCAP = std::numeric_limits<int64_t>::max() / 4;
  auto rlen = [&](size_t q) { const int g = (int)order[arow[q]]; return rp[g + 1] - rp[g]; };
  auto push_tile = [&](size_t a, size_t b, int64_t ne) {
    RowTile T{};
    T.lam = (int)(((ne + RAD_THREADS - 1) / RAD_THREADS + 3) & ~(int64_t)3);
    T.nrows = (int)(b - a);
    T.mesh = 0;
    tiles.push_back(T);
    tile_a.push_back(a);
    tile_ne.push_back(ne);
  };
  // One greedy pass. cap > 0: at most cap entries and cap + slack weighed
  // cost per tile; returns false once more than max_tiles are needed, and
  // counts the tiles closed by the row cap. cap == 0: cumulative equal
  // shares of total_cost over ntarget tiles.
  auto cut = [&](int64_t cap, int64_t slack, int64_t total_cost, int64_t ntarget, size_t max_tiles,
                 int* capped) -> bool {
    tiles.clear();
    tile_a.clear();
    tile_ne.clear();
    if (capped) *capped = 0;
    int64_t done_cost = 0;
    size_t a = 0;
    while (a < arow.size()) {
      if (tiles.size() >= max_tiles) return false;
      const int tid = (int)tiles.size();
      const int64_t bound = cap > 0 ? 0 : (int64_t)((double)total_cost * (double)(tid + 1) / (double)ntarget);
      size_t b = a;
      int64_t ne = 0;
      while (b < arow.size()) {
        if (b > a && (int64_t)(b - a) >= RAD_ROWS) {
          if (capped) ++*capped;
          break;
        }
        const int64_t len = rlen(b);
        if (cap > 0 && b > a && ne + len > cap) break;
        if (cap > 0 && b > a && ne + len + RAD_ROW_COST * (int64_t)(b - a + 1) > cap + slack) break;
        ne += len;
        ++b;
        if (cap == 0 && done_cost + ne + RAD_ROW_COST * (int64_t)(b - a) >= bound && tid + 1 < ntarget) break;
      }
      push_tile(a, b, ne);
      done_cost += ne + RAD_ROW_COST * (int64_t)(b - a);
      a = b;
    }
    return true;
  };
  {
    int64_t ng = std::max<int64_t>((RAD_MIN_TILE + RAD_GROUP - 1) / RAD_GROUP,
                                   (nnz + (int64_t)G * RAD_GROUP - 1) / ((int64_t)G * RAD_GROUP));
    bool ok = false;
    int capped = 0;
    for (int tries = 0; tries < 4; ++tries, ++ng) {
      ok = cut(ng * RAD_GROUP, NOCAP, 0, 0, (size_t)G, &capped);
      if (ok || capped > 0) break;   // a larger ng cannot lift the row cap
    }
    if (ok && !tiles.empty()) {
      int64_t extra = 0;
      for (const RowTile& T : tiles) extra += RAD_ROW_COST * T.nrows;
      const int64_t slack = extra / (int64_t)tiles.size();
      if (!cut(ng * RAD_GROUP, slack, 0, 0, (size_t)G, nullptr)) cut(ng * RAD_GROUP, NOCAP, 0, 0, (size_t)G, nullptr);
    } else if (!ok) {
      const int64_t ntarget = std::max<int64_t>(1, std::min<int64_t>(G, (nnz + RAD_MIN_TILE - 1) / RAD_MIN_TILE));
      const int64_t total_cost = nnz + RAD_ROW_COST * (int64_t)arow.size();
      cut(0, 0, total_cost, ntarget, (size_t)-1, nullptr);
    }
  }
  // per row: its tile and first entry within the tile; per tile: stored
  // offset and rows; then the exact halos on the device (the entries
  // sorted by (tile, column): runs = halo facets), splitting over-full tiles
  std::vector<int> tile_of((size_t)nt, 0), rowoff((size_t)nt, 0);
  std::vector<uint32_t> trow(arow.size());
  std::vector<int> rowj0(arow.size());
  std::vector<int> tfirst;
  int64_t stored_total = 0;
  int ntile = 0;
  dbuf<uint32_t> t_halo_tmp;
  dbuf<int> dtile_of, drowoff, dtfirst;
  dbuf<unsigned long long> key2, before;
  dbuf<uint32_t> idx2, flag;
  if (!tiles.empty()) {
    ILG_TRY(dtile_of.alloc(nt));
    ILG_TRY(drowoff.alloc(nt));
    ILG_TRY(key2.alloc(nnz));
    ILG_TRY(idx2.alloc(nnz));
    ILG_TRY(flag.alloc(nnz));
    ILG_TRY(before.alloc(nnz));
    ILG_TRY(t_halo_tmp.alloc(nnz));
  }
  // Tiles much larger than nnz / (4 x blocks) entries are halved as well
  // (when that is above RAD_SPLIT_MIN): with a few tiles per block the
  // longest-first schedule keeps the blocks' loads within a tile of each
  // other.
  const int64_t split_target = std::max<int64_t>(RAD_SPLIT_MIN, nnz / (4 * (int64_t)G));
  for (int iter = 0; !tiles.empty(); ++iter) {
    ntile = (int)tiles.size();
    stored_total = 0;
    int64_t rows_total = 0;
    for (int tid = 0; tid < ntile; ++tid) {
      RowTile& T = tiles[tid];
      T.e0 = stored_total;
      T.r0 = (int)rows_total;
      stored_total += (int64_t)T.lam * RAD_THREADS;
      int64_t j = 0;
      for (int q = 0; q < T.nrows; ++q) {
        const int p = arow[tile_a[tid] + q];
        const int g = (int)order[p];
        tile_of[g] = tid;
        rowoff[g] = (int)j;
        trow[(size_t)rows_total + q] = (uint32_t)p;
        rowj0[(size_t)rows_total + q] = (int)j;
        j += rp[g + 1] - rp[g];
      }
      rows_total += T.nrows;
    }
    ILG_TRY(dtfirst.reserve(ntile + 1));
    ILG_CUDA(cudaMemcpyAsync(dtile_of.p, tile_of.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(drowoff.p, rowoff.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, s));
    k_tile_keys<<<div_up(nnz, 256), 256, 0, s>>>(dkey.p, nnz, rb, dtile_of.p, key2.p, idx2.p);
    ILG_CUDA(cudaGetLastError());
    int tb = 1;
    while ((1 << tb) < ntile) ++tb;
    ILG_TRY(radix_sort_u64(key2.p, idx2.p, nnz, tb + rb, c.sort, s));
    k_run_flags<<<div_up(nnz, 256), 256, 0, s>>>(key2.p, nnz, flag.p);
    ILG_CUDA(cudaGetLastError());
    ILG_TRY(scan_exclusive_u32_to_u64(flag.p, before.p, nnz, c.scan, s));
    k_halo_runs<<<div_up(nnz, 256), 256, 0, s>>>(key2.p, flag.p, before.p, nnz, rb, t_halo_tmp.p, dtfirst.p);
    ILG_CUDA(cudaGetLastError());
    tfirst.assign((size_t)ntile + 1, 0);
    unsigned long long last_before = 0;
    uint32_t last_flag = 0;
    ILG_CUDA(cudaMemcpyAsync(tfirst.data(), dtfirst.p, (size_t)ntile * 4, cudaMemcpyDeviceToHost, s));
    ILG_CUDA(cudaMemcpyAsync(&last_before, before.p + nnz - 1, 8, cudaMemcpyDeviceToHost, s));
    ILG_CUDA(cudaMemcpyAsync(&last_flag, flag.p + nnz - 1, 4, cudaMemcpyDeviceToHost, s));
    ILG_CUDA(cudaStreamSynchronize(s));
    tfirst[ntile] = (int)(last_before + last_flag);
    bool split = false;
    std::vector<RowTile> nt_tiles;
    std::vector<size_t> nt_a;
    std::vector<int64_t> nt_ne;
    for (int tid = 0; tid < ntile; ++tid) {
      RowTile T = tiles[tid];
      T.h0 = tfirst[tid];
      T.nhalo = tfirst[tid + 1] - tfirst[tid];
      if (T.nhalo < 1) { set_error("row tile without a halo"); return ILG_ERR_CUDA; }
      const bool big = tile_ne[tid] > 2 * split_target;
      if ((T.nhalo <= RAD_HALO && !big) || T.nrows < 2) {
        if (T.nhalo > RAD_HALO) { set_error("row tile halo of %d facets", T.nhalo); return ILG_ERR_CUDA; }
        nt_tiles.push_back(T);
        nt_a.push_back(tile_a[tid]);
        nt_ne.push_back(tile_ne[tid]);
        continue;
      }
      // split at the row where the entries reach half
      split = true;
      const size_t a = tile_a[tid], b = a + T.nrows;
      size_t m = a;
      int64_t ne0 = 0;
      while (m + 1 < b && 2 * (ne0 + rlen(m)) <= tile_ne[tid]) ne0 += rlen(m++);
      if (m == a) ne0 += rlen(m++);
      for (int half = 0; half < 2; ++half) {
        const size_t ha = half ? m : a, hb = half ? b : m;
        const int64_t hne = half ? tile_ne[tid] - ne0 : ne0;
        RowTile H{};
        H.lam = (int)(((hne + RAD_THREADS - 1) / RAD_THREADS + 3) & ~(int64_t)3);
        H.nrows = (int)(hb - ha);
        H.mesh = 0;
        nt_tiles.push_back(H);
        nt_a.push_back(ha);
        nt_ne.push_back(hne);
      }
    }
    tiles.swap(nt_tiles);
    tile_a.swap(nt_a);
    tile_ne.swap(nt_ne);
    if (!split) break;
    if (iter > 40) { set_error("row tiles: halos do not fit after %d splits", iter); return ILG_ERR_CUDA; }
  }
  if (ntile > 0) {
    c.ntiles = ntile;
    c.tile_elems = stored_total;
    c.tiles_h = tiles;
    const int64_t ns = stored_total;
    ILG_TRY(c.tiles.alloc(ntile));
    ILG_TRY(c.t_cf.alloc(ns));
    ILG_TRY(c.t_vhi.alloc(ns));
    ILG_TRY(c.t_vlo.alloc(ns));
    ILG_TRY(c.t_vbf.alloc(ns));
    ILG_TRY(c.t_row.alloc(trow.size()));
    ILG_TRY(c.t_scale.alloc(trow.size()));
    ILG_TRY(c.t_halo.alloc(tfirst[ntile]));
    ILG_TRY(c.t_start.alloc((size_t)ntile * RAD_THREADS));
    ILG_TRY(c.tile_d2.alloc(2 * (size_t)ntile));
    dbuf<uint32_t> dsrc, dfac;
    dbuf<int> drowj0;
    dbuf<int64_t> dne;
    ILG_TRY(dsrc.alloc(ns));
    ILG_TRY(dfac.alloc(ns));
    ILG_TRY(drowj0.alloc(rowj0.size()));
    ILG_TRY(dne.alloc(ntile));
    ILG_CUDA(cudaMemcpyAsync(c.tiles.p, tiles.data(), tiles.size() * sizeof(RowTile), cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.t_row.p, trow.data(), trow.size() * 4, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(drowj0.p, rowj0.data(), rowj0.size() * 4, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(dne.p, tile_ne.data(), (size_t)ntile * 8, cudaMemcpyHostToDevice, s));
    ILG_CUDA(cudaMemcpyAsync(c.t_halo.p, t_halo_tmp.p, (size_t)tfirst[ntile] * 4, cudaMemcpyDeviceToDevice, s));
    // padding slots: no entry (zero halo index, no source)
    ILG_CUDA(cudaMemsetAsync(c.t_cf.p, 0, (size_t)ns * 2, s));
    ILG_CUDA(cudaMemsetAsync(dsrc.p, 0xff, (size_t)ns * 4, s));
    ILG_CUDA(cudaMemsetAsync(dfac.p, 0, (size_t)ns * 4, s));
    k_tile_slots<<<div_up(nnz, 256), 256, 0, s>>>(key2.p, idx2.p, flag.p, before.p, nnz, rb, dkey.p, dsv.p,
                                                  c.rowptr.p, drowoff.p, c.tiles.p, c.t_cf.p, dsrc.p, dfac.p);
    ILG_CUDA(cudaGetLastError());
    k_tile_starts<<<div_up((int64_t)ntile * RAD_THREADS, 256), 256, 0, s>>>(c.tiles.p, ntile, dne.p, drowj0.p,
                                                                            c.t_start.p);
    ILG_CUDA(cudaGetLastError());
    k_tile_fill<<<div_up(ns, 256), 256, 0, s>>>(dsrc.p, dfac.p, ns, c.val.p, c.row_scale.p, c.t_vhi.p, c.t_vlo.p,
                                                c.t_vbf.p);
    ILG_CUDA(cudaGetLastError());
    k_tile_scale<<<div_up((int64_t)trow.size(), 256), 256, 0, s>>>(c.t_row.p, c.rperm.p, (int)trow.size(),
                                                                  c.row_scale.p, c.t_scale.p);
    ILG_CUDA(cudaGetLastError());
    ILG_CUDA(cudaStreamSynchronize(s));
    c.sched_grid = radiosity_grid(ntile, ILG_PREC_FP64);
    ILG_TRY(radiosity_schedule(tiles, c.sched_grid, c.sched_start, c.sched_tile, s));
  } else {
    c.sched_grid = radiosity_grid(0, ILG_PREC_FP64);
    ILG_TRY(radiosity_schedule({}, c.sched_grid, c.sched_start, c.sched_tile, s));
    c.ntiles = 0;
    c.tile_elems = 0;
    c.tiles_h.clear();
    ILG_TRY(c.tiles.alloc(1));
    ILG_TRY(c.t_cf.alloc(1));
    ILG_TRY(c.t_vhi.alloc(1));
    ILG_TRY(c.t_vlo.alloc(1));
    ILG_TRY(c.t_vbf.alloc(1));
    ILG_TRY(c.t_row.alloc(1));
    ILG_TRY(c.t_scale.alloc(1));
    ILG_TRY(c.t_halo.alloc(1));
    ILG_TRY(c.t_start.alloc(RAD_THREADS));
    ILG_TRY(c.tile_d2.alloc(2));
  }
  ILG_TRY(c.row_act.alloc(nt));
  ILG_CUDA(cudaMemcpyAsync(c.row_act.p, act.data(), (size_t)nt, cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  return ILG_OK;
}

int radiosity_max_meshes() { return RAD_MAX_MESH; }
int radiosity_threads() { return RAD_THREADS; }
// 10 bytes per stored entry (u16 column, f32 hi, f32 lo or bf16): streamed
// when it would not stay in the 126 MB L2 between passes.
int radiosity_l2_stream(int64_t stored) { return stored * 10 > (int64_t)96 << 20 ? 1 : 0; }

size_t radiosity_barrier_words(int nmesh) { return 2 + 2 * 3 * (size_t)(nmesh > 0 ? nmesh : 1); }

// Cooperative grid size for ntiles tiles (at most the co-resident blocks).
// Both solves launch the same block shape and shared memory, so one grid
// (and one tile schedule) serves either precision.
int radiosity_grid(int ntiles, int precision) {
  (void)precision;
  if (radiosity_setup() != ILG_OK) return 1;
  int per_sm = std::min(g_rad_per_smm, g_rad_per_sm64);
  int grid = per_sm * g_rad_nsm;
  if (ntiles < grid) grid = ntiles;
  return grid < 1 ? 1 : grid;
}

// Tile cost in stored entries (RAD_ROW_COST per row, RAD_HALO_COST per halo
// facet, plus a fixed cost of one group for the tile's set-up).
int radiosity_schedule(const std::vector<RowTile>& tiles, int grid, dbuf<int>& start, dbuf<int>& order,
                       cudaStream_t s) {
  const int n = (int)tiles.size();
  if (grid < 1) grid = 1;
  std::vector<int> idx(n);
  std::vector<int64_t> cost(n);
  for (int t = 0; t < n; ++t) {
    const RowTile& T = tiles[t];
    idx[t] = t;
    cost[t] = (int64_t)T.lam * RAD_THREADS + RAD_ROW_COST * T.nrows + RAD_HALO_COST * T.nhalo + RAD_GROUP;
  }
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return cost[a] != cost[b] ? cost[a] > cost[b] : a < b; });
  std::vector<int64_t> load((size_t)grid, 0);
  std::vector<std::vector<int>> lists((size_t)grid);
  // least loaded block: a binary heap of (load, block)
  std::vector<std::pair<int64_t, int>> heap;
  for (int b = 0; b < grid; ++b) heap.push_back({0, b});
  auto cmp = [](const std::pair<int64_t, int>& a, const std::pair<int64_t, int>& b) {
    return a.first != b.first ? a.first > b.first : a.second > b.second;
  };
  std::make_heap(heap.begin(), heap.end(), cmp);
  for (int t : idx) {
    std::pop_heap(heap.begin(), heap.end(), cmp);
    auto& top = heap.back();
    lists[(size_t)top.second].push_back(t);
    top.first += cost[t];
    std::push_heap(heap.begin(), heap.end(), cmp);
  }
  std::vector<int> st((size_t)grid + 1, 0), ord;
  ord.reserve(n);
  for (int b = 0; b < grid; ++b) {
    std::sort(lists[(size_t)b].begin(), lists[(size_t)b].end());
    for (int t : lists[(size_t)b]) ord.push_back(t);
    st[(size_t)b + 1] = (int)ord.size();
  }
  ILG_TRY(start.alloc((size_t)grid + 1));
  ILG_TRY(order.alloc(n > 0 ? (size_t)n : 1));
  ILG_CUDA(cudaMemcpyAsync(start.p, st.data(), st.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  if (n > 0) ILG_CUDA(cudaMemcpyAsync(order.p, ord.data(), ord.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaStreamSynchronize(s));
  return ILG_OK;
}

// Launches the cooperative solve for every active mesh of the view with
// tiles. x: result (also the warm start when warm). Per-mesh sweep counts
// and residuals land in the mesh table.
int radiosity_inner(int max_sweeps) { return max_sweeps < 1 ? 1 : (max_sweeps < RAD_INNER ? max_sweeps : RAD_INNER); }

namespace {
// Waits at one grid barrier that expects `expected` arrivals: with
// expected > gridDim.x nobody can open it and every block's wait runs out.
__global__ void k_barrier_probe(unsigned* bar, unsigned expected, int* derr) {
  unsigned gen = 0;
  grid_barrier(bar, expected, gen, derr);
}
}  // namespace

// One cooperative launch of `blocks` blocks waiting at a barrier that
// `unreachable` keeps shut, with the poll limit set to `polls` for the
// launch (and restored after it). The wait's outcome is in the view's error
// flags, read by the caller.
int radiosity_barrier_probe(unsigned* bar, int* derr, int blocks, long long polls, int unreachable, cudaStream_t s) {
  if (blocks < 1 || blocks > 8 || polls < 1) { set_error("invalid barrier probe"); return ILG_ERR_ARG; }
  ILG_CUDA(cudaMemcpyToSymbolAsync(g_barrier_polls, &polls, sizeof(polls), 0, cudaMemcpyHostToDevice, s));
  ILG_CUDA(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), s));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(32);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const unsigned expected = (unsigned)blocks + (unreachable ? 1u : 0u);
  const cudaError_t e = cudaLaunchKernelEx(&cfg, k_barrier_probe, bar, expected, derr);
  const long long standard = BARRIER_POLLS;
  const cudaError_t e2 = cudaMemcpyToSymbolAsync(g_barrier_polls, &standard, sizeof(standard), 0,
                                                 cudaMemcpyHostToDevice, s);
  ILG_CUDA(e);
  ILG_CUDA(e2);
  ILG_CUDA(cudaStreamSynchronize(s));
  return ILG_OK;
}

int radiosity_launch(const StepView& v, double* x, int warm, int precision, int grid, int inner, bool lagged,
                     cudaStream_t s) {
  ILG_TRY(radiosity_setup());
  if (!v.blk_start || grid != v.sched_grid) {
    set_error("radiosity grid %d has no tile schedule (made for %d blocks)", grid, v.sched_grid);
    return ILG_ERR_ARG;
  }
  ILG_CUDA(cudaMemsetAsync(v.barrier, 0, 2 * sizeof(unsigned), s));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(RAD_BLOCK);
  cfg.dynamicSmemBytes = RAD_SMEM;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;   // all blocks co-resident: the grid barrier is safe
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (precision == ILG_PREC_MIXED && lagged)
    ILG_CUDA(cudaLaunchKernelEx(&cfg, k_radiosity_lagged, v, x, warm));
  else if (precision == ILG_PREC_MIXED)
    ILG_CUDA(cudaLaunchKernelEx(&cfg, k_radiosity_mixed, v, x, warm, radiosity_inner(inner)));
  else
    ILG_CUDA(cudaLaunchKernelEx(&cfg, k_radiosity64, v, x, warm));
  return ILG_OK;
}

}  // namespace ilg
