// common.cuh — error handling, device buffers and launch helpers shared by
// the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <string>
#include <utility>

#include "../../include/illum_gb300.h"

namespace ilg {

// Last error message of the calling thread (returned by ilg_last_error).
void set_error(const char* fmt, ...);

struct Status {
  int code = ILG_OK;
  explicit operator bool() const { return code != ILG_OK; }
};

#define ILG_CUDA(call)                                                            \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) {                                                      \
      ::ilg::set_error("%s:%d: %s failed: %s", __FILE__, __LINE__, #call,         \
                       cudaGetErrorString(e_));                                   \
      return ILG_ERR_CUDA;                                                        \
    }                                                                             \
  } while (0)

#define ILG_TRY(expr)            \
  do {                           \
    int rc_ = (expr);            \
    if (rc_ != ILG_OK) return rc_; \
  } while (0)

// Stream that orders the calling thread's device allocations: set, for the
// duration of an API call, to the stream of the context (or batch) it works
// on. With one, dbuf allocates from the device's stream-ordered pool and
// frees on that stream, so neither waits for work that other streams have
// queued (cudaFree synchronises the whole device, which stalls a context's
// set-up behind every other context's steps); without one it uses
// cudaMalloc / cudaFree.
extern thread_local cudaStream_t t_alloc_stream;
struct AllocOn {
  cudaStream_t prev;
  explicit AllocOn(cudaStream_t s) : prev(t_alloc_stream) { t_alloc_stream = s; }
  ~AllocOn() { t_alloc_stream = prev; }
  AllocOn(const AllocOn&) = delete;
  AllocOn& operator=(const AllocOn&) = delete;
};
// Keeps freed pool memory cached in the process (set once per device).
int alloc_pool_setup();
int pool_trim(cudaStream_t s);

// A stream destroyed last: the first member of an object whose buffers
// are freed on it, so their stream-ordered frees are queued before the
// stream goes (its pending work still completes after cudaStreamDestroy).
struct OwnedStream {
  cudaStream_t s = nullptr;
  OwnedStream() = default;
  OwnedStream(const OwnedStream&) = delete;
  OwnedStream& operator=(const OwnedStream&) = delete;
  ~OwnedStream() { if (s) cudaStreamDestroy(s); }
};

// Owning device buffer. Not copyable.
template <class T>
struct dbuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;   // the stream it was allocated on (and is freed on), or none
  dbuf() = default;
  dbuf(const dbuf&) = delete;
  dbuf& operator=(const dbuf&) = delete;
  dbuf(dbuf&& o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; o.s = nullptr; }
  dbuf& operator=(dbuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; s = o.s; o.p = nullptr; o.n = 0; o.s = nullptr; }
    return *this;
  }
  ~dbuf() { release(); }
  void release() {
    if (p) {
      if (s) cudaFreeAsync(p, s);
      else cudaFree(p);
    }
    p = nullptr;
    n = 0;
    s = nullptr;
  }
  int alloc(size_t count) {
    if (count == n && p) return ILG_OK;
    release();
    if (count == 0) return ILG_OK;
    const cudaStream_t st = t_alloc_stream;
    cudaError_t e = st ? cudaMallocAsync(&p, count * sizeof(T), st) : cudaMalloc(&p, count * sizeof(T));
    // the memory is used at once from the host and other streams: wait for
    // the allocation in its own stream (that stream only)
    if (e == cudaSuccess && st) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      if (p && st) cudaFreeAsync(p, st);
      p = nullptr;
      cudaGetLastError();   // an allocation failure is not sticky: clear it for the caller's later checks
      set_error("device allocation of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
      return ILG_ERR_NOMEM;
    }
    n = count;
    s = st;
    return ILG_OK;
  }
  // grow-only reallocation (contents not preserved)
  int reserve(size_t count) { return count <= n ? ILG_OK : alloc(count); }
};

inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// Double-float split on the host: x = hi + lo, hi = fl32(x), lo = fl32(x - hi).
inline float2 split_df_host(double x) {
  float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}

// Device error flags written by kernels (bounded waits that gave up, stack
// overflows, NaN form factors). One int per kind.
enum DevErr : int {
  DERR_STACK = 0,      // BVH traversal stack overflow
  DERR_NAN = 1,        // NaN form factor
  DERR_BARRIER = 2,    // grid barrier wait exceeded its iteration limit
  DERR_HORIZON = 3,    // horizon bisection deeper than the precomputed tree
  DERR_PIVOT = 4,      // zero pivot in a conduction column
  DERR_STREAM = 5,     // radiosity entry-stream copy wait exceeded its iteration limit
  DERR_COUNT = 8
};

// ---- primitives (primitives.cu) ----
// Exclusive prefix sum of n 64-bit counts; out may alias in. Uses tmp
// scratch grown on demand. *total receives the sum when non-null (device->host
// copy, synchronising the stream).
struct ScanScratch {
  dbuf<unsigned long long> a, b, c;
  void release() { a.release(); b.release(); c.release(); }
};
int scan_exclusive_u64(const unsigned long long* in, unsigned long long* out, int64_t n,
                       ScanScratch& tmp, cudaStream_t s);
int scan_exclusive_u32_to_u64(const uint32_t* in, unsigned long long* out, int64_t n,
                              ScanScratch& tmp, cudaStream_t s);

// Stable LSD radix sort of 64-bit keys on their low `bits` bits, carrying an
// optional 32-bit value. keys/vals are sorted in place (through alt buffers).
struct SortScratch {
  dbuf<unsigned long long> keys_alt;
  dbuf<uint32_t> vals_alt;
  dbuf<unsigned long long> hist;
  ScanScratch scan;
  void release() { keys_alt.release(); vals_alt.release(); hist.release(); scan.release(); }
};
int radix_sort_u64(unsigned long long* keys, uint32_t* vals, int64_t n, int bits, SortScratch& tmp,
                   cudaStream_t s);

}  // namespace ilg
