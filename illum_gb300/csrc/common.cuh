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

// Owning device buffer (cudaMalloc / cudaFree). Not copyable.
template <class T>
struct dbuf {
  T* p = nullptr;
  size_t n = 0;
  dbuf() = default;
  dbuf(const dbuf&) = delete;
  dbuf& operator=(const dbuf&) = delete;
  dbuf(dbuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  dbuf& operator=(dbuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~dbuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  int alloc(size_t count) {
    if (count == n && p) return ILG_OK;
    release();
    if (count == 0) return ILG_OK;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      set_error("cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
      return ILG_ERR_NOMEM;
    }
    n = count;
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
  DERR_COUNT = 8
};

// ---- primitives (primitives.cu) ----
// Exclusive prefix sum of n 64-bit counts; out may alias in. Uses tmp
// scratch grown on demand. *total receives the sum when non-null (device->host
// copy, synchronising the stream).
struct ScanScratch { dbuf<unsigned long long> a, b, c; };
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
};
int radix_sort_u64(unsigned long long* keys, uint32_t* vals, int64_t n, int bits, SortScratch& tmp,
                   cudaStream_t s);

}  // namespace ilg
