// gauss_seidel.cu — the reference's fixed-sweep radiosity solve: a forward
// solve of L x = E with L = I - tril(F), then gs_steps Gauss-Seidel sweeps
// x = L^{-1}(E - U x) with U = -triu(F), all in natural row order
// (src/cpp/arma_util.cpp:4-17, src/cpp/illum_cli.cpp:425-433).
//
// Natural-order Gauss-Seidel is a sparse lower-triangular solve per sweep.
// Row i depends on the rows j < i of its lower part, so rows are grouped in
// dependency levels (level(i) = 1 + max level of its lower columns, 0 for
// none) and each level is one launch, one thread per row: every lower column
// of a row is final before the row's level starts. The upper part reads the
// previous sweep's iterate from a second buffer (the sweep must not see
// values of rows j > i that a lower level already updated). Each row sums in
// the reference's order: the upper product accumulated from zero over its
// columns in ascending order (Armadillo's sparse product), added to E, then
// the lower terms in ascending column order (the forward solve); this file
// is compiled without fused multiply-adds, so the result equals the CPU
// oracle's restatement of that order bit for bit. The levels are found on
// the device by relaxation (one pass per level, each O(nnz)) the first time
// the mode is used after the form factors change; a mesh of 81,920 facets
// has a few hundred levels.
#include <algorithm>
#include <vector>

#include "internal.cuh"

namespace ilg {

namespace {

// One relaxation pass of the levels: lev[i] = 1 + max lev[j] over the
// row's lower columns (columns are ascending within a row).
__global__ void k_gs_levels(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col, int n, int* lev,
                            int* changed) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int m = 0;
  for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    int j = col[k];
    if (j >= i) break;
    m = max(m, __ldcg(lev + j) + 1);
  }
  if (m != lev[i]) {
    lev[i] = m;
    *changed = 1;
  }
}

// Right-hand side of a step's solve: the frame's direct flux, coupled as
// src/cpp/illum_cli.cpp:415-421 when the mesh follows the reference.
__global__ void k_gs_rhs(StepView v, double* Eg) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= v.nt) return;
  const MeshDesc& M = v.md[0];
  const double d = v.E[e_slot(M.frame) * v.nt + g];
  Eg[g] = M.coupling == ILG_COUPLE_REFERENCE ? (-v.Fsurf[g] + d) : d;
}

// One level of one sweep: rows[0..count).
__global__ void k_gs_level(const uint32_t* __restrict__ rows, int count, const int64_t* __restrict__ rowptr,
                           const int32_t* __restrict__ col, const double* __restrict__ val,
                           const double* __restrict__ E, const double* __restrict__ xold, double* xnew, int first) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = (int)rows[t];
  const int64_t k0 = rowptr[i], k1 = rowptr[i + 1];
  int64_t kd = k0;   // first column >= i
  while (kd < k1 && col[kd] < i) ++kd;
  // U = -triu(F) and L = I - tril(F) both hold F's diagonal (zero for
  // computed form factors): the upper product includes it, and the forward
  // solve divides by L's diagonal 1 - F_ii (exactly 1 without one)
  const double fii = (kd < k1 && col[kd] == i) ? val[kd] : 0.0;
  double b = E[i];
  if (!first) {
    double u = 0.0;
    for (int64_t k = kd; k < k1; ++k) u = u + val[k] * xold[col[k]];
    b = b + u;
  }
  double xi = b;
  for (int64_t k = k0; k < kd; ++k) xi = xi + val[k] * __ldcg(xnew + col[k]);
  xnew[i] = xi / (1.0 - fii);
}

// Squared residual of row i of (I - F) x = E, in the CPU oracle's order.
__global__ void k_gs_residual(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                              const double* __restrict__ val, const double* __restrict__ E,
                              const double* __restrict__ x, int n, double* r2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double ax = x[i];
  for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) ax = ax - val[k] * x[col[k]];
  const double r = ax - E[i];
  r2[i] = r * r;
}

}  // namespace

int gs_residual_launch(const Context& c, const double* E, const double* x, double* r2, cudaStream_t s) {
  k_gs_residual<<<div_up(c.nt, 256), 256, 0, s>>>(c.rowptr.p, c.col.p, c.val.p, E, x, c.nt, r2);
  ILG_CUDA(cudaGetLastError());
  return ILG_OK;
}

int gs_prepare(Context& c) {
  if (c.gs_ready) return ILG_OK;
  if (!c.have_F) { set_error("no form factors"); return ILG_ERR_ARG; }
  const int n = c.nt;
  dbuf<int> lev, flag;
  ILG_TRY(lev.alloc(n));
  ILG_TRY(flag.alloc(1));
  ILG_CUDA(cudaMemsetAsync(lev.p, 0, (size_t)n * sizeof(int), c.stream));
  for (int pass = 0;; ++pass) {
    if (pass > n) { set_error("Gauss-Seidel levels did not settle"); return ILG_ERR_DEVICE; }
    int h = 0;
    ILG_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), c.stream));
    k_gs_levels<<<div_up(n, 256), 256, 0, c.stream>>>(c.rowptr.p, c.col.p, n, lev.p, flag.p);
    ILG_CUDA(cudaGetLastError());
    ILG_CUDA(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    ILG_CUDA(cudaStreamSynchronize(c.stream));
    if (!h) break;
  }
  // rows in level order (a counting sort of N levels on the host)
  std::vector<int> lh(n);
  ILG_CUDA(cudaMemcpy(lh.data(), lev.p, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost));
  int nlev = n ? *std::max_element(lh.begin(), lh.end()) + 1 : 0;
  std::vector<int> ptr(nlev + 1, 0);
  for (int i = 0; i < n; ++i) ++ptr[lh[i] + 1];
  for (int l = 0; l < nlev; ++l) ptr[l + 1] += ptr[l];
  std::vector<uint32_t> rows(n);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int i = 0; i < n; ++i) rows[fill[lh[i]]++] = (uint32_t)i;
  ILG_TRY(c.gs_rows.alloc(std::max(n, 1)));
  ILG_TRY(c.gs_x.alloc(3 * (size_t)std::max(n, 1)));
  ILG_CUDA(cudaMemcpy(c.gs_rows.p, rows.data(), (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice));
  c.gs_lptr = std::move(ptr);
  c.gs_ready = true;
  return ILG_OK;
}

int gs_levels(const Context& c) { return c.gs_ready ? (int)c.gs_lptr.size() - 1 : 0; }

// 1 + gs_steps sweeps from zero of the system with right-hand side E
// (device, facet order); the result into x (device, facet order).
int gs_solve_launch(const Context& c, const double* E, double* x, int gs_steps, cudaStream_t s) {
  const int n = c.nt;
  double* buf[2] = {c.gs_x.p, c.gs_x.p + n};
  const int nlev = (int)c.gs_lptr.size() - 1;
  for (int sw = 0; sw <= gs_steps; ++sw) {
    double* xnew = sw == gs_steps ? x : buf[sw & 1];
    const double* xold = sw == 0 ? nullptr : buf[(sw - 1) & 1];
    for (int l = 0; l < nlev; ++l) {
      const int r0 = c.gs_lptr[l], cnt = c.gs_lptr[l + 1] - r0;
      k_gs_level<<<div_up(cnt, 128), 128, 0, s>>>(c.gs_rows.p + r0, cnt, c.rowptr.p, c.col.p, c.val.p, E, xold,
                                                 xnew, sw == 0 ? 1 : 0);
    }
    ILG_CUDA(cudaGetLastError());
  }
  return ILG_OK;
}

// A step's solve (the fused loop's radiosity phase in the fixed-sweep mode).
int gs_step_launch(const Context& c, const StepView& v, int gs_steps, cudaStream_t s) {
  double* Eg = c.gs_x.p + 2 * (size_t)c.nt;
  k_gs_rhs<<<div_up(c.nt, 256), 256, 0, s>>>(v, Eg);
  ILG_CUDA(cudaGetLastError());
  return gs_solve_launch(c, Eg, v.rad, gs_steps, s);
}

}  // namespace ilg
