// Standalone linear solves in the reference's matrix layouts:
//
//   gf_sparse_solve   K in SparseMatrix's layout (Eigen row-major CSR,
//                     0-based), replaces sparsesystem (reference
//                     src/SparseMatrix.cpp:74-166)
//   wide_band_solve   K in BandMatrix's LAPACK GB layout with a half
//                     bandwidth above 17, the wide branch of gf_band_solve
//                     (bandsystem, src/BandMatrix.cpp:257-287)
//
// Both factor on the GPU with the blocked no-pivot wide-band LU of the
// Shell_1 path (gf_shell.cu) run on a batch of one structure; systems with
// a half-bandwidth of at most 17 go to the 35-row band solver instead.
// The CSR path picks the narrower of the natural ordering and reverse
// Cuthill-McKee on the symmetrised pattern, as the batch path does for
// shells.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "../../include/giraffe_gpu.h"
#include "gf_host_internal.h"
#include "gf_kernels.cuh"
#include "gf_types.h"
#include "gf_wide.h"

using namespace gf;

namespace gf {

// CSR rows scattered into the wide band (column-major, W = 2w + 1 rows,
// entry (i, j) at (w + i - j) + j W) under the symmetric permutation perm,
// one thread per row: distinct rows own distinct band entries, and the
// entries of a row are summed in order, so duplicates add up the same way
// on every run.  The right-hand side is permuted alongside.
__global__ void k_csr_to_wide(int n, const int* rp, const int* ci, const double* v, const int* perm, double* a,
                              int w, int64_t W, const double* b, double* P) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int pi = perm[i];
  for (int k = rp[i]; k < rp[i + 1]; ++k) {
    const int pj = perm[ci[k]];
    a[(w + pi - pj) + (int64_t)pj * W] += v[k];
  }
  P[pi] = b[i];
}

// x[i] = y[perm[i]]
__global__ void k_unpermute(int n, const int* perm, const double* y, double* x) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = y[perm[i]];
}

}  // namespace gf

namespace {

using namespace gfh;

// Half-bandwidth max |i - j| of the pattern under the ordering pos (row or
// column i at pos[i]).
int csr_bandwidth(int n, const int* rp, const int* ci, const int* pos) {
  int w = 0;
  for (int i = 0; i < n; ++i)
    for (int k = rp[i]; k < rp[i + 1]; ++k) w = std::max(w, std::abs(pos[i] - pos[ci[k]]));
  return w;
}

}  // namespace

namespace gfh {

// Wide branch of gf_band_solve: the GB array goes into the wide band with
// one strided copy (each column's kl + ku + 1 stored entries keep their
// order), then the blocked LU runs.
int wide_band_solve(gf_ctx* ctx, int n, int kl, int ku, const double* ab, int ldab, double* b, int* info) {
  const int w = std::max(kl, ku);
  const int64_t W = 2 * (int64_t)w + 1;
  DevBufs mem;
  Helpers hl;
  double *dband = nullptr, *dP = nullptr, *dY = nullptr;
  if (!mem.get(&dband, (size_t)n * W) || !mem.get(&dP, (size_t)n) || !mem.get(&dY, (size_t)n)) {
    set_err(ctx, "gf_band_solve: device allocation of %lld bytes failed", (long long)(8 * ((size_t)n * W + 2 * n)));
    return GF_ERR_CUDA;
  }
  cudaStream_t s = ctx->stream;
  // GB entry (i, j) sits at row kl + ku + i - j of column j; the wide band
  // holds it at row w + i - j, so rows kl .. 2 kl + ku of a GB column land
  // on rows w - ku .. w + kl
  GF_CK(cudaMemsetAsync(dband, 0, sizeof(double) * (size_t)n * W, s));
  GF_CK(cudaMemcpy2DAsync(dband + (w - ku), sizeof(double) * W, ab + kl, sizeof(double) * ldab,
                          sizeof(double) * (kl + ku + 1), n, cudaMemcpyHostToDevice, s));
  GF_CK(cudaMemcpyAsync(dP, b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  WideBatch wb;
  if (!wb.init(ctx, mem, hl, n, w, dband, dP, dY)) {
    set_err(ctx, "gf_band_solve: set-up of the wide-band solve failed");
    return GF_ERR_CUDA;
  }
  int fail = 0;
  GF_CK(wb.solve(ctx, &fail));
  GF_CK(cudaMemcpy(b, dP, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (info) *info = fail;
  return GF_OK;
}

}  // namespace gfh

extern "C" {

int gf_sparse_solve(gf_ctx* ctx, int n, const int* row_ptr, const int* col_idx, const double* val, double* b,
                    int* info) {
  if (!ctx || n <= 0 || !row_ptr || !col_idx || !val || !b) {
    if (ctx) gfh::set_err(ctx, "gf_sparse_solve: invalid arguments");
    return GF_ERR_ARG;
  }
  if (row_ptr[0] != 0) {
    gfh::set_err(ctx, "gf_sparse_solve: row_ptr[0] must be 0 (0-based CSR)");
    return GF_ERR_ARG;
  }
  for (int i = 0; i < n; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) {
      gfh::set_err(ctx, "gf_sparse_solve: row_ptr decreases at row %d", i);
      return GF_ERR_ARG;
    }
  const int nnz = row_ptr[n];
  for (int k = 0; k < nnz; ++k)
    if (col_idx[k] < 0 || col_idx[k] >= n) {
      gfh::set_err(ctx, "gf_sparse_solve: column index %d out of range at entry %d", col_idx[k], k);
      return GF_ERR_ARG;
    }
  // ordering: natural, or reverse Cuthill-McKee on the symmetrised pattern
  // when that narrows the band
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  int w = csr_bandwidth(n, row_ptr, col_idx, perm.data());
  if (w > 2 * GF_KB) {
    std::vector<std::vector<int>> adj(n);
    for (int i = 0; i < n; ++i)
      for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        const int j = col_idx[k];
        if (j == i) continue;
        adj[i].push_back(j);
        adj[j].push_back(i);
      }
    for (auto& v : adj) {
      std::sort(v.begin(), v.end());
      v.erase(std::unique(v.begin(), v.end()), v.end());
    }
    const std::vector<int> order = gfh::rcm_order(n, adj);  // order[k] = row placed k-th
    std::vector<int> pos(n);
    for (int k = 0; k < n; ++k) pos[order[k]] = k;
    const int w_rcm = csr_bandwidth(n, row_ptr, col_idx, pos.data());
    if (w_rcm < w) {
      w = w_rcm;
      perm = pos;
    }
  }
  w = std::max(w, 1);
  if (w <= GF_KB) {
    // narrow: LAPACK GB of the permuted matrix, through gf_band_solve
    const int ldab = 3 * w + 1;
    std::vector<double> ab((size_t)n * ldab, 0.0), x(n);
    for (int i = 0; i < n; ++i)
      for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        const int pi = perm[i], pj = perm[col_idx[k]];
        ab[(size_t)(2 * w + pi - pj) + (size_t)pj * ldab] += val[k];
      }
    for (int i = 0; i < n; ++i) x[perm[i]] = b[i];
    int rc = gf_band_solve(ctx, n, w, w, ab.data(), ldab, x.data(), info);
    if (rc != GF_OK) return rc;
    for (int i = 0; i < n; ++i) b[i] = x[perm[i]];
    return GF_OK;
  }
  const int64_t W = 2 * (int64_t)w + 1;
  DevBufs mem;
  Helpers hl;
  double *dband = nullptr, *dP = nullptr, *dY = nullptr, *dv = nullptr, *db = nullptr;
  int *drp = nullptr, *dci = nullptr, *dperm = nullptr;
  if (!mem.get(&dband, (size_t)n * W) || !mem.get(&dP, (size_t)n) || !mem.get(&dY, (size_t)n) ||
      !mem.get(&dv, (size_t)nnz) || !mem.get(&db, (size_t)n) || !mem.get(&drp, (size_t)n + 1) ||
      !mem.get(&dci, (size_t)nnz) || !mem.get(&dperm, (size_t)n)) {
    gfh::set_err(ctx, "gf_sparse_solve: device allocation failed (half-bandwidth %d, %lld band bytes)", w,
                 (long long)(8 * (size_t)n * W));
    return GF_ERR_CUDA;
  }
  cudaStream_t s = ctx->stream;
  GF_CK(cudaMemsetAsync(dband, 0, sizeof(double) * (size_t)n * W, s));
  GF_CK(cudaMemcpyAsync(drp, row_ptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
  GF_CK(cudaMemcpyAsync(dci, col_idx, sizeof(int) * std::max(nnz, 1), cudaMemcpyHostToDevice, s));
  GF_CK(cudaMemcpyAsync(dv, val, sizeof(double) * std::max(nnz, 1), cudaMemcpyHostToDevice, s));
  GF_CK(cudaMemcpyAsync(db, b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  GF_CK(cudaMemcpyAsync(dperm, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  k_csr_to_wide<<<(n + 127) / 128, 128, 0, s>>>(n, drp, dci, dv, dperm, dband, w, W, db, dP);
  WideBatch wbt;
  if (!wbt.init(ctx, mem, hl, n, w, dband, dP, dY)) {
    gfh::set_err(ctx, "gf_sparse_solve: set-up of the wide-band solve failed");
    return GF_ERR_CUDA;
  }
  int fail = 0;
  GF_CK(wbt.solve(ctx, &fail));
  k_unpermute<<<(n + 127) / 128, 128, 0, s>>>(n, dperm, dP, db);
  GF_CK(cudaGetLastError());
  GF_CK(cudaMemcpyAsync(b, db, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  GF_CK(cudaStreamSynchronize(s));
  if (info) *info = fail;
  return GF_OK;
}

}  // extern "C"
