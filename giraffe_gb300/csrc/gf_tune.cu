// Autotuner of the wide-band LU's tile shapes (WideTiles): the rows per CTA
// of the bulk and of the first trsm, the corner update's tile edge and the
// rows per CTA of the triangular solves.  None of them changes any entry's
// arithmetic, so the choice is free to follow the clock.  For a
// half-bandwidth kl the tuner factors and solves a synthetic band of the same
// kl (diagonally dominant, kl + 12 panels of rows, so every panel's window has
// its full size) with the batch's trailing-update kernel, and walks the
// shapes one coordinate at a time from the defaults, keeping a change only
// when it is at least 2 % faster (best of three timed factor-and-solves each,
// CUDA events on the tuning stream).  Results are cached per context and kl.
#include <cuda_runtime.h>

#include <cfloat>

#include "gf_wide.h"

namespace gfh {

namespace {

__device__ __forceinline__ unsigned tune_hash(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return (unsigned)x;
}

// Band [n][2 kl + 1] (entry (i, j) at (kl + i - j) + j (2 kl + 1)): entries
// uniform in [-0.5, 0.5), the diagonal 2 kl + 2, zero outside the matrix.
__global__ void k_tune_fill(double* a, int n, int kl) {
  const int64_t W = 2 * (int64_t)kl + 1, total = (int64_t)n * W;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < total; x += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(x / W), row = (int)(x % W) - kl + j;
    double v = 0.0;
    if (row >= 0 && row < n) v = row == j ? 2.0 * kl + 2.0 : (tune_hash(x) >> 8) * 0x1p-24 - 0.5;
    a[x] = v;
  }
}

}  // namespace

WideTiles tune_wide_tiles(gf_ctx* ctx, int kl, int wide_update) {
  const long long key = (long long)kl * 4 + wide_update;
  auto it = ctx->tiles.find(key);
  if (it != ctx->tiles.end()) return it->second;
  WideTiles best;  // the defaults, also the answer when tuning cannot run
  const int n = kl + 12 * GF_WB_NB;
  const int64_t W = 2 * (int64_t)kl + 1;
  DevBufs mem;
  Helpers hl;
  double *band = nullptr, *band0 = nullptr, *P = nullptr, *y = nullptr;
  WideBatch wb;
  cudaStream_t s = ctx->stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  bool ok = mem.get(&band, (size_t)n * W) && mem.get(&band0, (size_t)n * W) && mem.get(&P, (size_t)n) &&
            mem.get(&y, (size_t)n) && wb.init(ctx, mem, hl, n, kl, band, P, y) &&
            cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
  if (ok) {
    wb.b.sh.wide_tc = wide_update;
    k_tune_fill<<<4 * 152, 256, 0, s>>>(band0, n, kl);
    ok = cudaMemsetAsync(P, 0, sizeof(double) * n, s) == cudaSuccess;
  }
  // best of three factor-and-solves at tile shapes t (ms); FLT_MAX on error
  auto time_at = [&](const WideTiles& t) -> float {
    float bestms = FLT_MAX;
    wb.b.sh.tiles = t;
    for (int r = 0; r < 3 && ok; ++r) {
      float ms = 0.f;
      if (cudaMemcpyAsync(band, band0, sizeof(double) * n * W, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
          cudaEventRecord(e0, s) != cudaSuccess) {
        ok = false;
        break;
      }
      launch_wide_solve(wb.b, s);
      if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        ok = false;
        break;
      }
      bestms = ms < bestms ? ms : bestms;
    }
    return bestms;
  };
  if (ok) {
    time_at(best);  // warm-up: first launches of every kernel
    float tb = time_at(best);
    const int first[] = {1, 2, 4}, corner[] = {4, 8}, bulk[] = {4, 8, 16}, rows[] = {32, 64};
    auto walk = [&](int WideTiles::*field, const int* vals, int nv) {
      for (int k = 0; k < nv && ok; ++k) {
        if (vals[k] == best.*field) continue;
        WideTiles t = best;
        t.*field = vals[k];
        const float ms = time_at(t);
        if (ms < 0.98f * tb) {
          best = t;
          tb = ms;
        }
      }
    };
    walk(&WideTiles::trsm_first, first, 3);
    walk(&WideTiles::corner, corner, 2);
    walk(&WideTiles::trsm_rb, bulk, 3);
    walk(&WideTiles::sub_rows, rows, 2);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaGetLastError();  // a failed trial leaves the defaults and no sticky error
  if (!ok) best = WideTiles();
  else ctx->tiles[key] = best;
  return best;
}

}  // namespace gfh
