// A one-structure wide-band system on the device for the standalone solves
// (gf_sparse.cu) and the modal analysis (gf_modal.cu): its buffers, the
// lookahead's helper streams and events, and the batch of one structure
// around a device wide band that the wide-band LU kernels (gf_shell.cu)
// take.  Internal to libgiraffe_gpu.so.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "gf_host_internal.h"
#include "gf_kernels.cuh"
#include "gf_types.h"

namespace gfh {

using namespace gf;

// Device buffers of one standalone system; freed on scope exit.
struct DevBufs {
  std::vector<void*> p;
  ~DevBufs() {
    for (void* q : p) cudaFree(q);
  }
  template <typename T> bool get(T** out, size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return false;
    p.push_back(q);
    *out = static_cast<T*>(q);
    return true;
  }
};

// Helper streams and events of the wide LU's lookahead; destroyed on scope
// exit.
struct Helpers {
  cudaStream_t aux[GF_WB_STREAMS] = {};
  cudaEvent_t evt[GF_WB_EVENTS] = {};
  ~Helpers() {
    for (auto& a : aux)
      if (a) cudaStreamDestroy(a);
    for (auto& e : evt)
      if (e) cudaEventDestroy(e);
  }
  bool create() {
    for (auto& a : aux)
      if (cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking) != cudaSuccess) return false;
    for (auto& e : evt)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return false;
    return true;
  }
};

// A one-structure batch around the wide band `wband` (n x (2w + 1)), the
// right-hand side / solution P and the scratch y, as the wide-band kernels
// read it.
struct WideBatch {
  Batch b{};
  StructInfo* dinf = nullptr;
  StructState* dst = nullptr;
  int* dws = nullptr;
  bool init(gf_ctx* ctx, DevBufs& mem, Helpers& hl, int n, int w, double* wband, double* P, double* y) {
    StructInfo inf{};
    inf.n_free = n;
    inf.wide = 1;
    inf.wkl = w;
    inf.n_panels = (n + GF_WB_NB - 1) / GF_WB_NB;
    StructState st0{};
    st0.phase = PH_ITER;
    st0.need_solve = 1;
    const int zero = 0;
    const int R = (w + 127) / 128 * 128;
    __nv_bfloat16* sl = nullptr;
    int* se = nullptr;
    unsigned long long* km = nullptr;
    int* err = nullptr;
    if (!mem.get(&dinf, 1) || !mem.get(&dst, 1) || !mem.get(&dws, 1) || !hl.create() ||
        !mem.get(&sl, (size_t)2 * 8 * R * GF_WB_NB) || !mem.get(&se, (size_t)2 * R) ||
        !mem.get(&km, (size_t)2 * 2 * GF_WB_NB) || !mem.get(&err, 1))
      return false;
    if (cudaMemsetAsync(km, 0, sizeof(unsigned long long) * 2 * 2 * GF_WB_NB, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(sl, 0, sizeof(__nv_bfloat16) * 2 * 8 * R * GF_WB_NB, ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(err, 0, sizeof(int), ctx->stream) != cudaSuccess)
      return false;
    cudaStream_t s = ctx->stream;
    if (cudaMemcpyAsync(dinf, &inf, sizeof(inf), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(dst, &st0, sizeof(st0), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(dws, &zero, sizeof(int), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return false;
    b.n_struct = 1;
    b.info = dinf;
    b.state = dst;
    b.P = P;
    b.y = y;
    ShellData& sd = b.sh;
    sd.n_wide = 1;
    sd.wide_structs = dws;
    sd.max_panels = inf.n_panels;
    sd.max_kl = w;
    sd.wband = wband;
    sd.wide_tc = ctx->wide_update;  // the context's choice (tcgen05 tensor cores by default)
    sd.oz_rows = R;
    sd.oz_slices = sl;
    sd.oz_exp = se;
    sd.oz_kmax = km;
    sd.oz_error = err;
    for (int k = 0; k < GF_WB_STREAMS; ++k) sd.aux[k] = hl.aux[k];
    for (int k = 0; k < GF_WB_EVENTS; ++k) sd.evt[k] = hl.evt[k];
    return true;
  }
  // Factor and solve on the context's stream; *fail = the pivot status.
  cudaError_t solve(gf_ctx* ctx, int* fail) {
    cudaStream_t s = ctx->stream;
    launch_wide_solve(b, s);
    StructState st0{};
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st0, dst, sizeof(st0), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    *fail = st0.info_fail;
    return e;
  }
};

}  // namespace gfh
