// Modal analysis on the GPU (reference src/Modal.cpp:131-199, Modal::Solve,
// with sparseeigen, src/SparseMatrix.cpp:270-420).  The reference mounts the
// modal mass M_AA (MountMassModal) and the tangent K_AA (MountLocal,
// MountElementLoads, MountLoads) at the step's configuration and asks ARPACK
// (arpack-ng's dnaupd / dneupd, mode 3: shift-invert with shift 0, 'LM')
// for the number_modes eigenvalues of K x = lambda M x nearest zero.
//
// Here both matrices are mounted on the device in the structure's own band
// (gf_iter.cu's static tangent; launch_modal_mass), K is factored once by
// the wide-band LU (gf_shell.cu), and the eigenpairs come from subspace
// iteration on the same shift-inverted operator K^-1 M (Bathe's method):
// a block of p = max(2 nev, nev + 8) vectors, X <- K^-1 M X, then
// Rayleigh-Ritz on the block (Kr = Y^T K Y = Y^T M X, Mr = Y^T M Y; the
// p x p generalized problem by Cholesky and cyclic Jacobi on the host),
// until the nev smallest Ritz values change by at most tol relative.  The
// Ritz values converge like (lambda_i / lambda_(p+1))^(2k).  The matrices
// of a Modal step at a configuration without follower loads are symmetric
// (K) and symmetric positive definite (M); a tangent that is not symmetric
// is refused.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/giraffe_gpu.h"
#include "gf_host_internal.h"
#include "gf_kernels.cuh"
#include "gf_types.h"
#include "gf_wide.h"

using namespace gf;
using namespace gfh;

namespace {

// y[:, q] = A x[:, q] for the nq columns (ld n) of x; A n x n in the band
// layout (kw + i - j) + j W.  One thread per row, the band row summed in
// column order.
__global__ void k_band_mv(int n, const double* A, int64_t W, int kw, const double* x, double* y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t q = blockIdx.y;
  const double* xq = x + q * n;
  const int j0 = max(0, i - kw), j1 = min(n - 1, i + kw);
  double acc = 0.0;
  for (int j = j0; j <= j1; ++j) acc = fma(A[(kw + i - j) + (int64_t)j * W], xq[j], acc);
  y[q * n + i] = acc;
}

// G[i + p j] = a[:, i] . b[:, j] (columns of length n): one CTA per entry,
// partial sums in a fixed order and a fixed tree.
__global__ void __launch_bounds__(256) k_gram(int n, int p, const double* a, const double* b, double* G) {
  const int i = blockIdx.x, j = blockIdx.y;
  __shared__ double red[256];
  double acc = 0.0;
  for (int k = threadIdx.x; k < n; k += 256) acc = fma(a[(int64_t)i * n + k], b[(int64_t)j * n + k], acc);
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) G[i + p * j] = red[0];
}

// x[:, j] = sum_i y[:, i] Z[i + p j]
__global__ void k_combine(int n, int p, const double* y, const double* Z, double* x) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int j = blockIdx.y;
  double acc = 0.0;
  for (int i = 0; i < p; ++i) acc = fma(y[(int64_t)i * n + k], Z[i + p * j], acc);
  x[(int64_t)j * n + k] = acc;
}

// Largest |A(i, j) - A(j, i)| and largest |A(i, j)| of a band, as FP64 bit
// patterns (non-negative doubles order like their bits): one thread per
// column.
__global__ void k_band_asym(int n, const double* A, int64_t W, int kw, unsigned long long* out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double da = 0.0, ma = fabs(A[kw + (int64_t)j * W]);
  for (int d = 1; d <= kw && j + d < n; ++d) {
    const double lo = A[(kw + d) + (int64_t)j * W];        // (j + d, j)
    const double up = A[(kw - d) + (int64_t)(j + d) * W];  // (j, j + d)
    da = fmax(da, fabs(lo - up));
    ma = fmax(ma, fmax(fabs(lo), fabs(up)));
  }
  atomicMax(out, (unsigned long long)__double_as_longlong(da));
  atomicMax(out + 1, (unsigned long long)__double_as_longlong(ma));
}

// Cholesky A = L L^T of a symmetric positive definite p x p matrix
// (column-major), L in the lower triangle; false if a pivot is not positive.
bool cholesky(std::vector<double>& A, int p) {
  for (int j = 0; j < p; ++j) {
    double d = A[j + p * j];
    for (int k = 0; k < j; ++k) d -= A[j + p * k] * A[j + p * k];
    if (!(d > 0.0)) return false;
    const double l = std::sqrt(d);
    A[j + p * j] = l;
    for (int i = j + 1; i < p; ++i) {
      double s = A[i + p * j];
      for (int k = 0; k < j; ++k) s -= A[i + p * k] * A[j + p * k];
      A[i + p * j] = s / l;
    }
    for (int i = 0; i < j; ++i) A[i + p * j] = 0.0;
  }
  return true;
}

// Cyclic Jacobi eigen-decomposition of a symmetric p x p matrix (rotations
// chosen by the Rutishauser formulas): A = V diag(w) V^T, w ascending.
void jacobi_eigen(std::vector<double> A, int p, std::vector<double>& w, std::vector<double>& V) {
  V.assign((size_t)p * p, 0.0);
  for (int i = 0; i < p; ++i) V[i + p * i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int j = 0; j < p; ++j)
      for (int i = 0; i < p; ++i) (i == j ? diag : off) += A[i + p * j] * A[i + p * j];
    if (off <= 1e-30 * diag) break;
    for (int q = 1; q < p; ++q)
      for (int r = 0; r < q; ++r) {
        const double arq = A[r + p * q];
        if (arq == 0.0) continue;
        const double theta = (A[q + p * q] - A[r + p * r]) / (2.0 * arq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < p; ++k) {  // columns r, q
          const double akr = A[k + p * r], akq = A[k + p * q];
          A[k + p * r] = c * akr - s * akq;
          A[k + p * q] = s * akr + c * akq;
        }
        for (int k = 0; k < p; ++k) {  // rows r, q
          const double ark = A[r + p * k], aqk = A[q + p * k];
          A[r + p * k] = c * ark - s * aqk;
          A[q + p * k] = s * ark + c * aqk;
        }
        for (int k = 0; k < p; ++k) {
          const double vkr = V[k + p * r], vkq = V[k + p * q];
          V[k + p * r] = c * vkr - s * vkq;
          V[k + p * q] = s * vkr + c * vkq;
        }
      }
  }
  std::vector<int> idx(p);
  for (int i = 0; i < p; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return A[a + p * a] < A[b + p * b]; });
  std::vector<double> Vs((size_t)p * p);
  w.resize(p);
  for (int k = 0; k < p; ++k) {
    w[k] = A[idx[k] + p * idx[k]];
    for (int i = 0; i < p; ++i) Vs[i + p * k] = V[i + p * idx[k]];
  }
  V.swap(Vs);
}

// The generalized p x p problem Kr z = theta Mr z (both symmetric, Mr
// positive definite): theta ascending, Z with Z^T Mr Z = I.
bool ritz(std::vector<double> Kr, std::vector<double> Mr, int p, std::vector<double>& theta, std::vector<double>& Z) {
  for (int j = 0; j < p; ++j)
    for (int i = 0; i < j; ++i) {
      const double k = 0.5 * (Kr[i + p * j] + Kr[j + p * i]), m = 0.5 * (Mr[i + p * j] + Mr[j + p * i]);
      Kr[i + p * j] = Kr[j + p * i] = k;
      Mr[i + p * j] = Mr[j + p * i] = m;
    }
  if (!cholesky(Mr, p)) return false;
  // C = L^-1 Kr L^-T: forward substitution on the columns, then the rows
  std::vector<double> C = Kr;
  for (int j = 0; j < p; ++j)
    for (int i = 0; i < p; ++i) {
      double s = C[i + p * j];
      for (int k = 0; k < i; ++k) s -= Mr[i + p * k] * C[k + p * j];
      C[i + p * j] = s / Mr[i + p * i];
    }
  for (int i = 0; i < p; ++i)
    for (int j = 0; j < p; ++j) {
      double s = C[i + p * j];
      for (int k = 0; k < j; ++k) s -= C[i + p * k] * Mr[j + p * k];
      C[i + p * j] = s / Mr[j + p * j];
    }
  std::vector<double> V;
  jacobi_eigen(C, p, theta, V);
  // Z = L^-T V
  Z = V;
  for (int j = 0; j < p; ++j)
    for (int i = p - 1; i >= 0; --i) {
      double s = Z[i + p * j];
      for (int k = i + 1; k < p; ++k) s -= Mr[k + p * i] * Z[k + p * j];
      Z[i + p * j] = s / Mr[i + p * i];
    }
  return true;
}

}  // namespace

int gf_structure_modal(gf_structure* S, double time, int n_modes, double tol, double* eig, double* modes,
                       int* iterations) {
  if (!S || n_modes <= 0 || !eig) return GF_ERR_ARG;
  gf_ctx* ctx = S->ctx;
  const int n = S->nf, kw = (int)S->kw;
  const int64_t W = S->W;
  if (n_modes > n) {
    set_err(ctx, "gf_structure_modal: %d modes asked of %d free DOFs", n_modes, n);
    return GF_ERR_ARG;
  }
  const int p = std::min(n, std::max(2 * n_modes, n_modes + 8));
  const double rtol = tol > 0.0 ? tol : 1e-12;
  cudaStream_t st = S->B->stream;
  // K_AA: the static tangent, in the structure's band
  int r = structure_static_tangent(S, time);
  if (r != GF_OK) return r;
  DevBufs mem;
  Helpers hl;
  double *Kc = nullptr, *Mb = nullptr, *X = nullptr, *Wm = nullptr, *Y = nullptr, *Ys = nullptr, *MY = nullptr,
         *G = nullptr, *Zd = nullptr;
  unsigned long long* asym = nullptr;
  const size_t band = (size_t)n * W, blk = (size_t)n * p;
  if (!mem.get(&Kc, band) || !mem.get(&Mb, band) || !mem.get(&X, blk) || !mem.get(&Wm, blk) || !mem.get(&Y, blk) ||
      !mem.get(&Ys, blk) || !mem.get(&MY, blk) || !mem.get(&G, (size_t)2 * p * p) || !mem.get(&Zd, (size_t)p * p) ||
      !mem.get(&asym, 2)) {
    set_err(ctx, "gf_structure_modal: device allocation failed");
    return GF_ERR_CUDA;
  }
  GF_CK(cudaMemcpyAsync(Kc, S->d_band, sizeof(double) * band, cudaMemcpyDeviceToDevice, st));
  // M_AA: the modal mass of every element, in the same band layout
  GF_CK(cudaMemsetAsync(Mb, 0, sizeof(double) * band, st));
  launch_modal_mass(S->B->b, Mb, W, kw, st);
  GF_CK(cudaMemsetAsync(asym, 0, 2 * sizeof(unsigned long long), st));
  k_band_asym<<<(n + 127) / 128, 128, 0, st>>>(n, Kc, W, kw, asym);
  unsigned long long ha[2];
  GF_CK(cudaMemcpyAsync(ha, asym, sizeof(ha), cudaMemcpyDeviceToHost, st));
  GF_CK(cudaStreamSynchronize(st));
  double da, ma;
  std::memcpy(&da, &ha[0], 8);
  std::memcpy(&ma, &ha[1], 8);
  if (da > 1e-9 * ma) {
    set_err(ctx, "gf_structure_modal: the tangent is not symmetric (relative asymmetry %.3g): the nonsymmetric "
                 "eigenproblem is not supported", da / ma);
    return GF_ERR_ARG;
  }
  // factor K once (the wide-band LU on a batch of one structure), with a
  // zero right-hand side
  WideBatch wb;
  if (!wb.init(ctx, mem, hl, n, kw, Kc, Ys, Y)) {
    set_err(ctx, "gf_structure_modal: device set-up failed");
    return GF_ERR_CUDA;
  }
  GF_CK(cudaMemsetAsync(Ys, 0, sizeof(double) * n, ctx->stream));
  GF_CK(cudaStreamSynchronize(st));
  int fail = 0;
  GF_CK(wb.solve(ctx, &fail));
  if (fail) {
    set_err(ctx, "gf_structure_modal: K_AA is singular (zero pivot in its factor)");
    return GF_ERR_SINGULAR;
  }
  Batch sb = wb.b;  // the substitution on the factor, p columns at once
  sb.P = Ys;
  sb.y = Y;
  sb.rhs_ld = n;
  // start block: a fixed pseudo-random sequence (64-bit LCG), the same on
  // every run
  std::vector<double> h((size_t)n * p);
  unsigned long long state = 0x9E3779B97F4A7C15ull;
  for (double& v : h) {
    state = state * 6364136223846793005ull + 1442695040888963407ull;
    v = (double)(state >> 11) * (1.0 / 9007199254740992.0) - 0.5;
  }
  GF_CK(cudaMemcpyAsync(X, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
  GF_CK(cudaStreamSynchronize(ctx->stream));
  std::vector<double> theta, prev, Z, Kr((size_t)p * p), Mr((size_t)p * p);
  const dim3 gmv((n + 127) / 128, p);
  int it = 0;
  bool conv = false;
  for (it = 1; it <= 300 && !conv; ++it) {
    cudaStream_t s = ctx->stream;
    k_band_mv<<<gmv, 128, 0, s>>>(n, Mb, W, kw, X, Wm);            // W = M X
    GF_CK(cudaMemcpyAsync(Ys, Wm, sizeof(double) * blk, cudaMemcpyDeviceToDevice, s));
    launch_wide_subst(sb, p, s);                                    // Y = K^-1 W (in Ys)
    k_band_mv<<<gmv, 128, 0, s>>>(n, Mb, W, kw, Ys, MY);           // M Y
    k_gram<<<dim3(p, p), 256, 0, s>>>(n, p, Ys, Wm, G);             // Kr = Y^T M X = Y^T K Y
    k_gram<<<dim3(p, p), 256, 0, s>>>(n, p, Ys, MY, G + p * p);     // Mr = Y^T M Y
    GF_CK(cudaGetLastError());
    GF_CK(cudaMemcpyAsync(Kr.data(), G, sizeof(double) * p * p, cudaMemcpyDeviceToHost, s));
    GF_CK(cudaMemcpyAsync(Mr.data(), G + p * p, sizeof(double) * p * p, cudaMemcpyDeviceToHost, s));
    GF_CK(cudaStreamSynchronize(s));
    if (!ritz(Kr, Mr, p, theta, Z)) {
      set_err(ctx, "gf_structure_modal: the projected mass is not positive definite (is M_AA singular?)");
      return GF_ERR_SINGULAR;
    }
    GF_CK(cudaMemcpyAsync(Zd, Z.data(), sizeof(double) * p * p, cudaMemcpyHostToDevice, s));
    k_combine<<<gmv, 128, 0, s>>>(n, p, Ys, Zd, X);                 // X = Y Z, M-orthonormal
    if (!prev.empty()) {
      double worst = 0.0;
      for (int k = 0; k < n_modes; ++k) worst = std::max(worst, std::fabs(theta[k] - prev[k]) / std::fabs(theta[k]));
      conv = worst <= rtol;
    }
    prev = theta;
  }
  GF_CK(cudaStreamSynchronize(ctx->stream));
  if (!conv) {
    set_err(ctx, "gf_structure_modal: no convergence to %.3g in 300 iterations", rtol);
    return GF_ERR_TIMEOUT;
  }
  for (int k = 0; k < n_modes; ++k) eig[k] = theta[k];
  if (iterations) *iterations = it - 1;
  if (modes) {
    GF_CK(cudaMemcpyAsync(h.data(), X, sizeof(double) * (size_t)n * n_modes, cudaMemcpyDeviceToHost, ctx->stream));
    GF_CK(cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < n_modes; ++k)
      for (int i = 0; i < n; ++i) modes[(size_t)k * n + i] = h[(size_t)k * n + (S->perm.empty() ? i : S->perm[i])];
  }
  return GF_OK;
}

int gf_modal(gf_ctx* ctx, const gf_model_desc* model, int n_modes, double tol, double* eig, double* modes,
             int* iterations) {
  if (!ctx || !model) return GF_ERR_ARG;
  gf_structure* S = gf_upload_structure(ctx, model, nullptr);
  if (!S) return GF_ERR_ARG;
  const int r = gf_structure_modal(S, model->solution.start_time, n_modes, tol, eig, modes, iterations);
  gf_structure_destroy(S);
  return r;
}
