// The wide-band LU of Shell_1 structures' K_AA and its triangular solves.
//
// Wide band: K_AA of a structure with free-DOF half-bandwidth kl is stored
// column-major with 2 kl + 1 rows.  No pivoting (the reference's tangent
// operators here are near-symmetric positive definite; a zero or non-finite
// pivot sets info_fail, which the step control treats like the reference's
// solver failure).  Right-looking blocked LU, GF_WB_NB columns per panel:
//   k_wb_diag    LU of the panel's diagonal block (one CTA per structure)
//   k_wb_trsm    L21 = A21 U11^-1 (row-parallel) and U12 = L11^-1 A12
//                (column-parallel), many CTAs
//   k_wb_update  A22 -= L21 U12, 64x64 tiles (the only dense contraction:
//                2 n kl^2 FP64 flops per factorization)
// and the solves k_wb_fwd (y = L^-1 b, b in P, y in y) and k_wb_bwd
// (x = U^-1 y into P), one launch per panel each.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cfloat>
#include <vector>

#include "gf_kernels.cuh"
#include "gf_math.cuh"
#include "gf_types.h"

namespace gf {

namespace {

__device__ __forceinline__ bool iterating_s(const StructState& s) { return s.phase == PH_ITER; }

// 1/p by two Newton-Raphson steps from the FP32 hardware approximation;
// exact division where the seed is out of FP32 range.
__device__ __forceinline__ double wb_recip(double p) {
  float pf = __double2float_rn(p);
  float af = fabsf(pf);
  if (!(af > 1e-30f && af < 1e30f)) return 1.0 / p;
  float rf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(pf));
  double r = (double)rf;
  double e = fma(-p, r, 1.0);
  r = fma(r, e, r);
  e = fma(-p, r, 1.0);
  return fma(r, e, r);
}

}  // namespace

// ---------------------------------------------------------------------------
// Wide-band LU.  Band pointer and geometry of wide structure w, in the
// factor's arithmetic type F (double: the FP64 LU in place of K_AA; float:
// the FP32 LU of the mixed-precision path, beside K_AA).
namespace {
template <typename F>
struct WBT {
  F* a;
  int n, kl;
  int64_t W;
  __device__ __forceinline__ F& at(int i, int j) const { return a[(kl + i - j) + (int64_t)j * W]; }
};
typedef WBT<double> WB;

// A structure whose K_AA this launch factors: iterating, asking for a
// solve, and in the FP64 fallback launches of the mixed path only those
// whose refinement did not finish.
__device__ __forceinline__ bool wide_active(const Batch& b, int s) {
  const StructState& st = b.state[s];
  return iterating_s(st) && st.need_solve && (!b.sh.fp64_pass || st.ir_fb);
}

__device__ __forceinline__ double* wb_base(const Batch& b, double*) { return b.sh.wband; }
__device__ __forceinline__ float* wb_base(const Batch& b, float*) { return b.sh.wband32; }

template <typename F = double>
__device__ __forceinline__ WBT<F> wb_of(const Batch& b, const StructInfo& inf) {
  WBT<F> w;
  w.a = wb_base(b, (F*)nullptr) + inf.wb_off;
  w.n = inf.n_free;
  w.kl = inf.wkl;
  w.W = 2 * (int64_t)inf.wkl + 1;
  return w;
}

// 1/p in the factor's type: FP64 by Newton steps from the FP32 seed, FP32
// correctly rounded.
__device__ __forceinline__ double wb_rcp(double p) { return wb_recip(p); }
__device__ __forceinline__ float wb_rcp(float p) { return __frcp_rn(p); }
// fused multiply-add in the factor's own type (no promotion of FP32 to FP64)
__device__ __forceinline__ double wfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float wfma(float a, float b, float c) { return fmaf(a, b, c); }

// Right-hand side and forward-substitution scratch of the solves in type F:
// the batch's P / y (FP64, column q of a multi-column solve at q rhs_ld), or
// the mixed path's FP32 r32 / y32.
__device__ __forceinline__ double* wb_rhs(const Batch& b, const StructInfo& inf, int q, double*) {
  return b.P + inf.dof_off + (int64_t)q * b.rhs_ld;
}
__device__ __forceinline__ double* wb_scratch(const Batch& b, const StructInfo& inf, int q, double*) {
  return b.y + inf.dof_off + (int64_t)q * b.rhs_ld;
}
__device__ __forceinline__ float* wb_rhs(const Batch& b, const StructInfo& inf, int, float*) {
  return b.sh.r32 + inf.dof_off;
}
__device__ __forceinline__ float* wb_scratch(const Batch& b, const StructInfo& inf, int, float*) {
  return b.sh.y32 + inf.dof_off;
}
constexpr int NB = GF_WB_NB;

// Panel index of a wide-band kernel: p >= 0 as given; inside a captured
// panel loop p = -1 - d, meaning the device counter plus d.
__device__ __forceinline__ int wb_panel(const Batch& b, int p) { return p >= 0 ? p : *b.sh.panel + (-1 - p); }
}  // namespace

// Column / row maxima of panel p's L21 and U12 for wide structure slot z
// (the tensor-core update balances k with them): [operand][k].
__device__ __forceinline__ unsigned long long* wb_kmax(const Batch& b, int z, int p) {
  return b.sh.oz_kmax + ((int64_t)z * 2 + (p & 1)) * 2 * NB;
}

// zero the wide band of iterating structures
__global__ void k_wb_zero(Batch b) {
  int s = b.sh.wide_structs[blockIdx.y];
  if (!iterating_s(b.state[s])) return;
  const StructInfo& inf = b.info[s];
  int64_t n = (int64_t)inf.n_free * (2 * (int64_t)inf.wkl + 1);
  double* a = b.sh.wband + inf.wb_off;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = 0.0;
}

// LU (no pivoting) of the diagonal block of panel p, in place, right-looking
// on a column-major copy in shared memory.  On this part an FP64 warp
// instruction occupies its sub-partition's FP64 unit for about 64 cycles
// and a dependent FP64 result takes as long, so the kernel is built around
// two costs: the FP64 issue of the trailing updates (about m^2 / 2 cycles per
// step for a trailing size m on one SM) and the dependent chain of each pivot
// (update the pivot, its reciprocal, the multipliers: about six FP64
// latencies).  The pivot warp (warp 8) owns column k + 1 at step k: it
// updates it, forms the next pivot's reciprocal and multipliers, while warps
// 0-7 update the other m (m - 1) entries of the trailing block packed
// densely over their lanes (entry e: column e / m, row e % m, so no lane
// idles until the last round), and one barrier closes the step.  Each entry
// sees the same operations in the same order as the textbook kij loop:
// multiplier l = a_ik * (1 / a_kk), then a_ij = fma(-l, a_kj, a_ij).
constexpr int DIAG_THREADS = 288;
template <typename F>
__global__ void __launch_bounds__(DIAG_THREADS) k_wb_diag(Batch b, int p) {
  p = wb_panel(b, p);
  if (p < 0) return;
  int s = b.sh.wide_structs[blockIdx.x];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WBT<F> w = wb_of<F>(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  __shared__ F Ac[NB][NB + 1];  // Ac[j][i] = A(i, j)
  __shared__ int fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) fail = 0;
  // this panel's L21 / U12 maxima start at zero (the buffer of its parity
  // was last read by the slicing of panel p - 2, which precedes this kernel)
  if (sizeof(F) == 8 && b.sh.wide_tc && tid < 2 * NB) wb_kmax(b, blockIdx.x, p)[tid] = 0ull;
  for (int x = tid; x < NB * NB; x += blockDim.x) {
    const int i = x % NB, j = x / NB;
    F v = F(0);
    if (i < nb && j < nb && abs(i - j) <= w.kl) v = w.at(j0 + i, j0 + j);
    Ac[j][i] = v;
  }
  __syncthreads();
  if (warp == 8 && nb > 0) {  // the multipliers of column 0
    const F piv = Ac[0][0];
    if (lane == 0 && (!(piv != 0.0) || !isfinite(piv))) fail = 1;
    const F r = wb_rcp(piv);
    if (1 + lane < nb) Ac[0][1 + lane] *= r;
    if (33 + lane < nb) Ac[0][33 + lane] *= r;
  }
  __syncthreads();
  for (int k = 0; k + 1 < nb; ++k) {
    const int m = nb - 1 - k;  // trailing rows and columns
    if (warp == 8) {
      // column k + 1: its update, then the next pivot and multipliers
      const int j = k + 1, i0 = j + lane, i1 = i0 + 32;
      const F u = Ac[j][k];
      if (i0 < nb) Ac[j][i0] = wfma(-Ac[k][i0], u, Ac[j][i0]);
      if (i1 < nb) Ac[j][i1] = wfma(-Ac[k][i1], u, Ac[j][i1]);
      __syncwarp();
      const F piv = Ac[j][j];
      if (lane == 0 && (!(piv != 0.0) || !isfinite(piv))) fail = 1;
      const F r = wb_rcp(piv);
      if (i0 > j && i0 < nb) Ac[j][i0] *= r;
      if (i1 < nb) Ac[j][i1] *= r;
    } else {
      // columns k + 2 .. nb - 1, m (m - 1) entries over 256 lanes
      const int tot = m * (m - 1);
      const float inv_m = 1.0f / (float)m;
      for (int e = tid; e < tot; e += 256) {
        const int jj = __float2int_rz(((float)e + 0.5f) * inv_m);  // e / m, exact for e < 4096
        const int ii = e - jj * m;
        const int i = k + 1 + ii, j = k + 2 + jj;
        Ac[j][i] = wfma(-Ac[k][i], Ac[j][k], Ac[j][i]);
      }
    }
    __syncthreads();
  }
  for (int x = tid; x < nb * nb; x += blockDim.x) {
    const int i = x % nb, j = x / nb;
    if (abs(i - j) <= w.kl) w.at(j0 + i, j0 + j) = Ac[j][i];
  }
  // a zero or non-finite pivot: the FP64 LU's solver failure; the FP32 LU
  // of the mixed path hands the solve to the FP64 fallback instead
  if (tid == 0 && fail) {
    if (sizeof(F) == 8) b.state[s].info_fail = 1;
    else b.state[s].ir_fb = 1;
  }
}

// L21 = A21 U11^-1 (row blocks) and U12 = L11^-1 A12 (column blocks) of
// panel p.  RB rows (or columns) per CTA, a warp each splitting the panel
// width; lane 0 forms each multiplier once and the warp reads it from shared
// memory (the FP64 pipe is scarce).  The launch covers rows (columns)
// row0 .. row0 + nblk RB - 1 below (right of) the panel's diagonal block:
// blockIdx.x < nblk an L21 row block, else a U12 column block.  The first
// NB rows and columns (the next panel's diagonal block, on the lookahead's
// critical path) are a launch of their own with two rows per CTA, spread
// over 64 SMs; the bulk runs beside it with eight.  Each CTA loads the half
// of the diagonal block its side reads (U11 for L21, L11 for U12).
template <typename F, int RB>
__global__ void __launch_bounds__(32 * RB) k_wb_trsm(Batch b, int p, int row0, int nblk) {
  p = wb_panel(b, p);
  if (p < 0) return;
  int s = b.sh.wide_structs[blockIdx.y];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WBT<F> w = wb_of<F>(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  const int m = min(w.kl, w.n - j0 - nb);  // rows below / columns right of the panel
  if (m <= 0) return;
  const bool lower = (int)blockIdx.x < nblk;
  const int rowb = row0 + RB * (lower ? (int)blockIdx.x : (int)blockIdx.x - nblk);
  if (rowb >= m) return;
  __shared__ F T[NB][NB + 1];  // the diagonal block's LU (the half this side reads)
  __shared__ F X[RB][NB + 1];
  __shared__ F rd[NB];         // reciprocals of U11's diagonal
  const int tid = threadIdx.x;
  for (int x = tid; x < NB * NB; x += blockDim.x) {
    int i = x % NB, j = x / NB;
    T[i][j] = ((lower ? i <= j : i > j) && i < nb && j < nb && abs(i - j) <= w.kl) ? w.at(j0 + i, j0 + j) : F(0);
  }
  if (lower)
    for (int k = tid; k < nb; k += blockDim.x) rd[k] = wb_rcp(w.at(j0 + k, j0 + k));
  const int r = tid >> 5, c = tid & 31;  // row (or column) r of the block, lane c
  const int g = j0 + nb + rowb + r;      // global row (lower) or column (upper)
  const bool live = g < j0 + nb + m;
  for (int k = c; k < NB; k += 32) {
    F v = F(0);
    if (live && k < nb) {
      if (lower) { if (g - (j0 + k) <= w.kl) v = w.at(g, j0 + k); }
      else { if (g - (j0 + k) <= w.kl) v = w.at(j0 + k, g); }
    }
    X[r][k] = v;
  }
  __syncthreads();
  // the row in registers, lane c holding entries c and c + 32: each step
  // broadcasts the finished entry k by shuffle (a dependent FP64 result
  // takes about 64 cycles on this part, a shuffle far less), and the half
  // with no live entry left (k >= 31 for the first) is skipped by a
  // warp-uniform branch instead of issued masked
  F v0 = X[r][c], v1 = X[r][c + 32];
  if (lower) {
    // x U11 = a: x_k = a_k / u_kk, then a_j -= x_k u_kj (j > k)
    for (int k = 0; k < nb; ++k) {
      const F xk = __shfl_sync(0xffffffffu, k < 32 ? v0 : v1, k & 31) * rd[k];
      if (k < 32) {
        if (c == k) v0 = xk;
      } else if (c == k - 32) {
        v1 = xk;
      }
      if (k < 31 && c > k) v0 -= xk * T[k][c];
      if (c + 32 > k && c + 32 < nb) v1 -= xk * T[k][c + 32];
    }
  } else {
    // L11 y = a (unit lower): y_k = a_k, then a_i -= l_ik y_k (i > k)
    for (int k = 0; k < nb; ++k) {
      const F yk = __shfl_sync(0xffffffffu, k < 32 ? v0 : v1, k & 31);
      if (k < 31 && c > k) v0 -= T[c][k] * yk;
      if (c + 32 > k && c + 32 < nb) v1 -= T[c + 32][k] * yk;
    }
  }
  X[r][c] = v0;
  X[r][c + 32] = v1;
  __syncthreads();
  for (int k = c; k < nb; k += 32) {
    if (!live || g - (j0 + k) > w.kl) continue;
    if (lower) w.at(g, j0 + k) = X[r][k];
    else w.at(j0 + k, g) = X[r][k];
  }
  if (sizeof(F) == 8 && b.sh.wide_tc)
  for (int k = tid; k < nb; k += blockDim.x) {
    // largest magnitude of column k of this block's L21 rows (row k of its
    // U12 columns), as FP64 bits, which order like the magnitudes; the
    // maximum over the CTAs is exact and independent of their order
    unsigned long long mx = 0;
    for (int q = 0; q < RB; ++q) {
      const int gq = j0 + nb + rowb + q;
      if (gq < j0 + nb + m && gq - (j0 + k) <= w.kl)
        mx = max(mx, (unsigned long long)__double_as_longlong((double)X[q][k]) & 0x7FFFFFFFFFFFFFFFull);
    }
    if (mx) atomicMax(wb_kmax(b, blockIdx.y, p) + (lower ? 0 : NB) + k, mx);
  }
}

// A22 -= L21 U12 over the (m x m) trailing window of panel p, 32x32 tiles
// (small tiles keep the FP64 work even across the SMs), each of 256
// threads a 2x2 block of outputs.
constexpr int UT = 32;
// part: 0 every tile, 1 only the tiles of the next panel's diagonal block
// (the first NB rows and columns of the window), 2 every other tile.
__global__ void __launch_bounds__(256) k_wb_update(Batch b, int p, int part) {
  p = wb_panel(b, p);
  if (p < 0) return;
  int s = b.sh.wide_structs[blockIdx.z];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WB w = wb_of(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  const int m = min(w.kl, w.n - j0 - nb);
  if (m <= 0) return;
  const int r0 = blockIdx.x * UT, c0 = blockIdx.y * UT;
  if (r0 >= m || c0 >= m) return;
  const bool corner = r0 < NB && c0 < NB;
  if ((part == 1 && !corner) || (part == 2 && corner)) return;
  __shared__ double Ls[NB][UT + 1];  // [k][row]
  __shared__ double Us[NB][UT + 1];  // [k][col]
  const int tid = threadIdx.x;
  const int base = j0 + nb;
  for (int x = tid; x < NB * UT; x += blockDim.x) {
    int i = x % UT, k = x / UT;
    int gk = j0 + k;
    int gi = base + r0 + i;
    Ls[k][i] = (k < nb && r0 + i < m && gi - gk <= w.kl) ? w.at(gi, gk) : 0.0;
    int gj = base + c0 + i;
    Us[k][i] = (k < nb && c0 + i < m && gj - gk <= w.kl) ? w.at(gk, gj) : 0.0;
  }
  __syncthreads();
  const int ty = tid >> 4, tx = tid & 15;
  double a00 = 0.0, a01 = 0.0, a10 = 0.0, a11 = 0.0;
#pragma unroll 8
  for (int k = 0; k < NB; ++k) {
    double l0 = Ls[k][ty], l1 = Ls[k][ty + 16], u0 = Us[k][tx], u1 = Us[k][tx + 16];
    a00 = fma(l0, u0, a00);
    a01 = fma(l0, u1, a01);
    a10 = fma(l1, u0, a10);
    a11 = fma(l1, u1, a11);
  }
  const int ri0 = r0 + ty, ri1 = r0 + ty + 16, cj0 = c0 + tx, cj1 = c0 + tx + 16;
  if (ri0 < m && cj0 < m) w.at(base + ri0, base + cj0) -= a00;
  if (ri0 < m && cj1 < m) w.at(base + ri0, base + cj1) -= a01;
  if (ri1 < m && cj0 < m) w.at(base + ri1, base + cj0) -= a10;
  if (ri1 < m && cj1 < m) w.at(base + ri1, base + cj1) -= a11;
}

// The corner of panel p's trailing update: the next panel's diagonal block
// (the first NB rows and columns of the window), on the lookahead's critical
// path.  CT x CT output tiles (8 x 8 by default: 64 CTAs); in a CTA four
// thread groups each sum a quarter of k (16 terms) for every output of the
// tile, and the quarters are added in a fixed order: an FP64 warp instruction holds its
// sub-partition's FP64 unit for about 64 cycles, so four warps on four
// sub-partitions finish the 64 terms four times sooner than one.
template <int CT>
__global__ void __launch_bounds__(4 * CT * CT) k_wb_corner(Batch b, int p) {
  p = wb_panel(b, p);
  if (p < 0) return;
  int s = b.sh.wide_structs[blockIdx.z];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WB w = wb_of(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  const int m = min(min(w.kl, w.n - j0 - nb), NB);
  const int r0 = blockIdx.x * CT, c0 = blockIdx.y * CT;
  if (r0 >= m || c0 >= m) return;
  __shared__ double Ls[NB][CT + 1];  // [k][row]
  __shared__ double Us[NB][CT + 1];  // [k][col]
  __shared__ double part[4][CT * CT];
  const int tid = threadIdx.x;
  const int base = j0 + nb;
  for (int x = tid; x < NB * CT; x += blockDim.x) {
    // rows of L21 along a band column are contiguous; U12's k along a
    // band column too
    const int i = x % CT, k = x / CT;
    const int gk = j0 + k, gi = base + r0 + i;
    Ls[k][i] = (k < nb && r0 + i < m && gi - gk <= w.kl) ? w.at(gi, gk) : 0.0;
    const int kk = x % NB, c = x / NB, gj = base + c0 + c;
    Us[kk][c] = (kk < nb && c0 + c < m && gj - (j0 + kk) <= w.kl) ? w.at(j0 + kk, gj) : 0.0;
  }
  __syncthreads();
  const int o = tid % (CT * CT), q = tid / (CT * CT);  // output, quarter of k
  const int ty = o / CT, tx = o % CT;
  double a = 0.0;
#pragma unroll
  for (int k = 16 * q; k < 16 * q + 16; ++k) a = fma(Ls[k][ty], Us[k][tx], a);
  part[q][o] = a;
  __syncthreads();
  if (q == 0 && r0 + ty < m && c0 + tx < m)
    w.at(base + r0 + ty, base + c0 + tx) -= (part[0][o] + part[1][o]) + (part[2][o] + part[3][o]);
}

// ---- the same trailing update on the tensor cores (Ozaki scheme) ----
// A22 -= L21 U12 for one 64x64 output tile with K = NB = 64, the FP64
// products emulated by bf16 tensor-core products of exact slices.  First
// every k of the panel is balanced: column k of L21 times 2^-f_k and row k
// of U12 times 2^f_k (exact, the products unchanged), f_k half the exponent
// difference of their largest entries.  Then each
// row of L21 (column of U12) gets the power of two 2^e just above its
// largest magnitude; an entry x becomes the 56-bit integer
// X = floor(|x| 2^(56 - e)), read off the FP64 bits with integer
// operations, cut into OZ_S = 8 slices of 7 bits, v_q = bits 49-7q .. 55-7q
// of X with the sign of x: x = 2^e sum_q v_q 2^-7(q+1) + r, |r| < 2^(e-56),
// every |v_q| <= 127 exact in bf16.  The slice products with q + t = d all
// weigh 2^-7(d+2); summed over k and over the d + 1 pairs they form an
// integer of magnitude below 8 * 64 * 127^2 < 2^23, which the FP32
// accumulators of mma.sync hold exactly.  The diagonals are combined
// exactly as two 64-bit integers (Horner in powers of 2^7: d = 0..4 and
// d = 5..7), joined by one FMA and scaled by the row and column powers of
// two.  What is left out (pairs with q + t > 7, the remainders r) is
// below about 2^-52 K max_k |L~_ik| max_k |U~_kj| for the balanced L~, U~:
// the FP64 rounding of the product when the terms of a row and a column
// are of like size, larger when a row holds entries far apart in
// magnitude that the balancing cannot bring together.  All
// slicing is integer work, so the FP64 pipe, the scarce one on this part,
// only sees a handful of operations per output entry.
constexpr int OZ_S = 8;    // slices per operand
constexpr int OZ_T = 64;   // slicing block (rows of L21, columns of U12); output tile columns
constexpr int OZ_TR = 32;  // output tile rows: two CTAs fit on an SM
constexpr int OZ_LD = 72;  // bf16 row stride of the slice tiles: 144 B, so the 8 rows of an ldmatrix hit distinct banks
constexpr int OZ_THREADS = 256;
constexpr size_t OZ_SMEM = sizeof(__nv_bfloat16) * OZ_S * (OZ_TR + OZ_T) * OZ_LD + sizeof(int) * (OZ_TR + OZ_T);

__device__ __forceinline__ void oz_ldmatrix_x4(unsigned (&r)[4], const __nv_bfloat16* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

__device__ __forceinline__ void oz_mma(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Magnitude bits of x (monotonic in |x| for finite values).
__device__ __forceinline__ unsigned long long oz_mag(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}

// Scale exponent from the largest magnitude's bits: e with max|x| < 2^e
// (biased: the FP64 exponent field of the maximum plus one); 0 for zero.
__device__ __forceinline__ int oz_exponent(unsigned long long mag) { return mag ? (int)(mag >> 52) + 1 : 0; }

// The slices of x under the biased row exponent eb, written to
// dst[q * stride] for q = 0..OZ_S-1.  Subnormal entries count as zero.
__device__ __forceinline__ void oz_split(double x, int eb, __nv_bfloat16* dst, int stride) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const int E2 = (int)((u >> 52) & 0x7FF);
  unsigned long long X = 0;
  if (E2 != 0) {
    const unsigned long long mant = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = E2 - eb + 4;  // X = floor(|x| 2^(56 - e)); sh <= 3
    X = sh >= 0 ? mant << sh : (sh > -64 ? mant >> (-sh) : 0ull);
  }
  const bool neg = (u >> 63) != 0;
#pragma unroll
  for (int q = 0; q < OZ_S; ++q) {
    const int v = (int)((X >> (49 - 7 * q)) & 127ull);
    dst[q * stride] = __float2bfloat16_rn((float)(neg ? -v : v));
  }
}

// Slice buffers of wide structure slot z (a panel's L21 rows and U12
// columns, each as OZ_S slices of 64 bf16 per row or column, and their
// biased scale exponents).
struct OzSlices {
  __nv_bfloat16 *L, *U;  // [slice][row or column][k]
  int *eL, *eU;
};
__device__ __forceinline__ OzSlices oz_slices(const Batch& b, int z) {
  const int64_t R = b.sh.oz_rows;
  OzSlices o;
  o.L = b.sh.oz_slices + (int64_t)z * 2 * OZ_S * R * NB;
  o.U = o.L + OZ_S * R * NB;
  o.eL = b.sh.oz_exp + (int64_t)z * 2 * R;
  o.eU = o.eL + R;
  return o;
}

// Slices of panel p's L21 (blockIdx.y = 0: SL_ROWS rows) or U12
// (blockIdx.y = 1: SL_ROWS columns) into the structure's slice buffers: the
// FP64 block through shared memory (consecutive threads walk a band column:
// down the rows of L21, along k for U12), the scale exponent of every row or
// column, then its OZ_S slices.  Rows or columns beyond the trailing window
// are zero.  Small blocks spread the panel over about a hundred CTAs: the
// work is a few loads and integer operations per entry, bound by latency.
constexpr int SL_ROWS = 16;
__global__ void __launch_bounds__(256) k_wb_slice(Batch b, int p) {
  p = wb_panel(b, p);
  if (p < 0) return;
  const int s = b.sh.wide_structs[blockIdx.z];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WB w = wb_of(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  const int m = min(w.kl, w.n - j0 - nb);
  if (m <= 0) return;
  const int r0 = blockIdx.x * SL_ROWS;
  if (r0 >= m) return;
  const bool lower = blockIdx.y == 0;
  __shared__ double F[SL_ROWS][NB + 1];  // [row or column][k]
  __shared__ int e[SL_ROWS];
  __shared__ double bal[NB];  // 2^-f_k for L21 columns, 2^f_k for U12 rows
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int base = j0 + nb;
  if (tid < NB) {
    // balance k: column k of L21 scaled by 2^-f_k and row k of U12 by 2^f_k
    // leaves every product L_ik U_kj as it is (powers of two, exact) and
    // brings the two maxima within a factor 2 of each other, so the
    // per-row (per-column) slicing exponents below do not depend on how
    // the DOFs of the panel are scaled
    const unsigned long long* km = wb_kmax(b, blockIdx.z, p);
    const unsigned long long ml = km[tid], mu = km[NB + tid];
    int f = 0;
    if (ml && mu) f = ((int)(ml >> 52) - (int)(mu >> 52)) >> 1;  // floor of half the exponent difference
    f = max(-1000, min(1000, f));
    bal[tid] = ldexp(1.0, lower ? -f : f);
  }
  __syncthreads();
  for (int x = tid; x < SL_ROWS * NB; x += blockDim.x) {
    const int i = lower ? x % SL_ROWS : x / NB, k = lower ? x / SL_ROWS : x % NB;
    const int gk = j0 + k, g = base + r0 + i;
    const bool live = k < nb && r0 + i < m && g - gk <= w.kl;
    F[i][k] = live ? (lower ? w.at(g, gk) : w.at(gk, g)) * bal[k] : 0.0;
  }
  __syncthreads();
  for (int i = warp; i < SL_ROWS; i += 8) {
    unsigned long long mx = max(oz_mag(F[i][lane]), oz_mag(F[i][lane + 32]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) e[i] = oz_exponent(mx);
  }
  __syncthreads();
  OzSlices o = oz_slices(b, blockIdx.z);
  __nv_bfloat16* dst = lower ? o.L : o.U;
  const int64_t R = b.sh.oz_rows;
  for (int x = tid; x < SL_ROWS * NB; x += blockDim.x) {
    const int i = x / NB, k = x % NB;
    // the 128-byte swizzle: 16-byte chunk k / 8 of row r stored at chunk
    // (k / 8) ^ (r & 7)
    const int r = r0 + i, ks = (((k >> 3) ^ (r & 7)) << 3) | (k & 7);
    oz_split(F[i][k], e[i], dst + (int64_t)r * NB + ks, (int)(R * NB));
  }
  if (tid < SL_ROWS) (lower ? o.eL : o.eU)[r0 + tid] = e[tid];
}

__device__ __forceinline__ void oz_cp16(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src));
}
__device__ __forceinline__ void oz_commit() { asm volatile("cp.async.commit_group;\n" ::); }
// Waits until at most `pending` of this thread's copy groups are in flight.
__device__ __forceinline__ void oz_wait(int pending) {
  switch (pending) {
    case 0: asm volatile("cp.async.wait_group 0;\n" ::); break;
    case 1: asm volatile("cp.async.wait_group 1;\n" ::); break;
    case 2: asm volatile("cp.async.wait_group 2;\n" ::); break;
    case 3: asm volatile("cp.async.wait_group 3;\n" ::); break;
    case 4: asm volatile("cp.async.wait_group 4;\n" ::); break;
    case 5: asm volatile("cp.async.wait_group 5;\n" ::); break;
    case 6: asm volatile("cp.async.wait_group 6;\n" ::); break;
    default: asm volatile("cp.async.wait_group 7;\n" ::); break;
  }
}

__global__ void __launch_bounds__(OZ_THREADS) k_wb_update_tc(Batch b, int p, int part) {
  p = wb_panel(b, p);
  if (p < 0) return;
  const int s = b.sh.wide_structs[blockIdx.z];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WB w = wb_of(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  const int m = min(w.kl, w.n - j0 - nb);
  if (m <= 0) return;
  const int r0 = blockIdx.x * OZ_TR, c0 = blockIdx.y * OZ_T;
  if (r0 >= m || c0 >= m) return;
  const bool corner = r0 < NB && c0 < NB;
  if ((part == 1 && !corner) || (part == 2 && corner)) return;
  extern __shared__ __align__(16) unsigned char oz_raw[];
  __nv_bfloat16* Ls = reinterpret_cast<__nv_bfloat16*>(oz_raw);  // [slice][row][k]
  __nv_bfloat16* Us = Ls + OZ_S * OZ_TR * OZ_LD;                  // [slice][col][k]
  int* eL = reinterpret_cast<int*>(Us + OZ_S * OZ_T * OZ_LD);
  int* eU = eL + OZ_TR;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int base = j0 + nb;
  // 1-3. the slices of this tile's rows and columns, one copy group per
  // slice index, so that the products of the first diagonals start while
  // the later slices are still on their way
  {
    const OzSlices o = oz_slices(b, blockIdx.z);
    const int64_t R = b.sh.oz_rows;
    for (int q = 0; q < OZ_S; ++q) {
      // 32 rows of L21 and 64 columns of U12, 8 chunks of 16 bytes each
      for (int x = tid; x < (OZ_TR + OZ_T) * 8; x += OZ_THREADS) {
        const int op = x >= OZ_TR * 8, y = x - op * OZ_TR * 8, i = y >> 3, c = y & 7;
        // chunk c of a row sits at chunk c ^ (row & 7) in global memory (r0
        // and c0 are multiples of 8)
        const __nv_bfloat16* src = (op ? o.U + (int64_t)q * R * NB + (int64_t)(c0 + i) * NB
                                       : o.L + (int64_t)q * R * NB + (int64_t)(r0 + i) * NB) + 8 * (c ^ (i & 7));
        __nv_bfloat16* dst = (op ? Us + q * OZ_T * OZ_LD : Ls + q * OZ_TR * OZ_LD) + i * OZ_LD + 8 * c;
        oz_cp16(dst, src);
      }
      oz_commit();
    }
    if (tid < OZ_TR) eL[tid] = o.eL[r0 + tid];
    if (tid < OZ_T) eU[tid] = o.eU[c0 + tid];
  }
  // 4. slice products on the tensor cores: warp (wm, wn) owns rows
  // 16 wm .. +15 and columns 16 wn .. +15 as 1 x 2 tiles of 16 x 8; the
  // fragments of the next 16-wide k step load while this one multiplies
  const int wm = warp >> 2, wn = warp & 3;
  long long hi[2][4];  // diagonals 0..4: sum_d c_d 2^(7 (4 - d)), exact (< 2^52)
  long long lo[2][4];  // diagonals 5..7: c_5 2^14 + c_6 2^7 + c_7, exact (< 2^38)
#pragma unroll
  for (int c = 0; c < 2; ++c)
#pragma unroll
    for (int q = 0; q < 4; ++q) hi[c][q] = lo[c][q] = 0;
  // ldmatrix row addresses of this lane: A (rows x k) and B (stored as
  // columns x k)
  const int a_row = wm * 16 + (lane & 7) + ((lane >> 3) & 1) * 8, a_col = (lane >> 4) * 8;
  const int b_row = wn * 16 + (lane & 7) + (lane >> 4) * 8, b_col = ((lane >> 3) & 1) * 8;
#pragma unroll 1
  for (int d = 0; d < OZ_S; ++d) {
    oz_wait(OZ_S - 1 - d);  // slices 0..d of both operands are in
    __syncthreads();
    float c32[2][4];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
      for (int q = 0; q < 4; ++q) c32[c][q] = 0.0f;
#pragma unroll 1
    for (int sa = 0; sa <= d; ++sa) {
      const __nv_bfloat16* As = Ls + sa * OZ_TR * OZ_LD + a_row * OZ_LD + a_col;
      const __nv_bfloat16* Bs = Us + (d - sa) * OZ_T * OZ_LD + b_row * OZ_LD + b_col;
      unsigned af[2][4], bf[2][4];  // [buffer][reg]
      oz_ldmatrix_x4(af[0], As);
      oz_ldmatrix_x4(bf[0], Bs);
#pragma unroll
      for (int ks = 0; ks < NB / 16; ++ks) {
        const int cur = ks & 1, nxt = cur ^ 1;
        if (ks + 1 < NB / 16) {
          oz_ldmatrix_x4(af[nxt], As + 16 * (ks + 1));
          oz_ldmatrix_x4(bf[nxt], Bs + 16 * (ks + 1));
        }
#pragma unroll
        for (int c = 0; c < 2; ++c) oz_mma(c32[c], af[cur], bf[cur][2 * c], bf[cur][2 * c + 1]);
      }
    }
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const long long v = __float2int_rn(c32[c][q]);  // |c| < 2^23: an exact 32-bit integer
        if (d <= 4) hi[c][q] = hi[c][q] * 128 + v;
        else lo[c][q] = lo[c][q] * 128 + v;
      }
  }
  // 5. A22 -= the product, in units of 2^(e_i + e_j - 63): hi 2^21 + lo
  // (accumulator entry q of tile c: row lane / 4 (+ 8 for q >= 2), column
  // 2 (lane % 4) + q % 2)
#pragma unroll
  for (int c = 0; c < 2; ++c)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = wm * 16 + (lane >> 2) + (q >= 2 ? 8 : 0);
      const int j = wn * 16 + 8 * c + 2 * (lane & 3) + (q & 1);
      if (r0 + i < m && c0 + j < m) {
        const double v = fma((double)hi[c][q], 0x1p21, (double)lo[c][q]);
        // eL, eU are biased exponents (1023 + e); the scale 2^(e_i + e_j - 63)
        const int k = eL[i] + eU[j] - 2046 - 63;
        const double scale =
            (k >= -1022 && k <= 1023) ? __longlong_as_double((long long)(k + 1023) << 52) : ldexp(1.0, k);
        w.at(base + r0 + i, base + c0 + j) -= v * scale;
      }
    }
}

// ---- the same trailing update on the 5th-generation tensor cores ----
// One CTA per 128 x 64 output tile.  The eight diagonals of slice products
// accumulate in tensor memory (8 x 64 FP32 columns: the whole 512 columns
// of the SM), issued by one thread as tcgen05.mma (M 128, N 64, K 16, bf16
// in, FP32 out) on shared-memory operands in the 128-byte swizzled K-major
// layout; the slices arrive by bulk copies (the TMA engine) completing on
// mbarriers: the tile's eight U12 slices (64 KB) at once, its L21 slices
// (16 KB each) through three stages, so slice q + 2 loads while the products
// of slice q run.  Accumulator d (q + t = d) gets (d + 1) products of K = 64,
// an exact integer below 2^23, as in the mma.sync version.  While the
// products run, sixteen warps load the tile's A22 into registers (warp w
// owns rows 32 (w % 4) .. + 31, the TMEM lanes it may read, a row per lane,
// and columns 16 (w / 4) .. + 15); then they read tensor memory, join the
// diagonals exactly in 64-bit integers, convert once, scale by the row and
// column powers of two through the exponent bits and write A22 back (column
// by column, so a warp writes 32 consecutive doubles).  Every wait is bounded; a wait that gives up marks the
// structure's solve failed and sets the batch's error word, and the CTA
// still waits (bounded) for its copies and products before it frees tensor
// memory.
constexpr int T5_M = 128;
constexpr int T5_N = 64;
constexpr int T5_STAGES = 3;
constexpr int T5_THREADS = 512;
constexpr int T5_COLS_PER_WARP = T5_N / (T5_THREADS / 128);  // 16
constexpr uint32_t T5_A_BYTES = T5_M * NB * 2;  // one L21 slice of a tile
constexpr uint32_t T5_B_BYTES = T5_N * NB * 2;  // one U12 slice of a tile
constexpr uint32_t T5_TMEM_COLS = OZ_S * T5_N;  // 512
constexpr size_t T5_SMEM = 1024 + OZ_S * T5_B_BYTES + T5_STAGES * T5_A_BYTES + 128 + T5_N * sizeof(int);
// instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B bf16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28
constexpr uint32_t T5_IDESC =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(T5_N >> 3) << 17) | ((uint32_t)(T5_M >> 4) << 24);
constexpr long long T5_WAIT_CYCLES = 2000000000ll;  // about a second at the SM clock

__device__ __forceinline__ uint32_t t5_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// groups 1024 bytes apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t t5_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void t5_mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void t5_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool t5_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the phase of parity `parity` to complete, for about a second at
// most; false if it did not.
__device__ __forceinline__ bool t5_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!t5_try_wait(bar, parity))
    if (clock64() - t0 > T5_WAIT_CYCLES) return false;
  return true;
}
__device__ __forceinline__ void t5_bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void t5_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(T5_IDESC), "r"(accumulate));
}
__device__ __forceinline__ void t5_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void t5_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void t5_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// Eight consecutive FP32 columns of this warp's 32 TMEM lanes (a lane each).
__device__ __forceinline__ void t5_ld8(uint32_t taddr, uint32_t (&v)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(taddr));
}
__device__ __forceinline__ void t5_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

__global__ void __launch_bounds__(T5_THREADS, 1) k_wb_update_t5(Batch b, int p, int part) {
  p = wb_panel(b, p);
  if (p < 0) return;
  const int s = b.sh.wide_structs[blockIdx.z];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WB w = wb_of(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  const int m = min(w.kl, w.n - j0 - nb);
  if (m <= 0) return;
  const int r0 = blockIdx.x * T5_M, c0 = blockIdx.y * T5_N;
  if (r0 >= m || c0 >= m) return;
  extern __shared__ __align__(16) unsigned char t5_raw[];
  unsigned char* base = t5_raw + ((1024u - (t5_smem(t5_raw) & 1023u)) & 1023u);
  unsigned char* Bs = base;                              // [slice][64 columns][128 B]
  unsigned char* As = Bs + OZ_S * T5_B_BYTES;            // [stage][128 rows][128 B]
  uint64_t* bars = reinterpret_cast<uint64_t*>(As + T5_STAGES * T5_A_BYTES);  // fullB, fullA[3], emptyA[3], done
  uint32_t* holder = reinterpret_cast<uint32_t*>(bars + 8);
  int* okflag = reinterpret_cast<int*>(holder + 1);
  int* eU = reinterpret_cast<int*>(bars + 16);
  const int tid = threadIdx.x, warp = tid >> 5;
  const OzSlices o = oz_slices(b, blockIdx.z);
  const int64_t R = b.sh.oz_rows;
  const uint32_t bar0 = t5_smem(bars);
  const uint32_t fullB = bar0, fullA = bar0 + 8, emptyA = bar0 + 32, done = bar0 + 56;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(t5_smem(holder)),
                 "r"(T5_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  if (tid == 0) {
    for (int i = 0; i < 8; ++i) t5_mbar_init(bar0 + 8 * i, 1);
    *okflag = 1;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (tid < T5_N) eU[tid] = o.eU[c0 + tid];
  const int lg = warp & 3, cq = warp >> 2;      // TMEM lane group, column group
  const int row = 32 * lg + (tid & 31);         // this thread's row of the tile
  const int eLr = o.eL[r0 + row];               // r0 + 127 < oz_rows
  t5_fence_before();
  __syncthreads();
  t5_fence_after();
  const uint32_t tmem = *holder;
  if (tid == 0) {
    // issue the loads, then the products slice by slice
    const uint32_t sA = t5_smem(As), sB = t5_smem(Bs);
    const unsigned char* gU = reinterpret_cast<const unsigned char*>(o.U + (int64_t)c0 * NB);
    const unsigned char* gL = reinterpret_cast<const unsigned char*>(o.L + (int64_t)r0 * NB);
    const int64_t slice_bytes = R * NB * 2;
    t5_expect_tx(fullB, OZ_S * T5_B_BYTES);
    for (int q = 0; q < OZ_S; ++q) t5_bulk_load(sB + q * T5_B_BYTES, gU + q * slice_bytes, T5_B_BYTES, fullB);
    for (int q = 0; q < T5_STAGES; ++q) {
      t5_expect_tx(fullA + 8 * q, T5_A_BYTES);
      t5_bulk_load(sA + q * T5_A_BYTES, gL + q * slice_bytes, T5_A_BYTES, fullA + 8 * q);
    }
    int issued[T5_STAGES] = {1, 1, 1}, landed[T5_STAGES] = {0, 0, 0};
    bool okB = false, ok = true;
    for (int q = 0; q < OZ_S && ok; ++q) {
      const int st = q % T5_STAGES;
      if (!t5_wait(fullA + 8 * st, (q / T5_STAGES) & 1)) { ok = false; break; }
      landed[st]++;
      if (!okB) {
        if (!t5_wait(fullB, 0)) { ok = false; break; }
        okB = true;
      }
      t5_fence_after();
      for (int t = 0; t + q < OZ_S; ++t)
        for (int kk = 0; kk < NB / 16; ++kk)
          t5_mma(tmem + (uint32_t)((q + t) * T5_N), t5_desc(sA + st * T5_A_BYTES + 32 * kk),
                 t5_desc(sB + t * T5_B_BYTES + 32 * kk), (q | kk) != 0);
      t5_commit(emptyA + 8 * st);
      if (q >= 1 && q + 2 < OZ_S) {
        // the stage of slice q - 1 takes slice q + 2 once its products ran
        const int sp = (q - 1) % T5_STAGES;
        if (!t5_wait(emptyA + 8 * sp, ((q - 1) / T5_STAGES) & 1)) { ok = false; break; }
        t5_expect_tx(fullA + 8 * sp, T5_A_BYTES);
        t5_bulk_load(sA + sp * T5_A_BYTES, gL + (q + 2) * slice_bytes, T5_A_BYTES, fullA + 8 * sp);
        issued[sp]++;
      }
    }
    t5_commit(done);  // arrives once every product issued so far has run
    if (!ok) {
      // let the copies in flight land before the CTA's shared memory goes
      *okflag = 0;
      for (int st = 0; st < T5_STAGES; ++st)
        for (int k = landed[st]; k < issued[st]; ++k) t5_wait(fullA + 8 * st, k & 1);
      if (!okB) t5_wait(fullB, 0);
    }
  }
  // epilogue: while the products run, every thread loads its part of its
  // row of the tile's A22 into registers (16 independent loads, so the L2
  // latency is paid once, not once per column); then it waits for the
  // products and reads its part of the accumulators
  const int base_row = j0 + nb;
  const int r = r0 + row;  // this thread's row of the window
  const bool row_live = r < m;
  const int cb = T5_COLS_PER_WARP * cq;  // first tile column of this thread
  double a22[T5_COLS_PER_WARP];
#pragma unroll
  for (int c = 0; c < T5_COLS_PER_WARP; ++c)
    a22[c] = (row_live && c0 + cb + c < m) ? w.at(base_row + r, base_row + c0 + cb + c) : 0.0;
  const bool ready = t5_wait(done, 0);
  if (!ready && tid == 0) t5_wait(done, 0);  // once more before tensor memory is freed
  __syncthreads();
  const bool good = ready && *okflag;
  if (!good && tid == 0) {
    atomicOr(b.sh.oz_error, 1);
    b.state[s].info_fail = 1;
  }
  t5_fence_after();
  if (good) {
    const uint32_t tl = tmem + ((uint32_t)(lg * 32) << 16);
#pragma unroll
    for (int j = 0; j < T5_COLS_PER_WARP / 8; ++j) {
      uint32_t v[OZ_S][8];
#pragma unroll
      for (int d = 0; d < OZ_S; ++d) t5_ld8(tl + (uint32_t)(d * T5_N + cb + 8 * j), v[d]);
      t5_wait_ld();
      if (!row_live) continue;
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) {
        const int c = c0 + cb + 8 * j + cc;
        if (c >= m || (part == 2 && r < NB && c < NB)) continue;
        int ci[OZ_S];
#pragma unroll
        for (int d = 0; d < OZ_S; ++d) ci[d] = __float2int_rn(__uint_as_float(v[d][cc]));
        // S = sum_d c_d 2^(7 (7 - d)), |S| < 2^73; T = floor(S / 2^10) in
        // 64 bits: pairs of diagonals first (|c_d 2^7 + c_(d+1)| < 2^31);
        // the bits dropped weigh below 2^-62 of the largest |S|, far under
        // the slicing's own truncation
        const int P0 = ci[0] * 128 + ci[1], P1 = ci[2] * 128 + ci[3], P2 = ci[4] * 128 + ci[5];
        const int P3 = (ci[6] * 128 + ci[7]) >> 10;
        const long long T = ((long long)P0 << 32) + ((long long)P1 << 18) + ((long long)P2 << 4) + (long long)P3;
        double dv = (double)T;
        // times 2^(e_i + e_j - 2046 - 53) through the exponent field
        const int k = eLr + eU[cb + 8 * j + cc] - 2046 - 53;
        if (dv != 0.0) {
          const long long bits = __double_as_longlong(dv);
          const int e = (int)((bits >> 52) & 0x7FF) + k;
          dv = (e > 0 && e < 2047) ? __longlong_as_double(bits + ((long long)k << 52)) : ldexp(dv, k);
        }
        w.at(base_row + r, base_row + c) = a22[8 * j + cc] - dv;
      }
    }
  }
  t5_fence_before();
  __syncthreads();
  if (warp == 0) {
    t5_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(T5_TMEM_COLS));
  }
}

// The triangular solves run one launch per panel, so a launch's latency is
// the solve's cost: each CTA takes SR rows of the panel's off-diagonal
// block (64 by default), its 4 SR threads four quarters (16 columns) of each
// row, and every
// thread loads its 16 entries into registers before the small triangle's
// dependent chain, so those loads hide behind it; the quarters are added in
// a fixed order.

// Forward substitution for panel p: y_p = L11^-1 b_p into y; then the rows
// below the panel: P_i -= L21(i, :) y_p.  Every CTA solves the small
// triangle redundantly; CTA 0 writes y_p.
template <typename F, int SR>
__global__ void __launch_bounds__(4 * SR) k_wb_fwd(Batch b, int p) {
  p = wb_panel(b, p);
  if (p < 0) return;
  int s = b.sh.wide_structs[blockIdx.y];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WBT<F> w = wb_of<F>(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  const int m = min(w.kl, w.n - j0 - nb);
  // right-hand side blockIdx.z of a multi-column solve (columns rhs_ld apart)
  F* P = wb_rhs(b, inf, blockIdx.z, (F*)nullptr);
  F* Y = wb_scratch(b, inf, blockIdx.z, (F*)nullptr);
  __shared__ F T[NB][NB + 1];  // the panel's diagonal block (L11 below the diagonal)
  __shared__ F ys[NB];
  __shared__ F part[4][SR];
  const int tid = threadIdx.x, r = tid % SR, q = tid / SR;
  const int row = blockIdx.x * SR + r, gi = j0 + nb + row;  // row below the panel
  F lv[16];
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    const int k = 16 * q + u;
    lv[u] = (row < m && k < nb && gi - (j0 + k) <= w.kl) ? w.at(gi, j0 + k) : F(0);
  }
  for (int x = tid; x < NB * NB; x += blockDim.x) {
    int i = x % NB, j = x / NB;
    T[i][j] = (i < nb && j < nb && abs(i - j) <= w.kl) ? w.at(j0 + i, j0 + j) : F(0);
  }
  __syncthreads();
  if (tid < 32) {
    // lanes hold entries k = lane and lane + 32
    F v0 = tid < nb ? P[j0 + tid] : F(0), v1 = tid + 32 < nb ? P[j0 + tid + 32] : F(0);
    for (int k = 0; k < nb; ++k) {
      F yk = __shfl_sync(0xffffffffu, k < 32 ? v0 : v1, k & 31);
      if (tid > k) v0 -= T[tid][k] * yk;
      if (tid + 32 > k) v1 -= T[tid + 32][k] * yk;
    }
    ys[tid] = v0;
    ys[tid + 32] = v1;
  }
  __syncthreads();
  if (blockIdx.x == 0)
    for (int k = tid; k < nb; k += blockDim.x) Y[j0 + k] = ys[k];
  F acc = F(0);
#pragma unroll
  for (int u = 0; u < 16; ++u) acc = wfma(lv[u], ys[16 * q + u], acc);
  part[q][r] = acc;
  __syncthreads();
  if (q == 0 && row < m) P[gi] -= (part[0][r] + part[1][r]) + (part[2][r] + part[3][r]);
}

// Backward substitution for panel p (last panel first): x_p = U11^-1 y_p into
// P; then the rows above the panel: y_i -= U(i, panel) x_p.
template <typename F, int SR>
__global__ void __launch_bounds__(4 * SR) k_wb_bwd(Batch b, int p) {
  p = wb_panel(b, p);
  if (p < 0) return;
  int s = b.sh.wide_structs[blockIdx.y];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WBT<F> w = wb_of<F>(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  // right-hand side blockIdx.z of a multi-column solve (columns rhs_ld apart)
  F* P = wb_rhs(b, inf, blockIdx.z, (F*)nullptr);
  F* Y = wb_scratch(b, inf, blockIdx.z, (F*)nullptr);
  __shared__ F T[NB][NB + 1];  // the panel's diagonal block (U11 on and above the diagonal)
  __shared__ F rdiag[NB];
  __shared__ F xs[NB];
  __shared__ F part[4][SR];
  const int tid = threadIdx.x, r = tid % SR, q = tid / SR;
  const int top = max(0, j0 - w.kl);
  const int gi = top + blockIdx.x * SR + r;  // row above the panel
  F lv[16];
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    const int k = 16 * q + u;
    lv[u] = (gi < j0 && k < nb && j0 + k - gi <= w.kl) ? w.at(gi, j0 + k) : F(0);
  }
  for (int x = tid; x < NB * NB; x += blockDim.x) {
    int i = x % NB, j = x / NB;
    T[i][j] = (i < nb && j < nb && abs(i - j) <= w.kl) ? w.at(j0 + i, j0 + j) : F(0);
  }
  __syncthreads();
  if (tid < nb) rdiag[tid] = wb_rcp(T[tid][tid]);
  __syncthreads();
  if (tid < 32) {
    F v0 = tid < nb ? Y[j0 + tid] : F(0), v1 = tid + 32 < nb ? Y[j0 + tid + 32] : F(0);
    for (int k = nb - 1; k >= 0; --k) {
      F mine = k < 32 ? v0 : v1;
      F xk = __shfl_sync(0xffffffffu, mine, k & 31) * rdiag[k];
      if (k < 32) { if (tid == k) v0 = xk; }
      else { if (tid + 32 == k) v1 = xk; }
      if (tid < k) v0 -= T[tid][k] * xk;
      if (tid + 32 < k) v1 -= T[tid + 32][k] * xk;
    }
    xs[tid] = v0;
    xs[tid + 32] = v1;
  }
  __syncthreads();
  if (blockIdx.x == 0)
    for (int k = tid; k < nb; k += blockDim.x) P[j0 + k] = xs[k];
  F acc = F(0);
#pragma unroll
  for (int u = 0; u < 16; ++u) acc = wfma(lv[u], xs[16 * q + u], acc);
  part[q][r] = acc;
  __syncthreads();
  if (q == 0 && gi < j0) Y[gi] -= (part[0][r] + part[1][r]) + (part[2][r] + part[3][r]);
}

// ---- mixed precision: FP32 factor, FP64 refinement ----
// The trailing update of the FP32 factor: A22 -= L21 U12 over panel p's
// window in 64x64 tiles on the FP32 pipe, each of 256 threads a 4x4 block
// of outputs (four consecutive rows of four columns, so the 16 lanes along a
// column write 256 contiguous bytes).  part as k_wb_update; the corner (the
// next panel's diagonal block, part 1) is the single tile (0, 0).
constexpr int U32T = 64;
__global__ void __launch_bounds__(256) k_wb_update32(Batch b, int p, int part) {
  p = wb_panel(b, p);
  if (p < 0) return;
  int s = b.sh.wide_structs[blockIdx.z];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WBT<float> w = wb_of<float>(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  const int m = min(w.kl, w.n - j0 - nb);
  if (m <= 0) return;
  const int r0 = blockIdx.x * U32T, c0 = blockIdx.y * U32T;
  if (r0 >= m || c0 >= m) return;
  const bool corner = blockIdx.x == 0 && blockIdx.y == 0;
  if ((part == 1 && !corner) || (part == 2 && corner)) return;
  __shared__ __align__(16) float Ls[NB][U32T + 4];  // [k][row]
  __shared__ __align__(16) float Us[NB][U32T + 4];  // [k][col]
  const int tid = threadIdx.x, base = j0 + nb;
  for (int x = tid; x < NB * U32T; x += 256) {
    // rows of L21 along a band column are contiguous; U12's k too
    const int i = x % U32T, k = x / U32T;
    const int gk = j0 + k, gi = base + r0 + i;
    Ls[k][i] = (k < nb && r0 + i < m && gi - gk <= w.kl) ? w.at(gi, gk) : 0.0f;
    const int kk = x % NB, c = x / NB, gj = base + c0 + c;
    Us[kk][c] = (kk < nb && c0 + c < m && gj - (j0 + kk) <= w.kl) ? w.at(j0 + kk, gj) : 0.0f;
  }
  __syncthreads();
  const int tr = tid & 15, tc = tid >> 4;  // rows 4 tr .. 4 tr + 3, columns 4 tc .. 4 tc + 3
  float acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[a][c] = 0.0f;
#pragma unroll 4
  for (int k = 0; k < NB; ++k) {
    const float4 l = *reinterpret_cast<const float4*>(&Ls[k][4 * tr]);
    const float4 u = *reinterpret_cast<const float4*>(&Us[k][4 * tc]);
    const float lv[4] = {l.x, l.y, l.z, l.w}, uv[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][c] = fmaf(lv[a], uv[c], acc[a][c]);
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int col = c0 + 4 * tc + c;
    if (col >= m) continue;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int row = r0 + 4 * tr + a;
      if (row < m) w.at(base + row, base + col) -= acc[a][c];
    }
  }
}

// Start of a mixed solve: K_AA rounded into wband32 (where the FP32 LU then
// forms), the Newton right-hand side saved in FP64 (ir_rhs) and rounded into
// r32, the slot's refinement state reset.
__global__ void __launch_bounds__(256) k_ir_begin(Batch b) {
  const int z = blockIdx.y, s = b.sh.wide_structs[z];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  const int64_t nband = (int64_t)inf.n_free * (2 * (int64_t)inf.wkl + 1);
  const double* src = b.sh.wband + inf.wb_off;
  float* dst = b.sh.wband32 + inf.wb_off;
  const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, dt = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = t0; i < nband; i += dt) dst[i] = __double2float_rn(src[i]);
  const double* P = b.P + inf.dof_off;
  for (int64_t i = t0; i < inf.n_free; i += dt) {
    b.sh.ir_rhs[inf.dof_off + i] = P[i];
    b.sh.r32[inf.dof_off + i] = __double2float_rn(P[i]);
  }
  if (t0 == 0) {
    WideIr& q = b.sh.ir[z];
    q.dn = 0;
    q.xn = 0;
    q.dprev = 0.0;
    q.k = 0;
    q.done = 0;
    b.state[s].ir_fb = 0;
  }
}

// r = b - K x in FP64 (K_AA in wband, x in P, b in ir_rhs), rounded into
// r32 for the next FP32 correction solve.  A CTA takes 256 rows and walks
// the columns j of their band, 256 at a time through shared memory; at each
// j its threads read K(i, j) of consecutive rows, contiguous in the
// column-major band.  Two accumulators per row halve the dependent FP64
// chain.
__global__ void __launch_bounds__(256) k_ir_residual(Batch b) {
  const int z = blockIdx.y, s = b.sh.wide_structs[z];
  if (!wide_active(b, s) || b.sh.ir[z].done) return;
  const StructInfo& inf = b.info[s];
  const int n = inf.n_free, kl = inf.wkl;
  const int i0 = blockIdx.x * 256;
  if (i0 >= n) return;
  const int i = i0 + threadIdx.x;
  const double* x = b.P + inf.dof_off;
  const WB w = wb_of(b, inf);
  __shared__ double xs[256];
  double acc0 = 0.0, acc1 = 0.0;
  const int jlo = max(0, i0 - kl), jhi = min(n, i0 + 256 + kl);
  for (int jt = jlo; jt < jhi; jt += 256) {
    __syncthreads();
    if (jt + (int)threadIdx.x < jhi) xs[threadIdx.x] = x[jt + threadIdx.x];
    __syncthreads();
    if (i >= n) continue;
    // the columns of this tile inside row i's band: |i - j| <= kl
    const int ta = max(0, i - kl - jt), te = min(min(256, jhi - jt), i + kl + 1 - jt);
    int t = ta;
    for (; t + 1 < te; t += 2) {
      acc0 = fma(w.at(i, jt + t), xs[t], acc0);
      acc1 = fma(w.at(i, jt + t + 1), xs[t + 1], acc1);
    }
    if (t < te) acc0 = fma(w.at(i, jt + t), xs[t], acc0);
  }
  if (i < n) b.sh.r32[inf.dof_off + i] = __double2float_rn(b.sh.ir_rhs[inf.dof_off + i] - (acc0 + acc1));
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// x += d in FP64 (d: the FP32 correction the solve left in r32; first: x =
// d, the first solve); the sweep's largest |d| and |x| raise the slot's
// maxima (FP64 bits of non-negative values order like the values, so the
// maxima do not depend on the CTAs' order).  A non-finite entry counts as
// an infinite |d|.
__global__ void __launch_bounds__(256) k_ir_correct(Batch b, int first) {
  const int z = blockIdx.y, s = b.sh.wide_structs[z];
  if (!wide_active(b, s) || b.sh.ir[z].done) return;
  const StructInfo& inf = b.info[s];
  double* x = b.P + inf.dof_off;
  const float* d = b.sh.r32 + inf.dof_off;
  double dm = 0.0, xm = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < inf.n_free; i += gridDim.x * blockDim.x) {
    const double di = (double)d[i], xi = first ? di : x[i] + di;
    x[i] = xi;
    if (!isfinite(xi)) dm = INFINITY;
    dm = fmax(dm, fabs(di));
    xm = fmax(xm, fabs(xi));
  }
  __shared__ double red[2][8];
  dm = warp_max(dm);
  xm = warp_max(xm);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    red[0][warp] = dm;
    red[1][warp] = xm;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q) {
      dm = fmax(dm, red[0][q]);
      xm = fmax(xm, red[1][q]);
    }
    WideIr& q = b.sh.ir[z];
    if (dm > 0.0) atomicMax(&q.dn, (unsigned long long)__double_as_longlong(dm));
    if (xm > 0.0) atomicMax(&q.xn, (unsigned long long)__double_as_longlong(xm));
  }
}

// After a correction, per slot: converged (|d| <= 2^-52 |x|), stalled
// (|d| > |d_prev| / 2: at the FP64 floor, or a factor too poor to refine),
// or out of sweeps (ir_max).  A stall above 2^-30 |x|, the sweep limit, a
// non-finite value or a failed FP32 pivot hand the solve to the FP64
// fallback (ir_fb).  ir_more[0]: a slot refines on (inside a captured pass
// also the refinement loop's condition h); ir_more[1]: a slot takes the
// fallback; ir_more[2] counts the sweeps run (sweep: called after one).
__global__ void k_ir_check(Batch b, cudaGraphConditionalHandle h, int use_h, int sweep) {
  __shared__ int more, fb;
  if (threadIdx.x == 0) {
    more = 0;
    fb = 0;
  }
  __syncthreads();
  for (int z = threadIdx.x; z < b.sh.n_wide; z += blockDim.x) {
    const int s = b.sh.wide_structs[z];
    if (!wide_active(b, s)) continue;
    WideIr& q = b.sh.ir[z];
    StructState& st = b.state[s];
    if (!q.done) {
      const double dn = __longlong_as_double((long long)q.dn), xn = __longlong_as_double((long long)q.xn);
      q.dn = 0;
      q.xn = 0;
      bool stop = false, bad = false;
      if (st.ir_fb || !(dn <= DBL_MAX) || !(xn <= DBL_MAX)) {
        stop = true;
        bad = true;
      } else if (q.k > 0) {
        st.ir_sweeps += 1;
        if (dn <= 0x1p-52 * xn) {
          stop = true;
        } else if (dn > 0.5 * q.dprev) {
          stop = true;
          bad = dn > 0x1p-30 * xn;
        } else if (q.k >= b.sh.ir_max) {
          stop = true;
          bad = true;
        }
      }
      q.dprev = dn;
      q.k += 1;
      if (stop) {
        q.done = 1;
        if (bad) {
          st.ir_fb = 1;
          st.ir_fallbacks += 1;
        }
      }
    }
    if (!q.done) atomicOr(&more, 1);
    if (st.ir_fb) atomicOr(&fb, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    b.sh.ir_more[0] = more;
    b.sh.ir_more[1] = fb;
    if (sweep) b.sh.ir_more[2] += 1;
    if (use_h) cudaGraphSetConditional(h, more ? 1u : 0u);
  }
}

// The FP64 fallback's condition: a slot whose refinement did not finish.
__global__ void k_ir_fb_cond(Batch b, cudaGraphConditionalHandle h) {
  cudaGraphSetConditional(h, b.sh.ir_more[1] ? 1u : 0u);
}

// The FP64 fallback's right-hand side: P = the saved Newton right-hand side
// (b: the fallback's view, so only structures with ir_fb are active);
// ir_more[3] counts the fallbacks run.
__global__ void k_ir_restore(Batch b) {
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) b.sh.ir_more[3] += 1;
  const int z = blockIdx.y, s = b.sh.wide_structs[z];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < inf.n_free; i += gridDim.x * blockDim.x)
    b.P[inf.dof_off + i] = b.sh.ir_rhs[inf.dof_off + i];
}

void launch_wide_zero(const Batch& b, cudaStream_t st) {
  if (b.sh.n_wide == 0) return;
  k_wb_zero<<<dim3(4 * 152, b.sh.n_wide), 256, 0, st>>>(b);
}

// Launches at the batch's tile shapes (b.sh.tiles).  The trsm of a panel:
// the first NB rows and columns (the next panel's diagonal block needs them)
// in CTAs of tiles.trsm_first rows, the rest in CTAs of tiles.trsm_rb.
static int trsm_first_blocks(const Batch& b) { return NB / b.sh.tiles.trsm_first; }
static int trsm_rest_blocks(const Batch& b) {
  const int kl = b.sh.max_kl, rb = b.sh.tiles.trsm_rb;
  return kl > NB ? (kl - NB + rb - 1) / rb : 0;
}
template <typename F, int RB>
static void trsm_at(const Batch& b, int p, int row0, int nblk, cudaStream_t st) {
  k_wb_trsm<F, RB><<<dim3(2 * nblk, b.sh.n_wide), 32 * RB, 0, st>>>(b, p, row0, nblk);
}
// rows row0 .. of panel p (and as many columns) in nblk CTAs of rb rows
template <typename F>
static void launch_trsm(const Batch& b, int p, int row0, int nblk, int rb, cudaStream_t st) {
  switch (rb) {
    case 1: trsm_at<F, 1>(b, p, row0, nblk, st); break;
    case 2: trsm_at<F, 2>(b, p, row0, nblk, st); break;
    case 4: trsm_at<F, 4>(b, p, row0, nblk, st); break;
    case 16: trsm_at<F, 16>(b, p, row0, nblk, st); break;
    default: trsm_at<F, 8>(b, p, row0, nblk, st); break;
  }
}
template <typename F> static void launch_trsm_first(const Batch& b, int p, cudaStream_t st) {
  launch_trsm<F>(b, p, 0, trsm_first_blocks(b), b.sh.tiles.trsm_first, st);
}
template <typename F> static void launch_trsm_rest(const Batch& b, int p, cudaStream_t st) {
  launch_trsm<F>(b, p, NB, trsm_rest_blocks(b), b.sh.tiles.trsm_rb, st);
}
static void launch_corner(const Batch& b, int p, cudaStream_t st) {
  const int nw = b.sh.n_wide;
  if (b.sh.tiles.corner == 4) k_wb_corner<4><<<dim3(NB / 4, NB / 4, nw), 64, 0, st>>>(b, p);
  else k_wb_corner<8><<<dim3(NB / 8, NB / 8, nw), 256, 0, st>>>(b, p);
}
// the triangular solves of panel p: rows of tiles.sub_rows per CTA, nrhs
// right-hand sides
template <typename F> static void launch_fwd(const Batch& b, int p, int nrhs, cudaStream_t st) {
  const int sr = b.sh.tiles.sub_rows, kl = b.sh.max_kl, nb = kl > 0 ? (kl + sr - 1) / sr : 1;
  if (sr == 32) k_wb_fwd<F, 32><<<dim3(nb, b.sh.n_wide, nrhs), 128, 0, st>>>(b, p);
  else k_wb_fwd<F, 64><<<dim3(nb, b.sh.n_wide, nrhs), 256, 0, st>>>(b, p);
}
template <typename F> static void launch_bwd(const Batch& b, int p, int nrhs, cudaStream_t st) {
  const int sr = b.sh.tiles.sub_rows, kl = b.sh.max_kl, nb = kl > 0 ? (kl + sr - 1) / sr : 1;
  if (sr == 32) k_wb_bwd<F, 32><<<dim3(nb, b.sh.n_wide, nrhs), 128, 0, st>>>(b, p);
  else k_wb_bwd<F, 64><<<dim3(nb, b.sh.n_wide, nrhs), 256, 0, st>>>(b, p);
}

// Panel loop with lookahead on three helper streams (fork / join by events,
// so a captured pass keeps the same dependencies):
//   main   trsm first(p) -> corner(p) -> [join trsm rest(p)] -> update rest(p)
//          -> [join diag(p+1)]
//   s4     [at the panel's start] trsm rest(p)
//   s2     [after corner(p)] diag(p+1)
//   s3     [after all trsm(p)] forward substitution of panel p
// The critical path per panel is the first trsm blocks, the corner and the
// next diagonal LU; the bulk trsm runs beside them, and the next diagonal LU
// and the forward substitution beside the bulk of the trailing update.  The
// backward substitution follows the last panel.
// The trailing update of panel p (part as in k_wb_update): on the tensor
// cores (64x64 tiles) when the batch asks for it, else in FP64 (32x32).
// The corner (the next panel's diagonal block, on the lookahead's critical
// path) always takes the FP64 kernel k_wb_corner: 64 small CTAs finish it
// sooner than one tensor-core CTA's load, slice and multiply sequence.
static void launch_wb_update(const Batch& b, int p, int part, cudaStream_t st) {
  const int nw = b.sh.n_wide, mr = b.sh.max_kl;
  if (b.sh.wide_tc && part != 1) {
    static const bool attr = [] {  // once per process, thread-safe
      cudaFuncSetAttribute(k_wb_update_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OZ_SMEM);
      cudaFuncSetAttribute(k_wb_update_t5, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T5_SMEM);
      return true;
    }();
    (void)attr;
    // the panel's slices (L21 rows and U12 columns), then the tiles
    k_wb_slice<<<dim3((mr + SL_ROWS - 1) / SL_ROWS, 2, nw), 256, 0, st>>>(b, p);
    if (b.sh.wide_tc == 1)  // GF_WIDE_TENSOR: tcgen05; 2, GF_WIDE_TENSOR_SYNC: mma.sync
      k_wb_update_t5<<<dim3((mr + T5_M - 1) / T5_M, (mr + T5_N - 1) / T5_N, nw), T5_THREADS, T5_SMEM, st>>>(b, p,
                                                                                                         part);
    else
      k_wb_update_tc<<<dim3((mr + OZ_TR - 1) / OZ_TR, (mr + OZ_T - 1) / OZ_T, nw), OZ_THREADS, OZ_SMEM, st>>>(b, p,
                                                                                                        part);
  } else if (part == 1) {
    launch_corner(b, p, st);
  } else {
    const int t = (mr + UT - 1) / UT;
    k_wb_update<<<dim3(t, t, nw), 256, 0, st>>>(b, p, part);
  }
}

// Panel-loop control inside a captured pass: the counter's start value,
// and the step at the end of each loop body, which also sets the loop's
// condition (continue while the counter stays in [0, limit)).
__global__ void k_wb_loop_set(int* counter, int v) { *counter = v; }
__global__ void k_wb_loop_step(int* counter, int step, int limit, cudaGraphConditionalHandle h) {
  const int c = *counter + step;
  *counter = c;
  cudaGraphSetConditional(h, (c >= 0 && c < limit) ? 1u : 0u);
}

namespace {
// A conditional handle on the graph that st captures into, its value reset
// to dflt at every launch of the graph.
cudaError_t make_cond(cudaStream_t st, cudaGraphConditionalHandle* h, unsigned dflt) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr);
  if (e != cudaSuccess) return e;
  return cudaGraphConditionalHandleCreate(h, g, dflt, cudaGraphCondAssignDefault);
}

// Appends a conditional node of the given type on handle h to the capture
// of st and returns its body graph, into which the caller captures the body.
cudaError_t add_cond(cudaStream_t st, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                     cudaGraph_t* body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd);
  if (e != cudaSuccess) return e;
  std::vector<cudaGraphNode_t> dv(deps, deps + nd);
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = type;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  if ((e = cudaGraphAddNode(&node, g, dv.data(), nullptr, dv.size(), &np)) != cudaSuccess) return e;
  *body = np.conditional.phGraph_out[0];
  return cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

// A WHILE node whose condition starts at 1 on every launch.
cudaError_t add_while(cudaStream_t st, cudaGraphConditionalHandle* h, cudaGraph_t* body) {
  cudaError_t e = make_cond(st, h, 1);
  return e != cudaSuccess ? e : add_cond(st, *h, cudaGraphCondTypeWhile, body);
}

// The trailing update of panel p in the factor's type (FP64: launch_wb_update
// with the batch's choice of kernel; FP32: k_wb_update32, the corner as its
// single tile).
void wb_update(const Batch& b, int p, int part, cudaStream_t st, double*) { launch_wb_update(b, p, part, st); }

// The next panel's diagonal LU, one CTA per structure on the lookahead's
// critical path, launched at the device's highest stream priority: the
// block scheduler then gives it the first free SM ahead of the trailing
// update's and the helper streams' CTAs (a captured launch keeps the
// priority as a node attribute).
template <typename F> void launch_diag(const Batch& b, int p, cudaStream_t st) {
  static const int prio = [] {
    int lo = 0, hi = 0;
    return cudaDeviceGetStreamPriorityRange(&lo, &hi) == cudaSuccess ? hi : 0;
  }();
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(b.sh.n_wide);
  cfg.blockDim = dim3(DIAG_THREADS);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = prio;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_wb_diag<F>, b, p);
}
void wb_update(const Batch& b, int p, int part, cudaStream_t st, float*) {
  const int t = part == 1 ? 1 : (b.sh.max_kl + U32T - 1) / U32T;
  k_wb_update32<<<dim3(t, t, b.sh.n_wide), 256, 0, st>>>(b, p, part);
}
}  // namespace

// The panel loops as two graph-resident WHILE loops (forward: factor and
// forward substitution, one panel per iteration; backward substitution, last
// panel first), used when a served wave's pass is captured: the pass graph
// then holds a dozen nodes whatever the panel count, instead of six launches
// per panel, and instantiates in a millisecond even while other waves run
// (a graph of thousands of launches took hundreds of milliseconds then, and
// held up the server's other CUDA calls).  One iteration keeps the
// lookahead of the launched form (next panel's diagonal LU and this panel's
// forward step beside the trailing update); it ends with the counter step.
// Each iteration costs a few microseconds more than the unrolled panel
// sequence, so the batch path, which captures once on an idle device, keeps
// the unrolled form.  F: the factor's type.
template <typename F>
static cudaError_t capture_wide_loops(const Batch& b, cudaStream_t st) {
  const ShellData& sd = b.sh;
  const int nw = sd.n_wide, mr = sd.max_kl, P = sd.max_panels;
  const int nrest = trsm_rest_blocks(b);
  (void)mr;
  cudaStream_t sb = sd.aux[2], s2 = sd.aux[0], s3 = sd.aux[1], s4 = sd.aux[3];
  cudaEvent_t e_start = sd.evt[0], e_trsm = sd.evt[1], e_corner = sd.evt[2], e_diag = sd.evt[3], e_fwd = sd.evt[4],
              e_rest = sd.evt[5];
  if (P <= 0) return cudaSuccess;
  cudaError_t e;
  cudaGraphConditionalHandle h;
  cudaGraph_t body, done;
  k_wb_loop_set<<<1, 1, 0, st>>>(sd.panel, 0);
  k_wb_diag<F><<<nw, DIAG_THREADS, 0, st>>>(b, 0);
  if ((e = add_while(st, &h, &body)) != cudaSuccess) return e;
  if ((e = cudaStreamBeginCaptureToGraph(sb, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
    return e;
  if (nrest) {
    cudaEventRecord(e_start, sb);
    cudaStreamWaitEvent(s4, e_start, 0);
    launch_trsm_rest<F>(b, -1, s4);
    cudaEventRecord(e_rest, s4);
  }
  launch_trsm_first<F>(b, -1, sb);
  wb_update(b, -1, 1, sb, (F*)nullptr);
  cudaEventRecord(e_corner, sb);
  cudaStreamWaitEvent(s2, e_corner, 0);
  launch_diag<F>(b, -2, s2);
  cudaEventRecord(e_diag, s2);
  if (nrest) cudaStreamWaitEvent(sb, e_rest, 0);
  cudaEventRecord(e_trsm, sb);
  cudaStreamWaitEvent(s3, e_trsm, 0);
  launch_fwd<F>(b, -1, 1, s3);
  cudaEventRecord(e_fwd, s3);
  wb_update(b, -1, 2, sb, (F*)nullptr);
  cudaStreamWaitEvent(sb, e_diag, 0);
  cudaStreamWaitEvent(sb, e_fwd, 0);
  k_wb_loop_step<<<1, 1, 0, sb>>>(sd.panel, 1, P, h);
  if ((e = cudaStreamEndCapture(sb, &done)) != cudaSuccess) return e;
  k_wb_loop_set<<<1, 1, 0, st>>>(sd.panel, P - 1);
  if ((e = add_while(st, &h, &body)) != cudaSuccess) return e;
  if ((e = cudaStreamBeginCaptureToGraph(sb, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
    return e;
  launch_bwd<F>(b, -1, 1, sb);
  k_wb_loop_step<<<1, 1, 0, sb>>>(sd.panel, -1, P, h);
  return cudaStreamEndCapture(sb, &done);
}

// The first error of a wide-band capture step on this thread (a failed
// conditional node or body capture), which the capturing caller reports:
// capture_error() returns it and clears it.
static thread_local cudaError_t g_capture_error = cudaSuccess;
static void capture_fail(cudaError_t e) {
  if (e != cudaSuccess && g_capture_error == cudaSuccess) g_capture_error = e;
}
cudaError_t wide_capture_error() {
  const cudaError_t e = g_capture_error;
  g_capture_error = cudaSuccess;
  return e;
}

// The same panel sequence on st alone, without the lookahead's helper
// streams, in dependency order (the kernels and their results are those of
// the lookahead form): the FP64 fallback inside the mixed path's captured
// pass, whose helper streams already belong to that capture.
template <typename F>
static void wide_factor_solve_serial(const Batch& b, cudaStream_t st) {
  const ShellData& sd = b.sh;
  const int nw = sd.n_wide, nrest = trsm_rest_blocks(b);
  k_wb_diag<F><<<nw, DIAG_THREADS, 0, st>>>(b, 0);
  for (int p = 0; p < sd.max_panels; ++p) {
    const bool next = p + 1 < sd.max_panels;
    if (nrest) launch_trsm_rest<F>(b, p, st);
    launch_trsm_first<F>(b, p, st);
    if (next) {
      wb_update(b, p, 1, st, (F*)nullptr);
      k_wb_diag<F><<<nw, DIAG_THREADS, 0, st>>>(b, p + 1);
    }
    launch_fwd<F>(b, p, 1, st);
    wb_update(b, p, next ? 2 : 0, st, (F*)nullptr);
  }
  for (int p = sd.max_panels - 1; p >= 0; --p) launch_bwd<F>(b, p, 1, st);
}

// Factor and solve in the factor's type F: FP64, the LU in place of K_AA
// and the solve on P; FP32 (mixed path), the LU in wband32 and the solve on
// r32.  Inside a served wave's capture the panel loops are graph loops
// (capture_wide_loops), else one launch sequence per panel with lookahead.
template <typename F>
static void wide_factor_solve(const Batch& b, cudaStream_t st, LaunchProf* prof) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (!prof && b.sh.loops_in_graph && b.sh.panel && cudaStreamIsCapturing(st, &cs) == cudaSuccess &&
      cs == cudaStreamCaptureStatusActive) {
    capture_fail(capture_wide_loops<F>(b, st));
    return;
  }
  const ShellData& sd = b.sh;
  const int nw = sd.n_wide;
  const int mr = sd.max_kl;  // largest kl over the wide structures
  const int nrest = trsm_rest_blocks(b);
  (void)mr;
  cudaStream_t s2 = sd.aux[0], s3 = sd.aux[1], s4 = sd.aux[3];
  // the helpers fork from the main stream at their first wait and join it
  // again before the backward substitution
  cudaEvent_t e_start = sd.evt[0], e_trsm = sd.evt[1], e_corner = sd.evt[2], e_diag = sd.evt[3], e_fwd = sd.evt[4],
              e_rest = sd.evt[5];
  { ProfScope q(prof, st, KC_WIDE_DIAG); k_wb_diag<F><<<nw, DIAG_THREADS, 0, st>>>(b, 0); }
  for (int p = 0; p < sd.max_panels; ++p) {
    bool next = p + 1 < sd.max_panels;
    if (nrest) {
      cudaEventRecord(e_start, st);
      cudaStreamWaitEvent(s4, e_start, 0);
      ProfScope q(prof, s4, KC_WIDE_TRSM);
      launch_trsm_rest<F>(b, p, s4);
      cudaEventRecord(e_rest, s4);
    }
    {
      ProfScope q(prof, st, KC_WIDE_TRSM);
      launch_trsm_first<F>(b, p, st);
    }
    if (next) {
      { ProfScope q(prof, st, KC_WIDE_UPDATE); wb_update(b, p, 1, st, (F*)nullptr); }
      cudaEventRecord(e_corner, st);
      cudaStreamWaitEvent(s2, e_corner, 0);
      { ProfScope q(prof, s2, KC_WIDE_DIAG); launch_diag<F>(b, p + 1, s2); }
      cudaEventRecord(e_diag, s2);
    }
    if (nrest) cudaStreamWaitEvent(st, e_rest, 0);
    cudaEventRecord(e_trsm, st);
    cudaStreamWaitEvent(s3, e_trsm, 0);
    { ProfScope q(prof, s3, KC_WIDE_SUBST); launch_fwd<F>(b, p, 1, s3); }
    if (next) {
      { ProfScope q(prof, st, KC_WIDE_UPDATE); wb_update(b, p, 2, st, (F*)nullptr); }
      cudaStreamWaitEvent(st, e_diag, 0);
    } else {
      { ProfScope q(prof, st, KC_WIDE_UPDATE); wb_update(b, p, 0, st, (F*)nullptr); }
    }
  }
  // join: every forward step is done before the backward substitution
  cudaEventRecord(e_fwd, s3);
  cudaStreamWaitEvent(st, e_fwd, 0);
  for (int p = sd.max_panels - 1; p >= 0; --p) {
    ProfScope q(prof, st, KC_WIDE_SUBST);
    launch_bwd<F>(b, p, 1, st);
  }
}

// One refinement sweep of the mixed path: the FP64 residual into r32, the
// FP32 forward and backward substitution with the FP32 LU (one launch per
// panel), x += d and the check, which sets the refinement loop's condition
// h when use_h.  (Served waves, whose passes hold the panel loops as graph
// loops, are built with the FP64 options and never refine.)
static void ir_sweep(const Batch& b, cudaStream_t st, cudaGraphConditionalHandle h, int use_h, LaunchProf* prof) {
  const ShellData& sd = b.sh;
  const int nw = sd.n_wide, P = sd.max_panels;
  const int rows = (P * NB + 255) / 256;
  { ProfScope q(prof, st, KC_WIDE_REFINE); k_ir_residual<<<dim3(rows, nw), 256, 0, st>>>(b); }
  for (int p = 0; p < P; ++p) {
    ProfScope q(prof, st, KC_WIDE_SUBST);
    launch_fwd<float>(b, p, 1, st);
  }
  for (int p = P - 1; p >= 0; --p) {
    ProfScope q(prof, st, KC_WIDE_SUBST);
    launch_bwd<float>(b, p, 1, st);
  }
  {
    ProfScope q(prof, st, KC_WIDE_REFINE);
    k_ir_correct<<<dim3(2 * 152, nw), 256, 0, st>>>(b, 0);
    k_ir_check<<<1, 128, 0, st>>>(b, h, use_h, 1);
  }
}

// Mixed precision (GF_PREC_MIXED): the FP32 LU of K_AA, its solve, then FP64
// iterative refinement against the FP64 K_AA until the corrections stop
// shrinking; a structure whose refinement does not reach the FP64 level is
// solved again by the FP64 LU.  Inside a captured pass the refinement loop
// is a WHILE node and the fallback an IF node, so the pass needs no host
// round trip; otherwise the host reads the loop's flags after each sweep.
static void wide_solve_mixed(const Batch& b, cudaStream_t st, LaunchProf* prof) {
  const ShellData& sd = b.sh;
  const int nw = sd.n_wide;
  Batch fb = b;  // the FP64 fallback's view
  fb.sh.fp64_pass = 1;
  { ProfScope q(prof, st, KC_WIDE_REFINE); k_ir_begin<<<dim3(4 * 152, nw), 256, 0, st>>>(b); }
  wide_factor_solve<float>(b, st, prof);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  const bool capturing = !prof && cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive;
  if (capturing) {
    // the bodies are captured on aux[4], which the pass's capture has not
    // forked into; a failed step is recorded for the capturing caller
    cudaStream_t sr = sd.aux[4];
    cudaGraphConditionalHandle h, hf;
    cudaGraph_t body, done;
    cudaError_t e;
    if ((e = make_cond(st, &h, 0)) != cudaSuccess) return capture_fail(e);
    k_ir_correct<<<dim3(2 * 152, nw), 256, 0, st>>>(b, 1);
    k_ir_check<<<1, 128, 0, st>>>(b, h, 1, 0);
    if ((e = add_cond(st, h, cudaGraphCondTypeWhile, &body)) != cudaSuccess) return capture_fail(e);
    if ((e = cudaStreamBeginCaptureToGraph(sr, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess)
      return capture_fail(e);
    ir_sweep(b, sr, h, 1, nullptr);
    if ((e = cudaStreamEndCapture(sr, &done)) != cudaSuccess) return capture_fail(e);
    if ((e = make_cond(st, &hf, 0)) != cudaSuccess) return capture_fail(e);
    k_ir_fb_cond<<<1, 1, 0, st>>>(b, hf);
    if ((e = add_cond(st, hf, cudaGraphCondTypeIf, &body)) != cudaSuccess) return capture_fail(e);
    if ((e = cudaStreamBeginCaptureToGraph(sr, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess)
      return capture_fail(e);
    k_ir_restore<<<dim3(2 * 152, nw), 256, 0, sr>>>(fb);
    wide_factor_solve_serial<double>(fb, sr);
    if ((e = cudaStreamEndCapture(sr, &done)) != cudaSuccess) return capture_fail(e);
    return;
  }
  {
    ProfScope q(prof, st, KC_WIDE_REFINE);
    k_ir_correct<<<dim3(2 * 152, nw), 256, 0, st>>>(b, 1);
    k_ir_check<<<1, 128, 0, st>>>(b, 0, 0, 0);
  }
  int more[2] = {0, 0};
  for (int k = 0; k <= sd.ir_max; ++k) {
    if (cudaMemcpyAsync(more, sd.ir_more, sizeof(more), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess || !more[0])
      break;
    ir_sweep(b, st, 0, 0, prof);
  }
  if (cudaMemcpyAsync(more, sd.ir_more, sizeof(more), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return;
  if (more[1]) {
    k_ir_restore<<<dim3(2 * 152, nw), 256, 0, st>>>(fb);
    wide_factor_solve<double>(fb, st, prof);
  }
}

void launch_wide_solve(const Batch& b, cudaStream_t st, LaunchProf* prof) {
  if (b.sh.n_wide == 0) return;
  if (b.mixed && b.sh.wband32) wide_solve_mixed(b, st, prof);
  else wide_factor_solve<double>(b, st, prof);
}

// Forward and backward substitution alone on a wide band that already holds
// its LU (a factor from launch_wide_solve), for nrhs right-hand sides at
// b.P + q b.rhs_ld (q < nrhs, scratch alike in b.y): the panel loops of
// launch_wide_solve without the factor, every column per launch.
void launch_wide_subst(const Batch& b, int nrhs, cudaStream_t st) {
  if (b.sh.n_wide == 0 || nrhs <= 0) return;
  for (int p = 0; p < b.sh.max_panels; ++p) launch_fwd<double>(b, p, nrhs, st);
  for (int p = b.sh.max_panels - 1; p >= 0; --p) launch_bwd<double>(b, p, nrhs, st);
}

// Launches of the panel loops: unrolled, the first diagonal LU, then per
// panel the first trsm blocks, update corner + next diagonal, the other trsm
// blocks, forward step, update rest, backward step (the last panel has no
// corner or next diagonal); graph loops, two loop-control kernels, the first
// diagonal LU, the same six or seven kernels and a counter step per forward
// iteration, and two kernels per backward one; the FP64 tensor-core update
// adds its slicing kernel per panel.
static int wide_factor_launches(const Batch& b, bool fp64) {
  const int P = b.sh.max_panels, per = 6 + (trsm_rest_blocks(b) ? 1 : 0);
  return (b.sh.loops_in_graph ? 3 + (per + 2) * P : 1 + per * P - 2) + (fp64 && b.sh.wide_tc ? P : 0);
}

// Per Newton pass; the mixed path adds its start, first correction and
// check and the fallback's condition, and its sweeps and fallbacks come on
// top (wide_refine_launches).
int wide_launches_per_pass(const Batch& b) {
  if (!b.sh.n_wide) return 0;
  if (b.mixed && b.sh.wband32) return wide_factor_launches(b, false) + 4;
  return wide_factor_launches(b, true);
}

// Launches of `sweeps` refinement sweeps (residual, forward and backward
// substitution, correction, check) and `fallbacks` FP64 fallbacks.
long long wide_refine_launches(const Batch& b, long long sweeps, long long fallbacks) {
  const int P = b.sh.max_panels;
  const long long per_sweep = 3 + 2 * P;
  return sweeps * per_sweep + fallbacks * (1 + wide_factor_launches(b, true));
}

}  // namespace gf
