// Chain solver kernels (see gf_chain.cuh).  One thread per item (element or
// corner): every FP64 warp instruction carries 32 independent items, which is
// what the FP64 unit's throughput needs.  The small dense solves factor the
// 6x6 pivot block in registers (reciprocals and multipliers kept there too)
// and then take the right-hand sides one column at a time, so no kernel here
// uses shared memory.
#include <cuda_runtime.h>

#include "gf_chain.cuh"
#include "gf_math.cuh"

namespace gf {

namespace {

constexpr int CT = 64;   // threads per block

// Scratch arrays are structure-of-arrays: entry x of chain element t at
// [x * n_chain_elems + t], entry x of corner k at [x * n_corners + k], so
// that the threads of a warp (consecutive items) touch consecutive addresses.
#define ELM(arr, t, x) (arr)[(int64_t)(x) * c.n_chain_elems + (t)]
#define CRN(arr, k, x) (arr)[(int64_t)(x) * c.n_corners + (k)]
constexpr int NC = 19;   // augmented columns: 6 (matrix) + 13 (right-hand sides)

__device__ __forceinline__ bool solving(const Batch& b, int s) {
  const StructState& st = b.state[s];
  return st.phase == PH_ITER && st.need_solve;
}

// Newton-Raphson reciprocal seeded by the FP32 hardware approximation (two
// steps r <- r + r (1 - p r)); exact division outside the FP32 range.
__device__ __forceinline__ double recip(double p) {
  float pf = __double2float_rn(p);
  float af = fabsf(pf);
  if (!(af > 1e-30f && af < 1e30f)) return 1.0 / p;
  float rf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(pf));
  double r = (double)rf;
  double e = fma(-p, r, 1.0);
  r = fma(r, e, r);
  e = fma(-p, r, 1.0);
  r = fma(r, e, r);
  return r;
}

// Gauss-Jordan on a thread's augmented matrix [D | R] in two phases, both in
// registers: gj6_factor eliminates D (6x6, row-major, every index static under
// the full unroll) and records each pivot's reciprocal and multipliers;
// gj6_apply then takes one right-hand-side column through the same steps in
// the same order (r_k *= 1/p_k, then r_i -= m_ik r_k), so each column needs
// its six entries only and no shared memory.  The operations on every entry
// are those of the joined elimination.  No pivoting; gj6_factor returns false
// on a zero or non-finite pivot.
__device__ __forceinline__ bool gj6_factor(double (&D)[36], double (&inv)[6], double (&mult)[36]) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const double p = D[k * 6 + k];
    if (!(p != 0.0) || !isfinite(p)) ok = false;
    inv[k] = recip(p);
    double dk[6];
#pragma unroll
    for (int c = k + 1; c < 6; ++c) {
      dk[c] = D[k * 6 + c] * inv[k];
      D[k * 6 + c] = dk[c];
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      if (i == k) continue;
      const double m = D[i * 6 + k];
      mult[k * 6 + i] = m;
#pragma unroll
      for (int c = k + 1; c < 6; ++c) D[i * 6 + c] = fma(-m, dk[c], D[i * 6 + c]);
    }
  }
  return ok;
}
__device__ __forceinline__ void gj6_apply(const double (&inv)[6], const double (&mult)[36], double (&r)[6]) {
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const double rk = r[k] * inv[k];
    r[k] = rk;
#pragma unroll
    for (int i = 0; i < 6; ++i)
      if (i != k) r[i] = fma(-mult[k * 6 + i], rk, r[i]);
  }
}

// ---- 1. condensation of the midside node of every chain element ----
__global__ void __launch_bounds__(CT) k_condense(Batch b, ChainData c) {
  int t = blockIdx.x * CT + threadIdx.x;
  if (t >= c.n_chain_elems) return;
  int e = c.elem_list[t];
  int s = b.estruct[e];
  if (!solving(b, s)) return;
  const StructInfo inf = b.info[s];
  const double* P = b.P + inf.dof_off;
  double D[36];  // K_mm (+ the load stiffness)
  // K of the chain comes from the element tangents (column-major 18x18,
  // DOFs of the first corner, the midside node, the last corner) plus the
  // nodal load stiffness of the midside node: the midside rows belong to
  // this element alone
  const double* Kb = b.Ke + e;  // structure-of-arrays: entry x at Kb[x * n_elem]
  const int64_t ne = b.n_elem;
#define K(x) Kb[(int64_t)(x) * ne]
  const double* nk = b.nodeK + (int64_t)b.enodes[3 * e + 1] * 9;
  int nm = b.enodes[3 * e + 1];
  bool fa = c.elem_corner_a[t] >= 0, fb = c.elem_corner_b[t] >= 0;
  int gm[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) gm[i] = b.gl[(int64_t)nm * 6 + i];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      double kmm = K((6 + i) + 18 * (6 + j));
      if (i >= 3 && j >= 3) kmm += nk[(i - 3) * 3 + j - 3];
      D[i * 6 + j] = kmm;
    }
  }
  double inv[6], mult[36];
  if (!gj6_factor(D, inv, mult)) b.state[s].info_fail = 1;
  // Z = K_mm^-1 [P_m | K_ma | K_mb] a column at a time, and with each column
  // its share of -A_as Z and -A_bs Z (6 x 13 each: the same FMA chain over j
  // for every entry)
#pragma unroll 1
  for (int q = 0; q < 13; ++q) {
    double r[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      if (q == 0) r[i] = P[gm[i]];
      else if (q < 7) r[i] = fa ? K((6 + i) + 18 * (q - 1)) : 0.0;
      else r[i] = fb ? K((6 + i) + 18 * (12 + q - 7)) : 0.0;
    }
    gj6_apply(inv, mult, r);
#pragma unroll
    for (int i = 0; i < 6; ++i) ELM(c.ez, t, i * 13 + q) = r[i];
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const bool free_side = side ? fb : fa;
      const int r0 = side ? 12 : 0;
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < 6; ++j) acc = fma(free_side ? K((r0 + i) + 18 * (6 + j)) : 0.0, r[j], acc);
        ELM(c.ec, t, i * 26 + side * 13 + q) = -acc;
      }
    }
  }
}

#undef K

// ---- 2. corner system ----
__global__ void k_corner_system(Batch b, ChainData c) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= c.n_corners) return;
  int s = c.corner_struct[k];
  if (!solving(b, s)) return;
  const StructInfo inf = b.info[s];
  const double* P = b.P + inf.dof_off;
  int node = c.corner_node[k];
  int eL = c.corner_left[k], eR = c.corner_right[k];
  int kp = c.corner_prev[k], kn = c.corner_next[k];
  int g[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) g[i] = b.gl[(int64_t)node * 6 + i];
  // K blocks from the element tangents: the corner is the last node of the
  // element on its left and the first of the one on its right (two terms,
  // so the sum does not depend on their order), then the nodal load
  // stiffness, as the band held them
  const int64_t ne = b.n_elem;  // element scratch: entry x of element e at [x * n_elem + e]
  const double* KL = eL >= 0 ? b.Ke + c.elem_list[eL] : nullptr;
  const double* KR = eR >= 0 ? b.Ke + c.elem_list[eR] : nullptr;
  const double* nk = b.nodeK + (int64_t)node * 9;
  for (int i = 0; i < 6; ++i) {
    for (int j = 0; j < 6; ++j) {
      double kl = KL ? KL[((12 + i) + 18 * (12 + j)) * ne] : 0.0;
      double kr = KR ? KR[(i + 18 * j) * ne] : 0.0;
      double d = kl + kr;
      if (i >= 3 && j >= 3) d += nk[(i - 3) * 3 + j - 3];
      if (eL >= 0) d += ELM(c.ec, eL, i * 26 + 13 + 7 + j);  // -A_bs Z_b of the left element
      if (eR >= 0) d += ELM(c.ec, eR, i * 26 + 1 + j);       // -A_as Z_a of the right element
      CRN(c.cD, k, i * 6 + j) = d;
      CRN(c.cU, k, i * 6 + j) =
          kn >= 0 ? KR[(i + 18 * (12 + j)) * ne] + (eR >= 0 ? ELM(c.ec, eR, i * 26 + 7 + j) : 0.0) : 0.0;
      CRN(c.cL, k, i * 6 + j) =
          kp >= 0 ? KL[((12 + i) + 18 * j) * ne] + (eL >= 0 ? ELM(c.ec, eL, i * 26 + 13 + 1 + j) : 0.0) : 0.0;
    }
    double r = P[g[i]];
    if (eL >= 0) r += ELM(c.ec, eL, i * 26 + 13);
    if (eR >= 0) r += ELM(c.ec, eR, i * 26);
    CRN(c.cb, k, i) = r;
  }
}

// ---- 3. cyclic reduction: eliminate odd positions ----
__global__ void __launch_bounds__(CT) k_cr_eliminate(Batch b, ChainData c, int lo, int hi) {
  int t = lo + blockIdx.x * CT + threadIdx.x;
  if (t >= hi) return;
  CrItem it = c.odd[t];
  if (!solving(b, it.structure)) return;
  int k = it.corner;
  double D[36];
#pragma unroll
  for (int q = 0; q < 36; ++q) D[q] = CRN(c.cD, k, q);
  double inv[6], mult[36];
  if (!gj6_factor(D, inv, mult)) b.state[it.structure].info_fail = 1;
  // Z = D^-1 [b | L | U], a column at a time
#pragma unroll 1
  for (int q = 0; q < 13; ++q) {
    double r[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      if (q == 0) r[i] = CRN(c.cb, k, i);
      else if (q < 7) r[i] = it.prev >= 0 ? CRN(c.cL, k, i * 6 + q - 1) : 0.0;
      else r[i] = it.next >= 0 ? CRN(c.cU, k, i * 6 + q - 7) : 0.0;
    }
    gj6_apply(inv, mult, r);
#pragma unroll
    for (int i = 0; i < 6; ++i) CRN(c.cz, k, i * 13 + q) = r[i];
  }
}

// Warp-per-item form of k_cr_eliminate for the small levels near the top of
// the reduction, where one item per thread would leave most of the FP64
// units idle: lane q holds column q of the augmented 6 x 19 matrix
// [D | b | L | U] in registers and the pivot column is broadcast by shuffle.
// The arithmetic is the same sequence as gj6_factor / gj6_apply (same products and
// FMAs on every entry), so both forms give the same bits.
__global__ void k_cr_eliminate_w(Batch b, ChainData c, int lo, int hi) {
  const int lane = threadIdx.x & 31;
  const int t = lo + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (t >= hi) return;
  CrItem it = c.odd[t];
  if (!solving(b, it.structure)) return;
  const int k = it.corner;
  double col[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double v = 0.0;
    if (lane < 6) v = CRN(c.cD, k, i * 6 + lane);
    else if (lane == 6) v = CRN(c.cb, k, i);
    else if (lane < 13) v = it.prev >= 0 ? CRN(c.cL, k, i * 6 + lane - 7) : 0.0;
    else if (lane < NC) v = it.next >= 0 ? CRN(c.cU, k, i * 6 + lane - 13) : 0.0;
    col[i] = v;
  }
  bool ok = true;
#pragma unroll
  for (int kk = 0; kk < 6; ++kk) {
    double p = __shfl_sync(0xffffffffu, col[kk], kk);
    if (!(p != 0.0) || !isfinite(p)) ok = false;
    double inv = recip(p);
    double m[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) m[i] = __shfl_sync(0xffffffffu, col[i], kk);
    if (lane > kk && lane < NC) {
      double rk = col[kk] * inv;
      col[kk] = rk;
#pragma unroll
      for (int i = 0; i < 6; ++i)
        if (i != kk) col[i] = fma(-m[i], rk, col[i]);
    }
  }
  if (!ok && lane == 0) b.state[it.structure].info_fail = 1;
  if (lane >= 6 && lane < NC)
#pragma unroll
    for (int i = 0; i < 6; ++i) CRN(c.cz, k, i * 13 + lane - 6) = col[i];
}

// ---- 3b. cyclic reduction: surviving positions absorb their neighbours ----
// D -= U ZL(next) + L ZU(prev);  b -= U Zb(next) + L Zb(prev);
// U <- -U ZU(next);  L <- -L ZL(prev)
__device__ __forceinline__ void cr_update_row(const ChainData& c, const CrItem& it, int i) {
  const int k = it.corner;
  const int zn = it.next, zp = it.prev;
  {
    double u[6], l[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      u[j] = CRN(c.cU, k, i * 6 + j);
      l[j] = CRN(c.cL, k, i * 6 + j);
    }
    double nb = CRN(c.cb, k, i), nD[6], nU[6], nL[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      nD[q] = CRN(c.cD, k, i * 6 + q);
      nU[q] = 0.0;
      nL[q] = 0.0;
    }
    if (zn >= 0) {
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        nb = fma(-u[j], CRN(c.cz, zn, j * 13), nb);
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          nD[q] = fma(-u[j], CRN(c.cz, zn, j * 13 + 1 + q), nD[q]);
          nU[q] = fma(-u[j], CRN(c.cz, zn, j * 13 + 7 + q), nU[q]);
        }
      }
    }
    if (zp >= 0) {
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        nb = fma(-l[j], CRN(c.cz, zp, j * 13), nb);
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          nD[q] = fma(-l[j], CRN(c.cz, zp, j * 13 + 7 + q), nD[q]);
          nL[q] = fma(-l[j], CRN(c.cz, zp, j * 13 + 1 + q), nL[q]);
        }
      }
    }
    CRN(c.cb, k, i) = nb;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      CRN(c.cD, k, i * 6 + q) = nD[q];
      CRN(c.cU, k, i * 6 + q) = nU[q];
      CRN(c.cL, k, i * 6 + q) = nL[q];
    }
  }
}

// Row per lane: six lanes per item (rows of the 6x6 blocks are
// independent), five items per warp.
__global__ void k_cr_update_w(Batch b, ChainData c, int lo, int hi) {
  const int lane = threadIdx.x & 31;
  if (lane >= 30) return;
  const int t = lo + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 5 + lane / 6;
  if (t >= hi) return;
  CrItem it = c.even[t];
  if (!solving(b, it.structure)) return;
  cr_update_row(c, it, lane % 6);
}

// ---- 3c. the last position of each chain ----
__global__ void __launch_bounds__(CT) k_cr_root(Batch b, ChainData c) {
  int t = blockIdx.x * CT + threadIdx.x;
  if (t >= c.n_roots) return;
  int k = c.roots[t];
  int s = c.corner_struct[k];
  if (!solving(b, s)) return;
  double D[36], r[6];
#pragma unroll
  for (int q = 0; q < 36; ++q) D[q] = CRN(c.cD, k, q);
#pragma unroll
  for (int i = 0; i < 6; ++i) r[i] = CRN(c.cb, k, i);
  double inv[6], mult[36];
  if (!gj6_factor(D, inv, mult)) b.state[s].info_fail = 1;
  gj6_apply(inv, mult, r);
#pragma unroll
  for (int i = 0; i < 6; ++i) CRN(c.cx, k, i) = r[i];
}

// ---- 4. back substitution: x = Zb - ZL x_prev - ZU x_next ----
// Row per lane: six lanes per item, five items per warp.
__global__ void k_cr_back(Batch b, ChainData c, int lo, int hi) {
  const int lane = threadIdx.x & 31;
  if (lane >= 30) return;
  const int t = lo + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 5 + lane / 6;
  if (t >= hi) return;
  CrItem it = c.odd[t];
  if (!solving(b, it.structure)) return;
  const int k = it.corner, i = lane % 6;
  double x = CRN(c.cz, k, i * 13);
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double xp = it.prev >= 0 ? CRN(c.cx, it.prev, j) : 0.0;
    double xn = it.next >= 0 ? CRN(c.cx, it.next, j) : 0.0;
    x = fma(-CRN(c.cz, k, i * 13 + 1 + j), xp, x);
    x = fma(-CRN(c.cz, k, i * 13 + 7 + j), xn, x);
  }
  CRN(c.cx, k, i) = x;
}

// ---- 4b. midside nodes, and the solution into P ----
__global__ void k_chain_scatter(Batch b, ChainData c) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= c.n_chain_elems) return;
  int e = c.elem_list[t];
  int s = b.estruct[e];
  if (!solving(b, s)) return;
  const StructInfo inf = b.info[s];
  double* P = b.P + inf.dof_off;
  int ka = c.elem_corner_a[t], kb = c.elem_corner_b[t];
  double xa[6], xb[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    xa[j] = ka >= 0 ? CRN(c.cx, ka, j) : 0.0;
    xb[j] = kb >= 0 ? CRN(c.cx, kb, j) : 0.0;
  }
  int nm = b.enodes[3 * e + 1];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double x = ELM(c.ez, t, i * 13);
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      x = fma(-ELM(c.ez, t, i * 13 + 1 + j), xa[j], x);
      x = fma(-ELM(c.ez, t, i * 13 + 7 + j), xb[j], x);
    }
    P[b.gl[(int64_t)nm * 6 + i]] = x;
  }
}

__global__ void k_corner_scatter(Batch b, ChainData c) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= c.n_corners) return;
  int s = c.corner_struct[k];
  if (!solving(b, s)) return;
  const StructInfo inf = b.info[s];
  double* P = b.P + inf.dof_off;
  int node = c.corner_node[k];
#pragma unroll
  for (int i = 0; i < 6; ++i) P[b.gl[(int64_t)node * 6 + i]] = CRN(c.cx, k, i);
}

}  // namespace

void launch_chain_solve(const Batch& b, const ChainData& c, cudaStream_t st) {
  if (c.n_chain_elems == 0) return;
  k_condense<<<(c.n_chain_elems + CT - 1) / CT, CT, 0, st>>>(b, c);
  if (c.n_corners > 0) {
    k_corner_system<<<(c.n_corners + 127) / 128, 128, 0, st>>>(b, c);
    // levels with fewer items than ~8 per FP64 unit take the lane-parallel
    // forms (same results, shorter per-item instruction chains)
    const int small = 152 * 4 * 8;
    for (int l = 0; l < c.n_levels; ++l) {
      int lo = c.odd_off[l], hi = c.odd_off[l + 1];
      if (hi - lo >= small) k_cr_eliminate<<<(hi - lo + CT - 1) / CT, CT, 0, st>>>(b, c, lo, hi);
      else if (hi > lo) k_cr_eliminate_w<<<(hi - lo + 3) / 4, 128, 0, st>>>(b, c, lo, hi);
      // the update runs row-per-lane at every level: the same FP64
      // instruction count as one item per thread, six times the warps
      int elo = c.even_off[l], ehi = c.even_off[l + 1];
      if (ehi > elo) k_cr_update_w<<<(ehi - elo + 19) / 20, 128, 0, st>>>(b, c, elo, ehi);
    }
    k_cr_root<<<(c.n_roots + CT - 1) / CT, CT, 0, st>>>(b, c);
    for (int l = c.n_levels - 1; l >= 0; --l) {
      int lo = c.odd_off[l], hi = c.odd_off[l + 1];
      if (hi > lo) k_cr_back<<<(hi - lo + 19) / 20, 128, 0, st>>>(b, c, lo, hi);
    }
    k_corner_scatter<<<(c.n_corners + 127) / 128, 128, 0, st>>>(b, c);
  }
  k_chain_scatter<<<(c.n_chain_elems + 127) / 128, 128, 0, st>>>(b, c);
}

}  // namespace gf
