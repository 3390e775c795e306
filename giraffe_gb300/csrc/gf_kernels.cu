// Device-resident Newton loop for batches of Beam_1 structures (see
// gf_kernels.cuh for the pass structure and the reference lines each kernel
// follows).
#include <cuda_runtime.h>

#include "gf_beam.cuh"
#include "gf_df64.cuh"
#include "gf_chain.cuh"
#include "../../include/giraffe_model.h"
#include "gf_kernels.cuh"

namespace gf {

namespace {

__device__ __forceinline__ bool iterating(const StructState& s) { return s.phase == PH_ITER; }

__device__ __forceinline__ double table_at(const Batch& b, int t, double time, int col) {
  const TableDev T = b.tables[t];
  const double* times = b.table_data + T.off;
  const double* vals = times + T.n_times;
  if (T.n_times == 0) return 0.0;
  if (time >= times[T.n_times - 1]) return vals[(T.n_times - 1) * T.n_cols + col];
  if (time <= times[0]) return vals[col];
  int idx = 0;
  while (time >= times[idx]) idx++;
  double f = (time - times[idx - 1]) / (times[idx] - times[idx - 1]);
  double a = vals[(idx - 1) * T.n_cols + col], c = vals[idx * T.n_cols + col];
  return a + f * (c - a);
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_or(int v) { return __any_sync(0xffffffffu, v); }

// Block-wide max of two values and an "any" flag (blockDim.x <= 1024).
struct Red3 { double a, b; int f; };
__device__ Red3 block_red(Red3 v) {
  __shared__ double sa[32], sb[32];
  __shared__ int sf[32];
  v.a = warp_max(v.a);
  v.b = warp_max(v.b);
  v.f = warp_or(v.f);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sa[w] = v.a; sb[w] = v.b; sf[w] = v.f; }
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  if (w == 0) {
    v.a = l < nw ? sa[l] : 0.0;
    v.b = l < nw ? sb[l] : 0.0;
    v.f = l < nw ? sf[l] : 0;
    v.a = warp_max(v.a);
    v.b = warp_max(v.b);
    v.f = warp_or(v.f);
    if (l == 0) { sa[0] = v.a; sb[0] = v.b; sf[0] = v.f; }
  }
  __syncthreads();
  Red3 r{sa[0], sb[0], sf[0]};
  __syncthreads();
  return r;
}

__device__ __forceinline__ bool nan_or_huge(double v) { return !(v == v) || v >= 1e300 || v <= -1e300; }

// ---- reductions of one structure spread over several CTAs ----
__device__ __forceinline__ int red_chunks(const StructInfo& inf) {
  return inf.n_free > 0 ? (inf.n_free + GF_RED_CHUNK - 1) / GF_RED_CHUNK : 1;
}
// Max of non-negative doubles through their bit patterns (exact, so the
// result does not depend on the order in which CTAs arrive).
__device__ __forceinline__ void red_max(unsigned long long* p, double v) {
  atomicMax(p, (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ double red_value(const unsigned long long* p) {
  return __longlong_as_double((long long)*(volatile const unsigned long long*)p);
}
// Counts this CTA in; true in every thread of the CTA that arrives last, to
// which the other CTAs' global writes are then visible (each thread fences
// its own writes before the count).
__device__ bool red_arrive(RedScratch& r, int n_chunks) {
  __shared__ int last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&r.ticket, 1) == n_chunks - 1;
  __syncthreads();
  if (last) __threadfence();
  return last;
}

// UpdateDyn for one node (reference src/Dynamic.cpp:480-580): Newmark
// velocity and acceleration of the free DOFs; the rotational ones are
// transported by Q_delta.  Nodes have all rotations free or all fixed
// (checked on the host), so the rotational vectors are complete.
__device__ void update_dyn_node(const Batch& b, const double* a, int node) {
  const int64_t o = (int64_t)node * 6;
  const int* gl = b.gl + o;
  const double* d = b.disp + o;
#pragma unroll
  for (int j = 0; j < 3; ++j)
    if (gl[j] >= 0) {
      b.vel[o + j] = d[j] * a[3] + b.copy_vel[o + j] * a[4] + b.copy_accel[o + j] * a[5];
      b.accel[o + j] = d[j] * a[0] - b.copy_vel[o + j] * a[1] - b.copy_accel[o + j] * a[2];
    }
  if (gl[3] >= 0 || gl[4] >= 0 || gl[5] >= 0) {
    V3<double> al = {{d[3], d[4], d[5]}}, va, aa;
    for (int j = 0; j < 3; ++j) {
      va[j] = d[3 + j] * a[3] + b.copy_vel[o + 3 + j] * a[4] + b.copy_accel[o + 3 + j] * a[5];
      aa[j] = d[3 + j] * a[0] - b.copy_vel[o + 3 + j] * a[1] - b.copy_accel[o + 3 + j] * a[2];
    }
    M3<double> Qd = rodrigues(al);
    va = mv(Qd, va);
    aa = mv(Qd, aa);
    for (int j = 0; j < 3; ++j)
      if (gl[3 + j] >= 0) {
        b.vel[o + 3 + j] = va[j];
        b.accel[o + 3 + j] = aa[j];
      }
  }
}

// ---------------------------------------------------------------------------
// initial state: the first solution step (reference src/Static.cpp:140-170)
__global__ void k_init_state(Batch b) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= b.n_struct) return;
  const StructParams p = b.step_params[b.info[s].step_off];
  b.params[s] = p;
  StructState& st = b.state[s];
  StructState z = {};
  z.phase = PH_START;
  z.time = p.start_time;
  z.time_step = p.time_step0;
  z.last_converged_time = p.start_time;
  st = z;
}

// reference src/Static.cpp:176-197 (+ NodalDisplacement::Mount, EulerAngles)
__global__ void k_step_begin(Batch b) {
  int s = blockIdx.x;
  StructState& st = b.state[s];
  __shared__ int go, zero_va;
  if (threadIdx.x == 0) {
    if (s == 0) *b.running = 0;
    go = st.phase == PH_START;
    zero_va = go && st.zero_va;
    if (go) {
      st.zero_va = 0;
      const StructParams& p = b.params[s];
      if (st.host_step) {
        // gf_begin_step: the caller's Static::Solve / Dynamic::Solve loop
        // advanced the time itself
        st.time_step = st.current_time_step;
        st.time = st.last_converged_time + st.current_time_step;
      } else {
        st.last_converged_time = st.time;
        st.time += st.time_step;
        if (st.time > 0.99999999 * p.end_time) {
          st.time = p.end_time;
          st.time_step = p.end_time - st.last_converged_time;
        }
        st.current_time_step = st.time_step;
      }
      if (p.dynamic) {
        // reference src/Dynamic.cpp:582-590
        double dt = st.time_step;
        st.a[0] = 1.0 / (dt * dt * p.beta);
        st.a[1] = 1.0 / (dt * p.beta);
        st.a[2] = 1.0 / (2.0 * p.beta) - 1.0;
        st.a[3] = p.gamma / (dt * p.beta);
        st.a[4] = 1.0 - p.gamma / p.beta;
        st.a[5] = dt * (1.0 - p.gamma / (2.0 * p.beta));
      }
      st.it = 1;
      st.res_conv = 0;
      st.gl_conv = 0;
      st.diverged = 0;
      st.info_fail = 0;
      st.phase = PH_ITER;
    }
  }
  __syncthreads();
  if (!go) return;
  const StructInfo inf = b.info[s];
  const bool dyn = b.params[s].dynamic;
  for (int i = threadIdx.x; i < inf.n_nodes * 6; i += blockDim.x) {
    int64_t q = (int64_t)inf.node_off * 6 + i;
    b.disp[q] = 0.0;
    if (zero_va) b.vel[q] = b.accel[q] = b.copy_vel[q] = b.copy_accel[q] = 0.0;
    if (dyn) {  // back to the converged velocities (a no-op after a commit)
      b.vel[q] = b.copy_vel[q];
      b.accel[q] = b.copy_accel[q];
    }
  }
  __syncthreads();
  double time = st.last_converged_time + st.current_time_step, dt = st.current_time_step;
  for (int e = threadIdx.x; e < b.n_disps; e += blockDim.x) {
    const DispEntry D = b.disps[e];
    if (D.structure != s) continue;
    int node = D.node;
    const int* cons = b.cons + (int64_t)node * 6;
    const int* gl = b.gl + (int64_t)node * 6;
    double dl[3], dg[3];
    for (int j = 0; j < 3; ++j) dl[j] = table_at(b, D.table, time, j) - table_at(b, D.table, time - dt, j);
    for (int j = 0; j < 3; ++j) dg[j] = D.CQ[j] * dl[0] + D.CQ[3 + j] * dl[1] + D.CQ[6 + j] * dl[2];
    for (int j = 0; j < 3; ++j)
      if (cons[j] == 1 && gl[j] == -1) {
        int64_t q = (int64_t)node * 6 + j;
        b.disp[q] = dg[j];
        if (dyn) {
          b.vel[q] = dg[j] / dt;
          b.accel[q] = (b.vel[q] - b.copy_vel[q]) / dt;
        }
      }
    double phi = cons[3] == 1 ? table_at(b, D.table, time, 3) : 0.0;
    double th = cons[4] == 1 ? table_at(b, D.table, time, 4) : 0.0;
    double psi = cons[5] == 1 ? table_at(b, D.table, time, 5) : 0.0;
    M3<double> Q;
    if (D.angular == GF_ANGLES_VECTOR) {
      // Euler rotation vector (phi, th, psi): Rodrigues parameters of length
      // 2 tan(|e| / 2) along e (reference src/NodalDisplacement.cpp:330-350)
      const double en = sqrt(phi * phi + th * th + psi * psi);
      const double inv = en != 0.0 ? 1.0 / en : 0.0;
      const double rod = 2.0 * tan(en / 2.0);
      const V3<double> r = {{rod * (inv * phi), rod * (inv * th), rod * (inv * psi)}};
      const M3<double> A = skew(r), A2 = mul(A, A);
      const double g = 4.0 / (4.0 + rod * rod);
      for (int k = 0; k < 9; ++k) Q[k] = g * (A[k] + 0.5 * A2[k]);
      Q[0] += 1.0;
      Q[4] += 1.0;
      Q[8] += 1.0;
    } else {
      Q[0] = cos(th) * cos(psi);
      Q[1] = sin(phi) * sin(th) * cos(psi) - cos(phi) * sin(psi);
      Q[2] = cos(phi) * sin(th) * cos(psi) + sin(phi) * sin(psi);
      Q[3] = cos(th) * sin(psi);
      Q[4] = sin(phi) * sin(th) * sin(psi) + cos(phi) * cos(psi);
      Q[5] = cos(phi) * sin(th) * sin(psi) - sin(phi) * cos(psi);
      Q[6] = -sin(th);
      Q[7] = sin(phi) * cos(th);
      Q[8] = cos(phi) * cos(th);
    }
    M3<double> CQ, Qi;
    for (int k = 0; k < 9; ++k) { CQ[k] = D.CQ[k]; Qi[k] = b.Qn[(int64_t)node * 9 + k]; }
    Q = tmul(CQ, mul(Q, CQ));
    M3<double> Qd = mul(Q, transpose(Qi));
    double tr = Qd[0] + Qd[4] + Qd[8];
    if (tr > 3.0) tr = 3.0;
    double ax[3] = {0.5 * (Qd[7] - Qd[5]), 0.5 * (Qd[2] - Qd[6]), 0.5 * (Qd[3] - Qd[1])};
    double al = 2.0 * sqrt((3.0 - tr) / (1.0 + tr));
    double theta = 2.0 * asin(sqrt((3.0 - tr) / 4.0));
    double eu = theta != 0.0 ? theta / sin(theta) : 0.0;
    for (int j = 3; j < 6; ++j)
      if (cons[j] == 1 && gl[j] == -1) {
        int64_t q = (int64_t)node * 6 + j;
        b.disp[q] = ((4.0 + al * al) / 4.0) * ax[j - 3];
        if (dyn) {
          b.vel[q] = eu * ax[j - 3] / dt;
          b.accel[q] = (b.vel[q] - b.copy_vel[q]) / dt;
        }
      }
  }
  if (dyn) {
    __syncthreads();
    for (int i = threadIdx.x; i < inf.n_nodes; i += blockDim.x) update_dyn_node(b, st.a, inf.node_off + i);
  }
}

// clear band and P of iterating structures
__global__ void k_zero(Batch b) {
  int s = blockIdx.y;
  if (!iterating(b.state[s])) return;
  const StructInfo inf = b.info[s];
  // wide structures: k_wb_zero; chain structures keep no band (nodeK instead)
  const bool chain_only = inf.is_chain && !b.full_band;
  int64_t nb = (inf.wide || chain_only) ? 0 : (int64_t)inf.n_free * GF_LDB;
  if (inf.is_chain) {
    double* nk = b.nodeK + (int64_t)inf.node_off * 9;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < inf.n_nodes * 9; i += gridDim.x * blockDim.x) nk[i] = 0.0;
  }
  double* band = b.band + inf.band_off;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x)
    band[i] = 0.0;
  double* P = b.P + inf.dof_off;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < inf.n_free; i += gridDim.x * blockDim.x) P[i] = 0.0;
}

// ---------------------------------------------------------------------------
// Beam_1 Mount + MountElementLoads (k_beam_tangent) and MountGlobal
// (k_beam_scatter).
//
// k_beam_tangent: one thread per element, every element of every iterating
// structure.  The two rotated Gauss-point operators live in shared memory
// ([g][entry][thread], conflict-free); the 18x18 tangent (column-major) and
// the 18 internal forces go to per-element scratch.  Keeping the band
// read-modify-write out of this FP64-bound kernel keeps global-load latency
// off its dependency chains.
// k_beam_scatter: one warp per element of one colour class; lanes walk the
// 324 tangent entries in column order, so the band updates of a column are
// contiguous.  Elements of one colour share no node, so the scatter needs no
// atomics and is deterministic.
constexpr int MOUNT_THREADS = 64;
// per thread: the two operators (OP_N stored entries each) and the internal
// force (18), so three CTAs fit on an SM; the inertial rotational tangents
// of Dynamic steps go to the element scratch b.Dm instead
constexpr int MOUNT_SMEM = (2 * OP_N + 18) * MOUNT_THREADS * (int)sizeof(double);

template <typename TK>
__global__ void __launch_bounds__(MOUNT_THREADS) k_beam_tangent(Batch b) {
  extern __shared__ unsigned char smem_raw[];
  TK* sM = reinterpret_cast<TK*>(smem_raw);
  const int tid = threadIdx.x;
  int e = blockIdx.x * MOUNT_THREADS + tid;
  if (e >= b.n_elem) return;
  int s = b.estruct[e];
  if (!iterating(b.state[s])) return;
  const BeamConst& c = b.bconst[e];
  const BeamHist& h = b.bhist[e];
  int nd[3] = {b.enodes[3 * e], b.enodes[3 * e + 1], b.enodes[3 * e + 2]};
  double d[18];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int q = 0; q < 6; ++q) d[6 * j + q] = b.disp[(int64_t)nd[j] * 6 + q];
  BeamInterp ip[2] = {beam_interp(c, d, 0), beam_interp(c, d, 1)};
  double* f = reinterpret_cast<double*>(sM + (size_t)2 * OP_N * MOUNT_THREADS) + tid;
  // inertial rotational tangents, 2 x 9, structure-of-arrays like K_e
  double* Dm = b.Dm + e;
  const int64_t dms = b.n_elem;
#pragma unroll
  for (int q = 0; q < 18; ++q) f[q * MOUNT_THREADS] = 0.0;
  const StructParams& pr = b.params[s];
  const bool dyn = pr.dynamic;
  const double* an = b.state[s].a;
#pragma unroll 1
  for (int g = 0; g < 2; ++g) {
    BeamGP kin;
    beam_kinematics(c, h, ip[g], g, kin);
    beam_gp_force(c, kin, g, f, MOUNT_THREADS);
    TK* M = sM + (size_t)g * OP_N * MOUNT_THREADS + tid;
    if constexpr (std::is_same<TK, double>::value) {
      beam_gp_operator<TK>(c, kin, M, MOUNT_THREADS);
      rotate_blocks9<TK>(c, M, MOUNT_THREADS);
    } else {
      // mixed precision: the operator in FP64, rounded to TK in place (a TK
      // is as wide as a double), then its rotation and the K_e expansion in
      // TK.  (Expanding in a kernel of its own, with many warps per SM, gains
      // nothing here: its FP64 <-> FP32-pair conversions take the FP64 pipe
      // as long as the products it moves off it.)
      static_assert(sizeof(TK) == sizeof(double), "operator storage");
      double* Md = reinterpret_cast<double*>(M);
      beam_gp_operator<double>(c, kin, Md, MOUNT_THREADS);
#pragma unroll 1
      for (int q = 0; q < OP_N; ++q) {
        const double v = Md[q * MOUNT_THREADS];
        M[q * MOUNT_THREADS] = TK(v);
      }
      rotate_blocks9<TK>(c, M, MOUNT_THREADS);
    }
  }
  double a1Mr = 0.0;
  if (dyn) {
    // MountMass + MountDyn: inertial force and mass/gyroscopic tangent
    double vel[18], acc[18];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        vel[6 * j + q] = b.copy_vel[(int64_t)nd[j] * 6 + q];
        acc[6 * j + q] = b.copy_accel[(int64_t)nd[j] * 6 + q];
      }
    double a6[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) a6[q] = an[q];
    const BeamHistAux& x = b.baux[e];
#pragma unroll 1
    for (int g = 0; g < 2; ++g)
      beam_gp_inertia(c, x, ip[g], vel, acc, a6, g, f, MOUNT_THREADS, Dm + (int64_t)g * 9 * dms, (int)dms);
    a1Mr = a6[0] * c.Mr;
  }
  // element scratch is structure-of-arrays (entry x of element e at
  // [x * n_elem + e]): the writes of a warp and the per-item reads of the
  // chain solver are coalesced
  double* Ke = b.Ke + e;
  const int64_t ne = b.n_elem;

#pragma unroll 1
  for (int J = 0; J < 3; ++J)
#pragma unroll 1
    for (int I = 0; I < 3; ++I)
      beam_K_block<TK>(c, sM + tid, sM + OP_N * MOUNT_THREADS + tid, I, J, MOUNT_THREADS, Ke, dyn, Dm,
                       Dm + 9 * dms, (int)dms, a1Mr, ne);
  // Rayleigh damping: on the iterations that form C_e, the stiffness part
  // of K_e alone (no inertial terms) goes to the damping scratch, where
  // k_beam_rayleigh turns it into C_e = alpha M_modal + beta K_e
  if (dyn && pr.ray_on && (pr.ray_update || !b.state[s].ray_init)) {
    double* Ce = b.RD + e;
#pragma unroll 1
    for (int J = 0; J < 3; ++J)
#pragma unroll 1
      for (int I = 0; I < 3; ++I)
        beam_K_block<TK>(c, sM + tid, sM + OP_N * MOUNT_THREADS + tid, I, J, MOUNT_THREADS, Ce, false, Dm,
                         Dm + 9 * dms, (int)dms, 0.0, ne);
  }
#pragma unroll
  for (int q = 0; q < 18; ++q) b.Fe[q * ne + e] = f[q * MOUNT_THREADS];
}

// MountDamping and the damping part of MountDyn (reference
// src/Beam_1.cpp:1641-1673).  On the iterations that form it (the step's
// first, or every one with Update 1), C_e = alpha M_modal + beta K_e; the
// modal mass is MountMassModal (src/Beam_1.cpp:1538-1553) with the
// EvaluateMassModal operator (src/Beam_1.cpp:1681-1774) of a section
// without a first moment of mass, blockdiag(Q Mr Q^T, Q Jr Q^T) with
// Q = Q(alpha_i) at each Gauss point, summed as wJ N^T D N (w = 1) and
// turned to the global frame block by block (T3^T B T3).  Every iteration
// then adds a4 C_e to K_e and C_e v to f_e, v the nodes' current
// velocities.  One thread per element; C_e is structure-of-arrays like K_e.
// The modal mass of a Beam_1 / Pipe_1 element: per Gauss point D[g][0] =
// Q Mr Q^T and D[g][1] = Q Jr Q^T (3x3 row-major) with Q = Q(alpha_i).
__device__ void beam_modal_D(const BeamConst& c, const BeamHistAux& x, double (*D)[2][9]) {
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    M3<double> Q = rodrigues(V3<double>{{x.alpha[g][0], x.alpha[g][1], x.alpha[g][2]}});
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        double mt = 0.0, jt = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          double qm = 0.0, qj = 0.0;
#pragma unroll
          for (int l = 0; l < 3; ++l) {
            qm += Q[i * 3 + l] * (l == k ? c.Mr : 0.0);
            qj += Q[i * 3 + l] * c.Jr[l * 3 + k];
          }
          mt += qm * Q[j * 3 + k];
          jt += qj * Q[j * 3 + k];
        }
        D[g][0][i * 3 + j] = mt;
        D[g][1][i * 3 + j] = jt;
      }
  }
}

// Block (node I, node J, translation/rotation bi, bj) of the element's modal
// mass in the global frame, 3x3 row-major: sum_g jac N_gI N_gJ D[g][bi]
// turned by T^T (.) T on the diagonal blocks bi == bj, zero off them.
__device__ void beam_modal_block(const BeamConst& c, const double (*D)[2][9], int I, int J, int bi, int bj,
                                 double* m) {
#pragma unroll
  for (int q = 0; q < 9; ++q) m[q] = 0.0;
  if (bi != bj) return;
  const double* T = c.T3;
  double loc[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    loc[q] = 0.0;
#pragma unroll
    for (int g = 0; g < 2; ++g) loc[q] += ((c.jac * c.N[g][I]) * D[g][bi][q]) * c.N[g][J];
  }
  double t2[9];  // loc T, then T^T (loc T)
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) t2[i * 3 + j] = loc[i * 3] * T[j] + loc[i * 3 + 1] * T[3 + j] + loc[i * 3 + 2] * T[6 + j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) m[i * 3 + j] = T[i] * t2[j] + T[3 + i] * t2[3 + j] + T[6 + i] * t2[6 + j];
}

__global__ void k_beam_rayleigh(Batch b) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= b.n_elem) return;
  const int s = b.estruct[e];
  const StructState& st = b.state[s];
  if (!iterating(st)) return;
  const StructParams& p = b.params[s];
  if (!p.dynamic || !p.ray_on) return;
  const int64_t ne = b.n_elem;
  double* C = b.RD + e;
  if (p.ray_update || !st.ray_init) {
    const BeamConst& c = b.bconst[e];
    double D[2][2][9];  // [Gauss point][translation, rotation][3x3 row-major]
    beam_modal_D(c, b.baux[e], D);
#pragma unroll 1
    for (int I = 0; I < 3; ++I)
#pragma unroll 1
      for (int J = 0; J < 3; ++J)
#pragma unroll 1
        for (int bi = 0; bi < 2; ++bi)
#pragma unroll 1
          for (int bj = 0; bj < 2; ++bj) {
            double m[9];
            beam_modal_block(c, D, I, J, bi, bj, m);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
              for (int j = 0; j < 3; ++j) {
                const int64_t xi = (6 * I + 3 * bi + i) + 18 * (6 * J + 3 * bj + j);
                C[xi * ne] = p.ray_alpha * m[i * 3 + j] + p.ray_beta * C[xi * ne];
              }
          }
  }
  const double a4 = st.a[3];
  double v[18];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const int64_t nd = b.enodes[3 * e + j];
#pragma unroll
    for (int q = 0; q < 6; ++q) v[6 * j + q] = b.vel[nd * 6 + q];
  }
#pragma unroll 1
  for (int q = 0; q < 18; ++q) {
    double acc = 0.0;
#pragma unroll 1
    for (int k = 0; k < 18; ++k) {
      const double cq = C[(int64_t)(q + 18 * k) * ne];
      acc += cq * v[k];
      b.Ke[(int64_t)(q + 18 * k) * ne + e] += a4 * cq;
    }
    b.Fe[(int64_t)q * ne + e] += acc;
  }
}

// Pipe_1::MountPipeSpecialLoads (reference src/Pipe_1.cpp:1441-1494): the
// internal pressure p0i of a PipeLoad acting on the internal area Aint, at
// the current iterate.  At each Gauss point, with Q = Q_delta Q_i,
// kappa = Q kappa_r and e3 = Q e3r (element frame), the line load
// (f, m) = -p0i Aint (kappa x e3, Xi^T (z' x e3)) and its stiffness Kext
// (6 x 12 on (u, alpha, u', alpha'): K1ua, K1aa, K2ua, K2au) enter as
// f_e -= jac T^T N^T (f, m) and K_e -= jac p0i Aint T^T N^T Kext Upsilon T.
// Its O1 term reads the element's scalar g, which the reference's Mount
// leaves at the second Gauss point's value (src/Pipe_1.cpp:890), for both
// points.  One thread per pressurized element, after k_beam_tangent has
// written K_e and f_e and before k_beam_rayleigh: in a Dynamic step the
// reference mounts loads before damping, so on the iterations that form
// C_e the load stiffness also goes into the stiffness part that C_e is
// made from.
__global__ void k_pipe_pressure(Batch b) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= b.n_pipe_press) return;
  const int e = b.pp_elem[q];
  const int s = b.estruct[e];
  const StructState& st = b.state[s];
  if (!iterating(st)) return;
  const StructParams& pr = b.params[s];
  const bool form_c = pr.dynamic && pr.ray_on && (pr.ray_update || !st.ray_init);
  const double p0i = table_at(b, b.pp_table[q], st.last_converged_time + st.current_time_step, 0);
  const double Aint = b.pp_aint[q];
  const BeamConst& c = b.bconst[e];
  const BeamHist& h = b.bhist[e];
  double d[18];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const int64_t nd = b.enodes[3 * e + j];
#pragma unroll
    for (int k = 0; k < 6; ++k) d[6 * j + k] = b.disp[nd * 6 + k];
  }
  M3<double> T;
#pragma unroll
  for (int i = 0; i < 9; ++i) T[i] = c.T3[i];
  const V3<double> e3r = {{c.e3r[0], c.e3r[1], c.e3r[2]}};
  const BeamInterp ip1 = beam_interp(c, d, 1);
  const double g_last = 4.0 / (4.0 + dot(ip1.alpha, ip1.alpha));
  const double pa = -p0i * Aint, sK = c.jac * p0i * Aint;
  const int64_t ne = b.n_elem;
  double* Ke = b.Ke + e;
  double* Fe = b.Fe + e;
  double* Ce = form_c ? b.RD + e : nullptr;
#pragma unroll 1
  for (int g = 0; g < 2; ++g) {
    const BeamInterp ip = beam_interp(c, d, g);
    double gg;
    M3<double> Qd, Xi, Qi;
    beam_rot(ip.alpha, gg, Qd, Xi);
    const M3<double> dA = skew(ip.dalpha);
    const double ad = dot(ip.alpha, ip.dalpha);
    M3<double> dXi;
#pragma unroll
    for (int i = 0; i < 9; ++i) dXi[i] = -0.5 * gg * (ad * Xi[i] - dA[i]);
#pragma unroll
    for (int i = 0; i < 9; ++i) Qi[i] = h.Q[g][i];
    V3<double> dz;
#pragma unroll
    for (int i = 0; i < 3; ++i) dz[i] = ip.du[i] + h.dz[g][i];
    const M3<double> Q = mul(Qd, Qi);
    V3<double> kap = tmv(Qi, tmv(Xi, ip.dalpha));
#pragma unroll
    for (int i = 0; i < 3; ++i) kap[i] += h.kap[g][i];
    const V3<double> kip = mv(Q, kap), e3 = mv(Q, e3r);
    const V3<double> fl = cross(kip, e3), ml = tmv(Xi, cross(dz, e3));
    const M3<double> E3 = skew(e3), Kp = skew(kip), dZ = skew(dz);
    const V3<double> c2 = cross(e3, dz), w = tmv(Xi, c2);
    const M3<double> S2 = skew(c2);
    const M3<double> A1 = mul(mul(Kp, E3), Xi), A2 = mul(E3, dXi), A3 = mul(mul(E3, Kp), Xi);
    const M3<double> B1 = tmul(Xi, mul(mul(dZ, E3), Xi));
    M3<double> K1ua, K1aa;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        K1ua[i * 3 + j] = A1[i * 3 + j] + A2[i * 3 + j] - A3[i * 3 + j];
        K1aa[i * 3 + j] = -0.5 * g_last * (w[i] * ip.alpha[j] - S2[i * 3 + j]) + B1[i * 3 + j];
      }
    // blocks of Kext in the global frame: T^T X T
    const M3<double> G1 = tmul(T, mul(K1ua, T)), G2 = tmul(T, mul(mul(E3, Xi), T));
    const M3<double> G3 = tmul(T, mul(tmul(Xi, E3), T)), G4 = tmul(T, mul(K1aa, T));
    const V3<double> fg = tmv(T, fl), mg = tmv(T, ml);
#pragma unroll 1
    for (int a = 0; a < 3; ++a) {
      const double Na = c.N[g][a];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        Fe[(int64_t)(6 * a + i) * ne] -= c.jac * Na * (pa * fg[i]);
        Fe[(int64_t)(6 * a + 3 + i) * ne] -= c.jac * Na * (pa * mg[i]);
      }
#pragma unroll 1
      for (int n = 0; n < 3; ++n) {
        const double Nb = c.N[g][n], dNb = c.dN[g][n];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const int x = i * 3 + j;
            // (u_a, alpha_b): K1ua Nb + K2ua dNb; (alpha_a, u_b): K2au dNb;
            // (alpha_a, alpha_b): K1aa Nb
            const int64_t x1 = (6 * a + i) + 18 * (6 * n + 3 + j), x2 = (6 * a + 3 + i) + 18 * (6 * n + j),
                          x3 = (6 * a + 3 + i) + 18 * (6 * n + 3 + j);
            const double v1 = sK * (Na * (Nb * G1[x] + dNb * G2[x])), v2 = sK * (Na * (dNb * G3[x])),
                         v3 = sK * (Na * (Nb * G4[x]));
            Ke[x1 * ne] -= v1;
            Ke[x2 * ne] -= v2;
            Ke[x3 * ne] -= v3;
            if (Ce) {
              Ce[x1 * ne] -= v1;
              Ce[x2 * ne] -= v2;
              Ce[x3 * ne] -= v3;
            }
          }
      }
    }
  }
}

// The modal mass of every Beam_1 / Pipe_1 element of colour class `color`
// added into the band M (entry (i, j) at (kw + i - j) + j W, free indices of
// b.gl): one thread per element, elements of a colour share no node.
__global__ void k_modal_mass_beam(Batch b, int color, double* M, int64_t W, int kw) {
  const int k = b.color_off[color] + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= b.color_off[color + 1]) return;
  const int e = b.color_elems[k];
  const BeamConst& c = b.bconst[e];
  double D[2][2][9];
  beam_modal_D(c, b.baux[e], D);
  int g[18];
#pragma unroll
  for (int a = 0; a < 18; ++a) g[a] = b.gl[(int64_t)b.enodes[3 * e + a / 6] * 6 + a % 6];
#pragma unroll 1
  for (int I = 0; I < 3; ++I)
#pragma unroll 1
    for (int J = 0; J < 3; ++J)
#pragma unroll 1
      for (int bi = 0; bi < 2; ++bi) {
        double m[9];
        beam_modal_block(c, D, I, J, bi, bi, m);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const int gr = g[6 * I + 3 * bi + i], gq = g[6 * J + 3 * bi + j];
            if (gr >= 0 && gq >= 0 && abs(gr - gq) <= kw) M[(kw + gr - gq) + (int64_t)gq * W] += m[i * 3 + j];
          }
      }
}

__global__ void k_beam_scatter(Batch b, int color) {
  int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  int k = b.color_off[color] + w;
  if (k >= b.color_off[color + 1]) return;
  int e = b.color_elems[k];
  int s = b.estruct[e];
  if (!iterating(b.state[s])) return;
  const StructInfo inf = b.info[s];
  int myg = -1;
  if (lane < 18) myg = b.gl[(int64_t)b.enodes[3 * e + lane / 6] * 6 + lane % 6];
  if (inf.is_chain && !b.full_band) {
    // the chain solver reads K_e directly; only the residual is assembled
    if (lane < 18 && myg >= 0) b.P[inf.dof_off + myg] += b.Fe[(int64_t)lane * b.n_elem + e];
    return;
  }
  const double* Ke = b.Ke + e;
  const int64_t ne = b.n_elem;
  double* band = b.band + inf.band_off;
  // uniform trip count: every lane takes part in every shuffle
  for (int base = 0; base < 324; base += 32) {
    int idx = base + lane;
    bool valid = idx < 324;
    int r = valid ? idx % 18 : 0, q = valid ? idx / 18 : 0;
    int gr = __shfl_sync(0xffffffffu, myg, r);
    int gq = __shfl_sync(0xffffffffu, myg, q);
    if (valid && gr >= 0 && gq >= 0) band[(GF_KB + gr - gq) + (int64_t)gq * GF_LDB] += Ke[idx * ne];
  }
  if (lane < 18 && myg >= 0) b.P[inf.dof_off + myg] += b.Fe[(int64_t)lane * ne + e];
}

// MountGlobal of the internal forces when every Beam_1 element of the batch
// belongs to a chain and no band is filled (the chain solver reads K_e from
// the element scratch): one thread per node DOF gathers the forces of the one
// or two elements on its node in a single launch, in place of the two colour
// passes of k_beam_scatter.  Chain element e of a structure sits on its local
// nodes 2e, 2e+1, 2e+2.  k_zero has just cleared P, so the sum (0 + f_a) + f_b
// formed here equals the colour-ordered scatter's, whichever element's colour
// comes first (IEEE addition is commutative).
__global__ void k_chain_gather_f(Batch b) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)b.n_nodes * 6) return;
  const int g = b.gl[t];
  if (g < 0) return;
  const int i = (int)(t / 6), q = (int)(t - (int64_t)i * 6);
  const int s = b.node_struct[i];
  const StructInfo& inf = b.info[s];
  if (!inf.is_chain || !iterating(b.state[s])) return;
  const int ln = i - inf.node_off, eo = inf.elem_off;
  const int64_t ne = b.n_elem;
  double v = 0.0;
  if (ln & 1) {
    v += b.Fe[(int64_t)(6 + q) * ne + eo + (ln >> 1)];
  } else {
    const int el = ln >> 1;
    if (el >= 1) v += b.Fe[(int64_t)(12 + q) * ne + eo + el - 1];
    if (el < inf.n_elem) v += b.Fe[(int64_t)q * ne + eo + el];
  }
  b.P[inf.dof_off + g] = v;
}

// NodalLoad::Mount for every load entry of a structure, in entry order (one
// thread per structure keeps the accumulation order fixed).
__global__ void k_loads(Batch b) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= b.n_struct || !iterating(b.state[s])) return;
  const StructInfo inf = b.info[s];
  const StructState& st = b.state[s];
  double time = st.last_converged_time + st.current_time_step;
  double* P = b.P + inf.dof_off;
  double* band = b.band + inf.band_off;
  const bool to_nodeK = inf.is_chain && !b.full_band;
  for (int l = inf.load_off; l < inf.load_off + inf.n_loads; ++l) {
    const LoadEntry L = b.loads[l];
    int node = L.node;
    const int* gl = b.gl + (int64_t)node * 6;
    V3<double> fl, ml;
    for (int i = 0; i < 3; ++i) {
      fl[i] = L.mult[i] * table_at(b, L.table, time, i);
      ml[i] = L.mult[3 + i] * table_at(b, L.table, time, i + 3);
    }
    M3<double> CQ;
    for (int q = 0; q < 9; ++q) CQ[q] = L.CQ[q];
    V3<double> fv = tmv(CQ, fl), mvv = tmv(CQ, ml);
    V3<double> al = {{b.disp[(int64_t)node * 6 + 3], b.disp[(int64_t)node * 6 + 4], b.disp[(int64_t)node * 6 + 5]}};
    double g = 4.0 / (4.0 + dot(al, al));
    M3<double> A = skew(al), Xi;
    for (int q = 0; q < 9; ++q) Xi[q] = g * 0.5 * A[q];
    Xi[0] += g; Xi[4] += g; Xi[8] += g;
    V3<double> mm = tmv(Xi, mvv);
    M3<double> V = opV(al, mm, g);
    for (int i = 0; i < 3; ++i)
      if (gl[i] >= 0) P[gl[i]] += -1.0 * fv[i];
    for (int i = 0; i < 3; ++i) {
      int gi = gl[3 + i];
      if (gi >= 0) P[gi] += -1.0 * mm[i];
      for (int j = 0; j < 3; ++j) {
        int gj = gl[3 + j];
        if (gi < 0 || gj < 0) continue;
        if (to_nodeK) b.nodeK[(int64_t)node * 9 + i * 3 + j] += -1.0 * V[i * 3 + j];
        else if (inf.wide) b.sh.wband[inf.wb_off + (inf.wkl + gi - gj) + (int64_t)gj * (2 * inf.wkl + 1)] += -1.0 * V[i * 3 + j];
        else band[(GF_KB + gi - gj) + (int64_t)gj * GF_LDB] += -1.0 * V[i * 3 + j];
      }
    }
  }
}

// P = -P; EstablishResidualCriteria at the first iteration;
// CheckResidualConvergence (reference src/ConvergenceCriteria.cpp:187-285,
// 460-598).
__global__ void k_residual(Batch b) {
  const int s = b.chunk_struct[blockIdx.x];
  StructState& st = b.state[s];
  if (!iterating(st)) return;
  const StructInfo inf = b.info[s];
  const StructParams& p = b.params[s];
  double* P = b.P + inf.dof_off;
  const int* d6 = b.dof_node6 + inf.dof_off;
  const int i1 = min(inf.n_free, b.chunk_start[blockIdx.x] + GF_RED_CHUNK);
  Red3 v{0.0, 0.0, 0};
  for (int i = b.chunk_start[blockIdx.x] + threadIdx.x; i < i1; i += blockDim.x) {
    double x = -1.0 * P[i];
    P[i] = x;
    double a = fabs(x);
    if (nan_or_huge(a)) v.f = 1;
    if (d6[i] % 6 < 3) { if (a > v.a) v.a = a; }
    else { if (a > v.b) v.b = a; }
  }
  Red3 r = block_red(v);
  RedScratch& R = b.red[s];
  if (threadIdx.x == 0) {
    red_max(&R.a, r.a);
    red_max(&R.b, r.b);
    if (r.f) atomicOr(&R.f, 1);
  }
  if (!red_arrive(R, red_chunks(inf))) return;
  if (threadIdx.x == 0) {
    r.a = red_value(&R.a);
    r.b = red_value(&R.b);
    r.f = *(volatile int*)&R.f;
    R = RedScratch{0ull, 0ull, 0ull, 0ull, 0, 0};
  }
  if (threadIdx.x == 0) {
    if (st.it == 1) {
      double pf = st.force_crit, pm = st.moment_crit;
      double fc = r.a * p.force_tol > p.force_min * p.force_tol ? r.a * p.force_tol : p.force_min * p.force_tol;
      double mc = r.b * p.moment_tol > p.moment_min * p.moment_tol ? r.b * p.moment_tol : p.moment_min * p.moment_tol;
      st.force_crit = (st.n_conv_evaluated * pf + fc) / (st.n_conv_evaluated + 1);
      st.moment_crit = (st.n_conv_evaluated * pm + mc) / (st.n_conv_evaluated + 1);
      st.n_conv_evaluated++;
    }
    if (r.f) st.diverged = 1;
    int conv = 1;
    if (r.a > p.divergence_ref || r.b > p.divergence_ref) {
      st.diverged = 1;
      conv = 0;
    } else {
      if (inf.has_force && r.a > st.force_crit) conv = 0;
      if (inf.has_moment && r.b > st.moment_crit) conv = 0;
    }
    st.res_conv = conv;
    st.last_res = fmax(r.a, r.b);
    st.need_solve = !(st.res_conv && st.gl_conv);
  }
}

// ---------------------------------------------------------------------------
// Banded LU without pivoting, fused forward substitution, back substitution;
// FP64.  One 4-warp CTA per structure.
//
// On this GPU a dependent FP64 operation costs ~64 cycles and an FP64 divide
// ~640, so the per-column critical path is what bounds a long chain.  The
// elimination is split so that warp 0 carries only that path with one column
// of lookahead: at step j it updates column j+1, forms the next pivot's
// reciprocal (Newton-Raphson iteration r <- r (2 - p r), seeded by the FP32
// approximate reciprocal, two steps) and the next multipliers, while warps
// 1-3 apply step j's rank-1 update to columns j+2..j+17 and the right-hand
// side.  Band columns stream through a 128-column shared-memory ring filled
// 32 columns at a time, two chunks ahead.  Row j of U (with the pivot
// reciprocal in place of the pivot) goes to b.U; the forward-substituted
// right-hand side goes to P, which the back substitution overwrites with x.
constexpr int RING = 128;
constexpr int CHUNK = 32;
constexpr int SOLVE_THREADS = 128;

// Newton-Raphson reciprocal of p, seeded by the hardware FP32 approximation;
// exact division where the seed is out of FP32 range.
__device__ __forceinline__ double recip_nr(double p) {
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

template <typename T>
__device__ __forceinline__ void load_chunk(const T* __restrict__ band, const double* __restrict__ rhs, T* ring,
                                           double* rring, int q, int n, int tid, int nthreads) {
  int c0 = q * CHUNK;
  if (c0 >= n) return;
  int nc = min(CHUNK, n - c0);
  int slot0 = c0 % RING;
  const T* src = band + (int64_t)c0 * GF_LDB;
  T* dst = ring + (int64_t)slot0 * GF_LDB;
  for (int i = tid; i < nc * GF_LDB; i += nthreads) dst[i] = src[i];
  for (int i = tid; i < nc; i += nthreads) rring[slot0 + i] = rhs[c0 + i];
}

__global__ void __launch_bounds__(SOLVE_THREADS) k_band_solve(Batch b) {
  int s = blockIdx.x;
  StructState& st = b.state[s];
  if (!iterating(st) || !st.need_solve) return;
  const StructInfo inf = b.info[s];
  if (inf.is_chain || inf.wide) return;
  const int n = inf.n_free;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  extern __shared__ unsigned char smem_raw[];
  double* ring = reinterpret_cast<double*>(smem_raw);
  double* rring = ring + RING * GF_LDB;
  __shared__ double lbuf[2][GF_KB + 1];
  __shared__ double invb[2];
  __shared__ int sfail;
  const double* band = b.band + inf.band_off;
  double* rhs = b.P + inf.dof_off;
  double* U = b.U + (int64_t)inf.dof_off * GF_UW;
  if (tid == 0) sfail = 0;
  load_chunk(band, rhs, ring, rring, 0, n, tid, SOLVE_THREADS);
  load_chunk(band, rhs, ring, rring, 1, n, tid, SOLVE_THREADS);
  load_chunk(band, rhs, ring, rring, 2, n, tid, SOLVE_THREADS);
  __syncthreads();
  // step 0 multipliers
  if (warp == 0) {
    double p = ring[GF_KB];
    double inv = recip_nr(p);
    if (lane >= 1 && lane <= GF_KB) lbuf[0][lane] = (lane < n) ? ring[GF_KB + lane] * inv : 0.0;
    if (lane == 0) {
      invb[0] = inv;
      if (!(p != 0.0) || !isfinite(p)) sfail = 1;
    }
  }
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    const int cur = j & 1;
    if (j % CHUNK == 0 && j > 0) load_chunk(band, rhs, ring, rring, j / CHUNK + 2, n, tid, SOLVE_THREADS);
    if (warp > 0) {
      // rank-1 update of columns j+2..j+17 (16 x 17 entries) and the rhs (17)
      for (int k = tid - 32; k < 16 * GF_KB + GF_KB; k += SOLVE_THREADS - 32) {
        if (k < 16 * GF_KB) {
          int r = k / 16 + 1, c = k % 16 + 2;
          int J = j + c;
          if (J < n) {
            double* col = ring + (int64_t)(J % RING) * GF_LDB;
            col[GF_KB + r - c] -= lbuf[cur][r] * col[GF_KB - c];
          }
        } else {
          int r = k - 16 * GF_KB + 1;
          if (j + r < n) rring[(j + r) % RING] -= lbuf[cur][r] * rring[j % RING];
        }
      }
    } else {
      // U row j (reciprocal pivot first), y_j
      if (lane >= 1 && lane <= GF_KB) {
        int J = j + lane;
        U[(int64_t)j * GF_UW + lane] = J < n ? ring[(int64_t)(J % RING) * GF_LDB + GF_KB - lane] : 0.0;
      } else if (lane == 0) {
        U[(int64_t)j * GF_UW] = invb[cur];
        rhs[j] = rring[j % RING];
      }
      if (j + 1 < n) {
        double* c1 = ring + (int64_t)((j + 1) % RING) * GF_LDB;
        if (lane >= 1 && lane <= GF_KB) c1[GF_KB + lane - 1] -= lbuf[cur][lane] * c1[GF_KB - 1];
        __syncwarp();
        double p = c1[GF_KB];
        double inv = recip_nr(p);
        if (lane >= 1 && lane <= GF_KB) lbuf[cur ^ 1][lane] = (j + 1 + lane < n) ? c1[GF_KB + lane] * inv : 0.0;
        if (lane == 0) {
          invb[cur ^ 1] = inv;
          if (!(p != 0.0) || !isfinite(p)) sfail = 1;
        }
      }
    }
    __syncthreads();
  }
  // back substitution, column oriented, warp 0: lane t (1..17) holds
  // y'_{j-t}; x_j = y'_j / u_jj, then y'_{j-t} -= U(j-t, j) x_j.
  if (warp == 0) {
    double yv = 0.0;  // lane 0: y'_j; lane t: y'_{j-t}
    {
      int i = n - 1 - lane;
      if (lane <= GF_KB && i >= 0) yv = rhs[i];
    }
    for (int j0 = n - 1; j0 >= 0; j0 -= CHUNK) {
      // per-chunk operands: lane t needs U(j - t, t) for j in the chunk, lane 0
      // the reciprocal pivots, lane 17 the y entering at j - 18
      double uo[CHUNK];
#pragma unroll
      for (int q = 0; q < CHUNK; ++q) {
        int j = j0 - q;
        double v = 0.0;
        if (j >= 0) {
          if (lane == 0) v = U[(int64_t)j * GF_UW];
          else if (lane <= GF_KB && j - lane >= 0) v = U[(int64_t)(j - lane) * GF_UW + lane];
          else if (lane == GF_KB + 1 && j - GF_KB - 1 >= 0) v = rhs[j - GF_KB - 1];
        }
        uo[q] = v;
      }
#pragma unroll
      for (int q = 0; q < CHUNK; ++q) {
        int j = j0 - q;
        if (j < 0) break;
        double xj = __shfl_sync(0xffffffffu, yv * uo[q], 0);
        if (lane == 0) rhs[j] = xj;
        if (lane >= 1 && lane <= GF_KB) yv = fma(-uo[q], xj, yv);
        // shift the window: lane t takes lane t+1's value; lane 17 takes y_{j-18}
        double nx = __shfl_down_sync(0xffffffffu, yv, 1);
        double ent = __shfl_sync(0xffffffffu, uo[q], GF_KB + 1);
        yv = lane < GF_KB ? nx : (lane == GF_KB ? ent : 0.0);
      }
    }
  }
  if (tid == 0) st.info_fail = sfail;
}

// UpdateDisps + CheckGLConvergence (reference src/Solution.cpp:390-423,
// src/ConvergenceCriteria.cpp:289-458)
__global__ void k_update(Batch b) {
  const int s = b.chunk_struct[blockIdx.x];
  StructState& st = b.state[s];
  if (!iterating(st) || !st.need_solve) return;
  const StructInfo inf = b.info[s];
  const StructParams& p = b.params[s];
  const double* P = b.P + inf.dof_off;
  const int* d6 = b.dof_node6 + inf.dof_off;
  const int i1 = min(inf.n_free, b.chunk_start[blockIdx.x] + GF_RED_CHUNK);
  Red3 inc{0.0, 0.0, 0}, val{0.0, 0.0, 0};
  for (int i = b.chunk_start[blockIdx.x] + threadIdx.x; i < i1; i += blockDim.x) {
    int q = d6[i];
    double x = P[i];
    double nv = b.disp[q] + x;
    b.disp[q] = nv;
    double a = fabs(x), v = fabs(nv);
    if (nan_or_huge(a)) inc.f = 1;
    if (q % 6 < 3) { if (a > inc.a) inc.a = a; if (v > val.a) val.a = v; }
    else { if (a > inc.b) inc.b = a; if (v > val.b) val.b = v; }
  }
  Red3 ri = block_red(inc);
  Red3 rv = block_red(val);
  RedScratch& R = b.red[s];
  if (threadIdx.x == 0) {
    red_max(&R.a, ri.a);
    red_max(&R.b, ri.b);
    red_max(&R.va, rv.a);
    red_max(&R.vb, rv.b);
    if (ri.f) atomicOr(&R.f, 1);
  }
  if (!red_arrive(R, red_chunks(inf))) return;
  // the last CTA: every increment of the structure is in place
  if (b.params[s].dynamic)
    for (int i = threadIdx.x; i < inf.n_nodes; i += blockDim.x) update_dyn_node(b, st.a, inf.node_off + i);
  if (threadIdx.x == 0) {
    ri.a = red_value(&R.a);
    ri.b = red_value(&R.b);
    rv.a = red_value(&R.va);
    rv.b = red_value(&R.vb);
    ri.f = *(volatile int*)&R.f;
    R = RedScratch{0ull, 0ull, 0ull, 0ull, 0, 0};
  }
  if (threadIdx.x == 0) {
    st.res_conv = 0;
    if (ri.f) st.diverged = 1;
    st.disp_crit = rv.a * p.disp_tol > p.disp_min * p.disp_tol ? p.disp_tol * rv.a : p.disp_min * p.disp_tol;
    st.rot_crit = rv.b * p.rot_tol > p.rot_min * p.rot_tol ? p.rot_tol * rv.b : p.rot_min * p.rot_tol;
    int conv = 1;
    if (st.disp_crit > p.divergence_ref || st.rot_crit > p.divergence_ref) {
      st.diverged = 1;
      conv = 0;
    } else {
      if (inf.has_force && ri.a > st.disp_crit) conv = 0;
      if (inf.has_moment && ri.b > st.rot_crit) conv = 0;
    }
    st.gl_conv = conv;
    st.last_inc = fmax(ri.a, ri.b);
  }
}

// Newton-loop end test, divergence, commit or bisection, step growth
// (reference src/Static.cpp:236-298).
__global__ void k_control(Batch b) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= b.n_struct) return;
  StructState& st = b.state[s];
  st.commit = 0;
  if (st.phase != PH_ITER) {
    if (st.phase == PH_START) atomicAdd(b.running, 1);
    return;
  }
  const StructParams& p = b.params[s];
  if (p.ray_on) st.ray_init = 1;  // the step's first iteration has formed C
  int both = st.res_conv && st.gl_conv;
  if ((st.it == p.max_it && !both) || (st.need_solve && st.info_fail)) st.diverged = 1;
  if (st.time_step < p.min_time_step && st.time != p.end_time) st.aborted = 1;
  st.it++;
  st.total_it++;
  if (st.need_solve) st.n_solves++;
  bool loop = !both && !st.diverged && !st.aborted;
  if (loop) {
    atomicAdd(b.running, 1);
    return;
  }
  st.mon_now = 0;
  if (!st.diverged) {
    st.converged_number++;
    st.commit = 1;
    st.commit_dyn = p.dynamic;
    st.convergence_counter++;
    // the monitor's rule, on the solution step that converged (reference
    // src/Static.cpp:268-276, src/Dynamic.cpp:392-399)
    st.conv_in_step++;
    const StructInfo& mi = b.info[s];
    if (mi.mon_n > 0 && !st.aborted && (st.conv_in_step % mi.mon_sample == 0 || st.time == p.end_time)) {
      st.mon_now = 1;
      st.mon_rows++;
    }
    if (st.it <= p.min_it || st.convergence_counter >= p.conv_increase) {
      st.time_step = st.time_step * p.inc_factor;
      if (st.time_step > p.max_time_step) st.time_step = p.max_time_step;
      st.convergence_counter = 0;
    }
  } else {
    st.time -= st.time_step;
    st.time_step = st.time_step / 2.0;
    st.diverged = 0;
    st.convergence_counter = 0;
    st.bisections++;
  }
  if ((st.time < p.end_time || st.diverged) && !st.aborted) {
    st.phase = PH_START;
    atomicAdd(b.running, 1);
  } else if (!st.aborted && st.step + 1 < b.info[s].n_steps) {
    // the next solution step (reference src/main.cpp:52-60) starts from
    // this state: its own step control, a fresh residual-criterion average
    // (src/Static.cpp:146, src/Dynamic.cpp:261), Rayleigh matrices formed
    // anew (Dynamic::Solve's `first`), and zero nodal velocities for a
    // Static step (ZerosVelAccel) or a Dynamic one with ZeroIC.  The commit
    // kernels of this pass still save the converged state of the step that
    // ended, with the ended step's Dynamic flag (commit_dyn) deciding
    // whether its velocities are saved, as SaveConfiguration does.
    st.step++;
    st.conv_in_step = 0;
    const StructParams np = b.step_params[b.info[s].step_off + st.step];
    b.params[s] = np;
    st.time = np.start_time;
    st.last_converged_time = np.start_time;
    st.time_step = np.time_step0;
    st.convergence_counter = 0;
    st.n_conv_evaluated = 0;
    st.ray_init = 0;
    st.zero_va = np.zero_va;
    st.phase = PH_START;
    atomicAdd(b.running, 1);
  } else {
    st.phase = st.aborted ? PH_ABORTED : PH_DONE;
  }
}

// SaveConfiguration: element Gauss-point history ...
__global__ void k_commit_elems(Batch b) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= b.n_elem) return;
  int s = b.estruct[e];
  if (!b.state[s].commit) return;
  double d[18];
  for (int j = 0; j < 3; ++j) {
    int nd = b.enodes[3 * e + j];
    for (int q = 0; q < 6; ++q) d[6 * j + q] = b.disp[(int64_t)nd * 6 + q];
  }
  BeamConst c = b.bconst[e];
  BeamHist h = b.bhist[e];
  BeamHistAux x = b.baux[e];
  beam_commit(c, h, x, d);
  b.bhist[e] = h;
  b.baux[e] = x;
}

// ... and nodal configuration (reference src/Node.cpp:325-370)
__global__ void k_commit_nodes(Batch b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.n_nodes) return;
  int s = b.node_struct[i];
  if (!b.state[s].commit) return;
  double* c = b.copy + (int64_t)i * 6;
  const double* d = b.disp + (int64_t)i * 6;
  for (int k = 0; k < 3; ++k) c[k] += d[k];
  V3<double> a1 = {{c[3], c[4], c[5]}}, a2 = {{d[3], d[4], d[5]}};
  V3<double> a3 = rodrigues_compose(a2, a1);
  for (int k = 0; k < 3; ++k) c[3 + k] = a3[k];
  M3<double> Q = rodrigues(a3);
  for (int k = 0; k < 9; ++k) b.Qn[(int64_t)i * 9 + k] = Q[k];
  // the converged velocities of a Dynamic step, also of its last step when
  // the next solution step's parameters are already in place
  if (b.state[s].commit_dyn)
    for (int k = 0; k < 6; ++k) {
      b.copy_vel[(int64_t)i * 6 + k] = b.vel[(int64_t)i * 6 + k];
      b.copy_accel[(int64_t)i * 6 + k] = b.accel[(int64_t)i * 6 + k];
    }
}

// Monitor line of one monitored node (Node::WriteMonitor, reference
// src/Node.cpp:227-320) after a committed step the monitor records: time,
// copy_coordinates, the load of every numbered DOF -- the elements'
// P_loading summed at the node (global_I_A at a free DOF, global_P_B at a
// constrained one; a DOF without a number keeps its last value) with the
// moments turned from pseudo-moments by Xi(alpha)^-T, alpha the node's
// rotation increment -- and the converged velocities and accelerations.
// One thread per monitored node.
__global__ void k_monitor_record(Batch b) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= b.mon_total) return;
  const int s = b.mon_struct[q];
  const StructState& st = b.state[s];
  if (!st.commit || !st.mon_now) return;
  const int row = st.mon_rows - 1;
  const int i = b.mon_node[q];
  double* L = b.mon_load + (int64_t)q * 6;
  double sum[6] = {0, 0, 0, 0, 0, 0};
  const int64_t ne = b.n_elem;
  for (int k = b.mon_adj_off[q]; k < b.mon_adj_off[q + 1]; ++k) {
    const int2 a = b.mon_adj[k];
    const int kind = a.y >> 6, at = a.y & 63;
    if (kind == 0) {
#pragma unroll
      for (int d = 0; d < 6; ++d) sum[d] += b.Fe[(int64_t)(6 * at + d) * ne + a.x];
    } else {
      const double* F = b.sh.Fe + (int64_t)a.x * 27;
#pragma unroll
      for (int d = 0; d < 3; ++d) sum[d] += F[3 * at + d];
      if (at >= 3)
#pragma unroll
        for (int d = 0; d < 3; ++d) sum[3 + d] += F[18 + 3 * (at - 3) + d];
    }
  }
#pragma unroll
  for (int d = 0; d < 6; ++d)
    if (b.gl[(int64_t)i * 6 + d] != -2) L[d] = sum[d];
  // pseudo-moment -> moment: m = Xi(alpha)^-T m
  const V3<double> al = {{b.disp[(int64_t)i * 6 + 3], b.disp[(int64_t)i * 6 + 4], b.disp[(int64_t)i * 6 + 5]}};
  const double g = 4.0 / (4.0 + dot(al, al));
  M3<double> A = skew(al), Xt;
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) Xt[r * 3 + c] = g * ((r == c ? 1.0 : 0.0) + 0.5 * A[c * 3 + r]);
  const double c00 = Xt[4] * Xt[8] - Xt[5] * Xt[7], c01 = Xt[5] * Xt[6] - Xt[3] * Xt[8],
               c02 = Xt[3] * Xt[7] - Xt[4] * Xt[6];
  const double id = 1.0 / (Xt[0] * c00 + Xt[1] * c01 + Xt[2] * c02);
  M3<double> inv;
  inv[0] = c00 * id;
  inv[1] = (Xt[2] * Xt[7] - Xt[1] * Xt[8]) * id;
  inv[2] = (Xt[1] * Xt[5] - Xt[2] * Xt[4]) * id;
  inv[3] = c01 * id;
  inv[4] = (Xt[0] * Xt[8] - Xt[2] * Xt[6]) * id;
  inv[5] = (Xt[2] * Xt[3] - Xt[0] * Xt[5]) * id;
  inv[6] = c02 * id;
  inv[7] = (Xt[1] * Xt[6] - Xt[0] * Xt[7]) * id;
  inv[8] = (Xt[0] * Xt[4] - Xt[1] * Xt[3]) * id;
  const V3<double> m = mv(inv, V3<double>{{L[3], L[4], L[5]}});
  L[3] = m[0];
  L[4] = m[1];
  L[5] = m[2];
  if (row < 0 || row >= b.mon_cap) return;
  double* o = b.mon_rec + ((int64_t)q * b.mon_cap + row) * 25;
  o[0] = st.time;
#pragma unroll
  for (int d = 0; d < 6; ++d) {
    o[1 + d] = b.copy[(int64_t)i * 6 + d];
    o[7 + d] = L[d];
    o[13 + d] = b.copy_vel[(int64_t)i * 6 + d];
    o[19 + d] = b.copy_accel[(int64_t)i * 6 + d];
  }
}

// Element-level entry (no batch): tangent and internal force, FP64.
__global__ void __launch_bounds__(MOUNT_THREADS) k_beam_elements(int n, const BeamConst* cs, const BeamHist* hs,
                                                                 const double* ds, double* Ks, double* fs) {
  extern __shared__ unsigned char smem_raw[];
  double* sM = reinterpret_cast<double*>(smem_raw);
  const int tid = threadIdx.x;
  int e = blockIdx.x * blockDim.x + tid;
  if (e >= n) return;
  const BeamConst& c = cs[e];
  const BeamHist& h = hs[e];
  double d[18];
  for (int q = 0; q < 18; ++q) d[q] = ds[(int64_t)e * 18 + q];
  BeamInterp ip[2] = {beam_interp(c, d, 0), beam_interp(c, d, 1)};
  double* f = sM + (size_t)2 * OP_N * MOUNT_THREADS + tid;
  for (int q = 0; q < 18; ++q) f[q * MOUNT_THREADS] = 0.0;
#pragma unroll 1
  for (int g = 0; g < 2; ++g) {
    BeamGP kin;
    beam_kinematics(c, h, ip[g], g, kin);
    beam_gp_force(c, kin, g, f, MOUNT_THREADS);
    double* M = sM + (size_t)g * OP_N * MOUNT_THREADS + tid;
    beam_gp_operator<double>(c, kin, M, MOUNT_THREADS);
    rotate_blocks9<double>(c, M, MOUNT_THREADS);
  }
  double* K = Ks + (int64_t)e * 324;
#pragma unroll 1
  for (int J = 0; J < 3; ++J)
#pragma unroll 1
    for (int I = 0; I < 3; ++I) beam_K_block<double>(c, sM + tid, sM + OP_N * MOUNT_THREADS + tid, I, J, MOUNT_THREADS, K);
  for (int q = 0; q < 18; ++q) fs[(int64_t)e * 18 + q] = f[q * MOUNT_THREADS];
}

// Element-level inertia (no batch): M (18x18 column-major, global) and F.
__global__ void k_beam_inertia_elements(int n, const BeamConst* cs, const BeamHistAux* xs, const double* ds,
                                        const double* vs, const double* as, const double* a, double* Ms,
                                        double* Fs) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const BeamConst& c = cs[e];
  double d[18], vel[18], acc[18], f[18], D[18];
  for (int q = 0; q < 18; ++q) {
    d[q] = ds[(int64_t)e * 18 + q];
    vel[q] = vs[(int64_t)e * 18 + q];
    acc[q] = as[(int64_t)e * 18 + q];
    f[q] = 0.0;
  }
  double an[6];
  for (int q = 0; q < 6; ++q) an[q] = a[q];
  for (int g = 0; g < 2; ++g) {
    BeamInterp ip = beam_interp(c, d, g);
    beam_gp_inertia(c, xs[e], ip, vel, acc, an, g, f, 1, D + 9 * g, 1);
  }
  for (int r = 0; r < 18; ++r)
    for (int q = 0; q < 18; ++q) Ms[(int64_t)e * 324 + r + 18 * q] = beam_M_entry(c, D, D + 9, 1, an[0] * c.Mr, r, q);
  for (int q = 0; q < 18; ++q) Fs[(int64_t)e * 18 + q] = f[q];
}

__global__ void k_beam_commit(int n, const BeamConst* cs, BeamHist* hs, BeamHistAux* xs, const double* ds) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double d[18];
  for (int q = 0; q < 18; ++q) d[q] = ds[(int64_t)e * 18 + q];
  BeamHist h = hs[e];
  BeamHistAux x = xs[e];
  beam_commit(cs[e], h, x, d);
  hs[e] = h;
  xs[e] = x;
}

}  // namespace

void launch_modal_mass(const Batch& b, double* M, int64_t W, int kw, cudaStream_t st) {
  for (int c = 0; c < b.n_colors; ++c) {
    const int cnt = b.color_off[c + 1] - b.color_off[c];
    if (cnt > 0) k_modal_mass_beam<<<(cnt + 63) / 64, 64, 0, st>>>(b, c, M, W, kw);
  }
  if (b.sh.n_shells) launch_shell_modal_mass(b, M, W, kw, st);
}


// ---------------------------------------------------------------------------
void launch_beam_inertia(int n, const BeamConst* c, const BeamHistAux* x, const double* d, const double* v,
                         const double* a_acc, const double* a, double* M, double* F, cudaStream_t st) {
  if (n > 0) k_beam_inertia_elements<<<(n + 63) / 64, 64, 0, st>>>(n, c, x, d, v, a_acc, a, M, F);
}

void launch_beam_commit(int n, const BeamConst* c, BeamHist* h, BeamHistAux* x, const double* d, cudaStream_t st) {
  if (n > 0) k_beam_commit<<<(n + 127) / 128, 128, 0, st>>>(n, c, h, x, d);
}

void launch_init_state(const Batch& b, cudaStream_t st) {
  if (b.n_struct == 0) return;
  k_init_state<<<(b.n_struct + 127) / 128, 128, 0, st>>>(b);
}


static void set_attrs();

static void launch_mount(const Batch& b, cudaStream_t st, LaunchProf* prof);

void launch_iteration_partial(const Batch& b_in, cudaStream_t st) {
  set_attrs();
  Batch b = b_in;
  b.full_band = 1;  // the assembly view: every structure's band is filled
  int ns = b.n_struct;
  k_step_begin<<<ns, 256, 0, st>>>(b);
  k_zero<<<dim3(8, ns), 256, 0, st>>>(b);
  launch_wide_zero(b, st);
  launch_mount(b, st, nullptr);
  launch_shell_mount(b, st);
  k_loads<<<(ns + 63) / 64, 64, 0, st>>>(b);
  k_residual<<<b.n_chunks, 256, 0, st>>>(b);
}

// The stages of one Newton iteration for a caller that runs its own step
// control (gf_begin_step, gf_assemble, gf_set_increment, gf_commit): every
// structure's band is filled (the assembly view), as the caller reads K_AA.
void launch_step_begin(const Batch& b, cudaStream_t st) { k_step_begin<<<b.n_struct, 256, 0, st>>>(b); }

void launch_assembly(const Batch& b_in, cudaStream_t st) {
  set_attrs();
  Batch b = b_in;
  b.full_band = 1;
  int ns = b.n_struct;
  k_zero<<<dim3(8, ns), 256, 0, st>>>(b);
  launch_wide_zero(b, st);
  launch_mount(b, st, nullptr);
  launch_shell_mount(b, st);
  k_loads<<<(ns + 63) / 64, 64, 0, st>>>(b);
  k_residual<<<b.n_chunks, 256, 0, st>>>(b);
}

void launch_increment(const Batch& b, cudaStream_t st) { k_update<<<b.n_chunks, 256, 0, st>>>(b); }

void launch_commit(const Batch& b, cudaStream_t st) {
  if (b.n_elem) k_commit_elems<<<(b.n_elem + 127) / 128, 128, 0, st>>>(b);
  if (b.sh.n_shells) launch_shell_commit(b, st);
  if (b.n_nodes) k_commit_nodes<<<(b.n_nodes + 127) / 128, 128, 0, st>>>(b);
}

// Shared-memory limits of the large kernels, once per process (the served
// path's builder thread and the caller's thread may both get here first; a
// function-local static is initialised by exactly one of them).
static void set_attrs() {
  static const bool done = [] {
    cudaFuncSetAttribute(k_beam_tangent<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, MOUNT_SMEM);
    cudaFuncSetAttribute(k_beam_tangent<f2>, cudaFuncAttributeMaxDynamicSharedMemorySize, MOUNT_SMEM);
    cudaFuncSetAttribute(k_band_solve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (RING * GF_LDB + RING) * (int)sizeof(double));
    return true;
  }();
  (void)done;
}

const char* kernel_class_name(int k) {
  static const char* names[KC_COUNT] = {"step_begin", "zero", "beam_tangent", "loads", "residual", "band_solve",
                                        "update", "control", "commit_elems", "commit_nodes", "chain_solve", "scatter",
                                        "shell_mount", "wide_diag", "wide_trsm", "wide_update", "wide_subst",
                                        "wide_refine"};
  return k >= 0 && k < KC_COUNT ? names[k] : "?";
}


static void launch_mount(const Batch& b, cudaStream_t st, LaunchProf* prof) {
  if (b.n_elem == 0) return;
  {
    ProfScope q(prof, st, KC_MOUNT);
    // mixed precision: the tangent operator in FP32-pair arithmetic on the
    // FP32 pipe; kinematics, internal force and everything after stay FP64
    const int smem = MOUNT_SMEM;
    if (b.mixed)
      k_beam_tangent<f2><<<(b.n_elem + MOUNT_THREADS - 1) / MOUNT_THREADS, MOUNT_THREADS, smem, st>>>(b);
    else
      k_beam_tangent<double><<<(b.n_elem + MOUNT_THREADS - 1) / MOUNT_THREADS, MOUNT_THREADS, smem, st>>>(b);
    // the pressure's load stiffness is part of the K_e that Rayleigh damping
    // reads (the reference mounts loads before damping)
    if (b.n_pipe_press) k_pipe_pressure<<<(b.n_pipe_press + 127) / 128, 128, 0, st>>>(b);
    if (b.any_rayleigh) k_beam_rayleigh<<<(b.n_elem + 127) / 128, 128, 0, st>>>(b);
  }
  if (!b.full_band && b.chain.n_chain_elems == b.n_elem) {
    // chains only: the residual is all the scatter would assemble
    ProfScope q(prof, st, KC_SCATTER);
    const int64_t nt = (int64_t)b.n_nodes * 6;
    k_chain_gather_f<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(b);
    return;
  }
  for (int c = 0; c < b.n_colors; ++c) {
    int cnt = b.color_off[c + 1] - b.color_off[c];
    if (cnt <= 0) continue;
    ProfScope q(prof, st, KC_SCATTER);
    k_beam_scatter<<<(cnt + 3) / 4, 128, 0, st>>>(b, c);
  }
}

void launch_iteration(const Batch& b, cudaStream_t st, bool commit_kernels, LaunchProf* prof) {
  set_attrs();
  int ns = b.n_struct;
  { ProfScope q(prof, st, KC_STEP_BEGIN); k_step_begin<<<ns, 256, 0, st>>>(b); }
  { ProfScope q(prof, st, KC_ZERO); k_zero<<<dim3(8, ns), 256, 0, st>>>(b); }
  if (b.sh.n_wide) { ProfScope q(prof, st, KC_ZERO); launch_wide_zero(b, st); }
  launch_mount(b, st, prof);
  if (b.sh.n_shells) { ProfScope q(prof, st, KC_SHELL); launch_shell_mount(b, st); }
  { ProfScope q(prof, st, KC_LOADS); k_loads<<<(ns + 63) / 64, 64, 0, st>>>(b); }
  { ProfScope q(prof, st, KC_RESIDUAL); k_residual<<<b.n_chunks, 256, 0, st>>>(b); }
  { ProfScope q(prof, st, KC_SOLVE); launch_band_solve(b, st); }
  if (b.chain.n_chain_elems) { ProfScope q(prof, st, KC_CHAIN); launch_chain_solve(b, b.chain, st); }
  if (b.sh.n_wide) launch_wide_solve(b, st, prof);
  { ProfScope q(prof, st, KC_UPDATE); k_update<<<b.n_chunks, 256, 0, st>>>(b); }
  { ProfScope q(prof, st, KC_CONTROL); k_control<<<(ns + 127) / 128, 128, 0, st>>>(b); }
  if (commit_kernels) {
    if (b.n_elem) { ProfScope q(prof, st, KC_COMMIT_ELEMS); k_commit_elems<<<(b.n_elem + 127) / 128, 128, 0, st>>>(b); }
    if (b.sh.n_shells) { ProfScope q(prof, st, KC_COMMIT_ELEMS); launch_shell_commit(b, st); }
    if (b.n_nodes) { ProfScope q(prof, st, KC_COMMIT_NODES); k_commit_nodes<<<(b.n_nodes + 127) / 128, 128, 0, st>>>(b); }
    if (b.mon_total) k_monitor_record<<<(b.mon_total + 127) / 128, 128, 0, st>>>(b);
  }
}

namespace {
template <typename T> __global__ void k_fp_probe(T* out, int iters, T a, T c) {
  T x0 = threadIdx.x, x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3), x4 = x0 + T(4), x5 = x0 + T(5),
    x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + c; x1 = x1 * a + c; x2 = x2 * a + c; x3 = x3 * a + c;
    x4 = x4 * a + c; x5 = x5 * a + c; x6 = x6 * a + c; x7 = x7 * a + c;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

void launch_fp_probe(bool fp64, void* out, int blocks, int threads, int iters, cudaStream_t st) {
  if (fp64)
    k_fp_probe<double><<<blocks, threads, 0, st>>>(static_cast<double*>(out), iters, 0.999, 0.001);
  else
    k_fp_probe<float><<<blocks, threads, 0, st>>>(static_cast<float*>(out), iters, 0.999f, 0.001f);
}

void launch_band_solve(const Batch& b, cudaStream_t st) {
  k_band_solve<<<b.n_struct, SOLVE_THREADS, (RING * GF_LDB + RING) * sizeof(double), st>>>(b);
}

void launch_beam_elements(int n, const BeamConst* c, const BeamHist* h, const double* d, double* K,
                          double* f, cudaStream_t st) {
  if (n <= 0) return;
  static const bool attr =
      cudaFuncSetAttribute(k_beam_elements, cudaFuncAttributeMaxDynamicSharedMemorySize, MOUNT_SMEM) == cudaSuccess;
  (void)attr;
  k_beam_elements<<<(n + MOUNT_THREADS - 1) / MOUNT_THREADS, MOUNT_THREADS, MOUNT_SMEM, st>>>(n, c, h, d, K, f);
}

}  // namespace gf
