// Shell_1 structures on the device: element tangent and internal force with
// the follower pressure and, in Dynamic steps, the inertial terms
// (k_shell_tangent), Rayleigh damping (k_shell_rayleigh), colour scatter
// into the wide band (k_shell_scatter), SaveLagrange (k_shell_commit), and
// the wide-band LU with its triangular solves for the K_AA of those
// structures.
//
// Element math restates reference src/Shell_1.cpp:
//   899-1332   Mount: incremental Rodrigues kinematics at the three midside
//              Gauss points, thickness integration (3 points) of the
//              compressible neo-Hookean law, generalized constitutive matrix
//              D (12x12), Psi (12x15), geometric part G (15x15),
//              K = T^T sum_g w (dN^T (Psi^T D Psi + G) dN) T
//   1392-1467  MountShellSpecialLoads: follower pressure and its tangent
//   1650-1664  SaveLagrange
//   2368-2544  MountMassModal, MountMass, MountDamping, MountDyn
// dN is block-sparse (each 3x3 block a scalar times I), so the products run
// over the 3x3 blocks that are not zero.
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

typedef V3<double> v3;
typedef M3<double> m3;

struct SGp {
  v3 u, u1, u2, al, al1, al2;
  double g;
  m3 Xi, Xi1, Xi2, Q;
  v3 z1, z2, eta1, eta2, k1, k2;
};

// Gauss-point kinematics of the increment d (27, element DOF order, global).
__device__ void shell_gp(const ShellConst& c, const ShellHist& h, const double* d, int g, SGp& k) {
  v3 ug = {{0, 0, 0}}, u1g = {{0, 0, 0}}, u2g = {{0, 0, 0}}, ag = {{0, 0, 0}}, a1g = {{0, 0, 0}},
     a2g = {{0, 0, 0}};
#pragma unroll
  for (int j = 0; j < 3; ++j) {
#pragma unroll
    for (int n = 0; n < 6; ++n) {
      ug[j] += d[3 * n + j] * c.Nu[g][n];
      u1g[j] += d[3 * n + j] * c.Nu1[g][n];
      u2g[j] += d[3 * n + j] * c.Nu2[g][n];
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      ag[j] += d[18 + 3 * m + j] * c.Na[g][m];
      a1g[j] += d[18 + 3 * m + j] * c.Na1[g][m];
      a2g[j] += d[18 + 3 * m + j] * c.Na2[g][m];
    }
  }
  m3 T;
#pragma unroll
  for (int q = 0; q < 9; ++q) T[q] = c.T3[q];
  k.u = mv(T, ug);
  k.u1 = mv(T, u1g);
  k.u2 = mv(T, u2g);
  k.al = mv(T, ag);
  k.al1 = mv(T, a1g);
  k.al2 = mv(T, a2g);
  double an2 = dot(k.al, k.al);
  k.g = 4.0 / (4.0 + an2);
  m3 A = skew(k.al), A2 = mul(A, A), Qd;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    Qd[q] = k.g * (A[q] + 0.5 * A2[q]);
    k.Xi[q] = k.g * 0.5 * A[q];
  }
  Qd[0] += 1.0; Qd[4] += 1.0; Qd[8] += 1.0;
  k.Xi[0] += k.g; k.Xi[4] += k.g; k.Xi[8] += k.g;
  m3 S1 = skew(k.al1), S2 = skew(k.al2);
  double p1 = dot(k.al, k.al1), p2 = dot(k.al, k.al2);
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    k.Xi1[q] = -0.5 * k.g * (p1 * k.Xi[q] - S1[q]);
    k.Xi2[q] = -0.5 * k.g * (p2 * k.Xi[q] - S2[q]);
  }
  m3 Qi;
#pragma unroll
  for (int q = 0; q < 9; ++q) Qi[q] = h.Q[g][q];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    k.z1[j] = k.u1[j] + h.z1[g][j];
    k.z2[j] = k.u2[j] + h.z2[g][j];
  }
  k.Q = mul(Qd, Qi);
  k.eta1 = tmv(k.Q, k.z1);
  k.eta2 = tmv(k.Q, k.z2);
  k.eta1[0] -= 1.0;
  k.eta2[1] -= 1.0;
  m3 XQ = mul(k.Xi, Qi);
  k.k1 = tmv(XQ, k.al1);
  k.k2 = tmv(XQ, k.al2);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    k.k1[j] += h.k1[g][j];
    k.k2[j] += h.k2[g][j];
  }
}

__device__ __forceinline__ void gather_d(const Batch& b, int e, double* d) {
  const int* nd = b.sh.snodes + 6 * e;
#pragma unroll
  for (int a = 0; a < 18; ++a) d[a] = b.disp[(int64_t)nd[a / 3] * 6 + a % 3];
#pragma unroll
  for (int a = 0; a < 9; ++a) d[18 + a] = b.disp[(int64_t)nd[3 + a / 3] * 6 + 3 + a % 3];
}

__device__ __forceinline__ m3 ld3(const double* p) {
  m3 r;
#pragma unroll
  for (int q = 0; q < 9; ++q) r[q] = p[q];
  return r;
}

// Table::GetValueAt (reference src/Table.cpp:73-102), first column:
// clamped outside the table, linear between the rows that bracket time.
__device__ __forceinline__ double table_value(const Batch& b, int t, double time) {
  const TableDev T = b.tables[t];
  const double* times = b.table_data + T.off;
  const double* vals = times + T.n_times;
  if (T.n_times == 0) return 0.0;
  if (time >= times[T.n_times - 1]) return vals[(int64_t)(T.n_times - 1) * T.n_cols];
  if (time <= times[0]) return vals[0];
  int idx = 0;
  while (time >= times[idx]) idx++;
  double f = (time - times[idx - 1]) / (times[idx] - times[idx - 1]);
  double a = vals[(int64_t)(idx - 1) * T.n_cols], c = vals[(int64_t)idx * T.n_cols];
  return a + f * (c - a);
}

}  // namespace

// Mount of one element at increment d: K (27x27 column-major, global
// frame; written from zero) and f (internal force, global frame).
__device__ void shell_mount(const ShellConst& c, const ShellHist& h, const double* d, double* K, double* f) {
  for (int q = 0; q < 729; ++q) K[q] = 0.0;
  double fl[27];
#pragma unroll
  for (int q = 0; q < 27; ++q) fl[q] = 0.0;
  const double mu = c.mu, la = c.lambda;
  const double csi[3] = {-0.77459666924148337703585307995648, 0.0, 0.77459666924148337703585307995648};
  const double wt[3] = {0.55555555555555555555555555555556, 0.88888888888888888888888888888889,
                        0.55555555555555555555555555555556};
  for (int g = 0; g < 3; ++g) {
    SGp k;
    shell_gp(c, h, d, g, k);
    // thickness integration: D blocks [row group (n1, m1, n2, m2)][column
    // group (eta1, kappa1, eta2, kappa2)] and the generalized stresses
    m3 D[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int x = 0; x < 9; ++x) D[r][q][x] = 0.0;
    v3 nr1 = {{0, 0, 0}}, nr2 = {{0, 0, 0}}, mr1 = {{0, 0, 0}}, mr2 = {{0, 0, 0}};
    const double jac = c.thick / 2.0;
    for (int q = 0; q < 3; ++q) {
      double zeta = c.thick * csi[q] / 2.0;
      double w = wt[q] * jac;
      double g11 = k.eta1[0] + zeta * k.k1[1], g12 = k.eta1[1] - zeta * k.k1[0], g13 = k.eta1[2];
      double g21 = k.eta2[0] + zeta * k.k2[1], g22 = k.eta2[1] - zeta * k.k2[0], g23 = k.eta2[2];
      double jb = (1.0 + g11) * (1.0 + g22) - g12 * g21;
      double v = (la * (jb * jb * jb - 1.0) + 2.0 * mu * (jb - 1.0)) / (la * jb * jb * jb + 2.0 * mu * jb);
      double den = la * jb * jb + 2.0 * mu;
      double dv = ((la + 2.0 * mu) * (3.0 * la * jb * jb + 2.0 * mu)) / (jb * jb * den * den);
      v3 t1 = {{mu * v * (1.0 + g22) + mu * (g11 - g22), mu * v * (-g21) + mu * (g12 + g21), mu * g13}};
      v3 t2 = {{mu * v * (-g12) + mu * (g12 + g21), mu * v * (1.0 + g11) + mu * (g22 - g11), mu * g23}};
      m3 C11 = {{mu * ((1.0 + g22) * (1.0 + g22) * dv + 1.0), -mu * (1.0 + g22) * g21 * dv, 0,
                 -mu * (1.0 + g22) * g21 * dv, mu * (g21 * g21 * dv + 1.0), 0, 0, 0, mu}};
      m3 C22 = {{mu * (g12 * g12 * dv + 1.0), -mu * ((1.0 + g11) * g12 * dv), 0,
                 -mu * ((1.0 + g11) * g12 * dv), mu * ((1.0 + g11) * (1.0 + g11) * dv + 1.0), 0, 0, 0, mu}};
      m3 C12 = {{-mu * ((1.0 + g22) * g12 * dv), mu * (v - 1.0 + (1.0 + g11) * (1.0 + g22) * dv), 0,
                 mu * (1.0 - v + g12 * g21 * dv), -mu * ((1.0 + g11) * g21 * dv), 0, 0, 0, 0}};
      m3 C21 = transpose(C12);
      // with E3r = skew(e3): C E3r, E3r C, E3r C E3r in closed form
      const m3* Cs[2][2] = {{&C11, &C12}, {&C21, &C22}};
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int bq = 0; bq < 2; ++bq) {
          const m3& C = *Cs[a][bq];
          m3 CE, EC, ECE;
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            CE[i * 3 + 0] = C[i * 3 + 1];
            CE[i * 3 + 1] = -C[i * 3 + 0];
            CE[i * 3 + 2] = 0.0;
          }
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            EC[0 * 3 + j] = -C[1 * 3 + j];
            EC[1 * 3 + j] = C[0 * 3 + j];
            EC[2 * 3 + j] = 0.0;
          }
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            ECE[0 * 3 + j] = -CE[1 * 3 + j];
            ECE[1 * 3 + j] = CE[0 * 3 + j];
            ECE[2 * 3 + j] = 0.0;
          }
          // rows: n_a (group 2a), m_a (group 2a+1); columns: eta_b (2b), kappa_b (2b+1)
#pragma unroll
          for (int x = 0; x < 9; ++x) {
            D[2 * a][2 * bq][x] += w * C[x];
            D[2 * a][2 * bq + 1][x] -= w * zeta * CE[x];
            D[2 * a + 1][2 * bq][x] += w * zeta * EC[x];
            D[2 * a + 1][2 * bq + 1][x] -= w * zeta * zeta * ECE[x];
          }
        }
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        nr1[j] += w * t1[j];
        nr2[j] += w * t2[j];
      }
      mr1[0] += w * zeta * (-t1[1]);
      mr1[1] += w * zeta * t1[0];
      mr2[0] += w * zeta * (-t2[1]);
      mr2[1] += w * zeta * t2[0];
    }
    D[1][1][8] = c.stiff_drill;
    D[3][3][8] = c.stiff_drill;
    mr1[2] = c.stiff_drill * k.k1[2];
    mr2[2] = c.stiff_drill * k.k2[2];
    // Psi blocks: P[r][r] (r = 0..3) and P[r][4]
    m3 Qt = transpose(k.Q);
    m3 QX = mul(Qt, k.Xi);
    m3 Z1 = skew(k.z1), Z2 = skew(k.z2);
    m3 Pd[4] = {Qt, QX, Qt, QX};
    m3 P4[4] = {mul(mul(Qt, Z1), k.Xi), mul(Qt, k.Xi1), mul(mul(Qt, Z2), k.Xi), mul(Qt, k.Xi2)};
    // M = Psi^T D Psi + G, 5x5 blocks
    m3 M[5][5];
    m3 DP4[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      m3 acc;
#pragma unroll
      for (int x = 0; x < 9; ++x) acc[x] = 0.0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        m3 t = mul(D[r][q], P4[q]);
#pragma unroll
        for (int x = 0; x < 9; ++x) acc[x] += t[x];
      }
      DP4[r] = acc;
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int q = 0; q < 4; ++q) M[a][q] = mul(tmul(Pd[a], D[a][q]), Pd[q]);
#pragma unroll
    for (int a = 0; a < 4; ++a) M[a][4] = tmul(Pd[a], DP4[a]);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      m3 acc;
#pragma unroll
      for (int x = 0; x < 9; ++x) acc[x] = 0.0;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        m3 t = tmul(P4[r], D[r][q]);
#pragma unroll
        for (int x = 0; x < 9; ++x) acc[x] += t[x];
      }
      M[4][q] = mul(acc, Pd[q]);
    }
    {
      m3 acc;
#pragma unroll
      for (int x = 0; x < 9; ++x) acc[x] = 0.0;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        m3 t = tmul(P4[r], DP4[r]);
#pragma unroll
        for (int x = 0; x < 9; ++x) acc[x] += t[x];
      }
      M[4][4] = acc;
    }
    // geometric part G
    v3 n1 = mv(k.Q, nr1), n2 = mv(k.Q, nr2), m1 = mv(k.Q, mr1), m2 = mv(k.Q, mr2);
    m3 Xi = k.Xi;
    m3 Gdua1 = mul(skew(n1), Xi), Gdua2 = mul(skew(n2), Xi);
#pragma unroll
    for (int x = 0; x < 9; ++x) { Gdua1[x] = -Gdua1[x]; Gdua2[x] = -Gdua2[x]; }
    m3 Vm1 = opV(k.al, m1, k.g), Vm2 = opV(k.al, m2, k.g);
    m3 Gaa;
    {
      m3 a1 = tmul(Xi, mul(mul(Z1, skew(n1)), Xi));
      m3 a2 = opV(k.al, mv(Z1, n1), k.g);
      m3 a3 = opdV(k.al, k.al1, m1, k.g);
      m3 a4 = tmul(k.Xi1, mul(skew(m1), Xi));
      m3 b1 = tmul(Xi, mul(mul(Z2, skew(n2)), Xi));
      m3 b2 = opV(k.al, mv(Z2, n2), k.g);
      m3 b3 = opdV(k.al, k.al2, m2, k.g);
      m3 b4 = tmul(k.Xi2, mul(skew(m2), Xi));
#pragma unroll
      for (int x = 0; x < 9; ++x) Gaa[x] = (a1[x] - a2[x] + a3[x] - a4[x]) + (b1[x] - b2[x] + b3[x] - b4[x]);
    }
    m3 Vm1t = transpose(Vm1), Vm2t = transpose(Vm2), Gdua1t = transpose(Gdua1), Gdua2t = transpose(Gdua2);
#pragma unroll
    for (int x = 0; x < 9; ++x) {
      M[0][4][x] += Gdua1[x];
      M[1][4][x] += Vm1t[x];
      M[2][4][x] += Gdua2[x];
      M[3][4][x] += Vm2t[x];
      M[4][0][x] += Gdua1t[x];
      M[4][1][x] += Vm1[x];
      M[4][2][x] += Gdua2t[x];
      M[4][3][x] += Vm2[x];
      M[4][4][x] += Gaa[x];
    }
    // generalized internal force q = Psi^T sigma
    v3 sg[4] = {nr1, mr1, nr2, mr2};
    v3 qv[5];
#pragma unroll
    for (int r = 0; r < 4; ++r) qv[r] = tmv(Pd[r], sg[r]);
    {
      v3 acc = {{0, 0, 0}};
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        v3 t = tmv(P4[r], sg[r]);
        acc[0] += t[0]; acc[1] += t[1]; acc[2] += t[2];
      }
      qv[4] = acc;
    }
    // dN coefficients: translation node a (0..5) sits in row blocks 0 (x1)
    // and 2 (x2); midside rotation node m in blocks 1 (x1), 3 (x2), 4
    const double a1w = c.alpha1;
    for (int a = 0; a < 9; ++a) {
      int ra[3];
      double ca[3];
      int na;
      if (a < 6) { ra[0] = 0; ca[0] = c.Nu1[g][a]; ra[1] = 2; ca[1] = c.Nu2[g][a]; na = 2; }
      else {
        int m = a - 6;
        ra[0] = 1; ca[0] = c.Na1[g][m]; ra[1] = 3; ca[1] = c.Na2[g][m]; ra[2] = 4; ca[2] = c.Na[g][m]; na = 3;
      }
      for (int i = 0; i < na; ++i)
#pragma unroll
        for (int x = 0; x < 3; ++x) fl[3 * a + x] += a1w * ca[i] * qv[ra[i]][x];
      for (int bb = 0; bb < 9; ++bb) {
        int rb[3];
        double cb[3];
        int nbq;
        if (bb < 6) { rb[0] = 0; cb[0] = c.Nu1[g][bb]; rb[1] = 2; cb[1] = c.Nu2[g][bb]; nbq = 2; }
        else {
          int m = bb - 6;
          rb[0] = 1; cb[0] = c.Na1[g][m]; rb[1] = 3; cb[1] = c.Na2[g][m]; rb[2] = 4; cb[2] = c.Na[g][m]; nbq = 3;
        }
        double blk[9];
#pragma unroll
        for (int x = 0; x < 9; ++x) blk[x] = 0.0;
        for (int i = 0; i < na; ++i)
          for (int j = 0; j < nbq; ++j) {
            double w = a1w * ca[i] * cb[j];
            const m3& Mb = M[ra[i]][rb[j]];
#pragma unroll
            for (int x = 0; x < 9; ++x) blk[x] += w * Mb[x];
          }
        // local-frame block (3a.., 3bb..), column-major 27x27
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) K[(3 * a + i) + 27 * (3 * bb + j)] += blk[i * 3 + j];
      }
    }
  }
  // to the global frame: every 3x3 block B -> T3^T B T3, in place
  m3 T;
#pragma unroll
  for (int q = 0; q < 9; ++q) T[q] = c.T3[q];
  for (int a = 0; a < 9; ++a)
    for (int bb = 0; bb < 9; ++bb) {
      m3 blk;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) blk[i * 3 + j] = K[(3 * a + i) + 27 * (3 * bb + j)];
      m3 o = tmul(T, mul(blk, T));
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) K[(3 * a + i) + 27 * (3 * bb + j)] = o[i * 3 + j];
    }
  for (int a = 0; a < 9; ++a) {
    v3 x = {{fl[3 * a], fl[3 * a + 1], fl[3 * a + 2]}};
    v3 y = tmv(T, x);
    f[3 * a] = y[0]; f[3 * a + 1] = y[1]; f[3 * a + 2] = y[2];
  }
}

// Follower pressure p at the current configuration (pu: displacements of
// the six nodes from the reference position, global): P_loading -= the
// consistent nodal load, K += its tangent.
__device__ void shell_pressure(const ShellConst& c, const double* pu, double p, bool area_update, double* K,
                               double* f) {
  {
    v3 e1 = {{c.T3[0], c.T3[1], c.T3[2]}}, e2 = {{c.T3[3], c.T3[4], c.T3[5]}};
    for (int kq = 0; kq < 6; ++kq) {
      v3 t1, t2;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        double s1 = 0.0, s2 = 0.0;
#pragma unroll
        for (int n = 0; n < 6; ++n) {
          s1 += c.N41[kq][n] * pu[3 * n + j];
          s2 += c.N42[kq][n] * pu[3 * n + j];
        }
        t1[j] = e1[j] + s1;
        t2[j] = e2[j] + s2;
      }
      v3 cr = cross(t1, t2);
      double nc = sqrt(dot(cr, cr));
      v3 np = {{(1.0 / nc) * cr[0], (1.0 / nc) * cr[1], (1.0 / nc) * cr[2]}};
      v3 qp = {{-p * np[0], -p * np[1], -p * np[2]}};
      double fac = area_update ? c.w4[kq] * nc : c.w4[kq];
#pragma unroll
      for (int n = 0; n < 6; ++n)
#pragma unroll
        for (int j = 0; j < 3; ++j) f[3 * n + j] -= fac * c.N4[kq][n] * qp[j];
      m3 S1 = skew(t1), S2 = skew(t2), Pm;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          Pm[i * 3 + j] = area_update ? (i == j ? 1.0 : 0.0) : (1.0 / nc) * ((i == j ? 1.0 : 0.0) - np[i] * np[j]);
      for (int bb = 0; bb < 6; ++bb) {
        m3 Bb;
#pragma unroll
        for (int x = 0; x < 9; ++x) Bb[x] = S1[x] * c.N42[kq][bb] - S2[x] * c.N41[kq][bb];
        m3 Kb = area_update ? Bb : mul(Pm, Bb);
        for (int a = 0; a < 6; ++a) {
          double w = c.w4[kq] * p * c.N4[kq][a];
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) K[(3 * a + i) + 27 * (3 * bb + j)] += w * Kb[i * 3 + j];
        }
      }
    }
  }
}

// MountMass and the mass part of MountDyn (reference
// src/Shell_1.cpp:2406-2498, 2536-2541).  At each of the three midside
// Gauss points (weight alpha1) the director fibre has mass coef1 per unit
// area and, about the midsurface, rotary inertia J_i = coef2 (I - d d^T)
// with d = Q(alpha_i) e3r; its inertial moment coef2 d x d'' equals
// J w' + w x J w.  In the element frame, with a[0..5] = a1..a6:
//   dT_u = coef1 (a1 du - a2 v_i - a3 acc_i)
//   dT_a = Xi(da) h,  h = J_i w2 + w1 x J_i w1,
//   w1 = a4 da + a5 w_i + a6 dw_i,  w2 = a1 da - a2 w_i - a3 dw_i
// (Newmark in the tangent space transported by Q_delta, as for Beam_1), and
// the exact tangent d dT_u/d du = a1 coef1 I,
//   d dT_a/d da = Xi (a1 J_i + a4 (skew(w1) J_i - skew(J_i w1)))
//                 - g^2/2 (h + da x h / 2) da^T - g/2 skew(h).
// The element adds alpha1 N^T dT to f and alpha1 N^T DdT N to K (global
// frame, column-major), N the 6x27 interpolation of the translations of the
// six nodes and the rotations of the midside nodes.  vel / acc: [6][6]
// converged nodal velocities and accelerations (global).
__device__ __noinline__ void shell_inertia(const ShellConst& c, const ShellHistAux& x, const double* d,
                                           const double* vel, const double* acc, const double* a, double* K,
                                           double* f) {
  const m3 T = ld3(c.T3);
  const double a1 = a[0], a2 = a[1], a3 = a[2], a4 = a[3], a5 = a[4], a6 = a[5];
  double wt[6][6];  // alpha1 sum_g Nu_n Nu_p
#pragma unroll
  for (int n = 0; n < 6; ++n)
#pragma unroll
    for (int q = 0; q < 6; ++q) wt[n][q] = 0.0;
#pragma unroll 1
  for (int g = 0; g < 3; ++g) {
    const double* Nu = c.Nu[g];
    const double* Na = c.Na[g];
    v3 du = {{0, 0, 0}}, vi = {{0, 0, 0}}, ai = {{0, 0, 0}}, da = {{0, 0, 0}}, wi = {{0, 0, 0}}, dwi = {{0, 0, 0}};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int n = 0; n < 6; ++n) {
        du[i] += d[3 * n + i] * Nu[n];
        vi[i] += vel[6 * n + i] * Nu[n];
        ai[i] += acc[6 * n + i] * Nu[n];
      }
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        da[i] += d[18 + 3 * m + i] * Na[m];
        wi[i] += vel[6 * (3 + m) + 3 + i] * Na[m];
        dwi[i] += acc[6 * (3 + m) + 3 + i] * Na[m];
      }
    }
    du = mv(T, du);
    vi = mv(T, vi);
    ai = mv(T, ai);
    da = mv(T, da);
    wi = mv(T, wi);
    dwi = mv(T, dwi);
    v3 fu;
#pragma unroll
    for (int i = 0; i < 3; ++i) fu[i] = c.coef1 * (a1 * du[i] - a2 * vi[i] - a3 * ai[i]);
    const m3 Qi = rodrigues(v3{{x.alpha[g][0], x.alpha[g][1], x.alpha[g][2]}});
    m3 Ji;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) Ji[i * 3 + j] = c.coef2 * ((i == j ? 1.0 : 0.0) - Qi[i * 3 + 2] * Qi[j * 3 + 2]);
    v3 w1, w2;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      w1[i] = a4 * da[i] + a5 * wi[i] + a6 * dwi[i];
      w2[i] = a1 * da[i] - a2 * wi[i] - a3 * dwi[i];
    }
    const v3 Jw1 = mv(Ji, w1), Jw2 = mv(Ji, w2), cr = cross(w1, Jw1);
    v3 h;
#pragma unroll
    for (int i = 0; i < 3; ++i) h[i] = Jw2[i] + cr[i];
    const double gg = 4.0 / (4.0 + dot(da, da));
    m3 Xi = skew(da);
#pragma unroll
    for (int q = 0; q < 9; ++q) Xi[q] *= 0.5 * gg;
    Xi[0] += gg;
    Xi[4] += gg;
    Xi[8] += gg;
    const v3 mom = mv(Xi, h);
    const m3 t = mul(skew(w1), Ji), SJw1 = skew(Jw1);
    m3 Dh;
#pragma unroll
    for (int q = 0; q < 9; ++q) Dh[q] = a1 * Ji[q] + a4 * (t[q] - SJw1[q]);
    m3 D = mul(Xi, Dh);
    const v3 axh = cross(da, h);
    const m3 Sh = skew(h);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        D[i * 3 + j] += -0.5 * gg * gg * (h[i] + 0.5 * axh[i]) * da[j] - 0.5 * gg * Sh[i * 3 + j];
    const m3 Dg = tmul(T, mul(D, T));
    const v3 gu = tmv(T, fu), ga = tmv(T, mom);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int n = 0; n < 6; ++n) f[3 * n + i] += c.alpha1 * Nu[n] * gu[i];
#pragma unroll
      for (int m = 0; m < 3; ++m) f[18 + 3 * m + i] += c.alpha1 * Na[m] * ga[i];
    }
#pragma unroll 1
    for (int m = 0; m < 3; ++m)
#pragma unroll 1
      for (int q = 0; q < 3; ++q) {
        const double w = c.alpha1 * Na[m] * Na[q];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) K[(18 + 3 * m + i) + 27 * (18 + 3 * q + j)] += w * Dg[i * 3 + j];
      }
#pragma unroll
    for (int n = 0; n < 6; ++n)
#pragma unroll
      for (int q = 0; q < 6; ++q) wt[n][q] += c.alpha1 * Nu[n] * Nu[q];
  }
  const double a1m = a1 * c.coef1;
#pragma unroll 1
  for (int n = 0; n < 6; ++n)
#pragma unroll 1
    for (int q = 0; q < 6; ++q)
#pragma unroll
      for (int i = 0; i < 3; ++i) K[(3 * n + i) + 27 * (3 * q + i)] += wt[n][q] * a1m;
}

// One thread per Shell_1 element of an iterating structure: Mount +
// MountElementLoads + the element's ShellLoad at the step's time; K (27x27,
// column-major, global frame) and f (P_loading) go to the element scratch.
__global__ void __launch_bounds__(64) k_shell_tangent(Batch b) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= b.sh.n_shells) return;
  int s = b.sh.sstruct[e];
  const StructState& st = b.state[s];
  if (!iterating_s(st)) return;
  double* K = b.sh.Ke + (int64_t)e * 729;
  double d[27], f[27];
  gather_d(b, e, d);
  shell_mount(b.sh.sconst[e], b.sh.shist[e], d, K, f);
  int pt = b.sh.spress[e];
  if (pt >= 0) {
    const int* nd = b.sh.snodes + 6 * e;
    double pu[18];
    for (int a = 0; a < 18; ++a) {
      int64_t q = (int64_t)nd[a / 3] * 6 + a % 3;
      pu[a] = b.copy[q] - b.xref[q] + d[a];  // xref: reference positions, 6 per node
    }
    shell_pressure(b.sh.sconst[e], pu, table_value(b, pt, st.time), b.sh.sarea[e] != 0, K, f);
  }
  const StructParams& pr = b.params[s];
  if (pr.dynamic) {
    // Rayleigh damping: on the iterations that form C_e, the stiffness
    // (with the pressure tangent, as MountLoads precedes MountDamping) goes
    // to the damping scratch, where k_shell_rayleigh turns it into
    // C_e = alpha M_modal + beta K_e
    if (pr.ray_on && (pr.ray_update || !st.ray_init)) {
      double* C = b.sh.RD + e;
      const int64_t ns = b.sh.n_shells;
#pragma unroll 1
      for (int q = 0; q < 729; ++q) C[q * ns] = K[q];
    }
    const int* nd = b.sh.snodes + 6 * e;
    double vel[36], acc[36];
#pragma unroll
    for (int j = 0; j < 6; ++j)
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        vel[6 * j + q] = b.copy_vel[(int64_t)nd[j] * 6 + q];
        acc[6 * j + q] = b.copy_accel[(int64_t)nd[j] * 6 + q];
      }
    shell_inertia(b.sh.sconst[e], b.sh.saux[e], d, vel, acc, st.a, K, f);
  }
  double* F = b.sh.Fe + (int64_t)e * 27;
#pragma unroll
  for (int a = 0; a < 27; ++a) F[a] = f[a];
}

// MountDamping and the damping part of MountDyn (reference
// src/Shell_1.cpp:2501-2541).  On the iterations that form it (the step's
// first, or every one with Update 1), C_e = alpha M_modal + beta K_e.  The
// modal mass is MountMassModal (src/Shell_1.cpp:2368-2396) over the
// six-point rule: at each point the rotation vector interpolated from the
// midside nodes' accumulated rotations (copy_coordinates 3..5) gives the
// director d = Q e3r, and EvaluateMassModal (src/Shell_1.cpp:3171-) the
// 6x6 operator blockdiag(coef1 I, coef2 (|d|^2 I - d d^T) + coef3 d d^T);
// the element sums w N^T D N and turns it to the global frame.  Every
// iteration then adds a4 C_e to K_e and C_e v to f_e, v the nodes' current
// velocities.  One warp per element, lane r < 27 owning row r of C_e, K_e
// and f_e (no lane reads another's row); C_e is structure-of-arrays.
// Row r of element e's modal mass (MountMassModal over the six-point rule,
// reference src/Shell_1.cpp:2368-2396, 3171-), global frame, into row[27].
__device__ void shell_modal_row(const Batch& b, int e, int r, double* row) {
  const ShellConst& c = b.sh.sconst[e];
  const int* nd = b.sh.snodes + 6 * e;
  const int n = r / 3, i = r % 3;  // row block (node 0..5 translations, 6..8 midside rotations), row in it
#pragma unroll
  for (int x = 0; x < 27; ++x) row[x] = 0.0;
  if (n < 6) {
    // translations: coef1 times the weights on the diagonal of each 3x3
    // node block (T^T I T = I)
#pragma unroll 1
    for (int q = 0; q < 6; ++q) {
      double w = 0.0;
#pragma unroll
      for (int k = 0; k < 6; ++k) w += c.w4[k] * c.N4[k][n] * c.N4[k][q];
      row[3 * q + i] = c.coef1 * w;
    }
  } else {
    // rotations of midside node m: row i of T^T R[m][q] T for q = 0..2
    const int m = n - 6;
    const m3 T = ld3(c.T3);
    double R[3][9];
#pragma unroll
    for (int q = 0; q < 3; ++q)
#pragma unroll
      for (int x = 0; x < 9; ++x) R[q][x] = 0.0;
#pragma unroll 1
    for (int k = 0; k < 6; ++k) {
      v3 al = {{0, 0, 0}};
#pragma unroll
      for (int mm = 0; mm < 3; ++mm)
#pragma unroll
        for (int j = 0; j < 3; ++j) al[j] += b.copy[(int64_t)nd[3 + mm] * 6 + 3 + j] * c.Na4[k][mm];
      al = mv(T, al);
      const m3 Q = rodrigues(al);
      const v3 dv = {{Q[2], Q[5], Q[8]}};
      const double d2 = dot(dv, dv);
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const double w = c.w4[k] * c.Na4[k][m] * c.Na4[k][q];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int j = 0; j < 3; ++j)
            R[q][a * 3 + j] += w * ((a == j ? c.coef2 * d2 : 0.0) + (c.coef3 - c.coef2) * dv[a] * dv[j]);
      }
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      m3 Rq;
#pragma unroll
      for (int x = 0; x < 9; ++x) Rq[x] = R[q][x];
      const m3 G = tmul(T, mul(Rq, T));
#pragma unroll
      for (int j = 0; j < 3; ++j) row[18 + 3 * q + j] = G[i * 3 + j];
    }
  }
}

__global__ void __launch_bounds__(128) k_shell_rayleigh(Batch b) {
  const int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int r = threadIdx.x & 31;
  if (e >= b.sh.n_shells || r >= 27) return;
  const int s = b.sh.sstruct[e];
  const StructState& st = b.state[s];
  if (!iterating_s(st)) return;
  const StructParams& p = b.params[s];
  if (!p.dynamic || !p.ray_on) return;
  const int64_t ns = b.sh.n_shells;
  double* C = b.sh.RD + e;
  const int* nd = b.sh.snodes + 6 * e;
  if (p.ray_update || !st.ray_init) {
    double row[27];
    shell_modal_row(b, e, r, row);
#pragma unroll 1
    for (int x = 0; x < 27; ++x) {
      const int64_t xi = r + 27 * x;
      C[xi * ns] = p.ray_alpha * row[x] + p.ray_beta * C[xi * ns];
    }
  }
  const double a4 = st.a[3];
  double* K = b.sh.Ke + (int64_t)e * 729;
  double acc = 0.0;
#pragma unroll 1
  for (int x = 0; x < 27; ++x) {
    const int node = x < 18 ? nd[x / 3] : nd[3 + (x - 18) / 3];
    const int k = x < 18 ? x % 3 : 3 + (x - 18) % 3;
    const double cx = C[(int64_t)(r + 27 * x) * ns];
    acc += cx * b.vel[(int64_t)node * 6 + k];
    K[r + 27 * x] += a4 * cx;
  }
  b.sh.Fe[(int64_t)e * 27 + r] += acc;
}

// The modal mass of every Shell_1 element of colour class `color` added into
// the band M (entry (i, j) at (kw + i - j) + j W, free indices of b.gl):
// one thread per element, elements of a colour share no node.
__global__ void k_modal_mass_shell(Batch b, int color, double* M, int64_t W, int kw) {
  const int k = b.sh.color_off[color] + blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= b.sh.color_off[color + 1]) return;
  const int e = b.sh.color_elems[k];
  const int* nd = b.sh.snodes + 6 * e;
  int g[27];
#pragma unroll 1
  for (int x = 0; x < 27; ++x) {
    const int node = x < 18 ? nd[x / 3] : nd[3 + (x - 18) / 3];
    g[x] = b.gl[(int64_t)node * 6 + (x < 18 ? x % 3 : 3 + (x - 18) % 3)];
  }
#pragma unroll 1
  for (int r = 0; r < 27; ++r) {
    if (g[r] < 0) continue;
    double row[27];
    shell_modal_row(b, e, r, row);
#pragma unroll 1
    for (int x = 0; x < 27; ++x)
      if (g[x] >= 0 && abs(g[r] - g[x]) <= kw) M[(kw + g[r] - g[x]) + (int64_t)g[x] * W] += row[x];
  }
}

void launch_shell_modal_mass(const Batch& b, double* M, int64_t W, int kw, cudaStream_t st) {
  for (int c = 0; c < b.sh.n_colors; ++c) {
    const int cnt = b.sh.color_off[c + 1] - b.sh.color_off[c];
    if (cnt > 0) k_modal_mass_shell<<<(cnt + 63) / 64, 64, 0, st>>>(b, c, M, W, kw);
  }
}

// Standalone elements (gf_shell_elements): n elements with their own
// constants, history and increments d ([n][27]); with pressure p[e] (NaN:
// none) at the displacement pu ([n][18]).
__global__ void __launch_bounds__(64) k_shell_elements(int n, const ShellConst* cs, const ShellHist* hs,
                                                       const double* ds, const double* pus, const double* ps,
                                                       int area_update, double* Ks, double* fs) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double d[27], f[27];
  for (int a = 0; a < 27; ++a) d[a] = ds[(int64_t)e * 27 + a];
  double* K = Ks + (int64_t)e * 729;
  shell_mount(cs[e], hs[e], d, K, f);
  double p = ps[e];
  if (p == p) {
    double pu[18];
    for (int a = 0; a < 18; ++a) pu[a] = pus[(int64_t)e * 18 + a];
    shell_pressure(cs[e], pu, p, area_update != 0, K, f);
  }
  for (int a = 0; a < 27; ++a) fs[(int64_t)e * 27 + a] = f[a];
}

// MountGlobal: one warp per element of one colour (no two elements of a
// colour share a node, so no two writers meet).  The element's free DOFs
// (structure-local, in the structure's reverse Cuthill-McKee numbering) go
// to the wide band and to P.
__global__ void k_shell_scatter(Batch b, int color) {
  int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int lo = b.sh.color_off[color], hi = b.sh.color_off[color + 1];
  if (lo + w >= hi) return;
  int e = b.sh.color_elems[lo + w];
  int s = b.sh.sstruct[e];
  if (!iterating_s(b.state[s])) return;
  const StructInfo& inf = b.info[s];
  const int* nd = b.sh.snodes + 6 * e;
  int myg = -1;
  if (lane < 27) {
    int node = lane < 18 ? nd[lane / 3] : nd[3 + (lane - 18) / 3];
    int k = lane < 18 ? lane % 3 : 3 + (lane - 18) % 3;
    myg = b.gl[(int64_t)node * 6 + k];
  }
  const double* K = b.sh.Ke + (int64_t)e * 729;
  const double* F = b.sh.Fe + (int64_t)e * 27;
  double* band = b.sh.wband + inf.wb_off;
  const int kl = inf.wkl;
  const int64_t W = 2 * kl + 1;
  if (lane < 27 && myg >= 0) b.P[inf.dof_off + myg] += F[lane];
  for (int base = 0; base < 729; base += 32) {
    int idx = base + lane;
    bool valid = idx < 729;
    int r = valid ? idx % 27 : 0, q = valid ? idx / 27 : 0;
    int gr = __shfl_sync(0xffffffffu, myg, r);
    int gq = __shfl_sync(0xffffffffu, myg, q);
    if (valid && gr >= 0 && gq >= 0) band[(kl + gr - gq) + (int64_t)gq * W] += K[idx];
  }
}

// SaveLagrange at the converged increment d.
__device__ void shell_commit(const ShellConst& c, ShellHist& h, ShellHistAux& x, const double* d) {
  for (int g = 0; g < 3; ++g) {
    SGp k;
    shell_gp(c, h, d, g, k);
    v3 ai = {{x.alpha[g][0], x.alpha[g][1], x.alpha[g][2]}};
    v3 an = rodrigues_compose(k.al, ai);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      h.k1[g][j] = k.k1[j];
      h.k2[g][j] = k.k2[j];
      h.z1[g][j] = k.z1[j];
      h.z2[g][j] = k.z2[j];
      x.u[g][j] += k.u[j];
      x.alpha[g][j] = an[j];
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) h.Q[g][q] = k.Q[q];
  }
}

// SaveLagrange of the structures that converged this pass.
__global__ void k_shell_commit(Batch b) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= b.sh.n_shells) return;
  int s = b.sh.sstruct[e];
  if (!b.state[s].commit) return;
  ShellHist h = b.sh.shist[e];
  ShellHistAux x = b.sh.saux[e];
  double d[27];
  gather_d(b, e, d);
  shell_commit(b.sh.sconst[e], h, x, d);
  b.sh.shist[e] = h;
  b.sh.saux[e] = x;
}

__global__ void k_shell_commit_elements(int n, const ShellConst* cs, ShellHist* hs, ShellHistAux* xs,
                                        const double* ds) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  ShellHist h = hs[e];
  ShellHistAux x = xs[e];
  double d[27];
  for (int a = 0; a < 27; ++a) d[a] = ds[(int64_t)e * 27 + a];
  shell_commit(cs[e], h, x, d);
  hs[e] = h;
  xs[e] = x;
}

// ---------------------------------------------------------------------------
// Wide-band LU.  Band pointer and geometry of wide structure w.
namespace {
struct WB {
  double* a;
  int n, kl;
  int64_t W;
  __device__ __forceinline__ double& at(int i, int j) const { return a[(kl + i - j) + (int64_t)j * W]; }
};

__device__ __forceinline__ bool wide_active(const Batch& b, int s) {
  const StructState& st = b.state[s];
  return iterating_s(st) && st.need_solve;
}

__device__ __forceinline__ WB wb_of(const Batch& b, const StructInfo& inf) {
  WB w;
  w.a = b.sh.wband + inf.wb_off;
  w.n = inf.n_free;
  w.kl = inf.wkl;
  w.W = 2 * (int64_t)inf.wkl + 1;
  return w;
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
__global__ void __launch_bounds__(DIAG_THREADS) k_wb_diag(Batch b, int p) {
  p = wb_panel(b, p);
  if (p < 0) return;
  int s = b.sh.wide_structs[blockIdx.x];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WB w = wb_of(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  __shared__ double Ac[NB][NB + 1];  // Ac[j][i] = A(i, j)
  __shared__ int fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) fail = 0;
  // this panel's L21 / U12 maxima start at zero (the buffer of its parity
  // was last read by the slicing of panel p - 2, which precedes this kernel)
  if (b.sh.wide_tc && tid < 2 * NB) wb_kmax(b, blockIdx.x, p)[tid] = 0ull;
  for (int x = tid; x < NB * NB; x += blockDim.x) {
    const int i = x % NB, j = x / NB;
    double v = 0.0;
    if (i < nb && j < nb && abs(i - j) <= w.kl) v = w.at(j0 + i, j0 + j);
    Ac[j][i] = v;
  }
  __syncthreads();
  if (warp == 8 && nb > 0) {  // the multipliers of column 0
    const double piv = Ac[0][0];
    if (lane == 0 && (!(piv != 0.0) || !isfinite(piv))) fail = 1;
    const double r = wb_recip(piv);
    if (1 + lane < nb) Ac[0][1 + lane] *= r;
    if (33 + lane < nb) Ac[0][33 + lane] *= r;
  }
  __syncthreads();
  for (int k = 0; k + 1 < nb; ++k) {
    const int m = nb - 1 - k;  // trailing rows and columns
    if (warp == 8) {
      // column k + 1: its update, then the next pivot and multipliers
      const int j = k + 1, i0 = j + lane, i1 = i0 + 32;
      const double u = Ac[j][k];
      if (i0 < nb) Ac[j][i0] = fma(-Ac[k][i0], u, Ac[j][i0]);
      if (i1 < nb) Ac[j][i1] = fma(-Ac[k][i1], u, Ac[j][i1]);
      __syncwarp();
      const double piv = Ac[j][j];
      if (lane == 0 && (!(piv != 0.0) || !isfinite(piv))) fail = 1;
      const double r = wb_recip(piv);
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
        Ac[j][i] = fma(-Ac[k][i], Ac[j][k], Ac[j][i]);
      }
    }
    __syncthreads();
  }
  for (int x = tid; x < nb * nb; x += blockDim.x) {
    const int i = x % nb, j = x / nb;
    if (abs(i - j) <= w.kl) w.at(j0 + i, j0 + j) = Ac[j][i];
  }
  if (tid == 0 && fail) b.state[s].info_fail = 1;
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
constexpr int TRSM_RB = 8;
constexpr int TRSM_RB_FIRST = 2;
template <int RB>
__global__ void __launch_bounds__(32 * RB) k_wb_trsm(Batch b, int p, int row0, int nblk) {
  p = wb_panel(b, p);
  if (p < 0) return;
  int s = b.sh.wide_structs[blockIdx.y];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WB w = wb_of(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  const int m = min(w.kl, w.n - j0 - nb);  // rows below / columns right of the panel
  if (m <= 0) return;
  const bool lower = (int)blockIdx.x < nblk;
  const int rowb = row0 + RB * (lower ? (int)blockIdx.x : (int)blockIdx.x - nblk);
  if (rowb >= m) return;
  __shared__ double T[NB][NB + 1];  // the diagonal block's LU (the half this side reads)
  __shared__ double X[RB][NB + 1];
  __shared__ double rd[NB];         // reciprocals of U11's diagonal
  const int tid = threadIdx.x;
  for (int x = tid; x < NB * NB; x += blockDim.x) {
    int i = x % NB, j = x / NB;
    T[i][j] = ((lower ? i <= j : i > j) && i < nb && j < nb && abs(i - j) <= w.kl) ? w.at(j0 + i, j0 + j) : 0.0;
  }
  if (lower && tid < nb) rd[tid] = wb_recip(w.at(j0 + tid, j0 + tid));
  const int r = tid >> 5, c = tid & 31;  // row (or column) r of the block, lane c
  const int g = j0 + nb + rowb + r;      // global row (lower) or column (upper)
  const bool live = g < j0 + nb + m;
  for (int k = c; k < NB; k += 32) {
    double v = 0.0;
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
  double v0 = X[r][c], v1 = X[r][c + 32];
  if (lower) {
    // x U11 = a: x_k = a_k / u_kk, then a_j -= x_k u_kj (j > k)
    for (int k = 0; k < nb; ++k) {
      const double xk = __shfl_sync(0xffffffffu, k < 32 ? v0 : v1, k & 31) * rd[k];
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
      const double yk = __shfl_sync(0xffffffffu, k < 32 ? v0 : v1, k & 31);
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
  if (b.sh.wide_tc && tid < nb) {
    // largest magnitude of column k of this block's L21 rows (row k of its
    // U12 columns), as FP64 bits, which order like the magnitudes; the
    // maximum over the CTAs is exact and independent of their order
    const int k = tid;
    unsigned long long mx = 0;
    for (int q = 0; q < RB; ++q) {
      const int gq = j0 + nb + rowb + q;
      if (gq < j0 + nb + m && gq - (j0 + k) <= w.kl)
        mx = max(mx, (unsigned long long)__double_as_longlong(X[q][k]) & 0x7FFFFFFFFFFFFFFFull);
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
// path.  8 x 8 output tiles over 64 CTAs; in a CTA four warps each sum a
// quarter of k (16 terms) for all 64 outputs of the tile, and the quarters
// are added in a fixed order: an FP64 warp instruction holds its
// sub-partition's FP64 unit for about 64 cycles, so four warps on four
// sub-partitions finish the 64 terms four times sooner than one.
constexpr int CT8 = 8;
constexpr int CORNER_THREADS = 256;
__global__ void __launch_bounds__(CORNER_THREADS) k_wb_corner(Batch b, int p) {
  p = wb_panel(b, p);
  if (p < 0) return;
  int s = b.sh.wide_structs[blockIdx.z];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WB w = wb_of(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  const int m = min(min(w.kl, w.n - j0 - nb), NB);
  const int r0 = blockIdx.x * CT8, c0 = blockIdx.y * CT8;
  if (r0 >= m || c0 >= m) return;
  __shared__ double Ls[NB][CT8 + 1];  // [k][row]
  __shared__ double Us[NB][CT8 + 1];  // [k][col]
  __shared__ double part[4][CT8 * CT8];
  const int tid = threadIdx.x;
  const int base = j0 + nb;
  for (int x = tid; x < NB * CT8; x += blockDim.x) {
    // rows of L21 along a band column are contiguous; U12's k along a
    // band column too
    const int i = x % CT8, k = x / CT8;
    const int gk = j0 + k, gi = base + r0 + i;
    Ls[k][i] = (k < nb && r0 + i < m && gi - gk <= w.kl) ? w.at(gi, gk) : 0.0;
    const int kk = x % NB, c = x / NB, gj = base + c0 + c;
    Us[kk][c] = (kk < nb && c0 + c < m && gj - (j0 + kk) <= w.kl) ? w.at(j0 + kk, gj) : 0.0;
  }
  __syncthreads();
  const int o = tid & 63, q = tid >> 6;  // output, quarter of k
  const int ty = o / CT8, tx = o % CT8;
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

// Forward substitution for panel p: y_p = L11^-1 b_p into y; then the rows
// below the panel: P_i -= L21(i, :) y_p.  Every CTA solves the small
// triangle redundantly; CTA 0 writes y_p.
__global__ void __launch_bounds__(256) k_wb_fwd(Batch b, int p) {
  p = wb_panel(b, p);
  if (p < 0) return;
  int s = b.sh.wide_structs[blockIdx.y];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WB w = wb_of(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  const int m = min(w.kl, w.n - j0 - nb);
  // right-hand side blockIdx.z of a multi-column solve (columns rhs_ld apart)
  double* P = b.P + inf.dof_off + (int64_t)blockIdx.z * b.rhs_ld;
  double* Y = b.y + inf.dof_off + (int64_t)blockIdx.z * b.rhs_ld;
  __shared__ double T[NB][NB + 1];  // the panel's diagonal block (L11 below the diagonal)
  __shared__ double ys[NB];
  const int tid = threadIdx.x;
  for (int x = tid; x < NB * NB; x += blockDim.x) {
    int i = x % NB, j = x / NB;
    T[i][j] = (i < nb && j < nb && abs(i - j) <= w.kl) ? w.at(j0 + i, j0 + j) : 0.0;
  }
  __syncthreads();
  if (tid < 32) {
    // lanes hold entries k = lane and lane + 32
    double v0 = tid < nb ? P[j0 + tid] : 0.0, v1 = tid + 32 < nb ? P[j0 + tid + 32] : 0.0;
    for (int k = 0; k < nb; ++k) {
      double yk = __shfl_sync(0xffffffffu, k < 32 ? v0 : v1, k & 31);
      if (tid > k) v0 -= T[tid][k] * yk;
      if (tid + 32 > k) v1 -= T[tid + 32][k] * yk;
    }
    ys[tid] = v0;
    ys[tid + 32] = v1;
  }
  __syncthreads();
  if (blockIdx.x == 0)
    for (int k = tid; k < nb; k += blockDim.x) Y[j0 + k] = ys[k];
  int i = nb + blockIdx.x * blockDim.x + tid;  // row offset from j0
  if (i < nb + m && j0 + i < w.n) {
    double acc = 0.0;
    for (int k = 0; k < nb; ++k)
      if (i - k <= w.kl) acc = fma(w.at(j0 + i, j0 + k), ys[k], acc);
    P[j0 + i] -= acc;
  }
}

// Backward substitution for panel p (last panel first): x_p = U11^-1 y_p into
// P; then the rows above the panel: y_i -= U(i, panel) x_p.
__global__ void __launch_bounds__(256) k_wb_bwd(Batch b, int p) {
  p = wb_panel(b, p);
  if (p < 0) return;
  int s = b.sh.wide_structs[blockIdx.y];
  if (!wide_active(b, s)) return;
  const StructInfo& inf = b.info[s];
  if (p >= inf.n_panels) return;
  WB w = wb_of(b, inf);
  const int j0 = p * NB, nb = min(NB, w.n - j0);
  // right-hand side blockIdx.z of a multi-column solve (columns rhs_ld apart)
  double* P = b.P + inf.dof_off + (int64_t)blockIdx.z * b.rhs_ld;
  double* Y = b.y + inf.dof_off + (int64_t)blockIdx.z * b.rhs_ld;
  __shared__ double T[NB][NB + 1];  // the panel's diagonal block (U11 on and above the diagonal)
  __shared__ double rdiag[NB];
  __shared__ double xs[NB];
  const int tid = threadIdx.x;
  for (int x = tid; x < NB * NB; x += blockDim.x) {
    int i = x % NB, j = x / NB;
    T[i][j] = (i < nb && j < nb && abs(i - j) <= w.kl) ? w.at(j0 + i, j0 + j) : 0.0;
  }
  __syncthreads();
  if (tid < nb) rdiag[tid] = wb_recip(T[tid][tid]);
  __syncthreads();
  if (tid < 32) {
    double v0 = tid < nb ? Y[j0 + tid] : 0.0, v1 = tid + 32 < nb ? Y[j0 + tid + 32] : 0.0;
    for (int k = nb - 1; k >= 0; --k) {
      double mine = k < 32 ? v0 : v1;
      double xk = __shfl_sync(0xffffffffu, mine, k & 31) * rdiag[k];
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
  const int top = max(0, j0 - w.kl);
  int i = top + blockIdx.x * blockDim.x + tid;
  if (i < j0) {
    double acc = 0.0;
    for (int k = 0; k < nb; ++k)
      if (j0 + k - i <= w.kl) acc = fma(w.at(i, j0 + k), xs[k], acc);
    Y[i] -= acc;
  }
}

void launch_shell_mount(const Batch& b, cudaStream_t st) {
  if (b.sh.n_shells == 0) return;
  k_shell_tangent<<<(b.sh.n_shells + 63) / 64, 64, 0, st>>>(b);
  if (b.sh.any_rayleigh) k_shell_rayleigh<<<(b.sh.n_shells + 3) / 4, 128, 0, st>>>(b);
  for (int c = 0; c < b.sh.n_colors; ++c) {
    int cnt = b.sh.color_off[c + 1] - b.sh.color_off[c];
    if (cnt <= 0) continue;
    k_shell_scatter<<<(cnt + 3) / 4, 128, 0, st>>>(b, c);
  }
}

void launch_wide_zero(const Batch& b, cudaStream_t st) {
  if (b.sh.n_wide == 0) return;
  k_wb_zero<<<dim3(4 * 152, b.sh.n_wide), 256, 0, st>>>(b);
}

// The trsm of a panel: the first NB rows and columns (the next panel's
// diagonal block needs them) in CTAs of TRSM_RB_FIRST, the rest in CTAs of
// TRSM_RB.
constexpr int TRSM_FIRST = NB / TRSM_RB_FIRST;
__host__ __device__ constexpr int trsm_rest_blocks(int kl) { return kl > NB ? (kl - NB + TRSM_RB - 1) / TRSM_RB : 0; }

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
    k_wb_corner<<<dim3(NB / CT8, NB / CT8, nw), CORNER_THREADS, 0, st>>>(b, p);
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
// Appends a WHILE conditional node to the capture of st (its condition
// starts at 1 on every launch) and returns its body graph, into which the
// caller captures one loop iteration.
cudaError_t add_while(cudaStream_t st, cudaGraphConditionalHandle* h, cudaGraph_t* body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd);
  if (e != cudaSuccess) return e;
  std::vector<cudaGraphNode_t> dv(deps, deps + nd);
  if ((e = cudaGraphConditionalHandleCreate(h, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = *h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  if ((e = cudaGraphAddNode(&node, g, dv.data(), nullptr, dv.size(), &np)) != cudaSuccess) return e;
  *body = np.conditional.phGraph_out[0];
  return cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
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
// the unrolled form.
static cudaError_t capture_wide_loops(const Batch& b, cudaStream_t st) {
  const ShellData& sd = b.sh;
  const int nw = sd.n_wide, mr = sd.max_kl, P = sd.max_panels;
  const int nrest = trsm_rest_blocks(mr), rb = (mr + 255) / 256;
  cudaStream_t sb = sd.aux[2], s2 = sd.aux[0], s3 = sd.aux[1], s4 = sd.aux[3];
  cudaEvent_t e_start = sd.evt[0], e_trsm = sd.evt[1], e_corner = sd.evt[2], e_diag = sd.evt[3], e_fwd = sd.evt[4],
              e_rest = sd.evt[5];
  if (P <= 0) return cudaSuccess;
  cudaError_t e;
  cudaGraphConditionalHandle h;
  cudaGraph_t body, done;
  k_wb_loop_set<<<1, 1, 0, st>>>(sd.panel, 0);
  k_wb_diag<<<nw, DIAG_THREADS, 0, st>>>(b, 0);
  if ((e = add_while(st, &h, &body)) != cudaSuccess) return e;
  if ((e = cudaStreamBeginCaptureToGraph(sb, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
    return e;
  if (nrest) {
    cudaEventRecord(e_start, sb);
    cudaStreamWaitEvent(s4, e_start, 0);
    k_wb_trsm<TRSM_RB><<<dim3(2 * nrest, nw), 32 * TRSM_RB, 0, s4>>>(b, -1, NB, nrest);
    cudaEventRecord(e_rest, s4);
  }
  k_wb_trsm<TRSM_RB_FIRST><<<dim3(2 * TRSM_FIRST, nw), 32 * TRSM_RB_FIRST, 0, sb>>>(b, -1, 0, TRSM_FIRST);
  launch_wb_update(b, -1, 1, sb);
  cudaEventRecord(e_corner, sb);
  cudaStreamWaitEvent(s2, e_corner, 0);
  k_wb_diag<<<nw, DIAG_THREADS, 0, s2>>>(b, -2);
  cudaEventRecord(e_diag, s2);
  if (nrest) cudaStreamWaitEvent(sb, e_rest, 0);
  cudaEventRecord(e_trsm, sb);
  cudaStreamWaitEvent(s3, e_trsm, 0);
  k_wb_fwd<<<dim3(rb, nw), 256, 0, s3>>>(b, -1);
  cudaEventRecord(e_fwd, s3);
  launch_wb_update(b, -1, 2, sb);
  cudaStreamWaitEvent(sb, e_diag, 0);
  cudaStreamWaitEvent(sb, e_fwd, 0);
  k_wb_loop_step<<<1, 1, 0, sb>>>(sd.panel, 1, P, h);
  if ((e = cudaStreamEndCapture(sb, &done)) != cudaSuccess) return e;
  k_wb_loop_set<<<1, 1, 0, st>>>(sd.panel, P - 1);
  if ((e = add_while(st, &h, &body)) != cudaSuccess) return e;
  if ((e = cudaStreamBeginCaptureToGraph(sb, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
    return e;
  k_wb_bwd<<<dim3(rb, nw), 256, 0, sb>>>(b, -1);
  k_wb_loop_step<<<1, 1, 0, sb>>>(sd.panel, -1, P, h);
  return cudaStreamEndCapture(sb, &done);
}

void launch_wide_solve(const Batch& b, cudaStream_t st, LaunchProf* prof) {
  if (b.sh.n_wide == 0) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (!prof && b.sh.loops_in_graph && b.sh.panel && cudaStreamIsCapturing(st, &cs) == cudaSuccess &&
      cs == cudaStreamCaptureStatusActive) {
    // an error here invalidates the capture, which the caller's end of
    // capture reports
    capture_wide_loops(b, st);
    return;
  }
  const ShellData& sd = b.sh;
  const int nw = sd.n_wide;
  const int mr = sd.max_kl;  // largest kl over the wide structures
  const int nrest = trsm_rest_blocks(mr);
  const int rb = (mr + 255) / 256;
  cudaStream_t s2 = sd.aux[0], s3 = sd.aux[1], s4 = sd.aux[3];
  // the helpers fork from the main stream at their first wait and join it
  // again before the backward substitution
  cudaEvent_t e_start = sd.evt[0], e_trsm = sd.evt[1], e_corner = sd.evt[2], e_diag = sd.evt[3], e_fwd = sd.evt[4],
              e_rest = sd.evt[5];
  { ProfScope q(prof, st, KC_WIDE_DIAG); k_wb_diag<<<nw, DIAG_THREADS, 0, st>>>(b, 0); }
  for (int p = 0; p < sd.max_panels; ++p) {
    bool next = p + 1 < sd.max_panels;
    if (nrest) {
      cudaEventRecord(e_start, st);
      cudaStreamWaitEvent(s4, e_start, 0);
      ProfScope q(prof, s4, KC_WIDE_TRSM);
      k_wb_trsm<TRSM_RB><<<dim3(2 * nrest, nw), 32 * TRSM_RB, 0, s4>>>(b, p, NB, nrest);
      cudaEventRecord(e_rest, s4);
    }
    {
      ProfScope q(prof, st, KC_WIDE_TRSM);
      k_wb_trsm<TRSM_RB_FIRST><<<dim3(2 * TRSM_FIRST, nw), 32 * TRSM_RB_FIRST, 0, st>>>(b, p, 0, TRSM_FIRST);
    }
    if (next) {
      { ProfScope q(prof, st, KC_WIDE_UPDATE); launch_wb_update(b, p, 1, st); }
      cudaEventRecord(e_corner, st);
      cudaStreamWaitEvent(s2, e_corner, 0);
      { ProfScope q(prof, s2, KC_WIDE_DIAG); k_wb_diag<<<nw, DIAG_THREADS, 0, s2>>>(b, p + 1); }
      cudaEventRecord(e_diag, s2);
    }
    if (nrest) cudaStreamWaitEvent(st, e_rest, 0);
    cudaEventRecord(e_trsm, st);
    cudaStreamWaitEvent(s3, e_trsm, 0);
    { ProfScope q(prof, s3, KC_WIDE_SUBST); k_wb_fwd<<<dim3(rb, nw), 256, 0, s3>>>(b, p); }
    if (next) {
      { ProfScope q(prof, st, KC_WIDE_UPDATE); launch_wb_update(b, p, 2, st); }
      cudaStreamWaitEvent(st, e_diag, 0);
    } else {
      { ProfScope q(prof, st, KC_WIDE_UPDATE); launch_wb_update(b, p, 0, st); }
    }
  }
  // join: every forward step is done before the backward substitution
  cudaEventRecord(e_fwd, s3);
  cudaStreamWaitEvent(st, e_fwd, 0);
  for (int p = sd.max_panels - 1; p >= 0; --p) {
    ProfScope q(prof, st, KC_WIDE_SUBST);
    k_wb_bwd<<<dim3(rb, nw), 256, 0, st>>>(b, p);
  }
}

// Forward and backward substitution alone on a wide band that already holds
// its LU (a factor from launch_wide_solve), for nrhs right-hand sides at
// b.P + q b.rhs_ld (q < nrhs, scratch alike in b.y): the panel loops of
// launch_wide_solve without the factor, every column per launch.
void launch_wide_subst(const Batch& b, int nrhs, cudaStream_t st) {
  if (b.sh.n_wide == 0 || nrhs <= 0) return;
  const int nw = b.sh.n_wide, rb = (b.sh.max_kl + 255) / 256;
  for (int p = 0; p < b.sh.max_panels; ++p) k_wb_fwd<<<dim3(rb, nw, nrhs), 256, 0, st>>>(b, p);
  for (int p = b.sh.max_panels - 1; p >= 0; --p) k_wb_bwd<<<dim3(rb, nw, nrhs), 256, 0, st>>>(b, p);
}

void launch_shell_elements(int n, const ShellConst* c, const ShellHist* h, const double* d, const double* pu,
                           const double* p, int area_update, double* K, double* f, cudaStream_t st) {
  if (n <= 0) return;
  k_shell_elements<<<(n + 63) / 64, 64, 0, st>>>(n, c, h, d, pu, p, area_update, K, f);
}

// Standalone inertia (gf_shell_inertia_elements): n elements with their own
// constants, history, increments d ([n][27]), converged nodal velocities v
// and accelerations a_acc ([n][36]) and Newmark coefficients a[6].
__global__ void __launch_bounds__(64) k_shell_inertia_elements(int n, const ShellConst* cs, const ShellHistAux* xs,
                                                               const double* ds, const double* vs, const double* as,
                                                               const double* a, double* Ms, double* Fs) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double d[27], vel[36], acc[36], f[27], an[6];
  for (int q = 0; q < 27; ++q) {
    d[q] = ds[(int64_t)e * 27 + q];
    f[q] = 0.0;
  }
  for (int q = 0; q < 36; ++q) {
    vel[q] = vs[(int64_t)e * 36 + q];
    acc[q] = as[(int64_t)e * 36 + q];
  }
  for (int q = 0; q < 6; ++q) an[q] = a[q];
  double* M = Ms + (int64_t)e * 729;
  for (int q = 0; q < 729; ++q) M[q] = 0.0;
  shell_inertia(cs[e], xs[e], d, vel, acc, an, M, f);
  for (int q = 0; q < 27; ++q) Fs[(int64_t)e * 27 + q] = f[q];
}

void launch_shell_inertia_elements(int n, const ShellConst* c, const ShellHistAux* x, const double* d,
                                   const double* v, const double* a_acc, const double* a, double* M, double* F,
                                   cudaStream_t st) {
  if (n > 0) k_shell_inertia_elements<<<(n + 63) / 64, 64, 0, st>>>(n, c, x, d, v, a_acc, a, M, F);
}

void launch_shell_commit_elements(int n, const ShellConst* c, ShellHist* h, ShellHistAux* x, const double* d,
                                  cudaStream_t st) {
  if (n <= 0) return;
  k_shell_commit_elements<<<(n + 127) / 128, 128, 0, st>>>(n, c, h, x, d);
}

void launch_shell_commit(const Batch& b, cudaStream_t st) {
  if (b.sh.n_shells == 0) return;
  k_shell_commit<<<(b.sh.n_shells + 127) / 128, 128, 0, st>>>(b);
}

}  // namespace gf

namespace gf {
int shell_launches_per_pass(const Batch& b) {
  int n = 0;
  if (b.sh.n_shells) {
    n += 2 + (b.sh.any_rayleigh ? 1 : 0);  // tangent (+ Rayleigh damping) + commit
    for (int c = 0; c < b.sh.n_colors; ++c) n += b.sh.color_off[c + 1] > b.sh.color_off[c];
  }
  // unrolled: the first diagonal LU, then per panel the first trsm blocks,
  // update corner + next diagonal, the other trsm blocks, forward step,
  // update rest, backward step (the last panel has no corner or next
  // diagonal); graph loops: two loop-control kernels, the first diagonal
  // LU, the same six or seven kernels and a counter step per forward
  // iteration, and two kernels per backward one
  if (b.sh.n_wide) {
    const int P = b.sh.max_panels, per = 6 + (trsm_rest_blocks(b.sh.max_kl) ? 1 : 0);
    n += (b.sh.loops_in_graph ? 3 + (per + 2) * P : 1 + per * P - 2) +
         (b.sh.wide_tc ? P : 0);  // the tensor-core update's slicing kernel
  }
  return n;
}
}  // namespace gf
