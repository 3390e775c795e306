// Shell_1 structures on the device: element tangent and internal force with
// the follower pressure and, in Dynamic steps, the inertial terms
// (k_shell_tangent), Rayleigh damping (k_shell_rayleigh), colour scatter
// into the wide band (k_shell_scatter) and SaveLagrange (k_shell_commit).
// The wide band's LU and solves are in gf_wideband.cu.
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
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

#include "gf_kernels.cuh"
#include "gf_math.cuh"
#include "gf_types.h"

namespace gf {

namespace {

__device__ __forceinline__ bool iterating_s(const StructState& s) { return s.phase == PH_ITER; }

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
  return n + wide_launches_per_pass(b);
}
}  // namespace gf
