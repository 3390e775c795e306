/*
 * Beam_1 element, CPU restatement.  TEST INFRASTRUCTURE (oracle): the
 * reference values for the CUDA element kernels and part of the timed CPU
 * baseline.
 *
 * Follows reference src/Beam_1.cpp: PreCalc 501-692 (constitutive matrix,
 * transformation, Gauss points, shape functions), Mount 695-835 (incremental
 * Rodrigues kinematics, constitutive and geometric stiffness, internal
 * force), TransformMatrix 1385-1427, SaveLagrange 1494-1506.  The products
 * DeltaN^T M DeltaN are expanded per 3x3 block instead of through dense
 * 9x18 matrices; the arithmetic is the same up to rounding order.
 */
#include "oracle_beam.h"

#include <string.h>

/* reference src/Beam_1.cpp:501-692 (Hooke material, non-special section) */
void oracle_beam_precalc(const double* x0, const double* x2, const double* mat, const double* sec,
                         const double* cs, double T0, ob_const* c, ob_hist* h) {
  double E = mat[0], nu = mat[1], rho = mat[2];
  double G = E / (2 * (1 + nu));
  double sf = 1.0;
  double A = sec[0], I1 = sec[1], I2 = sec[2], I12 = sec[3], It = sec[4], I33 = sec[5];
  memset(c, 0, sizeof(*c));
  c->D[0 * 6 + 0] = sf * G * A;
  c->D[1 * 6 + 1] = sf * G * A;
  c->D[2 * 6 + 2] = E * A;
  c->D[3 * 6 + 3] = E * I1;
  c->D[4 * 6 + 4] = E * I2;
  c->D[3 * 6 + 4] = E * I12;
  c->D[4 * 6 + 3] = E * I12;
  c->D[5 * 6 + 5] = G * It;
  c->Mr = rho * A;
  c->Jr[0] = rho * I1;
  c->Jr[4] = rho * I2;
  c->Jr[8] = rho * I33;
  c->Jr[1] = c->Jr[3] = rho * I12;
  cs_matrix(c->T3, cs);
  double e3[3] = {x2[0] - x0[0], x2[1] - x0[1], x2[2] - x0[2]};
  double len = sqrt(e3[0] * e3[0] + e3[1] * e3[1] + e3[2] * e3[2]);
  double inv = 1.0 / v3_norm(e3);
  for (int k = 0; k < 3; ++k) e3[k] = inv * e3[k];
  m3_vec(c->e3r, c->T3, e3);
  /* pre-tension T0: du0 = T0 / EA, reference length |x2 - x0| / (1 + du0),
   * dz_i = (1 + du0) e3 (reference src/Beam_1.cpp:616-621) */
  double du0 = T0 / c->D[2 * 6 + 2];
  c->jac = (len / (1.0 + du0)) / 2.0;
  for (int g = 0; g < 2; ++g) {
    double xi = g == 0 ? -0.577350269189626 : +0.577350269189626;
    c->N[g][0] = 0.5 * xi * (xi - 1.0);
    c->N[g][1] = 1.0 - xi * xi;
    c->N[g][2] = 0.5 * xi * (1.0 + xi);
    c->dN[g][0] = (1.0 / c->jac) * (xi - 0.5);
    c->dN[g][1] = (1.0 / c->jac) * (-2.0 * xi);
    c->dN[g][2] = (1.0 / c->jac) * (0.5 + xi);
  }
  if (h) {
    memset(h, 0, sizeof(*h));
    for (int g = 0; g < 2; ++g) {
      m3_eye(h->Q[g]);
      h->dz[g][2] = 1.0 + du0;
    }
  }
}

/* Gauss-point kinematics shared by Mount and SaveLagrange
 * (reference src/Beam_1.cpp:700-786). */
typedef struct {
  double alpha[3], dalpha[3], u[3], du[3];
  double an, g;
  double A[9], Qd[9], Xi[9], dXi[9], dz[3], dZ[9];
  double Qt[9]; /* (Q_delta Q_i)^T */
  double eta[3], kappa[3];
} gp_kin;

static void beam_gp_kinematics(const ob_const* c, const ob_hist* h, const double* d, int g, gp_kin* k) {
  double a[3] = {0, 0, 0}, da[3] = {0, 0, 0}, u[3] = {0, 0, 0}, du[3] = {0, 0, 0};
  for (int i = 0; i < 3; ++i)
    for (int n = 0; n < 3; ++n) {
      const double* dn = d + 6 * n;
      a[i] += dn[3 + i] * c->N[g][n];
      da[i] += dn[3 + i] * c->dN[g][n];
      u[i] += dn[i] * c->N[g][n];
      du[i] += dn[i] * c->dN[g][n];
    }
  m3_vec(k->alpha, c->T3, a);
  m3_vec(k->dalpha, c->T3, da);
  m3_vec(k->u, c->T3, u);
  m3_vec(k->du, c->T3, du);
  k->an = v3_norm(k->alpha);
  m3_skew(k->A, k->alpha);
  k->g = 4.0 / (4.0 + k->an * k->an);
  double A2[9];
  m3_mul(A2, k->A, k->A);
  for (int q = 0; q < 9; ++q) {
    k->Qd[q] = k->g * (k->A[q] + 0.5 * A2[q]);
    k->Xi[q] = k->g * 0.5 * k->A[q];
  }
  k->Qd[0] += 1.0; k->Qd[4] += 1.0; k->Qd[8] += 1.0;
  k->Xi[0] += k->g; k->Xi[4] += k->g; k->Xi[8] += k->g;
  double dA[9];
  m3_skew(dA, k->dalpha);
  double ad = v3_dot(k->alpha, k->dalpha);
  for (int q = 0; q < 9; ++q) k->dXi[q] = -0.5 * k->g * (ad * k->Xi[q] - dA[q]);
  for (int i = 0; i < 3; ++i) k->dz[i] = k->du[i] + h->dz[g][i];
  m3_skew(k->dZ, k->dz);
  double Q[9];
  m3_mul(Q, k->Qd, h->Q[g]);
  m3_transpose(k->Qt, Q);
  m3_vec(k->eta, k->Qt, k->dz);
  for (int i = 0; i < 3; ++i) k->eta[i] -= c->e3r[i];
  double t[3];
  m3_tvec(t, k->Xi, k->dalpha);
  m3_tvec(k->kappa, h->Q[g], t);
  for (int i = 0; i < 3; ++i) k->kappa[i] += h->kap[g][i];
}

/* reference src/Beam_1.cpp:695-835.  d is [3][6] nodal increments (global);
 * K is 18x18 column-major, f is 18; both are overwritten. */
void oracle_beam_mount(const ob_const* c, const ob_hist* h, const double* d, double* K, double* f,
                       double* strain_energy) {
  double Kl[18 * 18], fl[18];
  memset(Kl, 0, sizeof(Kl));
  memset(fl, 0, sizeof(fl));
  double se = 0.0;
  for (int g = 0; g < 2; ++g) {
    gp_kin k;
    beam_gp_kinematics(c, h, d, g, &k);
    /* B = B1 B2 (6x9): [[Qt, 0, Qt dZ Xi], [0, Qt Xi, Qt dXi]] */
    double B[6][9];
    memset(B, 0, sizeof(B));
    double t1[9], QdZXi[9], QXi[9], QdXi[9];
    m3_mul(t1, k.dZ, k.Xi);
    m3_mul(QdZXi, k.Qt, t1);
    m3_mul(QXi, k.Qt, k.Xi);
    m3_mul(QdXi, k.Qt, k.dXi);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        B[i][j] = k.Qt[i * 3 + j];
        B[i][6 + j] = QdZXi[i * 3 + j];
        B[3 + i][3 + j] = QXi[i * 3 + j];
        B[3 + i][6 + j] = QdXi[i * 3 + j];
      }
    /* sigma = D eps */
    double eps[6] = {k.eta[0], k.eta[1], k.eta[2], k.kappa[0], k.kappa[1], k.kappa[2]}, sig[6];
    for (int i = 0; i < 6; ++i) {
      double s = 0.0;
      for (int j = 0; j < 6; ++j) s += c->D[i * 6 + j] * eps[j];
      sig[i] = s;
    }
    /* M = B^T D B + G (9x9, row-major) */
    double DB[6][9], M[81];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 9; ++j) {
        double s = 0.0;
        for (int p = 0; p < 6; ++p) s += c->D[i * 6 + p] * B[p][j];
        DB[i][j] = s;
      }
    for (int i = 0; i < 9; ++i)
      for (int j = 0; j < 9; ++j) {
        double s = 0.0;
        for (int p = 0; p < 6; ++p) s += B[p][i] * DB[p][j];
        M[i * 9 + j] = s;
      }
    /* n = Q n_r, m = Q m_r with Q = Qt^T */
    double n[3], m[3];
    m3_tvec(n, k.Qt, sig);
    m3_tvec(m, k.Qt, sig + 3);
    double dZn[3], V1[9], V2[9], dV[9], Sn[9], Sm[9];
    m3_vec(dZn, k.dZ, n);
    op_V(V1, k.alpha, dZn, k.an);
    op_V(V2, k.alpha, m, k.an);
    op_dV(dV, k.alpha, k.dalpha, m, k.an);
    m3_skew(Sn, n);
    m3_skew(Sm, m);
    double Gua[9], Gau[9], Gaa[9], Gda[9], tmp[9], tmp2[9];
    m3_mul(Gua, Sn, k.Xi);
    for (int q = 0; q < 9; ++q) Gua[q] = -Gua[q];
    m3_tmul(Gau, k.Xi, Sn);
    m3_mul(tmp, k.dZ, Sn);
    m3_mul(tmp2, tmp, k.Xi);
    m3_tmul(Gaa, k.Xi, tmp2);
    m3_mul(tmp, Sm, k.Xi);
    m3_tmul(tmp2, k.dXi, tmp);
    for (int q = 0; q < 9; ++q) Gaa[q] = Gaa[q] - V1[q] + dV[q] - tmp2[q];
    m3_tmul(tmp2, k.Xi, tmp);
    for (int q = 0; q < 9; ++q) Gda[q] = V2[q] - tmp2[q];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        M[i * 9 + 6 + j] += Gua[i * 3 + j];
        M[(6 + i) * 9 + j] += Gau[i * 3 + j];
        M[(6 + i) * 9 + 6 + j] += Gaa[i * 3 + j];
        M[(3 + i) * 9 + 6 + j] += Gda[i * 3 + j];
        M[(6 + i) * 9 + 3 + j] += V2[i * 3 + j];
      }
    /* K += wJ DeltaN^T M DeltaN; DeltaN maps node I's (u, alpha) to
     * (u', alpha', alpha) = (dN_I u, dN_I alpha, N_I alpha) */
    double wJ = 1.0 * c->jac;
    const double* N = c->N[g];
    const double* dN = c->dN[g];
    for (int I = 0; I < 3; ++I)
      for (int J = 0; J < 3; ++J)
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) {
            double m00 = M[a * 9 + b], m01 = M[a * 9 + 3 + b], m02 = M[a * 9 + 6 + b];
            double m10 = M[(3 + a) * 9 + b], m11 = M[(3 + a) * 9 + 3 + b], m12 = M[(3 + a) * 9 + 6 + b];
            double m20 = M[(6 + a) * 9 + b], m21 = M[(6 + a) * 9 + 3 + b], m22 = M[(6 + a) * 9 + 6 + b];
            double uu = dN[I] * dN[J] * m00;
            double ua = dN[I] * (dN[J] * m01 + N[J] * m02);
            double au = (dN[I] * m10 + N[I] * m20) * dN[J];
            double aa = dN[I] * dN[J] * m11 + dN[I] * N[J] * m12 + N[I] * dN[J] * m21 + N[I] * N[J] * m22;
            int r = 6 * I + a, s = 6 * J + b;
            Kl[r + 18 * s] += wJ * uu;
            Kl[r + 18 * (s + 3)] += wJ * ua;
            Kl[(r + 3) + 18 * s] += wJ * au;
            Kl[(r + 3) + 18 * (s + 3)] += wJ * aa;
          }
    /* f += wJ DeltaN^T B^T sigma; B^T sigma = [n; Xi^T m; Xi^T dZ^T n + dXi^T m] */
    double s0[3] = {n[0], n[1], n[2]}, s1[3], s2[3], a1[3], a2[3];
    m3_tvec(s1, k.Xi, m);
    m3_tvec(a1, k.dZ, n);
    m3_tvec(a2, k.Xi, a1);
    m3_tvec(a1, k.dXi, m);
    for (int i = 0; i < 3; ++i) s2[i] = a2[i] + a1[i];
    for (int I = 0; I < 3; ++I)
      for (int i = 0; i < 3; ++i) {
        fl[6 * I + i] += wJ * dN[I] * s0[i];
        fl[6 * I + 3 + i] += wJ * (dN[I] * s1[i] + N[I] * s2[i]);
      }
    double e = 0.0;
    for (int i = 0; i < 6; ++i) e += sig[i] * eps[i];
    se += 0.5 * wJ * e;
  }
  /* global frame: K <- T^T K T, f <- T^T f (T = blockdiag(T3), reference
   * src/Beam_1.cpp:833-834) */
  const double* T = c->T3;
  for (int bi = 0; bi < 6; ++bi)
    for (int bj = 0; bj < 6; ++bj) {
      double blk[9], t2[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) blk[i * 3 + j] = Kl[(3 * bi + i) + 18 * (3 * bj + j)];
      m3_mul(t2, blk, T);
      m3_tmul(blk, T, t2);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) K[(3 * bi + i) + 18 * (3 * bj + j)] = blk[i * 3 + j];
    }
  for (int bi = 0; bi < 6; ++bi) m3_tvec(f + 3 * bi, T, fl + 3 * bi);
  if (strain_energy) *strain_energy = se;
}

/* reference src/Beam_1.cpp:1494-1506 */
void oracle_beam_commit(const ob_const* c, ob_hist* h, const double* d) {
  for (int g = 0; g < 2; ++g) {
    gp_kin k;
    beam_gp_kinematics(c, h, d, g, &k);
    double Q[9];
    m3_mul(Q, k.Qd, h->Q[g]);
    m3_copy(h->Q[g], Q);
    for (int i = 0; i < 3; ++i) {
      h->u[g][i] += k.u[i];
      h->kap[g][i] = k.kappa[i];
      h->dz[g][i] = k.dz[i];
    }
    double an[3];
    rodrigues_compose(an, k.alpha, h->alpha[g]);
    memcpy(h->alpha[g], an, sizeof(an));
  }
}

/* Beam_1::MountMass (reference src/Beam_1.cpp:1564-1638) for Hooke sections
 * (no offset of the mass centre).  At each Gauss point, in the element frame:
 *   translation  dT_u = Mr (a1 du - a2 v_i - a3 acc_i)
 *   rotation     omega = Q_d w1, omega_dot = Q_d w2 with w1 = a4 da + c1,
 *                w2 = a1 da + c2, c1 = a5 w_i + a6 dw_i, c2 = -a2 w_i - a3 dw_i
 *                (Newmark in the tangent space, transported by Q_d as in
 *                reference src/Dynamic.cpp:513-551); spatial inertia
 *                J = Q J_r Q^T, Q = Q_d Q(alpha_i);
 *                m = J omega_dot + omega x J omega;  dT_a = Xi(da)^T m.
 * Since Xi^T Q_d = Xi for Rodrigues parameters, dT_a = Xi(da) h with
 * h = J_i w2 + w1 x J_i w1, J_i = Q(alpha_i) J_r Q(alpha_i)^T.  The tangent is
 * its exact derivative:
 *   d dT_u / d du = a1 Mr I
 *   d dT_a / d da = Xi (a1 J_i + a4 (skew(w1) J_i - skew(J_i w1)))
 *                   - g^2/2 (h + da x h / 2) da^T - g/2 skew(h).
 * The element sums wJ N^T dT and wJ N^T DdT N and turns them to the global
 * frame. */
void oracle_gp_inertia(double Mr, const double* Jr, const double* alpha_i, const double* du, const double* da,
                       const double* vi, const double* ai, const double* wi, const double* dwi, const double* a,
                       double* dT, double* DdT, double* ke) {
  const double a1 = a[0], a2 = a[1], a3 = a[2], a4 = a[3], a5 = a[4], a6 = a[5];
  memset(DdT, 0, 36 * sizeof(double));
  for (int i = 0; i < 3; ++i) {
    dT[i] = Mr * (a1 * du[i] - a2 * vi[i] - a3 * ai[i]);
    DdT[i * 6 + i] = a1 * Mr;
  }
  double Qi[9], Ji[9], t[9];
  rodrigues_Q(Qi, alpha_i);
  m3_mul(t, Qi, Jr);
  m3_mult(Ji, t, Qi);
  double w1[3], w2[3], Jw1[3], Jw2[3], cr[3], hv[3];
  for (int i = 0; i < 3; ++i) {
    w1[i] = a4 * da[i] + a5 * wi[i] + a6 * dwi[i];
    w2[i] = a1 * da[i] - a2 * wi[i] - a3 * dwi[i];
  }
  m3_vec(Jw1, Ji, w1);
  m3_vec(Jw2, Ji, w2);
  v3_cross(cr, w1, Jw1);
  for (int i = 0; i < 3; ++i) hv[i] = Jw2[i] + cr[i];
  double n2 = v3_dot(da, da);
  double gg = 4.0 / (4.0 + n2);
  double A[9], Xi[9];
  m3_skew(A, da);
  for (int q = 0; q < 9; ++q) Xi[q] = gg * 0.5 * A[q];
  Xi[0] += gg; Xi[4] += gg; Xi[8] += gg;
  double m[3];
  m3_vec(m, Xi, hv);
  for (int i = 0; i < 3; ++i) dT[3 + i] = m[i];
  /* dh/dda = a1 J_i + a4 (skew(w1) J_i - skew(J_i w1)) */
  double Sw1[9], SJw1[9], Dh[9];
  m3_skew(Sw1, w1);
  m3_skew(SJw1, Jw1);
  m3_mul(t, Sw1, Ji);
  for (int q = 0; q < 9; ++q) Dh[q] = a1 * Ji[q] + a4 * (t[q] - SJw1[q]);
  double XDh[9], axh[3], hh[3], Sh[9];
  m3_mul(XDh, Xi, Dh);
  v3_cross(axh, da, hv);
  for (int i = 0; i < 3; ++i) hh[i] = hv[i] + 0.5 * axh[i];
  m3_skew(Sh, hv);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      DdT[(3 + i) * 6 + 3 + j] = XDh[i * 3 + j] - 0.5 * gg * gg * hh[i] * da[j] - 0.5 * gg * Sh[i * 3 + j];
  /* kinetic energy at the end of the step */
  double v1[3], om[3], Qd[9], Jom[3], Q[9], J[9];
  for (int i = 0; i < 3; ++i) v1[i] = a4 * du[i] + a5 * vi[i] + a6 * ai[i];
  rodrigues_Q(Qd, da);
  m3_vec(om, Qd, w1);
  m3_mul(Q, Qd, Qi);
  m3_mul(t, Q, Jr);
  m3_mult(J, t, Q);
  m3_vec(Jom, J, om);
  *ke = 0.5 * Mr * v3_dot(v1, v1) + 0.5 * v3_dot(om, Jom);
}

void oracle_beam_inertia(const ob_const* c, const ob_hist* h, const double* d, const double* vel,
                         const double* acc, const double* a, double* K, double* f, double* kinetic) {
  double Kl[18 * 18], fl[18];
  memset(Kl, 0, sizeof(Kl));
  memset(fl, 0, sizeof(fl));
  double ke = 0.0;
  for (int g = 0; g < 2; ++g) {
    const double* N = c->N[g];
    double da[3] = {0, 0, 0}, du[3] = {0, 0, 0}, wi[3] = {0, 0, 0}, dwi[3] = {0, 0, 0}, vi[3] = {0, 0, 0},
           ai[3] = {0, 0, 0};
    for (int i = 0; i < 3; ++i)
      for (int n = 0; n < 3; ++n) {
        da[i] += d[6 * n + 3 + i] * N[n];
        du[i] += d[6 * n + i] * N[n];
        wi[i] += vel[6 * n + 3 + i] * N[n];
        dwi[i] += acc[6 * n + 3 + i] * N[n];
        vi[i] += vel[6 * n + i] * N[n];
        ai[i] += acc[6 * n + i] * N[n];
      }
    m3_vec(da, c->T3, da);
    m3_vec(du, c->T3, du);
    m3_vec(wi, c->T3, wi);
    m3_vec(dwi, c->T3, dwi);
    m3_vec(vi, c->T3, vi);
    m3_vec(ai, c->T3, ai);
    double dT[6], DdT[36], kg;
    oracle_gp_inertia(c->Mr, c->Jr, h->alpha[g], du, da, vi, ai, wi, dwi, a, dT, DdT, &kg);
    double wJ = 1.0 * c->jac;
    for (int I = 0; I < 3; ++I) {
      for (int i = 0; i < 6; ++i) fl[6 * I + i] += wJ * N[I] * dT[i];
      for (int J = 0; J < 3; ++J)
        for (int i = 0; i < 6; ++i)
          for (int j = 0; j < 6; ++j) Kl[(6 * I + i) + 18 * (6 * J + j)] += wJ * N[I] * N[J] * DdT[i * 6 + j];
    }
    ke += wJ * kg;
  }
  const double* T = c->T3;
  for (int bi = 0; bi < 6; ++bi)
    for (int bj = 0; bj < 6; ++bj) {
      double blk[9], t2[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) blk[i * 3 + j] = Kl[(3 * bi + i) + 18 * (3 * bj + j)];
      m3_mul(t2, blk, T);
      m3_tmul(blk, T, t2);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) K[(3 * bi + i) + 18 * (3 * bj + j)] += blk[i * 3 + j];
    }
  for (int bi = 0; bi < 6; ++bi) {
    double t3[3];
    m3_tvec(t3, T, fl + 3 * bi);
    for (int i = 0; i < 3; ++i) f[3 * bi + i] += t3[i];
  }
  if (kinetic) *kinetic = ke;
}

/* Beam_1::MountMassModal (reference src/Beam_1.cpp:1538-1553) for sections
 * without a first moment of mass (br = 0: Hooke rectangles and tubes): at
 * each Gauss point EvaluateMassModal (src/Beam_1.cpp:1681-1774) gives the
 * 6x6 operator blockdiag(Q Mr Q^T, Q Jr Q^T), Q = Q(alpha_i) the Rodrigues
 * rotation of the Gauss point's committed rotation vector and Mr = rho A I;
 * the element sums wJ N^T D N (w = 1) and turns the 18x18 to the global
 * frame as transform^T M transform.  M: 18x18 column-major. */
void oracle_beam_modal_mass(const ob_const* c, const ob_hist* h, double* M) {
  double Ml[18 * 18];
  memset(Ml, 0, sizeof(Ml));
  for (int g = 0; g < 2; ++g) {
    double Q[9], t[9], Mt[9], Jt[9], Mr[9] = {c->Mr, 0, 0, 0, c->Mr, 0, 0, 0, c->Mr};
    rodrigues_Q(Q, h->alpha[g]);
    m3_mul(t, Q, Mr);
    m3_mult(Mt, t, Q);
    m3_mul(t, Q, c->Jr);
    m3_mult(Jt, t, Q);
    double D[36];
    memset(D, 0, sizeof(D));
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        D[i * 6 + j] = Mt[i * 3 + j];
        D[(3 + i) * 6 + 3 + j] = Jt[i * 3 + j];
      }
    const double* N = c->N[g];
    for (int I = 0; I < 3; ++I)
      for (int J = 0; J < 3; ++J)
        for (int i = 0; i < 6; ++i)
          for (int j = 0; j < 6; ++j) Ml[(6 * I + i) + 18 * (6 * J + j)] += ((c->jac * N[I]) * D[i * 6 + j]) * N[J];
  }
  const double* T = c->T3;
  for (int bi = 0; bi < 6; ++bi)
    for (int bj = 0; bj < 6; ++bj) {
      double blk[9], t2[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) blk[i * 3 + j] = Ml[(3 * bi + i) + 18 * (3 * bj + j)];
      m3_mul(t2, blk, T);
      m3_tmul(blk, T, t2);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) M[(3 * bi + i) + 18 * (3 * bj + j)] = blk[i * 3 + j];
    }
}

/* Pipe_1::PreCalc (reference src/Pipe_1.cpp:1106-1156): Beam_1's geometry
 * and shape functions with the PipeSection's constitutive matrix
 * diag(GA, GA, EA, EI, EI, GJ), mass Rho per unit length and rotary
 * inertia Rho ((De/2)^2 - (Di/2)^2) diag(1/4, 1/4, 1/2).  ps: EA, EI, GJ,
 * GA, Rho, CDt, CDn, CAt, CAn, De, Di. */
void oracle_pipe_precalc(const double* x0, const double* x2, const double* ps, const double* cs, ob_const* c,
                         ob_hist* h) {
  /* the geometry as Beam_1 without pre-tension; then the pipe's constants */
  const double unit_mat[3] = {1.0, 0.0, 0.0}, unit_sec[6] = {1.0, 1.0, 1.0, 0.0, 1.0, 1.0};
  oracle_beam_precalc(x0, x2, unit_mat, unit_sec, cs, 0.0, c, h);
  const double EA = ps[0], EI = ps[1], GJ = ps[2], GA = ps[3], Rho = ps[4], De = ps[9], Di = ps[10];
  memset(c->D, 0, sizeof(c->D));
  c->D[0 * 6 + 0] = GA;
  c->D[1 * 6 + 1] = GA;
  c->D[2 * 6 + 2] = EA;
  c->D[3 * 6 + 3] = EI;
  c->D[4 * 6 + 4] = EI;
  c->D[5 * 6 + 5] = GJ;
  c->Mr = Rho;
  m3_zero(c->Jr);
  const double rr = (De / 2.0) * (De / 2.0) - (Di / 2.0) * (Di / 2.0);
  c->Jr[0] = (Rho * rr / 4.0);
  c->Jr[4] = (Rho * rr / 4.0);
  c->Jr[8] = (Rho * rr / 2.0);
}

/* MountPipeSpecialLoads (reference src/Pipe_1.cpp:1441-1494): the internal
 * pressure p0i on the internal area Aint of a Pipe_1 element at the current
 * iterate.  At each Gauss point, with Q = Q_delta Q_i, k = Q kappa_r and
 * e3 = Q e3r (local frame): the load f = -p0i Aint (k x e3), the moment
 * m = -p0i Aint Xi^T (z' x e3), and the load stiffness Kext (6 x 12, on
 * (u, alpha, u', alpha')).  P -= jac T^T N^T (f, m); K -= jac p0i Aint
 * T^T N^T Kext Upsilon T.  K is 18x18 column-major, global frame. */
void oracle_pipe_pressure(const ob_const* c, const ob_hist* h, const double* d, double p0i, double Aint, double* K,
                          double* f) {
  const double mult = 1.0 * c->jac;
  /* The reference's O1 term reads the element's scalar member g, which
   * Pipe_1::Mount leaves at the value of its last Gauss point
   * (src/Pipe_1.cpp:890): both Gauss points use g of the second. */
  gp_kin k1;
  beam_gp_kinematics(c, h, d, 1, &k1);
  const double g_last = k1.g;
  for (int g = 0; g < 2; ++g) {
    gp_kin k;
    beam_gp_kinematics(c, h, d, g, &k);
    double Q[9];
    m3_transpose(Q, k.Qt);
    double kip[3], e3ip[3];
    m3_vec(kip, Q, k.kappa);
    m3_vec(e3ip, Q, c->e3r);
    const double pa = -p0i * Aint;
    double cr[3], t1[3], tl[6];
    v3_cross(cr, kip, e3ip);
    for (int i = 0; i < 3; ++i) tl[i] = pa * cr[i];
    v3_cross(cr, k.dz, e3ip);
    m3_tvec(t1, k.Xi, cr);
    for (int i = 0; i < 3; ++i) tl[3 + i] = pa * t1[i];
    double E3[9], Kp[9];
    m3_skew(E3, e3ip);
    m3_skew(Kp, kip);
    /* O1 = -0.5 g (Xi^T (e3 x z') alpha^T - skew(e3 x z')), g of the last
   * Gauss point */
    double c2[3], w[3], S2[9], O1[9];
    v3_cross(c2, e3ip, k.dz);
    m3_tvec(w, k.Xi, c2);
    m3_skew(S2, c2);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) O1[i * 3 + j] = -0.5 * g_last * (w[i] * k.alpha[j] - S2[i * 3 + j]);
    /* K1ua = Kp E3 Xi + E3 dXi - E3 Kp Xi; K1aa = O1 + Xi^T dZ E3 Xi;
     * K2ua = E3 Xi; K2au = Xi^T E3 */
    double a1[9], a2[9], K1ua[9], K1aa[9], K2ua[9], K2au[9];
    m3_mul(a1, Kp, E3);
    m3_mul(K1ua, a1, k.Xi);
    m3_mul(a2, E3, k.dXi);
    for (int q = 0; q < 9; ++q) K1ua[q] += a2[q];
    m3_mul(a1, E3, Kp);
    m3_mul(a2, a1, k.Xi);
    for (int q = 0; q < 9; ++q) K1ua[q] -= a2[q];
    m3_mul(a1, k.dZ, E3);
    m3_mul(a2, a1, k.Xi);
    m3_tmul(K1aa, k.Xi, a2);
    for (int q = 0; q < 9; ++q) K1aa[q] += O1[q];
    m3_mul(K2ua, E3, k.Xi);
    m3_tmul(K2au, k.Xi, E3);
    /* Kext (6 x 12, row-major): (0:3, 3:6) K1ua, (3:6, 3:6) K1aa,
     * (0:3, 9:12) K2ua, (3:6, 6:9) K2au */
    double Kx[6][12];
    memset(Kx, 0, sizeof(Kx));
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        Kx[i][3 + j] = K1ua[i * 3 + j];
        Kx[3 + i][3 + j] = K1aa[i * 3 + j];
        Kx[i][9 + j] = K2ua[i * 3 + j];
        Kx[3 + i][6 + j] = K2au[i * 3 + j];
      }
    /* force: P -= mult T^T N^T tl */
    for (int a = 0; a < 3; ++a) {
      const double Na = c->N[g][a];
      for (int blk = 0; blk < 2; ++blk) {
        double v[3], r[3];
        for (int i = 0; i < 3; ++i) v[i] = Na * tl[3 * blk + i];
        m3_tvec(r, c->T3, v);
        for (int i = 0; i < 3; ++i) f[6 * a + 3 * blk + i] -= mult * r[i];
      }
    }
    /* stiffness: K -= s T^T (N^T Kext Upsilon) T, node blocks (a, b):
     * N_a (N_b Kext[:, 0:6] + dN_b Kext[:, 6:12]) */
    const double s = mult * p0i * Aint;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        const double Na = c->N[g][a], Nb = c->N[g][b], dNb = c->dN[g][b];
        for (int p = 0; p < 2; ++p)
          for (int q = 0; q < 2; ++q) {
            double X[9], Y[9], Z[9];
            for (int i = 0; i < 3; ++i)
              for (int j = 0; j < 3; ++j)
                X[i * 3 + j] = Na * (Nb * Kx[3 * p + i][3 * q + j] + dNb * Kx[3 * p + i][6 + 3 * q + j]);
            m3_tmul(Y, c->T3, X); /* T3^T X */
            m3_mul(Z, Y, c->T3);  /* T3^T X T3 */
            for (int i = 0; i < 3; ++i)
              for (int j = 0; j < 3; ++j) {
                const int r = 6 * a + 3 * p + i, col = 6 * b + 3 * q + j;
                K[r + 18 * col] -= s * Z[i * 3 + j];
              }
          }
      }
  }
}
