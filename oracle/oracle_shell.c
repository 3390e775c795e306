/*
 * Shell_1 element, CPU restatement.  TEST INFRASTRUCTURE (oracle): the
 * reference values the CUDA Shell_1 path is tested against.
 *
 * Follows reference src/Shell_1.cpp:
 *   1666-2365  PreCalc (local frame, Lame constants, drilling stiffness,
 *              shape functions at the three midside Gauss points, the
 *              six-point surface rule of Cowper (1973))
 *   899-1332   Mount (incremental Rodrigues kinematics, thickness
 *              integration of the compressible neo-Hookean law, 12x12
 *              generalized constitutive matrix, Psi operator, geometric
 *              part G, K = T^T (sum dN^T (Psi^T D Psi + G) dN) T)
 *   1392-1467  MountShellSpecialLoads (follower pressure and its tangent)
 *   1650-1664  SaveLagrange
 *   1470-1510  TransformMatrix
 *   2406-2498  MountMass (through the Gauss-point inertia shared with
 *              Beam_1: a director fibre of mass coef1 per unit area and
 *              rotary inertia coef2 (I - e3r e3r^T), whose inertial moment
 *              coef2 d x (d'') equals J w' + w x J w with J = Q Jr Q^T)
 *   2368-2396  MountMassModal and EvaluateMassModal (3171-)
 */
#include "oracle_shell.h"
#include "giraffe_oracle.h"
#include "oracle_beam.h"

#include <string.h>

/* corner / midside translation shape functions and their x1, x2
 * derivatives from area coordinates L and their derivatives Lx1, Lx2
 * (reference src/Shell_1.cpp:2063-2089) */
static void shape_u(const double* L, const double* L1, const double* L2, double* N, double* N1, double* N2) {
  N[0] = (2 * L[0] - 1) * L[0];
  N[1] = (2 * L[1] - 1) * L[1];
  N[2] = (2 * L[2] - 1) * L[2];
  N[3] = 4 * L[0] * L[1];
  N[4] = 4 * L[1] * L[2];
  N[5] = 4 * L[2] * L[0];
  const double* D[2] = {L1, L2};
  double* O[2] = {N1, N2};
  for (int q = 0; q < 2; ++q) {
    const double* Ld = D[q];
    double* o = O[q];
    o[0] = 4 * Ld[0] * L[0] - Ld[0];
    o[1] = 4 * Ld[1] * L[1] - Ld[1];
    o[2] = 4 * Ld[2] * L[2] - Ld[2];
    o[3] = 4 * Ld[0] * L[1] + 4 * L[0] * Ld[1];
    o[4] = 4 * Ld[1] * L[2] + 4 * L[1] * Ld[2];
    o[5] = 4 * Ld[2] * L[0] + 4 * L[2] * Ld[0];
  }
}

static double tri_area(const double* a, const double* b, const double* c) {
  double u[3], v[3], w[3];
  for (int k = 0; k < 3; ++k) { u[k] = b[k] - a[k]; v[k] = c[k] - a[k]; }
  v3_cross(w, u, v);
  return 0.5 * v3_norm(w);
}

void oracle_shell_precalc(const double* xyz, const double* mat, double thickness, os_const* c, os_hist* h) {
  memset(c, 0, sizeof(*c));
  memset(h, 0, sizeof(*h));
  const double *x1 = xyz, *x2 = xyz + 3, *x3 = xyz + 6;
  double a[3], b[3], n[3];
  for (int k = 0; k < 3; ++k) { a[k] = x2[k] - x1[k]; b[k] = x3[k] - x1[k]; }
  v3_cross(n, a, b);
  double nn = v3_norm(n);
  double A = 0.5 * nn;
  c->area = A;
  /* frame: e3r normal, e1r the projection of global x (y when x is nearly
   * normal), e2r = e3r x e1r */
  double e1[3], e2[3], e3[3];
  for (int k = 0; k < 3; ++k) e3[k] = (1.0 / nn) * n[k];
  double eg[3] = {1.0, 0.0, 0.0};
  if (fabs(v3_dot(eg, e3)) >= 1.0 - 1e-4) { eg[0] = 0.0; eg[1] = 1.0; }
  double dd = v3_dot(eg, e3);
  for (int k = 0; k < 3; ++k) e1[k] = eg[k] - dd * e3[k];
  double n1 = v3_norm(e1);
  for (int k = 0; k < 3; ++k) e1[k] = (1.0 / n1) * e1[k];
  v3_cross(e2, e3, e1);
  for (int k = 0; k < 3; ++k) {
    c->er[k] = e1[k]; c->er[3 + k] = e2[k]; c->er[6 + k] = e3[k];
    c->T3[k] = e1[k]; c->T3[3 + k] = e2[k]; c->T3[6 + k] = e3[k];
  }
  double E = mat[0], nu = mat[1];
  c->mu = E / (2.0 * (1 + nu));
  c->lambda = 2.0 * c->mu * nu / (1 - 2.0 * nu);
  c->stiff_drill = E * thickness * thickness * thickness;
  c->thick = thickness;
  c->coef1 = thickness * mat[2];
  c->coef2 = (1.0 / 12.0) * thickness * thickness * thickness * mat[2];
  c->coef3 = mat[2] * thickness * A / (3 * 3.1415926535897932384626433832795);
  /* area-coordinate derivatives in the local frame */
  double d23[3], d31[3], d12[3], d32[3], d13[3], d21[3];
  for (int k = 0; k < 3; ++k) {
    d23[k] = x2[k] - x3[k]; d31[k] = x3[k] - x1[k]; d12[k] = x1[k] - x2[k];
    d32[k] = x3[k] - x2[k]; d13[k] = x1[k] - x3[k]; d21[k] = x2[k] - x1[k];
  }
  double Lx1[3] = {0.5 * v3_dot(d23, e2) / A, 0.5 * v3_dot(d31, e2) / A, 0.5 * v3_dot(d12, e2) / A};
  double Lx2[3] = {0.5 * v3_dot(d32, e1) / A, 0.5 * v3_dot(d13, e1) / A, 0.5 * v3_dot(d21, e1) / A};
  for (int g = 0; g < 3; ++g) {
    const double* xp = xyz + 3 * (3 + g);
    double L[3] = {tri_area(xp, x2, x3) / A, tri_area(xp, x3, x1) / A, tri_area(xp, x1, x2) / A};
    shape_u(L, Lx1, Lx2, c->Nu[g], c->Nu1[g], c->Nu2[g]);
    c->Na[g][0] = 1 - 2 * L[2];
    c->Na[g][1] = 1 - 2 * L[0];
    c->Na[g][2] = 1 - 2 * L[1];
    c->Na1[g][0] = -2 * Lx1[2]; c->Na1[g][1] = -2 * Lx1[0]; c->Na1[g][2] = -2 * Lx1[1];
    c->Na2[g][0] = -2 * Lx2[2]; c->Na2[g][1] = -2 * Lx2[0]; c->Na2[g][2] = -2 * Lx2[1];
  }
  /* six-point rule (Cowper 1973): area coordinates and weights */
  static const double pa = 0.816847572980459, pb = 0.091576213509771, pc = 0.108103018168070,
                      pd = 0.445948490915965, wa = 0.109951743655322, wb = 0.223381589678011;
  const double Lc[6][3] = {{pa, pb, pb}, {pb, pa, pb}, {pb, pb, pa}, {pc, pd, pd}, {pd, pc, pd}, {pd, pd, pc}};
  for (int k = 0; k < 6; ++k) {
    c->w4[k] = A * (k < 3 ? wa : wb);
    shape_u(Lc[k], Lx1, Lx2, c->N4[k], c->N41[k], c->N42[k]);
    c->Na4[k][0] = 1 - 2 * Lc[k][2];
    c->Na4[k][1] = 1 - 2 * Lc[k][0];
    c->Na4[k][2] = 1 - 2 * Lc[k][1];
  }
  c->alpha1 = A / 3.0;
  for (int g = 0; g < 3; ++g) {
    m3_eye(h->Q[g]);
    h->z1[g][0] = 1.0;
    h->z2[g][1] = 1.0;
  }
}

/* Gauss-point kinematics of the current increment (local frame). */
typedef struct {
  double u[3], u1[3], u2[3], al[3], al1[3], al2[3];
  double an, g;
  double Qd[9], Xi[9], Xi1[9], Xi2[9];
  double z1[3], z2[3];
  double Q[9];  /* Q_delta Q_i */
  double eta1[3], eta2[3], k1[3], k2[3];
} sgp;

static void shell_gp(const os_const* c, const os_hist* h, const double* d, int g, sgp* k) {
  double ug[3] = {0, 0, 0}, u1g[3] = {0, 0, 0}, u2g[3] = {0, 0, 0};
  double ag[3] = {0, 0, 0}, a1g[3] = {0, 0, 0}, a2g[3] = {0, 0, 0};
  for (int j = 0; j < 3; ++j) {
    for (int n = 0; n < 6; ++n) {
      ug[j] += d[3 * n + j] * c->Nu[g][n];
      u1g[j] += d[3 * n + j] * c->Nu1[g][n];
      u2g[j] += d[3 * n + j] * c->Nu2[g][n];
    }
    for (int m = 0; m < 3; ++m) {
      ag[j] += d[18 + 3 * m + j] * c->Na[g][m];
      a1g[j] += d[18 + 3 * m + j] * c->Na1[g][m];
      a2g[j] += d[18 + 3 * m + j] * c->Na2[g][m];
    }
  }
  m3_vec(k->u, c->T3, ug);
  m3_vec(k->u1, c->T3, u1g);
  m3_vec(k->u2, c->T3, u2g);
  m3_vec(k->al, c->T3, ag);
  m3_vec(k->al1, c->T3, a1g);
  m3_vec(k->al2, c->T3, a2g);
  k->an = v3_norm(k->al);
  double A[9], A2[9];
  m3_skew(A, k->al);
  m3_mul(A2, A, A);
  k->g = 4.0 / (4.0 + k->an * k->an);
  for (int q = 0; q < 9; ++q) {
    k->Qd[q] = k->g * (A[q] + 0.5 * A2[q]);
    k->Xi[q] = k->g * 0.5 * A[q];
  }
  k->Qd[0] += 1.0; k->Qd[4] += 1.0; k->Qd[8] += 1.0;
  k->Xi[0] += k->g; k->Xi[4] += k->g; k->Xi[8] += k->g;
  /* Xi_x = -g/2 ((alpha . alpha_x) Xi - skew(alpha_x)) */
  double S1[9], S2[9];
  m3_skew(S1, k->al1);
  m3_skew(S2, k->al2);
  double p1 = v3_dot(k->al, k->al1), p2 = v3_dot(k->al, k->al2);
  for (int q = 0; q < 9; ++q) {
    k->Xi1[q] = -0.5 * k->g * (p1 * k->Xi[q] - S1[q]);
    k->Xi2[q] = -0.5 * k->g * (p2 * k->Xi[q] - S2[q]);
  }
  for (int j = 0; j < 3; ++j) {
    k->z1[j] = k->u1[j] + h->z1[g][j];
    k->z2[j] = k->u2[j] + h->z2[g][j];
  }
  m3_mul(k->Q, k->Qd, h->Q[g]);
  m3_tvec(k->eta1, k->Q, k->z1);
  m3_tvec(k->eta2, k->Q, k->z2);
  k->eta1[0] -= 1.0;
  k->eta2[1] -= 1.0;
  /* kappa_r = Q_i^T Xi^T alpha_x + kappa_r_i, with Q_i^T Xi^T = (Xi Q_i)^T */
  double XQ[9];
  m3_mul(XQ, k->Xi, h->Q[g]);
  m3_tvec(k->k1, XQ, k->al1);
  m3_tvec(k->k2, XQ, k->al2);
  for (int j = 0; j < 3; ++j) {
    k->k1[j] += h->k1[g][j];
    k->k2[j] += h->k2[g][j];
  }
}

/* small dense helpers (row-major) */
static void mm(double* C, const double* A, const double* B, int n, int k, int m) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < m; ++j) {
      double s = 0.0;
      for (int q = 0; q < k; ++q) s += A[i * k + q] * B[q * m + j];
      C[i * m + j] = s;
    }
}

static void put3(double* M, int ld, int r0, int c0, const double* B) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M[(r0 + i) * ld + c0 + j] = B[i * 3 + j];
}

void oracle_shell_mount(const os_const* c, const os_hist* h, const double* d, double* K, double* f,
                        double* strain_energy) {
  double Kl[27 * 27], fl[27];
  memset(Kl, 0, sizeof(Kl));
  memset(fl, 0, sizeof(fl));
  double energy = 0.0;
  const double mu = c->mu, la = c->lambda;
  static const double E3r[9] = {0, -1, 0, 1, 0, 0, 0, 0, 0}; /* skew(e3) */
  for (int g = 0; g < 3; ++g) {
    sgp k;
    shell_gp(c, h, d, g, &k);
    /* thickness integration (3-point Gauss) */
    double dn1e1[9] = {0}, dn1e2[9] = {0}, dn1k1[9] = {0}, dn1k2[9] = {0};
    double dn2e1[9] = {0}, dn2e2[9] = {0}, dn2k1[9] = {0}, dn2k2[9] = {0};
    double dm1e1[9] = {0}, dm1e2[9] = {0}, dm1k1[9] = {0}, dm1k2[9] = {0};
    double dm2e1[9] = {0}, dm2e2[9] = {0}, dm2k1[9] = {0}, dm2k2[9] = {0};
    double nr1[3] = {0, 0, 0}, nr2[3] = {0, 0, 0}, mr1[3] = {0, 0, 0}, mr2[3] = {0, 0, 0};
    double psi_t = 0.0;
    const double jac = c->thick / 2.0;
    static const double csi[3] = {-0.77459666924148337703585307995648, 0.0, 0.77459666924148337703585307995648};
    static const double wt[3] = {0.55555555555555555555555555555556, 0.88888888888888888888888888888889,
                                 0.55555555555555555555555555555556};
    for (int q = 0; q < 3; ++q) {
      double zeta = c->thick * csi[q] / 2.0;
      double w = wt[q] * jac;
      /* gamma_r = eta_r + zeta kappa_r x e3 ; (kappa x e3) = (k_y, -k_x, 0) */
      double g1[3] = {k.eta1[0] + zeta * k.k1[1], k.eta1[1] - zeta * k.k1[0], k.eta1[2]};
      double g2[3] = {k.eta2[0] + zeta * k.k2[1], k.eta2[1] - zeta * k.k2[0], k.eta2[2]};
      double g11 = g1[0], g12 = g1[1], g13 = g1[2], g21 = g2[0], g22 = g2[1], g23 = g2[2];
      double jb = (1.0 + g11) * (1.0 + g22) - g12 * g21;
      double v = (la * (jb * jb * jb - 1.0) + 2.0 * mu * (jb - 1.0)) / (la * jb * jb * jb + 2.0 * mu * jb);
      double den = la * jb * jb + 2.0 * mu;
      double dv = ((la + 2.0 * mu) * (3.0 * la * jb * jb + 2.0 * mu)) / (jb * jb * den * den);
      double t1[3] = {mu * v * (1.0 + g22) + mu * (g11 - g22), mu * v * (-g21) + mu * (g12 + g21), mu * g13};
      double t2[3] = {mu * v * (-g12) + mu * (g12 + g21), mu * v * (1.0 + g11) + mu * (g22 - g11), mu * g23};
      double C11[9] = {mu * ((1.0 + g22) * (1.0 + g22) * dv + 1.0), -mu * (1.0 + g22) * g21 * dv, 0,
                       -mu * (1.0 + g22) * g21 * dv, mu * (g21 * g21 * dv + 1.0), 0, 0, 0, mu};
      double C22[9] = {mu * (g12 * g12 * dv + 1.0), -mu * ((1.0 + g11) * g12 * dv), 0,
                       -mu * ((1.0 + g11) * g12 * dv), mu * ((1.0 + g11) * (1.0 + g11) * dv + 1.0), 0, 0, 0, mu};
      double C12[9] = {-mu * ((1.0 + g22) * g12 * dv), mu * (v - 1.0 + (1.0 + g11) * (1.0 + g22) * dv), 0,
                       mu * (1.0 - v + g12 * g21 * dv), -mu * ((1.0 + g11) * g21 * dv), 0, 0, 0, 0};
      double C21[9];
      m3_transpose(C21, C12);
      double T[9], U[9];
      const double* Cs[4] = {C11, C12, C21, C22};
      double* dn_e[4] = {dn1e1, dn1e2, dn2e1, dn2e2};
      double* dn_k[4] = {dn1k1, dn1k2, dn2k1, dn2k2};
      double* dm_e[4] = {dm1e1, dm1e2, dm2e1, dm2e2};
      double* dm_k[4] = {dm1k1, dm1k2, dm2k1, dm2k2};
      for (int s = 0; s < 4; ++s) {
        const double* Cm = Cs[s];
        m3_mul(T, Cm, E3r);  /* C E3r */
        m3_mul(U, E3r, Cm);  /* E3r C */
        double V[9];
        m3_mul(V, U, E3r);   /* E3r C E3r */
        for (int e = 0; e < 9; ++e) {
          dn_e[s][e] += w * Cm[e];
          dn_k[s][e] -= w * zeta * T[e];
          dm_e[s][e] += w * zeta * U[e];
          dm_k[s][e] -= w * zeta * zeta * V[e];
        }
      }
      /* e3 x tau = (-tau_y, tau_x, 0) */
      for (int j = 0; j < 3; ++j) { nr1[j] += w * t1[j]; nr2[j] += w * t2[j]; }
      double c1[3] = {-t1[1], t1[0], 0.0}, c2[3] = {-t2[1], t2[0], 0.0};
      for (int j = 0; j < 3; ++j) { mr1[j] += w * zeta * c1[j]; mr2[j] += w * zeta * c2[j]; }
      double g33 = sqrt((la + 2.0 * mu) / (la * jb * jb + 2.0 * mu)) - 1.0;
      double JF = jb * (1 + g33);
      double I1 = (1.0 + g11) * (1.0 + g11) + g12 * g12 + g13 * g13 + g21 * g21 + (1.0 + g22) * (1.0 + g22) +
                  g23 * g23 + (1.0 + g33) * (1.0 + g33);
      double psi = 0.5 * la * (0.5 * (JF * JF - 1.0) - log(JF)) + 0.5 * mu * (I1 - 3.0 - 2.0 * log(JF));
      psi_t += w * psi;
    }
    /* generalized constitutive matrix: rows (n1, m1, n2, m2), columns
     * (eta1, kappa1, eta2, kappa2); drilling stiffness on the in-plane
     * curvature about e3 */
    double D[144];
    memset(D, 0, sizeof(D));
    put3(D, 12, 0, 0, dn1e1); put3(D, 12, 0, 3, dn1k1); put3(D, 12, 0, 6, dn1e2); put3(D, 12, 0, 9, dn1k2);
    put3(D, 12, 3, 0, dm1e1); put3(D, 12, 3, 3, dm1k1); put3(D, 12, 3, 6, dm1e2); put3(D, 12, 3, 9, dm1k2);
    put3(D, 12, 6, 0, dn2e1); put3(D, 12, 6, 3, dn2k1); put3(D, 12, 6, 6, dn2e2); put3(D, 12, 6, 9, dn2k2);
    put3(D, 12, 9, 0, dm2e1); put3(D, 12, 9, 3, dm2k1); put3(D, 12, 9, 6, dm2e2); put3(D, 12, 9, 9, dm2k2);
    D[5 * 12 + 5] = c->stiff_drill;
    D[11 * 12 + 11] = c->stiff_drill;
    mr1[2] = c->stiff_drill * k.k1[2];
    mr2[2] = c->stiff_drill * k.k2[2];
    double sig[12];
    for (int j = 0; j < 3; ++j) { sig[j] = nr1[j]; sig[3 + j] = mr1[j]; sig[6 + j] = nr2[j]; sig[9 + j] = mr2[j]; }
    /* Psi (12 x 15) */
    double Psi[180];
    memset(Psi, 0, sizeof(Psi));
    double Qt[9], B[9], Cc[9], Z1[9], Z2[9];
    m3_transpose(Qt, k.Q);
    m3_skew(Z1, k.z1);
    m3_skew(Z2, k.z2);
    put3(Psi, 15, 0, 0, Qt);
    put3(Psi, 15, 6, 6, Qt);
    m3_mul(B, Qt, k.Xi);
    put3(Psi, 15, 3, 3, B);
    put3(Psi, 15, 9, 9, B);
    m3_mul(Cc, Qt, Z1); m3_mul(B, Cc, k.Xi); put3(Psi, 15, 0, 12, B);
    m3_mul(B, Qt, k.Xi1); put3(Psi, 15, 3, 12, B);
    m3_mul(Cc, Qt, Z2); m3_mul(B, Cc, k.Xi); put3(Psi, 15, 6, 12, B);
    m3_mul(B, Qt, k.Xi2); put3(Psi, 15, 9, 12, B);
    /* M = Psi^T D Psi (15 x 15) */
    double PT[180], PTD[180], M[225];
    for (int i = 0; i < 12; ++i)
      for (int j = 0; j < 15; ++j) PT[j * 12 + i] = Psi[i * 15 + j];
    mm(PTD, PT, D, 15, 12, 12);
    mm(M, PTD, Psi, 15, 12, 15);
    /* geometric part G (15 x 15) */
    double n1[3], n2[3], m1[3], m2[3];
    m3_vec(n1, k.Q, nr1);
    m3_vec(n2, k.Q, nr2);
    m3_vec(m1, k.Q, mr1);
    m3_vec(m2, k.Q, mr2);
    double Zn1[3], Zn2[3];
    m3_vec(Zn1, Z1, n1);
    m3_vec(Zn2, Z2, n2);
    double V1[9], V2[9], Vm1[9], Vm2[9], dV1[9], dV2[9];
    op_V(V1, k.al, Zn1, k.an);
    op_V(V2, k.al, Zn2, k.an);
    op_V(Vm1, k.al, m1, k.an);
    op_V(Vm2, k.al, m2, k.an);
    op_dV(dV1, k.al, k.al1, m1, k.an);
    op_dV(dV2, k.al, k.al2, m2, k.an);
    double Sn1[9], Sn2[9], Sm1[9], Sm2[9];
    m3_skew(Sn1, n1); m3_skew(Sn2, n2); m3_skew(Sm1, m1); m3_skew(Sm2, m2);
    double Gdua1[9], Gdua2[9], Gaa1[9], Gaa2[9];
    m3_mul(Gdua1, Sn1, k.Xi);
    m3_mul(Gdua2, Sn2, k.Xi);
    for (int e = 0; e < 9; ++e) { Gdua1[e] = -1.0 * Gdua1[e]; Gdua2[e] = -1.0 * Gdua2[e]; }
    /* G_aa = Xi^T (Z skew(n)) Xi - V(alpha, Z n) + dV(alpha, alpha_x, m) - Xi_x^T (skew(m) Xi) */
    const double* Zs[2] = {Z1, Z2};
    const double* Sns[2] = {Sn1, Sn2};
    const double* Sms[2] = {Sm1, Sm2};
    const double* Xix[2] = {k.Xi1, k.Xi2};
    const double* Vs[2] = {V1, V2};
    const double* dVs[2] = {dV1, dV2};
    double* Gaa[2] = {Gaa1, Gaa2};
    for (int s = 0; s < 2; ++s) {
      double P1[9], P2[9], P3[9], R1[9], R2[9];
      m3_mul(P1, Zs[s], Sns[s]);
      m3_mul(P2, P1, k.Xi);
      m3_tmul(P3, k.Xi, P2);  /* Xi^T (Z skew(n)) Xi */
      m3_mul(R1, Sms[s], k.Xi);
      m3_tmul(R2, Xix[s], R1);
      for (int e = 0; e < 9; ++e) Gaa[s][e] = P3[e] - Vs[s][e] + dVs[s][e] - R2[e];
    }
    double G[225];
    memset(G, 0, sizeof(G));
    double Tt[9];
    put3(G, 15, 0, 12, Gdua1);
    m3_transpose(Tt, Vm1); put3(G, 15, 3, 12, Tt);
    put3(G, 15, 6, 12, Gdua2);
    m3_transpose(Tt, Vm2); put3(G, 15, 9, 12, Tt);
    m3_transpose(Tt, Gdua1); put3(G, 15, 12, 0, Tt);
    put3(G, 15, 12, 3, Vm1);
    m3_transpose(Tt, Gdua2); put3(G, 15, 12, 6, Tt);
    put3(G, 15, 12, 9, Vm2);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) G[(12 + i) * 15 + 12 + j] = Gaa1[i * 3 + j] + Gaa2[i * 3 + j];
    for (int e = 0; e < 225; ++e) M[e] += G[e];
    /* generalized internal force Psi^T sigma */
    double qv[15];
    for (int j = 0; j < 15; ++j) {
      double s = 0.0;
      for (int i = 0; i < 12; ++i) s += Psi[i * 15 + j] * sig[i];
      qv[j] = s;
    }
    /* dN coefficients: row block r, node block a (6 translation blocks,
     * then the 3 midside rotation blocks) */
    double cf[5][9];
    memset(cf, 0, sizeof(cf));
    for (int a = 0; a < 6; ++a) { cf[0][a] = c->Nu1[g][a]; cf[2][a] = c->Nu2[g][a]; }
    for (int m = 0; m < 3; ++m) {
      cf[1][6 + m] = c->Na1[g][m];
      cf[3][6 + m] = c->Na2[g][m];
      cf[4][6 + m] = c->Na[g][m];
    }
    for (int a = 0; a < 9; ++a)
      for (int b = 0; b < 9; ++b)
        for (int r = 0; r < 5; ++r) {
          if (cf[r][a] == 0.0) continue;
          for (int s = 0; s < 5; ++s) {
            if (cf[s][b] == 0.0) continue;
            double wgt = c->alpha1 * cf[r][a] * cf[s][b];
            for (int i = 0; i < 3; ++i)
              for (int j = 0; j < 3; ++j) Kl[(3 * a + i) * 27 + 3 * b + j] += wgt * M[(3 * r + i) * 15 + 3 * s + j];
          }
        }
    for (int a = 0; a < 9; ++a)
      for (int r = 0; r < 5; ++r)
        if (cf[r][a] != 0.0)
          for (int i = 0; i < 3; ++i) fl[3 * a + i] += c->alpha1 * cf[r][a] * qv[3 * r + i];
    energy += c->alpha1 * psi_t;
  }
  /* to the global frame: block-diagonal transform with T3 */
  for (int a = 0; a < 9; ++a)
    for (int b = 0; b < 9; ++b) {
      double Bl[9], t[9], o[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Bl[i * 3 + j] = Kl[(3 * a + i) * 27 + 3 * b + j];
      m3_mul(t, Bl, c->T3);
      m3_tmul(o, c->T3, t);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) K[(3 * a + i) + 27 * (3 * b + j)] = o[i * 3 + j];
    }
  for (int a = 0; a < 9; ++a) m3_tvec(f + 3 * a, c->T3, fl + 3 * a);
  if (strain_energy) *strain_energy = energy;
}

void oracle_shell_commit(const os_const* c, os_hist* h, const double* d) {
  for (int g = 0; g < 3; ++g) {
    sgp k;
    shell_gp(c, h, d, g, &k);
    for (int j = 0; j < 3; ++j) {
      h->k1[g][j] = k.k1[j];
      h->k2[g][j] = k.k2[j];
    }
    m3_copy(h->Q[g], k.Q);
    double an[3];
    rodrigues_compose(an, k.al, h->alpha[g]);
    for (int j = 0; j < 3; ++j) {
      h->u[g][j] += k.u[j];
      h->alpha[g][j] = an[j];
      h->z1[g][j] = k.z1[j];
      h->z2[g][j] = k.z2[j];
    }
  }
}

void oracle_shell_pressure(const os_const* c, const double* pu, double p, int area_update, double* K, double* P) {
  const double* e1 = c->er;
  const double* e2 = c->er + 3;
  for (int k = 0; k < 6; ++k) {
    double t1[3], t2[3];
    for (int j = 0; j < 3; ++j) {
      double s1 = 0.0, s2 = 0.0;
      for (int n = 0; n < 6; ++n) {
        s1 += c->N41[k][n] * pu[3 * n + j];
        s2 += c->N42[k][n] * pu[3 * n + j];
      }
      t1[j] = e1[j] + s1;
      t2[j] = e2[j] + s2;
    }
    double cr[3];
    v3_cross(cr, t1, t2);
    double nc = v3_norm(cr);
    double np[3] = {(1.0 / nc) * cr[0], (1.0 / nc) * cr[1], (1.0 / nc) * cr[2]};
    double q[3] = {-p * np[0], -p * np[1], -p * np[2]};
    double fac = area_update ? c->w4[k] * nc : c->w4[k];
    for (int n = 0; n < 6; ++n)
      for (int j = 0; j < 3; ++j) P[3 * n + j] -= fac * c->N4[k][n] * q[j];
    /* load stiffness: (I - n n^T)/|t1 x t2| (or I with area update) times
     * skew(t1) N_x2 - skew(t2) N_x1 */
    double S1[9], S2[9], Pm[9];
    m3_skew(S1, t1);
    m3_skew(S2, t2);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double pr = (i == j ? 1.0 : 0.0) - np[i] * np[j];
        Pm[i * 3 + j] = area_update ? (i == j ? 1.0 : 0.0) : (1.0 / nc) * pr;
      }
    for (int b = 0; b < 6; ++b) {
      double Bb[9], Kb[9];
      for (int e = 0; e < 9; ++e) Bb[e] = S1[e] * c->N42[k][b] - S2[e] * c->N41[k][b];
      if (area_update) m3_copy(Kb, Bb);
      else m3_mul(Kb, Pm, Bb);
      for (int a = 0; a < 6; ++a) {
        double w = c->w4[k] * p * c->N4[k][a];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) K[(3 * a + i) + 27 * (3 * b + j)] += w * Kb[i * 3 + j];
      }
    }
  }
}

int oracle_shell_element(const double* xyz18, const double* mat3, double thickness, int n_hist,
                         const double* hist_disp, const double* disp27, int with_pressure, double pressure,
                         int area_update, double* K, double* f) {
  os_const c;
  os_hist h;
  oracle_shell_precalc(xyz18, mat3, thickness, &c, &h);
  double pu[18];
  memset(pu, 0, sizeof(pu));
  for (int q = 0; q < n_hist; ++q) {
    oracle_shell_commit(&c, &h, hist_disp + 27 * q);
    for (int i = 0; i < 18; ++i) pu[i] += hist_disp[27 * q + i];
  }
  oracle_shell_mount(&c, &h, disp27, K, f, NULL);
  if (with_pressure) {
    for (int i = 0; i < 18; ++i) pu[i] += disp27[i];
    oracle_shell_pressure(&c, pu, pressure, area_update, K, f);
  }
  return 0;
}

/* TransformMatrix (reference src/Shell_1.cpp:1470-1510) applied to a local
 * 27x27 (row-major Kl) and 27-vector: T^T Kl T added to K (column-major). */
static void shell_to_global(const os_const* c, const double* Kl, const double* fl, double* K, double* f) {
  for (int a = 0; a < 9; ++a)
    for (int b = 0; b < 9; ++b) {
      double Bl[9], t[9], o[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Bl[i * 3 + j] = Kl[(3 * a + i) * 27 + 3 * b + j];
      m3_mul(t, Bl, c->T3);
      m3_tmul(o, c->T3, t);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) K[(3 * a + i) + 27 * (3 * b + j)] += o[i * 3 + j];
    }
  if (f)
    for (int a = 0; a < 9; ++a) {
      double t3[3];
      m3_tvec(t3, c->T3, fl + 3 * a);
      for (int i = 0; i < 3; ++i) f[3 * a + i] += t3[i];
    }
}

/* rows of the 6x27 interpolation N (translations of the six nodes, rotations
 * of the midside nodes): N[i][col] for row i < 3 at col 3n+i with Nu[n], for
 * row 3+i at col 18+3m+i with Na[m] */
static void shell_add_NtDN(const double* Nu, const double* Na, const double* D, double w, double* Kl) {
  int col[6][6];
  double val[6][6];
  for (int i = 0; i < 3; ++i)
    for (int n = 0; n < 6; ++n) { col[i][n] = 3 * n + i; val[i][n] = Nu[n]; }
  for (int i = 0; i < 3; ++i)
    for (int n = 0; n < 6; ++n) {
      col[3 + i][n] = n < 3 ? 18 + 3 * n + i : -1;
      val[3 + i][n] = n < 3 ? Na[n] : 0.0;
    }
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double dij = D[i * 6 + j];
      if (dij == 0.0) continue;
      for (int p = 0; p < 6; ++p) {
        if (col[i][p] < 0) continue;
        for (int q = 0; q < 6; ++q) {
          if (col[j][q] < 0) continue;
          Kl[col[i][p] * 27 + col[j][q]] += w * val[i][p] * dij * val[j][q];
        }
      }
    }
}

void oracle_shell_inertia(const os_const* c, const os_hist* h, const double* d, const double* vel,
                          const double* acc, const double* a, double* K, double* f, double* kinetic) {
  double Kl[27 * 27], fl[27];
  memset(Kl, 0, sizeof(Kl));
  memset(fl, 0, sizeof(fl));
  const double Jr[9] = {c->coef2, 0, 0, 0, c->coef2, 0, 0, 0, 0};
  double ke = 0.0;
  for (int g = 0; g < 3; ++g) {
    const double* Nu = c->Nu[g];
    const double* Na = c->Na[g];
    double du[3] = {0, 0, 0}, da[3] = {0, 0, 0}, vi[3] = {0, 0, 0}, ai[3] = {0, 0, 0}, wi[3] = {0, 0, 0},
           dwi[3] = {0, 0, 0};
    for (int i = 0; i < 3; ++i) {
      for (int n = 0; n < 6; ++n) {
        du[i] += d[3 * n + i] * Nu[n];
        vi[i] += vel[6 * n + i] * Nu[n];
        ai[i] += acc[6 * n + i] * Nu[n];
      }
      for (int m = 0; m < 3; ++m) {
        da[i] += d[18 + 3 * m + i] * Na[m];
        wi[i] += vel[6 * (3 + m) + 3 + i] * Na[m];
        dwi[i] += acc[6 * (3 + m) + 3 + i] * Na[m];
      }
    }
    m3_vec(du, c->T3, du);
    m3_vec(da, c->T3, da);
    m3_vec(vi, c->T3, vi);
    m3_vec(ai, c->T3, ai);
    m3_vec(wi, c->T3, wi);
    m3_vec(dwi, c->T3, dwi);
    double dT[6], DdT[36], kg;
    oracle_gp_inertia(c->coef1, Jr, h->alpha[g], du, da, vi, ai, wi, dwi, a, dT, DdT, &kg);
    for (int i = 0; i < 3; ++i) {
      for (int n = 0; n < 6; ++n) fl[3 * n + i] += c->alpha1 * Nu[n] * dT[i];
      for (int m = 0; m < 3; ++m) fl[18 + 3 * m + i] += c->alpha1 * Na[m] * dT[3 + i];
    }
    shell_add_NtDN(Nu, Na, DdT, c->alpha1, Kl);
    ke += c->alpha1 * kg;
  }
  shell_to_global(c, Kl, fl, K, f);
  if (kinetic) *kinetic = ke;
}

void oracle_shell_modal_mass(const os_const* c, const double* rot, double* M) {
  double Ml[27 * 27];
  memset(Ml, 0, sizeof(Ml));
  memset(M, 0, sizeof(double) * 27 * 27);
  for (int k = 0; k < 6; ++k) {
    double al[3] = {0, 0, 0};
    for (int i = 0; i < 3; ++i)
      for (int m = 0; m < 3; ++m) al[i] += rot[3 * m + i] * c->Na4[k][m];
    m3_vec(al, c->T3, al);
    /* director d = Q(alpha) e3r; rotation block coef2 (|d|^2 I - d d^T) +
     * coef3 d d^T (EvaluateMassModal) */
    double Q[9], dv[3];
    rodrigues_Q(Q, al);
    for (int i = 0; i < 3; ++i) dv[i] = Q[i * 3 + 2];
    double d2 = v3_dot(dv, dv);
    double D[36];
    memset(D, 0, sizeof(D));
    for (int i = 0; i < 3; ++i) {
      D[i * 6 + i] = c->coef1;
      for (int j = 0; j < 3; ++j)
        D[(3 + i) * 6 + 3 + j] = (i == j ? c->coef2 * d2 : 0.0) + (c->coef3 - c->coef2) * dv[i] * dv[j];
    }
    shell_add_NtDN(c->N4[k], c->Na4[k], D, c->w4[k], Ml);
  }
  shell_to_global(c, Ml, NULL, M, NULL);
}
