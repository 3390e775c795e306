/* Shell_1 element restatement (oracle; test infrastructure).
 *
 * Six-node triangle, corners 1-3 with translations, midside nodes 4-6 with
 * translations and rotations: 27 element DOFs ordered as the reference's
 * Shell_1 (translations of nodes 1..6, then rotations of nodes 4..6).
 * Homogeneous section, Hooke material (compressible neo-Hookean response
 * integrated over the thickness, as reference src/Shell_1.cpp:1057-1158). */
#ifndef GIRAFFE_ORACLE_SHELL_H
#define GIRAFFE_ORACLE_SHELL_H
#include "oracle_common.h"

/* Per-element constants from Shell_1::PreCalc (reference
 * src/Shell_1.cpp:1666-2365). */
typedef struct os_const {
  double T3[9];       /* transform3: rows e1r, e2r, e3r */
  double er[9];       /* e1r, e2r, e3r (global) */
  double mu, lambda, stiff_drill, thick, area, alpha1;
  /* mass per unit area, rotary inertia of the fibre, drilling inertia of the
   * modal mass (reference src/Shell_1.cpp:2022-2024) */
  double coef1, coef2, coef3;
  /* shape data at the three midside Gauss points:
   * Nu[6], Na[3], and their x1 / x2 derivatives */
  double Nu[3][6], Nu1[3][6], Nu2[3][6];
  double Na[3][3], Na1[3][3], Na2[3][3];
  /* six-point rule for surface loads: weights and corner/midside
   * translation shape functions with their x1 / x2 derivatives */
  double w4[6];
  double N4[6][6], N41[6][6], N42[6][6];
  double Na4[6][3];   /* midside rotation shape functions at the six points */
} os_const;

/* Gauss-point history (reference src/Shell_1.cpp:1650-1664, 2357-2362). */
typedef struct os_hist {
  double Q[3][9];
  double k1[3][3], k2[3][3];
  double z1[3][3], z2[3][3];
  double u[3][3], alpha[3][3];
} os_hist;

/* xyz: 6 x 3 reference coordinates; mat: E, nu, rho; thickness. */
void oracle_shell_precalc(const double* xyz, const double* mat, double thickness, os_const* c, os_hist* h);
/* Mount (reference src/Shell_1.cpp:899-1332): d = 27 increments in element
 * DOF order (global frame).  K: 27x27 column-major (global frame), f: the
 * internal force vector (i_loading). */
void oracle_shell_mount(const os_const* c, const os_hist* h, const double* d, double* K, double* f,
                        double* strain_energy);
/* SaveLagrange at the converged increments d. */
void oracle_shell_commit(const os_const* c, os_hist* h, const double* d);
/* MountMass (reference src/Shell_1.cpp:2406-2498): inertial force and the
 * mass/gyroscopic tangent at the three midside Gauss points.  d: the 27
 * increments; vel / acc: [6][6] converged nodal velocities and accelerations
 * (global); a: Newmark a1..a6.  Adds to K (27x27 column-major, global) and f;
 * *kinetic (if not NULL) receives the kinetic energy at the end of the step. */
void oracle_shell_inertia(const os_const* c, const os_hist* h, const double* d, const double* vel,
                          const double* acc, const double* a, double* K, double* f, double* kinetic);
/* MountMassModal (reference src/Shell_1.cpp:2368-2396): the modal mass over
 * the six-point rule, from rot = [3][3] accumulated rotation vectors of the
 * midside nodes (copy_coordinates 3..5, global).  M: 27x27 column-major,
 * global frame: the alpha term of Rayleigh damping. */
void oracle_shell_modal_mass(const os_const* c, const double* rot, double* M);
/* Follower pressure (reference src/Shell_1.cpp:1392-1467): pu = 18 current
 * nodal displacements from the reference configuration (translations of
 * nodes 1..6, global), p = pressure.  Adds to P (unbalanced vector) and K. */
void oracle_shell_pressure(const os_const* c, const double* pu, double p, int area_update, double* K, double* P);
#endif
