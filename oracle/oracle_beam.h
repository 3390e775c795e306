/* Beam_1 element restatement (oracle; test infrastructure). */
#ifndef GIRAFFE_ORACLE_BEAM_H
#define GIRAFFE_ORACLE_BEAM_H
#include "oracle_common.h"

/* Per-element constants from Beam_1::PreCalc. */
typedef struct ob_const {
  double T3[9];    /* transform3: rows E1, E2, E3 of the element CS */
  double D[36];    /* 6x6 constitutive matrix, row-major */
  double e3r[3];   /* element axis in the local frame */
  double jac;      /* L/2 */
  double N[2][3];  /* shape functions at the two Gauss points */
  double dN[2][3]; /* their derivatives (divided by the jacobian) */
  double Mr;       /* mass per unit length */
  double Jr[9];    /* rotary inertia per unit length */
} ob_const;

/* Gauss-point history (LagrangeSave, reference src/LagrangeSave.h:11-17). */
typedef struct ob_hist {
  double Q[2][9];
  double dz[2][3];
  double kap[2][3];
  double u[2][3];
  double alpha[2][3];
} ob_hist;

void oracle_beam_precalc(const double* x0, const double* x2, const double* mat, const double* sec,
                         const double* cs, double pretension, ob_const* c, ob_hist* h);
void oracle_beam_mount(const ob_const* c, const ob_hist* h, const double* d, double* K, double* f,
                       double* strain_energy);
/* Pipe_1::PreCalc from a PipeSection (EA, EI, GJ, GA, Rho, CDt, CDn, CAt,
 * CAn, De, Di) and MountPipeSpecialLoads (internal pressure p0i on the
 * internal area Aint; adds to K, 18x18 column-major, and f). */
void oracle_pipe_precalc(const double* x0, const double* x2, const double* ps, const double* cs, ob_const* c,
                         ob_hist* h);
void oracle_pipe_pressure(const ob_const* c, const ob_hist* h, const double* d, double p0i, double Aint, double* K,
                          double* f);
void oracle_beam_commit(const ob_const* c, ob_hist* h, const double* d);
/* One Gauss point of the inertia of a rigid cross-section (Beam_1) or
 * director fibre (Shell_1), in the element frame: mass Mr per unit length or
 * area, rotary inertia Jr in the reference frame, committed rotation vector
 * alpha_i, increments du / da, converged translational velocity and
 * acceleration vi / ai, angular velocity and acceleration wi / dwi, Newmark
 * coefficients a[6].  dT: 6 inertial forces, DdT: 6x6 row-major tangent,
 * *ke: kinetic energy density at the end of the step. */
void oracle_gp_inertia(double Mr, const double* Jr, const double* alpha_i, const double* du, const double* da,
                       const double* vi, const double* ai, const double* wi, const double* dwi, const double* a,
                       double* dT, double* DdT, double* ke);
/* Inertial force and its tangent (MountMass, Newmark coefficients a[6]);
 * vel/acc: [3][6] converged nodal velocities and accelerations. Adds to K
 * (18x18 column-major, global frame) and f. */
void oracle_beam_inertia(const ob_const* c, const ob_hist* h, const double* d, const double* vel,
                         const double* acc, const double* a, double* K, double* f, double* kinetic);
/* Modal mass (MountMassModal) in the global frame, 18x18 column-major:
 * the alpha term of Rayleigh damping. */
void oracle_beam_modal_mass(const ob_const* c, const ob_hist* h, double* M);
#endif
