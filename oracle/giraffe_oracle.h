/*
 * CPU oracle for the implicit Beam_1 / Shell_1 path.
 *
 * TEST INFRASTRUCTURE.  This library restates the reference's algorithm in
 * plain C so that the CUDA library can be checked against it and so that the
 * reference's CPU path can be timed on the GPU host, where the reference
 * itself is not available.  Only the test suite, the smoke check and the
 * CPU legs of bench.py load it; the product path never does.
 *
 * Parity is pinned: tests compare this oracle with the reference's own
 * sources compiled by oracle/build_ref.py (where the reference tree exists)
 * and with the golden fixtures generated from that build
 * (tests/golden/make_golden.py).
 */
#ifndef GIRAFFE_ORACLE_H
#define GIRAFFE_ORACLE_H
#include "../include/giraffe_model.h"
#ifdef __cplusplus
extern "C" {
#endif

/* Optional per-converged-step record.  nodes receives, per record and node,
 * copy_coordinates (translation + accumulated Rodrigues vector) followed by
 * the nodal rotation tensor Q (row-major): 15 doubles.  gp_Q receives, per
 * record, beam element and Gauss point, the Gauss point's Q_i (row-major). */
typedef struct oracle_record {
  int cap;
  int n;
  double* time;
  int* iterations;
  double* nodes;
  double* gp_Q;
  /* Monitor lines (optional): for the mon_n nodes mon_nodes, every
   * mon_sample-th converged step of a solution step and its end (and the
   * start of the first step), Node::WriteMonitor's 31 columns per node:
   * monitor[row][node][31], at most mon_cap rows; mon_rows receives the
   * count. */
  int mon_n;
  const int* mon_nodes;
  int mon_sample;
  int mon_cap;
  int mon_rows;
  double* monitor;
} oracle_record;

/* Runs the structure's solution step.  final_nodes (n_nodes x 15, optional)
 * receives the final nodal state; stats (4 ints, optional) receives converged
 * steps, Newton iterations, bisections and the aborted flag.  Returns 0 when
 * the step finished, 1 when it aborted, -1 for an unsupported model. */
int oracle_solve(const gf_model_desc* m, oracle_record* rec, double* final_nodes, int* stats);

/* Independent structures solved concurrently on `threads` host threads.
 * Returns the number of structures that did not finish. */
int oracle_solve_batch(int n, const gf_model_desc* models, double** final_nodes, int* stats,
                       int threads);

/* One Beam_1 element: PreCalc from nodal coordinates (3x3), material
 * (E, nu, rho), section (A, I11, I22, I12, It, I33) and CS (E1, E3); n_hist
 * committed increments (each 18 values, nodes x 6) build the Gauss-point
 * history; then Mount at disp18.  K: 18x18 column-major, f: 18. */
int oracle_beam_element(const double* xyz9, const double* mat3, const double* sec6, const double* cs6,
                        int n_hist, const double* hist_disp, const double* disp18, double* K, double* f);

/* K_AA (static tangent at the step's start) and M_AA (the modal mass of
 * MountMassModal) of a Modal solution step, GB storage as
 * oracle_first_tangent; K == NULL fills dims only. */
int oracle_modal_matrices(const gf_model_desc* m, double* K, double* M, int* dims);

/* One Pipe_1 element: as oracle_beam_element with a pipe section (EA, EI,
 * GJ, GA, Rho, CDt, CDn, CAt, CAn, De, Di) and, when p0i != 0, the
 * internal-pressure load of MountPipeSpecialLoads added to K and f. */
int oracle_pipe_element(const double* xyz9, const double* ps11, const double* cs6, int n_hist,
                        const double* hist_disp, const double* disp18, double p0i, double* K, double* f);

/* One Shell_1 element: PreCalc from nodal coordinates (6x3), material
 * (E, nu, rho) and thickness; n_hist committed increments (each 27 values in
 * element DOF order: translations of nodes 1..6, rotations of nodes 4..6)
 * build the Gauss-point history; then Mount at disp27, and with
 * with_pressure the follower pressure at the current configuration.
 * K: 27x27 column-major, f: 27 (P_loading). */
int oracle_shell_element(const double* xyz18, const double* mat3, double thickness, int n_hist,
                         const double* hist_disp, const double* disp27, int with_pressure, double pressure,
                         int area_update, double* K, double* f);
/* Shell_1 MountMass of one element after n_hist committed increments:
 * vel36 / acc36 = [6][6] converged nodal velocities and accelerations
 * (global), Newmark time step and parameters; M: 27x27 column-major,
 * F: 27, *ke. */
int oracle_shell_inertia_element(const double* xyz18, const double* mat3, double thickness, int n_hist,
                                 const double* hist_disp, const double* disp27, const double* vel36,
                                 const double* acc36, double dt, double beta, double gamma, double* M, double* F,
                                 double* ke);

#ifdef __cplusplus
}
#endif
#endif
