/*
 * giraffe_model.h — flat description of one structure for the implicit
 * Beam_1 / Shell_1 path.  It carries what the reference reads from an input
 * deck for that path (reference src/IO.cpp:288-657): nodes, Hooke materials,
 * beam sections, shell sections, coordinate systems, Beam_1 and Shell_1
 * elements, nodal constraints, nodal loads, shell pressure loads, nodal
 * prescribed displacements, a sequence of Static and Dynamic solution steps
 * and the convergence criteria.  All indices are 0-based; all arrays are row-major
 * and owned by the caller for the duration of the call that takes them.
 *
 * Both the CUDA library (libgiraffe_gpu.so) and the CPU oracle take this
 * struct, so a caller builds a structure once and hands it to either.
 */
#ifndef GIRAFFE_MODEL_H
#define GIRAFFE_MODEL_H
#ifdef __cplusplus
extern "C" {
#endif

enum { GF_STATIC = 0, GF_DYNAMIC = 1 };
enum { GF_LOAD_NODAL = 0, GF_LOAD_SHELL_PRESSURE = 1, GF_LOAD_PIPE_PRESSURE = 2 };

/* A time table (reference src/Table.cpp:73-102: piecewise linear, clamped
 * to the first/last row outside its range).  values is [n_times][n_cols]. */
typedef struct gf_table {
  int n_times;
  int n_cols;
  const double* times;
  const double* values;
} gf_table;

/* NodalLoad (reference src/NodalLoad.cpp:322-401): force and moment, in the
 * coordinate system cs, split evenly over the nodes of the set, six table
 * columns (FX FY FZ MX MY MZ).  ShellLoad (reference src/ShellLoad.cpp:133-148
 * and src/Shell_1.cpp:1392-1467): follower pressure on a set of Shell_1
 * elements, one table column.  PipeLoad (reference src/PipeLoad.cpp,
 * src/Pipe_1.cpp:1441-1494): pressure on a set of Pipe_1 elements (items are
 * beam indices of Pipe_1 elements), four table columns P0I P0E RhoI RhoE, of
 * which the internal pressure P0I acts (on the section's internal area). */
typedef struct gf_load {
  int type;            /* GF_LOAD_NODAL, GF_LOAD_SHELL_PRESSURE or GF_LOAD_PIPE_PRESSURE */
  int n_items;         /* nodes (nodal), shell elements or Pipe_1 beams (pressure) */
  const int* items;
  int cs;              /* coordinate system of a nodal load */
  int area_update;     /* pressure: 1 = follow the current area */
  gf_table table;
} gf_load;

/* NodalDisplacement (reference src/NodalDisplacement.cpp:158-208): the six
 * table columns are prescribed UX UY UZ ROTX ROTY ROTZ in cs; the rotation
 * columns are Euler angles (AngularParameters EulerAngles, the default) or
 * the components of an Euler rotation vector (EulerVector,
 * src/NodalDisplacement.cpp:327-350). */
enum { GF_ANGLES_EULER = 0, GF_ANGLES_VECTOR = 1 };
typedef struct gf_displacement {
  int n_nodes;
  const int* nodes;
  int cs;
  gf_table table;
  int angular; /* GF_ANGLES_EULER or GF_ANGLES_VECTOR */
} gf_displacement;

/* Static (reference src/Static.cpp:43-130) and Dynamic
 * (reference src/Dynamic.cpp:66-241) solution-step parameters. */
typedef struct gf_solution {
  int type;            /* GF_STATIC or GF_DYNAMIC */
  double start_time;
  double end_time;
  double time_step;
  double max_time_step;
  double min_time_step;
  int max_it;
  int min_it;
  int conv_increase;
  double inc_factor;
  /* Dynamic only: Newmark and Rayleigh parameters */
  double beta;
  double gamma;
  double rayleigh_alpha;
  double rayleigh_beta;
  int update_rayleigh;
  int zero_ic;         /* Dynamic: ZeroIC, start from zero nodal velocities and
                          accelerations (reference src/Dynamic.cpp:209-216) */
} gf_solution;

/* ConvergenceCriteria (reference src/ConvergenceCriteria.cpp:15-60 gives the
 * defaults used by gf_default_criteria). */
typedef struct gf_criteria {
  double force_tol, moment_tol, force_min, moment_min, constraint_min;
  double disp_tol, rot_tol, lag_tol, disp_min, rot_min, lag_min;
  double divergence_ref;
} gf_criteria;

typedef struct gf_model_desc {
  int n_nodes;
  const double* node_xyz;        /* [n_nodes][3] reference coordinates */
  int n_materials;
  const double* materials;       /* [n][3]: E, nu, rho (Hooke) */
  int n_sections;
  const double* sections;        /* [n][6]: A, I11, I22, I12, It, I33 */
  int n_shell_sections;
  const double* shell_sections;  /* [n][1]: thickness (Homogeneous) */
  int n_cs;
  const double* cs;              /* [n][6]: E1 then E3 (E2 = E3 x E1) */
  int n_beams;
  const int* beams;              /* [n][6]: 3 nodes, material, section, cs */
  int n_shells;
  const int* shells;             /* [n][9]: 6 nodes, material, shell section, cs */
  const int* constraints;        /* [n_nodes][6]: 1 = prescribed DOF, or NULL */
  int n_loads;
  const gf_load* loads;
  int n_displacements;
  const gf_displacement* displacements;
  gf_solution solution;
  gf_criteria criteria;
  const double* beam_pretension; /* [n_beams]: Beam_1 PreTension T0 (force), or NULL
                                    (reference src/Beam_1.cpp:420-428, 616-621) */
  /* Solution steps after `solution`, run in sequence from the state the
   * previous one ends in (reference src/main.cpp:52-60).  Each starts at the
   * previous step's end time (src/Database.cpp:759-768; their start_time is
   * not read), restarts the residual-criterion average and the step control
   * (src/Static.cpp:143-166, src/Dynamic.cpp:257-287); a Static step zeroes
   * the nodal velocities and accelerations (Solution::ZerosVelAccel), a
   * Dynamic step keeps them unless zero_ic.  Constraints and prescribed
   * displacements apply to every step. */
  int n_next_steps;
  const gf_solution* next_steps;
  /* Pipe_1 elements (reference src/Pipe_1.cpp): Beam_1's kinematics with a
   * PipeSection's stiffness and mass (src/Pipe_1.cpp:1106-1156) and PipeLoad
   * pressures.  A Pipe_1 element is an entry of `beams` whose
   * beam_pipe_section is >= 0: its material and section columns are not read,
   * its stiffness is D = diag(GA, GA, EA, EI, EI, GJ), its mass Rho per unit
   * length and its rotary inertia Rho ((De/2)^2 - (Di/2)^2) diag(1/4, 1/4,
   * 1/2). */
  int n_pipe_sections;
  const double* pipe_sections;   /* [n][11]: EA, EI, GJ, GA, Rho, CDt, CDn, CAt, CAn, De, Di */
  const int* beam_pipe_section;  /* [n_beams]: -1 for Beam_1, else the pipe section; or NULL */
  /* Monitor (reference src/Monitor.cpp:112-195): MonitorNodes (0-based) and
   * Sample; lines are kept when gf_solve_opts.monitor_rows > 0 */
  int n_monitor_nodes;
  const int* monitor_nodes;
  int monitor_sample;
} gf_model_desc;

#ifdef __cplusplus
}
#endif
#endif
