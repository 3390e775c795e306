/*
 * Static solution of one structure, CPU restatement.  TEST INFRASTRUCTURE
 * (oracle): the reference values for the CUDA solver and the timed CPU
 * baseline.
 *
 * Follows, for Beam_1 structures with nodal loads, constraints and prescribed
 * displacements:
 *   reference src/Static.cpp:140-311        load-step and Newton loops
 *   reference src/Solution.cpp:40-118       free/fixed DOF numbering
 *   reference src/Solution.cpp:121-224      DOF activation
 *   reference src/Solution.cpp:390-423      UpdateDisps
 *   reference src/Solution.cpp:426-575      Save/RestoreConfiguration
 *   reference src/Solution.cpp:798-849      Zeros, Clear
 *   reference src/ConvergenceCriteria.cpp:187-618
 *   reference src/NodalLoad.cpp:230-401     (UpdateforSolutionStep, Mount)
 *   reference src/NodalDisplacement.cpp:158-208, 327-410 (EulerAngles, EulerVector)
 *   reference src/Node.cpp:325-370          SaveConfiguration
 * The linear solve (PARDISO in the reference, src/SparseMatrix.cpp:74-166)
 * is an FP64 banded LU with partial pivoting on the same K_AA.
 *
 * Note on reference src/Static.cpp:214-215: global_X_B is cleared by
 * Clear() (src/Solution.cpp:841) at the top of every Newton iteration, after
 * MountDisplacements filled it, so the K_AB X_B correction multiplies a zero
 * vector; prescribed increments act through the nodal displacements alone.
 * The oracle therefore omits that product.
 */
#include "giraffe_oracle.h"

#include <float.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "band_lu.h"
#include "oracle_beam.h"
#include "oracle_shell.h"

static void newmark_coeff(double dt, double beta, double gamma, double* a);

typedef struct {
  const gf_model_desc* m;
  int nn, nb;
  int* GL;       /* [nn][6]: >0 free (1-based), <0 fixed, 0 inactive */
  int* active;   /* [nn][6] */
  int* cons;     /* [nn][6] */
  int n_free, n_fixed, kl, ku, ldab;
  int kl_nat;    /* half-bandwidth under the reference's numbering */
  double* disp;  /* increments in the step (Node::displacements) */
  double* copy;  /* Node::copy_coordinates */
  double* Qn;    /* Node::Q */
  double* vel; double* accel; double* copy_vel; double* copy_accel;
  ob_const* bc;
  ob_hist* bh;
  int ns;
  os_const* sc;
  os_hist* sh;
  double* ab; int* ipiv; double* PA;
  int* pf;      /* free DOF (GL - 1) -> row / column of the band solver */
  /* criteria state */
  double force_crit, moment_crit, disp_crit, rot_crit;
  int n_conv_evaluated;
  int diverged;
  /* loads: per nodal load, force/moment multipliers */
  double (*mult)[6];
  double last_converged_time, current_time_step;
  int dynamic;
  double a[6];  /* Newmark coefficients of the current step */
  /* Rayleigh damping (Beam_1::MountDamping, reference
   * src/Beam_1.cpp:1641-1665): C_e = alpha M_modal + beta K_e per element,
   * formed at the first Newton iteration of the step (the Dynamic::Solve
   * flag `first`) or at every iteration with Update 1 */
  int ray, ray_update, ray_init;
  double ray_alpha, ray_beta;
  double* rd;   /* [nb][18x18] column-major */
  double* rds;  /* [ns][27x27] column-major (Shell_1::MountDamping) */
  /* PipeLoads on each beam, in load order: load indices
   * pp_load[pp_off[e] .. pp_off[e + 1]) */
  int* pp_off;
  int* pp_load;
  /* Node::WriteMonitor's load vector per node and DOF at the last assembly:
   * the element P_loading summed into every active DOF (global_I_A for the
   * free ones, global_P_B for the fixed ones, which also carries -f of a
   * NodalLoad on them), and the monitor's persistent load rows */
  double* nload;
  double* mon_load;
  int sol_index;  /* index of the running solution step (the monitor starts with the first) */
} ost;

static void ost_free(ost* s) {
  free(s->GL); free(s->active); free(s->cons); free(s->disp); free(s->copy); free(s->Qn);
  free(s->vel); free(s->accel); free(s->copy_vel); free(s->copy_accel);
  free(s->bc); free(s->bh); free(s->sc); free(s->sh); free(s->ab); free(s->ipiv); free(s->PA); free(s->mult);
  free(s->rd); free(s->rds); free(s->pf); free(s->pp_off); free(s->pp_load); free(s->nload); free(s->mon_load);
}

/* global DOF numbers (GLs) of a Shell_1 element's 27 DOFs: translations of
 * nodes 1..6, then rotations of nodes 4..6 (reference
 * src/Shell_1.cpp:1513-1560) */
static void shell_dofs(const ost* s, int e, int* g) {
  const int* q = s->m->shells + 9 * e;
  for (int a = 0; a < 18; ++a) g[a] = s->GL[6 * q[a / 3] + a % 3];
  for (int a = 0; a < 9; ++a) g[18 + a] = s->GL[6 * q[3 + a / 3] + 3 + a % 3];
}

static void shell_increments(const ost* s, int e, double* d) {
  const int* q = s->m->shells + 9 * e;
  for (int a = 0; a < 18; ++a) d[a] = s->disp[6 * q[a / 3] + a % 3];
  for (int a = 0; a < 9; ++a) d[18 + a] = s->disp[6 * q[3 + a / 3] + 3 + a % 3];
}

static int ost_init(ost* s, const gf_model_desc* m) {
  memset(s, 0, sizeof(*s));
  s->m = m;
  s->nn = m->n_nodes;
  s->nb = m->n_beams;
  int nn = s->nn;
  s->GL = calloc((size_t)nn * 6, sizeof(int));
  s->active = calloc((size_t)nn * 6, sizeof(int));
  s->cons = calloc((size_t)nn * 6, sizeof(int));
  s->disp = calloc((size_t)nn * 6, sizeof(double));
  s->copy = calloc((size_t)nn * 6, sizeof(double));
  s->Qn = calloc((size_t)nn * 9, sizeof(double));
  s->vel = calloc((size_t)nn * 6, sizeof(double));
  s->accel = calloc((size_t)nn * 6, sizeof(double));
  s->copy_vel = calloc((size_t)nn * 6, sizeof(double));
  s->copy_accel = calloc((size_t)nn * 6, sizeof(double));
  s->bc = calloc((size_t)(s->nb ? s->nb : 1), sizeof(ob_const));
  s->bh = calloc((size_t)(s->nb ? s->nb : 1), sizeof(ob_hist));
  s->ns = m->n_shells;
  s->sc = calloc((size_t)(s->ns ? s->ns : 1), sizeof(os_const));
  s->sh = calloc((size_t)(s->ns ? s->ns : 1), sizeof(os_hist));
  s->mult = calloc((size_t)(m->n_loads ? m->n_loads : 1), sizeof(*s->mult));
  s->nload = calloc((size_t)nn * 6, sizeof(double));
  s->mon_load = calloc((size_t)nn * 6, sizeof(double));
  /* Node::Read sets copy_coordinates to the reference position
   * (reference src/Node.cpp:160-175); rotations start at zero */
  for (int i = 0; i < nn; ++i) {
    m3_eye(s->Qn + 9 * i);
    for (int k = 0; k < 3; ++k) s->copy[6 * i + k] = m->node_xyz[3 * i + k];
  }
  /* PipeLoad element lists (reference src/PipeLoad.cpp:123-138): the loads
   * of each Pipe_1 element in load order */
  s->pp_off = calloc((size_t)s->nb + 1, sizeof(int));
  int n_pp = 0;
  for (int l = 0; l < m->n_loads; ++l)
    if (m->loads[l].type == GF_LOAD_PIPE_PRESSURE) {
      for (int q = 0; q < m->loads[l].n_items; ++q) {
        const int e = m->loads[l].items[q];
        if (e < 0 || e >= s->nb || !m->beam_pipe_section || m->beam_pipe_section[e] < 0) return -1;
        s->pp_off[e + 1]++;
        ++n_pp;
      }
    }
  for (int e = 0; e < s->nb; ++e) s->pp_off[e + 1] += s->pp_off[e];
  s->pp_load = calloc((size_t)(n_pp ? n_pp : 1), sizeof(int));
  {
    int* fill = calloc((size_t)s->nb + 1, sizeof(int));
    for (int l = 0; l < m->n_loads; ++l)
      if (m->loads[l].type == GF_LOAD_PIPE_PRESSURE)
        for (int q = 0; q < m->loads[l].n_items; ++q) {
          const int e = m->loads[l].items[q];
          s->pp_load[s->pp_off[e] + fill[e]++] = l;
        }
    free(fill);
  }
  /* Beam_1::PreCalc */
  for (int e = 0; e < s->nb; ++e) {
    const int* b = m->beams + 6 * e;
    const int ps = m->beam_pipe_section ? m->beam_pipe_section[e] : -1;
    if (ps >= 0) /* Pipe_1::PreCalc */
      oracle_pipe_precalc(m->node_xyz + 3 * b[0], m->node_xyz + 3 * b[2], m->pipe_sections + 11 * ps,
                          m->cs + 6 * b[5], s->bc + e, s->bh + e);
    else
      oracle_beam_precalc(m->node_xyz + 3 * b[0], m->node_xyz + 3 * b[2], m->materials + 3 * b[3],
                          m->sections + 6 * b[4], m->cs + 6 * b[5], m->beam_pretension ? m->beam_pretension[e] : 0.0,
                          s->bc + e, s->bh + e);
  }
  /* Shell_1::PreCalc */
  for (int e = 0; e < s->ns; ++e) {
    const int* q = m->shells + 9 * e;
    double xyz[18];
    for (int j = 0; j < 6; ++j) memcpy(xyz + 3 * j, m->node_xyz + 3 * q[j], 3 * sizeof(double));
    oracle_shell_precalc(xyz, m->materials + 3 * q[6], m->shell_sections[q[7]], s->sc + e, s->sh + e);
  }
  /* DOFsActive: Beam_1 activates all six DOFs of its nodes; Shell_1 the
   * translations of its six nodes and the rotations of its midside nodes
   * (reference src/Beam_1.cpp:39-57, src/Shell_1.cpp:51-68) */
  for (int e = 0; e < s->nb; ++e)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 6; ++k) s->active[6 * m->beams[6 * e + j] + k] = 1;
  for (int e = 0; e < s->ns; ++e)
    for (int j = 0; j < 6; ++j)
      for (int k = 0; k < (j < 3 ? 3 : 6); ++k) s->active[6 * m->shells[9 * e + j] + k] = 1;
  if (m->constraints)
    for (int i = 0; i < nn * 6; ++i) s->cons[i] = m->constraints[i] ? 1 : 0;
  /* SetGlobalDOFs */
  int fr = 0, fx = 0;
  for (int i = 0; i < nn; ++i)
    for (int k = 0; k < 6; ++k) {
      if (s->cons[6 * i + k] == 0 && s->active[6 * i + k] == 1) s->GL[6 * i + k] = ++fr;
      if (s->cons[6 * i + k] == 1 && s->active[6 * i + k] == 1) s->GL[6 * i + k] = -(++fx);
    }
  s->n_free = fr;
  s->n_fixed = fx;
  /* bandwidth of K_AA under this numbering */
  int kl = 0;
  for (int e = 0; e < s->nb; ++e)
    for (int a = 0; a < 18; ++a)
      for (int b = 0; b < 18; ++b) {
        int ga = s->GL[6 * m->beams[6 * e + a / 6] + a % 6], gb = s->GL[6 * m->beams[6 * e + b / 6] + b % 6];
        if (ga > 0 && gb > 0 && ga - gb > kl) kl = ga - gb;
      }
  for (int e = 0; e < s->ns; ++e) {
    int g[27];
    shell_dofs(s, e, g);
    for (int a = 0; a < 27; ++a)
      for (int b = 0; b < 27; ++b)
        if (g[a] > 0 && g[b] > 0 && g[a] - g[b] > kl) kl = g[a] - g[b];
  }
  for (int l = 0; l < m->n_loads; ++l)
    if (m->loads[l].type == GF_LOAD_NODAL)
      for (int q = 0; q < m->loads[l].n_items; ++q) {
        int node = m->loads[l].items[q];
        for (int a = 3; a < 6; ++a)
          for (int b = 3; b < 6; ++b) {
            int ga = s->GL[6 * node + a], gb = s->GL[6 * node + b];
            if (ga > 0 && gb > 0 && ga - gb > kl) kl = ga - gb;
          }
      }
  s->kl_nat = kl;
  /* the band solver's order of the free DOFs: the reference's numbering,
   * or reverse Cuthill-McKee when that gives a narrower band */
  s->pf = malloc(sizeof(int) * (size_t)(fr ? fr : 1));
  for (int i = 0; i < fr; ++i) s->pf[i] = i;
  if (fr > 1) {
    size_t np = 0, cap = (size_t)s->nb * 324 + (size_t)s->ns * 729 + 1;
    int* pi = malloc(sizeof(int) * cap);
    int* pj = malloc(sizeof(int) * cap);
    for (int e = 0; e < s->nb; ++e)
      for (int a = 0; a < 18; ++a)
        for (int b = 0; b < 18; ++b) {
          int ga = s->GL[6 * m->beams[6 * e + a / 6] + a % 6], gb = s->GL[6 * m->beams[6 * e + b / 6] + b % 6];
          if (ga > 0 && gb > 0 && ga < gb) { pi[np] = ga - 1; pj[np] = gb - 1; np++; }
        }
    for (int e = 0; e < s->ns; ++e) {
      int g[27];
      shell_dofs(s, e, g);
      for (int a = 0; a < 27; ++a)
        for (int b = 0; b < 27; ++b)
          if (g[a] > 0 && g[b] > 0 && g[a] < g[b]) { pi[np] = g[a] - 1; pj[np] = g[b] - 1; np++; }
    }
    int *xadj, *adj;
    oracle_graph(fr, np, pi, pj, &xadj, &adj);
    int* perm = malloc(sizeof(int) * (size_t)fr);
    oracle_rcm(fr, xadj, adj, perm);
    if (oracle_perm_bandwidth(fr, xadj, adj, perm) < kl) {
      memcpy(s->pf, perm, sizeof(int) * (size_t)fr);
      kl = oracle_perm_bandwidth(fr, xadj, adj, perm);
    }
    free(perm); free(xadj); free(adj); free(pi); free(pj);
  }
  s->kl = s->ku = kl;
  s->ldab = 2 * kl + kl + 1;
  s->ab = malloc(sizeof(double) * (size_t)s->ldab * (size_t)(fr ? fr : 1));
  s->ipiv = malloc(sizeof(int) * (size_t)(fr ? fr : 1));
  s->PA = malloc(sizeof(double) * (size_t)(fr ? fr : 1));
  /* NodalLoad::UpdateforSolutionStep */
  for (int l = 0; l < m->n_loads; ++l) {
    const gf_load* L = m->loads + l;
    if (L->type != GF_LOAD_NODAL) continue;
    int cnt[6] = {0, 0, 0, 0, 0, 0};
    for (int q = 0; q < L->n_items; ++q)
      for (int k = 0; k < 6; ++k)
        if (s->active[6 * L->items[q] + k] != 0) cnt[k]++;
    for (int k = 0; k < 6; ++k) s->mult[l][k] = 1.0 / cnt[k];
  }
  return 0;
}

/* ---- global assembly ---- */
static void add_K(ost* s, int ga, int gb, double v) {
  if (ga > 0 && gb > 0) GB_AT(s->ab, s->ldab, s->kl, s->ku, s->pf[ga - 1], s->pf[gb - 1]) += v;
}

static void assemble(ost* s) {
  const gf_model_desc* m = s->m;
  memset(s->ab, 0, sizeof(double) * (size_t)s->ldab * (size_t)(s->n_free ? s->n_free : 1));
  memset(s->PA, 0, sizeof(double) * (size_t)(s->n_free ? s->n_free : 1));
  memset(s->nload, 0, sizeof(double) * 6 * (size_t)s->nn);
  double K[324], f[18], d[18];
  const double tnow = s->last_converged_time + s->current_time_step;
  for (int e = 0; e < s->nb; ++e) {
    const int* b = m->beams + 6 * e;
    for (int j = 0; j < 3; ++j) memcpy(d + 6 * j, s->disp + 6 * b[j], 6 * sizeof(double));
    oracle_beam_mount(s->bc + e, s->bh + e, d, K, f, NULL);
    /* PipeLoad on a Pipe_1 element (MountLoads, reference
     * src/PipeLoad.cpp Mount -> src/Pipe_1.cpp:1441-1494) */
    for (int q = s->pp_off[e]; q < s->pp_off[e + 1]; ++q) {
      const gf_load* L = m->loads + s->pp_load[q];
      const double* ps = m->pipe_sections + 11 * m->beam_pipe_section[e];
      const double Aint = OR_PI * ps[10] * ps[10] / 4.0;
      oracle_pipe_pressure(s->bc + e, s->bh + e, d, table_at(&L->table, tnow, 0), Aint, K, f);
    }
    if (s->dynamic) {
      /* MountMass + MountDamping + MountDyn (reference
       * src/Beam_1.cpp:1564-1673): K += M (+ a4 C), f += f_inertial (+ C v) */
      double v[18], ac[18];
      for (int j = 0; j < 3; ++j) {
        memcpy(v + 6 * j, s->copy_vel + 6 * b[j], 6 * sizeof(double));
        memcpy(ac + 6 * j, s->copy_accel + 6 * b[j], 6 * sizeof(double));
      }
      double* rd = s->ray ? s->rd + (size_t)324 * e : NULL;
      if (rd && (s->ray_update || !s->ray_init)) {
        double Mm[324];
        oracle_beam_modal_mass(s->bc + e, s->bh + e, Mm);
        for (int x = 0; x < 324; ++x) rd[x] = s->ray_alpha * Mm[x] + s->ray_beta * K[x];
      }
      oracle_beam_inertia(s->bc + e, s->bh + e, d, v, ac, s->a, K, f, NULL);
      if (rd) {
        double vi[18];
        for (int j = 0; j < 3; ++j) memcpy(vi + 6 * j, s->vel + 6 * b[j], 6 * sizeof(double));
        for (int x = 0; x < 324; ++x) K[x] += s->a[3] * rd[x];
        for (int q = 0; q < 18; ++q) {
          double acc = 0.0;
          for (int k = 0; k < 18; ++k) acc += rd[q + 18 * k] * vi[k];
          f[q] += acc;
        }
      }
    }
    int g[18];
    for (int a = 0; a < 18; ++a) g[a] = s->GL[6 * b[a / 6] + a % 6];
    for (int a = 0; a < 18; ++a) {
      if (g[a] != 0) s->nload[6 * b[a / 6] + a % 6] += f[a];
      if (g[a] > 0) s->PA[g[a] - 1] += f[a];
      for (int c = 0; c < 18; ++c) add_K(s, g[a], g[c], K[a + 18 * c]);
    }
  }
  double time = s->last_converged_time + s->current_time_step;
  /* Shell_1: Mount + MountElementLoads, then the ShellLoads acting on the
   * element (MountLoads, reference src/ShellLoad.cpp:133-148), then
   * MountGlobal */
  double Ks[729], fs[27], ds[27];
  for (int e = 0; e < s->ns; ++e) {
    shell_increments(s, e, ds);
    oracle_shell_mount(s->sc + e, s->sh + e, ds, Ks, fs, NULL);
    for (int l = 0; l < m->n_loads; ++l) {
      const gf_load* L = m->loads + l;
      if (L->type != GF_LOAD_SHELL_PRESSURE) continue;
      for (int q = 0; q < L->n_items; ++q) {
        if (L->items[q] != e) continue;
        double pu[18];
        const int* nd = m->shells + 9 * e;
        for (int a = 0; a < 18; ++a) {
          int node = nd[a / 3], k = a % 3;
          pu[a] = s->copy[6 * node + k] - m->node_xyz[3 * node + k] + s->disp[6 * node + k];
        }
        oracle_shell_pressure(s->sc + e, pu, table_at(&L->table, time, 0), L->area_update, Ks, fs);
      }
    }
    if (s->dynamic) {
      /* MountMass + MountDamping + MountDyn (reference
       * src/Shell_1.cpp:2406-2544): C from the stiffness that includes the
       * follower-pressure tangent, then K += M (+ a4 C), f += f_inertial
       * (+ C v) */
      const int* nd = m->shells + 9 * e;
      double v[36], ac[36];
      for (int j = 0; j < 6; ++j) {
        memcpy(v + 6 * j, s->copy_vel + 6 * nd[j], 6 * sizeof(double));
        memcpy(ac + 6 * j, s->copy_accel + 6 * nd[j], 6 * sizeof(double));
      }
      double* rd = s->ray ? s->rds + (size_t)729 * e : NULL;
      if (rd && (s->ray_update || !s->ray_init)) {
        double Mm[729], rot[9];
        for (int j = 0; j < 3; ++j) memcpy(rot + 3 * j, s->copy + 6 * nd[3 + j] + 3, 3 * sizeof(double));
        oracle_shell_modal_mass(s->sc + e, rot, Mm);
        for (int x = 0; x < 729; ++x) rd[x] = s->ray_alpha * Mm[x] + s->ray_beta * Ks[x];
      }
      oracle_shell_inertia(s->sc + e, s->sh + e, ds, v, ac, s->a, Ks, fs, NULL);
      if (rd) {
        double vi[27];
        for (int a = 0; a < 18; ++a) vi[a] = s->vel[6 * nd[a / 3] + a % 3];
        for (int a = 0; a < 9; ++a) vi[18 + a] = s->vel[6 * nd[3 + a / 3] + 3 + a % 3];
        for (int x = 0; x < 729; ++x) Ks[x] += s->a[3] * rd[x];
        for (int q = 0; q < 27; ++q) {
          double acc = 0.0;
          for (int k = 0; k < 27; ++k) acc += rd[q + 27 * k] * vi[k];
          fs[q] += acc;
        }
      }
    }
    int g[27];
    shell_dofs(s, e, g);
    for (int a = 0; a < 27; ++a) {
      if (g[a] != 0) {
        const int* nd = m->shells + 9 * e;
        const int node = a < 18 ? nd[a / 3] : nd[3 + (a - 18) / 3], k = a < 18 ? a % 3 : 3 + (a - 18) % 3;
        s->nload[6 * node + k] += fs[a];
      }
      if (g[a] > 0) s->PA[g[a] - 1] += fs[a];
      for (int c = 0; c < 27; ++c) add_K(s, g[a], g[c], Ks[a + 27 * c]);
    }
  }
  /* NodalLoad::Mount: P_A += -f, -Xi^T m pseudo-moments, K_AA += -V(alpha, Xi^T m) */
  for (int l = 0; l < m->n_loads; ++l) {
    const gf_load* L = m->loads + l;
    if (L->type != GF_LOAD_NODAL) continue;
    double CQ[9];
    cs_matrix(CQ, m->cs + 6 * L->cs);
    for (int q = 0; q < L->n_items; ++q) {
      int node = L->items[q];
      double fl[3], ml[3], fv[3], mv[3];
      for (int i = 0; i < 3; ++i) {
        fl[i] = s->mult[l][i] * table_at(&L->table, time, i);
        ml[i] = s->mult[l][3 + i] * table_at(&L->table, time, i + 3);
      }
      m3_tvec(fv, CQ, fl);
      m3_tvec(mv, CQ, ml);
      const double* al = s->disp + 6 * node + 3;
      double an = v3_norm(al), A[9], Xi[9];
      double gg = 4.0 / (4.0 + an * an);
      m3_skew(A, al);
      for (int k = 0; k < 9; ++k) Xi[k] = gg * 0.5 * A[k];
      Xi[0] += gg; Xi[4] += gg; Xi[8] += gg;
      double mm[3], V[9];
      m3_tvec(mm, Xi, mv);
      op_V(V, al, mm, an);
      for (int i = 0; i < 3; ++i) {
        int gi = s->GL[6 * node + i];
        if (s->active[6 * node + i] == 1 && gi > 0) s->PA[gi - 1] += -1.0 * fv[i];
        if (s->active[6 * node + i] == 1 && gi < 0) s->nload[6 * node + i] += -1.0 * fv[i];
      }
      for (int i = 0; i < 3; ++i) {
        int gi = s->GL[6 * node + 3 + i];
        if (s->active[6 * node + 3 + i] == 1 && gi > 0) s->PA[gi - 1] += -1.0 * mm[i];
        if (s->active[6 * node + 3 + i] == 1 && gi < 0) s->nload[6 * node + 3 + i] += -1.0 * mm[i];
        for (int j = 0; j < 3; ++j)
          if (s->active[6 * node + 3 + j] == 1) add_K(s, gi, s->GL[6 * node + 3 + j], -1.0 * V[i * 3 + j]);
      }
    }
  }
  for (int i = 0; i < s->n_free; ++i) s->PA[i] = -1.0 * s->PA[i];
}

/* ---- convergence criteria (reference src/ConvergenceCriteria.cpp) ---- */
static int nan_or_huge(double v) { return !(v == v) || v >= 1e300 || v <= -1e300; }

static void establish_residual_criteria(ost* s) {
  const gf_criteria* c = &s->m->criteria;
  double mf = 0, mm = 0;
  for (int i = 0; i < s->nn; ++i)
    for (int k = 0; k < 6; ++k) {
      int g = s->GL[6 * i + k];
      if (g > 0) {
        double v = fabs(s->PA[g - 1]);
        if (k < 3 && v > mf) mf = v;
        if (k >= 3 && v > mm) mm = v;
      }
    }
  double pf = s->force_crit, pm = s->moment_crit;
  s->force_crit = mf * c->force_tol > c->force_min * c->force_tol ? mf * c->force_tol : c->force_min * c->force_tol;
  s->moment_crit = mm * c->moment_tol > c->moment_min * c->moment_tol ? mm * c->moment_tol : c->moment_min * c->moment_tol;
  s->force_crit = (s->n_conv_evaluated * pf + s->force_crit) / (s->n_conv_evaluated + 1);
  s->moment_crit = (s->n_conv_evaluated * pm + s->moment_crit) / (s->n_conv_evaluated + 1);
  s->n_conv_evaluated++;
}

static int check_residual(ost* s) {
  const gf_criteria* c = &s->m->criteria;
  double mf = 0, mm = 0;
  int has_f = 0, has_m = 0;
  for (int i = 0; i < s->nn; ++i)
    for (int k = 0; k < 6; ++k) {
      int g = s->GL[6 * i + k];
      if (g > 0) {
        double v = fabs(s->PA[g - 1]);
        if (nan_or_huge(v)) s->diverged = 1;
        if (k < 3) { has_f = 1; if (v > mf) mf = v; }
        else { has_m = 1; if (v > mm) mm = v; }
      }
    }
  if (mf > c->divergence_ref || mm > c->divergence_ref) { s->diverged = 1; return 0; }
  int ok = 1;
  if (has_f && mf > s->force_crit) ok = 0;
  if (has_m && mm > s->moment_crit) ok = 0;
  return ok;
}

static int check_gl(ost* s) {
  const gf_criteria* c = &s->m->criteria;
  double mdi = 0, mri = 0, mdv = 0, mrv = 0;
  int has_d = 0, has_r = 0;
  for (int i = 0; i < s->nn; ++i)
    for (int k = 0; k < 6; ++k) {
      int g = s->GL[6 * i + k];
      if (g > 0) {
        double inc = fabs(s->PA[g - 1]);
        if (nan_or_huge(inc)) s->diverged = 1;
        double val = fabs(s->disp[6 * i + k]);
        if (k < 3) { has_d = 1; if (inc > mdi) mdi = inc; if (val > mdv) mdv = val; }
        else { has_r = 1; if (inc > mri) mri = inc; if (val > mrv) mrv = val; }
      }
    }
  s->disp_crit = mdv * c->disp_tol > c->disp_min * c->disp_tol ? c->disp_tol * mdv : c->disp_min * c->disp_tol;
  s->rot_crit = mrv * c->rot_tol > c->rot_min * c->rot_tol ? c->rot_tol * mrv : c->rot_min * c->rot_tol;
  if (s->disp_crit > c->divergence_ref || s->rot_crit > c->divergence_ref) { s->diverged = 1; return 0; }
  int ok = 1;
  if (has_d && mdi > s->disp_crit) ok = 0;
  if (has_r && mri > s->rot_crit) ok = 0;
  return ok;
}

/* ---- prescribed displacements (reference src/NodalDisplacement.cpp:158-208) ---- */
static void euler_angles_Q(double* Q, double phi, double th, double psi) {
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

static void mount_displacements(ost* s) {
  const gf_model_desc* m = s->m;
  double time = s->last_converged_time + s->current_time_step, dt = s->current_time_step;
  for (int l = 0; l < m->n_displacements; ++l) {
    const gf_displacement* D = m->displacements + l;
    double CQ[9];
    cs_matrix(CQ, m->cs + 6 * D->cs);
    for (int q = 0; q < D->n_nodes; ++q) {
      int node = D->nodes[q];
      double dl[3], dg[3];
      for (int j = 0; j < 3; ++j) dl[j] = table_at(&D->table, time, j) - table_at(&D->table, time - dt, j);
      m3_tvec(dg, CQ, dl);
      for (int j = 0; j < 3; ++j)
        if (s->cons[6 * node + j] == 1 && s->active[6 * node + j] == 1) {
          s->disp[6 * node + j] = dg[j];
          s->vel[6 * node + j] = dg[j] / dt;
          s->accel[6 * node + j] = (s->vel[6 * node + j] - s->copy_vel[6 * node + j]) / dt;
        }
      /* rotations: EulerAngles, reference src/NodalDisplacement.cpp:327-410 */
      double phi = s->cons[6 * node + 3] == 1 ? table_at(&D->table, time, 3) : 0.0;
      double th = s->cons[6 * node + 4] == 1 ? table_at(&D->table, time, 4) : 0.0;
      double psi = s->cons[6 * node + 5] == 1 ? table_at(&D->table, time, 5) : 0.0;
      double Q[9], t[9], Qd[9];
      if (D->angular == GF_ANGLES_VECTOR) {
        /* EulerVector: Rodrigues parameters of length 2 tan(|e|/2) along e
         * (reference src/NodalDisplacement.cpp:330-350) */
        double en = sqrt(phi * phi + th * th + psi * psi), inv = en != 0.0 ? 1.0 / en : 0.0;
        double rod = 2.0 * tan(en / 2.0);
        double rv[3] = {rod * (inv * phi), rod * (inv * th), rod * (inv * psi)}, A[9], A2[9];
        double g = 4.0 / (4.0 + rod * rod);
        m3_skew(A, rv);
        m3_mul(A2, A, A);
        for (int k = 0; k < 9; ++k) Q[k] = g * (A[k] + 0.5 * A2[k]);
        Q[0] += 1.0; Q[4] += 1.0; Q[8] += 1.0;
      } else {
        euler_angles_Q(Q, phi, th, psi);
      }
      m3_mul(t, Q, CQ);
      m3_tmul(Q, CQ, t);
      m3_mult(Qd, Q, s->Qn + 9 * node);
      double tr = Qd[0] + Qd[4] + Qd[8];
      if (tr > 3.0) tr = 3.0;
      double ax[3] = {0.5 * (Qd[7] - Qd[5]), 0.5 * (Qd[2] - Qd[6]), 0.5 * (Qd[3] - Qd[1])};
      double theta = 2.0 * asin(sqrt((3.0 - tr) / 4.0));
      double eu[3] = {0, 0, 0};
      if (theta != 0.0)
        for (int k = 0; k < 3; ++k) eu[k] = (theta / sin(theta)) * ax[k];
      double alpha = 2.0 * sqrt((3.0 - tr) / (1.0 + tr));
      double rod[3];
      for (int k = 0; k < 3; ++k) rod[k] = ((4.0 + alpha * alpha) / 4.0) * ax[k];
      for (int j = 3; j < 6; ++j)
        if (s->cons[6 * node + j] == 1 && s->active[6 * node + j] == 1) {
          s->disp[6 * node + j] = rod[j - 3];
          s->vel[6 * node + j] = eu[j - 3] / dt;
          s->accel[6 * node + j] = (s->vel[6 * node + j] - s->copy_vel[6 * node + j]) / dt;
        }
    }
  }
}

/* ---- commit (reference src/Node.cpp:325-370, src/Beam_1.cpp:1494-1506) ---- */
static void save_configuration(ost* s) {
  for (int i = 0; i < s->nn; ++i) {
    double* c = s->copy + 6 * i;
    const double* d = s->disp + 6 * i;
    for (int k = 0; k < 3; ++k) c[k] += d[k];
    double a3[3];
    rodrigues_compose(a3, d + 3, c + 3);
    memcpy(c + 3, a3, sizeof(a3));
    rodrigues_Q(s->Qn + 9 * i, a3);
    for (int k = 0; k < 6; ++k) {
      s->copy_accel[6 * i + k] = s->accel[6 * i + k];
      s->copy_vel[6 * i + k] = s->vel[6 * i + k];
    }
  }
  double d[18];
  for (int e = 0; e < s->nb; ++e) {
    const int* b = s->m->beams + 6 * e;
    for (int j = 0; j < 3; ++j) memcpy(d + 6 * j, s->disp + 6 * b[j], 6 * sizeof(double));
    oracle_beam_commit(s->bc + e, s->bh + e, d);
  }
  double ds[27];
  for (int e = 0; e < s->ns; ++e) {
    shell_increments(s, e, ds);
    oracle_shell_commit(s->sc + e, s->sh + e, ds);
  }
}

static void record(ost* s, oracle_record* rec, double time, int iterations) {
  if (!rec || rec->n >= rec->cap) return;
  int r = rec->n++;
  if (rec->time) rec->time[r] = time;
  if (rec->iterations) rec->iterations[r] = iterations;
  if (rec->nodes) {
    double* o = rec->nodes + (size_t)r * s->nn * 15;
    for (int i = 0; i < s->nn; ++i) {
      memcpy(o + 15 * i, s->copy + 6 * i, 6 * sizeof(double));
      memcpy(o + 15 * i + 6, s->Qn + 9 * i, 9 * sizeof(double));
    }
  }
  if (rec->gp_Q) {
    double* o = rec->gp_Q + (size_t)r * s->nb * 18;
    for (int e = 0; e < s->nb; ++e) memcpy(o + 18 * e, s->bh[e].Q, 18 * sizeof(double));
  }
}

/* One monitor line per monitored node (Node::WriteMonitor, reference
 * src/Node.cpp:227-320): time, copy_coordinates 0..2, the Euler rotation
 * vector of the accumulated Rodrigues vector (2 atan(|a| / 2) a / |a|,
 * src/Node.cpp:350-358), the load of every active DOF (I_A free, P_B fixed,
 * kept from the previous line where a DOF has no number yet), its moments
 * turned from pseudo-moments by Xi(alpha)^-T with alpha the node's last
 * rotation increment, the same six again (the local columns equal the
 * global ones in the spatial description), copy_vel and copy_accel. */
static void monitor_row(ost* s, oracle_record* rec, double time, int numbered) {
  if (!rec || !rec->monitor || rec->mon_n <= 0 || rec->mon_rows >= rec->mon_cap) return;
  double* row = rec->monitor + (size_t)rec->mon_rows * rec->mon_n * 31;
  rec->mon_rows++;
  for (int q = 0; q < rec->mon_n; ++q) {
    const int i = rec->mon_nodes[q];
    double* o = row + 31 * q;
    double* L = s->mon_load + 6 * i;
    if (numbered)
      for (int k = 0; k < 6; ++k)
        if (s->active[6 * i + k] == 1 && s->GL[6 * i + k] != 0) L[k] = s->nload[6 * i + k];
    const double* a = s->disp + 6 * i + 3;
    const double an = v3_norm(a), g = 4.0 / (4.0 + an * an);
    double A[9], Xt[9], inv[9], mo[3];
    m3_skew(A, a);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) Xt[r * 3 + c] = g * ((r == c ? 1.0 : 0.0) + 0.5 * A[c * 3 + r]);
    m3_inverse(inv, Xt);
    m3_vec(mo, inv, L + 3);
    for (int k = 0; k < 3; ++k) L[3 + k] = mo[k];
    o[0] = time;
    for (int k = 0; k < 3; ++k) o[1 + k] = s->copy[6 * i + k];
    const double* r3 = s->copy + 6 * i + 3;
    const double rn = v3_norm(r3), th = 2.0 * atan(rn / 2.0);
    for (int k = 0; k < 3; ++k) o[4 + k] = rn != 0.0 ? (th / rn) * r3[k] : 0.0;
    for (int k = 0; k < 6; ++k) o[7 + k] = o[13 + k] = L[k];
    for (int k = 0; k < 6; ++k) {
      o[19 + k] = s->copy_vel[6 * i + k];
      o[25 + k] = s->copy_accel[6 * i + k];
    }
  }
}

static int solve_linear(ost* s) {
  const int n = s->n_free;
  if (n == 0) return 0;
  int info = oracle_gbtrf(n, s->kl, s->ku, s->ab, s->ldab, s->ipiv);
  if (info) return 1;
  double* w = malloc(sizeof(double) * (size_t)n);
  for (int i = 0; i < n; ++i) w[s->pf[i]] = s->PA[i];
  oracle_gbtrs(n, s->kl, s->ku, s->ab, s->ldab, s->ipiv, w);
  for (int i = 0; i < n; ++i) s->PA[i] = w[s->pf[i]];
  free(w);
  for (int i = 0; i < n; ++i)
    if (!(s->PA[i] == s->PA[i])) return 1;
  return 0;
}

/* reference src/Static.cpp:140-311 */
static int static_solve(ost* s, const gf_solution* so, double start_time, oracle_record* rec, int* stats) {
  int aborted = 0, convergence_counter = 0, converged_number = 0, total_it = 0, bisections = 0;
  s->n_conv_evaluated = 0;
  s->last_converged_time = start_time;
  record(s, rec, start_time, 0);
  if (s->sol_index == 0) monitor_row(s, rec, start_time, 0);
  double time_step = so->time_step, time = s->last_converged_time;
  s->diverged = 0;
  for (int i = 0; i < s->nn * 6; ++i) s->copy_vel[i] = s->copy_accel[i] = s->vel[i] = s->accel[i] = 0.0;
  while ((time < so->end_time || s->diverged) && !aborted) {
    s->last_converged_time = time;
    time += time_step;
    if (time > 0.99999999 * so->end_time) {
      time = so->end_time;
      time_step = so->end_time - s->last_converged_time;
    }
    s->current_time_step = time_step;
    int it = 1;
    memset(s->disp, 0, sizeof(double) * 6 * (size_t)s->nn);
    mount_displacements(s);
    int res_conv = 0, gl_conv = 0;
    s->diverged = 0;
    while ((!res_conv || !gl_conv) && !s->diverged && !aborted) {
      assemble(s);
      if (it == 1) establish_residual_criteria(s);
      res_conv = check_residual(s);
      if (getenv("ORACLE_DEBUG")) {
        double mf = 0; for (int i = 0; i < s->n_free; ++i) if (fabs(s->PA[i]) > mf) mf = fabs(s->PA[i]);
        fprintf(stderr, "t=%g it=%d maxres=%.6e crit=%.3e\n", time, it, mf, s->force_crit);
      }
      int info_fail = 0;
      if (!(res_conv && gl_conv)) {
        info_fail = solve_linear(s);
        res_conv = 0;
        for (int i = 0; i < s->nn; ++i)
          for (int k = 0; k < 6; ++k)
            if (s->cons[6 * i + k] == 0 && s->active[6 * i + k] == 1)
              s->disp[6 * i + k] += s->PA[s->GL[6 * i + k] - 1];
        gl_conv = check_gl(s);
      }
      if ((it == so->max_it && !(res_conv && gl_conv)) || info_fail) s->diverged = 1;
      if (time_step < so->min_time_step && time != so->end_time) aborted = 1;
      it++;
      total_it++;
    }
    if (!s->diverged) {
      converged_number++;
      save_configuration(s);
      convergence_counter++;
      if (it <= so->min_it || convergence_counter >= so->conv_increase) {
        time_step = time_step * so->inc_factor;
        if (time_step > so->max_time_step) time_step = so->max_time_step;
        convergence_counter = 0;
      }
      if (!aborted) record(s, rec, time, it - 1);
      if (!aborted && rec && rec->mon_n > 0 &&
          (converged_number % (rec->mon_sample > 0 ? rec->mon_sample : 1) == 0 || time == so->end_time))
        monitor_row(s, rec, time, 1);
    } else {
      memset(s->disp, 0, sizeof(double) * 6 * (size_t)s->nn);
      for (int i = 0; i < s->nn * 6; ++i) { s->vel[i] = s->copy_vel[i]; s->accel[i] = s->copy_accel[i]; }
      time -= time_step;
      time_step = time_step / 2.0;
      s->diverged = 0;
      convergence_counter = 0;
      bisections++;
    }
  }
  if (stats) {
    stats[0] = converged_number;
    stats[1] = total_it;
    stats[2] = bisections;
    stats[3] = aborted;
  }
  return aborted ? 1 : 0;
}

/* UpdateDyn (reference src/Dynamic.cpp:480-580): Newmark velocities and
 * accelerations of the free DOFs; rotational ones transported by Q_delta.
 * The rotational scratch vectors persist across nodes within one call, as in
 * the reference (it only matters for nodes with some rotations fixed). */
static void update_dyn(ost* s) {
  const double* a = s->a;
  double vaux[3] = {0, 0, 0}, aaux[3] = {0, 0, 0};
  for (int i = 0; i < s->nn; ++i) {
    const double* d = s->disp + 6 * i;
    for (int j = 0; j < 3; ++j)
      if (s->GL[6 * i + j] > 0) {
        s->vel[6 * i + j] = d[j] * a[3] + s->copy_vel[6 * i + j] * a[4] + s->copy_accel[6 * i + j] * a[5];
        s->accel[6 * i + j] = d[j] * a[0] - s->copy_vel[6 * i + j] * a[1] - s->copy_accel[6 * i + j] * a[2];
      }
    double Qd[9];
    rodrigues_Q(Qd, d + 3);
    for (int j = 3; j < 6; ++j)
      if (s->GL[6 * i + j] > 0) {
        vaux[j - 3] = d[j] * a[3] + s->copy_vel[6 * i + j] * a[4] + s->copy_accel[6 * i + j] * a[5];
        aaux[j - 3] = d[j] * a[0] - s->copy_vel[6 * i + j] * a[1] - s->copy_accel[6 * i + j] * a[2];
      }
    m3_vec(vaux, Qd, vaux);
    m3_vec(aaux, Qd, aaux);
    for (int j = 3; j < 6; ++j)
      if (s->GL[6 * i + j] > 0) {
        s->vel[6 * i + j] = vaux[j - 3];
        s->accel[6 * i + j] = aaux[j - 3];
      }
  }
}

/* reference src/Dynamic.cpp:255-468 (no contact, no special constraints,
 * no InitialConditions blocks) */
static int dynamic_solve(ost* s, const gf_solution* so, double start_time, oracle_record* rec, int* stats) {
  int aborted = 0, convergence_counter = 0, converged_number = 0, total_it = 0, bisections = 0;
  s->n_conv_evaluated = 0;
  s->last_converged_time = start_time;
  record(s, rec, start_time, 0);
  if (s->sol_index == 0) monitor_row(s, rec, start_time, 0);
  double time_step = so->time_step, time = s->last_converged_time;
  /* ComputeInitialConditions (reference src/Solution.cpp:866-885): Zeros(),
   * ZeroIC when asked, then a SaveConfiguration that leaves every node's
   * configuration unchanged and makes the velocities the converged ones */
  memset(s->disp, 0, sizeof(double) * 6 * (size_t)s->nn);
  if (so->zero_ic)
    for (int i = 0; i < s->nn * 6; ++i) s->vel[i] = s->accel[i] = 0.0;
  for (int i = 0; i < s->nn * 6; ++i) { s->copy_vel[i] = s->vel[i]; s->copy_accel[i] = s->accel[i]; }
  s->ray_init = 0; /* Dynamic::Solve's `first`: C is formed anew */
  s->diverged = 0;
  while ((time < so->end_time || s->diverged) && !aborted) {
    s->last_converged_time = time;
    time += time_step;
    if (time > 0.99999999 * so->end_time) {
      time = so->end_time;
      time_step = so->end_time - s->last_converged_time;
    }
    s->current_time_step = time_step;
    newmark_coeff(time_step, so->beta, so->gamma, s->a);
    int it = 1;
    memset(s->disp, 0, sizeof(double) * 6 * (size_t)s->nn);
    mount_displacements(s);
    update_dyn(s);
    int res_conv = 0, gl_conv = 0;
    s->diverged = 0;
    while ((!res_conv || !gl_conv) && !s->diverged && !aborted) {
      assemble(s);
      s->ray_init = 1;
      if (it == 1) establish_residual_criteria(s);
      res_conv = check_residual(s);
      int info_fail = 0;
      if (!(res_conv && gl_conv)) {
        info_fail = solve_linear(s);
        res_conv = 0;
        for (int i = 0; i < s->nn; ++i)
          for (int k = 0; k < 6; ++k)
            if (s->cons[6 * i + k] == 0 && s->active[6 * i + k] == 1)
              s->disp[6 * i + k] += s->PA[s->GL[6 * i + k] - 1];
        update_dyn(s);
        gl_conv = check_gl(s);
      }
      if ((it == so->max_it && !(res_conv && gl_conv)) || info_fail) s->diverged = 1;
      if (time_step < so->min_time_step && time != so->end_time) aborted = 1;
      it++;
      total_it++;
    }
    if (!s->diverged) {
      converged_number++;
      save_configuration(s);
      convergence_counter++;
      if (!aborted) record(s, rec, time, it - 1);
      if (!aborted && rec && rec->mon_n > 0 &&
          (converged_number % (rec->mon_sample > 0 ? rec->mon_sample : 1) == 0 || time == so->end_time))
        monitor_row(s, rec, time, 1);
      if (it <= so->min_it || convergence_counter >= so->conv_increase) {
        time_step = time_step * so->inc_factor;
        if (time_step > so->max_time_step) time_step = so->max_time_step;
        convergence_counter = 0;
      }
    } else {
      memset(s->disp, 0, sizeof(double) * 6 * (size_t)s->nn);
      for (int i = 0; i < s->nn * 6; ++i) { s->vel[i] = s->copy_vel[i]; s->accel[i] = s->copy_accel[i]; }
      time -= time_step;
      time_step = time_step / 2.0;
      s->diverged = 0;
      convergence_counter = 0;
      bisections++;
    }
  }
  if (stats) {
    stats[0] = converged_number;
    stats[1] = total_it;
    stats[2] = bisections;
    stats[3] = aborted;
  }
  return aborted ? 1 : 0;
}

static void final_state(ost* s, double* out) {
  if (!out) return;
  for (int i = 0; i < s->nn; ++i) {
    memcpy(out + 15 * i, s->copy + 6 * i, 6 * sizeof(double));
    memcpy(out + 15 * i + 6, s->Qn + 9 * i, 9 * sizeof(double));
  }
}

/* The solution steps in sequence (reference src/main.cpp:52-60), each
 * starting at the previous one's end time (src/Database.cpp:759-768);
 * stats add up over the steps. */
int oracle_solve(const gf_model_desc* m, oracle_record* rec, double* final_nodes, int* stats) {
  ost s;
  if (ost_init(&s, m) != 0) {
    ost_free(&s);
    return -1;
  }
  int r = 0, total[4] = {0, 0, 0, 0};
  double start = m->solution.start_time;
  for (int k = 0; k <= m->n_next_steps && r == 0; ++k) {
    const gf_solution* so = k == 0 ? &m->solution : m->next_steps + (k - 1);
    s.sol_index = k;
    s.dynamic = so->type == GF_DYNAMIC;
    s.ray = s.dynamic && (so->rayleigh_alpha != 0.0 || so->rayleigh_beta != 0.0);
    if (s.ray) {
      s.ray_alpha = so->rayleigh_alpha;
      s.ray_beta = so->rayleigh_beta;
      s.ray_update = so->update_rayleigh;
      if (!s.rd) s.rd = calloc((size_t)324 * (s.nb ? s.nb : 1), sizeof(double));
      if (!s.rds) s.rds = calloc((size_t)729 * (s.ns ? s.ns : 1), sizeof(double));
    }
    int st[4] = {0, 0, 0, 0};
    r = s.dynamic ? dynamic_solve(&s, so, start, rec, st) : static_solve(&s, so, start, rec, st);
    for (int q = 0; q < 4; ++q) total[q] += st[q];
    start = so->end_time;
  }
  if (stats) memcpy(stats, total, sizeof(total));
  final_state(&s, final_nodes);
  ost_free(&s);
  return r;
}

int oracle_solve_batch(int n, const gf_model_desc* models, double** final_nodes, int* stats,
                       int threads) {
  int fails = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : 1) reduction(+ : fails)
  for (int i = 0; i < n; ++i)
    fails += oracle_solve(models + i, NULL, final_nodes ? final_nodes[i] : NULL, stats ? stats + 4 * i : NULL) != 0;
  return fails;
}

/* ---- element-level entry points for known-answer tests ---- */
int oracle_beam_element(const double* xyz9, const double* mat3, const double* sec6, const double* cs6,
                        int n_hist, const double* hist_disp, const double* disp18, double* K, double* f) {
  ob_const c;
  ob_hist h;
  oracle_beam_precalc(xyz9, xyz9 + 6, mat3, sec6, cs6, 0.0, &c, &h);
  for (int q = 0; q < n_hist; ++q) oracle_beam_commit(&c, &h, hist_disp + 18 * q);
  oracle_beam_mount(&c, &h, disp18, K, f, NULL);
  return 0;
}

/* One Pipe_1 element: PreCalc from the pipe section ps11, the committed
 * history, Mount at disp18 and, when p0i != 0, MountPipeSpecialLoads of an
 * internal pressure p0i (reference src/Pipe_1.cpp:836-974, 1106-1156,
 * 1441-1494).  K 18x18 column-major, f 18. */
int oracle_pipe_element(const double* xyz9, const double* ps11, const double* cs6, int n_hist,
                        const double* hist_disp, const double* disp18, double p0i, double* K, double* f) {
  ob_const c;
  ob_hist h;
  oracle_pipe_precalc(xyz9, xyz9 + 6, ps11, cs6, &c, &h);
  for (int q = 0; q < n_hist; ++q) oracle_beam_commit(&c, &h, hist_disp + 18 * q);
  oracle_beam_mount(&c, &h, disp18, K, f, NULL);
  if (p0i != 0.0) oracle_pipe_pressure(&c, &h, disp18, p0i, OR_PI * ps11[10] * ps11[10] / 4.0, K, f);
  return 0;
}

/* Tangent and residual of the first Newton iteration of the first load step
 * (all increments zero): K_AA in GB storage (ldab = 3 kl + 1, column-major,
 * n_free columns) and P_A.  dims receives n_free and kl.  With ab == NULL only
 * dims is filled. */
int oracle_first_tangent(const gf_model_desc* m, double* ab, double* PA, int* dims) {
  ost s;
  if (ost_init(&s, m) != 0) {
    ost_free(&s);
    return -1;
  }
  const int n = s.n_free, kn = s.kl_nat, ld = 3 * kn + 1;
  dims[0] = n;
  dims[1] = kn;
  if (ab) {
    s.last_converged_time = m->solution.start_time;
    s.current_time_step = m->solution.time_step;
    mount_displacements(&s);
    assemble(&s);
    /* back to the reference's numbering */
    memset(ab, 0, sizeof(double) * (size_t)ld * (size_t)n);
    for (int j = 0; j < n; ++j)
      for (int i = j - kn < 0 ? 0 : j - kn; i <= j + kn && i < n; ++i) {
        int pi = s.pf[i], pj = s.pf[j], d = pi - pj;
        if (d <= s.kl && -d <= s.ku) GB_AT(ab, ld, kn, kn, i, j) = GB_AT(s.ab, s.ldab, s.kl, s.ku, pi, pj);
      }
    memcpy(PA, s.PA, sizeof(double) * (size_t)n);
  }
  ost_free(&s);
  return 0;
}

/* The two matrices of a Modal solution step (reference
 * src/Modal.cpp:131-166): K_AA of MountLocal + MountElementLoads +
 * MountLoads at the step's start with zero increments (the static tangent),
 * and M_AA of MountMassModal (Beam_1 / Pipe_1 src/Beam_1.cpp:1538-1553 and
 * Shell_1 src/Shell_1.cpp:3171-), both in GB storage (ldab = 3 kl + 1,
 * column-major, n_free columns) in the reference's numbering.  dims
 * receives n_free and kl; with K == NULL only dims is filled. */
int oracle_modal_matrices(const gf_model_desc* m, double* K, double* M, int* dims) {
  ost s;
  if (ost_init(&s, m) != 0) {
    ost_free(&s);
    return -1;
  }
  const int n = s.n_free, kn = s.kl_nat, ld = 3 * kn + 1;
  dims[0] = n;
  dims[1] = kn;
  if (K) {
    s.last_converged_time = m->solution.start_time;
    s.current_time_step = 0.0;
    assemble(&s);
    for (int pass = 0; pass < 2; ++pass) {
      double* out = pass == 0 ? K : M;
      if (pass == 1) {
        /* the modal mass of every element, scattered as the tangent is */
        memset(s.ab, 0, sizeof(double) * (size_t)s.ldab * (size_t)(s.n_free ? s.n_free : 1));
        double Mm[729];
        for (int e = 0; e < s.nb; ++e) {
          const int* b = m->beams + 6 * e;
          oracle_beam_modal_mass(s.bc + e, s.bh + e, Mm);
          int g[18];
          for (int a = 0; a < 18; ++a) g[a] = s.GL[6 * b[a / 6] + a % 6];
          for (int a = 0; a < 18; ++a)
            for (int c = 0; c < 18; ++c) add_K(&s, g[a], g[c], Mm[a + 18 * c]);
        }
        for (int e = 0; e < s.ns; ++e) {
          const int* nd = m->shells + 9 * e;
          double rot[9];
          for (int j = 0; j < 3; ++j) memcpy(rot + 3 * j, s.copy + 6 * nd[3 + j] + 3, 3 * sizeof(double));
          oracle_shell_modal_mass(s.sc + e, rot, Mm);
          int g[27];
          shell_dofs(&s, e, g);
          for (int a = 0; a < 27; ++a)
            for (int c = 0; c < 27; ++c) add_K(&s, g[a], g[c], Mm[a + 27 * c]);
        }
      }
      memset(out, 0, sizeof(double) * (size_t)ld * (size_t)n);
      for (int j = 0; j < n; ++j)
        for (int i = j - kn < 0 ? 0 : j - kn; i <= j + kn && i < n; ++i) {
          int pi = s.pf[i], pj = s.pf[j], d = pi - pj;
          if (d <= s.kl && -d <= s.ku) GB_AT(out, ld, kn, kn, i, j) = GB_AT(s.ab, s.ldab, s.kl, s.ku, pi, pj);
        }
    }
  }
  ost_free(&s);
  return 0;
}

/* Newmark coefficients (reference src/Dynamic.cpp:582-590). */
static void newmark_coeff(double dt, double beta, double gamma, double* a) {
  a[0] = 1.0 / (dt * dt * beta);
  a[1] = 1.0 / (dt * beta);
  a[2] = 1.0 / (2.0 * beta) - 1.0;
  a[3] = gamma / (dt * beta);
  a[4] = 1.0 - gamma / beta;
  a[5] = dt * (1.0 - gamma / (2.0 * beta));
}

int oracle_beam_inertia_element(const double* xyz9, const double* mat3, const double* sec6, const double* cs6,
                                int n_hist, const double* hist_disp, const double* disp18, const double* vel18,
                                const double* acc18, double dt, double beta, double gamma, double* M, double* F,
                                double* ke) {
  ob_const c;
  ob_hist h;
  oracle_beam_precalc(xyz9, xyz9 + 6, mat3, sec6, cs6, 0.0, &c, &h);
  for (int q = 0; q < n_hist; ++q) oracle_beam_commit(&c, &h, hist_disp + 18 * q);
  double a[6];
  newmark_coeff(dt, beta, gamma, a);
  memset(M, 0, sizeof(double) * 324);
  memset(F, 0, sizeof(double) * 18);
  oracle_beam_inertia(&c, &h, disp18, vel18, acc18, a, M, F, ke);
  return 0;
}

int oracle_shell_inertia_element(const double* xyz18, const double* mat3, double thickness, int n_hist,
                                 const double* hist_disp, const double* disp27, const double* vel36,
                                 const double* acc36, double dt, double beta, double gamma, double* M, double* F,
                                 double* ke) {
  os_const c;
  os_hist h;
  oracle_shell_precalc(xyz18, mat3, thickness, &c, &h);
  for (int q = 0; q < n_hist; ++q) oracle_shell_commit(&c, &h, hist_disp + 27 * q);
  double a[6];
  newmark_coeff(dt, beta, gamma, a);
  memset(M, 0, sizeof(double) * 729);
  memset(F, 0, sizeof(double) * 27);
  oracle_shell_inertia(&c, &h, disp27, vel36, acc36, a, M, F, ke);
  return 0;
}
