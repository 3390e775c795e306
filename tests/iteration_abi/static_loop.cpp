// A GIRAFFE Static::Solve loop (reference src/Static.cpp:140-311) with its
// ConvergenceCriteria checks (src/ConvergenceCriteria.cpp:187-458), as a
// maintainer leaves it after binding the structure to the GPU: the
// element, load and global-assembly calls, UpdateDisps, SaveConfiguration
// and RestoreConfiguration go through the Newton-iteration boundary of
// libgiraffe_gpu.so, and sparsesystem through gf_sparse_solve.  The step
// control, the criteria and the host copy of the nodal increments stay
// the caller's, in the reference's order.
//
// Built by tests/test_gpu_iteration_abi.py with g++ against include/ and
// libgiraffe_gpu.so, and called through ctypes with the same
// gf_model_desc the batch path takes.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "giraffe_gpu.h"

namespace {

bool nan_or_huge(double v) { return !(v == v) || v >= 1e300 || v <= -1e300; }

// ConvergenceCriteria state of one solution step
struct Criteria {
  const gf_criteria* c;
  double force_crit = 0, moment_crit = 0, disp_crit = 0, rot_crit = 0;
  int n_conv_evaluated = 0;
  bool diverged = false;
};

// EstablishResidualCriteria: criteria from the first residual of the step,
// averaged over the steps so far
void establish(Criteria& k, const std::vector<int>& dof, const std::vector<double>& P) {
  double mf = 0, mm = 0;
  for (size_t i = 0; i < P.size(); ++i) {
    const double v = std::fabs(P[i]);
    if (dof[i] % 6 < 3) mf = std::fmax(mf, v);
    else mm = std::fmax(mm, v);
  }
  const gf_criteria* c = k.c;
  const double pf = k.force_crit, pm = k.moment_crit;
  double fc = mf * c->force_tol > c->force_min * c->force_tol ? mf * c->force_tol : c->force_min * c->force_tol;
  double mc = mm * c->moment_tol > c->moment_min * c->moment_tol ? mm * c->moment_tol : c->moment_min * c->moment_tol;
  k.force_crit = (k.n_conv_evaluated * pf + fc) / (k.n_conv_evaluated + 1);
  k.moment_crit = (k.n_conv_evaluated * pm + mc) / (k.n_conv_evaluated + 1);
  k.n_conv_evaluated++;
}

// CheckResidualConvergence
bool check_residual(Criteria& k, const std::vector<int>& dof, const std::vector<double>& P) {
  double mf = 0, mm = 0;
  bool has_f = false, has_m = false;
  for (size_t i = 0; i < P.size(); ++i) {
    const double v = std::fabs(P[i]);
    if (nan_or_huge(v)) k.diverged = true;
    if (dof[i] % 6 < 3) { has_f = true; mf = std::fmax(mf, v); }
    else { has_m = true; mm = std::fmax(mm, v); }
  }
  if (mf > k.c->divergence_ref || mm > k.c->divergence_ref) { k.diverged = true; return false; }
  return !((has_f && mf > k.force_crit) || (has_m && mm > k.moment_crit));
}

// CheckGLConvergence: increments x against the step's nodal displacements
bool check_gl(Criteria& k, const std::vector<int>& dof, const std::vector<double>& x,
              const std::vector<double>& disp) {
  double mdi = 0, mri = 0, mdv = 0, mrv = 0;
  bool has_d = false, has_r = false;
  for (size_t i = 0; i < x.size(); ++i) {
    const double inc = std::fabs(x[i]), val = std::fabs(disp[dof[i]]);
    if (nan_or_huge(inc)) k.diverged = true;
    if (dof[i] % 6 < 3) { has_d = true; mdi = std::fmax(mdi, inc); mdv = std::fmax(mdv, val); }
    else { has_r = true; mri = std::fmax(mri, inc); mrv = std::fmax(mrv, val); }
  }
  const gf_criteria* c = k.c;
  k.disp_crit = mdv * c->disp_tol > c->disp_min * c->disp_tol ? c->disp_tol * mdv : c->disp_min * c->disp_tol;
  k.rot_crit = mrv * c->rot_tol > c->rot_min * c->rot_tol ? c->rot_tol * mrv : c->rot_min * c->rot_tol;
  if (k.disp_crit > c->divergence_ref || k.rot_crit > c->divergence_ref) { k.diverged = true; return false; }
  return !((has_d && mdi > k.disp_crit) || (has_r && mri > k.rot_crit));
}

}  // namespace

// Runs the model's first solution step (a Static step) to its end.
// final_nodes: n_nodes x 15 (as gf_batch_results); stats: converged steps,
// Newton iterations (assemblies), bisections, aborted.  Returns 0, or the
// first nonzero status of a library call.
extern "C" int drive_static(gf_ctx* gpu, const gf_model_desc* m, double* final_nodes, int* stats) {
  gf_structure* s = gf_upload_structure(gpu, m, nullptr);
  if (!s) {
    std::fprintf(stderr, "gf_upload_structure: %s\n", gf_last_error(gpu));
    return GF_ERR_ARG;
  }
  int dims[4];
  gf_structure_dims(s, dims);
  const int n = dims[0], nnz = dims[1], nn = dims[3];
  std::vector<int> dof(n), row_ptr(n + 1), col_idx(nnz);
  gf_structure_dofs(s, dof.data());
  gf_structure_pattern(s, row_ptr.data(), col_idx.data());
  std::vector<double> K(nnz), P(n), disp(6 * (size_t)nn);
  const gf_solution& so = m->solution;
  Criteria crit;
  crit.c = &m->criteria;
  int rc = 0;
  bool aborted = false;
  int convergence_counter = 0, converged_number = 0, total_it = 0, bisections = 0;
  double last_converged_time = so.start_time;
  double time_step = so.time_step, time = last_converged_time;
  crit.diverged = false;
  while ((time < so.end_time || crit.diverged) && !aborted) {
    last_converged_time = time;
    time += time_step;
    if (time > 0.99999999 * so.end_time) {
      time = so.end_time;
      time_step = so.end_time - last_converged_time;
    }
    int it = 1;
    // Zeros + MountDisplacements
    if ((rc = gf_begin_step(s, last_converged_time, time_step))) break;
    std::fill(disp.begin(), disp.end(), 0.0);
    bool res_conv = false, gl_conv = false;
    crit.diverged = false;
    while ((!res_conv || !gl_conv) && !crit.diverged && !aborted) {
      // Clear, MountLocal, MountElementLoads, MountLoads, MountGlobal,
      // P_A = -P_A, MountSparse; K_AB X_B multiplies the zero X_B that
      // Clear leaves (src/Static.cpp:214-216)
      if ((rc = gf_assemble(s, GF_LAYOUT_CSR, K.data(), P.data()))) break;
      if (it == 1) establish(crit, dof, P);
      res_conv = check_residual(crit, dof, P);
      int info_fail = 0;
      if (!(res_conv && gl_conv)) {
        // sparsesystem
        if ((rc = gf_sparse_solve(gpu, n, row_ptr.data(), col_idx.data(), K.data(), P.data(), &info_fail))) break;
        res_conv = false;
        // UpdateDisps, on the device and in the caller's nodal increments
        if ((rc = gf_set_increment(s, P.data()))) break;
        for (int i = 0; i < n; ++i) disp[dof[i]] += P[i];
        gl_conv = check_gl(crit, dof, P, disp);
      }
      if ((it == so.max_it && !(res_conv && gl_conv)) || info_fail == 1) crit.diverged = true;
      if (time_step < so.min_time_step && time != so.end_time) aborted = true;
      ++it;
      ++total_it;
    }
    if (rc) break;
    if (!crit.diverged) {
      ++converged_number;
      if ((rc = gf_commit(s))) break;  // SaveConfiguration
      ++convergence_counter;
      if (it <= so.min_it || convergence_counter >= so.conv_increase) {
        time_step = time_step * so.inc_factor;
        if (time_step > so.max_time_step) time_step = so.max_time_step;
        convergence_counter = 0;
      }
    } else {
      if ((rc = gf_rollback(s))) break;  // RestoreConfiguration
      time -= time_step;
      time_step = time_step / 2.0;
      crit.diverged = false;
      convergence_counter = 0;
      ++bisections;
    }
  }
  if (rc) std::fprintf(stderr, "library call failed (%d): %s\n", rc, gf_last_error(gpu));
  if (!rc) rc = gf_structure_nodes(s, final_nodes, nullptr);
  stats[0] = converged_number;
  stats[1] = total_it;
  stats[2] = bisections;
  stats[3] = aborted ? 1 : 0;
  gf_structure_destroy(s);
  return rc;
}
