// The Newton-iteration boundary: a device-resident structure that the
// reference's own Static::Solve / Dynamic::Solve loop drives one call per
// step of its loop (reference src/Static.cpp:176-250,
// src/Dynamic.cpp:320-379), and element entries that take the reference's
// per-Gauss-point state as the reference stores it (LagrangeSave,
// src/LagrangeSave.h:11-17; Shell_1's own *_i arrays, src/Shell_1.h:117-127).
//
//   gf_upload_structure   DOFsActive + SetGlobalDOFs + SetGlobalSize and the
//                         elements' PreCalc (src/Solution.cpp:40-224,
//                         577-654): the structure, numbered, on the device
//   gf_begin_step         Zeros + MountDisplacements (src/Static.cpp:190-192;
//                         Dynamic: the Newmark predictor, src/Dynamic.cpp)
//   gf_assemble           Clear + MountLocal + MountElementLoads + MountLoads
//                         + MountGlobal + the sign flip of P_A + MountSparse
//                         (src/Static.cpp:206-216): K_AA in SparseMatrix's
//                         CSR or BandMatrix's GB layout, and P_A
//   gf_set_increment      UpdateDisps (src/Solution.cpp:390-423; Dynamic:
//                         UpdateDyn, src/Dynamic.cpp:480-580)
//   gf_commit             SaveConfiguration (src/Solution.cpp:426-500)
//   gf_rollback           RestoreConfiguration (src/Solution.cpp:502-575)
//
// Every vector crosses the boundary in the reference's free-DOF numbering
// (node by node, DOF by DOF, fixed and inactive DOFs skipped); the solver
// numbering inside (reverse Cuthill-McKee for some Shell_1 structures) stays
// inside.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/giraffe_gpu.h"
#include "gf_host_internal.h"
#include "gf_kernels.cuh"
#include "gf_types.h"

using namespace gf;
using namespace gfh;


namespace {

// Sets the Newton iteration counter of the structure (the residual criteria
// are established at iteration 1), or, with it < 0, marks an assembly done:
// Rayleigh matrices formed once per step are kept from now on, as the batch
// path's control kernel does after a pass.
__global__ void k_iter_set(Batch b, int it, int need_solve, int phase, int commit) {
  StructState& st = b.state[0];
  if (it > 0) st.it = it;
  if (it < 0 && b.params[0].ray_on) st.ray_init = 1;
  if (need_solve >= 0) st.need_solve = need_solve;
  if (phase >= 0) st.phase = phase;
  if (commit >= 0) {
    st.commit = commit;
    st.commit_dyn = b.params[0].dynamic;
  }
}

// Starts the step at (last_converged_time, time_step) of the caller.
__global__ void k_iter_begin(Batch b, double t0, double dt) {
  StructState& st = b.state[0];
  st.phase = PH_START;
  st.host_step = 1;
  st.last_converged_time = t0;
  st.current_time_step = dt;
}

// Moves the structure to solution step k of its description: that step's
// parameters, a fresh Rayleigh matrix, zero velocities if the step asks
// (reference src/main.cpp:52-60 with the transition of the batch path).
__global__ void k_iter_step(Batch b, int k) {
  StructState& st = b.state[0];
  const StructParams np = b.step_params[b.info[0].step_off + k];
  b.params[0] = np;
  st.step = k;
  st.ray_init = 0;
  st.zero_va = np.zero_va;
}

// The static tangent of the structure's current configuration, as a Modal
// step mounts it (reference src/Modal.cpp:157-166): the step's parameters
// with inertia and damping off for the assembly (restore = 0), then the
// step's own parameters again (restore = 1).
__global__ void k_iter_static(Batch b, int restore) {
  StructParams& p = b.params[0];
  if (restore) {
    p = b.step_params[b.info[0].step_off + b.state[0].step];
  } else {
    p.dynamic = 0;
    p.ray_on = 0;
  }
}

__global__ void k_csr_gather(int64_t nnz, const int64_t* src, const double* band, double* val) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nnz) return;
  const int64_t o = src[q];
  val[q] = o >= 0 ? band[o] : 0.0;
}

template <typename T> bool dev_alloc(gf_ctx* ctx, T** p, size_t n) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(n, 1) * sizeof(T));
  if (e != cudaSuccess) return set_err(ctx, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e));
  return true;
}

int sync(gf_structure* S) {
  gf_ctx* ctx = S->ctx;
  GF_CK(cudaGetLastError());
  GF_CK(cudaStreamSynchronize(S->B->stream));
  return GF_OK;
}

// Gauss-point state in the reference's layout <-> the kernels' layout
// (Q_i column-major there, row-major here).
void beam_state_in(const double* L2, BeamHist& h, BeamHistAux& x) {
  for (int g = 0; g < 2; ++g) {
    const double* L = L2 + g * GF_BEAM_LAG;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) h.Q[g][3 * i + j] = L[i + 3 * j];
    for (int i = 0; i < 3; ++i) {
      x.alpha[g][i] = L[9 + i];
      h.kap[g][i] = L[12 + i];
      x.u[g][i] = L[15 + i];
      h.dz[g][i] = L[18 + i];
    }
  }
}
void beam_state_out(const BeamHist& h, const BeamHistAux& x, double* L2) {
  for (int g = 0; g < 2; ++g) {
    double* L = L2 + g * GF_BEAM_LAG;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) L[i + 3 * j] = h.Q[g][3 * i + j];
    for (int i = 0; i < 3; ++i) {
      L[9 + i] = x.alpha[g][i];
      L[12 + i] = h.kap[g][i];
      L[15 + i] = x.u[g][i];
      L[18 + i] = h.dz[g][i];
    }
  }
}
void shell_state_in(const double* L3, ShellHist& h, ShellHistAux& x) {
  for (int g = 0; g < 3; ++g) {
    const double* L = L3 + g * GF_SHELL_LAG;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) h.Q[g][3 * i + j] = L[i + 3 * j];
    for (int i = 0; i < 3; ++i) {
      x.u[g][i] = L[9 + i];
      x.alpha[g][i] = L[12 + i];
      h.k1[g][i] = L[15 + i];
      h.k2[g][i] = L[18 + i];
      h.z1[g][i] = L[21 + i];
      h.z2[g][i] = L[24 + i];
    }
  }
}
void shell_state_out(const ShellHist& h, const ShellHistAux& x, double* L3) {
  for (int g = 0; g < 3; ++g) {
    double* L = L3 + g * GF_SHELL_LAG;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) L[i + 3 * j] = h.Q[g][3 * i + j];
    for (int i = 0; i < 3; ++i) {
      L[9 + i] = x.u[g][i];
      L[12 + i] = x.alpha[g][i];
      L[15 + i] = h.k1[g][i];
      L[18 + i] = h.k2[g][i];
      L[21 + i] = h.z1[g][i];
      L[24 + i] = h.z2[g][i];
    }
  }
}

}  // namespace

namespace gfh {
// K_AA of the structure's current configuration with zero increments and
// the loads at `time`, statically (no inertia or damping), in the
// structure's band (S->d_band, solver numbering).  Ends any step the caller
// had begun: a new gf_begin_step follows.
int structure_static_tangent(gf_structure* S, double time) {
  gf_ctx* ctx = S->ctx;
  gf_batch* B = S->B;
  cudaStream_t st = B->stream;
  k_iter_static<<<1, 1, 0, st>>>(B->b, 0);
  k_iter_begin<<<1, 1, 0, st>>>(B->b, time, 0.0);
  launch_step_begin(B->b, st);
  k_iter_set<<<1, 1, 0, st>>>(B->b, 1, -1, -1, -1);
  launch_assembly(B->b, st);
  k_iter_static<<<1, 1, 0, st>>>(B->b, 1);
  k_iter_set<<<1, 1, 0, st>>>(B->b, 0, -1, PH_START, 0);
  S->in_step = false;
  GF_CK(cudaGetLastError());
  return GF_OK;
}
}  // namespace gfh

extern "C" {

gf_structure* gf_upload_structure(gf_ctx* ctx, const gf_model_desc* model, const gf_solve_opts* opts) {
  if (!ctx || !model) {
    set_err(ctx, "gf_upload_structure: invalid arguments");
    return nullptr;
  }
  gf_solve_opts o;
  if (opts) o = *opts; else gf_default_opts(&o);
  o.use_graph = 0;
  gf_batch* B = gf_batch_create(ctx, 1, model, &o);
  if (!B) return nullptr;
  gf_structure* S = new gf_structure();
  S->ctx = ctx;
  S->B = B;
  const StructInfo& inf = B->info[0];
  S->nf = inf.n_free;
  S->n_nodes = inf.n_nodes;
  S->perm = B->perm[0];
  // h_gl holds the solver's free index of every node DOF; perm maps the
  // reference's index to the solver's
  std::vector<int> inv(S->nf);
  for (int i = 0; i < S->nf; ++i) inv[S->perm.empty() ? i : S->perm[i]] = i;
  S->dof_node.assign(S->nf, -1);
  for (int q = 0; q < inf.n_nodes * 6; ++q) {
    const int g = B->h_gl[(size_t)inf.node_off * 6 + q];
    if (g >= 0) S->dof_node[inv[g]] = q;
  }
  // CSR pattern and the band offset of every entry
  std::vector<std::vector<int>> rows;
  const int64_t nnz = csr_rows(B, 0, rows);
  if (nnz > INT32_MAX) {
    set_err(ctx, "gf_upload_structure: %lld nonzeros exceed 32-bit CSR indices", (long long)nnz);
    gf_batch_destroy(B);
    delete S;
    return nullptr;
  }
  S->W = inf.wide ? 2 * (int64_t)inf.wkl + 1 : GF_LDB;
  S->kw = inf.wide ? inf.wkl : GF_KB;
  S->d_band = inf.wide ? B->b.sh.wband + inf.wb_off : B->b.band + inf.band_off;
  std::vector<int64_t> src((size_t)std::max<int64_t>(nnz, 1));
  S->rp.assign(S->nf + 1, 0);
  S->ci.reserve((size_t)nnz);
  int64_t q = 0;
  for (int i = 0; i < S->nf; ++i) {
    S->rp[i] = (int)q;
    const int64_t pi = S->perm.empty() ? i : S->perm[i];
    for (int j : rows[i]) {
      const int64_t pj = S->perm.empty() ? j : S->perm[j];
      S->ci.push_back(j);
      src[q] = std::llabs(pi - pj) <= S->kw ? (S->kw + pi - pj) + pj * S->W : -1;
      S->kb = std::max(S->kb, std::abs(i - j));
      ++q;
    }
  }
  S->rp[S->nf] = (int)q;
  if (!dev_alloc(ctx, &S->d_src, src.size()) || !dev_alloc(ctx, &S->d_val, src.size()) ||
      cudaMemcpy(S->d_src, src.data(), sizeof(int64_t) * src.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      batch_reset(B) != GF_OK || cudaStreamSynchronize(B->stream) != cudaSuccess) {
    if (ctx->err.empty()) set_err(ctx, "gf_upload_structure: device set-up failed");
    gf_structure_destroy(S);
    return nullptr;
  }
  return S;
}

void gf_structure_destroy(gf_structure* S) {
  if (!S) return;
  if (S->d_src) cudaFree(S->d_src);
  if (S->d_val) cudaFree(S->d_val);
  gf_batch_destroy(S->B);
  delete S;
}

int gf_structure_dims(const gf_structure* S, int* dims) {
  if (!S || !dims) return GF_ERR_ARG;
  dims[0] = S->nf;
  dims[1] = S->rp.empty() ? 0 : S->rp.back();
  dims[2] = S->kb;
  dims[3] = S->n_nodes;
  return GF_OK;
}

int gf_structure_dofs(const gf_structure* S, int* dof_node) {
  if (!S || !dof_node) return GF_ERR_ARG;
  std::memcpy(dof_node, S->dof_node.data(), sizeof(int) * S->nf);
  return GF_OK;
}

int gf_structure_pattern(const gf_structure* S, int* row_ptr, int* col_idx) {
  if (!S) return GF_ERR_ARG;
  if (row_ptr) std::memcpy(row_ptr, S->rp.data(), sizeof(int) * S->rp.size());
  if (col_idx && !S->ci.empty()) std::memcpy(col_idx, S->ci.data(), sizeof(int) * S->ci.size());
  return GF_OK;
}

int gf_structure_set_step(gf_structure* S, int k) {
  if (!S || k < 0 || k >= S->B->info[0].n_steps) {
    set_err(S ? S->ctx : nullptr, "gf_structure_set_step: no solution step %d", k);
    return GF_ERR_ARG;
  }
  k_iter_step<<<1, 1, 0, S->B->stream>>>(S->B->b, k);
  return sync(S);
}

int gf_begin_step(gf_structure* S, double last_converged_time, double time_step) {
  if (!S || !(time_step > 0.0)) {
    set_err(S ? S->ctx : nullptr, "gf_begin_step: invalid arguments");
    return GF_ERR_ARG;
  }
  cudaStream_t st = S->B->stream;
  k_iter_begin<<<1, 1, 0, st>>>(S->B->b, last_converged_time, time_step);
  launch_step_begin(S->B->b, st);
  S->iteration = 1;
  S->in_step = true;
  return sync(S);
}

int gf_assemble(gf_structure* S, int layout, double* K, double* P_A) {
  if (!S || (layout != GF_LAYOUT_CSR && layout != GF_LAYOUT_GB)) return GF_ERR_ARG;
  gf_ctx* ctx = S->ctx;
  if (!S->in_step) {
    set_err(ctx, "gf_assemble: no step begun (gf_begin_step)");
    return GF_ERR_ARG;
  }
  gf_batch* B = S->B;
  cudaStream_t st = B->stream;
  const StructInfo& inf = B->info[0];
  k_iter_set<<<1, 1, 0, st>>>(B->b, S->iteration, -1, -1, -1);
  launch_assembly(B->b, st);
  k_iter_set<<<1, 1, 0, st>>>(B->b, -1, -1, -1, -1);
  const int nf = S->nf;
  if (P_A) {
    S->h_tmp.resize(nf);
    GF_CK(cudaMemcpyAsync(S->h_tmp.data(), B->b.P + inf.dof_off, sizeof(double) * nf, cudaMemcpyDeviceToHost, st));
  }
  if (K && layout == GF_LAYOUT_CSR) {
    const int64_t nnz = S->rp.back();
    if (nnz) {
      k_csr_gather<<<(unsigned)((nnz + 255) / 256), 256, 0, st>>>(nnz, S->d_src, S->d_band, S->d_val);
      GF_CK(cudaMemcpyAsync(K, S->d_val, sizeof(double) * nnz, cudaMemcpyDeviceToHost, st));
    }
  }
  std::vector<double> band;
  if (K && layout == GF_LAYOUT_GB) {
    band.resize((size_t)nf * S->W);
    GF_CK(cudaMemcpyAsync(band.data(), S->d_band, sizeof(double) * band.size(), cudaMemcpyDeviceToHost, st));
  }
  int r = sync(S);
  if (r != GF_OK) return r;
  auto pm = [&](int i) { return S->perm.empty() ? i : S->perm[i]; };
  if (P_A)
    for (int i = 0; i < nf; ++i) P_A[i] = S->h_tmp[pm(i)];
  if (K && layout == GF_LAYOUT_GB) {
    // BandMatrix storage (LAPACK GB, ldab = 3 kb + 1): entry (i, j) at
    // (2 kb + i - j) + j ldab
    const int kb = S->kb, ldab = 3 * kb + 1;
    std::memset(K, 0, sizeof(double) * (size_t)ldab * nf);
    for (int i = 0; i < nf; ++i)
      for (int k = S->rp[i]; k < S->rp[i + 1]; ++k) {
        const int j = S->ci[k];
        const int64_t pi = pm(i), pj = pm(j);
        if (std::llabs(pi - pj) > S->kw) continue;
        K[(size_t)(2 * kb + i - j) + (size_t)j * ldab] = band[(size_t)(S->kw + pi - pj) + (size_t)pj * S->W];
      }
  }
  return GF_OK;
}


int gf_set_increment(gf_structure* S, const double* x) {
  if (!S || !x) return GF_ERR_ARG;
  gf_ctx* ctx = S->ctx;
  if (!S->in_step) {
    set_err(ctx, "gf_set_increment: no step begun (gf_begin_step)");
    return GF_ERR_ARG;
  }
  gf_batch* B = S->B;
  cudaStream_t st = B->stream;
  const int nf = S->nf;
  S->h_tmp.resize(nf);
  for (int i = 0; i < nf; ++i) S->h_tmp[S->perm.empty() ? i : S->perm[i]] = x[i];
  GF_CK(cudaMemcpyAsync(B->b.P + B->info[0].dof_off, S->h_tmp.data(), sizeof(double) * nf, cudaMemcpyHostToDevice,
                        st));
  k_iter_set<<<1, 1, 0, st>>>(B->b, 0, 1, PH_ITER, -1);
  launch_increment(B->b, st);
  S->iteration++;
  return sync(S);
}

int gf_commit(gf_structure* S) {
  if (!S || !S->in_step) {
    set_err(S ? S->ctx : nullptr, "gf_commit: no step begun");
    return GF_ERR_ARG;
  }
  cudaStream_t st = S->B->stream;
  k_iter_set<<<1, 1, 0, st>>>(S->B->b, 0, -1, -1, 1);
  launch_commit(S->B->b, st);
  k_iter_set<<<1, 1, 0, st>>>(S->B->b, 0, -1, PH_START, 0);
  S->in_step = false;
  return sync(S);
}

int gf_rollback(gf_structure* S) {
  if (!S) return GF_ERR_ARG;
  gf_ctx* ctx = S->ctx;
  gf_batch* B = S->B;
  cudaStream_t st = B->stream;
  const size_t o = (size_t)B->info[0].node_off * 6, n = (size_t)S->n_nodes * 6 * sizeof(double);
  GF_CK(cudaMemsetAsync(B->b.disp + o, 0, n, st));
  GF_CK(cudaMemcpyAsync(B->b.vel + o, B->b.copy_vel + o, n, cudaMemcpyDeviceToDevice, st));
  GF_CK(cudaMemcpyAsync(B->b.accel + o, B->b.copy_accel + o, n, cudaMemcpyDeviceToDevice, st));
  k_iter_set<<<1, 1, 0, st>>>(B->b, 0, -1, PH_START, 0);
  S->in_step = false;
  return sync(S);
}

int gf_structure_nodes(gf_structure* S, double* nodes, double* increments) {
  if (!S) return GF_ERR_ARG;
  gf_ctx* ctx = S->ctx;
  gf_batch* B = S->B;
  cudaStream_t st = B->stream;
  const size_t nn = (size_t)S->n_nodes, o = (size_t)B->info[0].node_off;
  std::vector<double> c(nn * 6), q(nn * 9);
  if (nodes) {
    GF_CK(cudaMemcpyAsync(c.data(), B->b.copy + o * 6, sizeof(double) * c.size(), cudaMemcpyDeviceToHost, st));
    GF_CK(cudaMemcpyAsync(q.data(), B->b.Qn + o * 9, sizeof(double) * q.size(), cudaMemcpyDeviceToHost, st));
  }
  if (increments)
    GF_CK(cudaMemcpyAsync(increments, B->b.disp + o * 6, sizeof(double) * nn * 6, cudaMemcpyDeviceToHost, st));
  int r = sync(S);
  if (r != GF_OK) return r;
  if (nodes)
    for (size_t i = 0; i < nn; ++i) {
      std::memcpy(nodes + 15 * i, &c[6 * i], 6 * sizeof(double));
      std::memcpy(nodes + 15 * i + 6, &q[9 * i], 9 * sizeof(double));
    }
  return GF_OK;
}

// ---- element entries on the reference's per-Gauss-point state ----

int gf_beam_mount(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* sec, const double* cs,
                  const double* lag, const double* disp, double* K, double* f) {
  if (!ctx || n <= 0 || !xyz || !mat || !sec || !cs || !lag || !disp || !K || !f) {
    set_err(ctx, "gf_beam_mount: invalid arguments");
    return GF_ERR_ARG;
  }
  std::vector<BeamConst> c(n);
  std::vector<BeamHist> h(n);
  std::vector<BeamHistAux> x(n);
  for (int e = 0; e < n; ++e) {
    beam_precalc(xyz + 9 * (size_t)e, xyz + 9 * (size_t)e + 6, mat + 3 * (size_t)e, sec + 6 * (size_t)e,
                 cs + 6 * (size_t)e, c[e], h[e], x[e], 0.0);
    beam_state_in(lag + (size_t)e * 2 * GF_BEAM_LAG, h[e], x[e]);
  }
  BeamConst* dc = nullptr;
  BeamHist* dh = nullptr;
  double *dd = nullptr, *dK = nullptr, *df = nullptr;
  int rc = GF_OK;
  if (!dev_alloc(ctx, &dc, n) || !dev_alloc(ctx, &dh, n) || !dev_alloc(ctx, &dd, (size_t)n * 18) ||
      !dev_alloc(ctx, &dK, (size_t)n * 324) || !dev_alloc(ctx, &df, (size_t)n * 18)) {
    rc = GF_ERR_CUDA;
  } else {
    cudaStream_t st = ctx->stream;
    cudaMemcpyAsync(dc, c.data(), sizeof(BeamConst) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dh, h.data(), sizeof(BeamHist) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dd, disp, sizeof(double) * (size_t)n * 18, cudaMemcpyHostToDevice, st);
    launch_beam_elements(n, dc, dh, dd, dK, df, st);
    cudaMemcpyAsync(K, dK, sizeof(double) * (size_t)n * 324, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(f, df, sizeof(double) * (size_t)n * 18, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      rc = GF_ERR_CUDA;
      set_err(ctx, "gf_beam_mount: %s", cudaGetErrorString(e));
    }
  }
  cudaFree(dc); cudaFree(dh); cudaFree(dd); cudaFree(dK); cudaFree(df);
  return rc;
}

int gf_beam_save_lagrange(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* sec,
                          const double* cs, double* lag, const double* disp) {
  if (!ctx || n <= 0 || !xyz || !mat || !sec || !cs || !lag || !disp) {
    set_err(ctx, "gf_beam_save_lagrange: invalid arguments");
    return GF_ERR_ARG;
  }
  std::vector<BeamConst> c(n);
  std::vector<BeamHist> h(n);
  std::vector<BeamHistAux> x(n);
  for (int e = 0; e < n; ++e) {
    beam_precalc(xyz + 9 * (size_t)e, xyz + 9 * (size_t)e + 6, mat + 3 * (size_t)e, sec + 6 * (size_t)e,
                 cs + 6 * (size_t)e, c[e], h[e], x[e], 0.0);
    beam_state_in(lag + (size_t)e * 2 * GF_BEAM_LAG, h[e], x[e]);
  }
  BeamConst* dc = nullptr;
  BeamHist* dh = nullptr;
  BeamHistAux* dx = nullptr;
  double* dd = nullptr;
  int rc = GF_OK;
  if (!dev_alloc(ctx, &dc, n) || !dev_alloc(ctx, &dh, n) || !dev_alloc(ctx, &dx, n) ||
      !dev_alloc(ctx, &dd, (size_t)n * 18)) {
    rc = GF_ERR_CUDA;
  } else {
    cudaStream_t st = ctx->stream;
    cudaMemcpyAsync(dc, c.data(), sizeof(BeamConst) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dh, h.data(), sizeof(BeamHist) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dx, x.data(), sizeof(BeamHistAux) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dd, disp, sizeof(double) * (size_t)n * 18, cudaMemcpyHostToDevice, st);
    launch_beam_commit(n, dc, dh, dx, dd, st);
    cudaMemcpyAsync(h.data(), dh, sizeof(BeamHist) * n, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(x.data(), dx, sizeof(BeamHistAux) * n, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      rc = GF_ERR_CUDA;
      set_err(ctx, "gf_beam_save_lagrange: %s", cudaGetErrorString(e));
    } else {
      for (int e2 = 0; e2 < n; ++e2) beam_state_out(h[e2], x[e2], lag + (size_t)e2 * 2 * GF_BEAM_LAG);
    }
  }
  cudaFree(dc); cudaFree(dh); cudaFree(dx); cudaFree(dd);
  return rc;
}

int gf_shell_mount(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* thick, const double* lag,
                   const double* disp, const double* cur_xyz, const double* pressure, int area_update, double* K,
                   double* f) {
  if (!ctx || n <= 0 || !xyz || !mat || !thick || !lag || !disp || !K || !f || (pressure && !cur_xyz)) {
    set_err(ctx, "gf_shell_mount: invalid arguments");
    return GF_ERR_ARG;
  }
  std::vector<ShellConst> c(n);
  std::vector<ShellHist> h(n);
  std::vector<ShellHistAux> x(n);
  std::vector<double> pu((size_t)n * 18, 0.0), p(n, std::nan(""));
  for (int e = 0; e < n; ++e) {
    shell_precalc(xyz + 18 * (size_t)e, mat + 3 * (size_t)e, thick[e], c[e], h[e], x[e]);
    shell_state_in(lag + (size_t)e * 3 * GF_SHELL_LAG, h[e], x[e]);
    if (pressure) {
      // follower pressure at the displaced configuration: the nodes' current
      // positions (copy_coordinates) plus this iteration's increments
      for (int a = 0; a < 18; ++a)
        pu[(size_t)e * 18 + a] = cur_xyz[(size_t)e * 18 + a] - xyz[(size_t)e * 18 + a] + disp[(size_t)e * 27 + a];
      p[e] = pressure[e];
    }
  }
  ShellConst* dc = nullptr;
  ShellHist* dh = nullptr;
  double *dd = nullptr, *dpu = nullptr, *dp = nullptr, *dK = nullptr, *df = nullptr;
  int rc = GF_OK;
  if (!dev_alloc(ctx, &dc, n) || !dev_alloc(ctx, &dh, n) || !dev_alloc(ctx, &dd, (size_t)n * 27) ||
      !dev_alloc(ctx, &dpu, (size_t)n * 18) || !dev_alloc(ctx, &dp, (size_t)n) || !dev_alloc(ctx, &dK, (size_t)n * 729) ||
      !dev_alloc(ctx, &df, (size_t)n * 27)) {
    rc = GF_ERR_CUDA;
  } else {
    cudaStream_t st = ctx->stream;
    cudaMemcpyAsync(dc, c.data(), sizeof(ShellConst) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dh, h.data(), sizeof(ShellHist) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dd, disp, sizeof(double) * (size_t)n * 27, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dpu, pu.data(), sizeof(double) * pu.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dp, p.data(), sizeof(double) * p.size(), cudaMemcpyHostToDevice, st);
    launch_shell_elements(n, dc, dh, dd, dpu, dp, area_update, dK, df, st);
    cudaMemcpyAsync(K, dK, sizeof(double) * (size_t)n * 729, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(f, df, sizeof(double) * (size_t)n * 27, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      rc = GF_ERR_CUDA;
      set_err(ctx, "gf_shell_mount: %s", cudaGetErrorString(e));
    }
  }
  cudaFree(dc); cudaFree(dh); cudaFree(dd); cudaFree(dpu); cudaFree(dp); cudaFree(dK); cudaFree(df);
  return rc;
}

int gf_shell_save_lagrange(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* thick, double* lag,
                           const double* disp) {
  if (!ctx || n <= 0 || !xyz || !mat || !thick || !lag || !disp) {
    set_err(ctx, "gf_shell_save_lagrange: invalid arguments");
    return GF_ERR_ARG;
  }
  std::vector<ShellConst> c(n);
  std::vector<ShellHist> h(n);
  std::vector<ShellHistAux> x(n);
  for (int e = 0; e < n; ++e) {
    shell_precalc(xyz + 18 * (size_t)e, mat + 3 * (size_t)e, thick[e], c[e], h[e], x[e]);
    shell_state_in(lag + (size_t)e * 3 * GF_SHELL_LAG, h[e], x[e]);
  }
  ShellConst* dc = nullptr;
  ShellHist* dh = nullptr;
  ShellHistAux* dx = nullptr;
  double* dd = nullptr;
  int rc = GF_OK;
  if (!dev_alloc(ctx, &dc, n) || !dev_alloc(ctx, &dh, n) || !dev_alloc(ctx, &dx, n) ||
      !dev_alloc(ctx, &dd, (size_t)n * 27)) {
    rc = GF_ERR_CUDA;
  } else {
    cudaStream_t st = ctx->stream;
    cudaMemcpyAsync(dc, c.data(), sizeof(ShellConst) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dh, h.data(), sizeof(ShellHist) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dx, x.data(), sizeof(ShellHistAux) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dd, disp, sizeof(double) * (size_t)n * 27, cudaMemcpyHostToDevice, st);
    launch_shell_commit_elements(n, dc, dh, dx, dd, st);
    cudaMemcpyAsync(h.data(), dh, sizeof(ShellHist) * n, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(x.data(), dx, sizeof(ShellHistAux) * n, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      rc = GF_ERR_CUDA;
      set_err(ctx, "gf_shell_save_lagrange: %s", cudaGetErrorString(e));
    } else {
      for (int e2 = 0; e2 < n; ++e2) shell_state_out(h[e2], x[e2], lag + (size_t)e2 * 3 * GF_SHELL_LAG);
    }
  }
  cudaFree(dc); cudaFree(dh); cudaFree(dx); cudaFree(dd);
  return rc;
}

}  // extern "C"
