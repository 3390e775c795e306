// Kernels of the device-resident Newton loop for batches of Beam_1
// structures.  One pass of the loop ("iteration") runs, for every structure
// whose step is in progress:
//
//   step_begin   load-step start: time advance, zero increments, prescribed
//                displacements (reference src/Static.cpp:176-197)
//   zero         clear K_AA band and P (reference src/Solution.cpp:833-849)
//   beam_mount   per colour: element tangent + internal force, scattered into
//                the band and P (reference src/Beam_1.cpp:695-843, 1429-1492)
//   loads        nodal loads, pseudo-moments, load stiffness
//                (reference src/NodalLoad.cpp:322-401)
//   residual     P = -P, criteria at the first iteration, residual check
//                (reference src/Static.cpp:210-221, ConvergenceCriteria.cpp)
//   band_solve   K_AA x = P (replaces sparsesystem, src/SparseMatrix.cpp:74-166)
//   update       UpdateDisps + increment check (src/Solution.cpp:390-423,
//                src/ConvergenceCriteria.cpp:289-458)
//   control      divergence, bisection, step growth (src/Static.cpp:236-298)
//   commit       SaveConfiguration (src/Node.cpp:325-370, Beam_1 1494-1506)
//
// Structures that are not iterating skip every kernel, so one launch
// sequence (captured as a CUDA graph) serves structures at different load
// steps.
#pragma once
#include <nvtx3/nvToolsExt.h>

#include "gf_types.h"

namespace gf {

// Optional per-kernel timing: when non-null, every launch of kernel class k
// is bracketed by events ev[2*i], ev[2*i+1] and recorded in cls[i].
struct LaunchProf {
  cudaEvent_t* ev;
  int* cls;
  int cap;
  int n;
};
enum KernelClass {
  KC_STEP_BEGIN = 0, KC_ZERO, KC_MOUNT, KC_LOADS, KC_RESIDUAL, KC_SOLVE, KC_UPDATE, KC_CONTROL,
  KC_COMMIT_ELEMS, KC_COMMIT_NODES, KC_CHAIN, KC_SCATTER, KC_SHELL, KC_WIDE_DIAG, KC_WIDE_TRSM, KC_WIDE_UPDATE,
  KC_WIDE_SUBST, KC_WIDE_REFINE, KC_COUNT
};
const char* kernel_class_name(int k);

// A named NVTX range for timeline tools (Nsight Systems): host phases of the
// library, and each kernel class of a profiled (launched, not replayed)
// pass.  Without an attached tool the calls return at once.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

// Brackets one launch with profiling events and an NVTX range of its
// kernel class (no-op when p is null).
struct ProfScope {
  LaunchProf* p;
  cudaStream_t st;
  int idx;
  ProfScope(LaunchProf* p_, cudaStream_t s, int k) : p(p_), st(s), idx(-1) {
    if (p && p->n < p->cap) {
      idx = p->n++;
      p->cls[idx] = k;
      nvtxRangePushA(kernel_class_name(k));
      cudaEventRecord(p->ev[2 * idx], st);
    }
  }
  ~ProfScope() {
    if (idx >= 0) {
      cudaEventRecord(p->ev[2 * idx + 1], st);
      nvtxRangePop();
    }
  }
};

void launch_iteration(const Batch& b, cudaStream_t st, bool commit_kernels = true, LaunchProf* prof = nullptr);
// FMA throughput probe: 8 independent chains per thread, `iters` steps.
void launch_fp_probe(bool fp64, void* out, int blocks, int threads, int iters, cudaStream_t st);
// First half of a pass (step start, zero, mount, loads, residual): leaves the
// assembled K_AA and P_A of the first iteration in the batch buffers.
void launch_iteration_partial(const Batch& b, cudaStream_t st);
// Commit of n standalone elements with nodal increments d ([n][18]).
void launch_beam_commit(int n, const BeamConst* c, BeamHist* h, BeamHistAux* x, const double* d, cudaStream_t st);
void launch_init_state(const Batch& b, cudaStream_t st);
// Stages of one Newton iteration driven by the caller's own step control:
// step start (prescribed displacements, Newmark predictor), assembly into
// every structure's band and P (P = -P at the end), the increment P added
// to the nodal displacements (UpdateDisps, UpdateDyn), SaveConfiguration of
// the structures whose commit flag is set.
void launch_step_begin(const Batch& b, cudaStream_t st);
void launch_assembly(const Batch& b, cudaStream_t st);
void launch_increment(const Batch& b, cudaStream_t st);
void launch_commit(const Batch& b, cudaStream_t st);
// Inertial force and tangent of n standalone elements; a: 6 Newmark
// coefficients in device memory.
void launch_beam_inertia(int n, const BeamConst* c, const BeamHistAux* x, const double* d, const double* v,
                         const double* a_acc, const double* a, double* M, double* F, cudaStream_t st);

// Element-level entry: tangent (18x18 column-major) and internal force of n
// elements in the global frame, FP64.  d: [n][18] nodal increments.
void launch_beam_elements(int n, const BeamConst* c, const BeamHist* h, const double* d, double* K,
                          double* f, cudaStream_t st);

// Shell_1 structures (gf_shell.cu): element tangent + follower pressure and
// the colour scatter into the wide band; zeroing of the wide band; the
// wide-band LU and triangular solves; SaveLagrange.
void launch_shell_mount(const Batch& b, cudaStream_t st);
void launch_wide_zero(const Batch& b, cudaStream_t st);
void launch_wide_solve(const Batch& b, cudaStream_t st, LaunchProf* prof = nullptr);
void launch_wide_subst(const Batch& b, int nrhs, cudaStream_t st);
// The first error of a wide-band capture step (a conditional node or body
// capture) since the last call on this thread; clears it.
cudaError_t wide_capture_error();
// The modal mass (MountMassModal) of every element added into a band of the
// structure's layout: entry (i, j) at (kw + i - j) + j W.
void launch_modal_mass(const Batch& b, double* M, int64_t W, int kw, cudaStream_t st);
void launch_shell_modal_mass(const Batch& b, double* M, int64_t W, int kw, cudaStream_t st);
void launch_shell_commit(const Batch& b, cudaStream_t st);
// Standalone Shell_1 elements (gf_shell_elements): d [n][27], pu [n][18],
// p [n] (NaN: no pressure); K [n][729] column-major, f [n][27].
void launch_shell_elements(int n, const ShellConst* c, const ShellHist* h, const double* d, const double* pu,
                           const double* p, int area_update, double* K, double* f, cudaStream_t st);
void launch_shell_commit_elements(int n, const ShellConst* c, ShellHist* h, ShellHistAux* x, const double* d,
                                  cudaStream_t st);
void launch_shell_inertia_elements(int n, const ShellConst* c, const ShellHistAux* x, const double* d,
                                   const double* v, const double* a_acc, const double* a, double* M, double* F,
                                   cudaStream_t st);
// Kernel launches of one pass of the shell and wide-band kernels.
int shell_launches_per_pass(const Batch& b);
int wide_launches_per_pass(const Batch& b);
long long wide_refine_launches(const Batch& b, long long sweeps, long long fallbacks);

// Band factor + solve of independent systems in the batch layout
// (GF_LDB rows); FP64.  Returns per-system info in state[].info_fail.
void launch_band_solve(const Batch& b, cudaStream_t st);

}  // namespace gf
