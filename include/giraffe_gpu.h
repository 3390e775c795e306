/*
 * giraffe_gpu.h — C ABI of the GB300 implementation of GIRAFFE's implicit
 * nonlinear finite-element step for Beam_1 and Shell_1 structures (Static and
 * Dynamic solution steps).
 *
 * Every function is extern "C", takes plain pointers and sizes, returns an
 * int status (0 = success) unless stated otherwise, and records a message
 * for gf_last_error on failure.  Host arrays are owned by the caller.  A
 * context owns one CUDA stream on one device; calls on one context must not
 * overlap.
 *
 * Reference interfaces each entry point replaces (paths in the reference
 * repository alfredogneto/GIRAFFE):
 *   gf_solve / gf_batch_*   Solution::Solve of a Static or Dynamic solution
 *                           step for one or many structures:
 *                           src/Static.cpp:140-311, src/Dynamic.cpp:255-590 with
 *                           Solution::MountLocal/MountGlobal/UpdateDisps/
 *                           SaveConfiguration/RestoreConfiguration
 *                           (src/Solution.cpp:227-575) and the
 *                           ConvergenceCriteria checks
 *                           (src/ConvergenceCriteria.cpp:187-618)
 *   gf_beam_inertia_elements Beam_1::MountMass (src/Beam_1.cpp:1564-1638)
 *   gf_shell_inertia_elements Shell_1::MountMass (src/Shell_1.cpp:2406-2498)
 *   gf_shell_elements       Shell_1::PreCalc + SaveLagrange + Mount +
 *                           MountElementLoads + MountShellSpecialLoads
 *                           (src/Shell_1.cpp:899-1467, 1650-2365)
 *   gf_beam_elements        Beam_1::PreCalc + SaveLagrange + Mount +
 *                           MountElementLoads (src/Beam_1.cpp:501-843,
 *                           1494-1506)
 *   gf_batch_assemble       MountLocal + MountLoads + MountGlobal +
 *                           SparseMatrix::Mount into the BandMatrix layout
 *                           (src/Solution.cpp:227-349, src/SparseMatrix.cpp:58-71,
 *                           src/BandMatrix.cpp:221-250)
 *   gf_batch_assemble_csr   the same into the SparseMatrix CSR layout
 *                           (src/SparseMatrix.cpp:58-71)
 *   gf_band_solve           bandsystem (src/BandMatrix.cpp:257-287)
 *   gf_sparse_solve         the Newton solve sparsesystem
 *                           (src/SparseMatrix.cpp:74-166) on SparseMatrix's CSR
 *   gf_upload_structure ... Solution's per-iteration helpers on one device-
 *   gf_rollback             resident structure (section "Newton-iteration
 *                           boundary" below)
 *   gf_beam_mount,          Beam_1::Mount / SaveLagrange and Shell_1::Mount /
 *   gf_*_save_lagrange,     SaveLagrange on the reference's stored Gauss-point
 *   gf_shell_mount          state
 */
#ifndef GIRAFFE_GPU_H
#define GIRAFFE_GPU_H
#include <stddef.h>

#include "giraffe_model.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gf_ctx gf_ctx;
typedef struct gf_batch gf_batch;

enum {
  GF_OK = 0,
  GF_ERR_ARG = 1,      /* invalid argument or unsupported model */
  GF_ERR_CUDA = 2,     /* CUDA runtime error */
  GF_ERR_SINGULAR = 3, /* zero or non-finite pivot (info_fail = 1 in the reference) */
  GF_ERR_TIMEOUT = 4   /* a bounded device wait gave up */
};

enum { GF_PREC_FP64 = 0, GF_PREC_MIXED = 1 };

typedef struct gf_solve_opts {
  int precision;   /* GF_PREC_FP64 (plain) or GF_PREC_MIXED: the Beam_1
                      tangent's rotation and K_e expansion in FP32-pair
                      arithmetic (the operator itself FP64), and Shell_1 wide-band
                      K_AA factored in FP32 (its LU beside the FP64 K_AA) with
                      FP64 iterative refinement (x += K32^-1 (b - K x)) until
                      a correction is below 2^-52 |x| or shrinks by less than
                      half; a solve that stalls above 2^-30 |x|, or is still
                      refining after max_refine sweeps, is refactored in FP64
                      (reference: src/SparseMatrix.cpp:74-166, PARDISO with
                      iterative refinement) */
  int poll_every;  /* Newton passes between host checks for completion */
  int use_graph;   /* capture one Newton pass as a CUDA graph */
  int wide_update; /* Shell_1 wide-band LU trailing update: GF_WIDE_TENSOR (the
                      default: FP64 products emulated from exact bf16 slices
                      on the tensor cores, Ozaki scheme, tcgen05.mma with
                      tensor-memory accumulators), GF_WIDE_TENSOR_SYNC (the
                      same emulation on warp-level mma.sync) or GF_WIDE_FP64
                      (FP64 FMA).  The emulated product of row i of L21 and
                      column j of U12 (K = 64 terms) errs by at most about
                      2^-52 K max_k |L_ik 2^-f_k| max_k |2^f_k U_kj|, where
                      2^f_k is a power-of-two balancing of the panel's column
                      k of L21 against row k of U12 (chosen per panel); for
                      rows whose terms differ greatly in magnitude that can
                      exceed the FP64 rounding of the product sum */
  int max_passes;  /* host cap on the Newton passes of one gf_batch_run;
                      beyond it the run stops with GF_ERR_TIMEOUT (0: the
                      default of 4,000,000) */
  int monitor_rows; /* monitor lines kept per structure with a Monitor
                      (gf_model_desc monitor_nodes; 0: none recorded) */
  int max_refine;  /* GF_PREC_MIXED: FP64 refinement sweeps of a wide-band
                      solve before its FP64 fallback (0: the default of 30) */
  int wide_tiles[4]; /* Shell_1 wide-band LU tile shapes: rows per CTA of the
                      bulk trsm (4, 8, 16) and of the first trsm (1, 2, 4),
                      the corner update's tile edge (4, 8), rows per CTA of
                      the triangular solves (32, 64).  An entry of 0 is picked
                      by the autotuner, which times the shapes on a synthetic
                      band of the structures' half-bandwidth once per context
                      (served waves take the defaults 8, 2, 8, 64).  No
                      choice changes any result. */
} gf_solve_opts;
enum { GF_WIDE_FP64 = 0, GF_WIDE_TENSOR = 1, GF_WIDE_TENSOR_SYNC = 2 };

/* Per-structure result of a solution step. */
typedef struct gf_stats {
  int converged_steps;    /* converged load steps */
  int newton_iterations;  /* Newton passes (element mounts) */
  int bisections;         /* rolled-back steps */
  int aborted;            /* 1 when the step size fell below MinTimeStep */
  int linear_solves;      /* linear solves performed */
  int refine_sweeps;      /* GF_PREC_MIXED: FP64 refinement sweeps of the FP32 wide-band factor */
  int fp64_fallbacks;     /* GF_PREC_MIXED: wide-band solves refactored in FP64 */
} gf_stats;

/* Context on CUDA device `device`; NULL on failure. */
gf_ctx* gf_create(int device);
void gf_destroy(gf_ctx* ctx);
const char* gf_last_error(const gf_ctx* ctx);
void gf_default_opts(gf_solve_opts* opts);
/* Options of the context's standalone solves (gf_band_solve and
 * gf_sparse_solve, which have no options argument, as bandsystem and
 * sparsesystem have none): their wide-band trailing update follows
 * opts->wide_update (GF_WIDE_TENSOR until set).  The batch entry points take
 * their own options. */
int gf_ctx_set_opts(gf_ctx* ctx, const gf_solve_opts* opts);

/* Uploads n structures into one device batch: each a sequence of Static and
 * Dynamic solution steps of Beam_1 elements or of Shell_1 elements (with
 * follower pressures), with nodal loads, constraints and prescribed
 * displacements.  Shell_1 structures are solved by the wide-band LU on the
 * narrower of the reference's numbering and reverse Cuthill-McKee. */
gf_batch* gf_batch_create(gf_ctx* ctx, int n, const gf_model_desc* models, const gf_solve_opts* opts);
void gf_batch_destroy(gf_batch* batch);
/* Restores the initial configuration of every structure (device side). */
int gf_batch_reset(gf_batch* batch);
/* Runs every structure's solution step to its end (or abort) on the device. */
int gf_batch_run(gf_batch* batch);
/* Runs at most max_passes Newton passes (fewer only in effect: passes after
 * every structure finished change nothing); *running receives the number of
 * structures still running.  gf_batch_run continues from where it stops. */
int gf_batch_step(gf_batch* batch, int max_passes, int* running);
/* Checkpoint / resume of a batch between passes (the in-memory counterpart
 * of the reference's last converged configuration, Solution::
 * SaveConfiguration / RestoreConfiguration, src/Solution.cpp:426-575, here
 * with the step machine and the Gauss-point histories, so a restore resumes
 * exactly): gf_batch_snapshot copies the batch's device state into `host`
 * (gf_batch_snapshot_bytes long, a header first: structure, node, element
 * and shell counts, damping flags, total size), gf_batch_restore puts it
 * back.  A snapshot whose header does not match the batch (taken from a
 * batch of other structures) is refused with GF_ERR_ARG and nothing is
 * written. */
int gf_batch_snapshot_bytes(const gf_batch* batch, size_t* bytes);
int gf_batch_snapshot(gf_batch* batch, void* host);
int gf_batch_restore(gf_batch* batch, const void* host);
/* Final nodal state per structure: final_nodes[s] holds n_nodes x 15 doubles
 * (copy_coordinates: position and accumulated Rodrigues vector, then the
 * nodal rotation tensor Q row-major); stats may be NULL. */
int gf_batch_results(gf_batch* batch, double* const* final_nodes, gf_stats* stats);
/* Device time of the last gf_batch_run in milliseconds (CUDA events on the
 * batch's stream), and the number of kernels it launched. */
double gf_batch_last_ms(const gf_batch* batch);
long long gf_batch_last_launches(const gf_batch* batch);
/* First Newton pass of structure s from its initial configuration: K_AA in
 * the reference's BandMatrix storage (LAPACK GB, ldab = 3*kb + 1 rows, kb =
 * the structure's half-bandwidth, n_free columns) and P_A after the sign
 * flip.  dims (optional) receives n_free and kb. */
int gf_batch_assemble(gf_batch* batch, int s, double* ab, double* PA, int* dims);
/* The same first-pass K_AA in the reference's SparseMatrix layout
 * (src/SparseMatrix.cpp:58-71: Eigen RowMajor CSR, 0-based, the union of
 * every element's free-DOF pattern with duplicates summed, zeros kept):
 * row_ptr (n_free + 1), col_idx and val (nnz), P_A (n_free), all in the
 * reference's DOF numbering.  dims receives n_free and nnz; call with NULL
 * arrays first to size them. */
int gf_batch_assemble_csr(gf_batch* batch, int s, int* row_ptr, int* col_idx, double* val, double* PA, int* dims);

/* Runs `steps` complete solves of the batch (each: reset to the initial
 * configuration, then run to the end) back to back and returns their total
 * device time in milliseconds through *ms (CUDA events on the batch's
 * stream). */
int gf_batch_solve_timed(gf_batch* batch, int steps, double* ms);
/* One reset + run without graph capture, with CUDA events around every
 * kernel; per kernel class k (0 <= k < GF_N_KERNELS, names from
 * gf_kernel_name) *ms_out[k] receives the summed device time and
 * launches_out[k] the launch count. */
enum { GF_N_KERNELS = 18 };
int gf_batch_profile(gf_batch* batch, double* ms_out, long long* launches_out);
const char* gf_kernel_name(int k);
/* Bytes the batch moved host->device when it was created, and bytes
 * gf_batch_results moves device->host. */
int gf_batch_bytes(const gf_batch* batch, long long* h2d, long long* d2h);
/* Algorithmic work of the last run: per-structure Newton passes summed into
 * the factor/solve flop count 2 n kl ku + 2 n (kl + ku) and the assembly
 * bytes 8 [6 N_nodes + 80 N_e + 35 n + n] per pass (nodal state, element
 * constants and history, band and right-hand side); mount_flops counts 9000
 * FP64 flops per Beam_1 element mount. */
int gf_batch_work(const gf_batch* batch, double* lu_flops, double* asm_bytes, double* mount_flops);
/* Host wall time in ms: ms[0] model work of gf_batch_create (checks,
 * numbering, PreCalc, colouring, chain tables), ms[1] its device
 * allocations, ms[2] its host->device uploads, ms[3] CUDA-graph capture and
 * instantiation in the first gf_batch_run, ms[4] the last gf_batch_results.
 * Writes min(n, 5) values. */
int gf_batch_host_ms(const gf_batch* batch, double* ms, int n);
/* Measured FP64 and FP32 FMA throughput of the device (TFLOP/s). */
int gf_device_fp_peaks(gf_ctx* ctx, double* fp64_tflops, double* fp32_tflops);

/* Convenience: create, run, fetch results and destroy. */
int gf_solve(gf_ctx* ctx, int n, const gf_model_desc* models, const gf_solve_opts* opts,
             double* const* final_nodes, gf_stats* stats);

/* n independent Beam_1 elements: PreCalc from nodal coordinates (n x 9),
 * material (n x 3: E, nu, rho), section (n x 6: A, I11, I22, I12, It, I33)
 * and CS (n x 6: E1, E3); n_hist committed increments per element
 * (n x n_hist x 18) build the Gauss-point history; then Mount at disp
 * (n x 18).  K: n x 324 (column-major 18x18), f: n x 18 (P_loading). */
int gf_beam_elements(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* sec,
                     const double* cs, int n_hist, const double* hist_disp, const double* disp, double* K,
                     double* f);

/* n independent Shell_1 elements (replaces Shell_1::PreCalc + SaveLagrange +
 * Mount + MountElementLoads + MountShellSpecialLoads, reference
 * src/Shell_1.cpp:1666-2365, 1650-1664, 899-1332, 1384-1467; homogeneous
 * section, Hooke material): PreCalc from the six nodal coordinates (n x 18),
 * material (n x 3: E, nu, rho) and thickness (n); n_hist committed
 * increments per element (n x n_hist x 27, element DOF order: translations
 * of nodes 1..6, then rotations of nodes 4..6) build the Gauss-point
 * history; then Mount at disp (n x 27).  pressure (n, may be NULL; NaN =
 * none) adds the follower pressure at the displaced configuration (history
 * plus disp) with the reference's AreaUpdate flag area_update.  K: n x 729
 * (column-major 27x27), f: n x 27 (P_loading). */
int gf_shell_elements(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* thick, int n_hist,
                      const double* hist_disp, const double* disp, const double* pressure, int area_update, double* K,
                      double* f);

/* Inertial contributions of n independent Beam_1 elements (replaces
 * Beam_1::MountMass, reference src/Beam_1.cpp:1564-1638, for Hooke
 * sections): geometry, history and increments as gf_beam_elements, plus the
 * converged nodal velocities and accelerations (n x 18 each) and the Newmark
 * step (dt, beta, gamma; reference src/Dynamic.cpp:582-590).  M: n x 324
 * mass/gyroscopic tangent (column-major), F: n x 18 inertial force. */
int gf_beam_inertia_elements(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* sec,
                             const double* cs, int n_hist, const double* hist_disp, const double* disp,
                             const double* vel, const double* acc, double dt, double beta, double gamma,
                             double* M, double* F);

/* Inertial contributions of n independent Shell_1 elements (replaces
 * Shell_1::MountMass, reference src/Shell_1.cpp:2406-2498): geometry,
 * material, thickness, history and increments as gf_shell_elements, plus the
 * converged nodal velocities and accelerations of the six nodes (n x 36
 * each, six per node, global frame) and the Newmark step (dt, beta, gamma;
 * reference src/Dynamic.cpp:582-590).  M: n x 729 mass/gyroscopic tangent
 * (column-major), F: n x 27 inertial force. */
int gf_shell_inertia_elements(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* thick,
                              int n_hist, const double* hist_disp, const double* disp, const double* vel,
                              const double* acc, double dt, double beta, double gamma, double* M, double* F);

/* Solves A x = b for a banded matrix given in the reference's BandMatrix
 * storage (LAPACK GB: entry (i,j) at ab[(kl+ku+i-j) + j*ldab], ldab >=
 * 2*kl+ku+1), without pivoting, FP64.  kl, ku <= 17 run on the 35-row band
 * solver; wider bands on the blocked wide-band LU with half-bandwidth
 * max(kl, ku).  b is overwritten by x.  *info receives 0 or 1 (zero or
 * non-finite pivot), as bandsystem's info_fail. */
int gf_band_solve(gf_ctx* ctx, int n, int kl, int ku, const double* ab, int ldab, double* b, int* info);

/* Replaces sparsesystem (src/SparseMatrix.cpp:74-166, the Newton step's
 * solve) for one system K x = b, K in SparseMatrix's layout: Eigen
 * row-major CSR, 0-based (row_ptr[n+1], col_idx[nnz], val[nnz]; entries
 * repeated within a row are summed).  The unknowns are ordered by the
 * narrower of their natural order and reverse Cuthill-McKee on the
 * symmetrised pattern; the factorization is the no-pivot banded LU of
 * gf_band_solve on the GPU, FP64.  b (n) is overwritten by x.  *info
 * receives 0 or 1 (zero or non-finite pivot), as sparsesystem's info_fail;
 * the return value reports argument and CUDA errors. */
int gf_sparse_solve(gf_ctx* ctx, int n, const int* row_ptr, const int* col_idx, const double* val, double* b,
                    int* info);

/* Device bytes a batch of these n structures holds (gf_batch_create's
 * allocations, each rounded to 256 bytes); checks the descriptions as
 * gf_batch_create does.  Needs no device; ctx may be NULL. */
int gf_batch_device_bytes(gf_ctx* ctx, int n, const gf_model_desc* models, size_t* bytes);

/* ---- Served path: continuous batching under a device-memory budget ----
 * No counterpart in the reference, which solves one input deck per process.
 * A server owns one device allocation of hbm_budget bytes.  Submitted
 * structures queue until there is room; each admission takes every queued
 * structure that fits (first come, first served, up to max_wave_structs) into
 * a new device batch, a "wave", on its own stream, so waves admitted while
 * others run overlap on the device.  Every structure keeps its state on the
 * device for all its load steps; its result is reported as soon as it
 * finishes, and its wave's memory returns to the budget when the wave's last
 * structure finishes.  Results equal those of gf_solve on the structure
 * alone.  All progress happens inside gf_server_poll; calls on one server
 * must not overlap. */
typedef struct gf_server gf_server;

typedef struct gf_server_opts {
  size_t hbm_budget;     /* bytes of device memory for structures */
  int max_waves;         /* batches in flight at once (each its own stream) */
  int max_wave_structs;  /* structures per batch */
  int passes_per_chunk;  /* Newton passes enqueued between two state reads */
  int max_wave_passes;   /* Newton passes after which a wave's unfinished
                            structures are reported with GF_ERR_TIMEOUT
                            (0: the default of 4,000,000) */
  int precision;         /* the waves' gf_solve_opts.precision: GF_PREC_FP64
                            (default) or GF_PREC_MIXED */
} gf_server_opts;

typedef struct gf_server_result {
  long long tag;             /* as given to gf_server_submit */
  int status;                /* GF_OK, or GF_ERR_TIMEOUT / GF_ERR_CUDA */
  int pad;
  gf_stats stats;
  double queued_ms;          /* submit -> admission */
  double total_ms;           /* submit -> result reported */
} gf_server_result;

typedef struct gf_server_status {
  int queued;                /* submitted, not admitted */
  int waves;                 /* batches on the device */
  int structures;            /* admitted, not yet reported */
  int pad;
  size_t budget_in_use;      /* bytes of the budget held by waves */
  long long passes;          /* Newton passes launched so far */
  long long launches;        /* kernels launched so far */
  long long reported;        /* results reported so far */
} gf_server_status;

void gf_server_default_opts(gf_server_opts* opts);
gf_server* gf_server_create(gf_ctx* ctx, const gf_server_opts* opts);
void gf_server_destroy(gf_server* srv);
/* Queues one structure.  The arrays model points to and final_nodes
 * (n_nodes x 15 doubles, as gf_batch_results) must stay valid until its
 * result is reported.  GF_ERR_ARG if the model is invalid or needs more than
 * the whole budget. */
int gf_server_submit(gf_server* srv, const gf_model_desc* model, double* final_nodes, long long tag);
/* Reads finished work, retires finished waves, admits queued structures and
 * keeps two chunks of passes in flight per wave; returns at once.  Up to
 * max_results finished structures go to results (*n_results of them); the
 * rest wait for the next call. */
int gf_server_poll(gf_server* srv, gf_server_result* results, int max_results, int* n_results);
int gf_server_get_status(const gf_server* srv, gf_server_status* status);

/* No counterpart in the reference.  The same solve as gf_band_solve for
 * narrow bands (kl, ku <= GF_KB = 17, the bands of Beam_1 chains and
 * frames), same arguments and results, for callers that must not allocate
 * device memory per call: a host loop that runs under another allocator's
 * budget, or one that cannot afford cudaMalloc/cudaFree, which synchronise
 * the whole device.  Work arrays live in one static device array per device
 * sized for GF_NOALLOC_MAX_N unknowns (about 7 MB); no cudaMalloc, cudaFree
 * or other allocating routine is called.  n > GF_NOALLOC_MAX_N, kl > 17 or
 * ku > 17 return GF_ERR_ARG (use gf_band_solve).  The first call on each device looks up the array's
 * address (cudaGetSymbolAddress); make that first call before any stream
 * capture.  Every context on a device shares the array: overlapping calls on
 * one device, from two threads or two contexts, race. */
enum { GF_NOALLOC_MAX_N = 16384, GF_NOALLOC_MAX_KB = 17 };
int gf_band_solve_noalloc(gf_ctx* ctx, int n, int kl, int ku, const double* ab, int ldab, double* b, int* info);

/* ---- Newton-iteration boundary ----
 * A device-resident structure driven by the caller's own Static::Solve /
 * Dynamic::Solve loop, one call per stage of an iteration, in the order of
 * reference src/Static.cpp:176-298:
 *
 *   gf_begin_step(t_last, dt)   Zeros + MountDisplacements (+ the Newmark
 *                               predictor of a Dynamic step)
 *   loop: gf_assemble           Clear + MountLocal + MountElementLoads +
 *                               MountLoads + MountGlobal + P_A = -P_A +
 *                               MountSparse (src/Static.cpp:206-216)
 *         (the caller's criteria and sparsesystem / gf_sparse_solve)
 *         gf_set_increment(x)   UpdateDisps (src/Solution.cpp:390-423; Dynamic:
 *                               UpdateDyn, src/Dynamic.cpp:480-580)
 *   gf_commit                   SaveConfiguration (src/Solution.cpp:426-500)
 *   or gf_rollback              RestoreConfiguration (src/Solution.cpp:502-575)
 *
 * Every vector is in the reference's free-DOF numbering (SetGlobalDOFs,
 * src/Solution.cpp:40-118: node by node, DOF by DOF, fixed and inactive DOFs
 * skipped); gf_structure_dofs gives node * 6 + DOF of each free index.  The
 * structure's nodal configuration and Gauss-point histories stay on the
 * device between calls. */
typedef struct gf_structure gf_structure;
enum { GF_LAYOUT_CSR = 0, GF_LAYOUT_GB = 1 };

/* Uploads one structure (its first solution step's parameters; see
 * gf_structure_set_step), numbers its DOFs and runs the elements' PreCalc:
 * replaces DOFsActive + SetGlobalDOFs + SetGlobalSize (src/Solution.cpp:
 * 40-224, 577-654).  NULL on failure (gf_last_error). */
gf_structure* gf_upload_structure(gf_ctx* ctx, const gf_model_desc* model, const gf_solve_opts* opts);
void gf_structure_destroy(gf_structure* s);
/* dims[0] free DOFs n, dims[1] nonzeros of K_AA's CSR pattern, dims[2] its
 * half-bandwidth kb (GB storage has ldab = 3 kb + 1), dims[3] nodes. */
int gf_structure_dims(const gf_structure* s, int* dims);
/* dof_node[i] = node * 6 + DOF (0-based) of free index i. */
int gf_structure_dofs(const gf_structure* s, int* dof_node);
/* K_AA's CSR pattern (SparseMatrix::m_matrix: row-major, 0-based, the union
 * of the element patterns, zeros kept): row_ptr (n + 1), col_idx (nnz). */
int gf_structure_pattern(const gf_structure* s, int* row_ptr, int* col_idx);
/* Makes solution step k of the description (0: `solution`, k > 0:
 * next_steps[k - 1]) the current one (src/main.cpp:52-60). */
int gf_structure_set_step(gf_structure* s, int k);
/* Starts a load / time step at last_converged_time + time_step. */
int gf_begin_step(gf_structure* s, double last_converged_time, double time_step);
/* Assembles at the current iterate: K (CSR values in gf_structure_pattern's
 * order, nnz doubles, or GB storage, ldab x n doubles, ldab = 3 kb + 1, per
 * layout; may be NULL) and P_A (n, after the sign flip: f_ext - f_int; may be
 * NULL). */
int gf_assemble(gf_structure* s, int layout, double* K, double* P_A);
/* Adds the Newton increment x (n) to the nodal displacements. */
int gf_set_increment(gf_structure* s, const double* x);
int gf_commit(gf_structure* s);
int gf_rollback(gf_structure* s);
/* Current state: nodes (n_nodes x 15: the committed copy_coordinates, then
 * the nodal rotation tensor row-major) and increments (n_nodes x 6, the
 * step's Node::displacements); either may be NULL. */
int gf_structure_nodes(gf_structure* s, double* nodes, double* increments);

/* ---- Monitor ----
 * gf_batch_monitor returns structure s's monitor lines after a run: for
 * each of its monitor_nodes, the lines Node::WriteMonitor writes (reference
 * src/Node.cpp:227-320; src/Monitor.cpp:384-401 calls it at the first
 * solution step's start, after every monitor_sample-th converged step of a
 * solution step and at a step's end): 31 columns TIME, X Y Z (position),
 * ROTX ROTY ROTZ (Euler rotation vector), FX FY FZ MX MY MZ (the elements'
 * internal force at a free DOF, the reaction at a constrained one; moments
 * from the pseudo-moments), the same six as the local columns (equal in the
 * spatial description), the velocities and the accelerations.  out is
 * [node][line][31] (NULL: dims only); dims[0] monitored nodes, dims[1]
 * lines returned, dims[2] lines the run produced (more than dims[1] when
 * gf_solve_opts.monitor_rows ran out).  A NodalLoad acting on a constrained
 * DOF is not added to its reaction column. */
int gf_batch_monitor(gf_batch* b, int s, double* out, int* dims);

/* The wide-band LU tile shapes the batch runs with (gf_solve_opts.wide_tiles
 * order; all 0 for a batch without Shell_1 structures). */
int gf_batch_wide_tiles(const gf_batch* b, int* tiles);

/* ---- Modal analysis ----
 * gf_structure_modal replaces Modal::Solve (src/Modal.cpp:131-199) with its
 * eigen solve sparseeigen (src/SparseMatrix.cpp:270-420, ARPACK shift-invert
 * with shift 0): the n_modes smallest eigenvalues of K_AA x = lambda M_AA x,
 * K_AA the static tangent of the structure's current configuration with the
 * loads at `time` (MountLocal + MountElementLoads + MountLoads) and M_AA the
 * modal mass (MountMassModal).  Subspace iteration on K^-1 M with the
 * wide-band factor of K on the device, until the n_modes smallest Ritz values
 * change by at most tol relative (tol <= 0: 1e-12); at most 300 iterations
 * (ARPACK's iparam[2] in the reference), else GF_ERR_TIMEOUT.  eig receives
 * the n_modes eigenvalues ascending (real: the reference's Im column is 0 for
 * these symmetric problems); modes (may be NULL) the M-orthonormal modes,
 * n_modes x n free DOFs in the reference's numbering; iterations (may be
 * NULL) the iterations taken.  A nonsymmetric K_AA (follower loads) is
 * refused with GF_ERR_ARG, a singular one with GF_ERR_SINGULAR.  gf_modal is
 * the Modal step of a structure at its start (solution.start_time). */
int gf_structure_modal(gf_structure* s, double time, int n_modes, double tol, double* eig, double* modes,
                       int* iterations);
int gf_modal(gf_ctx* ctx, const gf_model_desc* model, int n_modes, double tol, double* eig, double* modes,
             int* iterations);

/* ---- Element entries on the reference's stored Gauss-point state ----
 * gf_beam_mount replaces Beam_1::Mount + MountElementLoads
 * (src/Beam_1.cpp:695-843) for n elements; their state is given as the
 * reference's LagrangeSave holds it (src/LagrangeSave.h:11-17), per element
 * and Gauss point GF_BEAM_LAG doubles: Q_i (3x3 column-major, as Matrix
 * stores it), alpha_i, kappa_i_ref, u_i, dz_i (3 each; LagrangeSave's
 * d_alpha_i and theta_i are not read by Mount or SaveLagrange).  Geometry,
 * material, section and CS as gf_beam_elements (no pre-tension); disp
 * (n x 18) are the nodes' Node::displacements.  gf_beam_save_lagrange
 * replaces Beam_1::SaveLagrange (src/Beam_1.cpp:1494-1506): it updates lag
 * in place.  The state of a new element is Q_i = I, dz_i = (0, 0, 1), the
 * rest zero (src/LagrangeSave.cpp). */
enum { GF_BEAM_LAG = 21, GF_SHELL_LAG = 27 };
int gf_beam_mount(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* sec, const double* cs,
                  const double* lag, const double* disp, double* K, double* f);
int gf_beam_save_lagrange(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* sec,
                          const double* cs, double* lag, const double* disp);
/* The same for Shell_1 (Shell_1::Mount + MountElementLoads +
 * MountShellSpecialLoads, src/Shell_1.cpp:899-1467; SaveLagrange, 1650-1664):
 * per element and Gauss point GF_SHELL_LAG doubles of Shell_1's own state
 * (src/Shell_1.h:117-127): Q_i (3x3 column-major), u_i, alpha_i, kappa_r1_i,
 * kappa_r2_i, z_x1_i, z_x2_i (3 each); a new element has Q_i = I,
 * z_x1_i = (1, 0, 0), z_x2_i = (0, 1, 0), the rest zero.  With a follower
 * pressure (pressure[n], NULL for none), cur_xyz (n x 18) gives the six nodes'
 * current positions (copy_coordinates) before this iteration's increments. */
int gf_shell_mount(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* thick, const double* lag,
                   const double* disp, const double* cur_xyz, const double* pressure, int area_update, double* K,
                   double* f);
int gf_shell_save_lagrange(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* thick, double* lag,
                           const double* disp);

#ifdef __cplusplus
}
#endif
#endif
