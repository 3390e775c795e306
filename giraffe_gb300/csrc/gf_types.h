// Device data layout of a batch of structures (shared by host and device
// code).  A batch holds many independent structures; nodes, elements and free
// DOFs of each structure are contiguous ranges of the batch-wide arrays.
//
// HBM layout (all structure-of-arrays over the batch):
//   nodes     disp[6], copy[6] (position + accumulated Rodrigues vector),
//             Qn[9], gl[6] (local free index or -1), node_struct
//   elements  enodes[3], estruct, BeamConst (PreCalc constants of Beam_1 or
//             of a Pipe_1 from its PipeSection),
//             BeamHist (Gauss-point history read by Mount), BeamHistAux
//             (u_i, alpha_i written at commit)
//   DOFs      dof_node6 (node*6 + k of each free DOF), P (residual, then the
//             Newton increment), y (forward-substituted right-hand side)
//   band      per structure, column-major with GF_LDB = 2*GF_KB+1 rows:
//             entry (i, j) of K_AA at band[(GF_KB + i - j) + j*GF_LDB]
//             (the reference's BandMatrix GB layout without the kl fill rows,
//             reference src/BandMatrix.cpp:214,246), FP64 and an FP32 copy
//   factor    U rows: n_free x (GF_KB+1), [j][c] = U(j, j+c)
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#define GF_KB 17
#define GF_LDB (2 * GF_KB + 1)
#define GF_UW (GF_KB + 1)
#define GF_WB_STREAMS 5  // helper streams of the wide-band lookahead
#define GF_WB_EVENTS 6

namespace gf {

struct BeamConst {
  double T3[9];
  double Dd[6];
  double D34;
  double e3r[3];
  double jac;
  double N[2][3];
  double dN[2][3];
  double Mr;
  double Jr[9];
};

struct BeamHist {
  double Q[2][9];
  double dz[2][3];
  double kap[2][3];
};

struct BeamHistAux {
  double u[2][3];
  double alpha[2][3];
};

// Shell_1 PreCalc constants (reference src/Shell_1.cpp:1666-2365): local
// frame rows e1r, e2r, e3r; Lame constants and drilling stiffness; shape
// functions at the three midside Gauss points (translations Nu of the six
// nodes, rotations Na of the three midside nodes, with x1 / x2 derivatives);
// the six-point surface rule (weights w4, translation shape functions and
// derivatives) used by the follower pressure.
struct ShellConst {
  double T3[9];
  double mu, lambda, stiff_drill, thick, alpha1;
  double coef1, coef2, coef3;  // fibre mass per area, its rotary inertia, drilling inertia (modal mass)
  double Nu[3][6], Nu1[3][6], Nu2[3][6];
  double Na[3][3], Na1[3][3], Na2[3][3];
  double w4[6];
  double N4[6][6], N41[6][6], N42[6][6];
  double Na4[6][3];  // midside rotation shape functions at the six points
};

// Shell_1 Gauss-point history read by Mount: Q_i, kappa_r1_i, kappa_r2_i,
// z_x1_i, z_x2_i (reference src/Shell_1.cpp:1650-1664).
struct ShellHist {
  double Q[3][9];
  double k1[3][3], k2[3][3];
  double z1[3][3], z2[3][3];
};

// Written at commit only: u_i and alpha_i.
struct ShellHistAux {
  double u[3][3];
  double alpha[3][3];
};

// Wide-band LU panel width (columns per panel).
#define GF_WB_NB 64
#define GF_IR_MAX 30  // default FP64 refinement sweeps of the FP32 wide-band factor before the FP64 fallback

enum Phase : int { PH_START = 0, PH_ITER = 1, PH_DONE = 2, PH_ABORTED = 3 };

// Per-structure parameters (Static solution step + ConvergenceCriteria).
struct StructParams {
  double start_time, end_time, time_step0, max_time_step, min_time_step, inc_factor;
  int max_it, min_it, conv_increase, dynamic;  // dynamic: Newmark step (Dynamic::Solve)
  double beta, gamma;  // Newmark parameters
  double force_tol, moment_tol, force_min, moment_min, disp_tol, rot_tol, disp_min, rot_min,
      divergence_ref;
  // Rayleigh damping of a Dynamic step (Beam_1::MountDamping): C_e = alpha
  // M_modal + beta K_e, formed at the first Newton iteration of the step
  // (or at every iteration with ray_update)
  double ray_alpha, ray_beta;
  int ray_on, ray_update;
  // the step starts from zero nodal velocities and accelerations: a Static
  // step (Solution::ZerosVelAccel) or a Dynamic one with ZeroIC
  int zero_va;
  int pad_p;
};

// Per-structure ranges in the batch arrays.
struct StructInfo {
  int node_off, n_nodes;
  int elem_off, n_elem;
  int dof_off, n_free;
  int64_t band_off;  // in entries; band of n_free columns x GF_LDB
  int has_force, has_moment;  // free translational / rotational DOFs exist
  int load_off, n_loads;  // nodal load entries of this structure
  int is_chain;  // solved by the chain solver (else by the band LU)
  // wide-band structures (Shell_1): K_AA column-major with 2 wkl + 1 rows,
  // entry (i, j) at wband[wb_off + (wkl + i - j) + j (2 wkl + 1)]; the free
  // DOFs are numbered in reverse Cuthill-McKee node order
  int wide;
  int wkl;
  int n_panels;  // ceil(n_free / GF_WB_NB)
  int pad_w;
  // solution steps: Batch::step_params[step_off .. step_off + n_steps)
  int step_off, n_steps;
  int64_t wb_off;    // into ShellData::wband
  // monitored nodes (a deck's Monitor block): Batch::mon_* entries
  // [mon_off, mon_off + mon_n), a line after every mon_sample-th converged
  // step of a solution step and at its end
  int mon_off, mon_n, mon_sample, pad_m;
};

// Per-structure Newton / load-step control state (reference
// src/Static.cpp:140-311 as a state machine).
// DOFs per CTA of the residual and update reductions (k_residual,
// k_update): a structure's free DOFs are split into chunks of this size,
// at least one per structure.
#define GF_RED_CHUNK 2048

// Per-structure partial results of those reductions across their CTAs:
// maxima of non-negative values as the bit patterns of the doubles (which
// order as unsigned integers), the NaN flag, and the count of CTAs done.
struct RedScratch {
  unsigned long long a, b, va, vb;
  int f, ticket;
};

struct StructState {
  int phase;
  int it;
  int res_conv, gl_conv, diverged, aborted, need_solve, info_fail;
  int convergence_counter, converged_number, n_conv_evaluated, total_it, bisections;
  int commit;  // set by control for the commit kernel
  int n_solves;  // linear solves performed
  int ray_init;       // Rayleigh matrices formed (after the step's first iteration)
  int step;           // current solution step of the structure
  int zero_va;        // zero the nodal velocities / accelerations before the next time step
  int conv_in_step;   // steps converged in the current solution step (the monitor's sample count)
  int mon_rows;       // monitor lines recorded so far
  int mon_now;        // this pass committed a step that the monitor records
  int commit_dyn;     // the committed step's solution step was Dynamic (its velocities are saved)
  int host_step;      // the caller's step control set last_converged_time and
                      // current_time_step (gf_begin_step): step_begin keeps them
  int ir_sweeps;      // FP64 refinement sweeps of the FP32 wide-band factor (all solves)
  int ir_fallbacks;   // solves that refinement did not finish: refactored in FP64
  int ir_fb;          // this solve takes the FP64 fallback
  double time, time_step, last_converged_time, current_time_step;
  double force_crit, moment_crit, disp_crit, rot_crit;
  double last_res, last_inc;
  double a[6];  // Newmark coefficients of the current step
};

// One nodal load entry (one node of a NodalLoad node set).
struct LoadEntry {
  int structure;
  int node;  // batch-wide node index
  int table;  // index into the table arrays
  int pad;
  double CQ[9];  // coordinate system rows (E1, E2, E3)
  double mult[6];
};

// One prescribed-displacement node (one node of a NodalDisplacement set).
struct DispEntry {
  int structure;
  int node;
  int table;
  int angular;  // GF_ANGLES_EULER or GF_ANGLES_VECTOR
  double CQ[9];
};

struct TableDev {
  int n_times, n_cols;
  int64_t off;  // into the batch's table storage: times then values
};

// Chain solver data (see gf_chain.cuh).
#define CR_MAX_LEVELS 24

// One cyclic-reduction item: a corner position with its neighbours at the
// item's level (-1 when absent).
struct CrItem {
  int corner;  // batch-wide corner index
  int prev;
  int next;
  int structure;
};

struct ChainData {
  int n_chain_elems;   // elements of chain structures
  int n_corners;       // free corners of chain structures
  int n_levels;
  int* elem_list;      // batch element ids of chain elements
  int* elem_corner_a;  // corner index of the element's first corner (-1 if fixed)
  int* elem_corner_b;  // corner index of the element's last corner (-1 if fixed)
  int* corner_node;    // batch node id of each free corner
  int* corner_struct;
  int* corner_left;    // chain element to the left (-1 if none)
  int* corner_right;   // chain element to the right (-1 if none)
  int* corner_prev;    // previous free corner of the same chain (-1 if none)
  int* corner_next;    // next free corner (-1 if none)
  // scratch below is structure-of-arrays: entry x of item i at [x * n_items + i]
  double* ez;          // [6*13][chain elem]  Z_s = A_ss^{-1}[b_s | A_sa | A_sb]
  double* ec;          // [6*26][chain elem]  -A_as Z_s (13 cols), -A_bs Z_s (13 cols)
  double* cD;          // [36][corner] (row-major 6x6 per corner)
  double* cL;          // [36][corner]
  double* cU;          // [36][corner]
  double* cb;          // [6][corner]
  double* cz;          // [6*13][corner]  Z = D^{-1}[b | L | U] of an eliminated corner
  double* cx;          // [6][corner]  solution
  CrItem* odd;         // per level: eliminated positions
  int odd_off[CR_MAX_LEVELS + 1];
  CrItem* even;        // per level: surviving positions with at least one eliminated neighbour
  int even_off[CR_MAX_LEVELS + 1];
  int* roots;          // per chain structure: the corner left after all levels
  int n_roots;
};

// Shell_1 elements and the wide-band storage of their structures.
// Tile shapes of the wide-band LU that leave every entry's arithmetic as it
// is (so any choice gives the same bits): rows per CTA of the bulk trsm (4,
// 8 or 16) and of the first trsm on the critical path (1, 2 or 4), the
// output tile edge of the corner update (4 or 8), rows per CTA of the
// triangular solves (32 or 64).  Picked by timing (the autotuner) or pinned
// by the caller.
struct WideTiles {
  int trsm_rb = 8;
  int trsm_first = 2;
  int corner = 8;
  int sub_rows = 64;
};

// Refinement state of one wide structure slot (mixed precision): the
// largest |correction| and |x| of the current sweep (FP64 bits, raised by
// atomicMax), the previous sweep's |correction|, sweeps of this solve.
struct WideIr {
  unsigned long long dn, xn;
  double dprev;
  int k, done;
};

struct ShellData {
  int n_shells;
  int n_wide;       // structures solved by the wide-band LU
  int max_panels;   // over those structures
  int max_kl;       // over those structures
  int* wide_structs;  // [n_wide] structure indices
  int* snodes;      // [n_shells][6] batch node ids
  int* sstruct;
  int* spress;      // table index of the follower pressure on the element, or -1
  int* sarea;       // AreaUpdate flag of that pressure
  ShellConst* sconst;
  ShellHist* shist;
  ShellHistAux* saux;
  double* Ke;       // [n_shells][27 x 27] column-major (global frame)
  double* Fe;       // [n_shells][27]
  // Rayleigh damping matrix per element (27x27 column-major,
  // structure-of-arrays: entry x of element e at [x * n_shells + e]);
  // allocated when any_rayleigh
  double* RD;
  int any_rayleigh;
  int* color_elems;
  int color_off[17];
  int n_colors;
  double* wband;
  // mixed precision (GF_PREC_MIXED): K_AA stays in wband (FP64) for the
  // residuals; its LU is formed in wband32 (FP32, same geometry) and the
  // solution refined in FP64: r32 / y32 the FP32 right-hand side and the
  // forward-substitution scratch, ir_rhs the Newton right-hand side, ir the
  // per-slot refinement state.  fp64_pass is set on the host's copy of the
  // batch for the FP64 fallback launches (only structures with ir_fb run).
  float* wband32;
  float* r32;
  float* y32;
  double* ir_rhs;
  struct WideIr* ir;
  WideTiles tiles;   // tile shapes of this batch's wide-band LU
  int* ir_more;      // [0] a slot still refines, [1] a slot needs the FP64 fallback,
                     // [2] sweeps run, [3] fallbacks run (both cumulative)
  int fp64_pass;
  int ir_max;        // refinement sweeps before the FP64 fallback
  int* panel;       // device panel counter of the captured panel loops
  int loops_in_graph;  // capture the panel loops as graph WHILE loops (served waves)
  int wide_tc;         // trailing update: 0 FP64 FMA, 1 tcgen05 Ozaki slices, 2 mma.sync Ozaki slices
  // the tensor-core update's slices of a panel: per wide structure slot,
  // [2 operands][8 slices][oz_rows][64] bf16 and [2][oz_rows] exponents;
  // every 128-byte row of 64 slices is stored with its eight 16-byte chunks
  // permuted (chunk c at c ^ (row & 7)), the 128-byte swizzle of the tensor
  // cores' shared-memory operands, so a tile of rows is one bulk copy
  int oz_rows;         // max_kl rounded up to 128
  __nv_bfloat16* oz_slices;
  int* oz_exp;
  // per wide structure slot, [2 panel parities][2 operands][64]: the
  // magnitude bits of the largest entry of each column k of a panel's L21
  // and of each row k of its U12 (zeroed by the panel's diagonal LU, raised
  // by its trsm), from which the slicing balances k by a power of two
  unsigned long long* oz_kmax;
  // nonzero when a bounded wait of the tensor-core update gave up (its
  // structures are then reported as failed solves)
  int* oz_error;
  // host handles of the wide-band lookahead: helper streams and the events
  // that fork from and join into the pass's stream; aux[2] roots the
  // captured panel-loop bodies, aux[3] runs the bulk trsm beside the first
  // blocks and the corner update, aux[4] roots the captured bodies of the
  // refinement loop and of the FP64 fallback
  cudaStream_t aux[GF_WB_STREAMS];
  // [0] panel start, [1] after trsm, [2] after the corner update, [3] after
  // diag, [4] end of forward, [5] after the bulk trsm
  cudaEvent_t evt[GF_WB_EVENTS];
};

// Device pointers of a batch.
struct Batch {
  int n_struct, n_nodes, n_elem, n_free;
  int n_loads, n_disps, n_tables;
  // nodes
  double* disp;
  double* copy;
  double* xref;        // reference positions (initial copy: 6 per node)
  double* Qn;
  double* vel;         // Newmark velocities (dynamic structures)
  double* accel;
  double* copy_vel;    // converged velocities / accelerations
  double* copy_accel;
  int* gl;
  int* cons;
  int* node_struct;
  // elements
  int* enodes;
  int* estruct;
  BeamConst* bconst;
  BeamHist* bhist;
  BeamHistAux* baux;
  int* color_elems;  // elements grouped by colour
  int color_off[9];  // colour c = color_elems[color_off[c] .. color_off[c+1])
  int n_colors;
  // DOFs
  int* dof_node6;
  double* P;
  double* y;
  int64_t rhs_ld;  // column stride of a multi-column wide-band substitution (0: one column)
  // band and factor
  double* Ke;  // per-element tangent scratch (18x18 column-major)
  double* Fe;  // per-element internal force scratch
  double* band;
  double* U;
  float* U32;
  // structures
  StructInfo* info;
  StructParams* params;       // the current solution step's parameters
  StructParams* step_params;  // every solution step of every structure
  StructState* state;
  // PipeLoad internal pressures: one entry per pressurized Pipe_1 element
  // (batch element index, table of P0I P0E RhoI RhoE, internal area)
  int n_pipe_press;
  int* pp_elem;
  int* pp_table;
  double* pp_aint;
  // monitored nodes: batch node, structure, element incidences
  // mon_adj[mon_adj_off[q] .. mon_adj_off[q + 1]) (x: element, y: 64 * kind
  // + the node's place in it; kind 0 Beam_1 / Pipe_1, 1 Shell_1), the load
  // each keeps between lines (Node::load) and the lines, [q][mon_cap][25]:
  // time, copy_coordinates (6), load (6), copy_vel (6), copy_accel (6)
  int mon_total, mon_cap;
  int* mon_node;
  int* mon_struct;
  int* mon_adj_off;
  int2* mon_adj;
  double* mon_load;
  double* mon_rec;
  // loads
  LoadEntry* loads;
  DispEntry* disps;
  TableDev* tables;
  double* table_data;
  // chain structures: the nodal load stiffness (rotation block, row-major
  // 3x3 per node); their solver reads K from the element tangents and this,
  // so their band is neither cleared nor filled -- unless full_band (the
  // assembly view of gf_batch_assemble), which fills the band for every
  // structure
  double* nodeK;
  int full_band;
  int mixed;  // 1: Beam_1 tangent operator in FP32-pair arithmetic
  int* running;  // structures still running after the last pass
  // Rayleigh damping matrix per element (18x18, structure-of-arrays: entry
  // x of element e at [x * n_elem + e]); allocated when any_rayleigh
  double* RD;
  int any_rayleigh;
  int any_dynamic;  // a structure has a Dynamic solution step
  // inertial rotational tangents of the Beam_1 Gauss points (2 x 9 per
  // element, structure-of-arrays like Ke); allocated when any_dynamic
  double* Dm;
  // reduction chunks: chunk k covers free DOFs [chunk_start[k],
  // chunk_start[k] + GF_RED_CHUNK) of structure chunk_struct[k]
  int n_chunks;
  int* chunk_struct;
  int* chunk_start;
  RedScratch* red;  // [n_struct], zero between kernels
  ChainData chain;
  ShellData sh;
};

}  // namespace gf
