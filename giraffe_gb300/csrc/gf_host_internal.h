// Internal host types of libgiraffe_gpu.so shared by the batch path
// (gf_host.cu) and the served path (gf_server.cu).  Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/giraffe_gpu.h"
#include "gf_types.h"

struct gf_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // options of the standalone solves (gf_band_solve, gf_sparse_solve):
  // wide_update picks their wide-band trailing update
  int wide_update = GF_WIDE_TENSOR;
  // the autotuner's wide-band tile shapes, per half-bandwidth and update kind
  std::map<long long, gf::WideTiles> tiles;
  // pinned staging of gf_batch_results' read-back (grown on demand, freed
  // with the context)
  void* pin = nullptr;
  size_t pin_bytes = 0;
  // a pinned block of at least n bytes, or nullptr when none can be had
  void* pinned(size_t n) {
    if (n <= pin_bytes) return pin;
    if (pin) cudaFreeHost(pin);
    pin = nullptr;
    pin_bytes = 0;
    if (cudaMallocHost(&pin, n) != cudaSuccess) {
      pin = nullptr;
      return nullptr;
    }
    pin_bytes = n;
    return pin;
  }
};

// First-fit sub-allocator over one allocation (the served path's device
// budget, or its pinned host staging).  Blocks are 256-byte aligned;
// freeing merges neighbours.  Thread-safe: the served path's builder thread
// allocates while the polling thread frees.
struct DevArena {
  char* base = nullptr;
  size_t size = 0;
  std::map<size_t, size_t> free_blocks;  // offset -> bytes
  std::map<size_t, size_t> used;         // offset -> bytes
  size_t in_use = 0;
  mutable std::mutex mu;
  void init(void* p, size_t n) {
    std::lock_guard<std::mutex> g(mu);
    base = static_cast<char*>(p);
    size = n;
    free_blocks.clear();
    used.clear();
    in_use = 0;
    if (n) free_blocks[0] = n;
  }
  void* alloc(size_t n) {
    std::lock_guard<std::mutex> g(mu);
    n = (std::max<size_t>(n, 1) + 255) / 256 * 256;
    for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it) {
      if (it->second < n) continue;
      size_t off = it->first, rest = it->second - n;
      free_blocks.erase(it);
      if (rest) free_blocks[off + n] = rest;
      used[off] = n;
      in_use += n;
      return base + off;
    }
    return nullptr;
  }
  void release(void* p) {
    std::lock_guard<std::mutex> g(mu);
    auto it = used.find(static_cast<size_t>(static_cast<char*>(p) - base));
    if (it == used.end()) return;
    size_t off = it->first, n = it->second;
    used.erase(it);
    in_use -= n;
    auto nx = free_blocks.lower_bound(off);
    if (nx != free_blocks.end() && nx->first == off + n) {
      n += nx->second;
      free_blocks.erase(nx);
    }
    auto pv = free_blocks.lower_bound(off);
    if (pv != free_blocks.begin()) {
      --pv;
      if (pv->first + pv->second == off) {
        pv->second += n;
        return;
      }
    }
    free_blocks[off] = n;
  }
  size_t largest_free() const {
    std::lock_guard<std::mutex> g(mu);
    size_t m = 0;
    for (const auto& f : free_blocks) m = std::max(m, f.second);
    return m;
  }
  size_t bytes_in_use() const {
    std::lock_guard<std::mutex> g(mu);
    return in_use;
  }
};

// Host arrays whose elements are default-initialised (left unset for plain
// types): the batch build writes every element itself, from several threads,
// so the pages are first touched in parallel instead of by one zero fill.
template <typename T> struct DefaultInitAlloc : std::allocator<T> {
  template <typename U> struct rebind { using other = DefaultInitAlloc<U>; };
  DefaultInitAlloc() = default;
  template <typename U> DefaultInitAlloc(const DefaultInitAlloc<U>&) noexcept {}
  template <typename U> void construct(U* p) noexcept { ::new (static_cast<void*>(p)) U; }
  template <typename U, typename... A> void construct(U* p, A&&... a) {
    ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
  }
};
template <typename T> using hvec = std::vector<T, DefaultInitAlloc<T>>;

struct gf_batch {
  gf_ctx* ctx = nullptr;
  gf_solve_opts opts{};
  gf::Batch b{};
  cudaStream_t stream = nullptr;  // the context's stream, or a served wave's own
  DevArena* arena = nullptr;      // served waves: allocations come from the server's budget
  DevArena* host_stage = nullptr; // served waves: pinned staging for the uploads
  std::vector<void*> staged;      // staging blocks in use until the uploads land
  bool count_only = false;        // size the batch without touching the device
  size_t counted_bytes = 0;
  // host copies needed for results and resets
  std::vector<gf::StructInfo> info;
  std::vector<int> kb;  // true half-bandwidth per structure
  std::vector<void*> allocs;
  // initial configuration (device) for gf_batch_reset
  double* copy0 = nullptr;
  double* Qn0 = nullptr;
  gf::BeamHist* bhist0 = nullptr;
  gf::BeamHistAux* baux0 = nullptr;
  gf::ShellHist* shist0 = nullptr;
  gf::ShellHistAux* saux0 = nullptr;
  // wide (Shell_1) structures: the reference's free-DOF index -> the
  // solver's (reverse Cuthill-McKee) index; empty for the others
  std::vector<std::vector<int>> perm;
  // host copies for the CSR view of K_AA (gf_batch_assemble_csr): free index
  // (solver numbering) of every node DOF, element nodes, per-structure shell
  // offsets
  hvec<int> h_gl, h_enodes, h_snodes;
  std::vector<int> shell_off;
  // the monitor's first line of each monitored entry (the first solution
  // step's start: the reference coordinates; loads, rotations, velocities
  // zero): x, y, z and the start time
  std::vector<double> mon_first;
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  long long last_launches = 0;
  int ir_seen[2] = {0, 0};  // refinement sweeps and FP64 fallbacks counted so far (mixed path)
  int launches_per_pass = 0;
  int* h_running = nullptr;  // pinned
  long long h2d_bytes = 0;
  // host wall time (ms) of gf_batch_create, split into model work (checks,
  // numbering, PreCalc, colouring, chain tables), device allocation and
  // host->device uploads; CUDA-graph capture + instantiation of the first
  // gf_batch_run; the last gf_batch_results
  double host_ms[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
};

// A device-resident structure driven one Newton iteration at a time
// (gf_iter.cu) and its modal analysis (gf_modal.cu).
struct gf_structure {
  gf_ctx* ctx = nullptr;
  gf_batch* B = nullptr;
  int nf = 0;            // free DOFs
  int kb = 0;            // half-bandwidth of K_AA in the reference's numbering
  int n_nodes = 0;
  std::vector<int> perm;      // reference free index -> solver index (empty: the same)
  std::vector<int> dof_node;  // reference free index -> node * 6 + DOF
  std::vector<int> rp, ci;    // CSR pattern (reference numbering)
  int64_t* d_src = nullptr;   // per CSR entry: offset into the structure's band, or -1
  double* d_val = nullptr;    // CSR values on the device
  double* d_band = nullptr;   // the structure's band (solver numbering)
  int64_t W = 0, kw = 0;      // band rows and half-bandwidth (solver numbering)
  int iteration = 0;
  bool in_step = false;
  std::vector<double> h_tmp;
};

namespace gfh {
bool set_err(gf_ctx* ctx, const char* fmt, ...);
// Builds the device batch of n structures (or, with B->count_only, only
// counts its device bytes).
int build_batch(gf_batch* B, int n, const gf_model_desc* models);
// Initial configuration and step state, enqueued on B->stream.
int batch_reset(gf_batch* B);
// Captures one Newton pass as a CUDA graph on B->stream (opts.use_graph).
int ensure_graph(gf_batch* B);
// Device bytes of a batch of these structures built with opts (NULL: the
// defaults), without touching the device.
int batch_device_bytes(gf_ctx* ctx, int n, const gf_model_desc* models, const gf_solve_opts* opts, size_t* bytes);
// Kernel launches of one Newton pass.
int count_launches_per_pass(const gf_batch* B);
// The wide-band LU's tile shapes for half-bandwidth kl and trailing-update
// kind wide_update, timed on a synthetic band once per context (gf_tune.cu);
// the defaults when tuning cannot run.
gf::WideTiles tune_wide_tiles(gf_ctx* ctx, int kl, int wide_update);
// Host wall clock in milliseconds.
double host_now_ms();
// Reverse Cuthill-McKee order of a graph given by adjacency lists
// (order[k] = the vertex placed k-th).
std::vector<int> rcm_order(int nn, const std::vector<std::vector<int>>& adj);
// gf_band_solve for half-bandwidths above 17: the blocked wide-band LU on a
// one-structure batch (gf_sparse.cu).
int wide_band_solve(gf_ctx* ctx, int n, int kl, int ku, const double* ab, int ldab, double* b, int* info);
// Host PreCalc of one Beam_1 element (end nodes x0, x2; Hooke material E,
// nu, rho; section A, I11, I22, I12, It, I33; CS rows E1, E3; pre-tension
// T0) into its constants and initial Gauss-point history, and of one Shell_1
// element (six nodes, material, thickness).
void beam_precalc(const double* x0, const double* x2, const double* mat, const double* sec, const double* cs,
                  gf::BeamConst& c, gf::BeamHist& h, gf::BeamHistAux& x, double T0);
void shell_precalc(const double* xyz, const double* mat, double thick, gf::ShellConst& c, gf::ShellHist& h,
                   gf::ShellHistAux& x);
// CSR pattern of structure s's K_AA in the reference's free-DOF numbering
// (sorted columns per row); returns nnz.
int64_t csr_rows(const gf_batch* B, int s, std::vector<std::vector<int>>& rows);
// K_AA of a device-resident structure's current configuration, static, with
// the loads at `time`, into its band (gf_iter.cu).
int structure_static_tangent(gf_structure* S, double time);
}  // namespace gfh

#define GF_CK(call)                                                                          \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      gfh::set_err(ctx, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return GF_ERR_CUDA;                                                                    \
    }                                                                                        \
  } while (0)
