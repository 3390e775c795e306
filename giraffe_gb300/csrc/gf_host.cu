// Host side of the GB300 implicit Beam_1 path: builds device batches from
// gf_model_desc structures (DOF numbering, colouring, PreCalc constants,
// loads), drives the device-resident Newton loop, and implements the C ABI
// declared in include/giraffe_gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "../../include/giraffe_gpu.h"
#include "gf_host_internal.h"
#include "gf_kernels.cuh"
#include "gf_types.h"

using namespace gf;
using namespace gfh;

// FP64 flops of one Beam_1 Mount on the device (both Gauss points: kinematics,
// stresses, internal force, B^T D B + G, block rotation and the 18x18
// expansion), counted from the operation sequence of gf_beam.cuh.
#define GF_BEAM_MOUNT_FLOPS 9000.0


namespace gfh {

bool set_err(gf_ctx* ctx, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  return false;
}

#define CK(call)                                                                             \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      set_err(ctx, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return GF_ERR_CUDA;                                                                    \
    }                                                                                        \
  } while (0)

// ---- host restatements of PreCalc (reference src/Beam_1.cpp:501-692,
// src/CoordinateSystem.cpp:68-92) ----
void cs_rows(double* Q, const double* e1e3) {
  double e1[3] = {e1e3[0], e1e3[1], e1e3[2]}, e3[3] = {e1e3[3], e1e3[4], e1e3[5]};
  double e2[3] = {e3[1] * e1[2] - e3[2] * e1[1], e3[2] * e1[0] - e3[0] * e1[2], e3[0] * e1[1] - e3[1] * e1[0]};
  auto nrm = [](const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
  double n1 = nrm(e1), n2 = nrm(e2), n3 = nrm(e3);
  for (int k = 0; k < 3; ++k) {
    Q[k] = n1 != 1.0 ? e1[k] * (1.0 / n1) : e1[k];
    Q[3 + k] = n2 != 1.0 ? e2[k] * (1.0 / n2) : e2[k];
    Q[6 + k] = n3 != 1.0 ? e3[k] * (1.0 / n3) : e3[k];
  }
}

void beam_precalc(const double* x0, const double* x2, const double* mat, const double* sec, const double* cs,
                  BeamConst& c, BeamHist& h, BeamHistAux& x, double T0 = 0.0) {
  std::memset(&c, 0, sizeof(c));
  std::memset(&h, 0, sizeof(h));
  std::memset(&x, 0, sizeof(x));
  double E = mat[0], nu = mat[1], rho = mat[2];
  double G = E / (2 * (1 + nu));
  double sf = 1.0;
  double A = sec[0], I1 = sec[1], I2 = sec[2], I12 = sec[3], It = sec[4], I33 = sec[5];
  c.Dd[0] = sf * G * A;
  c.Dd[1] = sf * G * A;
  c.Dd[2] = E * A;
  c.Dd[3] = E * I1;
  c.Dd[4] = E * I2;
  c.Dd[5] = G * It;
  c.D34 = E * I12;
  c.Mr = rho * A;
  c.Jr[0] = rho * I1;
  c.Jr[4] = rho * I2;
  c.Jr[8] = rho * I33;
  c.Jr[1] = c.Jr[3] = rho * I12;
  cs_rows(c.T3, cs);
  double e3[3] = {x2[0] - x0[0], x2[1] - x0[1], x2[2] - x0[2]};
  double len = std::sqrt(e3[0] * e3[0] + e3[1] * e3[1] + e3[2] * e3[2]);
  double inv = 1.0 / len;
  for (int k = 0; k < 3; ++k) e3[k] = inv * e3[k];
  for (int i = 0; i < 3; ++i) c.e3r[i] = c.T3[i * 3] * e3[0] + c.T3[i * 3 + 1] * e3[1] + c.T3[i * 3 + 2] * e3[2];
  // pre-strain of a pre-tension T0: the reference length is the distance of
  // the end nodes shortened by 1 + T0 / EA, and the Gauss points start
  // stretched (reference src/Beam_1.cpp:616-621)
  const double du0 = T0 / c.Dd[2];
  c.jac = (len / (1.0 + du0)) / 2.0;
  for (int g = 0; g < 2; ++g) {
    double xi = g == 0 ? -0.577350269189626 : +0.577350269189626;
    c.N[g][0] = 0.5 * xi * (xi - 1.0);
    c.N[g][1] = 1.0 - xi * xi;
    c.N[g][2] = 0.5 * xi * (1.0 + xi);
    c.dN[g][0] = (1.0 / c.jac) * (xi - 0.5);
    c.dN[g][1] = (1.0 / c.jac) * (-2.0 * xi);
    c.dN[g][2] = (1.0 / c.jac) * (0.5 + xi);
  }
  for (int g = 0; g < 2; ++g) {
    h.Q[g][0] = h.Q[g][4] = h.Q[g][8] = 1.0;
    h.dz[g][2] = 1.0 + du0;
  }
}

// Pipe_1::PreCalc (reference src/Pipe_1.cpp:1106-1156): Beam_1's frame, e3r,
// length and shape functions (no pre-tension), with the PipeSection's
// constitutive matrix diag(GA, GA, EA, EI, EI, GJ), mass Rho per unit length
// and rotary inertia Rho ((De/2)^2 - (Di/2)^2) diag(1/4, 1/4, 1/2).  ps:
// EA, EI, GJ, GA, Rho, CDt, CDn, CAt, CAn, De, Di.
void pipe_precalc(const double* x0, const double* x2, const double* ps, const double* cs, BeamConst& c, BeamHist& h,
                  BeamHistAux& x) {
  const double unit_mat[3] = {1.0, 0.0, 0.0}, unit_sec[6] = {1.0, 1.0, 1.0, 0.0, 1.0, 1.0};
  beam_precalc(x0, x2, unit_mat, unit_sec, cs, c, h, x, 0.0);
  const double EA = ps[0], EI = ps[1], GJ = ps[2], GA = ps[3], Rho = ps[4], De = ps[9], Di = ps[10];
  c.Dd[0] = GA;
  c.Dd[1] = GA;
  c.Dd[2] = EA;
  c.Dd[3] = EI;
  c.Dd[4] = EI;
  c.Dd[5] = GJ;
  c.D34 = 0.0;
  c.Mr = Rho;
  for (int k = 0; k < 9; ++k) c.Jr[k] = 0.0;
  const double rr = (De / 2.0) * (De / 2.0) - (Di / 2.0) * (Di / 2.0);
  c.Jr[0] = (Rho * rr / 4.0);
  c.Jr[4] = (Rho * rr / 4.0);
  c.Jr[8] = (Rho * rr / 2.0);
}

template <typename T> bool dmalloc(gf_ctx* ctx, T** p, size_t n) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T));
  if (e != cudaSuccess) return set_err(ctx, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e));
  return true;
}


// ---- host restatement of Shell_1::PreCalc (reference
// src/Shell_1.cpp:1666-2365, homogeneous section, Hooke material) ----
static double tri_area2(const double* a, const double* b, const double* c) {
  double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, v[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  double w[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
  return 0.5 * std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
}

static void shell_shapes(const double* L, const double* L1, const double* L2, double* N, double* N1, double* N2) {
  N[0] = (2 * L[0] - 1) * L[0];
  N[1] = (2 * L[1] - 1) * L[1];
  N[2] = (2 * L[2] - 1) * L[2];
  N[3] = 4 * L[0] * L[1];
  N[4] = 4 * L[1] * L[2];
  N[5] = 4 * L[2] * L[0];
  const double* D[2] = {L1, L2};
  double* O[2] = {N1, N2};
  for (int q = 0; q < 2; ++q) {
    const double* Ld = D[q];
    O[q][0] = 4 * Ld[0] * L[0] - Ld[0];
    O[q][1] = 4 * Ld[1] * L[1] - Ld[1];
    O[q][2] = 4 * Ld[2] * L[2] - Ld[2];
    O[q][3] = 4 * Ld[0] * L[1] + 4 * L[0] * Ld[1];
    O[q][4] = 4 * Ld[1] * L[2] + 4 * L[1] * Ld[2];
    O[q][5] = 4 * Ld[2] * L[0] + 4 * L[2] * Ld[0];
  }
}

void shell_precalc(const double* xyz, const double* mat, double thick, ShellConst& c, ShellHist& h, ShellHistAux& x) {
  std::memset(&c, 0, sizeof(c));
  std::memset(&h, 0, sizeof(h));
  std::memset(&x, 0, sizeof(x));
  const double *x1 = xyz, *x2 = xyz + 3, *x3 = xyz + 6;
  double a[3], b[3];
  for (int k = 0; k < 3; ++k) { a[k] = x2[k] - x1[k]; b[k] = x3[k] - x1[k]; }
  double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
  double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  double A = 0.5 * nn;
  double e3[3], e1[3], e2[3];
  for (int k = 0; k < 3; ++k) e3[k] = (1.0 / nn) * n[k];
  double eg[3] = {1.0, 0.0, 0.0};
  if (std::fabs(e3[0]) >= 1.0 - 1e-4) { eg[0] = 0.0; eg[1] = 1.0; }
  double dd = eg[0] * e3[0] + eg[1] * e3[1] + eg[2] * e3[2];
  for (int k = 0; k < 3; ++k) e1[k] = eg[k] - dd * e3[k];
  double n1 = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
  for (int k = 0; k < 3; ++k) e1[k] = (1.0 / n1) * e1[k];
  e2[0] = e3[1] * e1[2] - e3[2] * e1[1];
  e2[1] = e3[2] * e1[0] - e3[0] * e1[2];
  e2[2] = e3[0] * e1[1] - e3[1] * e1[0];
  for (int k = 0; k < 3; ++k) { c.T3[k] = e1[k]; c.T3[3 + k] = e2[k]; c.T3[6 + k] = e3[k]; }
  double E = mat[0], nu = mat[1];
  c.mu = E / (2.0 * (1 + nu));
  c.lambda = 2.0 * c.mu * nu / (1 - 2.0 * nu);
  c.stiff_drill = E * thick * thick * thick;
  c.thick = thick;
  auto dotv = [](const double* p, const double* q) { return p[0] * q[0] + p[1] * q[1] + p[2] * q[2]; };
  double d23[3], d31[3], d12[3], d32[3], d13[3], d21[3];
  for (int k = 0; k < 3; ++k) {
    d23[k] = x2[k] - x3[k]; d31[k] = x3[k] - x1[k]; d12[k] = x1[k] - x2[k];
    d32[k] = x3[k] - x2[k]; d13[k] = x1[k] - x3[k]; d21[k] = x2[k] - x1[k];
  }
  double Lx1[3] = {0.5 * dotv(d23, e2) / A, 0.5 * dotv(d31, e2) / A, 0.5 * dotv(d12, e2) / A};
  double Lx2[3] = {0.5 * dotv(d32, e1) / A, 0.5 * dotv(d13, e1) / A, 0.5 * dotv(d21, e1) / A};
  for (int g = 0; g < 3; ++g) {
    const double* xp = xyz + 3 * (3 + g);
    double L[3] = {tri_area2(xp, x2, x3) / A, tri_area2(xp, x3, x1) / A, tri_area2(xp, x1, x2) / A};
    shell_shapes(L, Lx1, Lx2, c.Nu[g], c.Nu1[g], c.Nu2[g]);
    c.Na[g][0] = 1 - 2 * L[2]; c.Na[g][1] = 1 - 2 * L[0]; c.Na[g][2] = 1 - 2 * L[1];
    c.Na1[g][0] = -2 * Lx1[2]; c.Na1[g][1] = -2 * Lx1[0]; c.Na1[g][2] = -2 * Lx1[1];
    c.Na2[g][0] = -2 * Lx2[2]; c.Na2[g][1] = -2 * Lx2[0]; c.Na2[g][2] = -2 * Lx2[1];
  }
  // six-point surface rule of Cowper (1973)
  const double pa = 0.816847572980459, pb = 0.091576213509771, pc = 0.108103018168070, pd = 0.445948490915965;
  const double wa = 0.109951743655322, wb = 0.223381589678011;
  const double Lc[6][3] = {{pa, pb, pb}, {pb, pa, pb}, {pb, pb, pa}, {pc, pd, pd}, {pd, pc, pd}, {pd, pd, pc}};
  for (int k = 0; k < 6; ++k) {
    c.w4[k] = A * (k < 3 ? wa : wb);
    shell_shapes(Lc[k], Lx1, Lx2, c.N4[k], c.N41[k], c.N42[k]);
  }
  c.alpha1 = A / 3.0;
  // inertia of the director fibre and drilling inertia of the modal mass
  // (reference src/Shell_1.cpp:2022-2024); PI as reference src/Geometry.h:4
  c.coef1 = thick * mat[2];
  c.coef2 = (1.0 / 12.0) * thick * thick * thick * mat[2];
  c.coef3 = mat[2] * thick * A / (3 * 3.1415926535897932384626433832795);
  for (int k = 0; k < 6; ++k) {
    c.Na4[k][0] = 1 - 2 * Lc[k][2];
    c.Na4[k][1] = 1 - 2 * Lc[k][0];
    c.Na4[k][2] = 1 - 2 * Lc[k][1];
  }
  for (int g = 0; g < 3; ++g) {
    h.Q[g][0] = h.Q[g][4] = h.Q[g][8] = 1.0;
    h.z1[g][0] = 1.0;
    h.z2[g][1] = 1.0;
  }
}

// Reverse Cuthill-McKee order of the nodes of one structure (node graph:
// nodes that share an element).  Each connected component starts from a
// pseudo-peripheral node (repeated breadth-first search from a node of
// minimum degree in the last level); neighbours are visited by increasing
// degree; the final order is reversed.  Nodes without elements keep their
// place at the end.
std::vector<int> rcm_order(int nn, const std::vector<std::vector<int>>& adj) {
  std::vector<int> deg(nn), order;
  order.reserve(nn);
  for (int i = 0; i < nn; ++i) deg[i] = (int)adj[i].size();
  std::vector<char> seen(nn, 0);
  std::vector<int> level(nn, -1);
  auto bfs_last = [&](int r, int* ecc) {
    std::vector<int> q{r};
    std::fill(level.begin(), level.end(), -1);
    level[r] = 0;
    for (size_t h = 0; h < q.size(); ++h)
      for (int v : adj[q[h]])
        if (level[v] < 0) { level[v] = level[q[h]] + 1; q.push_back(v); }
    int last = level[q.back()];
    *ecc = last;
    int best = q.back();
    for (int v : q)
      if (level[v] == last && deg[v] < deg[best]) best = v;
    return best;
  };
  for (;;) {
    int start = -1;
    for (int i = 0; i < nn; ++i)
      if (!seen[i] && deg[i] > 0 && (start < 0 || deg[i] < deg[start])) start = i;
    if (start < 0) break;
    int ecc = 0, e2 = 0;
    int cand = bfs_last(start, &ecc);
    for (int it = 0; it < 8; ++it) {
      int nxt = bfs_last(cand, &e2);
      if (e2 <= ecc) break;
      start = cand;
      ecc = e2;
      cand = nxt;
    }
    std::vector<int> q{start};
    seen[start] = 1;
    for (size_t h = 0; h < q.size(); ++h) {
      std::vector<int> nb;
      for (int v : adj[q[h]])
        if (!seen[v]) nb.push_back(v);
      std::sort(nb.begin(), nb.end(), [&](int x, int y) { return deg[x] != deg[y] ? deg[x] < deg[y] : x < y; });
      for (int v : nb) { seen[v] = 1; q.push_back(v); }
    }
    order.insert(order.end(), q.rbegin(), q.rend());
  }
  for (int i = 0; i < nn; ++i)
    if (!seen[i]) order.push_back(i);
  return order;
}

}  // namespace gfh

namespace gfh {

double host_now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <typename T> bool balloc(gf_batch* B, T** p, size_t n) {
  size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  if (B->count_only) {
    B->counted_bytes += (bytes + 255) / 256 * 256;
    *p = nullptr;
    return true;
  }
  struct Clock {
    double* acc;
    double t0;
    ~Clock() { *acc += host_now_ms() - t0; }
  } clock{&B->host_ms[1], host_now_ms()};
  if (B->arena) {
    void* q = B->arena->alloc(bytes);
    if (!q) return set_err(B->ctx, "device budget exhausted (%zu bytes requested, %zu free in the largest block)",
                           bytes, B->arena->largest_free());
    *p = static_cast<T*>(q);
  } else if (!dmalloc(B->ctx, p, n)) {
    return false;
  }
  B->allocs.push_back(*p);
  return true;
}

template <typename T, typename A> bool upload(gf_batch* B, T** p, const std::vector<T, A>& v) {
  if (!balloc(B, p, v.size())) return false;
  B->h2d_bytes += (long long)(v.size() * sizeof(T));
  if (!v.empty() && !B->count_only) {
    // through pinned staging when the batch has some (the copy then does not
    // wait for other streams' work); else from the pageable source, staged
    // by the driver before return; ordered on the batch's stream
    const double t0 = host_now_ms();
    const size_t bytes = v.size() * sizeof(T);
    void* src = const_cast<T*>(v.data());
    if (B->host_stage) {
      if (void* h = B->host_stage->alloc(bytes)) {
        std::memcpy(h, v.data(), bytes);
        B->staged.push_back(h);
        src = h;
      }
    }
    cudaError_t e = cudaMemcpyAsync(*p, src, bytes, cudaMemcpyHostToDevice, B->stream);
    B->host_ms[2] += host_now_ms() - t0;
    if (e != cudaSuccess) return set_err(B->ctx, "upload failed: %s", cudaGetErrorString(e));
  }
  return true;
}

namespace {

std::string strf(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return buf;
}

// Runs f(s) for s in [0, n) on up to 16 host threads, structures handed out
// one at a time; inline when the batch is small (work: nodes + elements).
template <typename F> void parallel_structures(int n, size_t work, F f) {
  unsigned hw = std::thread::hardware_concurrency();
  int T = (int)std::min<unsigned>(hw ? hw : 1u, 16u);
  if (work < 50000) T = 1;
  T = std::min(T, n);
  if (T <= 1) {
    for (int s = 0; s < n; ++s) f(s);
    return;
  }
  std::atomic<int> next{0};
  auto worker = [&]() {
    for (int s; (s = next.fetch_add(1)) < n;) f(s);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < T; ++t) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
}

// One structure after the numbering pass.
struct StructPlan {
  std::string err;                  // non-empty: the structure is rejected
  std::vector<int> active, c6, g6;  // per node DOF: element-activated, constrained, free index (-1 fixed, -2 inactive)
  std::vector<int> dofs;            // local node DOF (6 node + k) of each free index, in the solver's order
  std::vector<int> perm;            // wide structures: the reference's free index -> the solver's
  std::vector<char> node_free;      // chain structures: node fully free
  int nf = 0, kb = 0, kl_nat = 0, wkl = 0;
  bool has_f = false, has_m = false, wide = false, chain = false;
  int n_colors = 0, n_scolors = 0;  // set by the fill pass
};

// Checks, activation and DOF numbering of one structure (SetGlobalDOFs,
// reference src/Solution.cpp:40-118), its half-bandwidth and whether it is a
// chain.
void plan_structure(const gf_model_desc& m, int s, StructPlan& P) {
  if (m.solution.type != GF_STATIC && m.solution.type != GF_DYNAMIC) {
    P.err = strf("structure %d: unknown solution type", s);
    return;
  }
  if (m.n_next_steps < 0 || (m.n_next_steps > 0 && !m.next_steps)) {
    P.err = strf("structure %d: invalid solution step list", s);
    return;
  }
  bool any_dynamic = m.solution.type == GF_DYNAMIC;
  for (int k = 0; k < m.n_next_steps; ++k) {
    if (m.next_steps[k].type != GF_STATIC && m.next_steps[k].type != GF_DYNAMIC) {
      P.err = strf("structure %d: unknown solution type in step %d", s, k + 2);
      return;
    }
    any_dynamic = any_dynamic || m.next_steps[k].type == GF_DYNAMIC;
  }
  if (m.n_shells && m.n_beams) {
    P.err = strf("structure %d: structures mixing Beam_1 and Shell_1 elements are not supported", s);
    return;
  }
  const int nn = m.n_nodes;
  const bool wide = m.n_shells > 0;
  P.wide = wide;
  std::vector<int>& active = P.active;
  std::vector<int>& c6 = P.c6;
  std::vector<int>& g6 = P.g6;
  active.assign((size_t)nn * 6, 0);
  c6.assign((size_t)nn * 6, 0);
  g6.assign((size_t)nn * 6, -2);
  for (int e = 0; e < m.n_shells; ++e) {
    const int* q = m.shells + 9 * e;
    for (int j = 0; j < 6; ++j) {
      if (q[j] < 0 || q[j] >= nn) {
        P.err = strf("structure %d: shell %d has node %d out of range", s, e, q[j]);
        return;
      }
      // Shell_1 activates translations everywhere, rotations on the
      // midside nodes (reference src/Shell_1.cpp:51-68)
      for (int k = 0; k < (j < 3 ? 3 : 6); ++k) active[6 * q[j] + k] = 1;
    }
    if (q[6] < 0 || q[6] >= m.n_materials || q[7] < 0 || q[7] >= m.n_shell_sections) {
      P.err = strf("structure %d: shell %d refers to a missing material or shell section", s, e);
      return;
    }
  }
  for (int e = 0; e < m.n_beams; ++e) {
    for (int j = 0; j < 3; ++j) {
      int nd = m.beams[6 * e + j];
      if (nd < 0 || nd >= nn) {
        P.err = strf("structure %d: beam %d has node %d out of range", s, e, nd);
        return;
      }
      for (int k = 0; k < 6; ++k) active[6 * nd + k] = 1;
    }
    const int ps = m.beam_pipe_section ? m.beam_pipe_section[e] : -1;
    if (ps >= 0) {
      // a Pipe_1 element: its pipe section and CS (material and section unused)
      if (ps >= m.n_pipe_sections || !m.pipe_sections || m.beams[6 * e + 5] < 0 || m.beams[6 * e + 5] >= m.n_cs) {
        P.err = strf("structure %d: pipe %d refers to a missing pipe section or CS", s, e);
        return;
      }
    } else if (m.beams[6 * e + 3] < 0 || m.beams[6 * e + 3] >= m.n_materials || m.beams[6 * e + 4] < 0 ||
               m.beams[6 * e + 4] >= m.n_sections || m.beams[6 * e + 5] < 0 || m.beams[6 * e + 5] >= m.n_cs) {
      P.err = strf("structure %d: beam %d refers to a missing material, section or CS", s, e);
      return;
    }
  }
  if (m.constraints)
    for (int i = 0; i < nn * 6; ++i) c6[i] = m.constraints[i] ? 1 : 0;
  // Node-major numbering.  Shell structures number their free DOFs in
  // reverse Cuthill-McKee node order instead when that gives the narrower
  // band (the solver's numbering; results are reported per node, and
  // gf_batch_assemble maps back to the reference's numbering through perm).
  std::vector<int> g_nat;
  auto number = [&](const std::vector<int>& order, std::vector<int>& g, std::vector<int>* dofs) {
    int q = 0;
    for (int i : order)
      for (int k = 0; k < 6; ++k) {
        if (!active[6 * i + k]) continue;
        if (c6[6 * i + k] == 0) {
          g[6 * i + k] = q++;
          if (dofs) dofs->push_back(6 * i + k);
        } else {
          g[6 * i + k] = -1;
        }
      }
    return q;
  };
  auto shell_band = [&](const std::vector<int>& g) {
    int kl = 0;
    for (int e = 0; e < m.n_shells; ++e) {
      const int* q = m.shells + 9 * e;
      int lo = INT_MAX, hi = -1;
      for (int a = 0; a < 27; ++a) {
        int d = a < 18 ? g[6 * q[a / 3] + a % 3] : g[6 * q[3 + (a - 18) / 3] + 3 + (a - 18) % 3];
        if (d >= 0) { lo = std::min(lo, d); hi = std::max(hi, d); }
      }
      if (hi >= 0) kl = std::max(kl, hi - lo);
    }
    return kl;
  };
  std::vector<int> natural(nn);
  for (int i = 0; i < nn; ++i) natural[i] = i;
  int nf = 0;
  if (wide) {
    g_nat.assign((size_t)nn * 6, -2);
    number(natural, g_nat, nullptr);
    P.kl_nat = shell_band(g_nat);
    std::vector<std::vector<int>> adj(nn);
    for (int e = 0; e < m.n_shells; ++e) {
      const int* q = m.shells + 9 * e;
      for (int a = 0; a < 6; ++a)
        for (int c = 0; c < 6; ++c)
          if (a != c) adj[q[a]].push_back(q[c]);
    }
    for (auto& v : adj) {
      std::sort(v.begin(), v.end());
      v.erase(std::unique(v.begin(), v.end()), v.end());
    }
    nf = number(rcm_order(nn, adj), g6, &P.dofs);
    P.wkl = shell_band(g6);
    if (P.wkl > P.kl_nat) {  // keep the natural numbering when it is narrower
      g6 = g_nat;
      P.dofs.clear();
      for (int i = 0; i < nn * 6; ++i)
        if (g6[i] >= 0) P.dofs.push_back(i);
      P.wkl = P.kl_nat;
    }
    P.perm.assign(nf, 0);
    for (int i = 0; i < nn * 6; ++i)
      if (g_nat[i] >= 0) P.perm[g_nat[i]] = g6[i];
  } else {
    P.dofs.reserve((size_t)nn * 6);
    nf = number(natural, g6, &P.dofs);
  }
  P.nf = nf;
  for (int d : P.dofs) {
    if (d % 6 < 3) P.has_f = true; else P.has_m = true;
  }
  // half-bandwidth: the widest spread of free indices within one element
  int kbs = 0;
  for (int e = 0; e < m.n_beams; ++e) {
    int lo = INT_MAX, hi = -1;
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 6; ++k) {
        int g = g6[6 * m.beams[6 * e + j] + k];
        if (g >= 0) { lo = std::min(lo, g); hi = std::max(hi, g); }
      }
    if (hi >= 0) kbs = std::max(kbs, hi - lo);
  }
  if (kbs > GF_KB) {
    P.err = strf("structure %d: K_AA half-bandwidth %d exceeds %d (node-major numbering of a chain gives 17)", s, kbs,
                 GF_KB);
    return;
  }
  P.kb = wide ? P.kl_nat : kbs;
  if (any_dynamic)
    for (int i = 0; i < nn; ++i) {
      int fr = (g6[6 * i + 3] >= 0) + (g6[6 * i + 4] >= 0) + (g6[6 * i + 5] >= 0);
      if (fr != 0 && fr != 3) {
        P.err = strf("structure %d: dynamic nodes need all rotations free or all fixed (node %d)", s, i);
        return;
      }
    }
  // chain structure: elements on nodes (2e, 2e+1, 2e+2), every node fully
  // free or fully fixed, midside and interior corner nodes free
  bool chain = m.n_beams > 0 && nn == 2 * m.n_beams + 1;
  for (int e = 0; chain && e < m.n_beams; ++e)
    chain = m.beams[6 * e] == 2 * e && m.beams[6 * e + 1] == 2 * e + 1 && m.beams[6 * e + 2] == 2 * e + 2;
  P.node_free.assign(nn, 0);
  for (int i = 0; chain && i < nn; ++i) {
    int f = 0;
    for (int k = 0; k < 6; ++k) f += g6[6 * i + k] >= 0;
    if (f != 0 && f != 6) chain = false;
    P.node_free[i] = f == 6;
    bool interior = i > 0 && i < nn - 1;
    if (interior && !P.node_free[i]) chain = false;
  }
  P.chain = chain;
}

}  // namespace

// A device array initialised from another device array of the batch (the
// initial states kept for gf_batch_reset).
template <typename T> bool dup(gf_batch* B, T** p, const T* src, size_t n) {
  if (!balloc(B, p, n)) return false;
  if (n && !B->count_only) {
    cudaError_t e = cudaMemcpyAsync(*p, src, n * sizeof(T), cudaMemcpyDeviceToDevice, B->stream);
    if (e != cudaSuccess) return set_err(B->ctx, "device copy failed: %s", cudaGetErrorString(e));
  }
  return true;
}

// A zero-filled device array.
template <typename T> bool zeroed(gf_batch* B, T** p, size_t n) {
  if (!balloc(B, p, n)) return false;
  if (!B->count_only) {
    cudaError_t e = cudaMemsetAsync(*p, 0, std::max<size_t>(n, 1) * sizeof(T), B->stream);
    if (e != cudaSuccess) return set_err(B->ctx, "device memset failed: %s", cudaGetErrorString(e));
  }
  return true;
}

int build_batch(gf_batch* B, int n, const gf_model_desc* models) {
  gf_ctx* ctx = B->ctx;
  Batch& b = B->b;
  {
    const int* wt = B->opts.wide_tiles;
    if ((wt[0] && wt[0] != 4 && wt[0] != 8 && wt[0] != 16) || (wt[1] && wt[1] != 1 && wt[1] != 2 && wt[1] != 4) ||
        (wt[2] && wt[2] != 4 && wt[2] != 8) || (wt[3] && wt[3] != 32 && wt[3] != 64)) {
      set_err(ctx, "wide_tiles: bulk trsm rows 4/8/16, first trsm rows 1/2/4, corner tile 4/8, solve rows 32/64");
      return GF_ERR_ARG;
    }
  }
  // ---- numbering pass (parallel over structures) ----
  std::vector<StructPlan> plan(n);
  size_t work = 0;
  for (int s = 0; s < n; ++s) work += (size_t)std::max(models[s].n_nodes, 0) + std::max(models[s].n_beams, 0) +
                                      std::max(models[s].n_shells, 0);
  parallel_structures(n, work, [&](int s) { plan_structure(models[s], s, plan[s]); });
  for (int s = 0; s < n; ++s)
    if (!plan[s].err.empty()) {
      set_err(ctx, "%s", plan[s].err.c_str());
      return GF_ERR_ARG;
    }
  // ---- offsets (serial) ----
  std::vector<int> node_offs(n), elem_offs(n), shell_offs(n), dof_offs(n);
  int node_off = 0, elem_off = 0, dof_off = 0, shell_off = 0;
  std::vector<int> wide_structs;
  int64_t wb_total = 0;
  int max_panels = 0, max_wkl = 0;
  B->perm.assign(n, std::vector<int>());
  B->info.assign(n, StructInfo{});
  B->kb.assign(n, 0);
  B->shell_off.assign(n, 0);
  for (int s = 0; s < n; ++s) {
    const gf_model_desc& m = models[s];
    StructPlan& P = plan[s];
    node_offs[s] = node_off;
    elem_offs[s] = elem_off;
    shell_offs[s] = shell_off;
    dof_offs[s] = dof_off;
    StructInfo& inf = B->info[s];
    inf.node_off = node_off;
    inf.n_nodes = m.n_nodes;
    inf.elem_off = elem_off;
    inf.n_elem = m.n_beams;
    inf.dof_off = dof_off;
    inf.n_free = P.nf;
    inf.band_off = (int64_t)dof_off * GF_LDB;
    inf.has_force = P.has_f;
    inf.has_moment = P.has_m;
    inf.is_chain = P.chain ? 1 : 0;
    if (P.wide) {
      inf.wide = 1;
      inf.wkl = std::max(P.wkl, 1);
      inf.n_panels = (P.nf + GF_WB_NB - 1) / GF_WB_NB;
      inf.wb_off = wb_total;
      wb_total += (int64_t)std::max(P.nf, 1) * (2 * inf.wkl + 1);
      wide_structs.push_back(s);
      max_panels = std::max(max_panels, inf.n_panels);
      max_wkl = std::max(max_wkl, inf.wkl);
      B->perm[s] = std::move(P.perm);
    }
    B->kb[s] = P.kb;
    B->shell_off[s] = shell_off;
    node_off += m.n_nodes;
    elem_off += m.n_beams;
    shell_off += m.n_shells;
    // padding: every structure's DOF range starts at a multiple of 32
    dof_off += (P.nf + 31) / 32 * 32;
  }
  // ---- fill pass (parallel over structures): nodes, DOF map, PreCalc and
  // colouring of the elements ----
  hvec<double> copy((size_t)node_off * 6), Qn((size_t)node_off * 9);
  hvec<int> gl((size_t)node_off * 6), cons((size_t)node_off * 6), node_struct(node_off);
  hvec<int> dof_node6(dof_off);
  hvec<BeamConst> bconst(elem_off);
  hvec<BeamHist> bhist(elem_off);
  hvec<BeamHistAux> baux(elem_off);
  hvec<int> enodes((size_t)elem_off * 3), estruct(elem_off), ecolor(elem_off);
  hvec<ShellConst> sconst(shell_off);
  hvec<ShellHist> shist(shell_off);
  hvec<ShellHistAux> saux(shell_off);
  hvec<int> snodes((size_t)shell_off * 6), sstruct(shell_off), spress(shell_off), sarea(shell_off), scolor(shell_off);
  parallel_structures(n, work, [&](int s) {
    const gf_model_desc& m = models[s];
    StructPlan& P = plan[s];
    const int nn = m.n_nodes, no = node_offs[s], eo = elem_offs[s], so = shell_offs[s];
    const int dof_end = s + 1 < n ? dof_offs[s + 1] : dof_off;
    for (int i = 0; i < nn; ++i) {
      double* x = &copy[(size_t)(no + i) * 6];
      for (int k = 0; k < 3; ++k) { x[k] = m.node_xyz[3 * i + k]; x[3 + k] = 0.0; }
      double* q = &Qn[(size_t)(no + i) * 9];
      for (int k = 0; k < 9; ++k) q[k] = k % 4 == 0 ? 1.0 : 0.0;
      for (int k = 0; k < 6; ++k) {
        gl[(size_t)(no + i) * 6 + k] = P.g6[6 * i + k];
        cons[(size_t)(no + i) * 6 + k] = P.c6[6 * i + k];
      }
      node_struct[no + i] = s;
    }
    for (int q = 0; q < P.nf; ++q) dof_node6[dof_offs[s] + q] = no * 6 + P.dofs[q];
    for (int q = dof_offs[s] + P.nf; q < dof_end; ++q) dof_node6[q] = -1;  // padding
    // elements: PreCalc + greedy colouring by shared nodes
    std::vector<unsigned> node_colors(nn, 0u);
    for (int e = 0; e < m.n_beams; ++e) {
      const int* be = m.beams + 6 * e;
      const int ps = m.beam_pipe_section ? m.beam_pipe_section[e] : -1;
      if (ps >= 0)
        pipe_precalc(m.node_xyz + 3 * be[0], m.node_xyz + 3 * be[2], m.pipe_sections + 11 * ps, m.cs + 6 * be[5],
                     bconst[eo + e], bhist[eo + e], baux[eo + e]);
      else
        beam_precalc(m.node_xyz + 3 * be[0], m.node_xyz + 3 * be[2], m.materials + 3 * be[3],
                     m.sections + 6 * be[4], m.cs + 6 * be[5], bconst[eo + e], bhist[eo + e], baux[eo + e],
                     m.beam_pretension ? m.beam_pretension[e] : 0.0);
      for (int j = 0; j < 3; ++j) enodes[(size_t)(eo + e) * 3 + j] = no + be[j];
      estruct[eo + e] = s;
      unsigned used = node_colors[be[0]] | node_colors[be[1]] | node_colors[be[2]];
      int col = 0;
      while (col < 8 && (used >> col) & 1u) ++col;
      if (col >= 8) {
        P.err = strf("structure %d: element colouring needs more than 8 colours", s);
        return;
      }
      for (int j = 0; j < 3; ++j) node_colors[be[j]] |= 1u << col;
      ecolor[eo + e] = col;
      P.n_colors = std::max(P.n_colors, col + 1);
    }
    // Shell_1 PreCalc and greedy colouring (up to 16 colours)
    for (int e = 0; e < m.n_shells; ++e) {
      const int* q = m.shells + 9 * e;
      double xyz[18];
      for (int j = 0; j < 6; ++j)
        for (int k = 0; k < 3; ++k) xyz[3 * j + k] = m.node_xyz[3 * q[j] + k];
      shell_precalc(xyz, m.materials + 3 * q[6], m.shell_sections[q[7]], sconst[so + e], shist[so + e], saux[so + e]);
      for (int j = 0; j < 6; ++j) snodes[(size_t)(so + e) * 6 + j] = no + q[j];
      sstruct[so + e] = s;
      spress[so + e] = -1;  // set by the pressure loads below
      sarea[so + e] = 0;
      unsigned used = 0;
      for (int j = 0; j < 6; ++j) used |= node_colors[q[j]];
      int col = 0;
      while (col < 16 && (used >> col) & 1u) ++col;
      if (col >= 16) {
        P.err = strf("structure %d: shell colouring needs more than 16 colours", s);
        return;
      }
      for (int j = 0; j < 6; ++j) node_colors[q[j]] |= 1u << col;
      scolor[so + e] = col;
      P.n_scolors = std::max(P.n_scolors, col + 1);
    }
  });
  int max_color = 0, max_scolor = 0;
  for (int s = 0; s < n; ++s) {
    if (!plan[s].err.empty()) {
      set_err(ctx, "%s", plan[s].err.c_str());
      return GF_ERR_ARG;
    }
    max_color = std::max(max_color, plan[s].n_colors);
    max_scolor = std::max(max_scolor, plan[s].n_scolors);
  }
  // ---- tables, loads, prescribed displacements, step parameters (serial) ----
  std::vector<StructParams> params(n), step_params;
  std::vector<LoadEntry> loads;
  std::vector<int> pp_elem, pp_table;
  std::vector<double> pp_aint;
  std::vector<int> mon_node, mon_struct, mon_adj_off(1, 0);
  std::vector<int2> mon_adj;
  B->mon_first.clear();
  std::vector<DispEntry> disps;
  std::vector<TableDev> tables;
  std::vector<double> tdata;
  for (int s = 0; s < n; ++s) {
    const gf_model_desc& m = models[s];
    const StructPlan& P = plan[s];
    const std::vector<int>& active = P.active;
    const std::vector<int>& g6 = P.g6;
    const int node_off = node_offs[s], shell_off = shell_offs[s];
    StructInfo& inf = B->info[s];
    // tables and nodal loads (NodalLoad::UpdateforSolutionStep, reference
    // src/NodalLoad.cpp:235-263)
    auto add_table = [&](const gf_table& t) {
      TableDev d{t.n_times, t.n_cols, (int64_t)tdata.size()};
      for (int i = 0; i < t.n_times; ++i) tdata.push_back(t.times[i]);
      for (int i = 0; i < t.n_times * t.n_cols; ++i) tdata.push_back(t.values[i]);
      tables.push_back(d);
      return (int)tables.size() - 1;
    };
    inf.load_off = (int)loads.size();
    std::vector<char> pipe_pressed;
    for (int l = 0; l < m.n_loads; ++l) {
      const gf_load& L = m.loads[l];
      if (L.type == GF_LOAD_SHELL_PRESSURE) {
        // ShellLoad (reference src/ShellLoad.cpp:133-148): one follower
        // pressure per element
        if (L.table.n_cols < 1) { set_err(ctx, "structure %d: pressure table needs 1 column", s); return GF_ERR_ARG; }
        int t = add_table(L.table);
        for (int q = 0; q < L.n_items; ++q) {
          int e = L.items[q];
          if (e < 0 || e >= m.n_shells) { set_err(ctx, "structure %d: pressure on missing shell %d", s, e); return GF_ERR_ARG; }
          if (spress[shell_off + e] >= 0) {
            set_err(ctx, "structure %d: shell %d carries more than one pressure load", s, e);
            return GF_ERR_ARG;
          }
          spress[shell_off + e] = t;
          sarea[shell_off + e] = L.area_update ? 1 : 0;
        }
        continue;
      }
      if (L.type == GF_LOAD_PIPE_PRESSURE) {
        // PipeLoad (reference src/PipeLoad.cpp:123-138): the internal
        // pressure P0I of its table on each Pipe_1 of the set, one PipeLoad
        // per element
        if (L.table.n_cols < 1) { set_err(ctx, "structure %d: PipeLoad table needs P0I", s); return GF_ERR_ARG; }
        int t = add_table(L.table);
        for (int q = 0; q < L.n_items; ++q) {
          const int e = L.items[q];
          const int ps = e >= 0 && e < m.n_beams && m.beam_pipe_section ? m.beam_pipe_section[e] : -1;
          if (ps < 0) { set_err(ctx, "structure %d: PipeLoad on %d, which is not a Pipe_1", s, e); return GF_ERR_ARG; }
          if (pipe_pressed.empty()) pipe_pressed.assign((size_t)m.n_beams, 0);
          if (pipe_pressed[e]) {
            set_err(ctx, "structure %d: pipe %d carries more than one PipeLoad", s, e);
            return GF_ERR_ARG;
          }
          pipe_pressed[e] = 1;
          const double Di = m.pipe_sections[11 * ps + 10];
          pp_elem.push_back(elem_offs[s] + e);
          pp_table.push_back(t);
          pp_aint.push_back(3.1415926535897932384626433832795 * Di * Di / 4.0);
        }
        continue;
      }
      if (L.type != GF_LOAD_NODAL) { set_err(ctx, "structure %d: unknown load type", s); return GF_ERR_ARG; }
      if (L.table.n_cols < 6) { set_err(ctx, "structure %d: nodal load table needs 6 columns", s); return GF_ERR_ARG; }
      int cnt[6] = {0, 0, 0, 0, 0, 0};
      for (int q = 0; q < L.n_items; ++q)
        for (int k = 0; k < 6; ++k)
          if (active[6 * L.items[q] + k] != 0) cnt[k]++;
      int t = add_table(L.table);
      double CQ[9];
      cs_rows(CQ, m.cs + 6 * L.cs);
      for (int q = 0; q < L.n_items; ++q) {
        LoadEntry le{};
        le.structure = s;
        le.node = node_off + L.items[q];
        le.table = t;
        std::memcpy(le.CQ, CQ, sizeof(CQ));
        for (int k = 0; k < 6; ++k) le.mult[k] = 1.0 / cnt[k];
        loads.push_back(le);
        // load stiffness couples the node's rotations
        for (int a = 3; a < 6; ++a)
          for (int c = 3; c < 6; ++c) {
            int ga = g6[6 * L.items[q] + a], gc = g6[6 * L.items[q] + c];
            if (ga >= 0 && gc >= 0 && std::abs(ga - gc) > GF_KB) { set_err(ctx, "load bandwidth"); return GF_ERR_ARG; }
          }
      }
    }
    inf.n_loads = (int)loads.size() - inf.load_off;
    // monitored nodes (Monitor: Sample, MonitorNodes) and the elements that
    // meet at each
    inf.mon_off = (int)mon_node.size();
    inf.mon_n = 0;
    inf.mon_sample = std::max(m.monitor_sample, 1);
    if (B->opts.monitor_rows > 0 && m.n_monitor_nodes > 0 && m.monitor_nodes) {
      for (int q = 0; q < m.n_monitor_nodes; ++q) {
        const int nd = m.monitor_nodes[q];
        if (nd < 0 || nd >= m.n_nodes) { set_err(ctx, "structure %d: monitored node %d out of range", s, nd); return GF_ERR_ARG; }
        mon_node.push_back(node_off + nd);
        mon_struct.push_back(s);
        for (int e = 0; e < m.n_beams; ++e)
          for (int j = 0; j < 3; ++j)
            if (m.beams[6 * e + j] == nd) mon_adj.push_back(make_int2(elem_offs[s] + e, j));
        for (int e = 0; e < m.n_shells; ++e)
          for (int j = 0; j < 6; ++j)
            if (m.shells[9 * e + j] == nd) mon_adj.push_back(make_int2(shell_off + e, 64 + j));
        mon_adj_off.push_back((int)mon_adj.size());
        B->mon_first.push_back(m.node_xyz[3 * nd]);
        B->mon_first.push_back(m.node_xyz[3 * nd + 1]);
        B->mon_first.push_back(m.node_xyz[3 * nd + 2]);
        B->mon_first.push_back(m.solution.start_time);
        inf.mon_n++;
      }
    }
    for (int l = 0; l < m.n_displacements; ++l) {
      const gf_displacement& D = m.displacements[l];
      if (D.table.n_cols < 6) { set_err(ctx, "structure %d: displacement table needs 6 columns", s); return GF_ERR_ARG; }
      int t = add_table(D.table);
      double CQ[9];
      cs_rows(CQ, m.cs + 6 * D.cs);
      for (int q = 0; q < D.n_nodes; ++q) {
        DispEntry de{};
        de.structure = s;
        de.node = node_off + D.nodes[q];
        de.table = t;
        de.angular = D.angular == GF_ANGLES_VECTOR ? GF_ANGLES_VECTOR : GF_ANGLES_EULER;
        std::memcpy(de.CQ, CQ, sizeof(CQ));
        disps.push_back(de);
      }
    }
    // the structure's solution steps: each starts where the previous one
    // ends (reference src/Database.cpp:759-768)
    inf.step_off = (int)step_params.size();
    inf.n_steps = 1 + m.n_next_steps;
    double start = m.solution.start_time;
    for (int k = 0; k < inf.n_steps; ++k) {
      const gf_solution& so = k == 0 ? m.solution : m.next_steps[k - 1];
      StructParams p{};
      p.start_time = start;
      p.end_time = so.end_time;
      p.time_step0 = so.time_step;
      p.max_time_step = so.max_time_step;
      p.min_time_step = so.min_time_step;
      p.inc_factor = so.inc_factor;
      p.max_it = so.max_it;
      p.min_it = so.min_it;
      p.conv_increase = so.conv_increase;
      p.dynamic = so.type == GF_DYNAMIC;
      if (p.dynamic) b.any_dynamic = 1;
      p.zero_va = !p.dynamic || so.zero_ic;
      p.beta = so.beta;
      p.gamma = so.gamma;
      const gf_criteria& cr = m.criteria;
      p.force_tol = cr.force_tol;
      p.moment_tol = cr.moment_tol;
      p.force_min = cr.force_min;
      p.moment_min = cr.moment_min;
      p.disp_tol = cr.disp_tol;
      p.rot_tol = cr.rot_tol;
      p.disp_min = cr.disp_min;
      p.rot_min = cr.rot_min;
      p.divergence_ref = cr.divergence_ref;
      if (so.type == GF_DYNAMIC && (so.rayleigh_alpha != 0.0 || so.rayleigh_beta != 0.0)) {
        p.ray_on = 1;
        p.ray_alpha = so.rayleigh_alpha;
        p.ray_beta = so.rayleigh_beta;
        p.ray_update = so.update_rayleigh ? 1 : 0;
        if (m.n_beams) b.any_rayleigh = 1;
        if (m.n_shells) b.sh.any_rayleigh = 1;
      }
      step_params.push_back(p);
      start = so.end_time;
    }
    params[s] = step_params[inf.step_off];
  }
  b.n_struct = n;
  b.n_nodes = node_off;
  b.n_elem = elem_off;
  b.n_free = dof_off;
  b.n_loads = (int)loads.size();
  b.n_pipe_press = (int)pp_elem.size();
  b.mon_total = (int)mon_node.size();
  b.mon_cap = b.mon_total ? B->opts.monitor_rows : 0;
  b.n_disps = (int)disps.size();
  b.n_tables = (int)tables.size();
  // chain solver data: sizes and offsets per structure (serial), then the
  // tables of each structure filled in parallel
  {
    ChainData& cd = b.chain;
    const int NL = CR_MAX_LEVELS;
    std::vector<int> Mc(n, 0), tb(n, 0), cb(n, 0), rpos(n, -1);
    std::vector<int> opos((size_t)n * NL, 0), epos((size_t)n * NL, 0);
    std::vector<int> ocnt(NL, 0), ecnt(NL, 0);
    int n_t = 0, n_c = 0, n_levels = 0, n_roots = 0;
    for (int s = 0; s < n; ++s) {
      if (!plan[s].chain) continue;
      const int mm = B->info[s].n_elem;
      const std::vector<char>& fr = plan[s].node_free;
      int M = 0;
      for (int ci = 0; ci <= mm; ++ci) M += fr[2 * ci] != 0;
      Mc[s] = M;
      tb[s] = n_t;
      cb[s] = n_c;
      n_t += mm;
      n_c += M;
      if (M >= 1) rpos[s] = n_roots++;
      int l = 0;
      for (int h = 1; h < M; h *= 2, ++l) {
        if (l >= NL) { set_err(ctx, "chain too long for %d reduction levels", NL); return GF_ERR_ARG; }
        // odd items kp = h, 3h, 5h, ... < M; even items kp = 0, 2h, 4h, ... < M
        opos[(size_t)s * NL + l] = ocnt[l];
        ocnt[l] += (M - h - 1) / (2 * h) + 1;
        epos[(size_t)s * NL + l] = ecnt[l];
        ecnt[l] += (M + 2 * h - 1) / (2 * h);
      }
      n_levels = std::max(n_levels, l);
    }
    for (int l = 0, o = 0, e = 0; l <= NL; ++l) {
      cd.odd_off[l] = o;
      cd.even_off[l] = e;
      if (l < NL) { o += ocnt[l]; e += ecnt[l]; }
    }
    hvec<int> elem_list(n_t), eca(n_t), ecb(n_t), cnode(n_c), cstruct(n_c), cleft(n_c), cright(n_c), cprev(n_c),
        cnext(n_c), roots(n_roots);
    hvec<CrItem> odd(cd.odd_off[NL]), even(cd.even_off[NL]);
    parallel_structures(n, work, [&](int s) {
      if (!plan[s].chain) return;
      const StructInfo& inf = B->info[s];
      const int mm = inf.n_elem, M = Mc[s], cbase = cb[s], tbase = tb[s];
      const std::vector<char>& fr = plan[s].node_free;
      // corner slots: the chain's corners in the order of cyclic reduction,
      // position 0, then the odd multiples of the largest power of two below
      // M, ..., then the odd positions; at every level the items eliminated
      // (the odd multiples of 2^l) are one contiguous run and the surviving
      // ones the run before it, so a level's loads are contiguous in the
      // structure-of-arrays scratch
      std::vector<int> slot(std::max(M, 1));
      {
        int r = 0;
        if (M > 0) slot[0] = r++;
        int hmax = 1;
        while (hmax * 2 < M) hmax *= 2;
        for (int h = hmax; h >= 1 && M > 1; h /= 2)
          for (int kp = h; kp < M; kp += 2 * h) slot[kp] = r++;
      }
      std::vector<int> pos(mm + 1, -1);
      for (int ci = 0, k = 0; ci <= mm; ++ci)
        if (fr[2 * ci]) pos[ci] = slot[k++];
      for (int e = 0; e < mm; ++e) {
        elem_list[tbase + e] = inf.elem_off + e;
        eca[tbase + e] = pos[e] >= 0 ? cbase + pos[e] : -1;
        ecb[tbase + e] = pos[e + 1] >= 0 ? cbase + pos[e + 1] : -1;
      }
      for (int ci = 0, k = 0; ci <= mm; ++ci) {
        if (pos[ci] < 0) continue;
        const int c = cbase + pos[ci];
        cnode[c] = inf.node_off + 2 * ci;
        cstruct[c] = s;
        cleft[c] = ci >= 1 ? tbase + ci - 1 : -1;
        cright[c] = ci < mm ? tbase + ci : -1;
        cprev[c] = k > 0 ? cbase + slot[k - 1] : -1;
        cnext[c] = k + 1 < M ? cbase + slot[k + 1] : -1;
        ++k;
      }
      if (rpos[s] >= 0) roots[rpos[s]] = cbase + slot[0];
      int l = 0;
      for (int h = 1; h < M; h *= 2, ++l) {
        CrItem* o = &odd[cd.odd_off[l] + opos[(size_t)s * NL + l]];
        for (int kp = h; kp < M; kp += 2 * h)
          *o++ = CrItem{cbase + slot[kp], cbase + slot[kp - h], kp + h < M ? cbase + slot[kp + h] : -1, s};
        CrItem* v = &even[cd.even_off[l] + epos[(size_t)s * NL + l]];
        for (int kp = 0; kp < M; kp += 2 * h) {
          bool hp = kp - h >= 0, hn = kp + h < M;
          *v++ = CrItem{cbase + slot[kp], hp ? cbase + slot[kp - h] : -1, hn ? cbase + slot[kp + h] : -1, s};
        }
      }
    });
    cd.n_chain_elems = (int)elem_list.size();
    cd.n_corners = (int)cnode.size();
    cd.n_levels = n_levels;
    cd.n_roots = (int)roots.size();
    if (cd.n_chain_elems) {
      size_t ne = elem_list.size(), nc = std::max<size_t>(cnode.size(), 1);
      if (!upload(B, &cd.elem_list, elem_list) || !upload(B, &cd.elem_corner_a, eca) ||
          !upload(B, &cd.elem_corner_b, ecb) || !upload(B, &cd.corner_node, cnode) ||
          !upload(B, &cd.corner_struct, cstruct) || !upload(B, &cd.corner_left, cleft) ||
          !upload(B, &cd.corner_right, cright) || !upload(B, &cd.corner_prev, cprev) ||
          !upload(B, &cd.corner_next, cnext) || !upload(B, &cd.odd, odd) || !upload(B, &cd.even, even) ||
          !upload(B, &cd.roots, roots) || !balloc(B, &cd.ez, ne * 78) || !balloc(B, &cd.ec, ne * 156) ||
          !balloc(B, &cd.cD, nc * 36) || !balloc(B, &cd.cL, nc * 36) || !balloc(B, &cd.cU, nc * 36) ||
          !balloc(B, &cd.cb, nc * 6) || !balloc(B, &cd.cz, nc * 78) || !balloc(B, &cd.cx, nc * 6))
        return GF_ERR_CUDA;
    }
  }
  // colour lists
  std::vector<int> color_elems;
  b.n_colors = max_color;
  for (int c = 0; c < max_color; ++c) {
    b.color_off[c] = (int)color_elems.size();
    for (int e = 0; e < elem_off; ++e)
      if (ecolor[e] == c) color_elems.push_back(e);
  }
  b.color_off[max_color] = (int)color_elems.size();
  // Shell_1 arrays, colour lists and the wide band
  ShellData& sd = b.sh;
  sd.n_shells = shell_off;
  sd.n_wide = (int)wide_structs.size();
  sd.max_panels = max_panels;
  sd.max_kl = max_wkl;
  sd.n_colors = max_scolor;
  std::vector<int> scolor_elems;
  for (int c = 0; c < max_scolor; ++c) {
    sd.color_off[c] = (int)scolor_elems.size();
    for (int e = 0; e < shell_off; ++e)
      if (scolor[e] == c) scolor_elems.push_back(e);
  }
  sd.color_off[max_scolor] = (int)scolor_elems.size();
  if (shell_off) {
    if (!upload(B, &sd.snodes, snodes) || !upload(B, &sd.sstruct, sstruct) || !upload(B, &sd.spress, spress) ||
        !upload(B, &sd.sarea, sarea) || !upload(B, &sd.sconst, sconst) || !upload(B, &sd.shist, shist) ||
        !upload(B, &sd.saux, saux) || !dup(B, &B->shist0, sd.shist, shist.size()) ||
        !dup(B, &B->saux0, sd.saux, saux.size()) ||
        !upload(B, &sd.color_elems, scolor_elems) || !balloc(B, &sd.Ke, (size_t)shell_off * 729) ||
        !balloc(B, &sd.Fe, (size_t)shell_off * 27) ||
        (sd.any_rayleigh && !balloc(B, &sd.RD, (size_t)shell_off * 729)))
      return GF_ERR_CUDA;
  }
  if (!wide_structs.empty()) {
    if (!upload(B, &sd.wide_structs, wide_structs) || !balloc(B, &sd.wband, (size_t)wb_total) ||
        !balloc(B, &sd.panel, 1))
      return GF_ERR_CUDA;
    if (B->opts.precision == GF_PREC_MIXED) {
      // the FP32 LU beside the FP64 K_AA, its right-hand side and scratch,
      // the saved Newton right-hand side and the refinement state
      if (!balloc(B, &sd.wband32, (size_t)wb_total) || !balloc(B, &sd.r32, (size_t)dof_off) ||
          !balloc(B, &sd.y32, (size_t)dof_off) || !balloc(B, &sd.ir_rhs, (size_t)dof_off) ||
          !zeroed(B, &sd.ir, wide_structs.size()) || !zeroed(B, &sd.ir_more, 4))
        return GF_ERR_CUDA;
    }
    if (B->opts.wide_update == GF_WIDE_TENSOR || B->opts.wide_update == GF_WIDE_TENSOR_SYNC) {
      // slices of one panel per wide structure for the tensor-core update
      sd.oz_rows = (max_wkl + 127) / 128 * 128;  // whole 128-row tiles of the tensor-core update
      const size_t nw = wide_structs.size(), R = (size_t)sd.oz_rows;
      if (!zeroed(B, &sd.oz_slices, nw * 2 * 8 * R * GF_WB_NB) || !balloc(B, &sd.oz_exp, nw * 2 * R) ||
          !zeroed(B, &sd.oz_kmax, nw * 2 * 2 * GF_WB_NB) || !zeroed(B, &sd.oz_error, 1))
        return GF_ERR_CUDA;
    }
    if (!B->count_only) {
      for (auto& a : sd.aux) CK(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking));
      for (auto& e : sd.evt) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
  }
  // device arrays
  const size_t n6 = (size_t)node_off * 6;
  if (!upload(B, &b.copy, copy) || !upload(B, &b.Qn, Qn) || !zeroed(B, &b.disp, n6) || !upload(B, &b.gl, gl) ||
      !zeroed(B, &b.vel, n6) || !zeroed(B, &b.accel, n6) || !zeroed(B, &b.copy_vel, n6) ||
      !zeroed(B, &b.copy_accel, n6) ||
      !upload(B, &b.cons, cons) || !upload(B, &b.node_struct, node_struct) || !upload(B, &b.enodes, enodes) ||
      !upload(B, &b.estruct, estruct) || !upload(B, &b.bconst, bconst) || !upload(B, &b.bhist, bhist) ||
      !upload(B, &b.baux, baux) || !upload(B, &b.color_elems, color_elems) || !upload(B, &b.dof_node6, dof_node6) ||
      !upload(B, &b.info, B->info) || !upload(B, &b.params, params) || !upload(B, &b.step_params, step_params) ||
      !upload(B, &b.loads, loads) || !upload(B, &b.pp_elem, pp_elem) || !upload(B, &b.pp_table, pp_table) ||
      !upload(B, &b.pp_aint, pp_aint) || !upload(B, &b.mon_node, mon_node) ||
      !upload(B, &b.mon_struct, mon_struct) || !upload(B, &b.mon_adj_off, mon_adj_off) ||
      !upload(B, &b.mon_adj, mon_adj) || !balloc(B, &b.mon_load, (size_t)b.mon_total * 6) ||
      !balloc(B, &b.mon_rec, (size_t)b.mon_total * b.mon_cap * 25) ||
      !upload(B, &b.disps, disps) || !upload(B, &b.tables, tables) || !upload(B, &b.table_data, tdata) ||
      !dup(B, &B->copy0, b.copy, copy.size()) || !dup(B, &B->Qn0, b.Qn, Qn.size()) ||
      !dup(B, &B->bhist0, b.bhist, bhist.size()) || !dup(B, &B->baux0, b.baux, baux.size()))
    return GF_ERR_CUDA;
  if (!balloc(B, &b.P, (size_t)dof_off) || !balloc(B, &b.y, (size_t)dof_off) ||
      !balloc(B, &b.band, (size_t)dof_off * GF_LDB) || !balloc(B, &b.U, (size_t)dof_off * GF_UW) ||
      !balloc(B, &b.state, (size_t)n) || !balloc(B, &b.running, 1) ||
      !balloc(B, &b.Ke, (size_t)elem_off * 324) || !balloc(B, &b.Fe, (size_t)elem_off * 18) ||
      !balloc(B, &b.nodeK, (size_t)std::max(node_off, 1) * 9) ||
      !balloc(B, &b.RD, b.any_rayleigh ? (size_t)elem_off * 324 : 1) ||
      !balloc(B, &b.Dm, b.any_dynamic ? (size_t)elem_off * 18 : 1))
    return GF_ERR_CUDA;
  // reduction chunks of k_residual / k_update
  {
    std::vector<int> cs, c0;
    for (int s = 0; s < n; ++s) {
      const int nf = B->info[s].n_free, nch = nf > 0 ? (nf + GF_RED_CHUNK - 1) / GF_RED_CHUNK : 1;
      for (int k = 0; k < nch; ++k) {
        cs.push_back(s);
        c0.push_back(k * GF_RED_CHUNK);
      }
    }
    b.n_chunks = (int)cs.size();
    if (!upload(B, &b.chunk_struct, cs) || !upload(B, &b.chunk_start, c0) || !zeroed(B, &b.red, (size_t)n))
      return GF_ERR_CUDA;
  }
  b.full_band = 0;
  b.xref = B->copy0;
  if (B->count_only) return GF_OK;
  B->h_gl = std::move(gl);
  B->h_enodes = std::move(enodes);
  B->h_snodes = std::move(snodes);
  CK(cudaMemsetAsync(b.band, 0, sizeof(double) * (size_t)std::max(dof_off, 1) * GF_LDB, B->stream));
  CK(cudaMemsetAsync(b.P, 0, sizeof(double) * (size_t)std::max(dof_off, 1), B->stream));
  CK(cudaMemsetAsync(b.nodeK, 0, sizeof(double) * (size_t)std::max(node_off, 1) * 9, B->stream));
  b.mixed = B->opts.precision == GF_PREC_MIXED;
  b.sh.ir_max = B->opts.max_refine > 0 ? B->opts.max_refine : GF_IR_MAX;
  b.sh.wide_tc = b.sh.oz_slices != nullptr ? B->opts.wide_update : GF_WIDE_FP64;
  if (b.sh.n_wide) {
    // tile shapes: the caller's entries, the others from the autotuner
    // (served waves, whose device memory comes from the server's budget,
    // take the defaults rather than time a synthetic band beside it)
    const int* wt = B->opts.wide_tiles;
    WideTiles t;
    if (!(wt[0] && wt[1] && wt[2] && wt[3]) && !B->arena) t = tune_wide_tiles(B->ctx, b.sh.max_kl, b.sh.wide_tc);
    if (wt[0]) t.trsm_rb = wt[0];
    if (wt[1]) t.trsm_first = wt[1];
    if (wt[2]) t.corner = wt[2];
    if (wt[3]) t.sub_rows = wt[3];
    b.sh.tiles = t;
  }
  return GF_OK;
}

int count_launches_per_pass(const gf_batch* B) {
  int colors = 0;
  for (int c = 0; c < B->b.n_colors; ++c) colors += B->b.color_off[c + 1] > B->b.color_off[c];
  const ChainData& cd = B->b.chain;
  // chains only: one gather launch in place of the colour passes
  if (B->b.n_elem && !B->b.full_band && cd.n_chain_elems == B->b.n_elem) colors = 1;
  int chain_launches = 0;
  if (cd.n_chain_elems) {
    chain_launches = 2;
    if (cd.n_corners) {
      chain_launches += 3;
      for (int l = 0; l < cd.n_levels; ++l)
        chain_launches += 2 * (cd.odd_off[l + 1] > cd.odd_off[l]) + (cd.even_off[l + 1] > cd.even_off[l]);
    }
  }
  return 10 + colors + chain_launches + shell_launches_per_pass(B->b) + (B->b.any_rayleigh ? 1 : 0) +
         (B->b.n_pipe_press ? 1 : 0) + (B->b.mon_total ? 1 : 0);
}

int batch_reset(gf_batch* B) {
  gf_ctx* ctx = B->ctx;
  Batch& b = B->b;
  cudaStream_t st = B->stream;
  CK(cudaMemcpyAsync(b.copy, B->copy0, sizeof(double) * (size_t)b.n_nodes * 6, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(b.Qn, B->Qn0, sizeof(double) * (size_t)b.n_nodes * 9, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(b.bhist, B->bhist0, sizeof(BeamHist) * (size_t)b.n_elem, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(b.baux, B->baux0, sizeof(BeamHistAux) * (size_t)b.n_elem, cudaMemcpyDeviceToDevice, st));
  if (b.sh.n_shells) {
    CK(cudaMemcpyAsync(b.sh.shist, B->shist0, sizeof(ShellHist) * (size_t)b.sh.n_shells, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(b.sh.saux, B->saux0, sizeof(ShellHistAux) * (size_t)b.sh.n_shells, cudaMemcpyDeviceToDevice, st));
  }
  const size_t n6 = sizeof(double) * (size_t)std::max(b.n_nodes, 1) * 6;
  CK(cudaMemsetAsync(b.disp, 0, n6, st));
  CK(cudaMemsetAsync(b.vel, 0, n6, st));
  CK(cudaMemsetAsync(b.accel, 0, n6, st));
  CK(cudaMemsetAsync(b.copy_vel, 0, n6, st));
  CK(cudaMemsetAsync(b.copy_accel, 0, n6, st));
  if (b.mon_total) CK(cudaMemsetAsync(b.mon_load, 0, sizeof(double) * (size_t)b.mon_total * 6, st));
  launch_init_state(b, st);
  CK(cudaGetLastError());
  return GF_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

gf_ctx* gf_create(int device) {
  gf_ctx* ctx = new gf_ctx();
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return nullptr;
  }
  return ctx;
}

void gf_destroy(gf_ctx* ctx) {
  if (!ctx) return;
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->pin) cudaFreeHost(ctx->pin);
  delete ctx;
}

const char* gf_last_error(const gf_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int gf_ctx_set_opts(gf_ctx* ctx, const gf_solve_opts* opts) {
  if (!ctx || !opts ||
      (opts->wide_update != GF_WIDE_FP64 && opts->wide_update != GF_WIDE_TENSOR &&
       opts->wide_update != GF_WIDE_TENSOR_SYNC)) {
    set_err(ctx, "gf_ctx_set_opts: invalid arguments");
    return GF_ERR_ARG;
  }
  ctx->wide_update = opts->wide_update;
  return GF_OK;
}

void gf_default_opts(gf_solve_opts* o) {
  o->precision = GF_PREC_FP64;
  o->poll_every = 8;
  o->use_graph = 1;
  o->wide_update = GF_WIDE_TENSOR;
  o->max_passes = 0;
  o->monitor_rows = 0;
  o->max_refine = 0;
  for (int& t : o->wide_tiles) t = 0;
}

gf_batch* gf_batch_create(gf_ctx* ctx, int n, const gf_model_desc* models, const gf_solve_opts* opts) {
  if (!ctx || n <= 0 || !models) {
    set_err(ctx, "gf_batch_create: invalid arguments");
    return nullptr;
  }
  cudaSetDevice(ctx->device);
  gf_batch* B = new gf_batch();
  B->ctx = ctx;
  B->stream = ctx->stream;
  if (opts) B->opts = *opts; else gf_default_opts(&B->opts);
  if (B->opts.poll_every <= 0) B->opts.poll_every = 8;
  NvtxRange range("gf_batch_create");
  const double t0 = host_now_ms();
  if (build_batch(B, n, models) != GF_OK || cudaMallocHost(&B->h_running, sizeof(int)) != cudaSuccess ||
      cudaEventCreate(&B->ev0) != cudaSuccess || cudaEventCreate(&B->ev1) != cudaSuccess) {
    std::string e = ctx->err;
    gf_batch_destroy(B);
    ctx->err = e.empty() ? "gf_batch_create failed" : e;
    return nullptr;
  }
  B->launches_per_pass = count_launches_per_pass(B);
  B->host_ms[0] = host_now_ms() - t0 - B->host_ms[1] - B->host_ms[2];
  return B;
}

void gf_batch_destroy(gf_batch* B) {
  if (!B) return;
  if (B->graph) cudaGraphExecDestroy(B->graph);
  for (auto& a : B->b.sh.aux)
    if (a) cudaStreamDestroy(a);
  for (auto& e : B->b.sh.evt)
    if (e) cudaEventDestroy(e);
  for (void* p : B->allocs) {
    if (B->arena) B->arena->release(p);
    else cudaFree(p);
  }
  if (B->h_running) cudaFreeHost(B->h_running);
  if (B->ev0) cudaEventDestroy(B->ev0);
  if (B->ev1) cudaEventDestroy(B->ev1);
  delete B;
}

int gf_batch_reset(gf_batch* B) {
  if (!B) return GF_ERR_ARG;
  gf_ctx* ctx = B->ctx;
  int r = batch_reset(B);
  if (r != GF_OK) return r;
  CK(cudaStreamSynchronize(B->stream));
  return GF_OK;
}

}  // extern "C"

namespace gfh {
int ensure_graph(gf_batch* B) {
  gf_ctx* ctx = B->ctx;
  cudaStream_t st = B->stream;
  if (B->opts.use_graph && !B->graph) {
    NvtxRange range("capture Newton pass");
    const double t0 = host_now_ms();
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    wide_capture_error();  // clear
    launch_iteration(B->b, st);
    const cudaError_t ce = wide_capture_error();
    CK(cudaStreamEndCapture(st, &g));
    if (ce != cudaSuccess) {
      cudaGraphDestroy(g);
      set_err(ctx, "capture of the wide-band loops failed: %s", cudaGetErrorString(ce));
      return GF_ERR_CUDA;
    }
    // per-node priorities (the wide-band LU's critical-path kernels) in a
    // batch's own graph; a served wave's graph runs at its stream's priority,
    // which orders the waves against each other
    CK(cudaGraphInstantiate(&B->graph, g, B->arena ? 0 : cudaGraphInstantiateFlagUseNodePriority));
    CK(cudaGraphDestroy(g));
    B->host_ms[3] = host_now_ms() - t0;
  }
  return GF_OK;
}

// Launches Newton passes until no structure is running; polls the device
// every opts.poll_every passes.
int run_passes(gf_batch* B, long long* passes_out, LaunchProf* prof = nullptr) {
  gf_ctx* ctx = B->ctx;
  cudaStream_t st = B->stream;
  const Batch& b = B->b;
  long long passes = 0;
  const long long cap = B->opts.max_passes > 0 ? B->opts.max_passes : 4000000;
  for (;;) {
    for (int k = 0; k < B->opts.poll_every; ++k) {
      if (B->graph && !prof) {
        CK(cudaGraphLaunch(B->graph, st));
      } else {
        launch_iteration(b, st, true, prof);
      }
      ++passes;
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(B->h_running, b.running, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (*B->h_running == 0) break;
    if (passes >= cap) {
      set_err(ctx, "gf_batch_run: %lld Newton passes without completion", passes);
      return GF_ERR_TIMEOUT;
    }
  }
  *passes_out = passes;
  return GF_OK;
}
}  // namespace gfh

// Launches of the mixed path's refinement sweeps and FP64 fallbacks since
// the last call, from the device counters (the stream is idle here).
static long long refine_launches(gf_batch* B) {
  const int* cnt = B->b.sh.ir_more;
  if (!cnt) return 0;
  int c[4];
  if (cudaMemcpy(c, cnt, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
  const long long n = gf::wide_refine_launches(B->b, c[2] - B->ir_seen[0], c[3] - B->ir_seen[1]);
  B->ir_seen[0] = c[2];
  B->ir_seen[1] = c[3];
  return n;
}

extern "C" {

int gf_batch_run(gf_batch* B) {
  if (!B) return GF_ERR_ARG;
  NvtxRange range("gf_batch_run");
  gf_ctx* ctx = B->ctx;
  cudaStream_t st = B->stream;
  int r = ensure_graph(B);
  if (r != GF_OK) return r;
  CK(cudaEventRecord(B->ev0, st));
  long long passes = 0;
  r = run_passes(B, &passes);
  if (r != GF_OK) return r;
  CK(cudaEventRecord(B->ev1, st));
  CK(cudaEventSynchronize(B->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, B->ev0, B->ev1));
  B->last_ms = ms;
  B->last_launches = passes * B->launches_per_pass + refine_launches(B);
  return GF_OK;
}

int gf_batch_step(gf_batch* B, int max_passes, int* running) {
  if (!B || max_passes <= 0) return GF_ERR_ARG;
  gf_ctx* ctx = B->ctx;
  cudaStream_t st = B->stream;
  int r = ensure_graph(B);
  if (r != GF_OK) return r;
  for (int k = 0; k < max_passes; ++k) {
    if (B->graph) {
      CK(cudaGraphLaunch(B->graph, st));
    } else {
      launch_iteration(B->b, st);
    }
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(B->h_running, B->b.running, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (running) *running = *B->h_running;
  return GF_OK;
}

}  // extern "C"

namespace {
// The device state a batch carries from one Newton pass to the next: nodal
// increments, configurations, velocities and accelerations (current and
// converged), Gauss-point histories, the per-structure step machine, and
// the Rayleigh matrices when they are formed once per step.  Everything
// else is rebuilt by every pass.
std::vector<std::pair<void*, size_t>> state_parts(const gf_batch* B) {
  const Batch& b = B->b;
  const size_t nn = (size_t)b.n_nodes, ne = (size_t)b.n_elem, ns = (size_t)b.sh.n_shells;
  std::vector<std::pair<void*, size_t>> v = {
      {b.disp, 8 * 6 * nn},      {b.copy, 8 * 6 * nn},      {b.Qn, 8 * 9 * nn},
      {b.vel, 8 * 6 * nn},       {b.accel, 8 * 6 * nn},     {b.copy_vel, 8 * 6 * nn},
      {b.copy_accel, 8 * 6 * nn}, {b.bhist, sizeof(BeamHist) * ne}, {b.baux, sizeof(BeamHistAux) * ne},
      {b.state, sizeof(StructState) * (size_t)b.n_struct}, {b.params, sizeof(StructParams) * (size_t)b.n_struct}};
  if (ns) {
    v.push_back({b.sh.shist, sizeof(ShellHist) * ns});
    v.push_back({b.sh.saux, sizeof(ShellHistAux) * ns});
  }
  if (b.any_rayleigh) v.push_back({b.RD, 8 * 324 * ne});
  if (b.sh.any_rayleigh) v.push_back({b.sh.RD, 8 * 729 * ns});
  return v;
}

// Header at the start of a snapshot: what the batch's layout depends on,
// so a snapshot is restored only into a batch laid out the same way.
struct SnapshotHeader {
  unsigned long long magic;  // kSnapshotMagic
  unsigned version;
  int n_struct;
  long long n_nodes, n_elem, n_shells;
  int rayleigh_beam, rayleigh_shell;
  unsigned long long total_bytes;  // header included
};
constexpr unsigned long long kSnapshotMagic = 0x50414e5346524947ull;  // "GIRFSNAP"
constexpr unsigned kSnapshotVersion = 1;

SnapshotHeader snapshot_header(const gf_batch* B) {
  const Batch& b = B->b;
  SnapshotHeader h{};
  h.magic = kSnapshotMagic;
  h.version = kSnapshotVersion;
  h.n_struct = b.n_struct;
  h.n_nodes = b.n_nodes;
  h.n_elem = b.n_elem;
  h.n_shells = b.sh.n_shells;
  h.rayleigh_beam = b.any_rayleigh ? 1 : 0;
  h.rayleigh_shell = b.sh.any_rayleigh ? 1 : 0;
  size_t n = sizeof(SnapshotHeader);
  for (const auto& p : state_parts(B)) n += p.second;
  h.total_bytes = n;
  return h;
}
}  // namespace

extern "C" {

int gf_batch_snapshot_bytes(const gf_batch* B, size_t* bytes) {
  if (!B || !bytes) return GF_ERR_ARG;
  *bytes = (size_t)snapshot_header(B).total_bytes;
  return GF_OK;
}

int gf_batch_snapshot(gf_batch* B, void* host) {
  if (!B || !host) return GF_ERR_ARG;
  gf_ctx* ctx = B->ctx;
  const SnapshotHeader hd = snapshot_header(B);
  std::memcpy(host, &hd, sizeof(hd));
  char* h = static_cast<char*>(host) + sizeof(hd);
  for (const auto& p : state_parts(B)) {
    if (p.second) CK(cudaMemcpyAsync(h, p.first, p.second, cudaMemcpyDeviceToHost, B->stream));
    h += p.second;
  }
  CK(cudaStreamSynchronize(B->stream));
  return GF_OK;
}

int gf_batch_restore(gf_batch* B, const void* host) {
  if (!B || !host) return GF_ERR_ARG;
  gf_ctx* ctx = B->ctx;
  SnapshotHeader got;
  std::memcpy(&got, host, sizeof(got));
  const SnapshotHeader want = snapshot_header(B);
  if (got.magic != kSnapshotMagic || got.version != kSnapshotVersion) {
    set_err(ctx, "gf_batch_restore: not a batch snapshot (bad magic or version)");
    return GF_ERR_ARG;
  }
  if (got.n_struct != want.n_struct || got.n_nodes != want.n_nodes || got.n_elem != want.n_elem ||
      got.n_shells != want.n_shells || got.rayleigh_beam != want.rayleigh_beam ||
      got.rayleigh_shell != want.rayleigh_shell || got.total_bytes != want.total_bytes) {
    set_err(ctx, "gf_batch_restore: snapshot of a different batch (structures %d/%d, nodes %lld/%lld, "
                 "elements %lld/%lld, shells %lld/%lld, bytes %llu/%llu)",
            got.n_struct, want.n_struct, got.n_nodes, want.n_nodes, got.n_elem, want.n_elem, got.n_shells,
            want.n_shells, got.total_bytes, want.total_bytes);
    return GF_ERR_ARG;
  }
  const char* h = static_cast<const char*>(host) + sizeof(got);
  for (const auto& p : state_parts(B)) {
    if (p.second) CK(cudaMemcpyAsync(p.first, h, p.second, cudaMemcpyHostToDevice, B->stream));
    h += p.second;
  }
  CK(cudaStreamSynchronize(B->stream));
  return GF_OK;
}

int gf_batch_solve_timed(gf_batch* B, int steps, double* ms_out) {
  if (!B || steps <= 0) return GF_ERR_ARG;
  gf_ctx* ctx = B->ctx;
  cudaStream_t st = B->stream;
  int r = ensure_graph(B);
  if (r != GF_OK) return r;
  long long launches = 0;
  CK(cudaEventRecord(B->ev0, st));
  for (int k = 0; k < steps; ++k) {
    r = batch_reset(B);
    if (r != GF_OK) return r;
    long long passes = 0;
    r = run_passes(B, &passes);
    if (r != GF_OK) return r;
    launches += passes * B->launches_per_pass + 1;
  }
  CK(cudaEventRecord(B->ev1, st));
  CK(cudaEventSynchronize(B->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, B->ev0, B->ev1));
  *ms_out = ms;
  B->last_ms = ms / steps;
  B->last_launches = launches + refine_launches(B);
  return GF_OK;
}

static_assert(GF_N_KERNELS == KC_COUNT, "the ABI's kernel class count");

int gf_batch_profile(gf_batch* B, double* ms_out, long long* launches_out) {
  if (!B) return GF_ERR_ARG;
  gf_ctx* ctx = B->ctx;
  cudaStream_t st = B->stream;
  int r = batch_reset(B);
  if (r != GF_OK) return r;
  const int cap = 1 << 18;
  std::vector<cudaEvent_t> ev(2 * cap);
  std::vector<int> cls(cap);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  LaunchProf prof{ev.data(), cls.data(), cap, 0};
  long long passes = 0;
  r = run_passes(B, &passes, &prof);
  CK(cudaStreamSynchronize(st));
  for (int k = 0; k < GF_N_KERNELS; ++k) { ms_out[k] = 0.0; launches_out[k] = 0; }
  for (int i = 0; i < prof.n; ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
    ms_out[cls[i]] += ms;
    launches_out[cls[i]] += 1;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (r != GF_OK) return r;
  if (prof.n >= cap) {
    set_err(ctx, "gf_batch_profile: more than %d launches", cap);
    return GF_ERR_ARG;
  }
  return GF_OK;
}

const char* gf_kernel_name(int k) { return kernel_class_name(k); }

int gf_batch_bytes(const gf_batch* B, long long* h2d, long long* d2h) {
  if (!B) return GF_ERR_ARG;
  if (h2d) *h2d = B->h2d_bytes;
  if (d2h) *d2h = (long long)B->b.n_nodes * 15 * (long long)sizeof(double) +
                  (long long)B->b.n_struct * (long long)sizeof(StructState);
  return GF_OK;
}

int gf_batch_work(const gf_batch* B, double* lu_flops, double* asm_bytes, double* mount_flops) {
  if (!B) return GF_ERR_ARG;
  gf_ctx* ctx = B->ctx;
  const Batch& b = B->b;
  int n = b.n_struct;
  std::vector<StructState> st(n);
  CK(cudaMemcpy(st.data(), b.state, sizeof(StructState) * n, cudaMemcpyDeviceToHost));
  double lu = 0, ab = 0, mf = 0;
  for (int s = 0; s < n; ++s) {
    const StructInfo& inf = B->info[s];
    double nf = inf.n_free, kl = B->kb[s];
    if (inf.wide) kl = inf.wkl;
    lu += st[s].n_solves * (2.0 * nf * kl * kl + 2.0 * nf * (kl + kl));
    ab += st[s].total_it * 8.0 * (6.0 * inf.n_nodes + 80.0 * inf.n_elem + (2 * kl + 1) * nf + nf);
    mf += st[s].total_it * (double)inf.n_elem * GF_BEAM_MOUNT_FLOPS;
  }
  if (lu_flops) *lu_flops = lu;
  if (asm_bytes) *asm_bytes = ab;
  if (mount_flops) *mount_flops = mf;
  return GF_OK;
}

int gf_device_fp_peaks(gf_ctx* ctx, double* fp64_tflops, double* fp32_tflops) {
  if (!ctx) return GF_ERR_ARG;
  cudaStream_t st = ctx->stream;
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  int blocks = sms * 8, threads = 256;
  void* out = nullptr;
  CK(cudaMalloc(&out, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int pass = 0; pass < 2; ++pass) {
    bool f64 = pass == 0;
    int iters = f64 ? 2048 : 65536;
    launch_fp_probe(f64, out, blocks, threads, 64, st);  // warm-up
    cudaEventRecord(e0, st);
    launch_fp_probe(f64, out, blocks, threads, iters, st);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    double tf = 2.0 * 8 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
    if (f64 && fp64_tflops) *fp64_tflops = tf;
    if (!f64 && fp32_tflops) *fp32_tflops = tf;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  CK(cudaGetLastError());
  return GF_OK;
}

double gf_batch_last_ms(const gf_batch* B) { return B ? B->last_ms : 0.0; }
long long gf_batch_last_launches(const gf_batch* B) { return B ? B->last_launches : 0; }

int gf_batch_results(gf_batch* B, double* const* final_nodes, gf_stats* stats) {
  if (!B) return GF_ERR_ARG;
  gf_ctx* ctx = B->ctx;
  const Batch& b = B->b;
  NvtxRange range("gf_batch_results");
  const double t0 = host_now_ms();
  int n = b.n_struct;
  std::vector<StructState> st(n);
  CK(cudaMemcpy(st.data(), b.state, sizeof(StructState) * n, cudaMemcpyDeviceToHost));
  if (stats)
    for (int s = 0; s < n; ++s) {
      gf_stats z{};
      z.converged_steps = st[s].converged_number;
      z.newton_iterations = st[s].total_it;
      z.bisections = st[s].bisections;
      z.aborted = st[s].phase == PH_ABORTED || st[s].aborted;
      z.linear_solves = st[s].n_solves;
      z.refine_sweeps = st[s].ir_sweeps;
      z.fp64_fallbacks = st[s].ir_fallbacks;
      stats[s] = z;
    }
  if (final_nodes) {
    // through the context's pinned staging (a pageable copy when none)
    const size_t nc = (size_t)b.n_nodes * 6, nq = (size_t)b.n_nodes * 9;
    hvec<double> hc, hq;
    double* copy = static_cast<double*>(ctx->pinned(sizeof(double) * (nc + nq)));
    double* Qn = copy ? copy + nc : nullptr;
    if (!copy) {
      hc.resize(nc);
      hq.resize(nq);
      copy = hc.data();
      Qn = hq.data();
    }
    CK(cudaMemcpyAsync(copy, b.copy, sizeof(double) * nc, cudaMemcpyDeviceToHost, B->stream));
    CK(cudaMemcpyAsync(Qn, b.Qn, sizeof(double) * nq, cudaMemcpyDeviceToHost, B->stream));
    CK(cudaStreamSynchronize(B->stream));
    parallel_structures(n, (size_t)b.n_nodes, [&](int s) {
      double* o = final_nodes[s];
      if (!o) return;
      const StructInfo& inf = B->info[s];
      const double* x = &copy[(size_t)inf.node_off * 6];
      const double* q = &Qn[(size_t)inf.node_off * 9];
      for (int i = 0; i < inf.n_nodes; ++i) {
        for (int k = 0; k < 6; ++k) o[15 * i + k] = x[6 * i + k];
        for (int k = 0; k < 9; ++k) o[15 * i + 6 + k] = q[9 * i + k];
      }
    });
  }
  B->host_ms[4] = host_now_ms() - t0;
  return GF_OK;
}

int gf_batch_wide_tiles(const gf_batch* B, int* tiles) {
  if (!B || !tiles) return GF_ERR_ARG;
  const WideTiles& t = B->b.sh.tiles;
  const bool w = B->b.sh.n_wide > 0;
  tiles[0] = w ? t.trsm_rb : 0;
  tiles[1] = w ? t.trsm_first : 0;
  tiles[2] = w ? t.corner : 0;
  tiles[3] = w ? t.sub_rows : 0;
  return GF_OK;
}

int gf_batch_monitor(gf_batch* B, int s, double* out, int* dims) {
  if (!B || !dims || s < 0 || s >= B->b.n_struct) return GF_ERR_ARG;
  gf_ctx* ctx = B->ctx;
  const StructInfo& inf = B->info[s];
  StructState st{};
  GF_CK(cudaMemcpy(&st, B->b.state + s, sizeof(st), cudaMemcpyDeviceToHost));
  const int made = inf.mon_n ? st.mon_rows : 0, kept = std::min(made, B->b.mon_cap);
  dims[0] = inf.mon_n;
  dims[1] = inf.mon_n ? 1 + kept : 0;
  dims[2] = inf.mon_n ? 1 + made : 0;
  if (!out || !inf.mon_n) return GF_OK;
  std::vector<double> rec((size_t)inf.mon_n * B->b.mon_cap * 25);
  GF_CK(cudaMemcpy(rec.data(), B->b.mon_rec + (size_t)inf.mon_off * B->b.mon_cap * 25, sizeof(double) * rec.size(),
                   cudaMemcpyDeviceToHost));
  const int rows = 1 + kept;
  for (int q = 0; q < inf.mon_n; ++q) {
    const double* first = &B->mon_first[4 * (size_t)(inf.mon_off + q)];
    double* o = out + (size_t)q * rows * 31;
    std::memset(o, 0, sizeof(double) * 31);
    o[0] = first[3];
    for (int k = 0; k < 3; ++k) o[1 + k] = first[k];
    for (int r = 0; r < kept; ++r) {
      const double* x = &rec[((size_t)q * B->b.mon_cap + r) * 25];
      double* L = o + (size_t)(r + 1) * 31;
      L[0] = x[0];
      for (int k = 0; k < 3; ++k) L[1 + k] = x[1 + k];
      // the Euler rotation vector of the accumulated Rodrigues vector
      // (reference src/Node.cpp:350-358)
      const double an = std::sqrt(x[4] * x[4] + x[5] * x[5] + x[6] * x[6]);
      const double th = 2.0 * std::atan(an / 2.0);
      for (int k = 0; k < 3; ++k) L[4 + k] = an != 0.0 ? (th / an) * x[4 + k] : 0.0;
      for (int k = 0; k < 6; ++k) L[7 + k] = L[13 + k] = x[7 + k];
      for (int k = 0; k < 6; ++k) L[19 + k] = x[13 + k];
      for (int k = 0; k < 6; ++k) L[25 + k] = x[19 + k];
    }
  }
  return GF_OK;
}

int gf_batch_host_ms(const gf_batch* B, double* ms, int n) {
  if (!B || !ms || n < 0) return GF_ERR_ARG;
  for (int i = 0; i < n && i < 5; ++i) ms[i] = B->host_ms[i];
  return GF_OK;
}

}  // extern "C"

namespace {
// The first Newton pass of structure s from its initial configuration, read
// back: K_AA in the solver's band layout (leading dimension W, half
// bandwidth kw) and P_A, both in the solver's numbering.
}  // namespace

namespace gfh {
// The CSR pattern of structure s's K_AA in the reference's free-DOF
// numbering: row i holds the sorted columns j that some element couples to
// i (the union of every element's free-DOF pattern, as SparseMatrix::setValue
// of every element entry followed by setFromTriplets).  Returns nnz.
int64_t csr_rows(const gf_batch* B, int s, std::vector<std::vector<int>>& rows) {
  const StructInfo& inf = B->info[s];
  const int nf = inf.n_free;
  const std::vector<int>& perm = B->perm[s];
  std::vector<int> inv(nf);  // solver index -> the reference's index
  for (int i = 0; i < nf; ++i) inv[perm.empty() ? i : perm[i]] = i;
  rows.assign(nf, {});
  auto add_elem = [&](const int* dofs, int nd) {
    for (int a = 0; a < nd; ++a) {
      if (dofs[a] < 0) continue;
      for (int c = 0; c < nd; ++c)
        if (dofs[c] >= 0) rows[inv[dofs[a]]].push_back(inv[dofs[c]]);
    }
  };
  for (int e = inf.elem_off; e < inf.elem_off + inf.n_elem; ++e) {
    int d[18];
    for (int a = 0; a < 18; ++a) d[a] = B->h_gl[(size_t)B->h_enodes[3 * e + a / 6] * 6 + a % 6];
    add_elem(d, 18);
  }
  int s_lo = B->shell_off[s];
  int s_hi = s + 1 < (int)B->shell_off.size() ? B->shell_off[s + 1] : B->b.sh.n_shells;
  for (int e = s_lo; e < s_hi; ++e) {
    int d[27];
    for (int a = 0; a < 18; ++a) d[a] = B->h_gl[(size_t)B->h_snodes[6 * e + a / 3] * 6 + a % 3];
    for (int a = 0; a < 9; ++a) d[18 + a] = B->h_gl[(size_t)B->h_snodes[6 * e + 3 + a / 3] * 6 + 3 + a % 3];
    add_elem(d, 27);
  }
  int64_t nnz = 0;
  for (auto& r : rows) {
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    nnz += (int64_t)r.size();
  }
  return nnz;
}
}  // namespace gfh

namespace {
int first_pass_band(gf_batch* B, int s, std::vector<double>& band, std::vector<double>& P, int64_t& W,
                    int64_t& kw) {
  gf_ctx* ctx = B->ctx;
  const Batch& b = B->b;
  const StructInfo& inf = B->info[s];
  int r = batch_reset(B);
  if (r != GF_OK) return r;
  // one partial pass: step start, zero, mount, loads, residual
  Batch bb = b;
  launch_iteration_partial(bb, B->stream);
  CK(cudaGetLastError());
  const int nf = inf.n_free;
  W = inf.wide ? 2 * (int64_t)inf.wkl + 1 : GF_LDB;
  kw = inf.wide ? inf.wkl : GF_KB;
  band.assign((size_t)nf * W, 0.0);
  P.assign(nf, 0.0);
  const double* src = inf.wide ? b.sh.wband + inf.wb_off : b.band + inf.band_off;
  CK(cudaMemcpyAsync(band.data(), src, sizeof(double) * band.size(), cudaMemcpyDeviceToHost, B->stream));
  CK(cudaMemcpyAsync(P.data(), b.P + inf.dof_off, sizeof(double) * P.size(), cudaMemcpyDeviceToHost, B->stream));
  CK(cudaStreamSynchronize(B->stream));
  return batch_reset(B) == GF_OK ? GF_OK : GF_ERR_CUDA;
}
}  // namespace

extern "C" {

int gf_batch_assemble(gf_batch* B, int s, double* ab, double* PA, int* dims) {
  if (!B || s < 0 || s >= B->b.n_struct) return GF_ERR_ARG;
  const StructInfo& inf = B->info[s];
  int kb = B->kb[s];
  if (dims) { dims[0] = inf.n_free; dims[1] = kb; }
  if (!ab && !PA) return GF_OK;
  std::vector<double> band, P;
  int64_t W = 0, kw = 0;
  int r = first_pass_band(B, s, band, P, W, kw);
  if (r != GF_OK) return r;
  const int nf = inf.n_free;
  // the reference's numbering: identity, or back from the solver's
  // reverse Cuthill-McKee numbering for wide structures
  const std::vector<int>& perm = B->perm[s];
  auto pm = [&](int i) { return perm.empty() ? i : perm[i]; };
  int ldab = 3 * kb + 1;
  if (ab) {
    std::memset(ab, 0, sizeof(double) * (size_t)ldab * nf);
    for (int j = 0; j < nf; ++j)
      for (int i = std::max(0, j - kb); i <= std::min(nf - 1, j + kb); ++i) {
        int64_t pi = pm(i), pj = pm(j);
        if (std::llabs(pi - pj) > kw) continue;
        ab[(size_t)(2 * kb + i - j) + (size_t)j * ldab] = band[(size_t)(kw + pi - pj) + (size_t)pj * W];
      }
  }
  if (PA)
    for (int i = 0; i < nf; ++i) PA[i] = P[pm(i)];
  return GF_OK;
}

int gf_batch_assemble_csr(gf_batch* B, int s, int* row_ptr, int* col_idx, double* val, double* PA, int* dims) {
  if (!B || s < 0 || s >= B->b.n_struct) return GF_ERR_ARG;
  gf_ctx* ctx = B->ctx;
  if (B->h_gl.empty()) {
    set_err(ctx, "gf_batch_assemble_csr: the batch keeps no host numbering");
    return GF_ERR_ARG;
  }
  const StructInfo& inf = B->info[s];
  const int nf = inf.n_free;
  const std::vector<int>& perm = B->perm[s];
  std::vector<std::vector<int>> rows;
  int64_t nnz = csr_rows(B, s, rows);
  if (nnz > INT32_MAX) {
    set_err(ctx, "gf_batch_assemble_csr: %lld nonzeros exceed 32-bit CSR indices", (long long)nnz);
    return GF_ERR_ARG;
  }
  if (dims) { dims[0] = nf; dims[1] = (int)nnz; }
  if (!row_ptr && !col_idx && !val && !PA) return GF_OK;
  std::vector<double> band, P;
  int64_t W = 0, kw = 0;
  int r = first_pass_band(B, s, band, P, W, kw);
  if (r != GF_OK) return r;
  int64_t q = 0;
  for (int i = 0; i < nf; ++i) {
    if (row_ptr) row_ptr[i] = (int)q;
    int64_t pi = perm.empty() ? i : perm[i];
    for (int j : rows[i]) {
      int64_t pj = perm.empty() ? j : perm[j];
      if (col_idx) col_idx[q] = j;
      if (val) val[q] = std::llabs(pi - pj) <= kw ? band[(size_t)(kw + pi - pj) + (size_t)pj * W] : 0.0;
      ++q;
    }
  }
  if (row_ptr) row_ptr[nf] = (int)q;
  if (PA)
    for (int i = 0; i < nf; ++i) PA[i] = P[perm.empty() ? i : perm[i]];
  return GF_OK;
}

int gf_solve(gf_ctx* ctx, int n, const gf_model_desc* models, const gf_solve_opts* opts, double* const* final_nodes,
             gf_stats* stats) {
  gf_batch* B = gf_batch_create(ctx, n, models, opts);
  if (!B) return GF_ERR_ARG;
  int r = gf_batch_reset(B);
  if (r == GF_OK) r = gf_batch_run(B);
  if (r == GF_OK) r = gf_batch_results(B, final_nodes, stats);
  gf_batch_destroy(B);
  return r;
}

int gf_beam_elements(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* sec, const double* cs,
                     int n_hist, const double* hist_disp, const double* disp, double* K, double* f) {
  if (!ctx || n <= 0) return GF_ERR_ARG;
  std::vector<BeamConst> c(n);
  std::vector<BeamHist> h(n);
  std::vector<BeamHistAux> x(n);
  for (int e = 0; e < n; ++e)
    beam_precalc(xyz + 9 * e, xyz + 9 * e + 6, mat + 3 * e, sec + 6 * e, cs + 6 * e, c[e], h[e], x[e]);
  BeamConst* dc = nullptr;
  BeamHist* dh = nullptr;
  BeamHistAux* dx = nullptr;
  double *dd = nullptr, *dK = nullptr, *df = nullptr;
  int rc = GF_OK;
  if (!dmalloc(ctx, &dc, n) || !dmalloc(ctx, &dh, n) || !dmalloc(ctx, &dx, n) || !dmalloc(ctx, &dd, (size_t)n * 18) ||
      !dmalloc(ctx, &dK, (size_t)n * 324) || !dmalloc(ctx, &df, (size_t)n * 18)) {
    rc = GF_ERR_CUDA;
  } else {
    cudaStream_t st = ctx->stream;
    cudaMemcpyAsync(dc, c.data(), sizeof(BeamConst) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dh, h.data(), sizeof(BeamHist) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dx, x.data(), sizeof(BeamHistAux) * n, cudaMemcpyHostToDevice, st);
    std::vector<double> step((size_t)n * 18);
    for (int q = 0; q < n_hist; ++q) {
      for (int e = 0; e < n; ++e)
        std::memcpy(&step[(size_t)e * 18], hist_disp + ((size_t)e * n_hist + q) * 18, 18 * sizeof(double));
      cudaMemcpyAsync(dd, step.data(), sizeof(double) * step.size(), cudaMemcpyHostToDevice, st);
      launch_beam_commit(n, dc, dh, dx, dd, st);
      cudaStreamSynchronize(st);
    }
    cudaMemcpyAsync(dd, disp, sizeof(double) * (size_t)n * 18, cudaMemcpyHostToDevice, st);
    launch_beam_elements(n, dc, dh, dd, dK, df, st);
    cudaMemcpyAsync(K, dK, sizeof(double) * (size_t)n * 324, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(f, df, sizeof(double) * (size_t)n * 18, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_err(ctx, "gf_beam_elements: %s", cudaGetErrorString(e));
      rc = GF_ERR_CUDA;
    }
  }
  cudaFree(dc); cudaFree(dh); cudaFree(dx); cudaFree(dd); cudaFree(dK); cudaFree(df);
  return rc;
}

int gf_shell_elements(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* thick, int n_hist,
                      const double* hist_disp, const double* disp, const double* pressure, int area_update, double* K,
                      double* f) {
  if (!ctx || n <= 0 || !xyz || !mat || !thick || !disp || !K || !f || n_hist < 0 || (n_hist && !hist_disp)) {
    set_err(ctx, "gf_shell_elements: invalid arguments");
    return GF_ERR_ARG;
  }
  std::vector<ShellConst> c(n);
  std::vector<ShellHist> h(n);
  std::vector<ShellHistAux> x(n);
  std::vector<double> pu((size_t)n * 18, 0.0), p(n, std::nan(""));
  for (int e = 0; e < n; ++e) {
    shell_precalc(xyz + 18 * (size_t)e, mat + 3 * (size_t)e, thick[e], c[e], h[e], x[e]);
    for (int a = 0; a < 18; ++a) {
      double v = disp[(size_t)e * 27 + a];
      for (int q = 0; q < n_hist; ++q) v += hist_disp[((size_t)e * n_hist + q) * 27 + a];
      pu[(size_t)e * 18 + a] = v;
    }
    if (pressure) p[e] = pressure[e];
  }
  ShellConst* dc = nullptr;
  ShellHist* dh = nullptr;
  ShellHistAux* dx = nullptr;
  double *dd = nullptr, *dpu = nullptr, *dp = nullptr, *dK = nullptr, *df = nullptr;
  int rc = GF_OK;
  if (!dmalloc(ctx, &dc, n) || !dmalloc(ctx, &dh, n) || !dmalloc(ctx, &dx, n) || !dmalloc(ctx, &dd, (size_t)n * 27) ||
      !dmalloc(ctx, &dpu, (size_t)n * 18) || !dmalloc(ctx, &dp, (size_t)n) || !dmalloc(ctx, &dK, (size_t)n * 729) ||
      !dmalloc(ctx, &df, (size_t)n * 27)) {
    rc = GF_ERR_CUDA;
  } else {
    cudaStream_t st = ctx->stream;
    cudaMemcpyAsync(dc, c.data(), sizeof(ShellConst) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dh, h.data(), sizeof(ShellHist) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dx, x.data(), sizeof(ShellHistAux) * n, cudaMemcpyHostToDevice, st);
    std::vector<double> step((size_t)n * 27);
    for (int q = 0; q < n_hist; ++q) {
      for (int e = 0; e < n; ++e)
        std::memcpy(&step[(size_t)e * 27], hist_disp + ((size_t)e * n_hist + q) * 27, 27 * sizeof(double));
      cudaMemcpyAsync(dd, step.data(), sizeof(double) * step.size(), cudaMemcpyHostToDevice, st);
      launch_shell_commit_elements(n, dc, dh, dx, dd, st);
      cudaStreamSynchronize(st);
    }
    cudaMemcpyAsync(dd, disp, sizeof(double) * (size_t)n * 27, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dpu, pu.data(), sizeof(double) * pu.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dp, p.data(), sizeof(double) * p.size(), cudaMemcpyHostToDevice, st);
    launch_shell_elements(n, dc, dh, dd, dpu, dp, area_update, dK, df, st);
    cudaMemcpyAsync(K, dK, sizeof(double) * (size_t)n * 729, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(f, df, sizeof(double) * (size_t)n * 27, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_err(ctx, "gf_shell_elements: %s", cudaGetErrorString(e));
      rc = GF_ERR_CUDA;
    }
  }
  cudaFree(dc); cudaFree(dh); cudaFree(dx); cudaFree(dd); cudaFree(dpu); cudaFree(dp); cudaFree(dK); cudaFree(df);
  return rc;
}

int gf_shell_inertia_elements(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* thick,
                              int n_hist, const double* hist_disp, const double* disp, const double* vel,
                              const double* acc, double dt, double beta, double gamma, double* M, double* F) {
  if (!ctx || n <= 0 || !xyz || !mat || !thick || !disp || !vel || !acc || !M || !F || n_hist < 0 ||
      (n_hist && !hist_disp) || !(dt > 0.0) || !(beta > 0.0)) {
    set_err(ctx, "gf_shell_inertia_elements: invalid arguments");
    return GF_ERR_ARG;
  }
  std::vector<ShellConst> c(n);
  std::vector<ShellHist> h(n);
  std::vector<ShellHistAux> x(n);
  for (int e = 0; e < n; ++e) shell_precalc(xyz + 18 * (size_t)e, mat + 3 * (size_t)e, thick[e], c[e], h[e], x[e]);
  double a[6] = {1.0 / (dt * dt * beta), 1.0 / (dt * beta), 1.0 / (2.0 * beta) - 1.0, gamma / (dt * beta),
                 1.0 - gamma / beta, dt * (1.0 - gamma / (2.0 * beta))};
  ShellConst* dc = nullptr;
  ShellHist* dh = nullptr;
  ShellHistAux* dx = nullptr;
  double *dd = nullptr, *dv = nullptr, *da = nullptr, *dA = nullptr, *dM = nullptr, *dF = nullptr;
  int rc = GF_OK;
  if (!dmalloc(ctx, &dc, n) || !dmalloc(ctx, &dh, n) || !dmalloc(ctx, &dx, n) || !dmalloc(ctx, &dd, (size_t)n * 27) ||
      !dmalloc(ctx, &dv, (size_t)n * 36) || !dmalloc(ctx, &da, (size_t)n * 36) || !dmalloc(ctx, &dA, 6) ||
      !dmalloc(ctx, &dM, (size_t)n * 729) || !dmalloc(ctx, &dF, (size_t)n * 27)) {
    rc = GF_ERR_CUDA;
  } else {
    cudaStream_t st = ctx->stream;
    cudaMemcpyAsync(dc, c.data(), sizeof(ShellConst) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dh, h.data(), sizeof(ShellHist) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dx, x.data(), sizeof(ShellHistAux) * n, cudaMemcpyHostToDevice, st);
    std::vector<double> step((size_t)n * 27);
    for (int q = 0; q < n_hist; ++q) {
      for (int e = 0; e < n; ++e)
        std::memcpy(&step[(size_t)e * 27], hist_disp + ((size_t)e * n_hist + q) * 27, 27 * sizeof(double));
      cudaMemcpyAsync(dd, step.data(), sizeof(double) * step.size(), cudaMemcpyHostToDevice, st);
      launch_shell_commit_elements(n, dc, dh, dx, dd, st);
      cudaStreamSynchronize(st);
    }
    cudaMemcpyAsync(dd, disp, sizeof(double) * (size_t)n * 27, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dv, vel, sizeof(double) * (size_t)n * 36, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(da, acc, sizeof(double) * (size_t)n * 36, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dA, a, sizeof(a), cudaMemcpyHostToDevice, st);
    launch_shell_inertia_elements(n, dc, dx, dd, dv, da, dA, dM, dF, st);
    cudaMemcpyAsync(M, dM, sizeof(double) * (size_t)n * 729, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(F, dF, sizeof(double) * (size_t)n * 27, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_err(ctx, "gf_shell_inertia_elements: %s", cudaGetErrorString(e));
      rc = GF_ERR_CUDA;
    }
  }
  cudaFree(dc); cudaFree(dh); cudaFree(dx); cudaFree(dd); cudaFree(dv); cudaFree(da); cudaFree(dA);
  cudaFree(dM); cudaFree(dF);
  return rc;
}

int gf_beam_inertia_elements(gf_ctx* ctx, int n, const double* xyz, const double* mat, const double* sec,
                             const double* cs, int n_hist, const double* hist_disp, const double* disp,
                             const double* vel, const double* acc, double dt, double beta, double gamma, double* M,
                             double* F) {
  if (!ctx || n <= 0 || !(dt > 0.0) || !(beta > 0.0)) return GF_ERR_ARG;
  std::vector<BeamConst> c(n);
  std::vector<BeamHist> h(n);
  std::vector<BeamHistAux> x(n);
  for (int e = 0; e < n; ++e)
    beam_precalc(xyz + 9 * e, xyz + 9 * e + 6, mat + 3 * e, sec + 6 * e, cs + 6 * e, c[e], h[e], x[e]);
  double a[6] = {1.0 / (dt * dt * beta), 1.0 / (dt * beta), 1.0 / (2.0 * beta) - 1.0, gamma / (dt * beta),
                 1.0 - gamma / beta, dt * (1.0 - gamma / (2.0 * beta))};
  BeamConst* dc = nullptr;
  BeamHist* dh = nullptr;
  BeamHistAux* dx = nullptr;
  double *dd = nullptr, *dv = nullptr, *da = nullptr, *dA = nullptr, *dM = nullptr, *dF = nullptr;
  int rc = GF_OK;
  if (!dmalloc(ctx, &dc, n) || !dmalloc(ctx, &dh, n) || !dmalloc(ctx, &dx, n) || !dmalloc(ctx, &dd, (size_t)n * 18) ||
      !dmalloc(ctx, &dv, (size_t)n * 18) || !dmalloc(ctx, &da, (size_t)n * 18) || !dmalloc(ctx, &dA, 6) ||
      !dmalloc(ctx, &dM, (size_t)n * 324) || !dmalloc(ctx, &dF, (size_t)n * 18)) {
    rc = GF_ERR_CUDA;
  } else {
    cudaStream_t st = ctx->stream;
    cudaMemcpyAsync(dc, c.data(), sizeof(BeamConst) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dh, h.data(), sizeof(BeamHist) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dx, x.data(), sizeof(BeamHistAux) * n, cudaMemcpyHostToDevice, st);
    std::vector<double> step((size_t)n * 18);
    for (int q = 0; q < n_hist; ++q) {
      for (int e = 0; e < n; ++e)
        std::memcpy(&step[(size_t)e * 18], hist_disp + ((size_t)e * n_hist + q) * 18, 18 * sizeof(double));
      cudaMemcpyAsync(dd, step.data(), sizeof(double) * step.size(), cudaMemcpyHostToDevice, st);
      launch_beam_commit(n, dc, dh, dx, dd, st);
      cudaStreamSynchronize(st);
    }
    cudaMemcpyAsync(dd, disp, sizeof(double) * (size_t)n * 18, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dv, vel, sizeof(double) * (size_t)n * 18, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(da, acc, sizeof(double) * (size_t)n * 18, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dA, a, sizeof(a), cudaMemcpyHostToDevice, st);
    launch_beam_inertia(n, dc, dx, dd, dv, da, dA, dM, dF, st);
    cudaMemcpyAsync(M, dM, sizeof(double) * (size_t)n * 324, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(F, dF, sizeof(double) * (size_t)n * 18, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_err(ctx, "gf_beam_inertia_elements: %s", cudaGetErrorString(e));
      rc = GF_ERR_CUDA;
    }
  }
  cudaFree(dc); cudaFree(dh); cudaFree(dx); cudaFree(dd); cudaFree(dv); cudaFree(da); cudaFree(dA);
  cudaFree(dM); cudaFree(dF);
  return rc;
}

int gf_band_solve(gf_ctx* ctx, int n, int kl, int ku, const double* ab, int ldab, double* b, int* info) {
  if (!ctx || n <= 0 || kl < 0 || ku < 0 || ldab < 2 * kl + ku + 1 || !ab || !b) {
    set_err(ctx, "gf_band_solve: invalid arguments");
    return GF_ERR_ARG;
  }
  if (kl > GF_KB || ku > GF_KB) return wide_band_solve(ctx, n, kl, ku, ab, ldab, b, info);
  int npad = (n + 31) / 32 * 32;
  std::vector<double> band((size_t)npad * GF_LDB, 0.0);
  for (int j = 0; j < n; ++j)
    for (int i = std::max(0, j - ku); i <= std::min(n - 1, j + kl); ++i)
      band[(size_t)(GF_KB + i - j) + (size_t)j * GF_LDB] = ab[(size_t)(kl + ku + i - j) + (size_t)j * ldab];
  Batch bt{};
  bt.n_struct = 1;
  StructInfo inf{};
  inf.n_free = n;
  StructState st0{};
  st0.phase = PH_ITER;
  st0.need_solve = 1;
  double *dband = nullptr, *dP = nullptr, *dU = nullptr;
  StructInfo* dinf = nullptr;
  StructState* dst = nullptr;
  int rc = GF_OK;
  if (!dmalloc(ctx, &dband, band.size()) || !dmalloc(ctx, &dP, (size_t)npad) || !dmalloc(ctx, &dU, (size_t)npad * GF_UW) ||
      !dmalloc(ctx, &dinf, 1) || !dmalloc(ctx, &dst, 1)) {
    rc = GF_ERR_CUDA;
  } else {
    cudaStream_t s = ctx->stream;
    cudaMemcpyAsync(dband, band.data(), sizeof(double) * band.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dP, b, sizeof(double) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dinf, &inf, sizeof(inf), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dst, &st0, sizeof(st0), cudaMemcpyHostToDevice, s);
    bt.band = dband;
    bt.P = dP;
    bt.U = dU;
    bt.info = dinf;
    bt.state = dst;
    launch_band_solve(bt, s);
    cudaMemcpyAsync(b, dP, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&st0, dst, sizeof(st0), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_err(ctx, "gf_band_solve: %s", cudaGetErrorString(e));
      rc = GF_ERR_CUDA;
    }
    if (info) *info = st0.info_fail;
  }
  cudaFree(dband); cudaFree(dP); cudaFree(dU); cudaFree(dinf); cudaFree(dst);
  return rc;
}

}  // extern "C"

// ---- gf_band_solve_noalloc: the banded solve staged through static device
// scratch instead of per-call buffers ----
namespace {
constexpr size_t round256(size_t doubles) { return (doubles + 31) / 32 * 32; }
constexpr size_t NA_BAND = (size_t)GF_NOALLOC_MAX_N * GF_LDB;  // band, GF layout
constexpr size_t NA_P = NA_BAND;                                // right-hand side / solution
constexpr size_t NA_U = NA_P + round256(GF_NOALLOC_MAX_N);      // U rows
constexpr size_t NA_INFO = NA_U + round256((size_t)GF_NOALLOC_MAX_N * GF_UW);
constexpr size_t NA_STATE = NA_INFO + round256((sizeof(StructInfo) + 7) / 8);
constexpr size_t NA_TOTAL = NA_STATE + round256((sizeof(StructState) + 7) / 8);
constexpr int NA_MAX_DEVICES = 64;
// Per-device address of the scratch array, looked up on the first call on
// that device.  Two threads making their first call at once both store the
// same pointer; the atomics make that well defined.
std::atomic<void*> g_noalloc_base[NA_MAX_DEVICES] = {};

struct DeviceGuard {
  int prev = -1;
  bool switched = false;
  ~DeviceGuard() {
    if (switched) cudaSetDevice(prev);
  }
};
}  // namespace

// about 7 MB per device: GF_NOALLOC_MAX_N x (GF_LDB + 1 + GF_UW) doubles
static __device__ __align__(256) double g_noalloc_scratch[NA_TOTAL];

// Zeroes every scratch band entry that is not a stored entry of the caller's
// matrix: rows outside the kl/ku band and the triangle corners (i < 0 or
// i >= n), whatever an earlier call or the caller's unreferenced GB entries
// left there.
__global__ void k_noalloc_band_clean(double* band, int n, int kl, int ku) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * GF_LDB) return;
  int j = (int)(t / GF_LDB), r = (int)(t % GF_LDB);
  int i = j + r - GF_KB;
  if (r < GF_KB - ku || r > GF_KB + kl || i < 0 || i >= n) band[t] = 0.0;
}

extern "C" int gf_band_solve_noalloc(gf_ctx* ctx, int n, int kl, int ku, const double* ab, int ldab, double* b,
                                     int* info) {
  if (!ctx) return GF_ERR_ARG;
  if (n <= 0 || kl < 0 || ku < 0 || kl > GF_KB || ku > GF_KB || ldab < 2 * kl + ku + 1 || !ab || !b) {
    set_err(ctx, "gf_band_solve_noalloc: invalid arguments (kl, ku must be <= %d)", GF_KB);
    return GF_ERR_ARG;
  }
  if (n > GF_NOALLOC_MAX_N) {
    set_err(ctx, "gf_band_solve_noalloc: n = %d exceeds the static scratch limit GF_NOALLOC_MAX_N = %d; "
                 "use gf_band_solve", n, (int)GF_NOALLOC_MAX_N);
    return GF_ERR_ARG;
  }
  if (ctx->device < 0 || ctx->device >= NA_MAX_DEVICES) {
    set_err(ctx, "gf_band_solve_noalloc: device %d out of range", ctx->device);
    return GF_ERR_ARG;
  }
  DeviceGuard guard;
  CK(cudaGetDevice(&guard.prev));
  if (guard.prev != ctx->device) {
    CK(cudaSetDevice(ctx->device));
    guard.switched = true;
  }
  double* base = static_cast<double*>(g_noalloc_base[ctx->device].load(std::memory_order_acquire));
  if (!base) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_err(ctx, "gf_band_solve_noalloc: cudaGetSymbolAddress of the static scratch failed: %s",
              cudaGetErrorString(e));
      return GF_ERR_CUDA;
    }
    g_noalloc_base[ctx->device].store(p, std::memory_order_release);
    base = static_cast<double*>(p);
  }
  double* dband = base;
  double* dP = base + NA_P;
  double* dU = base + NA_U;
  StructInfo* dinf = reinterpret_cast<StructInfo*>(base + NA_INFO);
  StructState* dst = reinterpret_cast<StructState*>(base + NA_STATE);
  StructInfo inf{};
  inf.n_free = n;
  StructState st0{};
  st0.phase = PH_ITER;
  st0.need_solve = 1;
  cudaStream_t s = ctx->stream;
  // column j's stored rows kl .. 2kl+ku of ab land on band rows GF_KB-ku .. GF_KB+kl
  CK(cudaMemcpy2DAsync(dband + (GF_KB - ku), sizeof(double) * GF_LDB, ab + kl, sizeof(double) * (size_t)ldab,
                       sizeof(double) * (size_t)(kl + ku + 1), (size_t)n, cudaMemcpyHostToDevice, s));
  int64_t cells = (int64_t)n * GF_LDB;
  k_noalloc_band_clean<<<(unsigned)((cells + 255) / 256), 256, 0, s>>>(dband, n, kl, ku);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(dP, b, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dinf, &inf, sizeof(inf), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dst, &st0, sizeof(st0), cudaMemcpyHostToDevice, s));
  Batch bt{};
  bt.n_struct = 1;
  bt.band = dband;
  bt.P = dP;
  bt.U = dU;
  bt.info = dinf;
  bt.state = dst;
  launch_band_solve(bt, s);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(b, dP, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&st0, dst, sizeof(st0), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (info) *info = st0.info_fail;
  return GF_OK;
}

namespace gfh {
// Device bytes of a batch of these structures built with opts (NULL: the
// defaults); no device work.
int batch_device_bytes(gf_ctx* ctx, int n, const gf_model_desc* models, const gf_solve_opts* opts, size_t* bytes) {
  if (n <= 0 || !models || !bytes) {
    set_err(ctx, "gf_batch_device_bytes: invalid arguments");
    return GF_ERR_ARG;
  }
  gf_batch B;
  B.ctx = ctx;
  B.count_only = true;
  if (opts) B.opts = *opts; else gf_default_opts(&B.opts);
  int r = build_batch(&B, n, models);
  if (r != GF_OK) return r;
  *bytes = B.counted_bytes;
  return GF_OK;
}
}  // namespace gfh

extern "C" int gf_batch_device_bytes(gf_ctx* ctx, int n, const gf_model_desc* models, size_t* bytes) {
  return batch_device_bytes(ctx, n, models, nullptr, bytes);
}
