// Driver for the reference build (oracle/_ref/libgiraffe_ref.so).  TEST
// INFRASTRUCTURE: it runs the reference's own sources on decks written in the
// reference's .inp syntax and records what the reference would write, so that
// the oracle restatement and the committed golden fixtures can be pinned to
// the reference itself.  Never loaded by the product path.
//
// The deck loop mirrors reference src/IO.cpp:288-657 for the keywords of the
// implicit beam/shell path: each block reads a count, then for each entry a
// type keyword and the reference object's own Read().  Database::PreCalc is
// restated for the same objects (reference src/Database.cpp:704-759), and the
// solution sequence follows reference src/main.cpp:49-62.
#include "Beam_1.h"
#include "ConvergenceCriteria.h"
#include "CoordinateSystem.h"
#include "Database.h"
#include "Dynamic.h"
#include "Hooke.h"
#include "LagrangeSave.h"
#include "Modal.h"
#include "Monitor.h"
#include "NodalConstraint.h"
#include "NodalDisplacement.h"
#include "NodalLoad.h"
#include "Node.h"
#include "NodeSet.h"
#include "PipeLoad.h"
#include "PipeSection.h"
#include "Pipe_1.h"
#include "SecRectangle.h"
#include "SecTube.h"
#include "Shell_1.h"
#include "ElementSet.h"
#include "ShellLoad.h"
#include "ShellSectionHomogeneous.h"
#include "SolverOptions.h"
#include "Static.h"

#include <cstdio>
#include <cstring>

#include "ref_hooks.h"

extern Database db;
void TryComment(FILE* f);
RefHooks ref_hooks_storage;

void ref_record_state(int solution, double time) {
  FILE* f = ref_hooks_storage.rec;
  if (!f) return;
  fprintf(f, "T %d %.17g\n", solution, time);
  for (int i = 0; i < db.number_nodes; ++i) {
    Node* n = db.nodes[i];
    fprintf(f, "N %d", i + 1);
    for (int k = 0; k < 6; ++k) fprintf(f, " %.17g", n->copy_coordinates[k]);
    for (int k = 0; k < 9; ++k) fprintf(f, " %.17g", n->Q->getMatrix()[k]);
    fprintf(f, "\n");
  }
  for (int e = 0; e < db.number_elements; ++e) {
    LagrangeSave* lag = nullptr;
    if (typeid(*db.elements[e]) == typeid(Beam_1)) lag = static_cast<Beam_1*>(db.elements[e])->lag_save;
    else if (typeid(*db.elements[e]) == typeid(Pipe_1)) lag = static_cast<Pipe_1*>(db.elements[e])->lag_save;
    if (!lag) continue;
    for (int g = 0; g < 2; ++g) {
      fprintf(f, "G %d %d", e + 1, g);
      for (int k = 0; k < 9; ++k) fprintf(f, " %.17g", lag->Q_i[g]->getMatrix()[k]);
      fprintf(f, "\n");
    }
  }
  fflush(f);
}

namespace {
template <typename Base, typename Make>
bool read_block(FILE* f, int& count, Base**& arr, Make make) {
  char s[1000];
  if (fscanf(f, "%999s", s) != 1) return false;
  count = atoi(s);
  arr = new Base*[count];
  for (int i = 0; i < count; ++i) {
    TryComment(f);
    if (fscanf(f, "%999s", s) != 1) return false;
    arr[i] = make(s);
    if (!arr[i]) {
      fprintf(stderr, "ref deck: unsupported entry '%s'\n", s);
      count = i;
      return false;
    }
    if (!arr[i]->Read(f)) {
      fprintf(stderr, "ref deck: error reading '%s' %d\n", s, i + 1);
      count = i + 1;
      return false;
    }
  }
  return true;
}

// Skips tokens until the next first-level keyword; used for the output blocks
// (Monitor, PostFiles) that the recording hooks replace.
bool is_keyword(const char* s) {
  static const char* k[] = {"SolutionSteps", "Nodes", "Elements", "Materials", "Sections",
                            "ShellSections", "CoordinateSystems", "NodeSets", "Loads",
                            "Displacements", "Constraints", "ConvergenceCriteria", "SolverOptions",
                            "Monitor", "PostFiles", "ElementSets", "Environment", "PipeSections", nullptr};
  for (int i = 0; k[i]; ++i)
    if (!strcmp(s, k[i])) return true;
  return false;
}
}  // namespace

extern "C" {

// Reads a deck.  Returns 0 on success.
int giraffe_ref_load(const char* path) {
  FILE* f = fopen(path, "r");
  if (!f) return 1;
  char s[1000];
  bool ok = true;
  bool have = false;
  while (ok && (have || fscanf(f, "%999s", s) == 1)) {
    have = false;
    if (s[0] == '/' && (s[1] == '/' || s[1] == '*')) {
      // re-read as a comment: step back over the token is not possible, so
      // consume the rest of a line comment here
      if (s[1] == '/') { int c; while ((c = fgetc(f)) != EOF && c != '\n') {} }
      else if (!strstr(s + 2, "*/")) { int p = 0, c; while ((c = fgetc(f)) != EOF) { if (p == '*' && c == '/') break; p = c; } }
      continue;
    }
    if (!strcmp(s, "SolutionSteps")) {
      ok = read_block<Solution>(f, db.number_solutions, db.solution, [](const char* t) -> Solution* {
        if (!strcmp(t, "Static")) return new Static();
        if (!strcmp(t, "Dynamic")) return new Dynamic();
        if (!strcmp(t, "Modal")) return new Modal();
        return nullptr;
      });
      db.solution_exist = true;
      // reference src/Database.cpp:760-770 (no Modal steps here)
      double start = 0.0;
      for (int i = 0; i < db.number_solutions; ++i) {
        db.solution[i]->start_time = start;
        start = db.solution[i]->end_time;
      }
    } else if (!strcmp(s, "Nodes")) {
      if (fscanf(f, "%999s", s) != 1) { ok = false; break; }
      db.number_nodes = atoi(s);
      db.nodes = new Node*[db.number_nodes];
      for (int i = 0; i < db.number_nodes && ok; ++i) {
        db.nodes[i] = new Node(db.number_GLs_node);
        TryComment(f);
        ok = db.nodes[i]->Read(f);
      }
      db.nodes_exist = true;
    } else if (!strcmp(s, "Elements")) {
      ok = read_block<Element>(f, db.number_elements, db.elements, [](const char* t) -> Element* {
        if (!strcmp(t, "Beam_1")) return new Beam_1();
        if (!strcmp(t, "Shell_1")) return new Shell_1();
        if (!strcmp(t, "Pipe_1")) return new Pipe_1();
        return nullptr;
      });
      db.elements_exist = true;
    } else if (!strcmp(s, "PipeSections")) {
      // reference src/IO.cpp:1282-1301: PipeSection::Read takes its own "PS"
      if (fscanf(f, "%999s", s) != 1) { ok = false; break; }
      db.number_pipe_sections = atoi(s);
      db.pipe_sections = new PipeSection*[db.number_pipe_sections];
      for (int i = 0; i < db.number_pipe_sections && ok; ++i) {
        db.pipe_sections[i] = new PipeSection();
        TryComment(f);
        ok = db.pipe_sections[i]->Read(f);
      }
      db.pipe_sections_exist = true;
    } else if (!strcmp(s, "Materials")) {
      ok = read_block<Material>(f, db.number_materials, db.materials, [](const char* t) -> Material* {
        return !strcmp(t, "Hooke") ? new Hooke() : nullptr;
      });
      db.materials_exist = true;
    } else if (!strcmp(s, "Sections")) {
      ok = read_block<Section>(f, db.number_sections, db.sections, [](const char* t) -> Section* {
        if (!strcmp(t, "Rectangle")) return new SecRectangle();
        if (!strcmp(t, "Tube")) return new SecTube();
        return nullptr;
      });
      db.sections_exist = true;
    } else if (!strcmp(s, "ShellSections")) {
      ok = read_block<ShellSection>(f, db.number_shell_sections, db.shell_sections,
                                    [](const char* t) -> ShellSection* {
                                      return !strcmp(t, "Homogeneous") ? new ShellSectionHomogeneous() : nullptr;
                                    });
      db.shell_sections_exist = true;
    } else if (!strcmp(s, "CoordinateSystems")) {
      if (fscanf(f, "%999s", s) != 1) { ok = false; break; }
      db.number_CS = atoi(s);
      db.CS = new CoordinateSystem*[db.number_CS];
      for (int i = 0; i < db.number_CS && ok; ++i) {
        db.CS[i] = new CoordinateSystem();
        TryComment(f);
        ok = db.CS[i]->Read(f);
      }
      db.CS_exist = true;
    } else if (!strcmp(s, "NodeSets")) {
      if (fscanf(f, "%999s", s) != 1) { ok = false; break; }
      db.number_node_sets = atoi(s);
      db.node_sets = new NodeSet*[db.number_node_sets];
      for (int i = 0; i < db.number_node_sets && ok; ++i) {
        db.node_sets[i] = new NodeSet();
        TryComment(f);
        ok = db.node_sets[i]->Read(f);
      }
      db.node_sets_exist = true;
    } else if (!strcmp(s, "ElementSets")) {
      if (fscanf(f, "%999s", s) != 1) { ok = false; break; }
      db.number_element_sets = atoi(s);
      db.element_sets = new ElementSet*[db.number_element_sets];
      for (int i = 0; i < db.number_element_sets && ok; ++i) {
        db.element_sets[i] = new ElementSet();
        TryComment(f);
        ok = db.element_sets[i]->Read(f);
      }
      db.element_sets_exist = true;
    } else if (!strcmp(s, "Loads")) {
      ok = read_block<Load>(f, db.number_loads, db.loads, [](const char* t) -> Load* {
        if (!strcmp(t, "NodalLoad")) return new NodalLoad();
        if (!strcmp(t, "ShellLoad")) return new ShellLoad();
        if (!strcmp(t, "PipeLoad")) return new PipeLoad();
        return nullptr;
      });
      db.loads_exist = true;
    } else if (!strcmp(s, "Displacements")) {
      ok = read_block<Displacement>(f, db.number_displacements, db.displacements,
                                    [](const char* t) -> Displacement* {
                                      return !strcmp(t, "NodalDisplacement") ? new NodalDisplacement() : nullptr;
                                    });
      db.displacements_exist = true;
    } else if (!strcmp(s, "Constraints")) {
      ok = read_block<Constraint>(f, db.number_constraints, db.constraints, [](const char* t) -> Constraint* {
        return !strcmp(t, "NodalConstraint") ? new NodalConstraint() : nullptr;
      });
      db.constraints_exist = true;
    } else if (!strcmp(s, "ConvergenceCriteria")) {
      TryComment(f);
      ok = db.conv_criteria->Read(f);
    } else if (!strcmp(s, "SolverOptions")) {
      TryComment(f);
      ok = db.solver_options->Read(f);
    } else if (!strcmp(s, "Monitor")) {
      // the reference's own reader (src/Monitor.cpp:112-195); the recording
      // hook writes the monitored nodes' lines
      db.monitor = new Monitor();
      ok = db.monitor->Read(f);
      db.monitor_exist = true;
    } else if (!strcmp(s, "PostFiles")) {
      while (fscanf(f, "%999s", s) == 1) {
        if (is_keyword(s)) { have = true; break; }
      }
    } else {
      fprintf(stderr, "ref deck: unsupported keyword '%s'\n", s);
      ok = false;
    }
  }
  fclose(f);
  if (!ok) return 2;
  // reference src/Database.cpp:704-759, restricted to the objects above
  for (int i = 0; i < db.number_sections; ++i) db.sections[i]->PreCalc();
  for (int i = 0; i < db.number_elements; ++i) db.elements[i]->PreCalc();
  for (int i = 0; i < db.number_loads; ++i) db.loads[i]->PreCalc();
  for (int i = 0; i < db.number_constraints; ++i) db.constraints[i]->PreCalc();
  for (int i = 0; i < db.number_displacements; ++i) db.displacements[i]->PreCalc();
  db.solver_options->PreCalc();
  return 0;
}

// Runs every solution step of the loaded deck (reference src/main.cpp:49-62).
// Each converged configuration is appended to rec_path; the reference's
// console report goes to log_path (either may be null).  Returns 0 when all
// steps finished, 1 when the reference aborted.
int giraffe_ref_solve(const char* rec_path, const char* log_path) {
  ref_hooks_storage.rec = rec_path ? fopen(rec_path, "w") : nullptr;
  ref_hooks_storage.log = log_path ? fopen(log_path, "w") : nullptr;
  bool converged = true;
  for (int i = 0; i < db.number_solutions && converged; ++i) {
    db.current_solution_number = i + 1;
    converged = db.solution[i]->Solve();
  }
  if (ref_hooks_storage.rec) fclose(ref_hooks_storage.rec);
  if (ref_hooks_storage.log) fclose(ref_hooks_storage.log);
  ref_hooks_storage.rec = ref_hooks_storage.log = nullptr;
  return converged ? 0 : 1;
}

// ---- element-level access for known-answer fixtures ----
int giraffe_ref_n_nodes() { return db.number_nodes; }
int giraffe_ref_n_elements() { return db.number_elements; }

// Prepares DOF numbering the way the first solution step does
// (reference src/Static.cpp:161-163).
void giraffe_ref_prepare() {
  db.current_solution_number = 1;
  db.solution[0]->DOFsActive();
  db.solution[0]->SetGlobalDOFs();
  db.solution[0]->SetGlobalSize();
}

void giraffe_ref_set_increment(int node, const double* d6) {
  for (int k = 0; k < 6; ++k) db.nodes[node - 1]->displacements[k] = d6[k];
}

// Element::Mount + MountElementLoads (reference src/Solution.cpp:227-262).
// K receives the element tangent (column-major, nDOFs x nDOFs) and P the
// unbalanced element vector P_loading.  Returns nDOFs.
int giraffe_ref_element_mount(int e, double* K, double* P) {
  Element* el = db.elements[e - 1];
  el->Mount();
  el->MountElementLoads();
  int n = el->nDOFs;
  Matrix* stiff = nullptr;
  Matrix* load = nullptr;
  if (typeid(*el) == typeid(Beam_1)) {
    stiff = static_cast<Beam_1*>(el)->stiffness;
    load = static_cast<Beam_1*>(el)->P_loading;
  } else if (typeid(*el) == typeid(Pipe_1)) {
    stiff = static_cast<Pipe_1*>(el)->stiffness;
    load = static_cast<Pipe_1*>(el)->P_loading;
  } else if (typeid(*el) == typeid(Shell_1)) {
    stiff = static_cast<Shell_1*>(el)->stiffness;
    load = static_cast<Shell_1*>(el)->P_loading;
  }
  if (!stiff) return 0;
  memcpy(K, stiff->getMatrix(), sizeof(double) * n * n);
  memcpy(P, load->getMatrix(), sizeof(double) * n);
  return n;
}

// Converged nodal velocities and accelerations (Node::copy_vel / copy_accel).
void giraffe_ref_set_vel_accel(int node, const double* vel6, const double* accel6) {
  for (int k = 0; k < 6; ++k) {
    db.nodes[node - 1]->copy_vel[k] = vel6[k];
    db.nodes[node - 1]->copy_accel[k] = accel6[k];
  }
}

// Beam_1 inertial contributions of the first solution step, which must be
// Dynamic: Newmark coefficients for time step dt
// (reference src/Dynamic.cpp:582-590), then Mount (Gauss-point increments)
// and MountMass (reference src/Beam_1.cpp:1564-1638).  M: 18x18 column-major
// mass/gyroscopic tangent, F: inertial_loading, *ke: kinetic energy.
int giraffe_ref_beam_inertia(int e, double dt, double* M, double* F, double* ke) {
  if (typeid(*db.solution[0]) != typeid(Dynamic)) return 0;
  Dynamic* d = static_cast<Dynamic*>(db.solution[0]);
  d->CalculateNewmarkCoeff(dt);
  db.current_solution_number = 1;
  Element* el = db.elements[e - 1];
  if (typeid(*el) != typeid(Beam_1)) return 0;
  Beam_1* b = static_cast<Beam_1*>(el);
  b->Mount();
  b->MountMass();
  memcpy(M, b->mass->getMatrix(), sizeof(double) * 324);
  memcpy(F, b->inertial_loading->getMatrix(), sizeof(double) * 18);
  *ke = b->kinetic_energy;
  return 18;
}

// Commits the current increments as converged (reference
// src/Solution.cpp:426-530 for nodes and elements) and zeroes them
// (reference src/Solution.cpp:798-814).  SaveLagrange reads the Gauss-point
// quantities of the last Mount, so every element is mounted at the committed
// increments first, as the converged Newton iteration does.
void giraffe_ref_commit() {
  for (int i = 0; i < db.number_elements; ++i) db.elements[i]->Mount();
  for (int i = 0; i < db.number_nodes; ++i) db.nodes[i]->SaveConfiguration();
  for (int i = 0; i < db.number_elements; ++i) db.elements[i]->SaveLagrange();
  for (int i = 0; i < db.number_nodes; ++i)
    for (int k = 0; k < 6; ++k) db.nodes[i]->displacements[k] = 0.0;
}
}

// Shell_1 Mount + MountElementLoads + MountShellSpecialLoads of load number
// l (1-based) with the load evaluated at time t (reference
// src/Shell_1.cpp:1392-1467).  K: 27x27 column-major, P: P_loading.
extern "C" int giraffe_ref_shell_pressure(int e, int l, double t, double* K, double* P) {
  Element* el = db.elements[e - 1];
  if (typeid(*el) != typeid(Shell_1)) return 0;
  db.last_converged_time = t;
  db.current_time_step = 0.0;
  Shell_1* s = static_cast<Shell_1*>(el);
  s->Mount();
  s->MountElementLoads();
  s->MountShellSpecialLoads(l);
  memcpy(K, s->stiffness->getMatrix(), sizeof(double) * 27 * 27);
  memcpy(P, s->P_loading->getMatrix(), sizeof(double) * 27);
  return 27;
}

// Shell_1 inertial contributions of the first solution step, which must be
// Dynamic: Newmark coefficients for time step dt, then Zeros, Mount
// (Gauss-point increments) and MountMass (reference
// src/Shell_1.cpp:2406-2498).  M: 27x27 column-major mass/gyroscopic
// tangent, F: inertial_loading, *ke: kinetic energy.
extern "C" int giraffe_ref_shell_inertia(int e, double dt, double* M, double* F, double* ke) {
  if (typeid(*db.solution[0]) != typeid(Dynamic)) return 0;
  Dynamic* d = static_cast<Dynamic*>(db.solution[0]);
  d->CalculateNewmarkCoeff(dt);
  db.current_solution_number = 1;
  Element* el = db.elements[e - 1];
  if (typeid(*el) != typeid(Shell_1)) return 0;
  Shell_1* s = static_cast<Shell_1*>(el);
  s->Zeros();
  s->Mount();
  s->MountMass();
  memcpy(M, s->mass->getMatrix(), sizeof(double) * 27 * 27);
  memcpy(F, s->inertial_loading->getMatrix(), sizeof(double) * 27);
  *ke = s->kinetic_energy;
  return 27;
}

// Pipe_1 Mount + MountElementLoads + MountPipeSpecialLoads of load number l
// (1-based) with the load evaluated at time t (reference
// src/Pipe_1.cpp:1441-1494).  K: 18x18 column-major, P: P_loading.
extern "C" int giraffe_ref_pipe_pressure(int e, int l, double t, double* K, double* P) {
  Element* el = db.elements[e - 1];
  if (typeid(*el) != typeid(Pipe_1)) return 0;
  db.last_converged_time = t;
  db.current_time_step = 0.0;
  Pipe_1* p = static_cast<Pipe_1*>(el);
  p->Mount();
  p->MountElementLoads();
  p->MountPipeSpecialLoads(l);
  memcpy(K, p->stiffness->getMatrix(), sizeof(double) * 18 * 18);
  memcpy(P, p->P_loading->getMatrix(), sizeof(double) * 18);
  return 18;
}

// The two matrices of a Modal step (reference src/Modal.cpp:131-166,
// without the ARPACK eigen solve that follows them): the modal mass M_AA
// (MountMassModal, MountDynModal, MountGlobal, MountSparse), then the
// tangent K_AA (MountLocal, MountElementLoads, MountSpecialConstraints,
// MountContacts, MountLoads, MountGlobal, MountSparse), both written dense
// and column-major (n x n) in the reference's own DOF numbering.  Returns n,
// or 0 when n exceeds n_max.
static void ref_dense(SparseMatrix& A, double* out, int n) {
  if (!A.mounted) A.Mount();
  for (int i = 0; i < n * n; ++i) out[i] = 0.0;
  const double* a = A.m_matrix.valuePtr();
  const int* ia = A.m_matrix.outerIndexPtr();
  const int* ja = A.m_matrix.innerIndexPtr();
  for (int i = 0; i < A.m_matrix.rows(); ++i)
    for (int p = ia[i]; p < ia[i + 1]; ++p) out[i + (size_t)n * ja[p]] += a[p];
}

extern "C" int giraffe_ref_modal_matrices(double* K, double* M, int n_max) {
  Modal md;
  db.current_solution_number = 1;
  md.DOFsActive();
  md.SetGlobalDOFs();
  md.SetGlobalSize();
  const int n = db.global_stiffness_AA.rows;
  if (n > n_max) return 0;
  md.Zeros();
  md.Clear();
  md.ZerosLocalMatrices();
  md.MountMassModal();
  md.MountDynModal();
  md.MountGlobal();
  md.MountSparse();
  ref_dense(db.global_stiffness_AA, M, n);
  md.Clear();
  md.ZerosLocalMatrices();
  md.MountLocal();
  md.MountElementLoads();
  md.MountSpecialConstraints();
  md.MountContacts();
  md.MountLoads();
  md.MountGlobal();
  md.MountSparse();
  ref_dense(db.global_stiffness_AA, K, n);
  return n;
}
