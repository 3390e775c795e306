// Support code for the reference build (oracle/_ref).  TEST INFRASTRUCTURE:
// it lets the reference's own Beam_1 / Shell_1 / Static / Dynamic sources
// run on Linux without oneMKL, PARDISO, Eigen, ARPACK or the post-processing
// writers, so that their outputs can pin the oracle restatement.  Nothing
// here is part of the product path.
//
// What it supplies:
//  * the global Database object and a constructor that sets the same
//    defaults as reference src/Database.cpp:185-335 for the fields the hot
//    path reads (everything else stays zero from static initialisation);
//  * SparseMatrix (reference src/SparseMatrix.h:7-34) over the CSR stand-in,
//    with sparsesystem solving by FP64 banded LU with partial pivoting in
//    place of PARDISO phase 13 (reference src/SparseMatrix.cpp:74-166);
//  * TryComment with the comment rules of reference src/IO.cpp:688-736;
//  * recording hooks in place of PostFiles/Monitor output, which capture the
//    converged nodal state each time the reference would write results.
#include "Database.h"
#include "ConvergenceCriteria.h"
#include "Matrix.h"
#include "Node.h"
#include "PostFiles.h"
#include "Monitor.h"
#include "SolverOptions.h"
#include "SparseMatrix.h"

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../band_lu.h"
#include "ref_hooks.h"

Database db;

Database::Database() {
  number_GLs_node = 6;
  sprintf(version, "2.0.135");
  conv_criteria = new ConvergenceCriteria();
  solver_options = new SolverOptions();
  post_files = reinterpret_cast<PostFiles*>(&ref_hooks_storage);
  solver_options_exist = true;
  flag_nGL_changed = true;
  last_converged_time = 0.0;
  current_time_step = 0.0;
}
Database::~Database() {}

int Database::myprintf(const char* format, ...) {
  if (!ref_hooks_storage.log) return 0;
  va_list ap;
  va_start(ap, format);
  int r = vfprintf(ref_hooks_storage.log, format, ap);
  va_end(ap);
  return r;
}

// ---- comments in decks (reference src/IO.cpp:688-752) ----
void TryComment(FILE* f) {
  for (;;) {
    fpos_t pos;
    fgetpos(f, &pos);
    char s[10000];
    if (fscanf(f, "%9999s", s) != 1) { fsetpos(f, &pos); return; }
    if (s[0] == '/' && s[1] == '/') {
      int c;
      while ((c = fgetc(f)) != EOF && c != '\n') {}
      continue;
    }
    if (s[0] == '/' && s[1] == '*') {
      if (!strstr(s + 2, "*/")) {
        int prev = 0, c;
        while ((c = fgetc(f)) != EOF) {
          if (prev == '*' && c == '/') break;
          prev = c;
        }
      }
      continue;
    }
    fsetpos(f, &pos);
    return;
  }
}

// ---- recording hooks in place of the result writers ----
void PostFiles::UpdateSinglePartPostFiles(int solution, double time, int file_index) {
  (void)file_index;
  ref_record_state(solution, time);
}
void PostFiles::WriteConfigurationResults(int, double, int) {}
// Monitor::UpdateMonitor: each monitored node's own monitor line
// (Node::WriteMonitor, reference src/Node.cpp:227-320, the reference's code
// and format) into the record, tagged "M <node>".
void Monitor::UpdateMonitor(double time) {
  FILE* f = ref_hooks_storage.rec;
  if (!f) return;
  for (size_t i = 0; i < nodes.size(); ++i) {
    fprintf(f, "M %d\t", nodes[i]);
    db.nodes[nodes[i] - 1]->WriteMonitor(f, false, time);
  }
  first_record = false;
}

// ---- SparseMatrix over the CSR stand-in ----
SparseMatrix::SparseMatrix() {
  mounted = false;
  rows = 1; cols = 1; non_null_estimative = 1;
  m_matrix.resize(1, 1);
}
SparseMatrix::SparseMatrix(int r, int c, int nnz) {
  rows = r; cols = c; non_null_estimative = nnz;
  m_matrix.resize(r, c);
  tripletList.reserve(2 * (size_t)nnz);
  mounted = false;
}
SparseMatrix::SparseMatrix(SparseMatrix& o) {
  rows = o.rows; cols = o.cols; m_matrix = o.m_matrix;
  non_null_estimative = o.non_null_estimative; mounted = o.mounted; tripletList = o.tripletList;
}
SparseMatrix::~SparseMatrix() {}
void SparseMatrix::Clear() {
  tripletList.clear();
  mounted = false;
}
void SparseMatrix::setValue(int i, int j, double v) {
  if (i + 1 > m_matrix.rows() || j + 1 > m_matrix.cols())
    printf("Error assigning sparse matrix value\n");
  else
    tripletList.push_back(T(i, j, v));
  mounted = false;
}
void SparseMatrix::Mount() {
  m_matrix.setFromTriplets(tripletList.begin(), tripletList.end());
  mounted = true;
}
SparseMatrix& SparseMatrix::operator=(SparseMatrix const& o) {
  rows = o.rows; cols = o.cols; m_matrix = o.m_matrix;
  non_null_estimative = o.non_null_estimative; mounted = o.mounted; tripletList = o.tripletList;
  return *this;
}
Matrix operator*(SparseMatrix& A, Matrix& x) {
  if (!A.mounted) A.Mount();
  Matrix y((long)A.m_matrix.rows(), 1);
  const double* a = A.m_matrix.valuePtr();
  const int* ia = A.m_matrix.outerIndexPtr();
  const int* ja = A.m_matrix.innerIndexPtr();
  for (int i = 0; i < A.m_matrix.rows(); ++i)
    for (int p = ia[i]; p < ia[i + 1]; ++p) y(i, 0) += a[p] * x(ja[p], 0);
  return y;
}

// PARDISO substitute: FP64 band LU with partial pivoting, in the CSR
// numbering or, where that narrows the band, in reverse Cuthill-McKee order
// (PARDISO reorders too: nested dissection, reference
// src/SparseMatrix.cpp:93-94).  info_fail follows the reference convention
// (0 ok, 1 failure).
Matrix sparsesystem(SparseMatrix& A, Matrix& b, int* info_fail, int, int) {
  if (!A.mounted) A.Mount();
  int n = (int)A.m_matrix.rows();
  Matrix x(n);
  *info_fail = 0;
  if (n == 0) return x;
  const double* a = A.m_matrix.valuePtr();
  const int* ia = A.m_matrix.outerIndexPtr();
  const int* ja = A.m_matrix.innerIndexPtr();
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  int kl = 0, ku = 0;
  for (int i = 0; i < n; ++i)
    for (int p = ia[i]; p < ia[i + 1]; ++p) {
      int d = ja[p] - i;
      if (d > ku) ku = d;
      if (-d > kl) kl = -d;
    }
  if (n > 1) {
    std::vector<int> pi, pj;
    for (int i = 0; i < n; ++i)
      for (int p = ia[i]; p < ia[i + 1]; ++p) { pi.push_back(i); pj.push_back(ja[p]); }
    int *xadj, *adj;
    oracle_graph(n, pi.size(), pi.data(), pj.data(), &xadj, &adj);
    std::vector<int> rcm(n);
    oracle_rcm(n, xadj, adj, rcm.data());
    int bw = oracle_perm_bandwidth(n, xadj, adj, rcm.data());
    if (bw < (kl > ku ? kl : ku)) {
      perm = rcm;
      kl = ku = bw;
    }
    free(xadj);
    free(adj);
  }
  int ldab = 2 * kl + ku + 1;
  std::vector<double> ab((size_t)ldab * n, 0.0), w(n);
  std::vector<int> ipiv(n);
  for (int i = 0; i < n; ++i)
    for (int p = ia[i]; p < ia[i + 1]; ++p) GB_AT(ab.data(), ldab, kl, ku, perm[i], perm[ja[p]]) += a[p];
  for (int i = 0; i < n; ++i) w[perm[i]] = b(i, 0);
  int info = oracle_gbtrf(n, kl, ku, ab.data(), ldab, ipiv.data());
  if (info != 0) { *info_fail = 1; return x; }
  oracle_gbtrs(n, kl, ku, ab.data(), ldab, ipiv.data(), w.data());
  for (int i = 0; i < n; ++i) x(i, 0) = w[perm[i]];
  for (int i = 0; i < n; ++i)
    if (!(x(i, 0) == x(i, 0))) *info_fail = 1;
  return x;
}
