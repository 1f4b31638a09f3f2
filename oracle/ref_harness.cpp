// Fixture harness over the NeoPZ reference library itself (oracle/_ref/libpzref.so,
// built by oracle/ref_build.mk).  Test infrastructure: it writes the
// reference-side fixtures under tests/golden/ (tests/golden/make_ref_fixtures.py
// runs it); nothing in the product links or runs it.
//
// One run builds one workload through the reference's public API, as a user
// program would (the mesh: oracle/ref_cases.h) ->
//   TPZLinearAnalysis(cmesh, false) -> SetStructuralMatrix(TPZSSpStructMatrix
//   or TPZSpStructMatrix over TPZStructMatrixOR, serial) -> Assemble() ->
//   TPZStepSolver CG with a Jacobi TPZStepSolver (SetJacobi(1, 0, 0)) ->
//   Solve()
// and writes the CSR (IA, JA, A), the load vector, the solution and the
// solver's counts as raw little-endian arrays plus a small JSON file.
//
// Usage: ref_harness CASE N P SYM TOL OUTDIR [COEF_FILE] [ORDER_FILE]
//   CASE, COEF_FILE (float64 per volume cell), ORDER_FILE (int32 per volume
//     cell): the workloads of oracle/ref_cases.h
//   SYM: 1 = TPZSSpStructMatrix (upper CSR), 0 = TPZSpStructMatrix (full CSR)
//   TOL: CG tolerance (0 = assemble only)
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "TPZLinearAnalysis.h"
#include "TPZSSpStructMatrix.h"
#include "TPZSpStructMatrix.h"
#include "pzstepsolver.h"
#include "pzstrmatrixor.h"
#include "pzsysmp.h"
#include "pzysmp.h"
#include "ref_cases.h"

template <class T>
static std::vector<T> read_file(const std::string &path, size_t n) {
  std::vector<T> v(n);
  FILE *f = fopen(path.c_str(), "rb");
  if (!f || fread(v.data(), sizeof(T), n, f) != n) {
    fprintf(stderr, "cannot read %zu items from %s\n", n, path.c_str());
    exit(2);
  }
  fclose(f);
  return v;
}

template <class T>
static void write_file(const std::string &path, const T *p, size_t n) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f || fwrite(p, sizeof(T), n, f) != n) {
    fprintf(stderr, "cannot write %s\n", path.c_str());
    exit(2);
  }
  fclose(f);
}

int main(int argc, char **argv) {
  if (argc < 7) {
    fprintf(stderr, "usage: ref_harness CASE N P SYM TOL OUTDIR [COEF_FILE] [ORDER_FILE]\n");
    return 2;
  }
  const std::string cs = argv[1];
  const int n = atoi(argv[2]), p = atoi(argv[3]), sym = atoi(argv[4]);
  const double tol = atof(argv[5]);
  const std::string out = argv[6];
  const bool is3d = ref_case_is3d(cs);
  const int64_t ncell = is3d ? (int64_t)n * n * n : (int64_t)n * n;
  std::vector<double> coef;
  std::vector<int> order;
  if (argc > 7 && std::string(argv[7]) != "-") coef = read_file<double>(argv[7], ncell);
  if (argc > 8) order = read_file<int>(argv[8], ncell);

  TPZCompMesh *cmesh = ref_case_mesh(cs, n, p, coef, order);
  if (!cmesh) return 3;
  TPZGeoMesh *gmesh = cmesh->Reference();

  TPZLinearAnalysis an(cmesh, false);
  if (sym) {
    TPZSSpStructMatrix<STATE, TPZStructMatrixOR<STATE>> str(cmesh);
    str.SetNumThreads(0);
    an.SetStructuralMatrix(str);
  } else {
    TPZSpStructMatrix<STATE, TPZStructMatrixOR<STATE>> str(cmesh);
    str.SetNumThreads(0);
    an.SetStructuralMatrix(str);
  }
  TPZStepSolver<STATE> direct;
  direct.SetDirect(ELDLt);
  an.SetSolver(direct);
  an.Assemble();
  TPZAutoPointer<TPZMatrix<STATE>> mat = an.MatrixSolver<STATE>().Matrix();
  const int64_t neq = cmesh->NEquations();
  TPZVec<int64_t> IA, JA;
  TPZVec<STATE> A;
  if (sym) {
    auto *s = dynamic_cast<TPZSYsmpMatrix<STATE> *>(mat.operator->());
    IA = s->IA();
    JA = s->JA();
    A = s->A();
  } else {
    auto *f = dynamic_cast<TPZFYsmpMatrix<STATE> *>(mat.operator->());
    f->GetData(IA, JA, A);
  }
  TPZFMatrix<STATE> &rhs = an.Rhs();
  std::vector<double> F(neq);
  for (int64_t i = 0; i < neq; i++) F[i] = rhs(i, 0);
  write_file(out + "/ia.bin", IA.begin(), IA.size());
  write_file(out + "/ja.bin", JA.begin(), JA.size());
  write_file(out + "/a.bin", A.begin(), A.size());
  write_file(out + "/f.bin", F.data(), F.size());

  int64_t iters = -1;
  double resid = -1.0;
  if (tol > 0 && sym) {
    TPZStepSolver<STATE> jac(mat), cg(mat);
    jac.SetJacobi(1, 0., 0);
    cg.SetCG(200000, jac, tol, 0);
    an.SetSolver(cg);
    an.Solve();
    auto *solver = dynamic_cast<TPZStepSolver<STATE> *>(an.Solver());
    iters = solver->NumIterations();
    resid = solver->GetTolerance();
    TPZFMatrix<STATE> &sol = an.Solution();
    std::vector<double> x(neq);
    for (int64_t i = 0; i < neq; i++) x[i] = sol(i, 0);
    write_file(out + "/x.bin", x.data(), x.size());
  }
  std::ofstream js(out + "/info.json");
  js.precision(17);
  js << "{\"case\": \"" << cs << "\", \"n\": " << n << ", \"p\": " << p << ", \"sym\": " << sym << ", \"neq\": " << neq
     << ", \"nnz\": " << JA.size() << ", \"tol\": " << tol << ", \"cg_iterations\": " << iters
     << ", \"cg_resid\": " << resid << ", \"nconnects\": " << cmesh->NConnects() << "}\n";
  delete cmesh;
  delete gmesh;
  return 0;
}
