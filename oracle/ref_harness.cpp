// Fixture harness over the NeoPZ reference library itself (oracle/_ref/libpzref.so,
// built by oracle/ref_build.mk).  Test infrastructure: it writes the
// reference-side fixtures under tests/golden/ (tests/golden/make_ref_fixtures.py
// runs it); nothing in the product links or runs it.
//
// One run builds one workload through the reference's public API, as a user
// program would:
//   TPZGeoMeshTools::CreateGeoMeshOnGrid -> TPZCompMesh (SetDefaultOrder,
//   SetAllCreateFunctionsContinuous, materials + TPZBndCondT, AutoBuild) ->
//   TPZLinearAnalysis(cmesh, false) -> SetStructuralMatrix(TPZSSpStructMatrix
//   or TPZSpStructMatrix over TPZStructMatrixOR, serial) -> Assemble() ->
//   TPZStepSolver CG with a Jacobi TPZStepSolver (SetJacobi(1, 0, 0)) ->
//   Solve()
// and writes the CSR (IA, JA, A), the load vector, the solution and the
// solver's counts as raw little-endian arrays plus a small JSON file.
//
// Usage: ref_harness CASE N P SYM TOL OUTDIR [COEF_FILE] [ORDER_FILE]
//   CASE: poisson2d | darcy2d | darcy3d | elast3d | elast3d_c5 | elast3d_hp
//     (elast3d: body force (0,0,-1); elast3d_c5: no body force; both with a
//     clamped base and the traction (0,0,-1) on top)
//   SYM: 1 = TPZSSpStructMatrix (upper CSR), 0 = TPZSpStructMatrix (full CSR)
//   TOL: CG tolerance (0 = assemble only)
//   COEF_FILE: float64 per volume cell (permeability or Young modulus)
//   ORDER_FILE: int32 per volume cell (preferred order, elast3d_hp)
// Per-cell coefficients are given as one material per cell (material id
// 1000 + cell); the boundary materials hang off the first of them (their
// contributions do not read the volume coefficient).
#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "MMeshType.h"
#include "TPZBndCondT.h"
#include "TPZElasticity3D.h"
#include "TPZGeoMeshTools.h"
#include "TPZLinearAnalysis.h"
#include "TPZMatPoisson.h"
#include "TPZSSpStructMatrix.h"
#include "TPZSpStructMatrix.h"
#include "DarcyFlow/TPZDarcyFlow.h"
#include "pzcmesh.h"
#include "pzgmesh.h"
#include "pzintel.h"
#include "pzstepsolver.h"
#include "pzstrmatrixor.h"
#include "pzsysmp.h"
#include "pzysmp.h"

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
  const bool is3d = cs == "darcy3d" || cs == "elast3d" || cs == "elast3d_c5" || cs == "elast3d_hp";
  const bool traction = cs == "elast3d" || cs == "elast3d_c5";
  const int dim = is3d ? 3 : 2;
  const int64_t ncell = is3d ? (int64_t)n * n * n : (int64_t)n * n;
  std::vector<double> coef;
  std::vector<int> order;
  if (argc > 7 && std::string(argv[7]) != "-") coef = read_file<double>(argv[7], ncell);
  if (argc > 8) order = read_file<int>(argv[8], ncell);

  // geometric mesh: matids {volume, boundary ids in the generator's side order}
  TPZManVector<int, 7> matids;
  if (cs == "poisson2d" || cs == "darcy2d") matids = {1, -1, -1, -1, -1};
  else if (cs == "darcy3d") matids = {1, -1, -1, -1, -1, -1, -1};
  else if (traction) matids = {1, -1, -2, -2, -2, -2, -3};  // clamped base, free sides, traction on top
  else matids = {1, -1, -2, -2, -2, -2, -2};                       // hp: clamped base only
  TPZManVector<REAL, 3> minX = {0., 0., 0.}, maxX = {1., 1., is3d ? 1. : 0.};
  TPZManVector<int, 3> ndiv(dim, n);
  TPZGeoMesh *gmesh = TPZGeoMeshTools::CreateGeoMeshOnGrid(
      dim, minX, maxX, matids, ndiv, is3d ? MMeshType::EHexahedral : MMeshType::EQuadrilateral, true);
  // volume elements are created first, in cell order
  int64_t nvol = 0;
  for (int64_t i = 0; i < gmesh->NElements(); i++)
    if (gmesh->Element(i)->Dimension() == dim) {
      if (i != nvol) {
        fprintf(stderr, "volume elements are not first\n");
        return 3;
      }
      if (!coef.empty()) gmesh->Element(i)->SetMaterialId(1000 + (int)i);
      nvol++;
    }
  if (nvol != ncell) {
    fprintf(stderr, "cell count mismatch\n");
    return 3;
  }

  TPZCompMesh *cmesh = new TPZCompMesh(gmesh);
  cmesh->SetDefaultOrder(p);
  cmesh->SetDimModel(dim);
  cmesh->SetAllCreateFunctionsContinuous();
  const int nvolmat = coef.empty() ? 1 : (int)ncell;
  TPZMaterial *first = nullptr;
  for (int c = 0; c < nvolmat; c++) {
    const int id = coef.empty() ? 1 : 1000 + c;
    TPZMaterial *m = nullptr;
    if (cs == "poisson2d") {
      auto *mp = new TPZMatPoisson<STATE>(id, 2);
      auto f = [](const TPZVec<REAL> &x, TPZVec<STATE> &v) {
        v[0] = 2. * M_PI * M_PI * std::sin(M_PI * x[0]) * std::sin(M_PI * x[1]);
      };
      mp->SetForcingFunction(f, 2);
      m = mp;
    } else if (cs == "darcy2d" || cs == "darcy3d") {
      auto *md = new TPZDarcyFlow(id, dim);
      if (!coef.empty()) md->SetConstantPermeability(coef[c]);
      auto f = [](const TPZVec<REAL> &, TPZVec<STATE> &v) { v[0] = 1.; };
      md->SetForcingFunction(f, 0);
      m = md;
    } else {
      TPZManVector<STATE, 3> force = {0., 0., cs == "elast3d_c5" ? 0. : -1.};
      const STATE E = coef.empty() ? 1. : coef[c];
      m = new TPZElasticity3D(id, E, 0.3, force);
    }
    cmesh->InsertMaterialObject(m);
    if (!first) first = m;
  }
  const int nst = first->NStateVariables();
  TPZFNMatrix<9, STATE> val1(nst, nst, 0.);
  TPZManVector<STATE, 3> val2(nst, 0.);
  auto *bnd = dynamic_cast<TPZMaterialT<STATE> *>(first)->CreateBC(first, -1, 0, val1, val2);
  cmesh->InsertMaterialObject(bnd);
  if (traction) {
    TPZManVector<STATE, 3> t = {0., 0., -1.};
    auto *top = dynamic_cast<TPZMaterialT<STATE> *>(first)->CreateBC(first, -3, 1, val1, t);
    cmesh->InsertMaterialObject(top);
  }
  cmesh->AutoBuild();

  if (!order.empty()) {
    // every side takes the largest preferred order of the volume elements on it
    cmesh->LoadReferences();
    std::map<std::vector<int64_t>, int> side_max;
    auto side_key = [](TPZGeoEl *g, int s) {
      std::vector<int64_t> k;
      for (int i = 0; i < g->NSideNodes(s); i++) k.push_back(g->SideNodeIndex(s, i));
      std::sort(k.begin(), k.end());
      return k;
    };
    for (int64_t i = 0; i < cmesh->NElements(); i++) {
      TPZCompEl *cel = cmesh->Element(i);
      TPZGeoEl *g = cel ? cel->Reference() : nullptr;
      if (!g || g->Dimension() != dim) continue;
      const int o = order[g->Index()];
      dynamic_cast<TPZInterpolatedElement *>(cel)->SetPreferredOrder(o);
      for (int s = g->NCornerNodes(); s < g->NSides(); s++) {
        auto k = side_key(g, s);
        side_max[k] = std::max(side_max[k], o);
      }
    }
    for (int64_t i = 0; i < cmesh->NElements(); i++) {
      TPZCompEl *cel = cmesh->Element(i);
      TPZGeoEl *g = cel ? cel->Reference() : nullptr;
      if (!g || g->Dimension() != dim) continue;
      auto *intel = dynamic_cast<TPZInterpolatedElement *>(cel);
      for (int s = g->NCornerNodes(); s < g->NSides(); s++) intel->SetSideOrder(s, side_max[side_key(g, s)]);
    }
    cmesh->ExpandSolution();
  }

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
