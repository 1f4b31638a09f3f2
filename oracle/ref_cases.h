// The workloads of the reference-side fixtures, built through the NeoPZ
// reference library's public API as a user program builds them:
//   TPZGeoMeshTools::CreateGeoMeshOnGrid -> TPZCompMesh (SetDefaultOrder,
//   SetAllCreateFunctionsContinuous, materials + TPZBndCondT, AutoBuild)
// Test infrastructure: used by oracle/ref_harness.cpp (fixture writer) and
// tests/binding_check.cpp (the NeoPZ-side binding against the same meshes).
//
//   CASE: poisson2d | darcy2d | darcy3d | elast3d | elast3d_c5 | elast3d_hp
//     (elast3d: body force (0,0,-1); elast3d_c5: no body force; both with a
//     clamped base and the traction (0,0,-1) on top)
//   coef: float64 per volume cell (permeability or Young modulus), or empty
//   order: int per volume cell (preferred order, elast3d_hp), or empty
// Per-cell coefficients are given as one material per cell (material id
// 1000 + cell); the boundary materials hang off the first of them (their
// contributions do not read the volume coefficient).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "DarcyFlow/TPZDarcyFlow.h"
#include "MMeshType.h"
#include "TPZBndCondT.h"
#include "TPZElasticity3D.h"
#include "TPZGeoMeshTools.h"
#include "TPZMatPoisson.h"
#include "pzcmesh.h"
#include "pzgmesh.h"
#include "pzintel.h"

inline bool ref_case_is3d(const std::string &cs) {
  return cs == "darcy3d" || cs == "elast3d" || cs == "elast3d_c5" || cs == "elast3d_hp";
}

// The computational mesh of one workload (its geometric mesh is cmesh->Reference()); nullptr after printing why.
inline TPZCompMesh *ref_case_mesh(const std::string &cs, int n, int p, const std::vector<double> &coef,
                                  const std::vector<int> &order) {
  const bool is3d = ref_case_is3d(cs);
  const bool traction = cs == "elast3d" || cs == "elast3d_c5";
  const int dim = is3d ? 3 : 2;
  const int64_t ncell = is3d ? (int64_t)n * n * n : (int64_t)n * n;
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
        return nullptr;
      }
      if (!coef.empty()) gmesh->Element(i)->SetMaterialId(1000 + (int)i);
      nvol++;
    }
  if (nvol != ncell) {
    fprintf(stderr, "cell count mismatch\n");
    return nullptr;
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
  return cmesh;
}
