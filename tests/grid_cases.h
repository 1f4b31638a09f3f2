// The workloads of the reference-side fixtures as the host grid builder
// (neopz_gb300/host/pz_grid.h) describes them: the same cases, material ids,
// forcing and boundary conditions as the reference-library meshes of
// oracle/ref_cases.h.  Shared by tests/abi_driver.cpp and tests/binding_check.cpp.
#pragma once
#include <cstring>
#include <string>

#include "gpz.h"
#include "pz_grid.h"

static const double kGridBigNumber = 1e17 * 2.0 / 3.0;  // TPZMaterial::fBigNumber

inline bool grid_case_is3d(const std::string &cs) {
  return cs == "darcy3d" || cs == "elast3d" || cs == "elast3d_c5" || cs == "elast3d_hp";
}

inline gpz_material grid_case_material(int kind, int dim, double fx, double fy, double fz, int forcing, int porder) {
  gpz_material m;
  std::memset(&m, 0, sizeof(m));
  m.kind = kind;
  m.dim = dim;
  m.scale = 1.0;
  m.E = 1.0;
  m.nu = 0.3;
  m.coef_const = 1.0;
  m.force[0] = fx;
  m.force[1] = fy;
  m.force[2] = fz;
  m.forcing = forcing;
  m.forcing_porder = porder;
  m.bignumber = kGridBigNumber;
  return m;
}

inline gpz_bc grid_case_bc(int type, double v0, double v1, double v2) {
  gpz_bc b;
  std::memset(&b, 0, sizeof(b));
  b.type = type;
  b.material = 0;
  b.val2[0] = v0;
  b.val2[1] = v1;
  b.val2[2] = v2;
  return b;
}

// The grid of one case (gpzh_grid_free it), or nullptr.  coef / order: per volume cell, or nullptr.
inline void *grid_case(const std::string &cs, int n, int p, const double *coef, const int32_t *order) {
  const bool is3d = grid_case_is3d(cs);
  gpzh_grid_spec s;
  std::memset(&s, 0, sizeof(s));
  s.dim = is3d ? 3 : 2;
  for (int d = 0; d < 3; d++) {
    s.ndiv[d] = d < s.dim ? n : 1;
    s.minX[d] = 0.0;
    s.maxX[d] = d < s.dim ? 1.0 : 0.0;
  }
  s.create_bc = 1;
  s.default_order = p;
  s.nmat = 1;
  s.mat_id[0] = 1;
  const int mats3[7] = {1, -1, -1, -1, -1, -1, -1}, mats2[5] = {1, -1, -1, -1, -1},
            traction[7] = {1, -1, -2, -2, -2, -2, -3}, hp[7] = {1, -1, -2, -2, -2, -2, -2};
  const bool top = cs == "elast3d" || cs == "elast3d_c5";
  const int *mid = top ? traction : cs == "elast3d_hp" ? hp : is3d ? mats3 : mats2;
  for (int k = 0; k < (is3d ? 7 : 5); k++) s.matids[k] = mid[k];
  s.nbc = 1;
  s.bc_id[0] = -1;
  s.bcs[0] = grid_case_bc(0, 0, 0, 0);
  if (cs == "poisson2d") {
    s.mats[0] = grid_case_material(GPZ_MAT_POISSON, 2, 1.0, 0, 0, GPZ_F_SINPROD, 2);
  } else if (cs == "darcy2d" || cs == "darcy3d") {
    s.mats[0] = grid_case_material(GPZ_MAT_DARCY, s.dim, 1.0, 0, 0, GPZ_F_CONST, 0);
  } else if (cs == "elast3d" || cs == "elast3d_c5" || cs == "elast3d_hp") {
    s.mats[0] = grid_case_material(GPZ_MAT_ELAST3D, 3, 0, 0, cs == "elast3d_c5" ? 0.0 : -1.0, GPZ_F_CONST, 0);
    if (top) {
      s.nbc = 2;
      s.bc_id[1] = -3;
      s.bcs[1] = grid_case_bc(1, 0, 0, -1.0);
    }
  } else {
    return nullptr;
  }
  s.elem_coef = coef;
  s.elem_order = order;
  return gpzh_grid_build(&s);
}
