// The NeoPZ-side binding (neopz_gb300/neopz_binding/gpz_neopz.h) compiled
// against the reference library's own headers and linked with it
// (oracle/_ref/libpzref.so) and with libgpz / libgpzhost.
//
// For one workload of oracle/ref_cases.h (the reference-library mesh) it
//   1. runs gpz_neopz::ExtractMesh on the TPZCompMesh and compares the
//      descriptor, field by field, with the host grid builder's descriptor of
//      the same workload (tests/grid_cases.h), whose pattern, values and
//      solutions the GPU tests hold to the reference's fixtures: nodes,
//      element types / corner nodes / orders / side connects, connect orders,
//      block positions and sizes, the material and boundary data each element
//      resolves to and its coefficient;
//   2. drives TPZLinearAnalysis with TPZSSpStructMatrixGPU as the struct
//      matrix and a TPZStepSolver CG over a Jacobi step solver.  Without a
//      GPU the first device call (gpz_ctx_create in Create) stops with
//      DebugStop, as the reference reports errors; with one, the device
//      matrix, load vector and CG solution are compared with the reference's
//      own serial TPZSSpStructMatrix assembly and CG.
// Prints one JSON object; exit 0 when every comparison holds.
//
// Usage: binding_check CASE N P [COEF_FILE|-] [ORDER_FILE]
#include <cmath>
#include <cstdio>
#include <exception>
#include <string>
#include <vector>

#include "TPZLinearAnalysis.h"
#include "TPZSSpStructMatrix.h"
#include "gpz_neopz.h"
#include "grid_cases.h"
#include "pzstrmatrixor.h"
#include "ref_cases.h"

template <class T>
static std::vector<T> read_file(const char *path, size_t n) {
  std::vector<T> v(n);
  FILE *f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), sizeof(T), n, f) != n) {
    std::fprintf(stderr, "cannot read %s\n", path);
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

static std::vector<std::string> g_bad;
static void expect(bool ok, const std::string &what) {
  if (!ok && g_bad.size() < 20) g_bad.push_back(what);
}

template <class T>
static bool same_vec(const TPZVec<T> &a, const TPZVec<T> &b) {
  if (a.size() != b.size()) return false;
  for (int64_t i = 0; i < a.size(); i++)
    if (a[i] != b[i]) return false;
  return true;
}

static bool same_material(const gpz_material &a, const gpz_material &b) {
  bool ok = a.kind == b.kind && a.dim == b.dim && a.scale == b.scale && a.nu == b.nu && a.forcing == b.forcing &&
            a.forcing_porder == b.forcing_porder && a.bignumber == b.bignumber;
  for (int j = 0; j < 3; j++) ok = ok && a.force[j] == b.force[j];
  return ok;
}

static bool same_bc(const gpz_bc &a, const gpz_bc &b) {
  bool ok = a.type == b.type;
  for (int j = 0; j < 9; j++) ok = ok && a.val1[j] == b.val1[j];
  for (int j = 0; j < 3; j++) ok = ok && a.val2[j] == b.val2[j];
  return ok;
}

// the coefficient element e computes with: el_coef, else the material's constant
static double coef_of(const gpz_mesh_desc &d, int64_t e) {
  if (d.el_coef) return d.el_coef[e];
  const gpz_material &m = d.mats[d.el_mat[e]];
  return m.kind == GPZ_MAT_ELAST3D ? m.E : m.coef_const;
}

static void compare(const gpz_mesh_desc &a, const gpz_mesh_desc &b) {
  expect(a.dim == b.dim && a.nstate == b.nstate, "dim / nstate");
  expect(a.nnodes == b.nnodes, "nnodes");
  for (int64_t i = 0; i < 3 * a.nnodes && a.nnodes == b.nnodes; i++)
    if (a.node_xyz[i] != b.node_xyz[i]) {
      expect(false, "node_xyz[" + std::to_string(i) + "]");
      break;
    }
  expect(a.nel == b.nel, "nel");
  expect(a.nconnects == b.nconnects, "nconnects");
  expect(a.neq == b.neq, "neq");
  if (a.nel != b.nel || a.nconnects != b.nconnects) return;
  for (int64_t e = 0; e < a.nel; e++) {
    const std::string el = "element " + std::to_string(e);
    expect(a.el_type[e] == b.el_type[e], el + " type");
    expect(a.el_order[e] == b.el_order[e], el + " order");
    for (int k = 0; k < 8; k++) expect(a.el_nodes[8 * e + k] == b.el_nodes[8 * e + k], el + " node");
    for (int k = 0; k < 27; k++) expect(a.el_conn[27 * e + k] == b.el_conn[27 * e + k], el + " connect");
    const int ma = a.el_mat[e], mb = b.el_mat[e];
    expect((ma < 0) == (mb < 0), el + " volume / boundary");
    if (ma >= 0 && mb >= 0) {
      expect(same_material(a.mats[ma], b.mats[mb]), el + " material");
      expect(coef_of(a, e) == coef_of(b, e), el + " coefficient");
    } else if (ma < 0 && mb < 0) {
      expect(same_bc(a.bcs[-ma - 1], b.bcs[-mb - 1]), el + " boundary condition");
    }
  }
  for (int64_t c = 0; c < a.nconnects; c++) {
    const std::string cn = "connect " + std::to_string(c);
    expect(a.conn_order[c] == b.conn_order[c], cn + " order");
    expect(a.block_pos[c] == b.block_pos[c], cn + " block position");
    expect(a.block_size[c] == b.block_size[c], cn + " block size");
  }
}

int main(int argc, char **argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: binding_check CASE N P [COEF_FILE|-] [ORDER_FILE]\n");
    return 2;
  }
  const std::string cs = argv[1];
  const int n = std::atoi(argv[2]), p = std::atoi(argv[3]);
  const bool is3d = ref_case_is3d(cs);
  const int64_t ncell = is3d ? (int64_t)n * n * n : (int64_t)n * n;
  std::vector<double> coef;
  std::vector<int32_t> order;
  if (argc > 4 && std::string(argv[4]) != "-") coef = read_file<double>(argv[4], ncell);
  if (argc > 5) order = read_file<int32_t>(argv[5], ncell);
  const std::vector<int> order_int(order.begin(), order.end());

  TPZCompMesh *cmesh = ref_case_mesh(cs, n, p, coef, order_int);
  if (!cmesh) return 3;
  // the forcing functions of oracle/ref_cases.h, as device forcing declarations
  std::map<int, gpz_neopz::DeviceForcing> forcing;
  gpz_neopz::DeviceForcing f;
  if (cs == "poisson2d") {
    f.kind = GPZ_F_SINPROD;  // 2 pi^2 sin(pi x) sin(pi y), SetForcingFunction(f, 2)
    f.force[0] = 1.0;
    f.porder = 2;
    forcing[gpz_neopz::kAllMaterials] = f;
  } else if (cs == "darcy2d" || cs == "darcy3d") {
    f.kind = GPZ_F_CONST;  // 1, SetForcingFunction(f, 0)
    f.force[0] = 1.0;
    forcing[gpz_neopz::kAllMaterials] = f;
  }
  gpz_neopz::MeshDesc m;
  const std::string why = gpz_neopz::ExtractMesh(cmesh, forcing, m);
  expect(why.empty(), "ExtractMesh: " + why);
  void *grid = grid_case(cs, n, p, coef.empty() ? nullptr : coef.data(), order.empty() ? nullptr : order.data());
  gpz_mesh_desc gd;
  if (!grid || gpzh_grid_desc(grid, &gd) != GPZ_OK) {
    std::fprintf(stderr, "grid build failed\n");
    return 3;
  }
  if (why.empty()) compare(m.desc, gd);

  // the analysis with the device struct matrix
  gpz_ctx *probe = nullptr;
  const int rc_ctx = gpz_ctx_create(&probe, 0);
  if (probe) gpz_ctx_destroy(probe);
  bool stopped = false;
  double mat_err = -1, rhs_err = -1, sol_err = -1;
  int64_t cg_gpu = -1, cg_ref = -1;
  {
    TPZLinearAnalysis an(cmesh, false);
    gpz_neopz::TPZSSpStructMatrixGPU<STATE> str(cmesh);
    for (auto &kv : forcing) str.SetDeviceForcing(kv.first, kv.second);
    an.SetStructuralMatrix(str);
    TPZStepSolver<STATE> direct;
    direct.SetDirect(ELDLt);
    an.SetSolver(direct);
    try {
      an.Assemble();
    } catch (const std::exception &) {
      stopped = true;
    }
    if (!stopped) {
      // a device is present: hold the device system and CG to the reference's serial assembly and CG
      TPZAutoPointer<TPZMatrix<STATE>> mat = an.MatrixSolver<STATE>().Matrix();
      auto *g = dynamic_cast<TPZSYsmpMatrix<STATE> *>(mat.operator->());
      TPZFMatrix<STATE> rhs_gpu = an.Rhs();
      TPZLinearAnalysis ref(cmesh, false);
      TPZSSpStructMatrix<STATE, TPZStructMatrixOR<STATE>> rstr(cmesh);
      rstr.SetNumThreads(0);
      ref.SetStructuralMatrix(rstr);
      ref.SetSolver(direct);
      ref.Assemble();
      TPZAutoPointer<TPZMatrix<STATE>> rmat = ref.MatrixSolver<STATE>().Matrix();
      auto *r = dynamic_cast<TPZSYsmpMatrix<STATE> *>(rmat.operator->());
      expect(g && r && same_vec(g->IA(), r->IA()) && same_vec(g->JA(), r->JA()), "device CSR pattern");
      mat_err = rhs_err = 0;
      if (g && r && g->A().size() == r->A().size())
        for (int64_t i = 0; i < g->A().size(); i++)
          mat_err = std::max(mat_err, std::abs(g->A()[i] - r->A()[i]) / (1.0 + std::abs(r->A()[i])));
      TPZFMatrix<STATE> &rhs_ref = ref.Rhs();
      for (int64_t i = 0; i < rhs_gpu.Rows(); i++)
        rhs_err = std::max(rhs_err, std::abs(rhs_gpu(i, 0) - rhs_ref(i, 0)) / (1.0 + std::abs(rhs_ref(i, 0))));
      expect(mat_err <= 1e-12 && rhs_err <= 1e-12, "device values");
      const REAL tol = 1e-10;
      TPZStepSolver<STATE> jac(mat), cg(mat), rjac(rmat), rcg(rmat);
      jac.SetJacobi(1, 0., 0);
      cg.SetCG(200000, jac, tol, 0);
      an.SetSolver(cg);
      an.Solve();
      rjac.SetJacobi(1, 0., 0);
      rcg.SetCG(200000, rjac, tol, 0);
      ref.SetSolver(rcg);
      ref.Solve();
      cg_gpu = dynamic_cast<TPZStepSolver<STATE> *>(an.Solver())->NumIterations();
      cg_ref = dynamic_cast<TPZStepSolver<STATE> *>(ref.Solver())->NumIterations();
      TPZFMatrix<STATE> &xs = an.Solution(), &xr = ref.Solution();
      double num = 0, den = 0;
      for (int64_t i = 0; i < xr.Rows(); i++) {
        const double d = xs(i, 0) - xr(i, 0);
        num += d * d;
        den += xr(i, 0) * xr(i, 0);
      }
      sol_err = std::sqrt(num / std::max(den, 1e-300));
      expect(sol_err <= 1e-8, "device CG solution");
    } else {
      expect(rc_ctx == GPZ_E_NO_DEVICE, "DebugStop without a GPU but gpz_ctx_create gave " + std::to_string(rc_ctx));
    }
  }
  std::printf("{\"case\": \"%s\", \"n\": %d, \"p\": %d, \"nel\": %lld, \"neq\": %lld, \"nconnects\": %lld, "
              "\"nmats\": %d, \"nbcs\": %d, \"ctx_create\": %d, \"stopped\": %s, \"mat_err\": %g, "
              "\"rhs_err\": %g, \"sol_err\": %g, \"cg_gpu\": %lld, \"cg_ref\": %lld, \"mismatches\": [",
              cs.c_str(), n, p, (long long)m.desc.nel, (long long)m.desc.neq, (long long)m.desc.nconnects,
              m.desc.nmat, m.desc.nbc, rc_ctx, stopped ? "true" : "false", mat_err, rhs_err, sol_err,
              (long long)cg_gpu, (long long)cg_ref);
  for (size_t i = 0; i < g_bad.size(); i++) std::printf("%s\"%s\"", i ? ", " : "", g_bad[i].c_str());
  std::printf("]}\n");
  gpzh_grid_free(grid);
  TPZGeoMesh *gmesh = cmesh->Reference();
  delete cmesh;
  delete gmesh;
  return g_bad.empty() ? 0 : 1;
}
