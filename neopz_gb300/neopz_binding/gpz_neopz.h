// NeoPZ-side binding of the GPU path: the C++ classes a NeoPZ program uses in
// place of the reference's CPU struct matrix and sparse matrix, built on the
// C ABI of include/gpz.h.  Header-only; compile it with the NeoPZ headers
// (and -include cstdint with g++ 13) and link libgpz.so next to libpz.
//
//   TPZSSpStructMatrixGPU<STATE> str(cmesh);       // in place of
//                                                  // TPZSSpStructMatrix<STATE, TPZStructMatrixOR<STATE>>
//   an.SetStructuralMatrix(str);
//   an.Assemble();   // Create(): mesh upload + device pattern; Assemble(): device assembly
//   an.Solve();      // TPZStepSolver -> TPZSYsmpMatrixGPU::SolveCG / SolveJacobi -> gpz_solve
//
// Classes and the reference interfaces they implement:
//   TPZStructMatrixGPU<TVar>: the parallel layer, TPZStrMatParInterface
//     (StrMatrix/TPZStrMatParInterface.h:44-91), in place of TPZStructMatrixOR
//     (StrMatrix/pzstrmatrixor.h:30);
//   TPZSSpStructMatrixGPU<TVar>: the symmetric struct matrix, TPZStructMatrixT
//     + the layer above, in place of TPZSSpStructMatrix
//     (StrMatrix/TPZSSpStructMatrix.h:18); Create() builds the
//     TPZSSpStructMatrix pattern on the device (bit-exact with
//     SetupMatrixData, StrMatrix/TPZSSpStructMatrix.cpp:31-193);
//   TPZSYsmpMatrixGPU<TVar>: TPZSYsmpMatrix (Matrix/pzsysmp.h:20-240) whose
//     MultAdd / SolveCG / SolveJacobi (Matrix/pzmatrix.h:204,417,460) run on
//     the device; the values are also kept on the host (A()) after each
//     assembly, so every other TPZSYsmpMatrix member works unchanged.
//   ExtractMesh(): the gpz_mesh_desc of a TPZCompMesh (the arrays
//     TPZCompMesh::ComputeElGraph and TPZElementMatrix::
//     ComputeDestinationIndices read, Mesh/pzcmesh.cpp:1214-1262,
//     Mesh/pzelmat.cpp:37-96).
//
// Errors follow the reference's convention: a negative status becomes
// DebugStop() (Common/pzerror.cpp:7-27), which throws.  There is no CPU
// fallback: without a GPU, Create() stops at gpz_ctx_create.
#pragma once

#include <cmath>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "DarcyFlow/TPZDarcyFlow.h"
#include "TPZBndCondT.h"
#include "TPZElasticity3D.h"
#include "TPZMatPoisson.h"
#include "TPZStrMatParInterface.h"
#include "TPZStructMatrixT.h"
#include "gpz.h"
#include "pzcmesh.h"
#include "pzerror.h"
#include "pzgmesh.h"
#include "pzblockdiag.h"
#include "pzinterpolationspace.h"
#include "pzseqsolver.h"
#include "pzstepsolver.h"
#include "pzsysmp.h"
#include "tpzsparseblockdiagonal.h"

namespace gpz_neopz {

// A device-evaluable forcing of a volume material: the reference keeps its
// forcing function as an opaque std::function (TPZMaterialT::fForcingFunction),
// so the program declares it per material id (kind GPZ_F_*, force values, the
// SetForcingFunction pOrder), or once for every material under kAllMaterials.
// TPZElasticity3D's constant body force (its fForce) is read from the material.
struct DeviceForcing {
  int kind = GPZ_F_NONE;
  double force[3] = {0.0, 0.0, 0.0};
  int porder = 0;
};
constexpr int kAllMaterials = -2147483647 - 1;

// TPZElasticity3D's body force: a protected member read through a derived class's pointer to member.
struct Elasticity3DForce : TPZElasticity3D {
  static const TPZManVector<STATE, 3> &Of(const TPZElasticity3D &m) { return m.*(&Elasticity3DForce::fForce); }
};

// Owns the arrays a gpz_mesh_desc points into.
struct MeshDesc {
  std::vector<double> xyz, coef;
  std::vector<int32_t> type, mat, order, corder, bsize;
  std::vector<int64_t> nodes, conn, bpos;
  std::vector<gpz_material> mats;
  std::vector<gpz_bc> bcs;
  gpz_mesh_desc desc{};
};

inline int gpz_type_of(MElementType t) {
  return t == EOned ? GPZ_EL_LINE : t == EQuadrilateral ? GPZ_EL_QUAD : t == ECube ? GPZ_EL_HEX : 0;
}

// The descriptor of cmesh (after AutoBuild and the analysis' equation
// numbering).  Volume materials of one kind and the same constant data
// share one gpz_material; the per-element Young modulus (TPZElasticity3D::
// GetE) or permeability (TPZDarcyFlow::GetPermeability at the element's
// centroid) goes to el_coef.  Returns an empty string, or why the mesh
// cannot go to the device (element or material outside the supported set).
inline std::string ExtractMesh(TPZCompMesh *cmesh, const std::map<int, DeviceForcing> &forcing, MeshDesc &m) {
  TPZGeoMesh *gmesh = cmesh->Reference();
  const int64_t nnodes = gmesh->NNodes();
  m = MeshDesc{};
  m.xyz.resize(3 * nnodes);
  for (int64_t i = 0; i < nnodes; i++)
    for (int j = 0; j < 3; j++) m.xyz[3 * i + j] = gmesh->NodeVec()[i].Coord(j);
  std::map<const TPZMaterial *, int> volmat, bcmat;
  std::map<std::vector<double>, int> volkey;
  int nstate = 1;
  for (int64_t el = 0; el < cmesh->NElements(); el++) {
    TPZCompEl *cel = cmesh->Element(el);
    if (!cel) continue;
    TPZGeoEl *gel = cel->Reference();
    const int t = gpz_type_of(gel->Type());
    if (!t) return "element type outside line / quadrilateral / hexahedron";
    TPZMaterial *mat = cel->Material();
    int32_t mref = 0;
    double coef = 1.0;
    if (auto *bc = dynamic_cast<TPZBndCondT<STATE> *>(mat)) {
      auto it = bcmat.find(mat);
      if (it == bcmat.end()) {
        if (bc->Type() != 0 && bc->Type() != 1) return "boundary condition type other than 0 / 1";
        gpz_bc b{};
        b.type = bc->Type();
        b.material = 0;  // the BC contributions do not read the volume coefficient
        const TPZFMatrix<STATE> &v1 = bc->Val1();
        for (int i = 0; i < v1.Rows() && i < 3; i++)
          for (int j = 0; j < v1.Cols() && j < 3; j++) b.val1[3 * i + j] = v1.GetVal(i, j);
        for (int i = 0; i < bc->Val2().size() && i < 3; i++) b.val2[i] = bc->Val2()[i];
        it = bcmat.emplace(mat, (int)m.bcs.size()).first;
        m.bcs.push_back(b);
      }
      mref = -it->second - 1;
    } else {
      gpz_material g{};
      g.scale = 1.0;
      g.E = 1.0;
      g.nu = 0.3;
      g.coef_const = 1.0;
      g.bignumber = mat->BigNumber();
      auto fh = forcing.find(mat->Id());
      if (fh == forcing.end()) fh = forcing.find(kAllMaterials);
      if (fh != forcing.end()) {
        g.forcing = fh->second.kind;
        for (int j = 0; j < 3; j++) g.force[j] = fh->second.force[j];
        g.forcing_porder = fh->second.porder;
      }
      if (auto *e3 = dynamic_cast<TPZElasticity3D *>(mat)) {
        g.kind = GPZ_MAT_ELAST3D;
        g.dim = 3;
        g.nu = e3->GetPoisson();
        coef = e3->GetE();
        nstate = 3;
        for (int j = 0; j < 3; j++)
          if (e3->GetPrestress(j) != 0.0) return "TPZElasticity3D with a prestress";
        if (fh == forcing.end()) {  // TPZElasticity3D::Contribute adds fForce at every point
          g.forcing = GPZ_F_CONST;
          for (int j = 0; j < 3; j++) g.force[j] = Elasticity3DForce::Of(*e3)[j];
        }
      } else if (auto *d = dynamic_cast<TPZDarcyFlow *>(mat)) {
        g.kind = GPZ_MAT_DARCY;
        g.dim = d->Dimension();
        TPZManVector<REAL, 3> xc(3, 0.0), xi(gel->Dimension(), 0.0);
        gel->CenterPoint(gel->NSides() - 1, xi);
        gel->X(xi, xc);
        coef = d->GetPermeability(xc);
      } else if (auto *p = dynamic_cast<TPZMatPoisson<STATE> *>(mat)) {
        g.kind = GPZ_MAT_POISSON;
        g.dim = p->Dimension();
        g.scale = p->ScaleFactor();
      } else {
        return "volume material other than TPZMatPoisson / TPZDarcyFlow / TPZElasticity3D";
      }
      if (g.forcing == GPZ_F_NONE && mat->HasForcingFunction())
        return "a forcing function without a DeviceForcing declaration for material " + std::to_string(mat->Id());
      const std::vector<double> key{(double)g.kind, (double)g.dim, g.scale, g.nu, (double)g.forcing, g.force[0],
                                    g.force[1], g.force[2], (double)g.forcing_porder, g.bignumber};
      auto it = volkey.find(key);
      if (it == volkey.end()) {
        it = volkey.emplace(key, (int)m.mats.size()).first;
        m.mats.push_back(g);
      }
      mref = it->second;
    }
    m.type.push_back(t);
    m.mat.push_back(mref);
    m.coef.push_back(coef);
    auto *isp = dynamic_cast<TPZInterpolationSpace *>(cel);
    m.order.push_back(isp ? isp->GetPreferredOrder() : 1);
    for (int k = 0; k < 8; k++) m.nodes.push_back(k < gel->NCornerNodes() ? gel->NodeIndex(k) : -1);
    const int64_t first = m.conn.size();
    for (int sd = 0; sd < 27; sd++)  // slots past the element's sides repeat its first connect
      m.conn.push_back(sd < gel->NSides() ? cmesh->ConnectVec()[cel->ConnectIndex(sd)].SequenceNumber() : m.conn[first]);
  }
  const int64_t nconn = cmesh->Block().NBlocks();
  m.corder.assign(nconn, 0);
  m.bpos.assign(nconn, 0);
  m.bsize.assign(nconn, 0);
  for (int64_t ci = 0; ci < cmesh->NConnects(); ci++) {
    const TPZConnect &c = cmesh->ConnectVec()[ci];
    const int64_t sq = c.SequenceNumber();
    if (sq < 0 || sq >= nconn) continue;
    m.corder[sq] = c.Order();
  }
  for (int64_t sq = 0; sq < nconn; sq++) {
    m.bpos[sq] = cmesh->Block().Position((int)sq);
    m.bsize[sq] = cmesh->Block().Size((int)sq);
  }
  gpz_mesh_desc &d = m.desc;
  d.dim = cmesh->Dimension();
  d.nstate = nstate;
  d.nnodes = nnodes;
  d.node_xyz = m.xyz.data();
  d.nel = (int64_t)m.type.size();
  d.el_type = m.type.data();
  d.el_mat = m.mat.data();
  d.el_nodes = m.nodes.data();
  d.el_order = m.order.data();
  d.el_conn = m.conn.data();
  d.el_coef = m.coef.data();
  d.nconnects = nconn;
  d.conn_order = m.corder.data();
  d.block_pos = m.bpos.data();
  d.block_size = m.bsize.data();
  d.neq = cmesh->NEquations();
  d.nmat = (int32_t)m.mats.size();
  d.mats = m.mats.data();
  d.nbc = (int32_t)m.bcs.size();
  d.bcs = m.bcs.data();
  return "";
}

// The column-major storage of a TPZFMatrix (its Elem() is protected)
template <class TVar>
inline TVar *Data(TPZFMatrix<TVar> &m) {
  return m.Rows() * m.Cols() ? &m(0, 0) : nullptr;
}
template <class TVar>
inline const TVar *Data(const TPZFMatrix<TVar> &m) {
  return m.Rows() * m.Cols() ? &const_cast<TPZFMatrix<TVar> &>(m)(0, 0) : nullptr;
}

inline int check(int rc, gpz_ctx *ctx = nullptr) {
  if (rc < 0) {
    PZError << "gpz: " << gpz_get_error_string(rc) << (ctx ? std::string(" (") + gpz_last_error_detail(ctx) + ")" : "")
            << std::endl;
    DebugStop();
  }
  return rc;
}

// One device context shared by a struct matrix, its clones and the matrices it creates.
struct Device {
  gpz_ctx *ctx = nullptr;
  MeshDesc mesh;
  int assembled = -1;  // precision of the last gpz_assemble (GPZ_PREC_*), -1 before the first
  Device() { check(gpz_ctx_create(&ctx, 0)); }
  Device(const Device &) = delete;
  Device &operator=(const Device &) = delete;
  ~Device() {
    if (ctx) gpz_ctx_destroy(ctx);
  }
  void Assemble(int precision) {
    check(gpz_assemble(ctx, precision), ctx);
    assembled = precision;
  }
};

// The device preconditioner of the preconditioner TPZStepSolver::SetCG was given:
//   a Jacobi step solver (SetJacobi)                          -> GPZ_PRECOND_JACOBI;
//   a step solver over a TPZSparseBlockDiagonal, or the TPZSequenceSolver of
//   TPZAnalysis::BuildPreconditioner(EBlockJacobi, false)
//   (Analysis/TPZAnalysis.cpp:1008-1085: node-set blocks)  -> GPZ_PRECOND_NODESET_JACOBI;
//   a step solver over a TPZBlockDiagonal (BuildPreconditioner(EBlockJacobi, true):
//   TPZBlockDiagonalStructMatrix, one block per connect)   -> GPZ_PRECOND_BLOCK_JACOBI;
// -1 for anything else (the other block kinds of BuildPreconditioner have no
// device counterpart: name one with SetDevicePreconditioner).
template <class TVar>
inline int DevicePrecondOf(TPZSolver &pre) {
  if (dynamic_cast<TPZSequenceSolver<TVar> *>(&pre)) return GPZ_PRECOND_NODESET_JACOBI;
  if (auto *ms = dynamic_cast<TPZMatrixSolver<TVar> *>(&pre)) {
    if (ms->Solver() == TPZMatrixSolver<TVar>::EJacobi) return GPZ_PRECOND_JACOBI;
    TPZMatrix<TVar> *m = ms->Matrix().operator->();
    if (dynamic_cast<TPZSparseBlockDiagonal<TVar> *>(m)) return GPZ_PRECOND_NODESET_JACOBI;
    if (dynamic_cast<TPZBlockDiagonal<TVar> *>(m)) return GPZ_PRECOND_BLOCK_JACOBI;
  }
  return -1;
}

// TPZSYsmpMatrix whose products and iterative solves run on the device.
template <class TVar = STATE>
class TPZSYsmpMatrixGPU : public TPZSYsmpMatrix<TVar> {
 public:
  TPZSYsmpMatrixGPU(int64_t rows, int64_t cols, std::shared_ptr<Device> dev)
      : TPZSYsmpMatrix<TVar>(rows, cols), fDev(std::move(dev)) {}
  TPZSYsmpMatrixGPU(const TPZSYsmpMatrixGPU &) = default;
  TPZMatrix<TVar> *Clone() const override { return new TPZSYsmpMatrixGPU(*this); }
  // z = alpha A x + beta y (opt: transpose, the same for a symmetric matrix)
  void MultAdd(const TPZFMatrix<TVar> &x, const TPZFMatrix<TVar> &y, TPZFMatrix<TVar> &z, const TVar alpha = 1.,
               const TVar beta = 0., const int opt = 0) const override {
    if (x.Cols() != 1) {
      TPZSYsmpMatrix<TVar>::MultAdd(x, y, z, alpha, beta, opt);
      return;
    }
    z.Redim(this->Rows(), 1);
    check(gpz_spmv(fDev->ctx, alpha, Data(x), beta, beta != TVar(0) ? Data(y) : nullptr, Data(z)), fDev->ctx);
  }
  // TPZStepSolver::SetCG(n, pre, tol, FromCurrent) (Matrix/pzmatrix.cpp:750-758
  // -> cg.h): the device CG with the preconditioner DevicePrecondOf maps `pre`
  // to, or the one SetDevicePreconditioner chose (then the mixed CG if asked)
  void SolveCG(int64_t &numiterations, TPZSolver &preconditioner, const TPZFMatrix<TVar> &F,
               TPZFMatrix<TVar> &result, TPZFMatrix<TVar> *residual, REAL &tol, const int FromCurrent = 0) override {
    gpz_solver_opts o{};
    o.solver = fMixed ? GPZ_SOLVER_MIXED_CG : GPZ_SOLVER_CG;
    o.precond = fPrecondSet ? fPrecond : DevicePrecondOf<TVar>(preconditioner);
    if (o.precond < 0) {
      PZError << "TPZSYsmpMatrixGPU::SolveCG: no device counterpart of this preconditioner "
                 "(SetDevicePreconditioner names one)" << std::endl;
      DebugStop();
    }
    o.max_iter = numiterations;
    o.tol = tol;
    o.check_every = 32;
    o.use_graph = 1;
    o.reliable_delta = 1e-2;
    o.from_current = FromCurrent;
    o.spmv_variant = -1;
    gpz_solve_report rep{};
    result.Redim(this->Rows(), 1);
    if (fMixed && fDev->assembled != GPZ_PREC_MIXED) fDev->Assemble(GPZ_PREC_MIXED);  // + the FP32 operator
    check(gpz_solve(fDev->ctx, &o, Data(F), Data(result), &rep), fDev->ctx);
    if (residual) {
      residual->Redim(this->Rows(), 1);
      check(gpz_spmv(fDev->ctx, -1.0, Data(result), 1.0, Data(F), Data(*residual)), fDev->ctx);
    }
    numiterations = rep.iterations;  // as TPZStepSolver reports them (Solvers/pzstepsolver.cpp:107-112)
    tol = rep.resid;
  }
  // TPZStepSolver::SetGMRES(n, numvectors, pre, tol, FromCurrent) (Solvers/LinearSolvers/gmres.h:68-168):
  // the device GMRES(numvectors) with Jacobi or 3x3-block Jacobi
  void SolveGMRES(int64_t &numiterations, TPZSolver &preconditioner, TPZFMatrix<TVar> &H, int &numvectors,
                  const TPZFMatrix<TVar> &F, TPZFMatrix<TVar> &result, TPZFMatrix<TVar> *residual, REAL &tol,
                  const int FromCurrent) override {
    gpz_solver_opts o{};
    o.solver = GPZ_SOLVER_GMRES;
    o.precond = fPrecondSet ? fPrecond : DevicePrecondOf<TVar>(preconditioner);
    if (o.precond == GPZ_PRECOND_NODESET_JACOBI) o.precond = GPZ_PRECOND_BLOCK_JACOBI;
    if (o.precond != GPZ_PRECOND_JACOBI && o.precond != GPZ_PRECOND_BLOCK_JACOBI) {
      PZError << "TPZSYsmpMatrixGPU::SolveGMRES: the device GMRES takes Jacobi or block Jacobi" << std::endl;
      DebugStop();
    }
    o.gmres_krylov = numvectors;
    o.max_iter = numiterations;
    o.tol = tol;
    o.use_graph = 1;
    o.from_current = FromCurrent;
    gpz_solve_report rep{};
    result.Redim(this->Rows(), 1);
    check(gpz_solve(fDev->ctx, &o, Data(F), Data(result), &rep), fDev->ctx);
    if (residual) {
      residual->Redim(this->Rows(), 1);
      check(gpz_spmv(fDev->ctx, -1.0, Data(result), 1.0, Data(F), Data(*residual)), fDev->ctx);
    }
    numiterations = rep.iterations;
    tol = rep.resid;
  }
  // TPZStepSolver::SetJacobi(n, tol, FromCurrent) as the solver (Matrix/pzmatrix.cpp:643-667)
  void SolveJacobi(int64_t &numiterations, const TPZFMatrix<TVar> &F, TPZFMatrix<TVar> &result,
                   TPZFMatrix<TVar> *residual, TPZFMatrix<TVar> &scratch, REAL &tol,
                   const int FromCurrent = 0) override {
    gpz_solver_opts o{};
    o.solver = GPZ_SOLVER_JACOBI;
    o.max_iter = numiterations;
    o.tol = tol;
    o.check_every = 32;
    o.use_graph = 1;
    o.from_current = FromCurrent;
    gpz_solve_report rep{};
    result.Redim(this->Rows(), 1);
    check(gpz_solve(fDev->ctx, &o, Data(F), Data(result), &rep), fDev->ctx);
    if (residual) {
      residual->Redim(this->Rows(), 1);
      check(gpz_spmv(fDev->ctx, -1.0, Data(result), 1.0, Data(F), Data(*residual)), fDev->ctx);
    }
  }
  // GPZ_PRECOND_JACOBI / BLOCK_JACOBI / NODESET_JACOBI (CG) or TWO_LEVEL (mixed CG)
  void SetDevicePreconditioner(int precond, bool mixed) {
    fPrecond = precond;
    fPrecondSet = true;
    fMixed = mixed || precond == GPZ_PRECOND_TWO_LEVEL;
  }

 private:
  std::shared_ptr<Device> fDev;
  int fPrecond = GPZ_PRECOND_JACOBI;
  bool fPrecondSet = false;
  bool fMixed = false;
};

// The parallel layer: assembly on the device into the TPZSYsmpMatrixGPU the struct matrix created.
template <class TVar = STATE>
class TPZStructMatrixGPU : public virtual TPZStrMatParInterface {
 public:
  void Assemble(TPZBaseMatrix &stiffness, TPZBaseMatrix &rhs, TPZAutoPointer<TPZGuiInterface> gui) override {
    gpz_set_killed(fDev->ctx, gui && gui->AmIKilled());  // pzstrmatrixor.cpp:490: stop before any work
    const int rc = check(gpz_assemble(fDev->ctx, fPrecision), fDev->ctx);
    if (rc == GPZ_CANCELLED) return;
    fDev->assembled = fPrecision;
    if (auto *s = dynamic_cast<TPZSYsmpMatrix<TVar> *>(&stiffness))
      check(gpz_matrix_download(fDev->ctx, &s->A()[0]), fDev->ctx);  // host copy: GetVal, Print, direct solvers
    auto &f = dynamic_cast<TPZFMatrix<TVar> &>(rhs);
    check(gpz_rhs_download(fDev->ctx, Data(f)), fDev->ctx);
  }
  void Assemble(TPZBaseMatrix &rhs, TPZAutoPointer<TPZGuiInterface> gui) override {  // residual only
    gpz_set_killed(fDev->ctx, gui && gui->AmIKilled());
    if (check(gpz_assemble_rhs(fDev->ctx), fDev->ctx) == GPZ_CANCELLED) return;
    check(gpz_rhs_download(fDev->ctx, Data(dynamic_cast<TPZFMatrix<TVar> &>(rhs))), fDev->ctx);
  }
  void SetDeviceForcing(int matid, const DeviceForcing &f) { fForcing[matid] = f; }
  // GPZ_PREC_FP64 (default) or GPZ_PREC_MIXED: the latter also builds the FP32 operator of the mixed CG
  void SetDevicePrecision(int precision) { fPrecision = precision; }

 protected:
  std::shared_ptr<Device> &Dev() {
    if (!fDev) fDev = std::make_shared<Device>();
    return fDev;
  }
  std::map<int, DeviceForcing> fForcing;
  int fPrecision = GPZ_PREC_FP64;
  std::shared_ptr<Device> fDev;  // created by the first Create()
};

// TPZSSpStructMatrix on the device: the upper-triangular CSR of
// TPZSSpStructMatrix::SetupMatrixData built by gpz_pattern_build.
template <class TVar = STATE>
class TPZSSpStructMatrixGPU : public TPZStructMatrixT<TVar>, public TPZStructMatrixGPU<TVar> {
 public:
  using TPZStructMatrixT<TVar>::TPZStructMatrixT;
  TPZStructMatrix *Clone() override { return new TPZSSpStructMatrixGPU(*this); }
  TPZMatrix<TVar> *Create() override {
    auto &dev = this->Dev();
    const std::string why = ExtractMesh(this->Mesh(), this->fForcing, dev->mesh);
    if (!why.empty()) {
      PZError << "TPZSSpStructMatrixGPU: " << why << std::endl;
      DebugStop();
    }
    check(gpz_mesh_upload(dev->ctx, &dev->mesh.desc), dev->ctx);
    if (this->EquationFilter().IsActive()) {
      const int64_t n = this->EquationFilter().NEqExpand();
      TPZVec<int64_t> orig(n), dest(n);
      for (int64_t i = 0; i < n; i++) orig[i] = dest[i] = i;
      this->EquationFilter().Filter(orig, dest);
      check(gpz_equation_filter(dev->ctx, orig.size(), &orig[0]), dev->ctx);
    }
    int64_t nnz = 0;
    check(gpz_pattern_build(dev->ctx, 1, &nnz), dev->ctx);
    const int64_t neq = this->EquationFilter().NActiveEquations();
    auto *mat = new TPZSYsmpMatrixGPU<TVar>(neq, neq, dev);
    TPZVec<int64_t> IA(neq + 1), JA(nnz);
    TPZVec<TVar> A(nnz, 0.);
    check(gpz_pattern_download(dev->ctx, &IA[0], &JA[0]), dev->ctx);
    mat->SetData(IA, JA, A);
    return mat;
  }
  int ClassId() const override { return Hash("TPZSSpStructMatrixGPU") ^ TPZStructMatrixT<TVar>::ClassId() << 1; }
  void Read(TPZStream &buf, void *context) override { TPZStructMatrixT<TVar>::Read(buf, context); }
  void Write(TPZStream &buf, int withclassid) const override { TPZStructMatrixT<TVar>::Write(buf, withclassid); }
};

}  // namespace gpz_neopz
