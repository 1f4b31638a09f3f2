// Exact-solution error norms on the device: TPZAnalysis::PostProcessError
// (Analysis/TPZAnalysis.cpp:625-650) -> TPZCompMesh::EvaluateError
// (Mesh/pzcmesh.cpp:1497-1551) -> TPZInterpolationSpace::EvaluateError
// (Mesh/pzinterpolationspace.cpp:1108-1200) -> the material's Errors().
//
// The reference calls a user function for the exact solution at every point;
// across the C ABI the exact solution is data instead.  gpz_error_points
// lists the physical coordinates of every error-rule point (element after
// element, volume elements only), the caller evaluates its exact solution
// there, and gpz_error_evaluate integrates the norms: one CTA per element,
// one thread per point, the element's solution coefficients gathered once into
// shared memory, a fixed-order tree reduction of the point sums (the results do
// not depend on scheduling).  Per-element errors are sqrt(sum_q w |J| v_q), as
// EvaluateError leaves them; the mesh totals are sqrt(sum_e err_e^2) in element
// order, as TPZCompMesh::EvaluateError sums them.
#include <cmath>

#include "gpz_internal.h"
#include "gpz_shapes.h"

namespace gpz {

ErrorEval::~ErrorEval() { reset(); }

void ErrorEval::reset() {
  for (Tab *t : tabs) delete t;
  tabs.clear();
  exact_order = -1;
  npts = 0;
  nerr = 0;
  h_pt_off.clear();
}

namespace {

constexpr int kErrThreads = 128;
constexpr int kMaxErrQp = 1331;  // an order-20 cube rule: 11^3 points

// Error rule order (Mesh/pzinterpolationspace.cpp:1140-1156): the element
// rule's order raised to the exact solution's polynomial order, unless that
// exceeds the rule's maximum (GetMaxOrder: 36 for TPZIntQuad, 20 for
// TPZIntCube3D, Integral/pzquad.h:217,299).  TPZIntQuad::GetOrder returns the
// requested order; TPZIntCube3D::GetOrder the Gauss rule's own order,
// 2 (npoints - 1) (Integral/pzquad.cpp:176-194,289-305,
// Integral/tpzgaussrule.cpp:170-181).
int error_order(int type, int intorder, int exact_order) {
  const int maxo = type == GPZ_EL_HEX ? 20 : 36;
  int prev = intorder;
  if (type == GPZ_EL_HEX) {
    int n = (int)(0.51 * (intorder + 2));
    if (n < 1) n = 1;
    prev = 2 * (n - 1);
  }
  if (maxo > exact_order) return prev > exact_order ? prev : exact_order;
  return maxo;
}

struct ErrArgs {
  const double *phi, *dphi, *w;  // error tables [nq][nt], [nq][dim][nt], [nq]
  const int *sside, *sk;         // table shape -> side, index inside the side
  const uint8_t *act_full, *act_k;
  const int32_t *act_n;          // hp classes: the element's active shapes
  const int64_t *elems;
  int nq, nt, ncorner, dim, nst, kind, mdim, hp, nerr, points_only;
  const double *xyz;
  const int64_t *el_nodes, *el_conn, *bpos;
  const double *coef;
  double coef_const, nu;
  const int64_t *pt_off;
  const double *sol, *uex, *duex;
  double *xout, *el;
  int64_t neq;
  int *err;
};

// Errors() at one point, the per-material formulas of TPZMatPoisson::Errors
// (Material/Poisson/TPZMatPoisson.cpp:173-218), TPZDarcyFlow::Errors
// (Material/DarcyFlow/TPZDarcyFlow.cpp:268-327) and TPZElasticity3D::Errors
// (Material/Elasticity/TPZElasticity3D.cpp:1081-1133, stress of
// ComputeStressVector/ComputeStressTensor :1152-1192 without prestress).
// gradu and due are [3][nst] (direction, state) in xyz coordinates.
template <int NST>
__device__ __forceinline__ void material_errors(const ErrArgs &P, double coef, const double (&u)[3],
                                                const double (&gradu)[9], const double *__restrict__ ue,
                                                const double *__restrict__ due, double (&v)[6]) {
#pragma unroll
  for (int k = 0; k < 6; k++) v[k] = 0.0;
  if (NST == 1 && P.kind == GPZ_MAT_POISSON) {
    double diff = u[0] - ue[0];
    v[1] = diff * diff;
#pragma unroll
    for (int id = 0; id < 3; id++)
      if (id < P.mdim) {
        diff = gradu[id] - due[id];
        v[2] += diff * diff;
      }
    v[0] = v[1] + v[2];
  } else if (NST == 1) {  // TPZDarcyFlow
    double diff = fabs(u[0] - ue[0]);
    v[1] = diff * diff;
    double s = 0.0;
#pragma unroll
    for (int id = 0; id < 3; id++)
      if (id < P.mdim) s += coef * fabs(gradu[id] - due[id]);
    v[2] = fabs(s * s);
    v[0] = v[1] + v[2];
#pragma unroll
    for (int id = 0; id < 3; id++)
      if (id < P.mdim) {
        const double d = fabs(due[id] + coef * gradu[id]);  // exact flux - (-k grad u)
        v[3 + id] = d * d;
      }
  } else {
    double L2 = 0.0, semi = 0.0, D[3][3];
    for (int i = 0; i < 3; i++) L2 += (u[i] - ue[i]) * (u[i] - ue[i]);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        D[i][j] = gradu[i * 3 + j] - due[i * 3 + j];
        semi += D[i][j] * D[i][j];
      }
    const double E = coef, ni = P.nu;
    const double c1 = -1. + ni, c2 = -1. + ni + 2. * ni * ni, c3 = 2. * (1. + ni);
    const double s0 = E * (D[0][0] * c1 - (D[1][1] + D[2][2]) * ni) / c2;
    const double s1 = E * (D[1][1] * c1 - (D[0][0] + D[2][2]) * ni) / c2;
    const double s2 = E * (D[2][2] * c1 - (D[0][0] + D[1][1]) * ni) / c2;
    const double s3 = E * (D[1][0] + D[0][1]) / c3;
    const double s4 = E * (D[2][0] + D[0][2]) / c3;
    const double s5 = E * (D[2][1] + D[1][2]) / c3;
    const double S[3][3] = {{s0, s3, s4}, {s3, s1, s5}, {s4, s5, s2}};
    double energy = 0.0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) energy += D[i][j] * S[i][j];
    v[0] = energy;
    v[1] = L2;
    v[2] = semi;
  }
}

// TPZGeoEl::Jacobian (Mesh/pzgeoel.cpp:1167-1345): J^-1 (dim x dim, in axes
// coordinates for a quad), |det J| and the axes (rows; the identity in 3D).
__device__ __forceinline__ double jac_axes(int D, const double (&gx)[3][3], double (&jinv)[3][3],
                                           double (&axes)[3][3]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      jinv[i][j] = 0.0;
      axes[i][j] = i == j ? 1.0 : 0.0;
    }
  if (D == 2) {
    double n1 = 0.0, d12 = 0.0, n2 = 0.0, v1t[3], v2t[3];
    for (int i = 0; i < 3; i++) {
      n1 += gx[i][0] * gx[i][0];
      d12 += gx[i][0] * gx[i][1];
    }
    n1 = sqrt(n1);
    for (int i = 0; i < 3; i++) {
      v1t[i] = gx[i][0] / n1;
      v2t[i] = gx[i][1] - d12 * v1t[i] / n1;
      n2 += v2t[i] * v2t[i];
    }
    n2 = sqrt(n2);
    const double j00 = n1, j01 = d12 / n1, j11 = n2, det = j00 * j11;
    jinv[0][0] = j11 / det;
    jinv[1][1] = j00 / det;
    jinv[0][1] = -j01 / det;
    for (int i = 0; i < 3; i++) {
      axes[0][i] = v1t[i];
      axes[1][i] = v2t[i] / n2;
    }
    return fabs(det);
  }
  const double(&a)[3][3] = gx;
  const double det = -a[0][2] * a[1][1] * a[2][0] + a[0][1] * a[1][2] * a[2][0] + a[0][2] * a[1][0] * a[2][1] -
                     a[0][0] * a[1][2] * a[2][1] - a[0][1] * a[1][0] * a[2][2] + a[0][0] * a[1][1] * a[2][2];
  jinv[0][0] = (-a[1][2] * a[2][1] + a[1][1] * a[2][2]) / det;
  jinv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
  jinv[0][2] = (-a[0][2] * a[1][1] + a[0][1] * a[1][2]) / det;
  jinv[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) / det;
  jinv[1][1] = (-a[0][2] * a[2][0] + a[0][0] * a[2][2]) / det;
  jinv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
  jinv[2][0] = (-a[1][1] * a[2][0] + a[1][0] * a[2][1]) / det;
  jinv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
  jinv[2][2] = (-a[0][1] * a[1][0] + a[0][0] * a[1][1]) / det;
  return fabs(det);
}

// One CTA per element of one bucket; D element dimension, NST states.
// points_only: write the physical point coordinates (TPZGeoEl::X) and stop;
// else integrate the error values.
template <int D, int NST>
__global__ void __launch_bounds__(kErrThreads) k_error(ErrArgs P) {
  __shared__ double sC[24];
  __shared__ double sU[kMaxShapes * 3];
  __shared__ int sIdx[kMaxShapes];
  __shared__ double sRed[6][kErrThreads];
  __shared__ double sCoef;
  const int64_t ie = blockIdx.x;
  const int64_t e = P.elems[ie];
  const int tid = threadIdx.x, nc = P.ncorner, nt = P.nt;
  const int NSH = P.hp ? P.act_n[ie] : nt;
  if (tid < nc * 3) {
    const int k = tid / 3, j = tid % 3;
    sC[tid] = P.xyz[P.el_nodes[e * 8 + k] * 3 + j];
  }
  if (!P.points_only) {
    // TPZInterpolationSpace::ReallyComputeSolutionT (Mesh/pzinterpolationspace.cpp:135-178):
    // the element's coefficients, connect block position + shape index * nstate + state
    for (int a = tid; a < NSH; a += blockDim.x) {
      const int fa = P.hp ? (int)P.act_full[ie * kMaxShapes + a] : a;
      const int ka = P.hp ? (int)P.act_k[ie * kMaxShapes + a] : P.sk[a];
      const int64_t row = P.bpos[P.el_conn[e * 27 + P.sside[fa]]] + (int64_t)ka * NST;
      sIdx[a] = fa;
      for (int s = 0; s < NST; s++) {
        double v = 0.0;
        if (row + s < 0 || row + s >= P.neq) atomicOr(P.err, 32);
        else v = P.sol[row + s];
        sU[a * NST + s] = v;
      }
    }
    if (tid == 0) sCoef = P.coef ? P.coef[e] : P.coef_const;
  }
  __syncthreads();
  double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  const int64_t p0 = P.pt_off[e];
  for (int q = tid; q < P.nq; q += blockDim.x) {
    // corner shapes are the table's first nc: they give X and the Jacobian
    double x[3] = {0.0, 0.0, 0.0}, gx[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int k = 0; k < nc; k++) {
      const double ph = P.phi[q * nt + k];
#pragma unroll
      for (int j = 0; j < 3; j++) {
        x[j] += ph * sC[k * 3 + j];
#pragma unroll
        for (int d = 0; d < D; d++) gx[j][d] += sC[k * 3 + j] * P.dphi[(q * D + d) * nt + k];
      }
    }
    if (P.points_only) {
#pragma unroll
      for (int j = 0; j < 3; j++) P.xout[(p0 + q) * 3 + j] = x[j];
      continue;
    }
    double jinv[3][3], axes[3][3];
    const double det = jac_axes(D, gx, jinv, axes);
    double u[3] = {0.0, 0.0, 0.0}, dsol[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int a = 0; a < NSH; a++) {
      const int fa = sIdx[a];
      const double ph = P.phi[q * nt + fa];
      double g[3] = {0.0, 0.0, 0.0};  // dphix = jacinv^T dphi (Mesh/TPZCompElH1.cpp:139-149)
#pragma unroll
      for (int d = 0; d < D; d++)
#pragma unroll
        for (int j = 0; j < D; j++) g[d] += jinv[j][d] * P.dphi[(q * D + j) * nt + fa];
#pragma unroll
      for (int s = 0; s < NST; s++) {
        const double xv = sU[a * NST + s];
        u[s] += ph * xv;
#pragma unroll
        for (int d = 0; d < D; d++) dsol[d][s] += g[d] * xv;
      }
    }
    // TPZAxesTools::Axes2XYZ (Util/pzaxestools.h:61-86): gradu = axes^T dsol
    double gradu[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int s = 0; s < NST; s++) {
        double t = 0.0;
#pragma unroll
        for (int d = 0; d < D; d++) t += axes[d][i] * dsol[d][s];
        gradu[i * NST + s] = t;
      }
    double v[6];
    material_errors<NST>(P, sCoef, u, gradu, P.uex + (p0 + q) * NST, P.duex + (p0 + q) * 3 * NST, v);
    const double wd = P.w[q] * det;
#pragma unroll
    for (int k = 0; k < 6; k++) acc[k] += wd * v[k];
  }
  if (P.points_only) return;
#pragma unroll
  for (int k = 0; k < 6; k++) sRed[k][tid] = acc[k];
  __syncthreads();
  for (int st = kErrThreads / 2; st > 0; st >>= 1) {
    if (tid < st)
#pragma unroll
      for (int k = 0; k < 6; k++) sRed[k][tid] += sRed[k][tid + st];
    __syncthreads();
  }
  if (tid < P.nerr) P.el[e * P.nerr + tid] = sqrt(sRed[tid][0]);
}

}  // namespace

void error_prepare(Ctx &c, int exact_order) {
  ErrorEval &R = c.er;
  if (R.exact_order == exact_order) return;
  R.reset();
  GPZ_REQUIRE(exact_order >= 0, GPZ_E_INVALID, "exact-solution order");
  GPZ_REQUIRE(c.dim >= 2, GPZ_E_UNSUPPORTED_ELEMENT, "error norms need quadrilateral or hexahedral volume elements");
  int nerr = 0;
  for (const gpz_material &m : c.mats) nerr = std::max(nerr, m.kind == GPZ_MAT_DARCY ? 6 : 3);
  std::vector<int64_t> count(c.nel, 0);
  for (size_t bi = 0; bi < c.buckets.size(); bi++) {
    const Bucket *b = c.buckets[bi];
    if (b->key.is_bc || b->dim != c.dim) continue;
    ErrorEval::Tab *t = new ErrorEval::Tab();
    R.tabs.push_back(t);
    t->bucket = (int)bi;
    std::vector<double> pts, w;
    gauss_rule(b->key.type, error_order(b->key.type, b->key.intorder, exact_order), pts, w);
    t->nq = (int)w.size();
    GPZ_REQUIRE(t->nq <= kMaxErrQp, GPZ_E_UNSUPPORTED_ELEMENT, "error rule has too many points");
    const int nt = b->nshape, D = b->dim;
    std::vector<double> phi((size_t)t->nq * nt), dphi((size_t)t->nq * D * nt);
    double ph[kMaxShapes], dph[3 * kMaxShapes];
    for (int q = 0; q < t->nq; q++) {
      const int n = eval_shapes(b->key.type, b->key.orders, b->key.trans, &pts[q * D], ph, dph, kMaxShapes);
      GPZ_REQUIRE(n == nt, GPZ_E_INVALID, "error table shape count");
      for (int a = 0; a < nt; a++) {
        phi[(size_t)q * nt + a] = ph[a];
        for (int d = 0; d < D; d++) dphi[((size_t)q * D + d) * nt + a] = dph[d * kMaxShapes + a];
      }
    }
    t->phi.upload(phi.data(), phi.size(), c.stream);
    t->dphi.upload(dphi.data(), dphi.size(), c.stream);
    t->w.upload(w.data(), w.size(), c.stream);
    for (int64_t e : b->elems) count[e] = t->nq;
  }
  R.h_pt_off.assign(c.nel + 1, 0);
  for (int64_t e = 0; e < c.nel; e++) R.h_pt_off[e + 1] = R.h_pt_off[e] + count[e];
  R.npts = R.h_pt_off[c.nel];
  R.pt_off.upload(R.h_pt_off.data(), R.h_pt_off.size(), c.stream);
  R.nerr = nerr;
  R.exact_order = exact_order;
  GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
}

static void launch_error(Ctx &c, const ErrArgs &P, int64_t nblocks) {
  void (*k)(ErrArgs) = nullptr;
  if (P.dim == 2 && P.nst == 1) k = k_error<2, 1>;
  else if (P.dim == 3 && P.nst == 1) k = k_error<3, 1>;
  else if (P.dim == 3 && P.nst == 3) k = k_error<3, 3>;
  GPZ_REQUIRE(k != nullptr, GPZ_E_UNSUPPORTED_ELEMENT, "error norms for this element dimension / state count");
  k<<<(unsigned)nblocks, kErrThreads, 0, c.stream>>>(P);
  GPZ_CUDA_TRY(cudaGetLastError());
  c.launches++;
}

static ErrArgs err_args(Ctx &c, const ErrorEval::Tab &t, int points_only) {
  const Bucket &b = *c.buckets[t.bucket];
  const gpz_material &m = c.mats[b.key.mat_index];
  ErrArgs P{};
  P.phi = t.phi.p;
  P.dphi = t.dphi.p;
  P.w = t.w.p;
  P.sside = b.d_shape_side.p;
  P.sk = b.d_shape_k.p;
  P.act_full = b.d_act_full.p;
  P.act_k = b.d_act_k.p;
  P.act_n = b.d_act_n.p;
  P.elems = b.d_elems.p;
  P.nq = t.nq;
  P.nt = b.nshape;
  P.ncorner = b.ncorner;
  P.dim = b.dim;
  P.nst = c.nstate;
  P.kind = m.kind;
  P.mdim = m.dim;
  P.hp = b.hp ? 1 : 0;
  P.nerr = c.er.nerr;
  P.points_only = points_only;
  P.xyz = c.d_xyz.p;
  P.el_nodes = c.d_el_nodes.p;
  P.el_conn = c.d_el_conn.p;
  P.bpos = c.d_block_pos.p;
  P.coef = c.d_coef.p;
  P.coef_const = m.kind == GPZ_MAT_ELAST3D ? m.E : m.coef_const;
  P.nu = m.nu;
  P.pt_off = c.er.pt_off.p;
  P.neq = c.neq_mesh;
  P.err = c.d_err.p;
  return P;
}

void error_points(Ctx &c, double *xyz_host) {
  ErrorEval &R = c.er;
  R.xyz.alloc(std::max<int64_t>(R.npts, 1) * 3);
  for (const ErrorEval::Tab *t : R.tabs) {
    const Bucket &b = *c.buckets[t->bucket];
    if (b.elems.empty()) continue;
    ErrArgs P = err_args(c, *t, 1);
    P.xout = R.xyz.p;
    launch_error(c, P, (int64_t)b.elems.size());
  }
  if (R.npts)
    GPZ_CUDA_TRY(cudaMemcpyAsync(xyz_host, R.xyz.p, R.npts * 3 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
}

void error_evaluate(Ctx &c, const double *sol_dev, const double *uex_host, const double *duex_host, double *errors,
                    double *el_host) {
  ErrorEval &R = c.er;
  const int ns = c.nstate;
  R.uex.upload(uex_host, (size_t)R.npts * ns, c.stream);
  R.duex.upload(duex_host, (size_t)R.npts * 3 * ns, c.stream);
  R.el.alloc(std::max<int64_t>(c.nel, 1) * R.nerr);
  R.el.zero(c.stream);
  for (const ErrorEval::Tab *t : R.tabs) {
    const Bucket &b = *c.buckets[t->bucket];
    if (b.elems.empty()) continue;
    ErrArgs P = err_args(c, *t, 0);
    P.sol = sol_dev;
    P.uex = R.uex.p;
    P.duex = R.duex.p;
    P.el = R.el.p;
    launch_error(c, P, (int64_t)b.elems.size());
  }
  std::vector<double> el((size_t)c.nel * R.nerr);
  if (c.nel)
    GPZ_CUDA_TRY(cudaMemcpyAsync(el.data(), R.el.p, el.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
  // TPZCompMesh::EvaluateError: sum of squares in element order, then sqrt
  std::vector<double> tot(R.nerr, 0.0);
  for (int64_t e = 0; e < c.nel; e++)
    for (int k = 0; k < R.nerr; k++) tot[k] += el[(size_t)e * R.nerr + k] * el[(size_t)e * R.nerr + k];
  for (int k = 0; k < R.nerr; k++) errors[k] = std::sqrt(tot[k]);
  if (el_host) std::copy(el.begin(), el.end(), el_host);
}

}  // namespace gpz
