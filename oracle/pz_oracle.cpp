// ============================================================================
//  TEST INFRASTRUCTURE ONLY -- the CPU oracle for the NeoPZ linear FEM path.
//
//  This file restates, in plain single-file C++, what the reference NeoPZ
//  library computes on the path  TPZLinearAnalysis::Assemble -> TPZStructMatrix
//  (TPZSSpStructMatrix / TPZSpStructMatrix, TPZStructMatrixOR) ->
//  TPZCompEl::CalcStiff -> TPZMaterial::Contribute -> TPZSYsmpMatrix/TPZFYsmpMatrix
//  and  TPZLinearAnalysis::Solve -> TPZStepSolver -> CG / GMRES / Jacobi.
//  Every function cites the reference file:line it follows.
//
//  The tests compare the GPU library (libgpz.so) against it, and it is the CPU
//  baseline timed beside it.  The product never links, loads or calls it; only the
//  tests, the smoke check and the CPU-baseline leg of the benchmark do.
//
//  Parity pins (see tests/test_oracle_golden.py): the reference's own unit
//  test golden data (cube elasticity 9x9, Darcy master quad, 1D tridiagonal
//  known matrix) and equation/nnz/iteration counts produced by the reference
//  library on the same synthetic grids.
// ============================================================================
#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <thread>
#include <vector>

namespace orc {

enum { T_LINE = 1, T_QUAD = 2, T_CUBE = 3 };

// ---------------------------------------------------------------------------
// Quadrature: Integral/tpzgaussrule.cpp:170-239 (ComputingGaussLegendreQuadrature).
// Points are stored in the interleaved order -z0,+z0,-z1,+z1,... with z0 the
// largest root; Newton iterations in long double.
// ---------------------------------------------------------------------------
static int gauss_npoints(int order) {
  int n = (int)(0.51 * (order + 2));  // tpzgaussrule.cpp:172
  if (n < 1) n = 1;
  return n;
}

static void gauss_legendre(int n, std::vector<double> &loc, std::vector<double> &w) {
  loc.assign(n, 0.0);
  w.assign(n, 0.0);
  long double tol = 1.0L;
  while (1.0L < (long double)(1.0L + tol)) tol /= 2.0L;  // machinePrecision(), tpzgaussrule.cpp:552-564
  tol *= 2.0L;
  const long double PI = 3.141592653589793238462643383279502884L;
  int m = (n + 1) / 2;
  for (int i = 0; i < m; i++) {
    long double z = cosl(PI * ((long double)i + 0.75L) / ((long double)n + 0.5L));
    long double z1, pp = 0, p1 = 0, p2 = 0, p3;
    for (int it = 0; it < 200; it++) {
      p1 = 1.0L;
      p2 = 0.0L;
      for (int j = 0; j < n; j++) {
        p3 = p2;
        p2 = p1;
        p1 = ((2.0L * j + 1.0L) * z * p2 - j * p3) / (j + 1.0L);
      }
      long double den = z * z - 1.0L;
      pp = n * (z * p1 - p2) / den;
      z1 = z;
      z = z1 - p1 / pp;
      if (fabsl(z - z1) <= tol) break;
    }
    long double weight = 2.0L / ((1.0L - z * z) * pp * pp);
    loc[2 * i] = (double)(-z);
    w[2 * i] = (double)weight;
    if (2 * i + 1 < n) {
      loc[2 * i + 1] = (double)z;
      w[2 * i + 1] = (double)weight;
    }
  }
}

// Tensor rules: TPZIntQuad::Point (Integral/pzquad.cpp:153-167, eta index fastest)
// and TPZIntCube3D::Point (Integral/pzquad.cpp:270-281, ksi index fastest).
struct IntRule {
  int dim = 0;
  std::vector<double> pts;  // [np][dim]
  std::vector<double> wts;
};

static IntRule make_rule(int type, int order) {
  IntRule r;
  int n = gauss_npoints(order);
  std::vector<double> l, w;
  gauss_legendre(n, l, w);
  if (type == T_LINE) {
    r.dim = 1;
    for (int i = 0; i < n; i++) { r.pts.push_back(l[i]); r.wts.push_back(w[i]); }
  } else if (type == T_QUAD) {
    r.dim = 2;
    for (int ip = 0; ip < n * n; ip++) {
      int ik = ip / n, ie = ip % n;
      r.pts.push_back(l[ik]); r.pts.push_back(l[ie]);
      r.wts.push_back(w[ik] * w[ie]);
    }
  } else {
    r.dim = 3;
    for (int ip = 0; ip < n * n * n; ip++) {
      int ik = ip % n, ie = (ip % (n * n)) / n, iz = ip / (n * n);
      r.pts.push_back(l[ik]); r.pts.push_back(l[ie]); r.pts.push_back(l[iz]);
      r.wts.push_back(w[ik] * w[ie] * w[iz]);
    }
  }
  return r;
}

// ---------------------------------------------------------------------------
// Topology tables: Topology/tpzline.cpp, Topology/tpzquadrilateral.cpp:236-240,
// Topology/tpzcube.cpp:31-82,899-931, Topology/tpzcube.h:271-275.
// ---------------------------------------------------------------------------
static const int kCubeEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 4}, {1, 5},
                                     {2, 6}, {3, 7}, {4, 5}, {5, 6}, {6, 7}, {7, 4}};
static const int kCubeFace[6][4] = {{0, 1, 2, 3}, {0, 1, 5, 4}, {1, 2, 6, 5},
                                    {3, 2, 6, 7}, {0, 3, 7, 4}, {4, 5, 6, 7}};
static const int kCubeHigh[27][7] = {
    {8, 11, 12, 20, 21, 24, 26}, {8, 9, 13, 20, 21, 22, 26}, {9, 10, 14, 20, 22, 23, 26},
    {10, 11, 15, 20, 23, 24, 26}, {12, 16, 19, 21, 24, 25, 26}, {13, 16, 17, 21, 22, 25, 26},
    {14, 17, 18, 22, 23, 25, 26}, {15, 18, 19, 23, 24, 25, 26}, {20, 21, 26}, {20, 22, 26},
    {20, 23, 26}, {20, 24, 26}, {21, 24, 26}, {21, 22, 26}, {22, 23, 26}, {23, 24, 26},
    {21, 25, 26}, {22, 25, 26}, {23, 25, 26}, {24, 25, 26}, {26}, {26}, {26}, {26}, {26}, {26}, {-1}};
static const int kCubeNHigh[27] = {7, 7, 7, 7, 7, 7, 7, 7, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 1, 1, 1, 1, 1, 1, 0};

static int nsides(int t) { return t == T_LINE ? 3 : (t == T_QUAD ? 9 : 27); }
static int ncorner(int t) { return t == T_LINE ? 2 : (t == T_QUAD ? 4 : 8); }
static int tdim(int t) { return t; }
static int side_dim(int t, int s) {
  if (s < ncorner(t)) return 0;
  if (t == T_LINE) return 1;
  if (t == T_QUAD) return s < 8 ? 1 : 2;
  return s < 20 ? 1 : (s < 26 ? 2 : 3);
}
// Local corner ids of side s (SideNodeLocId / ContainedSideLocId for the corner part).
static std::vector<int> side_nodes(int t, int s) {
  int nc = ncorner(t);
  if (s < nc) return {s};
  if (t == T_LINE) return {0, 1};
  if (t == T_QUAD) {
    if (s < 8) return {(s - 4) % 4, (s - 3) % 4};
    return {0, 1, 2, 3};
  }
  if (s < 20) return {kCubeEdge[s - 8][0], kCubeEdge[s - 8][1]};
  if (s < 26) return {kCubeFace[s - 20][0], kCubeFace[s - 20][1], kCubeFace[s - 20][2], kCubeFace[s - 20][3]};
  return {0, 1, 2, 3, 4, 5, 6, 7};
}

// NConnectShapeF: Shape/pzshapelinear.cpp:367-372, Shape/pzshapequad.cpp:468-480,
// Shape/pzshapecube.cpp:555-566.
static int nconnect_shape(int t, int s, int order) {
  int d = side_dim(t, s);
  if (d == 0) return 1;
  if (d == 1) return order - 1;
  if (d == 2) return (order - 1) * (order - 1);
  return (order - 1) * (order - 1) * (order - 1);
}

// TPZQuadrilateral::GetTransformId (Topology/tpzquadrilateral.cpp:591-618).
static int quad_transform_id(const int64_t *id) {
  int id0 = (id[0] < id[1]) ? 0 : 1;
  int id1 = (id[2] < id[3]) ? 2 : 3;
  int minid = (id[id0] < id[id1]) ? id0 : id1;
  id0 = (minid + 1) % 4;
  id1 = (minid + 3) % 4;
  int64_t mg = id[minid];
  if (id[id0] < id[id1]) {
    if (mg == id[0]) return 0;
    if (mg == id[1]) return 2;
    if (mg == id[2]) return 4;
    if (mg == id[3]) return 6;
  } else {
    if (mg == id[0]) return 1;
    if (mg == id[1]) return 3;
    if (mg == id[2]) return 5;
    if (mg == id[3]) return 7;
  }
  return 0;
}
// TPZShapeQuad::gTrans2dQ (Shape/pzshapequad.cpp:23-32).
static const double kTrans2dQ[8][2][2] = {
    {{1., 0.}, {0., 1.}}, {{0., 1.}, {1., 0.}}, {{0., 1.}, {-1., 0.}}, {{-1., 0.}, {0., 1.}},
    {{-1., 0.}, {0., -1.}}, {{0., -1.}, {-1., 0.}}, {{0., -1.}, {1., 0.}}, {{1., 0.}, {0., -1.}}};

// Side transform = ParametricTransform(transid) * TransformElementToSide(side)
// (Shape/pzgenericshape.cpp:12-68; Topology/tpzcube.cpp:583-655;
//  Topology/tpzquadrilateral.cpp:296-326; Topology/tpzline.cpp:285-300).
// The sum vectors are all zero for these element types.
struct SideTrans {
  int rows = 0, cols = 0;
  double m[3][3] = {{0}};
};

static SideTrans elem_to_side(int t, int s) {
  SideTrans tr;
  tr.rows = side_dim(t, s);
  tr.cols = tdim(t);
  if (t == T_LINE) {
    if (s == 2) tr.m[0][0] = 1.0;
  } else if (t == T_QUAD) {
    switch (s) {
      case 4: tr.m[0][0] = 1.0; break;
      case 5: tr.m[0][1] = 1.0; break;
      case 6: tr.m[0][0] = -1.0; break;
      case 7: tr.m[0][1] = -1.0; break;
      case 8: tr.m[0][0] = 1.0; tr.m[1][1] = 1.0; break;
      default: break;
    }
  } else {
    switch (s) {
      case 8: case 16: tr.m[0][0] = 1.0; break;
      case 9: case 17: tr.m[0][1] = 1.0; break;
      case 10: case 18: tr.m[0][0] = -1.0; break;
      case 11: case 19: tr.m[0][1] = -1.0; break;
      case 12: case 13: case 14: case 15: tr.m[0][2] = 1.0; break;
      case 20: case 25: tr.m[0][0] = 1.0; tr.m[1][1] = 1.0; break;
      case 21: case 23: tr.m[0][0] = 1.0; tr.m[1][2] = 1.0; break;
      case 22: case 24: tr.m[0][1] = 1.0; tr.m[1][2] = 1.0; break;
      case 26: tr.m[0][0] = tr.m[1][1] = tr.m[2][2] = 1.0; break;
      default: break;
    }
  }
  return tr;
}

static SideTrans side_transform(int t, int s, const int64_t *ids) {
  SideTrans te = elem_to_side(t, s);
  int sd = side_dim(t, s);
  if (t == T_CUBE && s == 26) return te;  // interior of a 3D element: no orientation
  std::vector<int> sn = side_nodes(t, s);
  double P[2][2] = {{0, 0}, {0, 0}};
  if (sd == 1) {
    int tid = ids[sn[0]] < ids[sn[1]] ? 0 : 1;  // GetTransformId for ribs
    P[0][0] = tid ? -1.0 : 1.0;                  // TPZShapeLinear::ParametricTransform
  } else if (sd == 2) {
    int64_t loc[4] = {ids[sn[0]], ids[sn[1]], ids[sn[2]], ids[sn[3]]};
    int tid = quad_transform_id(loc);
    P[0][0] = kTrans2dQ[tid][0][0]; P[0][1] = kTrans2dQ[tid][0][1];
    P[1][0] = kTrans2dQ[tid][1][0]; P[1][1] = kTrans2dQ[tid][1][1];
  }
  SideTrans r;
  r.rows = te.rows;
  r.cols = te.cols;
  for (int i = 0; i < sd; i++)
    for (int j = 0; j < te.cols; j++) {
      double acc = 0.0;
      for (int k = 0; k < sd; k++) acc += P[i][k] * te.m[k][j];
      r.m[i][j] = acc;
    }
  return r;
}

// ---------------------------------------------------------------------------
// H1 shape functions: TPZShapeH1<TSHAPE>::Shape (Shape/TPZShapeH1.cpp:41-116)
// with ShapeCorner / ShapeGenerating / ShapeInternal of
// Shape/pzshapelinear.cpp:15-32,195-205,306-312, Shape/pzshapequad.cpp:36-96,317-337,
// Shape/pzshapecube.cpp:36-152,460-530.  fOrthogonal = Chebyshev.
// ---------------------------------------------------------------------------
static void chebyshev(double x, int num, double *phi, double *dphi) {
  if (num <= 0) return;
  phi[0] = 1.0; dphi[0] = 0.0;
  if (num == 1) return;
  phi[1] = x; dphi[1] = 1.0;
  for (int o = 2; o < num; o++) {
    phi[o] = 2.0 * x * phi[o - 1] - phi[o - 2];
    dphi[o] = 2.0 * x * dphi[o - 1] + 2.0 * phi[o - 1] - dphi[o - 2];
  }
}

static void corner_shapes(int t, const double *pt, double *phi, double *dphi /*[3][27]*/) {
  if (t == T_LINE) {
    phi[0] = (1 - pt[0]) / 2.; phi[1] = (1 + pt[0]) / 2.;
    dphi[0 * 27 + 0] = -0.5; dphi[0 * 27 + 1] = 0.5;
    return;
  }
  double x[2] = {(1. - pt[0]) / 2., (1. + pt[0]) / 2.}, dx[2] = {-0.5, 0.5};
  double y[2] = {(1. - pt[1]) / 2., (1. + pt[1]) / 2.}, dy[2] = {-0.5, 0.5};
  if (t == T_QUAD) {
    const int ix[4] = {0, 1, 1, 0}, iy[4] = {0, 0, 1, 1};
    for (int k = 0; k < 4; k++) {
      phi[k] = x[ix[k]] * y[iy[k]];
      dphi[0 * 27 + k] = dx[ix[k]] * y[iy[k]];
      dphi[1 * 27 + k] = x[ix[k]] * dy[iy[k]];
    }
    return;
  }
  double z[2] = {(1. - pt[2]) / 2., (1. + pt[2]) / 2.}, dz[2] = {-0.5, 0.5};
  const int ix[8] = {0, 1, 1, 0, 0, 1, 1, 0}, iy[8] = {0, 0, 1, 1, 0, 0, 1, 1}, iz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  for (int k = 0; k < 8; k++) {
    phi[k] = x[ix[k]] * y[iy[k]] * z[iz[k]];
    dphi[0 * 27 + k] = dx[ix[k]] * y[iy[k]] * z[iz[k]];
    dphi[1 * 27 + k] = x[ix[k]] * dy[iy[k]] * z[iz[k]];
    dphi[2 * 27 + k] = x[ix[k]] * y[iy[k]] * dz[iz[k]];
  }
}

// Blend ("generating") functions for every side, made unitary.
static void shape_generating(int t, double *pb, double *db /*[3][27]*/) {
  int D = tdim(t);
  auto prod = [&](int is, int a, int b) {
    pb[is] = pb[a] * pb[b];
    for (int d = 0; d < D; d++) db[d * 27 + is] = db[d * 27 + a] * pb[b] + pb[a] * db[d * 27 + b];
  };
  if (t == T_LINE) {
    prod(2, 0, 1);
    pb[2] *= 4.; db[2] *= 4.;
    return;
  }
  if (t == T_QUAD) {
    for (int is = 4; is < 8; is++) prod(is, is % 4, (is + 1) % 4);
    prod(8, 0, 2);
    for (int is = 4; is < 8; is++) {
      pb[is] += pb[8];
      for (int d = 0; d < 2; d++) db[d * 27 + is] += db[d * 27 + 8];
      pb[is] *= 4.;
      for (int d = 0; d < 2; d++) db[d * 27 + is] *= 4.;
    }
    pb[8] *= 16.;
    for (int d = 0; d < 2; d++) db[d * 27 + 8] *= 16.;
    return;
  }
  for (int is = 8; is < 20; is++) prod(is, kCubeEdge[is - 8][0], kCubeEdge[is - 8][1]);
  for (int is = 20; is < 26; is++) prod(is, kCubeFace[is - 20][0], kCubeFace[is - 20][2]);
  prod(26, 0, 6);
  for (int is = 8; is < 27; is++) {
    for (int h = 0; h < kCubeNHigh[is]; h++) {
      int hs = kCubeHigh[is][h];
      pb[is] += pb[hs];
      for (int d = 0; d < 3; d++) db[d * 27 + is] += db[d * 27 + hs];
    }
    int sd = side_dim(T_CUBE, is);
    double mult = sd == 1 ? 4. : (sd == 2 ? 16. : 64.);
    pb[is] *= mult;
    for (int d = 0; d < 3; d++) db[d * 27 + is] *= mult;
  }
}

// ShapeInternal(side, x, order): Chebyshev (products) of the side coordinates.
static int shape_internal(int sd, const double *x, int order, double *phin, double *dphin /*[3][64]*/) {
  double p0[8], d0[8], p1[8], d1[8], p2[8], d2[8];
  if (sd == 1) {
    int num = order - 1;
    chebyshev(x[0], num, p0, d0);
    for (int i = 0; i < num; i++) { phin[i] = p0[i]; dphin[i] = d0[i]; }
    return num;
  }
  int o = order - 1;
  chebyshev(x[0], o, p0, d0);
  chebyshev(x[1], o, p1, d1);
  if (sd == 2) {
    for (int i = 0; i < o; i++)
      for (int j = 0; j < o; j++) {
        int idx = i * o + j;
        phin[idx] = p0[i] * p1[j];
        dphin[0 * 64 + idx] = d0[i] * p1[j];
        dphin[1 * 64 + idx] = p0[i] * d1[j];
      }
    return o * o;
  }
  chebyshev(x[2], o, p2, d2);
  for (int i = 0; i < o; i++)
    for (int j = 0; j < o; j++)
      for (int k = 0; k < o; k++) {
        int idx = o * (o * i + j) + k;
        phin[idx] = p0[i] * p1[j] * p2[k];
        dphin[0 * 64 + idx] = d0[i] * p1[j] * p2[k];
        dphin[1 * 64 + idx] = p0[i] * d1[j] * p2[k];
        dphin[2 * 64 + idx] = p0[i] * p1[j] * d2[k];
      }
  return o * o * o;
}

// Evaluate all shapes of an element; returns the number of shapes.
// orders: one per non-corner side; dphi is [dim][maxshape] with row stride ldd.
static int shape_h1(int t, const int64_t *ids, const int *orders, const double *pt, double *phi, double *dphi, int ldd) {
  int D = tdim(t), NC = ncorner(t), NS = nsides(t);
  double cp[27], cd[3 * 27];
  corner_shapes(t, pt, cp, cd);
  for (int k = 0; k < NC; k++) {
    phi[k] = cp[k];
    for (int d = 0; d < D; d++) dphi[d * ldd + k] = cd[d * 27 + k];
  }
  double pb[27], db[3 * 27];
  for (int k = 0; k < NC; k++) {
    pb[k] = cp[k];
    for (int d = 0; d < D; d++) db[d * 27 + k] = cd[d * 27 + k];
  }
  int shape = NC;
  bool any = false;
  for (int s = NC; s < NS; s++) any |= nconnect_shape(t, s, orders[s - NC]) > 0;
  if (!any) return shape;
  shape_generating(t, pb, db);
  for (int s = NC; s < NS; s++) {
    int ns = nconnect_shape(t, s, orders[s - NC]);
    if (ns == 0) continue;
    phi[shape] = pb[s];
    for (int d = 0; d < D; d++) dphi[d * ldd + shape] = db[d * 27 + s];
    shape++;
    if (ns == 1) continue;
    SideTrans tr = side_transform(t, s, ids);
    int sd = side_dim(t, s);
    double out[3] = {0, 0, 0};
    for (int i = 0; i < sd; i++)
      for (int j = 0; j < D; j++) out[i] += tr.m[i][j] * pt[j];
    double phin[64], dphin[3 * 64];
    shape_internal(sd, out, orders[s - NC], phin, dphin);
    double aux[3][64];
    for (int i = 1; i < ns; i++)
      for (int xj = 0; xj < D; xj++) {
        if (sd < 3) {
          double acc = 0.0;
          for (int k = 0; k < sd; k++) acc += tr.m[k][xj] * dphin[k * 64 + i];
          aux[xj][i] = acc;
        } else {
          aux[xj][i] = dphin[xj * 64 + i];
        }
      }
    for (int i = 1; i < ns; i++) {
      phi[shape] = pb[s] * phin[i];
      for (int xj = 0; xj < D; xj++) dphi[xj * ldd + shape] = db[xj * 27 + s] * phin[i] + pb[s] * aux[xj][i];
      shape++;
    }
  }
  return shape;
}

// ---------------------------------------------------------------------------
// Geometry: TPZGeoCube/TPZGeoQuad/TPZGeoLinear::GradX (Geom/TPZGeoCube.h:124-150,
// Geom/pzgeoquad.h:144-168) and TPZGeoEl::Jacobian (Mesh/pzgeoel.cpp:1167-1345).
// ---------------------------------------------------------------------------
struct Jac {
  double detjac;
  double jinv[3][3];
  double x[3];
};

static Jac jacobian(int t, const double *coords /*[nc][3]*/, const double *pt) {
  int NC = ncorner(t), D = tdim(t);
  double cp[27], cd[3 * 27];
  corner_shapes(t, pt, cp, cd);
  double gx[3][3] = {{0}};
  Jac J;
  for (int i = 0; i < 3; i++) {
    J.x[i] = 0.0;
    for (int k = 0; k < NC; k++) J.x[i] += cp[k] * coords[k * 3 + i];
  }
  for (int k = 0; k < NC; k++)
    for (int j = 0; j < 3; j++)
      for (int d = 0; d < D; d++) gx[j][d] += coords[k * 3 + j] * cd[d * 27 + k];
  std::memset(J.jinv, 0, sizeof(J.jinv));
  if (D == 1) {
    double n = 0.0;
    for (int i = 0; i < 3; i++) n += gx[i][0] * gx[i][0];
    n = std::sqrt(n);
    J.detjac = n;
    J.jinv[0][0] = 1.0 / n;
  } else if (D == 2) {
    double n1 = 0.0, d12 = 0.0, v2t[3], n2 = 0.0;
    for (int i = 0; i < 3; i++) { n1 += gx[i][0] * gx[i][0]; d12 += gx[i][0] * gx[i][1]; }
    n1 = std::sqrt(n1);
    for (int i = 0; i < 3; i++) {
      double v1t = gx[i][0] / n1;
      v2t[i] = gx[i][1] - d12 * v1t / n1;
      n2 += v2t[i] * v2t[i];
    }
    n2 = std::sqrt(n2);
    double j00 = n1, j01 = d12 / n1, j10 = 0.0, j11 = n2;
    J.detjac = j00 * j11 - j10 * j01;
    J.jinv[0][0] = +j11 / J.detjac;
    J.jinv[1][1] = +j00 / J.detjac;
    J.jinv[0][1] = -j01 / J.detjac;
    J.jinv[1][0] = -j10 / J.detjac;
  } else {
    double (&a)[3][3] = gx;
    double det = 0.0;
    det -= a[0][2] * a[1][1] * a[2][0];
    det += a[0][1] * a[1][2] * a[2][0];
    det += a[0][2] * a[1][0] * a[2][1];
    det -= a[0][0] * a[1][2] * a[2][1];
    det -= a[0][1] * a[1][0] * a[2][2];
    det += a[0][0] * a[1][1] * a[2][2];
    J.detjac = det;
    J.jinv[0][0] = (-a[1][2] * a[2][1] + a[1][1] * a[2][2]) / det;
    J.jinv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
    J.jinv[0][2] = (-a[0][2] * a[1][1] + a[0][1] * a[1][2]) / det;
    J.jinv[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) / det;
    J.jinv[1][1] = (-a[0][2] * a[2][0] + a[0][0] * a[2][2]) / det;
    J.jinv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
    J.jinv[2][0] = (-a[1][1] * a[2][0] + a[1][0] * a[2][1]) / det;
    J.jinv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
    J.jinv[2][2] = (-a[0][1] * a[1][0] + a[0][0] * a[1][1]) / det;
  }
  return J;
}

// ---------------------------------------------------------------------------
// Mesh, materials, boundary conditions.
// ---------------------------------------------------------------------------
}  // namespace orc

extern "C" {

// Material kinds: TPZMatPoisson (Material/Poisson/TPZMatPoisson.cpp:19-43),
// TPZDarcyFlow (Material/DarcyFlow/TPZDarcyFlow.cpp:19-47),
// TPZElasticity3D CODE3 (Material/Elasticity/TPZElasticity3D.cpp:269-400).
enum { ORC_POISSON = 1, ORC_DARCY = 2, ORC_ELAST3D = 3, ORC_MOCK = 4 };
// Forcing kinds: none, constant vector, 2 pi^2 sin(pi x) sin(pi y) [sin(pi z)] scaled by force[0],
// force[0] + force[1] |x|^2 (the TestError.cpp right-hand side 4 - 2x^2 - 2y^2 with force = (4, -2)).
enum { ORC_F_NONE = 0, ORC_F_CONST = 1, ORC_F_SINPROD = 2, ORC_F_QUADRATIC = 3 };

typedef struct {
  int id;
  int kind;
  int dim;
  double scale;       // TPZMatPoisson::fScale
  double E, nu;       // elasticity
  double force[3];
  int forcing;
  int forcing_porder; // SetForcingFunction(f, pOrder)
  double coef_const;  // constant permeability / conductivity
  double bignumber;   // TPZMaterial::fBigNumber
  double mock_ek[4];  // ORC_MOCK: fixed 2x2 element matrix (1D test material)
} orc_material;

typedef struct {
  int id;
  int matid;  // volume material it refers to
  int type;   // 0 Dirichlet (penalty), 1 Neumann
  double val1[9];
  double val2[3];
} orc_bc;

typedef struct {
  int dim;          // 1, 2 or 3
  int ndiv[3];
  double minX[3], maxX[3];
  int matids[7];
  int create_bc;
  int default_order;
  int nmat;
  orc_material mats[4];
  int nbc;
  orc_bc bcs[8];
  const double *elem_coef;  // per volume element (gel index) coefficient: permeability or E; may be null
  const int *elem_order;    // per volume element preferred order (hp); may be null
} orc_grid_spec;
}

namespace orc {

struct GeoEl {
  int type;
  int matid;
  int64_t nodes[8];
};

struct CompEl {
  int64_t gel;
  int type;
  int is_bc;
  int mat;  // index into mats (volume) or bcs (bc)
  int64_t conn[27];
  int order;  // fPreferredOrder
};

struct Mesh {
  orc_grid_spec spec;
  std::vector<double> coef;
  std::vector<int> elorder;
  std::vector<double> nodes;  // [n][3]
  std::vector<GeoEl> gels;
  int64_t nvol = 0;
  std::vector<CompEl> cels;
  std::vector<int> conn_order, conn_nshape, conn_dim;
  std::vector<int64_t> block_pos, block_size;
  int nstate = 1;
  int64_t neq = 0;
};

static int find_mat(const Mesh &m, int id) {
  for (int i = 0; i < m.spec.nmat; i++)
    if (m.spec.mats[i].id == id) return i;
  return -1;
}
static int find_bc(const Mesh &m, int id) {
  for (int i = 0; i < m.spec.nbc; i++)
    if (m.spec.bcs[i].id == id) return i;
  return -1;
}

// TPZGenGrid2D::Read + SetBC (Pre/TPZGenGrid2D.cpp:64-75,434-503,545-649,706-765)
static void grid2d(Mesh &m) {
  const orc_grid_spec &s = m.spec;
  int nx = s.ndiv[0], ny = s.ndiv[1];
  double dx = (s.maxX[0] - s.minX[0]) / nx, dy = (s.maxX[1] - s.minX[1]) / ny;
  for (int i = 0; i < (nx + 1) * (ny + 1); i++) {
    int ix = i % (nx + 1), iy = i / (nx + 1);
    m.nodes.push_back(s.minX[0] + ix * dx);
    m.nodes.push_back(s.minX[1] + iy * dy);
    m.nodes.push_back(0.0);
  }
  auto G = [&](int x, int y) { return (int64_t)y * (nx + 1) + x; };
  for (int i = 0; i < nx * ny; i++) {
    int xel = i % nx, yel = (i / nx) % ny;
    GeoEl g{T_QUAD, s.matids[0], {G(xel, yel), G(xel + 1, yel), G(xel + 1, yel + 1), G(xel, yel + 1)}};
    m.gels.push_back(g);
  }
  m.nvol = (int64_t)nx * ny;
  if (!s.create_bc) return;
  for (int side = 4; side < 8; side++) {
    int64_t first = 0, last = 0, inc = 1;
    if (side == 4) { first = 0; last = nx; inc = 1; }
    if (side == 5) { first = nx - 1; last = (int64_t)nx * ny; inc = nx; }
    if (side == 6) { first = (int64_t)nx * (ny - 1); last = (int64_t)nx * ny; inc = 1; }
    if (side == 7) { first = 0; inc = nx; last = first + (int64_t)ny * inc; }
    for (int64_t iel = first; iel < last; iel += inc) {
      const GeoEl &v = m.gels[iel];
      GeoEl g{T_LINE, s.matids[side - 3], {v.nodes[(side - 4) % 4], v.nodes[(side - 3) % 4]}};
      m.gels.push_back(g);
    }
  }
}

// TPZGenGrid3D::BuildVolumetricElements / BuildBoundaryElements (Pre/TPZGenGrid3D.cpp:51-235,239-398)
static void grid3d(Mesh &m) {
  const orc_grid_spec &s = m.spec;
  int nx = s.ndiv[0], ny = s.ndiv[1], nz = s.ndiv[2];
  for (int iz = 0; iz <= nz; iz++)
    for (int iy = 0; iy <= ny; iy++)
      for (int ix = 0; ix <= nx; ix++) {
        m.nodes.push_back(s.minX[0] + ((s.maxX[0] - s.minX[0]) * ix) / nx);
        m.nodes.push_back(s.minX[1] + ((s.maxX[1] - s.minX[1]) * iy) / ny);
        m.nodes.push_back(s.minX[2] + ((s.maxX[2] - s.minX[2]) * iz) / nz);
      }
  int64_t sx = nx + 1, sxy = (int64_t)(nx + 1) * (ny + 1);
  for (int iz = 0; iz < nz; iz++)
    for (int iy = 0; iy < ny; iy++)
      for (int ix = 0; ix < nx; ix++) {
        int64_t f = iz * sxy + iy * sx + ix;
        GeoEl g{T_CUBE, s.matids[0], {f, f + 1, f + 1 + sx, f + sx, f + sxy, f + 1 + sxy, f + 1 + sx + sxy, f + sx + sxy}};
        m.gels.push_back(g);
      }
  m.nvol = (int64_t)nx * ny * nz;
  if (!s.create_bc) return;
  // matids order: {vol, zmin, xmin, ymin, xmax, ymax, zmax} (TPZGeoMeshTools.cpp:189-196)
  int mZmin = s.matids[1], mXmin = s.matids[2], mYmin = s.matids[3], mXmax = s.matids[4], mYmax = s.matids[5], mZmax = s.matids[6];
  for (int iz = 0; iz < nz + 1; iz += nz)
    for (int iy = 0; iy < ny; iy++)
      for (int ix = 0; ix < nx; ix++) {
        int64_t f = iz * sxy + iy * sx + ix;
        GeoEl g{T_QUAD, iz == 0 ? mZmin : mZmax, {f, f + 1, f + sx + 1, f + sx}};
        m.gels.push_back(g);
      }
  for (int iz = 0; iz < nz; iz++)
    for (int iy = 0; iy < ny + 1; iy += ny)
      for (int ix = 0; ix < nx; ix++) {
        int64_t f = iz * sxy + iy * sx + ix;
        GeoEl g{T_QUAD, iy == 0 ? mYmin : mYmax, {f, f + 1, f + sxy + 1, f + sxy}};
        m.gels.push_back(g);
      }
  for (int iz = 0; iz < nz; iz++)
    for (int iy = 0; iy < ny; iy++)
      for (int ix = 0; ix < nx + 1; ix += nx) {
        int64_t f = iz * sxy + iy * sx + ix;
        GeoEl g{T_QUAD, ix == 0 ? mXmin : mXmax, {f, f + sx, f + sxy + sx, f + sxy}};
        m.gels.push_back(g);
      }
}

// TPZGeoMesh of a 1D grid of line elements (the StructMatrixUnitTest mesh).
static void grid1d(Mesh &m) {
  const orc_grid_spec &s = m.spec;
  int nx = s.ndiv[0];
  for (int i = 0; i <= nx; i++) {
    m.nodes.push_back(s.minX[0] + ((s.maxX[0] - s.minX[0]) * i) / nx);
    m.nodes.push_back(0.0);
    m.nodes.push_back(0.0);
  }
  for (int i = 0; i < nx; i++) {
    GeoEl g{T_LINE, s.matids[0], {i, i + 1}};
    m.gels.push_back(g);
  }
  m.nvol = nx;
}

// AutoBuild: TPZCreateApproximationSpace::BuildMesh (Mesh/pzcreateapproxspace.cpp:252-325)
// creates computational elements in geometric-element order; each
// TPZCompElH1 constructor (Mesh/TPZCompElH1.cpp:16-24) calls CreateMidSideConnect
// (Mesh/pzintel.cpp:652-730) for every side in side order, reusing the connect of
// a neighbour that already has one and otherwise allocating a new connect whose
// sequence number is the creation count.  In a conforming grid a side is
// identified by the set of its corner nodes.
static void build_comp(Mesh &m) {
  std::map<std::vector<int64_t>, int64_t> side_conn;
  int nstate = 1;
  for (int i = 0; i < m.spec.nmat; i++)
    if (m.spec.mats[i].kind == ORC_ELAST3D) nstate = 3;
  m.nstate = nstate;
  for (int64_t ig = 0; ig < (int64_t)m.gels.size(); ig++) {
    const GeoEl &g = m.gels[ig];
    int imat = find_mat(m, g.matid), ibc = -1;
    if (imat < 0) {
      ibc = find_bc(m, g.matid);
      if (ibc < 0) continue;  // no material object: no computational element
    }
    CompEl c;
    c.gel = ig;
    c.type = g.type;
    c.is_bc = ibc >= 0;
    c.mat = c.is_bc ? ibc : imat;
    c.order = m.spec.default_order;
    if (!c.is_bc && ig < m.nvol && !m.elorder.empty()) c.order = m.elorder[ig];
    for (int s = 0; s < nsides(g.type); s++) {
      std::vector<int> sn = side_nodes(g.type, s);
      std::vector<int64_t> key;
      for (int k : sn) key.push_back(g.nodes[k]);
      std::sort(key.begin(), key.end());
      auto it = side_conn.find(key);
      if (it != side_conn.end()) {
        c.conn[s] = it->second;
      } else {
        int sd = side_dim(g.type, s);
        int order = sd == 0 ? 1 : m.spec.default_order;
        int64_t idx = (int64_t)m.conn_order.size();
        m.conn_order.push_back(order);
        m.conn_dim.push_back(sd);
        m.conn_nshape.push_back(nconnect_shape(g.type, s, order));
        side_conn[key] = idx;
        c.conn[s] = idx;
      }
    }
    m.cels.push_back(c);
  }
  // hp: the harness sets every shared side to the largest preferred order of the
  // volume elements on it (TPZCompElH1::SetSideOrder, Mesh/TPZCompElH1.cpp:165-208,
  // which resizes the connect's block)
  if (!m.elorder.empty()) {
    std::vector<int> mx(m.conn_order.size(), 0);
    for (const CompEl &c : m.cels)
      if (!c.is_bc)
        for (int s = ncorner(c.type); s < nsides(c.type); s++) mx[c.conn[s]] = std::max(mx[c.conn[s]], c.order);
    for (size_t i = 0; i < mx.size(); i++)
      if (m.conn_dim[i] > 0 && mx[i] > 0) m.conn_order[i] = mx[i];
    for (const CompEl &c : m.cels)
      for (int s = 0; s < nsides(c.type); s++) {
        int64_t ci = c.conn[s];
        m.conn_nshape[ci] = nconnect_shape(c.type, s, m.conn_order[ci]);
      }
  }
}

// TPZInterpolatedElement::MaxOrder: the largest order of the element's connects.
// SetSideOrder calls AdjustIntegrationRule (Mesh/pzinterpolationspace.cpp:69-83) on
// every element at a side whose order changed, so the integration order of an hp
// element is IntegrationRuleOrder(MaxOrder); for uniform p it is that of p.
static int max_order(const Mesh &m, const CompEl &c);

static void init_blocks(Mesh &m) {
  int64_t nb = (int64_t)m.conn_order.size();
  m.block_pos.assign(nb + 1, 0);
  m.block_size.assign(nb, 0);
  for (int64_t i = 0; i < nb; i++) {
    m.block_size[i] = (int64_t)m.conn_nshape[i] * m.nstate;
    m.block_pos[i + 1] = m.block_pos[i] + m.block_size[i];
  }
  m.neq = m.block_pos[nb];
}

// Local shape count per connect of a comp element (TPZInterpolationSpace::InitializeElementMatrix,
// Mesh/pzinterpolationspace.cpp:1717-1774) and destination indices
// (TPZElementMatrix::ComputeDestinationIndices, Mesh/pzelmat.cpp:37-96).
static int element_dest(const Mesh &m, const CompEl &c, int64_t *dest) {
  int n = 0;
  for (int s = 0; s < nsides(c.type); s++) {
    int64_t ci = c.conn[s];
    for (int64_t k = 0; k < m.block_size[ci]; k++) dest[n++] = m.block_pos[ci] + k;
  }
  return n;
}

static int max_order(const Mesh &m, const CompEl &c) {
  int mo = 1;
  for (int s = 0; s < nsides(c.type); s++) mo = std::max(mo, m.conn_order[c.conn[s]]);
  return mo;
}

static void side_orders_of(const Mesh &m, const CompEl &c, int *orders) {
  for (int s = ncorner(c.type); s < nsides(c.type); s++) orders[s - ncorner(c.type)] = m.conn_order[c.conn[s]];
}

static void forcing_value(const orc_material &mat, const double *x, double *f) {
  f[0] = f[1] = f[2] = 0.0;
  if (mat.forcing == ORC_F_CONST) {
    f[0] = mat.force[0]; f[1] = mat.force[1]; f[2] = mat.force[2];
  } else if (mat.forcing == ORC_F_SINPROD) {
    const double pi = M_PI;
    double v = mat.force[0] * (mat.dim == 2 ? 2 * pi * pi : 3 * pi * pi) * std::sin(pi * x[0]) * std::sin(pi * x[1]);
    if (mat.dim == 3) v *= std::sin(pi * x[2]);
    f[0] = v;
  } else if (mat.forcing == ORC_F_QUADRATIC) {
    double r2 = x[0] * x[0] + x[1] * x[1];
    if (mat.dim == 3) r2 += x[2] * x[2];
    f[0] = mat.force[0] + mat.force[1] * r2;
  }
}

// Material weak forms at one integration point.  ek is column-major n x n.
static void contribute(int kind, int dim, double scale, double coefE, double nu, double weight, int nshape,
                       const double *phi, const double *dx, int ldd, const double *f, double *ek, double *ef, int n) {
  if (kind == ORC_POISSON) {  // TPZMatPoisson::Contribute (Material/Poisson/TPZMatPoisson.cpp:19-43)
    for (int i = 0; i < nshape; i++) {
      for (int j = 0; j < nshape; j++) {
        double dd = 0.0;
        for (int x = 0; x < dim; x++) dd += dx[x * ldd + i] * dx[x * ldd + j];
        ek[(size_t)j * n + i] += weight * scale * dd;
      }
      ef[i] += weight * scale * phi[i] * f[0];
    }
  } else if (kind == ORC_DARCY) {  // TPZDarcyFlow::Contribute (Material/DarcyFlow/TPZDarcyFlow.cpp:19-47)
    double src = -f[0];
    for (int in = 0; in < nshape; in++) {
      ef[in] -= weight * src * phi[in];
      for (int jn = 0; jn < nshape; jn++)
        for (int kd = 0; kd < dim; kd++) ek[(size_t)jn * n + in] += weight * (dx[kd * ldd + in] * coefE * dx[kd * ldd + jn]);
    }
  } else if (kind == ORC_ELAST3D) {  // TPZElasticity3D::Contribute, CODE3 (Material/Elasticity/TPZElasticity3D.cpp:269-400)
    double E = coefE;
    double C1 = E / (2. + 2. * nu);  // TPZElasticity3D::SetC (Material/Elasticity/TPZElasticity3D.h:183-188)
    double C2 = E * nu / (-1. + nu + 2. * nu * nu);
    double C3 = E * (nu - 1.) / (-1. + nu + 2. * nu * nu);
    for (int jn = 0; jn < nshape; jn++) {
      double dj[3] = {dx[0 * ldd + jn], dx[1 * ldd + jn], dx[2 * ldd + jn]};
      for (int kd = 0; kd < 3; kd++) ef[jn * 3 + kd] += weight * (f[kd] * phi[jn]);
      for (int in = 0; in < nshape; in++) {
        double Dv[3][3];
        for (int ud = 0; ud < 3; ud++)
          for (int vd = 0; vd < 3; vd++) Dv[vd][ud] = dx[vd * ldd + in] * dj[ud];
        auto EK = [&](int r, int cc) -> double & { return ek[(size_t)cc * n + r]; };
        EK(in * 3 + 0, jn * 3 + 0) += weight * ((Dv[1][1] + Dv[2][2]) * C1 + Dv[0][0] * C3);
        EK(in * 3 + 1, jn * 3 + 0) += weight * (Dv[0][1] * C1 - Dv[1][0] * C2);
        EK(in * 3 + 2, jn * 3 + 0) += weight * (Dv[0][2] * C1 - Dv[2][0] * C2);
        EK(in * 3 + 0, jn * 3 + 1) += weight * (Dv[1][0] * C1 - Dv[0][1] * C2);
        EK(in * 3 + 1, jn * 3 + 1) += weight * ((Dv[0][0] + Dv[2][2]) * C1 + Dv[1][1] * C3);
        EK(in * 3 + 2, jn * 3 + 1) += weight * (Dv[1][2] * C1 - Dv[2][1] * C2);
        EK(in * 3 + 0, jn * 3 + 2) += weight * (Dv[2][0] * C1 - Dv[0][2] * C2);
        EK(in * 3 + 1, jn * 3 + 2) += weight * (Dv[2][1] * C1 - Dv[1][2] * C2);
        EK(in * 3 + 2, jn * 3 + 2) += weight * ((Dv[0][0] + Dv[1][1]) * C1 + Dv[2][2] * C3);
      }
    }
  }
}

// TPZInterpolationSpace::CalcStiffInternal (Mesh/pzinterpolationspace.cpp:403-473):
// qp loop, J and dphix = jacinv^T dphi (Mesh/TPZCompElH1.cpp:139-149), weight *= |detJ|,
// then Contribute / ContributeBC.  ek is column-major n x n (TPZFMatrix layout).
static int calc_stiff(const Mesh &m, const CompEl &c, double *ek, double *ef) {
  const GeoEl &g = m.gels[c.gel];
  int t = c.type, NC = ncorner(t), D = tdim(t);
  int orders[26];
  side_orders_of(m, c, orders);
  int nshape = NC;
  for (int s = NC; s < nsides(t); s++) nshape += nconnect_shape(t, s, orders[s - NC]);
  int ns = m.nstate, n = nshape * ns;
  std::fill(ek, ek + (size_t)n * n, 0.0);
  std::fill(ef, ef + n, 0.0);
  double coords[8 * 3];
  for (int k = 0; k < NC; k++)
    for (int j = 0; j < 3; j++) coords[k * 3 + j] = m.nodes[g.nodes[k] * 3 + j];
  // integration order (TPZIntelGen ctor, Mesh/pzelctemp.cpp:36-47; TPZMatSingleSpace.cpp:61-72),
  // of MaxOrder after the hp side orders are set
  int porder = max_order(m, c);
  int intorder;
  const orc_material *vm = c.is_bc ? &m.spec.mats[find_mat(m, m.spec.bcs[c.mat].matid)] : &m.spec.mats[c.mat];
  if (!c.is_bc && vm->kind == ORC_ELAST3D) {
    intorder = 2 * porder;  // TPZElasticity3D::IntegrationRuleOrder
  } else if (!c.is_bc && porder < vm->forcing_porder) {
    intorder = vm->forcing_porder + porder;
  } else {
    intorder = 2 * porder;
  }
  if (!c.is_bc && vm->kind == ORC_MOCK) {
    // TPZMatTest (UnitTest_PZ/TestStruct/StructMatrixUnitTest.cpp:333-362): fixed ek
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) ek[j * n + i] = vm->mock_ek[i * 2 + j];
    return n;
  }
  IntRule rule = make_rule(t, intorder);
  std::vector<double> phi(nshape), dphi(3 * nshape), dx(3 * nshape);
  double coefE = vm->kind == ORC_ELAST3D ? vm->E : vm->coef_const;
  if (!c.is_bc && !m.coef.empty() && c.gel < m.nvol) coefE = m.coef[c.gel];
  for (size_t ip = 0; ip < rule.wts.size(); ip++) {
    const double *pt = &rule.pts[ip * rule.dim];
    double weight = rule.wts[ip];
    Jac J = jacobian(t, coords, pt);
    shape_h1(t, g.nodes, orders, pt, phi.data(), dphi.data(), nshape);
    for (int i = 0; i < D; i++)
      for (int k = 0; k < nshape; k++) {
        double acc = 0.0;
        for (int j = 0; j < D; j++) acc += J.jinv[j][i] * dphi[j * nshape + k];
        dx[i * nshape + k] = acc;
      }
    weight *= std::fabs(J.detjac);
    if (!c.is_bc) {
      double f[3];
      forcing_value(*vm, J.x, f);
      contribute(vm->kind, vm->dim, vm->scale, coefE, vm->nu, weight, nshape, phi.data(), dx.data(), nshape, f, ek, ef, n);
    } else {
      const orc_bc &bc = m.spec.bcs[c.mat];
      double big = vm->kind == ORC_ELAST3D ? 1.e12 : vm->bignumber;  // TPZElasticity3D.cpp:632
      if (vm->kind == ORC_ELAST3D) {  // TPZElasticity3D::ContributeBC (Material/Elasticity/TPZElasticity3D.cpp:616-700)
        for (int in = 0; in < nshape; in++) {
          if (bc.type == 0) {
            for (int kd = 0; kd < 3; kd++) ef[3 * in + kd] += big * bc.val2[kd] * phi[in] * weight;
            for (int jn = 0; jn < nshape; jn++)
              for (int kd = 0; kd < 3; kd++) ek[(size_t)(3 * jn + kd) * n + 3 * in + kd] += big * phi[in] * phi[jn] * weight;
          } else if (bc.type == 1) {
            for (int kd = 0; kd < 3; kd++) ef[3 * in + kd] += bc.val2[kd] * phi[in] * weight;
          }
        }
      } else if (vm->kind == ORC_POISSON) {  // TPZMatPoisson::ContributeBC (Material/Poisson/TPZMatPoisson.cpp:46-125)
        for (int in = 0; in < nshape; in++) {
          if (bc.type == 0) {
            ef[in] += big * bc.val2[0] * phi[in] * weight;
            for (int jn = 0; jn < nshape; jn++) ek[(size_t)jn * n + in] += big * phi[in] * phi[jn] * weight;
          } else if (bc.type == 1) {
            ef[in] += bc.val2[0] * vm->scale * phi[in] * weight;
          }
        }
      } else if (vm->kind == ORC_DARCY) {  // TPZDarcyFlow::ContributeBC (Material/DarcyFlow/TPZDarcyFlow.cpp:49-96)
        for (int in = 0; in < nshape; in++) {
          if (bc.type == 0) {
            ef[in] += (big * phi[in] * weight) * bc.val2[0];
            for (int jn = 0; jn < nshape; jn++) ek[(size_t)jn * n + in] += big * phi[in] * phi[jn] * weight;
          } else if (bc.type == 1) {
            ef[in] += bc.val2[0] * (phi[in] * weight);
          }
        }
      }
    }
  }
  return n;
}

// ---------------------------------------------------------------------------
// Exact-solution error norms: TPZCompMesh::EvaluateError (Mesh/pzcmesh.cpp:1497-1551)
// over the elements in element order, TPZInterpolationSpace::EvaluateError
// (Mesh/pzinterpolationspace.cpp:1108-1200) per element and the materials'
// Errors() at each point.  The exact solution is data here: the points of every
// element's error rule are listed first (error_points), the caller evaluates
// its exact solution u[s] and gradient du[d][s] (direction d, state s, the
// TPZFMatrix dsol layout) at them, and error_eval integrates.
// ---------------------------------------------------------------------------
// Error rule order: the element rule's order raised to the exact solution's
// polynomial order, unless that exceeds the rule's maximum
// (Mesh/pzinterpolationspace.cpp:1140-1156).  GetMaxOrder is 36 for
// TPZIntQuad and 20 for TPZIntCube3D (Integral/pzquad.h:217,299);
// TPZIntQuad::GetOrder returns the requested order, TPZIntCube3D::GetOrder
// the rule's own, 2 (npoints - 1) (Integral/pzquad.cpp:176-194,289-305,
// Integral/tpzgaussrule.cpp:170-181).
static int error_order(int t, int intorder, int exact_order) {
  int maxo = t == T_CUBE ? 20 : 36;
  int prev = t == T_CUBE ? 2 * (gauss_npoints(intorder) - 1) : intorder;
  if (maxo > exact_order) return prev > exact_order ? prev : exact_order;
  return maxo;
}

static int element_intorder(const Mesh &m, const CompEl &c) {
  int porder = max_order(m, c);
  const orc_material &vm = m.spec.mats[c.mat];
  if (vm.kind == ORC_ELAST3D) return 2 * porder;
  if (porder < vm.forcing_porder) return vm.forcing_porder + porder;
  return 2 * porder;
}

static int nerrors_of(int kind) { return kind == ORC_DARCY ? 6 : 3; }

// Errors() at one point: TPZMatPoisson (Material/Poisson/TPZMatPoisson.cpp:173-218),
// TPZDarcyFlow (Material/DarcyFlow/TPZDarcyFlow.cpp:268-327), TPZElasticity3D
// (Material/Elasticity/TPZElasticity3D.cpp:1081-1133 with ComputeStressVector,
// :1178-1192, and ComputeStressTensor, :1152-1166; no prestress).  gradu and due
// are [3][ns] in xyz; coef is the element's permeability or Young modulus.
static void material_errors(const orc_material &mat, double coef, int ns, const double *u, const double *gradu,
                            const double *ue, const double *due, double *v) {
  for (int k = 0; k < 6; k++) v[k] = 0.0;
  if (mat.kind == ORC_POISSON) {
    double diff = u[0] - ue[0];
    v[1] = diff * diff;
    v[2] = 0.0;
    for (int id = 0; id < mat.dim; id++) {
      diff = gradu[id] - due[id];
      v[2] += diff * diff;
    }
    v[0] = v[1] + v[2];
  } else if (mat.kind == ORC_DARCY) {
    double diff = std::fabs(u[0] - ue[0]);
    v[1] = diff * diff;
    double gd[3] = {0.0, 0.0, 0.0};
    for (int id = 0; id < mat.dim; id++) gd[id] += std::fabs(gradu[id] - due[id]);
    diff = 0.0;
    for (int id = 0; id < mat.dim; id++) diff += coef * gd[id];
    v[2] += std::fabs(diff * diff);
    v[0] = v[1] + v[2];
    for (int id = 0; id < mat.dim; id++) {
      double flux = -coef * gradu[id];
      diff = std::fabs(due[id] - flux);
      v[3 + id] = diff * diff;
    }
  } else if (mat.kind == ORC_ELAST3D) {
    double L2 = 0.0;
    for (int i = 0; i < 3; i++) L2 += (u[i] - ue[i]) * (u[i] - ue[i]);
    double semi = 0.0, D[3][3];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        D[i][j] = gradu[i * ns + j] - due[i * ns + j];
        semi += D[i][j] * D[i][j];
      }
    const double E = coef, ni = mat.nu;
    const double const1 = -1. + ni, const2 = -1. + ni + 2. * ni * ni, const3 = 2. * (1. + ni);
    double sv[6];
    sv[0] = E * (D[0][0] * const1 - (D[1][1] + D[2][2]) * ni) / const2;
    sv[1] = E * (D[1][1] * const1 - (D[0][0] + D[2][2]) * ni) / const2;
    sv[2] = E * (D[2][2] * const1 - (D[0][0] + D[1][1]) * ni) / const2;
    sv[3] = E * (D[1][0] + D[0][1]) / const3;
    sv[4] = E * (D[2][0] + D[0][2]) / const3;
    sv[5] = E * (D[2][1] + D[1][2]) / const3;
    const double S[3][3] = {{sv[0], sv[3], sv[4]}, {sv[3], sv[1], sv[5]}, {sv[4], sv[5], sv[2]}};
    double energy = 0.0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) energy += D[i][j] * S[i][j];
    v[1] = L2;
    v[2] = semi;
    v[0] = energy;
  }
}

static bool has_error(const Mesh &m, const CompEl &c) { return !c.is_bc && tdim(c.type) == m.spec.dim; }

// Physical coordinates (TPZGeoEl::X) of every error-rule point, element after element.
static int64_t error_points(const Mesh &m, int exact_order, double *xyz) {
  int64_t np = 0;
  for (const CompEl &c : m.cels) {
    if (!has_error(m, c)) continue;
    const GeoEl &g = m.gels[c.gel];
    double coords[8 * 3];
    for (int k = 0; k < ncorner(c.type); k++)
      for (int j = 0; j < 3; j++) coords[k * 3 + j] = m.nodes[g.nodes[k] * 3 + j];
    IntRule rule = make_rule(c.type, error_order(c.type, element_intorder(m, c), exact_order));
    for (size_t ip = 0; ip < rule.wts.size(); ip++, np++) {
      if (!xyz) continue;
      Jac J = jacobian(c.type, coords, &rule.pts[ip * rule.dim]);
      for (int j = 0; j < 3; j++) xyz[np * 3 + j] = J.x[j];
    }
  }
  return np;
}

// Per-element errors (sqrt of the integrated values, as EvaluateError leaves
// them; zero rows for boundary elements) and the mesh totals sqrt(sum_e err_e^2).
static int error_eval(const Mesh &m, int exact_order, const double *sol, const double *uex, const double *duex,
                      double *errors, double *el) {
  const int ns = m.nstate;
  int nerr = 0;
  for (int i = 0; i < m.spec.nmat; i++) nerr = std::max(nerr, nerrors_of(m.spec.mats[i].kind));
  std::vector<double> tot(nerr, 0.0);
  int64_t np = 0;
  for (size_t ic = 0; ic < m.cels.size(); ic++) {
    const CompEl &c = m.cels[ic];
    double ee[6] = {0, 0, 0, 0, 0, 0};
    if (has_error(m, c)) {
      const GeoEl &g = m.gels[c.gel];
      const orc_material &vm = m.spec.mats[c.mat];
      int t = c.type, NC = ncorner(t), D = tdim(t);
      int orders[26];
      side_orders_of(m, c, orders);
      int nshape = NC;
      for (int s = NC; s < nsides(t); s++) nshape += nconnect_shape(t, s, orders[s - NC]);
      std::vector<int64_t> dest(nshape * ns);
      element_dest(m, c, dest.data());
      double coords[8 * 3];
      for (int k = 0; k < NC; k++)
        for (int j = 0; j < 3; j++) coords[k * 3 + j] = m.nodes[g.nodes[k] * 3 + j];
      double coef = vm.kind == ORC_ELAST3D ? vm.E : vm.coef_const;
      if (!m.coef.empty() && c.gel < m.nvol) coef = m.coef[c.gel];
      IntRule rule = make_rule(t, error_order(t, element_intorder(m, c), exact_order));
      std::vector<double> phi(nshape), dphi(3 * nshape), dx(3 * nshape);
      for (size_t ip = 0; ip < rule.wts.size(); ip++, np++) {
        const double *pt = &rule.pts[ip * rule.dim];
        double weight = rule.wts[ip];
        Jac J = jacobian(t, coords, pt);
        shape_h1(t, g.nodes, orders, pt, phi.data(), dphi.data(), nshape);
        for (int i = 0; i < D; i++)
          for (int k = 0; k < nshape; k++) {
            double acc = 0.0;
            for (int j = 0; j < D; j++) acc += J.jinv[j][i] * dphi[j * nshape + k];
            dx[i * nshape + k] = acc;
          }
        // TPZInterpolationSpace::ReallyComputeSolutionT (Mesh/pzinterpolationspace.cpp:135-178)
        double u[3] = {0, 0, 0}, dsol[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int iv = 0; iv < nshape * ns; iv++) {
          const double xv = sol[dest[iv]];
          u[iv % ns] += phi[iv / ns] * xv;
          for (int d = 0; d < D; d++) dsol[d][iv % ns] += dx[d * nshape + iv / ns] * xv;
        }
        // TPZAxesTools::Axes2XYZ (Util/pzaxestools.h:61-86) with the axes of
        // TPZGeoEl::Jacobian (Mesh/pzgeoel.cpp:1228-1292; the identity in 3D)
        double axes[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        if (D == 2) {
          double cp[27], cd[3 * 27], v1[3] = {0, 0, 0}, v2[3] = {0, 0, 0};
          corner_shapes(t, pt, cp, cd);
          for (int k = 0; k < NC; k++)
            for (int i = 0; i < 3; i++) {
              v1[i] += coords[k * 3 + i] * cd[0 * 27 + k];
              v2[i] += coords[k * 3 + i] * cd[1 * 27 + k];
            }
          double n1 = 0.0, d12 = 0.0, n2 = 0.0, v1t[3], v2t[3];
          for (int i = 0; i < 3; i++) { n1 += v1[i] * v1[i]; d12 += v1[i] * v2[i]; }
          n1 = std::sqrt(n1);
          for (int i = 0; i < 3; i++) {
            v1t[i] = v1[i] / n1;
            v2t[i] = v2[i] - d12 * v1t[i] / n1;
            n2 += v2t[i] * v2t[i];
          }
          n2 = std::sqrt(n2);
          for (int i = 0; i < 3; i++) {
            axes[0][i] = v1t[i];
            axes[1][i] = v2t[i] / n2;
          }
        }
        double gradu[3 * 3] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int i = 0; i < 3; i++)
          for (int s2 = 0; s2 < ns; s2++) {
            double acc = 0.0;
            for (int d = 0; d < D; d++) acc += axes[d][i] * dsol[d][s2];
            gradu[i * ns + s2] = acc;
          }
        double v[6];
        material_errors(vm, coef, ns, u, gradu, &uex[np * ns], &duex[np * 3 * ns], v);
        weight *= std::fabs(J.detjac);
        for (int k = 0; k < nerr; k++) ee[k] += weight * v[k];
      }
      for (int k = 0; k < nerr; k++) ee[k] = std::sqrt(ee[k]);
    }
    for (int k = 0; k < nerr; k++) {
      if (el) el[ic * nerr + k] = ee[k];
      tot[k] += ee[k] * ee[k];
    }
  }
  for (int k = 0; k < nerr; k++) errors[k] = std::sqrt(tot[k]);
  return nerr;
}

// ---------------------------------------------------------------------------
// CSR pattern: TPZCompMesh::ComputeElGraph (Mesh/pzcmesh.cpp:1214-1262),
// TPZRenumbering::ConvertGraph (External/TPZRenumbering.cpp:76-105),
// TPZSSpStructMatrix::SetupMatrixData (StrMatrix/TPZSSpStructMatrix.cpp:50-193, upper)
// and TPZSpStructMatrix::SetupMatrixData (StrMatrix/TPZSpStructMatrix.cpp:53-190, full).
// ---------------------------------------------------------------------------
static void node_graph(const Mesh &m, std::vector<int64_t> &ng, std::vector<int64_t> &ngi) {
  int64_t nn = (int64_t)m.conn_order.size();
  std::vector<std::vector<int64_t>> n2e(nn);
  for (int64_t e = 0; e < (int64_t)m.cels.size(); e++) {
    const CompEl &c = m.cels[e];
    for (int s = 0; s < nsides(c.type); s++) n2e[c.conn[s]].push_back(e);
  }
  ngi.assign(nn + 1, 0);
  ng.clear();
  for (int64_t nod = 0; nod < nn; nod++) {
    std::set<int64_t> con;
    for (int64_t e : n2e[nod]) {
      const CompEl &c = m.cels[e];
      for (int s = 0; s < nsides(c.type); s++) con.insert(c.conn[s]);
    }
    con.erase(nod);
    for (int64_t v : con) ng.push_back(v);
    ngi[nod + 1] = (int64_t)ng.size();
  }
}

static void setup_pattern(const Mesh &m, int sym, std::vector<int64_t> &IA, std::vector<int64_t> &JA) {
  std::vector<int64_t> ng, ngi;
  node_graph(m, ng, ngi);
  int64_t nb = (int64_t)m.conn_order.size();
  IA.assign(m.neq + 1, 0);
  JA.clear();
  int64_t ieq = 0;
  for (int64_t i = 0; i < nb; i++) {
    int64_t isz = m.block_size[i], ipos = m.block_pos[i];
    if (isz == 0) continue;
    for (int64_t k = 0; k < isz; k++, ieq++) {
      IA[ieq] = (int64_t)JA.size();
      auto add = [&](int64_t col) {
        int64_t csz = m.block_size[col], cpos = m.block_pos[col];
        for (int64_t jj = 0; jj < csz; jj++) {
          if (sym && cpos + jj < ieq) continue;
          JA.push_back(cpos + jj);
        }
      };
      if (sym) {
        bool diag = false;
        for (int64_t j = ngi[i]; j < ngi[i + 1]; j++) {
          int64_t col = ng[j];
          if (col < i) continue;
          if (!diag && col > i) { diag = true; add(i); }
          if (m.block_size[col] == 0) continue;
          add(col);
        }
        if (!diag) add(i);
      } else {
        size_t first = JA.size();
        add(i);
        for (int64_t j = ngi[i]; j < ngi[i + 1]; j++) {
          int64_t col = ng[j];
          if (m.block_size[col] == 0) continue;
          add(col);
        }
        std::stable_sort(JA.begin() + first, JA.end());
      }
    }
    (void)ipos;
  }
  IA[ieq] = (int64_t)JA.size();
}

// TPZSYsmpMatrix::AddKel (Matrix/pzsysmp.cpp:369-411) and TPZFYsmpMatrix::AddKel
// (Matrix/pzysmp.cpp:177-218): skip |value| < 1e-12 (IsZero, Common/pzreal.h:736-742),
// "next slot" fast path else linear search of the row.
static void add_kel(int sym, const int64_t *IA, const int64_t *JA, double *A, const double *ek, int n, const int64_t *dest) {
  int64_t k = 0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      int64_t ipos = dest[i], jpos = dest[j];
      if (sym && jpos < ipos) continue;
      double value = ek[(size_t)j * n + i];
      if (std::fabs(value) < 1.e-12) continue;
      k++;
      if (k >= IA[ipos] && k < IA[ipos + 1] && JA[k] == jpos) {
        A[k] += value;
      } else {
        for (k = IA[ipos]; k < IA[ipos + 1]; k++)
          if (JA[k] == jpos) { A[k] += value; break; }
      }
    }
}

}  // namespace orc

// ============================================================================
// extern "C" API used by the tests and by the CPU-baseline leg of the benchmark.
// ============================================================================
using namespace orc;

extern "C" {

void *orc_mesh_create(const orc_grid_spec *spec) {
  Mesh *m = new Mesh();
  m->spec = *spec;
  if (spec->dim == 1) grid1d(*m);
  else if (spec->dim == 2) grid2d(*m);
  else grid3d(*m);
  if (spec->elem_coef) m->coef.assign(spec->elem_coef, spec->elem_coef + m->nvol);
  if (spec->elem_order) m->elorder.assign(spec->elem_order, spec->elem_order + m->nvol);
  m->spec.elem_coef = nullptr;
  m->spec.elem_order = nullptr;
  build_comp(*m);
  init_blocks(*m);
  return m;
}

void orc_mesh_free(void *h) { delete (Mesh *)h; }

int64_t orc_neq(void *h) { return ((Mesh *)h)->neq; }
int64_t orc_ncel(void *h) { return (int64_t)((Mesh *)h)->cels.size(); }
int64_t orc_nconnects(void *h) { return (int64_t)((Mesh *)h)->conn_order.size(); }
int64_t orc_nnodes(void *h) { return (int64_t)((Mesh *)h)->nodes.size() / 3; }
int orc_nstate(void *h) { return ((Mesh *)h)->nstate; }

// Element info: type, is_bc, number of local equations, destination indices,
// connect (sequence number) list, geometric element index.
int orc_cel_info(void *h, int64_t ic, int *type, int *is_bc, int64_t *gel, int64_t *conn, int64_t *dest) {
  Mesh *m = (Mesh *)h;
  const CompEl &c = m->cels[ic];
  *type = c.type;
  *is_bc = c.is_bc;
  *gel = c.gel;
  if (conn)
    for (int s = 0; s < nsides(c.type); s++) conn[s] = c.conn[s];
  int64_t tmp[27 * 64 * 3];
  int n = element_dest(*m, c, dest ? dest : tmp);
  return n;
}

void orc_block_info(void *h, int64_t *pos, int64_t *size) {
  Mesh *m = (Mesh *)h;
  for (size_t i = 0; i < m->block_size.size(); i++) { pos[i] = m->block_pos[i]; size[i] = m->block_size[i]; }
}

void orc_nodes(void *h, double *xyz) {
  Mesh *m = (Mesh *)h;
  std::copy(m->nodes.begin(), m->nodes.end(), xyz);
}

// Move the mesh nodes (the same numbering): a distorted, non-affine mesh
// for the tests, as a user program editing TPZGeoNode coordinates would.
void orc_set_nodes(void *h, const double *xyz) {
  Mesh *m = (Mesh *)h;
  std::copy(xyz, xyz + m->nodes.size(), m->nodes.begin());
}

int orc_calc_stiff(void *h, int64_t ic, double *ek, double *ef) {
  Mesh *m = (Mesh *)h;
  return calc_stiff(*m, m->cels[ic], ek, ef);
}

// Error norms against an exact solution given at the error-rule points
// (TPZAnalysis::PostProcessError, Analysis/TPZAnalysis.cpp:625-650):
// orc_error_points returns the number of points and, with xyz, their
// coordinates; orc_error_eval returns the number of norms.
int64_t orc_error_points(void *h, int exact_order, double *xyz) { return error_points(*(Mesh *)h, exact_order, xyz); }

int orc_error_eval(void *h, int exact_order, const double *sol, const double *uex, const double *duex, double *errors,
                   double *el) {
  return error_eval(*(Mesh *)h, exact_order, sol, uex, duex, errors, el);
}

// H1 shape functions of one element type at one point (for the shape-table tests).
int orc_shape(int type, const int64_t *ids, const int *orders, const double *pt, double *phi, double *dphi, int ldd) {
  return shape_h1(type, ids, orders, pt, phi, dphi, ldd);
}

// One Contribute call (the material unit tests): ek column-major n x n, n = nshape * nstate.
void orc_contribute(int kind, int dim, double scale, double coef, double nu, double weight, int nshape, const double *phi,
                    const double *dphix, const double *force, double *ek, double *ef) {
  int n = kind == ORC_ELAST3D ? 3 * nshape : nshape;
  double f[3] = {force[0], force[1], force[2]};
  contribute(kind, dim, scale, coef, nu, weight, nshape, phi, dphix, nshape, f, ek, ef, n);
}

int orc_gauss(int order, double *loc, double *w) {
  std::vector<double> l, ww;
  int n = gauss_npoints(order);
  gauss_legendre(n, l, ww);
  for (int i = 0; i < n; i++) { loc[i] = l[i]; w[i] = ww[i]; }
  return n;
}

// Pattern: returns nnz; fills IA (neq+1) and JA (nnz) when both non-null.
int64_t orc_pattern(void *h, int sym, int64_t *IA, int64_t *JA) {
  Mesh *m = (Mesh *)h;
  std::vector<int64_t> ia, ja;
  setup_pattern(*m, sym, ia, ja);
  if (IA && JA) {
    std::copy(ia.begin(), ia.end(), IA);
    std::copy(ja.begin(), ja.end(), JA);
  }
  return (int64_t)ja.size();
}

// Serial or threaded (TPZStructMatrixOR) assembly into a given CSR.
// StrMatrix/pzstrmatrixor.cpp:106-365 (serial) and :478-513,587-845 (threads
// compute CalcStiff, the calling thread scatters in strict element order).
int orc_assemble(void *h, int sym, const int64_t *IA, const int64_t *JA, double *A, double *F, int nthreads) {
  Mesh *m = (Mesh *)h;
  int64_t nnz = IA[m->neq];
  std::fill(A, A + nnz, 0.0);
  std::fill(F, F + m->neq, 0.0);
  int64_t ncel = (int64_t)m->cels.size();
  const int MAXN = 64 * 3;
  if (nthreads <= 1) {
    std::vector<double> ek((size_t)MAXN * MAXN), ef(MAXN);
    std::vector<int64_t> dest(MAXN);
    for (int64_t e = 0; e < ncel; e++) {
      int n = calc_stiff(*m, m->cels[e], ek.data(), ef.data());
      element_dest(*m, m->cels[e], dest.data());
      add_kel(sym, IA, JA, A, ek.data(), n, dest.data());
      for (int i = 0; i < n; i++) F[dest[i]] += ef[i];  // TPZFMatrix::AddFel (Matrix/pzfmatrix.cpp:268-320)
    }
    return 0;
  }
  // producer/consumer: a ring of element-matrix slots filled by workers,
  // consumed (scattered) in element order by this thread.
  const int NSLOT = 4 * nthreads;
  struct Slot {
    std::vector<double> ek, ef;
    int n = 0;
    std::atomic<int64_t> tag{-1};  // element index whose matrices the slot holds
  };
  std::vector<Slot> slots(NSLOT);
  for (auto &s : slots) { s.ek.resize((size_t)MAXN * MAXN); s.ef.resize(MAXN); }
  std::atomic<int64_t> next{0};
  std::atomic<int64_t> consumed{0};
  auto worker = [&]() {
    for (;;) {
      int64_t e = next.fetch_add(1);
      if (e >= ncel) return;
      Slot &s = slots[e % NSLOT];
      while (e - consumed.load(std::memory_order_acquire) >= NSLOT) std::this_thread::yield();
      s.n = calc_stiff(*m, m->cels[e], s.ek.data(), s.ef.data());
      s.tag.store(e, std::memory_order_release);
    }
  };
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; t++) th.emplace_back(worker);
  std::vector<int64_t> dest(MAXN);
  for (int64_t e = 0; e < ncel; e++) {
    Slot &s = slots[e % NSLOT];
    while (s.tag.load(std::memory_order_acquire) != e) std::this_thread::yield();
    element_dest(*m, m->cels[e], dest.data());
    add_kel(sym, IA, JA, A, s.ek.data(), s.n, dest.data());
    for (int i = 0; i < s.n; i++) F[dest[i]] += s.ef[i];
    consumed.store(e + 1, std::memory_order_release);
  }
  for (auto &t : th) t.join();
  return 0;
}

// TPZSYsmpMatrix::MultAdd (Matrix/pzsysmp.cpp:189-232; symmetric, upper stored)
// and TPZFYsmpMatrix::MultAdd (Matrix/pzysmp.cpp:527-624; full).  z = A x.
void orc_spmv(int64_t n, int sym, const int64_t *IA, const int64_t *JA, const double *A, const double *x, double *z) {
  for (int64_t i = 0; i < n; i++) z[i] = 0.0;
  for (int64_t row = 0; row < n; row++)
    for (int64_t iv = IA[row]; iv < IA[row + 1]; iv++) {
      int64_t ic = JA[iv];
      z[row] += A[iv] * x[ic];
      if (sym && row != ic) z[ic] += A[iv] * x[row];
    }
}

static double dot(int64_t n, const double *a, const double *b) {
  double s = 0.0;
  for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

// CG with the Jacobi TPZStepSolver as preconditioner: Solvers/LinearSolvers/cg.h:29-132
// and TPZMatrix::SolveJacobi (Matrix/pzmatrix.cpp:643-667, one sweep from zero,
// z = r / diag; the extra Residual() SpMV it performs is reproduced when
// jacobi_residual != 0 so that the CPU timing matches the reference's cost).
int orc_cg_jacobi(int64_t n, int sym, const int64_t *IA, const int64_t *JA, const double *A, const double *b, double *x,
                  int64_t maxit, double tol, int jacobi_residual, int64_t *iters_out, double *resid_out, double *hist) {
  std::vector<double> diag(n), r(n), z(n), p(n), q(n), scratch(n);
  for (int64_t i = 0; i < n; i++) {
    double d = 0.0;
    for (int64_t k = IA[i]; k < IA[i + 1]; k++)
      if (JA[k] == i) { d = A[k]; break; }
    diag[i] = d;
  }
  double normb = std::sqrt(dot(n, b, b));
  for (int64_t i = 0; i < n; i++) { x[i] = 0.0; r[i] = b[i]; }
  if (normb == 0.0) normb = 1.0;
  double resid = std::sqrt(dot(n, r.data(), r.data())) / normb;
  if (resid <= tol) { *iters_out = 0; *resid_out = resid; return 0; }
  double rho = 0, rho_1 = 0;
  for (int64_t it = 1; it <= maxit; it++) {
    for (int64_t i = 0; i < n; i++) z[i] = r[i] / diag[i];
    if (jacobi_residual) orc_spmv(n, sym, IA, JA, A, z.data(), scratch.data());
    rho = dot(n, r.data(), z.data());
    if (it == 1) p = z;
    else {
      double beta = rho / rho_1;
      for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];  // TimesBetaPlusZ
    }
    orc_spmv(n, sym, IA, JA, A, p.data(), q.data());
    double alpha = rho / dot(n, p.data(), q.data());
    for (int64_t i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
    resid = std::sqrt(dot(n, r.data(), r.data())) / normb;
    if (hist) hist[it - 1] = resid;
    if (resid <= tol) { *iters_out = it; *resid_out = resid; return 0; }
    rho_1 = rho;
  }
  *iters_out = maxit;
  *resid_out = resid;
  return 1;
}

// Stationary Jacobi iteration, TPZStepSolver::SetJacobi as the solver
// (Solvers/pzstepsolver.cpp:94-98).  sym != 0: TPZSYsmpMatrix inherits
// TPZMatrix::SolveJacobi (Matrix/pzmatrix.cpp:643-667): r = b - A x (from
// current) or r = b, x = 0; while it < maxit and ||r|| > tol: x += r / a_ii,
// r = b - A x.  sym == 0: the TPZFYsmpMatrix override (Matrix/pzysmp.cpp:
// 725-781) always makes the first sweep (x = b / a_ii from zero) and then
// continues as above for at most maxit sweeps in all.  The tolerance is on
// the absolute residual norm.  iters_out receives the sweeps performed (the
// reference leaves numiterations at its input value), resid_out the final
// ||b - A x||.
int orc_jacobi(int64_t n, int sym, const int64_t *IA, const int64_t *JA, const double *A, const double *b, double *x,
               int64_t maxit, double tol, int from_current, int64_t *iters_out, double *resid_out) {
  std::vector<double> diag(n), r(n), ax(n);
  for (int64_t i = 0; i < n; i++) {
    double d = 0.0;
    for (int64_t k = IA[i]; k < IA[i + 1]; k++)
      if (JA[k] == i) { d = A[k]; break; }
    diag[i] = d;
  }
  auto residual = [&]() {
    orc_spmv(n, sym, IA, JA, A, x, ax.data());
    for (int64_t i = 0; i < n; i++) r[i] = b[i] - ax[i];
    return std::sqrt(dot(n, r.data(), r.data()));
  };
  int64_t it = 0;
  double res;
  if (from_current) {
    res = residual();
  } else {
    for (int64_t i = 0; i < n; i++) { x[i] = 0.0; r[i] = b[i]; }
    res = std::sqrt(dot(n, r.data(), r.data()));
  }
  if (!sym) {
    for (int64_t i = 0; i < n; i++) x[i] += r[i] / diag[i];
    it = 1;
    res = residual();
  }
  for (; it < maxit && res > tol; it++) {
    for (int64_t i = 0; i < n; i++) x[i] += r[i] / diag[i];
    res = residual();
  }
  *iters_out = it;
  *resid_out = res;
  return res <= tol ? 0 : 1;
}

// Sloan renumbering as the reference runs it: TPZSloanRenumbering::Resequence
// (External/TPZSloanRenumbering.cpp:23-175) over the node graph of
// TPZRenumbering::ConvertGraph (External/TPZRenumbering.cpp:76-105), with the
// pseudo-peripheral pair of TPZCutHillMcKee::SGraph (External/TPZCutHillMcKee.cpp:
// 16-30, 93-119, 121-260), the SList queue (External/TPZSloanRenumbering.h:20-86:
// append once ever, remove by moving the last entry into the hole) and
// FindHighestPriority's scan for the first entry of largest priority
// (TPZSloanRenumbering.cpp:177-192).  Weights W1 = 1, W2 = 2.  Returns 0, or 1
// when not every node is reached (the reference stops there).
int orc_sloan(int64_t nnodes, int64_t nel, const int64_t *eptr, const int64_t *eg, int64_t *perm_gather,
              int64_t *perm_scatter) {
  // node graph: std::set of the element lists through each node, self erased
  std::vector<std::vector<int64_t>> n2e(nnodes);
  for (int64_t e = 0; e < nel; e++)
    for (int64_t k = eptr[e]; k < eptr[e + 1]; k++) n2e[eg[k]].push_back(e);
  std::vector<int64_t> gptr(nnodes + 1, 0), gadj;
  for (int64_t v = 0; v < nnodes; v++) {
    std::set<int64_t> con;
    for (int64_t e : n2e[v]) con.insert(eg + eptr[e], eg + eptr[e + 1]);
    con.erase(v);
    gadj.insert(gadj.end(), con.begin(), con.end());
    gptr[v + 1] = (int64_t)gadj.size();
  }
  auto degree = [&](int64_t v) { return gptr[v + 1] - gptr[v]; };
  // RootedLevelStructure: each level from GetAdjacentNodes(previous level, processed)
  auto levels = [&](int64_t root) {
    std::vector<std::vector<int64_t>> L;
    std::vector<int64_t> processed(nnodes, 0), level{root};
    for (int64_t il = 0; il < nnodes && !level.empty(); il++) {
      for (int64_t v : level) processed[v] = 1;
      L.push_back(level);
      std::vector<int64_t> next, history(nnodes, 0);
      for (int64_t p : L.back())
        for (int64_t k = gptr[p]; k < gptr[p + 1]; k++) {
          const int64_t v = gadj[k];
          if (processed[v] == 0 && history[v] == 0) {
            next.push_back(v);
            history[v] = 1;
          }
        }
      level = next;
    }
    return L;
  };
  // PseudoPeripheralNodes
  int64_t mindeg = 1000000, start = -1, end = -1;
  for (int64_t v = 0; v < nnodes; v++)
    if (degree(v) < mindeg) {
      mindeg = degree(v);
      start = v;
    }
  if (start < 0) return 1;
  std::vector<std::vector<int64_t>> LS = levels(start);
  int64_t count = 0;
  while (count < 10 || end == -1) {
    count++;
    const int64_t cps = start, cpe = end;
    const int64_t nlev = (int64_t)LS.size();
    if (!nlev) break;
    std::vector<int64_t> last = LS[nlev - 1];
    const int64_t nelsOrig = (int64_t)last.size();
    std::multimap<int64_t, int64_t> bydeg;  // SortNodes
    for (int64_t v : last) bydeg.insert(std::make_pair(degree(v), v));
    last.clear();
    for (auto &kv : bydeg) last.push_back(kv.second);
    std::map<int64_t, int64_t> shrink;  // ShrinkLastLevel
    for (int64_t v : last) shrink[degree(v)] = v;
    last.clear();
    for (auto &kv : shrink) last.push_back(kv.second);
    const int64_t newsize = (nelsOrig + 2) / 2;
    if (newsize < (int64_t)last.size()) last.resize(newsize);
    int64_t we = 1000000000L, hs = nlev;
    for (int64_t q : last) {
      std::vector<std::vector<int64_t>> loc = levels(q);
      const int64_t h = (int64_t)loc.size();
      int64_t w = 0;
      for (auto &l : loc) w = std::max<int64_t>(w, (int64_t)l.size());
      if (h > hs && w < we) {
        start = q;
        LS = loc;
        break;
      } else if (w < we) {
        end = q;
        we = w;
      }
    }
    if (cps == start && cpe == end) break;
  }
  if (start < 0 || end < 0) return 1;
  std::vector<int64_t> dist(nnodes, -1);
  std::vector<std::vector<int64_t>> LE = levels(end);
  for (int64_t l = 0; l < (int64_t)LE.size(); l++)
    for (int64_t v : LE[l]) dist[v] = l;
  for (int64_t v = 0; v < nnodes; v++)
    if (dist[v] < 0) return 1;
  const int64_t W1 = 1, W2 = 2;
  std::vector<int64_t> priority(nnodes);
  for (int64_t i = 0; i < nnodes; i++) priority[i] = W1 * dist[i] - W2 * (degree(i) + 1);
  enum { EInactive = 0, EPreActive = 1, EActive = 2, EPostActive = 3 };
  std::vector<int> status(nnodes, EInactive);
  std::vector<int64_t> qlist(nnodes), hist(nnodes, 0);
  int64_t qsize = 0, nr = 0;
  auto push_back = [&](int64_t v) {
    if (hist[v]) return false;
    hist[v] = 1;
    qlist[qsize++] = v;
    return true;
  };
  status[start] = EPreActive;
  push_back(start);
  while (qsize) {
    int64_t index = 0, cur = qlist[0], np = priority[cur];
    for (int64_t i = 1; i < qsize; i++)
      if (priority[qlist[i]] > np) {
        cur = qlist[i];
        np = priority[cur];
        index = i;
      }
    qlist[index] = qlist[qsize - 1];
    qsize--;
    if (status[cur] == EPreActive) {
      for (int64_t k = gptr[cur]; k < gptr[cur + 1]; k++) {
        const int64_t a = gadj[k];
        priority[a] += W2;
        if (push_back(a) == true && status[a] == EInactive) status[a] = EPreActive;
      }
    }
    perm_scatter[nr++] = cur;
    status[cur] = EPostActive;
    for (int64_t k = gptr[cur]; k < gptr[cur + 1]; k++) {
      const int64_t a = gadj[k];
      if (status[a] != EPreActive) continue;
      status[a] = EActive;
      priority[a] += W2;
      for (int64_t j = gptr[a]; j < gptr[a + 1]; j++) {
        const int64_t q = gadj[j];
        if (status[q] != EPostActive) {
          const int pr = (int)priority[q];
          priority[q] = pr + W2;
        }
        if (push_back(q) == true && status[q] == EInactive) status[q] = EPreActive;
      }
    }
  }
  if (nr != nnodes) return 1;
  for (int64_t i = 0; i < nnodes; i++) perm_gather[perm_scatter[i]] = i;
  return 0;
}

// CG with a block-Jacobi preconditioner over consecutive equation blocks of
// size bs (TPZBlockDiagonal, Matrix/pzblockdiag.h:21, built over the mesh's
// connect blocks as TPZAnalysis::BuildPreconditioner(EBlockJacobi) does for
// one-shape connects, Analysis/TPZAnalysis.cpp:995-1090); blocks inverted by
// Gaussian elimination with partial pivoting.
int orc_cg_block_jacobi(int64_t n, int sym, const int64_t *IA, const int64_t *JA, const double *A, const double *b,
                        double *x, int bs, int64_t maxit, double tol, int64_t *iters_out, double *resid_out) {
  int64_t nb = n / bs;
  std::vector<double> inv((size_t)nb * bs * bs, 0.0);
  for (int64_t B = 0; B < nb; B++) {
    std::vector<double> m((size_t)bs * bs, 0.0), e((size_t)bs * bs, 0.0);
    for (int s = 0; s < bs; s++) {
      int64_t r = B * bs + s;
      for (int64_t k = IA[r]; k < IA[r + 1]; k++) {
        int64_t c = JA[k];
        if (c >= B * bs && c < (B + 1) * bs) {
          m[s * bs + (c - B * bs)] = A[k];
          if (sym) m[(c - B * bs) * bs + s] = A[k];
        }
      }
      e[s * bs + s] = 1.0;
    }
    for (int col = 0; col < bs; col++) {
      int piv = col;
      for (int r = col + 1; r < bs; r++)
        if (std::fabs(m[r * bs + col]) > std::fabs(m[piv * bs + col])) piv = r;
      for (int k = 0; k < bs; k++) { std::swap(m[col * bs + k], m[piv * bs + k]); std::swap(e[col * bs + k], e[piv * bs + k]); }
      double d = m[col * bs + col];
      for (int k = 0; k < bs; k++) { m[col * bs + k] /= d; e[col * bs + k] /= d; }
      for (int r = 0; r < bs; r++) {
        if (r == col) continue;
        double f = m[r * bs + col];
        for (int k = 0; k < bs; k++) { m[r * bs + k] -= f * m[col * bs + k]; e[r * bs + k] -= f * e[col * bs + k]; }
      }
    }
    std::copy(e.begin(), e.end(), inv.begin() + (size_t)B * bs * bs);
  }
  auto M = [&](const double *r, double *z) {
    for (int64_t B = 0; B < nb; B++)
      for (int s = 0; s < bs; s++) {
        double acc = 0.0;
        for (int t = 0; t < bs; t++) acc += inv[(size_t)B * bs * bs + s * bs + t] * r[B * bs + t];
        z[B * bs + s] = acc;
      }
  };
  std::vector<double> r(n), z(n), p(n), q(n);
  double normb = std::sqrt(dot(n, b, b));
  for (int64_t i = 0; i < n; i++) { x[i] = 0.0; r[i] = b[i]; }
  if (normb == 0.0) normb = 1.0;
  double resid = std::sqrt(dot(n, r.data(), r.data())) / normb;
  if (resid <= tol) { *iters_out = 0; *resid_out = resid; return 0; }
  double rho = 0, rho_1 = 0;
  for (int64_t it = 1; it <= maxit; it++) {
    M(r.data(), z.data());
    rho = dot(n, r.data(), z.data());
    if (it == 1) p = z;
    else {
      double beta = rho / rho_1;
      for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
    }
    orc_spmv(n, sym, IA, JA, A, p.data(), q.data());
    double alpha = rho / dot(n, p.data(), q.data());
    for (int64_t i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
    resid = std::sqrt(dot(n, r.data(), r.data())) / normb;
    if (resid <= tol) { *iters_out = it; *resid_out = resid; return 0; }
    rho_1 = rho;
  }
  *iters_out = maxit;
  *resid_out = resid;
  return 1;
}

// Restarted, left-preconditioned GMRES(m) with Jacobi: Solvers/LinearSolvers/gmres.h:68-168
// (MGS Arnoldi, Givens rotations, Update back-solve :20-35).
int orc_gmres_jacobi(int64_t n, int sym, const int64_t *IA, const int64_t *JA, const double *A, const double *b, double *x,
                     int m, int64_t maxit, double tol, int64_t *iters_out, double *resid_out) {
  std::vector<double> diag(n);
  for (int64_t i = 0; i < n; i++) {
    double d = 0.0;
    for (int64_t k = IA[i]; k < IA[i + 1]; k++)
      if (JA[k] == i) { d = A[k]; break; }
    diag[i] = d;
  }
  auto M = [&](const double *in, double *out) { for (int64_t i = 0; i < n; i++) out[i] = in[i] / diag[i]; };
  auto nrm = [&](const std::vector<double> &v) { return std::sqrt(dot(n, v.data(), v.data())); };
  std::vector<double> r(n), w(n), w1(n), tmp(n);
  M(b, r.data());
  double normb = nrm(r);
  for (int64_t i = 0; i < n; i++) { x[i] = 0.0; r[i] = b[i]; }
  M(r.data(), w.data());
  r = w;
  double beta = nrm(r);
  if (normb == 0.0) normb = 1;
  double resid = beta / normb;
  if (resid <= tol) {
    for (int64_t i = 0; i < n; i++) x[i] += r[i];
    *iters_out = 0; *resid_out = resid; return 0;
  }
  std::vector<std::vector<double>> v(m + 1, std::vector<double>(n));
  std::vector<double> H((size_t)(m + 1) * (m + 1), 0.0), s(m + 1), cs(m + 1), sn(m + 1);
  auto h = [&](int i, int j) -> double & { return H[(size_t)j * (m + 1) + i]; };
  auto gen = [](double &dx, double &dy, double &c, double &sv) {
    if (dy == 0.0) { c = 1.0; sv = 0.0; }
    else if (std::fabs(dy) > std::fabs(dx)) { double t = dx / dy; sv = 1.0 / std::sqrt(1.0 + t * t); c = t * sv; }
    else { double t = dy / dx; c = 1.0 / std::sqrt(1.0 + t * t); sv = t * c; }
  };
  auto app = [](double &dx, double &dy, double c, double sv) { double t = c * dx + sv * dy; dy = -sv * dx + c * dy; dx = t; };
  auto update = [&](int k) {
    std::vector<double> y(s);
    for (int i = k; i >= 0; i--) {
      y[i] /= h(i, i);
      for (int j = i - 1; j >= 0; j--) y[j] -= h(j, i) * y[i];
    }
    for (int j = 0; j <= k; j++)
      for (int64_t q = 0; q < n; q++) x[q] += y[j] * v[j][q];
  };
  int64_t j = 1;
  while (j <= maxit) {
    for (int64_t i = 0; i < n; i++) v[0][i] = r[i] * (1.0 / beta);
    std::fill(s.begin(), s.end(), 0.0);
    s[0] = beta;
    for (int i = 0; i < m && j <= maxit; i++, j++) {
      orc_spmv(n, sym, IA, JA, A, v[i].data(), w1.data());
      M(w1.data(), w.data());
      for (int k = 0; k <= i; k++) {
        h(k, i) = dot(n, w.data(), v[k].data());
        for (int64_t q = 0; q < n; q++) w[q] -= h(k, i) * v[k][q];
      }
      h(i + 1, i) = nrm(w);
      for (int64_t q = 0; q < n; q++) v[i + 1][q] = w[q] * (1.0 / h(i + 1, i));
      for (int k = 0; k < i; k++) app(h(k, i), h(k + 1, i), cs[k], sn[k]);
      gen(h(i, i), h(i + 1, i), cs[i], sn[i]);
      app(h(i, i), h(i + 1, i), cs[i], sn[i]);
      app(s[i], s[i + 1], cs[i], sn[i]);
      resid = std::fabs(s[i + 1]) / normb;
      if (resid < tol) {
        update(i);
        *iters_out = j; *resid_out = resid; return 0;
      }
    }
    update(m - 1);
    orc_spmv(n, sym, IA, JA, A, x, tmp.data());
    for (int64_t i = 0; i < n; i++) tmp[i] = b[i] - tmp[i];
    M(tmp.data(), r.data());
    beta = nrm(r);
    resid = beta / normb;
    if (resid < tol) { *iters_out = j; *resid_out = resid; return 0; }
  }
  *iters_out = maxit;
  *resid_out = resid;
  return 1;
}

// Node-set blocks as TPZAnalysis::BuildPreconditioner(EBlockJacobi, overlap =
// false) computes them (Analysis/TPZAnalysis.cpp:1008-1085), restated as the
// reference writes them: TPZNodesetCompute::AnalyseGraph / AnalyseNode
// (External/tpznodesetcompute.cpp:47-188) on std::set copies of the closed
// neighbourhoods, recomputed when cleared, includes() and operator!= per
// neighbour, recursion into proper subsets, identical sets sharing the
// sequence number; BuildNodeGraph (:190-209), ExpandGraph over the TPZBlock
// (:528-562) and ColorGraph (:567-607).  The node graph is ConvertGraph's
// (External/TPZRenumbering.cpp:76-105).  Returns 0, or 1 at the reference's
// DebugStop (an identical set numbered apart).
namespace orc {
struct Nodeset {
  const std::vector<int64_t> &ng, &ngi;
  std::vector<int64_t> seq;
  std::vector<int> level;
  std::vector<char> included;
  std::vector<int64_t> card;
  int64_t maxseq = -1;
  int maxlevel = -1;
  bool ok = true;
  Nodeset(const std::vector<int64_t> &g, const std::vector<int64_t> &gi)
      : ng(g), ngi(gi), seq(gi.size() - 1, -1), level(gi.size() - 1, 0), included(gi.size() - 1, 0) {}
  void fill(int64_t v, std::vector<std::set<int64_t>> &ns) {
    if (ns[v].size()) return;
    ns[v].insert(ng.begin() + ngi[v], ng.begin() + ngi[v + 1]);
    ns[v].insert(v);
  }
  void analyse(int64_t node, std::vector<std::set<int64_t>> &ns) {
    if (seq[node] != -1) return;
    fill(node, ns);
    int minlevel = 0;
    std::vector<int64_t> equalnodes;
    for (auto it = ns[node].begin(); it != ns[node].end(); ++it) {
      const int64_t other = *it;
      if (other == node) continue;
      fill(other, ns);
      const bool inc = std::includes(ns[node].begin(), ns[node].end(), ns[other].begin(), ns[other].end());
      const bool diff = ns[node] != ns[other];
      if (inc && diff) {
        included[other] = 1;
        analyse(other, ns);
        minlevel = std::max(minlevel, level[other] + 1);
      } else if (!diff) {
        if (included[node]) included[other] = 1;
        equalnodes.push_back(other);
      }
      if (inc && diff && seq[other] != -1) {
        included[other] = 1;
        minlevel = std::max(minlevel, level[other] + 1);
      } else if (!diff && seq[other] != -1) {
        minlevel = std::max(minlevel, level[other]);
        ok = false;
      }
    }
    maxseq++;
    seq[node] = maxseq;
    card.push_back(1);
    maxlevel = std::max(maxlevel, minlevel);
    level[node] = minlevel;
    ns[node].erase(node);
    for (auto it = ns[node].begin(); it != ns[node].end(); ++it) {
      const int64_t other = *it;
      if (seq[other] != -1 && level[other] <= minlevel) {
        ns[other].clear();
        if (other == node) { ok = false; break; }
      }
    }
    ns[node].clear();
    for (int64_t o : equalnodes) {
      seq[o] = maxseq;
      level[o] = minlevel;
      ns[o].clear();
      card[maxseq]++;
    }
  }
};
}  // namespace orc

int orc_nodeset(int64_t nnodes, int64_t nel, const int64_t *eptr, const int64_t *eg, const int64_t *block_pos,
                const int64_t *block_size, int64_t neq, int64_t *blockindex, int64_t *blockeqs, int64_t *nblocks,
                int *colors, int *ncolors, int64_t *seqnum, int *level) {
  std::vector<std::vector<int64_t>> n2e(nnodes);
  for (int64_t e = 0; e < nel; e++)
    for (int64_t k = eptr[e]; k < eptr[e + 1]; k++) n2e[eg[k]].push_back(e);
  std::vector<int64_t> ngi(nnodes + 1, 0), ng;
  for (int64_t v = 0; v < nnodes; v++) {
    std::set<int64_t> con;
    for (int64_t e : n2e[v]) con.insert(eg + eptr[e], eg + eptr[e + 1]);
    con.erase(v);
    ng.insert(ng.end(), con.begin(), con.end());
    ngi[v + 1] = (int64_t)ng.size();
  }
  orc::Nodeset an(ng, ngi);
  {
    std::vector<std::set<int64_t>> ns(nnodes);
    for (int64_t in = 0; in < nnodes; in++) an.analyse(in, ns);
  }
  if (!an.ok) return 1;
  // BuildNodeGraph
  const int64_t nseq = (int64_t)an.card.size();
  std::vector<int64_t> bgi(nseq + 1, 0), bg(nnodes);
  if (nseq >= 1) bgi[1] = 0;
  for (int64_t s = 2; s <= nseq; s++) bgi[s] = bgi[s - 1] + an.card[s - 2];
  for (int64_t in = 0; in < nnodes; in++) {
    const int64_t sn = an.seq[in];
    bg[bgi[sn + 1]] = in;
    bgi[sn + 1]++;
  }
  // ExpandGraph
  int64_t counter = 0, blcounter = 0;
  std::vector<int64_t> egi(nseq + 1, 0);
  std::vector<int64_t> expg;
  for (int64_t ibl = 0; ibl < nseq; ibl++) {
    for (int64_t ieq = bgi[ibl]; ieq < bgi[ibl + 1]; ieq++) {
      const int64_t bsz = block_size[bg[ieq]], pos = block_pos[bg[ieq]];
      for (int64_t b = 0; b < bsz; b++) { expg.push_back(pos + b); counter++; }
    }
    if (egi[blcounter] != counter) egi[++blcounter] = counter;
  }
  // ColorGraph
  std::vector<int> eqcolor(neq), col(blcounter, -1);
  int color = 0;
  bool hasuncolored = true;
  while (hasuncolored) {
    hasuncolored = false;
    std::fill(eqcolor.begin(), eqcolor.end(), -1);
    for (int64_t ibl = 0; ibl < blcounter; ibl++) {
      if (col[ibl] != -1) continue;
      int64_t ieq;
      for (ieq = egi[ibl]; ieq < egi[ibl + 1]; ieq++)
        if (eqcolor[expg[ieq]] == color) break;
      if (ieq != egi[ibl + 1]) {
        hasuncolored = true;
      } else {
        col[ibl] = color;
        for (ieq = egi[ibl]; ieq < egi[ibl + 1]; ieq++) eqcolor[expg[ieq]] = color;
      }
    }
    color++;
  }
  *nblocks = blcounter;
  std::copy(egi.begin(), egi.begin() + blcounter + 1, blockindex);
  std::copy(expg.begin(), expg.end(), blockeqs);
  if (colors) std::copy(col.begin(), col.end(), colors);
  if (ncolors) *ncolors = color;
  if (seqnum) std::copy(an.seq.begin(), an.seq.end(), seqnum);
  if (level) std::copy(an.level.begin(), an.level.end(), level);
  return 0;
}

// CG with the node-set block preconditioner that BuildSequenceSolver returns for
// one colour (Analysis/TPZAnalysis.cpp:1093-1107): a TPZStepSolver(ELU) over a
// TPZSparseBlockDiagonal (Matrix/tpzsparseblockdiagonal.cpp) whose blocks
// UpdateFrom copies out of the matrix (GetSub, :300-322), factored by
// TPZFMatrix::Decompose_LU without pivoting, a zero pivot (IsZero, |a| <
// 1e-12) replaced by 1 (Matrix/pzfmatrix.cpp:1285-1320), and solved by
// TPZFMatrix::Substitution (:1354-1385) on the gathered residual; equations in
// no block get zero (Substitution zeroes B before the scatter, :148-156).  The
// CG loop is that of orc_cg_block_jacobi (Solvers/LinearSolvers/cg.h:29-132).
int orc_cg_sparse_block_jacobi(int64_t n, int sym, const int64_t *IA, const int64_t *JA, const double *A,
                               const double *b, double *x, int64_t nblocks, const int64_t *blockindex,
                               const int64_t *blockeqs, int64_t maxit, double tol, int64_t *iters_out,
                               double *resid_out) {
  std::vector<int64_t> local(n, -1), lupos(nblocks + 1, 0);
  for (int64_t B = 0; B < nblocks; B++) {
    const int64_t bs = blockindex[B + 1] - blockindex[B];
    lupos[B + 1] = lupos[B] + bs * bs;
  }
  std::vector<double> lu(lupos[nblocks], 0.0);
  for (int64_t B = 0; B < nblocks; B++) {
    const int64_t b0 = blockindex[B], bs = blockindex[B + 1] - b0;
    double *m = lu.data() + lupos[B];  // column-major bs x bs, as TPZFMatrix
    for (int64_t s = 0; s < bs; s++) local[blockeqs[b0 + s]] = s;
    for (int64_t s = 0; s < bs; s++) {
      const int64_t r = blockeqs[b0 + s];
      for (int64_t k = IA[r]; k < IA[r + 1]; k++) {
        const int64_t t = local[JA[k]];
        if (t < 0) continue;
        m[t * bs + s] = A[k];
        if (sym) m[s * bs + t] = A[k];
      }
    }
    for (int64_t s = 0; s < bs; s++) local[blockeqs[b0 + s]] = -1;
    for (int64_t k = 0; k < bs; k++) {
      double pivot = m[k * bs + k];
      if (std::fabs(pivot) < 1.e-12) { m[k * bs + k] = 1.0; pivot = 1.0; }
      for (int64_t i = k + 1; i < bs; i++) m[k * bs + i] /= pivot;
      for (int64_t j = k + 1; j < bs; j++) {
        const double kj = m[j * bs + k];
        for (int64_t i = k + 1; i < bs; i++) m[j * bs + i] -= m[k * bs + i] * kj;
      }
    }
  }
  auto M = [&](const double *r, double *z) {
    for (int64_t i = 0; i < n; i++) z[i] = 0.0;
    std::vector<double> y;
    for (int64_t B = 0; B < nblocks; B++) {
      const int64_t b0 = blockindex[B], bs = blockindex[B + 1] - b0;
      const double *m = lu.data() + lupos[B];
      y.assign(bs, 0.0);
      for (int64_t s = 0; s < bs; s++) y[s] = r[blockeqs[b0 + s]];
      for (int64_t i = 0; i < bs; i++)
        for (int64_t j = 0; j < i; j++) y[i] -= m[j * bs + i] * y[j];
      for (int64_t i = bs - 1; i >= 0; i--) {
        for (int64_t j = i + 1; j < bs; j++) y[i] -= m[j * bs + i] * y[j];
        y[i] /= m[i * bs + i];
      }
      for (int64_t s = 0; s < bs; s++) z[blockeqs[b0 + s]] += y[s];
    }
  };
  std::vector<double> r(n), z(n), p(n), q(n);
  double normb = std::sqrt(dot(n, b, b));
  for (int64_t i = 0; i < n; i++) { x[i] = 0.0; r[i] = b[i]; }
  if (normb == 0.0) normb = 1.0;
  double resid = std::sqrt(dot(n, r.data(), r.data())) / normb;
  if (resid <= tol) { *iters_out = 0; *resid_out = resid; return 0; }
  double rho = 0, rho_1 = 0;
  for (int64_t it = 1; it <= maxit; it++) {
    M(r.data(), z.data());
    rho = dot(n, r.data(), z.data());
    if (it == 1) p = z;
    else {
      double beta = rho / rho_1;
      for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
    }
    orc_spmv(n, sym, IA, JA, A, p.data(), q.data());
    double alpha = rho / dot(n, p.data(), q.data());
    for (int64_t i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
    resid = std::sqrt(dot(n, r.data(), r.data())) / normb;
    if (resid <= tol) { *iters_out = it; *resid_out = resid; return 0; }
    rho_1 = rho;
  }
  *iters_out = maxit;
  *resid_out = resid;
  return 1;
}

}  // extern "C"

