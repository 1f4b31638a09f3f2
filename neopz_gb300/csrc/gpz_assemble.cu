// Element integration and atomic-free coloured scatter (FP64 parity path).
//
// One CTA per element.  Per integration point: the geometric Jacobian from the
// corner coordinates (TPZGeoEl::Jacobian, Mesh/pzgeoel.cpp:1167-1345), the
// physical gradients dphix = jacinv^T dphi (Mesh/TPZCompElH1.cpp:139-149) and
// the weight w |detJ| (Mesh/pzinterpolationspace.cpp:454-470).  Then, per pair
// of shapes (a <= b), the gradient Gram S_ab = sum_q w_q g_a g_b^T from which the
// material block is formed (TPZMatPoisson / TPZDarcyFlow / TPZElasticity3D
// CODE3), and the block plus its transpose are added into the full CSR through
// the element's block-offset table.  Elements of one colour share no connect,
// so the read-modify-write needs no atomics.  Entries with |v| < 1e-12 are
// skipped exactly as TPZSYsmpMatrix::AddKel does (Matrix/pzsysmp.cpp:369-411).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <memory>

#include "gpz_internal.h"
#include "gpz_shapes.h"

namespace gpz {

bool BucketKey::operator<(const BucketKey &o) const {
  if (type != o.type) return type < o.type;
  if (is_bc != o.is_bc) return is_bc < o.is_bc;
  if (mat_kind != o.mat_kind) return mat_kind < o.mat_kind;
  if (mat_index != o.mat_index) return mat_index < o.mat_index;
  if (intorder != o.intorder) return intorder < o.intorder;
  if (hp != o.hp) return hp < o.hp;
  for (int i = 0; i < 19; i++)
    if (orders[i] != o.orders[i]) return orders[i] < o.orders[i];
  for (int i = 0; i < 19; i++)
    if (trans[i] != o.trans[i]) return trans[i] < o.trans[i];
  return false;
}

namespace {

struct ElemArgs {
  const double *phi, *dphi, *w;
  const double *ghat;  // reference Gram [NT][NT][3][3] of a volume hex bucket, or null
  const int *sside, *sk;
  int nq, ncorner, nsides, nshape;
  const double *xyz;
  const int64_t *el_nodes, *el_conn, *bpos;
  const int32_t *el_mat;
  const double *coef;
  int kind, mdim, forcing, bc_type;
  int rhs_only;  // load vector only (TPZStructMatrix::Assemble(rhs)): no matrix, no pattern needed
  double scale, E, nu, coef_const, big;
  double force[3], val2[3];
  const int64_t *ia, *offbase;
  const int32_t *off;
  double *a, *f;
  float *a32;  // the FP32 element pass: matrix into this FP32 CSR, no load vector
  int64_t nnz, neq;
  int *err;
  // shared element matrix (a volume bucket whose elements are translates of one box): K_e = s_e kref
  // (s_e the element's coefficient, kref the matrix at coefficient 1), F_e = fref when the forcing is constant
  const double *kref, *fref;
  // reference mode: the first element's matrix at coefficient 1 and its load vector into these dense arrays
  double *kdense, *fdense;
};

// Geometric Jacobian at one point: returns |detJ| and fills jinv (row-major dim x dim)
template <int DIM>
__device__ double jacobian_at(const double *cx /*[nc][3]*/, const double *dcorner /*[DIM][nc]*/, int nc,
                              double jinv[3][3]) {
  double gx[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int k = 0; k < nc; k++)
    for (int j = 0; j < 3; j++)
      for (int d = 0; d < DIM; d++) gx[j][d] += cx[k * 3 + j] * dcorner[d * 8 + k];
  double det;
  if (DIM == 1) {
    double n = sqrt(gx[0][0] * gx[0][0] + gx[1][0] * gx[1][0] + gx[2][0] * gx[2][0]);
    det = n;
    jinv[0][0] = 1.0 / n;
  } else if (DIM == 2) {
    double n1 = 0.0, d12 = 0.0, n2 = 0.0;
    for (int i = 0; i < 3; i++) { n1 += gx[i][0] * gx[i][0]; d12 += gx[i][0] * gx[i][1]; }
    n1 = sqrt(n1);
    for (int i = 0; i < 3; i++) {
      double v = gx[i][1] - d12 * (gx[i][0] / n1) / n1;
      n2 += v * v;
    }
    n2 = sqrt(n2);
    double j00 = n1, j01 = d12 / n1, j11 = n2;
    det = j00 * j11;
    jinv[0][0] = j11 / det;
    jinv[1][1] = j00 / det;
    jinv[0][1] = -j01 / det;
    jinv[1][0] = 0.0;
  } else {
    const double(&a)[3][3] = gx;
    det = -a[0][2] * a[1][1] * a[2][0] + a[0][1] * a[1][2] * a[2][0] + a[0][2] * a[1][0] * a[2][1] -
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
  }
  return fabs(det);
}

__device__ __forceinline__ void corner_grad(int nc, int dim, const double *pt, double *phic, double *dc /*[3][8]*/) {
  // master corners in the reference's node order
  const signed char sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
                    sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
  for (int k = 0; k < nc; k++) {
    double s[3] = {(double)sx[k], (double)sy[k], (double)sz[k]};
    if (dim == 1) s[0] = (k == 0) ? -1.0 : 1.0;
    double f[3], g[3];
    for (int a = 0; a < dim; a++) { f[a] = (1.0 + s[a] * pt[a]) / 2.0; g[a] = s[a] / 2.0; }
    double v = 1.0;
    for (int a = 0; a < dim; a++) v *= f[a];
    phic[k] = v;
    for (int a = 0; a < dim; a++) {
      double d = g[a];
      for (int b = 0; b < dim; b++)
        if (b != a) d *= f[b];
      dc[a * 8 + k] = d;
    }
  }
}

__device__ __forceinline__ void forcing_at(const ElemArgs &P, const double *x, double *fv) {
  fv[0] = fv[1] = fv[2] = 0.0;
  if (P.forcing == GPZ_F_CONST) {
    fv[0] = P.force[0]; fv[1] = P.force[1]; fv[2] = P.force[2];
  } else if (P.forcing == GPZ_F_SINPROD) {
    const double pi = 3.141592653589793238462643383279502884;
    double v = P.force[0] * (P.mdim == 2 ? 2.0 * pi * pi : 3.0 * pi * pi) * sin(pi * x[0]) * sin(pi * x[1]);
    if (P.mdim == 3) v *= sin(pi * x[2]);
    fv[0] = v;
  } else if (P.forcing == GPZ_F_QUADRATIC) {
    double r2 = x[0] * x[0] + x[1] * x[1];
    if (P.mdim == 3) r2 += x[2] * x[2];
    fv[0] = P.force[0] + P.force[1] * r2;
  }
}

// Active shapes of the elements of an hp class (one row of kMaxShapes per element).
struct HpArgs {
  const uint8_t *full;  // index into the class table
  const uint8_t *k;     // index inside its side (the element's own enumeration)
  const int32_t *n;     // number of shapes of the element
};

// NSH_T table shapes (0: read at run time), DIM element dimension, NST states
// per shape, BC boundary element.  HP: the element uses a subset of the table's
// shapes (hp element of uneven side orders; the H1 shapes of a side of order o
// are among those of the same side at the class order, with the same values),
// listed per element in H.  Any block size that is a multiple of 32 works; the
// hp classes' block size is autotuned.
// One element's matrix and load vector, scattered into the CSR (or, in the
// reference mode, into dense arrays; with F32, the matrix alone into the FP32
// CSR of the mixed solves).  In the queue kernel below the
// read-modify-writes of the matrix and the load vector read through L2 (ld.cg):
// one CTA handles elements of several colours there, and a line cached in its
// SM's L1 by an earlier colour may since have been changed by another SM.
template <int NSH_T, int DIM, int NST, bool BC, bool HP, bool QUEUE, bool F32 = false>
__device__ __forceinline__ void elem_body(const ElemArgs &P, const HpArgs &H, const int64_t *__restrict__ elems,
                                          int64_t ie) {
  extern __shared__ double sm[];
  const int NT = NSH_T > 0 ? NSH_T : P.nshape;  // shapes of the table (its row stride)
  const int NSH = HP ? H.n[ie] : NT;            // shapes of this element
  const int nq = P.nq;
  double *sG = sm;                                    // [nq][NSH][DIM] (volume)
  double *sW = sG + (BC ? 0 : nq * NSH * DIM);        // [nq]
  double *sX = sW + nq;                               // [nq][3]
  double *sC = sX + nq * 3;                           // [8][3] corners
  int64_t *sRow = (int64_t *)(sC + 24);               // [NSH] first equation of each shape
  int *sSide = (int *)(sRow + NSH);                   // [NSH]
  int *sIdx = sSide + NSH;                            // [NSH] table index of each shape
  int *sK = sIdx + NSH;                               // [NSH] index of the shape inside its side
  __shared__ double sCoef;
  __shared__ int64_t sOffBase;

  const int64_t e = elems[ie];
  const int tid = threadIdx.x;
  const int nc = P.ncorner;

  if (tid < nc * 3) {
    int k = tid / 3, j = tid % 3;
    int64_t node = P.el_nodes[e * 8 + k];
    sC[k * 3 + j] = P.xyz[node * 3 + j];
  }
  for (int a = tid; a < NSH; a += blockDim.x) {
    const int fa = HP ? (int)H.full[ie * kMaxShapes + a] : a;
    const int ka = HP ? (int)H.k[ie * kMaxShapes + a] : P.sk[a];
    const int side = P.sside[fa];
    const int64_t cn = P.el_conn[e * 27 + side];
    sRow[a] = P.bpos[cn] + (int64_t)ka * NST;
    sSide[a] = side;
    sIdx[a] = fa;
    sK[a] = ka;
  }
  __shared__ int sAff;
  __shared__ double sJi[3][3], sDet;
  const bool shared = !BC && P.kref != nullptr, dense = !BC && P.kdense != nullptr;
  if (tid == 0) {
    sOffBase = (P.rhs_only || dense) ? 0 : P.offbase[e];
    double cf = P.kind == GPZ_MAT_ELAST3D ? P.E : P.coef_const;
    if (!BC && P.coef) cf = P.coef[e];
    sCoef = dense && P.kind != GPZ_MAT_POISSON ? 1.0 : cf;  // the reference matrix is at coefficient 1
    sAff = 0;
  }
  __syncthreads();
  if (!BC && !shared && DIM == 3 && P.ghat != nullptr && tid == 0) {
    // affine hex: the trilinear map's xi.eta, xi.zeta, eta.zeta and xi.eta.zeta
    // coefficients vanish, the Jacobian is constant and the element Gram is
    // |J| Jinv^T G Jinv with the bucket's reference Gram G
    const signed char c4[8] = {1, -1, 1, -1, 1, -1, 1, -1}, c5[8] = {1, -1, -1, 1, -1, 1, 1, -1},
                      c6[8] = {1, 1, -1, -1, -1, -1, 1, 1}, c7[8] = {-1, 1, -1, 1, 1, -1, 1, -1};
    double big = 0.0, hi = 0.0;
    for (int j = 0; j < 3; j++) {
      double t4 = 0, t5 = 0, t6 = 0, t7 = 0, mn = sC[j], mx = sC[j];
      for (int k = 0; k < 8; k++) {
        const double x = sC[k * 3 + j];
        t4 += c4[k] * x;
        t5 += c5[k] * x;
        t6 += c6[k] * x;
        t7 += c7[k] * x;
        mn = fmin(mn, x);
        mx = fmax(mx, x);
      }
      hi = fmax(hi, fmax(fmax(fabs(t4), fabs(t5)), fmax(fabs(t6), fabs(t7))));
      big = fmax(big, mx - mn);
    }
    if (hi <= 1e-12 * big) {
      // the Jacobian from the corner gradients at the first point (as at every point)
      double dc[3 * 8];
      for (int k = 0; k < nc; k++)
        for (int d = 0; d < DIM; d++) dc[d * 8 + k] = P.dphi[(0 * DIM + d) * NT + k];
      double ji[3][3];
      sDet = jacobian_at<DIM>(sC, dc, nc, ji);
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) sJi[i][j] = ji[i][j];
      sAff = 1;
    }
  }
  __syncthreads();
  const bool aff = sAff != 0;

  // per-point geometry (a shared element matrix with a constant forcing needs none)
  const bool geo = !(shared && P.fref != nullptr);
  for (int q = tid; geo && q < nq; q += blockDim.x) {
    double pt[3] = {0, 0, 0};
    // reference point recovered from the corner table is not needed: use dcorner at the point
    // (the bucket tables hold the point implicitly through phi of the corner shapes)
    double phic[8], dc[3 * 8];
    // corner shapes are the first nc shapes of the table; their gradients give J
    for (int k = 0; k < nc; k++) {
      phic[k] = P.phi[q * NT + k];  // the corner shapes are the table's first nc, active in every element
      for (int d = 0; d < DIM; d++) dc[d * 8 + k] = P.dphi[(q * DIM + d) * NT + k];
    }
    (void)pt;
    double jinv[3][3];
    const double det = aff ? sDet : jacobian_at<DIM>(sC, dc, nc, jinv);
    sW[q] = P.w[q] * det;
    for (int j = 0; j < 3; j++) {
      double x = 0.0;
      for (int k = 0; k < nc; k++) x += phic[k] * sC[k * 3 + j];
      sX[q * 3 + j] = x;
    }
    if (!BC && !aff && !shared) {
      // store jinv temporarily in sG is not possible; compute gradients directly
      for (int a = 0; a < NSH; a++) {
        const int fa = HP ? sIdx[a] : a;
        for (int d = 0; d < DIM; d++) {
          double g = 0.0;
          for (int j = 0; j < DIM; j++) g += jinv[j][d] * P.dphi[(q * DIM + j) * NT + fa];
          sG[(q * NSH + a) * DIM + d] = g;
        }
      }
    }
  }
  __syncthreads();

  const double coef = sCoef;
  // ---- load vector
  for (int idx = tid; !F32 && idx < NSH * NST; idx += blockDim.x) {
    int a = idx / NST, s = idx % NST;
    const int fa = HP ? sIdx[a] : a;
    double acc = 0.0;
    if (shared && P.fref != nullptr) {
      acc = P.fref[idx];
    } else if (!BC) {
      for (int q = 0; q < nq; q++) {
        double fv[3];
        forcing_at(P, &sX[q * 3], fv);
        double ph = P.phi[q * NT + fa];
        if (P.kind == GPZ_MAT_POISSON) acc += sW[q] * P.scale * ph * fv[0];
        else if (P.kind == GPZ_MAT_DARCY) acc += sW[q] * fv[0] * ph;
        else acc += sW[q] * (fv[s] * ph);
      }
    } else {
      double m = 0.0;
      for (int q = 0; q < nq; q++) m += P.phi[q * NT + fa] * sW[q];
      if (P.bc_type == 0) acc = P.big * P.val2[s] * m;
      else if (P.bc_type == 1) acc = P.val2[s] * m * (P.kind == GPZ_MAT_POISSON ? P.scale : 1.0);
    }
    if (dense) {
      P.fdense[idx] = acc;
      continue;
    }
    int64_t row = sRow[a] + s;
    if (row < 0 || row >= P.neq) {
      atomicOr(P.err, 16);
      continue;
    }
    P.f[row] = (QUEUE ? __ldcg(P.f + row) : P.f[row]) + acc;
  }
  if ((BC && P.bc_type != 0) || P.rhs_only) return;

  // ---- matrix: pairs a <= b
  double C1 = 0, C2 = 0, C3 = 0;
  if (!BC && P.kind == GPZ_MAT_ELAST3D) {
    double E = coef, nu = P.nu;
    C1 = E / (2. + 2. * nu);
    C2 = E * nu / (-1. + nu + 2. * nu * nu);
    C3 = E * (nu - 1.) / (-1. + nu + 2. * nu * nu);
  }
  const int ns = P.nsides;
  for (int idx = tid; idx < NSH * NSH; idx += blockDim.x) {
    const int a = idx / NSH, b = idx % NSH;
    if (a > b) continue;
    double K[NST][NST];
    if (shared) {
      const int nd = NSH * NST;
      const double cs = P.kind == GPZ_MAT_POISSON ? 1.0 : coef;
      for (int s = 0; s < NST; s++)
        for (int t = 0; t < NST; t++) K[s][t] = cs * P.kref[(size_t)(a * NST + s) * nd + b * NST + t];
    } else if (BC) {
      const int fa = HP ? sIdx[a] : a, fb = HP ? sIdx[b] : b;
      double m = 0.0;
      for (int q = 0; q < nq; q++) m += sW[q] * P.phi[q * NT + fa] * P.phi[q * NT + fb];
      for (int s = 0; s < NST; s++)
        for (int t = 0; t < NST; t++) K[s][t] = (s == t) ? P.big * m : 0.0;
    } else if (aff) {
      // S = |J| Jinv^T G_ab Jinv (S[d][e] = sum_q w |J| g_a,d g_b,e as below)
      const int fa = HP ? sIdx[a] : a, fb = HP ? sIdx[b] : b;
      const double *G = P.ghat + ((size_t)fa * NT + fb) * 9;
      double M1[3][3], S[3][3];
      for (int i = 0; i < 3; i++)
        for (int e2 = 0; e2 < 3; e2++) M1[i][e2] = G[i * 3 + 0] * sJi[0][e2] + G[i * 3 + 1] * sJi[1][e2] + G[i * 3 + 2] * sJi[2][e2];
      for (int d = 0; d < 3; d++)
        for (int e2 = 0; e2 < 3; e2++)
          S[d][e2] = sDet * (sJi[0][d] * M1[0][e2] + sJi[1][d] * M1[1][e2] + sJi[2][d] * M1[2][e2]);
      if (NST == 1) {
        K[0][0] = (P.kind == GPZ_MAT_POISSON ? P.scale : coef) * (S[0][0] + S[1][1] + S[2][2]);
      } else {
        double tr = S[0][0] + S[1][1] + S[2][2];
        for (int s = 0; s < NST; s++)
          for (int t = 0; t < NST; t++)
            K[s][t] = (s == t) ? (tr - S[s][s]) * C1 + S[s][s] * C3 : S[t][s] * C1 - S[s][t] * C2;
      }
    } else if (NST == 1) {
      double acc = 0.0;
      for (int q = 0; q < nq; q++) {
        const double *ga = &sG[(q * NSH + a) * DIM], *gb = &sG[(q * NSH + b) * DIM];
        double d = 0.0;
        for (int x = 0; x < DIM; x++) d += ga[x] * gb[x];
        acc += sW[q] * d;
      }
      K[0][0] = (P.kind == GPZ_MAT_POISSON ? P.scale : coef) * acc;
    } else {
      double S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      for (int q = 0; q < nq; q++) {
        const double *ga = &sG[(q * NSH + a) * DIM], *gb = &sG[(q * NSH + b) * DIM];
        const double w = sW[q];
        double wa0 = w * ga[0], wa1 = w * ga[1], wa2 = w * ga[2];
        S[0][0] += wa0 * gb[0]; S[0][1] += wa0 * gb[1]; S[0][2] += wa0 * gb[2];
        S[1][0] += wa1 * gb[0]; S[1][1] += wa1 * gb[1]; S[1][2] += wa1 * gb[2];
        S[2][0] += wa2 * gb[0]; S[2][1] += wa2 * gb[1]; S[2][2] += wa2 * gb[2];
      }
      double tr = S[0][0] + S[1][1] + S[2][2];
      for (int s = 0; s < NST; s++)
        for (int t = 0; t < NST; t++)
          K[s][t] = (s == t) ? (tr - S[s][s]) * C1 + S[s][s] * C3 : S[t][s] * C1 - S[s][t] * C2;
    }
    if (dense) {
      const int nd = NSH * NST;
      for (int s = 0; s < NST; s++)
        for (int t = 0; t < NST; t++) {
          P.kdense[(size_t)(a * NST + s) * nd + b * NST + t] = K[s][t];
          P.kdense[(size_t)(b * NST + t) * nd + a * NST + s] = K[s][t];
        }
      continue;
    }
    // scatter the (a,b) block and, off the diagonal, its transpose into (b,a)
    const int sa = sSide[a], sb = sSide[b];
    const int32_t oab = P.off[sOffBase + sa * ns + sb];
    const int32_t oba = P.off[sOffBase + sb * ns + sa];
    if (oab < 0 || oba < 0) {
      atomicOr(P.err, 32);
      continue;
    }
    const int ka = sK[a] * NST, kb = sK[b] * NST;
    if (F32) {
      int64_t slot[2][NST][NST];
      float old[2][NST][NST];
      bool bad = false;
#pragma unroll
      for (int s = 0; s < NST; s++)
#pragma unroll
        for (int t = 0; t < NST; t++) {
          slot[0][s][t] = P.ia[sRow[a] + s] + oab + kb + t;
          slot[1][s][t] = P.ia[sRow[b] + t] + oba + ka + s;
        }
#pragma unroll
      for (int h = 0; h < 2; h++)
#pragma unroll
        for (int s = 0; s < NST; s++)
#pragma unroll
          for (int t = 0; t < NST; t++) {
            const int64_t q = slot[h][s][t];
            const bool use = fabs(K[s][t]) >= 1.e-12 && (h == 0 || a != b);
            bad |= use && (q < 0 || q >= P.nnz);
            old[h][s][t] = use && q >= 0 && q < P.nnz ? P.a32[q] : 0.f;
          }
      if (bad) atomicOr(P.err, 64);
#pragma unroll
      for (int h = 0; h < 2; h++)
#pragma unroll
        for (int s = 0; s < NST; s++)
#pragma unroll
          for (int t = 0; t < NST; t++) {
            const int64_t q = slot[h][s][t];
            if (fabs(K[s][t]) >= 1.e-12 && (h == 0 || a != b) && q >= 0 && q < P.nnz)
              P.a32[q] = old[h][s][t] + (float)K[s][t];
          }
      continue;
    }
    // the block's (and its transpose's) slots are distinct entries of the CSR: every old value is loaded
    // before the first store, so the loads are in flight together instead of one per store
    int64_t slot[2][NST][NST];
    double old[2][NST][NST];
    bool bad = false;
#pragma unroll
    for (int s = 0; s < NST; s++) {
      const int64_t base = P.ia[sRow[a] + s] + oab + kb;
#pragma unroll
      for (int t = 0; t < NST; t++) slot[0][s][t] = base + t;
    }
#pragma unroll
    for (int t = 0; t < NST; t++) {
      const int64_t base = P.ia[sRow[b] + t] + oba + ka;
#pragma unroll
      for (int s = 0; s < NST; s++) slot[1][s][t] = base + s;
    }
#pragma unroll
    for (int h = 0; h < 2; h++)
#pragma unroll
      for (int s = 0; s < NST; s++)
#pragma unroll
        for (int t = 0; t < NST; t++) {
          const int64_t q = slot[h][s][t];
          const bool use = fabs(K[s][t]) >= 1.e-12 && (h == 0 || a != b);
          bad |= use && (q < 0 || q >= P.nnz);
          old[h][s][t] = use && q >= 0 && q < P.nnz ? (QUEUE ? __ldcg(P.a + q) : P.a[q]) : 0.0;
        }
    if (bad) atomicOr(P.err, 64);
#pragma unroll
    for (int h = 0; h < 2; h++)
#pragma unroll
      for (int s = 0; s < NST; s++)
#pragma unroll
        for (int t = 0; t < NST; t++) {
          const int64_t q = slot[h][s][t];
          if (fabs(K[s][t]) >= 1.e-12 && (h == 0 || a != b) && q >= 0 && q < P.nnz) P.a[q] = old[h][s][t] + K[s][t];
        }
  }
}

// one CTA per element (a launch per bucket and colour)
template <int NSH_T, int DIM, int NST, bool BC, bool HP>
__global__ void __launch_bounds__(256) k_elem_fp64(ElemArgs P, HpArgs H, const int64_t *__restrict__ elems,
                                                   int64_t nelems) {
  const int64_t ie = blockIdx.x;
  if (ie >= nelems) return;
  elem_body<NSH_T, DIM, NST, BC, HP, false>(P, H, elems, ie);
}

// the FP32 element pass of the element types the tensor-core kernel does not take
template <int NSH_T, int DIM, int NST, bool BC, bool HP>
__global__ void __launch_bounds__(256) k_elem_f32(ElemArgs P, HpArgs H, const int64_t *__restrict__ elems,
                                                  int64_t nelems) {
  const int64_t ie = blockIdx.x;
  if (ie >= nelems) return;
  elem_body<NSH_T, DIM, NST, BC, HP, false, true>(P, H, elems, ie);
}

// Persistent form (one launch per bucket, every colour): resident CTAs take the
// bucket's elements from a work counter in colour order; an element of colour c
// starts once every element of the earlier colours is done (a second counter;
// elements of one colour share no connect, so the scatter needs no atomics).
// Items are taken in order and each is held by a running CTA, so every wait
// ends; it is bounded all the same, and a wait that gives up sets an error flag
// and stops its CTA.
struct QueueArgs {
  unsigned long long *next, *done;  // work counter, finished elements
  const int64_t *cbeg;              // [ncol + 1] colour boundaries in the bucket's element list
  int ncol;
};
constexpr int kQueueWaitTries = 1 << 24;

template <int NSH_T, int DIM, int NST, bool BC, bool HP>
__global__ void __launch_bounds__(256) k_elem_fp64_queue(ElemArgs P, HpArgs H, const int64_t *__restrict__ elems,
                                                         int64_t nelems, QueueArgs Q) {
  __shared__ int64_t s_item;
  for (;;) {
    if (threadIdx.x == 0) {
      int64_t it = (int64_t)atomicAdd(Q.next, 1ull);
      if (it < nelems) {
        int c = 0;
        while (c + 1 < Q.ncol && Q.cbeg[c + 1] <= it) c++;
        const unsigned long long need = (unsigned long long)Q.cbeg[c];
        int tries = 0;
        while (*(volatile unsigned long long *)Q.done < need) {
          if (++tries > kQueueWaitTries) {
            atomicOr(P.err, 32768);
            it = nelems;  // give up: this CTA stops
            break;
          }
          __nanosleep(128);
        }
        __threadfence();  // the earlier colours' writes before this element's reads
      }
      s_item = it;
    }
    __syncthreads();
    const int64_t it = s_item;
    if (it >= nelems) return;
    elem_body<NSH_T, DIM, NST, BC, HP, true>(P, H, elems, it);
    __threadfence();  // this element's writes before it is counted done
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(Q.done, 1ull);
  }
}

size_t smem_bytes(int nsh, int dim, int nq, bool bc) {
  size_t d = (bc ? 0 : (size_t)nq * nsh * dim) + nq + (size_t)nq * 3 + 24;
  return d * sizeof(double) + (size_t)nsh * (sizeof(int64_t) + 3 * sizeof(int)) + 16;
}

typedef void (*ElemKernel)(ElemArgs, HpArgs, const int64_t *, int64_t);
typedef void (*QueueKernel)(ElemArgs, HpArgs, const int64_t *, int64_t, QueueArgs);
struct Kernels {
  ElemKernel one = nullptr;    // a CTA per element, a launch per colour
  QueueKernel queue = nullptr;  // persistent, every colour in one launch
};

template <int NSH, int DIM, int NST, bool BC, bool HP = false>
Kernels pick() {
  return Kernels{k_elem_fp64<NSH, DIM, NST, BC, HP>, k_elem_fp64_queue<NSH, DIM, NST, BC, HP>};
}

// compile-time shape counts of the uniform-order elements; nullptr: use the batched run-time kernel
Kernels select_kernel(int type, int nshape, int nstate, bool bc) {
  // volume hexes (3D) and quads (2D); boundary quads (3D faces) and lines (2D edges)
  if (type == GPZ_EL_HEX && !bc) {
    if (nstate == 1) {
      if (nshape == 8) return pick<8, 3, 1, false>();
      if (nshape == 27) return pick<27, 3, 1, false>();
      if (nshape == 64) return pick<64, 3, 1, false>();
    } else {
      if (nshape == 8) return pick<8, 3, 3, false>();
      if (nshape == 27) return pick<27, 3, 3, false>();
      if (nshape == 64) return pick<64, 3, 3, false>();
    }
  }
  if (type == GPZ_EL_QUAD && !bc && nstate == 1) {
    if (nshape == 4) return pick<4, 2, 1, false>();
    if (nshape == 9) return pick<9, 2, 1, false>();
    if (nshape == 16) return pick<16, 2, 1, false>();
  }
  if (type == GPZ_EL_QUAD && bc) {
    if (nstate == 1) {
      if (nshape == 4) return pick<4, 2, 1, true>();
      if (nshape == 9) return pick<9, 2, 1, true>();
      if (nshape == 16) return pick<16, 2, 1, true>();
    } else {
      if (nshape == 4) return pick<4, 2, 3, true>();
      if (nshape == 9) return pick<9, 2, 3, true>();
      if (nshape == 16) return pick<16, 2, 3, true>();
    }
  }
  if (type == GPZ_EL_LINE && bc && nstate == 1) {
    if (nshape == 2) return pick<2, 1, 1, true>();
    if (nshape == 3) return pick<3, 1, 1, true>();
    if (nshape == 4) return pick<4, 1, 1, true>();
  }
  return Kernels{};
}

// FP64 integration with the FP32 scatter: boundary elements and 2D quads (the
// volume hexes go to the tensor-core kernel)
template <int NSH, int DIM, int NST, bool BC, bool HP = false>
ElemKernel pick32() {
  return k_elem_f32<NSH, DIM, NST, BC, HP>;
}
ElemKernel select_f32(int type, int nshape, int nstate, bool bc, bool hp) {
  if (type == GPZ_EL_QUAD && !bc && nstate == 1) {
    if (hp) return pick32<0, 2, 1, false, true>();
    if (nshape == 4) return pick32<4, 2, 1, false>();
    if (nshape == 9) return pick32<9, 2, 1, false>();
    if (nshape == 16) return pick32<16, 2, 1, false>();
  }
  if (type == GPZ_EL_QUAD && bc) {
    if (nstate == 1) {
      if (hp) return pick32<0, 2, 1, true, true>();
      if (nshape == 4) return pick32<4, 2, 1, true>();
      if (nshape == 9) return pick32<9, 2, 1, true>();
      if (nshape == 16) return pick32<16, 2, 1, true>();
    } else {
      if (hp) return pick32<0, 2, 3, true, true>();
      if (nshape == 4) return pick32<4, 2, 3, true>();
      if (nshape == 9) return pick32<9, 2, 3, true>();
      if (nshape == 16) return pick32<16, 2, 3, true>();
    }
  }
  if (type == GPZ_EL_LINE && bc && nstate == 1) {
    if (hp) return pick32<0, 1, 1, true, true>();
    if (nshape == 2) return pick32<2, 1, 1, true>();
    if (nshape == 3) return pick32<3, 1, 1, true>();
    if (nshape == 4) return pick32<4, 1, 1, true>();
  }
  return nullptr;
}

// the run-time kernel of an hp class
Kernels select_hp(int type, int nstate, bool bc) {
  if (type == GPZ_EL_HEX && !bc) return nstate == 1 ? pick<0, 3, 1, false, true>() : pick<0, 3, 3, false, true>();
  if (type == GPZ_EL_QUAD && !bc && nstate == 1) return pick<0, 2, 1, false, true>();
  if (type == GPZ_EL_QUAD && bc) return nstate == 1 ? pick<0, 2, 1, true, true>() : pick<0, 2, 3, true, true>();
  if (type == GPZ_EL_LINE && bc && nstate == 1) return pick<0, 1, 1, true, true>();
  return Kernels{};
}

__global__ void k_extract_diag(const double *__restrict__ a, const int64_t *__restrict__ diagpos, int64_t neq,
                               double *__restrict__ dinv) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < neq) dinv[r] = 1.0 / a[diagpos[r]];
}

__global__ void k_to_fp32(const double *__restrict__ a, float *__restrict__ b, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) b[i] = (float)a[i];
}

}  // namespace

void build_buckets(Ctx &c, const gpz_mesh_desc &d) {
  for (Bucket *b : c.buckets) delete b;
  c.buckets.clear();
  c.rp_bucket = nullptr;
  const auto t0 = std::chrono::steady_clock::now();
  // rows of the hp elements' active shapes (written and read for hp elements only)
  std::unique_ptr<uint8_t[]> act_full(new uint8_t[(size_t)c.nel * kMaxShapes]),
      act_k(new uint8_t[(size_t)c.nel * kMaxShapes]);
  std::vector<int32_t> act_n(c.nel, 0);
  // the bucket key of element e, and for an hp element its active shapes
  auto key_of = [&](int64_t e, BucketKey &k) {
    k = BucketKey{};
    k.type = d.el_type[e];
    GPZ_REQUIRE(k.type == GPZ_EL_LINE || k.type == GPZ_EL_QUAD || k.type == GPZ_EL_HEX, GPZ_E_UNSUPPORTED_ELEMENT,
                "element type");
    const ElemTopo &t = topo(k.type);
    k.is_bc = d.el_mat[e] < 0;
    const gpz_material *m;
    if (k.is_bc) {
      int ib = -d.el_mat[e] - 1;
      GPZ_REQUIRE(ib < d.nbc, GPZ_E_INVALID, "bc index");
      int im = d.bcs[ib].material;
      GPZ_REQUIRE(im >= 0 && im < d.nmat, GPZ_E_INVALID, "bc material index");
      m = &d.mats[im];
      GPZ_REQUIRE(d.bcs[ib].type == 0 || d.bcs[ib].type == 1, GPZ_E_UNSUPPORTED_MATERIAL, "bc type");
    } else {
      GPZ_REQUIRE(d.el_mat[e] < d.nmat, GPZ_E_INVALID, "material index");
      m = &d.mats[d.el_mat[e]];
    }
    k.mat_kind = m->kind;
    k.mat_index = d.el_mat[e];
    GPZ_REQUIRE(m->kind == GPZ_MAT_POISSON || m->kind == GPZ_MAT_DARCY || m->kind == GPZ_MAT_ELAST3D,
                GPZ_E_UNSUPPORTED_MATERIAL, "material kind");
    // IntegrationRuleOrder(MaxOrder): the largest order of the element's connects
    // (hp sides set by SetSideOrder re-run AdjustIntegrationRule,
    // Mesh/pzinterpolationspace.cpp:69-83); equal to the element's p when p is uniform
    int eorder[19];
    int p = 1;
    bool uniform = true;
    for (int s = t.ncorner; s < t.nsides; s++) {
      eorder[s - t.ncorner] = d.conn_order[d.el_conn[e * 27 + s]];
      p = std::max(p, eorder[s - t.ncorner]);
    }
    for (int s = t.ncorner; s < t.nsides; s++) uniform &= eorder[s - t.ncorner] == p;
    if (k.is_bc || m->kind == GPZ_MAT_ELAST3D) k.intorder = 2 * p;
    else k.intorder = (p < m->forcing_porder) ? m->forcing_porder + p : 2 * p;
    // uniform elements keep their own tables; an element of uneven side orders
    // joins the hp class of its largest order, whose table is the full element
    k.hp = uniform ? 0 : 1;
    for (int s = t.ncorner; s < t.nsides; s++) {
      int o = uniform ? eorder[s - t.ncorner] : p;
      k.orders[s - t.ncorner] = o;
      k.trans[s - t.ncorner] = side_nshape(k.type, s, o) > 1 ? side_orientation(k.type, s, &d.el_nodes[e * 8]) : 0;
    }
    if (!k.hp) {
      int n = t.ncorner;
      for (int s = t.ncorner; s < t.nsides; s++) n += side_nshape(k.type, s, k.orders[s - t.ncorner]);
      if (!select_kernel(k.type, n, c.nstate, k.is_bc).one) k.hp = 1;  // no compile-time kernel: same table, run-time path
    }
    if (k.hp) {
      // active shapes of this element among the class table's: corners, then per
      // side its order-o functions, found by their Chebyshev index tuple
      int n = 0;
      uint8_t *rf = &act_full[e * kMaxShapes], *rk = &act_k[e * kMaxShapes];
      std::fill(rf, rf + kMaxShapes, (uint8_t)0);
      std::fill(rk, rk + kMaxShapes, (uint8_t)0);
      for (int a = 0; a < t.ncorner; a++, n++) {
        rf[n] = (uint8_t)a;
        rk[n] = 0;
      }
      int tstart = t.ncorner;
      for (int s = t.ncorner; s < t.nsides; s++) {
        const int o = eorder[s - t.ncorner], sd = t.side_dim[s];
        const int ns = side_nshape(k.type, s, o), nsf = side_nshape(k.type, s, p);
        const int m = o - 1, mf = p - 1;
        for (int kk = 0; kk < ns; kk++, n++) {
          int full;
          if (sd == 1) full = kk;
          else if (sd == 2) full = (kk / m) * mf + kk % m;
          else full = ((kk / (m * m)) * mf + (kk / m) % m) * mf + kk % m;
          rf[n] = (uint8_t)(tstart + full);
          rk[n] = (uint8_t)kk;
        }
        tstart += nsf;
      }
      act_n[e] = n;
    }
  };
  // a new bucket's shape tables (quadrature, shapes and gradients per point, the reference Gram of volume hexes)
  auto make_bucket = [&](const BucketKey &k) {
    const ElemTopo &t = topo(k.type);
    Bucket *b = new Bucket();
    b->key = k;
    b->nsides = t.nsides;
    b->ncorner = t.ncorner;
    b->dim = t.dim;
    b->nstate = c.nstate;
    std::vector<double> pts;
    gauss_rule(k.type, k.intorder, pts, b->w);
    b->nq = (int)b->w.size();
    if (b->nq > kMaxQp) {
      delete b;
      throw Error{GPZ_E_UNSUPPORTED_ELEMENT, "too many integration points"};
    }
    double phi[kMaxShapes], dphi[3 * kMaxShapes];
    int so[kMaxShapes], sk[kMaxShapes];
    for (int q = 0; q < b->nq; q++) {
      int n = eval_shapes(k.type, k.orders, k.trans, &pts[q * t.dim], phi, dphi, kMaxShapes, so, sk);
      if (q == 0) {
        b->nshape = n;
        b->shape_side.assign(so, so + n);
        b->shape_k.assign(sk, sk + n);
        b->phi.resize((size_t)b->nq * n);
        b->dphi.resize((size_t)b->nq * t.dim * n);
      }
      for (int a = 0; a < n; a++) {
        b->phi[q * n + a] = phi[a];
        for (int dd = 0; dd < t.dim; dd++) b->dphi[(q * t.dim + dd) * n + a] = dphi[dd * kMaxShapes + a];
      }
    }
    b->ndof = b->nshape * c.nstate;
    if (k.type == GPZ_EL_HEX && !k.is_bc) {
      // compensated (Neumaier) double sums over the points, shape rows on the host threads (a software
      // long double, as on aarch64, is ~100x slower for the order-3 tables)
      const int nt = b->nshape;
      b->ghat.assign((size_t)nt * nt * 9, 0.0);
      host_parallel(nt, [&](int64_t a0, int64_t a1) {
        for (int64_t a = a0; a < a1; a++)
          for (int bb = 0; bb < nt; bb++)
            for (int i = 0; i < 3; i++)
              for (int j = 0; j < 3; j++) {
                double sum = 0.0, comp = 0.0;
                for (int q = 0; q < b->nq; q++) {
                  const double x = b->w[q] * b->dphi[(q * 3 + i) * nt + a] * b->dphi[(q * 3 + j) * nt + bb];
                  const double t = sum + x;
                  comp += std::fabs(sum) >= std::fabs(x) ? (sum - t) + x : (x - t) + sum;
                  sum = t;
                }
                b->ghat[((size_t)a * nt + bb) * 9 + i * 3 + j] = sum + comp;
              }
      }, 8);
    }
    b->hp = k.hp != 0;
    const bool ok = b->hp ? select_hp(k.type, c.nstate, k.is_bc).one != nullptr
                          : select_kernel(k.type, b->nshape, c.nstate, k.is_bc).one != nullptr;
    if (!ok) {
      delete b;
      throw Error{GPZ_E_UNSUPPORTED_ELEMENT, "no kernel for this element bucket"};
    }
    return b;
  };
  // keys in parallel over chunks of elements (each chunk's distinct keys in first-occurrence order), then
  // buckets created in the order of their first element, as one pass over the elements would
  const int64_t nchunk = std::max<int64_t>(1, std::min<int64_t>(256, c.nel / 4096));
  std::vector<std::map<BucketKey, int>> ckey(nchunk);
  std::vector<std::vector<const BucketKey *>> corder(nchunk);
  std::vector<int32_t> el_key(c.nel, 0);
  host_parallel(
      nchunk,
      [&](int64_t c0, int64_t c1) {
        BucketKey k;
        for (int64_t ch = c0; ch < c1; ch++) {
          const BucketKey *last = nullptr;
          int last_i = -1;
          for (int64_t e = c.nel * ch / nchunk; e < c.nel * (ch + 1) / nchunk; e++) {
            key_of(e, k);
            if (!last || *last < k || k < *last) {
              auto it = ckey[ch].find(k);
              if (it == ckey[ch].end()) {
                it = ckey[ch].emplace(k, (int)corder[ch].size()).first;
                corder[ch].push_back(&it->first);
              }
              last = &it->first;
              last_i = it->second;
            }
            el_key[e] = last_i;
          }
        }
      },
      1);
  std::map<BucketKey, int> index;
  std::vector<std::vector<int>> remap(nchunk);
  for (int64_t ch = 0; ch < nchunk; ch++)
    for (const BucketKey *k : corder[ch]) {
      auto it = index.find(*k);
      if (it == index.end()) {
        it = index.emplace(*k, (int)c.buckets.size()).first;
        c.buckets.push_back(make_bucket(*k));
      }
      remap[ch].push_back(it->second);
    }
  std::vector<int> el_bucket(c.nel, -1);
  host_parallel(nchunk, [&](int64_t c0, int64_t c1) {
    for (int64_t ch = c0; ch < c1; ch++)
      for (int64_t e = c.nel * ch / nchunk; e < c.nel * (ch + 1) / nchunk; e++) el_bucket[e] = remap[ch][el_key[e]];
  }, 1);
  const auto t1 = std::chrono::steady_clock::now();
  // greedy first-fit colouring by shared non-empty connects (gpz_element_colours)
  int nsides_of_type[4] = {0, topo(GPZ_EL_LINE).nsides, topo(GPZ_EL_QUAD).nsides, topo(GPZ_EL_HEX).nsides};
  std::vector<int32_t> colour(c.nel, 0);
  int32_t ncol = 0;
  const int crc = colour_mesh_elements(d, nsides_of_type, colour.data(), &ncol);
  GPZ_REQUIRE(crc == GPZ_OK, GPZ_E_INVALID, "element colouring: a connect out of range or more than 64 colours");
  c.ncolours = ncol;
  const auto t2 = std::chrono::steady_clock::now();
  for (Bucket *b : c.buckets) b->colour_begin.assign(ncol + 1, 0);
  for (int64_t e = 0; e < c.nel; e++) c.buckets[el_bucket[e]]->colour_begin[colour[e] + 1]++;
  for (Bucket *b : c.buckets) {
    for (int k = 0; k < ncol; k++) b->colour_begin[k + 1] += b->colour_begin[k];
    b->elems.assign(b->colour_begin[ncol], 0);
  }
  std::vector<std::vector<int64_t>> fillpos(c.buckets.size());
  for (size_t i = 0; i < c.buckets.size(); i++)
    fillpos[i].assign(c.buckets[i]->colour_begin.begin(), c.buckets[i]->colour_begin.end() - 1);
  for (int64_t e = 0; e < c.nel; e++) {
    int bi = el_bucket[e];
    c.buckets[bi]->elems[fillpos[bi][colour[e]]++] = e;
  }
  // per-element active shapes of the hp classes, in each class's element order
  for (Bucket *b : c.buckets) {
    if (!b->hp) continue;
    const size_t ne = b->elems.size();
    b->act_full.assign(ne * kMaxShapes, 0);
    b->act_k.assign(ne * kMaxShapes, 0);
    b->act_n.assign(ne, 0);
    for (size_t i = 0; i < ne; i++) {
      const int64_t e = b->elems[i];
      std::copy(&act_full[e * kMaxShapes], &act_full[e * kMaxShapes] + kMaxShapes, &b->act_full[i * kMaxShapes]);
      std::copy(&act_k[e * kMaxShapes], &act_k[e * kMaxShapes] + kMaxShapes, &b->act_k[i * kMaxShapes]);
      b->act_n[i] = act_n[e];
    }
    b->d_act_full.upload(b->act_full.data(), b->act_full.size(), c.stream);
    b->d_act_k.upload(b->act_k.data(), b->act_k.size(), c.stream);
    b->d_act_n.upload(b->act_n.data(), b->act_n.size(), c.stream);
  }
  for (Bucket *b : c.buckets) {
    b->d_phi.upload(b->phi.data(), b->phi.size(), c.stream);
    b->d_dphi.upload(b->dphi.data(), b->dphi.size(), c.stream);
    b->d_w.upload(b->w.data(), b->w.size(), c.stream);
    if (!b->ghat.empty()) b->d_ghat.upload(b->ghat.data(), b->ghat.size(), c.stream);
    b->d_shape_side.upload(b->shape_side.data(), b->shape_side.size(), c.stream);
    b->d_shape_k.upload(b->shape_k.data(), b->shape_k.size(), c.stream);
    b->d_elems.upload(b->elems.data(), b->elems.size(), c.stream);
    b->d_cbeg.upload(b->colour_begin.data(), b->colour_begin.size(), c.stream);
    b->d_q.alloc(2);
  }
  GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
  const auto t3 = std::chrono::steady_clock::now();
  auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
    return std::to_string(std::chrono::duration<double, std::milli>(b - a).count());
  };
  c.bucket_report = "{\"keys\": " + ms(t0, t1) + ", \"colouring\": " + ms(t1, t2) + ", \"lists_tables\": " +
                    ms(t2, t3) + "}";
}

namespace {

ElemArgs args_of(Ctx &c, const Bucket *b) {
  ElemArgs P{};
  P.phi = b->d_phi.p;
  P.dphi = b->d_dphi.p;
  P.w = b->d_w.p;
  P.ghat = b->d_ghat.p;
  P.sside = b->d_shape_side.p;
  P.sk = b->d_shape_k.p;
  P.nq = b->nq;
  P.ncorner = b->ncorner;
  P.nsides = b->nsides;
  P.nshape = b->nshape;
  P.xyz = c.d_xyz.p;
  P.el_nodes = c.d_el_nodes.p;
  P.el_conn = c.d_el_conn.p;
  P.bpos = c.d_block_pos.p;
  P.el_mat = c.d_el_mat.p;
  P.coef = c.d_coef.p;
  const int64_t e_any = b->elems[0];
  const int mi = c.h_el_mat[e_any];
  const gpz_material *m;
  if (mi < 0) {
    const gpz_bc &bc = c.bcs[-mi - 1];
    m = &c.mats[bc.material];
    P.bc_type = bc.type;
    for (int k = 0; k < 3; k++) P.val2[k] = bc.val2[k];
  } else {
    m = &c.mats[mi];
  }
  P.kind = m->kind;
  P.mdim = m->dim;
  P.forcing = m->forcing;
  P.scale = m->scale;
  P.E = m->E;
  P.nu = m->nu;
  P.coef_const = m->coef_const;
  P.big = m->kind == GPZ_MAT_ELAST3D ? 1.e12 : m->bignumber;  // TPZElasticity3D.cpp:632
  for (int k = 0; k < 3; k++) P.force[k] = m->force[k];
  const bool flt = c.flt.active;  // the element kernels fill the mesh-level CSR under a filter
  P.ia = flt ? c.flt.m_ia.p : c.d_ia.p;
  P.offbase = c.d_offbase.p;
  P.off = c.d_off.p;
  P.a = flt ? c.flt.m_a.p : c.d_a.p;
  P.f = c.d_f.p;
  P.nnz = flt ? c.flt.m_nnz : c.nnz;
  P.neq = c.neq_mesh;
  P.err = c.d_err.p;
  if (b->shared == 1) {
    P.kref = b->d_kref.p;
    P.fref = (m->forcing == GPZ_F_CONST || m->forcing == GPZ_F_NONE) ? b->d_fref.p : nullptr;
  }
  return P;
}

// 1 in *flag when an element of the list is not a translate of the first: its
// trilinear map has xi.eta, xi.zeta, eta.zeta or xi.eta.zeta terms, or its
// gradient (the xi, eta, zeta terms) differs from the first element's, by more
// than 1e-13 of the element's extent
__device__ __forceinline__ void hex_map_terms(const int64_t *__restrict__ el_nodes, const double *__restrict__ xyz,
                                              int64_t e, double (&t)[3][7], double &ext) {
  const signed char sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  ext = 0.0;
  for (int j = 0; j < 3; j++) {
    for (int d = 0; d < 7; d++) t[j][d] = 0.0;
    double mn = 1e300, mx = -1e300;
    for (int k = 0; k < 8; k++) {
      const double x = xyz[el_nodes[e * 8 + k] * 3 + j];
      const int a = sg[k][0], b = sg[k][1], c = sg[k][2];
      t[j][0] += a * x;
      t[j][1] += b * x;
      t[j][2] += c * x;
      t[j][3] += a * b * x;
      t[j][4] += a * c * x;
      t[j][5] += b * c * x;
      t[j][6] += a * b * c * x;
      mn = fmin(mn, x);
      mx = fmax(mx, x);
    }
    ext = fmax(ext, mx - mn);
  }
}

__global__ void k_translates(const int64_t *__restrict__ elems, int64_t n, const int64_t *__restrict__ el_nodes,
                             const double *__restrict__ xyz, int *__restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double t0[3][7], t[3][7], ext0, ext;
  hex_map_terms(el_nodes, xyz, elems[0], t0, ext0);
  hex_map_terms(el_nodes, xyz, elems[i], t, ext);
  const double tol = 1e-13 * ext;
  bool ok = ext > 0.0;
  for (int j = 0; j < 3; j++) {
    for (int d = 0; d < 3; d++) ok = ok && fabs(t[j][d] - t0[j][d]) <= tol;
    for (int d = 3; d < 7; d++) ok = ok && fabs(t[j][d]) <= tol;
  }
  if (!ok) atomicOr(flag, 1);
}

// ---- row-owner assembly of a shared-matrix bucket.  With K_e = c_e kref the
// matrix rows of one unit (the nstate equations of one shape of one connect)
// are sums over the unit's incidences (element e, shape a) of c_e times row a
// of kref: one warp per unit adds them in shared memory, column block by
// column block through the element's slot-offset table, and writes the rows
// once, whole and coalesced.  The coloured scatter instead reads and writes
// every row once per colour of the elements around it, and the rows (10 GB
// for 64^3 Q2 elasticity) do not stay in L2 between colours.  The products
// are those of the scatter (kref is symmetric, so row b of the transposed
// block is row b of kref) with the same |K| >= 1e-12 rule; only the order of
// the sums over a unit's elements differs.  The load vector stays with the
// element kernels (their load-vector-only mode), so that it keeps the order of
// TPZStructMatrix::Assemble(rhs).
constexpr int kRpMaxInc = 64;

__global__ void k_rp_incidences(int pass, const int64_t *__restrict__ elems, int64_t ne, int nsh,
                                const int *__restrict__ sside, const int *__restrict__ sk,
                                const int64_t *__restrict__ el_conn, const int64_t *__restrict__ bpos, int nst,
                                int64_t nunits, unsigned long long *__restrict__ cnt,
                                const int64_t *__restrict__ ptr, int64_t *__restrict__ inc, int *__restrict__ bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ne * nsh; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ie = i / nsh;
    const int a = (int)(i - ie * nsh);
    const int64_t row = bpos[el_conn[elems[ie] * 27 + sside[a]]] + (int64_t)sk[a] * nst;
    const int64_t u = row / nst;
    if (row < 0 || row % nst != 0 || u >= nunits) {
      atomicOr(bad, 1);
      continue;
    }
    const unsigned long long k = atomicAdd(cnt + u, 1ull);
    if (pass == 1) inc[ptr[u] + (int64_t)k] = (ie << 8) | a;
  }
}

// each unit's incidences in increasing order (a fixed order of the sums)
__global__ void k_rp_sort(const int64_t *__restrict__ ptr, int64_t nunits, int64_t *__restrict__ inc,
                          int *__restrict__ bad) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p0 = ptr[u], n = ptr[u + 1] - p0;
    if (n > kRpMaxInc) {
      atomicOr(bad, 2);
      continue;
    }
    for (int64_t i = 1; i < n; i++) {
      const int64_t v = inc[p0 + i];
      int64_t j = i - 1;
      while (j >= 0 && inc[p0 + j] > v) {
        inc[p0 + j + 1] = inc[p0 + j];
        j--;
      }
      inc[p0 + j + 1] = v;
    }
  }
}

// the longest row of the units, units without incidences, units whose rows differ in length
__global__ void k_rp_rows(const int64_t *__restrict__ ptr, int64_t nunits, const int64_t *__restrict__ ia, int nst,
                          int *__restrict__ out /* lmax, empty, uneven */) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    if (ptr[u + 1] == ptr[u]) {
      atomicOr(out + 1, 1);
      continue;
    }
    const int64_t L = ia[u * nst + 1] - ia[u * nst];
    for (int s = 1; s < nst; s++)
      if (ia[u * nst + s + 1] - ia[u * nst + s] != L) atomicOr(out + 2, 1);
    atomicMax(out, L < (1 << 30) ? (int)L : (1 << 30));
  }
}

// An incidence as the row pass reads it, one 16-byte load: the element's row
// of slot offsets for the shape's side (offbase[e] + side * nsides), the
// element (its coefficient is read at run time) and the shape.
struct RpRec {
  int64_t orow;
  int32_t e, a;
};

__global__ void k_rp_records(const int64_t *__restrict__ inc, int64_t n, const int64_t *__restrict__ elems,
                             const int64_t *__restrict__ offbase, const int *__restrict__ sside, int ns,
                             RpRec *__restrict__ rec) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t code = inc[i];
    const int64_t e = elems[code >> 8];
    const int a = (int)(code & 255);
    rec[i] = RpRec{offbase[e] + (int64_t)sside[a] * ns, (int32_t)e, a};
  }
}

// Before each row pass: the range of |c_e| over the bucket, and kref with the
// entries that the |c_e kref| >= 1e-12 rule drops for every c_e in that range
// set to zero (kp).  amb = 1 when some entry is kept for part of the range
// only; the row pass then applies the rule product by product.
// GB300's FP64 rate bounds the row pass: without the test each kept entry
// costs one multiply and one add (Q2 elasticity: 942 of kref's 6561 entries
// are rounding-level and are dropped whatever the coefficient).
// rng[0], rng[1]: the bit patterns of min and max |c_e| (non-negative doubles
// order as their bits), set beforehand to a huge value and to 0
__global__ void __launch_bounds__(256) k_rp_range(ElemArgs P, const int64_t *__restrict__ elems, int64_t ne,
                                                  unsigned long long *__restrict__ rng) {
  double lo = 1e300, hi = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ne; i += (int64_t)gridDim.x * blockDim.x) {
    double cf = P.kind == GPZ_MAT_ELAST3D ? P.E : P.coef_const;
    if (P.coef) cf = P.coef[elems[i]];
    const double cs = fabs(P.kind == GPZ_MAT_POISSON ? 1.0 : cf);
    lo = fmin(lo, cs);
    hi = fmax(hi, cs);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(rng, (unsigned long long)__double_as_longlong(lo));
    atomicMax(rng + 1, (unsigned long long)__double_as_longlong(hi));
  }
}

__global__ void k_rp_prune(const double *__restrict__ kref, int n, const unsigned long long *__restrict__ rng,
                           double *__restrict__ kp, int *__restrict__ amb) {
  const double lo = __longlong_as_double((long long)rng[0]), hi = __longlong_as_double((long long)rng[1]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double k = kref[i], ak = fabs(k);
    // margins of 1e-12 relative cover the rounding of the product and of these tests
    const bool never = ak * hi * (1.0 + 1e-12) < 1e-12, always = ak * lo * (1.0 - 1e-12) >= 1e-12;
    kp[i] = never ? 0.0 : k;
    if (!never && !always) atomicOr(amb, 1);
  }
}

// One warp per unit, persistent; the next unit's bounds and row start are
// loaded while the current one runs.  A unit's incidences go in chunks of up
// to 8: lanes 0..7 load a chunk's records and coefficients at once and shuffle
// them to the warp, every lane issues the chunk's offset loads for its column
// shapes together, and the additions run incidence by incidence with a warp
// barrier between them (two elements' shapes may share a column), each
// block's nine old values read before its nine stores.  The rows of a unit
// are consecutive and of equal length, so row s starts at ia[u NST] + s L.
// kref sits in shared memory when it fits (kref_sh).
template <int NST>
__global__ void __launch_bounds__(512) k_rowpass(ElemArgs P, const int64_t *__restrict__ ptr,
                                                 const RpRec *__restrict__ rec, const double *__restrict__ kp,
                                                 const int *__restrict__ amb_p, int64_t nunits, int lmax,
                                                 int kref_sh) {
  extern __shared__ double rp_sm[];
  const int nsh = P.nshape, nd = nsh * NST;
  const double *kref = kp;
  double *acc_base = rp_sm;
  if (kref_sh) {
    for (int i = threadIdx.x; i < nd * nd; i += blockDim.x) rp_sm[i] = kp[i];
    kref = rp_sm;
    acc_base = rp_sm + nd * nd;
    __syncthreads();
  }
  const bool amb = *amb_p != 0;
  const long long kTiny = __double_as_longlong(1.e-12);
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double *acc = acc_base + (size_t)wid * NST * lmax;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + wid;
  int64_t np0 = 0, np1 = 0, nrb = 0, nre = 0;
  if (u < nunits) {
    np0 = ptr[u];
    np1 = ptr[u + 1];
    nrb = P.ia[u * NST];
    nre = P.ia[u * NST + 1];
  }
  for (; u < nunits; u += nw) {
    const int64_t p0 = np0, p1 = np1, rb = nrb;
    const int L = (int)(nre - nrb);
    if (u + nw < nunits) {
      np0 = ptr[u + nw];
      np1 = ptr[u + nw + 1];
      nrb = P.ia[(u + nw) * NST];
      nre = P.ia[(u + nw) * NST + 1];
    }
    if (p0 == p1) continue;
    if (L > lmax) {  // the host sized the accumulators from these rows
      if (lane == 0) atomicOr(P.err, 64);
      continue;
    }
    for (int j = lane; j < NST * L; j += 32) acc[j] = 0.0;
    __syncwarp();
    for (int64_t pc = p0; pc < p1; pc += 8) {
      const int m = (int)(p1 - pc < 8 ? p1 - pc : 8);
      int a_l = 0;
      int64_t ob_l = 0;
      double cs_l = 0.0;
      if (lane < m) {
        const RpRec r = rec[pc + lane];
        a_l = r.a;
        ob_l = r.orow;
        double cf = P.kind == GPZ_MAT_ELAST3D ? P.E : P.coef_const;
        if (P.coef) cf = P.coef[r.e];
        cs_l = P.kind == GPZ_MAT_POISSON ? 1.0 : cf;
      }
      int64_t obj[8];
#pragma unroll
      for (int j = 0; j < 8; j++) obj[j] = __shfl_sync(FULL, ob_l, j);
      for (int bb = 0; bb < nsh; bb += 32) {
        const int b = bb + lane;
        const bool act = b < nsh;
        const int sb = act ? P.sside[b] : 0, kb = act ? P.sk[b] * NST : 0;
        int32_t ofs[8];
#pragma unroll
        for (int j = 0; j < 8; j++) ofs[j] = (act && j < m) ? P.off[obj[j] + sb] : 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int aj = __shfl_sync(FULL, a_l, j);
          const double csj = __shfl_sync(FULL, cs_l, j);
          const bool first = j == 0 && pc == p0;  // the unit's first incidence: 0 + v is v, a store
          if (j < m && act) {
            const int o = ofs[j] + kb;
            if (ofs[j] < 0 || o + NST > L) {
              atomicOr(P.err, 32);
            } else {
              const double *kr = kref + (size_t)(aj * NST) * nd + b * NST;
              double k[NST][NST], old[NST][NST];
#pragma unroll
              for (int s = 0; s < NST; s++)
#pragma unroll
                for (int t = 0; t < NST; t++) {
                  k[s][t] = kr[s * nd + t];
                  old[s][t] = acc[s * L + o + t];
                }
              if (!amb) {  // kept entries pass the rule for every coefficient of the bucket: no test;
                           // product and sum rounded apart (never fused), as the scatter forms them
#pragma unroll
                for (int s = 0; s < NST; s++)
#pragma unroll
                  for (int t = 0; t < NST; t++)
                    if (__double_as_longlong(k[s][t]) << 1) {
                      const double v = __dmul_rn(csj, k[s][t]);
                      acc[s * L + o + t] = first ? v : __dadd_rn(old[s][t], v);
                    }
              } else {  // the rule per product, compared on the bits (|v| >= 1e-12 for finite v)
#pragma unroll
                for (int s = 0; s < NST; s++)
#pragma unroll
                  for (int t = 0; t < NST; t++) {
                    const double v = __dmul_rn(csj, k[s][t]);
                    if ((__double_as_longlong(v) & 0x7fffffffffffffffLL) >= kTiny)
                      acc[s * L + o + t] = first ? v : __dadd_rn(old[s][t], v);
                  }
              }
            }
          }
          __syncwarp();
        }
      }
    }
#pragma unroll
    for (int s = 0; s < NST; s++) {
      double *dst = P.a + rb + (int64_t)s * L;
      for (int j = lane; j < L; j += 32) dst[j] = acc[s * L + j];
    }
    __syncwarp();
  }
}

constexpr int kRpSmem = 220 * 1024;

// Incidence lists of the largest shared-matrix bucket (mesh-dependent, built
// once), then, for the current pattern, its longest row and whether its units
// cover every equation.  Leaves c.rp_bucket null when no bucket qualifies.
void rowpass_prepare(Ctx &c) {
  cudaStream_t s = c.stream;
  c.rp_bucket = nullptr;
  const int nst = c.nstate;
  if (c.flt.active || (nst != 1 && nst != 3) || c.neq_mesh % nst != 0) return;
  Bucket *best = nullptr;
  for (Bucket *b : c.buckets)
    if (b->shared == 1 && b->rowpass != 0 && b->nshape <= 64 && (!best || b->elems.size() > best->elems.size()))
      best = b;
  if (!best) return;
  Bucket *b = best;
  const int64_t nunits = c.neq_mesh / nst, ne = (int64_t)b->elems.size();
  DBuf<int> flags;
  flags.alloc(4);
  if (b->rowpass < 0) {
    DBuf<unsigned long long> cnt;
    cnt.alloc(nunits + 1);
    cnt.zero(s);
    flags.zero(s);
    const unsigned g = (unsigned)std::min<int64_t>(grid_for(ne * b->nshape, 256), 152 * 16);
    k_rp_incidences<<<g, 256, 0, s>>>(0, b->d_elems.p, ne, b->nshape, b->d_shape_side.p, b->d_shape_k.p,
                                      c.d_el_conn.p, c.d_block_pos.p, nst, nunits, cnt.p, nullptr, nullptr, flags.p);
    c.launches++;
    b->d_rp_ptr.alloc(nunits + 1);
    exclusive_scan_i64((const int64_t *)cnt.p, b->d_rp_ptr.p, nunits + 1, s, c);
    b->d_rp_inc.alloc(std::max<int64_t>(ne * b->nshape, 1));
    cnt.zero(s);
    k_rp_incidences<<<g, 256, 0, s>>>(1, b->d_elems.p, ne, b->nshape, b->d_shape_side.p, b->d_shape_k.p,
                                      c.d_el_conn.p, c.d_block_pos.p, nst, nunits, cnt.p, b->d_rp_ptr.p,
                                      b->d_rp_inc.p, flags.p);
    c.launches++;
    k_rp_sort<<<grid_for(nunits, 256), 256, 0, s>>>(b->d_rp_ptr.p, nunits, b->d_rp_inc.p, flags.p);
    c.launches++;
    GPZ_CUDA_TRY(cudaGetLastError());
    int h = 0;
    GPZ_CUDA_TRY(cudaMemcpyAsync(&h, flags.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));
    b->rowpass = h ? 0 : 1;
    if (!b->rowpass) {
      b->d_rp_ptr.release();
      b->d_rp_inc.release();
      return;
    }
  }
  const int64_t ninc = ne * b->nshape;
  b->d_rp_rec.alloc(std::max<int64_t>(ninc, 1) * 2);  // RpRec, 16 bytes each
  const int64_t ndk = (int64_t)b->nshape * nst;
  b->d_rp_kp.alloc(ndk * ndk + 3);  // the pruned kref, then the |c_e| range and the flag amb
  k_rp_records<<<grid_for(ninc, 256), 256, 0, s>>>(b->d_rp_inc.p, ninc, b->d_elems.p, c.d_offbase.p,
                                                    b->d_shape_side.p, b->nsides, (RpRec *)b->d_rp_rec.p);
  c.launches++;
  flags.zero(s);
  k_rp_rows<<<grid_for(nunits, 256), 256, 0, s>>>(b->d_rp_ptr.p, nunits, c.d_ia.p, nst, flags.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  int h[3] = {0, 0, 0};
  GPZ_CUDA_TRY(cudaMemcpyAsync(h, flags.p, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  const int64_t per_warp = (int64_t)nst * h[0] * (int64_t)sizeof(double);
  const int64_t nd = (int64_t)b->nshape * nst, kref_bytes = nd * nd * (int64_t)sizeof(double);
  const bool kref_sh = kref_bytes <= 64 * 1024 && kref_bytes + per_warp <= kRpSmem;
  const int64_t room = kRpSmem - (kref_sh ? kref_bytes : 0);
  if (h[2] || h[0] <= 0 || per_warp > room) return;
  const int warps = (int)std::min<int64_t>(16, room / per_warp);
  const size_t sh = (size_t)warps * per_warp + (kref_sh ? (size_t)kref_bytes : 0);
  auto k = nst == 3 ? k_rowpass<3> : k_rowpass<1>;
  GPZ_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
  int dev = 0, nsm = 0, per = 0;
  GPZ_CUDA_TRY(cudaGetDevice(&dev));
  GPZ_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  GPZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, warps * 32, sh));
  c.rp_lmax = h[0];
  c.rp_warps = warps;
  c.rp_kref_sh = kref_sh ? 1 : 0;
  c.rp_smem = (int)sh;
  c.rp_grid = std::max(1, per) * std::max(1, nsm);
  c.rp_full = h[1] == 0;
  c.rp_bucket = b;
}

void launch_rowpass(Ctx &c) {
  Bucket *b = c.rp_bucket;
  const ElemArgs P = args_of(c, b);
  const int64_t nunits = c.neq_mesh / c.nstate;
  const size_t sh = (size_t)c.rp_smem;
  const RpRec *rec = (const RpRec *)b->d_rp_rec.p;
  const int nd = b->nshape * c.nstate;
  double *kp = b->d_rp_kp.p;
  unsigned long long *rng = (unsigned long long *)(kp + (size_t)nd * nd);
  int *amb = (int *)(rng + 2);
  const int64_t ne = (int64_t)b->elems.size();
  GPZ_CUDA_TRY(cudaMemsetAsync(rng, 0x7f, sizeof(unsigned long long), c.stream));  // about 1.4e306
  GPZ_CUDA_TRY(cudaMemsetAsync(rng + 1, 0, sizeof(unsigned long long) + sizeof(int), c.stream));
  k_rp_range<<<(unsigned)std::min<int64_t>(grid_for(ne, 256), 152 * 4), 256, 0, c.stream>>>(P, b->d_elems.p, ne, rng);
  k_rp_prune<<<grid_for((int64_t)nd * nd, 256), 256, 0, c.stream>>>(P.kref, nd * nd, rng, kp, amb);
  c.launches += 2;
  if (c.nstate == 3)
    k_rowpass<3><<<c.rp_grid, c.rp_warps * 32, sh, c.stream>>>(P, b->d_rp_ptr.p, rec, kp, amb, nunits,
                                                                c.rp_lmax, c.rp_kref_sh);
  else
    k_rowpass<1><<<c.rp_grid, c.rp_warps * 32, sh, c.stream>>>(P, b->d_rp_ptr.p, rec, kp, amb, nunits,
                                                                c.rp_lmax, c.rp_kref_sh);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
}

// element integration + scatter of every bucket, colour by colour; the hp
// classes run with `threads` (0: the class's tuned block size).  queue: one
// persistent launch per bucket over all its colours instead (k_elem_fp64_queue).
void launch_elements(Ctx &c, int threads, bool rhs_only = false, bool set_attrs = true, bool queue = false) {
  cudaStream_t s = c.stream;
  if (queue) {
    int dev = 0, nsm = 0;
    if (set_attrs) {
      GPZ_CUDA_TRY(cudaGetDevice(&dev));
      GPZ_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    }
    for (Bucket *b : c.buckets) {
      const int64_t ne = (int64_t)b->elems.size();
      if (!ne) continue;
      ElemArgs P = args_of(c, b);
      P.rhs_only = rhs_only ? 1 : 0;
      if (b == c.rp_bucket) P.rhs_only = 1;  // the matrix came from k_rowpass
      const size_t sh = smem_bytes(b->nshape, b->dim, b->nq, b->key.is_bc);
      const Kernels K = b->hp ? select_hp(b->key.type, c.nstate, b->key.is_bc)
                              : select_kernel(b->key.type, b->nshape, c.nstate, b->key.is_bc);
      HpArgs H{nullptr, nullptr, nullptr};
      int nt = 128;
      if (b->hp) {
        H.full = b->d_act_full.p;
        H.k = b->d_act_k.p;
        H.n = b->d_act_n.p;
        nt = threads > 0 ? threads : b->threads;
      }
      if (set_attrs) {  // resident CTAs for this block size (kept for the captured replays)
        if (sh > 48 * 1024)
          GPZ_CUDA_TRY(cudaFuncSetAttribute(K.queue, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
        int per = 0;
        GPZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, K.queue, nt, sh));
        b->qgrid = (int)std::max<int64_t>(1, std::min<int64_t>(ne, (int64_t)std::max(per, 1) * nsm));
      }
      b->d_q.zero(s);
      const QueueArgs Q{b->d_q.p, b->d_q.p + 1, b->d_cbeg.p, c.ncolours};
      K.queue<<<b->qgrid, nt, sh, s>>>(P, H, b->d_elems.p, ne, Q);
      c.launches++;
      GPZ_CUDA_TRY(cudaGetLastError());
    }
    return;
  }
  for (int col = 0; col < c.ncolours; col++) {
    for (Bucket *b : c.buckets) {
      int64_t e0 = b->colour_begin[col], e1 = b->colour_begin[col + 1];
      if (e1 == e0) continue;
      ElemArgs P = args_of(c, b);
      P.rhs_only = rhs_only ? 1 : 0;
      if (b == c.rp_bucket) P.rhs_only = 1;
      size_t sh = smem_bytes(b->nshape, b->dim, b->nq, b->key.is_bc);
      ElemKernel k;
      HpArgs H{nullptr, nullptr, nullptr};
      int nt = 128;
      if (b->hp) {
        k = select_hp(b->key.type, c.nstate, b->key.is_bc).one;
        H.full = b->d_act_full.p + e0 * kMaxShapes;
        H.k = b->d_act_k.p + e0 * kMaxShapes;
        H.n = b->d_act_n.p + e0;
        nt = threads > 0 ? threads : b->threads;
      } else {
        k = select_kernel(b->key.type, b->nshape, c.nstate, b->key.is_bc).one;
      }
      if (sh > 48 * 1024 && set_attrs)
        GPZ_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
      k<<<(unsigned)(e1 - e0), nt, sh, s>>>(P, H, b->d_elems.p + e0, e1 - e0);
      c.launches++;
      GPZ_CUDA_TRY(cudaGetLastError());
    }
  }
}

// Shared element matrices: a volume hex bucket (not an hp class) whose elements
// are all translates of its first element gets that element's matrix at
// coefficient 1 (kref) and its load vector (fref), computed once by the element
// kernel in its dense mode; the bucket's assembly then scales kref by each
// element's coefficient (K is linear in E, k; TPZElasticity3D's C1, C2, C3 are
// proportional to E) instead of integrating it, and takes fref as the load
// vector when the forcing is constant.
void shared_setup(Ctx &c) {
  cudaStream_t s = c.stream;
  for (Bucket *b : c.buckets) {
    if (b->shared >= 0) continue;
    b->shared = 0;
    if (b->hp || b->key.is_bc || b->key.type != GPZ_EL_HEX || b->elems.empty()) continue;
    const int64_t n = (int64_t)b->elems.size();
    DBuf<int> flag;
    flag.alloc(1);
    flag.zero(s);
    k_translates<<<grid_for(n, 256), 256, 0, s>>>(b->d_elems.p, n, c.d_el_nodes.p, c.d_xyz.p, flag.p);
    c.launches++;
    int h = 1;
    GPZ_CUDA_TRY(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));
    if (h) continue;
    const int nd = b->nshape * c.nstate;
    b->d_kref.alloc((size_t)nd * nd);
    b->d_fref.alloc((size_t)nd);
    ElemArgs P = args_of(c, b);
    P.kdense = b->d_kref.p;
    P.fdense = b->d_fref.p;
    const size_t sh = smem_bytes(b->nshape, b->dim, b->nq, false);
    ElemKernel k = select_kernel(b->key.type, b->nshape, c.nstate, false).one;
    if (sh > 48 * 1024) GPZ_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
    HpArgs H{nullptr, nullptr, nullptr};
    k<<<1, 128, sh, s>>>(P, H, b->d_elems.p, 1);
    c.launches++;
    GPZ_CUDA_TRY(cudaGetLastError());
    check_device_flag(c, "reference element matrix");
    b->shared = 1;
  }
}

}  // namespace

void assemble_fp64(Ctx &c) {
  cudaStream_t s = c.stream;
  shared_setup(c);
  if (!c.asm_graph) rowpass_prepare(c);  // a new pattern (or the first assembly)
  const bool flt = c.flt.active;
  c.d_a.alloc(std::max<int64_t>(c.nnz, 1));
  if (flt) c.flt.m_a.alloc(std::max<int64_t>(c.flt.m_nnz, 1));
  DBuf<double> &target = flt ? c.flt.m_a : c.d_a;
  c.d_f.alloc(std::max<int64_t>(c.neq_mesh, 1));
  // autotuner of the hp classes' run-time kernel: time one full assembly per
  // block size (the values do not depend on it: one CTA per element, fixed
  // summation order) and keep the fastest
  bool tune = false;
  for (Bucket *b : c.buckets) tune |= b->hp && !b->tuned;
  std::string key;
  if (tune && !c.tune_cache.empty()) {
    key = tune_key(c, "hp_block");
    const int cached = tune_cache_lookup(c, key);
    if (cached > 0) {  // a block size stored by an earlier run on this device and mesh
      for (Bucket *b : c.buckets)
        if (b->hp) {
          b->threads = cached;
          b->tuned = true;
        }
      c.asm_tune_report = "{\"cached\": true, \"chosen\": " + std::to_string(cached) + "}";
      tune = false;
    }
  }
  if (tune) {
    const int cand[3] = {64, 128, 256};
    float best = 1e30f;
    int best_t = 128;
    std::string rep = "{";
    cudaEvent_t e0, e1;
    GPZ_CUDA_TRY(cudaEventCreate(&e0));
    GPZ_CUDA_TRY(cudaEventCreate(&e1));
    for (int i = 0; i < 3; i++) {
      if (!c.rp_bucket || !c.rp_full) target.zero(s);
      c.d_f.zero(s);
      GPZ_CUDA_TRY(cudaEventRecord(e0, s));
      launch_elements(c, cand[i]);
      GPZ_CUDA_TRY(cudaEventRecord(e1, s));
      GPZ_CUDA_TRY(cudaEventSynchronize(e1));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      rep += (i ? ", \"" : "\"") + std::to_string(cand[i]) + "\": " + std::to_string(ms);
      if (ms < best) {
        best = ms;
        best_t = cand[i];
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (Bucket *b : c.buckets)
      if (b->hp) {
        b->threads = best_t;
        b->tuned = true;
      }
    c.asm_tune_report = rep + ", \"chosen\": " + std::to_string(best_t) + "}";
    if (!key.empty()) tune_cache_store(c, key, best_t, c.asm_tune_report);
  }
  // launch mode: a launch per bucket and colour, or one persistent launch per bucket over all its colours
  // (the work-counter kernel); one full assembly timed in each after a warm-up, the faster kept.  The
  // element kernel and the order of the contributions within a bucket are the same; across buckets the
  // persistent mode adds one bucket after the other, so the sums agree to the last bits only.
  if (c.asm_queue < 0) {
    std::string key;
    int cached = -1;
    if (!c.tune_cache.empty()) {
      key = tune_key(c, "asm_mode");
      cached = tune_cache_lookup(c, key);
    }
    if (cached >= 0) {
      c.asm_queue = cached;
      c.asm_mode_report = std::string("{\"cached\": true, \"chosen\": \"") +
                          (cached ? "persistent" : "per_colour") + "\"}";
    } else {
      cudaEvent_t e0, e1;
      GPZ_CUDA_TRY(cudaEventCreate(&e0));
      GPZ_CUDA_TRY(cudaEventCreate(&e1));
      float ms[2] = {0.f, 0.f};
      for (int q = 0; q < 2; q++)
        for (int rep = 0; rep < 2; rep++) {
          if (!c.rp_bucket || !c.rp_full) target.zero(s);  // timing only: a covering row pass rewrites every row
          c.d_f.zero(s);
          GPZ_CUDA_TRY(cudaEventRecord(e0, s));
          launch_elements(c, 0, false, true, q == 1);
          GPZ_CUDA_TRY(cudaEventRecord(e1, s));
          GPZ_CUDA_TRY(cudaEventSynchronize(e1));
          cudaEventElapsedTime(&ms[q], e0, e1);
        }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      check_device_flag(c, "element assembly launch modes");
      c.asm_queue = ms[1] < ms[0] ? 1 : 0;
      c.asm_mode_report = "{\"per_colour\": " + std::to_string(ms[0]) + ", \"persistent\": " +
                          std::to_string(ms[1]) + ", \"chosen\": \"" +
                          (c.asm_queue ? "persistent" : "per_colour") + "\"}";
      if (!key.empty()) tune_cache_store(c, key, c.asm_queue, c.asm_mode_report);
    }
  }
  c.d_dinv.alloc(std::max<int64_t>(c.neq, 1));
  auto body = [&](bool set_attrs) {
    if (!c.rp_bucket || !c.rp_full) target.zero(s);
    c.d_f.zero(s);
    if (c.rp_bucket) launch_rowpass(c);
    launch_elements(c, 0, false, set_attrs, c.asm_queue == 1);
    if (flt) {
      filter_values(c);
      filter_zero_inactive(c, c.d_f.p);
    }
    k_extract_diag<<<grid_for(c.neq, 256), 256, 0, s>>>(c.d_a.p, c.d_diagpos.p, c.neq, c.d_dinv.p);
    c.launches++;
    GPZ_CUDA_TRY(cudaGetLastError());
  };
  if (c.asm_graph) {
    // same pattern and buffers: replay the captured assembly
    GPZ_CUDA_TRY(cudaGraphLaunch(c.asm_graph, s));
    c.launches += c.asm_graph_launches;
  } else {
    // first assembly of this pattern runs eagerly (kernel attributes set, hp
    // block sizes tuned); its launch sequence is then captured for the next ones
    body(true);
    const int64_t l0 = c.launches;
    cudaGraph_t g;
    GPZ_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    body(false);
    GPZ_CUDA_TRY(cudaStreamEndCapture(s, &g));
    c.asm_graph_launches = c.launches - l0;
    c.launches = l0;
    GPZ_CUDA_TRY(cudaGraphInstantiate(&c.asm_graph, g, 0));
    GPZ_CUDA_TRY(cudaGraphDestroy(g));
  }
  GPZ_CUDA_TRY(cudaGetLastError());
  c.have_a32 = false;
  c.a32_tensor = false;
  c.have_bjinv = false;
  c.have_vbinv = false;
  c.tl.have_inv = false;
}

// load vector alone (TPZStructMatrix::Assemble(rhs), StrMatrix/pzstrmatrixor.cpp:75-103):
// the same element kernels, stopped before the element matrix
void assemble_rhs(Ctx &c) {
  shared_setup(c);
  c.d_f.alloc(std::max<int64_t>(c.neq_mesh, 1));
  c.d_f.zero(c.stream);
  launch_elements(c, 0, true, true, c.asm_queue == 1);
  if (c.flt.active) filter_zero_inactive(c, c.d_f.p);
}

void to_fp32(Ctx &c) {
  k_to_fp32<<<152 * 8, 256, 0, c.stream>>>(c.d_a.p, c.d_a32.p, c.nnz);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
}

// The FP32 element pass of the mixed assembly: every element's matrix formed
// again in FP32 and added into the FP32 full CSR d_a32, colour by colour -- the
// volume hexes as 3xTF32 tcgen05 products (gpz_elem_tc.cu), the other element
// types (penalty faces, 2D quads) by the FP64 element kernel with an FP32
// scatter.  The FP32 operator of the mixed solves is then built from these
// values instead of rounding the FP64 matrix.
void assemble_fp32_elements(Ctx &c) {
  cudaStream_t s = c.stream;
  c.d_a32.alloc(std::max<int64_t>(c.nnz, 1));
  cudaEvent_t e0, e1;
  GPZ_CUDA_TRY(cudaEventCreate(&e0));
  GPZ_CUDA_TRY(cudaEventCreate(&e1));
  GPZ_CUDA_TRY(cudaEventRecord(e0, s));
  c.d_a32.zero(s);
  int64_t ntc = 0, ncc = 0;
  for (int col = 0; col < c.ncolours; col++) {
    for (Bucket *b : c.buckets) {
      const int64_t b0 = b->colour_begin[col], b1 = b->colour_begin[col + 1];
      if (b1 == b0) continue;
      if (elem_tc_supported(c, b)) {
        elem_tc_launch(c, b, b0, b1, s);
        ntc += b1 - b0;
        continue;
      }
      const ElemKernel k = select_f32(b->key.type, b->nshape, c.nstate, b->key.is_bc, b->hp);
      GPZ_REQUIRE(k != nullptr, GPZ_E_UNSUPPORTED_ELEMENT, "no FP32 element kernel for this bucket");
      ElemArgs P = args_of(c, b);
      P.kref = P.fref = nullptr;
      P.a32 = c.d_a32.p;
      const size_t sh = smem_bytes(b->nshape, b->dim, b->nq, b->key.is_bc);
      HpArgs H{nullptr, nullptr, nullptr};
      int nt = 128;
      if (b->hp) {
        H.full = b->d_act_full.p + b0 * kMaxShapes;
        H.k = b->d_act_k.p + b0 * kMaxShapes;
        H.n = b->d_act_n.p + b0;
        nt = b->threads;
      }
      if (sh > 48 * 1024) GPZ_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
      k<<<(unsigned)(b1 - b0), nt, sh, s>>>(P, H, b->d_elems.p + b0, b1 - b0);
      c.launches++;
      GPZ_CUDA_TRY(cudaGetLastError());
      ncc += b1 - b0;
    }
  }
  GPZ_CUDA_TRY(cudaEventRecord(e1, s));
  GPZ_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  check_device_flag(c, "FP32 element matrices");
  c.a32_tensor = true;
  std::string per;
  for (const Bucket *b : c.buckets)
    if (b->tc_per_sm > 0)
      per += std::string(per.empty() ? "" : ", ") + "\"" + std::to_string(b->nshape) + (b->hp ? "_hp" : "") +
             "\": " + std::to_string(b->tc_per_sm);
  c.fp32_report = "{\"source\": \"element_matrices_fp32\", \"tensor_core_elements\": " + std::to_string(ntc) +
                  ", \"cuda_core_elements\": " + std::to_string(ncc) + ", \"ms\": " + std::to_string(ms) +
                  ", \"ctas_per_sm\": {" + per + "}}";
}

}  // namespace gpz
