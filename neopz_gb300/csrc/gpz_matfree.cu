// Matrix-free FP32 operator of 3D elasticity for the mixed CG's inner SpMV.
//
// q = A p is evaluated element by element instead of from stored 3x3 blocks:
// for every volume element (TPZElasticity3D, Material/Elasticity/TPZElasticity3D.cpp:269-400,
// whose element matrix is K_st(a,b) = mu delta_st grad(phi_a).grad(phi_b)
// + mu d_t phi_a d_s phi_b + lambda d_s phi_a d_t phi_b, lambda = -C2, mu = C1)
//   y_a = sum_q w_q |J_q| [mu (H + H^T) + lambda tr(H) I] grad(phi_a),  H = grad(u) = sum_b u_b grad(phi_b)^T,
// and for every penalty-Dirichlet face (TPZElasticity3D::ContributeBC type 0)
//   y_a = big sum_q w_q |J_q| phi_a (sum_b phi_b u_b).
// It is the operator of the assembled matrix (up to FP32 rounding and the
// 1e-12 entries AddKel skips): the CG's FP64 true residual still uses the
// assembled FP64 CSR.  Per application it reads the element records (corner
// coordinates, block rows, lambda and mu: ~220 B per element) and gathers /
// scatters the nodal vectors, instead of streaming ~2.7 GB of blocks at 64^3.
//
// Q2 hexes (27 shapes, 27 points): one warp per element; lane q keeps its
// point's reference gradients (81 floats) in registers and the shapes'
// gradients sit in shared memory, both loaded once per CTA; per element the
// nodal values and the per-point stress pass through shared memory.  p^T q is
// the sum of the element energies u_e^T K_e u_e.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "gpz_internal.h"
#include "gpz_shapes.h"
#include "gpz_solver_common.cuh"
#include "gpz_tc.cuh"

namespace gpz {

namespace {

constexpr int kNS = 27;  // Q2 hex shapes
constexpr int kNQ = 27;  // 3 x 3 x 3 Gauss points
constexpr int kFS = 9;   // Q2 face shapes
constexpr int kFQ = 9;   // 3 x 3 face points
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ double x_of(const double (&cx)[8][3], int k, int j) { return cx[k][j]; }

// element records: corner coordinates, block rows of the shapes, (lambda, mu),
// and for affine hexes the constant inverse Jacobian and |det J|
__global__ void k_mf_records(int64_t n, const int64_t *__restrict__ elems, const int64_t *__restrict__ el_nodes,
                             const double *__restrict__ xyz, const int64_t *__restrict__ el_conn,
                             const int64_t *__restrict__ bpos, const int *__restrict__ sside,
                             const int *__restrict__ sk, int nsh, int nc, const double *__restrict__ coef, double E0,
                             double nu, float *__restrict__ rxyz, int32_t *__restrict__ rrows, float *__restrict__ rlm,
                             float *__restrict__ rgeo, int *__restrict__ err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t e = elems[i];
  double cx[8][3];
  for (int k = 0; k < nc; k++) {
    const int64_t node = el_nodes[e * 8 + k];
    for (int j = 0; j < 3; j++) {
      cx[k][j] = xyz[node * 3 + j];
      rxyz[(i * nc + k) * 3 + j] = (float)cx[k][j];
    }
  }
  if (rgeo) {
    // affine hex (vanishing xi.eta, xi.zeta, eta.zeta, xi.eta.zeta coefficients):
    // constant Jacobian; (Jinv, |det J|), det 0 marks a non-affine element
    const signed char sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                  {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    double hi = 0.0, big = 0.0, a[3][3];
    for (int j = 0; j < 3; j++) {
      double t4 = 0, t5 = 0, t6 = 0, t7 = 0, mn = cx[0][j], mx = cx[0][j];
      for (int k = 0; k < 8; k++) {
        const double x = cx[k][j];
        t4 += sg[k][0] * sg[k][1] * x;
        t5 += sg[k][0] * sg[k][2] * x;
        t6 += sg[k][1] * sg[k][2] * x;
        t7 += sg[k][0] * sg[k][1] * sg[k][2] * x;
        mn = fmin(mn, x);
        mx = fmax(mx, x);
      }
      hi = fmax(hi, fmax(fmax(fabs(t4), fabs(t5)), fmax(fabs(t6), fabs(t7))));
      big = fmax(big, mx - mn);
      for (int d = 0; d < 3; d++) {
        double t = 0.0;
        for (int k = 0; k < 8; k++) t += sg[k][d] * x_of(cx, k, j);
        a[j][d] = t / 8.0;
      }
    }
    float *g = rgeo + i * 10;
    if (hi <= 1e-12 * big) {
      const double det = -a[0][2] * a[1][1] * a[2][0] + a[0][1] * a[1][2] * a[2][0] + a[0][2] * a[1][0] * a[2][1] -
                         a[0][0] * a[1][2] * a[2][1] - a[0][1] * a[1][0] * a[2][2] + a[0][0] * a[1][1] * a[2][2];
      const double id = 1.0 / det;
      g[0] = (float)((-a[1][2] * a[2][1] + a[1][1] * a[2][2]) * id);
      g[1] = (float)((a[0][2] * a[2][1] - a[0][1] * a[2][2]) * id);
      g[2] = (float)((-a[0][2] * a[1][1] + a[0][1] * a[1][2]) * id);
      g[3] = (float)((a[1][2] * a[2][0] - a[1][0] * a[2][2]) * id);
      g[4] = (float)((-a[0][2] * a[2][0] + a[0][0] * a[2][2]) * id);
      g[5] = (float)((a[0][2] * a[1][0] - a[0][0] * a[1][2]) * id);
      g[6] = (float)((-a[1][1] * a[2][0] + a[1][0] * a[2][1]) * id);
      g[7] = (float)((a[0][1] * a[2][0] - a[0][0] * a[2][1]) * id);
      g[8] = (float)((-a[0][1] * a[1][0] + a[0][0] * a[1][1]) * id);
      g[9] = (float)fabs(det);
    } else {
      for (int k = 0; k < 10; k++) g[k] = 0.f;
    }
  }
  for (int a = 0; a < nsh; a++) {
    const int64_t eq = bpos[el_conn[e * 27 + sside[a]]] + (int64_t)sk[a] * 3;
    if (eq % 3 != 0) atomicOr(err, 4096);
    rrows[i * nsh + a] = (int32_t)(eq / 3);
  }
  if (rlm) {
    const double E = coef ? coef[e] : E0;
    const double mu = E / (2. + 2. * nu);                  // C1
    const double lam = -(E * nu / (-1. + nu + 2. * nu * nu));  // -C2
    rlm[2 * i] = (float)lam;
    rlm[2 * i + 1] = (float)mu;
  }
}

// One penalty face by one warp: big sum_q w |J| phi_a (sum_b phi_b u_b) added to q, its energy to en.
// sphi / sd / sw: the face tables in shared memory; su, sc, st: the warp's own scratch.
__device__ __forceinline__ void mf_face(int64_t i, int lane, const float *sphi, const float *sd, const float *sw,
                                        float (*su)[4], float *sc, float (*st)[4], float big,
                                        const float *__restrict__ rxyz, const int32_t *__restrict__ rows,
                                        const float4 *__restrict__ p4, float4 *__restrict__ q4, KSum &en) {
  int32_t row = 0;
  float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
  if (lane < kFS) {
    row = rows[i * kFS + lane];
    u = p4[row];
    su[lane][0] = u.x;
    su[lane][1] = u.y;
    su[lane][2] = u.z;
  }
  if (lane < 12) sc[lane] = rxyz[i * 12 + lane];
  __syncwarp();
  if (lane < kFQ) {
    const int q = lane;
    float g0[3] = {0.f, 0.f, 0.f}, g1[3] = {0.f, 0.f, 0.f};
    for (int k = 0; k < 4; k++)
      for (int j = 0; j < 3; j++) {
        g0[j] += sc[k * 3 + j] * sd[(q * 2 + 0) * kFS + k];
        g1[j] += sc[k * 3 + j] * sd[(q * 2 + 1) * kFS + k];
      }
    const float cx = g0[1] * g1[2] - g0[2] * g1[1], cy = g0[2] * g1[0] - g0[0] * g1[2],
                cz = g0[0] * g1[1] - g0[1] * g1[0];
    const float wd = big * sw[q] * sqrtf(cx * cx + cy * cy + cz * cz);
    float uq[3] = {0.f, 0.f, 0.f};
    for (int b = 0; b < kFS; b++) {
      const float ph = sphi[q * kFS + b];
      for (int s = 0; s < 3; s++) uq[s] += ph * su[b][s];
    }
    for (int s = 0; s < 3; s++) st[q][s] = wd * uq[s];
  }
  __syncwarp();
  if (lane < kFS) {
    float y[3] = {0.f, 0.f, 0.f};
    for (int q = 0; q < kFQ; q++) {
      const float ph = sphi[q * kFS + lane];
      for (int s = 0; s < 3; s++) y[s] += st[q][s] * ph;
    }
    en.add(y[0] * u.x + y[1] * u.y + y[2] * u.z);
    red_add_f4(&q4[row], make_float4(y[0], y[1], y[2], 0.f));
  }
  __syncwarp();
}

// penalty faces: y_a += big sum_q w |J| phi_a phi_b u_b; their energy goes to *energy
__global__ void __launch_bounds__(kThreads) k_mf_faces(int64_t n, const float *__restrict__ rxyz,
                                                       const int32_t *__restrict__ rows, const float *__restrict__ phi,
                                                       const float *__restrict__ dphi, const float *__restrict__ w,
                                                       float big, const float4 *__restrict__ p4,
                                                       float4 *__restrict__ q4, double *__restrict__ energy, Red R) {
  if (!active(R.iscal)) return;
  __shared__ float sphi[kFQ * kFS], sd[kFQ * 2 * kFS], sw[kFQ];
  __shared__ float su[kWarps][kFS][4], sc[kWarps][12], st[kWarps][kFQ][4];
  for (int k = threadIdx.x; k < kFQ * kFS; k += blockDim.x) sphi[k] = phi[k];
  for (int k = threadIdx.x; k < kFQ * 2 * kFS; k += blockDim.x) sd[k] = dphi[k];
  if (threadIdx.x < kFQ) sw[threadIdx.x] = w[threadIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  KSum en;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n;
       i += ((int64_t)gridDim.x * blockDim.x) >> 5)
    mf_face(i, lane, sphi, sd, sw, su[wp], sc[wp], st[wp], big, rxyz, rows, p4, q4, en);
  double v[1] = {en.get()}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) *energy = tot[0];
}

// volume elements (Q2 hexes); pq = element energies + the faces' (*face_energy).
// 128-thread CTAs, 3 per SM: lane q keeps its point's reference gradients in
// registers (81 floats); the shapes' gradients sit in shared memory as
// [point][shape] float4 rows (conflict-free 16-byte loads); the next
// element's records are loaded while the current one is computed.
constexpr int kMfThreads = 128;
constexpr int kMfWarps = kMfThreads / 32;
__global__ void __launch_bounds__(kMfThreads, 3) k_mf_hex27(int64_t n, const float *__restrict__ rxyz,
                                                            const int32_t *__restrict__ rows,
                                                            const float *__restrict__ rlm,
                                                            const float *__restrict__ rgeo,
                                                            const float *__restrict__ dphi /*[q][3][a]*/,
                                                            const float *__restrict__ w,
                                                            const float4 *__restrict__ p4, float4 *__restrict__ q4,
                                                            const double *__restrict__ face_energy, Red R) {
  if (!active(R.iscal)) return;
  __shared__ float4 sdt[kNQ][32];            // [q][a] = (d0, d1, d2, 0) of shape a at point q
  __shared__ float4 su[kMfWarps][kNS];
  __shared__ float sc[kMfWarps][24 + 10];  // corners, then the affine geometry (Jinv, |det|)
  __shared__ float4 st[kMfWarps][kNQ][3];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  for (int k = threadIdx.x; k < kNQ * 32; k += blockDim.x) {
    const int q = k / 32, a = k % 32;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a < kNS) {
      v.x = dphi[(q * 3 + 0) * kNS + a];
      v.y = dphi[(q * 3 + 1) * kNS + a];
      v.z = dphi[(q * 3 + 2) * kNS + a];
    }
    sdt[q][a] = v;
  }
  float D[3][kNS], wq = 0.f;
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int b = 0; b < kNS; b++) D[j][b] = lane < kNQ ? dphi[(lane * 3 + j) * kNS + b] : 0.f;
  if (lane < kNQ) wq = w[lane];
  __syncthreads();
  KSum en;
  const int64_t step = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  // records of the first element
  int32_t row = 0;
  float cxv = 0.f, gv = 0.f, lam = 0.f, mu = 0.f;
  if (i < n) {
    if (lane < kNS) row = rows[i * kNS + lane];
    if (lane < 24) cxv = rxyz[i * 24 + lane];
    if (lane < 10) gv = rgeo[i * 10 + lane];
    lam = rlm[2 * i];
    mu = rlm[2 * i + 1];
  }
  for (; i < n; i += step) {
    float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
    if (lane < kNS) {
      u = p4[row];
      su[wp][lane] = u;
    }
    if (lane < 24) sc[wp][lane] = cxv;
    if (lane < 10) sc[wp][24 + lane] = gv;
    const float lam_i = lam, mu_i = mu;
    const int32_t row_i = row;
    // prefetch the next element's records
    const int64_t nx = i + step;
    if (nx < n) {
      if (lane < kNS) row = rows[nx * kNS + lane];
      if (lane < 24) cxv = rxyz[nx * 24 + lane];
      if (lane < 10) gv = rgeo[nx * 10 + lane];
      lam = rlm[2 * nx];
      mu = rlm[2 * nx + 1];
    }
    __syncwarp();
    if (lane < kNQ) {
      float ji[3][3], det;
      if (sc[wp][24 + 9] > 0.f) {
        // affine element: the constant Jacobian of the records
#pragma unroll
        for (int k = 0; k < 9; k++) ji[k / 3][k % 3] = sc[wp][24 + k];
        det = sc[wp][24 + 9];
      } else {
        // Jacobian from the corner shapes (the first 8 of the table), as TPZGeoEl::Jacobian
        float a[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
        for (int k = 0; k < 8; k++)
#pragma unroll
          for (int j = 0; j < 3; j++)
#pragma unroll
            for (int d = 0; d < 3; d++) a[j][d] += sc[wp][k * 3 + j] * D[d][k];
        det = -a[0][2] * a[1][1] * a[2][0] + a[0][1] * a[1][2] * a[2][0] + a[0][2] * a[1][0] * a[2][1] -
              a[0][0] * a[1][2] * a[2][1] - a[0][1] * a[1][0] * a[2][2] + a[0][0] * a[1][1] * a[2][2];
        const float id = 1.f / det;
        ji[0][0] = (-a[1][2] * a[2][1] + a[1][1] * a[2][2]) * id;
        ji[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * id;
        ji[0][2] = (-a[0][2] * a[1][1] + a[0][1] * a[1][2]) * id;
        ji[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) * id;
        ji[1][1] = (-a[0][2] * a[2][0] + a[0][0] * a[2][2]) * id;
        ji[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * id;
        ji[2][0] = (-a[1][1] * a[2][0] + a[1][0] * a[2][1]) * id;
        ji[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * id;
        ji[2][2] = (-a[0][1] * a[1][0] + a[0][0] * a[1][1]) * id;
      }
      // reference gradient of u at the point, then physical H[s][d] = sum_j Hh[s][j] ji[j][d]
      float hh[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
      for (int b = 0; b < kNS; b++) {
        const float4 ub = su[wp][b];
#pragma unroll
        for (int j = 0; j < 3; j++) {
          hh[0][j] += ub.x * D[j][b];
          hh[1][j] += ub.y * D[j][b];
          hh[2][j] += ub.z * D[j][b];
        }
      }
      float H[3][3];
#pragma unroll
      for (int s2 = 0; s2 < 3; s2++)
#pragma unroll
        for (int d = 0; d < 3; d++) H[s2][d] = hh[s2][0] * ji[0][d] + hh[s2][1] * ji[1][d] + hh[s2][2] * ji[2][d];
      const float wd = wq * fabsf(det);
      const float lt = lam_i * (H[0][0] + H[1][1] + H[2][2]);
      float T[3][3];
#pragma unroll
      for (int s2 = 0; s2 < 3; s2++)
#pragma unroll
        for (int d = 0; d < 3; d++) T[s2][d] = wd * (mu_i * (H[s2][d] + H[d][s2]) + (s2 == d ? lt : 0.f));
      // back to reference derivatives: Th[s][j] = sum_d T[s][d] ji[j][d]
#pragma unroll
      for (int s2 = 0; s2 < 3; s2++) {
        float4 t;
        t.x = T[s2][0] * ji[0][0] + T[s2][1] * ji[0][1] + T[s2][2] * ji[0][2];
        t.y = T[s2][0] * ji[1][0] + T[s2][1] * ji[1][1] + T[s2][2] * ji[1][2];
        t.z = T[s2][0] * ji[2][0] + T[s2][1] * ji[2][1] + T[s2][2] * ji[2][2];
        t.w = 0.f;
        st[wp][lane][s2] = t;
      }
    }
    __syncwarp();
    if (lane < kNS) {
      float y0 = 0.f, y1 = 0.f, y2 = 0.f;
#pragma unroll
      for (int q = 0; q < kNQ; q++) {
        const float4 t0 = st[wp][q][0], t1 = st[wp][q][1], t2 = st[wp][q][2];
        const float4 g = sdt[q][lane];
        y0 += t0.x * g.x + t0.y * g.y + t0.z * g.z;
        y1 += t1.x * g.x + t1.y * g.y + t1.z * g.z;
        y2 += t2.x * g.x + t2.y * g.y + t2.z * g.z;
      }
      en.add(y0 * u.x + y1 * u.y + y2 * u.z);
      red_add_f4(&q4[row_i], make_float4(y0, y1, y2, 0.f));
    }
    __syncwarp();
  }
  double v[1] = {en.get()}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    const double pq = tot[0] + (face_energy ? *face_energy : 0.0);
    R.scal[S_PQ] = pq;
    R.scal[S_ALPHA] = R.scal[S_RHO] / pq;
    R.iscal[I_SP32]++;
  }
}


// ---------------------------------------------------------------- sum-factorised variant
// The 27 Q2 functions of the hex span the tensor space Q2, so each element's
// field is also given by its values v at the 27 Lagrange nodes (-1, 0, 1)^3:
// v = Phi c with Phi[j][a] = phi_a(node j) (125 nonzeros; one long row, the
// interior node).  On nodal values the reference gradients at the 3 x 3 x 3
// Gauss points factor into 1D contractions with the 3 x 3 Lagrange value and
// derivative matrices B, D: 8 x 81 multiply-adds per component instead of
// 27 x 81, and the transposed contractions and Phi^T bring the stresses back.
// One warp per element; the 27 active lanes are (component, pencil) in the
// tensor stages and points in the pointwise stage, exchanging through shared
// memory.  The arithmetic is the element operator of k_mf_hex27 with another
// summation order.
constexpr int kSfThreads = 128;
constexpr int kSfWarps = kSfThreads / 32;
constexpr int kSfMaxNz = 160;  // stored nonzeros of Phi (rows of <= 9, plus the long row)
// table layout (floats): B[3][3], D[3][3], w[27], corner gradients [27][3][8],
// long row [27], row values, column values
constexpr int SF_B = 0, SF_D = 9, SF_W = 18, SF_DC = 45, SF_LONG = SF_DC + 27 * 24, SF_RV = SF_LONG + 27,
              SF_CV = SF_RV + kSfMaxNz, SF_NF = SF_CV + kSfMaxNz;
// index layout (ints): row pointers [28], column pointers [28], row columns, column rows, long row index
constexpr int SFI_RP = 0, SFI_CP = 28, SFI_RC = 56, SFI_CR = SFI_RC + kSfMaxNz, SFI_LONG = SFI_CR + kSfMaxNz,
              SFI_NI = SFI_LONG + 1;

// 1D Lagrange values B[q][j] and derivatives D[q][j] at the 3 Gauss points:
// warp-uniform operands, read through the constant cache
__constant__ float c_sfB[9], c_sfD[9];

// Shared-memory layouts (component s, tensor indices a, b, c of 0..2): each is
// a position map under which the warp's 27 addresses fall in 27 distinct
// banks in both stages that access the buffer (the writer's and the reader's
// lane patterns differ), so no tensor stage has bank conflicts.
__device__ __forceinline__ int sf_v(int s, int a, int b, int c) { return 3 * s + a + 9 * b + 29 * c; }   // nodal
__device__ __forceinline__ int sf_t1(int s, int a, int b, int c) { return 9 * s + a + 3 * b + 29 * c; }  // (j1, j2, q3)
__device__ __forceinline__ int sf_t2(int s, int a, int b, int c) { return 3 * s + a + 27 * b + 9 * c; }  // (j1, q2, q3)
__device__ __forceinline__ int sf_h(int s, int d, int q) { return 27 * s + 81 * d + q; }

struct SfWarp {
  float4 su[27];   // element coefficients (3 components per shape)
  float v[85];     // nodal values sf_v, later the adjoint's nodal output
  float t1[2][85]; // zeta contractions (B, D) sf_t1
  float t2[3][81]; // eta contractions (BB, DB, BD) sf_t2
  float h[243];    // reference gradients sf_h(s, d, q), then the pulled-back stresses
  float geo[34];   // corners, then the affine geometry (Jinv, |det J|)
};

__global__ void __launch_bounds__(kSfThreads, 5) k_mf_hex27_sf(int64_t n, const float *__restrict__ rxyz,
                                                               const int32_t *__restrict__ rows,
                                                               const float *__restrict__ rlm,
                                                               const float *__restrict__ rgeo,
                                                               const float *__restrict__ tabf,
                                                               const int *__restrict__ tabi,
                                                               const float4 *__restrict__ p4, float4 *__restrict__ q4,
                                                               const double *__restrict__ face_energy, Red R) {
  if (!active(R.iscal)) return;
  __shared__ float sf[SF_NF];
  __shared__ int si[SFI_NI];
  __shared__ SfWarp sw[kSfWarps];
  for (int k = threadIdx.x; k < SF_NF; k += blockDim.x) sf[k] = tabf[k];
  for (int k = threadIdx.x; k < SFI_NI; k += blockDim.x) si[k] = tabi[k];
  __syncthreads();
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  SfWarp &W = sw[wp];
  const float *B = c_sfB, *D = c_sfD;
  const int jl = si[SFI_LONG];
  // this lane's row (node j = lane) and column (shape a = lane) of Phi, in registers
  constexpr int kRow = 9, kCol = 8;
  float rv[kRow], cv[kCol];
  uint32_t rc[3] = {0u, 0u, 0u}, cr[2] = {0u, 0u};  // indices (< 27), four per word
  int nrow = 0, ncol = 0;
  if (lane < kNS) {
    const int r0 = si[SFI_RP + lane], c0 = si[SFI_CP + lane];
    nrow = lane == jl ? 0 : min(kRow, si[SFI_RP + lane + 1] - r0);
    ncol = min(kCol, si[SFI_CP + lane + 1] - c0);
#pragma unroll
    for (int k = 0; k < kRow; k++) {
      rv[k] = k < nrow ? sf[SF_RV + r0 + k] : 0.f;
      rc[k / 4] |= (uint32_t)(k < nrow ? si[SFI_RC + r0 + k] : 0) << (8 * (k % 4));
    }
#pragma unroll
    for (int k = 0; k < kCol; k++) {
      cv[k] = k < ncol ? sf[SF_CV + c0 + k] : 0.f;
      const int jn = k < ncol ? si[SFI_CR + c0 + k] : 0;  // node -> its sf_v offset (component 0)
      cr[k / 4] |= (uint32_t)sf_v(0, jn % 3, (jn / 3) % 3, jn / 9) << (8 * (k % 4));
    }
  }
  const float flong = lane < kNS ? sf[SF_LONG + lane] : 0.f;
  const int vlane = sf_v(0, lane % 3, (lane / 3) % 3, lane / 9), vlong = sf_v(0, jl % 3, (jl / 3) % 3, jl / 9);
  // stage lanes: component s and pencil p (two tensor indices of 0..2)
  const bool act = lane < 27;
  const int s = act ? lane / 9 : 0, p = lane % 9;
  const int pa = p % 3, pb = p / 3;
  KSum en;
  const int64_t step = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int32_t row = 0;
  float cxv = 0.f, gv = 0.f, lam = 0.f, mu = 0.f;
  if (i < n) {
    if (lane < kNS) row = rows[i * kNS + lane];
    if (lane < 24) cxv = rxyz[i * 24 + lane];
    if (lane < 10) gv = rgeo[i * 10 + lane];
    lam = rlm[2 * i];
    mu = rlm[2 * i + 1];
  }
  for (; i < n; i += step) {
    float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
    if (lane < kNS) {
      u = p4[row];
      W.su[lane] = u;
    }
    if (lane < 24) W.geo[lane] = cxv;
    if (lane < 10) W.geo[24 + lane] = gv;
    const float lam_i = lam, mu_i = mu;
    const int32_t row_i = row;
    const int64_t nx = i + step;
    if (nx < n) {
      if (lane < kNS) row = rows[nx * kNS + lane];
      if (lane < 24) cxv = rxyz[nx * 24 + lane];
      if (lane < 10) gv = rgeo[nx * 10 + lane];
      lam = rlm[2 * nx];
      mu = rlm[2 * nx + 1];
    }
    __syncwarp();
    // v = Phi c: short rows by their lane, the long row as a warp sum
    {
      float a0 = 0.f, a1 = 0.f, a2 = 0.f;
      if (lane < kNS && lane != jl) {
#pragma unroll
        for (int k = 0; k < kRow; k++) {
          if (k >= nrow) break;
          const float4 c = W.su[(rc[k / 4] >> (8 * (k % 4))) & 0xffu];
          a0 = fmaf(rv[k], c.x, a0);
          a1 = fmaf(rv[k], c.y, a1);
          a2 = fmaf(rv[k], c.z, a2);
        }
        W.v[vlane] = a0;
        W.v[vlane + 3] = a1;
        W.v[vlane + 6] = a2;
      }
      float b0 = flong * u.x, b1 = flong * u.y, b2 = flong * u.z;
      for (int o = 16; o > 0; o >>= 1) {
        b0 += __shfl_xor_sync(0xffffffffu, b0, o);
        b1 += __shfl_xor_sync(0xffffffffu, b1, o);
        b2 += __shfl_xor_sync(0xffffffffu, b2, o);
      }
      if (lane == 0) {
        W.v[vlong] = b0;
        W.v[vlong + 3] = b1;
        W.v[vlong + 6] = b2;
      }
    }
    __syncwarp();
    // zeta: lane (s, j1 = pa, j2 = pb)
    if (act) {
      const float x0 = W.v[sf_v(s, pa, pb, 0)], x1 = W.v[sf_v(s, pa, pb, 1)], x2 = W.v[sf_v(s, pa, pb, 2)];
#pragma unroll
      for (int q3 = 0; q3 < 3; q3++) {
        W.t1[0][sf_t1(s, pa, pb, q3)] = B[q3 * 3] * x0 + B[q3 * 3 + 1] * x1 + B[q3 * 3 + 2] * x2;
        W.t1[1][sf_t1(s, pa, pb, q3)] = D[q3 * 3] * x0 + D[q3 * 3 + 1] * x1 + D[q3 * 3 + 2] * x2;
      }
    }
    __syncwarp();
    // eta: lane (s, j1 = pa, q3 = pb)
    if (act) {
      const float y0 = W.t1[0][sf_t1(s, pa, 0, pb)], y1 = W.t1[0][sf_t1(s, pa, 1, pb)],
                  y2 = W.t1[0][sf_t1(s, pa, 2, pb)];
      const float z0 = W.t1[1][sf_t1(s, pa, 0, pb)], z1 = W.t1[1][sf_t1(s, pa, 1, pb)],
                  z2 = W.t1[1][sf_t1(s, pa, 2, pb)];
#pragma unroll
      for (int q2 = 0; q2 < 3; q2++) {
        const int o = sf_t2(s, pa, q2, pb);
        W.t2[0][o] = B[q2 * 3] * y0 + B[q2 * 3 + 1] * y1 + B[q2 * 3 + 2] * y2;
        W.t2[1][o] = D[q2 * 3] * y0 + D[q2 * 3 + 1] * y1 + D[q2 * 3 + 2] * y2;
        W.t2[2][o] = B[q2 * 3] * z0 + B[q2 * 3 + 1] * z1 + B[q2 * 3 + 2] * z2;
      }
    }
    __syncwarp();
    // xi: lane (s, q2 = pa, q3 = pb) -> reference gradients at q = q1 + 3 p
    if (act) {
      const int b = sf_t2(s, 0, pa, pb);  // + j1
      const float g0 = W.t2[0][b], g1 = W.t2[0][b + 1], g2 = W.t2[0][b + 2];
      const float e0 = W.t2[1][b], e1 = W.t2[1][b + 1], e2 = W.t2[1][b + 2];
      const float f0 = W.t2[2][b], f1 = W.t2[2][b + 1], f2 = W.t2[2][b + 2];
#pragma unroll
      for (int q1 = 0; q1 < 3; q1++) {
        const int q = q1 + 3 * p;
        W.h[sf_h(s, 0, q)] = D[q1 * 3] * g0 + D[q1 * 3 + 1] * g1 + D[q1 * 3 + 2] * g2;
        W.h[sf_h(s, 1, q)] = B[q1 * 3] * e0 + B[q1 * 3 + 1] * e1 + B[q1 * 3 + 2] * e2;
        W.h[sf_h(s, 2, q)] = B[q1 * 3] * f0 + B[q1 * 3 + 1] * f1 + B[q1 * 3 + 2] * f2;
      }
    }
    __syncwarp();
    // pointwise: lane q
    if (lane < kNQ) {
      const int q = lane;
      float ji[3][3], det;
      if (W.geo[24 + 9] > 0.f) {
#pragma unroll
        for (int k = 0; k < 9; k++) ji[k / 3][k % 3] = W.geo[24 + k];
        det = W.geo[24 + 9];
      } else {
        float a[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
        const float *dc = sf + SF_DC + q * 24;
#pragma unroll
        for (int k = 0; k < 8; k++)
#pragma unroll
          for (int j = 0; j < 3; j++)
#pragma unroll
            for (int d = 0; d < 3; d++) a[j][d] += W.geo[k * 3 + j] * dc[d * 8 + k];
        det = -a[0][2] * a[1][1] * a[2][0] + a[0][1] * a[1][2] * a[2][0] + a[0][2] * a[1][0] * a[2][1] -
              a[0][0] * a[1][2] * a[2][1] - a[0][1] * a[1][0] * a[2][2] + a[0][0] * a[1][1] * a[2][2];
        const float id = 1.f / det;
        ji[0][0] = (-a[1][2] * a[2][1] + a[1][1] * a[2][2]) * id;
        ji[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * id;
        ji[0][2] = (-a[0][2] * a[1][1] + a[0][1] * a[1][2]) * id;
        ji[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) * id;
        ji[1][1] = (-a[0][2] * a[2][0] + a[0][0] * a[2][2]) * id;
        ji[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * id;
        ji[2][0] = (-a[1][1] * a[2][0] + a[1][0] * a[2][1]) * id;
        ji[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * id;
        ji[2][2] = (-a[0][1] * a[1][0] + a[0][0] * a[1][1]) * id;
      }
      float hh[3][3], H[3][3], T[3][3];
#pragma unroll
      for (int s2 = 0; s2 < 3; s2++)
#pragma unroll
        for (int j = 0; j < 3; j++) hh[s2][j] = W.h[sf_h(s2, j, q)];
#pragma unroll
      for (int s2 = 0; s2 < 3; s2++)
#pragma unroll
        for (int d = 0; d < 3; d++) H[s2][d] = hh[s2][0] * ji[0][d] + hh[s2][1] * ji[1][d] + hh[s2][2] * ji[2][d];
      const float wd = sf[SF_W + q] * fabsf(det);
      const float lt = lam_i * (H[0][0] + H[1][1] + H[2][2]);
#pragma unroll
      for (int s2 = 0; s2 < 3; s2++)
#pragma unroll
        for (int d = 0; d < 3; d++) T[s2][d] = wd * (mu_i * (H[s2][d] + H[d][s2]) + (s2 == d ? lt : 0.f));
#pragma unroll
      for (int s2 = 0; s2 < 3; s2++)
#pragma unroll
        for (int j = 0; j < 3; j++)
          W.h[sf_h(s2, j, q)] = T[s2][0] * ji[j][0] + T[s2][1] * ji[j][1] + T[s2][2] * ji[j][2];
    }
    __syncwarp();
    // transposed xi: lane (s, q2 = pa, q3 = pb)
    if (act) {
      const int b = sf_t2(s, 0, pa, pb);  // + j1
      float g[3], e[3], f[3];
#pragma unroll
      for (int q1 = 0; q1 < 3; q1++) {
        g[q1] = W.h[sf_h(s, 0, q1 + 3 * p)];
        e[q1] = W.h[sf_h(s, 1, q1 + 3 * p)];
        f[q1] = W.h[sf_h(s, 2, q1 + 3 * p)];
      }
#pragma unroll
      for (int j1 = 0; j1 < 3; j1++) {
        W.t2[0][b + j1] = D[j1] * g[0] + D[3 + j1] * g[1] + D[6 + j1] * g[2];
        W.t2[1][b + j1] = B[j1] * e[0] + B[3 + j1] * e[1] + B[6 + j1] * e[2];
        W.t2[2][b + j1] = B[j1] * f[0] + B[3 + j1] * f[1] + B[6 + j1] * f[2];
      }
    }
    __syncwarp();
    // transposed eta: lane (s, j1 = pa, q3 = pb)
    if (act) {
      float g[3], e[3], f[3];
#pragma unroll
      for (int q2 = 0; q2 < 3; q2++) {
        const int o = sf_t2(s, pa, q2, pb);
        g[q2] = W.t2[0][o];
        e[q2] = W.t2[1][o];
        f[q2] = W.t2[2][o];
      }
#pragma unroll
      for (int j2 = 0; j2 < 3; j2++) {
        const int o = sf_t1(s, pa, j2, pb);
        W.t1[0][o] = B[j2] * g[0] + B[3 + j2] * g[1] + B[6 + j2] * g[2] + D[j2] * e[0] + D[3 + j2] * e[1] +
                     D[6 + j2] * e[2];
        W.t1[1][o] = B[j2] * f[0] + B[3 + j2] * f[1] + B[6 + j2] * f[2];
      }
    }
    __syncwarp();
    // transposed zeta: lane (s, j1 = pa, j2 = pb) -> nodal output
    if (act) {
      float g[3], f[3];
#pragma unroll
      for (int q3 = 0; q3 < 3; q3++) {
        g[q3] = W.t1[0][sf_t1(s, pa, pb, q3)];
        f[q3] = W.t1[1][sf_t1(s, pa, pb, q3)];
      }
#pragma unroll
      for (int j3 = 0; j3 < 3; j3++)
        W.v[sf_v(s, pa, pb, j3)] = B[j3] * g[0] + B[3 + j3] * g[1] + B[6 + j3] * g[2] + D[j3] * f[0] +
                                   D[3 + j3] * f[1] + D[6 + j3] * f[2];
    }
    __syncwarp();
    // y = Phi^T v: lane a, its column (<= 8 nodes)
    if (lane < kNS) {
      float y0 = 0.f, y1 = 0.f, y2 = 0.f;
#pragma unroll
      for (int k = 0; k < kCol; k++) {
        if (k >= ncol) break;
        const int o = (cr[k / 4] >> (8 * (k % 4))) & 0xffu;  // sf_v offset of the node, component 0
        y0 = fmaf(cv[k], W.v[o], y0);
        y1 = fmaf(cv[k], W.v[o + 3], y1);
        y2 = fmaf(cv[k], W.v[o + 6], y2);
      }
      en.add(y0 * u.x + y1 * u.y + y2 * u.z);
      red_add_f4(&q4[row_i], make_float4(y0, y1, y2, 0.f));
    }
    __syncwarp();
  }
  double v[1] = {en.get()}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    const double pq = tot[0] + (face_energy ? *face_energy : 0.0);
    R.scal[S_PQ] = pq;
    R.scal[S_ALPHA] = R.scal[S_RHO] / pq;
    R.iscal[I_SP32]++;
  }
}

// ---------------------------------------------------------------- tensor-core variant
// The same operator with the two element contractions on the 5th-generation
// tensor cores (tcgen05.mma kind::tf32, operands in shared memory, FP32
// accumulators in TMEM), as split 3xTF32 products (hi.hi + hi.lo + lo.hi, about
// FP32 accuracy).  A CTA of 4 warps takes tiles of 40 elements; matrix row
// r = 32 w + 3 e + s holds component s of element e of warp w (rows 30 and 31 of
// each warp are padding), so an element's three rows stay in one warp.
//   phase 1:  Hh[r][(q,j)] = sum_b U[r][b] D[b][(q,j)]       M 128, N 96 (81), K 32 (27)
//   pointwise: per (element, point) the Jacobian from the corners, the stress,
//              and back to reference derivatives TH; the element energy sum TH.Hh
//   phase 2:  Y[r][a] = sum_(q,j) TH[r][(q,j)] D[(q,j)][a]   M 128, N 32 (27), K 96 (81)
// Operands are K-major without swizzle: 8-row x 16-byte core matrices, K
// direction fastest (LBO 128 B, SBO = K/4 x 128 B).
constexpr int kTcThreads = 256;  // 8 warps: warps w and w + 4 share TMEM lane quarter w
constexpr int kTcEl = 40;   // elements per tile
constexpr int kTcElW = 10;  // per warp
constexpr uint32_t kB1 = 96 * 32 * 4, kB2 = 32 * 96 * 4, kA1 = 128 * 32 * 4, kA2 = 128 * 96 * 4;
constexpr uint32_t OFF_B1H = 0, OFF_B1L = OFF_B1H + kB1, OFF_B2H = OFF_B1L + kB1, OFF_B2L = OFF_B2H + kB2;
constexpr uint32_t OFF_A1H = OFF_B2L + kB2, OFF_A1L = OFF_A1H + kA1, OFF_A2H = OFF_A1L + kA1, OFF_A2L = OFF_A2H + kA2;
constexpr uint32_t OFF_CG = OFF_A2L + kA2, OFF_W = OFF_CG + 27 * 3 * 8 * 4, OFF_CX = OFF_W + 32 * 4;
constexpr uint32_t OFF_LM = OFF_CX + kTcEl * 24 * 4, OFF_GEO = OFF_LM + kTcEl * 2 * 4;
constexpr uint32_t OFF_ST1 = OFF_GEO + kTcEl * 10 * 4;
constexpr uint32_t OFF_TC_END = OFF_ST1 + 128 * 32 * 4;  // results staging (phase-2 rows)
constexpr int kTcGather = kTcEl * 32 / kTcThreads;        // (element, shape) items per thread
constexpr int kTcItems = (kTcEl * 27 + kTcThreads - 1) / kTcThreads;  // (element, point) items per thread

// U rows of a tile (the nodal values, split hi / lo), its corners and (lambda, mu);
// every load is issued before the first store
__device__ __forceinline__ void tc_gather(unsigned char *sm, int64_t e0, int64_t n, const int32_t *__restrict__ rows,
                                          const float4 *__restrict__ p4, const float *__restrict__ rxyz,
                                          const float *__restrict__ rlm, const float *__restrict__ rgeo, int tid) {
  int32_t ri[kTcGather];
  float4 pv[kTcGather];
#pragma unroll
  for (int k = 0; k < kTcGather; k++) {
    const int t = tid + k * kTcThreads, le = t / 32, b = t % 32;
    const int64_t e = e0 + le;
    ri[k] = (b < 27 && e < n) ? rows[e * 27 + b] : -1;
  }
#pragma unroll
  for (int k = 0; k < kTcGather; k++) pv[k] = ri[k] >= 0 ? p4[ri[k]] : make_float4(0.f, 0.f, 0.f, 0.f);
  float cv[4];
  float lv[2] = {0.f, 0.f};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int t = tid + k * kTcThreads;
    const int64_t e = e0 + t / 24;
    cv[k] = (t < kTcEl * 24 && e < n) ? rxyz[e * 24 + t % 24] : 0.f;
  }
  if (tid < kTcEl && e0 + tid < n) {
    lv[0] = rlm[2 * (e0 + tid)];
    lv[1] = rlm[2 * (e0 + tid) + 1];
  }
  float gv[2];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int t = tid + k * kTcThreads;
    gv[k] = (t < kTcEl * 10 && e0 + t / 10 < n) ? rgeo[(e0 + t / 10) * 10 + t % 10] : 0.f;
  }
#pragma unroll
  for (int k = 0; k < kTcGather; k++) {
    const int t = tid + k * kTcThreads, le = t / 32, b = t % 32;
    const int r0 = (le / kTcElW) * 32 + 3 * (le % kTcElW);
    st_split(sm + OFF_A1H, sm + OFF_A1L, kmaj(r0, b, 32), pv[k].x);
    st_split(sm + OFF_A1H, sm + OFF_A1L, kmaj(r0 + 1, b, 32), pv[k].y);
    st_split(sm + OFF_A1H, sm + OFF_A1L, kmaj(r0 + 2, b, 32), pv[k].z);
  }
  float *cx = (float *)(sm + OFF_CX), *lm = (float *)(sm + OFF_LM);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int t = tid + k * kTcThreads;
    if (t < kTcEl * 24) cx[t] = cv[k];
  }
  if (tid < kTcEl) {
    lm[2 * tid] = lv[0];
    lm[2 * tid + 1] = lv[1];
  }
  float *geo = (float *)(sm + OFF_GEO);
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int t = tid + k * kTcThreads;
    if (t < kTcEl * 10) geo[t] = gv[k];
  }
}

__global__ void __launch_bounds__(kTcThreads, 1) k_mf_hex27_tc(int64_t n, const float *__restrict__ rxyz,
                                                               const int32_t *__restrict__ rows,
                                                               const float *__restrict__ rlm,
                                                               const float *__restrict__ rgeo,
                                                               const float *__restrict__ dphi /*[q][3][a]*/,
                                                               const float *__restrict__ w,
                                                               const float4 *__restrict__ p4, float4 *__restrict__ q4,
                                                               const double *__restrict__ face_energy,
                                                               int *__restrict__ err, Red R) {
  if (!active(R.iscal)) return;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_mb[2];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float *cg = (float *)(sm + OFF_CG), *sw = (float *)(sm + OFF_W), *cx = (float *)(sm + OFF_CX);
  float *lm = (float *)(sm + OFF_LM);
  // constant operands: B1[n][b] = D(b at point q, direction j), n = 3q + j; B2[a][n] = the same transposed
  for (int i = tid; i < 96 * 32; i += blockDim.x) {
    const int nn = i / 32, b = i % 32;
    st_split(sm + OFF_B1H, sm + OFF_B1L, kmaj(nn, b, 32), (nn < 81 && b < 27) ? dphi[nn * 27 + b] : 0.f);
  }
  for (int i = tid; i < 32 * 96; i += blockDim.x) {
    const int a = i / 96, nn = i % 96;
    st_split(sm + OFF_B2H, sm + OFF_B2L, kmaj(a, nn, 96), (a < 27 && nn < 81) ? dphi[nn * 27 + a] : 0.f);
  }
  for (int i = tid; i < 27 * 3 * 8; i += blockDim.x) cg[i] = dphi[(i / 8) * 27 + i % 8];  // corner gradients
  if (tid < 27) sw[tid] = w[tid];
  for (uint32_t i = tid; i < (kA1 + kA1 + kA2 + kA2) / 4; i += blockDim.x) ((float *)(sm + OFF_A1H))[i] = 0.f;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&s_tmem)), "r"(256));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&s_mb[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&s_mb[1])));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("fence.proxy.async.shared::cta;");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tm = s_tmem;
  const uint32_t id1 = (1u << 4) | (2u << 7) | (2u << 10) | ((96u >> 3) << 17) | ((128u >> 4) << 24);
  const uint32_t id2 = (1u << 4) | (2u << 7) | (2u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);
  const uint32_t a1h = tc_smem(sm + OFF_A1H), a1l = tc_smem(sm + OFF_A1L), a2h = tc_smem(sm + OFF_A2H),
                 a2l = tc_smem(sm + OFF_A2L);
  const uint32_t b1h = tc_smem(sm + OFF_B1H), b1l = tc_smem(sm + OFF_B1L), b2h = tc_smem(sm + OFF_B2H),
                 b2l = tc_smem(sm + OFF_B2L);
  KSum en;
  uint32_t parity = 0;
  bool failed = false;
  if ((int64_t)blockIdx.x * kTcEl < n) tc_gather(sm, (int64_t)blockIdx.x * kTcEl, n, rows, p4, rxyz, rlm, rgeo, tid);
  for (int64_t tile = blockIdx.x; tile * kTcEl < n && !failed; tile += gridDim.x) {
    const int64_t e0 = tile * kTcEl;
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (tid == 0) {
      for (int k = 0; k < 4; k++) {
        const uint64_t ah = tc_desc(a1h + k * 256, 1024), al = tc_desc(a1l + k * 256, 1024);
        const uint64_t bh = tc_desc(b1h + k * 256, 1024), bl = tc_desc(b1l + k * 256, 1024);
        tc_mma(tm, ah, bh, id1, k > 0);
        tc_mma(tm, ah, bl, id1, 1u);
        tc_mma(tm, al, bh, id1, 1u);
      }
      tc_commit(&s_mb[0]);
    }
    bool ok = tc_wait(&s_mb[0], parity);
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    // phase-1 rows -> row-major staging (row r at A2H + (r / 32) * 12288 + (r % 32) * 324): warp w reads
    // TMEM lanes 32 (w % 4) .. + 31, columns 48 (w / 4) .. + 47
    const int quarter = warp & 3, half = warp >> 2;
    {
      float *stg = (float *)(sm + OFF_A2H + quarter * 4 * 24 * 128);
      float h[16];
      for (int c0 = 48 * half; c0 < 48 * half + 48; c0 += 16) {
        tc_ld16(tm + ((uint32_t)(quarter * 32) << 16) + c0, h);
#pragma unroll
        for (int j = 0; j < 16; j++)
          if (c0 + j < 81) stg[lane * 81 + c0 + j] = h[j];
      }
    }
    __syncthreads();
    // pointwise, item (element le, point q): Jacobian, stress, TH; the element energy TH . Hh
    float th[kTcItems][9];
#pragma unroll
    for (int k = 0; k < kTcItems; k++) {
#pragma unroll
      for (int m = 0; m < 9; m++) th[k][m] = 0.f;
      const int it = tid + k * kTcThreads;
      if (it >= kTcEl * 27) continue;
      const int le = it / 27, q = it % 27;
      if (e0 + le >= n) continue;
      const int rq = le / kTcElW, rl = 3 * (le % kTcElW);
      const float *srow = (const float *)(sm + OFF_A2H + rq * 4 * 24 * 128);
      float hh[3][3];
#pragma unroll
      for (int s2 = 0; s2 < 3; s2++)
#pragma unroll
        for (int j = 0; j < 3; j++) hh[s2][j] = srow[(rl + s2) * 81 + q * 3 + j];
      const float lam = lm[2 * le], mu = lm[2 * le + 1];
      const float *ce = cx + le * 24;
      const float *ge = (const float *)(sm + OFF_GEO) + le * 10;
      float ji[3][3], det;
      if (ge[9] > 0.f) {  // affine element: the constant Jacobian of the records
#pragma unroll
        for (int m = 0; m < 9; m++) ji[m / 3][m % 3] = ge[m];
        det = ge[9];
      } else {
        float a[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
        for (int c = 0; c < 8; c++)
#pragma unroll
          for (int j = 0; j < 3; j++)
#pragma unroll
            for (int d = 0; d < 3; d++) a[j][d] += ce[c * 3 + j] * cg[(q * 3 + d) * 8 + c];
        det = -a[0][2] * a[1][1] * a[2][0] + a[0][1] * a[1][2] * a[2][0] + a[0][2] * a[1][0] * a[2][1] -
              a[0][0] * a[1][2] * a[2][1] - a[0][1] * a[1][0] * a[2][2] + a[0][0] * a[1][1] * a[2][2];
        const float id = 1.f / det;
        ji[0][0] = (-a[1][2] * a[2][1] + a[1][1] * a[2][2]) * id;
        ji[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * id;
        ji[0][2] = (-a[0][2] * a[1][1] + a[0][1] * a[1][2]) * id;
        ji[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) * id;
        ji[1][1] = (-a[0][2] * a[2][0] + a[0][0] * a[2][2]) * id;
        ji[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * id;
        ji[2][0] = (-a[1][1] * a[2][0] + a[1][0] * a[2][1]) * id;
        ji[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * id;
        ji[2][2] = (-a[0][1] * a[1][0] + a[0][0] * a[1][1]) * id;
      }
      float H[3][3];
#pragma unroll
      for (int s2 = 0; s2 < 3; s2++)
#pragma unroll
        for (int d = 0; d < 3; d++) H[s2][d] = hh[s2][0] * ji[0][d] + hh[s2][1] * ji[1][d] + hh[s2][2] * ji[2][d];
      const float wd = sw[q] * fabsf(det);
      const float lt = lam * (H[0][0] + H[1][1] + H[2][2]);
      float e_q = 0.f;
#pragma unroll
      for (int s2 = 0; s2 < 3; s2++) {
        float T[3];
#pragma unroll
        for (int d = 0; d < 3; d++) T[d] = wd * (mu * (H[s2][d] + H[d][s2]) + (s2 == d ? lt : 0.f));
#pragma unroll
        for (int j = 0; j < 3; j++) {
          const float t = T[0] * ji[j][0] + T[1] * ji[j][1] + T[2] * ji[j][2];
          th[k][s2 * 3 + j] = t;
          e_q += t * hh[s2][j];
        }
      }
      en.add(e_q);
    }
    __syncthreads();  // all staging reads done before A2 is overwritten
#pragma unroll
    for (int k = 0; k < kTcItems; k++) {
      const int it = tid + k * kTcThreads;
      if (it >= kTcEl * 27) continue;
      const int le = it / 27, q = it % 27;
      const int r0 = (le / kTcElW) * 32 + 3 * (le % kTcElW);
#pragma unroll
      for (int s2 = 0; s2 < 3; s2++)
#pragma unroll
        for (int j = 0; j < 3; j++) st_split(sm + OFF_A2H, sm + OFF_A2L, kmaj(r0 + s2, q * 3 + j, 96), th[k][s2 * 3 + j]);
    }
    // K padding (columns 81..95) of the element rows, and the two padding rows of each quarter, are zero
    for (int t = tid; t < 128 * 15; t += kTcThreads) {
      const int r = t / 15, c = 81 + t % 15;
      st_split(sm + OFF_A2H, sm + OFF_A2L, kmaj(r, c, 96), 0.f);
    }
    for (int t = tid; t < 4 * 2 * 81; t += kTcThreads) {
      const int r = (t / 162) * 32 + 30 + (t / 81) % 2, c = t % 81;
      st_split(sm + OFF_A2H, sm + OFF_A2L, kmaj(r, c, 96), 0.f);
    }
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (tid == 0) {
      for (int k = 0; k < 12; k++) {
        const uint64_t ah = tc_desc(a2h + k * 256, 3072), al = tc_desc(a2l + k * 256, 3072);
        const uint64_t bh = tc_desc(b2h + k * 256, 3072), bl = tc_desc(b2l + k * 256, 3072);
        tc_mma(tm + 128, ah, bh, id2, k > 0);
        tc_mma(tm + 128, ah, bl, id2, 1u);
        tc_mma(tm + 128, al, bh, id2, 1u);
      }
      tc_commit(&s_mb[1]);
    }
    // the next tile's nodal values go into U while the phase-2 MMAs run (they read A2 / B2 only)
    if ((tile + gridDim.x) * kTcEl < n) tc_gather(sm, (tile + gridDim.x) * kTcEl, n, rows, p4, rxyz, rlm, rgeo, tid);
    ok = tc_wait(&s_mb[1], parity);
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    // results: rows -> staging -> one float4 atomic per (element, shape)
    float *st1 = (float *)(sm + OFF_ST1);
    {
      float y[16];
      tc_ld16(tm + ((uint32_t)(quarter * 32) << 16) + 128 + 16 * half, y);
#pragma unroll
      for (int j = 0; j < 16; j++) st1[(quarter * 32 + lane) * 32 + 16 * half + j] = y[j];
    }
    __syncthreads();
    for (int t = tid; t < kTcEl * 27; t += kTcThreads) {
      const int le = t / 27, a = t % 27;
      const int64_t e = e0 + le;
      if (e >= n) continue;
      const int r0 = (le / kTcElW) * 32 + 3 * (le % kTcElW);
      const float4 v = make_float4(st1[(r0 + 0) * 32 + a], st1[(r0 + 1) * 32 + a], st1[(r0 + 2) * 32 + a], 0.f);
      red_add_f4(&q4[rows[e * 27 + a]], v);
    }
    parity ^= 1u;
  }
  if (failed) {
    if (tid == 0) atomicOr(err, 8192);
    // let the MMAs in flight finish (bounded) before the accumulators are released
    tc_wait(&s_mb[0], parity);
    tc_wait(&s_mb[1], parity);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(256));
  double v[1] = {failed ? 0.0 : en.get()}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    const double pq = tot[0] + (face_energy ? *face_energy : 0.0);
    R.scal[S_PQ] = pq;
    R.scal[S_ALPHA] = R.scal[S_RHO] / pq;
    R.iscal[I_SP32]++;
  }
}


// ---------------------------------------------------------------- shared element matrix on the tensor cores
// When every volume element has the same affine Jacobian (a uniform grid: the
// elements differ by a translation) and one Poisson ratio, every element
// matrix is one matrix scaled by the element's shear modulus, K_e = mu_e Khat
// (TPZElasticity3D's C1, C2, C3 are all proportional to E).  The operator over
// a tile of 128 elements is then one product
//   Y[e][n] = sum_k U[e][k] Khat[n][k],   k, n = 3 a + s (shape a, component s),
// with U the elements' gathered coefficients: tcgen05.mma kind::tf32 with the
// 3xTF32 split (hi.hi + hi.lo + lo.hi, FP32 accumulation in TMEM), M = 128
// elements, N = 96 (81 rows), K = 88 (81 columns), both operands K-major
// without swizzle.
//
// The work is gathers of p and float4 atomics into q (the MMAs take ~1 us of a
// tile's time), so the CTA (one per SM, persistent over tiles) is split into
// two groups of 8 warps that run a two-stage pipeline:
//   gatherers: copy the tile's block rows into shared memory (one coalesced
//     13.8 KB block: the row array is padded to whole tiles), gather U (thread t
//     takes shapes [0, 12) or [12, 27) of element t mod 128), split it hi / lo
//     into the A operand, and one thread issues the MMAs of tile k into TMEM
//     accumulator pair k mod 2 and commits them to mma_done[k mod 2];
//   scatterers: copy the same rows into their own buffer, wait for
//     mma_done, read their lane quarter's results (warp w: elements
//     32 (w mod 4) + lane, columns [0, 48) or [48, 96)), add mu_e Y[e] to q
//     with float4 atomics, accumulate the element energy mu_e Y[e] . U[e]
//     (p . q) and arrive on tmem_free[k mod 2].
// Gathering tile k + 1 overlaps the scattering of tile k; the A operand is
// rewritten only after mma_done of the previous tile, an accumulator pair only
// after tmem_free of the tile two back.  Every wait is bounded: a timeout sets
// a shared abort flag that ends every other wait, the groups leave their loops
// together (votes over named barriers), the MMAs in flight are waited for
// (bounded), the TMEM is freed and an error flag recorded.
constexpr int kGmThreads = 512;             // 8 gatherer + 8 scatterer warps
constexpr int kGmGroup = 256;
constexpr int kGmEl = 128;                  // elements per tile (MMA M)
constexpr int kGmK = 88, kGmN = 96;         // padded K (81) and N (81)
constexpr int kGmSplit = 12;                // gather: shapes [0, 12) by group threads 0..127, [12, 27) by 128..255
constexpr uint32_t kGmSmall = 128;          // TMEM column offset of the correction accumulator
constexpr int64_t kTlMaxNc = 3000;          // largest coarse system of the two-level preconditioner
constexpr uint32_t kGmB = kGmN * kGmK * 4, kGmA = kGmEl * kGmK * 4, kGmR = kGmEl * kNS * 4;
constexpr uint32_t GM_BH = 0, GM_BL = kGmB, GM_AH = 2 * kGmB, GM_AL = 2 * kGmB + kGmA;
constexpr uint32_t GM_RG = 2 * kGmB + 2 * kGmA, GM_RS = GM_RG + kGmR, GM_END = GM_RS + kGmR;
static_assert(GM_AH % 1024 == 0 && GM_AL % 1024 == 0 && GM_RG % 16 == 0 && kGmR % 16 == 0, "operand alignment");
static_assert(GM_END <= 227 * 1024, "shared memory");

__device__ __forceinline__ float4 tf32_split4(float4 v, float4 &lo) {
  float4 h;
  h.x = tf32_rna(v.x);
  h.y = tf32_rna(v.y);
  h.z = tf32_rna(v.z);
  h.w = tf32_rna(v.w);
  lo.x = tf32_rna(v.x - h.x);
  lo.y = tf32_rna(v.y - h.y);
  lo.z = tf32_rna(v.z - h.z);
  lo.w = tf32_rna(v.w - h.w);
  return h;
}

// barrier `id` over n threads; true in every participant when v is true in all
__device__ __forceinline__ bool gm_vote(int id, int n, bool v) {
  uint32_t r;
  asm volatile("{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.and.pred p, %2, %3, q;\nselp.u32 %0, 1, 0, p;\n}\n"
               : "=r"(r)
               : "r"((uint32_t)v), "r"(id), "r"(n)
               : "memory");
  return r != 0;
}
__device__ __forceinline__ void gm_bar(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }

// bounded wait on an mbarrier phase that also ends when another thread has aborted
__device__ __forceinline__ bool gm_wait(uint64_t *mb, uint32_t parity, volatile int *abort) {
  for (int it = 0; it < kTcWaitTries; it++) {
    if (mb_test(mb, parity)) return true;
    if (*abort) return false;
    if (it > 16) __nanosleep(64);
  }
  *abort = 1;
  return false;
}

// a streamed 16-byte load that does not allocate in L1 (the L1 left beside the
// operands keeps the gathered p values instead)
__device__ __forceinline__ int4 ld_stream4(const int4 *p) {
  int4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

// the tile's block rows [128][27] into shared memory (coalesced; padded tiles)
__device__ __forceinline__ void gm_rows(unsigned char *dst, const int4 *__restrict__ rows4, int64_t tile, int gl) {
  constexpr int n4 = (int)(kGmR / 16);
  const int4 *src = rows4 + (size_t)tile * n4;
#pragma unroll
  for (int i = gl; i < n4; i += kGmGroup) ((int4 *)dst)[i] = ld_stream4(src + i);
}

// Half of one element's row of U: shapes [A0, A1) -> columns [3 A0, 3 A1),
// the last half also writes the zero padding up to K.  Rows of padding
// elements (-1) are zero.
template <int A0, int A1>
__device__ __forceinline__ void gm_gather(unsigned char *sm, const int32_t *rw, int le, const float4 *__restrict__ p4) {
  constexpr int NA = A1 - A0, K0 = 3 * A0, K1 = A1 == kNS ? kGmK : 3 * A1, NV = K1 - K0;
  static_assert(K0 % 4 == 0 && NV % 4 == 0, "16-byte chunks");
  float v[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) v[k] = 0.f;
#pragma unroll
  for (int a = 0; a < NA; a++) {
    const int32_t r = rw[le * kNS + A0 + a];
    const float4 pv = r >= 0 ? p4[r] : make_float4(0.f, 0.f, 0.f, 0.f);
    v[3 * a] = pv.x;
    v[3 * a + 1] = pv.y;
    v[3 * a + 2] = pv.z;
  }
  if (A0 == 0) {
    // Khat annihilates translations (the eight corner shapes sum to one, the others vanish at the
    // corners): subtracting corner 0's value from the corner coefficients leaves Y unchanged and
    // makes the TF32 split's error relative to the element's variation instead of its mean, so smooth
    // fields (where the element contributions nearly cancel) keep FP32 accuracy
    static_assert(A1 >= 8, "the first half holds the eight corner shapes");
    const float c0 = v[0], c1 = v[1], c2 = v[2];
#pragma unroll
    for (int a = 0; a < 8; a++) {
      v[3 * a] -= c0;
      v[3 * a + 1] -= c1;
      v[3 * a + 2] -= c2;
    }
  }
#pragma unroll
  for (int c = 0; c < NV / 4; c++) {
    float4 lo;
    const float4 hi = tf32_split4(make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]), lo);
    const uint32_t off = kmaj(le, K0 + 4 * c, kGmK);
    *(float4 *)(sm + GM_AH + off) = hi;
    *(float4 *)(sm + GM_AL + off) = lo;
  }
}

// Half of one element's results: TMEM columns [C0, C0 + 48) of the warp's
// lane quarter (lane = element), shapes [A0, A1), read 16 columns at a time
// (a shape whose three columns straddle two reads takes the last two of the
// previous one); the p loads of a read's shapes are issued together.
template <int C0, int A0, int A1>
__device__ __forceinline__ void gm_scatter(uint32_t taddr, int64_t e, bool valid, const int32_t *rw, int le,
                                           const float *__restrict__ rlm, const float4 *__restrict__ p4,
                                           float4 *__restrict__ q4, KSum &en) {
  const float mu = valid ? rlm[2 * e + 1] : 0.f;
  float prev[2] = {0.f, 0.f};
#pragma unroll
  for (int c = 0; c < 48; c += 16) {
    float t[16], u[16];
    tc_ld16(taddr + C0 + c, t);
    tc_ld16(taddr + kGmSmall + C0 + c, u);
#pragma unroll
    for (int j = 0; j < 16; j++) t[j] += u[j];
    if (valid) {
      int32_t r[A1 - A0];
      float4 pv[A1 - A0];
#pragma unroll
      for (int a = A0; a < A1; a++) {
        const int j2 = 3 * a + 2 - C0;  // the shape's last column: handled in the read that holds it
        if (j2 >= c && j2 < c + 16) {
          r[a - A0] = rw[le * kNS + a];
          pv[a - A0] = p4[r[a - A0]];
        }
      }
#pragma unroll
      for (int a = A0; a < A1; a++) {
        const int j0 = 3 * a - C0, j2 = j0 + 2;
        if (j2 >= c && j2 < c + 16) {
          float yc[3];
#pragma unroll
          for (int d = 0; d < 3; d++) yc[d] = j0 + d >= c ? t[j0 + d - c] : prev[j0 + d - c + 2];
          const float4 yv = make_float4(mu * yc[0], mu * yc[1], mu * yc[2], 0.f);
          en.add(yv.x * pv[a - A0].x + yv.y * pv[a - A0].y + yv.z * pv[a - A0].z);
          red_add_f4(&q4[r[a - A0]], yv);
        }
      }
    }
    prev[0] = t[14];
    prev[1] = t[15];
  }
}

// hi.hi into the accumulator at column tm, the correction products hi.lo + lo.hi
// into their own accumulator at tm + kGmSmall: summed at their own scale, they
// are not rounded against the large hi.hi sums (the epilogue adds the two)
__device__ __forceinline__ void gm_mma(uint32_t tm, uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl) {
  const uint32_t id = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kGmN >> 3) << 17) | ((uint32_t)(kGmEl >> 4) << 24);
  constexpr uint32_t sbo = (kGmK / 4) * 128;
#pragma unroll 1
  for (int k = 0; k < kGmK / 8; k++) {
    const uint64_t dah = tc_desc(ah + k * 256, sbo), dal = tc_desc(al + k * 256, sbo);
    const uint64_t dbh = tc_desc(bh + k * 256, sbo), dbl = tc_desc(bl + k * 256, sbo);
    tc_mma(tm + kGmSmall, dal, dbh, id, k > 0);
    tc_mma(tm + kGmSmall, dah, dbl, id, 1u);
    tc_mma(tm, dah, dbh, id, k > 0);
  }
}

// rows: [ntile * 128][27] block rows, -1 past the n elements
__global__ void __launch_bounds__(kGmThreads, 1) k_mf_hex27_gm(int64_t n, const int32_t *__restrict__ rows,
                                                               const float *__restrict__ rlm,
                                                               const float4 *__restrict__ bsplit,
                                                               const float4 *__restrict__ p4, float4 *__restrict__ q4,
                                                               const double *__restrict__ face_energy,
                                                               int *__restrict__ err, Red R) {
  if (!active(R.iscal)) return;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;
  __shared__ __align__(8) uint64_t s_done[2], s_free[2];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool gatherer = tid < kGmGroup;
  const int gl = tid & (kGmGroup - 1);
  const int4 *rows4 = (const int4 *)rows;
  // Khat hi / lo, already in the operand layout
  for (uint32_t i = tid; i < 2 * kGmB / 16; i += kGmThreads) ((float4 *)(sm + GM_BH))[i] = bsplit[i];
  asm volatile("fence.proxy.async.shared::cta;");  // B is read by the MMAs (async proxy)
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&s_tmem)), "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    s_abort = 0;
    for (int b = 0; b < 2; b++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&s_done[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(&s_free[b])), "r"(kGmGroup));
    }
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tm = s_tmem;
  const uint32_t ah = tc_smem(sm + GM_AH), al = tc_smem(sm + GM_AL), bh = tc_smem(sm + GM_BH),
                 bl = tc_smem(sm + GM_BL);
  const int64_t ntile = (n + kGmEl - 1) / kGmEl;
  KSum en;
  int last = -1;  // the issuer's last committed tile
  if (gatherer) {
    const int le = gl & (kGmEl - 1), half = gl >> 7;
    const int32_t *rw = (const int32_t *)(sm + GM_RG);
    int k = 0;
    for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x, k++) {
      const int b = k & 1;
      gm_rows(sm + GM_RG, rows4, tile, gl);  // the previous tile's rows were last read before its MMA issue
      bool ok = true;
      if (gl == 0 && k >= 2) ok = gm_wait(&s_free[b], (uint32_t)((k - 2) >> 1) & 1u, &s_abort);
      if (ok && k >= 1) ok = gm_wait(&s_done[(k - 1) & 1], (uint32_t)((k - 1) >> 1) & 1u, &s_abort);
      if (!gm_vote(1, kGmGroup, ok)) break;  // also orders the row copies before their reads
      if (half == 0) gm_gather<0, kGmSplit>(sm, rw, le, p4);
      else gm_gather<kGmSplit, kNS>(sm, rw, le, p4);
      asm volatile("fence.proxy.async.shared::cta;");
      gm_bar(1, kGmGroup);
      if (gl == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        gm_mma(tm + (uint32_t)b * 256u, ah, al, bh, bl);
        tc_commit(&s_done[b]);
        last = k;
      }
    }
  } else {
    const int sw = warp - kGmGroup / 32, quarter = sw & 3, half = sw >> 2, le = quarter * 32 + lane;
    const int32_t *rw = (const int32_t *)(sm + GM_RS);
    int k = 0;
    for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x, k++) {
      const int b = k & 1;
      gm_rows(sm + GM_RS, rows4, tile, gl);
      const bool ok = gm_wait(&s_done[b], (uint32_t)(k >> 1) & 1u, &s_abort);
      if (!gm_vote(2, kGmGroup, ok)) break;  // uniform exit; orders the row copies before their reads
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int64_t e = tile * kGmEl + le;
      const uint32_t taddr = tm + ((uint32_t)(quarter * 32) << 16) + (uint32_t)b * 256u;
      if (half == 0) gm_scatter<0, 0, 16>(taddr, e, e < n, rw, le, rlm, p4, q4, en);
      else gm_scatter<48, 16, kNS>(taddr, e, e < n, rw, le, rlm, p4, q4, en);
      asm volatile("tcgen05.fence::before_thread_sync;");
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc_smem(&s_free[b])) : "memory");
      gm_bar(2, kGmGroup);  // the rows buffer is rewritten next
    }
  }
  __syncthreads();
  const bool failed = s_abort != 0;
  if (failed && tid == 0) {
    atomicOr(err, 16384);
    // the MMAs in flight write the accumulators: let them finish (bounded) before the TMEM is released
    if (last >= 0) tc_wait(&s_done[last & 1], (uint32_t)(last >> 1) & 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(512));
  double v[1] = {failed ? 0.0 : en.get()}, tot[1];
  if (grid_reduce<1, kGmThreads / 32>(v, R, tot) && threadIdx.x == 0) {
    const double pq = tot[0] + (face_energy ? *face_energy : 0.0);
    R.scal[S_PQ] = pq;
    R.scal[S_ALPHA] = R.scal[S_RHO] / pq;
    R.iscal[I_SP32]++;
  }
}

// ---------------------------------------------------------------- the same operator over lattice tiles
// On a grid whose elements are translates of one element along three lattice
// vectors (element e's corner 0 at x0 + i a1 + j a2 + k a3) every Q2 connect
// sits at a point of the doubled lattice (2i + ox, 2j + oy, 2k + oz), ox, oy,
// oz in {0, 1, 2} by side.  A CTA then takes blocks of 8 x 8 x 2 elements (one
// M = 128 tile of the Khat GEMM): a block's 17 x 17 x 5 connect values are read
// once into shared memory and the A operand is built from them; the results are
// added into a shared-memory tile with shared-memory atomics, and the connects
// strictly inside the block, which belong to no other block, are written with
// plain stores, those on its faces (and those on penalty faces, which the face
// kernel has already added into q) with vector reductions.  Per element that is
// ~11 global reads and ~6 global writes instead of the 27 gathers and 27
// reductions of k_mf_hex27_gm; the MMAs, the 3xTF32 split and the translation
// subtraction are the same.  Like k_mf_hex27_gm the CTA runs two warp groups
// in a two-stage pipeline over blocks:
//   loaders (warps 0..7): the block's connect values (loaded into registers
//     while the previous block's MMAs ran) into shared memory, the A rows, the
//     MMAs into TMEM accumulator pair k mod 2, committed to mma_done;
//   writers (warps 8..15): wait for mma_done, add mu_e Y into result tile
//     k mod 2, release the accumulators (tmem_free), then write the block out;
//     p . q is summed there as sum over the block's connects of p_n . y_n.
// Waits are bounded and end together on a shared abort flag, as in k_mf_hex27_gm.
constexpr int kGtThreads = 512;  // 8 loader + 8 writer warps
constexpr int kGtGroup = 256;
constexpr int kGtTx = 8, kGtTy = 8, kGtTz = 2;  // elements per block (8 x 8 x 2 = 128 = one tile)
constexpr int kGtNx = 2 * kGtTx + 1, kGtNy = 2 * kGtTy + 1, kGtNz = 2 * kGtTz + 1;
constexpr int kGtNodes = kGtNx * kGtNy * kGtNz;  // 1445
constexpr int kGtPre = (kGtNodes + kGtGroup - 1) / kGtGroup;  // connects per group thread
// shared-memory tiles: one plane per component, slot (x / 2 + (x odd) 9) + 20 (y + 17 z): the 32 lanes of a
// warp (elements (lx, ly) of one layer, one shape) then hit 32 distinct banks
constexpr int kGtP = 20, kGtSlots = kGtP * kGtNy * kGtNz;            // 1700 slots per plane
constexpr uint32_t kGtYt = 3 * kGtSlots * 4;                          // one tile: float [3][kGtSlots]
constexpr uint32_t GT_UT = 2 * kGmB + 2 * kGmA;                       // the connect values
constexpr uint32_t GT_YT = GT_UT + kGtYt;                             // two result tiles
constexpr uint32_t GT_MU = GT_YT + 2 * kGtYt;                         // float [2][128] mu of the blocks' elements
constexpr uint32_t GT_END = GT_MU + 2 * kGmEl * 4;
static_assert(GT_UT % 16 == 0 && GT_END <= 225 * 1024, "shared memory");
static_assert(kGtTx * kGtTy * kGtTz == kGmEl, "one tile per block");

static_assert(kNS == 27, "GtArgs holds 27 shapes");

__device__ __forceinline__ int gt_slot(int x, int y, int z) { return (x >> 1) + (x & 1) * 9 + kGtP * (y + kGtNy * z); }

struct GtBlock {
  int tx, ty, tz, ex, ey, ez;  // block position, elements present per direction
};
__device__ __forceinline__ GtBlock gt_block(const GtArgs &G, int64_t tile) {
  GtBlock b;
  b.tx = (int)(tile % G.ntx);
  b.ty = (int)((tile / G.ntx) % G.nty);
  b.tz = (int)(tile / ((int64_t)G.ntx * G.nty));
  b.ex = min(kGtTx, G.mx - kGtTx * b.tx);
  b.ey = min(kGtTy, G.my - kGtTy * b.ty);
  b.ez = min(kGtTz, G.mz - kGtTz * b.tz);
  return b;
}
// block row of connect n of a block (-1: none)
__device__ __forceinline__ int32_t gt_row(const GtArgs &G, const GtBlock &b, const int32_t *__restrict__ nmap, int n) {
  const int x = n % kGtNx, y = (n / kGtNx) % kGtNy, z = n / (kGtNx * kGtNy);
  if (n >= kGtNodes || x > 2 * b.ex || y > 2 * b.ey || z > 2 * b.ez) return -1;
  const int64_t NX = 2 * G.mx + 1, NY = 2 * G.my + 1;
  return nmap[(2 * kGtTx * b.tx + x) + NX * ((2 * kGtTy * b.ty + y) + NY * (int64_t)(2 * kGtTz * b.tz + z))];
}

// nmap: [(2 mx + 1)(2 my + 1)(2 mz + 1)] block row of each lattice connect (-1: none);
// emu: [mx my mz] mu of the element at each lattice cell (-1: none); face: [block rows] 1 on penalty faces
struct GtFaces {  // the penalty faces, applied by the same CTAs before the blocks (k_mf_faces' work)
  int64_t n;
  const float *rxyz, *phi, *dphi, *w;
  const int32_t *rows;
  float big;
};

__global__ void __launch_bounds__(kGtThreads, 1) k_mf_hex27_gt(GtArgs G, const int32_t *__restrict__ nmap,
                                                               const float *__restrict__ emu,
                                                               const uint8_t *__restrict__ face,
                                                               const float4 *__restrict__ bsplit,
                                                               const float4 *__restrict__ p4, float4 *__restrict__ q4,
                                                               GtFaces F, int *__restrict__ err, Red R) {
  if (!active(R.iscal)) return;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;
  __shared__ __align__(8) uint64_t s_done[2], s_free[2];
  __shared__ int8_t s_off[kNS][3];
  __shared__ float s_fphi[kFQ * kFS], s_fd[kFQ * 2 * kFS], s_fw[kFQ];
  __shared__ float s_fu[kGtThreads / 32][kFS][4], s_fc[kGtThreads / 32][12], s_ft[kGtThreads / 32][kFQ][4];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool loader = tid < kGtGroup;
  const int gl = tid & (kGtGroup - 1);
  float *ut = (float *)(sm + GT_UT);
  if (tid == 0) {  // constant indices: the kernel parameter is not copied to local memory
#pragma unroll
    for (int a = 0; a < kNS; a++)
#pragma unroll
      for (int r = 0; r < 3; r++) s_off[a][r] = G.off[a][r];
  }
  for (uint32_t i = tid; i < 2 * kGmB / 16; i += kGtThreads) ((float4 *)(sm + GM_BH))[i] = bsplit[i];
  for (uint32_t i = tid; i < 2 * kGtYt / 4; i += kGtThreads) ((float *)(sm + GT_YT))[i] = 0.f;
  asm volatile("fence.proxy.async.shared::cta;");
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&s_tmem)), "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    s_abort = 0;
    for (int b = 0; b < 2; b++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&s_done[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(&s_free[b])), "r"(kGtGroup));
    }
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  for (int k = tid; k < kFQ * kFS; k += kGtThreads) s_fphi[k] = F.phi[k];
  for (int k = tid; k < kFQ * 2 * kFS; k += kGtThreads) s_fd[k] = F.dphi[k];
  if (tid < kFQ) s_fw[tid] = F.w[tid];
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tm = s_tmem;
  const uint32_t ah = tc_smem(sm + GM_AH), al = tc_smem(sm + GM_AL), bh = tc_smem(sm + GM_BH),
                 bl = tc_smem(sm + GM_BL);
  const int64_t ntile = (int64_t)G.ntx * G.nty * G.ntz;
  KSum en;
  // the penalty faces (their connects are written by the blocks with reductions, never with plain stores)
  for (int64_t i = (int64_t)blockIdx.x * (kGtThreads / 32) + warp; i < F.n; i += (int64_t)gridDim.x * (kGtThreads / 32))
    mf_face(i, lane, s_fphi, s_fd, s_fw, s_fu[warp], s_fc[warp], s_ft[warp], F.big, F.rxyz, F.rows, p4, q4, en);
  int last = -1;  // the issuer's last committed block
  if (loader) {
    int32_t pbr[kGtPre];
    float4 pval[kGtPre];
    float pmu = 0.f;
    auto fetch = [&](int64_t tile) {
      const GtBlock b = gt_block(G, tile);
#pragma unroll
      for (int i = 0; i < kGtPre; i++) pbr[i] = gt_row(G, b, nmap, gl + i * kGtGroup);
#pragma unroll
      for (int i = 0; i < kGtPre; i++) pval[i] = pbr[i] >= 0 ? p4[pbr[i]] : make_float4(0.f, 0.f, 0.f, 0.f);
      pmu = 0.f;
      if (gl < kGmEl) {
        const int lx = gl % kGtTx, ly = (gl / kGtTx) % kGtTy, lz = gl / (kGtTx * kGtTy);
        if (lx < b.ex && ly < b.ey && lz < b.ez)
          pmu = emu[(int64_t)(kGtTx * b.tx + lx) + (int64_t)G.mx * ((kGtTy * b.ty + ly) + (int64_t)G.my * (kGtTz * b.tz + lz))];
      }
    };
    if (blockIdx.x < ntile) fetch(blockIdx.x);
    int k = 0;
    for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x, k++) {
      const int bf = k & 1;
      bool ok = true;
      if (gl == 0 && k >= 2) ok = gm_wait(&s_free[bf], (uint32_t)((k - 2) >> 1) & 1u, &s_abort);
      if (ok && k >= 1) ok = gm_wait(&s_done[(k - 1) & 1], (uint32_t)((k - 1) >> 1) & 1u, &s_abort);  // A free
      if (!gm_vote(1, kGtGroup, ok)) break;
      // the block's values (the previous block's A rows, the only reader of ut, are built)
#pragma unroll
      for (int i = 0; i < kGtPre; i++) {
        const int n = gl + i * kGtGroup;
        if (n < kGtNodes) {
          const int sl = gt_slot(n % kGtNx, (n / kGtNx) % kGtNy, n / (kGtNx * kGtNy));
          ut[sl] = pval[i].x;
          ut[kGtSlots + sl] = pval[i].y;
          ut[2 * kGtSlots + sl] = pval[i].z;
        }
      }
      if (gl < kGmEl) ((float *)(sm + GT_MU))[bf * kGmEl + gl] = pmu > 0.f ? pmu : 0.f;
      gm_bar(1, kGtGroup);
      {
        // A rows: thread (element le, half): shapes [0, kGmSplit) with the translation removed, or the rest
        const int le = gl & (kGmEl - 1), half = gl >> 7;
        const int lx = le % kGtTx, ly = (le / kGtTx) % kGtTy, lz = le / (kGtTx * kGtTy);
        const bool live = ((const float *)(sm + GT_MU))[bf * kGmEl + le] > 0.f;
        auto gather = [&](auto A0c, auto A1c) {
          constexpr int A0 = decltype(A0c)::value, A1 = decltype(A1c)::value;
          constexpr int K0 = 3 * A0, K1 = A1 == kNS ? kGmK : 3 * A1, NV = K1 - K0;
          float v[NV];
#pragma unroll
          for (int kk = 0; kk < NV; kk++) v[kk] = 0.f;
          if (live) {
#pragma unroll
            for (int a = A0; a < A1; a++) {
              const int sl = gt_slot(2 * lx + s_off[a][0], 2 * ly + s_off[a][1], 2 * lz + s_off[a][2]);
              v[3 * (a - A0)] = ut[sl];
              v[3 * (a - A0) + 1] = ut[kGtSlots + sl];
              v[3 * (a - A0) + 2] = ut[2 * kGtSlots + sl];
            }
          }
          if (A0 == 0) {  // Khat annihilates translations: corner 0's value off the corner coefficients
            const float c0 = v[0], c1 = v[1], c2 = v[2];
#pragma unroll
            for (int a = 0; a < 8; a++) {
              v[3 * a] -= c0;
              v[3 * a + 1] -= c1;
              v[3 * a + 2] -= c2;
            }
          }
#pragma unroll
          for (int c4 = 0; c4 < NV / 4; c4++) {
            float4 lo;
            const float4 hi = tf32_split4(make_float4(v[4 * c4], v[4 * c4 + 1], v[4 * c4 + 2], v[4 * c4 + 3]), lo);
            const uint32_t off = kmaj(le, K0 + 4 * c4, kGmK);
            *(float4 *)(sm + GM_AH + off) = hi;
            *(float4 *)(sm + GM_AL + off) = lo;
          }
        };
        if (half == 0) gather(std::integral_constant<int, 0>(), std::integral_constant<int, kGmSplit>());
        else gather(std::integral_constant<int, kGmSplit>(), std::integral_constant<int, kNS>());
      }
      asm volatile("fence.proxy.async.shared::cta;");
      gm_bar(1, kGtGroup);
      if (gl == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        gm_mma(tm + (uint32_t)bf * 256u, ah, al, bh, bl);
        tc_commit(&s_done[bf]);
        last = k;
      }
      if (tile + gridDim.x < ntile) fetch(tile + gridDim.x);  // in flight during the MMAs
    }
  } else {
    const int sw = warp - kGtGroup / 32, quarter = sw & 3, h = sw >> 2, le = quarter * 32 + lane;
    const int lx = le % kGtTx, ly = (le / kGtTx) % kGtTy, lz = le / (kGtTx * kGtTy);
    // the block's connect rows (bit 30: on a penalty face) and p values for the write-out and p . q, loaded
    // for the next block while this one's MMAs and results are waited for
    int32_t br[kGtPre];
    float4 pv[kGtPre];
    auto fetch = [&](int64_t tile) {
      const GtBlock b = gt_block(G, tile);
#pragma unroll
      for (int i = 0; i < kGtPre; i++) br[i] = gt_row(G, b, nmap, gl + i * kGtGroup);
#pragma unroll
      for (int i = 0; i < kGtPre; i++) {
        pv[i] = br[i] >= 0 ? p4[br[i]] : make_float4(0.f, 0.f, 0.f, 0.f);
        if (br[i] >= 0 && face[br[i]]) br[i] |= 1 << 30;
      }
    };
    if (blockIdx.x < ntile) fetch(blockIdx.x);
    int k = 0;
    for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x, k++) {
      const int bf = k & 1;
      float *yt = (float *)(sm + GT_YT + bf * kGtYt);
      const bool ok = gm_wait(&s_done[bf], (uint32_t)(k >> 1) & 1u, &s_abort);
      if (!gm_vote(2, kGtGroup, ok)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      {
        // warp w reads its lane quarter (element 32 (w mod 4) + lane), columns [48 h, 48 h + 48) = shapes
        // [16 h, 16 h + 16), and adds mu_e Y into result tile k mod 2
        const uint32_t taddr = tm + ((uint32_t)(quarter * 32) << 16) + (uint32_t)bf * 256u + (uint32_t)(48 * h);
        float y[48];
#pragma unroll
        for (int c = 0; c < 48; c += 16) {
          float t[16], u[16];
          tc_ld16(taddr + c, t);
          tc_ld16(taddr + kGmSmall + c, u);
#pragma unroll
          for (int j = 0; j < 16; j++) y[c + j] = t[j] + u[j];
        }
        const float mu = ((const float *)(sm + GT_MU))[bf * kGmEl + le];
        if (mu > 0.f) {
#pragma unroll
          for (int j = 0; j < 16; j++) {
            const int a = 16 * h + j;
            if (a < kNS) {
              const int sl = gt_slot(2 * lx + s_off[a][0], 2 * ly + s_off[a][1], 2 * lz + s_off[a][2]);
              atomicAdd(&yt[sl], mu * y[3 * j]);
              atomicAdd(&yt[kGtSlots + sl], mu * y[3 * j + 1]);
              atomicAdd(&yt[2 * kGtSlots + sl], mu * y[3 * j + 2]);
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc_smem(&s_free[bf])) : "memory");
      gm_bar(2, kGtGroup);
      // the block into q (plain stores strictly inside, reductions on its faces and on penalty faces); p . q
      const GtBlock b = gt_block(G, tile);
#pragma unroll
      for (int i = 0; i < kGtPre; i++) {
        const int n = gl + i * kGtGroup;
        if (br[i] < 0) continue;
        const int x = n % kGtNx, y = (n / kGtNx) % kGtNy, z = n / (kGtNx * kGtNy);
        const int sl = gt_slot(x, y, z);
        const int32_t r = br[i] & ~(1 << 30);
        const float4 v = make_float4(yt[sl], yt[kGtSlots + sl], yt[2 * kGtSlots + sl], 0.f);
        yt[sl] = yt[kGtSlots + sl] = yt[2 * kGtSlots + sl] = 0.f;  // for block k + 2 (after the writers' next vote)
        en.add(v.x * pv[i].x + v.y * pv[i].y + v.z * pv[i].z);
        const bool inside = x > 0 && x < 2 * b.ex && y > 0 && y < 2 * b.ey && z > 0 && z < 2 * b.ez && !(br[i] & (1 << 30));
        if (inside) q4[r] = v;
        else red_add_f4(&q4[r], v);
      }
      if (tile + gridDim.x < ntile) fetch(tile + gridDim.x);
    }
  }
  __syncthreads();
  const bool failed = s_abort != 0;
  if (failed && tid == 0) {
    atomicOr(err, 16384);
    if (last >= 0) tc_wait(&s_done[last & 1], (uint32_t)(last >> 1) & 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(512));
  double v[1] = {failed ? 0.0 : en.get()}, tot[1];
  if (grid_reduce<1, kGtThreads / 32>(v, R, tot) && threadIdx.x == 0) {
    const double pq = tot[0];
    R.scal[S_PQ] = pq;
    R.scal[S_ALPHA] = R.scal[S_RHO] / pq;
    R.iscal[I_SP32]++;
  }
}

// lattice position of each volume element's corner 0: t = Ainv (x - x0), integer to 1e-6
__global__ void k_gt_lattice(int64_t n, const int64_t *__restrict__ elems, const int64_t *__restrict__ el_nodes,
                             const double *__restrict__ xyz, double x0, double y0, double z0, const double *__restrict__ ainv,
                             int32_t *__restrict__ lat, int *__restrict__ lmm, int *__restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t node = el_nodes[elems[i] * 8];
  const double d[3] = {xyz[node * 3] - x0, xyz[node * 3 + 1] - y0, xyz[node * 3 + 2] - z0};
  for (int r = 0; r < 3; r++) {
    const double t = ainv[3 * r] * d[0] + ainv[3 * r + 1] * d[1] + ainv[3 * r + 2] * d[2];
    const long long li = llround(t);
    if (fabs(t - (double)li) > 1e-6 || li < -(1ll << 20) || li > (1ll << 20)) atomicOr(flag, 1);
    lat[i * 3 + r] = (int)li;
    atomicMin(&lmm[r], (int)li);
    atomicMax(&lmm[3 + r], (int)li);
  }
}

// the connect map of the doubled lattice and the elements' mu per lattice cell; flag 2 when two elements
// share a cell, one lattice point gets two connects or one connect two lattice points (its block's plain
// stores would then not be the only writes of that connect)
__global__ void k_gt_maps(int64_t n, const int32_t *__restrict__ lat, const int32_t *__restrict__ rows,
                          const float *__restrict__ rlm, GtArgs G, int lx0, int ly0, int lz0, int32_t *__restrict__ nmap,
                          float *__restrict__ emu, int32_t *__restrict__ owner, int *__restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int I = lat[i * 3] - lx0, J = lat[i * 3 + 1] - ly0, K = lat[i * 3 + 2] - lz0;
  const int64_t cell = (int64_t)I + (int64_t)G.mx * (J + (int64_t)G.my * K);
  if (atomicCAS((int *)&emu[cell], __float_as_int(-1.f), __float_as_int(rlm[2 * i + 1])) != __float_as_int(-1.f))
    atomicOr(flag, 2);
  const int NX = 2 * G.mx + 1, NY = 2 * G.my + 1;
  for (int a = 0; a < kNS; a++) {
    const int32_t r = rows[i * kNS + a];
    const int64_t idx = (int64_t)(2 * I + G.off[a][0]) + (int64_t)NX * ((2 * J + G.off[a][1]) + (int64_t)NY * (2 * K + G.off[a][2]));
    const int old = atomicCAS(&nmap[idx], -1, r);
    if (old != -1 && old != r) atomicOr(flag, 2);
    if (r >= 0) {
      const int ow = atomicCAS(&owner[r], -1, (int)idx);
      if (ow != -1 && ow != (int)idx) atomicOr(flag, 2);
    }
  }
}

__global__ void k_gt_faces(int64_t n, const int32_t *__restrict__ frows, uint8_t *__restrict__ face) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && frows[i] >= 0) face[frows[i]] = 1;
}

// The FP64 affine Jacobian of every volume element against element 0's: flag 1
// when one is not affine or differs (the shared element matrix does not apply);
// element 0's Jinv (row-major, Jinv[j][d] = d xi_j / d x_d) and |det J| to ref.
__device__ bool gm_affine(const int64_t *__restrict__ el_nodes, const double *__restrict__ xyz, int64_t e,
                          double (&a)[3][3], double &scale) {
  const signed char sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  double cx[8][3];
  for (int k = 0; k < 8; k++)
    for (int j = 0; j < 3; j++) cx[k][j] = xyz[el_nodes[e * 8 + k] * 3 + j];
  double hi = 0.0, big = 0.0;
  for (int j = 0; j < 3; j++) {
    double t4 = 0, t5 = 0, t6 = 0, t7 = 0, mn = cx[0][j], mx = cx[0][j];
    for (int k = 0; k < 8; k++) {
      const double x = cx[k][j];
      t4 += sg[k][0] * sg[k][1] * x;
      t5 += sg[k][0] * sg[k][2] * x;
      t6 += sg[k][1] * sg[k][2] * x;
      t7 += sg[k][0] * sg[k][1] * sg[k][2] * x;
      mn = fmin(mn, x);
      mx = fmax(mx, x);
    }
    hi = fmax(hi, fmax(fmax(fabs(t4), fabs(t5)), fmax(fabs(t6), fabs(t7))));
    big = fmax(big, mx - mn);
    for (int d = 0; d < 3; d++) {
      double t = 0.0;
      for (int k = 0; k < 8; k++) t += sg[k][d] * cx[k][j];
      a[j][d] = t / 8.0;
    }
  }
  scale = big;
  return hi <= 1e-12 * big;
}

__global__ void k_mf_uniform(int64_t n, const int64_t *__restrict__ elems, const int64_t *__restrict__ el_nodes,
                             const double *__restrict__ xyz, double *__restrict__ ref, int *__restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a0[3][3], a[3][3], s0, s;
  const bool aff0 = gm_affine(el_nodes, xyz, elems[0], a0, s0);
  const bool aff = gm_affine(el_nodes, xyz, elems[i], a, s);
  bool same = aff0 && aff;
  for (int j = 0; j < 3; j++)
    for (int d = 0; d < 3; d++) same = same && fabs(a[j][d] - a0[j][d]) <= 1e-12 * s0;
  if (!same) atomicOr(flag, 1);
  if (i == 0 && aff0) {
    const double det = -a0[0][2] * a0[1][1] * a0[2][0] + a0[0][1] * a0[1][2] * a0[2][0] +
                       a0[0][2] * a0[1][0] * a0[2][1] - a0[0][0] * a0[1][2] * a0[2][1] -
                       a0[0][1] * a0[1][0] * a0[2][2] + a0[0][0] * a0[1][1] * a0[2][2];
    const double id = 1.0 / det;
    ref[0] = (-a0[1][2] * a0[2][1] + a0[1][1] * a0[2][2]) * id;
    ref[1] = (a0[0][2] * a0[2][1] - a0[0][1] * a0[2][2]) * id;
    ref[2] = (-a0[0][2] * a0[1][1] + a0[0][1] * a0[1][2]) * id;
    ref[3] = (a0[1][2] * a0[2][0] - a0[1][0] * a0[2][2]) * id;
    ref[4] = (-a0[0][2] * a0[2][0] + a0[0][0] * a0[2][2]) * id;
    ref[5] = (a0[0][2] * a0[1][0] - a0[0][0] * a0[1][2]) * id;
    ref[6] = (-a0[1][1] * a0[2][0] + a0[1][0] * a0[2][1]) * id;
    ref[7] = (a0[0][1] * a0[2][0] - a0[0][0] * a0[2][1]) * id;
    ref[8] = (-a0[0][1] * a0[1][0] + a0[0][0] * a0[1][1]) * id;
    ref[9] = fabs(det);
  }
}


// ---------------------------------------------------------------- two-level preconditioner: set-up kernels
// hex corner k at lattice offset (kOffX[k], kOffY[k], kOffZ[k]) from corner 0
__constant__ int c_tlOff[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

// lattice coordinates of every volume element's corner 0 relative to element
// 0's (box size h); lmm[0..2] min, lmm[3..5] max over all corners; err bit
// 1 << 17 when a corner is off the lattice
__global__ void k_tl_lattice(int64_t n, const int64_t *__restrict__ elems, const int64_t *__restrict__ el_nodes,
                             const double *__restrict__ xyz, double x0, double y0, double z0, double hx, double hy,
                             double hz, int32_t *__restrict__ lat, int *__restrict__ lmm, int *__restrict__ err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t e = elems[i];
  const double o[3] = {x0, y0, z0}, h[3] = {hx, hy, hz};
  int l0[3] = {0, 0, 0};
  for (int k = 0; k < 8; k++) {
    const int64_t node = el_nodes[e * 8 + k];
    for (int d = 0; d < 3; d++) {
      const double t = (xyz[node * 3 + d] - o[d]) / h[d];
      const long long li = llround(t);
      if (fabs(t - (double)li) > 1e-6 || li < -(1ll << 30) || li > (1ll << 30)) atomicOr(err, 1 << 17);
      if (k == 0) l0[d] = (int)li;
      else if ((int)li - l0[d] != c_tlOff[k][d]) atomicOr(err, 1 << 17);
      atomicMin(&lmm[d], (int)li);
      atomicMax(&lmm[3 + d], (int)li);
    }
  }
  for (int d = 0; d < 3; d++) lat[i * 3 + d] = l0[d];
}

// vertex map, coarse box and sub position of every volume element
__global__ void k_tl_vertices(int64_t n, const int64_t *__restrict__ elems, const int64_t *__restrict__ el_conn,
                              const int64_t *__restrict__ bpos, const int32_t *__restrict__ lat, int mx, int my, int mz,
                              int lx0, int ly0, int lz0, int nvx, int nvy, int s, int mcx, int mcy,
                              int32_t *__restrict__ vtx_eq, int32_t *__restrict__ el_cell, int32_t *__restrict__ el_sub) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t e = elems[i];
  const int a = lat[i * 3] - mx, b = lat[i * 3 + 1] - my, c = lat[i * 3 + 2] - mz;
  for (int k = 0; k < 8; k++) {
    const int64_t v = (int64_t)(a + c_tlOff[k][0]) + (int64_t)nvx * ((b + c_tlOff[k][1]) + (int64_t)nvy * (c + c_tlOff[k][2]));
    vtx_eq[v] = (int32_t)bpos[el_conn[e * 27 + k]];
  }
  const int I = a / s, J = b / s, K = c / s;
  el_cell[i] = I + mcx * (J + mcy * K);
  el_sub[i] = (a - I * s) + s * ((b - J * s) + s * (c - K * s));
  (void)lx0; (void)ly0; (void)lz0;
}

__global__ void k_tl_browvtx(int64_t nv, const int32_t *__restrict__ vtx_eq, int32_t *__restrict__ brow_vtx) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int32_t eq = vtx_eq[v];
  if (eq >= 0) brow_vtx[eq / 3] = (int32_t)v;
}

// coarse nodes whose trilinear function is nonzero at a vertex of a penalty face
__global__ void k_tl_fixnodes(int64_t n, const int64_t *__restrict__ elems, const int64_t *__restrict__ el_conn,
                              const int64_t *__restrict__ bpos, const int32_t *__restrict__ brow_vtx, int nvx, int nvy,
                              int s, int mcx, int mcy, int mcz, int32_t *__restrict__ cfix) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t e = elems[i];
  for (int k = 0; k < 4; k++) {
    const int32_t v = brow_vtx[bpos[el_conn[e * 27 + k]] / 3];
    if (v < 0) continue;
    const int vi = v % nvx, vj = (v / nvx) % nvy, vk = v / (nvx * nvy);
    const int I = min(vi / s, mcx - 1), J = min(vj / s, mcy - 1), K = min(vk / s, mcz - 1);
    const int ri = vi - I * s, rj = vj - J * s, rk = vk - K * s;
    for (int cn = 0; cn < 8; cn++) {
      const int bx = c_tlOff[cn][0], by = c_tlOff[cn][1], bz = c_tlOff[cn][2];
      const bool nz = (bx ? ri > 0 : ri < s) && (by ? rj > 0 : rj < s) && (bz ? rk > 0 : rk < s);
      if (nz) cfix[(I + bx) + (mcx + 1) * ((J + by) + (mcy + 1) * (K + bz))] = 1;
    }
  }
}

// coarse box matrices sum_e mu_e T[sub_e], scattered into the dense coarse matrix
__global__ void __launch_bounds__(256) k_tl_cells(const int32_t *__restrict__ cell_off,
                                                  const int32_t *__restrict__ cell_el,
                                                  const int32_t *__restrict__ el_sub, const int64_t *__restrict__ elems,
                                                  const double *__restrict__ coef, double E0, double mufac,
                                                  const double *__restrict__ tsub, int mcx, int mcy, int64_t nc,
                                                  double *__restrict__ ac) {
  const int cell = blockIdx.x;
  const int I = cell % mcx, J = (cell / mcx) % mcy, K = cell / (mcx * mcy);
  for (int t = threadIdx.x; t < 576; t += blockDim.x) {
    double acc = 0.0;
    for (int32_t k = cell_off[cell]; k < cell_off[cell + 1]; k++) {
      const int32_t i = cell_el[k];
      const double mu = (coef ? coef[elems[i]] : E0) * mufac;
      acc += mu * tsub[(size_t)el_sub[i] * 576 + t];
    }
    const int r = t / 24, c = t % 24;  // (coarse corner, component)
    const int rn = r / 3, rs = r % 3, cn = c / 3, cs = c % 3;
    const int64_t nr = (I + c_tlOff[rn][0]) + (int64_t)(mcx + 1) * ((J + c_tlOff[rn][1]) + (int64_t)(mcy + 1) * (K + c_tlOff[rn][2]));
    const int64_t ncn = (I + c_tlOff[cn][0]) + (int64_t)(mcx + 1) * ((J + c_tlOff[cn][1]) + (int64_t)(mcy + 1) * (K + c_tlOff[cn][2]));
    atomicAdd(&ac[(3 * nr + rs) * nc + 3 * ncn + cs], acc);
  }
}

// removed coarse nodes: zero row and column, unit diagonal
__global__ void k_tl_fixrows(int64_t nc, const int32_t *__restrict__ cfix, double *__restrict__ ac) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc * nc) return;
  const int64_t i = t / nc, j = t % nc;
  if (cfix[i / 3] || cfix[j / 3]) ac[t] = i == j ? 1.0 : 0.0;
}

// Blocked in-place Gauss-Jordan inversion of the SPD coarse matrix (no
// pivoting), in the element type T (the set-up runs it in FP32), pivot blocks of kGjB rows.  With A = [[D, R], [C, E]] for
// the current pivot block D: D <- P = D^-1 (k_gj_diag), R <- P R (k_gj_row),
// E <- E - C (P R) (k_gj_trail, with the original C), C <- -C P (k_gj_col).
constexpr int kGjB = 32;

// P = D^-1 of the pivot block, Gauss-Jordan in shared memory by one CTA
template <class T>
__global__ void __launch_bounds__(256) k_gj_diag(int64_t n, int64_t k0, T *__restrict__ A, int *__restrict__ err) {
  __shared__ T D[kGjB][kGjB + 1];
  const int b = (int)min((int64_t)kGjB, n - k0);
  for (int t = threadIdx.x; t < b * b; t += blockDim.x) D[t / b][t % b] = A[(k0 + t / b) * n + k0 + t % b];
  __syncthreads();
  for (int k = 0; k < b; k++) {
    const T piv = D[k][k];
    if (threadIdx.x == 0 && !(piv > T(0))) atomicOr(err, 1 << 18);
    const T ip = T(1) / piv;
    __syncthreads();
    if (threadIdx.x < b) D[k][threadIdx.x] = (threadIdx.x == k ? T(1) : D[k][threadIdx.x]) * ip;
    __syncthreads();
    for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
      const int i = t / b, j = t % b;
      if (i == k) continue;
      const T f = D[i][k];
      // every thread reads D[i][k] before any writes it: the column k entries are written last, below
      if (j != k) D[i][j] -= f * D[k][j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < b; i += blockDim.x)
      if (i != k) D[i][k] = -D[i][k] * D[k][k];
    __syncthreads();
  }
  for (int t = threadIdx.x; t < b * b; t += blockDim.x) A[(k0 + t / b) * n + k0 + t % b] = D[t / b][t % b];
}

// R <- P R: row panel (rows k0.., the columns outside the block), one thread per column
template <class T>
__global__ void __launch_bounds__(256) k_gj_row(int64_t n, int64_t k0, T *__restrict__ A) {
  __shared__ T P[kGjB][kGjB];
  const int b = (int)min((int64_t)kGjB, n - k0);
  for (int t = threadIdx.x; t < b * b; t += blockDim.x) P[t / b][t % b] = A[(k0 + t / b) * n + k0 + t % b];
  __syncthreads();
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n || (j >= k0 && j < k0 + b)) return;
  T r[kGjB];
  for (int t = 0; t < b; t++) r[t] = A[(k0 + t) * n + j];
  for (int i = 0; i < b; i++) {
    T acc = T(0);
    for (int t = 0; t < b; t++) acc += P[i][t] * r[t];
    A[(k0 + i) * n + j] = acc;
  }
}

// E <- E - C R' over 64 x 64 tiles of the matrix outside the pivot rows and columns (R' = the updated
// row panel, C = the column panel not updated yet); each thread a 4 x 4 sub-tile
template <class T>
__global__ void __launch_bounds__(256) k_gj_trail(int64_t n, int64_t k0, T *__restrict__ A) {
  __shared__ T Cs[64][kGjB + 1], Rs[kGjB][64 + 1];
  const int b = (int)min((int64_t)kGjB, n - k0);
  const int64_t i0 = (int64_t)blockIdx.y * 64, j0 = (int64_t)blockIdx.x * 64;
  for (int t = threadIdx.x; t < 64 * kGjB; t += blockDim.x) {
    const int r = t / kGjB, c = t % kGjB;
    Cs[r][c] = (i0 + r < n && c < b) ? A[(i0 + r) * n + k0 + c] : T(0);
  }
  for (int t = threadIdx.x; t < kGjB * 64; t += blockDim.x) {
    const int r = t / 64, c = t % 64;
    Rs[r][c] = (r < b && j0 + c < n) ? A[(k0 + r) * n + j0 + c] : T(0);
  }
  __syncthreads();
  const int ti = (threadIdx.x / 16) * 4, tj = (threadIdx.x % 16) * 4;
  T acc[4][4] = {};
  for (int t = 0; t < b; t++)
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
      for (int v = 0; v < 4; v++) acc[u][v] += Cs[ti + u][t] * Rs[t][tj + v];
#pragma unroll
  for (int u = 0; u < 4; u++)
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const int64_t i = i0 + ti + u, j = j0 + tj + v;
      if (i >= n || j >= n || (i >= k0 && i < k0 + b) || (j >= k0 && j < k0 + b)) continue;
      A[i * n + j] -= acc[u][v];
    }
}

// C <- -C P: column panel (rows outside the block, columns k0..), one thread per row
template <class T>
__global__ void __launch_bounds__(256) k_gj_col(int64_t n, int64_t k0, T *__restrict__ A) {
  __shared__ T P[kGjB][kGjB];
  const int b = (int)min((int64_t)kGjB, n - k0);
  for (int t = threadIdx.x; t < b * b; t += blockDim.x) P[t / b][t % b] = A[(k0 + t / b) * n + k0 + t % b];
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || (i >= k0 && i < k0 + b)) return;
  T c[kGjB];
  for (int t = 0; t < b; t++) c[t] = A[i * n + k0 + t];
  for (int j = 0; j < b; j++) {
    T acc = T(0);
    for (int t = 0; t < b; t++) acc += c[t] * P[t][j];
    A[i * n + k0 + j] = -acc;
  }
}

// B = the symmetrised FP32 copy of the FP64 n x n matrix A
__global__ void k_tl_sym32(int64_t n, const double *__restrict__ A, float *__restrict__ B) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * n) return;
  const int64_t i = t / n, j = t % n;
  B[t] = (float)(0.5 * (A[i * n + j] + A[j * n + i]));
}

// B[i][j] (rows of ldc floats, zero past column n) = the symmetrised A (n x n, FP32)
__global__ void k_tl_pad32(int64_t n, int64_t ldc, const float *__restrict__ A, float *__restrict__ B) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * ldc) return;
  const int64_t i = t / ldc, j = t % ldc;
  B[t] = j < n ? 0.5f * (A[i * n + j] + A[j * n + i]) : 0.f;
}

template <class K>
int mf_grid(K kernel, int threads) {
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
  // grid_reduce's partial-sum buffer holds kGridBlocks CTAs
  return std::max(1, std::min(kGridBlocks, nsm * std::max(per, 1)));
}

}  // namespace

// Tables of the sum-factorised operator for the volume bucket: Phi at the
// Lagrange nodes (-1, 0, 1)^3 from the bucket's own shape functions, the 1D
// Lagrange values and derivatives at the rule's 1D Gauss points, the weights
// and the corner-shape gradients.  Built in FP64 and checked: the factorised
// gradients must reproduce the bucket's table at every point (1e-10), else
// the variant is not offered.
bool sf_tables(Ctx &c, const Bucket &vol) {
  const BucketKey &k = vol.key;
  std::vector<double> g1, w1;
  gauss_rule(GPZ_EL_LINE, k.intorder, g1, w1);
  if ((int)g1.size() != 3) return false;
  const double node[3] = {-1.0, 0.0, 1.0};
  auto lag = [&](int j, double x) {
    return j == 0 ? 0.5 * x * (x - 1.0) : j == 1 ? 1.0 - x * x : 0.5 * x * (x + 1.0);
  };
  auto dlag = [&](int j, double x) { return j == 0 ? x - 0.5 : j == 1 ? -2.0 * x : x + 0.5; };
  double Bd[3][3], Dd[3][3];
  for (int q = 0; q < 3; q++)
    for (int j = 0; j < 3; j++) {
      Bd[q][j] = lag(j, g1[q]);
      Dd[q][j] = dlag(j, g1[q]);
    }
  double phi[kMaxShapes], dph[3 * kMaxShapes];
  std::vector<double> P((size_t)kNQ * kNS);
  for (int j = 0; j < kNQ; j++) {
    const double pt[3] = {node[j % 3], node[(j / 3) % 3], node[j / 9]};
    if (eval_shapes(k.type, k.orders, k.trans, pt, phi, dph, kMaxShapes) != kNS) return false;
    for (int a = 0; a < kNS; a++) P[j * kNS + a] = std::fabs(phi[a]) > 1e-13 ? phi[a] : 0.0;
  }
  // the factorised reference gradients reproduce the table
  double worst = 0.0, scale = 0.0;
  for (int q = 0; q < kNQ; q++) {
    const int q1 = q % 3, q2 = (q / 3) % 3, q3 = q / 9;
    for (int a = 0; a < kNS; a++) {
      double g[3] = {0.0, 0.0, 0.0};
      for (int j = 0; j < kNQ; j++) {
        const int j1 = j % 3, j2 = (j / 3) % 3, j3 = j / 9;
        const double pa = P[j * kNS + a];
        if (pa == 0.0) continue;
        g[0] += pa * Dd[q1][j1] * Bd[q2][j2] * Bd[q3][j3];
        g[1] += pa * Bd[q1][j1] * Dd[q2][j2] * Bd[q3][j3];
        g[2] += pa * Bd[q1][j1] * Bd[q2][j2] * Dd[q3][j3];
      }
      for (int d = 0; d < 3; d++) {
        const double t = vol.dphi[((size_t)q * 3 + d) * kNS + a];
        worst = std::max(worst, std::fabs(g[d] - t));
        scale = std::max(scale, std::fabs(t));
      }
    }
  }
  if (!(worst <= 1e-10 * scale)) return false;
  std::vector<float> tf(SF_NF, 0.f);
  std::vector<int> ti(SFI_NI, 0);
  for (int q = 0; q < 3; q++)
    for (int j = 0; j < 3; j++) {
      tf[SF_B + q * 3 + j] = (float)Bd[q][j];
      tf[SF_D + q * 3 + j] = (float)Dd[q][j];
    }
  for (int q = 0; q < kNQ; q++) {
    tf[SF_W + q] = (float)vol.w[q];
    for (int d = 0; d < 3; d++)
      for (int kk = 0; kk < 8; kk++) tf[SF_DC + q * 24 + d * 8 + kk] = (float)vol.dphi[((size_t)q * 3 + d) * kNS + kk];
  }
  // rows of <= 9 nonzeros by their lane; at most one longer row, summed across the warp
  int jl = -1, nr = 0, nc = 0;
  for (int j = 0; j < kNQ; j++) {
    int len = 0;
    for (int a = 0; a < kNS; a++) len += P[j * kNS + a] != 0.0;
    if (len > 9) {
      if (jl >= 0) return false;
      jl = j;
    }
  }
  if (jl < 0) jl = 0;  // every row short: row 0 goes the warp-sum way
  for (int a = 0; a < kNS; a++) {
    int len = 0;
    for (int j = 0; j < kNQ; j++) len += P[j * kNS + a] != 0.0;
    if (len > 8) return false;  // the kernel keeps <= 8 entries of a column in registers
  }
  for (int j = 0; j < kNQ; j++) {
    ti[SFI_RP + j] = nr;
    if (j == jl) continue;
    for (int a = 0; a < kNS; a++)
      if (P[j * kNS + a] != 0.0) {
        if (nr >= kSfMaxNz) return false;
        ti[SFI_RC + nr] = a;
        tf[SF_RV + nr++] = (float)P[j * kNS + a];
      }
  }
  ti[SFI_RP + kNQ] = nr;
  for (int a = 0; a < kNS; a++) tf[SF_LONG + a] = (float)P[jl * kNS + a];
  for (int a = 0; a < kNS; a++) {
    ti[SFI_CP + a] = nc;
    for (int j = 0; j < kNQ; j++)
      if (P[j * kNS + a] != 0.0) {
        if (nc >= kSfMaxNz) return false;
        ti[SFI_CR + nc] = j;
        tf[SF_CV + nc++] = (float)P[j * kNS + a];
      }
  }
  ti[SFI_CP + kNS] = nc;
  ti[SFI_LONG] = jl;
  c.mf.sf_tab.upload(tf.data(), tf.size(), c.stream);
  c.mf.sf_idx.upload(ti.data(), ti.size(), c.stream);
  // B and D depend only on the 3-point rule: the same values for every context
  GPZ_CUDA_TRY(cudaMemcpyToSymbolAsync(c_sfB, tf.data() + SF_B, 9 * sizeof(float), 0, cudaMemcpyHostToDevice, c.stream));
  GPZ_CUDA_TRY(cudaMemcpyToSymbolAsync(c_sfD, tf.data() + SF_D, 9 * sizeof(float), 0, cudaMemcpyHostToDevice, c.stream));
  GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
  return true;
}

// TF32 (10-bit mantissa) rounding to nearest, ties away from zero: the value
// cvt.rna.tf32.f32 gives, on the host
static float tf32_round_host(float x) {
  uint32_t b;
  std::memcpy(&b, &x, 4);
  if ((b & 0x7f800000u) != 0x7f800000u) b = (b + 0x1000u) & ~0x1fffu;
  float r;
  std::memcpy(&r, &b, 4);
  return r;
}

// The element matrix of a Q2 hex elasticity element for mu = 1 (E = 2 + 2 nu,
// TPZElasticity3D's CODE3 coefficients C1 = 1, C2, C3), from the bucket's
// reference Gram and the element's constant Jinv / |det J| (ref[0..9]): the
// formula of the FP64 affine assembly.  K[(3 a + s) * 81 + 3 b + t].
static void khat_elasticity(const Bucket &vol, const double *ref, double nu, std::vector<double> &K) {
  const double E = 2.0 + 2.0 * nu;
  const double C1 = E / (2. + 2. * nu), C2 = E * nu / (-1. + nu + 2. * nu * nu),
               C3 = E * (nu - 1.) / (-1. + nu + 2. * nu * nu);
  double ji[3][3];
  for (int k = 0; k < 9; k++) ji[k / 3][k % 3] = ref[k];
  const double det = ref[9];
  K.assign((size_t)81 * 81, 0.0);
  for (int a = 0; a < kNS; a++)
    for (int b = 0; b < kNS; b++) {
      const double *G = vol.ghat.data() + ((size_t)a * kNS + b) * 9;
      double M1[3][3], S[3][3];
      for (int i = 0; i < 3; i++)
        for (int e2 = 0; e2 < 3; e2++) M1[i][e2] = G[i * 3 + 0] * ji[0][e2] + G[i * 3 + 1] * ji[1][e2] + G[i * 3 + 2] * ji[2][e2];
      for (int d = 0; d < 3; d++)
        for (int e2 = 0; e2 < 3; e2++) S[d][e2] = det * (ji[0][d] * M1[0][e2] + ji[1][d] * M1[1][e2] + ji[2][d] * M1[2][e2]);
      const double tr = S[0][0] + S[1][1] + S[2][2];
      for (int si = 0; si < 3; si++)
        for (int t = 0; t < 3; t++)
          K[(size_t)(3 * a + si) * 81 + 3 * b + t] =
              si == t ? (tr - S[si][si]) * C1 + S[si][si] * C3 : S[t][si] * C1 - S[si][t] * C2;
    }
}

// The shared element matrix of a uniform volume bucket: every element's FP64
// affine Jacobian is checked against element 0's on the device; when they all
// agree, Khat (the element matrix for mu = 1, i.e. E = 2 + 2 nu) is formed in
// FP64 from the bucket's reference Gram with TPZElasticity3D's CODE3
// coefficients, as the FP64 assembly forms affine element matrices, and
// uploaded split into TF32 hi / lo in the K-major operand layout.
static bool gm_tables(Ctx &c, const Bucket &vol, double nu) {
  MatFree &M = c.mf;
  if (vol.ghat.empty() || vol.nshape != kNS) return false;
  cudaStream_t s = c.stream;
  M.gm_ref.alloc(10);
  M.gm_flag.alloc(1);
  M.gm_flag.zero(s);
  M.gm_ref.zero(s);
  k_mf_uniform<<<grid_for(M.nvol, 256), 256, 0, s>>>(M.nvol, vol.d_elems.p, c.d_el_nodes.p, c.d_xyz.p, M.gm_ref.p,
                                                      M.gm_flag.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  int flag = 0;
  double ref[10];
  GPZ_CUDA_TRY(cudaMemcpyAsync(&flag, M.gm_flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(ref, M.gm_ref.p, sizeof(ref), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  if (flag != 0 || !(ref[9] > 0.0)) return false;
  std::vector<double> K;
  khat_elasticity(vol, ref, nu, K);
  std::vector<float> hl(2 * kGmB / 4, 0.f);
  for (int nn = 0; nn < 81; nn++)
    for (int k = 0; k < 81; k++) {
      const double v = K[(size_t)nn * 81 + k];
      const float hi = tf32_round_host((float)v);
      const float lo = tf32_round_host((float)(v - (double)hi));
      const uint32_t off = kmaj(nn, k, kGmK) / 4;
      hl[off] = hi;
      hl[kGmB / 4 + off] = lo;
    }
  M.gm_b.upload(hl.data(), hl.size(), s);
  GPZ_CUDA_TRY(cudaFuncSetAttribute(k_mf_hex27_gm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GM_END));
  int dev = 0, nsm = 0;
  GPZ_CUDA_TRY(cudaGetDevice(&dev));
  GPZ_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  M.grid_gm = std::max(1, std::min(kGridBlocks, nsm));  // one CTA per SM, persistent over tiles
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  return true;
}

// The lattice maps of the tiled operator (k_mf_hex27_gt): false when the
// translated elements do not fill a lattice of their edge vectors
// a1 = x1 - x0, a2 = x3 - x0, a3 = x4 - x0 (corner numbering of TPZGeoCube).
static bool gt_build(Ctx &c, const Bucket &vol) {
  MatFree &M = c.mf;
  M.gt_ready = false;
  cudaStream_t s = c.stream;
  const int64_t n = M.nvol;
  int64_t nd[8];
  GPZ_CUDA_TRY(cudaMemcpy(nd, c.d_el_nodes.p + vol.elems[0] * 8, sizeof(nd), cudaMemcpyDeviceToHost));
  double X[8][3];
  for (int k = 0; k < 8; k++) GPZ_CUDA_TRY(cudaMemcpy(X[k], c.d_xyz.p + nd[k] * 3, 3 * sizeof(double), cudaMemcpyDeviceToHost));
  double A[3][3];  // columns a1, a2, a3
  for (int r = 0; r < 3; r++) {
    A[r][0] = X[1][r] - X[0][r];
    A[r][1] = X[3][r] - X[0][r];
    A[r][2] = X[4][r] - X[0][r];
  }
  const double det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                     A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
  if (!(std::fabs(det) > 0.0)) return false;
  double inv[9];
  inv[0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) / det;
  inv[1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / det;
  inv[2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / det;
  inv[3] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / det;
  inv[4] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / det;
  inv[5] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / det;
  inv[6] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) / det;
  inv[7] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / det;
  inv[8] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / det;
  DBuf<double> dinv;
  DBuf<int32_t> lat;
  DBuf<int> lmm, flag;
  dinv.upload(inv, 9, s);
  lat.alloc((size_t)n * 3);
  lmm.alloc(6);
  flag.alloc(1);
  flag.zero(s);
  const int init[6] = {1 << 30, 1 << 30, 1 << 30, -(1 << 30), -(1 << 30), -(1 << 30)};
  GPZ_CUDA_TRY(cudaMemcpyAsync(lmm.p, init, sizeof(init), cudaMemcpyHostToDevice, s));
  k_gt_lattice<<<grid_for(n, 256), 256, 0, s>>>(n, vol.d_elems.p, c.d_el_nodes.p, c.d_xyz.p, X[0][0], X[0][1], X[0][2],
                                                dinv.p, lat.p, lmm.p, flag.p);
  c.launches++;
  int hm[6], hf = 0;
  GPZ_CUDA_TRY(cudaMemcpyAsync(hm, lmm.p, sizeof(hm), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(&hf, flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  if (hf) return false;
  GtArgs G{};
  G.mx = hm[3] - hm[0] + 1;
  G.my = hm[4] - hm[1] + 1;
  G.mz = hm[5] - hm[2] + 1;
  const int64_t ncell = (int64_t)G.mx * G.my * G.mz;
  const int64_t nnode = (int64_t)(2 * G.mx + 1) * (2 * G.my + 1) * (2 * G.mz + 1);
  if (ncell < n || ncell > 8 * n || nnode >= INT32_MAX) return false;  // a sparse lattice: the tiles would be mostly empty
  G.ntx = (G.mx + kGtTx - 1) / kGtTx;
  G.nty = (G.my + kGtTy - 1) / kGtTy;
  G.ntz = (G.mz + kGtTz - 1) / kGtTz;
  // shape a's connect: the mean of its side's corners on the doubled lattice
  static const int co[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  const ElemTopo &t = topo(GPZ_EL_HEX);
  for (int a = 0; a < kNS; a++) {
    const int sd = vol.shape_side[a];
    const int nn = t.side_nnode[sd];
    for (int r = 0; r < 3; r++) {
      int sum = 0;
      for (int k = 0; k < nn; k++) sum += 2 * co[t.side_node[sd][k]][r];
      if (sum % nn) return false;
      G.off[a][r] = (int8_t)(sum / nn);
    }
  }
  M.gt_nmap.alloc(nnode);
  GPZ_CUDA_TRY(cudaMemsetAsync(M.gt_nmap.p, 0xff, nnode * sizeof(int32_t), s));
  M.gt_emu.alloc(ncell);
  {
    std::vector<float> neg(ncell, -1.f);
    M.gt_emu.upload(neg.data(), neg.size(), s);
  }
  DBuf<int32_t> owner;
  owner.alloc(std::max<int64_t>(c.neq / 3, 1));
  GPZ_CUDA_TRY(cudaMemsetAsync(owner.p, 0xff, owner.n * sizeof(int32_t), s));
  k_gt_maps<<<grid_for(n, 256), 256, 0, s>>>(n, lat.p, M.vrows.p, M.vlm.p, G, hm[0], hm[1], hm[2], M.gt_nmap.p,
                                             M.gt_emu.p, owner.p, flag.p);
  c.launches++;
  M.gt_face.alloc(std::max<int64_t>(c.neq / 3, 1));
  M.gt_face.zero(s);
  if (M.nface) {
    k_gt_faces<<<grid_for(M.nface * kFS, 256), 256, 0, s>>>(M.nface * kFS, M.frows.p, M.gt_face.p);
    c.launches++;
  }
  GPZ_CUDA_TRY(cudaMemcpyAsync(&hf, flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  GPZ_CUDA_TRY(cudaGetLastError());
  if (hf) return false;
  M.gt = G;
  GPZ_CUDA_TRY(cudaFuncSetAttribute(k_mf_hex27_gt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GT_END));
  int dev = 0, nsm = 0;
  GPZ_CUDA_TRY(cudaGetDevice(&dev));
  GPZ_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  M.grid_gt = (int)std::max<int64_t>(1, std::min<int64_t>(std::min(kGridBlocks, nsm), (int64_t)G.ntx * G.nty * G.ntz));
  M.gt_ready = true;
  return true;
}

// ---------------------------------------------------------------- two-level preconditioner set-up
// Geometry part, once per mesh: the fine lattice of the uniform grid, the
// coarse boxes (s^3 elements each, about `target` boxes per direction), the
// vertex map, the coarse nodes touching penalty-Dirichlet equations, and the
// tables T[sub] = P_sub^T Khat_vv P_sub (mu = 1) of a fine element at each of
// the s^3 positions inside its coarse box.
int two_level_build(Ctx &c) {
  TwoLevel &T = c.tl;
  T.ready = false;
  T.have_inv = false;
  if (c.nstate != 3 || c.flt.active) return GPZ_E_INVALID;
  for (int32_t b : c.h_block_size)
    if (b != 0 && b != 3) return GPZ_E_INVALID;
  Bucket *vol = nullptr;
  std::vector<Bucket *> fixb;
  for (Bucket *b : c.buckets) {
    if (b->hp) return GPZ_E_INVALID;
    const int mi = c.h_el_mat[b->elems[0]];
    if (!b->key.is_bc) {
      if (vol || b->key.type != GPZ_EL_HEX || b->nshape != kNS || b->key.mat_kind != GPZ_MAT_ELAST3D ||
          b->ghat.empty())
        return GPZ_E_INVALID;
      vol = b;
    } else if (c.bcs[-mi - 1].type == 0) {
      if (b->key.type != GPZ_EL_QUAD) return GPZ_E_INVALID;
      fixb.push_back(b);
    }
  }
  if (!vol) return GPZ_E_INVALID;
  for (int k = 0; k < 8; k++)
    if (vol->shape_side[k] != k) return GPZ_E_INVALID;  // corner shapes first
  cudaStream_t s = c.stream;
  const int64_t n = (int64_t)vol->elems.size();
  // every element the same axis-aligned box
  DBuf<double> ref;
  DBuf<int> flag;
  ref.alloc(10);
  flag.alloc(1);
  ref.zero(s);
  flag.zero(s);
  k_mf_uniform<<<grid_for(n, 256), 256, 0, s>>>(n, vol->d_elems.p, c.d_el_nodes.p, c.d_xyz.p, ref.p, flag.p);
  c.launches++;
  double hr[10];
  int hf = 0;
  int64_t node0 = 0;
  GPZ_CUDA_TRY(cudaMemcpyAsync(hr, ref.p, sizeof(hr), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(&hf, flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(&node0, c.d_el_nodes.p + vol->elems[0] * 8, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  if (hf != 0 || !(hr[9] > 0.0)) return GPZ_E_INVALID;
  double jmax = 0.0;
  for (int k = 0; k < 9; k++) jmax = std::max(jmax, std::fabs(hr[k]));
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      if ((i != j && std::fabs(hr[i * 3 + j]) > 1e-12 * jmax) || (i == j && !(hr[i * 3 + j] > 0.0)))
        return GPZ_E_INVALID;
  double x0[3];
  GPZ_CUDA_TRY(cudaMemcpy(x0, c.d_xyz.p + node0 * 3, sizeof(x0), cudaMemcpyDeviceToHost));
  const double h[3] = {2.0 / hr[0], 2.0 / hr[4], 2.0 / hr[8]};  // J = h / 2 on the diagonal
  // lattice
  DBuf<int32_t> lat, cell;
  DBuf<int> lmm;
  lat.alloc((size_t)n * 3);
  cell.alloc((size_t)n);
  lmm.alloc(6);
  const int init[6] = {1 << 30, 1 << 30, 1 << 30, -(1 << 30), -(1 << 30), -(1 << 30)};
  GPZ_CUDA_TRY(cudaMemcpyAsync(lmm.p, init, sizeof(init), cudaMemcpyHostToDevice, s));
  k_tl_lattice<<<grid_for(n, 256), 256, 0, s>>>(n, vol->d_elems.p, c.d_el_nodes.p, c.d_xyz.p, x0[0], x0[1], x0[2],
                                                h[0], h[1], h[2], lat.p, lmm.p, c.d_err.p);
  c.launches++;
  int hm[6];
  GPZ_CUDA_TRY(cudaMemcpyAsync(hm, lmm.p, sizeof(hm), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  check_device_flag(c, "two-level lattice");
  int64_t g = 0;
  for (int d = 0; d < 3; d++) {
    T.lx[d] = hm[3 + d] - hm[d];
    if (T.lx[d] < 2) return GPZ_E_INVALID;
    g = std::__gcd<int64_t>(g, T.lx[d]);
  }
  // s divides every lx; pick the one whose smallest box count is closest to the target
  int best = -1;
  for (int64_t cand = 1; cand <= g; cand++) {
    if (g % cand) continue;
    const int64_t mmin = std::min(T.lx[0], std::min(T.lx[1], T.lx[2])) / cand;
    const int64_t nn = (T.lx[0] / cand + 1) * (T.lx[1] / cand + 1) * (T.lx[2] / cand + 1);
    if (mmin < 1 || 3 * nn > kTlMaxNc) continue;
    if (best < 0 || std::llabs(mmin - T.target) < std::llabs(std::min(T.lx[0], std::min(T.lx[1], T.lx[2])) / best - T.target))
      best = (int)cand;
  }
  if (best < 0) return GPZ_E_INVALID;
  T.s = best;
  for (int d = 0; d < 3; d++) T.m[d] = (int)(T.lx[d] / T.s);
  T.nnode = (int64_t)(T.m[0] + 1) * (T.m[1] + 1) * (T.m[2] + 1);
  T.nc = 3 * T.nnode;
  T.ncell = (int64_t)T.m[0] * T.m[1] * T.m[2];
  const int nvx = (int)T.lx[0] + 1, nvy = (int)T.lx[1] + 1;
  const int64_t nv = (int64_t)nvx * nvy * (T.lx[2] + 1);
  if (nv >= INT32_MAX) return GPZ_E_INVALID;  // the application kernels index the vertex lattice in 32 bits
  T.vtx_eq.alloc(nv);
  GPZ_CUDA_TRY(cudaMemsetAsync(T.vtx_eq.p, 0xff, nv * sizeof(int32_t), s));
  T.el_sub.alloc(n);
  k_tl_vertices<<<grid_for(n, 256), 256, 0, s>>>(n, vol->d_elems.p, c.d_el_conn.p, c.d_block_pos.p, lat.p, hm[0],
                                                 hm[1], hm[2], 0, 0, 0, nvx, nvy, T.s, T.m[0], T.m[1], T.vtx_eq.p,
                                                 cell.p, T.el_sub.p);
  c.launches++;
  const int64_t nbrow = c.neq / 3;
  T.brow_vtx.alloc(std::max<int64_t>(nbrow, 1));
  GPZ_CUDA_TRY(cudaMemsetAsync(T.brow_vtx.p, 0xff, T.brow_vtx.n * sizeof(int32_t), s));
  k_tl_browvtx<<<grid_for(nv, 256), 256, 0, s>>>(nv, T.vtx_eq.p, T.brow_vtx.p);
  c.launches++;
  T.cfix.alloc(T.nnode);
  T.cfix.zero(s);
  for (Bucket *b : fixb) {
    const int64_t nb = (int64_t)b->elems.size();
    k_tl_fixnodes<<<grid_for(nb, 256), 256, 0, s>>>(nb, b->d_elems.p, c.d_el_conn.p, c.d_block_pos.p, T.brow_vtx.p,
                                                    nvx, nvy, T.s, T.m[0], T.m[1], T.m[2], T.cfix.p);
    c.launches++;
  }
  // elements grouped by coarse box (counting sort on the host)
  std::vector<int32_t> hc(n), fixed(T.nnode);
  GPZ_CUDA_TRY(cudaMemcpyAsync(hc.data(), cell.p, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(fixed.data(), T.cfix.p, T.nnode * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  GPZ_CUDA_TRY(cudaGetLastError());
  std::vector<int32_t> off(T.ncell + 1, 0), el(n);
  for (int64_t i = 0; i < n; i++) off[hc[i] + 1]++;
  for (int64_t k = 0; k < T.ncell; k++) off[k + 1] += off[k];
  {
    std::vector<int32_t> fill(off.begin(), off.end() - 1);
    for (int64_t i = 0; i < n; i++) el[fill[hc[i]]++] = (int32_t)i;
  }
  T.nfixed = 0;
  for (int32_t f : fixed) T.nfixed += f != 0;
  T.cell_off.upload(off.data(), off.size(), s);
  T.cell_el.upload(el.data(), el.size(), s);
  // tables: fine corner k of the element at sub position (a, b, c) sits at (a, b, c) + off[k] in its coarse box
  std::vector<double> K;
  const gpz_material &mat = c.mats[c.h_el_mat[vol->elems[0]]];
  khat_elasticity(*vol, hr, mat.nu, K);
  T.mufac = 1.0 / (2.0 + 2.0 * mat.nu);
  T.E0 = mat.E;
  static const int off8[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  const int ss = T.s, nsub = ss * ss * ss;
  std::vector<double> tab((size_t)nsub * 576);
  for (int sub = 0; sub < nsub; sub++) {
    const int sa = sub % ss, sb = (sub / ss) % ss, sc = sub / (ss * ss);
    double W[8][8];  // fine corner k -> coarse corner cn
    for (int k = 0; k < 8; k++) {
      const double t[3] = {(double)(sa + off8[k][0]) / ss, (double)(sb + off8[k][1]) / ss,
                           (double)(sc + off8[k][2]) / ss};
      for (int cn = 0; cn < 8; cn++) {
        double w = 1.0;
        for (int d = 0; d < 3; d++) w *= off8[cn][d] ? t[d] : 1.0 - t[d];
        W[k][cn] = w;
      }
    }
    double *Tt = tab.data() + (size_t)sub * 576;
    for (int r = 0; r < 24; r++)
      for (int q = 0; q < 24; q++) {
        const int rn = r / 3, rs = r % 3, qn = q / 3, qs = q % 3;
        double acc = 0.0;
        for (int k = 0; k < 8; k++) {
          if (W[k][rn] == 0.0) continue;
          for (int kk = 0; kk < 8; kk++)
            acc += W[k][rn] * K[(size_t)(3 * k + rs) * 81 + 3 * kk + qs] * W[kk][qn];
        }
        Tt[r * 24 + q] = acc;
      }
  }
  T.tsub.upload(tab.data(), tab.size(), s);
  T.ac.alloc((size_t)T.nc * T.nc);
  T.ldc = (T.nc + 3) / 4 * 4;
  T.acinv32.alloc((size_t)T.nc * T.ldc);
  T.rc.alloc(T.nc);
  T.zc.alloc(T.nc);
  T.boxpart.alloc((size_t)T.ncell * 24);
  T.z32.alloc(std::max<int64_t>(c.neq, 1));
  T.rc.zero(s);
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  T.ready = true;
  return GPZ_OK;
}

// Coarse matrix of the current assembly (per coarse box sum_e mu_e T[sub_e], FP64),
// removed nodes, then its inverse by blocked in-place Gauss-Jordan on the
// symmetrised FP32 copy, padded rows for the coarse solve.
void two_level_assemble(Ctx &c) {
  TwoLevel &T = c.tl;
  cudaStream_t s = c.stream;
  Bucket *vol = nullptr;
  for (Bucket *b : c.buckets)
    if (!b->key.is_bc) vol = b;
  T.ac.zero(s);
  k_tl_cells<<<(unsigned)T.ncell, 256, 0, s>>>(T.cell_off.p, T.cell_el.p, T.el_sub.p, vol->d_elems.p, c.d_coef.p,
                                               T.E0, T.mufac, T.tsub.p, T.m[0], T.m[1], T.nc, T.ac.p);
  c.launches++;
  const int64_t nn = T.nc * T.nc;
  k_tl_fixrows<<<grid_for(nn, 256), 256, 0, s>>>(T.nc, T.cfix.p, T.ac.p);
  c.launches++;
  // the inverse in FP32 (the FP32 pipe is many times the FP64 one here, and the inverse is applied in
  // FP32): Gauss-Jordan without pivoting is stable on the SPD coarse matrix
  T.ac32.alloc((size_t)T.nc * T.nc);
  k_tl_sym32<<<grid_for(nn, 256), 256, 0, s>>>(T.nc, T.ac.p, T.ac32.p);
  c.launches++;
  const unsigned tiles = (unsigned)((T.nc + 63) / 64);
  for (int64_t k0 = 0; k0 < T.nc; k0 += kGjB) {
    k_gj_diag<float><<<1, 256, 0, s>>>(T.nc, k0, T.ac32.p, c.d_err.p);
    k_gj_row<float><<<grid_for(T.nc, 256), 256, 0, s>>>(T.nc, k0, T.ac32.p);
    k_gj_trail<float><<<dim3(tiles, tiles), 256, 0, s>>>(T.nc, k0, T.ac32.p);
    k_gj_col<float><<<grid_for(T.nc, 256), 256, 0, s>>>(T.nc, k0, T.ac32.p);
    c.launches += 4;
  }
  k_tl_pad32<<<grid_for(T.nc * T.ldc, 256), 256, 0, s>>>(T.nc, T.ldc, T.ac32.p, T.acinv32.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  check_device_flag(c, "two-level coarse matrix");
  T.have_inv = true;
}

// ---------------------------------------------------------------- scalar shared element matrix (3D Q2 Darcy / Poisson)
// The scalar counterpart of k_mf_hex27_gm for TPZMatPoisson / TPZDarcyFlow on a
// grid of translated Q2 hexes: K_e = k_e Khat (27 x 27; Khat the assembly's
// reference element matrix at coefficient 1, the Poisson scale included), so the
// operator over a tile of 128 elements is Y = U Khat^T: tcgen05.mma kind::tf32,
// 3xTF32, M 128, N 32, K 32.  A 256-thread CTA (two per SM, persistent over
// tiles) runs the same two-stage pipeline as the elasticity kernel with one
// thread per element in each group: 4 gatherer warps (rows copied as one block,
// the element's 27 values gathered, the translation removed -- Khat annihilates
// constants -- and split into the A operand; thread 0 issues the MMAs into
// accumulator pair k mod 2) and 4 scatterer warps (lane quarter = warp, 32
// columns read from TMEM, k_e Y added to q with scalar reductions, the element
// energy for p.q).  The penalty faces of every Dirichlet side (one table per
// face bucket) are applied by the same CTAs before the tiles, a warp per face.
namespace {
constexpr int kG1Threads = 256, kG1Group = 128, kG1El = 128, kG1K = 32, kG1N = 32;
constexpr uint32_t kG1Small = 32;  // TMEM column offset of the correction accumulator (buffer b at 64 b)
constexpr uint32_t kG1B = kG1N * kG1K * 4, kG1A = kG1El * kG1K * 4, kG1R = kG1El * kNS * 4;
constexpr uint32_t G1_BH = 0, G1_BL = kG1B, G1_AH = 2048 * 4, G1_AL = G1_AH + kG1A;
constexpr uint32_t G1_RG = G1_AL + kG1A, G1_RS = G1_RG + kG1R, G1_END = G1_RS + kG1R;
static_assert(G1_AH >= 2 * kG1B && G1_AH % 1024 == 0 && G1_AL % 1024 == 0 && G1_RG % 16 == 0, "operand alignment");
constexpr int kF1MaxTab = 16;  // face tables (one per penalty face bucket)

__device__ __forceinline__ void red_add_f1(float *p, float v) {
  asm volatile("red.relaxed.gpu.global.add.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}

// rows[i][a] (equation of shape a), coef[i] (the element's k, or 1), padded to whole tiles with -1 / 0
__global__ void k_mf1_records(int64_t n, const int64_t *__restrict__ elems, const int64_t *__restrict__ el_conn,
                              const int64_t *__restrict__ bpos, const int *__restrict__ sside,
                              const int *__restrict__ sk, const double *__restrict__ coef, double cconst,
                              int32_t *__restrict__ rows, float *__restrict__ rcoef) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t e = elems[i];
  for (int a = 0; a < kNS; a++) rows[i * kNS + a] = (int32_t)(bpos[el_conn[e * 27 + sside[a]]] + sk[a]);
  rcoef[i] = (float)(coef ? coef[e] : cconst);
}

// face records of a scalar problem: corners [i][4][3] and the equation of each of the 9 shapes
__global__ void k_mf1_face_records(int64_t n, const int64_t *__restrict__ elems, const int64_t *__restrict__ el_nodes,
                                   const double *__restrict__ xyz, const int64_t *__restrict__ el_conn,
                                   const int64_t *__restrict__ bpos, const int *__restrict__ sside,
                                   const int *__restrict__ sk, float *__restrict__ rxyz, int32_t *__restrict__ rows) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t e = elems[i];
  for (int k = 0; k < 4; k++)
    for (int j = 0; j < 3; j++) rxyz[(i * 4 + k) * 3 + j] = (float)xyz[el_nodes[e * 8 + k] * 3 + j];
  for (int a = 0; a < kFS; a++) rows[i * kFS + a] = (int32_t)(bpos[el_conn[e * 27 + sside[a]]] + sk[a]);
}

// penalty faces of a scalar problem: y_a += big sum_q w |J| phi_a phi_b u_b, one warp per face, the face's
// table (its bucket's shapes, gradients and weights) by index; their energy to *energy
constexpr int kF1Tab = kFQ * kFS + kFQ * 2 * kFS + kFQ;  // one face table: phi, dphi, w

// One penalty face of a scalar problem by one warp (table T in shared memory; su, sc, sq: the warp's scratch)
__device__ __forceinline__ void mf_face1(int64_t i, int lane, const float *T, float *su, float *sc, float *sq,
                                         float big, const float *__restrict__ rxyz, const int32_t *__restrict__ rows,
                                         const float *__restrict__ p, float *__restrict__ q, KSum &en) {
  const float *phi = T, *dphi = T + kFQ * kFS, *w = dphi + kFQ * 2 * kFS;
  int32_t row = 0;
  float u = 0.f;
  if (lane < kFS) {
    row = rows[i * kFS + lane];
    u = p[row];
    su[lane] = u;
  }
  if (lane < 12) sc[lane] = rxyz[i * 12 + lane];
  __syncwarp();
  if (lane < kFQ) {
    const int qp = lane;
    float g0[3] = {0.f, 0.f, 0.f}, g1[3] = {0.f, 0.f, 0.f};
    for (int k = 0; k < 4; k++)
      for (int j = 0; j < 3; j++) {
        g0[j] += sc[k * 3 + j] * dphi[(qp * 2 + 0) * kFS + k];
        g1[j] += sc[k * 3 + j] * dphi[(qp * 2 + 1) * kFS + k];
      }
    const float cx = g0[1] * g1[2] - g0[2] * g1[1], cy = g0[2] * g1[0] - g0[0] * g1[2],
                cz = g0[0] * g1[1] - g0[1] * g1[0];
    float uq = 0.f;
    for (int b = 0; b < kFS; b++) uq += phi[qp * kFS + b] * su[b];
    sq[qp] = big * w[qp] * sqrtf(cx * cx + cy * cy + cz * cz) * uq;
  }
  __syncwarp();
  if (lane < kFS) {
    float y = 0.f;
    for (int qp = 0; qp < kFQ; qp++) y += sq[qp] * phi[qp * kFS + lane];
    en.add(y * u);
    red_add_f1(&q[row], y);
  }
  __syncwarp();
}


__device__ __forceinline__ void g1_mma(uint32_t tm, uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl) {
  const uint32_t id = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kG1N >> 3) << 17) | ((uint32_t)(kG1El >> 4) << 24);
  constexpr uint32_t sbo = (kG1K / 4) * 128;
#pragma unroll 1
  for (int k = 0; k < kG1K / 8; k++) {
    const uint64_t dah = tc_desc(ah + k * 256, sbo), dal = tc_desc(al + k * 256, sbo);
    const uint64_t dbh = tc_desc(bh + k * 256, sbo), dbl = tc_desc(bl + k * 256, sbo);
    tc_mma(tm + kG1Small, dal, dbh, id, k > 0);
    tc_mma(tm + kG1Small, dah, dbl, id, 1u);
    tc_mma(tm, dah, dbh, id, k > 0);
  }
}

// rows: [ntile * 128][27] equations, -1 past the n elements; coef [ntile * 128]
struct G1Faces {  // the penalty faces, applied by the same CTAs before the tiles
  int64_t n;
  const float *rxyz, *tabs;
  const int32_t *rows;
  const uint8_t *tab;
  int ntab;
  float big;
};

__global__ void __launch_bounds__(kG1Threads, 2) k_mf_hex27_gm1(int64_t n, const int32_t *__restrict__ rows,
                                                                const float *__restrict__ coef,
                                                                const float4 *__restrict__ bsplit,
                                                                const float *__restrict__ p, float *__restrict__ q,
                                                                G1Faces F, int *__restrict__ err, Red R) {
  if (!active(R.iscal)) return;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;
  __shared__ __align__(8) uint64_t s_done[2], s_free[2];
  __shared__ float s_ft[kF1MaxTab * kF1Tab];
  __shared__ float s_fu[kG1Threads / 32][kFS], s_fc[kG1Threads / 32][12], s_fq[kG1Threads / 32][kFQ];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool gatherer = tid < kG1Group;
  const int gl = tid & (kG1Group - 1);
  const int4 *rows4 = (const int4 *)rows;
  for (uint32_t i = tid; i < 2 * kG1B / 16; i += kG1Threads) ((float4 *)(sm + G1_BH))[i] = bsplit[i];
  for (int k = tid; k < F.ntab * kF1Tab; k += kG1Threads) s_ft[k] = F.tabs[k];
  asm volatile("fence.proxy.async.shared::cta;");
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&s_tmem)), "r"(128));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    s_abort = 0;
    for (int b = 0; b < 2; b++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&s_done[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(&s_free[b])), "r"(kG1Group));
    }
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tm = s_tmem;
  const uint32_t ah = tc_smem(sm + G1_AH), al = tc_smem(sm + G1_AL), bh = tc_smem(sm + G1_BH),
                 bl = tc_smem(sm + G1_BL);
  const int64_t ntile = (n + kG1El - 1) / kG1El;
  constexpr int n4 = (int)(kG1R / 16);
  KSum en;
  // the penalty faces first (the tiles add into q with reductions only, so the order does not matter)
  for (int64_t f = (int64_t)blockIdx.x * (kG1Threads / 32) + warp; f < F.n; f += (int64_t)gridDim.x * (kG1Threads / 32))
    mf_face1(f, lane, s_ft + (int)F.tab[f] * kF1Tab, s_fu[warp], s_fc[warp], s_fq[warp], F.big, F.rxyz, F.rows, p, q, en);
  int last = -1;
  if (gatherer) {
    const int32_t *rw = (const int32_t *)(sm + G1_RG);
    int k = 0;
    for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x, k++) {
      const int b = k & 1;
      for (int i = gl; i < n4; i += kG1Group) ((int4 *)(sm + G1_RG))[i] = ld_stream4(rows4 + (size_t)tile * n4 + i);
      bool ok = true;
      if (gl == 0 && k >= 2) ok = gm_wait(&s_free[b], (uint32_t)((k - 2) >> 1) & 1u, &s_abort);
      if (ok && k >= 1) ok = gm_wait(&s_done[(k - 1) & 1], (uint32_t)((k - 1) >> 1) & 1u, &s_abort);
      if (!gm_vote(1, kG1Group, ok)) break;
      float v[kG1K];
#pragma unroll
      for (int a = 0; a < kG1K; a++) v[a] = 0.f;
#pragma unroll
      for (int a = 0; a < kNS; a++) {
        const int32_t r = rw[gl * kNS + a];
        v[a] = r >= 0 ? p[r] : 0.f;
      }
      // Khat annihilates constants (the corner shapes sum to one): remove corner 0's value from the
      // corner coefficients so the TF32 split's error is relative to the element's variation
      const float c0 = v[0];
#pragma unroll
      for (int a = 0; a < 8; a++) v[a] -= c0;
#pragma unroll
      for (int c = 0; c < kG1K / 4; c++) {
        float4 lo;
        const float4 hi = tf32_split4(make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]), lo);
        const uint32_t off = kmaj(gl, 4 * c, kG1K);
        *(float4 *)(sm + G1_AH + off) = hi;
        *(float4 *)(sm + G1_AL + off) = lo;
      }
      asm volatile("fence.proxy.async.shared::cta;");
      gm_bar(1, kG1Group);
      if (gl == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        g1_mma(tm + (uint32_t)b * 64u, ah, al, bh, bl);
        tc_commit(&s_done[b]);
        last = k;
      }
    }
  } else {
    const int32_t *rw = (const int32_t *)(sm + G1_RS);
    const int quarter = warp - kG1Group / 32, le = quarter * 32 + lane;
    int k = 0;
    for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x, k++) {
      const int b = k & 1;
      for (int i = gl; i < n4; i += kG1Group) ((int4 *)(sm + G1_RS))[i] = ld_stream4(rows4 + (size_t)tile * n4 + i);
      const bool ok = gm_wait(&s_done[b], (uint32_t)(k >> 1) & 1u, &s_abort);
      if (!gm_vote(2, kG1Group, ok)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t taddr = tm + ((uint32_t)(quarter * 32) << 16) + (uint32_t)b * 64u;
      float y[32], t[16];
      tc_ld16(taddr, y);
      tc_ld16(taddr + 16, y + 16);
      tc_ld16(taddr + kG1Small, t);
#pragma unroll
      for (int j = 0; j < 16; j++) y[j] += t[j];
      tc_ld16(taddr + kG1Small + 16, t);
#pragma unroll
      for (int j = 0; j < 16; j++) y[16 + j] += t[j];
      const int64_t e = tile * kG1El + le;
      if (e < n) {
        const float ke = coef[e];
#pragma unroll
        for (int a = 0; a < kNS; a++) {
          const int32_t r = rw[le * kNS + a];
          const float ya = ke * y[a];
          en.add(ya * p[r]);
          red_add_f1(&q[r], ya);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc_smem(&s_free[b])) : "memory");
      gm_bar(2, kG1Group);
    }
  }
  __syncthreads();
  const bool failed = s_abort != 0;
  if (failed && tid == 0) {
    atomicOr(err, 16384);
    if (last >= 0) tc_wait(&s_done[last & 1], (uint32_t)(last >> 1) & 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(128));
  double vv[1] = {failed ? 0.0 : en.get()}, tot[1];
  if (grid_reduce<1>(vv, R, tot) && threadIdx.x == 0) {
    const double pq = tot[0];
    R.scal[S_PQ] = pq;
    R.scal[S_ALPHA] = R.scal[S_RHO] / pq;
    R.iscal[I_SP32]++;
  }
}
}  // namespace

// Records of the scalar shared-matrix operator; false when the mesh is not one
// bucket of translated Q2 hexes of a scalar material (its reference matrix from
// the shared-matrix assembly) with penalty-Dirichlet or Neumann quad faces.
bool matfree1_build(Ctx &c) {
  MatFree1 &M = c.mf1;
  M.ready = false;
  if (c.nstate != 1 || c.dim != 3 || c.flt.active) return false;
  Bucket *vol = nullptr;
  std::vector<Bucket *> faces;
  for (Bucket *b : c.buckets) {
    if (b->hp) return false;
    const int mi = c.h_el_mat[b->elems[0]];
    if (!b->key.is_bc) {
      if (vol || b->key.type != GPZ_EL_HEX || b->nshape != kNS || b->shared != 1 ||
          (b->key.mat_kind != GPZ_MAT_POISSON && b->key.mat_kind != GPZ_MAT_DARCY))
        return false;
      vol = b;
    } else {
      const gpz_bc &bc = c.bcs[-mi - 1];
      if (bc.type == 1) continue;  // Neumann: load vector only
      if (bc.type != 0 || b->key.type != GPZ_EL_QUAD || b->nshape != kFS || b->nq != kFQ) return false;
      faces.push_back(b);
    }
  }
  if (!vol || (int)faces.size() > kF1MaxTab) return false;
  cudaStream_t s = c.stream;
  const gpz_material &m = c.mats[c.h_el_mat[vol->elems[0]]];
  M.nvol = (int64_t)vol->elems.size();
  const size_t npad = (size_t)((M.nvol + kG1El - 1) / kG1El) * kG1El;
  M.vrows.alloc(npad * kNS);
  GPZ_CUDA_TRY(cudaMemsetAsync(M.vrows.p, 0xFF, npad * kNS * sizeof(int32_t), s));
  M.vcoef.alloc(npad);
  M.vcoef.zero(s);
  const bool darcy = m.kind == GPZ_MAT_DARCY;
  k_mf1_records<<<grid_for(M.nvol, 256), 256, 0, s>>>(M.nvol, vol->d_elems.p, c.d_el_conn.p, c.d_block_pos.p,
                                                      vol->d_shape_side.p, vol->d_shape_k.p,
                                                      darcy ? c.d_coef.p : nullptr, darcy ? m.coef_const : 1.0,
                                                      M.vrows.p, M.vcoef.p);
  c.launches++;
  // Khat: the shared-matrix assembly's reference element matrix (coefficient 1), split into TF32 hi / lo
  std::vector<double> K((size_t)kNS * kNS);
  GPZ_CUDA_TRY(cudaMemcpyAsync(K.data(), vol->d_kref.p, K.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<float> hl(2 * kG1B / 4, 0.f);
  for (int nn = 0; nn < kNS; nn++)
    for (int k = 0; k < kNS; k++) {
      const double v = K[(size_t)nn * kNS + k];
      const float hi = tf32_round_host((float)v);
      const float lo = tf32_round_host((float)(v - (double)hi));
      const uint32_t off = kmaj(nn, k, kG1K) / 4;
      hl[off] = hi;
      hl[kG1B / 4 + off] = lo;
    }
  M.b.upload(hl.data(), hl.size(), s);
  // penalty faces: records of every Dirichlet bucket, each with its own table
  M.nface = 0;
  for (Bucket *f : faces) M.nface += (int64_t)f->elems.size();
  M.ntab = (int)faces.size();
  if (M.nface) {
    M.fxyz.alloc((size_t)M.nface * 12);
    M.frows.alloc((size_t)M.nface * kFS);
    M.ftab.alloc((size_t)M.nface);
    std::vector<float> tabs;
    std::vector<uint8_t> ftab;
    int64_t off = 0;
    for (int t = 0; t < (int)faces.size(); t++) {
      Bucket *f = faces[t];
      const int64_t nf = (int64_t)f->elems.size();
      k_mf1_face_records<<<grid_for(nf, 256), 256, 0, s>>>(nf, f->d_elems.p, c.d_el_nodes.p, c.d_xyz.p,
                                                           c.d_el_conn.p, c.d_block_pos.p, f->d_shape_side.p,
                                                           f->d_shape_k.p, M.fxyz.p + off * 12, M.frows.p + off * kFS);
      c.launches++;
      for (double x : f->phi) tabs.push_back((float)x);
      for (double x : f->dphi) tabs.push_back((float)x);
      for (double x : f->w) tabs.push_back((float)x);
      ftab.insert(ftab.end(), (size_t)nf, (uint8_t)t);
      off += nf;
    }
    M.ftab.upload(ftab.data(), ftab.size(), s);
    M.ftabs.upload(tabs.data(), tabs.size(), s);
    M.energy.alloc(1);
  }
  M.big = (float)m.bignumber;
  GPZ_CUDA_TRY(cudaGetLastError());
  check_device_flag(c, "scalar matrix-free records");
  GPZ_CUDA_TRY(cudaFuncSetAttribute(k_mf_hex27_gm1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G1_END));
  int dev = 0, nsm = 0;
  GPZ_CUDA_TRY(cudaGetDevice(&dev));
  GPZ_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  M.grid = std::max(1, std::min(kGridBlocks, 2 * nsm));  // two 67 KB CTAs per SM
  M.ready = true;
  return true;
}

// q = A32 p for the scalar shared-matrix operator (q zeroed by the caller), p.q and alpha
void matfree1_spmv(Ctx &c, cudaStream_t s, const float *p, float *q) {
  MatFree1 &M = c.mf1;
  SolverWork &w = c.sw;
  Red R{w.partial.p, w.counter.p, w.scal.p, w.iscal.p};
  // (the penalty faces are applied by the same CTAs)
  k_mf_hex27_gm1<<<M.grid, kG1Threads, G1_END, s>>>(
      M.nvol, M.vrows.p, M.vcoef.p, (const float4 *)M.b.p, p, q,
      G1Faces{M.nface, M.fxyz.p, M.ftabs.p, M.frows.p, M.ftab.p, M.ntab, M.big}, c.d_err.p, R);
  c.launches++;
}

// Build the element records of the matrix-free operator; false when the mesh
// is not made of uniform Q2 hex elasticity elements plus penalty / traction faces.
bool matfree_build(Ctx &c) {
  MatFree &M = c.mf;
  M.ready = false;
  M.gm_ready = false;
  if (c.nstate != 3) return false;
  Bucket *vol = nullptr;
  std::vector<Bucket *> faces;
  for (Bucket *b : c.buckets) {
    if (b->hp) return false;
    const int mi = c.h_el_mat[b->elems[0]];
    if (!b->key.is_bc) {
      if (b->key.type != GPZ_EL_HEX || b->nshape != kNS || b->nq != kNQ || b->key.mat_kind != GPZ_MAT_ELAST3D ||
          vol)
        return false;
      vol = b;
    } else {
      const gpz_bc &bc = c.bcs[-mi - 1];
      if (bc.type == 1) continue;  // traction: load vector only
      if (bc.type != 0 || b->key.type != GPZ_EL_QUAD || b->nshape != kFS || b->nq != kFQ) return false;
      faces.push_back(b);
    }
  }
  if (!vol || faces.size() > 1) return false;
  cudaStream_t s = c.stream;
  const gpz_material &m = c.mats[c.h_el_mat[vol->elems[0]]];
  auto f32 = [&](const std::vector<double> &v, DBuf<float> &out) {
    std::vector<float> t(v.begin(), v.end());
    out.upload(t.data(), t.size(), s);
  };
  M.nvol = (int64_t)vol->elems.size();
  M.vxyz.alloc((size_t)M.nvol * 24);
  // block rows padded to whole tiles of the shared-matrix kernel with -1 (it copies a tile's rows as one block)
  const size_t vrows_n = (size_t)((M.nvol + kGmEl - 1) / kGmEl) * kGmEl * kNS;
  M.vrows.alloc(vrows_n);
  GPZ_CUDA_TRY(cudaMemsetAsync(M.vrows.p, 0xFF, vrows_n * sizeof(int32_t), s));
  M.vlm.alloc((size_t)M.nvol * 2);
  M.vgeo.alloc((size_t)M.nvol * 10);
  f32(vol->dphi, M.vdphi);
  f32(vol->w, M.vw);
  k_mf_records<<<grid_for(M.nvol, 256), 256, 0, s>>>(M.nvol, vol->d_elems.p, c.d_el_nodes.p, c.d_xyz.p, c.d_el_conn.p,
                                                     c.d_block_pos.p, vol->d_shape_side.p, vol->d_shape_k.p, kNS, 8,
                                                     c.d_coef.p, m.E, m.nu, M.vxyz.p, M.vrows.p, M.vlm.p, M.vgeo.p,
                                                     c.d_err.p);
  c.launches++;
  M.nface = 0;
  if (!faces.empty()) {
    Bucket *f = faces[0];
    M.nface = (int64_t)f->elems.size();
    M.fxyz.alloc((size_t)M.nface * 12);
    M.frows.alloc((size_t)M.nface * kFS);
    f32(f->phi, M.fphi);
    f32(f->dphi, M.fdphi);
    f32(f->w, M.fw);
    M.big = 1.e12f;  // TPZElasticity3D.cpp:632
    k_mf_records<<<grid_for(M.nface, 256), 256, 0, s>>>(M.nface, f->d_elems.p, c.d_el_nodes.p, c.d_xyz.p,
                                                        c.d_el_conn.p, c.d_block_pos.p, f->d_shape_side.p,
                                                        f->d_shape_k.p, kFS, 4, nullptr, 0.0, 0.0, M.fxyz.p,
                                                        M.frows.p, nullptr, nullptr, c.d_err.p);
    c.launches++;
  }
  M.energy.alloc(1);
  GPZ_CUDA_TRY(cudaGetLastError());
  check_device_flag(c, "matrix-free records");
  M.sf_ready = sf_tables(c, *vol);
  M.grid_vol = mf_grid(k_mf_hex27, kMfThreads);
  // a warp per face: no more CTAs than the faces fill (every CTA takes part in the energy's grid reduction)
  M.grid_face = (int)std::max<int64_t>(1, std::min<int64_t>(mf_grid(k_mf_faces, kThreads), (M.nface + kWarps - 1) / kWarps));
  GPZ_CUDA_TRY(cudaFuncSetAttribute(k_mf_hex27_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OFF_TC_END));
  {
    int dev = 0, nsm = 0;
    GPZ_CUDA_TRY(cudaGetDevice(&dev));
    GPZ_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    M.grid_tc = std::max(1, std::min(kGridBlocks, nsm));  // one 187 KB CTA per SM, persistent over tiles
  }
  M.grid_sf = mf_grid(k_mf_hex27_sf, kSfThreads);
  M.gm_ready = gm_tables(c, *vol, m.nu);
  M.gt_ready = M.gm_ready && gt_build(c, *vol);
  M.ready = true;
  return true;
}

// q4 = A p4 (q4 zeroed by the caller), p.q and alpha as the block SpMV kernels;
// mode 1: the tcgen05 3xTF32 volume kernel, 2: sum-factorised, 3: the shared
// element matrix on the tensor cores, 0: the CUDA-core element kernel
void matfree_spmv(Ctx &c, cudaStream_t s, int mode) {
  MatFree &M = c.mf;
  SolverWork &w = c.sw;
  Red R{w.partial.p, w.counter.p, w.scal.p, w.iscal.p};
  const float4 *p4 = (const float4 *)w.pm.p;
  float4 *q4 = (float4 *)w.q32.p;
  if (M.nface && mode != 4) {  // (the lattice-block kernel applies the faces itself)
    k_mf_faces<<<M.grid_face, kThreads, 0, s>>>(M.nface, M.fxyz.p, M.frows.p, M.fphi.p, M.fdphi.p, M.fw.p, M.big, p4,
                                                q4, M.energy.p, R);
    c.launches++;
  }
  const double *fe = M.nface ? M.energy.p : nullptr;
  if (mode == 1)
    k_mf_hex27_tc<<<M.grid_tc, kTcThreads, OFF_TC_END, s>>>(M.nvol, M.vxyz.p, M.vrows.p, M.vlm.p, M.vgeo.p, M.vdphi.p,
                                                            M.vw.p, p4, q4, fe, c.d_err.p, R);
  else if (mode == 3)
    k_mf_hex27_gm<<<M.grid_gm, kGmThreads, GM_END, s>>>(M.nvol, M.vrows.p, M.vlm.p, (const float4 *)M.gm_b.p, p4, q4, fe,
                                                        c.d_err.p, R);
  else if (mode == 4)
    k_mf_hex27_gt<<<M.grid_gt, kGtThreads, GT_END, s>>>(
        M.gt, M.gt_nmap.p, M.gt_emu.p, M.gt_face.p, (const float4 *)M.gm_b.p, p4, q4,
        GtFaces{M.nface, M.fxyz.p, M.fphi.p, M.fdphi.p, M.fw.p, M.frows.p, M.big}, c.d_err.p, R);
  else if (mode == 2)
    k_mf_hex27_sf<<<M.grid_sf, kSfThreads, 0, s>>>(M.nvol, M.vxyz.p, M.vrows.p, M.vlm.p, M.vgeo.p, M.sf_tab.p,
                                                   M.sf_idx.p, p4, q4, fe, R);
  else
    k_mf_hex27<<<M.grid_vol, kMfThreads, 0, s>>>(M.nvol, M.vxyz.p, M.vrows.p, M.vlm.p, M.vgeo.p, M.vdphi.p, M.vw.p, p4, q4,
                                                 fe, R);
  c.launches++;
}

}  // namespace gpz
