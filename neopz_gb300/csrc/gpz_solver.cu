// Iterative solvers on the device.
//
// * spmv: full CSR (int64 row pointers, int32 columns), y = alpha A x + beta y;
//   replaces TPZSYsmpMatrix::MultAdd / TPZFYsmpMatrix::MultAdd.
// * Jacobi-PCG exactly as Solvers/LinearSolvers/cg.h:29-132 with the Jacobi
//   TPZStepSolver (z = r / diag, Matrix/pzmatrix.cpp:643-667): stop on the
//   recursive ||r||/||b|| <= tol, counting iterations as the reference does.
//   Three kernels per iteration (p update; q = A p with p.q; x, r update with
//   r.z and r.r), each reduction finished by the last CTA in a fixed order so
//   results are deterministic.  Convergence and the iteration count live on
//   the device, so a batch of iterations is captured once as a CUDA graph and
//   replayed; kernels of a converged solve return at entry.
// * Mixed CG: the same recurrence with q = A32 p32 (FP32 values and FP32
//   accumulation, 8 bytes per stored entry instead of 12), FP64 x, r, dots and
//   scalars, and reliable updates: when ||r|| has dropped by `reliable_delta`
//   since the last update, or the recursive residual meets the tolerance, the
//   true residual b - A64 x is recomputed in FP64 and replaces r.  The solve
//   stops only on the true FP64 residual.
#include <algorithm>
#include <cmath>
#include <vector>

#include "gpz_internal.h"
#include "gpz_learned.cuh"
#include "gpz_solver_common.cuh"

namespace gpz {

LnView learned_view(Ctx &c);

namespace {


// ---------------------------------------------------------------- SpMV
// TPR threads cooperate on one row.
// All TPR-row kernels walk rows in warp-uniform groups so that every lane of a
// warp reaches the shuffles: lane l of a warp handles row r0 + l / TPR.
#define GPZ_ROW_LOOP(TPR, n)                                                                   \
  const int sub = threadIdx.x % TPR;                                                           \
  const int64_t rows_per_warp = 32 / TPR;                                                      \
  const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;               \
  const int64_t nwarps = (int64_t)gridDim.x * blockDim.x / 32;                                 \
  for (int64_t r0 = warp_id * rows_per_warp; r0 < (n); r0 += nwarps * rows_per_warp)

template <int TPR>
__device__ __forceinline__ double row_dot64(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                            const double *__restrict__ a, const double *__restrict__ x, int64_t r,
                                            int sub, bool valid) {
  // two independent load/FMA chains per lane; matrix streams bypass L1 (read once).
  // FP64 instructions are the scarce resource on this part, so the row is
  // split over few lanes (pick_tpr64) and combined with few FP64 adds.
  double s0 = 0.0, s1 = 0.0;
  int64_t k0 = valid ? ia[r] : 0, k1 = valid ? ia[r + 1] : 0;
  int64_t k = k0 + sub;
  for (; k + TPR < k1; k += 2 * TPR) {
    const int c0 = __ldcs(&ja[k]), c1 = __ldcs(&ja[k + TPR]);
    const double a0 = __ldcs(&a[k]), a1 = __ldcs(&a[k + TPR]);
    s0 = fma(a0, __ldg(&x[c0]), s0);
    s1 = fma(a1, __ldg(&x[c1]), s1);
  }
  if (k < k1) s0 = fma(__ldcs(&a[k]), __ldg(&x[__ldcs(&ja[k])]), s0);
  double s = s0 + s1;
  for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
  return s;
}

template <int TPR>
__device__ __forceinline__ float row_dot32(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                           const float *__restrict__ a, const float *__restrict__ x, int64_t r,
                                           int sub, bool valid) {
  float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
  int64_t k0 = valid ? ia[r] : 0, k1 = valid ? ia[r + 1] : 0;
  int64_t k = k0 + sub;
  for (; k + 3 * TPR < k1; k += 4 * TPR) {
    const int c0 = __ldcs(&ja[k]), c1 = __ldcs(&ja[k + TPR]), c2 = __ldcs(&ja[k + 2 * TPR]),
              c3 = __ldcs(&ja[k + 3 * TPR]);
    const float a0 = __ldcs(&a[k]), a1 = __ldcs(&a[k + TPR]), a2 = __ldcs(&a[k + 2 * TPR]),
                a3 = __ldcs(&a[k + 3 * TPR]);
    s0 = fmaf(a0, __ldg(&x[c0]), s0);
    s1 = fmaf(a1, __ldg(&x[c1]), s1);
    s2 = fmaf(a2, __ldg(&x[c2]), s2);
    s3 = fmaf(a3, __ldg(&x[c3]), s3);
  }
  for (; k < k1; k += TPR) s0 = fmaf(__ldcs(&a[k]), __ldg(&x[__ldcs(&ja[k])]), s0);
  float s = (s0 + s1) + (s2 + s3);
  for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
  return s;
}

template <int TPR>
__global__ void __launch_bounds__(kThreads) k_spmv64(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                     const double *__restrict__ a, const double *__restrict__ x,
                                                     double *__restrict__ y, const double *__restrict__ yin,
                                                     double alpha, double beta, int64_t n) {
  GPZ_ROW_LOOP(TPR, n) {
    const int64_t r = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = r < n;
    double s = row_dot64<TPR>(ia, ja, a, x, r, sub, valid);
    if (sub == 0 && valid) y[r] = alpha * s + (yin ? beta * yin[r] : 0.0);
  }
}

// q = A p with p.q (iteration kernel C of the FP64 CG)
template <int TPR, bool F32>
__global__ void __launch_bounds__(kThreads) k_cg_spmv(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                      const double *__restrict__ a64, const float *__restrict__ a32,
                                                      const double *__restrict__ p, const float *__restrict__ p32,
                                                      double *__restrict__ q, int64_t n, Red R) {
  static_assert(!F32, "the FP32 iteration uses k_mx_csr / k_mx_sell3");
  if (!active(R.iscal)) return;
  double pq = 0.0;
  GPZ_ROW_LOOP(TPR, n) {
    const int64_t r = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = r < n;
    const double s = row_dot64<TPR>(ia, ja, a64, p, r, sub, valid);
    if (sub == 0 && valid) {
      q[r] = s;
      pq += p[r] * s;
    }
  }
  double v[1] = {pq}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    R.scal[S_PQ] = tot[0];
    R.scal[S_ALPHA] = R.scal[S_RHO] / tot[0];
    R.iscal[I_SP64]++;
  }
}

// Preconditioner: pointwise Jacobi (z_i = r_i / a_ii, TPZMatrix::SolveJacobi
// one sweep) or connect-block Jacobi with 3x3 inverses (TPZBlockDiagonal over
// the mesh blocks).  The vector kernels walk "units": rows, or block rows.
struct Prec {
  const double *dinv;
  const double *binv;  // [nunits][9] when block
  int block;
};

__device__ __forceinline__ void apply_prec(const Prec &M, const double *__restrict__ r, int64_t u, double *z) {
  if (!M.block) {
    z[0] = r[u] * M.dinv[u];
  } else {
    const double *B = M.binv + 9 * u;
    const double r0 = r[3 * u], r1 = r[3 * u + 1], r2 = r[3 * u + 2];
    z[0] = B[0] * r0 + B[1] * r1 + B[2] * r2;
    z[1] = B[3] * r0 + B[4] * r1 + B[5] * r2;
    z[2] = B[6] * r0 + B[7] * r1 + B[8] * r2;
  }
}

// kernel B: p = z + beta p, first iteration (or after a restart) p = z
__global__ void __launch_bounds__(kThreads) k_cg_p(const double *__restrict__ r, Prec M, double *__restrict__ p,
                                                   int64_t nunits, Red R) {
  if (!active(R.iscal)) return;
  const bool first = R.iscal[I_IT] == 0 || R.iscal[I_RESTART] != 0;
  const double beta = first ? 0.0 : R.scal[S_BETA];
  const int bs = M.block ? 3 : 1;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    double z[3];
    apply_prec(M, r, u, z);
    for (int k = 0; k < bs; k++) {
      const int64_t i = u * bs + k;
      const double pi = first ? z[k] : z[k] + beta * p[i];
      p[i] = pi;
    }
  }
}

// kernel D: alpha = rho / pq; x += alpha p; r -= alpha q; rho' = r.(M r), rr = r.r
__global__ void __launch_bounds__(kThreads) k_cg_update(double *__restrict__ x, double *__restrict__ r,
                                                        const double *__restrict__ p, const double *__restrict__ q,
                                                        Prec M, int64_t nunits, int mixed, Red R) {
  if (!active(R.iscal)) return;
  const double pq = R.scal[S_PQ];
  const double alpha = R.scal[S_ALPHA];
  const int bs = M.block ? 3 : 1;
  double rz = 0.0, rr = 0.0;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    for (int k = 0; k < bs; k++) {
      const int64_t i = u * bs + k;
      x[i] = x[i] + alpha * p[i];
      const double ri = r[i] - alpha * q[i];
      r[i] = ri;
      rr += ri * ri;
    }
    double z[3];
    apply_prec(M, r, u, z);
    for (int k = 0; k < bs; k++) rz += r[u * bs + k] * z[k];
  }
  double v[2] = {rz, rr}, tot[2];
  if (grid_reduce<2>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    if (!(pq > 0.0) || !isfinite(tot[1]) || !isfinite(tot[0])) is[I_BREAK] = 1;
    s[S_RHO1] = s[S_RHO];
    s[S_RHO] = tot[0];
    s[S_BETA] = tot[0] / s[S_RHO1];
    s[S_RR] = tot[1];
    if (tot[1] > s[S_MAXRR]) s[S_MAXRR] = tot[1];
    const double resid = sqrt(tot[1]) / s[S_NORMB];
    s[S_RESID] = resid;
    is[I_IT] += 1;
    is[I_RESTART] = 0;
    if (is[I_BREAK]) is[I_CONV] = 2;
    else if (!mixed) {
      if (resid <= s[S_TOL]) is[I_CONV] = 1;
    } else if (resid <= s[S_TOL] || tot[1] < s[S_DELTA2] * s[S_MAXRR]) {
      is[I_UPDATE] = 1;
    }
  }
}

// kernel E (mixed): when requested, r = b - A64 x in FP64 (residual replacement)
template <int TPR>
__global__ void __launch_bounds__(kThreads) k_reliable(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                       const double *__restrict__ a, const double *__restrict__ x,
                                                       const double *__restrict__ b, double *__restrict__ r, int64_t n,
                                                       Red R) {
  if (R.iscal[I_UPDATE] != 1 || R.iscal[I_CONV] != 0) return;
  double rr = 0.0;
  GPZ_ROW_LOOP(TPR, n) {
    const int64_t i = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = i < n;
    double s = row_dot64<TPR>(ia, ja, a, x, i, sub, valid);
    if (sub == 0 && valid) {
      const double ri = b[i] - s;
      r[i] = ri;
      rr += ri * ri;
    }
  }
  double v[1] = {rr}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    s[S_RR] = tot[0];
    s[S_MAXRR] = tot[0];
    s[S_TRUERR] = tot[0];
    const double resid = sqrt(tot[0]) / s[S_NORMB];
    s[S_RESID] = resid;
    is[I_NUPD] += 1;
    is[I_SP64] += 1;
    if (resid <= s[S_TOL]) is[I_CONV] = 1;
    is[I_UPDATE] = 2;
  }
}

// rho = r.(M r) for a freshly computed residual (after init or a replacement).
// When the replaced residual differs from the recursive one by a large factor
// in the preconditioner norm (FP32 drift carried over from the early, large
// updates), beta = rho_true / rho_old would blow the direction up, so the
// direction restarts (p = z) instead.
__global__ void __launch_bounds__(kThreads) k_precond_dot(const double *__restrict__ r, Prec M, int64_t nunits, Red R) {
  if (R.iscal[I_UPDATE] != 2) return;
  const int bs = M.block ? 3 : 1;
  double rz = 0.0;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    double z[3];
    apply_prec(M, r, u, z);
    for (int k = 0; k < bs; k++) rz += r[u * bs + k] * z[k];
  }
  double v[1] = {rz}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    if (is[I_IT] > 0 && (tot[0] > 4.0 * s[S_RHO] || tot[0] < 0.25 * s[S_RHO])) {
      is[I_RESTART] = 1;
      is[I_NRESTART] += 1;
    }
    s[S_RHO] = tot[0];
    s[S_BETA] = s[S_RHO1] != 0.0 ? tot[0] / s[S_RHO1] : 0.0;
    is[I_UPDATE] = 0;
  }
}

// initial residual: r = b (x = 0) or r = b - A x; rr, normb; rho follows in k_precond_dot
template <int TPR>
__global__ void __launch_bounds__(kThreads) k_cg_init(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                      const double *__restrict__ a, double *__restrict__ x,
                                                      const double *__restrict__ b, double *__restrict__ r, int64_t n,
                                                      int from_current, Red R) {
  double rr = 0.0, bb = 0.0;
  GPZ_ROW_LOOP(TPR, n) {
    const int64_t i = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = i < n;
    double s = 0.0;
    if (from_current) s = row_dot64<TPR>(ia, ja, a, x, i, sub, valid);
    if (sub == 0 && valid) {
      const double bi = b[i];
      const double ri = bi - s;
      if (!from_current) x[i] = 0.0;
      r[i] = ri;
      rr += ri * ri;
      bb += bi * bi;
    }
  }
  double v[2] = {rr, bb}, tot[2];
  if (grid_reduce<2>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    double normb = sqrt(tot[1]);
    if (normb == 0.0) normb = 1.0;
    s[S_NORMB] = normb;
    s[S_RHO1] = 0.0;
    s[S_RR] = tot[0];
    s[S_MAXRR] = tot[0];
    const double resid = sqrt(tot[0]) / normb;
    s[S_RESID] = resid;
    is[I_IT] = 0;
    is[I_CONV] = (resid <= s[S_TOL]) ? 1 : 0;
    is[I_UPDATE] = 2;
  }
}

// true residual norm ||b - A x||^2 into scal[S_TRUERR]
template <int TPR>
__global__ void __launch_bounds__(kThreads) k_true_resid(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                         const double *__restrict__ a, const double *__restrict__ x,
                                                         const double *__restrict__ b, int64_t n, Red R) {
  double rr = 0.0;
  GPZ_ROW_LOOP(TPR, n) {
    const int64_t i = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = i < n;
    double s = row_dot64<TPR>(ia, ja, a, x, i, sub, valid);
    if (sub == 0 && valid) {
      const double ri = b[i] - s;
      rr += ri * ri;
    }
  }
  double v[1] = {rr}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) R.scal[S_TRUERR] = tot[0];
}

// ---- stationary Jacobi: TPZStepSolver::SetJacobi as the solver
// (TPZMatrix::SolveJacobi, Matrix/pzmatrix.cpp:643-667, and the TPZFYsmpMatrix
// override, Matrix/pzysmp.cpp:725-781).  A sweep is x += r / a_ii (a division,
// as the reference) and then r = b - A x with ||r|| against the absolute
// tolerance in S_TOL; sweeps of a batch after convergence (or a NaN norm)
// return at entry.  The first sweep of a full (TPZFYsmpMatrix) pattern is unconditional: the
// start kernel clears I_CONV for it.
__global__ void k_jac_start(Red R, int first_sweep_always) {
  double *s = R.scal;
  int64_t *is = R.iscal;
  is[I_IT] = 0;
  const double res = sqrt(s[S_RR]);
  is[I_CONV] = first_sweep_always ? 0 : res <= s[S_TOL] ? 1 : res > s[S_TOL] ? 0 : 2;
}

__global__ void __launch_bounds__(kThreads) k_jac_x(const double *__restrict__ a, const int64_t *__restrict__ diagpos,
                                                    const double *__restrict__ r, double *__restrict__ x, int64_t n,
                                                    const int64_t *__restrict__ is) {
  if (!active(is)) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += r[i] / a[diagpos[i]];
}

template <int TPR>
__global__ void __launch_bounds__(kThreads) k_jac_resid(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                        const double *__restrict__ a, const double *__restrict__ x,
                                                        const double *__restrict__ b, double *__restrict__ r, int64_t n,
                                                        Red R) {
  if (!active(R.iscal)) return;
  double rr = 0.0;
  GPZ_ROW_LOOP(TPR, n) {
    const int64_t i = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = i < n;
    const double s = row_dot64<TPR>(ia, ja, a, x, i, sub, valid);
    if (sub == 0 && valid) {
      const double ri = b[i] - s;
      r[i] = ri;
      rr += ri * ri;
    }
  }
  double v[1] = {rr}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    const double res = sqrt(tot[0]);
    s[S_RR] = tot[0];
    s[S_RESID] = res / s[S_NORMB];
    is[I_SP64]++;
    is[I_IT]++;
    // the reference's loop runs while ||r|| > tol: a NaN norm ends it too (I_CONV = 2, not converged)
    if (res <= s[S_TOL]) is[I_CONV] = 1;
    else if (!(res > s[S_TOL])) is[I_CONV] = 2;
  }
}

// ---- setup kernels for the mixed path and the block preconditioner
template <typename TA>
__global__ void k_build_bsr3(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                             const TA *__restrict__ a, int64_t nbrow, int64_t *__restrict__ bptr,
                             int32_t *__restrict__ bcol, float *__restrict__ bval, int *__restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int64_t I = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  if (I >= nbrow) return;
  const int64_t r0 = 3 * I;
  const int64_t len = ia[r0 + 1] - ia[r0];
  if (len % 3 != 0 || ia[r0 + 2] - ia[r0 + 1] != len || ia[r0 + 3] - ia[r0 + 2] != len || ia[r0] % 9 != 0) {
    if (lane == 0) atomicOr(err, 128);
    return;
  }
  const int64_t nb = len / 3, b0 = ia[r0] / 9;
  if (lane == 0) {
    bptr[I] = b0;
    if (I == nbrow - 1) bptr[nbrow] = b0 + nb;
  }
  float *v = bval + 9 * b0;
  for (int64_t j = lane; j < nb; j += 32) {
    bcol[b0 + j] = ja[ia[r0] + 3 * j] / 3;
    for (int s = 0; s < 3; s++)
      for (int t = 0; t < 3; t++) v[(3 * s + t) * nb + j] = (float)a[ia[r0 + s] + 3 * j + t];
  }
}

// fill the sliced-ELL planes from the full FP64 CSR (rows 3I..3I+2 of block
// row I share their columns; block column j covers columns 3j'..3j'+2)
template <typename TA>
__global__ void k_fill_sell3(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                             const TA *__restrict__ a, const int64_t *__restrict__ soff,
                             const int32_t *__restrict__ slen, const int32_t *__restrict__ sperm, int64_t nslice,
                             int64_t plane, int32_t *__restrict__ scol, float *__restrict__ sval, int *__restrict__ err) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t sl = g / 32;
  const int t = (int)(g % 32);
  if (sl >= nslice) return;
  const int I = sperm[sl * 32 + t];
  const int len = slen[sl];
  int64_t r0 = 0, nb = 0;
  if (I >= 0) {
    r0 = 3 * (int64_t)I;
    const int64_t l0 = ia[r0 + 1] - ia[r0];
    if (l0 % 3 != 0 || ia[r0 + 2] - ia[r0 + 1] != l0 || ia[r0 + 3] - ia[r0 + 2] != l0 || l0 / 3 > len) {
      atomicOr(err, 128);
      return;
    }
    nb = l0 / 3;
  }
  for (int j = 0; j < len; j++) {
    const int64_t e = soff[sl] + (int64_t)j * 32 + t;
    if (j < nb) {
      scol[e] = ja[ia[r0] + 3 * j] / 3;
      for (int s = 0; s < 3; s++)
        for (int u = 0; u < 3; u++) sval[(3 * s + u) * plane + e] = (float)a[ia[r0 + s] + 3 * j + u];
    } else {
      scol[e] = I >= 0 ? I : 0;  // padding: zero block on a cached column
      for (int k = 0; k < 9; k++) sval[k * plane + e] = 0.f;
    }
  }
}

__global__ void k_block_inv3(const double *__restrict__ a, const int64_t *__restrict__ diagpos, int64_t nbrow,
                             double *__restrict__ binv, int *__restrict__ err) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nbrow) return;
  double m[3][3];
  for (int s = 0; s < 3; s++)
    for (int t = 0; t < 3; t++) m[s][t] = a[diagpos[3 * u + s] + (t - s)];
  const double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
  const double c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
  const double c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
  const double det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
  if (!(fabs(det) > 0.0)) {
    atomicOr(err, 256);
    return;
  }
  const double id = 1.0 / det;
  double *B = binv + 9 * u;
  B[0] = c00 * id;
  B[1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
  B[2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
  B[3] = c01 * id;
  B[4] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
  B[5] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
  B[6] = c02 * id;
  B[7] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
  B[8] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
}

// ======================================================================
// Mixed-precision CG: every per-entry operation of the inner iteration is
// FP32 (GB300 issues FP64 at a small fraction of its FP32 rate, so even a few
// FP64 instructions per row cost as much as the FP32 matrix stream).  FP64 is
// kept for: the solution x (the FP32 increment dx accumulated since the last
// reliable update is folded into it), the true residual b - A64 x of every
// reliable update, the dot-product accumulation (compensated FP32 partial
// sums per thread, FP64 across threads and CTAs) and the alpha/beta scalars.
// ======================================================================

// compensated (Kahan) FP32 accumulation of one thread's terms

struct Prec32 {
  const float *dinv;  // [neq]
  const float *binv;  // [nbrow][9]
  int block;
};

// p is stored padded to four floats per 3-row block when the 3x3 block SpMV
// reads it; pidx maps an equation to its slot.
__device__ __forceinline__ int64_t pidx(int64_t i, int padded) { return padded ? (i / 3) * 4 + i % 3 : i; }

__device__ __forceinline__ void apply_prec32(const Prec32 &M, const float *__restrict__ r, int64_t u, float *z) {
  if (!M.block) {
    z[0] = r[u] * M.dinv[u];
  } else {
    const float *B = M.binv + 9 * u;
    const float r0 = r[3 * u], r1 = r[3 * u + 1], r2 = r[3 * u + 2];
    z[0] = fmaf(B[0], r0, fmaf(B[1], r1, B[2] * r2));
    z[1] = fmaf(B[3], r0, fmaf(B[4], r1, B[5] * r2));
    z[2] = fmaf(B[6], r0, fmaf(B[7], r1, B[8] * r2));
  }
}

// p = z + beta p (z = M r), or p = z at the first iteration / after a restart
__global__ void __launch_bounds__(kThreads) k_mx_p(const float *__restrict__ r, Prec32 M, float *__restrict__ p,
                                                   int padded, float *__restrict__ qzero, int64_t nunits, Red R) {
  if (!active(R.iscal)) return;
  const bool first = R.iscal[I_IT] == 0 || R.iscal[I_RESTART] != 0;
  const float beta = first ? 0.f : (float)R.scal[S_BETA];
  const int bs = M.block ? 3 : 1;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    float z[3];
    apply_prec32(M, r, u, z);
    for (int k = 0; k < bs; k++) {
      const int64_t j = pidx(u * bs + k, padded);
      p[j] = first ? z[k] : fmaf(beta, p[j], z[k]);
      if (qzero) qzero[j] = 0.f;  // the symmetric SpMV accumulates q with atomics
    }
  }
}

// q = A32 p over 3x3 block rows; a warp owns a tile of 32 block rows, lane t
// keeps row t's result so the epilogue (q store, p.q) runs with all lanes.
__global__ void __launch_bounds__(kThreads) k_mx_bsr3(const int64_t *__restrict__ bptr, const int32_t *__restrict__ bcol,
                                                      const float *__restrict__ bval, const float4 *__restrict__ p4,
                                                      float *__restrict__ q, int64_t nbrow, Red R) {
  if (!active(R.iscal)) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int64_t nwarps = (int64_t)gridDim.x * blockDim.x / 32;
  KSum pq;
  for (int64_t I0 = warp_id * 32; I0 < nbrow; I0 += nwarps * 32) {
    const int nrow = (int)min((int64_t)32, nbrow - I0);
    const int64_t mybeg = lane < nrow ? bptr[I0 + lane] : 0;
    const int64_t myend = lane < nrow ? bptr[I0 + lane + 1] : 0;
    float m0 = 0.f, m1 = 0.f, m2 = 0.f;
    for (int t = 0; t < nrow; t++) {
      const int64_t b0 = __shfl_sync(0xffffffffu, mybeg, t);
      const int nb = (int)(__shfl_sync(0xffffffffu, myend, t) - b0);
      const float *v = bval + 9 * b0;
      float a0 = 0.f, a1 = 0.f, a2 = 0.f;
      for (int j = lane; j < nb; j += 32) {
        const float4 xv = __ldg(&p4[__ldcs(&bcol[b0 + j])]);
        a0 = fmaf(__ldcs(&v[0 * nb + j]), xv.x, a0);
        a0 = fmaf(__ldcs(&v[1 * nb + j]), xv.y, a0);
        a0 = fmaf(__ldcs(&v[2 * nb + j]), xv.z, a0);
        a1 = fmaf(__ldcs(&v[3 * nb + j]), xv.x, a1);
        a1 = fmaf(__ldcs(&v[4 * nb + j]), xv.y, a1);
        a1 = fmaf(__ldcs(&v[5 * nb + j]), xv.z, a1);
        a2 = fmaf(__ldcs(&v[6 * nb + j]), xv.x, a2);
        a2 = fmaf(__ldcs(&v[7 * nb + j]), xv.y, a2);
        a2 = fmaf(__ldcs(&v[8 * nb + j]), xv.z, a2);
      }
      for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
      }
      if (lane == t) {
        m0 = a0;
        m1 = a1;
        m2 = a2;
      }
    }
    if (lane < nrow) {
      const int64_t I = I0 + lane;
      q[3 * I] = m0;
      q[3 * I + 1] = m1;
      q[3 * I + 2] = m2;
      const float4 pv = p4[I];
      pq.add(pv.x * m0);
      pq.add(pv.y * m1);
      pq.add(pv.z * m2);
    }
  }
  double vv[1] = {pq.get()}, tot[1];
  if (grid_reduce<1>(vv, R, tot) && threadIdx.x == 0) {
    R.scal[S_PQ] = tot[0];
    R.scal[S_ALPHA] = R.scal[S_RHO] / tot[0];
    R.iscal[I_SP32]++;
  }
}

// the same with two block rows in flight per warp (row t and row t + 16 of the
// tile processed together), doubling the independent loads per lane
__global__ void __launch_bounds__(kThreads) k_mx_bsr3x2(const int64_t *__restrict__ bptr, const int32_t *__restrict__ bcol,
                                                        const float *__restrict__ bval, const float4 *__restrict__ p4,
                                                        float *__restrict__ q, int64_t nbrow, Red R) {
  if (!active(R.iscal)) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int64_t nwarps = (int64_t)gridDim.x * blockDim.x / 32;
  KSum pq;
  for (int64_t I0 = warp_id * 32; I0 < nbrow; I0 += nwarps * 32) {
    const int nrow = (int)min((int64_t)32, nbrow - I0);
    const int64_t mybeg = lane < nrow ? bptr[I0 + lane] : 0;
    const int64_t myend = lane < nrow ? bptr[I0 + lane + 1] : 0;
    float m0 = 0.f, m1 = 0.f, m2 = 0.f;
    for (int t = 0; t < 16; t++) {
      const int tb = t + 16;
      const int64_t b0 = __shfl_sync(0xffffffffu, mybeg, t), e0 = __shfl_sync(0xffffffffu, myend, t);
      const int64_t b1 = __shfl_sync(0xffffffffu, mybeg, tb), e1 = __shfl_sync(0xffffffffu, myend, tb);
      const int na = t < nrow ? (int)(e0 - b0) : 0;
      const int nbb = tb < nrow ? (int)(e1 - b1) : 0;
      const float *va = bval + 9 * b0, *vb = bval + 9 * b1;
      float a0 = 0.f, a1 = 0.f, a2 = 0.f, c0 = 0.f, c1 = 0.f, c2 = 0.f;
      const int nmax = na > nbb ? na : nbb;
      for (int j = lane; j < nmax; j += 32) {
        if (j < na) {
          const float4 xv = __ldg(&p4[__ldcs(&bcol[b0 + j])]);
          a0 = fmaf(__ldcs(&va[0 * na + j]), xv.x, a0);
          a0 = fmaf(__ldcs(&va[1 * na + j]), xv.y, a0);
          a0 = fmaf(__ldcs(&va[2 * na + j]), xv.z, a0);
          a1 = fmaf(__ldcs(&va[3 * na + j]), xv.x, a1);
          a1 = fmaf(__ldcs(&va[4 * na + j]), xv.y, a1);
          a1 = fmaf(__ldcs(&va[5 * na + j]), xv.z, a1);
          a2 = fmaf(__ldcs(&va[6 * na + j]), xv.x, a2);
          a2 = fmaf(__ldcs(&va[7 * na + j]), xv.y, a2);
          a2 = fmaf(__ldcs(&va[8 * na + j]), xv.z, a2);
        }
        if (j < nbb) {
          const float4 xv = __ldg(&p4[__ldcs(&bcol[b1 + j])]);
          c0 = fmaf(__ldcs(&vb[0 * nbb + j]), xv.x, c0);
          c0 = fmaf(__ldcs(&vb[1 * nbb + j]), xv.y, c0);
          c0 = fmaf(__ldcs(&vb[2 * nbb + j]), xv.z, c0);
          c1 = fmaf(__ldcs(&vb[3 * nbb + j]), xv.x, c1);
          c1 = fmaf(__ldcs(&vb[4 * nbb + j]), xv.y, c1);
          c1 = fmaf(__ldcs(&vb[5 * nbb + j]), xv.z, c1);
          c2 = fmaf(__ldcs(&vb[6 * nbb + j]), xv.x, c2);
          c2 = fmaf(__ldcs(&vb[7 * nbb + j]), xv.y, c2);
          c2 = fmaf(__ldcs(&vb[8 * nbb + j]), xv.z, c2);
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
        c0 += __shfl_xor_sync(0xffffffffu, c0, o);
        c1 += __shfl_xor_sync(0xffffffffu, c1, o);
        c2 += __shfl_xor_sync(0xffffffffu, c2, o);
      }
      if (lane == t) { m0 = a0; m1 = a1; m2 = a2; }
      if (lane == tb) { m0 = c0; m1 = c1; m2 = c2; }
    }
    if (lane < nrow) {
      const int64_t I = I0 + lane;
      q[3 * I] = m0;
      q[3 * I + 1] = m1;
      q[3 * I + 2] = m2;
      const float4 pv = p4[I];
      pq.add(pv.x * m0);
      pq.add(pv.y * m1);
      pq.add(pv.z * m2);
    }
  }
  double vv[1] = {pq.get()}, tot[1];
  if (grid_reduce<1>(vv, R, tot) && threadIdx.x == 0) {
    R.scal[S_PQ] = tot[0];
    R.scal[S_ALPHA] = R.scal[S_RHO] / tot[0];
    R.iscal[I_SP32]++;
  }
}

// ---- q = A32 p with the tile's value and column streams staged by TMA
// Each CTA walks tiles of kTmaRows block rows.  Thread 0 issues two bulk
// copies (cp.async.bulk, completion counted on an mbarrier) of the next tile's
// contiguous values and columns into the other shared-memory stage while the
// eight warps compute the current tile from shared memory; only the p gather
// still reads global memory.  Bulk copies need 16-byte aligned addresses and
// sizes, so each copy starts at the 16-byte boundary below the tile and the
// kernel indexes from the remainder.  Every wait is bounded: on a timeout the
// kernel records an error flag, waits (bounded) for its own copies and leaves.
constexpr int kTmaRows = 16;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  for (int64_t i = 0; i < (1ll << 24); i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

struct TmaArgs {
  const int64_t *bptr;
  const int32_t *bcol;
  const float *bval;
  const float4 *p4;
  float *q;
  int64_t nbrow, ntiles;
  uint32_t vcap, ccap;  // stage capacities in bytes
  int *err;
};

__device__ __forceinline__ void tma_issue(const TmaArgs &A, int64_t tile, float *sv, int32_t *sc, uint64_t *bar) {
  const int64_t I0 = tile * kTmaRows;
  const int64_t I1 = min(I0 + kTmaRows, A.nbrow);
  const int64_t b0 = A.bptr[I0], b1 = A.bptr[I1];
  const uintptr_t v0 = (uintptr_t)(A.bval + 9 * b0), v1 = (uintptr_t)(A.bval + 9 * b1);
  const uintptr_t c0 = (uintptr_t)(A.bcol + b0), c1 = (uintptr_t)(A.bcol + b1);
  const uintptr_t va = v0 & ~(uintptr_t)15, ca = c0 & ~(uintptr_t)15;
  uint32_t vb = (uint32_t)(((v1 - va) + 15) & ~(uintptr_t)15), cb = (uint32_t)(((c1 - ca) + 15) & ~(uintptr_t)15);
  if (vb == 0) vb = 16;  // (a tile always holds a diagonal block; stay within the allocation slack anyway)
  if (cb == 0) cb = 16;
  if (vb > A.vcap || cb > A.ccap) {  // cannot happen with the host's capacity; never copy out of bounds
    atomicOr(A.err, 1024);
    vb = 16;
    cb = 16;
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_expect_tx(bar, vb + cb);
  bulk_g2s(sv, (const void *)va, vb, bar);
  bulk_g2s(sc, (const void *)ca, cb, bar);
}

__global__ void __launch_bounds__(kThreads) k_mx_bsr3_tma(TmaArgs A, Red R) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ bool s_ok;
  if (!active(R.iscal)) return;
  float *sv[2] = {(float *)smem, (float *)(smem + A.vcap)};
  int32_t *sc[2] = {(int32_t *)(smem + 2 * A.vcap), (int32_t *)(smem + 2 * A.vcap + A.ccap)};
  uint64_t *bar = (uint64_t *)(smem + 2 * A.vcap + 2 * A.ccap);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int64_t first = blockIdx.x, step = gridDim.x;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (first < A.ntiles) tma_issue(A, first, sv[0], sc[0], &bar[0]);
  }
  __syncthreads();
  KSum pq;
  bool ok = true, next_issued = false;
  int it = 0;
  for (int64_t t = first; t < A.ntiles; t += step, it++) {
    const int st = it & 1;
    const uint32_t par = (uint32_t)((it >> 1) & 1);
    if (threadIdx.x == 0) {
      next_issued = t + step < A.ntiles;
      if (next_issued) tma_issue(A, t + step, sv[st ^ 1], sc[st ^ 1], &bar[st ^ 1]);
      s_ok = mbar_wait_bounded(&bar[st], par);  // one thread decides, so the exit is uniform
    }
    __syncthreads();
    if (!s_ok) {
      ok = false;
      break;
    }
    mbar_wait_bounded(&bar[st], par);  // already complete: gives every thread the acquire
    const int64_t I0 = t * kTmaRows;
    const int nrow = (int)min((int64_t)kTmaRows, A.nbrow - I0);
    const int64_t bt = A.bptr[I0];
    const int dv = (int)(((uintptr_t)(A.bval + 9 * bt) & 15) / 4);
    const int dc = (int)(((uintptr_t)(A.bcol + bt) & 15) / 4);
    for (int r = warp; r < nrow; r += nwarp) {
      const int64_t I = I0 + r;
      const int64_t b0 = A.bptr[I];
      const int nb = (int)(A.bptr[I + 1] - b0);
      const float *v = sv[st] + dv + 9 * (b0 - bt);
      const int32_t *cc = sc[st] + dc + (b0 - bt);
      float a0 = 0.f, a1 = 0.f, a2 = 0.f;
      for (int j = lane; j < nb; j += 32) {
        const float4 xv = __ldg(&A.p4[cc[j]]);
        a0 = fmaf(v[0 * nb + j], xv.x, a0);
        a0 = fmaf(v[1 * nb + j], xv.y, a0);
        a0 = fmaf(v[2 * nb + j], xv.z, a0);
        a1 = fmaf(v[3 * nb + j], xv.x, a1);
        a1 = fmaf(v[4 * nb + j], xv.y, a1);
        a1 = fmaf(v[5 * nb + j], xv.z, a1);
        a2 = fmaf(v[6 * nb + j], xv.x, a2);
        a2 = fmaf(v[7 * nb + j], xv.y, a2);
        a2 = fmaf(v[8 * nb + j], xv.z, a2);
      }
      for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
      }
      if (lane == 0) {
        A.q[3 * I] = a0;
        A.q[3 * I + 1] = a1;
        A.q[3 * I + 2] = a2;
        const float4 pv = A.p4[I];
        pq.add(pv.x * a0);
        pq.add(pv.y * a1);
        pq.add(pv.z * a2);
      }
    }
    __syncthreads();  // the stage is free for the copy issued next iteration
  }
  if (!ok) {
    // record, then give both copies still in flight -- the stage whose wait
    // timed out and the next tile's, issued just before -- another bounded
    // wait, so that no bulk copy lands in this CTA's shared memory after it leaves
    if (threadIdx.x == 0) {
      atomicOr(A.err, 512);
      mbar_wait_bounded(&bar[it & 1], (uint32_t)((it >> 1) & 1));
      if (next_issued) mbar_wait_bounded(&bar[(it & 1) ^ 1], (uint32_t)(((it + 1) >> 1) & 1));
    }
    __syncthreads();
  }
  double vv[1] = {pq.get()}, tot[1];
  if (grid_reduce<1>(vv, R, tot) && threadIdx.x == 0) {
    R.scal[S_PQ] = tot[0];
    R.scal[S_ALPHA] = R.scal[S_RHO] / tot[0];
    R.iscal[I_SP32]++;
  }
}

// ---- q = A32 p from the upper triangle of 3x3 blocks only (A symmetric)
// Block row I stores its diagonal block and the blocks J > I (9 planes per
// row, as the full block CSR).  y_I gets B p_J; the transposed products B^T p_I
// go to block row J with one float4 atomic add each (q is padded to four floats
// per block row and zeroed by the p-update kernel).  p.q is summed from the
// symmetric form: p_I.B p_I on the diagonal, 2 p_I.B p_J off it.
__global__ void __launch_bounds__(kThreads) k_mx_sym3(const int64_t *__restrict__ uptr, const int32_t *__restrict__ ucol,
                                                      const float *__restrict__ uval, const float4 *__restrict__ p4,
                                                      float4 *__restrict__ q4, int64_t nbrow, Red R) {
  if (!active(R.iscal)) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int64_t nwarps = (int64_t)gridDim.x * blockDim.x / 32;
  KSum pq;
  for (int64_t I = warp_id; I < nbrow; I += nwarps) {
    const int64_t b0 = uptr[I];
    const int nb = (int)(uptr[I + 1] - b0);
    const float *v = uval + 9 * b0;
    const float4 xi = __ldg(&p4[I]);
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    for (int j = lane; j < nb; j += 32) {
      const int J = __ldcs(&ucol[b0 + j]);
      const float4 xj = __ldg(&p4[J]);
      const float m00 = __ldcs(&v[0 * nb + j]), m01 = __ldcs(&v[1 * nb + j]), m02 = __ldcs(&v[2 * nb + j]);
      const float m10 = __ldcs(&v[3 * nb + j]), m11 = __ldcs(&v[4 * nb + j]), m12 = __ldcs(&v[5 * nb + j]);
      const float m20 = __ldcs(&v[6 * nb + j]), m21 = __ldcs(&v[7 * nb + j]), m22 = __ldcs(&v[8 * nb + j]);
      const float y0 = fmaf(m00, xj.x, fmaf(m01, xj.y, m02 * xj.z));
      const float y1 = fmaf(m10, xj.x, fmaf(m11, xj.y, m12 * xj.z));
      const float y2 = fmaf(m20, xj.x, fmaf(m21, xj.y, m22 * xj.z));
      a0 += y0;
      a1 += y1;
      a2 += y2;
      const float d = fmaf(xi.x, y0, fmaf(xi.y, y1, xi.z * y2));
      if (J != I) {
        float4 t;
        t.x = fmaf(m00, xi.x, fmaf(m10, xi.y, m20 * xi.z));
        t.y = fmaf(m01, xi.x, fmaf(m11, xi.y, m21 * xi.z));
        t.z = fmaf(m02, xi.x, fmaf(m12, xi.y, m22 * xi.z));
        t.w = 0.f;
        red_add_f4(&q4[J], t);
        pq.add(2.f * d);
      } else {
        pq.add(d);
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) red_add_f4(&q4[I], make_float4(a0, a1, a2, 0.f));
  }
  double vv[1] = {pq.get()}, tot[1];
  if (grid_reduce<1>(vv, R, tot) && threadIdx.x == 0) {
    R.scal[S_PQ] = tot[0];
    R.scal[S_ALPHA] = R.scal[S_RHO] / tot[0];
    R.iscal[I_SP32]++;
  }
}

// upper triangle of the block CSR: the suffix of every sorted block row from
// its diagonal block (counts first, then the copy)
__global__ void k_upper_count(const int64_t *__restrict__ bptr, const int32_t *__restrict__ bcol, int64_t nbrow,
                              int64_t *__restrict__ ucount, int *__restrict__ err) {
  const int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= nbrow) return;
  int64_t lo = bptr[I], hi = bptr[I + 1];
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (bcol[mid] < I) lo = mid + 1;
    else hi = mid;
  }
  if (lo >= bptr[I + 1] || bcol[lo] != I) atomicOr(err, 2048);
  ucount[I] = bptr[I + 1] - lo;
}

__global__ void k_upper_fill(const int64_t *__restrict__ bptr, const int32_t *__restrict__ bcol,
                             const float *__restrict__ bval, const int64_t *__restrict__ uptr, int64_t nbrow,
                             int32_t *__restrict__ ucol, float *__restrict__ uval) {
  const int lane = threadIdx.x & 31;
  const int64_t I = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  if (I >= nbrow) return;
  const int64_t b0 = bptr[I], nb = bptr[I + 1] - b0, u0 = uptr[I], nu = uptr[I + 1] - u0, skip = nb - nu;
  const float *v = bval + 9 * b0;
  float *w = uval + 9 * u0;
  for (int64_t j = lane; j < nu; j += 32) {
    ucol[u0 + j] = bcol[b0 + skip + j];
    for (int k = 0; k < 9; k++) w[k * nu + j] = v[k * nb + skip + j];
  }
}

// q = A32 p for 3x3 blocks in sliced ELL: slices of 32 block rows (sorted by
// length inside windows so a slice pads little), lane t owns row t of its
// slice and walks the slice's block columns; entry k (0..8) of the blocks of a
// slice column lives in plane k, so every load of a warp is 32 consecutive
// floats and every lane runs a long, independent FMA chain (no reductions).
__global__ void __launch_bounds__(kThreads) k_mx_sell3(const int64_t *__restrict__ soff, const int32_t *__restrict__ slen,
                                                       const int32_t *__restrict__ sperm, const int32_t *__restrict__ scol,
                                                       const float *__restrict__ sval, int64_t plane,
                                                       const float4 *__restrict__ p4, float *__restrict__ q,
                                                       int64_t nslice, Red R) {
  if (!active(R.iscal)) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int64_t nwarps = (int64_t)gridDim.x * blockDim.x / 32;
  KSum pq;
  for (int64_t sl = warp_id; sl < nslice; sl += nwarps) {
    const int64_t off = soff[sl] + lane;
    const int len = slen[sl];
    const int I = sperm[sl * 32 + lane];
    const int32_t *cp = scol + off;
    const float *vp = sval + off;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
#pragma unroll 2
    for (int j = 0; j < len; j++) {
      const int64_t e = (int64_t)j * 32;
      const float4 xv = __ldg(&p4[__ldcs(cp + e)]);
      a0 = fmaf(__ldcs(vp + e), xv.x, a0);
      a0 = fmaf(__ldcs(vp + plane + e), xv.y, a0);
      a0 = fmaf(__ldcs(vp + 2 * plane + e), xv.z, a0);
      a1 = fmaf(__ldcs(vp + 3 * plane + e), xv.x, a1);
      a1 = fmaf(__ldcs(vp + 4 * plane + e), xv.y, a1);
      a1 = fmaf(__ldcs(vp + 5 * plane + e), xv.z, a1);
      a2 = fmaf(__ldcs(vp + 6 * plane + e), xv.x, a2);
      a2 = fmaf(__ldcs(vp + 7 * plane + e), xv.y, a2);
      a2 = fmaf(__ldcs(vp + 8 * plane + e), xv.z, a2);
    }
    if (I >= 0) {
      q[3 * (int64_t)I] = a0;
      q[3 * (int64_t)I + 1] = a1;
      q[3 * (int64_t)I + 2] = a2;
      const float4 pv = p4[I];
      pq.add(pv.x * a0);
      pq.add(pv.y * a1);
      pq.add(pv.z * a2);
    }
  }
  double vv[1] = {pq.get()}, tot[1];
  if (grid_reduce<1>(vv, R, tot) && threadIdx.x == 0) {
    R.scal[S_PQ] = tot[0];
    R.scal[S_ALPHA] = R.scal[S_RHO] / tot[0];
    R.iscal[I_SP32]++;
  }
}

// q = A32 p over scalar CSR rows (FP32 values, TPR lanes per row)
template <int TPR>
__global__ void __launch_bounds__(kThreads) k_mx_csr(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                     const float *__restrict__ a32, const float *__restrict__ p,
                                                     float *__restrict__ q, int64_t n, Red R) {
  if (!active(R.iscal)) return;
  KSum pq;
  GPZ_ROW_LOOP(TPR, n) {
    const int64_t r = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = r < n;
    const float s = row_dot32<TPR>(ia, ja, a32, p, r, sub, valid);
    if (sub == 0 && valid) {
      q[r] = s;
      pq.add(p[r] * s);
    }
  }
  double vv[1] = {pq.get()}, tot[1];
  if (grid_reduce<1>(vv, R, tot) && threadIdx.x == 0) {
    R.scal[S_PQ] = tot[0];
    R.scal[S_ALPHA] = R.scal[S_RHO] / tot[0];
    R.iscal[I_SP32]++;
  }
}

// alpha = rho / pq; dx += alpha p; r -= alpha q; rho' = r.(M r), rr = r.r
__global__ void __launch_bounds__(kThreads) k_mx_update(float *__restrict__ dx, float *__restrict__ r,
                                                        const float *__restrict__ p, const float *__restrict__ q,
                                                        Prec32 M, int padded, int qpad, int64_t nunits, Red R) {
  if (!active(R.iscal)) return;
  const double pq = R.scal[S_PQ];
  const float alpha = (float)R.scal[S_ALPHA];
  const int bs = M.block ? 3 : 1;
  KSum rz, rr;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    for (int k = 0; k < bs; k++) {
      const int64_t i = u * bs + k;
      const float pi = p[pidx(i, padded)];
      dx[i] = fmaf(alpha, pi, dx[i]);
      const float ri = fmaf(-alpha, q[pidx(i, qpad)], r[i]);
      r[i] = ri;
      rr.add(ri * ri);
    }
    float z[3];
    apply_prec32(M, r, u, z);
    for (int k = 0; k < bs; k++) rz.add(r[u * bs + k] * z[k]);
  }
  double v[2] = {rz.get(), rr.get()}, tot[2];
  if (grid_reduce<2>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    if (!(pq > 0.0) || !isfinite(tot[1]) || !isfinite(tot[0])) is[I_BREAK] = 1;
    s[S_RHO1] = s[S_RHO];
    s[S_RHO] = tot[0];
    s[S_BETA] = tot[0] / s[S_RHO1];
    s[S_RR] = tot[1];
    if (tot[1] > s[S_MAXRR]) s[S_MAXRR] = tot[1];
    const double resid = sqrt(tot[1]) / s[S_NORMB];
    s[S_RESID] = resid;
    is[I_IT] += 1;
    is[I_RESTART] = 0;
    if (is[I_BREAK]) is[I_CONV] = 2;
    else if (resid <= s[S_TOL] || tot[1] < s[S_DELTA2] * s[S_MAXRR]) is[I_UPDATE] = 1;
  }
}

// fold the FP32 increment into the FP64 solution (when an update is requested,
// or unconditionally with force = 1 at the end of a solve)
__global__ void __launch_bounds__(kThreads) k_mx_foldx(double *__restrict__ x, float *__restrict__ dx, int64_t n,
                                                       int force, Red R) {
  if (!force && (R.iscal[I_UPDATE] != 1 || R.iscal[I_CONV] != 0)) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += (double)dx[i];
    dx[i] = 0.f;
  }
}

// r32 = r64 after a true-residual computation; rho = r.(M r) and the restart rule
__global__ void __launch_bounds__(kThreads) k_mx_r32(const double *__restrict__ r64, float *__restrict__ r32,
                                                     Prec32 M, int64_t nunits, Red R) {
  if (R.iscal[I_UPDATE] != 2) return;
  const int bs = M.block ? 3 : 1;
  KSum rz;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    for (int k = 0; k < bs; k++) r32[u * bs + k] = (float)r64[u * bs + k];
    float z[3];
    apply_prec32(M, r32, u, z);
    for (int k = 0; k < bs; k++) rz.add(r32[u * bs + k] * z[k]);
  }
  double v[1] = {rz.get()}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    if (is[I_IT] > 0 && (tot[0] > 4.0 * s[S_RHO] || tot[0] < 0.25 * s[S_RHO])) {
      is[I_RESTART] = 1;
      is[I_NRESTART] += 1;
    }
    s[S_RHO] = tot[0];
    s[S_BETA] = s[S_RHO1] != 0.0 ? tot[0] / s[S_RHO1] : 0.0;
    is[I_UPDATE] = 0;
  }
}

// ---- variable-size block Jacobi: whole connect blocks of any size
// (TPZBlockDiagonal of TPZBlockDiagonalStructMatrix, overlap = true) or the
// node-set blocks of TPZNodesetCompute (TPZSparseBlockDiagonal, overlap =
// false), Analysis/TPZAnalysis.cpp:1008-1107.  The FP64 vector kernels of CG
// walk blocks: one thread per block updates the block's equations and applies
// the block's inverse to them (blocks of 3 to a few dozen equations; the
// thread re-reads its own writes); the FP32 kernels of the mixed CG below take
// one thread per equation.
struct VBlk {
  const int64_t *off;     // [nb + 1] into eq
  const int64_t *eq;      // the blocks' equations
  const int64_t *ioff;    // [nb] first entry of the block's inverse
  const double *inv;      // FP64 inverses, row-major
  const float *inv32;     // FP32 copies (mixed CG), column-major
  int64_t nb;
  const int64_t *tile;    // [ntile + 1] first block of each tile of at most kThreads equations
  const int32_t *posblk;  // position in eq -> block
  int64_t ntile;
};

// z_i = sum_j inv[i][j] r[eq_j] for the n equations of one block (n <= kVbMax)
constexpr int kVbMax = 96;

// Gather block b of the matrix (full CSR) into its inverse slot, then invert
// it in place by Gauss-Jordan elimination without pivoting (the
// TPZFMatrix::Decompose_LU of TPZSparseBlockDiagonal does not pivot either).
// One warp per block: lanes over the rows for the gather, over the columns of
// each row for the elimination.  A zero or non-finite pivot sets err.
__global__ void __launch_bounds__(kThreads) k_vb_inv(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                     const double *__restrict__ a, VBlk V,
                                                     const int32_t *__restrict__ eqblk,
                                                     const int32_t *__restrict__ eqloc, double *__restrict__ inv,
                                                     int *__restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int64_t wstep = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < V.nb; b += wstep) {
    const int64_t o = V.off[b];
    const int n = (int)(V.off[b + 1] - o);
    double *M = inv + V.ioff[b];
    if (n > kVbMax) {
      if (lane == 0) atomicOr(err, 1 << 15);
      continue;
    }
    for (int k = lane; k < n * n; k += 32) M[k] = 0.0;
    __syncwarp();
    for (int i = lane; i < n; i += 32) {
      const int64_t e = V.eq[o + i];
      for (int64_t k = ia[e]; k < ia[e + 1]; k++) {
        const int32_t col = ja[k];
        if (eqblk[col] == (int32_t)b) M[i * n + eqloc[col]] = a[k];
      }
    }
    __syncwarp();
    bool bad = false;
    for (int k = 0; k < n; k++) {
      const double piv = M[k * n + k];
      bad = bad || !(piv != 0.0) || !isfinite(piv);
      const double pinv = 1.0 / piv;
      __syncwarp();
      for (int j = lane; j < n; j += 32) M[k * n + j] = (j == k ? 1.0 : M[k * n + j]) * pinv;
      __syncwarp();
      for (int i = 0; i < n; i++) {
        if (i == k) continue;
        const double f = M[i * n + k];
        __syncwarp();
        for (int j = lane; j < n; j += 32) M[i * n + j] = (j == k ? 0.0 : M[i * n + j]) - f * M[k * n + j];
        __syncwarp();
      }
    }
    if (bad && lane == 0) atomicOr(err, 256);
  }
}

// equation -> (block, position) maps for the gather above
__global__ void k_vb_maps(VBlk V, int32_t *__restrict__ eqblk, int32_t *__restrict__ eqloc) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= V.nb) return;
  for (int64_t k = V.off[b]; k < V.off[b + 1]; k++) {
    eqblk[V.eq[k]] = (int32_t)b;
    eqloc[V.eq[k]] = (int32_t)(k - V.off[b]);
  }
}

// z = M r over the variable blocks (gpz_precond_apply)
__global__ void __launch_bounds__(kThreads) k_vb_apply(const double *__restrict__ r, VBlk V, double *__restrict__ z) {
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < V.nb; b += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = V.off[b];
    const int n = (int)(V.off[b + 1] - o);
    const double *B = V.inv + V.ioff[b];
    for (int i = 0; i < n; i++) {
      double acc = 0.0;
      for (int j = 0; j < n; j++) acc += B[i * n + j] * r[V.eq[o + j]];
      z[V.eq[o + i]] = acc;
    }
  }
}

// z = M r for the point or 3x3 block Jacobi preconditioner
__global__ void __launch_bounds__(kThreads) k_prec_apply(const double *__restrict__ r, Prec M, int64_t nunits,
                                                         double *__restrict__ z) {
  const int bs = M.block ? 3 : 1;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    double t[3];
    apply_prec(M, r, u, t);
    for (int k = 0; k < bs; k++) z[u * bs + k] = t[k];
  }
}

// FP64 CG, kernel B: p = M r + beta p (p = M r at the first iteration / after a restart)
__global__ void __launch_bounds__(kThreads) k_vb_p(const double *__restrict__ r, VBlk V, double *__restrict__ p, Red R) {
  if (!active(R.iscal)) return;
  const bool first = R.iscal[I_IT] == 0 || R.iscal[I_RESTART] != 0;
  const double beta = first ? 0.0 : R.scal[S_BETA];
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < V.nb; b += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = V.off[b];
    const int n = (int)(V.off[b + 1] - o);
    const double *B = V.inv + V.ioff[b];
    for (int i = 0; i < n; i++) {
      double z = 0.0;
      for (int j = 0; j < n; j++) z += B[i * n + j] * r[V.eq[o + j]];
      const int64_t e = V.eq[o + i];
      p[e] = first ? z : z + beta * p[e];
    }
  }
}

// FP64 CG, kernel D: x += alpha p; r -= alpha q; rho' = r.(M r), rr = r.r (epilogue of k_cg_update)
__global__ void __launch_bounds__(kThreads) k_vb_update(double *__restrict__ x, double *__restrict__ r,
                                                        const double *__restrict__ p, const double *__restrict__ q,
                                                        VBlk V, Red R) {
  if (!active(R.iscal)) return;
  const double pq = R.scal[S_PQ];
  const double alpha = R.scal[S_ALPHA];
  double rz = 0.0, rr = 0.0;
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < V.nb; b += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = V.off[b];
    const int n = (int)(V.off[b + 1] - o);
    for (int i = 0; i < n; i++) {
      const int64_t e = V.eq[o + i];
      x[e] = x[e] + alpha * p[e];
      const double ri = r[e] - alpha * q[e];
      r[e] = ri;
      rr += ri * ri;
    }
    const double *B = V.inv + V.ioff[b];
    for (int i = 0; i < n; i++) {
      double z = 0.0;
      for (int j = 0; j < n; j++) z += B[i * n + j] * r[V.eq[o + j]];
      rz += r[V.eq[o + i]] * z;
    }
  }
  double v[2] = {rz, rr}, tot[2];
  if (grid_reduce<2>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    if (!(pq > 0.0) || !isfinite(tot[1]) || !isfinite(tot[0])) is[I_BREAK] = 1;
    s[S_RHO1] = s[S_RHO];
    s[S_RHO] = tot[0];
    s[S_BETA] = tot[0] / s[S_RHO1];
    s[S_RR] = tot[1];
    if (tot[1] > s[S_MAXRR]) s[S_MAXRR] = tot[1];
    const double resid = sqrt(tot[1]) / s[S_NORMB];
    s[S_RESID] = resid;
    is[I_IT] += 1;
    is[I_RESTART] = 0;
    if (is[I_BREAK]) is[I_CONV] = 2;
    else if (resid <= s[S_TOL]) is[I_CONV] = 1;
  }
}

// rho = r.(M r) after the initial residual (epilogue of k_precond_dot)
__global__ void __launch_bounds__(kThreads) k_vb_dot(const double *__restrict__ r, VBlk V, Red R) {
  if (R.iscal[I_UPDATE] != 2) return;
  double rz = 0.0;
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < V.nb; b += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = V.off[b];
    const int n = (int)(V.off[b + 1] - o);
    const double *B = V.inv + V.ioff[b];
    for (int i = 0; i < n; i++) {
      double z = 0.0;
      for (int j = 0; j < n; j++) z += B[i * n + j] * r[V.eq[o + j]];
      rz += r[V.eq[o + i]] * z;
    }
  }
  double v[1] = {rz}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    if (is[I_IT] > 0 && (tot[0] > 4.0 * s[S_RHO] || tot[0] < 0.25 * s[S_RHO])) {
      is[I_RESTART] = 1;
      is[I_NRESTART] += 1;
    }
    s[S_RHO] = tot[0];
    s[S_BETA] = s[S_RHO1] != 0.0 ? tot[0] / s[S_RHO1] : 0.0;
    is[I_UPDATE] = 0;
  }
}

// The FP32 kernels of the mixed CG take one thread per equation: a CTA walks
// tiles of whole blocks (at most kThreads equations), puts the tile's residual
// into shared memory and each thread forms its row of the block's product from
// there, the inverse read column by column (inv32 is column-major, so a
// block's threads read consecutive words).

// inv32[ioff + j n + i] = inv[ioff + i n + j] in FP32
__global__ void __launch_bounds__(kThreads) k_vb_inv32t(VBlk V, float *__restrict__ inv32) {
  const int64_t npos = V.nb > 0 ? V.off[V.nb] : 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < npos; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = V.posblk[k], o = V.off[b];
    const int n = (int)(V.off[b + 1] - o), i = (int)(k - o);
    const double *B = V.inv + V.ioff[b];
    float *T = inv32 + V.ioff[b];
    for (int j = 0; j < n; j++) T[j * n + i] = (float)B[i * n + j];
  }
}

// this thread's equation in tile t: n = 0 past the tile's end; s0 = the
// block's first slot in the tile's shared residual (the thread's own slot is
// threadIdx.x)
struct VbRow {
  int64_t e;
  int n, i, s0;
  const float *Bt;
};
__device__ __forceinline__ VbRow vb_row(const VBlk &V, int64_t t) {
  VbRow w{0, 0, 0, 0, nullptr};
  const int64_t k0 = V.off[V.tile[t]], k = k0 + threadIdx.x;
  if (k < V.off[V.tile[t + 1]]) {
    const int64_t b = V.posblk[k], o = V.off[b];
    w.n = (int)(V.off[b + 1] - o);
    w.i = (int)(k - o);
    w.s0 = (int)(o - k0);
    w.e = V.eq[k];
    w.Bt = V.inv32 + V.ioff[b];
  }
  return w;
}
__device__ __forceinline__ float vb_rowdot(const VbRow &w, const float *sh) {
  float z = 0.f;
  for (int j = 0; j < w.n; j++) z = fmaf(w.Bt[j * w.n + w.i], sh[w.s0 + j], z);
  return z;
}

// mixed CG: p = M r + beta p in FP32 (p and the atomically accumulated q padded like k_mx_p)
__global__ void __launch_bounds__(kThreads) k_vb32_p(const float *__restrict__ r, VBlk V, float *__restrict__ p,
                                                     int padded, float *__restrict__ qzero, Red R) {
  __shared__ float sh[kThreads];
  if (!active(R.iscal)) return;
  const bool first = R.iscal[I_IT] == 0 || R.iscal[I_RESTART] != 0;
  const float beta = first ? 0.f : (float)R.scal[S_BETA];
  for (int64_t t = blockIdx.x; t < V.ntile; t += gridDim.x) {
    const VbRow w = vb_row(V, t);
    if (w.n) sh[threadIdx.x] = r[w.e];
    __syncthreads();
    if (w.n) {
      const float z = vb_rowdot(w, sh);
      const int64_t jj = pidx(w.e, padded);
      p[jj] = first ? z : fmaf(beta, p[jj], z);
      if (qzero) qzero[jj] = 0.f;
    }
    __syncthreads();
  }
}

// mixed CG: dx += alpha p; r -= alpha q; rho' = r.(M r), rr = r.r (epilogue of k_mx_update)
__global__ void __launch_bounds__(kThreads) k_vb32_update(float *__restrict__ dx, float *__restrict__ r,
                                                          const float *__restrict__ p, const float *__restrict__ q,
                                                          VBlk V, int padded, int qpad, Red R) {
  __shared__ float sh[kThreads];
  if (!active(R.iscal)) return;
  const double pq = R.scal[S_PQ];
  const float alpha = (float)R.scal[S_ALPHA];
  KSum rz, rr;
  for (int64_t t = blockIdx.x; t < V.ntile; t += gridDim.x) {
    const VbRow w = vb_row(V, t);
    float ri = 0.f;
    if (w.n) {
      dx[w.e] = fmaf(alpha, p[pidx(w.e, padded)], dx[w.e]);
      ri = fmaf(-alpha, q[pidx(w.e, qpad)], r[w.e]);
      r[w.e] = ri;
      rr.add(ri * ri);
      sh[threadIdx.x] = ri;
    }
    __syncthreads();
    if (w.n) rz.add(ri * vb_rowdot(w, sh));
    __syncthreads();
  }
  double v[2] = {rz.get(), rr.get()}, tot[2];
  if (grid_reduce<2>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    if (!(pq > 0.0) || !isfinite(tot[1]) || !isfinite(tot[0])) is[I_BREAK] = 1;
    s[S_RHO1] = s[S_RHO];
    s[S_RHO] = tot[0];
    s[S_BETA] = tot[0] / s[S_RHO1];
    s[S_RR] = tot[1];
    if (tot[1] > s[S_MAXRR]) s[S_MAXRR] = tot[1];
    const double resid = sqrt(tot[1]) / s[S_NORMB];
    s[S_RESID] = resid;
    is[I_IT] += 1;
    is[I_RESTART] = 0;
    if (is[I_BREAK]) is[I_CONV] = 2;
    else if (resid <= s[S_TOL] || tot[1] < s[S_DELTA2] * s[S_MAXRR]) is[I_UPDATE] = 1;
  }
}

// mixed CG: r32 = r64 after a true-residual computation; rho = r.(M r), restart rule (epilogue of k_mx_r32)
__global__ void __launch_bounds__(kThreads) k_vb32_r32(const double *__restrict__ r64, float *__restrict__ r32, VBlk V,
                                                       Red R) {
  __shared__ float sh[kThreads];
  if (R.iscal[I_UPDATE] != 2) return;
  KSum rz;
  for (int64_t t = blockIdx.x; t < V.ntile; t += gridDim.x) {
    const VbRow w = vb_row(V, t);
    float ri = 0.f;
    if (w.n) {
      ri = (float)r64[w.e];
      r32[w.e] = ri;
      sh[threadIdx.x] = ri;
    }
    __syncthreads();
    if (w.n) rz.add(ri * vb_rowdot(w, sh));
    __syncthreads();
  }
  double v[1] = {rz.get()}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    if (is[I_IT] > 0 && (tot[0] > 4.0 * s[S_RHO] || tot[0] < 0.25 * s[S_RHO])) {
      is[I_RESTART] = 1;
      is[I_NRESTART] += 1;
    }
    s[S_RHO] = tot[0];
    s[S_BETA] = s[S_RHO1] != 0.0 ? tot[0] / s[S_RHO1] : 0.0;
    is[I_UPDATE] = 0;
  }
}

// ---- two-level block Jacobi (mixed CG): z = B^-1 r + P Ac^-1 P^T r, B the 3x3
// connect blocks, P trilinear from the coarse nodes to the vertex connects
// (see TwoLevel).  One application: k_tl_restrict (rc = P^T r), k_tl_csolve
// (zc = Ac^-1 rc, dense FP32), k_tl_z (z, rho = r.z, beta); then k_tl_p.
struct TlView {
  const int32_t *vtx_eq, *brow_vtx, *cfix;
  const float *acinv;  // [nc][ldc], rows padded to 16 bytes
  float *rc, *zc, *z;
  int nvx, nvy, nvz, s, mx, my, mz;
  int64_t nc, ldc;
  float *boxpart;      // [mx my mz][8][3]
};
TlView tl_view(TwoLevel &T) {
  return TlView{T.vtx_eq.p, T.brow_vtx.p, T.cfix.p, T.acinv32.p, T.rc.p, T.zc.p, T.z32.p, (int)T.lx[0] + 1,
                (int)T.lx[1] + 1, (int)T.lx[2] + 1, T.s, T.m[0], T.m[1], T.m[2], T.nc, T.ldc, T.boxpart.p};
}

// coarse position of lattice vertex v: box (I, J, K) and its local offsets
__device__ __forceinline__ void tl_locate(const TlView &T, int64_t v, int &I, int &J, int &K, float &tx, float &ty,
                                          float &tz) {
  const int v32 = (int)v;  // the vertex lattice has fewer than 2^31 vertices (two_level_build checks)
  const int vi = v32 % T.nvx, vj = (v32 / T.nvx) % T.nvy, vk = v32 / (T.nvx * T.nvy);
  I = min(vi / T.s, T.mx - 1);
  J = min(vj / T.s, T.my - 1);
  K = min(vk / T.s, T.mz - 1);
  const float is = 1.0f / (float)T.s;
  tx = (float)(vi - I * T.s) * is;
  ty = (float)(vj - J * T.s) * is;
  tz = (float)(vk - K * T.s) * is;
}
constexpr int kTlMaxSmem = 3072;  // coarse dofs kept in shared memory by the restriction (>= the largest system)

// rc = P^T r; r64 (optional): after a residual replacement (I_UPDATE 2) the
// FP64 residual is read instead of r (the learned flexible CG refreshes r
// only in its z kernel, which runs after this one).  One CTA per coarse box:
// the box's own vertices (lattice ranges [I s, (I + 1) s) per direction, the
// last box also the upper boundary, as tl_locate assigns them) give its eight
// corners' 24 sums, reduced in the CTA without atomics; the last CTA to finish
// adds the boxes' sums into rc node by node in a fixed order (deterministic).
__global__ void __launch_bounds__(kThreads) k_tl_restrict(const float *__restrict__ r, const double *__restrict__ r64,
                                                          TlView T, Red R) {
  if (!active(R.iscal)) return;
  __shared__ float sred[kThreads / 32][24];
  __shared__ bool last;
  const int box = blockIdx.x;
  const int I = box % T.mx, J = (box / T.mx) % T.my, K = box / (T.mx * T.my);
  const int x0 = I * T.s, y0 = J * T.s, z0 = K * T.s;
  const int cx = (I == T.mx - 1 ? T.nvx : x0 + T.s) - x0, cy = (J == T.my - 1 ? T.nvy : y0 + T.s) - y0,
            cz = (K == T.mz - 1 ? T.nvz : z0 + T.s) - z0;
  const float is = 1.0f / (float)T.s;
  const bool fresh = r64 && R.iscal[I_UPDATE] == 2;
  float acc[24];
#pragma unroll
  for (int k = 0; k < 24; k++) acc[k] = 0.f;
  for (int t = threadIdx.x; t < cx * cy * cz; t += blockDim.x) {
    const int li = t % cx, lj = (t / cx) % cy, lk = t / (cx * cy);
    const int64_t v = (x0 + li) + (int64_t)T.nvx * ((y0 + lj) + (int64_t)T.nvy * (z0 + lk));
    const int32_t eq = T.vtx_eq[v];
    if (eq < 0) continue;
    const float r0 = fresh ? (float)r64[eq] : r[eq], r1 = fresh ? (float)r64[eq + 1] : r[eq + 1],
                r2 = fresh ? (float)r64[eq + 2] : r[eq + 2];
    const float tx = (float)li * is, ty = (float)lj * is, tz = (float)lk * is;
#pragma unroll
    for (int cn = 0; cn < 8; cn++) {
      const float w = ((cn & 1) ? tx : 1.f - tx) * ((cn & 2) ? ty : 1.f - ty) * ((cn & 4) ? tz : 1.f - tz);
      acc[3 * cn] = fmaf(w, r0, acc[3 * cn]);
      acc[3 * cn + 1] = fmaf(w, r1, acc[3 * cn + 1]);
      acc[3 * cn + 2] = fmaf(w, r2, acc[3 * cn + 2]);
    }
  }
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 24; k++) {
    const float sum = warp_sumf(acc[k]);
    if (lane == 0) sred[wp][k] = sum;
  }
  __syncthreads();
  if (threadIdx.x < 24) {
    float sum = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) sum += sred[w][threadIdx.x];
    T.boxpart[(size_t)box * 24 + threadIdx.x] = sum;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(R.counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  const volatile float *bp = T.boxpart;
  const int nx = T.mx + 1, ny = T.my + 1;
  for (int64_t k = threadIdx.x; k < T.nc; k += blockDim.x) {
    const int node = (int)(k / 3), comp = (int)(k % 3);
    const int a = node % nx, b = (node / nx) % ny, c = node / (nx * ny);
    float sum = 0.f;
    for (int cn = 0; cn < 8; cn++) {
      const int bi = a - (cn & 1), bj = b - ((cn >> 1) & 1), bk = c - (cn >> 2);
      if (bi < 0 || bj < 0 || bk < 0 || bi >= T.mx || bj >= T.my || bk >= T.mz) continue;
      sum += bp[((size_t)(bi + T.mx * (bj + T.my * bk))) * 24 + cn * 3 + comp];
    }
    T.rc[k] = sum;
  }
  if (threadIdx.x == 0) *R.counter = 0u;
}

// zc = Ac^-1 rc (removed nodes: zero); one warp per coarse row, float4 loads of
// the padded rows (the padding columns are zero) against rc staged in shared memory
__global__ void __launch_bounds__(kThreads) k_tl_csolve(TlView T, Red R) {
  if (!active(R.iscal)) return;
  __shared__ __align__(16) float src[kTlMaxSmem];
  for (int64_t k = threadIdx.x; k < T.ldc; k += blockDim.x) src[k] = k < T.nc ? T.rc[k] : 0.f;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t n4 = T.ldc / 4;
  for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < T.nc;
       row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    const float4 *a = (const float4 *)(T.acinv + row * T.ldc);
    for (int64_t j = lane; j < n4; j += 32) {
      const float4 v = a[j], x = ((const float4 *)src)[j];
      acc[0] = fmaf(v.x, x.x, acc[0]);
      acc[1] = fmaf(v.y, x.y, acc[1]);
      acc[2] = fmaf(v.z, x.z, acc[2]);
      acc[3] = fmaf(v.w, x.w, acc[3]);
    }
    float t = (acc[0] + acc[1]) + (acc[2] + acc[3]);
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) T.zc[row] = T.cfix[row / 3] ? 0.f : t;
  }
}

// z = B^-1 r + P zc per 3x3 block row; rho = r.z (KSum), beta; after a residual
// replacement (I_UPDATE 2, set by k_reliable or the initial residual) the
// direction restarts when the replaced residual's norm differs from the
// recursive one by more than 2x; rc cleared for the next application.
__global__ void __launch_bounds__(kThreads) k_tl_z(const float *__restrict__ r, Prec32 M, TlView T, int64_t nunits,
                                                   Red R) {
  if (!active(R.iscal)) return;
  // the coarse correction (at most kTlMaxSmem values) staged in shared memory: each vertex row reads 24 of them
  __shared__ float szc[kTlMaxSmem];
  for (int64_t k = threadIdx.x; k < T.nc; k += blockDim.x) szc[k] = T.zc[k];
  __syncthreads();
  KSum rz;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    float z[3];
    apply_prec32(M, r, u, z);
    const int32_t v = T.brow_vtx[u];
    if (v >= 0) {
      int I, J, K;
      float t[3];
      tl_locate(T, v, I, J, K, t[0], t[1], t[2]);
#pragma unroll
      for (int cn = 0; cn < 8; cn++) {
        const int bx = cn & 1, by = (cn >> 1) & 1, bz = cn >> 2;
        const float w = (bx ? t[0] : 1.f - t[0]) * (by ? t[1] : 1.f - t[1]) * (bz ? t[2] : 1.f - t[2]);
        if (w == 0.f) continue;
        const int nd = (I + bx) + (T.mx + 1) * ((J + by) + (T.my + 1) * (K + bz));
        z[0] = fmaf(w, szc[3 * nd], z[0]);
        z[1] = fmaf(w, szc[3 * nd + 1], z[1]);
        z[2] = fmaf(w, szc[3 * nd + 2], z[2]);
      }
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
      T.z[3 * u + k] = z[k];
      rz.add(r[3 * u + k] * z[k]);
    }
  }
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < T.nc; k += (int64_t)gridDim.x * blockDim.x)
    T.rc[k] = 0.f;
  double v[1] = {rz.get()}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    if (!isfinite(tot[0]) || !(tot[0] > 0.0)) {
      is[I_BREAK] = 1;
      is[I_CONV] = 2;
    }
    if (is[I_UPDATE] == 2) {
      const double q = s[S_RRREC] > 0.0 ? s[S_TRUERR] / s[S_RRREC] : 1.0;
      if (is[I_IT] > 0 && (q > 4.0 || q < 0.25)) {
        is[I_RESTART] = 1;
        is[I_NRESTART] += 1;
      }
      is[I_UPDATE] = 0;
    }
    s[S_RHO1] = s[S_RHO];
    s[S_RHO] = tot[0];
    s[S_BETA] = s[S_RHO1] != 0.0 ? tot[0] / s[S_RHO1] : 0.0;
  }
}

// p = z + beta p (p = z at the first iteration / after a restart)
__global__ void __launch_bounds__(kThreads) k_tl_p(const float *__restrict__ z, float *__restrict__ p, int padded,
                                                   float *__restrict__ qzero, int64_t n, Red R) {
  if (!active(R.iscal)) return;
  const bool first = R.iscal[I_IT] == 0 || R.iscal[I_RESTART] != 0;
  const float beta = first ? 0.f : (float)R.scal[S_BETA];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = pidx(i, padded);
    p[j] = first ? z[i] : fmaf(beta, p[j], z[i]);
    if (qzero) qzero[j] = 0.f;
  }
}

// dx += alpha p; r -= alpha q; rr (the recursive ||r||^2 kept for the restart rule); the
// reliable-update request as k_mx_update; rho follows in k_tl_z
__global__ void __launch_bounds__(kThreads) k_tl_update(float *__restrict__ dx, float *__restrict__ r,
                                                        const float *__restrict__ p, const float *__restrict__ q,
                                                        int padded, int qpad, int64_t n, Red R) {
  if (!active(R.iscal)) return;
  const double pq = R.scal[S_PQ];
  const float alpha = (float)R.scal[S_ALPHA];
  KSum rr;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    dx[i] = fmaf(alpha, p[pidx(i, padded)], dx[i]);
    const float ri = fmaf(-alpha, q[pidx(i, qpad)], r[i]);
    r[i] = ri;
    rr.add(ri * ri);
  }
  double v[1] = {rr.get()}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    if (!(pq > 0.0) || !isfinite(tot[0])) is[I_BREAK] = 1;
    s[S_RR] = tot[0];
    s[S_RRREC] = tot[0];
    if (tot[0] > s[S_MAXRR]) s[S_MAXRR] = tot[0];
    const double resid = sqrt(tot[0]) / s[S_NORMB];
    s[S_RESID] = resid;
    is[I_IT] += 1;
    is[I_RESTART] = 0;
    if (is[I_BREAK]) is[I_CONV] = 2;
    else if (resid <= s[S_TOL] || tot[0] < s[S_DELTA2] * s[S_MAXRR]) is[I_UPDATE] = 1;
  }
}

// r32 = r64 after a true-residual computation (I_UPDATE 2; k_tl_z then forms rho and clears the flag)
__global__ void __launch_bounds__(kThreads) k_tl_r32(const double *__restrict__ r64, float *__restrict__ r32, int64_t n,
                                                     Red R) {
  if (R.iscal[I_UPDATE] != 2) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    r32[i] = (float)r64[i];
}

__global__ void k_to_f32(const double *__restrict__ a, float *__restrict__ b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

int pick_tpr(int64_t nnz, int64_t n) {  // FP64 rows: few lanes per row
  double avg = n ? (double)nnz / (double)n : 0.0;
  if (avg > 24) return 8;
  return 4;
}

int pick_tpr32(int64_t nnz, int64_t n) {  // FP32 rows: coalescing first
  double avg = n ? (double)nnz / (double)n : 0.0;
  if (avg > 48) return 32;
  if (avg > 20) return 16;
  if (avg > 8) return 8;
  return 4;
}

// ---------------------------------------------------------------- GMRES
// Restarted, left-preconditioned GMRES(m) of Solvers/LinearSolvers/gmres.h:68-168
// (SIAM Templates p. 20): modified Gram-Schmidt Arnoldi, Givens rotations,
// back-substitution Update (gmres.h:20-35).  The Krylov basis is kept
// unnormalised: column j of V holds v_j / vscale[j], so that normalising a new
// vector costs no extra pass; every consumer multiplies by vscale[j].
//
// One Arnoldi step i is 2 + (i + 1) kernels: w = A v_i; w = M w with
// h(0,i) = w.v_0; then for k = 0..i: w -= h(k,i) v_k fused with the next dot
// (h(k+1,i) = w.v_{k+1}, or ||w|| when k = i).  The CTA that finishes ||w||
// also applies the rotations and decides convergence.  A whole restart cycle
// is captured once as a CUDA graph; a device state word, written only by the
// last CTA of a reduction or by a one-thread kernel, lets every later kernel
// of a finished solve return at entry.
enum { GM_STATE = 0, GM_J, GM_K, GM_UPD, GM_MAXIT, GM_ITERS, GM_SP64, GM_NI };
enum { GMS_RUN = 0, GMS_CONV_PENDING = 1, GMS_CONV = 2, GMS_MAXIT_PENDING = 3, GMS_MAXIT = 4, GMS_BREAK = 5 };
enum { GMD_NORMB = 0, GMD_RESID, GMD_TOL, GMD_NS };

struct Gm {
  double *V;       // [m+1][n], column j scaled by vscale[j]
  double *H;       // [(m+1) x (m+1)], column-major, H(i,j) = H[j*(m+1)+i]
  double *s, *cs, *sn, *vscale, *y;
  double *d;       // GMD_* scalars
  int64_t *is;     // GM_* integers
  int m;
  int64_t n;
};

__device__ __forceinline__ double &gm_h(const Gm &G, int i, int j) { return G.H[(size_t)j * (G.m + 1) + i]; }
__device__ __forceinline__ bool gm_running(const Gm &G) { return G.is[GM_STATE] == GMS_RUN; }

__device__ __forceinline__ void gm_gen_rot(double dx, double dy, double &c, double &sv) {  // GeneratePlaneRotation
  if (dy == 0.0) {
    c = 1.0;
    sv = 0.0;
  } else if (fabs(dy) > fabs(dx)) {
    const double t = dx / dy;
    sv = 1.0 / sqrt(1.0 + t * t);
    c = t * sv;
  } else {
    const double t = dy / dx;
    c = 1.0 / sqrt(1.0 + t * t);
    sv = t * c;
  }
}
__device__ __forceinline__ void gm_app_rot(double &dx, double &dy, double c, double sv) {  // ApplyPlaneRotation
  const double t = c * dx + sv * dy;
  dy = -sv * dx + c * dy;
  dx = t;
}

// ||M b|| (the GMRES normb), ||b|| (for the reported true residual), x = 0 unless from_current
__global__ void __launch_bounds__(kThreads) k_gm_init(const double *__restrict__ b, double *__restrict__ x, Prec M,
                                                      int64_t nunits, int from_current, Gm G, double *normb_true,
                                                      Red R) {
  const int bs = M.block ? 3 : 1;
  double mbb = 0.0, bb = 0.0;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    double z[3];
    apply_prec(M, b, u, z);
    for (int k = 0; k < bs; k++) {
      const int64_t i = u * bs + k;
      mbb += z[k] * z[k];
      bb += b[i] * b[i];
      if (!from_current) x[i] = 0.0;
    }
  }
  double v[2] = {mbb, bb}, tot[2];
  if (grid_reduce<2>(v, R, tot) && threadIdx.x == 0) {
    const double nb = sqrt(tot[0]);
    G.d[GMD_NORMB] = nb == 0.0 ? 1.0 : nb;
    const double nt = sqrt(tot[1]);
    *normb_true = nt == 0.0 ? 1.0 : nt;
  }
}

// t = b - A x into V[0] (restart residual, before the preconditioner)
template <int TPR>
__global__ void __launch_bounds__(kThreads) k_gm_resid_spmv(const int64_t *__restrict__ ia,
                                                            const int32_t *__restrict__ ja,
                                                            const double *__restrict__ a,
                                                            const double *__restrict__ x,
                                                            const double *__restrict__ b, int initial, Gm G) {
  if (!initial) {
    const int64_t st = G.is[GM_STATE];
    if (G.is[GM_UPD] != 1 || (st != GMS_RUN && st != GMS_MAXIT_PENDING)) return;
  }
  GPZ_ROW_LOOP(TPR, G.n) {
    const int64_t i = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = i < G.n;
    const double s = row_dot64<TPR>(ia, ja, a, x, i, sub, valid);
    if (sub == 0 && valid) G.V[i] = b[i] - s;
  }
}

// r = M t in place in V[0], beta = ||r||; starts the next cycle or ends the solve
__global__ void __launch_bounds__(kThreads) k_gm_resid_prec(Prec M, int64_t nunits, int initial, Gm G, Red R) {
  if (!initial) {
    const int64_t st = G.is[GM_STATE];
    if (G.is[GM_UPD] != 1 || (st != GMS_RUN && st != GMS_MAXIT_PENDING)) return;
  }
  const int bs = M.block ? 3 : 1;
  double rr = 0.0;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    double z[3];
    apply_prec(M, G.V, u, z);
    for (int k = 0; k < bs; k++) {
      G.V[u * bs + k] = z[k];
      rr += z[k] * z[k];
    }
  }
  double v[1] = {rr}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    const double beta = sqrt(tot[0]);
    const double resid = beta / G.d[GMD_NORMB];
    int64_t *is = G.is;
    G.vscale[0] = beta > 0.0 ? 1.0 / beta : 0.0;
    for (int k = 0; k <= G.m; k++) G.s[k] = 0.0;
    G.s[0] = beta;
    G.d[GMD_RESID] = resid;
    is[GM_SP64] += 1;
    is[GM_UPD] = 0;
    if (!isfinite(resid)) {
      is[GM_STATE] = GMS_BREAK;
    } else if (initial) {
      // gmres.h:97-103: already converged -> x += r, max_iter = 0
      is[GM_STATE] = resid <= G.d[GMD_TOL] ? GMS_CONV : GMS_RUN;
      if (is[GM_STATE] == GMS_CONV) is[GM_ITERS] = 0;
      else if (is[GM_MAXIT] < 1) is[GM_STATE] = GMS_MAXIT;
    } else if (resid < G.d[GMD_TOL]) {
      is[GM_STATE] = GMS_CONV;
      is[GM_ITERS] = is[GM_J];
    } else if (is[GM_STATE] == GMS_MAXIT_PENDING) {
      is[GM_STATE] = GMS_MAXIT;
    }
  }
}

// w = vscale[i] A V[i] into V[i+1]
template <int TPR>
__global__ void __launch_bounds__(kThreads) k_gm_spmv(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                      const double *__restrict__ a, int i, Gm G) {
  if (!gm_running(G)) return;
  const double *vi = G.V + (size_t)i * G.n;
  double *w = G.V + (size_t)(i + 1) * G.n;
  const double sc = G.vscale[i];
  GPZ_ROW_LOOP(TPR, G.n) {
    const int64_t r = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = r < G.n;
    const double s = row_dot64<TPR>(ia, ja, a, vi, r, sub, valid);
    if (sub == 0 && valid) w[r] = sc * s;
  }
}

// w = M w, h(0,i) = w . v_0
__global__ void __launch_bounds__(kThreads) k_gm_prec_dot(Prec M, int64_t nunits, int i, Gm G, Red R) {
  if (!gm_running(G)) return;
  double *w = G.V + (size_t)(i + 1) * G.n;
  const double *v0 = G.V;
  const int bs = M.block ? 3 : 1;
  double d = 0.0;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    double z[3];
    apply_prec(M, w, u, z);
    for (int k = 0; k < bs; k++) {
      const int64_t q = u * bs + k;
      w[q] = z[k];
      d += z[k] * v0[q];
    }
  }
  double v[1] = {d}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) gm_h(G, 0, i) = tot[0] * G.vscale[0];
}

// w -= h(k,i) v_k, then h(k+1,i) = w . v_{k+1} (k < i) or, for k = i, the step's end:
// h(i+1,i) = ||w||, rotations, residual estimate |s(i+1)| / normb, convergence.
__global__ void __launch_bounds__(kThreads) k_gm_mgs(int i, int k, Gm G, Red R) {
  if (!gm_running(G)) return;
  double *w = G.V + (size_t)(i + 1) * G.n;
  const double *vk = G.V + (size_t)k * G.n;
  const double c = gm_h(G, k, i) * G.vscale[k];
  const bool last_k = k == i;
  const double *vn = last_k ? w : G.V + (size_t)(k + 1) * G.n;
  double d = 0.0;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < G.n; q += (int64_t)gridDim.x * blockDim.x) {
    const double wq = w[q] - c * vk[q];
    w[q] = wq;
    d += wq * (last_k ? wq : vn[q]);
  }
  double v[1] = {d}, tot[1];
  if (!grid_reduce<1>(v, R, tot) || threadIdx.x != 0) return;
  if (!last_k) {
    gm_h(G, k + 1, i) = tot[0] * G.vscale[k + 1];
    return;
  }
  int64_t *is = G.is;
  const double hn = sqrt(tot[0]);
  gm_h(G, i + 1, i) = hn;
  G.vscale[i + 1] = hn > 0.0 ? 1.0 / hn : 0.0;
  for (int kk = 0; kk < i; kk++) gm_app_rot(gm_h(G, kk, i), gm_h(G, kk + 1, i), G.cs[kk], G.sn[kk]);
  gm_gen_rot(gm_h(G, i, i), gm_h(G, i + 1, i), G.cs[i], G.sn[i]);
  gm_app_rot(gm_h(G, i, i), gm_h(G, i + 1, i), G.cs[i], G.sn[i]);
  gm_app_rot(G.s[i], G.s[i + 1], G.cs[i], G.sn[i]);
  const double resid = fabs(G.s[i + 1]) / G.d[GMD_NORMB];
  G.d[GMD_RESID] = resid;
  is[GM_SP64] += 1;
  if (!isfinite(resid)) {
    is[GM_STATE] = GMS_BREAK;
  } else if (resid < G.d[GMD_TOL]) {
    is[GM_STATE] = GMS_CONV_PENDING;
    is[GM_K] = i;
    is[GM_ITERS] = is[GM_J];
  } else {
    is[GM_J] += 1;
    if (is[GM_J] > is[GM_MAXIT]) {
      is[GM_STATE] = GMS_MAXIT_PENDING;
      is[GM_K] = i;
    } else if (i == G.m - 1) {
      is[GM_K] = i;
    }
  }
}

// Update (gmres.h:20-35): y = H(0:k,0:k)^-1 s(0:k), premultiplied by vscale;
// one thread.  Also arms (GM_UPD = 1) or disarms the x update that follows.
__global__ void k_gm_solve_y(Gm G) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int64_t *is = G.is;
  const int64_t st = is[GM_STATE];
  if (st != GMS_RUN && st != GMS_CONV_PENDING && st != GMS_MAXIT_PENDING) {
    is[GM_UPD] = 0;
    return;
  }
  const int k = (int)is[GM_K];
  for (int j = 0; j <= k; j++) G.y[j] = G.s[j];
  for (int i = k; i >= 0; i--) {
    G.y[i] /= gm_h(G, i, i);
    for (int j = i - 1; j >= 0; j--) G.y[j] -= gm_h(G, j, i) * G.y[i];
  }
  for (int j = 0; j <= k; j++) G.y[j] *= G.vscale[j];
  is[GM_UPD] = 1;
  if (st == GMS_CONV_PENDING) is[GM_STATE] = GMS_CONV;
}

// x += sum_{j<=k} y_j v_j
__global__ void __launch_bounds__(kThreads) k_gm_update_x(double *__restrict__ x, Gm G) {
  if (G.is[GM_UPD] != 1) return;
  const int k = (int)G.is[GM_K];
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < G.n; q += (int64_t)gridDim.x * blockDim.x) {
    double acc = x[q];
    for (int j = 0; j <= k; j++) acc += G.y[j] * G.V[(size_t)j * G.n + q];
    x[q] = acc;
  }
}

// x += r (gmres.h:99-100) when the initial residual already meets the tolerance
__global__ void __launch_bounds__(kThreads) k_gm_add_r(double *__restrict__ x, Gm G) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < G.n; q += (int64_t)gridDim.x * blockDim.x)
    x[q] += G.V[q];
}

// ---------------------------------------------------------------- flexible CG with the learned preconditioner
// Notay's flexible CG (one stored direction): alpha = rho / (p.q),
// beta = -(z_new . q) / (p.q), rho = z_new . r_new, with z = M r from
// gpz_learned.cuh.  When the learned correction is not a descent direction
// (z.r <= 0 or not finite) that iteration uses Jacobi (z = r / diag) instead;
// I_RESTART carries that choice to the direction update and I_NRESTART counts it.
__global__ void __launch_bounds__(kThreads) k_fcg_update(double *__restrict__ x, double *__restrict__ r,
                                                         float *__restrict__ r32, const double *__restrict__ p,
                                                         const double *__restrict__ q, int64_t n, int mixed, Red R) {
  if (!active(R.iscal)) return;
  const double alpha = R.scal[S_ALPHA];
  double rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    const double ri = r[i] - alpha * q[i];
    r[i] = ri;
    r32[i] = (float)ri;
    rr += ri * ri;
  }
  double v[1] = {rr}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    const double resid = sqrt(tot[0]) / s[S_NORMB];
    s[S_RR] = tot[0];
    s[S_RESID] = resid;
    is[I_IT] += 1;
    if (tot[0] > s[S_MAXRR]) s[S_MAXRR] = tot[0];
    if (!(s[S_PQ] > 0.0) || !isfinite(resid)) {
      is[I_BREAK] = 1;
      is[I_CONV] = 2;
    } else if (!mixed) {
      if (resid <= s[S_TOL]) is[I_CONV] = 1;
    } else if (resid <= s[S_TOL] || tot[0] < s[S_DELTA2] * s[S_MAXRR]) {
      is[I_UPDATE] = 1;  // the FP32-value q has drifted r: replace it by b - A64 x (k_reliable)
    }
  }
}

// q = A32 p32 (FP32 values and accumulation, the mixed learned flexible CG), p.q in FP64
template <int TPR>
__global__ void __launch_bounds__(kThreads) k_lfcg_spmv(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                        const float *__restrict__ a32, const float *__restrict__ p32,
                                                        const double *__restrict__ p, double *__restrict__ q, int64_t n,
                                                        Red R) {
  if (!active(R.iscal)) return;
  double pq = 0.0;
  GPZ_ROW_LOOP(TPR, n) {
    const int64_t i = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = i < n;
    const float sv = row_dot32<TPR>(ia, ja, a32, p32, i, sub, valid);
    if (sub == 0 && valid) {
      const double qi = (double)sv;
      q[i] = qi;
      pq += p[i] * qi;
    }
  }
  double v[1] = {pq}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    R.scal[S_PQ] = tot[0];
    R.scal[S_ALPHA] = R.scal[S_RHO] / tot[0];
    R.iscal[I_SP32]++;
  }
}

// reads the FP32 copy of r written by the update, or the FP64 r when it was
// just (re)computed (start, residual replacement: I_UPDATE == 2)
__global__ void __launch_bounds__(kThreads) k_fcg_t(LnView L, const double *__restrict__ r64,
                                                    const float *__restrict__ r32, Red R) {
  if (!active(R.iscal)) return;
  const bool fresh = R.iscal[I_UPDATE] == 2;
  if (L.NS >= 32) {  // a warp per element (3D elasticity: 81 equations)
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < L.E; e += nw) {
      if (fresh) ln_elem_t_warp<double, true>(L, r64, e, lane);
      else ln_elem_t_warp<float, true>(L, r32, e, lane);
    }
  } else {  // a thread per (element, column)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < L.E * L.R; i += (int64_t)gridDim.x * blockDim.x) {
      if (fresh) ln_elem_t16<double>(L, r64, i);
      else ln_elem_t16<float>(L, r32, i);
    }
  }
}

// ---- learned flexible CG over the mixed CG's FP32 operator (3 states: 3x3
// blocks or matrix-free elements).  As in the mixed CG, r, p, z and the
// solution increment dx are FP32 (x += dx and r = b - A64 x at reliable
// updates, k_mx_foldx / k_reliable); dots, alpha and beta are FP64.  p32 is in
// the operator's padded input layout, q32 in its output layout (qpad), and
// k_lfb_p clears q32 for the next accumulating launch (qzero).
__global__ void __launch_bounds__(kThreads) k_lfb_update(float *__restrict__ dx, float *__restrict__ r32,
                                                         const float *__restrict__ p32, const float *__restrict__ q32,
                                                         int qpad, int64_t n, Red R) {
  if (!active(R.iscal)) return;
  const float alpha = (float)R.scal[S_ALPHA];
  KSum rr;  // compensated FP32 partial sums: GB300's FP64 rate would bound this kernel
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    dx[i] = fmaf(alpha, p32[pidx(i, 1)], dx[i]);
    const float ri = fmaf(-alpha, q32[pidx(i, qpad)], r32[i]);
    r32[i] = ri;
    rr.add(ri * ri);
  }
  double v[1] = {rr.get()}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    const double resid = sqrt(tot[0]) / s[S_NORMB];
    s[S_RR] = tot[0];
    s[S_RESID] = resid;
    is[I_IT] += 1;
    if (tot[0] > s[S_MAXRR]) s[S_MAXRR] = tot[0];
    if (!(s[S_PQ] > 0.0) || !isfinite(resid)) {
      is[I_BREAK] = 1;
      is[I_CONV] = 2;
    } else if (resid <= s[S_TOL] || tot[0] < s[S_DELTA2] * s[S_MAXRR]) {
      is[I_UPDATE] = 1;  // replace r by b - A64 x (k_mx_foldx, k_reliable)
    }
  }
}

// z = M r (FP32 out), the dots of the flexible recurrence and of the Jacobi
// fallback; after a replacement (I_UPDATE == 2) r is the fresh FP64 residual
// and r32 is refreshed from it
__global__ void __launch_bounds__(kThreads) k_lfb_z(LnView L, const double *__restrict__ r64, float *__restrict__ r32,
                                                    const float *__restrict__ q32, int qpad, float *__restrict__ z32,
                                                    Red R) {
  if (!active(R.iscal)) return;
  const bool first = R.iscal[I_IT] == 0;
  const bool fresh = R.iscal[I_UPDATE] == 2;
  const float alpha = expf(*L.loga);
  // FP32 arithmetic, compensated FP32 partial dots (FP64 across threads and CTAs)
  KSum zr, zq, jr, jq;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += (int64_t)gridDim.x * blockDim.x) {
    float ri;
    if (fresh) {
      ri = (float)r64[i];
      r32[i] = ri;
    } else {
      ri = r32[i];
    }
    const float di = L.dinv32[i];
    const float zi = fmaf(alpha * di, ri, ln_node_corr_ne(L, i));
    const float ji = di * ri;
    z32[i] = zi;
    zr.add(zi * ri);
    jr.add(ji * ri);
    if (!first) {
      const float qi = q32[pidx(i, qpad)];
      zq.add(zi * qi);
      jq.add(ji * qi);
    }
  }
  double v[4] = {zr.get(), zq.get(), jr.get(), jq.get()}, tot[4];
  if (grid_reduce<4>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    const bool ok = tot[0] > 0.0 && isfinite(tot[0]) && isfinite(tot[1]);
    is[I_RESTART] = ok ? 0 : 1;
    if (!ok) is[I_NRESTART] += 1;
    s[S_RHO] = ok ? tot[0] : tot[2];
    s[S_BETA] = first ? 0.0 : -(ok ? tot[1] : tot[3]) / s[S_PQ];
    if (is[I_UPDATE] == 2) is[I_UPDATE] = 0;
  }
}

// The same for meshes whose connects all carry 3 equations (Q2 elasticity):
// one thread per connect; its elements (the connect -> element list, in the
// order of the incidence lists) and their t_e are loaded once for the three
// equations, whose incidence-ordered rows sit at ne_ptr[eq] + r.
__global__ void __launch_bounds__(kThreads) k_lfb_z3(LnView L, const int64_t *__restrict__ ce_ptr,
                                                     const int32_t *__restrict__ ce_idx,
                                                     const int64_t *__restrict__ bpos,
                                                     const int32_t *__restrict__ bsize, int64_t nconn,
                                                     const double *__restrict__ r64, float *__restrict__ r32,
                                                     const float *__restrict__ q32, int qpad, float *__restrict__ z32,
                                                     const float *__restrict__ bjinv32, TlView T,
                                                     float *__restrict__ zb, Red R) {
  if (!active(R.iscal)) return;
  const bool first = R.iscal[I_IT] == 0;
  const bool fresh = R.iscal[I_UPDATE] == 2;
  const float alpha = expf(*L.loga);
  KSum zr, zq, jr, jq;
  for (int64_t cn = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; cn < nconn; cn += (int64_t)gridDim.x * blockDim.x) {
    if (bsize[cn] != 3) continue;
    const int64_t eq0 = bpos[cn];
    // the base preconditioner of this connect: point Jacobi, or its 3x3 block plus the coarse correction
    float rv[3], bz[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int j = 0; j < 3; j++) {
      rv[j] = fresh ? (float)r64[eq0 + j] : r32[eq0 + j];
      if (fresh) r32[eq0 + j] = rv[j];
    }
    if (bjinv32) {
      const float *Bk = bjinv32 + 9 * (eq0 / 3);
#pragma unroll
      for (int j = 0; j < 3; j++) bz[j] = fmaf(Bk[3 * j], rv[0], fmaf(Bk[3 * j + 1], rv[1], Bk[3 * j + 2] * rv[2]));
    } else {
#pragma unroll
      for (int j = 0; j < 3; j++) bz[j] = L.dinv32[eq0 + j] * rv[j];
    }
    float cz[3] = {0.f, 0.f, 0.f};
    if (T.zc) {
      const int32_t v = T.brow_vtx[eq0 / 3];
      if (v >= 0) {
        int I, J, K;
        float t[3];
        tl_locate(T, v, I, J, K, t[0], t[1], t[2]);
#pragma unroll
        for (int c8 = 0; c8 < 8; c8++) {
          const int bx = c8 & 1, by = (c8 >> 1) & 1, bz8 = c8 >> 2;
          const float w = (bx ? t[0] : 1.f - t[0]) * (by ? t[1] : 1.f - t[1]) * (bz8 ? t[2] : 1.f - t[2]);
          if (w == 0.f) continue;
          const int64_t nd = (I + bx) + (int64_t)(T.mx + 1) * ((J + by) + (int64_t)(T.my + 1) * (K + bz8));
#pragma unroll
          for (int j = 0; j < 3; j++) cz[j] = fmaf(w, __ldcg(&T.zc[3 * nd + j]), cz[j]);
        }
      }
    }
    const int64_t c0 = ce_ptr[cn], m = ce_ptr[cn + 1] - c0;
    const int64_t p0 = L.ne_ptr[eq0], p1 = L.ne_ptr[eq0 + 1], p2 = L.ne_ptr[eq0 + 2];
    float a[3] = {0.f, 0.f, 0.f};
    for (int64_t r = 0; r < m; r++) {
      const int32_t e = ce_idx[c0 + r];
      const float4 t0 = *(const float4 *)(L.t + (size_t)e * 8), t1 = *(const float4 *)(L.t + (size_t)e * 8 + 4);
      const int64_t pr[3] = {p0 + r, p1 + r, p2 + r};
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const uint4 v = *(const uint4 *)(L.F16ne + (size_t)pr[j] * 8);
        a[j] += __uint_as_float(v.x << 16) * t0.x + __uint_as_float(v.x & 0xffff0000u) * t0.y +
                __uint_as_float(v.y << 16) * t0.z + __uint_as_float(v.y & 0xffff0000u) * t0.w +
                __uint_as_float(v.z << 16) * t1.x + __uint_as_float(v.z & 0xffff0000u) * t1.y +
                __uint_as_float(v.w << 16) * t1.z + __uint_as_float(v.w & 0xffff0000u) * t1.w;
      }
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int64_t i = eq0 + j;
      const float ri = rv[j];
      const float zi = fmaf(alpha, bz[j], L.mdsq[i] * a[j]) + cz[j];
      const float ji = bz[j] + cz[j];  // the base alone: the fallback direction
      z32[i] = zi;
      if (zb) zb[i] = ji;
      zr.add(zi * ri);
      jr.add(ji * ri);
      if (!first) {
        const float qi = q32[pidx(i, qpad)];
        zq.add(zi * qi);
        jq.add(ji * qi);
      }
    }
  }
  double v[4] = {zr.get(), zq.get(), jr.get(), jq.get()}, tot[4];
  if (grid_reduce<4>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    const bool ok = tot[0] > 0.0 && isfinite(tot[0]) && isfinite(tot[1]);
    is[I_RESTART] = ok ? 0 : 1;
    if (!ok) is[I_NRESTART] += 1;
    s[S_RHO] = ok ? tot[0] : tot[2];
    s[S_BETA] = first ? 0.0 : -(ok ? tot[1] : tot[3]) / s[S_PQ];
    if (is[I_UPDATE] == 2) is[I_UPDATE] = 0;
  }
  if (T.zc)  // the coarse residual starts from zero at the next application
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < T.nc; k += (int64_t)gridDim.x * blockDim.x)
      T.rc[k] = 0.f;
}

// p = z + beta p; in an iteration that fell back (I_RESTART) z is the base preconditioner's alone:
// zb when given, else the point Jacobi D^-1 r
__global__ void __launch_bounds__(kThreads) k_lfb_p(const float *__restrict__ z32, const float *__restrict__ r32,
                                                    const float *__restrict__ dinv32, const float *__restrict__ zb,
                                                    float *__restrict__ p32, float *__restrict__ q32, int qpad,
                                                    int qzero, int64_t n, Red R) {
  if (!active(R.iscal)) return;
  const bool jac = R.iscal[I_RESTART] != 0;
  const bool first = R.iscal[I_IT] == 0;
  const float beta = (float)R.scal[S_BETA];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float zi = jac ? (zb ? zb[i] : dinv32[i] * r32[i]) : z32[i];
    const int64_t k = pidx(i, 1);
    p32[k] = first ? zi : fmaf(beta, p32[k], zi);
    if (qzero) q32[pidx(i, qpad)] = 0.f;
  }
}

__global__ void __launch_bounds__(kThreads) k_fcg_z(LnView L, const double *__restrict__ r,
                                                    const double *__restrict__ q, const double *__restrict__ dinv,
                                                    double *__restrict__ z, Red R) {
  if (!active(R.iscal)) return;
  const bool first = R.iscal[I_IT] == 0;
  const double alpha = exp((double)*L.loga);
  double zr = 0.0, zq = 0.0, jr = 0.0, jq = 0.0;  // jr, jq: the Jacobi fallback's dots (FP64: its beta)
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += (int64_t)gridDim.x * blockDim.x) {
    const double zi = alpha * L.dinv[i] * r[i] + (double)ln_node_corr_ne(L, i);
    const double ri = r[i];
    const double ji = dinv[i] * ri;
    z[i] = zi;
    zr += zi * ri;
    jr += ji * ri;
    if (!first) {
      const double qi = q[i];
      zq += zi * qi;
      jq += ji * qi;
    }
  }
  double v[4] = {zr, zq, jr, jq}, tot[4];
  if (grid_reduce<4>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    const bool ok = tot[0] > 0.0 && isfinite(tot[0]) && isfinite(tot[1]);
    is[I_RESTART] = ok ? 0 : 1;
    if (!ok) is[I_NRESTART] += 1;
    s[S_RHO] = ok ? tot[0] : tot[2];
    s[S_BETA] = first ? 0.0 : -(ok ? tot[1] : tot[3]) / s[S_PQ];
    if (is[I_UPDATE] == 2) is[I_UPDATE] = 0;
  }
}

__global__ void __launch_bounds__(kThreads) k_fcg_p(const double *__restrict__ z, const double *__restrict__ r,
                                                    const double *__restrict__ dinv, double *__restrict__ p,
                                                    float *__restrict__ p32, int64_t n, Red R) {
  if (!active(R.iscal)) return;
  const bool jac = R.iscal[I_RESTART] != 0;
  const bool first = R.iscal[I_IT] == 0;
  const double beta = R.scal[S_BETA];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double zi = jac ? dinv[i] * r[i] : z[i];
    const double pi = first ? zi : zi + beta * p[i];
    p[i] = pi;
    if (p32) p32[i] = (float)pi;
  }
}

#define GPZ_TPR_SWITCH(tpr, KERNEL_CALL) \
  switch (tpr) {                         \
    case 32: { constexpr int T = 32; KERNEL_CALL; } break; \
    case 16: { constexpr int T = 16; KERNEL_CALL; } break; \
    case 8: { constexpr int T = 8; KERNEL_CALL; } break;   \
    default: { constexpr int T = 4; KERNEL_CALL; } break;  \
  }

}  // namespace

void spmv_device(Ctx &c, const double *x, double *y, double alpha, double beta, const double *yin) {
  int tpr = pick_tpr(c.nnz, c.neq);
  GPZ_TPR_SWITCH(tpr, (k_spmv64<T><<<wave(k_spmv64<T>), kThreads, 0, c.stream>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, x, y, yin,
                                                                            alpha, beta, c.neq)));
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
}

// uniform 3x3 connect blocks (elasticity with one shape per connect)?
// (connects without shape functions hold no equations and are skipped, so the
// equation blocks are then 3k .. 3k+2 for k < neq / 3)
// Three states per shape, stored consecutively: the matrix is made of 3x3
// blocks (one per pair of shapes) whenever every connect block holds whole
// shapes, i.e. its size is a multiple of 3 (hp connects carry several shapes).
bool blocks_are_3(const Ctx &c) {
  if (c.nstate != 3 || c.neq == 0 || c.flt.active) return false;  // a filter may split the connect blocks
  for (int32_t s : c.h_block_size)
    if (s % 3 != 0) return false;
  return true;
}

// Sliced ELL of 3x3 blocks: block-row lengths from the row pointers, rows
// sorted by length (descending, stable) inside windows of `window` rows.
void build_sell(Ctx &c, Ctx::Sell &S, int64_t window) {
  std::vector<int64_t> ia(c.neq + 1);
  GPZ_CUDA_TRY(cudaMemcpyAsync(ia.data(), c.d_ia.p, (c.neq + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, c.stream));
  GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
  std::vector<int32_t> nb(c.nbrow);
  for (int64_t I = 0; I < c.nbrow; I++) nb[I] = (int32_t)((ia[3 * I + 1] - ia[3 * I]) / 3);
  std::vector<int32_t> perm(c.nbrow);
  for (int64_t I = 0; I < c.nbrow; I++) perm[I] = (int32_t)I;
  for (int64_t w0 = 0; w0 < c.nbrow; w0 += window) {
    int64_t w1 = std::min<int64_t>(w0 + window, c.nbrow);
    std::stable_sort(perm.begin() + w0, perm.begin() + w1, [&](int32_t x, int32_t y) { return nb[x] > nb[y]; });
  }
  S.window = window;
  S.nslice = (c.nbrow + 31) / 32;
  perm.resize(S.nslice * 32, -1);
  std::vector<int32_t> slen(S.nslice);
  std::vector<int64_t> soff(S.nslice + 1, 0);
  for (int64_t sl = 0; sl < S.nslice; sl++) {
    int32_t m = 0;
    for (int t = 0; t < 32; t++) {
      int32_t I = perm[sl * 32 + t];
      if (I >= 0) m = std::max(m, nb[I]);
    }
    slen[sl] = m;
    soff[sl + 1] = soff[sl] + 32 * (int64_t)m;
  }
  S.plane = soff[S.nslice];
  S.sperm.upload(perm.data(), perm.size(), c.stream);
  S.slen.upload(slen.data(), slen.size(), c.stream);
  S.soff.upload(soff.data(), soff.size(), c.stream);
  S.scol.alloc(std::max<int64_t>(S.plane, 1));
  S.sval.alloc((size_t)std::max<int64_t>(S.plane, 1) * 9);
  if (c.a32_tensor)
    k_fill_sell3<float><<<grid_for(S.nslice * 32, 256), 256, 0, c.stream>>>(
        c.d_ia.p, c.d_ja.p, c.d_a32.p, S.soff.p, S.slen.p, S.sperm.p, S.nslice, S.plane, S.scol.p, S.sval.p, c.d_err.p);
  else
    k_fill_sell3<double><<<grid_for(S.nslice * 32, 256), 256, 0, c.stream>>>(
        c.d_ia.p, c.d_ja.p, c.d_a.p, S.soff.p, S.slen.p, S.sperm.p, S.nslice, S.plane, S.scol.p, S.sval.p, c.d_err.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  check_device_flag(c, "sliced ELL of 3x3 blocks");
}

void alloc_work(Ctx &c, bool mixed);
Red red_of(Ctx &c);

// one launch of the FP32 3x3 SpMV variant v: q32 = A32 pm
void launch_spmv32(Ctx &c, int v, const Ctx::Sell &S, Red R, cudaStream_t s) {
  SolverWork &w = c.sw;
  if ((v >= 5 && v <= 8) || v == 10) {
    matfree_spmv(c, s, v == 10 ? 4 : v - 5);  // element by element (gpz_matfree.cu), counts its own launches
    return;
  }
  if (v == 0) {
    k_mx_bsr3<<<wave(k_mx_bsr3), kThreads, 0, s>>>(c.d_bptr.p, c.d_bcol.p, c.d_bval.p, (const float4 *)w.pm.p, w.q32.p,
                                                   c.nbrow, R);
  } else if (v == 1) {
    k_mx_bsr3x2<<<wave(k_mx_bsr3x2), kThreads, 0, s>>>(c.d_bptr.p, c.d_bcol.p, c.d_bval.p, (const float4 *)w.pm.p,
                                                       w.q32.p, c.nbrow, R);
  } else if (v == 4) {
    k_mx_sym3<<<wave(k_mx_sym3), kThreads, 0, s>>>(c.d_uptr.p, c.d_ucol.p, c.d_uval.p, (const float4 *)w.pm.p,
                                                   (float4 *)w.q32.p, c.nbrow, R);
  } else if (v == 3) {
    TmaArgs A{c.d_bptr.p, c.d_bcol.p, c.d_bval.p, (const float4 *)w.pm.p, w.q32.p, c.nbrow,
              (c.nbrow + kTmaRows - 1) / kTmaRows, c.tma_vcap, c.tma_ccap, c.d_err.p};
    const size_t sh = 2 * (size_t)c.tma_vcap + 2 * (size_t)c.tma_ccap + 16;
    k_mx_bsr3_tma<<<c.tma_grid, kThreads, sh, s>>>(A, R);
  } else {
    k_mx_sell3<<<wave(k_mx_sell3), kThreads, 0, s>>>(S.soff.p, S.slen.p, S.sperm.p, S.scol.p, S.sval.p, S.plane,
                                                     (const float4 *)w.pm.p, w.q32.p, S.nslice, R);
  }
  c.launches++;
}

const char *spmv32_name(int v);
void tune_scalar32(Ctx &c, int only, bool timing);

// Autotuner of the mixed CG's SpMV: every candidate layout / kernel is built
// and timed (CUDA events, 5 launches after 2 warm-up launches) on this matrix;
// the fastest is kept and the other layouts are released.
void finish_layout(Ctx &c, Ctx::Sell *cand, int k);

void tune_spmv32(Ctx &c, int only, bool timing) {
  cudaStream_t s = c.stream;
  alloc_work(c, true);
  SolverWork &w = c.sw;
  std::vector<float> ones(w.pm.n, 1.0f);
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.pm.p, ones.data(), ones.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  int64_t hi[I_NISCAL] = {0};
  hi[I_MAXIT] = 1;
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.iscal.p, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
  Red R = red_of(c);
  Ctx::Sell cand[2];
  const int64_t windows[2] = {64, 2048};
  struct Res { int v; int64_t window; float ms; };
  std::vector<Res> res;
  cudaEvent_t e0, e1;
  GPZ_CUDA_TRY(cudaEventCreate(&e0));
  GPZ_CUDA_TRY(cudaEventCreate(&e1));
  auto time_it = [&](int v, const Ctx::Sell &S) {
    if (!timing) return 0.0f;  // layout rebuilt for a known choice
    for (int i = 0; i < 2; i++) launch_spmv32(c, v, S, R, s);
    GPZ_CUDA_TRY(cudaEventRecord(e0, s));
    for (int i = 0; i < 5; i++) launch_spmv32(c, v, S, R, s);
    GPZ_CUDA_TRY(cudaEventRecord(e1, s));
    GPZ_CUDA_TRY(cudaEventSynchronize(e1));
    GPZ_CUDA_TRY(cudaGetLastError());
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms / 5;
  };
  auto want0 = [&](int v) { return only < 0 || only == v; };
  // The matrix-free operators are timed first (their records are cheap to
  // build); an assembled layout whose HBM bytes alone, at the device's
  // theoretical bandwidth, take longer than the best time measured so far
  // cannot win and is neither built nor timed.
  double peak_gbs = 0.0;
  {
    int dev = 0, clk_khz = 0, bus_bits = 0;
    GPZ_CUDA_TRY(cudaGetDevice(&dev));
    cudaDeviceGetAttribute(&clk_khz, cudaDevAttrMemoryClockRate, dev);
    cudaDeviceGetAttribute(&bus_bits, cudaDevAttrGlobalMemoryBusWidth, dev);
    peak_gbs = 2.0 * clk_khz * 1e3 * bus_bits / 8.0 / 1e9;
  }
  const double nb_full = (double)c.nnz / 9.0, nb_upper = (nb_full + (double)c.nbrow) / 2.0;
  auto floor_ms = [&](int v) {
    const double blocks = v == 4 ? nb_upper : nb_full;
    const double bytes = blocks * 40.0 + (double)(c.nbrow + 1) * 8.0 + (double)c.nbrow * 32.0;
    return peak_gbs > 0.0 ? bytes / (peak_gbs * 1e9) * 1e3 : 0.0;
  };
  float best_mf = -1.f;
  std::string pruned;
  if (timing && only < 0 && (want0(5) || want0(6) || want0(7) || want0(8) || want0(10)) && matfree_build(c)) {
    res.push_back({5, 0, time_it(5, cand[0])});
    if (c.mf.sf_ready) res.push_back({7, 0, time_it(7, cand[0])});
    res.push_back({6, 0, time_it(6, cand[0])});
    check_device_flag(c, "tensor-core matrix-free operator");
    if (c.mf.gm_ready) {
      res.push_back({8, 0, time_it(8, cand[0])});
      check_device_flag(c, "shared-element-matrix tensor-core operator");
    }
    if (c.mf.gt_ready) {
      res.push_back({10, 0, time_it(10, cand[0])});
      check_device_flag(c, "shared-element-matrix operator over lattice blocks");
    }
    for (const Res &r : res) best_mf = best_mf < 0.f ? r.ms : std::min(best_mf, r.ms);
  }
  auto want = [&](int v) {
    if (!want0(v)) return false;
    if (timing && best_mf > 0.f && floor_ms(v) >= best_mf) {
      const char *nm[5] = {"block_csr", "block_csr_2rows", "sliced_ell", "block_csr_tma_staged",
                           "upper_blocks_float4_atomics"};
      pruned += std::string(pruned.empty() ? "" : ", ") + "\"" + nm[v] + "\": " + std::to_string(floor_ms(v));
      return false;
    }
    return true;
  };
  if (want(0)) res.push_back({0, 0, time_it(0, cand[0])});
  if (want(1)) res.push_back({1, 0, time_it(1, cand[0])});
  if (want(3)) {
    // TMA-staged variant: per-stage capacity from the largest tile (+ alignment slack)
    std::vector<int64_t> bp(c.nbrow + 1);
    GPZ_CUDA_TRY(cudaMemcpyAsync(bp.data(), c.d_bptr.p, (c.nbrow + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));
    int64_t maxb = 0;
    for (int64_t I0 = 0; I0 < c.nbrow; I0 += kTmaRows)
      maxb = std::max(maxb, bp[std::min<int64_t>(I0 + kTmaRows, c.nbrow)] - bp[I0]);
    c.tma_vcap = (uint32_t)(((36 * maxb + 32) + 127) & ~127ll);
    c.tma_ccap = (uint32_t)(((4 * maxb + 32) + 127) & ~127ll);
    const size_t sh = 2 * (size_t)c.tma_vcap + 2 * (size_t)c.tma_ccap + 16;
    if (sh <= 200 * 1024) {
      GPZ_CUDA_TRY(cudaFuncSetAttribute(k_mx_bsr3_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
      int per = 0, nsm = 0, dev = 0;
      GPZ_CUDA_TRY(cudaGetDevice(&dev));
      GPZ_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
      GPZ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mx_bsr3_tma, kThreads, sh));
      c.tma_grid = std::max(1, std::min(kGridBlocks, nsm * std::max(per, 1)));
      res.push_back({3, 0, time_it(3, cand[0])});
      check_device_flag(c, "TMA-staged block SpMV");
    }
  }
  for (int k = 0; k < 2 && want(2); k++) {
    if (only == 2 && windows[k] != c.sell_window_tuned) continue;
    build_sell(c, cand[k], windows[k]);
    res.push_back({2, windows[k], time_it(2, cand[k])});
  }
  if (want(4)) {
    DBuf<int64_t> ucount;
    ucount.alloc(c.nbrow + 1);
    ucount.zero(s);
    k_upper_count<<<grid_for(c.nbrow, 256), 256, 0, s>>>(c.d_bptr.p, c.d_bcol.p, c.nbrow, ucount.p, c.d_err.p);
    c.launches++;
    GPZ_CUDA_TRY(cudaGetLastError());
    check_device_flag(c, "upper block count");
    c.d_uptr.alloc(c.nbrow + 1);
    exclusive_scan_i64(ucount.p, c.d_uptr.p, c.nbrow + 1, s, c);
    int64_t nu = 0;
    GPZ_CUDA_TRY(cudaMemcpyAsync(&nu, c.d_uptr.p + c.nbrow, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));
    c.d_ucol.alloc(std::max<int64_t>(nu, 1));
    c.d_uval.alloc((size_t)std::max<int64_t>(nu, 1) * 9);
    k_upper_fill<<<grid_for(c.nbrow * 32, 256), 256, 0, s>>>(c.d_bptr.p, c.d_bcol.p, c.d_bval.p, c.d_uptr.p, c.nbrow,
                                                             c.d_ucol.p, c.d_uval.p);
    c.launches++;
    GPZ_CUDA_TRY(cudaGetLastError());
    res.push_back({4, 0, time_it(4, cand[0])});
  }
  if (best_mf < 0.f && (want0(5) || want0(6) || want0(7) || want0(8) || want0(10)) && matfree_build(c)) {
    if (want0(5)) res.push_back({5, 0, time_it(5, cand[0])});
    if (want0(7) && c.mf.sf_ready) res.push_back({7, 0, time_it(7, cand[0])});
    if (want0(6)) {
      res.push_back({6, 0, time_it(6, cand[0])});
      check_device_flag(c, "tensor-core matrix-free operator");
    }
    if (want0(8) && c.mf.gm_ready) {
      res.push_back({8, 0, time_it(8, cand[0])});
      check_device_flag(c, "shared-element-matrix tensor-core operator");
    }
    if (want0(10) && c.mf.gt_ready) {
      res.push_back({10, 0, time_it(10, cand[0])});
      check_device_flag(c, "shared-element-matrix operator over lattice blocks");
    }
  }
  if (res.empty()) res.push_back({0, 0, time_it(0, cand[0])});
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  size_t best = 0;
  for (size_t i = 1; i < res.size(); i++)
    if (res[i].ms < res[best].ms) best = i;
  c.spmv32_variant = res[best].v;
  if (!timing) {
    finish_layout(c, cand, res[best].window == windows[0] ? 0 : 1);
    return;
  }
  c.sell_window_tuned = res[best].window ? res[best].window : c.sell_window_tuned;
  std::string rep = "{";
  for (size_t i = 0; i < res.size(); i++) {
    const char *nm = res[i].v == 0 ? "block_csr"
                     : res[i].v == 1 ? "block_csr_2rows"
                     : res[i].v == 3 ? "block_csr_tma_staged"
                     : res[i].v == 4 ? "upper_blocks_float4_atomics"
                     : res[i].v == 5 ? "matrix_free_elements"
                     : res[i].v == 6 ? "matrix_free_tcgen05_3xtf32"
                     : res[i].v == 7 ? "matrix_free_sum_factorised"
                     : res[i].v == 8 ? "matrix_free_shared_matrix_tcgen05"
                     : res[i].v == 10 ? "matrix_free_shared_matrix_lattice_blocks"
                                      : "sliced_ell";
    rep += std::string(i ? ", " : "") + "\"" + nm + (res[i].v == 2 ? "_w" + std::to_string(res[i].window) : "") +
           "\": " + std::to_string(res[i].ms);
  }
  int64_t nu = (c.nnz / 9 + c.nbrow) / 2;  // the block pattern is symmetric with every diagonal block stored
  if (c.d_uptr.p) {
    GPZ_CUDA_TRY(cudaMemcpy(&nu, c.d_uptr.p + c.nbrow, sizeof(int64_t), cudaMemcpyDeviceToHost));
  }
  if (!pruned.empty()) rep += ", \"pruned_by_byte_floor_ms\": {" + pruned + "}";
  c.tune_report = rep + ", \"chosen\": \"" + spmv32_name(res[best].v) + "\", \"block_rows\": " + std::to_string(c.nbrow) +
                  ", \"blocks_full\": " + std::to_string(c.nnz / 9) + ", \"blocks_upper\": " + std::to_string(nu) +
                  "}";
  finish_layout(c, cand, res[best].window == windows[0] ? 0 : 1);
}

// keep the chosen layout's arrays, drop the other candidates' (the block CSR
// stays allocated: the next assembly rebuilds the layout from it)
void finish_layout(Ctx &c, Ctx::Sell *cand, int k) {
  if (c.spmv32_variant != 2) {
    for (int i = 0; i < 2; i++) {
      cand[i].scol.release();
      cand[i].sval.release();
    }
  }
  if (c.spmv32_variant != 4) {
    c.d_uptr.release();
    c.d_ucol.release();
    c.d_uval.release();
  }
  if (c.spmv32_variant == 2) {
    Ctx::Sell &S = cand[k];
    c.sell.nslice = S.nslice;
    c.sell.plane = S.plane;
    c.sell.window = S.window;
    std::swap(c.sell.soff.p, S.soff.p); std::swap(c.sell.soff.n, S.soff.n);
    std::swap(c.sell.slen.p, S.slen.p); std::swap(c.sell.slen.n, S.slen.n);
    std::swap(c.sell.sperm.p, S.sperm.p); std::swap(c.sell.sperm.n, S.sperm.n);
    std::swap(c.sell.scol.p, S.scol.p); std::swap(c.sell.scol.n, S.scol.n);
    std::swap(c.sell.sval.p, S.sval.p); std::swap(c.sell.sval.n, S.sval.n);
  }
}

const char *spmv32_name(int v) {
  static const char *names[11] = {"block_csr", "block_csr_2rows", "sliced_ell", "block_csr_tma_staged",
                                  "upper_blocks_float4_atomics", "matrix_free_elements", "matrix_free_tcgen05_3xtf32",
                                  "matrix_free_sum_factorised", "matrix_free_shared_matrix_tcgen05",
                                  "matrix_free_shared_matrix_tcgen05_scalar", "matrix_free_shared_matrix_lattice_blocks"};
  return v >= 0 && v < 11 ? names[v] : "unknown";
}

void make_fp32_copy(Ctx &c, int variant) {
  c.have_bsr3 = false;
  if (blocks_are_3(c)) {
    c.nbrow = c.neq / 3;
    std::string key;
    int cached = -1;
    if (variant < 0 && c.spmv32_tuned < 0 && !c.tune_cache.empty()) {
      key = tune_key(c, "spmv32");
      cached = tune_cache_lookup(c, key);
    }
    // the block CSR: the source of every assembled layout; a known matrix-free choice does not read it
    const int known = variant >= 0 ? variant : c.spmv32_tuned >= 0 ? c.spmv32_tuned : cached;
    if (!((known >= 5 && known <= 8) || known == 10)) {
      c.d_bptr.alloc(c.nbrow + 1);
      c.d_bcol.alloc(std::max<int64_t>(c.nnz / 9, 1) + 16);  // slack for 16-byte rounded bulk copies
      c.d_bval.alloc(std::max<int64_t>(c.nnz, 1) + 16);
      if (c.a32_tensor)  // the FP32 element pass of this assembly
        k_build_bsr3<float><<<grid_for(c.nbrow * 32, 256), 256, 0, c.stream>>>(
            c.d_ia.p, c.d_ja.p, c.d_a32.p, c.nbrow, c.d_bptr.p, c.d_bcol.p, c.d_bval.p, c.d_err.p);
      else
        k_build_bsr3<double><<<grid_for(c.nbrow * 32, 256), 256, 0, c.stream>>>(
            c.d_ia.p, c.d_ja.p, c.d_a.p, c.nbrow, c.d_bptr.p, c.d_bcol.p, c.d_bval.p, c.d_err.p);
      c.launches++;
      GPZ_CUDA_TRY(cudaGetLastError());
      check_device_flag(c, "3x3 block CSR");
    }
    c.have_bsr3 = true;
    if (!c.a32_tensor) c.d_a32.release();  // (the FP32 element values stay: a later rebuild reads them)
    if (variant < 0 && c.spmv32_tuned >= 0) {
      tune_spmv32(c, c.spmv32_tuned, false);  // same pattern: rebuild the chosen layout only
    } else if (cached >= 0) {
      tune_spmv32(c, cached, false);  // a choice stored by an earlier run on this device and mesh
      c.spmv32_tuned = c.spmv32_variant;
      c.tune_report = std::string("{\"cached\": true, \"chosen\": \"") + spmv32_name(c.spmv32_variant) +
                      "\", \"block_rows\": " + std::to_string(c.nbrow) + "}";
    } else {
      tune_spmv32(c, variant, true);
      if (variant < 0) {
        c.spmv32_tuned = c.spmv32_variant;
        if (!key.empty()) tune_cache_store(c, key, c.spmv32_variant, c.tune_report);
      }
    }
  } else {
    if (!c.a32_tensor) {
      c.d_a32.alloc(std::max<int64_t>(c.nnz, 1));
      to_fp32(c);
    }
    std::string key;
    int cached = -1;
    if (variant < 0 && c.spmv32_tuned < 0 && !c.tune_cache.empty()) {
      key = tune_key(c, "spmv32");
      cached = tune_cache_lookup(c, key);
    }
    const int want = variant >= 0 ? variant : c.spmv32_tuned >= 0 ? c.spmv32_tuned : cached;
    tune_scalar32(c, want, want < 0);
    if (variant < 0) {
      if (c.spmv32_tuned < 0 && !key.empty() && cached < 0) tune_cache_store(c, key, c.spmv32_variant, c.tune_report);
      c.spmv32_tuned = c.spmv32_variant;
    }
  }
  c.have_a32 = true;
}

// FP32 operator of the scalar mixed CG: the FP32 CSR copy (k_mx_csr, variant 0)
// or, on translated Q2 hex grids, the scalar shared-matrix tcgen05 operator
// (variant 9); with timing, both are timed on this system (CUDA events, 5
// launches after 2) and the faster kept, else `only` is taken (-1: the CSR).
void tune_scalar32(Ctx &c, int only, bool timing) {
  c.spmv32_variant = 0;
  const bool mf = (timing || only == 9) && matfree1_build(c);
  if (!mf) {
    if (timing) c.tune_report = "{\"csr_fp32\": null, \"chosen\": \"csr_fp32\"}";
    return;
  }
  if (!timing) {
    c.spmv32_variant = 9;
    return;
  }
  cudaStream_t s = c.stream;
  alloc_work(c, true);
  SolverWork &w = c.sw;
  std::vector<float> ones(w.pm.n, 1.0f);
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.pm.p, ones.data(), ones.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  int64_t hi[I_NISCAL] = {0};
  hi[I_MAXIT] = 1;
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.iscal.p, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
  Red R = red_of(c);
  cudaEvent_t e0, e1;
  GPZ_CUDA_TRY(cudaEventCreate(&e0));
  GPZ_CUDA_TRY(cudaEventCreate(&e1));
  float ms[2] = {0.f, 0.f};
  for (int v = 0; v < 2; v++) {
    auto launch = [&]() {
      if (v == 1) {
        matfree1_spmv(c, s, w.pm.p, w.q32.p);
      } else {
        GPZ_TPR_SWITCH(pick_tpr32(c.nnz, c.neq), (k_mx_csr<T><<<wave(k_mx_csr<T>), kThreads, 0, s>>>(
                                                     c.d_ia.p, c.d_ja.p, c.d_a32.p, w.pm.p, w.q32.p, c.neq, R)));
        c.launches++;
      }
    };
    for (int i = 0; i < 2; i++) launch();
    GPZ_CUDA_TRY(cudaEventRecord(e0, s));
    for (int i = 0; i < 5; i++) launch();
    GPZ_CUDA_TRY(cudaEventRecord(e1, s));
    GPZ_CUDA_TRY(cudaEventSynchronize(e1));
    GPZ_CUDA_TRY(cudaGetLastError());
    cudaEventElapsedTime(&ms[v], e0, e1);
    ms[v] /= 5;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  check_device_flag(c, "scalar shared-element-matrix tensor-core operator");
  c.spmv32_variant = ms[1] < ms[0] ? 9 : 0;
  c.tune_report = "{\"csr_fp32\": " + std::to_string(ms[0]) + ", \"matrix_free_shared_matrix_tcgen05_scalar\": " +
                  std::to_string(ms[1]) + ", \"chosen\": \"" +
                  (c.spmv32_variant == 9 ? "matrix_free_shared_matrix_tcgen05_scalar" : "csr_fp32") + "\"}";
}

void build_block_jacobi(Ctx &c) {
  // per-shape 3x3 blocks: the connect blocks of TPZBlockDiagonal when every connect carries one shape
  GPZ_REQUIRE(blocks_are_3(c), GPZ_E_INVALID,
              "block Jacobi needs 3 states per shape (nstate 3) and no equation filter");
  const int64_t nb = c.neq / 3;
  c.d_bjinv.alloc((size_t)nb * 9);
  k_block_inv3<<<grid_for(nb, 256), 256, 0, c.stream>>>(c.d_a.p, c.d_diagpos.p, nb, c.d_bjinv.p, c.d_err.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  check_device_flag(c, "block Jacobi inverse");
  c.have_bjinv = true;
}

// every connect block holds 0 or 3 equations: the 3x3 block path applies
bool connect_blocks_are_3(const Ctx &c) {
  if (!blocks_are_3(c)) return false;
  for (int32_t s : c.h_block_size)
    if (s != 0 && s != 3) return false;
  return true;
}

// Blocks of the variable-size block Jacobi: kind GPZ_PRECOND_BLOCK_JACOBI = one
// block per connect (TPZBlockDiagonalStructMatrix, StrMatrix/pzbdstrmatrix.cpp:
// 13-97), GPZ_PRECOND_NODESET_JACOBI = the node-set blocks of the element
// graph (gpz_nodeset_blocks, TPZNodesetCompute); then the inverses of the
// assembled matrix's diagonal blocks on the device.
void build_vblocks(Ctx &c, int kind) {
  GPZ_REQUIRE(!c.flt.active && c.neq > 0, GPZ_E_INVALID,
              "block Jacobi with whole connect / node-set blocks: not available under an equation filter");
  cudaStream_t s = c.stream;
  if (c.vb_kind != kind) {
    std::vector<int64_t> off(1, 0), eq;
    const int64_t nconn = (int64_t)c.h_block_size.size();
    if (kind == GPZ_PRECOND_BLOCK_JACOBI) {
      for (int64_t cn = 0; cn < nconn; cn++) {
        if (c.h_block_size[cn] <= 0) continue;
        for (int32_t k = 0; k < c.h_block_size[cn]; k++) eq.push_back(c.h_block_pos[cn] + k);
        off.push_back((int64_t)eq.size());
      }
    } else {
      // TPZCompMesh::ComputeElGraph: every element's side connects
      const int64_t nel = (int64_t)c.h_el_type.size();
      std::vector<int64_t> gi(nel + 1, 0), g;
      for (int64_t e = 0; e < nel; e++) {
        const int t = c.h_el_type[e];
        const int ns = t == GPZ_EL_LINE ? 3 : (t == GPZ_EL_QUAD ? 9 : 27);
        for (int k = 0; k < ns; k++) g.push_back(c.h_el_conn[e * 27 + k]);
        gi[e + 1] = (int64_t)g.size();
      }
      std::vector<int64_t> bsz(c.h_block_size.begin(), c.h_block_size.end());
      std::vector<int64_t> bi(nconn + 1), be(std::max<int64_t>(c.neq, 1));
      std::vector<int> col(std::max<int64_t>(nconn, 1));
      int64_t nb = 0;
      int ncol = 0;
      const int rc = gpz_nodeset_blocks(nconn, nel, gi.data(), g.data(), c.h_block_pos.data(), bsz.data(), c.neq,
                                        bi.data(), be.data(), &nb, col.data(), &ncol, nullptr, nullptr);
      GPZ_REQUIRE(rc == GPZ_OK, rc, "node-set blocks of the element graph");
      off.assign(bi.begin(), bi.begin() + nb + 1);
      eq.assign(be.begin(), be.begin() + off[nb]);
    }
    int64_t nb = (int64_t)off.size() - 1;
    {  // blocks of one size next to each other (largest first): a warp's threads walk blocks of one size
      std::vector<int64_t> order(nb);
      for (int64_t b = 0; b < nb; b++) order[b] = b;
      std::stable_sort(order.begin(), order.end(),
                       [&](int64_t x, int64_t y) { return off[x + 1] - off[x] > off[y + 1] - off[y]; });
      std::vector<int64_t> off2(1, 0), eq2;
      eq2.reserve(eq.size());
      for (int64_t b : order) {
        eq2.insert(eq2.end(), eq.begin() + off[b], eq.begin() + off[b + 1]);
        off2.push_back((int64_t)eq2.size());
      }
      off.swap(off2);
      eq.swap(eq2);
    }
    std::vector<int64_t> ioff(std::max<int64_t>(nb, 1), 0);
    int64_t tot = 0;
    int maxn = 0;
    for (int64_t b = 0; b < nb; b++) {
      const int64_t n = off[b + 1] - off[b];
      GPZ_REQUIRE(n <= kVbMax, GPZ_E_INVALID, "block Jacobi: a block larger than 96 equations");
      ioff[b] = tot;
      tot += n * n;
      maxn = std::max(maxn, (int)n);
    }
    // tiles of whole consecutive blocks with at most kThreads equations (one CTA
    // of the FP32 kernels each), and position -> block
    std::vector<int64_t> tile(1, 0);
    std::vector<int32_t> posblk(std::max<size_t>(eq.size(), 1), 0);
    for (int64_t b = 0; b < nb; b++) {
      for (int64_t k = off[b]; k < off[b + 1]; k++) posblk[k] = (int32_t)b;
      if (off[b + 1] - off[tile.back()] > kThreads) tile.push_back(b);
    }
    if (nb > 0) tile.push_back(nb);
    c.d_vb_off.upload(off.data(), off.size(), s);
    c.d_vb_eq.upload(eq.data(), std::max<size_t>(eq.size(), 1), s);
    c.d_vb_ioff.upload(ioff.data(), ioff.size(), s);
    c.d_vb_tile.upload(tile.data(), tile.size(), s);
    c.d_vb_posblk.upload(posblk.data(), posblk.size(), s);
    c.vb_ntile = (int64_t)tile.size() - 1;
    c.d_vb_inv.alloc(std::max<int64_t>(tot, 1));
    c.d_vb_eqblk.alloc(std::max<int64_t>(c.neq, 1));
    c.d_vb_eqloc.alloc(std::max<int64_t>(c.neq, 1));
    GPZ_CUDA_TRY(cudaMemsetAsync(c.d_vb_eqblk.p, 0xff, c.d_vb_eqblk.n * sizeof(int32_t), s));  // -1: no block
    c.vb_nb = nb;
    c.vb_maxn = maxn;
    const VBlk V{c.d_vb_off.p, c.d_vb_eq.p, c.d_vb_ioff.p, nullptr, nullptr, nb};
    k_vb_maps<<<grid_for(std::max<int64_t>(nb, 1), 256), 256, 0, s>>>(V, c.d_vb_eqblk.p, c.d_vb_eqloc.p);
    c.launches++;
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));  // the host arrays above go out of scope
    c.vb_kind = kind;
    c.d_vb_inv32.release();
  }
  const VBlk V{c.d_vb_off.p, c.d_vb_eq.p, c.d_vb_ioff.p, nullptr, nullptr, c.vb_nb};
  k_vb_inv<<<grid_for(std::max<int64_t>(c.vb_nb, 1) * 32, 256), 256, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, V,
                                                                              c.d_vb_eqblk.p, c.d_vb_eqloc.p,
                                                                              c.d_vb_inv.p, c.d_err.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  check_device_flag(c, "block Jacobi inverses");
  c.have_vbinv = true;
}

VBlk vblk_of(const Ctx &c) {
  return VBlk{c.d_vb_off.p, c.d_vb_eq.p,     c.d_vb_ioff.p, c.d_vb_inv.p, c.d_vb_inv32.p,
              c.vb_nb,      c.d_vb_tile.p, c.d_vb_posblk.p, c.vb_ntile};
}

// ---- solver workspace and the iteration plan

void alloc_work(Ctx &c, bool mixed) {
  SolverWork &w = c.sw;
  int64_t n = std::max<int64_t>(c.neq, 1);
  w.r.alloc(n);
  w.p.alloc(n);
  w.q.alloc(n);
  w.x.alloc(n);
  w.b.alloc(n);
  if (mixed) {
    w.pm.alloc(c.have_bsr3 ? (size_t)std::max<int64_t>(c.nbrow, 1) * 4 : (size_t)n);
    w.r32.alloc(n);
    w.q32.alloc(c.have_bsr3 ? std::max<size_t>((size_t)n, (size_t)c.nbrow * 4) : (size_t)n);
    w.dx32.alloc(n);
  }
  w.partial.alloc((size_t)kGridBlocks * 4);
  w.scal.alloc(S_NSCAL);
  w.iscal.alloc(I_NISCAL);
  w.counter.alloc(1);
  w.counter.zero(c.stream);
}

Red red_of(Ctx &c) { return Red{c.sw.partial.p, c.sw.counter.p, c.sw.scal.p, c.sw.iscal.p}; }

struct Plan {
  bool mixed, block, bsr;
  bool mf1 = false;  // scalar shared-matrix operator (spmv variant 9)
  bool vb = false;  // variable-size block Jacobi
  bool tl = false;  // two-level block Jacobi (mixed CG)
  TlView T;
  int tpr, tpr32;
  int64_t nunits;
  Prec M;
  Prec32 M32;
  VBlk V;
};

// one application of the two-level preconditioner to r32 (after a possible residual refresh)
void launch_tl_apply(Ctx &c, const Plan &P, Red R, cudaStream_t s) {
  SolverWork &w = c.sw;
  k_tl_r32<<<wave(k_tl_r32), kThreads, 0, s>>>(w.r.p, w.r32.p, c.neq, R);
  k_tl_restrict<<<P.T.mx * P.T.my * P.T.mz, kThreads, 0, s>>>(w.r32.p, nullptr, P.T, R);
  k_tl_csolve<<<wave(k_tl_csolve), kThreads, 0, s>>>(P.T, R);
  k_tl_z<<<wave(k_tl_z), kThreads, 0, s>>>(w.r32.p, P.M32, P.T, P.nunits, R);
  c.launches += 4;
}

void launch_iteration(Ctx &c, const Plan &P) {
  SolverWork &w = c.sw;
  Red R = red_of(c);
  if (!P.mixed) {
    if (P.vb) k_vb_p<<<wave(k_vb_p), kThreads, 0, c.stream>>>(w.r.p, P.V, w.p.p, R);
    else k_cg_p<<<wave(k_cg_p), kThreads, 0, c.stream>>>(w.r.p, P.M, w.p.p, P.nunits, R);
    GPZ_TPR_SWITCH(P.tpr, (k_cg_spmv<T, false><<<wave(k_cg_spmv<T, false>), kThreads, 0, c.stream>>>(
                              c.d_ia.p, c.d_ja.p, c.d_a.p, nullptr, w.p.p, nullptr, w.q.p, c.neq, R)));
    if (P.vb) k_vb_update<<<wave(k_vb_update), kThreads, 0, c.stream>>>(w.x.p, w.r.p, w.p.p, w.q.p, P.V, R);
    else k_cg_update<<<wave(k_cg_update), kThreads, 0, c.stream>>>(w.x.p, w.r.p, w.p.p, w.q.p, P.M, P.nunits, 0, R);
    c.launches += 3;
    return;
  }
  const int padded = P.bsr ? 1 : 0;
  const bool sym = P.bsr && c.spmv32_variant >= 4;  // 4..8: q accumulated with atomics
  if (P.tl) {
    k_tl_p<<<wave(k_tl_p), kThreads, 0, c.stream>>>(P.T.z, w.pm.p, padded, sym ? w.q32.p : nullptr, c.neq, R);
    if (P.bsr) {
      launch_spmv32(c, c.spmv32_variant, c.sell, R, c.stream);
      c.launches--;
    } else {
      GPZ_TPR_SWITCH(P.tpr32, (k_mx_csr<T><<<wave(k_mx_csr<T>), kThreads, 0, c.stream>>>(
                                  c.d_ia.p, c.d_ja.p, c.d_a32.p, w.pm.p, w.q32.p, c.neq, R)));
    }
    k_tl_update<<<wave(k_tl_update), kThreads, 0, c.stream>>>(w.dx32.p, w.r32.p, w.pm.p, w.q32.p, padded,
                                                              sym ? 1 : 0, c.neq, R);
    k_mx_foldx<<<wave(k_mx_foldx), kThreads, 0, c.stream>>>(w.x.p, w.dx32.p, c.neq, 0, R);
    GPZ_TPR_SWITCH(P.tpr, (k_reliable<T><<<wave(k_reliable<T>), kThreads, 0, c.stream>>>(
                              c.d_ia.p, c.d_ja.p, c.d_a.p, w.x.p, w.b.p, w.r.p, c.neq, R)));
    launch_tl_apply(c, P, R, c.stream);
    c.launches += 5;
    return;
  }
  float *qz = (sym || P.mf1) ? w.q32.p : nullptr;  // q accumulated with atomics: zeroed with p
  if (P.vb)
    k_vb32_p<<<wave(k_vb32_p), kThreads, 0, c.stream>>>(w.r32.p, P.V, w.pm.p, padded, qz, R);
  else
    k_mx_p<<<wave(k_mx_p), kThreads, 0, c.stream>>>(w.r32.p, P.M32, w.pm.p, padded, qz, P.nunits, R);
  if (P.bsr) {
    launch_spmv32(c, c.spmv32_variant, c.sell, R, c.stream);
    c.launches--;
  } else if (P.mf1) {
    matfree1_spmv(c, c.stream, w.pm.p, w.q32.p);
    c.launches--;
  } else {
    GPZ_TPR_SWITCH(P.tpr32, (k_mx_csr<T><<<wave(k_mx_csr<T>), kThreads, 0, c.stream>>>(c.d_ia.p, c.d_ja.p, c.d_a32.p,
                                                                                      w.pm.p, w.q32.p, c.neq, R)));
  }
  if (P.vb)
    k_vb32_update<<<wave(k_vb32_update), kThreads, 0, c.stream>>>(w.dx32.p, w.r32.p, w.pm.p, w.q32.p, P.V, padded,
                                                                  sym ? 1 : 0, R);
  else
    k_mx_update<<<wave(k_mx_update), kThreads, 0, c.stream>>>(w.dx32.p, w.r32.p, w.pm.p, w.q32.p, P.M32, padded,
                                                              sym ? 1 : 0, P.nunits, R);
  k_mx_foldx<<<wave(k_mx_foldx), kThreads, 0, c.stream>>>(w.x.p, w.dx32.p, c.neq, 0, R);
  GPZ_TPR_SWITCH(P.tpr, (k_reliable<T><<<wave(k_reliable<T>), kThreads, 0, c.stream>>>(c.d_ia.p, c.d_ja.p, c.d_a.p,
                                                                                        w.x.p, w.b.p, w.r.p, c.neq, R)));
  if (P.vb) k_vb32_r32<<<wave(k_vb32_r32), kThreads, 0, c.stream>>>(w.r.p, w.r32.p, P.V, R);
  else k_mx_r32<<<wave(k_mx_r32), kThreads, 0, c.stream>>>(w.r.p, w.r32.p, P.M32, P.nunits, R);
  c.launches += 6;
}


// Restarted GMRES(m) with Jacobi / block-Jacobi (TPZMatrix::SolveGMRES ->
// GMRES, Matrix/pzmatrix.cpp:767-800, Solvers/LinearSolvers/gmres.h:68-168).
// The reported iteration count and residual are the reference's: fNumIterations
// is the Arnoldi step count j as the template returns it, and fTol the
// preconditioned residual estimate ||M r|| / ||M b||.  One difference, on the
// not-converged path only: when max_iter ends a cycle early the update uses
// the columns that were built (the template's Update(x, m-1, ...) would also
// read columns left over from the previous cycle).
int solve_gmres(Ctx &c, const gpz_solver_opts &o, gpz_solve_report &rep) {
  GPZ_REQUIRE(o.precond == GPZ_PRECOND_JACOBI || o.precond == GPZ_PRECOND_BLOCK_JACOBI || o.precond == 0,
              GPZ_E_INVALID, "preconditioner not available");
  const int m = o.gmres_krylov > 0 ? o.gmres_krylov : 30;
  GPZ_REQUIRE(m <= 512, GPZ_E_INVALID, "gmres_krylov must be in 1..512");
  const bool block = o.precond == GPZ_PRECOND_BLOCK_JACOBI;
  if (block && !c.have_bjinv) build_block_jacobi(c);
  alloc_work(c, false);
  SolverWork &w = c.sw;
  cudaStream_t s = c.stream;
  const int64_t n = c.neq;
  const size_t nh = (size_t)(m + 1) * (m + 1), nv = (size_t)m + 2;
  w.gm_v.alloc((size_t)(m + 1) * (size_t)std::max<int64_t>(n, 1));
  w.gm_d.alloc(nh + 5 * nv + GMD_NS);
  w.gm_i.alloc(GM_NI);
  Gm G;
  G.V = w.gm_v.p;
  G.H = w.gm_d.p;
  G.s = G.H + nh;
  G.cs = G.s + nv;
  G.sn = G.cs + nv;
  G.vscale = G.sn + nv;
  G.y = G.vscale + nv;
  G.d = G.y + nv;
  G.is = w.gm_i.p;
  G.m = m;
  G.n = n;
  const Prec M{c.d_dinv.p, block ? c.d_bjinv.p : nullptr, block ? 1 : 0};
  const int64_t nunits = block ? n / 3 : n;
  const int tpr = pick_tpr(c.nnz, c.neq);
  Red R = red_of(c);

  cudaEvent_t ev0, ev1;
  GPZ_CUDA_TRY(cudaEventCreate(&ev0));
  GPZ_CUDA_TRY(cudaEventCreate(&ev1));
  GPZ_CUDA_TRY(cudaEventRecord(ev0, s));
  w.gm_d.zero(s);
  double hd[GMD_NS] = {0};
  hd[GMD_TOL] = o.tol;
  int64_t hi[GM_NI] = {0};
  hi[GM_J] = 1;
  hi[GM_MAXIT] = o.max_iter;
  hi[GM_ITERS] = o.max_iter;
  GPZ_CUDA_TRY(cudaMemcpyAsync(G.d, hd, sizeof(hd), cudaMemcpyHostToDevice, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(G.is, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
  double hs[S_NSCAL] = {0};
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.scal.p, hs, sizeof(hs), cudaMemcpyHostToDevice, s));

  k_gm_init<<<wave(k_gm_init), kThreads, 0, s>>>(w.b.p, w.x.p, M, nunits, o.from_current, G, w.scal.p + S_NORMB, R);
  GPZ_TPR_SWITCH(tpr, (k_gm_resid_spmv<T><<<wave(k_gm_resid_spmv<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p,
                                                                                         w.x.p, w.b.p, 1, G)));
  k_gm_resid_prec<<<wave(k_gm_resid_prec), kThreads, 0, s>>>(M, nunits, 1, G, R);
  c.launches += 3;
  GPZ_CUDA_TRY(cudaGetLastError());
  GPZ_CUDA_TRY(cudaMemcpyAsync(hi, G.is, sizeof(hi), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  if (hi[GM_STATE] == GMS_CONV) {
    k_gm_add_r<<<wave(k_gm_add_r), kThreads, 0, s>>>(w.x.p, G);
    c.launches++;
  }

  auto launch_cycle = [&]() {
    for (int i = 0; i < m; i++) {
      GPZ_TPR_SWITCH(tpr, (k_gm_spmv<T><<<wave(k_gm_spmv<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, i, G)));
      k_gm_prec_dot<<<wave(k_gm_prec_dot), kThreads, 0, s>>>(M, nunits, i, G, R);
      for (int k = 0; k <= i; k++) k_gm_mgs<<<wave(k_gm_mgs), kThreads, 0, s>>>(i, k, G, R);
    }
    k_gm_solve_y<<<1, 32, 0, s>>>(G);
    k_gm_update_x<<<wave(k_gm_update_x), kThreads, 0, s>>>(w.x.p, G);
    GPZ_TPR_SWITCH(tpr, (k_gm_resid_spmv<T><<<wave(k_gm_resid_spmv<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p,
                                                                                           c.d_a.p, w.x.p, w.b.p, 0,
                                                                                           G)));
    k_gm_resid_prec<<<wave(k_gm_resid_prec), kThreads, 0, s>>>(M, nunits, 0, G, R);
  };
  const int64_t per_cycle = (int64_t)m * (m + 1) / 2 + 2 * (int64_t)m + 4;
  const bool use_graph = o.use_graph && m <= 64;
  cudaGraphExec_t exec = nullptr;
  if (hi[GM_STATE] == GMS_RUN && use_graph) {
    cudaGraph_t g;
    GPZ_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    launch_cycle();
    GPZ_CUDA_TRY(cudaStreamEndCapture(s, &g));
    GPZ_CUDA_TRY(cudaGraphInstantiate(&exec, g, 0));
    GPZ_CUDA_TRY(cudaGraphDestroy(g));
  }
  // the device ends the solve by itself after max_iter Arnoldi steps; the
  // host bound only guards against a state machine that never finishes
  const int64_t max_cycles = o.max_iter / m + 3;
  int64_t cycles = 0;
  bool cancelled = false;
  while (hi[GM_STATE] == GMS_RUN && cycles < max_cycles) {
    if (c.killed.load()) {
      cancelled = true;
      break;
    }
    if (exec) GPZ_CUDA_TRY(cudaGraphLaunch(exec, s));
    else launch_cycle();
    c.launches += per_cycle;
    cycles++;
    GPZ_CUDA_TRY(cudaGetLastError());
    GPZ_CUDA_TRY(cudaMemcpyAsync(hi, G.is, sizeof(hi), cudaMemcpyDeviceToHost, s));
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  }
  if (exec) cudaGraphExecDestroy(exec);
  GPZ_TPR_SWITCH(tpr, (k_true_resid<T><<<wave(k_true_resid<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, w.x.p,
                                                                                   w.b.p, c.neq, R)));
  c.launches++;
  GPZ_CUDA_TRY(cudaEventRecord(ev1, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(hs, w.scal.p, sizeof(hs), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(hd, G.d, sizeof(hd), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(hi, G.is, sizeof(hi), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  check_device_flag(c, "GMRES");
  GPZ_REQUIRE(cancelled ||
                  (hi[GM_STATE] != GMS_RUN && hi[GM_STATE] != GMS_CONV_PENDING && hi[GM_STATE] != GMS_MAXIT_PENDING),
              GPZ_E_DEVICE_CHECK, "GMRES state machine did not finish");
  rep.iterations = cancelled ? hi[GM_J] - 1 : hi[GM_ITERS];  // GM_J counts from 1 (gmres.h's j)
  rep.resid = hd[GMD_RESID];
  rep.true_resid = std::sqrt(hs[S_TRUERR]) / hs[S_NORMB];
  rep.seconds = ms * 1e-3;
  rep.spmv_fp64 = hi[GM_SP64] + 1;
  rep.spmv_fp32 = 0;
  rep.reliable_updates = 0;
  rep.restarts = cycles;
  c.have_solution = true;
  if (hi[GM_STATE] == GMS_BREAK) return GPZ_E_BREAKDOWN;
  if (cancelled) return GPZ_CANCELLED;
  return hi[GM_STATE] == GMS_CONV ? GPZ_OK : GPZ_NOT_CONVERGED;
}

// Flexible CG with the learned preconditioner (GPZ_SOLVER_LEARNED_FCG).  The
// stopping rule is the reference's (recursive ||r||/||b|| <= tol, cg.h:100);
// afterwards the true FP64 residual is recomputed and, if it misses the
// tolerance, the solve restarts from the current x (at most three times).
// mixed: q = A32 p32 with FP32 values (scalar problems: the FP32 CSR copy),
// FP64 x, r, z, dots and scalars; when ||r|| has dropped by reliable_delta (or
// meets the tolerance) r is replaced by b - A64 x in FP64, and the solve stops
// only on that true residual.
int solve_learned(Ctx &c, const gpz_solver_opts &o, gpz_solve_report &rep, bool mixed) {
  GPZ_REQUIRE(!c.flt.active, GPZ_E_INVALID, "learned preconditioner: not available under an equation filter");
  if (mixed && (!c.have_a32 || (o.spmv_variant >= 0 && (c.have_bsr3 || c.nstate == 1) &&
                                o.spmv_variant != c.spmv32_variant)))
    make_fp32_copy(c, o.spmv_variant);
  learned_prepare(c);
  // scalar problems: FP32 CSR (k_lfcg_spmv); 3 states: the mixed CG's FP32
  // operator in the layout the autotuner chose (3x3 blocks or matrix-free)
  const bool blk = mixed && c.have_bsr3;
  const int v32 = c.spmv32_variant;
  const int qpad = blk && v32 >= 4 ? 1 : 0;  // padded, accumulated with atomics
  alloc_work(c, mixed);
  SolverWork &w = c.sw;
  w.z.alloc(std::max<int64_t>(c.neq, 1));
  w.r32.alloc(std::max<int64_t>(c.neq, 1));
  if (!blk) w.pm.alloc(std::max<int64_t>(c.neq, 1));
  const int tpr32 = pick_tpr32(c.nnz, c.neq);
  float *p32 = mixed ? w.pm.p : nullptr;
  cudaStream_t s = c.stream;
  if (blk) {
    w.z32.alloc(std::max<int64_t>(c.neq, 1));
    w.pm.zero(s);
    w.q32.zero(s);
    w.dx32.zero(s);
  }
  const int tpr = pick_tpr(c.nnz, c.neq);
  const LnView L = learned_view(c);
  Red R = red_of(c);
  const int batch = o.check_every > 0 ? o.check_every : 32;
  cudaEvent_t ev0, ev1;
  GPZ_CUDA_TRY(cudaEventCreate(&ev0));
  GPZ_CUDA_TRY(cudaEventCreate(&ev1));
  GPZ_CUDA_TRY(cudaEventRecord(ev0, s));
  int64_t per_iter = mixed ? 6 : 5;  // the FP32 operator counts its own launches (measured at capture)
  // connects of 0 or 3 equations and rank 8: the connect-wise z kernel
  bool by_connect = blk && c.ln.R == 8;
  for (int64_t cn = 0; cn < c.nconnects && by_connect; cn++)
    by_connect = c.h_block_size[cn] == 0 || c.h_block_size[cn] == 3;
  // base preconditioner under the learned correction: point Jacobi (precond 0 / JACOBI), the 3x3 connect
  // blocks (BLOCK_JACOBI) or the two-level block Jacobi (TWO_LEVEL); the blocks need the connect-wise kernel
  GPZ_REQUIRE(o.precond == 0 || o.precond == GPZ_PRECOND_JACOBI || o.precond == GPZ_PRECOND_BLOCK_JACOBI ||
                  o.precond == GPZ_PRECOND_TWO_LEVEL,
              GPZ_E_INVALID, "learned flexible CG: base preconditioner not available");
  const bool lblock = o.precond == GPZ_PRECOND_BLOCK_JACOBI || o.precond == GPZ_PRECOND_TWO_LEVEL;
  const bool ltl = o.precond == GPZ_PRECOND_TWO_LEVEL;
  GPZ_REQUIRE(!lblock || by_connect, GPZ_E_INVALID,
              "learned flexible CG with a block base: needs the FP32 3x3-block operator (3 equations per connect) "
              "and rank 8");
  if (ltl && !c.tl.ready)
    GPZ_REQUIRE(two_level_build(c) == GPZ_OK, GPZ_E_INVALID,
                "two-level base: needs one uniform grid of axis-aligned Q2 hex elasticity elements");
  if (ltl && !c.tl.have_inv) two_level_assemble(c);
  if (lblock) {
    if (!c.have_bjinv) build_block_jacobi(c);
    c.d_bjinv32.alloc((size_t)(c.neq / 3) * 9);
    k_to_f32<<<wave(k_to_f32), kThreads, 0, s>>>(c.d_bjinv.p, c.d_bjinv32.p, (int64_t)(c.neq / 3) * 9);
    c.launches++;
  }
  TlView TV{};
  float *zb = nullptr;
  if (ltl) {
    TwoLevel &T = c.tl;
    TV = tl_view(T);
    T.rc.zero(s);
    zb = T.z32.p;
  }
  auto apply_z32 = [&]() {
    if (ltl) {  // the coarse correction of the current residual first
      k_tl_restrict<<<TV.mx * TV.my * TV.mz, kThreads, 0, s>>>(w.r32.p, w.r.p, TV, R);
      k_tl_csolve<<<wave(k_tl_csolve), kThreads, 0, s>>>(TV, R);
      c.launches += 2;
    }
    if (by_connect)
      k_lfb_z3<<<wave(k_lfb_z3), kThreads, 0, s>>>(L, c.ln.ce_ptr.p, c.ln.ce_idx.p, c.d_block_pos.p,
                                                   c.d_block_size.p, c.nconnects, w.r.p, w.r32.p, w.q32.p, qpad,
                                                   w.z32.p, lblock ? c.d_bjinv32.p : nullptr, TV, zb, R);
    else
      k_lfb_z<<<wave(k_lfb_z), kThreads, 0, s>>>(L, w.r.p, w.r32.p, w.q32.p, qpad, w.z32.p, R);
    c.launches++;
  };
  auto iteration = [&]() {
    if (blk) {
      launch_spmv32(c, v32, c.sell, R, s);
      k_lfb_update<<<wave(k_lfb_update), kThreads, 0, s>>>(w.dx32.p, w.r32.p, w.pm.p, w.q32.p, qpad, c.neq, R);
      k_mx_foldx<<<wave(k_mx_foldx), kThreads, 0, s>>>(w.x.p, w.dx32.p, c.neq, 0, R);
      GPZ_TPR_SWITCH(tpr, (k_reliable<T><<<wave(k_reliable<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p,
                                                                                    w.x.p, w.b.p, w.r.p, c.neq, R)));
      k_fcg_t<<<wave(k_fcg_t), kThreads, 0, s>>>(L, w.r.p, w.r32.p, R);
      apply_z32();
      k_lfb_p<<<wave(k_lfb_p), kThreads, 0, s>>>(w.z32.p, w.r32.p, L.dinv32, zb, w.pm.p, w.q32.p, qpad, qpad,
                                                 c.neq, R);
      c.launches += 5;
      return;
    }
    if (mixed) {
      GPZ_TPR_SWITCH(tpr32, (k_lfcg_spmv<T><<<wave(k_lfcg_spmv<T>), kThreads, 0, s>>>(
                                c.d_ia.p, c.d_ja.p, c.d_a32.p, p32, w.p.p, w.q.p, c.neq, R)));
      c.launches++;
    } else {
      GPZ_TPR_SWITCH(tpr, (k_cg_spmv<T, false><<<wave(k_cg_spmv<T, false>), kThreads, 0, s>>>(
                              c.d_ia.p, c.d_ja.p, c.d_a.p, nullptr, w.p.p, nullptr, w.q.p, c.neq, R)));
      c.launches++;
    }
    k_fcg_update<<<wave(k_fcg_update), kThreads, 0, s>>>(w.x.p, w.r.p, w.r32.p, w.p.p, w.q.p, c.neq, mixed ? 1 : 0,
                                                         R);
    if (mixed)
      GPZ_TPR_SWITCH(tpr, (k_reliable<T><<<wave(k_reliable<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p,
                                                                                    w.x.p, w.b.p, w.r.p, c.neq, R)));
    k_fcg_t<<<wave(k_fcg_t), kThreads, 0, s>>>(L, w.r.p, w.r32.p, R);
    k_fcg_z<<<wave(k_fcg_z), kThreads, 0, s>>>(L, w.r.p, w.q.p, c.d_dinv.p, w.z.p, R);
    k_fcg_p<<<wave(k_fcg_p), kThreads, 0, s>>>(w.z.p, w.r.p, c.d_dinv.p, w.p.p, p32, c.neq, R);
    c.launches += mixed ? 5 : 4;
  };
  cudaGraphExec_t exec = nullptr;
  int64_t total_it = 0, nfallback = 0, nupd = 0, nspmv64 = 0, hstate[I_NISCAL] = {0};
  double hs[S_NSCAL] = {0};
  int rc = GPZ_NOT_CONVERGED;
  for (int pass = 0; pass < 4; pass++) {
    for (int k = 0; k < S_NSCAL; k++) hs[k] = 0.0;
    hs[S_TOL] = o.tol;
    hs[S_DELTA2] = (o.reliable_delta > 0 ? o.reliable_delta : 1e-2);
    hs[S_DELTA2] *= hs[S_DELTA2];
    int64_t hi[I_NISCAL] = {0};
    hi[I_MAXIT] = o.max_iter - total_it;
    GPZ_CUDA_TRY(cudaMemcpyAsync(w.scal.p, hs, sizeof(hs), cudaMemcpyHostToDevice, s));
    GPZ_CUDA_TRY(cudaMemcpyAsync(w.iscal.p, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
    const int from_current = pass > 0 ? 1 : o.from_current;
    GPZ_TPR_SWITCH(tpr, (k_cg_init<T><<<wave(k_cg_init<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, w.x.p,
                                                                               w.b.p, w.r.p, c.neq, from_current, R)));
    k_fcg_t<<<wave(k_fcg_t), kThreads, 0, s>>>(L, w.r.p, w.r32.p, R);  // k_cg_init leaves I_UPDATE = 2: FP64 r
    if (blk) {
      apply_z32();
      k_lfb_p<<<wave(k_lfb_p), kThreads, 0, s>>>(w.z32.p, w.r32.p, L.dinv32, zb, w.pm.p, w.q32.p, qpad, qpad,
                                                 c.neq, R);
      c.launches -= 1;
    } else {
      k_fcg_z<<<wave(k_fcg_z), kThreads, 0, s>>>(L, w.r.p, w.q.p, c.d_dinv.p, w.z.p, R);
      k_fcg_p<<<wave(k_fcg_p), kThreads, 0, s>>>(w.z.p, w.r.p, c.d_dinv.p, w.p.p, p32, c.neq, R);
    }
    c.launches += 4;
    GPZ_CUDA_TRY(cudaGetLastError());
    if (o.use_graph && !exec) {
      cudaGraph_t g;
      GPZ_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      const int64_t l0 = c.launches;
      for (int i = 0; i < batch; i++) iteration();
      GPZ_CUDA_TRY(cudaStreamEndCapture(s, &g));
      per_iter = (c.launches - l0) / batch;
      c.launches = l0;
      GPZ_CUDA_TRY(cudaGraphInstantiate(&exec, g, 0));
      GPZ_CUDA_TRY(cudaGraphDestroy(g));
    }
    bool cancelled = false;
    for (;;) {
      GPZ_CUDA_TRY(cudaMemcpyAsync(hstate, w.iscal.p, sizeof(hstate), cudaMemcpyDeviceToHost, s));
      GPZ_CUDA_TRY(cudaStreamSynchronize(s));
      if (hstate[I_CONV] != 0 || hstate[I_IT] >= hi[I_MAXIT]) break;
      if (c.killed.load()) {
        cancelled = true;
        break;
      }
      if (exec) {
        GPZ_CUDA_TRY(cudaGraphLaunch(exec, s));
        c.launches += (int64_t)batch * per_iter;
      } else {
        for (int i = 0; i < batch; i++) iteration();
      }
      GPZ_CUDA_TRY(cudaGetLastError());
    }
    if (blk) {
      k_mx_foldx<<<wave(k_mx_foldx), kThreads, 0, s>>>(w.x.p, w.dx32.p, c.neq, 1, R);
      c.launches++;
    }
    GPZ_TPR_SWITCH(tpr, (k_true_resid<T><<<wave(k_true_resid<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p,
                                                                                     w.x.p, w.b.p, c.neq, R)));
    c.launches++;
    GPZ_CUDA_TRY(cudaMemcpyAsync(hs, w.scal.p, sizeof(hs), cudaMemcpyDeviceToHost, s));
    GPZ_CUDA_TRY(cudaMemcpyAsync(hstate, w.iscal.p, sizeof(hstate), cudaMemcpyDeviceToHost, s));
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));
    total_it += hstate[I_IT];
    nfallback += hstate[I_NRESTART];
    nupd += hstate[I_NUPD];
    nspmv64 += hstate[I_SP64];
    if (hstate[I_BREAK]) {
      rc = GPZ_E_BREAKDOWN;
      break;
    }
    if (cancelled) {
      rc = GPZ_CANCELLED;
      break;
    }
    const double true_resid = std::sqrt(hs[S_TRUERR]) / hs[S_NORMB];
    if (hstate[I_CONV] == 1 && true_resid <= o.tol) {
      rc = GPZ_OK;
      break;
    }
    if (hstate[I_CONV] != 1 || total_it >= o.max_iter) break;  // budget spent
  }
  if (exec) cudaGraphExecDestroy(exec);
  GPZ_CUDA_TRY(cudaEventRecord(ev1, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  check_device_flag(c, "learned flexible CG");
  rep.iterations = total_it;
  rep.resid = hs[S_RESID];
  rep.true_resid = std::sqrt(hs[S_TRUERR]) / hs[S_NORMB];
  rep.seconds = ms * 1e-3;
  rep.spmv_fp64 = mixed ? nspmv64 + 1 : total_it + 1;
  rep.spmv_fp32 = mixed ? total_it : 0;
  rep.reliable_updates = nupd;
  rep.restarts = nfallback;  // iterations that fell back to Jacobi
  c.have_solution = true;
  return rc;
}

// Training pairs from the Jacobi-PCG iterates of the assembled system
// (cg.h:29-132): a first solve to `tol` gives x* and the iteration count K;
// a second, identical (deterministic) run snapshots r_k and x_k at up to
// `npairs` iterations spaced geometrically over 1..K.  Returns the number of pairs taken.
int collect_cg_pairs(Ctx &c, int npairs, double tol, int64_t max_iter, double *R_out, double *X_out, double *xstar,
                     int64_t *iters) {
  alloc_work(c, false);
  SolverWork &w = c.sw;
  cudaStream_t s = c.stream;
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.b.p, c.d_f.p, c.neq * sizeof(double), cudaMemcpyDeviceToDevice, s));
  gpz_solver_opts o{};
  o.solver = GPZ_SOLVER_CG;
  o.precond = GPZ_PRECOND_JACOBI;
  o.max_iter = max_iter;
  o.tol = tol;
  o.check_every = 32;
  o.use_graph = 1;
  gpz_solve_report rep{};
  solve(c, o, rep);
  const int64_t K = rep.iterations;
  *iters = K;
  GPZ_CUDA_TRY(cudaMemcpyAsync(xstar, w.x.p, c.neq * sizeof(double), cudaMemcpyDeviceToDevice, s));
  if (K < 1) return 0;
  // geometric spacing over 1..K: the early, rough errors (which a local
  // correction can remove) are as well represented as the late, smooth ones
  std::vector<int64_t> snap;
  for (int j = 0; j < npairs; j++) {
    int64_t k = (int64_t)std::llround(std::pow((double)K, (double)(j + 1) / (double)(npairs + 1)));
    k = std::max<int64_t>(1, std::min<int64_t>(K - 1, k));  // x_K = x*: no error left to learn from
    if (k >= 1 && (snap.empty() || k > snap.back())) snap.push_back(k);
  }
  Plan P;
  P.mixed = false;
  P.block = false;
  P.bsr = false;
  P.tpr = pick_tpr(c.nnz, c.neq);
  P.tpr32 = 0;
  P.nunits = c.neq;
  P.M = Prec{c.d_dinv.p, nullptr, 0};
  double hs[S_NSCAL] = {0};
  hs[S_TOL] = 0.0;  // run exactly K iterations
  int64_t hi[I_NISCAL] = {0};
  hi[I_MAXIT] = K;
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.scal.p, hs, sizeof(hs), cudaMemcpyHostToDevice, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.iscal.p, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
  Red Rd = red_of(c);
  GPZ_TPR_SWITCH(P.tpr, (k_cg_init<T><<<wave(k_cg_init<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, w.x.p,
                                                                               w.b.p, w.r.p, c.neq, 0, Rd)));
  k_precond_dot<<<wave(k_precond_dot), kThreads, 0, s>>>(w.r.p, P.M, P.nunits, Rd);
  c.launches += 2;
  size_t j = 0;
  for (int64_t it = 1; it <= K && j < snap.size(); it++) {
    launch_iteration(c, P);
    if (it == snap[j]) {
      GPZ_CUDA_TRY(cudaMemcpyAsync(R_out + j * c.neq, w.r.p, c.neq * sizeof(double), cudaMemcpyDeviceToDevice, s));
      GPZ_CUDA_TRY(cudaMemcpyAsync(X_out + j * c.neq, w.x.p, c.neq * sizeof(double), cudaMemcpyDeviceToDevice, s));
      j++;
    }
  }
  GPZ_CUDA_TRY(cudaGetLastError());
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  check_device_flag(c, "training pairs");
  return (int)j;
}

// Stationary Jacobi iteration (kernels k_jac_*): two launches per sweep, a
// batch of sweeps captured once as a CUDA graph, convergence read back per
// batch.  rep.iterations is the number of sweeps performed.
int solve_jacobi(Ctx &c, const gpz_solver_opts &o, gpz_solve_report &rep) {
  GPZ_REQUIRE(o.precond == GPZ_PRECOND_JACOBI || o.precond == 0, GPZ_E_INVALID,
              "the Jacobi iteration takes no preconditioner");
  alloc_work(c, false);
  SolverWork &w = c.sw;
  cudaStream_t s = c.stream;
  const int tpr = pick_tpr(c.nnz, c.neq);
  const int full = c.user_sym ? 0 : 1;
  const int64_t maxit = full ? std::max<int64_t>(o.max_iter, 1) : o.max_iter;
  const int batch = o.check_every > 0 ? o.check_every : 32;
  cudaEvent_t ev0, ev1;
  GPZ_CUDA_TRY(cudaEventCreate(&ev0));
  GPZ_CUDA_TRY(cudaEventCreate(&ev1));
  GPZ_CUDA_TRY(cudaEventRecord(ev0, s));
  double hs[S_NSCAL] = {0};
  hs[S_TOL] = o.tol;
  int64_t hi[I_NISCAL] = {0};
  hi[I_MAXIT] = maxit;
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.scal.p, hs, sizeof(hs), cudaMemcpyHostToDevice, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.iscal.p, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
  Red R = red_of(c);
  GPZ_TPR_SWITCH(tpr, (k_cg_init<T><<<wave(k_cg_init<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, w.x.p,
                                                                             w.b.p, w.r.p, c.neq, o.from_current, R)));
  k_jac_start<<<1, 1, 0, s>>>(R, full);
  c.launches += 2;
  GPZ_CUDA_TRY(cudaGetLastError());
  auto sweeps = [&](int k) {
    for (int i = 0; i < k; i++) {
      k_jac_x<<<wave(k_jac_x), kThreads, 0, s>>>(c.d_a.p, c.d_diagpos.p, w.r.p, w.x.p, c.neq, w.iscal.p);
      GPZ_TPR_SWITCH(tpr, (k_jac_resid<T><<<wave(k_jac_resid<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p,
                                                                                     w.x.p, w.b.p, w.r.p, c.neq, R)));
      c.launches += 2;
    }
  };
  cudaGraphExec_t exec = nullptr;
  if (o.use_graph) {
    cudaGraph_t g;
    GPZ_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int64_t l0 = c.launches;
    sweeps(batch);
    GPZ_CUDA_TRY(cudaStreamEndCapture(s, &g));
    c.launches = l0;
    GPZ_CUDA_TRY(cudaGraphInstantiate(&exec, g, 0));
    GPZ_CUDA_TRY(cudaGraphDestroy(g));
  }
  int64_t hstate[I_NISCAL];
  bool cancelled = false;
  for (;;) {
    GPZ_CUDA_TRY(cudaMemcpyAsync(hstate, w.iscal.p, sizeof(hstate), cudaMemcpyDeviceToHost, s));
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));
    if (hstate[I_CONV] != 0 || hstate[I_IT] >= maxit) break;
    if (c.killed.load()) {
      cancelled = true;
      break;
    }
    if (exec) {
      GPZ_CUDA_TRY(cudaGraphLaunch(exec, s));
      c.launches += 2 * (int64_t)batch;
    } else {
      sweeps(batch);
    }
    GPZ_CUDA_TRY(cudaGetLastError());
  }
  if (exec) cudaGraphExecDestroy(exec);
  GPZ_TPR_SWITCH(tpr, (k_true_resid<T><<<wave(k_true_resid<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, w.x.p,
                                                                                   w.b.p, c.neq, R)));
  c.launches++;
  GPZ_CUDA_TRY(cudaEventRecord(ev1, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(hs, w.scal.p, sizeof(hs), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(hstate, w.iscal.p, sizeof(hstate), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  check_device_flag(c, "Jacobi iteration");
  rep.iterations = hstate[I_IT];
  rep.resid = hs[S_RESID];
  rep.true_resid = std::sqrt(hs[S_TRUERR]) / hs[S_NORMB];
  rep.seconds = ms * 1e-3;
  rep.spmv_fp64 = hstate[I_SP64] + (o.from_current ? 1 : 0) + 1;  // + the final true residual
  rep.spmv_fp32 = 0;
  rep.reliable_updates = 0;
  rep.restarts = 0;
  c.have_solution = true;
  if (cancelled) return GPZ_CANCELLED;
  return hstate[I_CONV] == 1 ? GPZ_OK : GPZ_NOT_CONVERGED;
}

int solve(Ctx &c, const gpz_solver_opts &o, gpz_solve_report &rep) {
  if (o.solver == GPZ_SOLVER_JACOBI) return solve_jacobi(c, o, rep);
  if (o.solver == GPZ_SOLVER_GMRES) return solve_gmres(c, o, rep);
  if (o.solver == GPZ_SOLVER_LEARNED_FCG || o.solver == GPZ_SOLVER_LEARNED_MIXED_FCG)
    return solve_learned(c, o, rep, o.solver == GPZ_SOLVER_LEARNED_MIXED_FCG);
  const bool mixed = o.solver == GPZ_SOLVER_MIXED_CG;
  GPZ_REQUIRE(o.solver == GPZ_SOLVER_CG || mixed, GPZ_E_INVALID, "solver kind not available");
  GPZ_REQUIRE(o.precond == GPZ_PRECOND_JACOBI || o.precond == GPZ_PRECOND_BLOCK_JACOBI ||
                  o.precond == GPZ_PRECOND_NODESET_JACOBI || o.precond == GPZ_PRECOND_TWO_LEVEL || o.precond == 0,
              GPZ_E_INVALID, "preconditioner not available");
  const bool tl = o.precond == GPZ_PRECOND_TWO_LEVEL;
  GPZ_REQUIRE(!tl || mixed, GPZ_E_INVALID, "the two-level preconditioner is built for the mixed CG");
  if (tl && !c.tl.ready)
    GPZ_REQUIRE(two_level_build(c) == GPZ_OK, GPZ_E_INVALID,
                "two-level preconditioner: needs one uniform grid of axis-aligned Q2 hex elasticity elements "
                "(3 equations per connect, no equation filter) and at most 3000 coarse equations");
  // whole connect blocks of other sizes than 3, and the node-set blocks: variable-size block Jacobi
  const bool vb = o.precond == GPZ_PRECOND_NODESET_JACOBI ||
                  (o.precond == GPZ_PRECOND_BLOCK_JACOBI && !connect_blocks_are_3(c));
  const bool block = (o.precond == GPZ_PRECOND_BLOCK_JACOBI && !vb) || tl;
  if (mixed && (!c.have_a32 || (o.spmv_variant >= 0 && (c.have_bsr3 || c.nstate == 1) &&
                                o.spmv_variant != c.spmv32_variant)))
    make_fp32_copy(c, o.spmv_variant);
  if (block && !c.have_bjinv) build_block_jacobi(c);
  if (vb && (!c.have_vbinv || c.vb_kind != o.precond)) build_vblocks(c, o.precond);
  if (tl && !c.tl.have_inv) two_level_assemble(c);
  alloc_work(c, mixed);
  SolverWork &w = c.sw;
  cudaStream_t s = c.stream;
  Plan P;
  P.mixed = mixed;
  P.block = block;
  P.bsr = mixed && c.have_bsr3;
  P.mf1 = mixed && !c.have_bsr3 && c.spmv32_variant == 9 && c.mf1.ready;
  P.tpr = pick_tpr(c.nnz, c.neq);
  P.tpr32 = pick_tpr32(c.nnz, c.neq);
  P.nunits = block ? c.neq / 3 : c.neq;
  P.M = Prec{c.d_dinv.p, block ? c.d_bjinv.p : nullptr, block ? 1 : 0};
  P.vb = vb;
  if (mixed) {
    // FP32 copies of the preconditioner
    if (vb) {
      if (!c.d_vb_inv32.p || c.d_vb_inv32.n != c.d_vb_inv.n) c.d_vb_inv32.alloc(c.d_vb_inv.n);
      k_vb_inv32t<<<wave(k_vb_inv32t), kThreads, 0, s>>>(vblk_of(c), c.d_vb_inv32.p);
    } else if (block) {
      c.d_bjinv32.alloc((size_t)P.nunits * 9);
      k_to_f32<<<wave(k_to_f32), kThreads, 0, s>>>(c.d_bjinv.p, c.d_bjinv32.p, (int64_t)P.nunits * 9);
    } else {
      c.d_dinv32.alloc(std::max<int64_t>(c.neq, 1));
      k_to_f32<<<wave(k_to_f32), kThreads, 0, s>>>(c.d_dinv.p, c.d_dinv32.p, c.neq);
    }
    c.launches++;
    P.M32 = Prec32{block ? nullptr : c.d_dinv32.p, block ? c.d_bjinv32.p : nullptr, block ? 1 : 0};
    w.dx32.zero(s);
    w.pm.zero(s);
  }
  P.V = vblk_of(c);
  P.tl = tl;
  if (tl) {
    TwoLevel &T = c.tl;
    P.T = tl_view(T);
    T.rc.zero(s);
  }
  const int batch = o.check_every > 0 ? o.check_every : 32;

  cudaEvent_t ev0, ev1;
  GPZ_CUDA_TRY(cudaEventCreate(&ev0));
  GPZ_CUDA_TRY(cudaEventCreate(&ev1));
  GPZ_CUDA_TRY(cudaEventRecord(ev0, s));

  double hs[S_NSCAL] = {0};
  hs[S_TOL] = o.tol;
  hs[S_DELTA2] = (o.reliable_delta > 0 ? o.reliable_delta : 1e-2);
  hs[S_DELTA2] *= hs[S_DELTA2];
  int64_t hi[I_NISCAL] = {0};
  hi[I_MAXIT] = o.max_iter;
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.scal.p, hs, sizeof(hs), cudaMemcpyHostToDevice, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.iscal.p, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
  Red R = red_of(c);
  GPZ_TPR_SWITCH(P.tpr, (k_cg_init<T><<<wave(k_cg_init<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, w.x.p,
                                                                               w.b.p, w.r.p, c.neq, o.from_current,
                                                                               R)));
  if (tl) {
    launch_tl_apply(c, P, R, s);
    c.launches -= 1;  // with k_cg_init: five launches
  } else if (mixed && vb) k_vb32_r32<<<wave(k_vb32_r32), kThreads, 0, s>>>(w.r.p, w.r32.p, P.V, R);
  else if (mixed) k_mx_r32<<<wave(k_mx_r32), kThreads, 0, s>>>(w.r.p, w.r32.p, P.M32, P.nunits, R);
  else if (vb) k_vb_dot<<<wave(k_vb_dot), kThreads, 0, s>>>(w.r.p, P.V, R);
  else k_precond_dot<<<wave(k_precond_dot), kThreads, 0, s>>>(w.r.p, P.M, P.nunits, R);
  c.launches += 2;
  GPZ_CUDA_TRY(cudaGetLastError());

  cudaGraphExec_t exec = nullptr;
  const int per_iter = tl ? 9 : (mixed ? 6 : 3);
  if (o.use_graph) {
    cudaGraph_t g;
    GPZ_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int64_t l0 = c.launches;
    for (int i = 0; i < batch; i++) launch_iteration(c, P);
    GPZ_CUDA_TRY(cudaStreamEndCapture(s, &g));
    c.launches = l0;
    GPZ_CUDA_TRY(cudaGraphInstantiate(&exec, g, 0));
    GPZ_CUDA_TRY(cudaGraphDestroy(g));
  }
  int64_t hstate[I_NISCAL];
  bool cancelled = false;
  for (;;) {
    if (c.killed.load()) {
      cancelled = true;
      break;
    }
    if (exec) {
      GPZ_CUDA_TRY(cudaGraphLaunch(exec, s));
      c.launches += (int64_t)batch * per_iter;
    } else {
      for (int i = 0; i < batch; i++) launch_iteration(c, P);
    }
    GPZ_CUDA_TRY(cudaGetLastError());
    GPZ_CUDA_TRY(cudaMemcpyAsync(hstate, w.iscal.p, sizeof(hstate), cudaMemcpyDeviceToHost, s));
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));
    if (hstate[I_CONV] != 0 || hstate[I_IT] >= o.max_iter) break;
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (mixed) {
    k_mx_foldx<<<wave(k_mx_foldx), kThreads, 0, s>>>(w.x.p, w.dx32.p, c.neq, 1, R);
    c.launches++;
  }
  GPZ_TPR_SWITCH(P.tpr, (k_true_resid<T><<<wave(k_true_resid<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p,
                                                                                     w.x.p, w.b.p, c.neq, R)));
  c.launches++;
  GPZ_CUDA_TRY(cudaEventRecord(ev1, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(hs, w.scal.p, sizeof(hs), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(hstate, w.iscal.p, sizeof(hstate), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  check_device_flag(c, "iterative solve");
  rep.iterations = hstate[I_IT];
  rep.resid = hs[S_RESID];
  rep.true_resid = std::sqrt(hs[S_TRUERR]) / hs[S_NORMB];
  rep.seconds = ms * 1e-3;
  rep.spmv_fp64 = hstate[I_SP64] + 1;
  rep.spmv_fp32 = hstate[I_SP32];
  rep.reliable_updates = hstate[I_NUPD];
  rep.restarts = hstate[I_NRESTART];
  c.have_solution = true;
  if (hstate[I_BREAK]) return GPZ_E_BREAKDOWN;
  if (cancelled && hstate[I_CONV] == 0) return GPZ_CANCELLED;
  return hstate[I_CONV] == 1 ? GPZ_OK : GPZ_NOT_CONVERGED;
}

// Base pieces for training the learned correction on a block base (device
// vectors, FP64 out): z = B^-1 r over the 3x3 connect blocks, and the coarse
// part P Ac^-1 P^T r of the two-level preconditioner (FP32 inside).
void base_block_apply(Ctx &c, const double *r, double *z) {
  if (!c.have_bjinv) build_block_jacobi(c);
  const Prec M{c.d_dinv.p, c.d_bjinv.p, 1};
  k_prec_apply<<<wave(k_prec_apply), kThreads, 0, c.stream>>>(r, M, c.neq / 3, z);
  c.launches++;
}

__global__ void __launch_bounds__(kThreads) k_tl_coarse_only(TlView T, int64_t nunits, double *__restrict__ z) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nunits; u += (int64_t)gridDim.x * blockDim.x) {
    float cz[3] = {0.f, 0.f, 0.f};
    const int32_t v = T.brow_vtx[u];
    if (v >= 0) {
      int I, J, K;
      float t[3];
      tl_locate(T, v, I, J, K, t[0], t[1], t[2]);
      for (int c8 = 0; c8 < 8; c8++) {
        const int bx = c8 & 1, by = (c8 >> 1) & 1, bz = c8 >> 2;
        const float w = (bx ? t[0] : 1.f - t[0]) * (by ? t[1] : 1.f - t[1]) * (bz ? t[2] : 1.f - t[2]);
        if (w == 0.f) continue;
        const int64_t nd = (I + bx) + (int64_t)(T.mx + 1) * ((J + by) + (int64_t)(T.my + 1) * (K + bz));
        for (int j = 0; j < 3; j++) cz[j] = fmaf(w, __ldcg(&T.zc[3 * nd + j]), cz[j]);
      }
    }
    for (int j = 0; j < 3; j++) z[3 * u + j] = cz[j];
  }
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < T.nc; k += (int64_t)gridDim.x * blockDim.x)
    T.rc[k] = 0.f;
}

void base_coarse_apply(Ctx &c, const double *r, double *z) {
  GPZ_REQUIRE(c.tl.ready || two_level_build(c) == GPZ_OK, GPZ_E_INVALID,
              "two-level base: needs one uniform grid of axis-aligned Q2 hex elasticity elements");
  if (!c.tl.have_inv) two_level_assemble(c);
  alloc_work(c, true);
  SolverWork &w = c.sw;
  TwoLevel &T = c.tl;
  const TlView TV = tl_view(T);
  int64_t hi[I_NISCAL] = {0};
  hi[I_MAXIT] = 1;
  hi[I_UPDATE] = 2;  // the restriction reads the FP64 residual
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.iscal.p, hi, sizeof(hi), cudaMemcpyHostToDevice, c.stream));
  const Red R = red_of(c);
  k_tl_restrict<<<TV.mx * TV.my * TV.mz, kThreads, 0, c.stream>>>(w.r32.p, r, TV, R);
  k_tl_csolve<<<wave(k_tl_csolve), kThreads, 0, c.stream>>>(TV, R);
  k_tl_coarse_only<<<wave(k_tl_coarse_only), kThreads, 0, c.stream>>>(TV, c.neq / 3, z);
  c.launches += 3;
  GPZ_CUDA_TRY(cudaGetLastError());
}

// z = M r for a CG preconditioner of the assembled system (host FP64 vectors):
// what one application inside GPZ_SOLVER_CG (FP64: Jacobi, block Jacobi,
// node-set blocks) or GPZ_SOLVER_MIXED_CG (FP32: the two-level preconditioner) computes
void precond_apply(Ctx &c, int precond, const double *hr, double *hz) {
  GPZ_REQUIRE(precond == GPZ_PRECOND_JACOBI || precond == GPZ_PRECOND_BLOCK_JACOBI ||
                  precond == GPZ_PRECOND_NODESET_JACOBI || precond == GPZ_PRECOND_TWO_LEVEL,
              GPZ_E_INVALID, "preconditioner kind");
  cudaStream_t s = c.stream;
  const bool tl = precond == GPZ_PRECOND_TWO_LEVEL;
  const bool vb = precond == GPZ_PRECOND_NODESET_JACOBI ||
                  (precond == GPZ_PRECOND_BLOCK_JACOBI && !connect_blocks_are_3(c));
  const bool block = (precond == GPZ_PRECOND_BLOCK_JACOBI && !vb) || tl;
  if (tl) {
    if (!c.have_a32) make_fp32_copy(c, -1);
    if (!c.tl.ready)
      GPZ_REQUIRE(two_level_build(c) == GPZ_OK, GPZ_E_INVALID, "two-level preconditioner: not a uniform Q2 hex grid");
    if (!c.tl.have_inv) two_level_assemble(c);
  }
  if (block && !c.have_bjinv) build_block_jacobi(c);
  if (vb && (!c.have_vbinv || c.vb_kind != precond)) build_vblocks(c, precond);
  alloc_work(c, tl);
  SolverWork &w = c.sw;
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.r.p, hr, c.neq * sizeof(double), cudaMemcpyHostToDevice, s));
  if (tl) {
    Plan P;
    P.nunits = c.neq / 3;
    c.d_bjinv32.alloc((size_t)P.nunits * 9);
    k_to_f32<<<wave(k_to_f32), kThreads, 0, s>>>(c.d_bjinv.p, c.d_bjinv32.p, (int64_t)P.nunits * 9);
    P.M32 = Prec32{nullptr, c.d_bjinv32.p, 1};
    TwoLevel &T = c.tl;
    P.T = tl_view(T);
    T.rc.zero(s);
    double hs[S_NSCAL] = {0};
    int64_t hi[I_NISCAL] = {0};
    hi[I_MAXIT] = 1;
    hi[I_UPDATE] = 2;  // r32 = r
    GPZ_CUDA_TRY(cudaMemcpyAsync(w.scal.p, hs, sizeof(hs), cudaMemcpyHostToDevice, s));
    GPZ_CUDA_TRY(cudaMemcpyAsync(w.iscal.p, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
    launch_tl_apply(c, P, red_of(c), s);
    c.launches++;
    std::vector<float> z(c.neq);
    GPZ_CUDA_TRY(cudaMemcpyAsync(z.data(), T.z32.p, c.neq * sizeof(float), cudaMemcpyDeviceToHost, s));
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));
    for (int64_t i = 0; i < c.neq; i++) hz[i] = z[i];
  } else {
    if (vb) {
      k_vb_apply<<<wave(k_vb_apply), kThreads, 0, s>>>(w.r.p, vblk_of(c), w.q.p);
    } else {
      const Prec M{c.d_dinv.p, block ? c.d_bjinv.p : nullptr, block ? 1 : 0};
      k_prec_apply<<<wave(k_prec_apply), kThreads, 0, s>>>(w.r.p, M, block ? c.neq / 3 : c.neq, w.q.p);
    }
    c.launches++;
    GPZ_CUDA_TRY(cudaMemcpyAsync(hz, w.q.p, c.neq * sizeof(double), cudaMemcpyDeviceToHost, s));
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  }
  GPZ_CUDA_TRY(cudaGetLastError());
  check_device_flag(c, "preconditioner application");
}

// y = A32 x with the mixed CG's FP32 operator in its current layout (the
// autotuned one, or `variant` >= 0), from and to host FP64 vectors
void spmv32_apply(Ctx &c, int variant, const double *hx, double *hy) {
  if (!c.have_a32 || (variant >= 0 && (c.have_bsr3 || c.nstate == 1) && variant != c.spmv32_variant))
    make_fp32_copy(c, variant);
  alloc_work(c, true);
  SolverWork &w = c.sw;
  cudaStream_t s = c.stream;
  const bool padded_in = c.have_bsr3;
  const bool padded_out = c.have_bsr3 && c.spmv32_variant >= 4;
  std::vector<float> xin(w.pm.n, 0.f);
  for (int64_t i = 0; i < c.neq; i++) xin[padded_in ? 4 * (i / 3) + i % 3 : i] = (float)hx[i];
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.pm.p, xin.data(), xin.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  w.q32.zero(s);
  double hs[S_NSCAL] = {0};
  hs[S_RHO] = 1.0;
  int64_t hi[I_NISCAL] = {0};
  hi[I_MAXIT] = 1;
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.scal.p, hs, sizeof(hs), cudaMemcpyHostToDevice, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.iscal.p, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
  Red R = red_of(c);
  if (c.have_bsr3) {
    launch_spmv32(c, c.spmv32_variant, c.sell, R, s);
  } else if (c.spmv32_variant == 9 && c.mf1.ready) {
    matfree1_spmv(c, s, w.pm.p, w.q32.p);
  } else {
    GPZ_TPR_SWITCH(pick_tpr32(c.nnz, c.neq), (k_mx_csr<T><<<wave(k_mx_csr<T>), kThreads, 0, s>>>(
                                                 c.d_ia.p, c.d_ja.p, c.d_a32.p, w.pm.p, w.q32.p, c.neq, R)));
    c.launches++;
  }
  GPZ_CUDA_TRY(cudaGetLastError());
  std::vector<float> yout(w.q32.n);
  GPZ_CUDA_TRY(cudaMemcpyAsync(yout.data(), w.q32.p, yout.size() * sizeof(float), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  check_device_flag(c, "FP32 SpMV");
  for (int64_t i = 0; i < c.neq; i++) hy[i] = yout[padded_out ? 4 * (i / 3) + i % 3 : i];
}

void solver_prepare(Ctx &c, bool mixed) {
  if (mixed && !c.have_a32) make_fp32_copy(c);
  alloc_work(c, mixed);
}

double time_spmv(Ctx &c, bool f32, int reps) {
  if (f32 && !c.have_a32) make_fp32_copy(c);
  alloc_work(c, f32);
  SolverWork &w = c.sw;
  cudaStream_t s = c.stream;
  std::vector<double> ones(c.neq, 1.0);
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.p.p, ones.data(), c.neq * sizeof(double), cudaMemcpyHostToDevice, s));
  if (f32) {
    std::vector<float> o1(w.pm.n, 1.0f);
    GPZ_CUDA_TRY(cudaMemcpyAsync(w.pm.p, o1.data(), o1.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  }
  int64_t hi[I_NISCAL] = {0};
  hi[I_MAXIT] = 1;
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.iscal.p, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
  Red R = red_of(c);
  const int tpr = pick_tpr(c.nnz, c.neq);
  auto launch = [&]() {
    if (f32 && c.have_bsr3) {
      launch_spmv32(c, c.spmv32_variant, c.sell, R, s);
      c.launches--;
    } else if (f32 && c.spmv32_variant == 9 && c.mf1.ready) {
      matfree1_spmv(c, s, w.pm.p, w.q32.p);
      c.launches--;
    } else if (f32) {
      GPZ_TPR_SWITCH(pick_tpr32(c.nnz, c.neq), (k_mx_csr<T><<<wave(k_mx_csr<T>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a32.p, w.pm.p,
                                                                              w.q32.p, c.neq, R)));
    } else {
      GPZ_TPR_SWITCH(tpr, (k_cg_spmv<T, false><<<wave(k_cg_spmv<T, false>), kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, nullptr,
                                                                                w.p.p, nullptr, w.q.p, c.neq, R)));
    }
    c.launches++;
  };
  for (int i = 0; i < 3; i++) launch();
  cudaEvent_t e0, e1;
  GPZ_CUDA_TRY(cudaEventCreate(&e0));
  GPZ_CUDA_TRY(cudaEventCreate(&e1));
  GPZ_CUDA_TRY(cudaEventRecord(e0, s));
  for (int i = 0; i < reps; i++) launch();
  GPZ_CUDA_TRY(cudaEventRecord(e1, s));
  GPZ_CUDA_TRY(cudaEventSynchronize(e1));
  GPZ_CUDA_TRY(cudaGetLastError());
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / reps;
}

}  // namespace gpz
