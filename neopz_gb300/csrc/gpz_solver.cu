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
#include <cmath>

#include "gpz_internal.h"

namespace gpz {

namespace {

constexpr int kThreads = 256;
constexpr int kGridBlocks = 152 * 8;  // 8 CTAs of 256 threads per SM, 152 SMs

// device scalar slots
enum { S_RHO = 0, S_RHO1, S_PQ, S_RR, S_NORMB, S_TOL, S_MAXRR, S_DELTA2, S_RESID, S_TRUERR, S_NSCAL };
enum { I_CONV = 0, I_IT, I_MAXIT, I_UPDATE, I_NUPD, I_SP64, I_SP32, I_BREAK, I_NISCAL };

struct Red {
  double *partial;   // [grid][4]
  unsigned *counter;
  double *scal;
  int64_t *iscal;
};

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block-reduce NV values, publish the block partial, and return true in the
// last block to finish (after which tot[] holds the grid totals, summed in
// block order).
template <int NV>
__device__ bool grid_reduce(double (&v)[NV], const Red &R, double (&tot)[NV]) {
  __shared__ double sh[NV][kThreads / 32];
  __shared__ bool last;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int k = 0; k < NV; k++) {
    double s = warp_sum(v[k]);
    if (lane == 0) sh[k][w] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < NV; k++) {
      double s = 0.0;
      for (int i = 0; i < kThreads / 32; i++) s += sh[k][i];
      R.partial[(size_t)blockIdx.x * 4 + k] = s;
    }
    __threadfence();
    unsigned t = atomicAdd(R.counter, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc[NV];
  for (int k = 0; k < NV; k++) acc[k] = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
    for (int k = 0; k < NV; k++) acc[k] += ((volatile double *)R.partial)[(size_t)i * 4 + k];
  __syncthreads();
  for (int k = 0; k < NV; k++) {
    double s = warp_sum(acc[k]);
    if (lane == 0) sh[k][w] = s;
  }
  __syncthreads();
  for (int k = 0; k < NV; k++) {
    double s = 0.0;
    for (int i = 0; i < kThreads / 32; i++) s += sh[k][i];
    tot[k] = s;
  }
  if (threadIdx.x == 0) *R.counter = 0u;
  return true;
}

__device__ __forceinline__ bool active(const int64_t *is) { return is[I_CONV] == 0 && is[I_IT] < is[I_MAXIT]; }

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
  double s = 0.0;
  int64_t k0 = valid ? ia[r] : 0, k1 = valid ? ia[r + 1] : 0;
  for (int64_t k = k0 + sub; k < k1; k += TPR) s += a[k] * __ldg(&x[ja[k]]);
  for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
  return s;
}

template <int TPR>
__device__ __forceinline__ float row_dot32(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                           const float *__restrict__ a, const float *__restrict__ x, int64_t r,
                                           int sub, bool valid) {
  float s = 0.0f;
  int64_t k0 = valid ? ia[r] : 0, k1 = valid ? ia[r + 1] : 0;
  for (int64_t k = k0 + sub; k < k1; k += TPR) s = fmaf(a[k], __ldg(&x[ja[k]]), s);
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

// q = A p with p.q (iteration kernel C), FP64 or FP32 values
template <int TPR, bool F32>
__global__ void __launch_bounds__(kThreads) k_cg_spmv(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                      const double *__restrict__ a64, const float *__restrict__ a32,
                                                      const double *__restrict__ p, const float *__restrict__ p32,
                                                      double *__restrict__ q, int64_t n, Red R) {
  if (!active(R.iscal)) return;
  double pq = 0.0;
  GPZ_ROW_LOOP(TPR, n) {
    const int64_t r = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = r < n;
    double s;
    if (F32) s = (double)row_dot32<TPR>(ia, ja, a32, p32, r, sub, valid);
    else s = row_dot64<TPR>(ia, ja, a64, p, r, sub, valid);
    if (sub == 0 && valid) {
      q[r] = s;
      pq += p[r] * s;
    }
  }
  double v[1] = {pq}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) {
    R.scal[S_PQ] = tot[0];
    if (F32) R.iscal[I_SP32]++;
    else R.iscal[I_SP64]++;
  }
}

// kernel B: p = z + beta p (z = dinv r), first iteration p = z
__global__ void __launch_bounds__(kThreads) k_cg_p(const double *__restrict__ r, const double *__restrict__ dinv,
                                                   double *__restrict__ p, float *__restrict__ p32, int64_t n, Red R) {
  if (!active(R.iscal)) return;
  const bool first = R.iscal[I_IT] == 0;
  const double beta = first ? 0.0 : R.scal[S_RHO] / R.scal[S_RHO1];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double z = r[i] * dinv[i];
    double pi = first ? z : z + beta * p[i];
    p[i] = pi;
    if (p32) p32[i] = (float)pi;
  }
}

// kernel D: alpha = rho / pq; x += alpha p; r -= alpha q; rho' = r.z, rr = r.r
__global__ void __launch_bounds__(kThreads) k_cg_update(double *__restrict__ x, double *__restrict__ r,
                                                        const double *__restrict__ p, const double *__restrict__ q,
                                                        const double *__restrict__ dinv, int64_t n, int mixed, Red R) {
  if (!active(R.iscal)) return;
  const double pq = R.scal[S_PQ];
  const double alpha = R.scal[S_RHO] / pq;
  double rz = 0.0, rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double xi = x[i] + alpha * p[i];
    double ri = r[i] - alpha * q[i];
    x[i] = xi;
    r[i] = ri;
    rz += ri * (ri * dinv[i]);
    rr += ri * ri;
  }
  double v[2] = {rz, rr}, tot[2];
  if (grid_reduce<2>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    if (!(pq > 0.0) || !isfinite(tot[1])) is[I_BREAK] = 1;
    s[S_RHO1] = s[S_RHO];
    s[S_RHO] = tot[0];
    s[S_RR] = tot[1];
    double resid = sqrt(tot[1]) / s[S_NORMB];
    s[S_RESID] = resid;
    is[I_IT] += 1;
    if (is[I_BREAK]) is[I_CONV] = 2;
    else if (!mixed) {
      if (resid <= s[S_TOL]) is[I_CONV] = 1;
    } else {
      if (resid <= s[S_TOL] || tot[1] < s[S_DELTA2] * s[S_MAXRR]) is[I_UPDATE] = 1;
    }
  }
}

// kernel E (mixed): when flagged, r = b - A64 x in FP64 and restart the
// residual bookkeeping from it.
template <int TPR>
__global__ void __launch_bounds__(kThreads) k_reliable(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                       const double *__restrict__ a, const double *__restrict__ x,
                                                       const double *__restrict__ b, const double *__restrict__ dinv,
                                                       double *__restrict__ r, int64_t n, Red R) {
  if (R.iscal[I_UPDATE] == 0 || R.iscal[I_CONV] != 0) return;
  double rz = 0.0, rr = 0.0;
  GPZ_ROW_LOOP(TPR, n) {
    const int64_t i = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = i < n;
    double s = row_dot64<TPR>(ia, ja, a, x, i, sub, valid);
    if (sub == 0 && valid) {
      double ri = b[i] - s;
      r[i] = ri;
      rz += ri * (ri * dinv[i]);
      rr += ri * ri;
    }
  }
  double v[2] = {rz, rr}, tot[2];
  if (grid_reduce<2>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    s[S_RHO] = tot[0];
    s[S_RR] = tot[1];
    s[S_MAXRR] = tot[1];
    s[S_TRUERR] = tot[1];
    double resid = sqrt(tot[1]) / s[S_NORMB];
    s[S_RESID] = resid;
    is[I_UPDATE] = 0;
    is[I_NUPD] += 1;
    is[I_SP64] += 1;
    if (resid <= s[S_TOL]) is[I_CONV] = 1;
  }
}

// initial residual: r = b (x = 0) or r = b - A x; rho = r.z, rr = r.r, normb
template <int TPR>
__global__ void __launch_bounds__(kThreads) k_cg_init(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                                                      const double *__restrict__ a, double *__restrict__ x,
                                                      const double *__restrict__ b, const double *__restrict__ dinv,
                                                      double *__restrict__ r, int64_t n, int from_current, Red R) {
  double rz = 0.0, rr = 0.0, bb = 0.0;
  GPZ_ROW_LOOP(TPR, n) {
    const int64_t i = r0 + (threadIdx.x & 31) / TPR;
    const bool valid = i < n;
    double s = 0.0;
    if (from_current) s = row_dot64<TPR>(ia, ja, a, x, i, sub, valid);
    if (sub == 0 && valid) {
      double bi = b[i];
      double ri = bi - s;
      if (!from_current) x[i] = 0.0;
      r[i] = ri;
      rz += ri * (ri * dinv[i]);
      rr += ri * ri;
      bb += bi * bi;
    }
  }
  double v[3] = {rz, rr, bb}, tot[3];
  if (grid_reduce<3>(v, R, tot) && threadIdx.x == 0) {
    double *s = R.scal;
    int64_t *is = R.iscal;
    double normb = sqrt(tot[2]);
    if (normb == 0.0) normb = 1.0;
    s[S_NORMB] = normb;
    s[S_RHO] = tot[0];
    s[S_RHO1] = 0.0;
    s[S_RR] = tot[1];
    s[S_MAXRR] = tot[1];
    double resid = sqrt(tot[1]) / normb;
    s[S_RESID] = resid;
    is[I_IT] = 0;
    is[I_CONV] = (resid <= s[S_TOL]) ? 1 : 0;
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
      double ri = b[i] - s;
      rr += ri * ri;
    }
  }
  double v[1] = {rr}, tot[1];
  if (grid_reduce<1>(v, R, tot) && threadIdx.x == 0) R.scal[S_TRUERR] = tot[0];
}

int pick_tpr(int64_t nnz, int64_t n) {
  double avg = n ? (double)nnz / (double)n : 0.0;
  if (avg > 48) return 32;
  if (avg > 20) return 16;
  if (avg > 8) return 8;
  return 4;
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
  GPZ_TPR_SWITCH(tpr, (k_spmv64<T><<<kGridBlocks, kThreads, 0, c.stream>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, x, y, yin,
                                                                            alpha, beta, c.neq)));
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
}

namespace {

void alloc_work(Ctx &c, bool mixed) {
  SolverWork &w = c.sw;
  int64_t n = std::max<int64_t>(c.neq, 1);
  w.r.alloc(n);
  w.p.alloc(n);
  w.q.alloc(n);
  w.x.alloc(n);
  w.b.alloc(n);
  if (mixed) w.p32.alloc(n);
  w.partial.alloc((size_t)kGridBlocks * 4);
  w.scal.alloc(S_NSCAL);
  w.iscal.alloc(I_NISCAL);
  w.counter.alloc(1);
  w.counter.zero(c.stream);
}

Red red_of(Ctx &c) { return Red{c.sw.partial.p, c.sw.counter.p, c.sw.scal.p, c.sw.iscal.p}; }

void launch_iteration(Ctx &c, bool mixed, int tpr) {
  SolverWork &w = c.sw;
  Red R = red_of(c);
  k_cg_p<<<kGridBlocks, kThreads, 0, c.stream>>>(w.r.p, c.d_dinv.p, w.p.p, mixed ? w.p32.p : nullptr, c.neq, R);
  if (mixed) {
    GPZ_TPR_SWITCH(tpr, (k_cg_spmv<T, true><<<kGridBlocks, kThreads, 0, c.stream>>>(
                            c.d_ia.p, c.d_ja.p, nullptr, c.d_a32.p, w.p.p, w.p32.p, w.q.p, c.neq, R)));
  } else {
    GPZ_TPR_SWITCH(tpr, (k_cg_spmv<T, false><<<kGridBlocks, kThreads, 0, c.stream>>>(
                            c.d_ia.p, c.d_ja.p, c.d_a.p, nullptr, w.p.p, nullptr, w.q.p, c.neq, R)));
  }
  k_cg_update<<<kGridBlocks, kThreads, 0, c.stream>>>(w.x.p, w.r.p, w.p.p, w.q.p, c.d_dinv.p, c.neq, mixed ? 1 : 0,
                                                      R);
  c.launches += 3;
  if (mixed) {
    GPZ_TPR_SWITCH(tpr, (k_reliable<T><<<kGridBlocks, kThreads, 0, c.stream>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, w.x.p,
                                                                                w.b.p, c.d_dinv.p, w.r.p, c.neq, R)));
    c.launches++;
  }
}

}  // namespace

int solve(Ctx &c, const gpz_solver_opts &o, gpz_solve_report &rep) {
  const bool mixed = o.solver == GPZ_SOLVER_MIXED_CG;
  GPZ_REQUIRE(o.solver == GPZ_SOLVER_CG || mixed, GPZ_E_INVALID, "solver kind not available");
  GPZ_REQUIRE(o.precond == GPZ_PRECOND_JACOBI || o.precond == 0, GPZ_E_INVALID, "preconditioner not available");
  if (mixed && !c.have_a32) make_fp32_copy(c);
  SolverWork &w = c.sw;
  cudaStream_t s = c.stream;
  const int tpr = pick_tpr(c.nnz, c.neq);
  const int batch = o.check_every > 0 ? o.check_every : 32;

  cudaEvent_t ev0, ev1;
  GPZ_CUDA_TRY(cudaEventCreate(&ev0));
  GPZ_CUDA_TRY(cudaEventCreate(&ev1));
  GPZ_CUDA_TRY(cudaEventRecord(ev0, s));

  double hs[S_NSCAL] = {0};
  hs[S_TOL] = o.tol;
  hs[S_DELTA2] = (o.reliable_delta > 0 ? o.reliable_delta : 1e-3);
  hs[S_DELTA2] *= hs[S_DELTA2];
  int64_t hi[I_NISCAL] = {0};
  hi[I_MAXIT] = o.max_iter;
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.scal.p, hs, sizeof(hs), cudaMemcpyHostToDevice, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(w.iscal.p, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
  Red R = red_of(c);
  GPZ_TPR_SWITCH(tpr, (k_cg_init<T><<<kGridBlocks, kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, w.x.p, w.b.p,
                                                                      c.d_dinv.p, w.r.p, c.neq, o.from_current, R)));
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());

  cudaGraphExec_t exec = nullptr;
  if (o.use_graph) {
    cudaGraph_t g;
    GPZ_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int64_t l0 = c.launches;
    for (int i = 0; i < batch; i++) launch_iteration(c, mixed, tpr);
    GPZ_CUDA_TRY(cudaStreamEndCapture(s, &g));
    int64_t per_graph = c.launches - l0;
    c.launches = l0;
    GPZ_CUDA_TRY(cudaGraphInstantiate(&exec, g, 0));
    GPZ_CUDA_TRY(cudaGraphDestroy(g));
    (void)per_graph;
  }
  const int per_iter = mixed ? 4 : 3;
  int64_t hstate[I_NISCAL];
  for (;;) {
    if (exec) {
      GPZ_CUDA_TRY(cudaGraphLaunch(exec, s));
      c.launches += (int64_t)batch * per_iter;
    } else {
      for (int i = 0; i < batch; i++) launch_iteration(c, mixed, tpr);
    }
    GPZ_CUDA_TRY(cudaGetLastError());
    GPZ_CUDA_TRY(cudaMemcpyAsync(hstate, w.iscal.p, sizeof(hstate), cudaMemcpyDeviceToHost, s));
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));
    if (hstate[I_CONV] != 0 || hstate[I_IT] >= o.max_iter) break;
  }
  if (exec) cudaGraphExecDestroy(exec);
  GPZ_TPR_SWITCH(tpr, (k_true_resid<T><<<kGridBlocks, kThreads, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_a.p, w.x.p, w.b.p,
                                                                         c.neq, R)));
  c.launches++;
  GPZ_CUDA_TRY(cudaEventRecord(ev1, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(hs, w.scal.p, sizeof(hs), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaMemcpyAsync(hstate, w.iscal.p, sizeof(hstate), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  rep.iterations = hstate[I_IT];
  rep.resid = hs[S_RESID];
  rep.true_resid = std::sqrt(hs[S_TRUERR]) / hs[S_NORMB];
  rep.seconds = ms * 1e-3;
  rep.spmv_fp64 = hstate[I_SP64] + 1;
  rep.spmv_fp32 = hstate[I_SP32];
  rep.reliable_updates = hstate[I_NUPD];
  c.have_solution = true;
  if (hstate[I_BREAK]) return GPZ_E_BREAKDOWN;
  return hstate[I_CONV] == 1 ? GPZ_OK : GPZ_NOT_CONVERGED;
}

void solver_prepare(Ctx &c, bool mixed) { alloc_work(c, mixed); }

}  // namespace gpz
