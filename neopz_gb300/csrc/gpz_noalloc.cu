// Jacobi-preconditioned FP64 CG that allocates nothing: gpz_cg_jacobi_noalloc.
//
// Who needs it: callers that may not allocate device memory while they solve
// -- a code that has reserved all of HBM for its own pool, a solver called
// from inside another library's memory-managed region, or a time-stepping
// loop that must not touch the allocator after start-up.  The regular
// gpz_solve keeps its work vectors in the context, which allocates them on
// first use.
//
// How: the work vectors (r, p, q, 1/diag), the per-CTA partial sums, the
// scalars and the grid-reduction counter live in one file-scope static device
// array, sized for GPZ_NOALLOC_MAX_EQ equations (about 8.4 MB).  The array's
// device address is looked up once per device (cudaGetSymbolAddress, with that
// device current) the first time the entry point runs there; that first call
// may make the CUDA runtime load this library's device code, so make it once
// during start-up, before any stream capture and before the region that must
// not allocate.  After that a call only launches kernels, sets the flag block
// with cudaMemsetAsync and reads the flag block back with cudaMemcpyAsync into
// host stack memory.  The host waits on the stream every 32 iterations to read
// that block, so each call blocks the calling thread until the solve ends.
//
// Sharing: every call on a device uses the same array.  The reduction counter
// and the flags must start at zero; each call clears them itself before its
// first kernel.  Two calls that overlap in time on one device (different
// host threads or streams) race on the array and give wrong results: issue
// them one after the other.
//
// Algorithm: the CG of Solvers/LinearSolvers/cg.h:29-132 with the Jacobi
// preconditioner of TPZMatrix::SolveJacobi (Matrix/pzmatrix.cpp:643-667), zero
// initial guess, ||b|| = 0 -> 1, stop on the recursive ||r||/||b|| <= tol, over
// a full CSR matrix (TPZFYsmpMatrix layout, Matrix/pzysmp.h).  The reference
// has no counterpart of the allocation-free form: its solver allocates its
// vectors on every call.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <mutex>

#include "gpz.h"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxGrid = 1024;            // CTAs of every launch; partial sums per CTA
constexpr int kBatch = 32;                // iterations between host reads of the flag block
constexpr int64_t kMaxEq = GPZ_NOALLOC_MAX_EQ;

// scratch layout, in doubles
constexpr int64_t kOffR = 0;
constexpr int64_t kOffP = kMaxEq;
constexpr int64_t kOffQ = 2 * kMaxEq;
constexpr int64_t kOffD = 3 * kMaxEq;
constexpr int kNumPart = 3;
constexpr int64_t kOffPart = 4 * kMaxEq;  // kNumPart * kMaxGrid partial sums
constexpr int64_t kOffScal = kOffPart + kNumPart * kMaxGrid;
constexpr int kNumScal = 8;
constexpr int64_t kOffFlag = kOffScal + kNumScal;
constexpr int kNumFlag = 8;               // unsigned 64-bit words
constexpr int64_t kScratchDoubles = kOffFlag + kNumFlag;

enum { SC_RHO, SC_ALPHA, SC_BETA, SC_NORMB, SC_RESID, SC_TOL };
enum { FL_COUNTER, FL_STOP, FL_IT, FL_MAXIT };
enum { STOP_NONE = 0, STOP_CONV = 1, STOP_MAXIT = 2, STOP_BREAK = 3, STOP_BAD_INPUT = 4 };

static_assert(kOffFlag % 2 == 0, "flag block alignment");

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

struct View {
  double *r, *p, *q, *dinv, *part, *scal;
  unsigned long long *flag;
};

__host__ __device__ inline View view_of(double *base) {
  View v;
  v.r = base + kOffR;
  v.p = base + kOffP;
  v.q = base + kOffQ;
  v.dinv = base + kOffD;
  v.part = base + kOffPart;
  v.scal = base + kOffScal;
  v.flag = reinterpret_cast<unsigned long long *>(base + kOffFlag);
  return v;
}

__device__ inline bool stopped(const View &s) {
  return *reinterpret_cast<volatile unsigned long long *>(&s.flag[FL_STOP]) != STOP_NONE;
}

// Sum NV values over the CTA into thread 0.
template <int NV>
__device__ inline void block_sum(double (&v)[NV]) {
  __shared__ double sh[NV][kWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k][w] = v[k];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = 0.0;
      for (int i = 0; i < kWarps; ++i) t += sh[k][i];
      v[k] = t;
    }
  __syncthreads();
}

// Deterministic grid reduction: every CTA stores its partial sums, the last
// CTA to arrive adds them in CTA order.  Returns true in the last CTA, whose
// thread 0 then holds the totals in v; that CTA also re-arms the counter.
template <int NV>
__device__ inline bool grid_sum(const View &s, double (&v)[NV]) {
  __shared__ bool last;
  block_sum<NV>(v);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) s.part[k * kMaxGrid + blockIdx.x] = v[k];
    __threadfence();
    const unsigned long long prev = atomicAdd(&s.flag[FL_COUNTER], 1ull);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double t[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) t[k] = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
#pragma unroll
    for (int k = 0; k < NV; ++k) t[k] += __ldcg(&s.part[k * kMaxGrid + i]);
  block_sum<NV>(t);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = t[k];
    s.flag[FL_COUNTER] = 0;
  }
  return true;
}

// r = b, 1/diag, ||b||, rho = r . (D^-1 r).  Also checks the CSR arrays
// (row pointers inside [0, nnz] and non-decreasing, columns inside [0, n))
// and that every row has a finite, non-zero diagonal; any failure stops the
// solve before the first iteration.  x is not written here: k_na_zero_x
// clears it once the checks have passed, so bad input leaves x as it was.
__global__ void __launch_bounds__(kThreads) k_na_start(int64_t n, int64_t nnz, const int64_t *__restrict__ ia,
                                                       const int32_t *__restrict__ ja, const double *__restrict__ a,
                                                       const double *__restrict__ b, double tol, int64_t maxit,
                                                       View s) {
  double v[3] = {0.0, 0.0, 0.0};  // b.b, b.(D^-1 b), bad rows
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double bi = b[i];
    const int64_t k0 = ia[i], k1 = ia[i + 1];
    bool ok = k0 >= 0 && k1 >= k0 && k1 <= nnz;
    double d = 0.0;
    bool found = false;
    if (ok)
      for (int64_t k = k0; k < k1; ++k) {
        const int32_t c = ja[k];
        if (c < 0 || c >= n) ok = false;
        if (c == i && !found) {
          d = a[k];
          found = true;
        }
      }
    ok = ok && found && d != 0.0 && isfinite(d);
    const double di = ok ? 1.0 / d : 0.0;
    s.r[i] = bi;
    s.p[i] = 0.0;
    s.dinv[i] = di;
    v[0] += bi * bi;
    v[1] += bi * (di * bi);
    v[2] += ok ? 0.0 : 1.0;
  }
  if (grid_sum<3>(s, v) && threadIdx.x == 0) {
    const double nb = sqrt(v[0]);
    const double normb = nb == 0.0 ? 1.0 : nb;
    const double resid = nb / normb;
    s.scal[SC_NORMB] = normb;
    s.scal[SC_RHO] = v[1];
    s.scal[SC_BETA] = 0.0;
    s.scal[SC_ALPHA] = 0.0;
    s.scal[SC_TOL] = tol;
    s.scal[SC_RESID] = resid;
    s.flag[FL_IT] = 0;
    s.flag[FL_MAXIT] = (unsigned long long)maxit;
    unsigned long long stop = STOP_NONE;
    if (v[2] != 0.0) stop = STOP_BAD_INPUT;
    else if (resid <= tol) stop = STOP_CONV;
    else if (maxit <= 0) stop = STOP_MAXIT;
    s.flag[FL_STOP] = stop;
  }
}

// x = 0 (the zero initial guess of cg.h), unless the input checks failed
__global__ void __launch_bounds__(kThreads) k_na_zero_x(int64_t n, double *__restrict__ x, View s) {
  if (*reinterpret_cast<volatile unsigned long long *>(&s.flag[FL_STOP]) == STOP_BAD_INPUT) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = 0.0;
}

// p = D^-1 r + beta p  (beta = 0 in the first iteration, p = 0 from the start kernel)
__global__ void __launch_bounds__(kThreads) k_na_direction(int64_t n, View s) {
  if (stopped(s)) return;
  const double beta = s.scal[SC_BETA];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s.p[i] = s.dinv[i] * s.r[i] + beta * s.p[i];
}

// q = A p (one warp per row), alpha = rho / (p . q)
__global__ void __launch_bounds__(kThreads) k_na_spmv(int64_t n, const int64_t *__restrict__ ia,
                                                      const int32_t *__restrict__ ja, const double *__restrict__ a,
                                                      View s) {
  if (stopped(s)) return;
  const int lane = threadIdx.x & 31;
  double v[1] = {0.0};
  for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n;
       row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    double t = 0.0;
    for (int64_t k = ia[row] + lane; k < ia[row + 1]; k += 32) t += a[k] * s.p[ja[k]];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) {
      s.q[row] = t;
      v[0] += s.p[row] * t;
    }
  }
  if (grid_sum<1>(s, v) && threadIdx.x == 0) {
    const double pq = v[0];
    if (!(pq > 0.0) || !isfinite(pq)) s.flag[FL_STOP] = STOP_BREAK;
    else s.scal[SC_ALPHA] = s.scal[SC_RHO] / pq;
  }
}

// x += alpha p, r -= alpha q, rho' = r . (D^-1 r), ||r||; convergence test and beta
__global__ void __launch_bounds__(kThreads) k_na_update(int64_t n, double *__restrict__ x, View s) {
  if (stopped(s)) return;
  const double alpha = s.scal[SC_ALPHA];
  double v[2] = {0.0, 0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double pi = s.p[i];
    x[i] += alpha * pi;
    const double r = s.r[i] - alpha * s.q[i];
    s.r[i] = r;
    v[0] += r * (s.dinv[i] * r);
    v[1] += r * r;
  }
  if (grid_sum<2>(s, v) && threadIdx.x == 0) {
    const unsigned long long it = s.flag[FL_IT] + 1;
    s.flag[FL_IT] = it;
    const double resid = sqrt(v[1]) / s.scal[SC_NORMB];
    s.scal[SC_RESID] = resid;
    if (resid <= s.scal[SC_TOL]) {
      s.flag[FL_STOP] = STOP_CONV;
    } else if (!isfinite(resid)) {
      s.flag[FL_STOP] = STOP_BREAK;
    } else {
      s.scal[SC_BETA] = v[0] / s.scal[SC_RHO];
      s.scal[SC_RHO] = v[0];
      if (it >= s.flag[FL_MAXIT]) s.flag[FL_STOP] = STOP_MAXIT;
    }
  }
}

std::mutex g_setup_mu;
constexpr int kMaxDevices = 64;
double *g_scratch_ptr[kMaxDevices] = {};

// One-time, per device: the address of the static scratch array on the current device.
int scratch_on_current_device(double **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return GPZ_E_NO_DEVICE;
  }
  if (dev < 0 || dev >= kMaxDevices) return GPZ_E_INVALID;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return GPZ_E_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_scratch_ptr[dev];
  return GPZ_OK;
}

inline int grid_for(int64_t work_items) {
  const int64_t g = (work_items + kThreads - 1) / kThreads;
  return (int)(g < 1 ? 1 : (g > kMaxGrid ? kMaxGrid : g));
}

}  // namespace

extern "C" int gpz_cg_jacobi_noalloc(void *stream, int64_t neq, int64_t nnz, const int64_t *ia, const int32_t *ja, const double *a,
                                     const double *b, double *x, int64_t max_iter, double tol, int64_t *iterations,
                                     double *resid) {
  if (iterations) *iterations = 0;
  if (resid) *resid = 0.0;
  if (neq < 0 || nnz < 0 || max_iter < 0 || !(tol >= 0.0)) return GPZ_E_INVALID;
  if (neq > kMaxEq) return GPZ_E_TOO_LARGE;
  if (neq == 0) return GPZ_OK;
  if (!ia || !ja || !a || !b || !x) return GPZ_E_INVALID;
  double *base = nullptr;
  int rc = scratch_on_current_device(&base);
  if (rc != GPZ_OK) return rc;
  const View s = view_of(base);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (st) {  // a stream of another device would launch against the wrong device's scratch
    int sdev = -1, cur = -1;
    if (cudaStreamGetDevice(st, &sdev) != cudaSuccess || cudaGetDevice(&cur) != cudaSuccess) {
      cudaGetLastError();
      return GPZ_E_INVALID;
    }
    if (sdev != cur) return GPZ_E_INVALID;
  }

  // the counter and the flags start at zero on every call
  if (cudaMemsetAsync(s.flag, 0, kNumFlag * sizeof(unsigned long long), st) != cudaSuccess) {
    cudaGetLastError();
    return GPZ_E_CUDA;
  }
  const int gv = grid_for(neq);
  const int gs = grid_for(neq * 32);
  k_na_start<<<gv, kThreads, 0, st>>>(neq, nnz, ia, ja, a, b, tol, max_iter, s);
  k_na_zero_x<<<gv, kThreads, 0, st>>>(neq, x, s);
  unsigned long long hflag[kNumFlag] = {};
  double hscal[kNumScal] = {};
  const int64_t nbatch = max_iter / kBatch + 2;  // the device stops itself at max_iter
  bool done = false;
  for (int64_t bt = 0; bt <= nbatch; ++bt) {
    if (cudaGetLastError() != cudaSuccess) return GPZ_E_CUDA;
    if (cudaMemcpyAsync(hflag, s.flag, sizeof(hflag), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      cudaGetLastError();
      return GPZ_E_CUDA;
    }
    if (hflag[FL_STOP] != STOP_NONE) {
      done = true;
      break;
    }
    for (int k = 0; k < kBatch; ++k) {
      k_na_direction<<<gv, kThreads, 0, st>>>(neq, s);
      k_na_spmv<<<gs, kThreads, 0, st>>>(neq, ia, ja, a, s);
      k_na_update<<<gv, kThreads, 0, st>>>(neq, x, s);
    }
  }
  if (cudaMemcpyAsync(hscal, s.scal, sizeof(hscal), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return GPZ_E_CUDA;
  }
  if (!done) return GPZ_E_DEVICE_CHECK;
  if (iterations) *iterations = (int64_t)hflag[FL_IT];
  if (resid) *resid = hscal[SC_RESID];
  switch (hflag[FL_STOP]) {
    case STOP_CONV: return GPZ_OK;
    case STOP_MAXIT: return GPZ_NOT_CONVERGED;
    case STOP_BREAK: return GPZ_E_BREAKDOWN;
    case STOP_BAD_INPUT: return GPZ_E_INVALID;
    default: return GPZ_E_DEVICE_CHECK;
  }
}
