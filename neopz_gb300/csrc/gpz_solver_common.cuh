// Device helpers shared by the solver kernels (gpz_solver.cu) and the
// matrix-free operator (gpz_matfree.cu): grid sizing, the device scalar slots
// of the Krylov recurrences and the deterministic grid reduction.
#pragma once
#include <cstdint>

#include "gpz_internal.h"

namespace gpz {
namespace {

constexpr int kThreads = 256;
constexpr int kGridBlocks = 152 * 8;  // upper bound of the grid-stride grids (partial-sum buffer size)

// Grid-stride kernels run exactly one wave: SMs x resident CTAs of this kernel.
template <class K>
int wave(K kernel) {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 152;
  }
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kThreads, 0);
  if (per <= 0) per = 1;
  int g = nsm * per;
  return g > kGridBlocks ? kGridBlocks : g;
}

// device scalar slots
// alpha and beta are formed once, by the CTA that finishes the reduction they depend on
enum { S_RHO = 0, S_RHO1, S_PQ, S_RR, S_NORMB, S_TOL, S_MAXRR, S_DELTA2, S_RESID, S_TRUERR, S_ALPHA, S_BETA, S_RRREC,
       S_NSCAL };
enum { I_CONV = 0, I_IT, I_MAXIT, I_UPDATE, I_NUPD, I_SP64, I_SP32, I_BREAK, I_RESTART, I_NRESTART, I_NISCAL };

struct Red {
  double *partial;   // [grid][4]
  unsigned *counter;
  double *scal;
  int64_t *iscal;
};

// q += v as one vector reduction in L2 without a returned value (the float4
// atomicAdd returns the old value, whose registers the thread then holds until
// the response arrives)
__device__ __forceinline__ void red_add_f4(float4 *p, float4 v) {
  asm volatile("red.relaxed.gpu.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z),
               "f"(v.w)
               : "memory");
}

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
// block order).  CTAs of up to MAXW warps.
template <int NV, int MAXW = kThreads / 32>
__device__ bool grid_reduce(double (&v)[NV], const Red &R, double (&tot)[NV]) {
  __shared__ double sh[NV][MAXW];
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
      for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sh[k][i];
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
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sh[k][i];
    tot[k] = s;
  }
  if (threadIdx.x == 0) *R.counter = 0u;
  return true;
}

__device__ __forceinline__ bool active(const int64_t *is) { return is[I_CONV] == 0 && is[I_IT] < is[I_MAXIT]; }

struct KSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double get() const { return (double)s - (double)c; }
};

}  // namespace
}  // namespace gpz
