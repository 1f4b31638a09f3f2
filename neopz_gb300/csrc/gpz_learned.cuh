// Device view of the learned preconditioner shared by the network kernels
// (gpz_learned.cu) and the flexible CG (gpz_solver.cu).
//
// The preconditioner is linear and symmetric positive definite in the
// residual by construction; what is learned is how it depends on the
// coefficient field:
//
//   M r = S (alpha u + m .* sum_e Q_e^T F_e F_e^T Q_e (m .* u)),   u = S r,
//
// with S = diag(a_ii)^-1/2 (the symmetric Jacobi scaling), m the mask that is 0
// on penalty-Dirichlet equations (where Jacobi is already exact), Q_e the
// gather of element e's equations (its destination indices, in the order of
// TPZElementMatrix::ComputeDestinationIndices, Mesh/pzelmat.cpp:37-96) and
// F_e an NS x R factor per element; alpha = exp(a) > 0 a learned scale of the
// Jacobi part.  The factors come from an element-to-node
// message-passing network over the element coefficients (see gpz_learned.cu),
// evaluated once per solve; each application costs one gather, 2 NS R
// multiply-adds per element and one gather back per equation.
#pragma once
#include <cstdint>

namespace gpz {

struct LnView {
  const float *F;         // [E][NS][R] element factors
  const uint16_t *F16;    // the same rounded to bfloat16 for the solves (half the bytes per application)
  const uint16_t *F16ne;  // bfloat16 rows in incidence order (row k belongs to incidence k of ne_idx)
  const int32_t *dest;    // [E][NS] element equations
  const int64_t *ne_ptr;  // [neq+1] equation -> (element, local) incidences
  const int32_t *ne_idx;  // e * NS + local
  const float *mdsq;      // [neq] m_i S_i (0 on penalty-Dirichlet equations)
  const double *dinv;     // [neq] 1 / a_ii
  const float *dinv32;    // the same in FP32
  const float *loga;      // log of the learned scale of the Jacobi part (one parameter)
  float *t;               // [E][R] F_e^T Q_e (m .* u)
  int64_t E, n;
  int NS, R;
};

// The correction runs in FP32 (this part's FP64 rate is a small fraction of
// its FP32 rate); only the Jacobi part z = r / a_ii stays FP64.
// One thread per (element, column k): t_e[k] = sum_loc F_e[loc][k] m S r[dest].
template <class T>
__device__ __forceinline__ void ln_elem_t(const LnView &L, const T *__restrict__ r, int64_t idx) {
  const int32_t e = (int32_t)idx / L.R;  // E * R < 2^31 (checked at set-up)
  const int k = (int)idx - e * L.R;
  const int32_t *d = L.dest + e * L.NS;
  const float *f = L.F + (size_t)e * L.NS * L.R + k;
  float acc = 0.f;
  for (int loc = 0; loc < L.NS; loc++) {
    const int32_t q = d[loc];
    acc += f[(size_t)loc * L.R] * (L.mdsq[q] * (float)r[q]);
  }
  L.t[idx] = acc;
}

constexpr int kLnMaxR = 8;  // largest rank R of the factors

// one factor row F_e[loc][0..R) (el = e * NS + loc) as floats; B16: from the
// bfloat16 copy (one 16-byte load for R = 8)
template <bool B16>
__device__ __forceinline__ void ln_row(const LnView &L, size_t el, float (&f)[kLnMaxR]) {
  if (B16) {
    const uint16_t *h = L.F16 + el * L.R;
    if (L.R == 8) {
      const uint4 v = *(const uint4 *)h;
      const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int k = 0; k < 4; k++) {
        f[2 * k] = __uint_as_float(w[k] << 16);
        f[2 * k + 1] = __uint_as_float(w[k] & 0xffff0000u);
      }
    } else {
#pragma unroll
      for (int k = 0; k < kLnMaxR; k++) f[k] = k < L.R ? __uint_as_float((uint32_t)h[k] << 16) : 0.f;
    }
  } else {
    const float *g = L.F + el * L.R;
    if (L.R == 8) {
      const float4 a = *(const float4 *)g, b = *(const float4 *)(g + 4);
      f[0] = a.x; f[1] = a.y; f[2] = a.z; f[3] = a.w; f[4] = b.x; f[5] = b.y; f[6] = b.z; f[7] = b.w;
    } else {
#pragma unroll
      for (int k = 0; k < kLnMaxR; k++) f[k] = k < L.R ? g[k] : 0.f;
    }
  }
}

// t_e = F_e^T Q_e (m .* S r) with one warp per element (elements of 32 or more
// equations): lanes over the element's equations, then a warp sum per column;
// lane k writes t_e[k].
template <class T, bool B16>
__device__ __forceinline__ void ln_elem_t_warp(const LnView &L, const T *__restrict__ r, int64_t e, int lane) {
  float acc[kLnMaxR];
#pragma unroll
  for (int k = 0; k < kLnMaxR; k++) acc[k] = 0.f;
  const int32_t *d = L.dest + e * L.NS;
  for (int loc = lane; loc < L.NS; loc += 32) {
    const int32_t q = d[loc];
    const float v = L.mdsq[q] * (float)r[q];
    float f[kLnMaxR];
    ln_row<B16>(L, (size_t)e * L.NS + loc, f);
#pragma unroll
    for (int k = 0; k < kLnMaxR; k++) acc[k] += f[k] * v;
  }
#pragma unroll
  for (int k = 0; k < kLnMaxR; k++) {
    if (k >= L.R) break;
    float s = acc[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == k) L.t[e * L.R + k] = s;
  }
}

// the same with one thread per (element, column k), for small elements
template <class T>
__device__ __forceinline__ void ln_elem_t16(const LnView &L, const T *__restrict__ r, int64_t idx) {
  const int32_t e = (int32_t)idx / L.R;
  const int k = (int)idx - e * L.R;
  const int32_t *d = L.dest + e * L.NS;
  const uint16_t *h = L.F16 + (size_t)e * L.NS * L.R + k;
  float acc = 0.f;
  for (int loc = 0; loc < L.NS; loc++) {
    const int32_t q = d[loc];
    acc += __uint_as_float((uint32_t)h[(size_t)loc * L.R] << 16) * (L.mdsq[q] * (float)r[q]);
  }
  L.t[idx] = acc;
}

// correction at equation i: m_i S_i sum_{(e,loc) at i} F_e[loc] . t_e
template <bool B16>
__device__ __forceinline__ float ln_node_corr_t(const LnView &L, int64_t i) {
  float c = 0.f;
  for (int64_t k = L.ne_ptr[i]; k < L.ne_ptr[i + 1]; k++) {
    const int32_t el = L.ne_idx[k];
    const int32_t e = el / L.NS;
    float f[kLnMaxR];
    ln_row<B16>(L, (size_t)el, f);
    const float *t = L.t + (size_t)e * L.R;
    if (L.R == 8) {
      const float4 t0 = *(const float4 *)t, t1 = *(const float4 *)(t + 4);
      c += f[0] * t0.x + f[1] * t0.y + f[2] * t0.z + f[3] * t0.w + f[4] * t1.x + f[5] * t1.y + f[6] * t1.z +
           f[7] * t1.w;
    } else {
      for (int j = 0; j < L.R; j++) c += f[j] * t[j];
    }
  }
  return L.mdsq[i] * c;
}
__device__ __forceinline__ float ln_node_corr(const LnView &L, int64_t i) { return ln_node_corr_t<false>(L, i); }

// the same for the solves, from the incidence-ordered bfloat16 rows: the rows of
// consecutive equations are contiguous, so a warp streams them
__device__ __forceinline__ float ln_node_corr_ne(const LnView &L, int64_t i) {
  float c = 0.f;
  for (int64_t k = L.ne_ptr[i]; k < L.ne_ptr[i + 1]; k++) {
    const int32_t e = L.ne_idx[k] / L.NS;
    const uint16_t *h = L.F16ne + (size_t)k * L.R;
    const float *t = L.t + (size_t)e * L.R;
    if (L.R == 8) {
      const uint4 v = *(const uint4 *)h;
      const float4 t0 = *(const float4 *)t, t1 = *(const float4 *)(t + 4);
      c += __uint_as_float(v.x << 16) * t0.x + __uint_as_float(v.x & 0xffff0000u) * t0.y +
           __uint_as_float(v.y << 16) * t0.z + __uint_as_float(v.y & 0xffff0000u) * t0.w +
           __uint_as_float(v.z << 16) * t1.x + __uint_as_float(v.z & 0xffff0000u) * t1.y +
           __uint_as_float(v.w << 16) * t1.z + __uint_as_float(v.w & 0xffff0000u) * t1.w;
    } else {
      for (int j = 0; j < L.R; j++) c += __uint_as_float((uint32_t)h[j] << 16) * t[j];
    }
  }
  return L.mdsq[i] * c;
}

// z_i = alpha r_i / a_ii + correction, alpha = exp(loga)
template <class T>
__device__ __forceinline__ double ln_node_z(const LnView &L, const T *__restrict__ r, double alpha, int64_t i) {
  return alpha * L.dinv[i] * (double)r[i] + (double)ln_node_corr(L, i);
}

}  // namespace gpz
