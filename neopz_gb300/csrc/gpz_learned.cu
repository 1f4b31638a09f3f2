// Learned preconditioner: an element-to-node message-passing network over the
// element coefficients that produces the per-element factors F_e of the
// symmetric positive definite preconditioner described in gpz_learned.cuh,
// and its training on the GPU (forward, backward and Adam kernels written
// here).  No counterpart in the reference; it plugs into the flexible CG of
// gpz_solver.cu and falls back to Jacobi (TPZMatrix::SolveJacobi,
// Matrix/pzmatrix.cpp:643-667) whenever its correction is not a descent
// direction.
//
// Network (H = 32 channels, one per warp lane; one warp per element or connect):
//   h0_e  = tanh(W0 x_e + b0),                x_e = log(coefficient of e)
//   for l = 1, 2:
//     n_c   = mean_{e at connect c} h_e        (element -> node)
//     nb_e  = mean_{c of e} n_c                (node -> element)
//     h_e  += tanh(W_l [h_e; nb_e] + b_l)
//   F_e   = Wo h2_e + bo                       (NS x R factor, local equations x rank)
// Parameters, in this order (floats): W0[H] b0[H] W1[H][2H] b1[H] W2[H][2H]
// b2[H] Wo[NS*R][H] bo[NS*R] a (the Jacobi part is scaled by exp(a)).
//
// Training data are residual / error pairs (r_k, e_k = x* - x_k) of the
// Jacobi-PCG iterates of the system itself (collect_cg_pairs).  The loss is
// the energy norm of the error left by one application, per pair,
//   L = mean_j (M r_j - e_j)^T A (M r_j - e_j) / e_j^T A e_j,
// over the non-Dirichlet equations (both vectors masked), evaluated with the
// FP64 CSR matrix.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <vector>

#include "gpz_internal.h"
#include <cuda_bf16.h>

#include "gpz_learned.cuh"

namespace gpz {

namespace {

constexpr int kH = 32;
constexpr int kT = 256;
constexpr int kMaxR = 8;
constexpr int kMaxNS = 192;
constexpr int kMaxSeg = 64;
constexpr int kRedBlocks = 256;

struct Offs {
  int64_t W0, b0, W1, b1, W2, b2, Wo, bo, a, total;
};
Offs offs_of(int NR) {
  Offs o;
  o.W0 = 0;
  o.b0 = o.W0 + kH;
  o.W1 = o.b0 + kH;
  o.b1 = o.W1 + kH * 2 * kH;
  o.W2 = o.b1 + kH;
  o.b2 = o.W2 + kH * 2 * kH;
  o.Wo = o.b2 + kH;
  o.bo = o.Wo + (int64_t)NR * kH;
  o.a = o.bo + NR;
  o.total = o.a + 1;
  return o;
}

// activation planes in Learned::act ([E][H] each, nm is [nconn][H])
enum { A_H0 = 0, A_NB1, A_Y1, A_H1, A_NB2, A_Y2, A_H2, A_NE };
// backward planes in Learned::back
enum { B_DH = 0, B_DH2, B_DPRE, B_DNB, B_NE };

__device__ __forceinline__ int64_t gwarp() { return ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ int64_t nwarp() { return ((int64_t)gridDim.x * blockDim.x) >> 5; }
__device__ __forceinline__ int64_t gthread() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t nthread() { return (int64_t)gridDim.x * blockDim.x; }

int grid_w(int64_t nwarps) {  // CTAs of kT threads for one warp per item
  int64_t g = (nwarps + (kT / 32) - 1) / (kT / 32);
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 16));
}
int grid_t(int64_t n) {
  int64_t g = (n + kT - 1) / kT;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 16));
}

// ---------------------------------------------------------------- forward
__global__ void __launch_bounds__(kT) k_ln_h0(int64_t E, const float *__restrict__ feat, const float *__restrict__ P,
                                              int64_t oW0, int64_t ob0, float *__restrict__ h0) {
  for (int64_t k = gthread(); k < E * kH; k += nthread()) {
    const int c = (int)(k & (kH - 1));
    h0[k] = tanhf(P[oW0 + c] * feat[k >> 5] + P[ob0 + c]);
  }
}

// per connect: out = scale * sum_{e at c} in_e, scale = 1/count (mean) or a constant
__global__ void __launch_bounds__(kT) k_ln_node_gather(int64_t nconn, const int64_t *__restrict__ ce_ptr,
                                                       const int32_t *__restrict__ ce_idx,
                                                       const float *__restrict__ in, float *__restrict__ out,
                                                       int mean, float scale) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = gwarp(); i < nconn; i += nwarp()) {
    const int64_t k0 = ce_ptr[i], k1 = ce_ptr[i + 1];
    float s = 0.f;
    for (int64_t k = k0; k < k1; k++) s += in[(int64_t)ce_idx[k] * kH + lane];
    if (mean) s = k1 > k0 ? s / (float)(k1 - k0) : 0.f;
    else s *= scale;
    out[i * kH + lane] = s;
  }
}

// h_out = h + tanh(W [h; nb] + b), nb = mean over the element's connects of nm
__global__ void __launch_bounds__(kT) k_ln_layer(int64_t E, int nsides, const int32_t *__restrict__ ec,
                                                 const float *__restrict__ hprev, const float *__restrict__ nm,
                                                 const float *__restrict__ W, const float *__restrict__ b,
                                                 float *__restrict__ nb_out, float *__restrict__ y_out,
                                                 float *__restrict__ h_out) {
  __shared__ float Wt[2 * kH][kH + 1];  // Wt[j][c] = W[c][j]
  for (int k = threadIdx.x; k < kH * 2 * kH; k += blockDim.x) Wt[k % (2 * kH)][k / (2 * kH)] = W[k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const float bc = b[lane];
  for (int64_t e = gwarp(); e < E; e += nwarp()) {
    float nbv = 0.f;
    for (int s = 0; s < nsides; s++) nbv += nm[(int64_t)ec[e * nsides + s] * kH + lane];
    nbv /= (float)nsides;
    const float hv = hprev[e * kH + lane];
    float pre = bc;
#pragma unroll
    for (int j = 0; j < kH; j++)
      pre += Wt[j][lane] * __shfl_sync(0xffffffffu, hv, j) + Wt[kH + j][lane] * __shfl_sync(0xffffffffu, nbv, j);
    const float y = tanhf(pre);
    nb_out[e * kH + lane] = nbv;
    y_out[e * kH + lane] = y;
    h_out[e * kH + lane] = hv + y;
  }
}

// F_e = Wo h2_e + bo (Wo staged in shared memory, rows padded to 33 floats)
__global__ void __launch_bounds__(kT) k_ln_out(int64_t E, int NR, const float *__restrict__ h2,
                                               const float *__restrict__ Wo, const float *__restrict__ bo,
                                               float *__restrict__ F) {
  extern __shared__ float sm[];
  for (int k = threadIdx.x; k < NR * kH; k += blockDim.x) sm[(k / kH) * (kH + 1) + (k % kH)] = Wo[k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int64_t e = gwarp(); e < E; e += nwarp()) {
    const float hv = h2[e * kH + lane];
    for (int base = 0; base < NR; base += 32) {
      const int o = base + lane;
      float acc = 0.f;
#pragma unroll
      for (int j = 0; j < kH; j++) {
        const float hj = __shfl_sync(0xffffffffu, hv, j);
        if (o < NR) acc += sm[o * (kH + 1) + j] * hj;
      }
      if (o < NR) F[e * NR + o] = acc + bo[o];
    }
  }
}

// ---------------------------------------------------------------- backward
// dF_e = sum_j ge_j t_j^T + ue_j s_j^T with ue = Q_e(m S r_j), ge = Q_e(m S g_j),
// t = F_e^T ue, s = F_e^T ge (the derivative of g^T Q^T F F^T Q u)
__global__ void __launch_bounds__(kT) k_ln_dF(int64_t E, int NS, int R, const int32_t *__restrict__ dest,
                                              const float *__restrict__ F, const double *__restrict__ mask,
                                              const double *__restrict__ dsq, int P, int64_t n,
                                              const double *__restrict__ pr, const double *__restrict__ pg,
                                              float *__restrict__ dF) {
  constexpr int kLoc = kMaxNS / 32;
  const int lane = threadIdx.x & 31;
  for (int64_t e = gwarp(); e < E; e += nwarp()) {
    double acc[kLoc][kMaxR];
#pragma unroll
    for (int m = 0; m < kLoc; m++)
#pragma unroll
      for (int k = 0; k < kMaxR; k++) acc[m][k] = 0.0;
    for (int j = 0; j < P; j++) {
      double ue[kLoc], ge[kLoc];
#pragma unroll
      for (int m = 0; m < kLoc; m++) {
        const int loc = lane + 32 * m;
        ue[m] = ge[m] = 0.0;
        if (loc < NS) {
          const int32_t q = dest[e * NS + loc];
          const double w = mask[q] * dsq[q];
          ue[m] = w * pr[(size_t)j * n + q];
          ge[m] = w * pg[(size_t)j * n + q];
        }
      }
#pragma unroll
      for (int k = 0; k < kMaxR; k++) {
        if (k >= R) break;
        double tk = 0.0, sk = 0.0;
#pragma unroll
        for (int m = 0; m < kLoc; m++) {
          const int loc = lane + 32 * m;
          if (loc < NS) {
            const double f = F[((size_t)e * NS + loc) * R + k];
            tk += f * ue[m];
            sk += f * ge[m];
          }
        }
        for (int o = 16; o > 0; o >>= 1) {
          tk += __shfl_xor_sync(0xffffffffu, tk, o);
          sk += __shfl_xor_sync(0xffffffffu, sk, o);
        }
#pragma unroll
        for (int m = 0; m < kLoc; m++) acc[m][k] += ge[m] * tk + ue[m] * sk;
      }
    }
#pragma unroll
    for (int m = 0; m < kLoc; m++) {
      const int loc = lane + 32 * m;
#pragma unroll
      for (int k = 0; k < kMaxR; k++)
        if (loc < NS && k < R) dF[((size_t)e * NS + loc) * R + k] = (float)acc[m][k];
    }
  }
}

// dh2_e = Wo^T dF_e
__global__ void __launch_bounds__(kT) k_ln_out_back(int64_t E, int NR, const float *__restrict__ dF,
                                                    const float *__restrict__ Wo, float *__restrict__ dh) {
  extern __shared__ float sm[];
  for (int k = threadIdx.x; k < NR * kH; k += blockDim.x) sm[(k / kH) * (kH + 1) + (k % kH)] = Wo[k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int64_t e = gwarp(); e < E; e += nwarp()) {
    float acc = 0.f;
    for (int base = 0; base < NR; base += 32) {
      const float v = base + lane < NR ? dF[e * NR + base + lane] : 0.f;
#pragma unroll
      for (int jj = 0; jj < 32; jj++) {
        const float d = __shfl_sync(0xffffffffu, v, jj);
        if (base + jj < NR) acc += sm[(base + jj) * (kH + 1) + lane] * d;
      }
    }
    dh[e * kH + lane] = acc;
  }
}

// through h_out = h + tanh(pre): dpre = dh (1 - y^2); dh_prev = dh + (W^T dpre)[:H]; dnb = (W^T dpre)[H:]
__global__ void __launch_bounds__(kT) k_ln_layer_back(int64_t E, const float *__restrict__ dh,
                                                      const float *__restrict__ y, const float *__restrict__ W,
                                                      float *__restrict__ dpre, float *__restrict__ dh_prev,
                                                      float *__restrict__ dnb) {
  __shared__ float Ws[kH][2 * kH + 1];
  for (int k = threadIdx.x; k < kH * 2 * kH; k += blockDim.x) Ws[k / (2 * kH)][k % (2 * kH)] = W[k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int64_t e = gwarp(); e < E; e += nwarp()) {
    const float d = dh[e * kH + lane];
    const float yy = y[e * kH + lane];
    const float dp = d * (1.f - yy * yy);
    float glo = 0.f, ghi = 0.f;
#pragma unroll
    for (int cc = 0; cc < kH; cc++) {
      const float dc = __shfl_sync(0xffffffffu, dp, cc);
      glo += Ws[cc][lane] * dc;
      ghi += Ws[cc][kH + lane] * dc;
    }
    dpre[e * kH + lane] = dp;
    dh_prev[e * kH + lane] = d + glo;
    dnb[e * kH + lane] = ghi;
  }
}

// dh_e += sum_{c of e} dnm_c / count(c)   (transpose of the element -> node mean)
__global__ void __launch_bounds__(kT) k_ln_elem_acc(int64_t E, int nsides, const int32_t *__restrict__ ec,
                                                    const int64_t *__restrict__ ce_ptr,
                                                    const float *__restrict__ dnm, float *__restrict__ dh) {
  const int lane = threadIdx.x & 31;
  for (int64_t e = gwarp(); e < E; e += nwarp()) {
    float acc = 0.f;
    for (int s = 0; s < nsides; s++) {
      const int32_t c = ec[e * nsides + s];
      const int64_t cnt = ce_ptr[c + 1] - ce_ptr[c];
      acc += dnm[(int64_t)c * kH + lane] / (float)cnt;
    }
    dh[e * kH + lane] += acc;
  }
}

__global__ void __launch_bounds__(kT) k_ln_h0_back(int64_t E, const float *__restrict__ dh,
                                                   const float *__restrict__ h0, float *__restrict__ dpre) {
  for (int64_t k = gthread(); k < E * kH; k += nthread()) dpre[k] = dh[k] * (1.f - h0[k] * h0[k]);
}

// out[a][b] = sum_{e in segment} A[e][a] B(e,b) (b < n1 + n2), out[a][n1+n2] = sum A[e][a]
__global__ void __launch_bounds__(kT) k_ln_outer(int64_t E, int64_t seg, int na, int lda, const float *__restrict__ A,
                                                 int n1, int ld1, const float *__restrict__ B1, int n2, int ld2,
                                                 const float *__restrict__ B2, float *__restrict__ partial) {
  const int nb = n1 + n2;
  const int64_t nout = (int64_t)na * (nb + 1);
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nout) return;
  const int a = (int)(o / (nb + 1)), b = (int)(o % (nb + 1));
  const int64_t e0 = (int64_t)blockIdx.y * seg, e1 = std::min<int64_t>(E, e0 + seg);
  double acc = 0.0;
  for (int64_t e = e0; e < e1; e++) {
    const float bv = b < n1 ? B1[e * ld1 + b] : (b < nb ? B2[e * ld2 + (b - n1)] : 1.f);
    acc += (double)A[e * lda + a] * (double)bv;
  }
  partial[(int64_t)blockIdx.y * nout + o] = (float)acc;
}

// sum the segments in order; weights go to grad[oW + a*nb + b], biases to grad[ob + a]
__global__ void __launch_bounds__(kT) k_ln_outer_reduce(int S, int na, int nb, const float *__restrict__ partial,
                                                        float *__restrict__ grad, int64_t oW, int64_t ob) {
  const int64_t nout = (int64_t)na * (nb + 1);
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nout) return;
  double s = 0.0;
  for (int i = 0; i < S; i++) s += partial[(int64_t)i * nout + o];
  const int a = (int)(o / (nb + 1)), b = (int)(o % (nb + 1));
  if (b < nb) grad[oW + (int64_t)a * nb + b] = (float)s;
  else grad[ob + a] = (float)s;
}

__global__ void __launch_bounds__(kT) k_ln_adam(int64_t np, float *__restrict__ p, const float *__restrict__ g,
                                                float *__restrict__ m, float *__restrict__ v, float lr, float b1,
                                                float b2, float eps, float c1, float c2) {
  for (int64_t i = gthread(); i < np; i += nthread()) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// ---------------------------------------------------------------- preconditioner application, loss pieces
__global__ void __launch_bounds__(kT) k_ln_apply_t(LnView L, const double *__restrict__ r) {
  for (int64_t i = gthread(); i < L.E * L.R; i += nthread()) ln_elem_t<double>(L, r, i);
}
__global__ void __launch_bounds__(kT) k_ln_apply_z(LnView L, const double *__restrict__ r, double *__restrict__ z) {
  const double alpha = exp((double)*L.loga);
  for (int64_t i = gthread(); i < L.n; i += nthread()) z[i] = ln_node_z<double>(L, r, alpha, i);
}
// z = alpha pb + correction: the preconditioner on a block base (pb = B^-1 r precomputed)
__global__ void __launch_bounds__(kT) k_ln_apply_zb(LnView L, const double *__restrict__ pb, double *__restrict__ z) {
  const double alpha = exp((double)*L.loga);
  for (int64_t i = gthread(); i < L.n; i += nthread()) z[i] = alpha * pb[i] + (double)ln_node_corr(L, i);
}
__global__ void __launch_bounds__(kT) k_ln_fill(int64_t n, double v, double *__restrict__ x) {
  for (int64_t i = gthread(); i < n; i += nthread()) x[i] = v;
}

// sum_i g_i (r_i / a_ii): the derivative of g^T z w.r.t. alpha, per pair
__global__ void __launch_bounds__(kT) k_ln_dot3_part(int64_t n, const double *__restrict__ g,
                                                     const double *__restrict__ dinv, const double *__restrict__ r,
                                                     double *__restrict__ part) {
  __shared__ double sh[kT / 32];
  double s = 0.0;
  for (int64_t i = gthread(); i < n; i += nthread()) s += g[i] * dinv[i] * r[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kT / 32; w++) t += sh[w];
    part[blockIdx.x] = t;
  }
}
// grad[a] = alpha * sum over pairs (terms[j] filled by k_ln_dot_fin)
__global__ void k_ln_alpha_grad(int P, const double *__restrict__ terms, const float *__restrict__ params, int64_t oa,
                                float *__restrict__ grad) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double t = 0.0;
  for (int j = 0; j < P; j++) t += terms[j];
  grad[oa] = (float)(exp((double)params[oa]) * t);
}
__global__ void __launch_bounds__(kT) k_ln_masked_diff(int64_t n, const double *__restrict__ mask,
                                                       const double *__restrict__ a, const double *__restrict__ b,
                                                       double *__restrict__ w) {
  for (int64_t i = gthread(); i < n; i += nthread()) w[i] = mask[i] * (a[i] - (b ? b[i] : 0.0));
}
// deterministic dot product: per-CTA partials, then one CTA sums them in order
__global__ void __launch_bounds__(kT) k_ln_dot_part(int64_t n, const double *__restrict__ x,
                                                    const double *__restrict__ y, double *__restrict__ part) {
  __shared__ double sh[kT / 32];
  double s = 0.0;
  for (int64_t i = gthread(); i < n; i += nthread()) s += x[i] * y[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kT / 32; w++) t += sh[w];
    part[blockIdx.x] = t;
  }
}
__global__ void k_ln_dot_fin(int nb, const double *__restrict__ part, double *__restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < nb; i++) t += part[i];
    *out = t;
  }
}
// g = 2 / (P e^T A e) * m .* (A w); loss slot = w^T A w / e^T A e
__global__ void __launch_bounds__(kT) k_ln_pair_grad(int64_t n, int P, const double *__restrict__ mask,
                                                     const double *__restrict__ aw, const double *__restrict__ sc,
                                                     double *__restrict__ g) {
  const double s = sc[0] > 0.0 ? 2.0 / ((double)P * sc[0]) : 0.0;  // a pair with no error contributes nothing
  for (int64_t i = gthread(); i < n; i += nthread()) g[i] = s * mask[i] * aw[i];
}
__global__ void __launch_bounds__(kT) k_ln_dsq(int64_t n, const double *__restrict__ dinv,
                                               const double *__restrict__ mask, double *__restrict__ dsq,
                                               float *__restrict__ mdsq, float *__restrict__ dinv32) {
  for (int64_t i = gthread(); i < n; i += nthread()) {
    const double d = dinv[i];
    const double s = d > 0.0 ? sqrt(d) : 0.0;
    dsq[i] = s;
    mdsq[i] = (float)(mask[i] * s);
    dinv32[i] = (float)d;
  }
}
__global__ void __launch_bounds__(kT) k_ln_axpy(int64_t n, double a, const double *__restrict__ x,
                                                const double *__restrict__ y, double *__restrict__ z) {
  for (int64_t i = gthread(); i < n; i += nthread()) z[i] = y[i] + a * x[i];
}

// ---------------------------------------------------------------- host side
uint64_t splitmix(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double normal01(uint64_t &s) {  // Box-Muller on two 53-bit uniforms
  const double u1 = ((splitmix(s) >> 11) + 1.0) * (1.0 / 9007199254740993.0);
  const double u2 = (splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

int sides_of(int type) { return type == GPZ_EL_HEX ? 27 : (type == GPZ_EL_QUAD ? 9 : 3); }

// dest[k][0 .. NS): the equations of volume element k, its connects in side order, each connect's block
__global__ void k_ln_dest(int64_t E, int ns, int NS, const int32_t *__restrict__ ec, const int64_t *__restrict__ bpos,
                          const int32_t *__restrict__ bsize, int32_t *__restrict__ dest, int *__restrict__ err) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= E) return;
  int32_t *d = dest + k * NS;
  int cnt = 0;
  for (int s = 0; s < ns; s++) {
    const int32_t cn = ec[k * ns + s];
    const int n = bsize[cn];
    if (cnt + n > NS) {
      atomicOr(err, 1 << 21);
      return;
    }
    for (int j = 0; j < n; j++) d[cnt + j] = (int32_t)(bpos[cn] + j);
    cnt += n;
  }
}

void setup_mesh(Ctx &c, int R) {
  Learned &L = c.ln;
  GPZ_REQUIRE(c.have_mesh, GPZ_E_NOT_READY, "no mesh");
  GPZ_REQUIRE(!c.flt.active, GPZ_E_INVALID, "learned preconditioner: not available under an equation filter");
  GPZ_REQUIRE(R >= 1 && R <= kMaxR, GPZ_E_INVALID, "rank must be in 1..8");
  L.h_vel.clear();
  int vtype = -1;
  for (int64_t e = 0; e < c.nel; e++)
    if (c.h_el_mat[e] >= 0) {
      if (vtype < 0) vtype = c.h_el_type[e];
      GPZ_REQUIRE(c.h_el_type[e] == vtype, GPZ_E_UNSUPPORTED_ELEMENT,
                  "learned preconditioner: all volume elements must have one type");
      L.h_vel.push_back(e);
    }
  GPZ_REQUIRE(!L.h_vel.empty(), GPZ_E_INVALID, "no volume elements");
  const int ns = sides_of(vtype);
  const int64_t E = (int64_t)L.h_vel.size();
  // equations per element (every volume element the same count), the elements' connects
  int NS = 0;
  for (int s = 0; s < ns; s++) NS += c.h_block_size[c.h_el_conn[L.h_vel[0] * 27 + s]];
  std::vector<int32_t> ec((size_t)E * ns);
  std::atomic<int> uneven{0};
  host_parallel(E, [&](int64_t k0, int64_t k1) {
    for (int64_t k = k0; k < k1; k++) {
      const int64_t e = L.h_vel[k];
      int cnt = 0;
      for (int s = 0; s < ns; s++) {
        const int64_t cn = c.h_el_conn[e * 27 + s];
        ec[k * ns + s] = (int32_t)cn;
        cnt += c.h_block_size[cn];
      }
      if (cnt != NS) uneven.store(1, std::memory_order_relaxed);
    }
  });
  GPZ_REQUIRE(!uneven.load(), GPZ_E_UNSUPPORTED_ELEMENT,
              "learned preconditioner: all volume elements must have the same number of equations");
  GPZ_REQUIRE(NS >= 1 && NS <= kMaxNS && NS * R * (kH + 1) * 4 <= 200 * 1024, GPZ_E_UNSUPPORTED_ELEMENT,
              "learned preconditioner: too many equations per element");
  GPZ_REQUIRE(E * NS * R < (int64_t)INT32_MAX, GPZ_E_INVALID, "learned preconditioner: mesh too large");
  // penalty-Dirichlet equations
  std::vector<double> mask(c.neq, 1.0);
  for (int64_t e = 0; e < c.nel; e++) {
    const int m = c.h_el_mat[e];
    if (m >= 0) continue;
    const int b = -m - 1;
    if (b < 0 || b >= (int)c.bcs.size() || c.bcs[b].type != 0) continue;
    const int nsb = sides_of(c.h_el_type[e]);
    for (int s = 0; s < nsb; s++) {
      const int64_t cn = c.h_el_conn[e * 27 + s];
      for (int j = 0; j < c.h_block_size[cn]; j++) mask[c.h_block_pos[cn] + j] = 0.0;
    }
  }
  // connect -> volume elements, each connect's elements in increasing order (counted and filled on the host
  // threads, then each short list sorted: the same lists as one pass over the elements)
  std::vector<int64_t> ce_ptr(c.nconnects + 1, 0);
  host_parallel(E * ns, [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; i++) __atomic_fetch_add(&ce_ptr[ec[i] + 1], (int64_t)1, __ATOMIC_RELAXED);
  });
  for (int64_t i = 0; i < c.nconnects; i++) ce_ptr[i + 1] += ce_ptr[i];
  std::vector<int32_t> ce_idx(ce_ptr.back());
  {
    std::vector<int64_t> f(ce_ptr.begin(), ce_ptr.end() - 1);
    host_parallel(E, [&](int64_t k0, int64_t k1) {
      for (int64_t k = k0; k < k1; k++)
        for (int s = 0; s < ns; s++)
          ce_idx[__atomic_fetch_add(&f[ec[k * ns + s]], (int64_t)1, __ATOMIC_RELAXED)] = (int32_t)k;
    });
    host_parallel(c.nconnects, [&](int64_t i0, int64_t i1) {
      for (int64_t i = i0; i < i1; i++) std::sort(ce_idx.begin() + ce_ptr[i], ce_idx.begin() + ce_ptr[i + 1]);
    });
  }
  cudaStream_t st = c.stream;
  L.ec.upload(ec.data(), ec.size(), st);
  L.ce_ptr.upload(ce_ptr.data(), ce_ptr.size(), st);
  L.ce_idx.upload(ce_idx.data(), std::max<size_t>(ce_idx.size(), 1), st);
  // each element's equations, in TPZElementMatrix::ComputeDestinationIndices order, built on the device
  L.dest.alloc((size_t)E * NS);
  k_ln_dest<<<grid_for(E, 256), 256, 0, st>>>(E, ns, NS, L.ec.p, c.d_block_pos.p, c.d_block_size.p, L.dest.p,
                                               c.d_err.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  L.have_ne = false;
  L.mask.upload(mask.data(), mask.size(), st);
  L.dsq.alloc(std::max<int64_t>(c.neq, 1));
  L.mdsq.alloc(std::max<int64_t>(c.neq, 1));
  L.feat.alloc(E);
  L.F.alloc((size_t)E * NS * R);
  L.t.alloc((size_t)E * R);
  L.act.alloc((size_t)E * kH * A_NE + (size_t)c.nconnects * kH);
  L.back.alloc((size_t)E * kH * B_NE + (size_t)c.nconnects * kH + (size_t)E * NS * R);
  const Offs o = offs_of(NS * R);
  const int64_t maxout = std::max<int64_t>((int64_t)NS * R * (kH + 1), kH * (2 * kH + 1));
  L.partial.alloc((size_t)kMaxSeg * maxout);
  L.red.alloc(kRedBlocks);
  L.R = R;
  L.NS = NS;
  L.nsides = ns;
  L.E = E;
  L.nconn = c.nconnects;
  L.nparams = o.total;
  L.ready = true;
  GPZ_CUDA_TRY(cudaStreamSynchronize(st));
  check_device_flag(c, "learned element equations");
  ensure_node_incidence(c);
}

void init_params(Ctx &c, uint64_t seed) {
  Learned &L = c.ln;
  const Offs o = offs_of(L.NS * L.R);
  std::vector<float> p(o.total, 0.f);
  uint64_t s = seed * 0x2545F4914F6CDD1Dull + 1;
  for (int i = 0; i < kH; i++) p[o.W0 + i] = (float)(0.5 * normal01(s));
  const double sw = 1.0 / std::sqrt(2.0 * kH);
  for (int i = 0; i < kH * 2 * kH; i++) p[o.W1 + i] = (float)(sw * normal01(s));
  for (int i = 0; i < kH * 2 * kH; i++) p[o.W2 + i] = (float)(sw * normal01(s));
  for (int64_t i = 0; i < (int64_t)L.NS * L.R * kH; i++) p[o.Wo + i] = (float)(0.01 * normal01(s));
  L.params.upload(p.data(), p.size(), c.stream);
  L.grad.alloc(o.total);
  L.m1.alloc(o.total);
  L.m2.alloc(o.total);
  L.m1.zero(c.stream);
  L.m2.zero(c.stream);
  L.adam_t = 0;
  L.have_params = true;
}

// the solves' copy of the factors, rounded to nearest bfloat16
__global__ void __launch_bounds__(kT) k_ln_to_bf16(int64_t n, const float *__restrict__ F, uint16_t *__restrict__ h) {
  for (int64_t i = gthread(); i < n; i += nthread()) h[i] = __bfloat16_as_ushort(__float2bfloat16_rn(F[i]));
}

// the same rows in incidence order: row k = row ne_idx[k] of the element-ordered copy
__global__ void __launch_bounds__(kT) k_ln_rows_by_incidence(int64_t n, int R, const int32_t *__restrict__ ne_idx,
                                                             const uint16_t *__restrict__ h, uint16_t *__restrict__ hne) {
  for (int64_t k = gthread(); k < n * R; k += nthread()) hne[k] = h[(int64_t)ne_idx[k / R] * R + k % R];
}

LnView view_of(Ctx &c) {
  Learned &L = c.ln;
  LnView v;
  v.F = L.F.p;
  v.F16 = L.F16.p;
  v.F16ne = L.F16ne.p;
  v.dest = L.dest.p;
  v.ne_ptr = L.ne_ptr.p;
  v.ne_idx = L.ne_idx.p;
  v.mdsq = L.mdsq.p;
  v.dinv = c.d_dinv.p;
  v.dinv32 = L.dinv32.p;
  v.loga = L.params.p + offs_of(L.NS * L.R).a;
  v.t = L.t.p;
  v.E = L.E;
  v.n = c.neq;
  v.NS = L.NS;
  v.R = L.R;
  return v;
}

float *act(Ctx &c, int plane) { return c.ln.act.p + (size_t)plane * c.ln.E * kH; }
float *nm_buf(Ctx &c) { return c.ln.act.p + (size_t)A_NE * c.ln.E * kH; }
float *bk(Ctx &c, int plane) { return c.ln.back.p + (size_t)plane * c.ln.E * kH; }
float *dnm_buf(Ctx &c) { return c.ln.back.p + (size_t)B_NE * c.ln.E * kH; }
float *dF_buf(Ctx &c) { return dnm_buf(c) + (size_t)c.ln.nconn * kH; }

void refresh_features(Ctx &c) {
  Learned &L = c.ln;
  std::vector<double> coef(c.nel, 1.0);
  if (c.d_coef.p && c.d_coef.n >= (size_t)c.nel)
    GPZ_CUDA_TRY(cudaMemcpyAsync(coef.data(), c.d_coef.p, c.nel * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
  std::vector<float> f(L.E);
  for (int64_t k = 0; k < L.E; k++) {
    const double v = coef[L.h_vel[k]];
    f[k] = v > 0.0 ? (float)std::log(v) : 0.f;
  }
  L.feat.upload(f.data(), f.size(), c.stream);
}

void forward(Ctx &c) {
  Learned &L = c.ln;
  const Offs o = offs_of(L.NS * L.R);
  const float *P = L.params.p;
  cudaStream_t s = c.stream;
  const int ge = grid_w(L.E), gc = grid_w(L.nconn);
  k_ln_h0<<<grid_t(L.E * kH), kT, 0, s>>>(L.E, L.feat.p, P, o.W0, o.b0, act(c, A_H0));
  k_ln_node_gather<<<gc, kT, 0, s>>>(L.nconn, L.ce_ptr.p, L.ce_idx.p, act(c, A_H0), nm_buf(c), 1, 1.f);
  k_ln_layer<<<ge, kT, 0, s>>>(L.E, L.nsides, L.ec.p, act(c, A_H0), nm_buf(c), P + o.W1, P + o.b1, act(c, A_NB1),
                               act(c, A_Y1), act(c, A_H1));
  k_ln_node_gather<<<gc, kT, 0, s>>>(L.nconn, L.ce_ptr.p, L.ce_idx.p, act(c, A_H1), nm_buf(c), 1, 1.f);
  k_ln_layer<<<ge, kT, 0, s>>>(L.E, L.nsides, L.ec.p, act(c, A_H1), nm_buf(c), P + o.W2, P + o.b2, act(c, A_NB2),
                               act(c, A_Y2), act(c, A_H2));
  const int NR = L.NS * L.R;
  const size_t smem = (size_t)NR * (kH + 1) * sizeof(float);
  GPZ_CUDA_TRY(cudaFuncSetAttribute(k_ln_out, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_ln_out<<<ge, kT, smem, s>>>(L.E, NR, act(c, A_H2), P + o.Wo, P + o.bo, L.F.p);
  c.launches += 6;
  GPZ_CUDA_TRY(cudaGetLastError());
}

void outer(Ctx &c, int na, int lda, const float *A, int n1, int ld1, const float *B1, int n2, int ld2, const float *B2,
           int64_t oW, int64_t ob) {
  Learned &L = c.ln;
  const int64_t seg = std::max<int64_t>(256, (L.E + kMaxSeg - 1) / kMaxSeg);
  const int S = (int)((L.E + seg - 1) / seg);
  const int64_t nout = (int64_t)na * (n1 + n2 + 1);
  dim3 g((unsigned)((nout + kT - 1) / kT), (unsigned)S);
  k_ln_outer<<<g, kT, 0, c.stream>>>(L.E, seg, na, lda, A, n1, ld1, B1, n2, ld2, B2, L.partial.p);
  k_ln_outer_reduce<<<(unsigned)((nout + kT - 1) / kT), kT, 0, c.stream>>>(S, na, n1 + n2, L.partial.p, L.grad.p, oW,
                                                                          ob);
  c.launches += 2;
}

// gradient of the loss w.r.t. the parameters, given pg = dL/dz for every pair
void backward(Ctx &c) {
  Learned &L = c.ln;
  const Offs o = offs_of(L.NS * L.R);
  const float *P = L.params.p;
  cudaStream_t s = c.stream;
  const int ge = grid_w(L.E), gc = grid_w(L.nconn);
  const int NR = L.NS * L.R;
  k_ln_dF<<<ge, kT, 0, s>>>(L.E, L.NS, L.R, L.dest.p, L.F.p, L.mask.p, L.dsq.p, L.npairs, c.neq, L.pr.p, L.pg.p,
                            dF_buf(c));
  const size_t smem = (size_t)NR * (kH + 1) * sizeof(float);
  GPZ_CUDA_TRY(cudaFuncSetAttribute(k_ln_out_back, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_ln_out_back<<<ge, kT, smem, s>>>(L.E, NR, dF_buf(c), P + o.Wo, bk(c, B_DH2));
  outer(c, NR, NR, dF_buf(c), kH, kH, act(c, A_H2), 0, 0, nullptr, o.Wo, o.bo);
  // layer 2: h2 = h1 + tanh(W2 [h1; nb2] + b2)
  k_ln_layer_back<<<ge, kT, 0, s>>>(L.E, bk(c, B_DH2), act(c, A_Y2), P + o.W2, bk(c, B_DPRE), bk(c, B_DH),
                                    bk(c, B_DNB));
  outer(c, kH, kH, bk(c, B_DPRE), kH, kH, act(c, A_H1), kH, kH, act(c, A_NB2), o.W2, o.b2);
  k_ln_node_gather<<<gc, kT, 0, s>>>(L.nconn, L.ce_ptr.p, L.ce_idx.p, bk(c, B_DNB), dnm_buf(c), 0,
                                     1.f / (float)L.nsides);
  k_ln_elem_acc<<<ge, kT, 0, s>>>(L.E, L.nsides, L.ec.p, L.ce_ptr.p, dnm_buf(c), bk(c, B_DH));
  // layer 1: h1 = h0 + tanh(W1 [h0; nb1] + b1); dh (grad of h1) -> dh2 plane reused for grad of h0
  k_ln_layer_back<<<ge, kT, 0, s>>>(L.E, bk(c, B_DH), act(c, A_Y1), P + o.W1, bk(c, B_DPRE), bk(c, B_DH2),
                                    bk(c, B_DNB));
  outer(c, kH, kH, bk(c, B_DPRE), kH, kH, act(c, A_H0), kH, kH, act(c, A_NB1), o.W1, o.b1);
  k_ln_node_gather<<<gc, kT, 0, s>>>(L.nconn, L.ce_ptr.p, L.ce_idx.p, bk(c, B_DNB), dnm_buf(c), 0,
                                     1.f / (float)L.nsides);
  k_ln_elem_acc<<<ge, kT, 0, s>>>(L.E, L.nsides, L.ec.p, L.ce_ptr.p, dnm_buf(c), bk(c, B_DH2));
  // layer 0: h0 = tanh(W0 x + b0)
  k_ln_h0_back<<<grid_t(L.E * kH), kT, 0, s>>>(L.E, bk(c, B_DH2), act(c, A_H0), bk(c, B_DPRE));
  outer(c, kH, kH, bk(c, B_DPRE), 1, 1, L.feat.p, 0, 0, nullptr, o.W0, o.b0);
  c.launches += 10;
  GPZ_CUDA_TRY(cudaGetLastError());
}

void dot(Ctx &c, const double *x, const double *y, double *out) {
  k_ln_dot_part<<<kRedBlocks, kT, 0, c.stream>>>(c.neq, x, y, c.ln.red.p);
  k_ln_dot_fin<<<1, 32, 0, c.stream>>>(kRedBlocks, c.ln.red.p, out);
  c.launches += 2;
}

void apply_M(Ctx &c, const double *r, double *z) {
  LnView v = view_of(c);
  k_ln_apply_t<<<grid_t(c.ln.E * c.ln.R), kT, 0, c.stream>>>(v, r);
  k_ln_apply_z<<<grid_t(c.neq), kT, 0, c.stream>>>(v, r, z);
  c.launches += 2;
}

// e^T A e of every masked pair error
void pair_norms(Ctx &c) {
  Learned &L = c.ln;
  const int64_t n = c.neq;
  for (int j = 0; j < L.npairs; j++) {
    double *w = L.pw.p + (size_t)j * n, *aw = L.paw.p + (size_t)j * n;
    k_ln_masked_diff<<<grid_t(n), kT, 0, c.stream>>>(n, L.mask.p, L.pe.p + (size_t)j * n, nullptr, w);
    spmv_device(c, w, aw, 1.0, 0.0, nullptr);
    dot(c, w, aw, L.pscal.p + 2 * j);
    c.launches += 2;
  }
}

void alloc_pairs(Ctx &c, int P) {
  Learned &L = c.ln;
  const size_t sz = (size_t)P * std::max<int64_t>(c.neq, 1);
  L.pr.alloc(sz);
  L.pe.alloc(sz);
  L.pz.alloc(sz);
  L.pw.alloc(sz);
  L.paw.alloc(sz);
  L.pg.alloc(sz);
  L.pscal.alloc((size_t)2 * P);
  L.aterm.alloc(P);
  L.npairs = P;
}

// Training on a block base: pb_j = B^-1 r_j for every pair, and with the
// two-level base the coarse part P Ac^-1 P^T r_j taken off the target e_j
// (the correction is trained for what the base leaves); the pair norms follow
// the new targets.
void prepare_base(Ctx &c) {
  Learned &L = c.ln;
  if (L.base == 0 || L.npairs == 0) return;
  const int64_t n = c.neq;
  L.pb.alloc((size_t)L.npairs * n);
  L.ones.alloc(n);
  k_ln_fill<<<grid_t(n), kT, 0, c.stream>>>(n, 1.0, L.ones.p);
  c.launches++;
  for (int j = 0; j < L.npairs; j++) {
    const double *r = L.pr.p + (size_t)j * n;
    base_block_apply(c, r, L.pb.p + (size_t)j * n);
    if (L.base == GPZ_PRECOND_TWO_LEVEL) {
      double *tmp = L.pw.p + (size_t)j * n;  // scratch: overwritten by every loss evaluation
      base_coarse_apply(c, r, tmp);
      k_ln_axpy<<<grid_t(n), kT, 0, c.stream>>>(n, -1.0, tmp, L.pe.p + (size_t)j * n, L.pe.p + (size_t)j * n);
      c.launches++;
    }
  }
  GPZ_CUDA_TRY(cudaGetLastError());
}

// mean loss over the pairs; with want_grad the parameter gradient lands in ln.grad
double loss_and_grad(Ctx &c, bool want_grad) {
  Learned &L = c.ln;
  GPZ_REQUIRE(L.npairs > 0, GPZ_E_NOT_READY, "no training pairs");
  forward(c);
  const int64_t n = c.neq;
  for (int j = 0; j < L.npairs; j++) {
    const double *r = L.pr.p + (size_t)j * n;
    double *z = L.pz.p + (size_t)j * n, *w = L.pw.p + (size_t)j * n, *aw = L.paw.p + (size_t)j * n;
    if (L.base) {
      LnView v = view_of(c);
      k_ln_apply_t<<<grid_t(L.E * L.R), kT, 0, c.stream>>>(v, r);
      k_ln_apply_zb<<<grid_t(n), kT, 0, c.stream>>>(v, L.pb.p + (size_t)j * n, z);
      c.launches += 2;
    } else {
      apply_M(c, r, z);
    }
    k_ln_masked_diff<<<grid_t(n), kT, 0, c.stream>>>(n, L.mask.p, z, L.pe.p + (size_t)j * n, w);
    spmv_device(c, w, aw, 1.0, 0.0, nullptr);
    dot(c, w, aw, L.pscal.p + 2 * j + 1);
    if (want_grad)
      k_ln_pair_grad<<<grid_t(n), kT, 0, c.stream>>>(n, L.npairs, L.mask.p, aw, L.pscal.p + 2 * j,
                                                     L.pg.p + (size_t)j * n);
    c.launches += 3;
  }
  if (want_grad) {
    backward(c);
    const Offs o = offs_of(L.NS * L.R);
    for (int j = 0; j < L.npairs; j++) {
      // d(g^T z)/d(log alpha) = alpha g^T (base r): base r = D^-1 r, or the block base pb
      k_ln_dot3_part<<<kRedBlocks, kT, 0, c.stream>>>(n, L.pg.p + (size_t)j * n, L.base ? L.ones.p : c.d_dinv.p,
                                                      L.base ? L.pb.p + (size_t)j * n : L.pr.p + (size_t)j * n,
                                                      L.red.p);
      k_ln_dot_fin<<<1, 32, 0, c.stream>>>(kRedBlocks, L.red.p, L.aterm.p + j);
    }
    k_ln_alpha_grad<<<1, 32, 0, c.stream>>>(L.npairs, L.aterm.p, L.params.p, o.a, L.grad.p);
    c.launches += 2 * L.npairs + 1;
  }
  std::vector<double> sc((size_t)2 * L.npairs);
  GPZ_CUDA_TRY(cudaMemcpyAsync(sc.data(), L.pscal.p, sc.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
  double loss = 0.0;
  for (int j = 0; j < L.npairs; j++)
    if (sc[2 * j] > 0.0) loss += sc[2 * j + 1] / sc[2 * j];
  return loss / L.npairs;
}

}  // namespace

// equation -> (element, local) lists of the gather form of the correction,
// built on the device from the connect -> element lists: the m elements of a
// connect's list (in element order) give each of its equations m incidences,
// in the same order.
namespace {
__global__ void k_ln_ne_count(int64_t nconn, const int64_t *__restrict__ ce_ptr, const int32_t *__restrict__ bsize,
                              int64_t *__restrict__ cnt) {
  const int64_t cn = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cn < nconn) cnt[cn] = (ce_ptr[cn + 1] - ce_ptr[cn]) * (int64_t)bsize[cn];
}
__global__ void k_ln_ne_fill(int64_t nconn, int ns, int NS, const int64_t *__restrict__ ce_ptr,
                             const int32_t *__restrict__ ce_idx, const int32_t *__restrict__ ec,
                             const int64_t *__restrict__ bpos, const int32_t *__restrict__ bsize,
                             const int64_t *__restrict__ base, int64_t *__restrict__ ne_ptr,
                             int32_t *__restrict__ ne_idx, int *__restrict__ err) {
  const int64_t cn = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cn >= nconn) return;
  const int64_t m = ce_ptr[cn + 1] - ce_ptr[cn];
  const int bs = bsize[cn];
  for (int j = 0; j < bs; j++) ne_ptr[bpos[cn] + j] = base[cn] + j * m;
  for (int64_t r = 0; r < m; r++) {
    const int32_t k = ce_idx[ce_ptr[cn] + r];
    int off = 0, s = 0;
    for (; s < ns; s++) {
      const int32_t cs = ec[(int64_t)k * ns + s];
      if (cs == cn) break;
      off += bsize[cs];
    }
    if (s == ns || off + bs > NS) {
      atomicOr(err, 64);
      continue;
    }
    for (int j = 0; j < bs; j++) ne_idx[base[cn] + j * m + r] = (int32_t)((int64_t)k * NS + off + j);
  }
}
}  // namespace

void ensure_node_incidence(Ctx &c) {
  Learned &L = c.ln;
  if (L.have_ne) return;
  cudaStream_t st = c.stream;
  DBuf<int64_t> cnt, base;
  cnt.alloc(c.nconnects + 1);
  cnt.zero(st);
  base.alloc(c.nconnects + 1);
  k_ln_ne_count<<<grid_for(c.nconnects, 256), 256, 0, st>>>(c.nconnects, L.ce_ptr.p, c.d_block_size.p, cnt.p);
  exclusive_scan_i64(cnt.p, base.p, c.nconnects + 1, st, c);
  L.ne_ptr.alloc(c.neq + 1);
  L.ne_idx.alloc(std::max<int64_t>(L.E * L.NS, 1));
  k_ln_ne_fill<<<grid_for(c.nconnects, 256), 256, 0, st>>>(c.nconnects, L.nsides, L.NS, L.ce_ptr.p, L.ce_idx.p,
                                                           L.ec.p, c.d_block_pos.p, c.d_block_size.p, base.p,
                                                           L.ne_ptr.p, L.ne_idx.p, c.d_err.p);
  c.launches += 2;
  GPZ_CUDA_TRY(cudaGetLastError());
  // ne_ptr[neq] = the total number of incidences
  GPZ_CUDA_TRY(cudaMemcpyAsync(L.ne_ptr.p + c.neq, base.p + c.nconnects, sizeof(int64_t), cudaMemcpyDeviceToDevice, st));
  GPZ_CUDA_TRY(cudaStreamSynchronize(st));
  check_device_flag(c, "learned node incidence");
  L.have_ne = true;
}

// S = diag^-1/2, m S and the FP32 1 / a_ii of the assembled matrix
void scaling(Ctx &c) {
  Learned &L = c.ln;
  L.dinv32.alloc(std::max<int64_t>(c.neq, 1));
  k_ln_dsq<<<grid_t(c.neq), kT, 0, c.stream>>>(c.neq, c.d_dinv.p, L.mask.p, L.dsq.p, L.mdsq.p, L.dinv32.p);
  c.launches++;
}

void learned_prepare(Ctx &c) {
  Learned &L = c.ln;
  GPZ_REQUIRE(L.ready && L.have_params, GPZ_E_NOT_READY, "learned preconditioner not initialised");
  GPZ_REQUIRE(c.have_matrix, GPZ_E_NOT_READY, "not assembled");
  refresh_features(c);
  scaling(c);
  forward(c);
  const int64_t nf = L.E * L.NS * L.R;
  L.F16.alloc(std::max<int64_t>(nf, 1));
  k_ln_to_bf16<<<grid_t(nf), kT, 0, c.stream>>>(nf, L.F.p, L.F16.p);
  ensure_node_incidence(c);
  L.F16ne.alloc(std::max<int64_t>(nf, 1));
  k_ln_rows_by_incidence<<<grid_t(nf), kT, 0, c.stream>>>(L.E * L.NS, L.R, L.ne_idx.p, L.F16.p, L.F16ne.p);
  c.launches += 2;
  GPZ_CUDA_TRY(cudaGetLastError());
}

LnView learned_view(Ctx &c) { return view_of(c); }

}  // namespace gpz

using gpz::Ctx;

namespace {
template <class F>
int guarded_ln(gpz_ctx *ctx, F &&f) {
  if (!ctx) return GPZ_E_INVALID;
  Ctx &c = ctx->c;
  try {
    GPZ_CUDA_TRY(cudaSetDevice(c.device));
    GPZ_REQUIRE(!c.flt.active, GPZ_E_INVALID, "learned preconditioner: not available under an equation filter");
    return f(c);
  } catch (const gpz::Error &e) {
    c.last_error = e.msg;
    if (e.code == GPZ_E_CUDA || e.code == GPZ_E_NOMEM) cudaGetLastError();
    return e.code;
  } catch (const std::bad_alloc &) {
    c.last_error = "host allocation failed";
    return GPZ_E_NOMEM;
  } catch (...) {
    c.last_error = "unexpected host exception";
    return GPZ_E_INVALID;
  }
}
}  // namespace

extern "C" {

int gpz_learned_init(gpz_ctx *ctx, int rank, uint64_t seed) {
  return guarded_ln(ctx, [&](Ctx &c) {
    gpz::setup_mesh(c, rank);
    gpz::init_params(c, seed);
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return GPZ_OK;
  });
}

int gpz_learned_num_params(gpz_ctx *ctx, int64_t *n) {
  return guarded_ln(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(n && c.ln.ready, GPZ_E_NOT_READY, "learned preconditioner not initialised");
    *n = c.ln.nparams;
    return GPZ_OK;
  });
}

int gpz_learned_get_params(gpz_ctx *ctx, float *out, int64_t n) {
  return guarded_ln(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.ln.have_params, GPZ_E_NOT_READY, "learned preconditioner not initialised");
    GPZ_REQUIRE(out && n == c.ln.nparams, GPZ_E_INVALID, "parameter count");
    GPZ_CUDA_TRY(cudaMemcpyAsync(out, c.ln.params.p, n * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return GPZ_OK;
  });
}

int gpz_learned_set_params(gpz_ctx *ctx, const float *in, int64_t n) {
  return guarded_ln(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.ln.have_params, GPZ_E_NOT_READY, "learned preconditioner not initialised");
    GPZ_REQUIRE(in && n == c.ln.nparams, GPZ_E_INVALID, "parameter count");
    GPZ_CUDA_TRY(cudaMemcpyAsync(c.ln.params.p, in, n * sizeof(float), cudaMemcpyHostToDevice, c.stream));
    c.ln.m1.zero(c.stream);
    c.ln.m2.zero(c.stream);
    c.ln.adam_t = 0;
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return GPZ_OK;
  });
}

int gpz_learned_collect(gpz_ctx *ctx, int npairs, double tol, int64_t max_iter, int64_t *cg_iterations) {
  return guarded_ln(ctx, [&](Ctx &c) {
    gpz::Learned &L = c.ln;
    GPZ_REQUIRE(L.ready, GPZ_E_NOT_READY, "learned preconditioner not initialised");
    gpz::ensure_node_incidence(c);
    GPZ_REQUIRE(c.have_matrix, GPZ_E_NOT_READY, "not assembled");
    GPZ_REQUIRE(npairs >= 1 && npairs <= 256 && tol > 0 && max_iter > 0, GPZ_E_INVALID, "arguments");
    gpz::alloc_pairs(c, npairs);
    int64_t its = 0;
    // residuals into pr, iterates into pw, the converged solution into pz[0]
    const int got = gpz::collect_cg_pairs(c, npairs, tol, max_iter, L.pr.p, L.pw.p, L.pz.p, &its);
    GPZ_REQUIRE(got >= 1, GPZ_E_INVALID, "the Jacobi-PCG run gave no iterates to sample");
    L.npairs = got;
    for (int j = 0; j < got; j++)  // e_j = x* - x_j
      gpz::k_ln_axpy<<<gpz::grid_t(c.neq), gpz::kT, 0, c.stream>>>(c.neq, -1.0, L.pw.p + (size_t)j * c.neq, L.pz.p,
                                                                    L.pe.p + (size_t)j * c.neq);
    GPZ_CUDA_TRY(cudaGetLastError());
    gpz::refresh_features(c);
    gpz::scaling(c);
    gpz::prepare_base(c);
    gpz::pair_norms(c);
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    if (cg_iterations) *cg_iterations = its;
    return GPZ_OK;
  });
}

int gpz_learned_set_base(gpz_ctx *ctx, int precond) {
  return guarded_ln(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.ln.ready, GPZ_E_NOT_READY, "learned preconditioner not initialised");
    GPZ_REQUIRE(precond == 0 || precond == GPZ_PRECOND_JACOBI || precond == GPZ_PRECOND_BLOCK_JACOBI ||
                    precond == GPZ_PRECOND_TWO_LEVEL,
                GPZ_E_INVALID, "base preconditioner");
    GPZ_REQUIRE(precond <= GPZ_PRECOND_JACOBI || (c.nstate == 3 && !c.flt.active), GPZ_E_INVALID,
                "a block base needs 3 equations per connect");
    c.ln.base = precond == GPZ_PRECOND_JACOBI ? 0 : precond;
    c.ln.npairs = 0;  // pairs are prepared for one base: collect or set them again
    return GPZ_OK;
  });
}

int gpz_learned_set_pairs(gpz_ctx *ctx, int npairs, const double *r, const double *e) {
  return guarded_ln(ctx, [&](Ctx &c) {
    gpz::Learned &L = c.ln;
    GPZ_REQUIRE(L.ready, GPZ_E_NOT_READY, "learned preconditioner not initialised");
    gpz::ensure_node_incidence(c);
    GPZ_REQUIRE(c.have_matrix, GPZ_E_NOT_READY, "not assembled");
    GPZ_REQUIRE(npairs >= 1 && npairs <= 256 && r && e, GPZ_E_INVALID, "arguments");
    gpz::alloc_pairs(c, npairs);
    const size_t bytes = (size_t)npairs * c.neq * sizeof(double);
    GPZ_CUDA_TRY(cudaMemcpyAsync(L.pr.p, r, bytes, cudaMemcpyHostToDevice, c.stream));
    GPZ_CUDA_TRY(cudaMemcpyAsync(L.pe.p, e, bytes, cudaMemcpyHostToDevice, c.stream));
    gpz::refresh_features(c);
    gpz::scaling(c);
    gpz::prepare_base(c);
    gpz::pair_norms(c);
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return GPZ_OK;
  });
}

int gpz_learned_loss_grad(gpz_ctx *ctx, double *loss, float *grad, int64_t n) {
  return guarded_ln(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.ln.have_params, GPZ_E_NOT_READY, "learned preconditioner not initialised");
    GPZ_REQUIRE(!grad || n == c.ln.nparams, GPZ_E_INVALID, "parameter count");
    gpz::ensure_node_incidence(c);
    const double l = gpz::loss_and_grad(c, grad != nullptr);
    if (grad) {
      GPZ_CUDA_TRY(cudaMemcpyAsync(grad, c.ln.grad.p, n * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
      GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    }
    if (loss) *loss = l;
    return GPZ_OK;
  });
}

int gpz_learned_train(gpz_ctx *ctx, int steps, double lr, double *loss_first, double *loss_last) {
  return guarded_ln(ctx, [&](Ctx &c) {
    gpz::Learned &L = c.ln;
    GPZ_REQUIRE(L.have_params, GPZ_E_NOT_READY, "learned preconditioner not initialised");
    GPZ_REQUIRE(steps >= 1 && lr > 0, GPZ_E_INVALID, "arguments");
    gpz::ensure_node_incidence(c);
    double l0 = 0, l1 = 0;
    const float b1 = 0.9f, b2 = 0.999f;
    for (int s = 0; s < steps; s++) {
      l1 = gpz::loss_and_grad(c, true);
      if (s == 0) l0 = l1;
      L.adam_t++;
      const float c1 = 1.f - std::pow(b1, (float)L.adam_t), c2 = 1.f - std::pow(b2, (float)L.adam_t);
      gpz::k_ln_adam<<<gpz::grid_t(L.nparams), gpz::kT, 0, c.stream>>>(L.nparams, L.params.p, L.grad.p, L.m1.p,
                                                                        L.m2.p, (float)lr, b1, b2, 1e-8f, c1, c2);
      c.launches++;
    }
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    if (loss_first) *loss_first = l0;
    if (loss_last) *loss_last = l1;
    return GPZ_OK;
  });
}

}  // extern "C"
