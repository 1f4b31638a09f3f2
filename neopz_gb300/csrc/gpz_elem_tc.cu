// Element matrices on the tensor cores: the FP32 copy of the system that the
// mixed solves' inner operator reads, formed from 3xTF32 tcgen05 products.
//
// TPZCompEl::CalcStiff (Mesh/pzinterpolationspace.cpp:403-473) adds, point by
// point, w |J| times the material's bilinear form of the physical gradients
// (TPZMatPoisson::Contribute, Material/Poisson/TPZMatPoisson.cpp:19-43;
// TPZDarcyFlow; TPZElasticity3D::Contribute, Material/Elasticity/TPZElasticity3D.cpp:85-413).
// Every such form is built from the gradient Gram
//   S_ab[i][j] = sum_q w_q |J_q| g_a,i(q) g_b,j(q)    (g_a = J^-T grad phi_a)
// which, for one element, is the product X X^T of
//   X[(i, a)][q] = sqrt(w_q |J_q|) g_a,i(q)           (3 NT rows, nq columns)
// -- one GEMM per element: M 128 (per tile of 128 rows), N = 3 NT padded, K = nq
// padded to 8, as tcgen05.mma.kind::tf32 with the 3xTF32 split (lo.hi + hi.lo +
// hi.hi into one FP32 accumulator in TMEM, about FP32 accuracy).  The epilogue
// forms the material's blocks from the Gram (Poisson / Darcy: k tr S;
// elasticity CODE3: K_st = delta_st ((tr S - S_ss) mu + S_ss (lambda + 2 mu)) +
// (1 - delta_st)(S_ts mu + S_st lambda)) and adds the element's rows into the
// FP32 full CSR through the element's side-pair offset table; elements of one
// colour share no connect, so the read-modify-write needs no atomics.  The
// Jacobians are formed in FP32 from corner coordinates taken relative to the
// element's first corner.
//
// A CTA of 8 warps (16 for the order-3 table) is persistent over the elements
// of one bucket and colour: per element it builds X (hi, lo) in shared memory,
// one thread issues the MMAs and commits to an mbarrier, and the next element's
// connectivity and corners are loaded while they run; all wait (bounded; a
// timeout sets an error flag and ends the CTA after the MMAs in flight are
// waited for), the accumulator is staged through shared memory (over the
// operands, which the MMAs no longer read) and scattered through the element's
// offset table, read into shared memory with its rows' starts.  TMEM columns per CTA: 32 (Q1), 128 (Q2), 512 (Q3, two
// row tiles); the launcher sizes the dynamic shared memory so that the CTAs
// resident on one SM never ask for more than the SM's 512 columns.
#include <algorithm>
#include <cmath>
#include <vector>

#include "gpz_internal.h"
#include "gpz_tc.cuh"

namespace gpz {

namespace {

// threads per CTA: 8 warps, 16 for the order-3 table (one CTA per SM there: 512 TMEM columns, 154 KB of
// operands); warps w, w + 4, ... share TMEM lane quarter w % 4
__host__ __device__ constexpr int et_threads(int nt) { return nt >= 64 ? 512 : 256; }
constexpr int kEtMaxQ = 64;      // integration points (hex 4 x 4 x 4)
constexpr int kErrEtRange = 1 << 19, kErrEtWait = 1 << 20;

struct EtArgs {
  const float *dphi;  // [nq][3][NT] reference gradients of the bucket's table
  const float *w;     // [nq]
  const int *sside, *sk;
  int nq, kp, nsides, nst, kind;
  const double *xyz;
  const int64_t *el_nodes, *el_conn, *bpos;
  const double *coef;
  double E, nu, coef_const, scale;
  const int64_t *ia, *offbase;
  const int32_t *off;
  float *a;
  int64_t nnz, neq;
  int *err;
};

struct EtHp {
  const uint8_t *full, *k;  // active shapes of an hp element: table index, index inside its side
  const int32_t *n;
};

// sizes of the GEMM of a table of NT shapes
__host__ __device__ constexpr int et_rows(int nt) { return 3 * nt; }
__host__ __device__ constexpr int et_mt(int nt) { return (3 * nt + 127) / 128; }           // row tiles
__host__ __device__ constexpr int et_np(int nt) { return (3 * nt + 31) / 32 * 32; }        // N (columns)
__host__ __device__ constexpr int et_cols(int nt) {                                         // TMEM allocation
  return et_mt(nt) * et_np(nt) <= 32 ? 32 : et_mt(nt) * et_np(nt) <= 64 ? 64 : et_mt(nt) * et_np(nt) <= 128 ? 128
         : et_mt(nt) * et_np(nt) <= 256 ? 256 : 512;
}
// dynamic shared memory: [operands hi, lo | staging] region, then the per-point matrices, corners, element rows
__host__ __device__ inline uint32_t et_region(int nt, int kp) {
  const uint32_t ops = 2u * (uint32_t)et_mt(nt) * 128u * (uint32_t)kp * 4u;
  const uint32_t stage = (uint32_t)et_rows(nt) * (uint32_t)(et_np(nt) + 4) * 4u;
  return ((ops > stage ? ops : stage) + 1023u) / 1024u * 1024u;
}
constexpr int kEtSides = 27;  // sides of a hex (the offset table is kEtSides^2)
__host__ __device__ inline uint32_t et_smem(int nt, int kp) {
  return et_region(nt, kp) + kEtMaxQ * 9 * 4 + 24 * 4 + (uint32_t)nt * 8 + 3u * (uint32_t)nt * 4 +
         kEtSides * kEtSides * 4 + 8 + 3u * (uint32_t)nt * 8 + 64;
}

// One element's data, loaded by every thread for its own part: corner coordinate tid (tid < 24, relative to
// corner 0), shape tid's first equation, side, table index and index inside its side (tid < nsh), and (thread 0)
// the offset-table start and the coefficient.  Loaded for the next element while the MMAs of the current one run.
struct EtElem {
  float cx;
  int64_t row, offbase;
  int side, fa, ka, nsh;
  double cf;
};

template <int NT, bool HP>
__device__ __forceinline__ EtElem et_fetch(const EtArgs &P, const EtHp &H, const int64_t *__restrict__ elems,
                                           int64_t ie, int tid) {
  EtElem r{};
  const int64_t e = elems[ie];
  r.nsh = HP ? H.n[ie] : NT;
  if (tid < 24) {
    const int k = tid / 3, j = tid % 3;
    const int64_t node = P.el_nodes[e * 8 + k], node0 = P.el_nodes[e * 8];
    r.cx = (float)(P.xyz[node * 3 + j] - P.xyz[node0 * 3 + j]);
  }
  if (tid < r.nsh) {
    r.fa = HP ? (int)H.full[ie * kMaxShapes + tid] : tid;
    r.ka = HP ? (int)H.k[ie * kMaxShapes + tid] : P.sk[tid];
    r.side = P.sside[r.fa];
    r.row = P.bpos[P.el_conn[e * 27 + r.side]] + (int64_t)r.ka * P.nst;
  }
  if (tid == 0) {
    r.offbase = P.offbase[e];
    r.cf = P.coef ? P.coef[e] : (P.kind == GPZ_MAT_ELAST3D ? P.E : P.coef_const);
  }
  return r;
}

template <int NT, bool HP>
__global__ void __launch_bounds__(et_threads(NT)) k_elem_tc(EtArgs P, EtHp H, const int64_t *__restrict__ elems,
                                                        int64_t n) {
  constexpr int R = et_rows(NT), MT = et_mt(NT), NP = et_np(NT), LD = NP + 4;
  constexpr uint32_t COLS = et_cols(NT);
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_mb;
  __shared__ float s_c[3];
  __shared__ int64_t s_offbase;
  __shared__ int s_nsh;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kp = P.kp;
  const uint32_t opsz = (uint32_t)MT * 128u * (uint32_t)kp * 4u;  // bytes of one operand copy
  float *xh = (float *)sm, *xl = (float *)(sm + opsz);
  float *pst = (float *)sm;  // staged accumulator [R][LD] (over the operands)
  const uint32_t region = et_region(NT, kp);
  float *sMq = (float *)(sm + region);  // [nq][3][3] sqrt(w |J|) Jinv^T per point
  float *sCx = sMq + kEtMaxQ * 9;       // [8][3] corners relative to corner 0
  int64_t *sRow = (int64_t *)(sCx + 24);
  int *sSide = (int *)(sRow + NT), *sIdx = sSide + NT, *sK = sIdx + NT;
  int *sOff = sK + NT;                                                          // [27][27] side-pair offsets
  int64_t *sIa = (int64_t *)(((uintptr_t)(sOff + kEtSides * kEtSides) + 7) & ~(uintptr_t)7);  // [NT][3] row starts
  constexpr int kEtThreads = et_threads(NT);
  static_assert(NT < kEtThreads, "one thread per shape");

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&s_tmem)),
                 "r"(COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&s_mb)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tm = s_tmem;
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NP >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
  const uint32_t sbo = (uint32_t)(kp / 4) * 128u;
  const uint32_t ah = tc_smem(xh), al = tc_smem(xl);
  uint32_t phase = 0;
  bool failed = false;

  EtElem nx{};
  if (blockIdx.x < n) nx = et_fetch<NT, HP>(P, H, elems, blockIdx.x, tid);
  for (int64_t ie = blockIdx.x; ie < n; ie += gridDim.x) {
    if (tid < 24) sCx[tid] = nx.cx;
    if (tid < nx.nsh) {
      sRow[tid] = nx.row;
      sSide[tid] = nx.side;
      sIdx[tid] = nx.fa;
      sK[tid] = nx.ka;
    }
    if (tid == 0) {
      s_nsh = nx.nsh;
      s_offbase = nx.offbase;
      const double cf = nx.cf;
      if (P.kind == GPZ_MAT_ELAST3D) {
        const double nu = P.nu;
        s_c[0] = (float)(cf / (2. + 2. * nu));                          // C1 = mu
        s_c[1] = (float)(cf * nu / (-1. + nu + 2. * nu * nu));          // C2 = -lambda
        s_c[2] = (float)(cf * (nu - 1.) / (-1. + nu + 2. * nu * nu));   // C3 = lambda + 2 mu
      } else {
        s_c[0] = (float)(P.kind == GPZ_MAT_POISSON ? P.scale : cf);
        s_c[1] = s_c[2] = 0.f;
      }
    }
    __syncthreads();
    const int nsh = s_nsh;
    // the element's side-pair offset table and its rows' starts, read once (the scatter looks them up)
    for (int i = tid; i < P.nsides * P.nsides; i += kEtThreads) sOff[i] = P.off[s_offbase + i];
    for (int i = tid; i < nsh * P.nst; i += kEtThreads) {
      const int64_t row = sRow[i / P.nst] + i % P.nst;
      sIa[i] = (row >= 0 && row < P.neq) ? P.ia[row] : -1;
    }
    // per point: the Jacobian from the corner shapes' gradients (the table's first 8 shapes)
    for (int q = tid; q < P.nq; q += kEtThreads) {
      float a[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
      for (int k = 0; k < 8; k++)
        for (int d = 0; d < 3; d++) {
          const float dn = P.dphi[(q * 3 + d) * NT + k];
          for (int j = 0; j < 3; j++) a[j][d] = fmaf(sCx[k * 3 + j], dn, a[j][d]);
        }
      const float det = -a[0][2] * a[1][1] * a[2][0] + a[0][1] * a[1][2] * a[2][0] + a[0][2] * a[1][0] * a[2][1] -
                        a[0][0] * a[1][2] * a[2][1] - a[0][1] * a[1][0] * a[2][2] + a[0][0] * a[1][1] * a[2][2];
      float ji[3][3];
      ji[0][0] = (-a[1][2] * a[2][1] + a[1][1] * a[2][2]) / det;
      ji[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
      ji[0][2] = (-a[0][2] * a[1][1] + a[0][1] * a[1][2]) / det;
      ji[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) / det;
      ji[1][1] = (-a[0][2] * a[2][0] + a[0][0] * a[2][2]) / det;
      ji[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
      ji[2][0] = (-a[1][1] * a[2][0] + a[1][0] * a[2][1]) / det;
      ji[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
      ji[2][2] = (-a[0][1] * a[1][0] + a[0][0] * a[1][1]) / det;
      const float sw = sqrtf(P.w[q] * fabsf(det));
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) sMq[q * 9 + i * 3 + j] = sw * ji[j][i];  // g_i = sum_j Jinv[j][i] dphi_j
    }
    __syncthreads();
    // X (hi, lo) written in the operand's own order (consecutive threads, consecutive words): word
    // idx = 32 core + 4 (r & 7) + (q & 3) with core = (r >> 3)(kp / 4) + (q >> 2); zeros in the padding
    const int kq = kp >> 2, nwords = MT * 128 * kp;
    for (int idx = tid; idx < nwords; idx += kEtThreads) {
      const int core = idx >> 5, within = idx & 31;
      const int r = (core / kq) * 8 + (within >> 2), q = (core % kq) * 4 + (within & 3);
      float v = 0.f;
      if (r < R && q < P.nq) {
        const int i = r / NT, a = r - i * NT;
        if (a < nsh) {
          const float *m = sMq + q * 9 + i * 3;
          const float *d = P.dphi + (size_t)q * 3 * NT + (HP ? sIdx[a] : a);
          v = fmaf(m[0], __ldg(d), fmaf(m[1], __ldg(d + NT), m[2] * __ldg(d + 2 * NT)));
        }
      }
      const float h = tf32_rna(v);
      xh[idx] = h;
      xl[idx] = tf32_rna(v - h);
    }
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
      for (int t = 0; t < MT; t++) {
        const uint32_t at = (uint32_t)t * 16u * sbo;  // rows 128 t ...
#pragma unroll 1
        for (int ks = 0; ks < kp / 8; ks++) {
          const uint32_t ko = (uint32_t)ks * 256u;
          const uint32_t d = tm + (uint32_t)(t * NP);
          tc_mma(d, tc_desc(al + at + ko, sbo), tc_desc(ah + ko, sbo), idesc, ks > 0);
          tc_mma(d, tc_desc(ah + at + ko, sbo), tc_desc(al + ko, sbo), idesc, 1u);
          tc_mma(d, tc_desc(ah + at + ko, sbo), tc_desc(ah + ko, sbo), idesc, 1u);
        }
      }
      tc_commit(&s_mb);
    }
    if (ie + gridDim.x < n) nx = et_fetch<NT, HP>(P, H, elems, ie + gridDim.x, tid);  // in flight during the MMAs
    const bool ok = tc_wait(&s_mb, phase);
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
    // accumulator rows -> staging (float4 stores; the row stride LD = 4 mod 32 words keeps them conflict-free)
    {
      const int quarter = warp & 3, part = warp >> 2, nparts = kEtThreads / 128;
#pragma unroll 1
      for (int t = 0; t < MT; t++) {
        const int r = t * 128 + quarter * 32 + lane;
#pragma unroll 1
        for (int c0 = part * 16; c0 < NP; c0 += 16 * nparts) {
          float v[16];
          tc_ld16(tm + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(t * NP + c0), v);
          if (r < R) {
            float4 *dst = (float4 *)(pst + (size_t)r * LD + c0);
#pragma unroll
            for (int j = 0; j < 4; j++) dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
          }
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    // Rigid translations: the corner shapes sum to one, so their gradients sum to zero and the element matrix
    // annihilates a constant field exactly.  The 3xTF32 products keep about 21 bits, so the Gram's rows for
    // corner 0 are replaced by minus the sum over corners 1..7 (then the columns the same way): a constant
    // field then meets only the FP32 rounding of the entries, as in a rounded FP64 matrix.
    for (int it = tid; it < 3 * R; it += kEtThreads) {
      const int i = it / R, c = it - i * R;
      float sum = 0.f;
#pragma unroll
      for (int k = 1; k < 8; k++) sum += pst[(size_t)(i * NT + k) * LD + c];
      pst[(size_t)(i * NT) * LD + c] = -sum;
    }
    __syncthreads();
    for (int it = tid; it < 3 * R; it += kEtThreads) {
      const int j = it / R, r = it - j * R;
      float sum = 0.f;
#pragma unroll
      for (int k = 1; k < 8; k++) sum += pst[(size_t)r * LD + j * NT + k];
      pst[(size_t)r * LD + j * NT] = -sum;
    }
    __syncthreads();
    // the element's rows into the FP32 CSR: a task is a shape a and 32 shapes b (one per lane)
    const int nbc = (nsh + 31) >> 5, ns = P.nsides;
    const float C1 = s_c[0], C2 = s_c[1], C3 = s_c[2];
    for (int task = warp; task < nsh * nbc; task += kEtThreads / 32) {
      const int a = task / nbc, b = (task - a * nbc) * 32 + lane;
      if (b >= nsh) continue;
      float S[3][3];
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) S[i][j] = pst[(size_t)(i * NT + a) * LD + j * NT + b];
      const float tr = S[0][0] + S[1][1] + S[2][2];
      const int32_t oab = sOff[sSide[a] * ns + sSide[b]];
      if (oab < 0) {
        atomicOr(P.err, kErrEtRange);
        continue;
      }
      if (P.nst == 1) {
        const int64_t slot = sIa[a] >= 0 ? sIa[a] + oab + sK[b] : -1;
        const float v = C1 * tr;
        if (slot < 0 || slot >= P.nnz) {
          atomicOr(P.err, kErrEtRange);
          continue;
        }
        if (fabsf(v) >= 1e-12f) P.a[slot] += v;
        continue;
      }
      float K[3][3];
#pragma unroll
      for (int s = 0; s < 3; s++)
#pragma unroll
        for (int t = 0; t < 3; t++)
          K[s][t] = (s == t) ? (tr - S[s][s]) * C1 + S[s][s] * C3 : S[t][s] * C1 - S[s][t] * C2;
      int64_t slot[3];
      bool bad = false;
#pragma unroll
      for (int s = 0; s < 3; s++) {
        slot[s] = sIa[a * 3 + s] >= 0 ? sIa[a * 3 + s] + oab + (int64_t)sK[b] * 3 : -1;
        bad |= slot[s] < 0 || slot[s] + 2 >= P.nnz;
      }
      if (bad) {
        atomicOr(P.err, kErrEtRange);
        continue;
      }
      float old[3][3];
#pragma unroll
      for (int s = 0; s < 3; s++)
#pragma unroll
        for (int t = 0; t < 3; t++) old[s][t] = P.a[slot[s] + t];
#pragma unroll
      for (int s = 0; s < 3; s++)
#pragma unroll
        for (int t = 0; t < 3; t++)
          if (fabsf(K[s][t]) >= 1e-12f) P.a[slot[s] + t] = old[s][t] + K[s][t];
    }
    __syncthreads();  // staging, rows and corners are the next element's
  }
  if (failed && tid == 0) {
    atomicOr(P.err, kErrEtWait);
    tc_wait(&s_mb, phase);  // the MMAs of the element in flight, before the columns are freed
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(COLS));
}

typedef void (*EtKernel)(EtArgs, EtHp, const int64_t *, int64_t);

EtKernel et_kernel(int nt, bool hp) {
  if (nt == 8) return hp ? k_elem_tc<8, true> : k_elem_tc<8, false>;
  if (nt == 27) return hp ? k_elem_tc<27, true> : k_elem_tc<27, false>;
  if (nt == 64) return hp ? k_elem_tc<64, true> : k_elem_tc<64, false>;
  return nullptr;
}

}  // namespace

bool elem_tc_supported(const Ctx &c, const Bucket *b) {
  return !b->key.is_bc && b->key.type == GPZ_EL_HEX && b->dim == 3 && b->ncorner == 8 && b->nq <= kEtMaxQ &&
         (c.nstate == 1 || c.nstate == 3) && et_kernel(b->nshape, b->hp) != nullptr &&
         (b->key.mat_kind == GPZ_MAT_POISSON || b->key.mat_kind == GPZ_MAT_DARCY ||
          b->key.mat_kind == GPZ_MAT_ELAST3D) &&
         !c.flt.active;
}

// One bucket's elements [e0, e1) (one colour) on the tensor cores, into c.d_a32.
void elem_tc_launch(Ctx &c, Bucket *b, int64_t e0, int64_t e1, cudaStream_t s) {
  const int nt = b->nshape, kp = (b->nq + 7) / 8 * 8;
  const EtKernel k = et_kernel(nt, b->hp);
  if (!b->d_dphi32.p) {  // FP32 tables of the bucket (once)
    std::vector<float> d(b->dphi.begin(), b->dphi.end()), w(b->w.begin(), b->w.end());
    b->d_dphi32.upload(d.data(), d.size(), s);
    b->d_w32.upload(w.data(), w.size(), s);
  }
  if (b->tc_smem == 0) {
    int dev = 0, nsm = 0, smem_sm = 0, reserved = 0;
    GPZ_CUDA_TRY(cudaGetDevice(&dev));
    GPZ_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    GPZ_CUDA_TRY(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    GPZ_CUDA_TRY(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev));
    uint32_t smem = et_smem(nt, kp);
    const int cols = et_cols(nt);
    constexpr uint32_t kMaxDyn = 225u * 1024u;  // 227 KB per CTA less the static shared memory
    GPZ_REQUIRE(smem <= kMaxDyn, GPZ_E_UNSUPPORTED_ELEMENT, "tensor-core element kernel: shared memory");
    GPZ_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxDyn));
    cudaFuncAttributes fa{};
    GPZ_CUDA_TRY(cudaFuncGetAttributes(&fa, k));
    // resident CTAs per SM from the kernel's registers (allocated per warp in units of 256), the threads and
    // the shared memory; the CTAs resident on one SM must not ask for more than its 512 TMEM columns (an
    // allocation would wait for another CTA to end), so the shared memory is padded until they cannot
    const int regs_warp = (fa.numRegs * 32 + 255) / 256 * 256;
    const int nth = et_threads(nt);
    const int per_regs = regs_warp > 0 ? 65536 / (regs_warp * (nth / 32)) : 8;
    auto per_of = [&](uint32_t sm) {
      const int per_smem = (int)((uint32_t)smem_sm / (sm + (uint32_t)fa.sharedSizeBytes + (uint32_t)reserved));
      return std::min(std::min(per_regs, 2048 / nth), per_smem);
    };
    int per = per_of(smem);
    while (per * cols > 512 && smem + 2048 <= kMaxDyn) {
      smem += 2048;
      per = per_of(smem);
    }
    GPZ_REQUIRE(per >= 1 && per * cols <= 512, GPZ_E_CUDA, "tensor-core element kernel: no resident CTA");
    b->tc_smem = (int)smem;
    b->tc_resident = per * nsm;
    b->tc_per_sm = per;
  }
  EtArgs P{};
  P.dphi = b->d_dphi32.p;
  P.w = b->d_w32.p;
  P.sside = b->d_shape_side.p;
  P.sk = b->d_shape_k.p;
  P.nq = b->nq;
  P.kp = kp;
  P.nsides = b->nsides;
  P.nst = c.nstate;
  const gpz_material &m = c.mats[c.h_el_mat[b->elems[0]]];
  P.kind = m.kind;
  P.xyz = c.d_xyz.p;
  P.el_nodes = c.d_el_nodes.p;
  P.el_conn = c.d_el_conn.p;
  P.bpos = c.d_block_pos.p;
  P.coef = c.d_coef.p;
  P.E = m.E;
  P.nu = m.nu;
  P.coef_const = m.coef_const;
  P.scale = m.scale;
  P.ia = c.d_ia.p;
  P.offbase = c.d_offbase.p;
  P.off = c.d_off.p;
  P.a = c.d_a32.p;
  P.nnz = c.nnz;
  P.neq = c.neq;
  P.err = c.d_err.p;
  EtHp H{nullptr, nullptr, nullptr};
  if (b->hp) {
    H.full = b->d_act_full.p + e0 * kMaxShapes;
    H.k = b->d_act_k.p + e0 * kMaxShapes;
    H.n = b->d_act_n.p + e0;
  }
  const int64_t ne = e1 - e0;
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ne, b->tc_resident));
  k<<<grid, et_threads(nt), (size_t)b->tc_smem, s>>>(P, H, b->d_elems.p + e0, ne);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
}

}  // namespace gpz
