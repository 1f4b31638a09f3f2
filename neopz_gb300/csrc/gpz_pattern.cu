// CSR sparsity pattern built on the device from the element graph.
//
// Restates TPZCompMesh::ComputeElGraph (Mesh/pzcmesh.cpp:1214-1262),
// TPZRenumbering::ConvertGraph (External/TPZRenumbering.cpp:76-105: for every
// connect the sorted set of connects sharing an element, itself excluded) and
// TPZSpStructMatrix::SetupMatrixData (StrMatrix/TPZSpStructMatrix.cpp:53-190:
// row = equations of the diagonal block followed by every neighbour block,
// sorted).  TPZSSpStructMatrix's upper-triangular pattern
// (StrMatrix/TPZSSpStructMatrix.cpp:50-193) is the suffix of each full row that
// starts at the diagonal, so it is derived from the full one.  Blocks of size
// zero (connects without shape functions) are skipped as NumActive()==0 does.
#include <algorithm>
#include <climits>

#include "gpz_internal.h"

namespace gpz {

namespace {

constexpr int kWarpsPerBlock = 8;
constexpr int kGather = 1024;  // connects gathered around one connect (with repeats)

__device__ __forceinline__ int nsides_of(int t) { return t == GPZ_EL_LINE ? 3 : (t == GPZ_EL_QUAD ? 9 : 27); }

__global__ void k_conn_elem_count(const int32_t *__restrict__ type, const int64_t *__restrict__ conn,
                                  const int32_t *__restrict__ bsize, int64_t nel, int64_t nconn,
                                  int64_t *__restrict__ cnt, int *__restrict__ err) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  int ns = nsides_of(type[e]);
  for (int s = 0; s < ns; s++) {
    int64_t c = conn[e * 27 + s];
    if (c < 0 || c >= nconn) {
      atomicOr(err, 1);
      return;
    }
    if (bsize[c] > 0) atomicAdd((unsigned long long *)&cnt[c], 1ull);
  }
}

__global__ void k_conn_elem_fill(const int32_t *__restrict__ type, const int64_t *__restrict__ conn,
                                 const int32_t *__restrict__ bsize, int64_t nel, const int64_t *__restrict__ off,
                                 int64_t *__restrict__ fill, int64_t *__restrict__ c2e) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  int ns = nsides_of(type[e]);
  for (int s = 0; s < ns; s++) {
    int64_t c = conn[e * 27 + s];
    if (bsize[c] > 0) {
      unsigned long long k = atomicAdd((unsigned long long *)&fill[c], 1ull);
      c2e[off[c] + (int64_t)k] = e;
    }
  }
}

// One warp per connect: gather the connects of every element around it,
// bitonic-sort them in shared memory and keep the distinct non-empty ones.
// mode 0 counts, mode 1 writes the list with the prefix of block sizes.
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_neighbours(int mode, const int32_t *__restrict__ type, const int64_t *__restrict__ conn,
                 const int32_t *__restrict__ bsize, int64_t nconn, const int64_t *__restrict__ c2e_off,
                 const int64_t *__restrict__ c2e, int64_t *__restrict__ nbr_cnt, const int64_t *__restrict__ nbr_off,
                 int32_t *__restrict__ nbr, int64_t *__restrict__ nbr_pfx, int32_t *__restrict__ nbr_owner,
                 int *__restrict__ err) {
  __shared__ int32_t sbuf[kWarpsPerBlock][kGather];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int64_t c = (int64_t)blockIdx.x * kWarpsPerBlock + w;
  if (c >= nconn) return;
  if (bsize[c] == 0) {
    if (mode == 0 && lane == 0) nbr_cnt[c] = 0;
    return;
  }
  int32_t *buf = sbuf[w];
  // gather
  int k = 0;
  int64_t e0 = c2e_off[c], e1 = c2e_off[c + 1];
  bool overflow = false;
  for (int64_t ie = e0; ie < e1; ie++) {
    int64_t e = c2e[ie];
    int ns = nsides_of(type[e]);
    if (k + ns > kGather) {
      overflow = true;
      break;
    }
    for (int s = lane; s < ns; s += 32) {
      int64_t n = conn[e * 27 + s];
      buf[k + s] = bsize[n] > 0 ? (int32_t)n : INT_MAX;
    }
    k += ns;
  }
  if (overflow) {
    if (lane == 0) atomicOr(err, 2);
    return;
  }
  int P = 32;
  while (P < k) P <<= 1;
  for (int i = k + lane; i < P; i += 32) buf[i] = INT_MAX;
  __syncwarp();
  // bitonic sort of P entries
  for (int size = 2; size <= P; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = lane; i < P / 2; i += 32) {
        int lo = 2 * i - (i & (stride - 1));
        int hi = lo + stride;
        bool up = ((lo & size) == 0);
        int32_t a = buf[lo], b = buf[hi];
        if ((a > b) == up) {
          buf[lo] = b;
          buf[hi] = a;
        }
      }
      __syncwarp();
    }
  }
  // distinct values in order
  int64_t out = 0;
  int64_t base = mode == 1 ? nbr_off[c] : 0;
  int64_t run = 0;  // running prefix of block sizes
  for (int i0 = 0; i0 < P; i0 += 32) {
    int i = i0 + lane;
    int32_t v = buf[i];
    bool keep = (v != INT_MAX) && (i == 0 || buf[i - 1] != v);
    unsigned m = __ballot_sync(0xffffffffu, keep);
    int rank = __popc(m & ((1u << lane) - 1));
    int32_t sz = keep ? bsize[v] : 0;
    // inclusive warp scan of the kept sizes
    int64_t incl = sz;
    for (int d = 1; d < 32; d <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += y;
    }
    if (mode == 1 && keep) {
      nbr[base + out + rank] = v;
      nbr_pfx[base + out + rank] = run + incl - sz;
      nbr_owner[base + out + rank] = (int32_t)c;
    }
    out += __popc(m);
    run += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (mode == 0 && lane == 0) nbr_cnt[c] = out;
}

__global__ void k_rowlen(const int64_t *__restrict__ nbr_off, const int32_t *__restrict__ nbr,
                         const int64_t *__restrict__ nbr_pfx, const int32_t *__restrict__ bsize,
                         const int64_t *__restrict__ bpos, int64_t nconn, int64_t *__restrict__ rowlen) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nconn) return;
  int sz = bsize[c];
  if (sz == 0) return;
  int64_t b = nbr_off[c], e = nbr_off[c + 1];
  int64_t L = nbr_pfx[e - 1] + bsize[nbr[e - 1]];
  for (int k = 0; k < sz; k++) rowlen[bpos[c] + k] = L;
}

__global__ void k_fill_ja(const int32_t *__restrict__ nbr, const int64_t *__restrict__ nbr_pfx,
                          const int32_t *__restrict__ nbr_owner, int64_t nentries, const int32_t *__restrict__ bsize,
                          const int64_t *__restrict__ bpos, const int64_t *__restrict__ ia, int32_t *__restrict__ ja) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nentries) return;
  int32_t c = nbr_owner[i], n = nbr[i];
  int szc = bsize[c], szn = bsize[n];
  int64_t pc = bpos[c], pn = bpos[n], pf = nbr_pfx[i];
  for (int k = 0; k < szc; k++) {
    int64_t base = ia[pc + k] + pf;
    for (int t = 0; t < szn; t++) ja[base + t] = (int32_t)(pn + t);
  }
}

// ---- equation filter (TPZEquationFilter::SetActiveEquations / Filter,
// StrMatrix/TPZEquationFilter.h; applied to the pattern as
// TPZSSpStructMatrix::SetupMatrixData, StrMatrix/TPZSSpStructMatrix.cpp:49-193,
// and TPZSpStructMatrix::SetupMatrixData, StrMatrix/TPZSpStructMatrix.cpp:53-190,
// apply it: rows and columns of inactive equations are dropped and the active
// ones renumbered in increasing order, which keeps every row sorted)
__global__ void k_flt_dest(const int64_t *__restrict__ act, int64_t n, int64_t *__restrict__ dest) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dest[act[i]] = i;
}

__global__ void k_flt_gather(const double *__restrict__ v, const int64_t *__restrict__ idx, int64_t n,
                             double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = v[idx[i]];
}

__global__ void k_flt_scatter(const double *__restrict__ v, const int64_t *__restrict__ idx, int64_t n,
                              double *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[idx[i]] = v[i];
}

__global__ void k_flt_zero_inactive(const int64_t *__restrict__ dest, int64_t n, double *__restrict__ f) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && dest[i] < 0) f[i] = 0.0;
}

__global__ void k_flt_count(const int64_t *__restrict__ m_ia, const int32_t *__restrict__ m_ja,
                            const int64_t *__restrict__ act, const int64_t *__restrict__ dest, int64_t n,
                            int64_t *__restrict__ rowlen) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t r = act[i];
  int64_t cnt = 0;
  for (int64_t k = m_ia[r]; k < m_ia[r + 1]; k++) cnt += dest[m_ja[k]] >= 0 ? 1 : 0;
  rowlen[i] = cnt;
}

__global__ void k_flt_fill(const int64_t *__restrict__ m_ia, const int32_t *__restrict__ m_ja,
                           const int64_t *__restrict__ act, const int64_t *__restrict__ dest, int64_t n,
                           const int64_t *__restrict__ ia, int32_t *__restrict__ ja, int64_t *__restrict__ keep) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t r = act[i];
  int64_t p = ia[i];
  for (int64_t k = m_ia[r]; k < m_ia[r + 1]; k++) {
    const int64_t d = dest[m_ja[k]];
    if (d >= 0) {
      ja[p] = (int32_t)d;
      keep[p] = k;
      p++;
    }
  }
}

__device__ __forceinline__ int64_t find_col(const int32_t *__restrict__ ja, int64_t lo, int64_t hi, int64_t col) {
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (ja[mid] < col) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void k_diagpos(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja, int64_t neq,
                          int64_t *__restrict__ diagpos, int64_t *__restrict__ uplen, int *__restrict__ err) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= neq) return;
  int64_t k = find_col(ja, ia[r], ia[r + 1], r);
  if (k >= ia[r + 1] || ja[k] != r) {
    atomicOr(err, 4);
    k = ia[r];
  }
  diagpos[r] = k;
  if (uplen) uplen[r] = ia[r + 1] - k;
}

// a warp per row (a CTA per row launched millions of small CTAs)
__global__ void k_fill_upper(const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                             const int64_t *__restrict__ diagpos, const int64_t *__restrict__ ia_up, int64_t neq,
                             int32_t *__restrict__ ja_up) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= neq) return;
  const int64_t d = diagpos[r], n = ia[r + 1] - d, o = ia_up[r];
  for (int64_t k = lane; k < n; k += 32) ja_up[o + k] = ja[d + k];
}

// Offset of block B inside the rows of block A, for every side pair of every
// element: the position of column pos_B in row pos_A (all rows of one block
// share their column structure in the full pattern).
__global__ void k_elem_offsets(const int32_t *__restrict__ type, const int64_t *__restrict__ conn,
                               const int32_t *__restrict__ bsize, const int64_t *__restrict__ bpos,
                               const int64_t *__restrict__ ia, const int32_t *__restrict__ ja,
                               const int64_t *__restrict__ offbase, int64_t nel, int32_t *__restrict__ off,
                               int *__restrict__ err) {
  int64_t e = blockIdx.x;
  if (e >= nel) return;
  int ns = nsides_of(type[e]);
  for (int idx = threadIdx.x; idx < ns * ns; idx += blockDim.x) {
    int sa = idx / ns, sb = idx % ns;
    int64_t A = conn[e * 27 + sa], B = conn[e * 27 + sb];
    int32_t v = -1;
    if (bsize[A] > 0 && bsize[B] > 0) {
      int64_t r = bpos[A];
      int64_t k = find_col(ja, ia[r], ia[r + 1], bpos[B]);
      if (k >= ia[r + 1] || ja[k] != bpos[B]) atomicOr(err, 8);
      else v = (int32_t)(k - ia[r]);
    }
    off[offbase[e] + idx] = v;
  }
}

}  // namespace

void build_pattern(Ctx &c) {
  cudaStream_t s = c.stream;
  const int64_t nel = c.nel, nconn = c.nconnects;
  DBuf<int64_t> cnt, c2e_off, fill, c2e;
  cnt.alloc(nconn + 1);
  cnt.zero(s);
  c2e_off.alloc(nconn + 1);
  k_conn_elem_count<<<grid_for(nel, 256), 256, 0, s>>>(c.d_el_type.p, c.d_el_conn.p, c.d_block_size.p, nel, nconn,
                                                       cnt.p, c.d_err.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  check_device_flag(c, "connect/element count");
  exclusive_scan_i64(cnt.p, c2e_off.p, nconn + 1, s, c);
  int64_t total = 0;
  GPZ_CUDA_TRY(cudaMemcpyAsync(&total, c2e_off.p + nconn, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  fill.alloc(nconn);
  fill.zero(s);
  c2e.alloc(std::max<int64_t>(total, 1));
  k_conn_elem_fill<<<grid_for(nel, 256), 256, 0, s>>>(c.d_el_type.p, c.d_el_conn.p, c.d_block_size.p, nel,
                                                      c2e_off.p, fill.p, c2e.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());

  DBuf<int64_t> nbr_cnt, nbr_off, nbr_pfx;
  DBuf<int32_t> nbr, nbr_owner;
  nbr_cnt.alloc(nconn + 1);
  nbr_cnt.zero(s);
  nbr_off.alloc(nconn + 1);
  unsigned nb = (unsigned)((nconn + kWarpsPerBlock - 1) / kWarpsPerBlock);
  k_neighbours<<<nb, kWarpsPerBlock * 32, 0, s>>>(0, c.d_el_type.p, c.d_el_conn.p, c.d_block_size.p, nconn, c2e_off.p,
                                                   c2e.p, nbr_cnt.p, nullptr, nullptr, nullptr, nullptr, c.d_err.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  check_device_flag(c, "neighbour count");
  exclusive_scan_i64(nbr_cnt.p, nbr_off.p, nconn + 1, s, c);
  int64_t nentries = 0;
  GPZ_CUDA_TRY(cudaMemcpyAsync(&nentries, nbr_off.p + nconn, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  nbr.alloc(std::max<int64_t>(nentries, 1));
  nbr_pfx.alloc(std::max<int64_t>(nentries, 1));
  nbr_owner.alloc(std::max<int64_t>(nentries, 1));
  k_neighbours<<<nb, kWarpsPerBlock * 32, 0, s>>>(1, c.d_el_type.p, c.d_el_conn.p, c.d_block_size.p, nconn, c2e_off.p,
                                                   c2e.p, nullptr, nbr_off.p, nbr.p, nbr_pfx.p, nbr_owner.p, c.d_err.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());

  // row lengths -> IA -> JA
  DBuf<int64_t> rowlen;
  rowlen.alloc(c.neq + 1);
  rowlen.zero(s);
  k_rowlen<<<grid_for(nconn, 256), 256, 0, s>>>(nbr_off.p, nbr.p, nbr_pfx.p, c.d_block_size.p, c.d_block_pos.p, nconn,
                                                rowlen.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  c.d_ia.alloc(c.neq + 1);
  exclusive_scan_i64(rowlen.p, c.d_ia.p, c.neq + 1, s, c);
  GPZ_CUDA_TRY(cudaMemcpyAsync(&c.nnz, c.d_ia.p + c.neq, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  GPZ_REQUIRE(c.nnz < (int64_t)INT32_MAX * 2, GPZ_E_INVALID, "pattern too large");
  c.d_ja.alloc(std::max<int64_t>(c.nnz, 1));
  k_fill_ja<<<grid_for(nentries, 256), 256, 0, s>>>(nbr.p, nbr_pfx.p, nbr_owner.p, nentries, c.d_block_size.p,
                                                    c.d_block_pos.p, c.d_ia.p, c.d_ja.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
}

void build_upper(Ctx &c) {
  cudaStream_t s = c.stream;
  DBuf<int64_t> uplen;
  uplen.alloc(c.neq + 1);
  uplen.zero(s);
  c.d_diagpos.alloc(c.neq);
  k_diagpos<<<grid_for(c.neq, 256), 256, 0, s>>>(c.d_ia.p, c.d_ja.p, c.neq, c.d_diagpos.p, uplen.p, c.d_err.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  check_device_flag(c, "diagonal search");
  c.d_ia_up.alloc(c.neq + 1);
  exclusive_scan_i64(uplen.p, c.d_ia_up.p, c.neq + 1, s, c);
  GPZ_CUDA_TRY(cudaMemcpyAsync(&c.nnz_upper, c.d_ia_up.p + c.neq, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  c.d_ja_up.alloc(std::max<int64_t>(c.nnz_upper, 1));
  if (c.neq > 0) {
    k_fill_upper<<<grid_for(c.neq * 32, 256), 256, 0, s>>>(c.d_ia.p, c.d_ja.p, c.d_diagpos.p, c.d_ia_up.p, c.neq,
                                                           c.d_ja_up.p);
    c.launches++;
    GPZ_CUDA_TRY(cudaGetLastError());
  }
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
}

// the active set and the mesh -> condensed map on the device (set when the
// filter is given, so that a load-vector-only assembly can use them too)
void filter_prepare(Ctx &c) {
  auto &F = c.flt;
  const int64_t n = (int64_t)F.h_act.size();
  cudaStream_t s = c.stream;
  F.act.upload(F.h_act.data(), n, s);
  F.dest.alloc(c.neq_mesh);
  GPZ_CUDA_TRY(cudaMemsetAsync(F.dest.p, 0xff, c.neq_mesh * sizeof(int64_t), s));  // -1
  k_flt_dest<<<grid_for(n, 256), 256, 0, s>>>(F.act.p, n, F.dest.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
}

template <class T>
static void swap_buf(DBuf<T> &a, DBuf<T> &b) {
  std::swap(a.p, b.p);
  std::swap(a.n, b.n);
}

// The mesh-level full CSR in c.d_ia / c.d_ja (after build_pattern, build_upper
// and build_element_offsets) becomes the assembly's target (c.flt.m_*), and the
// system arrays are rebuilt over the active equations.
void condense_pattern(Ctx &c) {
  cudaStream_t s = c.stream;
  auto &F = c.flt;
  const int64_t n = (int64_t)F.h_act.size();
  swap_buf(c.d_ia, F.m_ia);
  swap_buf(c.d_ja, F.m_ja);
  swap_buf(c.d_diagpos, F.m_diagpos);
  F.m_nnz = c.nnz;
  filter_prepare(c);
  DBuf<int64_t> rowlen;
  rowlen.alloc(n + 1);
  rowlen.zero(s);
  k_flt_count<<<grid_for(n, 256), 256, 0, s>>>(F.m_ia.p, F.m_ja.p, F.act.p, F.dest.p, n, rowlen.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  c.d_ia.alloc(n + 1);
  exclusive_scan_i64(rowlen.p, c.d_ia.p, n + 1, s, c);
  GPZ_CUDA_TRY(cudaMemcpyAsync(&c.nnz, c.d_ia.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  GPZ_CUDA_TRY(cudaStreamSynchronize(s));
  c.d_ja.alloc(std::max<int64_t>(c.nnz, 1));
  F.keep.alloc(std::max<int64_t>(c.nnz, 1));
  k_flt_fill<<<grid_for(n, 256), 256, 0, s>>>(F.m_ia.p, F.m_ja.p, F.act.p, F.dest.p, n, c.d_ia.p, c.d_ja.p,
                                              F.keep.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
  c.neq = n;
  build_upper(c);  // the system's diagonal slots and upper triangle
}

// TPZEquationFilter::Gather (mesh -> active equations), ::Scatter (active
// equations -> mesh, zeros elsewhere), and the zeros the reference's filtered
// rhs assembly leaves at inactive equations (StrMatrix/pzstrmatrixor.cpp:43-71)
void filter_gather(Ctx &c, const double *v_mesh, double *v_sys) {
  k_flt_gather<<<grid_for(c.neq, 256), 256, 0, c.stream>>>(v_mesh, c.flt.act.p, c.neq, v_sys);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
}
void filter_scatter(Ctx &c, const double *v_sys, double *v_mesh) {
  GPZ_CUDA_TRY(cudaMemsetAsync(v_mesh, 0, c.neq_mesh * sizeof(double), c.stream));
  k_flt_scatter<<<grid_for(c.neq, 256), 256, 0, c.stream>>>(v_sys, c.flt.act.p, c.neq, v_mesh);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
}
void filter_zero_inactive(Ctx &c, double *f_mesh) {
  k_flt_zero_inactive<<<grid_for(c.neq_mesh, 256), 256, 0, c.stream>>>(c.flt.dest.p, c.neq_mesh, f_mesh);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
}
void filter_values(Ctx &c) {
  k_flt_gather<<<grid_for(c.nnz, 256), 256, 0, c.stream>>>(c.flt.m_a.p, c.flt.keep.p, c.nnz, c.d_a.p);
  c.launches++;
  GPZ_CUDA_TRY(cudaGetLastError());
}

void build_element_offsets(Ctx &c) {
  cudaStream_t s = c.stream;
  std::vector<int64_t> base(c.nel + 1, 0);
  for (int64_t e = 0; e < c.nel; e++) {
    int t = c.h_el_type[e];
    int ns = t == GPZ_EL_LINE ? 3 : (t == GPZ_EL_QUAD ? 9 : 27);
    base[e + 1] = base[e] + ns * ns;
  }
  c.d_offbase.upload(base.data(), c.nel + 1, s);
  c.d_off.alloc(std::max<int64_t>(base[c.nel], 1));
  if (c.nel > 0) {
    k_elem_offsets<<<(unsigned)c.nel, 128, 0, s>>>(c.d_el_type.p, c.d_el_conn.p, c.d_block_size.p, c.d_block_pos.p,
                                                  c.d_ia.p, c.d_ja.p, c.d_offbase.p, c.nel, c.d_off.p, c.d_err.p);
    c.launches++;
    GPZ_CUDA_TRY(cudaGetLastError());
  }
  check_device_flag(c, "element offsets");
}

}  // namespace gpz
