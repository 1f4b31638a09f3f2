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
#include <cmath>
#include <vector>

#include "gpz_internal.h"
#include "gpz_solver_common.cuh"

namespace gpz {

namespace {

constexpr int kNS = 27;  // Q2 hex shapes
constexpr int kNQ = 27;  // 3 x 3 x 3 Gauss points
constexpr int kFS = 9;   // Q2 face shapes
constexpr int kFQ = 9;   // 3 x 3 face points
constexpr int kWarps = kThreads / 32;

// element records: corner coordinates, block rows of the shapes, (lambda, mu)
__global__ void k_mf_records(int64_t n, const int64_t *__restrict__ elems, const int64_t *__restrict__ el_nodes,
                             const double *__restrict__ xyz, const int64_t *__restrict__ el_conn,
                             const int64_t *__restrict__ bpos, const int *__restrict__ sside,
                             const int *__restrict__ sk, int nsh, int nc, const double *__restrict__ coef, double E0,
                             double nu, float *__restrict__ rxyz, int32_t *__restrict__ rrows, float *__restrict__ rlm,
                             int *__restrict__ err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t e = elems[i];
  for (int k = 0; k < nc; k++) {
    const int64_t node = el_nodes[e * 8 + k];
    for (int j = 0; j < 3; j++) rxyz[(i * nc + k) * 3 + j] = (float)xyz[node * 3 + j];
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
       i += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    int32_t row = 0;
    float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
    if (lane < kFS) {
      row = rows[i * kFS + lane];
      u = p4[row];
      su[wp][lane][0] = u.x;
      su[wp][lane][1] = u.y;
      su[wp][lane][2] = u.z;
    }
    if (lane < 12) sc[wp][lane] = rxyz[i * 12 + lane];
    __syncwarp();
    if (lane < kFQ) {
      const int q = lane;
      float g0[3] = {0.f, 0.f, 0.f}, g1[3] = {0.f, 0.f, 0.f};
      for (int k = 0; k < 4; k++)
        for (int j = 0; j < 3; j++) {
          g0[j] += sc[wp][k * 3 + j] * sd[(q * 2 + 0) * kFS + k];
          g1[j] += sc[wp][k * 3 + j] * sd[(q * 2 + 1) * kFS + k];
        }
      const float cx = g0[1] * g1[2] - g0[2] * g1[1], cy = g0[2] * g1[0] - g0[0] * g1[2],
                  cz = g0[0] * g1[1] - g0[1] * g1[0];
      const float wd = big * sw[q] * sqrtf(cx * cx + cy * cy + cz * cz);
      float uq[3] = {0.f, 0.f, 0.f};
      for (int b = 0; b < kFS; b++) {
        const float ph = sphi[q * kFS + b];
        for (int s = 0; s < 3; s++) uq[s] += ph * su[wp][b][s];
      }
      for (int s = 0; s < 3; s++) st[wp][q][s] = wd * uq[s];
    }
    __syncwarp();
    if (lane < kFS) {
      float y[3] = {0.f, 0.f, 0.f};
      for (int q = 0; q < kFQ; q++) {
        const float ph = sphi[q * kFS + lane];
        for (int s = 0; s < 3; s++) y[s] += st[wp][q][s] * ph;
      }
      en.add(y[0] * u.x + y[1] * u.y + y[2] * u.z);
      atomicAdd(&q4[row], make_float4(y[0], y[1], y[2], 0.f));
    }
    __syncwarp();
  }
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
                                                            const float *__restrict__ dphi /*[q][3][a]*/,
                                                            const float *__restrict__ w,
                                                            const float4 *__restrict__ p4, float4 *__restrict__ q4,
                                                            const double *__restrict__ face_energy, Red R) {
  if (!active(R.iscal)) return;
  __shared__ float4 sdt[kNQ][32];            // [q][a] = (d0, d1, d2, 0) of shape a at point q
  __shared__ float4 su[kMfWarps][kNS];
  __shared__ float sc[kMfWarps][24];
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
  float cxv = 0.f, lam = 0.f, mu = 0.f;
  if (i < n) {
    if (lane < kNS) row = rows[i * kNS + lane];
    if (lane < 24) cxv = rxyz[i * 24 + lane];
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
    const float lam_i = lam, mu_i = mu;
    const int32_t row_i = row;
    // prefetch the next element's records
    const int64_t nx = i + step;
    if (nx < n) {
      if (lane < kNS) row = rows[nx * kNS + lane];
      if (lane < 24) cxv = rxyz[nx * 24 + lane];
      lam = rlm[2 * nx];
      mu = rlm[2 * nx + 1];
    }
    __syncwarp();
    if (lane < kNQ) {
      // Jacobian from the corner shapes (the first 8 of the table), as TPZGeoEl::Jacobian
      float a[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
      for (int k = 0; k < 8; k++)
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
          for (int d = 0; d < 3; d++) a[j][d] += sc[wp][k * 3 + j] * D[d][k];
      const float det = -a[0][2] * a[1][1] * a[2][0] + a[0][1] * a[1][2] * a[2][0] + a[0][2] * a[1][0] * a[2][1] -
                        a[0][0] * a[1][2] * a[2][1] - a[0][1] * a[1][0] * a[2][2] + a[0][0] * a[1][1] * a[2][2];
      const float id = 1.f / det;
      float ji[3][3];
      ji[0][0] = (-a[1][2] * a[2][1] + a[1][1] * a[2][2]) * id;
      ji[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * id;
      ji[0][2] = (-a[0][2] * a[1][1] + a[0][1] * a[1][2]) * id;
      ji[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) * id;
      ji[1][1] = (-a[0][2] * a[2][0] + a[0][0] * a[2][2]) * id;
      ji[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * id;
      ji[2][0] = (-a[1][1] * a[2][0] + a[1][0] * a[2][1]) * id;
      ji[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * id;
      ji[2][2] = (-a[0][1] * a[1][0] + a[0][0] * a[1][1]) * id;
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
      atomicAdd(&q4[row_i], make_float4(y0, y1, y2, 0.f));
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

// Build the element records of the matrix-free operator; false when the mesh
// is not made of uniform Q2 hex elasticity elements plus penalty / traction faces.
bool matfree_build(Ctx &c) {
  MatFree &M = c.mf;
  M.ready = false;
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
  M.vrows.alloc((size_t)M.nvol * kNS);
  M.vlm.alloc((size_t)M.nvol * 2);
  f32(vol->dphi, M.vdphi);
  f32(vol->w, M.vw);
  k_mf_records<<<grid_for(M.nvol, 256), 256, 0, s>>>(M.nvol, vol->d_elems.p, c.d_el_nodes.p, c.d_xyz.p, c.d_el_conn.p,
                                                     c.d_block_pos.p, vol->d_shape_side.p, vol->d_shape_k.p, kNS, 8,
                                                     c.d_coef.p, m.E, m.nu, M.vxyz.p, M.vrows.p, M.vlm.p, c.d_err.p);
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
                                                        M.frows.p, nullptr, c.d_err.p);
    c.launches++;
  }
  M.energy.alloc(1);
  GPZ_CUDA_TRY(cudaGetLastError());
  check_device_flag(c, "matrix-free records");
  M.grid_vol = mf_grid(k_mf_hex27, kMfThreads);
  M.grid_face = mf_grid(k_mf_faces, kThreads);
  M.ready = true;
  return true;
}

// q4 = A p4 (q4 zeroed by the caller), p.q and alpha as the block SpMV kernels
void matfree_spmv(Ctx &c, cudaStream_t s) {
  MatFree &M = c.mf;
  SolverWork &w = c.sw;
  Red R{w.partial.p, w.counter.p, w.scal.p, w.iscal.p};
  const float4 *p4 = (const float4 *)w.pm.p;
  float4 *q4 = (float4 *)w.q32.p;
  if (M.nface) {
    k_mf_faces<<<M.grid_face, kThreads, 0, s>>>(M.nface, M.fxyz.p, M.frows.p, M.fphi.p, M.fdphi.p, M.fw.p, M.big, p4,
                                                q4, M.energy.p, R);
    c.launches++;
  }
  k_mf_hex27<<<M.grid_vol, kMfThreads, 0, s>>>(M.nvol, M.vxyz.p, M.vrows.p, M.vlm.p, M.vdphi.p, M.vw.p, p4, q4,
                                             M.nface ? M.energy.p : nullptr, R);
  c.launches++;
}

}  // namespace gpz
