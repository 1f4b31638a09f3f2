// Internal declarations of libgpz (the sm_103a implementation behind include/gpz.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <exception>
#include <thread>
#include <string>
#include <vector>

#include "../../include/gpz.h"

namespace gpz {

// ---------------------------------------------------------------- errors
struct Error {
  int code;
  std::string msg;
};

#define GPZ_CUDA_TRY(expr)                                                                  \
  do {                                                                                      \
    cudaError_t _e = (expr);                                                                \
    if (_e != cudaSuccess) {                                                                \
      throw ::gpz::Error{_e == cudaErrorMemoryAllocation ? GPZ_E_NOMEM : GPZ_E_CUDA,        \
                         std::string(#expr) + ": " + cudaGetErrorString(_e)};               \
    }                                                                                       \
  } while (0)

#define GPZ_REQUIRE(cond, code, text)                  \
  do {                                                 \
    if (!(cond)) throw ::gpz::Error{(code), (text)};   \
  } while (0)

// ---------------------------------------------------------------- device buffers
template <class T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    release();
    if (count == 0) return;
    GPZ_CUDA_TRY(cudaMalloc((void **)&p, count * sizeof(T)));
    n = count;
  }
  void upload(const T *h, size_t count, cudaStream_t s) {
    alloc(count);
    if (count) GPZ_CUDA_TRY(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void zero(cudaStream_t s) {
    if (n) GPZ_CUDA_TRY(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
};

// ---------------------------------------------------------------- element buckets
// Elements that share element type, side orders, side orientations, material
// kind and role (volume / boundary) share their shape tables and their kernel.
constexpr int kMaxShapes = 64;   // hex p=3: 64 scalar shapes
constexpr int kMaxQp = 64;       // hex 4x4x4 Gauss points

struct BucketKey {
  int type, is_bc, mat_kind, mat_index, intorder;  // mat_index: the element's el_mat value
  int hp;              // 1: hp class (orders below are the class order; elements use subsets)
  int orders[19];      // order of each non-corner side
  int trans[19];       // orientation id of each non-corner side (0 when irrelevant)
  bool operator<(const BucketKey &o) const;
};

struct Bucket {
  BucketKey key;
  int nsides = 0, ncorner = 0, dim = 0, nshape = 0, nq = 0, nstate = 1, ndof = 0;
  // host tables
  std::vector<double> phi, dphi, w;          // [nq][nshape], [nq][dim][nshape], [nq]
  std::vector<int> shape_side, shape_k;      // shape -> side, index inside the side
  // device tables
  DBuf<double> d_phi, d_dphi, d_w;
  // reference Gram of the volume hex tables: G[a][b][i][j] = sum_q w_q dphi_i(a) dphi_j(b) (affine elements)
  std::vector<double> ghat;
  DBuf<double> d_ghat;
  DBuf<int> d_shape_side, d_shape_k;
  // elements of this bucket grouped by colour
  std::vector<int64_t> elems;                // global element indices
  std::vector<int64_t> colour_begin;         // [ncolours+1]
  DBuf<int64_t> d_elems;
  // hp class: elements of uneven side orders up to the class order share the
  // tables of the full element of that order; per element (in elems order) the
  // active shapes as indices into the table and as indices inside their side
  bool hp = false;
  std::vector<uint8_t> act_full, act_k;      // [elems][kMaxShapes]
  std::vector<int32_t> act_n;                // [elems]
  DBuf<uint8_t> d_act_full, d_act_k;
  DBuf<int32_t> d_act_n;
  int threads = 128;                         // block size (autotuned for hp classes)
  bool tuned = false;
  // shared element matrix: 1 when every element is a translate of the first (same affine
  // Jacobian), so K_e = coefficient_e x kref; -1 before the check
  int shared = -1;
  DBuf<double> d_kref, d_fref;               // [ndof][ndof] at coefficient 1, [ndof] load vector
  // row-owner assembly of a shared-matrix bucket (k_rowpass): per unit of nstate
  // equations (one shape of one connect) the bucket's (element, shape)
  // incidences, sorted, packed as (index in elems << 8 | shape); -1 before the
  // lists are built, 0 when the bucket does not qualify
  int rowpass = -1;
  DBuf<int64_t> d_rp_ptr, d_rp_inc;
  DBuf<int64_t> d_rp_rec;  // per incidence, for the current pattern: slot-offset row, element, shape
  DBuf<double> d_rp_kp;    // kref without the entries the 1e-12 rule always drops, then a flag
  // persistent launch over all colours: colour boundaries, work / done counters, resident CTAs
  DBuf<int64_t> d_cbeg;
  DBuf<unsigned long long> d_q;
  int qgrid = 1;
  // tensor-core FP32 element matrices (gpz_elem_tc.cu): FP32 tables, dynamic shared memory, resident CTAs
  DBuf<float> d_dphi32, d_w32;
  int tc_smem = 0, tc_resident = 0, tc_per_sm = 0;
};

// ---------------------------------------------------------------- solver workspace
struct SolverWork {
  DBuf<double> r, z, p, q, x, b, t;
  DBuf<float> pm, r32, q32, dx32;  // mixed CG inner vectors (pm padded x4 for the block SpMV)
  DBuf<float> z32;                 // learned flexible CG over the FP32 operator: z = M r
  DBuf<double> partial;        // per-CTA partial sums
  DBuf<double> scal;           // device scalars (see gpz_solver.cu)
  DBuf<unsigned int> counter;  // last-block counters
  DBuf<int64_t> iscal;         // device integer scalars
  DBuf<double> gm_v;           // GMRES Krylov basis [m+1][neq]
  DBuf<double> gm_d;           // GMRES Hessenberg, rotations, y, scalars
  DBuf<int64_t> gm_i;          // GMRES state words
  size_t nblk = 0;
};

// ---------------------------------------------------------------- learned preconditioner
// Element-to-node message-passing network that produces per-element factors
// F_e of the preconditioner in gpz_learned.cuh (gpz_learned.cu).
struct Learned {
  bool ready = false;                        // mesh incidence built
  bool have_params = false;
  int R = 4, NS = 0, nsides = 0;
  int64_t E = 0, nconn = 0, nparams = 0, adam_t = 0;
  std::vector<int64_t> h_vel;                // volume element -> element index
  DBuf<int32_t> ec;                          // [E][nsides] connects of each volume element
  DBuf<int64_t> ce_ptr;                      // connect -> volume elements
  DBuf<int32_t> ce_idx;
  DBuf<int32_t> dest;                        // [E][NS]
  DBuf<int64_t> ne_ptr;                      // equation -> (element, local), built when first needed
  DBuf<int32_t> ne_idx;
  bool have_ne = false;
  DBuf<double> mask, dsq;                    // [neq]
  DBuf<float> mdsq;                          // [neq] mask * dsq
  DBuf<float> dinv32;                        // [neq] 1 / a_ii in FP32 (the FP32 recurrence of the mixed path)
  DBuf<float> feat;                          // [E] log coefficient
  DBuf<float> params, grad, m1, m2;
  DBuf<float> F;                             // [E][NS][R]
  DBuf<uint16_t> F16;                        // F in bfloat16, read by the solves
  DBuf<uint16_t> F16ne;                      // its rows in incidence (ne_idx) order
  DBuf<float> t;                             // [E][R]
  DBuf<float> act, back, partial;            // activations, backward buffers, outer-product partials
  DBuf<double> red;                          // dot-product partials
  int npairs = 0;
  DBuf<double> pr, pe, pz, pw, paw, pg;      // [P][neq] residuals, errors, M r, masked error of M r, A w, dL/dz
  DBuf<double> pscal;                        // [P][2] e^T A e, loss
  DBuf<double> aterm;                        // [P] alpha-gradient terms
  // base preconditioner the correction is trained on: 0 point Jacobi (alpha D^-1 r), or
  // GPZ_PRECOND_BLOCK_JACOBI / GPZ_PRECOND_TWO_LEVEL: alpha B^-1 r (+ the coarse part, taken off the targets)
  int base = 0;
  DBuf<double> pb, ones;                     // [P][neq] B^-1 r_j; [neq] ones
};

// ---------------------------------------------------------------- matrix-free operator
// lattice blocks of the tiled shared-element-matrix operator (gpz_matfree.cu, k_mf_hex27_gt)
struct GtArgs {
  int mx, my, mz;            // elements per lattice direction
  int ntx, nty, ntz;         // blocks of 8 x 8 x 2 elements per direction
  int8_t off[27][3];         // doubled-lattice offset of each Q2 shape's connect
};

// Element records of the FP32 matrix-free elasticity operator (gpz_matfree.cu),
// a candidate of the mixed CG's SpMV autotuner.
struct MatFree {
  bool ready = false;
  int64_t nvol = 0, nface = 0;
  DBuf<float> vxyz, vlm, vdphi, vw;          // volume: corners [n][8][3], (lambda, mu) [n][2], tables
  DBuf<float> vgeo;                          // [n][10] affine elements: Jinv (row-major), |det J| (0: not affine)
  DBuf<int32_t> vrows;                       // [n][27] block row of each shape
  DBuf<float> fxyz, fphi, fdphi, fw;         // penalty faces
  DBuf<int32_t> frows;
  DBuf<double> energy;                       // the faces' share of p.q
  float big = 0.f;
  int grid_vol = 1, grid_face = 1, grid_tc = 1, grid_sf = 1;
  bool sf_ready = false;                     // the sum-factorised tables of the volume bucket were built
  DBuf<float> sf_tab;                        // 1D Lagrange values / derivatives, weights, corner gradients, Phi
  DBuf<int> sf_idx;
  // shared element matrix: every volume element has the same affine Jacobian,
  // so K_e = mu_e Khat; Khat (81 x 81, for mu = 1) split into TF32 hi / lo in
  // the tensor-core operand layout
  bool gm_ready = false;
  int grid_gm = 1;
  DBuf<float> gm_b;                          // [2][96 x 88] hi, lo (K-major core matrices)
  DBuf<double> gm_ref;                       // element 0's Jinv (9) and |det J|
  DBuf<int> gm_flag;
  // the same operator over lattice blocks (the translated elements fill a lattice of their edge vectors)
  bool gt_ready = false;
  int grid_gt = 1;
  GtArgs gt{};
  DBuf<int32_t> gt_nmap;                     // [(2 mx + 1)(2 my + 1)(2 mz + 1)] block row of each lattice connect
  DBuf<float> gt_emu;                        // [mx my mz] mu of the element of each lattice cell (-1: none)
  DBuf<uint8_t> gt_face;                     // [block rows] 1 on a penalty face
};

// scalar shared element matrix (3D Q2 Darcy / Poisson on translated grids):
// K_e = k_e Khat, Khat (27 x 27, coefficient 1) split into TF32 hi / lo
struct MatFree1 {
  bool ready = false;
  int64_t nvol = 0, nface = 0;
  int ntab = 0, grid = 1;
  DBuf<int32_t> vrows;                       // [ntile * 128][27] equations, -1 padding
  DBuf<float> vcoef;                         // [ntile * 128] element coefficient (k, or 1)
  DBuf<float> b;                             // [2][32 x 32] Khat hi, lo (K-major core matrices)
  DBuf<float> fxyz, ftabs;                   // penalty faces: corners, stacked per-bucket tables
  DBuf<int32_t> frows;
  DBuf<uint8_t> ftab;                        // table of each face
  DBuf<double> energy;
  float big = 0.f;
};

// ---------------------------------------------------------------- two-level preconditioner
// Additive two-level block Jacobi for uniform Q2 hex grids (every volume
// element a translate of one axis-aligned box): M = B^-1 + P Ac^-1 P^T with B
// the 3x3 connect blocks, P the trilinear interpolation from a coarse grid of
// m^3 boxes (s^3 fine elements each) to the vertex connects, Ac = P^T A P the
// Galerkin coarse matrix (from the vertex block of the element matrix, exact for
// the hierarchical basis: its vertex functions are the trilinear ones), coarse
// nodes whose functions touch a penalty-Dirichlet equation removed.
struct TwoLevel {
  bool ready = false;                        // geometry part built for the current mesh
  bool have_inv = false;                     // coarse inverse of the current assembly
  int target = 8;                            // coarse boxes per direction asked for
  int64_t lx[3] = {0, 0, 0};                 // fine lattice cells per direction
  int s = 0;                                 // fine cells per coarse box (every direction)
  int m[3] = {0, 0, 0};                      // coarse boxes per direction
  int64_t nnode = 0, nc = 0, ncell = 0, nfixed = 0;
  double mufac = 0.0, E0 = 1.0;              // mu_e = coef_e * mufac (E0 without coefficients)
  DBuf<int32_t> vtx_eq;                      // [(lx+1)(ly+1)(lz+1)] first equation of the vertex, -1 none
  DBuf<int32_t> brow_vtx;                    // [nbrow] lattice vertex of a vertex block row, -1 otherwise
  DBuf<int32_t> cell_off, cell_el, el_sub;   // volume elements grouped by coarse box; sub position
  DBuf<double> tsub;                         // [s^3][24][24] P^T Khat_vv P for mu = 1
  DBuf<int32_t> cfix;                        // [nnode] 1: removed (touches a penalty equation)
  DBuf<double> ac;                           // [nc][nc] coarse matrix (FP64 sums)
  DBuf<float> ac32;                          // [nc][nc] its FP32 copy, then the inverse
  DBuf<float> acinv32;                       // [nc][ldc] (rows padded to 16 bytes)
  int64_t ldc = 0;
  DBuf<float> rc, zc, z32;                   // coarse residual / correction, preconditioned residual
  DBuf<float> boxpart;                       // [ncell][8 corners][3] the restriction's per-box sums
};

// ---------------------------------------------------------------- the context
// ---------------------------------------------------------------- exact-solution errors
// Error-rule tables of the volume buckets and the layout of the error points
// (gpz_error.cu); rebuilt when the exact-solution order or the mesh changes.
struct ErrorEval {
  struct Tab {
    int bucket = 0, nq = 0;
    DBuf<double> phi, dphi, w;               // [nq][nshape], [nq][dim][nshape], [nq]
  };
  int exact_order = -1;                      // -1: not prepared
  int nerr = 0;                              // norms per element (3; 6 with a Darcy material)
  int64_t npts = 0;
  std::vector<Tab *> tabs;
  std::vector<int64_t> h_pt_off;             // [nel+1] first error point of each element
  DBuf<int64_t> pt_off;
  DBuf<double> xyz, uex, duex, sol, el;      // points, exact values [npts][nstate], gradients [npts][3][nstate]
  ErrorEval() = default;
  ErrorEval(const ErrorEval &) = delete;
  ErrorEval &operator=(const ErrorEval &) = delete;
  ~ErrorEval();
  void reset();
};

struct Ctx {
  int device = 0;
  std::atomic<int> killed{0};  // gpz_set_killed; read between batches of device work
  cudaStream_t stream = nullptr;
  std::string last_error;
  int64_t launches = 0;

  // mesh
  bool have_mesh = false;
  int dim = 0, nstate = 1;
  int64_t nel = 0, nnodes = 0, nconnects = 0, neq = 0;  // neq: equations of the system (the solves' size)
  int64_t neq_mesh = 0;                      // equations of the mesh (larger than neq under an equation filter)
  std::vector<gpz_material> mats;
  std::vector<gpz_bc> bcs;
  std::vector<int32_t> h_el_type, h_el_mat;
  std::vector<int64_t> h_el_conn;            // [nel][27]
  std::vector<int64_t> h_block_pos;
  std::vector<int32_t> h_block_size;
  DBuf<double> d_xyz, d_coef;
  DBuf<int64_t> d_el_nodes, d_el_conn, d_block_pos;
  DBuf<int32_t> d_el_type, d_el_mat, d_block_size, d_conn_order;
  std::vector<Bucket *> buckets;
  cudaGraphExec_t asm_graph = nullptr;       // captured assembly of the current pattern (replayed)
  // the bucket whose matrix the row-owner pass assembles (null: every bucket
  // scatters), its longest row, warps per CTA and whether its rows cover every
  // equation (then the matrix needs no clearing); set with the pattern
  Bucket *rp_bucket = nullptr;
  int rp_lmax = 0, rp_warps = 0, rp_grid = 0, rp_kref_sh = 0, rp_smem = 0;
  bool rp_full = false;
  int64_t asm_graph_launches = 0;
  std::string asm_tune_report;               // block-size timings of the hp element kernels
  int asm_queue = 0;                         // 1: persistent launches per bucket, 0: a launch per colour (the
                                             // default), -1: timed at the next assembly (gpz_assembly_mode)
  bool asm_mode_auto = false;                // the launch mode is autotuned (gpz_assembly_mode(-1))
  std::string asm_mode_report;               // the timings of the two launch modes
  std::string upload_report, bucket_report;  // host-side timings of the last mesh upload (ms)
  std::string pattern_report;                // stage timings of the last pattern build (ms)
  int ncolours = 0;
  DBuf<int> d_err;                           // device-side check flag

  // pattern (always the full CSR; the upper triangle is derived when requested)
  bool have_pattern = false;
  int user_sym = 0;
  int64_t nnz = 0, nnz_upper = 0;
  DBuf<int64_t> d_ia;                        // [neq+1]
  DBuf<int32_t> d_ja;                        // [nnz]
  DBuf<int64_t> d_ia_up;
  DBuf<int32_t> d_ja_up;
  DBuf<int64_t> d_diagpos;                   // [neq] slot of the diagonal entry
  DBuf<int64_t> d_offbase;                   // [nel] start of the element's offset table
  DBuf<int32_t> d_off;                       // element side-pair offsets inside a block row

  // TPZEquationFilter (StrMatrix/TPZEquationFilter.h): with an active set the
  // system is the mesh-level CSR restricted to the active rows and columns,
  // renumbered in increasing order; the element kernels assemble into the
  // mesh-level arrays, which a gather condenses
  struct EqFilter {
    bool active = false;
    std::vector<int64_t> h_act;              // sorted, unique (mesh numbering)
    DBuf<int64_t> act;                       // [neq] active equations
    DBuf<int64_t> dest;                      // [neq_mesh] condensed index, or -1
    DBuf<int64_t> keep;                      // [nnz] mesh-level slot of each condensed entry
    DBuf<int64_t> m_ia, m_diagpos;           // mesh-level full CSR, the assembly's target
    DBuf<int32_t> m_ja;
    DBuf<double> m_a;
    int64_t m_nnz = 0;
    DBuf<double> xfull;                      // a solution expanded to the mesh equations
  } flt;

  // values
  bool have_matrix = false;
  bool have_rhs = false;                     // load vector assembled (with or without the matrix)
  DBuf<double> d_a, d_f, d_dinv;
  DBuf<float> d_a32;                         // FP32 CSR copy for the inner solves
  bool have_a32 = false;
  // source of the FP32 values (gpz_fp32_elements): 0 rounded from the FP64 matrix, 1 element matrices
  // formed again in FP32 (3xTF32 tensor-core products on the hexes) into d_a32 at each mixed assembly
  int fp32_src = 0;
  bool a32_tensor = false;                   // d_a32 holds the FP32 element pass of the current assembly
  std::string fp32_report;
  // FP32 3x3 blocks for the mixed CG (instead of d_a32), in the layout the
  // SpMV autotuner measured fastest on this matrix
  bool have_bsr3 = false;
  int spmv32_tuned = -1;                     // variant the autotuner chose for the current pattern (-1: not yet)
  int64_t sell_window_tuned = 2048;          // its sliced-ELL sort window
  int spmv32_variant = 0;                    // 0 block CSR, 1 two rows in flight, 2 sliced ELL, 3 TMA-staged,
                                             // 4 upper triangle with float4 atomics
  uint32_t tma_vcap = 0, tma_ccap = 0;       // shared-memory stage capacities of the TMA-staged kernel
  int tma_grid = 1;
  std::string tune_report;
  std::string tune_cache;                    // file of autotuner choices (gpz_tuning_cache), empty: none
  int64_t nbrow = 0;
  DBuf<int64_t> d_bptr, d_uptr;              // block CSR and its upper triangle: [nbrow+1]
  DBuf<int32_t> d_ucol;
  DBuf<float> d_uval;
  DBuf<int32_t> d_bcol;
  DBuf<float> d_bval;                        // per block row: 9 planes of its blocks
  struct Sell {
    int64_t nslice = 0, plane = 0, window = 0;
    DBuf<int64_t> soff;                      // [nslice+1] first block of each slice
    DBuf<int32_t> slen, sperm, scol;         // slice lengths, rows of each slice, block columns
    DBuf<float> sval;                        // 9 planes of `plane` floats
  } sell;
  DBuf<double> d_bjinv;                      // block-Jacobi inverses [neq/3][9]
  DBuf<float> d_bjinv32, d_dinv32;           // FP32 preconditioners of the mixed CG
  bool have_bjinv = false;
  // variable-size block Jacobi (whole connect blocks of any size, or the
  // node-set blocks): block b holds equations vb_eq[vb_off[b] .. vb_off[b+1])
  // and its inverse (row-major) at vb_inv[vb_ioff[b]]; the FP32 copy of the
  // mixed CG is column-major.  Tile t (one CTA of the FP32 kernels) holds
  // blocks vb_tile[t] .. vb_tile[t+1], at most 256 equations.
  int vb_kind = 0;                           // 0 none, GPZ_PRECOND_BLOCK_JACOBI or GPZ_PRECOND_NODESET_JACOBI
  int64_t vb_nb = 0, vb_ntile = 0;
  int vb_maxn = 0;
  DBuf<int64_t> d_vb_off, d_vb_eq, d_vb_ioff, d_vb_tile;
  DBuf<int32_t> d_vb_eqblk, d_vb_eqloc;      // equation -> block, position inside it
  DBuf<int32_t> d_vb_posblk;                 // position in vb_eq -> block
  DBuf<double> d_vb_inv;
  DBuf<float> d_vb_inv32;
  bool have_vbinv = false;
  TwoLevel tl;
  int bj_bs = 0;

  SolverWork sw;
  bool have_solution = false;
  Learned ln;
  MatFree mf;
  MatFree1 mf1;
  ErrorEval er;

  ~Ctx();
};

// error.cu
void error_prepare(Ctx &c, int exact_order);
void error_points(Ctx &c, double *xyz_host);
void error_evaluate(Ctx &c, const double *sol_dev, const double *uex_host, const double *duex_host, double *errors,
                    double *el_host);
// pattern.cu
void build_pattern(Ctx &c);
void build_upper(Ctx &c);
void build_element_offsets(Ctx &c);
void condense_pattern(Ctx &c);  // restrict the system to the equation filter's active set
void filter_prepare(Ctx &c);    // the active set and the mesh -> condensed map on the device
void filter_gather(Ctx &c, const double *v_mesh, double *v_sys);
void filter_scatter(Ctx &c, const double *v_sys, double *v_mesh);
void filter_zero_inactive(Ctx &c, double *f_mesh);
void filter_values(Ctx &c);     // condensed values from the mesh-level ones (c.flt.keep)
// assemble.cu
void build_buckets(Ctx &c, const gpz_mesh_desc &d);
// greedy first-fit element colours (gpz_colour.cpp); nsides_of_type[type] sides per element type
int colour_mesh_elements(const gpz_mesh_desc &d, const int *nsides_of_type, int32_t *colours, int32_t *ncolours);
void assemble_fp64(Ctx &c);
void assemble_rhs(Ctx &c);
void make_fp32_copy(Ctx &c, int variant = -1);
void to_fp32(Ctx &c);
void assemble_fp32_elements(Ctx &c);  // FP32 element matrices into d_a32 (the tensor cores for the hexes)
// elem_tc.cu
bool elem_tc_supported(const Ctx &c, const Bucket *b);
void elem_tc_launch(Ctx &c, Bucket *b, int64_t e0, int64_t e1, cudaStream_t s);
void build_block_jacobi(Ctx &c);
// solver.cu
void spmv_device(Ctx &c, const double *x, double *y, double alpha, double beta, const double *yin);
int solve(Ctx &c, const gpz_solver_opts &o, gpz_solve_report &rep);
void spmv32_apply(Ctx &c, int variant, const double *hx, double *hy);
void precond_apply(Ctx &c, int precond, const double *hr, double *hz);
void base_block_apply(Ctx &c, const double *r, double *z);   // device vectors: z = B^-1 r (3x3 connect blocks)
void base_coarse_apply(Ctx &c, const double *r, double *z);  // device vectors: z = P Ac^-1 P^T r (two-level)
int collect_cg_pairs(Ctx &c, int npairs, double tol, int64_t max_iter, double *R, double *X, double *xstar,
                     int64_t *iters);
// matfree.cu
bool matfree_build(Ctx &c);
bool matfree1_build(Ctx &c);
void matfree1_spmv(Ctx &c, cudaStream_t s, const float *p, float *q);
int two_level_build(Ctx &c);     // geometry part (once per mesh); GPZ_OK or GPZ_E_INVALID when not a uniform grid
void two_level_assemble(Ctx &c); // coarse matrix and its inverse for the current assembly
void matfree_spmv(Ctx &c, cudaStream_t s, int mode);  // 0 CUDA cores, 1 tcgen05, 2 sum-factorised, 3 shared matrix,
                                                      // 4 shared matrix over lattice blocks
// learned.cu
void learned_prepare(Ctx &c);
void ensure_node_incidence(Ctx &c);                // features, scaling and factors F for the assembled system
// scan.cu
void exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t s, Ctx &c);
void check_device_flag(Ctx &c, const char *where);
// on-disk cache of the autotuners' choices (gpz_tune_cache.cpp): the key of the
// current mesh, pattern and device for one tuner; a stored choice or -1; a new one
std::string tune_key(Ctx &c, const char *tuner);
int tune_cache_lookup(const Ctx &c, const std::string &key);
void tune_cache_store(const Ctx &c, const std::string &key, int choice, const std::string &report);

// body(begin, end) over contiguous chunks of [0, n) on up to 16 host threads (one when n < min_chunk);
// an exception thrown by a chunk is rethrown in the caller after every thread has joined (the lowest chunk's)
template <class F>
void host_parallel(int64_t n, F &&body, int64_t min_chunk = 16384) {
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min(nt, 16u));
  if (n < 2 * min_chunk) nt = 1;
  if (nt == 1) {
    if (n > 0) body((int64_t)0, n);
    return;
  }
  std::vector<std::exception_ptr> err(nt);
  std::vector<std::thread> th;
  th.reserve(nt);
  for (unsigned t = 0; t < nt; t++)
    th.emplace_back([&, t]() {
      try {
        body(n * (int64_t)t / (int64_t)nt, n * (int64_t)(t + 1) / (int64_t)nt);
      } catch (...) {
        err[t] = std::current_exception();
      }
    });
  for (auto &x : th) x.join();
  for (auto &x : err)
    if (x) std::rethrow_exception(x);
}

inline int grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > 2147483647LL) g = 2147483647LL;
  return (int)g;
}

}  // namespace gpz

// the opaque handle of include/gpz.h
struct gpz_ctx {
  gpz::Ctx c;
};
