/*
 * gpz.h -- C ABI of the GB300 (sm_103a) implementation of the NeoPZ linear
 * FEM hot path: global assembly (TPZLinearAnalysis::Assemble through
 * TPZStructMatrix into TPZSYsmpMatrix / TPZFYsmpMatrix CSR) and the
 * iterative solve (TPZStepSolver CG / GMRES with Jacobi or block Jacobi).
 *
 * Plain C types only: pointers, sizes and POD structs.  Every call returns a
 * status code (GPZ_OK = 0, negative = error, positive = solver did not
 * converge) and never throws.  One context owns one CUDA stream and every
 * device buffer it allocates; a context is used by one host thread at a time.
 *
 * The reference interfaces each entry point replaces are cited beside it
 * (paths relative to the NeoPZ source tree).
 */
#ifndef GPZ_H
#define GPZ_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------
 * The reference aborts through DebugStop() (Common/pzerror.cpp:7-27); the C++
 * plugin classes map negative codes back to DebugStop(). */
#define GPZ_OK 0
#define GPZ_NOT_CONVERGED 1            /* CG/GMRES hit max_iter (cg.h:129-131 returns 1) */
#define GPZ_CANCELLED 2                /* gpz_set_killed(ctx, 1) was set: the call stopped (see gpz_set_killed) */
#define GPZ_E_INVALID (-1)             /* bad argument / inconsistent descriptor */
#define GPZ_E_CUDA (-2)                /* CUDA runtime error */
#define GPZ_E_NOMEM (-3)               /* device allocation failed */
#define GPZ_E_UNSUPPORTED_MATERIAL (-4)
#define GPZ_E_UNSUPPORTED_ELEMENT (-5)
#define GPZ_E_NOT_READY (-6)           /* call order violated (e.g. assemble before pattern) */
#define GPZ_E_DEVICE_CHECK (-7)        /* a kernel's own bounds / invariant check failed */
#define GPZ_E_NO_DEVICE (-8)           /* no CUDA device visible */
#define GPZ_E_BREAKDOWN (-9)           /* NaN / non-positive curvature in the Krylov recurrence */
#define GPZ_E_TOO_LARGE (-10)          /* problem exceeds the fixed scratch of gpz_cg_jacobi_noalloc */

/* ---- element types (TPZShapeLinear / TPZShapeQuad / TPZShapeCube) -------- */
#define GPZ_EL_LINE 1
#define GPZ_EL_QUAD 2
#define GPZ_EL_HEX 3

/* ---- material kinds ------------------------------------------------------ */
#define GPZ_MAT_POISSON 1   /* TPZMatPoisson::Contribute  Material/Poisson/TPZMatPoisson.cpp:19-43 */
#define GPZ_MAT_DARCY 2     /* TPZDarcyFlow::Contribute   Material/DarcyFlow/TPZDarcyFlow.cpp:19-47 */
#define GPZ_MAT_ELAST3D 3   /* TPZElasticity3D CODE3      Material/Elasticity/TPZElasticity3D.cpp:269-400 */

/* forcing functions the device evaluates at the physical integration point */
#define GPZ_F_NONE 0
#define GPZ_F_CONST 1       /* force[0..2] */
#define GPZ_F_SINPROD 2     /* force[0] * d pi^2 prod_k sin(pi x_k) */
#define GPZ_F_QUADRATIC 3   /* force[0] + force[1] |x|^2 (4 - 2x^2 - 2y^2 of UnitTest_PZ/TestMesh/TestError.cpp:62-68) */

typedef struct {
  int32_t kind;           /* GPZ_MAT_* */
  int32_t dim;            /* TPZMatPoisson/TPZDarcyFlow fDim */
  double scale;           /* TPZMatPoisson::fScale */
  double E, nu;           /* TPZElasticity3D fE, fPoisson (E overridden per element by el_coef) */
  double coef_const;      /* constant permeability (TPZIsotropicPermeability) */
  double force[3];
  int32_t forcing;        /* GPZ_F_* */
  int32_t forcing_porder; /* SetForcingFunction(f, pOrder): raises the integration order */
  double bignumber;       /* TPZMaterial::fBigNumber (Material/TPZMaterial.h:125) */
} gpz_material;

typedef struct {
  int32_t type;           /* 0 Dirichlet (penalty), 1 Neumann (TPZBndCondT types) */
  int32_t material;       /* index of the volume material in gpz_mesh_desc::mats */
  double val1[9];
  double val2[3];
} gpz_bc;

/* The computational mesh as the TPZCompMesh holds it after AutoBuild: one
 * entry per computational element (volume and boundary) in element order,
 * each with its corner nodes (TPZGeoEl::NodeIndex), preferred order and the
 * connect (sequence number) of every side (TPZCompEl::ConnectIndex ->
 * TPZConnect::SequenceNumber), plus the block structure (TPZBlock Position /
 * Size).  This is exactly what TPZCompMesh::ComputeElGraph and
 * TPZElementMatrix::ComputeDestinationIndices (Mesh/pzelmat.cpp:37-96) read. */
typedef struct {
  int32_t dim;              /* 1, 2 or 3 */
  int32_t nstate;           /* 1 (scalar) or 3 (elasticity) */
  int64_t nnodes;
  const double *node_xyz;   /* [nnodes][3] */
  int64_t nel;
  const int32_t *el_type;   /* GPZ_EL_* */
  const int32_t *el_mat;    /* >= 0: volume material index; < 0: -(bc index) - 1 */
  const int64_t *el_nodes;  /* [nel][8] corner node indices (unused slots -1) */
  const int32_t *el_order;  /* [nel] preferred interpolation order (fPreferredOrder) */
  const int64_t *el_conn;   /* [nel][27] connect sequence number of each side */
  const double *el_coef;    /* [nel] per-element permeability / Young modulus, or NULL */
  int64_t nconnects;
  const int32_t *conn_order;/* [nconnects] TPZConnect::Order */
  const int64_t *block_pos; /* [nconnects] TPZBlock::Position */
  const int32_t *block_size;/* [nconnects] TPZBlock::Size = NShape * NState */
  int64_t neq;
  int32_t nmat;
  const gpz_material *mats;
  int32_t nbc;
  const gpz_bc *bcs;
} gpz_mesh_desc;

typedef struct gpz_ctx gpz_ctx;

/* ---- context ------------------------------------------------------------- */
int gpz_ctx_create(gpz_ctx **out, int device);
int gpz_ctx_destroy(gpz_ctx *ctx);
const char *gpz_get_error_string(int code);
const char *gpz_last_error_detail(gpz_ctx *ctx);
/* The CUDA stream (cudaStream_t) every call of this context is ordered on. */
void *gpz_ctx_stream(gpz_ctx *ctx);
/* Number of kernels this context has launched since creation (graph nodes count). */
int64_t gpz_kernel_launches(gpz_ctx *ctx);

/* ---- mesh ---------------------------------------------------------------
 * Replaces the host-side extraction of TPZStructMatrix::Assemble: copies the
 * element / connect / block arrays to the device, builds the element buckets
 * (type, order signature, material) and the atomic-free element colouring
 * (TPZStructMatrix::ComputeElementColors, StrMatrix/TPZStructMatrix.cpp:104-161). */
int gpz_mesh_upload(gpz_ctx *ctx, const gpz_mesh_desc *desc);

/* ---- bandwidth / profile reduction ------------------------------------------
 * Replaces TPZSloanRenumbering::Resequence (External/TPZSloanRenumbering.cpp:
 * 23-175), the renumbering TPZAnalysis::OptimizeBandwidth applies before
 * assembling (Analysis/TPZAnalysis.cpp:228-300), with the same permutation.
 * Host code: the algorithm is one sequential greedy front; it needs no context
 * and no GPU.  Inputs are TPZCompMesh::ComputeElGraph's lists
 * (Mesh/pzcmesh.cpp:1214-1262): elgraphindex[nel+1] offsets into elgraph, the
 * independent connect sequence numbers of each element, nnodes of them.
 * Outputs: perm_gather[old sequence number] = new one (the vector
 * TPZCompMesh::Permute takes) and perm_scatter[k] = the connect numbered k.
 * GPZ_E_INVALID for an index out of range or a graph that is not connected
 * (the reference stops there as well); nnodes = 0 returns GPZ_OK untouched. */
int gpz_sloan_resequence(int64_t nnodes, int64_t nel, const int64_t *elgraphindex, const int64_t *elgraph,
                         int64_t *perm_gather, int64_t *perm_scatter);

/* ---- element colouring of the atomic-free scatter --------------------------------
 * The colouring gpz_mesh_upload gives the elements (the idea of
 * TPZStructMatrix::ComputeElementColors, StrMatrix/TPZStructMatrix.cpp:104-161):
 * greedy first fit in element order; elements sharing a non-empty connect get
 * different colours, so one colour's elements write disjoint rows and CSR
 * slots and the assembly launches one colour at a time without atomics.
 * Host code, no context and no GPU.  Inputs: ComputeElGraph's lists as for
 * gpz_sloan_resequence (the connects of every element) and the connects'
 * block sizes (NShape x NState; empty connects impose nothing).  Outputs:
 * colours[nel], *ncolours.  GPZ_E_INVALID for a connect out of range or more
 * than 64 colours. */
int gpz_element_colours(int64_t nel, const int64_t *elgraphindex, const int64_t *elgraph, int64_t nconnects,
                        const int64_t *block_size, int32_t *colours, int32_t *ncolours);

/* ---- node-set blocks of the block-Jacobi preconditioner ----------------------
 * Replaces the block construction of TPZAnalysis::BuildPreconditioner(
 * EBlockJacobi, overlap = false) (Analysis/TPZAnalysis.cpp:1008-1085):
 * TPZNodesetCompute::AnalyseGraph + BuildNodeGraph + ExpandGraph + ColorGraph
 * (External/tpznodesetcompute.cpp:47-209, 528-607) over the node graph of
 * TPZRenumbering::ConvertGraph.  Host code, no context and no GPU.  Inputs:
 * ComputeElGraph's lists as for gpz_sloan_resequence (nnodes connects), and the
 * mesh's TPZBlock: block_position / block_size of every connect, neq equations.
 * Outputs, in the reference's order: nblocks equation blocks,
 * blockindex[nblocks+1] offsets into blockeqs (capacities: nnodes + 1 and the
 * sum of block_size), the blocks' colours (colors[nblocks], ncolors; blocks of
 * disjoint connects never clash, so ncolors = 1), and, if non-NULL, every
 * connect's sequence number and level (fSeqNumber / fLevel, nnodes each).
 * GPZ_E_INVALID for an index or block out of range. */
int gpz_nodeset_blocks(int64_t nnodes, int64_t nel, const int64_t *elgraphindex, const int64_t *elgraph,
                       const int64_t *block_position, const int64_t *block_size, int64_t neq,
                       int64_t *blockindex, int64_t *blockeqs, int64_t *nblocks, int *colors, int *ncolors,
                       int64_t *seqnum, int *level);

/* ---- equation filter ----------------------------------------------------
 * Replaces TPZEquationFilter::SetActiveEquations / Reset
 * (StrMatrix/TPZEquationFilter.h) on the structural matrix.  Call after
 * gpz_mesh_upload and before gpz_pattern_build (a new filter drops the
 * pattern and the values).  active: mesh equation numbers, any order,
 * duplicates removed; nactive < 0 resets the filter (all equations active).
 * Under an active set of n equations, as the reference does:
 *   - the pattern, matrix, gpz_spmv and gpz_solve are over the n active
 *     equations, renumbered in increasing mesh order (the mesh-level pattern
 *     restricted to active rows and columns, StrMatrix/TPZSSpStructMatrix.cpp:
 *     49-193 / TPZSpStructMatrix.cpp:53-190; element contributions to an
 *     inactive row or column are dropped, TPZEquationFilter::Filter);
 *   - the load vector (gpz_rhs_download) keeps the mesh's size with zeros at
 *     the inactive equations (TPZEquationFilter::Scatter after the condensed
 *     assembly, StrMatrix/pzstrmatrixor.cpp:43-71); gpz_solve with b = NULL
 *     gathers its active entries (TPZLinearAnalysis::SolveT,
 *     Analysis/TPZLinearAnalysis.cpp:194);
 *   - gpz_error_evaluate with sol = NULL scatters the device solution to the
 *     mesh equations with zeros elsewhere (TPZLinearAnalysis.cpp:197); a host
 *     sol has the mesh's size.
 * The 3x3-block FP32 layouts, the matrix-free operators, block Jacobi and the
 * learned preconditioner need whole connect blocks: under a filter the mixed
 * CG uses the FP32 CSR copy, and block Jacobi and gpz_learned_* return
 * GPZ_E_INVALID.  gpz_pattern_upload is not available under a filter. */
int gpz_equation_filter(gpz_ctx *ctx, int64_t nactive, const int64_t *active);

/* ---- sparsity pattern ----------------------------------------------------
 * Replaces TPZSSpStructMatrix::Create / SetupMatrixData (sym = 1, upper
 * triangle; StrMatrix/TPZSSpStructMatrix.cpp:31-193) and
 * TPZSpStructMatrix::SetupMatrixData (sym = 0, full rows;
 * StrMatrix/TPZSpStructMatrix.cpp:53-190), built on the device from the
 * element graph (TPZCompMesh::ComputeElGraph, TPZRenumbering::ConvertGraph).
 * Returns the number of stored entries in *nnz_out. */
int gpz_pattern_build(gpz_ctx *ctx, int sym, int64_t *nnz_out);
/* Alternatively adopt a host pattern (IA, JA as TPZSYsmpMatrix::IA()/JA()). */
int gpz_pattern_upload(gpz_ctx *ctx, int sym, int64_t neq, const int64_t *IA, const int64_t *JA);
/* Stored entries of the full and of the upper-triangular pattern. */
int gpz_pattern_info(gpz_ctx *ctx, int64_t *nnz_full, int64_t *nnz_upper);
/* Copy the device pattern to the host (IA: neq+1, JA: nnz, as int64). */
int gpz_pattern_download(gpz_ctx *ctx, int64_t *IA, int64_t *JA);

/* ---- assembly -------------------------------------------------------------
 * Replaces TPZStructMatrixOR::Assemble (StrMatrix/pzstrmatrixor.cpp:43-71,106-365)
 * with its TPZCompEl::CalcStiff (Mesh/pzinterpolationspace.cpp:403-473),
 * TPZMaterial::Contribute/ContributeBC, TPZSYsmpMatrix::AddKel
 * (Matrix/pzsysmp.cpp:369-411; entries |v| < 1e-12 skipped as IsZero does),
 * TPZFMatrix::AddFel and TPZSYsmpMatrix::ComputeDiagonal (EndCreateAssemble).
 * precision: GPZ_PREC_FP64 (the parity path) or GPZ_PREC_MIXED (FP64 matrix for
 * the true residual plus an FP32 copy built for the inner solves). */
#define GPZ_PREC_FP64 0
#define GPZ_PREC_MIXED 1
int gpz_assemble(gpz_ctx *ctx, int precision);
/* Source of the FP32 values that GPZ_PREC_MIXED gives the inner solves (no
 * counterpart in the reference, whose matrices have one precision):
 * GPZ_FP32_ROUNDED (the default) rounds the FP64 matrix; GPZ_FP32_ELEMENTS
 * forms every element matrix again in FP32 -- the volume hexes as one tcgen05
 * GEMM per element (the gradient Gram X X^T, X[(i,a)][q] = sqrt(w|J|) dphi_a/dx_i,
 * 3xTF32 split, FP32 accumulation; the material's blocks formed from it as
 * TPZMatPoisson / TPZDarcyFlow / TPZElasticity3D::Contribute form them), the
 * other element types by the FP64 element kernel with an FP32 scatter -- and
 * adds them into the FP32 CSR.  The FP64 matrix (true residual, parity) is
 * assembled either way; under an equation filter the values are rounded.  The
 * assembly report's "fp32_elements" gives the element counts and the pass's time. */
#define GPZ_FP32_ROUNDED 0
#define GPZ_FP32_ELEMENTS 1
int gpz_fp32_elements(gpz_ctx *ctx, int source);
/* The FP32 full-CSR values (nnz floats) of the last GPZ_PREC_MIXED assembly:
 * the scalar problems' FP32 CSR, or the FP32 element pass's values.
 * GPZ_E_NOT_READY when the FP32 operator holds its values in another layout. */
int gpz_matrix_fp32_download(gpz_ctx *ctx, float *A);
/* Download the assembled values (nnz doubles) and the load vector (neq). */
/* Load vector only (TPZStructMatrix::Assemble(rhs, gui), StrMatrix/pzstrmatrixor.cpp:75-103;
 * TPZLinearAnalysis::AssembleResidual): the same element kernels stopped
 * before the element matrix; needs the mesh, not the pattern.  Read it with
 * gpz_rhs_download. */
int gpz_assemble_rhs(gpz_ctx *ctx);
int gpz_matrix_download(gpz_ctx *ctx, double *A);
int gpz_rhs_download(gpz_ctx *ctx, double *F);
/* Overwrite the device load vector (a user right-hand side). */
int gpz_rhs_upload(gpz_ctx *ctx, const double *F);

/* ---- SpMV -----------------------------------------------------------------
 * TPZSYsmpMatrix::MultAdd / TPZFYsmpMatrix::MultAdd (Matrix/pzsysmp.cpp:189-232,
 * Matrix/pzysmp.cpp:527-624):  z = alpha A x + beta y, host vectors. */
int gpz_spmv(gpz_ctx *ctx, double alpha, const double *x, double beta, const double *y, double *z);

/* y = A32 x with the FP32 operator of the mixed solvers (host FP64 vectors):
 * the layout the SpMV autotuner chose, or `variant` (GPZ solver option
 * spmv_variant, 0..8 or 10) for 3-state problems; the FP32 CSR copy, or 9, otherwise. */
int gpz_spmv_fp32(gpz_ctx *ctx, int variant, const double *x, double *y);

/* ---- cancellation ---------------------------------------------------------
 * Replaces TPZGuiInterface::SetKilled / AmIKilled (Common/TPZGuiInterface.cpp:
 * 80-87).  The reference polls AmIKilled before it starts the assembly threads
 * and after each CalcStiff (StrMatrix/pzstrmatrixor.cpp:182,490) and returns
 * silently.  Here gpz_assemble / gpz_assemble_rhs return GPZ_CANCELLED without
 * assembling while the flag is set, and every iterative solve polls it between
 * batches of iterations (CUDA-graph launches) and returns GPZ_CANCELLED with the
 * last completed batch's iterate and report.  The flag stays set until cleared
 * with gpz_set_killed(ctx, 0).  This is the one entry point that may be called
 * from another thread while a call on the same context runs: it only stores
 * the flag (no CUDA call). */
int gpz_set_killed(gpz_ctx *ctx, int killed);

/* ---- solve ----------------------------------------------------------------
 * TPZStepSolver::Solve (Solvers/pzstepsolver.cpp:64-169) with SetCG / SetGMRES
 * and a Jacobi (SetJacobi(1,0,0)) or block-Jacobi preconditioner. */
#define GPZ_SOLVER_CG 1            /* Solvers/LinearSolvers/cg.h:29-132 */
#define GPZ_SOLVER_GMRES 2         /* Solvers/LinearSolvers/gmres.h:68-168 */
#define GPZ_SOLVER_MIXED_CG 3      /* FP32-value SpMV CG, FP64 x/dots, reliable FP64 residual updates */
#define GPZ_SOLVER_LEARNED_FCG 4   /* flexible CG with the learned preconditioner (gpz_learned_*), FP64 */
#define GPZ_SOLVER_LEARNED_MIXED_FCG 5 /* the same with FP32-value SpMV, FP64 x/r/dots and true-residual
                                          replacement (reliable_delta); scalar problems */
#define GPZ_SOLVER_JACOBI 6        /* the stationary Jacobi iteration, SetJacobi as the solver
                                      (Solvers/pzstepsolver.cpp:94-98): TPZMatrix::SolveJacobi
                                      (Matrix/pzmatrix.cpp:643-667) for a symmetric pattern, the
                                      TPZFYsmpMatrix override (Matrix/pzysmp.cpp:725-781, first sweep
                                      always made) for a full one; tol is on the ABSOLUTE ||b - A x||,
                                      iterations = sweeps performed; precond must be 0 or JACOBI */
#define GPZ_PRECOND_JACOBI 1       /* TPZMatrix::SolveJacobi, one sweep (Matrix/pzmatrix.cpp:643-667) */
#define GPZ_PRECOND_BLOCK_JACOBI 2 /* connect blocks, TPZBlockDiagonal (Matrix/pzblockdiag.h:21):
                                      TPZAnalysis::BuildPreconditioner(EBlockJacobi, overlap = true)
                                      (Analysis/TPZAnalysis.cpp:1073-1080) with its
                                      TPZBlockDiagonalStructMatrix connect blocks, one block of
                                      NShape x NState equations per connect.  CG and the mixed CG
                                      invert each whole connect block (3x3 blocks when every
                                      connect carries one shape, p <= 2; blocks of 6, 12, 24 ...
                                      for the connects of order 3).  GMRES splits a larger connect
                                      block into its shapes' 3x3 blocks */
#define GPZ_PRECOND_NODESET_JACOBI 3 /* node-set blocks: TPZAnalysis::BuildPreconditioner(EBlockJacobi,
                                      overlap = false) (Analysis/TPZAnalysis.cpp:1008-1085,1093-1107):
                                      the blocks of gpz_nodeset_blocks (TPZNodesetCompute) of the
                                      mesh's element graph, each inverted on the device (Gauss-Jordan
                                      without pivoting, the TPZSparseBlockDiagonal LU without
                                      pivoting up to rounding); CG and the mixed CG only */

#define GPZ_PRECOND_TWO_LEVEL 4    /* mixed CG only; no counterpart among BuildPreconditioner's options (the
                                      reference's multigrid is TPZMGSolver, Solvers/Multigrid/pzmgsolver.cpp,
                                      over a TPZTransfer between meshes).  Additive two-level block Jacobi:
                                      M = B^-1 + P Ac^-1 P^T with B the 3x3 connect blocks of
                                      GPZ_PRECOND_BLOCK_JACOBI, P the trilinear interpolation from a coarse
                                      grid of boxes (each s^3 fine elements; gpz_two_level_config) to the
                                      vertex connects, Ac = P^T A P the Galerkin coarse matrix (coarse
                                      nodes touching a penalty-Dirichlet equation removed), inverted on
                                      the device.  Needs one uniform grid of axis-aligned Q2 hex
                                      elasticity elements (every element a translate of one box) and at
                                      most 3000 coarse equations; GPZ_E_INVALID otherwise. */

typedef struct {
  int32_t solver;          /* GPZ_SOLVER_* */
  int32_t precond;         /* GPZ_PRECOND_*; for the learned solvers the base under the correction
                              (GPZ_PRECOND_JACOBI, or BLOCK_JACOBI / TWO_LEVEL with the mixed one) */
  int64_t max_iter;
  double tol;              /* stop when ||r||/||b|| <= tol (recursive r, as cg.h:100);
                              GPZ_SOLVER_JACOBI: when ||b - A x|| <= tol */
  int32_t gmres_krylov;    /* GMRES restart length (SetGMRES numvectors) */
  int32_t check_every;     /* iterations per graph launch between convergence checks */
  double reliable_delta;   /* mixed CG: true-residual update when ||r|| < delta * max||r|| */
  int32_t use_graph;       /* capture the iteration batch in a CUDA graph */
  int32_t from_current;    /* FromCurrent: start from x instead of zero */
  int32_t spmv_variant;    /* mixed CG: -1 = autotuned; 0 block CSR, 1 two rows in flight, 2 sliced ELL,
                              3 TMA-staged block CSR, 4 upper triangle with float4 atomics,
                              5 matrix-free elements (uniform Q2 hex elasticity + penalty faces),
                              6 the same on the tensor cores (tcgen05, 3xTF32),
                              7 the same sum-factorised on Lagrange nodal values,
                              8 the same when every element has one affine Jacobian (uniform grid):
                                K_e = mu_e Khat as one tcgen05 3xTF32 GEMM per tile of elements;
                              10 8 over lattice blocks of 8 x 8 x 2 elements (the translated elements fill
                                a lattice): the block's connect values and results in shared memory, plain
                                stores inside the block, reductions on its faces;
                              scalar problems (Poisson, Darcy): 0 the FP32 CSR copy, 9 the scalar
                                counterpart of 8 (3D Q2 hexes, K_e = k_e Khat, penalty faces) */
} gpz_solver_opts;

typedef struct {
  int64_t iterations;      /* fNumIterations */
  double resid;            /* final recursive ||r||/||b|| (fTol on return) */
  double true_resid;       /* ||b - A x|| / ||b|| recomputed in FP64 on the device */
  double seconds;          /* device time of the solve */
  int64_t spmv_fp64;       /* FP64 SpMVs performed */
  int64_t spmv_fp32;       /* FP32-value SpMVs performed */
  int64_t reliable_updates;
  int64_t restarts;        /* mixed CG: direction restarts at residual replacement */
} gpz_solve_report;

/* z = M r for one preconditioner of the assembled system, as the solvers apply
 * it: TPZStepSolver::Solve on the preconditioner step solver
 * (Solvers/pzstepsolver.cpp:64-169; Jacobi, the connect / node-set block
 * Jacobi of BuildPreconditioner, FP64) or the mixed CG's two-level
 * preconditioner (FP32).  Host vectors of the system's size. */
int gpz_precond_apply(gpz_ctx *ctx, int precond, const double *r, double *z);

/* Two-level preconditioner: coarse boxes per direction asked for (default 8;
 * the grid takes the divisor s of its cell counts that comes closest), and
 * after a two-level solve its shape: info[9] = fine cells per direction (3),
 * s, coarse boxes per direction (3), coarse equations, removed coarse nodes.
 * No counterpart in the reference. */
int gpz_two_level_config(gpz_ctx *ctx, int coarse_boxes);
int gpz_two_level_info(gpz_ctx *ctx, int64_t *info);

/* b: host load vector (NULL = use the assembled device rhs); x: host solution
 * (in: initial guess if from_current, out: solution; may be NULL to keep the
 * solution on the device only). */
int gpz_solve(gpz_ctx *ctx, const gpz_solver_opts *opts, const double *b, double *x, gpz_solve_report *rep);
/* Download the device solution of the last solve. */
int gpz_solution_download(gpz_ctx *ctx, double *x);

/* ---- measurement -----------------------------------------------------------
 * Average device time (CUDA events on the context stream) of one launch of a
 * hot kernel over `reps` back-to-back launches on the assembled system:
 * GPZ_KERNEL_SPMV_FP64 / GPZ_KERNEL_SPMV_FP32 (the q = A p kernel of the CG
 * iteration) and GPZ_KERNEL_ASSEMBLE (one full FP64 assembly). */
#define GPZ_KERNEL_SPMV_FP64 1
#define GPZ_KERNEL_SPMV_FP32 2
#define GPZ_KERNEL_ASSEMBLE 3
int gpz_time_kernel(gpz_ctx *ctx, int which, int reps, double *ms_per_launch);
/* ---- exact-solution error norms -----------------------------------------
 * Replace TPZAnalysis::PostProcessError (Analysis/TPZAnalysis.cpp:625-650) ->
 * TPZCompMesh::EvaluateError (Mesh/pzcmesh.cpp:1497-1551) ->
 * TPZInterpolationSpace::EvaluateError (Mesh/pzinterpolationspace.cpp:1108-1200).
 * The reference calls the exact-solution function set by SetExact(f, order)
 * at every integration point; across this ABI the exact solution is data:
 *
 *   gpz_error_points(ctx, order, &n, NULL);   -> n, the number of points
 *   gpz_error_points(ctx, order, &n, xyz);    -> xyz[n][3], TPZGeoEl::X of each
 *       point of every volume element's error rule (element order, rule order)
 *   ... the caller evaluates u[n][nstate] and du[n][3][nstate] there
 *       (du[p][d][s] = d u_s / d x_d, the TPZFMatrix dsol layout) ...
 *   gpz_error_evaluate(ctx, order, sol, u, du, &nerr, errors, el_errors);
 *
 * order is the exact solution's polynomial order (SetExactSol's pOrder): the
 * element rule is raised to it as EvaluateError does.  sol: host solution
 * [neq], or NULL for the last gpz_solve solution kept on the device.
 * errors[nerr] receives the mesh norms sqrt(sum_e err_e^2) (nerr = 3:
 * TPZMatPoisson / TPZElasticity3D [energy or H1, L2, H1 semi-norm]; 6 with a
 * TPZDarcyFlow material, which adds the flux components), el_errors
 * [nel][nerr] (may be NULL) the per-element errors EvaluateError stores
 * (zero rows for boundary elements). */
int gpz_error_points(gpz_ctx *ctx, int32_t exact_order, int64_t *npoints, double *xyz);
int gpz_error_evaluate(gpz_ctx *ctx, int32_t exact_order, const double *sol, const double *u_exact,
                       const double *du_exact, int32_t *nerrors, double *errors, double *el_errors);

/* JSON text of the SpMV autotuner's measurements (ms per launch of every
 * candidate layout / kernel of the mixed CG) for the assembled system. */
int gpz_tuning_report(gpz_ctx *ctx, char *buf, int64_t len);
/* On-disk cache of the autotuners' choices (the FP32 operator layout of the
 * mixed solves, the block size of the hp element kernels): with a file set, a
 * pattern whose key (tuner, device, sizes, a hash of the mesh connectivity,
 * tuner version) is in the file takes the stored choice instead of timing the
 * candidates, and a new measurement is appended (JSON lines; the reports then
 * carry "cached": true).  NULL: no cache (the default).  An unreadable or
 * unwritable file only means the tuners measure again. */
int gpz_tuning_cache(gpz_ctx *ctx, const char *path);
/* Launch mode of the element kernels: -1 autotuned at the first assembly of a
 * mesh (both timed on one full assembly, the faster kept), 0 a launch per
 * element bucket and colour (a CTA per element; the default), 1 one persistent
 * launch per bucket over all its colours: resident CTAs take elements from a
 * work counter in colour order, an element of colour c waits (bounded) until
 * every element of the earlier colours is done -- the OT scheduler of
 * TPZStructMatrixOT (StrMatrix/pzstrmatrixot.cpp:486-551) on the device.  The
 * matrices agree to the last bits (the order of the contributions of different
 * buckets to one entry differs). */
int gpz_assembly_mode(gpz_ctx *ctx, int mode);
/* JSON text of the element batching: uniform-order buckets (compile-time
 * kernels), hp classes (elements of uneven side orders sharing the table of
 * the full element of their largest order, one run-time kernel per class and
 * colour), colours, and the hp kernels' block-size autotuner timings (ms of one
 * assembly per candidate); the FP32 element pass, the mesh upload and pattern
 * stage timings; and "row_owner_pass": the bucket of hexes that are all
 * translates of one element (K_e = c_e K_1) whose matrix is assembled row by
 * row -- one warp per connect sums its elements' rows and writes the connect's
 * rows once -- before the other buckets scatter into it (its elements, the
 * longest row, warps per CTA, whether the matrix is cleared first), or null. */
int gpz_assembly_report(gpz_ctx *ctx, char *buf, int64_t len);

/* ---- coefficient update -------------------------------------------------
 * Replace the per-element coefficients (el_coef of gpz_mesh_desc) of the
 * uploaded mesh, keeping its numbering and pattern: the reference's loop of
 * re-assembling the same TPZCompMesh with new material data.  The matrix must
 * be assembled again afterwards. */
int gpz_mesh_set_coef(gpz_ctx *ctx, const double *el_coef);

/* ---- learned preconditioner ----------------------------------------------
 * No counterpart in the reference.  A symmetric positive definite
 * preconditioner M r = S (u + m .* sum_e Q_e^T F_e F_e^T Q_e (m .* u)),
 * u = S r, S = diag(A)^-1/2, m = 0 on penalty-Dirichlet equations, whose
 * per-element factors F_e (equations x rank) come from an element-to-node
 * message-passing network over log(el_coef) (3 layers, 32 channels), used by
 * GPZ_SOLVER_LEARNED_FCG (flexible CG; an iteration whose correction is not a
 * descent direction uses Jacobi).  The network is trained on the GPU on
 * residual / error pairs of the Jacobi-PCG iterates of assembled systems.
 * Needs one element type and one equation count for all volume elements. */
/* Build the element incidence of the uploaded mesh and random initial
 * parameters (rank 1..8 columns per element factor; seed of the init). */
int gpz_learned_init(gpz_ctx *ctx, int rank, uint64_t seed);
int gpz_learned_num_params(gpz_ctx *ctx, int64_t *n);
int gpz_learned_get_params(gpz_ctx *ctx, float *out, int64_t n);
int gpz_learned_set_params(gpz_ctx *ctx, const float *in, int64_t n);
/* Training pairs of the assembled system: Jacobi-PCG to `tol` gives x*, an
 * identical second run samples npairs (r_k, x* - x_k) spread over its
 * iterations; cg_iterations receives the Jacobi-PCG iteration count. */
int gpz_learned_collect(gpz_ctx *ctx, int npairs, double tol, int64_t max_iter, int64_t *cg_iterations);
/* Training pairs given by the caller: r[npairs][neq], e[npairs][neq] (host). */
int gpz_learned_set_pairs(gpz_ctx *ctx, int npairs, const double *r, const double *e);
/* Loss mean_j (M r_j - e_j)^T A (M r_j - e_j) / e_j^T A e_j over the
 * non-Dirichlet equations, and (grad != NULL) its gradient w.r.t. the n
 * parameters. */
int gpz_learned_loss_grad(gpz_ctx *ctx, double *loss, float *grad, int64_t n);
/* `steps` Adam steps (learning rate lr) on the current pairs; the losses
 * before the first and the last step. */
int gpz_learned_train(gpz_ctx *ctx, int steps, double lr, double *loss_first, double *loss_last);
/* Base preconditioner the correction is trained on and solved with (the
 * solver's opts.precond): 0 / GPZ_PRECOND_JACOBI (M r = S(alpha u + ...) as
 * above), GPZ_PRECOND_BLOCK_JACOBI (alpha B^-1 r with the 3x3 connect blocks
 * in place of alpha D^-1 r) or GPZ_PRECOND_TWO_LEVEL (the same plus the
 * coarse correction P Ac^-1 P^T r, which the training takes off the error
 * targets).  Clears the training pairs: collect or set them after this call. */
int gpz_learned_set_base(gpz_ctx *ctx, int precond);

/* ---- allocation-free solve -------------------------------------------------
 * No counterpart in the reference (its CG allocates its work vectors on every
 * call).  Jacobi-preconditioned FP64 CG with the algorithm of gpz_solve's
 * GPZ_SOLVER_CG / GPZ_PRECOND_JACOBI (Solvers/LinearSolvers/cg.h:29-132), zero
 * initial guess, on a caller-owned full CSR matrix (TPZFYsmpMatrix layout)
 * already on the device, for callers that may not allocate device memory
 * while they solve (an application that has handed all of HBM to its own
 * pool, or a loop that must not touch the allocator after start-up).
 *
 * It allocates nothing: its work vectors live in one fixed static device
 * array sized for GPZ_NOALLOC_MAX_EQ equations (about 8.4 MB per device);
 * larger systems return GPZ_E_TOO_LARGE.  The first call on a device looks the
 * array up (cudaGetSymbolAddress with that device current), which may make the
 * CUDA runtime load the library's device code: make that first call during
 * start-up, before any stream capture.  Every call on a device shares the
 * array, so calls must not overlap in time on one device (one after the
 * other, from any thread or stream, is fine).
 *
 * stream: cudaStream_t of the current device (NULL = legacy default stream;
 * a stream of another device returns GPZ_E_INVALID); d_ia[neq+1] (int64),
 * d_ja[nnz] (int32), d_a[nnz], d_b[neq], d_x[neq]: device pointers; x is
 * overwritten with the solution.  Every call blocks the calling host thread
 * until the solve has finished on `stream` (it reads the device's stop flag
 * every 32 iterations); iterations / resid (host, may be NULL) receive
 * fNumIterations and the final ||r||/||b||.  Bad row pointers or columns, or
 * a missing / zero diagonal, return GPZ_E_INVALID before the first iteration
 * and leave x unchanged. */
#define GPZ_NOALLOC_MAX_EQ 262144
int gpz_cg_jacobi_noalloc(void *stream, int64_t neq, int64_t nnz, const int64_t *d_ia, const int32_t *d_ja,
                          const double *d_a, const double *d_b, double *d_x, int64_t max_iter, double tol,
                          int64_t *iterations, double *resid);

#ifdef __cplusplus
}
#endif
#endif /* GPZ_H */
