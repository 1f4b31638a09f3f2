// C ABI entry points (include/gpz.h).  No exception crosses this boundary.
#include <chrono>
#include <algorithm>
#include <cstring>

#include "gpz_internal.h"
#include "gpz_shapes.h"

namespace gpz {
void solver_prepare(Ctx &c, bool mixed);
double time_spmv(Ctx &c, bool f32, int reps);

void drop_assembly_graph(Ctx &c) {
  if (c.asm_graph) cudaGraphExecDestroy(c.asm_graph);
  c.asm_graph = nullptr;
  c.rp_bucket = nullptr;  // chosen again, with the pattern, by the next assembly
}

Ctx::~Ctx() {
  drop_assembly_graph(*this);
  for (Bucket *b : buckets) delete b;
  buckets.clear();
}
}  // namespace gpz

using namespace gpz;


namespace {

template <class F>
int guarded(gpz_ctx *ctx, F &&f) {
  if (!ctx) return GPZ_E_INVALID;
  try {
    GPZ_CUDA_TRY(cudaSetDevice(ctx->c.device));
    int rc = f(ctx->c);
    return rc;
  } catch (const Error &e) {
    ctx->c.last_error = e.msg;
    if (e.code == GPZ_E_CUDA || e.code == GPZ_E_NOMEM) cudaGetLastError();  // clear a non-sticky error
    return e.code;
  } catch (const std::bad_alloc &) {
    ctx->c.last_error = "host allocation failed";
    return GPZ_E_NOMEM;
  } catch (...) {
    ctx->c.last_error = "unexpected host exception";
    return GPZ_E_INVALID;
  }
}

}  // namespace

extern "C" {

const char *gpz_get_error_string(int code) {
  switch (code) {
    case GPZ_OK: return "ok";
    case GPZ_NOT_CONVERGED: return "iterative solver did not converge within max_iter";
    case GPZ_CANCELLED: return "cancelled by gpz_set_killed";
    case GPZ_E_INVALID: return "invalid argument";
    case GPZ_E_CUDA: return "CUDA runtime error";
    case GPZ_E_NOMEM: return "device memory allocation failed";
    case GPZ_E_UNSUPPORTED_MATERIAL: return "material or boundary condition has no device implementation";
    case GPZ_E_UNSUPPORTED_ELEMENT: return "element type/order has no device kernel";
    case GPZ_E_NOT_READY: return "call order violated (mesh -> pattern -> assemble -> solve)";
    case GPZ_E_DEVICE_CHECK: return "a device-side bounds or invariant check failed";
    case GPZ_E_NO_DEVICE: return "no CUDA device";
    case GPZ_E_BREAKDOWN: return "Krylov breakdown (non-positive curvature or non-finite residual)";
    case GPZ_E_TOO_LARGE: return "system larger than GPZ_NOALLOC_MAX_EQ equations (fixed scratch of the allocation-free CG)";
    default: return "unknown status";
  }
}

int gpz_ctx_create(gpz_ctx **out, int device) {
  if (!out) return GPZ_E_INVALID;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return GPZ_E_NO_DEVICE;
  }
  if (device < 0 || device >= n) return GPZ_E_INVALID;
  gpz_ctx *ctx = new (std::nothrow) gpz_ctx();
  if (!ctx) return GPZ_E_NOMEM;
  ctx->c.device = device;
  int rc = guarded(ctx, [](Ctx &c) {
    GPZ_CUDA_TRY(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    c.d_err.alloc(1);
    c.d_err.zero(c.stream);
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return GPZ_OK;
  });
  if (rc != GPZ_OK) {
    delete ctx;
    return rc;
  }
  *out = ctx;
  return GPZ_OK;
}

int gpz_ctx_destroy(gpz_ctx *ctx) {
  if (!ctx) return GPZ_E_INVALID;
  cudaSetDevice(ctx->c.device);
  if (ctx->c.stream) cudaStreamSynchronize(ctx->c.stream);
  cudaStream_t s = ctx->c.stream;
  delete ctx;  // frees every device buffer
  if (s) cudaStreamDestroy(s);
  return GPZ_OK;
}

const char *gpz_last_error_detail(gpz_ctx *ctx) { return ctx ? ctx->c.last_error.c_str() : ""; }
void *gpz_ctx_stream(gpz_ctx *ctx) { return ctx ? (void *)ctx->c.stream : nullptr; }
int64_t gpz_kernel_launches(gpz_ctx *ctx) { return ctx ? ctx->c.launches : 0; }

int gpz_mesh_upload(gpz_ctx *ctx, const gpz_mesh_desc *d) {
  return guarded(ctx, [d](Ctx &c) {
    GPZ_REQUIRE(d, GPZ_E_INVALID, "null descriptor");
    GPZ_REQUIRE(d->dim >= 1 && d->dim <= 3, GPZ_E_INVALID, "dim");
    GPZ_REQUIRE(d->nstate == 1 || d->nstate == 3, GPZ_E_INVALID, "nstate");
    GPZ_REQUIRE(d->nel >= 0 && d->nnodes >= 0 && d->nconnects >= 0 && d->neq >= 0, GPZ_E_INVALID, "sizes");
    GPZ_REQUIRE(d->neq < INT32_MAX, GPZ_E_INVALID, "neq must fit 32-bit column indices");
    const auto t0 = std::chrono::steady_clock::now();
    GPZ_REQUIRE(d->node_xyz && d->el_type && d->el_mat && d->el_nodes && d->el_order && d->el_conn &&
                    d->conn_order && d->block_pos && d->block_size && (d->nmat == 0 || d->mats),
                GPZ_E_INVALID, "null array");
    // TPZBlock positions are consecutive in sequence-number order; the pattern
    // builder relies on it (columns sorted by connect = sorted by equation).
    // (checked on the host threads; the first failing chunk's message is the one reported)
    GPZ_REQUIRE(d->nconnects == 0 || d->block_pos[0] == 0, GPZ_E_INVALID,
                "block positions must be consecutive in connect order");
    GPZ_REQUIRE(d->nconnects > 0 || d->neq == 0, GPZ_E_INVALID, "sum of block sizes != neq");
    host_parallel(d->nconnects, [&](int64_t i0, int64_t i1) {
      for (int64_t i = i0; i < i1; i++) {
        GPZ_REQUIRE(d->block_size[i] >= 0, GPZ_E_INVALID, "block size");
        const int64_t next = i + 1 < d->nconnects ? d->block_pos[i + 1] : d->neq;
        GPZ_REQUIRE(d->block_pos[i] + d->block_size[i] == next, GPZ_E_INVALID,
                    i + 1 < d->nconnects ? "block positions must be consecutive in connect order"
                                         : "sum of block sizes != neq");
      }
    });
    host_parallel(d->nel, [&](int64_t e0, int64_t e1) {
      for (int64_t e = e0; e < e1; e++) {
        int t = d->el_type[e];
        GPZ_REQUIRE(t == GPZ_EL_LINE || t == GPZ_EL_QUAD || t == GPZ_EL_HEX, GPZ_E_UNSUPPORTED_ELEMENT, "element type");
        const ElemTopo &tp = topo(t);
        for (int k = 0; k < tp.ncorner; k++) {
          int64_t nd = d->el_nodes[e * 8 + k];
          GPZ_REQUIRE(nd >= 0 && nd < d->nnodes, GPZ_E_INVALID, "corner node index");
        }
        for (int s = 0; s < tp.nsides; s++) {
          int64_t cn = d->el_conn[e * 27 + s];
          GPZ_REQUIRE(cn >= 0 && cn < d->nconnects, GPZ_E_INVALID, "connect index");
        }
        GPZ_REQUIRE(d->el_order[e] >= 1 && d->el_order[e] <= 3, GPZ_E_UNSUPPORTED_ELEMENT, "order must be 1..3");
      }
    });
    const auto t1 = std::chrono::steady_clock::now();
    c.dim = d->dim;
    c.nstate = d->nstate;
    c.nel = d->nel;
    c.nnodes = d->nnodes;
    c.nconnects = d->nconnects;
    c.neq = d->neq;
    c.neq_mesh = d->neq;
    c.flt.active = false;  // a new mesh starts without an equation filter
    c.flt.h_act.clear();
    c.mats.assign(d->mats, d->mats + d->nmat);
    c.bcs.assign(d->bcs, d->bcs + d->nbc);
    c.h_el_type.assign(d->el_type, d->el_type + d->nel);
    c.h_el_mat.assign(d->el_mat, d->el_mat + d->nel);
    c.h_el_conn.assign(d->el_conn, d->el_conn + d->nel * 27);
    c.h_block_pos.assign(d->block_pos, d->block_pos + d->nconnects);
    c.h_block_size.assign(d->block_size, d->block_size + d->nconnects);
    cudaStream_t s = c.stream;
    c.d_xyz.upload(d->node_xyz, d->nnodes * 3, s);
    c.d_el_type.upload(d->el_type, d->nel, s);
    c.d_el_mat.upload(d->el_mat, d->nel, s);
    c.d_el_nodes.upload(d->el_nodes, d->nel * 8, s);
    c.d_el_conn.upload(d->el_conn, d->nel * 27, s);
    c.d_conn_order.upload(d->conn_order, d->nconnects, s);
    c.d_block_size.upload(d->block_size, d->nconnects, s);
    c.d_block_pos.upload(d->block_pos, d->nconnects, s);
    if (d->el_coef) c.d_coef.upload(d->el_coef, d->nel, s);
    else c.d_coef.release();
    GPZ_CUDA_TRY(cudaStreamSynchronize(s));
    const auto t2 = std::chrono::steady_clock::now();
    build_buckets(c, *d);
    const auto t3 = std::chrono::steady_clock::now();
    auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
      return std::to_string(std::chrono::duration<double, std::milli>(b - a).count());
    };
    c.upload_report = "{\"checks\": " + ms(t0, t1) + ", \"copies\": " + ms(t1, t2) + ", \"buckets\": " + ms(t2, t3) +
                      ", \"bucket_parts\": " + c.bucket_report + "}";
    c.er.reset();
    c.have_mesh = true;
    c.have_pattern = c.have_matrix = c.have_solution = c.have_a32 = c.have_bjinv = c.have_rhs = false;
    c.a32_tensor = false;
    c.fp32_report.clear();
    c.have_vbinv = false;
    c.vb_kind = 0;
    c.tl.ready = c.tl.have_inv = false;
    if (c.asm_mode_auto) c.asm_queue = -1;  // an autotuned launch mode is timed again for the new buckets
    c.asm_mode_report.clear();
    c.asm_tune_report.clear();
    drop_assembly_graph(c);
    return GPZ_OK;
  });
}

int gpz_mesh_set_coef(gpz_ctx *ctx, const double *el_coef) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_mesh, GPZ_E_NOT_READY, "no mesh");
    GPZ_REQUIRE(el_coef, GPZ_E_INVALID, "null coefficients");
    const double *before = c.d_coef.p;
    c.d_coef.upload(el_coef, c.nel, c.stream);
    c.have_matrix = c.have_solution = c.have_rhs = false;
    if (c.d_coef.p != before) drop_assembly_graph(c);  // the captured kernels hold the coefficient pointer
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return GPZ_OK;
  });
}

int gpz_precond_apply(gpz_ctx *ctx, int precond, const double *r, double *z) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_matrix, GPZ_E_NOT_READY, "no assembled matrix");
    GPZ_REQUIRE(r && z, GPZ_E_INVALID, "null vector");
    precond_apply(c, precond, r, z);
    return GPZ_OK;
  });
}

int gpz_two_level_config(gpz_ctx *ctx, int coarse_boxes) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(coarse_boxes >= 1 && coarse_boxes <= 64, GPZ_E_INVALID, "coarse boxes per direction: 1..64");
    c.tl.target = coarse_boxes;
    c.tl.ready = c.tl.have_inv = false;
    return GPZ_OK;
  });
}

int gpz_two_level_info(gpz_ctx *ctx, int64_t *info) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(info, GPZ_E_INVALID, "null info");
    GPZ_REQUIRE(c.tl.ready, GPZ_E_NOT_READY, "no two-level solve on this mesh yet");
    const TwoLevel &T = c.tl;
    const int64_t v[8] = {T.lx[0], T.lx[1], T.lx[2], T.s, T.m[0], T.m[1], T.m[2], T.nc};
    for (int k = 0; k < 8; k++) info[k] = v[k];
    info[8] = T.nfixed;
    return GPZ_OK;
  });
}

int gpz_equation_filter(gpz_ctx *ctx, int64_t nactive, const int64_t *active) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_mesh, GPZ_E_NOT_READY, "no mesh");
    std::vector<int64_t> v;
    if (nactive >= 0) {
      GPZ_REQUIRE(nactive > 0 && active, GPZ_E_INVALID, "active equations");
      v.assign(active, active + nactive);
      for (int64_t q : v) GPZ_REQUIRE(q >= 0 && q < c.neq_mesh, GPZ_E_INVALID, "active equation out of range");
      std::sort(v.begin(), v.end());  // SetActiveEquations: duplicates removed, increasing order
      v.erase(std::unique(v.begin(), v.end()), v.end());
    }
    c.flt.active = nactive >= 0;
    c.flt.h_act.swap(v);
    if (c.flt.active) filter_prepare(c);
    // another system: its pattern and values are built again
    c.neq = c.neq_mesh;
    c.have_pattern = false;
    c.have_matrix = false;
    c.have_solution = false;
    c.have_a32 = false;
    c.a32_tensor = false;
    c.have_bsr3 = false;
    c.have_bjinv = false;
    c.have_vbinv = false;
    c.vb_kind = 0;
    c.tl.ready = c.tl.have_inv = false;
    c.spmv32_tuned = -1;
    drop_assembly_graph(c);
    return GPZ_OK;
  });
}

int gpz_pattern_build(gpz_ctx *ctx, int sym, int64_t *nnz_out) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_mesh, GPZ_E_NOT_READY, "no mesh");
    c.neq = c.neq_mesh;
    const auto t0 = std::chrono::steady_clock::now();
    build_pattern(c);
    const auto t1 = std::chrono::steady_clock::now();
    build_upper(c);
    const auto t2 = std::chrono::steady_clock::now();
    build_element_offsets(c);
    const auto t3 = std::chrono::steady_clock::now();
    auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
      return std::to_string(std::chrono::duration<double, std::milli>(b - a).count());
    };
    c.pattern_report = "{\"full_csr\": " + ms(t0, t1) + ", \"upper_and_diagonal\": " + ms(t1, t2) +
                       ", \"element_offsets\": " + ms(t2, t3) + "}";
    if (c.flt.active) condense_pattern(c);
    c.user_sym = sym ? 1 : 0;
    c.have_pattern = true;
    c.spmv32_tuned = -1;  // a new pattern is tuned again at its first mixed assembly
    drop_assembly_graph(c);
    c.have_matrix = false;
    if (nnz_out) *nnz_out = sym ? c.nnz_upper : c.nnz;
    return GPZ_OK;
  });
}

int gpz_pattern_upload(gpz_ctx *ctx, int sym, int64_t neq, const int64_t *IA, const int64_t *JA) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_mesh, GPZ_E_NOT_READY, "no mesh");
    GPZ_REQUIRE(!c.flt.active, GPZ_E_INVALID, "under an equation filter the pattern is built on the device");
    GPZ_REQUIRE(neq == c.neq_mesh && IA && JA, GPZ_E_INVALID, "pattern size");
    GPZ_REQUIRE(!sym, GPZ_E_INVALID, "upload the full pattern (TPZFYsmpMatrix layout); the upper one is derived");
    int64_t nnz = IA[neq];
    std::vector<int32_t> ja32(nnz);
    for (int64_t k = 0; k < nnz; k++) {
      GPZ_REQUIRE(JA[k] >= 0 && JA[k] < neq, GPZ_E_INVALID, "column index");
      ja32[k] = (int32_t)JA[k];
    }
    c.nnz = nnz;
    c.d_ia.upload(IA, neq + 1, c.stream);
    c.d_ja.upload(ja32.data(), nnz, c.stream);
    build_upper(c);
    build_element_offsets(c);
    c.user_sym = 0;
    c.have_pattern = true;
    c.spmv32_tuned = -1;  // a new pattern is tuned again at its first mixed assembly
    drop_assembly_graph(c);
    c.have_matrix = false;
    return GPZ_OK;
  });
}

int gpz_assembly_report(gpz_ctx *ctx, char *buf, int64_t len) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_mesh && buf && len > 0, GPZ_E_INVALID, "arguments");
    int64_t nb = 0, nhp = 0, ehp = 0, eun = 0;
    for (const Bucket *b : c.buckets) {
      if (b->hp) {
        nhp++;
        ehp += (int64_t)b->elems.size();
      } else {
        nb++;
        eun += (int64_t)b->elems.size();
      }
    }
    std::string r = "{\"uniform_buckets\": " + std::to_string(nb) + ", \"uniform_elements\": " + std::to_string(eun) +
                    ", \"hp_classes\": " + std::to_string(nhp) + ", \"hp_elements\": " + std::to_string(ehp) +
                    ", \"colours\": " + std::to_string(c.ncolours) + ", \"hp_block_size_ms\": " +
                    (c.asm_tune_report.empty() ? std::string("null") : c.asm_tune_report) + ", \"launch_mode_ms\": " +
                    (c.asm_mode_report.empty() ? std::string("null") : c.asm_mode_report) + ", \"fp32_elements\": " +
                    (c.fp32_report.empty() ? std::string("null") : c.fp32_report) + ", \"mesh_upload_ms\": " +
                    (c.upload_report.empty() ? std::string("null") : c.upload_report) + ", \"pattern_ms\": " +
                    (c.pattern_report.empty() ? std::string("null") : c.pattern_report) + ", \"row_owner_pass\": " +
                    (c.rp_bucket ? "{\"elements\": " + std::to_string(c.rp_bucket->elems.size()) +
                                       ", \"longest_row\": " + std::to_string(c.rp_lmax) +
                                       ", \"warps_per_cta\": " + std::to_string(c.rp_warps) +
                                       ", \"matrix_cleared\": " + (c.rp_full ? "false" : "true") + "}"
                                 : std::string("null")) +
                    "}";
    GPZ_REQUIRE((int64_t)r.size() < len, GPZ_E_INVALID, "buffer too small");
    std::copy(r.begin(), r.end(), buf);
    buf[r.size()] = 0;
    return GPZ_OK;
  });
}

int gpz_pattern_info(gpz_ctx *ctx, int64_t *nnz_full, int64_t *nnz_upper) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_pattern, GPZ_E_NOT_READY, "no pattern");
    if (nnz_full) *nnz_full = c.nnz;
    if (nnz_upper) *nnz_upper = c.nnz_upper;
    return GPZ_OK;
  });
}

int gpz_pattern_download(gpz_ctx *ctx, int64_t *IA, int64_t *JA) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_pattern, GPZ_E_NOT_READY, "no pattern");
    GPZ_REQUIRE(IA && JA, GPZ_E_INVALID, "null output");
    const DBuf<int64_t> &ia = c.user_sym ? c.d_ia_up : c.d_ia;
    const DBuf<int32_t> &ja = c.user_sym ? c.d_ja_up : c.d_ja;
    int64_t nnz = c.user_sym ? c.nnz_upper : c.nnz;
    GPZ_CUDA_TRY(cudaMemcpyAsync(IA, ia.p, (c.neq + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, c.stream));
    std::vector<int32_t> tmp(nnz);
    if (nnz) GPZ_CUDA_TRY(cudaMemcpyAsync(tmp.data(), ja.p, nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, c.stream));
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    for (int64_t k = 0; k < nnz; k++) JA[k] = tmp[k];
    return GPZ_OK;
  });
}

int gpz_set_killed(gpz_ctx *ctx, int killed) {
  if (!ctx) return GPZ_E_INVALID;
  ctx->c.killed.store(killed ? 1 : 0);
  return GPZ_OK;
}

int gpz_assemble(gpz_ctx *ctx, int precision) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_pattern, GPZ_E_NOT_READY, "no pattern");
    if (c.killed.load()) return GPZ_CANCELLED;  // StrMatrix/pzstrmatrixor.cpp:490
    GPZ_REQUIRE(precision == GPZ_PREC_FP64 || precision == GPZ_PREC_MIXED, GPZ_E_INVALID, "precision");
    assemble_fp64(c);
    if (precision == GPZ_PREC_MIXED) {
      // the FP32 values: element matrices formed again in FP32 (the tensor cores for the hexes), or the
      // FP64 matrix rounded; under an equation filter always the latter
      if (c.fp32_src == 1 && !c.flt.active) assemble_fp32_elements(c);
      make_fp32_copy(c);
    }
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    check_device_flag(c, "assembly");
    c.have_matrix = true;
    c.have_rhs = true;
    return GPZ_OK;
  });
}

int gpz_assemble_rhs(gpz_ctx *ctx) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_mesh, GPZ_E_NOT_READY, "no mesh");
    if (c.killed.load()) return GPZ_CANCELLED;
    assemble_rhs(c);
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    check_device_flag(c, "load vector assembly");
    c.have_rhs = true;
    return GPZ_OK;
  });
}

int gpz_error_points(gpz_ctx *ctx, int32_t exact_order, int64_t *npoints, double *xyz) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_mesh, GPZ_E_NOT_READY, "no mesh");
    GPZ_REQUIRE(npoints, GPZ_E_INVALID, "null npoints");
    error_prepare(c, exact_order);
    *npoints = c.er.npts;
    if (xyz) {
      error_points(c, xyz);
      check_device_flag(c, "error points");
    }
    return GPZ_OK;
  });
}

int gpz_error_evaluate(gpz_ctx *ctx, int32_t exact_order, const double *sol, const double *u_exact,
                       const double *du_exact, int32_t *nerrors, double *errors, double *el_errors) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_mesh, GPZ_E_NOT_READY, "no mesh");
    GPZ_REQUIRE(errors, GPZ_E_INVALID, "null errors");
    error_prepare(c, exact_order);
    GPZ_REQUIRE(c.er.npts == 0 || (u_exact && du_exact), GPZ_E_INVALID, "null exact solution");
    const double *sol_dev = c.sw.x.p;
    if (sol) {
      c.er.sol.upload(sol, c.neq_mesh, c.stream);
      sol_dev = c.er.sol.p;
    } else {
      GPZ_REQUIRE(c.have_solution && c.sw.x.p, GPZ_E_NOT_READY, "no solution on the device");
      if (c.flt.active) {  // TPZEquationFilter::Scatter of the condensed solution (Analysis/TPZLinearAnalysis.cpp:197)
        c.flt.xfull.alloc(std::max<int64_t>(c.neq_mesh, 1));
        filter_scatter(c, c.sw.x.p, c.flt.xfull.p);
        sol_dev = c.flt.xfull.p;
      }
    }
    error_evaluate(c, sol_dev, u_exact, du_exact, errors, el_errors);
    check_device_flag(c, "error norms");
    if (nerrors) *nerrors = c.er.nerr;
    return GPZ_OK;
  });
}

namespace {
__global__ void k_gather_upper(const double *__restrict__ a, const int64_t *__restrict__ diagpos,
                               const int64_t *__restrict__ ia, const int64_t *__restrict__ ia_up, int64_t neq,
                               double *__restrict__ out) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // a warp per row
  const int lane = threadIdx.x & 31;
  if (r >= neq) return;
  const int64_t d = diagpos[r], n = ia[r + 1] - d, o = ia_up[r];
  for (int64_t k = lane; k < n; k += 32) out[o + k] = a[d + k];
}
}  // namespace

int gpz_matrix_download(gpz_ctx *ctx, double *A) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_matrix, GPZ_E_NOT_READY, "not assembled");
    GPZ_REQUIRE(A, GPZ_E_INVALID, "null output");
    if (!c.user_sym) {
      GPZ_CUDA_TRY(cudaMemcpyAsync(A, c.d_a.p, c.nnz * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    } else {
      DBuf<double> up;
      up.alloc(std::max<int64_t>(c.nnz_upper, 1));
      if (c.neq) {
        k_gather_upper<<<grid_for(c.neq * 32, 256), 256, 0, c.stream>>>(c.d_a.p, c.d_diagpos.p, c.d_ia.p, c.d_ia_up.p, c.neq,
                                                              up.p);
        c.launches++;
        GPZ_CUDA_TRY(cudaGetLastError());
      }
      GPZ_CUDA_TRY(cudaMemcpyAsync(A, up.p, c.nnz_upper * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
      GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    }
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return GPZ_OK;
  });
}

int gpz_rhs_download(gpz_ctx *ctx, double *F) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_matrix || c.have_rhs, GPZ_E_NOT_READY, "not assembled");
    GPZ_CUDA_TRY(cudaMemcpyAsync(F, c.d_f.p, c.neq_mesh * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return GPZ_OK;
  });
}

int gpz_rhs_upload(gpz_ctx *ctx, const double *F) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_matrix, GPZ_E_NOT_READY, "not assembled");
    GPZ_REQUIRE(F, GPZ_E_INVALID, "null input");
    GPZ_CUDA_TRY(cudaMemcpyAsync(c.d_f.p, F, c.neq_mesh * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return GPZ_OK;
  });
}

int gpz_spmv(gpz_ctx *ctx, double alpha, const double *x, double beta, const double *y, double *z) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_matrix, GPZ_E_NOT_READY, "not assembled");
    GPZ_REQUIRE(x && z, GPZ_E_INVALID, "null vector");
    DBuf<double> dx, dy, dz;
    dx.upload(x, c.neq, c.stream);
    if (y && beta != 0.0) dy.upload(y, c.neq, c.stream);
    dz.alloc(std::max<int64_t>(c.neq, 1));
    spmv_device(c, dx.p, dz.p, alpha, beta, (y && beta != 0.0) ? dy.p : nullptr);
    GPZ_CUDA_TRY(cudaMemcpyAsync(z, dz.p, c.neq * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return GPZ_OK;
  });
}

int gpz_spmv_fp32(gpz_ctx *ctx, int variant, const double *x, double *y) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_matrix, GPZ_E_NOT_READY, "not assembled");
    GPZ_REQUIRE(x && y && variant >= -1 && variant <= 10, GPZ_E_INVALID, "arguments");
    spmv32_apply(c, variant, x, y);
    return GPZ_OK;
  });
}

int gpz_solve(gpz_ctx *ctx, const gpz_solver_opts *opts, const double *b, double *x, gpz_solve_report *rep) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_matrix, GPZ_E_NOT_READY, "not assembled");
    GPZ_REQUIRE(opts && opts->max_iter >= 0 && opts->tol >= 0, GPZ_E_INVALID, "options");
    bool mixed = opts->solver == GPZ_SOLVER_MIXED_CG;
    solver_prepare(c, mixed);
    cudaStream_t s = c.stream;
    if (b) GPZ_CUDA_TRY(cudaMemcpyAsync(c.sw.b.p, b, c.neq * sizeof(double), cudaMemcpyHostToDevice, s));
    else if (c.flt.active) filter_gather(c, c.d_f.p, c.sw.b.p);  // TPZEquationFilter::Gather (TPZLinearAnalysis.cpp:194)
    else GPZ_CUDA_TRY(cudaMemcpyAsync(c.sw.b.p, c.d_f.p, c.neq * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (opts->from_current) {
      GPZ_REQUIRE(x, GPZ_E_INVALID, "from_current needs x");
      GPZ_CUDA_TRY(cudaMemcpyAsync(c.sw.x.p, x, c.neq * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    gpz_solve_report r{};
    int rc = gpz::solve(c, *opts, r);
    if (x) {
      GPZ_CUDA_TRY(cudaMemcpyAsync(x, c.sw.x.p, c.neq * sizeof(double), cudaMemcpyDeviceToHost, s));
      GPZ_CUDA_TRY(cudaStreamSynchronize(s));
    }
    if (rep) *rep = r;
    return rc;
  });
}

int gpz_solution_download(gpz_ctx *ctx, double *x) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_solution, GPZ_E_NOT_READY, "no solution");
    GPZ_CUDA_TRY(cudaMemcpyAsync(x, c.sw.x.p, c.neq * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return GPZ_OK;
  });
}

int gpz_time_kernel(gpz_ctx *ctx, int which, int reps, double *ms_per_launch) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(c.have_matrix, GPZ_E_NOT_READY, "not assembled");
    GPZ_REQUIRE(reps > 0 && ms_per_launch, GPZ_E_INVALID, "arguments");
    if (which == GPZ_KERNEL_SPMV_FP64 || which == GPZ_KERNEL_SPMV_FP32) {
      *ms_per_launch = time_spmv(c, which == GPZ_KERNEL_SPMV_FP32, reps);
    } else if (which == GPZ_KERNEL_ASSEMBLE) {
      cudaEvent_t e0, e1;
      GPZ_CUDA_TRY(cudaEventCreate(&e0));
      GPZ_CUDA_TRY(cudaEventCreate(&e1));
      assemble_fp64(c);
      GPZ_CUDA_TRY(cudaEventRecord(e0, c.stream));
      for (int i = 0; i < reps; i++) assemble_fp64(c);
      GPZ_CUDA_TRY(cudaEventRecord(e1, c.stream));
      GPZ_CUDA_TRY(cudaEventSynchronize(e1));
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      *ms_per_launch = ms / reps;
      check_device_flag(c, "assembly");
    } else {
      GPZ_REQUIRE(false, GPZ_E_INVALID, "kernel id");
    }
    return GPZ_OK;
  });
}

int gpz_assembly_mode(gpz_ctx *ctx, int mode) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(mode >= -1 && mode <= 1, GPZ_E_INVALID, "mode: -1 autotuned, 0 per colour, 1 persistent");
    c.asm_queue = mode;
    c.asm_mode_auto = mode < 0;
    c.asm_mode_report = mode < 0 ? std::string() : std::string("{\"set\": \"") + (mode ? "persistent" : "per_colour") + "\"}";
    drop_assembly_graph(c);  // the captured launches follow the mode
    return GPZ_OK;
  });
}

int gpz_fp32_elements(gpz_ctx *ctx, int source) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(source == GPZ_FP32_ROUNDED || source == GPZ_FP32_ELEMENTS, GPZ_E_INVALID, "source");
    c.fp32_src = source;
    return GPZ_OK;
  });
}

int gpz_matrix_fp32_download(gpz_ctx *ctx, float *A) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(A, GPZ_E_INVALID, "null output");
    GPZ_REQUIRE(c.have_a32 && c.d_a32.p && (int64_t)c.d_a32.n >= c.nnz, GPZ_E_NOT_READY,
                "no FP32 CSR values (assemble with GPZ_PREC_MIXED; with 3x3 blocks they are kept only from the "
                "FP32 element pass)");
    if (c.nnz) GPZ_CUDA_TRY(cudaMemcpyAsync(A, c.d_a32.p, c.nnz * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
    GPZ_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return GPZ_OK;
  });
}

int gpz_tuning_cache(gpz_ctx *ctx, const char *path) {
  return guarded(ctx, [&](Ctx &c) {
    c.tune_cache = path ? std::string(path) : std::string();
    return GPZ_OK;
  });
}

int gpz_tuning_report(gpz_ctx *ctx, char *buf, int64_t len) {
  return guarded(ctx, [&](Ctx &c) {
    GPZ_REQUIRE(buf && len > 0, GPZ_E_INVALID, "buffer");
    std::string r = c.tune_report.empty() ? std::string("{}") : c.tune_report;
    int64_t n = std::min<int64_t>((int64_t)r.size(), len - 1);
    std::memcpy(buf, r.data(), n);
    buf[n] = 0;
    return GPZ_OK;
  });
}

}  // extern "C"
