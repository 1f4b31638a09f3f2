// A C++ program that runs the whole GPU path through include/gpz.h alone, as
// the NeoPZ-side binding does: the grid mesh of a workload from the host
// library (neopz_gb300/host/pz_grid.h, the numbering of CreateGeoMeshOnGrid +
// AutoBuild), then gpz_ctx_create -> gpz_mesh_upload -> gpz_pattern_build ->
// gpz_pattern_download -> gpz_assemble -> gpz_matrix_download /
// gpz_rhs_download -> gpz_solve (FP64 Jacobi-PCG to the workload's tolerance,
// then the mixed CG to a true 1e-8) -> the solutions.  It writes what it got
// as raw arrays (ia, ja, a, f, x, x_mixed) plus info.json; the test compares
// them with the reference library's own fixtures (tests/golden/ref_*.npz).
//
// Usage: abi_driver CASE N P SYM TOL OUTDIR [COEF_FILE|-] [ORDER_FILE]
//   CASE: poisson2d | darcy2d | darcy3d | elast3d | elast3d_c5 | elast3d_hp (tests/grid_cases.h)
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "grid_cases.h"

template <class T>
static std::vector<T> read_file(const char *path, size_t n) {
  std::vector<T> v(n);
  FILE *f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), sizeof(T), n, f) != n) {
    std::fprintf(stderr, "cannot read %s\n", path);
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

template <class T>
static void write_file(const std::string &path, const T *p, size_t n) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f || std::fwrite(p, sizeof(T), n, f) != n) {
    std::fprintf(stderr, "cannot write %s\n", path.c_str());
    std::exit(2);
  }
  std::fclose(f);
}

static void check(int rc, const char *what, gpz_ctx *ctx) {
  if (rc < 0) {
    std::fprintf(stderr, "%s: %d %s (%s)\n", what, rc, gpz_get_error_string(rc), ctx ? gpz_last_error_detail(ctx) : "");
    std::exit(3);
  }
}

int main(int argc, char **argv) {
  if (argc < 7) {
    std::fprintf(stderr, "usage: abi_driver CASE N P SYM TOL OUTDIR [COEF_FILE|-] [ORDER_FILE]\n");
    return 2;
  }
  const std::string cs = argv[1];
  const int n = std::atoi(argv[2]), p = std::atoi(argv[3]), sym = std::atoi(argv[4]);
  const double tol = std::atof(argv[5]);
  const std::string out = argv[6];
  const bool is3d = grid_case_is3d(cs);
  const int64_t ncell = is3d ? (int64_t)n * n * n : (int64_t)n * n;
  std::vector<double> coef;
  std::vector<int32_t> order;
  if (argc > 7 && std::string(argv[7]) != "-") coef = read_file<double>(argv[7], ncell);
  if (argc > 8) order = read_file<int32_t>(argv[8], ncell);

  void *grid = grid_case(cs, n, p, coef.empty() ? nullptr : coef.data(), order.empty() ? nullptr : order.data());
  if (!grid) {
    std::fprintf(stderr, "grid build failed\n");
    return 3;
  }
  gpz_mesh_desc desc;
  check(gpzh_grid_desc(grid, &desc), "grid descriptor", nullptr);
  const int64_t neq = desc.neq;

  gpz_ctx *ctx = nullptr;
  check(gpz_ctx_create(&ctx, 0), "context", nullptr);
  check(gpz_mesh_upload(ctx, &desc), "mesh upload", ctx);
  int64_t nnz = 0;
  check(gpz_pattern_build(ctx, sym, &nnz), "pattern build", ctx);
  std::vector<int64_t> ia(neq + 1), ja(nnz);
  check(gpz_pattern_download(ctx, ia.data(), ja.data()), "pattern download", ctx);
  check(gpz_assemble(ctx, GPZ_PREC_FP64), "assemble", ctx);
  std::vector<double> a(nnz), f(neq), x(neq, 0.0), xm(neq, 0.0);
  check(gpz_matrix_download(ctx, a.data()), "matrix download", ctx);
  check(gpz_rhs_download(ctx, f.data()), "rhs download", ctx);
  write_file(out + "/ia.bin", ia.data(), ia.size());
  write_file(out + "/ja.bin", ja.data(), ja.size());
  write_file(out + "/a.bin", a.data(), a.size());
  write_file(out + "/f.bin", f.data(), f.size());
  gpz_solver_opts o;
  std::memset(&o, 0, sizeof(o));
  gpz_solve_report rep, repm;
  std::memset(&rep, 0, sizeof(rep));
  std::memset(&repm, 0, sizeof(repm));
  int rc = 0, rcm = 0;
  if (tol > 0 && sym) {
    o.solver = GPZ_SOLVER_CG;
    o.precond = GPZ_PRECOND_JACOBI;
    o.max_iter = 200000;
    o.tol = tol;
    o.check_every = 64;
    o.use_graph = 1;
    o.spmv_variant = -1;
    rc = gpz_solve(ctx, &o, nullptr, x.data(), &rep);
    check(rc, "FP64 CG", ctx);
    check(gpz_assemble(ctx, GPZ_PREC_MIXED), "mixed assemble", ctx);
    o.solver = GPZ_SOLVER_MIXED_CG;
    o.precond = desc.nstate == 3 ? GPZ_PRECOND_BLOCK_JACOBI : GPZ_PRECOND_JACOBI;
    o.tol = 1e-8;
    o.reliable_delta = 1e-2;
    rcm = gpz_solve(ctx, &o, nullptr, xm.data(), &repm);
    check(rcm, "mixed CG", ctx);
    write_file(out + "/x.bin", x.data(), x.size());
    write_file(out + "/x_mixed.bin", xm.data(), xm.size());
  }
  FILE *js = std::fopen((out + "/info.json").c_str(), "w");
  std::fprintf(js,
               "{\"neq\": %lld, \"nnz\": %lld, \"cg_rc\": %d, \"cg_iterations\": %lld, \"cg_true_resid\": %.17g, "
               "\"mixed_rc\": %d, \"mixed_iterations\": %lld, \"mixed_true_resid\": %.17g, \"launches\": %lld}\n",
               (long long)neq, (long long)nnz, rc, (long long)rep.iterations, rep.true_resid, rcm,
               (long long)repm.iterations, repm.true_resid, (long long)gpz_kernel_launches(ctx));
  std::fclose(js);
  gpz_ctx_destroy(ctx);
  gpzh_grid_free(grid);
  return 0;
}
