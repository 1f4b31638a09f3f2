"""Parity of the GPU path (libgpz.so through its C ABI) with the CPU oracle.

Tolerances (FP64 path):
* CSR row pointers and column indices: bit-exact (TPZSSpStructMatrix upper and
  TPZSpStructMatrix full patterns);
* matrix values: per row, max |a_gpu - a_ref| <= 1e-12 * max |a_ref| of that row
  (the GPU sums element contributions in colour order, the reference in
  element order, and forms the Gram before the material combination);
* load vector: max |f_gpu - f_ref| <= 1e-12 * max |f_ref|;
* Jacobi-PCG: same algorithm and stopping rule; solution within 1e-8
  relative.  With penalty Dirichlet rows (1e12 .. 6.7e16 on the diagonal) the
  iteration count depends on the summation order (the oracle itself gives
  different counts with and without fused multiply-adds), so counts must agree
  within max(3, 10%) -- 30% for the 6.7e16-penalty Poisson/Darcy systems,
  where sequential, numpy and GPU row sums already give 34 / 28 / 27
  iterations on the 16x16 Q2 case.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _gpz():
    from neopz_gb300 import gpz
    return gpz


def _row_rel(ia, a, ref):
    worst = 0.0
    for r in range(len(ia) - 1):
        s, e = ia[r], ia[r + 1]
        m = np.max(np.abs(ref[s:e]))
        d = np.max(np.abs(a[s:e] - ref[s:e]))
        if m > 0:
            worst = max(worst, d / m)
        else:
            assert d == 0.0
    return worst


def _cases():
    g = _gpz()
    rng = np.random.default_rng(7)
    k2 = np.exp(rng.standard_normal(16 * 16))
    k3 = np.exp(rng.standard_normal(4 ** 3))
    E3 = np.exp(rng.standard_normal(3 ** 3))
    o3, o2 = g.hp_orders(27, 3), g.hp_orders(36, 5)
    E3h = np.exp(0.5 * rng.standard_normal(27))
    k2h = np.exp(rng.standard_normal(36))
    return {
        "poisson2d_p1": (lambda: O.poisson2d(16, 1), lambda: g.poisson2d(16, 1)),
        "poisson2d_p2": (lambda: O.poisson2d(16, 2), lambda: g.poisson2d(16, 2)),
        "poisson2d_p3": (lambda: O.poisson2d(8, 3), lambda: g.poisson2d(8, 3)),
        "darcy2d_p2": (lambda: O.darcy(2, 16, 2, k2), lambda: g.darcy(2, 16, 2, k2)),
        "darcy3d_p2": (lambda: O.darcy(3, 4, 2, k3), lambda: g.darcy(3, 4, 2, k3)),
        "elast3d_p1": (lambda: O.elasticity3d(3, 1, E=E3), lambda: g.elasticity3d(3, 1, E=E3)),
        "elast3d_p2": (lambda: O.elasticity3d(3, 2, E=E3), lambda: g.elasticity3d(3, 2, E=E3)),
        "elast3d_p3": (lambda: O.elasticity3d(2, 3), lambda: g.elasticity3d(2, 3)),
        # hp: per-element orders in {1,2,3}, shared sides at the largest (batched run-time kernels)
        "elast3d_hp": (lambda: O.elasticity3d_hp(3, o3, E=E3h), lambda: g.elasticity3d_hp(3, o3, E=E3h)),
        "darcy2d_hp": (lambda: O.darcy_hp(6, o2, k2h), lambda: g.darcy_hp(6, o2, k2h)),
        # a translated, non-cubic box of hexes with a position-dependent load: the shared element matrix
        # (every element a translate of the first) with per-element load vectors
        "poisson3d_box_p2": (lambda: _poisson3d_box_oracle(), lambda: _poisson3d_box_gpz(g)),
    }


_BOX = dict(n=(3, 4, 2), lo=(0.25, -0.5, 1.0), hi=(1.0, 0.5, 1.3))


def _poisson3d_box_oracle():
    mats = [O.material(1, O.ORC_POISSON, 3, scale=1.5, forcing=O.ORC_F_SINPROD, force=(1.0, 0, 0), forcing_porder=2)]
    return O.OracleMesh(3, _BOX["n"], _BOX["lo"], _BOX["hi"], [1, -1, -1, -1, -1, -1, -1], True, 2, mats,
                        [O.bc(-1, 1, 0)])


def _poisson3d_box_gpz(g):
    mats = [(1, g.material(g.GPZ_MAT_POISSON, 3, scale=1.5, forcing=g.GPZ_F_SINPROD, force=(1.0, 0, 0),
                           forcing_porder=2))]
    return g.Grid(3, _BOX["n"], _BOX["lo"], _BOX["hi"], [1, -1, -1, -1, -1, -1, -1], True, 2, mats, [(-1, g.bc(0, 0))])


CASES = ["poisson2d_p1", "poisson2d_p2", "poisson2d_p3", "darcy2d_p2", "darcy3d_p2", "elast3d_p1", "elast3d_p2",
         "elast3d_p3", "elast3d_hp", "darcy2d_hp", "poisson3d_box_p2"]


@pytest.fixture(scope="module")
def built():
    import __graft_entry__
    __graft_entry__.build()
    return _cases()


@pytest.mark.parametrize("sym", [True, False])
@pytest.mark.parametrize("case", CASES)
def test_pattern_matrix_rhs(built, case, sym):
    g = _gpz()
    mk_o, mk_g = built[case]
    om, grid = mk_o(), mk_g()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    nnz = ctx.build_pattern(sym)
    ia, ja = ctx.pattern()
    oia, oja = om.pattern(sym)
    assert nnz == len(oja)
    assert np.array_equal(ia, oia) and np.array_equal(ja, oja)
    ctx.assemble(g.GPZ_PREC_FP64)
    a, f = ctx.matrix(), ctx.rhs()
    oa, of = om.assemble(sym, oia, oja)
    assert _row_rel(oia, a, oa) <= 1e-12
    assert np.max(np.abs(f - of)) <= 1e-12 * max(np.max(np.abs(of)), 1e-300)
    # SpMV (TPZSYsmpMatrix / TPZFYsmpMatrix::MultAdd) on a random vector
    x = np.random.default_rng(1).standard_normal(om.neq)
    z = ctx.spmv(x)
    zr = O.spmv(sym, oia, oja, oa, x)
    assert np.max(np.abs(z - zr)) <= 1e-11 * np.max(np.abs(zr))
    ctx.close()


@pytest.mark.parametrize("case", ["poisson2d_p2", "darcy2d_p2", "elast3d_p2", "elast3d_p3", "elast3d_hp",
                                  "darcy2d_hp"])
def test_jacobi_pcg_matches_oracle(built, case):
    g = _gpz()
    mk_o, mk_g = built[case]
    om, grid = mk_o(), mk_g()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    ctx.assemble(g.GPZ_PREC_FP64)
    tol = 1e-10
    sol = ctx.solve(tol=tol, max_iter=20000)
    oia, oja = om.pattern(True)
    oa, of = om.assemble(True, oia, oja)
    ref = O.cg_jacobi(True, oia, oja, oa, of, 20000, tol)
    assert sol["rc"] == 0 and ref["rc"] == 0
    assert np.linalg.norm(sol["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    frac = 0.3 if case.startswith(("poisson", "darcy")) else 0.1
    assert abs(sol["iterations"] - ref["iters"]) <= max(3, frac * ref["iters"]), (sol["iterations"], ref["iters"])
    ctx.close()


def test_jacobi_pcg_graph_and_eager_agree(built):
    g = _gpz()
    grid = built["elast3d_p2"][1]()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble()
    s1 = ctx.solve(tol=1e-9, use_graph=True, check_every=16)
    s2 = ctx.solve(tol=1e-9, use_graph=False, check_every=7)
    assert s1["iterations"] == s2["iterations"]
    assert np.array_equal(s1["x"], s2["x"])  # deterministic reductions
    ctx.close()


@pytest.mark.parametrize("case", ["poisson2d_p2", "elast3d_p2", "darcy3d_p2", "elast3d_hp"])
def test_mixed_cg_reaches_true_fp64_residual(built, case):
    g = _gpz()
    mk_o, mk_g = built[case]
    om, grid = mk_o(), mk_g()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    ctx.assemble(g.GPZ_PREC_MIXED)
    tol = 1e-8
    sol = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, tol=tol, max_iter=20000, reliable_delta=1e-2)
    assert sol["rc"] == 0
    assert sol["true_resid"] <= tol
    assert sol["spmv_fp32"] > 0 and sol["reliable_updates"] >= 1
    oia, oja = om.pattern(True)
    oa, of = om.assemble(True, oia, oja)
    ref = O.cg_jacobi(True, oia, oja, oa, of, 20000, 1e-12)
    # error against the FP64 oracle's tight solution: held to the 1e-8 bar of the
    # mixed-precision design at the true-residual tolerance 1e-8
    err = np.linalg.norm(sol["x"] - ref["x"]) / np.linalg.norm(ref["x"])
    assert err <= 1e-8, err
    ctx.close()


@pytest.mark.parametrize("case", ["elast3d_p1", "elast3d_p2", "elast3d_hp"])
def test_block_jacobi_pcg_matches_oracle(built, case):
    """Connect-block Jacobi CG against the oracle's TPZBlockDiagonal-preconditioned CG over the same connect
    blocks (3x3 at p <= 2; whole blocks of 3 to 24 equations on the hp mesh)."""
    g = _gpz()
    mk_o, mk_g = built[case]
    om, grid = mk_o(), mk_g()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    ctx.assemble()
    tol = 1e-10
    sol = ctx.solve(precond=g.GPZ_PRECOND_BLOCK_JACOBI, tol=tol, max_iter=20000)
    oia, oja = om.pattern(True)
    oa, of = om.assemble(True, oia, oja)
    # the connect blocks of TPZBlockDiagonalStructMatrix: 3 equations each at p <= 2, 3 to 24 on the hp mesh
    bp, bs = om.blocks()
    keep = bs > 0
    bi = np.concatenate([[0], np.cumsum(bs[keep])]).astype(np.int64)
    be = np.concatenate([np.arange(p, p + n) for p, n in zip(bp[keep], bs[keep])]).astype(np.int64)
    ref = O.cg_sparse_block_jacobi(True, oia, oja, oa, of, bi, be, 20000, tol)
    assert sol["rc"] == 0 and ref["rc"] == 0
    assert np.linalg.norm(sol["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    assert abs(sol["iterations"] - ref["iters"]) <= max(3, 0.1 * ref["iters"]), (sol["iterations"], ref["iters"])
    ctx.close()


def test_mixed_block_jacobi_bsr3(built):
    """FP32 3x3 block-CSR SpMV + block Jacobi: the mixed path of the elasticity benchmark."""
    g = _gpz()
    mk_o, mk_g = built["elast3d_p2"]
    om, grid = mk_o(), mk_g()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble(g.GPZ_PREC_MIXED)
    sol = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_BLOCK_JACOBI, tol=1e-8, reliable_delta=1e-2)
    assert sol["rc"] == 0 and sol["true_resid"] <= 1e-8 and sol["spmv_fp32"] > 0
    oia, oja = om.pattern(True)
    oa, of = om.assemble(True, oia, oja)
    ref = O.cg_jacobi(True, oia, oja, oa, of, 20000, 1e-12)
    assert np.linalg.norm(sol["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    ctx.close()


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5, 6, 7, 8, 10])
def test_mixed_spmv_variants_converge(built, variant):
    """Every layout / kernel the SpMV autotuner can pick gives the same converged solution."""
    g = _gpz()
    rng = np.random.default_rng(11)
    E = np.exp(rng.standard_normal(5 ** 3))
    om, grid = O.elasticity3d(5, 2, E=E), g.elasticity3d(5, 2, E=E)
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble(g.GPZ_PREC_MIXED)
    sol = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_BLOCK_JACOBI, tol=1e-8, reliable_delta=1e-2,
                    spmv_variant=variant)
    assert sol["rc"] == 0 and sol["true_resid"] <= 1e-8
    oia, oja = om.pattern(True)
    oa, of = om.assemble(True, oia, oja)
    ref = O.cg_jacobi(True, oia, oja, oa, of, 20000, 1e-12)
    assert np.linalg.norm(sol["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    ctx.close()


@pytest.mark.parametrize("m", [30, 5])
@pytest.mark.parametrize("case", ["poisson2d_p2", "darcy2d_p2", "elast3d_p2"])
def test_gmres_jacobi_matches_oracle(built, case, m):
    """Restarted Jacobi-GMRES(m) (gmres.h:68-168) against the oracle's restatement: same
    stopping rule on the preconditioned residual; solution within 1e-8, Arnoldi step count
    within max(3, 10%)."""
    g = _gpz()
    mk_o, mk_g = built[case]
    om, grid = mk_o(), mk_g()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble()
    tol = 1e-10
    sol = ctx.solve(solver=g.GPZ_SOLVER_GMRES, tol=tol, max_iter=20000, gmres_krylov=m)
    oia, oja = om.pattern(False)
    oa, of = om.assemble(False, oia, oja)
    ref = O.gmres_jacobi(False, oia, oja, oa, of, m, 20000, tol)
    assert sol["rc"] == 0 and ref["rc"] == 0 and sol["resid"] < tol
    assert np.linalg.norm(sol["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    assert abs(sol["iterations"] - ref["iters"]) <= max(3, 0.1 * ref["iters"]), (sol["iterations"], ref["iters"])
    ctx.close()


def test_gmres_graph_eager_budget_and_block_jacobi(built):
    g = _gpz()
    om, grid = built["elast3d_p2"][0](), built["elast3d_p2"][1]()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble()
    s1 = ctx.solve(solver=g.GPZ_SOLVER_GMRES, tol=1e-10, gmres_krylov=20, use_graph=True)
    s2 = ctx.solve(solver=g.GPZ_SOLVER_GMRES, tol=1e-10, gmres_krylov=20, use_graph=False)
    assert s1["rc"] == 0 and s1["iterations"] == s2["iterations"] and np.array_equal(s1["x"], s2["x"])
    # iteration budget: not converged, fNumIterations = max_iter
    s3 = ctx.solve(solver=g.GPZ_SOLVER_GMRES, tol=1e-10, gmres_krylov=20, max_iter=7)
    assert s3["rc"] == 1 and s3["iterations"] == 7 and s3["resid"] > 1e-10
    # connect-block Jacobi: converges to the same solution, in fewer steps than point Jacobi
    s4 = ctx.solve(solver=g.GPZ_SOLVER_GMRES, precond=g.GPZ_PRECOND_BLOCK_JACOBI, tol=1e-10, gmres_krylov=20)
    assert s4["rc"] == 0
    oia, oja = om.pattern(False)
    oa, of = om.assemble(False, oia, oja)
    ref = O.cg_jacobi(False, oia, oja, oa, of, 20000, 1e-12)
    for s in (s1, s4):
        assert np.linalg.norm(s["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    ctx.close()


def test_hp_batching_uses_classes_and_autotuner(built):
    """Elements of uneven side orders are assembled by the hp classes (run-time kernel, block size
    autotuned once), uniform ones by their compile-time buckets; the autotuned block size does not change
    the assembled values."""
    g = _gpz()
    grid = built["elast3d_hp"][1]()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble()
    rep = ctx.assembly_report()
    assert rep["hp_classes"] >= 1 and rep["hp_elements"] >= 1
    assert rep["hp_block_size_ms"]["chosen"] in (64, 128, 256)
    a1 = ctx.matrix()
    ctx.assemble()
    assert np.array_equal(a1, ctx.matrix())
    ctx.close()


@pytest.mark.parametrize("case", ["poisson2d_p2", "elast3d_p2", "elast3d_hp"])
def test_rhs_only_assembly(built, case):
    """TPZStructMatrix::Assemble(rhs): the load vector without the matrix, identical to the full assembly's,
    and to the oracle's within 1e-12; also before any pattern exists."""
    g = _gpz()
    mk_o, mk_g = built[case]
    om, grid = mk_o(), mk_g()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.assemble_rhs()
    f0 = ctx.rhs()
    ctx.build_pattern(True)
    ctx.assemble()
    assert np.array_equal(f0, ctx.rhs())
    oia, oja = om.pattern(True)
    _, of = om.assemble(True, oia, oja)
    assert np.max(np.abs(f0 - of)) <= 1e-12 * np.max(np.abs(of))
    ctx.close()


def test_assembly_graph_replay(built):
    """The second assembly of a pattern replays the captured CUDA graph: identical values; after new
    coefficients, the replay equals a fresh context's eager assembly."""
    g = _gpz()
    n = 3
    rng = np.random.default_rng(21)
    E1, E2 = np.exp(rng.standard_normal(n ** 3)), np.exp(rng.standard_normal(n ** 3))
    grid = g.elasticity3d(n, 2, E=E1)
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble()
    a1, f1 = ctx.matrix(), ctx.rhs()
    ctx.assemble()
    assert np.array_equal(a1, ctx.matrix()) and np.array_equal(f1, ctx.rhs())
    ctx.set_coef(grid, E2)
    ctx.assemble()
    a2 = ctx.matrix()
    fresh = g.Context(0)
    fresh.upload_mesh(g.elasticity3d(n, 2, E=E2))
    fresh.build_pattern(False)
    fresh.assemble()
    assert np.array_equal(a2, fresh.matrix())
    fresh.close()
    ctx.close()


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5, 6, 7, 8, 10])
def test_fp32_operator_layouts_match_fp64_spmv(built, variant):
    """Every FP32 operator layout of the mixed CG (block CSR, two rows, sliced ELL, TMA-staged, upper blocks
    with atomics, matrix-free elements on CUDA cores, on the tensor cores in 3xTF32, sum-factorised on
    Lagrange nodal values, and the shared element matrix of a uniform grid as one tcgen05 3xTF32 GEMM per tile)
    applies the assembled operator: within 1e-5 of the FP64 CSR SpMV,
    normwise and on the non-penalty rows alone."""
    g = _gpz()
    rng = np.random.default_rng(12)
    n = 5
    E = np.exp(rng.standard_normal(n ** 3))
    grid = g.elasticity3d(n, 2, E=E)
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble(g.GPZ_PREC_MIXED)
    x = rng.standard_normal(grid.neq)
    y64 = ctx.spmv(x)
    y32 = ctx.spmv_fp32(x, variant)
    assert np.linalg.norm(y32 - y64) <= 1e-5 * np.linalg.norm(y64)
    ia, ja = ctx.pattern()
    a = ctx.matrix()
    diag = np.array([a[ia[i]:ia[i + 1]][ja[ia[i]:ia[i + 1]] == i][0] for i in range(grid.neq)])
    inner = diag < 1e6 * np.median(diag)  # rows without the 1e12 penalty
    assert np.linalg.norm((y32 - y64)[inner]) <= 1e-5 * np.linalg.norm(y64[inner])
    if variant == 8:  # a uniform grid: the shared element matrix is offered and is the operator applied
        assert ctx.tuning_report()["chosen"] == "matrix_free_shared_matrix_tcgen05"
    if variant == 10:  # the same over lattice blocks (5^3 elements: partial blocks in every direction)
        assert ctx.tuning_report()["chosen"] == "matrix_free_shared_matrix_lattice_blocks"
    ctx.close()


@pytest.mark.parametrize("shape", [(17, 9, 5), (16, 16, 4), (30, 30, 30), (12, 10, 6, "sheared")])
def test_shared_matrix_operator_over_lattice_blocks(built, shape):
    """The shared-element-matrix operator over lattice blocks of 8 x 8 x 2 elements: full and partial blocks,
    more blocks than CTAs (30^3: 960 blocks), a box of unequal sides and a sheared one (lattice vectors not
    orthogonal).  It applies the assembled operator
    (1e-5 against the FP64 SpMV, the same bar as the tile operator it restructures) and the mixed CG over it
    reaches a true 1e-8 with the solution within 1e-8 of the FP64 solution."""
    g = _gpz()
    rng = np.random.default_rng(17)
    nx, ny, nz = shape[:3]
    mats = [(1, g.material(g.GPZ_MAT_ELAST3D, 3, E=1.0, nu=0.3, force=(0.0, 0.0, -1.0), forcing=g.GPZ_F_CONST))]
    grid = g.Grid(3, (nx, ny, nz), (0, 0, 0), (1.0, 0.7, 0.4), [1, -1, -2, -2, -2, -2, -2], True, 2, mats,
                  [(-1, g.bc(0, 0))], elem_coef=np.exp(rng.standard_normal(nx * ny * nz)))
    if len(shape) > 3:  # a sheared box: the elements stay translates, the lattice vectors are not orthogonal
        xyz = grid.nodes()
        xyz[:, 0] += 0.3 * xyz[:, 1] + 0.2 * xyz[:, 2]
        xyz[:, 1] += 0.15 * xyz[:, 2]
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble(g.GPZ_PREC_MIXED)
    x = rng.standard_normal(grid.neq)
    y64 = ctx.spmv(x)
    y32 = ctx.spmv_fp32(x, 10)
    assert ctx.tuning_report()["chosen"] == "matrix_free_shared_matrix_lattice_blocks"
    assert np.linalg.norm(y32 - y64) <= 1e-5 * np.linalg.norm(y64)
    y8 = ctx.spmv_fp32(x, 8)  # the tile operator: same products, another summation order
    assert np.linalg.norm(y32 - y8) <= 1e-6 * np.linalg.norm(y64)
    if nx * ny * nz <= 17 * 9 * 5:
        sol = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_BLOCK_JACOBI, tol=1e-8,
                        reliable_delta=1e-2, spmv_variant=10)
        ref = ctx.solve(tol=1e-12, max_iter=50000)
        assert sol["rc"] == 0 and sol["true_resid"] <= 1e-8
        assert np.linalg.norm(sol["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    ctx.close()


@pytest.mark.parametrize("case", ["darcy3d_p2", "poisson3d_box_p2"])
def test_scalar_shared_matrix_operator(built, case):
    """The scalar shared-element-matrix operator (3D Q2 Darcy / Poisson on translated hexes: K_e = k_e Khat as
    one tcgen05 3xTF32 GEMM per tile of 128 elements, penalty faces of every Dirichlet side) applies the
    assembled operator within 1e-5 of the FP64 SpMV, normwise and on the rows without a penalty, on a smooth
    field as well as a random one (the translation removed before the TF32 split keeps smooth fields exact);
    the mixed CG over it reaches a true FP64 residual of 1e-8 with a solution within 1e-8 of the oracle's
    tight solve, more tiles than SMs included (10^3 and 12^3 elements)."""
    g = _gpz()
    for mk in ((built[case][1]), (lambda: g.darcy(3, 12, 2, np.exp(np.random.default_rng(5).standard_normal(1728))))):
        grid = mk()
        ctx = g.Context(0)
        ctx.upload_mesh(grid)
        ctx.build_pattern(True)
        ctx.assemble(g.GPZ_PREC_MIXED)
        rng = np.random.default_rng(3)
        ia, ja = ctx.pattern()
        a = ctx.matrix()
        # the upper CSR: diagonal first in each row
        diag = np.array([a[ia[i]] for i in range(grid.neq)])
        inner = diag < 1e6 * np.median(diag)
        for x in (rng.standard_normal(grid.neq), 1.0 + 1e-3 * np.arange(grid.neq) / grid.neq):
            y64 = ctx.spmv(x)
            y32 = ctx.spmv_fp32(x, 9)
            assert np.linalg.norm(y32 - y64) <= 1e-5 * np.linalg.norm(y64)
            assert np.linalg.norm((y32 - y64)[inner]) <= 1e-5 * np.linalg.norm(y64[inner])
        tight = ctx.solve(tol=1e-12, max_iter=100000)
        mx = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, tol=1e-8, reliable_delta=1e-2, spmv_variant=9, max_iter=100000)
        assert mx["rc"] == 0 and mx["true_resid"] <= 1e-8 and mx["spmv_fp32"] > 0
        assert np.linalg.norm(mx["x"] - tight["x"]) <= 1e-8 * np.linalg.norm(tight["x"])
        ctx.close()


def test_shared_element_matrix_operator_more_tiles_than_sms(built):
    """The shared-element-matrix operator over more tiles of 128 elements than there are CTAs (each CTA
    loops over tiles, alternating its two TMEM accumulators) and a ragged last tile: 30^3 elements, 211 tiles."""
    g = _gpz()
    rng = np.random.default_rng(13)
    n = 30
    grid = g.elasticity3d(n, 2, E=np.exp(rng.standard_normal(n ** 3)))
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble(g.GPZ_PREC_MIXED)
    x = rng.standard_normal(grid.neq)
    y64 = ctx.spmv(x)
    y32 = ctx.spmv_fp32(x, 8)
    assert ctx.tuning_report()["chosen"] == "matrix_free_shared_matrix_tcgen05"
    assert np.linalg.norm(y32 - y64) <= 1e-5 * np.linalg.norm(y64)
    sol = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_BLOCK_JACOBI, tol=1e-8, reliable_delta=1e-2,
                    spmv_variant=8)
    ref = ctx.solve(tol=1e-12, max_iter=50000)
    assert sol["rc"] == 0 and sol["true_resid"] <= 1e-8
    assert np.linalg.norm(sol["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    ctx.close()


def test_distorted_mesh_general_quadrature_path(built):
    """Non-affine hexes (nodes moved): the per-point Jacobian path of the element kernel matches the oracle
    within 1e-12, and every FP32 operator layout still applies the assembled operator."""
    g = _gpz()
    rng = np.random.default_rng(31)
    n = 3
    E = np.exp(rng.standard_normal(n ** 3))
    om, grid = O.elasticity3d(n, 2, E=E), g.elasticity3d(n, 2, E=E)
    xyz = om.nodes()
    shift = 0.12 / n * rng.uniform(-1.0, 1.0, xyz.shape)
    moved = xyz + shift
    om.set_nodes(moved)
    gx = grid.nodes()
    assert np.array_equal(gx, xyz)
    gx[:] = moved
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble(g.GPZ_PREC_MIXED)
    ia, ja = ctx.pattern()
    oia, oja = om.pattern(False)
    assert np.array_equal(ia, oia) and np.array_equal(ja, oja)
    a, f = ctx.matrix(), ctx.rhs()
    oa, of = om.assemble(False, oia, oja)
    assert _row_rel(oia, a, oa) <= 1e-12
    assert np.max(np.abs(f - of)) <= 1e-12 * np.max(np.abs(of))
    assert ctx.assembly_report()["row_owner_pass"] is None  # no shared element matrix: the coloured scatter
    x = rng.standard_normal(grid.neq)
    y64 = ctx.spmv(x)
    for v in (0, 4, 5, 6, 7, 8):
        assert np.linalg.norm(ctx.spmv_fp32(x, v) - y64) <= 1e-5 * np.linalg.norm(y64), v
        if v == 8:  # elements of different Jacobians: no shared element matrix, another layout applies
            assert ctx.tuning_report()["chosen"] != "matrix_free_shared_matrix_tcgen05"
    ctx.close()


@pytest.mark.parametrize("case", ["elast3d_p2", "elast3d_p3", "darcy3d_p2", "poisson3d_box_p2", "elast3d_hp"])
def test_row_owner_assembly_of_shared_matrix_buckets(built, case):
    """A bucket whose elements are translates of one hex (K_e = c_e kref) is assembled row by row: one warp
    per (connect, shape) adds its elements' rows of c_e kref in shared memory and writes the rows once.  The
    matrix agrees with the oracle to 1e-12 of each row's largest entry (Q2 and Q3 elasticity, scalar Q2, a
    translated non-cubic box); the load vector stays that of the load-vector-only assembly, bit for bit.  On
    the hp mesh a uniform bucket may take the pass; the matrix is then cleared first for the other rows."""
    g = _gpz()
    mk_o, mk_g = built[case]
    om, grid = mk_o(), mk_g()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.assemble_rhs()
    f0 = ctx.rhs()
    ctx.build_pattern(False)
    ctx.assemble()
    rp = ctx.assembly_report()["row_owner_pass"]
    if case == "elast3d_hp":
        assert rp is None or rp["matrix_cleared"] is True
    else:
        assert rp is not None and rp["elements"] > 0 and rp["matrix_cleared"] is False
        assert rp["longest_row"] == max(np.diff(ctx.pattern()[0]))
    oia, oja = om.pattern(False)
    oa, of = om.assemble(False, oia, oja)
    assert _row_rel(oia, ctx.matrix(), oa) <= 1e-12
    assert np.array_equal(f0, ctx.rhs())
    a1 = ctx.matrix()
    ctx.assemble()  # the captured replay
    assert np.array_equal(a1, ctx.matrix())
    ctx.close()
