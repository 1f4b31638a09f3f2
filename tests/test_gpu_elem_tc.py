"""FP32 element matrices formed on the tensor cores (gpz_fp32_elements(GPZ_FP32_ELEMENTS)).

With that source the mixed assembly forms every volume hex's matrix again as one tcgen05 GEMM (the gradient
Gram X X^T, 3xTF32, FP32 accumulation; FP32 Jacobians) and the other elements (penalty faces, 2D quads) by
the FP64 element kernel with an FP32 scatter, into the FP32 CSR the mixed solves read.

Tolerances (written here): the FP32 values within 1e-5 of each row's largest entry against the oracle's
FP64 assembly (FP32 rounding of the geometry and of the products, summed over up to eight elements); the
FP32 operator built from them within 1e-5 (2-norm) of the FP64 SpMV in every assembled layout; the mixed
CG over them to a true FP64 residual of 1e-8 with the solution within 1e-8 of the FP64 solution.  The FP64
matrix of the same assembly stays the parity one (1e-12).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import __graft_entry__
    __graft_entry__.build()
    from neopz_gb300 import gpz
    return gpz


def _row_rel(ia, a, ref):
    worst = 0.0
    for r in range(len(ia) - 1):
        s, e = ia[r], ia[r + 1]
        m = np.max(np.abs(ref[s:e]))
        if m > 0:
            worst = max(worst, np.max(np.abs(a[s:e] - ref[s:e])) / m)
    return worst


def _distort(om, grid, seed, amount):
    rng = np.random.default_rng(seed)
    xyz = om.nodes()
    moved = xyz + amount * rng.uniform(-1.0, 1.0, xyz.shape)
    om.set_nodes(moved)
    gx = grid.nodes()
    gx[:] = moved


def _case(g, name):
    rng = np.random.default_rng(23)
    if name == "elast3d_p1":
        E = np.exp(rng.standard_normal(27))
        return O.elasticity3d(3, 1, E=E), g.elasticity3d(3, 1, E=E)
    if name == "elast3d_p2":
        E = np.exp(rng.standard_normal(27))
        return O.elasticity3d(3, 2, E=E), g.elasticity3d(3, 2, E=E)
    if name == "elast3d_p3":
        return O.elasticity3d(2, 3), g.elasticity3d(2, 3)
    if name == "elast3d_hp":
        o = g.hp_orders(27, 3)
        E = np.exp(0.5 * rng.standard_normal(27))
        return O.elasticity3d_hp(3, o, E=E), g.elasticity3d_hp(3, o, E=E)
    if name == "elast3d_p2_distorted":
        E = np.exp(rng.standard_normal(27))
        om, grid = O.elasticity3d(3, 2, E=E), g.elasticity3d(3, 2, E=E)
        _distort(om, grid, 31, 0.04)
        return om, grid
    if name == "darcy3d_p2":
        k = np.exp(rng.standard_normal(64))
        return O.darcy(3, 4, 2, k), g.darcy(3, 4, 2, k)
    if name == "darcy3d_hp":  # 3D hp Darcy: scalar hp classes of order 2 and 3
        k = np.exp(rng.standard_normal(27))
        o = g.hp_orders(27, 9)
        matids = [1, -1, -1, -1, -1, -1, -1]
        om = O.OracleMesh(3, (3, 3, 3), (0, 0, 0), (1, 1, 1), matids, True, 1,
                          [O.material(1, O.ORC_DARCY, 3, forcing=O.ORC_F_CONST, force=(1.0, 0, 0))], [O.bc(-1, 1, 0)],
                          elem_coef=k, elem_order=o)
        grid = g.Grid(3, (3, 3, 3), (0, 0, 0), (1, 1, 1), matids, True, 1,
                      [(1, g.material(g.GPZ_MAT_DARCY, 3, forcing=g.GPZ_F_CONST, force=(1.0, 0, 0)))],
                      [(-1, g.bc(0, 0))], elem_coef=k, elem_order=o)
        return om, grid
    if name == "poisson2d_p2":  # no hexes: every element through the FP32 scatter of the FP64 kernel
        return O.poisson2d(16, 2), g.poisson2d(16, 2)
    raise KeyError(name)


CASES = ["elast3d_p1", "elast3d_p2", "elast3d_p3", "elast3d_hp", "elast3d_p2_distorted", "darcy3d_p2",
         "darcy3d_hp", "poisson2d_p2"]


@pytest.mark.parametrize("case", CASES)
def test_fp32_element_matrices_match_the_oracle(g, case):
    om, grid = _case(g, case)
    oia, oja = om.pattern(False)
    oa, of = om.assemble(False, oia, oja)
    ctx = g.Context(0)
    ctx.fp32_elements(g.GPZ_FP32_ELEMENTS)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble(g.GPZ_PREC_MIXED)
    ia, ja = ctx.pattern()
    assert np.array_equal(ia, oia) and np.array_equal(ja, oja)
    assert _row_rel(oia, ctx.matrix(), oa) <= 1e-12  # the FP64 matrix of the same assembly
    a32 = ctx.matrix_fp32().astype(np.float64)
    err = _row_rel(oia, a32, oa)
    print(f"{case}: FP32 element matrices, worst row-relative difference {err:.3e}")
    assert err <= 1e-5
    rep = ctx.assembly_report()["fp32_elements"]
    assert rep["tensor_core_elements"] == (grid.nvol if grid.desc.dim == 3 else 0)
    assert rep["tensor_core_elements"] + rep["cuda_core_elements"] == grid.nel
    # every assembled layout of the FP32 operator reads these values
    x = np.random.default_rng(5).standard_normal(grid.neq)
    y64 = ctx.spmv(x)
    for v in ((0, 1, 2, 3, 4) if grid.desc.nstate == 3 else (0,)):
        assert np.linalg.norm(ctx.spmv_fp32(x, v) - y64) <= 1e-5 * np.linalg.norm(y64), v
    ctx.close()


@pytest.mark.parametrize("case", ["elast3d_p2_distorted_8", "elast3d_hp_4"])
def test_mixed_cg_over_tensor_core_element_matrices(g, case):
    rng = np.random.default_rng(41)
    if case == "elast3d_p2_distorted_8":
        n = 8
        E = np.exp(rng.standard_normal(n ** 3))
        grid = g.elasticity3d(n, 2, E=E)
        gx = grid.nodes()
        gx[:] = gx + 0.3 / n * rng.uniform(-1.0, 1.0, gx.shape) * (gx > 1e-12) * (gx < 1 - 1e-12)
    else:
        n = 4
        grid = g.elasticity3d_hp(n, g.hp_orders(n ** 3, 7), E=np.exp(0.5 * rng.standard_normal(n ** 3)))
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble(g.GPZ_PREC_FP64)
    ref = ctx.solve(solver=g.GPZ_SOLVER_CG, precond=g.GPZ_PRECOND_JACOBI, tol=1e-13, max_iter=100000)
    assert ref["rc"] == 0
    ctx.fp32_elements(g.GPZ_FP32_ELEMENTS)
    ctx.assemble(g.GPZ_PREC_MIXED)
    assert ctx.assembly_report()["fp32_elements"]["tensor_core_elements"] > 0
    sol = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_BLOCK_JACOBI, tol=1e-8, max_iter=100000,
                    reliable_delta=1e-2, spmv_variant=0)
    assert sol["rc"] == 0 and sol["true_resid"] <= 1e-8
    assert np.linalg.norm(sol["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    # the same solve over the rounded FP64 matrix takes about as many iterations
    ctx.fp32_elements(g.GPZ_FP32_ROUNDED)
    ctx.assemble(g.GPZ_PREC_MIXED)
    rnd = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_BLOCK_JACOBI, tol=1e-8, max_iter=100000,
                    reliable_delta=1e-2, spmv_variant=0)
    assert rnd["rc"] == 0
    print(f"{case}: mixed CG iterations over the FP32 element pass {sol['iterations']}, "
          f"over the rounded FP64 matrix {rnd['iterations']}")
    assert abs(sol["iterations"] - rnd["iterations"]) <= max(3, 0.05 * rnd["iterations"])
    ctx.close()
