"""Block Jacobi with the reference's blocks in the device CG.

TPZAnalysis::BuildPreconditioner(EBlockJacobi, overlap) (Analysis/
TPZAnalysis.cpp:1008-1107): overlap = true takes one block per connect
(TPZBlockDiagonalStructMatrix), overlap = false the node-set blocks of
TPZNodesetCompute solved by TPZSparseBlockDiagonal.  On the device both are
variable-size blocks inverted by Gauss-Jordan without pivoting and applied by
the FP64 CG (GPZ_SOLVER_CG) and the mixed CG.  Against the oracle's block-LU CG
over the same blocks (orc_cg_sparse_block_jacobi): solution within 1e-8 and
iteration count within max(3, 10%) in FP64; the mixed CG reaches a true FP64
residual 1e-8 with a solution error at most 1e-8 against a tight FP64 solve.
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


def _connect_blocks(om):
    bp, bs = om.blocks()
    keep = bs > 0
    bi = np.concatenate([[0], np.cumsum(bs[keep])]).astype(np.int64)
    be = np.concatenate([np.arange(p, p + n) for p, n in zip(bp[keep], bs[keep])]).astype(np.int64)
    return bi, be


def _nodeset_blocks(g, grid):
    ei, eg = grid.element_graph()
    d = grid.desc
    nn = d.nconnects
    bp = np.ctypeslib.as_array(d.block_pos, shape=(nn,)).astype(np.int64)
    bs = np.ctypeslib.as_array(d.block_size, shape=(nn,)).astype(np.int64)
    r = g.nodeset_blocks(nn, ei, eg, bp, bs, grid.neq)
    return r["blockindex"], r["blockeqs"]


def _cases(g):
    n, nh = 6, 4
    E = g.lognormal(n ** 3, 1.0, 5)
    orders = g.hp_orders(nh ** 3, 3)
    Eh = g.lognormal(nh ** 3, 0.5, 3)
    return {
        "elast3d_q2": (lambda: O.elasticity3d(n, 2, E=E, body_force=(0, 0, 0)),
                       lambda: g.elasticity3d(n, 2, E=E, body_force=(0.0, 0.0, 0.0))),
        "elast3d_hp": (lambda: O.elasticity3d_hp(nh, orders, E=Eh), lambda: g.elasticity3d_hp(nh, orders, E=Eh)),
    }


@pytest.mark.parametrize("kind", ["nodeset", "connect"])
@pytest.mark.parametrize("case", ["elast3d_q2", "elast3d_hp"])
def test_block_jacobi_cg_matches_oracle_block_lu(g, case, kind):
    mk_o, mk_g = _cases(g)[case]
    om, grid = mk_o(), mk_g()
    bi, be = _nodeset_blocks(g, grid) if kind == "nodeset" else _connect_blocks(om)
    if kind == "nodeset":
        assert np.diff(bi).max() > 3  # blocks larger than a connect exist
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    ctx.assemble()
    tol = 1e-10
    pre = g.GPZ_PRECOND_NODESET_JACOBI if kind == "nodeset" else g.GPZ_PRECOND_BLOCK_JACOBI
    sol = ctx.solve(precond=pre, tol=tol, max_iter=20000)
    ia, ja = om.pattern(True)
    a, f = om.assemble(True, ia, ja)
    ref = O.cg_sparse_block_jacobi(True, ia, ja, a, f, bi, be, 20000, tol)
    assert sol["rc"] == 0 and ref["rc"] == 0
    assert np.linalg.norm(sol["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    assert abs(sol["iterations"] - ref["iters"]) <= max(3, 0.1 * ref["iters"]), (sol["iterations"], ref["iters"])
    # the mixed CG with the same blocks: true FP64 residual 1e-8, solution within 1e-8 of a tight FP64 solve
    tight = ctx.solve(tol=1e-13, max_iter=50000)
    ctx.assemble(g.GPZ_PREC_MIXED)
    mx = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=pre, tol=1e-8, max_iter=20000, reliable_delta=1e-2)
    assert mx["rc"] == 0 and mx["true_resid"] <= 1e-8 and mx["spmv_fp32"] > 0
    assert np.linalg.norm(mx["x"] - tight["x"]) <= 1e-8 * np.linalg.norm(tight["x"])
    ctx.close()


def test_nodeset_blocks_fewer_iterations_than_connect_blocks_on_hp(g):
    """On the hp mesh the node-set blocks merge higher-order connects with their neighbours' and the CG needs
    markedly fewer iterations than with the connect blocks (the oracle: 189 against 264 at 4^3)."""
    mk_o, mk_g = _cases(g)["elast3d_hp"]
    grid = mk_g()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    ctx.assemble()
    ns = ctx.solve(precond=g.GPZ_PRECOND_NODESET_JACOBI, tol=1e-8, max_iter=20000, want_x=False)
    cb = ctx.solve(precond=g.GPZ_PRECOND_BLOCK_JACOBI, tol=1e-8, max_iter=20000, want_x=False)
    assert ns["rc"] == 0 and cb["rc"] == 0
    assert ns["iterations"] < 0.85 * cb["iterations"], (ns["iterations"], cb["iterations"])
    ctx.close()


def test_nodeset_preconditioner_refused_where_not_built(g):
    """GMRES and the stationary Jacobi iteration take no node-set blocks; under an equation filter the blocks
    would be split: each returns GPZ_E_INVALID and the context stays usable."""
    grid = g.elasticity3d(3, 2)
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    ctx.assemble()
    for solver in (g.GPZ_SOLVER_GMRES, g.GPZ_SOLVER_JACOBI):
        with pytest.raises(g.GpzError) as e:
            ctx.solve(solver=solver, precond=g.GPZ_PRECOND_NODESET_JACOBI, tol=1e-8)
        assert e.value.code == -1
    assert ctx.solve(precond=g.GPZ_PRECOND_NODESET_JACOBI, tol=1e-10)["rc"] == 0
    ctx.close()
