"""Edge cases of the C ABI on the GPU: call-order violations and bad mesh descriptors are rejected with their
status codes before any device work and leave the context usable; a zero load vector is converged at entry for
every solver (cg.h:29-132 takes ||b|| = 1 when b = 0, so the initial residual 0 meets any tolerance); the
smallest meshes (one element) give the oracle's pattern bit-exactly and its values within 1e-12.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GPZ_E_INVALID, GPZ_E_UNSUPPORTED_ELEMENT, GPZ_E_NOT_READY = -1, -5, -6


def _gpz():
    from neopz_gb300 import gpz
    return gpz


@pytest.fixture(scope="module")
def built():
    import __graft_entry__
    __graft_entry__.build()
    return True


def _raises(code, fn, *a, **kw):
    g = _gpz()
    with pytest.raises(g.GpzError) as e:
        fn(*a, **kw)
    assert e.value.code == code, (e.value.code, code)


def test_call_order_and_bad_descriptors(built):
    g = _gpz()
    ctx = g.Context(0)
    _raises(GPZ_E_NOT_READY, ctx.build_pattern, True)
    grid = g.poisson2d(4, 2)
    d = grid.desc
    for arr, idx, bad, code in ((d.el_conn, 3, d.nconnects, GPZ_E_INVALID), (d.el_conn, 5, -1, GPZ_E_INVALID),
                                (d.el_nodes, 2, d.nnodes, GPZ_E_INVALID),
                                (d.el_order, 0, 4, GPZ_E_UNSUPPORTED_ELEMENT)):
        old = arr[idx]
        arr[idx] = bad
        _raises(code, ctx.upload_mesh, grid)
        arr[idx] = old
    ctx.upload_mesh(grid)
    _raises(GPZ_E_NOT_READY, ctx.assemble)
    ctx.build_pattern(True)
    _raises(GPZ_E_NOT_READY, ctx.solve)
    ctx.assemble()
    _raises(GPZ_E_INVALID, ctx.solve, max_iter=-1)
    _raises(GPZ_E_INVALID, ctx.solve, solver=99)
    _raises(GPZ_E_INVALID, ctx.solve, solver=g.GPZ_SOLVER_JACOBI, precond=g.GPZ_PRECOND_BLOCK_JACOBI)
    r = ctx.solve(tol=1e-10)
    assert r["rc"] == g.GPZ_OK
    ctx.close()


@pytest.mark.parametrize("sym", [True, False])
def test_zero_load_vector_converges_at_entry(built, sym):
    g = _gpz()
    ctx = g.Context(0)
    ctx.upload_mesh(g.elasticity3d(2, 2))
    ctx.build_pattern(sym)
    ctx.assemble(g.GPZ_PREC_MIXED)
    b = np.zeros(ctx.neq)
    for solver in (g.GPZ_SOLVER_CG, g.GPZ_SOLVER_MIXED_CG, g.GPZ_SOLVER_GMRES, g.GPZ_SOLVER_JACOBI):
        r = ctx.solve(solver=solver, precond=0 if solver == g.GPZ_SOLVER_JACOBI else g.GPZ_PRECOND_JACOBI, b=b,
                      tol=1e-12)
        assert r["rc"] == g.GPZ_OK, solver
        if sym or solver != g.GPZ_SOLVER_JACOBI:
            assert r["iterations"] == 0, (solver, r["iterations"])
        assert np.all(r["x"] == 0.0), solver  # the full-pattern Jacobi's forced sweep adds 0 / a_ii
    ctx.close()


@pytest.mark.parametrize("case", ["poisson2d_p1", "poisson2d_p3", "darcy3d_p2", "elast3d_p1", "elast3d_p3"])
@pytest.mark.parametrize("sym", [True, False])
def test_single_element_meshes(built, case, sym):
    g = _gpz()
    om, grid = {"poisson2d_p1": (O.poisson2d(1, 1), g.poisson2d(1, 1)),
                "poisson2d_p3": (O.poisson2d(1, 3), g.poisson2d(1, 3)),
                "darcy3d_p2": (O.darcy(3, 1, 2, np.array([2.5])), g.darcy(3, 1, 2, np.array([2.5]))),
                "elast3d_p1": (O.elasticity3d(1, 1), g.elasticity3d(1, 1)),
                "elast3d_p3": (O.elasticity3d(1, 3), g.elasticity3d(1, 3))}[case]
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(sym)
    ia, ja = ctx.pattern()
    oia, oja = om.pattern(sym)
    assert np.array_equal(ia, oia) and np.array_equal(ja, oja)
    ctx.assemble()
    oa, of = om.assemble(sym, oia, oja)
    a, f = ctx.matrix(), ctx.rhs()
    for r in range(om.neq):
        s, e = oia[r], oia[r + 1]
        assert np.max(np.abs(a[s:e] - oa[s:e])) <= 1e-12 * np.max(np.abs(oa[s:e]))
    assert np.max(np.abs(f - of)) <= 1e-12 * max(np.max(np.abs(of)), 1e-300)
    sol = ctx.solve(tol=1e-12, max_iter=10000)
    ref = O.cg_jacobi(sym, oia, oja, oa, of, 10000, 1e-12)
    assert sol["rc"] == 0 and ref["rc"] == 0
    assert np.linalg.norm(sol["x"] - ref["x"]) <= 1e-8 * max(np.linalg.norm(ref["x"]), 1e-300)
    ctx.close()
