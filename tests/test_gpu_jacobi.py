"""The stationary Jacobi solver on the GPU (gpz_solve with GPZ_SOLVER_JACOBI: TPZStepSolver::SetJacobi as the
solver, Solvers/pzstepsolver.cpp:94-98) against the oracle's restatement of TPZMatrix::SolveJacobi
(Matrix/pzmatrix.cpp:643-667, symmetric pattern) and of the TPZFYsmpMatrix override (Matrix/pzysmp.cpp:725-781,
full pattern).

Tolerances: after a fixed number of sweeps the iterates agree within 1e-12 relative to max |x| (the GPU sums
each row in its own order, the oracle's symmetric product adds the transposed upper entries); a converged solve
stops on the absolute ||b - A x|| at the oracle's sweep count within 1 and its solution agrees within 1e-8; a
divergent iteration (3D Q1 elasticity: Jacobi's iteration matrix has spectral radius above one) stops where the
norm stops being a number, within one sweep of the oracle.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _gpz():
    from neopz_gb300 import gpz
    return gpz


@pytest.fixture(scope="module")
def built():
    import __graft_entry__
    __graft_entry__.build()
    return True


def _setup(om, grid, sym):
    g = _gpz()
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(sym)
    ctx.assemble(g.GPZ_PREC_FP64)
    ia, ja = om.pattern(sym)
    a, f = om.assemble(sym, ia, ja)
    return ctx, (ia, ja, a, f)


def _jac(ctx, **kw):
    g = _gpz()
    return ctx.solve(solver=g.GPZ_SOLVER_JACOBI, precond=0, **kw)


@pytest.mark.parametrize("sym", [True, False])
@pytest.mark.parametrize("case", ["poisson2d_p2", "elast3d_p2"])
def test_jacobi_sweeps_match_oracle(built, case, sym):
    g = _gpz()
    rng = np.random.default_rng(3)
    E = np.exp(rng.standard_normal(27))
    om, grid = {"poisson2d_p2": (O.poisson2d(8, 2), g.poisson2d(8, 2)),
                "elast3d_p2": (O.elasticity3d(3, 2, E=E), g.elasticity3d(3, 2, E=E))}[case]
    ctx, (ia, ja, a, f) = _setup(om, grid, sym)
    for k in (1, 7, 40):
        out = _jac(ctx, max_iter=k, tol=0.0)
        ref = O.jacobi(sym, ia, ja, a, f, k, 0.0)
        assert out["iterations"] == ref["iters"] == k
        scale = np.max(np.abs(ref["x"]))
        assert np.max(np.abs(out["x"] - ref["x"])) <= 1e-12 * scale, k
        assert out["spmv_fp64"] == k + 1  # the sweeps and the final true residual
    # FromCurrent: 7 sweeps from the 40-sweep iterate are 47 sweeps from zero
    x40 = _jac(ctx, max_iter=40, tol=0.0)["x"]
    out = _jac(ctx, max_iter=7, tol=0.0, x0=x40)
    ref = O.jacobi(sym, ia, ja, a, f, 47, 0.0)
    assert out["iterations"] == 7
    assert np.max(np.abs(out["x"] - ref["x"])) <= 1e-12 * np.max(np.abs(ref["x"]))
    # graph replay and eager launches, any batch length: the same bits
    e1 = _jac(ctx, max_iter=23, tol=0.0, use_graph=False, check_every=5)
    e2 = _jac(ctx, max_iter=23, tol=0.0, use_graph=True, check_every=32)
    assert np.array_equal(e1["x"], e2["x"])
    ctx.close()


@pytest.mark.parametrize("sym", [True, False])
def test_jacobi_edge_cases(built, sym):
    """numiterations = 0 and an initial residual within the tolerance: no sweep through TPZMatrix::SolveJacobi,
    one sweep (x = b / diag) through the TPZFYsmpMatrix override."""
    g = _gpz()
    om, grid = O.poisson2d(8, 1), g.poisson2d(8, 1)
    ctx, (ia, ja, a, f) = _setup(om, grid, sym)
    big = 2 * np.linalg.norm(f)
    # the device's own values (the same pattern as the oracle's, values within 1e-12) give b / diag exactly
    gf, ga = ctx.rhs(), ctx.matrix()
    gd = np.array([ga[ia[r] + np.searchsorted(ja[ia[r]:ia[r + 1]], r)] for r in range(len(ia) - 1)])
    for maxit, tol in ((0, 0.0), (10, big)):
        out = _jac(ctx, max_iter=maxit, tol=tol)
        ref = O.jacobi(sym, ia, ja, a, f, maxit, tol)
        assert out["iterations"] == ref["iters"] == (0 if sym else 1)
        if sym:
            assert np.all(out["x"] == 0.0) and np.all(ref["x"] == 0.0)
        else:
            assert np.array_equal(out["x"], gf / gd)  # correctly rounded division on both sides
            assert np.max(np.abs(out["x"] - ref["x"])) <= 1e-12 * np.max(np.abs(ref["x"]))
    ctx.close()


@pytest.mark.parametrize("sym", [True, False])
def test_jacobi_converges_like_oracle(built, sym):
    g = _gpz()
    om, grid = O.poisson2d(16, 1), g.poisson2d(16, 1)
    ctx, (ia, ja, a, f) = _setup(om, grid, sym)
    tol = 1e-9 * np.linalg.norm(f)
    out = _jac(ctx, max_iter=100000, tol=tol)
    ref = O.jacobi(sym, ia, ja, a, f, 100000, tol)
    assert out["rc"] == g.GPZ_OK and ref["rc"] == 0
    assert abs(out["iterations"] - ref["iters"]) <= 1, (out["iterations"], ref["iters"])
    assert np.linalg.norm(out["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    assert out["true_resid"] * np.linalg.norm(f) <= 1.01 * tol
    # the budget is honoured: not converged after 50 sweeps
    short = _jac(ctx, max_iter=50, tol=tol)
    assert short["rc"] == g.GPZ_NOT_CONVERGED and short["iterations"] == 50
    ctx.close()


def test_jacobi_divergence_stops_like_oracle(built):
    g = _gpz()
    om, grid = O.elasticity3d(3, 1), g.elasticity3d(3, 1)
    ctx, (ia, ja, a, f) = _setup(om, grid, True)
    tol = 1e-9 * np.linalg.norm(f)
    ref = O.jacobi(True, ia, ja, a, f, 20000, tol)
    assert ref["rc"] == 1 and np.isnan(ref["resid"]) and ref["iters"] < 20000
    out = _jac(ctx, max_iter=20000, tol=tol)
    assert out["rc"] == g.GPZ_NOT_CONVERGED
    assert abs(out["iterations"] - ref["iters"]) <= 1, (out["iterations"], ref["iters"])
    ctx.close()
