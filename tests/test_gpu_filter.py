"""The equation filter on the GPU (gpz_equation_filter: TPZEquationFilter::SetActiveEquations / Reset on the
structural matrix, StrMatrix/TPZEquationFilter.h) against the oracle's restatement (oracle.filter_system).

Tolerances: the condensed pattern bit-exact (IA, JA); values per row within 1e-12 of the row's largest entry;
the mesh-size load vector within 1e-12 of its largest entry, zeros at the inactive equations exactly; Jacobi-PCG
solutions of the condensed system within 1e-8; the mixed CG (FP32 CSR copy: a filter may split the connect
blocks) to a true FP64 residual of 1e-8.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GPZ_E_INVALID = -1


def _gpz():
    from neopz_gb300 import gpz
    return gpz


@pytest.fixture(scope="module")
def built():
    import __graft_entry__
    __graft_entry__.build()
    return True


def _case(g, name):
    rng = np.random.default_rng(13)
    E = np.exp(rng.standard_normal(27))
    k = np.exp(rng.standard_normal(64))
    return {"elast3d_p2": (O.elasticity3d(3, 2, E=E), g.elasticity3d(3, 2, E=E)),
            "poisson2d_p2": (O.poisson2d(8, 2), g.poisson2d(8, 2)),
            "darcy2d_p3": (O.darcy(2, 8, 3, k), g.darcy(2, 8, 3, k))}[name]


@pytest.mark.parametrize("sym", [True, False])
@pytest.mark.parametrize("case", ["elast3d_p2", "poisson2d_p2", "darcy2d_p3"])
def test_filtered_system_matches_oracle(built, case, sym):
    g = _gpz()
    om, grid = _case(g, case)
    rng = np.random.default_rng(2)
    active = rng.choice(om.neq, size=int(0.8 * om.neq), replace=False)  # splits connect blocks too
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.equation_filter(active)
    nnz = ctx.build_pattern(sym)
    ia, ja = ctx.pattern()
    oia, oja = om.pattern(sym)
    oa, of = om.assemble(sym, oia, oja)
    cia, cja, ca, fm, fc = O.filter_system(sym, oia, oja, oa, of, active)
    assert ctx.neq == len(cia) - 1 and nnz == len(cja)
    assert np.array_equal(ia, cia) and np.array_equal(ja, cja)
    ctx.assemble(g.GPZ_PREC_MIXED)
    a, f = ctx.matrix(), ctx.rhs()
    for r in range(ctx.neq):
        s, e = cia[r], cia[r + 1]
        assert np.max(np.abs(a[s:e] - ca[s:e])) <= 1e-12 * np.max(np.abs(ca[s:e]))
    inactive = np.setdiff1d(np.arange(om.neq), active)
    assert f.shape == (om.neq,) and np.all(f[inactive] == 0.0)
    assert np.max(np.abs(f - fm)) <= 1e-12 * np.max(np.abs(fm))
    # the solves work on the condensed system; b = None gathers the active load entries
    ref = O.cg_jacobi(sym, cia, cja, ca, fc, 20000, 1e-11)
    cg = ctx.solve(tol=1e-11, max_iter=20000)
    assert cg["rc"] == 0 and ref["rc"] == 0 and cg["x"].shape == (ctx.neq,)
    assert np.linalg.norm(cg["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    mx = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, tol=1e-8, max_iter=20000, reliable_delta=1e-2)
    assert mx["rc"] == 0 and mx["true_resid"] <= 1e-8
    assert np.linalg.norm(mx["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    z = ctx.spmv(ref["x"])
    zr = O.spmv(sym, cia, cja, ca, ref["x"])
    assert np.max(np.abs(z - zr)) <= 1e-11 * np.max(np.abs(zr))
    ctx.close()


def test_filter_error_norms_reset_and_refusals(built):
    g = _gpz()
    om, grid = _case(g, "elast3d_p2")
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    active = np.arange(0, om.neq, 2)
    ctx.equation_filter(active)
    # the load vector alone, before any pattern: zeros at the inactive equations
    assert ctx.assemble_rhs() == g.GPZ_OK
    oia, oja = om.pattern(True)
    _, of = om.assemble(True, oia, oja)
    fm = of.copy()
    fm[1::2] = 0.0
    f0 = ctx.rhs()
    assert np.all(f0[1::2] == 0.0) and np.max(np.abs(f0 - fm)) <= 1e-12 * np.max(np.abs(fm))
    ctx.build_pattern(True)
    ctx.assemble()
    x = ctx.solve(tol=1e-10, max_iter=20000)["x"]
    # the device solution is scattered to the mesh equations for the error norms
    xs = np.zeros(om.neq)
    xs[active] = x
    exact = lambda p: (np.zeros((len(p), 3)), np.zeros((len(p), 3, 3)))  # noqa: E731
    t_dev, _ = ctx.evaluate_error(exact, 2)
    t_host, _ = ctx.evaluate_error(exact, 2, sol=xs)
    assert np.array_equal(t_dev, t_host) and np.all(t_dev[:3] > 0)
    # connect blocks are split: block Jacobi and the learned preconditioner refuse
    with pytest.raises(g.GpzError) as e:
        ctx.solve(precond=g.GPZ_PRECOND_BLOCK_JACOBI)
    assert e.value.code == GPZ_E_INVALID
    with pytest.raises(g.GpzError) as e:
        ctx.learned_init(rank=8, seed=0)
    assert e.value.code == GPZ_E_INVALID
    # Reset: the full system again, as without a filter
    ctx.equation_filter(None)
    ctx.build_pattern(True)
    ia, ja = ctx.pattern()
    assert np.array_equal(ia, oia) and np.array_equal(ja, oja) and ctx.neq == om.neq
    ctx.assemble()
    r = ctx.solve(tol=1e-10, max_iter=20000)
    assert r["rc"] == 0 and r["x"].shape == (om.neq,)
    ctx.close()
