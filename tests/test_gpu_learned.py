"""The learned preconditioner on the GPU (libgpz.so, through its C ABI).

* gradient check: the GPU forward / backward kernels (FP32 network, FP64
  loss) against the float64 numpy oracle -- loss within 1e-4, gradient within
  1e-3 relative in norm, per parameter block;
* training on the GPU lowers the loss, and the trained network gains over
  the method without it: flexible CG with the learned preconditioner needs at
  most 75% of the Jacobi-PCG iterations on unseen coefficient fields (64 x 64
  Q2 Darcy, GRF permeability, 40 training fields), also with the FP32-value
  SpMV (learned + mixed), reaching
  the same true FP64 residual; at a tight tolerance its solution matches the
  oracle's CG solution within 1e-8;
* Jacobi stays the fallback: with a broken network every iteration falls
  back to Jacobi and the solve still converges;
* against the block-Jacobi mixed CG (the method without the network on the
  same base), the committed elasticity weights cut the iterations on unseen
  16^3 fields.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O
from oracle import learned_oracle as LO

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import __graft_entry__
    __graft_entry__.build()
    from neopz_gb300 import gpz
    return gpz


def _ctx(g, grid):
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble()
    return ctx


def test_learned_gradient_matches_oracle(g):
    n, R = 4, 4
    k = g.grf2d(n, seed=5)
    grid = g.darcy(2, n, 2, k)
    ctx = _ctx(g, grid)
    npar = ctx.learned_init(rank=R, seed=1)
    rng = np.random.default_rng(0)
    p = (0.3 * rng.standard_normal(npar)).astype(np.float32)
    ctx.set_learned_params(p)
    P = 3
    Rs, Es = rng.standard_normal((P, grid.neq)), rng.standard_normal((P, grid.neq))
    ctx.learned_set_pairs(Rs, Es)
    loss, grad = ctx.learned_loss_grad()
    ia, ja = ctx.pattern()
    A = sp.csr_matrix((ctx.matrix(), ja, ia), shape=(grid.neq, grid.neq))
    om = O.darcy(2, n, 2, k)
    mesh = LO.mesh_from_oracle(om, A, k)
    lref, gref = LO.loss_and_grad(mesh, A, p.astype(np.float64), R, Rs, Es)
    assert abs(loss - lref) <= 1e-4 * abs(lref), (loss, lref)
    off, _ = LO.layout(mesh.NS, R)
    for name, (a, m) in off.items():
        d = np.linalg.norm(grad[a:a + m] - gref[a:a + m])
        assert d <= 1e-3 * max(np.linalg.norm(gref[a:a + m]), 1e-6 * np.linalg.norm(gref)), name
    ctx.close()


def test_learned_training_gains_over_jacobi(g):
    n = 64
    grid = g.darcy(2, n, 2, g.grf2d(n, seed=0))
    ctx = _ctx(g, grid)
    ctx.learned_init(rank=4, seed=0)
    from neopz_gb300 import learned
    first, last, _, hist = learned.train(ctx, grid, lambda s: g.grf2d(n, seed=s), range(1, 41), val_every=10)
    assert hist[-1]["kept_fields"] in (10, 20, 30, 40)
    assert last < 0.95 * first, (first, last)  # per-field losses differ; the iteration gain below is the test
    for s in (10000, 10001, 10002):
        k = g.grf2d(n, seed=s)
        ctx.set_coef(grid, k)
        ctx.assemble()
        jac = ctx.solve(tol=1e-8)
        lrn = ctx.solve(solver=g.GPZ_SOLVER_LEARNED_FCG, tol=1e-8)
        assert jac["rc"] == 0 and lrn["rc"] == 0
        assert lrn["true_resid"] <= 1e-8 and lrn["restarts"] == 0
        assert lrn["iterations"] <= 0.75 * jac["iterations"], (s, lrn["iterations"], jac["iterations"])
        # learned + mixed: FP32-value SpMV, FP64 true-residual replacement; same true tolerance
        mx = ctx.solve(solver=g.GPZ_SOLVER_LEARNED_MIXED_FCG, tol=1e-8, reliable_delta=1e-2)
        assert mx["rc"] == 0 and mx["true_resid"] <= 1e-8 and mx["spmv_fp32"] > 0 and mx["reliable_updates"] >= 1
        assert mx["iterations"] <= 0.8 * jac["iterations"], (s, mx["iterations"], jac["iterations"])
        tight = ctx.solve(solver=g.GPZ_SOLVER_LEARNED_FCG, tol=1e-11)
        om = O.darcy(2, n, 2, k)
        oia, oja = om.pattern(True)
        oa, of = om.assemble(True, oia, oja)
        ref = O.cg_jacobi(True, oia, oja, oa, of, 20000, 1e-12)
        assert np.linalg.norm(tight["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
        # true residual 1e-8; the solution error against the FP64 oracle's tight solve is held to 1e-8
        assert np.linalg.norm(mx["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    ctx.close()


def test_learned_falls_back_to_jacobi(g):
    n = 16
    grid = g.darcy(2, n, 2, g.grf2d(n, seed=2))
    ctx = _ctx(g, grid)
    npar = ctx.learned_init(rank=4, seed=0)
    ctx.set_learned_params(np.full(npar, np.nan, np.float32))
    jac = ctx.solve(tol=1e-8)
    lrn = ctx.solve(solver=g.GPZ_SOLVER_LEARNED_FCG, tol=1e-8)
    assert lrn["rc"] == 0 and lrn["true_resid"] <= 1e-8
    assert lrn["restarts"] >= lrn["iterations"]  # every application fell back
    assert abs(lrn["iterations"] - jac["iterations"]) <= max(3, 0.1 * jac["iterations"])
    ctx.close()


def test_learned_gradient_matches_oracle_elasticity(g):
    """The same check on 3D Q2 elasticity (81 equations per element, rank 8): every kernel of the 3-state,
    rank-8 path (element gathers, dF outer products, the output layer) against the numpy oracle."""
    n, R = 2, 8
    rng = np.random.default_rng(3)
    E = np.exp(rng.standard_normal(n ** 3))
    grid = g.elasticity3d(n, 2, E=E, top_traction=False)  # penalty-Dirichlet base only: the mask of both sides
    ctx = _ctx(g, grid)
    npar = ctx.learned_init(rank=R, seed=2)
    p = (0.2 * rng.standard_normal(npar)).astype(np.float32)
    ctx.set_learned_params(p)
    P = 2
    Rs, Es = rng.standard_normal((P, grid.neq)), rng.standard_normal((P, grid.neq))
    ctx.learned_set_pairs(Rs, Es)
    loss, grad = ctx.learned_loss_grad()
    ia, ja = ctx.pattern()
    A = sp.csr_matrix((ctx.matrix(), ja, ia), shape=(grid.neq, grid.neq))
    om = O.elasticity3d(n, 2, E=E, top_traction=False)
    mesh = LO.mesh_from_oracle(om, A, E)
    lref, gref = LO.loss_and_grad(mesh, A, p.astype(np.float64), R, Rs, Es)
    assert abs(loss - lref) <= 1e-4 * abs(lref), (loss, lref)
    off, _ = LO.layout(mesh.NS, R)
    for name, (a, m) in off.items():
        d = np.linalg.norm(grad[a:a + m] - gref[a:a + m])
        assert d <= 1e-3 * max(np.linalg.norm(gref[a:a + m]), 1e-6 * np.linalg.norm(gref)), name
    ctx.close()


def test_learned_elasticity_weights_gain_and_mixed_path(g):
    """The committed elasticity weights (trained on the GPU on 200 seeded 16^3 fields, neopz_gb300/data) on unseen 16^3
    fields: the learned flexible CG needs at most 85% of the Jacobi-PCG iterations; the learned + mixed
    path (the mixed CG's FP32 operator chosen by the autotuner, FP32 recurrence, FP64 true-residual
    replacement) reaches the same true residual 1e-8 in about as many iterations, and its solution is
    within 1e-8 of a tight FP64 solve."""
    import os
    from neopz_gb300 import learned
    w = np.load(os.path.join(learned.DATA, "learned_elasticity3d_q2.npy"))
    n = 16
    grid, coef = learned.elasticity3d(n)
    ctx = learned.context_for(grid, rank=8, seed=0, params=w)
    for s in (10000, 10001):
        ctx.set_coef(grid, coef(s))
        ctx.assemble()
        jac = ctx.solve(tol=1e-8, want_x=False)
        lrn = ctx.solve(solver=g.GPZ_SOLVER_LEARNED_FCG, tol=1e-8, want_x=False)
        assert jac["rc"] == 0 and lrn["rc"] == 0 and lrn["restarts"] == 0
        assert lrn["iterations"] <= 0.85 * jac["iterations"], (s, lrn["iterations"], jac["iterations"])
        ref = ctx.solve(tol=1e-12, max_iter=50000)
        ctx.assemble(g.GPZ_PREC_MIXED)
        mx = ctx.solve(solver=g.GPZ_SOLVER_LEARNED_MIXED_FCG, tol=1e-8, reliable_delta=1e-2)
        assert mx["rc"] == 0 and mx["true_resid"] <= 1e-8 and mx["spmv_fp32"] > 0 and mx["reliable_updates"] >= 1
        assert mx["iterations"] <= 1.1 * lrn["iterations"], (s, mx["iterations"], lrn["iterations"])
        assert np.linalg.norm(mx["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    ctx.close()


def test_learned_mixed_elasticity_falls_back(g):
    """The FP32 learned + mixed path of 3-state problems keeps the Jacobi fallback: with a broken network every
    iteration falls back and the solve still reaches the true residual."""
    n = 6
    grid = g.elasticity3d(n, 2, E=np.exp(np.random.default_rng(4).standard_normal(n ** 3)))
    ctx = _ctx(g, grid)
    npar = ctx.learned_init(rank=8, seed=0)
    ctx.set_learned_params(np.full(npar, np.nan, np.float32))
    ctx.assemble(g.GPZ_PREC_MIXED)
    jac = ctx.solve(tol=1e-8)
    mx = ctx.solve(solver=g.GPZ_SOLVER_LEARNED_MIXED_FCG, tol=1e-8, reliable_delta=1e-2)
    assert mx["rc"] == 0 and mx["true_resid"] <= 1e-8
    assert mx["restarts"] >= mx["iterations"] - 1  # every application fell back
    tight = ctx.solve(tol=1e-12)
    assert np.linalg.norm(mx["x"] - tight["x"]) <= 1e-8 * np.linalg.norm(tight["x"])
    ctx.close()


def test_learned_mixed_elasticity_equation_wise_path(g):
    """Rank 4 (not the connect-wise kernel's rank 8): the equation-wise node correction of the FP32 learned +
    mixed path reaches the same true residual as the FP64 learned flexible CG with the same network, in at most
    1.5x its iterations (the FP32 recurrence on the 1e12-penalty rows costs iterations on small meshes), and the
    solution is within 1e-8 of a tight FP64 solve."""
    n = 6
    grid = g.elasticity3d(n, 2, E=np.exp(np.random.default_rng(9).standard_normal(n ** 3)))
    ctx = _ctx(g, grid)
    npar = ctx.learned_init(rank=4, seed=3)
    ctx.set_learned_params((0.05 * np.random.default_rng(1).standard_normal(npar)).astype(np.float32))
    f64 = ctx.solve(solver=g.GPZ_SOLVER_LEARNED_FCG, tol=1e-8)
    ctx.assemble(g.GPZ_PREC_MIXED)
    mx = ctx.solve(solver=g.GPZ_SOLVER_LEARNED_MIXED_FCG, tol=1e-8, reliable_delta=1e-2)
    assert f64["rc"] == 0 and mx["rc"] == 0 and mx["true_resid"] <= 1e-8
    assert mx["iterations"] <= 1.5 * f64["iterations"], (mx["iterations"], f64["iterations"])
    tight = ctx.solve(tol=1e-12)
    assert np.linalg.norm(mx["x"] - tight["x"]) <= 1e-8 * np.linalg.norm(tight["x"])
    ctx.close()


def test_learned_correction_gains_over_the_block_jacobi_cg(g):
    """The ablation against the method the correction has to beat: on unseen 16^3 fields, the learned + mixed
    flexible CG on the 3x3 connect-block Jacobi base (the committed elasticity weights) needs at most 90% of
    the iterations of the mixed CG with the same block Jacobi and no network (measured: 465 against 567-581),
    both to a true FP64 residual of 1e-8, with solutions within 1e-8 of a tight FP64 solve.  On the two-level
    base the same network adds iterations (313-328 against 256-264), which is why the faster two-level CG is
    reported beside the learned path rather than under it."""
    import os
    from neopz_gb300 import learned
    w = np.load(os.path.join(learned.DATA, "learned_elasticity3d_q2.npy"))
    grid, coef = learned.elasticity3d(16)
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    ctx.assemble(g.GPZ_PREC_MIXED)
    ctx.learned_init(rank=8, seed=0)
    ctx.set_learned_params(w)
    kw = dict(tol=1e-8, max_iter=200000, reliable_delta=1e-2, check_every=16)
    for s in (10000, 10001):
        ctx.set_coef(grid, coef(s))
        ctx.assemble(g.GPZ_PREC_MIXED)
        base = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_BLOCK_JACOBI, **kw)
        lrn = ctx.solve(solver=g.GPZ_SOLVER_LEARNED_MIXED_FCG, precond=g.GPZ_PRECOND_BLOCK_JACOBI, **kw)
        assert base["rc"] == 0 and lrn["rc"] == 0 and base["true_resid"] <= 1e-8 and lrn["true_resid"] <= 1e-8
        assert lrn["iterations"] <= 0.9 * base["iterations"], (s, lrn["iterations"], base["iterations"])
        ctx.assemble(g.GPZ_PREC_FP64)
        tight = ctx.solve(tol=1e-12, max_iter=50000)
        for r in (base, lrn):
            assert np.linalg.norm(r["x"] - tight["x"]) <= 1e-8 * np.linalg.norm(tight["x"])
    ctx.close()
