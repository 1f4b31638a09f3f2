"""Cancellation (gpz_set_killed, the counterpart of TPZGuiInterface::SetKilled / AmIKilled,
Common/TPZGuiInterface.cpp:80-87, polled in StrMatrix/pzstrmatrixor.cpp:182,490).

A set flag makes assemblies return GPZ_CANCELLED before any work and solves return GPZ_CANCELLED at their next
batch boundary; clearing it restores normal calls.  The flag is set from a second host thread while a long
Jacobi iteration runs: the solve ends at a batch boundary with a consistent iterate (the failure is made on the
host; no device work is interrupted).
"""
import threading
import time

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


def test_flag_set_before_the_calls(built):
    g = _gpz()
    ctx = g.Context(0)
    ctx.upload_mesh(g.poisson2d(16, 2))
    ctx.build_pattern(True)
    assert ctx.assemble() == g.GPZ_OK
    ctx.set_killed(True)
    assert ctx.assemble() == g.GPZ_CANCELLED
    assert ctx.assemble_rhs() == g.GPZ_CANCELLED
    for solver in (g.GPZ_SOLVER_CG, g.GPZ_SOLVER_MIXED_CG, g.GPZ_SOLVER_GMRES, g.GPZ_SOLVER_JACOBI):
        r = ctx.solve(solver=solver, tol=1e-10, max_iter=5000)
        assert r["rc"] == g.GPZ_CANCELLED and r["iterations"] == 0, (solver, r["rc"], r["iterations"])
    ctx.set_killed(False)
    assert ctx.assemble() == g.GPZ_OK
    r = ctx.solve(tol=1e-10, max_iter=5000)
    assert r["rc"] == g.GPZ_OK
    om = O.poisson2d(16, 2)
    ia, ja = om.pattern(True)
    a, f = om.assemble(True, ia, ja)
    ref = O.cg_jacobi(True, ia, ja, a, f, 5000, 1e-10)
    assert np.linalg.norm(r["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    ctx.close()


def test_flag_set_from_another_thread_during_a_solve(built):
    g = _gpz()
    om, grid = O.poisson2d(32, 1), g.poisson2d(32, 1)
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    ctx.assemble()
    maxit, batch = 2_000_000, 32
    out = {}

    def run():
        out["r"] = ctx.solve(solver=g.GPZ_SOLVER_JACOBI, precond=0, tol=0.0, max_iter=maxit, check_every=batch)

    t = threading.Thread(target=run)
    t0 = time.time()
    t.start()
    time.sleep(0.5)
    ctx.set_killed(True)
    t.join(timeout=120)
    assert not t.is_alive()
    r = out["r"]
    assert r["rc"] == g.GPZ_CANCELLED, (r["rc"], r["iterations"], time.time() - t0)
    assert 0 < r["iterations"] < maxit and r["iterations"] % batch == 0
    # the iterate is the converged Jacobi fixed point (hundreds of sweeps reach it), with its own report
    ia, ja = om.pattern(False)
    a, f = om.assemble(False, ia, ja)
    A = np.zeros((om.neq, om.neq))
    for row in range(om.neq):
        A[row, ja[ia[row]:ia[row + 1]]] = a[ia[row]:ia[row + 1]]
    xs = np.linalg.solve(A, f)
    assert np.linalg.norm(r["x"] - xs) <= 1e-8 * np.linalg.norm(xs)
    assert r["spmv_fp64"] == r["iterations"] + 1
    ctx.set_killed(False)
    again = ctx.solve(solver=g.GPZ_SOLVER_JACOBI, precond=0, tol=1e-9 * np.linalg.norm(f), max_iter=100000)
    assert again["rc"] == g.GPZ_OK
    ctx.close()
