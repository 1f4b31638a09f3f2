"""The allocation-free CG entry point, gpz_cg_jacobi_noalloc, through the C ABI.

It must give the solution of the context's FP64 Jacobi-PCG (gpz_solve with
GPZ_SOLVER_CG / GPZ_PRECOND_JACOBI, the algorithm of cg.h) on the same system:
both follow the same recurrence and stopping rule but reduce in a different
order, so the solutions must agree within 1e-8 relative and the iteration
counts within max(3, 10%).  Two calls in a row must give identical results:
the shared static scratch carries nothing from one call to the next.

The caller owns every device buffer (torch tensors here); the entry point
itself allocates nothing.  Systems above GPZ_NOALLOC_MAX_EQ are refused with
GPZ_E_TOO_LARGE before any device work, which the CPU-only test checks.
"""
import ctypes

import numpy as np
import pytest

GPZ_NOALLOC_MAX_EQ = 262144
GPZ_E_TOO_LARGE = -10
GPZ_E_INVALID = -1


@pytest.fixture(scope="module")
def g():
    import __graft_entry__
    __graft_entry__.build()
    from neopz_gb300 import gpz
    return gpz


def _entry(g):
    f = g.lib().gpz_cg_jacobi_noalloc
    f.restype = ctypes.c_int
    i64, vp = ctypes.c_int64, ctypes.c_void_p
    f.argtypes = [vp, i64, i64, vp, vp, vp, vp, vp, i64, ctypes.c_double, ctypes.POINTER(i64),
                  ctypes.POINTER(ctypes.c_double)]
    return f


def _call(f, stream, neq, nnz, ia, ja, a, b, x, max_iter, tol):
    its, res = ctypes.c_int64(-1), ctypes.c_double(-1.0)
    rc = f(stream, neq, nnz, ia, ja, a, b, x, max_iter, tol, ctypes.byref(its), ctypes.byref(res))
    return rc, its.value, res.value


def test_noalloc_rejects_oversized_and_bad_arguments_without_device_work(g):
    f = _entry(g)
    rc, its, res = _call(f, None, GPZ_NOALLOC_MAX_EQ + 1, 0, None, None, None, None, None, 100, 1e-8)
    assert rc == GPZ_E_TOO_LARGE and its == 0 and res == 0.0
    assert "GPZ_NOALLOC_MAX_EQ" in g.lib().gpz_get_error_string(rc).decode()
    assert _call(f, None, -1, 0, None, None, None, None, None, 100, 1e-8)[0] == GPZ_E_INVALID
    assert _call(f, None, 10, 0, None, None, None, None, None, -1, 1e-8)[0] == GPZ_E_INVALID
    assert _call(f, None, 10, 0, None, None, None, None, None, 100, float("nan"))[0] == GPZ_E_INVALID
    assert _call(f, None, 0, 0, None, None, None, None, None, 100, 1e-8)[0] == 0  # empty system


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["poisson2d_q2", "elasticity3d_q2"])
def test_noalloc_matches_context_jacobi_pcg(g, case):
    import torch

    if case == "poisson2d_q2":
        grid = g.poisson2d(16, 2)
    else:
        E = np.exp(np.random.default_rng(3).standard_normal(4 ** 3))
        grid = g.elasticity3d(4, 2, E=E)
    tol, max_iter = 1e-10, 20000
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)  # full CSR (TPZFYsmpMatrix layout)
    ctx.assemble(g.GPZ_PREC_FP64)
    ref = ctx.solve(tol=tol, max_iter=max_iter)
    assert ref["rc"] == 0
    ia, ja = ctx.pattern()
    a, b = ctx.matrix(), ctx.rhs()
    ctx.close()

    dev = torch.device("cuda:0")
    d_ia = torch.from_numpy(np.ascontiguousarray(ia, dtype=np.int64)).to(dev)
    d_ja = torch.from_numpy(np.ascontiguousarray(ja, dtype=np.int32)).to(dev)
    d_a = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
    d_b = torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).to(dev)
    d_x = torch.from_numpy(np.full(len(b), np.nan)).to(dev)  # overwritten by the call
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    f = _entry(g)
    neq, nnz = len(b), len(ja)
    xs = []
    free_before = None
    for _ in range(2):
        rc, its, res = _call(f, stream, neq, nnz, d_ia.data_ptr(), d_ja.data_ptr(), d_a.data_ptr(), d_b.data_ptr(),
                             d_x.data_ptr(), max_iter, tol)
        assert rc == 0, rc
        assert res <= tol
        assert abs(its - ref["iterations"]) <= max(3, 0.1 * ref["iterations"]), (its, ref["iterations"])
        x = d_x.cpu().numpy().copy()
        assert np.linalg.norm(x - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
        xs.append((its, res, x))
        d_x.copy_(torch.from_numpy(np.full(neq, np.nan)))
        torch.cuda.synchronize()
        if free_before is None:  # after the first call (which looks the scratch up) nothing is allocated
            free_before = torch.cuda.mem_get_info(dev)[0]
    assert xs[0][0] == xs[1][0] and xs[0][1] == xs[1][1] and np.array_equal(xs[0][2], xs[1][2])
    assert torch.cuda.mem_get_info(dev)[0] == free_before, "device free memory changed across calls"

    # a stream of the current device is accepted; the legacy default stream (NULL) too
    rc, its, _ = _call(f, None, neq, nnz, d_ia.data_ptr(), d_ja.data_ptr(), d_a.data_ptr(), d_b.data_ptr(),
                       d_x.data_ptr(), max_iter, tol)
    assert rc == 0 and its == xs[0][0]

    # a budget of a few iterations: not converged, iteration count = max_iter
    rc, its, res = _call(f, stream, neq, nnz, d_ia.data_ptr(), d_ja.data_ptr(), d_a.data_ptr(), d_b.data_ptr(),
                         d_x.data_ptr(), 5, tol)
    assert rc == 1 and its == 5 and res > tol

    # the kernel's own input checks: a zero diagonal and a column outside [0, neq)
    # stop the solve before the first iteration
    row0 = np.arange(ia[0], ia[1])
    kd = int(row0[ja[row0] == 0][0])
    a_bad = a.copy()
    a_bad[kd] = 0.0
    d_abad = torch.from_numpy(a_bad).to(dev)
    ja_bad = np.ascontiguousarray(ja, dtype=np.int32).copy()
    ja_bad[int(ia[1])] = neq
    d_jabad = torch.from_numpy(ja_bad).to(dev)
    torch.cuda.synchronize()
    for jj, aa in ((d_ja, d_abad), (d_jabad, d_a)):
        d_x.fill_(7.0)
        torch.cuda.synchronize()
        rc, its, _ = _call(f, stream, neq, nnz, d_ia.data_ptr(), jj.data_ptr(), aa.data_ptr(), d_b.data_ptr(),
                           d_x.data_ptr(), max_iter, tol)
        assert rc == GPZ_E_INVALID and its == 0
        assert bool(torch.all(d_x == 7.0)), "bad input must leave x unchanged"
    # and a good call right after still solves
    rc, its, res = _call(f, stream, neq, nnz, d_ia.data_ptr(), d_ja.data_ptr(), d_a.data_ptr(), d_b.data_ptr(),
                         d_x.data_ptr(), max_iter, tol)
    assert rc == 0 and its == xs[0][0] and np.array_equal(d_x.cpu().numpy(), xs[0][2])
