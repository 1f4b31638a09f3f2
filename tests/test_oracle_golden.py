"""Pins the CPU oracle against the reference's own known answers (CPU only).

* golden matrices of the reference's Catch2 tests (committed fixture);
* counts printed by the reference library on the benchmark grids;
* properties the reference's tests rely on (quadrature exactness, H1
  conformity of the hierarchical shapes across shared sides).
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_unit_golden.json")))


def _contribute(kind, dim, coef, nu, weight, phi, dphix, force=(0, 0, 0), scale=1.0):
    nshape = len(phi)
    n = 3 * nshape if kind == O.ORC_ELAST3D else nshape
    ek = np.zeros(n * n)
    ef = np.zeros(n)
    phi = np.ascontiguousarray(phi, np.float64)
    dphix = np.ascontiguousarray(dphix, np.float64)
    f = np.ascontiguousarray(force, np.float64)
    O.lib().orc_contribute(kind, dim, scale, coef, nu, weight, nshape, O._p(phi), O._p(dphix), O._p(f),
                           O._p(ek), O._p(ef))
    return ek.reshape(n, n).T.copy(), ef


def test_cube_elasticity_9x9_golden():
    g = GOLD["cube_elasticity_9x9"]
    ek, _ = _contribute(O.ORC_ELAST3D, 3, g["E"], g["nu"], g["weight"], np.zeros(3), np.eye(3))
    assert np.allclose(ek, ek.T, atol=1e-8)
    assert np.max(np.abs(ek - np.array(g["matrix"]))) <= g["margin"]


def test_darcy_master_quad_golden():
    g = GOLD["darcy_master_quad_4x4"]
    loc, w = O.gauss(g["intrule_order"])
    n = len(loc)
    ek = np.zeros((4, 4))
    for ip in range(n * n):  # TPZIntQuad ordering: eta fastest
        ik, ie = ip // n, ip % n
        phi, dphi = O.shape(O.T_QUAD, g["ids"], [1] * 5, [loc[ik], loc[ie]])
        e, _ = _contribute(O.ORC_DARCY, 2, g["perm"], 0.0, w[ik] * w[ie], phi, dphi)
        ek += e
    assert np.max(np.abs(ek - np.array(g["matrix"]))) <= g["margin"]


@pytest.mark.parametrize("sym", [True, False])
def test_known_matrix_1d(sym):
    g = GOLD["known_matrix_1d"]
    ek = np.array(g["mock_ek"]).reshape(-1)
    mats = [O.material(1, O.ORC_MOCK, 1, mock_ek=tuple(ek))]
    m = O.OracleMesh(1, (g["n_el"], 1, 1), (0, 0, 0), (g["n_el"], 0, 0), [1], False, g["order"], mats, [])
    assert m.neq == g["n_el"] + 1
    ia, ja = m.pattern(sym)
    a, _ = m.assemble(sym, ia, ja)
    A = np.zeros((m.neq, m.neq))
    for r in range(m.neq):
        for k in range(ia[r], ia[r + 1]):
            A[r, ja[k]] = a[k]
            if sym:
                A[ja[k], r] = a[k]
    n = m.neq
    assert A[0, 0] == g["diag_end"] and A[n - 1, n - 1] == g["diag_end"]
    for i in range(1, n - 1):
        assert A[i, i] == g["diag_mid"] and A[i, i - 1] == g["offdiag"] and A[i, i + 1] == g["offdiag"]


def test_poisson2d_reference_counts():
    g = GOLD["reference_run_counts"]["poisson2d_q2_64"]
    m = O.poisson2d(64, 2)
    assert m.neq == g["neq"]
    ia, ja = m.pattern(True)
    assert len(ja) == g["nnz_upper"]
    a, f = m.assemble(True, ia, ja)
    r = O.cg_jacobi(True, ia, ja, a, f, 20000, 1e-10)
    assert r["iters"] == g["cg_iters_1e10"]
    # the discrete solution approximates sin(pi x) sin(pi y): peak 1
    assert abs(r["x"].max() - 1.0) < 1e-6


@pytest.mark.slow
def test_elasticity16_reference_counts():
    g = GOLD["reference_run_counts"]["elast3d_q2_16"]
    m = O.elasticity3d(16, 2)
    assert m.neq == g["neq"]
    ia, ja = m.pattern(True)
    assert len(ja) == g["nnz_upper"]
    a, f = m.assemble(True, ia, ja, nthreads=4)
    r = O.cg_jacobi(True, ia, ja, a, f, 5000, 1e-8)
    assert r["iters"] == g["cg_iters_1e8"]


def test_threaded_assembly_equals_serial():
    # StructMatrixUnitTest "Compare parallel and serial matrices": |diff| <= 10 eps
    m = O.elasticity3d(4, 2)
    ia, ja = m.pattern(True)
    a0, f0 = m.assemble(True, ia, ja, nthreads=0)
    a4, f4 = m.assemble(True, ia, ja, nthreads=4)
    assert np.array_equal(a0, a4) and np.array_equal(f0, f4)


def test_sym_and_full_patterns_agree():
    m = O.elasticity3d(3, 2)
    ia, ja = m.pattern(True)
    ib, jb = m.pattern(False)
    a, f = m.assemble(True, ia, ja)
    b, g = m.assemble(False, ib, jb)
    x = np.random.default_rng(0).standard_normal(m.neq)
    assert np.allclose(O.spmv(True, ia, ja, a, x), O.spmv(False, ib, jb, b, x), rtol=1e-12, atol=1e-9)
    assert np.array_equal(f, g)
    # full rows sorted, upper rows start at the diagonal
    for r in range(m.neq):
        assert np.all(np.diff(jb[ib[r]:ib[r + 1]]) > 0)
        assert ja[ia[r]] == r


@pytest.mark.parametrize("npts", [1, 2, 3, 4, 5])
def test_gauss_exactness(npts):
    order = 2 * npts - 2
    loc, w = O.gauss(order)
    assert len(loc) == npts
    for k in range(2 * npts):
        exact = 0.0 if k % 2 else 2.0 / (k + 1)
        assert abs(np.sum(w * loc ** k) - exact) < 1e-14


@pytest.mark.parametrize("p", [2, 3])
def test_h1_conformity_across_shared_face(p):
    """Two hexes sharing the face x=+1 / x=-1 of their master elements: the traces of the
    shapes of the shared connects must coincide (orientation from global node ids)."""
    rng = np.random.default_rng(p)
    gid = rng.permutation(12)
    # element A: x in [-1,1]; element B: x in [1,3]; shared face nodes 1,2,6,5 of A = 0,3,7,4 of B
    A = [gid[i] for i in (0, 1, 2, 3, 4, 5, 6, 7)]
    B = [gid[i] for i in (1, 8, 9, 2, 5, 10, 11, 6)]
    orders = [p] * 19
    # shapes of A on its face 22 (x=+1) vs B on its face 24 (x=-1), same physical point (y, z)
    for (y, z) in [(-0.3, 0.7), (0.5, -0.2), (0.9, 0.1)]:
        pa, _ = O.shape(O.T_CUBE, A, orders, [1.0, y, z])
        pb, _ = O.shape(O.T_CUBE, B, orders, [-1.0, y, z])
        # map connect-wise: corner shapes of shared nodes
        for la, lb in [(1, 0), (2, 3), (6, 7), (5, 4)]:
            assert abs(pa[la] - pb[lb]) < 1e-13
        # shapes attached to the shared face connect and its edges
        def side_range(orders_, side):
            first = 8 + sum(_nconn(s, p) for s in range(8, side))
            return first, first + _nconn(side, p)
        for sa, sb in [(22, 24), (9, 11), (14, 15), (17, 19), (13, 12)]:
            fa, la_ = side_range(orders, sa)
            fb, lb_ = side_range(orders, sb)
            assert np.allclose(pa[fa:la_], pb[fb:lb_], atol=1e-12), (sa, sb)


def _nconn(side, p):
    if side < 8:
        return 1
    if side < 20:
        return p - 1
    if side < 26:
        return (p - 1) ** 2
    return (p - 1) ** 3


def test_shape_derivatives_match_finite_differences():
    ids = [5, 2, 7, 0, 3, 6, 1, 4]
    orders = [3] * 19
    x = np.array([0.21, -0.37, 0.55])
    phi, dphi = O.shape(O.T_CUBE, ids, orders, x)
    h = 1e-6
    for d in range(3):
        e = np.zeros(3)
        e[d] = h
        fd = (O.shape(O.T_CUBE, ids, orders, x + e)[0] - O.shape(O.T_CUBE, ids, orders, x - e)[0]) / (2 * h)
        assert np.allclose(fd, dphi[d], atol=1e-7)


@pytest.mark.parametrize("m", [30, 5])
def test_oracle_gmres_matches_cg_solution(m):
    """Restarted Jacobi-GMRES(m) (gmres.h) converges to the CG solution; a small m restarts many times."""
    E = np.exp(np.random.default_rng(7).standard_normal(27))
    om = O.elasticity3d(3, 2, E=E)
    ia, ja = om.pattern(False)
    a, f = om.assemble(False, ia, ja)
    cg = O.cg_jacobi(False, ia, ja, a, f, 20000, 1e-12)
    g = O.gmres_jacobi(False, ia, ja, a, f, m, 20000, 1e-10)
    assert g["rc"] == 0 and g["resid"] < 1e-10 and g["iters"] > m
    assert np.linalg.norm(g["x"] - cg["x"]) <= 1e-8 * np.linalg.norm(cg["x"])
    # the iteration budget is honoured and reported as the reference does
    g2 = O.gmres_jacobi(False, ia, ja, a, f, m, 7, 1e-10)
    assert g2["rc"] == 1 and g2["iters"] == 7


def test_learned_oracle_gradient_matches_finite_differences():
    """The numpy oracle of the learned preconditioner: analytic gradient = central differences (float64)."""
    import scipy.sparse as sp
    from oracle import learned_oracle as LO

    rng = np.random.default_rng(3)
    k = np.exp(rng.standard_normal(9))
    om = O.darcy(2, 3, 2, k)
    ia, ja = om.pattern(False)
    a, f = om.assemble(False, ia, ja)
    A = sp.csr_matrix((a, ja, ia), shape=(om.neq, om.neq))
    mesh = LO.mesh_from_oracle(om, A, k)
    R = 2
    _, n = LO.layout(mesh.NS, R)
    p = rng.standard_normal(n) * 0.3
    Rs, Es = rng.standard_normal((2, om.neq)), rng.standard_normal((2, om.neq))
    loss, g = LO.loss_and_grad(mesh, A, p, R, Rs, Es)
    assert abs(loss - LO.loss_only(mesh, A, p, R, Rs, Es)) <= 1e-12 * abs(loss)
    idx = np.append(rng.choice(n - 1, 60, replace=False), n - 1)  # the last parameter is the Jacobi scale
    h = 1e-6
    for i in idx:
        e = np.zeros(n)
        e[i] = h
        fd = (LO.loss_only(mesh, A, p + e, R, Rs, Es) - LO.loss_only(mesh, A, p - e, R, Rs, Es)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, np.abs(g).max()), (i, fd, g[i])


def _dense(ia, ja, a, n):
    A = np.zeros((n, n))
    for r in range(n):
        A[r, ja[ia[r]:ia[r + 1]]] = a[ia[r]:ia[r + 1]]
    return A


def _quadratic_exact(xyz):
    """(x^2 - 1)(y^2 - 1) and its gradient, the exact solution of UnitTest_PZ/TestMesh/TestError.cpp:50-59."""
    x, y = xyz[:, 0], xyz[:, 1]
    u = ((x * x - 1) * (y * y - 1))[:, None]
    du = np.zeros((len(x), 3, 1))
    du[:, 0, 0] = 2 * x * (y * y - 1)
    du[:, 1, 0] = 2 * y * (x * x - 1)
    return u, du


def test_error_known_answer_poisson():
    """The error test of UnitTest_PZ/TestMesh/TestError.cpp:20-41 (TPZAnalysis::PostProcessError after a direct
    solve, exact order 4), on quadrilaterals: the exact solution is in the order-2 space of quads, so the three
    norms (H1, L2, H1 semi-norm) drop from O(1) at p = 1 to the reference's bound of 10 machine epsilons for
    p = 2, 3, 4 (the triangles of the reference reach it at p = 4)."""
    eps = np.finfo(float).eps
    prev = None
    for p in range(1, 5):
        om = O.poisson_square_quadratic(2, p)
        ia, ja = om.pattern(False)
        a, f = om.assemble(False, ia, ja)
        x = np.linalg.solve(_dense(ia, ja, a, om.neq), f)
        u, du = _quadratic_exact(om.error_points(4))
        tot, el = om.error_eval(4, x, u, du)
        assert tot.shape == (3,) and el.shape == (om.ncel, 3)
        assert np.allclose(np.sqrt((el ** 2).sum(0)), tot, rtol=1e-14)
        if p == 1:
            assert np.all(tot > 0.1)
        else:
            # at the rounding floor the norms are no longer ordered in p
            assert np.all(tot <= 10 * eps), (p, tot)
            assert np.all(tot <= prev) or p > 2
        prev = tot


def test_error_norms_of_known_fields():
    """Norms of an exact field against the zero solution, integrated by the error rule: the L2 and H1
    semi-norms of (x^2 - 1)(y^2 - 1) on [-1, 1]^2 are 16/15 and sqrt(256/45); the uniform strain u = (x, 0, 0)
    on the unit cube gives L2^2 = 1/3, semi-norm 1 and energy E (1 - nu) / ((1 + nu)(1 - 2 nu))."""
    om = O.poisson_square_quadratic(3, 2)
    u, du = _quadratic_exact(om.error_points(4))
    tot, _ = om.error_eval(4, np.zeros(om.neq), u, du)
    assert abs(tot[1] - 16 / 15) <= 1e-13
    assert abs(tot[2] - np.sqrt(256 / 45)) <= 1e-13
    assert abs(tot[0] ** 2 - (tot[1] ** 2 + tot[2] ** 2)) <= 1e-13
    nu = 0.3
    om = O.elasticity3d(2, 2, nu=nu)
    xyz = om.error_points(2)
    u = np.zeros((len(xyz), 3))
    u[:, 0] = xyz[:, 0]
    du = np.zeros((len(xyz), 3, 3))
    du[:, 0, 0] = 1.0
    tot, el = om.error_eval(2, np.zeros(om.neq), u, du)
    assert abs(tot[1] ** 2 - 1 / 3) <= 1e-13
    assert abs(tot[2] - 1.0) <= 1e-13
    assert abs(tot[0] ** 2 - (1 - nu) / ((1 + nu) * (1 - 2 * nu))) <= 1e-13
    assert np.all(el[8:] == 0.0)  # boundary elements carry no error


def _dense(ia, ja, a, n):
    A = np.zeros((n, n))
    for r in range(n):
        A[r, ja[ia[r]:ia[r + 1]]] = a[ia[r]:ia[r + 1]]
    return A


def test_oracle_jacobi_iteration():
    """The stationary Jacobi solver (SetJacobi as the solver): the oracle's sweeps against a numpy restatement of
    TPZMatrix::SolveJacobi (Matrix/pzmatrix.cpp:643-667) on a dense copy, the TPZFYsmpMatrix override's first
    sweep (Matrix/pzysmp.cpp:725-781), FromCurrent restarts and convergence on the absolute residual norm."""
    om = O.poisson2d(8, 1)
    ia, ja = om.pattern(False)
    a, f = om.assemble(False, ia, ja)
    sa, sj = om.pattern(True)
    sv, sf = om.assemble(True, sa, sj)
    n = om.neq
    A = _dense(ia, ja, a, n)
    d = np.diag(A).copy()
    x = np.zeros(n)
    r = f.copy()
    for _ in range(5):
        x = x + r / d
        r = f - A @ x
    for sym, (pi, pj, pv) in ((True, (sa, sj, sv)), (False, (ia, ja, a))):
        out = O.jacobi(sym, pi, pj, pv, f, 5, 0.0)
        assert out["iters"] == 5 and out["rc"] == 1
        assert np.max(np.abs(out["x"] - x)) <= 1e-12 * np.max(np.abs(x))
        assert abs(out["resid"] - np.linalg.norm(r)) <= 1e-9 * np.linalg.norm(r)
        # FromCurrent: 2 + 3 sweeps are the 5 sweeps
        x2 = O.jacobi(sym, pi, pj, pv, f, 2, 0.0)["x"]
        out3 = O.jacobi(sym, pi, pj, pv, f, 3, 0.0, x0=x2)
        assert out3["iters"] == 3
        assert np.max(np.abs(out3["x"] - out["x"])) <= 1e-14 * np.max(np.abs(x))
    # numiterations = 0, or a tolerance the initial residual meets: no sweep for TPZMatrix::SolveJacobi, one
    # sweep (x = b / diag) for the TPZFYsmpMatrix override
    big = 2 * np.linalg.norm(f)
    for maxit, tol in ((0, 0.0), (10, big)):
        s0 = O.jacobi(True, sa, sj, sv, f, maxit, tol)
        f0 = O.jacobi(False, ia, ja, a, f, maxit, tol)
        assert s0["iters"] == 0 and np.all(s0["x"] == 0.0)
        assert f0["iters"] == 1 and np.array_equal(f0["x"], f / d)
    # convergence on the absolute ||b - A x||, to the direct solution
    tol = 1e-9 * np.linalg.norm(f)
    conv = O.jacobi(True, sa, sj, sv, f, 100000, tol)
    assert conv["rc"] == 0 and 10 < conv["iters"] < 100000 and conv["resid"] <= tol
    xs = np.linalg.solve(A, f)
    assert np.linalg.norm(conv["x"] - xs) <= 1e-6 * np.linalg.norm(xs)
    assert np.linalg.norm(f - A @ conv["x"]) <= 1.01 * tol


def test_oracle_equation_filter():
    """The oracle's equation filter against dense restrictions: the condensed full matrix is A[act][:, act], the
    condensed upper pattern its upper triangle (rows still start at the diagonal), and the load vector keeps the
    mesh's size with zeros at the inactive equations."""
    om = O.poisson2d(4, 2)
    rng = np.random.default_rng(8)
    active = rng.choice(om.neq, size=om.neq - 11, replace=False)
    act = np.sort(active)
    for sym in (False, True):
        ia, ja = om.pattern(sym)
        a, f = om.assemble(sym, ia, ja)
        ic, jc, vc, fm, fc = O.filter_system(sym, ia, ja, a, f, np.concatenate([active, active[:5]]))
        n = len(act)
        D = _dense(ia, ja, a, om.neq)
        C = _dense(ic, jc, vc, n)
        assert np.array_equal(C, D[np.ix_(act, act)])
        for r in range(n):
            row = jc[ic[r]:ic[r + 1]]
            assert np.all(np.diff(row) > 0) and (not sym or row[0] == r)
        assert np.array_equal(fc, f[act]) and np.all(fm[np.setdiff1d(np.arange(om.neq), act)] == 0.0)
        assert np.array_equal(fm[act], f[act])
