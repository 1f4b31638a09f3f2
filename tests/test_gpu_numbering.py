"""The GPU path consumes whatever connect numbering the host mesh holds (the reference renumbers connects with
TPZAnalysis::OptimizeBandwidth / TPZSloanRenumbering before it assembles, Analysis/TPZAnalysis.cpp:228-300):
with the connects of the same mesh renumbered at random or by gpz_sloan_resequence, the pattern, matrix, load vector and solution are those
of the original numbering permuted -- the pattern exactly, values and load vector within 1e-12, solutions within
1e-8.  The original numbering is pinned to the oracle by the parity tests.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIDES = {1: 3, 2: 9, 3: 27}


def _gpz():
    from neopz_gb300 import gpz
    return gpz


@pytest.fixture(scope="module")
def built():
    import __graft_entry__
    __graft_entry__.build()
    return True


def _arr(ptr, n):
    return np.ctypeslib.as_array(ptr, shape=(n,))


def _renumber(grid, perm):
    """Renumber the connects of grid's descriptor in place (connect c gets number perm[c]); returns old -> new
    equation map."""
    d = grid.desc
    nc, nel = d.nconnects, d.nel
    size = _arr(d.block_size, nc).copy()
    order = _arr(d.conn_order, nc).copy()
    pos = _arr(d.block_pos, nc).copy()
    new_size = np.empty_like(size)
    new_order = np.empty_like(order)
    new_size[perm] = size
    new_order[perm] = order
    new_pos = np.concatenate([[0], np.cumsum(new_size)[:-1]]).astype(np.int64)
    _arr(d.block_size, nc)[:] = new_size
    _arr(d.conn_order, nc)[:] = new_order
    _arr(d.block_pos, nc)[:] = new_pos
    conn = _arr(d.el_conn, nel * 27)
    types = _arr(d.el_type, nel)
    for e in range(nel):
        ns = SIDES[int(types[e])]
        conn[e * 27:e * 27 + ns] = perm[conn[e * 27:e * 27 + ns]]
    eqmap = np.empty(d.neq, np.int64)
    for c in range(nc):
        eqmap[pos[c]:pos[c] + size[c]] = new_pos[perm[c]] + np.arange(size[c])
    return eqmap


def _dense(ia, ja, a, n):
    A = np.zeros((n, n))
    for r in range(n):
        A[r, ja[ia[r]:ia[r + 1]]] = a[ia[r]:ia[r + 1]]
    return A


def _system(g, grid, sym):
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(sym)
    ia, ja = ctx.pattern()
    ctx.assemble()
    a, f = ctx.matrix(), ctx.rhs()
    x = ctx.solve(tol=1e-11, max_iter=20000)["x"]
    ctx.close()
    return ia, ja, a, f, x


@pytest.mark.parametrize("kind", ["random", "sloan"])
@pytest.mark.parametrize("case", ["elast3d_p2", "elast3d_hp", "darcy2d_p3"])
def test_renumbered_connects_give_the_permuted_system(built, case, kind):
    """kind "sloan": the permutation TPZAnalysis::OptimizeBandwidth applies (gpz_sloan_resequence)."""
    g = _gpz()
    rng = np.random.default_rng(21)
    E = np.exp(rng.standard_normal(27))
    k = np.exp(rng.standard_normal(36))
    make = {"elast3d_p2": lambda: g.elasticity3d(3, 2, E=E),
            "elast3d_hp": lambda: g.elasticity3d_hp(3, g.hp_orders(27, 3), E=E),
            "darcy2d_p3": lambda: g.darcy(2, 6, 3, k)}[case]
    base, moved = make(), make()
    nc = moved.desc.nconnects
    if kind == "random":
        perm = np.random.default_rng(5).permutation(nc)
    else:
        ei, eg = moved.element_graph()
        perm = g.sloan_resequence(nc, ei, eg)[0]
        eqmap_helper = make().permute_connects(perm)  # the Python helper gives the same equation map
    eqmap = _renumber(moved, perm)
    if kind == "sloan":
        assert np.array_equal(eqmap, eqmap_helper)
    n = base.neq
    for sym in (False, True):
        ia, ja, a, f, x = _system(g, base, sym)
        ib, jb, b, h, y = _system(g, moved, sym)
        # pattern: the permuted structure, exactly
        rows = np.repeat(np.arange(n), np.diff(ia))
        pr, pc = eqmap[rows], eqmap[ja]
        if sym:
            pr, pc = np.minimum(pr, pc), np.maximum(pr, pc)
        want = set(zip(pr.tolist(), pc.tolist()))
        got = set(zip(np.repeat(np.arange(n), np.diff(ib)).tolist(), jb.tolist()))
        assert got == want and len(jb) == len(ja)
        A = _dense(ia, ja, a, n)
        B = _dense(ib, jb, b, n)
        Ap = np.zeros_like(A)
        Ap[np.ix_(eqmap, eqmap)] = A
        if sym:
            Ap = np.triu(Ap) + np.triu(Ap.T, 1)  # the upper pattern holds max(i, j) columns
        assert np.all(np.max(np.abs(B - Ap), axis=1) <= 1e-12 * np.max(np.abs(Ap), axis=1))  # per row
        assert np.max(np.abs(h[eqmap] - f)) <= 1e-12 * np.max(np.abs(f))
        assert np.linalg.norm(y[eqmap] - x) <= 1e-8 * np.linalg.norm(x)
