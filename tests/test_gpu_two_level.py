"""The two-level block-Jacobi preconditioner of the mixed CG (GPZ_PRECOND_TWO_LEVEL).

M = B^-1 + P Ac^-1 P^T: B the 3x3 connect blocks, P the trilinear
interpolation from a coarse grid of boxes (s^3 fine elements each) to the
vertex connects, Ac = P^T A P; coarse nodes whose function is nonzero at a
penalty-Dirichlet vertex are removed.  Checked here:
* one application (gpz_precond_apply) against the same M built in numpy /
  scipy from the assembled matrix and the mesh geometry: within 1e-5 (the
  device applies it in FP32);
* the mixed CG with it reaches a true FP64 residual 1e-8 on the C5 workload's
  small instances with a solution error at most 1e-8 against the reference
  library's own FP64 solution (tests/golden), in far fewer iterations than
  with the connect blocks alone;
* meshes it is not built for (distorted or hp) and the FP64 CG are refused
  with GPZ_E_INVALID.
"""
import numpy as np
import pytest

import refcases as RC

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import __graft_entry__
    __graft_entry__.build()
    from neopz_gb300 import gpz
    return gpz


def _reference_m(grid, ctx, info):
    """B^-1 and (P, Ac^-1, kept coarse dofs) from the host mesh and the downloaded full CSR."""
    import scipy.sparse as sp
    d = grid.desc
    nel, nn = d.nel, d.nnodes
    types = np.ctypeslib.as_array(d.el_type, shape=(nel,))
    mats = np.ctypeslib.as_array(d.el_mat, shape=(nel,))
    enodes = np.ctypeslib.as_array(d.el_nodes, shape=(nel, 8))
    econn = np.ctypeslib.as_array(d.el_conn, shape=(nel, 27))
    bpos = np.ctypeslib.as_array(d.block_pos, shape=(d.nconnects,))
    xyz = np.ctypeslib.as_array(d.node_xyz, shape=(nn, 3))
    vol = np.where(types == 3)[0]
    h = xyz[enodes[vol[0], 6]] - xyz[enodes[vol[0], 0]]
    x0 = xyz[enodes[vol, 0]].min(axis=0)
    s, m = info["s"], np.array(info["coarse_boxes"])
    # vertex connects: lattice position -> first equation
    vx = {}
    for e in vol:
        for k in range(8):
            li = tuple(np.rint((xyz[enodes[e, k]] - x0) / h).astype(int))
            vx[li] = bpos[econn[e, k]]
    nnode = int(np.prod(m + 1))

    def weights(li):
        cell = np.minimum(np.array(li) // s, m - 1)
        t = (np.array(li) - cell * s) / s
        out = []
        for cn in range(8):
            b = np.array([cn & 1, (cn >> 1) & 1, cn >> 2])
            w = np.prod(np.where(b == 1, t, 1 - t))
            if w != 0:
                c = cell + b
                out.append((int(c[0] + (m[0] + 1) * (c[1] + (m[1] + 1) * c[2])), w))
        return out
    rows, cols, vals = [], [], []
    for li, eq in vx.items():
        for node, w in weights(li):
            for comp in range(3):
                rows.append(eq + comp)
                cols.append(3 * node + comp)
                vals.append(w)
    neq = grid.neq
    P = sp.csr_matrix((vals, (rows, cols)), shape=(neq, 3 * nnode))
    # coarse nodes touching a penalty-Dirichlet face
    fixed = np.zeros(nnode, bool)
    bcs = [d.bcs[i] for i in range(d.nbc)]
    for e in np.where(mats < 0)[0]:
        if bcs[-mats[e] - 1].type != 0:
            continue
        for k in range(4):
            li = tuple(np.rint((xyz[enodes[e, k]] - x0) / h).astype(int))
            for node, _ in weights(li):
                fixed[node] = True
    ia, ja = ctx.pattern()
    A = sp.csr_matrix((ctx.matrix(), ja, ia), shape=(neq, neq))
    Ac = (P.T @ A @ P).toarray()
    keep = np.repeat(~fixed, 3)
    Aci = np.zeros_like(Ac)
    Aci[np.ix_(keep, keep)] = np.linalg.inv(Ac[np.ix_(keep, keep)])
    rr = np.repeat(np.arange(neq), np.diff(ia))
    inb = rr // 3 == ja // 3
    Bl = np.zeros((neq // 3, 3, 3))
    Bl[rr[inb] // 3, rr[inb] % 3, ja[inb] % 3] = ctx.matrix()[inb]
    Bi = np.linalg.inv(Bl)
    return lambda r: np.einsum("bij,bj->bi", Bi, r.reshape(-1, 3)).reshape(-1) + P @ (Aci @ (P.T @ r)), fixed


@pytest.mark.parametrize("n,boxes", [(6, 2), (8, 4), (8, 2)])
def test_two_level_application_matches_numpy(g, n, boxes):
    E = g.lognormal(n ** 3, 1.0, 5)
    grid = g.elasticity3d(n, 2, E=E, body_force=(0.0, 0.0, 0.0))
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble(g.GPZ_PREC_MIXED)
    ctx.two_level_config(boxes)
    r = np.random.default_rng(7).standard_normal(grid.neq)
    z = ctx.precond_apply(g.GPZ_PRECOND_TWO_LEVEL, r)
    info = ctx.two_level_info()
    assert info["fine_cells"] == [n, n, n] and info["s"] * info["coarse_boxes"][0] == n
    M, fixed = _reference_m(grid, ctx, info)
    assert info["removed_nodes"] == int(fixed.sum()) > 0
    zr = M(r)
    assert np.linalg.norm(z - zr) <= 1e-5 * np.linalg.norm(zr)
    ctx.close()


@pytest.mark.parametrize("name", ["c5_elast3d_8_q2", "c5_elast3d_16_q2"])
def test_two_level_mixed_cg_against_reference(g, name):
    fx = RC.load(name)
    grid = RC.problem(g, fx)
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    ctx.assemble(g.GPZ_PREC_MIXED)
    tl = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_TWO_LEVEL, tol=1e-8, max_iter=20000,
                   reliable_delta=1e-2)
    bj = ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_BLOCK_JACOBI, tol=1e-8, max_iter=20000,
                   reliable_delta=1e-2)
    assert tl["rc"] == 0 and tl["true_resid"] <= 1e-8 and bj["rc"] == 0
    assert RC.rel_err(tl["x"], fx) <= 1e-8
    assert tl["iterations"] <= 0.7 * bj["iterations"], (tl["iterations"], bj["iterations"])
    ctx.close()


def test_two_level_refused_where_not_built(g):
    rng = np.random.default_rng(3)
    # a distorted mesh: the elements are not translates of one box
    grid = g.elasticity3d(3, 2)
    xyz = grid.nodes()
    xyz[:] = xyz + 0.1 / 3 * rng.uniform(-1, 1, xyz.shape)
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    ctx.assemble(g.GPZ_PREC_MIXED)
    with pytest.raises(g.GpzError) as e:
        ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_TWO_LEVEL, tol=1e-8)
    assert e.value.code == -1
    assert ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_BLOCK_JACOBI, tol=1e-8,
                     reliable_delta=1e-2)["rc"] == 0
    ctx.close()
    # an hp mesh (connects of more than 3 equations), and the FP64 CG
    grid = g.elasticity3d_hp(3, g.hp_orders(27, 3))
    ctx = g.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    ctx.assemble(g.GPZ_PREC_MIXED)
    with pytest.raises(g.GpzError):
        ctx.solve(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_TWO_LEVEL, tol=1e-8)
    with pytest.raises(g.GpzError):
        ctx.solve(solver=g.GPZ_SOLVER_CG, precond=g.GPZ_PRECOND_TWO_LEVEL, tol=1e-8)
    ctx.close()
