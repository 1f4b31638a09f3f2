"""TEST INFRASTRUCTURE ONLY: ctypes front end of the CPU oracle (pz_oracle.cpp).

The tests compare the GPU library against the oracle, and the oracle is the CPU
baseline of the benchmark.  It is imported by tests/, by ``__graft_entry__.smoke()`` and by the
CPU-baseline leg of ``bench.py`` only; the product (``neopz_gb300``) never
imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "pz_oracle.cpp")
_LIB = os.path.join(_HERE, "_build", "liborc.so")

ORC_POISSON, ORC_DARCY, ORC_ELAST3D, ORC_MOCK = 1, 2, 3, 4
ORC_F_NONE, ORC_F_CONST, ORC_F_SINPROD, ORC_F_QUADRATIC = 0, 1, 2, 3
T_LINE, T_QUAD, T_CUBE = 1, 2, 3
BIGNUMBER = 10.0 ** 17 * 2 / 3  # TPZMaterial::fBigNumber default for double


class orc_material(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int), ("kind", ctypes.c_int), ("dim", ctypes.c_int),
                ("scale", ctypes.c_double), ("E", ctypes.c_double), ("nu", ctypes.c_double),
                ("force", ctypes.c_double * 3), ("forcing", ctypes.c_int),
                ("forcing_porder", ctypes.c_int), ("coef_const", ctypes.c_double),
                ("bignumber", ctypes.c_double), ("mock_ek", ctypes.c_double * 4)]


class orc_bc(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int), ("matid", ctypes.c_int), ("type", ctypes.c_int),
                ("val1", ctypes.c_double * 9), ("val2", ctypes.c_double * 3)]


class orc_grid_spec(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("ndiv", ctypes.c_int * 3),
                ("minX", ctypes.c_double * 3), ("maxX", ctypes.c_double * 3),
                ("matids", ctypes.c_int * 7), ("create_bc", ctypes.c_int),
                ("default_order", ctypes.c_int), ("nmat", ctypes.c_int),
                ("mats", orc_material * 4), ("nbc", ctypes.c_int), ("bcs", orc_bc * 8),
                ("elem_coef", ctypes.POINTER(ctypes.c_double)),
                ("elem_order", ctypes.POINTER(ctypes.c_int))]


def build(force=False):
    """Compile the oracle with g++ (works on x86_64 and aarch64)."""
    os.makedirs(os.path.dirname(_LIB), exist_ok=True)
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
                               _SRC, "-o", _LIB])
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        vp, i64, i32, dp = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        P = ctypes.POINTER
        L.orc_mesh_create.restype = vp
        L.orc_mesh_create.argtypes = [P(orc_grid_spec)]
        L.orc_mesh_free.argtypes = [vp]
        for f in ("orc_neq", "orc_ncel", "orc_nconnects", "orc_nnodes"):
            getattr(L, f).restype = i64
            getattr(L, f).argtypes = [vp]
        L.orc_nstate.restype = i32
        L.orc_nstate.argtypes = [vp]
        L.orc_cel_info.restype = i32
        L.orc_cel_info.argtypes = [vp, i64, P(i32), P(i32), P(i64), vp, vp]
        L.orc_block_info.argtypes = [vp, vp, vp]
        L.orc_nodes.argtypes = [vp, vp]
        L.orc_set_nodes.argtypes = [vp, vp]
        L.orc_calc_stiff.restype = i32
        L.orc_calc_stiff.argtypes = [vp, i64, vp, vp]
        L.orc_shape.restype = i32
        L.orc_shape.argtypes = [i32, vp, vp, vp, vp, vp, i32]
        L.orc_contribute.argtypes = [i32, i32, dp, dp, dp, dp, i32, vp, vp, vp, vp, vp]
        L.orc_gauss.restype = i32
        L.orc_gauss.argtypes = [i32, vp, vp]
        L.orc_pattern.restype = i64
        L.orc_pattern.argtypes = [vp, i32, vp, vp]
        L.orc_assemble.restype = i32
        L.orc_assemble.argtypes = [vp, i32, vp, vp, vp, vp, i32]
        L.orc_spmv.argtypes = [i64, i32, vp, vp, vp, vp, vp]
        L.orc_cg_jacobi.restype = i32
        L.orc_cg_jacobi.argtypes = [i64, i32, vp, vp, vp, vp, vp, i64, dp, i32, P(i64), P(dp), vp]
        L.orc_jacobi.restype = i32
        L.orc_jacobi.argtypes = [i64, i32, vp, vp, vp, vp, vp, i64, dp, i32, P(i64), P(dp)]
        L.orc_sloan.restype = i32
        L.orc_sloan.argtypes = [i64, i64, vp, vp, vp, vp]
        L.orc_cg_block_jacobi.restype = i32
        L.orc_nodeset.restype = i32
        L.orc_nodeset.argtypes = [i64, i64, vp, vp, vp, vp, i64, vp, vp, P(i64), vp, P(i32), vp, vp]
        L.orc_cg_sparse_block_jacobi.restype = i32
        L.orc_cg_sparse_block_jacobi.argtypes = [i64, i32, vp, vp, vp, vp, vp, i64, vp, vp, i64, dp, P(i64), P(dp)]
        L.orc_cg_block_jacobi.argtypes = [i64, i32, vp, vp, vp, vp, vp, i32, i64, dp, P(i64), P(dp)]
        L.orc_error_points.restype = i64
        L.orc_error_points.argtypes = [vp, i32, vp]
        L.orc_error_eval.restype = i32
        L.orc_error_eval.argtypes = [vp, i32, vp, vp, vp, vp, vp]
        L.orc_gmres_jacobi.restype = i32
        L.orc_gmres_jacobi.argtypes = [i64, i32, vp, vp, vp, vp, vp, i32, i64, dp, P(i64), P(dp)]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def material(id, kind, dim, scale=1.0, E=1.0, nu=0.3, force=(0.0, 0.0, 0.0), forcing=ORC_F_NONE,
             forcing_porder=0, coef_const=1.0, bignumber=BIGNUMBER, mock_ek=(0, 0, 0, 0)):
    m = orc_material()
    m.id, m.kind, m.dim, m.scale, m.E, m.nu = id, kind, dim, scale, E, nu
    for i in range(3):
        m.force[i] = force[i]
    m.forcing, m.forcing_porder, m.coef_const, m.bignumber = forcing, forcing_porder, coef_const, bignumber
    for i in range(4):
        m.mock_ek[i] = mock_ek[i]
    return m


def bc(id, matid, type, val2=(0.0, 0.0, 0.0), val1=None):
    b = orc_bc()
    b.id, b.matid, b.type = id, matid, type
    for i in range(3):
        b.val2[i] = val2[i]
    if val1 is not None:
        for i in range(9):
            b.val1[i] = val1[i]
    return b


class OracleMesh:
    """A grid mesh + computational mesh + equation numbering built by the oracle."""

    def __init__(self, dim, ndiv, minX, maxX, matids, create_bc, order, mats, bcs,
                 elem_coef=None, elem_order=None):
        L = lib()
        s = orc_grid_spec()
        s.dim = dim
        for i in range(3):
            s.ndiv[i] = ndiv[i] if i < len(ndiv) else 1
            s.minX[i] = minX[i]
            s.maxX[i] = maxX[i]
        for i, mid in enumerate(matids):
            s.matids[i] = mid
        s.create_bc = int(create_bc)
        s.default_order = order
        s.nmat = len(mats)
        for i, m in enumerate(mats):
            s.mats[i] = m
        s.nbc = len(bcs)
        for i, b in enumerate(bcs):
            s.bcs[i] = b
        self._coef = None if elem_coef is None else np.ascontiguousarray(elem_coef, dtype=np.float64)
        self._order = None if elem_order is None else np.ascontiguousarray(elem_order, dtype=np.int32)
        if self._coef is not None:
            s.elem_coef = self._coef.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        if self._order is not None:
            s.elem_order = self._order.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        self.h = L.orc_mesh_create(ctypes.byref(s))
        self.neq = L.orc_neq(self.h)
        self.ncel = L.orc_ncel(self.h)
        self.nconnects = L.orc_nconnects(self.h)
        self.nstate = L.orc_nstate(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mesh_free(self.h)
            self.h = None

    def blocks(self):
        pos = np.zeros(self.nconnects, np.int64)
        size = np.zeros(self.nconnects, np.int64)
        lib().orc_block_info(self.h, _p(pos), _p(size))
        return pos, size

    def nodes(self):
        n = lib().orc_nnodes(self.h)
        xyz = np.zeros((n, 3))
        lib().orc_nodes(self.h, _p(xyz))
        return xyz

    def set_nodes(self, xyz):
        xyz = np.ascontiguousarray(xyz, np.float64)
        lib().orc_set_nodes(self.h, _p(xyz))

    def cel(self, ic):
        t, b, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int64()
        conn = np.zeros(27, np.int64)
        dest = np.zeros(27 * 64 * 3, np.int64)
        n = lib().orc_cel_info(self.h, ic, ctypes.byref(t), ctypes.byref(b), ctypes.byref(g), _p(conn), _p(dest))
        ns = {T_LINE: 3, T_QUAD: 9, T_CUBE: 27}[t.value]
        return dict(type=t.value, is_bc=b.value, gel=g.value, conn=conn[:ns].copy(), dest=dest[:n].copy())

    def calc_stiff(self, ic):
        ek = np.zeros((192, 192))
        ef = np.zeros(192)
        n = lib().orc_calc_stiff(self.h, ic, _p(ek), _p(ef))
        # the C side writes an n x n column-major matrix at the start of the buffer
        flat = ek.reshape(-1)[: n * n].reshape(n, n).T.copy()
        return flat, ef[:n].copy()

    def error_points(self, exact_order):
        """Coordinates [npts][3] of the error-rule points, element after element (volume elements)."""
        n = lib().orc_error_points(self.h, int(exact_order), None)
        xyz = np.zeros((n, 3))
        lib().orc_error_points(self.h, int(exact_order), _p(xyz))
        return xyz

    def error_eval(self, exact_order, sol, u_exact, du_exact):
        """Error norms of sol against the exact solution values u_exact [npts][nstate] and gradients
        du_exact [npts][3][nstate] at error_points(): (mesh totals, per-element errors [ncel][nerr])."""
        sol = np.ascontiguousarray(sol, np.float64)
        ue = np.ascontiguousarray(u_exact, np.float64)
        due = np.ascontiguousarray(du_exact, np.float64)
        tot = np.zeros(6)
        el = np.zeros((self.ncel, 6))
        ne = lib().orc_error_eval(self.h, int(exact_order), _p(sol), _p(ue), _p(due), _p(tot), _p(el))
        return tot[:ne].copy(), el.reshape(-1)[: self.ncel * ne].reshape(self.ncel, ne).copy()

    def pattern(self, sym):
        nnz = lib().orc_pattern(self.h, int(sym), None, None)
        ia = np.zeros(self.neq + 1, np.int64)
        ja = np.zeros(nnz, np.int64)
        lib().orc_pattern(self.h, int(sym), _p(ia), _p(ja))
        return ia, ja

    def assemble(self, sym, ia, ja, nthreads=0):
        a = np.zeros(int(ia[-1]))
        f = np.zeros(self.neq)
        lib().orc_assemble(self.h, int(sym), _p(ia), _p(ja), _p(a), _p(f), int(nthreads))
        return a, f


def spmv(sym, ia, ja, a, x):
    z = np.zeros(len(ia) - 1)
    lib().orc_spmv(len(ia) - 1, int(sym), _p(ia), _p(ja), _p(a), _p(np.ascontiguousarray(x, np.float64)), _p(z))
    return z


def cg_jacobi(sym, ia, ja, a, b, maxit, tol, jacobi_residual=False, history=False):
    n = len(ia) - 1
    x = np.zeros(n)
    it, res = ctypes.c_int64(), ctypes.c_double()
    hist = np.zeros(maxit) if history else None
    rc = lib().orc_cg_jacobi(n, int(sym), _p(ia), _p(ja), _p(a), _p(np.ascontiguousarray(b)), _p(x), maxit, tol,
                             int(jacobi_residual), ctypes.byref(it), ctypes.byref(res), _p(hist))
    out = dict(x=x, iters=it.value, resid=res.value, rc=rc)
    if history:
        out["hist"] = hist[: it.value].copy()
    return out


def sloan(nnodes, elgraphindex, elgraph):
    """TPZSloanRenumbering::Resequence as the reference runs it: (rc, perm_gather, perm_scatter)."""
    ei = np.ascontiguousarray(elgraphindex, np.int64)
    eg = np.ascontiguousarray(elgraph, np.int64)
    g = np.zeros(nnodes, np.int64)
    sc = np.zeros(nnodes, np.int64)
    rc = lib().orc_sloan(nnodes, len(ei) - 1, _p(ei), _p(eg), _p(g), _p(sc))
    return rc, g, sc


def nodeset(nnodes, elgraphindex, elgraph, block_pos, block_size, neq):
    """TPZNodesetCompute's blocks as BuildPreconditioner(EBlockJacobi, overlap = false) computes them:
    (rc, dict of blockindex, blockeqs, colors, ncolors, seqnum, level)."""
    ei = np.ascontiguousarray(elgraphindex, np.int64)
    eg = np.ascontiguousarray(elgraph, np.int64)
    bp = np.ascontiguousarray(block_pos, np.int64)
    bs = np.ascontiguousarray(block_size, np.int64)
    bidx = np.zeros(nnodes + 1, np.int64)
    beqs = np.zeros(max(int(bs.sum()), 1), np.int64)
    cols = np.zeros(max(nnodes, 1), np.int32)
    seq = np.zeros(max(nnodes, 1), np.int64)
    lev = np.zeros(max(nnodes, 1), np.int32)
    nb, nc = ctypes.c_int64(0), ctypes.c_int32(0)
    rc = lib().orc_nodeset(nnodes, len(ei) - 1, _p(ei), _p(eg), _p(bp), _p(bs), neq, _p(bidx), _p(beqs),
                           ctypes.byref(nb), _p(cols), ctypes.byref(nc), _p(seq), _p(lev))
    nb = nb.value
    return rc, dict(blockindex=bidx[:nb + 1], blockeqs=beqs[:bidx[nb]], colors=cols[:nb], ncolors=nc.value,
                    seqnum=seq[:nnodes], level=lev[:nnodes])


def cg_sparse_block_jacobi(sym, ia, ja, a, b, blockindex, blockeqs, maxit, tol):
    """CG preconditioned by LU solves of the given equation blocks (the TPZSparseBlockDiagonal step solver)."""
    n = len(ia) - 1
    x = np.zeros(n)
    bi = np.ascontiguousarray(blockindex, np.int64)
    be = np.ascontiguousarray(blockeqs, np.int64)
    it, res = ctypes.c_int64(), ctypes.c_double()
    rc = lib().orc_cg_sparse_block_jacobi(n, int(sym), _p(ia), _p(ja), _p(a), _p(np.ascontiguousarray(b)), _p(x),
                                          len(bi) - 1, _p(bi), _p(be), maxit, tol, ctypes.byref(it),
                                          ctypes.byref(res))
    return dict(x=x, iters=it.value, resid=res.value, rc=rc)


def filter_system(sym, ia, ja, a, f, active):
    """An equation filter (TPZEquationFilter::SetActiveEquations, StrMatrix/TPZEquationFilter.h) applied as the
    reference applies it to an assembled system: TPZSSpStructMatrix / TPZSpStructMatrix::SetupMatrixData
    (StrMatrix/TPZSSpStructMatrix.cpp:49-193, StrMatrix/TPZSpStructMatrix.cpp:53-190) keep the rows and
    columns of active equations, renumbered in increasing order (fDestIndices); the filtered AddKel drops every
    element entry with an inactive row or column (TPZEquationFilter::Filter), so the condensed values are the
    mesh-level ones at the kept positions; the load vector assembled over the active equations is scattered
    back to the mesh's size with zeros elsewhere (StrMatrix/pzstrmatrixor.cpp:43-71), and the solve takes its
    gathered entries (Analysis/TPZLinearAnalysis.cpp:194).  Returns (ia, ja, a) of the condensed system, the
    mesh-size load vector and the condensed one."""
    n = len(ia) - 1
    act = np.unique(np.asarray(active, np.int64))
    dest = np.full(n, -1, np.int64)
    dest[act] = np.arange(len(act))
    ic, jc, vc = [0], [], []
    for r in act:
        cols = np.asarray(ja[ia[r]:ia[r + 1]])
        keep = dest[cols] >= 0
        jc.append(dest[cols[keep]])
        vc.append(np.asarray(a[ia[r]:ia[r + 1]])[keep])
        ic.append(ic[-1] + int(keep.sum()))
    fm = np.array(f, np.float64)
    fm[dest < 0] = 0.0
    return (np.array(ic, np.int64), np.concatenate(jc).astype(np.int64), np.concatenate(vc), fm,
            np.asarray(f, np.float64)[act])


def jacobi(sym, ia, ja, a, b, maxit, tol, x0=None):
    """Stationary Jacobi (TPZStepSolver::SetJacobi as the solver); tol on the absolute ||b - A x||; x0 = the
    FromCurrent initial guess."""
    n = len(ia) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    it, res = ctypes.c_int64(), ctypes.c_double()
    rc = lib().orc_jacobi(n, int(sym), _p(ia), _p(ja), _p(a), _p(np.ascontiguousarray(b)), _p(x), maxit, tol,
                          int(x0 is not None), ctypes.byref(it), ctypes.byref(res))
    return dict(x=x, iters=it.value, resid=res.value, rc=rc)


def cg_block_jacobi(sym, ia, ja, a, b, bs, maxit, tol):
    n = len(ia) - 1
    x = np.zeros(n)
    it, res = ctypes.c_int64(), ctypes.c_double()
    rc = lib().orc_cg_block_jacobi(n, int(sym), _p(ia), _p(ja), _p(a), _p(np.ascontiguousarray(b)), _p(x), bs, maxit,
                                   tol, ctypes.byref(it), ctypes.byref(res))
    return dict(x=x, iters=it.value, resid=res.value, rc=rc)


def gmres_jacobi(sym, ia, ja, a, b, m, maxit, tol):
    n = len(ia) - 1
    x = np.zeros(n)
    it, res = ctypes.c_int64(), ctypes.c_double()
    rc = lib().orc_gmres_jacobi(n, int(sym), _p(ia), _p(ja), _p(a), _p(np.ascontiguousarray(b)), _p(x), m, maxit,
                                tol, ctypes.byref(it), ctypes.byref(res))
    return dict(x=x, iters=it.value, resid=res.value, rc=rc)


def gauss(order):
    loc = np.zeros(64)
    w = np.zeros(64)
    n = lib().orc_gauss(order, _p(loc), _p(w))
    return loc[:n].copy(), w[:n].copy()


def shape(type, ids, orders, pt):
    ids = np.ascontiguousarray(ids, np.int64)
    orders = np.ascontiguousarray(orders, np.int32)
    pt = np.ascontiguousarray(pt, np.float64)
    phi = np.zeros(216)
    dphi = np.zeros(3 * 216)
    n = lib().orc_shape(type, _p(ids), _p(orders), _p(pt), _p(phi), _p(dphi), 216)
    return phi[:n].copy(), dphi.reshape(3, 216)[:, :n].copy()


# ---------------------------------------------------------------------------
# The synthetic workloads, as the reference user programs would build them.
# ---------------------------------------------------------------------------
def poisson_square_quadratic(n, p):
    """The error known-answer mesh of UnitTest_PZ/TestMesh/TestError.cpp:43-160 on quadrilaterals:
    [-1, 1]^2 in n x n quads of order p, -lap u = 4 - 2x^2 - 2y^2 (pOrder 2), u = 0 penalty Dirichlet;
    exact solution (x^2 - 1)(y^2 - 1) (in the order-2 space of quads)."""
    mats = [material(1, ORC_POISSON, 2, forcing=ORC_F_QUADRATIC, force=(4.0, -2.0, 0), forcing_porder=2)]
    bcs = [bc(-1, 1, 0)]
    return OracleMesh(2, (n, n), (-1, -1, 0), (1, 1, 0), [1, -1, -1, -1, -1], True, p, mats, bcs)


def poisson2d(n=64, p=2):
    """64x64 quads, H1 p, f = 2 pi^2 sin(pi x) sin(pi y) (pOrder 2), u = 0 penalty Dirichlet."""
    mats = [material(1, ORC_POISSON, 2, forcing=ORC_F_SINPROD, force=(1.0, 0, 0), forcing_porder=2)]
    bcs = [bc(-1, 1, 0)]
    return OracleMesh(2, (n, n), (0, 0, 0), (1, 1, 0), [1, -1, -1, -1, -1], True, p, mats, bcs)


def elasticity3d(n, p=2, E=None, nu=0.3, top_traction=True, side_bc=False, body_force=(0.0, 0.0, -1.0)):
    """Unit cube n^3 hexes, clamped z=0 face (type 0), traction (0,0,-1) on top (type 1),
    body force body_force; E per element (array) or 1."""
    mats = [material(1, ORC_ELAST3D, 3, E=1.0, nu=nu, force=tuple(body_force), forcing=ORC_F_CONST)]
    bcs = [bc(-1, 1, 0)]
    if top_traction:
        bcs.append(bc(-3, 1, 1, val2=(0, 0, -1.0)))
    matids = [1, -1, -2, -2, -2, -2, -3]
    return OracleMesh(3, (n, n, n), (0, 0, 0), (1, 1, 1), matids, True, p, mats, bcs, elem_coef=E)


def elasticity3d_hp(n, orders, E=None, nu=0.3):
    """hp elasticity: unit cube n^3 hexes, preferred order orders[e] per element (shared sides take the
    largest), body force (0,0,-1), clamped z=0 face; E per element (array) or 1."""
    mats = [material(1, ORC_ELAST3D, 3, E=1.0, nu=nu, force=(0, 0, -1.0), forcing=ORC_F_CONST)]
    bcs = [bc(-1, 1, 0)]
    matids = [1, -1, -2, -2, -2, -2, -2]
    return OracleMesh(3, (n, n, n), (0, 0, 0), (1, 1, 1), matids, True, 1, mats, bcs, elem_coef=E,
                      elem_order=np.ascontiguousarray(orders, np.int32))


def darcy_hp(n, orders, perm, rhs=1.0):
    """hp Darcy on the unit square, n x n quads of preferred orders orders[e], u = 0 on the boundary."""
    mats = [material(1, ORC_DARCY, 2, forcing=ORC_F_CONST, force=(rhs, 0, 0))]
    bcs = [bc(-1, 1, 0)]
    return OracleMesh(2, (n, n), (0, 0, 0), (1, 1, 0), [1, -1, -1, -1, -1], True, 1, mats, bcs, elem_coef=perm,
                      elem_order=np.ascontiguousarray(orders, np.int32))


def darcy(dim, n, p, perm, rhs=1.0):
    """-div(k grad u) = rhs on the unit square/cube with u = 0 penalty Dirichlet on every face."""
    mats = [material(1, ORC_DARCY, dim, forcing=ORC_F_CONST, force=(rhs, 0, 0))]
    bcs = [bc(-1, 1, 0)]
    if dim == 2:
        return OracleMesh(2, (n, n), (0, 0, 0), (1, 1, 0), [1, -1, -1, -1, -1], True, p, mats, bcs, elem_coef=perm)
    return OracleMesh(3, (n, n, n), (0, 0, 0), (1, 1, 1), [1, -1, -1, -1, -1, -1, -1], True, p, mats, bcs,
                      elem_coef=perm)
