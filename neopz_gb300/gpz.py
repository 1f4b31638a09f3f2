"""ctypes binding of the C ABI (include/gpz.h) and of the host grid builder.

This is the Python face of the product used by the benchmark and the tests;
every numerical operation runs in libgpz.so on the GPU.  Loading fails loudly
when the shared libraries have not been built, and creating a context fails
when no CUDA device is visible: there is no CPU path.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBGPZ = os.path.join(_HERE, "_build", "libgpz.so")
LIBHOST = os.path.join(_HERE, "_build", "libgpzhost.so")

GPZ_OK, GPZ_NOT_CONVERGED, GPZ_CANCELLED = 0, 1, 2
GPZ_EL_LINE, GPZ_EL_QUAD, GPZ_EL_HEX = 1, 2, 3
GPZ_MAT_POISSON, GPZ_MAT_DARCY, GPZ_MAT_ELAST3D = 1, 2, 3
GPZ_F_NONE, GPZ_F_CONST, GPZ_F_SINPROD, GPZ_F_QUADRATIC = 0, 1, 2, 3
GPZ_PREC_FP64, GPZ_PREC_MIXED = 0, 1
GPZ_FP32_ROUNDED, GPZ_FP32_ELEMENTS = 0, 1
GPZ_SOLVER_CG, GPZ_SOLVER_GMRES, GPZ_SOLVER_MIXED_CG, GPZ_SOLVER_LEARNED_FCG, GPZ_SOLVER_LEARNED_MIXED_FCG = 1, 2, 3, 4, 5
GPZ_SOLVER_JACOBI = 6
GPZ_PRECOND_JACOBI, GPZ_PRECOND_BLOCK_JACOBI, GPZ_PRECOND_NODESET_JACOBI, GPZ_PRECOND_TWO_LEVEL = 1, 2, 3, 4
GPZ_KERNEL_SPMV_FP64, GPZ_KERNEL_SPMV_FP32, GPZ_KERNEL_ASSEMBLE = 1, 2, 3
BIGNUMBER = 10.0 ** 17 * 2 / 3  # TPZMaterial::fBigNumber default for double


class gpz_material(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("dim", ctypes.c_int32), ("scale", ctypes.c_double),
                ("E", ctypes.c_double), ("nu", ctypes.c_double), ("coef_const", ctypes.c_double),
                ("force", ctypes.c_double * 3), ("forcing", ctypes.c_int32), ("forcing_porder", ctypes.c_int32),
                ("bignumber", ctypes.c_double)]


class gpz_bc(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("material", ctypes.c_int32), ("val1", ctypes.c_double * 9),
                ("val2", ctypes.c_double * 3)]


_P = ctypes.POINTER


class gpz_mesh_desc(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("nstate", ctypes.c_int32), ("nnodes", ctypes.c_int64),
                ("node_xyz", _P(ctypes.c_double)), ("nel", ctypes.c_int64), ("el_type", _P(ctypes.c_int32)),
                ("el_mat", _P(ctypes.c_int32)), ("el_nodes", _P(ctypes.c_int64)), ("el_order", _P(ctypes.c_int32)),
                ("el_conn", _P(ctypes.c_int64)), ("el_coef", _P(ctypes.c_double)), ("nconnects", ctypes.c_int64),
                ("conn_order", _P(ctypes.c_int32)), ("block_pos", _P(ctypes.c_int64)),
                ("block_size", _P(ctypes.c_int32)), ("neq", ctypes.c_int64), ("nmat", ctypes.c_int32),
                ("mats", _P(gpz_material)), ("nbc", ctypes.c_int32), ("bcs", _P(gpz_bc))]


class gpz_solver_opts(ctypes.Structure):
    _fields_ = [("solver", ctypes.c_int32), ("precond", ctypes.c_int32), ("max_iter", ctypes.c_int64),
                ("tol", ctypes.c_double), ("gmres_krylov", ctypes.c_int32), ("check_every", ctypes.c_int32),
                ("reliable_delta", ctypes.c_double), ("use_graph", ctypes.c_int32), ("from_current", ctypes.c_int32),
                ("spmv_variant", ctypes.c_int32)]


class gpz_solve_report(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int64), ("resid", ctypes.c_double), ("true_resid", ctypes.c_double),
                ("seconds", ctypes.c_double), ("spmv_fp64", ctypes.c_int64), ("spmv_fp32", ctypes.c_int64),
                ("reliable_updates", ctypes.c_int64), ("restarts", ctypes.c_int64)]


class gpzh_grid_spec(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("ndiv", ctypes.c_int32 * 3), ("minX", ctypes.c_double * 3),
                ("maxX", ctypes.c_double * 3), ("matids", ctypes.c_int32 * 7), ("create_bc", ctypes.c_int32),
                ("default_order", ctypes.c_int32), ("nmat", ctypes.c_int32), ("mat_id", ctypes.c_int32 * 4),
                ("mats", gpz_material * 4), ("nbc", ctypes.c_int32), ("bc_id", ctypes.c_int32 * 8),
                ("bcs", gpz_bc * 8), ("elem_coef", _P(ctypes.c_double)), ("elem_order", _P(ctypes.c_int32))]


class GpzError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gpz error {code}: {msg}")
        self.code = code


_lib = None
_host = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIBGPZ):
            raise ImportError(f"{LIBGPZ} is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIBGPZ)
        vp, i64, i32, dp = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        L.gpz_ctx_create.argtypes = [_P(vp), i32]
        L.gpz_ctx_destroy.argtypes = [vp]
        L.gpz_two_level_config.argtypes = [vp, i32]
        L.gpz_two_level_info.argtypes = [vp, vp]
        L.gpz_precond_apply.argtypes = [vp, i32, vp, vp]
        L.gpz_learned_set_base.argtypes = [vp, i32]
        L.gpz_get_error_string.restype = ctypes.c_char_p
        L.gpz_get_error_string.argtypes = [i32]
        L.gpz_last_error_detail.restype = ctypes.c_char_p
        L.gpz_last_error_detail.argtypes = [vp]
        L.gpz_ctx_stream.restype = vp
        L.gpz_ctx_stream.argtypes = [vp]
        L.gpz_kernel_launches.restype = i64
        L.gpz_kernel_launches.argtypes = [vp]
        L.gpz_mesh_upload.argtypes = [vp, _P(gpz_mesh_desc)]
        L.gpz_pattern_build.argtypes = [vp, i32, _P(i64)]
        L.gpz_pattern_upload.argtypes = [vp, i32, i64, vp, vp]
        L.gpz_pattern_download.argtypes = [vp, vp, vp]
        L.gpz_pattern_info.argtypes = [vp, _P(i64), _P(i64)]
        L.gpz_time_kernel.argtypes = [vp, i32, i32, _P(dp)]
        L.gpz_tuning_report.argtypes = [vp, ctypes.c_char_p, i64]
        L.gpz_tuning_cache.argtypes = [vp, ctypes.c_char_p]
        L.gpz_assembly_mode.argtypes = [vp, ctypes.c_int]
        L.gpz_fp32_elements.argtypes = [vp, ctypes.c_int]
        L.gpz_matrix_fp32_download.argtypes = [vp, vp]
        L.gpz_assemble.argtypes = [vp, i32]
        L.gpz_set_killed.argtypes = [vp, i32]
        L.gpz_equation_filter.argtypes = [vp, i64, vp]
        L.gpz_sloan_resequence.argtypes = [i64, i64, vp, vp, vp, vp]
        L.gpz_nodeset_blocks.argtypes = [i64, i64, vp, vp, vp, vp, i64, vp, vp, _P(i64), vp, _P(i32), vp, vp]
        L.gpz_element_colours.argtypes = [i64, vp, vp, i64, vp, vp, _P(i32)]
        L.gpz_matrix_download.argtypes = [vp, vp]
        L.gpz_rhs_download.argtypes = [vp, vp]
        L.gpz_rhs_upload.argtypes = [vp, vp]
        L.gpz_spmv.argtypes = [vp, dp, vp, dp, vp, vp]
        L.gpz_solve.argtypes = [vp, _P(gpz_solver_opts), vp, vp, _P(gpz_solve_report)]
        L.gpz_solution_download.argtypes = [vp, vp]
        L.gpz_mesh_set_coef.argtypes = [vp, vp]
        L.gpz_assembly_report.argtypes = [vp, ctypes.c_char_p, i64]
        L.gpz_assemble_rhs.argtypes = [vp]
        L.gpz_spmv_fp32.argtypes = [vp, i32, vp, vp]
        L.gpz_error_points.argtypes = [vp, i32, _P(i64), vp]
        L.gpz_error_evaluate.argtypes = [vp, i32, vp, vp, vp, _P(i32), vp, vp]
        L.gpz_learned_init.argtypes = [vp, i32, ctypes.c_uint64]
        L.gpz_learned_num_params.argtypes = [vp, _P(i64)]
        L.gpz_learned_get_params.argtypes = [vp, vp, i64]
        L.gpz_learned_set_params.argtypes = [vp, vp, i64]
        L.gpz_learned_collect.argtypes = [vp, i32, dp, i64, _P(i64)]
        L.gpz_learned_set_pairs.argtypes = [vp, i32, vp, vp]
        L.gpz_learned_loss_grad.argtypes = [vp, _P(dp), vp, i64]
        L.gpz_learned_train.argtypes = [vp, i32, dp, _P(dp), _P(dp)]
        _lib = L
    return _lib


def host():
    global _host
    if _host is None:
        lib()
        if not os.path.exists(LIBHOST):
            raise ImportError(f"{LIBHOST} is not built")
        H = ctypes.CDLL(LIBHOST)
        vp, i64 = ctypes.c_void_p, ctypes.c_int64
        H.gpzh_grid_build.restype = vp
        H.gpzh_grid_build.argtypes = [_P(gpzh_grid_spec)]
        H.gpzh_grid_free.argtypes = [vp]
        H.gpzh_grid_desc.argtypes = [vp, _P(gpz_mesh_desc)]
        for f in ("gpzh_grid_neq", "gpzh_grid_nel", "gpzh_grid_nvol"):
            getattr(H, f).restype = i64
            getattr(H, f).argtypes = [vp]
        H.gpzh_grid_dest.restype = ctypes.c_int
        H.gpzh_grid_dest.argtypes = [vp, i64, vp]
        H.gpzh_grid_cells.restype = ctypes.c_int
        H.gpzh_grid_cells.argtypes = [vp, vp]
        _host = H
    return _host


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def material(kind, dim, scale=1.0, E=1.0, nu=0.3, coef_const=1.0, force=(0.0, 0.0, 0.0), forcing=GPZ_F_NONE,
             forcing_porder=0, bignumber=BIGNUMBER):
    m = gpz_material()
    m.kind, m.dim, m.scale, m.E, m.nu, m.coef_const = kind, dim, scale, E, nu, coef_const
    for i in range(3):
        m.force[i] = force[i]
    m.forcing, m.forcing_porder, m.bignumber = forcing, forcing_porder, bignumber
    return m


def bc(type, material_index, val2=(0.0, 0.0, 0.0)):
    b = gpz_bc()
    b.type, b.material = type, material_index
    for i in range(3):
        b.val2[i] = val2[i]
    return b


class Grid:
    """A computational mesh on a grid domain built by the host library (pz_grid.cpp)."""

    def __init__(self, dim, ndiv, minX, maxX, matids, create_bc, order, mats, bcs, elem_coef=None,
                 elem_order=None):
        H = host()
        s = gpzh_grid_spec()
        s.dim = dim
        for i in range(3):
            s.ndiv[i] = ndiv[i] if i < len(ndiv) else 1
            s.minX[i], s.maxX[i] = minX[i], maxX[i]
        for i, m in enumerate(matids):
            s.matids[i] = m
        s.create_bc, s.default_order = int(create_bc), order
        s.nmat = len(mats)
        for i, (mid, m) in enumerate(mats):
            s.mat_id[i], s.mats[i] = mid, m
        s.nbc = len(bcs)
        for i, (bid, b) in enumerate(bcs):
            s.bc_id[i], s.bcs[i] = bid, b
        self._coef = None if elem_coef is None else np.ascontiguousarray(elem_coef, np.float64)
        self._order = None if elem_order is None else np.ascontiguousarray(elem_order, np.int32)
        if self._coef is not None:
            s.elem_coef = self._coef.ctypes.data_as(_P(ctypes.c_double))
        if self._order is not None:
            s.elem_order = self._order.ctypes.data_as(_P(ctypes.c_int32))
        self.h = H.gpzh_grid_build(ctypes.byref(s))
        if not self.h:
            raise GpzError(-3, "grid build failed")
        self.neq = H.gpzh_grid_neq(self.h)
        self.nel = H.gpzh_grid_nel(self.h)
        self.nvol = H.gpzh_grid_nvol(self.h)
        self.desc = gpz_mesh_desc()
        H.gpzh_grid_desc(self.h, ctypes.byref(self.desc))

    def nodes(self):
        """Node coordinates [nnodes][3] of the descriptor (a writable view: edit before upload_mesh)."""
        return np.ctypeslib.as_array(self.desc.node_xyz, shape=(self.desc.nnodes, 3))

    def element_graph(self):
        """TPZCompMesh::ComputeElGraph of the descriptor: (elgraphindex [nel+1], elgraph), the connects of every
        element (boundary elements included)."""
        d = self.desc
        types = np.ctypeslib.as_array(d.el_type, shape=(d.nel,))
        conn = np.ctypeslib.as_array(d.el_conn, shape=(d.nel * 27,))
        ns = np.array([0, 3, 9, 27])[types]
        idx = np.concatenate([[0], np.cumsum(ns)]).astype(np.int64)
        keep = np.arange(27)[None, :] < ns[:, None]  # the first ns[e] sides of element e, in element order
        g = conn.reshape(d.nel, 27)[keep]
        return idx, g.astype(np.int64)

    def permute_connects(self, perm_gather):
        """TPZCompMesh::Permute (Mesh/pzcmesh.cpp:1399-1460) on the descriptor: connect s gets sequence number
        perm_gather[s]; block sizes, orders and positions follow.  Returns old -> new equation map."""
        d = self.desc
        nc, nel = d.nconnects, d.nel
        perm = np.asarray(perm_gather, np.int64)
        size = np.ctypeslib.as_array(d.block_size, shape=(nc,)).copy()
        order = np.ctypeslib.as_array(d.conn_order, shape=(nc,)).copy()
        pos = np.ctypeslib.as_array(d.block_pos, shape=(nc,)).copy()
        new_size, new_order = np.empty_like(size), np.empty_like(order)
        new_size[perm] = size
        new_order[perm] = order
        new_pos = np.concatenate([[0], np.cumsum(new_size)[:-1]]).astype(np.int64)
        np.ctypeslib.as_array(d.block_size, shape=(nc,))[:] = new_size
        np.ctypeslib.as_array(d.conn_order, shape=(nc,))[:] = new_order
        np.ctypeslib.as_array(d.block_pos, shape=(nc,))[:] = new_pos
        conn = np.ctypeslib.as_array(d.el_conn, shape=(nel * 27,))
        types = np.ctypeslib.as_array(d.el_type, shape=(nel,))
        for e in range(nel):
            ns = (0, 3, 9, 27)[int(types[e])]
            conn[e * 27:e * 27 + ns] = perm[conn[e * 27:e * 27 + ns]]
        eqmap = np.empty(d.neq, np.int64)
        for c in range(nc):
            eqmap[pos[c]:pos[c] + size[c]] = new_pos[perm[c]] + np.arange(size[c])
        return eqmap

    def cells(self):
        """Grid cell of every element (-1 for boundary elements)."""
        c = np.zeros(self.nel, np.int64)
        host().gpzh_grid_cells(self.h, _p(c))
        return c

    def element_coef(self, cell_coef):
        """Per-element coefficient array (the el_coef of the descriptor) from per-cell values."""
        c = self.cells()
        out = np.zeros(self.nel)
        out[c >= 0] = np.asarray(cell_coef, np.float64)[c[c >= 0]]
        return out

    def dest(self, e):
        d = np.zeros(64 * 3 * 27, np.int64)
        n = host().gpzh_grid_dest(self.h, e, _p(d))
        return d[:n].copy()

    def __del__(self):
        if getattr(self, "h", None):
            host().gpzh_grid_free(self.h)
            self.h = None


class Context:
    """One gpz context (one CUDA stream, its device buffers)."""

    def __init__(self, device=0):
        L = lib()
        h = ctypes.c_void_p()
        rc = L.gpz_ctx_create(ctypes.byref(h), device)
        if rc != GPZ_OK:
            raise GpzError(rc, L.gpz_get_error_string(rc).decode())
        self.h = h
        self.neq = 0
        self.nnz = 0

    def _check(self, rc, allow=()):
        if rc != GPZ_OK and rc not in allow:
            L = lib()
            raise GpzError(rc, L.gpz_get_error_string(rc).decode() + ": " + L.gpz_last_error_detail(self.h).decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            lib().gpz_ctx_destroy(self.h)
            self.h = None

    __del__ = close

    @property
    def stream(self):
        return lib().gpz_ctx_stream(self.h)

    def launches(self):
        return lib().gpz_kernel_launches(self.h)

    def upload_mesh(self, grid):
        self._grid = grid
        self._check(lib().gpz_mesh_upload(self.h, ctypes.byref(grid.desc)))
        self.neq = grid.neq       # equations of the system (the active ones under an equation filter)
        self.neq_mesh = grid.neq  # equations of the mesh
        self.nel = grid.nel

    def build_pattern(self, sym):
        nnz = ctypes.c_int64()
        self._check(lib().gpz_pattern_build(self.h, int(sym), ctypes.byref(nnz)))
        self.nnz = nnz.value
        return self.nnz

    def nnz_full(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._check(lib().gpz_pattern_info(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value

    def time_kernel(self, which, reps):
        ms = ctypes.c_double()
        self._check(lib().gpz_time_kernel(self.h, which, reps, ctypes.byref(ms)))
        return ms.value

    def assembly_mode(self, mode):
        """-1 autotuned, 0 a launch per element bucket and colour (the default), 1 persistent per bucket."""
        self._check(lib().gpz_assembly_mode(self.h, int(mode)))

    def fp32_elements(self, source):
        """Source of the FP32 values of GPZ_PREC_MIXED: GPZ_FP32_ROUNDED (the FP64 matrix rounded, the default)
        or GPZ_FP32_ELEMENTS (element matrices formed again in FP32: 3xTF32 tcgen05 products on the hexes)."""
        self._check(lib().gpz_fp32_elements(self.h, int(source)))

    def matrix_fp32(self):
        """FP32 values of the last mixed assembly on the full CSR pattern (gpz_matrix_fp32_download)."""
        a = np.zeros(self.nnz_full(), dtype=np.float32)
        self._check(lib().gpz_matrix_fp32_download(self.h, _p(a)))
        return a

    def tuning_cache(self, path):
        """File of the autotuners' choices kept across runs (gpz_tuning_cache); None: no cache."""
        self._cache_path = None if path is None else str(path).encode()
        self._check(lib().gpz_tuning_cache(self.h, self._cache_path))

    def tuning_report(self):
        import json
        buf = ctypes.create_string_buffer(4096)
        self._check(lib().gpz_tuning_report(self.h, buf, 4096))
        return json.loads(buf.value.decode())

    def pattern(self):
        ia = np.zeros(self.neq + 1, np.int64)
        ja = np.zeros(self.nnz, np.int64)
        self._check(lib().gpz_pattern_download(self.h, _p(ia), _p(ja)))
        return ia, ja

    def assemble(self, precision=GPZ_PREC_FP64):
        """GPZ_OK, or GPZ_CANCELLED (nothing assembled) while set_killed(True) holds."""
        return self._check(lib().gpz_assemble(self.h, precision), allow=(GPZ_CANCELLED,))

    def set_killed(self, killed=True):
        """TPZGuiInterface::SetKilled: assemblies return GPZ_CANCELLED, solves stop at their next batch boundary;
        callable from another thread while a call on this context runs."""
        self._check(lib().gpz_set_killed(self.h, int(bool(killed))))

    def matrix(self):
        a = np.zeros(self.nnz)
        self._check(lib().gpz_matrix_download(self.h, _p(a)))
        return a

    def equation_filter(self, active=None):
        """TPZEquationFilter::SetActiveEquations (active: mesh equation numbers) or Reset (None); call before
        build_pattern.  The system then has the active equations in increasing order."""
        if active is None:
            self._check(lib().gpz_equation_filter(self.h, -1, None))
            self.neq = self.neq_mesh
            return
        a = np.ascontiguousarray(active, np.int64)
        self._check(lib().gpz_equation_filter(self.h, len(a), _p(a)))
        self.neq = len(np.unique(a))

    def rhs(self):
        """The load vector over the mesh equations (zeros at inactive ones under an equation filter)."""
        f = np.zeros(self.neq_mesh)
        self._check(lib().gpz_rhs_download(self.h, _p(f)))
        return f

    def spmv(self, x, alpha=1.0, beta=0.0, y=None):
        z = np.zeros(self.neq)
        x = np.ascontiguousarray(x, np.float64)
        yy = None if y is None else np.ascontiguousarray(y, np.float64)
        self._check(lib().gpz_spmv(self.h, alpha, _p(x), beta, _p(yy), _p(z)))
        return z

    def spmv_fp32(self, x, variant=-1):
        """y = A32 x with the mixed solvers' FP32 operator (autotuned layout, or `variant`)."""
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.neq)
        self._check(lib().gpz_spmv_fp32(self.h, variant, _p(x), _p(y)))
        return y

    def error_points(self, exact_order):
        """Coordinates [npts][3] of the error-rule points of every volume element (element order)."""
        n = ctypes.c_int64()
        self._check(lib().gpz_error_points(self.h, int(exact_order), ctypes.byref(n), None))
        xyz = np.zeros((n.value, 3))
        self._check(lib().gpz_error_points(self.h, int(exact_order), ctypes.byref(n), _p(xyz)))
        return xyz

    def error_norms(self, exact_order, u_exact, du_exact, sol=None):
        """Error norms against the exact solution values u_exact [npts][nstate] and gradients
        du_exact [npts][3][nstate] at error_points(exact_order); sol: host solution, or None for the last
        solve's device solution.  Returns (mesh norms [nerr], per-element errors [nel][nerr])."""
        ue = np.ascontiguousarray(u_exact, np.float64)
        due = np.ascontiguousarray(du_exact, np.float64)
        x = None if sol is None else np.ascontiguousarray(sol, np.float64)
        tot = np.zeros(6)
        el = np.zeros(self.nel * 6)
        ne = ctypes.c_int32()
        self._check(lib().gpz_error_evaluate(self.h, int(exact_order), _p(x), _p(ue), _p(due), ctypes.byref(ne),
                                             _p(tot), _p(el)))
        k = ne.value
        return tot[:k].copy(), el[: self.nel * k].reshape(self.nel, k).copy()

    def evaluate_error(self, exact, exact_order, sol=None):
        """TPZAnalysis::PostProcessError with a vectorised exact solution: exact(xyz [n][3]) ->
        (u [n][nstate], du [n][3][nstate])."""
        u, du = exact(self.error_points(exact_order))
        return self.error_norms(exact_order, u, du, sol)

    def assemble_rhs(self):
        """Load vector alone (no matrix); read it with rhs()."""
        return self._check(lib().gpz_assemble_rhs(self.h), allow=(GPZ_CANCELLED,))

    def assembly_report(self):
        import json
        buf = ctypes.create_string_buffer(4096)
        self._check(lib().gpz_assembly_report(self.h, buf, 4096))
        return json.loads(buf.value.decode())

    def set_coef(self, grid, cell_coef):
        """New per-cell coefficients for the uploaded mesh (same numbering and pattern)."""
        self._coef_keep = np.ascontiguousarray(grid.element_coef(cell_coef))
        self._check(lib().gpz_mesh_set_coef(self.h, _p(self._coef_keep)))

    # ---- learned preconditioner
    def learned_init(self, rank=4, seed=0):
        self._check(lib().gpz_learned_init(self.h, rank, seed))
        n = ctypes.c_int64()
        self._check(lib().gpz_learned_num_params(self.h, ctypes.byref(n)))
        self.learned_nparams = n.value
        return n.value

    def learned_params(self):
        p = np.zeros(self.learned_nparams, np.float32)
        self._check(lib().gpz_learned_get_params(self.h, _p(p), len(p)))
        return p

    def set_learned_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self._check(lib().gpz_learned_set_params(self.h, _p(p), len(p)))

    def learned_set_base(self, precond):
        self._check(lib().gpz_learned_set_base(self.h, int(precond)))

    def learned_collect(self, npairs=16, tol=1e-12, max_iter=200000):
        its = ctypes.c_int64()
        self._check(lib().gpz_learned_collect(self.h, npairs, tol, max_iter, ctypes.byref(its)))
        return its.value

    def learned_set_pairs(self, R, E):
        R = np.ascontiguousarray(R, np.float64)
        E = np.ascontiguousarray(E, np.float64)
        self._check(lib().gpz_learned_set_pairs(self.h, R.shape[0], _p(R), _p(E)))

    def learned_loss_grad(self, want_grad=True):
        loss = ctypes.c_double()
        g = np.zeros(self.learned_nparams, np.float32) if want_grad else None
        self._check(lib().gpz_learned_loss_grad(self.h, ctypes.byref(loss), _p(g), self.learned_nparams))
        return loss.value, g

    def learned_train(self, steps=8, lr=3e-3):
        l0, l1 = ctypes.c_double(), ctypes.c_double()
        self._check(lib().gpz_learned_train(self.h, steps, lr, ctypes.byref(l0), ctypes.byref(l1)))
        return l0.value, l1.value

    def precond_apply(self, precond, r):
        r = np.ascontiguousarray(r, np.float64)
        z = np.zeros(self.neq)
        self._check(lib().gpz_precond_apply(self.h, int(precond), _p(r), _p(z)))
        return z

    def two_level_config(self, coarse_boxes):
        self._check(lib().gpz_two_level_config(self.h, int(coarse_boxes)))

    def two_level_info(self):
        v = np.zeros(9, np.int64)
        self._check(lib().gpz_two_level_info(self.h, _p(v)))
        return dict(fine_cells=v[0:3].tolist(), s=int(v[3]), coarse_boxes=v[4:7].tolist(), coarse_eqs=int(v[7]),
                    removed_nodes=int(v[8]))

    def solution(self):
        """The device solution of the last solve (gpz_solution_download)."""
        x = np.zeros(self.neq)
        self._check(lib().gpz_solution_download(self.h, _p(x)))
        return x

    def solve(self, solver=GPZ_SOLVER_CG, precond=GPZ_PRECOND_JACOBI, max_iter=20000, tol=1e-8, b=None,
              check_every=32, reliable_delta=1e-3, use_graph=True, x0=None, want_x=True, gmres_krylov=30,
              spmv_variant=-1):
        o = gpz_solver_opts()
        o.solver, o.precond, o.max_iter, o.tol = solver, precond, max_iter, tol
        o.gmres_krylov, o.check_every, o.reliable_delta, o.use_graph = gmres_krylov, check_every, reliable_delta, \
            int(use_graph)
        o.from_current = int(x0 is not None)
        o.spmv_variant = spmv_variant
        rep = gpz_solve_report()
        x = None
        if want_x or x0 is not None:
            x = np.zeros(self.neq) if x0 is None else np.array(x0, np.float64)
        bb = None if b is None else np.ascontiguousarray(b, np.float64)
        rc = self._check(lib().gpz_solve(self.h, ctypes.byref(o), _p(bb), _p(x), ctypes.byref(rep)),
                         allow=(GPZ_NOT_CONVERGED, GPZ_CANCELLED))
        return dict(rc=rc, x=x, iterations=rep.iterations, resid=rep.resid, true_resid=rep.true_resid,
                    seconds=rep.seconds, spmv_fp64=rep.spmv_fp64, spmv_fp32=rep.spmv_fp32,
                    reliable_updates=rep.reliable_updates, restarts=rep.restarts)


# ---------------------------------------------------------------------------
# Synthetic workloads (the user programs of the reference's configurations).
# ---------------------------------------------------------------------------
def sloan_resequence(nnodes, elgraphindex, elgraph):
    """TPZSloanRenumbering::Resequence on the host (gpz_sloan_resequence): (perm_gather, perm_scatter)."""
    ei = np.ascontiguousarray(elgraphindex, np.int64)
    eg = np.ascontiguousarray(elgraph, np.int64)
    g = np.zeros(nnodes, np.int64)
    s = np.zeros(nnodes, np.int64)
    rc = lib().gpz_sloan_resequence(nnodes, len(ei) - 1, _p(ei), _p(eg), _p(g), _p(s))
    if rc != GPZ_OK:
        raise GpzError(rc, lib().gpz_get_error_string(rc).decode())
    return g, s


def element_colours(elgraphindex, elgraph, block_size):
    """The element colouring of the atomic-free scatter (gpz_element_colours): (colours [nel], ncolours)."""
    ei = np.ascontiguousarray(elgraphindex, np.int64)
    eg = np.ascontiguousarray(elgraph, np.int64)
    bs = np.ascontiguousarray(block_size, np.int64)
    nel = len(ei) - 1
    col = np.zeros(max(nel, 1), np.int32)
    nc = ctypes.c_int32(0)
    rc = lib().gpz_element_colours(nel, _p(ei), _p(eg), len(bs), _p(bs), _p(col), ctypes.byref(nc))
    if rc != 0:
        raise GpzError(rc, lib().gpz_get_error_string(rc).decode())
    return col[:nel], nc.value


def nodeset_blocks(nnodes, elgraphindex, elgraph, block_pos, block_size, neq):
    """The node-set blocks of BuildPreconditioner(EBlockJacobi, overlap = false) on the host
    (gpz_nodeset_blocks): dict of blockindex, blockeqs (the equations of each block), colors, ncolors and the
    connects' seqnum / level."""
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
    rc = lib().gpz_nodeset_blocks(nnodes, len(ei) - 1, _p(ei), _p(eg), _p(bp), _p(bs), neq, _p(bidx), _p(beqs),
                                  ctypes.byref(nb), _p(cols), ctypes.byref(nc), _p(seq), _p(lev))
    if rc != GPZ_OK:
        raise GpzError(rc, lib().gpz_get_error_string(rc).decode())
    nb = nb.value
    return dict(blockindex=bidx[:nb + 1], blockeqs=beqs[:bidx[nb]], colors=cols[:nb], ncolors=nc.value,
                seqnum=seq[:nnodes], level=lev[:nnodes])


def poisson_square_quadratic(n, p):
    """[-1, 1]^2 in n x n quads of order p, -lap u = 4 - 2x^2 - 2y^2 (pOrder 2), u = 0 penalty Dirichlet: the
    error known-answer problem of UnitTest_PZ/TestMesh/TestError.cpp:43-160 (there on triangles), whose exact
    solution (x^2 - 1)(y^2 - 1) lies in the order-2 space of quadrilaterals."""
    mats = [(1, material(GPZ_MAT_POISSON, 2, forcing=GPZ_F_QUADRATIC, force=(4.0, -2.0, 0), forcing_porder=2))]
    bcs = [(-1, bc(0, 0))]
    return Grid(2, (n, n), (-1, -1, 0), (1, 1, 0), [1, -1, -1, -1, -1], True, p, mats, bcs)


def poisson2d(n=64, p=2):
    """Unit square, n x n quads, H1 p, f = 2 pi^2 sin(pi x) sin(pi y) (pOrder 2), u = 0 penalty Dirichlet."""
    mats = [(1, material(GPZ_MAT_POISSON, 2, forcing=GPZ_F_SINPROD, force=(1.0, 0, 0), forcing_porder=2))]
    bcs = [(-1, bc(0, 0))]
    return Grid(2, (n, n), (0, 0, 0), (1, 1, 0), [1, -1, -1, -1, -1], True, p, mats, bcs)


def elasticity3d(n, p=2, E=None, nu=0.3, top_traction=True, body_force=(0.0, 0.0, -1.0)):
    """Unit cube, n^3 hexes, E per element (or 1), nu, body force, z=0 clamped, traction (0,0,-1) on top."""
    mats = [(1, material(GPZ_MAT_ELAST3D, 3, E=1.0, nu=nu, force=body_force, forcing=GPZ_F_CONST))]
    bcs = [(-1, bc(0, 0))]
    if top_traction:
        bcs.append((-3, bc(1, 0, (0, 0, -1.0))))
    return Grid(3, (n, n, n), (0, 0, 0), (1, 1, 1), [1, -1, -2, -2, -2, -2, -3], True, p, mats, bcs, elem_coef=E)


def elasticity3d_hp(n, orders, E=None, nu=0.3, body_force=(0.0, 0.0, -1.0)):
    """hp elasticity (the 40^3 uneven-p workload at n = 40): unit cube n^3 hexes, preferred order orders[e] per
    element, every shared side at the largest order of its elements (SetSideOrder max rule), body force,
    clamped z = 0 face."""
    mats = [(1, material(GPZ_MAT_ELAST3D, 3, E=1.0, nu=nu, force=body_force, forcing=GPZ_F_CONST))]
    bcs = [(-1, bc(0, 0))]
    return Grid(3, (n, n, n), (0, 0, 0), (1, 1, 1), [1, -1, -2, -2, -2, -2, -2], True, 1, mats, bcs, elem_coef=E,
                elem_order=orders)


def darcy_hp(n, orders, perm, rhs=1.0):
    """hp Darcy on the unit square: n x n quads of preferred orders orders[e], u = 0 on the boundary."""
    mats = [(1, material(GPZ_MAT_DARCY, 2, forcing=GPZ_F_CONST, force=(rhs, 0, 0)))]
    bcs = [(-1, bc(0, 0))]
    return Grid(2, (n, n), (0, 0, 0), (1, 1, 0), [1, -1, -1, -1, -1], True, 1, mats, bcs, elem_coef=perm,
                elem_order=orders)


def hp_orders(ncells, seed, low=1, high=3):
    """Preferred orders uniform in {low..high} per element from a seeded PCG64 stream."""
    return np.random.default_rng(seed).integers(low, high + 1, ncells).astype(np.int32)


def darcy(dim, n, p, perm, rhs=1.0):
    """-div(k grad u) = rhs on the unit square/cube, u = 0 penalty Dirichlet on the whole boundary."""
    mats = [(1, material(GPZ_MAT_DARCY, dim, forcing=GPZ_F_CONST, force=(rhs, 0, 0)))]
    bcs = [(-1, bc(0, 0))]
    if dim == 2:
        return Grid(2, (n, n), (0, 0, 0), (1, 1, 0), [1, -1, -1, -1, -1], True, p, mats, bcs, elem_coef=perm)
    return Grid(3, (n, n, n), (0, 0, 0), (1, 1, 1), [1, -1, -1, -1, -1, -1, -1], True, p, mats, bcs, elem_coef=perm)


def grf2d(n, sigma=1.5, ell=0.1, seed=0):
    """exp(g) on the n x n cell centroids of the unit square, g a Gaussian random field with covariance
    sigma^2 exp(-|x - y|^2 / (2 ell^2)), sampled by circulant embedding on the 2n x 2n periodic grid
    (negative eigenvalues of the embedding clipped to zero) from a seeded PCG64 stream; cell index
    ix + n iy, the element order of the grid."""
    m, h = 2 * n, 1.0 / n
    i = np.arange(m)
    d = np.minimum(i, m - i) * h
    c = sigma ** 2 * np.exp(-(d[:, None] ** 2 + d[None, :] ** 2) / (2 * ell ** 2))
    lam = np.maximum(np.real(np.fft.fft2(c)), 0.0)
    rng = np.random.default_rng(seed)
    xi = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    g = np.real(np.fft.fft2(np.sqrt(lam / (m * m)) * xi))[:n, :n]
    return np.exp(g.reshape(-1))


def darcy_grf(n, p=2, seed=0, sigma=1.5, ell=0.1):
    """-div(k grad u) = 1 on the unit square, n x n quads of order p, k = grf2d(n, sigma, ell, seed), u = 0 on the
    boundary (the learned-preconditioner workload)."""
    return darcy(2, n, p, grf2d(n, sigma, ell, seed))


def lognormal(ncells, sigma, seed):
    """Per-element coefficients exp(N(0, sigma^2)), i.i.d. from a seeded PCG64 stream."""
    return np.exp(sigma * np.random.default_rng(seed).standard_normal(ncells))
