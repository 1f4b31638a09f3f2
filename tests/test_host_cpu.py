"""CPU-only checks of the product's host side (no GPU needed).

* the host grid builder numbers equations exactly as the reference does (the
  oracle restates CreateMidSideConnect's neighbour search; the product uses
  grid entities);
* libgpz.so loads and exports every function include/gpz.h declares;
* without a GPU the library refuses to create a context (no CPU fallback).
"""
import os
import re

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def g():
    import __graft_entry__
    __graft_entry__.build()
    from neopz_gb300 import gpz
    return gpz


def _same_numbering(om, grid):
    assert om.neq == grid.neq
    assert om.ncel == grid.nel
    for e in range(om.ncel):
        assert np.array_equal(om.cel(e)["dest"], grid.dest(e)), e


def test_numbering_hp(g):
    """hp meshes (per-element orders, shared sides at the largest order): same equations per element."""
    E = np.exp(0.5 * np.random.default_rng(4).standard_normal(27))
    orders = g.hp_orders(27, 3)
    _same_numbering(O.elasticity3d_hp(3, orders, E=E), g.elasticity3d_hp(3, orders, E=E))
    o2 = g.hp_orders(36, 5)
    k = np.exp(np.random.default_rng(1).standard_normal(36))
    _same_numbering(O.darcy_hp(6, o2, k), g.darcy_hp(6, o2, k))


@pytest.mark.parametrize("n,p", [(4, 1), (6, 2), (5, 3)])
def test_numbering_2d(g, n, p):
    _same_numbering(O.poisson2d(n, p), g.poisson2d(n, p))


@pytest.mark.parametrize("n,p", [(2, 1), (3, 2), (2, 3)])
def test_numbering_3d_elasticity(g, n, p):
    _same_numbering(O.elasticity3d(n, p), g.elasticity3d(n, p))


def test_numbering_3d_darcy_all_faces(g):
    k = np.ones(27)
    _same_numbering(O.darcy(3, 3, 2, k), g.darcy(3, 3, 2, k))


def test_reference_counts_from_host_numbering(g):
    # equation counts the reference prints for the benchmark grids
    assert g.poisson2d(64, 2).neq == 16641
    assert g.elasticity3d(16, 2).neq == 107811
    assert g.elasticity3d(32, 2).neq == 823875


def test_library_exports_every_declared_symbol(g):
    import ctypes
    hdr = open(os.path.join(ROOT, "include", "gpz.h")).read()
    names = set(re.findall(r"\b(gpz_[a-z0-9_]+)\s*\(", hdr))
    assert len(names) >= 15
    L = ctypes.CDLL(g.LIBGPZ)
    for n in sorted(names):
        assert hasattr(L, n), n
    H = ctypes.CDLL(g.LIBHOST)
    hh = open(os.path.join(ROOT, "neopz_gb300", "host", "pz_grid.h")).read()
    for n in set(re.findall(r"\b(gpzh_[a-z0-9_]+)\s*\(", hh)):
        assert hasattr(H, n), n


def test_no_gpu_no_context(g):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    with pytest.raises(g.GpzError) as ei:
        g.Context(0)
    assert ei.value.code == -8  # GPZ_E_NO_DEVICE


def _replica_rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, _ = bench.dist_info()
    t = bench.max_over_ranks(1.0 + 0.5 * rank, w, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, t))


def test_replica_timing_takes_the_slowest_rank():
    """bench.py's N > 1 path (replicas, one system per rank, no data-path collective): the ranks read their
    place from the torchrun environment and the job's step time is the slowest rank's; world size 2 over gloo."""
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_replica_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 1.5), (1, 2, 1.5)]


def _profile(nodes_of_element, perm, nnodes):
    """Envelope of the connect graph under a numbering: sum over nodes of (number - smallest neighbour number)."""
    low = np.arange(nnodes)
    for nodes in nodes_of_element:
        p = perm[nodes]
        low[p] = np.minimum(low[p], p.min())
    return int(np.sum(np.arange(nnodes) - low))


@pytest.mark.parametrize("case", ["poisson2d_p1", "poisson2d_p3", "elast3d_p2", "elast3d_hp", "darcy3d_p2",
                                  "elast3d_p2_12"])
def test_sloan_matches_the_reference_algorithm(g, case):
    """gpz_sloan_resequence (segment-tree queue) gives exactly the permutation of the oracle's literal restatement
    of TPZSloanRenumbering::Resequence (a scan of the whole queue per node), on meshes whose element graphs come
    from the host grid builder (TPZCompMesh::ComputeElGraph: boundary elements included); the result does not
    depend on the order of the connects inside an element (ConvertGraph sorts)."""
    grid = {"poisson2d_p1": lambda: g.poisson2d(9, 1), "poisson2d_p3": lambda: g.poisson2d(5, 3),
            "elast3d_p2": lambda: g.elasticity3d(4, 2), "elast3d_hp": lambda: g.elasticity3d_hp(3, g.hp_orders(27, 3)),
            "darcy3d_p2": lambda: g.darcy(3, 3, 2, np.ones(27)), "elast3d_p2_12": lambda: g.elasticity3d(12, 2)}[case]()
    ei, eg = grid.element_graph()
    nn = grid.desc.nconnects
    pg, ps = g.sloan_resequence(nn, ei, eg)
    rc, og, osc = O.sloan(nn, ei, eg)
    assert rc == 0 and np.array_equal(pg, og) and np.array_equal(ps, osc)
    assert np.array_equal(np.sort(pg), np.arange(nn)) and np.array_equal(pg[ps], np.arange(nn))
    rng = np.random.default_rng(1)
    eg2 = eg.copy()
    for e in range(len(ei) - 1):
        rng.shuffle(eg2[ei[e]:ei[e + 1]])
    assert np.array_equal(g.sloan_resequence(nn, ei, eg2)[0], pg)


def test_sloan_reduces_the_profile_of_a_scrambled_numbering(g):
    """Numbered at random, a 3D Q2 mesh's connect graph has a large envelope; Sloan's numbering of the same graph
    (the labels permuted, so its input order carries no locality) takes it below a fifth of that and below the
    grid's creation order (8^3 hexes: 1.58M against 2.82M and 11.6M)."""
    grid = g.elasticity3d(8, 2)
    ei, eg = grid.element_graph()
    nn = grid.desc.nconnects
    scr = np.random.default_rng(3).permutation(nn)
    egs = scr[eg]
    elems = [egs[ei[e]:ei[e + 1]] for e in range(len(ei) - 1)]
    pg, _ = g.sloan_resequence(nn, ei, egs)
    p_random = _profile(elems, np.arange(nn), nn)
    p_sloan = _profile(elems, pg, nn)
    p_grid = _profile([eg[ei[e]:ei[e + 1]] for e in range(len(ei) - 1)], np.arange(nn), nn)
    assert p_sloan < 0.2 * p_random and p_sloan < p_grid, (p_sloan, p_grid, p_random)  # 1.58M, 2.82M, 11.6M


def test_sloan_rejects_bad_graphs(g):
    with pytest.raises(g.GpzError):
        g.sloan_resequence(4, np.array([0, 2, 4]), np.array([0, 1, 2, 4]))  # node index out of range
    with pytest.raises(g.GpzError):
        g.sloan_resequence(4, np.array([0, 2, 4]), np.array([0, 1, 2, 3]))  # two components
    assert O.sloan(4, np.array([0, 2, 4]), np.array([0, 1, 2, 3]))[0] == 1


def _blocks_of(grid):
    d = grid.desc
    nn = d.nconnects
    bp = np.ctypeslib.as_array(d.block_pos, shape=(nn,)).copy()
    bs = np.ctypeslib.as_array(d.block_size, shape=(nn,)).copy()
    return nn, bp, bs


@pytest.mark.parametrize("case", ["poisson2d_p1", "poisson2d_p3", "elast3d_p2", "elast3d_hp", "darcy3d_p2",
                                  "elast3d_p2_12"])
def test_nodeset_blocks_match_the_reference_algorithm(g, case):
    """gpz_nodeset_blocks (subset relations marked once per adjacency entry) gives exactly what the oracle's
    literal restatement of TPZNodesetCompute (std::set node sets, includes() per neighbour, recursion) gives:
    the blocks and their equations in order, the colours, every connect's sequence number and level.  The
    blocks cover every equation once (the connects' blocks are disjoint, so one colour), and the result does not
    depend on the order of the connects inside an element."""
    grid = {"poisson2d_p1": lambda: g.poisson2d(9, 1), "poisson2d_p3": lambda: g.poisson2d(5, 3),
            "elast3d_p2": lambda: g.elasticity3d(4, 2), "elast3d_hp": lambda: g.elasticity3d_hp(3, g.hp_orders(27, 3)),
            "darcy3d_p2": lambda: g.darcy(3, 3, 2, np.ones(27)), "elast3d_p2_12": lambda: g.elasticity3d(12, 2)}[case]()
    ei, eg = grid.element_graph()
    nn, bp, bs = _blocks_of(grid)
    r = g.nodeset_blocks(nn, ei, eg, bp, bs, grid.neq)
    rc, o = O.nodeset(nn, ei, eg, bp, bs, grid.neq)
    assert rc == 0
    for k in ("blockindex", "blockeqs", "colors", "seqnum", "level"):
        assert np.array_equal(r[k], o[k]), k
    assert r["ncolors"] == o["ncolors"] == 1
    assert np.array_equal(np.sort(r["blockeqs"]), np.arange(grid.neq))
    rng = np.random.default_rng(2)
    eg2 = eg.copy()
    for e in range(len(ei) - 1):
        rng.shuffle(eg2[ei[e]:ei[e + 1]])
    r2 = g.nodeset_blocks(nn, ei, eg2, bp, bs, grid.neq)
    assert np.array_equal(r2["blockeqs"], r["blockeqs"]) and np.array_equal(r2["blockindex"], r["blockindex"])


@pytest.mark.parametrize("kind,n", [("elast3d", 4), ("elast3d", 8), ("elast3d", 16), ("darcy3d", 5),
                                    ("poisson2d", 3), ("poisson2d", 9)])
def test_nodeset_blocks_of_q2_grids(g, kind, n):
    """Known structure on n^d Q2 grids (nstate equations per connect): a connect's node set is the union of the
    elements around it, so two connects share a block only when every element of one is an element of the
    other and back.  Away from the outer layer of elements no two connects have the same set (m^d one-connect
    blocks, m = 2n - 3); in the outer layer a boundary connect merges with the connects of the one, two or four
    elements it touches.  3D: 6 m^2 blocks of 2 connects, 12 m of 4 and 8 corner blocks of 8 (the corner
    vertex, three edges, three faces and the interior of a corner element); 2D: 4 m of 2 and 4 of 4."""
    grid = {"elast3d": lambda: g.elasticity3d(n, 2), "darcy3d": lambda: g.darcy(3, n, 2, np.ones(n ** 3)),
            "poisson2d": lambda: g.poisson2d(n, 2)}[kind]()
    ns = 3 if kind == "elast3d" else 1
    ei, eg = grid.element_graph()
    nn, bp, bs = _blocks_of(grid)
    r = g.nodeset_blocks(nn, ei, eg, bp, bs, grid.neq)
    sizes, counts = np.unique(np.diff(r["blockindex"]), return_counts=True)
    m = 2 * n - 3
    want = {1: m ** 3, 2: 6 * m ** 2, 4: 12 * m, 8: 8} if kind != "poisson2d" else {1: m ** 2, 2: 4 * m, 4: 4}
    assert dict(zip(sizes.tolist(), counts.tolist())) == {ns * k: v for k, v in want.items()}
    assert r["level"].max() == (2 if kind == "poisson2d" else 3)


def test_nodeset_block_preconditioner_in_the_oracle(g):
    """The preconditioner these blocks make (LU solves of the matrix's diagonal blocks over the node sets, the
    step solver BuildSequenceSolver returns for one colour), in the oracle's CG on 6^3 Q2 elasticity with
    lognormal E: the same solution as Jacobi-PCG and fewer iterations than point Jacobi or the 3x3 connect
    blocks (389 against 545 and 427 at 1e-10)."""
    n = 6
    E = g.lognormal(n ** 3, 1.0, 5)
    grid = g.elasticity3d(n, 2, E=E)
    om = O.elasticity3d(n, 2, E=E)
    ei, eg = grid.element_graph()
    nn, bp, bs = _blocks_of(grid)
    r = g.nodeset_blocks(nn, ei, eg, bp, bs, grid.neq)
    ia, ja = om.pattern(True)
    a, f = om.assemble(True, ia, ja)
    ref = O.cg_jacobi(True, ia, ja, a, f, 20000, 1e-10)
    cb = O.cg_block_jacobi(True, ia, ja, a, f, 3, 20000, 1e-10)
    ns = O.cg_sparse_block_jacobi(True, ia, ja, a, f, r["blockindex"], r["blockeqs"], 20000, 1e-10)
    assert ref["rc"] == cb["rc"] == ns["rc"] == 0
    assert np.linalg.norm(ns["x"] - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    assert ns["iters"] < cb["iters"] < ref["iters"], (ns["iters"], cb["iters"], ref["iters"])
    # the same routine over the 3x3 connect blocks reproduces the dedicated connect-block CG
    cs = O.cg_sparse_block_jacobi(True, ia, ja, a, f, np.arange(0, grid.neq + 1, 3), np.arange(grid.neq), 20000,
                                  1e-10)
    assert abs(cs["iters"] - cb["iters"]) <= 3 and np.linalg.norm(cs["x"] - cb["x"]) <= 1e-8 * np.linalg.norm(cb["x"])


def test_nodeset_rejects_bad_input(g):
    ei, eg = np.array([0, 2, 4]), np.array([0, 1, 1, 2])
    ones = np.ones(3, np.int64)
    with pytest.raises(g.GpzError):
        g.nodeset_blocks(3, ei, np.array([0, 1, 1, 3]), np.arange(3), ones, 3)  # connect index out of range
    with pytest.raises(g.GpzError):
        g.nodeset_blocks(3, ei, eg, np.array([0, 1, 3]), ones, 3)  # a block past the last equation
    r = g.nodeset_blocks(3, ei, eg, np.arange(3), ones, 3)
    # 0 and 2 are proper subsets of 1's set {0, 1, 2}: numbered first, at level 0; 1 at level 1
    assert np.array_equal(r["seqnum"], [0, 2, 1]) and np.array_equal(r["level"], [0, 1, 0])
    assert np.array_equal(r["blockindex"], [0, 1, 2, 3]) and np.array_equal(r["blockeqs"], [0, 2, 1])
    e = g.nodeset_blocks(0, np.array([0]), np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros(0, np.int64), 0)
    assert e["ncolors"] == 1 and len(e["blockindex"]) == 1


def test_hp_block_jacobi_variants_in_the_oracle(g):
    """On an hp mesh (4^3 hexes, p in {1,2,3}) the reference's connect blocks (TPZBlockDiagonalStructMatrix: one
    block of nshape x 3 equations per connect, 3 to 24 here; what GPZ_PRECOND_BLOCK_JACOBI applies in the device
    CG) and the per-shape 3x3 blocks (the device GMRES's split of a larger connect block) give the same solution
    and CG iteration counts within 5% (264 and 271 to 1e-8); the node-set blocks of overlap = false need
    markedly fewer (189)."""
    n = 4
    orders = g.hp_orders(n ** 3, 3)
    E = g.lognormal(n ** 3, 0.5, 3)
    grid = g.elasticity3d_hp(n, orders, E=E)
    om = O.elasticity3d_hp(n, orders, E=E)
    nn, bp, bs = _blocks_of(grid)
    keep = bs > 0
    assert bs[keep].max() == 24
    bi = np.concatenate([[0], np.cumsum(bs[keep])]).astype(np.int64)
    be = np.concatenate([np.arange(p, p + s) for p, s in zip(bp[keep], bs[keep])]).astype(np.int64)
    ia, ja = om.pattern(True)
    a, f = om.assemble(True, ia, ja)
    shape3 = O.cg_block_jacobi(True, ia, ja, a, f, 3, 20000, 1e-8)
    conn = O.cg_sparse_block_jacobi(True, ia, ja, a, f, bi, be, 20000, 1e-8)
    ei, eg = grid.element_graph()
    r = g.nodeset_blocks(nn, ei, eg, bp, bs, grid.neq)
    ns = O.cg_sparse_block_jacobi(True, ia, ja, a, f, r["blockindex"], r["blockeqs"], 20000, 1e-8)
    assert shape3["rc"] == conn["rc"] == ns["rc"] == 0
    assert abs(conn["iters"] - shape3["iters"]) <= 0.05 * conn["iters"], (conn["iters"], shape3["iters"])
    assert ns["iters"] < 0.85 * conn["iters"], (ns["iters"], conn["iters"])
    for s in (shape3, ns):
        assert np.linalg.norm(s["x"] - conn["x"]) <= 1e-6 * np.linalg.norm(conn["x"])


def test_cxx_program_uses_the_c_abi(g, tmp_path):
    """A C++ translation unit that includes only include/gpz.h compiles with g++, links libgpz.so and runs: the
    host-only entry points give the node-set blocks and the Sloan order of a three-connect chain, and a context
    is refused with GPZ_E_NO_DEVICE when no GPU is visible (no CPU fallback behind the ABI)."""
    import subprocess
    import torch
    build = os.path.join(ROOT, "neopz_gb300", "_build")
    exe = str(tmp_path / "abi_consumer")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_consumer.cpp"), "-L" + build, "-lgpz", "-Wl,-rpath," + build,
                    "-o", exe], check=True)
    out = subprocess.run([exe], check=True, stdout=subprocess.PIPE, text=True).stdout.splitlines()
    assert out[0] == "nodeset 0 3 1 0 2 1"
    assert out[1].startswith("sloan 0 ") and sorted(map(int, out[1].split()[2:])) == [0, 1, 2]
    assert out[2] == ("context 0" if torch.cuda.is_available() else "context -8")  # -8: GPZ_E_NO_DEVICE


@pytest.mark.parametrize("case", ["poisson2d_q2", "elast3d_q2", "elast3d_hp", "darcy2d_q3"])
def test_element_colouring_invariant(g, case):
    """The colouring of the atomic-free scatter (gpz_element_colours, what gpz_mesh_upload colours the buckets
    with): no two elements of one colour share a non-empty connect -- so one colour's elements write disjoint
    rows and CSR slots -- and every colour below the count is used.  A uniform grid needs the 2^d colours of its
    cell parities (4 for quads, 8 for hexes, boundary elements included)."""
    if case == "poisson2d_q2":
        grid, want = g.poisson2d(12, 2), 4
    elif case == "elast3d_q2":
        grid, want = g.elasticity3d(6, 2), 8
    elif case == "elast3d_hp":
        grid, want = g.elasticity3d_hp(5, g.hp_orders(125, 3)), 8
    else:
        grid, want = g.darcy(2, 9, 3, g.lognormal(81, 1.0, 2)), 4
    ei, eg = grid.element_graph()
    nn, bp, bs = _blocks_of(grid)
    col, nc = g.element_colours(ei, eg, bs)
    assert nc == want and set(col.tolist()) == set(range(nc))
    owner = {}
    for e in range(len(ei) - 1):
        for cn in eg[ei[e]:ei[e + 1]]:
            if bs[cn] == 0:
                continue
            key = (int(cn), int(col[e]))
            assert key not in owner, f"elements {owner.get(key)} and {e} share connect {cn} in colour {col[e]}"
            owner[key] = e
    with pytest.raises(g.GpzError):
        g.element_colours(ei, np.where(eg == eg[0], nn, eg), bs)  # a connect out of range
