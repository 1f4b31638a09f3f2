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
