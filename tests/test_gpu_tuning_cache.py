"""The on-disk cache of the autotuners' choices (gpz_tuning_cache).

* FP32 operator of the mixed CG (3D Q2 elasticity): the first context measures
  every candidate and appends its choice to the file; a second context on the
  same mesh takes the stored choice without timing ("cached": true), and its
  mixed solve takes the same path (iterations within 3, solution within 1e-7);
  a different mesh gets its own key and is measured.
* hp element kernels: the block size measured by the first assembly is stored
  and reused the same way; the matrices are identical (one CTA per element,
  fixed summation order, whatever the block size).
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import __graft_entry__
    __graft_entry__.build()
    from neopz_gb300 import gpz
    return gpz


def _ctx(g, grid, path):
    ctx = g.Context(0)
    ctx.tuning_cache(path)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    return ctx


def test_operator_choice_is_cached(g, tmp_path):
    path = tmp_path / "tune.jsonl"
    grid = g.elasticity3d(6, 2, E=np.exp(np.random.default_rng(3).standard_normal(216)))
    a = _ctx(g, grid, path)
    a.assemble(g.GPZ_PREC_MIXED)
    ra = a.tuning_report()
    assert not ra.get("cached") and ra["chosen"]
    kw = dict(solver=g.GPZ_SOLVER_MIXED_CG, precond=g.GPZ_PRECOND_BLOCK_JACOBI, tol=1e-8, reliable_delta=1e-2)
    sa = a.solve(**kw)
    lines = [json.loads(x) for x in open(path)]
    assert len(lines) == 1 and lines[0]["key"].startswith("spmv32|") and lines[0]["report"]["chosen"] == ra["chosen"]
    b = _ctx(g, grid, path)
    b.assemble(g.GPZ_PREC_MIXED)
    rb = b.tuning_report()
    assert rb["cached"] is True and rb["chosen"] == ra["chosen"]
    sb = b.solve(**kw)
    # the operator's float4 reductions make the summation order run-dependent: same method, not the same bits
    assert abs(sb["iterations"] - sa["iterations"]) <= 3
    assert np.linalg.norm(sb["x"] - sa["x"]) <= 1e-7 * np.linalg.norm(sa["x"])
    assert len(open(path).readlines()) == 1  # a hit appends nothing
    other = _ctx(g, g.elasticity3d(5, 2), path)
    other.assemble(g.GPZ_PREC_MIXED)
    assert not other.tuning_report().get("cached")
    assert len(open(path).readlines()) == 2
    for c in (a, b, other):
        c.close()


def test_hp_block_size_is_cached(g, tmp_path):
    path = tmp_path / "tune.jsonl"
    grid = g.elasticity3d_hp(3, g.hp_orders(27, 3))
    a = _ctx(g, grid, path)
    a.assemble(g.GPZ_PREC_FP64)
    ra = a.assembly_report()
    b = _ctx(g, grid, path)
    b.assemble(g.GPZ_PREC_FP64)
    rb = b.assembly_report()
    ta, tb = ra["hp_block_size_ms"], rb["hp_block_size_ms"]
    assert not ta.get("cached") and tb["cached"] is True and tb["chosen"] == ta["chosen"]
    assert np.array_equal(a.matrix(), b.matrix()) and np.array_equal(a.rhs(), b.rhs())
    a.close()
    b.close()
