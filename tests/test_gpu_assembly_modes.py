"""The two launch modes of the element kernels (gpz_assembly_mode): a launch per
bucket and colour, and one persistent launch per bucket whose resident CTAs take
elements from a work counter in colour order, waiting (bounded) for the earlier
colours -- the device form of TPZStructMatrixOT's colour scheduler.

Both give the oracle's matrix and load vector (values within 1e-12 of each
row's largest entry) and agree with each other to 1e-14 (the contributions of
different buckets to one entry are added in another order); with mode -1 both
are timed and the choice reported; a graph replay in the persistent mode gives
the same values.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import __graft_entry__
    __graft_entry__.build()
    from neopz_gb300 import gpz
    return gpz


def _row_rel(ia, a, ref):
    worst = 0.0
    for r in range(len(ia) - 1):
        s, e = ia[r], ia[r + 1]
        m = np.max(np.abs(ref[s:e]))
        if m > 0:
            worst = max(worst, np.max(np.abs(a[s:e] - ref[s:e])) / m)
    return worst


def _cases(g):
    rng = np.random.default_rng(11)
    E = np.exp(rng.standard_normal(27))
    o = g.hp_orders(27, 4)
    k = np.exp(rng.standard_normal(36))
    return [(O.elasticity3d(3, 2, E=E), g.elasticity3d(3, 2, E=E)),
            (O.elasticity3d_hp(3, o, E=E), g.elasticity3d_hp(3, o, E=E)),
            (O.darcy(2, 6, 2, k), g.darcy(2, 6, 2, k))]


@pytest.mark.parametrize("which", [0, 1, 2])
def test_persistent_and_per_colour_launches_agree(g, which):
    om, grid = _cases(g)[which]
    oia, oja = om.pattern(False)
    oa, of = om.assemble(False, oia, oja)
    out = []
    for mode in (0, 1):
        ctx = g.Context(0)
        ctx.assembly_mode(mode)
        ctx.upload_mesh(grid)
        ctx.build_pattern(False)
        ctx.assemble(g.GPZ_PREC_FP64)
        ctx.assemble(g.GPZ_PREC_FP64)  # the captured graph replayed
        a, f = ctx.matrix(), ctx.rhs()
        assert _row_rel(oia, a, oa) <= 1e-12
        assert np.max(np.abs(f - of)) <= 1e-12 * np.max(np.abs(of))
        out.append((a, f))
        ctx.close()
    (a0, f0), (a1, f1) = out
    assert _row_rel(oia, a1, a0) <= 1e-14 and np.max(np.abs(f1 - f0)) <= 1e-14 * np.max(np.abs(f0))


def test_launch_mode_is_autotuned(g):
    grid = g.elasticity3d_hp(4, g.hp_orders(64, 7))
    ctx = g.Context(0)
    ctx.assembly_mode(-1)
    ctx.upload_mesh(grid)
    ctx.build_pattern(True)
    ctx.assemble(g.GPZ_PREC_FP64)
    rep = ctx.assembly_report()["launch_mode_ms"]
    assert rep["chosen"] in ("per_colour", "persistent")
    assert rep["per_colour"] > 0 and rep["persistent"] > 0
    ctx.close()
