"""The oracle against fixtures the NeoPZ reference library itself wrote
(tests/golden/ref_*.npz; see tests/refcases.py for what they hold and the
tolerances).  Pins the oracle's pattern, values, load vectors and CG to the
reference: CSR bit-exact (upper and full), values and loads within 1e-12,
the Jacobi-PCG solution within 1e-10 of the reference's tight solve and its
iteration count within max(3, 10%) of the reference's."""
import numpy as np
import pytest

import refcases as RC
from oracle import oracle as O

CG_MAX_NNZ = 3_000_000  # the oracle's serial CG on the larger fixtures would take minutes


@pytest.fixture(scope="module", autouse=True)
def built():
    O.build()


@pytest.mark.parametrize("name", RC.names())
def test_oracle_matches_reference_fixture(name):
    fx = RC.load(name)
    sym = bool(int(fx["sym"]))
    m = RC.problem(O, fx)
    ia, ja = m.pattern(sym)
    a, f = m.assemble(sym, ia, ja, nthreads=4)
    RC.check_system(fx, ia, ja, a, f)
    if "x" not in fx or len(ja) > CG_MAX_NNZ:
        return
    cfg = O.cg_jacobi(sym, ia, ja, a, f, 200000, float(fx["tol"]), jacobi_residual=True)
    ref_it = int(fx["cg_iterations"])
    assert abs(cfg["iters"] - ref_it) <= max(3, 0.1 * ref_it), (cfg["iters"], ref_it)
    tight = O.cg_jacobi(sym, ia, ja, a, f, 200000, float(fx["tight_tol"]))
    assert RC.rel_err(tight["x"], fx) <= 1e-10
