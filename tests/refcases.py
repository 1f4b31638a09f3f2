"""The reference-written fixtures (tests/golden/ref_*.npz, made by
tests/golden/make_ref_fixtures.py from the NeoPZ library itself) and the
matching problems of the oracle and of the GPU library.

Checks shared by the oracle test (CPU) and the GPU test:
* pattern: SHA-256 of the row pointers and columns (int64) equal to the
  reference's -- bit-exact;
* values: per row |(A v)_i - (A v)_ref,i| <= 1e-12 (|A| |v|)_ref,i for the
  seeded probe v (every stored value enters at its row's scale), the diagonal
  within 1e-12 relative, and where the fixture holds them all values within
  1e-12 of their row's largest;
* load vector within 1e-12 of its largest entry.
"""
import glob
import hashlib
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(GOLDEN, "ref_*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, "ref_" + name + ".npz"))
    return {k: z[k] for k in z.files}


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i8").tobytes()).hexdigest()


def problem(mod, fx):
    """The workload of fixture fx built by `mod` (oracle.oracle or neopz_gb300.gpz)."""
    case, n, p = str(fx["case"]), int(fx["n"]), int(fx["p"])
    coef = fx.get("coef")
    if case == "poisson2d":
        return mod.poisson2d(n, p)
    if case == "darcy2d":
        return mod.darcy(2, n, p, coef)
    if case == "darcy3d":
        return mod.darcy(3, n, p, coef)
    if case == "elast3d_hp":
        return mod.elasticity3d_hp(n, fx["orders"], E=coef)
    if case == "elast3d_c5":
        return mod.elasticity3d(n, p, E=coef, body_force=(0.0, 0.0, 0.0))
    raise ValueError(case)


def full_product(sym, ia, ja, a, v):
    rows = np.repeat(np.arange(len(ia) - 1), np.diff(ia))
    y = np.zeros(len(ia) - 1)
    np.add.at(y, rows, a * v[ja])
    if sym:
        off = rows != ja
        np.add.at(y, ja[off], a[off] * v[rows[off]])
    return y


def check_system(fx, ia, ja, a, f):
    """Assert the pattern, values and load vector of a system against fixture fx."""
    sym = int(fx["sym"])
    assert len(ia) - 1 == int(fx["neq"]) and len(ja) == int(fx["nnz"])
    assert sha(ia) == str(fx["ia_sha256"]), "row pointers differ from the reference"
    assert sha(ja) == str(fx["ja_sha256"]), "columns differ from the reference"
    ia, ja = np.asarray(ia, np.int64), np.asarray(ja, np.int64)
    v = np.random.default_rng(int(fx["av_seed"])).standard_normal(len(ia) - 1)
    av = full_product(sym, ia, ja, a, v)
    scale = fx["absav"] if "absav" in fx else full_product(sym, ia, ja, np.abs(a), np.abs(v))
    bad = np.abs(av - fx["av"]) > 1e-12 * scale + 1e-300
    assert not bad.any(), f"A v differs from the reference in {int(bad.sum())} rows"
    if "diag" in fx:
        rows = np.repeat(np.arange(len(ia) - 1), np.diff(ia))
        d = np.zeros(len(ia) - 1)
        d[rows[rows == ja]] = a[rows == ja]
        assert np.all(np.abs(d - fx["diag"]) <= 1e-12 * np.abs(fx["diag"]))
    if "a" in fx:
        ref = fx["a"]
        for r in range(len(ia) - 1):
            s, e = ia[r], ia[r + 1]
            assert np.max(np.abs(a[s:e] - ref[s:e])) <= 1e-12 * np.max(np.abs(ref[s:e]))
    assert np.max(np.abs(f - fx["f"])) <= 1e-12 * np.max(np.abs(fx["f"]))


def rel_err(x, fx):
    return float(np.linalg.norm(x - fx["x"]) / np.linalg.norm(fx["x"]))
