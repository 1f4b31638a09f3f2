"""Write tests/golden/ref_*.npz: fixtures produced by the NeoPZ reference library itself.

Builds the reference library and the fixture harness (oracle/ref_build.mk,
oracle/ref_harness.cpp), runs the harness on small instances of the five
workloads (and the 2D Poisson workload at its full 64 x 64 size), and keeps,
per instance:

* ``ia_sha256`` / ``ja_sha256``: SHA-256 of the reference's CSR row pointers
  and columns as little-endian int64 (TPZSSpStructMatrix upper or
  TPZSpStructMatrix full pattern): a bit-exact pattern check in 64 bytes;
* ``diag``: the matrix diagonal; ``av`` and ``absav``: A v and |A| |v| for a
  seeded vector v (the symmetric product for the upper pattern), which pin
  every stored value to the row's scale; ``a``: the values themselves for the
  small patterns;
* ``f``: the load vector;
* ``cg_iterations`` / ``cg_resid``: the reference's TPZStepSolver CG with
  Jacobi (SetJacobi(1, 0, 0)) to the workload's tolerance;
* ``x``: the reference's solution of the same CG to ``tight_tol`` (the FP64
  solution the GPU paths are measured against).

The inputs (per-cell coefficients, orders) come from the same seeded
generators the tests and the benchmark use (neopz_gb300.gpz).

Usage:  python tests/golden/make_ref_fixtures.py REFERENCE_ROOT   (the NeoPZ source tree; required)
The fixtures are committed; the tests never read the reference tree.
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

AV_SEED = 20241204
STORE_A_MAX_NNZ = 200000


def cases():
    from neopz_gb300 import gpz
    return [
        dict(name="c1_poisson2d_64_q2", case="poisson2d", n=64, p=2, sym=1, tol=1e-10, tight_tol=1e-13),
        dict(name="c1_poisson2d_64_q2_full", case="poisson2d", n=64, p=2, sym=0, tol=0.0),
        dict(name="c2_darcy3d_8_q2", case="darcy3d", n=8, p=2, sym=1, tol=1e-8, tight_tol=1e-13,
             coef=gpz.lognormal(8 ** 3, 1.0, 1)),
        dict(name="c3_elast3d_hp_6", case="elast3d_hp", n=6, p=1, sym=1, tol=1e-8, tight_tol=1e-13,
             coef=gpz.lognormal(6 ** 3, 0.5, 3), orders=gpz.hp_orders(6 ** 3, 3)),
        dict(name="c4_darcy2d_grf_32_q2", case="darcy2d", n=32, p=2, sym=1, tol=1e-8, tight_tol=1e-13,
             coef=gpz.grf2d(32, seed=10000)),
        dict(name="c5_elast3d_8_q2", case="elast3d_c5", n=8, p=2, sym=1, tol=1e-8, tight_tol=1e-13,
             coef=gpz.lognormal(8 ** 3, 1.0, 5)),
        dict(name="c5_elast3d_8_q2_full", case="elast3d_c5", n=8, p=2, sym=0, tol=0.0,
             coef=gpz.lognormal(8 ** 3, 1.0, 5)),
        dict(name="c5_elast3d_16_q2", case="elast3d_c5", n=16, p=2, sym=1, tol=1e-8, tight_tol=1e-13,
             coef=gpz.lognormal(16 ** 3, 1.0, 5), lean=True),
    ]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i8").tobytes()).hexdigest()


def full_product(sym, ia, ja, a, v):
    """A v for the stored pattern: the upper triangle expanded symmetrically when sym."""
    rows = np.repeat(np.arange(len(ia) - 1), np.diff(ia))
    y = np.zeros(len(ia) - 1)
    np.add.at(y, rows, a * v[ja])
    if sym:
        off = rows != ja
        np.add.at(y, ja[off], a[off] * v[rows[off]])
    return y


def run_harness(harness, c, tol, d):
    args = [harness, c["case"], str(c["n"]), str(c["p"]), str(c["sym"]), repr(tol), d]
    if "coef" in c:
        np.ascontiguousarray(c["coef"], np.float64).tofile(os.path.join(d, "coef.bin"))
        args.append(os.path.join(d, "coef.bin"))
    elif "orders" in c:
        args.append("-")
    if "orders" in c:
        np.ascontiguousarray(c["orders"], np.int32).tofile(os.path.join(d, "orders.bin"))
        args.append(os.path.join(d, "orders.bin"))
    subprocess.run(args, check=True, stdout=subprocess.DEVNULL)
    info = json.load(open(os.path.join(d, "info.json")))
    out = dict(info=info, ia=np.fromfile(os.path.join(d, "ia.bin"), np.int64),
               ja=np.fromfile(os.path.join(d, "ja.bin"), np.int64), a=np.fromfile(os.path.join(d, "a.bin")),
               f=np.fromfile(os.path.join(d, "f.bin")))
    if os.path.exists(os.path.join(d, "x.bin")):
        out["x"] = np.fromfile(os.path.join(d, "x.bin"))
    return out


def main(ref_root):
    subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "ref_build.mk"), "REF=" + ref_root,
                    "-j%d" % (os.cpu_count() or 4)], check=True, cwd=ROOT)
    harness = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
    for c in cases():
        with tempfile.TemporaryDirectory() as d:
            r = run_harness(harness, c, c["tol"], d)
            ia, ja, a = r["ia"], r["ja"], r["a"]
            neq = len(ia) - 1
            v = np.random.default_rng(AV_SEED).standard_normal(neq)
            rows = np.repeat(np.arange(neq), np.diff(ia))
            diag = np.zeros(neq)
            diag[rows[rows == ja]] = a[rows == ja]
            fx = dict(case=c["case"], n=c["n"], p=c["p"], sym=c["sym"], neq=neq, nnz=len(ja),
                      ia_sha256=sha(ia), ja_sha256=sha(ja), av_seed=AV_SEED,
                      av=full_product(c["sym"], ia, ja, a, v), f=r["f"])
            if not c.get("lean"):
                fx.update(diag=diag, absav=full_product(c["sym"], ia, ja, np.abs(a), np.abs(v)))
            if len(ja) <= STORE_A_MAX_NNZ:
                fx["a"] = a
            if "coef" in c:
                fx["coef"] = np.asarray(c["coef"], np.float64)
            if "orders" in c:
                fx["orders"] = np.asarray(c["orders"], np.int32)
            if c["tol"] > 0:
                fx.update(tol=c["tol"], cg_iterations=r["info"]["cg_iterations"], cg_resid=r["info"]["cg_resid"])
                t = run_harness(harness, c, c["tight_tol"], d)
                fx.update(tight_tol=c["tight_tol"], x=t["x"], tight_iterations=t["info"]["cg_iterations"],
                          tight_resid=t["info"]["cg_resid"])
        path = os.path.join(HERE, "ref_" + c["name"] + ".npz")
        np.savez_compressed(path, **fx)
        print(f"{c['name']}: neq {neq} nnz {len(ja)} cg {fx.get('cg_iterations')} -> {os.path.basename(path)} "
              f"({os.path.getsize(path) / 1e3:.0f} kB)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_ref_fixtures.py <path of the NeoPZ source tree>")
    main(sys.argv[1])
