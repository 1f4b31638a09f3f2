"""The NeoPZ-side binding (neopz_gb300/neopz_binding/gpz_neopz.h) compiled
against the reference library's own headers and linked with it, run on the
workloads of the reference-side fixtures (tests/binding_check.cpp):

* gpz_neopz::ExtractMesh of the reference's TPZCompMesh gives, field by field,
  the descriptor of the host grid builder for the same workload, the one the
  GPU fixture tests hold to the reference's pattern, values and solutions
  (so a NeoPZ program hands the device exactly that system);
* TPZLinearAnalysis with TPZSSpStructMatrixGPU and a CG TPZStepSolver stops
  through DebugStop at the first device call when no GPU is visible (no CPU
  fallback); with a GPU, the device system and CG solution are held to the
  reference's serial TPZSSpStructMatrix assembly and CG (1e-12 on values,
  1e-8 on the solution).

Needs the reference sources (the binding includes their headers) and the
reference library build (oracle/ref_build.mk); skipped where either is absent.
"""
import json
import os
import subprocess

import numpy as np
import pytest

import refcases as RC

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("NEOPZ_REFERENCE", "/root/reference")
MK = os.path.join(ROOT, "oracle", "ref_build.mk")
EXE = os.path.join(ROOT, "oracle", "_ref", "binding_check")


@pytest.fixture(scope="module")
def binding_check():
    if not os.path.isdir(os.path.join(REF, "StrMatrix")):
        pytest.skip("reference sources absent")
    if not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libpzref.so")):
        pytest.skip("reference library not built (make -f oracle/ref_build.mk)")
    import __graft_entry__
    __graft_entry__.build()
    subprocess.run(["make", "-s", "-f", MK, f"REF={REF}", "binding"], check=True, cwd=ROOT)
    return EXE


CASES = [("poisson2d", 4, 2, None, None), ("darcy2d", 5, 2, "coef", None), ("darcy3d", 3, 2, None, None),
         ("elast3d", 2, 2, None, None), ("elast3d_c5", 3, 2, "coef", None), ("elast3d_hp", 3, 1, "coef", "orders")]


@pytest.mark.parametrize("case,n,p,coef,orders", CASES)
def test_binding_extracts_the_device_mesh_and_drives_the_analysis(binding_check, tmp_path, case, n, p, coef,
                                                                 orders):
    rng = np.random.default_rng(7)
    ncell = n ** 3 if case in ("darcy3d", "elast3d", "elast3d_c5", "elast3d_hp") else n ** 2
    args = [binding_check, case, str(n), str(p)]
    if coef:
        np.exp(rng.standard_normal(ncell)).astype(np.float64).tofile(tmp_path / "coef.bin")
        args.append(str(tmp_path / "coef.bin"))
    elif orders:
        args.append("-")
    if orders:
        rng.integers(1, 4, ncell).astype(np.int32).tofile(tmp_path / "orders.bin")
        args.append(str(tmp_path / "orders.bin"))
    out = subprocess.run(args, capture_output=True, text=True)
    line = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert line, out.stdout[-2000:] + out.stderr[-2000:]
    r = json.loads(line[-1])
    assert r["mismatches"] == [], r
    assert out.returncode == 0, r
    if r["ctx_create"] == -8:  # GPZ_E_NO_DEVICE: the analysis stopped at the first device call
        assert r["stopped"] is True
    else:
        assert r["mat_err"] <= 1e-12 and r["rhs_err"] <= 1e-12 and r["sol_err"] <= 1e-8, r


def test_binding_on_a_fixture_workload(binding_check, tmp_path):
    """The 2D Darcy fixture's own permeability field (tests/golden/ref_c4_darcy2d_grf_32_q2.npz)."""
    fx = RC.load("c4_darcy2d_grf_32_q2")
    np.ascontiguousarray(fx["coef"], np.float64).tofile(tmp_path / "coef.bin")
    out = subprocess.run([binding_check, "darcy2d", str(int(fx["n"])), str(int(fx["p"])), str(tmp_path / "coef.bin")],
                         capture_output=True, text=True)
    r = json.loads([ln for ln in out.stdout.splitlines() if ln.startswith("{")][-1])
    assert r["mismatches"] == [] and out.returncode == 0, r
    assert r["neq"] == int(fx["neq"])
