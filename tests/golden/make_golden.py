"""Regenerate tests/golden/reference_unit_golden.json from the reference's own unit tests.

Reads, as text, the known answers that NeoPZ's Catch2 tests hold for this path:

* UnitTest_PZ/TestMaterial/CubeStiffMatrix.txt, read by
  UnitTest_PZ/TestMaterial/TestMaterial.cpp:42-58 (TPZElasticity3D::Contribute,
  E=1000, nu=0.2, weight 8, identity gradients; margin 0.01 at :80);
* the master-quad TPZDarcyFlow matrix of
  UnitTest_PZ/TestMaterial/TestDarcyFlow.cpp:94-99 (margin 1e-5 at :105);
* the 1D "Assemble known matrix" answer of
  UnitTest_PZ/TestStruct/StructMatrixUnitTest.cpp:183-213 (20 line elements,
  TPZMatTest ek = [[2,1],[1,2]] at :345-351).

It also records equation, nonzero and CG-iteration counts that the reference
library itself printed for the synthetic grids of the benchmark (a run of the
reference's TPZSSpStructMatrix / TPZSpStructMatrix + TPZStepSolver CG with
Jacobi on the configurations below).

Usage:  python tests/golden/make_golden.py REFERENCE_ROOT   (the NeoPZ source tree; required)
The fixture is committed; the tests never read the reference tree.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    out = {}
    with open(os.path.join(ref, "UnitTest_PZ/TestMaterial/CubeStiffMatrix.txt")) as f:
        lines = f.read().split("\n")[1:]
    vals = [float(v) for v in " ".join(lines).split()]
    assert len(vals) == 81
    out["cube_elasticity_9x9"] = dict(
        source="UnitTest_PZ/TestMaterial/CubeStiffMatrix.txt (TestMaterial.cpp:18-86)",
        E=1000.0, nu=0.2, weight=8.0, margin=0.01, matrix=[vals[i * 9:(i + 1) * 9] for i in range(9)])

    src = open(os.path.join(ref, "UnitTest_PZ/TestMaterial/TestDarcyFlow.cpp")).read()
    m = re.search(r"TEST_CASE\(\"test_matriz_darcy\".*?RightStiff\[4\]\[4\]\s*=\s*\{(.*?)\};", src, re.S)
    rows = re.findall(r"\{([^{}]*)\}", m.group(1))
    mat = []
    for r in rows:
        entries = []
        for x in r.split(","):
            x = x.strip()
            num, den = x.split("/")
            entries.append(float(num.rstrip(".")) / float(den.rstrip(".")))
        mat.append(entries)
    out["darcy_master_quad_4x4"] = dict(
        source="UnitTest_PZ/TestMaterial/TestDarcyFlow.cpp:21-46,86-108",
        order=1, ids=[0, 1, 2, 3], intrule_order=2, perm=1.0, margin=1e-5, matrix=mat)

    st = open(os.path.join(ref, "UnitTest_PZ/TestStruct/StructMatrixUnitTest.cpp")).read()
    nel = int(re.search(r"constexpr int nEl\{(\d+)\}", st).group(1))
    assert "ek.PutVal(0,0,2)" in st and "ek.PutVal(0,1,1)" in st
    out["known_matrix_1d"] = dict(
        source="UnitTest_PZ/TestStruct/StructMatrixUnitTest.cpp:61-104,183-213,333-381",
        n_el=nel, order=1, mock_ek=[[2.0, 1.0], [1.0, 2.0]], diag_end=2.0, diag_mid=4.0, offdiag=1.0)

    out["reference_run_counts"] = dict(
        note="printed by the reference library (TPZSSpStructMatrix/TPZSpStructMatrix, TPZStepSolver CG + "
             "Jacobi(1,0,0)) on the same synthetic grids; counts are independent of the equation ordering",
        poisson2d_q2_64=dict(neq=16641, nnz_upper=139905, cg_iters_1e10=114,
                             setup="CreateGeoMeshOnGrid 2D 64x64 quads, p=2, f=2pi^2 sin sin (pOrder 2), "
                                   "penalty Dirichlet u=0 on all edges"),
        elast3d_q2_16=dict(neq=107811, nnz_upper=9714006, cg_iters_1e8=262,
                           setup="unit cube 16^3 hexes, p=2, E=1, nu=0.3, body force (0,0,-1), z=0 clamped "
                                 "(type 0), traction (0,0,-1) on z=1 (type 1)"),
        elast3d_q2_32=dict(neq=823875, nnz_upper=76797606),
        elast3d_q2_64=dict(neq=6440067, nnz_upper=610745670, nnz_full=1215051273))
    with open(os.path.join(HERE, "reference_unit_golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "reference_unit_golden.json"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the NeoPZ source tree>")
    main(sys.argv[1])
