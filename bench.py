"""Benchmark: time to ||r||/||b|| < 1e-8 on 3D Q2 linear elasticity (64^3 hexes) on one GB300.

One step = the hot path over the synthetic system: global assembly into the
CSR (FP64 parity assembly + the FP32 operator of the inner solves) and the
iterative solve to a TRUE FP64 residual below 1e-8 with the learned + mixed
flexible PCG (the committed elasticity weights on the two-level block-Jacobi
base, FP32 operator and recurrence, FP64 true-residual replacement).  `value`
is device time with the mesh and pattern resident in HBM (CUDA events on the
library's stream); `e2e` is the same pipeline through the public C ABI from
host buffers (mesh upload, pattern build, assembly, weights, solve, solution
download).  The plain FP64 Jacobi-PCG of the reference (same algorithm, on the
GPU) is timed once beside it as the path's own baseline; the mixed two-level
CG (the same method without the network) and the mixed block-Jacobi CG are
timed once each as the other comparisons (`--path` picks the timed one).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--n 64]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "s to ||r||/||b||<1e-8: learned+mixed PCG vs FP64 Jacobi-PCG (GB300); elem/s"
LEARNED_WEIGHTS = os.path.join(ROOT, "neopz_gb300", "data", "learned_elasticity3d_q2.npy")
LEARNED_RANK = 8
LEARNED_BASE = 4  # GPZ_PRECOND_TWO_LEVEL: the base under the learned correction
# solver paths of a step: the metric's learned + mixed flexible PCG (the correction on the two-level base), the
# mixed CG with that base alone (the method without the network), the mixed block-Jacobi CG, the FP64 Jacobi-PCG
PATH_KEY = {"learned": "learned_mixed_fcg", "two_level": "mixed_two_level_cg", "mixed": "mixed_block_jacobi_cg",
            "learned_block": "learned_mixed_fcg_block_jacobi", "fp64": "fp64_jacobi_pcg"}
PATH_CHECK = {"learned": 16, "two_level": 16, "mixed": 64, "learned_block": 64, "fp64": 64}  # per convergence check
PATH_DESC = {
    "learned": ("FP64 assembly + FP32 operator ({op}); learned + mixed flexible PCG: learned element-to-node "
                "correction (rank {rank}, weights {weights}, trained on the GPU) on the two-level block-Jacobi base "
                "(3x3 connect blocks + Galerkin coarse grid), FP32 recurrence, FP64 x/dots/alpha/beta, reliable "
                "FP64 true-residual updates"),
    "two_level": ("FP64 assembly + FP32 operator ({op}); mixed CG with the two-level block-Jacobi preconditioner "
                  "(3x3 connect blocks + Galerkin coarse grid of 8^3 boxes, coarse inverse on the device), FP32 "
                  "recurrence, FP64 x/dots, reliable FP64 true-residual updates"),
    "mixed": ("FP64 assembly + FP32 operator ({op}); mixed CG with connect-block (3x3) Jacobi, FP32 recurrence, "
              "FP64 x/dots, reliable FP64 true-residual updates"),
    "learned_block": ("FP64 assembly + FP32 operator ({op}); learned + mixed flexible PCG with the same network on "
                      "the connect-block (3x3) Jacobi base: the ablation against mixed_block_jacobi_cg"),
    "fp64": "FP64 assembly; FP64 Jacobi-PCG (the reference's algorithm)"}
TOL = 1e-8
ERR_REF_TOL = 1e-12  # true residual of the FP64 solve the solution errors are measured against
SEED = 5
# HBM bytes per stored block measured by ncu for the SpMV kernels (32^3 case):
# k_mx_sym3 375.6 MB read + 3.3 MB written over 8,624,609 upper blocks
NCU_TRAFFIC_PER_BLOCK = {"upper_blocks_float4_atomics": (375.615488e6 + 3.251968e6) / 8624609}
# the shared-element-matrix operator on the 40^3 case (64,000 volume elements, one launch inside a solve):
# dram__bytes_read.sum + dram__bytes_write.sum per volume element (profiles/matfree_shared_matrix_elasticity_q2.txt)
NCU_TRAFFIC_PER_ELEMENT = {"matrix_free_shared_matrix_tcgen05": (24.5696e6 + 0.0) / 64000,
                           # the lattice-block operator on the same 40^3 case (profiles/matfree_lattice_blocks_elasticity_q2.txt)
                           "matrix_free_shared_matrix_lattice_blocks": (17.261312e6 + 0.0) / 64000}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-baseline", action="store_true", help="skip the FP64 Jacobi-PCG reference solve")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end C-ABI leg")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-preconditioner (2D Darcy) leg")
    ap.add_argument("--no-hp", action="store_true", help="skip the hp (uneven-order) assembly leg")
    ap.add_argument("--hp-n", type=int, default=40, help="hexes per direction of the hp leg")
    ap.add_argument("--no-poisson3d", action="store_true", help="skip the 3D scalar (64^3 Q2 Darcy) leg")
    ap.add_argument("--poisson3d-n", type=int, default=64, help="hexes per direction of the 3D scalar leg")
    ap.add_argument("--poisson3d-variant", type=int, default=-1,
                    help="FP32 operator of the 3D scalar leg: -1 autotuned, 0 the FP32 CSR, 9 the shared matrix")
    ap.add_argument("--no-sloan", action="store_true", help="skip the host graph legs (Sloan renumbering, node-set blocks)")
    ap.add_argument("--spmv-variant", type=int, default=-1,
                    help="FP32 operator of the mixed solves: -1 autotuned, else the gpz_solver_opts spmv_variant")
    ap.add_argument("--path", default="learned", choices=["learned", "two_level", "mixed"],
                    help="solver of the timed step: learned + mixed flexible PCG on the two-level base, the mixed "
                         "two-level CG, or the mixed block-Jacobi CG")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(t, world, device):
    """Replicas: every rank times its own system, and the job's time per step is the slowest rank's
    (an all-reduce MAX; device "cuda" under NCCL, "cpu" under gloo)."""
    if world == 1:
        return t
    import torch
    import torch.distributed as dist
    x = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(x, op=dist.ReduceOp.MAX)
    return float(x.item())


class Clocks:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, device):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

        def run():
            try:
                p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                     stderr=subprocess.DEVNULL, text=True)
            except OSError:
                return
            while not self._stop.is_set():
                line = p.stdout.readline()
                if not line:
                    break
                self.samples.append([x.strip() for x in line.split(",")])
            p.terminate()

        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=3)
        sm = [float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            for i, nm in enumerate(names):
                if len(s) > 4 + i and s[4 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


def make_problem(n):
    from neopz_gb300 import gpz
    E = gpz.lognormal(n ** 3, 1.0, SEED)
    return gpz.elasticity3d(n, 2, E=E, nu=0.3, top_traction=True, body_force=(0.0, 0.0, 0.0)), E


def mesh_bytes(grid):
    d = grid.desc
    return (d.nnodes * 3 * 8 + d.nel * (4 + 4 + 8 * 8 + 4 + 27 * 8 + (8 if d.el_coef else 0)) +
            d.nconnects * (4 + 8 + 4))


def run_gpu(args):
    import torch
    from neopz_gb300 import gpz

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = local
    torch.cuda.set_device(dev)
    n = args.n
    t0 = time.perf_counter()
    grid, E = make_problem(n)
    t_mesh = time.perf_counter() - t0
    ctx = gpz.Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    ctx.upload_mesh(grid)
    t0 = time.perf_counter()
    nnz_upper = ctx.build_pattern(True)
    torch.cuda.synchronize()
    t_pattern = time.perf_counter() - t0
    nnz = ctx.nnz_full()
    nel = grid.nel
    nvol = grid.nvol

    weights = np.load(LEARNED_WEIGHTS)
    ctx.assemble(gpz.GPZ_PREC_FP64)
    ctx.learned_init(rank=LEARNED_RANK, seed=0)
    ctx.set_learned_params(weights)

    def step(path=None):
        """One step: assembly (FP64 matrix + the FP32 operator of the mixed paths) and the solve to a true FP64
        ||r||/||b|| < 1e-8 on `path` (the timed one by default)."""
        path = args.path if path is None else path
        ctx.assemble(gpz.GPZ_PREC_FP64 if path == "fp64" else gpz.GPZ_PREC_MIXED)
        kw = dict(tol=TOL, max_iter=200000, check_every=PATH_CHECK[path], want_x=False)
        if path == "learned":
            return ctx.solve(solver=gpz.GPZ_SOLVER_LEARNED_MIXED_FCG, precond=LEARNED_BASE, reliable_delta=1e-2,
                             spmv_variant=args.spmv_variant, **kw)
        if path == "learned_block":
            return ctx.solve(solver=gpz.GPZ_SOLVER_LEARNED_MIXED_FCG, precond=gpz.GPZ_PRECOND_BLOCK_JACOBI,
                             reliable_delta=1e-2, spmv_variant=args.spmv_variant, **kw)
        if path in ("two_level", "mixed"):
            pre = gpz.GPZ_PRECOND_TWO_LEVEL if path == "two_level" else gpz.GPZ_PRECOND_BLOCK_JACOBI
            return ctx.solve(solver=gpz.GPZ_SOLVER_MIXED_CG, precond=pre, reliable_delta=1e-2,
                             spmv_variant=args.spmv_variant, **kw)
        return ctx.solve(solver=gpz.GPZ_SOLVER_CG, **kw)

    def timed(fn):
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e0.record(stream)
        r = fn()
        with torch.cuda.stream(stream):
            e1.record(stream)
        torch.cuda.synchronize()
        return r, e0.elapsed_time(e1) / 1e3

    # the reference's plain FP64 Jacobi-PCG on the GPU (the 3x target's denominator)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    fp64, t_fp64, x_fp64 = {"iterations": None, "true_resid": None}, None, None
    if not args.no_fp64_baseline:
        with torch.cuda.stream(stream):
            e0.record(stream)
        fp64 = step("fp64")
        with torch.cuda.stream(stream):
            e1.record(stream)
        torch.cuda.synchronize()
        t_fp64 = e0.elapsed_time(e1) / 1e3
        x_fp64 = ctx.solution()
    for _ in range(args.warmup):
        step()
    # element matrices + scatter alone (FP64), for elements/s
    t_asm = ctx.time_kernel(gpz.GPZ_KERNEL_ASSEMBLE, 3) / 1e3
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(dev)
    clocks.start()
    l0 = ctx.launches()
    with torch.cuda.stream(stream):
        e0.record(stream)
    reps = [step() for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        e1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.launches() - l0
    ms_step = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    t_step = ms_step / 1e3
    t_step = max_over_ranks(t_step, world, "cuda")
    last = reps[-1]
    x_step = ctx.solution()  # the last timed step's solution (outside the timed region)
    # the other mixed paths, one step each (after a warm-up step): the two-level CG without the network (the
    # method without the learned correction), the block-Jacobi CG, and the network on the block-Jacobi base
    others = {}
    for path in [q for q in ("learned", "two_level", "mixed", "learned_block") if q != args.path]:
        step(path)
        r, t = timed(lambda: step(path))
        others[path] = (r, t, ctx.solution())
    # solution error against the FP64 solution: the FP64 Jacobi-PCG (the parity-tested path, the same algorithm
    # as the reference's CG) run to a true residual of 1e-12, well below the 1e-8 stop of the compared solves
    accuracy = {}
    if not args.no_fp64_baseline:
        ctx.assemble(gpz.GPZ_PREC_FP64)
        tight = ctx.solve(solver=gpz.GPZ_SOLVER_CG, tol=ERR_REF_TOL, max_iter=400000, check_every=64)
        xr = tight["x"]
        nr = float(np.linalg.norm(xr))
        accuracy = {
            "reference_solution": (f"FP64 Jacobi-PCG (GPU, parity-tested against the oracle and the reference's "
                                   f"fixtures) to a true residual {ERR_REF_TOL:g}: {tight['iterations']} iterations, "
                                   f"true residual {tight['true_resid']:.3g}"),
            "value_path": float(np.linalg.norm(x_step - xr) / nr),
            **{PATH_KEY[q]: float(np.linalg.norm(v[2] - xr) / nr) for q, v in others.items()},
            "fp64_jacobi_pcg": float(np.linalg.norm(x_fp64 - xr) / nr) if x_fp64 is not None else None,
            "bar": 1e-8}
        del xr, tight
        ctx.assemble(gpz.GPZ_PREC_MIXED)  # back to the timed path's operator for the kernel timings below

    # roofline of the dominant kernel: the FP32 3x3-block SpMV of the inner CG, in the
    # layout the library's autotuner chose (HBM bytes that layout must stream per launch)
    tune = ctx.tuning_report()
    ms32 = ctx.time_kernel(gpz.GPZ_KERNEL_SPMV_FP32, 20)
    ms64 = ctx.time_kernel(gpz.GPZ_KERNEL_SPMV_FP64, 10)
    neq = grid.neq
    nbrow = neq // 3
    chosen = tune.get("chosen", "block_csr")
    mf_flops = None
    matfree = chosen in ("matrix_free_elements", "matrix_free_sum_factorised", "matrix_free_tcgen05_3xtf32",
                         "matrix_free_shared_matrix_tcgen05", "matrix_free_shared_matrix_lattice_blocks")
    mma_flops = None
    if matfree:
        # element records (corners 96 B, block rows 108 B, lambda/mu 8 B, affine geometry 40 B), penalty-face
        # records (48 + 36 B),
        # p read once and q accumulated once (16 B per block row each)
        nface = (n + 0) * (n + 0)
        nblk = 0
        l2_atomics = 27 * nvol + 9 * nface
        if chosen == "matrix_free_shared_matrix_tcgen05":
            kern = ("k_mf_hex27_gm: matrix-free Q2 elasticity on a translated grid, K_e = mu_e Khat as one tcgen05 "
                    "kind::tf32 3xTF32 GEMM per tile of 128 elements (M 128, N 96, K 88), gatherer and scatterer warp "
                    "groups, float4 vector reductions into q (block rows + mu per element and one pass of p and q are "
                    "its HBM bytes)")
            # algorithmic FLOPs: the 81 x 81 product per element; the MMAs execute 3 products of the padded tile
            mf_flops = nvol * 2 * 81 * 81 + nface * 2 * 9 * 9 * 6
            mma_flops = -(-nvol // 128) * 3 * 2 * 128 * 96 * 88
        elif chosen == "matrix_free_shared_matrix_lattice_blocks":
            kern = ("k_mf_hex27_gt: the same K_e = mu_e Khat tcgen05 3xTF32 GEMM over lattice blocks of 8 x 8 x 2 "
                    "elements: a block's connect values and results in shared memory, plain stores inside the block, "
                    "float4 reductions on its faces, loader and writer warp groups pipelined over blocks (mu per "
                    "element, the lattice connect map and one pass of p and q are its HBM bytes)")
            mf_flops = nvol * 2 * 81 * 81 + nface * 2 * 9 * 9 * 6
            mma_flops = -(-nvol // 128) * 3 * 2 * 128 * 96 * 88
            # reductions: the connects on block faces (17 x 17 x 5 box less its 15 x 15 x 3 inside) and penalty faces
            l2_atomics = -(-n // 8) * -(-n // 8) * -(-n // 2) * (17 * 17 * 5 - 15 * 15 * 3) + 9 * nface
        elif chosen == "matrix_free_sum_factorised":
            kern = ("k_mf_hex27_sf: matrix-free Q2 elasticity, sum-factorised on Lagrange nodal values, one warp per "
                    "element (CUDA-core FP32; records + one pass of p and q are its HBM bytes)")
            # FLOPs per element: Phi and Phi^T (2 x 2 x 125 x 3), the 1D contractions forward and back
            # (2 x 2 x 8 x 81 x 3), per point the Jacobian products and the stress (27 x (2 x 2 x 27 + 30))
            mf_flops = nvol * (2 * 2 * 125 * 3 + 2 * 2 * 8 * 81 * 3 + 27 * (2 * 2 * 27 + 30)) + nface * 2 * 9 * 9 * 6
        else:
            kern = ("k_mf_hex27" + ("_tc" if chosen.endswith("3xtf32") else "") + ": matrix-free Q2 elasticity, one "
                    "warp per element (records + one pass of p and q are its HBM bytes)")
            # FLOPs per element: per point, grad(u) from 27 shapes (2 x 243), geometry ~110, stress and the two
            # Jacobian products ~60 + 2 x 27; per shape, the 27-point back-projection (2 x 27 x 9)
            mf_flops = nvol * (27 * (2 * 243 + 110 + 60 + 2 * 27) + 27 * 2 * 27 * 9) + nface * 2 * 9 * 9 * 6
    elif chosen == "upper_blocks_float4_atomics":
        nblk = tune["blocks_upper"]
        kern = "k_mx_sym3: upper 3x3 blocks (36 B values + 4 B column), transposed products as float4 atomics in L2"
        l2_atomics = nblk
    else:
        nblk = tune.get("blocks_full", nnz // 9)
        kern = "k_mx_" + chosen + ": full 3x3 blocks (36 B values + 4 B column)"
        l2_atomics = 0
    # values + columns + block-row pointers + p (16 B per block row, read once) + q (written once)
    bytes32 = nblk * (36 + 4) + (nbrow + 1) * 8 + nbrow * 16 + nbrow * 16
    if matfree:
        rec = 108 + 8 if chosen == "matrix_free_shared_matrix_tcgen05" else 96 + 108 + 8 + 40
        bytes32 = nvol * rec + nface * (48 + 36) + nbrow * 16 + nbrow * 16
        if chosen == "matrix_free_shared_matrix_lattice_blocks":  # mu per element; connect map and face flag per row
            bytes32 = nvol * 4 + nbrow * (4 + 1) + nface * (48 + 36) + nbrow * 16 + nbrow * 16
    bytes64 = nnz * (8 + 4) + (neq + 1) * 8 + neq * 8 + neq * 8 + neq * 8
    pk = peaks()
    hbm = pk.get("hbm_gbs", 6800.0)
    ach = bytes32 / (ms32 * 1e-3) / 1e9
    # ncu capture of this kernel on a smaller case (dram__bytes_read.sum + dram__bytes_write.sum per launch),
    # scaled to this size by the stored blocks or the volume elements it streams
    traffic = None
    if chosen in NCU_TRAFFIC_PER_BLOCK:
        traffic = int(NCU_TRAFFIC_PER_BLOCK[chosen] * nblk)
    elif chosen in NCU_TRAFFIC_PER_ELEMENT:
        traffic = int(NCU_TRAFFIC_PER_ELEMENT[chosen] * nvol)

    # exact-solution error norms (TPZAnalysis::PostProcessError) of the last solution kept on the device,
    # against u = 0: the norms (energy, L2, H1 semi) of the solution itself, the load having no closed-form
    # solution; the evaluation call includes the upload of the exact values (zeros) at every point
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    exyz = ctx.error_points(2)
    t1 = time.perf_counter()
    ue, due = np.zeros((len(exyz), 3)), np.zeros((len(exyz), 3, 3))
    t2 = time.perf_counter()
    enorm, _ = ctx.error_norms(2, ue, due)
    t3 = time.perf_counter()
    err_leg = {"exact_order": 2, "points": int(len(exyz)), "solution_norms": [float(v) for v in enorm],
               "points_s": round(t1 - t0, 4), "evaluate_s": round(t3 - t2, 4),
               "volume_elements_per_s": round(nvol / (t3 - t2), 1),
               "h2d_bytes": int(ue.nbytes + due.nbytes)}
    del exyz, ue, due

    # end to end through the C ABI from host buffers
    e2e_times, e2e_phases = [], []
    b_in = mesh_bytes(grid)
    for _ in range(0 if args.no_e2e else max(1, min(args.steps, 2))):
        torch.cuda.synchronize()
        ph = {}
        t0 = time.perf_counter()
        tp = t0

        def mark(name):
            nonlocal tp
            t = time.perf_counter()
            ph[name] = round(t - tp, 4)
            tp = t
        c2 = gpz.Context(dev)
        mark("context")
        c2.upload_mesh(grid)
        mark("mesh_upload")
        ph["mesh_upload_parts_ms"] = c2.assembly_report().get("mesh_upload_ms")
        tp = time.perf_counter()
        c2.build_pattern(True)
        mark("pattern")
        c2.assemble(gpz.GPZ_PREC_MIXED)
        mark("assembly_and_operator_autotune")
        kw = dict(tol=TOL, max_iter=200000, reliable_delta=1e-2, check_every=PATH_CHECK[args.path], want_x=True)
        if args.path == "learned":
            c2.learned_init(rank=LEARNED_RANK, seed=0)
            mark("learned_setup")
            c2.set_learned_params(weights)
            mark("learned_weights")
            r2 = c2.solve(solver=gpz.GPZ_SOLVER_LEARNED_MIXED_FCG, precond=LEARNED_BASE, **kw)
        else:
            r2 = c2.solve(solver=gpz.GPZ_SOLVER_MIXED_CG, precond=gpz.GPZ_PRECOND_TWO_LEVEL if args.path ==
                          "two_level" else gpz.GPZ_PRECOND_BLOCK_JACOBI, **kw)
        torch.cuda.synchronize()
        mark("solve_and_download")
        e2e_times.append(time.perf_counter() - t0)
        e2e_phases.append(ph)
        assert r2["true_resid"] <= TOL
        c2.close()
    t_e2e = min(e2e_times) if e2e_times else None
    e2e_best = e2e_phases[e2e_times.index(t_e2e)] if e2e_times else None

    out = {
        "metric": METRIC, "value": round(t_step, 6), "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
        "config": {"workload": f"3D linear elasticity {n}^3 hex Q2 (TPZElasticity3D), E lognormal(sigma=1) seed {SEED}, "
                               "nu=0.3, clamped z=0 (penalty), traction (0,0,-1) on z=1",
                   "neq": neq, "nnz_full": nnz, "nnz_upper": nnz_upper, "elements": nel, "volume_elements": nvol,
                   "path": PATH_DESC[args.path].format(rank=LEARNED_RANK, weights=os.path.relpath(LEARNED_WEIGHTS,
                                                                                                   ROOT),
                                                      op=chosen),
                   "l2": "inputs larger than L2 (matrix > 129 MB)",
                   "parallelism": f"replicas x{world}"},
        "solution_rel_err_vs_fp64": accuracy.get("value_path"),
        "solution_error": accuracy,
        "solve": {"iterations": last["iterations"], "true_resid": last["true_resid"],
                  "reliable_updates": last["reliable_updates"], "spmv_fp32": last["spmv_fp32"],
                  "spmv_fp64": last["spmv_fp64"], "restarts": last["restarts"], "solve_s": last["seconds"]},
        "fp64_jacobi_pcg": {"seconds": t_fp64, "iterations": fp64["iterations"], "true_resid": fp64["true_resid"],
                            "speedup_of_value": (t_fp64 / t_step) if t_fp64 else None},
        **{PATH_KEY[q]: {"seconds": round(t, 6), "iterations": r["iterations"], "true_resid": r["true_resid"],
                         "solve_s": r["seconds"], "speedup_vs_fp64_jacobi_pcg": (t_fp64 / t) if t_fp64 else None,
                         "path": PATH_DESC[q].format(rank=LEARNED_RANK, weights=os.path.relpath(LEARNED_WEIGHTS,
                                                                                                   ROOT), op=chosen),
                         "note": "one step (assembly + solve), timed once after the timed steps"}
           for q, (r, t, _) in others.items()},
        "assembly": {"fp64_seconds": t_asm, "elements_per_s": nel / t_asm, "volume_elements_per_s": nvol / t_asm,
                     "pattern_build_s": t_pattern, "host_mesh_build_s": t_mesh},
        "e2e": {"value": round(t_e2e, 6) if t_e2e else None, "unit": "s", "phases_s": e2e_best, "h2d_bytes_per_step": int(b_in + (weights.nbytes if args.path == "learned" else 0)),
                "d2h_bytes_per_step": int(neq * 8)},
        "roofline": {"bound": "hbm", "kernel": kern, "achieved": round(ach, 1),
                     "peak": hbm, "unit": "GB/s", "frac": round(ach / hbm, 4), "traffic": traffic,
                     "l2_float4_atomics_per_launch": l2_atomics,
                     "algorithmic_bytes": int(bytes32), "ms_per_launch": ms32,
                     "fp32_tflops": (round(mf_flops / (ms32 * 1e-3) / 1e12, 2) if mf_flops else None),
                     "tensor_mma_tflops": (round(mma_flops / (ms32 * 1e-3) / 1e12, 2) if mma_flops else None),
                     "fp32_peak_tflops_nominal": (round(152 * 128 * 2 * 2.07e9 / 1e12, 1) if mf_flops else None),
                     "fp64_spmv": {"ms_per_launch": ms64,
                                   "achieved_gbs": round(bytes64 / (ms64 * 1e-3) / 1e9, 1)},
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if "fallback" not in pk else
                     "fallback 6.8 TB/s"},
        "spmv_autotune_ms": ctx.tuning_report(),
        "error_norms": err_leg,
        "clocks": clk,
        "gpu_launches": int(launches),
    }
    if rank == 0 and not args.no_learned:
        out["learned_darcy2d"] = learned_leg(gpz, dev)
    if rank == 0 and not args.no_hp:
        out["hp_elasticity"] = hp_leg(gpz, dev, args.hp_n)
    if rank == 0 and not args.no_sloan:
        out["sloan_renumbering"], out["nodeset_blocks"] = sloan_leg(gpz, n)
    if rank == 0 and not args.no_poisson3d:
        out["poisson3d"] = poisson3d_leg(gpz, dev, args.poisson3d_n, args.poisson3d_variant)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(fp64["iterations"], n)
    if rank == 0:
        print(json.dumps(out))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def hp_leg(gpz, dev, n=40):
    """Assembly of the uneven-order workload: 3D elasticity on 40^3 hexes, preferred order uniform in {1,2,3}
    per element (seed 3), shared sides at the largest order, E lognormal(sigma=0.5), nu=0.3, body force
    (0,0,-1), clamped base; plus its solve (mixed CG, block Jacobi) to the same true FP64 residual."""
    orders = gpz.hp_orders(n ** 3, 3)
    E = gpz.lognormal(n ** 3, 0.5, 3)
    grid = gpz.elasticity3d_hp(n, orders, E=E)
    ctx = gpz.Context(dev)
    ctx.assembly_mode(-1)  # time both launch modes (per colour, persistent) on the first assembly
    ctx.upload_mesh(grid)
    nnz = ctx.build_pattern(True)
    ctx.assemble()  # the first assembly runs the hp kernels' block-size and launch-mode autotuners
    ms = ctx.time_kernel(gpz.GPZ_KERNEL_ASSEMBLE, 3)
    rep = ctx.assembly_report()
    ctx.assemble(gpz.GPZ_PREC_MIXED)
    sol = ctx.solve(solver=gpz.GPZ_SOLVER_MIXED_CG, precond=gpz.GPZ_PRECOND_BLOCK_JACOBI, tol=TOL, max_iter=200000,
                    reliable_delta=1e-2, check_every=64, want_x=False)
    # the node-set blocks of BuildPreconditioner(EBlockJacobi, overlap = false): the higher-order connects merged
    # with their neighbours' (built on the host before the solve's timed region)
    ns = ctx.solve(solver=gpz.GPZ_SOLVER_MIXED_CG, precond=gpz.GPZ_PRECOND_NODESET_JACOBI, tol=TOL,
                   max_iter=200000, reliable_delta=1e-2, check_every=64, want_x=False)
    fp32 = fp32_element_pass(gpz, ctx, precond=gpz.GPZ_PRECOND_BLOCK_JACOBI)
    ctx.close()
    return {"workload": f"3D elasticity {n}^3 hexes, p uniform in {{1,2,3}} per element (seed 3, max rule on shared "
                        "sides), E lognormal(sigma=0.5) seed 3, nu=0.3, body force (0,0,-1), clamped z=0",
            "neq": grid.neq, "nnz_upper": nnz, "elements": grid.nel, "assembly_fp64_s": ms / 1e3,
            "elements_per_s": grid.nel / (ms / 1e3), "batching": rep,
            "mixed_cg": {"iterations": sol["iterations"], "true_resid": sol["true_resid"], "seconds": sol["seconds"],
                         "rc": sol["rc"]},
            "mixed_cg_nodeset_blocks": {"iterations": ns["iterations"], "true_resid": ns["true_resid"],
                                        "seconds": ns["seconds"], "rc": ns["rc"]},
            "fp32_element_pass": fp32}


def fp32_element_pass(gpz, ctx, precond, variant=-1):
    """The FP32 element pass (gpz_fp32_elements: the hexes' element matrices as 3xTF32 tcgen05 GEMMs, into the
    FP32 CSR of the mixed solves) on an assembled context: its time (CUDA events, the second of two mixed
    assemblies) and the mixed CG over the FP32 operator built from it, beside the same solve over the rounded
    FP64 matrix."""
    ctx.fp32_elements(gpz.GPZ_FP32_ELEMENTS)
    for _ in range(2):
        ctx.assemble(gpz.GPZ_PREC_MIXED)
    rep = ctx.assembly_report()["fp32_elements"]
    sol = ctx.solve(solver=gpz.GPZ_SOLVER_MIXED_CG, precond=precond, tol=TOL, max_iter=200000, reliable_delta=1e-2,
                    check_every=64, want_x=False, spmv_variant=variant)
    ctx.fp32_elements(gpz.GPZ_FP32_ROUNDED)
    return {"pass_ms": rep["ms"], "tensor_core_elements": rep["tensor_core_elements"],
            "cuda_core_elements": rep["cuda_core_elements"],
            "tensor_core_elements_per_s": rep["tensor_core_elements"] / (rep["ms"] / 1e3) if rep["ms"] else None,
            "fp32_operator": ctx.tuning_report().get("chosen"),
            "mixed_cg": {"iterations": sol["iterations"], "seconds": sol["seconds"], "true_resid": sol["true_resid"],
                         "rc": sol["rc"]}}


def sloan_leg(gpz, n):
    """Host graph work on the benchmark mesh's connect graph: TPZAnalysis::OptimizeBandwidth's Sloan
    renumbering (gpz_sloan_resequence) with the graph's profile before and after, and the node-set blocks of
    BuildPreconditioner(EBlockJacobi, overlap = false) (gpz_nodeset_blocks) with their size histogram."""
    try:
        grid = gpz.elasticity3d(n, 2)
        ei, eg = grid.element_graph()
        nn = grid.desc.nconnects
    except Exception as exc:  # a host-side leg: report, do not stop the benchmark
        return {"error": repr(exc)}, {"error": repr(exc)}
    workload = f"connect graph of the {n}^3 Q2 hex mesh (boundary elements included)"
    try:
        t0 = time.perf_counter()
        pg, _ = gpz.sloan_resequence(nn, ei, eg)
        dt = time.perf_counter() - t0

        def envelope(perm):
            low = np.arange(nn)
            for e in range(len(ei) - 1):
                p = perm[eg[ei[e]:ei[e + 1]]]
                low[p] = np.minimum(low[p], p.min())
            return int(np.sum(np.arange(nn) - low))

        sloan = {"workload": workload, "connects": nn,
                 "seconds": round(dt, 3), "graph_build_threads": min(16, os.cpu_count() or 1),
                 "numbering_threads": 1, "envelope_creation_order": envelope(np.arange(nn)),
                 "envelope_sloan": envelope(pg)}
    except Exception as exc:
        sloan = {"error": repr(exc)}
    try:
        bp = np.ctypeslib.as_array(grid.desc.block_pos, shape=(nn,)).copy()
        bs = np.ctypeslib.as_array(grid.desc.block_size, shape=(nn,)).copy()
        t0 = time.perf_counter()
        r = gpz.nodeset_blocks(nn, ei, eg, bp, bs, grid.neq)
        dt = time.perf_counter() - t0
        sizes, counts = np.unique(np.diff(r["blockindex"]), return_counts=True)
        nodeset = {"workload": workload, "connects": nn, "equations": grid.neq, "seconds": round(dt, 3),
                   "relation_threads": min(16, os.cpu_count() or 1), "numbering_threads": 1,
                   "blocks": int(len(r["blockindex"]) - 1), "colors": r["ncolors"],
                   "block_sizes": {str(int(k)): int(v) for k, v in zip(sizes, counts)}}
    except Exception as exc:
        nodeset = {"error": repr(exc)}
    return sloan, nodeset


def poisson3d_leg(gpz, dev, n=64, variant=-1):
    """The 3D scalar workload: -div(k grad u) = 1 on the unit cube, 64^3 Q2 hexes (2,146,689 equations),
    k lognormal(sigma=1) per element (seed 1), u = 0 on the boundary: FP64 assembly, then the mixed CG (the FP32
    operator the autotuner picks: the FP32 CSR copy or the scalar shared-element-matrix tcgen05 kernel; Jacobi)
    and the FP64 Jacobi-PCG, both to a true FP64 residual 1e-8."""
    k = gpz.lognormal(n ** 3, 1.0, 1)
    grid = gpz.darcy(3, n, 2, k)
    ctx = gpz.Context(dev)
    ctx.upload_mesh(grid)
    nnz = ctx.build_pattern(True)
    ctx.assemble()
    ms = ctx.time_kernel(gpz.GPZ_KERNEL_ASSEMBLE, 3)
    f64 = ctx.solve(tol=TOL, max_iter=200000, check_every=64, want_x=False)
    ctx.assemble(gpz.GPZ_PREC_MIXED)
    for _ in range(2):  # the second is timed (graphs instantiated)
        mx = ctx.solve(solver=gpz.GPZ_SOLVER_MIXED_CG, tol=TOL, max_iter=200000, reliable_delta=1e-2,
                       check_every=64, want_x=False, spmv_variant=variant)
    tune = ctx.tuning_report()
    op_ms = ctx.time_kernel(gpz.GPZ_KERNEL_SPMV_FP32, 20)
    fp32 = fp32_element_pass(gpz, ctx, gpz.GPZ_PRECOND_JACOBI, variant=0)  # the CSR copy reads the pass's values
    ctx.close()
    return {"workload": f"3D Darcy/Poisson {n}^3 hex Q2, k lognormal(sigma=1) seed 1, u = 0 on the boundary (penalty)",
            "neq": grid.neq, "nnz_upper": nnz, "assembly_fp64_s": ms / 1e3, "volume_elements_per_s": n ** 3 / (ms / 1e3),
            "fp64_jacobi_pcg": {"iterations": f64["iterations"], "seconds": f64["seconds"],
                                "true_resid": f64["true_resid"]},
            "mixed_cg": {"iterations": mx["iterations"], "seconds": mx["seconds"], "true_resid": mx["true_resid"],
                         "speedup_vs_fp64_jacobi_pcg": f64["seconds"] / mx["seconds"] if mx["seconds"] else None,
                         "fp32_operator": tune.get("chosen"), "operator_autotune_ms": tune,
                         "operator_ms_per_launch": op_ms},
            "fp32_element_pass": fp32}


def learned_leg(gpz, dev, n=256, seeds=(10000, 10001, 10002)):
    """Learned flexible CG against FP64 Jacobi-PCG on the 2D Darcy workload the network was trained
    for (256^2 Q2 quads, GRF permeability, unseen seeds), with the committed weights."""
    wfile = os.path.join(ROOT, "neopz_gb300", "data", "learned_darcy2d_q2.npy")
    grid = gpz.darcy_grf(n, 2, seed=seeds[0])
    ctx = gpz.Context(dev)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble()
    ctx.learned_init(rank=4)
    ctx.set_learned_params(np.load(wfile))
    rows = []
    for s in seeds:
        ctx.set_coef(grid, gpz.grf2d(n, seed=s))
        ctx.assemble()
        for _ in range(2):  # the second of each is timed (graphs instantiated, caches warm)
            jac = ctx.solve(tol=TOL, max_iter=200000, want_x=False)
            lrn = ctx.solve(solver=gpz.GPZ_SOLVER_LEARNED_FCG, tol=TOL, max_iter=200000, want_x=False)
            lmx = ctx.solve(solver=gpz.GPZ_SOLVER_LEARNED_MIXED_FCG, tol=TOL, max_iter=200000, reliable_delta=1e-2,
                            want_x=False)
        assert lrn["rc"] == 0 and lrn["true_resid"] <= TOL and lmx["rc"] == 0 and lmx["true_resid"] <= TOL
        rows.append(dict(seed=s, jacobi_iterations=jac["iterations"], jacobi_s=round(jac["seconds"], 6),
                         learned_iterations=lrn["iterations"], learned_s=round(lrn["seconds"], 6),
                         learned_true_resid=lrn["true_resid"], jacobi_fallbacks=lrn["restarts"],
                         learned_mixed_iterations=lmx["iterations"], learned_mixed_s=round(lmx["seconds"], 6),
                         learned_mixed_true_resid=lmx["true_resid"],
                         learned_mixed_reliable_updates=lmx["reliable_updates"]))
    ctx.close()
    tj = sum(r["jacobi_s"] for r in rows)
    tl = sum(r["learned_s"] for r in rows)
    tm = sum(r["learned_mixed_s"] for r in rows)
    return {"workload": f"2D Darcy {n}^2 Q2 quads, k = exp(GRF sigma 1.5, correlation 0.1), unseen seeds "
                        f"{seeds[0]}..{seeds[-1]}, tol {TOL} (true FP64 residual)",
            "weights": "neopz_gb300/data/learned_darcy2d_q2.npy (trained on the GPU: 2000 fields, checkpoint selected on validation fields)",
            "fields": rows, "iterations_ratio": round(sum(r["learned_iterations"] for r in rows) /
                                                      sum(r["jacobi_iterations"] for r in rows), 3),
            "speedup_vs_fp64_jacobi_pcg": round(tj / tl, 3),
            "learned_mixed_speedup_vs_fp64_jacobi_pcg": round(tj / tm, 3)}


def cpu_sample(n_sample, iters_full, n_full, threads, cg_iters=30):
    """The oracle (the reference's algorithm restated: OR threaded assembly,
    serial symmetric SpMV, Jacobi with its extra Residual SpMV) on an
    n_sample^3 instance of the same workload; extrapolated to n_full^3."""
    from oracle import oracle as O
    E = np.exp(np.random.default_rng(SEED).standard_normal(n_sample ** 3))
    t0 = time.perf_counter()
    m = O.elasticity3d(n_sample, 2, E=E)
    ia, ja = m.pattern(True)
    t_pat = time.perf_counter() - t0
    t0 = time.perf_counter()
    a, f = m.assemble(True, ia, ja, nthreads=threads)
    t_asm = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.cg_jacobi(True, ia, ja, a, f, cg_iters, 0.0, jacobi_residual=True)
    t_it = (time.perf_counter() - t0) / cg_iters
    nel_s = m.ncel
    nnz_s = len(ja)
    # scale: assembly by element count, pattern and iterations by stored entries
    nel_full = n_full ** 3 + 2 * n_full ** 2
    nnz_full = 610745670 if n_full == 64 else nnz_s * (n_full / n_sample) ** 3
    scale_nnz = nnz_full / nnz_s
    total = t_pat * scale_nnz + t_asm * nel_full / nel_s + t_it * scale_nnz * iters_full
    return total, dict(n=n_sample, t_pattern=t_pat, t_assemble=t_asm, t_cg_iter=t_it, elements=nel_s, nnz=nnz_s,
                       asm_el_per_s=nel_s / t_asm)


def cpu_baseline(iters_full, n_full):
    threads = os.cpu_count() or 1
    iters = iters_full if iters_full else JACOBI_ITERS_64_DEFAULT
    total, d = cpu_sample(12, iters, n_full, threads)
    return {"value": round(total, 2), "unit": "s", "cores": threads, "kind": "port",
            "sample": f"oracle on a {d['n']}^3 instance of the same workload: pattern {d['t_pattern']:.2f}s, "
                      f"threaded OR assembly {d['t_assemble']:.2f}s ({d['asm_el_per_s']:.0f} el/s, {threads} threads), "
                      f"{d['t_cg_iter']*1e3:.1f} ms per serial Jacobi-PCG iteration; extrapolated to {n_full}^3 by "
                      f"element count (assembly) and stored entries x {iters} FP64 Jacobi-PCG iterations (solve)"}


def run_reference(args):
    """The reference arm on the host cores, at the benchmark's own size: the oracle (the reference's algorithm
    restated and pinned to the reference library's fixtures) builds the full 64^3 system once -- the
    TPZSSpStructMatrix pattern (timed) and the TPZStructMatrixOR assembly on every host thread (timed) --
    and every step times one Jacobi-PCG iteration of it (TPZSYsmpMatrix::MultAdd is serial, the Jacobi step
    with its extra Residual SpMV, as the reference runs them).  value = pattern + assembly + the FP64
    Jacobi-PCG iteration count to 1e-8 x the median step: extrapolated in the iteration count only."""
    rank, world, local = dist_info()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    n = args.n
    E = np.exp(np.random.default_rng(SEED).standard_normal(n ** 3))
    t0 = time.perf_counter()
    m = O.elasticity3d(n, 2, E=E, body_force=(0.0, 0.0, 0.0))
    ia, ja = m.pattern(True)
    t_pattern = time.perf_counter() - t0
    t0 = time.perf_counter()
    a, f = m.assemble(True, ia, ja, nthreads=threads)
    t_asm = time.perf_counter() - t0
    for _ in range(args.warmup):  # warm-up: one SpMV each (the memory of the matrix paged in)
        O.spmv(True, ia, ja, a, f)
    its = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t1 = time.perf_counter()
        O.cg_jacobi(True, ia, ja, a, f, 1, 0.0, jacobi_residual=True)
        its.append(time.perf_counter() - t1)
    wall = time.perf_counter() - t0
    t_it = statistics.median(its)
    iters = JACOBI_ITERS_64_DEFAULT if n == 64 else None
    if iters is None:  # another size: the oracle's own count (small sizes only)
        iters = O.cg_jacobi(True, ia, ja, a, f, 200000, TOL)["iters"]
    value = t_pattern + t_asm + iters * t_it
    sample = (f"oracle at the full {n}^3 size ({len(ia) - 1} equations, {len(ja)} stored upper entries): pattern "
              f"{t_pattern:.1f} s, threaded OR assembly {t_asm:.1f} s ({m.ncel / t_asm:.0f} elements/s, {threads} "
              f"threads), {t_it:.2f} s per serial Jacobi-PCG iteration (median of {args.steps}); extrapolated to "
              f"{iters} iterations, the FP64 Jacobi-PCG count to 1e-8 of this system measured on the GB300 with the "
              "same algorithm")
    out = {"metric": METRIC, "value": round(value, 2), "unit": "s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(wall / args.steps * 1e3, 1), "higher_is_better": False,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": {"workload": f"3D linear elasticity {n}^3 hex Q2, E lognormal(sigma=1) seed {SEED}, nu=0.3, "
                                  "clamped base, top traction", "parallelism": "host threads",
                      "same_config": True},
           "cpu_baseline": {"value": round(value, 2), "unit": "s", "cores": threads, "kind": "port",
                            "sample": sample},
           "phases_s": {"pattern": round(t_pattern, 2), "assembly": round(t_asm, 2),
                        "jacobi_pcg_iteration": round(t_it, 3), "iterations": iters},
           "e2e": {"value": round(value, 2), "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# FP64 Jacobi-PCG iterations to 1e-8 of the seeded 64^3 system, measured on the
# GB300 with the FP64 parity path (same algorithm as the reference's CG + Jacobi)
JACOBI_ITERS_64_DEFAULT = 2255


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
