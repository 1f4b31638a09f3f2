"""Training driver of the learned preconditioner.

The work runs on the GPU, in the library's own kernels (libgpz.so): Jacobi-PCG
solves that produce the residual / error pairs, and the network's forward,
backward and Adam steps.  This module only loops over coefficient fields:
for every seed it sets the field (gpz_mesh_set_coef), assembles, collects
pairs from the Jacobi-PCG iterates (gpz_learned_collect) and takes a few
Adam steps on them (gpz_learned_train).

    python -m neopz_gb300.learned --workload darcy2d --n 256 --fields 2000 \
        --out neopz_gb300/data/learned_darcy2d_q2.npy

The saved file holds the float32 parameter vector in the layout of
gpz_learned.cu; `Context.set_learned_params` loads it into a context whose
mesh has the same element type, order and state count.
"""
import argparse
import json
import os
import time

import numpy as np

from . import gpz

HERE = os.path.dirname(os.path.abspath(__file__))
DATA = os.path.join(HERE, "data")


def darcy2d(n, p=2):
    """C4-type workload: -div(k grad u) = 1 on the unit square, k = exp(GRF, sigma 1.5, correlation 0.1)."""
    grid = gpz.darcy(2, n, p, gpz.grf2d(n, seed=0))
    return grid, (lambda seed: gpz.grf2d(n, seed=seed))


def elasticity3d(n, p=2):
    """C5-type workload: 3D elasticity, E lognormal (sigma 1) per element, nu 0.3, clamped base, top traction."""
    grid = gpz.elasticity3d(n, p, E=gpz.lognormal(n ** 3, 1.0, 0), nu=0.3, body_force=(0.0, 0.0, 0.0))
    return grid, (lambda seed: gpz.lognormal(n ** 3, 1.0, seed))


WORKLOADS = {"darcy2d": darcy2d, "elasticity3d": elasticity3d}


def context_for(grid, rank=4, seed=0, params=None):
    ctx = gpz.Context(0)
    ctx.upload_mesh(grid)
    ctx.build_pattern(False)
    ctx.assemble()
    ctx.learned_init(rank=rank, seed=seed)
    if params is not None:
        ctx.set_learned_params(params)
    return ctx


def validate(ctx, grid, coef_of_seed, seeds, tol=1e-8, base=gpz.GPZ_PRECOND_JACOBI):
    """Learned flexible-CG iterations summed over validation fields: the FP64 solver on the Jacobi base, the
    mixed one (FP32 operator) on a block base, which only it applies."""
    its = 0
    for s in seeds:
        ctx.set_coef(grid, coef_of_seed(s))
        if base == gpz.GPZ_PRECOND_JACOBI:
            ctx.assemble()
            its += ctx.solve(solver=gpz.GPZ_SOLVER_LEARNED_FCG, tol=tol, want_x=False)["iterations"]
        else:
            ctx.assemble(gpz.GPZ_PREC_MIXED)
            its += ctx.solve(solver=gpz.GPZ_SOLVER_LEARNED_MIXED_FCG, precond=base, tol=tol, reliable_delta=1e-2,
                             want_x=False)["iterations"]
    return its


def train(ctx, grid, coef_of_seed, seeds, steps=8, lr=3e-3, npairs=16, tol=1e-12, log_every=0, lr_final=None,
          val_seeds=(20000, 20001), val_every=50, base=gpz.GPZ_PRECOND_JACOBI):
    """Online training over the fields of `seeds` (learning rate decayed from lr to lr_final on a cosine).

    The energy-norm loss flattens early while the parameters can keep drifting in directions that
    lengthen the Krylov iteration, so every `val_every` fields the learned flexible CG is run on the
    validation fields and the parameters with the fewest iterations are kept (restored at the end).
    Returns (first loss, last loss, seconds, validation history)."""
    import math
    seeds = list(seeds)
    lr_final = lr / 10 if lr_final is None else lr_final
    t0 = time.time()
    first = last = None
    history = []
    best = None
    ctx.learned_set_base(base)
    for i, s in enumerate(seeds):
        ctx.set_coef(grid, coef_of_seed(s))
        ctx.assemble(gpz.GPZ_PREC_FP64 if base == gpz.GPZ_PRECOND_JACOBI else gpz.GPZ_PREC_MIXED)
        ctx.learned_collect(npairs=npairs, tol=tol)
        li = lr_final + (lr - lr_final) * 0.5 * (1 + math.cos(math.pi * i / max(1, len(seeds) - 1)))
        l0, l1 = ctx.learned_train(steps=steps, lr=li)
        first = l0 if first is None else first
        last = l1
        done = i + 1
        if val_seeds and (done % val_every == 0 or done == len(seeds)):
            its = validate(ctx, grid, coef_of_seed, val_seeds, base=base)
            history.append({"fields": done, "validation_iterations": its, "loss": l1})
            if best is None or its < best[0]:
                best = (its, ctx.learned_params(), done)
        if log_every and done % log_every == 0:
            print(json.dumps({"fields": done, "loss": l1, "seconds": round(time.time() - t0, 1),
                              "validation": history[-1] if history else None}), flush=True)
    if best is not None:
        # set_learned_params also clears the Adam moments: a later train() call starts afresh from here
        ctx.set_learned_params(best[1])
        history.append({"kept_fields": best[2], "validation_iterations": best[0]})
    return first, last, time.time() - t0, history


def evaluate(ctx, grid, coef_of_seed, seeds, tol=1e-8, precond=gpz.GPZ_PRECOND_JACOBI):
    """Jacobi-PCG (or block Jacobi) against the learned flexible CG on the fields of `seeds`."""
    out = []
    for s in seeds:
        ctx.set_coef(grid, coef_of_seed(s))
        ctx.assemble()
        base = ctx.solve(tol=tol, precond=precond, want_x=False)
        lrn = ctx.solve(solver=gpz.GPZ_SOLVER_LEARNED_FCG, tol=tol, want_x=False)
        # learned + the FP32 operator (FP32 CSR for scalar problems; the autotuned 3x3-block or
        # matrix-free operator for elasticity, which needs a mixed assembly)
        if grid.desc.nstate == 3:
            ctx.assemble(gpz.GPZ_PREC_MIXED)
        m = ctx.solve(solver=gpz.GPZ_SOLVER_LEARNED_MIXED_FCG, tol=tol, reliable_delta=1e-2, want_x=False)
        mixed = dict(learned_mixed_iterations=m["iterations"], learned_mixed_seconds=m["seconds"],
                     learned_mixed_true_resid=m["true_resid"], learned_mixed_rc=m["rc"])
        out.append(dict(seed=s, base_precond="block_jacobi" if precond == gpz.GPZ_PRECOND_BLOCK_JACOBI else "jacobi",
                        **mixed,
                        base_iterations=base["iterations"], base_seconds=base["seconds"],
                        learned_iterations=lrn["iterations"], learned_seconds=lrn["seconds"],
                        learned_true_resid=lrn["true_resid"], fallbacks=lrn["restarts"], rc=lrn["rc"]))
    return out


def evaluate_mixed(ctx, grid, coef_of_seed, seeds, base, tol=1e-8):
    """The mixed CG on `base` against the learned + mixed flexible CG on the same base (the method without the
    network against the method with it), same FP32 operator, same true FP64 residual."""
    out = []
    for s in seeds:
        ctx.set_coef(grid, coef_of_seed(s))
        ctx.assemble(gpz.GPZ_PREC_MIXED)
        kw = dict(tol=tol, reliable_delta=1e-2, want_x=False)
        for _ in range(2):  # the second of each is timed (graphs instantiated, caches warm)
            b = ctx.solve(solver=gpz.GPZ_SOLVER_MIXED_CG, precond=base, **kw)
            m = ctx.solve(solver=gpz.GPZ_SOLVER_LEARNED_MIXED_FCG, precond=base, **kw)
        out.append(dict(seed=s, base_iterations=b["iterations"], base_seconds=b["seconds"],
                        learned_iterations=m["iterations"], learned_seconds=m["seconds"],
                        learned_true_resid=m["true_resid"], fallbacks=m["restarts"], rc=m["rc"]))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="darcy2d")
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--p", type=int, default=2)
    ap.add_argument("--fields", type=int, default=2000, help="training fields (seeds 1..fields)")
    ap.add_argument("--steps", type=int, default=8, help="Adam steps per field")
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--pairs", type=int, default=16)
    ap.add_argument("--rank", type=int, default=4)
    ap.add_argument("--init-seed", type=int, default=0)
    ap.add_argument("--eval", type=int, default=5, help="evaluation fields (seeds 10000..)")
    ap.add_argument("--eval-n", type=int, default=0, help="evaluate on another grid size (0: the training size)")
    ap.add_argument("--block", action="store_true", help="also evaluate against block-Jacobi PCG")
    ap.add_argument("--val-every", type=int, default=50, help="validation (checkpoint selection) interval in fields")
    ap.add_argument("--weights", default="", help="start from these parameters (with --fields 0: evaluate only)")
    ap.add_argument("--base", choices=["jacobi", "block", "two_level"], default="jacobi",
                    help="base preconditioner under the correction (block bases: the mixed solver, elasticity)")
    ap.add_argument("--out", default="")
    a = ap.parse_args(argv)
    grid, coef = WORKLOADS[a.workload](a.n, a.p)
    ctx = context_for(grid, a.rank, a.init_seed, np.load(a.weights) if a.weights else None)
    first = last = None
    secs, hist = 0.0, []
    base = {"jacobi": gpz.GPZ_PRECOND_JACOBI, "block": gpz.GPZ_PRECOND_BLOCK_JACOBI,
            "two_level": gpz.GPZ_PRECOND_TWO_LEVEL}[a.base]
    if a.fields > 0:
        first, last, secs, hist = train(ctx, grid, coef, range(1, a.fields + 1), a.steps, a.lr, a.pairs,
                                        log_every=max(1, a.fields // 10), val_every=a.val_every, base=base)
    params = ctx.learned_params()
    if a.out:
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        np.save(a.out, params)
    res = dict(workload=a.workload, n=a.n, p=a.p, fields=a.fields, steps=a.steps, lr=a.lr, pairs=a.pairs,
               rank=a.rank, base=a.base, loss_first=first, loss_last=last, train_seconds=round(secs, 1),
               validation=hist)
    if a.eval:
        if a.eval_n and a.eval_n != a.n:
            ctx.close()
            grid, coef = WORKLOADS[a.workload](a.eval_n, a.p)
            ctx = context_for(grid, a.rank, a.init_seed, params)
        if base == gpz.GPZ_PRECOND_JACOBI:
            res["eval"] = evaluate(ctx, grid, coef, range(10000, 10000 + a.eval))
        else:
            res["eval"] = evaluate_mixed(ctx, grid, coef, range(10000, 10000 + a.eval), base)
        if a.block:
            res["eval_block"] = evaluate(ctx, grid, coef, range(10000, 10000 + a.eval),
                                         precond=gpz.GPZ_PRECOND_BLOCK_JACOBI)
    ctx.close()
    print(json.dumps(res), flush=True)
    return res


if __name__ == "__main__":
    main()
