#!/usr/bin/env python3
"""Train the learned block preconditioner of the PCG reduced-system solver.

Training data: reduced camera systems of loop-shaped bundle adjustments (the
1500-camera loop generator, one seed per scene) and their exact solutions,
produced by this library's exact solver during LM runs (sgba_pcg_collect: the
Jacobi-scaled system of each LM step and its solution by the float-float band
LDL^T).  Training: Adam on the energy-norm error of one preconditioned step
(sgba_pcg_train; forward and backward are the library's CUDA kernels).  The
result is written as an .npz holding the FP32 parameters and a summary of the
held-out evaluation (PCG iterations and residuals with block-Jacobi and with
the learned correction on scenes not used for training).

    python sophus-rs_gb300/pcg_train.py --out sophus-rs_gb300/weights/pcg_mpnn_loop.npz
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def fixed(pkg, n, nu):
    return pkg.OptParams(num_iterations=n, initial_lm_damping=nu, function_tolerance=0.0, gradient_tolerance=0.0,
                         parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)


def collect(pkg, ts, seeds, n_cam, n_pt, per_seed, log):
    N = pkg.native
    for s in seeds:
        t0 = time.perf_counter()
        prob = pkg.synth.generate(pkg.synth.LOOP, n_cam=n_cam, n_pt=n_pt, seed=s)
        with N.Problem(prob, device=0) as gp:
            gp.init(fixed(pkg, per_seed + 1, prob.initial_lm_damping))
            for _ in range(per_seed):
                gp.step()
                gp.collect(ts)
        log("seed %d: %d systems (%.1f s), set size %d" % (s, per_seed, time.perf_counter() - t0, len(ts)))


def evaluate(pkg, ts, model, cap, tol, big_cap):
    N = pkg.native
    out = {"block_jacobi": [], "learned": []}
    for i in range(len(ts)):
        for name, mode, m in (("block_jacobi", N.LINSOLVE_PCG_BLOCK_JACOBI, None),
                              ("learned", N.LINSOLVE_PCG_LEARNED, model)):
            it, rr, st = ts.evaluate(i, mode, m, max_iterations=cap, tolerance=tol)
            it_big, rr_big, st_big = ts.evaluate(i, mode, m, max_iterations=big_cap, tolerance=tol)
            out[name].append({"relres_at_cap": rr, "converged_at_cap": st == 0,
                              "iterations_to_tol": it_big if st_big == 0 else None, "relres_big": rr_big})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "weights", "pcg_mpnn_loop.npz"))
    ap.add_argument("--n-cam", type=int, default=1500)
    ap.add_argument("--n-pt", type=int, default=300000)
    ap.add_argument("--train-seeds", type=int, default=100)
    ap.add_argument("--per-seed", type=int, default=20)
    ap.add_argument("--test-seeds", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--cap", type=int, default=50)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--big-cap", type=int, default=20000)
    args = ap.parse_args()

    import __graft_entry__ as graft

    pkg = graft.load_package()
    N = pkg.native
    log = lambda m: print(m, flush=True)  # noqa: E731
    base = pkg.synth.BASE_SEED + 1000
    train_seeds = [base + i for i in range(args.train_seeds)]
    test_seeds = [base + 100000 + i for i in range(args.test_seeds)]
    with N.PcgTrainSet(device=0) as ts, N.PcgTrainSet(device=0) as held, N.PcgModel(device=0, seed=1) as model:
        collect(pkg, ts, train_seeds, args.n_cam, args.n_pt, args.per_seed, log)
        collect(pkg, held, test_seeds, args.n_cam, args.n_pt, 3, log)
        held_before = [held.loss_grad(model, i, with_grad=False) for i in range(len(held))]
        t0 = time.perf_counter()
        losses = ts.train(model, epochs=args.epochs, batch=args.batch, learning_rate=args.lr, seed=2)
        train_s = time.perf_counter() - t0
        log("training: %d systems x %d epochs in %.1f s; epoch losses %s" % (len(ts), args.epochs, train_s,
                                                                            np.array2string(losses, precision=4)))
        held_after = [held.loss_grad(model, i, with_grad=False) for i in range(len(held))]
        ev = evaluate(pkg, held, model, args.cap, args.tol, args.big_cap)
        summary = {
            "train_systems": len(ts), "train_seeds": args.train_seeds, "systems_per_seed": args.per_seed,
            "n_cam": args.n_cam, "n_pt": args.n_pt, "epochs": args.epochs, "batch": args.batch, "lr": args.lr,
            "train_seconds": train_s, "epoch_loss": losses.tolist(),
            "held_out_systems": len(held), "held_out_loss_untrained": float(np.mean(held_before)),
            "held_out_loss_trained": float(np.mean(held_after)), "cap": args.cap, "tol": args.tol,
            "evaluation": ev,
        }
        log(json.dumps({k: v for k, v in summary.items() if k != "evaluation"}))
        for name in ("block_jacobi", "learned"):
            its = [e["iterations_to_tol"] for e in ev[name]]
            rr = [e["relres_at_cap"] for e in ev[name]]
            log("%s: iterations to %.0e %s; relres after %d: median %.3e; converged within the cap: %d/%d"
                % (name, args.tol, its, args.cap, float(np.median(rr)),
                   sum(e["converged_at_cap"] for e in ev[name]), len(ev[name])))
        os.makedirs(os.path.dirname(args.out), exist_ok=True)
        np.savez(args.out, params=model.params(), summary=json.dumps(summary))
        log("wrote %s" % args.out)


if __name__ == "__main__":
    main()
