"""The trained learned preconditioner (sophus-rs_gb300/weights/pcg_mpnn_loop.npz,
made by sophus-rs_gb300/pcg_train.py from 1500-camera loop systems) on
held-out loop systems (seeds not used in training), against the method
without it: block-Jacobi PCG (the same network with a zero output head).

What it gains: the energy-norm error of the first preconditioned step (the
training objective) drops below block-Jacobi's on every held-out system.
What it does not: the PCG iteration count.  The loop's reduced system keeps
its global bending modes (block-Jacobi-preconditioned condition number
~1.8e7); a per-pose 6x6 correction cannot lift them, so with the cap of 50
iterations both preconditioners fall back to the exact factorization on
every solve, and the learned path's LM trajectory is the exact path's."""
import numpy as np
import pytest

from conftest import fixed_iter_params

pytestmark = pytest.mark.gpu


def _held_out(pkg, ts, seed, n_systems=2):
    prob = pkg.synth.generate(pkg.synth.LOOP, n_cam=1500, n_pt=300000, seed=seed)
    with pkg.native.Problem(prob, device=0) as gp:
        gp.init(fixed_iter_params(pkg, n_systems + 1, prob.initial_lm_damping))
        for _ in range(n_systems):
            gp.step()
            gp.collect(ts)
    return prob


def test_trained_preconditioner_on_held_out_loops(pkg):
    N = pkg.native
    held_seed = pkg.synth.BASE_SEED + 1000 + 200000  # outside the training seeds
    with N.PcgModel.load(device=0) as trained, N.PcgModel(device=0) as bj, N.PcgTrainSet(device=0) as ts:
        bj.set_params(np.zeros(N.PcgModel.num_params(), np.float32))  # L = 0: block-Jacobi
        _held_out(pkg, ts, held_seed)
        rows = []
        for i in range(len(ts)):
            lt = ts.loss_grad(trained, i, with_grad=False)
            lb = ts.loss_grad(bj, i, with_grad=False)
            it_b, rr_b, st_b = ts.evaluate(i, N.LINSOLVE_PCG_BLOCK_JACOBI, None, 50, 1e-8)
            it_l, rr_l, st_l = ts.evaluate(i, N.LINSOLVE_PCG_LEARNED, trained, 50, 1e-8)
            rows.append((lt, lb, rr_b, rr_l, st_b, st_l))
            print("system %d: one-step loss learned %.4f vs block-Jacobi %.4f; relres after 50 PCG iterations "
                  "learned %.3e vs block-Jacobi %.3e (status %d / %d)" % (i, lt, lb, rr_l, rr_b, st_l, st_b))
        for lt, lb, *_ in rows:
            assert lt < lb  # the gain in the training objective
        # both hit the cap: the exact factorization is the fallback
        assert all(st_b == 1 and st_l == 1 for *_, st_b, st_l in rows)


def test_learned_path_matches_oracle_on_a_loop(pkg, oracle):
    """LM on a 300-camera loop with the learned PCG solver: every solve falls
    back, and the trajectory is bit-identical to the exact path's (which
    matches the oracle)."""
    N = pkg.native
    prob = pkg.synth.generate(pkg.synth.LOOP, n_cam=300, n_pt=30000, seed=pkg.synth.BASE_SEED + 2)
    params = fixed_iter_params(pkg, 4, prob.initial_lm_damping)
    with N.PcgModel.load(device=0) as model:
        with N.Problem(prob, device=0) as gp:
            gp.set_linear_solver(N.LINSOLVE_PCG_LEARNED, 50, 1e-8, model)
            recs, _ = gp.optimize(params)
            st = gp.pcg_stats()
    with N.Problem(prob, device=0) as gp:
        exact, _ = gp.optimize(params)
    assert st.fallbacks == st.solves == 4
    assert [r.merit for r in recs] == [r.merit for r in exact]
