"""PCG on the reduced camera system (sgba_set_linear_solver) and the learned
block preconditioner's kernels.

  * the GPU loss and its gradient (hand-written forward and backward
    kernels, BF16 weights, FP32 arithmetic) against the FP64 restatement in
    oracle/pcg_mpnn.py on the same systems and the same BF16-rounded weights;
  * training lowers the loss;
  * with PCG the LM trajectory still matches the oracle (PCG converged
    within its cap on the sphere; on a loop it falls back to the exact
    factorization, and the trajectory is bit-identical to the exact path)."""
import os
import sys

import numpy as np
import pytest

from conftest import fixed_iter_params
from pcg_systems import random_system, scaled_system

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pcg_mpnn as M  # noqa: E402

COST_RTOL = 1e-6


def _real_system(pkg, n_cam=10, seed=5):
    prob = pkg.synth.generate(pkg.synth.LOOP, n_cam=n_cam, n_pt=40 * n_cam, seed=pkg.synth.BASE_SEED + seed)
    with pkg.native.Problem(prob, device=0) as gp:
        gp.init(fixed_iter_params(pkg, 5, prob.initial_lm_damping))
        gp.step()
        return scaled_system(gp)


def test_loss_and_gradient_match_fp64_restatement(pkg):
    N = pkg.native
    systems = [(12,) + random_system(12, seed=21), _real_system(pkg)]
    with N.PcgModel(device=0, seed=7) as model, N.PcgTrainSet(device=0) as ts:
        params = model.params()
        for k, (nf, r, c, bl, b, x) in enumerate(systems):
            ts.add(nf, r, c, bl, b, x)
            gl, gg = ts.loss_grad(model, k)
            ol, og = M.gradient(params.astype(np.float64), nf, r, c, bl, b, x, bf16=True)
            rel = np.linalg.norm(gg - og) / np.linalg.norm(og)
            print("system %d: loss gpu %.9e fp64 %.9e, gradient rel err %.2e" % (k, gl, ol, rel))
            assert abs(gl - ol) <= 1e-4 * abs(ol)
            assert rel < 2e-3
            lay, _ = M.layout()
            for name, (o, s) in lay.items():
                n = int(np.prod(s))
                ref = og[o:o + n]
                if np.linalg.norm(ref) > 1e-6 * np.linalg.norm(og):
                    assert np.linalg.norm(gg[o:o + n] - ref) <= 1e-2 * np.linalg.norm(ref), name


def test_training_lowers_the_loss(pkg):
    N = pkg.native
    with N.PcgModel(device=0, seed=3) as model, N.PcgTrainSet(device=0) as ts:
        for s in range(6):
            nf, r, c, bl, b, x = (16,) + random_system(16, seed=100 + s)
            ts.add(nf, r, c, bl, b, x)
        before = [ts.loss_grad(model, i, with_grad=False) for i in range(len(ts))]
        losses = ts.train(model, epochs=30, batch=2, learning_rate=3e-3, seed=1)
        after = [ts.loss_grad(model, i, with_grad=False) for i in range(len(ts))]
        print("mean loss before %.4e, after %.4e; epochs %s" % (np.mean(before), np.mean(after), losses[[0, -1]]))
        assert np.mean(after) < 0.9 * np.mean(before)
        # bit-reproducible training
        with N.PcgModel(device=0, seed=3) as m2:
            ts.train(m2, epochs=30, batch=2, learning_rate=3e-3, seed=1)
            assert np.array_equal(m2.params(), model.params())


@pytest.mark.parametrize("mode", [1, 2])
def test_pcg_trajectory_sphere(pkg, oracle, mode):
    """The 100-camera sphere: PCG reaches 1e-8 within 50 iterations, the
    exact factorization is skipped, and the trajectory matches the oracle."""
    N = pkg.native
    prob = pkg.synth.generate(pkg.synth.SPHERE, seed=pkg.synth.BASE_SEED + 1)
    params = fixed_iter_params(pkg, 6, prob.initial_lm_damping)
    with N.PcgModel(device=0) as model:
        with N.Problem(prob, device=0) as gp:
            gp.set_linear_solver(mode, 50, 1e-8, model if mode == 2 else None)
            recs, _ = gp.optimize(params)
            st = gp.pcg_stats()
    orecs, _, _ = oracle.optimize(prob, params, n_threads=8)
    g = np.array([r.merit for r in recs])
    o = np.array([r.merit for r in orecs])
    print("mode %d: PCG solves %d, fallbacks %d, iterations %d, dev %.2e"
          % (mode, st.solves, st.fallbacks, st.iterations, np.max(np.abs(g - o) / o)))
    assert st.solves >= 6 and st.fallbacks == 0
    assert np.max(np.abs(g - o) / o) < COST_RTOL


def test_pcg_fallback_on_loop_is_the_exact_path(pkg):
    """A 300-camera loop needs ~1.7e3 block-Jacobi PCG iterations for 1e-8:
    with a cap of 50 every solve falls back, bit-identical to the exact path."""
    N = pkg.native
    prob = pkg.synth.generate(pkg.synth.LOOP, n_cam=300, n_pt=30000, seed=pkg.synth.BASE_SEED + 2)
    params = fixed_iter_params(pkg, 4, prob.initial_lm_damping)
    with N.Problem(prob, device=0) as gp:
        exact, _ = gp.optimize(params)
    with N.Problem(prob, device=0) as gp:
        gp.set_linear_solver(1, 50, 1e-8)
        pcg, _ = gp.optimize(params)
        st = gp.pcg_stats()
    assert st.solves == 4 and st.fallbacks == 4
    assert [r.merit for r in exact] == [r.merit for r in pcg]


def test_collect_and_evaluate(pkg):
    """sgba_pcg_collect stores the scaled system and its exact solution:
    PCG on the stored system converges to it."""
    N = pkg.native
    prob = pkg.synth.generate(pkg.synth.SPHERE, seed=pkg.synth.BASE_SEED + 1)
    with N.Problem(prob, device=0) as gp, N.PcgTrainSet(device=0) as ts, N.PcgModel(device=0) as model:
        gp.init(fixed_iter_params(pkg, 5, prob.initial_lm_damping))
        gp.step()
        gp.collect(ts)
        assert len(ts) == 1
        assert ts.loss_grad(model, 0, with_grad=False) > 0.0
        it, rr, st = ts.evaluate(0, 1, max_iterations=200, tolerance=1e-10)
        print("stored sphere system: block-Jacobi PCG %d iterations, relres %.2e, status %d" % (it, rr, st))
        assert st == 0 and rr <= 1e-10
