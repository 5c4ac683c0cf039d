"""The oracle with Free pinhole intrinsics (family kinds (F, F, M)): the first
step of the scope table's next row (free intrinsics), checked on the CPU
before any GPU kernel exists for it.

  J_cam         pinhole_reprojection.rs:85 (-dx_distort_params, affine.rs:77-108)
                against central differences of the residual
  schur_vs_dense   schur_ldlt.rs:1083-1127 (1e-9), with the intrinsics block
  ba_converges  ba_problem.rs:517-547: free intrinsics started 1 % off, poses
                0 and 1 fixed; pose RMS < 0.01, point RMS < 0.1
"""
import numpy as np

from test_oracle_reference import project_true


def _problem(pkg, seed, free=True):
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=4, n_pt=20, seed=seed)
    prob.obs_uv = project_true(prob) + 0.15 * (np.random.default_rng(2).random(prob.obs_uv.shape) - 0.5)
    prob.poses[:2] = prob.poses_true[:2]  # poses 0 and 1 fixed at the truth (no gauge left)
    prob.pose_const[:2] = 1
    truth = np.array(prob.intrinsics, float)
    prob.intrinsics = truth * np.array([0.99, 0.99, 1.0, 1.0]) + np.array([0.0, 0.0, 1.0, 1.0])
    cond = prob.copy()  # the same problem with the intrinsics Conditioned
    prob.intrinsics_free = free
    return prob, cond, truth


def test_intrinsics_jacobian_vs_central_differences(pkg, oracle):
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=5, n_pt=40, seed=3)
    intr = np.array(prob.intrinsics, float)
    for o in range(0, prob.n_obs, max(1, prob.n_obs // 25)):
        pose, pt, uv = prob.poses[prob.obs_cam[o]], prob.points[prob.obs_pt[o]], prob.obs_uv[o]
        J = oracle.eval_term_intrinsics(pose, pt, intr)
        num = np.zeros((2, 4))
        for k in range(4):
            h = 1e-6 * max(1.0, abs(intr[k]))
            ip, im = intr.copy(), intr.copy()
            ip[k] += h
            im[k] -= h
            rp = oracle.eval_term(pose, pt, ip, uv, 0.0)[0]
            rm = oracle.eval_term(pose, pt, im, uv, 0.0)[0]
            num[:, k] = (rp - rm) / (2 * h)
        np.testing.assert_allclose(J, num, rtol=1e-6, atol=1e-8)


def test_free_intrinsics_schur_vs_dense(pkg, oracle):
    prob, _, _ = _problem(pkg, seed=3)
    for nu in (1e-2, 1.0):
        H, b = oracle.dense_system(prob, nu)
        nf = int(np.sum(prob.pose_const == 0))
        assert H.shape[0] == 4 + 6 * nf + 3 * prob.n_pt  # intrinsics first
        dense = np.linalg.solve(H, b)
        delta, S, rhs = oracle.schur_step(prob, nu)
        np.testing.assert_allclose(delta, dense, rtol=1e-9, atol=1e-9 * np.abs(dense).max())


def test_free_intrinsics_ba_converges(pkg, oracle):
    params = pkg.OptParams(num_iterations=20, initial_lm_damping=1.0, function_tolerance=0.0, gradient_tolerance=0.0,
                           parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)
    for seed in (pkg.synth.BASE_SEED, 5):
        prob, cond, truth = _problem(pkg, seed)
        recs, poses, points, intr = oracle.optimize(prob, params, with_intrinsics=True)
        pose_rms = np.sqrt(np.mean(np.sum((poses[:, 4:] - prob.poses_true[:, 4:]) ** 2, axis=1)))
        pt_rms = np.sqrt(np.mean(np.sum((points - prob.points_true) ** 2, axis=1)))
        assert pose_rms < 0.01 and pt_rms < 0.1, (seed, pose_rms, pt_rms)
        # the intrinsics moved (fx towards the truth) and the fit is far better
        # than with them held Conditioned at the perturbed start
        assert abs(intr[0] - truth[0]) < 0.25 * abs(prob.intrinsics[0] - truth[0])
        rc, _, _, intr_c = oracle.optimize(cond, params, with_intrinsics=True)
        np.testing.assert_array_equal(intr_c, cond.intrinsics)
        assert recs[-1].merit < 0.2 * rc[-1].merit


def test_conditioned_intrinsics_stay_fixed(pkg, oracle):
    """With the flag off nothing about the intrinsics changes (the path the GPU
    implements); the trajectory equals the one without the flag set at all."""
    prob, cond, _ = _problem(pkg, seed=7, free=False)
    params = pkg.OptParams(num_iterations=6, initial_lm_damping=1.0, function_tolerance=0.0, gradient_tolerance=0.0,
                           parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)
    a, pa, qa, ia = oracle.optimize(prob, params, with_intrinsics=True)
    b, pb, qb = oracle.optimize(cond, params)
    assert [r.merit for r in a] == [r.merit for r in b]
    np.testing.assert_array_equal(pa, pb)
    np.testing.assert_array_equal(ia, prob.intrinsics)
