"""A second cost function on the Schur path: Isometry3PriorCostTerm
(isometry3_prior.rs), in the oracle. No GPU kernel exists for it yet.

  SE(3) log          affine_group_template.rs:362-370, rotation3.rs:389-410,778-800:
                     log(exp(xi)) = xi on both branches
  prior Jacobian     the dual-number derivative of log(exp(x) T E^-1) at x = 0,
                     against central differences
  assembly           evaluated_term.rs:286-327 (J^T W J, J^T W g, g^T W g),
                     cost_system.rs:229-236 (nu I once per reduced term)
  optimize_with_priors  cam_calib.rs:249-342: all poses free, the gauge held by
                     priors (precision 1e4 I) on poses 0 and 1 at the truth;
                     |t(pose 2) - t_true| < 0.1 after 10 iterations
"""
import copy

import numpy as np

from test_oracle_reference import project_true


def _quat(axis, angle):
    axis = np.asarray(axis, float) / np.linalg.norm(axis)
    return np.concatenate([[np.cos(angle / 2)], np.sin(angle / 2) * axis])


def _spd(rng, scale=1.0):
    A = rng.standard_normal((6, 6))
    return scale * (A @ A.T + 6 * np.eye(6))


def test_se3_log_inverts_exp(oracle):
    rng = np.random.default_rng(0)
    cases = [np.zeros(6), np.array([1e-8, -2e-8, 3e-9, 0.1, 0.2, -0.3]), np.array([0.0, 0.0, 2.5, 1.0, -2.0, 0.5])]
    cases += [rng.standard_normal(6) * s for s in (1e-4, 0.3, 1.0)]
    for xi in cases:
        np.testing.assert_allclose(oracle.se3_log(oracle.se3_exp(xi)), xi, rtol=1e-9, atol=1e-12)
    for _ in range(5):
        T = np.concatenate([_quat(rng.standard_normal(3), rng.uniform(0, 3.0)), rng.standard_normal(3)])
        np.testing.assert_allclose(oracle.se3_exp(oracle.se3_log(T)), T, rtol=1e-12, atol=1e-12)


def test_prior_residual_and_jacobian(oracle):
    rng = np.random.default_rng(1)
    for _ in range(6):
        mean = np.concatenate([_quat(rng.standard_normal(3), rng.uniform(0, 2.0)), rng.standard_normal(3)])
        pose = oracle.se3_mul(oracle.se3_exp(0.2 * rng.standard_normal(6)), mean)
        W = _spd(rng)
        r, J, cost = oracle.eval_prior(pose, mean, W)
        np.testing.assert_allclose(r, oracle.se3_log(oracle.se3_mul(pose, oracle.se3_inverse(mean))), atol=1e-15)
        np.testing.assert_allclose(cost, r @ W @ r, rtol=1e-13)
        h = 1e-6
        for k in range(6):
            d = np.zeros(6)
            d[k] = h
            rp = oracle.eval_prior(oracle.se3_mul(oracle.se3_exp(d), pose), mean, W)[0]
            rm = oracle.eval_prior(oracle.se3_mul(oracle.se3_exp(-d), pose), mean, W)[0]
            np.testing.assert_allclose(J[:, k], (rp - rm) / (2 * h), rtol=1e-6, atol=1e-8)
    r, J, cost = oracle.eval_prior(mean, mean, W)
    assert np.abs(r).max() < 1e-15 and cost < 1e-28
    np.testing.assert_allclose(J, np.eye(6), atol=1e-12)  # d log(exp(x)) / dx = I at the identity


def _with_priors(prob, poses, means, Ws):
    P = copy.deepcopy(prob)
    P.prior_pose = np.array(poses, np.int32)
    P.prior_mean = np.array(means, float)
    P.prior_precision = np.array(Ws, float)
    return P


def test_prior_assembly_in_the_normal_equations(pkg, oracle):
    """H and the gradient gain J^T W J (+ nu I once per pose, however many
    priors it has) and -J^T W g on the pose's block; a constant pose gains
    nothing; the total cost gains g^T W g."""
    rng = np.random.default_rng(2)
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=5, n_pt=40, seed=3)
    prob.pose_const = np.zeros(5, np.uint8)
    prob.pose_const[4] = 1
    means = [oracle.se3_mul(oracle.se3_exp(0.05 * rng.standard_normal(6)), prob.poses[j]) for j in (2, 0, 2, 4)]
    Ws = [_spd(rng, 10.0) for _ in range(4)]
    pp = _with_priors(prob, [2, 0, 2, 4], means, Ws)
    nu = 0.5
    H0, b0 = oracle.dense_system(prob, nu)
    H1, b1 = oracle.dense_system(pp, nu)
    dH, db = H1 - H0, b1 - b0
    expect_H, expect_b, cost = np.zeros_like(dH), np.zeros_like(db), 0.0
    for j, (k_list) in ((0, [1]), (2, [0, 2]), (4, [3])):
        for k in k_list:
            r, J, c = oracle.eval_prior(prob.poses[j], means[k], Ws[k])
            cost += c
            if j == 4:
                continue  # constant pose: no block
            o = 6 * j  # poses 0..3 are free, in order
            expect_H[o:o + 6, o:o + 6] += J.T @ Ws[k] @ J
            expect_b[o:o + 6] -= J.T @ Ws[k] @ r
        if j != 4:
            expect_H[6 * j:6 * j + 6, 6 * j:6 * j + 6] += nu * np.eye(6)
    scale = np.abs(expect_H).max()
    np.testing.assert_allclose(dH, expect_H, rtol=0, atol=1e-9 * scale)
    np.testing.assert_allclose(db, expect_b, rtol=0, atol=1e-9 * max(1.0, np.abs(expect_b).max()))
    np.testing.assert_allclose(oracle.total_cost(pp) - oracle.total_cost(prob), cost, rtol=1e-9)
    # the Schur path solves the system with the priors in it
    dense = np.linalg.solve(H1, b1)
    delta, _, _ = oracle.schur_step(pp, nu)
    np.testing.assert_allclose(delta, dense, rtol=1e-9, atol=1e-9 * np.abs(dense).max())


def test_optimize_with_priors(pkg, oracle):
    """cam_calib.rs:249-342 on the Schur path (points Marginalized): no pose is
    constant; priors with precision 1e4 I on poses 0 and 1 at the truth hold
    the gauge; the reference asserts |t(pose 2) - t_true(pose 2)| < 0.1."""
    params = pkg.OptParams(num_iterations=10, initial_lm_damping=1.0, function_tolerance=0.0, gradient_tolerance=0.0,
                           parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)
    for seed in (pkg.synth.BASE_SEED, 5):
        prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=5, n_pt=40, seed=seed)
        prob.obs_uv = project_true(prob) + (np.random.default_rng(seed).random(prob.obs_uv.shape) - 0.5)
        prob.pose_const = np.zeros(prob.n_cam, np.uint8)
        pp = _with_priors(prob, [0, 1], prob.poses_true[:2], [1e4 * np.eye(6)] * 2)
        recs, poses, points = oracle.optimize(pp, params)
        err = np.abs(poses[2, 4:] - prob.poses_true[2, 4:]).max()
        assert err < 0.1, (seed, err)
        # the priors hold poses 0 and 1 near the truth, and the fit improved
        assert np.abs(poses[:2, 4:] - prob.poses_true[:2, 4:]).max() < 0.01
        assert recs[-1].merit < 0.1 * oracle.total_cost(pp)
