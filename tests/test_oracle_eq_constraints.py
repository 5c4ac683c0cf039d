"""Equality constraints on the Schur path: the range-space KKT solve. The oracle
checks it on the CPU; no GPU kernel exists for it yet.

  TranslationNormConstraint  ba_scale_constraint.rs:57-100: c(T) = |t(T)| - r,
                             Jacobian under exp(x) * T; against central differences
  kkt_range_space            schur_ldlt.rs:1134-1215: the reduced KKT step
                             against a dense KKT solve (1e-9), and G dx = -c
  schur_solvers_converge     ba_scale_constraint.rs:261-287: EUCM intrinsics free,
                             only pose 0 fixed, |t(pose 1)| = r; pose and point
                             RMS < 0.1, |c| < 1e-4
  schur_matches_standard     ba_scale_constraint.rs:290-307: the same LM loop with
                             the full KKT system solved densely (the non-Schur
                             solver) follows the same trajectory
"""
import copy

import numpy as np

from test_oracle_free_intrinsics import _eucm_problem

PARAMS = dict(num_iterations=20, initial_lm_damping=1.0, function_tolerance=0.0, gradient_tolerance=0.0,
              parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)


def _scale_problem(pkg, seed):
    """BaScaleConstraintProblem::new(4, 20) (ba_scale_constraint.rs:117-121):
    the EUCM BA problem with only pose 0 fixed, and |t(pose 1)| held at its
    true norm."""
    prob, _ = _eucm_problem(pkg, seed)
    prob.pose_const[:] = 0
    prob.pose_const[0] = 1
    prob.eq_pose = np.array([1], np.int32)
    prob.eq_radius = np.array([np.linalg.norm(prob.poses_true[1, 4:])])
    return prob


def _rms(prob, poses, points):
    pose_rms = np.sqrt(np.mean(np.sum((poses[:, 4:] - prob.poses_true[:, 4:]) ** 2, axis=1)))
    pt_rms = np.sqrt(np.mean(np.sum((points - prob.points_true) ** 2, axis=1)))
    return pose_rms, pt_rms


def _dense_kkt(prob, oracle, H, b, lam):
    """[H G^T; G 0] and [b + G^T lam; -c] over the active scalars (intrinsics
    first when free, then the free poses, then the points)."""
    c, J = oracle.eq_eval(prob)
    n, m = H.shape[0], c.shape[0]
    c0 = 6 if prob.intrinsics_free else 0
    nf_idx = np.cumsum(prob.pose_const == 0) - 1
    G = np.zeros((m, n))
    for k, j in enumerate(prob.eq_pose):
        G[k, c0 + 6 * nf_idx[j]:c0 + 6 * nf_idx[j] + 6] = J[k]
    K = np.zeros((n + m, n + m))
    K[:n, :n] = H
    K[n:, :n] = G
    K[:n, n:] = G.T
    return K, np.concatenate([b + G.T @ lam, -c]), G, c


def test_translation_norm_jacobian_vs_central_differences(pkg, oracle):
    prob = _scale_problem(pkg, seed=3)
    prob.eq_pose = np.array([1, 2, 3], np.int32)
    prob.eq_radius = np.array([1.0, 2.0, 0.5])
    c, J = oracle.eq_eval(prob)
    for k, j in enumerate(prob.eq_pose):
        assert c[k] == np.linalg.norm(prob.poses[j, 4:]) - prob.eq_radius[k]
        num = np.zeros(6)
        for i in range(6):
            d = np.zeros(6)
            d[i] = 1e-6
            P = prob.poses.copy()
            P[j] = oracle.se3_mul(oracle.se3_exp(d), prob.poses[j])
            cp = oracle.eq_eval(prob, P)[0][k]
            P[j] = oracle.se3_mul(oracle.se3_exp(-d), prob.poses[j])
            cm = oracle.eq_eval(prob, P)[0][k]
            num[i] = (cp - cm) / 2e-6
        np.testing.assert_allclose(J[k], num, rtol=1e-6, atol=1e-8)
        assert np.all(J[k, :3] == 0.0)  # a rotation about the origin keeps |t| (tangent: rotation first)


def test_kkt_step_vs_dense(pkg, oracle):
    """schur_ldlt.rs:1134-1215: the range-space step equals the dense KKT solve
    and satisfies the linearised constraint G dx = -c."""
    for seed, free in ((3, True), (4, False)):
        prob = _scale_problem(pkg, seed)
        prob.intrinsics_free = free
        prob.eq_pose = np.array([1, 3], np.int32)
        prob.eq_radius = np.linalg.norm(prob.poses_true[[1, 3], 4:], axis=1) * np.array([1.02, 0.97])
        for nu, lam in ((1e-2, np.zeros(2)), (1.0, np.array([3.0, -1.5]))):
            H, b = oracle.dense_system(prob, nu)
            K, rhs, G, c = _dense_kkt(prob, oracle, H, b, lam)
            dense = np.linalg.solve(K, rhs)
            step = oracle.schur_kkt_step(prob, nu, lam)
            np.testing.assert_allclose(step, dense, rtol=1e-9, atol=1e-9 * np.abs(dense).max())
            n = H.shape[0]
            np.testing.assert_allclose(G @ step[:n], -c, rtol=1e-9, atol=1e-12)


def test_kkt_step_without_constraints_is_the_schur_step(pkg, oracle):
    prob, _ = _eucm_problem(pkg, seed=5)
    delta, _, _ = oracle.schur_step(prob, 0.3)
    np.testing.assert_array_equal(oracle.schur_kkt_step(prob, 0.3, np.zeros(0)), delta)


def test_constraint_on_a_constant_pose_is_singular(pkg, oracle):
    """G S^-1 G^T is zero when the constrained pose is constant
    (SingularKktConstraint, schur_ldlt.rs:723-728)."""
    prob = _scale_problem(pkg, seed=3)
    prob.eq_pose = np.array([0], np.int32)
    try:
        oracle.schur_kkt_step(prob, 1.0, np.zeros(1))
    except RuntimeError as e:
        assert "-2" in str(e)
    else:
        raise AssertionError("expected a singular KKT system")


def test_scale_constraint_schur_converges(pkg, oracle):
    """ba_scale_constraint.rs:261-287 (SchurBlockSparseLdlt, points Marginalized)."""
    params = pkg.OptParams(**PARAMS)
    for seed in (pkg.synth.BASE_SEED, 5):
        prob = _scale_problem(pkg, seed)
        recs, poses, points, intr = oracle.optimize(prob, params, with_intrinsics=True)
        pose_rms, pt_rms = _rms(prob, poses, points)
        assert pose_rms < 0.1 and pt_rms < 0.1, (seed, pose_rms, pt_rms)
        c, _ = oracle.eq_eval(prob, poses)
        assert abs(c[0]) < 1e-4, c  # constraint_satisfied (ba_scale_constraint.rs:210-214)
        assert recs[-1].merit < oracle.total_cost(prob)


def _clone(prob):
    P = copy.deepcopy(prob)  # keeps the attributes set on top of the synthetic problem
    P.intrinsics = np.array(prob.intrinsics, float)
    P.eucm_alpha_beta = np.array(prob.eucm_alpha_beta, float)
    return P


def _standard_lm(prob, oracle, n_iter, nu):
    """The LM loop of step_nlls_inner (optimizer_step.rs:365-430) with the full
    KKT system solved densely, as the non-Schur solvers do: returns the merit
    after each step and the final poses and points."""
    P = _clone(prob)
    lam = np.zeros(len(prob.eq_pose))
    merit = oracle.total_cost(P)
    merits = []
    free = [j for j in range(P.n_cam) if not P.pose_const[j]]
    for _ in range(n_iter):
        H, b = oracle.dense_system(P, nu)
        K, rhs, _, _ = _dense_kkt(P, oracle, H, b, lam)
        delta = np.linalg.solve(K, rhs)
        n = H.shape[0]
        T = _clone(P)
        T.intrinsics = P.intrinsics + delta[:4]
        T.eucm_alpha_beta = P.eucm_alpha_beta + delta[4:6]
        T.poses = P.poses.copy()
        for i, j in enumerate(free):
            T.poses[j] = oracle.se3_mul(oracle.se3_exp(delta[6 + 6 * i:12 + 6 * i]), P.poses[j])
        T.points = P.points + delta[6 + 6 * len(free):n].reshape(-1, 3)
        new = oracle.total_cost(T)
        pred = nu * delta @ delta + delta @ rhs  # compute_gain_ratio (optimizer_helpers.rs:159-173)
        rho = (merit - new) / pred
        if rho > 0 and new < merit:
            nu *= max(1.0 - (2.0 * rho - 1.0) ** 3, 1.0 / 3.0)
            P, merit = T, new
            lam = lam - delta[n:]
        else:
            nu *= 2.0
        merits.append(merit)
    return np.array(merits), P.poses, P.points


def test_scale_constraint_schur_matches_standard(pkg, oracle):
    """ba_scale_constraint.rs:290-307, held tighter: the Schur KKT path and
    the dense KKT path agree step by step."""
    prob = _scale_problem(pkg, pkg.synth.BASE_SEED)
    n_iter = 12
    params = pkg.OptParams(**dict(PARAMS, num_iterations=n_iter))
    recs, poses, points, _ = oracle.optimize(prob, params, with_intrinsics=True)
    merits, dposes, dpoints = _standard_lm(prob, oracle, n_iter, 1.0)
    np.testing.assert_allclose([r.merit for r in recs], merits, rtol=1e-9)
    np.testing.assert_allclose(poses, dposes, rtol=0, atol=1e-9)
    np.testing.assert_allclose(points, dpoints, rtol=0, atol=1e-9)
