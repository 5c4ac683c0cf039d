"""The CPU oracle against restatements of the reference's own tests.

sophus-rs ships no golden vectors for this path; its tests are tolerance
tests, restated here with the reference's tolerances:
  Lie Jacobians        crates/sophus_lie/src/lie_group/real_lie_group.rs:340-390
  schur_vs_dense       crates/sophus_solver/src/ldlt/schur_ldlt.rs:1083-1127 (1e-9)
  parallel_vs_seq      crates/sophus_solver/src/ldlt/schur_ldlt.rs:1214-1253
  simple_cam_tests     crates/sophus_opt/src/example_problems/cam_calib.rs:348-365 (0.1)
  ba_converges         crates/sophus_opt/src/example_problems/ba_problem.rs:517-547 (0.01 / 0.1)
plus closed-form known answers for the SE(3) group operations.
"""
import math

import numpy as np
import pytest

from conftest import fixed_iter_params


def _quat_z(theta):
    return np.array([math.cos(theta / 2), 0.0, 0.0, math.sin(theta / 2)])


def test_se3_exp_known_answers(oracle):
    # exp(0) = identity
    np.testing.assert_array_equal(oracle.se3_exp(np.zeros(6)), [1, 0, 0, 0, 0, 0, 0])
    # pure rotation about z by 0.7 rad
    e = oracle.se3_exp([0, 0, 0.7, 0, 0, 0])
    np.testing.assert_allclose(e[:4], _quat_z(0.7), atol=1e-15)
    np.testing.assert_allclose(e[4:], 0.0, atol=1e-15)
    # pure translation: V(0) = I
    e = oracle.se3_exp([0, 0, 0, 1.0, -2.0, 0.5])
    np.testing.assert_allclose(e, [1, 0, 0, 0, 1.0, -2.0, 0.5], atol=1e-15)
    # rotation about z with translation along x: V(w) nu = [sin t/t, (1-cos t)/t, 0] for nu = e_x
    t = 0.9
    e = oracle.se3_exp([0, 0, t, 1.0, 0, 0])
    np.testing.assert_allclose(e[4:], [math.sin(t) / t, (1 - math.cos(t)) / t, 0.0], atol=1e-14)


def test_se3_group_axioms(oracle):
    rng = np.random.default_rng(0)
    for _ in range(20):
        a = oracle.se3_exp(rng.normal(size=6))
        b = oracle.se3_exp(rng.normal(size=6))
        ident = oracle.se3_mul(a, oracle.se3_inverse(a))
        np.testing.assert_allclose(ident, [1, 0, 0, 0, 0, 0, 0], atol=1e-14)
        assert ident[0] >= 0.0  # disambiguated
        ab = oracle.se3_mul(a, b)
        abi = oracle.se3_mul(oracle.se3_inverse(b), oracle.se3_inverse(a))
        np.testing.assert_allclose(oracle.se3_mul(ab, abi), [1, 0, 0, 0, 0, 0, 0], atol=1e-13)


def test_exp_taylor_branches_are_continuous(oracle):
    # rotation3.rs:363-387 (theta^2 <= EPS^2) and mat_v :761-778 (theta^2 <= EPS)
    for th in (0.9e-6, 1.1e-6, 0.99e-3, 1.01e-3):
        w = np.array([th, 0.0, 0.0])
        e = oracle.se3_exp(np.concatenate([w, [0.3, 0.2, 0.1]]))
        assert abs(np.linalg.norm(e[:4]) - 1.0) < 1e-12
        np.testing.assert_allclose(e[1], math.sin(th / 2), rtol=1e-9)


def _random_term(rng):
    pose = np.concatenate([[1, 0, 0, 0], [0, 0, 0]])
    pose = np.array(pose, dtype=float)
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    pose[:4] = q if q[0] >= 0 else -q
    pose[4:] = rng.normal(size=3)
    # a point in front of the camera
    R = _rot(pose[:4])
    p_cam = np.array([rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(3, 8)])
    p_world = R @ p_cam + pose[4:]
    return pose, p_world


def _rot(q):
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def test_reprojection_jacobians_vs_dual_and_finite_difference(oracle):
    """dx_exp_x_times_point_at_0-based analytic Jacobians == dual numbers ==
    symmetric finite differences (real_lie_group.rs:340-390; tolerance 1e-3 there)."""
    rng = np.random.default_rng(1)
    intr = np.array([500.0, 480.0, 320.0, 240.0])
    for _ in range(25):
        pose, pw = _random_term(rng)
        uv = rng.uniform([0, 0], [640, 480])
        r, jp, jm, w, c = oracle.eval_term(pose, pw, intr, uv, 0.0)
        djp, djm = oracle.eval_term_dual(pose, pw, intr, uv)
        np.testing.assert_allclose(jp, djp, rtol=1e-10, atol=1e-9)
        np.testing.assert_allclose(jm, djm, rtol=1e-10, atol=1e-9)
        h = 1e-6
        fd_p = np.zeros((2, 6))
        for k in range(6):
            xi = np.zeros(6)
            xi[k] = h
            rp = oracle.eval_term(oracle.se3_mul(oracle.se3_exp(xi), pose), pw, intr, uv, 0.0)[0]
            rm = oracle.eval_term(oracle.se3_mul(oracle.se3_exp(-xi), pose), pw, intr, uv, 0.0)[0]
            fd_p[:, k] = (rp - rm) / (2 * h)
        fd_m = np.zeros((2, 3))
        for k in range(3):
            d = np.zeros(3)
            d[k] = h
            fd_m[:, k] = (oracle.eval_term(pose, pw + d, intr, uv, 0.0)[0] -
                          oracle.eval_term(pose, pw - d, intr, uv, 0.0)[0]) / (2 * h)
        np.testing.assert_allclose(jp, fd_p, rtol=1e-3, atol=1e-3)
        np.testing.assert_allclose(jm, fd_m, rtol=1e-3, atol=1e-3)


def test_huber_weight_and_cost(oracle):
    """robust_kernel.rs: w = sqrt(rho(|r|)) / |r|, cost = rho(|r|), no 1/2."""
    pose = np.array([1, 0, 0, 0, 0, 0, 0], float)
    intr = np.array([500.0, 500.0, 320.0, 240.0])
    pw = np.array([0.1, -0.2, 4.0])
    proj = np.array([500 * 0.1 / 4 + 320, 500 * -0.2 / 4 + 240])
    for off, delta in [((0.3, 0.4), 1.0), ((3.0, 4.0), 1.0), ((0.0, 0.0), 1.0), ((3.0, 4.0), 0.0)]:
        uv = proj + np.array(off)
        r, _, _, w, c = oracle.eval_term(pose, pw, intr, uv, delta)
        n = math.hypot(*off)
        np.testing.assert_allclose(r, off, atol=1e-12)
        if delta <= 0:
            assert w == 1.0 and abs(c - n * n) < 1e-12
        elif n == 0:
            assert w == 0.0 and c == 0.0
        elif n <= delta:
            assert abs(c - n * n) < 1e-12
        else:
            assert abs(c - (2 * delta * n - delta * delta)) < 1e-12
            assert abs(w - math.sqrt(2 * delta * n - delta * delta) / n) < 1e-15


def _small_problem(pkg, n_cam=5, n_pt=40, seed=3):
    return pkg.synth.generate(pkg.synth.CIRCLE, n_cam=n_cam, n_pt=n_pt, seed=seed)


def test_schur_vs_dense_equivalence(pkg, oracle):
    # Well-conditioned like the reference's synthetic SPD matrix: two fixed
    # cameras remove the scale gauge.
    prob = _small_problem(pkg)
    prob.pose_const[1] = 1
    for nu in (1e-2, 1.0):
        H, b = oracle.dense_system(prob, nu)
        dense = np.linalg.solve(H, b)
        delta, S, rhs = oracle.schur_step(prob, nu)
        np.testing.assert_allclose(delta, dense, rtol=1e-9, atol=1e-9 * np.abs(dense).max())


def test_parallel_vs_sequential_schur(pkg, oracle):
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=8, n_pt=3000, seed=11)
    prob.pose_const[1] = 1  # no scale gauge: a well-conditioned reduced system
    d1, S1, r1 = oracle.schur_step(prob, 1e-2, n_threads=1)
    d4, S4, r4 = oracle.schur_step(prob, 1e-2, n_threads=4)
    np.testing.assert_allclose(S4, S1, rtol=1e-12, atol=1e-12 * np.abs(S1).max())
    np.testing.assert_allclose(d4, d1, rtol=1e-9, atol=1e-9 * np.abs(d1).max())


def test_block_ldlt_vs_dense_and_psd_pivots(oracle):
    rng = np.random.default_rng(5)
    A = rng.normal(size=(36, 36))
    A = A @ A.T + 0.1 * np.eye(36)
    b = rng.normal(size=36)
    np.testing.assert_allclose(oracle.block_ldlt_solve(A, b), np.linalg.solve(A, b), rtol=1e-9)
    # PSD: a zero direction gets a zero pivot and a zero solution component
    B = rng.normal(size=(12, 11))
    P = B @ B.T  # rank 11
    rhs = P @ rng.normal(size=12)  # consistent right-hand side
    x = oracle.block_ldlt_solve(P, rhs)
    assert np.all(np.isfinite(x))
    np.testing.assert_allclose(P @ x, rhs, atol=1e-8 * np.abs(rhs).max())


def test_simple_cam_marg_points(pkg, oracle):
    """Three cameras along y, cameras 0 and 1 fixed, camera 2 starts at camera 1:
    translation of camera 2 within 0.1 of the truth (cam_calib.rs:268-300)."""
    rng = np.random.default_rng(0)
    fx, fy, cx, cy = 600.0, 600.0, 320.0, 240.0
    t_true = np.array([[0, 0, 0], [0, 1, 0], [0, 2, 0]], float)
    pts, cams, pids, uvs = [], [], [], []
    for i in range(40):
        u, v = rng.uniform(0, 639), rng.uniform(0, 479)
        p = np.array([(u - cx) / fx * 10, (v - cy) / fy * 10, 10.0])
        pts.append(p)
        for c in range(3):
            x = p - t_true[c]
            cams.append(c)
            pids.append(i)
            uvs.append([fx * x[0] / x[2] + cx + rng.uniform(-0.5, 0.5), fy * x[1] / x[2] + cy + rng.uniform(-0.5, 0.5)])
    poses = np.array([[1, 0, 0, 0, *t_true[0]], [1, 0, 0, 0, *t_true[1]], [1, 0, 0, 0, *t_true[1]]], float)
    prob = pkg.BAProblem(poses=poses, points=np.array(pts), intrinsics=np.array([fx, fy, cx, cy]),
                         obs_cam=np.array(cams, np.int32), obs_pt=np.array(pids, np.int32),
                         obs_uv=np.array(uvs), huber_delta=1.0, pose_const=np.array([1, 1, 0], np.uint8))
    params = pkg.OptParams(num_iterations=25, initial_lm_damping=1.0)
    recs, poses_out, _ = oracle.optimize(prob, params)
    np.testing.assert_allclose(poses_out[2, 4:], t_true[2], atol=0.1)


def project_true(prob):
    """Noise-free pixels of every observation at the ground truth."""
    fx, fy, cx, cy = prob.intrinsics
    uv = np.zeros((prob.n_obs, 2))
    for o in range(prob.n_obs):
        T = prob.poses_true[prob.obs_cam[o]]
        x = _rot(T[:4]).T @ (prob.points_true[prob.obs_pt[o]] - T[4:])
        uv[o] = [fx * x[0] / x[2] + cx, fy * x[1] / x[2] + cy]
    return uv


def test_ba_converges(pkg, oracle):
    """Converges to the ground truth (up to the scale gauge about camera 0):
    pose RMS < 0.01, point RMS < 0.1 (ba_problem.rs:517-547)."""
    prob = _small_problem(pkg, n_cam=4, n_pt=20, seed=pkg.synth.BASE_SEED)
    # the reference's pixel noise: 0.15 * U(-0.5, 0.5) per coordinate (ba_problem.rs:251-253)
    prob.obs_uv = project_true(prob) + 0.15 * (np.random.default_rng(2).random(prob.obs_uv.shape) - 0.5)
    params = pkg.OptParams(num_iterations=30, initial_lm_damping=1.0)
    recs, poses, points = oracle.optimize(prob, params)
    c0 = prob.poses_true[0, 4:]
    s = np.sum((points - c0) * (prob.points_true - c0)) / np.sum((points - c0) ** 2)
    pose_rms = np.sqrt(np.mean(np.sum((c0 + s * (poses[:, 4:] - c0) - prob.poses_true[:, 4:]) ** 2, axis=1)))
    pt_rms = np.sqrt(np.mean(np.sum((c0 + s * (points - c0) - prob.points_true) ** 2, axis=1)))
    assert pose_rms < 0.01 and pt_rms < 0.1, (pose_rms, pt_rms)


def test_lm_reference_semantics(pkg, oracle):
    """Fixed iteration count, gain-ratio rules and Nielsen damping update
    (optimizer.rs:463-480): accepted steps never increase the merit, a reject
    doubles nu, an accept multiplies it by max(1/3, 1 - (2 rho - 1)^3)."""
    prob = _small_problem(pkg, n_cam=6, n_pt=200, seed=9)
    params = fixed_iter_params(pkg, 12, 1e-4)
    recs, _, _ = oracle.optimize(prob, params)
    assert len(recs) == 12 and recs[-1].termination == 4
    nu = 1e-4
    merit = oracle.total_cost(prob)
    for r in recs:
        if r.accepted:
            assert r.merit < merit and r.gain_ratio > 0
            x = 2 * r.gain_ratio - 1
            nu *= max(1 - x ** 3, 1 / 3)
            merit = r.merit
        else:
            nu *= 2
            assert r.merit == merit
        assert r.lm_damping == pytest.approx(nu, rel=1e-12)


def test_termination_reasons(pkg, oracle):
    prob = _small_problem(pkg, n_cam=5, n_pt=60, seed=4)
    # function tolerance stops early
    p = pkg.OptParams(num_iterations=100, initial_lm_damping=1e-4, function_tolerance=1e-3)
    recs, _, _ = oracle.optimize(prob, p)
    assert recs[-1].termination == 1 and len(recs) < 100
    # gradient tolerance above the initial gradient stops at once, without a step
    p = pkg.OptParams(num_iterations=100, initial_lm_damping=1e-4, gradient_tolerance=1e30)
    recs, _, _ = oracle.optimize(prob, p)
    assert len(recs) == 1 and recs[0].termination == 2
    # max consecutive rejects with a huge step count and tiny tolerance
    p = pkg.OptParams(num_iterations=1000, initial_lm_damping=1e-4, function_tolerance=0.0,
                      gradient_tolerance=0.0, parameter_tolerance=0.0, max_consecutive_rejects=3)
    recs, _, _ = oracle.optimize(prob, p)
    assert recs[-1].termination in (5,)
