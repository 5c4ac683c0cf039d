"""The oracle beyond the GPU path: Free intrinsics (family kinds (F, F, M)),
the EUCM camera and covariance queries, checked on the CPU before any GPU
kernel exists for them.

  J_cam            pinhole_reprojection.rs:85 (-dx_distort_params, affine.rs:77-108),
                   enhanced_unified.rs:55-215; against central differences
  schur_vs_dense   schur_ldlt.rs:1083-1127 (1e-9), with the intrinsics block
  ba_converges     ba_problem.rs:517-547: free intrinsics started off the truth,
                   poses 0 and 1 fixed; pose RMS < 0.01, point RMS < 0.1
  inverse_block    schur_ldlt.rs:815-957 against the dense inverse of H
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
        np.testing.assert_array_equal(intr_c, list(cond.intrinsics) + [0.0, 0.0])
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
    np.testing.assert_array_equal(ia, list(prob.intrinsics) + [0.0, 0.0])


# ---- EUCM (the camera of the reference's BA example problem) -------------
# enhanced_unified.rs:55-215; EucmCameraReprojectionCostTerm, ba_problem.rs:69-110;
# the reference's true / initial params, ba_problem.rs:162-166,294-304.
EUCM_TRUE = np.array([300.0, 300.0, 320.0, 240.0, 0.5, 1.0])
EUCM_INIT = np.array([297.0, 297.0, 321.0, 241.0, 0.495, 1.0])


def _rot(q):
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _eucm_project(params, x_cam):
    fx, fy, cx, cy, alpha, beta = params
    x, y = x_cam[0] / x_cam[2], x_cam[1] / x_cam[2]
    rho = np.sqrt(beta * (x * x + y * y) + 1.0)
    norm = alpha * rho + (1.0 - alpha)
    return np.array([fx * x / norm + cx, fy * y / norm + cy])


def _eucm_problem(pkg, seed, free=True):
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=4, n_pt=20, seed=seed)
    uv = np.zeros((prob.n_obs, 2))
    for o in range(prob.n_obs):
        T = prob.poses_true[prob.obs_cam[o]]
        uv[o] = _eucm_project(EUCM_TRUE, _rot(T[:4]).T @ (prob.points_true[prob.obs_pt[o]] - T[4:]))
    prob.obs_uv = uv + 0.15 * (np.random.default_rng(2).random(uv.shape) - 0.5)
    prob.poses[:2] = prob.poses_true[:2]
    prob.pose_const[:2] = 1
    prob.intrinsics = EUCM_INIT[:4].copy()
    cond = prob.copy()
    for pr in (prob, cond):
        pr.camera_model = 1
        pr.eucm_alpha_beta = EUCM_INIT[4:].copy()
    prob.intrinsics_free = free
    return prob, cond


def test_eucm_jacobians_vs_central_differences(pkg, oracle):
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=5, n_pt=40, seed=3)
    intr = EUCM_TRUE.copy()
    for o in range(0, prob.n_obs, max(1, prob.n_obs // 20)):
        pose, pt, uv = prob.poses[prob.obs_cam[o]], prob.points[prob.obs_pt[o]], prob.obs_uv[o]
        r0, Jp, Jm, Jc = oracle.eval_term_ex(pose, pt, intr, 1, uv)

        def res(ps=pose, p=pt, k=intr):
            return oracle.eval_term_ex(ps, p, k, 1, uv)[0]
        h = 1e-6
        for k in range(6):  # left perturbation exp(delta) * T_wc
            d = np.zeros(6)
            d[k] = h
            rp = res(ps=oracle.se3_mul(oracle.se3_exp(d), pose))
            rm = res(ps=oracle.se3_mul(oracle.se3_exp(-d), pose))
            np.testing.assert_allclose(Jp[:, k], (rp - rm) / (2 * h), rtol=1e-5, atol=1e-5)
        for k in range(3):
            e = np.zeros(3)
            e[k] = h
            np.testing.assert_allclose(Jm[:, k], (res(p=pt + e) - res(p=pt - e)) / (2 * h), rtol=1e-5, atol=1e-5)
        for k in range(6):
            hk = 1e-6 * max(1.0, abs(intr[k]))
            ip, im = intr.copy(), intr.copy()
            ip[k] += hk
            im[k] -= hk
            np.testing.assert_allclose(Jc[:, k], (res(k=ip) - res(k=im)) / (2 * hk), rtol=1e-5, atol=1e-6)


def test_eucm_with_alpha_zero_is_the_pinhole(pkg, oracle):
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=5, n_pt=40, seed=4)
    intr = np.array(list(prob.intrinsics) + [0.0, 0.7])
    for o in range(0, prob.n_obs, 37):
        pose, pt, uv = prob.poses[prob.obs_cam[o]], prob.points[prob.obs_pt[o]], prob.obs_uv[o]
        r_e, jp_e, jm_e, jc_e = oracle.eval_term_ex(pose, pt, intr, 1, uv)
        r_p, jp_p, jm_p, jc_p = oracle.eval_term_ex(pose, pt, intr, 0, uv)
        np.testing.assert_allclose(r_e, r_p, rtol=1e-12, atol=1e-9)
        np.testing.assert_allclose(jp_e, jp_p, rtol=1e-12, atol=1e-9)
        np.testing.assert_allclose(jm_e, jm_p, rtol=1e-12, atol=1e-9)
        np.testing.assert_allclose(jc_e[:, :4], jc_p, rtol=1e-12, atol=1e-12)


def test_eucm_free_intrinsics_schur_vs_dense(pkg, oracle):
    prob, _ = _eucm_problem(pkg, seed=3)
    for nu in (1e-2, 1.0):
        H, b = oracle.dense_system(prob, nu)
        nf = int(np.sum(prob.pose_const == 0))
        assert H.shape[0] == 6 + 6 * nf + 3 * prob.n_pt
        dense = np.linalg.solve(H, b)
        delta, S, rhs = oracle.schur_step(prob, nu)
        np.testing.assert_allclose(delta, dense, rtol=1e-9, atol=1e-9 * np.abs(dense).max())


def test_eucm_ba_converges(pkg, oracle):
    """ba_problem.rs:517-547 with its EUCM camera free: pose RMS < 0.01,
    point RMS < 0.1 after 20 iterations from the reference's initial params."""
    params = pkg.OptParams(num_iterations=20, initial_lm_damping=1.0, function_tolerance=0.0, gradient_tolerance=0.0,
                           parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)
    for seed in (pkg.synth.BASE_SEED, 5):
        prob, cond = _eucm_problem(pkg, seed)
        recs, poses, points, intr = oracle.optimize(prob, params, with_intrinsics=True)
        pose_rms = np.sqrt(np.mean(np.sum((poses[:, 4:] - prob.poses_true[:, 4:]) ** 2, axis=1)))
        pt_rms = np.sqrt(np.mean(np.sum((points - prob.points_true) ** 2, axis=1)))
        assert pose_rms < 0.01 and pt_rms < 0.1, (seed, pose_rms, pt_rms)
        rc, _, _ = oracle.optimize(cond, params)
        assert recs[-1].merit < rc[-1].merit
        assert abs(intr[0] - EUCM_TRUE[0]) < abs(EUCM_INIT[0] - EUCM_TRUE[0])


# ---- covariance queries (SchurFactor::inverse_block, schur_ldlt.rs:815-957) ----


def _dense_offsets(prob, c0):
    nf_idx = np.cumsum(prob.pose_const == 0) - 1
    nf = int(np.sum(prob.pose_const == 0))
    return (lambda j: c0 + 6 * int(nf_idx[j])), (lambda q: c0 + 6 * nf + 3 * q)


def test_covariance_blocks_vs_dense_inverse(pkg, oracle):
    """Every kind of block against the inverse of the dense undamped H."""
    cases = []
    prob, _, _ = _problem(pkg, seed=3, free=False)  # pinhole, intrinsics Conditioned
    cases.append((prob, 0))
    prob, _ = _eucm_problem(pkg, seed=3)  # EUCM, intrinsics free (6 params first)
    cases.append((prob, 6))
    for prob, c0 in cases:
        H, _ = oracle.dense_system(prob, 0.0)
        cov = np.linalg.inv(H)
        pose_off, pt_off = _dense_offsets(prob, c0)
        scale = np.abs(cov).max()
        free_poses = [j for j in range(prob.n_cam) if not prob.pose_const[j]]
        pairs = [((1, free_poses[0]), (1, free_poses[-1])), ((1, free_poses[-1]), (2, 5)), ((2, 5), (1, free_poses[0])),
                 ((2, 3), (2, 3)), ((2, 3), (2, 11))]
        if c0:
            pairs += [((0, 0), (0, 0)), ((0, 0), (1, free_poses[0])), ((2, 7), (0, 0))]
        for row, col in pairs:
            blk = oracle.covariance_block(prob, row, col)
            def rng(v):
                kind, idx = v
                return (slice(0, c0) if kind == 0 else slice(pose_off(idx), pose_off(idx) + 6) if kind == 1
                        else slice(pt_off(idx), pt_off(idx) + 3))
            np.testing.assert_allclose(blk, cov[rng(row), rng(col)], rtol=1e-7, atol=1e-9 * scale)
        # constant poses and Conditioned intrinsics have no block (the reference returns None)
        assert oracle.covariance_block(prob, (1, 0), (1, 0)) is None
        if not c0:
            assert oracle.covariance_block(prob, (0, 0), (0, 0)) is None


# ---- min-norm pseudo-inverse for a rank-deficient S (min_norm_ldlt.rs:55-140) ----


def test_min_norm_pseudo_inverse_vs_svd(oracle):
    """E G^-1 diag(d_J)^-1 G^-1 E^T of the block LDL^T against the SVD
    pseudo-inverse. The factor zeroes a pivot below 1e-12 x max(1, the running
    largest pivot of its block); matrices of norm ~1e-2 keep their roundoff
    pivots (~1e-18) far below that floor and their true pivots far above it."""
    rng = np.random.default_rng(0)
    for n, r in ((24, 24), (24, 19), (24, 13), (36, 30)):
        B = rng.standard_normal((n, r))
        A = 1e-2 * (B @ B.T) / r
        P, rank = oracle.min_norm_pinv(A)
        assert rank == r
        ref = np.linalg.pinv(A, rcond=1e-10, hermitian=True)
        np.testing.assert_allclose(P, ref, rtol=0, atol=1e-9 * np.abs(ref).max())


def test_covariance_with_an_unobserved_free_pose(pkg, oracle):
    """A free pose with no observations leaves six exact zero pivots in S: the
    free x free blocks are those of the pseudo-inverse, zero for that pose."""
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=6, n_pt=60, seed=3)
    keep = prob.obs_cam != 2
    prob.obs_cam, prob.obs_pt, prob.obs_uv = prob.obs_cam[keep], prob.obs_pt[keep], prob.obs_uv[keep]
    prob.pose_const = np.zeros(6, np.uint8)
    prob.pose_const[0] = 1
    H, _ = oracle.dense_system(prob, 0.0)
    nf = 30
    S_dense = H[:nf, :nf] - H[:nf, nf:] @ np.linalg.solve(H[nf:, nf:], H[:nf, nf:].T)
    assert np.all(S_dense[6:12] == 0.0)  # pose 2 is free block 1 (pose 0 is constant)
    ref = np.linalg.pinv(S_dense, rcond=1e-12, hermitian=True)
    for a in range(1, 6):
        for b in range(1, 6):
            blk = oracle.covariance_block(prob, (1, a), (1, b))
            np.testing.assert_allclose(blk, ref[6 * (a - 1):6 * a, 6 * (b - 1):6 * b], rtol=0,
                                       atol=1e-7 * np.abs(ref).max())
    assert np.all(oracle.covariance_block(prob, (1, 2), (1, 2)) == 0.0)


def test_ring_box_eucm_scene_converges(pkg, oracle):
    """The reference's BA benchmark scene (BaProblem::new(10, 500), restated by
    synth.ring_box_eucm): every camera sees every point of the open box through
    the wide EUCM camera; with the params free the oracle meets the bars of the
    reference's ba_converges (pose RMS < 0.01, point RMS < 0.1) in its 20
    iterations, and with them Conditioned at the truth (ba_bench's
    "conditioned" rows) as well."""
    params = pkg.OptParams(num_iterations=20, initial_lm_damping=1.0, function_tolerance=0.0, gradient_tolerance=0.0,
                           parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)
    prob = pkg.synth.ring_box_eucm()
    assert (prob.n_cam, prob.n_pt, prob.n_obs) == (10, 500, 5000)
    assert prob.huber_delta == 0.0 and list(prob.pose_const[:3]) == [1, 1, 0]
    cond = prob.copy()
    cond.intrinsics_free = False
    cond.intrinsics = prob.intrinsics_true[:4].copy()
    cond.eucm_alpha_beta = prob.intrinsics_true[4:].copy()
    for p in (prob, cond):
        recs, poses, points, intr = oracle.optimize(p, params, with_intrinsics=True)
        pose_rms = np.sqrt(np.mean(np.sum((poses[:, 4:] - p.poses_true[:, 4:]) ** 2, axis=1)))
        pt_rms = np.sqrt(np.mean(np.sum((points - p.points_true) ** 2, axis=1)))
        assert pose_rms < 0.01 and pt_rms < 0.1, (p.intrinsics_free, pose_rms, pt_rms)
        assert recs[-1].merit < 0.05 * recs[0].merit
