"""Covariance and precision queries of the solution on the GPU
(OptimizationSolution::covariance_block / precision_block,
crates/sophus_opt/src/nlls/optimizer_types.rs:277-370, over the final Hessian of
Optimizer::build_solution, optimizer.rs:609-646), through
sgba_covariance_prepare / sgba_covariance_blocks, against the oracle's
restatement of SchurFactor::inverse_block (schur_ldlt.rs:815-957) and the
oracle's dense undamped H.

  kinds            pose x pose, pose x point, point x pose, point x point
                   (same and different points), every block within 1e-7 of
                   the oracle relative to the largest entry of the blocks
  solvers' shapes  a circle (dense S), a 30-camera sphere, a 100-camera loop
                   (sparse S: the merge of two poses' term lists), the EUCM
                   camera
  pseudo-inverse   a free pose without observations: six zero pivots, the
                   min-norm S+ (min_norm_ldlt.rs:55-140), zero for that pose
  cost functions   pose priors and pose-graph edges in H and S (every pose free,
                   priors holding the gauge)
  precision        blocks of the undamped H against the oracle's dense H
  free camera      the camera params Free (pinhole and EUCM): their block
                   first, coupled to every pose and point; every kind of
                   block with the camera against the oracle
  None / errors    constant poses, indices out of range, unknown kinds, a
                   query before prepare, equality constraints"""
import copy

import numpy as np
import pytest

from conftest import fixed_iter_params
from test_oracle_free_intrinsics import _eucm_problem, _problem

pytestmark = pytest.mark.gpu

REL = 1e-7


def _solve(pkg, prob, n_iter=4):
    params = fixed_iter_params(pkg, n_iter, prob.initial_lm_damping)
    gp = pkg.native.Problem(prob, device=0)
    if getattr(prob, "prior_pose", None) is not None and len(prob.prior_pose):
        gp.set_pose_priors(prob.prior_pose, prob.prior_mean, prob.prior_precision)
    gp.optimize(params)
    poses, points = gp.variables()
    at = copy.copy(prob)  # keeps the priors and edges set on the problem
    at.poses, at.points = poses, points
    return gp, at


def _queries(prob, free_poses, points):
    P, Q = 1, 2
    a, b = free_poses[0], free_poses[-1]
    c = free_poses[len(free_poses) // 2]
    p, q = points[0], points[-1]
    return [((P, a), (P, a)), ((P, a), (P, b)), ((P, b), (P, c)), ((P, c), (Q, p)), ((Q, q), (P, a)),
            ((Q, p), (Q, p)), ((Q, p), (Q, q)), ((Q, q), (Q, q))]


def _check(gp, oracle, at, queries):
    got = gp.covariance_blocks(queries)
    ref = [oracle.covariance_block(at, row, col) for row, col in queries]
    scale = max(np.abs(r).max() for r in ref)
    worst = 0.0
    for (row, col), g, r in zip(queries, got, ref):
        assert g is not None and g.shape == r.shape, (row, col)
        worst = max(worst, float(np.abs(g - r).max() / scale))
    assert worst < REL, worst
    return worst


def _point_const(prob):
    return np.zeros(prob.n_pt, np.uint8) if prob.point_const is None else np.asarray(prob.point_const)


def _observed_points(prob, k):
    cnt = np.bincount(prob.obs_pt, minlength=prob.n_pt)
    pc = _point_const(prob)
    idx = [q for q in range(prob.n_pt) if cnt[q] >= 3 and not pc[q]]
    return [idx[0], idx[len(idx) // 3], idx[-1]][:k]


@pytest.mark.parametrize("shape", ["circle", "sphere30", "loop100"])
def test_covariance_blocks_match_oracle(pkg, oracle, shape):
    if shape == "circle":
        prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=8, n_pt=300, seed=pkg.synth.BASE_SEED + 51)
    elif shape == "sphere30":
        prob = pkg.synth.generate(pkg.synth.SPHERE, n_cam=30, n_pt=3000, seed=pkg.synth.BASE_SEED + 52)
    else:
        prob = pkg.synth.generate(pkg.synth.LOOP, n_cam=100, n_pt=8000, seed=pkg.synth.BASE_SEED + 53)
    # two constant poses hold the scale: without them S is gauge-deficient
    # and its smallest pivot is rounding noise (no covariance to compare)
    prob.pose_const[:2] = 1
    gp, at = _solve(pkg, prob)
    with gp:
        info = gp.covariance_prepare()
        free = [j for j in range(prob.n_cam) if not prob.pose_const[j]]
        assert info.n == 6 * len(free) and info.rank == info.n
        worst = _check(gp, oracle, at, _queries(prob, free, _observed_points(prob, 3)))
    print("covariance (%s, n=%d): vs oracle %.2e; assemble %.2f ms, factor %.2f ms, inverse %.2f ms, %d launches"
          % (shape, info.n, worst, info.ms_assemble, info.ms_factor, info.ms_inverse, info.kernel_launches))


def test_covariance_eucm_camera(pkg, oracle):
    _, cond = _eucm_problem(pkg, 3)
    gp, at = _solve(pkg, cond)
    with gp:
        gp.covariance_prepare()
        free = [j for j in range(cond.n_cam) if not cond.pose_const[j]]
        _check(gp, oracle, at, _queries(cond, free, _observed_points(cond, 2)))


def test_covariance_pseudo_inverse_unobserved_pose(pkg, oracle):
    """Pose 2 has no observations: its six pivots are exactly zero and the
    free x free blocks are those of the min-norm pseudo-inverse (poses 0 and 1
    constant: no gauge left besides that pose)."""
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=6, n_pt=60, seed=3)
    keep = prob.obs_cam != 2
    prob.obs_cam, prob.obs_pt, prob.obs_uv = prob.obs_cam[keep], prob.obs_pt[keep], prob.obs_uv[keep]
    prob.pose_const = np.zeros(6, np.uint8)
    prob.pose_const[:2] = 1
    with pkg.native.Problem(prob, device=0) as gp:
        info = gp.covariance_prepare()
        assert info.n == 24 and info.rank == 18
        queries = [((1, a), (1, b)) for a in range(2, 6) for b in range(2, 6)]
        got = gp.covariance_blocks(queries)
        ref = [oracle.covariance_block(prob, r, c) for r, c in queries]
        scale = max(np.abs(r).max() for r in ref)
        for (row, col), g, r in zip(queries, got, ref):
            np.testing.assert_allclose(g, r, rtol=0, atol=REL * scale, err_msg=str((row, col)))
        assert np.all(gp.covariance_block((1, 2), (1, 2)) == 0.0)
        # point blocks still follow through S+
        q = _observed_points(prob, 1)[0]
        _check(gp, oracle, prob, [((2, q), (2, q)), ((1, 3), (2, q))])


def test_covariance_with_priors_and_edges(pkg, oracle):
    """Every pose free, priors on poses 0 and 1 holding the gauge, odometry
    edges: their J^T W J and J_m^T J_n enter H and S."""
    rng = np.random.default_rng(9)
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=6, n_pt=200, seed=pkg.synth.BASE_SEED + 54)
    prob.pose_const = np.zeros(6, np.uint8)
    T = prob.poses_true
    pairs = [(0, 1), (1, 2), (2, 3), (4, 5), (5, 0)]
    mns = []
    for m, n in pairs:
        rel = oracle.se3_mul(oracle.se3_inverse(T[m]), T[n])
        mns.append(oracle.se3_mul(oracle.se3_exp(0.01 * rng.standard_normal(6)), rel))
    prob.edge_pose = np.array(pairs, np.int32)
    prob.edge_mn = np.array(mns, float)
    prob.prior_pose = np.array([0, 1], np.int32)
    prob.prior_mean = T[:2].copy()
    prob.prior_precision = np.array([1e4 * np.eye(6)] * 2)
    gp, at = _solve(pkg, prob, n_iter=3)
    with gp:
        gp.covariance_prepare()
        worst = _check(gp, oracle, at, _queries(prob, list(range(6)), _observed_points(prob, 2)))
        # precision: the pose x pose block of an edge is J_m^T J_n
        H, _ = oracle.dense_system(at, 0.0)
        np.testing.assert_allclose(gp.precision_block((1, 1), (1, 2)), H[6:12, 12:18], rtol=1e-9,
                                   atol=1e-9 * np.abs(H[:36, :36]).max())
        np.testing.assert_allclose(gp.precision_block((1, 0), (1, 0)), H[0:6, 0:6], rtol=1e-9,
                                   atol=1e-9 * np.abs(H[:36, :36]).max())
        assert np.all(gp.precision_block((1, 0), (1, 3)) == 0.0)
    print("covariance with priors and edges: vs oracle %.2e" % worst)


def test_precision_blocks_match_dense_hessian(pkg, oracle):
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=6, n_pt=120, seed=pkg.synth.BASE_SEED + 55)
    prob.pose_const[:2] = 1
    gp, at = _solve(pkg, prob, n_iter=2)
    H, _ = oracle.dense_system(at, 0.0)
    fidx = np.cumsum(at.pose_const == 0) - 1
    nf = int(np.sum(at.pose_const == 0))
    midx = np.cumsum(_point_const(at) == 0) - 1
    po = lambda j: slice(6 * fidx[j], 6 * fidx[j] + 6)
    pt = lambda q: slice(6 * nf + 3 * midx[q], 6 * nf + 3 * midx[q] + 3)
    q0, q1 = _observed_points(at, 2)
    cam_of_q0 = int([c for c in at.obs_cam[at.obs_pt == q0] if not at.pose_const[c]][-1])
    cases = [((1, 2), (1, 2), po(2), po(2)), ((1, 2), (1, 4), po(2), po(4)),
             ((1, cam_of_q0), (2, q0), po(cam_of_q0), pt(q0)), ((2, q0), (1, cam_of_q0), pt(q0), po(cam_of_q0)),
             ((2, q0), (2, q0), pt(q0), pt(q0)), ((2, q0), (2, q1), pt(q0), pt(q1))]
    with gp:
        gp.covariance_prepare()
        got = gp.covariance_blocks([(r, c) for r, c, _, _ in cases], pkg.native.QUERY_PRECISION)
        for (row, col, rs, cs), g in zip(cases, got):
            ref = H[rs, cs]
            np.testing.assert_allclose(g, ref, rtol=1e-10, atol=1e-10 * np.abs(H).max(), err_msg=str((row, col)))


def test_none_and_errors(pkg):
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=5, n_pt=80, seed=pkg.synth.BASE_SEED + 56)
    prob.point_const = np.zeros(prob.n_pt, np.uint8)
    prob.point_const[7] = 1
    prob.pose_const[:2] = 1
    with pkg.native.Problem(prob, device=0) as gp:
        with pytest.raises(pkg.native.SgbaError) as e:
            gp.covariance_block((1, 2), (1, 2))  # before prepare
        assert e.value.status == pkg.native.ERR_STATE
        gp.covariance_prepare()
        res = gp.covariance_blocks([((1, 0), (1, 1)),   # pose 0 is constant
                                    ((1, 1), (1, 99)),  # out of range
                                    ((2, 7), (2, 7)),   # a constant point
                                    ((2, -1), (1, 2)),
                                    ((1, 2), (1, 2))])
        assert res[0] is None and res[1] is None and res[2] is None and res[3] is None
        assert res[4].shape == (6, 6) and np.allclose(res[4], res[4].T, rtol=0, atol=1e-12 * np.abs(res[4]).max())
        assert np.all(np.linalg.eigvalsh(res[4]) > 0)
        assert gp.covariance_block((0, 0), (1, 2)) is None  # Conditioned camera params: no block
        with pytest.raises(pkg.native.SgbaError):
            gp.covariance_blocks([((5, 0), (1, 2))])  # no such kind
        gp.covariance_release()
        with pytest.raises(pkg.native.SgbaError):
            gp.covariance_block((1, 2), (1, 2))
    prob2 = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=6, n_pt=100, seed=pkg.synth.BASE_SEED + 42)
    with pkg.native.Problem(prob2, device=0) as gp:
        gp.set_eq_constraints([2], [4.0])
        with pytest.raises(pkg.native.SgbaError) as e:
            gp.covariance_prepare()  # the constraint-projected covariance is not on this path
        assert e.value.status == pkg.native.ERR_UNSUPPORTED


def test_python_mirror_solution_queries(pkg, oracle):
    """optimize_nlls's solution answers covariance_block / precision_block by
    family name, as the reference's OptimizationSolution does."""
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=5, n_pt=60, seed=pkg.synth.BASE_SEED + 57)
    prob.pose_const[:2] = 1
    K = pkg.VarKind
    variables = (pkg.VarBuilder.new()
                 .add_family("cams", pkg.VarFamily.new(K.Conditioned, [pkg.PinholeCameraF64(prob.intrinsics)]))
                 .add_family("poses", pkg.VarFamily.new_with_const_ids(
                     K.Free, [pkg.Isometry3F64(p) for p in prob.poses], [0, 1]))
                 .add_family("points", pkg.VarFamily.new(K.Marginalized, prob.points))
                 .build())
    idx = np.stack([np.zeros(prob.n_obs, np.int64), prob.obs_cam, prob.obs_pt], axis=1)
    reproj = pkg.CostFn.new_boxed_robust(
        None, pkg.CostTerms.new(["cams", "poses", "points"], pkg.PinholeReprojectionTerms(prob.obs_uv, idx)),
        pkg.RobustKernel.Huber(pkg.HuberKernel.new(prob.huber_delta)))
    params = fixed_iter_params(pkg, 3, prob.initial_lm_damping)
    sol = pkg.optimize_nlls(variables, [reproj], [], params)
    try:
        at = prob.copy()
        at.poses = np.array([p.params() if hasattr(p, "params") else p for p in sol.variables.collection["poses"].members])
        at.points = np.asarray(sol.variables.collection["points"].members)
        q = _observed_points(prob, 1)[0]
        for (fr, ir, fc, ic), row, col in ((("poses", 2, "poses", 3), (1, 2), (1, 3)),
                                           (("points", q, "poses", 4), (2, q), (1, 4))):
            g = sol.covariance_block(fr, ir, fc, ic)
            r = oracle.covariance_block(at, row, col)
            np.testing.assert_allclose(g, r, rtol=0, atol=REL * np.abs(r).max())
        assert sol.covariance_block("poses", 0, "poses", 0) is None  # constant
        assert sol.covariance_block("cams", 0, "poses", 2) is None   # Conditioned family
        H, _ = oracle.dense_system(at, 0.0)
        np.testing.assert_allclose(sol.precision_block("poses", 2, "poses", 2), H[0:6, 0:6], rtol=1e-10,
                                   atol=1e-10 * np.abs(H).max())
    finally:
        sol.close()


@pytest.mark.parametrize("n_cam", [300, 1500])
def test_hessian_times_covariance_is_identity_loop(pkg, n_cam):
    """At the loop sizes (1500 cameras, 300,000 points: the headline problem),
    where the oracle's dense restatement is too slow, a size-independent
    identity: the row of pose i of the undamped H times the covariance's column
    of pose j is delta_ij I, i.e.
        H_ii Cov_ij + sum over the points q that pose i sees of W_iq Cov_qj,
    every block from one batched query of each kind.  The deviation is
    bounded by about cond(S) eps: 1e-6 at 300 cameras, 1e-5 at 1500 (S's
    condition number ~6e10 there)."""
    prob = pkg.synth.generate(pkg.synth.LOOP, n_cam=n_cam, n_pt=200 * n_cam, seed=pkg.synth.BASE_SEED)
    prob.pose_const[:2] = 1
    params = fixed_iter_params(pkg, 2, prob.initial_lm_damping)
    with pkg.native.Problem(prob, device=0) as gp:
        gp.optimize(params)
        info = gp.covariance_prepare()
        assert info.rank == info.n == 6 * (n_cam - 2)
        i = n_cam // 2
        qs = np.unique(prob.obs_pt[prob.obs_cam == i])
        worst = 0.0
        for j in (i, i + 1, 5):
            prec = gp.covariance_blocks([((1, i), (1, i))] + [((1, i), (2, int(q))) for q in qs],
                                        pkg.native.QUERY_PRECISION)
            cov = gp.covariance_blocks([((1, i), (1, j))] + [((2, int(q)), (1, j)) for q in qs])
            R = prec[0] @ cov[0]
            for W, C in zip(prec[1:], cov[1:]):
                R += W @ C
            worst = max(worst, float(np.abs(R - (np.eye(6) if j == i else 0.0)).max()))
    print("H Cov = I on the %d-camera loop (n=%d): max deviation %.2e over %d points; assemble %.1f ms, "
          "factor %.1f ms, inverse %.1f ms, %d launches"
          % (n_cam, info.n, worst, len(qs), info.ms_assemble, info.ms_factor, info.ms_inverse, info.kernel_launches))
    assert worst < (1e-6 if n_cam <= 300 else 1e-5)


@pytest.mark.parametrize("model", ["pinhole", "eucm"])
def test_covariance_free_camera_params(pkg, oracle, model):
    """Free camera params (the reference's optimize with free intrinsics):
    camera x camera, camera x pose, camera x point, pose x point and
    point x point blocks against the oracle, and the camera's precision
    blocks against the oracle's dense H."""
    prob = _problem(pkg, seed=3, free=True)[0] if model == "pinhole" else _eucm_problem(pkg, 3)[0]
    params = fixed_iter_params(pkg, 4, 1.0)
    with pkg.native.Problem(prob, device=0) as gp:
        gp.optimize(params)
        poses, points = gp.variables()
        intr = gp.intrinsics()
        at = copy.copy(prob)
        at.poses, at.points = poses, points
        at.intrinsics = intr[:4].copy()
        if len(intr) == 6:
            at.eucm_alpha_beta = intr[4:].copy()
        info = gp.covariance_prepare()
        nk = len(intr)
        free = [j for j in range(prob.n_cam) if not prob.pose_const[j]]
        assert info.n == 6 + 6 * len(free) and info.rank == info.n
        p, q = _observed_points(prob, 2)
        a = free[-1]
        queries = [((0, 0), (0, 0)), ((0, 0), (1, a)), ((1, a), (0, 0)), ((0, 0), (2, p)), ((2, q), (0, 0)),
                   ((1, a), (2, p)), ((2, p), (2, p)), ((2, p), (2, q))]
        worst = _check(gp, oracle, at, queries)
        assert gp.covariance_block((0, 0), (0, 0)).shape == (nk, nk)
        H, _ = oracle.dense_system(at, 0.0)
        fidx = {j: k for k, j in enumerate(free)}
        prec = gp.covariance_blocks([((0, 0), (0, 0)), ((0, 0), (1, a)), ((0, 0), (2, p))], pkg.native.QUERY_PRECISION)
        scale = np.abs(H).max()
        np.testing.assert_allclose(prec[0], H[:nk, :nk], rtol=1e-10, atol=1e-12 * scale)
        np.testing.assert_allclose(prec[1], H[:nk, nk + 6 * fidx[a]:nk + 6 * fidx[a] + 6], rtol=1e-10,
                                   atol=1e-12 * scale)
        nf = len(free)
        np.testing.assert_allclose(prec[2], H[:nk, nk + 6 * nf + 3 * p:nk + 6 * nf + 3 * p + 3], rtol=1e-10,
                                   atol=1e-12 * scale)
    print("covariance with free camera params (%s): vs oracle %.2e" % (model, worst))
