"""Pose priors on the GPU: the Isometry3PriorCostTerm cost function
(crates/sophus_opt/src/nlls/functor_library/costs/isometry3_prior.rs) beside
the reprojection cost, through sgba_set_pose_priors, against the oracle's
restatement (ora_problem.n_prior).

  residual / Jacobian  log(T E^-1), d log(exp(x) T E^-1) / dx at 0 (forward-mode
                       derivatives in f64 on the GPU, dual numbers in the oracle)
  assembly             J^T W J and -J^T W g on the pose's block, nu I once per
                       pose with priors, cost g^T W g (evaluated_term.rs:286-327)
  optimize_with_priors cam_calib.rs:249-342 on the Schur path: all poses free,
                       priors 1e4 I on poses 0 and 1 at the truth hold the gauge;
                       the reference asserts |t(pose 2) - t_true| < 0.1
Per-iteration cost within 1e-6 of the oracle."""
import numpy as np
import pytest

from conftest import fixed_iter_params
from test_oracle_reference import project_true

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-6


def _spd(rng, scale=1.0):
    A = rng.standard_normal((6, 6))
    return scale * (A @ A.T + 6 * np.eye(6))


def _with_priors(prob, poses, means, Ws):
    P = prob.copy()
    P.prior_pose = np.array(poses, np.int32)
    P.prior_mean = np.array(means, float)
    P.prior_precision = np.array(Ws, float)
    return P


def _gpu(pkg, prob, params):
    with pkg.native.Problem(prob, device=0) as gp:
        gp.set_pose_priors(prob.prior_pose, prob.prior_mean, prob.prior_precision)
        recs, term = gp.optimize(params)
        poses, points = gp.variables()
        cost = gp.cost()
    return recs, poses, points, cost


def _check_trajectory(grecs, orecs):
    g = np.array([r.merit for r in grecs])
    o = np.array([r.merit for r in orecs])
    assert len(g) == len(o)
    dev = np.max(np.abs(g - o) / o)
    assert dev < COST_RTOL, (dev, g, o)
    return dev


def test_priors_match_oracle_per_iteration(pkg, oracle):
    """Priors on free poses (two on one pose) and on the constant pose, with
    the Huber reprojection cost, 10 LM iterations."""
    rng = np.random.default_rng(11)
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=6, n_pt=300, seed=pkg.synth.BASE_SEED + 21)
    prob.pose_const = np.zeros(6, np.uint8)
    prob.pose_const[5] = 1
    sel = [2, 0, 2, 5]
    means = [oracle.se3_mul(oracle.se3_exp(0.05 * rng.standard_normal(6)), prob.poses_true[j]) for j in sel]
    pp = _with_priors(prob, sel, means, [_spd(rng, 50.0) for _ in sel])
    params = fixed_iter_params(pkg, 10, prob.initial_lm_damping)
    grecs, gposes, _, gcost = _gpu(pkg, pp, params)
    orecs, oposes, _ = oracle.optimize(pp, params, n_threads=8)
    dev = _check_trajectory(grecs, orecs)
    print("priors: per-iteration cost vs oracle %.2e" % dev)
    assert np.abs(gposes[:, 4:] - oposes[:, 4:]).max() < 1e-6
    assert gcost == grecs[-1].merit


def test_optimize_with_priors_cam_calib(pkg, oracle):
    """The reference's optimize_with_priors on the GPU: no pose is constant,
    the priors on poses 0 and 1 hold the gauge."""
    params = pkg.OptParams(num_iterations=10, initial_lm_damping=1.0, function_tolerance=0.0, gradient_tolerance=0.0,
                           parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)
    for seed in (pkg.synth.BASE_SEED, 5):
        prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=5, n_pt=40, seed=seed)
        prob.obs_uv = project_true(prob) + (np.random.default_rng(seed).random(prob.obs_uv.shape) - 0.5)
        prob.pose_const = np.zeros(prob.n_cam, np.uint8)
        pp = _with_priors(prob, [0, 1], prob.poses_true[:2], [1e4 * np.eye(6)] * 2)
        grecs, gposes, _, _ = _gpu(pkg, pp, params)
        orecs, _, _ = oracle.optimize(pp, params, n_threads=8)
        _check_trajectory(grecs, orecs)
        assert np.abs(gposes[2, 4:] - prob.poses_true[2, 4:]).max() < 0.1
        assert np.abs(gposes[:2, 4:] - prob.poses_true[:2, 4:]).max() < 0.01


def test_prior_set_replaced_and_removed(pkg):
    """A new set replaces the old one; an empty set gives back the problem
    without priors, bit for bit; bad indices and quaternions are refused."""
    rng = np.random.default_rng(3)
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=6, n_pt=200, seed=pkg.synth.BASE_SEED + 22)
    params = fixed_iter_params(pkg, 6, prob.initial_lm_damping)
    with pkg.native.Problem(prob, device=0) as gp:
        plain, _ = gp.optimize(params)
    with pkg.native.Problem(prob, device=0) as gp:
        gp.set_pose_priors([1], [prob.poses_true[1]], [_spd(rng)])
        with_prior, _ = gp.optimize(params)
        gp.set_variables(prob.poses, prob.points)
        gp.set_pose_priors(np.zeros(0, np.int32), np.zeros((0, 7)), np.zeros((0, 6, 6)))
        removed, _ = gp.optimize(params)
        with pytest.raises(pkg.native.SgbaError):
            gp.set_pose_priors([6], [prob.poses_true[1]], [np.eye(6)])
        bad = prob.poses_true[1].copy()
        bad[0] = 2.0
        with pytest.raises(pkg.native.SgbaError):
            gp.set_pose_priors([1], [bad], [np.eye(6)])
    assert [r.merit for r in removed] == [r.merit for r in plain]
    assert with_prior[0].merit > plain[0].merit


def test_python_mirror_prior_cost_fn(pkg, oracle):
    """optimize_nlls of the Python mirror with a reprojection CostFn and an
    Isometry3PriorCostTerm CostFn on the pose family (cam_calib.rs:249-342's
    shape: every pose free, priors on poses 0 and 1)."""
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=5, n_pt=60, seed=pkg.synth.BASE_SEED + 23)
    prob.pose_const = np.zeros(prob.n_cam, np.uint8)
    K = pkg.VarKind
    variables = (pkg.VarBuilder.new()
                 .add_family("cams", pkg.VarFamily.new(K.Conditioned, [pkg.PinholeCameraF64(prob.intrinsics)]))
                 .add_family("poses", pkg.VarFamily.new(K.Free, [pkg.Isometry3F64(p) for p in prob.poses]))
                 .add_family("points", pkg.VarFamily.new(K.Marginalized, prob.points))
                 .build())
    idx = np.stack([np.zeros(prob.n_obs, np.int64), prob.obs_cam, prob.obs_pt], axis=1)
    reproj = pkg.CostFn.new_boxed_robust(
        None, pkg.CostTerms.new(["cams", "poses", "points"], pkg.PinholeReprojectionTerms(prob.obs_uv, idx)),
        pkg.RobustKernel.Huber(pkg.HuberKernel.new(prob.huber_delta)))
    W = 1e4 * np.eye(6)
    priors = pkg.CostFn.new_boxed(None, pkg.CostTerms.new(
        ["poses"], [pkg.Isometry3PriorCostTerm(pkg.Isometry3F64(prob.poses_true[j]), W, [j]) for j in (0, 1)]))
    params = fixed_iter_params(pkg, 8, prob.initial_lm_damping)
    sol = pkg.optimize_nlls(variables, [reproj, priors], [], params)
    pp = _with_priors(prob, [0, 1], prob.poses_true[:2], [W, W])
    orecs, _, _ = oracle.optimize(pp, params, n_threads=8)
    assert len(sol.steps) == len(orecs)
    g = np.array([st.merit for st in sol.steps])
    o = np.array([r.merit for r in orecs])
    assert np.max(np.abs(g - o) / o) < COST_RTOL
