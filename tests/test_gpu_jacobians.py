"""Per-term Jacobians of the GPU linearization against the oracle's dual-number
Jacobians.

The reference evaluates PinholeCameraReprojectionCostTerm::eval with
DualScalar forward mode (crates/sophus_opt/src/nlls/functor_library/costs/pinhole_reprojection.rs:60-95;
the Lie-group Jacobian convention is checked in
crates/sophus_lie/src/lie_group/real_lie_group.rs:340-390).  The oracle
restates that dual-number evaluation (ora_eval_term_dual).  Here every entry of
J_pose (2x6) and J_point (2x3) that the GPU kernels compute (jacobians_f for the
FP32 linearization, jacobians_dd for the float-float one) is compared entry by
entry, so a sign or ordering error that would cancel in J^T J shows up.

Bars: FP32 1e-5 of the term's largest entry, float-float 1e-10."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5
DD_TOL = 1e-10


def _oracle_jacobians(oracle, prob, cams, pts):
    jp = np.empty((len(cams), 2, 6))
    jm = np.empty((len(cams), 2, 3))
    for k, (c, p) in enumerate(zip(cams, pts)):
        jp[k], jm[k] = oracle.eval_term_dual(prob.poses[c], prob.points[p], prob.intrinsics, np.zeros(2))
    return jp, jm


def _rel_err(g, o):
    """Per term: max entry error over the term's largest entry (pose and point
    blocks together)."""
    scale = np.maximum(np.abs(o).reshape(len(o), -1).max(axis=1), 1e-300)
    return (np.abs(g - o).reshape(len(o), -1).max(axis=1) / scale)


def _check(pkg, oracle, prob, sample, seed=0):
    rng = np.random.default_rng(seed)
    idx = np.arange(prob.n_obs) if sample is None else rng.choice(prob.n_obs, size=sample, replace=False)
    cams, pts = prob.obs_cam[idx], prob.obs_pt[idx]
    ojp, ojm = _oracle_jacobians(oracle, prob, cams, pts)
    out = {}
    with pkg.native.Problem(prob, device=0) as gp:
        for prec, tol in ((0, FP32_TOL), (1, DD_TOL)):
            gjp, gjm = gp.jacobians(cams, pts, precision=prec)
            e = np.maximum(_rel_err(gjp, ojp), _rel_err(gjm, ojm))
            out[prec] = float(e.max())
            assert e.max() < tol, (prec, e.max(), int(np.argmax(e)))
        # after a few LM iterations the variables have moved: the kernels read
        # the problem's current state
        gp.optimize(pkg.OptParams(num_iterations=2, initial_lm_damping=prob.initial_lm_damping,
                                  function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0,
                                  max_consecutive_rejects=1 << 40))
        poses, points = gp.variables()
        moved = prob.copy()
        moved.poses, moved.points = poses, points
        ojp2, ojm2 = _oracle_jacobians(oracle, moved, cams, pts)
        gjp, gjm = gp.jacobians(cams, pts, precision=1)
        e = np.maximum(_rel_err(gjp, ojp2), _rel_err(gjm, ojm2))
        assert e.max() < DD_TOL, e.max()
    return out


def test_jacobians_match_dual_numbers_config0(pkg, oracle):
    prob = pkg.synth.generate(pkg.synth.CIRCLE, seed=pkg.synth.BASE_SEED)
    errs = _check(pkg, oracle, prob, sample=None)
    print("config 0, every term: max rel entry error FP32 %.2e, float-float %.2e" % (errs[0], errs[1]))


def test_jacobians_match_dual_numbers_loop(pkg, oracle):
    prob = pkg.synth.generate(pkg.synth.LOOP, n_cam=300, n_pt=30000, seed=pkg.synth.BASE_SEED + 2)
    errs = _check(pkg, oracle, prob, sample=4000, seed=1)
    print("300-camera loop, 4000 terms: max rel entry error FP32 %.2e, float-float %.2e" % (errs[0], errs[1]))


def test_jacobian_query_rejects_bad_indices(pkg):
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=4, n_pt=30, seed=3)
    with pkg.native.Problem(prob, device=0) as gp:
        with pytest.raises(pkg.native.SgbaError) as e:
            gp.jacobians([0, 4], [0, 1])
        assert e.value.status == pkg.native.ERR_INVALID_ARGUMENT
        with pytest.raises(pkg.native.SgbaError):
            gp.jacobians([0], [0], precision=2)
