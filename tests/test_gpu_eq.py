"""Equality constraints on the GPU: TranslationNormConstraint
|t(pose)| = r (crates/sophus_opt/src/example_problems/ba_scale_constraint.rs:
57-100) through sgba_set_eq_constraints, solved with each LM step by the
range-space KKT method of the Schur solver (schur_ldlt.rs:674-772) inside the
one-CTA float-float solver, against the oracle's restatement (ora_problem.n_eq).

  schur_solvers_converge  ba_scale_constraint.rs:261-287: EUCM camera params
                          free, only pose 0 fixed, |t(pose 1)| = r; per-iteration
                          cost within 1e-6 of the oracle, |c| < 1e-4, pose and
                          point RMS < 0.1
  two constraints         a pinhole circle, constraints on two poses
  limits                  constant poses, more than 8 constraints and systems
                          outside the one-CTA solver are refused"""
import numpy as np
import pytest

from conftest import fixed_iter_params
from test_oracle_free_intrinsics import _eucm_problem

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-6


def _run(pkg, prob, params, **kw):
    with pkg.native.Problem(prob, device=0, **kw) as gp:
        gp.set_eq_constraints(prob.eq_pose, prob.eq_radius)
        recs, _ = gp.optimize(params)
        poses, points = gp.variables()
    return recs, poses, points


def _check(grecs, orecs):
    g = np.array([r.merit for r in grecs])
    o = np.array([r.merit for r in orecs])
    assert len(g) == len(o)
    dev = float(np.max(np.abs(g - o) / o))
    assert dev < COST_RTOL, (dev, g, o)
    return dev


def test_scale_constraint_matches_oracle(pkg, oracle):
    params = pkg.OptParams(num_iterations=20, initial_lm_damping=1.0, function_tolerance=0.0, gradient_tolerance=0.0,
                           parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)
    for seed in (pkg.synth.BASE_SEED, 5):
        prob, _ = _eucm_problem(pkg, seed)
        prob.pose_const[:] = 0
        prob.pose_const[0] = 1
        prob.eq_pose = np.array([1], np.int32)
        prob.eq_radius = np.array([np.linalg.norm(prob.poses_true[1, 4:])])
        grecs, gposes, gpoints = _run(pkg, prob, params, intrinsics_free=True)
        orecs, _, _, _ = oracle.optimize(prob, params, with_intrinsics=True)
        dev = _check(grecs, orecs)
        print("scale constraint (seed %d): per-iteration cost vs oracle %.2e" % (seed, dev))
        c, _ = oracle.eq_eval(prob, gposes)
        assert abs(c[0]) < 1e-4
        pose_rms = np.sqrt(np.mean(np.sum((gposes[:, 4:] - prob.poses_true[:, 4:]) ** 2, axis=1)))
        pt_rms = np.sqrt(np.mean(np.sum((gpoints - prob.points_true) ** 2, axis=1)))
        assert pose_rms < 0.1 and pt_rms < 0.1


def test_two_constraints_pinhole(pkg, oracle):
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=8, n_pt=300, seed=pkg.synth.BASE_SEED + 41)
    prob.eq_pose = np.array([3, 6], np.int32)
    prob.eq_radius = np.array([np.linalg.norm(prob.poses_true[j, 4:]) for j in (3, 6)])
    params = fixed_iter_params(pkg, 10, prob.initial_lm_damping)
    grecs, gposes, _ = _run(pkg, prob, params)
    orecs, _, _ = oracle.optimize(prob, params, n_threads=8)
    dev = _check(grecs, orecs)
    print("two constraints: per-iteration cost vs oracle %.2e" % dev)
    c, _ = oracle.eq_eval(prob, gposes)
    assert np.abs(c).max() < 1e-4


def test_constraint_limits(pkg):
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=6, n_pt=100, seed=pkg.synth.BASE_SEED + 42)
    with pkg.native.Problem(prob, device=0) as gp:
        with pytest.raises(pkg.native.SgbaError):
            gp.set_eq_constraints([0], [4.0])  # pose 0 is constant
        with pytest.raises(pkg.native.SgbaError):
            gp.set_eq_constraints(np.ones(9, np.int32), np.full(9, 4.0))
        gp.set_eq_constraints([2], [4.0])
        gp.set_eq_constraints(np.zeros(0, np.int32), np.zeros(0))  # removed again
    loop = pkg.synth.generate(pkg.synth.LOOP, n_cam=100, n_pt=8000, seed=pkg.synth.BASE_SEED + 43)
    with pkg.native.Problem(loop, device=0) as gp:
        with pytest.raises(pkg.native.SgbaError):
            gp.set_eq_constraints([5], [50.0])  # the band solver
