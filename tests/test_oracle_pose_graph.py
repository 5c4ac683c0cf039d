"""A two-pose cost function on the Schur path: PoseGraph3CostTerm
(pose_graph3.rs), in the oracle. No GPU kernel exists for it yet. Its terms
add pose-pose blocks to S that no shared point creates.

  Jacobians      -/+ dx log(a exp(x) b) at 0 against central differences in
                 each pose
  assembly       J_m^T J_m + nu I, J_n^T J_n + nu I (nu once per reduced term),
                 J_m^T J_n off the diagonal, -J^T g, cost g^T g
  Schur          the step with the edges equals the dense solve
  odometry + BA  exact relative poses from the truth between consecutive
                 cameras, pose 0 fixed: at the combined optimum the gradient
                 vanishes and the edge cost is no higher than at the
                 reprojection-only optimum
"""
import copy

import numpy as np

from test_oracle_reference import project_true


def _with_edges(prob, pairs, mns):
    P = copy.deepcopy(prob)
    P.edge_pose = np.array(pairs, np.int32).reshape(-1, 2)
    P.edge_mn = np.array(mns, float).reshape(-1, 7)
    return P


def _rel(oracle, tm, tn):
    return oracle.se3_mul(oracle.se3_inverse(tm), tn)


def test_edge_residual_and_jacobians(oracle):
    rng = np.random.default_rng(4)
    for _ in range(5):
        tm = oracle.se3_exp(rng.standard_normal(6))
        tn = oracle.se3_exp(rng.standard_normal(6))
        mn = oracle.se3_mul(oracle.se3_exp(0.1 * rng.standard_normal(6)), _rel(oracle, tm, tn))
        r, Jm, Jn, cost = oracle.eval_edge(tm, tn, mn)
        expect = oracle.se3_log(oracle.se3_mul(_rel(oracle, tm, tn), oracle.se3_inverse(mn)))
        np.testing.assert_allclose(r, expect, atol=1e-14)
        np.testing.assert_allclose(cost, r @ r, rtol=1e-13)
        np.testing.assert_array_equal(Jm, -Jn)
        h = 1e-6
        for k in range(6):
            d = np.zeros(6)
            d[k] = h
            for J, which in ((Jm, 0), (Jn, 1)):
                args_p, args_m = [tm, tn], [tm, tn]
                args_p[which] = oracle.se3_mul(oracle.se3_exp(d), args_p[which])
                args_m[which] = oracle.se3_mul(oracle.se3_exp(-d), args_m[which])
                num = (oracle.eval_edge(*args_p, mn)[0] - oracle.eval_edge(*args_m, mn)[0]) / (2 * h)
                np.testing.assert_allclose(J[:, k], num, rtol=1e-6, atol=1e-7)


def test_edge_assembly_and_schur(pkg, oracle):
    rng = np.random.default_rng(5)
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=6, n_pt=40, seed=3)
    prob.pose_const = np.zeros(6, np.uint8)
    prob.pose_const[5] = 1
    pairs = [(3, 1), (0, 2), (3, 1), (4, 5)]  # a repeated pair, and an edge to the constant pose
    mns = [oracle.se3_mul(oracle.se3_exp(0.05 * rng.standard_normal(6)), _rel(oracle, prob.poses[m], prob.poses[n]))
           for m, n in pairs]
    pg = _with_edges(prob, pairs, mns)
    nu = 0.25
    H0, b0 = oracle.dense_system(prob, nu)
    H1, b1 = oracle.dense_system(pg, nu)
    eH, eb, cost = np.zeros_like(H0), np.zeros_like(b0), 0.0
    blk = lambda j: slice(6 * j, 6 * j + 6)  # noqa: E731  poses 0..4 are free, in order
    for (m, n), mn in zip(pairs, mns):
        r, Jm, Jn, c = oracle.eval_edge(prob.poses[m], prob.poses[n], mn)
        cost += c
        for j, J in ((m, Jm), (n, Jn)):
            if j == 5:
                continue
            eH[blk(j), blk(j)] += J.T @ J
            eb[blk(j)] -= J.T @ r
        if 5 not in (m, n):
            eH[blk(m), blk(n)] += Jm.T @ Jn
            eH[blk(n), blk(m)] += Jn.T @ Jm
    for j in (0, 1, 2, 3, 4):  # one nu per reduced term and free argument: (0,2), (3,1) once, (4,5)
        eH[blk(j), blk(j)] += nu * np.eye(6)
    scale = np.abs(eH).max()
    np.testing.assert_allclose(H1 - H0, eH, rtol=0, atol=1e-9 * scale)
    np.testing.assert_allclose(b1 - b0, eb, rtol=0, atol=1e-9 * max(1.0, np.abs(eb).max()))
    np.testing.assert_allclose(oracle.total_cost(pg) - oracle.total_cost(prob), cost, rtol=1e-9)
    dense = np.linalg.solve(H1, b1)
    delta, S, _ = oracle.schur_step(pg, nu)
    np.testing.assert_allclose(delta, dense, rtol=1e-9, atol=1e-9 * np.abs(dense).max())
    # S holds the (3, 1) block although no point couples it more than before
    S0 = oracle.schur_step(prob, nu)[1]
    assert np.abs((S - S0)[blk(3), blk(1)]).max() > 0


def _edge_cost(oracle, poses, pairs, mns):
    return sum(oracle.eval_edge(poses[m], poses[n], mn)[3] for (m, n), mn in zip(pairs, mns))


def test_odometry_edges_at_the_combined_optimum(pkg, oracle):
    """Relative poses from the truth between consecutive cameras, pose 0
    fixed. At the optimum of reprojection + edges: the gradient vanishes, and
    both the edge cost and the combined cost are no higher than at the
    reprojection-only optimum. Plain least squares: with a Huber kernel the
    reference scales the residual but not J (evaluated_term.rs:294-297), so
    its normal-equation gradient is not the gradient of the cost."""
    params = pkg.OptParams(num_iterations=30, initial_lm_damping=1.0, function_tolerance=0.0, gradient_tolerance=0.0,
                           parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)
    for seed in (pkg.synth.BASE_SEED, 5):
        prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=6, n_pt=40, seed=seed)
        prob.huber_delta = 0.0
        prob.obs_uv = project_true(prob) + 2.0 * (np.random.default_rng(seed).random(prob.obs_uv.shape) - 0.5)
        prob.pose_const = np.zeros(6, np.uint8)
        prob.pose_const[0] = 1
        prob.poses[0] = prob.poses_true[0]
        pairs = [(j, j + 1) for j in range(5)]
        mns = [_rel(oracle, prob.poses_true[m], prob.poses_true[n]) for m, n in pairs]
        pg = _with_edges(prob, pairs, mns)
        _, p_ba, q_ba = oracle.optimize(prob, params)
        recs, p_pg, q_pg = oracle.optimize(pg, params)
        assert _edge_cost(oracle, p_pg, pairs, mns) <= _edge_cost(oracle, p_ba, pairs, mns)
        at_ba = copy.deepcopy(pg)
        at_ba.poses, at_ba.points = p_ba, q_ba
        assert recs[-1].merit <= oracle.total_cost(at_ba)
        at_pg = copy.deepcopy(pg)
        at_pg.poses, at_pg.points = p_pg, q_pg
        _, b0 = oracle.dense_system(pg, 0.0)
        _, b1 = oracle.dense_system(at_pg, 0.0)
        assert np.abs(b1).max() < 1e-9 * np.abs(b0).max(), (seed, np.abs(b1).max(), np.abs(b0).max())
