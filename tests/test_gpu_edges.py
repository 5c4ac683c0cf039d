"""Pose-graph edges on the GPU: the PoseGraph3CostTerm cost function
(crates/sophus_opt/src/nlls/functor_library/costs/pose_graph3.rs) beside the
reprojection cost, through sgba_problem_create_graph, against the oracle's
restatement (ora_problem.n_edge).

  residual / Jacobians  log(T_m^-1 T_n M^-1); J_n = D, J_m = -D with D the
                        derivative of log(T_m^-1 exp(x) T_n M^-1) at 0
                        (forward-mode derivatives in f64 on the GPU)
  assembly              J_m^T J_m, J_n^T J_n (+ nu I once per reduced term) on
                        the diagonal, J_m^T J_n on the block of S between the
                        two poses (a new block where no point joins them),
                        -J^T g, cost g^T g
Problems with edges get the float-float linearization.  Per-iteration cost
within 1e-6 of the oracle on a dense circle problem and a 30-camera sphere
(the one-CTA float-float solver) and on a loop whose edges join cameras far
apart (the band solver); the cluster solver of larger dense systems is held to
its measured limit (FP32 factor, refined)."""
import numpy as np
import pytest

from conftest import fixed_iter_params

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-6


def _with_edges(prob, pairs, mns):
    P = prob.copy()
    P.edge_pose = np.array(pairs, np.int32).reshape(-1, 2)
    P.edge_mn = np.array(mns, float).reshape(-1, 7)
    return P


def _noisy_rel(oracle, rng, tm, tn, s):
    rel = oracle.se3_mul(oracle.se3_inverse(tm), tn)
    return oracle.se3_mul(oracle.se3_exp(s * rng.standard_normal(6)), rel)


def _compare(pkg, oracle, pp, n_iter, threads=8):
    params = fixed_iter_params(pkg, n_iter, pp.initial_lm_damping)
    with pkg.native.Problem(pp, device=0) as gp:
        grecs, _ = gp.optimize(params)
        lay = gp.layout()
        gposes, _ = gp.variables()
    orecs, oposes, _ = oracle.optimize(pp, params, n_threads=threads)
    g = np.array([r.merit for r in grecs])
    o = np.array([r.merit for r in orecs])
    assert len(g) == len(o) == n_iter
    dev = float(np.max(np.abs(g - o) / o))
    assert dev < COST_RTOL, (dev, g, o)
    return dev, lay, gposes, oposes


def test_odometry_edges_circle(pkg, oracle):
    """Consecutive cameras joined by noisy relative poses (duplicated once, a
    reversed pair, an edge on the constant camera), 10 LM iterations."""
    rng = np.random.default_rng(5)
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=8, n_pt=300, seed=pkg.synth.BASE_SEED + 31)
    T = prob.poses_true
    pairs = [(j, j + 1) for j in range(7)] + [(3, 4), (6, 2), (0, 5)]
    mns = [_noisy_rel(oracle, rng, T[m], T[n], 0.01) for m, n in pairs]
    pp = _with_edges(prob, pairs, mns)
    dev, lay, gposes, oposes = _compare(pkg, oracle, pp, 10)
    print("edges (circle): per-iteration cost vs oracle %.2e, solver %d" % (dev, lay.solver))
    assert np.abs(gposes[:, 4:] - oposes[:, 4:]).max() < 1e-6


def _sphere_edges(pkg, oracle, n_cam, n_pt, n_edges, seed):
    rng = np.random.default_rng(seed)
    prob = pkg.synth.generate(pkg.synth.SPHERE, n_cam=n_cam, n_pt=n_pt, seed=pkg.synth.BASE_SEED + 1)
    T = prob.poses_true
    pairs = [(int(a), int(b)) for a, b in rng.integers(0, prob.n_cam, size=(n_edges, 2)) if a != b]
    return _with_edges(prob, pairs, [_noisy_rel(oracle, rng, T[m], T[n], 0.005) for m, n in pairs])


def test_edges_sphere_dense(pkg, oracle):
    """Random edges on a 30-camera sphere (dense S of 174 rows: the one-CTA
    float-float solver)."""
    pp = _sphere_edges(pkg, oracle, 30, 6000, 20, 6)
    dev, lay, _, _ = _compare(pkg, oracle, pp, 6, threads=16)
    print("edges (30-camera sphere): per-iteration cost vs oracle %.2e, solver %d" % (dev, lay.solver))
    assert lay.solver == pkg.native.SOLVER_DENSE_SMALL


def test_edges_sphere_cluster_solver_precision_limit(pkg, oracle):
    """The measured limit of larger dense systems with edges: the cluster
    solver factors the Jacobi-scaled S in FP32 and refines against the
    float-float S; the edges hold the scale ~1e6 times more weakly than the
    pixel terms, and the refinement leaves ~1e-4 of the cost along that
    direction (594 rows, 40 random edges).  The bar here is that limit, not
    the parity bar."""
    pp = _sphere_edges(pkg, oracle, 100, 20000, 40, 6)
    params = fixed_iter_params(pkg, 6, pp.initial_lm_damping)
    with pkg.native.Problem(pp, device=0) as gp:
        grecs, _ = gp.optimize(params)
        lay = gp.layout()
    orecs, _, _ = oracle.optimize(pp, params, n_threads=16)
    g = np.array([r.merit for r in grecs])
    o = np.array([r.merit for r in orecs])
    dev = float(np.max(np.abs(g - o) / o))
    print("edges (100-camera sphere, cluster solver): per-iteration cost vs oracle %.2e" % dev)
    assert lay.solver == pkg.native.SOLVER_DENSE_CLUSTER
    assert abs(g[0] - o[0]) / o[0] < 1e-9 and dev < 1e-3


def test_loop_closure_edge_band_solver(pkg, oracle):
    """A 100-camera loop with edges between cameras that share no point: the
    edges' blocks of S lie outside the band of the tracks, in the rows of the
    last cameras (the dense border of the banded solver)."""
    rng = np.random.default_rng(7)
    prob = pkg.synth.generate(pkg.synth.LOOP, n_cam=100, n_pt=8000, seed=pkg.synth.BASE_SEED + 32)
    T = prob.poses_true
    pairs = [(5, 80), (20, 90), (45, 95)]
    pp = _with_edges(prob, pairs, [_noisy_rel(oracle, rng, T[m], T[n], 0.002) for m, n in pairs])
    with pkg.native.Problem(pp, device=0) as gp:
        (_, _), (sr, sc) = gp.export_pattern()
        blocks = set(zip(sr.tolist(), sc.tolist()))
    # free blocks are the poses after the constant camera 0: pose j -> block j - 1
    for m, n in pairs:
        assert (max(m, n) - 1, min(m, n) - 1) in blocks
    dev, lay, _, _ = _compare(pkg, oracle, pp, 6, threads=16)
    print("edges (loop): per-iteration cost vs oracle %.2e, solver %d" % (dev, lay.solver))


def test_edges_with_priors_and_checks(pkg, oracle):
    """Edges and priors together; invalid edges are refused at creation."""
    rng = np.random.default_rng(8)
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=6, n_pt=200, seed=pkg.synth.BASE_SEED + 33)
    prob.pose_const = np.zeros(6, np.uint8)
    T = prob.poses_true
    pairs = [(0, 1), (1, 2), (4, 5)]
    pp = _with_edges(prob, pairs, [_noisy_rel(oracle, rng, T[m], T[n], 0.01) for m, n in pairs])
    pp.prior_pose = np.array([0], np.int32)
    pp.prior_mean = T[:1].copy()
    pp.prior_precision = np.array([1e3 * np.eye(6)])
    params = fixed_iter_params(pkg, 8, pp.initial_lm_damping)
    with pkg.native.Problem(pp, device=0) as gp:
        gp.set_pose_priors(pp.prior_pose, pp.prior_mean, pp.prior_precision)
        grecs, _ = gp.optimize(params)
    orecs, _, _ = oracle.optimize(pp, params, n_threads=8)
    g = np.array([r.merit for r in grecs])
    o = np.array([r.merit for r in orecs])
    assert np.max(np.abs(g - o) / o) < COST_RTOL
    for bad_pairs, bad_mn in (([(2, 2)], [T[0]]), ([(0, 6)], [T[0]]), ([(0, 1)], [np.r_[2.0, 0, 0, 0, 0, 0, 0]])):
        with pytest.raises(pkg.native.SgbaError):
            pkg.native.Problem(_with_edges(prob, bad_pairs, bad_mn), device=0)
