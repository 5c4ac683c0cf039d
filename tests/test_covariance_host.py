"""Covariance queries on the CPU: the oracle's restatement of
SchurFactor::inverse_block (schur_ldlt.rs:815-957) with the pose priors and
pose-graph edges in H, against the inverse of the oracle's dense undamped H;
and the Python mirror's OptimizationSolution.covariance_block /
precision_block mapping of family names to query kinds (the reference's
optimizer_types.rs:277-370), with a stand-in for the device problem."""
import numpy as np
import pytest


def _prior_edge_problem(pkg, oracle):
    rng = np.random.default_rng(9)
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=5, n_pt=60, seed=pkg.synth.BASE_SEED + 54)
    prob.pose_const = np.zeros(5, np.uint8)
    T = prob.poses_true
    pairs = [(0, 1), (1, 2), (3, 4), (4, 0)]
    mns = []
    for m, n in pairs:
        rel = oracle.se3_mul(oracle.se3_inverse(T[m]), T[n])
        mns.append(oracle.se3_mul(oracle.se3_exp(0.01 * rng.standard_normal(6)), rel))
    P = prob.copy()
    P.edge_pose = np.array(pairs, np.int32)
    P.edge_mn = np.array(mns, float)
    P.prior_pose = np.array([0, 1], np.int32)
    P.prior_mean = T[:2].copy()
    P.prior_precision = np.array([1e4 * np.eye(6)] * 2)
    return P


def test_oracle_covariance_with_priors_and_edges_vs_dense_inverse(pkg, oracle):
    """Every pose free, priors on poses 0 and 1, edges: the oracle's blocks
    through the Schur complement equal the blocks of the dense H^-1."""
    prob = _prior_edge_problem(pkg, oracle)
    H, _ = oracle.dense_system(prob, 0.0)
    cov = np.linalg.inv(H)
    nf = prob.n_cam
    pose = lambda j: slice(6 * j, 6 * j + 6)
    point = lambda q: slice(6 * nf + 3 * q, 6 * nf + 3 * q + 3)
    scale = np.abs(cov[:6 * nf, :6 * nf]).max()
    for row, col, rs, cs in (((1, 2), (1, 2), pose(2), pose(2)), ((1, 0), (1, 4), pose(0), pose(4)),
                             ((1, 3), (2, 7), pose(3), point(7)), ((2, 7), (2, 7), point(7), point(7)),
                             ((2, 5), (2, 9), point(5), point(9))):
        blk = oracle.covariance_block(prob, row, col)
        np.testing.assert_allclose(blk, cov[rs, cs], rtol=1e-7, atol=1e-9 * scale, err_msg=str((row, col)))


class _FakeNative:
    """Records the queries the solution makes (no device)."""

    def __init__(self):
        self.prepared = 0
        self.calls = []

    def covariance_prepare(self):
        self.prepared += 1

    def covariance_block(self, row, col):
        self.calls.append(("cov", row, col))
        if row[0] == 0 or col[0] == 0:
            return None  # the device answers None for Conditioned camera params
        return np.zeros((6 if row[0] == 1 else 3, 6 if col[0] == 1 else 3))

    def precision_block(self, row, col):
        self.calls.append(("prec", row, col))
        return np.zeros((6 if row[0] == 1 else 3, 6 if col[0] == 1 else 3))

    def close(self):
        pass


def test_solution_maps_family_names_to_query_kinds(pkg):
    fake = _FakeNative()
    sol = pkg.OptimizationSolution(None, 0.0, [], fake, ["cams", "poses", "points"])
    assert sol.covariance_block("poses", 3, "points", 11).shape == (6, 3)
    assert sol.precision_block("points", 2, "points", 2).shape == (3, 3)
    assert sol.covariance_block("cams", 0, "poses", 1) is None  # the camera family goes to the device as kind 0
    assert sol.covariance_block("poses", 1, "no_such_family", 0) is None
    assert fake.prepared == 1  # prepared once, on the first query
    assert fake.calls == [("cov", (1, 3), (2, 11)), ("prec", (2, 2), (2, 2)), ("cov", (0, 0), (1, 1))]
    with pytest.raises(pkg.NllsError):
        pkg.OptimizationSolution(None, 0.0, []).covariance_block("poses", 1, "poses", 1)


def test_oracle_covariance_free_pinhole_params_vs_dense_inverse(pkg, oracle):
    """Free pinhole params (4, the oracle's camera block padded to 6 rows in S):
    camera, pose and point blocks against the dense H^-1, whose camera block
    has the 4 real rows first."""
    from test_oracle_free_intrinsics import _problem

    prob, _, _ = _problem(pkg, seed=3, free=True)
    H, _ = oracle.dense_system(prob, 0.0)
    cov = np.linalg.inv(H)
    c0 = 4
    nf = int(np.sum(prob.pose_const == 0))
    fidx = np.cumsum(prob.pose_const == 0) - 1
    cam = slice(0, c0)
    pose = lambda j: slice(c0 + 6 * fidx[j], c0 + 6 * fidx[j] + 6)
    point = lambda q: slice(c0 + 6 * nf + 3 * q, c0 + 6 * nf + 3 * q + 3)
    scale = np.abs(cov).max()
    for row, col, rs, cs in (((0, 0), (0, 0), cam, cam), ((0, 0), (1, 3), cam, pose(3)),
                             ((2, 4), (0, 0), point(4), cam), ((1, 2), (2, 4), pose(2), point(4)),
                             ((2, 4), (2, 6), point(4), point(6))):
        blk = oracle.covariance_block(prob, row, col)
        np.testing.assert_allclose(blk, cov[rs, cs], rtol=1e-7, atol=1e-9 * scale, err_msg=str((row, col)))
