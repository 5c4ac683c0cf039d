"""The enhanced unified camera model (EUCM) on the GPU, the camera of the
reference's BA example problem (EucmCameraReprojectionCostTerm,
crates/sophus_opt/src/example_problems/ba_problem.rs:69-110; the camera
crates/sophus_sensor/src/distortions/enhanced_unified.rs:55-215), with its
params Conditioned (kinds C, F, M) and Free (kinds F, F, M).

Checked against the oracle (camera_model 1, oracle/sgba_oracle.cpp): J_pose
and J_point per term against the oracle's analytic f64 Jacobians (themselves
checked against central differences on the CPU), the per-iteration cost
within 1e-6 relative, the LM step against an f64 solve of the exported
reduced system, the reference's ba_converges bars, and the Python mirror with
an EnhancedUnifiedCameraF64 family."""
import numpy as np
import pytest

from conftest import fixed_iter_params

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-6
FP32_TOL = 1e-5
DD_TOL = 1e-10
# the reference's true / initial EUCM params (ba_problem.rs:162-166,294-304)
EUCM_TRUE = np.array([300.0, 300.0, 320.0, 240.0, 0.5, 1.0])
EUCM_INIT = np.array([297.0, 297.0, 321.0, 241.0, 0.495, 1.0])


def _rotations(q):
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((len(q), 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - w * z)
    R[:, 0, 2] = 2 * (x * z + w * y)
    R[:, 1, 0] = 2 * (x * y + w * z)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - w * x)
    R[:, 2, 0] = 2 * (x * z - w * y)
    R[:, 2, 1] = 2 * (y * z + w * x)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def _eucm_uv(params, poses, points, cams, pts):
    """EUCM projection of every observation (enhanced_unified.rs:59-88)."""
    fx, fy, cx, cy, alpha, beta = params
    T = poses[cams]
    xc = np.einsum("kji,kj->ki", _rotations(T[:, :4]), points[pts] - T[:, 4:])
    x, y = xc[:, 0] / xc[:, 2], xc[:, 1] / xc[:, 2]
    rho = np.sqrt(beta * (x * x + y * y) + 1.0)
    norm = alpha * rho + (1.0 - alpha)
    return np.stack([fx * x / norm + cx, fy * y / norm + cy], axis=1)


def _eucm_scene(pkg, kind, seed, free, fix_two=False, **kw):
    """A synthetic scene observed through the reference's true EUCM camera
    (uniform noise of +-0.075 px), started from its initial params."""
    prob = pkg.synth.generate(kind, seed=seed, **kw)
    uv = _eucm_uv(EUCM_TRUE, prob.poses_true, prob.points_true, prob.obs_cam, prob.obs_pt)
    prob.obs_uv = uv + 0.15 * (np.random.default_rng(seed).random(uv.shape) - 0.5)
    if fix_two:  # ba_problem.rs: poses 0 and 1 fixed at the truth (no gauge left)
        prob.poses[:2] = prob.poses_true[:2]
        prob.pose_const[:2] = 1
    prob.intrinsics = EUCM_INIT[:4].copy()
    prob.camera_model = pkg.native.CAMERA_EUCM
    prob.eucm_alpha_beta = EUCM_INIT[4:].copy()
    prob.intrinsics_free = free
    return prob


def _rel_err(g, o):
    scale = np.maximum(np.abs(o).reshape(len(o), -1).max(axis=1), 1e-300)
    return np.abs(g - o).reshape(len(o), -1).max(axis=1) / scale


def test_eucm_jacobians_match_oracle(pkg, oracle):
    prob = _eucm_scene(pkg, pkg.synth.CIRCLE, pkg.synth.BASE_SEED, free=False)
    intr6 = EUCM_INIT
    cams, pts = prob.obs_cam, prob.obs_pt
    ojp = np.empty((prob.n_obs, 2, 6))
    ojm = np.empty((prob.n_obs, 2, 3))
    for k in range(prob.n_obs):
        _, ojp[k], ojm[k], _ = oracle.eval_term_ex(prob.poses[cams[k]], prob.points[pts[k]], intr6, 1,
                                                   prob.obs_uv[k])
    errs = {}
    with pkg.native.Problem(prob, device=0) as gp:
        for prec, tol in ((0, FP32_TOL), (1, DD_TOL)):
            gjp, gjm = gp.jacobians(cams, pts, precision=prec)
            e = np.maximum(_rel_err(gjp, ojp), _rel_err(gjm, ojm))
            errs[prec] = float(e.max())
            assert e.max() < tol, (prec, e.max(), int(np.argmax(e)))
    print("EUCM, every term of config 0: max rel entry error FP32 %.2e, float-float %.2e" % (errs[0], errs[1]))


@pytest.mark.parametrize("kind,n_iter,free", [(0, 10, False), (0, 10, True), (1, 6, False), (1, 6, True)])
def test_eucm_trajectory_matches_oracle(pkg, oracle, kind, n_iter, free):
    prob = _eucm_scene(pkg, kind, pkg.synth.BASE_SEED + kind, free)
    params = fixed_iter_params(pkg, n_iter, prob.initial_lm_damping)
    with pkg.native.Problem(prob, device=0) as gp:
        assert gp.layout().intrinsics_rows == (6 if free else 0)
        grecs, _ = gp.optimize(params)
        gposes, gpoints = gp.variables()
        gintr = gp.intrinsics()
    orecs, oposes, opoints, ointr = oracle.optimize(prob, params, n_threads=8, with_intrinsics=True)
    g = np.array([r.merit for r in grecs])
    o = np.array([r.merit for r in orecs])
    dev = np.abs(g - o) / o
    print("EUCM kind %d free %d: per-iteration cost deviation max %.2e; params gpu %s oracle %s"
          % (kind, free, dev.max(), gintr, ointr))
    assert len(g) == len(o) == n_iter
    assert dev.max() < COST_RTOL
    assert len(gintr) == 6
    if free:
        assert g[-1] < 0.5 * g[0]  # the initial params are corrected
        np.testing.assert_allclose(gintr, ointr, rtol=1e-5)
    else:
        np.testing.assert_array_equal(gintr, EUCM_INIT)
    assert np.abs(gpoints - opoints).max() < 1e-4 * max(1.0, np.abs(opoints).max())


def test_eucm_free_step_vs_f64_solve(pkg):
    prob = _eucm_scene(pkg, pkg.synth.CIRCLE, pkg.synth.BASE_SEED, free=True)
    with pkg.native.Problem(prob, device=0) as gp:
        gp.init(fixed_iter_params(pkg, 5, prob.initial_lm_damping))
        errs = []
        for _ in range(3):
            poses, _ = gp.variables()
            gp.step()
            S, rhs, delta = gp.last_system()
            x64 = np.linalg.solve(S, rhs)
            n = S.shape[0]
            c = poses[np.where(prob.pose_const == 1)[0][0], 4:]
            v = np.zeros(n)
            for k, j in enumerate(np.where(prob.pose_const == 0)[0]):
                v[6 + 6 * k + 3:6 + 6 * k + 6] = poses[j, 4:] - c
            v /= np.linalg.norm(v)
            proj = lambda x: x - v * (v @ x)  # noqa: E731
            errs.append(np.linalg.norm(proj(delta[:n]) - proj(x64)) / np.linalg.norm(proj(x64)))
            assert np.any(delta[4:6] != 0.0)  # alpha and beta move: no padding rows
    print("EUCM free: step error vs f64 solve", errs)
    assert max(errs) < 1e-6


def test_eucm_ba_converges_reference_configuration(pkg, oracle):
    """ba_problem.rs:517-547: EUCM params free from the reference's initial
    values, poses 0 and 1 fixed, 20 iterations at initial damping 1.0; pose
    RMS < 0.01 and point RMS < 0.1, and the trajectory equals the oracle's."""
    params = pkg.OptParams(num_iterations=20, initial_lm_damping=1.0, function_tolerance=0.0, gradient_tolerance=0.0,
                           parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)
    for seed in (pkg.synth.BASE_SEED, 5):
        prob = _eucm_scene(pkg, pkg.synth.CIRCLE, seed, free=True, fix_two=True, n_cam=4, n_pt=20)
        with pkg.native.Problem(prob, device=0) as gp:
            grecs, _ = gp.optimize(params)
            poses, points = gp.variables()
            gintr = gp.intrinsics()
        pose_rms = np.sqrt(np.mean(np.sum((poses[:, 4:] - prob.poses_true[:, 4:]) ** 2, axis=1)))
        pt_rms = np.sqrt(np.mean(np.sum((points - prob.points_true) ** 2, axis=1)))
        assert pose_rms < 0.01 and pt_rms < 0.1, (seed, pose_rms, pt_rms)
        orecs, _, _, ointr = oracle.optimize(prob, params, with_intrinsics=True)
        g = np.array([r.merit for r in grecs])
        o = np.array([r.merit for r in orecs])
        assert np.max(np.abs(g - o) / np.maximum(o, 1e-300)) < COST_RTOL
        assert abs(gintr[0] - EUCM_TRUE[0]) < abs(EUCM_INIT[0] - EUCM_TRUE[0])


def test_python_mirror_eucm_camera_family(pkg, oracle):
    prob = _eucm_scene(pkg, pkg.synth.CIRCLE, pkg.synth.BASE_SEED + 7, free=True, n_cam=8, n_pt=300)
    K = pkg.VarKind
    cam = pkg.EnhancedUnifiedCameraF64(EUCM_INIT)
    variables = (pkg.VarBuilder.new()
                 .add_family("cams", pkg.VarFamily.new(K.Free, [cam]))
                 .add_family("poses", pkg.VarFamily.new_with_const_ids(
                     K.Free, [pkg.Isometry3F64(p) for p in prob.poses], [0]))
                 .add_family("points", pkg.VarFamily.new(K.Marginalized, prob.points))
                 .build())
    idx = np.stack([np.zeros(prob.n_obs, np.int64), prob.obs_cam, prob.obs_pt], axis=1)
    terms = pkg.CostTerms.new(["cams", "poses", "points"], pkg.EucmReprojectionTerms(prob.obs_uv, idx))
    cost = pkg.CostFn.new_boxed_robust((), terms, pkg.RobustKernel.Huber(pkg.HuberKernel.new(1.0)))
    params = fixed_iter_params(pkg, 8, 1e-4)
    sol = pkg.optimize_nlls(variables, [cost], [], params)
    orecs, _, _, ointr = oracle.optimize(prob, params, with_intrinsics=True)
    g = np.array([s.merit for s in sol.steps])
    o = np.array([r.merit for r in orecs])
    assert np.max(np.abs(g - o) / o) < COST_RTOL
    out = sol.variables.get_members("cams")[0]
    assert isinstance(out, pkg.EnhancedUnifiedCameraF64)
    np.testing.assert_allclose(out.params, ointr, rtol=1e-5)


@pytest.mark.parametrize("free", [True, False])
def test_eucm_reference_benchmark_scene(pkg, oracle, free):
    """The scene of the reference's BA benchmark (BaProblem::new(10, 500):
    ring of 10 cameras around an open box, EUCM camera, no robust kernel, 20
    iterations at damping 1.0, poses 0 and 1 fixed), params Free (ba_bench's
    "free" rows) or Conditioned at the truth ("conditioned" rows): the
    per-iteration cost equals the oracle's, and the ba_converges bars hold."""
    prob = pkg.synth.ring_box_eucm(intrinsics_free=free)
    if not free:
        prob.intrinsics = prob.intrinsics_true[:4].copy()
        prob.eucm_alpha_beta = prob.intrinsics_true[4:].copy()
    params = pkg.OptParams(num_iterations=20, initial_lm_damping=1.0, function_tolerance=0.0, gradient_tolerance=0.0,
                           parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)
    with pkg.native.Problem(prob, device=0) as gp:
        grecs, _ = gp.optimize(params)
        poses, points = gp.variables()
        gintr = gp.intrinsics()
    orecs, _, _, ointr = oracle.optimize(prob, params, n_threads=8, with_intrinsics=True)
    g = np.array([r.merit for r in grecs])
    o = np.array([r.merit for r in orecs])
    dev = np.abs(g - o) / o
    pose_rms = np.sqrt(np.mean(np.sum((poses[:, 4:] - prob.poses_true[:, 4:]) ** 2, axis=1)))
    pt_rms = np.sqrt(np.mean(np.sum((points - prob.points_true) ** 2, axis=1)))
    print("ring-box EUCM free %d: cost deviation max %.2e, pose RMS %.2e, point RMS %.2e, params %s"
          % (free, dev.max(), pose_rms, pt_rms, gintr))
    assert len(g) == len(o) == 20 and dev.max() < COST_RTOL
    assert pose_rms < 0.01 and pt_rms < 0.1
    np.testing.assert_allclose(gintr, ointr, rtol=1e-5)
