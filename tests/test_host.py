"""Host-side logic without a GPU: the synthetic generator and the sophus_opt
mirror's configuration checks (validate_solver_config,
crates/sophus_opt/src/nlls/optimizer.rs:649-717)."""
import numpy as np
import pytest


def test_synth_is_deterministic_and_shaped(pkg):
    a = pkg.synth.generate(pkg.synth.CIRCLE, seed=pkg.synth.BASE_SEED)
    b = pkg.synth.generate(pkg.synth.CIRCLE, seed=pkg.synth.BASE_SEED)
    for f in ("poses", "points", "obs_cam", "obs_pt", "obs_uv"):
        assert np.array_equal(getattr(a, f), getattr(b, f))
    assert a.n_cam == 10 and a.n_pt == 500 and 4000 < a.n_obs <= 5000
    assert a.pose_const[0] == 1 and a.pose_const[1:].sum() == 0
    np.testing.assert_allclose(np.linalg.norm(a.poses[:, :4], axis=1), 1.0, atol=1e-12)
    c = pkg.synth.generate(pkg.synth.CIRCLE, seed=pkg.synth.BASE_SEED + 1)
    assert not np.array_equal(a.obs_uv, c.obs_uv)


def test_synth_sphere_track_lengths(pkg):
    s = pkg.synth.generate(pkg.synth.SPHERE, seed=pkg.synth.BASE_SEED + 1)
    assert s.n_cam == 100 and s.n_pt == 20000
    L = np.bincount(s.obs_pt, minlength=s.n_pt)
    assert L.min() >= 2 and L.max() <= 40
    assert 400_000 < s.n_obs < 560_000
    # each point's cameras are distinct
    pairs = s.obs_pt.astype(np.int64) * 1000 + s.obs_cam
    assert np.unique(pairs).size == s.n_obs


def test_synth_loop_tracks_are_consecutive(pkg):
    s = pkg.synth.generate(pkg.synth.LOOP, n_cam=300, n_pt=3000, seed=pkg.synth.BASE_SEED + 2)
    order = np.lexsort((s.obs_cam, s.obs_pt))
    pt, cam = s.obs_pt[order], s.obs_cam[order]
    for i in range(0, 3000, 97):
        cams = cam[pt == i]
        assert 2 <= cams.size <= 25
        span = (cams.max() - cams.min()) if (cams.max() - cams.min()) < 150 else (cams.min() + 300 - cams.max())
        assert span <= 25


def _ba_vars(pkg, kinds, n=3):
    poses = [pkg.Isometry3F64.identity() for _ in range(n)]
    return (pkg.VarBuilder.new()
            .add_family("cams", pkg.VarFamily.new(kinds[0], [pkg.PinholeCameraF64([500, 500, 320, 240])]))
            .add_family("poses", pkg.VarFamily.new_with_const_ids(kinds[1], poses, [0]))
            .add_family("points", pkg.VarFamily.new(kinds[2], np.zeros((4, 3))))
            .build())


def _cost(pkg):
    terms = pkg.CostTerms.new(["cams", "poses", "points"],
                              [pkg.PinholeCameraReprojectionCostTerm([320.0, 240.0], [0, 1, 0])])
    return pkg.CostFn.new_boxed_robust((), terms, pkg.RobustKernel.Huber(pkg.HuberKernel.new(1.0)))


def test_config_errors_mirror_reference(pkg):
    K = pkg.VarKind
    schur = pkg.OptParams(solver=pkg.LinearSolverEnum.SchurBlockSparseLdlt)
    with pytest.raises(pkg.SchurMissingFreeOrMarg):
        pkg.optimize_nlls(_ba_vars(pkg, (K.Conditioned, K.Free, K.Free)), [_cost(pkg)], [], schur)
    with pytest.raises(pkg.SchurCostConnectsTwoMargFamilies):
        pkg.optimize_nlls(_ba_vars(pkg, (K.Free, K.Marginalized, K.Marginalized)), [_cost(pkg)], [], schur)
    with pytest.raises(pkg.NotOnGpuPath):
        pkg.optimize_nlls(_ba_vars(pkg, (K.Conditioned, K.Free, K.Marginalized)), [_cost(pkg)], [],
                          pkg.OptParams())  # default solver is FaerSparseLdlt, not Schur
    with pytest.raises(pkg.NotOnGpuPath):
        pkg.optimize_nlls(_ba_vars(pkg, (K.Conditioned, K.Free, K.Marginalized)), [_cost(pkg)], ["eq"], schur)


def test_opt_params_defaults_match_reference(pkg):
    p = pkg.OptParams()  # optimizer_types.rs:226-240
    assert (p.num_iterations, p.initial_lm_damping, p.parallelize, p.skip_final_hessian) == (100, 10.0, True, False)
    assert (p.function_tolerance, p.gradient_tolerance, p.parameter_tolerance) == (1e-10, 1e-14, 1e-12)
    assert p.max_consecutive_rejects == 20
    assert p.solver == pkg.LinearSolverEnum.FaerSparseLdlt and not p.solver.is_schur()
    assert pkg.LinearSolverEnum.SchurBlockSparseLdlt.is_schur()


def test_isometry_params_validation(pkg):
    with pytest.raises(ValueError):
        pkg.Isometry3F64([0.9, 0, 0, 0, 0, 0, 0])
    p = pkg.Isometry3F64([-1.0, 0, 0, 0, 1, 2, 3])  # disambiguated to w >= 0
    assert p.params()[0] == 1.0 and list(p.translation()) == [1, 2, 3]


def test_huber_kernel_matches_reference_formula(pkg):
    k = pkg.HuberKernel.new(1.0)
    assert k.apply(0.5) == 0.25 and k.apply(3.0) == 5.0
    assert k.weight(0.0) == 0.0 and abs(k.weight(3.0) - np.sqrt(5.0) / 3.0) < 1e-15


def test_concurrent_validation_reports_first_bad_observation(pkg):
    """sgba_problem_create validates observations in parallel chunks on the
    host worker pool; the error names the first bad observation, as a
    sequential scan would, also with several host threads creating problems
    at once (their parallel regions share the pool). No CUDA call is reached."""
    import threading

    base = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=10, n_pt=6000, seed=pkg.synth.BASE_SEED + 7)
    assert base.n_obs > 40000  # several chunks of the parallel scan
    E = pkg.native.SgbaError
    errors = []

    def worker(t):
        try:
            for r in range(8):
                first = 1000 + 5000 * t + 37 * r
                bad = base.copy()
                bad.obs_pt[base.n_obs - 3] = base.n_pt + 1  # a later bad one, in another chunk
                bad.obs_pt[first] = base.n_pt
                try:
                    pkg.native.Problem(bad, device=0)
                    errors.append("thread %d: no error" % t)
                except E as e:
                    if e.status != pkg.native.ERR_INVALID_ARGUMENT or "observation %d:" % first not in e.message:
                        errors.append("thread %d: %s" % (t, e.message))
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append("thread %d: %r" % (t, e))

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors


def test_prior_cost_fn_checks_before_any_gpu_call(pkg):
    """The mirror accepts one Isometry3PriorCostTerm CostFn on the reprojection
    cost's pose family, without a robust kernel; other shapes raise
    NotOnGpuPath before a problem is created."""
    prob = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=4, n_pt=20, seed=7)
    K = pkg.VarKind
    variables = (pkg.VarBuilder.new()
                 .add_family("cams", pkg.VarFamily.new(K.Conditioned, [pkg.PinholeCameraF64(prob.intrinsics)]))
                 .add_family("poses", pkg.VarFamily.new_with_const_ids(
                     K.Free, [pkg.Isometry3F64(p) for p in prob.poses], [0]))
                 .add_family("points", pkg.VarFamily.new(K.Marginalized, prob.points))
                 .build())
    idx = np.stack([np.zeros(prob.n_obs, np.int64), prob.obs_cam, prob.obs_pt], axis=1)
    reproj = pkg.CostFn.new_boxed(
        None, pkg.CostTerms.new(["cams", "poses", "points"], pkg.PinholeReprojectionTerms(prob.obs_uv, idx)))
    term = pkg.Isometry3PriorCostTerm(prob.poses[1], np.eye(6), [1])
    prior = pkg.CostFn.new_boxed(None, pkg.CostTerms.new(["poses"], [term]))
    assert isinstance(prior.cost_terms.terms, pkg.PriorTerms) and len(prior.cost_terms.terms) == 1
    params = pkg.OptParams(num_iterations=2, solver=pkg.LinearSolverEnum.SchurBlockSparseLdlt)
    with pytest.raises(pkg.NotOnGpuPath):
        pkg.optimize_nlls(variables, [reproj, prior, prior], [], params)
    robust = pkg.CostFn.new_boxed_robust(None, pkg.CostTerms.new(["poses"], [term]),
                                         pkg.RobustKernel.Huber(pkg.HuberKernel.new(1.0)))
    with pytest.raises(pkg.NotOnGpuPath):
        pkg.optimize_nlls(variables, [reproj, robust], [], params)
    other = pkg.CostFn.new_boxed(None, pkg.CostTerms.new(["cams"], [term]))
    with pytest.raises(pkg.NotOnGpuPath):
        pkg.optimize_nlls(variables, [reproj, other], [], params)
