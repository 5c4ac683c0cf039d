"""Free pinhole intrinsics on the GPU (the reference's kinds (F, F, M): the
"cams" family Free, J_cam of PinholeCameraReprojectionCostTerm,
crates/sophus_opt/src/nlls/functor_library/costs/pinhole_reprojection.rs:85;
the reference's ba_converges runs this configuration with its own camera,
crates/sophus_opt/src/example_problems/ba_problem.rs:517-547).

Checked against the oracle (intrinsics_free, oracle/sgba_oracle.cpp):
per-iteration cost within 1e-6 relative, the final intrinsics, the LM step
against an f64 solve of the exported reduced system (intrinsics block first,
as the reference orders its families), the reduced-system pattern, the
Python mirror with a Free camera family, and the configurations rejected."""
import numpy as np
import pytest

from conftest import fixed_iter_params

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-6


def _free(pkg, kind=0, seed_off=0, **kw):
    prob = pkg.synth.generate(kind, seed=pkg.synth.BASE_SEED + seed_off, **kw)
    prob.intrinsics = prob.intrinsics * np.array([1.02, 0.985, 1.0, 1.0]) + np.array([0.0, 0.0, 3.0, -2.0])
    prob.intrinsics_free = True
    return prob


@pytest.mark.parametrize("kind,n_iter", [(0, 10), (1, 6)])
def test_free_intrinsics_trajectory_matches_oracle(pkg, oracle, kind, n_iter):
    prob = _free(pkg, kind, seed_off=kind)
    params = fixed_iter_params(pkg, n_iter, prob.initial_lm_damping)
    with pkg.native.Problem(prob, device=0) as gp:
        assert gp.layout().intrinsics_rows == 6
        grecs, _ = gp.optimize(params)
        gintr = gp.intrinsics()
    orecs, _, _, ointr = oracle.optimize(prob, params, n_threads=8, with_intrinsics=True)
    g = np.array([r.merit for r in grecs])
    o = np.array([r.merit for r in orecs])
    dev = np.abs(g - o) / o
    print("kind %d: per-iteration cost deviation %s; intrinsics gpu %s oracle %s" % (kind, dev, gintr, ointr[:4]))
    assert len(g) == len(o) == n_iter
    assert dev.max() < COST_RTOL
    # past convergence the cost is flat along the weakest intrinsics direction
    # (cy of a 10-camera circle moves by ~1e-3 px at a cost change of 1e-9), so
    # the parameters agree to 1e-5 relative where the costs agree to 1e-8
    assert np.all(np.abs(gintr - ointr[:4]) <= 1e-5 * np.abs(ointr[:4]))
    assert g[-1] < 0.5 * g[0]  # the wrong initial intrinsics are corrected


def test_free_intrinsics_step_vs_f64_solve(pkg):
    prob = _free(pkg, 0)
    with pkg.native.Problem(prob, device=0) as gp:
        gp.init(fixed_iter_params(pkg, 5, prob.initial_lm_damping))
        errs = []
        for _ in range(3):
            poses, _ = gp.variables()
            gp.step()
            S, rhs, delta = gp.last_system()
            x64 = np.linalg.solve(S, rhs)
            # outside the scale gauge (free poses' translations about the constant camera)
            n = S.shape[0]
            c = poses[np.where(prob.pose_const == 1)[0][0], 4:]
            v = np.zeros(n)
            for k, j in enumerate(np.where(prob.pose_const == 0)[0]):
                v[6 + 6 * k + 3:6 + 6 * k + 6] = poses[j, 4:] - c
            v /= np.linalg.norm(v)
            proj = lambda x: x - v * (v @ x)  # noqa: E731
            errs.append(np.linalg.norm(proj(delta[:n]) - proj(x64)) / np.linalg.norm(proj(x64)))
            assert np.all(delta[4:6] == 0.0)  # the padding rows of the intrinsics block
    print("free intrinsics: step error vs f64 solve", errs)
    assert max(errs) < 1e-6


def test_free_intrinsics_pattern(pkg):
    prob = _free(pkg, 0)
    with pkg.native.Problem(prob, device=0) as gp:
        lay = gp.layout()
        (hr, hc), (sr, sc) = gp.export_pattern()
    with pkg.native.Problem(_free(pkg, 0).copy(), device=0, intrinsics_free=False) as gp:
        lay0 = gp.layout()
        (hr0, hc0), (sr0, sc0) = gp.export_pattern()
    nf = lay.n_free_poses
    s_blocks = set(zip(sr.tolist(), sc.tolist()))
    assert (0, 0) in s_blocks and all((1 + j, 0) in s_blocks for j in range(nf))
    assert {(r + 1, c + 1) for r, c in zip(sr0.tolist(), sc0.tolist())} <= s_blocks
    assert len(sr) == lay.n_s_blocks == lay0.n_s_blocks + 1 + nf
    assert len(hr) == lay.n_h_blocks and all(r >= c for r, c in zip(hr.tolist(), hc.tolist()))


def test_python_mirror_free_camera_family(pkg, oracle):
    prob = _free(pkg, 0, seed_off=7, n_cam=8, n_pt=300)
    K = pkg.VarKind
    variables = (pkg.VarBuilder.new()
                 .add_family("cams", pkg.VarFamily.new(K.Free, [pkg.PinholeCameraF64(prob.intrinsics)]))
                 .add_family("poses", pkg.VarFamily.new_with_const_ids(
                     K.Free, [pkg.Isometry3F64(p) for p in prob.poses], [0]))
                 .add_family("points", pkg.VarFamily.new(K.Marginalized, prob.points))
                 .build())
    idx = np.stack([np.zeros(prob.n_obs, np.int64), prob.obs_cam, prob.obs_pt], axis=1)
    terms = pkg.CostTerms.new(["cams", "poses", "points"], pkg.PinholeReprojectionTerms(prob.obs_uv, idx))
    cost = pkg.CostFn.new_boxed_robust((), terms, pkg.RobustKernel.Huber(pkg.HuberKernel.new(1.0)))
    params = fixed_iter_params(pkg, 8, 1e-4)
    sol = pkg.optimize_nlls(variables, [cost], [], params)
    orecs, _, _, ointr = oracle.optimize(prob, params, with_intrinsics=True)
    g = np.array([s.merit for s in sol.steps])
    o = np.array([r.merit for r in orecs])
    assert np.max(np.abs(g - o) / o) < COST_RTOL
    cam = sol.variables.get_members("cams")[0]
    np.testing.assert_allclose(cam.params, ointr[:4], rtol=1e-6)


def test_free_intrinsics_rejected_configurations(pkg):
    E = pkg.native.SgbaError
    loop = pkg.synth.generate(pkg.synth.LOOP, n_cam=100, n_pt=3000, seed=pkg.synth.BASE_SEED + 2)
    with pytest.raises(E) as e:
        pkg.native.Problem(loop, device=0, intrinsics_free=True)
    assert e.value.status == pkg.native.ERR_UNSUPPORTED
    with pkg.native.Problem(_free(pkg, 0), device=0) as gp:
        with pytest.raises(E) as e:
            gp.set_linear_solver(pkg.native.LINSOLVE_PCG_BLOCK_JACOBI)
        assert e.value.status == pkg.native.ERR_UNSUPPORTED
