"""Batched optimisation of independent local windows (5-40 cameras, 200-4000
points per window) through sgba_batch_optimize.

Every window must come out exactly as sgba_optimize computes it alone: the
batched launches run each window's blocks with the kernel bodies and grids of
its own launches, so the results are bit-identical whatever the batch holds
and whichever schedule the autotuner picks; and every window matches the
oracle per iteration within the parity tolerance."""
import os
import numpy as np
import pytest

from conftest import fixed_iter_params

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-6


def _windows(pkg, n):
    return [pkg.synth.generate(pkg.synth.WINDOW, seed=pkg.synth.BASE_SEED + 3 + w) for w in range(n)]


def test_batch_equals_single_and_oracle(pkg, oracle):
    wins = _windows(pkg, 6)
    params = fixed_iter_params(pkg, 10, wins[0].initial_lm_damping)
    probs = [pkg.native.Problem(w, device=0) for w in wins]
    try:
        out = pkg.native.batch_optimize(probs, params)
        stats = pkg.native.batch_last_stats()
        batch_vars = [p.variables() for p in probs]
    finally:
        for p in probs:
            p.close()
    assert stats["batched_windows"] == len(wins) and stats["kernel_launches"] > 0
    for w, (recs, term, ms, final_cost, status) in enumerate(out):
        assert status == pkg.native.OK
        assert term == pkg.native.TERM_MAX_ITERATIONS and len(recs) == 10
        assert ms > 0.0 and np.isfinite(final_cost)
        with pkg.native.Problem(wins[w], device=0) as gp:
            srecs, sterm = gp.optimize(params)
            sposes, spoints = gp.variables()
        assert [r.merit for r in recs] == [r.merit for r in srecs]
        assert np.array_equal(batch_vars[w][0], sposes) and np.array_equal(batch_vars[w][1], spoints)
        assert final_cost == srecs[-1].merit
    for w in (0, 2, 3):  # 9, 34 and 5 cameras
        orecs, _, _ = oracle.optimize(wins[w], params, n_threads=8)
        g = np.array([r.merit for r in out[w][0]])
        o = np.array([r.merit for r in orecs])
        assert np.max(np.abs(g - o) / o) < COST_RTOL


def test_batch_reports_per_window_errors(pkg):
    good = _windows(pkg, 1)[0]
    bad = good.copy()
    bad.point_const = np.ones(bad.n_pt, np.uint8)  # nothing marginalized: the Schur solver refuses it
    params = fixed_iter_params(pkg, 3, good.initial_lm_damping)
    with pkg.native.Problem(good, device=0) as p0, pkg.native.Problem(bad, device=0) as p1:
        out = pkg.native.batch_optimize([p0, p1], params)
    assert out[0][4] == pkg.native.OK and len(out[0][0]) == 3
    assert out[1][4] == pkg.native.ERR_SCHUR_MISSING_FREE_OR_MARG


def test_mixed_sizes_keep_launch_limits(pkg):
    """Kernel launch limits (dynamic shared memory) are per function and per
    device, shared by every problem in the process: creating a small problem
    after a large one has captured its iteration graph must not break the
    large one's launches."""
    big = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=40, n_pt=4000, seed=pkg.synth.BASE_SEED + 41)
    small = pkg.synth.generate(pkg.synth.CIRCLE, n_cam=5, n_pt=200, seed=pkg.synth.BASE_SEED + 42)
    params = fixed_iter_params(pkg, 3, big.initial_lm_damping)
    with pkg.native.Problem(big, device=0) as gb:
        first, _ = gb.optimize(params)
        with pkg.native.Problem(small, device=0) as gs:
            gs.optimize(fixed_iter_params(pkg, 3, small.initial_lm_damping))
        second, _ = gb.optimize(params)
    assert len(first) == len(second) == 3
    assert np.isfinite(second[-1].merit)


def test_batch_graph_reuse_and_recapture(pkg):
    """Repeated batches over the same windows reuse the batched graphs and give
    bit-identical results; more iterations (larger record buffers, graphs
    captured again) still match the windows optimised one by one."""
    wins = _windows(pkg, 4)
    p10 = fixed_iter_params(pkg, 10, wins[0].initial_lm_damping)
    p12 = fixed_iter_params(pkg, 12, wins[0].initial_lm_damping)
    probs = [pkg.native.Problem(w, device=0) for w in wins]
    try:
        first = pkg.native.batch_optimize(probs, p10)
        for p, w in zip(probs, wins):
            p.set_variables(w.poses, w.points)
        again = pkg.native.batch_optimize(probs, p10)
        for a, b in zip(first, again):
            assert [r.merit for r in a[0]] == [r.merit for r in b[0]] and a[3] == b[3]
        for p, w in zip(probs, wins):
            p.set_variables(w.poses, w.points)
        longer = pkg.native.batch_optimize(probs, p12)
    finally:
        for p in probs:
            p.close()
    for w, (recs, term, ms, final_cost, status) in enumerate(longer):
        assert status == pkg.native.OK and len(recs) == 12
        with pkg.native.Problem(wins[w], device=0) as gp:
            srecs, _ = gp.optimize(p12)
        assert [r.merit for r in recs] == [r.merit for r in srecs]


def _run_batch(pkg, wins, params, free=()):
    probs = [pkg.native.Problem(w, device=0, intrinsics_free=(k in free)) for k, w in enumerate(wins)]
    try:
        out = pkg.native.batch_optimize(probs, params)
        stats = pkg.native.batch_last_stats()
        variables = [p.variables() for p in probs]
    finally:
        for p in probs:
            p.close()
    return out, stats, variables


def test_every_schedule_gives_the_same_results(pkg, monkeypatch):
    """The schedules the autotuner chooses from (window groups on separate
    streams, windows ordered by work or as given) change only which CTAs run
    side by side: each one reproduces the windows bit for bit."""
    wins = _windows(pkg, 9)
    params = fixed_iter_params(pkg, 5, wins[0].initial_lm_damping)
    runs = []
    for sc, groups in enumerate((1, 2, 4, 1)):
        monkeypatch.setenv("SGBA_BATCH_SCHEDULE", str(sc))
        out, stats, variables = _run_batch(pkg, wins, params)
        assert stats["schedule"] == sc and stats["groups"] == groups and stats["batched_windows"] == 9
        assert all(o[4] == pkg.native.OK for o in out)
        runs.append((out, variables))
    monkeypatch.delenv("SGBA_BATCH_SCHEDULE")
    ref_out, ref_vars = runs[0]
    for out, variables in runs[1:]:
        for w in range(len(wins)):
            assert [r.merit for r in out[w][0]] == [r.merit for r in ref_out[w][0]]
            assert np.array_equal(variables[w][0], ref_vars[w][0]) and np.array_equal(variables[w][1], ref_vars[w][1])


def test_mixed_batch_runs_batched_and_stream_windows(pkg):
    """Windows the batched launches do not cover (free intrinsics here) run on
    their own streams in the same call; both kinds equal their single runs."""
    wins = _windows(pkg, 4)
    params = fixed_iter_params(pkg, 6, wins[0].initial_lm_damping)
    out, stats, variables = _run_batch(pkg, wins, params, free=(1, 3))
    assert stats["batched_windows"] == 2
    for w, win in enumerate(wins):
        assert out[w][4] == pkg.native.OK and len(out[w][0]) == 6
        with pkg.native.Problem(win, device=0, intrinsics_free=(w in (1, 3))) as gp:
            srecs, _ = gp.optimize(params)
            sposes, spoints = gp.variables()
        assert [r.merit for r in out[w][0]] == [r.merit for r in srecs]
        assert np.array_equal(variables[w][0], sposes) and np.array_equal(variables[w][1], spoints)


def test_autotuner_settles_on_the_fastest_schedule(pkg):
    """With no schedule forced, the first call for a shape times one LM
    iteration per candidate; the next call runs the fastest of them."""
    wins = _windows(pkg, 12)
    params = fixed_iter_params(pkg, 6, wins[0].initial_lm_damping)
    assert "SGBA_BATCH_SCHEDULE" not in os.environ
    _, first, _ = _run_batch(pkg, wins, params)
    _, second, _ = _run_batch(pkg, wins, params)
    assert second["tuned"] and all(m > 0.0 for m in second["schedule_ms"])
    assert second["schedule"] == int(np.argmin(second["schedule_ms"]))
    assert first["batched_windows"] == second["batched_windows"] == 12


def test_concurrent_creation_equals_sequential(pkg):
    """Windows created concurrently on host threads (create_problems) optimise
    exactly as windows created one by one."""
    wins = _windows(pkg, 8)
    params = fixed_iter_params(pkg, 4, wins[0].initial_lm_damping)
    seq = [pkg.native.Problem(w, device=0) for w in wins]
    con = pkg.native.create_problems(wins, device=0, threads=4)
    try:
        a = pkg.native.batch_optimize(seq, params)
        b = pkg.native.batch_optimize(con, params)
        for w in range(len(wins)):
            assert [r.merit for r in a[w][0]] == [r.merit for r in b[w][0]]
            assert np.array_equal(seq[w].variables()[0], con[w].variables()[0])
    finally:
        for p in seq + con:
            p.close()
