#!/usr/bin/env python3
"""Benchmark of the GB300 Schur-LM bundle-adjustment path.

Default workload (the configuration the headline target is stated on): 1500
SE(3) cameras along a radius-50 m loop facing outward (lateral jitter
N(0, 0.2^2) m), 300,000 points on a radius-60 m cylinder wall, each seen by a
run of consecutive cameras of length Geom(0.12) clipped to [3, 25]
(~2.5M observations), pinhole fx=fy=500, Huber 1 px, camera 0 fixed, initial
damping 1e-4, 15 LM iterations.  Synthetic, seeded (seed 20261205).  The
reduced camera system is a band plus the loop-closure border, factored in
float-float by the banded solver (nested dissection: the loop's two arcs in
parallel, the separator and the closure in a dense corner).

A "step" is one LM iteration over the whole problem (linearize, Schur
complement, factor + solve, back-substitute, update, trial cost, decision).
`value` is LM iterations/s with the problem resident in HBM (device time from
CUDA events, L2 flushed before every step).  `e2e` is the same metric through
the C ABI (sgba_optimize, the optimize_nlls drop-in) starting from pinned
host buffers: every step uploads the problem, runs the 15-iteration
optimization and reads the variables back.

--workload sphere / windows measure the other benchmark configurations (the
100-camera sphere and the 1024 batched local windows) with the same contract;
--workload eucm the problem of the reference's own BA benchmark (10 cameras
around an open box, one EUCM camera whose six params are free).
--impl reference times the CPU restatement of the reference algorithm (the
oracle) on the host cores on the same workload; that arm maps only the
oracle's library (which carries its own copy of the scene generator).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "BA LM iters/sec + Jacobian obs/sec; learned-PCG vs exact LDLt at equal cost"
UNIT = "LM iters/s"
WORKLOADS = {
    "loop": dict(kind=2, n_cam=1500, n_pt=300000, seed=20261203 + 2, n_iter=15,
                 desc=("loop BA: 1500 SE(3) cams on a r=50 m loop facing outward, 300000 points on a r=60 m "
                       "cylinder, consecutive-camera tracks Geom(0.12) clipped to [3,25] (~2.5M obs), Huber 1 px, "
                       "nu0=1e-4, 15 LM iterations; banded float-float LDL^T of the reduced camera system (nested "
                       "dissection: two arcs in parallel), float-float linearization")),
    "sphere": dict(kind=1, n_cam=0, n_pt=0, seed=20261203 + 1, n_iter=20,
                   desc=("sphere BA: 100 SE(3) cams (99 free) on a r=6 m Fibonacci sphere, 20000 points in "
                         "[-2,2]^3, each seen by U{10..40} of its visible cams (~499k obs), pinhole "
                         "500/500/320/240, Huber 1 px, nu0=1e-4, 20 LM iterations; dense FP32-factor + "
                         "float-float-refined reduced camera system")),
    "eucm": dict(gen="ring_box_eucm", n_cam=10, n_pt=500, seed=20261203 + 5, n_iter=20,
                 desc=("the reference's BA benchmark problem (BaProblem::new(10, 500)): 10 SE(3) cams on a r=8 m "
                       "ring looking at an open box of 500 points (5000 obs), one EUCM camera with its 6 params "
                       "Free (300/300/320/240/0.5/1.0 true, 297/297/321/241/0.495/1.0 initial), poses 0 and 1 "
                       "fixed, uniform +-0.075 px noise, no robust kernel, nu0=1.0, 20 LM iterations; one-CTA "
                       "float-float solver, float-float linearization")),
}
DEFAULT_WORKLOAD = "loop"
N_WINDOWS = 1024
WINDOW_ITERS = 10


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _barrier_and_max(value, ws):
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "", 1).isdigit())
        mx = max(float(r[2]) for r in rows if r[2].replace(".", "", 1).isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _profile_traffic(workload):
    """DRAM bytes per launch of each kernel of a workload, from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(workload, {})
    except Exception:
        return {}


def _kernel_bytes(name, lay, prob):
    """Algorithmic (compulsory) HBM bytes per launch of each kernel.

    N_z = terms with a free pose and a marginalized point.  With the
    float-float linearization (loop-shaped problems) Z is also kept as
    float-float pairs (144 bytes used per term) and the residuals carry low
    parts (8 bytes per observation)."""
    n_obs = prob.n_obs
    n_pt = prob.n_pt
    n_cam = prob.n_cam
    nf = lay.n_free_poses
    nz = lay.n_h_blocks - nf - lay.n_marg_points
    dd = bool(getattr(lay, "float_float_lin", 0))
    zb = 144 if dd else 72  # Z read per term
    if name == "schur":
        # read Z of every term once, U and the damping counts of each pose,
        # write every lower S block once in f64
        return zb * nz + (288 + 8) * nf + 288 * lay.n_s_blocks
    if name == "landmark":
        # per observation: residual (8, + 8 low parts) + pose index (4) + term bounds (8); per term: Z out
        # (72 FP32, + 144 float-float); per point: position (24) + C^-1 (48) + C^-1 b (24) + neg gradient (24);
        # per camera: pose table (48 FP32 or 96 float-float)
        if dd:
            return 28 * n_obs + (72 + 144) * nz + 120 * n_pt + 96 * n_cam
        return 20 * n_obs + 72 * nz + 120 * n_pt + 48 * n_cam
    if name == "cost":
        # per observation: uv f64 (16) + indices (8) + residual out (8, + 8 low parts); points (24); poses (96)
        return (40 if dd else 32) * n_obs + 24 * n_pt + 96 * n_cam
    if name == "camera":
        # per observation: residual (8, + 8); per term: point (24) + Z + C^-1 b (24); per tile partial out
        return ((16 if dd else 8) * n_obs + (24 + zb + 24) * nz + 33 * 8 * ((lay.n_terms + 255) // 256))
    if name == "backsub":
        return zb * nz + (48 + 24 + 24) * lay.n_marg_points + 48 * nf
    if name == "factor":
        n6 = 6 * nf
        if getattr(lay, "solver", 0) == 1:
            # banded solver: the band of S read once in f64 (row r: columns r-W+1..r) and the border rows;
            # the float-float band written (scaled S), read and written back once by the factor, read by
            # the sweep-matrix kernel, which writes the two per-panel sweep matrices (the band's size each),
            # read once by each sweep; border rows and the rhs (nbd + 1 rows of the band width) in and out
            # in float-float; the corner (m x m) written, factored in place and read by its sweep matrices
            nb = n6 - lay.border_rows
            w = lay.band_width
            m = lay.border_rows
            return (8 * nb * w + 8 * m * n6 + 8 * nb * w * 8 + 16 * (m + 1) * nb * 2 + 8 * m * m * 4)
        # single-launch cluster solver: read S once as float-float (8 B per entry) and the
        # reduced rhs (f64); write the step as f64 and as float-float pairs
        return 8 * n6 * n6 + 8 * n6 + 16 * n6
    return None


def _make_problem(synth, wl, seed, lib_path=None):
    """The workload's scene from the package's generators (`synth` is the
    package's synth module or a copy loaded on its own)."""
    if wl.get("gen") == "ring_box_eucm":
        return synth.ring_box_eucm(n_cam=wl["n_cam"], n_pt=wl["n_pt"], seed=seed)
    return synth.generate(wl["kind"], n_cam=wl["n_cam"], n_pt=wl["n_pt"], seed=seed, lib_path=lib_path)


def _load_pkg():
    import __graft_entry__ as graft

    if not all(os.path.exists(os.path.join(graft.PKG_DIR, f)) for f in ("libsgba.so", "libsgba_synth.so")):
        graft.build_native()
        graft.build_synth()
    return graft.load_package()


def _fixed(pkg_or_ns, n_iter, nu0):
    """OptParams with every tolerance disabled: a fixed number of LM iterations."""
    return pkg_or_ns.OptParams(num_iterations=n_iter, initial_lm_damping=nu0, function_tolerance=0.0,
                               gradient_tolerance=0.0, parameter_tolerance=0.0, max_consecutive_rejects=1 << 40)


def _step_errors(gp, prob, n_steps):
    """The first LM steps against an FP64 LDL^T of the same reduced system
    (outside the gauge); None where scipy is missing."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    try:
        import scipy.sparse  # noqa: F401
        from step_error import step_errors
    except Exception:
        return None
    return step_errors(gp, prob, n_steps)


def _learned_pcg(pkg, prob, device, K, W, n_iter):
    native = pkg.native
    if not os.path.exists(native.TRAINED_WEIGHTS):
        return {"unavailable": "no trained weights (%s)" % os.path.relpath(native.TRAINED_WEIGHTS, ROOT)}
    with native.PcgModel.load(device=device) as model:
        with native.Problem(prob, device=device) as gp:
            gp.set_linear_solver(native.LINSOLVE_PCG_LEARNED, 50, 1e-8, model)
            gp.init(_fixed(pkg, W + K + 1000, prob.initial_lm_damping))
            gp.bench_iterations(W, flush_l2=True)
            ms, _ = gp.bench_iterations(K, flush_l2=True)
            st = gp.pcg_stats()
        with native.Problem(prob, device=device) as gp:
            gp.set_linear_solver(native.LINSOLVE_PCG_LEARNED, 50, 1e-8, model)
            recs, _ = gp.optimize(_fixed(pkg, n_iter, prob.initial_lm_damping))
            st2 = gp.pcg_stats()
    return {"value": K / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms / K,
            "pcg_solves": int(st.solves), "pcg_fallbacks": int(st.fallbacks),
            "fallback_rate": st.fallbacks / max(1, st.solves),
            "mean_pcg_iterations": st.iterations / max(1, st.solves),
            "final_cost": recs[-1].merit, "solve_fallback_rate": st2.fallbacks / max(1, st2.solves),
            "config": "PCG (learned block preconditioner, 3-layer message passing, hidden 64, BF16 weights), "
                      "cap 50 iterations, tolerance 1e-8 relative residual, exact factorization as fallback"}


def run_gpu(args, ws, rank, local):
    import numpy as np

    pkg = _load_pkg()
    native = pkg.native
    wl = WORKLOADS[args.workload]
    prob = _make_problem(pkg.synth, wl, wl["seed"] + rank)
    K, W = args.steps, args.warmup
    params = _fixed(pkg, W + K + 1000, prob.initial_lm_damping)
    device = local
    out = {}
    with native.Problem(prob, device=device) as gp:
        lay = gp.layout()
        gp.init(params)
        gp.bench_iterations(W, flush_l2=True)
        _barrier(ws)
        clocks = ClockSampler(device)
        clocks.start()
        ms, launches = gp.bench_iterations(K, flush_l2=True)
        clk = clocks.stop()
        ms_max = _barrier_and_max(ms, ws)
        # per-kernel live timing (same stream, CUDA events, L2 flushed)
        kernels = {"schur": native.KERNEL_SCHUR, "landmark": native.KERNEL_LANDMARK,
                   "camera": native.KERNEL_CAMERA, "cost": native.KERNEL_COST,
                   "factor": native.KERNEL_FACTOR, "backsub": native.KERNEL_BACKSUB}
        kt = {k: gp.bench_kernel(v, reps=max(5, K), flush_l2=True) for k, v in kernels.items()}
        # phase breakdown of a few iterations (events between phases; not the headline number)
        gp.set_profiling(True)
        n_prof = 5
        gp.optimize(_fixed(pkg, n_prof, prob.initial_lm_damping))
        pr = gp.profile()
        out["phase_ms"] = {"linearize": pr.ms_linearize / n_prof, "schur": pr.ms_schur / n_prof,
                           "factor_solve": pr.ms_factor / n_prof, "update": pr.ms_update / n_prof,
                           "cost_decide": pr.ms_cost / n_prof}
        out["lay"] = lay
    # the learned-PCG solver of the reduced system (PCG with the trained block
    # preconditioner, 50 iterations to 1e-8, the exact factorization as its
    # fallback) on the same workload: device-resident rate and the final cost
    # of the same optimisation, against the plain path
    out["learned_pcg"] = (_learned_pcg(pkg, prob, device, K, W, wl["n_iter"])
                          if rank == 0 and not prob.intrinsics_free else None)
    # the LM step against an FP64 LDL^T of the same reduced system, first steps
    # from the workload's start (not timed)
    if rank == 0 and not args.no_cpu_baseline:
        with native.Problem(prob, device=device) as gp:
            gp.init(_fixed(pkg, 20, prob.initial_lm_damping))
            out["step_err"] = _step_errors(gp, prob, 2 if prob.n_cam > 200 else 3)
    # end-to-end through the C ABI from (pinned) host buffers
    e2e_steps = max(1, min(3, K))
    host = prob
    try:
        import torch

        def pin(a):
            t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
            return t.numpy()

        host = prob.copy()
        for f in ("poses", "points", "obs_cam", "obs_pt", "obs_uv", "pose_const"):
            setattr(host, f, pin(getattr(prob, f)))
        pinned = True
    except Exception:
        pinned = False
    e2e_params = _fixed(pkg, wl["n_iter"], prob.initial_lm_damping)
    # one untimed warm-up of the path (context, module load); its per-iteration
    # merits are compared with the oracle's below
    with native.Problem(host, device=device) as gp:
        warm_recs, _ = gp.optimize(e2e_params)
        gp.variables()
    gpu_merits = [r.merit for r in warm_recs]
    _barrier(ws)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        with native.Problem(host, device=device) as gp:
            gp.optimize(e2e_params)
            poses, points = gp.variables()
    e2e_s = _barrier_and_max(time.perf_counter() - t0, ws)
    h2d = (host.poses.nbytes + host.points.nbytes + host.obs_cam.nbytes + host.obs_pt.nbytes +
           host.obs_uv.nbytes + host.pose_const.nbytes)
    d2h = poses.nbytes + points.nbytes
    out.update(dict(ms=ms_max, launches=launches, kt=kt, clk=clk, e2e_s=e2e_s, e2e_steps=e2e_steps, h2d=h2d,
                    d2h=d2h, pinned=pinned, prob=prob, gpu_merits=gpu_merits))
    return out


def run_windows(args, ws, rank, local):
    """Config: N_WINDOWS independent windows, WINDOW_ITERS LM iterations each, one
    sgba_batch_optimize call per step (all windows concurrently)."""
    import numpy as np

    pkg = _load_pkg()
    native = pkg.native
    base = pkg.synth.BASE_SEED + 3 + rank * N_WINDOWS
    wins = [pkg.synth.generate(pkg.synth.WINDOW, seed=base + w) for w in range(N_WINDOWS)]
    params = _fixed(pkg, WINDOW_ITERS, wins[0].initial_lm_damping)
    K, W = args.steps, args.warmup
    probs = [native.Problem(w, device=local) for w in wins]
    try:
        for _ in range(W):
            native.batch_optimize(probs, params)
        _barrier(ws)
        clocks = ClockSampler(local)
        clocks.start()
        t0 = time.perf_counter()
        ms = []
        launches = 0
        for _ in range(K):
            out = native.batch_optimize(probs, params)
            for (recs, term, wms, fc, st) in out:
                if st != native.OK:
                    raise RuntimeError("window failed with status %d: %s" % (st, native.last_error()))
                ms.append(wms)
            launches += sum(int(p.profile().kernel_launches) for p in probs)
            bstats = native.batch_last_stats()
            launches += bstats["kernel_launches"]
        dt = _barrier_and_max(time.perf_counter() - t0, ws)
        clk = clocks.stop()
        # per-window solve time: each window optimised alone (one sgba_optimize,
        # device time of its LM iterations and final linearisation) on a sample
        solo = []
        for p, w in zip(probs[:64], wins[:64]):
            p.set_variables(w.poses, w.points)
            p.optimize(params)
            solo.append(p.profile().ms_total)
    finally:
        for p in probs:
            p.close()
    # end to end: create (upload) + batch + read back, from host arrays
    t0 = time.perf_counter()
    for _ in range(max(1, min(3, K))):
        ps = native.create_problems(wins, device=local)  # concurrent set-up on the host threads
        try:
            native.batch_optimize(ps, params)
            res = [p.variables() for p in ps]
        finally:
            for p in ps:
                p.close()
    e2e_steps = max(1, min(3, K))
    e2e_s = _barrier_and_max(time.perf_counter() - t0, ws)
    h2d = sum(w.poses.nbytes + w.points.nbytes + w.obs_cam.nbytes + w.obs_pt.nbytes + w.obs_uv.nbytes
              + w.pose_const.nbytes for w in wins)
    d2h = sum(a.nbytes + b.nbytes for a, b in res)
    ms = np.array(ms)
    solo = np.array(solo)
    return dict(value=N_WINDOWS * K * ws / dt, dt=dt, launches=launches, batch=bstats,
                p50=float(np.percentile(solo, 50)),
                p99=float(np.percentile(solo, 99)), batch_p50=float(np.percentile(ms, 50)),
                batch_p99=float(np.percentile(ms, 99)), clk=clk, e2e=N_WINDOWS * e2e_steps * ws / e2e_s, h2d=h2d,
                d2h=d2h, n_obs=int(sum(w.n_obs for w in wins)), wins=wins, params=params, pkg=pkg)


class _Params:
    """The OptParams fields the oracle reads (the CPU legs do not import the
    package)."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


class _OracleNS:
    OptParams = _Params


def _oracle():
    """The oracle (CPU restatement of the reference), built if needed."""
    import __graft_entry__ as graft

    graft.build_oracle()
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bindings as ob

    return ob


def _oracle_generate(kind, n_cam=0, n_pt=0, seed=0, wl=None):
    """A scene from the generator that the oracle library carries (the same
    source as libsgba_synth.so; ring_box_eucm is numpy), loaded without the
    package."""
    import importlib.util

    ob = _oracle()
    spec = importlib.util.spec_from_file_location("sgba_scene_gen", os.path.join(ROOT, "sophus-rs_gb300", "synth.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    if wl is not None:
        return _make_problem(mod, wl, seed, lib_path=ob.LIB), mod
    return mod.generate(kind, n_cam=n_cam, n_pt=n_pt, seed=seed, lib_path=ob.LIB), mod


def cpu_baseline(prob, n_iter, threads):
    ob = _oracle()
    params = _fixed(_OracleNS, n_iter, prob.initial_lm_damping)
    t0 = time.perf_counter()
    recs, _, _ = ob.optimize(prob, params, n_threads=threads)
    dt = time.perf_counter() - t0
    cpu_baseline.last_merits = [r.merit for r in recs]
    return len(recs) / dt, dt


def cpu_windows(wins, threads):
    """The oracle on a sample of windows, windows spread over the host threads."""
    import concurrent.futures

    ob = _oracle()
    params = _fixed(_OracleNS, WINDOW_ITERS, wins[0].initial_lm_damping)
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda w: ob.optimize(w, params, n_threads=1), wins))
    dt = time.perf_counter() - t0
    return len(wins) / dt, dt


def run_reference(args):
    """--impl reference: the oracle on the host cores, on this arm's workload."""
    threads = os.cpu_count() or 1
    if args.workload == "windows":
        base = 20261203 + 3
        wins = [_oracle_generate(3, seed=base + w)[0] for w in range(16)]
        v, dt = cpu_windows(wins, threads)
        line = {"metric": METRIC, "value": v, "unit": "windows/s", "impl": "reference", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / len(wins),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": _windows_config(),
                "cpu_baseline": {"value": v, "unit": "windows/s", "cores": threads, "kind": "port",
                                 "sample": "%d windows, %d LM iterations each, one per thread at a time"
                                           % (len(wins), WINDOW_ITERS)},
                "e2e": {"value": v, "unit": "windows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    wl = WORKLOADS[args.workload]
    prob, _ = _oracle_generate(None, seed=wl["seed"], wl=wl)
    cpu_baseline(prob, 1, threads)  # warm caches / page in
    v, dt = cpu_baseline(prob, args.steps, threads)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": _config(args.workload, prob),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d LM iterations of the workload on %d threads (setup included)"
                                       % (args.steps, threads)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _config(workload, prob):
    """The line's config: the same keys on both arms."""
    return {"workload": WORKLOADS[workload]["desc"], "n_cam": int(prob.n_cam), "n_pt": int(prob.n_pt),
            "n_obs": int(prob.n_obs), "lm_iterations_per_solve": WORKLOADS[workload]["n_iter"],
            "l2": "flushed (256 MiB write) before every step", "parallelism": "single GPU"}


def _windows_config():
    return {"workload": "%d local windows (cams U{5..40}, points U{200..4000}), %d LM iterations each, "
                        "one sgba_batch_optimize per step" % (N_WINDOWS, WINDOW_ITERS),
            "l2": "inputs larger than L2 (all windows resident)", "parallelism": "single GPU"}


def main():
    if "--workload" in sys.argv and "windows" in sys.argv:
        # one CUDA stream per window: let the streams map onto more hardware
        # queues than the default 8 (must be set before the CUDA context exists)
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=["loop", "sphere", "windows", "eucm"],
                    help="loop: the 1500-camera loop (the headline configuration); sphere / windows: the "
                         "100-camera sphere and the batched local windows; eucm: the reference's own BA "
                         "benchmark problem (EUCM camera, params free)")
    ap.add_argument("--profile-iters", type=int, default=0,
                    help="profiling mode: only set up the workload and run this many LM iterations")
    ap.add_argument("--profile-cams", type=int, default=0,
                    help="profiling mode: the loop workload at this many cameras (200 points per camera), a "
                         "small case for multi-pass profiler captures")
    ap.add_argument("--profile-windows", type=int, default=N_WINDOWS,
                    help="profiling mode of the windows workload: this many windows, two batched calls (the "
                         "first settles the schedule autotuner)")
    args = ap.parse_args()
    if args.profile_iters > 0 and args.workload == "windows":
        pkg = _load_pkg()
        wins = [pkg.synth.generate(pkg.synth.WINDOW, seed=pkg.synth.BASE_SEED + 3 + w)
                for w in range(args.profile_windows)]
        probs = [pkg.native.Problem(w, device=0) for w in wins]
        try:
            for _ in range(2):
                pkg.native.batch_optimize(probs, _fixed(pkg, args.profile_iters, wins[0].initial_lm_damping))
            print(json.dumps({"profile_iters": args.profile_iters, "windows": len(wins),
                              "batch": pkg.native.batch_last_stats()}))
        finally:
            for p in probs:
                p.close()
        return
    if args.profile_iters > 0:
        pkg = _load_pkg()
        wl = dict(WORKLOADS[args.workload if args.workload in WORKLOADS else DEFAULT_WORKLOAD])
        if args.profile_cams > 0 and wl.get("kind") == 2:
            wl["n_cam"], wl["n_pt"] = args.profile_cams, 200 * args.profile_cams
        prob = _make_problem(pkg.synth, wl, wl["seed"])
        with pkg.native.Problem(prob, device=0) as gp:
            recs, _ = gp.optimize(_fixed(pkg, args.profile_iters, prob.initial_lm_damping))
        print(json.dumps({"profile_iters": len(recs), "final_merit": recs[-1].merit}))
        return
    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist

        backend = "gloo" if args.impl == "reference" else "nccl"
        dist.init_process_group(backend=backend)

    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return

    if args.workload == "windows":
        out = run_windows(args, ws, rank, local)
        if rank != 0:
            return
        line = {
            "metric": METRIC, "value": out["value"], "unit": "windows/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * out["dt"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 (Jacobians/products) + float-float sums + f64 update", "data": "synthetic",
            "config": _windows_config(),
            "n_obs_total": out["n_obs"],
            "window_ms": {"solo_p50": out["p50"], "solo_p99": out["p99"], "batch_ms": out["batch"]["ms"],
                          "note": "solo: one window optimised alone (10 LM iterations + final linearisation, "
                                  "device time), 64 windows; batch_ms: device time of one batched call (all "
                                  "windows, init to final linearisation)"},
            "batch": {"batched_windows": out["batch"]["batched_windows"], "schedule": out["batch"]["schedule"],
                      "groups": out["batch"]["groups"], "order_by_work": bool(out["batch"]["order"]),
                      "autotuner_settled": out["batch"]["tuned"],
                      "schedule_ms_per_lm_iteration": out["batch"]["schedule_ms"],
                      "launches_per_call": out["batch"]["kernel_launches"],
                      "note": "every kernel of an LM iteration launched once for all windows (one CUDA graph per "
                              "iteration and window group); the autotuner times one LM iteration per candidate "
                              "schedule (groups 1/2/4 ordered by work, 1 as given) and keeps the fastest"},
            "gpu_launches": int(out["launches"]),
            "roofline": None,
            "e2e": {"value": out["e2e"], "unit": "windows/s", "h2d_bytes_per_step": int(out["h2d"]),
                    "d2h_bytes_per_step": int(out["d2h"]),
                    "step": "create+upload all windows (concurrently on the host threads), batch optimize, "
                            "read back"},
            "clocks": out["clk"],
        }
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            v, dt = cpu_windows(out["wins"][:64], threads)
            line["cpu_baseline"] = {"value": v, "unit": "windows/s", "cores": threads, "kind": "port",
                                    "sample": "64 windows, %d LM iterations each, one per thread at a time (%.1f s)"
                                              % (WINDOW_ITERS, dt)}
        print(json.dumps(line))
        return

    out = run_gpu(args, ws, rank, local)
    if rank != 0:
        return
    prob, lay, kt = out["prob"], out["lay"], out["kt"]
    K = args.steps
    value = K * ws / (out["ms"] / 1000.0)
    ms_per_step = out["ms"] / K
    dominant = max(kt, key=kt.get)
    hbm_peak, peak_src = _peaks()
    traffic = _profile_traffic(args.workload)
    rl_kernel = dominant if _kernel_bytes(dominant, lay, prob) is not None else max(
        (k for k in kt if _kernel_bytes(k, lay, prob) is not None), key=kt.get)
    alg = _kernel_bytes(rl_kernel, lay, prob)
    achieved = alg / (kt[rl_kernel] / 1000.0) / 1e9
    roofline = {"bound": "hbm", "kernel": rl_kernel, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes": alg, "ms_per_launch": kt[rl_kernel],
                "traffic": traffic.get(rl_kernel)}
    # every timed kernel against the same peak: algorithmic bytes per launch
    # over its live time, with its DRAM traffic per launch from ncu
    kernel_roofline = {}
    for k, ms in kt.items():
        b = _kernel_bytes(k, lay, prob)
        if b is not None and ms > 0:
            a = b / (ms / 1000.0) / 1e9
            kernel_roofline[k] = {"achieved_gbs": a, "frac": a / hbm_peak, "algorithmic_bytes": b,
                                  "ms_per_launch": ms, "traffic": traffic.get(k)}
    if rl_kernel == "factor":
        n6 = 6 * lay.n_free_poses
        if lay.solver == 1:
            nb = n6 - lay.border_rows
            if lay.border_rows > lay.band_width:
                roofline["note"] = ("latency-bound dependency chains: nested dissection of the loop, two arcs of "
                                    "~%d panel steps of 24 pivots factored and swept concurrently (one 16-CTA "
                                    "cluster each), then the %d-row corner as a dense band"
                                    % ((nb // 2 + 23) // 24, lay.border_rows))
            else:
                roofline["note"] = ("latency-bound dependency chain: banded float-float LDL^T in one 16-CTA "
                                    "cluster (%d panel steps of 24 pivots), forward/backward sweeps of the same "
                                    "length" % ((nb + 23) // 24))
        elif lay.solver == 3:
            roofline["note"] = ("latency-bound dependency chain: float-float LDL^T of the %d-row reduced system "
                                "in one CTA, one barrier per pivot" % (n6 + lay.intrinsics_rows))
        else:
            roofline["note"] = ("latency-bound dependency chain (one cluster of 16 CTAs: %d panel steps, then a "
                                "forward and a backward sweep per solve, one solve plus one or two refinement "
                                "solves); FP32 work %.0f MFLOP per launch" % ((n6 + 23) // 24, n6 ** 3 / 3e6))
    phase = out.get("phase_ms") or {}
    lin_ms = phase.get("linearize")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("float-float (Jacobians, products, sums, LDL^T) + f64 update" if lay.float_float_lin
                  else "fp32 (Jacobians/products) + float-float sums + f64 update"),
        "data": "synthetic",
        "config": _config(args.workload, prob),
        "layout": {"n_terms": int(lay.n_terms), "n_schur_pairs": int(lay.n_schur_pairs),
                   "n_s_blocks": int(lay.n_s_blocks), "solver": int(lay.solver), "band_width": int(lay.band_width),
                   "border_rows": int(lay.border_rows), "float_float_lin": int(lay.float_float_lin),
                   "ranks": "independent replicas" if ws > 1 else "single GPU"},
        # N_obs x iterations / linearize time (the landmark and camera passes)
        "jacobian_obs_per_s": (prob.n_obs / (lin_ms / 1000.0)) if lin_ms else None,
        "kernel_ms": kt,
        "phase_ms_per_iteration": phase,
        "roofline": roofline,
        "kernel_roofline": kernel_roofline,
        "gpu_launches": int(out["launches"]),
        "e2e": {"value": WORKLOADS[args.workload]["n_iter"] * out["e2e_steps"] * ws / out["e2e_s"], "unit": UNIT,
                "h2d_bytes_per_step": int(out["h2d"]), "d2h_bytes_per_step": int(out["d2h"]),
                "step": "create+upload, optimize (%d LM iterations), read back" % WORKLOADS[args.workload]["n_iter"],
                "pinned_host": out["pinned"]},
        "clocks": out["clk"],
    }
    lp = out.get("learned_pcg")
    if lp:
        if "value" in lp:
            gm = out.get("gpu_merits", [])
            lp["ratio_vs_plain"] = lp["value"] / value
            if gm:
                lp["final_cost_rel_gap_vs_plain"] = abs(lp["final_cost"] - gm[-1]) / abs(gm[-1])
        line["learned_pcg"] = lp
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        n_iter = WORKLOADS[args.workload]["n_iter"]
        v0, _ = cpu_baseline(prob, 1, threads)  # rate estimate
        # the whole solve when it takes at most ~40 s of CPU (it is also the
        # parity reference), else a sample of ~10 s
        n_cpu = n_iter if n_iter / v0 <= 40.0 else int(min(max(2, round(10.0 * v0)), 400))
        v, dt = cpu_baseline(prob, n_cpu, threads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "%d LM iterations of the workload on %d threads (%.1f s, setup included)"
                                          % (n_cpu, threads, dt)}
        # the same optimisation from the same start: per-iteration merit of the
        # e2e run against the oracle's (FP64 restatement of the reference)
        ora = getattr(cpu_baseline, "last_merits", [])
        gpu = out.get("gpu_merits", [])
        k = min(len(ora), len(gpu))
        if k > 0:
            devs = [abs(g - o) / abs(o) for g, o in zip(gpu[:k], ora[:k])]
            line["parity"] = {"per_iteration_cost_max_rel_dev": max(devs), "iterations_compared": k,
                              "per_iteration_cost_rel_dev": devs,
                              "final_cost_rel_gap": devs[-1],
                              "reference": "oracle (FP64 CPU restatement of the reference)"}
            if args.workload == "loop":
                line["parity"]["note"] = ("from iteration 11 this trajectory amplifies rounding: the FP64 oracle "
                                          "itself, run with 16 and with 15 threads, separates by 2e-6..6e-6 at "
                                          "iterations 13-15")
        if out.get("step_err") is not None:
            line.setdefault("parity", {})["step_error_vs_f64_ldlt"] = out["step_err"]
            line["parity"]["step_error_note"] = ("|dx_gpu - dx_f64| / |dx_f64| outside the scale gauge, first "
                                                 "LM steps, dx_f64 from an FP64 sparse LU of the same reduced "
                                                 "system")
    print(json.dumps(line))


if __name__ == "__main__":
    main()
