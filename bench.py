#!/usr/bin/env python3
"""Benchmark of the GB300 Schur-LM bundle-adjustment path.

Workload (the configuration the headline metric is quoted on): 100 SE(3)
cameras on a radius-6 m Fibonacci sphere looking at the origin, 20,000 points
uniform in [-2, 2]^3, each seen by 10..40 of the cameras that see it
(~499k observations), pinhole fx=fy=500, Huber 1 px, camera 0 fixed,
initial damping 1e-4.  Synthetic, seeded (seed 20261204).

A "step" is one LM iteration over the whole problem (linearize, Schur
complement, factor + solve, back-substitute, update, trial cost, decision).
`value` is LM iterations/s with the problem resident in HBM (device time from
CUDA events, L2 flushed before every step).  `e2e` is the same metric through
the C ABI (sgba_optimize, the optimize_nlls drop-in) starting from host
buffers: every step uploads the problem, runs the 20-iteration optimization
and reads the variables back.

--impl reference times the CPU restatement of the reference algorithm on the
host cores on the same workload.
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
SEED = 20261203 + 1
N_ITER_WORKLOAD = 20
WORKLOAD = ("sphere BA: 100 SE(3) cams (99 free) on a r=6 m Fibonacci sphere, 20000 points in [-2,2]^3, "
            "each seen by U{10..40} of its visible cams (~499k obs), pinhole 500/500/320/240, Huber 1 px, "
            "nu0=1e-4, Schur LM with dense FP32-factor + f64-refined reduced camera system")
# Other workloads (parity-test configurations, measured with --workload):
#   loop    1500 cameras on a r=50 m loop, 300,000 points on a r=60 m cylinder, consecutive-camera
#           tracks of Geom(0.12) clipped to [3, 25] (~2.5M obs), 15 LM iterations; banded solver and
#           float-float linearization
#   windows 1024 independent local windows (cameras U{5..40}, points U{200..4000}), 10 LM iterations
#           each, optimised concurrently by sgba_batch_optimize
WORKLOADS = {
    "sphere": dict(kind="SPHERE", n_cam=0, n_pt=0, seed=SEED, n_iter=N_ITER_WORKLOAD, desc=WORKLOAD),
    "loop": dict(kind="LOOP", n_cam=1500, n_pt=300000, seed=20261203 + 2, n_iter=15,
                 desc=("loop BA: 1500 SE(3) cams on a r=50 m loop facing outward, 300000 points on a r=60 m "
                       "cylinder, consecutive-camera tracks Geom(0.12) clipped to [3,25] (~2.5M obs), Huber 1 px, "
                       "nu0=1e-4; banded float-float LDL^T of the reduced camera system, float-float linearization")),
}
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
    """Algorithmic (compulsory) HBM bytes per launch of each kernel."""
    n_obs = prob.n_obs
    n_pt = prob.n_pt
    n_cam = prob.n_cam
    nf = lay.n_free_poses
    nz = lay.n_h_blocks - nf - lay.n_marg_points  # terms with a free pose and a marginalized point
    if name == "schur":
        # read Z (18 f32) of every term once, U and the damping counts of each pose,
        # write every lower S block once in f64
        return 72 * nz + (288 + 8) * nf + 288 * lay.n_s_blocks
    if name == "landmark":
        # per observation: residual (8) + pose index (4) + term bounds (8); per term: Z (72);
        # per point: position (24) + C^-1 (48) + C^-1 b (24) + neg gradient (24)
        return 20 * n_obs + 72 * nz + 120 * n_pt + 48 * n_cam
    if name == "cost":
        # per observation: uv f64 (16) + indices (8) + residual out (8); points (24); poses (96)
        return 32 * n_obs + 24 * n_pt + 96 * n_cam
    if name == "camera":
        # per term: residual (8) + point (24) + Z (72) + C^-1 b (24); per tile partial out
        return (8 + 24) * n_obs + (72 + 24) * nz + 33 * 8 * ((lay.n_terms + 255) // 256)
    if name == "backsub":
        return 72 * nz + (48 + 24 + 24) * lay.n_marg_points + 48 * nf
    if name == "factor":
        n6 = 6 * nf
        if getattr(lay, "solver", 0) == 1:
            # banded solver: the band of S read once in f64 (row r: columns r-W+1..r) and the border rows;
            # the float-float band written (scaled S), read and written back once by the factor, read by the
            # two sweeps; border rows and the rhs (nbd + 1 rows of the band width) in and out in float-float
            nb = n6 - lay.border_rows
            w = lay.band_width
            return 8 * nb * w + 8 * lay.border_rows * n6 + 8 * nb * w * 5 + 16 * (lay.border_rows + 1) * nb * 2
        # single-launch cluster solver: read S once as float-float (8 B per entry) and the
        # reduced rhs (f64); write the step as f64 and as float-float pairs
        return 8 * n6 * n6 + 8 * n6 + 16 * n6
    return None


def run_gpu(args, ws, rank, local):
    import numpy as np

    import __graft_entry__ as graft

    if not os.path.exists(os.path.join(graft.PKG_DIR, "libsgba.so")):
        graft.build_native()
    pkg = graft.load_package()
    native = pkg.native
    wl = WORKLOADS[args.workload]
    prob = pkg.synth.generate(getattr(pkg.synth, wl["kind"]), n_cam=wl["n_cam"], n_pt=wl["n_pt"],
                              seed=wl["seed"] + rank)
    K, W = args.steps, args.warmup
    params = pkg.OptParams(num_iterations=W + K + 1000, initial_lm_damping=prob.initial_lm_damping,
                           function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0,
                           max_consecutive_rejects=1 << 40, solver=pkg.LinearSolverEnum.SchurBlockSparseLdlt)
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
        gp.optimize(pkg.OptParams(num_iterations=n_prof, initial_lm_damping=prob.initial_lm_damping,
                                  function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0,
                                  max_consecutive_rejects=1 << 40, solver=pkg.LinearSolverEnum.SchurBlockSparseLdlt))
        pr = gp.profile()
        out["phase_ms"] = {"linearize": pr.ms_linearize / n_prof, "schur": pr.ms_schur / n_prof,
                           "factor_solve": pr.ms_factor / n_prof, "update": pr.ms_update / n_prof,
                           "cost_decide": pr.ms_cost / n_prof}
        out["lay"] = lay
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
    e2e_params = pkg.OptParams(num_iterations=wl["n_iter"], initial_lm_damping=prob.initial_lm_damping,
                               function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0,
                               max_consecutive_rejects=1 << 40, solver=pkg.LinearSolverEnum.SchurBlockSparseLdlt)
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

    import __graft_entry__ as graft

    if not os.path.exists(os.path.join(graft.PKG_DIR, "libsgba.so")):
        graft.build_native()
    pkg = graft.load_package()
    native = pkg.native
    base = pkg.synth.BASE_SEED + 3 + rank * N_WINDOWS
    wins = [pkg.synth.generate(pkg.synth.WINDOW, seed=base + w) for w in range(N_WINDOWS)]
    params = pkg.OptParams(num_iterations=WINDOW_ITERS, initial_lm_damping=wins[0].initial_lm_damping,
                           function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0,
                           max_consecutive_rejects=1 << 40, solver=pkg.LinearSolverEnum.SchurBlockSparseLdlt)
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
        dt = _barrier_and_max(time.perf_counter() - t0, ws)
        clk = clocks.stop()
    finally:
        for p in probs:
            p.close()
    # end to end: create (upload) + batch + read back, from host arrays
    t0 = time.perf_counter()
    for _ in range(max(1, min(3, K))):
        ps = [native.Problem(w, device=local) for w in wins]
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
    return dict(value=N_WINDOWS * K * ws / dt, dt=dt, launches=launches, p50=float(np.percentile(ms, 50)),
                p99=float(np.percentile(ms, 99)), clk=clk, e2e=N_WINDOWS * e2e_steps * ws / e2e_s, h2d=h2d, d2h=d2h,
                n_obs=int(sum(w.n_obs for w in wins)), wins=wins, params=params, pkg=pkg)


def cpu_baseline(prob, pkg, n_iter, threads):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bindings as ob  # the oracle: CPU restatement of the reference

    import __graft_entry__ as graft

    graft.build_oracle()
    params = pkg.OptParams(num_iterations=n_iter, initial_lm_damping=prob.initial_lm_damping,
                           function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0,
                           max_consecutive_rejects=1 << 40)
    t0 = time.perf_counter()
    recs, _, _ = ob.optimize(prob, params, n_threads=threads)
    dt = time.perf_counter() - t0
    cpu_baseline.last_merits = [r.merit for r in recs]
    return len(recs) / dt, dt


def cpu_windows(wins, pkg, threads):
    """The oracle on a sample of windows, windows spread over the host threads."""
    import concurrent.futures

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bindings as ob  # the oracle: CPU restatement of the reference

    import __graft_entry__ as graft

    graft.build_oracle()
    params = pkg.OptParams(num_iterations=WINDOW_ITERS, initial_lm_damping=wins[0].initial_lm_damping,
                           function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0,
                           max_consecutive_rejects=1 << 40)
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda w: ob.optimize(w, params, n_threads=1), wins))
    dt = time.perf_counter() - t0
    return len(wins) / dt, dt


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
    ap.add_argument("--workload", default="sphere", choices=["sphere", "loop", "windows"],
                    help="sphere: the headline configuration; loop / windows: the 1500-camera loop and the "
                         "batched local windows")
    ap.add_argument("--profile-iters", type=int, default=0,
                    help="profiling mode: only set up the workload and run this many LM iterations")
    args = ap.parse_args()
    if args.profile_iters > 0:
        import __graft_entry__ as graft

        pkg = graft.load_package()
        wl = WORKLOADS["loop" if args.workload == "loop" else "sphere"]
        prob = pkg.synth.generate(getattr(pkg.synth, wl["kind"]), n_cam=wl["n_cam"], n_pt=wl["n_pt"], seed=wl["seed"])
        params = pkg.OptParams(num_iterations=args.profile_iters, initial_lm_damping=prob.initial_lm_damping,
                               function_tolerance=0.0, gradient_tolerance=0.0, parameter_tolerance=0.0,
                               max_consecutive_rejects=1 << 40, solver=pkg.LinearSolverEnum.SchurBlockSparseLdlt)
        with pkg.native.Problem(prob, device=0) as gp:
            recs, _ = gp.optimize(params)
        print(json.dumps({"profile_iters": len(recs), "final_merit": recs[-1].merit}))
        return
    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist

        backend = "gloo" if args.impl == "reference" else "nccl"
        dist.init_process_group(backend=backend)

    import __graft_entry__ as graft

    if args.impl == "reference":
        if rank != 0:
            return
        if not os.path.exists(os.path.join(graft.PKG_DIR, "libsgba.so")):
            graft.build_native()
        pkg = graft.load_package()
        if args.workload == "windows":
            wins = [pkg.synth.generate(pkg.synth.WINDOW, seed=pkg.synth.BASE_SEED + 3 + w) for w in range(16)]
            threads = os.cpu_count() or 1
            v, dt = cpu_windows(wins, pkg, threads)
            line = {"metric": METRIC, "value": v, "unit": "windows/s", "impl": "reference", "n_gpus": args.gpus,
                    "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / len(wins),
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                    "data": "synthetic", "config": {"workload": "windows", "n_windows": len(wins)},
                    "cpu_baseline": {"value": v, "unit": "windows/s", "cores": threads, "kind": "port",
                                     "sample": "%d windows, %d LM iterations each, one per thread at a time"
                                               % (len(wins), WINDOW_ITERS)},
                    "e2e": {"value": v, "unit": "windows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
            print(json.dumps(line))
            return
        wl = WORKLOADS[args.workload]
        prob = pkg.synth.generate(getattr(pkg.synth, wl["kind"]), n_cam=wl["n_cam"], n_pt=wl["n_pt"], seed=wl["seed"])
        threads = os.cpu_count() or 1
        cpu_baseline(prob, pkg, max(1, args.warmup // 5), threads)  # warm caches / page in
        v, dt = cpu_baseline(prob, pkg, args.steps, threads)
        line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic",
                "config": {"workload": wl["desc"], "n_obs": int(prob.n_obs)},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": "%d LM iterations of the workload on %d threads (setup included)"
                                           % (args.steps, threads)},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
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
            "config": {"workload": "%d local windows (cams U{5..40}, points U{200..4000}), %d LM iterations each, "
                                   "one sgba_batch_optimize per step" % (N_WINDOWS, WINDOW_ITERS),
                       "n_obs_total": out["n_obs"], "l2": "inputs larger than L2 (all windows resident)"},
            "window_ms": {"p50": out["p50"], "p99": out["p99"]},
            "gpu_launches": int(out["launches"]),
            "roofline": None,
            "e2e": {"value": out["e2e"], "unit": "windows/s", "h2d_bytes_per_step": int(out["h2d"]),
                    "d2h_bytes_per_step": int(out["d2h"]),
                    "step": "create+upload all windows, batch optimize, read back"},
            "clocks": out["clk"],
        }
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            v, dt = cpu_windows(out["wins"][:64], out["pkg"], threads)
            line["cpu_baseline"] = {"value": v, "unit": "windows/s", "cores": threads, "kind": "port",
                                    "sample": "64 windows, %d LM iterations each, one per thread at a time (%.1f s)"
                                              % (WINDOW_ITERS, dt)}
        print(json.dumps(line))
        return

    out = run_gpu(args, ws, rank, local)
    if rank != 0:
        return
    pkg = graft.load_package()
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
            roofline["note"] = ("latency-bound dependency chain: banded float-float LDL^T in one 16-CTA cluster "
                                "(%d panel steps of 24 pivots), forward/backward sweeps of the same length"
                                % ((n6 - lay.border_rows + 23) // 24))
        else:
            roofline["note"] = ("latency-bound dependency chain (one cluster of 16 CTAs: %d panel steps, then a "
                                "forward and a backward sweep per solve, one solve plus one or two refinement "
                                "solves); FP32 work %.0f MFLOP per launch" % ((n6 + 23) // 24, n6 ** 3 / 3e6))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak" if ws > 1 else "weak",
        "vs_baseline": None,
        "dtype": ("float-float (Jacobians, products, sums, LDL^T) + f64 update" if lay.float_float_lin
                  else "fp32 (Jacobians/products) + float-float sums + f64 update"),
        "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload]["desc"], "n_obs": int(prob.n_obs), "n_terms": int(lay.n_terms),
                   "n_schur_pairs": int(lay.n_schur_pairs), "l2": "flushed (256 MiB write) before every step",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "jacobian_obs_per_s": value * prob.n_obs,
        "kernel_ms": kt,
        "phase_ms_per_iteration": out.get("phase_ms"),
        "roofline": roofline,
        "kernel_roofline": kernel_roofline,
        "gpu_launches": int(out["launches"]),
        "e2e": {"value": WORKLOADS[args.workload]["n_iter"] * out["e2e_steps"] * ws / out["e2e_s"], "unit": UNIT,
                "h2d_bytes_per_step": int(out["h2d"]), "d2h_bytes_per_step": int(out["d2h"]),
                "step": "create+upload, optimize (%d LM iterations), read back" % WORKLOADS[args.workload]["n_iter"],
                "pinned_host": out["pinned"]},
        "clocks": out["clk"],
    }
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v0, _ = cpu_baseline(prob, pkg, 2, threads)  # rate estimate; sample ~10 s of CPU work
        n_cpu = int(min(max(2, round(10.0 * v0)), 400))
        v, dt = cpu_baseline(prob, pkg, n_cpu, threads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "%d LM iterations of the workload on %d threads (%.1f s, setup included)"
                                          % (n_cpu, threads, dt)}
        # the same optimisation from the same start: per-iteration merit of the
        # e2e run against the oracle's (FP64 restatement of the reference)
        ora = getattr(cpu_baseline, "last_merits", [])
        gpu = out.get("gpu_merits", [])
        k = min(len(ora), len(gpu))
        if k > 0:
            dev = max(abs(g - o) / abs(o) for g, o in zip(gpu[:k], ora[:k]) if o != 0.0)
            line["parity"] = {"per_iteration_cost_max_rel_dev": dev, "iterations_compared": k,
                              "final_cost_rel_gap": abs(gpu[k - 1] - ora[k - 1]) / abs(ora[k - 1]),
                              "reference": "oracle (FP64 CPU restatement of the reference)"}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
