#!/usr/bin/env python
"""Benchmark of the implicit bond-based PD step on GB300.

Metric: implicit steps/s at ~1M particles (CG relative residual 1e-6).
Workload: ~1M particles filling an ellipsoid (semi-axes 0.5 x 0.35 x 0.3 m,
jittered lattice, horizon 5r, stretch limit 0.015) struck by a rigid sphere
(r = 0.1 m, 10 m/s, penalty contact, in contact from the first step),
Newmark-beta dt = 5e-5 s, FP32 force/SpMV with FP64-grade CG dot products.
One step = one Simulator::advance() (force/breakage pass, device-resident CG
to rel. 1e-6, update, adaptive-dt rollbacks included).  The CG starts from the
history-projection guess (warm_start 2: the previous solution plus its Galerkin
correction in the span of the last 8 solutions; the tolerance is unchanged);
the same steps started from the previous solution alone, as the reference
starts them, are timed in the same run and reported as config.plain_guess
(--warm-start 0 makes that the measured configuration).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl gb300 (default): the CUDA library through its C ABI.  `value` is
device-timed (CUDA events on the library's stream, inputs resident in HBM),
`e2e` is wall time through the public API from host arrays (upload, GPU bond
build, and per step advance + position download), `roofline` is the SpMV
kernel's algorithmic bytes per launch over its event-timed mean duration.

--impl reference: the CPU oracle port of the reference step (the reference
itself needs CUSP and sm_20 and does not build here) on the host cores, on
the same full-size scene, W warm-up steps then K timed steps, no scaling.
The scene is built by lattice.py loaded by path, so this arm never maps the
GPU library.  The GPU arm's cpu_baseline times the first steps of the same
full-size scene with the same oracle.

Multi-GPU (torchrun): independent replicas, one per GPU ("replicas only"):
value = total steps of all ranks / max rank time.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG_NAME = "sci-solver_peridynamic_gb300"
METRIC = "implicit steps/s at 1M particles (CG rel. residual 1e-6)"
TARGET_N = 1_000_000
CPU_SAMPLE_STEPS = 2    # the GPU arm's cpu_baseline: the first steps of the same full-size scene
WORKLOAD_FMT = ("ellipsoid_impact: %d particles, semi-axes 0.5/0.35/0.3 m, spacing %.5f m, horizon 5r, "
                "s0 0.015, rigid sphere r=0.1 m at 10 m/s (penalty contact), Newmark-beta dt=5e-5 s, CG rel 1e-6")


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--n", type=int, default=TARGET_N, help="target particle count")
    ap.add_argument("--lanes", type=int, default=0, help="lanes per particle row (0 = automatic)")
    ap.add_argument("--unroll", type=int, default=0, help="SpMV gather unroll 1/2/4 (0 = automatic)")
    ap.add_argument("--spmv-path", type=int, default=0,
                    help="1 shared-memory tiles, 2 per-bond gathers, 3 lattice stencil, 0 automatic")
    ap.add_argument("--workload", choices=("ellipsoid", "batched", "learned", "beam"), default="ellipsoid",
                    help="ellipsoid: the 1M-particle headline; batched: 64 scenes in one batch; learned: "
                         "learned vs plain CG warm start on the 16^3 cube; beam: FP32 vs FP64 notched beam")
    ap.add_argument("--check-every", type=int, default=10, help="beam: steps between FP32/FP64 comparisons")
    ap.add_argument("--warm-start", type=int, default=2, choices=(0, 2),
                    help="ellipsoid: CG initial guess, 0 previous solution (the reference's), 2 history projection "
                         "(default; the same steps with guess 0 are timed too and reported as plain_guess)")
    ap.add_argument("--history", type=int, default=0, help="warm start 2: solutions kept (0 = 8)")
    ap.add_argument("--cg-loop", type=int, default=0, choices=(0, 1),
                    help="CG loop: 0 = CUDA graph with a device-side while node, 1 = host-checked batches")
    ap.add_argument("--precond", type=int, default=0, choices=(0, 1, 2),
                    help="CG preconditioner: 0 none (the reference's), 1 diagonal, 2 3x3 diagonal blocks")
    ap.add_argument("--no-plain", action="store_true", help="skip the previous-solution-guess comparison run")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-guess study on the 16^3 cube")
    return ap.parse_args(argv)


# ---- distributed plumbing (replicas only) -----------------------------------------
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_init(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def reduce_max(dist, value: float) -> float:
    """Max of a float over all ranks (gloo, CPU tensor)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, value: float) -> float:
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---- clocks ------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.2)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel: str = "k_spmv"):
    """DRAM bytes per launch of a kernel from profiles/ncu_traffic.txt
    (lines "kernel bytes_per_launch particles bonds"), scaled to this run by
    the caller; None when absent."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        with open(path) as fh:
            for line in fh:
                parts = line.split()
                if len(parts) >= 4 and parts[0] == kernel:
                    return float(parts[1]), float(parts[2]), float(parts[3])
    except OSError:
        pass
    return None


# ---- the CPU oracle on the same workload ---------------------------------------------------
def lattice_module():
    """sci-solver_peridynamic_gb300/lattice.py loaded by path: it builds the
    scene arrays with numpy alone, so the CPU legs never import the package
    (which would map the GPU library)."""
    import importlib.util
    path = os.path.join(ROOT, PKG_NAME, "lattice.py")
    spec = importlib.util.spec_from_file_location("pd_lattice_standalone", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def cpu_oracle_run(n_target, warmup, steps):
    """The oracle port of the reference step (FP64, OpenMP over particles) on
    the full workload: the same ellipsoid scene at n_target particles, bonds
    built, `warmup` untimed steps, then `steps` timed one by one.  Returns a
    dict: steps_per_s, particles, spacing, timed_s, cg_iterations_per_step,
    setup_s (scene, bonds and warm-up)."""
    from oracle import oracle as O
    O.build_oracle()
    body = lattice_module().ellipsoid_impact(target_n=n_target, gap=0.0)
    t0 = time.perf_counter()
    o = O.OracleSim(O.params_from_body(body))
    o.set_particles(body["pos"], body["vel"], body["act"])
    o.make_ready()
    o.advance(warmup)
    t_setup = time.perf_counter() - t0
    iters = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        o.advance(1)
        iters += o.cg_iters
    dt = time.perf_counter() - t0
    return {"steps_per_s": steps / dt, "particles": int(body["pos"].shape[0]), "spacing": body["spacing"],
            "timed_s": dt, "cg_iterations_per_step": iters / max(steps, 1), "setup_s": t_setup}


def spmv_variant(opt, args):
    """The product in use, as pd_get_options reports it."""
    how = "fixed" if args.spmv_path else "autotuned"
    if opt.spmv_path == 3:
        return "lattice stencil (brick halos in shared memory, 1/d0 table per stencil entry) (%s)" % how
    return "%s, %d lanes x %d unroll (%s)" % ("shared-memory tiles" if opt.spmv_path == 1 else "per-bond gathers",
                                             opt.lanes_per_particle, opt.spmv_unroll, how)


# ---- GPU arm -------------------------------------------------------------------------------
def run_gb300(args):
    world, rank, local = dist_env()
    dist = dist_init(world)
    import torch
    pkg = importlib.import_module(PKG_NAME)
    scenes = importlib.import_module(PKG_NAME + ".scenes")
    torch.cuda.set_device(local)
    sc = scenes.ellipsoid_impact(target_n=args.n, gap=0.0)
    if args.lanes:
        sc.opt.lanes_per_particle = args.lanes
    if args.unroll:
        sc.opt.spmv_unroll = args.unroll
    sc.opt.spmv_path = args.spmv_path
    sc.opt.warm_start = args.warm_start
    sc.opt.history_size = args.history
    sc.opt.cg_loop = args.cg_loop
    sc.opt.preconditioner = args.precond
    sim = scenes.make_simulator(sc, device=local)
    sim.makeReady()
    sim.advance(args.warmup)
    sim.synchronize()
    stream = torch.cuda.ExternalStream(sim.stream_handle(), device=torch.device("cuda", local))
    sim.set_profiling(True)
    sim.reset_kernel_times()
    st0 = sim.stats()
    launches0 = sim.launch_count()
    sampler = ClockSampler(local)
    sampler.start()
    barrier(dist)
    sim.synchronize()
    torch.cuda.synchronize(local)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    sim.advance(args.steps)
    ev1.record(stream)
    sim.synchronize()
    torch.cuda.synchronize(local)
    barrier(dist)
    clocks = sampler.stop()
    ms = ev0.elapsed_time(ev1)
    ms_max = reduce_max(dist, ms)
    st1 = sim.stats()
    launches = sim.launch_count() - launches0
    kt = sim.kernel_times()
    iters = st1.total_cg_iterations - st0.total_cg_iterations
    n = sc.n
    bonds = 0.5 * (st0.bonds_alive + st1.bonds_alive)
    # SpMV: 4 B column index per live bond + p, X, u and A p (16 B each) per particle
    spmv_launches, spmv_ms = kt["spmv"]
    spmv_bytes = 4.0 * bonds + 64.0 * n
    spmv_s = (spmv_ms / 1e3) / max(spmv_launches, 1)
    achieved = spmv_bytes / spmv_s / 1e9 if spmv_launches else None
    peak, peak_kind = measured_peak_hbm()
    traffic = None
    kernel_name = "k_spmv_lattice" if sim.params()[2].spmv_path == 3 else "k_spmv"
    tr = ncu_traffic(kernel_name)
    if tr is not None:
        bytes_ref, n_ref, b_ref = tr
        traffic = bytes_ref * (4.0 * bonds + 64.0 * n) / (4.0 * b_ref + 64.0 * n_ref)
    total_steps = reduce_sum(dist, float(args.steps))
    value = total_steps / (ms_max / 1e3)
    shares = {k: round(v[1] / max(ms, 1e-9), 4) for k, v in kt.items()}
    result = {
        "metric": METRIC,
        "value": round(value, 4),
        "unit": "steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_max / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 force/SpMV, f64 stretch test + master state, double-float->f64 dots",
        "data": "synthetic (seeded jittered lattice ellipsoid)",
        "config": {
            "workload": WORKLOAD_FMT % (n, sc.info["spacing"]),
            "particles": n,
            "bonds_alive": int(bonds),
            "cg_iterations_per_step": round(iters / args.steps, 2),
            "cg_initial_guess": ("previous solution (the reference's)" if args.warm_start == 0 else
                                 "history projection: previous solution + Galerkin correction in the span of "
                                 "the last %d solutions" % (sim.params()[2].history_size or 8)),
            "spmv_variant": spmv_variant(sim.params()[2], args),
            "cg_loop": ("CUDA graph per solve: a while node repeats %d iterations until the device-side test "
                        "stops it" % (sc.opt.cg_check_interval or 4) if args.cg_loop == 0 else
                        "host-launched batches, a read-back of the test after each"),
            "cg_graph_solves": int(st1.cg_graph_solves - st0.cg_graph_solves),
            "cg_preconditioner": ("none (the reference's plain CG)", "inverse diagonal",
                                  "inverse 3x3 diagonal blocks")[args.precond],
            "host_syncs_per_step": round((st1.host_syncs - st0.host_syncs) / args.steps, 2),
            "parallelism": "replicas x%d" % world,
            "l2": ("inputs larger than L2 (1/d0 stencil table %.0f MB + particle state > 129 MB L2)" % (320 * n / 1e6)
                   if sim.params()[2].spmv_path == 3 else
                   "inputs larger than L2 (bond columns + 1/d0 %.0f MB + particle state > 129 MB L2)" % (8 * bonds / 1e6)),
        },
        "gpu_launches": int(launches),
        "kernel_time_share": shares,
        "roofline": {
            "kernel": "%s (matrix-free A*p)" % kernel_name,
            "bound": "hbm",
            "achieved": round(achieved, 1) if achieved else None,
            "peak": peak,
            "peak_kind": peak_kind,
            "unit": "GB/s",
            "frac": round(achieved / peak, 4) if achieved else None,
            "traffic": round(traffic) if traffic else None,
            "algorithmic_bytes_per_launch": int(spmv_bytes),
            "mean_launch_us": round(spmv_s * 1e6, 2),
            "launches": int(spmv_launches),
        },
        "clocks": clocks,
    }
    # the same steps with the reference's initial guess (the previous solution)
    if args.warm_start and not args.no_plain:
        sc0 = scenes.ellipsoid_impact(target_n=args.n, gap=0.0)
        for f in ("lanes_per_particle", "spmv_unroll", "spmv_path", "cg_loop", "cg_check_interval", "preconditioner"):
            setattr(sc0.opt, f, getattr(sc.opt, f))
        sc0.opt.warm_start = 0
        sim0 = scenes.make_simulator(sc0, device=local)
        sim0.makeReady()
        sim0.advance(args.warmup)
        sim0.synchronize()
        stream0 = torch.cuda.ExternalStream(sim0.stream_handle(), device=torch.device("cuda", local))
        p0 = sim0.stats().total_cg_iterations
        barrier(dist)
        torch.cuda.synchronize(local)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream0)
        sim0.advance(args.steps)
        e1.record(stream0)
        sim0.synchronize()
        torch.cuda.synchronize(local)
        ms0 = reduce_max(dist, e0.elapsed_time(e1))
        it0 = sim0.stats().total_cg_iterations - p0
        result["config"]["plain_guess"] = {
            "value": round(total_steps / (ms0 / 1e3), 4), "unit": "steps/s",
            "cg_iterations_per_step": round(it0 / args.steps, 2),
            "note": "same workload and steps, CG started from the previous solution as the reference does"}
        result["config"]["cg_iterations_vs_plain"] = round(iters / max(it0, 1), 4)
        sim0.close()
    # end to end through the public API, from host arrays
    if not args.no_e2e:
        import numpy as np
        sim2 = pkg.Simulator(local, sc.sim, sc.run, sc.opt)
        sim2.get_pd_position()[:] = sc.pos
        sim2.get_pd_velocity()[:] = sc.vel
        sim2.get_pd_activity()[:] = sc.act
        # the step's result goes straight into a pinned host buffer
        host_pos = torch.empty((n, 4), dtype=torch.float64, pin_memory=True).numpy()
        barrier(dist)
        t0 = time.perf_counter()
        sim2.makeReady()
        for _ in range(args.warmup + args.steps):
            sim2.advance(1)
            sim2.get(pkg.VAR_POSITION, out=host_pos)
        sim2.synchronize()
        t_e2e = reduce_max(dist, time.perf_counter() - t0)
        nsteps = args.warmup + args.steps
        h2d = (sc.pos.nbytes + sc.vel.nbytes + sc.act.nbytes) / nsteps
        result["e2e"] = {"value": round(reduce_sum(dist, float(nsteps)) / t_e2e, 4), "unit": "steps/s",
                         "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(32 * n),
                         "includes": "pd_set_particles + pd_make_ready (GPU bond build) once, then per step "
                                     "pd_advance(1) + pd_get(POSITION) to host; wall clock"}
        sim2.close()
    # the metric's second half: CG iterations per step with the learned guess
    # against the plain one (16^3 cube, held-out seed)
    if rank == 0 and world == 1 and not args.no_learned:
        r = learned_study(local, 3)
        result["learned_vs_plain"] = r
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count()
        os.environ.setdefault("OMP_NUM_THREADS", str(cores))
        k = min(args.steps, CPU_SAMPLE_STEPS)
        c = cpu_oracle_run(args.n, 0, k)
        result["cpu_baseline"] = {
            "value": round(c["steps_per_s"], 6), "unit": "steps/s", "cores": cores, "kind": "port",
            "sample": "oracle (FP64 restatement of the reference step, OpenMP over particles) on the same "
                      "%d-particle scene, steps 1..%d timed (%.1f s, %.1f CG iterations per step); no scaling"
                      % (c["particles"], k, c["timed_s"], c["cg_iterations_per_step"]),
        }
    sim.close()
    if rank == 0:
        print(json.dumps(result), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_reference(args):
    """The reference's step on the host cores: the oracle port (the reference
    itself needs CUSP and sm_20 and its kernels cannot be built on the GPU
    box), on the full workload, W warm-up steps then K timed steps, with all
    host threads.  Rank 0 only; the package is never imported here."""
    world, rank, local = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    c = cpu_oracle_run(args.n, args.warmup, args.steps)
    v, n_s = c["steps_per_s"], c["particles"]
    sample = ("oracle port of the reference step (FP64, OpenMP over particles on %d threads; the reference itself "
              "needs CUSP and sm_20) on the full %d-particle scene: %d warm-up steps, then steps %d..%d timed "
              "(%.1f s, %.1f CG iterations per step, CG started from the previous solution as the reference does); "
              "set-up and warm-up %.1f s" % (cores, n_s, args.warmup, args.warmup + 1, args.warmup + args.steps,
                                            c["timed_s"], c["cg_iterations_per_step"], c["setup_s"]))
    result = {
        "metric": METRIC, "value": round(v, 6), "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 / v, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered lattice ellipsoid)",
        "config": {"workload": WORKLOAD_FMT % (n_s, c["spacing"]), "particles": n_s,
                   "cg_iterations_per_step": round(c["cg_iterations_per_step"], 2)},
        "impl": "reference",
        "cpu_baseline": {"value": round(v, 6), "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": round(v, 6), "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(result), flush=True)


# ---- other workloads (one JSON line each; not the headline metric) ----------------------
def _timed(stream_handle, fn, local):
    import torch
    stream = torch.cuda.ExternalStream(stream_handle, device=torch.device("cuda", local))
    torch.cuda.synchronize(local)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    fn()
    ev1.record(stream)
    torch.cuda.synchronize(local)
    return ev0.elapsed_time(ev1)


def _batch_arm(pkg, scenes, lst, local, args, warm_start, params=None):
    """One timed run of the batch: returns (ms, stats dict, config, clocks)."""
    o = pkg.BatchOptions()
    pkg.library().pd_batch_options_default(o)
    o.warm_start = warm_start
    b = pkg.Batch(local, o)
    for sc in lst:
        scenes.add_to_batch(b, sc)
    b.makeReady()
    if params is not None:
        b.ws_set_params(params)
    cfg = b.config()
    b.advance(args.warmup)
    k_all = range(len(lst))
    it0 = sum(b.stats(k).total_cg_iterations for k in k_all)
    kept0 = sum(b.stats(k).ws_guesses_kept for k in k_all)
    skipped0 = sum(b.stats(k).ws_guesses_skipped for k in k_all)
    l0 = b.launch_count()
    sampler = ClockSampler(local)
    sampler.start()
    ms = _timed(b.stream_handle(), lambda: b.advance(args.steps), local)
    clocks = sampler.stop()
    st = {
        "launches": b.launch_count() - l0,
        "iters": sum(b.stats(k).total_cg_iterations for k in k_all) - it0,
        "kept": sum(b.stats(k).ws_guesses_kept for k in k_all) - kept0,
        "skipped": sum(b.stats(k).ws_guesses_skipped for k in k_all) - skipped0,
        "bonds": sum(b.stats(k).bonds_alive for k in k_all),
        "max_iters": max(b.stats(k).last_cg_iterations for k in k_all),
        "converged": all(b.stats(k).cg_converged for k in k_all),
        "positions": [b.get(k, pkg.VAR_POSITION) for k in k_all],
        "alive": [sum(len(r) for r in b.alive_sets(k)) for k in k_all],
    }
    b.close()
    return ms, st, cfg, clocks


def run_batched(args):
    """64 independent scenes (log-uniform 4096..65536 particles, horizons
    4/5/6, impacts 1-10 m/s) stepped together by the batch API with the
    learned warm start on (a network trained on the GPU from plain-solver
    data of four other scenes of the same family), beside the plain batch and
    the same scenes stepped one pd_handle at a time."""
    import numpy as np
    import torch
    pkg = importlib.import_module(PKG_NAME)
    scenes = importlib.import_module(PKG_NAME + ".scenes")
    ws = importlib.import_module(PKG_NAME + ".warmstart")
    local = 0
    torch.cuda.set_device(local)
    lst = scenes.batched_scenes(count=64, seed=0)
    n_total = sum(sc.n for sc in lst)
    # training data from four scenes of another draw (plain solver), 40 steps each
    t0 = time.perf_counter()
    train_lst = scenes.batched_scenes(count=4, seed=1)
    X, T = ws.collect(lambda k: train_lst[k], seeds=range(len(train_lst)), steps=40, samples_per_step=256)
    params, loss = ws.train(X, T, iterations=2000)
    t_train = time.perf_counter() - t0
    ms_p, st_p, cfg_p, _ = _batch_arm(pkg, scenes, lst, local, args, 0)
    ms, st, cfg, clocks = _batch_arm(pkg, scenes, lst, local, args, 1, params)
    pos_diff = max(float(np.abs(a[:, :3] - b[:, :3]).max() / max(np.abs(b[:, :3]).max(), 1e-300))
                   for a, b in zip(st["positions"], st_p["positions"]))
    # the same scenes, one handle each, stepped in turn (plain warm start)
    sims = []
    for sc in lst:
        s = scenes.make_simulator(sc, local)
        s.makeReady()
        s.advance(args.warmup)
        s.synchronize()
        sims.append(s)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for s in sims:
            s.advance(1)
    for s in sims:
        s.synchronize()
    t_seq = time.perf_counter() - t0
    for s in sims:
        s.close()
    bonds = st["bonds"]
    spmv_bytes = 4.0 * bonds + 64.0 * n_total
    achieved = spmv_bytes / (cfg.tuned_spmv_ms / 1e3) / 1e9 if cfg.tuned_spmv_ms > 0 else None
    peak, peak_kind = measured_peak_hbm()
    value = args.steps / (ms / 1e3)
    result = {
        "metric": "batched implicit steps/s (64 scenes, every scene advances one step), learned warm start on",
        "value": round(value, 4), "unit": "steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 force/SpMV, f64 stretch test + master state, double-float->f64 dots, bf16 MLP (f32 accum)",
        "data": "synthetic (seeded jittered blocks and balls)",
        "config": {"workload": "64 impact bodies, %d particles in total (log-uniform 4096..65536 each), horizons "
                               "4/5/6 r, impacts 1-10 m/s, blocks implicit Euler dt=1e-4, balls Newmark dt=5e-5, "
                               "CG rel 1e-6, learned warm start" % n_total,
                   "particles": n_total, "bonds_alive": int(bonds), "scenes": len(lst),
                   "cg_iterations_per_step_all_scenes": round(st["iters"] / args.steps, 1),
                   "cg_iterations_last_step_max": int(st["max_iters"]),
                   "learned_guesses_kept": "%d of %d scene-steps" % (st["kept"], args.steps * len(lst)),
                   "learned_pass_paused": ("%d of %d scene-steps (3 rejected guesses in a row pause a scene's "
                                           "learned pass; retried every 16 steps)" % (st["skipped"],
                                                                                      args.steps * len(lst))),
                   "network": "trained on the GPU from %d plain-solver pairs of 4 other scenes in %.1f s "
                              "(loss %.4g)" % (X.shape[0], t_train, loss),
                   "launch_shape": {"lanes": cfg.lanes_per_particle, "unroll": cfg.spmv_unroll,
                                    "item_rows": cfg.item_rows, "work_items": cfg.work_items,
                                    "grid_pre": cfg.grid_pre, "grid_cg": cfg.grid_cg,
                                    "autotuned": bool(cfg.autotuned)},
                   "l2": "inputs larger than L2 (bond columns + 1/d0 %.0f MB)" % (8 * bonds / 1e6)},
        "gpu_launches": int(st["launches"]),
        "scene_steps_per_s": round(value * len(lst), 2),
        "particle_steps_per_s": round(value * n_total, 1),
        "plain_warm_start": {"value": round(args.steps / (ms_p / 1e3), 4), "unit": "steps/s",
                             "cg_iterations_per_step_all_scenes": round(st_p["iters"] / args.steps, 1),
                             "what": "the same batch with the previous solution as the CG guess (the reference's)"},
        "learned_vs_plain": {"cg_iteration_ratio": round(st_p["iters"] / max(st["iters"], 1), 4),
                             "speed_ratio": round(ms_p / ms, 4),
                             "alive_bonds_identical": st["alive"] == st_p["alive"],
                             "max_position_difference_rel": pos_diff,
                             "all_cg_converged": bool(st["converged"] and st_p["converged"])},
        "unbatched": {"value": round(args.steps / t_seq, 4), "unit": "steps/s",
                      "what": "the same 64 scenes as 64 pd_handles (plain warm start), pd_advance(1) each in turn, "
                              "wall clock"},
        "roofline": {"kernel": "SpMV phase of k_batch_cg over all scenes (autotuner timing)", "bound": "hbm",
                     "achieved": round(achieved, 1) if achieved else None, "peak": peak, "peak_kind": peak_kind,
                     "unit": "GB/s", "frac": round(achieved / peak, 4) if achieved else None, "traffic": None,
                     "algorithmic_bytes_per_launch": int(spmv_bytes)},
        "clocks": clocks,
    }
    print(json.dumps(result), flush=True)


LEARNED_GUESSES = {0: "previous solution (the reference's)", 1: "learned correction (network alone, guarded)",
                   2: "history projection", 3: "history projection + learned column"}


def learned_study(local=0, warmup=3, steps_total=100):
    """Learned vs plain CG initial guesses on the 16^3 cube: 5 training seeds x
    100 steps x 100 sampled particles = 50k pairs from the plain solver, BF16
    network trained on the GPU, then the held-out seed-0 scene stepped with
    each initial guess (0 previous solution, 1 network alone with its guard,
    2 history projection, 3 history projection with the network's correction
    as one more column).  Returns a dict (no JSON printing)."""
    import numpy as np
    pkg = importlib.import_module(PKG_NAME)
    scenes = importlib.import_module(PKG_NAME + ".scenes")
    ws = importlib.import_module(PKG_NAME + ".warmstart")
    t0 = time.perf_counter()
    X, T = ws.collect(lambda s: scenes.cube_lattice(seed=s), seeds=[1, 2, 3, 4, 5], steps=100, samples_per_step=100)
    t_collect = time.perf_counter() - t0
    t0 = time.perf_counter()
    params, loss = ws.train(X, T, iterations=3000)
    t_train = time.perf_counter() - t0
    out = {}
    steps = steps_total - warmup
    for mode in (0, 1, 2, 3):
        sc = scenes.cube_lattice(seed=0)
        sc.opt.warm_start = mode
        sim = scenes.make_simulator(sc, local)
        sim.makeReady()
        if mode in (1, 3):
            sim.ws_set_params(params)
        sim.advance(warmup)
        st0 = sim.stats()
        ms = _timed(sim.stream_handle(), lambda: sim.advance(steps), local)
        st1 = sim.stats()
        out[mode] = {
            "guess": LEARNED_GUESSES[mode],
            "steps_per_s": round(steps / (ms / 1e3), 3),
            "cg_iterations_per_step": round((st1.total_cg_iterations - st0.total_cg_iterations) / steps, 2),
            "guesses_kept": int(st1.ws_guesses_kept - st0.ws_guesses_kept),
            "learned_column_used": int(st1.ws_learned_used - st0.ws_learned_used),
            "position": sim.get(pkg.VAR_POSITION), "alive": sim.alive_sets(),
        }
        sim.close()
    pl = out[0]
    res = {"workload": "cube_lattice 16^3 = 4096 particles, implicit Euler dt=1e-4, CG rel 1e-6, steps %d..%d of "
                       "held-out seed 0" % (warmup + 1, steps_total),
           "training_pairs": int(X.shape[0]), "train_iterations": 3000, "final_loss": float(loss),
           "collect_s": round(t_collect, 2), "train_s": round(t_train, 2), "guesses": {}}
    for mode, r in out.items():
        same = all(np.array_equal(a, c) for a, c in zip(pl["alive"], r["alive"]))
        dpos = float(np.abs(pl["position"] - r["position"])[:, :3].max() / np.abs(pl["position"][:, :3]).max())
        res["guesses"][str(mode)] = {k: r[k] for k in ("guess", "steps_per_s", "cg_iterations_per_step",
                                                        "guesses_kept", "learned_column_used")}
        res["guesses"][str(mode)].update({
            "cg_iterations_vs_plain": round(pl["cg_iterations_per_step"] / max(r["cg_iterations_per_step"], 1e-9), 4),
            "steps_per_s_vs_plain": round(r["steps_per_s"] / pl["steps_per_s"], 4),
            "same_broken_bond_set_as_plain": bool(same), "max_position_difference_rel": dpos})
    best = max(res["guesses"].values(), key=lambda g: g["cg_iterations_vs_plain"])
    res["target_1p5x_steps_per_s_met"] = bool(max(g["steps_per_s_vs_plain"] for g in res["guesses"].values()) >= 1.5)
    res["best_cg_iterations_vs_plain"] = best["cg_iterations_vs_plain"]
    return res


def run_learned(args):
    """The learned-guess study as its own JSON line (bench.py --workload learned)."""
    import torch
    torch.cuda.set_device(0)
    r = learned_study(0, args.warmup)
    g = r["guesses"]
    result = {
        "metric": "CG iterations per step, learned vs plain warm start (rel. residual 1e-6)",
        "value": g["3"]["cg_iterations_vs_plain"], "unit": "plain/learned iterations ratio (history projection + "
        "learned column)", "higher_is_better": True, "n_gpus": 1, "steps": 100 - args.warmup, "warmup": args.warmup,
        "dtype": "bf16 MLP (f32 accumulate), f32/f64 CG",
        "data": "synthetic (16^3 jittered cube, training seeds 1-5, evaluation seed 0)",
        "config": {k: v for k, v in r.items() if k != "guesses"}, "guesses": g,
    }
    print(json.dumps(result), flush=True)


def _bond_set_difference(sim_a, sim_b):
    """Bonds alive in exactly one of two runs of the same scene (each bond
    counted once).  Rows are compared by count and an order-free hash of
    their live neighbours; only rows that differ are compared exactly."""
    import numpy as np
    ra, la, ca = sim_a.bond_rows()
    rb, lb, cb = sim_b.bond_rows()

    def row_hash(rp, bl, cnt):
        v = bl.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)
        v ^= v >> np.uint64(29)
        cs = np.zeros(v.size + 1, np.uint64)
        np.cumsum(v, dtype=np.uint64, out=cs[1:])
        start = rp[:-1].astype(np.int64)
        return cs[start + cnt] - cs[start]

    ha, hb = row_hash(ra, la, ca), row_hash(rb, lb, cb)
    rows = np.nonzero((ca != cb) | (ha != hb))[0]
    diff = 0
    for i in rows:
        a = la[ra[i]:ra[i] + ca[i]]
        b = lb[rb[i]:rb[i] + cb[i]]
        diff += len(np.setxor1d(a, b))
    return diff // 2


def run_beam(args):
    """Precision study: the notched beam (2M particles, horizon 6r, three-point
    bending) stepped in mixed precision and in FP64 side by side; every
    --check-every steps the positions and the broken-bond sets are compared."""
    import numpy as np
    import torch
    pkg = importlib.import_module(PKG_NAME)
    scenes = importlib.import_module(PKG_NAME + ".scenes")
    local = 0
    torch.cuda.set_device(local)
    sims = {}
    for prec in (pkg.PRECISION_MIXED, pkg.PRECISION_FP64):
        sc = scenes.notched_beam(target_n=args.n if args.n != TARGET_N else 2_000_000, precision=prec)
        s = scenes.make_simulator(sc, local)
        s.makeReady()
        sims[prec] = s
    n = sc.n
    mixed, fp64 = sims[pkg.PRECISION_MIXED], sims[pkg.PRECISION_FP64]
    b0 = fp64.stats().bonds_initial
    rows = []
    t_mixed = t_fp64 = 0.0
    done = 0
    while done < args.steps:
        k = min(args.check_every, args.steps - done)
        t_mixed += _timed(mixed.stream_handle(), lambda: mixed.advance(k), local)
        t_fp64 += _timed(fp64.stream_handle(), lambda: fp64.advance(k), local)
        done += k
        xm, xd = mixed.get(pkg.VAR_POSITION), fp64.get(pkg.VAR_POSITION)
        um = xm - sc.pos
        ud = xd - sc.pos
        err_x = float(np.abs(xm - xd)[:, :3].max() / np.abs(xd[:, :3]).max())
        err_u = float(np.abs(um - ud)[:, :3].max() / max(np.abs(ud[:, :3]).max(), 1e-300))
        diff = _bond_set_difference(mixed, fp64)
        rows.append({"step": done, "pos_rel_err": err_x, "disp_rel_err": err_u, "bond_set_diff": int(diff),
                     "bonds_broken_fp64": int(b0 - fp64.stats().bonds_alive),
                     "cg_iters_mixed": int(mixed.stats().last_cg_iterations),
                     "cg_iters_fp64": int(fp64.stats().last_cg_iterations),
                     "ticks_mixed": int(mixed.stats().time_step_ticks),
                     "ticks_fp64": int(fp64.stats().time_step_ticks)})
    result = {
        "metric": "FP32 vs FP64 step on the notched beam: max position error per check, bond-set differences",
        "value": max(r["pos_rel_err"] for r in rows), "unit": "max relative position difference",
        "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "warmup": 0, "dtype": "f32 vs f64",
        "data": "synthetic (seeded jittered notched beam)",
        "config": {"workload": "notched_beam %d particles, 1.0x0.2x0.2 m, notch 0.05 m, horizon 6r, s0 0.01, "
                               "load strip at 1 m/s, Newmark dt=5e-5, CG rel 1e-6" % n,
                   "check_every": args.check_every, "bonds_initial": int(b0)},
        "mixed_steps_per_s": round(args.steps / (t_mixed / 1e3), 4),
        "fp64_steps_per_s": round(args.steps / (t_fp64 / 1e3), 4),
        "checks": rows,
    }
    for s in sims.values():
        s.close()
    print(json.dumps(result), flush=True)


def main(argv=None):
    args = parse_args(argv)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "learned":
        run_learned(args)
    elif args.workload == "beam":
        run_beam(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
