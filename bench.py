#!/usr/bin/env python
"""Benchmark of the implicit bond-based PD step on GB300.

Metric: implicit steps/s at ~1M particles (CG relative residual 1e-6).
Workload: ~1M particles filling an ellipsoid (semi-axes 0.5 x 0.35 x 0.3 m,
jittered lattice, horizon 5r, stretch limit 0.015) struck by a rigid sphere
(r = 0.1 m, 10 m/s, penalty contact, in contact from the first step),
Newmark-beta dt = 5e-5 s, FP32 force/SpMV with FP64-grade CG dot products.
One step = one Simulator::advance() (force/breakage pass, device-resident CG
to rel. 1e-6, update, adaptive-dt rollbacks included).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl gb300 (default): the CUDA library through its C ABI.  `value` is
device-timed (CUDA events on the library's stream, inputs resident in HBM),
`e2e` is wall time through the public API from host arrays (upload, GPU bond
build, and per step advance + position download), `roofline` is the SpMV
kernel's algorithmic bytes per launch over its event-timed mean duration.

--impl reference: the CPU oracle port of the reference step (the reference
itself needs CUSP and sm_20 and does not build here) on the host cores, on a
bounded sample: the same scene built at 1/8 of the particle count, steps/s
scaled by the particle ratio.

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
SAMPLE_DIV = 8          # CPU sample: same scene at 1/8 of the particles
TARGET_N = 1_000_000


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--n", type=int, default=TARGET_N, help="target particle count")
    ap.add_argument("--lanes", type=int, default=0, help="lanes per particle row (0 = automatic)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
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


# ---- the CPU sample ------------------------------------------------------------------
def cpu_sample_scene(pkg_scenes, n_full):
    return pkg_scenes.ellipsoid_impact(target_n=max(1000, n_full // SAMPLE_DIV), gap=0.0)


def oracle_for(scene):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import make_oracle
    return make_oracle(scene)


def cpu_steps_per_s(pkg_scenes, n_full, warmup, steps):
    """Oracle (FP64 reference restatement) on the 1/8 sample: W untimed steps,
    then `steps` timed; steps/s scaled to the full particle count."""
    from oracle import oracle as O
    O.build_oracle()
    sc = cpu_sample_scene(pkg_scenes, n_full)
    o = oracle_for(sc)
    o.advance(warmup)
    t0 = time.perf_counter()
    o.advance(steps)
    dt = time.perf_counter() - t0
    scale = sc.n / float(n_full)
    return steps / dt * scale, sc.n, dt


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
    tr = ncu_traffic("k_spmv")
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
            "workload": "ellipsoid_impact: %d particles, semi-axes 0.5/0.35/0.3 m, spacing %.5f m, horizon 5r, "
                        "s0 0.015, rigid sphere r=0.1 m at 10 m/s (penalty contact), Newmark-beta dt=5e-5 s, "
                        "CG rel 1e-6" % (n, sc.info["spacing"]),
            "particles": n,
            "bonds_alive": int(bonds),
            "cg_iterations_per_step": round(iters / args.steps, 2),
            "spmv_variant": "%d lanes x %d unroll (autotuned)" % (sim.params()[2].lanes_per_particle,
                                                                   sim.params()[2].spmv_unroll),
            "parallelism": "replicas x%d" % world,
            "l2": "inputs larger than L2 (bond list %.0f MB + particle state > 129 MB L2)" % (4 * bonds / 1e6),
        },
        "gpu_launches": int(launches),
        "kernel_time_share": shares,
        "roofline": {
            "kernel": "k_spmv (matrix-free A*p)",
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
    # end to end through the public API, from host arrays
    if not args.no_e2e:
        import numpy as np
        sim2 = pkg.Simulator(local, sc.sim, sc.run, sc.opt)
        sim2.get_pd_position()[:] = sc.pos
        sim2.get_pd_velocity()[:] = sc.vel
        sim2.get_pd_activity()[:] = sc.act
        host_pos = np.zeros((n, 4))
        barrier(dist)
        t0 = time.perf_counter()
        sim2.makeReady()
        for _ in range(args.warmup + args.steps):
            sim2.advance(1)
            host_pos[:] = sim2.get(pkg.VAR_POSITION)
        sim2.synchronize()
        t_e2e = reduce_max(dist, time.perf_counter() - t0)
        nsteps = args.warmup + args.steps
        h2d = (sc.pos.nbytes + sc.vel.nbytes + sc.act.nbytes) / nsteps
        result["e2e"] = {"value": round(reduce_sum(dist, float(nsteps)) / t_e2e, 4), "unit": "steps/s",
                         "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(32 * n),
                         "includes": "pd_set_particles + pd_make_ready (GPU bond build) once, then per step "
                                     "pd_advance(1) + pd_get(POSITION) to host; wall clock"}
        sim2.close()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count()
        os.environ.setdefault("OMP_NUM_THREADS", str(cores))
        k = min(args.steps, 3)
        v, n_s, dt = cpu_steps_per_s(scenes, n, args.warmup, k)
        result["cpu_baseline"] = {
            "value": round(v, 6), "unit": "steps/s", "cores": cores, "kind": "port",
            "sample": "oracle (FP64 restatement of the reference step, OpenMP over particles) on the same scene "
                      "built with %d particles (1/%d), steps %d..%d timed (%.1f s), steps/s scaled by %d/%d"
                      % (n_s, SAMPLE_DIV, args.warmup + 1, args.warmup + k, dt, n_s, n),
        }
    sim.close()
    if rank == 0:
        print(json.dumps(result), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_reference(args):
    world, rank, local = dist_env()
    if rank != 0:
        return
    scenes = importlib.import_module(PKG_NAME + ".scenes")
    cores = os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    v, n_s, dt = cpu_steps_per_s(scenes, args.n, args.warmup, args.steps)
    sample = ("oracle port of the reference step (FP64, OpenMP over particles; the reference itself needs CUSP "
              "and sm_20) on the same scene built with %d particles (1/%d), %d timed steps after %d warm-up "
              "(%.1f s), steps/s scaled by %d/%d" % (n_s, SAMPLE_DIV, args.steps, args.warmup, dt, n_s, args.n))
    result = {
        "metric": METRIC, "value": round(v, 6), "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 / v, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered lattice ellipsoid)",
        "config": {"workload": "ellipsoid_impact at %d particles (sampled at %d)" % (args.n, n_s)},
        "impl": "reference",
        "cpu_baseline": {"value": round(v, 6), "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": round(v, 6), "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(result), flush=True)


def main(argv=None):
    args = parse_args(argv)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
