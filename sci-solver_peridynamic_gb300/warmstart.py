"""Training pipeline of the learned CG warm start (no reference counterpart).

The plain solver generates the data: each step of a run with collection on
records, for a sample of free particles, the 64 features computed before
the CG and the normalised change of the solution the CG produced.  The
network is trained on the GPU by the library's own BF16 tensor-core forward
and backward kernels (pd_mlp_train), then loaded into a simulator with
warm_start = 1, where the CG still runs to the same tolerance.
"""
from __future__ import annotations

import numpy as np

from . import PRECISION_MIXED, mlp_init, mlp_train
from .scenes import make_simulator


def collect(scene_factory, seeds, steps, samples_per_step, device=0):
    """Runs the plain solver on scene_factory(seed) for each seed; returns (X, T)."""
    xs, ts = [], []
    for seed in seeds:
        sc = scene_factory(seed)
        sc.opt.precision = PRECISION_MIXED
        sc.opt.warm_start = 0
        sim = make_simulator(sc, device)
        sim.makeReady()
        sim.ws_collect(samples_per_step, samples_per_step * steps)
        sim.advance(steps)
        X, T = sim.ws_dataset(samples_per_step * steps)
        xs.append(X)
        ts.append(T)
        sim.close()
    return np.concatenate(xs), np.concatenate(ts)


def train(X, T, iterations=3000, batch=1024, lr=1e-3, seed=1, device=0):
    p0 = mlp_init(seed)
    return mlp_train(X, T, p0, iterations=iterations, batch=batch, lr=lr, seed=seed, device=device)


def compare(scene, params, steps, device=0):
    """CG iterations per step and positions of the plain and the learned warm start."""
    out = {}
    for mode in (0, 1):
        scene.opt.warm_start = mode
        sim = make_simulator(scene, device)
        sim.makeReady()
        if mode == 1:
            sim.ws_set_params(params)
        iters = []
        for _ in range(steps):
            sim.advance(1)
            iters.append(sim.stats().last_cg_iterations)
        from . import VAR_POSITION
        out["learned" if mode else "plain"] = {
            "iters": np.array(iters), "position": sim.get(VAR_POSITION),
            "kept": sim.stats().ws_guesses_kept, "converged": sim.CGConvergence(),
        }
        sim.close()
    scene.opt.warm_start = 0
    return out
