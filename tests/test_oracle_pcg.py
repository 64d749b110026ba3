"""The oracle's preconditioned CG (the preconditioner option's checker, no
GPU).  The reference runs plain CG (its cusp::precond::diagonal is commented
out, src/core/simulator.cu:767-769); preconditioning must not change what a
solve converges to, only the path: with a tight tolerance the preconditioned
runs keep the plain run's broken-bond sets and time steps and agree on the
positions to the tolerance."""
import importlib

import numpy as np
import pytest

from helpers import make_oracle, rel_err, same_sets


@pytest.fixture(scope="module")
def scenes():
    return importlib.import_module("sci-solver_peridynamic_gb300.scenes")


def _run(scenes, precond, steps=50):
    pdgb = importlib.import_module("sci-solver_peridynamic_gb300")
    sc = scenes.reference_block(n_side=6, seed=5, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=150.0,
                                cg_tol=1e-12)
    sc.opt.preconditioner = precond
    o = make_oracle(sc)
    its = 0
    for _ in range(steps):
        o.advance(1)
        its += o.lib.pdo_last_cg_iters(o.h)
    return o, its


def test_preconditioned_oracle_keeps_the_plain_solution(scenes):
    plain, it0 = _run(scenes, 0)
    its = {}
    for mode in (1, 2):
        o, its[mode] = _run(scenes, mode)
        assert same_sets(o.alive_sets(), plain.alive_sets()), f"mode {mode}"
        assert o.dt_ticks == plain.dt_ticks
        assert rel_err(o.position, plain.position) < 1e-9, f"mode {mode}"
    # 50 steps: 1218 plain, 1159 diagonal, 1131 block iterations
    assert its[2] < it0
    assert int(np.sum(plain.bond_top + 1)) < len(plain.bond_list), "the block breaks bonds"
