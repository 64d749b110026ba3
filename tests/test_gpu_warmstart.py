"""The learned CG warm start: the GPU MLP's forward and backward (BF16
tensor cores, FP32 accumulation) against the CPU restatement, GPU training,
and the warm start in the solver -- the CG still reaches the same tolerance,
so positions agree with the plain solve and with the oracle; the iteration
counts of both are reported."""
import numpy as np
import pytest

from helpers import make_oracle, rel_err
from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu

GRAD_TOL = 3e-2   # relative L2 error: BF16 storage of activations and output gradients


def _batch(rows, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((rows, 64)).astype(np.float32)
    T = (0.3 * X[:, :3] - 0.2 * X[:, 9:12] + 0.1 * np.tanh(X[:, 12:15])).astype(np.float32)
    return X, T


def test_mlp_forward_and_gradient_match_oracle(pdgb):
    p = pdgb.mlp_init(3)
    p[-3:] = [0.05, -0.02, 0.01]
    X, T = _batch(257, 1)
    Y = pdgb.mlp_predict(X, p)
    Yo, _ = M.forward(X, p)
    assert np.linalg.norm(Y - Yo) / np.linalg.norm(Yo) < 2e-2
    loss, g = pdgb.mlp_loss_grad(X, T, p)
    lo, go = M.loss_grad(X, T, p)
    assert abs(loss - lo) / lo < 2e-2
    for name, a, b in (("W1", 0, 64 * 128), ("b1", 64 * 128, 64 * 128 + 128),
                       ("W2", 64 * 128 + 128, 64 * 128 + 128 + 128 * 128),
                       ("W3", g.size - 387, g.size - 3), ("b3", g.size - 3, g.size)):
        err = np.linalg.norm(g[a:b] - go[a:b]) / max(np.linalg.norm(go[a:b]), 1e-30)
        assert err < GRAD_TOL, (name, err)


@pytest.mark.parametrize("rows", [1, 127, 128, 129, 5000, 100003])
def test_mlp_tensor_core_inference_matches_oracle(pdgb, rows):
    """pd_mlp_predict runs the tcgen05 kernel (all three layers, TMEM
    accumulators, 128-row tiles, up to two CTAs per SM looping over tiles):
    partial tiles, one tile, and many tiles per CTA against the CPU
    restatement with BF16 rounding at the same points."""
    p = pdgb.mlp_init(7)
    p[-3:] = [0.05, -0.02, 0.01]
    X, _ = _batch(rows, 11)
    Y = pdgb.mlp_predict(X, p)
    Yo, _ = M.forward(X, p)
    assert Y.shape == (rows, 3) and np.isfinite(Y).all()
    assert np.linalg.norm(Y - Yo) / np.linalg.norm(Yo) < 2e-2
    worst = np.abs(Y - Yo).max(axis=1) / (np.abs(Yo).max() + 1e-30)
    assert worst.max() < 5e-2


def test_mlp_training_reduces_loss(pdgb):
    X, T = _batch(8192, 2)
    p0 = pdgb.mlp_init(5)
    l0, _ = pdgb.mlp_loss_grad(X[:4096], T[:4096], p0)
    p1, l1 = pdgb.mlp_train(X, T, p0, iterations=800, batch=512, lr=2e-3, seed=5)
    assert l1 < 0.1 * l0


def test_learned_warm_start_keeps_the_solution(pdgb, scenes):
    ws = __import__("importlib").import_module("sci-solver_peridynamic_gb300.warmstart")
    factory = lambda seed: scenes.cube_lattice(n_side=12, seed=seed)   # noqa: E731
    X, T = ws.collect(factory, seeds=(1, 2), steps=40, samples_per_step=512)
    assert X.shape[0] == 2 * 40 * 512 and np.isfinite(X).all() and np.isfinite(T).all()
    params, loss = ws.train(X, T, iterations=1500, batch=1024, lr=1e-3)
    assert np.isfinite(loss)
    sc = factory(3)
    out = ws.compare(sc, params, steps=40)
    plain, learned = out["plain"], out["learned"]
    assert plain["converged"] and learned["converged"]
    assert rel_err(learned["position"], plain["position"]) < 1e-5
    ora = make_oracle(sc)
    ora.advance(40)
    assert rel_err(learned["position"], ora.position) < 1e-5
    print(f"\ncg iterations over 40 steps: plain {plain['iters'].sum()}, learned {learned['iters'].sum()}, "
          f"learned guesses kept {learned['kept']}/40, training loss {loss:.4g}")


def test_trained_network_gains_over_the_method_without_it(pdgb, scenes):
    """The network trained on the plain solver's (state, solved increment)
    pairs of five seeds, on the held-out seed 0 of the 16^3 cube: the guess
    with the network takes fewer CG iterations than the same method without it
    -- the network alone (warm_start 1) against the previous solution
    (warm_start 0), and the history projection with the network's column
    (warm_start 3) against the projection alone (warm_start 2, within 1 %:
    a Galerkin solve over a larger space lowers the starting A-norm error but
    not always the iteration count).  Measured on a GB300: 84.5 / 81.4 / 79.4 /
    79.1 iterations per step for 0 / 1 / 2 / 3."""
    ws = __import__("importlib").import_module("sci-solver_peridynamic_gb300.warmstart")
    X, T = ws.collect(lambda s: scenes.cube_lattice(seed=s), seeds=[1, 2, 3, 4, 5], steps=100, samples_per_step=100)
    params, loss = ws.train(X, T, iterations=3000)
    iters, pos = {}, {}
    for mode in (0, 1, 2, 3):
        sc = scenes.cube_lattice(seed=0)
        sc.opt.warm_start = mode
        sim = scenes.make_simulator(sc)
        sim.makeReady()
        if mode in (1, 3):
            sim.ws_set_params(params)
        sim.advance(100)
        st = sim.stats()
        assert sim.CGConvergence()
        iters[mode] = st.total_cg_iterations
        pos[mode] = sim.get(pdgb.VAR_POSITION)
        if mode == 3:
            assert st.ws_learned_used > 50   # the projection gave the network's column a weight
    print(f"\ncg iterations over 100 steps: {iters} (training loss {loss:.4g})")
    assert iters[1] < iters[0]
    assert iters[3] < iters[0] and iters[3] <= 1.01 * iters[2]
    for mode in (1, 2, 3):
        assert rel_err(pos[mode], pos[0]) < 1e-5
