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
