"""The matrix-free system operator (pd_apply_operator) against the oracle's
assembled matrix A = M + beta h^2 K applied by computeAx's restatement
(src/core/cg_solver.cuh:343-383)."""
import numpy as np
import pytest

from helpers import make_oracle

pytestmark = pytest.mark.gpu


def apply_on_device(pdgb, sim, x_caller, entry=None):
    """y = A x through the C ABI; x, y in caller order.  Returns (y, <x, A x>)."""
    import torch
    v = sim.operator_view()
    n = v.n
    dt = torch.float32 if v.precision == pdgb.PRECISION_MIXED else torch.float64
    perm = sim.get(pdgb.VAR_SLOT_PERMUTATION)
    x_slot = torch.zeros((n, 4), dtype=dt, device="cuda")
    x_slot[:, :3] = torch.as_tensor(x_caller[perm, :3], dtype=dt, device="cuda")
    y_slot = torch.full_like(x_slot, float("nan"))
    dot = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    if entry is None:
        sim.apply_operator(x_slot.data_ptr(), y_slot.data_ptr(), dot.data_ptr())
    else:
        entry(v, x_slot.data_ptr(), y_slot.data_ptr(), dot.data_ptr())
    sim.synchronize()
    torch.cuda.synchronize()
    y = np.zeros((n, 4))
    y[perm] = y_slot.double().cpu().numpy()
    xs = np.zeros((n, 4))
    xs[perm] = x_slot.double().cpu().numpy()
    return y, float(dot.item()), xs


def _scene(pdgb, scenes, precision):
    sc = scenes.reference_block(n_side=8, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=300.0, cg_tol=1e-10)
    sc.opt.precision = precision
    return sc


@pytest.mark.parametrize("precision,tol", [(1, 1e-12), (0, 2e-5)])
def test_operator_matches_assembled_matrix(pdgb, scenes, precision, tol):
    sc = _scene(pdgb, scenes, precision)
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    ora = make_oracle(sc)
    steps = 33          # past the phase-in, bonds broken, dt halved
    sim.advance(steps)
    ora.advance(steps)
    rng = np.random.default_rng(5)
    x = np.zeros((sc.n, 4))
    x[:, :3] = rng.standard_normal((sc.n, 3))
    y, dot, xs = apply_on_device(pdgb, sim, x)
    y_ref = ora.apply_A(xs)
    err = np.abs(y[:, :3] - y_ref[:, :3]).max() / np.abs(y_ref[:, :3]).max()
    assert err < tol
    assert abs(dot - float(np.sum(xs[:, :3] * y_ref[:, :3]))) <= tol * abs(dot)


def test_operator_view_fields(pdgb, scenes):
    sc = _scene(pdgb, scenes, 0)
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    v = sim.operator_view()
    assert v.n == sc.n and v.row_ptr and v.bond_slot and v.perm and v.ref_pos and v.disp
    assert v.lanes_per_particle in (4, 8, 16, 32) and v.blocks > 0
    assert v.mass == sc.sim.pd_particle_mass
