"""The matrix-free system operator (pd_apply_operator) against the oracle's
assembled matrix A = M + beta h^2 K applied by computeAx's restatement
(src/core/cg_solver.cuh:343-383)."""
import numpy as np
import pytest

from helpers import apply_on_device, make_oracle

pytestmark = pytest.mark.gpu


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
