"""pd_sph_collide (the reference's collideDifferentParticles,
src/core/simulator.cuh:1590-1733) against the oracle's restatement
(oracle/pd_oracle.c pdo_sph_collide): a cloud of SPH particles around a PD
block, on the reference's grid of the block's simulation parameters.  The SPH
corrections and the PD velocities must agree bit for bit (both in FP64 in the
reference's operation order), and the handle then keeps stepping in step
with the oracle."""
import numpy as np
import pytest

from helpers import assert_positions, make_oracle, same_sets

pytestmark = pytest.mark.gpu


def _cloud(sc, n, seed):
    rng = np.random.default_rng(seed)
    lo = sc.pos[:, :3].min(0) - 1.0e-3
    hi = sc.pos[:, :3].max(0) + 1.0e-3
    pos = np.zeros((n, 4))
    pos[:, :3] = lo + (hi - lo) * rng.random((n, 3))
    vel = np.zeros((n, 4))
    vel[:, :3] = rng.normal(0.0, 0.5, (n, 3))
    return pos, vel


def _grid(sc):
    m = sc.sim
    return (np.array([m.boundary_min_x, m.boundary_min_y, m.boundary_min_z]), m.cell_size,
            np.array([m.num_cell_x, m.num_cell_y, m.num_cell_z], dtype=np.int32), m.sph_particle_radius,
            m.sph_particle_mass)


@pytest.mark.parametrize("precision", [1, 0])
@pytest.mark.parametrize("slip", [1.0, 0.25])
def test_sph_collision_matches_oracle(pdgb, scenes, precision, slip):
    sc = scenes.reference_block(n_side=8, seed=5, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=150.0,
                                cg_tol=1e-10)
    sc.opt.precision = precision
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    ora = make_oracle(sc)
    pos, vel = _cloud(sc, 4000, seed=3)
    pg, vg = pos.copy(), vel.copy()
    po, vo = pos.copy(), vel.copy()
    lo, cell, n, r_sph, m_sph = _grid(sc)
    cg = sim.sph_collide(pg, vg, slip)
    co = ora.sph_collide(lo, cell, n, r_sph, m_sph, slip, po, vo)
    assert cg == co and cg > 100, (cg, co)
    np.testing.assert_array_equal(pg, po)
    np.testing.assert_array_equal(vg, vo)
    hit = np.any(pg != pos, axis=1)
    assert hit.sum() == cg
    np.testing.assert_array_equal(sim.get(pdgb.VAR_VELOCITY)[:, :3], ora.velocity[:, :3])
    # the corrected SPH particles sit at r_sph + r_pd from the PD particle they hit
    # (the distance divisor is rounded to FP32, as the reference's fmaxf)
    x = sim.get(pdgb.VAR_POSITION)[:, :3]
    dmin = np.array([np.min(np.linalg.norm(x - p[:3], axis=1)) for p in pg[hit][:200]])
    assert np.all(dmin <= (r_sph + sc.sim.pd_particle_radius) * (1 + 1e-6))
    # the PD velocities set by the collision carry into the next steps
    for _ in range(2):
        sim.advance(5)
        ora.advance(5)
        assert same_sets(sim.alive_sets(), ora.alive_sets())
        assert sim.stats().time_step_ticks == ora.dt_ticks
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, precision, f"after SPH collision, slip {slip}")


def test_sph_collision_after_steps_and_errors(pdgb, scenes):
    """The same after 20 steps (FP64 state from the step, not the input), an
    empty SPH set, and the argument checks."""
    sc = scenes.reference_block(n_side=8, seed=5, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=150.0,
                                cg_tol=1e-12)
    sc.opt.precision = 1
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    ora = make_oracle(sc)
    sim.advance(20)
    ora.advance(20)
    pos, vel = _cloud(sc, 3000, seed=9)
    pg, vg, po, vo = pos.copy(), vel.copy(), pos.copy(), vel.copy()
    lo, cell, n, r_sph, m_sph = _grid(sc)
    cg = sim.sph_collide(pg, vg, 1.0)
    co = ora.sph_collide(lo, cell, n, r_sph, m_sph, 1.0, po, vo)
    assert cg == co and cg > 50
    np.testing.assert_allclose(pg, po, rtol=0, atol=1e-12 * np.abs(po).max())
    np.testing.assert_allclose(vg, vo, rtol=0, atol=1e-9 * np.abs(vo).max())
    assert sim.sph_collide(np.zeros((0, 4)), np.zeros((0, 4))) == 0
    with pytest.raises(ValueError):
        sim.sph_collide(np.zeros((3, 3)), np.zeros((3, 3)))
    fresh = scenes.make_simulator(sc)
    with pytest.raises(pdgb.PdError) as e:
        fresh.sph_collide(pos.copy(), vel.copy())
    assert e.value.status == 3
