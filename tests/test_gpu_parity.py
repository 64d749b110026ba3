"""Parity of the CUDA path (through the C ABI) against the CPU oracle.

Bond lists and broken-bond sets must match exactly; positions and
velocities within the stated tolerances:
  FP64 mode:  1e-9 relative (differences come only from summation order)
  mixed mode: 1e-5 relative after the full run (FP32 forces/SpMV)
"""
import numpy as np
import pytest

from helpers import make_oracle, rel_err, same_sets

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-9
MIXED_TOL = 1e-5


def _run_pair(pdgb, scenes, scene, steps, check_every=10):
    sim = scenes.make_simulator(scene)
    sim.makeReady()
    ora = make_oracle(scene)
    assert same_sets(sim.alive_sets(), ora.alive_sets()), "initial bond lists differ"
    done = 0
    while done < steps:
        k = min(check_every, steps - done)
        sim.advance(k)
        ora.advance(k)
        done += k
        assert same_sets(sim.alive_sets(), ora.alive_sets()), f"broken-bond sets differ at step {done}"
        assert sim.stats().time_step_ticks == ora.dt_ticks
    return sim, ora


def test_bonds_reference_block(pdgb, scenes):
    for seed in (1, 2, 3):
        sc = scenes.reference_block(n_side=9, seed=seed)
        sim = scenes.make_simulator(sc)
        sim.makeReady()
        ora = make_oracle(sc)
        assert same_sets(sim.alive_sets(), ora.alive_sets())
        np.testing.assert_array_equal(sim.get(pdgb.VAR_ORIGINAL_STRETCH), ora.original_stretch)


def test_bonds_cube_lattice(pdgb, scenes):
    sc = scenes.cube_lattice(n_side=12, seed=3)
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    ora = make_oracle(sc)
    assert same_sets(sim.alive_sets(), ora.alive_sets())


@pytest.mark.parametrize("coeff,interior", [(4.001, 26), (5.001, 80), (6.001, 92)])
def test_bond_count_known_answer(pdgb, scenes, coeff, interior):
    """Unjittered lattice: interior particles have 26 / 80 / 92 bonds for
    horizons of 2 / 2.5 / 3 spacings."""
    sc = scenes.reference_block(n_side=9, pd_kernel_coeff=coeff, jitter=0.0)
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    cnt = sim.get(pdgb.VAR_BOND_COUNT)
    assert cnt.max() == interior
    assert cnt[4 * 81 + 4 * 9 + 4] == interior


def test_step_fp64_implicit_euler(pdgb, scenes):
    sc = scenes.reference_block(n_side=8, integrator=pdgb.IMPLICIT_EULER)
    sc.opt.precision = pdgb.PRECISION_FP64
    sim, ora = _run_pair(pdgb, scenes, sc, 40)
    assert rel_err(sim.get(pdgb.VAR_POSITION), ora.position) < FP64_TOL
    assert rel_err(sim.get(pdgb.VAR_VELOCITY), ora.velocity) < 1e-7
    assert abs(sim.stats().last_cg_iterations - ora.cg_iters) <= 1


def test_step_fp64_newmark_breaking(pdgb, scenes):
    sc = scenes.reference_block(n_side=8, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=300.0)
    sc.opt.precision = pdgb.PRECISION_FP64
    sim, ora = _run_pair(pdgb, scenes, sc, 60)
    st = sim.stats()
    assert st.bonds_alive < st.bonds_initial, "scene should break bonds"
    assert rel_err(sim.get(pdgb.VAR_POSITION), ora.position) < FP64_TOL


def test_step_mixed_newmark_breaking(pdgb, scenes):
    sc = scenes.reference_block(n_side=8, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=300.0,
                                cg_tol=1e-9)
    sim, ora = _run_pair(pdgb, scenes, sc, 60)
    assert rel_err(sim.get(pdgb.VAR_POSITION), ora.position) < MIXED_TOL


def test_cube_lattice_mixed_100_steps(pdgb, scenes):
    """The small plain-method workload: 16^3, clamped base, CG rel 1e-6."""
    sc = scenes.cube_lattice()
    sim, ora = _run_pair(pdgb, scenes, sc, 100, check_every=20)
    assert rel_err(sim.get(pdgb.VAR_POSITION), ora.position) < MIXED_TOL
    v, vo = sim.get(pdgb.VAR_VELOCITY), ora.velocity
    assert np.abs(v - vo)[:, :3].max() / np.abs(vo).max() < 1e-3
    assert sim.CGConvergence()


def test_errors(pdgb, scenes):
    sc = scenes.reference_block(n_side=5)
    sc.opt.max_bonds_per_particle = 10
    sim = scenes.make_simulator(sc)
    with pytest.raises(pdgb.PdError) as e:
        sim.makeReady()
    assert e.value.status == 4
    sc = scenes.reference_block(n_side=4)
    sim = scenes.make_simulator(sc)
    with pytest.raises(pdgb.PdError) as e:
        sim.advance(1)
    assert e.value.status == 3


@pytest.mark.parametrize("n_side", [1, 2])
def test_tiny_scenes(pdgb, scenes, n_side):
    sc = scenes.reference_block(n_side=n_side)
    sc.opt.precision = pdgb.PRECISION_FP64
    sim, ora = _run_pair(pdgb, scenes, sc, 5, check_every=5)
    assert rel_err(sim.get(pdgb.VAR_POSITION), ora.position) < FP64_TOL
