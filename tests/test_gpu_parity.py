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


@pytest.mark.parametrize("coeff,interior", [(3.999, 26), (4.001, 32), (5.001, 80), (5.999, 92), (6.001, 122)])
def test_bond_count_known_answer(pdgb, scenes, coeff, interior):
    """Unjittered lattice, horizon = coeff * spacing / 2: an interior particle
    bonds every lattice vector v with |v| < coeff/2 spacings (|v|^2 in
    {1,2,3} -> 26, +{4} -> 32, +{5,6} -> 80, +{8} -> 92, +{9} -> 122)."""
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
    # the broken-bond mask export: per row, the bond-list entries it marks are
    # exactly the oracle's initial neighbours that are no longer alive
    rp, bl = sim.get(pdgb.VAR_BOND_ROW_PTR), sim.get(pdgb.VAR_BOND_LIST)
    mask, cnt = sim.get(pdgb.VAR_BROKEN_MASK), sim.get(pdgb.VAR_BOND_COUNT)
    assert mask.shape == bl.shape and int(mask.sum()) == int(rp[-1] - cnt.sum()) > 0
    for i, alive in enumerate(ora.alive_sets()):
        row, m = bl[rp[i]:rp[i + 1]], mask[rp[i]:rp[i + 1]]
        assert np.array_equal(np.sort(row[m == 1]), np.setdiff1d(row, alive)), i


def test_cube_lattice_mixed_100_steps(pdgb, scenes):
    """The small plain-method workload: 16^3, clamped base, CG rel 1e-6."""
    sc = scenes.cube_lattice()
    sim, ora = _run_pair(pdgb, scenes, sc, 100, check_every=20)
    assert rel_err(sim.get(pdgb.VAR_POSITION), ora.position) < MIXED_TOL
    # implicit Euler damps the impact out: the block is at rest after 100 steps,
    # so velocity errors are measured against the initial speed (5 m/s)
    v, vo = sim.get(pdgb.VAR_VELOCITY), ora.velocity
    vscale = max(np.abs(vo).max(), np.abs(sc.vel).max())
    assert np.abs(v - vo)[:, :3].max() / vscale < MIXED_TOL
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


@pytest.mark.parametrize("precision,tol", [(1, FP64_TOL), (0, MIXED_TOL)])
def test_newmark_dt_halving_and_doubling(pdgb, scenes, precision, tol):
    """Breaking stops mid-run: pd_time_step goes 128 -> 64 -> 128 -> 64 -> 128;
    the doubled step is used by the same step's assembly, solve and update."""
    sc = scenes.reference_block(n_side=7, seed=5, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=150.0,
                                cg_tol=1e-10)
    sc.opt.precision = precision
    sim, ora = _run_pair(pdgb, scenes, sc, 90, check_every=5)
    assert rel_err(sim.get(pdgb.VAR_POSITION), ora.position) < tol


@pytest.mark.parametrize("path", [1, 2])
def test_spmv_paths_mixed_breaking(pdgb, scenes, path):
    """Both mixed SpMV paths (shared-memory tiles, per-bond gathers) against
    the oracle on a breaking, rolling-back Newmark run."""
    sc = scenes.reference_block(n_side=8, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=300.0,
                                cg_tol=1e-9)
    sc.opt.spmv_path = path
    sim, ora = _run_pair(pdgb, scenes, sc, 60)
    assert sim.params()[2].spmv_path == path
    assert sim.stats().bonds_alive < sim.stats().bonds_initial
    assert rel_err(sim.get(pdgb.VAR_POSITION), ora.position) < MIXED_TOL


@pytest.mark.parametrize("path", [1, 2])
def test_spmv_paths_cube(pdgb, scenes, path):
    sc = scenes.cube_lattice(n_side=12, seed=2)
    sc.opt.spmv_path = path
    sim, ora = _run_pair(pdgb, scenes, sc, 40, check_every=20)
    assert sim.params()[2].spmv_path == path
    assert rel_err(sim.get(pdgb.VAR_POSITION), ora.position) < MIXED_TOL


def test_spmv_tiled_large_autotuned(pdgb, scenes):
    """Above 20000 particles the SpMV shape is measured (and the bond slots
    reordered for each candidate shape); the tiled and the gather paths give
    the same run (within the CG tolerance) and match the oracle."""
    runs = {}
    for path in (0, 1, 2):
        sc = scenes.impact_body(24000, "ball", coeff=5.0, speed=6.0, seed=4, steps=6)
        sc.opt.spmv_path = path
        sim = scenes.make_simulator(sc)
        sim.makeReady()
        sim.advance(6)
        assert sim.params()[2].spmv_path == (2 if path == 0 else path)
        runs[path] = sim
    ora = make_oracle(sc)
    ora.advance(6)
    for path, sim in runs.items():
        assert same_sets(sim.alive_sets(), ora.alive_sets())
        assert rel_err(sim.get(pdgb.VAR_POSITION), ora.position) < MIXED_TOL, path


@pytest.mark.parametrize("precision,tol", [(1, FP64_TOL), (0, MIXED_TOL)])
def test_pd_pd_contact(pdgb, scenes, precision, tol):
    """Two blocks collide: the PD-PD contact forces (collidePDParticles,
    off in the reference build) against the oracle's brute-force pairs."""
    sc = scenes.two_blocks(precision=precision)
    sim, ora = _run_pair(pdgb, scenes, sc, 80, check_every=20)
    assert rel_err(sim.get(pdgb.VAR_POSITION), ora.position) < tol
    assert rel_err(sim.get(pdgb.VAR_VELOCITY), ora.velocity) < max(tol, 1e-7) * 100
    # the contact changed the motion: without it the blocks pass into each other
    free = scenes.make_simulator(scenes.two_blocks(precision=precision, contact=False))
    free.makeReady()
    free.advance(80)
    x, xf = sim.get(pdgb.VAR_POSITION), free.get(pdgb.VAR_POSITION)
    n = x.shape[0] // 2
    assert x[:n, 0].max() < xf[:n, 0].max() - 0.2 * sc.info["spacing"]
