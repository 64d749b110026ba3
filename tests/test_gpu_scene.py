"""The example scene on the GPU (src/examples/scene.cpp): an OBJ mesh scaled
into the box and filled with a lattice, against the reference's own Scene
(golden fixtures from tests/golden/make_mesh_golden.py).  Particle counts,
positions and velocities must be identical."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "mesh_fill.npz")
CASES = ["icosphere", "torus_quads", "box_on_lattice", "blob_offset_box", "icosphere_jittered"]


def _scene(pdgb, g, name, tmp_path):
    obj = tmp_path / (name + ".obj")
    obj.write_bytes(g[name + "/obj"].tobytes())
    prm = g[name + "/params"]
    sp = pdgb.SystemParameter()
    sim, run = sp.getSimulationParameters(), sp.getRunningParameters()
    sim.boundary_min_x, sim.boundary_min_y, sim.boundary_min_z = prm[0:3]
    sim.boundary_max_x, sim.boundary_max_y, sim.boundary_max_z = prm[3:6]
    sim.pd_particle_radius = prm[6]
    sim.scaleFactor = prm[7]
    run.mesh_translation_x, run.mesh_translation_y, run.mesh_translation_z = prm[8:11]
    run.pd_initial_velocity = prm[11]
    run.obj_file = str(obj).encode()
    run.gpu_device = 0
    return sim, run, int(prm[12])


@pytest.mark.parametrize("name", CASES)
def test_mesh_fill_matches_reference_scene(pdgb, tmp_path, name):
    g = np.load(GOLDEN)
    sim, run, arrangement = _scene(pdgb, g, name, tmp_path)
    scene = pdgb.Scene(sim, run, arrangement, jitter_seed=1)
    pos_ref, vel_ref = g[name + "/pos"], g[name + "/vel"]
    assert sim.num_pd_particle == pos_ref.shape[0]
    act, pos, vel = scene.initPeridynamicsParticles()
    np.testing.assert_array_equal(pos, pos_ref)
    np.testing.assert_array_equal(vel, vel_ref)
    assert (act == pdgb.ACTIVE).all()


def test_scene_to_simulator(pdgb, scenes, tmp_path):
    """The reference's main loop: Scene sets num_pd_particle and fills the
    arrays, the Simulator steps them (examples/main.cpp:35-116)."""
    g = np.load(GOLDEN)
    sim, run, _ = _scene(pdgb, g, "icosphere", tmp_path)
    sim.pd_kernel_coeff = 5.001
    sim.pd_horizon = 5.001 * sim.pd_particle_radius
    sim.pd_particle_mass = 1e-3
    sim.pd_time_step = 128
    run.pd_stretch_limit_s0 = 1e-3
    scene = pdgb.Scene(sim, run)
    act, pos, vel = scene.initPeridynamicsParticles()
    opt = pdgb.default_options()
    opt.bond_stiffness = 1e6
    opt.time_step_base = 1e-5 / 128
    opt.cg_relative_tolerance = 1e-6
    simulator = pdgb.Simulator(0, sim, run, opt)
    simulator.get_pd_position()[:] = pos
    simulator.get_pd_velocity()[:] = vel
    simulator.get_pd_activity()[:] = act
    simulator.makeReady()
    simulator.advance(3)
    assert simulator.get_current_step() == 3 and simulator.CGConvergence()
    assert simulator.stats().bonds_initial > 0


def test_scene_errors(pdgb, tmp_path):
    sp = pdgb.SystemParameter()
    sim, run = sp.getSimulationParameters(), sp.getRunningParameters()
    run.obj_file = str(tmp_path / "missing.obj").encode()
    sim.pd_particle_radius = 0.02
    with pytest.raises(pdgb.PdError) as e:
        pdgb.Scene(sim, run)
    assert e.value.status == 6
    (tmp_path / "empty.obj").write_text("# nothing\n")
    run.obj_file = str(tmp_path / "empty.obj").encode()
    with pytest.raises(pdgb.PdError) as e:
        pdgb.Scene(sim, run)
    assert e.value.status == 1
