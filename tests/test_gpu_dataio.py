"""DataIO (src/core/dataIO.cu): frame files, simulation-info files and
checkpoint / restart through the C ABI.

Frames must hold exactly the exported arrays in the reference's layout;
sim_info.dat must be the reference's SimulationParameters struct; a run
restored from a checkpoint must continue bit for bit.
"""
import ctypes as C
import os

import numpy as np
import pytest

from helpers import same_sets

pytestmark = pytest.mark.gpu


class RefSimulationParameters(C.Structure):
    """Field order and types of the reference's SimulationParameters
    (src/core/parameters.h:16-88 with real_t = double)."""
    _fields_ = (
        [(k, C.c_int) for k in ("num_total_particle", "num_sph_particle", "num_pd_particle", "num_cell_x",
                                "num_cell_y", "num_cell_z", "num_cells", "num_clists")]
        + [(k, C.c_double) for k in ("cell_size", "sph_kernel_coeff", "pd_kernel_coeff", "sph_particle_mass",
                                     "pd_particle_mass", "sph_sph_viscosity", "sph_boundary_viscosity",
                                     "sph_pd_slip", "boundary_min_x", "boundary_min_y", "boundary_min_z",
                                     "boundary_max_x", "boundary_max_y", "boundary_max_z", "pd_min_x",
                                     "pd_min_y", "pd_min_z", "pd_max_x", "pd_max_y", "pd_max_z")]
        + [(k, C.c_int) for k in ("boundaryPlaneSize", "boundaryPlaneBottomIndex", "boundaryPlaneBottomSize",
                                  "boundaryPlaneTopIndex", "boundaryPlaneTopSize", "boundaryPlaneFrontIndex",
                                  "boundaryPlaneFrontSize", "boundaryPlaneBackIndex", "boundaryPlaneBackSize",
                                  "boundaryPlaneLeftSideIndex", "boundaryPlaneLeftSideSize",
                                  "boundaryPlaneRightSideIndex", "boundaryPlaneRightSideSize",
                                  "pd_max_num_bonds", "pd_time_step")]
        + [(k, C.c_double) for k in ("sph_kernel_smooth_length", "sph_kernel_smooth_length_squared",
                                     "sph_particle_radius", "sph_kernel_poly6", "sph_kernel_spiky",
                                     "sph_rest_density", "pd_particle_radius", "pd_horizon", "pd_C_times_V",
                                     "sph_pd_min_distance", "clockScale", "scaleFactor")]
    )


def _with_output(sc, path):
    sc.run.saving_path = str(path).encode()
    sc.run.dump_velocity = 1
    sc.run.dump_activity = 1
    sc.run.dump_pd_bond_list_top = 1
    return sc


def test_frames_and_sim_info(pdgb, scenes, tmp_path):
    sc = _with_output(scenes.reference_block(n_side=8, integrator=pdgb.NEWMARK_BETA, adaptive=1,
                                             expansion=300.0), tmp_path)
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    n = sc.n
    cnt0 = sim.get(pdgb.VAR_BOND_COUNT)
    expected = {}
    for frame in (1, 2):
        sim.dataIO_newFrame()
        sim.dataIO_getDataAndWrite()
        assert sim.dataIO_savedFrame() == frame
        expected[frame] = (sim.get(pdgb.VAR_POSITION_SCALED), sim.get(pdgb.VAR_VELOCITY),
                           sim.get(pdgb.VAR_BOND_COUNT))
        sim.advance(60)
    data = tmp_path / "DATA"
    for frame, (x, v, cnt) in expected.items():
        pos = np.fromfile(data / "PD_POSITION" / f"frame.{frame}", np.float64).reshape(n, 4)
        np.testing.assert_array_equal(pos, x)
        vel = np.fromfile(data / "PD_VELOCITY" / f"frame.{frame}", np.float64).reshape(n, 4)
        np.testing.assert_array_equal(vel, v)
        act = np.fromfile(data / "PD_ACTIVITY" / f"frame.{frame}", np.int32)
        np.testing.assert_array_equal(act, sc.act)
        top = np.fromfile(data / "PD_BOND_LIST_TOP" / f"frame.{frame}", np.int32)
        np.testing.assert_array_equal(top, cnt - 1)
        otop = np.fromfile(data / "PD_ORIGINAL_BOND_COUNT" / f"frame.{frame}", np.int32)
        np.testing.assert_array_equal(otop, cnt0 - 1)
    assert (expected[2][2] < cnt0).any(), "the scene should break bonds between the frames"
    for d in ("SPH_POSITION", "SPH_VELOCITY", "SPH_ACTIVITY", "STATE"):
        assert (data / d).is_dir()
    raw = (data / "sim_info.dat").read_bytes()
    assert len(raw) == C.sizeof(RefSimulationParameters)
    info = RefSimulationParameters.from_buffer_copy(raw)
    s, _, _ = sim.params()
    assert info.num_pd_particle == n and info.num_total_particle == n and info.num_sph_particle == 0
    assert info.pd_horizon == s.pd_horizon and info.pd_particle_radius == s.pd_particle_radius
    assert info.scaleFactor == s.scaleFactor and info.pd_kernel_coeff == s.pd_kernel_coeff
    assert info.pd_max_num_bonds == s.pd_max_num_bonds
    assert info.boundary_max_z == s.boundary_max_z
    assert info.pd_min_x == pytest.approx(sc.pos[:, 0].min()) and info.pd_max_y == pytest.approx(sc.pos[:, 1].max())
    viz = (data / "viz_info.dat").read_text().splitlines()
    assert f"num_pd_particle {n}" in viz
    assert any(line.startswith("pd_horizon ") for line in viz) and len(viz) == 21


@pytest.mark.parametrize("precision", [0, 1])
def test_checkpoint_restart_bitwise(pdgb, scenes, tmp_path, precision):
    """Saving at step 25 and restoring into a fresh handle continues the run
    exactly as if it had not been interrupted (breaking Newmark scene with
    time-step rollbacks)."""
    def scene():
        sc = scenes.reference_block(n_side=7, seed=5, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=150.0,
                                    cg_tol=1e-10)
        sc.opt.precision = precision
        return _with_output(sc, tmp_path)

    ref = scenes.make_simulator(scene())
    ref.makeReady()
    ref.advance(70)
    a = scenes.make_simulator(scene())
    a.makeReady()
    a.advance(25)
    a.dataIO_newFrame()
    a.dataIO_saveState(25)
    assert os.path.exists(tmp_path / "DATA" / "STATE" / "state.25")
    a.close()
    b = scenes.make_simulator(scene())
    b.makeReady()
    b.dataIO_loadState(25)
    assert b.get_current_step() == 25 and b.dataIO_savedFrame() == 1
    b.advance(45)
    np.testing.assert_array_equal(b.get(pdgb.VAR_POSITION), ref.get(pdgb.VAR_POSITION))
    np.testing.assert_array_equal(b.get(pdgb.VAR_VELOCITY), ref.get(pdgb.VAR_VELOCITY))
    assert same_sets(b.alive_sets(), ref.alive_sets())
    sb, sr = b.stats(), ref.stats()
    assert sb.current_step == sr.current_step == 70
    assert sb.time_step_ticks == sr.time_step_ticks and sb.total_cg_iterations == sr.total_cg_iterations
    assert sb.bonds_alive < sb.bonds_initial


def test_load_state_errors(pdgb, scenes, tmp_path):
    sc = _with_output(scenes.reference_block(n_side=5), tmp_path)
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    sim.advance(2)
    sim.dataIO_saveState(2)
    with pytest.raises(pdgb.PdError) as e:
        sim.dataIO_loadState(3)          # no such file
    assert e.value.status == 6
    other = scenes.make_simulator(_with_output(scenes.reference_block(n_side=4), tmp_path))
    other.makeReady()
    with pytest.raises(pdgb.PdError) as e:
        other.dataIO_loadState(2)        # another particle count
    assert e.value.status == 8
    fresh = scenes.make_simulator(_with_output(scenes.reference_block(n_side=5), tmp_path))
    with pytest.raises(pdgb.PdError) as e:
        fresh.dataIO_loadState(2)        # before make_ready
    assert e.value.status == 3


def test_checkpoint_restart_with_history_guess(pdgb, scenes, tmp_path):
    """warm_start = 2: a restored handle starts with an empty projection
    history (the history is not part of the checkpoint), so it continues
    within the CG tolerance of the uninterrupted run rather than bit for bit:
    the same bond sets and time steps, positions to 1e-7 relative."""
    def scene():
        sc = scenes.reference_block(n_side=7, seed=5, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=150.0,
                                    cg_tol=1e-10)
        sc.opt.warm_start = 2
        return _with_output(sc, tmp_path)

    ref = scenes.make_simulator(scene())
    ref.makeReady()
    ref.advance(50)
    a = scenes.make_simulator(scene())
    a.makeReady()
    a.advance(25)
    a.dataIO_saveState(25)
    a.close()
    b = scenes.make_simulator(scene())
    b.makeReady()
    b.dataIO_loadState(25)
    b.advance(25)
    assert same_sets(b.alive_sets(), ref.alive_sets())
    assert b.stats().time_step_ticks == ref.stats().time_step_ticks
    x, xr = b.get(pdgb.VAR_POSITION)[:, :3], ref.get(pdgb.VAR_POSITION)[:, :3]
    assert np.abs(x - xr).max() <= 1e-7 * np.abs(xr).max()
    assert b.stats().ws_guesses_kept > 0
