"""Checkpoints in the reference's own layout (DataIO::saveState / loadState,
src/core/dataIO.cu:123-198; the layout restated in tests/golden/ref_state.py
from src/core/memory_manager.h:29-90 and memory_manager.cu:16-178).

* What pd_dataio_save_state_reference writes is that layout, and its arrays
  are the handle's (read back with the restated layout).
* A handle continues from a file it wrote itself, and pd_dataio_load_state
  finds the reference layout when there is no checkpoint of its own.
* A state of the ORACLE (the reference step restated) written in that layout
  is read by a fresh handle, which then continues in step with the oracle.
"""
import os

import numpy as np
import pytest

from golden import ref_state
from helpers import assert_positions, make_oracle, same_sets
from test_gpu_dataio import RefSimulationParameters

pytestmark = pytest.mark.gpu


def _sim_info(root):
    raw = open(os.path.join(root, "DATA", "sim_info.dat"), "rb").read()
    assert len(raw) == __import__("ctypes").sizeof(RefSimulationParameters)
    return RefSimulationParameters.from_buffer_copy(raw)


def _counts(info):
    return (info.num_sph_particle, info.num_pd_particle, info.num_cells, info.num_clists, info.boundaryPlaneSize)


def _scene(pdgb, scenes, tmp_path, precision, integrator=None, adaptive=1):
    sc = scenes.reference_block(n_side=7, seed=5, integrator=pdgb.NEWMARK_BETA if integrator is None else integrator,
                                adaptive=adaptive, expansion=150.0, cg_tol=1e-10)
    sc.opt.precision = precision
    sc.run.saving_path = str(tmp_path).encode()
    return sc


@pytest.mark.parametrize("precision", [1, 0])
def test_reference_layout_holds_the_handles_arrays(pdgb, scenes, tmp_path, precision):
    sc = _scene(pdgb, scenes, tmp_path, precision)
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    sim.advance(45)                 # bonds break from step ~40
    sim.dataIO_newFrame()
    sim.dataIO_saveStateReference(45)
    info = _sim_info(tmp_path)
    path = os.path.join(tmp_path, "STATE", "state.45")
    d = ref_state.read(path, _counts(info), info.scaleFactor)
    assert d["file_size"] == d["expected_size"] and d["savedFrame"] == 1
    n = sc.n
    x = sim.get(pdgb.VAR_POSITION)
    np.testing.assert_allclose(d["PD_POSITION"][:, :3], x[:, :3], rtol=1e-15, atol=0)
    np.testing.assert_array_equal(d["PD_VELOCITY"][:, :3], sim.get(pdgb.VAR_VELOCITY)[:, :3])
    np.testing.assert_array_equal(d["PD_STRETCH"], sim.get(pdgb.VAR_STRETCH))
    np.testing.assert_array_equal(d["PD_ORIGINAL_STRETCH"], sim.get(pdgb.VAR_ORIGINAL_STRETCH))
    np.testing.assert_array_equal(d["PD_NEW_STRETCH"], sim.get(pdgb.VAR_NEW_STRETCH))
    np.testing.assert_array_equal(d["PD_ACTIVITY"], sc.act)
    cnt = sim.get(pdgb.VAR_BOND_COUNT)
    np.testing.assert_array_equal(d["PD_BOND_LIST_TOP"], cnt - 1)
    rp = sim.get(pdgb.VAR_BOND_ROW_PTR)
    np.testing.assert_array_equal(d["PD_ORIGINAL_BOND_LIST_TOP"], np.diff(rp) - 1)
    assert np.all(d["PD_BOND_LIST_TOP_BACKUP"] >= d["PD_BOND_LIST_TOP"])
    bl = d["PD_BOND_LIST"].reshape(ref_state.MAX_BONDS, n)
    alive = sim.alive_sets()
    for p in range(n):
        assert np.array_equal(np.sort(bl[:cnt[p], p]), alive[p]), p
    assert sim.stats().bonds_alive < sim.stats().bonds_initial   # the file carries broken bonds


@pytest.mark.parametrize("precision", [1, 0])
def test_reference_layout_round_trip(pdgb, scenes, tmp_path, precision):
    """Save past step 45 in the reference layout, where the adaptive
    scheme's sub-step count is 0 (the reference's file does not hold it),
    load into a fresh handle (through pd_dataio_load_state, which falls back
    to the reference layout), continue 20 steps: the uninterrupted run's bond
    sets and time steps; the bond rows come back in the file's order, so
    positions agree to the summation order (FP64 1e-9, mixed as the parity
    tests)."""
    a = scenes.make_simulator(_scene(pdgb, scenes, tmp_path, precision))
    a.makeReady()
    a.advance(45)
    while a.stats().substep != 0 and a.get_current_step() < 80:
        a.advance(1)
    k = a.get_current_step()
    assert a.stats().substep == 0
    a.dataIO_saveStateReference(k)
    a.close()
    ref = scenes.make_simulator(_scene(pdgb, scenes, tmp_path, precision))
    ref.makeReady()
    ref.advance(k + 20)
    b = scenes.make_simulator(_scene(pdgb, scenes, tmp_path, precision))
    b.makeReady()
    b.dataIO_loadState(k)           # no DATA/STATE/state.<k>: the reference layout is read
    assert b.get_current_step() == k
    b.advance(20)
    assert same_sets(b.alive_sets(), ref.alive_sets())
    assert b.stats().time_step_ticks == ref.stats().time_step_ticks
    sc = _scene(pdgb, scenes, tmp_path, precision)
    assert_positions(b.get(pdgb.VAR_POSITION), ref.get(pdgb.VAR_POSITION), sc.pos, precision,
                     "reference-layout round trip")


@pytest.mark.parametrize("precision", [1, 0])
def test_oracle_state_in_reference_layout_continues(pdgb, scenes, tmp_path, precision):
    """The oracle runs the breaking Newmark block past step 40 (bonds broken,
    time step halved), stopping where the adaptive scheme's sub-step count is 0
    (the reference keeps that count out of its file, and the loader starts it
    at 0); its state is written in the reference's layout with the run's
    sim_info.dat; a fresh handle loads it and both continue 15 steps in step."""
    sc = _scene(pdgb, scenes, tmp_path, precision)
    ora = make_oracle(sc)
    ora.advance(40)
    k = 40
    while ora.lib.pdo_substep(ora.h) != 0 and k < 60:
        ora.advance(1)
        k += 1
    assert ora.lib.pdo_substep(ora.h) == 0
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    sim.dataIO_getDataAndWrite()    # DATA/sim_info.dat of this scene
    info = _sim_info(tmp_path)
    info.pd_time_step = ora.dt_ticks
    info.clockScale = ora.clock_scale
    open(os.path.join(tmp_path, "DATA", "sim_info.dat"), "wb").write(bytes(info))
    n = sc.n
    rp, col, top = ora.row_ptr, ora.bond_list, ora.bond_top
    assert int((top + 1).sum()) < int(np.diff(rp).sum())   # bonds are broken at the saved step
    bl = np.zeros((ref_state.MAX_BONDS, n), np.int32)
    for p in range(n):
        row = col[rp[p]:rp[p + 1]]
        bl[:len(row), p] = row
    opos = np.zeros((n, 4))
    opos[:, :3] = sc.pos[:, :3]
    arrays = {
        "PD_ACTIVITY": sc.act, "PD_POSITION": ora.position, "PD_POSITION_BACKUP": ora.position_backup,
        "PD_VELOCITY": ora.velocity, "PD_VELOCITY_BACKUP": ora.velocity_backup, "PD_ORIGINAL_POSITION": opos,
        "PD_ORIGINAL_STRETCH": ora.original_stretch, "PD_STRETCH": ora.stretch, "PD_NEW_STRETCH": ora.new_stretch,
        "PD_ORIGINAL_BOND_LIST_TOP": np.diff(rp).astype(np.int32) - 1, "PD_BOND_LIST": bl.reshape(-1),
        "PD_BOND_LIST_TOP": top, "PD_BOND_LIST_TOP_BACKUP": ora.bond_top_backup,
        "PD_SYSTEM_SOLUTION": ora.solution,
    }
    os.makedirs(os.path.join(tmp_path, "STATE"), exist_ok=True)
    ref_state.write(os.path.join(tmp_path, "STATE", "state.%d" % k), _counts(info), info.scaleFactor, 3, arrays)
    sim.dataIO_loadStateReference(k)
    assert sim.get_current_step() == k and sim.dataIO_savedFrame() == 3
    assert same_sets(sim.alive_sets(), ora.alive_sets())
    for _ in range(3):
        sim.advance(5)
        ora.advance(5)
        assert same_sets(sim.alive_sets(), ora.alive_sets())
        assert sim.stats().time_step_ticks == ora.dt_ticks
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, precision, "oracle state, reference layout")


def test_reference_layout_rejects_another_scene(pdgb, scenes, tmp_path):
    sc = _scene(pdgb, scenes, tmp_path, 1)
    a = scenes.make_simulator(sc)
    a.makeReady()
    a.advance(3)
    a.dataIO_saveStateReference(3)
    other = _scene(pdgb, scenes, tmp_path, 1)
    other.pos[:, 0] += 1e-3             # same count, other original positions
    b = scenes.make_simulator(other)
    b.makeReady()
    with pytest.raises(pdgb.PdError) as e:
        b.dataIO_loadStateReference(3)
    assert e.value.status == 8
