"""Batched stepping (pd_batch_*): every scene of a batch against the CPU
oracle and against its own single-scene Simulator.

Bond lists and broken-bond sets must match exactly, the time step and step
counter must follow the same adaptive history, positions within
  FP64 mode:  1e-9 relative (per-scene sums are reduced in another order)
  mixed mode: 1e-5 relative
"""
import numpy as np
import pytest

from helpers import assert_positions, make_oracle, rel_err, same_sets

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-9
MIXED_TOL = 1e-5


def _mix(pdgb, scenes, precision):
    """Blocks and balls of several horizons and both integrators, plus a
    reference-units block whose breaking halves and doubles the time step."""
    out = [
        scenes.impact_body(300, "block", coeff=5.0, speed=5.0, seed=1, precision=precision, steps=30),
        scenes.impact_body(400, "ball", coeff=6.0, speed=8.0, seed=2, precision=precision, steps=30),
        scenes.impact_body(250, "block", coeff=4.0, speed=2.0, seed=3, precision=precision, steps=30),
    ]
    rb = scenes.reference_block(n_side=7, seed=5, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=150.0,
                                cg_tol=1e-10)
    rb.opt.precision = precision
    out.append(rb)
    return out


def _batch(pdgb, scenes, lst, **opts):
    o = pdgb.BatchOptions()
    pdgb.library().pd_batch_options_default(o)
    for k, v in opts.items():
        setattr(o, k, v)
    b = pdgb.Batch(0, o)
    for sc in lst:
        scenes.add_to_batch(b, sc)
    b.makeReady()
    return b


@pytest.mark.parametrize("precision,tol", [(1, FP64_TOL), (0, MIXED_TOL)])
def test_batch_matches_oracle(pdgb, scenes, precision, tol):
    lst = _mix(pdgb, scenes, precision)
    b = _batch(pdgb, scenes, lst)
    oras = [make_oracle(sc) for sc in lst]
    for k, o in enumerate(oras):
        assert same_sets(b.alive_sets(k), o.alive_sets()), f"scene {k}: initial bonds differ"
    done = 0
    while done < 40:
        b.advance(10)
        for o in oras:
            o.advance(10)
        done += 10
        for k, o in enumerate(oras):
            st = b.stats(k)
            assert st.current_step == done
            assert st.time_step_ticks == o.dt_ticks, f"scene {k}: time step differs at step {done}"
            assert same_sets(b.alive_sets(k), o.alive_sets()), f"scene {k}: broken bonds differ at step {done}"
    for k, (sc, o) in enumerate(zip(lst, oras)):
        assert_positions(b.get(k, pdgb.VAR_POSITION), o.position, sc.pos, precision, f"batch scene {k}")
        assert b.stats(k).cg_converged == 1
    # the reference-units block broke bonds and went through rollbacks
    st = b.stats(3)
    assert st.bonds_alive < st.bonds_initial


def test_batch_matches_single_scene_simulators(pdgb, scenes):
    """Eight scenes of uneven sizes against eight separate pd_handles."""
    lst = scenes.batched_scenes(count=8, n_min=200, n_max=3000, seed=3, steps=20)
    b = _batch(pdgb, scenes, lst)
    sims = []
    for sc in lst:
        s = scenes.make_simulator(sc)
        s.makeReady()
        sims.append(s)
    b.advance(20)
    for s in sims:
        s.advance(20)
    offs = b.offsets()
    assert offs[-1] == sum(sc.n for sc in lst)
    for k, (sc, s) in enumerate(zip(lst, sims)):
        assert offs[k + 1] - offs[k] == sc.n
        assert same_sets(b.alive_sets(k), s.alive_sets()), f"scene {k}"
        sb, ss = b.stats(k), s.stats()
        assert sb.current_step == ss.current_step == 20
        assert sb.time_step_ticks == ss.time_step_ticks
        assert abs(sb.sim_time - ss.sim_time) <= 1e-15 * max(1.0, abs(ss.sim_time))
        x, xs = b.get(k, pdgb.VAR_POSITION), s.get(pdgb.VAR_POSITION)
        assert rel_err(x, xs) < MIXED_TOL, f"scene {k}"


def test_batch_graph_replay_is_deterministic(pdgb, scenes):
    """The graph replay and direct launches run the same item partition and
    reduction order: bitwise equal results."""
    lst = _mix(pdgb, scenes, 0)
    b1 = _batch(pdgb, scenes, lst, use_graph=1, lanes_per_particle=8, spmv_unroll=2, item_rows=128)
    b2 = _batch(pdgb, scenes, lst, use_graph=0, lanes_per_particle=8, spmv_unroll=2, item_rows=128)
    b1.advance(25)
    b2.advance(25)
    for k in range(len(lst)):
        np.testing.assert_array_equal(b1.get(k, pdgb.VAR_POSITION), b2.get(k, pdgb.VAR_POSITION))
        np.testing.assert_array_equal(b1.get(k, pdgb.VAR_VELOCITY), b2.get(k, pdgb.VAR_VELOCITY))


def test_batch_autotuned_shape(pdgb, scenes):
    """Above 20000 particles the launch shape is measured; any shape gives
    the single-scene results."""
    lst = [scenes.impact_body(9000, "block", coeff=5.0, speed=5.0, seed=11, steps=10),
           scenes.impact_body(12000, "ball", coeff=5.0, speed=6.0, seed=12, steps=10)]
    b = _batch(pdgb, scenes, lst)
    cfg = b.config()
    assert cfg.autotuned == 1
    assert cfg.lanes_per_particle in (4, 8) and cfg.spmv_unroll in (2, 4)
    assert cfg.item_rows in (64, 128, 256, 512)
    assert cfg.work_items == sum((sc.n + cfg.item_rows - 1) // cfg.item_rows for sc in lst)
    b.advance(5)
    for k, sc in enumerate(lst):
        s = scenes.make_simulator(sc)
        s.makeReady()
        s.advance(5)
        assert same_sets(b.alive_sets(k), s.alive_sets())
        assert rel_err(b.get(k, pdgb.VAR_POSITION), s.get(pdgb.VAR_POSITION)) < MIXED_TOL


def test_batch_errors(pdgb, scenes):
    b = pdgb.Batch(0)
    with pytest.raises(pdgb.PdError) as e:
        b.advance(1)
    assert e.value.status == 3          # not ready
    with pytest.raises(pdgb.PdError):
        b.makeReady()                    # no scenes
    sc = scenes.impact_body(100, "block", precision=0)
    scenes.add_to_batch(b, sc)
    sc64 = scenes.impact_body(100, "block", precision=1)
    with pytest.raises(pdgb.PdError) as e:
        scenes.add_to_batch(b, sc64)     # mixed precisions in one batch
    assert e.value.status == 1
    with pytest.raises(pdgb.PdError):
        b.get(5, pdgb.VAR_POSITION)      # scene out of range
    sch = scenes.impact_body(100, "block", precision=0)
    sch.opt.warm_start = 2
    with pytest.raises(pdgb.PdError) as e:
        scenes.add_to_batch(b, sch)      # the history projection is per handle only
    assert e.value.status == 1


def test_batch_learned_warm_start(pdgb, scenes):
    """Batch option warm_start = 1: one network for all scenes, the guess
    guarded per scene.  The CG still runs to each scene's tolerance, so every
    scene matches the oracle (same time-step history, same broken bonds) and
    its own Simulator with the same network; graph replay and direct launches
    agree bitwise."""
    ws = __import__("importlib").import_module("sci-solver_peridynamic_gb300.warmstart")
    X, T = ws.collect(lambda seed: scenes.cube_lattice(n_side=10, seed=seed), seeds=(1,), steps=20,
                      samples_per_step=256)
    params, loss = ws.train(X, T, iterations=300, batch=1024, lr=1e-3)
    assert np.isfinite(loss)
    lst = _mix(pdgb, scenes, 0)
    b = _batch(pdgb, scenes, lst, warm_start=1)
    b.ws_set_params(params)
    assert b.config().warm_start == 1
    b2 = _batch(pdgb, scenes, lst, warm_start=1, use_graph=0, lanes_per_particle=b.config().lanes_per_particle,
                spmv_unroll=b.config().spmv_unroll, item_rows=b.config().item_rows)
    b2.ws_set_params(params)
    oras = [make_oracle(sc) for sc in lst]
    done = 0
    while done < 40:
        b.advance(10)
        b2.advance(10)
        for o in oras:
            o.advance(10)
        done += 10
        for k, o in enumerate(oras):
            assert b.stats(k).time_step_ticks == o.dt_ticks, f"scene {k}: time step differs at step {done}"
            assert same_sets(b.alive_sets(k), o.alive_sets()), f"scene {k}: broken bonds differ at step {done}"
    kept = 0
    for k, (sc, o) in enumerate(zip(lst, oras)):
        st = b.stats(k)
        assert st.cg_converged == 1 and st.current_step == 40
        x = b.get(k, pdgb.VAR_POSITION)
        assert rel_err(x, o.position) < MIXED_TOL, f"scene {k}"
        np.testing.assert_array_equal(x, b2.get(k, pdgb.VAR_POSITION))
        sc.opt.warm_start = 1
        s = scenes.make_simulator(sc)
        s.makeReady()
        s.ws_set_params(params)
        s.advance(40)
        sc.opt.warm_start = 0
        assert same_sets(b.alive_sets(k), s.alive_sets()), f"scene {k}"
        assert rel_err(x, s.get(pdgb.VAR_POSITION)) < MIXED_TOL, f"scene {k}"
        kept += st.ws_guesses_kept
    print(f"\nbatched learned warm start: guesses kept {kept} of {40 * len(lst)}, training loss {loss:.4g}")


def test_batch_warm_start_needs_mixed_precision(pdgb, scenes):
    o = pdgb.BatchOptions()
    pdgb.library().pd_batch_options_default(o)
    o.warm_start = 1
    b = pdgb.Batch(0, o)
    scenes.add_to_batch(b, scenes.impact_body(100, "block", precision=1))
    with pytest.raises(pdgb.PdError) as e:
        b.makeReady()
    assert e.value.status == 1
    o.warm_start = 2
    with pytest.raises(pdgb.PdError) as e:
        pdgb.Batch(0, o)
    assert e.value.status == 1


def test_batch_pauses_the_learned_pass_of_rejecting_scenes(pdgb, scenes):
    """A network whose guesses the guard rejects: after 3 rejections in a row
    a scene pauses its learned pass (retrying every 16 steps), and starts
    from the previous solution exactly as the batch without the network --
    positions bit for bit.  Over 40 solves an always-rejecting scene is
    paused in 35 (steps 4-15, 17-31, 33-40)."""
    n_par = pdgb.library().pd_mlp_param_count()
    params = np.random.default_rng(3).normal(0.0, 0.5, n_par).astype(np.float32)
    lst = [scenes.impact_body(300, "block", coeff=5.0, speed=5.0, seed=1, precision=0, steps=40),
           scenes.impact_body(400, "ball", coeff=6.0, speed=8.0, seed=2, precision=0, steps=40),
           scenes.cube_lattice(n_side=8, seed=1)]
    b = _batch(pdgb, scenes, lst, warm_start=1)
    b.ws_set_params(params)
    plain = _batch(pdgb, scenes, lst, warm_start=0, lanes_per_particle=b.config().lanes_per_particle,
                   spmv_unroll=b.config().spmv_unroll, item_rows=b.config().item_rows)
    b.advance(40)
    plain.advance(40)
    rejecting = 0
    for k in range(len(lst)):
        st = b.stats(k)
        assert st.current_step == 40 and st.cg_converged == 1
        if st.ws_guesses_kept == 0:
            rejecting += 1
            assert st.ws_guesses_skipped == 35, f"scene {k}"
            np.testing.assert_array_equal(b.get(k, pdgb.VAR_POSITION), plain.get(k, pdgb.VAR_POSITION))
            assert st.total_cg_iterations == plain.stats(k).total_cg_iterations
        else:
            assert st.ws_guesses_skipped < 35
    assert rejecting > 0, "the random network's guesses are rejected"
