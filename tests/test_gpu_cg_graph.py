"""The CG loop as a CUDA graph (cg_loop 0, the default): a while node repeats
cg_check_interval iterations until the device-side convergence test stops it,
so a solve needs one host read-back.  It runs the kernels of the host-checked
loop (cg_loop 1) in the same order, so both give identical results, iteration
counts and broken-bond sets; the oracle pins the graph runs through every
other parity test (the graph is the default).  The reference's solve is the
CUSP cg of Simulator::solveLinearSystem (src/core/simulator.cu:735-799)."""
import numpy as np
import pytest

from helpers import assert_positions, make_oracle, same_sets

pytestmark = pytest.mark.gpu


def _run(scenes, sc, loop, steps, interval=0):
    sc.opt.cg_loop = loop
    sc.opt.cg_check_interval = interval
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    iters, retries = [], 0
    for _ in range(steps):
        sim.advance(1)
        st = sim.stats()
        iters.append(st.last_cg_iterations)
        retries += st.retries_last_step
    sim.rollbacks = retries
    return sim, iters


def _same_run(pdgb, a, b, ia, ib, what):
    assert ia == ib, f"{what}: CG iterations differ"
    assert same_sets(a.alive_sets(), b.alive_sets()), what
    assert a.stats().time_step_ticks == b.stats().time_step_ticks, what
    np.testing.assert_array_equal(a.get(pdgb.VAR_POSITION), b.get(pdgb.VAR_POSITION), err_msg=what)
    np.testing.assert_array_equal(a.get(pdgb.VAR_VELOCITY), b.get(pdgb.VAR_VELOCITY), err_msg=what)


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_loop_equals_host_loop_breaking_newmark(pdgb, scenes, precision):
    """Newmark with bond breaking and rollbacks (the time step halves and
    doubles): bitwise the host loop's run; one read-back per solve plus the
    adaptive scheme's test per integrate call."""
    runs = {}
    for loop in (0, 1):
        sc = scenes.reference_block(n_side=9, seed=5, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=150.0,
                                    cg_tol=1e-10)
        sc.opt.precision = precision
        runs[loop] = _run(scenes, sc, loop, 70)
    (g, ig), (h, ih) = runs[0], runs[1]
    _same_run(pdgb, g, h, ig, ih, f"precision {precision}")
    sg, sh = g.stats(), h.stats()
    assert sg.bonds_alive < sg.bonds_initial
    assert g.rollbacks > 0, "the run rolls back (the time step halves)"
    assert sg.cg_graph_solves == 70 and sh.cg_graph_solves == 0
    # per integrate call the adaptive test; per kept step the solve's read-back
    assert sg.host_syncs == (70 + g.rollbacks) + 70
    assert sh.host_syncs > sg.host_syncs


def test_graph_loop_sync_count_per_step(pdgb, scenes):
    """Implicit Euler without adaptivity: exactly one host wait per step."""
    sc = scenes.cube_lattice(n_side=10, seed=2)
    g, _ = _run(scenes, sc, 0, 20)
    st = g.stats()
    assert st.cg_graph_solves == 20
    assert st.host_syncs == 20


@pytest.mark.parametrize("interval", [2, 4, 6, 16])
def test_graph_body_lengths_and_lattice_direction_buffers(pdgb, scenes, interval):
    """The lattice product alternates two direction buffers by iteration
    parity; bodies of 2..16 iterations (and the history projection's device
    solve) give the host loop's run bit for bit, and the oracle's."""
    runs = {}
    for loop in (0, 1):
        sc = scenes.ellipsoid_impact(target_n=30_000, gap=0.0, dt=5e-5 * (1e6 / 30_000) ** (1 / 3), steps=10)
        sc.opt.spmv_path = 3
        sc.opt.warm_start = 2
        runs[loop] = _run(scenes, sc, loop, 10, interval)
    (g, ig), (h, ih) = runs[0], runs[1]
    assert g.params()[2].spmv_path == 3
    _same_run(pdgb, g, h, ig, ih, f"body {interval}")
    assert g.stats().cg_graph_solves == 10
    assert g.stats().ws_guesses_kept == h.stats().ws_guesses_kept > 0
    if interval == 4:
        ora = make_oracle(sc)
        ora.advance(10)
        assert same_sets(g.alive_sets(), ora.alive_sets())
        assert_positions(g.get(pdgb.VAR_POSITION), ora.position, sc.pos, 0, "graph loop, 30k impact")


@pytest.mark.parametrize("loop", [0, 1])
def test_iteration_limit_ends_the_graph(pdgb, scenes, loop):
    """A solve stopped by cg_max_iterations: the while node ends on the
    device's limit test, the solve reports no convergence and the handle
    stops advancing, as with the host loop."""
    sc = scenes.cube_lattice(n_side=8, seed=1)
    sc.opt.cg_max_iterations = 5
    sc.opt.cg_loop = loop
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    sim.advance(3)
    st = sim.stats()
    assert st.last_cg_iterations == 5
    assert st.cg_converged == 0
    assert st.current_step == 1
    assert st.cg_graph_solves == (1 if loop == 0 else 0)
