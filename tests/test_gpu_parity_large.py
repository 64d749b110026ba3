"""Parity at the benchmark's own scene family, at sizes where the oracle
still runs in seconds on the host cores.

* The 1M-particle ellipsoid impact (the bench's workload) built at 125,000
  particles -- the size of the CPU sample the reference arm once timed --
  with the time step scaled with the spacing (so dt * wave speed / spacing is
  the 1M workload's), in contact from the first step, mixed precision.  Both
  CG initial guesses run beside one oracle run (the oracle starts every solve
  from the previous solution, as the reference does): the bench's default
  history projection and the previous solution.
* The notched beam of the precision study at 50,000 particles (horizon 6r,
  three-point bending with a prescribed loading strip), FP64 and mixed, for
  50 steps: bonds break from step ~35 and the time step halves and doubles.
  (The impact breaks no bonds in its first 30 steps even at 80 m/s: its
  penalty contact is soft, so the 125k run checks unbroken sets.)

Every 5 steps: bond and broken-bond sets exact, time-step ticks equal.  At
the end: positions within 1e-5 of max |x| (mixed; 1e-9 FP64) and
displacements u = x - X within the stated bound of max |u_ref|.
"""
import math

import numpy as np
import pytest

from helpers import make_oracle, rel_disp_err, rel_err, same_sets

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5
FP64_TOL = 1e-9
# displacement bounds (of max |u_ref|): FP32 forces/products against the FP64
# oracle, CG stopped at rel. 1e-6 on both sides (measured on a GB300: 2.4e-6
# for the impact, 1.5e-7 for the beam in mixed precision, 1.1e-13 FP64)
MIXED_DISP_TOL = 2e-5
FP64_DISP_TOL = 5e-8


def _impact_125k(scenes, precision, warm_start):
    n = 125_000
    v = 4.0 / 3.0 * math.pi * 0.5 * 0.35 * 0.3
    dt = 5e-5 * (v / n) ** (1 / 3) / (v / 1e6) ** (1 / 3)
    sc = scenes.ellipsoid_impact(target_n=n, dt=dt, precision=precision, gap=0.0, steps=20)
    sc.opt.warm_start = warm_start
    return sc


def test_ellipsoid_impact_125k_matches_oracle(pdgb, scenes):
    steps = 20
    runs = {}
    for ws in (2, 0):
        sc = _impact_125k(scenes, pdgb.PRECISION_MIXED, ws)
        sim = scenes.make_simulator(sc)
        sim.makeReady()
        runs[ws] = sim
    ora = make_oracle(sc)
    assert sc.n > 120_000
    for sim in runs.values():
        assert same_sets(sim.alive_sets(), ora.alive_sets()), "initial bond lists differ"
    b0 = runs[0].stats().bonds_initial
    done = 0
    while done < steps:
        for sim in runs.values():
            sim.advance(5)
        ora.advance(5)
        done += 5
        for ws, sim in runs.items():
            assert sim.stats().time_step_ticks == ora.dt_ticks, (ws, done)
            assert same_sets(sim.alive_sets(), ora.alive_sets()), f"guess {ws}: broken bonds differ at step {done}"
    xo = ora.position
    for ws, sim in runs.items():
        x = sim.get(pdgb.VAR_POSITION)
        e_x, e_u = rel_err(x, xo), rel_disp_err(x, xo, sc.pos)
        print(f"125k impact, guess {ws}: position {e_x:.3e}, displacement {e_u:.3e}, "
              f"bonds alive {sim.stats().bonds_alive}/{b0}")
        assert e_x < MIXED_TOL, ws
        assert e_u < MIXED_DISP_TOL, ws
        assert sim.CGConvergence()
    assert runs[2].stats().ws_guesses_kept > 0


@pytest.mark.parametrize("precision", [1, 0])
def test_notched_beam_50k_matches_oracle(pdgb, scenes, precision):
    """Bonds start to break near the notch at step ~35 (the oracle: 26 broken
    by step 35, 62 by step 50), with the adaptive time step halving and
    doubling."""
    steps = 50
    sc = scenes.notched_beam(target_n=50_000, precision=precision, steps=steps)
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    ora = make_oracle(sc)
    assert same_sets(sim.alive_sets(), ora.alive_sets())
    done = 0
    while done < steps:
        sim.advance(5)
        ora.advance(5)
        done += 5
        assert sim.stats().time_step_ticks == ora.dt_ticks
        assert same_sets(sim.alive_sets(), ora.alive_sets()), f"broken bonds differ at step {done}"
    x, xo = sim.get(pdgb.VAR_POSITION), ora.position
    e_x, e_u = rel_err(x, xo), rel_disp_err(x, xo, sc.pos)
    st = sim.stats()
    print(f"50k beam, precision {precision}: position {e_x:.3e}, displacement {e_u:.3e}, "
          f"bonds alive {st.bonds_alive}/{st.bonds_initial}")
    assert st.bonds_alive < st.bonds_initial, "the beam should break bonds by step 50"
    if precision == pdgb.PRECISION_FP64:
        assert e_x < FP64_TOL and e_u < FP64_DISP_TOL
    else:
        assert e_x < MIXED_TOL and e_u < MIXED_DISP_TOL
    assert sim.CGConvergence()
