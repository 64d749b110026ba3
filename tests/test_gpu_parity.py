"""Parity of the CUDA path (through the C ABI) against the CPU oracle.

Bond lists and broken-bond sets must match exactly; positions and
velocities within the stated tolerances:
  FP64 mode:  1e-9 relative (differences come only from summation order)
  mixed mode: 1e-5 relative after the full run (FP32 forces/SpMV)
"""
import numpy as np
import pytest

from helpers import apply_on_device, assert_positions, make_oracle, rel_err, same_sets

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
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, 1, "fp64 implicit Euler")
    assert rel_err(sim.get(pdgb.VAR_VELOCITY), ora.velocity) < 1e-7
    assert abs(sim.stats().last_cg_iterations - ora.cg_iters) <= 1


def test_step_fp64_newmark_breaking(pdgb, scenes):
    sc = scenes.reference_block(n_side=8, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=300.0)
    sc.opt.precision = pdgb.PRECISION_FP64
    sim, ora = _run_pair(pdgb, scenes, sc, 60)
    st = sim.stats()
    assert st.bonds_alive < st.bonds_initial, "scene should break bonds"
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, 1, "fp64 Newmark breaking")


def test_step_mixed_newmark_breaking(pdgb, scenes):
    sc = scenes.reference_block(n_side=8, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=300.0,
                                cg_tol=1e-9)
    sim, ora = _run_pair(pdgb, scenes, sc, 60)
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, 0, "mixed Newmark breaking")
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
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, 0, "cube 100 steps")
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
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, 1, f"tiny {n_side}")


@pytest.mark.parametrize("precision,tol", [(1, FP64_TOL), (0, MIXED_TOL)])
def test_newmark_dt_halving_and_doubling(pdgb, scenes, precision, tol):
    """Breaking stops mid-run: pd_time_step goes 128 -> 64 -> 128 -> 64 -> 128;
    the doubled step is used by the same step's assembly, solve and update."""
    sc = scenes.reference_block(n_side=7, seed=5, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=150.0,
                                cg_tol=1e-10)
    sc.opt.precision = precision
    sim, ora = _run_pair(pdgb, scenes, sc, 90, check_every=5)
    assert rel_err(sim.get(pdgb.VAR_POSITION), ora.position) < tol
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, precision, "dt halving/doubling")


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
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, 0, f"spmv path {path} breaking")


@pytest.mark.parametrize("path", [1, 2])
def test_spmv_paths_cube(pdgb, scenes, path):
    sc = scenes.cube_lattice(n_side=12, seed=2)
    sc.opt.spmv_path = path
    sim, ora = _run_pair(pdgb, scenes, sc, 40, check_every=20)
    assert sim.params()[2].spmv_path == path
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, 0, f"spmv path {path} cube")


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
        # automatic: the ball is a lattice fill, so the stencil product is a candidate too
        assert sim.params()[2].spmv_path in ((2, 3) if path == 0 else (path,))
        runs[path] = sim
    ora = make_oracle(sc)
    ora.advance(6)
    for path, sim in runs.items():
        assert same_sets(sim.alive_sets(), ora.alive_sets())
        assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, 0, f"24k ball path {path}")


@pytest.mark.parametrize("precision,tol", [(1, FP64_TOL), (0, MIXED_TOL)])
def test_pd_pd_contact(pdgb, scenes, precision, tol):
    """Two blocks collide: the PD-PD contact forces (collidePDParticles,
    off in the reference build) against the oracle's brute-force pairs."""
    sc = scenes.two_blocks(precision=precision)
    sim, ora = _run_pair(pdgb, scenes, sc, 80, check_every=20)
    # mixed: the contact force switches on at a distance threshold, so FP32
    # positions near it change when a pair starts to push (measured 6.3e-5
    # of the displacement, against 1.5e-13 in FP64)
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, precision, "pd-pd contact",
                     disp_tol=2e-4 if precision == 0 else None)
    assert rel_err(sim.get(pdgb.VAR_VELOCITY), ora.velocity) < max(tol, 1e-7) * 100
    # the contact changed the motion: without it the blocks pass into each other
    free = scenes.make_simulator(scenes.two_blocks(precision=precision, contact=False))
    free.makeReady()
    free.advance(80)
    x, xf = sim.get(pdgb.VAR_POSITION), free.get(pdgb.VAR_POSITION)
    n = x.shape[0] // 2
    assert x[:n, 0].max() < xf[:n, 0].max() - 0.2 * sc.info["spacing"]


@pytest.mark.parametrize("precision", [1, 0])
def test_small_block_closed_form(pdgb, scenes, precision):
    """Known answer through the C ABI, no oracle: a jittered 2 x 2 x 2 block
    in which every pair is a bond shorter than horizon - r (vscale 1).  After
    one step, the next force pass and the operator A = m I + t2 K equal the
    closed forms of calculatePDForceDerivative (cg_solver.cuh:200-339) at the
    positions read back: f_p = c sum_q (d/d0 - 1) e_pq, K_pq = -J_pq,
    K_pp = sum_q J_pq, J = (c/d0)[(1 - d0/d) I + (d0/d) e e^T], with e the
    bond vector over its float-rounded length."""
    sc = scenes.reference_block(n_side=2, jitter=0.05, s0=0.5, drop=0.0)
    sc.opt.precision = precision
    for k in range(3):
        sc.opt.gravity[k] = 0.0
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    sim.advance(1)
    x = sim.get(pdgb.VAR_POSITION)[:, :3]
    X = sim.get(pdgb.VAR_ORIGINAL_POSITION)[:, :3]
    sim.advance(1)
    F = sim.get(pdgb.VAR_FORCE)[:, :3]
    n = sc.n
    assert list(sim.get(pdgb.VAR_BOND_COUNT)) == [n - 1] * n
    v = sim.operator_view()
    c, m, t2 = v.bond_coeff, v.mass, v.t2
    horizon = sc.sim.pd_horizon
    f = np.zeros((n, 3))
    K = np.zeros((3 * n, 3 * n))
    smin = 1.0
    for p in range(n):
        for q in range(n):
            if q == p:
                continue
            dx = x[q] - x[p]
            d = np.sqrt(np.dot(dx, dx))
            e = dx / float(np.float32(d))
            d0 = np.sqrt(np.dot(X[p] - X[q], X[p] - X[q]))
            assert d0 <= horizon - sc.sim.pd_particle_radius
            s = d / d0 - 1.0
            smin = min(smin, abs(s))
            f[p] += c * s * e
            J = (c / d0) * ((1.0 - d0 / d) * np.eye(3) + (d0 / d) * np.outer(e, e))
            K[3 * p:3 * p + 3, 3 * p:3 * p + 3] += J
            K[3 * p:3 * p + 3, 3 * q:3 * q + 3] -= J
    assert smin > 1e-5   # the block is deformed: every bond carries a force
    rng = np.random.default_rng(2)
    w = np.zeros((n, 4))
    w[:, :3] = rng.standard_normal((n, 3))
    y, dot, ws = apply_on_device(pdgb, sim, w)
    ws = ws[:, :3]
    y_ref = m * ws + t2 * (K @ ws.reshape(-1)).reshape(n, 3)
    fscale = np.abs(f).max()
    if precision == pdgb.PRECISION_FP64:
        # s = d/d0 - 1 carries the rounding of d and d0 amplified by 1/s
        assert np.abs(F - f).max() <= 1e-14 / smin * fscale
        assert np.abs(y[:, :3] - y_ref).max() <= 1e-12 * np.abs(y_ref).max()
        assert abs(dot - float(np.sum(ws * y_ref))) <= 1e-12 * abs(dot)
    else:
        # FP32 positions: each stretch within ~1e-6 of its FP64 value
        assert np.abs(F - f).max() <= 1e-6 * (n - 1) * c
        assert np.abs(y[:, :3] - y_ref).max() <= 2e-5 * np.abs(y_ref).max()
        assert abs(dot - float(np.sum(ws * y_ref))) <= 2e-5 * abs(dot)


def test_particles_leaving_the_supercell_window(pdgb, scenes):
    """Two bonded blocks flying apart at 200 m/s leave the 1024-supercell
    window around the initial bounding box (supercell 2^-7 m here, so +-4 m)
    within ~20 steps.  Their cell indices clamp, the two-word positions lose
    their error bound, and the break test of their bonds falls back to the
    reference's FP64 expression: bond sets stay the oracle's."""
    # CG rel. 1e-6: the right-hand side is dominated by the uniform 200 m/s,
    # and FP32 CG vectors cannot resolve a residual far below 1e-7 of it
    sc = scenes.two_blocks(n_side=4, spacing=0.002, gap_spacings=3.0, speed=-200.0, dt=1e-3, cg_tol=1e-6,
                           contact=False, steps=40)
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    ora = make_oracle(sc)
    for _ in range(4):
        sim.advance(10)
        ora.advance(10)
        assert sim.CGConvergence()
        assert same_sets(sim.alive_sets(), ora.alive_sets())
    assert sim.get_current_step() == 40
    x, xo = sim.get(pdgb.VAR_POSITION)[:, :3], ora.position[:, :3]
    assert np.abs(xo[:, 0]).max() > 5.0          # beyond the window
    assert np.abs(x - xo).max() <= 1e-6 * np.abs(xo).max()
    assert sim.CGConvergence()
