"""The lattice-stencil product (spmv_path 3): bodies filled on a simple-cubic
lattice are renumbered brick by brick and multiplied from a shared-memory
halo with a per-(row, stencil entry) 1/d0 table.  It must give the gather
product's operator (to FP32 summation order), the oracle's bond sets and
positions through breaking and adaptive rollbacks (the table follows the live
bonds), fall back to the gather product for bodies that are not a lattice
fill, and continue a checkpoint bit for bit."""
import numpy as np
import pytest

from helpers import apply_on_device, assert_positions, make_oracle, rel_err, same_sets

pytestmark = pytest.mark.gpu


def _run_pair(scenes, sc, steps, check_every=5):
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    ora = make_oracle(sc)
    assert same_sets(sim.alive_sets(), ora.alive_sets())
    done = 0
    while done < steps:
        k = min(check_every, steps - done)
        sim.advance(k)
        ora.advance(k)
        done += k
        assert same_sets(sim.alive_sets(), ora.alive_sets()), f"broken-bond sets differ at step {done}"
        assert sim.stats().time_step_ticks == ora.dt_ticks
    return sim, ora


def test_lattice_breaking_and_rollbacks_match_oracle(pdgb, scenes):
    """Reference units, Newmark with bond breaking: the time step halves and
    doubles (rollbacks restore broken bonds), jitter 0.1 spacing."""
    sc = scenes.reference_block(n_side=9, seed=5, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=150.0,
                                cg_tol=1e-10)
    sc.opt.spmv_path = 3
    sim, ora = _run_pair(scenes, sc, 90)
    assert sim.params()[2].spmv_path == 3, "the block is a lattice fill"
    st = sim.stats()
    assert st.bonds_alive < st.bonds_initial
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, 0, "lattice breaking")


@pytest.mark.parametrize("coeff", [4.0, 5.0, 6.0])
def test_lattice_cube_matches_oracle(pdgb, scenes, coeff):
    """Horizons of 2, 2.5 and 3 spacings (stencil reach 2 and 3 sites)."""
    sc = scenes.cube_lattice(n_side=12, seed=4, coeff=coeff)
    sc.opt.spmv_path = 3
    sim, ora = _run_pair(scenes, sc, 40, check_every=20)
    assert sim.params()[2].spmv_path == 3
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, 0, f"lattice cube coeff {coeff}")


def test_lattice_impact_with_history_guess(pdgb, scenes):
    """The benchmark's scene family (ellipsoid, sphere contact rows, history
    projection) at 30k particles: the automatic choice times the stencil
    against the gather shapes; both paths give the oracle's run."""
    runs = {}
    for path in (3, 2):
        sc = scenes.ellipsoid_impact(target_n=30_000, gap=0.0, dt=5e-5 * (1e6 / 30_000) ** (1 / 3), steps=15)
        sc.opt.spmv_path = path
        sc.opt.warm_start = 2
        sim = scenes.make_simulator(sc)
        sim.makeReady()
        sim.advance(15)
        assert sim.params()[2].spmv_path == path
        runs[path] = sim
    ora = make_oracle(sc)
    ora.advance(15)
    for path, sim in runs.items():
        assert same_sets(sim.alive_sets(), ora.alive_sets())
        assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, 0, f"30k impact path {path}")
    sc = scenes.ellipsoid_impact(target_n=30_000, gap=0.0)
    auto = scenes.make_simulator(sc)
    auto.makeReady()
    assert auto.params()[2].spmv_path in (2, 3)


@pytest.mark.parametrize("precision_tol", [2e-6])
def test_lattice_operator_equals_gather_operator(pdgb, scenes, precision_tol):
    """After 33 steps with broken bonds: y = A x of the stencil product equals
    the gather product's (the same per-bond arithmetic, another summation
    order) and the oracle's assembled matrix."""
    ys = {}
    for path in (3, 2):
        sc = scenes.reference_block(n_side=8, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=300.0,
                                    cg_tol=1e-10)
        sc.opt.spmv_path = path
        sim = scenes.make_simulator(sc)
        sim.makeReady()
        sim.advance(33)
        assert sim.params()[2].spmv_path == path
        rng = np.random.default_rng(5)
        x = np.zeros((sc.n, 4))
        x[:, :3] = rng.standard_normal((sc.n, 3))
        ys[path] = apply_on_device(pdgb, sim, x)
    (y3, d3, x3), (y2, d2, x2) = ys[3], ys[2]
    assert np.array_equal(x3, x2)
    scale = np.abs(y2[:, :3]).max()
    assert np.abs(y3[:, :3] - y2[:, :3]).max() <= precision_tol * scale
    assert abs(d3 - d2) <= precision_tol * abs(d2)
    ora = make_oracle(sc)
    ora.advance(33)
    y_ref = ora.apply_A(x3)
    assert np.abs(y3[:, :3] - y_ref[:, :3]).max() <= 2e-5 * np.abs(y_ref[:, :3]).max()


@pytest.mark.parametrize("kind", ["jitter", "doubled"])
def test_not_a_lattice_falls_back(pdgb, scenes, kind):
    """Particles more than 0.3 spacings from every site, or two particles on
    one site: the body keeps the gather product (and the oracle's results)."""
    sc = scenes.cube_lattice(n_side=8, seed=1, jitter=0.05)
    if kind == "jitter":
        sc.pos[::7, 0] += 0.4 * sc.info["spacing"]
    else:
        extra = sc.pos[: sc.n // 4].copy()
        extra[:, :3] += 0.15 * sc.info["spacing"]
        sc.pos = np.vstack([sc.pos, extra])
        sc.vel = np.vstack([sc.vel, sc.vel[: extra.shape[0]]])
        sc.act = np.concatenate([sc.act, sc.act[: extra.shape[0]]])
        sc.sim.num_pd_particle = sc.pos.shape[0]
    sc.opt.spmv_path = 3
    sim, ora = _run_pair(scenes, sc, 10)
    assert sim.params()[2].spmv_path == 2
    assert_positions(sim.get(pdgb.VAR_POSITION), ora.position, sc.pos, 0, f"fallback {kind}")


def test_lattice_checkpoint_restart_bitwise(pdgb, scenes, tmp_path):
    sc = scenes.reference_block(n_side=8, seed=11, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=300.0,
                                cg_tol=1e-10)
    sc.opt.spmv_path = 3
    sc.run.saving_path = str(tmp_path).encode()
    a = scenes.make_simulator(sc)
    a.makeReady()
    a.advance(20)
    a.dataIO_saveState(20)
    a.advance(20)
    b = scenes.make_simulator(sc)
    b.makeReady()
    assert b.params()[2].spmv_path == 3
    b.dataIO_loadState(20)
    b.advance(20)
    assert np.array_equal(a.get(pdgb.VAR_POSITION), b.get(pdgb.VAR_POSITION))
    assert same_sets(a.alive_sets(), b.alive_sets())


def test_lattice_operator_after_a_translation_of_several_supercells(pdgb, scenes):
    """A free lattice block flying at 60 m/s per axis for 40 steps moves 0.24
    m per axis, about four supercells: every particle's deviation from its
    site wraps (d + sup n with n != 0), and the stencil product must still
    equal the gather product (whose supercell words wrap the same way) and
    the oracle's assembled matrix; the run keeps the oracle's positions."""
    ys = {}
    for path in (3, 2):
        sc = scenes.impact_body(1728, "block", coeff=5.0, speed=0.0, seed=3, steps=40)
        sc.act[:] = pdgb.ACTIVE
        sc.vel[:, :3] = 60.0
        sc.opt.gravity[:] = (0.0, 0.0, 0.0)
        sc.opt.spmv_path = path
        sim = scenes.make_simulator(sc)
        sim.makeReady()
        sim.advance(40)
        assert sim.params()[2].spmv_path == path
        x = sim.get(pdgb.VAR_POSITION)[:, :3]
        assert np.all(x - sc.pos[:, :3] > 0.2), "the body moved by several supercells"
        rng = np.random.default_rng(7)
        v = np.zeros((sc.n, 4))
        v[:, :3] = rng.standard_normal((sc.n, 3))
        ys[path] = apply_on_device(pdgb, sim, v) + (sim,)
    (y3, d3, x3, s3), (y2, d2, x2, _) = ys[3], ys[2]
    scale = np.abs(y2[:, :3]).max()
    assert np.abs(y3[:, :3] - y2[:, :3]).max() <= 2e-6 * scale
    ora = make_oracle(sc)
    ora.advance(40)
    y_ref = ora.apply_A(x3)
    assert np.abs(y3[:, :3] - y_ref[:, :3]).max() <= 2e-5 * np.abs(y_ref[:, :3]).max()
    assert same_sets(s3.alive_sets(), ora.alive_sets())
    assert_positions(s3.get(pdgb.VAR_POSITION), ora.position, sc.pos, 0, "lattice block after translation")
