"""The oracle (pd_oracle.c) against golden vectors produced by the reference's
own kernels compiled on the host (tests/golden/make_golden.py).  The
restatement keeps the reference's operation order and must reproduce the
reference bit for bit: bond rows, s0_i, forces, positions, velocities, CG
iteration counts, dt ticks and broken-bond sets."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "ref_block_*.npz")))


def oracle_from_fixture(d):
    p = O.default_params()
    p.n = int(d["n"])
    p.integrator = int(d["integrator"])
    p.adaptive = int(d["adaptive"])
    p.horizon = float(d["horizon"])
    p.radius = float(d["radius"])
    p.bond_coeff = float(d["c_times_v"]) * (5.0 * 2.94315e9)
    p.mass = float(d["mass"])
    for k in range(3):
        p.box_min[k] = float(d["bmin"][k])
        p.box_max[k] = float(d["bmax"][k])
    p.s0 = float(np.float32(d["s0"]))
    p.cg_rel_tol = float(d["cg_tol"])
    o = O.OracleSim(p)
    o.set_particles(d["pos_in"], d["vel_in"])
    o.make_ready()
    return o


def csr_sets(rp, col):
    return [col[rp[i]:rp[i + 1]] for i in range(len(rp) - 1)]


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_matches_reference_kernels(path):
    d = np.load(path)
    o = oracle_from_fixture(d)
    np.testing.assert_array_equal(o.original_stretch, d["ostretch"])
    sets0 = csr_sets(d["bond_rp"], d["bond_col"])
    assert all(np.array_equal(a, b) for a, b in zip(o.alive_sets(), sets0))
    snap = set(int(k) for k in d["snap"])
    steps = len(d["cg_iters"])
    for k in range(1, steps + 1):
        o.advance()
        assert o.cg_iters == d["cg_iters"][k - 1], f"step {k}"
        assert o.dt_ticks == d["ticks"][k - 1], f"step {k}"
        assert o.retries == d["retries"][k - 1], f"step {k}"
        if k == 1:
            np.testing.assert_array_equal(o.force, d["force_step1"])
        if k in snap:
            np.testing.assert_array_equal(o.position, d[f"pos_{k}"])
            np.testing.assert_array_equal(o.velocity, d[f"vel_{k}"])
            sets = csr_sets(d[f"alive_rp_{k}"], d[f"alive_col_{k}"])
            assert all(np.array_equal(a, b) for a, b in zip(o.alive_sets(), sets)), f"step {k}"


def test_fixtures_present():
    names = {os.path.basename(p) for p in GOLDEN}
    assert {"ref_block_ie.npz", "ref_block_nm.npz", "ref_block_nm_double.npz"} <= names


@pytest.mark.skipif(not os.path.exists(O.REF_SO), reason="host build of the reference kernels absent")
def test_oracle_matches_reference_kernels_live():
    """Fresh scenes against the host-compiled reference (this container only)."""
    import importlib
    scenes = importlib.import_module("sci-solver_peridynamic_gb300.scenes")
    from helpers import make_oracle
    for seed, integ, exp_ in ((21, 0, 300.0), (22, 1, 250.0)):
        sc = scenes.reference_block(n_side=6, seed=seed, integrator=integ, adaptive=1, expansion=exp_)
        s = sc.sim
        r = O.RefSim(sc.n, integ, 1, s.pd_horizon, s.pd_particle_radius, s.pd_C_times_V, s.pd_particle_mass,
                     [s.boundary_min_x, s.boundary_min_y, s.boundary_min_z],
                     [s.boundary_max_x, s.boundary_max_y, s.boundary_max_z],
                     np.float32(sc.run.pd_stretch_limit_s0), cg_tol=sc.opt.cg_relative_tolerance)
        r.set_particles(sc.pos, sc.vel)
        r.make_ready()
        o = make_oracle(sc)
        for _ in range(30):
            r.advance()
            o.advance()
        np.testing.assert_array_equal(o.position, r.position)
        np.testing.assert_array_equal(o.velocity, r.velocity)
