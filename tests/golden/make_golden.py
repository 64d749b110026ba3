"""Generates the golden fixtures in tests/golden/ from the reference's own
kernels compiled on the host (oracle/_ref/libpdref.so, built by
oracle/build_ref.sh from the reference tree).  Run where the reference tree
is present:

    python tests/golden/make_golden.py [REFERENCE_ROOT]   (default: $PD_REFERENCE_ROOT)

Each fixture holds the resolved parameters, the seeded inputs and the
reference outputs (bond rows, s0, positions/velocities at selected steps,
CG iteration counts, dt ticks, broken-bond sets).  The scenes are jittered
8^3 blocks in the reference's units and physics (params.txt-style
parameters, gravity -y, C*V*PD_K stiffness, 2^-23 s time base).
"""
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

scenes = importlib.import_module("sci-solver_peridynamic_gb300.scenes")


def ref_from_scene(sc):
    s = sc.sim
    bmin = np.array([s.boundary_min_x, s.boundary_min_y, s.boundary_min_z])
    bmax = np.array([s.boundary_max_x, s.boundary_max_y, s.boundary_max_z])
    r = O.RefSim(sc.n, sc.run.integrator, sc.run.adaptive_integration, s.pd_horizon, s.pd_particle_radius,
                 s.pd_C_times_V, s.pd_particle_mass, bmin, bmax, np.float32(sc.run.pd_stretch_limit_s0),
                 cg_tol=sc.opt.cg_relative_tolerance, cg_max=sc.opt.cg_max_iterations)
    r.set_particles(sc.pos, sc.vel, sc.act)
    r.make_ready()
    return r, bmin, bmax


def csr(sets):
    rp = np.zeros(len(sets) + 1, np.int64)
    rp[1:] = np.cumsum([len(x) for x in sets])
    return rp, (np.concatenate(sets).astype(np.int32) if rp[-1] else np.zeros(0, np.int32))


def make(name, sc, steps, snap):
    r, bmin, bmax = ref_from_scene(sc)
    rp0, col0 = csr(r.alive_sets())
    out = {
        "n": sc.n, "integrator": sc.run.integrator, "adaptive": sc.run.adaptive_integration,
        "horizon": sc.sim.pd_horizon, "radius": sc.sim.pd_particle_radius, "c_times_v": sc.sim.pd_C_times_V,
        "mass": sc.sim.pd_particle_mass, "bmin": bmin, "bmax": bmax,
        "s0": np.float32(sc.run.pd_stretch_limit_s0), "cg_tol": sc.opt.cg_relative_tolerance,
        "pos_in": sc.pos, "vel_in": sc.vel, "ostretch": r.original_stretch, "bond_rp": rp0, "bond_col": col0,
    }
    iters, ticks, retries = [], [], []
    for k in range(1, steps + 1):
        retries.append(r.advance())
        iters.append(r.cg_iters)
        ticks.append(r.dt_ticks)
        if k == 1:
            out["force_step1"] = r.force
        if k in snap:
            out[f"pos_{k}"] = r.position
            out[f"vel_{k}"] = r.velocity
            rp, col = csr(r.alive_sets())
            out[f"alive_rp_{k}"] = rp
            out[f"alive_col_{k}"] = col
    out["cg_iters"] = np.array(iters, np.int32)
    out["ticks"] = np.array(ticks, np.int32)
    out["retries"] = np.array(retries, np.int32)
    out["snap"] = np.array(snap, np.int32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, sc.n, "bonds", len(col0), "final alive", out[f"alive_rp_{snap[-1]}"][-1], "ticks", sorted(set(ticks)))


if __name__ == "__main__":
    ref_root = sys.argv[1] if len(sys.argv) > 1 else O.reference_root()
    if O.build_ref(ref_root) is None:
        sys.exit("reference tree not found: pass its root or set PD_REFERENCE_ROOT")
    make("ref_block_ie", scenes.reference_block(n_side=8, seed=7), 40, [1, 10, 40])
    make("ref_block_nm", scenes.reference_block(n_side=8, seed=11, integrator=1, adaptive=1, expansion=300.0),
         60, [1, 30, 60])
    make("ref_block_ie_adaptive", scenes.reference_block(n_side=7, seed=3, integrator=0, adaptive=1,
                                                         expansion=2500.0), 40, [20, 40])
    # breaking stops, so the time step halves and later doubles again
    make("ref_block_nm_double", scenes.reference_block(n_side=7, seed=5, integrator=1, adaptive=1,
                                                       expansion=150.0), 90, [30, 50, 90])
