"""Seeded synthetic scenes for the PD step (the role of the reference's Scene,
src/examples/scene.cpp: lattice points -> host position/velocity/activity
arrays -> Simulator).

``reference_block``   a jittered lattice block in the reference's own units
                      and physics (params.txt keys, gravity -y, C*V*PD_K
                      stiffness, 2^-23 s time base, box reflection).
``cube_lattice``      16^3 lattice, SI units, clamped bottom layer, top layer
                      moving at -5 m/s (small plain-method workload).
``ellipsoid_impact``  ~1M particles in an ellipsoid struck by a rigid sphere,
                      Newmark-beta, mixed precision (large plain-method workload).
``notched_beam``      notched beam in three-point bending (precision study).
``impact_body``       a jittered block (clamped base, top layer moving down)
                      or ball (struck by a rigid sphere) of a given size.
``batched_scenes``    many impact bodies of log-uniform sizes (batched stepping).

SI-unit material: density 125 kg/m^3 (1e-3 kg per particle at 0.02 m
spacing) and bond stiffness c = 1e6 * (spacing / 0.02)^2, the scaling under
which a bond-based PD solid keeps its wave speed as the lattice is refined.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import (ACTIVE, CLAMPED, IMPLICIT_EULER, NEWMARK_BETA, PRECISION_MIXED, PRESCRIBED, RunningParameters,
               SimulationParameters, SolverOptions, SystemParameter, default_options)
from . import lattice as _lat
from .lattice import si_mass, si_stiffness  # noqa: F401  (re-exported)


@dataclasses.dataclass
class Scene:
    name: str
    sim: SimulationParameters
    run: RunningParameters
    opt: SolverOptions
    pos: np.ndarray      # (n, 4) float64
    vel: np.ndarray      # (n, 4) float64
    act: np.ndarray      # (n,) int32
    steps: int
    info: dict

    @property
    def n(self):
        return int(self.pos.shape[0])


_lattice = _lat.lattice


def _si_params(n, spacing, coeff, mass, s0, integrator, final_step):
    sp = SystemParameter()
    sim = sp.getSimulationParameters()
    run = sp.getRunningParameters()
    sim.num_pd_particle = n
    sim.pd_particle_radius = spacing / 2.0
    sim.pd_kernel_coeff = coeff
    sim.pd_horizon = coeff * spacing / 2.0
    sim.pd_particle_mass = mass
    sim.pd_time_step = 128
    sim.scaleFactor = 1.0
    sim.boundary_min_x = sim.boundary_min_y = sim.boundary_min_z = -1e30
    sim.boundary_max_x = sim.boundary_max_y = sim.boundary_max_z = 1e30
    run.integrator = integrator
    run.adaptive_integration = 0
    run.pd_stretch_limit_s0 = s0
    run.final_step = final_step
    return sim, run


def reference_block(n_side=8, seed=7, integrator=IMPLICIT_EULER, adaptive=0, expansion=300.0, drop=-0.05,
                    pd_kernel_coeff=5.001, s0=1e-3, jitter=0.1, cg_tol=1e-12):
    """A jittered n_side^3 block in the reference's units and physics.

    Parameters follow src/examples/params.txt (radius_pd_over_sph 1, box
    2 x 2 x 4, sph_kernel_coeff 4.001, pd_particle_mass 1000) through
    calculateDependentParameters; the block sits near the floor, with an
    x-expansion velocity field (breaks bonds under Newmark) and a small
    downward velocity.
    """
    sp = SystemParameter()
    sim, run = sp.getSimulationParameters(), sp.getRunningParameters()
    sim.pd_particle_radius = 1.0             # radius_pd_over_sph
    sim.boundary_min_x = sim.boundary_min_y = sim.boundary_min_z = 0.0
    sim.boundary_max_x, sim.boundary_max_y, sim.boundary_max_z = 2.0, 2.0, 4.0
    sim.sph_kernel_coeff = 4.001
    sim.pd_kernel_coeff = pd_kernel_coeff
    sim.pd_particle_mass = 1000.0
    run.pd_stretch_limit_s0 = s0
    run.integrator = integrator
    run.adaptive_integration = adaptive
    sp.derive()
    spacing = 2 * sim.pd_particle_radius
    rng = np.random.default_rng(seed)
    g = _lattice(n_side, n_side, n_side).astype(np.float64)
    n = g.shape[0]
    pos = np.zeros((n, 4))
    pos[:, :3] = 0.004 + g * spacing + rng.uniform(-jitter, jitter, (n, 3)) * spacing
    vel = np.zeros((n, 4))
    c = pos[:, :3].mean(0)
    vel[:, 0] = expansion * (pos[:, 0] - c[0])
    vel[:, 1] = drop
    sim.num_pd_particle = n
    opt = default_options()
    opt.cg_relative_tolerance = cg_tol
    return Scene("reference_block", sim, run, opt, pos, vel, np.zeros(n, np.int32), 40,
                 {"spacing": spacing, "seed": seed})


def cube_lattice(n_side=16, spacing=0.02, seed=0, jitter=0.05, coeff=5.0, s0=0.02, dt=1e-4, cg_tol=1e-6,
                 precision=PRECISION_MIXED, steps=100, top_velocity=-5.0):
    """16^3 simple-cubic lattice, spacing 0.02 m, jitter +-0.05 spacing,
    horizon 5r, m = 1e-3 kg, c = 1e6, s0 = 0.02, bottom layer clamped, top
    layer initial v_z = -5 m/s, gravity -9.81 z, implicit Euler dt = 1e-4,
    CG rel. tol 1e-6."""
    rng = np.random.default_rng(seed)
    g = _lattice(n_side, n_side, n_side)
    n = g.shape[0]
    pos = np.zeros((n, 4))
    pos[:, :3] = g * spacing + rng.uniform(-jitter, jitter, (n, 3)) * spacing
    vel = np.zeros((n, 4))
    act = np.full(n, ACTIVE, np.int32)
    act[g[:, 2] == 0] = CLAMPED
    vel[g[:, 2] == n_side - 1, 2] = top_velocity
    sim, run = _si_params(n, spacing, coeff, si_mass(spacing), s0, IMPLICIT_EULER, steps)
    opt = default_options()
    opt.precision = precision
    opt.cg_relative_tolerance = cg_tol
    opt.cg_max_iterations = 20000
    opt.time_step_base = dt / 128.0
    opt.bond_stiffness = si_stiffness(spacing)
    opt.gravity[:] = (0.0, 0.0, -9.81)
    opt.box_enabled = 0
    return Scene("cube_lattice", sim, run, opt, pos, vel, act, steps,
                 {"spacing": spacing, "seed": seed, "n_side": n_side})


def ellipsoid_impact(target_n=1_000_000, semi_axes=(0.5, 0.35, 0.3), seed=0, jitter=0.05, coeff=5.0, s0=0.015,
                     dt=5e-5, cg_tol=1e-6, precision=PRECISION_MIXED, steps=200, sphere_radius=0.1,
                     sphere_speed=10.0, spacing=None, gap=1.0):
    """Jittered lattice filling an ellipsoid, struck along -x by a rigid
    sphere (penalty contact), Newmark-beta dt = 5e-5, CG rel. tol 1e-6.
    The spacing is chosen so the particle count is ~target_n.  The sphere
    starts `gap` spacings beyond the outermost particle (gap <= 0: in
    contact from the first step).  Arrays and constants come from
    lattice.ellipsoid_impact."""
    b = _lat.ellipsoid_impact(target_n=target_n, semi_axes=semi_axes, seed=seed, jitter=jitter, coeff=coeff, s0=s0,
                              dt=dt, cg_tol=cg_tol, sphere_radius=sphere_radius, sphere_speed=sphere_speed,
                              spacing=spacing, gap=gap)
    spacing = b["spacing"]
    n = b["pos"].shape[0]
    sim, run = _si_params(n, spacing, coeff, b["mass"], s0, NEWMARK_BETA, steps)
    opt = default_options()
    opt.precision = precision
    opt.cg_relative_tolerance = b["cg_tol"]
    opt.cg_max_iterations = b["cg_max_iterations"]
    opt.time_step_base = b["dt"] / 128.0
    opt.bond_stiffness = b["stiffness"]
    opt.gravity[:] = b["gravity"]
    opt.box_enabled = 0
    opt.sphere_enabled = 1
    opt.sphere_radius = b["sphere_radius"]
    opt.sphere_center[:] = b["sphere_center"]
    opt.sphere_velocity[:] = b["sphere_velocity"]
    opt.sphere_stiffness = b["sphere_stiffness"]
    return Scene("ellipsoid_impact", sim, run, opt, b["pos"], b["vel"], b["act"], steps,
                 {"spacing": spacing, "seed": seed, "semi_axes": semi_axes})


def notched_beam(target_n=2_000_000, dims=(1.0, 0.2, 0.2), notch_depth=0.05, seed=0, jitter=0.05, coeff=6.0,
                 s0=0.01, dt=5e-5, cg_tol=1e-6, precision=PRECISION_MIXED, steps=500, load_speed=1.0,
                 spacing=None):
    """Beam along x with a notch at midspan from the bottom face; supports
    (clamped) under both ends, the loading strip on top at midspan moves
    down at load_speed (prescribed)."""
    L, W, H = dims
    if spacing is None:
        spacing = (L * W * H / target_n) ** (1.0 / 3.0)
    nx, ny, nz = (int(round(s / spacing)) for s in dims)
    g = _lattice(nx, ny, nz)
    p0 = (g + 0.5) * spacing
    notch = (np.abs(p0[:, 0] - L / 2) < spacing) & (p0[:, 2] < notch_depth)
    p0 = p0[~notch]
    n = p0.shape[0]
    rng = np.random.default_rng(seed)
    pos = np.zeros((n, 4))
    pos[:, :3] = p0 + rng.uniform(-jitter, jitter, (n, 3)) * spacing
    vel = np.zeros((n, 4))
    act = np.full(n, ACTIVE, np.int32)
    bottom = p0[:, 2] < 2 * spacing
    act[bottom & ((p0[:, 0] < 0.05 * L) | (p0[:, 0] > 0.95 * L))] = CLAMPED
    top = p0[:, 2] > H - 2 * spacing
    load = top & (np.abs(p0[:, 0] - L / 2) < 0.02 * L)
    act[load] = PRESCRIBED
    vel[load, 2] = -load_speed
    sim, run = _si_params(n, spacing, coeff, si_mass(spacing), s0, NEWMARK_BETA, steps)
    opt = default_options()
    opt.precision = precision
    opt.cg_relative_tolerance = cg_tol
    opt.cg_max_iterations = 20000
    opt.time_step_base = dt / 128.0
    opt.bond_stiffness = si_stiffness(spacing)
    opt.gravity[:] = (0.0, 0.0, -9.81)
    opt.box_enabled = 0
    return Scene("notched_beam", sim, run, opt, pos, vel, act, steps, {"spacing": spacing, "seed": seed})


def impact_body(n_target=8000, shape="block", coeff=5.0, speed=5.0, seed=0, spacing=0.02, jitter=0.05, s0=0.02,
                cg_tol=1e-6, precision=PRECISION_MIXED, steps=100):
    """A body of about n_target particles on a jittered simple-cubic lattice.

    shape "block": nx x ny x nz lattice, bottom layer clamped, top layer
    moving down at `speed`, implicit Euler dt = 1e-4 (the small plain-method
    set-up at another size).  shape "ball": lattice points inside a sphere,
    struck along -x by a rigid sphere (radius half the ball's, penalty
    contact, in contact from the first step) moving at `speed`,
    Newmark-beta dt = 5e-5.  Horizon coeff * spacing / 2, gravity -9.81 z."""
    rng = np.random.default_rng(seed)
    if shape == "block":
        side = max(2, int(round(n_target ** (1.0 / 3.0))))
        nz = max(2, int(round(n_target / (side * side))))
        g = _lattice(side, side, nz)
        p0 = g * spacing
        integrator, dt = IMPLICIT_EULER, 1e-4
    elif shape == "ball":
        R = (3.0 * n_target / (4.0 * math.pi)) ** (1.0 / 3.0)
        m = int(math.ceil(R)) + 1
        g = _lattice(2 * m + 1, 2 * m + 1, 2 * m + 1) - m
        g = g[(g.astype(np.float64) ** 2).sum(1) <= R * R]
        p0 = g * spacing
        integrator, dt = NEWMARK_BETA, 5e-5
    else:
        raise ValueError("shape must be 'block' or 'ball'")
    n = p0.shape[0]
    pos = np.zeros((n, 4))
    pos[:, :3] = p0 + rng.uniform(-jitter, jitter, (n, 3)) * spacing
    vel = np.zeros((n, 4))
    act = np.full(n, ACTIVE, np.int32)
    cstiff = si_stiffness(spacing)
    sim, run = _si_params(n, spacing, coeff, si_mass(spacing), s0, integrator, steps)
    opt = default_options()
    opt.precision = precision
    opt.cg_relative_tolerance = cg_tol
    opt.cg_max_iterations = 20000
    opt.time_step_base = dt / 128.0
    opt.bond_stiffness = cstiff
    opt.gravity[:] = (0.0, 0.0, -9.81)
    opt.box_enabled = 0
    if shape == "block":
        act[g[:, 2] == 0] = CLAMPED
        vel[g[:, 2] == g[:, 2].max(), 2] = -speed
    else:
        r_imp = 0.5 * R * spacing
        opt.sphere_enabled = 1
        opt.sphere_radius = r_imp
        opt.sphere_center[:] = (pos[:, 0].max() + r_imp, 0.0, 0.0)
        opt.sphere_velocity[:] = (-speed, 0.0, 0.0)
        opt.sphere_stiffness = cstiff / spacing
    return Scene("impact_body", sim, run, opt, pos, vel, act, steps,
                 {"spacing": spacing, "seed": seed, "shape": shape, "coeff": coeff, "speed": speed})


def two_blocks(n_side=6, spacing=0.02, gap_spacings=3.0, speed=5.0, seed=0, jitter=0.05, coeff=5.0, s0=0.02,
               dt=1e-4, cg_tol=1e-8, precision=PRECISION_MIXED, steps=80, contact=True):
    """Two jittered n_side^3 blocks moving toward each other along x at
    +-speed, gap_spacings lattice spacings apart (beyond the horizon, so no
    bond joins them), implicit Euler, no gravity.  With contact, the PD-PD
    contact force (distance 0.75 spacing) keeps them apart."""
    rng = np.random.default_rng(seed)
    g = _lattice(n_side, n_side, n_side).astype(np.float64)
    a = g * spacing
    b = g * spacing + np.array([(n_side - 1 + gap_spacings) * spacing, 0.0, 0.0])
    n = 2 * g.shape[0]
    pos = np.zeros((n, 4))
    pos[:, :3] = np.vstack([a, b]) + rng.uniform(-jitter, jitter, (n, 3)) * spacing
    vel = np.zeros((n, 4))
    vel[: n // 2, 0] = speed
    vel[n // 2:, 0] = -speed
    act = np.full(n, ACTIVE, np.int32)
    sim, run = _si_params(n, spacing, coeff, si_mass(spacing), s0, IMPLICIT_EULER, steps)
    opt = default_options()
    opt.precision = precision
    opt.cg_relative_tolerance = cg_tol
    opt.cg_max_iterations = 20000
    opt.time_step_base = dt / 128.0
    opt.bond_stiffness = si_stiffness(spacing)
    opt.gravity[:] = (0.0, 0.0, 0.0)
    opt.box_enabled = 0
    opt.contact_enabled = 1 if contact else 0
    opt.contact_distance = 0.75 * spacing
    opt.contact_stiffness = 1e7
    opt.contact_volume = 1.0
    return Scene("two_blocks", sim, run, opt, pos, vel, act, steps, {"spacing": spacing, "seed": seed})


def batched_scenes(count=64, n_min=4096, n_max=65536, seed=0, precision=PRECISION_MIXED, steps=100):
    """`count` impact bodies: particle counts log-uniform in [n_min, n_max],
    blocks and balls alternating at random, pd_kernel_coeff uniform in
    {4, 5, 6}, impact speed uniform in [1, 10] m/s."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        shape = "block" if rng.uniform() < 0.5 else "ball"
        coeff = float(rng.choice([4.0, 5.0, 6.0]))
        speed = float(rng.uniform(1.0, 10.0))
        out.append(impact_body(n, shape=shape, coeff=coeff, speed=speed, seed=seed * 1000 + k,
                               precision=precision, steps=steps))
    return out


def add_to_batch(batch, scene: Scene) -> int:
    """Adds a scene to a Batch (pd_batch_add_scene + its host arrays)."""
    return batch.add_scene(scene.sim, scene.run, scene.opt, scene.pos, scene.vel, scene.act)


def make_simulator(scene: Scene, device: int = 0):
    """Simulator with the scene's host arrays filled (examples/main.cpp:53-73)."""
    from . import Simulator
    simulator = Simulator(device, scene.sim, scene.run, scene.opt)
    simulator.get_pd_position()[:] = scene.pos
    simulator.get_pd_velocity()[:] = scene.vel
    simulator.get_pd_activity()[:] = scene.act
    return simulator
