"""Jittered-lattice bodies as plain numpy arrays, with the physical constants
of each scene, and nothing else: this module imports neither the package nor
its compiled library, so a caller can build a scene (for instance to time a
CPU implementation of the reference step on it) without loading the GPU
library.  ``scenes.py`` builds its Simulator inputs from the same functions.

The reference fills its bodies on a simple-cubic lattice of spacing 2 r
(src/examples/scene.cpp:33-135); these bodies use the same lattice, jittered
by a seeded uniform offset.

SI-unit material: density 125 kg/m^3 (1e-3 kg per particle at 0.02 m
spacing) and bond stiffness c = 1e6 * (spacing / 0.02)^2, the scaling under
which a bond-based PD solid keeps its wave speed as the lattice is refined.
"""
from __future__ import annotations

import math

import numpy as np

ACTIVE = 0          # pd_activity values (include/pd_gb300.h)
NEWMARK_BETA = 1    # pd_integrator


def lattice(nx, ny, nz):
    """Lattice indices in z-major, then y, then x order (as scene.cpp fills)."""
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)


def si_stiffness(spacing):
    return 1e6 * (spacing / 0.02) ** 2


def si_mass(spacing):
    return 1e-3 * (spacing / 0.02) ** 3


def ellipsoid_impact(target_n=1_000_000, semi_axes=(0.5, 0.35, 0.3), seed=0, jitter=0.05, coeff=5.0, s0=0.015,
                     dt=5e-5, cg_tol=1e-6, sphere_radius=0.1, sphere_speed=10.0, spacing=None, gap=1.0):
    """Jittered lattice filling an ellipsoid, struck along -x by a rigid
    sphere (penalty contact), Newmark-beta.  The spacing is chosen so the
    particle count is ~target_n.  The sphere starts `gap` spacings beyond the
    outermost particle (gap <= 0: in contact from the first step).

    Returns a dict: pos, vel (n x 4 float64), act (n int32) and the scene's
    constants (SI units): spacing, radius, horizon, coeff, mass, stiffness,
    dt, integrator, s0, gravity, cg_tol, cg_max_iterations, sphere_center,
    sphere_velocity, sphere_radius, sphere_stiffness."""
    a, b, c = semi_axes
    if spacing is None:
        spacing = (4.0 / 3.0 * math.pi * a * b * c / target_n) ** (1.0 / 3.0)
    nx, ny, nz = (int(math.floor(2 * s / spacing)) + 1 for s in semi_axes)
    g = lattice(nx, ny, nz)
    p0 = g * spacing - np.array([(nx - 1) * spacing / 2, (ny - 1) * spacing / 2, (nz - 1) * spacing / 2])
    inside = (p0[:, 0] / a) ** 2 + (p0[:, 1] / b) ** 2 + (p0[:, 2] / c) ** 2 <= 1.0
    p0 = p0[inside]
    n = p0.shape[0]
    rng = np.random.default_rng(seed)
    pos = np.zeros((n, 4))
    pos[:, :3] = p0 + rng.uniform(-jitter, jitter, (n, 3)) * spacing
    vel = np.zeros((n, 4))
    act = np.full(n, ACTIVE, np.int32)
    cstiff = si_stiffness(spacing)
    return {
        "pos": pos, "vel": vel, "act": act,
        "spacing": spacing, "radius": spacing / 2.0, "horizon": coeff * spacing / 2.0, "coeff": coeff,
        "mass": si_mass(spacing), "stiffness": cstiff, "dt": dt, "integrator": NEWMARK_BETA, "s0": s0,
        "gravity": (0.0, 0.0, -9.81), "cg_tol": cg_tol, "cg_max_iterations": 20000,
        "sphere_center": (pos[:, 0].max() + sphere_radius + gap * spacing, 0.0, 0.0),
        "sphere_velocity": (-sphere_speed, 0.0, 0.0), "sphere_radius": sphere_radius,
        # penalty stiffness of the order of one bond's (c / spacing); ten times
        # stiffer drives the compressed bonds under the impactor into an
        # indefinite tangent within ~10 steps, where CG (FP64 included) fails
        "sphere_stiffness": cstiff / spacing,
        "seed": seed, "semi_axes": tuple(semi_axes),
    }
