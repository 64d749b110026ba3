"""The oracle's SPH <-> PD collision (the checker of pd_sph_collide; the
reference's collideDifferentParticles, src/core/simulator.cuh:1590-1733),
against closed forms on a single PD particle, no GPU."""
import numpy as np
import pytest

from oracle import oracle as O

LO = np.zeros(3)
CELL = 1.0e-3
N = np.array([16, 16, 16], dtype=np.int32)
R_SPH = 2.5e-4


def _pd_state(vel=(0.0, 0.0, 0.0), mass=1000.0, radius=2.5e-4):
    p = O.default_params()
    p.n = 1
    p.horizon = 1.0e-3
    p.radius = radius
    p.mass = mass
    p.bond_coeff = 1.0
    o = O.OracleSim(p)
    pos = np.array([[5.0e-3, 5.0e-3, 5.0e-3, 0.0]])
    v = np.array([[vel[0], vel[1], vel[2], 0.0]])
    o.set_particles(pos, v, np.zeros(1, dtype=np.int32))
    o.make_ready()
    return o


@pytest.mark.parametrize("slip", [1.0, 0.0, 0.3])
def test_single_pair_closed_form(slip):
    vj = np.array([0.2, -0.1, 0.05])
    o = _pd_state(vel=vj)
    pj = o.position[0, :3].copy()
    m_i, m_j = 1.0, 1000.0
    d = np.array([3.0e-4, 1.0e-4, -0.5e-4])           # SPH particle at pj - d, closer than 5e-4
    pos = np.array([[*(pj - d), 0.0]])
    vi = np.array([1.0, 2.0, -0.5])
    vel = np.array([[*vi, 0.0]])
    assert o.sph_collide(LO, CELL, N, R_SPH, m_i, slip, pos, vel) == 1
    dist = np.linalg.norm(d)
    e = d / float(np.float32(dist))                      # the divisor rounded to float, as the reference
    np.testing.assert_allclose(pos[0, :3], pj - 5.0e-4 * e, rtol=0, atol=1e-18)
    vin, vjn = e * (e @ vi), e * (e @ vj)
    vit, vjt = vi - vin, vj - vjn
    vn = (m_i * vin + m_j * vjn) / (m_i + m_j)
    vit2 = ((m_i + m_j * slip) * vit + m_j * (1 - slip) * vjt) / (m_i + m_j)
    vjt2 = ((m_j + m_i * slip) * vjt + m_i * (1 - slip) * vit) / (m_i + m_j)
    np.testing.assert_allclose(vel[0, :3], vn + vit2, rtol=1e-14, atol=1e-16)
    np.testing.assert_allclose(o.velocity[0, :3], vn + vjt2, rtol=1e-14, atol=1e-16)
    if slip == 1.0:   # full slip: tangential parts untouched, normal momentum kept
        np.testing.assert_allclose(m_i * (vel[0, :3] - vit) + m_j * (o.velocity[0, :3] - vjt),
                                   m_i * vin + m_j * vjn, rtol=1e-12, atol=1e-15)


def test_out_of_reach_and_outside_grid():
    o = _pd_state()
    pj = o.position[0, :3]
    far = np.array([[*(pj + [6.0e-4, 0, 0]), 0.0]])     # beyond r_sph + r_pd
    out = np.array([[-1.0e-3, 5.0e-3, 5.0e-3, 0.0]])    # outside the grid
    for pos in (far, out):
        before = pos.copy()
        vel = np.ones((1, 4))
        assert o.sph_collide(LO, CELL, N, R_SPH, 1.0, 1.0, pos, vel) == 0
        np.testing.assert_array_equal(pos, before)


def test_two_sph_particles_one_pd_particle_smallest_index_writes():
    o = _pd_state(vel=(0.0, 0.0, 0.0))
    pj = o.position[0, :3]
    pos = np.array([[*(pj - [3e-4, 0, 0]), 0.0], [*(pj + [0, 3e-4, 0]), 0.0]])
    vel = np.array([[1.0, 0, 0, 0], [0, -1.0, 0, 0]])
    assert o.sph_collide(LO, CELL, N, R_SPH, 1.0, 1.0, pos, vel) == 2
    # the PD velocity is the one computed with the first SPH particle: along x
    v = o.velocity[0, :3]
    assert v[0] > 0 and v[1] == 0.0 and v[2] == 0.0
