"""Known answers for the oracle's force pass and assembled operator
(calculatePDForceDerivative, src/core/cg_solver.cuh:200-339, and
fillMatrixImplicitEuler / fillMatrixNewmarkBeta, implicit_euler.cuh:19-59,
newmark_beta.cuh:19-59):

* two particles: the bond force c (d/d0 - 1) vscale e and the operator
  A = m I + t2 [[J, -J], [-J, J]], J = (c/d0)[(1 - d0/d) I + (d0/d) e e^T],
  in closed form; e is the bond vector divided by the length rounded to
  float, as the reference's fmaxf(d, 1e-10) forms it;
* twelve particles (a jittered 2 x 2 x 3 block, every bond within horizon - r,
  so the surface factor vscale is 1): the assembled stiffness equals minus
  the central difference of the force, i.e. J is the force's exact tangent.

The reference's Jacobian does not carry vscale (cg_solver.cuh:292-299): for a
bond longer than horizon - r the force is scaled and the tangent is not; the
closed form below keeps that asymmetry."""
import numpy as np
import pytest

from oracle import oracle as O


def make(pos, horizon, radius=1.0, c=1e6, mass=2.0, integrator=0, ticks=128, dt_base=1e-6):
    p = O.default_params()
    p.n = len(pos)
    p.integrator = integrator
    p.adaptive = 0
    p.horizon, p.radius, p.bond_coeff, p.mass = horizon, radius, c, mass
    p.dt_base, p.dt_ticks = dt_base, ticks
    p.phase_in = 0
    for k in range(3):
        p.gravity[k] = 0.0
        p.box_min[k], p.box_max[k] = -1e300, 1e300
    o = O.OracleSim(p)
    o.set_particles(pos)
    o.set_stretch(np.full(len(pos), 0.5))   # nothing breaks
    o.make_ready()
    h = ticks * dt_base
    t2 = h * h if integrator == 0 else h * h / 4.0
    return o, t2


def assembled_matrix(o):
    """Dense 3n x 3n A from apply_A on unit vectors."""
    n = o.n
    A = np.zeros((3 * n, 3 * n))
    for col in range(3 * n):
        x = np.zeros((n, 4))
        x[col // 3, col % 3] = 1.0
        A[:, col] = o.apply_A(x)[:, :3].reshape(-1)
    return A


def bond_terms(xp, xq, Xp, Xq, c, horizon, radius):
    """Force on p and the bond's J, in the reference's operation order."""
    dx = xq - xp
    d = np.sqrt(np.dot(dx, dx))
    D = float(np.float32(max(np.float32(d), np.float32(1e-10))))
    e = dx / D
    d0 = np.sqrt(np.dot(Xp - Xq, Xp - Xq))
    s = d / d0 - 1.0
    vscale = 1.0 if d0 <= horizon - radius else 0.5 + (horizon - d0) / 2.0 / radius
    J = (c / d0) * ((1.0 - d0 / d) * np.eye(3) + (d0 / d) * np.outer(e, e))
    return c * s * vscale * e, J


@pytest.mark.parametrize("d0,integrator", [(2.0, 0), (2.0, 1), (4.5, 0)])
def test_two_particle_closed_form(d0, integrator):
    rng = np.random.default_rng(11)
    u = rng.standard_normal(3)
    u /= np.linalg.norm(u)
    pos = np.zeros((2, 4))
    pos[1, :3] = d0 * u
    horizon, radius, c, m = 5.001, 1.0, 1e6, 2.0
    o, t2 = make(pos, horizon, radius, c, m, integrator)
    assert list(o.bond_count) == [1, 1]
    x = pos.copy()
    x[:, :3] += 1e-3 * rng.standard_normal((2, 3))
    o.set_position(x)
    assert o.force_pass() == 0
    f_p, J = bond_terms(x[0, :3], x[1, :3], pos[0, :3], pos[1, :3], c, horizon, radius)
    F = o.force
    # s = d/d0 - 1 ~ 1e-3 carries the rounding of d and d0 amplified by 1/s
    tol = 1e-15 / abs(np.linalg.norm(x[1, :3] - x[0, :3]) / d0 - 1.0)
    np.testing.assert_allclose(F[0, :3], f_p, rtol=tol, atol=tol * np.abs(f_p).max())
    np.testing.assert_allclose(F[1, :3], -f_p, rtol=tol, atol=tol * np.abs(f_p).max())
    assert np.all(F[:, 3] == 0.0)
    o.assemble()
    A = assembled_matrix(o)
    K = np.block([[J, -J], [-J, J]])
    expect = m * np.eye(6) + t2 * K
    assert np.abs(A - expect).max() <= 1e-13 * np.abs(expect).max()
    # symmetric positive definite for a stretched bond
    assert np.allclose(A, A.T, rtol=0, atol=1e-15 * np.abs(A).max())


def test_jacobian_is_the_force_tangent():
    rng = np.random.default_rng(3)
    g = np.array([(i, j, k) for k in range(3) for j in range(2) for i in range(2)], np.float64)
    n = len(g)
    pos = np.zeros((n, 4))
    pos[:, :3] = 1.0 * g + rng.uniform(-0.05, 0.05, (n, 3))   # spacing 1, radius 0.5
    horizon, radius = 3.2, 0.5
    # every pair is a bond and every bond is shorter than horizon - radius
    dmax = max(np.linalg.norm(pos[a, :3] - pos[b, :3]) for a in range(n) for b in range(n))
    assert dmax < horizon - radius
    o, t2 = make(pos, horizon, radius, c=1e3, mass=1.0)
    assert list(o.bond_count) == [n - 1] * n
    x = pos.copy()
    x[:, :3] += 2e-3 * rng.standard_normal((n, 3))
    o.set_position(x)
    o.force_pass()
    o.assemble()
    K = (assembled_matrix(o) - 1.0 * np.eye(3 * n)) / t2
    eps = 1e-4
    dF = np.zeros((3 * n, 3 * n))
    for col in range(3 * n):
        xp, xm = x.copy(), x.copy()
        xp[col // 3, col % 3] += eps
        xm[col // 3, col % 3] -= eps
        o.set_position(xp)
        o.force_pass()
        fp = o.force[:, :3].reshape(-1)
        o.set_position(xm)
        o.force_pass()
        fm = o.force[:, :3].reshape(-1)
        dF[:, col] = (fp - fm) / (2 * eps)
    # the float-rounded normalisation of e makes the force step by ~6e-8 of
    # its size where the rounded length changes; over 2 eps that is noise of
    # ~1e-6 of K, well above the O(eps^2) truncation error
    assert np.abs(K + dF).max() <= 3e-6 * np.abs(K).max()
    # the stiffness is symmetric and its rows sum to zero (rigid translation)
    assert np.abs(K - K.T).max() <= 1e-12 * np.abs(K).max()
    for a in range(3):
        t = np.zeros(3 * n)
        t[a::3] = 1.0
        assert np.abs(K @ t).max() <= 1e-9 * np.abs(K).max()
