"""Test helpers: map a scene onto the oracle's resolved parameters and compare runs."""
import numpy as np

from oracle import oracle as O


def oracle_params(scene):
    sim, run, opt = scene.sim, scene.run, scene.opt
    p = O.default_params()
    p.n = scene.n
    p.integrator = run.integrator
    p.adaptive = run.adaptive_integration
    p.horizon = sim.pd_horizon
    p.radius = sim.pd_particle_radius
    p.bond_coeff = opt.bond_stiffness if opt.bond_stiffness > 0 else sim.pd_C_times_V * opt.pd_k
    p.mass = sim.pd_particle_mass
    p.dt_base = opt.time_step_base
    p.dt_ticks = sim.pd_time_step
    p.dt_ticks_min = opt.time_step_min
    p.max_substep = opt.max_substep
    p.phase_in = opt.phase_in_steps
    p.stretch_a, p.stretch_b, p.alpha = opt.stretch_a, opt.stretch_b, opt.alpha
    for k in range(3):
        p.gravity[k] = opt.gravity[k]
    if opt.box_enabled:
        lo = (sim.boundary_min_x, sim.boundary_min_y, sim.boundary_min_z)
        hi = (sim.boundary_max_x, sim.boundary_max_y, sim.boundary_max_z)
    else:
        lo, hi = (-1e300,) * 3, (1e300,) * 3
    for k in range(3):
        p.box_min[k], p.box_max[k] = lo[k], hi[k]
    p.restitution = opt.restitution
    p.cg_rel_tol = opt.cg_relative_tolerance
    p.cg_max_iter = opt.cg_max_iterations
    p.max_bonds = opt.max_bonds_per_particle
    p.s0 = float(np.float32(run.pd_stretch_limit_s0))
    p.sphere_on = opt.sphere_enabled
    for k in range(3):
        p.sphere_c0[k] = opt.sphere_center[k]
        p.sphere_v[k] = opt.sphere_velocity[k]
    p.sphere_radius = opt.sphere_radius
    p.sphere_k = opt.sphere_stiffness
    p.contact_on = opt.contact_enabled
    p.contact_dist = opt.contact_distance
    p.contact_k = opt.contact_stiffness
    p.contact_vol = opt.contact_volume
    p.precond = opt.preconditioner
    return p


def make_oracle(scene):
    o = O.OracleSim(oracle_params(scene))
    o.set_particles(scene.pos, scene.vel, scene.act)
    o.make_ready()
    return o


def same_sets(a, b):
    return len(a) == len(b) and all(np.array_equal(np.asarray(x), np.asarray(y)) for x, y in zip(a, b))


def rel_err(x, ref):
    """max |x - ref| / max |ref| over xyz."""
    x = np.asarray(x)[:, :3]
    ref = np.asarray(ref)[:, :3]
    scale = max(np.abs(ref).max(), 1e-300)
    return float(np.abs(x - ref).max() / scale)


def rel_disp_err(x, ref, x0):
    """max |x - ref| / max |ref - x0| over xyz: the error measured against the
    motion since x0 (the displacement), not against the coordinates."""
    x = np.asarray(x)[:, :3]
    ref = np.asarray(ref)[:, :3]
    x0 = np.asarray(x0)[:, :3]
    scale = max(np.abs(ref - x0).max(), 1e-300)
    return float(np.abs(x - ref).max() / scale)


# positions: of max |x_ref|; displacements u = x - x0: of max |u_ref|.
# Largest errors measured over the parity tests on a GB300: mixed 4.8e-6 of
# the displacement (PD-PD contact 6.3e-5, see its test), FP64 8.3e-9.
POS_TOL = {0: 1e-5, 1: 1e-9}      # mixed, FP64
DISP_TOL = {0: 2e-5, 1: 5e-8}


def assert_positions(x, ref, x0, precision, label="", disp_tol=None):
    """Positions within POS_TOL of max |ref| and displacements from x0 within
    DISP_TOL (or disp_tol) of the reference's largest displacement (precision
    0 mixed, 1 FP64).  Prints both errors (pytest -s shows them)."""
    e_x, e_u = rel_err(x, ref), rel_disp_err(x, ref, x0)
    print(f"[parity] {label}: position {e_x:.3e}, displacement {e_u:.3e}")
    assert e_x < POS_TOL[precision], f"{label}: position error {e_x:.3e}"
    tol_u = DISP_TOL[precision] if disp_tol is None else disp_tol
    assert e_u < tol_u, f"{label}: displacement error {e_u:.3e}"
    return e_x, e_u


def apply_on_device(pdgb, sim, x_caller, entry=None):
    """y = A x through the C ABI; x, y in caller order.  Returns (y, <x, A x>)."""
    import torch
    v = sim.operator_view()
    n = v.n
    dt = torch.float32 if v.precision == pdgb.PRECISION_MIXED else torch.float64
    perm = sim.get(pdgb.VAR_SLOT_PERMUTATION)
    x_slot = torch.zeros((n, 4), dtype=dt, device="cuda")
    x_slot[:, :3] = torch.as_tensor(x_caller[perm, :3], dtype=dt, device="cuda")
    y_slot = torch.full_like(x_slot, float("nan"))
    dot = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    if entry is None:
        sim.apply_operator(x_slot.data_ptr(), y_slot.data_ptr(), dot.data_ptr())
    else:
        entry(v, x_slot.data_ptr(), y_slot.data_ptr(), dot.data_ptr())
    sim.synchronize()
    torch.cuda.synchronize()
    y = np.zeros((n, 4))
    y[perm] = y_slot.double().cpu().numpy()
    xs = np.zeros((n, 4))
    xs[perm] = x_slot.double().cpu().numpy()
    return y, float(dot.item()), xs
