"""TEST INFRASTRUCTURE ONLY: ctypes front-end to the CPU oracle.

``OracleSim`` drives ``oracle/libpd_oracle.so`` (pd_oracle.c, the FP64
restatement of the reference step).  ``RefSim`` drives
``oracle/_ref/libpdref.so``, the reference's own kernels compiled on the host
by ``oracle/build_ref.sh``; it exists only where the reference tree was
available at build time.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module.  The product library never loads it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libpd_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpdref.so")

ACTIVE, SEMI_ACTIVE, INACTIVE, INVISIBLE, CLAMPED, PRESCRIBED = range(6)


def build_oracle(force: bool = False) -> str:
    """Compile pd_oracle.c (no FMA contraction, OpenMP) into oracle/libpd_oracle.so."""
    src = os.path.join(HERE, "pd_oracle.c")
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < max(
        os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "pd_oracle.h"))
    ):
        subprocess.check_call(
            ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
             src, "-o", ORACLE_SO, "-lm"]
        )
    return ORACLE_SO


def reference_root() -> str | None:
    """The reference project's root: the PD_REFERENCE_ROOT environment
    variable, else a checkout named `reference` beside this repository's
    directory, else None (the tree exists only where fixtures are made)."""
    env = os.environ.get("PD_REFERENCE_ROOT")
    if env:
        return env
    beside = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    return beside if os.path.isdir(os.path.join(beside, "src", "core")) else None


def build_ref(reference_root: str | None = None) -> str | None:
    """Build oracle/_ref/libpdref.so when the reference tree is present
    (argument, else reference_root()); None when it is not."""
    if reference_root is None:
        reference_root = globals()["reference_root"]()
    if not reference_root or not os.path.isdir(os.path.join(reference_root, "src", "core")):
        return None
    subprocess.check_call([os.path.join(HERE, "build_ref.sh"), reference_root],
                          stdout=subprocess.DEVNULL)
    return REF_SO


class PdoParams(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("integrator", C.c_int), ("adaptive", C.c_int),
        ("horizon", C.c_double), ("radius", C.c_double), ("bond_coeff", C.c_double),
        ("mass", C.c_double), ("dt_base", C.c_double), ("dt_ticks", C.c_int),
        ("dt_ticks_min", C.c_int), ("max_substep", C.c_int), ("phase_in", C.c_int),
        ("stretch_a", C.c_double), ("stretch_b", C.c_double), ("alpha", C.c_double),
        ("gravity", C.c_double * 3), ("box_min", C.c_double * 3), ("box_max", C.c_double * 3),
        ("restitution", C.c_double), ("cg_rel_tol", C.c_double), ("cg_max_iter", C.c_int),
        ("max_bonds", C.c_int), ("s0", C.c_double), ("sphere_on", C.c_int),
        ("sphere_c0", C.c_double * 3), ("sphere_v", C.c_double * 3),
        ("sphere_radius", C.c_double), ("sphere_k", C.c_double),
        ("contact_on", C.c_int), ("contact_dist", C.c_double), ("contact_k", C.c_double),
        ("contact_vol", C.c_double), ("precond", C.c_int),
    ]


_lib = None


def _load():
    global _lib
    if _lib is None:
        build_oracle()
        lib = C.CDLL(ORACLE_SO)
        P = C.POINTER
        dp = P(C.c_double)
        ip = P(C.c_int)
        lib.pdo_default_params.argtypes = [P(PdoParams)]
        lib.pdo_create.argtypes = [P(PdoParams)]
        lib.pdo_create.restype = C.c_void_p
        lib.pdo_destroy.argtypes = [C.c_void_p]
        lib.pdo_set_particles.argtypes = [C.c_void_p, dp, dp, ip]
        lib.pdo_set_stretch.argtypes = [C.c_void_p, dp]
        lib.pdo_set_position.argtypes = [C.c_void_p, dp]
        lib.pdo_make_ready.argtypes = [C.c_void_p]
        lib.pdo_advance.argtypes = [C.c_void_p]
        lib.pdo_force_pass.argtypes = [C.c_void_p, ip]
        lib.pdo_assemble.argtypes = [C.c_void_p]
        lib.pdo_apply_A.argtypes = [C.c_void_p, dp, dp]
        lib.pdo_sample_stretch.argtypes = [C.c_int, C.c_double, dp]
        lib.pdo_sph_collide.argtypes = [C.c_void_p, dp, C.c_double, ip, C.c_double, C.c_double, C.c_double, dp, dp,
                                        C.c_int]
        lib.pdo_sph_collide.restype = C.c_int
        for name in ("pdo_current_step", "pdo_cg_converged", "pdo_last_cg_iters", "pdo_dt_ticks",
                     "pdo_substep", "pdo_retries_last_step"):
            getattr(lib, name).argtypes = [C.c_void_p]
            getattr(lib, name).restype = C.c_int
        for name in ("pdo_last_cg_residual", "pdo_clock_scale", "pdo_sim_time"):
            getattr(lib, name).argtypes = [C.c_void_p]
            getattr(lib, name).restype = C.c_double
        lib.pdo_num_bonds_total.argtypes = [C.c_void_p]
        lib.pdo_num_bonds_total.restype = C.c_long
        for name in ("pdo_get_position", "pdo_get_velocity", "pdo_get_force", "pdo_get_solution",
                     "pdo_get_rhs", "pdo_get_stretch", "pdo_get_new_stretch",
                     "pdo_get_original_stretch"):
            getattr(lib, name).argtypes = [C.c_void_p, dp]
        lib.pdo_get_bond_count.argtypes = [C.c_void_p, ip]
        lib.pdo_get_row_ptr.argtypes = [C.c_void_p, P(C.c_long)]
        lib.pdo_get_bond_list.argtypes = [C.c_void_p, ip]
        for name in ("pdo_get_position_backup", "pdo_get_velocity_backup"):
            getattr(lib, name).argtypes = [C.c_void_p, dp]
        lib.pdo_get_top_backup.argtypes = [C.c_void_p, ip]
        lib.pdo_get_top.argtypes = [C.c_void_p, ip]
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def default_params() -> PdoParams:
    p = PdoParams()
    _load().pdo_default_params(C.byref(p))
    return p


def params_from_body(body: dict) -> PdoParams:
    """Oracle parameters of a lattice body (the dict of
    sci-solver_peridynamic_gb300/lattice.py: SI constants, no box, rigid
    sphere), on top of the reference's defaults (definitions.h).  Used where
    the GPU library must not be loaded (bench.py's reference arm); a CPU test
    checks it equals the parameters the package's scene maps to."""
    p = default_params()
    p.n = int(body["pos"].shape[0])
    p.integrator = int(body["integrator"])
    p.adaptive = 0
    p.horizon = body["horizon"]
    p.radius = body["radius"]
    p.bond_coeff = body["stiffness"]
    p.mass = body["mass"]
    p.dt_base = body["dt"] / 128.0
    p.dt_ticks = 128
    for k in range(3):
        p.gravity[k] = body["gravity"][k]
        p.box_min[k], p.box_max[k] = -1e300, 1e300
    p.cg_rel_tol = body["cg_tol"]
    p.cg_max_iter = body["cg_max_iterations"]
    p.s0 = float(np.float32(body["s0"]))
    p.sphere_on = 1
    for k in range(3):
        p.sphere_c0[k] = body["sphere_center"][k]
        p.sphere_v[k] = body["sphere_velocity"][k]
    p.sphere_radius = body["sphere_radius"]
    p.sphere_k = body["sphere_stiffness"]
    return p


def sample_stretch(n: int, s0: float) -> np.ndarray:
    out = np.zeros(n, np.float64)
    _load().pdo_sample_stretch(n, float(s0), _dp(out))
    return out


class OracleSim:
    """FP64 restatement of Simulator (pd_oracle.c)."""

    def __init__(self, params: PdoParams):
        self.lib = _load()
        self.p = params
        self.n = params.n
        self.h = self.lib.pdo_create(C.byref(params))
        if not self.h:
            raise RuntimeError("pdo_create failed")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.pdo_destroy(self.h)
            self.h = None

    def set_particles(self, pos4, vel4=None, act=None):
        pos4 = np.ascontiguousarray(pos4, np.float64).reshape(self.n, 4)
        vel4 = np.zeros_like(pos4) if vel4 is None else np.ascontiguousarray(vel4, np.float64).reshape(self.n, 4)
        act = np.zeros(self.n, np.int32) if act is None else np.ascontiguousarray(act, np.int32)
        self._keep = (pos4, vel4, act)
        self.lib.pdo_set_particles(self.h, _dp(pos4), _dp(vel4), _ip(act))

    def set_position(self, pos4):
        """Current positions only (test hook); reference positions are kept."""
        pos4 = np.ascontiguousarray(pos4, np.float64).reshape(self.n, 4)
        self._pos_keep = pos4
        self.lib.pdo_set_position(self.h, _dp(pos4))

    def set_stretch(self, s0):
        s0 = np.ascontiguousarray(s0, np.float64)
        self.lib.pdo_set_stretch(self.h, _dp(s0))

    def make_ready(self):
        if self.lib.pdo_make_ready(self.h) != 0:
            raise RuntimeError("oracle bond construction failed (row exceeds max_bonds)")

    def advance(self, steps: int = 1):
        for _ in range(steps):
            self.lib.pdo_advance(self.h)

    def force_pass(self) -> int:
        flag = np.zeros(1, np.int32)
        self.lib.pdo_force_pass(self.h, _ip(flag))
        return int(flag[0])

    def assemble(self):
        self.lib.pdo_assemble(self.h)

    def apply_A(self, x4):
        x4 = np.ascontiguousarray(x4, np.float64).reshape(self.n, 4)
        y = np.zeros_like(x4)
        self.lib.pdo_apply_A(self.h, _dp(x4), _dp(y))
        return y

    def _vec4(self, fn):
        out = np.zeros((self.n, 4), np.float64)
        getattr(self.lib, fn)(self.h, _dp(out))
        return out

    def _vec1(self, fn):
        out = np.zeros(self.n, np.float64)
        getattr(self.lib, fn)(self.h, _dp(out))
        return out

    position = property(lambda self: self._vec4("pdo_get_position"))
    position_backup = property(lambda self: self._vec4("pdo_get_position_backup"))
    velocity_backup = property(lambda self: self._vec4("pdo_get_velocity_backup"))

    @property
    def bond_top(self):
        out = np.zeros(self.n, np.int32)
        self.lib.pdo_get_top(self.h, _ip(out))
        return out

    @property
    def bond_top_backup(self):
        out = np.zeros(self.n, np.int32)
        self.lib.pdo_get_top_backup(self.h, _ip(out))
        return out
    velocity = property(lambda self: self._vec4("pdo_get_velocity"))
    force = property(lambda self: self._vec4("pdo_get_force"))
    solution = property(lambda self: self._vec4("pdo_get_solution"))
    rhs = property(lambda self: self._vec4("pdo_get_rhs"))
    stretch = property(lambda self: self._vec1("pdo_get_stretch"))
    new_stretch = property(lambda self: self._vec1("pdo_get_new_stretch"))
    original_stretch = property(lambda self: self._vec1("pdo_get_original_stretch"))

    @property
    def bond_count(self):
        out = np.zeros(self.n, np.int32)
        self.lib.pdo_get_bond_count(self.h, _ip(out))
        return out

    @property
    def row_ptr(self):
        out = np.zeros(self.n + 1, np.int64)
        self.lib.pdo_get_row_ptr(self.h, out.ctypes.data_as(C.POINTER(C.c_long)))
        return out

    @property
    def bond_list(self):
        nb = self.lib.pdo_num_bonds_total(self.h)
        out = np.zeros(max(nb, 1), np.int32)
        self.lib.pdo_get_bond_list(self.h, _ip(out))
        return out[:nb]

    def alive_sets(self):
        """List of sorted live-neighbour arrays, one per particle."""
        rp, col, cnt = self.row_ptr, self.bond_list, self.bond_count
        return [np.sort(col[rp[i]:rp[i] + cnt[i]]) for i in range(self.n)]

    def sph_collide(self, lo, cell, n, r_sph, m_sph, slip, pos, vel):
        """SPH <-> PD collision of (k, 4) float64 SPH arrays (updated in place)
        on the grid (lo, cell, n); returns the SPH particles corrected."""
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        n = np.ascontiguousarray(n, dtype=np.int32)
        assert pos.dtype == np.float64 and pos.flags.c_contiguous and vel.dtype == np.float64 and vel.flags.c_contiguous
        return self.lib.pdo_sph_collide(self.h, _dp(lo), float(cell), _ip(n), float(r_sph), float(m_sph),
                                        float(slip), _dp(pos), _dp(vel), len(pos))

    step = property(lambda self: self.lib.pdo_current_step(self.h))
    cg_converged = property(lambda self: bool(self.lib.pdo_cg_converged(self.h)))
    cg_iters = property(lambda self: self.lib.pdo_last_cg_iters(self.h))
    cg_residual = property(lambda self: self.lib.pdo_last_cg_residual(self.h))
    dt_ticks = property(lambda self: self.lib.pdo_dt_ticks(self.h))
    substep = property(lambda self: self.lib.pdo_substep(self.h))
    retries = property(lambda self: self.lib.pdo_retries_last_step(self.h))
    clock_scale = property(lambda self: self.lib.pdo_clock_scale(self.h))
    sim_time = property(lambda self: self.lib.pdo_sim_time(self.h))


class RefSim:
    """The reference's own kernels, host-compiled (oracle/_ref/libpdref.so).

    Reference mode only: gravity -y 9.8, stiffness pd_C_times_V * PD_K, time
    base 2^-23, box reflection, s0 from srand(1973).
    """

    MAX_BONDS = 528

    def __init__(self, n, integrator, adaptive, horizon, radius, c_times_v, mass, bmin, bmax,
                 s0, cg_tol=1e-20, cg_max=100000, so_path=REF_SO):
        if not os.path.exists(so_path):
            raise FileNotFoundError(so_path)
        lib = C.CDLL(so_path)
        P = C.POINTER
        dp, ip = P(C.c_double), P(C.c_int)
        lib.ref_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                   C.c_double, dp, dp, C.c_float, C.c_double, C.c_int]
        lib.ref_create.restype = C.c_void_p
        lib.ref_destroy.argtypes = [C.c_void_p]
        lib.ref_set_particles.argtypes = [C.c_void_p, dp, dp, ip]
        lib.ref_make_ready.argtypes = [C.c_void_p]
        lib.ref_make_ready.restype = C.c_int
        lib.ref_advance.argtypes = [C.c_void_p]
        lib.ref_advance.restype = C.c_int
        for name in ("ref_cg_iters", "ref_cg_converged", "ref_ticks", "ref_has_broken"):
            getattr(lib, name).argtypes = [C.c_void_p]
            getattr(lib, name).restype = C.c_int
        lib.ref_cg_residual.argtypes = [C.c_void_p]
        lib.ref_cg_residual.restype = C.c_double
        for name in ("ref_get_position", "ref_get_velocity", "ref_get_force", "ref_get_solution",
                     "ref_get_stretch", "ref_get_new_stretch", "ref_get_original_stretch"):
            getattr(lib, name).argtypes = [C.c_void_p, dp]
        lib.ref_get_bond_count.argtypes = [C.c_void_p, ip]
        lib.ref_get_bond_list.argtypes = [C.c_void_p, ip]
        self.lib = lib
        self.n = n
        bmin = np.ascontiguousarray(bmin, np.float64)
        bmax = np.ascontiguousarray(bmax, np.float64)
        self.h = lib.ref_create(n, integrator, adaptive, horizon, radius, c_times_v, mass,
                                _dp(bmin), _dp(bmax), float(s0), cg_tol, cg_max)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_destroy(self.h)
            self.h = None

    def set_particles(self, pos4, vel4=None, act=None):
        pos4 = np.ascontiguousarray(pos4, np.float64).reshape(self.n, 4)
        vel4 = np.zeros_like(pos4) if vel4 is None else np.ascontiguousarray(vel4, np.float64).reshape(self.n, 4)
        act = np.zeros(self.n, np.int32) if act is None else np.ascontiguousarray(act, np.int32)
        self._keep = (pos4, vel4, act)
        self.lib.ref_set_particles(self.h, _dp(pos4), _dp(vel4), _ip(act))

    def make_ready(self):
        return self.lib.ref_make_ready(self.h)

    def advance(self, steps=1):
        r = 0
        for _ in range(steps):
            r += self.lib.ref_advance(self.h)
        return r

    def _vec4(self, fn):
        out = np.zeros((self.n, 4), np.float64)
        getattr(self.lib, fn)(self.h, _dp(out))
        return out

    def _vec1(self, fn):
        out = np.zeros(self.n, np.float64)
        getattr(self.lib, fn)(self.h, _dp(out))
        return out

    position = property(lambda self: self._vec4("ref_get_position"))
    velocity = property(lambda self: self._vec4("ref_get_velocity"))
    force = property(lambda self: self._vec4("ref_get_force"))
    solution = property(lambda self: self._vec4("ref_get_solution"))
    stretch = property(lambda self: self._vec1("ref_get_stretch"))
    new_stretch = property(lambda self: self._vec1("ref_get_new_stretch"))
    original_stretch = property(lambda self: self._vec1("ref_get_original_stretch"))
    cg_iters = property(lambda self: self.lib.ref_cg_iters(self.h))
    cg_residual = property(lambda self: self.lib.ref_cg_residual(self.h))
    cg_converged = property(lambda self: bool(self.lib.ref_cg_converged(self.h)))
    dt_ticks = property(lambda self: self.lib.ref_ticks(self.h))

    @property
    def bond_count(self):
        out = np.zeros(self.n, np.int32)
        self.lib.ref_get_bond_count(self.h, _ip(out))
        return out

    def bond_rows(self):
        """Rows in the reference's current order (live bonds first)."""
        out = np.zeros(self.n * self.MAX_BONDS, np.int32)
        self.lib.ref_get_bond_list(self.h, _ip(out))
        bl = out.reshape(self.MAX_BONDS, self.n)
        cnt = self.bond_count
        return bl, cnt

    def alive_sets(self):
        bl, cnt = self.bond_rows()
        return [np.sort(bl[:cnt[i], i]) for i in range(self.n)]
