"""GB300 implicit bond-based peridynamics step -- Python host mirror.

A drop-in for the PD path of SCI-Solver_Peridynamic's PeriCUDAEngine.  The
classes here mirror the reference's host interface over the C ABI of
``libpd_gb300.so`` (``include/pd_gb300.h``):

  SystemParameter   src/core/parameters.h:146-162 (file -> SimulationParameters,
                    RunningParameters)
  Simulator         src/core/simulator.h:32-57 (makeReady, advance, finished,
                    CGConvergence, get_current_step, get_pd_position/velocity/
                    activity host arrays)

The compute path is the CUDA library; there is no CPU fallback: every call
that needs the device raises ``PdError`` when the library or the GPU is
missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libpd_gb300.so")

# pd_status
PD_OK = 0
STATUS_NAMES = {0: "PD_OK", 1: "PD_ERR_INVALID_ARGUMENT", 2: "PD_ERR_CUDA", 3: "PD_ERR_NOT_READY",
                4: "PD_ERR_BOND_OVERFLOW", 5: "PD_ERR_NO_DEVICE", 6: "PD_ERR_FILE", 7: "PD_ERR_OUT_OF_MEMORY",
                8: "PD_ERR_STATE"}
# pd_integrator
IMPLICIT_EULER, NEWMARK_BETA = 0, 1
# pd_activity
ACTIVE, SEMI_ACTIVE, INACTIVE, INVISIBLE, CLAMPED, PRESCRIBED = range(6)
# pd_precision
PRECISION_MIXED, PRECISION_FP64 = 0, 1
# pd_variable
(VAR_POSITION, VAR_VELOCITY, VAR_ACTIVITY, VAR_BOND_COUNT, VAR_STRETCH, VAR_ORIGINAL_STRETCH,
 VAR_NEW_STRETCH, VAR_FORCE, VAR_SOLUTION, VAR_BOND_ROW_PTR, VAR_BOND_LIST, VAR_POSITION_SCALED,
 VAR_ORIGINAL_POSITION, VAR_SLOT_PERMUTATION, VAR_BROKEN_MASK) = range(15)
# pd_kernel_class
KC_FORCE, KC_SPMV, KC_CG_VECTOR, KC_UPDATE = range(4)
KC_NAMES = ("force", "spmv", "cg_vector", "update", "guess")


class PdError(RuntimeError):
    def __init__(self, status, message=""):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class SimulationParameters(C.Structure):
    """pd_sim_params: PD fields of SimulationParameters (src/core/parameters.h:16-88)."""
    _fields_ = [
        ("num_pd_particle", C.c_int), ("num_cell_x", C.c_int), ("num_cell_y", C.c_int),
        ("num_cell_z", C.c_int), ("num_cells", C.c_int), ("cell_size", C.c_double),
        ("sph_kernel_coeff", C.c_double), ("pd_kernel_coeff", C.c_double),
        ("sph_particle_mass", C.c_double), ("pd_particle_mass", C.c_double),
        ("boundary_min_x", C.c_double), ("boundary_min_y", C.c_double), ("boundary_min_z", C.c_double),
        ("boundary_max_x", C.c_double), ("boundary_max_y", C.c_double), ("boundary_max_z", C.c_double),
        ("pd_max_num_bonds", C.c_int), ("pd_time_step", C.c_int),
        ("sph_particle_radius", C.c_double), ("pd_particle_radius", C.c_double),
        ("pd_horizon", C.c_double), ("pd_C_times_V", C.c_double), ("clockScale", C.c_double),
        ("scaleFactor", C.c_double),
    ]


class RunningParameters(C.Structure):
    """pd_run_params: RunningParameters (src/core/parameters.h:90-135)."""
    _fields_ = [
        ("adaptive_integration", C.c_int), ("gpu_device", C.c_int), ("step_per_frame", C.c_int),
        ("step_per_state", C.c_int), ("start_step", C.c_int), ("final_step", C.c_int),
        ("wall_thickness", C.c_int), ("tube_radius", C.c_int), ("sph_initial_velocity", C.c_float),
        ("mesh_translation_x", C.c_float), ("mesh_translation_y", C.c_float),
        ("mesh_translation_z", C.c_float), ("pd_stretch_limit_s0", C.c_float),
        ("pd_initial_velocity", C.c_float), ("dump_activity", C.c_int), ("dump_density", C.c_int),
        ("dump_velocity", C.c_int), ("dump_pd_bond_list_top", C.c_int), ("integrator", C.c_int),
        ("obj_file", C.c_char * 512), ("saving_path", C.c_char * 512),
    ]


class SolverOptions(C.Structure):
    """pd_solver_options: the reference's definitions.h constants plus this library's knobs."""
    _fields_ = [
        ("precision", C.c_int), ("cg_relative_tolerance", C.c_double), ("cg_max_iterations", C.c_int),
        ("time_step_base", C.c_double), ("time_step_min", C.c_int), ("max_substep", C.c_int),
        ("phase_in_steps", C.c_int), ("pd_k", C.c_double), ("bond_stiffness", C.c_double),
        ("gravity", C.c_double * 3), ("restitution", C.c_double), ("box_enabled", C.c_int),
        ("stretch_a", C.c_double), ("stretch_b", C.c_double), ("alpha", C.c_double),
        ("max_bonds_per_particle", C.c_int), ("sphere_enabled", C.c_int),
        ("sphere_center", C.c_double * 3), ("sphere_velocity", C.c_double * 3),
        ("sphere_radius", C.c_double), ("sphere_stiffness", C.c_double),
        ("lanes_per_particle", C.c_int), ("cg_check_interval", C.c_int), ("spmv_unroll", C.c_int),
        ("warm_start", C.c_int), ("spmv_path", C.c_int), ("contact_enabled", C.c_int),
        ("contact_distance", C.c_double), ("contact_stiffness", C.c_double), ("contact_volume", C.c_double),
        ("history_size", C.c_int), ("cg_loop", C.c_int), ("preconditioner", C.c_int),
    ]


class StepStats(C.Structure):
    _fields_ = [
        ("current_step", C.c_int), ("cg_converged", C.c_int), ("last_cg_iterations", C.c_int),
        ("last_cg_residual", C.c_double), ("last_cg_tolerance", C.c_double),
        ("total_cg_iterations", C.c_longlong), ("time_step_ticks", C.c_int), ("substep", C.c_int),
        ("retries_last_step", C.c_int), ("bonds_initial", C.c_longlong), ("bonds_alive", C.c_longlong),
        ("max_bonds_per_particle", C.c_int), ("clock_scale", C.c_double), ("sim_time", C.c_double),
        ("ws_guesses_kept", C.c_longlong), ("last_ws_residual_ratio", C.c_double),
        ("ws_learned_used", C.c_longlong), ("host_syncs", C.c_longlong), ("cg_graph_solves", C.c_longlong),
        ("ws_guesses_skipped", C.c_longlong),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class OperatorView(C.Structure):
    """pd_operator_view: device-side view of the current system operator."""
    _fields_ = [
        ("n", C.c_int), ("precision", C.c_int), ("lanes_per_particle", C.c_int), ("blocks", C.c_int),
        ("activity", C.c_void_p), ("row_ptr", C.c_void_p), ("bond_count", C.c_void_p),
        ("bond_slot", C.c_void_p), ("perm", C.c_void_p), ("ref_pos", C.c_void_p), ("disp", C.c_void_p),
        ("pos_cell", C.c_void_p), ("inv_d0", C.c_void_p), ("supercell_size", C.c_double),
        ("jac", C.c_void_p), ("jac_diag", C.c_void_p), ("mass", C.c_double), ("t2", C.c_double),
        ("bond_coeff", C.c_double), ("sphere_center_local", C.c_double * 3), ("sphere_stiffness", C.c_double),
    ]


class KernelTimes(C.Structure):
    _fields_ = [("launches", C.c_longlong * 5), ("total_ms", C.c_double * 5)]


_lib = None


class BatchOptions(C.Structure):
    """pd_batch_options: SpMV launch shape and item size (0 = autotune), graph
    replay, learned warm start (1: on, mixed precision)."""
    _fields_ = [("lanes_per_particle", C.c_int), ("spmv_unroll", C.c_int), ("item_rows", C.c_int),
                ("use_graph", C.c_int), ("warm_start", C.c_int)]


class BatchConfig(C.Structure):
    """pd_batch_config: the launch shape in use."""
    _fields_ = [("lanes_per_particle", C.c_int), ("spmv_unroll", C.c_int), ("item_rows", C.c_int),
                ("work_items", C.c_int), ("grid_pre", C.c_int), ("grid_cg", C.c_int), ("autotuned", C.c_int),
                ("tuned_spmv_ms", C.c_double), ("warm_start", C.c_int)]


def library(build_if_missing: bool = True):
    """Load libpd_gb300.so (building it first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        from importlib import import_module
        build_mod = import_module(__name__ + ".build")
        build_mod.build()
    if not os.path.exists(LIB_PATH):
        raise PdError(2, f"{LIB_PATH} is missing; run build.py")
    lib = C.CDLL(LIB_PATH)
    P = C.POINTER
    st = C.c_int
    vp = C.c_void_p
    sig = {
        "pd_params_default": (st, [P(SimulationParameters), P(RunningParameters)]),
        "pd_params_load": (st, [C.c_char_p, P(SimulationParameters), P(RunningParameters)]),
        "pd_params_derive": (st, [P(SimulationParameters), P(RunningParameters)]),
        "pd_solver_options_default": (st, [P(SolverOptions)]),
        "pd_create": (st, [P(SimulationParameters), P(RunningParameters), P(SolverOptions), P(vp)]),
        "pd_destroy": (st, [vp]),
        "pd_set_particles": (st, [vp, P(C.c_double), P(C.c_double), P(C.c_int32), C.c_int]),
        "pd_set_stretch_limits": (st, [vp, P(C.c_double), C.c_int]),
        "pd_make_ready": (st, [vp]),
        "pd_advance": (st, [vp, C.c_int]),
        "pd_finished": (st, [vp, P(C.c_int)]),
        "pd_cg_converged": (st, [vp, P(C.c_int)]),
        "pd_get_current_step": (st, [vp, P(C.c_int)]),
        "pd_get": (st, [vp, C.c_int, vp, C.c_size_t]),
        "pd_get_size": (st, [vp, C.c_int, P(C.c_size_t)]),
        "pd_get_stats": (st, [vp, P(StepStats)]),
        "pd_get_params": (st, [vp, P(SimulationParameters), P(RunningParameters), P(SolverOptions)]),
        "pd_set_profiling": (st, [vp, C.c_int]),
        "pd_get_kernel_times": (st, [vp, P(KernelTimes)]),
        "pd_reset_kernel_times": (st, [vp]),
        "pd_get_launch_count": (st, [vp, P(C.c_longlong)]),
        "pd_get_stream": (st, [vp, P(vp)]),
        "pd_get_operator_view": (st, [vp, P(OperatorView)]),
        "pd_apply_operator": (st, [vp, vp, vp, vp]),
        "pd_apply_operator_noalloc": (st, [P(OperatorView), vp, vp, vp, vp]),
        "pd_mlp_param_count": (C.c_size_t, []),
        "pd_mlp_init": (st, [C.c_uint, P(C.c_float)]),
        "pd_mlp_predict": (st, [C.c_int, P(C.c_float), C.c_longlong, P(C.c_float), P(C.c_float)]),
        "pd_mlp_loss_grad": (st, [C.c_int, P(C.c_float), P(C.c_float), C.c_int, P(C.c_float), P(C.c_float),
                                  P(C.c_double)]),
        "pd_mlp_train": (st, [C.c_int, P(C.c_float), P(C.c_float), C.c_longlong, C.c_int, C.c_int, C.c_float, C.c_uint,
                              P(C.c_float), P(C.c_double)]),
        "pd_ws_set_params": (st, [vp, P(C.c_float), C.c_size_t]),
        "pd_ws_get_params": (st, [vp, P(C.c_float), C.c_size_t]),
        "pd_ws_collect": (st, [vp, C.c_int, C.c_longlong]),
        "pd_ws_dataset": (st, [vp, P(C.c_float), P(C.c_float), C.c_longlong, P(C.c_longlong)]),
        "pd_synchronize": (st, [vp]),
        "pd_status_string": (C.c_char_p, [C.c_int]),
        "pd_last_error_message": (C.c_char_p, [vp]),
        "pd_abi_version": (C.c_int, []),
        "pd_sample_stretch_limits": (st, [C.c_float, C.c_int, P(C.c_double)]),
        "pd_adaptive_decide": (st, [C.c_int, C.c_int, C.c_int, C.c_int, P(C.c_int), P(C.c_int), P(C.c_int)]),
        "pd_dataio_get_data_and_write": (st, [vp]),
        "pd_dataio_new_frame": (st, [vp]),
        "pd_dataio_saved_frame": (st, [vp, P(C.c_size_t)]),
        "pd_dataio_save_state": (st, [vp, C.c_size_t]),
        "pd_dataio_load_state": (st, [vp, C.c_size_t]),
        "pd_dataio_save_state_reference": (st, [vp, C.c_size_t]),
        "pd_dataio_load_state_reference": (st, [vp, C.c_size_t]),
        "pd_sph_collide": (st, [vp, P(C.c_double), P(C.c_double), C.c_int, C.c_double, P(C.c_int)]),
        "pd_scene_create": (st, [P(SimulationParameters), P(RunningParameters), C.c_int, C.c_uint, P(vp)]),
        "pd_scene_particle_count": (st, [vp, P(C.c_int)]),
        "pd_scene_init_pd_particles": (st, [vp, P(C.c_int32), P(C.c_double), P(C.c_double)]),
        "pd_scene_destroy": (st, [vp]),
        "pd_scene_last_error_message": (C.c_char_p, []),
        "pd_batch_options_default": (st, [P(BatchOptions)]),
        "pd_batch_create": (st, [C.c_int, P(BatchOptions), P(vp)]),
        "pd_batch_destroy": (st, [vp]),
        "pd_batch_add_scene": (st, [vp, P(SimulationParameters), P(RunningParameters), P(SolverOptions),
                                    P(C.c_int)]),
        "pd_batch_set_particles": (st, [vp, C.c_int, P(C.c_double), P(C.c_double), P(C.c_int32), C.c_int]),
        "pd_batch_set_stretch_limits": (st, [vp, C.c_int, P(C.c_double), C.c_int]),
        "pd_batch_make_ready": (st, [vp]),
        "pd_batch_ws_set_params": (st, [vp, P(C.c_float), C.c_size_t]),
        "pd_batch_advance": (st, [vp, C.c_int]),
        "pd_batch_scene_count": (st, [vp, P(C.c_int)]),
        "pd_batch_scene_offsets": (st, [vp, P(C.c_int64), C.c_int]),
        "pd_batch_get": (st, [vp, C.c_int, C.c_int, vp, C.c_size_t]),
        "pd_batch_get_size": (st, [vp, C.c_int, C.c_int, P(C.c_size_t)]),
        "pd_batch_get_stats": (st, [vp, C.c_int, P(StepStats)]),
        "pd_batch_finished": (st, [vp, C.c_int, P(C.c_int)]),
        "pd_batch_get_config": (st, [vp, P(BatchConfig)]),
        "pd_batch_get_launch_count": (st, [vp, P(C.c_longlong)]),
        "pd_batch_get_stream": (st, [vp, P(vp)]),
        "pd_batch_synchronize": (st, [vp]),
        "pd_batch_last_error_message": (C.c_char_p, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(status, handle=None):
    if status != PD_OK:
        lib = library(False)
        msg = lib.pd_last_error_message(handle)
        raise PdError(status, msg.decode() if msg else "")


def default_options() -> SolverOptions:
    o = SolverOptions()
    _check(library().pd_solver_options_default(C.byref(o)))
    return o


def sample_stretch_limits(s0: float, n: int) -> np.ndarray:
    out = np.zeros(n, np.float64)
    _check(library().pd_sample_stretch_limits(C.c_float(s0), n, out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


def adaptive_decide(has_broken, ticks, substep, ticks_base=128, ticks_min=100, max_substep=10):
    t, s, rb = C.c_int(ticks), C.c_int(substep), C.c_int(0)
    _check(library().pd_adaptive_decide(int(has_broken), ticks_base, ticks_min, max_substep,
                                        C.byref(t), C.byref(s), C.byref(rb)))
    return t.value, s.value, bool(rb.value)


def apply_operator_noalloc(view: OperatorView, d_x: int, d_y: int, d_dot: int | None = None, stream: int = 0):
    """pd_apply_operator_noalloc: y = A x for callers that cannot allocate
    device memory; every pointer is a raw device address they own."""
    _check(library().pd_apply_operator_noalloc(C.byref(view), C.c_void_p(d_x), C.c_void_p(d_y),
                                               C.c_void_p(d_dot) if d_dot else None,
                                               C.c_void_p(stream) if stream else None))


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def mlp_param_count() -> int:
    return int(library().pd_mlp_param_count())


def mlp_init(seed: int = 1) -> np.ndarray:
    p = np.zeros(mlp_param_count(), np.float32)
    _check(library().pd_mlp_init(seed, _fp(p)))
    return p


def mlp_predict(X, params, device: int = 0) -> np.ndarray:
    X = np.ascontiguousarray(X, np.float32)
    params = np.ascontiguousarray(params, np.float32)
    Y = np.zeros((X.shape[0], 3), np.float32)
    _check(library().pd_mlp_predict(device, _fp(X), X.shape[0], _fp(params), _fp(Y)))
    return Y


def mlp_loss_grad(X, T, params, device: int = 0):
    X = np.ascontiguousarray(X, np.float32)
    T = np.ascontiguousarray(T, np.float32)
    params = np.ascontiguousarray(params, np.float32)
    g = np.zeros_like(params)
    loss = C.c_double()
    _check(library().pd_mlp_loss_grad(device, _fp(X), _fp(T), X.shape[0], _fp(params), _fp(g), C.byref(loss)))
    return loss.value, g


def mlp_train(X, T, params, iterations=2000, batch=1024, lr=1e-3, seed=1, device: int = 0):
    """Adam on the GPU; returns (trained params, loss over all rows)."""
    X = np.ascontiguousarray(X, np.float32)
    T = np.ascontiguousarray(T, np.float32)
    p = np.array(params, np.float32, copy=True)
    loss = C.c_double()
    _check(library().pd_mlp_train(device, _fp(X), _fp(T), X.shape[0], iterations, batch, lr, seed, _fp(p),
                                  C.byref(loss)))
    return p, loss.value


class SystemParameter:
    """SystemParameter (src/core/parameters.h:146-162)."""

    def __init__(self, param_file: str | None = None):
        self._sim = SimulationParameters()
        self._run = RunningParameters()
        lib = library()
        if param_file is None:
            _check(lib.pd_params_default(C.byref(self._sim), C.byref(self._run)))
        else:
            _check(lib.pd_params_load(param_file.encode(), C.byref(self._sim), C.byref(self._run)))

    def derive(self):
        """calculateDependentParameters, for parameters set in code."""
        _check(library().pd_params_derive(C.byref(self._sim), C.byref(self._run)))

    def getSimulationParameters(self) -> SimulationParameters:
        return self._sim

    def getRunningParameters(self) -> RunningParameters:
        return self._run


class Simulator:
    """Simulator (src/core/simulator.h:32-57) over the C ABI.

    As in the reference, the caller fills the host arrays returned by
    get_pd_position / get_pd_velocity / get_pd_activity before makeReady().
    """

    def __init__(self, deviceID: int, simParams: SimulationParameters, runningParams: RunningParameters,
                 options: SolverOptions | None = None):
        self.lib = library()
        self.sim = simParams
        self.run = runningParams
        self.run.gpu_device = deviceID
        self.options = options if options is not None else default_options()
        self.n = int(simParams.num_pd_particle)
        h = C.c_void_p()
        _check(self.lib.pd_create(C.byref(self.sim), C.byref(self.run), C.byref(self.options), C.byref(h)))
        self.h = h
        self._pos = np.zeros((self.n, 4), np.float64)
        self._vel = np.zeros((self.n, 4), np.float64)
        self._act = np.zeros(self.n, np.int32)
        self._s0 = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.pd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # host arrays filled by the caller before makeReady (examples/main.cpp:64-66)
    def get_pd_position(self) -> np.ndarray:
        return self._pos

    def get_pd_velocity(self) -> np.ndarray:
        return self._vel

    def get_pd_activity(self) -> np.ndarray:
        return self._act

    def set_stretch_limits(self, s0):
        self._s0 = np.ascontiguousarray(s0, np.float64)

    def makeReady(self):
        dp = C.POINTER(C.c_double)
        pos = np.ascontiguousarray(self._pos, np.float64)
        vel = np.ascontiguousarray(self._vel, np.float64)
        act = np.ascontiguousarray(self._act, np.int32)
        _check(self.lib.pd_set_particles(self.h, pos.ctypes.data_as(dp), vel.ctypes.data_as(dp),
                                         act.ctypes.data_as(C.POINTER(C.c_int32)), self.n), self.h)
        if self._s0 is not None:
            _check(self.lib.pd_set_stretch_limits(self.h, self._s0.ctypes.data_as(dp), self.n), self.h)
        _check(self.lib.pd_make_ready(self.h), self.h)

    def advance(self, nsteps: int = 1):
        _check(self.lib.pd_advance(self.h, int(nsteps)), self.h)

    def finished(self) -> bool:
        v = C.c_int()
        _check(self.lib.pd_finished(self.h, C.byref(v)), self.h)
        return bool(v.value)

    def CGConvergence(self) -> bool:
        v = C.c_int()
        _check(self.lib.pd_cg_converged(self.h, C.byref(v)), self.h)
        return bool(v.value)

    def get_current_step(self) -> int:
        v = C.c_int()
        _check(self.lib.pd_get_current_step(self.h, C.byref(v)), self.h)
        return v.value

    # exports (MemoryManager::downloadFromDevice equivalents)
    def get(self, var: int, out: np.ndarray | None = None) -> np.ndarray:
        """The variable in caller order; with `out` (C-contiguous, of the
        variable's byte size, e.g. a pinned buffer) it is written there."""
        size = C.c_size_t()
        _check(self.lib.pd_get_size(self.h, var, C.byref(size)), self.h)
        if out is not None:
            if not out.flags["C_CONTIGUOUS"] or out.nbytes != size.value:
                raise ValueError("get: out must be C-contiguous with %d bytes" % size.value)
            _check(self.lib.pd_get(self.h, var, out.ctypes.data_as(C.c_void_p), size.value), self.h)
            return out
        if var == VAR_BROKEN_MASK:
            out = np.zeros(size.value, np.uint8)
        elif var in (VAR_ACTIVITY, VAR_BOND_COUNT, VAR_BOND_LIST, VAR_SLOT_PERMUTATION):
            out = np.zeros(size.value // 4, np.int32)
        elif var == VAR_BOND_ROW_PTR:
            out = np.zeros(size.value // 8, np.int64)
        else:
            out = np.zeros(size.value // 8, np.float64)
        _check(self.lib.pd_get(self.h, var, out.ctypes.data_as(C.c_void_p), size.value), self.h)
        if var in (VAR_POSITION, VAR_VELOCITY, VAR_FORCE, VAR_SOLUTION, VAR_POSITION_SCALED, VAR_ORIGINAL_POSITION):
            out = out.reshape(self.n, 4)
        return out

    def downloadFromDevice(self, var: int) -> np.ndarray:
        """Refresh the host array like MemoryManager::downloadFromDevice
        (positions are multiplied by scaleFactor, memory_manager.cu:274-298)."""
        if var == VAR_POSITION:
            self._pos[:] = self.get(VAR_POSITION_SCALED)
            return self._pos
        if var == VAR_VELOCITY:
            self._vel[:] = self.get(VAR_VELOCITY)
            return self._vel
        return self.get(var)

    def bond_rows(self):
        """Per particle (caller order): sorted live neighbours, sorted broken ones."""
        rp = self.get(VAR_BOND_ROW_PTR)
        bl = self.get(VAR_BOND_LIST)
        cnt = self.get(VAR_BOND_COUNT)
        return rp, bl, cnt

    def alive_sets(self):
        rp, bl, cnt = self.bond_rows()
        return [bl[rp[i]:rp[i] + cnt[i]] for i in range(self.n)]

    def stats(self) -> StepStats:
        s = StepStats()
        _check(self.lib.pd_get_stats(self.h, C.byref(s)), self.h)
        return s

    def params(self):
        s, r, o = SimulationParameters(), RunningParameters(), SolverOptions()
        _check(self.lib.pd_get_params(self.h, C.byref(s), C.byref(r), C.byref(o)), self.h)
        return s, r, o

    def set_profiling(self, on: bool):
        _check(self.lib.pd_set_profiling(self.h, 1 if on else 0), self.h)

    def kernel_times(self):
        t = KernelTimes()
        _check(self.lib.pd_get_kernel_times(self.h, C.byref(t)), self.h)
        return {KC_NAMES[k]: (t.launches[k], t.total_ms[k]) for k in range(len(KC_NAMES))}

    def reset_kernel_times(self):
        _check(self.lib.pd_reset_kernel_times(self.h), self.h)

    def operator_view(self) -> OperatorView:
        v = OperatorView()
        _check(self.lib.pd_get_operator_view(self.h, C.byref(v)), self.h)
        return v

    def apply_operator(self, d_x: int, d_y: int, d_dot: int | None = None):
        """y = A x on device vectors given as raw device pointers (slot order)."""
        _check(self.lib.pd_apply_operator(self.h, C.c_void_p(d_x), C.c_void_p(d_y),
                                          C.c_void_p(d_dot) if d_dot else None), self.h)

    # learned warm start
    def ws_set_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        _check(self.lib.pd_ws_set_params(self.h, _fp(p), p.size), self.h)

    def ws_get_params(self) -> np.ndarray:
        p = np.zeros(mlp_param_count(), np.float32)
        _check(self.lib.pd_ws_get_params(self.h, _fp(p), p.size), self.h)
        return p

    def ws_collect(self, samples_per_step: int, capacity: int):
        _check(self.lib.pd_ws_collect(self.h, samples_per_step, capacity), self.h)

    def ws_dataset(self, max_rows: int = 1 << 22):
        rows = C.c_longlong()
        _check(self.lib.pd_ws_dataset(self.h, None, None, 0, C.byref(rows)), self.h)
        X = np.zeros((max_rows if max_rows else 1, 64), np.float32)
        T = np.zeros((max_rows if max_rows else 1, 3), np.float32)
        _check(self.lib.pd_ws_dataset(self.h, _fp(X), _fp(T), max_rows, C.byref(rows)), self.h)
        return X[:rows.value], T[:rows.value]

    # DataIO (src/core/dataIO.h:20-44): frames / sim_info / checkpoints under run.saving_path
    def dataIO_getDataAndWrite(self):
        _check(self.lib.pd_dataio_get_data_and_write(self.h), self.h)

    def dataIO_newFrame(self):
        _check(self.lib.pd_dataio_new_frame(self.h), self.h)

    def dataIO_savedFrame(self) -> int:
        v = C.c_size_t()
        _check(self.lib.pd_dataio_saved_frame(self.h, C.byref(v)), self.h)
        return v.value

    def dataIO_saveState(self, timestep: int):
        _check(self.lib.pd_dataio_save_state(self.h, int(timestep)), self.h)

    def dataIO_saveStateReference(self, timestep: int):
        """saveState in the reference's own layout (STATE/state.<step>)."""
        _check(self.lib.pd_dataio_save_state_reference(self.h, C.c_size_t(timestep)), self.h)

    def dataIO_loadStateReference(self, timestep: int):
        """loadState of a file in the reference's own layout (STATE/state.<step>)."""
        _check(self.lib.pd_dataio_load_state_reference(self.h, C.c_size_t(timestep)), self.h)

    def dataIO_loadState(self, timestep: int):
        _check(self.lib.pd_dataio_load_state(self.h, int(timestep)), self.h)

    def stream_handle(self) -> int:
        """cudaStream_t of this simulator, as an integer (for CUDA events)."""
        v = C.c_void_p()
        _check(self.lib.pd_get_stream(self.h, C.byref(v)), self.h)
        return v.value or 0

    def synchronize(self):
        _check(self.lib.pd_synchronize(self.h), self.h)

    def sph_collide(self, sph_pos, sph_vel, slip: float = 1.0) -> int:
        """SPH <-> PD collision (collideDifferentParticles) of the caller's SPH
        particles: (n, 4) float64 arrays of positions and velocities in
        internal units, corrected in place; the PD velocities of the handle
        are updated.  Returns the number of SPH particles corrected."""
        pos = np.ascontiguousarray(sph_pos, dtype=np.float64)
        vel = np.ascontiguousarray(sph_vel, dtype=np.float64)
        if pos.shape != vel.shape or pos.ndim != 2 or pos.shape[1] != 4:
            raise ValueError("sph_pos and sph_vel must be (n, 4) float64 arrays")
        c = C.c_int()
        _check(self.lib.pd_sph_collide(self.h, pos.ctypes.data_as(C.POINTER(C.c_double)),
                                       vel.ctypes.data_as(C.POINTER(C.c_double)), pos.shape[0], float(slip),
                                       C.byref(c)), self.h)
        if pos is not sph_pos:
            sph_pos[...] = pos
        if vel is not sph_vel:
            sph_vel[...] = vel
        return c.value

    def launch_count(self) -> int:
        v = C.c_longlong()
        _check(self.lib.pd_get_launch_count(self.h, C.byref(v)), self.h)
        return v.value


def _bcheck(status, batch=None):
    if status != PD_OK:
        lib = library(False)
        msg = lib.pd_batch_last_error_message(batch)
        raise PdError(status, msg.decode() if msg else "")


class Batch:
    """Many independent scenes stepped together (pd_batch_*, no reference
    counterpart).  Each scene has the parameter surface of one Simulator;
    per-scene exports and statistics answer as that Simulator would.

        b = Batch(device=0)
        k = b.add_scene(sim, run, options, pos4, vel4, activity, s0=None)
        b.makeReady(); b.advance(100); b.get(k, VAR_POSITION)
    """

    def __init__(self, device: int = 0, options: BatchOptions | None = None):
        self.lib = library()
        if options is None:
            options = BatchOptions()
            self.lib.pd_batch_options_default(C.byref(options))
        self.options = options
        h = C.c_void_p()
        _bcheck(self.lib.pd_batch_create(int(device), C.byref(options), C.byref(h)))
        self.h = h
        self.sizes = []

    def close(self):
        if getattr(self, "h", None):
            self.lib.pd_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, sim: SimulationParameters, run: RunningParameters, options: SolverOptions | None,
                  pos4, vel4=None, activity=None, s0=None) -> int:
        dp = C.POINTER(C.c_double)
        opts = options if options is not None else default_options()
        k = C.c_int()
        _bcheck(self.lib.pd_batch_add_scene(self.h, C.byref(sim), C.byref(run), C.byref(opts), C.byref(k)), self.h)
        n = int(sim.num_pd_particle)
        pos = np.ascontiguousarray(pos4, np.float64).reshape(n, 4)
        vel = np.ascontiguousarray(vel4 if vel4 is not None else np.zeros((n, 4)), np.float64).reshape(n, 4)
        act = np.ascontiguousarray(activity if activity is not None else np.zeros(n), np.int32)
        _bcheck(self.lib.pd_batch_set_particles(self.h, k.value, pos.ctypes.data_as(dp), vel.ctypes.data_as(dp),
                                                act.ctypes.data_as(C.POINTER(C.c_int32)), n), self.h)
        if s0 is not None:
            s = np.ascontiguousarray(s0, np.float64)
            _bcheck(self.lib.pd_batch_set_stretch_limits(self.h, k.value, s.ctypes.data_as(dp), n), self.h)
        self.sizes.append(n)
        return k.value

    def ws_set_params(self, params):
        """Parameters of the batch's warm-start network (options.warm_start = 1)."""
        p = np.ascontiguousarray(params, np.float32)
        _bcheck(self.lib.pd_batch_ws_set_params(self.h, _fp(p), p.size), self.h)

    def makeReady(self):
        _bcheck(self.lib.pd_batch_make_ready(self.h), self.h)

    def advance(self, nsteps: int = 1):
        _bcheck(self.lib.pd_batch_advance(self.h, int(nsteps)), self.h)

    def scene_count(self) -> int:
        v = C.c_int()
        _bcheck(self.lib.pd_batch_scene_count(self.h, C.byref(v)), self.h)
        return v.value

    def offsets(self) -> np.ndarray:
        n = self.scene_count()
        out = np.zeros(n + 1, np.int64)
        _bcheck(self.lib.pd_batch_scene_offsets(self.h, out.ctypes.data_as(C.POINTER(C.c_int64)), n + 1), self.h)
        return out

    def get(self, scene: int, var: int) -> np.ndarray:
        size = C.c_size_t()
        _bcheck(self.lib.pd_batch_get_size(self.h, scene, var, C.byref(size)), self.h)
        if var == VAR_BROKEN_MASK:
            out = np.zeros(size.value, np.uint8)
        elif var in (VAR_ACTIVITY, VAR_BOND_COUNT, VAR_BOND_LIST, VAR_SLOT_PERMUTATION):
            out = np.zeros(size.value // 4, np.int32)
        elif var == VAR_BOND_ROW_PTR:
            out = np.zeros(size.value // 8, np.int64)
        else:
            out = np.zeros(size.value // 8, np.float64)
        _bcheck(self.lib.pd_batch_get(self.h, scene, var, out.ctypes.data_as(C.c_void_p), size.value), self.h)
        if var in (VAR_POSITION, VAR_VELOCITY, VAR_FORCE, VAR_SOLUTION, VAR_POSITION_SCALED, VAR_ORIGINAL_POSITION):
            out = out.reshape(self.sizes[scene], 4)
        return out

    def alive_sets(self, scene: int):
        rp = self.get(scene, VAR_BOND_ROW_PTR)
        bl = self.get(scene, VAR_BOND_LIST)
        cnt = self.get(scene, VAR_BOND_COUNT)
        return [bl[rp[i]:rp[i] + cnt[i]] for i in range(self.sizes[scene])]

    def stats(self, scene: int) -> StepStats:
        s = StepStats()
        _bcheck(self.lib.pd_batch_get_stats(self.h, scene, C.byref(s)), self.h)
        return s

    def finished(self, scene: int) -> bool:
        v = C.c_int()
        _bcheck(self.lib.pd_batch_finished(self.h, scene, C.byref(v)), self.h)
        return bool(v.value)

    def config(self) -> BatchConfig:
        c = BatchConfig()
        _bcheck(self.lib.pd_batch_get_config(self.h, C.byref(c)), self.h)
        return c

    def launch_count(self) -> int:
        v = C.c_longlong()
        _bcheck(self.lib.pd_batch_get_launch_count(self.h, C.byref(v)), self.h)
        return v.value

    def stream_handle(self) -> int:
        v = C.c_void_p()
        _bcheck(self.lib.pd_batch_get_stream(self.h, C.byref(v)), self.h)
        return v.value or 0

    def synchronize(self):
        _bcheck(self.lib.pd_batch_synchronize(self.h), self.h)


class Scene:
    """The reference's example Scene (src/examples/scene.cpp) for PD particles:
    run.obj_file is scaled into the simulation box and filled with a lattice
    of spacing 2 r on the GPU.  Mirrors Scene(simParams, runningParams,
    arrangement) + initPeridynamicsParticles; sets simParams.num_pd_particle."""

    REGULAR_GRID = 0
    JITTERED_GRID = 1

    def __init__(self, simParams: SimulationParameters, runningParams: RunningParameters,
                 arrangement: int = 0, jitter_seed: int = 1):
        self.lib = library()
        h = C.c_void_p()
        st = self.lib.pd_scene_create(C.byref(simParams), C.byref(runningParams), int(arrangement),
                                      int(jitter_seed), C.byref(h))
        if st != PD_OK:
            msg = self.lib.pd_scene_last_error_message()
            raise PdError(st, msg.decode() if msg else "")
        self.h = h
        self.n = int(simParams.num_pd_particle)

    def close(self):
        if getattr(self, "h", None):
            self.lib.pd_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initPeridynamicsParticles(self):
        """(activity int32[n], positions double[n,4], velocities double[n,4])"""
        act = np.zeros(self.n, np.int32)
        pos = np.zeros((self.n, 4), np.float64)
        vel = np.zeros((self.n, 4), np.float64)
        dp = C.POINTER(C.c_double)
        _check(self.lib.pd_scene_init_pd_particles(self.h, act.ctypes.data_as(C.POINTER(C.c_int32)),
                                                   pos.ctypes.data_as(dp), vel.ctypes.data_as(dp)))
        return act, pos, vel
