"""Host-side logic, no GPU: the C ABI library loads and exports every entry
point declared in include/pd_gb300.h; parameter derivation follows
SystemParameter; the s0 stream matches glibc's rand() after srand(1973);
the adaptive time-step state machine; failure of device calls without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(pd_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(pdgb):
    lib = pdgb.library()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version(pdgb):
    assert pdgb.library().pd_abi_version() == 5


def test_params_file_and_derivation(pdgb, tmp_path):
    """Keys of the reference's params.txt; derived values of
    calculateDependentParameters (parameters.cu:351-453)."""
    f = tmp_path / "params.txt"
    f.write_text("\n".join([
        "gpu_device 0", "adaptive_integration 1 ", "num_pd_particle 10000", "pd_stretch_limit_s0 1e-3",
        "steps_per_frame 10", "final_step 100", "radius_pd_over_sph 1", "boundary_min_x 0", "boundary_min_y 0",
        "boundary_min_z 0", "boundary_max_x 2", "boundary_max_y 2", "boundary_max_z 4", "sph_kernel_coeff 4.001",
        "pd_kernel_coeff 5.001", "pd_particle_mass 1000", "// a comment line", "", "integrator newmark_beta",
        "sph_sph_viscosity 1e-5",
    ]))
    sp = pdgb.SystemParameter(str(f))
    s, r = sp.getSimulationParameters(), sp.getRunningParameters()
    assert r.adaptive_integration == 1 and r.step_per_frame == 10 and r.final_step == 100
    assert r.integrator == pdgb.NEWMARK_BETA
    assert r.pd_stretch_limit_s0 == np.float32(1e-3)
    cell = float(np.float32(max(np.float32(2 / 32), np.float32(2 / 32), np.float32(4 / 64))))
    sph_r = cell / 4.001
    rad = 1.0 * sph_r
    scale = 2 * rad / 0.0005
    assert s.cell_size == cell / scale
    assert s.pd_particle_radius == rad / scale
    assert s.pd_horizon == rad * 5.001 / scale
    assert s.pd_C_times_V == 18.0 / 3.14159265358979323846264 / 2.0 / 1296.0 / rad
    assert s.scaleFactor == scale
    assert s.boundary_max_z == 4 / scale
    assert s.pd_time_step == 128 and s.num_pd_particle == 10000


def test_params_missing_file(pdgb):
    with pytest.raises(pdgb.PdError) as e:
        pdgb.SystemParameter("/nonexistent/params.txt")
    assert e.value.status == 6


def test_stretch_stream_matches_glibc_rand(pdgb, oracle_mod):
    """pd_sample_stretch_limits restates glibc's rand(); the oracle calls the
    C library's rand() after srand(1973) (simulator.cu:802-822, 852-857)."""
    for s0 in (1e-3, 0.015, 0.02):
        a = pdgb.sample_stretch_limits(s0, 5000)
        b = oracle_mod.sample_stretch(5000, float(np.float32(s0)))
        np.testing.assert_array_equal(a, b)
    libc = ctypes.CDLL(None)
    libc.srand(1973)
    raw = [libc.rand() for _ in range(24)]
    s = sum(x / 2147483647.0 for x in raw[:12]) - 6.0
    assert pdgb.sample_stretch_limits(0.02, 2)[0] == (s * 0.01 + 1.0) * float(np.float32(0.02))


def reference_decide(has_broken, ticks, substep, base=128, tmin=100, maxsub=10):
    """simulator.cu:339-392 restated."""
    if has_broken:
        if ticks > tmin:
            return ticks // 2, substep, True
        substep = 1
    else:
        if substep > 0:
            substep += 1
        if substep >= maxsub:
            ticks *= 2
            substep = 0 if ticks >= base else 1
    return ticks, substep, False


def test_adaptive_state_machine(pdgb):
    rng = np.random.default_rng(0)
    t, s = 128, 0
    tr, sr = 128, 0
    for _ in range(2000):
        hb = bool(rng.random() < 0.15)
        t, s, rb = pdgb.adaptive_decide(hb, t, s)
        tr, sr, rbr = reference_decide(hb, tr, sr)
        assert (t, s, rb) == (tr, sr, rbr)
    assert pdgb.adaptive_decide(True, 128, 0) == (64, 0, True)
    assert pdgb.adaptive_decide(True, 64, 0) == (64, 1, False)
    t, s = 64, 1
    for _ in range(9):
        t, s, _ = pdgb.adaptive_decide(False, t, s)
    assert (t, s) == (128, 0)


def test_no_gpu_fails_loudly(pdgb, scenes):
    """Without a CUDA device the product path raises; there is no CPU fallback."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    sc = scenes.reference_block(n_side=3)
    with pytest.raises(pdgb.PdError) as e:
        scenes.make_simulator(sc)
    assert e.value.status == 5
    with pytest.raises(pdgb.PdError) as e:
        pdgb.Batch(0)
    assert e.value.status == 5


@pytest.mark.parametrize("field,value", [("spmv_path", 4), ("spmv_path", -1), ("lanes_per_particle", 6), ("spmv_unroll", 3)])
def test_invalid_spmv_options_rejected(pdgb, scenes, field, value):
    """Option checks run before any device call: an unsupported SpMV shape is
    an invalid argument (status 1), not a silent default."""
    sc = scenes.reference_block(n_side=3)
    setattr(sc.opt, field, value)
    with pytest.raises(pdgb.PdError) as e:
        scenes.make_simulator(sc)
    assert e.value.status == 1
    assert "SpMV options" in str(e.value)


@pytest.mark.parametrize("field,value", [("warm_start", 4), ("warm_start", -1), ("history_size", 9)])
def test_invalid_warm_start_rejected(pdgb, scenes, field, value):
    sc = scenes.reference_block(n_side=3)
    setattr(sc.opt, field, value)
    with pytest.raises(pdgb.PdError) as e:
        scenes.make_simulator(sc)
    assert e.value.status == 1
    assert "warm_start" in str(e.value)


@pytest.mark.parametrize("field,value", [("preconditioner", 3), ("preconditioner", -1)])
def test_invalid_preconditioner_rejected(pdgb, scenes, field, value):
    sc = scenes.reference_block(n_side=3)
    setattr(sc.opt, field, value)
    with pytest.raises(pdgb.PdError) as e:
        scenes.make_simulator(sc)
    assert e.value.status == 1
    assert "preconditioner" in str(e.value)


@pytest.mark.parametrize("field,value", [("cg_loop", 2), ("cg_loop", -1), ("cg_check_interval", -3)])
def test_invalid_cg_loop_rejected(pdgb, scenes, field, value):
    sc = scenes.reference_block(n_side=3)
    setattr(sc.opt, field, value)
    with pytest.raises(pdgb.PdError) as e:
        scenes.make_simulator(sc)
    assert e.value.status == 1
    assert "cg_loop" in str(e.value)


def test_solver_option_cg_loop_default(pdgb):
    """The graph-driven CG loop is the default."""
    assert pdgb.default_options().cg_loop == 0


def test_batch_scene_sizes():
    """The batched workload: 64 bodies, log-uniform sizes in [4096, 65536]
    (about 1.4M particles), horizons 4/5/6, impact speeds 1-10 m/s."""
    import importlib
    scenes = importlib.import_module("sci-solver_peridynamic_gb300.scenes")
    lst = scenes.batched_scenes()
    ns = np.array([sc.n for sc in lst])
    assert len(lst) == 64 and 1.2e6 < ns.sum() < 1.6e6
    assert ns.min() >= 0.9 * 4096 and ns.max() <= 1.1 * 65536
    assert {sc.info["coeff"] for sc in lst} == {4.0, 5.0, 6.0}
    assert {sc.info["shape"] for sc in lst} == {"block", "ball"}
    assert all(1.0 <= sc.info["speed"] <= 10.0 for sc in lst)


def test_solver_option_defaults(pdgb):
    o = pdgb.default_options()
    assert o.cg_relative_tolerance == 1e-20 and o.cg_max_iterations == 100000
    assert o.time_step_base == 1.0 / 8388608.0 and o.time_step_min == 100 and o.max_substep == 10
    assert o.phase_in_steps == 30 and o.pd_k == 5.0 * 2.94315e9 and o.max_bonds_per_particle == 528
    assert tuple(o.gravity) == (0.0, -9.8, 0.0) and o.restitution == 0.001


def test_mesh_fill_golden_pinned_to_reference():
    """The mesh-fill fixtures are the reference's own Scene output; where the
    host build of the reference is present, regenerate and compare."""
    import importlib.util
    path = os.path.join(os.path.dirname(__file__), "golden", "mesh_fill.npz")
    g = np.load(path)
    names = sorted({k.split("/")[0] for k in g.files})
    assert len(names) >= 5
    for n in names:
        assert g[n + "/pos"].shape[1] == 4 and g[n + "/pos"].shape[0] > 1000
    lib = os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref", "libpdscene.so")
    if not os.path.exists(lib):
        pytest.skip("host build of the reference scene not present")
    spec = importlib.util.spec_from_file_location("make_mesh_golden",
                                                  os.path.join(os.path.dirname(__file__), "golden",
                                                               "make_mesh_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    import ctypes
    import tempfile
    L = ctypes.CDLL(lib)
    with tempfile.TemporaryDirectory() as td:
        for name, (verts, faces), bmin, bmax, radius, sf, tr, v0, arr in mg.CASES:
            p = os.path.join(td, name + ".obj")
            with open(p, "w") as fh:
                fh.write(mg.obj_text(verts, faces))
            pos, vel = mg.reference_fill(L, p, bmin, bmax, radius, sf, tr, v0, arr)
            np.testing.assert_array_equal(pos, g[name + "/pos"])
            np.testing.assert_array_equal(vel, g[name + "/vel"])


def test_struct_mirrors_match_the_c_layout(pdgb):
    """The ctypes mirrors are as large as the C structs: the library's default
    fillers write the whole struct, so a mirror that is too short would let
    them write past it.  Each call gets a buffer of the mirror's size plus a
    sentinel tail, which must come back untouched, and the last field of each
    struct must be written (a mirror that is too long would leave it at the
    sentinel)."""
    import ctypes as C
    lib = pdgb.library()
    tail = 64
    cases = [(pdgb.SolverOptions, lib.pd_solver_options_default, "history_size", 0)]
    for cls, fn, last, expect in cases:
        size = C.sizeof(cls)
        buf = (C.c_ubyte * (size + tail))(*([0xA5] * (size + tail)))
        assert fn(C.cast(buf, C.POINTER(cls))) == 0
        assert bytes(buf[size:]) == bytes([0xA5] * tail), cls.__name__
        obj = cls.from_buffer(buf)
        assert getattr(obj, last) == expect, (cls.__name__, last)
    # the simulation and running parameters are filled together
    sim_cls, run_cls = pdgb.SimulationParameters, pdgb.RunningParameters
    sbuf = (C.c_ubyte * (C.sizeof(sim_cls) + tail))(*([0xA5] * (C.sizeof(sim_cls) + tail)))
    rbuf = (C.c_ubyte * (C.sizeof(run_cls) + tail))(*([0xA5] * (C.sizeof(run_cls) + tail)))
    assert lib.pd_params_default(C.cast(sbuf, C.POINTER(sim_cls)), C.cast(rbuf, C.POINTER(run_cls))) == 0
    assert bytes(sbuf[C.sizeof(sim_cls):]) == bytes([0xA5] * tail)
    assert bytes(rbuf[C.sizeof(run_cls):]) == bytes([0xA5] * tail)


def test_reference_state_layout_restatement(tmp_path):
    """The restated reference checkpoint layout (tests/golden/ref_state.py):
    every MemoryManager variable has a size, the PD-only sizes follow
    memory_manager.cu (528 bond slots, 72-byte Mat3x3 blocks), and a file
    written with it reads back."""
    import numpy as np
    from golden import ref_state
    n, cells = 10, 7
    sz = ref_state.sizes(0, n, cells, 0, 0)
    assert len(sz) == len(ref_state.VARIABLES) == 42
    assert sz["PD_BOND_LIST"] == 4 * 528 * n and sz["PD_SYSTEM_MATRIX"] == 72 * 528 * n
    assert sz["SPH_BOUNDARY_POSITION"] == 32 * 8 and sz["PD_CELL_END_INDEX"] == 4 * cells
    rng = np.random.default_rng(1)
    pos = np.zeros((n, 4))
    pos[:, :3] = rng.standard_normal((n, 3))
    top = np.arange(n, dtype=np.int32)
    path = tmp_path / "state.1"
    total = ref_state.write(path, (0, n, cells, 0, 0), 2.5, 7, {"PD_POSITION": pos, "PD_BOND_LIST_TOP": top})
    d = ref_state.read(path, (0, n, cells, 0, 0), 2.5)
    assert d["file_size"] == total and d["savedFrame"] == 7
    np.testing.assert_allclose(d["PD_POSITION"], pos, rtol=1e-15)
    np.testing.assert_array_equal(d["PD_BOND_LIST_TOP"], top)
