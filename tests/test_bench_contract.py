"""bench.py's reference arm (the CPU oracle timed on the host cores) keeps
the one-line JSON contract: the GPU arm's metric and unit, impl "reference",
a cpu_baseline describing the run, and an e2e entry with no device copies.
Runs on a small workload so that it finishes in seconds without a GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--n", "8000"], capture_output=True, text=True, timeout=600,
                         env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("implicit steps/s") and d["unit"] == "steps/s"
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_does_not_load_the_gpu_library():
    """The reference arm builds its scene with lattice.py alone: the package,
    and with it libpd_gb300.so, is never loaded in that process."""
    code = ("import sys; sys.argv=['bench.py']; sys.path.insert(0, %r); import bench; "
            "bench.main(['--impl', 'reference', '--steps', '1', '--warmup', '0', '--n', '3000']); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPPED' if 'libpd_gb300' in maps else 'NOT_MAPPED'); "
            "print('IMPORTED' if any(m.startswith('sci-solver_peridynamic_gb300') for m in sys.modules) "
            "else 'NOT_IMPORTED')" % ROOT)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT,
                         env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert out.returncode == 0, out.stderr[-2000:]
    assert "NOT_MAPPED" in out.stdout and "NOT_IMPORTED" in out.stdout, out.stdout[-500:]


def test_reference_arm_scene_is_the_package_scene(pdgb, scenes):
    """lattice.py + oracle.params_from_body give the oracle exactly the arrays
    and parameters that the package's ellipsoid scene maps to."""
    from oracle import oracle as O
    from helpers import oracle_params
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    body = bench.lattice_module().ellipsoid_impact(target_n=5000, gap=0.0)
    sc = scenes.ellipsoid_impact(target_n=5000, gap=0.0)
    assert np.array_equal(body["pos"], sc.pos) and np.array_equal(body["vel"], sc.vel)
    assert np.array_equal(body["act"], sc.act)
    a, b = O.params_from_body(body), oracle_params(sc)
    for name, _ in O.PdoParams._fields_:
        va, vb = getattr(a, name), getattr(b, name)
        if hasattr(va, "__len__"):
            va, vb = list(va), list(vb)
        assert va == vb, name
