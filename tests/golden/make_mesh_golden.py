"""Golden fixtures of the example-scene mesh fill, from the reference itself.

Builds procedural closed meshes (written here as OBJ text: a subdivided
icosahedron, a torus and a box written with quad faces, a star-shaped blob),
runs the reference's own Scene (src/examples/scene.cpp with mesh_query0.1's
point_inside_mesh, compiled on the host into oracle/_ref/libpdscene.so by
oracle/build_ref.sh) and stores the OBJ text, the parameters and the
resulting particles in tests/golden/mesh_fill.npz.

    PD_REFERENCE_ROOT=<reference root> bash oracle/build_ref.sh && python tests/golden/make_mesh_golden.py
"""
from __future__ import annotations

import ctypes
import math
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "libpdscene.so")


def obj_text(verts, faces):
    lines = ["# procedural mesh"]
    lines += ["v %.9g %.9g %.9g" % tuple(v) for v in verts]
    lines += ["f " + " ".join(str(i + 1) for i in f) for f in faces]
    return "\n".join(lines) + "\n"


def icosphere(levels=2):
    t = (1.0 + 5 ** 0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    v = [np.array(p, float) / np.linalg.norm(p) for p in v]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(levels):
        mid = {}
        nf = []

        def m(a, b):
            k = (min(a, b), max(a, b))
            if k not in mid:
                p = (v[a] + v[b]) / 2
                v.append(p / np.linalg.norm(p))
                mid[k] = len(v) - 1
            return mid[k]
        for a, b, c in f:
            ab, bc, ca = m(a, b), m(b, c), m(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    return [tuple(p) for p in v], f


def torus(R=1.0, r=0.35, nu=40, nv=20):
    verts, faces = [], []
    for i in range(nu):
        for j in range(nv):
            u, w = 2 * math.pi * i / nu, 2 * math.pi * j / nv
            verts.append(((R + r * math.cos(w)) * math.cos(u), (R + r * math.cos(w)) * math.sin(u), r * math.sin(w)))
    for i in range(nu):
        for j in range(nv):
            a, b = i * nv + j, ((i + 1) % nu) * nv + j
            c, d = ((i + 1) % nu) * nv + (j + 1) % nv, i * nv + (j + 1) % nv
            faces.append((a, b, c, d))   # quads: the OBJ reader splits them into fans
    return verts, faces


def box():
    v = [(x, y, z) for z in (0, 1) for y in (0, 1) for x in (0, 1)]
    f = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    return v, f


def blob(seed=3):
    v, f = icosphere(3)
    rng = np.random.default_rng(seed)
    k = rng.normal(size=(6, 3))
    out = []
    for p in v:
        p = np.array(p)
        s = 1.0 + 0.25 * sum(math.sin(3 * float(kk @ p)) for kk in k) / 6
        out.append(tuple(p * s))
    return out, f


def reference_fill(lib, obj, bmin, bmax, radius, scale_factor, translation, v0, arrangement):
    f = lib.ref_scene_fill
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_double,
                  ctypes.c_double, ctypes.POINTER(ctypes.c_float), ctypes.c_float, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_int]
    bm = (ctypes.c_double * 3)(*bmin)
    bM = (ctypes.c_double * 3)(*bmax)
    tr = (ctypes.c_float * 3)(*translation)
    libc = ctypes.CDLL(None)
    libc.srand(1)   # the stream of a process that never called srand
    n = f(obj.encode(), bm, bM, radius, scale_factor, tr, v0, arrangement, None, None, 0)
    pos = np.zeros((n, 4))
    vel = np.zeros((n, 4))
    libc.srand(1)
    f(obj.encode(), bm, bM, radius, scale_factor, tr, v0, arrangement, pos.ctypes.data, vel.ctypes.data, n)
    return pos, vel


CASES = [
    # name, mesh, box min, box max, radius, scaleFactor, translation, initial velocity, arrangement
    ("icosphere", icosphere(2), (0.0, 0.0, 0.0), (2.0, 2.0, 4.0), 0.02, 80.0, (8.0, 4.0, 16.0), -1.5, 0),
    ("torus_quads", torus(), (0.0, 0.0, 0.0), (2.0, 2.0, 4.0), 0.015, 1.0, (0.0, 0.0, 0.0), 0.0, 0),
    ("box_on_lattice", box(), (0.0, 0.0, 0.0), (2.0, 2.0, 4.0), 0.02, 1.0, (0.0, 0.0, 0.0), 0.0, 0),
    ("blob_offset_box", blob(), (-1.0, 0.5, -0.25), (1.5, 2.5, 3.0), 0.0125, 1.0, (0.0, 0.0, 0.0), 2.0, 0),
    ("icosphere_jittered", icosphere(2), (0.0, 0.0, 0.0), (2.0, 2.0, 4.0), 0.02, 1.0, (0.0, 0.0, 0.0), 0.0, 1),
]


def main():
    lib = ctypes.CDLL(LIB)
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for name, (verts, faces), bmin, bmax, radius, sf, tr, v0, arr in CASES:
            text = obj_text(verts, faces)
            path = os.path.join(td, name + ".obj")
            with open(path, "w") as fh:
                fh.write(text)
            pos, vel = reference_fill(lib, path, bmin, bmax, radius, sf, tr, v0, arr)
            out[name + "/obj"] = np.frombuffer(text.encode(), np.uint8)
            out[name + "/params"] = np.array(list(bmin) + list(bmax) + [radius, sf] + list(tr) + [v0, arr], float)
            out[name + "/pos"] = pos
            out[name + "/vel"] = vel
            print(name, "faces", len(faces), "particles", pos.shape[0])
    np.savez_compressed(os.path.join(HERE, "mesh_fill.npz"), **out)


if __name__ == "__main__":
    main()
