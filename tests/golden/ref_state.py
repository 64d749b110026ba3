"""TEST INFRASTRUCTURE: the reference's checkpoint layout, restated.

DataIO::saveState / loadState (src/core/dataIO.cu:123-198) write a size_t
savedFrame, then every MemoryManager array in the order of its Variables enum
(src/core/memory_manager.h:29-90), each with the byte size that
MemoryManager's constructor gives it (src/core/memory_manager.cu:16-178):
real_t = double (src/core/definitions.h:33-39), MAX_PD_BOND_COUNT = 528,
Mat3x3 = 3 double3 (72 bytes), Clist = 128 + 1 + 7 ints
(definitions.h:99-101,137-147).  The counts come from the run's
SimulationParameters (DATA/sim_info.dat).  Positions (SPH and PD, PD sorted and
original) are stored multiplied by scaleFactor (memory_manager.cu:274-298).

`write` builds such a file from arrays (used to hand the oracle's state to the
library's reader); `read` parses one (used to check the library's writer).
"""
from __future__ import annotations

import numpy as np

VARIABLES = [
    "SPH_TIMESTEP", "SPH_ACTIVITY", "SPH_VALIDITY", "SPH_POSITION", "SPH_VELOCITY", "SPH_FORCE",
    "SPH_SORTED_POSITION", "SPH_SORTED_VELOCITY", "SPH_SORTED_DENSITY", "SPH_SORTED_DENSITY_NORMALIZED",
    "SPH_SORTED_PRESSURE", "SPH_BOUNDARY_POSITION",
    "PD_ACTIVITY", "PD_POSITION", "PD_POSITION_BACKUP", "PD_VELOCITY", "PD_VELOCITY_BACKUP", "PD_FORCE",
    "PD_SORTED_POSITION", "PD_SORTED_VELOCITY", "PD_ORIGINAL_POSITION", "PD_ORIGINAL_STRETCH",
    "PD_ORIGINAL_BOND_LIST_TOP", "PD_STRETCH", "PD_NEW_STRETCH", "PD_BOND_LIST", "PD_BOND_LIST_TOP",
    "PD_BOND_LIST_TOP_BACKUP", "PD_CLIST",
    "PD_SYSTEM_MATRIX", "PD_SYSTEM_VECTOR", "PD_SYSTEM_SOLUTION", "PD_HAS_BROKEN_BOND",
    "CELL_PARTICLE_TYPE",
    "SPH_PARTICLE_TO_CELL_HASH", "SPH_PARTICLE_UNSORTED_INDEX", "SPH_CELL_START_INDEX", "SPH_CELL_END_INDEX",
    "PD_PARTICLE_TO_CELL_HASH", "PD_PARTICLE_UNSORTED_INDEX", "PD_CELL_START_INDEX", "PD_CELL_END_INDEX",
]
MAX_BONDS = 528
MAT3X3 = 72
CLIST = (128 + 1 + 7) * 4
SCALED = {"SPH_POSITION", "SPH_SORTED_POSITION", "SPH_BOUNDARY_POSITION", "PD_POSITION", "PD_SORTED_POSITION",
          "PD_ORIGINAL_POSITION"}
# element layout of the PD arrays the tests read or write
REAL4 = {"PD_POSITION", "PD_POSITION_BACKUP", "PD_VELOCITY", "PD_VELOCITY_BACKUP", "PD_FORCE", "PD_SORTED_POSITION",
         "PD_SORTED_VELOCITY", "PD_ORIGINAL_POSITION", "PD_SYSTEM_VECTOR", "PD_SYSTEM_SOLUTION"}
REAL = {"PD_ORIGINAL_STRETCH", "PD_STRETCH", "PD_NEW_STRETCH"}
INT = {"PD_ACTIVITY", "PD_ORIGINAL_BOND_LIST_TOP", "PD_BOND_LIST_TOP", "PD_BOND_LIST_TOP_BACKUP", "PD_BOND_LIST"}


def sizes(num_sph, num_pd, num_cells, num_clists, plane):
    """Byte size of every variable (memory_manager.cu:16-178)."""
    sph4, sph8, sph32 = 4 * num_sph, 8 * num_sph, 32 * num_sph
    pd4, pd8, pd32 = 4 * num_pd, 8 * num_pd, 32 * num_pd
    c4 = 4 * num_cells
    s = {
        "SPH_TIMESTEP": sph4, "SPH_ACTIVITY": sph4, "SPH_VALIDITY": sph4,
        "SPH_POSITION": sph32, "SPH_VELOCITY": sph32, "SPH_FORCE": sph32, "SPH_SORTED_POSITION": sph32,
        "SPH_SORTED_VELOCITY": sph32, "SPH_SORTED_DENSITY": sph8, "SPH_SORTED_DENSITY_NORMALIZED": sph8,
        "SPH_SORTED_PRESSURE": sph8,
        "SPH_BOUNDARY_POSITION": 32 * (2 * (plane + 2) * (plane + 2) + 4 * plane * (plane + 1)),
        "PD_ACTIVITY": pd4, "PD_ORIGINAL_BOND_LIST_TOP": pd4, "PD_BOND_LIST_TOP": pd4, "PD_BOND_LIST_TOP_BACKUP": pd4,
        "PD_ORIGINAL_STRETCH": pd8, "PD_STRETCH": pd8, "PD_NEW_STRETCH": pd8,
        "PD_BOND_LIST": pd4 * MAX_BONDS, "PD_CLIST": CLIST * num_clists,
        "PD_SYSTEM_MATRIX": num_pd * MAX_BONDS * MAT3X3, "PD_HAS_BROKEN_BOND": 4,
        "CELL_PARTICLE_TYPE": c4, "SPH_PARTICLE_TO_CELL_HASH": sph4, "SPH_PARTICLE_UNSORTED_INDEX": sph4,
        "SPH_CELL_START_INDEX": c4, "SPH_CELL_END_INDEX": c4, "PD_PARTICLE_TO_CELL_HASH": pd4,
        "PD_PARTICLE_UNSORTED_INDEX": pd4, "PD_CELL_START_INDEX": c4, "PD_CELL_END_INDEX": c4,
    }
    for name in REAL4:
        s[name] = pd32
    assert set(s) == set(VARIABLES)
    return s


def offsets(sz):
    off, o = {}, 8   # savedFrame
    for name in VARIABLES:
        off[name] = o
        o += sz[name]
    return off, o


def _dtype(name):
    return np.int32 if name in INT else np.float64


def write(path, counts, scale, saved_frame, arrays):
    """arrays: name -> numpy array in the reference's element layout
    (REAL4: (n, 4) float64 in internal units, unscaled; REAL: (n,); INT: (n,),
    PD_BOND_LIST: (528 * n,) bond-major).  Missing variables are zeros."""
    sz = sizes(*counts)
    off, total = offsets(sz)
    with open(path, "wb") as f:
        f.write(np.uint64(saved_frame).tobytes())
        for name in VARIABLES:
            if name in arrays:
                a = np.ascontiguousarray(arrays[name], dtype=_dtype(name)).copy()
                if name in SCALED:
                    a = a.reshape(-1, 4)
                    a[:, :3] *= scale
                b = a.tobytes()
                assert len(b) == sz[name], (name, len(b), sz[name])
                f.write(b)
            else:
                f.seek(sz[name], 1)
        f.truncate(total)
    return total


def read(path, counts, scale):
    """name -> array for the PD variables of REAL4 / REAL / INT, plus
    'savedFrame' and 'file_size'."""
    sz = sizes(*counts)
    off, total = offsets(sz)
    raw = open(path, "rb").read()
    out = {"savedFrame": int(np.frombuffer(raw[:8], np.uint64)[0]), "file_size": len(raw), "expected_size": total}
    for name in REAL4 | REAL | INT:
        a = np.frombuffer(raw[off[name]:off[name] + sz[name]], dtype=_dtype(name)).copy()
        if name in REAL4:
            a = a.reshape(-1, 4)
            if name in SCALED:
                a[:, :3] /= scale
        out[name] = a
    return out
