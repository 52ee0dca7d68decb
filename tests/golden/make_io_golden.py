"""Generate the checkpoint/output golden files in tests/golden/io from the
reference's own routines (3D/MPI/OTvortex/bkup.hpp and dataio.hpp,
2D/SERIAL/OTvortex/dataio.hpp, compiled by oracle/build.py::build_ref_io).

Run here, where the reference tree is present:
    python tests/golden/make_io_golden.py
The 1D output format is written inline by the 1D driver's main
(1D/SERIAL/shock/main.cpp:171-184), not by a routine that can be compiled on
its own; its golden file is written with the restatement in oracle/dataio.py.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mlau_gb300 import ics  # noqa: E402
from oracle import build, dataio  # noqa: E402

OUT = os.path.join(HERE, "io")
VARS = ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")
KEEP = ("bkup_stamp.dat", "bkup_time.dat", "bkup_data_00000.dat", "outdat_00003_00000.dat",
        "outdat_00002.dat", "params.dat", "offsets.dat", "t.dat")


def ptrs(st):
    arr = (C.POINTER(C.c_double) * 8)()
    for i, k in enumerate(VARS):
        arr[i] = st[k].ctypes.data_as(C.POINTER(C.c_double))
    return arr


def collect(src, dst):
    os.makedirs(dst, exist_ok=True)
    for f in os.listdir(src):
        if f in KEEP:
            shutil.copy(os.path.join(src, f), os.path.join(dst, f))


def main():
    lib = C.CDLL(build.build_ref_io())
    d = C.c_double
    # 3D state: padded 14 x 13 x 12 cells (interior 6 x 5 x 4), seeded
    # random-phase ICs
    st, m = ics.turbulence_3d(n=6, ny=5, nz=4, mach=0.3, seed=17)
    st = {k: np.ascontiguousarray(v) for k, v in st.items()}
    nz, ny, nx = st["ro"].shape
    x, y, z = (np.arange(k, dtype=np.float64) for k in (nx, ny, nz))
    with tempfile.TemporaryDirectory() as tmp:
        lib.ref_bkup_save(tmp.encode(), 40, 3, d(0.123456789), d(1e-3), d(0.2), nx * ny * nz, 0,
                          ptrs(st))
        lib.ref_dataio_3d(tmp.encode(), 0, 3, d(0.125), 0, nx, ny, nz, 4, 4, 4, d(m["gamma"]),
                          ptrs(st), x.ctypes.data_as(C.POINTER(C.c_double)),
                          y.ctypes.data_as(C.POINTER(C.c_double)),
                          z.ctypes.data_as(C.POINTER(C.c_double)))
        lib.ref_dataio_3d(tmp.encode(), 1, 3, d(0.25), 0, nx, ny, nz, 4, 4, 4, d(m["gamma"]),
                          ptrs(st), x.ctypes.data_as(C.POINTER(C.c_double)),
                          y.ctypes.data_as(C.POINTER(C.c_double)),
                          z.ctypes.data_as(C.POINTER(C.c_double)))
        collect(tmp, os.path.join(OUT, "3d"))
    np.savez_compressed(os.path.join(OUT, "3d_meta.npz"), gamma=m["gamma"],
                        shape=np.array(st["ro"].shape))
    # 2D state, FP64 serial output
    st2, m2 = ics.turbulence_2d(n=8, ny=6, seed=18, vrms=0.7)
    st2 = {k: np.ascontiguousarray(v) for k, v in st2.items()}
    ny2, nx2 = st2["ro"].shape
    with tempfile.TemporaryDirectory() as tmp:
        lib.ref_dataio_2d(tmp.encode(), 0, 2, d(0.5), nx2, ny2, 4, 4, d(m2["gamma"]), ptrs(st2))
        lib.ref_dataio_2d(tmp.encode(), 1, 2, d(0.75), nx2, ny2, 4, 4, d(m2["gamma"]), ptrs(st2))
        collect(tmp, os.path.join(OUT, "2d"))
    np.savez_compressed(os.path.join(OUT, "2d_meta.npz"), gamma=m2["gamma"],
                        shape=np.array(st2["ro"].shape))
    # 1D: restated format (the reference writes it inline in its main)
    st1, m1 = ics.riemann_1d(n=24, seed=19)
    os.makedirs(os.path.join(OUT, "1d"), exist_ok=True)
    name, data = dataio.outdat_f64(st1, 5, 1)
    with open(os.path.join(OUT, "1d", name), "wb") as fh:
        fh.write(data)
    np.savez_compressed(os.path.join(OUT, "1d_state.npz"), **st1, bx=m1["bx"])
    print("wrote", OUT)


if __name__ == "__main__":
    main()
