"""Count the reference algorithm's FP64 operations per zone-update, per phase.
TEST/MEASUREMENT INFRASTRUCTURE ONLY.

    python oracle/opcount.py   # prints JSON and rewrites mlau_gb300/opcounts.json

The counts come from oracle/opcount.cpp: the oracle's C restatement of the
reference driver compiled with a counting `double`.  Phases: prim (cell B +
primitives), aux (CT weights + shock sensors), rec (characteristic
reconstruction incl. the CT central-part interpolation), flux (Riemann solver
+ central/upwind split), emf (edge EMF), update (RK combine + CT curl).
Figures are per interior zone and per full RK step (all stages), and the
reconstruction/flux figures are also given per cell / face per sweep.
"""
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
PHASES = ("prim", "aux", "rec", "flux", "emf", "update")
OUT = os.path.join(ROOT, "mlau_gb300", "opcounts.json")


def build():
    so = os.path.join(HERE, "_build", "libopcount.so")
    src = os.path.join(HERE, "opcount.cpp")
    deps = [src, os.path.join(HERE, "mlau_oracle.c"), os.path.join(HERE, "oracle_point.h")]
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(d) for d in deps):
        os.makedirs(os.path.dirname(so), exist_ok=True)
        subprocess.run(["g++", "-O1", "-fPIC", "-shared", "-ffp-contract=off", "-w",
                        "-I" + HERE, "-o", so, src], check=True)
    return so


def count_3d(n=16, mach=1e-2, odr=4, flux=0, nrk=3, seed=0):
    from mlau_gb300 import ics
    st, m = ics.turbulence_3d(n=n, mach=mach, seed=seed, odr=odr)
    lib = C.CDLL(build())
    arrs = [st[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")]
    ptrs = (C.POINTER(C.c_double) * 8)(*[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs])
    out = np.zeros(32, dtype=np.int64)
    nz, ny, nx = st["ro"].shape
    lib.opcount_step3d(ptrs, C.c_double(0.3 * m["dx"] / m["vfast"]), C.c_double(m["dx"]), nx, ny,
                       nz, 4, C.c_double(m["gamma"]), odr, flux, nrk,
                       out.ctypes.data_as(C.POINTER(C.c_longlong)))
    ops = out.reshape(8, 4)
    zones = n ** 3
    res = {"config": f"3D {n}^3 interior (+4 ghosts), mach={mach}, odr={odr}, flux={flux}, nrk={nrk}",
           "per_zone_update": {}, "padded_cells": nx * ny * nz, "zones": zones}
    for p, name in enumerate(PHASES):
        add, mul, div, sq = (int(x) for x in ops[p])
        res["per_zone_update"][name] = {"add": add / zones, "mul": mul / zones, "div": div / zones,
                                        "sqrt": sq / zones, "total": (add + mul + div + sq) / zones}
    res["per_zone_update"]["all"] = sum(v["total"] for v in res["per_zone_update"].values())
    # per cell / face and sweep: the reference reconstructs len-4 cells and
    # evaluates len-5 faces per pencil, 3 sweeps x nrk stages
    npen = (nx * ny * nz) / nx
    rec_cells = 3 * nrk * npen * (nx - 4)
    faces = 3 * nrk * npen * (nx - 5)
    r = ops[2].sum()
    f = ops[3].sum()
    res["rec_per_cell"] = float(r) / rec_cells
    res["flux_per_face"] = float(f) / faces
    return res


def count_2d(n=64, vrms=0.5, odr=4, flux=1, nrk=3, seed=0):
    """2D periodic box of the random-phase recipe (LHLLD + WCNS4 by default)."""
    from mlau_gb300 import ics
    st, m = ics.turbulence_2d(n=n, seed=seed, odr=odr, vrms=vrms)
    lib = C.CDLL(build())
    arrs = [st[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")]
    ptrs = (C.POINTER(C.c_double) * 8)(*[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs])
    out = np.zeros(32, dtype=np.int64)
    ny, nx = st["ro"].shape
    lib.opcount_step2d(ptrs, C.c_double(0.3 * m["dx"] / m["vfast"]), C.c_double(m["dx"]), nx, ny,
                       4, C.c_double(m["gamma"]), odr, flux, nrk,
                       out.ctypes.data_as(C.POINTER(C.c_longlong)))
    ops = out.reshape(8, 4)
    zones = n ** 2
    res = {"config": f"2D {n}^2 interior (+4 ghosts), vrms={vrms}, odr={odr}, flux={flux}, nrk={nrk}",
           "per_zone_update": {}, "padded_cells": nx * ny, "zones": zones}
    for p, name in enumerate(PHASES):
        add, mul, div, sq = (int(x) for x in ops[p])
        res["per_zone_update"][name] = {"add": add / zones, "mul": mul / zones, "div": div / zones,
                                        "sqrt": sq / zones, "total": (add + mul + div + sq) / zones}
    res["per_zone_update"]["all"] = sum(v["total"] for v in res["per_zone_update"].values())
    npen = ny
    res["rec_per_cell"] = float(ops[2].sum()) / (2 * nrk * npen * (nx - 4))
    res["flux_per_face"] = float(ops[3].sum()) / (2 * nrk * npen * (nx - 5))
    return res


if __name__ == "__main__":
    out = {"method": "oracle/opcount.cpp: reference algorithm with a counting double; "
                     "div and sqrt count 1, compares/min/max/fabs not counted",
           "mlau_wcns4_lowmach": count_3d(n=16, mach=1e-2, odr=4, flux=0),
           "mlau_wcns4_mach1": count_3d(n=16, mach=1.5, odr=4, flux=0, seed=1)}
    for fl, name in ((1, "lhlld"), (2, "hlld"), (3, "roe")):
        out[f"{name}_wcns4_lowmach"] = count_3d(n=16, mach=1e-2, odr=4, flux=fl)
    out["lhlld_wcns4_2d"] = count_2d(n=64, vrms=0.5, odr=4, flux=1)
    txt = json.dumps(out, indent=1)
    print(txt)
    with open(OUT, "w") as fh:
        fh.write(txt + "\n")
