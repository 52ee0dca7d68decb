"""Generate tests/golden/point_api.npz from the reference's own point-function
headers.

Run here, where the reference tree is present:
    python tests/golden/make_point_golden.py
It compiles oracle/point_harness.cpp against the reference's
include/interp.h, mhd_eigen.h and mhd_flux.h (oracle/build.py), runs every
function on seeded inputs (tests/_point.py) and stores the inputs and the
reference's outputs.  tests/test_point_api.py and tests/test_gpu_point_api.py
compare include/mlau_point.h with them, on the host and in device code.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import _point as P  # noqa: E402
from oracle import build  # noqa: E402

SIZES = {"flux": 600, "interp": 400, "eigen": 60, "reconst": 300}
ODRS = (2, 4)  # reconstruction codes stored for the reconstructions
SEED = 20240


def main():
    ref = P.bind(build.build_point_harness("ref"))
    out = {}
    for kind, names in (("flux", P.FLUXES), ("interp", P.INTERPS), ("eigen", P.EIGENS)):
        rows = P.GENERATORS[kind](SIZES[kind], SEED)
        out[f"{kind}_in"] = rows
        out[f"{kind}_out"] = np.stack([P.run(ref, kind, w, rows) for w in range(len(names))])
    rows = P.reconst_inputs(SIZES["reconst"], SEED)
    out["reconst_in"] = rows
    out["reconst_odr"] = np.array(ODRS)
    out["reconst_out"] = np.stack([np.stack([P.run(ref, "reconst", w, rows, odr)
                                             for odr in ODRS]) for w in range(len(P.RECONSTS))])
    path = os.path.join(HERE, "point_api.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
