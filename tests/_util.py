"""Helpers shared by the tests: golden fixtures and state comparison."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
OFF = 4


def golden_cases(prefix):
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def load_golden(name):
    """(params dict, input state, {nsteps: output state}) with ghosts rebuilt."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    dim = int(z["dim"]) if "dim" in z.files else int(name[0])
    prm = {k: (z[k].item() if z[k].ndim == 0 else z[k]) for k in z.files
           if not (k.startswith("in_") or k.startswith("out"))}

    whole = "dnx" in z.files  # cases with boundary tables store whole arrays

    def state(prefix):
        s = {}
        for k in z.files:
            if k.startswith(prefix):
                a = z[k]
                if dim > 1 and not whole:
                    a = np.pad(a, OFF, mode="wrap")
                s[k[len(prefix):]] = np.ascontiguousarray(a, dtype=np.float64)
        return s

    outs = {}
    for k in z.files:
        if k.startswith("out") and k.endswith("_ro"):
            n = int(k[3:k.index("_")])
            outs[n] = state(f"out{n}_")
    return prm, state("in_"), outs


def equal_values(a, b, keys=None, equal_nan=False):
    """True when every array holds the same values (+0 and -0 compare equal;
    with equal_nan, NaNs in the same places also compare equal)."""
    keys = keys or b.keys()
    return all(np.array_equal(a[k], b[k], equal_nan=equal_nan) for k in keys)


def max_rel_diff(a, b, keys=None):
    keys = keys or b.keys()
    w = 0.0
    for k in keys:
        scale = max(np.abs(b[k]).max(), 1e-300)
        w = max(w, float(np.abs(a[k] - b[k]).max() / scale))
    return w
