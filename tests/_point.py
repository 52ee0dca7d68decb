"""Seeded inputs and ctypes bindings for the point-function interface tests
(oracle/point_harness.cpp compiled against the reference's headers or
against include/mlau_point.h; tests/c/point_api.cu on the GPU).

Rows follow the harness layouts.  Every generator mixes generic states with
the cases the functions branch on: identical left/right states, zero normal
or tangential field, exact zeros across a stencil (the reconstruction's
exact-zero guard), degenerate eigen-systems, low Mach numbers, strong
compression for the shock sensor."""
import ctypes as C

import numpy as np

FLUXES = ("mlau", "lhlld", "hlld", "roe", "hl3d2")
INTERPS = ("muscl_mm_flr", "muscl_mc_flr", "muscl_kr_flr", "wcns3_flr", "wcns4_flr",
           "muscl_mm_f", "muscl_mc_f", "muscl_kr_f", "wcns3_f", "wcns4_f", "minmod", "minmod3",
           "max", "min")
EIGENS = ("st", "mi", "ae")
RECONSTS = ("c", "m", "a", "plain")
WIDTH = {"flux": (18, 7), "interp": (5, 2), "eigen": (9, 105), "reconst": (37, 14)}


def bind(path):
    lib = C.CDLL(path)
    dp, i, lng = C.c_void_p, C.c_int, C.c_long
    for fn in ("ph_flux", "ph_interp", "ph_eigen"):
        getattr(lib, fn).argtypes = [i, lng, dp, dp]
        getattr(lib, fn).restype = i
    lib.ph_reconst.argtypes = [i, i, lng, dp, dp]
    lib.ph_reconst.restype = i
    if hasattr(lib, "ph_flux_f"):
        lib.ph_flux_f.argtypes = [i, lng, dp, dp]
        lib.ph_flux_f.restype = i
    return lib


def run(lib, kind, which, rows, odr=4, fn=None):
    rows = np.ascontiguousarray(rows, dtype=np.float64)
    n = rows.shape[0]
    out = np.zeros((n, WIDTH[kind][1]))
    p = rows.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p)
    if kind == "reconst":
        rc = lib.ph_reconst(which, odr, n, *p)
    else:
        rc = getattr(lib, fn or f"ph_{kind}")(which, n, *p)
    assert rc == 0
    return out


def same(a, b):
    """Equal values, NaNs in the same places, and the same bits wherever the
    value is not NaN (so signed zeros must agree; NaN payloads may differ
    between machines)."""
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape or not np.array_equal(a, b, equal_nan=True):
        return False
    ok = ~np.isnan(a)
    return bool(np.array_equal(a[ok].view(np.uint64), b[ok].view(np.uint64)))


def _mix(rng, n):
    """Category of each row: 0 generic, 1..5 special cases."""
    return rng.choice(6, size=n, p=[0.5, 0.1, 0.1, 0.1, 0.1, 0.1])


def flux_inputs(n, seed):
    rng = np.random.default_rng(seed)
    r = np.empty((n, 18))
    for side in (0, 7):
        r[:, side] = rng.uniform(0.05, 2.0, n)                     # ro
        r[:, side + 1:side + 4] = rng.uniform(-2.0, 2.0, (n, 3))   # vn vt vu
        r[:, side + 4:side + 6] = rng.uniform(-2.0, 2.0, (n, 2))   # bt bu
        r[:, side + 6] = rng.uniform(0.02, 2.0, n)                 # pr
    r[:, 14] = rng.uniform(-2.0, 2.0, n)                           # bnc
    r[:, 15] = rng.choice([5 / 3, 1.4, 2.0], n)                    # gamma
    r[:, 16:18] = rng.uniform(-1.0, 1.0, (n, 2))                   # dv
    cat = _mix(rng, n)
    r[cat == 1, 7:14] = r[cat == 1, 0:7]                           # equal states
    r[cat == 2, 14] = 0.0                                          # no normal field
    r[np.ix_(cat == 3, [4, 5, 11, 12])] = 0.0                      # no tangential field
    low = cat == 4                                                 # low Mach
    r[np.ix_(low, [1, 2, 3, 8, 9, 10])] *= 1e-4
    r[np.ix_(low, [4, 5, 11, 12, 14])] *= 1e-3
    r[cat == 5, 16] = -rng.uniform(0.5, 3.0, (cat == 5).sum())     # strong compression
    r[cat == 5, 17] = -rng.uniform(0.5, 3.0, (cat == 5).sum())
    return r


def interp_inputs(n, seed):
    rng = np.random.default_rng(seed)
    r = rng.uniform(-1.0, 1.0, (n, 5))
    cat = _mix(rng, n)
    k = cat == 1                                                   # linear data
    r[k] = rng.uniform(-1, 1, (k.sum(), 1)) + np.arange(5) * rng.uniform(-1, 1, (k.sum(), 1))
    r[cat == 2, 1:4] = r[cat == 2, 2:3]                            # flat centre
    r[cat == 3] = 0.0                                              # all zero
    k = cat == 4                                                   # a single jump
    r[k] = np.where(np.arange(5) < rng.integers(1, 5, (k.sum(), 1)), 0.1, 1.0)
    r[cat == 5] *= 1e-12                                           # tiny differences
    return r


def eigen_inputs(n, seed):
    rng = np.random.default_rng(seed)
    r = np.empty((n, 9))
    r[:, 0] = rng.uniform(0.05, 2.0, n)
    r[:, 1:4] = rng.uniform(-2.0, 2.0, (n, 3))
    r[:, 4:7] = rng.uniform(-2.0, 2.0, (n, 3))
    r[:, 7] = rng.uniform(0.02, 2.0, n)
    r[:, 8] = rng.choice([5 / 3, 1.4, 2.0], n)
    cat = _mix(rng, n)
    r[np.ix_(cat == 1, [5, 6])] = 0.0                              # no tangential field
    r[cat == 2, 4] = 0.0                                           # no normal field
    k = cat == 3                                                   # a2 == ca2
    r[k, 7] = r[k, 4] ** 2 / r[k, 8]
    r[np.ix_(cat == 3, [5, 6])] = 0.0
    r[np.ix_(cat == 4, [4, 5, 6])] = 0.0                           # no field at all
    r[np.ix_(cat == 5, [5, 6])] *= 1e-7                            # nearly normal field
    return r


def reconst_inputs(n, seed):
    rng = np.random.default_rng(seed)
    r = np.empty((n, 37))
    centre = np.empty((n, 7))
    centre[:, 0] = rng.uniform(0.1, 2.0, n)
    centre[:, 1:4] = rng.uniform(-1.5, 1.5, (n, 3))
    centre[:, 4:6] = rng.uniform(-1.5, 1.5, (n, 2))
    centre[:, 6] = rng.uniform(0.05, 2.0, n)
    amp = rng.choice([1e-1, 1e-2, 1e-4], n)[:, None]
    for v in range(7):
        pert = rng.uniform(-1.0, 1.0, (n, 5)) * amp * (np.abs(centre[:, v:v + 1]) + 0.1)
        r[:, 5 * v:5 * v + 5] = centre[:, v:v + 1] + pert
    r[:, 0:5] = np.abs(r[:, 0:5])
    r[:, 30:35] = np.abs(r[:, 30:35])
    r[:, 35] = rng.uniform(-1.5, 1.5, n)                           # bx
    r[:, 36] = rng.choice([5 / 3, 1.4, 2.0], n)                    # gamma
    cat = _mix(rng, n)
    r[cat == 1, 10:15] = 0.0                                       # vy == 0 across the stencil
    r[cat == 2, 25:30] = 0.0                                       # bz == 0
    r[np.ix_(cat == 3, list(range(20, 30)))] = 0.0                 # no tangential field
    r[cat == 4, 35] = 0.0                                          # no normal field
    k = cat == 5                                                   # supersonic
    r[np.ix_(k, list(range(5, 10)))] *= 4.0
    return r


GENERATORS = {"flux": flux_inputs, "interp": interp_inputs, "eigen": eigen_inputs,
              "reconst": reconst_inputs}
