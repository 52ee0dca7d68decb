"""The 3D configuration at its full size and length: 256^3 periodic box,
MLAU + WCNS4 + CT + RK3, gamma 5/3, 200 steps at a fixed dt (CFL 0.4 of the
initial state), rms Mach 1e-2 and 1e-4.  Both FP32-split forms - float-float
state arithmetic (MLAU_FP32_SPLIT) and FP64 state arithmetic
(MLAU_FP32_SPLIT_F64) - run beside the plain FP64 form from the same seeded
state.

Tolerances: relative L1 of density <= 1e-6 against the FP64 form (the
workload's bound), and per-variable guards that catch regressions (energy
<= 1e-6, face B <= 1e-5, momenta <= 1e-4: at Mach 1e-4 the momenta are 1e-4 of
the sound speed, so their relative error is the largest); max |div B| * dx /
max |B| <= 1e-12 for every form."""
import numpy as np
import pytest

import mlau_gb300 as M
from mlau_gb300 import ics

pytestmark = pytest.mark.gpu

INT = (slice(4, -4),) * 3
VARS = ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")
BOUND = {"ro": 1e-6, "en": 1e-6, "bx": 1e-5, "by": 1e-5, "bz": 1e-5,
         "mx": 1e-4, "my": 1e-4, "mz": 1e-4}


def l1_rel(a, b):
    return float(np.abs(a[INT] - b[INT]).sum() / np.abs(b[INT]).sum())


def run(st, m, steps, dt, precision):
    with M.Sim(3, st["ro"].shape, dx=m["dx"], dy=m["dy"], dz=m["dz"], gamma=m["gamma"], odr=4,
               flux="mlau", nrk=3, precision=precision) as s:
        s.upload(st)
        s.step(dt, steps)
        return s.download()


@pytest.mark.parametrize("mach", (1e-2, 1e-4))
def test_256_cubed_200_steps_split_forms_vs_fp64(mach):
    st, m = ics.turbulence_3d(n=256, mach=mach, seed=8)
    dt = 0.4 * m["dx"] / m["vfast"]
    ref = run(st, m, 200, dt, M.FP64)
    assert ics.div_b_3d(ref, m["dx"], m["dy"], m["dz"]) <= 1e-12
    for prec in (M.FP32_SPLIT, M.FP32_SPLIT_F64):
        got = run(st, m, 200, dt, prec)
        err = {k: l1_rel(got[k], ref[k]) for k in VARS}
        for k in VARS:
            assert np.isfinite(got[k]).all(), (prec, k)
            assert err[k] <= BOUND[k], (prec, k, err)
        assert ics.div_b_3d(got, m["dx"], m["dy"], m["dz"]) <= 1e-12, prec
