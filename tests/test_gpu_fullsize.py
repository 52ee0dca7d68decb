"""The workloads at their full sizes, checked through size-independent
properties (the oracle is too slow there, except in 1D):

* periodic boxes conserve the totals of every conserved variable and of each
  face-B component exactly in exact arithmetic (flux-form update and CT curl
  telescope), so the totals may drift only by round-off;
* the CT update keeps the discrete div B at round-off;
* the FP32-split form stays within its L1 bound of the FP64 form;
* the 1D Riemann problem (2048 cells to t_end) is small enough to compare
  with the oracle bit for bit."""
import numpy as np
import pytest

import mlau_gb300 as M
from mlau_gb300 import ics

pytestmark = pytest.mark.gpu

CONSERVED = ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")


def totals(st, dim, off=4):
    core = (slice(off, -off),) * dim
    return {k: float(np.sum(st[k][core], dtype=np.float64)) for k in CONSERVED}


def drift(a, b, scale):
    """Change of each total relative to the sum of |value| (variables that are
    identically zero, such as Bz in the 2D box, are left out)."""
    return {k: abs(a[k] - b[k]) / scale[k] for k in a if scale[k] > 0}


def test_2d_512_1000_steps_conserves_and_keeps_div_b():
    """Config C1 at full size: 512^2, LHLLD + WCNS4 + CT + RK3, 1000 steps."""
    st, m = ics.turbulence_2d(n=512, seed=3, vrms=0.5)
    dt = 0.4 * m["dx"] / m["vfast"]
    t0 = totals(st, 2)
    scale = {k: np.abs(st[k][4:-4, 4:-4]).sum() for k in CONSERVED}
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"], gamma=m["gamma"], odr=4,
               flux="lhlld") as s:
        s.upload(st)
        s.step(dt, 1000)
        out = s.download()
    for k, v in out.items():
        assert np.isfinite(v).all(), k
    d = drift(totals(out, 2), t0, scale)
    assert max(d.values()) <= 1e-12, d
    assert ics.div_b_2d(out, m["dx"], m["dy"]) <= 1e-12


@pytest.mark.parametrize("n", (256, 384))
def test_3d_full_size_split_and_fp64(n):
    """Config C2 at 256^3 and 384^3: both forms conserve the totals and keep
    div B; the split density stays within its L1 bound of FP64."""
    st, m = ics.turbulence_3d(n=n, mach=1e-2, seed=8)
    dt = 0.4 * m["dx"] / m["vfast"]
    steps = 6 if n == 256 else 3
    t0 = totals(st, 3)
    core = (slice(4, -4),) * 3
    scale = {k: np.abs(st[k][core]).sum() for k in CONSERVED}
    out = {}
    for prec in (M.FP64, M.FP32_SPLIT):
        with M.Sim(3, st["ro"].shape, dx=m["dx"], dy=m["dy"], dz=m["dz"], odr=4, flux="mlau",
                   precision=prec) as s:
            s.upload(st)
            s.step(dt, steps)
            out[prec] = s.download()
        d = drift(totals(out[prec], 3), t0, scale)
        tol = 1e-12 if prec == M.FP64 else 1e-10
        assert max(d.values()) <= tol, (prec, d)
        assert ics.div_b_3d(out[prec], m["dx"], m["dy"], m["dz"]) <= 1e-12, prec
    a, b = out[M.FP32_SPLIT]["ro"][core], out[M.FP64]["ro"][core]
    assert np.abs(a - b).sum() / np.abs(b).sum() <= 1e-6


def test_1d_riemann_2048_to_t_end_equals_oracle(port):
    """Config C0 at full size: 2048 cells, MLAU + MUSCL + RK3, open
    boundaries, dt from the initial state, run to t_end = 0.1."""
    st, m = ics.riemann_1d(n=2048, seed=0)
    dt = port.dt1d(st, m["bx"], m["gamma"], 0.4, m["dx"])
    ref = ics.copy_state(st)
    t, n = 0.0, 0
    while t < 0.1:
        port.step1d(ref, m["bx"], dt, m["dx"], gamma=m["gamma"], odr=2, flux="mlau", nrk=3)
        t += dt
        n += 1
    with M.Sim(1, st["ro"].shape, dx=m["dx"], gamma=m["gamma"], odr=2, flux="mlau", nrk=3) as s:
        s.set_bx(m["bx"])
        s.set_bc("open")
        s.upload(st)
        dt_g, _ = s.cfl(0.4, m["dx"], 1.0, 0.0)
        assert dt_g == dt
        s.step(dt, n)
        got = s.download()
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k
