"""FP32-split mode against the plain FP64 GPU path on the same inputs.

Both split forms: float-float state arithmetic (FP32_SPLIT) and FP64 state
arithmetic (FP32_SPLIT_F64).  Tolerance (stated by the workload spec):
relative L1 error of density <= 1e-6 with respect to the FP64 path; div B
stays at round-off because the CT curl differences the EMFs exactly (float-
float) or in FP64.  The other variables' L1 errors are checked against looser
per-variable bounds to catch regressions."""
import numpy as np
import pytest

import mlau_gb300 as M
from mlau_gb300 import ics

pytestmark = pytest.mark.gpu

RHO_L1_TOL = 1e-6
INT = (slice(4, -4),) * 3
SPLITS = (M.FP32_SPLIT, M.FP32_SPLIT_F64)


def l1_rel(a, b):
    return float(np.abs(a[INT] - b[INT]).sum() / np.abs(b[INT]).sum())


def run(st, m, steps, dt, precision, flux="mlau", odr=4):
    with M.Sim(3, st["ro"].shape, dx=m["dx"], dy=m["dy"], dz=m["dz"], odr=odr, flux=flux,
               precision=precision) as s:
        s.upload(st)
        s.step(dt, steps)
        return s.download()


@pytest.mark.parametrize("prec", SPLITS)
@pytest.mark.parametrize("flux", ("mlau", "lhlld"))
@pytest.mark.parametrize("mach", (1e-2, 1e-4))
def test_split_density_l1_vs_fp64(mach, flux, prec):
    """WCNS4 with MLAU or LHLLD: the sweep instances specialised for these
    schemes (packed FP32x2 reconstruction; MLAU also its packed flux)."""
    st, m = ics.turbulence_3d(n=32, mach=mach, seed=5)
    dt = 0.4 * m["dx"] / m["vfast"]
    ref = run(st, m, 50, dt, M.FP64, flux)
    got = run(st, m, 50, dt, prec, flux)
    err = {k: l1_rel(got[k], ref[k]) for k in ("ro", "en", "bx", "by", "bz")}
    assert err["ro"] <= RHO_L1_TOL, err
    assert err["en"] <= 1e-6 and max(err["bx"], err["by"], err["bz"]) <= 1e-5, err
    assert ics.div_b_3d(got, m["dx"], m["dy"], m["dz"]) <= 1e-12


@pytest.mark.parametrize("prec", SPLITS)
@pytest.mark.parametrize("flux", ("mlau", "lhlld", "hlld", "roe"))
def test_split_all_solvers_supersonic(flux, prec):
    """Mach ~1: the full 7-wave projection runs; states stay close to FP64."""
    st, m = ics.turbulence_3d(n=16, mach=1.0, seed=9)
    dt = 0.3 * m["dx"] / (m["vfast"] + 1.0)
    ref = run(st, m, 10, dt, M.FP64, flux)
    got = run(st, m, 10, dt, prec, flux)
    for k in ("ro", "en"):
        assert np.isfinite(got[k]).all()
        assert l1_rel(got[k], ref[k]) <= 1e-5, (k, l1_rel(got[k], ref[k]))


@pytest.mark.parametrize("prec", SPLITS)
@pytest.mark.parametrize("odr", (1, 2, 3, 5, 6))
def test_split_other_reconstructions(odr, prec):
    """Every reconstruction code (MUSCL minmod / MC / Koren, WCNS3, first
    order) in the split form stays close to FP64 and keeps div B."""
    st, m = ics.turbulence_3d(n=16, mach=0.3, seed=12 + odr, odr=odr)
    dt = 0.4 * m["dx"] / m["vfast"]
    ref = run(st, m, 10, dt, M.FP64, "lhlld", odr)
    got = run(st, m, 10, dt, prec, "lhlld", odr)
    assert l1_rel(got["ro"], ref["ro"]) <= RHO_L1_TOL, l1_rel(got["ro"], ref["ro"])
    assert ics.div_b_3d(got, m["dx"], m["dy"], m["dz"], odr=odr) <= 1e-12


@pytest.mark.parametrize("prec", SPLITS)
@pytest.mark.parametrize("shape", ((13, 11, 17), (21, 14, 9)))
def test_split_unaligned_grid(shape, prec):
    """Padded row lengths that are not multiples of 4: the FP32 scratch is
    pitched for the tensor maps; results stay close to FP64, ghosts periodic."""
    nx, ny, nz = shape
    st, m = ics.turbulence_3d(n=nx, ny=ny, nz=nz, mach=0.2, seed=31)
    dt = 0.4 * min(m["dx"], m["dy"], m["dz"]) / m["vfast"]
    ref = run(st, m, 8, dt, M.FP64)
    got = run(st, m, 8, dt, prec)
    assert l1_rel(got["ro"], ref["ro"]) <= RHO_L1_TOL
    assert ics.div_b_3d(got, m["dx"], m["dy"], m["dz"]) <= 1e-12
    for k, a in got.items():
        assert np.array_equal(np.pad(a[INT], 4, mode="wrap"), a), k


@pytest.mark.parametrize("prec", SPLITS)
def test_split_ghosts_are_periodic_images(prec):
    st, m = ics.turbulence_3d(n=12, mach=0.1, seed=2)
    got = run(st, m, 3, 1e-3, prec)
    for k, a in got.items():
        inner = a[INT]
        assert np.array_equal(np.pad(inner, 4, mode="wrap"), a), k


def dropin_steps(st, m, prec, nrk, calls):
    nz, ny, nx = st["ro"].shape
    M.set_scheme(3, 4, "mlau", nrk)
    M.set_precision(3, prec)
    try:
        for _ in range(calls):
            M.mhd_fd_ct_3d(*[st[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")],
                           1e-3, m["dx"], m["dy"], m["dz"], nx, ny, nz, 4, 4, 4, m["gamma"])
    finally:
        M.set_precision(3, M.FP64)
        M.set_scheme(3, 4, "mlau", 3)
        M.release_dropin()


@pytest.mark.parametrize("shape,prec", [((12, 16, 16), M.FP32_SPLIT), ((16, 16, 16), M.FP32_SPLIT),
                                        ((24, 16, 40), M.FP32_SPLIT), ((32, 32, 32), M.FP32_SPLIT),
                                        ((72, 24, 20), M.FP32_SPLIT), ((136, 12, 16), M.FP32_SPLIT),
                                        ((24, 16, 40), M.FP32_SPLIT_F64),
                                        ((72, 24, 20), M.FP32_SPLIT_F64)])
def test_split_dropin_driver(shape, prec):
    """mhd_fd_ct_3d in FP32-split mode runs the step over z-plane ranges so
    that its host copies overlap the first and last RK stages (1, 2, 4 and 8
    slabs here; the plan is checked on the CPU by tests/test_slab_plan.py);
    two calls in a row equal two handle-API steps bit for bit."""
    nzi, nyi, nxi = shape
    st, m = ics.turbulence_3d(n=nxi, ny=nyi, nz=nzi, mach=1e-2, seed=4)
    ref = run(st, m, 2, 1e-3, prec)
    dropin_steps(st, m, prec, 3, 2)
    for k in ref:
        assert np.array_equal(st[k], ref[k]), k


@pytest.mark.parametrize("nrk", (1, 2))
def test_split_dropin_driver_other_rk(nrk):
    """The same with RK1 (uploads and downloads in one stage) and RK2."""
    st, m = ics.turbulence_3d(n=20, ny=24, nz=72, mach=1e-2, seed=6)
    with M.Sim(3, st["ro"].shape, dx=m["dx"], dy=m["dy"], dz=m["dz"], odr=4, flux="mlau",
               nrk=nrk, precision=M.FP32_SPLIT) as s:
        s.upload(st)
        s.step(1e-3, 2)
        ref = s.download()
    dropin_steps(st, m, M.FP32_SPLIT, nrk, 2)
    for k in ref:
        assert np.array_equal(st[k], ref[k]), k
