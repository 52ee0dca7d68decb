"""GPU parity: the FP64 plain path through the C ABI against the CPU oracle
and the reference's golden vectors.  The bar is equal values (the plain path
reproduces the reference's arithmetic bit for bit; +0/-0 compare equal), which
is stricter than the rel. L-inf 1e-12 (one step) / 1e-9 (1000 steps) budget."""
import itertools

import numpy as np
import pytest

import mlau_gb300 as M
from _util import equal_values, golden_cases, load_golden, max_rel_diff
from mlau_gb300 import ics

pytestmark = pytest.mark.gpu

ORDERS = (1, 2, 3, 4, 5, 6)  # 5, 6: MUSCL with the MC / Koren limiter
FLUXES = ("mlau", "lhlld", "hlld", "roe")


def gpu_run(dim, st, steps, dt, **kw):
    bx = kw.pop("bx", None)
    bc = kw.pop("bc", None)
    tables = kw.pop("tables", None)
    eig = kw.pop("eig", "full")
    with M.Sim(dim, st["ro"].shape, **kw) as s:
        s.set_eigen(eig)
        if tables is not None and dim == 3:
            s.set_bc3d(*tables)
        if bx is not None:
            s.set_bx(bx)
        if bc is not None:
            s.set_bc(bc)
        if tables is not None and dim == 2:
            s.set_bc2d(*tables)
        s.upload(st)
        s.step(dt, steps)
        return s.download()


# --- golden vectors made by the reference itself -------------------------------
@pytest.mark.parametrize("name", golden_cases("3d"))
def test_golden_3d(name):
    prm, s, outs = load_golden(name)
    for n, ref in outs.items():
        tables = (prm["dnx"], prm["dny"], prm["dnz"]) if "dnx" in prm else None
        got = gpu_run(3, s, n, prm["dt"], dx=prm["dx"], dy=prm.get("dy", prm["dx"]),
                      dz=prm.get("dz", prm["dx"]), gamma=prm["gamma"], odr=prm["odr"],
                      flux=prm["flux"], eig=prm.get("eig", "full"), tables=tables)
        assert equal_values(got, ref), f"{name} after {n} steps: {max_rel_diff(got, ref)}"


@pytest.mark.parametrize("name", golden_cases("2d"))
def test_golden_2d(name):
    prm, s, outs = load_golden(name)
    for n, ref in outs.items():
        tables = (prm["dnx"], prm["dny"]) if "dnx" in prm else None
        got = gpu_run(2, s, n, prm["dt"], dx=prm["dx"], dy=prm.get("dy", prm["dx"]),
                      gamma=prm["gamma"], odr=prm["odr"], flux=prm["flux"], tables=tables,
                      eig=prm.get("eig", "full"))
        assert equal_values(got, ref), f"{name} after {n} steps: {max_rel_diff(got, ref)}"


@pytest.mark.parametrize("name", golden_cases("1d"))
def test_golden_1d(name):
    prm, s, outs = load_golden(name)
    for n, ref in outs.items():
        got = gpu_run(1, s, n, prm["dt"], dx=prm["dx"], gamma=prm["gamma"], odr=prm["odr"],
                      flux=prm["flux"], bx=prm["bx"], bc=prm["bc"], eig=prm.get("eig", "full"))
        assert equal_values(got, ref, keys=ref.keys()), f"{name} after {n} steps"


# --- oracle sweeps over every order x solver -----------------------------------
@pytest.mark.parametrize("odr,flux", list(itertools.product(ORDERS, FLUXES)))
def test_3d_vs_oracle(port, odr, flux):
    st, m = ics.turbulence_3d(n=8, ny=10, nz=6, mach=0.8, seed=odr * 11 + len(flux), odr=odr)
    ref = ics.copy_state(st)
    for _ in range(2):
        port.step3d(ref, 1e-3, m["dx"], m["dy"], m["dz"], odr=odr, flux=flux)
    got = gpu_run(3, st, 2, 1e-3, dx=m["dx"], dy=m["dy"], dz=m["dz"], odr=odr, flux=flux)
    assert equal_values(got, ref), max_rel_diff(got, ref)


@pytest.mark.parametrize("odr,flux", list(itertools.product(ORDERS, FLUXES)))
def test_2d_vs_oracle(port, odr, flux):
    st, m = ics.turbulence_2d(n=24, ny=18, seed=odr + 2 * len(flux), odr=odr, vrms=1.3)
    ref = ics.copy_state(st)
    for _ in range(3):
        port.step2d(ref, 2e-3, m["dx"], m["dy"], odr=odr, flux=flux)
    got = gpu_run(2, st, 3, 2e-3, dx=m["dx"], dy=m["dy"], odr=odr, flux=flux)
    assert equal_values(got, ref), max_rel_diff(got, ref)


@pytest.mark.parametrize("bc", ("open", "periodic"))
@pytest.mark.parametrize("odr,flux", list(itertools.product(ORDERS, FLUXES)))
def test_1d_vs_oracle(port, odr, flux, bc):
    st, m = ics.riemann_1d(n=96, seed=odr * 3 + len(flux))
    dt = port.dt1d(st, m["bx"], m["gamma"], 0.4, m["dx"])
    ref = ics.copy_state(st)
    for _ in range(8):
        port.step1d(ref, m["bx"], dt, m["dx"], gamma=m["gamma"], odr=odr, flux=flux, bc=bc)
    got = gpu_run(1, st, 8, dt, dx=m["dx"], gamma=m["gamma"], odr=odr, flux=flux, bx=m["bx"],
                  bc=bc)
    assert equal_values(got, ref, keys=ref.keys())


@pytest.mark.parametrize("bc", ("open", "periodic"))
@pytest.mark.parametrize("nrk", (1, 2, 3))
def test_1d_rk_orders_graphs_and_timing(port, nrk, bc):
    """1D with RK1-3: 20 steps (16 of them from a captured step graph, in
    which the open boundary runs on a forked stream) and the same 20 steps
    with per-kernel timing on (the open boundary in line) equal the oracle."""
    st, m = ics.riemann_1d(n=80, seed=40 + nrk)
    dt = port.dt1d(st, m["bx"], m["gamma"], 0.4, m["dx"])
    ref = ics.copy_state(st)
    for _ in range(20):
        port.step1d(ref, m["bx"], dt, m["dx"], gamma=m["gamma"], odr=2, flux="mlau", nrk=nrk,
                    bc=bc)
    for timing in (False, True):
        with M.Sim(1, st["ro"].shape, dx=m["dx"], gamma=m["gamma"], odr=2, flux="mlau",
                   nrk=nrk) as s:
            s.set_bx(m["bx"])
            s.set_bc(bc)
            s.upload(st)
            s.set_timing(timing)
            s.step(dt, 20)
            got = s.download()
        assert equal_values(got, ref, keys=ref.keys()), (timing, max_rel_diff(got, ref))


@pytest.mark.parametrize("nrk", (1, 2, 3))
def test_3d_rk_orders(port, nrk):
    st, m = ics.turbulence_3d(n=8, mach=0.4, seed=21)
    ref = ics.copy_state(st)
    port.step3d(ref, 1e-3, m["dx"], m["dy"], m["dz"], nrk=nrk)
    got = gpu_run(3, st, 1, 1e-3, dx=m["dx"], dy=m["dy"], dz=m["dz"], nrk=nrk)
    assert equal_values(got, ref)


def test_3d_inconsistent_ghosts(port):
    """Ghost cells that are not periodic images: the GPU must read exactly the
    cells the reference reads (raw ghosts for primitives, images for cell B)."""
    st, m = ics.turbulence_3d(n=8, mach=0.5, seed=13)
    rng = np.random.default_rng(0)
    for k in st:
        a = st[k].copy()
        a[:, :, :4] *= 1 + 1e-3 * rng.random(a[:, :, :4].shape)
        a[-4:] *= 1 + 1e-3 * rng.random(a[-4:].shape)
        st[k] = np.ascontiguousarray(a)
    ref = ics.copy_state(st)
    port.step3d(ref, 1e-3, m["dx"], m["dy"], m["dz"])
    got = gpu_run(3, st, 1, 1e-3, dx=m["dx"], dy=m["dy"], dz=m["dz"])
    assert equal_values(got, ref)


def test_3d_minimum_interior(port):
    """Interior width equal to the ghost depth (the smallest the fill allows)."""
    st, m = ics.turbulence_3d(n=4, ny=5, nz=4, mach=0.3, seed=17)
    ref = ics.copy_state(st)
    port.step3d(ref, 1e-3, m["dx"], m["dy"], m["dz"])
    got = gpu_run(3, st, 1, 1e-3, dx=m["dx"], dy=m["dy"], dz=m["dz"])
    assert equal_values(got, ref)


def test_3d_many_steps_low_mach(port):
    """40 steps at Mach 1e-2: still equal values (budget: rel 1e-9 at 1000)."""
    st, m = ics.turbulence_3d(n=12, mach=1e-2, seed=3)
    dt = 0.4 * m["dx"] / m["vfast"]
    ref = ics.copy_state(st)
    for _ in range(40):
        port.step3d(ref, dt, m["dx"], m["dy"], m["dz"])
    got = gpu_run(3, st, 40, dt, dx=m["dx"], dy=m["dy"], dz=m["dz"])
    assert equal_values(got, ref), max_rel_diff(got, ref)
    assert ics.div_b_3d(got, m["dx"], m["dy"], m["dz"]) <= 1e-12


def test_2d_many_steps(port):
    st, m = ics.turbulence_2d(n=48, seed=8)
    dt = 0.4 * m["dx"] / m["vfast"]
    ref = ics.copy_state(st)
    for _ in range(100):
        port.step2d(ref, dt, m["dx"], m["dy"])
    got = gpu_run(2, st, 100, dt, dx=m["dx"], dy=m["dy"], flux="lhlld")
    assert equal_values(got, ref), max_rel_diff(got, ref)
    assert not got["mz"].any() and not got["bz"].any()
    assert ics.div_b_2d(got, m["dx"], m["dy"]) <= 1e-12


def test_3d_1000_steps_with_cfl_dt(port):
    """1000 RK3 steps of the 3D driver's time loop (CFL dt every step) against
    the oracle: equal values (budget: rel. L-inf 1e-9), div B at round-off."""
    st, m = ics.turbulence_3d(n=12, mach=0.3, seed=21)
    ref = ics.copy_state(st)
    dr = min(m["dx"], m["dy"], m["dz"])
    with M.Sim(3, st["ro"].shape, dx=m["dx"], dy=m["dy"], dz=m["dz"], flux="mlau") as s:
        s.upload(st)
        dt_g = dt_c = 0.0
        for n in range(1000):
            dt_g, _ = s.cfl(0.4, dr, m["vfast"], dt_g)
            dt_c = port.cfl3d(ref, 0.4, dr, m["vfast"], dt_c)[0]
            assert dt_g == dt_c, n
            s.step(dt_g, 1)
            port.step3d(ref, dt_c, m["dx"], m["dy"], m["dz"], flux="mlau")
        got = s.download()
    assert max_rel_diff(got, ref) <= 1e-9
    assert equal_values(got, ref), max_rel_diff(got, ref)
    assert ics.div_b_3d(got, m["dx"], m["dy"], m["dz"]) <= 1e-12


def test_2d_1000_steps_with_cfl_dt(port):
    st, m = ics.turbulence_2d(n=32, ny=24, seed=22, vrms=0.8)
    ref = ics.copy_state(st)
    dr = min(m["dx"], m["dy"])
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"], flux="lhlld") as s:
        s.upload(st)
        dt_g = dt_c = 0.0
        for n in range(1000):
            dt_g, _ = s.cfl(0.4, dr, 0.0, dt_g)
            dt_c = port.cfl2d(ref, 0.4, dr, 0.0, dt_c)[0]
            assert dt_g == dt_c, n
            s.step(dt_g, 1)
            port.step2d(ref, dt_c, m["dx"], m["dy"], flux="lhlld")
        got = s.download()
    assert max_rel_diff(got, ref) <= 1e-9
    assert equal_values(got, ref), max_rel_diff(got, ref)
    assert ics.div_b_2d(got, m["dx"], m["dy"]) <= 1e-12


# --- CFL reduction -------------------------------------------------------------
def test_cfl_3d(port):
    st, m = ics.turbulence_3d(n=16, mach=0.6, seed=4)
    with M.Sim(3, st["ro"].shape, dx=m["dx"], dy=m["dy"], dz=m["dz"]) as s:
        s.upload(st)
        for vfast in (0.0, 1e6):
            dt, vm = s.cfl(0.4, m["dx"], vfast, 7.0)
            dt_o, vm_o = port.cfl3d(st, 0.4, m["dx"], vfast, 7.0)
            assert dt == dt_o and vm == vm_o


def test_cfl_2d_and_1d(port):
    st, m = ics.turbulence_2d(n=32, seed=4, vrms=1.1)
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"]) as s:
        s.upload(st)
        dt, vm = s.cfl(0.4, m["dx"], 0.0, 1.0)
        dt_o, vm_o = port.cfl2d(st, 0.4, m["dx"], 0.0, 1.0)
        assert dt == dt_o and vm == vm_o
    st, m = ics.riemann_1d(n=128, seed=4)
    with M.Sim(1, st["ro"].shape, dx=m["dx"], gamma=m["gamma"]) as s:
        s.set_bx(m["bx"])
        s.upload(st)
        dt, _ = s.cfl(0.4, m["dx"], 1.0)
        assert dt == port.dt1d(st, m["bx"], m["gamma"], 0.4, m["dx"])


def test_cfl_ignores_nan_cells(port):
    st, m = ics.turbulence_3d(n=8, mach=0.3, seed=6)
    st["ro"][6, 6, 6] = np.nan
    with M.Sim(3, st["ro"].shape, dx=m["dx"], dy=m["dy"], dz=m["dz"]) as s:
        s.upload(st)
        dt, vm = s.cfl(0.4, m["dx"], 0.0, 1.0)
    dt_o, vm_o = port.cfl3d(st, 0.4, m["dx"], 0.0, 1.0)
    assert dt == dt_o and vm == vm_o


# --- drop-in drivers (reference names, host arrays) ------------------------------
def test_dropin_3d(port):
    st, m = ics.turbulence_3d(n=8, mach=0.5, seed=31)
    nz, ny, nx = st["ro"].shape
    M.set_scheme(3, 4, "mlau", 3)
    ref = ics.copy_state(st)
    port.step3d(ref, 1e-3, m["dx"], m["dy"], m["dz"], odr=4, flux="mlau")
    M.mhd_fd_ct_3d(*[st[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")], 1e-3,
                   m["dx"], m["dy"], m["dz"], nx, ny, nz, 4, 4, 4, m["gamma"])
    assert equal_values(st, ref)


def test_dropin_3d_rejects_multirank():
    st, m = ics.turbulence_3d(n=4, mach=0.5, seed=1)
    nz, ny, nx = st["ro"].shape
    before = ics.copy_state(st)
    with pytest.raises(M.MlauError):
        M.mhd_fd_ct_3d(*[st[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")], 1e-3,
                       m["dx"], m["dy"], m["dz"], nx, ny, nz, 4, 4, 4, m["gamma"], 0, 2, 1, 1)
    assert equal_values(st, before)


def test_dropin_2d_and_1d(port):
    st, m = ics.turbulence_2d(n=24, seed=6)
    ny, nx = st["ro"].shape
    M.set_scheme(2, 4, "lhlld", 3)
    ref = ics.copy_state(st)
    port.step2d(ref, 1e-3, m["dx"], m["dy"], odr=4, flux="lhlld")
    M.mhd_fd_ct_2d(*[st[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")], 1e-3,
                   m["dx"], m["dy"], nx, ny, 4, 4, m["gamma"])
    assert equal_values(st, ref)
    st, m = ics.riemann_1d(n=64, seed=6)
    M.set_scheme(1, 2, "mlau", 3)
    M.set_bc_1d("open")
    dt = port.dt1d(st, m["bx"], m["gamma"], 0.4, m["dx"])
    ref = ics.copy_state(st)
    port.step1d(ref, m["bx"], dt, m["dx"], gamma=m["gamma"], odr=2, flux="mlau")
    M.mhd_fd4c_1d(*[st[k] for k in ("ro", "mx", "my", "mz", "en", "by", "bz")], m["bx"], dt,
                  m["dx"], st["ro"].shape[0], 4, m["gamma"])
    assert equal_values(st, ref)


@pytest.mark.parametrize("odr,flux", list(itertools.product(ORDERS, FLUXES)))
def test_miyoshi_vs_oracle(port, odr, flux):
    """Miyoshi's eigen-system (the headers' mhd_m_reconst) where the drivers
    use the full one, 3D, 2D and 1D, supersonic states; the oracle is pinned
    to the reference built with the call swapped in."""
    st, m = ics.turbulence_3d(n=10, ny=9, nz=8, mach=1.2, seed=odr * 5 + len(flux), odr=odr)
    ref = ics.copy_state(st)
    for _ in range(2):
        port.step3d(ref, 1e-3, m["dx"], m["dy"], m["dz"], odr=odr, flux=flux, eig="miyoshi")
    got = gpu_run(3, st, 2, 1e-3, dx=m["dx"], dy=m["dy"], dz=m["dz"], odr=odr, flux=flux,
                  eig="miyoshi")
    assert equal_values(got, ref, equal_nan=(flux == "roe")), max_rel_diff(got, ref)
    st, m = ics.turbulence_2d(n=24, ny=18, seed=odr + 7, odr=odr, vrms=1.5)
    ref = ics.copy_state(st)
    for _ in range(3):
        port.step2d(ref, 2e-3, m["dx"], m["dy"], odr=odr, flux=flux, eig="miyoshi")
    got = gpu_run(2, st, 3, 2e-3, dx=m["dx"], dy=m["dy"], odr=odr, flux=flux, eig="miyoshi")
    assert equal_values(got, ref, equal_nan=(flux == "roe")), max_rel_diff(got, ref)
    st, m = ics.riemann_1d(n=64, seed=odr * 7 + len(flux))
    v = st["mx"] / st["ro"]  # a uniform flow of 3 on top: supersonic cells
    st["en"] = st["en"] + 0.5 * st["ro"] * ((v + 3.0) ** 2 - v ** 2)
    st["mx"] = st["ro"] * (v + 3.0)
    dt = port.dt1d(st, m["bx"], m["gamma"], 0.4, m["dx"])
    ref, full = ics.copy_state(st), ics.copy_state(st)
    for _ in range(5):
        port.step1d(ref, m["bx"], dt, m["dx"], gamma=m["gamma"], odr=odr, flux=flux,
                    eig="miyoshi")
        port.step1d(full, m["bx"], dt, m["dx"], gamma=m["gamma"], odr=odr, flux=flux)
    assert not equal_values(ref, full, equal_nan=True)
    got = gpu_run(1, st, 5, dt, dx=m["dx"], gamma=m["gamma"], odr=odr, flux=flux, bx=m["bx"],
                  bc="open", eig="miyoshi")
    assert equal_values(got, ref, keys=ref.keys(), equal_nan=(flux == "roe"))


def test_miyoshi_refused_for_split():
    st, m = ics.turbulence_3d(n=8, mach=0.5, seed=1)
    with M.Sim(3, st["ro"].shape, dx=m["dx"], dy=m["dy"], dz=m["dz"],
               precision=M.FP32_SPLIT) as s:
        with pytest.raises(M.MlauError, match="FP64"):
            s.set_eigen("miyoshi")

