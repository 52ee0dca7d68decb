"""The MRX problem's operators on the GPU (resistive diffusion of the CT field
with its energy flux, viscosity; 2D/MPI/MRX/mhd_fd_ct_2d.c:726-1174) against
the oracle, which is pinned bit for bit to the reference's MRX driver file
(tests/test_oracle.py and the mrx2d_* golden vectors), plus the loop of the
MRX problem at its full size through size-independent properties."""
import ctypes as C
import itertools

import numpy as np
import pytest

import mlau_gb300 as M
from _util import equal_values, golden_cases, load_golden, max_rel_diff
from mlau_gb300 import ics

pytestmark = pytest.mark.gpu

TABLES = [
    ((0,) * 8, (0,) * 8),
    ics.MRX_TABLES,
    ((1, -1, 1, 1, 1, -1, 1, 1), (0,) * 8),
    ((1, -1, 1, 1, 1, -1, 1, 1), (1, 1, -1, 1, 1, 1, -1, 1)),
    ((1,) * 8, (-1,) * 8),
]


def state(odr, seed, tables, port, n=22, ny=16):
    st, m = ics.turbulence_2d(n=n, ny=ny, seed=seed, odr=odr, vrms=0.4)
    port.setbc2d(st, *tables)
    dt = 0.3 * m["dx"] / m["vfast"]
    return st, m, dt, 0.06 * m["dx"] ** 2 / dt


@pytest.mark.parametrize("tables", TABLES)
@pytest.mark.parametrize("odr,nrk", list(itertools.product((1, 2, 3, 4, 5, 6), (1, 2, 3))))
@pytest.mark.parametrize("op", ("resistive", "viscous"))
def test_operator_vs_oracle(port, op, odr, nrk, tables):
    st, m, dt, coef = state(odr, odr * 11 + nrk, tables, port)
    ref = ics.copy_state(st)
    kw = dict(gamma=m["gamma"], odr=odr, nrk=nrk, dnx=tables[0], dny=tables[1])
    for _ in range(3):
        getattr(port, op + "2d")(ref, coef, dt, m["dx"], m["dy"], **kw)
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"], odr=odr, flux="lhlld", nrk=nrk) as s:
        s.set_bc2d(*tables)
        s.upload(st)
        for _ in range(3):
            getattr(s, op)(coef, dt)
        got = s.download()
    assert equal_values(got, ref), max_rel_diff(got, ref)
    assert not equal_values(got, st)


@pytest.mark.parametrize("name", golden_cases("mrx"))
def test_mrx_loop_matches_golden(name):
    """Hyperbolic step + resistive diffusion + viscosity, as the MRX main loop,
    against the reference's own outputs."""
    prm, st, outs = load_golden(name)
    with M.Sim(2, st["ro"].shape, dx=prm["dx"], dy=prm["dy"], gamma=prm["gamma"],
               odr=prm["odr"], flux="lhlld", nrk=prm["nrk"]) as s:
        s.set_bc2d(prm["dnx"], prm["dny"])
        s.upload(st)
        done = 0
        for n in sorted(outs):
            for _ in range(n - done):
                s.step(prm["dt"], 1)
                s.resistive(prm["eta0"], prm["dt"])
                s.viscous(prm["nu0"], prm["dt"])
                if prm.get("kk0", 0.0) > 0:
                    assert s.conduction(prm["kk0"], prm["dt"]) > 1
            done = n
            got = s.download()
            assert equal_values(got, outs[n]), (n, max_rel_diff(got, outs[n]))


@pytest.mark.parametrize("kd", (0.1, 3.0, 30.0))
@pytest.mark.parametrize("tables", TABLES)
@pytest.mark.parametrize("odr", (1, 2, 3, 4, 5, 6))
def test_conduction_vs_oracle(port, odr, tables, kd):
    """Heat conduction: the same sweeps and the same result as the oracle,
    including the cases that run all 2048 sweeps without converging (a
    periodic y axis, where the reference's own y mirror of the temperature
    keeps the residual up)."""
    st, m, dt, _ = state(odr, odr * 13 + int(kd), tables, port)
    rng = np.random.default_rng(odr)
    st["en"] = st["en"] * (1 + 0.1 * rng.uniform(-1, 1, st["en"].shape))
    port.setbc2d(st, *tables)
    kk0 = kd * m["dx"] ** 2 / dt
    ref = ics.copy_state(st)
    n_ref, err = port.conduction2d(ref, kk0, dt, m["dx"], m["dy"], gamma=m["gamma"], odr=odr,
                                   dnx=tables[0], dny=tables[1])
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"], odr=odr, flux="lhlld") as s:
        s.set_bc2d(*tables)
        s.upload(st)
        if err:
            with pytest.raises(M.MlauError, match="did not converge"):
                s.conduction(kk0, dt)
            n = 2048
        else:
            n = s.conduction(kk0, dt)
        got = s.download()
    assert n == n_ref
    assert equal_values(got, ref), max_rel_diff(got, ref)


def test_conduction_dropin_vs_oracle_and_halt(port, tmp_path):
    """t_conduction through the reference's signature; a non-converging solve
    halts the process with the reference's messages and status 255."""
    import subprocess
    import sys

    L = M.lib()
    gx = (C.c_int * 8).in_dll(L, "dnxs")
    gy = (C.c_int * 8).in_dll(L, "dnys")
    tables = ics.MRX_TABLES
    st, m, dt, _ = state(4, 17, tables, port)
    rng = np.random.default_rng(3)
    st["en"] = st["en"] * (1 + 0.1 * rng.uniform(-1, 1, st["en"].shape))
    port.setbc2d(st, *tables)
    kk0 = 2.0 * m["dx"] ** 2 / dt
    ny, nx = st["ro"].shape
    assert L.mlau_set_scheme(2, 4, M.FLUX["lhlld"], 3) == 0
    try:
        for v in range(8):
            gx[v], gy[v] = tables[0][v], tables[1][v]
        ref, got = ics.copy_state(st), ics.copy_state(st)
        port.conduction2d(ref, kk0, dt, m["dx"], m["dy"], gamma=m["gamma"], odr=4,
                          dnx=tables[0], dny=tables[1])
        p = lambda k: got[k].ctypes.data_as(C.POINTER(C.c_double))
        L.t_conduction(*[p(k) for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")], kk0, dt,
                       m["dx"], m["dy"], nx, ny, 4, 4, m["gamma"], 0, 1, 1)
        assert equal_values(got, ref)
    finally:
        for v in range(8):
            gx[v] = gy[v] = 0
        L.mlau_set_scheme(2, 2, M.FLUX["lhlld"], 3)
        L.mlau_release_dropin()
    np.savez(tmp_path / "st.npz", **st)
    code = f"""
import ctypes as C, sys
import numpy as np
sys.path.insert(0, {repr(str(M.__file__).rsplit('/', 2)[0])})
import mlau_gb300 as M
L = M.lib()
z = np.load({repr(str(tmp_path / 'st.npz'))})
st = {{k: np.ascontiguousarray(z[k]) for k in z.files}}
ny, nx = st["ro"].shape
p = lambda k: st[k].ctypes.data_as(C.POINTER(C.c_double))
L.mlau_set_scheme(2, 4, 1, 3)
L.t_conduction(*[p(k) for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")], {kk0!r},
               {dt!r}, {m['dx']!r}, {m['dy']!r}, nx, ny, 4, 4, {m['gamma']!r}, 0, 1, 1)
print("returned")
"""
    # all-periodic tables (the library's defaults): the y mirror of the
    # temperature keeps the sweeps from converging
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 255, (r.returncode, r.stdout, r.stderr[-2000:])
    assert "Heat conduction did not converge. Calculation halted." in r.stdout
    assert "returned" not in r.stdout


@pytest.mark.parametrize("op", ("resistive", "viscous"))
def test_operator_many_blocks_vs_oracle(port, op):
    """A grid of several hundred blocks per launch, odd sizes."""
    st, m, dt, coef = state(4, 5, ics.MRX_TABLES, port, n=203, ny=97)
    ref = ics.copy_state(st)
    getattr(port, op + "2d")(ref, coef, dt, m["dx"], m["dy"], gamma=m["gamma"], odr=4, nrk=3,
                             dnx=ics.MRX_TABLES[0], dny=ics.MRX_TABLES[1])
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"], odr=4, flux="lhlld", nrk=3) as s:
        s.set_bc2d(*ics.MRX_TABLES)
        s.upload(st)
        getattr(s, op)(coef, dt)
        got = s.download()
    assert equal_values(got, ref)


def test_dropin_operators_vs_oracle(port):
    """diff_ctfield_e and ns_viscous_2d through the reference's signatures
    (host arrays, the library's boundary tables, MPI arguments of one rank)."""
    L = M.lib()
    tables = ics.MRX_TABLES
    gx = (C.c_int * 8).in_dll(L, "dnxs")
    gy = (C.c_int * 8).in_dll(L, "dnys")
    st, m, dt, coef = state(4, 9, tables, port)
    ny, nx = st["ro"].shape
    assert L.mlau_set_scheme(2, 4, M.FLUX["lhlld"], 3) == 0
    try:
        for v in range(8):
            gx[v], gy[v] = tables[0][v], tables[1][v]
        ref, got = ics.copy_state(st), ics.copy_state(st)
        kw = dict(gamma=m["gamma"], odr=4, nrk=3, dnx=tables[0], dny=tables[1])
        port.resistive2d(ref, coef, dt, m["dx"], m["dy"], **kw)
        port.viscous2d(ref, coef, dt, m["dx"], m["dy"], **kw)
        p = lambda k: got[k].ctypes.data_as(C.POINTER(C.c_double))
        L.diff_ctfield_e(p("en"), p("bx"), p("by"), p("bz"), coef, dt, m["dx"], m["dy"], nx, ny,
                         4, 4, m["gamma"], 0, 1, 1)
        L.ns_viscous_2d(p("ro"), p("mx"), p("my"), p("mz"), p("en"), coef, dt, m["dx"], m["dy"],
                        nx, ny, 4, 4, m["gamma"], 0, 1, 1)
        assert equal_values(got, ref), max_rel_diff(got, ref)
        # a table mixing periodic and wall entries on one axis is refused and
        # the arrays are left unchanged
        gy[0] = 0
        before = ics.copy_state(got)
        L.diff_ctfield_e(p("en"), p("bx"), p("by"), p("bz"), coef, dt, m["dx"], m["dy"], nx, ny,
                         4, 4, m["gamma"], 0, 1, 1)
        assert equal_values(got, before)
        assert "all zero or all nonzero" in M.last_error()
    finally:
        for v in range(8):
            gx[v] = gy[v] = 0
        L.mlau_set_scheme(2, 2, M.FLUX["lhlld"], 3)
        L.mlau_release_dropin()


def test_operators_refuse_other_simulations():
    st, m = ics.turbulence_3d(n=8, mach=0.5, seed=1)
    with M.Sim(3, st["ro"].shape, dx=m["dx"], dy=m["dy"], dz=m["dz"]) as s:
        with pytest.raises(M.MlauError, match="2D FP64"):
            s.resistive(1e-3, 1e-3)
    st, m = ics.turbulence_2d(n=16, seed=1)
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"]) as s:
        s.set_bc2d((0, 0, 0, 0, 1, 1, 1, 1), (0,) * 8)
        with pytest.raises(M.MlauError, match="all zero or all nonzero"):
            s.viscous(1e-3, 1e-3)


def totals(st, off=4):
    return {k: float(np.sum(st[k][off:-off, off:-off])) for k in st}


def test_mrx_full_size_loop():
    """The MRX problem at its full size (2048 x 256 cells, MC-limited MUSCL,
    LHLLD, RK3, Harris sheet): 200 loops of step + resistive diffusion +
    viscosity with the CFL dt of every loop.  Along the periodic x axis and
    with mirror walls in y, the scheme keeps div B as it was at round-off
    after the first loop (the initial state sets its ghosts analytically,
    with noise of their own, as the reference's does, so the first step's
    ghost fills move the boundary faces); the diffusion operators alone
    conserve the totals of B, momentum and energy where both axes are
    periodic."""
    st, m = ics.mrx_2d(seed=1)
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"], gamma=m["gamma"], odr=5,
               flux="lhlld", nrk=3) as s:
        s.set_bc2d(*m["tables"])
        s.upload(st)
        dt = m["dt"]
        for k in range(200):
            if k == 1:
                first = s.download()
            s.step(dt, 1)
            s.resistive(m["eta0"], dt)
            s.viscous(m["nu0"], dt)
            if k % 20 == 0:  # conduction along B (off in the reference's MRX setup)
                assert s.conduction(m["eta0"], dt) >= 1
            dt, _ = s.cfl(m["cfl"], m["dr"], m["vfast"], dt)
        out = s.download()
    for k, v in out.items():
        assert np.isfinite(v).all(), k
    # the perturbed Harris field is not discretely solenoidal: its div B stays
    assert ics.div_b_2d(out, m["dx"], m["dy"], odr=5, base=first) <= 1e-12
    assert out["ro"].min() > 0
    # the operators alone in a periodic box: flux form, so the totals telescope
    st, m2 = ics.turbulence_2d(n=512, ny=256, seed=4, vrms=0.5)
    dt = 0.3 * m2["dx"] / m2["vfast"]
    coef = 0.1 * m2["dx"] ** 2 / dt
    t0 = totals(st)
    scale = {k: np.abs(st[k][4:-4, 4:-4]).sum() for k in st}
    with M.Sim(2, st["ro"].shape, dx=m2["dx"], dy=m2["dy"], odr=4, flux="lhlld", nrk=3) as s:
        s.upload(st)
        for _ in range(100):
            s.resistive(coef, dt)
            s.viscous(coef, dt)
        out = s.download()
    t1 = totals(out)
    for k in ("mx", "my", "mz", "en", "bx", "by", "bz"):
        if scale[k] > 0:
            assert abs(t1[k] - t0[k]) / scale[k] <= 1e-12, k
    assert ics.div_b_2d(out, m2["dx"], m2["dy"], odr=4) <= 1e-12


def test_conduction_full_size_vs_oracle(port):
    """Heat conduction alone on the MRX grid (2048 x 256, walls in y) with a
    5 % pressure perturbation: the same sweep count and result as the oracle."""
    st, m3 = ics.mrx_2d(seed=2)
    rng = np.random.default_rng(2)
    st["en"] = st["en"] * (1 + 0.05 * rng.uniform(-1, 1, st["en"].shape))
    ref = ics.copy_state(st)
    kk0 = 0.5 * m3["dx"] ** 2 / m3["dt"]
    n_ref, err = port.conduction2d(ref, kk0, m3["dt"], m3["dx"], m3["dy"], gamma=m3["gamma"],
                                   odr=5, dnx=m3["tables"][0], dny=m3["tables"][1])
    with M.Sim(2, st["ro"].shape, dx=m3["dx"], dy=m3["dy"], gamma=m3["gamma"], odr=5,
               flux="lhlld") as s:
        s.set_bc2d(*m3["tables"])
        s.upload(st)
        n = s.conduction(kk0, m3["dt"])
        got = s.download()
    assert err == 0 and n == n_ref and equal_values(got, ref)


def test_mrx_problem_program_relinks(port, tmp_path):
    """A C++ program in the shape of MRX's main.cpp (its tables, the
    reference's prototypes with C++ linkage) links against the library in
    place of the driver file and gives the oracle's results for 3 loops of
    step + resistive diffusion + viscosity + heat conduction."""
    import os
    import subprocess

    st, m = ics.mrx_2d(n=96, ny=48, lx=24, seed=4)
    port.setbc2d(st, *ics.MRX_TABLES)
    rng = np.random.default_rng(4)
    st["en"] = st["en"] * (1 + 0.05 * rng.uniform(-1, 1, st["en"].shape))
    ny, nx = st["ro"].shape
    order = ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")
    np.concatenate([st[k].ravel() for k in order]).tofile(tmp_path / "in.bin")
    dt, eta0, nu0 = m["dt"], 0.05 * m["dx"] ** 2 / m["dt"], 0.04 * m["dx"] ** 2 / m["dt"]
    kk0 = 1.0 * m["dx"] ** 2 / m["dt"]
    src = os.path.join(os.path.dirname(__file__), "c", "mrx_dropin.cpp")
    exe = tmp_path / "mrx_dropin"
    libdir = os.path.dirname(M.LIB_PATH)
    subprocess.run(["g++", "-O1", src, "-o", str(exe), f"-L{libdir}", "-lmlau_gb300",
                    f"-Wl,-rpath,{libdir}"], check=True)
    args = [repr(v) for v in (dt, m["dx"], m["dy"], m["gamma"], eta0, nu0, kk0)]
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), str(nx),
                    str(ny), *args, "3"], check=True)
    raw = np.fromfile(tmp_path / "out.bin")
    got = {k: raw[i * nx * ny:(i + 1) * nx * ny].reshape(ny, nx) for i, k in enumerate(order)}
    ref = ics.copy_state(st)
    kw = dict(gamma=m["gamma"], odr=5, dnx=ics.MRX_TABLES[0], dny=ics.MRX_TABLES[1])
    for _ in range(3):
        port.step2d(ref, dt, m["dx"], m["dy"], flux="lhlld", nrk=3, **kw)
        port.resistive2d(ref, eta0, dt, m["dx"], m["dy"], nrk=3, **kw)
        port.viscous2d(ref, nu0, dt, m["dx"], m["dy"], nrk=3, **kw)
        n, err = port.conduction2d(ref, kk0, dt, m["dx"], m["dy"], **kw)
        assert err == 0
    assert equal_values(got, ref), max_rel_diff(got, ref)

