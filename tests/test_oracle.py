"""CPU tests of the oracle: pinned to the reference and to its golden vectors,
plus the invariants the reference's scheme guarantees."""
import itertools

import numpy as np
import pytest

from _util import equal_values, golden_cases, load_golden
from mlau_gb300 import ics
from oracle import Ref


@pytest.mark.parametrize("name", golden_cases("3d"))
def test_port_matches_golden_3d(port, name):
    prm, s, outs = load_golden(name)
    done = 0
    for n in sorted(outs):
        for _ in range(n - done):
            port.step3d(s, prm["dt"], prm["dx"], prm.get("dy", prm["dx"]), prm.get("dz", prm["dx"]),
                        gamma=prm["gamma"], odr=prm["odr"], flux=prm["flux"],
                        eig=prm.get("eig", "full"), dnx=prm.get("dnx"), dny=prm.get("dny"),
                        dnz=prm.get("dnz"))
        done = n
        assert equal_values(s, outs[n]), f"{name}: differs after {n} steps"


@pytest.mark.parametrize("name", golden_cases("2d"))
def test_port_matches_golden_2d(port, name):
    prm, s, outs = load_golden(name)
    done = 0
    for n in sorted(outs):
        for _ in range(n - done):
            port.step2d(s, prm["dt"], prm["dx"], prm.get("dy", prm["dx"]), gamma=prm["gamma"],
                        odr=prm["odr"], flux=prm["flux"], dnx=prm.get("dnx"), dny=prm.get("dny"),
                        eig=prm.get("eig", "full"))
        done = n
        assert equal_values(s, outs[n]), f"{name}: differs after {n} steps"


@pytest.mark.parametrize("name", golden_cases("1d"))
def test_port_matches_golden_1d(port, name):
    prm, s, outs = load_golden(name)
    done = 0
    for n in sorted(outs):
        for _ in range(n - done):
            port.step1d(s, prm["bx"], prm["dt"], prm["dx"], gamma=prm["gamma"], odr=prm["odr"],
                        flux=prm["flux"], bc=prm["bc"], eig=prm.get("eig", "full"))
        done = n
        assert equal_values(s, outs[n]), f"{name}: differs after {n} steps"


def run_mrx_loop(port, s, prm, nloop):
    """The MRX problem's main loop (2D/MPI/MRX/main.cpp:48-68) on the oracle:
    hyperbolic step (LHLLD), resistive diffusion, viscosity."""
    kw = dict(gamma=prm["gamma"], odr=prm["odr"], nrk=prm["nrk"], dnx=prm["dnx"], dny=prm["dny"])
    for _ in range(nloop):
        port.step2d(s, prm["dt"], prm["dx"], prm["dy"], flux="lhlld", **kw)
        port.resistive2d(s, prm["eta0"], prm["dt"], prm["dx"], prm["dy"], **kw)
        port.viscous2d(s, prm["nu0"], prm["dt"], prm["dx"], prm["dy"], **kw)
        if prm.get("kk0", 0.0) > 0:
            n, err = port.conduction2d(s, prm["kk0"], prm["dt"], prm["dx"], prm["dy"],
                                       **{k: kw[k] for k in ("gamma", "odr", "dnx", "dny")})
            assert err == 0 and n > 1


@pytest.mark.parametrize("name", golden_cases("mrx"))
def test_port_matches_golden_mrx(port, name):
    prm, s, outs = load_golden(name)
    done = 0
    for n in sorted(outs):
        run_mrx_loop(port, s, prm, n - done)
        done = n
        assert equal_values(s, outs[n]), f"{name}: differs after {n} loops"


needs_ref = pytest.mark.skipif(not Ref.available(), reason="reference tree not present")

MRX_TABLES = [((0,) * 8, (0,) * 8), ((0,) * 8, (1, 1, -1, 1, 1, 1, -1, 1)),
              ((1, -1, 1, 1, 1, -1, 1, 1), (1, 1, -1, 1, 1, 1, -1, 1))]


@needs_ref
@pytest.mark.parametrize("tables", MRX_TABLES)
@pytest.mark.parametrize("rodr,nrk", [(2, 2), (2, 3), (4, 2), (4, 3)])
def test_mrx_operators_match_reference(port, rodr, nrk, tables):
    """Each MRX operator alone against the reference's MRX driver file built
    with that ODR and R_K (its ODR 2 is reconstruction code 5 here)."""
    from oracle import RefMRX

    code = 5 if rodr == 2 else 4
    st, m = ics.turbulence_2d(n=14, ny=10, seed=rodr * 3 + nrk, odr=code, vrms=0.4)
    port.setbc2d(st, *tables)
    dt = 0.3 * m["dx"] / m["vfast"]
    coef = 0.08 * m["dx"] ** 2 / dt
    kw = dict(gamma=m["gamma"], nrk=nrk, dnx=tables[0], dny=tables[1])
    for op in ("step", "resistive2d", "viscous2d"):
        a, b = ics.copy_state(st), ics.copy_state(st)
        if op == "step":
            port.step2d(a, dt, m["dx"], m["dy"], odr=code, flux="lhlld", **kw)
            RefMRX.step(b, dt, m["dx"], m["dy"], odr=rodr, **kw)
        else:
            getattr(port, op)(a, coef, dt, m["dx"], m["dy"], odr=code, **kw)
            getattr(RefMRX, op)(b, coef, dt, m["dx"], m["dy"], odr=rodr, **kw)
        assert equal_values(a, b), op
        assert not equal_values(a, st), op


@needs_ref
@pytest.mark.parametrize("tables", MRX_TABLES)
@pytest.mark.parametrize("kd", (0.1, 3.0, 30.0))
@pytest.mark.parametrize("rodr", (2, 4))
def test_conduction_matches_reference(port, rodr, kd, tables):
    """Anisotropic heat conduction against the reference's t_conduction, at
    diffusion numbers kd from a few to ~100 sweeps; with a periodic y axis the
    reference's own mirror in y keeps the sweeps from converging, and both
    run the 2048 sweeps of its CMAX (its abort is a no-op in the one-rank
    stub)."""
    from oracle import RefMRX

    code = 5 if rodr == 2 else 4
    st, m = ics.turbulence_2d(n=14, ny=10, seed=rodr + int(kd), odr=code, vrms=0.4)
    rng = np.random.default_rng(7)
    st["en"] = st["en"] * (1 + 0.1 * rng.uniform(-1, 1, st["en"].shape))
    port.setbc2d(st, *tables)
    dt = 0.3 * m["dx"] / m["vfast"]
    kk0 = kd * m["dx"] ** 2 / dt
    a, b = ics.copy_state(st), ics.copy_state(st)
    kw = dict(gamma=m["gamma"], dnx=tables[0], dny=tables[1])
    n, err = port.conduction2d(a, kk0, dt, m["dx"], m["dy"], odr=code, **kw)
    RefMRX.conduction2d(b, kk0, dt, m["dx"], m["dy"], odr=rodr, **kw)
    assert equal_values(a, b)
    assert not equal_values(a, st)
    assert (err == -1) == (tables[1][0] == 0)
    assert n == 2048 if err else 1 < n < 2048

# reconstruction codes 1-4 (ODR) with every solver; 5, 6 (MUSCL with the MC /
# Koren limiter, built by swapping calc_flr's limiter call) with two solvers
SCHEMES = (list(itertools.product((1, 2, 3, 4), ("mlau", "lhlld", "hlld", "roe")))
           + list(itertools.product((5, 6), ("mlau", "lhlld"))))


@needs_ref
@pytest.mark.parametrize("odr,flux", SCHEMES)
def test_port_matches_reference_3d(port, odr, flux):
    st, m = ics.turbulence_3d(n=6, ny=7, nz=5, mach=0.8, seed=odr * 7 + len(flux), odr=odr)
    # inconsistent ghosts: the step must read exactly the reference's cells
    rng = np.random.default_rng(1)
    for k in st:
        g = st[k].copy()
        g[:4] *= 1 + 1e-3 * rng.random(g[:4].shape)
        st[k] = np.ascontiguousarray(g)
    a, b = ics.copy_state(st), ics.copy_state(st)
    for _ in range(2):
        port.step3d(a, 1e-3, m["dx"], m["dy"], m["dz"], odr=odr, flux=flux)
        Ref.step3d(b, 1e-3, m["dx"], m["dy"], m["dz"], odr=odr, flux=flux)
    assert equal_values(a, b)


@needs_ref
@pytest.mark.parametrize("odr,flux", SCHEMES)
def test_port_matches_reference_2d(port, odr, flux):
    st, m = ics.turbulence_2d(n=20, ny=14, seed=odr + 3, odr=odr, vrms=1.3)
    a, b = ics.copy_state(st), ics.copy_state(st)
    for _ in range(3):
        port.step2d(a, 2e-3, m["dx"], m["dy"], odr=odr, flux=flux)
        Ref.step2d(b, 2e-3, m["dx"], m["dy"], odr=odr, flux=flux)
    assert equal_values(a, b)


@needs_ref
@pytest.mark.parametrize("bc", ("open", "periodic"))
@pytest.mark.parametrize("odr,flux", SCHEMES)
def test_port_matches_reference_1d(port, odr, flux, bc):
    st, m = ics.riemann_1d(n=48, seed=odr * 5 + len(flux))
    dt = port.dt1d(st, m["bx"], m["gamma"], 0.4, m["dx"])
    a, b = ics.copy_state(st), ics.copy_state(st)
    for _ in range(6):
        port.step1d(a, m["bx"], dt, m["dx"], gamma=m["gamma"], odr=odr, flux=flux, bc=bc)
        Ref.step1d(b, m["bx"], dt, m["dx"], gamma=m["gamma"], odr=odr, flux=flux, bc=bc)
    assert equal_values(a, b)


@needs_ref
@pytest.mark.parametrize("nrk", (1, 2))
def test_port_matches_reference_rk_order(port, nrk):
    st, m = ics.turbulence_3d(n=6, mach=0.5, seed=9)
    a, b = ics.copy_state(st), ics.copy_state(st)
    port.step3d(a, 1e-3, m["dx"], m["dy"], m["dz"], nrk=nrk)
    Ref.step3d(b, 1e-3, m["dx"], m["dy"], m["dz"], nrk=nrk)
    assert equal_values(a, b)


def test_port_div_b_preserved(port):
    """CT keeps the scheme's discrete div B at round-off (mhd_fd_ct_3d.c:80-88)."""
    st, m = ics.turbulence_3d(n=10, mach=0.3, seed=2)
    d0 = ics.div_b_3d(st, m["dx"], m["dy"], m["dz"])
    for _ in range(10):
        port.step3d(st, 2e-3, m["dx"], m["dy"], m["dz"])
    d1 = ics.div_b_3d(st, m["dx"], m["dy"], m["dz"])
    assert d0 < 1e-13 and d1 < 1e-12


def test_port_zero_guard_2d(port):
    """Identically zero vz and Bz stay exactly zero (mhd_eigen.h:516-529)."""
    st, m = ics.turbulence_2d(n=16, seed=4)
    assert not st["mz"].any() and not st["bz"].any()
    for _ in range(5):
        port.step2d(st, 2e-3, m["dx"], m["dy"])
    assert not st["mz"].any() and not st["bz"].any()


def test_port_thread_count_independent(port, tmp_path):
    """The step has no reductions: results do not depend on thread count."""
    import os
    import subprocess
    import sys
    code = (
        "import sys,numpy as np; sys.path.insert(0,%r); from oracle import Port; "
        "from mlau_gb300 import ics; st,m=ics.turbulence_3d(n=8,mach=0.5,seed=3); "
        "Port.step3d(st,1e-3,m['dx'],m['dy'],m['dz']); np.save(sys.argv[1], st['en'])"
    ) % os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    outs = []
    for t in ("1", "4"):
        path = str(tmp_path / f"thr_{t}.npy")
        subprocess.run([sys.executable, "-c", code, path], check=True,
                       env={**os.environ, "OMP_NUM_THREADS": t})
        outs.append(np.load(path))
    assert np.array_equal(outs[0], outs[1])


def test_cfl_oracle_matches_formula(port):
    st, m = ics.turbulence_3d(n=8, mach=0.3, seed=5)
    dt, vmax = port.cfl3d(st, 0.4, m["dx"], 0.0, 1.0)
    assert vmax > 0 and abs(dt - 0.4 * m["dx"] / vmax) < 1e-18
    dt2, vm2 = port.cfl3d(st, 0.4, m["dx"], 1e9, 1.0)
    assert vm2 == 1e9


MIYOSHI = [(3, 4, "mlau"), (3, 4, "lhlld"), (3, 2, "lhlld"), (3, 3, "hlld"),
           (2, 4, "mlau"), (2, 4, "lhlld"), (2, 2, "lhlld"), (2, 3, "hlld"),
           (1, 2, "mlau"), (1, 4, "hlld")]


@needs_ref
@pytest.mark.parametrize("dim,odr,flux", MIYOSHI)
def test_port_matches_reference_miyoshi(port, dim, odr, flux):
    """Miyoshi's eigen-system (mhd_m_reconst) in place of the full one, against
    the reference drivers built with that call swapped in; supersonic states
    so that the full-system branch runs."""
    if dim == 3:
        st, m = ics.turbulence_3d(n=6, ny=7, nz=5, mach=1.2, seed=odr * 3 + len(flux), odr=odr)
        run = lambda f, s, e: f.step3d(s, 1e-3, m["dx"], m["dy"], m["dz"], odr=odr, flux=flux,
                                       eig=e)
    elif dim == 2:
        st, m = ics.turbulence_2d(n=20, ny=14, seed=odr + 3, odr=odr, vrms=1.5)
        run = lambda f, s, e: f.step2d(s, 2e-3, m["dx"], m["dy"], odr=odr, flux=flux, eig=e)
    else:
        st, m = ics.riemann_1d(n=48, seed=odr * 5)
        dt = port.dt1d(st, m["bx"], m["gamma"], 0.4, m["dx"])
        run = lambda f, s, e: f.step1d(s, m["bx"], dt, m["dx"], gamma=m["gamma"], odr=odr,
                                       flux=flux, eig=e)
    a, b, c = ics.copy_state(st), ics.copy_state(st), ics.copy_state(st)
    for _ in range(6 if dim == 1 else 3):
        run(port, a, "miyoshi")
        run(Ref, b, "miyoshi")
        run(port, c, "full")
    assert equal_values(a, b)
    assert not equal_values(a, c)


def run_rmi_loop(port, s, prm, k0, k1):
    """The RMI problem's main loop (2D/MPI/RMI/main.cpp:46-58) on the oracle:
    inflow with the stored draws, periodic exchange, step."""
    tables = (prm["dnx"], prm["dny"])
    for k in range(k0, k1):
        port.inject2d(s, prm["inflow_ro3"], prm["inflow_dro3"], prm["inflow_vy1"],
                      prm["inflow_bx1"], prm["inflow_by1"], prm["inflow_bz1"], prm["inflow_pr1"],
                      prm["inflow_vref"], prm["gamma"], noise=prm["draws"][k], dnx=tables[0],
                      dny=tables[1])
        port.step2d(s, prm["dt"], prm["dx"], prm["dy"], gamma=prm["gamma"], odr=prm["odr"],
                    flux=prm["flux"], dnx=tables[0], dny=tables[1])


@pytest.mark.parametrize("name", golden_cases("rmi"))
def test_port_matches_golden_rmi(port, name):
    prm, s, outs = load_golden(name)
    done = 0
    for n in sorted(outs):
        run_rmi_loop(port, s, prm, done, n)
        done = n
        assert equal_values(s, outs[n]), f"{name}: differs after {n} loops"


@needs_ref
@pytest.mark.parametrize("seed,perturb", [(0, False), (7, True), (123, True)])
def test_inflow_matches_reference(port, seed, perturb):
    """The RMI inflow against the reference's inj_ro (its random() draws after
    srandom(seed)), followed on both sides by the periodic x exchange."""
    from oracle import RefRMI

    st, m = ics.rmi_2d(n=32, ny=64)
    inf = m["inflow"]
    rng = np.random.default_rng(seed)
    for k in st:
        st[k] = st[k] + rng.uniform(-1e-3, 1e-3, st[k].shape)
    a, b = ics.copy_state(st), ics.copy_state(st)
    nx = st["ro"].shape[1]
    dro3 = inf["dro3"] if perturb else 0.0
    args = (inf["ro3"], dro3, inf["vy1"], inf["bx1"], inf["by1"], inf["bz1"], inf["pr1"],
            inf["vref"], m["gamma"])
    port.inject2d(a, *args, noise=ics.glibc_draws(seed, 4 * nx) if perturb else None,
                  dnx=m["tables"][0], dny=m["tables"][1])
    RefRMI.inject2d(b, *args, seed=seed)
    for f in b.values():
        for i in range(4):
            f[:, nx - 1 - i] = f[:, 7 - i]
            f[:, i] = f[:, nx - 8 + i]
    assert equal_values(a, b)
    assert not equal_values(a, st)


Z8, W8, N8 = (0,) * 8, (1, -1, 1, 1, 1, -1, 1, 1), (1,) * 8
TABLES_3D = [(Z8, Z8, (1, 1, 1, -1, 1, 1, 1, -1)), (W8, Z8, Z8), (Z8, (1, 1, -1, 1, 1, 1, -1, 1), Z8),
             (W8, (1, 1, -1, 1, 1, 1, -1, 1), (1, 1, 1, -1, 1, 1, 1, -1)), (N8, N8, N8)]


@needs_ref
@pytest.mark.parametrize("tables", TABLES_3D)
@pytest.mark.parametrize("odr,flux", [(4, "mlau"), (2, "lhlld"), (3, "hlld"), (5, "mlau"),
                                      (1, "roe")])
def test_port_matches_reference_3d_tables(port, odr, flux, tables):
    """The 3D step with the problem's tables (the MPI driver's exchange and
    mirrors at its three fill sites) against the reference driver built with
    the same tables."""
    st, m = ics.turbulence_3d(n=6, ny=7, nz=5, mach=0.8, seed=odr + len(flux), odr=odr)
    a, b = ics.copy_state(st), ics.copy_state(st)
    kw = dict(odr=odr, flux=flux, dnx=tables[0], dny=tables[1], dnz=tables[2])
    for _ in range(2):
        port.step3d(a, 1e-3, m["dx"], m["dy"], m["dz"], **kw)
        Ref.step3d(b, 1e-3, m["dx"], m["dy"], m["dz"], **kw)
    assert equal_values(a, b, equal_nan=True)

