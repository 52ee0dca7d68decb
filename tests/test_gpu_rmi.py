"""The RMI problem's inflow (inj_ro, 2D/MPI/RMI/inj_ro.hpp) on the GPU against
the oracle, which is pinned to the reference's own routine
(tests/test_oracle.py), the problem's main loop against the reference's
golden vectors, and the loop at the problem's full size."""
import numpy as np
import pytest

import mlau_gb300 as M
from _util import equal_values, golden_cases, load_golden, max_rel_diff
from mlau_gb300 import ics

pytestmark = pytest.mark.gpu


def inflow_args(inf, gamma=None, perturb=True):
    return (inf["ro3"], inf["dro3"] if perturb else 0.0, inf["vy1"], inf["bx1"], inf["by1"],
            inf["bz1"], inf["pr1"], inf["vref"])


@pytest.mark.parametrize("tables", [ics.RMI_TABLES, ((0,) * 8, (0,) * 8),
                                    ((1,) * 8, (1, 1, -1, 1, 1, 1, -1, 1))])
@pytest.mark.parametrize("perturb", (False, True))
def test_inflow_vs_oracle(port, perturb, tables):
    st, m = ics.rmi_2d(n=40, ny=96)
    rng = np.random.default_rng(3)
    for k in st:
        st[k] = st[k] + rng.uniform(-1e-3, 1e-3, st[k].shape)
    nx = st["ro"].shape[1]
    noise = ics.glibc_draws(11, 4 * nx) if perturb else None
    ref = ics.copy_state(st)
    port.inject2d(ref, *inflow_args(m["inflow"], perturb=perturb), m["gamma"], noise=noise,
                  dnx=tables[0], dny=tables[1])
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"], gamma=m["gamma"], odr=2,
               flux="lhlld") as s:
        s.set_bc2d(*tables)
        s.upload(st)
        s.inject(*inflow_args(m["inflow"], perturb=perturb), noise=noise)
        got = s.download()
    assert equal_values(got, ref), max_rel_diff(got, ref)


@pytest.mark.parametrize("name", golden_cases("rmi"))
def test_rmi_loop_matches_golden(name):
    """Inflow + exchange + MPI 2D step, the reference's own outputs."""
    prm, st, outs = load_golden(name)
    with M.Sim(2, st["ro"].shape, dx=prm["dx"], dy=prm["dy"], gamma=prm["gamma"],
               odr=prm["odr"], flux=prm["flux"], nrk=3) as s:
        s.set_bc2d(prm["dnx"], prm["dny"])
        s.upload(st)
        done = 0
        for n in sorted(outs):
            for k in range(done, n):
                s.inject(prm["inflow_ro3"], prm["inflow_dro3"], prm["inflow_vy1"],
                         prm["inflow_bx1"], prm["inflow_by1"], prm["inflow_bz1"],
                         prm["inflow_pr1"], prm["inflow_vref"], noise=prm["draws"][k])
                s.step(prm["dt"], 1)
            done = n
            got = s.download()
            assert equal_values(got, outs[n]), (n, max_rel_diff(got, outs[n]))


def test_rmi_loop_vs_oracle_with_cfl(port):
    """40 loops of the RMI problem at 32 x 512 with the CFL dt of every loop
    (the reference's CFLCHECK 1), the unperturbed inflow of its default."""
    st, m = ics.rmi_2d(n=32, ny=512)
    inf = m["inflow"]
    tables = m["tables"]
    ref = ics.copy_state(st)
    dt_ref, _ = port.cfl2d(ref, m["cfl"], m["dr"], m["vfast"], 0.0)
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"], gamma=m["gamma"], odr=2,
               flux="lhlld") as s:
        s.set_bc2d(*tables)
        s.upload(st)
        dt, _ = s.cfl(m["cfl"], m["dr"], m["vfast"], 0.0)
        assert dt == dt_ref
        for _ in range(40):
            port.inject2d(ref, *inflow_args(inf, perturb=False), m["gamma"], dnx=tables[0],
                          dny=tables[1])
            port.step2d(ref, dt_ref, m["dx"], m["dy"], gamma=m["gamma"], odr=2, flux="lhlld",
                        dnx=tables[0], dny=tables[1])
            dt_ref, _ = port.cfl2d(ref, m["cfl"], m["dr"], m["vfast"], dt_ref)
            s.inject(*inflow_args(inf, perturb=False))
            s.step(dt, 1)
            dt, _ = s.cfl(m["cfl"], m["dr"], m["vfast"], dt)
            assert dt == dt_ref
        got = s.download()
    assert equal_values(got, ref), max_rel_diff(got, ref)


def test_rmi_full_size():
    """The RMI problem at its size (128 x 10240, Mach 100 shock, density-10
    contact, Neumann y walls, inflow with the random perturbation): 300
    loops stay finite with positive density and pressure, and keep div B as
    it was after the first loop (the inflow rows are ghosts)."""
    st, m = ics.rmi_2d()
    inf = m["inflow"]
    nx = st["ro"].shape[1]
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"], gamma=m["gamma"], odr=2,
               flux="lhlld") as s:
        s.set_bc2d(*m["tables"])
        s.upload(st)
        dt, _ = s.cfl(m["cfl"], m["dr"], m["vfast"], 0.0)
        for k in range(300):
            s.inject(*inflow_args(inf), noise=ics.glibc_draws(100 + k, 4 * nx))
            s.step(dt, 1)
            if k == 0:
                first = s.download()
            dt, _ = s.cfl(m["cfl"], m["dr"], m["vfast"], dt)
        out = s.download()
    for k, v in out.items():
        assert np.isfinite(v).all(), k
    assert out["ro"][4:-4, 4:-4].min() > 0
    assert ics.div_b_2d(out, m["dx"], m["dy"], odr=2, base=first) <= 1e-12
