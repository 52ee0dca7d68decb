"""Generate the golden vectors in this directory from the reference itself.

Run here, where the reference tree is present:
    python tests/golden/make_golden.py [case names...]
It compiles the reference's own drivers (oracle/build.py, from the reference
sources) for each scheme variant, runs them on seeded inputs, and stores the
inputs and outputs.  3D/2D states are stored as their interior cells only: the
inputs are periodic (ghosts = periodic images) and every output ghost is a
periodic image too, so tests rebuild the ghosts with a periodic pad.  1D states
(open boundaries) are stored whole.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mlau_gb300 import ics  # noqa: E402
from oracle import Ref  # noqa: E402

OFF = 4
CASES_3D = [  # (name, n, mach, odr, flux, seed)
    ("3d_mlau_o4", 8, 0.9, 4, "mlau", 1),
    ("3d_lhlld_o4", 8, 0.9, 4, "lhlld", 2),
    ("3d_hlld_o4", 8, 0.9, 4, "hlld", 3),
    ("3d_roe_o4", 8, 0.9, 4, "roe", 4),
    ("3d_mlau_o2", 8, 0.9, 2, "mlau", 5),
    ("3d_lhlld_o3", 8, 0.9, 3, "lhlld", 6),
    ("3d_mlau_o4_lowmach", 8, 1e-2, 4, "mlau", 7),
    ("3d_mlau_o5", 8, 0.9, 5, "mlau", 8),
    ("3d_lhlld_o6", 8, 0.9, 6, "lhlld", 9),
    # Miyoshi's eigen-system swapped in for the full one (names ending _mi)
    ("3d_mlau_o4_mi", 8, 1.2, 4, "mlau", 10),
    ("3d_hlld_o3_mi", 8, 1.2, 3, "hlld", 11),
]
CASES_2D = [
    ("2d_lhlld_o4", 16, 4, "lhlld", 1),
    ("2d_mlau_o4", 16, 4, "mlau", 2),
    ("2d_hlld_o2", 16, 2, "hlld", 3),
    ("2d_roe_o4", 16, 4, "roe", 4),
    ("2d_lhlld_o1", 16, 1, "lhlld", 5),
    ("2d_lhlld_o5", 16, 5, "lhlld", 6),
    ("2d_mlau_o6", 16, 6, "mlau", 7),
    ("2d_lhlld_o4_mi", 16, 4, "lhlld", 8),
]
CASES_1D = [  # (name, n, odr, flux, bc, seed)
    ("1d_mlau_o2_open", 64, 2, "mlau", "open", 1),
    ("1d_lhlld_o1_open", 64, 1, "lhlld", "open", 2),
    ("1d_hlld_o4_open", 64, 4, "hlld", "open", 3),
    ("1d_roe_o3_open", 64, 3, "roe", "open", 4),
    ("1d_mlau_o4_periodic", 64, 4, "mlau", "periodic", 5),
    ("1d_mlau_o5_open", 64, 5, "mlau", "open", 6),
    ("1d_lhlld_o6_periodic", 64, 6, "lhlld", "periodic", 7),
    ("1d_mlau_o2_open_mi", 64, 2, "mlau", "open", 8),
]
# 2D with non-periodic boundary tables (the problem's dnxs / dnys), whole
# arrays stored: (name, n, odr, flux, seed, dnx, dny); the initial ghosts are
# filled with the tables first, as the problems' setbc does
KHI = ((0, 0, 0, 0, 0, 0, 0, 0), (1, 1, -1, 1, 1, 1, -1, 1))  # 2D/MPI/KHI/global.hpp:21-22
CASES_2D_WALLS = [
    ("2d_lhlld_o4_khi", 16, 4, "lhlld", 11, *KHI),
    ("2d_mlau_o5_khi", 16, 5, "mlau", 12, *KHI),
    ("2d_hlld_o2_walls", 16, 2, "hlld", 13, (1, -1, 1, 1, 1, -1, 1, 1), (1, 1, -1, 1, 1, 1, -1, 1)),
    ("2d_roe_o4_neumann", 16, 4, "roe", 14, (1,) * 8, (1,) * 8),
]
# The MRX problem's main loop (2D/MPI/MRX/main.cpp:48-68): hyperbolic step,
# resistive diffusion of B, viscosity and, where kd > 0, anisotropic heat
# conduction (diffusion number kd; the pressure is perturbed by 10 % so that
# the temperature varies); its driver file is built with ODR 2 (the
# MC-limited MUSCL, reconstruction code 5 here) or 4 and R_K 2 or 3; whole
# arrays stored: (name, nx, ny, ref odr, code, nrk, seed, dnx, dny, kd)
MRX_TABLES = ((0,) * 8, (1, 1, -1, 1, 1, 1, -1, 1))  # 2D/MPI/MRX/global.hpp:22-23
WALLS = (1, -1, 1, 1, 1, -1, 1, 1)
CASES_MRX = [
    ("mrx2d_o5_rk3", 24, 20, 2, 5, 3, 21, *MRX_TABLES, 0.0),
    ("mrx2d_o4_rk2", 24, 20, 4, 4, 2, 22, *MRX_TABLES, 0.0),
    ("mrx2d_o5_rk2_periodic", 20, 20, 2, 5, 2, 23, (0,) * 8, (0,) * 8, 0.0),
    ("mrx2d_o4_rk3_walls", 20, 24, 4, 4, 3, 24, WALLS, MRX_TABLES[1], 0.0),
    ("mrx2d_o5_rk3_cond", 24, 20, 2, 5, 3, 25, *MRX_TABLES, 2.0),
    ("mrx2d_o4_rk3_cond_walls", 20, 24, 4, 4, 3, 26, WALLS, MRX_TABLES[1], 2.0),
]
MRX_LOOPS = (1, 3)
# 3D with boundary tables (the MPI driver's mirrors), whole arrays stored:
# (name, n, odr, flux, seed, dnx, dny, dnz)
CASES_3D_WALLS = [
    ("3d_mlau_o4_walls", 6, 4, "mlau", 31, (0,) * 8, (1, 1, -1, 1, 1, 1, -1, 1),
     (1, 1, 1, -1, 1, 1, 1, -1)),
    ("3d_lhlld_o2_walls", 6, 2, "lhlld", 32, (1, -1, 1, 1, 1, -1, 1, 1), (1,) * 8, (0,) * 8),
]
# The RMI problem's main loop (2D/MPI/RMI/main.cpp:46-58): the inflow at the
# upper boundary (inj_ro, with its random() density perturbation drawn after
# srandom(seed + loop)), the periodic exchange along x, the MPI 2D step (ODR 2,
# LHLLD, RK3 - the serial driver with the same tables gives the same result);
# whole arrays and the draws stored: (name, n, ny, seed)
CASES_RMI = [("rmi2d_o2", 16, 48, 5)]
RMI_LOOPS = (1, 3)
STEPS = (1, 4)


def interior(a, dim):
    return np.ascontiguousarray(a[(slice(OFF, -OFF),) * dim])


def main(only=()):
    """Write every case, or only the named ones (existing files are kept)."""
    skip = (lambda name: bool(only) and name not in only)
    for name, n, mach, odr, flux, seed in CASES_3D:
        if skip(name):
            continue
        st, m = ics.turbulence_3d(n=n, mach=mach, seed=seed, odr=odr)
        dt = 0.3 * m["dx"] / m["vfast"]
        out = {"dt": dt, "dx": m["dx"], "gamma": m["gamma"], "odr": odr, "flux": flux}
        eig = "miyoshi" if name.endswith("_mi") else "full"
        if eig != "full":
            out["eig"] = eig
        for k, v in st.items():
            out["in_" + k] = interior(v, 3)
        s = ics.copy_state(st)
        done = 0
        for nstep in STEPS:
            for _ in range(nstep - done):
                Ref.step3d(s, dt, m["dx"], m["dy"], m["dz"], odr=odr, flux=flux, eig=eig)
            done = nstep
            for k, v in s.items():
                out[f"out{nstep}_" + k] = interior(v, 3)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    for name, n, odr, flux, seed in CASES_2D:
        if skip(name):
            continue
        st, m = ics.turbulence_2d(n=n, seed=seed, odr=odr, vrms=1.2)
        dt = 0.3 * m["dx"] / m["vfast"]
        out = {"dt": dt, "dx": m["dx"], "gamma": m["gamma"], "odr": odr, "flux": flux}
        eig = "miyoshi" if name.endswith("_mi") else "full"
        if eig != "full":
            out["eig"] = eig
        for k, v in st.items():
            out["in_" + k] = interior(v, 2)
        s = ics.copy_state(st)
        done = 0
        for nstep in STEPS:
            for _ in range(nstep - done):
                Ref.step2d(s, dt, m["dx"], m["dy"], odr=odr, flux=flux, eig=eig)
            done = nstep
            for k, v in s.items():
                out[f"out{nstep}_" + k] = interior(v, 2)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    for name, n, odr, flux, seed, dnx, dny in CASES_2D_WALLS:
        if skip(name):
            continue
        from oracle import Port
        st, m = ics.turbulence_2d(n=n, ny=n - 4, seed=seed, odr=odr, vrms=0.4)
        Port.setbc2d(st, dnx, dny)
        dt = 0.3 * m["dx"] / m["vfast"]
        out = {"dt": dt, "dx": m["dx"], "dy": m["dy"], "gamma": m["gamma"], "odr": odr,
               "flux": flux, "dnx": np.array(dnx), "dny": np.array(dny)}
        for k, v in st.items():
            out["in_" + k] = v.copy()
        s = ics.copy_state(st)
        done = 0
        for nstep in STEPS:
            for _ in range(nstep - done):
                Ref.step2d(s, dt, m["dx"], m["dy"], odr=odr, flux=flux, dnx=dnx, dny=dny)
            done = nstep
            for k, v in s.items():
                out[f"out{nstep}_" + k] = v.copy()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    for name, n, odr, flux, bc, seed in CASES_1D:
        if skip(name):
            continue
        st, m = ics.riemann_1d(n=n, seed=seed)
        from oracle import Port
        dt = Port.dt1d(st, m["bx"], m["gamma"], 0.4, m["dx"])
        out = {"dt": dt, "dx": m["dx"], "gamma": m["gamma"], "bx": m["bx"], "odr": odr,
               "flux": flux, "bc": bc}
        eig = "miyoshi" if name.endswith("_mi") else "full"
        if eig != "full":
            out["eig"] = eig
        for k, v in st.items():
            out["in_" + k] = v.copy()
        s = ics.copy_state(st)
        done = 0
        for nstep in STEPS:
            for _ in range(nstep - done):
                Ref.step1d(s, m["bx"], dt, m["dx"], gamma=m["gamma"], odr=odr, flux=flux, bc=bc,
                           eig=eig)
            done = nstep
            for k, v in s.items():
                out[f"out{nstep}_" + k] = v.copy()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    for name, nx, ny, rodr, code, nrk, seed, dnx, dny, kd in CASES_MRX:
        if skip(name):
            continue
        from oracle import Port, RefMRX
        st, m = ics.turbulence_2d(n=nx - 2 * OFF, ny=ny - 2 * OFF, seed=seed, odr=code, vrms=0.4)
        if kd > 0:
            rng = np.random.default_rng(seed)
            st["en"] = st["en"] * (1 + 0.1 * rng.uniform(-1, 1, st["en"].shape))
        Port.setbc2d(st, dnx, dny)
        dt = 0.3 * m["dx"] / m["vfast"]
        # diffusion numbers eta0*dt/dx^2 = 0.05, nu0*dt/dx^2 = 0.04
        eta0, nu0 = 0.05 * m["dx"] ** 2 / dt, 0.04 * m["dx"] ** 2 / dt
        kk0 = kd * m["dx"] ** 2 / dt
        out = {"dim": 2, "dt": dt, "dx": m["dx"], "dy": m["dy"], "gamma": m["gamma"], "odr": code,
               "nrk": nrk, "eta0": eta0, "nu0": nu0, "kk0": kk0, "dnx": np.array(dnx),
               "dny": np.array(dny)}
        for k, v in st.items():
            out["in_" + k] = v.copy()
        s = ics.copy_state(st)
        kw = dict(gamma=m["gamma"], odr=rodr, nrk=nrk, dnx=dnx, dny=dny)
        done = 0
        for nloop in MRX_LOOPS:
            for _ in range(nloop - done):
                RefMRX.step(s, dt, m["dx"], m["dy"], **kw)
                RefMRX.resistive2d(s, eta0, dt, m["dx"], m["dy"], **kw)
                RefMRX.viscous2d(s, nu0, dt, m["dx"], m["dy"], **kw)
                if kk0 > 0:
                    RefMRX.conduction2d(s, kk0, dt, m["dx"], m["dy"], **kw)
            done = nloop
            for k, v in s.items():
                out[f"out{nloop}_" + k] = v.copy()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    for name, n, odr, flux, seed, dnx, dny, dnz in CASES_3D_WALLS:
        if skip(name):
            continue
        st, m = ics.turbulence_3d(n=n, ny=n + 1, nz=n - 1, mach=0.8, seed=seed, odr=odr)
        dt = 0.3 * m["dx"] / m["vfast"]
        out = {"dim": 3, "dt": dt, "dx": m["dx"], "dy": m["dy"], "dz": m["dz"], "gamma": m["gamma"],
               "odr": odr, "flux": flux, "dnx": np.array(dnx), "dny": np.array(dny),
               "dnz": np.array(dnz)}
        for k, v in st.items():
            out["in_" + k] = v.copy()
        s = ics.copy_state(st)
        done = 0
        for nstep in STEPS:
            for _ in range(nstep - done):
                Ref.step3d(s, dt, m["dx"], m["dy"], m["dz"], odr=odr, flux=flux, dnx=dnx, dny=dny,
                           dnz=dnz)
            done = nstep
            for k, v in s.items():
                out[f"out{nstep}_" + k] = v.copy()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    for name, n, ny, seed in CASES_RMI:
        if skip(name):
            continue
        from oracle import Port, RefRMI
        st, m = ics.rmi_2d(n=n, ny=ny)
        inf = m["inflow"]
        dt, _ = Port.cfl2d(st, m["cfl"], m["dr"], m["vfast"], 0.0)
        nx = st["ro"].shape[1]
        draws = np.stack([ics.glibc_draws(seed + k, OFF * nx) for k in range(max(RMI_LOOPS))])
        out = {"dim": 2, "dt": dt, "dx": m["dx"], "dy": m["dy"], "gamma": m["gamma"], "odr": 2,
               "flux": "lhlld", "dnx": np.array(m["tables"][0]), "dny": np.array(m["tables"][1]),
               "draws": draws, **{"inflow_" + k: v for k, v in inf.items()}}
        for k, v in st.items():
            out["in_" + k] = v.copy()
        s = ics.copy_state(st)
        done = 0
        for nloop in RMI_LOOPS:
            for k in range(done, nloop):
                RefRMI.inject2d(s, inf["ro3"], inf["dro3"], inf["vy1"], inf["bx1"], inf["by1"],
                                inf["bz1"], inf["pr1"], inf["vref"], m["gamma"], seed=seed + k)
                for a in s.values():  # mpi_sdrv2d of one rank: x periodic
                    for i in range(OFF):
                        a[:, nx - 1 - i] = a[:, 2 * OFF - 1 - i]
                        a[:, i] = a[:, nx - 2 * OFF + i]
                Ref.step2d(s, dt, m["dx"], m["dy"], odr=2, flux="lhlld", dnx=m["tables"][0],
                           dny=m["tables"][1])
            done = nloop
            for k, v in s.items():
                out[f"out{nloop}_" + k] = v.copy()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote golden cases to", HERE)


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
