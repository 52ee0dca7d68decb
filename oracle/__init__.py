"""CPU oracles for the MLAU hot path.  TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this package, and only as the checker.  Two oracles:

* ``Port`` - the C restatement in this directory (mlau_oracle.c), built on
  any host by ``build.build_port()``.
* ``Ref`` - the reference's own drivers compiled from its sources by
  ``build.build_ref_variant()``; available only where the reference tree is.

Both take numpy float64 arrays (one per variable, x fastest) and update them
in place, exactly like the reference drivers.
"""
from __future__ import annotations

import ctypes as C
import numpy as np

from . import build

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_cdp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")

FLUX = {"mlau": 0, "lhlld": 1, "hlld": 2, "roe": 3}


def _flux_id(f):
    return FLUX[f] if isinstance(f, str) else int(f)


class Port:
    """ctypes binding of oracle/_build/liboracle.so."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = C.CDLL(build.build_port())
            d, i = C.c_double, C.c_int
            lib.oracle_fd_ct_3d.argtypes = [_dp] * 8 + [d, d, d, d] + [i] * 6 + [d, i, i, i]
            lib.oracle_fd_ct_3d.restype = None
            lib.oracle_fd_ct_3d_bc.argtypes = ([_dp] * 8 + [d, d, d, d] + [i] * 6 + [d, i, i, i]
                                               + [C.POINTER(C.c_int)] * 3)
            lib.oracle_fd_ct_3d_bc.restype = None
            lib.oracle_fd_ct_2d.argtypes = [_dp] * 8 + [d, d, d] + [i] * 4 + [d, i, i, i]
            lib.oracle_fd_ct_2d.restype = None
            pi8 = C.POINTER(C.c_int)
            lib.oracle_fd_ct_2d_bc.argtypes = [_dp] * 8 + [d, d, d] + [i] * 4 + [d, i, i, i, pi8, pi8]
            lib.oracle_fd_ct_2d_bc.restype = None
            lib.oracle_bc2d_state.argtypes = [_dp] * 8 + [i] * 4 + [pi8, pi8]
            lib.oracle_bc2d_state.restype = None
            lib.oracle_diff_ctfield_e.argtypes = [_dp] * 4 + [d, d, d, d, i, i, i, i, d, i, i, pi8, pi8]
            lib.oracle_diff_ctfield_e.restype = None
            lib.oracle_ns_viscous_2d.argtypes = [_cdp] + [_dp] * 4 + [d, d, d, d, i, i, i, i, d, i, i, pi8, pi8]
            lib.oracle_ns_viscous_2d.restype = None
            lib.oracle_t_conduction.argtypes = ([_cdp] * 4 + [_dp] + [_cdp] * 3
                                                + [d, d, d, d, i, i, i, i, d, i, pi8, pi8, i,
                                                   C.POINTER(i)])
            lib.oracle_t_conduction.restype = i
            lib.oracle_fd4c_1d.argtypes = [_dp] * 7 + [d, d, d, i, i, d, i, i, i, i]
            lib.oracle_fd4c_1d.restype = None
            lib.oracle_cfl_3d.argtypes = [_cdp] * 8 + [i] * 6 + [d, d, d, d, d, C.POINTER(d)]
            lib.oracle_cfl_3d.restype = d
            lib.oracle_cfl_2d.argtypes = [_cdp] * 8 + [i] * 4 + [d, d, d, d, d, C.POINTER(d)]
            lib.oracle_cfl_2d.restype = d
            lib.oracle_dt_1d.argtypes = [_cdp] * 7 + [d, i, d, d, d, d]
            lib.oracle_dt_1d.restype = d
            lib.oracle_rec_lr.argtypes = [i, _cdp, C.POINTER(d), C.POINTER(d)]
            lib.oracle_flux.argtypes = [i, _cdp, _cdp, _dp]
            lib.oracle_reconst.argtypes = [i, i, _cdp, d, d, _dp, _dp]
            lib.oracle_set_eigen.argtypes = [i]
            lib.oracle_set_eigen.restype = None
            lib.oracle_inj_ro.argtypes = ([_dp] * 8 + [i] * 4 + [d] * 9
                                          + [C.c_void_p, pi8, pi8])
            lib.oracle_inj_ro.restype = None
            cls._lib = lib
        return cls._lib

    @classmethod
    def _eig(cls, eig):
        """Context: the eigen-system ("full" or "miyoshi") for one call."""
        lib = cls.lib()

        class _Ctx:
            def __enter__(self):
                lib.oracle_set_eigen(1 if eig == "miyoshi" else 0)

            def __exit__(self, *a):
                lib.oracle_set_eigen(0)
        return _Ctx()

    @classmethod
    def step3d(cls, s, dt, dx, dy, dz, off=4, gamma=5 / 3, odr=4, flux="mlau", nrk=3,
               eig="full", dnx=None, dny=None, dnz=None):
        """dnx/dny/dnz: the problem's tables (NULL: periodic)."""
        nz, ny, nx = s["ro"].shape
        tab = lambda t: None if t is None else (C.c_int * 8)(*[int(x) for x in t])
        with cls._eig(eig):
            cls.lib().oracle_fd_ct_3d_bc(*[s[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by",
                                                          "bz")],
                                         dt, dx, dy, dz, nx, ny, nz, off, off, off, gamma, odr,
                                         _flux_id(flux), nrk, tab(dnx), tab(dny), tab(dnz))

    @classmethod
    def step2d(cls, s, dt, dx, dy, off=4, gamma=5 / 3, odr=4, flux="lhlld", nrk=3, dnx=None,
               dny=None, eig="full"):
        """dnx/dny: the problem's boundary tables (8 ints, order ro mx my mz en
        bx by bz; 0 periodic, -1 Dirichlet, +1 Neumann); None is periodic."""
        ny, nx = s["ro"].shape
        tab = lambda t: None if t is None else (C.c_int * 8)(*[int(x) for x in t])
        with cls._eig(eig):
            cls.lib().oracle_fd_ct_2d_bc(*[s[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by",
                                                          "bz")],
                                         dt, dx, dy, nx, ny, off, off, gamma, odr, _flux_id(flux),
                                         nrk, tab(dnx), tab(dny))

    @classmethod
    def resistive2d(cls, s, eta0, dt, dx, dy, off=4, gamma=5 / 3, odr=2, nrk=3, dnx=None, dny=None):
        """diff_ctfield_e of the MRX driver file, in place on en, bx, by, bz."""
        ny, nx = s["ro"].shape
        tab = lambda t: None if t is None else (C.c_int * 8)(*[int(x) for x in t])
        cls.lib().oracle_diff_ctfield_e(s["en"], s["bx"], s["by"], s["bz"], eta0, dt, dx, dy, nx,
                                        ny, off, off, gamma, odr, nrk, tab(dnx), tab(dny))

    @classmethod
    def viscous2d(cls, s, nu0, dt, dx, dy, off=4, gamma=5 / 3, odr=2, nrk=3, dnx=None, dny=None):
        """ns_viscous_2d of the MRX driver file, in place on mx, my, mz, en."""
        ny, nx = s["ro"].shape
        tab = lambda t: None if t is None else (C.c_int * 8)(*[int(x) for x in t])
        cls.lib().oracle_ns_viscous_2d(s["ro"], s["mx"], s["my"], s["mz"], s["en"], nu0, dt, dx,
                                       dy, nx, ny, off, off, gamma, odr, nrk, tab(dnx), tab(dny))

    @classmethod
    def conduction2d(cls, s, kk0, dt, dx, dy, off=4, gamma=5 / 3, odr=2, dnx=None, dny=None,
                     cmax=2048):
        """t_conduction of the MRX driver file, in place on en; returns
        (Gauss-Seidel sweeps, err) with err -1 when cmax sweeps ran."""
        ny, nx = s["ro"].shape
        tab = lambda t: None if t is None else (C.c_int * 8)(*[int(x) for x in t])
        err = C.c_int(0)
        n = cls.lib().oracle_t_conduction(*[s[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by",
                                                           "bz")],
                                          kk0, dt, dx, dy, nx, ny, off, off, gamma, odr, tab(dnx),
                                          tab(dny), cmax, C.byref(err))
        return n, err.value

    @classmethod
    def inject2d(cls, s, ro3, dro3, vy1, bx1, by1, bz1, pr1, vref, gamma, noise=None, off=4,
                 dnx=None, dny=None):
        """inj_ro of the RMI problem plus its main loop's periodic exchange,
        in place; noise: the uniform draws in loop order, or None."""
        ny, nx = s["ro"].shape
        tab = lambda t: None if t is None else (C.c_int * 8)(*[int(x) for x in t])
        nz = None if noise is None else np.ascontiguousarray(noise, dtype=np.float64)
        cls.lib().oracle_inj_ro(*[s[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")],
                                nx, ny, off, off, ro3, dro3, vy1, bx1, by1, bz1, pr1, vref, gamma,
                                None if nz is None else nz.ctypes.data_as(C.c_void_p), tab(dnx),
                                tab(dny))

    @classmethod
    def setbc2d(cls, s, dnx, dny, off=4):
        """Apply the boundary tables to a 2D state's ghost cells in place (the
        reference problems' setbc after initialisation)."""
        ny, nx = s["ro"].shape
        tab = lambda t: (C.c_int * 8)(*[int(x) for x in t])
        cls.lib().oracle_bc2d_state(*[s[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")],
                                    nx, ny, off, off, tab(dnx), tab(dny))

    @classmethod
    def step1d(cls, s, bx, dt, dx, off=4, gamma=2.0, odr=2, flux="mlau", nrk=3, bc="open",
               eig="full"):
        nx = s["ro"].shape[0]
        with cls._eig(eig):
            cls.lib().oracle_fd4c_1d(*[s[k] for k in ("ro", "mx", "my", "mz", "en", "by", "bz")],
                                     bx, dt, dx, nx, off, gamma, odr, _flux_id(flux), nrk,
                                     0 if bc == "open" else 1)

    @classmethod
    def cfl3d(cls, s, cfl, dr, vfast, dt_old, off=4, gamma=5 / 3):
        nz, ny, nx = s["ro"].shape
        vm = C.c_double()
        dt = cls.lib().oracle_cfl_3d(*[s[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")],
                                     nx, ny, nz, off, off, off, gamma, cfl, dr, vfast, dt_old,
                                     C.byref(vm))
        return dt, vm.value

    @classmethod
    def cfl2d(cls, s, cfl, dr, vfast, dt_old, off=4, gamma=5 / 3):
        ny, nx = s["ro"].shape
        vm = C.c_double()
        dt = cls.lib().oracle_cfl_2d(*[s[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")],
                                     nx, ny, off, off, gamma, cfl, dr, vfast, dt_old, C.byref(vm))
        return dt, vm.value

    @classmethod
    def dt1d(cls, s, bx, gamma, cfl, dx, vfloor=1.0):
        nx = s["ro"].shape[0]
        return cls.lib().oracle_dt_1d(*[s[k] for k in ("ro", "mx", "my", "mz", "en", "by", "bz")],
                                      bx, nx, gamma, cfl, dx, vfloor)

    @classmethod
    def flux(cls, which, left7, right7, bn, gamma, dv=(0.0, 0.0)):
        inp = np.ascontiguousarray(np.r_[left7, right7, bn, gamma], dtype=np.float64)
        out = np.zeros(7)
        cls.lib().oracle_flux(_flux_id(which), inp, np.ascontiguousarray(dv, dtype=np.float64), out)
        return out


class Ref:
    """ctypes binding of a reference-driver variant built into oracle/_ref."""

    _libs: dict = {}
    HEADERS = "ref"

    @staticmethod
    def available() -> bool:
        return build.reference_available()

    @classmethod
    def _get(cls, dim, odr, flux, nrk, bc="open", eig="full"):
        key = (dim, odr, flux, nrk, bc if dim == 1 else "", eig)
        if key not in cls._libs:
            lib = C.CDLL(build.build_ref_variant(dim, odr, flux, nrk, bc, eig == "miyoshi",
                                                 headers=cls.HEADERS))
            d, i = C.c_double, C.c_int
            if dim == 1:
                lib.ref_step_1d.argtypes = [_dp] * 7 + [d, d, d, i, i, d]
                lib.ref_step_1d.restype = None
            else:
                lib.ref_step.argtypes = [_dp] * 8 + [d, d, d, d] + [i] * 6 + [d]
                lib.ref_step.restype = None
            cls._libs[key] = lib
        return cls._libs[key]

    @classmethod
    def step3d(cls, s, dt, dx, dy, dz, off=4, gamma=5 / 3, odr=4, flux="mlau", nrk=3,
               eig="full", dnx=None, dny=None, dnz=None):
        """dnx/dny/dnz: tables written into the build's dnxs/dnys/dnzs for this
        call; None is periodic."""
        nz, ny, nx = s["ro"].shape
        lib = cls._get(3, odr, _flux_id(flux), nrk, eig=eig)
        gs = [(C.c_int * 8).in_dll(lib, nm) for nm in ("dnxs", "dnys", "dnzs")]
        for g, t in zip(gs, (dnx, dny, dnz)):
            for v in range(8):
                g[v] = 0 if t is None else int(t[v])
        try:
            lib.ref_step(*[s[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")],
                         dt, dx, dy, dz, nx, ny, nz, off, off, off, gamma)
        finally:
            for g in gs:
                for v in range(8):
                    g[v] = 0

    @classmethod
    def step2d(cls, s, dt, dx, dy, off=4, gamma=5 / 3, odr=4, flux="lhlld", nrk=3, dnx=None,
               dny=None, eig="full"):
        """dnx/dny: boundary tables written into the build's dnxs/dnys
        globals (global.hpp) for this call; None is periodic."""
        ny, nx = s["ro"].shape
        lib = cls._get(2, odr, _flux_id(flux), nrk, eig=eig)
        gx = (C.c_int * 8).in_dll(lib, "dnxs")
        gy = (C.c_int * 8).in_dll(lib, "dnys")
        for g, t in ((gx, dnx), (gy, dny)):
            for v in range(8):
                g[v] = 0 if t is None else int(t[v])
        try:
            lib.ref_step(*[s[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")],
                         dt, dx, dy, 1.0, nx, ny, 1, off, off, 0, gamma)
        finally:
            for g in (gx, gy):
                for v in range(8):
                    g[v] = 0

    @classmethod
    def step1d(cls, s, bx, dt, dx, off=4, gamma=2.0, odr=2, flux="mlau", nrk=3, bc="open",
               eig="full"):
        nx = s["ro"].shape[0]
        cls._get(1, odr, _flux_id(flux), nrk, bc, eig).ref_step_1d(
            *[s[k] for k in ("ro", "mx", "my", "mz", "en", "by", "bz")], bx, dt, dx, nx, off, gamma)


class RefOnMlauPoint(Ref):
    """The reference's own drivers compiled unchanged against this library's
    include/mlau_point.h in place of the reference's point-function headers
    (funcs.h, interp.h, mhd_eigen.h, mhd_flux.h)."""

    _libs: dict = {}
    HEADERS = "mlau"


class RefMRX:
    """ctypes binding of the reference's 2D MRX driver file (hyperbolic step
    with the MC limiter at ODR 2, resistive and viscous operators) built into
    oracle/_ref; boundary tables written into the build's dnxs/dnys."""

    _libs: dict = {}

    @classmethod
    def _get(cls, odr, nrk):
        key = (odr, nrk)
        if key not in cls._libs:
            lib = C.CDLL(build.build_ref_mrx(odr, nrk))
            d, i = C.c_double, C.c_int
            lib.ref_mrx_step.argtypes = [_dp] * 8 + [d, d, d, i, i, i, i, d]
            lib.ref_diff_ctfield_e.argtypes = [_dp] * 4 + [d, d, d, d, i, i, i, i, d]
            lib.ref_ns_viscous_2d.argtypes = [_dp] * 5 + [d, d, d, d, i, i, i, i, d]
            lib.ref_t_conduction.argtypes = [_dp] * 8 + [d, d, d, d, i, i, i, i, d]
            for f in (lib.ref_mrx_step, lib.ref_diff_ctfield_e, lib.ref_ns_viscous_2d,
                      lib.ref_t_conduction):
                f.restype = None
            cls._libs[key] = lib
        return cls._libs[key]

    @classmethod
    def _tables(cls, lib, dnx, dny):
        for name, t in (("dnxs", dnx), ("dnys", dny)):
            g = (C.c_int * 8).in_dll(lib, name)
            for v in range(8):
                g[v] = 0 if t is None else int(t[v])

    @classmethod
    def _call(cls, fn, lib, dnx, dny, *args):
        cls._tables(lib, dnx, dny)
        try:
            fn(*args)
        finally:
            cls._tables(lib, None, None)

    @classmethod
    def step(cls, s, dt, dx, dy, off=4, gamma=5 / 3, odr=2, nrk=3, dnx=None, dny=None):
        ny, nx = s["ro"].shape
        lib = cls._get(odr, nrk)
        cls._call(lib.ref_mrx_step, lib, dnx, dny,
                  *[s[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")],
                  dt, dx, dy, nx, ny, off, off, gamma)

    @classmethod
    def resistive2d(cls, s, eta0, dt, dx, dy, off=4, gamma=5 / 3, odr=2, nrk=3, dnx=None, dny=None):
        ny, nx = s["ro"].shape
        lib = cls._get(odr, nrk)
        cls._call(lib.ref_diff_ctfield_e, lib, dnx, dny, s["en"], s["bx"], s["by"], s["bz"], eta0,
                  dt, dx, dy, nx, ny, off, off, gamma)

    @classmethod
    def viscous2d(cls, s, nu0, dt, dx, dy, off=4, gamma=5 / 3, odr=2, nrk=3, dnx=None, dny=None):
        ny, nx = s["ro"].shape
        lib = cls._get(odr, nrk)
        cls._call(lib.ref_ns_viscous_2d, lib, dnx, dny, s["ro"], s["mx"], s["my"], s["mz"], s["en"],
                  nu0, dt, dx, dy, nx, ny, off, off, gamma)

    @classmethod
    def conduction2d(cls, s, kk0, dt, dx, dy, off=4, gamma=5 / 3, odr=2, nrk=3, dnx=None,
                     dny=None):
        """The reference's t_conduction (it aborts the process when the sweeps
        do not converge within its CMAX of 2048: keep cases convergent)."""
        ny, nx = s["ro"].shape
        lib = cls._get(odr, nrk)
        cls._call(lib.ref_t_conduction, lib, dnx, dny,
                  *[s[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")],
                  kk0, dt, dx, dy, nx, ny, off, off, gamma)


class RefRMI:
    """ctypes binding of the reference's RMI inflow routine (inj_ro.hpp)
    built into oracle/_ref."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = C.CDLL(build.build_ref_rmi())
            d, i = C.c_double, C.c_int
            lib.ref_inj_ro.argtypes = [_dp] * 8 + [i] * 4 + [d] * 9 + [C.c_uint]
            lib.ref_inj_ro.restype = None
            cls._lib = lib
        return cls._lib

    @classmethod
    def inject2d(cls, s, ro3, dro3, vy1, bx1, by1, bz1, pr1, vref, gamma, seed=0, off=4):
        """The routine alone (its random() draws from srandom(seed)); the
        periodic exchange of the main loop is not part of it."""
        ny, nx = s["ro"].shape
        cls.lib().ref_inj_ro(*[s[k] for k in ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")],
                             nx, ny, off, off, ro3, dro3, vy1, bx1, by1, bz1, pr1, vref, gamma,
                             seed)

