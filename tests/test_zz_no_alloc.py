"""The allocation-free 1D step (mlau_fd4c_1d_noalloc) against the existing 1D
entry point (the mlau_sim handle API).

Callers that cannot allocate device memory - code inside a host framework
that owns every device allocation, or a service holding a fixed device-memory
budget - pass arrays they already hold on the device; the entry point keeps
its scratch in a static device array.  Here the caller's arrays are the device
arrays of a simulation handle, so the test itself allocates through the
existing API while the entry point under test allocates nothing.

Tolerance: the same as the other parity tests - equal values (both paths run
the same FP64 kernels on the same inputs).  Two calls in a row, so the second
call runs on a scratch array that still holds the first call's contents.
This file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

import mlau_gb300 as M
from mlau_gb300 import ics

pytestmark = pytest.mark.gpu

V1 = ("ro", "mx", "my", "mz", "en", "by", "bz")


def _bind():
    L = M.lib()
    d, i = C.c_double, C.c_int
    L.mlau_fd4c_1d_noalloc.argtypes = [C.c_void_p] * 7 + [d, d, d, i, i, d, i, i, i, i, C.c_void_p]
    L.mlau_fd4c_1d_noalloc.restype = i
    return L


def _noalloc_step(L, sim, st, m, dt, odr, flux, nrk, bc):
    ptrs = [sim.device_ptr(k) for k in V1]
    rc = L.mlau_fd4c_1d_noalloc(*ptrs, m["bx"], dt, m["dx"], st["ro"].shape[0], 4, m["gamma"],
                                odr, M.FLUX[flux], nrk, M.BC1D[bc], sim.stream)
    assert rc == 0, M.last_error()


@pytest.mark.parametrize("bc,odr,flux,nrk", [("open", 2, "mlau", 3), ("periodic", 4, "lhlld", 3),
                                             ("open", 5, "hlld", 2), ("periodic", 3, "roe", 1)])
def test_noalloc_matches_handle_api_two_calls(bc, odr, flux, nrk):
    """Two checked calls in a row; between them a call on another grid size
    with another scheme, so the second checked call runs on scratch that a
    different layout left behind."""
    L = _bind()
    st, m = ics.riemann_1d(n=2048, seed=3)
    dt = 0.05 * m["dx"]
    kw = dict(dx=m["dx"], gamma=m["gamma"], odr=odr, flux=flux, nrk=nrk)
    other, mo = ics.riemann_1d(n=300, seed=8)
    okw = dict(dx=mo["dx"], gamma=mo["gamma"], odr=6 if odr != 6 else 2, flux="roe", nrk=3)
    with M.Sim(1, st["ro"].shape, **kw) as ref, M.Sim(1, st["ro"].shape, **kw) as mem, \
            M.Sim(1, other["ro"].shape, **okw) as side:
        for s in (ref, mem):
            s.set_bx(m["bx"])
            s.set_bc(bc)
            s.upload(st)
        side.set_bx(mo["bx"])
        side.upload(other)
        for call in range(2):
            _noalloc_step(L, mem, st, m, dt, odr, flux, nrk, bc)
            ref.step(dt, 1)
            mem.sync()
            got, want = mem.download(), ref.download()
            for k in V1:
                assert np.array_equal(got[k], want[k]), (call, k)
            if call == 0:
                # a different nx and scheme on the same stream between the checked calls
                side.sync()
                _noalloc_step(L, side, other, mo, 0.05 * mo["dx"], okw["odr"], "roe", 3, "open")
                side.sync()


def test_noalloc_rejects_oversize():
    L = _bind()
    with M.Sim(1, (64,), dx=1.0 / 56, gamma=2.0) as mem:
        ptrs = [mem.device_ptr(k) for k in V1]
        rc = L.mlau_fd4c_1d_noalloc(*ptrs, 0.8, 1e-3, 1.0 / 56, 16392 + 8, 4, 2.0, 2, 0, 3, 0,
                                    mem.stream)
        assert rc == -1 and "static scratch limit" in M.last_error()


def test_noalloc_rejects_shallow_ghosts():
    """Ghost depth 3 is refused: the flux kernels fill faces [3, nx-2) and a
    4th-order update from the first interior cell reads one face below."""
    L = _bind()
    with M.Sim(1, (64,), dx=1.0 / 56, gamma=2.0) as mem:
        ptrs = [mem.device_ptr(k) for k in V1]
        rc = L.mlau_fd4c_1d_noalloc(*ptrs, 0.8, 1e-3, 1.0 / 56, 64, 3, 2.0, 4, 0, 3, 0,
                                    mem.stream)
        assert rc == -1 and "bad geometry" in M.last_error()
