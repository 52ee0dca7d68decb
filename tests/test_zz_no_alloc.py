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


@pytest.mark.parametrize("bc,odr,flux", [("open", 2, "mlau"), ("periodic", 4, "lhlld")])
def test_noalloc_matches_handle_api_two_calls(bc, odr, flux):
    L = _bind()
    st, m = ics.riemann_1d(n=2048, seed=3)
    dt = 0.05 * m["dx"]
    nx = st["ro"].shape[0]
    kw = dict(dx=m["dx"], gamma=m["gamma"], odr=odr, flux=flux, nrk=3)
    with M.Sim(1, st["ro"].shape, **kw) as ref, M.Sim(1, st["ro"].shape, **kw) as mem:
        for s in (ref, mem):
            s.set_bx(m["bx"])
            s.set_bc(bc)
            s.upload(st)
        ptrs = [mem.device_ptr(k) for k in V1]
        for call in range(2):
            rc = L.mlau_fd4c_1d_noalloc(*ptrs, m["bx"], dt, m["dx"], nx, 4, m["gamma"], odr,
                                        M.FLUX[flux], 3, M.BC1D[bc], mem.stream)
            assert rc == 0, M.last_error()
            ref.step(dt, 1)
            mem.sync()
            got, want = mem.download(), ref.download()
            for k in V1:
                assert np.array_equal(got[k], want[k]), (call, k)


def test_noalloc_rejects_oversize():
    L = _bind()
    with M.Sim(1, (64,), dx=1.0 / 56, gamma=2.0) as mem:
        ptrs = [mem.device_ptr(k) for k in V1]
        rc = L.mlau_fd4c_1d_noalloc(*ptrs, 0.8, 1e-3, 1.0 / 56, 16392 + 8, 4, 2.0, 2, 0, 3, 0,
                                    mem.stream)
        assert rc == -1 and "static scratch limit" in M.last_error()
