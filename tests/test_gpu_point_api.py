"""The reference's point-function interface in CUDA device code.

tests/c/point_api.cu is written against the reference's signatures - the
drivers' func_flux pointer type over calc_flux_mlau / lhlld / hlld / roe /
hl3d2, the *_cal_flr and *_cal_f interpolations, mhd_c / m / a_reconst and
mhd_reconst taking a calc_flr function pointer - and compiled with nvcc
against include/mlau_point.h (--fmad=false, as the reference is built without
contraction).  Its device results must equal the reference headers' host
results stored in tests/golden/point_api.npz.

Tolerance: identical values (NaNs in the same places, signed zeros alike)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import _point as P
from _util import GOLDEN

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def dev(tmp_path_factory):
    from mlau_gb300 import _build
    out = str(tmp_path_factory.mktemp("pointapi") / "libpointapi.so")
    cmd = [_build.nvcc(), *_build.ARCH, "--fmad=false", "-O2", "-std=c++17", "-shared",
           "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c", "point_api.cu"), "-o", out]
    subprocess.run(cmd, check=True, capture_output=True)
    lib = C.CDLL(out)
    lib.point_api_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_long, C.c_void_p, C.c_void_p]
    lib.point_api_run.restype = C.c_int
    return lib


def run(lib, kind, which, rows, odr=4):
    rows = np.ascontiguousarray(rows, dtype=np.float64)
    width = {0: 7, 1: 2, 2: 14}[kind]
    out = np.zeros((rows.shape[0], width))
    rc = lib.point_api_run(kind, which, odr, rows.shape[0], rows.ctypes.data_as(C.c_void_p),
                           out.ctypes.data_as(C.c_void_p))
    assert rc == 0, f"CUDA error {rc}"
    return out


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLDEN, "point_api.npz"))


def test_device_fluxes_equal_reference(dev, golden):
    for w, name in enumerate(P.FLUXES):
        assert P.same(run(dev, 0, w, golden["flux_in"]), golden["flux_out"][w]), name


def test_device_interpolations_equal_reference(dev, golden):
    # max/min come from CUDA's math headers under nvcc (documented in mlau_point.h)
    for w, name in enumerate(P.INTERPS[:12]):
        assert P.same(run(dev, 1, w, golden["interp_in"]), golden["interp_out"][w]), name


def test_device_reconstructions_equal_reference(dev, golden):
    for w, name in enumerate(P.RECONSTS):
        for j, odr in enumerate(golden["reconst_odr"]):
            got = run(dev, 2, w, golden["reconst_in"], int(odr))
            assert P.same(got, golden["reconst_out"][w, j]), (name, odr)
