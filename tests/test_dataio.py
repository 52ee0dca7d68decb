"""Checkpoint and output file formats (CPU): the format restatement in
oracle/dataio.py against golden files written by the reference's own
routines, and against those routines directly where the reference is here."""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

from mlau_gb300 import ics
from oracle import build, dataio

GOLD = os.path.join(os.path.dirname(__file__), "golden", "io")
VARS = ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")


def read(path):
    with open(path, "rb") as fh:
        return fh.read()


def gold3d():
    files = {f: read(os.path.join(GOLD, "3d", f)) for f in os.listdir(os.path.join(GOLD, "3d"))}
    meta = np.load(os.path.join(GOLD, "3d_meta.npz"))
    return files, meta


def test_restatement_reads_and_rewrites_the_reference_checkpoint():
    files, meta = gold3d()
    stamp, st = dataio.read_bkup(files, tuple(meta["shape"]))
    assert stamp == (40, 3, 0.123456789, 1e-3, 0.2)
    again = dataio.bkup_files(st, *stamp)
    for name, data in again.items():
        assert data == files[name], name


def test_restatement_output_formats_match_the_reference_files():
    files, meta = gold3d()
    _, st = dataio.read_bkup(files, tuple(meta["shape"]))
    name, data = dataio.outdat_f32(st, 3, 0)
    assert data == files[name]
    m = dataio.meta_files(3, True, 0.125, float(meta["gamma"]))
    m = dataio.meta_files(3, False, 0.25, float(meta["gamma"]), t_before=m["t.dat"]) | {
        k: v for k, v in m.items() if k != "t.dat"}
    for k, v in m.items():
        assert v == files[k], k
    d2 = {f: read(os.path.join(GOLD, "2d", f)) for f in os.listdir(os.path.join(GOLD, "2d"))}
    meta2 = np.load(os.path.join(GOLD, "2d_meta.npz"))
    shape2 = tuple(meta2["shape"])
    raw = np.frombuffer(d2["outdat_00002.dat"], dtype="<f8")
    size = int(np.prod(shape2))
    st2 = {k: raw[i * size:(i + 1) * size].reshape(shape2) for i, k in enumerate(dataio.OUT_ORDER)}
    assert dataio.outdat_f64(st2, 2, 2)[1] == d2["outdat_00002.dat"]
    m2 = dataio.meta_files(2, True, 0.5, float(meta2["gamma"]))
    m2 = dataio.meta_files(2, False, 0.75, float(meta2["gamma"]), t_before=m2["t.dat"]) | {
        k: v for k, v in m2.items() if k != "t.dat"}
    for k, v in m2.items():
        assert v == d2[k], k


@pytest.mark.skipif(not build.reference_available(), reason="reference tree not present")
def test_restatement_matches_the_reference_routines_on_fresh_states():
    lib = C.CDLL(build.build_ref_io())
    d = C.c_double
    st, m = ics.turbulence_3d(n=4, ny=5, nz=4, mach=0.9, seed=23)
    st = {k: np.ascontiguousarray(v) for k, v in st.items()}
    nz, ny, nx = st["ro"].shape
    arr = (C.POINTER(C.c_double) * 8)(*[st[k].ctypes.data_as(C.POINTER(C.c_double)) for k in VARS])
    xyz = [np.zeros(k) for k in (nx, ny, nz)]
    with tempfile.TemporaryDirectory() as tmp:
        lib.ref_bkup_save(tmp.encode(), 7, 1, d(2.5), d(0.01), d(3.0), nx * ny * nz, 2, arr)
        lib.ref_dataio_3d(tmp.encode(), 5, 9, d(1.0), 2, nx, ny, nz, 4, 4, 4, d(m["gamma"]), arr,
                          *[a.ctypes.data_as(C.POINTER(C.c_double)) for a in xyz])
        want = dataio.bkup_files(st, 7, 1, 2.5, 0.01, 3.0, rank=2)
        assert set(want) == {"bkup_data_00002.dat"}
        assert read(os.path.join(tmp, "bkup_data_00002.dat")) == want["bkup_data_00002.dat"]
        name, data = dataio.outdat_f32(st, 9, 2)
        assert read(os.path.join(tmp, name)) == data
