"""Checkpoint and output files written from / read into device-resident
simulations: byte-identical to the files the reference's own routines wrote
(tests/golden/io), and a run restarted from a checkpoint continues exactly as
an uninterrupted one."""
import os

import numpy as np
import pytest

import mlau_gb300 as M
from mlau_gb300 import ics
from oracle import dataio

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "io")


def read(path):
    with open(path, "rb") as fh:
        return fh.read()


def sim_like(st, dim, **kw):
    return M.Sim(dim, st["ro"].shape, **kw)


def test_3d_checkpoint_and_fp32_output_are_byte_identical(tmp_path):
    meta = np.load(os.path.join(GOLD, "3d_meta.npz"))
    gdir = os.path.join(GOLD, "3d")
    with M.Sim(3, tuple(meta["shape"]), gamma=float(meta["gamma"])) as s:
        assert s.bkup_load(gdir) == (40, 3, 0.123456789, 1e-3, 0.2)
        s.bkup_save(str(tmp_path), 40, 3, 0.123456789, 1e-3, 0.2)
        s.outdat(str(tmp_path), 3, 0, M.OUT_F32_RANK)
        M.outdat_meta(str(tmp_path), 3, True, 0.125, float(meta["gamma"]))
        M.outdat_meta(str(tmp_path), 3, False, 0.25, float(meta["gamma"]))
    for f in ("bkup_stamp.dat", "bkup_time.dat", "bkup_data_00000.dat", "outdat_00003_00000.dat",
              "params.dat", "offsets.dat", "t.dat"):
        assert read(os.path.join(tmp_path, f)) == read(os.path.join(gdir, f)), f


def test_2d_fp64_output_is_byte_identical(tmp_path):
    meta = np.load(os.path.join(GOLD, "2d_meta.npz"))
    shape = tuple(meta["shape"])
    raw = np.frombuffer(read(os.path.join(GOLD, "2d", "outdat_00002.dat")), dtype="<f8")
    size = int(np.prod(shape))
    st = {k: raw[i * size:(i + 1) * size].reshape(shape).copy()
          for i, k in enumerate(dataio.OUT_ORDER)}
    with M.Sim(2, shape, gamma=float(meta["gamma"])) as s:
        s.upload(st)
        s.outdat(str(tmp_path), 2)
        # 2D checkpoint round trip through the restated format
        s.bkup_save(str(tmp_path), 12, 1, 0.5, 0.01, 0.6)
    assert read(os.path.join(tmp_path, "outdat_00002.dat")) == read(
        os.path.join(GOLD, "2d", "outdat_00002.dat"))
    want = dataio.bkup_files(st, 12, 1, 0.5, 0.01, 0.6)
    for name, data in want.items():
        assert read(os.path.join(tmp_path, name)) == data, name


def test_1d_output_is_byte_identical(tmp_path):
    z = np.load(os.path.join(GOLD, "1d_state.npz"))
    st = {k: z[k] for k in dataio.OUT_ORDER_1D}
    with M.Sim(1, st["ro"].shape) as s:
        s.upload(st)
        s.outdat(str(tmp_path), 5)
    assert read(os.path.join(tmp_path, "outdat_00005.dat")) == read(
        os.path.join(GOLD, "1d", "outdat_00005.dat"))


def test_load_without_a_checkpoint_changes_nothing(tmp_path):
    st, m = ics.turbulence_2d(n=16, seed=1)
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"]) as s:
        s.upload(st)
        assert s.bkup_load(str(tmp_path)) is None
        got = s.download()
    for k in st:
        assert np.array_equal(got[k], st[k])


@pytest.mark.parametrize("precision", [M.FP64, M.FP32_SPLIT])
def test_restart_from_checkpoint_continues_exactly(tmp_path, precision):
    st, m = ics.turbulence_3d(n=16, mach=0.1, seed=5)
    dt = 0.4 * m["dx"] / m["vfast"]
    kw = dict(dx=m["dx"], dy=m["dy"], dz=m["dz"], precision=precision)
    with M.Sim(3, st["ro"].shape, **kw) as s:
        s.upload(st)
        s.step(dt, 10)
        ref = s.download()
    with M.Sim(3, st["ro"].shape, **kw) as s:
        s.upload(st)
        s.step(dt, 4)
        s.bkup_save(str(tmp_path), 4, 0, 4 * dt, dt, 1.0)
    with M.Sim(3, st["ro"].shape, **kw) as s:
        n, cnt, tim, dt2, trec = s.bkup_load(str(tmp_path))
        assert (n, dt2) == (4, dt)
        s.step(dt2, 10 - n)
        got = s.download()
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k
