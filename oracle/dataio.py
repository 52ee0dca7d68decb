"""Restatement of the reference's checkpoint and output file formats.
TEST INFRASTRUCTURE ONLY: the tests check the library's writers and readers
against it; nothing in the library imports it.

* checkpoint, 3D/MPI/OTvortex/bkup.hpp:46-76 (same in 2D/MPI): bkup_stamp.dat
  is the text "%d %d\\n" (step, output count); bkup_time.dat the three doubles
  (time, dt, next output time); bkup_data_%05d.dat the whole padded arrays
  ro, mx, my, mz, bx, by, bz, en as raw FP64 (bkup.hpp:66-73).
* FP32 per-rank output, 3D/MPI/OTvortex/dataio.hpp:62-80: outdat_%05d_%05d.dat
  = ro, mx, my, mz, en, bx, by, bz each cast to float.
* FP64 serial output, 2D/SERIAL/OTvortex/dataio.hpp:28-38: outdat_%05d.dat of
  the same eight arrays as FP64; the 1D driver writes ro, mx, my, mz, en, by,
  bz (1D/SERIAL/shock/main.cpp:171-184).
* metadata at the first output: params.dat ("%f\\n" gamma; 1D "%.12f %.12f\\n"
  bx gamma), offsets.dat ("%d %d %d\\n" / "%d %d\\n"; 1D xoff.dat "%d\\n"),
  t.dat ("%f\\n" per output; 1D "%.12f\\n").
"""
from __future__ import annotations

import numpy as np

BKUP_ORDER = ("ro", "mx", "my", "mz", "bx", "by", "bz", "en")
OUT_ORDER = ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")
OUT_ORDER_1D = ("ro", "mx", "my", "mz", "en", "by", "bz")


def bkup_files(st, n, cnt, tim, dt, trec, rank=0):
    out = {}
    if rank == 0:
        out["bkup_stamp.dat"] = f"{n} {cnt}\n".encode()
        out["bkup_time.dat"] = np.array([tim, dt, trec], dtype="<f8").tobytes()
    out[f"bkup_data_{rank:05d}.dat"] = b"".join(
        np.ascontiguousarray(st[k], dtype="<f8").tobytes() for k in BKUP_ORDER)
    return out


def read_bkup(files, shape, rank=0):
    n, cnt = (int(x) for x in files["bkup_stamp.dat"].split())
    tim, dt, trec = np.frombuffer(files["bkup_time.dat"], dtype="<f8")
    raw = np.frombuffer(files[f"bkup_data_{rank:05d}.dat"], dtype="<f8")
    size = int(np.prod(shape))
    st = {k: raw[i * size:(i + 1) * size].reshape(shape).copy() for i, k in enumerate(BKUP_ORDER)}
    return (n, cnt, float(tim), float(dt), float(trec)), st


def outdat_f32(st, cnt, rank=0):
    data = b"".join(np.ascontiguousarray(st[k], dtype="<f8").astype("<f4").tobytes()
                    for k in OUT_ORDER)
    return f"outdat_{cnt:05d}_{rank:05d}.dat", data


def outdat_f64(st, cnt, dim):
    order = OUT_ORDER_1D if dim == 1 else OUT_ORDER
    data = b"".join(np.ascontiguousarray(st[k], dtype="<f8").tobytes() for k in order)
    return f"outdat_{cnt:05d}.dat", data


def meta_files(dim, first, tim, gamma, bx=0.0, xoff=4, yoff=4, zoff=4, t_before=b""):
    out = {}
    if first:
        if dim == 1:
            out["params.dat"] = b"%.12f %.12f\n" % (bx, gamma)
            out["xoff.dat"] = b"%d\n" % xoff
        else:
            out["params.dat"] = b"%f\n" % gamma
            out["offsets.dat"] = (b"%d %d\n" % (xoff, yoff) if dim == 2
                                  else b"%d %d %d\n" % (xoff, yoff, zoff))
        t_before = b""
    out["t.dat"] = t_before + ((b"%.12f\n" if dim == 1 else b"%f\n") % tim)
    return out
