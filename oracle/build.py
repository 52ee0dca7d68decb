"""Build recipes for the two CPU oracles.  TEST INFRASTRUCTURE ONLY.

* ``build_port()`` compiles this directory's C restatement
  (mlau_oracle.c) into ``oracle/_build/liboracle.so``.  It needs only gcc and
  works on any host, including the GPU machine.
* ``build_ref_variant(...)`` compiles the reference's own driver and boundary
  sources, read where they lie under the reference tree, into
  ``oracle/_ref/``.  The reference selects its scheme with ``#define`` lines
  and an uncommented ``func_flux=`` assignment inside each driver, so the
  recipe writes sed-style patched copies of those files into
  ``oracle/_ref/src/<variant>/`` (build intermediates, never committed) and
  compiles them with ``-O2 -fopenmp -ffp-contract=off`` (the reference's own
  flags, Makefile.inc:4, plus an explicit no-contraction flag) and the
  single-rank ``ref_stub/mpi.h``.

Usage: ``python oracle/build.py [--port] [--ref-all]``.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# the reference checkout: MLAU_REFERENCE_ROOT, else a directory named
# "reference" beside this repository's root
REF_ROOT = os.environ.get("MLAU_REFERENCE_ROOT") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")

FLUX_NAMES = {0: "mlau", 1: "lhlld", 2: "hlld", 3: "roe"}
CFLAGS = ["-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]


def port_path() -> str:
    return os.path.join(BUILD, "liboracle.so")


def build_port(force: bool = False) -> str:
    """Compile the C restatement; return the shared library path."""
    os.makedirs(BUILD, exist_ok=True)
    out = port_path()
    srcs = [os.path.join(HERE, f) for f in ("mlau_oracle.c", "mlau_oracle.h", "oracle_point.h")]
    if not force and os.path.exists(out):
        if os.path.getmtime(out) >= max(os.path.getmtime(s) for s in srcs):
            return out
    tmp = out + f".tmp{os.getpid()}"
    cmd = ["gcc", "-std=gnu11", *CFLAGS, "-o", tmp, os.path.join(HERE, "mlau_oracle.c"), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, out)
    return out


def reference_available() -> bool:
    return os.path.isfile(os.path.join(REF_ROOT, "include", "mhd_flux.h"))


def _variant_name(dim: int, odr: int, flux: int, nrk: int, bc: str, miyoshi: bool = False) -> str:
    return (f"ref{dim}d_o{odr}_{FLUX_NAMES[flux]}_rk{nrk}" + (f"_{bc}" if dim == 1 else "")
            + ("_mi" if miyoshi else ""))


# reconstruction codes 5 and 6: ODR 2 with calc_flr's MUSCL limiter swapped
# for the MC or Koren limiter of include/interp.h
LIMITER_SWAP = {5: "muscl_mc_cal_flr", 6: "muscl_kr_cal_flr"}


def _patch_driver(text: str, odr: int, flux: int, nrk: int, miyoshi: bool = False) -> str:
    if miyoshi:
        # the header's alternative eigen-system where the driver uses the full one
        text, nm = re.subn(r"\bmhd_c_reconst\(", "mhd_m_reconst(", text)
        if nm < 1:
            raise RuntimeError("reference driver layout not recognised; eigen patch failed")
    if odr in LIMITER_SWAP:
        text, n0 = re.subn(r"^(\s*)muscl_mm_cal_flr\(f\[1\],f\[2\],f\[3\],fl,fr\);",
                           lambda m: f"{m.group(1)}{LIMITER_SWAP[odr]}(f[1],f[2],f[3],fl,fr);",
                           text, count=1, flags=re.M)
        if n0 != 1:
            raise RuntimeError("reference calc_flr layout not recognised; limiter patch failed")
        odr = 2
    text, n1 = re.subn(r"^#define ODR \(\d\)", f"#define ODR ({odr})", text, count=1, flags=re.M)
    text, n2 = re.subn(r"^#define R_K \(\d\)", f"#define R_K ({nrk})", text, count=1, flags=re.M)
    text, n3 = re.subn(r"^(\s*)func_flux=&calc_flux_lhlld;",
                       lambda m: f"{m.group(1)}func_flux=&calc_flux_{FLUX_NAMES[flux]};",
                       text, count=1, flags=re.M)
    if (n1, n2, n3) != (1, 1, 1):
        raise RuntimeError("reference driver layout not recognised; patch failed")
    return text


REPO_INCLUDE = os.path.join(os.path.dirname(HERE), "include")
POINT_HEADERS = ("funcs.h", "interp.h", "mhd_eigen.h", "mhd_flux.h")


def point_shim_dir() -> str:
    """A directory of one-line headers named as the reference's point-function
    headers, each including this library's include/mlau_point.h: put first on
    the include path, it swaps the reference's point functions for the
    library's in a reference driver compiled unchanged."""
    d = os.path.join(REF_OUT, "shim")
    os.makedirs(d, exist_ok=True)
    for h in POINT_HEADERS:
        path = os.path.join(d, h)
        text = '#include "mlau_point.h"\n'
        if not os.path.exists(path) or open(path).read() != text:
            with open(path, "w") as fh:
                fh.write(text)
    return d


def build_ref_variant(dim: int, odr: int = 4, flux: int = 0, nrk: int = 3,
                      bc: str = "open", miyoshi: bool = False, headers: str = "ref") -> str:
    """Compile one scheme variant of the reference driver; return the .so path.

    dim 3: 3D/MPI/OTvortex/{mhd_fd_ct_3d.c,boundary.c}
    dim 2: 2D/SERIAL/OTvortex/{mhd_fd_ct_2d.c,boundary.c}
    dim 1: 1D/SERIAL/shock/{mhd_fd4c_1d.c,openbc1d_mhd.c} (bc="open") or
           1D/SERIAL/wave/{mhd_fd4c_1d.c,prdc_1d.c} (bc="periodic")
    headers "mlau": the same driver sources compiled against include/mlau_point.h
    in place of the reference's include/{funcs,interp,mhd_eigen,mhd_flux}.h.
    """
    if not reference_available():
        raise FileNotFoundError(f"reference tree not found at {REF_ROOT}")
    name = _variant_name(dim, odr, flux, nrk, bc, miyoshi) + ("_mlauhdr" if headers == "mlau" else "")
    out = os.path.join(REF_OUT, f"lib{name}.so")
    if os.path.exists(out):
        return out
    if dim == 3:
        d, drv, extra = "3D/MPI/OTvortex", "mhd_fd_ct_3d.c", ["boundary.c"]
    elif dim == 2:
        d, drv, extra = "2D/SERIAL/OTvortex", "mhd_fd_ct_2d.c", ["boundary.c"]
    elif bc == "open":
        d, drv, extra = "1D/SERIAL/shock", "mhd_fd4c_1d.c", ["openbc1d_mhd.c"]
    else:
        d, drv, extra = "1D/SERIAL/wave", "mhd_fd4c_1d.c", ["prdc_1d.c"]
    src_dir = os.path.join(REF_OUT, "src", name)
    os.makedirs(src_dir, exist_ok=True)
    with open(os.path.join(REF_ROOT, d, drv)) as fh:
        patched = _patch_driver(fh.read(), odr, flux, nrk, miyoshi)
    drv_copy = os.path.join(src_dir, drv.replace(".c", ".cpp"))
    with open(drv_copy, "w") as fh:
        fh.write(patched)
    srcs = [drv_copy] + [os.path.join(REF_ROOT, d, e) for e in extra]
    tmp = out + f".tmp{os.getpid()}"
    inc = ["-I" + point_shim_dir(), "-I" + REPO_INCLUDE] if headers == "mlau" else []
    cmd = ["g++", "-x", "c++", *CFLAGS, f"-DREF_DIM={dim}", *inc,
           "-I" + os.path.join(REF_ROOT, "include"), "-I" + os.path.join(HERE, "ref_stub"),
           "-o", tmp, *srcs, os.path.join(HERE, "ref_harness.cpp"), "-lm"]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)
    os.replace(tmp, out)
    return out


def build_point_harness(headers: str = "ref", out: str | None = None) -> str:
    """Compile oracle/point_harness.cpp against the reference's point-function
    headers (headers "ref", into oracle/_ref/libpoint_ref.so; needs the
    reference tree) or against include/mlau_point.h (headers "mlau", into
    `out`); return the .so path."""
    src = os.path.join(HERE, "point_harness.cpp")
    if headers == "ref":
        if not reference_available():
            raise FileNotFoundError(f"reference tree not found at {REF_ROOT}")
        out = out or os.path.join(REF_OUT, "libpoint_ref.so")
        inc = ["-DMLAU_POINT_REF", "-I" + os.path.join(REF_ROOT, "include")]
    else:
        out = out or os.path.join(BUILD, "libpoint_mlau.so")
        inc = ["-I" + REPO_INCLUDE]
    deps = [src] + ([os.path.join(REPO_INCLUDE, "mlau_point.h"),
                     os.path.join(os.path.dirname(HERE), "mlau_gb300", "csrc", "point.cuh")]
                    if headers != "ref" else [])
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    tmp = out + f".tmp{os.getpid()}"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w", *inc,
           "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)
    os.replace(tmp, out)
    return out


def build_ref_io() -> str:
    """Compile the reference's checkpoint and output routines
    (3D/MPI/OTvortex/bkup.hpp, 3D/MPI/OTvortex/dataio.hpp,
    2D/SERIAL/OTvortex/dataio.hpp) into oracle/_ref/libref_io.so through
    oracle/ref_io_harness.cpp; return its path."""
    if not reference_available():
        raise FileNotFoundError(f"reference tree not found at {REF_ROOT}")
    out = os.path.join(REF_OUT, "libref_io.so")
    src = os.path.join(HERE, "ref_io_harness.cpp")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    os.makedirs(REF_OUT, exist_ok=True)
    tmp = out + f".tmp{os.getpid()}"
    cmd = ["g++", "-O1", "-fPIC", "-shared", "-w", "-I" + REF_ROOT, "-o", tmp, src]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)
    os.replace(tmp, out)
    return out


def build_ref_mrx(odr: int = 2, nrk: int = 3) -> str:
    """Compile the reference's 2D MRX driver file (hyperbolic step with the MC
    limiter, resistive and viscous operators; 2D/MPI/MRX/mhd_fd_ct_2d.c with its
    ODR / R_K lines set) and 2D/MPI/MRX/boundary.c with the single-rank mpi.h
    stub and oracle/ref_mrx_harness.cpp; return the .so path."""
    if not reference_available():
        raise FileNotFoundError(f"reference tree not found at {REF_ROOT}")
    name = f"ref_mrx_o{odr}_rk{nrk}"
    out = os.path.join(REF_OUT, f"lib{name}.so")
    harness = os.path.join(HERE, "ref_mrx_harness.cpp")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(harness):
        return out
    d = os.path.join(REF_ROOT, "2D/MPI/MRX")
    with open(os.path.join(d, "mhd_fd_ct_2d.c")) as fh:
        text = fh.read()
    text, n1 = re.subn(r"^#define ODR \(\d\)", f"#define ODR ({odr})", text, count=1, flags=re.M)
    text, n2 = re.subn(r"^#define R_K \(\d\)", f"#define R_K ({nrk})", text, count=1, flags=re.M)
    if (n1, n2) != (1, 1):
        raise RuntimeError("reference MRX driver layout not recognised; patch failed")
    src_dir = os.path.join(REF_OUT, "src", name)
    os.makedirs(src_dir, exist_ok=True)
    drv = os.path.join(src_dir, "mhd_fd_ct_2d.cpp")
    with open(drv, "w") as fh:
        fh.write(text)
    tmp = out + f".tmp{os.getpid()}"
    cmd = ["g++", "-x", "c++", *CFLAGS, "-I" + os.path.join(REF_ROOT, "include"),
           "-I" + os.path.join(HERE, "ref_stub"), "-o", tmp, drv, os.path.join(d, "boundary.c"),
           harness, "-lm"]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)
    os.replace(tmp, out)
    return out


def build_ref_rmi() -> str:
    """Compile the reference's RMI inflow routine (2D/MPI/RMI/inj_ro.hpp) with
    oracle/ref_rmi_harness.cpp; return the .so path."""
    if not reference_available():
        raise FileNotFoundError(f"reference tree not found at {REF_ROOT}")
    out = os.path.join(REF_OUT, "libref_rmi.so")
    harness = os.path.join(HERE, "ref_rmi_harness.cpp")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(harness):
        return out
    os.makedirs(REF_OUT, exist_ok=True)
    tmp = out + f".tmp{os.getpid()}"
    cmd = ["g++", "-x", "c++", *CFLAGS, "-I" + os.path.join(REF_ROOT, "2D/MPI/RMI"),
           "-I" + os.path.join(HERE, "ref_stub"), "-o", tmp, harness, "-lm"]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)
    os.replace(tmp, out)
    return out


def all_variants():
    for dim in (3, 2):
        for odr in (1, 2, 3, 4):
            for flux in (0, 1, 2, 3):
                yield dict(dim=dim, odr=odr, flux=flux, nrk=3)
        for nrk in (1, 2):
            yield dict(dim=dim, odr=4, flux=0, nrk=nrk)
        for odr in (5, 6):
            for flux in (0, 1):
                yield dict(dim=dim, odr=odr, flux=flux, nrk=3)
    for bc in ("open", "periodic"):
        for odr in (1, 2, 3, 4):
            for flux in (0, 1, 2, 3):
                yield dict(dim=1, odr=odr, flux=flux, nrk=3, bc=bc)
        for odr in (5, 6):
            yield dict(dim=1, odr=odr, flux=0, nrk=3, bc=bc)
    # Miyoshi's eigen-system swapped in where the drivers use the full one
    for dim in (3, 2):
        for odr, flux in ((4, 0), (4, 1), (2, 1), (3, 2)):
            yield dict(dim=dim, odr=odr, flux=flux, nrk=3, miyoshi=True)
    for odr, flux in ((2, 0), (4, 2)):
        yield dict(dim=1, odr=odr, flux=flux, nrk=3, bc="open", miyoshi=True)


def build_ref_all(jobs: int = 8) -> list:
    with ThreadPoolExecutor(jobs) as ex:
        return list(ex.map(lambda kw: build_ref_variant(**kw), all_variants()))


if __name__ == "__main__":
    args = sys.argv[1:] or ["--port"]
    if "--port" in args:
        print(build_port(force=True))
    if "--ref-all" in args:
        for p in build_ref_all():
            print(p)
