"""CPU tests of the C ABI library: it loads, exports every symbol that
include/*.h declares (with C and, for the drop-in drivers, the reference's C++
linkage), and rejects bad arguments before touching the GPU."""
import ctypes as C
import glob
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# include/mlau_point.h is header-only: its functions are inline adapters that
# compile into the caller (tests/test_point_api.py builds and checks them)
HEADER_ONLY = ("mlau_point.h",)


def header_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        if os.path.basename(h) in HEADER_ONLY:
            continue
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M):
            if m.group(1) not in ("if", "return", "sizeof"):
                names.append(m.group(1))
    return sorted(set(names))


def exported():
    import mlau_gb300 as M
    out = subprocess.run(["nm", "-D", "--defined-only", M.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_library_loads(gpu_lib):
    assert os.path.exists(gpu_lib.LIB_PATH)


def test_header_symbols_exported(gpu_lib):
    syms = exported()
    missing = [n for n in header_functions() if n not in syms]
    assert not missing, missing
    assert len(header_functions()) >= 20


def test_cxx_linkage_drivers_exported(gpu_lib):
    syms = exported()
    for mangled in ("_Z12mhd_fd_ct_3dPdS_S_S_S_S_S_S_ddddiiiiiidiiii",
                    "_Z12mhd_fd_ct_2dPdS_S_S_S_S_S_S_dddiiiid",
                    "_Z12mhd_fd_ct_2dPdS_S_S_S_S_S_S_dddiiiidiii",
                    "_Z11mhd_fd4c_1dPdS_S_S_S_S_S_dddiid",
                    "_Z14diff_ctfield_ePdS_S_S_ddddiiiidiii",
                    "_Z13ns_viscous_2dPKdPdS1_S1_S1_ddddiiiidiii",
                    "_Z12t_conductionPKdS0_S0_S0_PdS0_S0_S0_ddddiiiidiii"):
        assert mangled in syms


def test_create_rejects_bad_geometry(gpu_lib):
    L = gpu_lib.lib()
    h = C.c_void_p()
    # interior narrower than the ghost depth
    rc = L.mlau_sim_create(C.byref(h), 3, 10, 10, 10, 4, 4, 4, 1.0, 1.0, 1.0, 5 / 3, 4, 0, 3, 0)
    assert rc == -1 and "interior" in gpu_lib.last_error()
    rc = L.mlau_sim_create(C.byref(h), 3, 16, 16, 16, 4, 4, 4, 1.0, 1.0, 1.0, 5 / 3, 7, 0, 3, 0)
    assert rc == -1
    rc = L.mlau_sim_create(C.byref(h), 2, 16, 16, 1, 4, 4, 0, 1.0, 1.0, 1.0, 0.9, 4, 0, 3, 0)
    assert rc == -1 and "gamma" in gpu_lib.last_error()
    rc = L.mlau_sim_create(C.byref(h), 1, 64, 1, 1, 4, 0, 0, 1.0, 1.0, 1.0, 2.0, 2, 0, 3, 1)
    assert rc == -1 and "precision" in gpu_lib.last_error()
    # ghost depth 3: the update's 4-point difference would read a face no
    # flux kernel writes (the reference fixes the depth at 4)
    for dim, g in ((1, (64, 1, 1, 3, 0, 0)), (2, (32, 32, 1, 3, 4, 0)), (3, (32, 32, 32, 4, 4, 3))):
        rc = L.mlau_sim_create(C.byref(h), dim, *g, 1.0, 1.0, 1.0, 5 / 3, 4, 0, 3, 0)
        assert rc == -1 and "ghost depth >= 4" in gpu_lib.last_error()


def test_set_scheme_validation(gpu_lib):
    L = gpu_lib.lib()
    assert L.mlau_set_scheme(3, 7, 0, 3) == -1
    assert L.mlau_set_scheme(3, 4, 9, 3) == -1
    assert L.mlau_set_bc_1d(7) == -1


def test_loading_fails_loudly_without_library(tmp_path, monkeypatch):
    import mlau_gb300 as M
    monkeypatch.setattr(M, "_lib", None)
    monkeypatch.setattr(M, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(M.MlauError):
        M.lib()


def test_problem_boundary_tables_reach_the_library(tmp_path):
    """A program that defines dnxs / dnys (as every reference problem's
    global.hpp does) overrides the library's weak all-zero tables."""
    import mlau_gb300
    import subprocess
    src = os.path.join(os.path.dirname(__file__), "c", "tables_probe.c")
    exe = tmp_path / "tables_probe"
    libdir = os.path.dirname(mlau_gb300.LIB_PATH)
    subprocess.run(["gcc", "-O1", src, "-o", str(exe), f"-L{libdir}", "-lmlau_gb300",
                    f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    got = np.array([int(v) for v in out]).reshape(8, 3)
    assert list(got[:, 0]) == [0] * 8
    assert list(got[:, 1]) == [1, 1, -1, 1, 1, 1, -1, 1]
    assert list(got[:, 2]) == [0] * 8


@pytest.mark.parametrize("prog", ("khi_dropin.c", "mrx_dropin.cpp"))
def test_problem_programs_link(gpu_lib, tmp_path, prog):
    """Programs in the shape of the reference's problems (their tables, the
    reference's prototypes, C or C++ linkage) link against the library
    alone: every driver symbol they use resolves (running them needs a GPU)."""
    src = os.path.join(ROOT, "tests", "c", prog)
    libdir = os.path.dirname(gpu_lib.LIB_PATH)
    cc = "g++" if prog.endswith(".cpp") else "gcc"
    r = subprocess.run([cc, "-O1", src, "-o", str(tmp_path / "a.out"), f"-L{libdir}",
                        "-lmlau_gb300", f"-Wl,-rpath,{libdir}", "-Wl,--no-undefined"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
