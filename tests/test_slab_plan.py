"""The plane schedule of the host-array FP32-split step
(mlau_gb300/csrc/slab_plan.h), replayed on the CPU by tests/c/slab_plan_check.cpp
against the kernels' own z read / write sets: every kernel reads planes that
this stage has produced (state planes: uploaded and waited for, at the right
RK version), no update overwrites a plane a later primitive recovery reads,
each plane goes back to the host once at its final version.  Grids of 4 to 300
interior planes, ghost depths 4 and 5, RK1-3, 1-16 slabs, 1-64 planes per
upload, z-tiles of 5, 16 and 32 cells."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_slab_plans_respect_every_dependence(tmp_path):
    exe = tmp_path / "slab_plan_check"
    subprocess.run(["g++", "-O2", "-std=c++17", os.path.join(ROOT, "tests", "c", "slab_plan_check.cpp"),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok ") and int(out.stdout.split()[1]) > 10000
