"""The C++ facade (include/avbdg_solver.hpp): a host program written the way code drives the
reference's avbd::Solver (fields, `new Rigid`, `new Joint`, step(), Rigid fields read back) is
compiled against the facade and the GPU library and must reproduce the digests the reference's
suite pins for its scenes."""

import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_gpu_facade_program_reproduces_pinned_digests(pkg, gpu, tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    lib_dir = os.path.dirname(pkg.LIB_PATH)
    exe = tmp_path / "facade_scenes"
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "facade_scenes.cpp"), "-o", str(exe), "-L" + lib_dir,
                    "-lavbdg", "-Wl,-rpath," + lib_dir], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {line.split()[0]: line.split() for line in out if line.strip()}
    pinned = pkg.scenes.PINNED_DIGESTS
    for name in ("stack", "interleaved", "mixed"):
        assert int(got[name][1], 16) == pinned[name], f"{name}: {got[name][1]}"
    assert int(got["mixed"][3]) > 0 and int(got["mixed"][5]) > 0
