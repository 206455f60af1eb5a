"""The C-ABI library loads and exports every entry point include/avbdg.h declares (no GPU needed),
the checkers export the same world API, and the scene generators are deterministic."""

import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "avbdg.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(avbdg_\w+)\s*\(", text, re.M)))


def test_header_declares_the_world_api():
    syms = header_symbols()
    for name in ["avbdg_world_create", "avbdg_world_step", "avbdg_world_step_interleaved",
                 "avbdg_world_get_body_state", "avbdg_world_dump_broadphase", "avbdg_last_error"]:
        assert name in syms


def test_library_exports_every_declared_symbol(pkg):
    lib_path = pkg.LIB_PATH
    if not os.path.exists(lib_path):
        from avbd_gb300 import build

        build.build()
    lib = ctypes.CDLL(lib_path)
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_params_default_matches_reference_defaults(pkg, oracle):
    lib = ctypes.CDLL(pkg.LIB_PATH)
    api_fn = lib.avbdg_params_default
    p = pkg.capi.Params()
    api_fn.argtypes = [ctypes.POINTER(pkg.capi.Params)]
    assert api_fn(ctypes.byref(p)) == 0
    q = oracle.default_params()
    for name, _ in pkg.capi.Params._fields_:
        assert getattr(p, name) == getattr(q, name), name


def test_reference_defaults(pkg, ref, oracle):
    a, b = ref.default_params(), oracle.default_params()
    for name, _ in pkg.capi.Params._fields_:
        assert getattr(a, name) == getattr(b, name), name


def test_world_create_without_gpu_fails_loudly(pkg):
    """On a machine with no CUDA device the GPU world refuses to exist (no CPU fallback)."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible here")
    with pytest.raises(pkg.capi.AvbdError) as e:
        pkg.world()
    assert e.value.code == pkg.capi.ERR_CUDA


def test_scene_generators_are_deterministic(pkg):
    s = pkg.scenes
    a, b = s.pile(count=200), s.pile(count=200)
    assert np.array_equal(a.position, b.position) and np.array_equal(a.orientation, b.orientation)
    p = s.pyramid420()
    assert p.n == 421 and p.dynamic == 420
    lat = s.lattice(nx=4, ny=4, nz=2)
    assert lat.n == 33
    full = s.pile()
    assert full.dynamic == 1653 + 32 and len(full.joints) == 32


def test_cpp_facade_compiles(tmp_path):
    """The C++ facade (include/avbdg_solver.hpp) and a host program written against it compile
    (linking and running need the GPU library and a device: tests/test_gpu_facade.py)."""
    import shutil
    import subprocess

    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off",
                    "-I" + os.path.join(ROOT, "include"), "-c", os.path.join(ROOT, "tests", "cpp", "facade_scenes.cpp"),
                    "-o", str(tmp_path / "facade.o")], check=True)
