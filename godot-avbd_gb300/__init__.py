"""GB300 AVBD rigid-body time-step: Python host side of the C ABI in include/avbdg.h.

The compute path is libavbdg.so (hand-written sm_103a kernels behind a C ABI). There is no CPU
fallback: `gpu_api()` raises if the library is not built or no CUDA device is visible.
"""

import ctypes
import os

from . import capi, scenes  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libavbdg.so")

_gpu = None


def load_library(path=LIB_PATH):
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with build.build() (no CPU fallback exists)")
    return ctypes.CDLL(path)


def gpu_api():
    """The avbdg_* world API of the GPU library."""
    global _gpu
    if _gpu is None:
        _gpu = capi.Api(load_library(), "avbdg_")
    return _gpu


def world(params=None, max_bodies=0, max_forces=0):
    """A new GPU world (one avbd::Solver equivalent)."""
    return capi.World(gpu_api(), params, max_bodies, max_forces)
