"""GB300 AVBD rigid-body time-step: Python host side of the C ABI in include/avbdg.h.

The compute path is libavbdg.so (hand-written sm_103a kernels behind a C ABI). There is no CPU
fallback: `gpu_api()` raises if the library is not built or no CUDA device is visible.
"""

import ctypes
import os

from . import capi, scenes  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libavbdg.so")
# The same kernels compiled with every floating-point value of the step in double precision; only
# used to state the float32 result's rounding error.
LIB64_PATH = os.path.join(HERE, "_build", "libavbdg64.so")

_gpu = {}


def load_library(path=LIB_PATH):
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with build.build() (no CPU fallback exists)")
    return ctypes.CDLL(path)


def gpu_api(fp64=False):
    """The avbdg_* world API of the GPU library (fp64=True: the FP64 build of the same kernels)."""
    if fp64 not in _gpu:
        _gpu[fp64] = capi.Api(load_library(LIB64_PATH if fp64 else LIB_PATH), "avbdg_")
    return _gpu[fp64]


def world(params=None, max_bodies=0, max_forces=0):
    """A new GPU world (one avbd::Solver equivalent)."""
    return capi.World(gpu_api(), params, max_bodies, max_forces)
