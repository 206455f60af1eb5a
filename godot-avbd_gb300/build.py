"""Build the GPU libraries in-tree, one nvcc process per translation unit:

  _build/libavbdg.so    the step in float32, bit for bit the reference's arithmetic
  _build/libavbdg64.so  the same sources compiled with -DAVBDG_FP64: every floating-point value of
                        the step in double precision (used to state the float32 result's error)

Floating-point flags are part of the contract: the step reproduces the reference solver bit for
bit only with no FMA contraction (device: --fmad=false; host: -ffp-contract=off) and IEEE
division and square root (nvcc's defaults, restated here).
"""

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libavbdg.so")
LIB64 = os.path.join(OUT, "libavbdg64.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-std=c++17", "-lineinfo",
    "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
    "-I" + os.path.join(ROOT, "include"),
]
SOURCES = ["prims.cu", "k_broad.cu", "k_manifold.cu", "k_solve.cu", "k_proj.cu", "k_io.cu", "k_relocate.cu", "k_sleep.cu", "k_query.cu", "engine.cu",
           "capi.cu", "server.cu", "sortkeys.cu"]
# (library, object directory, extra flags)
VARIANTS = [(LIB, OUT, []), (LIB64, os.path.join(OUT, "fp64"), ["-DAVBDG_FP64"])]


def nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else "nvcc"


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    """Compile every translation unit that changed and link both libraries. Returns the float32
    library's path."""
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    headers.append(os.path.join(ROOT, "include", "avbdg.h"))
    jobs, links = [], []
    for lib, objdir, extra in VARIANTS:
        os.makedirs(objdir, exist_ok=True)
        objs, changed = [], False
        for src in SOURCES:
            s = os.path.join(CSRC, src)
            o = os.path.join(objdir, src.replace(".cu", ".o"))
            objs.append(o)
            if force or _stale(o, [s] + headers):
                jobs.append([nvcc()] + NVCC_FLAGS + extra + ["-c", s, "-o", o])
                changed = True
        if changed or not os.path.exists(lib):
            links.append([nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs) + 1, os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
        list(ex.map(run, links))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
