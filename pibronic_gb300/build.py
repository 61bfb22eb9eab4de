"""Build the CUDA library ``_lib/libpibronic_gb300.so`` for sm_103a with nvcc.

Each ``csrc/*.cu`` is compiled to an object in parallel (one ``-gencode``), then linked into one
shared library in the package tree.  Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT_DIR = os.path.join(HERE, "_lib")
LIB_NAME = "libpibronic_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I" + INCLUDE]


def _nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pibronic_gb300")
    return path


def _deps():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def lib_path():
    return os.path.join(OUT_DIR, LIB_NAME)


def build(verbose=False, jobs=None):
    """Compile and link; returns the library path.  Raises RuntimeError on a compiler error."""
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    deps = _deps()
    objs, todo = [], []
    for src in sources:
        obj = os.path.join(OUT_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + deps):
            todo.append((src, obj))

    def compile_one(item):
        src, obj = item
        cmd = [nvcc] + ARCH + FLAGS + ["-c", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{res.stderr}")
        if verbose:
            print(os.path.basename(src), res.stderr.strip(), file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, max(1, os.cpu_count() or 1))) as ex:
        list(ex.map(compile_one, todo))
    lib = lib_path()
    if todo or _stale(lib, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stderr}")
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
