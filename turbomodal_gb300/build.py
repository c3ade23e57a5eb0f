"""In-tree build of libtmg.so (CUDA kernels for sm_103a + host runtime + C ABI).

Compiles the translation units in parallel with nvcc / g++ and links one shared library
next to this file.  No CMake; a rebuild only recompiles sources newer than their object.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtmg.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + CSRC, "-I" + os.path.join(ROOT, "include")] + ARCH
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-I" + CSRC]

# (source, extra flags).  fe.cu is built without FMA contraction so the element
# arithmetic is reproducible operation by operation.
UNITS = [
    ("fe.cu", ["--fmad=false"]),
    ("mf.cu", []),
    ("mf_tc.cu", []),
    ("lz.cu", []),
    ("engine.cu", []),
    ("dense.cu", []),
    ("sym.cpp", []),
]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps_newer(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    for f in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    return os.path.getmtime(os.path.join(ROOT, "include", "turbomodal_gb300.h")) > t


def _compile(src: str, extra: list[str]) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if not _deps_newer(obj, path):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc(), "-c", path, "-o", obj] + NVCC_FLAGS + extra
    else:
        cmd = [os.environ.get("CXX", "g++"), "-c", path, "-o", obj] + CXX_FLAGS + extra
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{out.stdout}\n{out.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(*u), UNITS))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [_nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-lcudart"]
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{out.stdout}\n{out.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
