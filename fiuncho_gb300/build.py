"""In-tree build of the CUDA library ``fiuncho_gb300/libfiuncho_gpu.so``.

Every ``csrc/*.cu`` translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into
one shared object with the CUDA runtime linked statically.  No torch, no
cmake: nvcc and the host compiler only.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "libfiuncho_gpu.so")
OBJ = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
                  "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfiuncho_gpu.so")
    return p


def _compile(src: str, extra) -> str:
    obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + NVFLAGS + list(extra) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


CPP_INCLUDE = os.path.join(HERE, "cpp", "include")
BIN = os.path.join(HERE, "bin")
CPP_TARGETS = {
    "fiuncho_gpu": os.path.join(HERE, "cpp", "fiuncho_gpu_main.cpp"),
    "test_gpusearch": os.path.join(os.path.dirname(HERE), "tests", "cpp", "test_gpusearch.cpp"),
    "dump_dataset": os.path.join(os.path.dirname(HERE), "tests", "cpp", "dump_dataset.cpp"),
}


def build_cpp(force: bool = False) -> dict:
    """The C++ host side: the CLI and the C++ drop-in test, linked against the library."""
    lib = build()
    os.makedirs(BIN, exist_ok=True)
    headers = glob.glob(os.path.join(CPP_INCLUDE, "fiuncho", "**", "*.h*"), recursive=True) + \
        glob.glob(os.path.join(INCLUDE, "**", "*.h"), recursive=True)
    out = {}
    for name, src in CPP_TARGETS.items():
        exe = os.path.join(BIN, name)
        deps = [src, lib] + headers
        if force or not os.path.exists(exe) or any(os.path.getmtime(d) > os.path.getmtime(exe) for d in deps):
            cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2", "-I", CPP_INCLUDE, "-I", INCLUDE, src,
                   "-o", exe, "-L", HERE, "-lfiuncho_gpu", "-Wl,-rpath," + HERE, "-pthread"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("g++ failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        out[name] = exe
    return out


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
