"""Build recipes for the CPU checker (test infrastructure only).

* ``build_oracle()`` compiles ``oracle/oracle.c`` (the C restatement) into
  ``oracle/liboracle.so`` with the host compiler; it builds on x86-64 and
  aarch64 alike.
* ``build_ref()`` compiles the reference's own hot-path sources, read where they
  lie in the reference tree, together with ``oracle/ref/ref_driver.cpp`` and
  the 1-rank ``oracle/ref/mpi.h`` into ``oracle/_ref/``:

  - ``libref_base.so``: ``src/base/{gt_combine,gt_popcnt,mi_compute}.cpp``,
    no ``ALIGN`` (the portable scalar build);
  - ``libref_base_seg.so``: the same with ``-DSEGMENT_SIZE=1474560``
    (``src/CMakeLists.txt:260-262``): ``ThreadedSearch`` runs its segmented
    search (``ThreadedSearch.h:65-69,79-140``);
  - ``libref_bench.so``: ``oracle/ref/bench_driver.cpp`` over the two
    sequential benchmark programs (``benchmarks/*_sequential_search.cpp``,
    their depth-first ``stack_search``) with the scalar kernels;
  - ``libref_avx512.so``: ``src/avx512bw/{gt_combine,gt_popcnt_avx512bw_lu,
    mi_compute_512}.cpp`` with ``-DALIGN=64 -march=native -ffast-math -lmvec``
    (the reference's default build on an AVX-512BW CPU without VPOPCNTDQ,
    ``src/CMakeLists.txt:18-77,208-252``), only on x86-64 hosts with avx512bw.

  Nothing is built when the reference tree is absent.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference tree this recipe compiles from: FIUNCHO_REFERENCE, else the
# development container's read-only checkout (absent on the GPU hosts, where
# nothing of it is built or read).
REF_ROOT = os.environ.get("FIUNCHO_REFERENCE", "/root/reference")
REF_OUT = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(HERE, "liboracle.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.c")
    if force or _stale(ORACLE_SO, [src, os.path.join(HERE, "ref", "tabledigest.h"), os.path.abspath(__file__)]):
        # hardware popcount: part of the aarch64 base ISA, an explicit flag on x86-64
        isa = ["-mpopcnt"] if platform.machine() in ("x86_64", "AMD64") else []
        _run(["gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", "-pthread"] + isa + [src, "-o", ORACLE_SO + ".tmp",
                                                                                      "-lm"])
        os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def reference_present() -> bool:
    return os.path.isdir(os.path.join(REF_ROOT, "include", "fiuncho"))


def _has_avx512bw() -> bool:
    if platform.machine() not in ("x86_64", "AMD64"):
        return False
    try:
        with open("/proc/cpuinfo") as f:
            return " avx512bw" in f.read()
    except OSError:
        return False


def build_ref(force: bool = False) -> dict:
    """Returns {name: path} of the reference libraries built (empty if the
    reference tree is not present)."""
    if not reference_present():
        return {}
    os.makedirs(REF_OUT, exist_ok=True)
    inc = ["-I", os.path.join(REF_ROOT, "include"), "-I", os.path.join(HERE, "ref")]
    driver = os.path.join(HERE, "ref", "ref_driver.cpp")
    shim = os.path.join(HERE, "ref", "mpi.h")
    digest_h = os.path.join(HERE, "ref", "tabledigest.h")
    built = {}
    base_srcs = [os.path.join(REF_ROOT, "src", "base", f) for f in ("gt_combine.cpp", "gt_popcnt.cpp", "mi_compute.cpp")]
    out = os.path.join(REF_OUT, "libref_base.so")
    if force or _stale(out, [driver, shim, digest_h] + base_srcs):
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread"] + inc + [driver] + base_srcs + ["-o", out])
    built["base"] = out
    out = os.path.join(REF_OUT, "libref_base_seg.so")
    if force or _stale(out, [driver, shim, digest_h] + base_srcs):
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", "-DSEGMENT_SIZE=1474560"] + inc +
             [driver] + base_srcs + ["-o", out])
    built["base_seg"] = out
    bench_driver = os.path.join(HERE, "ref", "bench_driver.cpp")
    bench_srcs = [os.path.join(REF_ROOT, "benchmarks", f)
                  for f in ("nonsegmented_sequential_search.cpp", "segmented_sequential_search.cpp", "utils.h")]
    out = os.path.join(REF_OUT, "libref_bench.so")
    if force or _stale(out, [bench_driver, shim] + bench_srcs + base_srcs):
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread"] + inc +
             ["-I", os.path.join(REF_ROOT, "benchmarks"), bench_driver] + base_srcs + ["-o", out])
    built["bench"] = out
    if _has_avx512bw():
        d = os.path.join(REF_ROOT, "src", "avx512bw")
        srcs = [os.path.join(d, f) for f in ("gt_combine.cpp", "gt_popcnt_avx512bw_lu.cpp", "mi_compute_512.cpp")]
        out = os.path.join(REF_OUT, "libref_avx512.so")
        if force or _stale(out, [driver, shim, digest_h] + srcs):
            _run(["g++", "-O3", "-std=c++17", "-march=native", "-ffast-math", "-DALIGN=64", "-fPIC", "-shared",
                  "-pthread"] + inc + [driver] + srcs + ["-o", out, "-lmvec"])
        built["avx512"] = out
    return built


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
