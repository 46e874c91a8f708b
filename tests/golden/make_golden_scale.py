"""Generates ``reference_scale.npz``: the reference's own results on the
full-size workloads, for the full-size parity tests.

Run where the reference tree is present (``FIUNCHO_REFERENCE`` names it):

    FIUNCHO_REFERENCE=<reference tree> python tests/golden/make_golden_scale.py [name ...]

It builds the reference's sources through ``oracle/build.py`` and calls them
through ``oracle/ref/ref_driver.cpp``.  The AVX-512BW build (the reference's
default build on this CPU, ``-DALIGN=64``) is used when it exists, else the
portable scalar build; both give identical tables.  For each workload of
``WORKLOADS`` below (seeded synthetic data from ``fiuncho_gb300.synth``):

* ``<name>_sha256``  -- SHA-256 of the packed data set (unaligned rows, the
  layout the library receives), so a test can tell whether the data it
  regenerated is the data the reference saw;
* ``<name>_digest``, ``<name>_count`` -- the digest of the reference's
  contingency tables of EVERY combination of the scan (oracle/ref/tabledigest.h:
  a 64-bit sum over combinations of a hash of the combination and its 3^k x 2
  cells, from GenotypeTable::combine / combine_and_popcnt), as uint64;
* ``<name>_combos``, ``<name>_vals`` -- ThreadedSearch::run's top-N
  (Distribution(snps, order-1, 1, 0), FP32 MI) with 8 threads;
* ``<name>_seconds`` -- wall time of the two reference runs.

The file holds a few KB, whatever the workload sizes.
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from fiuncho_gb300 import synth  # noqa: E402
from fiuncho_gb300.dataset import Dataset  # noqa: E402
from oracle import build as obuild  # noqa: E402
from oracle.oracle import Reference  # noqa: E402

# name -> (ScanSpec, what the library runs it on)
WORKLOADS = {
    # order 2, 1 000 x 2 000/2 000: packed-class order-2 tensor kernel
    "order2_1000x4000": synth.WORKLOADS["order2_1000x4000"],
    # order 3, 2 000 x 4 000/4 000 (the headline): packed-class order-3 tensor kernel
    "order3_2000x8000": synth.WORKLOADS["order3_2000x8000"],
    # order 2, 40 000 x 8 000/8 000: per-class order-2 tensor kernel
    "order2_40000x16000": synth.WORKLOADS["order2_40000x16000"],
    # order 4, 300 x 4 000/4 000: packed-class order-4 tensor kernel
    "order4_300x8000": synth.WORKLOADS["order4_300x8000"],
    # order 3 and 4 with classes too large to pack (9 000 / 9 800): per-class tensor kernels
    "order3_500x18800": synth.WORKLOADS["order3_500x18800"],
    "order4_100x18800": synth.WORKLOADS["order4_100x18800"],
}

THREADS = 8


def packed_sha256(ds) -> str:
    return hashlib.sha256(np.ascontiguousarray(ds.data, np.uint64).tobytes()).hexdigest()


def main(names):
    if not obuild.reference_present():
        sys.exit("reference tree not found; set FIUNCHO_REFERENCE")
    try:
        ref, align = Reference("avx512"), 64
    except FileNotFoundError:
        ref, align = Reference("base"), 0
    out_path = os.path.join(HERE, "reference_scale.npz")
    out = dict(np.load(out_path)) if os.path.exists(out_path) else {}
    out["build"] = np.array(ref.flavour)
    for name in names:
        spec = WORKLOADS[name]
        geno, is_case, _ = synth.simulate(spec)
        ds = Dataset.from_genotypes(geno, is_case)
        da = Dataset.from_genotypes(geno, is_case, align=align) if align else ds
        del geno
        rd = ref.from_packed(da.data, da.snps, da.cases, da.ctrls, da.cases_words, da.ctrls_words)
        t0 = time.time()
        dg, cnt = rd.table_digest(spec.order, threads=THREADS)
        t1 = time.time()
        c, v = rd.search(spec.order, spec.outputs, threads=THREADS)
        t2 = time.time()
        out[name + "_sha256"] = np.array(packed_sha256(ds))
        out[name + "_digest"] = np.array(dg, np.uint64)
        out[name + "_count"] = np.array(cnt, np.uint64)
        out[name + "_combos"] = c
        out[name + "_vals"] = v
        out[name + "_seconds"] = np.array([t1 - t0, t2 - t1])
        print("%s: digest %d over %d combinations (%.1f s), top-%d (%.1f s)" % (name, dg, cnt, t1 - t0,
                                                                                spec.outputs, t2 - t1), flush=True)
        np.savez(out_path, **out)


if __name__ == "__main__":
    main(sys.argv[1:] or list(WORKLOADS))
