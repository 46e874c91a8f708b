"""Generates ``reference_traversals.npz`` from the reference itself.

Run where the reference tree is present (``FIUNCHO_REFERENCE`` names it):

    python tests/golden/make_golden_traversals.py

It builds, through ``oracle/build.py``, the reference's ``ThreadedSearch`` with
``-DSEGMENT_SIZE=1474560`` (its segmented search, ``ThreadedSearch.h:79-140``)
and the two sequential benchmark programs
(``benchmarks/{non,}segmented_sequential_search.cpp``: a depth-first
traversal with a static stack, MI evaluated per combination or in blocks of
1 474 560 / 3^order tables) and records, per case, the genotype codes and
each variant's top-N (combinations and FP32 values, by descending value):

* ``<case>_geno`` (uint8 [snps, samples]) and ``<case>_is_case``;
* ``<case>_meta`` = [order, outputs];
* ``<case>_seg_{combos,vals}``: the segmented ThreadedSearch (1 thread);
* ``<case>_dfs_{combos,vals}`` / ``<case>_dfsseg_{combos,vals}``: the
  non-segmented and segmented benchmark programs.

Cases: three seeded synthetic scans (orders 2, 3, 4) and one with duplicated
SNP columns, whose equal MI values make the traversal order decide which tied
combinations a MaxArray keeps.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import build as obuild  # noqa: E402
from oracle.oracle import Reference, ReferenceBench  # noqa: E402
from fiuncho_gb300 import synth  # noqa: E402
from fiuncho_gb300.dataset import Dataset  # noqa: E402

# name -> (ScanSpec, duplicated columns (dst, src))
CASES = {
    "o3": (synth.ScanSpec(40, 333, 301, 3, 20, seed=11, planted=(3,), penetrance=0.7), ()),
    "o4": (synth.ScanSpec(30, 500, 480, 4, 25, seed=5), ()),
    "o2": (synth.ScanSpec(60, 999, 1001, 2, 30, seed=7), ()),
    "ties": (synth.ScanSpec(24, 400, 380, 3, 27, seed=21), ((3, 17), (9, 20), (11, 5), (14, 2))),
}


def case_data(name):
    spec, dups = CASES[name]
    geno, is_case, _ = synth.simulate(spec)
    for dst, src in dups:
        geno[dst] = geno[src]
    return spec, geno, is_case


def main():
    if not obuild.reference_present():
        sys.exit("the reference tree is not present")
    seg = Reference("base_seg")
    bench = ReferenceBench()
    out = {}
    for name in CASES:
        spec, geno, is_case = case_data(name)
        ds = Dataset.from_genotypes(geno, is_case)
        args = (ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words)
        k, n = spec.order, spec.outputs
        out[name + "_geno"] = geno.astype(np.uint8)
        out[name + "_is_case"] = is_case.astype(np.uint8)
        out[name + "_meta"] = np.array([k, n], np.int32)
        c, v = seg.from_packed(*args).search(k, n)
        out[name + "_seg_combos"], out[name + "_seg_vals"] = c, v
        for tag, s in (("dfs", 0), ("dfsseg", 1)):
            c, v = bench.stack_search(*args, k, n, s)
            out[name + "_%s_combos" % tag], out[name + "_%s_vals" % tag] = c, v
    path = os.path.join(HERE, "reference_traversals.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
