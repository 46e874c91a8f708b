"""Generates the golden fixtures in this folder from the reference itself.

Run in a checkout where the reference tree is present (``FIUNCHO_REFERENCE``
names it) -- it builds the reference's own sources through
``oracle/build.py`` and calls them through ``oracle/ref/ref_driver.cpp``:

    python tests/golden/make_golden.py

Outputs:

* ``reference_testdata.npz`` -- the reference's test data set
  (tests/data/test.tped + test.tfam: 10 SNPs, 9 000 cases, 9 800 controls)
  packed by the reference's own ``Dataset<uint64_t>::read`` (no ALIGN), the
  reference's contingency tables and FP32 MI of EVERY combination of order 2,
  3 and 4 (``combine`` + ``combine_and_popcnt`` + ``MutualInformation<float>``
  from src/base, and MI from the AVX-512 build), its ThreadedSearch top-90 per
  order, its MPIEngine (1 rank) top-90 at order 3, the row word counts with and
  without ALIGN=64, and the MPI3SNP order-3 list that tests/utils.h:49-84
  compares against (read from that file as text).
* ``reference_synth.npz`` -- a small seeded synthetic scan with odd class
  sizes (999 cases / 1 001 controls, 48 SNPs) as genotype codes, with the
  reference's ThreadedSearch top-50 for orders 2, 3 and 4, its tables/MI for
  1 500 sampled order-3 combinations, a 3-thread and a step-2/offset-1 run, and
  the digest (oracle/ref/tabledigest.h) of the reference's tables of every
  combination at orders 2, 3 and 4 and of a step-3/offset-2 order-3 layer.
"""
from __future__ import annotations

import itertools
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import build as obuild  # noqa: E402
from oracle.oracle import Reference  # noqa: E402
from fiuncho_gb300 import synth  # noqa: E402
from fiuncho_gb300.dataset import Dataset  # noqa: E402


def all_combos(n, k):
    return np.array(list(itertools.combinations(range(n), k)), dtype=np.int32)


def mpi3snp_list():
    txt = open(os.path.join(obuild.REF_ROOT, "tests", "utils.h")).read()
    body = txt[txt.index("mpi3snp_output{"):]
    body = body[: body.index("};")]
    pairs = re.findall(r"\{\{(\d+),\s*(\d+),\s*(\d+)\},\s*([0-9.]+)\}", body)
    combos = np.array([[int(a), int(b), int(c)] for a, b, c, _ in pairs], np.int32)
    vals = np.array([float(v) for *_, v in pairs], np.float64)
    return combos, vals


def main():
    if not obuild.reference_present():
        sys.exit("reference tree not found; set FIUNCHO_REFERENCE")
    base, avx = Reference("base"), None
    try:
        avx = Reference("avx512")
    except FileNotFoundError:
        pass
    D = os.path.join(obuild.REF_ROOT, "tests", "data")
    tped, tfam = os.path.join(D, "test.tped"), os.path.join(D, "test.tfam")
    d = base.read(tped, tfam)
    out = dict(data=d.packed(), meta=np.array([d.snps, d.cases, d.ctrls, d.cases_words, d.ctrls_words], np.int64))
    if avx is not None:
        da = avx.read(tped, tfam)
        out["words_align64"] = np.array([da.cases_words, da.ctrls_words], np.int64)
    for order in (2, 3, 4):
        cmb = all_combos(d.snps, order)
        cc, tt, mi = d.tables(order, cmb)
        out["o%d_combos" % order] = cmb
        out["o%d_cases" % order] = cc
        out["o%d_ctrls" % order] = tt
        out["o%d_mi_base" % order] = mi
        if avx is not None:
            out["o%d_mi_avx512" % order] = avx.mi(order, cc, tt, d.cases, d.ctrls)
        c, v = d.search(order, 90, threads=1)
        out["o%d_top90_combos" % order] = c
        out["o%d_top90_vals" % order] = v
    c, v = base.engine(tped, tfam, 3, 4, 90)
    out["engine_o3_top90_combos"], out["engine_o3_top90_vals"] = c, v
    mc, mv = mpi3snp_list()
    out["mpi3snp_combos"], out["mpi3snp_vals"] = mc, mv
    np.savez_compressed(os.path.join(HERE, "reference_testdata.npz"), **out)

    spec = synth.ScanSpec(48, 999, 1001, 3, 50, seed=7, planted=(2,), penetrance=0.7)
    geno, is_case, planted = synth.simulate(spec)
    ds = Dataset.from_genotypes(geno, is_case)
    rd = base.from_packed(ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words)
    out = dict(geno=geno, is_case=is_case, planted=np.array(planted, np.int32))
    for order in (2, 3, 4):
        c, v = rd.search(order, 50, threads=1)
        out["o%d_top50_combos" % order], out["o%d_top50_vals" % order] = c, v
    c, v = rd.search(3, 50, threads=3)
    out["o3_t3_combos"], out["o3_t3_vals"] = c, v
    c, v = rd.search(3, 50, threads=1, step=2, offset=1)
    out["o3_step2_off1_combos"], out["o3_step2_off1_vals"] = c, v
    # digest (oracle/ref/tabledigest.h) of every table of the scan, per order, and of a step-3/offset-2 layer
    for order in (2, 3, 4):
        dg, cnt = rd.table_digest(order, threads=2)
        out["o%d_digest" % order], out["o%d_digest_count" % order] = np.array(dg, np.uint64), np.array(cnt)
    dg, cnt = rd.table_digest(3, threads=1, step=3, offset=2)
    out["o3_step3_off2_digest"], out["o3_step3_off2_digest_count"] = np.array(dg, np.uint64), np.array(cnt)
    cmb = all_combos(ds.snps, 3)
    cmb = cmb[np.sort(np.random.default_rng(11).choice(len(cmb), 1500, replace=False))]
    cc, tt, mi = rd.tables(3, cmb)
    out["o3_sample_combos"] = cmb
    out["o3_cases"], out["o3_ctrls"], out["o3_mi_base"] = cc, tt, mi
    np.savez_compressed(os.path.join(HERE, "reference_synth.npz"), **out)
    for f in ("reference_testdata.npz", "reference_synth.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
