"""Pins the CPU oracle (oracle/oracle.c) against the reference's golden vectors
and known answers.  No GPU; runs wherever the committed fixtures are."""
import itertools
import math

import numpy as np
import pytest

from helpers import assert_ascending_unique, assert_sorted_desc, assert_topn_equivalent, exact_mi


def _meta(g):
    snps, cases, ctrls, cw, tw = (int(x) for x in g["meta"])
    return snps, cases, ctrls, cw, tw


# ---------------------------------------------------------------- data model
def test_dataset_shape_and_words(golden_testdata):
    """tests/dataset.cpp:10-23: 10 SNPs, 9000/9800, 141/154 words unaligned, 144/160 at ALIGN=64."""
    from fiuncho_gb300.dataset import words_for
    snps, cases, ctrls, cw, tw = _meta(golden_testdata)
    assert (snps, cases, ctrls, cw, tw) == (10, 9000, 9800, 141, 154)
    assert (words_for(cases, 64), words_for(ctrls, 64)) == tuple(golden_testdata["words_align64"]) == (144, 160)
    assert (words_for(cases, 32), words_for(ctrls, 32)) == (144, 156)


def test_dataset_one_hot_complete(golden_testdata):
    """tests/dataset.cpp:25-44: the three rows of every SNP popcount to the class size."""
    snps, cases, ctrls, cw, tw = _meta(golden_testdata)
    d = golden_testdata["data"].reshape(snps, 3 * (cw + tw))
    pc = np.vectorize(lambda x: bin(int(x)).count("1"))
    for i in range(snps):
        assert int(pc(d[i, : 3 * cw]).sum()) == cases
        assert int(pc(d[i, 3 * cw:]).sum()) == ctrls


# ---------------------------------------------------------------- kernels
def test_combine_identity(oracle, golden_testdata):
    """tests/genotypetable.cpp:12-37: combine row i == t1[i/3] & t2[i%3]."""
    snps, cases, ctrls, cw, tw = _meta(golden_testdata)
    d = golden_testdata["data"].reshape(snps, 3 * (cw + tw))
    t1, t2 = d[0, : 3 * cw], d[1, : 3 * cw]
    out = oracle.combine(t1, 3, t2, cw).reshape(9, cw)
    for i in range(9):
        assert np.array_equal(out[i], t1.reshape(3, cw)[i // 3] & t2.reshape(3, cw)[i % 3])


def test_popcnt_matches_combine_and_padding(oracle, golden_testdata):
    """tests/genotypetable.cpp:39-66: combine_and_popcnt == popcount of combine; padded cells are 0."""
    snps, cases, ctrls, cw, tw = _meta(golden_testdata)
    d = golden_testdata["data"].reshape(snps, 3 * (cw + tw))
    t1, t2 = d[0, 3 * cw:], d[1, 3 * cw:]
    gt = oracle.combine(t1, 3, t2, tw).reshape(9, tw)
    ct = oracle.popcnt(t1, 3, t2, tw, ct_size=16)
    for i in range(9):
        assert ct[i] == sum(bin(int(x)).count("1") for x in gt[i])
    assert np.all(ct[9:] == 0)


@pytest.mark.parametrize("order", [2, 3, 4])
def test_tables_bit_exact_vs_reference(oracle, golden_testdata, order):
    """Every combination of the reference test data: oracle tables == reference combine_and_popcnt."""
    snps, cases, ctrls, cw, tw = _meta(golden_testdata)
    cmb = golden_testdata["o%d_combos" % order]
    cc, tt = oracle.tables(golden_testdata["data"], cw, tw, order, cmb)
    assert np.array_equal(cc, golden_testdata["o%d_cases" % order])
    assert np.array_equal(tt, golden_testdata["o%d_ctrls" % order])


@pytest.mark.parametrize("order", [2, 3, 4])
def test_mi_f32_bit_exact_vs_reference_scalar(oracle, golden_testdata, order):
    """Oracle FP32 MI reproduces src/base/mi_compute.cpp bit for bit; FP64 MI bounds the reference's error."""
    snps, cases, ctrls, cw, tw = _meta(golden_testdata)
    o32, o64 = oracle.mi_batch(golden_testdata["o%d_cases" % order], golden_testdata["o%d_ctrls" % order],
                               cases, ctrls)
    assert np.array_equal(o32, golden_testdata["o%d_mi_base" % order])
    for key in ("o%d_mi_base" % order, "o%d_mi_avx512" % order):
        ref = golden_testdata[key].astype(np.float64)
        assert np.max(np.abs(ref - o64) / np.abs(o64)) < 1e-2


def test_mi_known_answers(oracle):
    """tests/mi.cpp:7-31: uniform table -> 0; cases[0]=9, ctrls[1]=18 -> 0.6365141682948129 (+-1e-5)."""
    cases = np.full(9, 1, np.uint32)
    ctrls = np.full(9, 2, np.uint32)
    v32, v64 = oracle.mi(cases, ctrls, 9, 18)
    assert abs(v32) < 1e-5 and abs(v64) < 1e-12
    cases = np.zeros(9, np.uint32)
    ctrls = np.zeros(9, np.uint32)
    cases[0], ctrls[1] = 9, 18
    v32, v64 = oracle.mi(cases, ctrls, 9, 18)
    assert abs(v32 - 0.6365141682948129) < 1e-5
    assert abs(v64 - 0.6365141682948129) < 1e-12
    # closed form: MI = H(Y) = -(1/3)ln(1/3) - (2/3)ln(2/3)
    assert abs(v64 - (math.log(3) - (2 / 3) * math.log(2))) < 1e-14


# ---------------------------------------------------------------- scheduling
def _py_prefixes(n, k, step, offset):
    allc = list(itertools.combinations(range(n), k))
    return [c for r, c in enumerate(allc) if r >= offset and (r - offset) % step == 0]


@pytest.mark.parametrize("n,k,step,offset", [(10, 1, 1, 0), (10, 2, 1, 0), (10, 2, 3, 2), (13, 3, 5, 4),
                                             (7, 3, 1, 40), (9, 2, 36, 35), (20, 2, 4, 0)])
def test_distribution_enumeration(oracle, n, k, step, offset):
    """Distribution.h:54-130: round-robin over the lexicographic (k)-combinations."""
    got = [tuple(r) for r in oracle.prefixes(n, k, step, offset)]
    assert got == _py_prefixes(n, k, step, offset)


def test_distribution_layers_partition(oracle):
    """Distribution::layer (Distribution.h:172-176): rank x thread layers cover every prefix once."""
    n, k, ranks, threads = 15, 2, 3, 4
    seen = []
    for r in range(ranks):
        for t in range(threads):
            seen += [tuple(x) for x in oracle.prefixes(n, k, ranks * threads, r * threads + t)]
    assert sorted(seen) == list(itertools.combinations(range(n), k))


# ---------------------------------------------------------------- search
@pytest.mark.parametrize("order", [2, 3, 4])
def test_search_f32_matches_reference(oracle, golden_testdata, order):
    """ThreadedSearch(1).run top-90: same set and identical FP32 values as the reference."""
    snps, cases, ctrls, cw, tw = _meta(golden_testdata)
    c, v32, v64, done = oracle.search(golden_testdata["data"], snps, cases, ctrls, cw, tw, order, 90, threads=1,
                                      mi_mode=0)
    rc, rv = golden_testdata["o%d_top90_combos" % order], golden_testdata["o%d_top90_vals" % order]
    assert done == math.comb(snps, order)
    assert {tuple(x) for x in c} == {tuple(x) for x in rc}
    assert np.array_equal(np.sort(v32), np.sort(rv))
    assert_sorted_desc(v32)
    assert_ascending_unique(c)


@pytest.mark.parametrize("order", [2, 3, 4])
@pytest.mark.parametrize("threads", [1, 4])
def test_search_f64_vs_reference_within_its_error(oracle, golden_testdata, order, threads):
    """FP64 ranking vs the reference's FP32 ranking: they may differ only where the
    reference's own FP32 error cannot order the values."""
    snps, cases, ctrls, cw, tw = _meta(golden_testdata)
    data = golden_testdata["data"]
    c, v32, v64, _ = oracle.search(data, snps, cases, ctrls, cw, tw, order, 90, threads=threads, mi_mode=1)
    rc = golden_testdata["o%d_top90_combos" % order]
    rv = golden_testdata["o%d_top90_vals" % order].astype(np.float64)
    ex = exact_mi(oracle, data, cw, tw, cases, ctrls, order, rc)
    ref_err = float(np.max(np.abs(rv - ex)))
    assert_topn_equivalent(c, rc, lambda cs: exact_mi(oracle, data, cw, tw, cases, ctrls, order, cs), 2 * ref_err)
    assert_sorted_desc(v64)
    assert_ascending_unique(c)


def test_search_matches_mpi3snp(oracle, golden_testdata):
    """tests/utils.h:49-101: order-3 top-90, normalised by the maximum, within 5e-4 of MPI3SNP's list."""
    snps, cases, ctrls, cw, tw = _meta(golden_testdata)
    c, v32, v64, _ = oracle.search(golden_testdata["data"], snps, cases, ctrls, cw, tw, 3, 90, mi_mode=1)
    norm = {tuple(x): v / golden_testdata["mpi3snp_vals"][0]
            for x, v in zip(golden_testdata["mpi3snp_combos"], golden_testdata["mpi3snp_vals"])}
    assert len(c) == 90
    for comb, v in zip(c, v64):
        assert abs(v / v64[0] - norm.get(tuple(comb), 0.0)) <= 5e-4


def test_engine_single_rank_matches(oracle, golden_testdata):
    """MPIEngine::run<ThreadedSearch> at one rank returns the ThreadedSearch result (MPIEngine.h:108-182)."""
    a = {tuple(x) for x in golden_testdata["engine_o3_top90_combos"]}
    b = {tuple(x) for x in golden_testdata["o3_top90_combos"]}
    assert a == b


# ---------------------------------------------------------------- synthetic, odd class sizes
def test_synth_fixture_regenerates(golden_synth):
    """The seeded generator still yields the fixture's genotypes (the fixture stores them anyway)."""
    from fiuncho_gb300 import synth
    spec = synth.ScanSpec(48, 999, 1001, 3, 50, seed=7, planted=(2,), penetrance=0.7)
    geno, is_case, planted = synth.simulate(spec)
    assert np.array_equal(geno, golden_synth["geno"])
    assert np.array_equal(is_case, golden_synth["is_case"])


@pytest.mark.parametrize("order", [2, 3, 4])
def test_synth_search_f32_matches_reference(oracle, golden_synth, order):
    from fiuncho_gb300.dataset import Dataset
    ds = Dataset.from_genotypes(golden_synth["geno"], golden_synth["is_case"])
    c, v32, _, _ = oracle.search(ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words, order, 50,
                                 mi_mode=0)
    rc, rv = golden_synth["o%d_top50_combos" % order], golden_synth["o%d_top50_vals" % order]
    assert {tuple(x) for x in c} == {tuple(x) for x in rc}
    assert np.array_equal(np.sort(v32), np.sort(rv))


def test_synth_distribution_runs_match_reference(oracle, golden_synth):
    """Reference 3-thread run and a step-2/offset-1 (rank 1 of 2) run."""
    from fiuncho_gb300.dataset import Dataset
    ds = Dataset.from_genotypes(golden_synth["geno"], golden_synth["is_case"])
    args = (ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words, 3, 50)
    c, v32, _, _ = oracle.search(*args, threads=3, mi_mode=0)
    assert np.array_equal(np.sort(v32), np.sort(golden_synth["o3_t3_vals"]))
    c, v32, _, _ = oracle.search(*args, threads=1, mi_mode=0, dist=(ds.snps, 2, 1))
    assert {tuple(x) for x in c} == {tuple(x) for x in golden_synth["o3_step2_off1_combos"]}
    assert np.array_equal(np.sort(v32), np.sort(golden_synth["o3_step2_off1_vals"]))


def test_synth_sampled_tables(oracle, golden_synth):
    from fiuncho_gb300.dataset import Dataset
    ds = Dataset.from_genotypes(golden_synth["geno"], golden_synth["is_case"])
    cc, tt = oracle.tables(ds.data, ds.cases_words, ds.ctrls_words, 3, golden_synth["o3_sample_combos"])
    assert np.array_equal(cc, golden_synth["o3_cases"]) and np.array_equal(tt, golden_synth["o3_ctrls"])
    o32, _ = oracle.mi_batch(cc, tt, ds.cases, ds.ctrls)
    assert np.array_equal(o32, golden_synth["o3_mi_base"])


# ---------------------------------------------------------------- table digest
def _synth_ds(g):
    from fiuncho_gb300.dataset import Dataset
    return Dataset.from_genotypes(g["geno"], g["is_case"])


@pytest.mark.parametrize("order", [2, 3, 4])
def test_digest_matches_reference(oracle, golden_synth, order):
    """The oracle's digest of every table of a scan (oracle/ref/tabledigest.h) equals the
    digest of the reference's own combine / combine_and_popcnt tables (fixture)."""
    ds = _synth_ds(golden_synth)
    dg, cnt = oracle.table_digest(ds.data, ds.snps, ds.cases_words, ds.ctrls_words, order, threads=3)
    assert cnt == int(golden_synth["o%d_digest_count" % order]) == math.comb(ds.snps, order)
    assert dg == int(golden_synth["o%d_digest" % order])


def test_digest_distribution_layer(oracle, golden_synth):
    """Digest of the tables a Distribution(48, 2, 3, 2) layer owns, as the reference enumerates them."""
    ds = _synth_ds(golden_synth)
    dg, cnt = oracle.table_digest(ds.data, ds.snps, ds.cases_words, ds.ctrls_words, 3, threads=1,
                                  dist=(ds.snps, 3, 2))
    assert cnt == int(golden_synth["o3_step3_off2_digest_count"])
    assert dg == int(golden_synth["o3_step3_off2_digest"])


def test_digest_detects_one_wrong_cell(oracle, golden_synth):
    """A single count changed by one in one cell of one combination changes the digest: the
    mistake is planted in the oracle's input (one sample's genotype moved), on the CPU."""
    from fiuncho_gb300.dataset import Dataset
    g = golden_synth["geno"].copy()
    g[5, 17] = (g[5, 17] + 1) % 3
    ds = Dataset.from_genotypes(g, golden_synth["is_case"])
    dg, _ = oracle.table_digest(ds.data, ds.snps, ds.cases_words, ds.ctrls_words, 2, threads=2)
    assert dg != int(golden_synth["o2_digest"])


def test_scale_fixture_layout():
    """The full-size fixture holds, per workload, the data set's SHA-256, the reference's digest of
    every table with its combination count C(snps, order), and its top-N."""
    import os
    from fiuncho_gb300 import synth
    path = os.path.join(os.path.dirname(__file__), "golden", "reference_scale.npz")
    g = dict(np.load(path))
    names = sorted({k.rsplit("_", 1)[0] for k in g if k.endswith("_digest")})
    assert names, "no workloads in the full-size fixture"
    for name in names:
        spec = synth.WORKLOADS[name]
        assert int(g[name + "_count"]) == math.comb(spec.snps, spec.order)
        c, v = g[name + "_combos"], g[name + "_vals"]
        assert c.shape == (spec.outputs, spec.order)
        assert_ascending_unique(c)
        assert_sorted_desc(v)
        assert len(str(g[name + "_sha256"])) == 64


# ------------------------------------------------ segmented evaluation and depth-first traversals
TRAVERSAL_CASES = ["o2", "o3", "o4", "ties"]


def _traversal_case(g, name):
    from fiuncho_gb300.dataset import Dataset
    ds = Dataset.from_genotypes(g[name + "_geno"], g[name + "_is_case"])
    order, outputs = (int(x) for x in g[name + "_meta"])
    return ds, order, outputs


def _by_value_then_combo(combos, vals):
    """A list ordered by descending value, ties by ascending combination (order-free comparison)."""
    return sorted(zip((-float(v) for v in vals), map(tuple, np.asarray(combos).tolist())))


@pytest.mark.parametrize("name", TRAVERSAL_CASES)
def test_depth_first_traversal_matches_reference(oracle, golden_traversals, name):
    """The oracle's depth-first traversal (stack_search of the benchmark programs, segmented
    and not) returns the reference programs' MaxArray content, ties at the cut-off included."""
    g = golden_traversals
    ds, order, outputs = _traversal_case(g, name)
    args = (ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words, order, outputs)
    for tag, block in (("dfs", 1), ("dfsseg", 1474560 // 3 ** order)):
        c, v, _, n = oracle.search_dfs(*args, block=block, mi_mode=0)
        assert n == math.comb(ds.snps, order)
        assert _by_value_then_combo(c, v) == _by_value_then_combo(g[name + "_%s_combos" % tag],
                                                                   g[name + "_%s_vals" % tag])


@pytest.mark.parametrize("name", TRAVERSAL_CASES)
def test_segmented_threaded_search_matches_oracle(oracle, golden_traversals, name):
    """ThreadedSearch built with SEGMENT_SIZE (MI in blocks, MaxArray fed in the same order)
    returns exactly the non-segmented list, which the oracle restates."""
    g = golden_traversals
    ds, order, outputs = _traversal_case(g, name)
    c, v, _, _ = oracle.search(ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words, order,
                               outputs, mi_mode=0)
    assert _by_value_then_combo(c, v) == _by_value_then_combo(g[name + "_seg_combos"], g[name + "_seg_vals"])


def test_traversal_order_decides_ties(golden_traversals):
    """With duplicated SNP columns the cut-off falls inside a group of equal MI values: the
    depth-first programs keep a different tied combination than ThreadedSearch, with the
    same value list."""
    g = golden_traversals
    a = set(map(tuple, g["ties_dfs_combos"].tolist()))
    b = set(map(tuple, g["ties_seg_combos"].tolist()))
    assert a != b and len(a ^ b) == 2
    assert np.array_equal(np.sort(g["ties_dfs_vals"]), np.sort(g["ties_seg_vals"]))


@pytest.mark.parametrize("order", [2, 3, 4])
def test_segmented_blocks_do_not_change_the_list(oracle, order):
    """MI in blocks of any size feeds the MaxArray in the same visiting order, so the
    segmented traversal returns the non-segmented list exactly (values and ties)."""
    from fiuncho_gb300 import Dataset, synth
    spec = synth.ScanSpec(26 if order < 4 else 18, 211, 190, order, 17, seed=31 + order)
    g, c, _ = synth.simulate(spec)
    g[5] = g[2]  # a duplicated column: ties in the list
    ds = Dataset.from_genotypes(g, c)
    args = (ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words, order, spec.outputs)
    base = oracle.search_dfs(*args, block=1, mi_mode=0)
    for block in (2, 7, 1000, 10 ** 6):
        got = oracle.search_dfs(*args, block=block, mi_mode=0)
        assert np.array_equal(got[0], base[0]) and np.array_equal(got[1], base[1]) and got[3] == base[3]
