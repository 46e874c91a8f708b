"""Parity of the CUDA path with the oracle and the reference's golden vectors.

Every call goes through the C ABI (libfiuncho_gpu.so via ctypes).  Tolerances:
contingency counts bit-exact; MI within 1e-5 relative of the FP64 oracle;
top-N lists identical except for combinations whose exact MI lies within
1e-5 (relative to the cutoff) of the cutoff.
"""
import math

import numpy as np
import pytest

from helpers import as_set, assert_ascending_unique, assert_sorted_desc, assert_topn_equivalent, exact_mi

pytestmark = pytest.mark.gpu

MI_RTOL = 1e-5


@pytest.fixture(scope="module")
def gs():
    from fiuncho_gb300 import GpuSearch
    return GpuSearch(0)


def _ds_from_golden(g):
    from fiuncho_gb300 import Dataset
    snps, cases, ctrls, cw, tw = (int(x) for x in g["meta"])
    return Dataset(cases, ctrls, snps, cw, tw, g["data"])


def _check_topn(oracle, ds, order, outputs, res, v64, dist=None, threads=8):
    # One worker owns the Distribution's own prefixes (ranks offset, offset+step, ...); the
    # oracle's threads would re-layer a step > 1 distribution (Distribution::layer), so use one.
    if dist is not None and dist[1] > 1:
        threads = 1
    c, _, o64, _ = oracle.search(ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words, order,
                                 outputs, threads=threads, mi_mode=1, dist=dist)
    got = np.array([r.combination for r in res], np.int32).reshape(-1, order)
    assert len(res) == len(c)
    assert_ascending_unique(got)
    assert_sorted_desc(v64)
    ex = lambda cs: exact_mi(oracle, ds.data, ds.cases_words, ds.ctrls_words, ds.cases, ds.ctrls, order, cs)
    if len(c):
        tol = MI_RTOL * abs(float(o64[-1])) + 1e-12
        assert_topn_equivalent(got, c, ex, tol)
        mine = ex(got)
        assert np.allclose(v64, mine, rtol=MI_RTOL, atol=1e-12)
        assert np.allclose([r.val for r in res], mine, rtol=MI_RTOL, atol=1e-9)
    return got


# --------------------------------------------------------------- kernel entries
def test_combine_and_popcnt_bit_exact(gs, oracle, golden_testdata):
    ds = _ds_from_golden(golden_testdata)
    cw, tw = ds.cases_words, ds.ctrls_words
    t1 = ds.data[: 3 * (cw + tw)]
    t2 = ds.data[3 * (cw + tw): 6 * (cw + tw)]
    out = gs.combine(t1, 3, t2, cw, tw)
    exp = np.concatenate([oracle.combine(t1[: 3 * cw], 3, t2[: 3 * cw], cw),
                          oracle.combine(t1[3 * cw:], 3, t2[3 * cw:], tw)])
    assert np.array_equal(out, exp)
    cc, tt = gs.combine_and_popcnt(out, 9, ds.data[6 * (cw + tw): 9 * (cw + tw)], cw, tw, ct_size=32)
    assert np.array_equal(cc, oracle.popcnt(out[: 9 * cw], 9, ds.data[6 * (cw + tw): 6 * (cw + tw) + 3 * cw], cw, 32))
    assert np.all(cc[27:] == 0) and np.all(tt[27:] == 0)


@pytest.mark.parametrize("order,kernel", [(2, 1), (3, 1), (4, 1), (2, 2), (3, 2), (4, 2), (2, 3), (3, 3), (4, 3),
                                          (2, 4), (3, 4), (4, 4)])
def test_hot_kernel_tables_bit_exact_reference(gs, golden_testdata, order, kernel):
    """Each counting kernel's own contingency tables for EVERY combination of the
    reference's test data == the reference's combine_and_popcnt tables
    (kernel 1: full table; 2, 3: core cells + exact marginals, POPC / Harley-Seal,
    at order 4 from triple cores; 4: core cells on the tcgen05 tensor cores -- with
    9 000 / 9 800 samples one accumulator per class at every order)."""
    from fiuncho_gb300 import Distribution, Resident
    ds = _ds_from_golden(golden_testdata)
    res = Resident(gs.ctx, ds)
    out = gs.scan_tables(res, order, Distribution(ds.snps, order - 1), kernel=kernel)
    prefixes = list(Distribution(ds.snps, order - 1))
    ref = {tuple(c): i for i, c in enumerate(golden_testdata["o%d_combos" % order])}
    n = 0
    for m, p in enumerate(prefixes):
        for l in range(p[-1] + 1, ds.snps):
            i = ref[tuple(p) + (l,)]
            assert np.array_equal(out[m, l, 0], golden_testdata["o%d_cases" % order][i])
            assert np.array_equal(out[m, l, 1], golden_testdata["o%d_ctrls" % order][i])
            n += 1
    assert n == math.comb(ds.snps, order)


def test_tables_entry_bit_exact(gs, oracle, golden_synth):
    from fiuncho_gb300 import Dataset, Resident
    ds = Dataset.from_genotypes(golden_synth["geno"], golden_synth["is_case"])
    res = Resident(gs.ctx, ds)
    cc, tt = gs.tables(res, 3, golden_synth["o3_sample_combos"])
    assert np.array_equal(cc, golden_synth["o3_cases"]) and np.array_equal(tt, golden_synth["o3_ctrls"])


def test_mi_known_answers_and_modes(gs, oracle, golden_testdata):
    """tests/mi.cpp:7-31 through MutualInformation::compute's replacement, both arithmetics."""
    for mode in (0, 1):
        v, v64 = gs.mi(np.full(9, 1, np.uint32), np.full(9, 2, np.uint32), 9, 18, mode=mode)
        assert abs(v[0]) < 1e-5 and abs(v64[0]) < 1e-9
        c = np.zeros(9, np.uint32)
        t = np.zeros(9, np.uint32)
        c[0], t[1] = 9, 18
        v, v64 = gs.mi(c, t, 9, 18, mode=mode)
        assert abs(v[0] - 0.6365141682948129) < 1e-5 and abs(v64[0] - 0.6365141682948129) < 1e-9
    snps, cases, ctrls, cw, tw = (int(x) for x in golden_testdata["meta"])
    cc, tt = golden_testdata["o3_cases"], golden_testdata["o3_ctrls"]
    _, o64 = oracle.mi_batch(cc, tt, cases, ctrls)
    for mode in (0, 1):
        v, v64 = gs.mi(cc, tt, cases, ctrls, mode=mode)
        assert np.allclose(v64, o64, rtol=MI_RTOL, atol=0)


# --------------------------------------------------------------- search on the reference's data
@pytest.mark.parametrize("order", [2, 3, 4])
def test_search_reference_testdata(gs, oracle, golden_testdata, order):
    from fiuncho_gb300 import Distribution
    ds = _ds_from_golden(golden_testdata)
    res, v64 = gs.run(ds, order, Distribution(ds.snps, order - 1), 90, with_fp64=True)
    got = _check_topn(oracle, ds, order, 90, res, v64)
    assert len(res) == min(90, math.comb(10, order))
    # the reference's own top-90 differs only where its FP32 error cannot order values
    rc = golden_testdata["o%d_top90_combos" % order]
    rv = golden_testdata["o%d_top90_vals" % order].astype(np.float64)
    ex = lambda cs: exact_mi(oracle, ds.data, ds.cases_words, ds.ctrls_words, ds.cases, ds.ctrls, order, cs)
    ref_err = float(np.max(np.abs(rv - ex(rc))))
    assert_topn_equivalent(got, rc, ex, 2 * ref_err + 1e-12)


def test_search_matches_mpi3snp(gs, golden_testdata):
    """tests/utils.h:49-101 through the GPU search: normalised order-3 top-90 within 5e-4 of MPI3SNP."""
    from fiuncho_gb300 import Distribution
    ds = _ds_from_golden(golden_testdata)
    res = gs.run(ds, 3, Distribution(ds.snps, 2), 90)
    norm = {tuple(x): v / golden_testdata["mpi3snp_vals"][0]
            for x, v in zip(golden_testdata["mpi3snp_combos"], golden_testdata["mpi3snp_vals"])}
    assert len(res) == 90
    for r in res:
        assert abs(r.val / res[0].val - norm.get(tuple(r.combination), 0.0)) <= 5e-4


def test_engine_single_rank(gs, golden_testdata):
    """MPIEngine().run(GpuSearch, ...) at one rank == GpuSearch.run (MPIEngine.h:108-182)."""
    from fiuncho_gb300 import Distribution, GpuSearch, MPIEngine
    ds = _ds_from_golden(golden_testdata)
    a = MPIEngine().run(GpuSearch, None, 3, 90, 0, dataset=ds)
    b = gs.run(ds, 3, Distribution(ds.snps, 2), 90)
    assert [r.combination for r in a] == [r.combination for r in b]


# --------------------------------------------------------------- synthetic data, distributions
@pytest.mark.parametrize("order", [2, 3, 4])
def test_search_synth_vs_reference(gs, oracle, golden_synth, order):
    from fiuncho_gb300 import Dataset, Distribution
    from fiuncho_gb300 import GpuSearch
    ds = Dataset.from_genotypes(golden_synth["geno"], golden_synth["is_case"])
    res, v64 = gs.run(ds, order, Distribution(ds.snps, order - 1), 50, with_fp64=True)
    # one-hot, whole data set: the tcgen05 kernels at orders 2-4; at order 4 the forced
    # pair-major CUDA-core kernel agrees
    assert gs.last_tile()[0] == 4
    if order == 4:
        g2 = GpuSearch(0, kernel=2)
        r2, v2 = g2.run(ds, 4, Distribution(ds.snps, 3), 50, with_fp64=True)
        assert g2.last_tile()[0] == 2
        assert [x.combination for x in r2] == [x.combination for x in res] and np.array_equal(v2, v64)
    got = _check_topn(oracle, ds, order, 50, res, v64)
    rc = golden_synth["o%d_top50_combos" % order]
    rv = golden_synth["o%d_top50_vals" % order].astype(np.float64)
    ex = lambda cs: exact_mi(oracle, ds.data, ds.cases_words, ds.ctrls_words, ds.cases, ds.ctrls, order, cs)
    assert_topn_equivalent(got, rc, ex, 2 * float(np.max(np.abs(rv - ex(rc)))) + 1e-12)


@pytest.mark.parametrize("step,offset", [(2, 1), (3, 0), (5, 4), (1000, 7)])
def test_search_distribution_layers(gs, oracle, golden_synth, step, offset):
    """A rank's Distribution(n, k, step, offset) share: same as the oracle's, and
    for (2, 1) the reference's own step-2/offset-1 run."""
    from fiuncho_gb300 import Dataset, Distribution
    ds = Dataset.from_genotypes(golden_synth["geno"], golden_synth["is_case"])
    d = Distribution(ds.snps, 2, step, offset)
    res, v64 = gs.run(ds, 3, d, 50, with_fp64=True)
    got = _check_topn(oracle, ds, 3, 50, res, v64, dist=(ds.snps, step, offset))
    if (step, offset) == (2, 1):
        rc = golden_synth["o3_step2_off1_combos"]
        ex = lambda cs: exact_mi(oracle, ds.data, ds.cases_words, ds.ctrls_words, ds.cases, ds.ctrls, 3, cs)
        rv = golden_synth["o3_step2_off1_vals"].astype(np.float64)
        assert_topn_equivalent(got, rc, ex, 2 * float(np.max(np.abs(rv - ex(rc)))) + 1e-12)


def test_rank_split_merges_to_full_run(gs, golden_synth):
    """Two ranks' results merged as MPIEngine does == one full run (MPIEngine.h:133-174)."""
    from fiuncho_gb300 import Dataset, Distribution, MPIEngine
    ds = Dataset.from_genotypes(golden_synth["geno"], golden_synth["is_case"])
    full = gs.run(ds, 3, Distribution(ds.snps, 2), 40)
    parts = gs.run(ds, 3, Distribution(ds.snps, 2, 2, 0), 40) + gs.run(ds, 3, Distribution(ds.snps, 2, 2, 1), 40)
    merged = MPIEngine().gather(parts, 40)
    assert [r.combination for r in merged] == [r.combination for r in full]


@pytest.mark.parametrize("order,n_shards", [(2, 3), (3, 2), (3, 7), (4, 3)])
def test_shards_merge_to_full_run(gs, golden_synth, order, n_shards):
    """The shards of the whole search (equal ranges of the serving kernel's work units)
    merged by (MI descending, combination ascending) == one full run, results and FP64
    values; each shard keeps the whole-data-set kernel."""
    from fiuncho_gb300 import Dataset, Distribution, FiunchoError, MPIEngine
    ds = Dataset.from_genotypes(golden_synth["geno"], golden_synth["is_case"])
    full, v_full = gs.run(ds, order, Distribution(ds.snps, order - 1), 40, with_fp64=True)
    kernel = gs.last_tile()[0]
    parts = []
    for sh in range(n_shards):
        r, v = gs.run_shard(ds, order, sh, n_shards, 40, with_fp64=True)
        assert gs.last_tile()[0] == kernel
        parts += [(-float(x), tuple(c.combination), float(x)) for c, x in zip(r, v)]
    parts.sort()
    assert [list(p[1]) for p in parts[:40]] == [r.combination for r in full]
    assert np.array_equal(np.array([p[2] for p in parts[:40]]), v_full)
    # MPIEngine's gather of the shards' Result lists gives the same combinations
    lists = sum((gs.run_shard(ds, order, sh, n_shards, 40) for sh in range(n_shards)), [])
    assert [r.combination for r in MPIEngine().gather(lists, 40)] == [r.combination for r in full]
    with pytest.raises(FiunchoError):
        gs.run_shard(ds, order, n_shards, n_shards, 40)


# --------------------------------------------------------------- edge cases
def test_edge_cases(gs, oracle):
    from fiuncho_gb300 import Dataset, Distribution, FiunchoError
    rng = np.random.default_rng(5)
    # ragged class sizes straddling word boundaries, including a single case
    for n_case, n_ctrl, snps, order in ((1, 130, 9, 2), (65, 63, 12, 3), (127, 1, 7, 4), (300, 301, 6, 5)):
        geno = rng.integers(0, 3, (snps, n_case + n_ctrl), dtype=np.uint8)
        is_case = np.r_[np.ones(n_case, np.uint8), np.zeros(n_ctrl, np.uint8)]
        ds = Dataset.from_genotypes(geno, is_case)
        out = math.comb(snps, order) + 5  # more outputs than combinations
        res, v64 = gs.run(ds, order, Distribution(snps, order - 1), out, with_fp64=True)
        assert len(res) == math.comb(snps, order)
        _check_topn(oracle, ds, order, out, res, v64)
    # order larger than the SNP count: no combinations
    ds = Dataset.from_genotypes(rng.integers(0, 3, (3, 50), dtype=np.uint8), np.r_[np.ones(25), np.zeros(25)])
    assert gs.run(ds, 4, Distribution(3, 3), 10) == []
    assert gs.run(ds, 2, Distribution(3, 1), 0) == []
    # invalid requests are rejected with errors, not results
    with pytest.raises(FiunchoError):
        gs.run(ds, 1, Distribution(3, 0), 10)
    with pytest.raises(FiunchoError):
        gs.run(ds, 2, Distribution(3, 2), 10)  # k must be order-1
    with pytest.raises(FiunchoError):
        gs.run(ds, 2, Distribution(4, 1), 10)  # n beyond the data set
    with pytest.raises(FiunchoError):
        gs.run(ds, 2, Distribution(3, 1), 10 ** 6)


def test_non_one_hot_data_bit_exact(gs, oracle):
    """Arbitrary bits (rows overlapping, bits in padding words) are still counted
    exactly as combine_and_popcnt counts them."""
    from fiuncho_gb300 import Dataset, Distribution, Resident
    rng = np.random.default_rng(9)
    snps, cw, tw = 8, 3, 2
    data = rng.integers(0, 2 ** 63, snps * 3 * (cw + tw), dtype=np.uint64)
    ds = Dataset(100, 70, snps, cw, tw, data)
    res = Resident(gs.ctx, ds)
    assert not res.one_hot
    out = gs.scan_tables(res, 3, Distribution(snps, 2))
    for m, p in enumerate(Distribution(snps, 2)):
        for l in range(p[-1] + 1, snps):
            cc, tt = oracle.tables(data, cw, tw, 3, np.array([p + [l]], np.int32))
            assert np.array_equal(out[m, l, 0], cc[0]) and np.array_equal(out[m, l, 1], tt[0])
    r, v64 = gs.run(ds, 3, Distribution(snps, 2), 20, with_fp64=True)
    _check_topn(oracle, ds, 3, 20, r, v64)


@pytest.mark.parametrize("n_case,n_ctrl,snps", [(1000, 777, 60), (65, 63, 40), (1, 513, 30), (4000, 4000, 70)])
def test_kernels_agree(oracle, n_case, n_ctrl, snps):
    """Full, elided-POPC and elided-Harley-Seal kernels give identical tables and
    identical top-N lists (word counts straddling the 8-word Harley-Seal blocks)."""
    from fiuncho_gb300 import Dataset, Distribution, GpuSearch, Resident
    rng = np.random.default_rng(n_case + n_ctrl + snps)
    maf = rng.uniform(0.05, 0.5, snps)[:, None]
    u = rng.random((snps, n_case + n_ctrl))
    geno = ((u >= (1 - maf) ** 2).astype(np.uint8) + (u >= 1 - maf ** 2)).astype(np.uint8)
    is_case = np.r_[np.ones(n_case, np.uint8), np.zeros(n_ctrl, np.uint8)]
    ds = Dataset.from_genotypes(geno, is_case)
    for order in (2, 3):
        outs, tabs = [], []
        for kernel in (1, 2, 3, 4):
            g = GpuSearch(0, kernel=kernel)
            res = Resident(g.ctx, ds)
            assert res.one_hot
            tabs.append(g.scan_tables(res, order, Distribution(snps, order - 1), kernel=kernel))
            r, v64 = g.run(res, order, Distribution(snps, order - 1), 40, with_fp64=True)
            outs.append(([x.combination for x in r], v64))
        for t in tabs[1:]:
            mask = tabs[0] != 0xFFFFFFFF
            assert np.array_equal(t[mask], tabs[0][mask])
        for o in outs[1:]:
            assert o[0] == outs[0][0] and np.array_equal(o[1], outs[0][1])
        r = [type("R", (), {"combination": c, "val": v})() for c, v in zip(outs[0][0], outs[0][1])]
        _check_topn(oracle, ds, order, 40, r, outs[0][1])


@pytest.mark.parametrize("n_case,n_ctrl,snps", [(1000, 777, 30), (65, 63, 26), (1, 513, 20), (4000, 4000, 28),
                                                 (130, 1, 23), (511, 1537, 33)])
def test_order4_kernels_agree(oracle, n_case, n_ctrl, snps):
    """Order 4: the reduced-work kernels (16 core cells counted, 65 derived from
    triple, pair and single cores; POPC and Harley-Seal counting) and the tcgen05
    kernel give the full kernel's tables for every combination and the same top-N,
    which matches the oracle."""
    from fiuncho_gb300 import Dataset, Distribution, GpuSearch, Resident
    rng = np.random.default_rng(n_case * 3 + n_ctrl + snps)
    maf = rng.uniform(0.05, 0.5, snps)[:, None]
    u = rng.random((snps, n_case + n_ctrl))
    geno = ((u >= (1 - maf) ** 2).astype(np.uint8) + (u >= 1 - maf ** 2)).astype(np.uint8)
    ds = Dataset.from_genotypes(geno, np.r_[np.ones(n_case, np.uint8), np.zeros(n_ctrl, np.uint8)])
    dist = Distribution(snps, 3)
    outs, tabs = [], []
    for kernel in (1, 2, 3, 4):  # every class pair here shares one tensor accumulator
        g = GpuSearch(0, kernel=kernel)
        res = Resident(g.ctx, ds)
        tabs.append(g.scan_tables(res, 4, dist, kernel=kernel))
        r, v64 = g.run(res, 4, dist, 40, with_fp64=True)
        assert g.last_tile()[0] == kernel
        outs.append(([x.combination for x in r], v64))
    mask = tabs[0] != 0xFFFFFFFF
    assert mask.sum() == math.comb(snps, 4) * 2 * 81
    for t in tabs[1:]:
        assert np.array_equal(t[mask], tabs[0][mask])
    for o in outs[1:]:
        assert o[0] == outs[0][0] and np.array_equal(o[1], outs[0][1])
    r = [type("R", (), {"combination": c, "val": v})() for c, v in zip(outs[0][0], outs[0][1])]
    _check_topn(oracle, ds, 4, 40, r, outs[0][1])
    # a Distribution layer (per-prefix schedule) against the full kernel
    layer = Distribution(snps, 3, 3, 1)
    g = GpuSearch(0)
    res = Resident(g.ctx, ds)
    full = g.scan_tables(res, 4, layer, kernel=1)
    mask = full != 0xFFFFFFFF
    for kernel in (2, 3):
        assert np.array_equal(g.scan_tables(res, 4, layer, kernel=kernel)[mask], full[mask])


@pytest.mark.parametrize("snps,n_case,n_ctrl", [(4, 1, 1), (5, 65, 63), (18, 130, 1), (20, 64, 64),
                                                (33, 4000, 4000), (40, 700, 2500), (21, 4100, 4000),
                                                (36, 200, 40000), (17, 9000, 9800)])
def test_tensor4_tile_edges(oracle, snps, n_case, n_ctrl):
    """Order-4 tcgen05 kernel vs the full-table kernel around the 16 k x 128 l work item
    (classes in one accumulator) and the 16 k x 64 l one (one accumulator per class):
    identical tables for every combination and identical top-N lists, checked against
    the oracle."""
    from fiuncho_gb300 import Distribution, GpuSearch, Resident
    ds = _one_hot_dataset(snps * 3 + n_case, snps, n_case, n_ctrl)
    g = GpuSearch(0)
    res = Resident(g.ctx, ds)
    dist = Distribution(snps, 3)
    full = g.scan_tables(res, 4, dist, kernel=1)
    tens = g.scan_tables(res, 4, dist, kernel=4)
    mask = full != 0xFFFFFFFF
    assert mask.sum() == math.comb(snps, 4) * 2 * 81
    assert np.array_equal(tens[mask], full[mask])
    out = min(20, math.comb(snps, 4))
    g.set_kernel(1)
    a = g.run(res, 4, dist, out, with_fp64=True)
    g.set_kernel(4)
    b = g.run(res, 4, dist, out, with_fp64=True)
    assert g.last_tile() == (4, 256)
    assert [x.combination for x in a[0]] == [x.combination for x in b[0]] and np.array_equal(a[1], b[1])
    _check_topn(oracle, ds, 4, out, b[0], b[1])


@pytest.mark.parametrize("snps,n_case,n_ctrl,out", [(150, 300, 300, 30), (145, 1000, 900, 5),
                                                    (140, 5000, 6000, 10)])
def test_tensor4_search_many_tiles(oracle, snps, n_case, n_ctrl, out):
    """Order-4 tcgen05 search over SNP counts spanning several 128-l tiles, with a
    tight threshold where the bounded estimate rejects nearly every combination:
    the result equals the exact pair-major kernel's and the oracle's."""
    from fiuncho_gb300 import Distribution, GpuSearch, Resident
    ds = _one_hot_dataset(snps + n_case, snps, n_case, n_ctrl)
    g = GpuSearch(0)
    res = Resident(g.ctx, ds)
    dist = Distribution(snps, 3)
    g.set_kernel(2)
    a = g.run(res, 4, dist, out, with_fp64=True)
    g.set_kernel(4)
    b = g.run(res, 4, dist, out, with_fp64=True)
    assert g.last_tile()[0] == 4
    assert [x.combination for x in a[0]] == [x.combination for x in b[0]] and np.array_equal(a[1], b[1])
    _check_topn(oracle, ds, 4, out, b[0], b[1], threads=16)


def test_order4_reduced_work_is_automatic(gs, golden_synth):
    """One-hot order-4 searches pick a reduced-work kernel by themselves (pair-major below
    1 024 samples, tcgen05 above, for the whole data set and for a Distribution layer of
    all SNPs; per-prefix for a layer of fewer SNPs); non-one-hot data keeps the full
    kernel."""
    from fiuncho_gb300 import Dataset, Distribution, GpuSearch, Resident
    ds = Dataset.from_genotypes(golden_synth["geno"], golden_synth["is_case"])
    g = GpuSearch(0)
    res = Resident(g.ctx, ds)
    g.run(res, 4, Distribution(ds.snps, 3), 10)
    assert g.last_tile()[0] in (2, 3, 4)
    g.run(res, 4, Distribution(ds.snps, 3, 3, 2), 10)  # 2 000 samples: the tensor kernel's layer mode
    assert g.last_tile()[0] == 4
    g.run(res, 4, Distribution(ds.snps - 3, 3, 3, 2), 10)
    assert g.last_tile()[0] in (2, 3)
    rng = np.random.default_rng(5)
    bad = Dataset(100, 70, 9, 2, 2, rng.integers(0, 2 ** 63, 9 * 3 * 4, dtype=np.uint64))
    g.run(bad, 4, Distribution(9, 3), 5)
    assert g.last_tile()[0] == 1
    # below 1 024 samples the pair-major kernel, with 1 024 or more the tcgen05 kernel
    small = _one_hot_dataset(8, 24, 300, 300)
    g.run(small, 4, Distribution(24, 3), 10)
    assert g.last_tile()[0] == 2
    big = _one_hot_dataset(9, 24, 2100, 2000)
    g.run(big, 4, Distribution(24, 3), 10)
    assert g.last_tile()[0] == 4


def test_tensor_kernel_scope(gs, golden_synth):
    """The tcgen05 kernels serve one-hot order-2/3/4 searches of the whole data set,
    order-2 Distribution layers of all SNPs, and order-3 layers of all SNPs when the
    classes pack (the pair kernel's list mode); layers of fewer SNPs fall back to the
    reduced-work kernel automatically and are refused when the tensor kernel is
    forced."""
    from fiuncho_gb300 import Dataset, Distribution, FiunchoError, GpuSearch, Resident
    ds = Dataset.from_genotypes(golden_synth["geno"], golden_synth["is_case"])
    g = GpuSearch(0)
    res = Resident(g.ctx, ds)
    g.run(res, 3, Distribution(ds.snps, 2), 10)
    assert g.last_tile()[0] == 4
    g.run(res, 3, Distribution(ds.snps, 2, 2, 1), 10)
    assert g.last_tile()[0] == 4
    g.run(res, 3, Distribution(ds.snps - 5, 2, 2, 1), 10)  # a layer of the first n - 5 SNPs
    assert g.last_tile()[0] in (2, 3)
    g.run(res, 2, Distribution(ds.snps, 1, 2, 0), 10)
    assert g.last_tile()[0] == 4
    g.run(res, 2, Distribution(ds.snps - 5, 1, 2, 0), 10)
    assert g.last_tile()[0] in (2, 3)
    g.run(res, 2, Distribution(ds.snps, 1), 10)
    assert g.last_tile()[0] == 4
    g.set_kernel(4)
    g.run(res, 3, Distribution(ds.snps, 2, 2, 1), 10)
    g.run(res, 2, Distribution(ds.snps, 1, 2, 1), 10)
    with pytest.raises(FiunchoError):
        g.run(res, 2, Distribution(ds.snps - 5, 1, 2, 1), 10)
    with pytest.raises(FiunchoError):
        g.run(res, 5, Distribution(ds.snps, 4), 10)


@pytest.mark.parametrize("order,n_ranks,nc,nt", [(3, r, 1300, 1217) for r in (2, 3, 4, 5, 6, 7)] +
                         [(3, r, 9000, 9800) for r in (2, 3, 5)] +
                         [(2, r, 1300, 1217) for r in (2, 3, 5, 7)] + [(2, r, 9000, 9800) for r in (2, 3, 7)] +
                         [(4, r, 1300, 1217) for r in (2, 3, 5, 7)] + [(4, r, 9000, 9800) for r in (2, 3)])
def test_rank_layers_on_the_tensor_kernel(oracle, order, n_ranks, nc, nt):
    """MPIEngine gives rank r of N the strided share Distribution(snps, order-1, N, r)
    (MPIEngine.h:133-134, Distribution.h:172-176): on the tensor kernels (order 3: the
    list modes of the pair and the per-class kernels; order 2: the owned SNPs of one
    residue mod N; order 4: the owned k of each pair (i, j); classes that pack and classes
    that do not), forced and
    automatic, every rank's list equals the oracle's list of that rank, and the ranks'
    lists merged as MPIEngine merges them give the whole search."""
    from fiuncho_gb300 import Dataset, Distribution, GpuSearch, MPIEngine, Resident
    rng = np.random.default_rng(100 + n_ranks + 10 * order)
    snps = {2: 700, 3: 170 if nc < 5000 else 90, 4: 60 if nc < 5000 else 40}[order]
    maf = rng.uniform(0.05, 0.5, snps)[:, None]
    u = rng.random((snps, nc + nt))
    geno = ((u >= (1 - maf) ** 2).astype(np.uint8) + (u >= 1 - maf ** 2)).astype(np.uint8)
    ds = Dataset.from_genotypes(geno, np.r_[np.ones(nc, np.uint8), np.zeros(nt, np.uint8)])
    parts = []
    for kernel in (4, 0):
        g = GpuSearch(0, kernel=kernel)
        res = Resident(g.ctx, ds)
        for r in range(n_ranks):
            out, v64 = g.run(res, order, Distribution(snps, order - 1, n_ranks, r), 30, with_fp64=True)
            assert g.last_tile()[0] == 4
            _check_topn(oracle, ds, order, 30, out, v64, dist=(snps, n_ranks, r))
            if kernel == 0:
                parts += out
    whole = GpuSearch(0).run(ds, order, Distribution(snps, order - 1), 30)
    assert [x.combination for x in MPIEngine().gather(parts, 30)] == [x.combination for x in whole]


@pytest.mark.parametrize("order", [2, 3, 4])
@pytest.mark.parametrize("nc,nt", [(999, 1001), (9000, 9800)])
@pytest.mark.parametrize("step,offset", [(2, 1), (3, 0), (3, 2), (64, 5), (200, 0)])
def test_layer_tables(gs, oracle, order, nc, nt, step, offset):
    """Every table of a Distribution layer on the tensor kernels (classes that pack and
    classes that do not) equals the oracle's: the digest of all of them and their count
    (order 2, 130 SNPs: tiles of 64 owned SNPs end inside the residue class and past it;
    order 3, 70 SNPs: 32 or 64 listed j per item; order 4, 40 SNPs: tiles of 16 owned k)."""
    from fiuncho_gb300 import Distribution
    from fiuncho_gb300.search import Resident
    ds = _one_hot_dataset(7 + step, {2: 130, 3: 70, 4: 40}[order], nc, nt)
    res = Resident(gs.ctx, ds)
    want = oracle.table_digest(ds.data, ds.snps, ds.cases_words, ds.ctrls_words, order,
                               dist=(ds.snps, step, offset))
    got = gs.scan_digest(res, order, Distribution(ds.snps, order - 1, step, offset), 4)
    assert got == want


def test_elided_rejects_non_one_hot(gs):
    from fiuncho_gb300 import Dataset, Distribution, FiunchoError, GpuSearch, Resident
    rng = np.random.default_rng(2)
    ds = Dataset(100, 70, 6, 2, 2, rng.integers(0, 2 ** 63, 6 * 3 * 4, dtype=np.uint64))
    g = GpuSearch(0, kernel=3)
    with pytest.raises(FiunchoError):
        g.run(ds, 2, Distribution(6, 1), 5)


def test_one_hot_flag(gs, golden_testdata):
    from fiuncho_gb300 import Resident
    assert Resident(gs.ctx, _ds_from_golden(golden_testdata)).one_hot


# --------------------------------------------------------------- workload shapes
def test_order2_1000x4000_top10(gs, oracle):
    """Order-2 scan, 1 000 SNPs x 2 000/2 000 samples, top-10 (full oracle comparison)."""
    from fiuncho_gb300 import Dataset, Distribution, synth
    spec = synth.WORKLOADS["order2_1000x4000"]
    geno, is_case, planted = synth.simulate(spec)
    ds = Dataset.from_genotypes(geno, is_case)
    res, v64 = gs.run(ds, 2, Distribution(ds.snps, 1), 10, with_fp64=True)
    _check_topn(oracle, ds, 2, 10, res, v64, threads=16)
    assert res[0].combination == list(planted[0])


def test_order3_300x8000_top100(gs, oracle):
    """Order 3 at the 4 000/4 000 row shape on 300 SNPs (4.5e6 combinations), full oracle comparison."""
    from fiuncho_gb300 import Dataset, Distribution, synth
    spec = synth.ScanSpec(300, 4000, 4000, 3, 100, seed=21, planted=(3,), penetrance=0.65)
    geno, is_case, planted = synth.simulate(spec)
    ds = Dataset.from_genotypes(geno, is_case)
    res, v64 = gs.run(ds, 3, Distribution(ds.snps, 2), 100, with_fp64=True)
    _check_topn(oracle, ds, 3, 100, res, v64, threads=16)


@pytest.mark.parametrize("order,kernel", [(2, 1), (3, 1), (4, 1), (2, 3), (3, 3), (3, 2), (4, 3), (4, 2)])
def test_tiles_agree(oracle, order, kernel):
    """Every l-tile width (threads per prefix 32/64/128/256) of each kernel gives
    the same tables, and searches with autotuning on/off give identical lists."""
    from fiuncho_gb300 import Dataset, Distribution, GpuSearch, Resident
    rng = np.random.default_rng(order * 10 + kernel)
    snps, n_case, n_ctrl = 45, 333, 700
    maf = rng.uniform(0.05, 0.5, snps)[:, None]
    u = rng.random((snps, n_case + n_ctrl))
    geno = ((u >= (1 - maf) ** 2).astype(np.uint8) + (u >= 1 - maf ** 2)).astype(np.uint8)
    ds = Dataset.from_genotypes(geno, np.r_[np.ones(n_case, np.uint8), np.zeros(n_ctrl, np.uint8)])
    g = GpuSearch(0)
    res = Resident(g.ctx, ds)
    dist = Distribution(snps, order - 1)
    tabs = [g.scan_tables(res, order, dist, kernel=kernel, tp=tp) for tp in (32, 64, 128, 256)]
    mask = tabs[0] != 0xFFFFFFFF
    for t in tabs[1:]:
        assert np.array_equal(t[mask], tabs[0][mask])
    g.set_kernel(kernel)
    a = g.run(res, order, dist, 30, with_fp64=True)
    g.set_autotune(False)
    b = g.run(res, order, dist, 30, with_fp64=True)
    assert [x.combination for x in a[0]] == [x.combination for x in b[0]] and np.array_equal(a[1], b[1])
    r = [type("R", (), {"combination": x.combination, "val": x.val})() for x in a[0]]
    _check_topn(oracle, ds, order, 30, r, a[1])


def test_lg2_prefilter_bound(gs):
    """The tensor kernels' single-precision MI estimate assumes its log2 is within
    2^-18 of the exact value on every input it can see (counts up to 2^17 - 1,
    shifted by 2^-20); checked exhaustively against double precision."""
    import ctypes as C
    err = C.c_double(-1)
    gs.ctx.check(gs.ctx.lib.fiu_probe_lg2_error(gs.ctx.h, (1 << 17) - 1, C.byref(err)))
    assert 0 <= err.value < 2.0 ** -18, err.value


def test_bounded_wait_gives_up(gs):
    """Failure detection without a fault: a device wait on an mbarrier phase that
    nothing completes gives up after its limit (the tensor kernels then report
    FIU_ERR_TIMEOUT) and the context stays usable; with the arrival it completes
    at once."""
    import ctypes as C
    done, ms = C.c_int(-1), C.c_double(-1)
    gs.ctx.check(gs.ctx.lib.fiu_probe_wait_limit(gs.ctx.h, 20000, 0, C.byref(done), C.byref(ms)))
    assert done.value == 0 and 20.0 <= ms.value < 1000.0, (done.value, ms.value)
    gs.ctx.check(gs.ctx.lib.fiu_probe_wait_limit(gs.ctx.h, 20000, 1, C.byref(done), C.byref(ms)))
    assert done.value == 1 and ms.value < 20.0, (done.value, ms.value)
    from fiuncho_gb300 import Dataset, Distribution
    ds = _one_hot_dataset(3, 30, 200, 200)  # the context still searches
    assert len(gs.run(ds, 3, Distribution(30, 2), 5)) == 5


def test_pair_kernel_launch_longer_than_a_wait_bound(gs, oracle):
    """An order-3 scan whose chunks run for seconds on the CTA-pair kernel
    (10 000 SNPs x 2 000/2 000 samples, 1.7e11 combinations, ~5 s): no wait of
    either CTA of a pair may span the launch, since every wait gives up after 2 s
    (FIU_ERR_TIMEOUT).  The returned values are checked against the oracle."""
    from fiuncho_gb300 import Distribution
    from helpers import assert_sorted_desc, exact_mi
    ds = _one_hot_dataset(17, 10000, 2000, 2000)
    results, v64 = gs.run(ds, 3, Distribution(ds.snps, 2), 20, with_fp64=True)
    assert gs.last_tile()[0] == 4  # the tensor kernel served it
    got = np.array([r.combination for r in results], np.int32)
    assert len(got) == 20
    assert_sorted_desc(v64)
    want = exact_mi(oracle, ds.data, ds.cases_words, ds.ctrls_words, ds.cases, ds.ctrls, 3, got)
    assert np.allclose(v64, want, rtol=1e-5, atol=1e-12)


def _one_hot_dataset(seed, snps, n_case, n_ctrl):
    from fiuncho_gb300 import Dataset
    rng = np.random.default_rng(seed)
    maf = rng.uniform(0.05, 0.5, snps)[:, None]
    u = rng.random((snps, n_case + n_ctrl))
    geno = ((u >= (1 - maf) ** 2).astype(np.uint8) + (u >= 1 - maf ** 2)).astype(np.uint8)
    return Dataset.from_genotypes(geno, np.r_[np.ones(n_case, np.uint8), np.zeros(n_ctrl, np.uint8)])


@pytest.mark.parametrize("snps,n_case,n_ctrl", [(3, 1, 1), (4, 65, 63), (33, 130, 1), (34, 64, 64),
                                                (97, 200, 129), (100, 129, 300), (130, 100, 60000),
                                                (40, 5000, 4100), (97, 4500, 4500), (98, 1, 9000)])
def test_tensor_tile_edges(oracle, snps, n_case, n_ctrl):
    """tcgen05 kernels vs the full-table kernel at tile edges (SNP counts around the
    32 x 128 and 32 x 96 work items, one-sample classes, odd word counts padded to 128
    samples), in both forms -- one accumulator for both classes (controls weighted by
    4^h, N 256) and one accumulator per class (N 192, classes too large to pack):
    identical tables for every combination and identical top-N lists."""
    from fiuncho_gb300 import Distribution, GpuSearch, Resident
    ds = _one_hot_dataset(snps * 7 + n_case, snps, n_case, n_ctrl)
    g = GpuSearch(0)
    res = Resident(g.ctx, ds)
    dist = Distribution(snps, 2)
    full = g.scan_tables(res, 3, dist, kernel=1)
    tens = g.scan_tables(res, 3, dist, kernel=4)
    mask = full != 0xFFFFFFFF
    assert np.array_equal(tens[mask], full[mask])
    out = min(20, math.comb(snps, 3))
    g.set_kernel(1)
    a = g.run(res, 3, dist, out, with_fp64=True)
    g.set_kernel(4)
    b = g.run(res, 3, dist, out, with_fp64=True)
    packed = any(4 ** h > n_case and n_case + 4 ** h * n_ctrl < 2 ** 24 for h in range(1, 9))
    assert g.last_tile() == (4, 256 if packed else 192)
    assert [x.combination for x in a[0]] == [x.combination for x in b[0]] and np.array_equal(a[1], b[1])
    _check_topn(oracle, ds, 3, out, b[0], b[1])


def test_tensor_prefilter_many_chunks(oracle):
    """A top-5 search over 260 SNPs runs many chunks with a tight threshold, where the
    single-precision prefilter rejects nearly every combination: the result equals the
    exact reduced-work kernel's and the oracle's."""
    from fiuncho_gb300 import Distribution, GpuSearch, Resident
    ds = _one_hot_dataset(5, 260, 1500, 1700)
    g = GpuSearch(0)
    res = Resident(g.ctx, ds)
    dist = Distribution(260, 2)
    g.set_kernel(3)
    a = g.run(res, 3, dist, 5, with_fp64=True)
    g.set_kernel(4)
    b = g.run(res, 3, dist, 5, with_fp64=True)
    assert g.last_tile()[0] == 4
    assert [x.combination for x in a[0]] == [x.combination for x in b[0]] and np.array_equal(a[1], b[1])
    _check_topn(oracle, ds, 3, 5, b[0], b[1], threads=16)


@pytest.mark.parametrize("snps,n_case,n_ctrl", [(2, 1, 1), (3, 65, 63), (66, 130, 1), (129, 200, 129),
                                                (130, 5000, 4100), (200, 100, 60000), (131, 1, 9000)])
def test_tensor2_tile_edges(oracle, snps, n_case, n_ctrl):
    """Order-2 tcgen05 kernel vs the full-table kernel around the 64 x 128 work item,
    with classes that share one accumulator and classes that do not: identical tables
    for every pair and identical top-N lists, checked against the oracle."""
    from fiuncho_gb300 import Distribution, GpuSearch, Resident
    ds = _one_hot_dataset(snps * 5 + n_ctrl, snps, n_case, n_ctrl)
    g = GpuSearch(0)
    res = Resident(g.ctx, ds)
    dist = Distribution(snps, 1)
    full = g.scan_tables(res, 2, dist, kernel=1)
    tens = g.scan_tables(res, 2, dist, kernel=4)
    mask = full != 0xFFFFFFFF
    assert np.array_equal(tens[mask], full[mask])
    out = min(30, math.comb(snps, 2))
    g.set_kernel(1)
    a = g.run(res, 2, dist, out, with_fp64=True)
    g.set_kernel(4)
    b = g.run(res, 2, dist, out, with_fp64=True)
    assert g.last_tile() == (4, 256)
    assert [x.combination for x in a[0]] == [x.combination for x in b[0]] and np.array_equal(a[1], b[1])
    _check_topn(oracle, ds, 2, out, b[0], b[1])


def test_order2_40000x16000_top1000(oracle):
    """Order 2 at full size (40 000 SNPs x 8 000/8 000 samples, 8e8 pairs, top-1 000): the
    tcgen05 kernel and the reduced-work CUDA-core kernel give identical lists and FP64
    values, and every returned MI equals the oracle's FP64 MI of its pair."""
    from fiuncho_gb300 import Dataset, Distribution, GpuSearch, Resident, synth
    spec = synth.WORKLOADS["order2_40000x16000"]
    geno, is_case, planted = synth.simulate(spec)
    ds = Dataset.from_genotypes(geno, is_case)
    del geno
    g = GpuSearch(0)
    res = Resident(g.ctx, ds)
    dist = Distribution(ds.snps, 1)
    g.set_kernel(4)
    a, av = g.run(res, 2, dist, 1000, with_fp64=True)
    g.set_kernel(3)
    b, bv = g.run(res, 2, dist, 1000, with_fp64=True)
    assert [x.combination for x in a] == [x.combination for x in b] and np.array_equal(av, bv)
    ex = exact_mi(oracle, ds.data, ds.cases_words, ds.ctrls_words, ds.cases, ds.ctrls, 2,
                  [x.combination for x in a])
    assert np.allclose(av, ex, rtol=1e-9, atol=0)
    assert_sorted_desc(av)


# ------------------------------------------------ segmented evaluation and depth-first traversals
@pytest.mark.parametrize("name", ["o2", "o3", "o4", "ties"])
def test_search_vs_reference_traversals(gs, oracle, golden_traversals, name):
    """The GPU list against the reference's segmented ThreadedSearch and its two depth-first
    benchmark programs (benchmarks/*_sequential_search.cpp): the same combinations up to ties
    at the cut-off.  On the tie case the cut-off falls inside a group of combinations whose
    tables are permutations of one another (duplicated SNP columns): the reference keeps the
    member its traversal meets first, the GPU the member with the larger double-precision MI
    (summed in table order, the members differ in the last bits), then the lower
    combination."""
    from fiuncho_gb300 import Dataset, Distribution
    g = golden_traversals
    ds = Dataset.from_genotypes(g[name + "_geno"], g[name + "_is_case"])
    order, outputs = (int(x) for x in g[name + "_meta"])
    res, v64 = gs.run(ds, order, Distribution(ds.snps, order - 1), outputs, with_fp64=True)
    got = _check_topn(oracle, ds, order, outputs, res, v64)
    ex = lambda cs: exact_mi(oracle, ds.data, ds.cases_words, ds.ctrls_words, ds.cases, ds.ctrls, order, cs)
    for tag in ("seg", "dfs", "dfsseg"):
        rc = g[name + "_%s_combos" % tag]
        rv = g[name + "_%s_vals" % tag].astype(np.float64)
        assert_topn_equivalent(got, rc, ex, 2 * float(np.max(np.abs(rv - ex(rc)))) + 1e-12)
    if name == "ties":
        tied = sorted(as_set(g["ties_seg_combos"]) ^ as_set(g["ties_dfs_combos"]))
        v = ex(tied)
        assert len(tied) == 2 and abs(v[0] - v[1]) <= 1e-12 * abs(v[0])
        assert len(as_set(got) & set(tied)) == 1
