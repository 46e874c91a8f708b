"""The batched form (fiu_search_batch): many scans of different orders, sizes
and sample counts progress together in rounds on the device (optionally one
CUDA graph); each scan's result must be identical to searching it alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scan_data(seed, snps, n_case, n_ctrl, one_hot=True):
    from fiuncho_gb300 import Dataset
    rng = np.random.default_rng(seed)
    if not one_hot:
        cw, tw = (n_case + 63) // 64, (n_ctrl + 63) // 64
        return Dataset(n_case, n_ctrl, snps, cw, tw, rng.integers(0, 2 ** 63, snps * 3 * (cw + tw), dtype=np.uint64))
    maf = rng.uniform(0.05, 0.5, snps)[:, None]
    u = rng.random((snps, n_case + n_ctrl))
    geno = ((u >= (1 - maf) ** 2).astype(np.uint8) + (u >= 1 - maf ** 2)).astype(np.uint8)
    return Dataset.from_genotypes(geno, np.r_[np.ones(n_case, np.uint8), np.zeros(n_ctrl, np.uint8)])


SCANS = [  # seed, snps, cases, ctrls, order, outputs, one_hot, (step, offset)
    (1, 300, 700, 900, 2, 50, True, (1, 0)),
    (2, 90, 2000, 1500, 3, 50, True, (1, 0)),
    (3, 40, 650, 1333, 4, 20, True, (1, 0)),
    (4, 120, 999, 1001, 3, 100, True, (3, 1)),
    (5, 60, 300, 200, 3, 30, False, (1, 0)),
    (6, 700, 1500, 1500, 2, 7, True, (1, 0)),
    (7, 25, 4000, 4100, 3, 2000, True, (1, 0)),  # fewer combinations than outputs
    (8, 12, 64, 64, 5, 10, True, (1, 0)),        # order 5: single-scan path inside the batch
    (9, 34, 1200, 800, 4, 40, True, (2, 1)),     # order 4, reduced-work kernel, a Distribution layer
    (10, 30, 500, 520, 4, 25, False, (1, 0)),    # order 4, full kernel
]


@pytest.fixture(scope="module")
def batch_setup():
    from fiuncho_gb300 import Distribution, GpuSearch, Resident
    gs = GpuSearch(0)
    reqs, alone = [], []
    for seed, snps, nc, nt, order, outputs, one_hot, (step, off) in SCANS:
        ds = _scan_data(seed, snps, nc, nt, one_hot)
        res = Resident(gs.ctx, ds)
        dist = Distribution(snps, order - 1, step, off)
        reqs.append((res, order, dist, outputs))
        alone.append(gs.run(res, order, dist, outputs, with_fp64=True))
    return gs, reqs, alone


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_identical_to_alone(batch_setup, use_graph):
    gs, reqs, alone = batch_setup
    got = gs.run_batch(reqs, use_graph=use_graph)
    for (r1, v1), (r2, v2) in zip(alone, got):
        assert [x.combination for x in r1] == [x.combination for x in r2]
        assert np.array_equal(v1, v2)
        assert [x.val for x in r1] == [x.val for x in r2]


def test_batch_repeatable_and_mixed_subsets(batch_setup):
    """A scan's result does not depend on which other scans share the rounds."""
    gs, reqs, alone = batch_setup
    for subset in ([0, 3], [1, 2, 4, 6], [5], list(range(len(reqs)))[::-1]):
        got = gs.run_batch([reqs[i] for i in subset])
        for i, (r, v) in zip(subset, got):
            assert [x.combination for x in r] == [x.combination for x in alone[i][0]]
            assert np.array_equal(v, alone[i][1])


def test_batch_against_oracle(batch_setup, oracle):
    """Spot check of two batched scans against the CPU oracle (top-N up to ties)."""
    import math
    import sys
    sys.path.insert(0, __import__("os").path.dirname(__file__))
    from helpers import assert_topn_equivalent, exact_mi
    gs, reqs, _ = batch_setup
    got = gs.run_batch(reqs)
    for i in (1, 2, 4, 8):
        seed, snps, nc, nt, order, outputs, one_hot, (step, off) = SCANS[i]
        ds = _scan_data(seed, snps, nc, nt, one_hot)
        c, _, o64, _ = oracle.search(ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words, order,
                                     outputs, threads=1, mi_mode=1, dist=(snps, step, off))
        r, v = got[i]
        comb = np.array([x.combination for x in r], np.int32)
        ex = lambda cs: exact_mi(oracle, ds.data, ds.cases_words, ds.ctrls_words, ds.cases, ds.ctrls, order, cs)
        assert_topn_equivalent(comb, c, ex, 1e-5 * abs(float(o64[-1])) + 1e-12)
        assert np.allclose(v, ex(comb), rtol=1e-9)


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_shards_identical_to_run_shard(batch_setup, use_graph):
    """Shard r of N of a whole-data-set scan in the batch (round kernels, tensor-core and
    pair-major lanes alike) gives the same list as run_shard on it alone, and the shards
    of a scan merged by (MI desc, combination asc) give the whole scan's list."""
    gs, reqs, alone = batch_setup
    whole = [(i, q) for i, q in enumerate(reqs) if q[2].step == 1 and q[2].offset == 0]
    sharded = []
    for i, (res, order, dist, outputs) in whole:
        for r in range(3):
            sharded.append((i, (res, order, dist, outputs, r, 3)))
    got = gs.run_batch([q for _, q in sharded], use_graph=use_graph)
    merged = {}
    for (i, (res, order, dist, outputs, r, n)), (rs, v) in zip(sharded, got):
        want, wv = gs.run_shard(res, order, r, n, outputs, with_fp64=True)
        assert [x.combination for x in rs] == [x.combination for x in want]
        assert np.array_equal(v, wv)
        merged.setdefault(i, []).extend(zip((-x for x in v), (x.combination for x in rs)))
    for i, (res, order, dist, outputs) in whole:
        m = sorted(merged[i])[:outputs]
        assert [c for _, c in m] == [x.combination for x in alone[i][0]]


def test_batch_rejects_shard_of_a_layer(batch_setup):
    from fiuncho_gb300 import FiunchoError
    gs, reqs, _ = batch_setup
    res, order, dist, outputs = reqs[3]  # a Distribution(..., 3, 1) layer
    with pytest.raises(FiunchoError):
        gs.run_batch([(res, order, dist, outputs, 0, 2)])
