"""The served request stream (fiu_server_*): continuous batching under a
device-memory budget.  Each scan's result must be the same alone and in the
mix (and equal to fiu_search's); latency statistics are reported."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ds(seed, snps, n_case, n_ctrl, one_hot=True):
    from fiuncho_gb300 import Dataset
    rng = np.random.default_rng(seed)
    if not one_hot:  # random bits: the full-table kernel in the rounds
        cw, tw = (n_case + 63) // 64, (n_ctrl + 63) // 64
        return Dataset(n_case, n_ctrl, snps, cw, tw, rng.integers(0, 2 ** 63, snps * 3 * (cw + tw), dtype=np.uint64))
    maf = rng.uniform(0.05, 0.5, snps)[:, None]
    u = rng.random((snps, n_case + n_ctrl))
    geno = ((u >= (1 - maf) ** 2).astype(np.uint8) + (u >= 1 - maf ** 2)).astype(np.uint8)
    return Dataset.from_genotypes(geno, np.r_[np.ones(n_case, np.uint8), np.zeros(n_ctrl, np.uint8)])


# seed, snps, cases, controls, order, outputs[, one-hot]: one-hot scans take the solo lane
# (tensor-core / pair-major kernels), the others the rounds
MIX = [(11, 400, 1200, 1300, 2, 50), (12, 150, 3000, 2500, 3, 50), (13, 60, 900, 700, 4, 25),
       (14, 900, 800, 800, 2, 20), (15, 220, 2000, 2000, 3, 100), (16, 35, 5000, 4000, 3, 10),
       (17, 70, 600, 500, 3, 30, False), (18, 40, 700, 650, 4, 20, False), (19, 300, 900, 900, 2, 15, False)]


def _same(a, b):
    (r1, v1, _), (r2, v2) = a, b
    assert [x.combination for x in r1] == [x.combination for x in r2]
    assert np.array_equal(v1, v2)


def test_server_alone_and_in_mix_identical():
    from fiuncho_gb300 import Distribution, GpuSearch, Server
    gs = GpuSearch(0)
    data = [_ds(*m[:4], *m[6:]) for m in MIX]
    ref = [gs.run(ds, m[4], Distribution(ds.snps, m[4] - 1), m[5], with_fp64=True) for ds, m in zip(data, MIX)]
    srv = Server(0)
    try:
        # alone, one after the other
        for ds, m, r in zip(data, MIX, ref):
            t = srv.submit(ds, m[4], m[5])
            _same(srv.result(t), r)
        # in the mix: all submitted at once, plus repeats arriving while others run
        tickets = [srv.submit(ds, m[4], m[5]) for ds, m in zip(data, MIX)]
        later = []
        for i in (4, 0, 2):
            time.sleep(0.01)
            later.append((i, srv.submit(data[i], MIX[i][4], MIX[i][5])))
        for i, t in enumerate(tickets):
            _same(srv.result(t), ref[i])
        for i, t in later:
            _same(srv.result(t), ref[i])
        st = srv.stats()
        assert st["completed"] == 2 * len(MIX) + 3 and st["failed"] == 0
        assert st["p50_ms"] > 0 and st["p99_ms"] >= st["p50_ms"]
        assert st["rounds"] > 0 and st["bytes_in_use"] == 0
        assert st["solo"] == 2 * 6 + 3  # the one-hot scans, twice, and the three repeats
    finally:
        srv.close()


@pytest.mark.parametrize("one_hot", [True, False])
def test_server_budget_admits_one_at_a_time(one_hot):
    """A budget that fits one scan at a time still completes everything, and the
    admitted scans never hold more than the budget, whether they run on the solo
    lanes (one-hot: tensor-core kernels) or in the rounds (not one-hot)."""
    from fiuncho_gb300 import Distribution, FiunchoError, GpuSearch, Server
    gs = GpuSearch(0)
    data = [_ds(20 + i, 200, 1000, 1000, one_hot) for i in range(4)]
    budget = 8 * 1024 * 1024
    srv = Server(0, budget_bytes=budget)
    try:
        tickets = [srv.submit(ds, 3, 20) for ds in data]
        seen = []
        pending = list(zip(data, tickets))
        while pending:
            seen.append(srv.stats()["bytes_in_use"])
            ds, t = pending[0]
            r = srv.result(t, 1)
            if r is None:
                continue
            _same(r, gs.run(ds, 3, Distribution(ds.snps, 2), 20, with_fp64=True))
            pending.pop(0)
        st = srv.stats()
        assert max(seen) <= budget and 0 < st["peak_bytes"] <= budget
        assert st["completed"] == 4 and st["bytes_in_use"] == 0
        assert st["solo"] == (4 if one_hot else 0)
        with pytest.raises(FiunchoError):
            srv.submit(_ds(30, 3000, 4000, 4000), 3, 10)  # larger than the whole budget
    finally:
        srv.close()


def test_server_concurrent_submitters():
    from fiuncho_gb300 import Server
    srv = Server(0)
    data = [_ds(40 + i, 120, 700, 800) for i in range(6)]
    out = {}

    def client(i):
        t = srv.submit(data[i], 2 + i % 2, 15)
        out[i] = srv.result(t)

    th = [threading.Thread(target=client, args=(i,)) for i in range(6)]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=120)
    try:
        assert len(out) == 6 and all(len(r[0]) == 15 for r in out.values())
        # an unknown (or already collected) ticket is an invalid argument
        from fiuncho_gb300 import _lib
        assert srv.lib.fiu_server_poll(srv.h, 123456789, 0, None, None, None, None, None) == _lib.FIU_ERR_INVALID
    finally:
        srv.close()


def test_server_solo_lanes_overlap():
    """Two tensor-core scans submitted together run on the two solo lanes at the
    same time (their device work overlaps) and give the results of each alone."""
    from fiuncho_gb300 import Distribution, GpuSearch, Server
    gs = GpuSearch(0)
    data = [_ds(50 + i, 1500, 3000, 3000) for i in range(2)]
    ref = [gs.run(ds, 3, Distribution(ds.snps, 2), 40, with_fp64=True) for ds in data]
    srv = Server(0)
    try:
        tickets = [srv.submit(ds, 3, 40) for ds in data]
        for t, r in zip(tickets, ref):
            _same(srv.result(t), r)
        st = srv.stats()
        assert st["completed"] == 2 and st["solo"] == 2
        assert st["overlapped"] == 2
    finally:
        srv.close()


def test_server_shards_identical_to_run_shard():
    """Shards submitted to the server (solo lanes and rounds) give run_shard's lists."""
    from fiuncho_gb300 import GpuSearch, Server
    gs = GpuSearch(0)
    cases = [(_ds(60, 700, 1500, 1500), 3, 30), (_ds(61, 90, 700, 650, one_hot=False), 3, 20),
             (_ds(62, 60, 2000, 1900), 4, 25)]
    srv = Server(0)
    try:
        tickets = [(srv.submit(ds, order, out, r, 4), ds, order, out, r) for ds, order, out in cases for r in range(4)]
        for t, ds, order, out, r in tickets:
            _same(srv.result(t), gs.run_shard(ds, order, r, 4, out, with_fp64=True))
        st = srv.stats()
        assert st["completed"] == len(tickets) and st["rounds"] > 0
    finally:
        srv.close()


def test_server_destroy_cancels_running_scans():
    """Destroying a server while a long scan runs on a solo lane returns once the scan's
    current chunk is done (the scan is cancelled), not after the whole scan."""
    from fiuncho_gb300 import Server
    ds = _ds(70, 4000, 4000, 4000)  # order 3: about 1e10 combinations x 8 000 samples, ~0.6 s
    srv = Server(0)
    srv.submit(ds, 3, 10)
    deadline = time.time() + 30
    while time.time() < deadline:  # admitted (its data set uploaded), then on a solo lane
        st = srv.stats()
        if st["queued"] == 0 and st["active"] == 1:
            break
        time.sleep(0.002)
    time.sleep(0.15)
    st = srv.stats()
    assert st["completed"] == 0, "the scan finished before the server was destroyed"
    t0 = time.perf_counter()
    srv.close()
    assert time.perf_counter() - t0 < 0.6


def test_server_shortest_first():
    """FIU_SERVE_SHORTEST_FIRST: with both solo lanes busy on two long scans, queued scans are
    taken least work first (the smallest finishes before the largest starts), and every
    result is the scan's result alone."""
    from fiuncho_gb300 import Distribution, GpuSearch, Server
    gs = GpuSearch(0)
    long_ds = [_ds(40 + i, 2000, 4000, 4000) for i in range(2)]
    small = [(50, 3000, 1000, 1000), (51, 2000, 1000, 1000), (52, 1000, 1000, 1000), (53, 400, 1000, 1000)]
    small_ds = [_ds(*m) for m in small]
    ref_long = [gs.run(ds, 3, Distribution(ds.snps, 2), 20, with_fp64=True) for ds in long_ds]
    ref_small = [gs.run(ds, 2, Distribution(ds.snps, 1), 20, with_fp64=True) for ds in small_ds]
    with pytest.raises(Exception):
        Server(0, policy=7)
    srv = Server(0, policy=Server.SHORTEST_FIRST)
    try:
        tl = [srv.submit(ds, 3, 20) for ds in long_ds]
        time.sleep(0.03)  # both lanes take a long scan
        ts, t0 = [], []
        for ds in small_ds:  # largest first
            t0.append(time.perf_counter())
            ts.append(srv.submit(ds, 2, 20))
        done = []
        for t, s0, r in zip(ts, t0, ref_small):
            res, v64, lat = srv.result(t)
            _same((res, v64, lat), r)
            done.append(s0 + lat / 1e3)
        for t, r in zip(tl, ref_long):
            _same(srv.result(t), r)
        assert done[3] < done[0], done
        st = srv.stats()
        assert st["completed"] == 6 and st["failed"] == 0
    finally:
        srv.close()
