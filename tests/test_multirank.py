"""Multi-rank MPIEngine on CPU: two `gloo` ranks, each searching its
Distribution(snps, order-1, 2, rank) share, rank 0 gathering (MPIEngine.h:133-174).

The per-rank search here is the oracle (the CPU restatement of the reference's
ThreadedSearch with one worker) standing in for the GPU search, so the test
covers the engine's split, serialisation, gather, sort and truncation on the
host exactly as a multi-GPU run uses them."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


class OracleSearch:
    """Search::run over the oracle (one worker), for the engine test."""

    def __init__(self, threads=1):
        from oracle.oracle import Oracle
        self.o = Oracle()
        self.threads = threads

    def run(self, ds, order, distribution, outputs):
        from fiuncho_gb300 import Result
        c, v, v64, _ = self.o.search(ds.data, ds.snps, ds.cases, ds.ctrls, ds.cases_words, ds.ctrls_words, order,
                                     outputs, threads=self.threads, mi_mode=1,
                                     dist=(distribution.n, distribution.step, distribution.offset))
        return [Result(list(map(int, cc)), float(x)) for cc, x in zip(c, v64)]


class ShardedOracleSearch(OracleSearch):
    """A search with run_shard (as GpuSearch has): MPIEngine then gives rank r
    shard r of N instead of the strided Distribution.  The oracle's shard r is
    a contiguous range of the prefix ordinals (the whole search's work units
    split in N equal ranges), searched prefix by prefix."""

    def run_shard(self, ds, order, shard, n_shards, outputs):
        from fiuncho_gb300 import Distribution, Result
        import math
        units = math.comb(ds.snps, order - 1)
        lo = units // n_shards * shard + min(shard, units % n_shards)
        hi = lo + units // n_shards + (1 if shard < units % n_shards else 0)
        res = []
        for m in range(lo, hi):
            res += self.run(ds, order, Distribution(ds.snps, order - 1, units, m), outputs)
        res.sort(key=lambda r: (-r.val, r.combination))
        return [Result(r.combination, r.val) for r in res[:outputs]]


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, data_path, out_path, sharded=False):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import torch.distributed as dist

    from fiuncho_gb300 import Dataset, MPIEngine
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        z = np.load(data_path)
        ds = Dataset.from_genotypes(z["geno"], z["is_case"])
        res = MPIEngine().run(ShardedOracleSearch if sharded else OracleSearch, None, 3, 25, dataset=ds)
        np.save(out_path % rank, np.array([r.combination + [r.val] for r in res], np.float64).reshape(-1, 4))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("sharded", [False, True])
def test_two_rank_gather_equals_single_rank(tmp_path, sharded):
    """Strided Distribution shares, or (a search with run_shard, as GpuSearch) shards
    of the whole search: either way rank 0's gathered result is the whole search's."""
    import multiprocessing as mp

    from fiuncho_gb300 import Dataset, Distribution
    rng = np.random.default_rng(11)
    snps, n_case, n_ctrl = 40, 300, 333
    maf = rng.uniform(0.05, 0.5, snps)[:, None]
    u = rng.random((snps, n_case + n_ctrl))
    geno = ((u >= (1 - maf) ** 2).astype(np.uint8) + (u >= 1 - maf ** 2)).astype(np.uint8)
    is_case = np.r_[np.ones(n_case, np.uint8), np.zeros(n_ctrl, np.uint8)]
    data_path = str(tmp_path / "data.npz")
    np.savez(data_path, geno=geno, is_case=is_case)
    out_path = str(tmp_path / "rank%d.npy")
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, data_path, out_path, sharded)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    for p in procs:
        if p.is_alive():
            p.kill()
            p.join()
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got0, got1 = np.load(out_path % 0), np.load(out_path % 1)
    assert got1.shape[0] == 0  # non-zero ranks return nothing (MPIEngine.h:176-181)
    ds = Dataset.from_genotypes(geno, is_case)
    full = OracleSearch().run(ds, 3, Distribution(snps, 2), 25)
    assert [list(map(int, r[:3])) for r in got0] == [r.combination for r in full]
    assert np.allclose(got0[:, 3], [r.val for r in full], rtol=1e-12)


def _rank_main_subgroup(rank, world, port, data_path, out_path):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import torch.distributed as dist

    from fiuncho_gb300 import Dataset, MPIEngine
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sub = dist.new_group([1, 2])  # every rank takes part in creating it
        if rank in (1, 2):
            z = np.load(data_path)
            ds = Dataset.from_genotypes(z["geno"], z["is_case"])
            res = MPIEngine(group=sub).run(OracleSearch, None, 3, 25, dataset=ds)
            np.save(out_path % rank, np.array([r.combination + [r.val] for r in res], np.float64).reshape(-1, 4))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_subgroup_gather_goes_to_the_groups_first_rank(tmp_path):
    """An engine over a process subgroup that leaves out global rank 0 gathers on the
    group's own rank 0 (global rank 1) and returns the whole search there."""
    import multiprocessing as mp

    from fiuncho_gb300 import Dataset, Distribution
    rng = np.random.default_rng(12)
    snps, n_case, n_ctrl = 30, 250, 260
    maf = rng.uniform(0.05, 0.5, snps)[:, None]
    u = rng.random((snps, n_case + n_ctrl))
    geno = ((u >= (1 - maf) ** 2).astype(np.uint8) + (u >= 1 - maf ** 2)).astype(np.uint8)
    is_case = np.r_[np.ones(n_case, np.uint8), np.zeros(n_ctrl, np.uint8)]
    data_path = str(tmp_path / "data.npz")
    np.savez(data_path, geno=geno, is_case=is_case)
    out_path = str(tmp_path / "rank%d.npy")
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main_subgroup, args=(r, 3, port, data_path, out_path)) for r in range(3)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    for p in procs:
        if p.is_alive():
            p.kill()
            p.join()
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got1, got2 = np.load(out_path % 1), np.load(out_path % 2)
    assert got2.shape[0] == 0
    ds = Dataset.from_genotypes(geno, is_case)
    full = OracleSearch().run(ds, 3, Distribution(snps, 2), 25)
    assert [list(map(int, r[:3])) for r in got1] == [r.combination for r in full]
