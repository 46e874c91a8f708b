"""The reference-facing search API on the GB300 library.

Mirrors the reference's public surface for the search path:

* ``Distribution`` -- ``Distribution<int>`` (include/fiuncho/Distribution.h:24-203)
* ``Result``       -- ``Result<int,float>`` (include/fiuncho/utils/Result.h:17-70)
* ``GpuSearch``    -- a ``Search`` (include/fiuncho/Search.h:19-46) whose
  ``run(dataset, order, distribution, outputs)`` executes on one GPU
* ``MPIEngine``    -- ``MPIEngine::run<T>(inputs, order, outputs, args...)``
  (include/fiuncho/MPIEngine.h:108-182): every rank reads the data set, takes
  ``Distribution(snps, order-1, size, rank)``, runs the search and rank 0
  gathers, sorts and truncates.  Ranks come from ``torch.distributed`` when it
  is initialised, otherwise there is one rank.

Errors are raised as ``FiunchoError`` (the reference throws
``std::runtime_error``).
"""
from __future__ import annotations

import ctypes as C
import functools

import numpy as np

from . import _lib
from ._lib import FiunchoError
from .dataset import Dataset


@functools.total_ordering
class Result:
    """``Result<int, float>``: ordered by ``val`` only (Result.h:22-33)."""

    __slots__ = ("combination", "val")

    def __init__(self, combination=(), val=0.0):
        self.combination = list(combination)
        self.val = float(val)

    def __lt__(self, other):
        return self.val < other.val

    def __eq__(self, other):
        return self.val == other.val and self.combination == other.combination

    def __hash__(self):
        return hash((tuple(self.combination), self.val))

    def str(self) -> str:
        """Text form ``"i j ... val"`` with 6 significant digits (Result.h:37-45)."""
        return " ".join(str(i) for i in self.combination) + " " + ("%g" % np.float32(self.val))

    __str__ = str

    def __repr__(self):
        return "Result(%s, %r)" % (self.combination, self.val)

    def serialize(self) -> bytes:
        """Binary form of Result::serialize (Result.h:47-56): size_t count, int
        indices, float value, native byte order."""
        c = np.asarray(self.combination, np.int32)
        return np.uint64(len(c)).tobytes() + c.tobytes() + np.float32(self.val).tobytes()

    @staticmethod
    def deserialize(buf: bytes, pos: int = 0):
        n = int(np.frombuffer(buf, np.uint64, 1, pos)[0])
        pos += 8
        comb = np.frombuffer(buf, np.int32, n, pos).tolist()
        pos += 4 * n
        val = float(np.frombuffer(buf, np.float32, 1, pos)[0])
        return Result(comb, val), pos + 4


class Distribution:
    """``Distribution<int>(n, k, step, offset)``; ``layer`` composes splits."""

    def __init__(self, n: int, k: int, step: int = 1, offset: int = 0):
        if step < 1 or offset < 0 or k < 0 or n < 0:
            raise ValueError("Distribution requires n, k, offset >= 0 and step >= 1")
        self.n, self.k, self.step, self.offset = int(n), int(k), int(step), int(offset)

    def layer(self, step: int, offset: int) -> "Distribution":
        return Distribution(self.n, self.k, self.step * step, self.offset * step + offset)

    def c_struct(self):
        return _lib.Distribution_t(self.n, self.k, self.step, self.offset)

    def __iter__(self):
        """Owned k-combinations in the reference's enumeration order."""
        import itertools
        for r, c in enumerate(itertools.combinations(range(self.n), self.k)):
            if r >= self.offset and (r - self.offset) % self.step == 0:
                yield list(c)

    def __repr__(self):
        return "Distribution(n=%d, k=%d, step=%d, offset=%d)" % (self.n, self.k, self.step, self.offset)


class Context:
    """One device context of the C library (stream + scratch)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.fiu_create(int(device), C.byref(h))
        if rc:
            raise FiunchoError(rc, "cannot create a context on CUDA device %d" % device)
        self.h = h
        self.device = device

    def check(self, rc):
        if rc:
            raise FiunchoError(rc, self.lib.fiu_last_error(self.h).decode())

    @property
    def launches(self) -> int:
        return int(self.lib.fiu_launch_count(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.fiu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _c_dataset(ds: Dataset):
    data = np.ascontiguousarray(ds.data, np.uint64)
    return _lib.Dataset_t(_lib.ptr(data, C.c_uint64), ds.snps, ds.cases, ds.ctrls, ds.cases_words,
                          ds.ctrls_words), data


class Resident:
    """A data set held in device memory (uploaded once, searched many times)."""

    def __init__(self, ctx: Context, ds: Dataset):
        self.ctx = ctx
        cds, self._keep = _c_dataset(ds)
        h = C.c_void_p()
        ctx.check(ctx.lib.fiu_dataset_upload(ctx.h, C.byref(cds), C.byref(h)))
        self.h = h
        self.snps, self.cases, self.ctrls = ds.snps, ds.cases, ds.ctrls
        self._keep = None

    @classmethod
    def adopt(cls, ctx: "Context", handle) -> "Resident":
        """Wraps a resident data set made by the library (e.g. fiu_dataset_upload_genotypes)."""
        r = cls.__new__(cls)
        r.ctx, r.h, r._keep = ctx, handle, None
        d = _lib.Dataset_t()
        ctx.check(ctx.lib.fiu_dataset_packed(ctx.h, handle, C.byref(d), None))
        r.snps, r.cases, r.ctrls = int(d.snps), int(d.cases), int(d.ctrls)
        return r

    @property
    def one_hot(self) -> bool:
        return bool(self.ctx.lib.fiu_dataset_is_one_hot(self.h))

    def free(self):
        if getattr(self, "h", None):
            self.ctx.lib.fiu_dataset_free(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _results(order, n, comb, vals):
    comb = comb[: n * order].reshape(n, order)
    return [Result(comb[i].tolist(), float(vals[i])) for i in range(n)]


class GpuSearch:
    """``Search`` implementation on one GB300 (the drop-in for ThreadedSearch).

    ``run(dataset, order, distribution, outputs)`` returns at most ``outputs``
    ``Result``s sorted by MI descending (ties: ascending combination)."""

    def __init__(self, device: int = 0, kernel: int = 0):
        self.ctx = Context(device)
        if kernel:
            self.set_kernel(kernel)

    def set_kernel(self, kernel: int):
        """Forces a counting kernel (fiuncho_gb300._lib.KERNEL_*); 0 = automatic."""
        self.ctx.check(self.ctx.lib.fiu_set_kernel(self.ctx.h, int(kernel)))

    def run(self, dataset, order: int, distribution: Distribution, outputs: int, with_fp64: bool = False):
        lib, ctx = self.ctx.lib, self.ctx
        outputs = int(outputs)
        comb = np.zeros(max(outputs, 1) * order, np.int32)
        vals = np.zeros(max(outputs, 1), np.float32)
        v64 = np.zeros(max(outputs, 1), np.float64)
        n = C.c_uint(0)
        dist = distribution.c_struct()
        if isinstance(dataset, Resident):
            ctx.check(lib.fiu_search_resident64(ctx.h, dataset.h, order, C.byref(dist), outputs,
                                                _lib.ptr(comb, C.c_int32), _lib.ptr(vals, C.c_float),
                                                _lib.ptr(v64, C.c_double), C.byref(n)))
        else:
            if with_fp64:
                res = Resident(ctx, dataset)
                try:
                    return self.run(res, order, distribution, outputs, with_fp64=True)
                finally:
                    res.free()
            cds, keep = _c_dataset(dataset)
            ctx.check(lib.fiu_search(ctx.h, C.byref(cds), order, C.byref(dist), outputs, _lib.ptr(comb, C.c_int32),
                                     _lib.ptr(vals, C.c_float), C.byref(n)))
        out = _results(order, n.value, comb, vals)
        if with_fp64:
            return out, v64[: n.value].copy()
        return out

    def run_shard(self, dataset, order: int, shard: int, n_shards: int, outputs: int, with_fp64: bool = False):
        """Shard ``shard`` of ``n_shards`` of the whole search (fiu_search_shard): equal
        ranges of the serving kernel's work units, so every shard keeps the
        whole-data-set kernels.  Merging all shards' results by (MI descending,
        combination ascending) gives the whole search's result."""
        lib, ctx = self.ctx.lib, self.ctx
        outputs = int(outputs)
        comb = np.zeros(max(outputs, 1) * order, np.int32)
        vals = np.zeros(max(outputs, 1), np.float32)
        v64 = np.zeros(max(outputs, 1), np.float64)
        n = C.c_uint(0)
        if isinstance(dataset, Resident):
            ctx.check(lib.fiu_search_shard_resident64(ctx.h, dataset.h, order, int(shard), int(n_shards), outputs,
                                                      _lib.ptr(comb, C.c_int32), _lib.ptr(vals, C.c_float),
                                                      _lib.ptr(v64, C.c_double), C.byref(n)))
        else:
            if with_fp64:
                res = Resident(ctx, dataset)
                try:
                    return self.run_shard(res, order, shard, n_shards, outputs, with_fp64=True)
                finally:
                    res.free()
            cds, keep = _c_dataset(dataset)
            ctx.check(lib.fiu_search_shard(ctx.h, C.byref(cds), order, int(shard), int(n_shards), outputs,
                                           _lib.ptr(comb, C.c_int32), _lib.ptr(vals, C.c_float), C.byref(n)))
        out = _results(order, n.value, comb, vals)
        if with_fp64:
            return out, v64[: n.value].copy()
        return out

    def run_batch(self, requests, use_graph: bool = True):
        """Many scans at once: requests = [(Resident, order, Distribution, outputs), ...], or
        (Resident, order, Distribution, outputs, shard, n_shards) for one shard of a whole
        scan (as run_shard).  Returns [(results, fp64 values)] in request order; raises if
        any scan failed."""
        lib, ctx = self.ctx.lib, self.ctx
        arr = (_lib.Scan_t * len(requests))()
        bufs = []
        for i, req in enumerate(requests):
            res, order, dist, outputs = req[:4]
            shard, n_shards = (req[4], req[5]) if len(req) > 4 else (0, 1)
            comb = np.zeros(max(outputs, 1) * order, np.int32)
            vals = np.zeros(max(outputs, 1), np.float32)
            v64 = np.zeros(max(outputs, 1), np.float64)
            bufs.append((comb, vals, v64))
            arr[i] = _lib.Scan_t(res.h, order, dist.c_struct(), outputs, _lib.ptr(comb, C.c_int32),
                                 _lib.ptr(vals, C.c_float), _lib.ptr(v64, C.c_double), 0, 0, shard, n_shards)
        ctx.check(lib.fiu_search_batch(ctx.h, arr, len(requests), 1 if use_graph else 0))
        out = []
        for i, (res, order, dist, outputs, *_) in enumerate(requests):
            if arr[i].status:
                raise FiunchoError(arr[i].status, "scan %d: %s" % (i, lib.fiu_last_error(ctx.h).decode()))
            n = arr[i].out_count
            comb, vals, v64 = bufs[i]
            out.append((_results(order, n, comb, vals), v64[:n].copy()))
        return out

    # kernel-level entries ----------------------------------------------------
    def tables(self, resident: Resident, order: int, combos):
        combos = np.ascontiguousarray(combos, np.int32).reshape(-1, order)
        q, cells = combos.shape[0], 3 ** order
        cc = np.zeros((q, cells), np.uint32)
        tt = np.zeros((q, cells), np.uint32)
        self.ctx.check(self.ctx.lib.fiu_tables(self.ctx.h, resident.h, order, _lib.ptr(combos, C.c_int32), q,
                                               _lib.ptr(cc, C.c_uint32), _lib.ptr(tt, C.c_uint32)))
        return cc, tt

    def set_autotune(self, enable: bool):
        self.ctx.check(self.ctx.lib.fiu_set_autotune(self.ctx.h, 1 if enable else 0))

    def last_tile(self):
        k, t = C.c_int(0), C.c_int(0)
        self.ctx.check(self.ctx.lib.fiu_last_tile(self.ctx.h, C.byref(k), C.byref(t)))
        return k.value, t.value

    def scan_tables(self, resident: Resident, order: int, distribution: Distribution, kernel: int = 0, tp: int = 0):
        import math
        total = math.comb(distribution.n, distribution.k)
        owned = (total - 1 - distribution.offset) // distribution.step + 1 if distribution.offset < total else 0
        cells = 3 ** order
        out = np.full(owned * resident.snps * 2 * cells, 0xFFFFFFFF, np.uint32)
        dist = distribution.c_struct()
        self.ctx.check(self.ctx.lib.fiu_scan_tables(self.ctx.h, resident.h, order, C.byref(dist), kernel + 256 * tp,
                                                    _lib.ptr(out, C.c_uint32), out.size))
        return out.reshape(owned, resident.snps, 2, cells)

    def scan_digest(self, resident: Resident, order: int, distribution: Distribution = None, kernel: int = 0):
        """Digest of every table of a scan as `kernel` computes them (fiu_scan_digest):
        (digest, combinations)."""
        dg, cnt = C.c_uint64(0), C.c_uint64(0)
        dist = distribution.c_struct() if distribution is not None else None
        self.ctx.check(self.ctx.lib.fiu_scan_digest(self.ctx.h, resident.h, order,
                                                    C.byref(dist) if dist is not None else None, kernel,
                                                    C.byref(dg), C.byref(cnt)))
        return int(dg.value), int(cnt.value)

    def combine(self, t1, size1, t2, cases_words, ctrls_words):
        t1 = np.ascontiguousarray(t1, np.uint64)
        t2 = np.ascontiguousarray(t2, np.uint64)
        out = np.zeros(3 * size1 * (cases_words + ctrls_words), np.uint64)
        self.ctx.check(self.ctx.lib.fiu_combine(self.ctx.h, _lib.ptr(t1, C.c_uint64), size1,
                                                _lib.ptr(t2, C.c_uint64), cases_words, ctrls_words,
                                                _lib.ptr(out, C.c_uint64)))
        return out

    def combine_and_popcnt(self, t1, size1, t2, cases_words, ctrls_words, ct_size=None):
        ct_size = ct_size or 3 * size1
        t1 = np.ascontiguousarray(t1, np.uint64)
        t2 = np.ascontiguousarray(t2, np.uint64)
        cc = np.zeros(ct_size, np.uint32)
        tt = np.zeros(ct_size, np.uint32)
        self.ctx.check(self.ctx.lib.fiu_combine_and_popcnt(self.ctx.h, _lib.ptr(t1, C.c_uint64), size1,
                                                           _lib.ptr(t2, C.c_uint64), cases_words, ctrls_words,
                                                           _lib.ptr(cc, C.c_uint32), _lib.ptr(tt, C.c_uint32),
                                                           ct_size))
        return cc, tt

    def mi(self, cases, ctrls, n_cases, n_ctrls, mode=0):
        cases = np.ascontiguousarray(cases, np.uint32)
        ctrls = np.ascontiguousarray(ctrls, np.uint32)
        if cases.ndim == 1:
            cases, ctrls = cases[None], ctrls[None]
        count, cells = cases.shape
        out = np.zeros(count, np.float32)
        o64 = np.zeros(count, np.float64)
        self.ctx.check(self.ctx.lib.fiu_mi_compute(self.ctx.h, _lib.ptr(cases, C.c_uint32),
                                                   _lib.ptr(ctrls, C.c_uint32), cells, count, n_cases, n_ctrls,
                                                   mode, _lib.ptr(out, C.c_float), _lib.ptr(o64, C.c_double)))
        return out, o64


class Server:
    """Served request stream (fiu_server_*): submit whole-data-set scans at
    any time; they are admitted against a device-memory budget and run with
    continuous batching.  ``result`` returns (results, fp64 values, latency ms)."""

    FIFO, SHORTEST_FIRST = 0, 1  # admission / solo-lane order (fiu_server_set_policy)

    def __init__(self, device: int = 0, budget_bytes: int = 0, policy: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.fiu_server_create(int(device), int(budget_bytes), C.byref(h))
        if rc:
            raise FiunchoError(rc, "cannot create a server on CUDA device %d" % device)
        self.h = h
        if policy:
            rc = self.lib.fiu_server_set_policy(self.h, int(policy))
            if rc:
                self.close()  # destroys the server once and drops the handle
                raise FiunchoError(rc, "unknown serving policy %d" % policy)
        self._orders = {}
        self._keep = {}

    def submit(self, ds: Dataset, order: int, outputs: int, shard: int = 0, n_shards: int = 1) -> int:
        """Queues a whole-data-set scan, or shard `shard` of `n_shards` of it."""
        cds, data = _c_dataset(ds)
        t = C.c_uint64(0)
        rc = self.lib.fiu_server_submit_shard(self.h, C.byref(cds), int(order), int(outputs), int(shard),
                                              int(n_shards), C.byref(t))
        if rc:
            raise FiunchoError(rc, "submit rejected")
        self._orders[t.value] = (order, outputs)
        return t.value

    def result(self, ticket: int, timeout_ms: int = -1):
        order, outputs = self._orders[ticket]
        comb = np.zeros(max(outputs, 1) * order, np.int32)
        vals = np.zeros(max(outputs, 1), np.float32)
        v64 = np.zeros(max(outputs, 1), np.float64)
        n = C.c_uint(0)
        lat = C.c_double(0)
        rc = self.lib.fiu_server_poll(self.h, ticket, int(timeout_ms), _lib.ptr(comb, C.c_int32),
                                      _lib.ptr(vals, C.c_float), _lib.ptr(v64, C.c_double), C.byref(n), C.byref(lat))
        if rc == _lib.FIU_ERR_TIMEOUT:
            return None
        del self._orders[ticket]
        if rc:
            raise FiunchoError(rc, "scan %d failed" % ticket)
        return _results(order, n.value, comb, vals), v64[: n.value].copy(), lat.value

    def stats(self) -> dict:
        st = _lib.ServerStats_t()
        rc = self.lib.fiu_server_stats(self.h, C.byref(st))
        if rc:
            raise FiunchoError(rc, "stats")
        return {f: getattr(st, f) for f, _ in _lib.ServerStats_t._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.fiu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MPIEngine:
    """``MPIEngine`` (include/fiuncho/MPIEngine.h:27-185) over torch.distributed
    ranks, or one rank when no process group exists."""

    def __init__(self, group=None):
        self.group = group
        try:
            import torch.distributed as dist
            if dist.is_available() and dist.is_initialized():
                self.dist = dist
                self.size = dist.get_world_size(group)
                self.rank = dist.get_rank(group)
                return
        except ImportError:
            pass
        self.dist, self.size, self.rank = None, 1, 0

    def run(self, search_cls, inputs, order: int, outputs: int, *args, dataset=None):
        ds = dataset if dataset is not None else Dataset.read(inputs)
        if ds.snps > 2 ** 31 - 1:
            raise FiunchoError(_lib.FIU_ERR_INVALID, "Input data limit exceeded: more than INT_MAX SNPs")
        search = search_cls(*args)
        if hasattr(search, "run_shard"):
            # the GPU search keeps the whole-data-set kernels: rank r searches
            # shard r of the work units instead of the strided prefix set
            # Distribution(snps, order-1, size, r); the gathered result is the same
            local = search.run_shard(ds, order, self.rank, self.size, outputs)
        else:
            local = search.run(ds, order, Distribution(ds.snps, order - 1, self.size, self.rank), outputs)
        return self.gather(local, outputs)

    def gather(self, local, outputs):
        """Serialised gather to rank 0, then sort (value desc, combination asc)
        and truncate (MPIEngine.h:139-174).  Non-zero ranks return []."""
        blob = b"".join(r.serialize() for r in local)
        if self.dist is None:
            blobs = [blob]
        else:
            blobs = [None] * self.size if self.rank == 0 else None
            # gather_object's dst is a global rank: the group's rank 0 in global numbering
            dst = self.dist.get_global_rank(self.group, 0) if self.group is not None else 0
            self.dist.gather_object(blob, blobs, dst=dst, group=self.group)
            if self.rank != 0:
                return []
        res = []
        for b in blobs:
            pos = 0
            while pos < len(b):
                r, pos = Result.deserialize(b, pos)
                res.append(r)
        res.sort(key=lambda r: (-r.val, r.combination))
        return res[:outputs]
