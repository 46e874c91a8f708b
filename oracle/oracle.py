"""ctypes front end of the CPU checker (test infrastructure only).

``Oracle`` wraps ``oracle/liboracle.so`` (the C restatement in ``oracle.c``);
``Reference`` wraps a library built from the reference's own sources under
``oracle/_ref/`` (present only where the reference tree was available when it
was built).  Only tests/, the smoke check and bench.py's CPU-baseline leg use
this module, and only as the checker.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def cells(order: int) -> int:
    return 3 ** order


class Oracle:
    def __init__(self):
        path = _build.build_oracle()
        L = C.CDLL(path)
        L.orc_pack.argtypes = [_u8p, _u8p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t, _u64p]
        L.orc_combine.argtypes = [_u64p, C.c_size_t, _u64p, C.c_size_t, _u64p]
        L.orc_popcnt.argtypes = [_u64p, C.c_size_t, _u64p, C.c_size_t, _u32p, C.c_size_t]
        L.orc_mi_f32.argtypes = [_u32p, _u32p, C.c_size_t, C.c_uint32, C.c_uint32]
        L.orc_mi_f32.restype = C.c_float
        L.orc_mi_f64.argtypes = [_u32p, _u32p, C.c_size_t, C.c_uint32, C.c_uint32]
        L.orc_mi_f64.restype = C.c_double
        L.orc_distribution_prefixes.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i32p, C.c_long]
        L.orc_distribution_prefixes.restype = C.c_long
        L.orc_search.argtypes = [_u64p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t, C.c_int,
                                 C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint, C.c_int, _i32p, _f32p, _f64p,
                                 C.POINTER(C.c_uint64)]
        L.orc_search.restype = C.c_long
        L.orc_tables.argtypes = [_u64p, C.c_size_t, C.c_size_t, C.c_int, _i32p, C.c_size_t, _u32p, _u32p]
        L.orc_tables.restype = C.c_int
        L.orc_mi_batch.argtypes = [_u32p, _u32p, C.c_size_t, C.c_size_t, C.c_uint32, C.c_uint32, _f32p, _f64p]
        L.orc_table_digest.argtypes = [_u64p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_int, C.c_int, C.c_int,
                                       C.c_int, C.c_int, C.POINTER(C.c_uint64)]
        L.orc_table_digest.restype = C.c_long
        L.orc_search_dfs.argtypes = [_u64p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t, C.c_int,
                                     C.c_size_t, C.c_uint, C.c_int, _i32p, _f32p, _f64p, C.POINTER(C.c_uint64)]
        L.orc_search_dfs.restype = C.c_long
        self.L = L

    # -- data model ---------------------------------------------------------
    def pack(self, geno: np.ndarray, is_case: np.ndarray, cases_words: int, ctrls_words: int) -> np.ndarray:
        geno = np.ascontiguousarray(geno, dtype=np.uint8)
        is_case = np.ascontiguousarray(is_case, dtype=np.uint8)
        snps, samples = geno.shape
        out = np.zeros(snps * 3 * (cases_words + ctrls_words), dtype=np.uint64)
        self.L.orc_pack(geno, is_case, snps, samples, cases_words, ctrls_words, out)
        return out

    def combine(self, t1, size1, t2, words):
        out = np.zeros(size1 * 3 * words, dtype=np.uint64)
        self.L.orc_combine(np.ascontiguousarray(t1, np.uint64), size1, np.ascontiguousarray(t2, np.uint64), words,
                           out)
        return out

    def popcnt(self, t1, size1, t2, words, ct_size=None):
        ct_size = ct_size or size1 * 3
        out = np.zeros(ct_size, dtype=np.uint32)
        self.L.orc_popcnt(np.ascontiguousarray(t1, np.uint64), size1, np.ascontiguousarray(t2, np.uint64), words,
                          out, ct_size)
        return out

    def mi(self, cases, ctrls, n_cases, n_ctrls):
        cases = np.ascontiguousarray(cases, np.uint32)
        ctrls = np.ascontiguousarray(ctrls, np.uint32)
        return (float(self.L.orc_mi_f32(cases, ctrls, cases.size, n_cases, n_ctrls)),
                float(self.L.orc_mi_f64(cases, ctrls, cases.size, n_cases, n_ctrls)))

    def mi_batch(self, cases, ctrls, n_cases, n_ctrls):
        cases = np.ascontiguousarray(cases, np.uint32)
        ctrls = np.ascontiguousarray(ctrls, np.uint32)
        count, size = cases.shape
        o32 = np.zeros(count, np.float32)
        o64 = np.zeros(count, np.float64)
        self.L.orc_mi_batch(cases, ctrls, size, count, n_cases, n_ctrls, o32, o64)
        return o32, o64

    def prefixes(self, n, k, step, offset):
        cnt = self.L.orc_distribution_prefixes(n, k, step, offset, np.zeros(1, np.int32), 0)
        out = np.zeros(max(cnt, 1) * k, np.int32)
        self.L.orc_distribution_prefixes(n, k, step, offset, out, cnt)
        return out[: cnt * k].reshape(cnt, k)

    def tables(self, data, cases_words, ctrls_words, order, combos):
        combos = np.ascontiguousarray(combos, np.int32).reshape(-1, order)
        q = combos.shape[0]
        cc = np.zeros((q, cells(order)), np.uint32)
        tt = np.zeros((q, cells(order)), np.uint32)
        rc = self.L.orc_tables(np.ascontiguousarray(data, np.uint64), cases_words, ctrls_words, order, combos, q,
                               cc, tt)
        assert rc == 0
        return cc, tt

    def search(self, data, snps, n_cases, n_ctrls, cases_words, ctrls_words, order, outputs, threads=1,
               mi_mode=1, dist=None):
        """Returns (combos[n, order] int32, vals float32, vals64 float64, combos evaluated)."""
        n, step, offset = dist if dist is not None else (snps, 1, 0)
        combos = np.zeros(max(outputs, 1) * order, np.int32)
        v32 = np.zeros(max(outputs, 1), np.float32)
        v64 = np.zeros(max(outputs, 1), np.float64)
        done = C.c_uint64(0)
        r = self.L.orc_search(np.ascontiguousarray(data, np.uint64), snps, n_cases, n_ctrls, cases_words,
                              ctrls_words, order, n, step, offset, threads, outputs, mi_mode, combos, v32, v64,
                              C.byref(done))
        if r < 0:
            raise ValueError("oracle search: invalid arguments")
        return combos[: r * order].reshape(r, order), v32[:r], v64[:r], int(done.value)


    def search_dfs(self, data, snps, n_cases, n_ctrls, cases_words, ctrls_words, order, outputs, block=1,
                   mi_mode=1):
        """The benchmark programs' depth-first traversal (block tables per MI batch; 1 = non-segmented).
        Returns (combos[n, order] int32, vals float32, vals64 float64, combos evaluated)."""
        combos = np.zeros(max(outputs, 1) * order, np.int32)
        v32 = np.zeros(max(outputs, 1), np.float32)
        v64 = np.zeros(max(outputs, 1), np.float64)
        done = C.c_uint64(0)
        r = self.L.orc_search_dfs(np.ascontiguousarray(data, np.uint64), snps, n_cases, n_ctrls, cases_words,
                                  ctrls_words, order, block, outputs, mi_mode, combos, v32, v64, C.byref(done))
        if r < 0:
            raise ValueError("oracle depth-first search: invalid arguments")
        return combos[: r * order].reshape(r, order), v32[:r], v64[:r], int(done.value)

    def table_digest(self, data, snps, cases_words, ctrls_words, order, threads=1, dist=None):
        """Digest (oracle/ref/tabledigest.h) of every table of a scan: (digest, combinations)."""
        n, step, offset = dist if dist is not None else (snps, 1, 0)
        out = C.c_uint64(0)
        r = self.L.orc_table_digest(np.ascontiguousarray(data, np.uint64), snps, cases_words, ctrls_words, order, n,
                                    step, offset, threads, C.byref(out))
        if r < 0:
            raise ValueError("oracle digest: invalid arguments")
        return int(out.value), int(r)


class Reference:
    """The reference's own code (built from its sources by oracle/build.py)."""

    def __init__(self, flavour: str = "base"):
        built = _build.build_ref()
        if flavour not in built:
            raise FileNotFoundError("reference build '%s' not available" % flavour)
        L = C.CDLL(built[flavour])
        L.ref_last_error.restype = C.c_char_p
        L.ref_align.restype = C.c_int
        L.ref_read.argtypes = [C.c_char_p, C.c_char_p]
        L.ref_read.restype = C.c_void_p
        L.ref_from_packed.argtypes = [_u64p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t]
        L.ref_from_packed.restype = C.c_void_p
        L.ref_free.argtypes = [C.c_void_p]
        L.ref_info.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(np.uintp, flags="C_CONTIGUOUS")]
        L.ref_packed.argtypes = [C.c_void_p, _u64p]
        L.ref_search.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint, _i32p, _f32p]
        L.ref_search.restype = C.c_long
        L.ref_engine.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_uint, _i32p, _f32p]
        L.ref_engine.restype = C.c_long
        L.ref_tables.argtypes = [C.c_void_p, C.c_int, _i32p, C.c_size_t, _u32p, _u32p, _f32p]
        L.ref_tables.restype = C.c_int
        L.ref_mi.argtypes = [C.c_int, _u32p, _u32p, C.c_size_t, C.c_uint, C.c_uint, _f32p]
        L.ref_mi.restype = C.c_int
        L.ref_table_digest.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_uint64),
                                       C.POINTER(C.c_uint64)]
        L.ref_table_digest.restype = C.c_int
        self.L = L
        self.flavour = flavour
        self.align = L.ref_align()

    def read(self, f1, f2=None):
        h = self.L.ref_read(f1.encode(), (f2 or "").encode())
        if not h:
            raise RuntimeError(self.L.ref_last_error().decode())
        return RefDataset(self, h)

    def from_packed(self, data, snps, cases, ctrls, cw, tw):
        h = self.L.ref_from_packed(np.ascontiguousarray(data, np.uint64), snps, cases, ctrls, cw, tw)
        return RefDataset(self, h)

    def engine(self, f1, f2, order, threads, outputs):
        combos = np.zeros(max(outputs, 1) * order, np.int32)
        vals = np.zeros(max(outputs, 1), np.float32)
        r = self.L.ref_engine(f1.encode(), (f2 or "").encode(), order, threads, outputs, combos, vals)
        if r < 0:
            raise RuntimeError(self.L.ref_last_error().decode())
        return combos[: r * order].reshape(r, order), vals[:r]

    def mi(self, order, cases, ctrls, n_cases, n_ctrls):
        cases = np.ascontiguousarray(cases, np.uint32).reshape(-1, cells(order))
        ctrls = np.ascontiguousarray(ctrls, np.uint32).reshape(-1, cells(order))
        out = np.zeros(cases.shape[0], np.float32)
        self.L.ref_mi(order, cases, ctrls, cases.shape[0], n_cases, n_ctrls, out)
        return out


class RefDataset:
    def __init__(self, ref: Reference, handle):
        self.ref, self.h = ref, handle
        info = np.zeros(5, np.uintp)
        ref.L.ref_info(handle, info)
        self.snps, self.cases, self.ctrls, self.cases_words, self.ctrls_words = (int(x) for x in info)

    def __del__(self):
        try:
            self.ref.L.ref_free(self.h)
        except Exception:
            pass

    def packed(self):
        out = np.zeros(self.snps * 3 * (self.cases_words + self.ctrls_words), np.uint64)
        self.ref.L.ref_packed(self.h, out)
        return out

    def search(self, order, outputs, threads=1, step=1, offset=0):
        combos = np.zeros(max(outputs, 1) * order, np.int32)
        vals = np.zeros(max(outputs, 1), np.float32)
        r = self.ref.L.ref_search(self.h, order, threads, step, offset, outputs, combos, vals)
        if r < 0:
            raise RuntimeError(self.ref.L.ref_last_error().decode())
        return combos[: r * order].reshape(r, order), vals[:r]

    def table_digest(self, order, threads=1, step=1, offset=0):
        """Digest (oracle/ref/tabledigest.h) of the reference's tables of every
        combination of Distribution(snps, order-1, step, offset): (digest, combinations)."""
        dg, cnt = C.c_uint64(0), C.c_uint64(0)
        if self.ref.L.ref_table_digest(self.h, order, threads, step, offset, C.byref(dg), C.byref(cnt)) != 0:
            raise RuntimeError(self.ref.L.ref_last_error().decode())
        return int(dg.value), int(cnt.value)

    def tables(self, order, combos):
        combos = np.ascontiguousarray(combos, np.int32).reshape(-1, order)
        q = combos.shape[0]
        cc = np.zeros((q, cells(order)), np.uint32)
        tt = np.zeros((q, cells(order)), np.uint32)
        mi = np.zeros(q, np.float32)
        self.ref.L.ref_tables(self.h, order, combos, q, cc, tt, mi)
        return cc, tt, mi


class ReferenceBench:
    """The reference's sequential benchmark programs' depth-first traversal
    (oracle/ref/bench_driver.cpp, built from their sources by oracle/build.py)."""

    def __init__(self):
        built = _build.build_ref()
        if "bench" not in built:
            raise FileNotFoundError("reference benchmark build not available")
        L = C.CDLL(built["bench"])
        L.ref_stack_search.argtypes = [_u64p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t, C.c_int,
                                       C.c_int, C.c_uint, _i32p, _f32p]
        L.ref_stack_search.restype = C.c_long
        self.L = L

    def stack_search(self, data, snps, cases, ctrls, cw, tw, order, outputs, segmented):
        """stack_search of the segmented or non-segmented program: (combos[n, order], vals float32),
        by descending value."""
        combos = np.zeros(max(outputs, 1) * order, np.int32)
        vals = np.zeros(max(outputs, 1), np.float32)
        r = self.L.ref_stack_search(np.ascontiguousarray(data, np.uint64), snps, cases, ctrls, cw, tw, order,
                                    int(bool(segmented)), outputs, combos, vals)
        if r < 0:
            raise RuntimeError("reference stack_search failed")
        return combos[: r * order].reshape(r, order), vals[:r]
