"""Fast data set ingest through the library: multi-threaded parsing of
.tped/.tfam or .raw files into genotype codes (``read_genotypes``) and
packing of the codes on the device (``upload_genotypes``), the GPU
counterparts of ``Dataset.read`` (include/fiuncho/Dataset.h:48-94) and its
host packer.  Parsing runs on the host cores and needs no GPU."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import FiunchoError


def read_genotypes(inputs, threads: int = 0, ctx=None):
    """(geno uint8 [snps, samples], is_case bool [samples]) of one .raw file or
    a .tped + .tfam pair (either order), parsed by `threads` host threads
    (0 = all cores).  Raises FiunchoError with the reader's message."""
    lib = _lib.load()
    inputs = list(inputs)
    if len(inputs) not in (1, 2):
        raise ValueError("Unrecognized number of input files to Dataset factory constructor")
    f1 = inputs[0].encode()
    f2 = inputs[1].encode() if len(inputs) == 2 else None
    h = C.c_void_p()
    cx = ctx.h if ctx is not None else None
    rc = lib.fiu_read_genotypes(cx, f1, f2, int(threads), C.byref(h))
    if rc:
        msg = lib.fiu_last_error(cx).decode()
        raise FiunchoError(rc, msg)
    try:
        snps, samples = C.c_uint64(0), C.c_uint64(0)
        codes, cases = C.POINTER(C.c_uint8)(), C.POINTER(C.c_uint8)()
        lib.fiu_genotypes_info(h, C.byref(snps), C.byref(samples), C.byref(codes), C.byref(cases))
        n, m = int(snps.value), int(samples.value)
        geno = np.ctypeslib.as_array(codes, shape=(n * m,)).copy().reshape(n, m) if n * m else \
            np.zeros((n, m), np.uint8)
        is_case = np.ctypeslib.as_array(cases, shape=(m,)).astype(bool) if m else np.zeros(0, bool)
    finally:
        lib.fiu_genotypes_free(h)
    return geno, is_case


def upload_genotypes(ctx, geno, is_case):
    """A Resident data set whose packed layout is built on the device from the codes."""
    from .search import Resident
    geno = np.ascontiguousarray(geno, np.uint8)
    flags = np.ascontiguousarray(np.asarray(is_case, bool).astype(np.uint8))
    snps, samples = geno.shape
    h = C.c_void_p()
    ctx.check(ctx.lib.fiu_dataset_upload_genotypes(ctx.h, _lib.ptr(geno, C.c_uint8), _lib.ptr(flags, C.c_uint8),
                                                   snps, samples, C.byref(h)))
    return Resident.adopt(ctx, h)


def packed(ctx, resident):
    """(packed words uint64, (snps, cases, ctrls, cases_words, ctrls_words)) of a resident data set."""
    d = _lib.Dataset_t()
    ctx.check(ctx.lib.fiu_dataset_packed(ctx.h, resident.h, C.byref(d), None))
    out = np.zeros(d.snps * 3 * (d.cases_words + d.ctrls_words), np.uint64)
    ctx.check(ctx.lib.fiu_dataset_packed(ctx.h, resident.h, None, _lib.ptr(out, C.c_uint64)))
    return out, (d.snps, d.cases, d.ctrls, d.cases_words, d.ctrls_words)
