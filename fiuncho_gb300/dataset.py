"""Host-side data model: the Python mirror of Fiuncho's ``Dataset<uint64_t>`` /
``GenotypeTable<uint64_t>`` (include/fiuncho/Dataset.h:26-152,
include/fiuncho/GenotypeTable.h:36-206) and of its two input readers.

Packed layout (identical to ``GenotypeTable::make_array``,
GenotypeTable.h:77-103): SNP-major; per SNP three case rows of
``cases_words`` uint64 followed by three control rows of ``ctrls_words``;
row g has bit set for every sample whose minor-allele count is g.  Within a
class, samples are shifted in most-significant-bit first, so the first sample
of a full word is bit 63, and the last, partial word of a row is
right-aligned (TPEDFile.hpp:205-254); words past the data are zero.

Row padding: with ``align`` = A bytes (the reference's ``ALIGN`` macro) a row
holds ceil(n / (8A)) * (A/8) words, otherwise ceil(n / 64)
(TPEDFile.hpp:282-292, RAWFile.hpp:299-309).
"""
from __future__ import annotations

import os
import re

import numpy as np


def words_for(n: int, align: int = 0) -> int:
    if align:
        nt, nbits = align // 8, align * 8
        return (n + nbits - 1) // nbits * nt
    return (n + 63) // 64


def pack_rows(geno: np.ndarray, is_case: np.ndarray, cases_words: int, ctrls_words: int) -> np.ndarray:
    """Pack minor-allele counts geno[snps, samples] into the reference layout."""
    geno = np.asarray(geno, dtype=np.uint8)
    is_case = np.asarray(is_case).astype(bool)
    snps = geno.shape[0]
    out = np.zeros((snps, 3 * (cases_words + ctrls_words)), dtype=np.uint64)
    for cls, (sel, words, off) in enumerate(((is_case, cases_words, 0), (~is_case, ctrls_words, 3 * cases_words))):
        g = geno[:, sel]
        n = g.shape[1]
        if n == 0:
            continue
        nfull, m = divmod(n, 64)
        nw = nfull + (1 if m else 0)
        if nw > words:
            raise ValueError("row of %d samples does not fit %d words" % (n, words))
        for k in range(3):
            bits = (g == k)
            if m:
                # right-align the last, partial word: its last sample lands in bit 0
                pad = np.zeros((snps, 64 - m), dtype=bool)
                bits = np.concatenate([bits[:, : nfull * 64], pad, bits[:, nfull * 64:]], axis=1)
            by = np.ascontiguousarray(np.packbits(bits, axis=1, bitorder="big"))
            w = by.reshape(snps, nw, 8).view(">u8").reshape(snps, nw).astype(np.uint64)
            out[:, off + k * words: off + k * words + nw] = w
    return out.reshape(-1)


class GenotypeTable:
    """View of one SNP (order 1) or a combined table: ``cases``/``ctrls`` are
    [3^order, words] uint64 arrays (GenotypeTable.h:36-206)."""

    def __init__(self, order, cases, ctrls):
        self.order = order
        self.size = 3 ** order
        self.cases = cases
        self.ctrls = ctrls
        self.cases_words = cases.shape[1]
        self.ctrls_words = ctrls.shape[1]


class Dataset:
    """``Dataset<uint64_t>``: ``snps`` single-SNP GenotypeTables over
    ``cases`` + ``ctrls`` individuals, stored contiguously (Dataset.h:26-152)."""

    def __init__(self, cases: int, ctrls: int, snps: int, cases_words: int, ctrls_words: int, data: np.ndarray):
        self.cases, self.ctrls, self.snps = int(cases), int(ctrls), int(snps)
        self.cases_words, self.ctrls_words = int(cases_words), int(ctrls_words)
        self.data = np.ascontiguousarray(data, dtype=np.uint64).reshape(-1)
        if self.data.size != self.snps * 3 * (self.cases_words + self.ctrls_words):
            raise ValueError("packed data size does not match snps x 3 x (cases_words + ctrls_words)")

    def __getitem__(self, i: int) -> GenotypeTable:
        per = 3 * (self.cases_words + self.ctrls_words)
        blk = self.data[i * per:(i + 1) * per]
        return GenotypeTable(1, blk[: 3 * self.cases_words].reshape(3, self.cases_words),
                             blk[3 * self.cases_words:].reshape(3, self.ctrls_words))

    @classmethod
    def from_genotypes(cls, geno, is_case, align: int = 0) -> "Dataset":
        is_case = np.asarray(is_case).astype(bool)
        cases = int(is_case.sum())
        ctrls = int(is_case.size - cases)
        cw, tw = words_for(cases, align), words_for(ctrls, align)
        return cls(cases, ctrls, geno.shape[0], cw, tw, pack_rows(geno, is_case, cw, tw))

    @classmethod
    def read(cls, inputs, align: int = 0) -> "Dataset":
        """Factory with the reference's dispatch rules (Dataset.h:48-94): one
        ``.raw`` file, or a ``.tped`` + ``.tfam`` pair in either order."""
        geno, is_case = read_genotypes(inputs)
        return cls.from_genotypes(geno, is_case, align)


# --------------------------------------------------------------------------
# Readers.  They return (geno uint8 [snps, samples], is_case bool [samples]).

def read_genotypes(inputs):
    inputs = list(inputs)
    if len(inputs) == 1:
        ext = os.path.splitext(inputs[0])[1]
        if ext == ".raw":
            return read_raw(inputs[0])
        raise ValueError("Unrecognized input file extension " + ext)
    if len(inputs) == 2:
        e1, e2 = (os.path.splitext(f)[1] for f in inputs)
        if e1 in (".tped", ".tfam"):
            if e1 == e2 or e2 not in (".tped", ".tfam"):
                raise ValueError('Expecting a tfam file after "%s", but found a %s' % (inputs[0], e2))
            tped, tfam = inputs if e1 == ".tped" else inputs[::-1]
            return read_tped(tped, tfam)
        raise ValueError("Unrecognized input file extension " + e1)
    raise ValueError("Unrecognized number of input files to Dataset factory constructor")


def read_tfam(path):
    """Phenotype column 6: 1 = control, 2 = case; anything else is an error
    (TPEDFile.hpp:72-143)."""
    ph = []
    with open(path) as f:
        for ln, line in enumerate(f, 1):
            t = line.split()
            if not t:
                continue
            if len(t) < 6 or t[5] not in ("1", "2"):
                raise ValueError("Error in %s:%d: parsing error" % (path, ln))
            ph.append(t[5] == "2")
    return np.array(ph, dtype=bool)


def read_tped(tped, tfam):
    """Nucleotides must be A/C/G/T; the minor allele is the rarer of the two
    lexicographically smallest nucleotides, ties going to the smaller one
    (TPEDFile.hpp:185-194); genotype = copies of the minor allele."""
    is_case = read_tfam(tfam)
    n = is_case.size
    rows = []
    with open(tped) as f:
        for ln, line in enumerate(f, 1):
            t = line.split()
            if not t:
                continue
            if len(t) < 4:
                raise ValueError("Error in %s:%d: invalid loci information" % (tped, ln))
            al = np.frombuffer("".join(t[4:]).encode(), dtype=np.uint8)
            if al.size != sum(len(x) for x in t[4:]) or np.any(~np.isin(al, np.frombuffer(b"ACGT", np.uint8))):
                raise ValueError("Error in %s:%d: invalid nucleotide value" % (tped, ln))
            if al.size % 2:
                raise ValueError("Error in %s:%d: odd number of nucleotides" % (tped, ln))
            if al.size != 2 * n:
                raise ValueError("Error in %s:%d: the number of nucleotides does not match the number of samples"
                                 % (tped, ln))
            present = sorted(set(al.tolist()))
            if len(present) >= 2:
                a1, a2 = present[0], present[1]
                c1, c2 = int((al == a1).sum()), int((al == a2).sum())
                minor = a2 if c1 > c2 else a1
            else:
                minor = -1  # monomorphic: no minor allele, every genotype is 0
            m = (al == minor).astype(np.uint8)
            rows.append(m[0::2] + m[1::2])
    return np.array(rows, dtype=np.uint8).reshape(len(rows), n), is_case


_WORD = re.compile(r"(\w+)")
_GENO_COL = re.compile(r"(\w+_[ACGT])|([A-Za-z0-9]+)")


def read_raw(path):
    """PLINK .raw (FID IID PAT MAT SEX PHENOTYPE <snp>_<allele> [<snp>_HET] ...)
    or GAMETES .raw (<snp> ... Class); PHENOTYPE is 1/2, Class is 0/1
    (RAWFile.hpp:18-207).  Only columns named <id>_<A|C|G|T> or plain
    alphanumeric ids are genotypes."""
    with open(path) as f:
        header = _WORD.findall(f.readline())
        i = 0
        while i < len(header) and i < 5 and header[i] in ("FID", "IID", "PAT", "MAT", "SEX"):
            i += 1
        has_info = i == 5
        cols = header[5:] if has_info else header
        ph_idx = [j for j, w in enumerate(cols) if w in ("PHENOTYPE", "Class")]
        if len(ph_idx) > 1:
            raise ValueError('Error while parsing "%s", multiple phenotype columns found' % path)
        if not ph_idx:
            raise ValueError('Error while parsing "%s", no phenotype column' % path)
        ph_idx = ph_idx[0]
        keep = np.array([j != ph_idx and _GENO_COL.fullmatch(w) is not None for j, w in enumerate(cols)])
        body = f.read().split()
    ncol = len(cols) + (5 if has_info else 0)
    if ncol == 0 or len(body) % ncol:
        raise ValueError('Error while parsing "%s": ragged rows' % path)
    tab = np.array(body, dtype=object).reshape(-1, ncol)[:, 5 if has_info else 0:]
    try:
        vals = tab.astype(np.int64)
    except ValueError:
        raise ValueError('Error while parsing "%s": non-numeric field' % path)
    ph = vals[:, ph_idx] + (0 if has_info else 1)
    geno = vals[:, keep].T.astype(np.uint8)
    return np.ascontiguousarray(geno), ph != 1
