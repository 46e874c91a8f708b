"""Seeded synthetic case/control genotype data with the shapes of the scans
this library is measured on.

Genotypes are minor-allele counts in {0, 1, 2} drawn under Hardy-Weinberg
equilibrium from a per-SNP minor-allele frequency (MAF) p:
P(0) = (1-p)^2, P(1) = 2p(1-p), P(2) = p^2.  A planted interaction raises the
case probability of individuals that satisfy it; the cohort is then balanced by
case/control sampling (individuals are drawn until each class quota is
filled), and samples are written cases first, then controls.

Named workloads (``WORKLOADS``):

* ``order2_1000x4000``   -- 1 000 SNPs, 2 000 cases / 2 000 controls, order 2,
  MAF ~ U(0.05, 0.5); one planted pair: carrying >= 1 minor allele at both
  sites gives case probability 0.7 (else 0.5).  Top-10.
* ``order3_2000x8000``   -- 2 000 SNPs, 4 000 / 4 000, order 3, MAF ~ U(0.05,
  0.5); one planted triple: all three carry a minor allele -> 0.65.  Top-100.
* ``order2_40000x16000`` -- 40 000 SNPs, 8 000 / 8 000, order 2, MAF ~
  Beta(0.5, 0.5) truncated to [0.01, 0.5] by rejection; five planted pairs
  with penetrance 0.6.  Top-1 000.
* ``order4_300x8000``   -- 300 SNPs, 4 000 / 4 000, order 4, MAF ~ U(0.05,
  0.5); one planted quadruple: all four carry a minor allele -> 0.7.  Top-100.
* ``order3_500x18800`` / ``order4_100x18800`` -- 500 (100) SNPs, 9 000 cases /
  9 800 controls (the class sizes of the reference's test data set), order 3
  (4), MAF ~ U(0.05, 0.5), one planted triple (quadruple) with penetrance 0.65
  (0.7).  Top-100 (top-50).  Classes this large do not share one FP32
  accumulator, so these exercise the per-class tensor kernels.
* ``batch_specs()``      -- 64 independent scans, seeds 1000+i: SNPs
  log-uniform in [500, 20 000], samples log-uniform in [1 000, 32 000], case
  fraction U(0.3, 0.7), order uniform in {2, 3, 4} (order-4 scans capped at
  400 SNPs), MAF ~ U(0.05, 0.5).  Top-50 each.  ``BATCH_BENCH`` scales the
  SNP counts down for the benchmark.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class ScanSpec:
    snps: int
    cases: int
    ctrls: int
    order: int
    outputs: int
    seed: int
    maf: str = "uniform"          # "uniform" (U(0.05,0.5)) or "beta" (Beta(.5,.5) in [0.01,0.5])
    planted: tuple = ()           # tuples of SNP counts per planted interaction, e.g. ((2,),) -> 1 pair
    rule: str = "any_minor"       # planted condition: every SNP carries >= 1 minor allele
    penetrance: float = 0.5

    @property
    def samples(self) -> int:
        return self.cases + self.ctrls

    def combos(self) -> int:
        return math.comb(self.snps, self.order)


WORKLOADS = {
    "order2_1000x4000": ScanSpec(1000, 2000, 2000, 2, 10, seed=1, planted=(2,), penetrance=0.7),
    "order3_2000x8000": ScanSpec(2000, 4000, 4000, 3, 100, seed=2, planted=(3,), penetrance=0.65),
    "order2_40000x16000": ScanSpec(40000, 8000, 8000, 2, 1000, seed=3, maf="beta", planted=(2, 2, 2, 2, 2),
                                   penetrance=0.6),
    "order4_300x8000": ScanSpec(300, 4000, 4000, 4, 100, seed=4, planted=(4,), penetrance=0.7),
    "order3_500x18800": ScanSpec(500, 9000, 9800, 3, 100, seed=5, planted=(3,), penetrance=0.65),
    "order4_100x18800": ScanSpec(100, 9000, 9800, 4, 50, seed=6, planted=(4,), penetrance=0.7),
}


def batch_specs(n_scans: int = 64, base_seed: int = 1000, outputs: int = 50, snp_range=(500, 20000),
                order4_cap: int = 400, sample_range=(1000, 32000)) -> list:
    """The uneven batch: one spec per scan, each drawn from its own seed (base_seed + i).

    Defaults are the full-size batch (SNPs log-uniform in [500, 20 000], order-4
    scans capped at 400 SNPs, samples log-uniform in [1 000, 32 000], case
    fraction U(0.3, 0.7), order uniform in {2, 3, 4}); the ranges scale it down."""
    specs = []
    for i in range(n_scans):
        rng = np.random.default_rng(base_seed + i)
        order = int(rng.integers(2, 5))
        hi = order4_cap if order == 4 else snp_range[1]
        lo = min(snp_range[0], hi)
        snps = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))) if hi > lo else hi
        snps = max(order, min(snps, hi))
        samples = int(round(math.exp(rng.uniform(math.log(sample_range[0]), math.log(sample_range[1])))))
        frac = float(rng.uniform(0.3, 0.7))
        cases = max(1, min(samples - 1, int(round(samples * frac))))
        specs.append(ScanSpec(snps, cases, samples - cases, order, outputs, seed=base_seed + i))
    return specs


# The batch used by the benchmark: the same distributions with SNP counts
# scaled to [200, 1 200] (order-4 scans capped at 150 SNPs) so that one batch
# is ~1e13 combinations x samples (the full-size batch is ~1.2e16).
BATCH_BENCH = dict(n_scans=64, base_seed=1000, outputs=50, snp_range=(200, 1200), order4_cap=150,
                   sample_range=(1000, 32000))


def _draw_maf(rng, n, kind):
    if kind == "uniform":
        return rng.uniform(0.05, 0.5, n)
    out = np.empty(n)
    filled = 0
    while filled < n:  # Beta(0.5, 0.5) truncated to [0.01, 0.5] by rejection
        x = rng.beta(0.5, 0.5, 2 * (n - filled) + 16)
        x = x[(x >= 0.01) & (x <= 0.5)]
        take = min(len(x), n - filled)
        out[filled:filled + take] = x[:take]
        filled += take
    return out


def _hwe(u, p):
    """Genotype from uniforms u and MAF p (broadcast): 0 w.p. (1-p)^2, 2 w.p. p^2, else 1."""
    q0 = (1.0 - p) ** 2
    q2 = 1.0 - p * p
    return (u >= q0).astype(np.uint8) + (u >= q2).astype(np.uint8)


def simulate(spec: ScanSpec, chunk: int = 2048):
    """Returns (geno uint8 [snps, samples], is_case uint8 [samples], planted list of SNP-index tuples).

    Samples are ordered cases first, then controls."""
    rng = np.random.default_rng(spec.seed)
    maf = _draw_maf(rng, spec.snps, spec.maf)
    planted = []
    if spec.planted:
        idx = rng.choice(spec.snps, size=sum(spec.planted), replace=False)
        pos = 0
        for k in spec.planted:
            planted.append(tuple(sorted(int(x) for x in idx[pos:pos + k])))
            pos += k
    psnps = sorted({s for t in planted for s in t})
    # Draw individuals until both class quotas are filled.
    sel_case, sel_ctrl, pool_geno = [], [], []
    n_case = n_ctrl = 0
    while n_case < spec.cases or n_ctrl < spec.ctrls:
        m = 2 * spec.samples
        g = _hwe(rng.random((len(psnps), m)), maf[psnps][:, None]) if psnps else np.zeros((0, m), np.uint8)
        pcase = np.full(m, 0.5)
        row = {s: r for r, s in enumerate(psnps)}
        for t in planted:
            hit = np.ones(m, bool)
            for s in t:
                hit &= g[row[s]] >= 1
            pcase[hit] = spec.penetrance
        is_case = rng.random(m) < pcase
        ci = np.nonzero(is_case)[0][: spec.cases - n_case]
        ti = np.nonzero(~is_case)[0][: spec.ctrls - n_ctrl]
        sel_case.append(g[:, ci])
        sel_ctrl.append(g[:, ti])
        n_case += len(ci)
        n_ctrl += len(ti)
    planted_geno = np.concatenate(sel_case + sel_ctrl, axis=1) if psnps else None
    geno = np.empty((spec.snps, spec.samples), np.uint8)
    for s0 in range(0, spec.snps, chunk):
        s1 = min(spec.snps, s0 + chunk)
        geno[s0:s1] = _hwe(rng.random((s1 - s0, spec.samples)), maf[s0:s1, None])
    if psnps:
        geno[psnps] = planted_geno
    is_case = np.zeros(spec.samples, np.uint8)
    is_case[: spec.cases] = 1
    return geno, is_case, planted


# ---------------------------------------------------------------------------
# Synthetic genotype files (PLINK .tped/.tfam and .raw) for the ingest path.

_LETTERS = np.frombuffer(b"ACGT", np.uint8)


def write_tped(prefix: str, geno: np.ndarray, is_case: np.ndarray, letters=None, chunk: int = 512):
    """Writes prefix.tped / prefix.tfam: one line per SNP ("chr id 0 pos" then two
    nucleotides per sample), genotype g written as g copies of the SNP's second
    letter.  letters: per-SNP (first, second) indices into ACGT (default A, C).
    Returns the two paths.  Which allele the reader takes as the minor follows
    its own rule (the rarer, ties to the smaller letter), so a file's codes
    are the written ones only where the second letter is the rarer."""
    geno = np.ascontiguousarray(geno, np.uint8)
    snps, n = geno.shape
    tfam = prefix + ".tfam"
    with open(tfam, "w") as f:
        for s in range(n):
            f.write("F%d I%d 0 0 1 %d\n" % (s, s, 2 if is_case[s] else 1))
    tped = prefix + ".tped"
    with open(tped, "wb") as f:
        for s0 in range(0, snps, chunk):
            s1 = min(snps, s0 + chunk)
            if letters is None:
                lut = np.array([b"A A ", b"A C ", b"C C "], dtype="S4").view(np.uint8).reshape(1, 3, 4)
                body = lut[0][geno[s0:s1]]
            else:
                a, b = _LETTERS[letters[s0:s1, 0]], _LETTERS[letters[s0:s1, 1]]
                sp = np.full(s1 - s0, ord(" "), np.uint8)
                lut = np.stack([np.stack([a, sp, a, sp], 1), np.stack([a, sp, b, sp], 1), np.stack([b, sp, b, sp], 1)], 1)
                body = lut[np.arange(s1 - s0)[:, None], geno[s0:s1]]
            body = body.reshape(s1 - s0, 4 * n)
            body[:, -1] = ord("\n")
            for r in range(s1 - s0):
                f.write(b"1 rs%d 0 %d " % (s0 + r, s0 + r))
                f.write(body[r].tobytes())
    return tped, tfam


def write_raw(path: str, geno: np.ndarray, is_case: np.ndarray, gametes: bool = False):
    """Writes a PLINK .raw (FID IID PAT MAT SEX PHENOTYPE rs<i>_A rs<i>_HET ...,
    phenotype 1/2) or, with gametes, a GAMETES .raw (P<i> ... Class, class 0/1)."""
    geno = np.ascontiguousarray(geno, np.uint8)
    snps, n = geno.shape
    with open(path, "w") as f:
        if gametes:
            f.write(" ".join(["P%d" % i for i in range(snps)] + ["Class"]) + "\n")
            for s in range(n):
                f.write(" ".join(map(str, geno[:, s].tolist())) + " %d\n" % (1 if is_case[s] else 0))
        else:
            cols = []
            for i in range(snps):
                cols += ["rs%d_A" % i, "rs%d_HET" % i]
            f.write("FID IID PAT MAT SEX PHENOTYPE " + " ".join(cols) + "\n")
            het = (geno == 1).astype(np.uint8)
            for s in range(n):
                v = np.empty(2 * snps, np.uint8)
                v[0::2], v[1::2] = geno[:, s], het[:, s]
                f.write("F%d I%d 0 0 1 %d " % (s, s, 2 if is_case[s] else 1) + " ".join(map(str, v.tolist())) + "\n")
    return path
