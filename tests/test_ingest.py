"""The library's multi-threaded genotype file parser (fiu_read_genotypes) gives
the same genotype codes and case flags as the reference-rule readers of
fiuncho_gb300.dataset (pinned to the reference's own reader on its test data
in test_boundary.py), and rejects the same malformed inputs.  Host only."""
import numpy as np
import pytest


def _data(seed, snps, n, interleave=True):
    rng = np.random.default_rng(seed)
    maf = rng.uniform(0.02, 0.6, snps)[:, None]  # some "minor" alleles above 0.5: the reader flips those
    u = rng.random((snps, n))
    geno = ((u >= (1 - maf) ** 2).astype(np.uint8) + (u >= 1 - maf ** 2)).astype(np.uint8)
    geno[3] = 0  # monomorphic
    geno[4] = 2
    is_case = rng.random(n) < 0.45 if interleave else np.r_[np.ones(n // 2, bool), np.zeros(n - n // 2, bool)]
    return geno, is_case


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_tped_codes_match_reference_rules(tmp_path, threads):
    from fiuncho_gb300 import dataset, ingest, synth
    geno, is_case = _data(1, 57, 1003)
    rng = np.random.default_rng(2)
    letters = np.sort(np.stack([rng.choice(4, 2, replace=False) for _ in range(57)]), axis=1)
    letters[::2] = letters[::2, ::-1]  # second letter sometimes the smaller one
    tped, tfam = synth.write_tped(str(tmp_path / "x"), geno, is_case, letters=letters)
    want_g, want_c = dataset.read_tped(tped, tfam)
    for files in ([tped, tfam], [tfam, tped]):
        g, c = ingest.read_genotypes(files, threads=threads)
        assert np.array_equal(g, want_g) and np.array_equal(c, want_c)


@pytest.mark.parametrize("gametes", [False, True])
def test_raw_codes_match_reference_rules(tmp_path, gametes):
    from fiuncho_gb300 import dataset, ingest, synth
    geno, is_case = _data(3, 31, 401)
    path = synth.write_raw(str(tmp_path / "x.raw"), geno, is_case, gametes=gametes)
    want_g, want_c = dataset.read_raw(path)
    g, c = ingest.read_genotypes([path], threads=4)
    assert np.array_equal(g, want_g) and np.array_equal(c, want_c)
    assert np.array_equal(g, geno) and np.array_equal(c, is_case)


def test_reader_errors(tmp_path):
    from fiuncho_gb300 import FiunchoError, ingest
    fam = tmp_path / "a.tfam"
    fam.write_text("F I 0 0 1 2\nF J 0 0 1 1\n")
    bad = {"b.tped": "1 rs 0 1 A A C X\n", "c.tped": "1 rs 0 1 A A C\n", "d.tped": "1 rs 0\n",
           "e.tped": "1 rs 0 1 A A\n"}
    for name, text in bad.items():
        p = tmp_path / name
        p.write_text("1 r 0 1 A A C C\n\n" + text)
        with pytest.raises(FiunchoError):
            ingest.read_genotypes([str(p), str(fam)])
    bad_fam = tmp_path / "bad.tfam"
    bad_fam.write_text("F I 0 0 1 3\n")
    ok = tmp_path / "ok.tped"
    ok.write_text("1 r 0 1 A A\n")
    with pytest.raises(FiunchoError):
        ingest.read_genotypes([str(ok), str(bad_fam)])
    with pytest.raises(FiunchoError):
        ingest.read_genotypes([str(tmp_path / "missing.tped"), str(fam)])
    raw = tmp_path / "r.raw"
    raw.write_text("FID IID PAT MAT SEX rs1_A\nF I 0 0 1 0\n")  # no phenotype column
    with pytest.raises(FiunchoError):
        ingest.read_genotypes([str(raw)])
    raw.write_text("FID IID PAT MAT SEX PHENOTYPE rs1_A\nF I 0 0 1 2 x\n")  # non-numeric
    with pytest.raises(FiunchoError):
        ingest.read_genotypes([str(raw)])
    with pytest.raises(FiunchoError):
        ingest.read_genotypes([str(tmp_path / "x.bed")])


def test_reference_reader_zeroes_a_class_word_the_library_keeps(tmp_path):
    """Where a class's sample count reaches a multiple of 64 and samples of the
    other class follow, the reference's reader writes that class's completed
    word again from its cleared buffer (TPEDFile.hpp:222-238), zeroing 64
    samples' genotypes.  The library keeps them (every SNP's rows stay one-hot);
    otherwise the two packings are identical.  Needs the reference build."""
    from fiuncho_gb300 import Dataset, ingest, synth
    from oracle import build as obuild
    if not obuild.reference_present():
        pytest.skip("reference tree not present")
    from oracle.oracle import Reference
    geno, _ = _data(5, 20, 200)
    is_case = np.r_[np.ones(128, bool), np.zeros(72, bool)]  # 128 cases (two full words), then controls
    tped, tfam = synth.write_tped(str(tmp_path / "q"), geno, is_case)
    ref = Reference("base").read(tped, tfam).packed().reshape(20, -1)
    mine = Dataset.from_genotypes(*ingest.read_genotypes([tped, tfam], threads=2))
    ours = mine.data.reshape(20, -1)
    cw = mine.cases_words
    cols = [k * cw + cw - 1 for k in range(3)]
    assert np.all(ref[:, cols] == 0) and not np.all(ours[:, cols] == 0)
    ours = ours.copy()
    ours[:, cols] = 0
    assert np.array_equal(ours, ref)
