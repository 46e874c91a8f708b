"""Device packing of genotype codes (fiu_dataset_upload_genotypes): the packed
layout built on the GPU is byte-identical to the reference reader's.

* The reference's own test data set, as its reader packed it (fixture): its
  codes, unpacked from that fixture, packed again on the device.
* Synthetic .tped and .raw files parsed by the library's threaded reader and
  packed on the device, against the host packer, and searched.
* A full-size file (40 000 SNPs x 16 000 samples, 2.6 GB of text) against the
  reference's reader on the same file (fixture, taken with the reference built
  from its sources).  That reader zeroes a class's last full word when the
  other class's samples follow it (TPEDFile.hpp:222-238 rewrite the word with
  the cleared buffer while the count stays a multiple of 64; here the 8 000
  cases, 125 full words, precede the controls), so the library's packing --
  which keeps those 64 cases' genotypes -- must equal the reference's once the
  same words are zeroed, and equal the fixture's digest of the correct packing."""
import hashlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from fiuncho_gb300 import Context
    return Context(0)


def unpack(data, snps, n_cases, n_ctrls, cw, tw):
    """Genotype codes [snps, cases + controls] (cases first) of a packed data set."""
    d = np.asarray(data, np.uint64).reshape(snps, 3 * (cw + tw))
    out = np.full((snps, n_cases + n_ctrls), 255, np.uint8)
    for cls, (cnt, W, off, s0) in enumerate(((n_cases, cw, 0, 0), (n_ctrls, tw, 3 * cw, n_cases))):
        b = np.arange(cnt)
        w, r = b // 64, cnt % 64
        bit = np.where((w == cnt // 64) & (r > 0), r - 1 - (b % 64), 63 - (b % 64)).astype(np.uint64)
        blk = out[:, s0:s0 + cnt]  # a view: assignments below land in out
        for g in range(3):
            words = d[:, off + g * W + w]
            blk[((words >> bit) & np.uint64(1)).astype(bool)] = g
    return out


def test_reference_test_data_packs_identically(ctx, golden_testdata):
    from fiuncho_gb300 import Dataset, ingest
    snps, cases, ctrls, cw, tw = (int(x) for x in golden_testdata["meta"])
    geno = unpack(golden_testdata["data"], snps, cases, ctrls, cw, tw)
    assert np.all(geno < 3), "every sample has one genotype"
    is_case = np.r_[np.ones(cases, bool), np.zeros(ctrls, bool)]
    assert np.array_equal(Dataset.from_genotypes(geno, is_case).data, golden_testdata["data"])
    res = ingest.upload_genotypes(ctx, geno, is_case)
    data, meta = ingest.packed(ctx, res)
    assert meta == (snps, cases, ctrls, cw, tw)
    assert np.array_equal(data, golden_testdata["data"])
    assert res.one_hot


@pytest.mark.parametrize("fmt", ["tped", "raw"])
def test_files_parse_and_pack_on_the_device(ctx, tmp_path, fmt):
    from fiuncho_gb300 import Dataset, Distribution, GpuSearch, Resident, dataset, ingest, synth
    rng = np.random.default_rng(9)
    snps, n = 150, 3001
    maf = rng.uniform(0.05, 0.5, snps)[:, None]
    u = rng.random((snps, n))
    geno = ((u >= (1 - maf) ** 2).astype(np.uint8) + (u >= 1 - maf ** 2)).astype(np.uint8)
    is_case = rng.random(n) < 0.4  # classes interleaved in the file
    if fmt == "tped":
        files = list(synth.write_tped(str(tmp_path / "x"), geno, is_case))
    else:
        files = [synth.write_raw(str(tmp_path / "x.raw"), geno, is_case)]
    g, c = ingest.read_genotypes(files, threads=6, ctx=ctx)
    want = Dataset.from_genotypes(*dataset.read_genotypes(files))
    res = ingest.upload_genotypes(ctx, g, c)
    data, meta = ingest.packed(ctx, res)
    assert meta == (want.snps, want.cases, want.ctrls, want.cases_words, want.ctrls_words)
    assert np.array_equal(data, want.data)
    gs = GpuSearch(0)
    host = Resident(gs.ctx, want)
    dev = ingest.upload_genotypes(gs.ctx, g, c)
    for order in (2, 3):
        a = gs.run(host, order, Distribution(snps, order - 1), 20, with_fp64=True)
        b = gs.run(dev, order, Distribution(snps, order - 1), 20, with_fp64=True)
        assert [x.combination for x in a[0]] == [x.combination for x in b[0]] and np.array_equal(a[1], b[1])


def test_full_size_file_packs_like_the_reference_reader(ctx, tmp_path):
    """40 000 SNPs x 8 000 / 8 000 samples written as .tped / .tfam (2.6 GB)."""
    from fiuncho_gb300 import ingest, synth
    scale = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_scale.npz")))
    if "order2_40000x16000_tped_sha256" not in scale:
        pytest.skip("fixture without the reference reader's digest")
    g, c, _ = synth.simulate(synth.WORKLOADS["order2_40000x16000"])
    tped, tfam = synth.write_tped(str(tmp_path / "cfg3"), g, c)
    del g, c
    geno, is_case = ingest.read_genotypes([tped, tfam], threads=0, ctx=ctx)
    os.remove(tped)
    res = ingest.upload_genotypes(ctx, geno, is_case)
    del geno
    data, meta = ingest.packed(ctx, res)
    assert meta == tuple(int(x) for x in scale["order2_40000x16000_tped_meta"])
    assert hashlib.sha256(data.tobytes()).hexdigest() == str(scale["order2_40000x16000_tped_sha256"])
    snps, _, _, cw, tw = meta
    quirk = data.reshape(snps, 3 * (cw + tw)).copy()
    quirk[:, scale["order2_40000x16000_tped_ref_zeroed_columns"]] = 0
    assert hashlib.sha256(quirk.tobytes()).hexdigest() == str(scale["order2_40000x16000_tped_ref_sha256"])
