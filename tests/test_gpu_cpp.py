"""The C++ host side on the GPU: the GpuSearch drop-in under MPIEngine (checks
of the reference's tests/threadedsearch.cpp and tests/mpiengine.cpp) and the
fiuncho_gpu command line (output lines of Result::str)."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def unpack_genotypes(data, snps, cases, ctrls, cw, tw):
    """Genotype codes (cases first, then controls) from the reference layout."""
    d = data.reshape(snps, 3 * (cw + tw))
    out = np.zeros((snps, cases + ctrls), np.uint8)
    for cls, (n, W, off) in enumerate(((cases, cw, 0), (ctrls, tw, 3 * cw))):
        s = np.arange(n)
        word = s // 64
        full = n // 64
        bit = np.where(word < full, 63 - (s % 64), (n % 64) - 1 - (s % 64))
        base = 0 if cls == 0 else cases
        for g in range(3):
            rows = d[:, off + g * W: off + (g + 1) * W]
            hit = (rows[:, word] >> bit.astype(np.uint64)) & np.uint64(1)
            out[:, base:base + n][hit.astype(bool)] = g
    return out


def write_gametes_raw(path, geno, cases):
    snps, n = geno.shape
    with open(path, "w") as f:
        f.write("\t".join(["N%d" % i for i in range(snps)] + ["Class"]) + "\n")
        for s in range(n):
            f.write("\t".join(str(int(x)) for x in geno[:, s]) + "\t%d\n" % (1 if s < cases else 0))


@pytest.fixture(scope="module")
def raw_file(golden_testdata, tmp_path_factory):
    snps, cases, ctrls, cw, tw = (int(x) for x in golden_testdata["meta"])
    geno = unpack_genotypes(golden_testdata["data"], snps, cases, ctrls, cw, tw)
    p = tmp_path_factory.mktemp("cpp") / "test.raw"
    write_gametes_raw(str(p), geno, cases)
    from fiuncho_gb300 import Dataset
    assert np.array_equal(Dataset.read([str(p)]).data, golden_testdata["data"])
    return str(p)


@pytest.fixture(scope="module")
def bins():
    from fiuncho_gb300 import build
    return build.build_cpp()


def test_cpp_gpusearch_reference_checks(bins, raw_file, golden_testdata, tmp_path):
    m = tmp_path / "mpi3snp.txt"
    m.write_text("".join("%d %d %d %.9g\n" % (int(a), int(b), int(c), float(v)) for (a, b, c), v in
                         zip(golden_testdata["mpi3snp_combos"], golden_testdata["mpi3snp_vals"])))
    r = subprocess.run([bins["test_gpusearch"], raw_file, str(m)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "PASS" in r.stdout, r.stdout + r.stderr


def test_cli_output_matches_python_api(bins, raw_file, tmp_path):
    from fiuncho_gb300 import Dataset, Distribution, GpuSearch
    out = tmp_path / "out.txt"
    r = subprocess.run([bins["fiuncho_gpu"], "-o", "3", "-n", "25", raw_file, str(out)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    ds = Dataset.read([raw_file])
    want = [x.str() for x in GpuSearch(0).run(ds, 3, Distribution(ds.snps, 2), 25)]
    assert out.read_text().splitlines() == want
    r = subprocess.run([bins["fiuncho_gpu"], "-o", "1", raw_file, str(out)], capture_output=True, text=True)
    assert r.returncode == 1 and "order" in r.stderr
