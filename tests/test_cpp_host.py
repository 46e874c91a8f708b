"""The C++ host side (no GPU): the GpuSearch drop-in compiles against the
reference's own headers, and the C++ mirror's readers pack like the reference."""
import os
import subprocess

import numpy as np
import pytest

from oracle.build import REF_ROOT as REF  # noqa: E402
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bins():
    from fiuncho_gb300 import build
    return build.build_cpp()


def test_gpusearch_compiles_against_reference_headers(tmp_path):
    """MPIEngine::run<GpuSearch>(...) of the reference's own MPIEngine.h (1-rank MPI stand-in)."""
    if not os.path.isdir(os.path.join(REF, "include", "fiuncho")):
        pytest.skip("reference headers not present")
    from fiuncho_gb300 import build
    lib = build.build()
    src = tmp_path / "dropin.cpp"
    src.write_text(
        "#include <algorithm>\n#include <bitset>\n#include <cmath>\n#include <filesystem>\n#include <map>\n"
        "#include <regex>\n#include <sstream>\n#include <iostream>\n#include \"mpi.h\"\n"
        "#include <fiuncho/MPIEngine.h>\n#include <fiuncho/GpuSearch.h>\n"
        "int main(int argc, char** argv) {\n"
        "  try { MPIEngine e; auto r = e.run<GpuSearch>({argv[1], argv[2]}, 3, 10, 0); std::cout << r.size(); }\n"
        "  catch (const std::runtime_error& x) { std::cout << \"runtime_error: \" << x.what(); return 3; }\n"
        "  return 0; }\n")
    exe = tmp_path / "dropin"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(REF, "include"),
                    "-I", os.path.join(ROOT, "oracle", "ref"), "-I", os.path.join(ROOT, "include"), str(src),
                    "-L", os.path.dirname(lib), "-lfiuncho_gpu", "-Wl,-rpath," + os.path.dirname(lib), "-pthread",
                    "-o", str(exe)], check=True, capture_output=True)
    import torch
    if not torch.cuda.is_available():
        d = os.path.join(REF, "tests", "data")
        r = subprocess.run([str(exe), d + "/test.tped", d + "/test.tfam"], capture_output=True, text=True)
        assert r.returncode == 3 and "cannot create a context" in r.stdout


def test_cpp_readers_pack_like_reference(bins, golden_testdata, tmp_path):
    d = os.path.join(REF, "tests", "data")
    if not os.path.exists(os.path.join(d, "test.tped")):
        pytest.skip("reference test data not present")
    for files in ([d + "/test.tped", d + "/test.tfam"], [d + "/test.tfam", d + "/test.tped"], [d + "/test.raw"],
                  [d + "/test.gametes.raw"]):
        out = tmp_path / "dump.bin"
        subprocess.run([bins["dump_dataset"], str(out)] + files, check=True)
        raw = np.fromfile(out, np.uint64)
        assert list(raw[:5]) == [10, 9000, 9800, 141, 154]
        assert np.array_equal(raw[5:], golden_testdata["data"]), files


def test_cpp_reader_errors(bins, tmp_path):
    (tmp_path / "a.tfam").write_text("f i 0 0 0 7\n")
    (tmp_path / "a.tped").write_text("1 rs 0 1 A C\n")
    r = subprocess.run([bins["dump_dataset"], str(tmp_path / "o"), str(tmp_path / "a.tped"), str(tmp_path / "a.tfam")],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "parsing error" in r.stderr
    r = subprocess.run([bins["dump_dataset"], str(tmp_path / "o"), str(tmp_path / "a.bed")], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "Unrecognized input file extension" in r.stderr
