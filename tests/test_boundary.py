"""The C-ABI boundary and the host-side mirror of the reference API (no GPU)."""
import ctypes
import os

import numpy as np
import pytest

from fiuncho_gb300 import _lib


def test_library_exports_every_declared_symbol():
    """libfiuncho_gpu.so loads (no GPU needed to load) and exports every function in include/*.h."""
    lib = _lib.load()
    declared = _lib.header_symbols()
    assert "fiu_search" in declared and "fiu_combine_and_popcnt" in declared
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) >= set(_lib._SIGS), "binding declares a function the header does not"


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.fiu_create(0, ctypes.byref(h)) != 0
    assert not h.value


def test_result_text_and_serialisation():
    from fiuncho_gb300 import Result
    r = Result([4, 8, 9], 0.137896782)
    assert r.str() == "4 8 9 0.137897"
    b = r.serialize()
    assert len(b) == 8 + 3 * 4 + 4  # size_t count + ints + float (Result.h:47-56)
    r2, pos = Result.deserialize(b)
    assert pos == len(b) and r2.combination == [4, 8, 9] and abs(r2.val - r.val) < 1e-7


def test_distribution_mirror(oracle):
    from fiuncho_gb300 import Distribution
    d = Distribution(12, 2, 3, 1)
    assert [tuple(c) for c in d] == [tuple(x) for x in oracle.prefixes(12, 2, 3, 1)]
    l = d.layer(2, 1)
    assert (l.step, l.offset) == (6, 3)
    with pytest.raises(ValueError):
        Distribution(10, 2, 0, 0)


def test_engine_single_rank_gather_sorts_and_truncates():
    from fiuncho_gb300 import MPIEngine, Result
    e = MPIEngine()
    assert (e.size, e.rank) == (1, 0)
    res = [Result([1, 2], 0.5), Result([0, 3], 0.9), Result([0, 1], 0.5)]
    out = e.gather(res, 2)
    assert [r.combination for r in out] == [[0, 3], [0, 1]]


def test_dataset_readers_match_packed_fixture(golden_testdata):
    """Our TPED / RAW / GAMETES readers produce the reference's packed bits (needs the reference's data files)."""
    from fiuncho_gb300 import Dataset
    from oracle.build import REF_ROOT as root
    d = os.path.join(root, "tests", "data")
    if not os.path.exists(os.path.join(d, "test.tped")):
        pytest.skip("reference test data not present")
    for files in ([d + "/test.tped", d + "/test.tfam"], [d + "/test.tfam", d + "/test.tped"], [d + "/test.raw"],
                  [d + "/test.gametes.raw"]):
        ds = Dataset.read(files)
        assert np.array_equal(ds.data, golden_testdata["data"]), files


def test_dataset_reader_errors(tmp_path):
    from fiuncho_gb300 import Dataset
    with pytest.raises(ValueError):
        Dataset.read([str(tmp_path / "x.bed")])
    with pytest.raises(ValueError):
        Dataset.read([str(tmp_path / "a.tped"), str(tmp_path / "b.tped")])
    (tmp_path / "t.tfam").write_text("f i 0 0 0 2\nf j 0 0 0 1\n")
    (tmp_path / "t.tped").write_text("1 rs1 0 1 A A C N\n")
    with pytest.raises(ValueError):
        Dataset.read([str(tmp_path / "t.tped"), str(tmp_path / "t.tfam")])
    (tmp_path / "t.tped").write_text("1 rs1 0 1 A A C C A\n")
    with pytest.raises(ValueError):
        Dataset.read([str(tmp_path / "t.tped"), str(tmp_path / "t.tfam")])
    (tmp_path / "u.tfam").write_text("f i 0 0 0 3\n")
    (tmp_path / "u.tped").write_text("1 rs1 0 1 A A\n")
    with pytest.raises(ValueError):
        Dataset.read([str(tmp_path / "u.tped"), str(tmp_path / "u.tfam")])


def test_pack_partial_word_right_aligned(oracle):
    """Partial last words are right-aligned (TPEDFile.hpp:240-254); packer == oracle packer for ragged sizes."""
    from fiuncho_gb300.dataset import pack_rows, words_for
    rng = np.random.default_rng(3)
    for n_case, n_ctrl in ((1, 1), (63, 65), (64, 64), (129, 7), (200, 0)):
        geno = rng.integers(0, 3, (5, n_case + n_ctrl), dtype=np.uint8)
        is_case = np.zeros(n_case + n_ctrl, np.uint8)
        is_case[rng.permutation(n_case + n_ctrl)[:n_case]] = 1
        cw, tw = words_for(n_case) + 1, max(words_for(n_ctrl), 1)
        assert np.array_equal(pack_rows(geno, is_case, cw, tw), oracle.pack(geno, is_case, cw, tw))


def test_server_rejected_policy_destroys_once(monkeypatch):
    """A refused serving policy destroys the new server exactly once (no second destroy
    when the Python object is collected)."""
    import gc

    from fiuncho_gb300 import _lib, search

    calls = []

    class FakeLib:
        def fiu_server_create(self, dev, budget, ph):
            ph._obj.value = 1234
            return 0

        def fiu_server_set_policy(self, h, policy):
            return 1

        def fiu_server_destroy(self, h):
            calls.append(h)

    monkeypatch.setattr(_lib, "load", lambda: FakeLib())
    with pytest.raises(search.FiunchoError):
        search.Server(0, policy=7)
    gc.collect()
    assert len(calls) == 1
