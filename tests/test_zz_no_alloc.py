"""fiu_mi_compute_noalloc: MI over caller-owned device tables with no device
allocation, for callers that cannot allocate (a host whose GPU memory belongs
to its own pool, a pipeline that cannot take cudaMalloc's device-wide
synchronisation).  Both entry points compute the same fixed-point key from
the same c ln c table, so its result must equal the allocating entry point's,
fiu_mi_compute (mode 0), bit for bit, on calls in a row -- the first call on
the device runs the table's set-up, the later ones reuse it.  Kept in a file
that is collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

def _tables(rng, count, cells, n_cases, n_ctrls):
    cases = rng.multinomial(n_cases, np.full(cells, 1.0 / cells), size=count).astype(np.uint32)
    p = rng.dirichlet(np.ones(cells), size=count)
    ctrls = np.stack([rng.multinomial(n_ctrls, q) for q in p]).astype(np.uint32)
    return cases, ctrls


def test_mi_compute_noalloc_matches_allocating_entry_point():
    import torch

    from fiuncho_gb300 import GpuSearch, _lib
    lib = _lib.load()
    gs = GpuSearch(0)
    rng = np.random.default_rng(2024)
    stream = torch.cuda.current_stream()
    for cells, count, n_cases, n_ctrls in ((27, 3000, 4000, 4000), (9, 1777, 9000, 9800), (81, 901, 65000, 536)):
        cases, ctrls = _tables(rng, count, cells, n_cases, n_ctrls)
        want, _ = gs.mi(cases, ctrls, n_cases, n_ctrls, mode=0)
        d_cases = torch.from_numpy(cases.view(np.int32)).cuda()
        d_ctrls = torch.from_numpy(ctrls.view(np.int32)).cuda()
        d_out = torch.full((count,), float("nan"), dtype=torch.float32, device="cuda")
        rc = lib.fiu_mi_compute_noalloc(ctypes.c_void_p(d_cases.data_ptr()), ctypes.c_void_p(d_ctrls.data_ptr()),
                                        cells, count, n_cases, n_ctrls, ctypes.c_void_p(d_out.data_ptr()),
                                        ctypes.c_void_p(stream.cuda_stream))
        assert rc == _lib.FIU_OK
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        np.testing.assert_array_equal(got, want)


def test_mi_compute_noalloc_rejects_oversized_requests():
    import torch

    from fiuncho_gb300 import _lib
    lib = _lib.load()
    buf = torch.zeros(27, dtype=torch.int32, device="cuda")
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    rc = lib.fiu_mi_compute_noalloc(p, p, 27, 1, _lib.FIU_NOALLOC_MAX_SAMPLES, 1, ctypes.c_void_p(out.data_ptr()),
                                    None)
    assert rc == _lib.FIU_ERR_UNSUPPORTED
