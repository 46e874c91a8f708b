"""Parity at the measured sizes: every contingency table and the top-N of the
full-size workloads against the reference's own results.

The reference (built from its sources, AVX-512BW build) produced, for each
workload of ``tests/golden/make_golden_scale.py``, the digest of its tables of
EVERY combination (``oracle/ref/tabledigest.h``: a 64-bit sum over the
combinations of a hash of the combination and its 3^k x 2 cells) and its
``ThreadedSearch::run`` top-N.  Here the library's own kernels compute the same
digest over the same combinations (``fiu_scan_digest``), so equal digests mean
every table of the scan is bit-exact (a mismatch in any cell of any combination
changes the sum except with probability about 2^-64).

Top-N rule: the reference ranks by its FP32 MI, the library by the exact MI;
the lists must be identical except for combinations whose exact MI lies within
the reference's own FP32 error (measured on the same list, doubled) of the
cutoff.  The library's values must be within 1e-5 relative of the FP64 oracle.
"""
import hashlib
import math
import os

import numpy as np
import pytest

from helpers import as_set, assert_ascending_unique, assert_sorted_desc, assert_topn_equivalent, exact_mi

pytestmark = pytest.mark.gpu

K_AUTO, K_FULL, K_POPC, K_HS, K_TENSOR = 0, 1, 2, 3, 4
MI_RTOL = 1e-5
SCALE = os.path.join(os.path.dirname(__file__), "golden", "reference_scale.npz")


@pytest.fixture(scope="module")
def gs():
    from fiuncho_gb300 import GpuSearch
    return GpuSearch(0)


@pytest.fixture(scope="module")
def scale():
    return dict(np.load(SCALE))


def _scale_names():
    g = np.load(SCALE)
    return sorted({k.rsplit("_", 1)[0] for k in g.files if k.endswith("_digest")})


# ---------------------------------------------------------------- every kernel, small data
@pytest.mark.parametrize("order,kernel", [(o, k) for o in (2, 3, 4) for k in (K_TENSOR, K_POPC, K_HS, K_FULL)])
def test_digest_every_kernel(gs, golden_synth, order, kernel):
    """Each kernel's own tables of every combination (48 SNPs, 999 / 1 001 samples) equal the
    reference's: digest and combination count."""
    from fiuncho_gb300 import Dataset
    from fiuncho_gb300.search import Resident
    ds = Dataset.from_genotypes(golden_synth["geno"], golden_synth["is_case"])
    res = Resident(gs.ctx, ds)
    dg, cnt = gs.scan_digest(res, order, None, kernel)
    assert cnt == int(golden_synth["o%d_digest_count" % order]) == math.comb(ds.snps, order)
    assert dg == int(golden_synth["o%d_digest" % order])


@pytest.mark.parametrize("kernel", [K_TENSOR, K_AUTO, K_POPC, K_HS, K_FULL])
def test_digest_distribution_layer(gs, golden_synth, kernel):
    """The tables of the combinations a Distribution(48, 2, 3, 2) layer owns."""
    from fiuncho_gb300 import Dataset, Distribution
    from fiuncho_gb300.search import Resident
    ds = Dataset.from_genotypes(golden_synth["geno"], golden_synth["is_case"])
    res = Resident(gs.ctx, ds)
    dg, cnt = gs.scan_digest(res, 3, Distribution(ds.snps, 2, 3, 2), kernel)
    assert cnt == int(golden_synth["o3_step3_off2_digest_count"])
    assert dg == int(golden_synth["o3_step3_off2_digest"])


# ---------------------------------------------------------------- full size
# kernels whose digest is taken besides the automatic choice (each a whole scan)
EXTRA_KERNELS = {
    "order2_1000x4000": (K_POPC, K_HS, K_FULL),
    "order3_2000x8000": (K_HS,),
    "order4_300x8000": (K_POPC,),
    "order3_500x18800": (K_HS,),
    "order4_100x18800": (K_POPC, K_FULL),
}


@pytest.mark.parametrize("name", _scale_names())
def test_full_size_parity(gs, oracle, scale, name):
    from fiuncho_gb300 import Dataset, Distribution, synth
    from fiuncho_gb300.search import Resident
    spec = synth.WORKLOADS[name]
    geno, is_case, _ = synth.simulate(spec)
    ds = Dataset.from_genotypes(geno, is_case)
    del geno
    sha = hashlib.sha256(np.ascontiguousarray(ds.data, np.uint64).tobytes()).hexdigest()
    assert sha == str(scale[name + "_sha256"]), "regenerated data set differs from the one the reference saw"
    res = Resident(gs.ctx, ds)
    want_dg, want_cnt = int(scale[name + "_digest"]), int(scale[name + "_count"])
    assert want_cnt == math.comb(spec.snps, spec.order)
    # every table, as the kernel the search picks computes it, and as the other kernels do
    for kernel in (K_AUTO,) + EXTRA_KERNELS.get(name, ()):
        dg, cnt = gs.scan_digest(res, spec.order, None, kernel)
        assert cnt == want_cnt, (kernel, cnt, want_cnt)
        assert dg == want_dg, "kernel %d: tables differ from the reference's" % kernel
    # the top-N against the reference's own list
    results, v64 = gs.run(res, spec.order, Distribution(ds.snps, spec.order - 1), spec.outputs, with_fp64=True)
    got = np.array([r.combination for r in results], np.int32).reshape(-1, spec.order)
    ref_c, ref_v = scale[name + "_combos"], scale[name + "_vals"].astype(np.float64)
    assert len(got) == len(ref_c) == spec.outputs
    assert_ascending_unique(got)
    assert_sorted_desc(v64)
    ex = lambda cs: exact_mi(oracle, ds.data, ds.cases_words, ds.ctrls_words, ds.cases, ds.ctrls, spec.order, cs)
    mine = ex(got)
    assert np.allclose(v64, mine, rtol=MI_RTOL, atol=1e-12), "FP64 MI differs from the oracle"
    ref_exact = ex(ref_c)
    ref_err = float(np.max(np.abs(ref_v - ref_exact)))
    assert ref_err <= 1e-2 * float(np.max(ref_exact)), "reference FP32 error larger than expected"
    tol = 2.0 * ref_err + 1e-9
    assert_topn_equivalent(got, ref_c, ex, tol)
    common = as_set(got) & as_set(ref_c)
    assert 2 * len(common) >= spec.outputs, "top-N lists share too few combinations"
