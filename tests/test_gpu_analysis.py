"""The encoder's block analysis on the GPU (ebivgpu_fdct_satd: forwardDCT and
satd, ebiv/transform.go:44-119) against the numpy restatement in
oracle/transform_ref.py, bit-exact, for every transform size, on residuals
in the encoder's range and on extreme values that exercise the int32
narrowing and wrap-around."""
import numpy as np
import pytest

import transform_ref
from govid_gb300 import ebiv

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [4, 8, 16])
def test_fdct_and_satd_match_the_oracle(gpu_required, n):
    rng = np.random.default_rng(n)
    a = ebiv.BlockAnalysis()
    for lo, hi, count in ((-255, 256, 1000), (-(1 << 24), 1 << 24, 257), (-(1 << 31), (1 << 31) - 1, 33)):
        blocks = rng.integers(lo, hi, size=(count, n, n), dtype=np.int64).astype(np.int32)
        coef, s = a.fdct_satd(blocks)
        assert (coef == transform_ref.forward_dct(blocks, n)).all()
        assert (s == transform_ref.satd(blocks, n)).all()
    # only one of the two outputs
    blocks = rng.integers(-255, 256, size=(5, n, n), dtype=np.int64).astype(np.int32)
    assert a.fdct_satd(blocks, coeffs=False)[0] is None
    assert a.fdct_satd(blocks, satd=False)[1] is None
