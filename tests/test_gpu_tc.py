"""tcgen05 split-TF32 GEMM against an FP64 reference (GB300 only)."""
import numpy as np
import pytest

from ttns_lib_gb300 import api

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("K,N", [(8, 16), (64, 64), (128, 64), (128, 32), (96, 128)])
def test_tc_gemm_split_tf32_matches_fp64(K, N):
    rng = np.random.default_rng(K * 1000 + N)
    a = rng.normal(size=(128, K))
    b = rng.normal(size=(N, K))
    d = api.device_tc_gemm(a, b)
    ref = a @ b.T
    # split TF32 (about 22 significant bits per operand) with FP32 accumulation:
    # absolute error ~ sqrt(K) * |a||b| * 2^-22
    err = np.abs(d - ref).max()
    assert err < 2e-5 * np.sqrt(K), err
    # a plain single-TF32 product would be ~2^-11 relative: check we are far below it
    assert err < 1e-3 * np.abs(ref).max()
