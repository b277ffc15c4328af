"""The tcgen05 building block of the radiance-cache MLP: one 128-row tile of
D = A . B^T with BF16 operands in shared memory and an FP32 accumulator in
tensor memory, against float64 numpy on the same BF16-rounded operands."""

import numpy as np
import pytest

from path_gb300 import api

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k,n", [(16, 16), (48, 64), (64, 64), (64, 16), (128, 128)])
def test_tc_gemm_matches_numpy(lib, k, n):
    rng = np.random.default_rng(k * 1000 + n)
    a = rng.normal(size=(128, k)).astype(np.float32)
    b = rng.normal(size=(n, k)).astype(np.float32)
    d, ar, br = api.debug_tc_gemm(a, b)
    ref = ar.astype(np.float64) @ br.astype(np.float64).T
    err = np.abs(d - ref).max() / np.abs(ref).max()
    print(f"k={k} n={n} max rel err {err:.2e}")
    assert err < 1e-5


def test_tensor_core_wait_that_runs_out_is_reported(lib):
    """The tensor-core kernels' mbarrier waits are bounded: with no MMA
    issued nothing arrives, the wait gives up, the call returns
    PATH_ERR_DEVICE_TIMEOUT (4), and the device computes correctly after."""
    assert api.debug_tc_wait_timeout(1 << 12) == 4
    rng = np.random.default_rng(5)
    a = rng.normal(size=(128, 32)).astype(np.float32)
    b = rng.normal(size=(32, 32)).astype(np.float32)
    d, ar, br = api.debug_tc_gemm(a, b)
    ref = ar.astype(np.float64) @ br.astype(np.float64).T
    assert np.abs(d - ref).max() / np.abs(ref).max() < 1e-5
