"""The learned surrogate of the bond-order term: tensor-core building block,
descriptors, network, training and the fallback to the exact kernel."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16(x):
    """FP32 -> BF16 (round to nearest even) -> FP32, as __float2bfloat16_rn."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("n,k", [(32, 16), (64, 32), (64, 64), (128, 128), (32, 128)])
def test_tensor_core_gemm(eng, n, k):
    rng = np.random.default_rng(n * 1000 + k)
    A = rng.standard_normal((128, k)).astype(np.float32)
    B = rng.standard_normal((n, k)).astype(np.float32)
    C = eng.tc_selftest(A, B)
    ref = bf16(A).astype(np.float64) @ bf16(B).astype(np.float64).T
    assert np.abs(C - ref).max() <= 1e-4 * np.abs(ref).max()
