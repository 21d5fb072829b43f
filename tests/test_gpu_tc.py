"""Tensor-core building blocks: tcgen05 BF16 products with operands in the
K-major and MN-major canonical shared-memory layouts, against the exact
product of the BF16-rounded inputs (FP32 accumulation tolerance)."""
import numpy as np
import pytest

import lcpgrid as L

pytestmark = pytest.mark.gpu


def bf16(x):
    import torch
    return torch.from_numpy(np.asarray(x, dtype=np.float32)).to(torch.bfloat16).to(torch.float64).numpy()


@pytest.fixture(scope="module")
def ctx():
    return L.Context(0)


@pytest.mark.parametrize("a_mn,b_mn", [(0, 0), (1, 1), (0, 1), (1, 0)])
@pytest.mark.parametrize("n,k", [(16, 16), (64, 32), (256, 64), (48, 48)])
def test_tc_selftest(ctx, a_mn, b_mn, n, k):
    rng = np.random.default_rng(n * 100 + k)
    a = rng.normal(size=(128, k)).astype(np.float32)
    b = rng.normal(size=(n, k)).astype(np.float32)
    d = ctx.tc_selftest(a, b, a_mn=bool(a_mn), b_mn=bool(b_mn))
    ref = bf16(a) @ bf16(b).T
    np.testing.assert_allclose(d, ref, rtol=0, atol=2e-5 * np.sqrt(k) * np.max(np.abs(ref)))
