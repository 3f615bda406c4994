"""GPU parity of the onesweep radix sort against a stable CPU sort."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,bits", [(1, 32), (2, 8), (4095, 32), (4096, 24), (4097, 16), (100_003, 32),
                                    (1 << 20, 24), (3_000_000, 32)])
def test_radix_sort_stable(cuda, n, bits):
    import torch
    from gsap_gb300 import Sap
    sap = Sap(max(n, 1) // 8 + 1)
    rng = np.random.default_rng(n)
    k = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    k[::5] = k[0]  # many ties
    if bits < 32:
        k &= np.uint32((1 << bits) - 1)
    v = np.arange(n, dtype=np.uint32)
    kd = torch.from_numpy(k.view(np.int32).copy()).to(cuda)
    vd = torch.from_numpy(v.view(np.int32).copy()).to(cuda)
    sap.radix_sort(kd, vd, bits)
    order = np.argsort(k, kind="stable")
    assert np.array_equal(vd.cpu().numpy().view(np.uint32), v[order])
    assert np.array_equal(kd.cpu().numpy().view(np.uint32), k[order])
