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


def _special_floats(n, seed):
    """Random floats of both signs over many binades, with -0.0, +0.0,
    +-inf, subnormals, NaNs of both signs and many ties."""
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(n) * np.exp(rng.uniform(-30, 30, n))).astype(np.float32)
    specials = np.array([-0.0, 0.0, np.inf, -np.inf, 1e-45, -1e-45, 1.1754942e-38, -1.1754942e-38,
                         np.finfo(np.float32).max, -np.finfo(np.float32).max], np.float32)
    k = min(n, 40 * len(specials))
    x[:k] = np.resize(specials, k)
    nan_pos = np.uint32(0x7FC00001)
    nan_neg = np.uint32(0xFFC00002)
    u = x.view(np.uint32)
    if n > 60:
        u[50] = nan_pos
        u[51] = nan_neg
    if n > 3:
        x[::9] = x[3]  # ties keep their input order
    return rng.permutation(x)


@pytest.mark.parametrize("n", [2, 31, 1000, 4096, 70_001, 1_000_003])
def test_radix_sort_f32_matches_float_flip_order(cuda, oracle_lib, n):
    """RadixSort::sort(float*, uint*, n, 32, true): keys in float order
    (-0.0 before +0.0, NaNs by sign at the ends), values moved with them,
    stable; checked against a stable sort on the reference's flip map."""
    import torch
    from gsap_gb300 import Sap
    x = _special_floats(n, n)
    v = np.arange(n, dtype=np.uint32)
    sap = Sap(max(n, 1) // 8 + 1)
    kd = torch.from_numpy(x.copy()).to(cuda)
    vd = torch.from_numpy(v.view(np.int32).copy()).to(cuda)
    sap.radix_sort_f32(kd, vd, 32, True)
    order = np.argsort(oracle_lib.float_flip(x), kind="stable")
    assert np.array_equal(kd.cpu().numpy().view(np.uint32), x.view(np.uint32)[order])
    assert np.array_equal(vd.cpu().numpy().view(np.uint32), v[order])
    # keys only
    kd = torch.from_numpy(x.copy()).to(cuda)
    sap.radix_sort_f32(kd, None, 32, True)
    assert np.array_equal(kd.cpu().numpy().view(np.uint32), x.view(np.uint32)[order])


def test_radix_sort_f32_unsigned_keys(cuda):
    """negativeKeys false: non-negative float keys sorted by their bit
    patterns on the low key_bits bits."""
    import torch
    from gsap_gb300 import Sap
    rng = np.random.default_rng(5)
    n = 200_000
    x = np.abs(rng.standard_normal(n).astype(np.float32)) * 1e3
    x[::4] = x[1]
    v = np.arange(n, dtype=np.uint32)
    sap = Sap(n // 8 + 1)
    kd = torch.from_numpy(x.copy()).to(cuda)
    vd = torch.from_numpy(v.view(np.int32).copy()).to(cuda)
    sap.radix_sort_f32(kd, vd, 32, False)
    order = np.argsort(x, kind="stable")
    assert np.array_equal(kd.cpu().numpy(), x[order])
    assert np.array_equal(vd.cpu().numpy().view(np.uint32), v[order])
    with pytest.raises(Exception, match="key_bits must be 32"):
        sap.radix_sort_f32(kd, vd, 24, True)
