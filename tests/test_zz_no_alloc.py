"""gsap_radix_sort_u32_noalloc against gsap_radix_sort_u32.

This file is named to be collected last, so the GPU test also runs after
every other test has used the device.  It must pass on its own as well
(`pytest tests/test_zz_no_alloc.py -m gpu`).
"""
import numpy as np
import pytest


def _keys(n, bits, seed):
    rng = np.random.default_rng(seed)
    k = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    k[::7] = k[0]  # ties: both sorts must keep input order
    if bits < 32:
        k &= np.uint32((1 << bits) - 1)
    return k


def test_noalloc_rejects_oversize(gsap_lib):
    # the size check comes before any device call, so this runs without a GPU
    from gsap_gb300.sap import NOALLOC_SORT_MAX_N
    st = gsap_lib.gsap_radix_sort_u32_noalloc(None, None, NOALLOC_SORT_MAX_N + 1, 32, None)
    assert st == 2  # GSAP_ERR_CAPACITY
    assert b"fixed scratch" in gsap_lib.gsap_last_error()


@pytest.mark.gpu
def test_noalloc_matches_handle_sort_twice(cuda):
    import torch
    from gsap_gb300 import Sap
    from gsap_gb300.sap import NOALLOC_SORT_MAX_N, radix_sort_noalloc

    cases = [(300_001, 32, 1), (NOALLOC_SORT_MAX_N, 24, 2)]  # two calls in a row, the second at the limit
    ref = Sap(NOALLOC_SORT_MAX_N // 8 + 1)
    host = []
    for n, bits, seed in cases:
        k = _keys(n, bits, seed)
        v = np.arange(n, dtype=np.uint32)[::-1].copy()
        host.append((k, v, bits))
    dev = [(torch.from_numpy(k.view(np.int32)).to(cuda), torch.from_numpy(v.view(np.int32)).to(cuda))
           for k, v, _ in host]
    expect = []
    for (kd, vd), (_, _, bits) in zip(dev, host):
        k2, v2 = kd.clone(), vd.clone()
        ref.radix_sort(k2, v2, bits)
        expect.append((k2, v2))
    torch.cuda.synchronize()

    radix_sort_noalloc(*dev[0], bits=host[0][2])  # first call on the device: set-up
    torch.cuda.synchronize()
    # no garbage collection inside the window: a cycle of earlier tests'
    # tensors freed there would move torch's count without our calls
    import gc
    gc.collect()
    gc.disable()
    try:
        free_before = torch.cuda.mem_get_info()[0]
        torch_before = torch.cuda.memory_allocated()
        radix_sort_noalloc(*dev[1], bits=host[1][2])
        radix_sort_noalloc(*dev[0], bits=host[0][2])  # already sorted input: must stay put
        torch.cuda.synchronize()
        torch_after = torch.cuda.memory_allocated()
        free_after = torch.cuda.mem_get_info()[0]
    finally:
        gc.enable()
    # torch's own allocator saw no allocation; the device's free memory (which
    # other processes on the GPU can also move) is checked as well
    assert torch_after == torch_before
    assert free_after == free_before, "device memory changed across no-alloc calls"

    for (kd, vd), (ke, ve), (k, v, _) in zip(dev, expect, host):
        assert torch.equal(kd, ke) and torch.equal(vd, ve)
        order = np.argsort(k, kind="stable")
        assert np.array_equal(kd.cpu().numpy().view(np.uint32), k[order])
        assert np.array_equal(vd.cpu().numpy().view(np.uint32), v[order])

    # keys only (no value buffer), once more on the same scratch
    k = _keys(50_000, 32, 3)
    kd = torch.from_numpy(k.view(np.int32)).to(cuda)
    radix_sort_noalloc(kd, None, bits=32)
    assert np.array_equal(kd.cpu().numpy().view(np.uint32), np.sort(k, kind="stable"))
