"""CPU tests of the C ABI's host-side argument checks: calls with a null
handle, an invalid configuration or an oversize request return their
status (and leave a message) before any CUDA call, so they run without a
GPU.  The reference aborts or prints on such input; this boundary reports."""
import ctypes as C
import re

import pytest

OK, INVALID, CAPACITY = 0, 1, 2


def last_error(lib):
    return lib.gsap_last_error().decode()


def test_create_rejects_bad_configs(gsap_lib):
    from gsap_gb300._lib import Config
    c = Config()
    gsap_lib.gsap_config_default(C.byref(c))
    c.sort_bits = 20
    assert not gsap_lib.gsap_sap_create(1000, C.byref(c))
    assert "sort_bits" in last_error(gsap_lib)
    gsap_lib.gsap_config_default(C.byref(c))
    assert not gsap_lib.gsap_sap_create(1 << 28, C.byref(c))  # 8 entries per object: past 2^30
    assert "2^30" in last_error(gsap_lib)


def test_null_handles_are_reported(gsap_lib):
    n = C.c_uint64(0)
    P = None
    calls = {
        "gsap_broadphase_aabb": lambda L: L.gsap_broadphase_aabb(P, P, P, 100, P, 0, P, C.byref(n), 0, P),
        # (a non-null offsets pointer, never read on the host, reaches the handle check)
        "gsap_broadphase_batched": lambda L: L.gsap_broadphase_batched(P, P, P, C.c_void_p(256), 2, 100, P, 0, P,
                                                                       C.byref(n), 0, P),
        "gsap_sap_collision": lambda L: L.gsap_sap_collision(P, 0.0, P, 100, P, P, None, None, 0, 0, P),
        "gsap_sap_check": lambda L: L.gsap_sap_check(P, P),
        "gsap_sap_scene_axes": lambda L: L.gsap_sap_scene_axes(P, 0, P, P),
        "gsap_radix_sort_u32": lambda L: L.gsap_radix_sort_u32(P, P, P, 10, 32, P),
        "gsap_radix_sort_f32": lambda L: L.gsap_radix_sort_f32(P, P, P, 10, 32, 1, P),
        "gsap_rb_step": lambda L: L.gsap_rb_step(P, P, 0.01, P),
        "gsap_rb_integrate": lambda L: L.gsap_rb_integrate(P, 0.01, P),
        "gsap_rb_set_body_data": lambda L: L.gsap_rb_set_body_data(P, P),
        "gsap_rb_get_state": lambda L: L.gsap_rb_get_state(P, P, P, P, P, P),
    }
    for name, call in calls.items():
        assert call(gsap_lib) == INVALID, name
        assert "null" in last_error(gsap_lib), name
    assert gsap_lib.gsap_broadphase_batched(P, P, P, P, 2, 100, P, 0, P, C.byref(n), 0, P) == INVALID
    assert "scene offsets" in last_error(gsap_lib)
    # destroying nothing is a no-op
    gsap_lib.gsap_sap_destroy(None)
    gsap_lib.gsap_rb_destroy(None)


@pytest.mark.parametrize("bits", [0, 33])
def test_noalloc_sort_argument_checks(gsap_lib, bits):
    from gsap_gb300.sap import NOALLOC_SORT_MAX_N as cap
    assert gsap_lib.gsap_radix_sort_u32_noalloc(None, None, cap + 1, 32, None) == CAPACITY
    assert "exceeds its fixed scratch" in last_error(gsap_lib)
    assert gsap_lib.gsap_radix_sort_u32_noalloc(None, None, 5, 32, None) == INVALID
    assert gsap_lib.gsap_radix_sort_u32_noalloc(C.c_void_p(256), None, 5, bits, None) == INVALID
    assert "bits" in last_error(gsap_lib)
    assert gsap_lib.gsap_radix_sort_u32_noalloc(None, None, 0, 32, None) == OK  # nothing to sort


def test_noalloc_python_device_checks():
    """The Python wrapper of the no-alloc sort refuses tensors that are not
    on CUDA or not on one device before it reaches the C ABI (stand-ins for
    tensors: only .is_cuda, .device and .numel are read)."""
    from gsap_gb300.sap import _noalloc_device

    class T:
        def __init__(self, dev, n=8, cuda=True):
            self.device, self._n, self.is_cuda = dev, n, cuda

        def numel(self):
            return self._n

    assert _noalloc_device(T("cuda:1"), T("cuda:1")) == "cuda:1"
    assert _noalloc_device(T("cuda:0"), None) == "cuda:0"
    with pytest.raises(ValueError, match="but vals on"):
        _noalloc_device(T("cuda:1"), T("cuda:0"))
    with pytest.raises(ValueError, match="CUDA tensor"):
        _noalloc_device(T("cpu", cuda=False), None)
    with pytest.raises(ValueError, match="same length"):
        _noalloc_device(T("cuda:0", 8), T("cuda:0", 9))


def test_noalloc_object_calls_no_allocator(gsap_lib):
    """The no-alloc translation unit references no device or host
    allocation routine of the CUDA runtime (its undefined symbols)."""
    import glob
    import os
    import subprocess
    from gsap_gb300 import build
    obj = os.path.join(build.BUILD, "api_noalloc.o")
    assert os.path.exists(obj)
    out = subprocess.run(["nm", "-u", obj], capture_output=True, text=True, check=True).stdout
    undef = {line.split()[-1] for line in out.splitlines() if line.strip()}
    banned = [s for s in undef if re.match(r"^_?(cudaMalloc|cudaFree|cuMemAlloc|cuMemFree|cudaHostAlloc)", s)]
    assert not banned, banned
    assert any("cudaGetSymbolAddress" in s for s in undef)
