"""Host-side mirror of the reference's ``Sap`` broadphase class.

``Sap(n)`` / ``Sap.collision(spacing, d_particle_data, pairs, pairs_entries)``
follow ``class Sap`` of sapDetection/Sap.h:12-24 (usage:
physicboxSap2.16_Fermi/readme.txt:1-7, cudaPhysics/demoParticles.h:898-903);
``broadphase`` / ``broadphase_batched`` are the AABB and batched forms of
the same pipeline.  Device memory is plain torch CUDA tensors; every call
goes through the C ABI of libgsap.so (include/gsap.h).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._lib import (AXIS_PCA, FLAG_GRAPH, FLAG_SORTED, FLAG_TEMPORAL, MODE_AABB, MODE_SPHERE, Config, GsapError,
                   check, load)


def _stream_ptr(stream) -> int:
    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream)


def _dev_ptr(t: torch.Tensor | None, name: str, dtype=None, cols=None) -> int | None:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise ValueError(f"{name} must be {dtype}, got {t.dtype}")
    if cols is not None and (t.dim() != 2 or t.shape[1] != cols):
        raise ValueError(f"{name} must have shape (n, {cols})")
    return t.data_ptr()


NOALLOC_SORT_MAX_N = 1 << 20  # GSAP_NOALLOC_SORT_MAX_N


def _noalloc_device(keys, vals):
    """The device the no-alloc sort runs on: the keys' device, which the
    values must share (the C side checks the pointers against the current
    device too)."""
    if not keys.is_cuda:
        raise ValueError("keys must be a CUDA tensor")
    if vals is not None:
        if not vals.is_cuda:
            raise ValueError("vals must be a CUDA tensor")
        if vals.device != keys.device:
            raise ValueError(f"keys are on {keys.device} but vals on {vals.device}")
        if vals.numel() != keys.numel():
            raise ValueError("keys and vals must have the same length")
    return keys.device


def radix_sort_noalloc(keys: torch.Tensor, vals: torch.Tensor | None = None, bits: int = 32, stream=None):
    """In-place stable sort like ``Sap.radix_sort`` that allocates no device
    memory and needs no handle: its scratch is a fixed static device array,
    so at most ``NOALLOC_SORT_MAX_N`` keys, and calls that overlap in time
    race.  The first call on a device does a synchronising set-up.  Runs on
    the keys' device (made current for the call), on `stream` or that
    device's current stream."""
    dev = _noalloc_device(keys, vals)
    _dev_ptr(keys, "keys", torch.int32)
    _dev_ptr(vals, "vals", torch.int32)
    with torch.cuda.device(dev):
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        elif stream.device != dev:
            raise ValueError(f"stream is on {stream.device}, keys on {dev}")
        check(load().gsap_radix_sort_u32_noalloc(keys.data_ptr(), vals.data_ptr() if vals is not None else None,
                                                 C.c_uint32(keys.numel()), C.c_uint32(bits),
                                                 C.c_void_p(_stream_ptr(stream))))


class Sap:
    """GB300 sweep-and-prune broadphase handle (owns all scratch)."""

    def __init__(self, max_n: int, mode: int = MODE_AABB, axis_mode: int = AXIS_PCA, max_scenes: int = 1,
                 entry_factor: int = 8, pair_factor: int = 16, sort_bits: int = 32, cell_factor: float = 2.0,
                 spin_limit: int = 0, sort_mode: int = 0, sort_tile: int = 0):
        L = load()
        cfg = Config()
        L.gsap_config_default(C.byref(cfg))
        cfg.mode, cfg.axis_mode, cfg.max_scenes = mode, axis_mode, max_scenes
        cfg.entry_factor, cfg.pair_factor, cfg.sort_bits = entry_factor, pair_factor, sort_bits
        cfg.cell_factor = cell_factor
        cfg.sort_mode = sort_mode
        cfg.sort_tile = sort_tile
        if spin_limit:
            cfg.spin_limit = spin_limit
        self.cfg = cfg
        self.max_n = int(max_n)
        self.mode = mode
        self._h = L.gsap_sap_create(C.c_uint32(self.max_n), C.byref(cfg))
        if not self._h:
            raise GsapError(3, _lib.last_error())
        self._count = None

    # ------------------------------------------------------------ lifecycle
    def close(self):
        if getattr(self, "_h", None):
            load().gsap_sap_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # ------------------------------------------------------- reference API
    def collision(self, spacing: float, particle_data: torch.Tensor, pairs: torch.Tensor,
                  pairs_entries: torch.Tensor, stream=None):
        """Sap::collision (Sap.cpp:211-335): spheres float4 (x, y, z, r) ->
        both-direction int2 pairs sorted by (first, second) and CSR
        pairEntries.  Returns (num_pairs, num_pair_entries)."""
        n = particle_data.shape[0]
        _dev_ptr(particle_data, "particle_data", torch.float32, 4)
        _dev_ptr(pairs, "pairs", torch.int32, 2)
        _dev_ptr(pairs_entries, "pairs_entries", torch.int32)
        np_, ne = C.c_int32(0), C.c_int32(0)
        st = load().gsap_sap_collision(self._h, C.c_float(spacing), particle_data.data_ptr(), C.c_uint32(n),
                                       pairs.data_ptr(), pairs_entries.data_ptr(), C.byref(np_), C.byref(ne),
                                       C.c_uint64(pairs.shape[0]), C.c_uint64(pairs_entries.numel()),
                                       C.c_void_p(_stream_ptr(stream)))
        check(st)
        return np_.value, ne.value

    # ----------------------------------------------------------- AABB form
    def broadphase(self, mn: torch.Tensor, mx: torch.Tensor | None = None, pairs: torch.Tensor | None = None,
                   sorted: bool = True, graph: bool = False, temporal: bool = False, stream=None) -> torch.Tensor:
        """Overlapping pairs (i < j) as an (P, 2) int32 tensor (uint32 ids).

        mn / mx: (n, 4) float32 CUDA tensors (AABB min / max; for the sphere
        predicate mn holds (x, y, z, r) and mx is None)."""
        n = mn.shape[0]
        _dev_ptr(mn, "mn", torch.float32, 4)
        _dev_ptr(mx, "mx", torch.float32, 4)
        flags = (FLAG_SORTED if sorted else 0) | (FLAG_GRAPH if graph else 0) | (FLAG_TEMPORAL if temporal else 0)
        if pairs is None:
            pairs = torch.empty((max(16, 8 * n), 2), dtype=torch.int32, device=mn.device)
        for _ in range(2):
            cnt = C.c_uint64(0)
            st = load().gsap_broadphase_aabb(self._h, mn.data_ptr(), mx.data_ptr() if mx is not None else None,
                                             C.c_uint32(n), pairs.data_ptr(), C.c_uint64(pairs.shape[0]), None,
                                             C.byref(cnt), C.c_uint32(flags), C.c_void_p(_stream_ptr(stream)))
            if st == 2 and cnt.value > pairs.shape[0]:
                pairs = torch.empty((int(cnt.value * 1.25) + 16, 2), dtype=torch.int32, device=mn.device)
                continue
            check(st)
            return pairs[: cnt.value]
        check(st)
        return pairs[: cnt.value]

    def autotune(self, mn: torch.Tensor, mx: torch.Tensor | None = None, offsets: torch.Tensor | None = None,
                 pairs: torch.Tensor | None = None, sorted: bool = True, graph: bool = True, reps: int = 3,
                 stream=None) -> dict:
        """Picks the sort (bucket, or radix with its tile size), key width and cell factor for
        this kind of input by timing a small grid on it (gsap_sap_autotune);
        the handle keeps the fastest.  Returns the chosen settings."""
        n = mn.shape[0]
        _dev_ptr(mn, "mn", torch.float32, 4)
        _dev_ptr(mx, "mx", torch.float32, 4)
        _dev_ptr(offsets, "offsets", torch.int32)
        flags = (FLAG_SORTED if sorted else 0) | (FLAG_GRAPH if graph else 0)
        if pairs is None:
            pairs = torch.empty((max(16, 8 * n), 2), dtype=torch.int32, device=mn.device)
        cfg = Config()
        S = offsets.numel() - 1 if offsets is not None else 0
        check(load().gsap_sap_autotune(self._h, mn.data_ptr(), mx.data_ptr() if mx is not None else None,
                                       offsets.data_ptr() if offsets is not None else None, C.c_uint32(S),
                                       C.c_uint32(n), pairs.data_ptr(), C.c_uint64(pairs.shape[0]),
                                       C.c_uint32(flags), C.c_int(reps), C.byref(cfg),
                                       C.c_void_p(_stream_ptr(stream))))
        return {"sort_bits": int(cfg.sort_bits), "cell_factor": float(cfg.cell_factor),
                "sort": "radix" if cfg.sort_mode == 0 else "bucket", "sort_tile": int(cfg.sort_tile)}

    def broadphase_async(self, mn, mx, pairs, d_count, sorted=False, graph=False, temporal=False, stream=None):
        """Asynchronous form: the pair count goes to the device tensor
        d_count (one int64); no host synchronisation.  Errors are picked up by
        check().  temporal: sweep with the previous call's grid while this
        call's PCA runs beside it (GSAP_FLAG_TEMPORAL)."""
        flags = (FLAG_SORTED if sorted else 0) | (FLAG_GRAPH if graph else 0) | (FLAG_TEMPORAL if temporal else 0)
        st = load().gsap_broadphase_aabb(self._h, mn.data_ptr(), mx.data_ptr() if mx is not None else None,
                                         C.c_uint32(mn.shape[0]), pairs.data_ptr(), C.c_uint64(pairs.shape[0]),
                                         C.c_void_p(d_count.data_ptr()), None, C.c_uint32(flags),
                                         C.c_void_p(_stream_ptr(stream)))
        check(st)

    def broadphase_batched(self, mn: torch.Tensor, mx: torch.Tensor | None, offsets: torch.Tensor,
                           pairs: torch.Tensor | None = None, sorted: bool = True, graph: bool = False,
                           temporal: bool = False, stream=None) -> torch.Tensor:
        """Batched scenes: offsets is a CUDA int32 tensor of S+1 scene
        starts.  Pairs use global ids and never cross scenes."""
        n = mn.shape[0]
        S = offsets.numel() - 1
        _dev_ptr(offsets, "offsets", torch.int32)
        flags = (FLAG_SORTED if sorted else 0) | (FLAG_GRAPH if graph else 0) | (FLAG_TEMPORAL if temporal else 0)
        if pairs is None:
            pairs = torch.empty((max(16, 8 * n), 2), dtype=torch.int32, device=mn.device)
        for _ in range(2):
            cnt = C.c_uint64(0)
            st = load().gsap_broadphase_batched(self._h, mn.data_ptr(), mx.data_ptr() if mx is not None else None,
                                                offsets.data_ptr(), C.c_uint32(S), C.c_uint32(n), pairs.data_ptr(),
                                                C.c_uint64(pairs.shape[0]), None, C.byref(cnt), C.c_uint32(flags),
                                                C.c_void_p(_stream_ptr(stream)))
            if st == 2 and cnt.value > pairs.shape[0]:
                pairs = torch.empty((int(cnt.value * 1.25) + 16, 2), dtype=torch.int32, device=mn.device)
                continue
            check(st)
            return pairs[: cnt.value]
        check(st)
        return pairs[: cnt.value]

    def check(self, stream=None):
        check(load().gsap_sap_check(self._h, C.c_void_p(_stream_ptr(stream))))

    # ------------------------------------------------------------- extras
    def scene_axes(self, scene: int = 0, stream=None) -> dict:
        out = (C.c_double * 17)()
        check(load().gsap_sap_scene_axes(self._h, C.c_uint32(scene), out, C.c_void_p(_stream_ptr(stream))))
        v = list(out)
        return {"axes": [v[0:3], v[3:6], v[6:9]], "eig": v[9:12], "mean": v[12:15], "grid": (int(v[15]), int(v[16]))}

    def radix_sort(self, keys: torch.Tensor, vals: torch.Tensor | None = None, bits: int = 32, stream=None):
        """In-place stable sort of int32-stored uint32 keys (and values)."""
        _dev_ptr(keys, "keys", torch.int32)
        _dev_ptr(vals, "vals", torch.int32)
        check(load().gsap_radix_sort_u32(self._h, keys.data_ptr(), vals.data_ptr() if vals is not None else None,
                                         C.c_uint32(keys.numel()), C.c_uint32(bits),
                                         C.c_void_p(_stream_ptr(stream))))

    def radix_sort_f32(self, keys: torch.Tensor, vals: torch.Tensor | None = None, key_bits: int = 32,
                       negative_keys: bool = True, stream=None):
        """RadixSort::sort(float*, uint*, n, keyBits, negativeKeys)
        (radixsort.h:180-198): in-place stable sort of float32 keys (and
        int32-stored uint32 values) in float order when negative_keys."""
        _dev_ptr(keys, "keys", torch.float32)
        _dev_ptr(vals, "vals", torch.int32)
        if vals is not None and vals.numel() != keys.numel():
            raise ValueError("keys and vals must have the same length")
        check(load().gsap_radix_sort_f32(self._h, keys.data_ptr(), vals.data_ptr() if vals is not None else None,
                                         C.c_uint32(keys.numel()), C.c_uint32(key_bits), C.c_int(int(negative_keys)),
                                         C.c_void_p(_stream_ptr(stream))))

    def stats(self, stream=None) -> dict:
        out = (C.c_uint64 * 8)()
        if load().gsap_debug_stats(self._h, out, C.c_void_p(_stream_ptr(stream))) != 0:
            raise GsapError(3, "stats read failed")
        v = list(out)
        return dict(zip(("entries", "tests", "pairs", "buckets", "qbits", "long_rows", "iters", "error"), v))

    def enable_timing(self, on: bool = True):
        load().gsap_sap_enable_timing(self._h, int(on))

    def stage_times(self) -> list[float]:
        out = (C.c_float * 8)()
        k = load().gsap_sap_stage_times(self._h, out, 8)
        return list(out)[:k]
