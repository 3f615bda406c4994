"""CPU oracle for the gSap broadphase and particle rigid-body step.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU legs of ``bench.py`` -- as the checker and the timed CPU baseline,
never as the thing measured on the GPU.  The product package ``gsap_gb300``
never imports it.

``liboracle.so`` is the C restatement of the reference (``bp.c``, ``rb.c``;
each routine cites the reference file:line it follows).  ``_ref/libgsapref.so``
is built only where the reference tree is mounted: it compiles the
reference's own ``Aabb::overlaps`` and particle rigid-body kernels for the
host and is used to pin the restatement and to generate ``tests/golden``.
"""
from __future__ import annotations

import ctypes as C
import fcntl
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None


_BUILT = False
_STAMP = os.path.join(HERE, ".built-for")  # machine type liboracle.so was built for


def _up_to_date() -> bool:
    lib = os.path.join(HERE, "liboracle.so")
    if not (os.path.exists(lib) and os.path.exists(_STAMP)):
        return False
    with open(_STAMP) as fh:
        if fh.read() != platform.machine():
            return False
    srcs = [os.path.join(HERE, f) for f in ("bp.c", "rb.c", "oracle.h", "Makefile")]
    return os.path.getmtime(lib) >= max(os.path.getmtime(f) for f in srcs)


def build(ref: bool = False) -> None:
    """Compile liboracle.so from source unless this machine type already
    built it from the current sources (a library built on another machine
    type is never reused), and the reference harness when ``ref``.  Builds
    are serialised across processes by a lock file, so workers that start
    together never load a library another one is still writing."""
    global _BUILT
    with open(os.path.join(HERE, ".build.lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        if not _BUILT:
            if not _up_to_date():
                subprocess.run(["make", "-s", "-B", "-C", HERE, "liboracle.so"], check=True)
                with open(_STAMP, "w") as fh:
                    fh.write(platform.machine())
            _BUILT = True
        if ref:
            extra = [f"REF={ref}"] if isinstance(ref, str) else []
            subprocess.run(["make", "-s", "-C", HERE, "ref", *extra], check=True)


def _i64(x):
    return C.c_int64(int(x))


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.orc_bf_aabb.argtypes = [P, P, C.c_uint32, P, C.c_int64, C.c_int]
        L.orc_bf_aabb.restype = C.c_int64
        L.orc_bf_sphere.argtypes = [P, C.c_uint32, P, C.c_int64, C.c_int]
        L.orc_bf_sphere.restype = C.c_int64
        L.orc_sap_ref.argtypes = [C.c_int, P, P, C.c_uint32, P, C.c_int64, C.c_int]
        L.orc_sap_ref.restype = C.c_int64
        L.orc_sap_ref_sampled.argtypes = [C.c_int, P, P, C.c_uint32, C.c_uint32, C.c_uint32, P, C.c_int64,
                                          C.c_int, P]
        L.orc_sap_ref_sampled.restype = C.c_int64
        L.orc_both_directions.argtypes = [P, C.c_int64, P, P]
        L.orc_both_directions.restype = C.c_int64
        L.orc_radix_sort_u32.argtypes = [P, P, C.c_uint32, C.c_int]
        L.orc_radix_sort_u32.restype = None
        L.orc_float_flip.argtypes = [C.c_float]
        L.orc_float_flip.restype = C.c_uint32
        L.orc_normalize_quats.argtypes = [P, C.c_int]
        L.orc_normalize_quats.restype = None
        L.orc_rb_step_ref.argtypes = [P, P, C.c_int64, C.c_int]
        L.orc_rb_step_ref.restype = C.c_int64
        L.orc_rb_step_cfg_f64.argtypes = [P, P, C.c_int]
        L.orc_rb_step_cfg_f64.restype = C.c_int64
        L.orc_rb_step_cfg_f64_amb.argtypes = [P, P, C.c_int, C.c_double, P]
        L.orc_rb_step_cfg_f64_amb.restype = C.c_int64
        L.orc_body_neighbours.argtypes = [C.c_int, P, P, P, C.c_int, C.c_int, P, P, C.c_int64]
        L.orc_body_neighbours.restype = C.c_int64
        L.orc_pairs_batched.argtypes = [P, P, P, C.c_int, C.c_uint32, P, C.c_int64, C.c_int]
        L.orc_pairs_batched.restype = C.c_int64
        _LIB = L
    return _LIB


def ref_lib():
    """The reference-source harness, or None where it was not built."""
    global _REF
    if _REF is None:
        path = os.path.join(HERE, "_ref", "libgsapref.so")
        if not os.path.exists(path):
            return None
        _REF = C.CDLL(path)
        _REF.ref_bf_aabb.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_int64]
        _REF.ref_bf_aabb.restype = C.c_int64
    return _REF


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _f4(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim == 2 and a.shape[1] == 3:
        a = np.ascontiguousarray(np.concatenate([a, np.zeros((a.shape[0], 1), np.float32)], 1))
    return a


def _run_pairs(fn, *args, cap=None):
    """Call a pair-producing routine twice if the first capacity is short."""
    cap = 1 << 16 if cap is None else cap
    while True:
        out = np.empty((max(cap, 1), 2), np.uint32)
        n = fn(*args, _ptr(out), _i64(cap))
        if n <= cap:
            return out[:n].copy()
        cap = int(n)


def bf_aabb(mn, mx, threads=0):
    """Sorted (i<j) uint32 pairs of the O(n^2) closed AABB test."""
    mn, mx = _f4(mn), _f4(mx)
    L = lib()
    return _run_pairs(lambda a, b, p, c: L.orc_bf_aabb(a, b, C.c_uint32(len(mn)), p, c, threads),
                      _ptr(mn), _ptr(mx))


def bf_sphere(spheres, threads=0):
    """Sorted (i<j) uint32 pairs of the strict squared sphere test."""
    s = _f4(spheres)
    L = lib()
    return _run_pairs(lambda a, p, c: L.orc_bf_sphere(a, C.c_uint32(len(s)), p, c, threads), _ptr(s))


def sap_ref(mode, mn, mx=None, threads=0, cap=None):
    """The reference SaP algorithm restated on the CPU (mode 0 AABB, 1 sphere).
    `cap` sizes the first output buffer; a call that finds more pairs runs
    again with room for all of them."""
    mn = _f4(mn)
    mx = _f4(mx) if mx is not None else None
    L = lib()
    return _run_pairs(lambda a, b, p, c: L.orc_sap_ref(mode, a, b, C.c_uint32(len(mn)), p, c, threads),
                      _ptr(mn), _ptr(mx), cap=cap)


def pairs_batched(mn, mx, offsets, bf_max=8192, threads=0, cap=1 << 22):
    """Sorted (i<j) pairs of every scene of a batch (global ids): the O(n^2)
    test for scenes of at most bf_max objects, the same predicate on the
    pairs whose x intervals meet for larger ones."""
    mn, mx = _f4(mn), _f4(mx)
    off = np.ascontiguousarray(offsets, np.int64)
    L = lib()
    return _run_pairs(lambda a, b, p, c: L.orc_pairs_batched(a, b, _ptr(off), len(off) - 1, C.c_uint32(bf_max), p,
                                                             c, threads), _ptr(mn), _ptr(mx), cap=cap)


def sap_ref_sampled(mode, mn, mx, parts, part, threads=0):
    """One call of orc_sap_ref with the sweeps started from slice `part` of
    `parts` contiguous slices of each sorted group, keeping no pairs:
    (pair count, seconds of the fixed stages, seconds of the stages that
    scale with the sweep starts)."""
    mn = _f4(mn)
    mx = _f4(mx) if mx is not None else None
    secs = np.zeros(2, np.float64)
    npairs = lib().orc_sap_ref_sampled(mode, _ptr(mn), _ptr(mx), C.c_uint32(len(mn)), C.c_uint32(parts),
                                       C.c_uint32(part), None, _i64(0), threads, _ptr(secs))
    return int(npairs), float(secs[0]), float(secs[1])


def both_directions(pairs):
    """Reference output format: both-direction int2 list and pairEntries."""
    pairs = np.ascontiguousarray(pairs, dtype=np.uint32)
    npairs = len(pairs)
    out = np.empty((max(2 * npairs, 1), 2), np.int32)
    maxid = int(pairs.max()) + 1 if npairs else 1
    ent = np.empty(maxid, np.int32)
    ne = lib().orc_both_directions(_ptr(pairs), _i64(npairs), _ptr(out), _ptr(ent))
    return out[: 2 * npairs].copy(), ent[:ne].copy()


def radix_sort_u32(keys, vals, bits=32):
    k = np.ascontiguousarray(keys, dtype=np.uint32).copy()
    v = np.ascontiguousarray(vals, dtype=np.uint32).copy()
    lib().orc_radix_sort_u32(_ptr(k), _ptr(v), C.c_uint32(len(k)), bits)
    return k, v


def float_flip(x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32)
    mask = np.where(u & 0x80000000, np.uint32(0xFFFFFFFF), np.uint32(0x80000000))
    return u ^ mask


def ref_bf_aabb(mn, mx):
    """The reference's own Aabb::overlaps in the Demo::cpuBroadphase loop."""
    R = ref_lib()
    if R is None:
        raise RuntimeError("reference harness not built (make -C oracle ref)")
    mn, mx = _f4(mn), _f4(mx)
    return _run_pairs(lambda a, b, p, c: R.ref_bf_aabb(a, b, C.c_uint32(len(mn)), p, c),
                      _ptr(mn), _ptr(mx))


# ----------------------------------------------------------------- rigid body

class RbStateF32(C.Structure):
    _fields_ = [("n_bodies", C.c_int), ("n_particles", C.c_int)] + [
        (name, C.c_void_p) for name in (
            "pos", "quat", "lin_vel", "ang_vel", "shape_idx", "p_start", "n_part", "inv_mass",
            "inv_inertia", "p_pos", "p_vel", "p_force", "p_mass", "ref_pos", "ref_mass",
            "shape_inv_inertia")]


class RefParams(C.Structure):
    _fields_ = [("dt", C.c_float), ("sp_multip", C.c_float), ("dp_multip", C.c_float),
                ("max_lin_vel", C.c_float), ("gravity_y", C.c_float),
                ("floor_clamp", C.c_int), ("torque_quirk", C.c_int), ("pair_loop_quirk", C.c_int)]


class CfgParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("k", C.c_double), ("eta", C.c_double), ("kt", C.c_double),
                ("gravity_y", C.c_double), ("box_lo", C.c_double * 3), ("box_hi", C.c_double * 3)]


class RbStateF64(C.Structure):
    _fields_ = [("n_bodies", C.c_int), ("n_particles", C.c_int)] + [
        (name, C.c_void_p) for name in (
            "pos", "quat", "lin_vel", "ang_vel", "shape_idx", "p_start", "n_part", "scene",
            "inv_mass", "ref_pos", "shape_inv_inertia", "p_pos", "p_vel", "p_force")]


def normalize_quats(q):
    """setRbData's upload normalisation, in place on an (n, 4) float32 array."""
    assert q.dtype == np.float32 and q.flags.c_contiguous
    lib().orc_normalize_quats(_ptr(q), len(q))
    return q


def rb_step_ref(state: dict, dt, sp_multip, dp_multip, max_lin_vel=0.0, gravity_y=-5.0,
                floor_clamp=True, torque_quirk=True, pair_loop_quirk=False, max_pairs=1 << 22, threads=0):
    """One reference-order FP32 step on a dict of numpy arrays (updated in place).

    Keys: pos, quat, lin_vel, ang_vel (nb,4) f32; shape_idx, p_start, n_part (nb,) i32;
    inv_mass (nb,) f32; inv_inertia (nb,12) f32; ref_pos (10*ns,4); ref_mass (10*ns,);
    shape_inv_inertia (ns,12); p_pos, p_vel, p_force (np,4); p_mass (np,).
    Returns the number of both-direction pairs.
    """
    s = RbStateF32()
    s.n_bodies = len(state["pos"])
    s.n_particles = len(state["p_pos"])
    for name, _ in RbStateF32._fields_[2:]:
        setattr(s, name, state[name].ctypes.data)
    p = RefParams(dt, sp_multip, dp_multip, max_lin_vel, gravity_y, int(floor_clamp), int(torque_quirk),
                  int(pair_loop_quirk))
    n = lib().orc_rb_step_ref(C.byref(s), C.byref(p), _i64(max_pairs), threads)
    if n < 0:
        raise RuntimeError("oracle pair capacity exceeded")
    return n


def rb_step_cfg_f64(state: dict, params: dict, threads=0, band=None):
    """One config-mode FP64 step on a dict of float64/int32 arrays (in place).
    With `band`, returns an int32 flag per body: 1 where a contact of the
    step has a penetration depth within +-band of zero (its onset can flip
    under a rounding of the state of that size)."""
    s = RbStateF64()
    s.n_bodies = len(state["pos"])
    s.n_particles = len(state["p_pos"])
    for name, _ in RbStateF64._fields_[2:]:
        arr = state.get(name)
        setattr(s, name, arr.ctypes.data if arr is not None else None)
    p = CfgParams()
    p.dt, p.k, p.eta, p.kt, p.gravity_y = (params[k] for k in ("dt", "k", "eta", "kt", "gravity_y"))
    for a in range(3):
        p.box_lo[a] = params["box_lo"][a]
        p.box_hi[a] = params["box_hi"][a]
    if band is None:
        return lib().orc_rb_step_cfg_f64(C.byref(s), C.byref(p), threads)
    amb = np.zeros(s.n_bodies, np.int32)
    lib().orc_rb_step_cfg_f64_amb(C.byref(s), C.byref(p), threads, C.c_double(band), _ptr(amb))
    return amb


def body_neighbours(bmin, bmax, scene=None, brute=False, threads=0):
    """Rows of the FP64 oracle's body pair search: (offsets[nb+1], ids)."""
    bmin = np.ascontiguousarray(bmin, np.float64)
    bmax = np.ascontiguousarray(bmax, np.float64)
    nb = len(bmin)
    sc = np.ascontiguousarray(scene, np.int32) if scene is not None else None
    cnt = np.zeros(nb + 1, np.int32)
    cap = 16 * nb + 16
    while True:
        nbr = np.empty(max(cap, 1), np.int32)
        tot = lib().orc_body_neighbours(nb, _ptr(bmin), _ptr(bmax), _ptr(sc), int(brute), threads, _ptr(cnt),
                                        _ptr(nbr), _i64(cap))
        if tot >= 0:
            return cnt, nbr[:tot].copy()
        cap = int(cnt[nb])
